/*
 * stim_oracle.c -- CPU oracle (test infrastructure only; see stim_oracle.h).
 *
 * Restates, in plain C over 64-bit words with shots on the minor axis (frame_simulator.h:45-59):
 *   - the .stim parser: dead space / comments (circuit.h:295-338), tags (circuit.h:364-420),
 *     parens arguments (circuit.h:423-445), targets (gate_target.h:75-195), REPEAT blocks
 *     (circuit.cc:254-300) and the fusion of adjacent identical instructions
 *     (circuit.cc:237-251, circuit_instruction.cc can_fuse);
 *   - circuit statistics (circuit_instruction.cc add_stats_to);
 *   - the frame rules of FrameSimulator<W> (frame_simulator.inl:139-912): Cliffords, classical
 *     feedback, M/MR/R in three bases, MPP / SPP / MXX / MYY / MZZ decompositions
 *     (gate_decomposition.cc:88-161, 163-250, 319-347), MPAD, DETECTOR, OBSERVABLE_INCLUDE,
 *     E / ELSE_CORRELATED_ERROR, heralded channels;
 * with every random bit taken from gfs_contract.h.
 */
#define _POSIX_C_SOURCE 200809L
#include "stim_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gfs_contract.h"
#include "gfs_gates.h"

/* ------------------------------------------------------------------------------------------------ */
/* Circuit representation                                                                           */
/* ------------------------------------------------------------------------------------------------ */

typedef struct ochan {
    int active;  /* p > 0 */
    int always;  /* p >= 1 */
    float inv_c;
    uint32_t *table;
    uint64_t cum[16];
    double total;
} ochan;

typedef struct oinst {
    gfs_gate gate;
    uint32_t *t;
    size_t nt, tcap;
    double *a;
    size_t na;
    char *tag;
    size_t taglen;
    size_t block;  /* REPEAT */
    uint64_t reps; /* REPEAT */
    ochan ch;      /* noise channel (hit probability) */
} oinst;

typedef struct oblock {
    oinst *ops;
    size_t n, cap;
} oblock;

struct oracle_circuit {
    oblock *blocks;
    size_t nblocks, bcap;
    uint64_t num_qubits, num_meas, num_dets, num_obs, max_lookback, num_inst;
};

typedef struct oerr {
    char *buf;
    size_t len;
    int failed;
} oerr;

static void seterr(oerr *e, const char *fmt, ...) {
    if (e->failed) {
        return;
    }
    e->failed = 1;
    if (e->buf && e->len) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(e->buf, e->len, fmt, ap);
        va_end(ap);
    }
}

static const gfs_gate_info *ginfo(gfs_gate g) {
    return gfs_gate_by_id(g);
}

/* ------------------------------------------------------------------------------------------------ */
/* Parser                                                                                           */
/* ------------------------------------------------------------------------------------------------ */

typedef struct oparse {
    const char *s;
    size_t n, k;
    oerr *e;
} oparse;

static int rd(oparse *p) {
    return p->k < p->n ? (unsigned char)p->s[p->k++] : EOF;
}

static int is_space(int c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f';
}

static void skip_dead_space(int *c, oparse *p) {
    for (;;) {
        while (*c != EOF && is_space(*c)) {
            *c = rd(p);
        }
        if (*c != '#') {
            return;
        }
        while (*c != '\n' && *c != EOF) {
            *c = rd(p);
        }
    }
}

static int next_line_arg(int *c, oparse *p, int space_required) {
    if (*c == '*') {
        return 1;
    }
    if (space_required) {
        if (*c != ' ' && *c != '#' && *c != '\t' && *c != '\n' && *c != '\r' && *c != '{' && *c != EOF) {
            seterr(p->e, "Targets must be separated by spacing.");
            return 0;
        }
    }
    while (*c == ' ' || *c == '\t' || *c == '\r') {
        *c = rd(p);
    }
    if (*c == '#') {
        do {
            *c = rd(p);
        } while (*c != '\n' && *c != EOF);
    }
    return *c != '\n' && *c != '{' && *c != EOF;
}

static uint32_t read_u24(int *c, oparse *p) {
    if (!(*c >= '0' && *c <= '9')) {
        seterr(p->e, "Expected a digit but got '%c'", *c);
        return 0;
    }
    uint32_t r = 0;
    do {
        r = r * 10 + (uint32_t)(*c - '0');
        if (r >= (1u << 24)) {
            seterr(p->e, "Number too large.");
            return 0;
        }
        *c = rd(p);
    } while (*c >= '0' && *c <= '9');
    return r;
}

static uint64_t read_u63(int *c, oparse *p) {
    if (!(*c >= '0' && *c <= '9')) {
        seterr(p->e, "Expected a digit but got '%c'", *c);
        return 0;
    }
    uint64_t r = 0;
    do {
        r = r * 10 + (uint64_t)(*c - '0');
        if (r >= ((uint64_t)1 << 63)) {
            seterr(p->e, "Number too large.");
            return 0;
        }
        *c = rd(p);
    } while (*c >= '0' && *c <= '9');
    return r;
}

static uint32_t read_pauli_target(int *c, oparse *p) {
    uint32_t m = 0;
    if (*c == 'x' || *c == 'X') {
        m = GFS_T_PAULI_X;
    } else if (*c == 'y' || *c == 'Y') {
        m = GFS_T_PAULI_X | GFS_T_PAULI_Z;
    } else {
        m = GFS_T_PAULI_Z;
    }
    *c = rd(p);
    if (*c == ' ') {
        seterr(p->e, "Pauli target followed by a space instead of a qubit index.");
        return 0;
    }
    return read_u24(c, p) | m;
}

static int expect_chars(oparse *p, const char *rest) {
    for (; *rest; rest++) {
        if (rd(p) != *rest) {
            return 0;
        }
    }
    return 1;
}

static uint32_t read_target(int *c, oparse *p) {
    if (*c >= '0' && *c <= '9') {
        return read_u24(c, p);
    }
    switch (*c) {
        case 'r': {
            if (!expect_chars(p, "ec[-")) {
                seterr(p->e, "Target started with 'r' but wasn't a record argument like 'rec[-1]'.");
                return 0;
            }
            *c = rd(p);
            uint32_t v = read_u24(c, p);
            if (*c != ']') {
                seterr(p->e, "Target started with 'r' but wasn't a record argument like 'rec[-1]'.");
                return 0;
            }
            *c = rd(p);
            return v | GFS_T_RECORD;
        }
        case 's': {
            if (!expect_chars(p, "weep[")) {
                seterr(p->e, "Target started with 's' but wasn't a sweep bit argument like 'sweep[5]'.");
                return 0;
            }
            *c = rd(p);
            uint32_t v = read_u24(c, p);
            if (*c != ']') {
                seterr(p->e, "Target started with 's' but wasn't a sweep bit argument like 'sweep[5]'.");
                return 0;
            }
            *c = rd(p);
            return v | GFS_T_SWEEP;
        }
        case '!': {
            *c = rd(p);
            uint32_t t;
            if (*c == 'X' || *c == 'x' || *c == 'Y' || *c == 'y' || *c == 'Z' || *c == 'z') {
                t = read_pauli_target(c, p);
            } else {
                t = read_u24(c, p);
            }
            return t ^ GFS_T_INVERTED;
        }
        case 'X':
        case 'Y':
        case 'Z':
        case 'x':
        case 'y':
        case 'z':
            return read_pauli_target(c, p);
        case '*':
            *c = rd(p);
            return GFS_T_COMBINER;
        default:
            seterr(p->e, "Unrecognized target prefix '%c'.", *c);
            return 0;
    }
}

static void push_target(oinst *op, uint32_t t) {
    if (op->nt == op->tcap) {
        op->tcap = op->tcap ? op->tcap * 2 : 8;
        op->t = (uint32_t *)realloc(op->t, op->tcap * sizeof(uint32_t));
    }
    op->t[op->nt++] = t;
}

static int is_double_char(int c) {
    return (c >= '0' && c <= '9') || c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-';
}

static size_t new_block(oracle_circuit *circ) {
    if (circ->nblocks == circ->bcap) {
        circ->bcap = circ->bcap ? circ->bcap * 2 : 4;
        circ->blocks = (oblock *)realloc(circ->blocks, circ->bcap * sizeof(oblock));
    }
    memset(&circ->blocks[circ->nblocks], 0, sizeof(oblock));
    return circ->nblocks++;
}

static oinst *push_op(oracle_circuit *circ, size_t b) {
    oblock *blk = &circ->blocks[b];
    if (blk->n == blk->cap) {
        blk->cap = blk->cap ? blk->cap * 2 : 16;
        blk->ops = (oinst *)realloc(blk->ops, blk->cap * sizeof(oinst));
    }
    oinst *op = &blk->ops[blk->n++];
    memset(op, 0, sizeof(*op));
    return op;
}

static void free_op(oinst *op) {
    free(op->t);
    free(op->a);
    free(op->tag);
}

static void validate(const oinst *op, oerr *e) {
    const gfs_gate_info *g = ginfo(op->gate);
    uint32_t f = g->flags;
    if (f & GFS_F_PAIRS) {
        if (f & GFS_F_PAULI_STRING) {
            size_t terms = op->nt;
            for (size_t k = 0; k < op->nt; k++) {
                if (op->t[k] & GFS_T_COMBINER) {
                    terms -= 2;
                }
            }
            if (terms & 1) {
                seterr(e, "The gate %s requires an even number of products to target.", g->name);
                return;
            }
        } else {
            if (op->nt & 1) {
                seterr(e, "Two qubit gate %s requires an even number of targets.", g->name);
                return;
            }
            for (size_t k = 0; k < op->nt; k += 2) {
                if (op->t[k] == op->t[k + 1]) {
                    seterr(e, "The two qubit gate %s was applied to a target pair with the same target twice.",
                           g->name);
                    return;
                }
            }
        }
    }
    if (g->arg_count == GFS_ARGS_ZERO_OR_ONE) {
        if (op->na > 1) {
            seterr(e, "Gate %s was given %zu parens arguments but takes 0 or 1 parens arguments.", g->name, op->na);
            return;
        }
    } else if (g->arg_count != GFS_ARGS_ANY && (int)op->na != g->arg_count) {
        seterr(e, "Gate %s was given %zu parens arguments but takes %d parens arguments.", g->name, op->na,
               g->arg_count);
        return;
    }
    if ((f & GFS_F_NO_TARGETS) && op->nt) {
        seterr(e, "Gate %s takes no targets but was given targets.", g->name);
        return;
    }
    if (f & GFS_F_DISJOINT_PROBS) {
        double total = 0;
        for (size_t k = 0; k < op->na; k++) {
            if (!(op->a[k] >= 0 && op->a[k] <= 1)) {
                seterr(e, "Gate %s only takes probability arguments.", g->name);
                return;
            }
            total += op->a[k];
        }
        if (total > 1.0000001) {
            seterr(e, "The disjoint probability arguments given to gate %s sum to more than 1.", g->name);
            return;
        }
    } else if (f & GFS_F_UINT_ARGS) {
        for (size_t k = 0; k < op->na; k++) {
            if (op->a[k] < 0 || op->a[k] != round(op->a[k])) {
                seterr(e, "Gate %s only takes non-negative integer arguments.", g->name);
                return;
            }
        }
    }
    uint32_t valid = GFS_T_VALUE_MASK;
    if (f & GFS_F_COMBINERS) {
        int allowed = 0, just = 0, failed = 0;
        for (size_t k = 0; k < op->nt; k++) {
            if (op->t[k] & GFS_T_COMBINER) {
                failed |= !allowed;
                allowed = 0;
                just = 1;
            } else {
                allowed = 1;
                just = 0;
            }
        }
        failed |= just;
        if (failed) {
            seterr(e, "Gate %s given combiners ('*') that aren't between other targets.", g->name);
            return;
        }
        valid |= GFS_T_COMBINER;
    }
    if (f & GFS_F_RESULTS) {
        valid |= GFS_T_INVERTED;
    }
    if (f & GFS_F_CAN_TARGET_BITS) {
        valid |= GFS_T_RECORD | GFS_T_SWEEP;
    }
    for (size_t k = 0; k < op->nt; k++) {
        uint32_t t = op->t[k];
        if (f & GFS_F_ONLY_REC) {
            int ok = (t & GFS_T_RECORD) || ((f & GFS_F_PAULI_STRING) && (t & (GFS_T_PAULI_X | GFS_T_PAULI_Z)));
            if (!ok) {
                seterr(e, "Gate %s only takes measurement record targets.", g->name);
                return;
            }
        } else if (f & GFS_F_PAULI_STRING) {
            if (!(t & (GFS_T_PAULI_X | GFS_T_PAULI_Z | GFS_T_COMBINER |
                       ((f & GFS_F_CAN_TARGET_BITS) ? (GFS_T_SWEEP | GFS_T_RECORD) : 0)))) {
                seterr(e, "Gate %s only takes Pauli targets.", g->name);
                return;
            }
        } else if (t != (t & valid)) {
            seterr(e, "Target has invalid modifiers for gate type '%s'.", g->name);
            return;
        }
    }
    if (op->gate == GFS_MPAD) {
        for (size_t k = 0; k < op->nt; k++) {
            if (op->t[k] > 1) {
                seterr(e, "Target is not valid for gate type 'MPAD'.");
                return;
            }
        }
    }
}

static int args_equal(const oinst *a, const oinst *b) {
    if (a->na != b->na) {
        return 0;
    }
    for (size_t k = 0; k < a->na; k++) {
        if (a->a[k] != b->a[k]) {
            return 0;
        }
    }
    return 1;
}

static int can_fuse(const oinst *a, const oinst *b) {
    if (a->gate != b->gate || !args_equal(a, b) || (ginfo(a->gate)->flags & GFS_F_NOT_FUSABLE)) {
        return 0;
    }
    if (a->taglen != b->taglen) {
        return 0;
    }
    return a->taglen == 0 || memcmp(a->tag, b->tag, a->taglen) == 0;
}

static void parse_block(oracle_circuit *circ, size_t b, oparse *p, int until_brace) {
    for (;;) {
        int c = rd(p);
        skip_dead_space(&c, p);
        if (c == EOF) {
            if (until_brace) {
                seterr(p->e, "Unterminated block. Got a '{' without an eventual '}'.");
            }
            return;
        }
        if (c == '}') {
            if (!until_brace) {
                seterr(p->e, "Uninitiated block. Got a '}' without a '{'.");
            }
            return;
        }
        char name[32];
        size_t nlen = 0;
        while (((c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || (c >= '0' && c <= '9') || c == '_') &&
               nlen < sizeof(name)) {
            name[nlen++] = (char)c;
            c = rd(p);
        }
        const gfs_gate_info *g = gfs_gate_by_name(name, nlen);
        if (!g) {
            seterr(p->e, "Gate not found: '%.*s'", (int)nlen, name);
            return;
        }
        oinst *op = push_op(circ, b);
        op->gate = g->id;
        if (c == '[') {
            size_t cap = 16;
            op->tag = (char *)malloc(cap);
            c = rd(p);
            while (c != ']') {
                if (c == '\r' || c == '\n' || c == EOF) {
                    seterr(p->e, "A tag wasn't closed with ']' before the end of the line.");
                    return;
                }
                char ch = (char)c;
                if (c == '\\') {
                    c = rd(p);
                    if (c == 'n') {
                        ch = '\n';
                    } else if (c == 'r') {
                        ch = '\r';
                    } else if (c == 'B') {
                        ch = '\\';
                    } else if (c == 'C') {
                        ch = ']';
                    } else {
                        seterr(p->e, "Unrecognized escape sequence.");
                        return;
                    }
                }
                if (op->taglen + 1 >= cap) {
                    cap *= 2;
                    op->tag = (char *)realloc(op->tag, cap);
                }
                op->tag[op->taglen++] = ch;
                c = rd(p);
            }
            c = rd(p);
        }
        if (c == '(') {
            size_t cap = 4;
            op->a = (double *)malloc(cap * sizeof(double));
            c = rd(p);
            while (c == ' ' || c == '\t') {
                c = rd(p);
            }
            for (;;) {
                char buf[64];
                size_t n = 0;
                while (n < sizeof(buf) - 1 && is_double_char(c)) {
                    buf[n++] = (char)c;
                    c = rd(p);
                }
                buf[n] = 0;
                char *end;
                double v = strtod(buf, &end);
                if (end != buf + n || n == 0 || isinf(v) || isnan(v)) {
                    seterr(p->e, "Not a real number: %s", buf);
                    return;
                }
                if (op->na == cap) {
                    cap *= 2;
                    op->a = (double *)realloc(op->a, cap * sizeof(double));
                }
                op->a[op->na++] = v;
                while (c == ' ' || c == '\t') {
                    c = rd(p);
                }
                if (c != ',') {
                    break;
                }
                c = rd(p);
                while (c == ' ' || c == '\t') {
                    c = rd(p);
                }
            }
            while (c == ' ' || c == '\t') {
                c = rd(p);
            }
            if (c != ')') {
                seterr(p->e, "Parens arguments for '%s' didn't end with a ')'.", g->name);
                return;
            }
            c = rd(p);
        }
        if (g->flags & GFS_F_BLOCK) {
            uint64_t reps = 0;
            int count = 0;
            while (next_line_arg(&c, p, 1)) {
                reps = read_u63(&c, p);
                count++;
                if (p->e->failed) {
                    return;
                }
            }
            if (p->e->failed) {
                return;
            }
            if (c != '{') {
                seterr(p->e, "Missing '{' at start of %s block.", g->name);
                return;
            }
            if (count != 1) {
                seterr(p->e, "Invalid instruction. Expected one repetition arg like `REPEAT 100 {`.");
                return;
            }
            if (reps == 0) {
                seterr(p->e, "Repeating 0 times is not supported.");
                return;
            }
            size_t child = new_block(circ);
            /* `op` may have moved when blocks were reallocated; re-fetch it. */
            op = &circ->blocks[b].ops[circ->blocks[b].n - 1];
            op->block = child;
            op->reps = reps;
            parse_block(circ, child, p, 1);
            if (p->e->failed) {
                return;
            }
        } else {
            int need_space = 1;
            while (next_line_arg(&c, p, need_space)) {
                uint32_t t = read_target(&c, p);
                if (p->e->failed) {
                    return;
                }
                push_target(op, t);
                need_space = !(t & GFS_T_COMBINER);
            }
            if (p->e->failed) {
                return;
            }
            if (c == '{') {
                seterr(p->e, "Unexpected '{'.");
                return;
            }
            validate(op, p->e);
            if (p->e->failed) {
                return;
            }
            oblock *blk = &circ->blocks[b];
            if (blk->n >= 2 && can_fuse(&blk->ops[blk->n - 2], op)) {
                oinst *prev = &blk->ops[blk->n - 2];
                for (size_t k = 0; k < op->nt; k++) {
                    push_target(prev, op->t[k]);
                }
                free_op(op);
                blk->n--;
            }
        }
        if (c == EOF) {
            if (until_brace) {
                seterr(p->e, "Unterminated block. Got a '{' without an eventual '}'.");
            }
            return;
        }
    }
}

/* ------------------------------------------------------------------------------------------------ */
/* Statistics and channel precomputation                                                            */
/* ------------------------------------------------------------------------------------------------ */

typedef struct ostats {
    uint64_t nq, nm, nd, no, lb, ni;
} ostats;

static uint64_t sat_add(uint64_t a, uint64_t b) {
    return a + b < a ? UINT64_MAX : a + b;
}
static uint64_t sat_mul(uint64_t a, uint64_t b) {
    if (a && b > UINT64_MAX / a) {
        return UINT64_MAX;
    }
    return a * b;
}

static uint64_t count_results(const oinst *op) {
    uint32_t f = ginfo(op->gate)->flags;
    if (!(f & GFS_F_RESULTS)) {
        return 0;
    }
    uint64_t n = op->nt;
    if (f & GFS_F_PAIRS) {
        return n >> 1;
    }
    if (f & GFS_F_COMBINERS) {
        for (size_t k = 0; k < op->nt; k++) {
            if (op->t[k] & GFS_T_COMBINER) {
                n -= 2;
            }
        }
    }
    return n;
}

static ostats block_stats(const oracle_circuit *circ, size_t b) {
    ostats s = {0, 0, 0, 0, 0, 0};
    const oblock *blk = &circ->blocks[b];
    for (size_t i = 0; i < blk->n; i++) {
        const oinst *op = &blk->ops[i];
        if (op->gate == GFS_REPEAT) {
            ostats sub = block_stats(circ, op->block);
            s.nq = sub.nq > s.nq ? sub.nq : s.nq;
            s.no = sub.no > s.no ? sub.no : s.no;
            s.lb = sub.lb > s.lb ? sub.lb : s.lb;
            s.nd = sat_add(s.nd, sat_mul(sub.nd, op->reps));
            s.nm = sat_add(s.nm, sat_mul(sub.nm, op->reps));
            s.ni = sat_add(s.ni, sat_mul(sub.ni, op->reps));
            continue;
        }
        s.ni++;
        for (size_t k = 0; k < op->nt; k++) {
            uint32_t t = op->t[k];
            uint32_t v = t & GFS_T_VALUE_MASK;
            if (op->gate != GFS_MPAD && !(t & (GFS_T_RECORD | GFS_T_SWEEP))) {
                if ((uint64_t)v + 1 > s.nq) {
                    s.nq = (uint64_t)v + 1;
                }
            }
            if ((t & GFS_T_RECORD) && v > s.lb) {
                s.lb = v;
            }
        }
        s.nm += count_results(op);
        if (op->gate == GFS_DETECTOR) {
            s.nd++;
        } else if (op->gate == GFS_OBSERVABLE_INCLUDE) {
            uint64_t k = (uint64_t)op->a[0] + 1;
            if (k > s.no) {
                s.no = k;
            }
        }
    }
    return s;
}

static void init_chan(ochan *ch, const double *w, size_t nw, double p) {
    memset(ch, 0, sizeof(*ch));
    ch->total = p;
    if (nw) {
        gfs_build_choice_table(w, (uint32_t)nw, ch->cum);
    }
    if (!(p > 0)) {
        return;
    }
    ch->active = 1;
    if (p >= 1) {
        ch->always = 1;
        return;
    }
    ch->table = (uint32_t *)malloc(GFS_TABLE_LEN * sizeof(uint32_t));
    gfs_build_gap_table(p, ch->table);
    ch->inv_c = gfs_inv_c(p);
}

static void prepare_channels(oracle_circuit *circ) {
    for (size_t b = 0; b < circ->nblocks; b++) {
        for (size_t i = 0; i < circ->blocks[b].n; i++) {
            oinst *op = &circ->blocks[b].ops[i];
            double p = 0;
            size_t nw = 0;
            switch (op->gate) {
                case GFS_PAULI_CHANNEL_1:
                case GFS_PAULI_CHANNEL_2:
                case GFS_HERALDED_PAULI_CHANNEL_1:
                    nw = op->na;
                    for (size_t k = 0; k < op->na; k++) {
                        p += op->a[k];
                    }
                    break;
                case GFS_X_ERROR:
                case GFS_Y_ERROR:
                case GFS_Z_ERROR:
                case GFS_DEPOLARIZE1:
                case GFS_DEPOLARIZE2:
                case GFS_E:
                case GFS_ELSE_CORRELATED_ERROR:
                case GFS_HERALDED_ERASE:
                    p = op->a[0];
                    break;
                default:
                    if ((ginfo(op->gate)->flags & GFS_F_RESULTS) && op->na) {
                        p = op->a[0];
                    }
            }
            init_chan(&op->ch, op->a, nw, p);
        }
    }
}

oracle_circuit *oracle_parse(const char *text, char *err, size_t err_len) {
    oerr e = {err, err_len, 0};
    oracle_circuit *circ = (oracle_circuit *)calloc(1, sizeof(oracle_circuit));
    new_block(circ);
    oparse p = {text, strlen(text), 0, &e};
    parse_block(circ, 0, &p, 0);
    if (e.failed) {
        oracle_free(circ);
        return NULL;
    }
    ostats s = block_stats(circ, 0);
    circ->num_qubits = s.nq;
    circ->num_meas = s.nm;
    circ->num_dets = s.nd;
    circ->num_obs = s.no;
    circ->max_lookback = s.lb;
    circ->num_inst = s.ni;
    prepare_channels(circ);
    return circ;
}

void oracle_free(oracle_circuit *c) {
    if (!c) {
        return;
    }
    for (size_t b = 0; b < c->nblocks; b++) {
        for (size_t i = 0; i < c->blocks[b].n; i++) {
            free_op(&c->blocks[b].ops[i]);
            free(c->blocks[b].ops[i].ch.table);
        }
        free(c->blocks[b].ops);
    }
    free(c->blocks);
    free(c);
}

void oracle_stats(const oracle_circuit *c, uint64_t *out) {
    out[0] = c->num_qubits;
    out[1] = c->num_meas;
    out[2] = c->num_dets;
    out[3] = c->num_obs;
    out[4] = c->max_lookback;
    out[5] = c->num_inst;
}

/* ------------------------------------------------------------------------------------------------ */
/* Simulation over one batch of shots                                                               */
/* ------------------------------------------------------------------------------------------------ */

typedef struct osim {
    const oracle_circuit *c;
    size_t nw;      /* u64 words per row */
    size_t nblocks; /* 128-shot blocks in the batch */
    uint64_t first_block;
    uint64_t seed;
    uint64_t *x, *z, *rec, *det, *obs, *occ, *tmp;
    uint64_t m, d, inst;
    /* decomposition scratch (per qubit) */
    uint8_t *px, *pz, *merged;
    uint32_t *qlist;
    oerr *e;
} osim;

#define XR(s, q) ((s)->x + (size_t)(q) * (s)->nw)
#define ZR(s, q) ((s)->z + (size_t)(q) * (s)->nw)

static void rand_row(osim *s, uint64_t *row, uint32_t purpose, uint64_t inst, uint32_t unit) {
    for (size_t b = 0; b < s->nblocks; b++) {
        gfs_u32x4 r = gfs_row_bits(s->seed, purpose, inst, unit, (uint32_t)(s->first_block + b));
        row[2 * b] = (uint64_t)r.v[0] | ((uint64_t)r.v[1] << 32);
        row[2 * b + 1] = (uint64_t)r.v[2] | ((uint64_t)r.v[3] << 32);
    }
}

static void row_xor(uint64_t *dst, const uint64_t *src, size_t n) {
    for (size_t k = 0; k < n; k++) {
        dst[k] ^= src[k];
    }
}

static void flip(uint64_t *row, size_t shot) {
    row[shot >> 6] ^= (uint64_t)1 << (shot & 63);
}

static uint64_t *lookback(osim *s, uint32_t k) {
    if (k == 0) {
        seterr(s->e, "Lookback must be non-zero.");
        return NULL;
    }
    if (k > s->m) {
        seterr(s->e, "Referred to a measurement record before the beginning of time.");
        return NULL;
    }
    return s->rec + (size_t)(s->m - k) * s->nw;
}

static uint64_t *new_result(osim *s) {
    uint64_t *r = s->rec + (size_t)s->m * s->nw;
    s->m++;
    return r;
}

/* hit callback context */
typedef void (*hit_fn)(osim *s, const oinst *op, size_t unit, size_t shot, gfs_stream *st, void *ctx);

/* The hits of every segment of a noise instruction (contract in gfs_contract.h). */
static void walk_hits(osim *s, const oinst *op, uint32_t purpose, size_t nunits, hit_fn fn, void *ctx) {
    const ochan *ch = &op->ch;
    if (!ch->active || nunits == 0) {
        return;
    }
    size_t nseg = (nunits + GFS_SEG_UNITS - 1) / GFS_SEG_UNITS;
    for (size_t b = 0; b < s->nblocks; b++) {
        for (size_t g = 0; g < nseg; g++) {
            size_t u0 = g * GFS_SEG_UNITS;
            size_t nu = nunits - u0 < GFS_SEG_UNITS ? nunits - u0 : GFS_SEG_UNITS;
            int32_t trials = (int32_t)(nu * GFS_BLOCK_SHOTS);
            gfs_stream st;
            gfs_stream_init(&st, s->seed, purpose, s->inst, (uint32_t)g, (uint32_t)(s->first_block + b));
            int32_t pos = -1;
            while ((pos = gfs_next_hit(&st, ch->table, ch->inv_c, pos, trials, ch->always)) >= 0) {
                fn(s, op, u0 + (size_t)pos / GFS_BLOCK_SHOTS, b * GFS_BLOCK_SHOTS + (size_t)pos % GFS_BLOCK_SHOTS,
                   &st, ctx);
            }
        }
    }
}

static void apply_pauli(osim *s, uint32_t q, size_t shot, uint32_t v) { /* 0=I 1=X 2=Y 3=Z */
    if (v == 1 || v == 2) {
        flip(XR(s, q), shot);
    }
    if (v == 2 || v == 3) {
        flip(ZR(s, q), shot);
    }
}

static void hit_x(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    flip(XR(s, op->t[u] & GFS_T_VALUE_MASK), shot);
}
static void hit_y(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    flip(XR(s, op->t[u] & GFS_T_VALUE_MASK), shot);
    flip(ZR(s, op->t[u] & GFS_T_VALUE_MASK), shot);
}
static void hit_z(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    flip(ZR(s, op->t[u] & GFS_T_VALUE_MASK), shot);
}
static void hit_dep1(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    uint32_t v = 1 + gfs_choice_uniform(gfs_stream_next(st), 3);
    uint32_t q = op->t[u] & GFS_T_VALUE_MASK;
    if (v & 1) {
        flip(XR(s, q), shot);
    }
    if (v & 2) {
        flip(ZR(s, q), shot);
    }
}
static void hit_dep2(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    uint32_t v = 1 + gfs_choice_uniform(gfs_stream_next(st), 15);
    uint32_t q1 = op->t[2 * u] & GFS_T_VALUE_MASK, q2 = op->t[2 * u + 1] & GFS_T_VALUE_MASK;
    if (v & 1) {
        flip(XR(s, q1), shot);
    }
    if (v & 2) {
        flip(ZR(s, q1), shot);
    }
    if (v & 4) {
        flip(XR(s, q2), shot);
    }
    if (v & 8) {
        flip(ZR(s, q2), shot);
    }
}
static void hit_pc1(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    uint32_t v = 1 + gfs_choice_weighted(gfs_stream_next(st), op->ch.cum, 3);
    apply_pauli(s, op->t[u] & GFS_T_VALUE_MASK, shot, v);
}
static void hit_pc2(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    uint32_t v = 1 + gfs_choice_weighted(gfs_stream_next(st), op->ch.cum, 15);
    apply_pauli(s, op->t[2 * u] & GFS_T_VALUE_MASK, shot, v >> 2);
    apply_pauli(s, op->t[2 * u + 1] & GFS_T_VALUE_MASK, shot, v & 3);
}
static void hit_mask(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    flip((uint64_t *)ctx, shot);
}
static void hit_result(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    uint64_t first = *(const uint64_t *)ctx;
    flip(s->rec + (size_t)(first + u) * s->nw, shot);
}
static void hit_erase(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    uint64_t first = *(const uint64_t *)ctx;
    uint32_t c = gfs_stream_next(st);
    uint32_t q = op->t[u] & GFS_T_VALUE_MASK;
    uint64_t *r = s->rec + (size_t)(first + u) * s->nw;
    r[shot >> 6] |= (uint64_t)1 << (shot & 63);
    if (c & 1) {
        flip(XR(s, q), shot);
    }
    if (c & 2) {
        flip(ZR(s, q), shot);
    }
}
static void hit_hpc1(osim *s, const oinst *op, size_t u, size_t shot, gfs_stream *st, void *ctx) {
    uint64_t first = *(const uint64_t *)ctx;
    uint32_t c = gfs_stream_next(st);
    uint64_t *r = s->rec + (size_t)(first + u) * s->nw;
    r[shot >> 6] |= (uint64_t)1 << (shot & 63);
    apply_pauli(s, op->t[u] & GFS_T_VALUE_MASK, shot, gfs_choice_weighted(c, op->ch.cum, 4));
}

/* --- single-qubit frame rules (frame_simulator.inl:344-384) --- */
static void g_hxz(osim *s, uint32_t q) {
    uint64_t *x = XR(s, q), *z = ZR(s, q);
    for (size_t k = 0; k < s->nw; k++) {
        uint64_t t = x[k];
        x[k] = z[k];
        z[k] = t;
    }
}
static void g_hxy(osim *s, uint32_t q) {
    row_xor(ZR(s, q), XR(s, q), s->nw);
}
static void g_hyz(osim *s, uint32_t q) {
    row_xor(XR(s, q), ZR(s, q), s->nw);
}
static void g_cxyz(osim *s, uint32_t q) {
    row_xor(XR(s, q), ZR(s, q), s->nw);
    row_xor(ZR(s, q), XR(s, q), s->nw);
}
static void g_czyx(osim *s, uint32_t q) {
    row_xor(ZR(s, q), XR(s, q), s->nw);
    row_xor(XR(s, q), ZR(s, q), s->nw);
}

/* --- two-qubit frame rules (frame_simulator.inl:386-630) --- */
static int is_bit(uint32_t t) {
    return (t & (GFS_T_RECORD | GFS_T_SWEEP)) != 0;
}

/* XOR a classical control bit row (record lookback or sweep bit; sweep bits read as zero). */
static void xor_control(osim *s, uint32_t c, uint64_t *dst) {
    if (c & GFS_T_RECORD) {
        uint64_t *r = lookback(s, c & GFS_T_VALUE_MASK);
        if (r) {
            row_xor(dst, r, s->nw);
        }
    }
}

static void single_cx(osim *s, uint32_t c, uint32_t t) {
    c &= ~GFS_T_INVERTED;
    t &= ~GFS_T_INVERTED;
    if (!is_bit(c) && !is_bit(t)) {
        row_xor(ZR(s, c), ZR(s, t), s->nw);
        row_xor(XR(s, t), XR(s, c), s->nw);
    } else if (is_bit(t)) {
        seterr(s->e, "Controlled X had a bit as its target, instead of its control.");
    } else {
        xor_control(s, c, XR(s, t & GFS_T_VALUE_MASK));
    }
}

static void single_cy(osim *s, uint32_t c, uint32_t t) {
    c &= ~GFS_T_INVERTED;
    t &= ~GFS_T_INVERTED;
    if (!is_bit(c) && !is_bit(t)) {
        uint64_t *x1 = XR(s, c), *z1 = ZR(s, c), *x2 = XR(s, t), *z2 = ZR(s, t);
        for (size_t k = 0; k < s->nw; k++) {
            z1[k] ^= x2[k] ^ z2[k];
            z2[k] ^= x1[k];
            x2[k] ^= x1[k];
        }
    } else if (is_bit(t)) {
        seterr(s->e, "Controlled Y had a bit as its target, instead of its control.");
    } else {
        xor_control(s, c, XR(s, t & GFS_T_VALUE_MASK));
        xor_control(s, c, ZR(s, t & GFS_T_VALUE_MASK));
    }
}

static void single_cz(osim *s, uint32_t c, uint32_t t) {
    c &= ~GFS_T_INVERTED;
    t &= ~GFS_T_INVERTED;
    if (!is_bit(c) && !is_bit(t)) {
        row_xor(ZR(s, c), XR(s, t), s->nw);
        row_xor(ZR(s, t), XR(s, c), s->nw);
    } else if (!is_bit(t)) {
        xor_control(s, c, ZR(s, t & GFS_T_VALUE_MASK));
    } else if (!is_bit(c)) {
        xor_control(s, t, ZR(s, c & GFS_T_VALUE_MASK));
    }
}

static void pair_rule(osim *s, gfs_gate g, uint32_t a, uint32_t b) {
    uint64_t *x1 = XR(s, a), *z1 = ZR(s, a), *x2 = XR(s, b), *z2 = ZR(s, b);
    for (size_t k = 0; k < s->nw; k++) {
        uint64_t X1 = x1[k], Z1 = z1[k], X2 = x2[k], Z2 = z2[k];
        switch (g) {
            case GFS_SWAP:
                x1[k] = X2;
                z1[k] = Z2;
                x2[k] = X1;
                z2[k] = Z1;
                break;
            case GFS_ISWAP:
            case GFS_ISWAP_DAG: {
                uint64_t dx = X1 ^ X2;
                z1[k] = Z2 ^ dx;
                z2[k] = Z1 ^ dx;
                x1[k] = X2;
                x2[k] = X1;
                break;
            }
            case GFS_CXSWAP:
                Z2 ^= Z1;
                Z1 ^= Z2;
                X1 ^= X2;
                X2 ^= X1;
                x1[k] = X1;
                z1[k] = Z1;
                x2[k] = X2;
                z2[k] = Z2;
                break;
            case GFS_CZSWAP:
                x1[k] = X2;
                z1[k] = Z2 ^ X1;
                x2[k] = X1;
                z2[k] = Z1 ^ X2;
                break;
            case GFS_SWAPCX:
                Z1 ^= Z2;
                Z2 ^= Z1;
                X2 ^= X1;
                X1 ^= X2;
                x1[k] = X1;
                z1[k] = Z1;
                x2[k] = X2;
                z2[k] = Z2;
                break;
            case GFS_SQRT_XX:
            case GFS_SQRT_XX_DAG: {
                uint64_t dz = Z1 ^ Z2;
                x1[k] = X1 ^ dz;
                x2[k] = X2 ^ dz;
                break;
            }
            case GFS_SQRT_YY:
            case GFS_SQRT_YY_DAG: {
                uint64_t d = X1 ^ Z1 ^ X2 ^ Z2;
                x1[k] = X1 ^ d;
                z1[k] = Z1 ^ d;
                x2[k] = X2 ^ d;
                z2[k] = Z2 ^ d;
                break;
            }
            case GFS_SQRT_ZZ:
            case GFS_SQRT_ZZ_DAG: {
                uint64_t dx = X1 ^ X2;
                z1[k] = Z1 ^ dx;
                z2[k] = Z2 ^ dx;
                break;
            }
            case GFS_XCX:
                x1[k] = X1 ^ Z2;
                x2[k] = X2 ^ Z1;
                break;
            case GFS_XCY:
                x1[k] = X1 ^ X2 ^ Z2;
                x2[k] = X2 ^ Z1;
                z2[k] = Z2 ^ Z1;
                break;
            case GFS_YCX:
                x2[k] = X2 ^ X1 ^ Z1;
                x1[k] = X1 ^ Z2;
                z1[k] = Z1 ^ Z2;
                break;
            case GFS_YCY: {
                uint64_t y1 = X1 ^ Z1, y2 = X2 ^ Z2;
                x1[k] = X1 ^ y2;
                z1[k] = Z1 ^ y2;
                x2[k] = X2 ^ y1;
                z2[k] = Z2 ^ y1;
                break;
            }
            default:
                break;
        }
    }
}

static void do_two_qubit(osim *s, const oinst *op) {
    for (size_t k = 0; k + 1 < op->nt && !s->e->failed; k += 2) {
        uint32_t a = op->t[k], b = op->t[k + 1];
        switch (op->gate) {
            case GFS_CX:
                single_cx(s, a, b);
                break;
            case GFS_CY:
                single_cy(s, a, b);
                break;
            case GFS_CZ:
                single_cz(s, a, b);
                break;
            case GFS_XCZ:
                single_cx(s, b, a);
                break;
            case GFS_YCZ:
                single_cy(s, b, a);
                break;
            case GFS_II:
                break;
            default:
                pair_rule(s, op->gate, a & GFS_T_VALUE_MASK, b & GFS_T_VALUE_MASK);
        }
    }
}

/* --- collapsing rules (frame_simulator.inl:172-317) --- */
static void collapse_one(osim *s, gfs_gate g, uint32_t q, uint32_t unit) {
    uint64_t *x = XR(s, q), *z = ZR(s, q);
    size_t nw = s->nw;
    switch (g) {
        case GFS_M:
            memcpy(new_result(s), x, nw * 8);
            rand_row(s, z, GFS_P_RAND, s->inst, unit);
            break;
        case GFS_MX:
            memcpy(new_result(s), z, nw * 8);
            rand_row(s, x, GFS_P_RAND, s->inst, unit);
            break;
        case GFS_MY: {
            uint64_t *r = new_result(s);
            for (size_t k = 0; k < nw; k++) {
                r[k] = x[k] ^ z[k];
            }
            /* x ^= z; record; z = rand; x ^= z  ==>  x = x ^ z_old ^ rand */
            for (size_t k = 0; k < nw; k++) {
                x[k] ^= z[k];
            }
            rand_row(s, z, GFS_P_RAND, s->inst, unit);
            row_xor(x, z, nw);
            break;
        }
        case GFS_MR:
            memcpy(new_result(s), x, nw * 8);
            memset(x, 0, nw * 8);
            rand_row(s, z, GFS_P_RAND, s->inst, unit);
            break;
        case GFS_MRX:
            memcpy(new_result(s), z, nw * 8);
            memset(z, 0, nw * 8);
            rand_row(s, x, GFS_P_RAND, s->inst, unit);
            break;
        case GFS_MRY: {
            uint64_t *r = new_result(s);
            for (size_t k = 0; k < nw; k++) {
                r[k] = x[k] ^ z[k];
            }
            rand_row(s, z, GFS_P_RAND, s->inst, unit);
            memcpy(x, z, nw * 8);
            break;
        }
        case GFS_R:
            memset(x, 0, nw * 8);
            rand_row(s, z, GFS_P_RAND, s->inst, unit);
            break;
        case GFS_RX:
            rand_row(s, x, GFS_P_RAND, s->inst, unit);
            memset(z, 0, nw * 8);
            break;
        case GFS_RY:
            rand_row(s, z, GFS_P_RAND, s->inst, unit);
            memcpy(x, z, nw * 8);
            break;
        default:
            break;
    }
}

static void flip_results(osim *s, const oinst *op, uint64_t first, size_t n) {
    walk_hits(s, op, GFS_P_MNOISE, n, hit_result, &first);
}

static void do_collapse(osim *s, const oinst *op) {
    uint64_t first = s->m;
    for (size_t k = 0; k < op->nt; k++) {
        collapse_one(s, op->gate, op->t[k] & GFS_T_VALUE_MASK, (uint32_t)k);
    }
    if (ginfo(op->gate)->flags & GFS_F_RESULTS) {
        flip_results(s, op, first, op->nt);
    }
}

/* --- MPP (gate_decomposition.cc:88-161) --- */
typedef struct qvec {
    uint32_t *v;
    size_t n, cap;
} qvec;
static void qpush(qvec *q, uint32_t x) {
    if (q->n == q->cap) {
        q->cap = q->cap ? q->cap * 2 : 16;
        q->v = (uint32_t *)realloc(q->v, q->cap * sizeof(uint32_t));
    }
    q->v[q->n++] = x;
}

typedef struct mpp_state {
    qvec hxz, hyz, cnot, meas, touched;
} mpp_state;

static void mpp_flush(osim *s, mpp_state *st, uint32_t *result) {
    if (st->meas.n == 0) {
        return;
    }
    for (size_t k = 0; k < st->hxz.n; k++) {
        g_hxz(s, st->hxz.v[k]);
    }
    for (size_t k = 0; k < st->hyz.n; k++) {
        g_hyz(s, st->hyz.v[k]);
    }
    for (size_t k = 0; k < st->cnot.n; k += 2) {
        single_cx(s, st->cnot.v[k], st->cnot.v[k + 1]);
    }
    for (size_t k = 0; k < st->meas.n; k++) {
        collapse_one(s, GFS_M, st->meas.v[k], (*result)++);
    }
    for (size_t k = 0; k < st->cnot.n; k += 2) {
        single_cx(s, st->cnot.v[k], st->cnot.v[k + 1]);
    }
    for (size_t k = 0; k < st->hyz.n; k++) {
        g_hyz(s, st->hyz.v[k]);
    }
    for (size_t k = 0; k < st->hxz.n; k++) {
        g_hxz(s, st->hxz.v[k]);
    }
    for (size_t k = 0; k < st->touched.n; k++) {
        s->merged[st->touched.v[k]] = 0;
    }
    st->hxz.n = st->hyz.n = st->cnot.n = st->meas.n = st->touched.n = 0;
}

/* Accumulates the product starting at targets[*start] into px/pz (for qubits in `q`);
   returns 1 if a product was read.  Classical bits go to `bits` when given. */
static int read_product(osim *s, const oinst *op, size_t *start, qvec *q, qvec *bits, int *imag_out) {
    if (*start >= op->nt) {
        return 0;
    }
    size_t end = *start + 1;
    while (end < op->nt && (op->t[end] & GFS_T_COMBINER)) {
        end += 2;
    }
    int imag = 0;
    for (size_t k = *start; k < end; k += 2) {
        uint32_t t = op->t[k];
        if (t & (GFS_T_PAULI_X | GFS_T_PAULI_Z)) {
            uint32_t qq = t & GFS_T_VALUE_MASK;
            uint8_t nx = (t & GFS_T_PAULI_X) ? 1 : 0, nz = (t & GFS_T_PAULI_Z) ? 1 : 0;
            uint8_t ox = s->px[qq], oz = s->pz[qq];
            if (!ox && !oz) {
                qpush(q, qq);
            }
            /* single-qubit Paulis anticommute when x1 z2 ^ z1 x2 is set */
            if ((ox & nz) ^ (oz & nx)) {
                imag ^= 1;
            }
            s->px[qq] ^= nx;
            s->pz[qq] ^= nz;
        } else if ((t & (GFS_T_RECORD | GFS_T_SWEEP)) && bits) {
            qpush(bits, t);
        } else {
            seterr(s->e, "Found an unsupported target in a Pauli product.");
            return 0;
        }
    }
    *imag_out = imag;
    *start = end;
    return 1;
}

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}

static void do_mpp(osim *s, const oinst *op) {
    mpp_state st;
    memset(&st, 0, sizeof(st));
    qvec q = {0};
    uint64_t first = s->m;
    uint32_t result = 0;
    size_t start = 0;
    int imag;
    while (!s->e->failed && read_product(s, op, &start, &q, NULL, &imag)) {
        if (imag) {
            seterr(s->e, "Acted on an anti-Hermitian operator (e.g. X0*Z0 instead of Y0) in MPP.");
            break;
        }
        /* active qubits in increasing order */
        qsort(q.v, q.n, sizeof(uint32_t), cmp_u32);
        size_t nactive = 0;
        int overlap = 0;
        for (size_t k = 0; k < q.n; k++) {
            uint32_t qq = q.v[k];
            if (nactive && q.v[nactive - 1] == qq) {
                continue; /* a qubit can be listed twice if its term cancelled and reappeared */
            }
            if (s->px[qq] || s->pz[qq]) {
                q.v[nactive++] = qq;
                if (s->merged[qq]) {
                    overlap = 1;
                }
            }
        }
        if (nactive == 0) {
            mpp_flush(s, &st, &result);
            memset(new_result(s), 0, s->nw * 8);
            result++;
        } else {
            if (overlap) {
                mpp_flush(s, &st, &result);
            }
            for (size_t k = 0; k < nactive; k++) {
                uint32_t qq = q.v[k];
                if (!s->merged[qq]) {
                    s->merged[qq] = 1;
                    qpush(&st.touched, qq);
                }
                if (s->px[qq]) {
                    qpush(s->pz[qq] ? &st.hyz : &st.hxz, qq);
                }
                if (k == 0) {
                    qpush(&st.meas, qq);
                } else {
                    qpush(&st.cnot, qq);
                    qpush(&st.cnot, q.v[0]);
                }
            }
        }
        for (size_t k = 0; k < nactive; k++) {
            s->px[q.v[k]] = s->pz[q.v[k]] = 0;
        }
        q.n = 0;
    }
    mpp_flush(s, &st, &result);
    if (op->na) {
        flip_results(s, op, first, result);
    }
    free(q.v);
    free(st.hxz.v);
    free(st.hyz.v);
    free(st.cnot.v);
    free(st.meas.v);
    free(st.touched.v);
}

/* --- SPP / SPP_DAG (gate_decomposition.cc:163-250) --- */
static void do_spp(osim *s, const oinst *op) {
    qvec q = {0}, bits = {0}, hxz = {0}, hyz = {0}, cnot = {0};
    size_t start = 0;
    int imag;
    while (!s->e->failed && (bits.n = 0, q.n = 0, read_product(s, op, &start, &q, &bits, &imag))) {
        if (imag) {
            seterr(s->e, "Acted on an anti-Hermitian operator (e.g. X0*Z0 instead of Y0) in SPP.");
            break;
        }
        qsort(q.v, q.n, sizeof(uint32_t), cmp_u32);
        hxz.n = hyz.n = cnot.n = 0;
        int64_t focus = -1;
        for (size_t k = 0; k < q.n; k++) {
            uint32_t qq = q.v[k];
            if ((k && q.v[k - 1] == qq) || (!s->px[qq] && !s->pz[qq])) {
                continue;
            }
            if (s->px[qq]) {
                qpush(s->pz[qq] ? &hyz : &hxz, qq);
            }
            if (focus < 0) {
                focus = qq;
            } else {
                qpush(&cnot, qq);
                qpush(&cnot, (uint32_t)focus);
            }
        }
        for (size_t k = 0; k < q.n; k++) {
            s->px[q.v[k]] = s->pz[q.v[k]] = 0;
        }
        if (focus < 0) {
            continue;
        }
        for (size_t k = 0; k < bits.n; k++) {
            qpush(&cnot, bits.v[k]);
            qpush(&cnot, (uint32_t)focus);
        }
        for (size_t k = 0; k < hxz.n; k++) {
            g_hxz(s, hxz.v[k]);
        }
        for (size_t k = 0; k < hyz.n; k++) {
            g_hyz(s, hyz.v[k]);
        }
        for (size_t k = 0; k < cnot.n; k += 2) {
            single_cx(s, cnot.v[k], cnot.v[k + 1]);
        }
        g_hxy(s, (uint32_t)focus); /* S and S_DAG act alike on frames */
        for (size_t k = 0; k < cnot.n; k += 2) {
            single_cx(s, cnot.v[k], cnot.v[k + 1]);
        }
        for (size_t k = 0; k < hyz.n; k++) {
            g_hyz(s, hyz.v[k]);
        }
        for (size_t k = 0; k < hxz.n; k++) {
            g_hxz(s, hxz.v[k]);
        }
    }
    free(q.v);
    free(bits.v);
    free(hxz.v);
    free(hyz.v);
    free(cnot.v);
}

/* --- MXX / MYY / MZZ (frame_simulator.inl:841-902, gate_decomposition.cc:319-347) --- */
static void do_pair_measure(osim *s, const oinst *op) {
    uint64_t first = s->m;
    uint32_t result = 0;
    size_t flushed = 0, cur = 0;
    qvec used = {0};
    while (flushed < op->nt) {
        int end_seg = 0;
        if (cur < op->nt) {
            uint32_t q0 = op->t[cur] & GFS_T_VALUE_MASK, q1 = op->t[cur + 1] & GFS_T_VALUE_MASK;
            if (s->merged[q0] || s->merged[q1]) {
                end_seg = 1;
            } else {
                s->merged[q0] = s->merged[q1] = 1;
                qpush(&used, q0);
                qpush(&used, q1);
                cur += 2;
            }
        } else {
            end_seg = 1;
        }
        if (end_seg) {
            for (int pass = 0; pass < 2; pass++) {
                for (size_t k = flushed; k < cur; k += 2) {
                    uint32_t a = op->t[k] & GFS_T_VALUE_MASK, b = op->t[k + 1] & GFS_T_VALUE_MASK;
                    if (op->gate == GFS_MXX) {
                        single_cx(s, a, b);
                    } else if (op->gate == GFS_MYY) {
                        single_cy(s, a, b);
                    } else {
                        single_cx(s, b, a);
                    }
                }
                if (pass == 0) {
                    gfs_gate mg = op->gate == GFS_MXX ? GFS_MX : op->gate == GFS_MYY ? GFS_MY : GFS_M;
                    for (size_t k = flushed; k < cur; k += 2) {
                        collapse_one(s, mg, op->t[k] & GFS_T_VALUE_MASK, result++);
                    }
                }
            }
            for (size_t k = 0; k < used.n; k++) {
                s->merged[used.v[k]] = 0;
            }
            used.n = 0;
            flushed = cur;
        }
    }
    free(used.v);
    if (op->na) {
        flip_results(s, op, first, result);
    }
}

static void do_detector(osim *s, const oinst *op) {
    uint64_t *r = s->det + (size_t)s->d * s->nw;
    s->d++;
    memset(r, 0, s->nw * 8);
    for (size_t k = 0; k < op->nt; k++) {
        uint64_t *src = lookback(s, op->t[k] & GFS_T_VALUE_MASK);
        if (!src) {
            return;
        }
        row_xor(r, src, s->nw);
    }
}

static void do_observable(osim *s, const oinst *op) {
    uint64_t *r = s->obs + (size_t)op->a[0] * s->nw;
    for (size_t k = 0; k < op->nt; k++) {
        uint32_t t = op->t[k];
        if (t & GFS_T_RECORD) {
            uint64_t *src = lookback(s, t & GFS_T_VALUE_MASK);
            if (!src) {
                return;
            }
            row_xor(r, src, s->nw);
        } else {
            uint32_t q = t & GFS_T_VALUE_MASK;
            if (t & GFS_T_PAULI_X) {
                row_xor(r, ZR(s, q), s->nw);
            }
            if (t & GFS_T_PAULI_Z) {
                row_xor(r, XR(s, q), s->nw);
            }
        }
    }
}

static void do_correlated(osim *s, const oinst *op) {
    if (op->gate == GFS_E) {
        memset(s->occ, 0, s->nw * 8);
    }
    memset(s->tmp, 0, s->nw * 8);
    walk_hits(s, op, GFS_P_NOISE, 1, hit_mask, s->tmp);
    for (size_t k = 0; k < s->nw; k++) {
        s->tmp[k] &= ~s->occ[k];
        s->occ[k] |= s->tmp[k];
    }
    for (size_t k = 0; k < op->nt; k++) {
        uint32_t t = op->t[k], q = t & GFS_T_VALUE_MASK;
        if (t & GFS_T_PAULI_X) {
            row_xor(XR(s, q), s->tmp, s->nw);
        }
        if (t & GFS_T_PAULI_Z) {
            row_xor(ZR(s, q), s->tmp, s->nw);
        }
    }
}

static void do_heralded(osim *s, const oinst *op) {
    uint64_t first = s->m;
    for (size_t k = 0; k < op->nt; k++) {
        memset(new_result(s), 0, s->nw * 8);
    }
    walk_hits(s, op, GFS_P_NOISE, op->nt, op->gate == GFS_HERALDED_ERASE ? hit_erase : hit_hpc1, &first);
}

static void do_op(osim *s, const oinst *op) {
    switch (op->gate) {
        case GFS_H:
        case GFS_H_NXZ:
        case GFS_SQRT_Y:
        case GFS_SQRT_Y_DAG:
            for (size_t k = 0; k < op->nt; k++) {
                g_hxz(s, op->t[k] & GFS_T_VALUE_MASK);
            }
            break;
        case GFS_S:
        case GFS_S_DAG:
        case GFS_H_XY:
        case GFS_H_NXY:
            for (size_t k = 0; k < op->nt; k++) {
                g_hxy(s, op->t[k] & GFS_T_VALUE_MASK);
            }
            break;
        case GFS_SQRT_X:
        case GFS_SQRT_X_DAG:
        case GFS_H_YZ:
        case GFS_H_NYZ:
            for (size_t k = 0; k < op->nt; k++) {
                g_hyz(s, op->t[k] & GFS_T_VALUE_MASK);
            }
            break;
        case GFS_C_XYZ:
        case GFS_C_NXYZ:
        case GFS_C_XNYZ:
        case GFS_C_XYNZ:
            for (size_t k = 0; k < op->nt; k++) {
                g_cxyz(s, op->t[k] & GFS_T_VALUE_MASK);
            }
            break;
        case GFS_C_ZYX:
        case GFS_C_NZYX:
        case GFS_C_ZNYX:
        case GFS_C_ZYNX:
            for (size_t k = 0; k < op->nt; k++) {
                g_czyx(s, op->t[k] & GFS_T_VALUE_MASK);
            }
            break;
        case GFS_CX:
        case GFS_CY:
        case GFS_CZ:
        case GFS_XCX:
        case GFS_XCY:
        case GFS_XCZ:
        case GFS_YCX:
        case GFS_YCY:
        case GFS_YCZ:
        case GFS_SWAP:
        case GFS_ISWAP:
        case GFS_ISWAP_DAG:
        case GFS_CXSWAP:
        case GFS_SWAPCX:
        case GFS_CZSWAP:
        case GFS_SQRT_XX:
        case GFS_SQRT_XX_DAG:
        case GFS_SQRT_YY:
        case GFS_SQRT_YY_DAG:
        case GFS_SQRT_ZZ:
        case GFS_SQRT_ZZ_DAG:
        case GFS_II:
            do_two_qubit(s, op);
            break;
        case GFS_M:
        case GFS_MX:
        case GFS_MY:
        case GFS_MR:
        case GFS_MRX:
        case GFS_MRY:
        case GFS_R:
        case GFS_RX:
        case GFS_RY:
            do_collapse(s, op);
            break;
        case GFS_MPP:
            do_mpp(s, op);
            break;
        case GFS_SPP:
        case GFS_SPP_DAG:
            do_spp(s, op);
            break;
        case GFS_MXX:
        case GFS_MYY:
        case GFS_MZZ:
            do_pair_measure(s, op);
            break;
        case GFS_MPAD: {
            uint64_t first = s->m;
            for (size_t k = 0; k < op->nt; k++) {
                memset(new_result(s), 0, s->nw * 8);
            }
            flip_results(s, op, first, op->nt);
            break;
        }
        case GFS_DETECTOR:
            do_detector(s, op);
            break;
        case GFS_OBSERVABLE_INCLUDE:
            do_observable(s, op);
            break;
        case GFS_X_ERROR:
            walk_hits(s, op, GFS_P_NOISE, op->nt, hit_x, NULL);
            break;
        case GFS_Y_ERROR:
            walk_hits(s, op, GFS_P_NOISE, op->nt, hit_y, NULL);
            break;
        case GFS_Z_ERROR:
            walk_hits(s, op, GFS_P_NOISE, op->nt, hit_z, NULL);
            break;
        case GFS_DEPOLARIZE1:
            walk_hits(s, op, GFS_P_NOISE, op->nt, hit_dep1, NULL);
            break;
        case GFS_DEPOLARIZE2:
            walk_hits(s, op, GFS_P_NOISE, op->nt / 2, hit_dep2, NULL);
            break;
        case GFS_PAULI_CHANNEL_1:
            walk_hits(s, op, GFS_P_NOISE, op->nt, hit_pc1, NULL);
            break;
        case GFS_PAULI_CHANNEL_2:
            walk_hits(s, op, GFS_P_NOISE, op->nt / 2, hit_pc2, NULL);
            break;
        case GFS_E:
        case GFS_ELSE_CORRELATED_ERROR:
            do_correlated(s, op);
            break;
        case GFS_HERALDED_ERASE:
        case GFS_HERALDED_PAULI_CHANNEL_1:
            do_heralded(s, op);
            break;
        default: /* TICK, coordinates, Pauli gates, I, II, I_ERROR, II_ERROR */
            break;
    }
    s->inst++;
}

static void run_block(osim *s, size_t b) {
    const oblock *blk = &s->c->blocks[b];
    for (size_t i = 0; i < blk->n && !s->e->failed; i++) {
        const oinst *op = &blk->ops[i];
        if (op->gate == GFS_REPEAT) {
            for (uint64_t r = 0; r < op->reps && !s->e->failed; r++) {
                run_block(s, op->block);
            }
        } else {
            do_op(s, op);
        }
    }
}

/* ------------------------------------------------------------------------------------------------ */
/* Output transposition: row-major [major][shot] -> shot-major bit-packed bytes                     */
/* ------------------------------------------------------------------------------------------------ */

/* In-place 64x64 bit-matrix transpose (bit j of a[i] <-> bit i of a[j]), recursive block swap. */
static void transpose64(uint64_t a[64]) {
    uint64_t m = 0x00000000FFFFFFFFull;
    for (int j = 32; j != 0; j >>= 1, m ^= (m << j)) {
        for (int k = 0; k < 64; k = ((k | j) + 1) & ~j) {
            uint64_t t = ((a[k] >> j) ^ a[k | j]) & m;
            a[k] ^= t << j;
            a[k | j] ^= t;
        }
    }
}

static void emit_rows(const uint64_t *rows, uint64_t nmajor, size_t nw, uint64_t shot0, uint64_t nshots,
                      uint8_t *out) {
    size_t bpr = (size_t)((nmajor + 7) / 8);
    uint64_t blk[64];
    for (uint64_t r0 = 0; r0 < nmajor; r0 += 64) {
        size_t nr = nmajor - r0 < 64 ? (size_t)(nmajor - r0) : 64;
        size_t nbytes = (nr + 7) / 8;
        for (size_t w = 0; w < nw; w++) {
            uint64_t sbase = (uint64_t)w * 64;
            if (sbase >= nshots) {
                break;
            }
            for (size_t i = 0; i < 64; i++) {
                blk[i] = i < nr ? rows[(size_t)(r0 + i) * nw + w] : 0;
            }
            transpose64(blk);
            for (size_t j = 0; j < 64 && sbase + j < nshots; j++) {
                uint8_t *dst = out + (size_t)(shot0 + sbase + j) * bpr + (size_t)(r0 / 8);
                uint64_t v = blk[j];
                for (size_t by = 0; by < nbytes; by++) {
                    dst[by] = (uint8_t)(v >> (8 * by));
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------------ */
/* Batches and threads                                                                              */
/* ------------------------------------------------------------------------------------------------ */

#define ORACLE_BATCH_BLOCKS 8

typedef struct ojob {
    const oracle_circuit *c;
    uint64_t seed, first_shot, num_shots;
    uint8_t *dets, *obs, *meas;
    int tid, nthreads;
    char err[256];
    int failed;
} ojob;

static void *job_main(void *arg) {
    ojob *j = (ojob *)arg;
    const oracle_circuit *c = j->c;
    oerr e = {j->err, sizeof(j->err), 0};
    osim s;
    memset(&s, 0, sizeof(s));
    s.c = c;
    s.e = &e;
    s.seed = j->seed;
    size_t nw_max = ORACLE_BATCH_BLOCKS * 2;
    size_t nq = (size_t)c->num_qubits;
    s.x = (uint64_t *)calloc(nq * nw_max + 1, 8);
    s.z = (uint64_t *)calloc(nq * nw_max + 1, 8);
    s.rec = (uint64_t *)calloc((size_t)c->num_meas * nw_max + 1, 8);
    s.det = (uint64_t *)calloc((size_t)c->num_dets * nw_max + 1, 8);
    s.obs = (uint64_t *)calloc((size_t)c->num_obs * nw_max + 1, 8);
    s.occ = (uint64_t *)calloc(nw_max, 8);
    s.tmp = (uint64_t *)calloc(nw_max, 8);
    s.px = (uint8_t *)calloc(nq + 1, 1);
    s.pz = (uint8_t *)calloc(nq + 1, 1);
    s.merged = (uint8_t *)calloc(nq + 1, 1);
    uint64_t total_blocks = (j->num_shots + GFS_BLOCK_SHOTS - 1) / GFS_BLOCK_SHOTS;
    uint64_t nbatches = (total_blocks + ORACLE_BATCH_BLOCKS - 1) / ORACLE_BATCH_BLOCKS;
    for (uint64_t bt = (uint64_t)j->tid; bt < nbatches && !e.failed; bt += (uint64_t)j->nthreads) {
        uint64_t b0 = bt * ORACLE_BATCH_BLOCKS;
        uint64_t nb = total_blocks - b0 < ORACLE_BATCH_BLOCKS ? total_blocks - b0 : ORACLE_BATCH_BLOCKS;
        s.nblocks = (size_t)nb;
        s.nw = (size_t)nb * 2;
        s.first_block = j->first_shot / GFS_BLOCK_SHOTS + b0;
        s.m = s.d = s.inst = 0;
        memset(s.x, 0, nq * s.nw * 8);
        for (size_t q = 0; q < nq; q++) {
            rand_row(&s, ZR(&s, q), GFS_P_RESET, 0, (uint32_t)q);
        }
        memset(s.obs, 0, (size_t)c->num_obs * s.nw * 8);
        memset(s.occ, 0, s.nw * 8);
        run_block(&s, 0);
        if (e.failed) {
            break;
        }
        uint64_t shot0 = b0 * GFS_BLOCK_SHOTS;
        uint64_t nshots = j->num_shots - shot0 < nb * GFS_BLOCK_SHOTS ? j->num_shots - shot0 : nb * GFS_BLOCK_SHOTS;
        if (j->dets) {
            emit_rows(s.det, c->num_dets, s.nw, shot0, nshots, j->dets);
        }
        if (j->obs) {
            emit_rows(s.obs, c->num_obs, s.nw, shot0, nshots, j->obs);
        }
        if (j->meas) {
            emit_rows(s.rec, c->num_meas, s.nw, shot0, nshots, j->meas);
        }
    }
    j->failed = e.failed;
    free(s.x);
    free(s.z);
    free(s.rec);
    free(s.det);
    free(s.obs);
    free(s.occ);
    free(s.tmp);
    free(s.px);
    free(s.pz);
    free(s.merged);
    return NULL;
}

int oracle_sample(const oracle_circuit *c, uint64_t seed, uint64_t first_shot, uint64_t num_shots, int num_threads,
                  uint8_t *dets, uint8_t *obs, uint8_t *meas, char *err, size_t err_len) {
    if (first_shot % GFS_BLOCK_SHOTS) {
        snprintf(err, err_len, "first_shot must be a multiple of 128");
        return -1;
    }
    if (num_threads < 1) {
        num_threads = 1;
    }
    if (num_threads > 256) {
        num_threads = 256;
    }
    ojob *jobs = (ojob *)calloc((size_t)num_threads, sizeof(ojob));
    pthread_t *th = (pthread_t *)calloc((size_t)num_threads, sizeof(pthread_t));
    for (int t = 0; t < num_threads; t++) {
        jobs[t].c = c;
        jobs[t].seed = seed;
        jobs[t].first_shot = first_shot;
        jobs[t].num_shots = num_shots;
        jobs[t].dets = dets;
        jobs[t].obs = obs;
        jobs[t].meas = meas;
        jobs[t].tid = t;
        jobs[t].nthreads = num_threads;
    }
    if (num_threads == 1) {
        job_main(&jobs[0]);
    } else {
        for (int t = 0; t < num_threads; t++) {
            pthread_create(&th[t], NULL, job_main, &jobs[t]);
        }
        for (int t = 0; t < num_threads; t++) {
            pthread_join(th[t], NULL);
        }
    }
    int rc = 0;
    for (int t = 0; t < num_threads; t++) {
        if (jobs[t].failed) {
            snprintf(err, err_len, "%s", jobs[t].err);
            rc = -1;
            break;
        }
    }
    free(jobs);
    free(th);
    return rc;
}

/* ------------------------------------------------------------------------------------------------ */
/* Measurements to detection events                                                                 */
/* ------------------------------------------------------------------------------------------------ */

/*
 * Restates measurements_to_detection_events_helper (src/stim/simulators/measurements_to_detection_events.inl
 * :29-131) for circuits whose sweep bits are all zero: walking the circuit with REPEAT unrolled, detector d
 * of a shot is the XOR of the measurement bits its rec targets name, inverted when the same bits of the
 * reference sample have odd parity; observable k likewise over all of its OBSERVABLE_INCLUDE rec targets
 * (Pauli targets only read the frame, which stays zero without sweep data).  Bit by bit, one shot at a time.
 */
typedef struct om2d {
    const uint8_t *meas; /* this shot's measurement bits */
    const uint8_t *ref;  /* reference sample bits, or NULL for zeros */
    uint8_t *dets, *obs;
    uint64_t nmeas, ndet;
    int failed;
} om2d;

static int obit(const uint8_t *row, uint64_t i) {
    return (row[i >> 3] >> (i & 7)) & 1;
}

static void om2d_block(const oracle_circuit *circ, size_t b, om2d *s) {
    const oblock *blk = &circ->blocks[b];
    for (size_t i = 0; i < blk->n && !s->failed; i++) {
        const oinst *op = &blk->ops[i];
        if (op->gate == GFS_REPEAT) {
            for (uint64_t r = 0; r < op->reps && !s->failed; r++) {
                om2d_block(circ, op->block, s);
            }
            continue;
        }
        if (op->gate == GFS_DETECTOR || op->gate == GFS_OBSERVABLE_INCLUDE) {
            int v = 0;
            for (size_t k = 0; k < op->nt; k++) {
                uint32_t t = op->t[k];
                if (!(t & GFS_T_RECORD)) {
                    continue;
                }
                uint64_t lb = t & GFS_T_VALUE_MASK;
                if (lb == 0 || lb > s->nmeas) {
                    s->failed = 1;
                    return;
                }
                uint64_t m = s->nmeas - lb;
                v ^= obit(s->meas, m) ^ (s->ref ? obit(s->ref, m) : 0);
            }
            if (op->gate == GFS_DETECTOR) {
                if (v) {
                    s->dets[s->ndet >> 3] |= (uint8_t)(1u << (s->ndet & 7));
                }
                s->ndet++;
            } else if (v) {
                uint64_t k = (uint64_t)op->a[0];
                s->obs[k >> 3] ^= (uint8_t)(1u << (k & 7));
            }
            continue;
        }
        s->nmeas += count_results(op);
    }
}

int oracle_m2d(const oracle_circuit *c, uint64_t shots, const uint8_t *meas, const uint8_t *ref, uint8_t *dets,
               uint8_t *obs, char *err, size_t err_len) {
    oerr e = {err, err_len, 0};
    uint64_t mrow = (c->num_meas + 7) / 8, drow = (c->num_dets + 7) / 8, orow = (c->num_obs + 7) / 8;
    memset(dets, 0, shots * drow);
    memset(obs, 0, shots * orow);
    for (uint64_t s = 0; s < shots; s++) {
        om2d st = {meas + s * mrow, ref, dets + s * drow, obs + s * orow, 0, 0, 0};
        om2d_block(c, 0, &st);
        if (st.failed) {
            seterr(&e, "lookback before the beginning of time");
            return -1;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------------ */
/* Detector error models                                                                            */
/* ------------------------------------------------------------------------------------------------ */

/*
 * Restates the reference's detector-error-model text format (src/stim/dem/detector_error_model.cc:195-360,
 * dem_instruction.cc validate) and DemSampler::resample (src/stim/simulators/dem_sampler.inl:51-77): the
 * error mechanisms are the `error` instructions with repeat blocks unrolled and shift_detectors applied; a
 * sampled or replayed error XORs its detector and observable targets.  Sampling follows the DEM purpose of
 * gfs_contract.h (mechanisms grouped by probability in order of first appearance, each group walked like a
 * noise instruction whose units are its mechanisms).
 */
struct oracle_dem {
    uint64_t nd, no;
    size_t ne, ecap;
    double *p;
    size_t *soff; /* ne + 1 */
    uint32_t *sym;
    size_t ns, scap;
};

typedef struct odp {
    const char *s;
    size_t n, k;
    oerr *e;
} odp;

static int odp_peek(odp *p) {
    return p->k < p->n ? (unsigned char)p->s[p->k] : -1;
}

static void odp_spaces(odp *p) {
    while (odp_peek(p) == ' ' || odp_peek(p) == '\t' || odp_peek(p) == '\r') {
        p->k++;
    }
}

static uint64_t odp_uint(odp *p) {
    int c = odp_peek(p);
    if (c < '0' || c > '9') {
        seterr(p->e, "Expected a digit");
        return 0;
    }
    uint64_t v = 0;
    while (odp_peek(p) >= '0' && odp_peek(p) <= '9') {
        v = v * 10 + (uint64_t)(p->s[p->k++] - '0');
    }
    return v;
}

static void odem_push_sym(oracle_dem *d, uint32_t v) {
    if (d->ns == d->scap) {
        d->scap = d->scap ? 2 * d->scap : 64;
        d->sym = (uint32_t *)realloc(d->sym, d->scap * sizeof(uint32_t));
    }
    d->sym[d->ns++] = v;
}

/* Reads one block's text range [p->k, end of block) once, applying it `reps` times: the text is re-read
 * for every repetition (a repeat body is short and the models in the tests are small). */
static void odem_block(odp *p, oracle_dem *d, uint64_t *off, int top);

static void odem_line(odp *p, oracle_dem *d, uint64_t *off) {
    char name[32];
    size_t nl = 0;
    while (1) {
        int c = odp_peek(p);
        if ((c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_') {
            if (nl < sizeof(name) - 1) {
                name[nl++] = (char)(c >= 'A' && c <= 'Z' ? c - 'A' + 'a' : c);
            }
            p->k++;
        } else {
            break;
        }
    }
    name[nl] = 0;
    if (odp_peek(p) == '[') { /* tag: ignored */
        while (odp_peek(p) != -1 && odp_peek(p) != ']') {
            if (odp_peek(p) == '\\') {
                p->k++;
            }
            p->k++;
        }
        p->k++;
    }
    double args[16];
    size_t na = 0;
    odp_spaces(p);
    if (odp_peek(p) == '(') {
        p->k++;
        while (1) {
            odp_spaces(p);
            if (odp_peek(p) == ')') {
                p->k++;
                break;
            }
            char *end;
            double v = strtod(p->s + p->k, &end);
            if (end == p->s + p->k) {
                seterr(p->e, "bad number");
                return;
            }
            if (na < 16) {
                args[na++] = v;
            }
            p->k = (size_t)(end - p->s);
            odp_spaces(p);
            if (odp_peek(p) == ',') {
                p->k++;
            }
        }
    }
    if (!strcmp(name, "repeat")) {
        odp_spaces(p);
        uint64_t reps = odp_uint(p);
        odp_spaces(p);
        if (odp_peek(p) != '{') {
            seterr(p->e, "Missing '{' at start of repeat block.");
            return;
        }
        p->k++;
        size_t start = p->k;
        if (reps == 0) {
            uint64_t scratch_off = 0;
            oracle_dem scratch = {0};
            odem_block(p, &scratch, &scratch_off, 0);
            free(scratch.p);
            free(scratch.soff);
            free(scratch.sym);
            return;
        }
        for (uint64_t r = 0; r < reps && !p->e->failed; r++) {
            p->k = start;
            odem_block(p, d, off, 0);
        }
        return;
    }
    int is_error = !strcmp(name, "error"), is_shift = !strcmp(name, "shift_detectors");
    int is_det = !strcmp(name, "detector"), is_obs = !strcmp(name, "logical_observable");
    if (!is_error && !is_shift && !is_det && !is_obs) {
        seterr(p->e, "Unrecognized instruction name: %s", name);
        return;
    }
    if (is_error) {
        if (na != 1 || args[0] < 0 || args[0] > 1) {
            seterr(p->e, "'error' instruction takes one probability");
            return;
        }
        if (d->ne + 1 >= d->ecap) {
            d->ecap = d->ecap ? 2 * d->ecap : 64;
            d->p = (double *)realloc(d->p, d->ecap * sizeof(double));
            d->soff = (size_t *)realloc(d->soff, (d->ecap + 1) * sizeof(size_t));
        }
        if (d->ne == 0) {
            d->soff[0] = 0;
        }
        d->p[d->ne] = args[0];
    }
    while (!p->e->failed) {
        odp_spaces(p);
        int c = odp_peek(p);
        if (c == -1 || c == '\n' || c == '#' || c == '}') {
            break;
        }
        if (c == '^') {
            p->k++;
            continue;
        }
        if (c == 'D' || c == 'd' || c == 'L' || c == 'l') {
            p->k++;
            uint64_t v = odp_uint(p);
            if (c == 'D' || c == 'd') {
                uint64_t id = *off + v;
                if (id + 1 > d->nd) {
                    d->nd = id + 1;
                }
                if (is_error) {
                    odem_push_sym(d, (uint32_t)id);
                }
            } else {
                if (v + 1 > d->no) {
                    d->no = v + 1;
                }
                if (is_error) {
                    odem_push_sym(d, (uint32_t)v | 0x80000000u); /* observables marked; resolved at the end */
                }
            }
            continue;
        }
        uint64_t v = odp_uint(p);
        if (is_shift) {
            *off += v;
        }
    }
    if (is_error) {
        d->ne++;
        d->soff[d->ne] = d->ns;
    }
}

static void odem_block(odp *p, oracle_dem *d, uint64_t *off, int top) {
    while (!p->e->failed) {
        odp_spaces(p);
        int c = odp_peek(p);
        if (c == '#') {
            while (odp_peek(p) != -1 && odp_peek(p) != '\n') {
                p->k++;
            }
            continue;
        }
        if (c == -1) {
            if (!top) {
                seterr(p->e, "Unterminated block.");
            }
            return;
        }
        if (c == '\n') {
            p->k++;
            continue;
        }
        if (c == '}') {
            p->k++;
            if (top) {
                seterr(p->e, "Uninitiated block.");
            }
            return;
        }
        odem_line(p, d, off);
    }
}

oracle_dem *oracle_dem_parse(const char *text, char *err, size_t err_len) {
    oerr e = {err, err_len, 0};
    oracle_dem *d = (oracle_dem *)calloc(1, sizeof(oracle_dem));
    d->soff = (size_t *)calloc(1, sizeof(size_t));
    odp p = {text, strlen(text), 0, &e};
    uint64_t off = 0;
    odem_block(&p, d, &off, 1);
    if (e.failed) {
        oracle_dem_free(d);
        return NULL;
    }
    for (size_t j = 0; j < d->ns; j++) {
        if (d->sym[j] & 0x80000000u) {
            d->sym[j] = (uint32_t)(d->nd + (d->sym[j] & 0x7FFFFFFFu));
        }
    }
    return d;
}

void oracle_dem_free(oracle_dem *d) {
    if (d) {
        free(d->p);
        free(d->soff);
        free(d->sym);
        free(d);
    }
}

void oracle_dem_stats(const oracle_dem *d, uint64_t *out3) {
    out3[0] = d->nd;
    out3[1] = d->no;
    out3[2] = d->ne;
}

static void odem_flip(const oracle_dem *d, size_t m, uint64_t s, uint8_t *dets, uint8_t *obs) {
    uint64_t drow = (d->nd + 7) / 8, orow = (d->no + 7) / 8;
    for (size_t j = d->soff[m]; j < d->soff[m + 1]; j++) {
        uint64_t o = d->sym[j];
        if (o < d->nd) {
            dets[s * drow + (o >> 3)] ^= (uint8_t)(1u << (o & 7));
        } else {
            o -= d->nd;
            obs[s * orow + (o >> 3)] ^= (uint8_t)(1u << (o & 7));
        }
    }
}

int oracle_dem_sample(const oracle_dem *d, uint64_t seed, uint64_t first_shot, uint64_t shots, uint8_t *dets,
                      uint8_t *obs, uint8_t *errs, const uint8_t *replay) {
    uint64_t drow = (d->nd + 7) / 8, orow = (d->no + 7) / 8, erow = (d->ne + 7) / 8;
    memset(dets, 0, shots * drow);
    memset(obs, 0, shots * orow);
    if (errs) {
        memset(errs, 0, shots * erow);
    }
    if (replay) {
        for (uint64_t s = 0; s < shots; s++) {
            for (size_t m = 0; m < d->ne; m++) {
                if ((replay[s * erow + (m >> 3)] >> (m & 7)) & 1) {
                    odem_flip(d, m, s, dets, obs);
                }
            }
        }
        if (errs) {
            memcpy(errs, replay, shots * erow);
        }
        return 0;
    }
    /* Groups by probability, in order of first appearance. */
    size_t *group = (size_t *)malloc((d->ne + 1) * sizeof(size_t));
    double *gp = (double *)malloc((d->ne + 1) * sizeof(double));
    size_t ng = 0;
    for (size_t m = 0; m < d->ne; m++) {
        size_t g = 0;
        while (g < ng && gp[g] != d->p[m]) {
            g++;
        }
        if (g == ng) {
            gp[ng++] = d->p[m];
        }
        group[m] = g;
    }
    uint32_t *table = (uint32_t *)malloc(GFS_TABLE_LEN * sizeof(uint32_t));
    size_t *members = (size_t *)malloc((d->ne + 1) * sizeof(size_t));
    for (size_t g = 0; g < ng; g++) {
        size_t n = 0;
        for (size_t m = 0; m < d->ne; m++) {
            if (group[m] == g) {
                members[n++] = m;
            }
        }
        double p = gp[g];
        if (!(p > 0)) {
            continue;
        }
        int always = p >= 1;
        float inv_c = 0;
        if (!always) {
            gfs_build_gap_table(p, table);
            inv_c = gfs_inv_c(p);
        }
        uint64_t nblk = (shots + 127) / 128;
        for (uint64_t b = 0; b < nblk; b++) {
            uint64_t block = first_shot / 128 + b;
            for (size_t seg = 0; GFS_DEM_SEG_UNITS * seg < n; seg++) {
                size_t units = n - GFS_DEM_SEG_UNITS * seg < GFS_DEM_SEG_UNITS ? n - GFS_DEM_SEG_UNITS * seg : GFS_DEM_SEG_UNITS;
                gfs_stream st;
                gfs_stream_init(&st, seed, GFS_P_DEM, g, (uint32_t)seg, (uint32_t)block);
                int32_t pos = -1;
                while ((pos = gfs_next_hit(&st, table, inv_c, pos, (int32_t)(units * 128), always)) >= 0) {
                    uint64_t s = b * 128 + ((uint32_t)pos & 127u);
                    if (s >= shots) {
                        continue;
                    }
                    size_t m = members[GFS_DEM_SEG_UNITS * seg + ((uint32_t)pos >> 7)];
                    odem_flip(d, m, s, dets, obs);
                    if (errs) {
                        errs[s * erow + (m >> 3)] |= (uint8_t)(1u << (m & 7));
                    }
                }
            }
        }
    }
    free(group);
    free(gp);
    free(table);
    free(members);
    return 0;
}
