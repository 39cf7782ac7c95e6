// .stim parser of the host library (grammar of the reference's circuit.cc:149-310, gate_target.h:75-195,
// circuit.h:295-445; validation of circuit_instruction.cc validate; statistics of add_stats_to).
#include "circuit.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace gfs {

const gfs_gate_info &gate_info(gfs_gate g) {
    static const gfs_gate_info *table[GFS_NUM_GATES] = {};
    static bool init = false;
    if (!init) {
        for (const auto &e : GFS_GATE_TABLE) {
            table[e.id] = &e;
        }
        init = true;
    }
    const gfs_gate_info *r = (g > 0 && g < GFS_NUM_GATES) ? table[g] : nullptr;
    if (!r) {
        throw std::invalid_argument("unknown gate");
    }
    return *r;
}

uint64_t Instruction::count_results() const {
    uint32_t f = gate_info(gate).flags;
    if (!(f & GFS_F_RESULTS)) {
        return 0;
    }
    uint64_t n = targets.size();
    if (f & GFS_F_PAIRS) {
        return n >> 1;
    }
    if (f & GFS_F_COMBINERS) {
        for (auto t : targets) {
            if (t & GFS_T_COMBINER) {
                n -= 2;
            }
        }
    }
    return n;
}

namespace {

struct Reader {
    std::string_view s;
    size_t k = 0;
    int get() {
        return k < s.size() ? (unsigned char)s[k++] : EOF;
    }
};

[[noreturn]] void fail(const std::string &msg) {
    throw std::invalid_argument(msg);
}

bool line_arg(int &c, Reader &r, bool space_required) {
    if (c == '*') {
        return true;
    }
    if (space_required && c != ' ' && c != '#' && c != '\t' && c != '\n' && c != '\r' && c != '{' && c != EOF) {
        fail("Targets must be separated by spacing.");
    }
    while (c == ' ' || c == '\t' || c == '\r') {
        c = r.get();
    }
    if (c == '#') {
        do {
            c = r.get();
        } while (c != '\n' && c != EOF);
    }
    return c != '\n' && c != '{' && c != EOF;
}

template <typename T>
T read_uint(int &c, Reader &r, T limit) {
    if (!(c >= '0' && c <= '9')) {
        fail(std::string("Expected a digit but got '") + (char)c + "'");
    }
    T v = 0;
    do {
        v = v * 10 + (T)(c - '0');
        if (v >= limit) {
            fail("Number too large.");
        }
        c = r.get();
    } while (c >= '0' && c <= '9');
    return v;
}

uint32_t read_pauli(int &c, Reader &r) {
    uint32_t m = (c == 'x' || c == 'X')   ? GFS_T_PAULI_X
                 : (c == 'y' || c == 'Y') ? (GFS_T_PAULI_X | GFS_T_PAULI_Z)
                                          : GFS_T_PAULI_Z;
    c = r.get();
    if (c == ' ') {
        fail("Pauli target followed by a space instead of a qubit index.");
    }
    return read_uint<uint32_t>(c, r, 1u << 24) | m;
}

void expect(Reader &r, const char *rest, const char *msg) {
    for (; *rest; rest++) {
        if (r.get() != *rest) {
            fail(msg);
        }
    }
}

uint32_t read_target(int &c, Reader &r) {
    if (c >= '0' && c <= '9') {
        return read_uint<uint32_t>(c, r, 1u << 24);
    }
    switch (c) {
        case 'r': {
            const char *msg = "Target started with 'r' but wasn't a record argument like 'rec[-1]'.";
            expect(r, "ec[-", msg);
            c = r.get();
            uint32_t v = read_uint<uint32_t>(c, r, 1u << 24);
            if (c != ']') {
                fail(msg);
            }
            c = r.get();
            return v | GFS_T_RECORD;
        }
        case 's': {
            const char *msg = "Target started with 's' but wasn't a sweep bit argument like 'sweep[5]'.";
            expect(r, "weep[", msg);
            c = r.get();
            uint32_t v = read_uint<uint32_t>(c, r, 1u << 24);
            if (c != ']') {
                fail(msg);
            }
            c = r.get();
            return v | GFS_T_SWEEP;
        }
        case '!': {
            c = r.get();
            uint32_t t = (c == 'X' || c == 'x' || c == 'Y' || c == 'y' || c == 'Z' || c == 'z')
                             ? read_pauli(c, r)
                             : read_uint<uint32_t>(c, r, 1u << 24);
            return t ^ GFS_T_INVERTED;
        }
        case 'X':
        case 'Y':
        case 'Z':
        case 'x':
        case 'y':
        case 'z':
            return read_pauli(c, r);
        case '*':
            c = r.get();
            return GFS_T_COMBINER;
        default:
            fail(std::string("Unrecognized target prefix '") + (char)c + "'.");
    }
}

void validate(const Instruction &op) {
    const auto &g = gate_info(op.gate);
    uint32_t f = g.flags;
    std::string name = g.name;
    if (f & GFS_F_PAIRS) {
        if (f & GFS_F_PAULI_STRING) {
            size_t terms = op.targets.size();
            for (auto t : op.targets) {
                if (t & GFS_T_COMBINER) {
                    terms -= 2;
                }
            }
            if (terms & 1) {
                fail("The gate " + name + " requires an even number of products to target.");
            }
        } else {
            if (op.targets.size() & 1) {
                fail("Two qubit gate " + name + " requires an even number of targets.");
            }
            for (size_t k = 0; k < op.targets.size(); k += 2) {
                if (op.targets[k] == op.targets[k + 1]) {
                    fail("The two qubit gate " + name +
                         " was applied to a target pair with the same target twice. Gates can't interact "
                         "targets with themselves.");
                }
            }
        }
    }
    if (g.arg_count == GFS_ARGS_ZERO_OR_ONE) {
        if (op.args.size() > 1) {
            fail("Gate " + name + " was given " + std::to_string(op.args.size()) +
                 " parens arguments but takes 0 or 1 parens arguments.");
        }
    } else if (g.arg_count != GFS_ARGS_ANY && op.args.size() != (size_t)g.arg_count) {
        fail("Gate " + name + " was given " + std::to_string(op.args.size()) + " parens arguments but takes " +
             std::to_string(g.arg_count) + " parens arguments.");
    }
    if ((f & GFS_F_NO_TARGETS) && !op.targets.empty()) {
        fail("Gate " + name + " takes no targets but was given targets.");
    }
    if (f & GFS_F_DISJOINT_PROBS) {
        double total = 0;
        for (double p : op.args) {
            if (!(p >= 0 && p <= 1)) {
                fail("Gate " + name + " only takes probability arguments, but one of its arguments wasn't a probability.");
            }
            total += p;
        }
        if (total > 1.0000001) {
            fail("The disjoint probability arguments given to gate " + name + " sum to more than 1.");
        }
    } else if (f & GFS_F_UINT_ARGS) {
        for (double p : op.args) {
            if (p < 0 || p != std::round(p)) {
                fail("Gate " + name + " only takes non-negative integer arguments.");
            }
        }
    }
    uint32_t valid = GFS_T_VALUE_MASK;
    if (f & GFS_F_COMBINERS) {
        bool allowed = false, just = false, failed = false;
        for (auto t : op.targets) {
            if (t & GFS_T_COMBINER) {
                failed |= !allowed;
                allowed = false;
                just = true;
            } else {
                allowed = true;
                just = false;
            }
        }
        if (failed || just) {
            fail("Gate " + name + " given combiners ('*') that aren't between other targets.");
        }
        valid |= GFS_T_COMBINER;
    }
    if (f & GFS_F_RESULTS) {
        valid |= GFS_T_INVERTED;
    }
    if (f & GFS_F_CAN_TARGET_BITS) {
        valid |= GFS_T_RECORD | GFS_T_SWEEP;
    }
    for (auto t : op.targets) {
        if (f & GFS_F_ONLY_REC) {
            bool ok = (t & GFS_T_RECORD) || ((f & GFS_F_PAULI_STRING) && (t & (GFS_T_PAULI_X | GFS_T_PAULI_Z)));
            if (!ok) {
                fail("Gate " + name + " only takes measurement record targets (rec[-k]).");
            }
        } else if (f & GFS_F_PAULI_STRING) {
            uint32_t ok_bits = GFS_T_PAULI_X | GFS_T_PAULI_Z | GFS_T_COMBINER;
            if (f & GFS_F_CAN_TARGET_BITS) {
                ok_bits |= GFS_T_RECORD | GFS_T_SWEEP;
            }
            if (!(t & ok_bits)) {
                fail("Gate " + name + " only takes Pauli targets ('X2', 'Y3', 'Z5', etc).");
            }
        } else if (t != (t & valid)) {
            fail("Target has invalid modifiers for gate type '" + name + "'.");
        }
    }
    if (op.gate == GFS_MPAD) {
        for (auto t : op.targets) {
            if (t > 1) {
                fail("Target is not valid for gate type 'MPAD'.");
            }
        }
    }
}

bool can_fuse(const Instruction &a, const Instruction &b) {
    return a.gate == b.gate && a.args == b.args && !(gate_info(a.gate).flags & GFS_F_NOT_FUSABLE) && a.tag == b.tag;
}

bool is_double_char(int c) {
    return (c >= '0' && c <= '9') || c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-';
}

void parse_into(Circuit &circ, Reader &r, bool until_brace) {
    for (;;) {
        int c = r.get();
        for (;;) {
            while (c != EOF && (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f')) {
                c = r.get();
            }
            if (c != '#') {
                break;
            }
            while (c != '\n' && c != EOF) {
                c = r.get();
            }
        }
        if (c == EOF) {
            if (until_brace) {
                fail("Unterminated block. Got a '{' without an eventual '}'.");
            }
            return;
        }
        if (c == '}') {
            if (!until_brace) {
                fail("Uninitiated block. Got a '}' without a '{'.");
            }
            return;
        }
        std::string name;
        while (((c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || (c >= '0' && c <= '9') || c == '_') &&
               name.size() < 32) {
            name.push_back((char)c);
            c = r.get();
        }
        const gfs_gate_info *g = gfs_gate_by_name(name.data(), name.size());
        if (!g) {
            fail("Gate not found: '" + name + "'");
        }
        Instruction op;
        op.gate = g->id;
        if (c == '[') {
            c = r.get();
            while (c != ']') {
                if (c == '\r' || c == '\n' || c == EOF) {
                    fail("A tag wasn't closed with ']' before the end of the line.");
                }
                if (c == '\\') {
                    c = r.get();
                    switch (c) {
                        case 'n':
                            op.tag.push_back('\n');
                            break;
                        case 'r':
                            op.tag.push_back('\r');
                            break;
                        case 'B':
                            op.tag.push_back('\\');
                            break;
                        case 'C':
                            op.tag.push_back(']');
                            break;
                        default:
                            fail("Unrecognized escape sequence in tag.");
                    }
                } else {
                    op.tag.push_back((char)c);
                }
                c = r.get();
            }
            c = r.get();
        }
        if (c == '(') {
            c = r.get();
            while (c == ' ' || c == '\t') {
                c = r.get();
            }
            for (;;) {
                std::string buf;
                while (buf.size() < 63 && is_double_char(c)) {
                    buf.push_back((char)c);
                    c = r.get();
                }
                // An empty number reads as 0, as in the reference (circuit.h read_normal_double): "X_ERROR() 0" is
                // X_ERROR(0) 0 and "H() 0" is H with one argument.
                char *end = nullptr;
                double v = std::strtod(buf.c_str(), &end);
                if (end != buf.c_str() + buf.size() || std::isinf(v) || std::isnan(v)) {
                    fail("Not a real number: " + buf);
                }
                op.args.push_back(v);
                while (c == ' ' || c == '\t') {
                    c = r.get();
                }
                if (c != ',') {
                    break;
                }
                c = r.get();
                while (c == ' ' || c == '\t') {
                    c = r.get();
                }
            }
            while (c == ' ' || c == '\t') {
                c = r.get();
            }
            if (c != ')') {
                fail(std::string("Parens arguments for '") + g->name + "' didn't end with a ')'.");
            }
            c = r.get();
        }
        if (g->flags & GFS_F_BLOCK) {
            std::vector<uint64_t> nums;
            while (line_arg(c, r, true)) {
                nums.push_back(read_uint<uint64_t>(c, r, (uint64_t)1 << 63));
            }
            if (c != '{') {
                fail(std::string("Missing '{' at start of ") + g->name + " block.");
            }
            if (nums.size() != 1) {
                fail("Invalid instruction. Expected one repetition arg like `REPEAT 100 {`.");
            }
            if (nums[0] == 0) {
                fail("Repeating 0 times is not supported.");
            }
            op.reps = nums[0];
            op.block = (uint32_t)circ.blocks.size();
            circ.blocks.emplace_back();
            parse_into(circ.blocks.back(), r, true);
            circ.ops.push_back(std::move(op));
        } else {
            bool need_space = true;
            while (line_arg(c, r, need_space)) {
                uint32_t t = read_target(c, r);
                op.targets.push_back(t);
                need_space = !(t & GFS_T_COMBINER);
            }
            if (c == '{') {
                fail("Unexpected '{'.");
            }
            validate(op);
            if (!circ.ops.empty() && can_fuse(circ.ops.back(), op)) {
                auto &prev = circ.ops.back().targets;
                prev.insert(prev.end(), op.targets.begin(), op.targets.end());
            } else {
                circ.ops.push_back(std::move(op));
            }
        }
        if (c == EOF) {
            if (until_brace) {
                fail("Unterminated block. Got a '{' without an eventual '}'.");
            }
            return;
        }
    }
}

uint64_t sat_add(uint64_t a, uint64_t b) {
    return a + b < a ? UINT64_MAX : a + b;
}
uint64_t sat_mul(uint64_t a, uint64_t b) {
    return (a && b > UINT64_MAX / a) ? UINT64_MAX : a * b;
}

}  // namespace

Circuit Circuit::parse(std::string_view text) {
    Circuit c;
    Reader r{text};
    parse_into(c, r, false);
    return c;
}

CircuitStats Circuit::stats() const {
    CircuitStats s;
    for (const auto &op : ops) {
        if (op.gate == GFS_REPEAT) {
            CircuitStats sub = blocks[op.block].stats();
            s.num_qubits = std::max(s.num_qubits, sub.num_qubits);
            s.num_observables = std::max(s.num_observables, sub.num_observables);
            s.max_lookback = std::max(s.max_lookback, sub.max_lookback);
            s.num_detectors = sat_add(s.num_detectors, sat_mul(sub.num_detectors, op.reps));
            s.num_measurements = sat_add(s.num_measurements, sat_mul(sub.num_measurements, op.reps));
            s.num_instances = sat_add(s.num_instances, sat_mul(sub.num_instances, op.reps));
            continue;
        }
        s.num_instances++;
        for (auto t : op.targets) {
            uint32_t v = t & GFS_T_VALUE_MASK;
            if (op.gate != GFS_MPAD && !(t & (GFS_T_RECORD | GFS_T_SWEEP))) {
                s.num_qubits = std::max<uint64_t>(s.num_qubits, (uint64_t)v + 1);
            }
            if (t & GFS_T_RECORD) {
                s.max_lookback = std::max<uint64_t>(s.max_lookback, v);
            }
        }
        s.num_measurements += op.count_results();
        if (op.gate == GFS_DETECTOR) {
            s.num_detectors++;
        } else if (op.gate == GFS_OBSERVABLE_INCLUDE) {
            s.num_observables = std::max<uint64_t>(s.num_observables, (uint64_t)op.args[0] + 1);
        }
    }
    return s;
}

}  // namespace gfs
