// Detector error model parsing and lowering (dem.h).
#include "dem.h"

#include <cmath>
#include <cstdlib>
#include <map>
#include <stdexcept>
#include <string>

#include "gfs_contract.h"

namespace gfs {

namespace {

enum class DemOp { ERROR, SHIFT_DETECTORS, DETECTOR, LOGICAL_OBSERVABLE, REPEAT };

struct DemTarget {
    enum Kind { DET, OBS, SEP, NUM } kind;
    uint64_t v;
};

struct DemInst {
    DemOp op;
    std::vector<double> args;
    std::vector<DemTarget> targets;
    size_t block = 0;  // REPEAT body
    uint64_t reps = 0;
};

struct DemBlock {
    std::vector<DemInst> ops;
};

struct Parser {
    std::string_view s;
    size_t k = 0;
    std::vector<DemBlock> blocks;

    int peek() const {
        return k < s.size() ? (unsigned char)s[k] : -1;
    }
    int get() {
        return k < s.size() ? (unsigned char)s[k++] : -1;
    }
    void skip_spaces() {
        while (peek() == ' ' || peek() == '\t' || peek() == '\r') {
            k++;
        }
    }
    void skip_comment() {
        if (peek() == '#') {
            while (peek() != -1 && peek() != '\n') {
                k++;
            }
        }
    }
    uint64_t read_uint() {
        int c = peek();
        if (!(c >= '0' && c <= '9')) {
            throw std::invalid_argument("Expected a digit but got '" + std::string(1, c < 0 ? ' ' : (char)c) + "'");
        }
        uint64_t v = 0;
        while (peek() >= '0' && peek() <= '9') {
            v = v * 10 + (uint64_t)(get() - '0');
            if (v >= (uint64_t)1 << 60) {
                throw std::out_of_range("Number too large.");
            }
        }
        return v;
    }
    DemOp read_name() {
        std::string name;
        while (true) {
            int c = peek();
            if ((c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || (c >= '0' && c <= '9') || c == '_') {
                name.push_back((char)std::tolower(c));
                k++;
            } else {
                break;
            }
        }
        if (name == "error") return DemOp::ERROR;
        if (name == "shift_detectors") return DemOp::SHIFT_DETECTORS;
        if (name == "detector") return DemOp::DETECTOR;
        if (name == "logical_observable") return DemOp::LOGICAL_OBSERVABLE;
        if (name == "repeat") return DemOp::REPEAT;
        throw std::out_of_range("Unrecognized instruction name: " + name);
    }
    void skip_tag() {
        if (peek() != '[') {
            return;
        }
        k++;
        while (true) {
            int c = get();
            if (c == -1 || c == '\n') {
                throw std::invalid_argument("Unterminated tag.");
            }
            if (c == '\\') {
                get();
                continue;
            }
            if (c == ']') {
                return;
            }
        }
    }
    // Parenthesized arguments, as the reference reads them (circuit.h read_parens_arguments, shared with circuits):
    // the '(' must follow the name or tag directly; numbers are runs of digits, '.', 'e', 'E', '+' and '-' (an
    // empty one reads as 0), separated by ',' with spaces or tabs around.
    std::vector<double> read_args() {
        std::vector<double> args;
        if (peek() != '(') {
            return args;
        }
        k++;
        auto blanks = [&]() {
            while (peek() == ' ' || peek() == '\t') {
                k++;
            }
        };
        auto number_char = [](int c) {
            return (c >= '0' && c <= '9') || c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-';
        };
        blanks();
        while (true) {
            std::string buf;
            while (buf.size() < 63 && number_char(peek())) {
                buf.push_back((char)get());
            }
            char *end = nullptr;
            const double v = std::strtod(buf.c_str(), &end);
            if (end != buf.c_str() + buf.size() || std::isinf(v) || std::isnan(v)) {
                throw std::invalid_argument("Not a real number: " + buf);
            }
            args.push_back(v);
            blanks();
            if (peek() != ',') {
                break;
            }
            k++;
            blanks();
        }
        blanks();
        if (get() != ')') {
            throw std::invalid_argument("Parens arguments for 'detector error model instruction' didn't end with a ')'.");
        }
        return args;
    }
    // Targets until the end of the line, as the reference reads them (circuit.h read_until_next_line_arg): they are
    // separated from the instruction and from one another by spaces or tabs; the line ends at a newline, a comment
    // or a block's '{', and a '}' closes a block only at the start of a line.
    static bool ends_target(int c) {
        return c == -1 || c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '#' || c == '{';
    }
    std::vector<DemTarget> read_targets() {
        std::vector<DemTarget> t;
        if (!ends_target(peek())) {
            throw std::invalid_argument("Targets must be separated by spacing.");
        }
        while (true) {
            skip_spaces();
            int c = peek();
            if (c == -1 || c == '\n' || c == '#' || c == '{') {
                return t;
            }
            if (c == 'D' || c == 'd') {
                k++;
                t.push_back({DemTarget::DET, read_uint()});
            } else if (c == 'L' || c == 'l') {
                k++;
                t.push_back({DemTarget::OBS, read_uint()});
            } else if (c == '^') {
                k++;
                t.push_back({DemTarget::SEP, 0});
            } else if (c >= '0' && c <= '9') {
                t.push_back({DemTarget::NUM, read_uint()});
            } else {
                throw std::invalid_argument("Unrecognized target prefix '" + std::string(1, (char)c) + "'.");
            }
            if (!ends_target(peek())) {
                throw std::invalid_argument("Targets must be separated by spacing.");
            }
        }
    }
    static void validate(const DemInst &in) {
        switch (in.op) {
            case DemOp::ERROR: {
                if (in.args.size() != 1) {
                    throw std::invalid_argument("'error' instruction takes 1 argument (a probability), but got " +
                                                std::to_string(in.args.size()) + " arguments.");
                }
                if (in.args[0] < 0 || in.args[0] > 1) {
                    throw std::invalid_argument("'error' instruction argument must be a probability (0 to 1) but got " +
                                                std::to_string(in.args[0]));
                }
                const auto &t = in.targets;
                if (!t.empty() && (t.front().kind == DemTarget::SEP || t.back().kind == DemTarget::SEP)) {
                    throw std::invalid_argument("First/last targets of 'error' instruction shouldn't be separators (^).");
                }
                for (size_t i = 0; i < t.size(); i++) {
                    if (i && t[i].kind == DemTarget::SEP && t[i - 1].kind == DemTarget::SEP) {
                        throw std::invalid_argument("'error' instruction has adjacent separators (^ ^).");
                    }
                    if (t[i].kind == DemTarget::NUM) {
                        throw std::invalid_argument("'error' instruction targets must be D#, L# or ^.");
                    }
                }
                break;
            }
            case DemOp::SHIFT_DETECTORS:
                if (in.targets.size() != 1 || in.targets[0].kind != DemTarget::NUM) {
                    throw std::invalid_argument("'shift_detectors' instruction takes 1 target, but got " +
                                                std::to_string(in.targets.size()) + " targets.");
                }
                break;
            case DemOp::DETECTOR:
                if (in.targets.size() != 1) {
                    throw std::invalid_argument("'detector' instruction takes 1 target but got " +
                                                std::to_string(in.targets.size()) + " arguments.");
                }
                if (in.targets[0].kind != DemTarget::DET) {
                    throw std::invalid_argument("'detector' instruction takes a relative detector target (D#).");
                }
                break;
            case DemOp::LOGICAL_OBSERVABLE:
                if (!in.args.empty()) {
                    throw std::invalid_argument("'logical_observable' instruction takes 0 arguments but got " +
                                                std::to_string(in.args.size()) + " arguments.");
                }
                if (in.targets.size() != 1) {
                    throw std::invalid_argument("'logical_observable' instruction takes 1 target but got " +
                                                std::to_string(in.targets.size()) + " arguments.");
                }
                if (in.targets[0].kind != DemTarget::OBS) {
                    throw std::invalid_argument(
                        "'logical_observable' instruction takes a logical observable target (L#).");
                }
                break;
            case DemOp::REPEAT:
                break;
        }
    }
    // Reads instructions into block b until the end of the text (top level) or a closing brace.
    void read_block(size_t b, bool top) {
        while (true) {
            skip_spaces();
            skip_comment();
            int c = peek();
            if (c == -1) {
                if (!top) {
                    throw std::out_of_range("Unterminated block. Got a '{' without an eventual '}'.");
                }
                return;
            }
            if (c == '\n') {
                k++;
                continue;
            }
            if (c == '}') {
                if (top) {
                    throw std::out_of_range("Uninitiated block. Got a '}' without a '{'.");
                }
                k++;
                return;
            }
            DemInst in;
            in.op = read_name();
            skip_tag();
            if (in.op != DemOp::REPEAT) {  // a repeat block takes no parenthesized arguments
                in.args = read_args();
            }
            in.targets = read_targets();
            skip_spaces();
            if (in.op == DemOp::REPEAT) {
                if (in.targets.empty()) {
                    throw std::invalid_argument("Missing repeat count of repeat block.");
                }
                if (in.targets.size() != 1 || in.targets[0].kind != DemTarget::NUM) {
                    throw std::invalid_argument("Too many numeric values given to repeat block.");
                }
                if (peek() != '{') {
                    throw std::invalid_argument("Missing '{' at start of repeat block.");
                }
                k++;
                in.reps = in.targets[0].v;
                in.targets.clear();
                in.block = blocks.size();
                blocks.emplace_back();
                read_block(in.block, false);
            } else {
                if (peek() == '{') {
                    throw std::invalid_argument("Unexpected '{'.");
                }
                validate(in);
            }
            blocks[b].ops.push_back(std::move(in));
        }
    }
};

// Unrolls block b into the model with detector offset `off`.
void flatten(const Parser &ps, size_t b, uint64_t &off, DemModel &m) {
    for (const DemInst &in : ps.blocks[b].ops) {
        switch (in.op) {
            case DemOp::REPEAT:
                for (uint64_t r = 0; r < in.reps; r++) {
                    flatten(ps, in.block, off, m);
                }
                break;
            case DemOp::SHIFT_DETECTORS:
                off += in.targets[0].v;
                break;
            case DemOp::DETECTOR:
                m.num_detectors = std::max<uint64_t>(m.num_detectors, off + in.targets[0].v + 1);
                break;
            case DemOp::LOGICAL_OBSERVABLE:
                m.num_observables = std::max<uint64_t>(m.num_observables, in.targets[0].v + 1);
                break;
            case DemOp::ERROR:
                m.p.push_back(in.args[0]);
                for (const DemTarget &t : in.targets) {
                    if (t.kind == DemTarget::DET) {
                        m.num_detectors = std::max<uint64_t>(m.num_detectors, off + t.v + 1);
                        m.sym.push_back((uint32_t)(off + t.v));  // tagged below once D is known
                        m.sym_off.push_back(0);                    // placeholder marker: detector
                    } else if (t.kind == DemTarget::OBS) {
                        m.num_observables = std::max<uint64_t>(m.num_observables, t.v + 1);
                        m.sym.push_back((uint32_t)t.v);
                        m.sym_off.push_back(1);  // placeholder marker: observable
                    }
                }
                m.sym_off.push_back(2);  // end of this mechanism
                if (m.p.size() > 0x7FFFFFFFull || m.sym.size() > 0x7FFFFFFFull) {
                    throw std::invalid_argument("detector error model too large for the GPU sampler");
                }
                break;
        }
    }
}

}  // namespace

DemModel parse_dem(std::string_view text) {
    Parser ps{text};
    ps.blocks.emplace_back();
    ps.read_block(0, true);
    DemModel m;
    uint64_t off = 0;
    flatten(ps, 0, off, m);
    if (m.num_detectors + m.num_observables > 0xFFFFFFFFull) {
        throw std::invalid_argument("too many detectors for the GPU sampler");
    }
    // Resolve the markers: observables after the detectors, and CSR offsets per mechanism.
    std::vector<uint32_t> sym, sym_off{0};
    size_t j = 0;
    for (uint32_t mk : m.sym_off) {
        if (mk == 2) {
            sym_off.push_back((uint32_t)sym.size());
            continue;
        }
        sym.push_back(mk == 0 ? m.sym[j] : (uint32_t)(m.num_detectors + m.sym[j]));
        j++;
    }
    m.sym.swap(sym);
    m.sym_off.swap(sym_off);
    return m;
}

DemLayout layout_dem(const DemModel &m) {
    DemLayout L;
    std::map<double, uint32_t> group_of;
    std::vector<std::vector<uint32_t>> members;
    for (uint32_t i = 0; i < (uint32_t)m.p.size(); i++) {
        auto it = group_of.find(m.p[i]);
        if (it == group_of.end()) {
            it = group_of.emplace(m.p[i], (uint32_t)members.size()).first;
            members.emplace_back();
        }
        members[it->second].push_back(i);
    }
    std::vector<double> gp(members.size());
    for (const auto &kv : group_of) {
        gp[kv.second] = kv.first;
    }
    for (uint32_t g = 0; g < (uint32_t)members.size(); g++) {
        DemGroup G{};
        G.first = (uint32_t)L.units.size();
        G.n = (uint32_t)members[g].size();
        const double p = gp[g];
        G.flags = (p > 0 ? 1u : 0u) | (p >= 1 ? 2u : 0u);
        if (p > 0 && p < 1) {
            G.table = (uint32_t)L.tables.size();
            L.tables.resize(L.tables.size() + GFS_TABLE_LEN);
            gfs_build_gap_table(p, L.tables.data() + G.table);
            G.inv_c = gfs_inv_c(p);
        }
        L.units.insert(L.units.end(), members[g].begin(), members[g].end());
        L.groups.push_back(G);
        if (p > 0) {
            for (uint32_t u0 = 0; u0 < G.n; u0 += kDemChunkUnits) {
                L.chunk_group.push_back(g);
                L.chunk_unit0.push_back(u0);
                L.chunk_units.push_back(std::min<uint32_t>(kDemChunkUnits, G.n - u0));
            }
        }
    }
    if (L.tables.empty()) {
        L.tables.resize(GFS_TABLE_LEN, 0);
    }
    // Outputs -> mechanisms, for replayed errors.
    const uint64_t n_out = m.num_detectors + m.num_observables;
    std::vector<uint32_t> count(n_out + 1, 0);
    for (uint32_t s : m.sym) {
        count[s + 1]++;
    }
    L.out_off.assign(n_out + 1, 0);
    for (uint64_t o = 0; o < n_out; o++) {
        L.out_off[o + 1] = L.out_off[o] + count[o + 1];
    }
    L.out_mech.assign(m.sym.size(), 0);
    std::vector<uint32_t> fill(L.out_off.begin(), L.out_off.end() - 1);
    for (uint32_t e = 0; e + 1 < (uint32_t)m.sym_off.size(); e++) {
        for (uint32_t j = m.sym_off[e]; j < m.sym_off[e + 1]; j++) {
            L.out_mech[fill[m.sym[j]]++] = e;
        }
    }
    return L;
}

}  // namespace gfs
