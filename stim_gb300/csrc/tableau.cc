// Host stabilizer tableau for the reference sample (see tableau.h).
//
// Aaronson-Gottesman tableau ("Improved simulation of stabilizer circuits", PRA 70, 052328, 2004): rows
// 0..n-1 destabilizers, n..2n-1 stabilizers, row 2n scratch; each row holds bit-packed X and Z parts and
// a sign, with X=Z=1 meaning Y.  Unitary gates are applied as their Heisenberg action on Paulis (the
// images of X and Z of each qubit, i.e. the gate's flow table, listed below from the reference's gate
// data), so one routine serves every one- and two-qubit Clifford.  Measurements follow the paper's
// procedure, with every random outcome forced to 0.
#include "tableau.h"

#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace gfs {
namespace {

// ---- Paulis with phases: x, z bits per qubit (X=Z=1 is Y) and a phase exponent of i. ----

// Exponent of i picked up by P1 * P2 on one qubit (Aaronson-Gottesman's g function).
int pauli_g(int x1, int z1, int x2, int z2) {
    if (!x1 && !z1) return 0;
    if (x1 && z1) return z2 - x2;
    if (x1) return z2 * (2 * x2 - 1);
    return x2 * (1 - 2 * z2);
}

struct P2 {  // a two-qubit Pauli with phase i^e
    int e = 0;
    int x[2] = {0, 0}, z[2] = {0, 0};
};

P2 mul(const P2 &a, const P2 &b) {
    P2 r;
    r.e = a.e + b.e;
    for (int k = 0; k < 2; k++) {
        r.e += pauli_g(a.x[k], a.z[k], b.x[k], b.z[k]);
        r.x[k] = a.x[k] ^ b.x[k];
        r.z[k] = a.z[k] ^ b.z[k];
    }
    r.e = ((r.e % 4) + 4) % 4;
    return r;
}

P2 parse_pauli(const char *s) {  // "+XZ", "-Y", ...
    P2 p;
    p.e = s[0] == '-' ? 2 : 0;
    for (int k = 0; s[1 + k] && k < 2; k++) {
        char c = s[1 + k];
        p.x[k] = (c == 'X' || c == 'Y') ? 1 : 0;
        p.z[k] = (c == 'Z' || c == 'Y') ? 1 : 0;
    }
    return p;
}

// Heisenberg images of the generators, as the reference's gate data lists them (flow_data in
// src/stim/gates/gate_data_hada.cc, _pauli.cc, _period_3.cc, _period_4.cc, _controlled.cc, _pp.cc,
// _swaps.cc): one-qubit gates give the images of X and Z; two-qubit gates those of X1, Z1, X2, Z2.
struct Flow {
    gfs_gate g;
    const char *img[4];
};
const Flow kFlows[] = {
    {GFS_I, {"+X", "+Z"}},
    {GFS_X, {"+X", "-Z"}},
    {GFS_Y, {"-X", "-Z"}},
    {GFS_Z, {"-X", "+Z"}},
    {GFS_H, {"+Z", "+X"}},
    {GFS_H_XY, {"+Y", "-Z"}},
    {GFS_H_YZ, {"-X", "+Y"}},
    {GFS_H_NXY, {"-Y", "-Z"}},
    {GFS_H_NXZ, {"-Z", "-X"}},
    {GFS_H_NYZ, {"-X", "-Y"}},
    {GFS_C_XYZ, {"+Y", "+X"}},
    {GFS_C_NXYZ, {"-Y", "-X"}},
    {GFS_C_XNYZ, {"-Y", "+X"}},
    {GFS_C_XYNZ, {"+Y", "-X"}},
    {GFS_C_ZYX, {"+Z", "+Y"}},
    {GFS_C_ZYNX, {"-Z", "+Y"}},
    {GFS_C_ZNYX, {"+Z", "-Y"}},
    {GFS_C_NZYX, {"-Z", "-Y"}},
    {GFS_SQRT_X, {"+X", "-Y"}},
    {GFS_SQRT_X_DAG, {"+X", "+Y"}},
    {GFS_SQRT_Y, {"-Z", "+X"}},
    {GFS_SQRT_Y_DAG, {"+Z", "-X"}},
    {GFS_S, {"+Y", "+Z"}},
    {GFS_S_DAG, {"-Y", "+Z"}},
    {GFS_XCX, {"+XI", "+ZX", "+IX", "+XZ"}},
    {GFS_XCY, {"+XI", "+ZY", "+XX", "+XZ"}},
    {GFS_XCZ, {"+XI", "+ZZ", "+XX", "+IZ"}},
    {GFS_YCX, {"+XX", "+ZX", "+IX", "+YZ"}},
    {GFS_YCY, {"+XY", "+ZY", "+YX", "+YZ"}},
    {GFS_YCZ, {"+XZ", "+ZZ", "+YX", "+IZ"}},
    {GFS_CX, {"+XX", "+ZI", "+IX", "+ZZ"}},
    {GFS_CY, {"+XY", "+ZI", "+ZX", "+ZZ"}},
    {GFS_CZ, {"+XZ", "+ZI", "+ZX", "+IZ"}},
    {GFS_II, {"+XI", "+ZI", "+IX", "+IZ"}},
    {GFS_SQRT_XX, {"+XI", "-YX", "+IX", "-XY"}},
    {GFS_SQRT_XX_DAG, {"+XI", "+YX", "+IX", "+XY"}},
    {GFS_SQRT_YY, {"-ZY", "+XY", "-YZ", "+YX"}},
    {GFS_SQRT_YY_DAG, {"+ZY", "-XY", "+YZ", "-YX"}},
    {GFS_SQRT_ZZ, {"+YZ", "+ZI", "+ZY", "+IZ"}},
    {GFS_SQRT_ZZ_DAG, {"-YZ", "+ZI", "-ZY", "+IZ"}},
    {GFS_SWAP, {"+IX", "+IZ", "+XI", "+ZI"}},
    {GFS_ISWAP, {"+ZY", "+IZ", "+YZ", "+ZI"}},
    {GFS_ISWAP_DAG, {"-ZY", "+IZ", "-YZ", "+ZI"}},
    {GFS_CXSWAP, {"+XX", "+IZ", "+XI", "+ZZ"}},
    {GFS_SWAPCX, {"+IX", "+ZZ", "+XX", "+ZI"}},
    {GFS_CZSWAP, {"+ZX", "+IZ", "+XZ", "+ZI"}},
};

// Conjugation table of a gate: for every input Pauli (index x1 | z1<<1 | x2<<2 | z2<<3) its image bits
// and whether the sign flips.
struct GateTable {
    int nq = 0;
    uint8_t out[16] = {};  // x1 | z1<<1 | x2<<2 | z2<<3
    uint8_t flip[16] = {};
};

GateTable build_table(const Flow &f) {
    GateTable t;
    t.nq = f.img[2] ? 2 : 1;
    P2 img[4];
    for (int k = 0; k < 2 * t.nq; k++) {
        img[k] = parse_pauli(f.img[k]);
    }
    const int n_in = t.nq == 1 ? 4 : 16;
    for (int in = 0; in < n_in; in++) {
        P2 acc;
        for (int q = 0; q < t.nq; q++) {
            const int x = (in >> (2 * q)) & 1, z = (in >> (2 * q + 1)) & 1;
            const P2 &ix = img[2 * q], &iz = img[2 * q + 1];
            if (x && z) {  // Y = i X Z
                P2 y = mul(ix, iz);
                y.e = (y.e + 1) % 4;
                acc = mul(acc, y);
            } else if (x) {
                acc = mul(acc, ix);
            } else if (z) {
                acc = mul(acc, iz);
            }
        }
        if (acc.e & 1) {
            throw std::logic_error("non-Hermitian gate image");
        }
        t.out[in] = (uint8_t)(acc.x[0] | acc.z[0] << 1 | acc.x[1] << 2 | acc.z[1] << 3);
        t.flip[in] = acc.e == 2;
    }
    return t;
}

const GateTable *table_for(gfs_gate g) {
    static const std::unordered_map<int, GateTable> tables = [] {
        std::unordered_map<int, GateTable> m;
        for (const Flow &f : kFlows) {
            m[(int)f.g] = build_table(f);
        }
        return m;
    }();
    auto it = tables.find((int)g);
    return it == tables.end() ? nullptr : &it->second;
}

class Tableau {
   public:
    explicit Tableau(size_t n) : n_(n), nw_((n + 63) / 64), rows_(2 * n + 1) {
        xs_.assign(rows_ * nw_, 0);
        zs_.assign(rows_ * nw_, 0);
        r_.assign(rows_, 0);
        for (size_t i = 0; i < n; i++) {
            set(xs_, i, i, 1);
            set(zs_, n + i, i, 1);
        }
    }

    void apply(const GateTable &t, size_t a, size_t b) {
        for (size_t i = 0; i < 2 * n_; i++) {
            unsigned in = get(xs_, i, a) | get(zs_, i, a) << 1;
            if (t.nq == 2) {
                in |= get(xs_, i, b) << 2 | get(zs_, i, b) << 3;
            }
            if (!in) {
                continue;
            }
            const unsigned o = t.out[in];
            set(xs_, i, a, o & 1);
            set(zs_, i, a, (o >> 1) & 1);
            if (t.nq == 2) {
                set(xs_, i, b, (o >> 2) & 1);
                set(zs_, i, b, (o >> 3) & 1);
            }
            r_[i] ^= t.flip[in];
        }
    }

    void apply(gfs_gate g, size_t a, size_t b = 0) {
        apply(*table_for(g), a, b);
    }

    // Z measurement with random outcomes forced to 0; the state collapses accordingly.
    bool measure_z(size_t q) {
        size_t p = SIZE_MAX;
        for (size_t i = n_; i < 2 * n_; i++) {
            if (get(xs_, i, q)) {
                p = i;
                break;
            }
        }
        if (p != SIZE_MAX) {
            for (size_t i = 0; i < 2 * n_; i++) {
                if (i != p && get(xs_, i, q)) {
                    rowsum(i, p);
                }
            }
            copy_row(p - n_, p);
            std::memset(&xs_[p * nw_], 0, nw_ * sizeof(uint64_t));
            std::memset(&zs_[p * nw_], 0, nw_ * sizeof(uint64_t));
            set(zs_, p, q, 1);
            r_[p] = 0;  // forced outcome 0
            return false;
        }
        const size_t s = 2 * n_;
        std::memset(&xs_[s * nw_], 0, nw_ * sizeof(uint64_t));
        std::memset(&zs_[s * nw_], 0, nw_ * sizeof(uint64_t));
        r_[s] = 0;
        for (size_t i = 0; i < n_; i++) {
            if (get(xs_, i, q)) {
                rowsum(s, i + n_);
            }
        }
        return r_[s];
    }

   private:
    static unsigned get(const std::vector<uint64_t> &v, size_t row, size_t q, size_t nw) {
        return (unsigned)((v[row * nw + (q >> 6)] >> (q & 63)) & 1u);
    }
    unsigned get(const std::vector<uint64_t> &v, size_t row, size_t q) const {
        return get(v, row, q, nw_);
    }
    void set(std::vector<uint64_t> &v, size_t row, size_t q, unsigned bit) {
        uint64_t &w = v[row * nw_ + (q >> 6)];
        const uint64_t m = (uint64_t)1 << (q & 63);
        w = bit ? (w | m) : (w & ~m);
    }
    void copy_row(size_t dst, size_t src) {
        std::memcpy(&xs_[dst * nw_], &xs_[src * nw_], nw_ * sizeof(uint64_t));
        std::memcpy(&zs_[dst * nw_], &zs_[src * nw_], nw_ * sizeof(uint64_t));
        r_[dst] = r_[src];
    }
    // Row h := row i * row h, with the phase rule of the paper evaluated 64 qubits at a time.
    void rowsum(size_t h, size_t i) {
        uint64_t *xh = &xs_[h * nw_], *zh = &zs_[h * nw_];
        const uint64_t *xi = &xs_[i * nw_], *zi = &zs_[i * nw_];
        long sum = 2 * (long)r_[h] + 2 * (long)r_[i];
        for (size_t w = 0; w < nw_; w++) {
            const uint64_t x1 = xi[w], z1 = zi[w], x2 = xh[w], z2 = zh[w];
            const uint64_t y1 = x1 & z1, ox1 = x1 & ~z1, oz1 = z1 & ~x1;
            const uint64_t y2 = x2 & z2, ox2 = x2 & ~z2, oz2 = z2 & ~x2;
            const uint64_t plus = (y1 & oz2) | (ox1 & y2) | (oz1 & ox2);
            const uint64_t minus = (y1 & ox2) | (ox1 & oz2) | (oz1 & y2);
            sum += __builtin_popcountll(plus) - __builtin_popcountll(minus);
            xh[w] = x2 ^ x1;
            zh[w] = z2 ^ z1;
        }
        r_[h] = (uint8_t)((((sum % 4) + 4) % 4) == 2);
    }

    size_t n_, nw_, rows_;
    std::vector<uint64_t> xs_, zs_;
    std::vector<uint8_t> r_;
};

bool is_qubit(uint32_t t) {
    return !(t & (GFS_T_RECORD | GFS_T_SWEEP | GFS_T_COMBINER));
}

class Runner {
   public:
    Runner(const Circuit &c, size_t nq, std::unordered_map<uint32_t, uint32_t> map)
        : circuit_(c), tab_(nq), map_(std::move(map)) {
    }

    std::vector<uint8_t> run() {
        block(circuit_);
        std::vector<uint8_t> out((rec_.size() + 7) / 8, 0);
        for (size_t k = 0; k < rec_.size(); k++) {
            if (rec_[k]) {
                out[k >> 3] |= (uint8_t)(1u << (k & 7));
            }
        }
        return out;
    }

   private:
    uint32_t q(uint32_t t) const {
        return map_.at(t & GFS_T_VALUE_MASK);
    }

    bool lookback(uint32_t t) const {
        const uint64_t k = t & GFS_T_VALUE_MASK;
        if (k == 0 || k > rec_.size()) {
            throw std::invalid_argument(k == 0 ? "Lookback must be non-zero."
                                               : "Referred to a measurement record before the beginning of time.");
        }
        return rec_[rec_.size() - k];
    }

    // The reference collapses the targets of an X- or Y-basis measurement or reset in ascending qubit order before it
    // reads any result (tableau_simulator.inl collapse_x / collapse_y gather them in a std::set), and those of a
    // Z-basis one in the order given (collapse_z).  The order decides which random outcome is the one forced to 0, so
    // X / Y targets are collapsed here in that order first; the per-target reads that follow are then deterministic.
    void collapse_sorted(const Instruction &op, gfs_gate basis) {
        if (basis == GFS_M || basis == GFS_MR || basis == GFS_R || op.targets.size() < 2) {
            return;
        }
        std::vector<uint32_t> vs;
        for (uint32_t t : op.targets) {
            vs.push_back(t & GFS_T_VALUE_MASK);
        }
        std::sort(vs.begin(), vs.end());
        vs.erase(std::unique(vs.begin(), vs.end()), vs.end());
        for (uint32_t v : vs) {
            measure(v, basis, false, false);
        }
    }

    void measure(uint32_t t, gfs_gate basis, bool reset_after, bool record = true) {
        const uint32_t a = q(t);
        if (basis == GFS_MX || basis == GFS_RX || basis == GFS_MRX) tab_.apply(GFS_H, a);
        if (basis == GFS_MY || basis == GFS_RY || basis == GFS_MRY) tab_.apply(GFS_H_YZ, a);
        const bool m = tab_.measure_z(a);
        if (record) {
            rec_.push_back((uint8_t)(m ^ ((t & GFS_T_INVERTED) ? 1 : 0)));
        }
        if (reset_after && m) {
            tab_.apply(GFS_X, a);
        }
        if (basis == GFS_MX || basis == GFS_RX || basis == GFS_MRX) tab_.apply(GFS_H, a);
        if (basis == GFS_MY || basis == GFS_RY || basis == GFS_MRY) tab_.apply(GFS_H_YZ, a);
    }

    // One Pauli product with sign (-1)^sign: factors (qubit, x, z).  measure = true records its
    // eigenvalue bit (outcome forced to 0 when random); otherwise applies exp(-i pi/4 P) (dag: +).
    void product(const std::vector<std::array<uint32_t, 3>> &f, bool sign, bool measure, bool dag,
                 bool record = true) {
        if (f.empty()) {
            if (measure && record) {
                rec_.push_back(sign);
            }
            return;
        }
        auto rotate = [&]() {
            for (auto &e : f) {
                if (e[1] && e[2]) {
                    tab_.apply(GFS_H_YZ, e[0]);
                } else if (e[1]) {
                    tab_.apply(GFS_H, e[0]);
                }
            }
        };
        auto fold = [&]() {
            for (size_t k = 1; k < f.size(); k++) {
                tab_.apply(GFS_CX, f[k][0], f[0][0]);
            }
        };
        rotate();
        fold();
        if (measure) {
            const bool m = tab_.measure_z(f[0][0]);
            if (record) {
                rec_.push_back((uint8_t)(m ^ sign));
            }
        } else {
            tab_.apply((sign ^ dag) ? GFS_S_DAG : GFS_S, f[0][0]);
        }
        fold();
        rotate();
    }

    // Splits MPP / SPP targets into products; returns factors and sign of each (records included).
    void products(const Instruction &op, bool measure, bool dag) {
        size_t k = 0;
        const auto &ts = op.targets;
        while (k < ts.size()) {
            size_t end = k + 1;
            while (end < ts.size() && (ts[end] & GFS_T_COMBINER)) {
                end += 2;
            }
            std::map<uint32_t, std::pair<int, int>> acc;
            int e = 0;
            for (size_t j = k; j < end; j += 2) {
                const uint32_t t = ts[j];
                if (t & (GFS_T_PAULI_X | GFS_T_PAULI_Z)) {
                    const int nx = (t & GFS_T_PAULI_X) ? 1 : 0, nz = (t & GFS_T_PAULI_Z) ? 1 : 0;
                    auto &a = acc[q(t)];
                    e += pauli_g(a.first, a.second, nx, nz);
                    a.first ^= nx;
                    a.second ^= nz;
                    if (t & GFS_T_INVERTED) {
                        e += 2;
                    }
                } else if (t & GFS_T_RECORD) {
                    if (lookback(t)) {
                        e += 2;
                    }
                } else if (t & GFS_T_SWEEP) {
                    // Sweep bits read as zero.
                } else {
                    throw std::invalid_argument("Found an unsupported target in a Pauli product.");
                }
            }
            e = ((e % 4) + 4) % 4;
            if (e & 1) {
                throw std::invalid_argument("Acted on an anti-Hermitian operator (e.g. X0*Z0 instead of Y0).");
            }
            std::vector<std::array<uint32_t, 3>> f;
            for (auto &a : acc) {
                if (a.second.first || a.second.second) {
                    f.push_back({a.first, (uint32_t)a.second.first, (uint32_t)a.second.second});
                }
            }
            product(f, e == 2, measure, dag);
            k = end;
        }
    }

    void two_qubit(const Instruction &op) {
        const gfs_gate g = op.gate;
        for (size_t k = 0; k + 1 < op.targets.size(); k += 2) {
            const uint32_t a = op.targets[k], b = op.targets[k + 1];
            const bool ca = !is_qubit(a), cb = !is_qubit(b);
            if (!ca && !cb) {
                tab_.apply(g, q(a), q(b));
                continue;
            }
            // Classical control: a record (or sweep) bit on the Z side applies the other side's Pauli.
            if (ca && cb) {
                continue;
            }
            const uint32_t bit = ca ? a : b, other = ca ? b : a;
            if (bit & GFS_T_SWEEP) {
                continue;
            }
            if (!lookback(bit)) {
                continue;
            }
            gfs_gate pauli;
            switch (g) {
                case GFS_CX:
                    pauli = GFS_X;
                    break;
                case GFS_CY:
                    pauli = GFS_Y;
                    break;
                case GFS_CZ:
                    pauli = GFS_Z;
                    break;
                case GFS_XCZ:
                    pauli = GFS_X;
                    break;
                case GFS_YCZ:
                    pauli = GFS_Y;
                    break;
                default:
                    throw std::invalid_argument("classically controlled gate not supported");
            }
            tab_.apply(pauli, q(other));
        }
    }

    // MXX / MYY / MZZ as the reference runs them (tableau_simulator.inl do_MXX and gate_decomposition.cc
    // decompose_pair_instruction_into_disjoint_segments): the pairs split into runs on disjoint qubits, and within a
    // run MXX / MYY collapse their pairs in ascending order of the first target's qubit, MZZ in the order given,
    // before the results are read in the order given.
    void pair_measure(const Instruction &op) {
        const uint32_t x = op.gate == GFS_MZZ ? 0 : 1, z = op.gate == GFS_MXX ? 0 : 1;
        auto pair_product = [&](size_t k, bool record) {
            const uint32_t a = op.targets[k], b = op.targets[k + 1];
            const bool sign = ((a ^ b) & GFS_T_INVERTED) != 0;
            if (q(a) == q(b)) {
                if (record) {
                    rec_.push_back(sign);
                }
                return;
            }
            product({{q(a), x, z}, {q(b), x, z}}, sign, true, false, record);
        };
        auto run = [&](size_t lo, size_t hi) {
            if (op.gate != GFS_MZZ) {
                std::vector<std::pair<uint32_t, size_t>> order;
                for (size_t k = lo; k < hi; k += 2) {
                    order.push_back({op.targets[k] & GFS_T_VALUE_MASK, k});
                }
                std::sort(order.begin(), order.end());
                for (const auto &e : order) {
                    pair_product(e.second, false);
                }
            }
            for (size_t k = lo; k < hi; k += 2) {
                pair_product(k, true);
            }
        };
        std::vector<uint32_t> used;
        size_t lo = 0;
        const size_t n = op.targets.size() & ~(size_t)1;
        for (size_t k = 0; k < n; k += 2) {
            const uint32_t v0 = op.targets[k] & GFS_T_VALUE_MASK, v1 = op.targets[k + 1] & GFS_T_VALUE_MASK;
            if (std::find(used.begin(), used.end(), v0) != used.end() ||
                std::find(used.begin(), used.end(), v1) != used.end()) {
                run(lo, k);
                lo = k;
                used.clear();
            }
            used.push_back(v0);
            used.push_back(v1);
        }
        if (lo < n) {
            run(lo, n);
        }
    }

    void instruction(const Instruction &op) {
        const gfs_gate g = op.gate;
        const uint32_t flags = gate_info(g).flags;
        switch (g) {
            case GFS_M:
            case GFS_MX:
            case GFS_MY:
                collapse_sorted(op, g);
                for (uint32_t t : op.targets) measure(t, g, false);
                return;
            case GFS_MR:
            case GFS_MRX:
            case GFS_MRY:
                collapse_sorted(op, g);
                for (uint32_t t : op.targets) measure(t, g, true);
                return;
            case GFS_R:
            case GFS_RX:
            case GFS_RY:
                collapse_sorted(op, g);
                for (uint32_t t : op.targets) measure(t, g, true, false);
                return;
            case GFS_MPAD:
                for (uint32_t t : op.targets) rec_.push_back((t & GFS_T_VALUE_MASK) != 0);
                return;
            case GFS_HERALDED_ERASE:
            case GFS_HERALDED_PAULI_CHANNEL_1:
                rec_.insert(rec_.end(), op.targets.size(), 0);
                return;
            case GFS_MPP:
                products(op, true, false);
                return;
            case GFS_SPP:
            case GFS_SPP_DAG:
                products(op, false, g == GFS_SPP_DAG);
                return;
            case GFS_MXX:
            case GFS_MYY:
            case GFS_MZZ:
                pair_measure(op);
                return;
            default:
                break;
        }
        if (flags & (GFS_F_NOISY | GFS_F_NO_EFFECT)) {
            return;
        }
        if (flags & GFS_F_PAIRS) {
            two_qubit(op);
            return;
        }
        if (flags & GFS_F_UNITARY) {
            for (uint32_t t : op.targets) tab_.apply(g, q(t));
            return;
        }
    }

    void block(const Circuit &c) {
        for (const Instruction &op : c.ops) {
            if (op.gate == GFS_REPEAT) {
                for (uint64_t k = 0; k < op.reps; k++) {
                    block(c.blocks[op.block]);
                }
                continue;
            }
            instruction(op);
        }
    }

    const Circuit &circuit_;
    Tableau tab_;
    std::unordered_map<uint32_t, uint32_t> map_;
    std::vector<uint8_t> rec_;
};

void collect(const Circuit &c, std::unordered_map<uint32_t, uint32_t> &map) {
    for (const Instruction &op : c.ops) {
        if (op.gate == GFS_REPEAT) {
            collect(c.blocks[op.block], map);
            continue;
        }
        if (op.gate == GFS_MPAD) {
            continue;
        }
        for (uint32_t t : op.targets) {
            if (is_qubit(t) && !map.count(t & GFS_T_VALUE_MASK)) {
                const uint32_t id = (uint32_t)map.size();
                map[t & GFS_T_VALUE_MASK] = id;
            }
        }
    }
}

}  // namespace

std::vector<uint8_t> reference_sample(const Circuit &circuit) {
    std::unordered_map<uint32_t, uint32_t> map;
    collect(circuit, map);
    const size_t nq = map.size();
    Runner r(circuit, nq, std::move(map));
    return r.run();
}

}  // namespace gfs
