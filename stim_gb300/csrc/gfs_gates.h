/*
 * gfs_gates.h -- the gate vocabulary of the .stim circuit format (names, aliases, argument counts,
 * target rules), as the reference defines it in src/stim/gates/gates.h:91-233 and the per-family
 * tables src/stim/gates/gate_data_*.cc.  Plain C so the product's parser and the CPU oracle read the
 * same table; the enum order is this project's own.
 */
#ifndef GFS_GATES_H
#define GFS_GATES_H

#include <stddef.h>
#include <stdint.h>

typedef enum gfs_gate {
    GFS_NOT_A_GATE = 0,
    GFS_DETECTOR,
    GFS_OBSERVABLE_INCLUDE,
    GFS_TICK,
    GFS_QUBIT_COORDS,
    GFS_SHIFT_COORDS,
    GFS_REPEAT,
    GFS_MPAD,
    GFS_MX,
    GFS_MY,
    GFS_M,
    GFS_MRX,
    GFS_MRY,
    GFS_MR,
    GFS_RX,
    GFS_RY,
    GFS_R,
    GFS_XCX,
    GFS_XCY,
    GFS_XCZ,
    GFS_YCX,
    GFS_YCY,
    GFS_YCZ,
    GFS_CX,
    GFS_CY,
    GFS_CZ,
    GFS_H,
    GFS_H_XY,
    GFS_H_YZ,
    GFS_H_NXY,
    GFS_H_NXZ,
    GFS_H_NYZ,
    GFS_DEPOLARIZE1,
    GFS_DEPOLARIZE2,
    GFS_X_ERROR,
    GFS_Y_ERROR,
    GFS_Z_ERROR,
    GFS_I_ERROR,
    GFS_II_ERROR,
    GFS_PAULI_CHANNEL_1,
    GFS_PAULI_CHANNEL_2,
    GFS_E,
    GFS_ELSE_CORRELATED_ERROR,
    GFS_HERALDED_ERASE,
    GFS_HERALDED_PAULI_CHANNEL_1,
    GFS_I,
    GFS_X,
    GFS_Y,
    GFS_Z,
    GFS_C_XYZ,
    GFS_C_ZYX,
    GFS_C_NXYZ,
    GFS_C_XNYZ,
    GFS_C_XYNZ,
    GFS_C_NZYX,
    GFS_C_ZNYX,
    GFS_C_ZYNX,
    GFS_SQRT_X,
    GFS_SQRT_X_DAG,
    GFS_SQRT_Y,
    GFS_SQRT_Y_DAG,
    GFS_S,
    GFS_S_DAG,
    GFS_II,
    GFS_SQRT_XX,
    GFS_SQRT_XX_DAG,
    GFS_SQRT_YY,
    GFS_SQRT_YY_DAG,
    GFS_SQRT_ZZ,
    GFS_SQRT_ZZ_DAG,
    GFS_MPP,
    GFS_SPP,
    GFS_SPP_DAG,
    GFS_SWAP,
    GFS_ISWAP,
    GFS_CXSWAP,
    GFS_SWAPCX,
    GFS_CZSWAP,
    GFS_ISWAP_DAG,
    GFS_MXX,
    GFS_MYY,
    GFS_MZZ,
    GFS_NUM_GATES
} gfs_gate;

/* Gate flags; meanings follow GateFlags in the reference (gates.h:192-233). */
enum {
    GFS_F_UNITARY = 1 << 0,
    GFS_F_NOISY = 1 << 1,
    GFS_F_DISJOINT_PROBS = 1 << 2,
    GFS_F_RESULTS = 1 << 3,
    GFS_F_NOT_FUSABLE = 1 << 4,
    GFS_F_BLOCK = 1 << 5,
    GFS_F_PAIRS = 1 << 6,
    GFS_F_PAULI_STRING = 1 << 7,
    GFS_F_ONLY_REC = 1 << 8,
    GFS_F_CAN_TARGET_BITS = 1 << 9,
    GFS_F_NO_TARGETS = 1 << 10,
    GFS_F_UINT_ARGS = 1 << 11,
    GFS_F_COMBINERS = 1 << 12,
    GFS_F_RESET = 1 << 13,
    GFS_F_NO_EFFECT = 1 << 14,
    GFS_F_SINGLE_QUBIT = 1 << 15,
};

#define GFS_ARGS_ANY (-1)
#define GFS_ARGS_ZERO_OR_ONE (-2)

typedef struct gfs_gate_info {
    const char *name;
    gfs_gate id;
    int arg_count;
    uint32_t flags;
} gfs_gate_info;

/* Target encoding (the same bit layout as the reference's GateTarget, gate_target.h:27-33). */
#define GFS_T_VALUE_MASK ((1u << 24) - 1u)
#define GFS_T_INVERTED (1u << 31)
#define GFS_T_PAULI_X (1u << 30)
#define GFS_T_PAULI_Z (1u << 29)
#define GFS_T_RECORD (1u << 28)
#define GFS_T_COMBINER (1u << 27)
#define GFS_T_SWEEP (1u << 26)

#define GFS__R GFS_F_RESULTS
#define GFS__N GFS_F_NOISY
#define GFS__P GFS_F_DISJOINT_PROBS
#define GFS__U GFS_F_UNITARY
#define GFS__S GFS_F_SINGLE_QUBIT
#define GFS__2 GFS_F_PAIRS

static const gfs_gate_info GFS_GATE_TABLE[] = {
    {"DETECTOR", GFS_DETECTOR, GFS_ARGS_ANY, GFS_F_ONLY_REC | GFS_F_NOT_FUSABLE | GFS_F_NO_EFFECT},
    {"OBSERVABLE_INCLUDE", GFS_OBSERVABLE_INCLUDE, 1,
     GFS_F_ONLY_REC | GFS_F_PAULI_STRING | GFS_F_NOT_FUSABLE | GFS_F_UINT_ARGS | GFS_F_NO_EFFECT},
    {"TICK", GFS_TICK, 0, GFS_F_NOT_FUSABLE | GFS_F_NO_TARGETS | GFS_F_NO_EFFECT},
    {"QUBIT_COORDS", GFS_QUBIT_COORDS, GFS_ARGS_ANY, GFS_F_NOT_FUSABLE | GFS_F_NO_EFFECT},
    {"SHIFT_COORDS", GFS_SHIFT_COORDS, GFS_ARGS_ANY, GFS_F_NOT_FUSABLE | GFS_F_NO_TARGETS | GFS_F_NO_EFFECT},
    {"REPEAT", GFS_REPEAT, 0, GFS_F_BLOCK | GFS_F_NOT_FUSABLE},
    {"MPAD", GFS_MPAD, GFS_ARGS_ZERO_OR_ONE, GFS__R | GFS__P},
    {"MX", GFS_MX, GFS_ARGS_ZERO_OR_ONE, GFS__S | GFS__R | GFS__N | GFS__P},
    {"MY", GFS_MY, GFS_ARGS_ZERO_OR_ONE, GFS__S | GFS__R | GFS__N | GFS__P},
    {"M", GFS_M, GFS_ARGS_ZERO_OR_ONE, GFS__S | GFS__R | GFS__N | GFS__P},
    {"MRX", GFS_MRX, GFS_ARGS_ZERO_OR_ONE, GFS__S | GFS__R | GFS__N | GFS__P | GFS_F_RESET},
    {"MRY", GFS_MRY, GFS_ARGS_ZERO_OR_ONE, GFS__S | GFS__R | GFS__N | GFS__P | GFS_F_RESET},
    {"MR", GFS_MR, GFS_ARGS_ZERO_OR_ONE, GFS__S | GFS__R | GFS__N | GFS__P | GFS_F_RESET},
    {"RX", GFS_RX, 0, GFS__S | GFS_F_RESET},
    {"RY", GFS_RY, 0, GFS__S | GFS_F_RESET},
    {"R", GFS_R, 0, GFS__S | GFS_F_RESET},
    {"XCX", GFS_XCX, 0, GFS__U | GFS__2},
    {"XCY", GFS_XCY, 0, GFS__U | GFS__2},
    {"XCZ", GFS_XCZ, 0, GFS__U | GFS__2 | GFS_F_CAN_TARGET_BITS},
    {"YCX", GFS_YCX, 0, GFS__U | GFS__2},
    {"YCY", GFS_YCY, 0, GFS__U | GFS__2},
    {"YCZ", GFS_YCZ, 0, GFS__U | GFS__2 | GFS_F_CAN_TARGET_BITS},
    {"CX", GFS_CX, 0, GFS__U | GFS__2 | GFS_F_CAN_TARGET_BITS},
    {"CY", GFS_CY, 0, GFS__U | GFS__2 | GFS_F_CAN_TARGET_BITS},
    {"CZ", GFS_CZ, 0, GFS__U | GFS__2 | GFS_F_CAN_TARGET_BITS},
    {"H", GFS_H, 0, GFS__S | GFS__U},
    {"H_XY", GFS_H_XY, 0, GFS__S | GFS__U},
    {"H_YZ", GFS_H_YZ, 0, GFS__S | GFS__U},
    {"H_NXY", GFS_H_NXY, 0, GFS__S | GFS__U},
    {"H_NXZ", GFS_H_NXZ, 0, GFS__S | GFS__U},
    {"H_NYZ", GFS_H_NYZ, 0, GFS__S | GFS__U},
    {"DEPOLARIZE1", GFS_DEPOLARIZE1, 1, GFS__S | GFS__N | GFS__P},
    {"DEPOLARIZE2", GFS_DEPOLARIZE2, 1, GFS__N | GFS__P | GFS__2},
    {"I_ERROR", GFS_I_ERROR, GFS_ARGS_ANY, GFS__S | GFS__N | GFS__P},
    {"II_ERROR", GFS_II_ERROR, GFS_ARGS_ANY, GFS__2 | GFS__N | GFS__P},
    {"X_ERROR", GFS_X_ERROR, 1, GFS__S | GFS__N | GFS__P},
    {"Y_ERROR", GFS_Y_ERROR, 1, GFS__S | GFS__N | GFS__P},
    {"Z_ERROR", GFS_Z_ERROR, 1, GFS__S | GFS__N | GFS__P},
    {"PAULI_CHANNEL_1", GFS_PAULI_CHANNEL_1, 3, GFS__S | GFS__N | GFS__P},
    {"PAULI_CHANNEL_2", GFS_PAULI_CHANNEL_2, 15, GFS__N | GFS__P | GFS__2},
    {"E", GFS_E, 1, GFS__N | GFS__P | GFS_F_PAULI_STRING | GFS_F_NOT_FUSABLE},
    {"ELSE_CORRELATED_ERROR", GFS_ELSE_CORRELATED_ERROR, 1,
     GFS__N | GFS__P | GFS_F_PAULI_STRING | GFS_F_NOT_FUSABLE},
    {"HERALDED_ERASE", GFS_HERALDED_ERASE, 1, GFS__S | GFS__N | GFS__P | GFS__R},
    {"HERALDED_PAULI_CHANNEL_1", GFS_HERALDED_PAULI_CHANNEL_1, 4, GFS__S | GFS__N | GFS__P | GFS__R},
    {"I", GFS_I, 0, GFS__S | GFS__U},
    {"X", GFS_X, 0, GFS__S | GFS__U},
    {"Y", GFS_Y, 0, GFS__S | GFS__U},
    {"Z", GFS_Z, 0, GFS__S | GFS__U},
    {"C_XYZ", GFS_C_XYZ, 0, GFS__S | GFS__U},
    {"C_ZYX", GFS_C_ZYX, 0, GFS__S | GFS__U},
    {"C_NXYZ", GFS_C_NXYZ, 0, GFS__S | GFS__U},
    {"C_XNYZ", GFS_C_XNYZ, 0, GFS__S | GFS__U},
    {"C_XYNZ", GFS_C_XYNZ, 0, GFS__S | GFS__U},
    {"C_NZYX", GFS_C_NZYX, 0, GFS__S | GFS__U},
    {"C_ZNYX", GFS_C_ZNYX, 0, GFS__S | GFS__U},
    {"C_ZYNX", GFS_C_ZYNX, 0, GFS__S | GFS__U},
    {"SQRT_X", GFS_SQRT_X, 0, GFS__S | GFS__U},
    {"SQRT_X_DAG", GFS_SQRT_X_DAG, 0, GFS__S | GFS__U},
    {"SQRT_Y", GFS_SQRT_Y, 0, GFS__S | GFS__U},
    {"SQRT_Y_DAG", GFS_SQRT_Y_DAG, 0, GFS__S | GFS__U},
    {"S", GFS_S, 0, GFS__S | GFS__U},
    {"S_DAG", GFS_S_DAG, 0, GFS__S | GFS__U},
    {"II", GFS_II, 0, GFS__U | GFS__2},
    {"SQRT_XX", GFS_SQRT_XX, 0, GFS__U | GFS__2},
    {"SQRT_XX_DAG", GFS_SQRT_XX_DAG, 0, GFS__U | GFS__2},
    {"SQRT_YY", GFS_SQRT_YY, 0, GFS__U | GFS__2},
    {"SQRT_YY_DAG", GFS_SQRT_YY_DAG, 0, GFS__U | GFS__2},
    {"SQRT_ZZ", GFS_SQRT_ZZ, 0, GFS__U | GFS__2},
    {"SQRT_ZZ_DAG", GFS_SQRT_ZZ_DAG, 0, GFS__U | GFS__2},
    {"MPP", GFS_MPP, GFS_ARGS_ZERO_OR_ONE, GFS__R | GFS__N | GFS_F_PAULI_STRING | GFS_F_COMBINERS | GFS__P},
    {"SPP", GFS_SPP, 0, GFS_F_PAULI_STRING | GFS_F_COMBINERS | GFS__U},
    {"SPP_DAG", GFS_SPP_DAG, 0, GFS_F_PAULI_STRING | GFS_F_COMBINERS | GFS__U},
    {"SWAP", GFS_SWAP, 0, GFS__U | GFS__2},
    {"ISWAP", GFS_ISWAP, 0, GFS__U | GFS__2},
    {"CXSWAP", GFS_CXSWAP, 0, GFS__U | GFS__2},
    {"SWAPCX", GFS_SWAPCX, 0, GFS__U | GFS__2},
    {"CZSWAP", GFS_CZSWAP, 0, GFS__U | GFS__2},
    {"ISWAP_DAG", GFS_ISWAP_DAG, 0, GFS__U | GFS__2},
    {"MXX", GFS_MXX, GFS_ARGS_ZERO_OR_ONE, GFS__2 | GFS__R | GFS__N | GFS__P},
    {"MYY", GFS_MYY, GFS_ARGS_ZERO_OR_ONE, GFS__2 | GFS__R | GFS__N | GFS__P},
    {"MZZ", GFS_MZZ, GFS_ARGS_ZERO_OR_ONE, GFS__2 | GFS__R | GFS__N | GFS__P},
};

typedef struct gfs_gate_alias {
    const char *name;
    gfs_gate id;
} gfs_gate_alias;

static const gfs_gate_alias GFS_GATE_ALIASES[] = {
    {"MZ", GFS_M},        {"MRZ", GFS_MR},    {"RZ", GFS_R},      {"ZCX", GFS_CX},
    {"CNOT", GFS_CX},     {"ZCY", GFS_CY},    {"ZCZ", GFS_CZ},    {"H_XZ", GFS_H},
    {"CORRELATED_ERROR", GFS_E},              {"SQRT_Z", GFS_S},  {"SQRT_Z_DAG", GFS_S_DAG},
    {"SWAPCZ", GFS_CZSWAP},
};

#undef GFS__R
#undef GFS__N
#undef GFS__P
#undef GFS__U
#undef GFS__S
#undef GFS__2

static inline int gfs_name_eq_ci(const char *a, size_t alen, const char *b) {
    size_t k = 0;
    for (; k < alen; k++) {
        char ca = a[k], cb = b[k];
        if (cb == 0) {
            return 0;
        }
        if (ca >= 'a' && ca <= 'z') {
            ca = (char)(ca - 'a' + 'A');
        }
        if (ca != cb) {
            return 0;
        }
    }
    return b[k] == 0;
}

static inline const gfs_gate_info *gfs_gate_by_id(gfs_gate g) {
    size_t n = sizeof(GFS_GATE_TABLE) / sizeof(GFS_GATE_TABLE[0]);
    for (size_t k = 0; k < n; k++) {
        if (GFS_GATE_TABLE[k].id == g) {
            return &GFS_GATE_TABLE[k];
        }
    }
    return NULL;
}

/* Case-insensitive lookup by name or alias; NULL when unknown. */
static inline const gfs_gate_info *gfs_gate_by_name(const char *name, size_t len) {
    size_t n = sizeof(GFS_GATE_TABLE) / sizeof(GFS_GATE_TABLE[0]);
    for (size_t k = 0; k < n; k++) {
        if (gfs_name_eq_ci(name, len, GFS_GATE_TABLE[k].name)) {
            return &GFS_GATE_TABLE[k];
        }
    }
    size_t na = sizeof(GFS_GATE_ALIASES) / sizeof(GFS_GATE_ALIASES[0]);
    for (size_t k = 0; k < na; k++) {
        if (gfs_name_eq_ci(name, len, GFS_GATE_ALIASES[k].name)) {
            return gfs_gate_by_id(GFS_GATE_ALIASES[k].id);
        }
    }
    return NULL;
}

#endif /* GFS_GATES_H */
