// Pauli-frame update rules of the Clifford gates, one 32-bit word of shots at a time (bit j of each word
// is shot j).  Shared by the CUDA kernels and by the host-side analysis of the lowered program, so both see
// exactly the same linear maps.  The rules restate frame_simulator.inl:344-630 of the reference: x / z are
// the X and Z components of the frame on a qubit.
#pragma once

#include <cstdint>

#include "program.h"

#if defined(__CUDACC__)
#define GFS_RULE_HD __host__ __device__ __forceinline__
#else
#define GFS_RULE_HD inline
#endif

namespace gfs {

// One-qubit rules (K1_*): H_XZ swaps x and z; H_XY / H_YZ / C_XYZ / C_ZYX fold one component into the other.
GFS_RULE_HD void rule1w(uint32_t sub, uint32_t &x, uint32_t &z) {
    switch (sub) {
        case K1_H_XZ: {
            const uint32_t t = x;
            x = z;
            z = t;
            break;
        }
        case K1_H_XY:
            z ^= x;
            break;
        case K1_H_YZ:
            x ^= z;
            break;
        case K1_C_XYZ:
            x ^= z;
            z ^= x;
            break;
        default:  // K1_C_ZYX
            z ^= x;
            x ^= z;
            break;
    }
}

// Two-qubit rules (K2_*, frame_simulator.inl:386-630).
GFS_RULE_HD void rule2(uint32_t sub, uint32_t &x1, uint32_t &z1, uint32_t &x2, uint32_t &z2) {
    switch (sub) {
        case K2_CX:
            z1 ^= z2;
            x2 ^= x1;
            break;
        case K2_CY:
            z1 ^= x2 ^ z2;
            z2 ^= x1;
            x2 ^= x1;
            break;
        case K2_CZ:
            z1 ^= x2;
            z2 ^= x1;
            break;
        case K2_XCX:
            x1 ^= z2;
            x2 ^= z1;
            break;
        case K2_XCY:
            x1 ^= x2 ^ z2;
            x2 ^= z1;
            z2 ^= z1;
            break;
        case K2_YCX:
            x2 ^= x1 ^ z1;
            x1 ^= z2;
            z1 ^= z2;
            break;
        case K2_YCY: {
            uint32_t y1 = x1 ^ z1, y2 = x2 ^ z2;
            x1 ^= y2;
            z1 ^= y2;
            x2 ^= y1;
            z2 ^= y1;
            break;
        }
        case K2_SWAP: {
            uint32_t t = x1;
            x1 = x2;
            x2 = t;
            t = z1;
            z1 = z2;
            z2 = t;
            break;
        }
        case K2_ISWAP: {
            uint32_t dx = x1 ^ x2;
            uint32_t t1 = z1 ^ dx, t2 = z2 ^ dx;
            z1 = t2;
            z2 = t1;
            uint32_t t = x1;
            x1 = x2;
            x2 = t;
            break;
        }
        case K2_CXSWAP:
            z2 ^= z1;
            z1 ^= z2;
            x1 ^= x2;
            x2 ^= x1;
            break;
        case K2_CZSWAP: {
            uint32_t t = x1;
            x1 = x2;
            x2 = t;
            t = z1;
            z1 = z2;
            z2 = t;
            z1 ^= x2;
            z2 ^= x1;
            break;
        }
        case K2_SWAPCX:
            z1 ^= z2;
            z2 ^= z1;
            x2 ^= x1;
            x1 ^= x2;
            break;
        case K2_SQRT_XX: {
            uint32_t dz = z1 ^ z2;
            x1 ^= dz;
            x2 ^= dz;
            break;
        }
        case K2_SQRT_YY: {
            uint32_t d = x1 ^ z1 ^ x2 ^ z2;
            x1 ^= d;
            z1 ^= d;
            x2 ^= d;
            z2 ^= d;
            break;
        }
        case K2_SQRT_ZZ: {
            uint32_t dx = x1 ^ x2;
            z1 ^= dx;
            z2 ^= dx;
            break;
        }
        default:
            break;
    }
}

}  // namespace gfs
