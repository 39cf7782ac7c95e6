// Result formats written on the device (sample_write): the sampler's shot-major bit-packed rows, still in HBM,
// are turned into the bytes of a result file (doc/result_formats.md; the reference's writers are
// src/stim/io/measure_record_writer.cc:61-211 and write_table_data, measure_record_writer.h:112-166), so that
// only the file's bytes cross the host link and the host merely writes them out.
//
// * 01: one thread per (shot, row byte) writes its eight characters; the last one of a row adds the newline.
// * ptb64: one warp per (64-shot group, 32 bit positions); lane b gathers bit (32c + b) of the group's 64 rows
//   into one little-endian 64-bit word.
// * hits, dets, r8 (variable length): one warp per shot measures its record (lanes take contiguous ranges of the
//   row so that the record's order is the lanes' order), an exclusive scan over shots places the records, and
//   the same warp then writes its record, each lane at the offset its predecessors leave it.
#include <cstdint>

#include "formats_device.h"

namespace gfs {

namespace {

__device__ __forceinline__ uint32_t ndigits(uint32_t v) {
    uint32_t n = 1;
    while (v >= 10) {
        v /= 10;
        n++;
    }
    return n;
}

// Writes v in decimal at p (exactly ndigits(v) characters).
__device__ __forceinline__ void put_dec(uint8_t *p, uint32_t v, uint32_t nd) {
    for (uint32_t i = nd; i-- > 0;) {
        p[i] = (uint8_t)('0' + v % 10);
        v /= 10;
    }
}

__device__ __forceinline__ uint32_t warp_excl_sum(uint32_t x, uint32_t lane) {
    uint32_t incl = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= (uint32_t)d) {
            incl += y;
        }
    }
    return incl - x;
}

// Lane `lane`'s contiguous range of row bytes [b0, b1).
__device__ __forceinline__ void lane_range(uint64_t nbytes, uint32_t lane, uint64_t *b0, uint64_t *b1) {
    const uint64_t per = (nbytes + 31) / 32;
    *b0 = min(nbytes, per * lane);
    *b1 = min(nbytes, *b0 + per);
}

// Bytes this lane's part of the record takes (WRITE = false) or writes them at `out` (WRITE = true).  `prev` is
// the row's last set bit before this lane's range (-1 for none), `mine` this lane's last set bit (-1 for none),
// `hits_after` whether later lanes hold set bits, `row_empty` whether the row has none at all.
template <bool WRITE>
__device__ __forceinline__ uint32_t lane_record(const FormatArgs &a, const uint8_t *row, uint64_t b0, uint64_t b1,
                                                int64_t prev, int64_t mine, bool hits_after, bool row_empty,
                                                bool first_lane, bool last_lane, uint8_t *out) {
    uint32_t n = 0;
    auto emit = [&](uint8_t c) {
        if (WRITE) {
            out[n] = c;
        }
        n++;
    };
    const uint32_t fmt = a.fmt;
    if (fmt == (uint32_t)Format::DETS && first_lane) {
        emit('s');
        emit('h');
        emit('o');
        emit('t');
    }
    for (uint64_t j = b0; j < b1; j++) {
        uint32_t byte = row[j];
        if (8 * j + 8 > a.nbits) {
            byte &= (1u << (a.nbits - 8 * j)) - 1u;
        }
        while (byte) {
            const uint32_t t = __ffs(byte) - 1;
            byte &= byte - 1;
            const uint64_t k = 8 * j + t;
            if (k >= a.nbits) {
                break;
            }
            if (fmt == (uint32_t)Format::HITS) {
                const uint32_t nd = ndigits((uint32_t)k);
                if (WRITE) {
                    put_dec(out + n, (uint32_t)k, nd);
                }
                n += nd;
                emit(((int64_t)k != mine || hits_after) ? ',' : '\n');  // ',' unless it is the row's last hit
            } else if (fmt == (uint32_t)Format::DETS) {
                const bool second = k >= a.transition;
                const uint32_t idx = (uint32_t)(second ? k - a.transition : k);
                emit(' ');
                emit(second ? a.c2 : a.c1);
                const uint32_t nd = ndigits(idx);
                if (WRITE) {
                    put_dec(out + n, idx, nd);
                }
                n += nd;
            } else {  // R8: the zeros since the previous set bit, a 255 for each full run of 255
                uint64_t z = (uint64_t)((int64_t)k - prev - 1);
                while (z >= 255) {
                    emit(255);
                    z -= 255;
                }
                emit((uint8_t)z);
                prev = (int64_t)k;
            }
        }
    }
    if (last_lane) {
        if (fmt == (uint32_t)Format::R8) {
            uint64_t z = (uint64_t)((int64_t)a.nbits - 1 - prev);
            while (z >= 255) {
                emit(255);
                z -= 255;
            }
            emit((uint8_t)z);
        } else if (fmt == (uint32_t)Format::DETS || (fmt == (uint32_t)Format::HITS && row_empty)) {
            emit('\n');
        }
    }
    return n;
}

// The last set bit of the row in bytes [b0, b1), or -1.
__device__ __forceinline__ int64_t lane_last_bit(const FormatArgs &a, const uint8_t *row, uint64_t b0, uint64_t b1) {
    for (uint64_t j = b1; j-- > b0;) {
        uint32_t byte = row[j];
        if (8 * j + 8 > a.nbits) {
            byte &= (1u << (a.nbits - 8 * j)) - 1u;  // padding bits past the row's last bit
        }
        if (byte) {
            return (int64_t)(8 * j + (31 - __clz(byte)));
        }
    }
    return -1;
}

// One warp per shot: WRITE = false stores the record length, WRITE = true writes the record at offs[shot].
template <bool WRITE>
__global__ void __launch_bounds__(256) fmt_record_kernel(const FormatArgs a) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t shot = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (shot >= a.shots) {
        return;
    }
    const uint8_t *row = a.rows + shot * a.stride;
    const uint64_t nbytes = (a.nbits + 7) / 8;
    uint64_t b0, b1;
    lane_range(nbytes, lane, &b0, &b1);
    // The previous set bit before this lane's range (r8) and whether later lanes hold hits (hits).
    const int64_t mine = lane_last_bit(a, row, b0, b1);
    int64_t prev = -1;
    {
        int64_t incl = mine;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d && y > incl) {
                incl = y;
            }
        }
        prev = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
        if (lane == 0) {
            prev = -1;
        }
    }
    const uint32_t any_mask = __ballot_sync(0xFFFFFFFFu, mine >= 0);
    const bool hits_after = lane < 31 && (any_mask >> (lane + 1)) != 0;
    const bool row_empty = any_mask == 0;
    const uint32_t n = lane_record<false>(a, row, b0, b1, prev, mine, hits_after, row_empty, lane == 0, lane == 31,
                                          nullptr);
    if (!WRITE) {
        const uint32_t total = __reduce_add_sync(0xFFFFFFFFu, n);
        if (lane == 0) {
            a.lens[shot] = total;
        }
        return;
    }
    const uint32_t at = warp_excl_sum(n, lane);
    lane_record<true>(a, row, b0, b1, prev, mine, hits_after, row_empty, lane == 0, lane == 31,
                      a.out + a.offs[shot] + at);
}

__global__ void __launch_bounds__(256) fmt_01_kernel(const FormatArgs a) {
    const uint64_t nbytes = (a.nbits + 7) / 8;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.shots * nbytes) {
        return;
    }
    const uint64_t shot = i / nbytes, j = i % nbytes;
    const uint32_t byte = a.rows[shot * a.stride + j];
    uint8_t *o = a.out + shot * (a.nbits + 1) + 8 * j;
    const uint32_t cnt = a.nbits - 8 * j < 8 ? (uint32_t)(a.nbits - 8 * j) : 8u;
    for (uint32_t t = 0; t < cnt; t++) {
        o[t] = (uint8_t)('0' + ((byte >> t) & 1u));
    }
    if (j == nbytes - 1) {
        o[cnt] = '\n';
    }
}

__global__ void __launch_bounds__(256) fmt_ptb64_kernel(const FormatArgs a) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t cols = (a.nbits + 31) / 32;
    const uint64_t w = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (w >= (a.shots / 64) * cols) {
        return;
    }
    const uint64_t g = w / cols, c = w % cols;
    const uint64_t m = 32 * c + lane;
    uint64_t word = 0;
    const uint8_t *rows = a.rows + g * 64 * a.stride;
    for (uint32_t j = 0; j < 64; j++) {
        const uint32_t byte = m < a.nbits ? rows[j * a.stride + m / 8] : 0u;
        word |= (uint64_t)((byte >> (m % 8)) & 1u) << j;
    }
    if (m < a.nbits) {
        reinterpret_cast<unsigned long long *>(a.out)[g * a.nbits + m] = word;
    }
}

// Exclusive scan of a.lens (shots entries) into a.offs (shots + 1 entries): per 1024 shots a block scan, then one
// CTA turns the block totals into block offsets (1024 at a time), then they are added.
__global__ void __launch_bounds__(1024) scan_blocks_kernel(const uint32_t *lens, uint64_t n, uint64_t *offs,
                                                           uint64_t *block_sums) {
    __shared__ uint64_t warp_tot[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint64_t i = (uint64_t)blockIdx.x * 1024 + threadIdx.x;
    const uint64_t x = i < n ? lens[i] : 0;
    uint64_t incl = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= (uint32_t)d) {
            incl += y;
        }
    }
    if (lane == 31) {
        warp_tot[warp] = incl;
    }
    __syncthreads();
    if (warp == 0) {
        uint64_t t = warp_tot[lane];
        uint64_t ti = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, ti, d);
            if (lane >= (uint32_t)d) {
                ti += y;
            }
        }
        warp_tot[lane] = ti - t;
        if (lane == 31) {
            block_sums[blockIdx.x] = ti;
        }
    }
    __syncthreads();
    if (i < n) {
        offs[i] = warp_tot[warp] + incl - x;
    }
}

__global__ void __launch_bounds__(1024) scan_sums_kernel(uint64_t *block_sums, uint64_t nblocks, uint64_t *total) {
    __shared__ uint64_t warp_tot[32];
    __shared__ uint64_t carry;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        carry = 0;
    }
    __syncthreads();
    for (uint64_t base = 0; base < nblocks; base += 1024) {
        const uint64_t i = base + threadIdx.x;
        const uint64_t x = i < nblocks ? block_sums[i] : 0;
        uint64_t incl = x;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) {
                incl += y;
            }
        }
        if (lane == 31) {
            warp_tot[warp] = incl;
        }
        __syncthreads();
        if (warp == 0) {
            uint64_t t = warp_tot[lane];
            uint64_t ti = t;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, ti, d);
                if (lane >= (uint32_t)d) {
                    ti += y;
                }
            }
            warp_tot[lane] = ti - t;
        }
        __syncthreads();
        const uint64_t c = carry;
        if (i < nblocks) {
            block_sums[i] = c + warp_tot[warp] + incl - x;
        }
        __syncthreads();
        if (threadIdx.x == 1023) {
            carry = c + warp_tot[warp] + incl;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *total = carry;
    }
}

__global__ void __launch_bounds__(1024) scan_add_kernel(uint64_t *offs, uint64_t n, const uint64_t *block_sums,
                                                        const uint64_t *total) {
    const uint64_t i = (uint64_t)blockIdx.x * 1024 + threadIdx.x;
    if (i < n) {
        offs[i] += block_sums[blockIdx.x];
    }
    if (i == n) {
        offs[n] = *total;
    }
}

}  // namespace

uint64_t fixed_format_bytes(Format f, uint64_t shots, uint64_t nbits) {
    switch (f) {
        case Format::F01:
            return shots * (nbits + 1);
        case Format::B8:
            return shots * ((nbits + 7) / 8);
        case Format::PTB64:
            return shots / 64 * nbits * 8;
        default:
            return 0;
    }
}

cudaError_t launch_format_lengths(const FormatArgs &a, uint64_t *block_sums, uint64_t *total, cudaStream_t stream) {
    if (a.shots == 0) {
        return cudaSuccess;
    }
    const uint64_t warps_blocks = (a.shots + 7) / 8;
    if (warps_blocks > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    fmt_record_kernel<false><<<(unsigned)warps_blocks, 256, 0, stream>>>(a);
    const uint64_t nblocks = (a.shots + 1024) / 1024;  // covers index `shots` for the total
    scan_blocks_kernel<<<(unsigned)nblocks, 1024, 0, stream>>>(a.lens, a.shots, a.offs, block_sums);
    scan_sums_kernel<<<1, 1024, 0, stream>>>(block_sums, nblocks, total);
    scan_add_kernel<<<(unsigned)nblocks, 1024, 0, stream>>>(a.offs, a.shots, block_sums, total);
    return cudaGetLastError();
}

cudaError_t launch_format_write(const FormatArgs &a, cudaStream_t stream) {
    if (a.shots == 0) {
        return cudaSuccess;
    }
    const Format f = (Format)a.fmt;
    if (f == Format::F01) {
        const uint64_t n = a.shots * ((a.nbits + 7) / 8);
        if (n == 0) {
            return cudaSuccess;
        }
        fmt_01_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(a);
    } else if (f == Format::PTB64) {
        const uint64_t w = (a.shots / 64) * ((a.nbits + 31) / 32);
        if (w == 0) {
            return cudaSuccess;
        }
        fmt_ptb64_kernel<<<(unsigned)((w + 7) / 8), 256, 0, stream>>>(a);
    } else if (f == Format::HITS || f == Format::DETS || f == Format::R8) {
        fmt_record_kernel<true><<<(unsigned)((a.shots + 7) / 8), 256, 0, stream>>>(a);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace gfs
