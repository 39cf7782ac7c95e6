// Result formats written on the device (sample_write): the sampler's shot-major bit-packed rows, still in HBM,
// are turned into the bytes of a result file (doc/result_formats.md; the reference's writers are
// src/stim/io/measure_record_writer.cc:61-211 and write_table_data, measure_record_writer.h:112-166), so that
// only the file's bytes cross the host link and the host merely writes them out.
//
// * 01: one thread per (shot, row byte) writes its eight characters; the last one of a row adds the newline.
// * ptb64: one warp per (64-shot group, 32 bit positions); lane b gathers bit (32c + b) of the group's 64 rows
//   into one little-endian 64-bit word.
// * hits, dets, r8 (variable length): one warp per shot measures its record, walking the row in 128-byte windows
//   (lane i on bytes 4i..4i+3, so the record's order is the lanes' order within a window), an exclusive scan over
//   shots places the records, and the same warp then writes its record, each lane at the offset its predecessors
//   leave it.
#include <cstdint>

#include "formats_device.h"

namespace gfs {

namespace {

__device__ __forceinline__ uint32_t ndigits(uint32_t v) {
    return v < 10u ? 1u
           : v < 100u ? 2u
           : v < 1000u ? 3u
           : v < 10000u ? 4u
           : v < 100000u ? 5u
           : v < 1000000u ? 6u
           : v < 10000000u ? 7u
           : v < 100000000u ? 8u
           : v < 1000000000u ? 9u
                             : 10u;
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

// The record bytes of the set bits of `word` (bit t = row bit base + t), given the row's last set bit before it
// (`prev`, -1 for none); WRITE also writes them at `o`.  hits: "k," per bit (the record's last ',' becomes its
// newline afterwards); dets: " D<k>" / " L<k - transition>"; r8: the zeros since the previous set bit, a 255 for
// each full run of 255.
template <bool WRITE>
__device__ __forceinline__ uint32_t word_record(const FormatArgs &a, uint32_t word, uint32_t base, int32_t prev,
                                                uint8_t *o) {
    uint32_t n = 0;
    while (word) {
        const uint32_t k = base + (uint32_t)(__ffs(word) - 1);
        word &= word - 1;
        if (a.fmt == (uint32_t)Format::HITS) {
            const uint32_t nd = ndigits(k);
            if (WRITE) {
                put_dec(o + n, k, nd);
                o[n + nd] = ',';
            }
            n += nd + 1;
        } else if (a.fmt == (uint32_t)Format::DETS) {
            const bool second = k >= a.transition;
            const uint32_t idx = second ? k - (uint32_t)a.transition : k;
            const uint32_t nd = ndigits(idx);
            if (WRITE) {
                o[n] = ' ';
                o[n + 1] = second ? a.c2 : a.c1;
                put_dec(o + n + 2, idx, nd);
            }
            n += nd + 2;
        } else {
            uint32_t z = k - (uint32_t)(prev + 1);
            prev = (int32_t)k;
            if (WRITE) {
                for (; z >= 255; z -= 255) {
                    o[n++] = 255;
                }
                o[n++] = (uint8_t)z;
            } else {
                n += z / 255 + 1;
            }
        }
    }
    return n;
}

// One warp per shot: WRITE = false stores the record length, WRITE = true writes the record at offs[shot].  The
// warp walks the row in windows of 128 bytes, lane i on bytes [4i, 4i + 4) of each (coalesced loads); a lane's
// part of the record goes where the lanes before it, and the earlier windows, leave off (warp prefix sums), and
// the row's last set bit before each lane comes from a warp max-scan carried across windows (r8's run lengths).
template <bool WRITE>
__global__ void __launch_bounds__(256) fmt_record_kernel(const FormatArgs a) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t shot = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (shot >= a.shots) {
        return;
    }
    const uint8_t *row = a.rows + shot * a.stride;
    const uint32_t nbits = (uint32_t)a.nbits, nbytes = (nbits + 7) / 8;
    uint8_t *const out = WRITE ? a.out + a.offs[shot] : nullptr;
    uint32_t pos = 0;   // record bytes so far
    int32_t carry = -1;  // the row's last set bit before the current window
    if (a.fmt == (uint32_t)Format::DETS) {
        if (WRITE && lane < 4) {
            out[lane] = (uint8_t)"shot"[lane];
        }
        pos = 4;
    }
    for (uint32_t w0 = 0; w0 < nbytes; w0 += 128) {
        const uint32_t b = w0 + 4 * lane, base = 8 * b;
        uint32_t word = 0;
#pragma unroll
        for (uint32_t t = 0; t < 4; t++) {
            if (b + t < nbytes) {
                word |= (uint32_t)row[b + t] << (8 * t);
            }
        }
        if (base >= nbits) {
            word = 0;
        } else if (nbits - base < 32) {
            word &= (1u << (nbits - base)) - 1u;  // padding bits past the row's last bit
        }
        const int32_t mine = word ? (int32_t)(base + 31 - __clz(word)) : -1;
        int32_t incl = mine;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d && y > incl) {
                incl = y;
            }
        }
        int32_t before = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
        if (lane == 0 || before < carry) {
            before = carry;
        }
        const uint32_t n = word_record<false>(a, word, base, before, nullptr);
        const uint32_t at = warp_excl_sum(n, lane);
        if (WRITE && n) {
            word_record<true>(a, word, base, before, out + pos + at);
        }
        pos += __shfl_sync(0xFFFFFFFFu, at + n, 31);
        const int32_t last = __shfl_sync(0xFFFFFFFFu, incl, 31);
        if (last > carry) {
            carry = last;
        }
    }
    // The record's end: r8's final run, dets' newline, hits' newline (in place of the last ',').
    uint32_t tail = 0;
    if (a.fmt == (uint32_t)Format::R8) {
        uint32_t z = nbits - 1 - (uint32_t)carry;  // carry = -1 gives nbits zeros
        tail = z / 255 + 1;
        if (WRITE && lane == 0) {
            uint8_t *o = out + pos;
            for (; z >= 255; z -= 255) {
                *o++ = 255;
            }
            *o = (uint8_t)z;
        }
    } else if (a.fmt == (uint32_t)Format::DETS || carry < 0) {
        tail = 1;
        if (WRITE && lane == 0) {
            out[pos] = '\n';
        }
    } else {
        __syncwarp();  // the ',' written by whichever lane held the row's last hit
        if (WRITE && lane == 0) {
            out[pos - 1] = '\n';
        }
    }
    if (!WRITE && lane == 0) {
        a.lens[shot] = pos + tail;
    }
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

// ptb64 straight from detector-major rows ([128-shot block][row] uint4, bit j of 32-bit word q = shot 32q + j): a
// 64-shot group's word for a bit is half of that bit's 16-byte row, so one thread per (block, bit) writes the
// words of the block's two groups; bits [0, n1) come from `first`, [n1, n1 + n2) from `second`.
__global__ void __launch_bounds__(256) fmt_ptb64_detmajor_kernel(const uint4 *first, uint64_t n1, const uint4 *second,
                                                                 uint64_t n2, uint64_t shots, uint8_t *out) {
    const uint64_t nbits = n1 + n2;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t blocks = (shots + 127) / 128;
    if (i >= blocks * nbits) {
        return;
    }
    const uint64_t b = i / nbits, m = i % nbits;
    const uint4 v = m < n1 ? first[b * n1 + m] : second[b * n2 + (m - n1)];
    unsigned long long *o = reinterpret_cast<unsigned long long *>(out);
    o[(2 * b) * nbits + m] = (unsigned long long)v.x | ((unsigned long long)v.y << 32);
    if ((2 * b + 1) * 64 < shots) {
        o[(2 * b + 1) * nbits + m] = (unsigned long long)v.z | ((unsigned long long)v.w << 32);
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

cudaError_t launch_ptb64_detmajor(const uint4 *first, uint64_t n1, const uint4 *second, uint64_t n2, uint64_t shots,
                                  uint8_t *out, cudaStream_t stream) {
    const uint64_t n = (shots + 127) / 128 * (n1 + n2);
    if (n == 0) {
        return cudaSuccess;
    }
    if (shots % 64 != 0 || (n + 255) / 256 > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    fmt_ptb64_detmajor_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(first, n1, second, n2, shots, out);
    return cudaGetLastError();
}

cudaError_t launch_format_lengths(const FormatArgs &a, uint64_t *block_sums, uint64_t *total, cudaStream_t stream) {
    if (a.shots == 0) {
        return cudaSuccess;
    }
    if (a.nbits >= (1ull << 31)) {  // bit indices are 32-bit in the record kernel
        return cudaErrorInvalidValue;
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
        if (a.nbits == 0) {  // every record is its newline alone
            return cudaMemsetAsync(a.out, '\n', a.shots, stream);
        }
        const uint64_t n = a.shots * ((a.nbits + 7) / 8);
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
