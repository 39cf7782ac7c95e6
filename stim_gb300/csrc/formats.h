// Result file formats of sample_write (see formats.cc).
#pragma once

#include <cstdint>
#include <cstdio>
#include <string_view>
#include <vector>

namespace gfs {

enum class Format { F01, B8, R8, PTB64, HITS, DETS };

// Throws std::invalid_argument with the reference's message for an unknown name.
Format parse_format(std::string_view name);

// Writes `shots` rows of `nbits` bits each (bit-packed little-endian rows, `stride` bytes apart).  For
// dets, bits [0, transition) are named with prefix c1 and the rest with c2, numbered from 0 at the
// transition (transition 0: all c2).  ptb64 needs shots % 64 == 0.
void write_rows(FILE *out, Format f, const uint8_t *rows, uint64_t stride, uint64_t shots, uint64_t nbits, char c1,
                char c2, uint64_t transition);

}  // namespace gfs
