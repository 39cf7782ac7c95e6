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

// Reads records of nm measurement, nd detector and nl observable bits, in that order (dets tokens M<k>, D<k>,
// L<k>), as the reference's MeasureRecordReader does (src/stim/io/measure_record_reader.inl).  read() fills one
// bit-packed row (ceil(bits / 8) bytes) and returns false at a clean end of data; malformed data throws
// std::invalid_argument with the reference's messages.
class RowReader {
  public:
    RowReader(FILE *in, Format f, uint64_t nm, uint64_t nd = 0, uint64_t nl = 0);
    bool read(uint8_t *row);
    // The format encodes a record of this size as no bytes, so the number of records cannot be known.
    bool empty_records() const;

  private:
    bool read_01(uint8_t *row);
    bool read_b8(uint8_t *row);
    bool read_hits(uint8_t *row);
    bool read_r8(uint8_t *row);
    bool read_dets(uint8_t *row);
    bool read_ptb64(uint8_t *row);
    FILE *in;
    Format f;
    uint64_t nm, nd, nl, n;
    std::vector<uint8_t> group;  // ptb64: the current 64-record group, n words of 64 bits
    uint32_t group_left = 0;
};

}  // namespace gfs
