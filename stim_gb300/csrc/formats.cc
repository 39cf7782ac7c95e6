// Result file formats of sample_write: 01, b8, r8, hits, dets, ptb64.
//
// The byte layouts are an interface (doc/result_formats.md); the rules restated here follow the
// reference's writers (src/stim/io/measure_record_writer.cc:61-211) and write_table_data
// (measure_record_writer.h:112-166): dets prefixes switch at a transition index and restart their
// numbering there, r8 emits 255 for a run of 255 zeros without a one and ends each shot with the run to
// one past its end, ptb64 needs a multiple of 64 shots and writes, per 64-shot group, one little-endian
// 64-bit word per bit position.
#include "formats.h"

#include <cinttypes>
#include <stdexcept>
#include <string>

namespace gfs {

Format parse_format(std::string_view name) {
    if (name == "01") return Format::F01;
    if (name == "b8") return Format::B8;
    if (name == "dets") return Format::DETS;
    if (name == "hits") return Format::HITS;
    if (name == "ptb64") return Format::PTB64;
    if (name == "r8") return Format::R8;
    throw std::invalid_argument("Unrecognized output format: '" + std::string(name) +
                                "'. Recognized formats are:\n    01\n    b8\n    dets\n    hits\n    ptb64\n    r8\n");
}

namespace {

inline bool bit(const uint8_t *row, uint64_t k) {
    return (row[k >> 3] >> (k & 7)) & 1;
}

void put_uint(std::string &s, uint64_t v) {
    char buf[24];
    int n = snprintf(buf, sizeof(buf), "%" PRIu64, v);
    s.append(buf, (size_t)n);
}

}  // namespace

void write_rows(FILE *out, Format f, const uint8_t *rows, uint64_t stride, uint64_t shots, uint64_t nbits, char c1,
                char c2, uint64_t transition) {
    if (f == Format::PTB64) {
        if (shots % 64 != 0) {
            throw std::invalid_argument("shots must be a multiple of 64 to use ptb64 format.");
        }
        std::vector<uint64_t> words(nbits);
        for (uint64_t g = 0; g < shots / 64; g++) {
            std::fill(words.begin(), words.end(), 0);
            for (uint64_t j = 0; j < 64; j++) {
                const uint8_t *row = rows + (g * 64 + j) * stride;
                for (uint64_t m = 0; m < nbits; m++) {
                    if (bit(row, m)) {
                        words[m] |= (uint64_t)1 << j;
                    }
                }
            }
            for (uint64_t m = 0; m < nbits; m++) {
                uint8_t le[8];
                for (int b = 0; b < 8; b++) {
                    le[b] = (uint8_t)(words[m] >> (8 * b));
                }
                fwrite(le, 1, 8, out);
            }
        }
        return;
    }
    if (transition == 0) {
        transition = nbits;
        c1 = c2;
    } else if (c1 == c2 || transition >= nbits) {
        transition = nbits;
    }
    const uint64_t nbytes = (nbits + 7) / 8;
    std::string s;
    for (uint64_t shot = 0; shot < shots; shot++) {
        const uint8_t *row = rows + shot * stride;
        s.clear();
        switch (f) {
            case Format::F01:
                for (uint64_t k = 0; k < nbits; k++) {
                    s.push_back(bit(row, k) ? '1' : '0');
                }
                s.push_back('\n');
                break;
            case Format::B8:
                s.append(reinterpret_cast<const char *>(row), nbytes);
                break;
            case Format::R8: {
                uint32_t run = 0;
                for (uint64_t k = 0; k < nbits; k++) {
                    if (bit(row, k)) {
                        s.push_back((char)run);
                        run = 0;
                    } else if (++run == 255) {
                        s.push_back((char)255);
                        run = 0;
                    }
                }
                s.push_back((char)run);
                break;
            }
            case Format::HITS: {
                bool first = true;
                for (uint64_t k = 0; k < nbits; k++) {
                    if (bit(row, k)) {
                        if (!first) {
                            s.push_back(',');
                        }
                        first = false;
                        put_uint(s, k);
                    }
                }
                s.push_back('\n');
                break;
            }
            case Format::DETS:
                s.append("shot");
                for (uint64_t k = 0; k < nbits; k++) {
                    if (bit(row, k)) {
                        s.push_back(' ');
                        s.push_back(k < transition ? c1 : c2);
                        put_uint(s, k < transition ? k : k - transition);
                    }
                }
                s.push_back('\n');
                break;
            default:
                break;
        }
        fwrite(s.data(), 1, s.size(), out);
    }
}

}  // namespace gfs
