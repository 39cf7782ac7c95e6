// Result file formats of sample_write: 01, b8, r8, hits, dets, ptb64.
//
// The byte layouts are an interface (doc/result_formats.md); the rules restated here follow the
// reference's writers (src/stim/io/measure_record_writer.cc:61-211) and write_table_data
// (measure_record_writer.h:112-166): dets prefixes switch at a transition index and restart their
// numbering there, r8 emits 255 for a run of 255 zeros without a one and ends each shot with the run to
// one past its end, ptb64 needs a multiple of 64 shots and writes, per 64-shot group, one little-endian
// 64-bit word per bit position.
#include "formats.h"

#include <algorithm>
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


// ---- Readers (convert_file) ----

namespace {

// Decimal digits starting at the next character; `next` receives the first character after them.
bool read_uint(FILE *in, uint64_t &value, int &next) {
    next = getc(in);
    if (next < '0' || next > '9') {
        return false;
    }
    value = 0;
    while (next >= '0' && next <= '9') {
        value = value * 10 + (uint64_t)(next - '0');
        next = getc(in);
    }
    return true;
}

inline void set_bit(uint8_t *row, uint64_t k) {
    row[k >> 3] |= (uint8_t)(1u << (k & 7));
}

}  // namespace

RowReader::RowReader(FILE *in_, Format f_, uint64_t nm_, uint64_t nd_, uint64_t nl_)
    : in(in_), f(f_), nm(nm_), nd(nd_), nl(nl_), n(nm_ + nd_ + nl_) {
}

bool RowReader::empty_records() const {
    return (f == Format::B8 || f == Format::PTB64) && n == 0;
}

bool RowReader::read(uint8_t *row) {
    switch (f) {
        case Format::F01:
            return read_01(row);
        case Format::B8:
            return read_b8(row);
        case Format::HITS:
            return read_hits(row);
        case Format::R8:
            return read_r8(row);
        case Format::DETS:
            return read_dets(row);
        default:
            return read_ptb64(row);
    }
}

bool RowReader::read_01(uint8_t *row) {
    std::fill(row, row + (n + 7) / 8, 0);
    for (uint64_t k = 0; k < n; k++) {
        const int b = getc(in);
        if (b == '1') {
            set_bit(row, k);
        } else if (b == '0') {
        } else if (b == EOF && k == 0) {
            return false;
        } else if (b == EOF || b == '\r' || b == '\n') {
            throw std::invalid_argument("01 data ended in middle of record at byte position " + std::to_string(k) +
                                        ".\nExpected bits per record was " + std::to_string(n) + ".");
        } else {
            throw std::invalid_argument("Unexpected character in 01 format data: '" + std::to_string(b) + "'.");
        }
    }
    int last = getc(in);
    if (n == 0 && last == EOF) {
        return false;
    }
    if (last == '\r') {
        last = getc(in);
    }
    if (last != '\n') {
        throw std::invalid_argument("01 data didn't end with a newline after the expected data length of '" +
                                    std::to_string(n) + "'.");
    }
    return true;
}

bool RowReader::read_b8(uint8_t *row) {
    const uint64_t nb = (n + 7) / 8;
    const size_t nr = fread(row, 1, nb, in);
    if (nr == 0) {
        return false;
    }
    if (nr != nb) {
        throw std::invalid_argument("b8 data ended in middle of record at byte position " + std::to_string(nr) +
                                    ".\nExpected bytes per record was " + std::to_string(nb) + " (" +
                                    std::to_string(n) + " bits padded).");
    }
    return true;
}

bool RowReader::read_hits(uint8_t *row) {
    std::fill(row, row + (n + 7) / 8, 0);
    const char *bad = "HITS data wasn't comma-separated integers terminated by a newline.";
    bool first = true;
    for (;;) {
        uint64_t v = 0;
        int next = 0;
        if (!read_uint(in, v, next)) {
            if (first && next == EOF) {
                return false;
            }
            if (first && next == '\r') {
                next = getc(in);
            }
            if (first && next == '\n') {
                return true;
            }
            throw std::invalid_argument(bad);
        }
        if (v >= n) {
            throw std::invalid_argument("hit index is too large.");
        }
        row[v >> 3] ^= (uint8_t)(1u << (v & 7));
        first = false;
        if (next == '\r') {
            next = getc(in);
            if (next == '\n') {
                return true;
            }
        } else if (next == '\n') {
            return true;
        }
        if (next != ',') {
            throw std::invalid_argument(bad);
        }
    }
}

bool RowReader::read_r8(uint8_t *row) {
    int c = getc(in);
    if (c == EOF) {
        return false;
    }
    std::fill(row, row + (n + 7) / 8, 0);
    uint64_t pos = 0;
    for (;;) {
        pos += (uint64_t)c;
        if (c != 255) {
            if (pos < n) {
                set_bit(row, pos);
                pos++;
            } else if (pos == n) {
                return true;
            } else {
                throw std::invalid_argument("r8 data jumped past expected end of encoded data. Expected to decode " +
                                            std::to_string(n) + " bits.");
            }
        }
        c = getc(in);
        if (c == EOF) {
            throw std::invalid_argument("End of file before end of r8 data. Expected to decode " + std::to_string(n) +
                                        " bits.");
        }
    }
}

bool RowReader::read_dets(uint8_t *row) {
    for (;;) {
        const int c = getc(in);
        if (c == ' ' || c == '\n' || c == '\r' || c == '\t') {
            continue;
        }
        if (c == EOF) {
            return false;
        }
        if (c != 's' || getc(in) != 'h' || getc(in) != 'o' || getc(in) != 't') {
            throw std::invalid_argument("DETS data didn't start with 'shot'");
        }
        break;
    }
    std::fill(row, row + (n + 7) / 8, 0);
    int c = getc(in);
    for (;;) {
        if (c == '\r') {
            c = getc(in);
        }
        if (c == '\n' || c == EOF) {
            return true;
        }
        if (c != ' ') {
            throw std::invalid_argument("DETS data wasn't single-space-separated with no trailing spaces.");
        }
        c = getc(in);
        uint64_t offset, length;
        if (c == 'M') {
            offset = 0;
            length = nm;
        } else if (c == 'D') {
            offset = nm;
            length = nd;
        } else if (c == 'L') {
            offset = nm + nd;
            length = nl;
        } else {
            throw std::invalid_argument("Unrecognized DETS prefix. Expected M or D or L not '" + std::to_string(c) +
                                        "'");
        }
        const char prefix = (char)c;
        uint64_t v = 0;
        if (!read_uint(in, v, c)) {
            throw std::invalid_argument("DETS data had a value prefix (M or D or L) not followed by an integer.");
        }
        if (v >= length) {
            throw std::invalid_argument("DETS data had a value larger than expected. Got " + std::string(1, prefix) +
                                        std::to_string(v) + " but expected length of " + std::string(1, prefix) +
                                        " space to be " + std::to_string(length) + ".");
        }
        set_bit(row, offset + v);
    }
}

bool RowReader::read_ptb64(uint8_t *row) {
    if (group_left == 0) {
        const uint64_t nb = n * 8;
        group.resize(nb);
        const size_t nr = nb ? fread(group.data(), 1, nb, in) : 0;
        if (nr == 0) {
            return false;
        }
        if (nr != nb) {
            throw std::invalid_argument("ptb64 data ended in middle of 64 record group at byte position " +
                                        std::to_string(nr) + ".\nExpected bytes per 64 records was " +
                                        std::to_string(nb) + " (" + std::to_string(n) + " bits padded).");
        }
        group_left = 64;
    }
    const uint32_t s = 64 - group_left;  // record within the group
    std::fill(row, row + (n + 7) / 8, 0);
    for (uint64_t k = 0; k < n; k++) {
        if ((group[8 * k + (s >> 3)] >> (s & 7)) & 1) {
            set_bit(row, k);
        }
    }
    group_left--;
    return true;
}

}  // namespace gfs
