// pre_io.cpp -- host side of preprocess: raw FASTA / FASTQ records and the
// _Clean / .frq writer.
//
// readFile (preprocess.cpp:74-242) reads its input with fgets into a
// 4096-byte buffer, so a line longer than 4095 bytes arrives as several
// pieces, each handled as a line of its own.  This parser maps the whole
// file into memory and cuts the same pieces (up to and including '\n', at
// most 4095 bytes), with the same end-of-file behaviour: a piece that ends
// at end of file without '\n' raises the end flag, and a read attempt at
// end of file yields the '$' marker the reference leaves in its buffer.
// Each piece is a C string (it ends at its first NUL byte, as
// string::assign(char*) does).  Kept on purpose, because they decide which
// bytes and labels reach the output:
//   * trailing whitespace is trimmed per piece, but a piece of whitespace
//     only is kept whole (find_last_not_of finds nothing), so a blank line
//     inside a FASTA record adds "\n" to the sequence;
//   * FASTA sequence pieces lose their trailing bytes outside
//     "nNATGCatgc", unless they hold none of those bytes;
//   * a piece starting with '$' ends the input;
//   * a FASTA header with no sequence after it counts as a record but
//     leaves the label unchanged, so the next read keeps the earlier label.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

struct crispy_raw {
    bool fastq = false;
    std::string bases;
    std::vector<int64_t> offsets;
    std::vector<int32_t> lengths;
    std::vector<uint8_t> freq;
    std::string labels;
    std::vector<int64_t> label_off;
    std::vector<int32_t> label_len;
    int32_t records = 0;
};

namespace {

constexpr size_t kPieceMax = 4095;   // fgets(buf, BUF_SIZE = 4096, ...) (preprocess.cpp:24)

// deleteSpaces (preprocess.cpp:58-64) keeps a piece made only of these
bool trim_space_char(unsigned char c) {
    return c == '\n' || c == '\r' || c == ' ' || c == '\t' || c == '\v' || c == '\f' || c == '\b';
}
// deleteSpacesInSeq (preprocess.cpp:65-71) cuts after the last of these
bool seq_keep_char(unsigned char c) {
    switch (c) {
        case 'n': case 'N': case 'A': case 'T': case 'G': case 'C': case 'a': case 't': case 'g': case 'c':
            return true;
        default:
            return false;
    }
}
bool is_space(unsigned char c) {   // isspace in the "C" locale
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// Length after deleteSpaces: trailing whitespace goes unless nothing else is left.
size_t space_trimmed(const char* p, size_t n) {
    size_t k = n;
    while (k > 0 && trim_space_char((unsigned char)p[k - 1])) --k;
    return k ? k : n;
}
// Length after deleteSpacesInSeq: cut after the last base letter, if any.
size_t seq_trimmed(const char* p, size_t n) {
    size_t k = n;
    while (k > 0 && !seq_keep_char((unsigned char)p[k - 1])) --k;
    return k ? k : n;
}

// A piece as a pointer into the file and its length up to the first NUL.
struct Piece {
    const char* p;
    size_t n;
    char raw0;   // first byte of the fgets buffer ('$' at end of file)
};

// fgets over an in-memory file.
struct PieceReader {
    const char* data;
    size_t size, pos = 0;
    bool eof = false;
    bool has_nul = true;   // false: the file holds no NUL byte, skip the per-piece scan
    // false at end of file (the reference's buffer then starts with '$')
    bool next(Piece& pc) {
        if (pos >= size) {
            eof = true;
            return false;
        }
        const size_t room = std::min(kPieceMax, size - pos);
        const char* p = data + pos;
        const void* nl = std::memchr(p, '\n', room);
        size_t take;
        if (nl) {
            take = (size_t)((const char*)nl - p) + 1;
        } else {
            take = room;
            if (room < kPieceMax) eof = true;   // the read ran into end of file
        }
        pos += take;
        const void* z = has_nul ? std::memchr(p, '\0', take) : nullptr;
        pc.p = p;
        pc.n = z ? (size_t)((const char*)z - p) : take;
        pc.raw0 = p[0];
        return true;
    }
};

// Appends one record: the sequence is already at bases[start, end).
void push(crispy_raw* r, int64_t start, const char* label, size_t label_n, uint8_t freq) {
    r->offsets.push_back(start);
    r->lengths.push_back((int32_t)((int64_t)r->bases.size() - start));
    r->freq.push_back(freq);
    // READ::initialize drops every whitespace byte of the label
    r->label_off.push_back((int64_t)r->labels.size());
    int32_t n = 0;
    for (size_t i = 0; i < label_n; ++i)
        if (!is_space((unsigned char)label[i])) { r->labels.push_back(label[i]); ++n; }
    r->label_len.push_back(n);
}

// deleteSpacesInSeq on the sequence collected since `start`.
void trim_tail(crispy_raw* r, int64_t start) {
    const size_t n = r->bases.size() - (size_t)start;
    r->bases.resize((size_t)start + seq_trimmed(r->bases.data() + start, n));
}

int parse_fasta(PieceReader& in, crispy_raw* r) {
    Piece pc{};
    if (!in.next(pc) || pc.n == 0 || pc.p[0] != '>') return CRISPY_E_INPUT;
    const char* label = pc.p;
    size_t label_n = space_trimmed(pc.p, pc.n);
    int64_t start = (int64_t)r->bases.size();   // first byte of the pending sequence
    int32_t idx = 0;
    bool ended = false;
    while (!in.eof) {
        if (!in.next(pc)) pc = Piece{"$", 1, '$'};
        const size_t k = space_trimmed(pc.p, pc.n);
        const char c0 = pc.n ? pc.p[0] : '\0';
        if (c0 != '>' && c0 != '$') {
            r->bases.append(pc.p, seq_trimmed(pc.p, k));
            continue;
        }
        if ((int64_t)r->bases.size() == start) {   // no sequence collected
            ++idx;
            if (pc.raw0 == '$') { ended = true; break; }
            continue;
        }
        trim_tail(r, start);
        push(r, start, label, label_n, 1);
        ++idx;
        start = (int64_t)r->bases.size();
        if (pc.raw0 == '$') { ended = true; break; }
        label = pc.p;
        label_n = k;
    }
    if (!ended && (int64_t)r->bases.size() != start) {
        trim_tail(r, start);
        push(r, start, label, label_n, 1);
        ++idx;
    }
    r->records = idx;
    return CRISPY_OK;
}

int parse_fastq(PieceReader& in, crispy_raw* r) {
    Piece pc{}, lab{};
    char last0 = 0;
    int32_t idx = 0;
    bool ended = false;
    int64_t seq_start = -1;   // the last record's sequence in bases
    // the reference tests feof() or a '$' first byte after each line; a
    // failed read keeps the previous buffer but always sets the end flag
    auto line = [&](Piece& out, bool reset) -> bool {
        if (reset) last0 = '$';
        if (in.next(out)) last0 = out.raw0;
        else out = Piece{"", 0, last0};
        return !(in.eof || last0 == '$');
    };
    while (!in.eof) {
        if (!line(lab, true)) { ended = true; break; }
        lab.n = space_trimmed(lab.p, lab.n);
        if (!line(pc, false)) { ended = true; break; }
        const size_t k = space_trimmed(pc.p, pc.n);
        seq_start = (int64_t)r->bases.size();
        r->bases.append(pc.p, k);
        push(r, seq_start, lab.p, lab.n, k ? 1 : 0);
        ++idx;
        if (!line(pc, false)) { ended = true; break; }
        if (!line(pc, false)) { ended = true; break; }
    }
    (void)ended;   // every exit of the loop above sets the end flag
    r->records = idx;
    return CRISPY_OK;
}

}  // namespace

namespace crispy {

int32_t raw_records(const crispy_raw* r) { return (int32_t)r->lengths.size(); }

int64_t raw_header_line(const crispy_raw* r, int32_t i) {
    const int64_t ll = r->label_len[i];
    return 2 + (r->fastq ? ll : std::max<int64_t>(0, ll - 1));   // "> " + label(.substr(1))
}

}  // namespace crispy

extern "C" {

int crispy_raw_load(const char* path, int fastq, crispy_raw** out) {
    if (!out || !path) return crispy::fail(nullptr, CRISPY_E_INPUT, "NULL argument");
    *out = nullptr;
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) return crispy::fail(nullptr, CRISPY_E_IO, "cannot open read file %s", path);
    struct stat sb;
    const char* data = nullptr;
    size_t size = 0;
    void* map = MAP_FAILED;
    std::string copy;   // for inputs that cannot be mapped (pipes, special files)
    if (::fstat(fd, &sb) == 0 && S_ISREG(sb.st_mode) && sb.st_size > 0) {
        size = (size_t)sb.st_size;
        map = ::mmap(nullptr, size, PROT_READ, MAP_PRIVATE | MAP_POPULATE, fd, 0);
    }
    if (map != MAP_FAILED) {
        data = static_cast<const char*>(map);
    } else {
        char buf[1 << 16];
        ssize_t got;
        while ((got = ::read(fd, buf, sizeof buf)) > 0) copy.append(buf, (size_t)got);
        if (got < 0) {
            ::close(fd);
            return crispy::fail(nullptr, CRISPY_E_IO, "cannot read %s", path);
        }
        data = copy.data();
        size = copy.size();
    }
    auto* r = new crispy_raw();
    r->fastq = fastq != 0;
    r->bases.reserve(size);
    PieceReader in{data, size};
    in.has_nul = size && std::memchr(data, '\0', size) != nullptr;
    const int rc = fastq ? parse_fastq(in, r) : parse_fasta(in, r);
    if (map != MAP_FAILED) ::munmap(map, size);
    ::close(fd);
    if (rc != CRISPY_OK) {
        delete r;
        return crispy::fail(nullptr, rc, "%s is not in FASTA format", path);
    }
    *out = r;
    return CRISPY_OK;
}

int crispy_raw_view(const crispy_raw* r, const char** seqbuf, const int64_t** offsets,
                    const int32_t** lengths, const uint8_t** freq, int32_t* n,
                    int32_t* records) {
    if (!r) return crispy::fail(nullptr, CRISPY_E_INPUT, "NULL handle");
    if (seqbuf) *seqbuf = r->bases.data();
    if (offsets) *offsets = r->offsets.data();
    if (lengths) *lengths = r->lengths.data();
    if (freq) *freq = r->freq.data();
    if (n) *n = (int32_t)r->lengths.size();
    if (records) *records = r->records;
    return CRISPY_OK;
}

int crispy_raw_label(const crispy_raw* r, int32_t i, const char** label, int32_t* len) {
    if (!r || i < 0 || (size_t)i >= r->label_len.size())
        return crispy::fail(nullptr, CRISPY_E_INPUT, "record index out of range");
    if (label) *label = r->labels.data() + r->label_off[i];
    if (len) *len = r->label_len[i];
    return CRISPY_OK;
}

void crispy_raw_free(crispy_raw* r) { delete r; }

// writeToFile (preprocess.cpp:562-601).  Records are formatted into a
// 4 MB buffer that is written out whenever it fills (one fwrite per
// buffer), so no copy of the whole output is ever held.
int crispy_pre_write(const crispy_raw* r, const int32_t* index, const int32_t* freq,
                     int32_t kept, const char* out_path, int fastq) {
    if (!r || !out_path || kept < 0 || (kept && (!index || !freq)))
        return crispy::fail(nullptr, CRISPY_E_INPUT, "NULL argument");
    const int32_t n = (int32_t)r->lengths.size();
    for (int32_t k = 0; k < kept; ++k)
        if (index[k] < 0 || index[k] >= n)
            return crispy::fail(nullptr, CRISPY_E_INPUT, "record index out of range");
    const std::string fname = std::string(out_path) + ".frq";
    FILE* fout = std::fopen(out_path, "wb");
    FILE* ff = std::fopen(fname.c_str(), "wb");
    if (!fout || !ff) {
        if (fout) std::fclose(fout);
        if (ff) std::fclose(ff);
        return crispy::fail(nullptr, CRISPY_E_IO, "cannot open output files %s / %s", out_path, fname.c_str());
    }
    constexpr size_t kChunk = 4u << 20;
    struct Out {
        FILE* f;
        std::vector<char> buf;
        size_t used = 0;
    };
    Out so{fout, std::vector<char>(kChunk)}, fo{ff, std::vector<char>(kChunk)};
    bool ok = true;
    auto put = [&](Out& o, const char* p, size_t len) {
        if (o.used + len > kChunk) {
            ok = ok && std::fwrite(o.buf.data(), 1, o.used, o.f) == o.used;
            o.used = 0;
            if (len > kChunk) {   // a read longer than the buffer goes out directly
                ok = ok && std::fwrite(p, 1, len, o.f) == len;
                return;
            }
        }
        std::memcpy(o.buf.data() + o.used, p, len);
        o.used += len;
    };
    char num[16];
    for (int32_t k = 0; k < kept && ok; ++k) {
        const int32_t i = index[k];
        const char* lab = r->labels.data() + r->label_off[i];
        size_t ll = (size_t)r->label_len[i];
        if (!fastq && ll > 0) { ++lab; --ll; }   // label.substr(1): drop the '>'
        put(so, "> ", 2);
        put(so, lab, ll);
        put(so, "\n", 1);
        put(so, r->bases.data() + r->offsets[i], (size_t)r->lengths[i]);
        put(so, "\n", 1);
        put(fo, lab, ll);
        // " %d\n"
        char* e = num + sizeof num;
        *--e = '\n';
        int64_t v = freq[k];
        const bool neg = v < 0;
        if (neg) v = -v;
        do { *--e = (char)('0' + v % 10); v /= 10; } while (v);
        if (neg) *--e = '-';
        *--e = ' ';
        put(fo, e, (size_t)(num + sizeof num - e));
    }
    if (ok && so.used) ok = std::fwrite(so.buf.data(), 1, so.used, fout) == so.used;
    if (ok && fo.used) ok = std::fwrite(fo.buf.data(), 1, fo.used, ff) == fo.used;
    ok = (std::fclose(fout) == 0) && ok;
    ok = (std::fclose(ff) == 0) && ok;
    return ok ? CRISPY_OK : crispy::fail(nullptr, CRISPY_E_IO, "short write to %s", out_path);
}

}  // extern "C"
