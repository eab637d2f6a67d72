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
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace crispy {

// An anonymous mapping that asks for transparent huge pages: the parse
// threads then take one fault per 2 MB instead of one per 4 KB.
FastaBuffer::~FastaBuffer() {
    if (p) ::munmap(p, n);
}
bool FastaBuffer::alloc(size_t bytes) {
    n = (bytes + (2u << 20) - 1) & ~(size_t)((2u << 20) - 1);
    void* m = ::mmap(nullptr, n, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (m == MAP_FAILED) {
        p = nullptr;
        n = 0;
        return false;
    }
    p = static_cast<char*>(m);
#ifdef MADV_HUGEPAGE
    ::madvise(p, n, MADV_HUGEPAGE);
#endif
    return true;
}

}  // namespace crispy

struct crispy_raw {
    bool fastq = false;
    std::string bases;                // FASTQ: sequences back to back
    crispy::FastaBuffer fa_bases;     // FASTA: sequences at their chunk's file offsets
    const char* data() const { return fa_bases.p ? fa_bases.p : bases.data(); }
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
// The letters a sequence piece is cut back to: deleteSpacesInSeq's
// "nNATGCatgc" (preprocess.cpp:65-71, genMain.cpp:175-181) or kmerDist's
// "ATGCatgc" (kmerMain.cpp:289-295).
struct KeepSet {
    bool in[256] = {};
    explicit KeepSet(const char* letters) {
        for (const char* c = letters; *c; ++c) in[(unsigned char)*c] = true;
    }
};
const KeepSet kPreKeep("nNATGCatgc");
bool is_space(unsigned char c) {   // isspace in the "C" locale
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// Length after deleteSpaces: trailing whitespace goes unless nothing else is left.
size_t space_trimmed(const char* p, size_t n) {
    size_t k = n;
    while (k > 0 && trim_space_char((unsigned char)p[k - 1])) --k;
    return k ? k : n;
}
// Length after deleteSpacesInSeq: cut after the last kept letter, if any.
size_t seq_trimmed(const char* p, size_t n, const KeepSet& keep) {
    size_t k = n;
    while (k > 0 && !keep.in[(unsigned char)p[k - 1]]) --k;
    return k ? k : n;
}

// READ::initialize drops every whitespace byte of the label.
void push_label(crispy_raw* r, const char* label, size_t label_n) {
    r->label_off.push_back((int64_t)r->labels.size());
    int32_t n = 0;
    for (size_t i = 0; i < label_n; ++i)
        if (!is_space((unsigned char)label[i])) { r->labels.push_back(label[i]); ++n; }
    r->label_len.push_back(n);
}

// A piece as a pointer into the file and its length up to the first NUL.
struct Piece {
    const char* p;
    size_t n;
    char raw0;   // first byte of the fgets buffer ('$' at end of file)
};

// fgets over an in-memory file.  `size` is where reading stops: the file's
// end (end-of-file rules apply) or, for a chunk, the start of its
// successor's first line (no end-of-file rules: stop_at_size).
struct PieceReader {
    const char* data;
    size_t size, pos = 0;
    bool eof = false;
    bool stop_at_size = false;
    bool has_nul = true;   // false: the file holds no NUL byte, skip the per-piece scan
    // false at end of file (the reference's buffer then starts with '$')
    bool next(Piece& pc) {
        if (pos >= size) {
            eof = true;
            return false;
        }
        if (stop_at_size) {   // a chunk's last line ends with '\n' right at size
            const size_t room = std::min(kPieceMax, size - pos);
            const char* p = data + pos;
            const void* nl = std::memchr(p, '\n', room);
            const size_t take = nl ? (size_t)((const char*)nl - p) + 1 : room;
            pos += take;
            const void* z = has_nul ? std::memchr(p, '\0', take) : nullptr;
            pc.p = p;
            pc.n = z ? (size_t)((const char*)z - p) : take;
            pc.raw0 = p[0];
            return true;
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
    push_label(r, label, label_n);
}

// ---- FASTA: chunks of the file tokenised in parallel, then readFile's
// state machine over the tokens in order ----
//
// Chunks start at a line that begins with '>' (a byte after '\n'), so they
// cut the file into the same fgets pieces as one sequential pass.  A chunk
// turns its pieces into tokens:
//   HEADER  a piece starting with '>' (label = the piece, trailing
//           whitespace trimmed);
//   SEQRUN  the sequence pieces between two other tokens, each trimmed and
//           copied back to back into the sequence buffer at the chunk's own
//           file offset (trimmed bytes never outrun the raw ones);
//   DOLLAR  a piece starting with '$', or the failed read at end of file
//           (the reference's buffer then starts with '$').
// The state machine then decides records and labels exactly as readFile
// does: a record is emitted at the next HEADER / DOLLAR when its sequence is
// not empty, a HEADER without sequence only counts, and DOLLAR ends input.
struct Tok {
    uint8_t kind;   // 0 HEADER, 1 SEQRUN, 2 DOLLAR
    int64_t a, b;   // HEADER: file offset, length; SEQRUN: buffer offset, length
};

void tokenise(const char* data, size_t begin, size_t end, bool last, const KeepSet* keep, char* out,
              std::vector<Tok>& toks) {
    PieceReader in{data, end, begin};
    in.has_nul = std::memchr(data + begin, '\0', end - begin) != nullptr;   // this chunk's pieces only
    in.stop_at_size = !last;
    Piece pc{};
    int64_t w = (int64_t)begin, run = -1;
    auto close_run = [&]() {
        if (run >= 0) toks.push_back(Tok{1, run, w - run});
        run = -1;
    };
    while (!in.eof) {
        if (!in.next(pc)) {
            if (last) {   // end of file: the '$' marker
                close_run();
                toks.push_back(Tok{2, 0, 0});
            }
            break;
        }
        const size_t k = space_trimmed(pc.p, pc.n);
        const char c0 = pc.n ? pc.p[0] : '\0';
        if (c0 != '>' && c0 != '$') {
            const size_t k2 = seq_trimmed(pc.p, k, *keep);
            if (run < 0) run = w;
            std::memcpy(out + w, pc.p, k2);
            w += (int64_t)k2;
            continue;
        }
        close_run();
        if (c0 == '>') toks.push_back(Tok{0, (int64_t)(pc.p - data), (int64_t)k});
        else toks.push_back(Tok{2, 0, 0});
    }
    close_run();
    // the rest of the chunk's region is never read as sequence; writing it
    // here keeps every page of the buffer resident before it is uploaded
    std::memset(out + w, 0, end - (size_t)w);
}

// The FASTA records of data[0, size): sequences into buf (at their chunk's
// offsets), their offsets and lengths; with labels != NULL also the label
// of each record (whitespace removed); *records = readIndex.
int scan_fasta(const char* data, size_t size, const KeepSet& keep, crispy::FastaBuffer& buf,
               std::vector<int64_t>& offsets, std::vector<int32_t>& lengths, crispy_raw* labels,
               int32_t* records) {
    if (size == 0 || data[0] != '>') return CRISPY_E_INPUT;
    // chunk boundaries: the first line start at or after each even cut that
    // begins with '>'; one chunk per MB, at most one per hardware thread and
    // 16 (the CRISPY_PARSE_CHUNKS environment variable sets the number:
    // tests use it to cut small files)
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int want = (int)std::max<size_t>(1, std::min<size_t>(std::min(16u, hw), size >> 20));
    if (const char* e = std::getenv("CRISPY_PARSE_CHUNKS")) want = std::max(1, std::min(256, std::atoi(e)));
    std::vector<size_t> cut{0};
    for (int t = 1; t < want; ++t) {
        size_t p = std::max(cut.back() + 1, size * (size_t)t / (size_t)want);
        while (p < size && !(data[p - 1] == '\n' && data[p] == '>')) {
            const void* nl = std::memchr(data + p, '\n', size - p);   // the next line start, past p
            p = nl ? (size_t)((const char*)nl - data) + 1 : size;
        }
        if (p >= size) break;
        cut.push_back(p);
    }
    cut.push_back(size);
    const int chunks = (int)cut.size() - 1;
    if (!buf.alloc(size + 16)) return CRISPY_E_OOM;
    std::vector<std::vector<Tok>> toks((size_t)chunks);
    if (chunks == 1) {
        tokenise(data, 0, size, true, &keep, buf.p, toks[0]);
    } else {
        std::vector<std::thread> th;
        for (int c = 0; c < chunks; ++c)
            th.emplace_back(tokenise, data, cut[c], cut[c + 1], c + 1 == chunks, &keep, buf.p, std::ref(toks[c]));
        for (auto& t : th) t.join();
    }
    // readFile's loop over the tokens (preprocess.cpp:100-166, 230-236; the
    // stages' readFile, kmerMain.cpp:298-397, runs the same loop)
    const Tok* label = nullptr;
    int64_t pend = -1, plen = 0;   // the pending sequence (buffer offset, length)
    int32_t idx = 0;
    bool ended = false, first = true;
    auto emit = [&]() {
        const int64_t n = (int64_t)seq_trimmed(buf.p + pend, (size_t)plen, keep);   // deleteSpacesInSeq(seq)
        offsets.push_back(pend);
        lengths.push_back((int32_t)n);
        if (labels) push_label(labels, data + label->a, (size_t)label->b);
        ++idx;
        pend = -1;
        plen = 0;
    };
    for (int c = 0; c < chunks && !ended; ++c) {
        for (const Tok& t : toks[c]) {
            if (first) {   // the first line must be a header (preprocess.cpp:107-118)
                if (t.kind != 0) return CRISPY_E_INPUT;
                label = &t;
                first = false;
                continue;
            }
            if (t.kind == 1) {
                if (pend < 0) pend = t.a;
                plen += t.b;
                continue;
            }
            if (plen == 0) {
                ++idx;
                pend = -1;
                if (t.kind == 2) { ended = true; break; }
                continue;
            }
            emit();
            if (t.kind == 2) { ended = true; break; }
            label = &t;
        }
    }
    if (first) return CRISPY_E_INPUT;
    if (!ended && plen > 0) emit();
    *records = idx;
    return CRISPY_OK;
}

int parse_fasta(const char* data, size_t size, crispy_raw* r) {
    const int rc = scan_fasta(data, size, kPreKeep, r->fa_bases, r->offsets, r->lengths, r, &r->records);
    r->freq.assign(r->offsets.size(), 1);
    return rc;
}

// The file mapped read-only (or read, where it cannot be mapped).
struct MappedFile {
    const char* data = nullptr;
    size_t size = 0;
    void* map = MAP_FAILED;
    int fd = -1;
    std::string copy;
    int open(const char* path) {
        fd = ::open(path, O_RDONLY);
        if (fd < 0) return CRISPY_E_IO;
        struct stat sb;
        if (::fstat(fd, &sb) == 0 && S_ISREG(sb.st_mode) && sb.st_size > 0) {
            size = (size_t)sb.st_size;
            map = ::mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);   // chunk threads fault their pages in
        }
        if (map != MAP_FAILED) {
            data = static_cast<const char*>(map);
            return CRISPY_OK;
        }
        char b[1 << 16];
        ssize_t got;
        while ((got = ::read(fd, b, sizeof b)) > 0) copy.append(b, (size_t)got);
        if (got < 0) return CRISPY_E_IO;
        data = copy.data();
        size = copy.size();
        return CRISPY_OK;
    }
    ~MappedFile() {
        if (map != MAP_FAILED) ::munmap(map, size);
        if (fd >= 0) ::close(fd);
    }
};

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

int scan_stage_fasta(const char* path, int flavour, FastaBuffer& buf, std::vector<int64_t>& offsets,
                     std::vector<int32_t>& lengths) {
    static const KeepSet kmer_keep("ATGCatgc"), gen_keep("nNATGCatgc");
    MappedFile f;
    if (f.open(path) != CRISPY_OK) return fail(nullptr, CRISPY_E_IO, "cannot open read file %s", path);
    int32_t records = 0;
    const int rc = scan_fasta(f.data, f.size, flavour ? gen_keep : kmer_keep, buf, offsets, lengths, nullptr,
                              &records);
    if (rc == CRISPY_E_INPUT) return fail(nullptr, rc, "%s is not in FASTA format", path);
    if (rc != CRISPY_OK) return fail(nullptr, rc, "cannot allocate the reads of %s", path);
    return CRISPY_OK;
}

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
    MappedFile f;
    if (f.open(path) != CRISPY_OK) return crispy::fail(nullptr, CRISPY_E_IO, "cannot open read file %s", path);
    auto* r = new crispy_raw();
    r->fastq = fastq != 0;
    int rc;
    if (fastq) {
        r->bases.reserve(f.size);
        PieceReader in{f.data, f.size};
        in.has_nul = f.size && std::memchr(f.data, '\0', f.size) != nullptr;
        rc = parse_fastq(in, r);
    } else {
        rc = parse_fasta(f.data, f.size, r);
    }
    if (rc != CRISPY_OK) {
        delete r;
        return rc == CRISPY_E_INPUT ? crispy::fail(nullptr, rc, "%s is not in FASTA format", path)
                                    : crispy::fail(nullptr, rc, "cannot allocate the records of %s", path);
    }
    *out = r;
    return CRISPY_OK;
}

int crispy_raw_view(const crispy_raw* r, const char** seqbuf, const int64_t** offsets,
                    const int32_t** lengths, const uint8_t** freq, int32_t* n,
                    int32_t* records) {
    if (!r) return crispy::fail(nullptr, CRISPY_E_INPUT, "NULL handle");
    if (seqbuf) *seqbuf = r->data();
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

// writeToFile (preprocess.cpp:562-601).  Every record's place in the two
// files is known from the lengths, so the records are formatted into two
// buffers by up to 16 threads over contiguous ranges of kept reads (the
// reads are gathered from scattered places of the record buffer), and each
// file is written with one fwrite.
int crispy_pre_write(const crispy_raw* r, const int32_t* index, const int32_t* freq,
                     int32_t kept, const char* out_path, int fastq) {
    if (!r || !out_path || kept < 0 || (kept && (!index || !freq)))
        return crispy::fail(nullptr, CRISPY_E_INPUT, "NULL argument");
    const int32_t n = (int32_t)r->lengths.size();
    for (int32_t k = 0; k < kept; ++k)
        if (index[k] < 0 || index[k] >= n)
            return crispy::fail(nullptr, CRISPY_E_INPUT, "record index out of range");
    auto label_of = [&](int32_t i, size_t* len) -> const char* {
        const char* lab = r->labels.data() + r->label_off[i];
        size_t ll = (size_t)r->label_len[i];
        if (!fastq && ll > 0) { ++lab; --ll; }   // label.substr(1): drop the '>'
        *len = ll;
        return lab;
    };
    auto digits = [](int64_t v) -> size_t {
        size_t d = v < 0 ? 2 : 1;
        for (v = v < 0 ? -v : v; v >= 10; v /= 10) ++d;
        return d;
    };
    std::vector<size_t> so((size_t)kept + 1, 0), fo((size_t)kept + 1, 0);
    for (int32_t k = 0; k < kept; ++k) {
        size_t ll;
        label_of(index[k], &ll);
        so[k + 1] = so[k] + 2 + ll + 1 + (size_t)r->lengths[index[k]] + 1;   // "> %s\n%s\n"
        fo[k + 1] = fo[k] + ll + 1 + digits(freq[k]) + 1;                    // "%s %d\n"
    }
    std::unique_ptr<char[]> sbuf(new char[so[kept] + 1]), fbuf(new char[fo[kept] + 1]);
    const char* bases = r->data();
    auto fill = [&](int32_t k0, int32_t k1) {
        for (int32_t k = k0; k < k1; ++k) {
            const int32_t i = index[k];
            size_t ll;
            const char* lab = label_of(i, &ll);
            char* o = sbuf.get() + so[k];
            *o++ = '>';
            *o++ = ' ';
            std::memcpy(o, lab, ll);
            o += ll;
            *o++ = '\n';
            std::memcpy(o, bases + r->offsets[i], (size_t)r->lengths[i]);
            o += r->lengths[i];
            *o = '\n';
            char* q = fbuf.get() + fo[k];
            std::memcpy(q, lab, ll);
            q += ll;
            *q++ = ' ';
            const size_t d = digits(freq[k]);
            int64_t v = freq[k];
            if (v < 0) { q[0] = '-'; v = -v; }
            for (size_t j = d; j > (freq[k] < 0 ? 1u : 0u); --j) { q[j - 1] = (char)('0' + v % 10); v /= 10; }
            q[d] = '\n';
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(16u, hw), (int64_t)kept / 4096));
    if (nt == 1) {
        fill(0, kept);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back(fill, (int32_t)((int64_t)kept * t / nt), (int32_t)((int64_t)kept * (t + 1) / nt));
        for (auto& x : th) x.join();
    }
    const std::string fname = std::string(out_path) + ".frq";
    FILE* fout = std::fopen(out_path, "wb");
    FILE* ff = std::fopen(fname.c_str(), "wb");
    if (!fout || !ff) {
        if (fout) std::fclose(fout);
        if (ff) std::fclose(ff);
        return crispy::fail(nullptr, CRISPY_E_IO, "cannot open output files %s / %s", out_path, fname.c_str());
    }
    bool ok = std::fwrite(sbuf.get(), 1, so[kept], fout) == so[kept];
    ok = std::fwrite(fbuf.get(), 1, fo[kept], ff) == fo[kept] && ok;
    ok = (std::fclose(fout) == 0) && ok;
    ok = (std::fclose(ff) == 0) && ok;
    return ok ? CRISPY_OK : crispy::fail(nullptr, CRISPY_E_IO, "short write to %s", out_path);
}

}  // extern "C"
