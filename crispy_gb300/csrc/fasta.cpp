// fasta.cpp -- host-side input handling shared by both stages.
//
// FASTA semantics follow readFile of the reference (kmerMain.cpp:298-397,
// genMain.cpp:184-277), which both stages implement with the same control
// flow: 4096-byte fgets pieces, trailing whitespace trimmed per piece,
// header pieces start with '>', sequence pieces lose their trailing
// characters outside a keep set ("ATGCatgc" for kmerDist, "nNATGCatgc" for
// genDist) and are concatenated; a read is emitted when the next header (or
// end of file) arrives and the collected sequence is non-empty.  Quirks kept
// on purpose so that read IDs and lengths match the reference exactly:
//   * an empty line inside a record contributes its '\n' to the sequence
//     (it only has whitespace, and whitespace-only pieces are not trimmed);
//   * a piece whose first byte is '$' is taken as end of input.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

struct crispy_reads {
    std::string bases;
    std::vector<int64_t> offsets;
    std::vector<int32_t> lengths;
    int32_t max_len = 0;
};

namespace {

constexpr size_t kPiece = 4096;  // kmerMain.h:24 / genMain.h:22 BUF_SIZE

const char* kSpace = " \n\r\t\v\f\b";

void rstrip_set_complement(std::string& s, const char* keep) {
    size_t last = s.find_last_of(keep);
    if (last != std::string::npos) s.erase(last + 1);
}

void rstrip_space(std::string& s) {
    size_t last = s.find_last_not_of(kSpace);
    if (last != std::string::npos) s.erase(last + 1);
}

}  // namespace

extern "C" {

int crispy_reads_load_fasta(const char* path, int flavour, crispy_reads** out) {
    if (!out || !path) return crispy::fail(nullptr, CRISPY_E_INPUT, "NULL argument");
    *out = nullptr;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return crispy::fail(nullptr, CRISPY_E_IO, "cannot open read file %s", path);
    const char* keep = flavour ? "nNATGCatgc" : "ATGCatgc";
    char piece[kPiece];
    if (!std::fgets(piece, kPiece, fp) || piece[0] != '>') {
        std::fclose(fp);
        return crispy::fail(nullptr, CRISPY_E_INPUT, "%s is not in FASTA format", path);
    }
    auto* r = new crispy_reads();
    std::string pending;
    auto emit = [&]() {
        rstrip_set_complement(pending, keep);
        r->offsets.push_back((int64_t)r->bases.size());
        r->lengths.push_back((int32_t)pending.size());
        r->max_len = std::max<int32_t>(r->max_len, (int32_t)pending.size());
        r->bases.append(pending);
        pending.clear();
    };
    enum { kMore, kEnd } state = kMore;
    while (state == kMore && !std::feof(fp)) {
        piece[0] = '$';  // stays '$' when fgets reaches end of file
        if (!std::fgets(piece, kPiece, fp)) { /* piece keeps the '$' marker */ }
        std::string s(piece);
        rstrip_space(s);
        const bool header_or_end = (s[0] == '>' || s[0] == '$');
        if (!header_or_end) {
            rstrip_set_complement(s, keep);
            pending += s;
        } else if (!pending.empty()) {
            emit();
            if (piece[0] == '$') state = kEnd;
        } else if (piece[0] == '$') {
            state = kEnd;
        }
    }
    if (state == kMore && !pending.empty()) emit();
    std::fclose(fp);
    *out = r;
    return CRISPY_OK;
}

int crispy_reads_view(const crispy_reads* r, const char** seqbuf, const int64_t** offsets,
                      const int32_t** lengths, int32_t* n, int32_t* max_len) {
    if (!r) return CRISPY_E_INPUT;
    if (seqbuf) *seqbuf = r->bases.data();
    if (offsets) *offsets = r->offsets.data();
    if (lengths) *lengths = r->lengths.data();
    if (n) *n = (int32_t)r->lengths.size();
    if (max_len) *max_len = r->max_len;
    return CRISPY_OK;
}

void crispy_reads_free(crispy_reads* r) { delete r; }

// kmerMain.cpp:43-48 (stage 0: 2 / log n) and genMain.cpp:42-47 (stage 1:
// 1 / log n): log2 above 500 reads, log10 otherwise, capped at 1, computed in
// double and narrowed to float.  A user value inside [0, 1] is kept.
float crispy_default_threshold(int n, float user_thr, int stage) {
    if (user_thr >= 0.0f && user_thr <= 1.0f) return user_thr;
    const double num = stage == 0 ? 2.0 : 1.0;
    const double v = n > 500 ? num / std::log2((double)n) : num / std::log10((double)n);
    return (float)(v < 1.0 ? v : 1.0);
}

// kmerMain.cpp:50-53.
int crispy_array_dim(int n) {
    if (n <= 0) return 0;
    int a = (int)(4 * std::pow(8.0, std::floor(std::log10((double)n)) - 1));
    return a > 1536 ? 1536 : a;
}

}  // extern "C"
