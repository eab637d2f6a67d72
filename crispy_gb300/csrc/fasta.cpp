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
// The scan itself (parallel chunks cut at header lines, then the loop over
// their tokens) is shared with preprocess's reader (pre_io.cpp).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

struct crispy_reads {
    crispy::FastaBuffer buf;   // each read at its chunk's offset
    std::vector<int64_t> offsets;
    std::vector<int32_t> lengths;
    int32_t max_len = 0;
};

extern "C" {

int crispy_reads_load_fasta(const char* path, int flavour, crispy_reads** out) {
    if (!out || !path) return crispy::fail(nullptr, CRISPY_E_INPUT, "NULL argument");
    *out = nullptr;
    auto* r = new crispy_reads();
    const int rc = crispy::scan_stage_fasta(path, flavour, r->buf, r->offsets, r->lengths);
    if (rc != CRISPY_OK) {
        delete r;
        return rc;
    }
    for (int32_t l : r->lengths) r->max_len = std::max(r->max_len, l);
    *out = r;
    return CRISPY_OK;
}

int crispy_reads_view(const crispy_reads* r, const char** seqbuf, const int64_t** offsets,
                      const int32_t** lengths, int32_t* n, int32_t* max_len) {
    if (!r) return CRISPY_E_INPUT;
    if (seqbuf) *seqbuf = r->buf.p;
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
