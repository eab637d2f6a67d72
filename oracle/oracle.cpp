/*
 * oracle.cpp -- CPU restatement of CRiSPy's kmerDist / genDist semantics.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  See oracle.h.  Citations are
 * file:line inside the reference project (src/kmerDist, src/genDist).
 *
 * The code is deliberately plain: it follows the reference's CPU loops
 * (sorted merge per pair; row-by-row DP over every L1 x L2 cell with an
 * in-band test) so that timing it is timing the reference's own algorithm.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

struct oracle_fasta {
    std::string buf;
    std::vector<int64_t> offsets;
    std::vector<int32_t> lengths;
    int32_t max_len = 0;
};

namespace {

// kmerMain.cpp:281-287 / genMain.cpp:167-173: drop trailing whitespace.
void trim_trailing_space(std::string& s) {
    size_t p = s.find_last_not_of(" \n\r\t\v\f\b");
    if (p != std::string::npos) s.resize(p + 1);
}

// kmerMain.cpp:289-295 (keep "ATGCatgc") / genMain.cpp:175-181 (also "nN"):
// drop trailing characters that are not in the keep set.  Interior
// characters are never touched.
void trim_trailing_invalid(std::string& s, const char* keep) {
    size_t p = s.find_last_of(keep);
    if (p != std::string::npos) s.resize(p + 1);
}

// 2-bit symbol code used by both stages: A=0 G=1 T=2 C=3, anything else 0
// (kmerMain.cpp:137-152, genMain.cpp:300-315).
inline int sym2(char c) {
    switch (c) {
        case 'G': return 1;
        case 'T': return 2;
        case 'C': return 3;
        default: return 0;
    }
}

constexpr int kGO = -10, kGE = -1, kMismatch = -4, kMatch = 5;  // genMain.h:32-35
constexpr int kNegInf = -1000000;                                 // genCPU.cpp:350,416
constexpr int64_t kPairsPerWindow = 576LL * 256 * 4;              // genMain.h:24-27
constexpr double kEps = 0.00001;                                  // kmerMain.h:27

// kmerMain.cpp:180 / genCUDA.cu:219: keep iff dist < thr or |dist-thr| < 1e-5
// (float subtraction, comparison in double).
inline bool keep(float d, float thr) {
    return d < thr || (double)std::fabs(d - thr) < kEps;
}

// kmerMain.cpp:117-154: T = L-K+1 rolling 2K-bit codes, then qsort with the
// signed-short comparator of kmerMain.cpp:275-278.
std::vector<uint16_t> tuples_of(const char* s, int len, int K) {
    int T = len - K + 1;
    std::vector<uint16_t> t(T > 0 ? T : 0);
    if (T <= 0) return t;
    uint32_t mask = (K >= 8) ? 0xFFFFu : ((1u << (2 * K)) - 1u);
    uint32_t v = 0;
    for (int p = 0; p < len; ++p) {
        v = ((v << 2) | (uint32_t)sym2(s[p])) & mask;
        if (p >= K - 1) t[p - K + 1] = (uint16_t)v;
    }
    std::sort(t.begin(), t.end(),
              [](uint16_t a, uint16_t b) { return (int16_t)a < (int16_t)b; });
    return t;
}

// kmerCPU.cpp:29-41: merge counting, comparisons as unsigned short.
int merge_count(const std::vector<uint16_t>& a, const std::vector<uint16_t>& b) {
    size_t k = 0, l = 0;
    int m = 0;
    while (k < a.size() && l < b.size()) {
        uint16_t x = a[k], y = b[l];
        m += (x == y);
        k += (x <= y);
        l += (x >= y);
    }
    return m;
}

// kmerCPU.cpp:43: dist = 1 - matches / min(T1, T2), single precision.
inline float kmer_dist(int matches, int t1, int t2) {
    int mn = t1 < t2 ? t1 : t2;
    return 1.0f - (float)matches / (float)mn;
}

}  // namespace

extern "C" {

// kmerMain.cpp:298-397 and genMain.cpp:184-277 (same control flow; only the
// trailing-trim set differs).  Lines are read with a 4096-byte fgets buffer,
// so over-long lines arrive in pieces exactly as in the reference.
int oracle_fasta_read(const char* path, int flavour, oracle_fasta** out) {
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return -1;
    const char* keepset = flavour ? "nNATGCatgc" : "ATGCatgc";
    char buffer[4096];
    if (!std::fgets(buffer, sizeof buffer, f) || buffer[0] != '>') {
        std::fclose(f);
        return -2;
    }
    oracle_fasta* res = new oracle_fasta();
    std::string seq;
    auto push = [&](std::string s) {
        trim_trailing_invalid(s, keepset);
        res->offsets.push_back((int64_t)res->buf.size());
        res->lengths.push_back((int32_t)s.size());
        if ((int32_t)s.size() > res->max_len) res->max_len = (int32_t)s.size();
        res->buf += s;
    };
    bool stopped = false;
    while (!std::feof(f)) {
        buffer[0] = '$';
        (void)!std::fgets(buffer, sizeof buffer, f);
        std::string line(buffer);
        trim_trailing_space(line);
        if (line[0] != '>' && line[0] != '$') {
            trim_trailing_invalid(line, keepset);
            seq += line;
            continue;
        }
        if (seq.empty()) {
            if (buffer[0] == '$') { stopped = true; break; }
            continue;
        }
        push(seq);
        seq.clear();
        if (buffer[0] == '$') { stopped = true; break; }
    }
    if (!stopped && !seq.empty()) push(seq);
    std::fclose(f);
    *out = res;
    return (int)res->lengths.size();
}

void oracle_fasta_get(const oracle_fasta* f, const char** seqbuf,
                      const int64_t** offsets, const int32_t** lengths,
                      int32_t* max_len) {
    *seqbuf = f->buf.data();
    *offsets = f->offsets.data();
    *lengths = f->lengths.data();
    *max_len = f->max_len;
}

void oracle_fasta_free(oracle_fasta* f) { delete f; }

// kmerMain.cpp:43-48 (num = 2) and genMain.cpp:42-47 (num = 1).
float oracle_default_threshold(int n, float user_thr, int num) {
    if (user_thr >= 0.0f && user_thr <= 1.0f) return user_thr;
    double v = (n > 500) ? (double)num / std::log2((double)n)
                         : (double)num / std::log10((double)n);
    return (float)(v < 1.0 ? v : 1.0);
}

// kmerMain.cpp:50-53.
int oracle_array_dim(int n) {
    int a = (int)(4 * std::pow(8.0, std::floor(std::log10((double)n)) - 1));
    return a > 1536 ? 1536 : a;
}

int oracle_kmer_matches(const char* a, int la, const char* b, int lb, int K) {
    return merge_count(tuples_of(a, la, K), tuples_of(b, lb, K));
}

// Output order of the GPU path: stages enumerate the upper triangle
// (diagonal included) of a stageDim x stageDim grid row-major
// (kmerMain.cpp:205-216 inverts exactly this enumeration); inside a stage the
// host scan visits row offset i then column offset j (kmerMain.cpp:175-195)
// and the kernel marks every (row, col) with row >= col or col >= n as
// 1.1, which never passes (kmerKernel.cu:32-50).
int64_t oracle_kmer_all(const char* seqbuf, const int64_t* offsets,
                        const int32_t* lengths, int n, int K, float thr,
                        int array_dim, int nthreads, int32_t* out_pairs,
                        float* out_dists, int64_t cap) {
    if (n <= 0 || array_dim <= 0 || K < 1 || K > 8) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    std::vector<std::vector<uint16_t>> tup(n);
#pragma omp parallel for schedule(dynamic, 64)
    for (int r = 0; r < n; ++r) tup[r] = tuples_of(seqbuf + offsets[r], lengths[r], K);

    const int A = array_dim;
    const int stage_dim = (n + A - 1) / A;
    int64_t total = 0;
    std::vector<std::vector<std::pair<int, float>>> rowbuf(A);
    for (int sx = 0; sx < stage_dim; ++sx) {
        for (int sy = sx; sy < stage_dim; ++sy) {
#pragma omp parallel for schedule(dynamic, 4)
            for (int i = 0; i < A; ++i) {
                rowbuf[i].clear();
                int row = sx * A + i;
                for (int j = 0; j < A; ++j) {
                    int col = sy * A + j;
                    if (!(row < col && col < n)) continue;
                    int m = merge_count(tup[row], tup[col]);
                    float d = kmer_dist(m, (int)tup[row].size(), (int)tup[col].size());
                    if (keep(d, thr)) rowbuf[i].push_back({col, d});
                }
            }
            for (int i = 0; i < A; ++i) {
                for (auto& e : rowbuf[i]) {
                    if (total < cap) {
                        out_pairs[2 * total] = sx * A + i;
                        out_pairs[2 * total + 1] = e.first;
                        if (out_dists) out_dists[total] = e.second;
                    }
                    ++total;
                }
            }
        }
    }
    return total;
}

// Survivors of the rows [row_lo, row_hi) against every later column, in
// (row, col) order: the same per-pair rule as oracle_kmer_all on a slice of
// the triangle, for checking full-size runs on a few rows.
int64_t oracle_kmer_rows(const char* seqbuf, const int64_t* offsets, const int32_t* lengths,
                         int n, int K, float thr, int row_lo, int row_hi, int nthreads,
                         int32_t* out_pairs, float* out_dists, int64_t cap) {
    if (n <= 0 || K < 1 || K > 8 || row_lo < 0 || row_hi > n || row_lo > row_hi) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    std::vector<std::vector<uint16_t>> tup(n);
#pragma omp parallel for schedule(dynamic, 256)
    for (int r = 0; r < n; ++r) tup[r] = tuples_of(seqbuf + offsets[r], lengths[r], K);
    const int rows = row_hi - row_lo;
    std::vector<std::vector<std::pair<int, float>>> rowbuf(rows);
    for (int i = 0; i < rows; ++i) {
        const int row = row_lo + i;
        const int chunks = 64;
        std::vector<std::vector<std::pair<int, float>>> part(chunks);
#pragma omp parallel for schedule(dynamic, 1)
        for (int c = 0; c < chunks; ++c) {
            const int64_t lo = row + 1 + (int64_t)(n - row - 1) * c / chunks;
            const int64_t hi = row + 1 + (int64_t)(n - row - 1) * (c + 1) / chunks;
            for (int64_t col = lo; col < hi; ++col) {
                const int m = merge_count(tup[row], tup[col]);
                const float d = kmer_dist(m, (int)tup[row].size(), (int)tup[col].size());
                if (keep(d, thr)) part[c].push_back({(int)col, d});
            }
        }
        for (auto& v : part) rowbuf[i].insert(rowbuf[i].end(), v.begin(), v.end());
    }
    int64_t total = 0;
    for (int i = 0; i < rows; ++i)
        for (auto& e : rowbuf[i]) {
            if (total < cap) {
                out_pairs[2 * total] = row_lo + i;
                out_pairs[2 * total + 1] = e.first;
                if (out_dists) out_dists[total] = e.second;
            }
            ++total;
        }
    return total;
}

// genCPU.cpp:290-466 (banded) and :81-225 (band <= 1: no band limit, which
// is the banded recurrence with every cell in band).  Rows i run over read2
// (pair[1]) and columns j over read1 (pair[0]); symbols are compared as the
// GPU path's 2-bit codes (genKernel.cu:437-447).
float oracle_gen_pair(const char* r1, int l1, const char* r2, int l2, int band,
                      int32_t* score, int32_t* ml_out, int32_t* al_out) {
    const int kband = (band <= 1) ? std::max(l1, l2) : (l1 + l2) / (band * 2);
    auto inside = [kband](int i, int j) { return i - j >= -kband && i - j <= kband; };
    std::vector<int> M[2], ML[2], AL[2];
    std::vector<signed char> ULD[2];
    for (int b = 0; b < 2; ++b) {
        M[b].assign(l1 + 1, 0); ML[b].assign(l1 + 1, 0); AL[b].assign(l1 + 1, 0);
        ULD[b].assign(l1 + 1, 0);
    }
    int cur = 0, pre = 1;
    for (int j = 1; j <= std::min(kband, l1); ++j) AL[cur][j] = j;  // genCPU.cpp:373-379
    int max_last_col = kNegInf, max_last_row = kNegInf;
    int ml_col = 0, al_col = 0, ml_row = 0, al_row = 0;
    for (int i = 1; i <= l2; ++i) {
        std::swap(cur, pre);
        if (i <= kband) {  // genCPU.cpp:390-396
            M[cur][0] = 0; ULD[cur][0] = 0; ML[cur][0] = 0; AL[cur][0] = i;
        }
        const int c2 = sym2(r2[i - 1]);
        for (int j = 1; j <= l1; ++j) {
            if (!inside(i, j)) { M[cur][j] = 0; continue; }
            const int hit = (c2 == sym2(r1[j - 1]));
            const int aligned = hit ? kMatch : kMismatch;
            int up = kNegInf, left = kNegInf;
            if (inside(i, j - 1)) {
                int u = ULD[cur][j - 1];
                up = M[cur][j - 1] + (u & 1) * kGO + ((u >> 2) & 1) * kGE;
            }
            if (inside(i - 1, j)) {
                int u = ULD[pre][j];
                left = M[pre][j] + (u & 1) * kGO + ((u >> 1) & 1) * kGE;
            }
            const int diag = M[pre][j - 1] + aligned;
            const int m = std::max(std::max(diag, up), left);
            M[cur][j] = m;
            if (m == diag) {  // tie-break order diag > up > left (genCPU.cpp:426-440)
                ULD[cur][j] = 1;
                ML[cur][j] = (ML[pre][j - 1] - hit) + 1;
                AL[cur][j] = AL[pre][j - 1] + 1;
            } else if (m == up) {
                ULD[cur][j] = 4;
                ML[cur][j] = ML[cur][j - 1] + 1;
                AL[cur][j] = AL[cur][j - 1] + 1;
            } else {
                ULD[cur][j] = 2;
                ML[cur][j] = ML[pre][j] + 1;
                AL[cur][j] = AL[pre][j] + 1;
            }
            if (i == l2 && m >= max_last_col) {  // last maximum wins
                max_last_col = m; ml_col = ML[cur][j]; al_col = AL[cur][j];
            }
            if (j == l1 && m >= max_last_row) {
                max_last_row = m; ml_row = ML[cur][j]; al_row = AL[cur][j];
            }
        }
    }
    const bool use_col = max_last_col > max_last_row;  // genCPU.cpp:461-464
    const int ml = use_col ? ml_col : ml_row;
    const int al = use_col ? al_col : al_row;
    if (score) *score = use_col ? max_last_col : max_last_row;
    if (ml_out) *ml_out = ml;
    if (al_out) *al_out = al;
    return (float)ml / (float)al;
}

void oracle_gen_all(const char* seqbuf, const int64_t* offsets,
                    const int32_t* lengths, int n, const int32_t* pairs,
                    int64_t npairs, int band, int nthreads, float* out_dist,
                    int32_t* out_score, int32_t* out_ml, int32_t* out_al) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    (void)n;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t p = 0; p < npairs; ++p) {
        const int a = pairs[2 * p], b = pairs[2 * p + 1];
        int32_t s, ml, al;
        float d = oracle_gen_pair(seqbuf + offsets[a], lengths[a], seqbuf + offsets[b],
                                  lengths[b], band, &s, &ml, &al);
        out_dist[p] = d;
        if (out_score) out_score[p] = s;
        if (out_ml) out_ml[p] = ml;
        if (out_al) out_al[p] = al;
    }
}

int64_t oracle_band_cells(int l1, int l2, int band) {
    const int kband = (band <= 1) ? std::max(l1, l2) : (l1 + l2) / (band * 2);
    int64_t cells = 0;
    for (int i = 1; i <= l2; ++i) {
        int lo = std::max(1, i - kband), hi = std::min(l1, i + kband);
        if (hi >= lo) cells += hi - lo + 1;
    }
    return cells;
}

// genCUDA.cu:150-254 with the chunk writer of :17-81.
int oracle_gen_chunks(const int32_t* pairs, const float* dists, int64_t npairs,
                      float thr, uint32_t* out_pairs, float* out_dists,
                      int64_t* chunk_sizes, int max_chunks) {
    int nchunks = 0;
    int64_t written = 0;
    std::vector<int64_t> pending;
    auto flush = [&]() {
        std::vector<int64_t> idx(pending);
        std::stable_sort(idx.begin(), idx.end(),
                         [&](int64_t x, int64_t y) { return dists[x] < dists[y]; });
        for (int64_t q : idx) {
            out_pairs[2 * written] = (uint32_t)pairs[2 * q];
            out_pairs[2 * written + 1] = (uint32_t)pairs[2 * q + 1];
            out_dists[written] = dists[q];
            ++written;
        }
        if (nchunks < max_chunks) chunk_sizes[nchunks] = (int64_t)pending.size();
        ++nchunks;
        pending.clear();
    };
    for (int64_t w = 0; w < npairs || (w == 0 && npairs == 0); w += kPairsPerWindow) {
        int64_t end = std::min(npairs, w + kPairsPerWindow);
        for (int64_t p = w; p < end; ++p)
            if (keep(dists[p], thr)) pending.push_back(p);
        if ((int64_t)pending.size() >= kPairsPerWindow) flush();
        if (npairs == 0) break;
    }
    if (!pending.empty()) flush();
    return nchunks;
}

}  // extern "C"
