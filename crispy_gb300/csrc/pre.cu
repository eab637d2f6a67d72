// pre.cu -- preprocess on GB300: read filters and duplicate merge.
//
// The reference (preprocess.cpp) keeps its reads in a std::list and, after
// the optional filters, sorts the whole list by (length, strcmp) with the
// list's stable merge sort and folds each run of equal sequences into its
// last read (mergeReads, :244-280).  Here the records go to the device once
// and everything after the host-side length statistics runs there:
//   1. pre_pad_kernel copies every read to a 16-byte aligned slot (zero
//      padded), so byte-wise comparisons become 128-bit loads;
//   2. pre_filter_kernel applies the length cut and the N/n check of
//      processReadLength (:322-392);
//   3. pre_primer_kernel runs SWLocalAlignment (:394-527) of the primer
//      against each read's first 2 x primer-length bytes, one thread per
//      read with its DP rows in shared memory;
//   4. the surviving read indices are sorted by (length, bytes, record
//      index): 2048-index tiles by a bitonic network in shared memory, then
//      merge passes in which each index finds its place in the partner run
//      by binary search.  The record index as last key makes every key
//      distinct, so the order equals the reference's stable sort;
//   5. pre_last_kernel flags the last read of each run of equal sequences;
//      compaction of those flags gives the kept reads and, from the gaps
//      between them, each run's size (the merged frequency: every read that
//      reaches the merge has frequency 1).
// Comparisons read the reads from L2: the padded copy of 100,000 reads of
// 300-500 bases is about 42 MB.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace crispy {
namespace {

constexpr uint32_t kNone = 0xffffffffu;   // tile padding: sorts after every read
constexpr int kTile = 2048;               // indices per bitonic tile
constexpr int kTileThreads = kTile / 2;
constexpr int kMaxPrimer = 256;           // primer bases the shared-memory DP rows allow

struct ReadSet {
    const uint4* pad;      // reads, each at a 16-byte aligned slot, zero padded
    const int64_t* woff;   // first 16-byte word of each read
    const int32_t* len;
};

__device__ __forceinline__ uint32_t be32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// strcmp-style order of two reads of equal length L (unsigned bytes).
__device__ __forceinline__ int cmp_bytes(const ReadSet& r, uint32_t a, uint32_t b, int L) {
    const uint4* pa = r.pad + r.woff[a];
    const uint4* pb = r.pad + r.woff[b];
    const int nw = (L + 15) >> 4;
    for (int w = 0; w < nw; ++w) {
        const uint4 x = __ldg(pa + w), y = __ldg(pb + w);
        if (x.x != y.x) return be32(x.x) < be32(y.x) ? -1 : 1;
        if (x.y != y.y) return be32(x.y) < be32(y.y) ? -1 : 1;
        if (x.z != y.z) return be32(x.z) < be32(y.z) ? -1 : 1;
        if (x.w != y.w) return be32(x.w) < be32(y.w) ? -1 : 1;
    }
    return 0;
}

// READ::operator< (preprocess.cpp:42-49) with the record index as last key.
__device__ __forceinline__ bool read_less(const ReadSet& r, uint32_t a, uint32_t b) {
    if (b == kNone) return a != kNone;
    if (a == kNone) return false;
    const int la = __ldg(r.len + a), lb = __ldg(r.len + b);
    if (la != lb) return la < lb;
    const int c = cmp_bytes(r, a, b, la);
    return c ? c < 0 : a < b;
}

__global__ void pre_pad_kernel(const uint8_t* __restrict__ seq, const int64_t* __restrict__ off,
                               const int32_t* __restrict__ len, const int64_t* __restrict__ woff,
                               int n, uint4* __restrict__ pad) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < n; r += nwarps) {
        const uint8_t* src = seq + off[r];
        const int L = len[r];
        uint4* dst = pad + woff[r];
        for (int w = lane; w < (L + 15) >> 4; w += 32) {
            uint32_t v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t word = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int p = 16 * w + 4 * q + b;
                    word |= (uint32_t)(p < L ? src[p] : 0u) << (8 * b);
                }
                v[q] = word;
            }
            dst[w] = make_uint4(v[0], v[1], v[2], v[3]);
        }
    }
}

// alive = frequency != 0, then (with the length check) the length cut and
// the N/n test of processReadLength.  counters[0]: reads cut by length,
// counters[1]: reads dropped for N/n.
__global__ void pre_filter_kernel(ReadSet r, const uint8_t* __restrict__ freq, int n, int length_check,
                                  unsigned long long lo, unsigned long long hi,
                                  uint8_t* __restrict__ alive, unsigned int* __restrict__ counters) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < n; i += nwarps) {
        bool a = freq[i] != 0;
        if (a && length_check) {
            const int L = r.len[i];
            const unsigned long long ul = (unsigned long long)L;
            if (ul < lo || ul > hi) {
                a = false;
                if (lane == 0) atomicAdd(&counters[0], 1u);
            } else {
                const uint4* p = r.pad + r.woff[i];
                bool hit = false;
                for (int w = lane; w < (L + 15) >> 4 && !hit; w += 32) {
                    const uint4 x = p[w];
                    // a byte is N or n iff (byte | 0x20) == 'n'; padding bytes are 0
                    hit = __vcmpeq4(x.x | 0x20202020u, 0x6e6e6e6eu) | __vcmpeq4(x.y | 0x20202020u, 0x6e6e6e6eu) |
                          __vcmpeq4(x.z | 0x20202020u, 0x6e6e6e6eu) | __vcmpeq4(x.w | 0x20202020u, 0x6e6e6e6eu);
                }
                if (__any_sync(0xffffffffu, hit)) {
                    a = false;
                    if (lane == 0) atomicAdd(&counters[1], 1u);
                }
            }
        }
        if (lane == 0) alive[i] = a ? 1 : 0;
    }
}

// SWLocalAlignment (preprocess.cpp:394-527) of the primer A (m bases)
// against B = the first min(2m, L) bytes of each alive read, and the
// decision of processPrimer (:530-560): the read goes when the best local
// alignment's start equals its end.  Scores: match +4, mismatch -1, gap -2,
// floor 0; ties of a cell go to 0, then diagonal, then the cell above (row
// i-1), then the left one; the best cell is the first in row-major order
// with the highest score and, among those, the fewest mismatches.  One
// thread per read; the previous row (score, start, mismatches) lives in
// shared memory as int16, laid out [column][thread].  counters[2] counts the
// reads dropped.
__global__ void pre_primer_kernel(ReadSet r, int n, const uint8_t* __restrict__ primer, int m, int max_mm,
                                  uint8_t* __restrict__ alive, unsigned int* __restrict__ counters) {
    extern __shared__ int16_t rows[];
    const int T = blockDim.x, t = threadIdx.x;
    const int cols = 2 * m + 1;
    int16_t* S = rows;
    int16_t* ST = rows + cols * T;
    int16_t* MM = rows + 2 * cols * T;
    const int64_t stride = (int64_t)gridDim.x * T;
    for (int64_t i0 = (int64_t)blockIdx.x * T + t; i0 < n; i0 += stride) {
        if (!alive[i0]) continue;
        const int L = r.len[i0];
        const int lb = min(2 * m, L);
        const uint8_t* B = reinterpret_cast<const uint8_t*>(r.pad + r.woff[i0]);
        for (int j = 0; j <= lb; ++j) { S[j * T + t] = 0; ST[j * T + t] = 0; MM[j * T + t] = 0; }
        int best = -9999, best_mm = 999, startA = 0, endA = 0;
        for (int i = 1; i <= m; ++i) {
            const uint8_t a = primer[i - 1];
            int dS = S[t], dST = ST[t], dMM = MM[t];   // row i-1, column 0
            int lS = 0, lST = i, lMM = 0;               // row i, column 0
            S[t] = 0; ST[t] = (int16_t)i; MM[t] = 0;
            for (int j = 1; j <= lb; ++j) {
                const int uS = S[j * T + t], uST = ST[j * T + t], uMM = MM[j * T + t];
                const bool eq = a == B[j - 1];
                const int t0 = dS + (eq ? 4 : -1), t1 = uS - 2, t2 = lS - 2;
                const int s = max(max(max(t0, t1), t2), 0);
                int st, mm;
                if (s == 0) { st = i - 1; mm = 0; }
                else if (s == t0) { st = dST; mm = dMM + (eq ? 0 : 1); }
                else if (s == t1) { st = uST; mm = uMM + 1; }
                else { st = lST; mm = lMM + 1; }
                if (best < s || (best == s && best_mm > mm)) { best = s; startA = st; endA = i; best_mm = mm; }
                S[j * T + t] = (int16_t)s; ST[j * T + t] = (int16_t)st; MM[j * T + t] = (int16_t)mm;
                dS = uS; dST = uST; dMM = uMM;
                lS = s; lST = st; lMM = mm;
            }
        }
        const int total = best_mm + startA + abs(m - endA);
        const int s0 = total <= max_mm ? startA : 0, e0 = total <= max_mm ? endA : 0;
        if (s0 == e0) {
            alive[i0] = 0;
            atomicAdd(&counters[2], 1u);
        }
    }
}

__global__ void __launch_bounds__(kTileThreads) pre_tile_sort_kernel(uint32_t* idx, int64_t m, ReadSet r) {
    __shared__ uint32_t s[kTile];
    const int64_t base = (int64_t)blockIdx.x * kTile;
    for (int t = threadIdx.x; t < kTile; t += kTileThreads) s[t] = base + t < m ? idx[base + t] : kNone;
    __syncthreads();
    for (int k = 2; k <= kTile; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int t = threadIdx.x;
            const int i = 2 * t - (t & (j - 1));   // bit j of i is clear; partner i + j
            const uint32_t a = s[i], b = s[i + j];
            const bool up = (i & k) == 0;
            if (up ? read_less(r, b, a) : read_less(r, a, b)) { s[i] = b; s[i + j] = a; }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < kTile; t += kTileThreads)
        if (base + t < m) idx[base + t] = s[t];
}

// One merge pass over sorted runs of `width`: each index moves to its
// position in the merged pair of runs, found by a binary search for the
// number of smaller keys in the partner run.
__global__ void pre_merge_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int64_t m,
                                 int64_t width, ReadSet r) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int64_t run = i / width;
    const int64_t base = (run & ~1LL) * width;
    const uint32_t x = src[i];
    int64_t lo, hi, p0, pos;
    if ((run & 1) == 0) {
        p0 = base + width;
        if (p0 >= m) { dst[i] = x; return; }
        lo = p0; hi = min(base + 2 * width, m);
        pos = i - base;
    } else {
        p0 = base;
        lo = base; hi = base + width;
        pos = i - (base + width);
    }
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (read_less(r, src[mid], x)) lo = mid + 1;
        else hi = mid;
    }
    dst[base + pos + (lo - p0)] = x;
}

// flag[p] = 1 where sorted[p] is the last read of its run of equal sequences.
__global__ void pre_last_kernel(const uint32_t* __restrict__ sorted, int64_t m, ReadSet r,
                                uint8_t* __restrict__ flag) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    bool last = true;
    if (p + 1 < m) {
        const uint32_t a = sorted[p], b = sorted[p + 1];
        const int la = r.len[a];
        last = la != r.len[b] || cmp_bytes(r, a, b, la) != 0;
    }
    flag[p] = last ? 1 : 0;
}

__global__ void pre_emit_kernel(const uint32_t* __restrict__ sorted, const uint32_t* __restrict__ pos,
                                int64_t kept, int32_t* __restrict__ out_idx, int32_t* __restrict__ out_freq) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kept) return;
    const int64_t p = pos[k];
    out_idx[k] = (int32_t)sorted[p];
    out_freq[k] = (int32_t)(p - (k ? (int64_t)pos[k - 1] : -1));
}

// Per kept read k (record out_idx[k]): its length as the stage's FASTA
// parser reads it back from the _Clean line "<seq>\n", its byte offset in
// the padded buffer, and bad[0] += 1 when the read holds a byte of
// deleteSpaces' set or is longer than 4,094 bytes.  For such reads that
// line does not come back as one piece with only the newline to trim.
// Otherwise the line loses the newline, then everything after its last
// base letter: ATGCatgc for kmerDist (kmerMain.cpp:289-295), nNATGCatgc for
// genDist (genMain.cpp:175-181); a read without one stays whole.
__global__ void pre_stage_kernel(ReadSet r, const int32_t* __restrict__ out_idx, int64_t kept, int flavour,
                                 int32_t* __restrict__ len_out, int64_t* __restrict__ off_out,
                                 unsigned int* __restrict__ bad) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kept) return;
    const int32_t i = out_idx[k];
    const int L = r.len[i];
    const uint8_t* b = reinterpret_cast<const uint8_t*>(r.pad + r.woff[i]);
    bool odd = L > 4094;
    int last = -1;
    for (int p = 0; p < L && !odd; ++p) {
        const uint8_t c = b[p];
        if ((c >= 8 && c <= 13) || c == ' ') odd = true;
        const uint8_t u = c & 0xDF;   // upper case
        if (u == 'A' || u == 'C' || u == 'G' || u == 'T' || (flavour && u == 'N')) last = p;
    }
    if (odd) atomicAdd(bad, 1u);
    len_out[k] = last >= 0 ? last + 1 : L;
    off_out[k] = r.woff[i] * 16;
}

int grid_for(int64_t items, int per_block, int cap) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((items + per_block - 1) / per_block, cap));
}

// (int) of a double as x86 and Arm both give it for values inside int's
// range; outside it the conversion saturates.
int to_int_sat(double v) {
    if (!(v == v)) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}

}  // namespace

int pre_stage_reads(crispy_ctx* ctx, const crispy_raw* raw, int flavour, const uint8_t** d_bytes,
                    size_t* bytes, const int64_t** d_off, std::vector<int32_t>& h_len) {
    PreJob& j = ctx->pre;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "no preprocess result on this context");
    if (!raw || raw_records(raw) != j.n)
        return fail(ctx, CRISPY_E_INPUT, "the raw records are not those of the last preprocess call");
    const int64_t kept = j.kept;
    // a header line longer than one 4,095-byte piece would come back with
    // its tail read as sequence
    for (int64_t k = 0; k < kept; ++k)
        if (raw_header_line(raw, j.h_idx[k]) + 1 > 4095)
            return fail(ctx, CRISPY_E_UNSUPPORTED,
                        "a kept read's header line exceeds 4095 bytes: read the _Clean file instead");
    h_len.resize((size_t)kept);
    *d_bytes = j.pad.as<uint8_t>();
    *bytes = j.pad.bytes;
    *d_off = nullptr;
    if (kept == 0) return CRISPY_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    CRISPY_TRY(ensure(ctx, j.stage_len, (size_t)kept * 4));
    CRISPY_TRY(ensure(ctx, j.stage_off, (size_t)kept * 8));
    CRISPY_CK(ctx, cudaMemsetAsync(j.counters.ptr, 0, 64, s));
    ReadSet rs{j.pad.as<uint4>(), j.woff.as<int64_t>(), j.len.as<int32_t>()};
    pre_stage_kernel<<<(unsigned)((kept + 255) / 256), 256, 0, s>>>(
        rs, j.out_idx.as<int32_t>(), kept, flavour, j.stage_len.as<int32_t>(), j.stage_off.as<int64_t>(),
        j.counters.as<unsigned int>() + 3);
    count_launch(ctx);
    CRISPY_CK(ctx, cudaGetLastError());
    unsigned int bad = 0;
    CRISPY_CK(ctx, cudaMemcpyAsync(h_len.data(), j.stage_len.ptr, (size_t)kept * 4, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(&bad, j.counters.as<unsigned int>() + 3, 4, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    if (bad)
        return fail(ctx, CRISPY_E_UNSUPPORTED,
                    "%u kept reads hold whitespace or exceed 4094 bytes: read the _Clean file instead", bad);
    *d_off = j.stage_off.as<int64_t>();
    return CRISPY_OK;
}

}  // namespace crispy

using namespace crispy;

extern "C" int crispy_preprocess(crispy_ctx* ctx, const char* seqbuf, const int64_t* offsets,
                                 const int32_t* lengths, const uint8_t* freq, int32_t n,
                                 const crispy_pre_opts* opts, int32_t* out_index, int32_t* out_freq,
                                 crispy_pre_stats* stats) {
    if (!ctx) return fail(nullptr, CRISPY_E_INPUT, "NULL context");
    if (n < 0 || (n > 0 && (!seqbuf || !offsets || !lengths || !freq || !out_index || !out_freq)))
        return fail(ctx, CRISPY_E_INPUT, "NULL argument");
    crispy_pre_stats st{};
    const crispy_pre_opts o = opts ? *opts : crispy_pre_opts{0, 1.0, nullptr, 2};
    const int m_primer = o.primer ? (int)std::strlen(o.primer) : 0;
    if (o.primer && m_primer > kMaxPrimer)
        return fail(ctx, CRISPY_E_UNSUPPORTED, "primer of %d bases: at most %d are supported", m_primer, kMaxPrimer);
    int64_t total_bytes = 0, words = 0;
    std::vector<int64_t> woff((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        if (lengths[i] < 0 || offsets[i] < 0) return fail(ctx, CRISPY_E_INPUT, "negative offset or length");
        total_bytes = std::max(total_bytes, offsets[i] + lengths[i]);
        woff[i] = words;
        words += (lengths[i] + 15) / 16;
    }

    // processReadLength's statistics, in record order and in double as the
    // reference sums them (preprocess.cpp:333-372).  Without a single read
    // the reference reports an error and applies neither the cut nor the N
    // check; st.length_reads = 0 then switches both off.
    unsigned long long lo = 0, hi = ~0ull;
    if (o.length_check) {
        double sum_len = 0.0, num = 0.0;
        for (int32_t i = 0; i < n; ++i)
            if (freq[i]) { sum_len += (double)lengths[i]; num += 1.0; }
        if (num >= 1.0) {
            const double ave = sum_len / num;
            double sum_diff = 0.0;
            int min_len = 65535, max_len = 0;
            for (int32_t i = 0; i < n; ++i) {
                if (!freq[i]) continue;
                const double diff = (double)(size_t)lengths[i] - ave;
                sum_diff += diff * diff;
                min_len = std::min(min_len, lengths[i]);
                max_len = std::max(max_len, lengths[i]);
            }
            sum_diff = sum_diff / num;
            const double sd = std::sqrt(sum_diff);
            st.length_reads = (int32_t)num;
            st.min_len0 = min_len;
            st.max_len0 = max_len;
            min_len = std::max(min_len, to_int_sat(ave - o.sd_allowed * sd));
            max_len = std::min(max_len, to_int_sat(ave + o.sd_allowed * sd));
            st.min_len = min_len;
            st.max_len = max_len;
            st.ave_len = ave;
            st.sd = sd;
            // length() < minLen and length() > maxLen compare as size_t
            lo = (unsigned long long)(long long)min_len;
            hi = (unsigned long long)(long long)max_len;
        }
    }
    if (n == 0) {
        ctx->pre.ready = true;
        ctx->pre.kept = 0;
        ctx->pre.n = 0;
        ctx->pre.h_idx.clear();
        if (stats) *stats = st;
        return CRISPY_OK;
    }

    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    PreJob& j = ctx->pre;
    j.ready = false;
    CRISPY_TRY(ensure(ctx, j.seq, (size_t)total_bytes + 16));
    CRISPY_TRY(ensure(ctx, j.off, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.len, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.freq, (size_t)n));
    CRISPY_TRY(ensure(ctx, j.woff, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.pad, (size_t)(words + 1) * 16));
    CRISPY_TRY(ensure(ctx, j.alive, (size_t)n));
    CRISPY_TRY(ensure(ctx, j.idx, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.idx_alt, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.flags, (size_t)n));
    CRISPY_TRY(ensure(ctx, j.pos, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.tiles, ((size_t)n / kScanTile + 2) * 4));
    CRISPY_TRY(ensure(ctx, j.out_idx, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.out_freq, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.counters, 64));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.seq.ptr, seqbuf, (size_t)total_bytes, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.off.ptr, offsets, (size_t)n * 8, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.len.ptr, lengths, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.freq.ptr, freq, (size_t)n, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.woff.ptr, woff.data(), (size_t)n * 8, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemsetAsync(j.counters.ptr, 0, 64, s));

    ReadSet rs{j.pad.as<uint4>(), j.woff.as<int64_t>(), j.len.as<int32_t>()};
    const int warp_grid = 8 * ctx->sm_count;   // 256-thread blocks, 8 warps each
    pre_pad_kernel<<<grid_for((int64_t)n * 32, 256, warp_grid), 256, 0, s>>>(
        j.seq.as<uint8_t>(), j.off.as<int64_t>(), j.len.as<int32_t>(), j.woff.as<int64_t>(), n, j.pad.as<uint4>());
    pre_filter_kernel<<<grid_for((int64_t)n * 32, 256, warp_grid), 256, 0, s>>>(
        rs, j.freq.as<uint8_t>(), n, st.length_reads > 0 ? 1 : 0, lo, hi, j.alive.as<uint8_t>(),
        j.counters.as<unsigned int>());
    count_launch(ctx, 2);
    if (o.primer) {
        CRISPY_TRY(ensure(ctx, j.primer, (size_t)m_primer + 16));
        if (m_primer) CRISPY_CK(ctx, cudaMemcpyAsync(j.primer.ptr, o.primer, (size_t)m_primer, cudaMemcpyHostToDevice, s));
        const size_t per_thread = (size_t)3 * (2 * m_primer + 1) * sizeof(int16_t);
        int threads = (int)std::min<size_t>(256, (size_t)(96 * 1024) / per_thread);
        threads = std::max(32, threads / 32 * 32);
        const size_t smem = per_thread * threads;
        CRISPY_CK(ctx, cudaFuncSetAttribute(pre_primer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        pre_primer_kernel<<<grid_for(n, threads, 4 * ctx->sm_count), threads, smem, s>>>(
            rs, n, j.primer.as<uint8_t>(), m_primer, o.max_mismatches, j.alive.as<uint8_t>(),
            j.counters.as<unsigned int>());
        count_launch(ctx);
    }
    CRISPY_CK(ctx, cudaGetLastError());

    // alive records -> indices (record order)
    int64_t m = 0;
    CRISPY_TRY(compact_flags(ctx, s, j.alive.as<uint8_t>(), n, j.idx.as<uint32_t>(), j.tiles.as<uint32_t>(),
                             j.tmp, &m));
    unsigned int cnt[4] = {0, 0, 0, 0};
    CRISPY_CK(ctx, cudaMemcpyAsync(cnt, j.counters.ptr, sizeof cnt, cudaMemcpyDeviceToHost, s));

    // sort by (length, bytes, record index)
    uint32_t* a = j.idx.as<uint32_t>();
    uint32_t* b = j.idx_alt.as<uint32_t>();
    if (m > 1) {
        pre_tile_sort_kernel<<<(unsigned)((m + kTile - 1) / kTile), kTileThreads, 0, s>>>(a, m, rs);
        count_launch(ctx);
        for (int64_t w = kTile; w < m; w <<= 1) {
            pre_merge_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(a, b, m, w, rs);
            count_launch(ctx);
            std::swap(a, b);
        }
    }
    int64_t kept = 0;
    if (m > 0) {
        pre_last_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(a, m, rs, j.flags.as<uint8_t>());
        count_launch(ctx);
        CRISPY_CK(ctx, cudaGetLastError());
        CRISPY_TRY(compact_flags(ctx, s, j.flags.as<uint8_t>(), m, j.pos.as<uint32_t>(), j.tiles.as<uint32_t>(),
                                 j.tmp, &kept));
        pre_emit_kernel<<<(unsigned)((kept + 255) / 256), 256, 0, s>>>(a, j.pos.as<uint32_t>(), kept,
                                                                       j.out_idx.as<int32_t>(),
                                                                       j.out_freq.as<int32_t>());
        count_launch(ctx);
        CRISPY_CK(ctx, cudaGetLastError());
        CRISPY_CK(ctx, cudaMemcpyAsync(out_index, j.out_idx.ptr, (size_t)kept * 4, cudaMemcpyDeviceToHost, s));
        CRISPY_CK(ctx, cudaMemcpyAsync(out_freq, j.out_freq.ptr, (size_t)kept * 4, cudaMemcpyDeviceToHost, s));
    }
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    j.kept = kept;
    j.n = n;
    j.h_idx.assign(out_index, out_index + kept);
    j.ready = true;
    st.length_discards = (int32_t)(cnt[0] + cnt[1]);
    st.primer_discards = (int32_t)cnt[2];
    st.merges = (int32_t)(m - kept);
    st.kept = (int32_t)kept;
    if (stats) *stats = st;
    return CRISPY_OK;
}
