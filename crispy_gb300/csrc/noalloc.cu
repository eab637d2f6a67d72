// noalloc.cu -- banded NW alignment for callers that cannot allocate.
//
// Some callers cannot call cudaMalloc: an application that carves all device
// memory into its own pool at start-up and forbids allocation afterwards, an
// embedding runtime whose memory accounting must not see foreign
// allocations, or code running where an allocation would synchronise the
// device at the wrong moment.  crispy_gen_align_noalloc serves them: the
// caller passes device buffers for the reads, the pairs and every output,
// and the per-thread DP rows live in one file-scope device array of fixed
// size (kScratchBytes), which every GPU that loads this library holds until
// the process exits.  Nothing here calls cudaMalloc, cudaFree or an
// allocating library routine.
//
// The array is shared by every call: calls that overlap on the GPU (two
// streams, two host threads) race on it and must be serialised by the
// caller.  Each call clears the part that must start at zero (the
// error word) before its kernel runs.
//
// Every call looks up the array's device address with cudaGetSymbolAddress,
// with the caller's device current (the lookup allocates nothing).  The
// address is not cached: after a cudaDeviceReset, or under a context other
// than the device's primary one, a cached address could point outside the
// current context.  The call is synchronous (it waits for its kernel to
// report bad inputs), so it cannot run inside a stream capture.
#include <cuda_runtime.h>

#include "internal.h"

namespace {

// 8 MiB of DP rows.  A thread aligning a pair of band half-width kb needs
// 6 * (2*kb + 3) ints; the call runs as many threads (a multiple of 32) as
// the array holds for the widest band of the call and rejects the call when
// not even one warp fits.
constexpr size_t kScratchBytes = 8u << 20;
constexpr size_t kScratchInts = kScratchBytes / sizeof(int);
constexpr size_t kErrorWord = kScratchInts - 1;   // last int: error flag
static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

constexpr int kNeg = -1048576;
constexpr int kRefNegInf = -1000000;
constexpr int kGO = -10, kGE = -1, kMatch = 5, kMismatch = -4;

__device__ __forceinline__ int sym_of(char ch) {
    return ch == 'G' ? 1 : ch == 'T' ? 2 : ch == 'C' ? 3 : 0;
}

struct Best {
    int m;
    unsigned l;
};

// Error bits in the error word: 1 = a pair index outside [0, n), 2 = a band
// wider than the rows the host sized, 4 = a read longer than max_len.  A
// rejected pair gets dist NaN and score / ml / al -1.
__device__ __forceinline__ void reject(int* err_word, int bit, int64_t p, float* dist, int32_t* score,
                                       int32_t* ml, int32_t* al) {
    atomicOr(err_word, bit);
    dist[p] = __int_as_float(0x7fc00000);
    if (score) score[p] = -1;
    if (ml) ml[p] = -1;
    if (al) al[p] = -1;
}

// The wide-band recurrence of gen.cu (rows over read2 = pair[1], columns over
// read1 = pair[0], band coordinates x = j - i + kb + 1), reading the ASCII
// reads directly so that no packed copy has to be allocated.
__global__ void __launch_bounds__(32) noalloc_wide_kernel(
    int* scratch, int row_stride, const char* __restrict__ seq, const int64_t* __restrict__ off,
    const int32_t* __restrict__ len, int n, int max_len, const int2* __restrict__ pairs, int64_t npairs,
    int band, float* __restrict__ dist, int32_t* __restrict__ score, int32_t* __restrict__ ml,
    int32_t* __restrict__ al) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const int rs = row_stride;
    int* base = scratch + tid * (int64_t)rs * 6;
    for (int64_t p = tid; p < npairs; p += nthreads) {
        const int2 pr = pairs[p];
        if (pr.x < 0 || pr.x >= n || pr.y < 0 || pr.y >= n) {
            reject(&scratch[kErrorWord], 1, p, dist, score, ml, al);
            continue;
        }
        const int l1 = len[pr.x], l2 = len[pr.y];
        if (l1 > max_len || l2 > max_len || l1 < 0 || l2 < 0) {
            reject(&scratch[kErrorWord], 4, p, dist, score, ml, al);
            continue;
        }
        const int kb = band >= 2 ? (l1 + l2) / (2 * band) : max(l1, l2);
        if (2 * kb + 3 > rs) {   // cannot happen once the lengths are checked; kept as a guard
            reject(&scratch[kErrorWord], 2, p, dist, score, ml, al);
            continue;
        }
        const int width = 2 * kb + 3;
        const char* s1 = seq + off[pr.x];
        const char* s2 = seq + off[pr.y];
        int* rowM[2] = {base, base + 3 * rs};
        int* rowC[2] = {base + rs, base + 4 * rs};
        int* rowL[2] = {base + 2 * rs, base + 5 * rs};
        for (int x = 0; x < width; ++x) { rowM[0][x] = kNeg; rowC[0][x] = 0; rowL[0][x] = 0; }
        for (int j = 0; j <= min(kb, l1); ++j) { rowM[0][j + kb + 1] = 0; rowL[0][j + kb + 1] = j; }
        Best col{kRefNegInf, 0u}, row{kRefNegInf, 0u};
        int cur = 0;
        for (int i = 1; i <= l2; ++i) {
            const int pre = cur;
            cur ^= 1;
            int* Mc = rowM[cur]; int* Cc = rowC[cur]; int* Lc = rowL[cur];
            const int* Mp = rowM[pre]; const int* Cp = rowC[pre]; const int* Lp = rowL[pre];
            for (int x = 0; x < width; ++x) { Mc[x] = kNeg; Cc[x] = 0; Lc[x] = 0; }
            if (i <= kb) { Mc[kb - i + 1] = 0; Lc[kb - i + 1] = i; }
            const int c2 = sym_of(s2[i - 1]);
            const int jlo = max(1, i - kb), jhi = min(l1, i + kb);
            for (int j = jlo; j <= jhi; ++j) {
                const int x = j - i + kb + 1;
                const bool match = sym_of(s1[j - 1]) == c2;
                const int md = Mp[x] + (match ? kMatch : kMismatch);
                const int cu = Cc[x - 1], cl = Cp[x + 1];
                const int upM = Mc[x - 1] + (cu == 1 ? kGO : (cu == 4 ? kGE : 0));
                const int lfM = Mp[x + 1] + (cl == 1 ? kGO : (cl == 2 ? kGE : 0));
                const int mx = max(md, max(upM, lfM));
                unsigned l;
                int code;
                if (mx == md) { code = 1; l = (unsigned)Lp[x] + (match ? 0x1u : 0x10001u); }
                else if (mx == upM) { code = 4; l = (unsigned)Lc[x - 1] + 0x10001u; }
                else { code = 2; l = (unsigned)Lp[x + 1] + 0x10001u; }
                Mc[x] = mx; Cc[x] = code; Lc[x] = (int)l;
                if (i == l2 && mx >= col.m) { col.m = mx; col.l = l; }
                if (j == l1 && mx >= row.m) { row.m = mx; row.l = l; }
            }
        }
        const bool use_col = col.m > row.m;
        const unsigned l = use_col ? col.l : row.l;
        const int mlv = (int)(l >> 16), alv = (int)(l & 0xffffu);
        dist[p] = __fdiv_rn((float)mlv, (float)alv);
        if (score) score[p] = use_col ? col.m : row.m;
        if (ml) ml[p] = mlv;
        if (al) al[p] = alv;
    }
}

}  // namespace

extern "C" int crispy_gen_align_noalloc(const char* d_seq, const int64_t* d_offsets,
                                        const int32_t* d_lengths, int n, int max_len,
                                        const int32_t* d_pairs, int64_t npairs, int band,
                                        float* d_dist, int32_t* d_score, int32_t* d_ml,
                                        int32_t* d_al, void* stream) {
    if (!d_seq || !d_offsets || !d_lengths || n <= 0 || (npairs > 0 && (!d_pairs || !d_dist)) ||
        npairs < 0)
        return crispy::fail(nullptr, CRISPY_E_INPUT, "gen_align_noalloc: NULL or empty argument");
    if (max_len <= 0 || max_len > CRISPY_MAX_READ_LEN)
        return crispy::fail(nullptr, CRISPY_E_UNSUPPORTED, "gen_align_noalloc: max_len %d outside 1..%d",
                            max_len, CRISPY_MAX_READ_LEN);
    if (band <= 0) band = 2;   // genMain.cpp:356-364
    const int kb_max = band >= 2 ? (2 * max_len) / (2 * band) : max_len;
    const int rs = 2 * kb_max + 3;
    const int64_t fit = (int64_t)((kScratchInts - 256) / ((size_t)rs * 6)) / 32 * 32;
    if (fit < 32)
        return crispy::fail(nullptr, CRISPY_E_UNSUPPORTED,
                            "gen_align_noalloc: band half-width %d needs more than the %zu-byte scratch",
                            kb_max, kScratchBytes);
    // the array's address in the current context, looked up on every call
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
        return crispy::fail(nullptr, CRISPY_E_DEVICE, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    int* scratch = static_cast<int*>(ptr);
    if (npairs == 0) return CRISPY_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((e = cudaMemsetAsync(scratch + kErrorWord, 0, sizeof(int), s)) != cudaSuccess)
        return crispy::fail(nullptr, CRISPY_E_DEVICE, "clear error word: %s", cudaGetErrorString(e));
    // one warp per block: threads stays a multiple of 32 and never exceeds
    // `fit`, so every thread's rows lie inside the array, below the error word
    const int64_t threads = std::min<int64_t>(fit, ((npairs + 31) / 32) * 32);
    noalloc_wide_kernel<<<(unsigned)(threads / 32), 32, 0, s>>>(
        scratch, rs, d_seq, d_offsets, d_lengths, n, max_len, reinterpret_cast<const int2*>(d_pairs), npairs,
        band, d_dist, d_score, d_ml, d_al);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return crispy::fail(nullptr, CRISPY_E_DEVICE, "gen_align_noalloc launch: %s", cudaGetErrorString(e));
    int flag = 0;
    if ((e = cudaMemcpyAsync(&flag, scratch + kErrorWord, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return crispy::fail(nullptr, CRISPY_E_DEVICE, "gen_align_noalloc: %s", cudaGetErrorString(e));
    if (flag)
        return crispy::fail(nullptr, CRISPY_E_INPUT,
                            "gen_align_noalloc: %s", (flag & 1) ? "a pair index is outside [0, n)"
                                                     : "a read is longer than max_len");
    return CRISPY_OK;
}
