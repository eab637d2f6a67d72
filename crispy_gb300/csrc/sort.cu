// sort.cu -- stable LSD radix sort and stable stream compaction.
//
// The reference orders each genDist output chunk with Thrust's device
// sort_by_key on float keys (genCUDA.cu:39-45), which is a stable radix sort,
// and orders kmerDist output by the host scan of whole tiles
// (kmerMain.cpp:175-195).  Both orders are reproduced here with one stable
// 8-bit LSD radix sort written for this library:
//   pass = histogram (per 4096-item tile) -> exclusive scan (digit-major)
//          -> stable scatter (in-tile rank via warp match + per-warp counts).
// Non-negative IEEE floats sort correctly as their uint32 bit patterns,
// which is all genDist needs (distances are ML/AL >= +0.0, never NaN).
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"

namespace crispy {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;                       // per thread
constexpr int kSortTile = kSortThreads * kSortItems; // 4096
constexpr int kWarps = kSortThreads / 32;

template <class K>
__device__ __forceinline__ uint32_t digit_of(K key, int shift) {
    return (uint32_t)(key >> shift) & 0xFFu;
}

template <class K>
__global__ void __launch_bounds__(kSortThreads) rs_hist(const K* __restrict__ keys, int64_t n,
                                                        int shift, uint32_t* __restrict__ hist,
                                                        int nblocks) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll 4
    for (int j = 0; j < kSortItems; ++j) {
        int64_t i = base + (int64_t)j * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[digit_of(keys[i], shift)], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of m uint32 values in place with one block; writes the sum
// to *total when total != nullptr.  The block walks the array in tiles of
// 4096 values (four consecutive values per thread, coalesced), carrying the
// running sum from tile to tile.
__global__ void __launch_bounds__(1024) scan_exclusive_1blk(uint32_t* __restrict__ v, int64_t m,
                                                            uint32_t* __restrict__ total) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t s_carry;
    const int t = threadIdx.x;
    const int lane = t & 31, w = t >> 5;
    if (t == 0) s_carry = 0;
    __syncthreads();
    const bool vec = (reinterpret_cast<uintptr_t>(v) & 15u) == 0;
    for (int64_t base = 0; base < m; base += 4096) {
        const int64_t i0 = base + 4 * (int64_t)t;
        uint32_t a[4];
        if (vec && i0 + 3 < m) {
            const uint4 q = *reinterpret_cast<const uint4*>(v + i0);
            a[0] = q.x; a[1] = q.y; a[2] = q.z; a[3] = q.w;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) a[k] = i0 + k < m ? v[i0 + k] : 0u;
        }
        const uint32_t sum = a[0] + a[1] + a[2] + a[3];
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            uint32_t z = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            wsum[lane] = z;
        }
        __syncthreads();
        const uint32_t carry = s_carry;
        uint32_t run = carry + x - sum + (w > 0 ? wsum[w - 1] : 0u);
        uint32_t out[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) { out[k] = run; run += a[k]; }
        if (vec && i0 + 3 < m) {
            *reinterpret_cast<uint4*>(v + i0) = make_uint4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) if (i0 + k < m) v[i0 + k] = out[k];
        }
        __syncthreads();   // every thread has read s_carry and wsum
        if (t == 1023) s_carry = carry + wsum[31];
        __syncthreads();
    }
    if (t == 0 && total) *total = s_carry;
}

template <class K, bool kVals>
__global__ void __launch_bounds__(kSortThreads) rs_scatter(const K* __restrict__ kin,
                                                           const uint32_t* __restrict__ vin,
                                                           K* __restrict__ kout,
                                                           uint32_t* __restrict__ vout, int64_t n,
                                                           int shift,
                                                           const uint32_t* __restrict__ offs,
                                                           int nblocks) {
    __shared__ uint32_t base[256];      // global position of the next item per digit
    __shared__ uint32_t wcnt[kWarps][256];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    base[t] = offs[(int64_t)t * nblocks + blockIdx.x];
    const int64_t tile = (int64_t)blockIdx.x * kSortTile;
    const uint32_t lt = (1u << lane) - 1u;
    for (int j = 0; j < kSortItems; ++j) {
#pragma unroll
        for (int q = 0; q < kWarps; ++q) wcnt[q][t] = 0;
        __syncthreads();
        const int64_t i = tile + (int64_t)j * kSortThreads + t;
        const bool valid = i < n;
        K key = valid ? kin[i] : K(0);
        uint32_t val = (kVals && valid) ? vin[i] : 0u;
        uint32_t d = valid ? digit_of(key, shift) : (0x100u + (uint32_t)lane);
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        // exclusive prefix over warps, per digit (thread t owns digit t)
        uint32_t run = 0;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) {
            uint32_t c = wcnt[q][t];
            wcnt[q][t] = run;
            run += c;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = base[d] + wcnt[w][d] + rank;
            kout[pos] = key;
            if (kVals) vout[pos] = val;
        }
        __syncthreads();
        base[t] += run;
    }
}

template <class K, bool kVals>
int radix_sort(crispy_ctx* ctx, cudaStream_t s, K* keys, K* keys_alt, uint32_t* vals,
               uint32_t* vals_alt, int64_t n, int key_bits, K** out_keys, uint32_t** out_vals,
               DevBuf& tmp) {
    *out_keys = keys;
    if (out_vals) *out_vals = vals;
    if (n <= 1) return CRISPY_OK;
    const int nblocks = (int)((n + kSortTile - 1) / kSortTile);
    CRISPY_TRY(ensure(ctx, tmp, (size_t)256 * nblocks * sizeof(uint32_t)));
    uint32_t* hist = tmp.as<uint32_t>();
    K *src = keys, *dst = keys_alt;
    uint32_t *vsrc = vals, *vdst = vals_alt;
    for (int shift = 0; shift < key_bits; shift += 8) {
        rs_hist<K><<<nblocks, kSortThreads, 0, s>>>(src, n, shift, hist, nblocks);
        scan_exclusive_1blk<<<1, 1024, 0, s>>>(hist, (int64_t)256 * nblocks, nullptr);
        rs_scatter<K, kVals><<<nblocks, kSortThreads, 0, s>>>(src, vsrc, dst, vdst, n, shift, hist,
                                                              nblocks);
        count_launch(ctx, 3);
        std::swap(src, dst);
        std::swap(vsrc, vdst);
    }
    CRISPY_CK(ctx, cudaGetLastError());
    *out_keys = src;
    if (out_vals) *out_vals = vsrc;
    return CRISPY_OK;
}

constexpr int kCmpThreads = 256;
constexpr int kCmpPer = kScanTile / kCmpThreads;  // 18
static_assert(kScanTile % kCmpThreads == 0, "tile");

__global__ void __launch_bounds__(kCmpThreads) cmp_count(const uint8_t* __restrict__ flags,
                                                         int64_t n, uint32_t* __restrict__ cnt) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    uint32_t c = 0;
    for (int j = 0; j < kCmpPer; ++j) {
        int64_t i = base + (int64_t)j * kCmpThreads + threadIdx.x;
        if (i < n) c += flags[i] != 0;
    }
    c = __reduce_add_sync(0xffffffffu, c);
    __shared__ uint32_t ws[kCmpThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int q = 0; q < kCmpThreads / 32; ++q) s += ws[q];
        cnt[blockIdx.x] = s;
    }
}

// Each thread owns kCmpPer consecutive items, so output order is item order.
__global__ void __launch_bounds__(kCmpThreads) cmp_scatter(const uint8_t* __restrict__ flags,
                                                           int64_t n,
                                                           const uint32_t* __restrict__ offs,
                                                           uint32_t* __restrict__ out) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kCmpPer;
    uint32_t mine = 0;
    uint32_t bits = 0;
#pragma unroll
    for (int j = 0; j < kCmpPer; ++j) {
        int64_t i = base + j;
        uint32_t f = (i < n) ? (flags[i] != 0) : 0u;
        bits |= f << j;
        mine += f;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __shared__ uint32_t ws[kCmpThreads / 32];
    if (lane == 31) ws[w] = x;
    __syncthreads();
    uint32_t wbase = 0;
    for (int q = 0; q < w; ++q) wbase += ws[q];
    uint32_t pos = offs[blockIdx.x] + wbase + x - mine;
    while (bits) {
        int j = __ffs(bits) - 1;
        bits &= bits - 1;
        out[pos++] = (uint32_t)(base + j);
    }
}

}  // namespace

size_t sort_tmp_bytes(int64_t n) {
    const int64_t nblocks = (n + kSortTile - 1) / kSortTile;
    return (size_t)256 * (size_t)std::max<int64_t>(nblocks, 1) * sizeof(uint32_t);
}

int sort_u64_payload(crispy_ctx* ctx, cudaStream_t s, uint64_t* keys, uint64_t* keys_alt,
                     uint32_t* vals, uint32_t* vals_alt, int64_t n, int key_bits, bool with_vals,
                     uint64_t** sorted_keys, uint32_t** sorted_vals, DevBuf& tmp) {
    if (with_vals)
        return radix_sort<uint64_t, true>(ctx, s, keys, keys_alt, vals, vals_alt, n, key_bits,
                                          sorted_keys, sorted_vals, tmp);
    return radix_sort<uint64_t, false>(ctx, s, keys, keys_alt, nullptr, nullptr, n, key_bits,
                                       sorted_keys, nullptr, tmp);
}

int sort_u32_payload(crispy_ctx* ctx, cudaStream_t s, uint32_t* keys, uint32_t* keys_alt,
                     uint32_t* vals, uint32_t* vals_alt, int64_t n, int key_bits,
                     uint32_t** sorted_keys, uint32_t** sorted_vals, DevBuf& tmp) {
    return radix_sort<uint32_t, true>(ctx, s, keys, keys_alt, vals, vals_alt, n, key_bits,
                                      sorted_keys, sorted_vals, tmp);
}

int compact_flags(crispy_ctx* ctx, cudaStream_t s, const uint8_t* flags, int64_t n,
                  uint32_t* out_idx, uint32_t* tile_counts, DevBuf& tmp, int64_t* total) {
    if (total) *total = 0;
    if (n <= 0) return CRISPY_OK;
    const int nt = (int)((n + kScanTile - 1) / kScanTile);
    CRISPY_TRY(ensure(ctx, tmp, (size_t)(nt + 1) * sizeof(uint32_t)));
    uint32_t* offs = tmp.as<uint32_t>();
    cmp_count<<<nt, kCmpThreads, 0, s>>>(flags, n, tile_counts);
    CRISPY_CK(ctx, cudaMemcpyAsync(offs, tile_counts, nt * sizeof(uint32_t),
                                   cudaMemcpyDeviceToDevice, s));
    scan_exclusive_1blk<<<1, 1024, 0, s>>>(offs, nt, offs + nt);
    cmp_scatter<<<nt, kCmpThreads, 0, s>>>(flags, n, offs, out_idx);
    count_launch(ctx, 3);
    CRISPY_CK(ctx, cudaGetLastError());
    if (!total) return CRISPY_OK;   // the caller reads tile_counts (and sums them) itself
    uint32_t tot = 0;
    CRISPY_CK(ctx, cudaMemcpyAsync(&tot, offs + nt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    *total = tot;
    return CRISPY_OK;
}

}  // namespace crispy
