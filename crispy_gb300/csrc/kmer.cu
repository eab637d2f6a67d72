// kmer.cu -- kmerDist on GB300: all-pairs k-mer distance with the cut
// threshold and sparse-pair compaction fused into the tile kernel.
//
// Reference semantics (kmerMain.cpp:117-216, kmerKernel.cu:19-51,
// kmerCUDA.cu:14-126): each read's K-mers are 2-bit codes (A0 G1 T2 C3,
// others 0) over T = L-K+1 windows; the count of shared K-mers between two
// reads is the sorted-merge count, which for K <= 7 equals the multiset
// min-sum  m = sum_k min(cnt_a[k], cnt_b[k]);  dist = 1 - m / min(Ta, Tb) in
// single precision; a pair survives iff dist < thr or |dist - thr| < 1e-5.
//
// GB300 design (no tensor cores: a min-sum is not a dense contraction):
//   * min(a, b) = sum_{t>=1} [a >= t][b >= t].  Every read becomes a list of
//     T "level entries" (t-1)*4^K + kmer, one per occurrence, where t is the
//     occurrence rank of that K-mer in the read.  Then
//         m(a, b) = #{ entries e of b : e in entries(a) }.
//   * A block owns 128 row reads (64 at K = 7, 32 at K = 8) and keeps their
//     entry sets in shared memory as bit planes: 128-bit word P[e] has bit r
//     set iff row read r holds entry e.  One 128-bit shared load answers one
//     column entry for 128 row reads.  Levels 1..levels live in dense planes
//     (two levels of 4^K words at K = 6, 128 KB); the rare entries of higher
//     level go to a small open-addressing hash table in shared memory, so
//     the footprint stays fixed whatever the reads hold.
//   * A warp owns 32 column reads (one per lane) and streams their entries
//     from an interleaved layout (eight consecutive entries of one read in a
//     uint4, the 32 reads' uint4 of one octet in one 512-byte line), gathers
//     the plane word of each, and adds its quarters into four sets of 32
//     bit-sliced counters with Harley-Seal carry-save trees (LOP3 work
//     only).  The next 16 entries are in flight while the current 16 are
//     reduced.  The streamed entries are precomputed 16-bit plane word
//     indices, ordered per 32-read group so that the 8 lanes of a
//     quarter-warp hit 8 different 16-byte banks; high-level entries and
//     pads index zero guard words, so the gather has no branch and the rare
//     high-level entries get a separate hash pass.
//   * Bounds skip work that cannot pass the cut, never changing a count
//     that can: at K <= 6 the batched form counts a hashed share of each
//     column's entries first and the rest only where a row may still pass
//     (m <= m0 + Ta - a0); at K = 8 pairs of reads with different H keys
//     need a read with |H| >= mmin[T], and same-key pairs whose H sums
//     already fall short of mmin[Ta] - |L_a| skip their L sums.
//   * The threshold is an integer test m >= mmin[min(Ta, Tb)], with mmin
//     tabulated on the host from the reference's float expression (the pass
//     predicate is monotone in m), first as a bit-sliced compare against a
//     per-lane lower bound, then exactly for the few candidates.  Survivors
//     leave through warp-aggregated atomics as (stage, row, col) sort keys;
//     one stable radix sort restores the reference's stage order.
//   * K = 8 (65,536 bins per level) and row groups whose high-level entries
//     would overflow the hash run through an exact dense-table kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"

namespace crispy {
namespace {

constexpr uint32_t kSentinel = 0xFFFFFFFFu;
constexpr int kTileThreads = 512;
constexpr int kTileWarps = kTileThreads / 32;
constexpr int kTileRows = 64;            // row reads per block: one 64-bit plane word
constexpr int kHashBits = 11;
constexpr int kHashSlots = 1 << kHashBits;   // high-level entries of one row group
constexpr int kHashMaxKeys = kHashSlots / 2; // load factor <= 1/2 keeps probes short
constexpr int kPlaneBudget = 128 * 1024;     // dense level planes per block
constexpr int kSplitDefault = 112;           // section 0 of the split streams: 112/256 of the entries

__device__ __forceinline__ uint32_t sym2(uint8_t c) {
    // A=0 G=1 T=2 C=3, everything else 0 (kmerMain.cpp:137-152)
    return c == 'G' ? 1u : c == 'T' ? 2u : c == 'C' ? 3u : 0u;
}

__device__ __forceinline__ uint32_t kmer_at(const uint8_t* s, int p, int K) {
    uint32_t v = 0;
    for (int q = 0; q < K; ++q) v = (v << 2) | sym2(s[p + q]);
    return v;
}

// Entry e of lane l inside a group block: four consecutive entries of one
// lane are one uint4, and the 32 lanes' uint4 of the same quad are adjacent.
__device__ __forceinline__ int64_t ent_at(int e, int lane) {
    return (int64_t)(e >> 2) * 128 + lane * 4 + (e & 3);
}

// ---------------------------------------------------------------------------
// Preparation: one block per read.  Occurrence ranks come from a shared
// histogram with two 16-bit counters per word (counts <= 2048), so K = 8
// (65,536 bins) fits in 128 KB.  Writes the read's level entries into its
// lane of the group's interleaved block, its largest multiplicity, its count
// of entries above the dense levels, and for K = 8 the (largest K-mer >=
// 0x8000, its count) key used by the quirk.
//
// Entry order inside a read's lane: its high-level entries (occurrence rank
// >= dense_levels) first, then its dense entries grouped by shared-memory
// bank (an entry's bank is its value mod 32; banks in the order lane,
// lane+1, ... mod 32), with the per-bank counts written to bcnt.  The tile kernel does not read this order directly: the
// schedule kernel below turns it into a bank-conflict-avoiding stream.
// ---------------------------------------------------------------------------
// Section of a dense level entry (its plane word index) when a read's
// dense entries are split in two (K <= 6): a multiplicative hash of the word
// index above its bank bits, so that every bank splits in the same ratio;
// section 0 iff the hash's top byte is below split.
__device__ __forceinline__ int split_section(uint32_t val, uint32_t split) {
    return ((val >> 3) * 0x9E3779B1u) >> 24 < split ? 0 : 1;
}

// Raw-list bucket of a dense level entry: K <= 7, the bank of its 32-bit
// word index (with a split, behind its section: 0..31 or 32..63); K = 8,
// the section (H = K-mer >= 0x8000 first) and the 4-byte bank of its 16-bit
// plane word.
__device__ __forceinline__ int prep_bucket(uint32_t val, int K, uint32_t split) {
    if (K == 8) {
        // the bank of the K-mer's 32-bit plane word (H: K-mer - 0x8000,
        // L: K-mer), per section
        const uint32_t v = val & 0xFFFFu;
        return (v >= 0x8000u ? 0 : 32) + (int)(v & 31u);
    }
    return (split ? 32 * split_section(val, split) : 0) + (int)(val & 31u);
}

constexpr int kPrepThreads = 256;
constexpr int kPrepPer = CRISPY_MAX_READ_LEN / kPrepThreads;   // positions per thread

// Per-read K-mer counts in shared memory.  Two 16-bit counts per 32-bit
// word (K <= 7, 32 KB at K = 7); at K = 8 five 12-bit counts per 64-bit word
// (102 KB instead of 128 KB, so that two blocks share an SM).  A count never
// exceeds a read's tuples (2041 < 4096), so no field overflows.
struct PrepHist16 {
    uint32_t* h;
    static constexpr size_t bytes(uint32_t K4) { return (size_t)((K4 + 1) / 2) * 4; }
    __device__ void clear_all(uint32_t K4) const {
        for (int i = threadIdx.x; i < (int)((K4 + 1) / 2); i += blockDim.x) h[i] = 0;
    }
    __device__ uint32_t add(uint32_t v) const {   // old count
        const uint32_t sh = (v & 1u) * 16u;
        return (atomicAdd(&h[v >> 1], 1u << sh) >> sh) & 0xFFFFu;
    }
    __device__ uint32_t get(uint32_t v) const { return (h[v >> 1] >> ((v & 1u) * 16u)) & 0xFFFFu; }
    __device__ void clear(uint32_t v) const { h[v >> 1] = 0; }
};
struct PrepHist12 {
    unsigned long long* h;
    static constexpr size_t bytes(uint32_t K4) { return (size_t)((K4 + 4) / 5) * 8; }
    __device__ void clear_all(uint32_t K4) const {
        for (int i = threadIdx.x; i < (int)((K4 + 4) / 5); i += blockDim.x) h[i] = 0ull;
    }
    __device__ uint32_t add(uint32_t v) const {
        const uint32_t w = v / 5u, sh = 12u * (v - 5u * w);
        return (uint32_t)(atomicAdd(&h[w], 1ull << sh) >> sh) & 0xFFFu;
    }
    __device__ uint32_t get(uint32_t v) const {
        const uint32_t w = v / 5u;
        return (uint32_t)(h[w] >> (12u * (v - 5u * w))) & 0xFFFu;
    }
    __device__ void clear(uint32_t v) const { h[v / 5u] = 0ull; }
};

template <typename Hist>
__global__ void __launch_bounds__(kPrepThreads) kmer_prep_kernel(
    const uint8_t* __restrict__ seq, const int64_t* __restrict__ off,
    const int32_t* __restrict__ tcount, int n, int K, int dense_levels,
    const int64_t* __restrict__ gstart, const int32_t* __restrict__ gent,
    uint32_t* __restrict__ ent, int32_t* __restrict__ cntmax, int32_t* __restrict__ nhigh,
    uint32_t* __restrict__ hinfo, uint16_t* __restrict__ bcnt, int32_t* __restrict__ nsec,
    uint32_t split) {
    extern __shared__ __align__(16) unsigned long long hist_words[];
    const Hist hist{reinterpret_cast<decltype(Hist::h)>(hist_words)};
    __shared__ int s_max, s_hpos;
    __shared__ uint32_t s_hmax;
    __shared__ int s_bcnt[64], s_bstart[64];
    const uint32_t K4 = 1u << (2 * K);
    // K = 8: two sections, H (K-mer >= 0x8000) then L, grouped by the 4-byte
    // bank of a 16-bit plane word; K <= 7: one section (two with a split),
    // grouped by the bank of a 32-bit word index (value mod 32)
    const int nsections = K == 8 || split ? 2 : 1;
    hist.clear_all(K4);
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        if (threadIdx.x == 0) { s_max = 0; s_hmax = 0; s_hpos = 0; }
        if (threadIdx.x < 64) s_bcnt[threadIdx.x] = 0;
        __syncthreads();
        const int T = tcount[r];
        const uint8_t* s = seq + off[r];
        uint32_t* dst = ent + gstart[r >> 5];
        const int lane = r & 31;
        const int E = gent[r >> 5];
        uint32_t val[kPrepPer];
        int rank[kPrepPer];
#pragma unroll
        for (int k = 0; k < kPrepPer; ++k) {
            const int p = threadIdx.x + k * kPrepThreads;
            rank[k] = -1;
            if (p < T) {
                const uint32_t v = kmer_at(s, p, K);
                const uint32_t t = hist.add(v);
                val[k] = t * K4 + v;
                if ((int)t >= dense_levels) {
                    dst[ent_at(atomicAdd(&s_hpos, 1), lane)] = val[k];
                } else {
                    rank[k] = atomicAdd(&s_bcnt[prep_bucket(val[k], K, split)], 1);
                }
            }
        }
        for (int p = T + threadIdx.x; p < E; p += blockDim.x) dst[ent_at(p, lane)] = kSentinel;
        __syncthreads();
        if (threadIdx.x < 32) {
            // bank order rotated by the lane: at a given position the 32
            // reads of a group sit in different banks, which keeps the
            // one-thread-per-column dense kernel free of bank conflicts
            const int i = threadIdx.x;
            int base = s_hpos;
            for (int sec = 0; sec < nsections; ++sec) {
                const int b = sec * 32 + ((i + lane) & 31);
                const int c = s_bcnt[b];
                int x = c;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, d);
                    if (i >= d) x += y;
                }
                s_bstart[b] = base + x - c;
                bcnt[(int64_t)r * (32 * nsections) + b] = (uint16_t)c;
                const int total = __shfl_sync(0xffffffffu, x, 31);
                if (nsec && i == 0) nsec[(int64_t)r * 2 + sec] = total;
                base += total;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kPrepPer; ++k)
            if (rank[k] >= 0) dst[ent_at(s_bstart[prep_bucket(val[k], K, split)] + rank[k], lane)] = val[k];
        __syncthreads();
        int mx = 0;
        uint32_t hm = 0;
#pragma unroll
        for (int k = 0; k < kPrepPer; ++k) {
            // this thread's positions are those of the first pass: reuse their K-mers
            const int p = threadIdx.x + k * kPrepThreads;
            if (p < T) {
                const uint32_t v = val[k] & (K4 - 1u);
                const int c = (int)hist.get(v);
                mx = max(mx, c);
                if (v >= 0x8000u) hm = max(hm, v);
            }
        }
        atomicMax(&s_max, mx);
        atomicMax(&s_hmax, hm);
        __syncthreads();
        if (threadIdx.x == 0) {
            cntmax[r] = s_max;
            nhigh[r] = s_hpos;
            uint32_t info = 0;
            if (K == 8 && s_hmax >= 0x8000u) {
                const uint32_t c = hist.get(s_hmax);
                info = (s_hmax << 16) | c;
            }
            hinfo[r] = info;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kPrepPer; ++k)
            if (threadIdx.x + k * kPrepThreads < T) hist.clear(val[k] & (K4 - 1u));
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Preparation, one warp per read (read sets whose reads hold at most
// kPrepWarpMaxT tuples).  The same outputs as kmer_prep_kernel -- the set of
// level entries of each read and of each of its buckets, the bucket and
// section counts, the largest multiplicity, the high-level count, the K = 8
// key -- without a block-wide histogram: occurrence ranks come from a
// 1,024-slot open-addressing table per warp in shared memory (key << 16 |
// count, one atomic per occurrence), so 48 warps of an SM work on 48 reads
// at once instead of two blocks on two.  Which occurrence of a K-mer gets
// which rank, and so the order of entries inside a bucket, is whatever the
// atomics give; every consumer treats a bucket as a set.
// ---------------------------------------------------------------------------
constexpr int kPrepWarpMaxT = 512;
constexpr int kPrepWarpPer = kPrepWarpMaxT / 32;   // positions per lane
constexpr int kPrepWarpSlots = 1024;                // table slots per warp (load <= 1/2)
constexpr int kPrepWarps = 8;                       // warps per block
constexpr uint32_t kPrepEmpty = 0xFFFFFFFFu;        // key 0xFFFF, count 0xFFFF: never a real slot

// Old count (the occurrence's rank) of K-mer v, after counting it.
__device__ __forceinline__ uint32_t warp_table_add(uint32_t* tbl, uint32_t v) {
    uint32_t h = (v * 0x9E3779B1u) >> 22;   // 10 bits: kPrepWarpSlots
    for (int probe = 0; probe < kPrepWarpSlots; ++probe) {
        const uint32_t cur = *reinterpret_cast<volatile uint32_t*>(tbl + h);
        if (cur == kPrepEmpty) {
            const uint32_t old = atomicCAS(&tbl[h], kPrepEmpty, (v << 16) | 1u);
            if (old == kPrepEmpty) return 0u;
            if ((old >> 16) == v) return atomicAdd(&tbl[h], 1u) & 0xFFFFu;
        } else if ((cur >> 16) == v) {
            return atomicAdd(&tbl[h], 1u) & 0xFFFFu;
        }
        h = (h + 1u) & (kPrepWarpSlots - 1u);
    }
    return 0u;   // unreachable: a read has at most kPrepWarpMaxT distinct K-mers
}

__device__ __forceinline__ uint32_t warp_table_count(const uint32_t* tbl, uint32_t v) {
    uint32_t h = (v * 0x9E3779B1u) >> 22;
    for (int probe = 0; probe < kPrepWarpSlots; ++probe) {
        const uint32_t cur = tbl[h];
        if (cur == kPrepEmpty) return 0u;
        if ((cur >> 16) == v) return cur & 0xFFFFu;
        h = (h + 1u) & (kPrepWarpSlots - 1u);
    }
    return 0u;
}

__global__ void __launch_bounds__(kPrepWarps * 32) kmer_prep_warp_kernel(
    const uint8_t* __restrict__ seq, const int64_t* __restrict__ off,
    const int32_t* __restrict__ tcount, int n, int K, int dense_levels,
    const int64_t* __restrict__ gstart, const int32_t* __restrict__ gent,
    uint32_t* __restrict__ ent, int32_t* __restrict__ cntmax, int32_t* __restrict__ nhigh,
    uint32_t* __restrict__ hinfo, uint16_t* __restrict__ bcnt, int32_t* __restrict__ nsec,
    uint32_t split) {
    __shared__ __align__(16) uint32_t s_tbl[kPrepWarps][kPrepWarpSlots];
    __shared__ int s_bc[kPrepWarps][64], s_bs[kPrepWarps][64];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t* tbl = s_tbl[w];
    int* bc = s_bc[w];
    int* bs = s_bs[w];
    const uint32_t K4 = 1u << (2 * K);
    const int nsections = K == 8 || split ? 2 : 1;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = blockIdx.x * kPrepWarps + w; r < n; r += gridDim.x * kPrepWarps) {
        uint4* t4 = reinterpret_cast<uint4*>(tbl);
        for (int i = lane; i < kPrepWarpSlots / 4; i += 32)
            t4[i] = make_uint4(kPrepEmpty, kPrepEmpty, kPrepEmpty, kPrepEmpty);
        bc[lane] = 0;
        bc[lane + 32] = 0;
        __syncwarp();
        const int T = tcount[r];
        const uint8_t* s = seq + off[r];
        uint32_t* dst = ent + gstart[r >> 5];
        const int rl = r & 31;
        const int E = gent[r >> 5];
        uint32_t val[kPrepWarpPer];
        int rank[kPrepWarpPer];   // rank in its bucket (dense), -1 high-level, -2 none
        int mx = 0;
        uint32_t hm = 0;
#pragma unroll
        for (int k = 0; k < kPrepWarpPer; ++k) {
            const int p = lane + 32 * k;
            rank[k] = -2;
            val[k] = 0;
            if (p < T) {
                const uint32_t v = kmer_at(s, p, K);
                const uint32_t t = warp_table_add(tbl, v);
                val[k] = t * K4 + v;
                mx = max(mx, (int)t + 1);
                if (v >= 0x8000u) hm = max(hm, v);
                rank[k] = (int)t >= dense_levels ? -1 : atomicAdd(&bc[prep_bucket(val[k], K, split)], 1);
            }
        }
        // high-level entries first, in warp order
        int hpos = 0;
#pragma unroll
        for (int k = 0; k < kPrepWarpPer; ++k) {
            const unsigned m = __ballot_sync(full, rank[k] == -1);
            if (rank[k] == -1) dst[ent_at(hpos + __popc(m & lt), rl)] = val[k];
            hpos += __popc(m);
        }
        __syncwarp();
        // then the dense entries by section and bank, banks rotated by the
        // read's lane in the group (the same order as kmer_prep_kernel)
        int base = hpos;
        for (int sec = 0; sec < nsections; ++sec) {
            const int b = sec * 32 + ((lane + rl) & 31);
            const int c = bc[b];
            int x = c;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(full, x, d);
                if (lane >= d) x += y;
            }
            bs[b] = base + x - c;
            bcnt[(int64_t)r * (32 * nsections) + b] = (uint16_t)c;
            const int total = __shfl_sync(full, x, 31);
            if (nsec && lane == 0) nsec[(int64_t)r * 2 + sec] = total;
            base += total;
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < kPrepWarpPer; ++k)
            if (rank[k] >= 0) dst[ent_at(bs[prep_bucket(val[k], K, split)] + rank[k], rl)] = val[k];
        for (int p = T + lane; p < E; p += 32) dst[ent_at(p, rl)] = kSentinel;
        mx = (int)__reduce_max_sync(full, (unsigned)mx);
        hm = __reduce_max_sync(full, hm);
        if (lane == 0) {
            cntmax[r] = mx;
            nhigh[r] = hpos;
            hinfo[r] = K == 8 && hm >= 0x8000u ? (hm << 16) | warp_table_count(tbl, hm) : 0u;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// K = 8 read order.  The tile kernel adds a pair's L half only where both
// reads have the same H key (largest H K-mer and its count, or no H K-mer).
// Sorting the reads by (H key, tuple count) puts reads of one key next to
// one another, so that most warps of the tile kernel hold no pair with
// [same] and skip their L phase; the tuple count keeps the 32-read groups'
// padding small.  One warp per read finds the largest H K-mer, then counts
// it; the sort key is (H key << tbits) | T, the payload the read index.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) kmer_hkey_kernel(const uint8_t* __restrict__ seq,
                                                        const int64_t* __restrict__ off,
                                                        const int32_t* __restrict__ tcount, int n,
                                                        int tbits, uint64_t* __restrict__ keys,
                                                        uint32_t* __restrict__ idx) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int r = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < n; r += nw) {
        const int T = tcount[r];
        const uint8_t* s = seq + off[r];
        uint32_t hm = 0;
        for (int p = lane; p < T; p += 32) {
            const uint32_t v = kmer_at(s, p, 8);
            if (v >= 0x8000u) hm = max(hm, v);
        }
        hm = __reduce_max_sync(full, hm);
        uint32_t c = 0;
        if (hm != 0u)
            for (int p = lane; p < T; p += 32) c += kmer_at(s, p, 8) == hm;
        c = __reduce_add_sync(full, c);
        if (lane == 0) {
            const uint32_t key = hm != 0u ? (hm << 16) | (c & 0xFFFFu) : 0u;
            keys[r] = ((uint64_t)key << tbits) | (uint32_t)T;
            idx[r] = (uint32_t)r;
        }
    }
}

__global__ void kmer_gather_off_kernel(const int64_t* __restrict__ off, const uint32_t* __restrict__ perm,
                                       int n, int64_t* __restrict__ offp, int32_t* __restrict__ permi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t r = perm[i];
        offp[i] = off[r];
        permi[i] = (int32_t)r;
    }
}

// ---------------------------------------------------------------------------
// Bank schedule of the tile stream.  The tile kernel's plane words are
// 64-bit (64 row reads), so a warp's gather is served as two half-warps of
// 16 lanes, and word w sits in double bank w mod 16.  One warp per 32-read
// group writes, for every step e < Et and lane l, the 16-bit plane word
// index that lane l gathers at step e, such that the 16 lanes of each half
// hit 16 different double banks where the counts allow.
//   * Ideal slots: lane l takes a bucket-h entry (h = word mod 16) at every
//     step with (e + l) mod 16 == h while it has bucket-h entries left; the
//     ideal buckets of a half at one step are a rotation, hence different.
//   * A lane whose ideal bucket is empty at step e (a hole) takes one of its
//     surplus entries (buckets with more entries than ideal slots) whose
//     bucket no other lane of its half uses at e; claims are settled by
//     match_any, lowest lane first, repeated until no lane can claim.
//   * Remaining holes take a wildcard: a guard word (always zero) in a
//     bucket still free at e.  High-level entries (looked up in the hash by a
//     separate pass) and the pad steps up to Et are the wildcards.  A lane
//     out of wildcards places a surplus entry anyway (a bank conflict).
// Every hole is filled by exactly one surplus entry or wildcard, because
// holes - surplus = Et - dense entries = wildcards for every lane.
// The raw list of a read is grouped by 32-bank (value mod 32), so bucket h
// draws first on bank h, then on bank h + 16.
// ---------------------------------------------------------------------------
constexpr int kSchedWarps = 4;
constexpr int kSchedChunk = 16;
constexpr int kSchedSpare = 24;   // spare steps per group (reads of >= 128 tuples)

__device__ __forceinline__ int nth_set_bit(unsigned m, int k) {   // 0-based; -1 if none
    for (int i = 0; i < k && m; ++i) m &= m - 1u;
    return m ? __ffs(m) - 1 : -1;
}

// One tile stream of one 32-read group (warp w of the block, lane = read).
// A gather of kB-bucket words is served per set of kB lanes (a wavefront);
// word w sits in bucket w mod kB.
//   kB = 8:  128-bit plane words, 8 quad banks per quarter-warp; bucket b
//            draws on the raw bank groups b, b + 8, b + 16, b + 24.
//   kB = 16: 64-bit plane words, 16 double banks per half-warp; bucket b
//            draws on the raw bank groups b and b + 16 (value mod 32).
//   kB = 32: 16-bit plane words, 32 four-byte banks over the whole warp;
//            bucket b is raw group b of the section.
// raw_cnt: this lane's 32 raw group counts; pos0: its first raw position
// of the section; the stream values are the plane word indices
// (value - vsub), and guard words (always zero) fill the wildcard steps.
struct SchedSmem {
    uint16_t cnt[kSchedWarps][32][33];    // entries per bucket
    uint16_t ov[kSchedWarps][32][33];     // surplus per bucket
    uint16_t next[kSchedWarps][32][33];   // next raw position per raw group
    uint16_t left[kSchedWarps][32][33];   // raw entries left per raw group
    uint8_t bank[kSchedWarps][kSchedChunk][32];
};

template <int kB>
__device__ void sched_stream(SchedSmem& sm, int w, int lane, bool active, const uint16_t* raw_cnt,
                             int pos0, int Et, const uint32_t* __restrict__ src, uint32_t vsub,
                             uint32_t guard0, uint32_t gstride, uint16_t* __restrict__ dst_group) {
    const unsigned full = 0xffffffffu;
    constexpr unsigned kMask = kB == 32 ? 0xffffffffu : (1u << kB) - 1u;
    constexpr int kSub = 32 / kB;                         // raw groups per bucket
    const int hs = lane & (32 - kB);                      // this lane set's bit offset in 32-bit masks
    const unsigned half_lt = ((1u << lane) - 1u) & (kMask << hs);
    for (int b = 0; b < 32; ++b) sm.left[w][lane][b] = active ? raw_cnt[b] : (uint16_t)0;
    // first raw position of each raw group: the prep kernel's lane-rotated order
    for (int i = 0, pos = pos0; i < 32; ++i) {
        const int b = (i + lane) & 31;
        sm.next[w][lane][b] = (uint16_t)pos;
        pos += sm.left[w][lane][b];
    }
    int D = 0;
    unsigned ovmask = 0;
    for (int b = 0; b < kB; ++b) {
        int c = 0;
#pragma unroll
        for (int i = 0; i < kSub; ++i) c += sm.left[w][lane][b + i * kB];
        const int o = (b - lane) & (kB - 1);
        const int slots = Et > o ? (Et - o + kB - 1) / kB : 0;
        const int ov = max(0, c - slots);
        sm.cnt[w][lane][b] = (uint16_t)c;
        sm.ov[w][lane][b] = (uint16_t)ov;
        D += c;
        if (ov) ovmask |= 1u << b;
    }
    int wild = Et - D;
    __syncwarp();
    uint4* dst = reinterpret_cast<uint4*>(dst_group) + lane;
    for (int e0 = 0; e0 < Et; e0 += kSchedChunk) {
        for (int i = 0; i < kSchedChunk; ++i) {
            const int e = e0 + i;
            const int h = (e + lane) & (kB - 1);
            const bool hole = (e / kB) >= (int)sm.cnt[w][lane][h];
            int bank = hole ? -1 : h;
            unsigned used = __reduce_or_sync(full, hole ? 0u : (1u << (h + hs)));
            bool open = hole;
            for (int round = 0; round < kB; ++round) {
                const unsigned cand = open ? (ovmask & ~(used >> hs) & kMask) : 0u;
                if (!__any_sync(full, cand != 0u)) break;
                const int prop = cand ? hs + __ffs(cand) - 1 : 64 + lane;
                const unsigned peers = __match_any_sync(full, prop);
                const bool win = cand && lane == __ffs(peers) - 1;
                if (win) {
                    bank = prop - hs;
                    open = false;
                    const int left = (int)sm.ov[w][lane][bank] - 1;
                    sm.ov[w][lane][bank] = (uint16_t)left;
                    if (left == 0) ovmask &= ~(1u << bank);
                }
                used |= __reduce_or_sync(full, win ? (1u << prop) : 0u);
            }
            const bool wl = open && wild > 0;
            const unsigned wm = __ballot_sync(full, wl);
            if (wl) {
                // the k-th wildcard lane of a half takes the k-th free bucket
                const int fb = nth_set_bit(~(used >> hs) & kMask, __popc(wm & half_lt));
                bank = kB + (fb >= 0 ? fb : 0);
                --wild;
            } else if (open) {
                const int b = ovmask ? __ffs(ovmask) - 1 : -1;
                if (b >= 0) {
                    bank = b;
                    const int left = (int)sm.ov[w][lane][b] - 1;
                    sm.ov[w][lane][b] = (uint16_t)left;
                    if (left == 0) ovmask &= ~(1u << b);
                } else {
                    bank = kB;   // unreachable by the count identity; stays in bounds
                }
            }
            sm.bank[w][i][lane] = (uint8_t)bank;
        }
        __syncwarp();
        // gather the chosen entries: positions first, then the loads
        uint32_t v[kSchedChunk];
#pragma unroll
        for (int i = 0; i < kSchedChunk; ++i) {
            const int b = sm.bank[w][i][lane];
            if (b < kB) {
                int bb = b;   // first raw group of the bucket with entries left
                for (int q = 1; q < kSub && !sm.left[w][lane][bb]; ++q) bb = b + q * kB;
                const int p = sm.next[w][lane][bb];
                sm.next[w][lane][bb] = (uint16_t)(p + 1);
                sm.left[w][lane][bb] = (uint16_t)(sm.left[w][lane][bb] - 1);
                v[i] = (uint32_t)p;
            } else {
                v[i] = 0x80000000u | (uint32_t)(b - kB);
            }
        }
#pragma unroll
        for (int i = 0; i < kSchedChunk; ++i) {
            const uint32_t x = v[i];
            // guard of bucket b: word guard0 + b (128-, 64- or 32-bit words,
            // bucket b) or halfword guard0 + 2b (16-bit words, 4-byte bank b)
            v[i] = (x & 0x80000000u) ? guard0 + (x & 31u) * gstride
                                     : __ldg(src + ent_at((int)x, lane)) - vsub;
        }
        // two octets of this lane: two uint4 of packed 16-bit word indices
#pragma unroll
        for (int o = 0; o < 2; ++o) {
            uint4 q;
            q.x = (v[8 * o + 0] & 0xFFFFu) | (v[8 * o + 1] << 16);
            q.y = (v[8 * o + 2] & 0xFFFFu) | (v[8 * o + 3] << 16);
            q.z = (v[8 * o + 4] & 0xFFFFu) | (v[8 * o + 5] << 16);
            q.w = (v[8 * o + 6] & 0xFFFFu) | (v[8 * o + 7] << 16);
            dst[(int64_t)((e0 >> 3) + o) * 32] = q;
        }
        __syncwarp();
    }
}

// K <= 7: one stream per group; kB = 8 for 128-bit plane words (K <= 6),
// 16 for 64-bit plane words (K = 7).
template <int kB>
__global__ void __launch_bounds__(kSchedWarps * 32) kmer_sched_kernel(
    const uint32_t* __restrict__ ent, const int64_t* __restrict__ gstart,
    const int64_t* __restrict__ tstart, const int32_t* __restrict__ tgent,
    const int32_t* __restrict__ nhigh, const uint16_t* __restrict__ bcnt, int n, int ngroups,
    uint32_t guard_word, uint16_t* __restrict__ tent) {
    __shared__ SchedSmem sm;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int g = blockIdx.x * kSchedWarps + w; g < ngroups; g += gridDim.x * kSchedWarps) {
        const int r = g * 32 + lane;
        const bool active = r < n;
        sched_stream<kB>(sm, w, lane, active, bcnt + (int64_t)(active ? r : 0) * 32,
                         active ? nhigh[r] : 0, tgent[g], ent + gstart[g], 0u, guard_word, 1u,
                         tent + tstart[g]);
    }
}

// K <= 6 with a split: two streams per group over the same 128-bit plane
// words, section 0 then section 1, each scheduled on its own.  A group's
// steps per stream (the largest section of its reads, rounded up to 16) are
// set here on the device: tgent = section 0, tgentL = section 1, and the
// section-1 stream starts right after section 0's, so the two read as one
// stream of tgent + tgentL steps.  tstart leaves room for 2 * gent steps,
// which bounds the sum (each section holds at most a read's tuples).
__global__ void __launch_bounds__(kSchedWarps * 32) kmer_sched_split_kernel(
    const uint32_t* __restrict__ ent, const int64_t* __restrict__ gstart,
    const int64_t* __restrict__ tstart, const int32_t* __restrict__ nhigh,
    const int32_t* __restrict__ nsec, const uint16_t* __restrict__ bcnt, int n, int ngroups,
    uint32_t guard_word, int32_t* __restrict__ tgent, int32_t* __restrict__ tgentL,
    uint16_t* __restrict__ tent) {
    __shared__ SchedSmem sm;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int g = blockIdx.x * kSchedWarps + w; g < ngroups; g += gridDim.x * kSchedWarps) {
        const int r = g * 32 + lane;
        const bool active = r < n;
        const int rr = active ? r : 0;
        const int nh = active ? nhigh[r] : 0;
        const int n0 = active ? nsec[(int64_t)rr * 2] : 0;
        const int n1 = active ? nsec[(int64_t)rr * 2 + 1] : 0;
        const int E0 = ((int)__reduce_max_sync(full, (unsigned)n0) + 15) / 16 * 16;
        const int E1 = ((int)__reduce_max_sync(full, (unsigned)n1) + 15) / 16 * 16;
        if (lane == 0) {
            tgent[g] = E0;
            tgentL[g] = E1;
        }
        sched_stream<8>(sm, w, lane, active, bcnt + (int64_t)rr * 64, nh, E0, ent + gstart[g], 0u,
                        guard_word, 1u, tent + tstart[g]);
        __syncwarp();
        sched_stream<8>(sm, w, lane, active, bcnt + (int64_t)rr * 64 + 32, nh + n0, E1, ent + gstart[g],
                        0u, guard_word, 1u, tent + tstart[g] + (int64_t)32 * E0);
        __syncwarp();
    }
}

// K = 8: an H stream and an L stream per group; the H section of a read's
// raw list follows its high-level entries, the L section follows the H
// section.  Each stream indexes a plane of 32-bit words (bank = word mod
// 32) whose guard words start at 32768: H: K-mer - 0x8000, L: K-mer.
// The steps of both streams per group are set here from the per-read
// section counts: H = the largest H section, rounded up to 16 (no spare
// steps: the H-only kernel is issue-bound, a bank conflict costs it less
// than a step); L = the largest L section plus kSchedSpare spare steps when
// it holds 64 entries or more, rounded up to 16.  tstart leaves room for
// 2 * gent + 32 steps, which bounds the two.
__global__ void __launch_bounds__(kSchedWarps * 32) kmer_sched8_kernel(
    const uint32_t* __restrict__ ent, const int64_t* __restrict__ gstart,
    const int64_t* __restrict__ tstart, int32_t* __restrict__ tgent,
    int32_t* __restrict__ tgentL, const int32_t* __restrict__ nhigh,
    const int32_t* __restrict__ nsec, const uint16_t* __restrict__ bcnt, int n, int ngroups,
    uint16_t* __restrict__ tent) {
    __shared__ SchedSmem sm;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int g = blockIdx.x * kSchedWarps + w; g < ngroups; g += gridDim.x * kSchedWarps) {
        const int r = g * 32 + lane;
        const bool active = r < n;
        const int rr = active ? r : 0;
        const int nh = active ? nhigh[r] : 0;
        const int nH = active ? nsec[(int64_t)rr * 2] : 0;
        const int nL = active ? nsec[(int64_t)rr * 2 + 1] : 0;
        const int mh = (int)__reduce_max_sync(full, (unsigned)nH);
        const int ml = (int)__reduce_max_sync(full, (unsigned)nL);
        const int EtH = (mh + 15) / 16 * 16;
        const int EtL = (ml + (ml >= 64 ? kSchedSpare : 0) + 15) / 16 * 16;
        if (lane == 0) {
            tgent[g] = EtH;
            tgentL[g] = EtL;
        }
        sched_stream<32>(sm, w, lane, active, bcnt + (int64_t)rr * 64, nh, EtH, ent + gstart[g],
                         0x8000u, 32768u, 1u, tent + tstart[g]);
        __syncwarp();
        sched_stream<32>(sm, w, lane, active, bcnt + (int64_t)rr * 64 + 32, nh + nH, EtL,
                         ent + gstart[g], 0u, 32768u, 1u, tent + tstart[g] + (int64_t)32 * EtH);
        __syncwarp();
    }
}

struct TileArgs {
    const uint32_t* ent;           // level entries, high-level ones first per read
    const int64_t* gstart;
    const int32_t* gent;
    const uint16_t* tent;          // scheduled 16-bit plane word indices
    const int64_t* tstart;         // per 32-read group, in 16-bit units
    const int32_t* tgent;
    const int32_t* nhigh;
    const int32_t* tcount;
    const uint8_t* dense_group;   // 32-read groups the dense kernel takes as rows
    const uint16_t* mmin;
    const uint16_t* smin;
    int n;
    uint32_t K4;
    int levels;                    // dense level planes in shared memory
    int A, stage_dim;
    unsigned long long* counter;
    uint64_t* keys;
    uint32_t* vals;
    int64_t cap;
    // plain: one rectangle of rows x cols (one reference stage)
    int r_lo, r_hi, c_lo, c_hi;
    // batched: work queue over row groups (all their columns, or the
    // column range of item_q)
    const int* items;
    int nitems;
    unsigned int* queue_head;
    // 65536 and 8 at run time: index arithmetic written as multiply(-high)
    // adds by them issues on the FMA pipe, next to the LOP3-bound CSA trees
    uint32_t k65536, k8;
    // K = 8
    const int32_t* tgentL;         // L-stream steps per group (H: tgent)
    const uint32_t* hinfo;         // per read: (largest H K-mer << 16) | its count, 0 if none
    int ngroups;
    // read order of the job (position -> read ID), nullptr: identity; with
    // an order, pairs are kept whose lower read ID lies in [olo, ohi)
    const int32_t* perm;
    int olo, ohi;
    // K = 8 batched split: per item the 32-read column groups [x, y) of the
    // two-phase kernel, which then keeps only pairs with [same]; the per-read
    // H / L entry counts (H-only kernel)
    const int2* item_q;
    int same_only;
    const int32_t* nsec;
    // K <= 6: split nonzero when the streams hold two sections (tgent steps
    // of section 0, then tgentL of section 1); bound nonzero when the tile
    // kernel bounds each pair after section 0 (the batched form), qfire the
    // lanes holding a column that start a full-pass round; gstat (may be
    // null) sums the entries of bound and full passes, the full-pass
    // columns and the rounds
    int split, bound, qfire;
    unsigned long long* gstat;
    // K = 8 same-key pass with queued L sums (kmer_tile8s_kernel): per
    // block, per lane slot, sq_cap items of B + 2 words
    uint32_t* sq;
    int64_t sq_cap;
    // Cohort (several jobs' reads back to back, each starting at a multiple
    // of 128 positions; 128-row kernel, batched form): per item its job and
    // its end column group; per job (base, n, A, stage_dim) and its
    // threshold tables at mmin / smin + tbl[job]; survivors carry the job
    // in key bits 44 and up and count per job in job_counter.
    const int* item_job;
    const int* item_cend;
    const int* item_cstart;   // first column group per item (nullptr: the row group's own)
    const int4* cjob;
    const int* ctbl;
    unsigned long long* job_counter;
};

// Parameters of the job a survivor belongs to (the whole run, or one job of
// a cohort): local positions are (r - base, c - base).
struct EmitJob {
    const uint16_t* mmin;
    const uint16_t* smin;
    int n, A, sd, base;
    uint64_t tag;
    unsigned long long* jcount;
};

__device__ __forceinline__ EmitJob emit_job_of(const TileArgs& a) {
    return EmitJob{a.mmin, a.smin, a.n, a.A, a.stage_dim, 0, 0ull, nullptr};
}

__device__ __forceinline__ void csa(uint32_t& h, uint32_t& l, uint32_t a, uint32_t b) {
    const uint32_t u = l ^ a;
    h = (l & a) | (u & b);
    l = u ^ b;
}

__device__ __forceinline__ uint64_t stage_key(int r, int c, int n, int A, int sd) {
    // kmerCUDA.cu:79-111 + Trag_reverse_eq (kmerMain.cpp:205-216): stages
    // enumerate the upper triangle of the stageDim grid row-major; inside a
    // stage the host scan is row-major (kmerMain.cpp:175-195).
    const int64_t sx = r / A, sy = c / A;
    const int64_t s = sx * sd - sx * (sx - 1) / 2 + (sy - sx);
    return ((uint64_t)s * (uint64_t)n + (uint64_t)r) * (uint64_t)n + (uint64_t)c;
}

// Survivor emission with one atomic per warp.  All 32 lanes call it.
// (r, c) are positions in the job's read order; with a read order (perm !=
// nullptr, K = 8) they map back to the caller's read IDs, the pair is
// reordered so that the lower ID comes first, and only pairs whose lower ID
// lies in [olo, ohi) are kept (the stage rows of one pass).
__device__ __forceinline__ void emit(unsigned long long* counter, uint64_t* keys, uint32_t* vals,
                                     int64_t cap, int n, int A, int sd, const int32_t* perm,
                                     int olo, int ohi, bool pass, int r, int c, int m, int mn,
                                     int base_pos = 0, uint64_t tag = 0, unsigned long long* jcount = nullptr) {
    if (perm != nullptr && pass) {
        const int pr = __ldg(perm + r), pc = __ldg(perm + c);
        r = min(pr, pc);
        c = max(pr, pc);
        pass = r >= olo && r < ohi;
    }
    const unsigned pm = __ballot_sync(0xffffffffu, pass);
    if (!pm) return;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    const int leader = __ffs(pm) - 1;
    if (lane == leader) {
        base = atomicAdd(counter, (unsigned long long)__popc(pm));
        if (jcount) atomicAdd(jcount, (unsigned long long)__popc(pm));
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pass) {
        const unsigned long long idx = base + __popc(pm & ((1u << lane) - 1u));
        if (idx < (unsigned long long)cap) {
            keys[idx] = tag | stage_key(r - base_pos, c - base_pos, n, A, sd);
            // kmerKernel.cu:47: 1.0f - (float)matches / min(T1, T2), IEEE
            const float d = __fsub_rn(1.0f, __fdiv_rn((float)m, (float)mn));
            vals[idx] = __float_as_uint(d);
        }
    }
}

__device__ __forceinline__ uint32_t hash_slot(uint32_t key) {
    return (key * 0x9E3779B1u) >> (32 - kHashBits);
}

// Row bits of a high-level entry (absent -> 0).  Rare path.
__device__ __noinline__ uint2 hash_find(const uint32_t* hkeys, const uint2* hmask, uint32_t key) {
    uint32_t h = hash_slot(key);
    for (int probe = 0; probe < kHashSlots; ++probe) {
        const uint32_t k = hkeys[h];
        if (k == key) return hmask[h];
        if (k == kSentinel) return make_uint2(0u, 0u);
        h = (h + 1) & (kHashSlots - 1);
    }
    return make_uint2(0u, 0u);
}

// Bit-sliced counters of 32 row reads: Harley-Seal levels 1, 2, 4, 8, 16
// and the binary count of thirty-twos above them.
template <int B>
struct Counter {
    uint32_t ones, twos, fours, eights, sixteens;
    uint32_t S[B - 5];
    __device__ __forceinline__ void clear() {
        ones = twos = fours = eights = sixteens = 0;
#pragma unroll
        for (int k = 0; k < B - 5; ++k) S[k] = 0;
    }
    // add 16 words; returns the carry out of the eights level (weight 16)
    __device__ __forceinline__ uint32_t add16(const uint32_t* w) {
        uint32_t twosA, twosB, foursA, foursB, eightsA, eightsB, c16;
        csa(twosA, ones, w[0], w[1]);
        csa(twosB, ones, w[2], w[3]);
        csa(foursA, twos, twosA, twosB);
        csa(twosA, ones, w[4], w[5]);
        csa(twosB, ones, w[6], w[7]);
        csa(foursB, twos, twosA, twosB);
        csa(eightsA, fours, foursA, foursB);
        csa(twosA, ones, w[8], w[9]);
        csa(twosB, ones, w[10], w[11]);
        csa(foursA, twos, twosA, twosB);
        csa(twosA, ones, w[12], w[13]);
        csa(twosB, ones, w[14], w[15]);
        csa(foursB, twos, twosA, twosB);
        csa(eightsB, fours, foursA, foursB);
        csa(c16, eights, eightsA, eightsB);
        return c16;
    }
    // add 8 words; returns the carry out of the fours level (weight 8)
    __device__ __forceinline__ uint32_t add8(const uint32_t* w) {
        uint32_t twosA, twosB, foursA, foursB, c8;
        csa(twosA, ones, w[0], w[1]);
        csa(twosB, ones, w[2], w[3]);
        csa(foursA, twos, twosA, twosB);
        csa(twosA, ones, w[4], w[5]);
        csa(twosB, ones, w[6], w[7]);
        csa(foursB, twos, twosA, twosB);
        csa(c8, fours, foursA, foursB);
        return c8;
    }
    // two 8-word carries into the eights level; returns the weight-16 carry
    __device__ __forceinline__ uint32_t merge_eights(uint32_t a, uint32_t b) {
        uint32_t c16;
        csa(c16, eights, a, b);
        return c16;
    }
    __device__ __forceinline__ void carry32(uint32_t carry) {
#pragma unroll
        for (int k = 0; k < B - 5; ++k) {
            const uint32_t t = S[k] & carry;
            S[k] ^= carry;
            carry = t;
        }
    }
    // two batches' sixteens carries: one CSA, one carry chain
    __device__ __forceinline__ void add_sixteens2(uint32_t a, uint32_t b) {
        uint32_t c32;
        csa(c32, sixteens, a, b);
        carry32(c32);
    }
    __device__ __forceinline__ void add_sixteens1(uint32_t a) {
        const uint32_t c32 = sixteens & a;
        sixteens ^= a;
        carry32(c32);
    }
    // bit planes X[k] of the 32 per-row counts
    __device__ __forceinline__ void planes(uint32_t* X) const {
        X[0] = X[1] = X[2] = X[3] = X[4] = 0;
#pragma unroll
        for (int k = 5; k < B; ++k) X[k] = S[k - 5];
        add_at(X, sixteens, 4);
        add_at(X, eights, 3);
        add_at(X, fours, 2);
        add_at(X, twos, 1);
        add_at(X, ones, 0);
    }
    __device__ __forceinline__ static void add_at(uint32_t* X, uint32_t v, int p) {
        uint32_t carry = v;
#pragma unroll
        for (int k = 0; k < B; ++k) {
            if (k >= p) {
                const uint32_t t = X[k] & carry;
                X[k] ^= carry;
                carry = t;
            }
        }
    }
};

// Gather the plane words of 16 scheduled entries (two uint4 of 16-bit word
// indices) and feed both 32-row halves; returns the two sixteens carries.
template <int B>
__device__ __forceinline__ void gather16(const char* __restrict__ Pb, uint4 q0, uint4 q1,
                                         uint32_t k65536, uint32_t k8, Counter<B>& lo,
                                         Counter<B>& hi, uint32_t& c16lo, uint32_t& c16hi) {
    const uint32_t x[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
    uint32_t wl[16], wh[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t ih = __umulhi(x[k], k65536);   // x >> 16
        const uint32_t il = x[k] - ih * k65536;       // x & 0xFFFF
        const uint2 p0 = *reinterpret_cast<const uint2*>(Pb + il * k8);
        const uint2 p1 = *reinterpret_cast<const uint2*>(Pb + ih * k8);
        wl[2 * k] = p0.x; wh[2 * k] = p0.y;
        wl[2 * k + 1] = p1.x; wh[2 * k + 1] = p1.y;
    }
    c16lo = lo.add16(wl);
    c16hi = hi.add16(wh);
}

// Threshold and emission for one 32-row half: candidates by a bit-sliced
// compare against a lower bound of mmin over the lane's pairs, then the
// exact test per candidate.
template <int B>
__device__ __forceinline__ void finish_half(const TileArgs& a, const EmitJob& ej, const uint32_t* X,
                                            uint32_t vmask, int rbase, int t_min, const int* rowT, int c,
                                            int tc) {
    const uint32_t lo = ej.smin[min(t_min, tc)];
    uint32_t cand = 0;
    if (vmask && lo < (1u << B)) {
        uint32_t gt = 0, eq = 0xffffffffu;
#pragma unroll
        for (int k = B - 1; k >= 0; --k) {
            const uint32_t bit = 0u - ((lo >> k) & 1u);
            gt |= eq & X[k] & ~bit;
            eq &= ~(X[k] ^ bit);
        }
        cand = (gt | eq) & vmask;
    }
    while (__any_sync(0xffffffffu, cand)) {
        bool pass = false;
        int r = 0, m = 0, mn = 1;
        if (cand) {
            const int b = __ffs(cand) - 1;
            cand &= cand - 1;
#pragma unroll
            for (int k = 0; k < B; ++k) m |= (int)((X[k] >> b) & 1u) << k;
            r = rbase + b;
            mn = min(rowT[b], tc);
            pass = m >= (int)ej.mmin[mn];
        }
        emit(a.counter, a.keys, a.vals, a.cap, ej.n, ej.A, ej.sd, a.perm, a.olo, a.ohi, pass, r, c, m, mn,
             ej.base, ej.tag, ej.jcount);
    }
}

__device__ __forceinline__ uint32_t half_mask(int span) {   // rows b < span
    return span >= 32 ? 0xffffffffu : (span <= 0 ? 0u : ((1u << span) - 1u));
}

template <int B>
__device__ void tile_columns(const TileArgs& a, const uint2* __restrict__ P,
                             const uint32_t* hkeys, const uint2* hmask, bool any_high, int rg,
                             uint32_t ok0, uint32_t ok1, int tmin0, int tmin1, const int* s_rowT,
                             int cg0, int cg1) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = rg * kTileRows;
    for (int cg = cg0 + warp; cg < cg1; cg += kTileWarps) {
        const int c = cg * 32 + lane;
        const bool col_ok = c >= a.c_lo && c < a.c_hi && c < a.n;
        uint32_t vm0 = 0, vm1 = 0;
        if (col_ok) {
            vm0 = half_mask(c - r0) & ok0;
            vm1 = half_mask(c - r0 - 32) & ok1;
        }
        if (!__any_sync(0xffffffffu, vm0 | vm1)) continue;
        // Scheduled stream: 16-bit plane word indices, eight per uint4;
        // high-level entries and pads index zero guard words.
        const int E = a.tgent[cg];
        const uint4* __restrict__ ep = reinterpret_cast<const uint4*>(a.tent + a.tstart[cg]) + lane;
        Counter<B> lo, hi;
        lo.clear();
        hi.clear();
        const char* __restrict__ Pb = reinterpret_cast<const char*>(P);
        // 32 entries per iteration: two 16-entry batches whose sixteens
        // carries meet in one CSA; the next batch is always in flight
        uint4 a0, a1;
        if (E > 0) { a0 = __ldg(ep); a1 = __ldg(ep + 32); }
        for (int e = 0; e < E; e += 32) {
            const bool two = e + 16 < E;
            uint4 b0, b1;
            if (two) {
                b0 = __ldg(ep + ((e + 16) >> 3) * 32);
                b1 = __ldg(ep + ((e + 16) >> 3) * 32 + 32);
            }
            uint32_t la, ha;
            gather16<B>(Pb, a0, a1, a.k65536, a.k8, lo, hi, la, ha);
            if (e + 32 < E) {
                a0 = __ldg(ep + ((e + 32) >> 3) * 32);
                a1 = __ldg(ep + ((e + 32) >> 3) * 32 + 32);
            }
            if (two) {
                uint32_t lb, hb;
                gather16<B>(Pb, b0, b1, a.k65536, a.k8, lo, hi, lb, hb);
                lo.add_sixteens2(la, lb);
                hi.add_sixteens2(ha, hb);
            } else {
                lo.add_sixteens1(la);
                hi.add_sixteens1(ha);
            }
        }
        uint32_t X0[B], X1[B];
        lo.planes(X0);
        hi.planes(X1);
        // High-level entries (rank >= levels) only meet high-level row
        // entries, which live in the hash; they lead each read's level list.
        if (any_high) {
            const int nh = col_ok ? a.nhigh[c] : 0;
            const int maxh = (int)__reduce_max_sync(0xffffffffu, (unsigned)nh);
            const uint32_t* __restrict__ rp = a.ent + a.gstart[cg];
            for (int j = 0; j < maxh; ++j) {
                const uint2 w = j < nh ? hash_find(hkeys, hmask, __ldg(rp + ent_at(j, lane)))
                                       : make_uint2(0u, 0u);
                Counter<B>::add_at(X0, w.x, 0);
                Counter<B>::add_at(X1, w.y, 0);
            }
        }
        const int tc = col_ok ? a.tcount[c] : 0;
        const EmitJob ej = emit_job_of(a);
        finish_half<B>(a, ej, X0, vm0, r0, tmin0, s_rowT, c, tc);
        finish_half<B>(a, ej, X1, vm1, r0 + 32, tmin1, s_rowT + 32, c, tc);
    }
}

template <int B>
__global__ void __launch_bounds__(kTileThreads, 1) kmer_tile_kernel(TileArgs a) {
    extern __shared__ __align__(16) uint2 P[];   // levels * K4 plane words + 32 guard words
    __shared__ uint32_t hkeys[kHashSlots];
    __shared__ uint2 hmask[kHashSlots];
    __shared__ int s_rowT[kTileRows];
    __shared__ int s_item[4];
    __shared__ int s_tmin[2], s_any_high;
    __shared__ uint32_t s_rows_ok[2];
    const bool queued = a.items != nullptr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int it = 0;; ++it) {
        // ---- fetch work: one 64-row group with all its column groups ----
        if (threadIdx.x == 0) {
            if (queued) {
                const unsigned w = atomicAdd(a.queue_head, 1u);
                s_item[3] = (int)w < a.nitems;
                if (s_item[3]) {
                    s_item[0] = a.items[w];
                    s_item[1] = 0;
                    s_item[2] = a.item_cend ? a.item_cend[w] : (a.n + 31) / 32;
                    s_item[4] = a.item_job ? a.item_job[w] : -1;
                }
            } else {
                s_item[0] = a.r_lo / kTileRows + blockIdx.x;
                s_item[1] = a.c_lo / 32;
                s_item[2] = (a.c_hi + 31) / 32;
                s_item[3] = it == 0;
            }
        }
        __syncthreads();
        if (!s_item[3]) break;
        const int rg = s_item[0], cg0 = s_item[1], cg1 = s_item[2];
        EmitJob ej = emit_job_of(a);
        if (queued && s_item[4] >= 0) {
            const int jb = s_item[4];
            const int4 cj = a.cjob[jb];
            ej.mmin = a.mmin + a.ctbl[jb];
            ej.smin = a.smin + a.ctbl[jb];
            ej.base = cj.x; ej.n = cj.y; ej.A = cj.z; ej.sd = cj.w;
            ej.tag = (uint64_t)jb << 44;
            ej.jcount = a.job_counter + jb;
        }
        __syncthreads();   // every thread has read s_item
        const int rlo = queued ? 0 : a.r_lo, rhi = queued ? a.n : min(a.r_hi, a.n);
        // ---- row group set-up: rows of dense 32-read groups are left to
        // kmer_dense_kernel ----
        if (warp < 2) {
            const int r = rg * kTileRows + warp * 32 + lane;
            const bool ok = r >= rlo && r < rhi && !a.dense_group[r >> 5];
            const int tr = ok ? a.tcount[r] : INT_MAX;
            s_rowT[warp * 32 + lane] = tr;
            const unsigned okm = __ballot_sync(0xffffffffu, ok);
            const int tm = (int)__reduce_min_sync(0xffffffffu, (unsigned)tr);
            if (lane == 0) { s_tmin[warp] = tm; s_rows_ok[warp] = okm; }
            if (warp == 0 && lane == 0) s_any_high = 0;
        }
        const int words = a.levels * (int)a.K4;   // + 32 zero guard words after the planes
        uint4* P4 = reinterpret_cast<uint4*>(P);
        for (int i = threadIdx.x; i < (words + 32) / 2; i += kTileThreads) P4[i] = make_uint4(0, 0, 0, 0);
        for (int i = threadIdx.x; i < kHashSlots; i += kTileThreads) {
            hkeys[i] = kSentinel;
            hmask[i] = make_uint2(0u, 0u);
        }
        __syncthreads();
        uint32_t* Pw = reinterpret_cast<uint32_t*>(P);
        uint32_t* hmw = reinterpret_cast<uint32_t*>(hmask);
        const uint32_t limit = (uint32_t)words;
        for (int b = warp; b < kTileRows; b += kTileWarps) {
            if (!((s_rows_ok[b >> 5] >> (b & 31)) & 1u)) continue;
            const int r = rg * kTileRows + b;
            const uint32_t* src = a.ent + a.gstart[r >> 5];
            const int T = s_rowT[b];
            const uint32_t bit = 1u << (b & 31);
            const int halfw = b >> 5;
            for (int e = lane; e < T; e += 32) {
                const uint32_t idx = src[ent_at(e, r & 31)];
                if (idx < limit) {
                    atomicOr(&Pw[2 * idx + halfw], bit);
                } else {
                    // high-level entry: open addressing; the host guarantees
                    // the group holds at most kHashMaxKeys of them
                    uint32_t h = hash_slot(idx);
                    for (int probe = 0; probe < kHashSlots; ++probe) {
                        const uint32_t old = atomicCAS(&hkeys[h], kSentinel, idx);
                        if (old == kSentinel || old == idx) {
                            atomicOr(&hmw[2 * h + halfw], bit);
                            break;
                        }
                        h = (h + 1) & (kHashSlots - 1);
                    }
                    s_any_high = 1;
                }
            }
        }
        __syncthreads();
        tile_columns<B>(a, P, hkeys, hmask, s_any_high != 0, rg, s_rows_ok[0], s_rows_ok[1],
                        s_tmin[0], s_tmin[1], s_rowT, max(cg0, 2 * rg), cg1);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// 128-row tile kernel (K <= 6).  The same algorithm with 128-bit plane words:
// one 16-byte shared load answers a column entry for 128 row reads, four
// 32-row words that feed four sets of bit-sliced counters.  A warp's 16-byte
// gather is served per quarter-warp, so the stream's schedule spreads the
// 8 lanes of a quarter over 8 quad banks (word mod 8).  Per row pair this
// halves the entry stream again and lowers the gather wavefronts against
// 64-row words (correlated reads spread better over fewer, larger buckets);
// the price is two dense levels at K = 6 (128 KB), the rarer third and later
// occurrences going to the hash.
// ---------------------------------------------------------------------------
constexpr int kRows128 = 128;

// 8 scheduled entries (one uint4 of 16-bit word indices): their 16-byte plane
// words, split into the four 32-row words, into the four counters.
template <int B>
__device__ __forceinline__ void gather8_128(const char* __restrict__ Pb, uint4 q, uint32_t k65536,
                                            uint32_t k16, Counter<B>* cnt, uint32_t* c8) {
    const uint32_t x[4] = {q.x, q.y, q.z, q.w};
    uint32_t w0[8], w1[8], w2[8], w3[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t ih = __umulhi(x[k], k65536);   // x >> 16
        const uint32_t il = x[k] - ih * k65536;       // x & 0xFFFF
        const uint4 p0 = *reinterpret_cast<const uint4*>(Pb + il * k16);
        const uint4 p1 = *reinterpret_cast<const uint4*>(Pb + ih * k16);
        w0[2 * k] = p0.x; w1[2 * k] = p0.y; w2[2 * k] = p0.z; w3[2 * k] = p0.w;
        w0[2 * k + 1] = p1.x; w1[2 * k + 1] = p1.y; w2[2 * k + 1] = p1.z; w3[2 * k + 1] = p1.w;
    }
    c8[0] = cnt[0].add8(w0);
    c8[1] = cnt[1].add8(w1);
    c8[2] = cnt[2].add8(w2);
    c8[3] = cnt[3].add8(w3);
}

// 16 entries (two uint4): the four weight-16 carries
template <int B>
__device__ __forceinline__ void gather16_128(const char* __restrict__ Pb, uint4 q0, uint4 q1,
                                             uint32_t k65536, uint32_t k16, Counter<B>* cnt,
                                             uint32_t* c16) {
    uint32_t a8[4], b8[4];
    gather8_128<B>(Pb, q0, k65536, k16, cnt, a8);
    gather8_128<B>(Pb, q1, k65536, k16, cnt, b8);
#pragma unroll
    for (int p = 0; p < 4; ++p) c16[p] = cnt[p].merge_eights(a8[p], b8[p]);
}

__device__ __noinline__ uint4 hash_find4(const uint32_t* hkeys, const uint4* hmask, uint32_t key) {
    uint32_t h = hash_slot(key);
    for (int probe = 0; probe < kHashSlots; ++probe) {
        const uint32_t k = hkeys[h];
        if (k == key) return hmask[h];
        if (k == kSentinel) return make_uint4(0u, 0u, 0u, 0u);
        h = (h + 1) & (kHashSlots - 1);
    }
    return make_uint4(0u, 0u, 0u, 0u);
}

// Bound pass (K <= 6 with a split).  A read's dense level entries are split
// in two sections by a hash of the plane word, each scheduled as its own
// stream.  The first pass over a column group counts section 0 only, m0.
// Every entry of row read a outside section 0 may still match, so
//     m <= m0 + (Ta - a0),   a0 = a's section-0 entries,
// and with Tb >= Ta the pair can pass only if m0 >= R_a = mmin[Ta] - Ta + a0,
// a per-row constant held as bit planes in shared memory.  A lane (column)
// with no row left alive is done; the others are pushed on the lane's own
// stack of column groups and later counted in full (both sections, the
// hash pass, the exact test).  A full-pass round takes one queued column
// group per lane, so each lane keeps its place in its group's bank
// schedule; lanes with nothing queued read guard words.  Columns shorter
// than a row of the quarter (never with reads in length order) stay alive.
constexpr int kQDepth = 8;    // column groups a lane may hold
constexpr int kQFire = 28;    // a full-pass round runs once this many lanes hold one
constexpr int kRPlanes = 12;  // bit planes of the per-row bound (counts < 4096)

// Guard-word indices of one quad of steps for lanes without entries: step
// k reads guard word (k + lane) mod 8, the bucket the schedule gives the
// lane there.
__device__ __forceinline__ uint4 guard_quad(uint32_t g0, int lane) {
    uint32_t v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = g0 + (uint32_t)((k + lane) & 7);
    return make_uint4(v[0] | (v[1] << 16), v[2] | (v[3] << 16), v[4] | (v[5] << 16), v[6] | (v[7] << 16));
}

// Counts of one column against the 128 row reads over steps [0, El) of its
// stream (lanes beyond El read guard words up to the warp's Emax): 32
// entries per iteration as two 16-entry batches, each gathered as two
// halves of 8 (register budget); the next batch is in flight.
template <int B, bool kLane>
__device__ __forceinline__ void accumulate128(const char* __restrict__ Pb, const uint4* __restrict__ ep,
                                              int El, int Emax, uint4 gq, uint32_t k65536, uint32_t k16,
                                              Counter<B>* cnt) {
#pragma unroll
    for (int q = 0; q < 4; ++q) cnt[q].clear();
    // kLane: steps per lane (full-pass rounds); otherwise every lane runs Emax
    auto ld = [&](int step) { return !kLane || step < El ? __ldg(ep + (step >> 3) * 32) : gq; };
    uint4 a0, a1;
    if (Emax > 0) { a0 = ld(0); a1 = ld(8); }
    for (int e = 0; e < Emax; e += 32) {
        const bool two = e + 16 < Emax;
        uint4 b0, b1;
        if (two) {
            b0 = ld(e + 16);
            b1 = ld(e + 24);
        }
        uint32_t ca[4];
        gather16_128<B>(Pb, a0, a1, k65536, k16, cnt, ca);
        if (e + 32 < Emax) {
            a0 = ld(e + 32);
            a1 = ld(e + 40);
        }
        if (two) {
            uint32_t cb[4];
            gather16_128<B>(Pb, b0, b1, k65536, k16, cnt, cb);
#pragma unroll
            for (int q = 0; q < 4; ++q) cnt[q].add_sixteens2(ca[q], cb[q]);
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) cnt[q].add_sixteens1(ca[q]);
        }
    }
}

// Row bounds of a 128-row block for the bound pass.
struct RowBound {
    const uint32_t* thr;    // [4][kRPlanes] bit planes of R_a per quarter
    const uint32_t* live;   // [4] rows that can pass at all
    const int* tmax;        // [4] largest row tuple count per quarter
};

// Stacks of the bound pass: s_q [warp][depth][lane] column groups, s_qn
// [warp][lane] their sizes, s_qoff [warp][lane] the first position of a
// warp's stack in its lane's pooled list (the warps' stacks in warp order).
struct Stacks {
    uint16_t* q;
    uint8_t* qn;
    uint8_t* qoff;
    int* next;     // [0]: next column group of the first passes, [1]: next pooled round
};

// Two phases.  First the warp's column groups [cg0, cg1), a bound pass
// each (every pass in full without a bound), with full-pass rounds whenever
// enough lanes hold a column or a stack is full.  Then (bound pass only) the
// stacks' remains of every warp are pooled: round i takes the i-th column
// of each lane's pooled list, so the last rounds of a row group run with
// full lanes.  Every thread of the block calls this (the pool phase starts
// with a block barrier).
template <int B>
__device__ void tile_columns128(const TileArgs& a, const EmitJob& ej, const uint4* __restrict__ P,
                                const uint32_t* hkeys, const uint4* hmask, bool any_high, int rg,
                                const uint32_t* s_rows_ok, const int* s_tmin, const int* s_rowT,
                                const RowBound rb, const Stacks sk, int cg0, int cg1) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = rg * kRows128;
    const char* __restrict__ Pb = reinterpret_cast<const char*>(P);
    const bool bound = a.bound != 0;
    const uint4 gq = guard_quad((uint32_t)a.levels * a.K4, lane);
    uint16_t* s_q = sk.q + warp * (kQDepth * 32);
    // with the bound pass, warps claim column groups and pooled rounds from
    // the block's counters (sk.next), so that they reach the pool's barrier
    // together; without it each warp takes every kTileWarps-th group
    int cg = cg0 + warp - kTileWarps;   // the column group of the current first pass
    int qn = 0;            // column groups on this lane's stack
    // pool: the lane's pooled columns, the rounds
    int pi = 0, pc = 0, pmax = 0;
    // entries gathered by live lanes: bound passes, full passes; full-pass
    // columns and rounds
    uint32_t st_bound = 0, st_full = 0, st_cols = 0, st_rounds = 0;
    for (int pool = 0; pool < (bound ? 2 : 1); ++pool) {
        if (pool) {
            sk.qn[warp * 32 + lane] = (uint8_t)qn;
            __syncthreads();
            if (threadIdx.x < 32) {
                int run = 0;
                for (int w = 0; w < kTileWarps; ++w) {
                    sk.qoff[w * 32 + threadIdx.x] = (uint8_t)run;
                    run += sk.qn[w * 32 + threadIdx.x];
                }
            }
            __syncthreads();
            pc = sk.qoff[(kTileWarps - 1) * 32 + lane] + sk.qn[(kTileWarps - 1) * 32 + lane];
            pmax = (int)__reduce_max_sync(full, (unsigned)pc);
        }
        for (;;) {
            bool round;
            if (pool) {
                int v = 0;
                if (lane == 0) v = atomicAdd(sk.next + 1, 1);
                pi = __shfl_sync(full, v, 0);
                if (pi >= pmax) break;
                round = true;
            } else {
                // a full-pass round when enough lanes hold a column or a stack is full
                const unsigned held = __ballot_sync(full, qn > 0);
                round = held != 0u && (__popc(held) >= a.qfire || __any_sync(full, qn == kQDepth));
                if (!round) {
                    if (bound) {
                        int v = 0;
                        if (lane == 0) v = atomicAdd(sk.next, 1);
                        cg = cg0 + __shfl_sync(full, v, 0);
                    } else {
                        cg += kTileWarps;
                    }
                    if (cg >= cg1) break;
                }
            }
            int ccg = 0;
            bool active = true;
            if (pool) {
                active = pi < pc;
                if (active) {
                    int w = 0;
                    while (w + 1 < kTileWarps && (int)sk.qoff[(w + 1) * 32 + lane] <= pi) ++w;
                    ccg = sk.q[w * (kQDepth * 32) + (pi - (int)sk.qoff[w * 32 + lane]) * 32 + lane];
                }
            } else if (round) {
                active = qn > 0;
                if (active) {
                    --qn;
                    ccg = s_q[qn * 32 + lane];
                }
            } else {
                ccg = cg;
            }
            const int c = ccg * 32 + lane;
            const bool col_ok = active && c >= a.c_lo && c < a.c_hi && c < a.n;
            uint32_t vm[4];
    #pragma unroll
            for (int q = 0; q < 4; ++q) vm[q] = col_ok ? half_mask(c - r0 - 32 * q) & s_rows_ok[q] : 0u;
            const bool any_vm = (vm[0] | vm[1] | vm[2] | vm[3]) != 0u;
            if (!__any_sync(full, any_vm)) continue;
            // bound pass: section 0 of the group; full pass: every step of the
            // lane's group (both sections with a split)
            int El = a.tgent[ccg];
            if (a.split && (round || !bound)) El += a.tgentL[ccg];
            const uint4* __restrict__ ep = reinterpret_cast<const uint4*>(a.tent + a.tstart[ccg]) + lane;
            Counter<B> cnt[4];
            if (round) {
                if (!any_vm) El = 0;
                const int Emax = (int)__reduce_max_sync(full, (unsigned)El);
                accumulate128<B, true>(Pb, ep, El, Emax, gq, a.k65536, a.k8 * 2u, cnt);
            } else {
                accumulate128<B, false>(Pb, ep, El, El, gq, a.k65536, a.k8 * 2u, cnt);
            }
            if (a.gstat && any_vm) {
                const int2 ns = *reinterpret_cast<const int2*>(a.nsec + 2 * (int64_t)c);
                if (round) {
                    st_full += (uint32_t)(ns.x + ns.y);
                    ++st_cols;
                } else {
                    st_bound += (uint32_t)ns.x;
                }
            }
            if (round && lane == 0) ++st_rounds;
            uint32_t X[4][B];
    #pragma unroll
            for (int q = 0; q < 4; ++q) cnt[q].planes(X[q]);
            const int tc = col_ok ? a.tcount[c] : 0;
            if (bound && !round) {
                bool alive = false;
    #pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (!vm[q]) continue;
                    if (tc < rb.tmax[q]) {
                        alive = true;
                        continue;
                    }
                    uint32_t gt = 0, eq = full;
    #pragma unroll
                    for (int k = B - 1; k >= 0; --k) {
                        const uint32_t rk = rb.thr[q * kRPlanes + k];
                        gt |= eq & X[q][k] & ~rk;
                        eq &= ~(X[q][k] ^ rk);
                    }
                    if ((gt | eq) & vm[q] & rb.live[q]) alive = true;
                }
                if (alive) {
                    s_q[qn * 32 + lane] = (uint16_t)ccg;
                    ++qn;
                }
                continue;
            }
            // rank >= levels: the hash (the entries lead each read's level list)
            if (any_high) {
                const int nh = col_ok ? a.nhigh[c] : 0;
                const int maxh = (int)__reduce_max_sync(full, (unsigned)nh);
                const uint32_t* __restrict__ rp = a.ent + a.gstart[ccg];
                for (int j = 0; j < maxh; ++j) {
                    const uint4 w = j < nh ? hash_find4(hkeys, hmask, __ldg(rp + ent_at(j, lane)))
                                           : make_uint4(0u, 0u, 0u, 0u);
                    Counter<B>::add_at(X[0], w.x, 0);
                    Counter<B>::add_at(X[1], w.y, 0);
                    Counter<B>::add_at(X[2], w.z, 0);
                    Counter<B>::add_at(X[3], w.w, 0);
                }
            }
    #pragma unroll
            for (int q = 0; q < 4; ++q)
                finish_half<B>(a, ej, X[q], vm[q], r0 + 32 * q, s_tmin[q], s_rowT + 32 * q, c, tc);
        }
    }
    if (a.gstat) {
        const uint32_t b = __reduce_add_sync(full, st_bound), f = __reduce_add_sync(full, st_full);
        const uint32_t k = __reduce_add_sync(full, st_cols);
        if (lane == 0) {
            atomicAdd(a.gstat + 0, (unsigned long long)b);
            atomicAdd(a.gstat + 1, (unsigned long long)f);
            atomicAdd(a.gstat + 2, (unsigned long long)k);
            atomicAdd(a.gstat + 3, (unsigned long long)st_rounds);
        }
    }
}

template <int B>
__global__ void __launch_bounds__(kTileThreads, 1) kmer_tile128_kernel(TileArgs a) {
    extern __shared__ __align__(16) uint4 P128[];   // levels * K4 plane words + 32 guard words
    uint4* P = P128;
    __shared__ uint32_t hkeys[kHashSlots];
    __shared__ uint4 hmask[kHashSlots];
    __shared__ int s_rowT[kRows128];
    __shared__ int s_item[5];
    __shared__ int s_tmin[4], s_any_high;
    __shared__ uint32_t s_rows_ok[4];
    // bound pass: per-row bounds and each warp's stacks of column groups
    __shared__ uint32_t s_rthr[4 * kRPlanes], s_rlive[4];
    __shared__ int s_tmax[4];
    __shared__ uint16_t s_q[kTileWarps * kQDepth * 32];
    __shared__ uint8_t s_qn[kTileWarps * 32], s_qoff[kTileWarps * 32];
    __shared__ int s_next[2];
    const bool queued = a.items != nullptr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int it = 0;; ++it) {
        if (threadIdx.x == 0) {
            if (queued) {
                const unsigned w = atomicAdd(a.queue_head, 1u);
                s_item[3] = (int)w < a.nitems;
                if (s_item[3]) {
                    s_item[0] = a.items[w];
                    s_item[1] = a.item_cstart ? a.item_cstart[w] : 0;
                    s_item[2] = a.item_cend ? a.item_cend[w] : (a.n + 31) / 32;
                    s_item[4] = a.item_job ? a.item_job[w] : -1;
                }
            } else {
                // one row group per x block; the stage's column groups are
                // split evenly over the y blocks
                const int cga = a.c_lo / 32, cgb = (a.c_hi + 31) / 32;
                const int per = (cgb - cga + (int)gridDim.y - 1) / (int)gridDim.y;
                s_item[0] = a.r_lo / kRows128 + blockIdx.x;
                s_item[1] = cga + (int)blockIdx.y * per;
                s_item[2] = min(cgb, s_item[1] + per);
                s_item[3] = it == 0 && s_item[1] < s_item[2];
            }
        }
        __syncthreads();
        if (!s_item[3]) break;
        const int rg = s_item[0], cg0 = s_item[1], cg1 = s_item[2];
        EmitJob ej = emit_job_of(a);
        if (queued && s_item[4] >= 0) {
            const int jb = s_item[4];
            const int4 cj = a.cjob[jb];
            ej.mmin = a.mmin + a.ctbl[jb];
            ej.smin = a.smin + a.ctbl[jb];
            ej.base = cj.x; ej.n = cj.y; ej.A = cj.z; ej.sd = cj.w;
            ej.tag = (uint64_t)jb << 44;
            ej.jcount = a.job_counter + jb;
        }
        __syncthreads();   // every thread has read s_item
        const int rlo = queued ? 0 : a.r_lo, rhi = queued ? a.n : min(a.r_hi, a.n);
        // ---- row group set-up: rows of dense 32-read groups are left to
        // kmer_dense_kernel ----
        if (warp < 4) {
            const int r = rg * kRows128 + warp * 32 + lane;
            const bool ok = r >= rlo && r < rhi && !a.dense_group[r >> 5];
            const int tr = ok ? a.tcount[r] : INT_MAX;
            s_rowT[warp * 32 + lane] = tr;
            const unsigned okm = __ballot_sync(0xffffffffu, ok);
            const int tm = (int)__reduce_min_sync(0xffffffffu, (unsigned)tr);
            if (lane == 0) { s_tmin[warp] = tm; s_rows_ok[warp] = okm; }
            if (warp == 0 && lane == 0) {
                s_any_high = 0;
                s_next[0] = 0;
                s_next[1] = 0;
            }
            if (a.bound) {
                // R = mmin[T] - (T - a0), at least 0; rows without a passing
                // count (mmin = 0xFFFF) are not live
                const int a0 = ok ? a.nsec[2 * (int64_t)r] : 0;
                const int mm = ok ? (int)ej.mmin[tr] : 0xFFFF;
                const bool live = ok && mm != 0xFFFF;
                const int R = live ? max(0, mm - (tr - a0)) : 0;
#pragma unroll
                for (int k = 0; k < kRPlanes; ++k) {
                    const unsigned pl = __ballot_sync(0xffffffffu, (R >> k) & 1);
                    if (lane == 0) s_rthr[warp * kRPlanes + k] = pl;
                }
                const unsigned lv = __ballot_sync(0xffffffffu, live);
                const int tmx = (int)__reduce_max_sync(0xffffffffu, ok ? (unsigned)tr : 0u);
                if (lane == 0) { s_rlive[warp] = lv; s_tmax[warp] = tmx; }
            }
        }
        const int words = a.levels * (int)a.K4;   // + 32 zero guard words after the planes
        for (int i = threadIdx.x; i < words + 32; i += kTileThreads) P[i] = make_uint4(0, 0, 0, 0);
        for (int i = threadIdx.x; i < kHashSlots; i += kTileThreads) {
            hkeys[i] = kSentinel;
            hmask[i] = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncthreads();
        uint32_t* Pw = reinterpret_cast<uint32_t*>(P);
        uint32_t* hmw = reinterpret_cast<uint32_t*>(hmask);
        const uint32_t limit = (uint32_t)words;
        for (int b = warp; b < kRows128; b += kTileWarps) {
            if (!((s_rows_ok[b >> 5] >> (b & 31)) & 1u)) continue;
            const int r = rg * kRows128 + b;
            const uint32_t* src = a.ent + a.gstart[r >> 5];
            const int T = s_rowT[b];
            const uint32_t bit = 1u << (b & 31);
            const int quarter = b >> 5;
            for (int e = lane; e < T; e += 32) {
                const uint32_t idx = src[ent_at(e, r & 31)];
                if (idx < limit) {
                    atomicOr(&Pw[4 * idx + quarter], bit);
                } else {
                    // high-level entry: open addressing; the host guarantees
                    // the group holds at most kHashMaxKeys of them
                    uint32_t h = hash_slot(idx);
                    for (int probe = 0; probe < kHashSlots; ++probe) {
                        const uint32_t old = atomicCAS(&hkeys[h], kSentinel, idx);
                        if (old == kSentinel || old == idx) {
                            atomicOr(&hmw[4 * h + quarter], bit);
                            break;
                        }
                        h = (h + 1) & (kHashSlots - 1);
                    }
                    s_any_high = 1;
                }
            }
        }
        __syncthreads();
        const RowBound rb{s_rthr, s_rlive, s_tmax};
        const Stacks sk{s_q, s_qn, s_qoff, s_next};
        tile_columns128<B>(a, ej, P, hkeys, hmask, s_any_high != 0, rg, s_rows_ok, s_tmin, s_rowT,
                           rb, sk, max(cg0, 4 * rg), cg1);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// K = 8.  The reference's merge for K = 8 gives
//     m = minsum(H) + [same] * minsum(L)
// (H = K-mers >= 0x8000, L = the rest; kmerMain.cpp:275-278 against
// kmerKernel.cu:37-45), so the two halves are counted apart.  [same] holds
// when the two reads' H keys (largest H K-mer and its count, or none) agree.
// Both K = 8 tile kernels own 32 row reads per block and hold one plane of
// 32-bit words in shared memory: the word of a K-mer (H: K-mer - 0x8000, L:
// K-mer; 32,768 words plus 32 guard words, 128 KB) has the bit of each row
// read with a first occurrence of it; repeated occurrences sit in a shared
// hash.  A lane owns one column read and gathers one word per step of the
// column group's scheduled stream (H and L streams, both by 32-bit bank):
// one LOP3 of the carry-save tree counts 32 rows.
//   * kmer_tile8h_kernel (batched form): the pairs whose H keys differ, with
//     the reads in H-key order all pairs outside the key groups: H only.
//   * kmer_tile8_kernel: H and then L with the plane refilled in between,
//     the H sums of up to kGroups8 column groups per warp kept in registers;
//     the batched form runs it over each row group's same-key column range,
//     the staged form over every pair of a stage.
// ---------------------------------------------------------------------------
constexpr int kRows8 = 32;
constexpr int kPlaneH = 32768 + 32;    // 32-bit plane words: K-mers + guard words
constexpr size_t kSmem8 = (size_t)kPlaneH * 4;
constexpr int kTile8HThreads = 1024;   // 32 warps: the stream loads' latency is hidden by warps
constexpr int kTile8HWarps = kTile8HThreads / 32;
// two-phase kernel: 32 warps while two groups' H sums fit 64 registers
// (counts of 9 bits and below), else 16 warps
template <int B>
constexpr int tile8_threads() { return B <= 9 ? 1024 : 512; }
constexpr int kGroups8 = 2;            // column groups per warp and round (two-phase kernel)

__device__ __noinline__ uint32_t hash_find8(const uint32_t* hkeys, const uint32_t* hmask,
                                            uint32_t key) {
    uint32_t h = hash_slot(key);
    for (int probe = 0; probe < kHashSlots; ++probe) {
        const uint32_t k = hkeys[h];
        if (k == key) return hmask[h];
        if (k == kSentinel) return 0u;
        h = (h + 1) & (kHashSlots - 1);
    }
    return 0u;
}

// 16 scheduled entries of one stream: their plane words into the counter;
// returns the weight-16 carry.
template <int B>
__device__ __forceinline__ uint32_t gather8h_c16(const uint32_t* __restrict__ plane, uint4 q0, uint4 q1,
                                                 Counter<B>& cnt) {
    const uint32_t x[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
    uint32_t w[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        w[2 * k] = plane[x[k] & 0xFFFFu];
        w[2 * k + 1] = plane[x[k] >> 16];
    }
    return cnt.add16(w);
}

// A column's stream (E steps, a multiple of 16) against the plane: two
// 16-entry batches per carry chain, the next pair's first batch in flight.
// E is the column group's step count, the same for every lane, so the
// second batch's branch does not diverge.
template <int B>
__device__ __forceinline__ void phase8h(const uint32_t* __restrict__ plane, const uint4* ep, int E,
                                        uint32_t* X) {
    const uint4 guard = make_uint4(0x80008000u, 0x80008000u, 0x80008000u, 0x80008000u);
    Counter<B> cnt;
    cnt.clear();
    uint4 a0 = 0 < E ? __ldg(ep) : guard, a1 = 0 < E ? __ldg(ep + 32) : guard;
    for (int e = 0; e < E; e += 32) {
        const bool two = e + 16 < E;
        const int ob = ((e + 16) >> 3) * 32, on = ((e + 32) >> 3) * 32;
        const uint4 b0 = two ? __ldg(ep + ob) : guard, b1 = two ? __ldg(ep + ob + 32) : guard;
        const uint4 n0 = e + 32 < E ? __ldg(ep + on) : guard, n1 = e + 32 < E ? __ldg(ep + on + 32) : guard;
        const uint32_t ca = gather8h_c16<B>(plane, a0, a1, cnt);
        if (two) cnt.add_sixteens2(ca, gather8h_c16<B>(plane, b0, b1, cnt));
        else cnt.add_sixteens1(ca);
        a0 = n0; a1 = n1;
    }
    cnt.planes(X);
}

// Count bound of the pairs without [same], whose m = minsum(H) <= min(|H_a|,
// |H_b|): such a pair passes only if m >= mmin[min(Ta, Tb)], i.e. only if
// the shorter read r (ties: either) has |H_r| >= mmin[T_r].  A read with
// that property is H-heavy; a pair of two reads that are not can be skipped
// without a gather.  |H| is at most the read's H section (first
// occurrences) plus its repeated entries.
__device__ __forceinline__ bool heavy8(const TileArgs& a, int r) {
    const int h = a.nsec[2 * (int64_t)r] + a.nhigh[r];
    return h >= (int)a.mmin[a.tcount[r]];
}

// phase8h with a stream length per lane (El steps; lanes past theirs read
// the guard word) and the warp's largest, Emax.
template <int B>
__device__ __forceinline__ void phase8h_lane(const uint32_t* __restrict__ plane, const uint4* ep, int El,
                                             int Emax, uint32_t* X) {
    const uint4 guard = make_uint4(0x80008000u, 0x80008000u, 0x80008000u, 0x80008000u);
    auto ld = [&](int step) { return step < El ? __ldg(ep + (step >> 3) * 32) : guard; };
    Counter<B> cnt;
    cnt.clear();
    uint4 a0 = ld(0), a1 = ld(8);
    for (int e = 0; e < Emax; e += 32) {
        const bool two = e + 16 < Emax;
        const uint4 b0 = two ? ld(e + 16) : guard, b1 = two ? ld(e + 24) : guard;
        const uint4 n0 = ld(e + 32), n1 = ld(e + 40);
        const uint32_t ca = gather8h_c16<B>(plane, a0, a1, cnt);
        if (two) cnt.add_sixteens2(ca, gather8h_c16<B>(plane, b0, b1, cnt));
        else cnt.add_sixteens1(ca);
        a0 = n0; a1 = n1;
    }
    cnt.planes(X);
}

// Per-block row state of both K = 8 kernels.
struct Rows8 {
    int rowT[kRows8];            // tuple counts (INT_MAX for rows not taken)
    uint32_t keyv[kRows8];       // the rows' distinct H keys ...
    uint32_t keym[kRows8];       // ... and the rows holding each
    int nkeys, tmin, rep;
    uint32_t rows_ok;
    int heavy;                   // some row taken is H-heavy
};

// Warp 0: the row group's rows in [rlo, rhi), their tuple counts and keys.
__device__ __forceinline__ void rows8_setup(const TileArgs& a, Rows8& rs, int rg, int rlo, int rhi) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int r = rg * kRows8 + lane;
    const bool ok = r >= rlo && r < rhi && r < a.n && !a.dense_group[rg];
    const int tr = ok ? a.tcount[r] : INT_MAX;
    const uint32_t hr = ok ? a.hinfo[r] : 0u;
    rs.rowT[lane] = tr;
    const unsigned okm = __ballot_sync(full, ok);
    const int tm = (int)__reduce_min_sync(full, (unsigned)tr);
    const unsigned rowsk = __match_any_sync(full, hr) & okm;
    const bool leader = ok && lane == __ffs(rowsk) - 1;
    const unsigned lm = __ballot_sync(full, leader);
    if (leader) {
        const int k = __popc(lm & ((1u << lane) - 1u));
        rs.keyv[k] = hr;
        rs.keym[k] = rowsk;
    }
    const bool hv = __any_sync(full, ok && heavy8(a, r));
    if (lane == 0) { rs.tmin = tm; rs.rows_ok = okm; rs.nkeys = __popc(lm); rs.heavy = hv; }
}

// The rows with the same H key as column key hc ([same] per row).
__device__ __forceinline__ uint32_t same8(const Rows8& rs, int nkeys, uint32_t hc) {
    uint32_t same = 0;
    for (int k = 0; k < nkeys; ++k) same |= rs.keyv[k] == hc ? rs.keym[k] : 0u;
    return same;
}

// All threads: zero the plane and the hash, then put the first occurrences
// of the rows' kH-section K-mers into the plane and their repeated ones into
// the hash (rs.rep set when there are any).  A read's level list holds its
// repeated entries first, then the H section, then the L section.  Ends
// with a barrier.
template <bool kH>
__device__ void fill8(const TileArgs& a, Rows8& rs, int rg, uint32_t* plane, uint32_t* hkeys,
                      uint32_t* hmask, int threads) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = threads >> 5;
    __syncthreads();   // the previous users of the plane and the hash are done
    uint4* P4 = reinterpret_cast<uint4*>(plane);
    for (int i = threadIdx.x; i < (int)(kSmem8 / 16); i += threads) P4[i] = make_uint4(0, 0, 0, 0);
    for (int i = threadIdx.x; i < kHashSlots; i += threads) { hkeys[i] = kSentinel; hmask[i] = 0u; }
    if (threadIdx.x == 0) rs.rep = 0;
    __syncthreads();
    const uint32_t* src = a.ent + a.gstart[rg];
    for (int b = warp; b < kRows8; b += warps) {
        if (!((rs.rows_ok >> b) & 1u)) continue;
        const int r = rg * kRows8 + b;
        const int nh = a.nhigh[r], nH = a.nsec[2 * (int64_t)r];
        // H: the repeated entries and the H section; L: the repeated entries
        // and the L section (positions past the H section)
        const int e_end = kH ? nh + nH : rs.rowT[b] - nH;
        for (int i = lane; i < e_end; i += 32) {
            const int e = kH || i < nh ? i : i + nH;
            const uint32_t idx = src[ent_at(e, b)];
            const bool hk = (idx & 0xFFFFu) >= 0x8000u;
            if (hk != kH) continue;
            if (idx < 65536u) {
                atomicOr(&plane[kH ? idx - 0x8000u : idx], 1u << b);
            } else {
                uint32_t h = hash_slot(idx);
                for (int probe = 0; probe < kHashSlots; ++probe) {
                    const uint32_t old = atomicCAS(&hkeys[h], kSentinel, idx);
                    if (old == kSentinel || old == idx) {
                        atomicOr(&hmask[h], 1u << b);
                        break;
                    }
                    h = (h + 1) & (kHashSlots - 1);
                }
                rs.rep = 1;
            }
        }
    }
    __syncthreads();
}

// One column's kH-section sums against the rows: the scheduled stream, then
// its repeated entries looked up in the hash.  Whole warps call it.
template <int B, bool kH>
__device__ __forceinline__ void column8(const TileArgs& a, const uint32_t* plane, const uint32_t* hkeys,
                                        const uint32_t* hmask, bool any_rep, int q, int c, bool okc,
                                        uint32_t* X) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint16_t* st = a.tent + a.tstart[q] + (kH ? 0 : 32LL * a.tgent[q]);
    phase8h<B>(plane, reinterpret_cast<const uint4*>(st) + lane, kH ? a.tgent[q] : a.tgentL[q], X);
    if (any_rep) {
        const int nh = okc ? a.nhigh[c] : 0;
        const int maxh = (int)__reduce_max_sync(full, (unsigned)nh);
        const uint32_t* rp = a.ent + a.gstart[q];
        for (int j = 0; j < maxh; ++j) {
            uint32_t w = 0;
            if (j < nh) {
                const uint32_t key = __ldg(rp + ent_at(j, lane));
                if (((key & 0xFFFFu) >= 0x8000u) == kH) w = hash_find8(hkeys, hmask, key);
            }
            Counter<B>::add_at(X, w, 0);
        }
    }
}

// Threshold and emission of one column's 32 row pairs (vmask: the pairs to
// consider): a lower bound of mmin first, then exact per candidate.
template <int B>
__device__ __forceinline__ void emit8(const TileArgs& a, const Rows8& rs, const uint32_t* X, uint32_t vmask,
                                      int r0, int c, int tc) {
    const uint32_t lo = a.smin[min(rs.tmin, tc)];
    uint32_t cand = 0;
    if (vmask && lo < (1u << B)) {
        uint32_t gt = 0, eq = 0xffffffffu;
#pragma unroll
        for (int k = B - 1; k >= 0; --k) {
            const uint32_t bit = ((lo >> k) & 1u) ? 0xffffffffu : 0u;
            gt |= eq & X[k] & ~bit;
            eq &= ~(X[k] ^ bit);
        }
        cand = (gt | eq) & vmask;
    }
    while (__any_sync(0xffffffffu, cand)) {
        bool pass = false;
        int r = 0, m = 0, mn = 1;
        if (cand) {
            const int bit = __ffs(cand) - 1;
            cand &= cand - 1;
#pragma unroll
            for (int k = 0; k < B; ++k) m |= (int)((X[k] >> bit) & 1u) << k;
            r = r0 + bit;
            mn = min(rs.rowT[bit], tc);
            pass = m >= (int)a.mmin[mn];
        }
        emit(a.counter, a.keys, a.vals, a.cap, a.n, a.A, a.stage_dim, a.perm, a.olo, a.ohi, pass, r, c, m, mn);
    }
}

template <int B>
__global__ void __launch_bounds__(kTile8HThreads, 1) kmer_tile8h_kernel(TileArgs a) {
    extern __shared__ __align__(16) uint32_t plane[];
    __shared__ uint32_t hkeys[kHashSlots];
    __shared__ uint32_t hmask[kHashSlots];
    __shared__ Rows8 rs;
    __shared__ int s_item;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned full = 0xffffffffu;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned w = atomicAdd(a.queue_head, 1u);
            s_item = (int)w < a.nitems ? a.items[w] : -1;
        }
        __syncthreads();
        const int rg = s_item;
        if (rg < 0) break;
        const int r0 = rg * kRows8;
        if (warp == 0) rows8_setup(a, rs, rg, 0, a.n);
        fill8<true>(a, rs, rg, plane, hkeys, hmask, kTile8HThreads);
        const bool any_rep = rs.rep != 0;
        const uint32_t rows_ok = rs.rows_ok;
        const int nkeys = rs.nkeys;
        for (int q = rg + warp; q < a.ngroups; q += kTile8HWarps) {
            const int c = 32 * q + lane;
            const bool okc = c < a.n;
            const uint32_t same = same8(rs, nkeys, okc ? a.hinfo[c] : 0u);
            // pairs with [same] belong to the two-phase kernel; the others
            // can pass only where the row group or the column is H-heavy
            const bool hv = okc && (rs.heavy || heavy8(a, c));
            const uint32_t vmask = hv ? (half_mask(c - r0) & rows_ok & ~same) : 0u;
            if (!__any_sync(full, vmask)) continue;
            uint32_t X[B];
            column8<B, true>(a, plane, hkeys, hmask, any_rep, q, c, okc, X);
            emit8<B>(a, rs, X, vmask, r0, c, okc ? a.tcount[c] : 0);
        }
        __syncthreads();
    }
}

template <int B>
__global__ void __launch_bounds__(tile8_threads<B>(), 1) kmer_tile8_kernel(TileArgs a) {
    constexpr int kTile8Threads = tile8_threads<B>();
    constexpr int kTile8Warps = kTile8Threads / 32;
    extern __shared__ __align__(16) uint32_t plane[];
    __shared__ uint32_t hkeys[kHashSlots];
    __shared__ uint32_t hmask[kHashSlots];
    __shared__ Rows8 rs;
    __shared__ int s_item[4];
    // bound of the pairs with [same] after their H sums: bit planes of the
    // rows' R = mmin[T] - |L| (at least 0) and of their tuple counts
    __shared__ uint32_t s_rthr[kRPlanes], s_rt[kRPlanes], s_rlive;
    const bool queued = a.items != nullptr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned full = 0xffffffffu;
    for (int it = 0;; ++it) {
        if (threadIdx.x == 0) {
            if (queued) {
                const unsigned w = atomicAdd(a.queue_head, 1u);
                s_item[3] = (int)w < a.nitems;
                if (s_item[3]) {
                    s_item[0] = a.items[w];
                    s_item[1] = a.item_q ? a.item_q[w].x : 0;
                    s_item[2] = a.item_q ? a.item_q[w].y : a.ngroups;
                }
            } else {
                s_item[0] = a.r_lo / kRows8 + blockIdx.x;
                s_item[1] = a.c_lo / 32;
                s_item[2] = (a.c_hi + 31) / 32;
                s_item[3] = it == 0;
            }
        }
        __syncthreads();
        if (!s_item[3]) break;
        const int rg = s_item[0], q0 = s_item[1], q1 = s_item[2];
        const int rlo = queued ? 0 : a.r_lo, rhi = queued ? a.n : min(a.r_hi, a.n);
        const int r0 = rg * kRows8;
        if (warp == 0) {
            rows8_setup(a, rs, rg, rlo, rhi);
            __syncwarp();
            // |L| is at most the L section plus the repeated entries
            const int r = r0 + lane;
            const bool ok = (rs.rows_ok >> lane) & 1u;
            const int tr = ok ? a.tcount[r] : 0;
            const int mm = ok ? (int)a.mmin[tr] : 0xFFFF;
            const int lb = ok ? a.nsec[2 * (int64_t)r + 1] + a.nhigh[r] : 0;
            const int R = mm != 0xFFFF ? max(0, mm - lb) : 0;
#pragma unroll
            for (int k = 0; k < kRPlanes; ++k) {
                const unsigned pr = __ballot_sync(full, (R >> k) & 1), pt = __ballot_sync(full, (tr >> k) & 1);
                if (lane == 0) { s_rthr[k] = pr; s_rt[k] = pt; }
            }
            const unsigned lv = __ballot_sync(full, ok && mm != 0xFFFF);
            if (lane == 0) s_rlive = lv;
        }
        __syncthreads();
        const uint32_t rows_ok = rs.rows_ok;
        const int nkeys = rs.nkeys;
        // rounds of kTile8Warps x kGroups8 column groups: H sums, then the
        // plane refilled with L, then L sums where [same] holds, and emission
        for (int base = max(q0, rg); base < q1; base += kTile8Warps * kGroups8) {
            fill8<true>(a, rs, rg, plane, hkeys, hmask, kTile8Threads);
            const bool rep_h = rs.rep != 0;
            uint32_t XH[kGroups8][B], same[kGroups8], vm[kGroups8];
            bool any_same = false;
#pragma unroll
            for (int g = 0; g < kGroups8; ++g) {
                const int q = base + warp * kGroups8 + g;
                const int c = 32 * q + lane;
                const bool okc = q < q1 && c >= a.c_lo && c < a.c_hi && c < a.n;
                same[g] = same8(rs, nkeys, okc ? a.hinfo[c] : 0u);
                // same_only: the H-only kernel has taken the pairs without
                // [same]; those can pass only where the row group or the
                // column is H-heavy
                const bool hv = okc && !a.same_only && (rs.heavy || heavy8(a, c));
                vm[g] = okc ? (half_mask(c - r0) & rows_ok & (same[g] | (hv ? 0xffffffffu : 0u))) : 0u;
#pragma unroll
                for (int k = 0; k < B; ++k) XH[g][k] = 0u;
                if (__any_sync(full, vm[g])) column8<B, true>(a, plane, hkeys, hmask, rep_h, q, c, okc, XH[g]);
                // a pair with [same] has m = mH + mL <= mH + |L_r|: with Tc >=
                // Tr it can pass only if mH >= R_r; rows longer than the
                // column keep their pairs
                const uint32_t sv = same[g] & vm[g];
                if (sv) {
                    const uint32_t tc = (uint32_t)(okc ? a.tcount[c] : 0);
                    uint32_t gt = 0, eq = full, tgt = 0, teq = full;
#pragma unroll
                    for (int k = kRPlanes - 1; k >= 0; --k) {
                        if (k < B) {
                            const uint32_t rk = s_rthr[k];
                            gt |= eq & XH[g][k] & ~rk;
                            eq &= ~(XH[g][k] ^ rk);
                        }
                        const uint32_t tk = s_rt[k], cb = ((tc >> k) & 1u) ? full : 0u;
                        tgt |= teq & tk & ~cb;
                        teq &= ~(tk ^ cb);
                    }
                    const uint32_t alive = sv & (((gt | eq) & s_rlive) | tgt);
                    vm[g] = (vm[g] & ~same[g]) | alive;
                }
                any_same |= (same[g] & vm[g]) != 0u;
            }
            // the L phase only where some pair of the block has [same]
            const bool blk_same = __syncthreads_or(any_same) != 0;
            bool rep_l = false;
            if (blk_same) {
                fill8<false>(a, rs, rg, plane, hkeys, hmask, kTile8Threads);
                rep_l = rs.rep != 0;
            }
#pragma unroll
            for (int g = 0; g < kGroups8; ++g) {
                if (!__any_sync(full, vm[g])) continue;
                const int q = base + warp * kGroups8 + g;
                const int c = 32 * q + lane;
                const bool okc = q < q1 && c >= a.c_lo && c < a.c_hi && c < a.n;
                uint32_t XL[B];
#pragma unroll
                for (int k = 0; k < B; ++k) XL[k] = 0u;
                if (blk_same && __any_sync(full, same[g] & vm[g]))
                    column8<B, false>(a, plane, hkeys, hmask, rep_l, q, c, okc, XL);
                // X = XH + (XL & same), bit-sliced
                uint32_t X[B];
                uint32_t carry = 0;
#pragma unroll
                for (int k = 0; k < B; ++k) {
                    const uint32_t y = XL[k] & same[g];
                    X[k] = XH[g][k] ^ y ^ carry;
                    carry = (XH[g][k] & y) | (carry & (XH[g][k] ^ y));
                }
                emit8<B>(a, rs, X, vm[g], r0, c, okc ? a.tcount[c] : 0);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Same-key pass with queued L sums (batched form, K = 8).  The two-phase
// kernel refills its plane twice per round of 64 column groups, and every
// warp waits at those barriers for the few that still have L work.  This
// kernel fills the H plane once per row group and takes the H sums of every
// column group of the row group's same-key range; a lane whose [same] pairs
// survive the bound (mH >= R_r, or a row longer than the column) stores its
// H sums, its alive rows and its column group in its own lane slot of the
// block's queue (global scratch, at most one item per slot and column
// group).  Then the plane is filled with L once, and rounds take the i-th
// item of every slot: each lane keeps its lane index, so the L stream's
// bank schedule still holds, and lanes past their stream read the guard.
// ---------------------------------------------------------------------------
template <int B>
__device__ __forceinline__ void column8L_lane(const TileArgs& a, const uint32_t* plane, const uint32_t* hkeys,
                                              const uint32_t* hmask, bool any_rep, int q, int c, bool okc,
                                              uint32_t* X) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint16_t* st = a.tent + a.tstart[q] + 32LL * a.tgent[q];
    const int El = okc ? a.tgentL[q] : 0;
    const int Emax = (int)__reduce_max_sync(full, (unsigned)El);
    phase8h_lane<B>(plane, reinterpret_cast<const uint4*>(st) + lane, El, Emax, X);
    if (any_rep) {
        const int nh = okc ? a.nhigh[c] : 0;
        const int maxh = (int)__reduce_max_sync(full, (unsigned)nh);
        const uint32_t* rp = a.ent + a.gstart[q];
        for (int j = 0; j < maxh; ++j) {
            uint32_t w = 0;
            if (j < nh) {
                const uint32_t key = __ldg(rp + ent_at(j, lane));
                if ((key & 0xFFFFu) < 0x8000u) w = hash_find8(hkeys, hmask, key);
            }
            Counter<B>::add_at(X, w, 0);
        }
    }
}

template <int B>
__global__ void __launch_bounds__(tile8_threads<B>(), 1) kmer_tile8s_kernel(TileArgs a) {
    constexpr int kThreads = tile8_threads<B>();
    constexpr int W = B + 2;   // queue item: H sums (B planes), alive rows, column group
    extern __shared__ __align__(16) uint32_t plane[];
    __shared__ uint32_t hkeys[kHashSlots];
    __shared__ uint32_t hmask[kHashSlots];
    __shared__ Rows8 rs;
    __shared__ int s_item[3], s_next[2], s_qn[32];
    __shared__ uint32_t s_rthr[kRPlanes], s_rt[kRPlanes], s_rlive;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned full = 0xffffffffu;
    uint32_t* qb = a.sq + (int64_t)blockIdx.x * a.sq_cap * W * 32;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned w = atomicAdd(a.queue_head, 1u);
            const bool ok = (int)w < a.nitems;
            s_item[0] = ok ? a.items[w] : -1;
            s_item[1] = ok ? a.item_q[w].x : 0;
            s_item[2] = ok ? a.item_q[w].y : 0;
            s_next[0] = 0;
            s_next[1] = 0;
        }
        if (threadIdx.x < 32) s_qn[threadIdx.x] = 0;
        __syncthreads();
        const int rg = s_item[0];
        if (rg < 0) break;
        const int q0 = max(s_item[1], rg), q1 = s_item[2];
        const int r0 = rg * kRows8;
        if (warp == 0) {
            rows8_setup(a, rs, rg, 0, a.n);
            __syncwarp();
            // R = mmin[T] - |L| (at least 0), |L| at most the L section plus
            // the repeated entries; the rows' tuple counts
            const int r = r0 + lane;
            const bool ok = (rs.rows_ok >> lane) & 1u;
            const int tr = ok ? a.tcount[r] : 0;
            const int mm = ok ? (int)a.mmin[tr] : 0xFFFF;
            const int lb = ok ? a.nsec[2 * (int64_t)r + 1] + a.nhigh[r] : 0;
            const int R = mm != 0xFFFF ? max(0, mm - lb) : 0;
#pragma unroll
            for (int k = 0; k < kRPlanes; ++k) {
                const unsigned pr = __ballot_sync(full, (R >> k) & 1), pt = __ballot_sync(full, (tr >> k) & 1);
                if (lane == 0) { s_rthr[k] = pr; s_rt[k] = pt; }
            }
            const unsigned lv = __ballot_sync(full, ok && mm != 0xFFFF);
            if (lane == 0) s_rlive = lv;
        }
        fill8<true>(a, rs, rg, plane, hkeys, hmask, kThreads);   // begins and ends with a barrier
        const bool rep_h = rs.rep != 0;
        const uint32_t rows_ok = rs.rows_ok;
        const int nkeys = rs.nkeys;
        // H sums of every column group of the range; survivors of the bound
        // go on the queue
        for (;;) {
            int v = 0;
            if (lane == 0) v = atomicAdd(&s_next[0], 1);
            const int q = q0 + __shfl_sync(full, v, 0);
            if (q >= q1) break;
            const int c = 32 * q + lane;
            const bool okc = c < a.n;
            const uint32_t same = same8(rs, nkeys, okc ? a.hinfo[c] : 0u);
            const uint32_t vm = okc ? (half_mask(c - r0) & rows_ok & same) : 0u;
            if (!__any_sync(full, vm)) continue;
            uint32_t XH[B];
            column8<B, true>(a, plane, hkeys, hmask, rep_h, q, c, okc, XH);
            if (vm) {
                const uint32_t tc = (uint32_t)a.tcount[c];
                uint32_t gt = 0, eq = full, tgt = 0, teq = full;
#pragma unroll
                for (int k = kRPlanes - 1; k >= 0; --k) {
                    if (k < B) {
                        const uint32_t rk = s_rthr[k];
                        gt |= eq & XH[k] & ~rk;
                        eq &= ~(XH[k] ^ rk);
                    }
                    const uint32_t tk = s_rt[k], cb = ((tc >> k) & 1u) ? full : 0u;
                    tgt |= teq & tk & ~cb;
                    teq &= ~(tk ^ cb);
                }
                const uint32_t alive = vm & (((gt | eq) & s_rlive) | tgt);
                if (alive) {
                    const int pos = atomicAdd(&s_qn[lane], 1);
                    uint32_t* it = qb + (int64_t)pos * W * 32 + lane;
#pragma unroll
                    for (int k = 0; k < B; ++k) it[k * 32] = XH[k];
                    it[B * 32] = alive;
                    it[(B + 1) * 32] = (uint32_t)q;
                }
            }
        }
        __syncthreads();
        const int pmax = (int)__reduce_max_sync(full, (unsigned)s_qn[lane]);
        if (pmax > 0) {
            fill8<false>(a, rs, rg, plane, hkeys, hmask, kThreads);
            const bool rep_l = rs.rep != 0;
            for (;;) {
                int v = 0;
                if (lane == 0) v = atomicAdd(&s_next[1], 1);
                const int i = __shfl_sync(full, v, 0);
                if (i >= pmax) break;
                const bool active = i < s_qn[lane];
                uint32_t XH[B], alive = 0;
                int q = 0;
                if (active) {
                    const uint32_t* it = qb + (int64_t)i * W * 32 + lane;
#pragma unroll
                    for (int k = 0; k < B; ++k) XH[k] = it[k * 32];
                    alive = it[B * 32];
                    q = (int)it[(B + 1) * 32];
                } else {
#pragma unroll
                    for (int k = 0; k < B; ++k) XH[k] = 0u;
                }
                const int c = 32 * q + lane;
                const bool okc = active && c < a.n;
                uint32_t XL[B];
                column8L_lane<B>(a, plane, hkeys, hmask, rep_l, q, c, okc, XL);
                // X = XH + (XL & alive), bit-sliced
                uint32_t X[B];
                uint32_t carry = 0;
#pragma unroll
                for (int k = 0; k < B; ++k) {
                    const uint32_t y = XL[k] & alive;
                    X[k] = XH[k] ^ y ^ carry;
                    carry = (XH[k] & y) | (carry & (XH[k] ^ y));
                }
                emit8<B>(a, rs, X, alive, r0, c, okc ? a.tcount[c] : 0);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Exact dense-table kernel: one row read per block with its full count
// table (two 16-bit counts per word) in shared memory; one column per
// thread walks its level entries (t, kmer) and counts [cnt_row[kmer] > t].
// Covers any K <= 8 and any multiplicity.  For K = 8 the reference's merge
// compares unsigned values over lists sorted as signed shorts
// (kmerMain.cpp:275-278 vs kmerKernel.cu:37-45), which yields
//     m = minsum(H) + [same] * minsum(L)
// with H = K-mers >= 0x8000, L = the rest, and [same] true iff both reads
// have no H K-mer or both have the same largest H K-mer with the same
// multiplicity.  The kernel keeps the two partial sums apart for that.
// ---------------------------------------------------------------------------
struct DenseArgs {
    const uint8_t* seq;
    const int64_t* off;
    const uint32_t* ent;
    const int64_t* gstart;
    const int32_t* tcount;
    const uint32_t* hinfo;
    const uint16_t* mmin;
    int n, K;
    int r_lo, r_hi, c_lo, c_hi;
    int A, stage_dim;
    const uint8_t* dense_group;   // nullptr: every row
    unsigned long long* counter;
    uint64_t* keys;
    uint32_t* vals;
    int64_t cap;
    const int32_t* perm;          // as in TileArgs
    int olo, ohi;
};

__global__ void __launch_bounds__(256) kmer_dense_kernel(DenseArgs a) {
    extern __shared__ uint32_t hist[];
    const uint32_t K4 = 1u << (2 * a.K);
    const int hwords = (int)((K4 + 1) / 2);
    for (int i = threadIdx.x; i < hwords; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (int r = a.r_lo + blockIdx.x; r < a.r_hi && r < a.n; r += gridDim.x) {
        if (a.dense_group && !a.dense_group[r >> 5]) continue;   // uniform per block
        const int Tr = a.tcount[r];
        const uint8_t* s = a.seq + a.off[r];
        for (int p = threadIdx.x; p < Tr; p += blockDim.x) {
            const uint32_t v = kmer_at(s, p, a.K);
            atomicAdd(&hist[v >> 1], 1u << ((v & 1u) * 16u));
        }
        __syncthreads();
        const uint32_t hr = a.hinfo[r];
        const int cstart = max(a.c_lo, r + 1);
        const int cend = min(a.c_hi, a.n);
        // whole warps iterate together so that emit() sees 32 lanes
        const int span = cend - cstart;
        const int rounds = span > 0 ? (span + blockDim.x - 1) / blockDim.x : 0;
        for (int q = 0; q < rounds; ++q) {
            const int c = cstart + q * blockDim.x + threadIdx.x;
            const bool ok = c < cend;
            int m = 0, mn = 1;
            bool pass = false;
            if (ok) {
                const int Tc = a.tcount[c];
                const uint32_t* ep = a.ent + a.gstart[c >> 5];
                const int cl = c & 31;
                int sum_lo = 0, sum_hi = 0;
                for (int e = 0; e < Tc; ++e) {
                    const uint32_t idx = __ldg(ep + ent_at(e, cl));
                    const uint32_t t = idx >> (2 * a.K), v = idx & (K4 - 1u);
                    const uint32_t cnt = (hist[v >> 1] >> ((v & 1u) * 16u)) & 0xFFFFu;
                    const int hit = cnt > t;
                    if (v >= 0x8000u) sum_hi += hit; else sum_lo += hit;
                }
                if (a.K == 8) {
                    const uint32_t hc = a.hinfo[c];
                    const bool same = (hr == 0 && hc == 0) || (hr != 0 && hr == hc);
                    m = sum_hi + (same ? sum_lo : 0);
                } else {
                    m = sum_hi + sum_lo;
                }
                mn = min(Tr, Tc);
                pass = m >= (int)a.mmin[mn];
            }
            emit(a.counter, a.keys, a.vals, a.cap, a.n, a.A, a.stage_dim, a.perm, a.olo, a.ohi, pass, r, c, m, mn);
        }
        __syncthreads();
        for (int p = threadIdx.x; p < Tr; p += blockDim.x) hist[kmer_at(s, p, a.K) >> 1] = 0;
        __syncthreads();
    }
}

__global__ void kmer_decode_kernel(const uint64_t* __restrict__ keys,
                                   const uint32_t* __restrict__ vals, int64_t count, int n,
                                   int2* __restrict__ pairs, float* __restrict__ dists) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint64_t k = keys[i];
    const uint64_t rc = k % ((uint64_t)n * (uint64_t)n);
    pairs[i] = make_int2((int)(rc / (uint64_t)n), (int)(rc % (uint64_t)n));
    if (dists) dists[i] = __uint_as_float(vals[i]);
}

// Cohort survivors after the sort: job in key bits 44 and up, then the
// job's own stage key; pairs come out at cohort positions (base added).
__global__ void kmer_decode_cohort_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                          int64_t count, const int4* __restrict__ cjob,
                                          int2* __restrict__ pairs, float* __restrict__ dists) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint64_t k = keys[i];
    const int4 cj = cjob[(int)(k >> 44)];
    const uint64_t n = (uint64_t)cj.y;
    const uint64_t rc = (k & ((1ull << 44) - 1)) % (n * n);
    pairs[i] = make_int2(cj.x + (int)(rc / n), cj.x + (int)(rc % n));
    if (dists) dists[i] = __uint_as_float(vals[i]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Pass predicate of kmerMain.cpp:180, evaluated in the reference's types.
inline bool keep_host(float d, float thr) {
    return d < thr || (double)std::fabs(d - thr) < 0.00001;
}

// mmin[t] = smallest m in [0, t] whose distance 1 - m/t passes, 0xFFFF if
// none.  The predicate is monotone in m (IEEE division and subtraction are
// monotone), so "m >= mmin[t]" is exactly the reference's test.
void build_mmin(float thr, int max_t, std::vector<uint16_t>& mmin, std::vector<uint16_t>& smin) {
    mmin.assign(max_t + 1, 0xFFFF);
    auto pass = [thr](int m, int t) {
        volatile float q = (float)m / (float)t;
        volatile float d = 1.0f - q;
        return keep_host(d, thr);
    };
    for (int t = 0; t <= max_t; ++t) {
        // smallest passing m in [0, t] by bisection (pass is monotone in m)
        if (!pass(t, t)) continue;
        int lo = 0, hi = t;
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            if (pass(mid, t)) hi = mid; else lo = mid + 1;
        }
        mmin[t] = (uint16_t)lo;
    }
    smin.assign(max_t + 1, 0xFFFF);
    uint16_t run = 0xFFFF;
    for (int t = max_t; t >= 0; --t) {
        run = std::min(run, mmin[t]);
        smin[t] = run;
    }
}

// Lanes holding a queued column that start a full-pass round of the bound
// pass (CRISPY_KMER_QFIRE, 1..32).
int kmer_qfire() {
    int v = kQFire;
    if (const char* e = std::getenv("CRISPY_KMER_QFIRE")) v = std::atoi(e);
    return std::max(1, std::min(32, v));
}

int bits_for(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) ++b;
    return b;
}

// Dense level planes kept in shared memory for K (0: dense kernel only).
// Row reads per tile block: 128-bit plane words for K <= 6, 64-bit for
// K = 7 (one 16,384-word level fills the budget), 32-bit for K = 8.
int tile_rows_for(int K) { return K == 8 ? kRows8 : K == 7 ? kTileRows : kRows128; }

int dense_levels_for(int K) {
    if (K >= 8) return 1;   // first occurrences in the 32-bit plane of the K = 8 kernels
    const int per_level = (1 << (2 * K)) * (tile_rows_for(K) / 8);   // bytes of one level's words
    return std::max(1, std::min(4, kPlaneBudget / per_level));
}

// Survivors a k-mer pass may keep on the device (CRISPY_KMER_DEVICE_PAIRS
// overrides, for tests): an eighth of the free memory at 40 bytes each.
int64_t kmer_device_pair_cap() {
    if (const char* e = std::getenv("CRISPY_KMER_DEVICE_PAIRS")) {
        const long long v = std::atoll(e);
        if (v > 0) return v;
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 1LL << 26;
    return std::max<int64_t>(1LL << 22, (int64_t)(free_b / 8 / 40));
}

using TileFn = void (*)(TileArgs);
TileFn tile8_fn_for(int B) {
    switch (B) {
        case 8: return kmer_tile8_kernel<8>;
        case 9: return kmer_tile8_kernel<9>;
        case 10: return kmer_tile8_kernel<10>;
        case 11: return kmer_tile8_kernel<11>;
        default: return kmer_tile8_kernel<12>;
    }
}

TileFn tile8s_fn_for(int B) {
    switch (B) {
        case 8: return kmer_tile8s_kernel<8>;
        case 9: return kmer_tile8s_kernel<9>;
        case 10: return kmer_tile8s_kernel<10>;
        case 11: return kmer_tile8s_kernel<11>;
        default: return kmer_tile8s_kernel<12>;
    }
}

TileFn tile8h_fn_for(int B) {
    switch (B) {
        case 8: return kmer_tile8h_kernel<8>;
        case 9: return kmer_tile8h_kernel<9>;
        case 10: return kmer_tile8h_kernel<10>;
        case 11: return kmer_tile8h_kernel<11>;
        default: return kmer_tile8h_kernel<12>;
    }
}

TileFn tile128_fn_for(int B) {
    switch (B) {
        case 8: return kmer_tile128_kernel<8>;
        case 9: return kmer_tile128_kernel<9>;
        case 10: return kmer_tile128_kernel<10>;
        case 11: return kmer_tile128_kernel<11>;
        default: return kmer_tile128_kernel<12>;
    }
}

TileFn tile_fn_for(int B) {
    switch (B) {
        case 8: return kmer_tile_kernel<8>;
        case 9: return kmer_tile_kernel<9>;
        case 10: return kmer_tile_kernel<10>;
        case 11: return kmer_tile_kernel<11>;
        default: return kmer_tile_kernel<12>;
    }
}

}  // namespace
}  // namespace crispy

using namespace crispy;

namespace crispy {
namespace {

// Group layout of the reads in the job's read order (tuple counts t[]):
// entries per lane and first entry of each 32-read group, uploaded with t.
// ---- the bound pass's split, tuned per read set --------------------------
// Section 0's share decides how many columns the bound pass leaves alive,
// which depends on the reads (99,999 reads of uneven lengths: 112/256 is
// best; 19,954 reads of N(250, 15): 144/256, and one pass is close).  The
// split fixes the stream layout, so each candidate costs a rebuild; the
// batched run times the tile kernel over every kKmerTuneStride-th row group
// for each candidate once per read set (read count, K and tuple counts) and
// keeps the fastest for the life of the process, from the read set's second
// batched run on (a one-shot run keeps the default).  Any split gives the
// same survivors, so tuning only picks speed.  CRISPY_KMER_SPLIT fixes the
// split; CRISPY_AUTOTUNE=0 keeps the default.
struct KmerTuneEntry {
    int n, k, split;
    float ms_best, ms_default;
    int row_groups;
};
std::mutex g_ktune_mu;
std::map<uint64_t, KmerTuneEntry> g_ktuned;
std::map<uint64_t, int> g_kseen;   // batched runs per read set not yet tuned
constexpr int kKmerTuneMinReads = 8192;
constexpr int kKmerTuneStride = 8;
constexpr int kKmerTuneChunk = 256;   // column groups per item of a timing sample
constexpr int kSplitCandidates[] = {kSplitDefault, 0, 96, 128, 144, 160};

bool kmer_autotune_enabled() {
    const char* e = std::getenv("CRISPY_AUTOTUNE");
    return !(e && e[0] == '0');
}

// CRISPY_KMER_SPLIT, when set (0..255)
bool kmer_split_env(int* v) {
    const char* e = std::getenv("CRISPY_KMER_SPLIT");
    if (!e) return false;
    if (v) *v = std::max(0, std::min(255, std::atoi(e)));
    return true;
}

// FNV-1a over the read count, K and the tuple counts (by read ID)
uint64_t kmer_fingerprint(const KmerJob& j) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t x) { h = (h ^ x) * 1099511628211ull; };
    mix((uint64_t)j.n);
    mix((uint64_t)j.k);
    for (int r = 0; r < j.n; ++r) mix((uint64_t)(uint32_t)j.h_t[r]);
    return h;
}

int kmer_groups(crispy_ctx* ctx, const int32_t* t) {
    KmerJob& j = ctx->kmer;
    const int n = j.n;
    j.h_gent.assign(j.ngroups, 0);
    j.h_gstart.assign(j.ngroups + 1, 0);
    for (int r = 0; r < n; ++r) j.h_gent[r >> 5] = std::max(j.h_gent[r >> 5], t[r]);
    j.h_tgent.assign(j.ngroups, 0);
    j.h_tstart.assign(j.ngroups + 1, 0);
    for (int g = 0; g < j.ngroups; ++g) {
        const int mt = j.h_gent[g];
        j.h_gent[g] = (mt + 15) / 16 * 16;
        j.h_gstart[g + 1] = j.h_gstart[g] + 32LL * j.h_gent[g];
        // K = 7: spare steps give the bank schedule wildcards; the 128-row
        // kernel (K <= 6) gains more from the steps saved than it loses to
        // the conflicts left
        const int spare = tile_rows_for(j.k) == kRows128 || mt < 128 ? 0 : kSchedSpare;
        j.h_tgent[g] = (mt + spare + 15) / 16 * 16;
        // split streams: the schedule kernel sets both sections' steps; room
        // for two sections of gent steps each
        j.h_tstart[g + 1] = j.h_tstart[g] + 32LL * (j.split ? 2 * j.h_gent[g] : j.h_tgent[g]);
    }
    j.nent = j.h_gstart[j.ngroups];
    j.ntent = j.h_tstart[j.ngroups];
    cudaStream_t s = ctx->stream;
    CRISPY_TRY(ensure(ctx, j.ent, (size_t)std::max<int64_t>(j.nent, 4) * 4));
    if (j.k != 8) CRISPY_TRY(ensure(ctx, j.tent, (size_t)std::max<int64_t>(j.ntent, 8) * 2));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.t.ptr, t, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.gstart.ptr, j.h_gstart.data(), (size_t)(j.ngroups + 1) * 8,
                                   cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.gent.ptr, j.h_gent.data(), (size_t)j.ngroups * 4,
                                   cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.tstart.ptr, j.h_tstart.data(), (size_t)(j.ngroups + 1) * 8,
                                   cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.tgent.ptr, j.h_tgent.data(), (size_t)j.ngroups * 4,
                                   cudaMemcpyHostToDevice, s));
    return CRISPY_OK;
}

// Per-read layout of a K-mer job from the read lengths (host metadata and
// the device buffers sized for it); the reads themselves come next.  K = 8
// jobs get their group layout at rebuild, in the read order built there.
int kmer_layout(crispy_ctx* ctx, const int32_t* lengths, int n, int k) {
    if (n > CRISPY_MAX_NUM_READS) return fail(ctx, CRISPY_E_UNSUPPORTED, "numReads %d > %d", n, CRISPY_MAX_NUM_READS);
    if (k < 1 || k > 8) return fail(ctx, CRISPY_E_UNSUPPORTED, "K = %d outside 1..8", k);
    KmerJob& j = ctx->kmer;
    j.ready = false;
    j.n = n;
    j.k = k;
    j.h_t.resize(n);
    j.max_len = 0;
    j.max_t = 0;
    for (int r = 0; r < n; ++r) {
        if (lengths[r] > CRISPY_MAX_READ_LEN)
            return fail(ctx, CRISPY_E_UNSUPPORTED, "read %d length %d > %d", r, lengths[r], CRISPY_MAX_READ_LEN);
        if (lengths[r] < k - 1)
            return fail(ctx, CRISPY_E_INPUT, "read %d length %d shorter than K-1", r, lengths[r]);
        j.h_t[r] = lengths[r] - k + 1;
        j.max_len = std::max(j.max_len, (int)lengths[r]);
        j.max_t = std::max(j.max_t, j.h_t[r]);
    }
    j.ngroups = (n + 31) / 32;
    j.split = 0;
    if (tile_rows_for(k) == kRows128) {
        // section 0's share of the dense entries in 1/256 (0: one section,
        // no bound pass): CRISPY_KMER_SPLIT, else the tuned split of this
        // read set, else the default
        if (!kmer_split_env(&j.split)) {
            j.split = kSplitDefault;
            if (kmer_autotune_enabled()) {
                std::lock_guard<std::mutex> g(g_ktune_mu);
                auto it = g_ktuned.find(kmer_fingerprint(j));
                if (it != g_ktuned.end()) j.split = it->second.split;
            }
        }
    }
    CRISPY_TRY(ensure(ctx, j.off, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.t, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.gstart, (size_t)(j.ngroups + 1) * 8));
    CRISPY_TRY(ensure(ctx, j.gent, (size_t)j.ngroups * 4));
    CRISPY_TRY(ensure(ctx, j.cntmax, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.hinfo, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.bcnt, (size_t)n * 128));
    CRISPY_TRY(ensure(ctx, j.tstart, (size_t)(j.ngroups + 1) * 8));
    CRISPY_TRY(ensure(ctx, j.tgent, (size_t)j.ngroups * 4));
    if (j.split) {
        CRISPY_TRY(ensure(ctx, j.tgentL, (size_t)j.ngroups * 4));
        CRISPY_TRY(ensure(ctx, j.nsec, (size_t)n * 8));
    }
    if (k != 8) return kmer_groups(ctx, j.h_t.data());
    CRISPY_TRY(ensure(ctx, j.tgentL, (size_t)j.ngroups * 4));
    CRISPY_TRY(ensure(ctx, j.nsec, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.t0, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.offp, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.perm, (size_t)n * 4));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.t0.ptr, j.h_t.data(), (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    return CRISPY_OK;
}

// K = 8 read order (kmer_hkey_kernel): the sorted order as perm (position ->
// read ID) and the reads' offsets in that order, then the group layout.
int kmer_order(crispy_ctx* ctx) {
    KmerJob& j = ctx->kmer;
    const int n = j.n;
    cudaStream_t s = ctx->stream;
    const int tbits = std::max(1, bits_for((uint64_t)j.max_t));
    CRISPY_TRY(ensure(ctx, j.keys, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.keys_alt, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, j.vals, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.vals_alt, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, j.sort_tmp, sort_tmp_bytes(n)));
    kmer_hkey_kernel<<<std::min((n + 7) / 8, ctx->sm_count * 16), 256, 0, s>>>(
        j.seq.as<uint8_t>(), j.off.as<int64_t>(), j.t0.as<int32_t>(), n, tbits, j.keys.as<uint64_t>(),
        j.vals.as<uint32_t>());
    count_launch(ctx);
    CRISPY_CK(ctx, cudaGetLastError());
    uint64_t* sk = nullptr;
    uint32_t* sv = nullptr;
    CRISPY_TRY(sort_u64_payload(ctx, s, j.keys.as<uint64_t>(), j.keys_alt.as<uint64_t>(), j.vals.as<uint32_t>(),
                                j.vals_alt.as<uint32_t>(), n, 32 + tbits, true, &sk, &sv, j.sort_tmp));
    kmer_gather_off_kernel<<<(n + 255) / 256, 256, 0, s>>>(j.off.as<int64_t>(), sv, n, j.offp.as<int64_t>(),
                                                           j.perm.as<int32_t>());
    count_launch(ctx);
    CRISPY_CK(ctx, cudaGetLastError());
    j.h_perm.resize(n);
    CRISPY_CK(ctx, cudaMemcpyAsync(j.h_perm.data(), j.perm.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    j.h_tpos.resize(n);
    for (int i = 0; i < n; ++i) {
        const int32_t r = j.h_perm[i];
        if (r < 0 || r >= n) return fail(ctx, CRISPY_E_STATE, "read order is not a permutation");
        j.h_tpos[i] = j.h_t[r];
    }
    return kmer_groups(ctx, j.h_tpos.data());
}

}  // namespace
}  // namespace crispy

extern "C" {

int crispy_kmer_prepare(crispy_ctx* ctx, const char* seqbuf, const int64_t* offsets,
                        const int32_t* lengths, int n, int k) {
    if (!ctx) return CRISPY_E_INPUT;
    if (!seqbuf || !offsets || !lengths || n <= 0)
        return fail(ctx, CRISPY_E_INPUT, "kmer_prepare: empty or NULL read set");
    cudaSetDevice(ctx->device);
    ctx->kmer.ready = false;
    int64_t end = 0;
    for (int r = 0; r < n; ++r) {
        if (offsets[r] < 0) return fail(ctx, CRISPY_E_INPUT, "read %d has a negative offset", r);
        end = std::max(end, offsets[r] + (int64_t)std::max(lengths[r], 0));
    }
    CRISPY_TRY(kmer_layout(ctx, lengths, n, k));
    KmerJob& j = ctx->kmer;
    cudaStream_t s = ctx->stream;
    CRISPY_TRY(ensure(ctx, j.seq, (size_t)end + 16));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.seq.ptr, seqbuf, end, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.off.ptr, offsets, (size_t)n * 8, cudaMemcpyHostToDevice, s));
    j.ready = true;   // reads are resident; the entries are built next
    return crispy_kmer_rebuild(ctx);
}

// The reads the last crispy_preprocess kept: a device-to-device copy of the
// padded reads plus their offsets, then the same build as kmer_prepare.
int crispy_kmer_prepare_from_pre(crispy_ctx* ctx, const crispy_raw* raw, int k) {
    if (!ctx) return CRISPY_E_INPUT;
    cudaSetDevice(ctx->device);
    ctx->kmer.ready = false;
    const uint8_t* d_bytes;
    size_t bytes;
    const int64_t* d_off;
    std::vector<int32_t> len;
    CRISPY_TRY(pre_stage_reads(ctx, raw, 0, &d_bytes, &bytes, &d_off, len));
    const int n = (int)len.size();
    if (n <= 0) return fail(ctx, CRISPY_E_INPUT, "kmer_prepare_from_pre: preprocess kept no read");
    CRISPY_TRY(kmer_layout(ctx, len.data(), n, k));
    KmerJob& j = ctx->kmer;
    cudaStream_t s = ctx->stream;
    CRISPY_TRY(ensure(ctx, j.seq, bytes + 16));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.seq.ptr, d_bytes, bytes, cudaMemcpyDeviceToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.off.ptr, d_off, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
    j.ready = true;
    return crispy_kmer_rebuild(ctx);
}

// Rebuild the level entries, multiplicities and K = 8 keys from the reads
// already resident on the device (no host transfer of reads).
int crispy_kmer_rebuild(crispy_ctx* ctx) {
    if (!ctx) return CRISPY_E_INPUT;
    KmerJob& j = ctx->kmer;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "kmer_rebuild before kmer_prepare");
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    const int n = j.n, k = j.k;
    // K = 8: entries and streams are laid out in the read order
    j.hkeys_ordered = false;
    if (k == 8) CRISPY_TRY(kmer_order(ctx));
    const int64_t* loff = k == 8 ? j.offp.as<int64_t>() : j.off.as<int64_t>();
    CRISPY_CK(ctx, cudaMemsetAsync(j.ent.ptr, 0xFF, (size_t)std::max<int64_t>(j.nent, 4) * 4, s));
    const uint32_t K4 = 1u << (2 * k);
    int32_t* cntmax = j.cntmax.as<int32_t>();
    int32_t* nhigh = cntmax + n;
    int32_t* d_nsec = k == 8 || j.split ? j.nsec.as<int32_t>() : nullptr;
    // one warp per read (a table of occurrence ranks per warp) where the
    // block kernel's histogram is large: K = 8, reads of up to 512 tuples
    // (measured 3.9 -> about 1.9 ms on the stress set; at K = 6 the two
    // kernels tie); CRISPY_KMER_PREP_WARP=1 / 0 forces it on / off
    const char* pw_env = std::getenv("CRISPY_KMER_PREP_WARP");
    const bool prep_warp = j.max_t <= kPrepWarpMaxT && (pw_env ? std::strcmp(pw_env, "0") != 0 : k == 8);
    if (prep_warp) {
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kmer_prep_warp_kernel, kPrepWarps * 32, 0);
        const int grid = std::min((n + kPrepWarps - 1) / kPrepWarps, ctx->sm_count * std::max(1, per_sm));
        kmer_prep_warp_kernel<<<grid, kPrepWarps * 32, 0, s>>>(
            j.seq.as<uint8_t>(), loff, j.t.as<int32_t>(), n, k, dense_levels_for(k), j.gstart.as<int64_t>(),
            j.gent.as<int32_t>(), j.ent.as<uint32_t>(), cntmax, nhigh, j.hinfo.as<uint32_t>(),
            j.bcnt.as<uint16_t>(), d_nsec, (uint32_t)j.split);
    } else {
        auto prep = k == 8 ? kmer_prep_kernel<PrepHist12> : kmer_prep_kernel<PrepHist16>;
        const size_t hsmem = k == 8 ? PrepHist12::bytes(K4) : PrepHist16::bytes(K4);
        CRISPY_CK(ctx, cudaFuncSetAttribute(prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsmem));
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prep, kPrepThreads, hsmem);
        const int grid = std::min(n, ctx->sm_count * std::max(1, std::min(per_sm, 8)));
        prep<<<grid, kPrepThreads, hsmem, s>>>(j.seq.as<uint8_t>(), loff,
                                                  j.t.as<int32_t>(), n, k, dense_levels_for(k),
                                                  j.gstart.as<int64_t>(), j.gent.as<int32_t>(),
                                                  j.ent.as<uint32_t>(), cntmax, nhigh,
                                                  j.hinfo.as<uint32_t>(), j.bcnt.as<uint16_t>(), d_nsec,
                                                  (uint32_t)j.split);
    }
    count_launch(ctx);
    CRISPY_CK(ctx, cudaGetLastError());
    const int levels = dense_levels_for(k);
    if (k == 8) {
        // the schedule kernel sets both streams' steps per group; the layout
        // leaves room for them (H <= gent, L <= gent + 32)
        j.h_tstart.assign(j.ngroups + 1, 0);
        for (int g = 0; g < j.ngroups; ++g) j.h_tstart[g + 1] = j.h_tstart[g] + 32LL * (2 * j.h_gent[g] + 32);
        j.ntent = j.h_tstart[j.ngroups];
        CRISPY_TRY(ensure(ctx, j.tent, (size_t)std::max<int64_t>(j.ntent, 8) * 2));
        CRISPY_CK(ctx, cudaMemcpyAsync(j.tstart.ptr, j.h_tstart.data(), (size_t)(j.ngroups + 1) * 8,
                                       cudaMemcpyHostToDevice, s));
        // the per-read H / L counts and H keys come back on a side stream
        // while the schedule runs
        j.h_nsec.resize(2 * (size_t)n);
        j.h_hinfo.resize(n);
        CRISPY_CK(ctx, cudaEventRecord(ctx->fork_ev, s));
        CRISPY_CK(ctx, cudaStreamWaitEvent(ctx->side[0], ctx->fork_ev, 0));
        CRISPY_CK(ctx, cudaMemcpyAsync(j.h_nsec.data(), j.nsec.ptr, (size_t)n * 8, cudaMemcpyDeviceToHost,
                                       ctx->side[0]));
        CRISPY_CK(ctx, cudaMemcpyAsync(j.h_hinfo.data(), j.hinfo.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost,
                                       ctx->side[0]));
        CRISPY_CK(ctx, cudaEventRecord(ctx->join_ev[0], ctx->side[0]));
        const int sgrid = std::min((j.ngroups + kSchedWarps - 1) / kSchedWarps, ctx->sm_count * 8);
        kmer_sched8_kernel<<<sgrid, kSchedWarps * 32, 0, s>>>(
            j.ent.as<uint32_t>(), j.gstart.as<int64_t>(), j.tstart.as<int64_t>(), j.tgent.as<int32_t>(),
            j.tgentL.as<int32_t>(), nhigh, j.nsec.as<int32_t>(), j.bcnt.as<uint16_t>(), n, j.ngroups,
            j.tent.as<uint16_t>());
        count_launch(ctx);
        CRISPY_CK(ctx, cudaGetLastError());
        CRISPY_CK(ctx, cudaEventSynchronize(ctx->join_ev[0]));
        // runs of equal H keys along the positions; the batched split needs
        // each key in one run (keys ascending, as the read order sorts them)
        j.h_run_lo.resize(n);
        j.h_run_hi.resize(n);
        j.hkeys_ordered = true;
        for (int i = 0; i < n;) {
            int e = i + 1;
            while (e < n && j.h_hinfo[e] == j.h_hinfo[i]) ++e;
            if (e < n && j.h_hinfo[e] < j.h_hinfo[i]) j.hkeys_ordered = false;
            for (int q = i; q < e; ++q) { j.h_run_lo[q] = i; j.h_run_hi[q] = e; }
            i = e;
        }
    } else if (levels > 0 && j.split) {
        const int sgrid = std::min((j.ngroups + kSchedWarps - 1) / kSchedWarps, ctx->sm_count * 8);
        kmer_sched_split_kernel<<<sgrid, kSchedWarps * 32, 0, s>>>(
            j.ent.as<uint32_t>(), j.gstart.as<int64_t>(), j.tstart.as<int64_t>(), nhigh, j.nsec.as<int32_t>(),
            j.bcnt.as<uint16_t>(), n, j.ngroups, (uint32_t)levels * (1u << (2 * k)), j.tgent.as<int32_t>(),
            j.tgentL.as<int32_t>(), j.tent.as<uint16_t>());
        count_launch(ctx);
        CRISPY_CK(ctx, cudaGetLastError());
    } else if (levels > 0) {
        const int sgrid = std::min((j.ngroups + kSchedWarps - 1) / kSchedWarps, ctx->sm_count * 8);
        auto sched = tile_rows_for(k) == kRows128 ? kmer_sched_kernel<8> : kmer_sched_kernel<16>;
        sched<<<sgrid, kSchedWarps * 32, 0, s>>>(
            j.ent.as<uint32_t>(), j.gstart.as<int64_t>(), j.tstart.as<int64_t>(), j.tgent.as<int32_t>(),
            nhigh, j.bcnt.as<uint16_t>(), n, j.ngroups, (uint32_t)levels * (1u << (2 * k)),
            j.tent.as<uint16_t>());
        count_launch(ctx);
        CRISPY_CK(ctx, cudaGetLastError());
    }
    j.h_cntmax.resize(2 * (size_t)n);
    CRISPY_CK(ctx, cudaMemcpyAsync(j.h_cntmax.data(), j.cntmax.ptr, (size_t)n * 8,
                                   cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    j.nsurv = 0;
    return CRISPY_OK;
}

// sample > 0: a timing run of the batched tile kernel over every sample-th
// row group (no graph, no dense-kernel rows, survivors left unsorted); its
// duration goes to *sample_ms.
static int kmer_run_impl(crispy_ctx* ctx, float thr, int mode, int dists, int64_t* npairs, int sample,
                         float* sample_ms) {
    if (!ctx) return CRISPY_E_INPUT;
    KmerJob& j = ctx->kmer;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "kmer_run before kmer_prepare");
    const int n = j.n, K = j.k;
    const int A = crispy_array_dim(n);
    if (A <= 0) return fail(ctx, CRISPY_E_UNSUPPORTED, "fewer than 10 reads: the reference has no tile size (arrayDim = 0)");
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    ctx->stats = crispy_stats{};
    ctx->ev_kmer.used = 0;
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_begin, s));
    const int sd = (n + A - 1) / A;
    const int64_t nstages = (int64_t)sd * (sd + 1) / 2;

    std::vector<uint16_t> mmin, smin;
    build_mmin(thr, j.max_t, mmin, smin);
    CRISPY_TRY(ensure(ctx, j.mmin, mmin.size() * 2));
    CRISPY_TRY(ensure(ctx, j.smin, smin.size() * 2));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.mmin.ptr, mmin.data(), mmin.size() * 2, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.smin.ptr, smin.data(), smin.size() * 2, cudaMemcpyHostToDevice, s));

    // Rows of tile row groups whose high-level entries exceed the hash go to
    // the dense kernel (flags per 32-read group).
    const int levels = dense_levels_for(K);
    const int rows_blk = tile_rows_for(K);   // row reads per tile block
    const int nrg = (n + rows_blk - 1) / rows_blk;
    std::vector<uint8_t> dense(j.ngroups, 0);
    bool any_dense = false;
    for (int rg = 0; rg < nrg; ++rg) {
        int64_t high = 0;
        for (int r = rg * rows_blk; r < std::min(n, rg * rows_blk + rows_blk); ++r) high += j.h_cntmax[n + r];
        if (levels == 0 || high > kHashMaxKeys) {
            for (int r = rg * rows_blk; r < std::min(n, rg * rows_blk + rows_blk); r += 32) dense[r >> 5] = 1;
            any_dense = true;
        }
    }
    const bool fast = levels > 0;
    CRISPY_TRY(ensure(ctx, j.work, (size_t)j.ngroups + 16));
    CRISPY_CK(ctx, cudaMemcpyAsync(j.work.ptr, dense.data(), j.ngroups, cudaMemcpyHostToDevice, s));

    const uint32_t K4 = 1u << (2 * K);
    const int B = std::max(8, bits_for((uint64_t)j.max_t));
    TileFn tile = K == 8 ? tile8_fn_for(B) : rows_blk == kRows128 ? tile128_fn_for(B) : tile_fn_for(B);
    const int tile_threads = K == 8 ? (B <= 9 ? tile8_threads<9>() : tile8_threads<10>()) : kTileThreads;
    const size_t tsmem = !fast ? 0 : K == 8 ? kSmem8     // one plane + guards
                                             : ((size_t)levels * K4 + 32) * (rows_blk / 8);   // planes + guards
    const size_t dsmem = (size_t)((K4 + 1) / 2) * 4;
    if (fast) CRISPY_CK(ctx, cudaFuncSetAttribute(tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
    // K = 8 batched: the H-only kernel over all row groups plus the two-phase
    // kernel over each row group's same-key column range (the H keys must be
    // in order along the positions, as the read order makes them)
    // (CRISPY_KMER_K8_SPLIT=0 selects the one-kernel form, the same
    // survivors: the two-phase kernel over every column)
    const char* split_env = std::getenv("CRISPY_KMER_K8_SPLIT");
    const bool split8 = fast && K == 8 && mode == CRISPY_MODE_BATCHED && j.hkeys_ordered &&
                        !(split_env && std::strcmp(split_env, "0") == 0);
    TileFn tile_h = split8 ? tile8h_fn_for(B) : nullptr;
    if (split8) CRISPY_CK(ctx, cudaFuncSetAttribute(tile_h, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem8));
    // the same-key ranges of the split: the kernel that queues its L sums
    // (CRISPY_KMER_K8_QUEUE=0 selects the two-phase kernel)
    const char* queue_env = std::getenv("CRISPY_KMER_K8_QUEUE");
    const bool queue8 = split8 && !(queue_env && std::strcmp(queue_env, "0") == 0);
    TileFn tile_s = queue8 ? tile8s_fn_for(B) : tile;
    if (queue8) CRISPY_CK(ctx, cudaFuncSetAttribute(tile_s, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem8));
    CRISPY_CK(ctx, cudaFuncSetAttribute(kmer_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem));

    // K = 8 jobs hold their reads in the read order built at rebuild: the
    // kernels run over positions, emit() maps them back to read IDs.
    const int32_t* perm = K == 8 ? j.perm.as<int32_t>() : nullptr;
    const int64_t* loff = K == 8 ? j.offp.as<int64_t>() : j.off.as<int64_t>();
    // One pass over the pairs whose lower read ID lies in [olo, ohi):
    // survivors (up to cap) as sort keys in j.keys / j.vals, their count in
    // *total.  Without a read order the kernels cover the rows [olo, ohi);
    // with one they cover every row and emit() keeps the range.
    auto run_pass = [&](int olo, int ohi, int64_t cap, int64_t* total_out) -> int {
        const int rlo = perm ? 0 : olo, rhi = perm ? n : ohi;
        CRISPY_TRY(ensure(ctx, j.keys, (size_t)cap * 8));
        CRISPY_TRY(ensure(ctx, j.keys_alt, (size_t)cap * 8));
        CRISPY_TRY(ensure(ctx, j.vals, (size_t)cap * 4));
        CRISPY_TRY(ensure(ctx, j.vals_alt, (size_t)cap * 4));
        CRISPY_TRY(ensure(ctx, j.counter, 64));
        CRISPY_CK(ctx, cudaMemsetAsync(j.counter.ptr, 0, 64, s));

        TileArgs ta{};
        ta.ent = j.ent.as<uint32_t>(); ta.gstart = j.gstart.as<int64_t>(); ta.gent = j.gent.as<int32_t>();
        ta.tent = j.tent.as<uint16_t>(); ta.tstart = j.tstart.as<int64_t>(); ta.tgent = j.tgent.as<int32_t>();
        ta.k65536 = 65536u; ta.k8 = 8u;
        ta.tgentL = j.tgentL.as<int32_t>(); ta.hinfo = j.hinfo.as<uint32_t>(); ta.ngroups = j.ngroups;
        ta.nhigh = j.cntmax.as<int32_t>() + n;
        ta.tcount = j.t.as<int32_t>(); ta.dense_group = j.work.as<uint8_t>();
        ta.mmin = j.mmin.as<uint16_t>(); ta.smin = j.smin.as<uint16_t>();
        ta.n = n; ta.K4 = K4; ta.levels = levels; ta.A = A; ta.stage_dim = sd;
        ta.counter = j.counter.as<unsigned long long>(); ta.keys = j.keys.as<uint64_t>();
        ta.vals = j.vals.as<uint32_t>(); ta.cap = cap;
        ta.perm = perm; ta.olo = olo; ta.ohi = ohi;
        ta.nsec = K == 8 || j.split ? j.nsec.as<int32_t>() : nullptr;
        ta.split = j.split;
        ta.bound = 0;
        ta.qfire = kmer_qfire();
        ta.gstat = nullptr;
        DenseArgs da{};
        da.perm = perm; da.olo = olo; da.ohi = ohi;
        da.seq = j.seq.as<uint8_t>(); da.off = loff; da.ent = ta.ent; da.gstart = ta.gstart;
        da.tcount = ta.tcount; da.hinfo = j.hinfo.as<uint32_t>(); da.mmin = ta.mmin;
        da.n = n; da.K = K; da.A = A; da.stage_dim = sd;
        da.dense_group = fast ? j.work.as<uint8_t>() : nullptr;
        da.counter = ta.counter; da.keys = ta.keys; da.vals = ta.vals; da.cap = cap;

        if (mode == CRISPY_MODE_PLAIN || mode == CRISPY_MODE_STAGED) {
            // One launch per reference stage, round-robin over 8 streams like
            // the reference's stage loop (kmerCUDA.cu:79-111).  PLAIN runs the
            // one-thread-per-pair dense kernel on every row, STAGED the
            // bit-sliced tile kernel (dense kernel only for its overflow rows).
            const bool tiles = fast && mode == CRISPY_MODE_STAGED;
            const bool dense_all = !tiles;
            cudaEvent_t fork;
            CRISPY_CK(ctx, cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
            CRISPY_CK(ctx, cudaEventRecord(fork, s));
            for (auto& ss : ctx->side) CRISPY_CK(ctx, cudaStreamWaitEvent(ss, fork, 0));
            ev_begin(ctx, ctx->ev_kmer, s);
            int64_t st = 0;
            for (int sx = rlo / A; sx * A < rhi; ++sx) {
                for (int sy = sx; sy < sd; ++sy, ++st) {
                    cudaStream_t ss = ctx->side[st % 8];
                    TileArgs t2 = ta;
                    t2.r_lo = sx * A; t2.r_hi = std::min(n, sx * A + A);
                    t2.c_lo = sy * A; t2.c_hi = std::min(n, sy * A + A);
                    if (tiles) {
                        // 128-row blocks split each stage's columns in two, which
                        // keeps as many blocks per stage as 64-row blocks give
                        const int rg0 = t2.r_lo / rows_blk, rg1 = (t2.r_hi - 1) / rows_blk;
                        const dim3 grid(rg1 - rg0 + 1, rows_blk == kRows128 ? 2 : 1);
                        tile<<<grid, tile_threads, tsmem, ss>>>(t2);
                        count_launch(ctx);
                    }
                    if (dense_all || any_dense) {
                        DenseArgs d2 = da;
                        if (dense_all) d2.dense_group = nullptr;
                        d2.r_lo = t2.r_lo; d2.r_hi = t2.r_hi; d2.c_lo = t2.c_lo; d2.c_hi = t2.c_hi;
                        kmer_dense_kernel<<<std::min(t2.r_hi - t2.r_lo, 4 * ctx->sm_count), 256, dsmem, ss>>>(d2);
                        count_launch(ctx);
                    }
                }
            }
            for (auto& ss : ctx->side) {
                cudaEvent_t join;
                CRISPY_CK(ctx, cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
                CRISPY_CK(ctx, cudaEventRecord(join, ss));
                CRISPY_CK(ctx, cudaStreamWaitEvent(s, join, 0));
                cudaEventDestroy(join);
            }
            ev_end(ctx, ctx->ev_kmer, s);
            cudaEventDestroy(fork);
            ctx->stats.kmer_launches += st;
        } else {
            // Batched: persistent launches over work queues of row groups
            // (each with all its columns), longest first.  K = 8 split: the
            // H-only kernel over the 32-row groups, then the two-phase kernel
            // over each row group's same-key column range.
            std::vector<int> items, items_s, s_cs, s_ce;
            std::vector<int2> q_s;
            if (split8) {
                // the H-only kernel's pairs (different H keys) can pass only
                // where one read is H-heavy (|H| >= mmin[T], heavy8): with no
                // such read it has nothing to do
                bool any_heavy = false;
                for (int i = 0; i < n && !any_heavy; ++i) {
                    const int h = j.h_nsec[2 * (size_t)i] + j.h_cntmax[(size_t)n + i];
                    any_heavy = h >= (int)mmin[j.h_tpos[i]];
                }
                for (int g = 0; g < j.ngroups && any_heavy; ++g)
                    if (!dense[g]) items.push_back(g);
                for (int g = 0; g < j.ngroups; ++g) {
                    const int r0 = g * kRows8, r1 = std::min(n, r0 + kRows8);
                    if (dense[g]) continue;
                    // columns of the keys of rows r0 .. r1-1: one range, the keys being in order
                    const int q0 = std::max(g, j.h_run_lo[r0] / 32);
                    const int q1 = (j.h_run_hi[r1 - 1] + 31) / 32;
                    if (q1 > q0) {
                        items_s.push_back(g);
                        q_s.push_back(make_int2(q0, q1));
                    }
                }
            } else if (fast) {
                for (int rg = rlo / rows_blk; rg * rows_blk < rhi; ++rg) {
                    if (sample > 0 && rg % sample != 0) continue;
                    bool any_rows = false;
                    for (int r = rg * rows_blk; r < std::min(n, rg * rows_blk + rows_blk); r += 32)
                        any_rows |= !dense[r >> 5];
                    if (!any_rows) continue;
                    if (sample > 0) {
                        // a timing sample: the row group's columns in chunks,
                        // so that the sample's items keep every SM busy
                        const int c0 = rg * (rows_blk / 32), c1 = (n + 31) / 32;
                        for (int c = c0; c < c1; c += kKmerTuneChunk) {
                            items.push_back(rg);
                            s_cs.push_back(c);
                            s_ce.push_back(std::min(c1, c + kKmerTuneChunk));
                        }
                    } else {
                        items.push_back(rg);
                    }
                }
            }
            if (!items.empty() || !items_s.empty()) {
                const size_t nh = items.size(), ns = items_s.size(), nc = s_cs.size();
                CRISPY_TRY(ensure(ctx, j.sort_tmp, ns * sizeof(int2) + (nh + ns + 2 * nc) * sizeof(int) + 64));
                int2* d_q = j.sort_tmp.as<int2>();
                int* d_items = reinterpret_cast<int*>(d_q + ns);
                int* d_items_s = d_items + nh;
                int* d_cs = d_items_s + ns;
                int* d_ce = d_cs + nc;
                unsigned int* head = reinterpret_cast<unsigned int*>(d_ce + nc);
                if (nc) {
                    CRISPY_CK(ctx, cudaMemcpyAsync(d_cs, s_cs.data(), nc * sizeof(int), cudaMemcpyHostToDevice, s));
                    CRISPY_CK(ctx, cudaMemcpyAsync(d_ce, s_ce.data(), nc * sizeof(int), cudaMemcpyHostToDevice, s));
                }
                if (nh) CRISPY_CK(ctx, cudaMemcpyAsync(d_items, items.data(), nh * sizeof(int), cudaMemcpyHostToDevice, s));
                if (ns) {
                    CRISPY_CK(ctx, cudaMemcpyAsync(d_items_s, items_s.data(), ns * sizeof(int), cudaMemcpyHostToDevice, s));
                    CRISPY_CK(ctx, cudaMemcpyAsync(d_q, q_s.data(), ns * sizeof(int2), cudaMemcpyHostToDevice, s));
                }
                CRISPY_CK(ctx, cudaMemsetAsync(head, 0, 8, s));
                const TileFn main_fn = split8 ? tile_h : tile;
                const size_t main_smem = split8 ? kSmem8 : tsmem;
                TileArgs t2 = ta;
                t2.r_lo = 0; t2.r_hi = n; t2.c_lo = 0; t2.c_hi = n;
                t2.items = d_items; t2.nitems = (int)nh; t2.queue_head = head;
                // the bound pass needs the columns of whole row groups (the
                // staged form's blocks hold too few to fill the lanes' stacks)
                t2.bound = j.split != 0;
                t2.gstat = j.split ? j.counter.as<unsigned long long>() + 1 : nullptr;
                if (nc) {
                    t2.item_cstart = d_cs;
                    t2.item_cend = d_ce;
                }
                TileArgs t3 = t2;
                t3.items = d_items_s; t3.nitems = (int)ns; t3.queue_head = head + 1;
                t3.item_q = d_q; t3.same_only = 1;
                int per_sm = 1, per_sm_s = 1;
                const int main_threads = split8 ? kTile8HThreads : tile_threads;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, main_fn, main_threads, main_smem);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_s, tile_s, tile_threads, tsmem);
                per_sm = std::max(1, per_sm);
                per_sm_s = std::max(1, per_sm_s);
                const int grid = (int)std::min<int64_t>((int64_t)per_sm * ctx->sm_count, (int64_t)nh);
                const int grid_s = (int)std::min<int64_t>((int64_t)per_sm_s * ctx->sm_count, (int64_t)ns);
                if (queue8 && ns) {
                    // queue scratch: per block and lane slot, one item per
                    // column group of the widest range
                    int64_t cap = 1;
                    for (size_t i = 0; i < ns; ++i)
                        cap = std::max<int64_t>(cap, q_s[i].y - std::max(q_s[i].x, items_s[i]));
                    CRISPY_TRY(ensure(ctx, j.sq, (size_t)grid_s * cap * (B + 2) * 32 * 4));
                    t3.sq = j.sq.as<uint32_t>();
                    t3.sq_cap = cap;
                }
                DenseArgs d2 = da;
                d2.r_lo = rlo; d2.r_hi = rhi; d2.c_lo = 0; d2.c_hi = n;
                const std::string key = "kmain," + key_of({(uint64_t)(uintptr_t)j.ent.ptr, (uint64_t)(uintptr_t)j.keys.ptr,
                    (uint64_t)(uintptr_t)j.vals.ptr, (uint64_t)(uintptr_t)j.counter.ptr, (uint64_t)(uintptr_t)d_q,
                    (uint64_t)(uintptr_t)j.mmin.ptr, (uint64_t)(uintptr_t)j.smin.ptr, (uint64_t)(uintptr_t)j.t.ptr,
                    (uint64_t)(uintptr_t)j.gstart.ptr, (uint64_t)(uintptr_t)j.gent.ptr, (uint64_t)(uintptr_t)j.work.ptr,
                    (uint64_t)(uintptr_t)j.seq.ptr, (uint64_t)(uintptr_t)loff, (uint64_t)(uintptr_t)j.hinfo.ptr,
                    (uint64_t)(uintptr_t)perm, (uint64_t)olo, (uint64_t)ohi,
                    (uint64_t)(uintptr_t)j.tent.ptr, (uint64_t)(uintptr_t)j.tstart.ptr, (uint64_t)(uintptr_t)j.tgent.ptr,
                    (uint64_t)(uintptr_t)j.cntmax.ptr, (uint64_t)(uintptr_t)j.tgentL.ptr, (uint64_t)(uintptr_t)j.nsec.ptr,
                    (uint64_t)n, (uint64_t)K, (uint64_t)B, (uint64_t)cap, (uint64_t)split8,
                    (uint64_t)nh, (uint64_t)ns, (uint64_t)grid, (uint64_t)grid_s, (uint64_t)any_dense, (uint64_t)A,
                    (uint64_t)rlo, (uint64_t)rhi, (uint64_t)j.split, (uint64_t)t2.bound, (uint64_t)t2.qfire,
                    (uint64_t)queue8, (uint64_t)(uintptr_t)t3.sq, (uint64_t)t3.sq_cap});
                if (sample > 0) {
                    cudaEvent_t e0, e1;
                    CRISPY_CK(ctx, cudaEventCreate(&e0));
                    CRISPY_CK(ctx, cudaEventCreate(&e1));
                    CRISPY_CK(ctx, cudaMemsetAsync(j.counter.ptr, 0, 64, s));
                    CRISPY_CK(ctx, cudaMemsetAsync(head, 0, 8, s));
                    CRISPY_CK(ctx, cudaEventRecord(e0, s));
                    if (nh) main_fn<<<grid, main_threads, main_smem, s>>>(t2);
                    CRISPY_CK(ctx, cudaEventRecord(e1, s));
                    count_launch(ctx);
                    CRISPY_CK(ctx, cudaEventSynchronize(e1));
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    CRISPY_CK(ctx, cudaGetLastError());
                    if (sample_ms) *sample_ms = ms;
                    *total_out = 0;
                    return CRISPY_OK;
                }
                ev_begin(ctx, ctx->ev_kmer, s);
                CRISPY_TRY(graph_run(ctx, s, key, [&]() -> int {
                    CRISPY_CK(ctx, cudaMemsetAsync(j.counter.ptr, 0, 64, s));
                    CRISPY_CK(ctx, cudaMemsetAsync(head, 0, 8, s));
                    if (nh) {
                        main_fn<<<grid, main_threads, main_smem, s>>>(t2);
                        count_launch(ctx);
                    }
                    if (ns) {
                        tile_s<<<grid_s, tile_threads, tsmem, s>>>(t3);
                        count_launch(ctx);
                    }
                    if (any_dense) {
                        kmer_dense_kernel<<<std::min(rhi - rlo, 8 * ctx->sm_count), 256, dsmem, s>>>(d2);
                        count_launch(ctx);
                    }
                    CRISPY_CK(ctx, cudaGetLastError());
                    return CRISPY_OK;
                }));
                ev_end(ctx, ctx->ev_kmer, s);
                ctx->stats.kmer_launches += 1;
            } else if (any_dense && sample == 0) {
                DenseArgs d2 = da;
                d2.r_lo = rlo; d2.r_hi = rhi; d2.c_lo = 0; d2.c_hi = n;
                kmer_dense_kernel<<<std::min(rhi - rlo, 8 * ctx->sm_count), 256, dsmem, s>>>(d2);
                count_launch(ctx);
            }
        }
        CRISPY_CK(ctx, cudaGetLastError());
        unsigned long long cnt[5] = {0, 0, 0, 0, 0};
        CRISPY_CK(ctx, cudaMemcpyAsync(cnt, j.counter.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, s));
        CRISPY_CK(ctx, cudaStreamSynchronize(s));
        *total_out = (int64_t)cnt[0];
        ctx->stats.kmer_bound_entries += (int64_t)cnt[1];
        ctx->stats.kmer_full_entries += (int64_t)cnt[2];
        ctx->stats.kmer_full_columns += (int64_t)cnt[3];
        ctx->stats.kmer_rounds += (int64_t)cnt[4];
        return CRISPY_OK;
    };
    // stable order: (stage, row, col)
    const int key_bits = bits_for((uint64_t)nstages * (uint64_t)n * (uint64_t)n);
    auto sort_decode = [&]() -> int {
        uint64_t* sk = nullptr;
        uint32_t* sv = nullptr;
        CRISPY_TRY(sort_u64_payload(ctx, s, j.keys.as<uint64_t>(), j.keys_alt.as<uint64_t>(),
                                    j.vals.as<uint32_t>(), j.vals_alt.as<uint32_t>(), j.nsurv, key_bits,
                                    dists != 0, &sk, &sv, j.sort_tmp));
        if (j.nsurv > 0) {
            kmer_decode_kernel<<<(unsigned)((j.nsurv + 255) / 256), 256, 0, s>>>(
                sk, sv, j.nsurv, n, j.pairs.as<int2>(), dists ? j.dists.as<float>() : nullptr);
            count_launch(ctx);
            CRISPY_CK(ctx, cudaGetLastError());
        }
        return CRISPY_OK;
    };
    // sort + decode the j.nsurv keys of the last pass into j.pairs / j.dists
    auto finish_pass = [&]() -> int {
        CRISPY_TRY(ensure(ctx, j.pairs, (size_t)std::max<int64_t>(j.nsurv, 1) * 8));
        CRISPY_TRY(ensure(ctx, j.dists, (size_t)std::max<int64_t>(j.nsurv, 1) * 4));
        CRISPY_TRY(ensure(ctx, j.sort_tmp, sort_tmp_bytes(j.nsurv)));
        if (mode == CRISPY_MODE_BATCHED && j.nsurv > 0) {
            const std::string key = "ksort," + key_of({(uint64_t)j.nsurv, (uint64_t)key_bits, (uint64_t)dists,
                (uint64_t)n, (uint64_t)(uintptr_t)j.keys.ptr, (uint64_t)(uintptr_t)j.keys_alt.ptr,
                (uint64_t)(uintptr_t)j.vals.ptr, (uint64_t)(uintptr_t)j.vals_alt.ptr,
                (uint64_t)(uintptr_t)j.sort_tmp.ptr, (uint64_t)(uintptr_t)j.pairs.ptr, (uint64_t)(uintptr_t)j.dists.ptr});
            return graph_run(ctx, s, key, sort_decode);
        }
        return sort_decode();
    };

    // Survivors held on the device at once: about 40 bytes each while sorted
    // (keys, values, their sort copies, pairs, distances).
    const int64_t dev_cap = kmer_device_pair_cap();
    int64_t cap = std::min(dev_cap, std::max<int64_t>(j.keys.bytes / 8, std::max<int64_t>(1 << 20, 16LL * n)));
    int64_t total = 0;
    j.spilled = false;
    CRISPY_TRY(run_pass(0, n, cap, &total));
    if (sample > 0) {
        j.nsurv = 0;
        return CRISPY_OK;
    }
    if (total > cap && total <= dev_cap) {
        cap = std::min(dev_cap, total + total / 8 + 1024);
        CRISPY_TRY(run_pass(0, n, cap, &total));
        if (total > cap) return fail(ctx, CRISPY_E_STATE, "survivor count changed between passes");
    }
    if (total <= cap) {
        j.nsurv = total;
        CRISPY_TRY(finish_pass());
    } else {
        // Spill: the survivors outgrow the device share.  Stage rows are
        // processed in ranges whose survivors fit; stage order is row-major
        // over stage rows, so each range's sorted pairs append in order to
        // one pinned host list (the count is known from the first pass).
        if (!perm && A % rows_blk != 0) return fail(ctx, CRISPY_E_OOM, "survivor list exceeds the device share");
        CRISPY_TRY(ensure_host(ctx, j.h_spill_pairs, (size_t)total * 8));
        if (dists) CRISPY_TRY(ensure_host(ctx, j.h_spill_dists, (size_t)total * 4));
        // expected survivors per stage row, proportional to its pairs
        std::vector<double> est(sd);
        const double per_pair = (double)total / ((double)n * (double)(n - 1) / 2.0);
        for (int sx = 0; sx < sd; ++sx) {
            const double r0 = sx * (double)A, r1 = std::min<double>(n, r0 + A);
            est[sx] = per_pair * ((r1 - r0) * (n - 1) - (r1 * (r1 - 1) - r0 * (r0 - 1)) / 2.0);
        }
        int64_t off = 0;
        for (int sx = 0; sx < sd;) {
            int sx1 = sx + 1;
            double acc = est[sx];
            while (sx1 < sd && acc + est[sx1] <= 0.5 * (double)dev_cap) acc += est[sx1++];
            int64_t t = 0;
            CRISPY_TRY(run_pass(sx * A, std::min(n, sx1 * A), dev_cap, &t));
            if (t > dev_cap) {
                if (sx1 - sx == 1) return fail(ctx, CRISPY_E_OOM, "one stage row's survivors exceed the device share");
                for (int q = sx; q < sx1; ++q) est[q] *= 2.0;   // denser than estimated: smaller ranges
                continue;
            }
            if (off + t > total) return fail(ctx, CRISPY_E_STATE, "survivor count changed between passes");
            j.nsurv = t;
            CRISPY_TRY(finish_pass());
            if (t > 0) {
                CRISPY_CK(ctx, cudaMemcpyAsync(j.h_spill_pairs.as<char>() + off * 8, j.pairs.ptr, (size_t)t * 8,
                                               cudaMemcpyDeviceToHost, s));
                if (dists)
                    CRISPY_CK(ctx, cudaMemcpyAsync(j.h_spill_dists.as<char>() + off * 4, j.dists.ptr,
                                                   (size_t)t * 4, cudaMemcpyDeviceToHost, s));
                CRISPY_CK(ctx, cudaStreamSynchronize(s));
            }
            off += t;
            sx = sx1;
        }
        if (off != total) return fail(ctx, CRISPY_E_STATE, "survivor count changed between passes");
        j.nsurv = total;
        j.spilled = true;
        ctx->stats.kmer_spilled = 1;
    }
    j.have_dists = dists != 0;
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_end, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    float tot = 0;
    cudaEventElapsedTime(&tot, ctx->t_begin, ctx->t_end);
    ctx->stats.total_ms = tot;
    ctx->stats.kmer_kernel_ms = ev_sum_ms(ctx->ev_kmer);
    ctx->stats.kmer_pairs = (int64_t)n * (n - 1) / 2;
    ctx->stats.kmer_survivors = j.nsurv;
    if (npairs) *npairs = j.nsurv;
    return CRISPY_OK;
}

// Stream layout and level entries again, for the job's current split.
static int kmer_relayout(crispy_ctx* ctx) {
    KmerJob& j = ctx->kmer;
    if (j.split) {
        CRISPY_TRY(ensure(ctx, j.tgentL, (size_t)j.ngroups * 4));
        CRISPY_TRY(ensure(ctx, j.nsec, (size_t)j.n * 8));
    }
    CRISPY_TRY(kmer_groups(ctx, j.h_t.data()));
    return crispy_kmer_rebuild(ctx);
}

// The split of this read set: the tuned one, or -- from its second batched
// run in this process on, when tuning can pay for itself -- each candidate
// timed on the row-group sample (two runs each, the faster counts) and the
// fastest kept.
static int kmer_tune_split(crispy_ctx* ctx, float thr) {
    KmerJob& j = ctx->kmer;
    const uint64_t fp = kmer_fingerprint(j);
    int best = -1;
    {
        std::lock_guard<std::mutex> g(g_ktune_mu);
        auto it = g_ktuned.find(fp);
        if (it != g_ktuned.end()) best = it->second.split;
        else if (g_kseen[fp]++ == 0) return CRISPY_OK;   // first run: the default split
    }
    if (best < 0) {
        float best_ms = 1e30f, dflt_ms = 0;
        for (int c : kSplitCandidates) {
            j.split = c;
            CRISPY_TRY(kmer_relayout(ctx));
            float ms = 1e30f;
            for (int rep = 0; rep < 2; ++rep) {
                float m = 0;
                CRISPY_TRY(kmer_run_impl(ctx, thr, CRISPY_MODE_BATCHED, 0, nullptr, kKmerTuneStride, &m));
                ms = std::min(ms, m);
            }
            if (c == kSplitDefault) dflt_ms = ms;
            if (ms < best_ms) { best_ms = ms; best = c; }
        }
        std::lock_guard<std::mutex> g(g_ktune_mu);
        g_ktuned[fp] = KmerTuneEntry{j.n, j.k, best, best_ms, dflt_ms,
                                     (int)((j.n + kRows128 * kKmerTuneStride - 1) / (kRows128 * kKmerTuneStride))};
    }
    if (j.split != best) {
        j.split = best;
        CRISPY_TRY(kmer_relayout(ctx));
    }
    return CRISPY_OK;
}

int crispy_kmer_run(crispy_ctx* ctx, float thr, int mode, int dists, int64_t* npairs) {
    if (!ctx) return CRISPY_E_INPUT;
    KmerJob& j = ctx->kmer;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "kmer_run before kmer_prepare");
    cudaSetDevice(ctx->device);
    if (mode == CRISPY_MODE_BATCHED && ctx->kmer_tune && tile_rows_for(j.k) == kRows128 &&
        j.n >= kKmerTuneMinReads && kmer_autotune_enabled() && !kmer_split_env(nullptr))
        CRISPY_TRY(kmer_tune_split(ctx, thr));
    return kmer_run_impl(ctx, thr, mode, dists, npairs, 0, nullptr);
}

int crispy_kmer_fetch(crispy_ctx* ctx, int32_t* pairs, float* dists, int64_t cap, int64_t* count) {
    if (!ctx) return CRISPY_E_INPUT;
    KmerJob& j = ctx->kmer;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "kmer_fetch before kmer_run");
    if (dists && !j.have_dists) return fail(ctx, CRISPY_E_STATE, "distances were not kept by kmer_run");
    const int64_t c = std::min(cap, j.nsurv);
    if (j.spilled) {
        if (c > 0 && pairs) std::memcpy(pairs, j.h_spill_pairs.ptr, (size_t)c * 8);
        if (c > 0 && dists) std::memcpy(dists, j.h_spill_dists.ptr, (size_t)c * 4);
        if (count) *count = c;
        return CRISPY_OK;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    if (c > 0 && pairs)
        CRISPY_CK(ctx, cudaMemcpyAsync(pairs, j.pairs.ptr, (size_t)c * 8, cudaMemcpyDeviceToHost, s));
    if (c > 0 && dists)
        CRISPY_CK(ctx, cudaMemcpyAsync(dists, j.dists.ptr, (size_t)c * 4, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    if (count) *count = c;
    return CRISPY_OK;
}

int crispy_kmer_stream(crispy_ctx* ctx, crispy_sink sink, void* user) {
    if (!ctx || !sink) return CRISPY_E_INPUT;
    KmerJob& j = ctx->kmer;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "kmer_stream before kmer_run");
    const int64_t batch = 1 << 20;
    if (j.spilled) {   // already in host memory
        for (int64_t at = 0; at < j.nsurv; at += batch) {
            const int64_t c = std::min(batch, j.nsurv - at);
            const float* d = j.have_dists ? j.h_spill_dists.as<float>() + at : nullptr;
            if (sink(user, 0, j.h_spill_pairs.as<char>() + at * 8, d, c) != 0)
                return fail(ctx, CRISPY_E_IO, "sink aborted");
        }
        return CRISPY_OK;
    }
    std::vector<int32_t> p((size_t)std::min(batch, std::max<int64_t>(j.nsurv, 1)) * 2);
    std::vector<float> d(j.have_dists ? p.size() / 2 : 0);
    cudaStream_t s = ctx->stream;
    for (int64_t at = 0; at < j.nsurv; at += batch) {
        const int64_t c = std::min(batch, j.nsurv - at);
        CRISPY_CK(ctx, cudaMemcpyAsync(p.data(), j.pairs.as<char>() + at * 8, (size_t)c * 8,
                                       cudaMemcpyDeviceToHost, s));
        if (j.have_dists)
            CRISPY_CK(ctx, cudaMemcpyAsync(d.data(), j.dists.as<char>() + at * 4, (size_t)c * 4,
                                           cudaMemcpyDeviceToHost, s));
        CRISPY_CK(ctx, cudaStreamSynchronize(s));
        if (sink(user, 0, p.data(), j.have_dists ? d.data() : nullptr, c) != 0)
            return fail(ctx, CRISPY_E_IO, "sink aborted");
    }
    return CRISPY_OK;
}

}  // extern "C"

namespace crispy {

// A cohort of k-mer jobs in one batched run (the server's cross-job
// batching): the reads prepared on ctx are the jobs' reads back to back,
// job c at positions [base, base + n) with base a multiple of 128.  One
// persistent 128-row tile launch takes every job's row groups from one work
// queue, each row group only over its own job's columns and with its job's
// threshold tables; the survivors of all jobs are sorted at once (job
// first, then each job's stage order) and decoded to cohort positions.
// On return counts[c] holds job c's survivors, contiguous in job order in
// the context's pair list.  CRISPY_E_UNSUPPORTED when the cohort needs a
// path the cohort form does not take (K > 6, rows for the dense kernel,
// more survivors than the device share): the caller then runs the jobs
// one by one.
// The bound pass's tuned splits, as JSON objects for crispy_tune_report
// (each preceded by ", ").
std::string kmer_tune_json() {
    std::string out;
    std::lock_guard<std::mutex> g(g_ktune_mu);
    for (auto& kv : g_ktuned) {
        char item[256];
        snprintf(item, sizeof item,
                 ", {\"stage\": \"kmer\", \"kernel\": \"kmer_tile128_kernel\", \"reads\": %d, \"k\": %d, "
                 "\"split\": %d, \"sample_row_groups\": %d, \"ms\": %.4f, \"default_ms\": %.4f}",
                 kv.second.n, kv.second.k, kv.second.split, kv.second.row_groups, kv.second.ms_best,
                 kv.second.ms_default);
        out += item;
    }
    return out;
}

int kmer_run_cohort(crispy_ctx* ctx, const std::vector<CohortJob>& jobs, std::vector<int64_t>& counts) {
    KmerJob& j = ctx->kmer;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "kmer cohort before kmer_prepare");
    const int n = j.n, K = j.k;
    const int nj = (int)jobs.size();
    if (K > 6 || nj < 1 || nj > 1024) return fail(ctx, CRISPY_E_UNSUPPORTED, "cohort: K %d, %d jobs", K, nj);
    const int levels = dense_levels_for(K);
    if (levels <= 0) return fail(ctx, CRISPY_E_UNSUPPORTED, "cohort: no shared-memory planes for K %d", K);
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    ctx->stats = crispy_stats{};
    ctx->ev_kmer.used = 0;
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_begin, s));
    // per job: tile size, threshold tables (one block of max_t + 1 entries each)
    std::vector<int4> cj(nj);
    std::vector<int> tbl(nj);
    std::vector<uint16_t> mmin_all, smin_all;
    int key_hi = 0;
    for (int c = 0; c < nj; ++c) {
        const CohortJob& q = jobs[c];
        const int A = crispy_array_dim(q.n);
        if (A <= 0 || q.base % kRows128 != 0 || q.base + q.n > n || q.n > 65536)
            return fail(ctx, CRISPY_E_UNSUPPORTED, "cohort: job %d (n %d at %d) unsupported", c, q.n, q.base);
        const int sd = (q.n + A - 1) / A;
        cj[c] = make_int4(q.base, q.n, A, sd);
        std::vector<uint16_t> mm, sm;
        build_mmin(q.thr, j.max_t, mm, sm);
        tbl[c] = (int)mmin_all.size();
        mmin_all.insert(mmin_all.end(), mm.begin(), mm.end());
        smin_all.insert(smin_all.end(), sm.begin(), sm.end());
        key_hi = std::max(key_hi, bits_for((uint64_t)sd * (sd + 1) / 2 * (uint64_t)q.n * (uint64_t)q.n));
    }
    if (key_hi > 44) return fail(ctx, CRISPY_E_UNSUPPORTED, "cohort: stage keys of %d bits", key_hi);
    // row groups of each job, each over its own job's column groups; rows of
    // 32-read groups with too many high-level entries would need the dense
    // kernel, which the cohort form does not run
    std::vector<int> items, item_job, item_cend;
    std::vector<std::pair<int64_t, int>> order;
    for (int c = 0; c < nj; ++c) {
        const int b = jobs[c].base, e = b + jobs[c].n;
        for (int rg = b / kRows128; rg * kRows128 < e; ++rg) {
            int64_t high = 0;
            for (int r = rg * kRows128; r < std::min(e, rg * kRows128 + kRows128); ++r) high += j.h_cntmax[n + r];
            if (high > kHashMaxKeys) return fail(ctx, CRISPY_E_UNSUPPORTED, "cohort: row group %d needs the dense kernel", rg);
            const int cend = (e + 31) / 32;
            order.push_back({-(int64_t)(cend - 4 * rg), (int)items.size()});
            items.push_back(rg);
            item_job.push_back(c);
            item_cend.push_back(cend);
        }
    }
    // most columns first
    std::sort(order.begin(), order.end());
    std::vector<int> it2(items.size()), ij2(items.size()), ic2(items.size());
    for (size_t i = 0; i < order.size(); ++i) {
        it2[i] = items[order[i].second];
        ij2[i] = item_job[order[i].second];
        ic2[i] = item_cend[order[i].second];
    }
    const size_t ni = it2.size();
    const size_t tb = mmin_all.size();
    // one device block: items | jobs | cends | cjob | tbl | job counters | head | tables
    const size_t off_job = ni * 4, off_cend = off_job + ni * 4, off_cj = (off_cend + ni * 4 + 15) / 16 * 16;
    const size_t off_tbl = off_cj + (size_t)nj * 16, off_cnt = (off_tbl + (size_t)nj * 4 + 7) / 8 * 8;
    const size_t off_head = off_cnt + (size_t)(nj + 1) * 8, off_mm = off_head + 16;
    const size_t off_sm = off_mm + tb * 2, off_dense = off_sm + tb * 2;
    const size_t total_bytes = off_dense + (size_t)j.ngroups + 16;   // dense flags: all zero
    CRISPY_TRY(ensure(ctx, j.work, total_bytes + 16));
    std::vector<char> blob(total_bytes, 0);
    std::memcpy(blob.data(), it2.data(), ni * 4);
    std::memcpy(blob.data() + off_job, ij2.data(), ni * 4);
    std::memcpy(blob.data() + off_cend, ic2.data(), ni * 4);
    std::memcpy(blob.data() + off_cj, cj.data(), (size_t)nj * 16);
    std::memcpy(blob.data() + off_tbl, tbl.data(), (size_t)nj * 4);
    std::memcpy(blob.data() + off_mm, mmin_all.data(), tb * 2);
    std::memcpy(blob.data() + off_sm, smin_all.data(), tb * 2);
    char* d = j.work.as<char>();
    CRISPY_CK(ctx, cudaMemcpyAsync(d, blob.data(), total_bytes, cudaMemcpyHostToDevice, s));
    // survivors: the same capacity rule as a single run over all positions
    const int64_t cap = std::min(kmer_device_pair_cap(), std::max<int64_t>(1 << 20, 16LL * n));
    CRISPY_TRY(ensure(ctx, j.keys, (size_t)cap * 8));
    CRISPY_TRY(ensure(ctx, j.keys_alt, (size_t)cap * 8));
    CRISPY_TRY(ensure(ctx, j.vals, (size_t)cap * 4));
    CRISPY_TRY(ensure(ctx, j.vals_alt, (size_t)cap * 4));
    CRISPY_TRY(ensure(ctx, j.counter, 64));
    CRISPY_CK(ctx, cudaMemsetAsync(j.counter.ptr, 0, 64, s));
    const uint32_t K4 = 1u << (2 * K);
    const int B = std::max(8, bits_for((uint64_t)j.max_t));
    TileFn tile = tile128_fn_for(B);
    const size_t tsmem = ((size_t)levels * K4 + 32) * (kRows128 / 8);
    CRISPY_CK(ctx, cudaFuncSetAttribute(tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
    TileArgs ta{};
    ta.ent = j.ent.as<uint32_t>(); ta.gstart = j.gstart.as<int64_t>(); ta.gent = j.gent.as<int32_t>();
    ta.tent = j.tent.as<uint16_t>(); ta.tstart = j.tstart.as<int64_t>(); ta.tgent = j.tgent.as<int32_t>();
    ta.k65536 = 65536u; ta.k8 = 8u;
    ta.hinfo = j.hinfo.as<uint32_t>(); ta.ngroups = j.ngroups;
    ta.nhigh = j.cntmax.as<int32_t>() + n;
    ta.tcount = j.t.as<int32_t>();
    ta.tgentL = j.tgentL.as<int32_t>();
    ta.nsec = j.split ? j.nsec.as<int32_t>() : nullptr;
    ta.split = j.split;
    ta.bound = j.split != 0;
    ta.qfire = kmer_qfire();
    ta.gstat = j.split ? j.counter.as<unsigned long long>() + 1 : nullptr;
    ta.dense_group = reinterpret_cast<const uint8_t*>(d + off_dense);   // no dense group (checked above)
    ta.mmin = reinterpret_cast<const uint16_t*>(d + off_mm);
    ta.smin = reinterpret_cast<const uint16_t*>(d + off_sm);
    ta.n = n; ta.K4 = K4; ta.levels = levels; ta.A = crispy_array_dim(n); ta.stage_dim = 1;
    ta.counter = j.counter.as<unsigned long long>(); ta.keys = j.keys.as<uint64_t>();
    ta.vals = j.vals.as<uint32_t>(); ta.cap = cap;
    ta.perm = nullptr; ta.olo = 0; ta.ohi = n;
    ta.r_lo = 0; ta.r_hi = n; ta.c_lo = 0; ta.c_hi = n;
    ta.items = reinterpret_cast<const int*>(d); ta.nitems = (int)ni;
    ta.queue_head = reinterpret_cast<unsigned int*>(d + off_head);
    ta.item_job = reinterpret_cast<const int*>(d + off_job);
    ta.item_cend = reinterpret_cast<const int*>(d + off_cend);
    ta.cjob = reinterpret_cast<const int4*>(d + off_cj);
    ta.ctbl = reinterpret_cast<const int*>(d + off_tbl);
    ta.job_counter = reinterpret_cast<unsigned long long*>(d + off_cnt);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tile, kTileThreads, tsmem);
    const int grid = (int)std::min<int64_t>((int64_t)std::max(1, per_sm) * ctx->sm_count, (int64_t)ni);
    if (ni > 0) {
        ev_begin(ctx, ctx->ev_kmer, s);
        tile<<<grid, kTileThreads, tsmem, s>>>(ta);
        ev_end(ctx, ctx->ev_kmer, s);
        count_launch(ctx);
        ctx->stats.kmer_launches += 1;
    }
    CRISPY_CK(ctx, cudaGetLastError());
    unsigned long long cnt[5] = {0, 0, 0, 0, 0};
    std::vector<unsigned long long> jc(nj);
    CRISPY_CK(ctx, cudaMemcpyAsync(cnt, j.counter.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(jc.data(), d + off_cnt, (size_t)nj * 8, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    const unsigned long long total = cnt[0];
    ctx->stats.kmer_bound_entries = (int64_t)cnt[1];
    ctx->stats.kmer_full_entries = (int64_t)cnt[2];
    ctx->stats.kmer_full_columns = (int64_t)cnt[3];
    ctx->stats.kmer_rounds = (int64_t)cnt[4];
    if ((int64_t)total > cap) return fail(ctx, CRISPY_E_UNSUPPORTED, "cohort: %llu survivors beyond the device share", total);
    j.nsurv = (int64_t)total;
    CRISPY_TRY(ensure(ctx, j.pairs, (size_t)std::max<int64_t>(j.nsurv, 1) * 8));
    CRISPY_TRY(ensure(ctx, j.dists, (size_t)std::max<int64_t>(j.nsurv, 1) * 4));
    CRISPY_TRY(ensure(ctx, j.sort_tmp, sort_tmp_bytes(j.nsurv)));
    uint64_t* sk = nullptr;
    uint32_t* sv = nullptr;
    CRISPY_TRY(sort_u64_payload(ctx, s, j.keys.as<uint64_t>(), j.keys_alt.as<uint64_t>(), j.vals.as<uint32_t>(),
                                j.vals_alt.as<uint32_t>(), j.nsurv, 44 + bits_for((uint64_t)nj), true, &sk, &sv,
                                j.sort_tmp));
    if (j.nsurv > 0) {
        kmer_decode_cohort_kernel<<<(unsigned)((j.nsurv + 255) / 256), 256, 0, s>>>(
            sk, sv, j.nsurv, ta.cjob, j.pairs.as<int2>(), j.dists.as<float>());
        count_launch(ctx);
        CRISPY_CK(ctx, cudaGetLastError());
    }
    j.spilled = false;
    j.have_dists = true;
    counts.assign(jc.begin(), jc.end());
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_end, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    float tot = 0;
    cudaEventElapsedTime(&tot, ctx->t_begin, ctx->t_end);
    ctx->stats.total_ms = tot;
    ctx->stats.kmer_kernel_ms = ev_sum_ms(ctx->ev_kmer);
    int64_t pairs = 0;
    for (const CohortJob& q : jobs) pairs += (int64_t)q.n * (q.n - 1) / 2;
    ctx->stats.kmer_pairs = pairs;
    ctx->stats.kmer_survivors = j.nsurv;
    return CRISPY_OK;
}

}  // namespace crispy
