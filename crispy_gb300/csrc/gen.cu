// gen.cu -- genDist on GB300: banded Needleman-Wunsch genetic distance.
//
// Reference semantics (genCPU.cpp:290-466 restated by genKernel.cu:372-780):
// rows i = 1..L2 run over read2 = pair[1], columns j = 1..L1 over read1 =
// pair[0]; cell (i, j) is in band iff |i - j| <= kBand, kBand =
// (L1 + L2) / (2 * band); row 0 / column 0 cells within the band hold
// M = 0, ML = 0, AL = index.  With up = (i, j-1), left = (i-1, j),
//   up   = M[up]   + GO*[up was diag]   + GE*[up was up]      (out of band: -1e6)
//   left = M[left] + GO*[left was diag] + GE*[left was left]  (out of band: -1e6)
//   diag = M[i-1][j-1] + (symbols equal ? 5 : -4)
//   M = max(diag, up, left), ties resolved diag > up > left;
//   ML = diag ? ML_d - match + 1 : ML_pred + 1;  AL = AL_pred + 1.
// The distance takes the last maximum (>=) of the last row and of the last
// column, prefers the column-of-last-row value only when strictly larger,
// and is (float)ML / (float)AL.  Symbols compare as 2-bit codes.
//
// GB300 design: one warp per pair sweeps anti-diagonals s = i + j.  The
// band's cells on one anti-diagonal sit at d = i - j with d = s (mod 2);
// slot q = (d + kBand) / 2 hosts them, so kBand + 1 slots cover the band and
// a slot alternates between diagonals 2q - kBand and 2q - kBand + 1.  Lane l
// owns C consecutive slots in registers.  Per step every slot needs its own
// previous cell (up or left), the neighbouring slot's previous cell (the
// other one) and its own cell two steps back (diag): one shuffle of the
// edge slot per step.  Each cell exports M plus the two gap-penalised copies
// M + pen_up and M + pen_left, so the receiver adds nothing.  Sequences sit
// 2 bits per symbol in shared memory and reach the slots through 16-symbol
// register windows refilled every 30 steps.  Steps away from the matrix
// border run a check-free body.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "gen_args.h"
#include "internal.h"

namespace crispy {
namespace {

constexpr int kNeg = -1048576;          // below any reachable score (|M| < 45,056)
constexpr int kRefNegInf = -1000000;    // genCPU.cpp:350 initial last-row/column maximum
constexpr int kGO = -10, kGE = -1, kMatch = 5, kMismatch = -4;  // genMain.h:32-35
constexpr int kGenThreads = 256;
constexpr int kGenWarps = kGenThreads / 32;
constexpr int kSmWords = 132;           // 128 words of 16 symbols + refill padding

__device__ __forceinline__ int kband_of(int l1, int l2, int band) {
    return band >= 2 ? (l1 + l2) / (2 * band) : max(l1, l2);
}

// 16 symbols starting at position pos (may be negative: zeros shift in).
__device__ __forceinline__ uint32_t window_at(const uint32_t* sm, int pos) {
    if (pos >= 16 * (kSmWords - 2)) return 0u;   // past any read: symbols unused
    if (pos >= 0) {
        const int k = pos >> 4, sh = (pos & 15) * 2;
        return sh ? (sm[k] << sh) | (sm[k + 1] >> (32 - sh)) : sm[k];
    }
    if (pos > -16) return sm[0] >> (-pos * 2);
    return 0u;
}

struct Best {
    int m;
    uint32_t l;
    int at;
};

__device__ __forceinline__ void track(Best& b, int m, uint32_t l, int at) {
    if (m >= b.m) { b.m = m; b.l = l; b.at = at; }
}

// Largest m over a G-lane sub-group, ties to the largest index `at`;
// returns the winner's packed ML|AL.
template <int G>
__device__ __forceinline__ Best group_best(Best b, int lane) {
    const long long mine = (long long)b.m * 4294967296LL + (long long)(unsigned)(b.at + 1);
    long long key = mine;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        long long other = __shfl_xor_sync(0xffffffffu, key, o);
        key = other > key ? other : key;
    }
    const unsigned group = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const unsigned who = __ballot_sync(0xffffffffu, mine == key) & group;
    const int src = __ffs(who) - 1;
    Best r;
    r.m = (int)(key >> 32);
    r.at = (int)(unsigned)(key & 0xffffffffu) - 1;
    r.l = __shfl_sync(0xffffffffu, b.l, src);
    return r;
}

// Scores are stored as V = M + 2s on anti-diagonal s = i + j.  All three
// candidates of a cell then carry the same offset 2s, so the maxima and
// tie-breaks are those of M, while the diagonal candidate becomes
// V(s-2) + 9*match and a gap candidate V(s-1) + pen + 2.
//
// ML and AL travel packed as (A << 16) | B with A = diagonal moves on the
// path and B = (i0 + j0) + A + matches, (i0, j0) the boundary cell the path
// starts from (whose packed value i0 + j0 is the reference's AL there, ML
// 0).  A diagonal move adds 0x10001 + match, a gap move adds nothing, and at
// the end ML = (i + j) - B, AL = (i + j) - A.
// A step at parity P reads the cells of steps s-2 (M[P], L[P]: the
// diagonal) and s-1 (M[P^1], L[P^1], U, F) and writes its cells over
// M[P], L[P], U and F.  So the buffers alternate by parity and nothing
// rotates; U and F update in place, slots ordered so that a neighbour is
// read before it is overwritten.
template <int C>
struct Lane {
    int M[2][C];               // V by step parity
    uint32_t L[2][C];          // packed path counters by step parity
    int U[C], F[C];            // gap-penalised copies (+2) of the last step
    uint32_t x0[C], x1[C];     // per-slot symbol XOR fields of the block, by parity
    int cap0[C], cap1[C];      // kNeg for a parity whose diagonal is out of band
};

// Per-pair values a sub-group holds (the same in all its lanes).
struct PairCtx {
    int kb, l1, l2, shift;   // shift = kb & 1: odd bands run one step late
    const int* one;          // GenArgs::one
};

// Block kinds.  kClean: no cell of the block touches the matrix border.
// kTrack: no boundary cell and no cell before the matrix (s >= kBand + 2),
// but last-row / last-column cells may appear; cells past the matrix are
// computed and ignored, since no in-matrix cell depends on them.  kFull:
// boundary cells, cells before the matrix and tracking.
constexpr int kClean = 0, kTrack = 1, kFull = 2;

// One anti-diagonal step at parity P for all C slots of this lane, the
// slot's F-th cell of this parity inside the current group of three.  The
// sub-group's own step is s = t - shift, which makes P = t & 1 for every
// sub-group of the warp.  dbase = 2*gl*C - kBand is the parity-0 diagonal
// of the lane's first slot.
template <int G, int C, int P, int F, int kMode>
__device__ __forceinline__ void step(Lane<C>& st, int gl, int s, int dbase, const PairCtx& pc,
                                     Best& col, Best& row) {
    constexpr int Q = P ^ 1;   // buffers of the previous step
    int nbM;
    uint32_t nbL;
    if (P == 0) {
        // left = slot q-1 (its gap-left copy), from the previous lane for c = 0
        nbM = __shfl_up_sync(0xffffffffu, st.F[C - 1], 1, G);
        nbL = __shfl_up_sync(0xffffffffu, st.L[Q][C - 1], 1, G);
        if (gl == 0) nbM = kNeg;
    } else {
        // up = slot q+1 (its gap-up copy), from the next lane for c = C-1
        nbM = __shfl_down_sync(0xffffffffu, st.U[0], 1, G);
        nbL = __shfl_down_sync(0xffffffffu, st.L[Q][0], 1, G);
        if (gl == G - 1) nbM = kNeg;
    }
#pragma unroll
    for (int k = 0; k < C; ++k) {
        // parity 0 reads slot c-1, so it runs c downwards; parity 1 reads
        // slot c+1 and runs upwards
        const int c = P == 0 ? C - 1 - k : k;
        int upM, lfM;
        uint32_t upL, lfL;
        if (P == 0) {
            upM = st.U[c]; upL = st.L[Q][c];
            lfM = c > 0 ? st.F[c - 1] : nbM;
            lfL = c > 0 ? st.L[Q][c - 1] : nbL;
        } else {
            upM = c < C - 1 ? st.U[c + 1] : nbM;
            upL = c < C - 1 ? st.L[Q][c + 1] : nbL;
            lfM = st.F[c]; lfL = st.L[Q][c];
        }
        const uint32_t xf = P == 0 ? st.x0[c] : st.x1[c];
        const bool match = (xf & (0xC0000000u >> (2 * F))) == 0u;
        // The ALU pipe carries the compares, maxima and selects; most adds
        // are multiply-adds by pc.one[] (runtime 1s) so that they issue on
        // the FMA pipe.
        const int pM = st.M[P][c];
        const uint32_t pL = st.L[P][c];
        int md = pM;
        if (match) md = pM * pc.one[0] + (kMatch - kMismatch);
        // max with predicate: isU = up >= left (up wins ties over left),
        // isD = diag >= max(up, left) (diag wins every tie)
        bool isU, isD;
        const int mul = __vibmax_s32(upM, lfM, &isU);
        const int mx = __vibmax_s32(md, mul, &isD);
        uint32_t ld = pL * (uint32_t)pc.one[1] + 0x10001u;
        if (match) ld = pL * (uint32_t)pc.one[2] + 0x10002u;
        uint32_t l = isD ? ld : (isU ? upL : lfL);
        int m = min(mx, P == 0 ? st.cap0[c] : st.cap1[c]);
        // gap-penalised copies (+2 offset): D -8/-8, U +1/+2, L +2/+1
        int u = m + 2, f = m + (2 + kGE);
        if (isU) { u = m * pc.one[3] + (2 + kGE); f = m * pc.one[4] + 2; }
        if (isD) { u = m * pc.one[5] + (2 + kGO); f = u; }
        if (kMode == kFull) {
            const int d = dbase + 2 * c + P;
            const int i = (s + d) >> 1, j = (s - d) >> 1;
            if (m == kNeg || i < 0 || j < 0) {
                m = kNeg; u = kNeg; f = kNeg; l = 0;
            } else if (i == 0 || j == 0) {
                m = 2 * s; u = m + 2; f = m + 2; l = (uint32_t)(i + j);
            } else {
                if (i == pc.l2 && j <= pc.l1) track(col, m - 2 * s, l, j);
                if (j == pc.l1 && i <= pc.l2) track(row, m - 2 * s, l, i);
            }
        }
        st.M[P][c] = m; st.L[P][c] = l; st.U[c] = u; st.F[c] = f;
    }
    if (kMode == kTrack) {
        // slot c sits on the last row when x + 2c == 0 (2i = 2*l2) and on
        // the last column when y - 2c == 0 (2j = 2*l1): once per slot and
        // parity, so one range test per step guards the rare work
        const int d0 = dbase + P;
        const int x = s + d0 - 2 * pc.l2;
        const int y = s - d0 - 2 * pc.l1;
        if ((x <= 0 && x > -2 * C) || (y >= 0 && y < 2 * C)) {
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int m = st.M[P][c];
                if (m == kNeg) continue;   // out of band
                const int i = (s + d0 + 2 * c) >> 1, j = (s - d0 - 2 * c) >> 1;
                if (x + 2 * c == 0 && j >= 1 && j <= pc.l1) track(col, m - 2 * s, st.L[P][c], j);
                if (y - 2 * c == 0 && i >= 1 && i <= pc.l2) track(row, m - 2 * s, st.L[P][c], i);
            }
        }
    }
}

// A block of kBlockSteps = 30 steps gives each slot 15 cells per parity;
// the symbols they compare are fields 0..14 of the XOR words built from the
// 16-symbol windows at the block start.  Groups of six steps test fields
// F = 0, 1, 2 and then shift the XOR words by three fields.
constexpr int kBlockSteps = 30;

template <int G, int C, int kMode>
__device__ __forceinline__ void block_steps(Lane<C>& st, int gl, int s0, const PairCtx& pc,
                                            Best& col, Best& row) {
    const int dbase = 2 * gl * C - pc.kb;
    if constexpr (kMode != kClean) {
        // the rarer border and tracking blocks: a two-step body that always
        // tests field 0 keeps their code small (instruction fetch)
#pragma unroll 1
        for (int t = 0; t < kBlockSteps; t += 2) {
            step<G, C, 0, 0, kMode>(st, gl, s0 + t, dbase, pc, col, row);
            step<G, C, 1, 0, kMode>(st, gl, s0 + t + 1, dbase, pc, col, row);
#pragma unroll
            for (int c = 0; c < C; ++c) { st.x0[c] <<= 2; st.x1[c] <<= 2; }
        }
    } else {
#pragma unroll 1
        for (int t = 0; t < kBlockSteps; t += 6) {
            step<G, C, 0, 0, kMode>(st, gl, s0 + t, dbase, pc, col, row);
            step<G, C, 1, 0, kMode>(st, gl, s0 + t + 1, dbase, pc, col, row);
            step<G, C, 0, 1, kMode>(st, gl, s0 + t + 2, dbase, pc, col, row);
            step<G, C, 1, 1, kMode>(st, gl, s0 + t + 3, dbase, pc, col, row);
            step<G, C, 0, 2, kMode>(st, gl, s0 + t + 4, dbase, pc, col, row);
            step<G, C, 1, 2, kMode>(st, gl, s0 + t + 5, dbase, pc, col, row);
#pragma unroll
            for (int c = 0; c < C; ++c) { st.x0[c] <<= 6; st.x1[c] <<= 6; }
        }
    }
}

template <int G, int C>
__device__ void align_sweep(Lane<C>& st, const uint32_t* sm1, const uint32_t* sm2, int gl,
                            const PairCtx& pc, int t_end, Best& col, Best& row) {
    const int clean_hi = 2 * min(pc.l1, pc.l2) - pc.kb - 1;
    for (int t0 = 0; t0 <= t_end; t0 += kBlockSteps) {
        const int s0 = t0 - pc.shift;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int d = 2 * (gl * C + c) - pc.kb;   // parity 0 at the block start
            const int i = (s0 + d) >> 1, j = (s0 - d) >> 1;
            // parity-0 cells compare read1[j-1+k] with read2[i-1+k],
            // parity-1 cells read1[j-1+k] with read2[i+k]
            const uint32_t w2 = window_at(sm2, i - 1);
            const uint32_t w1 = window_at(sm1, j - 1);
            st.x0[c] = w1 ^ w2;
            st.x1[c] = w1 ^ (w2 << 2);
        }
        const bool started = s0 >= pc.kb + 2;
        const bool clean = started && s0 + kBlockSteps - 1 < clean_hi;
        if (__all_sync(0xffffffffu, clean))
            block_steps<G, C, kClean>(st, gl, s0, pc, col, row);
        else if (__all_sync(0xffffffffu, started))
            block_steps<G, C, kTrack>(st, gl, s0, pc, col, row);
        else
            block_steps<G, C, kFull>(st, gl, s0, pc, col, row);
    }
}

// Packed (A << 16) | B of the chosen last-row / last-column cell -> ML, AL.
__device__ __forceinline__ void unpack_mlal(uint32_t l, int ij, int* ml, int* al) {
    if (ij < 0) { *ml = 0; *al = 0; return; }   // no tracked cell (reference: ML = AL = 0)
    *ml = ij - (int)(l & 0xffffu);
    *al = ij - (int)(l >> 16);
}

// One pair per G-lane sub-group (32/G pairs per warp), C band slots per
// lane, so a pair with kBand + 1 <= G*C slots fits.
template <int G, int C>
__global__ void __launch_bounds__(kGenThreads, C <= 3 ? 3 : (C <= 5 ? 2 : 1)) gen_warp_kernel(GenArgs a) {
    constexpr int kPerWarp = 32 / G;
    __shared__ uint32_t smem[kGenWarps][kPerWarp][2][kSmWords];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / G, gl = lane % G;
    uint32_t* sm1 = smem[warp][sub][0];
    uint32_t* sm2 = smem[warp][sub][1];
    int64_t base = a.queue ? -1 : ((int64_t)blockIdx.x * kGenWarps + warp) * kPerWarp;
    const int64_t stride = (int64_t)gridDim.x * kGenWarps * kPerWarp;
    for (;;) {
        if (a.queue) {
            unsigned w = 0;
            if (lane == 0) w = atomicAdd(a.queue, (unsigned)kPerWarp);
            base = __shfl_sync(0xffffffffu, w, 0);
        }
        if (base >= a.count) break;
        const int64_t item = base + sub;
        const bool valid = item < a.count;
        int64_t p = -1;
        PairCtx pc{0, 0, 0, 0, a.one};   // a.one decays to the kernel parameter array
        int2 pr = make_int2(0, 0);
        if (valid) {
            p = a.order ? (int64_t)a.order[item] : item;
            pr = a.pairs[p];
            pc.l1 = a.len[pr.x];
            pc.l2 = a.len[pr.y];
            pc.kb = kband_of(pc.l1, pc.l2, a.band);
        }
        pc.shift = pc.kb & 1;
        const int nw1 = (pc.l1 + 15) >> 4, nw2 = (pc.l2 + 15) >> 4;
        const uint32_t* g1 = a.packed + (valid ? a.woff[pr.x] : 0);
        const uint32_t* g2 = a.packed + (valid ? a.woff[pr.y] : 0);
        for (int k = gl; k < kSmWords; k += G) {
            sm1[k] = k < nw1 ? g1[k] : 0u;
            sm2[k] = k < nw2 ? g2[k] : 0u;
        }
        __syncwarp();
        Lane<C> st;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            st.M[0][c] = kNeg; st.M[1][c] = kNeg; st.U[c] = kNeg; st.F[c] = kNeg;
            st.L[0][c] = 0; st.L[1][c] = 0;
            // slot q hosts diagonals 2q - kb (parity 0) and 2q - kb + 1
            const int q = gl * C + c;
            st.cap0[c] = valid && 2 * q - pc.kb <= pc.kb ? INT_MAX : kNeg;
            st.cap1[c] = valid && 2 * q - pc.kb + 1 <= pc.kb ? INT_MAX : kNeg;
        }
        Best col{kRefNegInf, 0u, -1}, row{kRefNegInf, 0u, -1};
        // the sweep ends at the last in-band cell of the last row or column
        int s_end = 0;
        if (valid) {
            if (max(1, pc.l2 - pc.kb) <= min(pc.l1, pc.l2 + pc.kb)) s_end = pc.l2 + min(pc.l1, pc.l2 + pc.kb);
            if (max(1, pc.l1 - pc.kb) <= min(pc.l2, pc.l1 + pc.kb))
                s_end = max(s_end, pc.l1 + min(pc.l2, pc.l1 + pc.kb));
        }
        const int t_end = (int)__reduce_max_sync(0xffffffffu, (unsigned)(s_end + pc.shift));
        align_sweep<G, C>(st, sm1, sm2, gl, pc, t_end, col, row);
        col = group_best<G>(col, lane);
        row = group_best<G>(row, lane);
        if (gl == 0 && valid) {
            const bool use_col = col.m > row.m;   // genKernel.cu:765-768
            int mlv, alv;
            if (use_col) unpack_mlal(col.l, col.at < 0 ? -1 : pc.l2 + col.at, &mlv, &alv);
            else unpack_mlal(row.l, row.at < 0 ? -1 : row.at + pc.l1, &mlv, &alv);
            a.dist[p] = __fdiv_rn((float)mlv, (float)alv);
            if (a.score) a.score[p] = use_col ? col.m : row.m;
            if (a.ml) a.ml[p] = mlv;
            if (a.al) a.al[p] = alv;
        }
        __syncwarp();
        if (!a.queue) base += stride;
    }
}

// ---------------------------------------------------------------------------
// Wide-band path (kBand + 1 > 32 * 8 slots, e.g. -b 1, or -b 2 on long
// reads): one thread per pair, two band rows in global scratch, row by row
// over band cells only.  Same recurrence and tie-breaks.  Band coordinates:
// cell (i, j) sits at x = j - i + kBand + 1 in its row, so diag = (row-1, x),
// left = (row-1, x+1), up = (row, x-1); x = 0 and x = 2*kBand + 2 are guard
// slots that stay at the out-of-band sentinel.
// ---------------------------------------------------------------------------
struct WideArgs {
    GenArgs g;
    int* scratch;        // per thread: 2 rows x {M, code, ML|AL} x row_stride ints
    int row_stride;      // 2 * kbmax + 3
};

__device__ __forceinline__ uint32_t sym_at(const uint32_t* s, int p) {
    return (s[p >> 4] >> (30 - 2 * (p & 15))) & 3u;
}

__global__ void __launch_bounds__(128) gen_wide_kernel(WideArgs w) {
    const GenArgs& a = w.g;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const int rs = w.row_stride;
    int* base = w.scratch + tid * (int64_t)rs * 6;
    for (int64_t item = tid; item < a.count; item += nthreads) {
        const int64_t p = a.order ? (int64_t)a.order[item] : item;
        const int2 pr = a.pairs[p];
        const int l1 = a.len[pr.x], l2 = a.len[pr.y];
        const int kb = kband_of(l1, l2, a.band);
        const int width = 2 * kb + 3;
        const uint32_t* s1 = a.packed + a.woff[pr.x];
        const uint32_t* s2 = a.packed + a.woff[pr.y];
        int* rowM[2] = {base, base + 3 * rs};
        int* rowC[2] = {base + rs, base + 4 * rs};     // 0 boundary, 1 diag, 2 left, 4 up
        int* rowL[2] = {base + 2 * rs, base + 5 * rs};
        for (int x = 0; x < width; ++x) { rowM[0][x] = kNeg; rowC[0][x] = 0; rowL[0][x] = 0; }
        for (int j = 0; j <= min(kb, l1); ++j) {     // row 0 (genCPU.cpp:367-379)
            rowM[0][j + kb + 1] = 0; rowL[0][j + kb + 1] = j;
        }
        Best col{kRefNegInf, 0u, -1}, row{kRefNegInf, 0u, -1};
        int cur = 0;
        for (int i = 1; i <= l2; ++i) {
            const int pre = cur;
            cur ^= 1;
            int* Mc = rowM[cur]; int* Cc = rowC[cur]; int* Lc = rowL[cur];
            const int* Mp = rowM[pre]; const int* Cp = rowC[pre]; const int* Lp = rowL[pre];
            for (int x = 0; x < width; ++x) { Mc[x] = kNeg; Cc[x] = 0; Lc[x] = 0; }
            if (i <= kb) { Mc[kb - i + 1] = 0; Lc[kb - i + 1] = i; }   // column 0
            const uint32_t c2 = sym_at(s2, i - 1);
            const int jlo = max(1, i - kb), jhi = min(l1, i + kb);
            for (int j = jlo; j <= jhi; ++j) {
                const int x = j - i + kb + 1;
                const bool match = sym_at(s1, j - 1) == c2;
                const int md = Mp[x] + (match ? kMatch : kMismatch);
                const int cu = Cc[x - 1], cl = Cp[x + 1];
                const int upM = Mc[x - 1] + (cu == 1 ? kGO : (cu == 4 ? kGE : 0));
                const int lfM = Mp[x + 1] + (cl == 1 ? kGO : (cl == 2 ? kGE : 0));
                const int mx = max(md, max(upM, lfM));
                uint32_t l;
                int code;
                if (mx == md) { code = 1; l = (uint32_t)Lp[x] + (match ? 0x1u : 0x10001u); }
                else if (mx == upM) { code = 4; l = (uint32_t)Lc[x - 1] + 0x10001u; }
                else { code = 2; l = (uint32_t)Lp[x + 1] + 0x10001u; }
                Mc[x] = mx; Cc[x] = code; Lc[x] = (int)l;
                if (i == l2) track(col, mx, l, j);
                if (j == l1) track(row, mx, l, i);
            }
        }
        const bool use_col = col.m > row.m;
        const uint32_t l = use_col ? col.l : row.l;
        const int mlv = (int)(l >> 16), alv = (int)(l & 0xffffu);
        a.dist[p] = __fdiv_rn((float)mlv, (float)alv);
        if (a.score) a.score[p] = use_col ? col.m : row.m;
        if (a.ml) a.ml[p] = mlv;
        if (a.al) a.al[p] = alv;
    }
}

// 2-bit packing, 16 symbols per word, first symbol in the top bits
// (the reference packs 4 per ushort the same way, genMain.cpp:280-321).
__global__ void gen_pack_kernel(const uint8_t* __restrict__ seq, const int64_t* __restrict__ off,
                                const int32_t* __restrict__ len, const int64_t* __restrict__ woff,
                                int n, uint32_t* __restrict__ packed) {
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        const int L = len[r];
        const int nw = (L + 15) >> 4;
        const uint8_t* s = seq + off[r];
        for (int k = threadIdx.x; k < nw; k += blockDim.x) {
            uint32_t w = 0;
            for (int q = 0; q < 16; ++q) {
                const int p = k * 16 + q;
                uint32_t c = 0;
                if (p < L) {
                    const uint8_t ch = s[p];
                    c = ch == 'G' ? 1u : ch == 'T' ? 2u : ch == 'C' ? 3u : 0u;
                }
                w |= c << (30 - 2 * q);
            }
            packed[woff[r] + k] = w;
        }
    }
}

// genCUDA.cu:219: keep iff dist < thr or |dist - thr| < 1e-5 (float
// subtraction, double comparison).
__global__ void gen_flag_kernel(const float* __restrict__ dist, int64_t n, float thr,
                                uint8_t* __restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = dist[i];
    flags[i] = (d < thr || (double)fabsf(__fsub_rn(d, thr)) < 0.00001) ? 1 : 0;
}

__global__ void gen_keys_kernel(const float* __restrict__ dist, const uint32_t* __restrict__ surv,
                                int64_t base, int64_t count, uint32_t* __restrict__ keys,
                                uint32_t* __restrict__ vals) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t p = surv[base + i];
    keys[i] = __float_as_uint(dist[p]);
    vals[i] = p;
}

// pair_base: the job's first position in a cohort's read set (0 otherwise),
// so that output pairs hold the job's own read indices.
__global__ void gen_gather_kernel(const int2* __restrict__ pairs, const uint32_t* __restrict__ keys,
                                  const uint32_t* __restrict__ vals, int64_t count,
                                  uint2* __restrict__ out_pairs, float* __restrict__ out_dists,
                                  int pair_base = 0) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int2 pr = pairs[vals[i]];
    out_pairs[i] = make_uint2((uint32_t)(pr.x - pair_base), (uint32_t)(pr.y - pair_base));
    out_dists[i] = __uint_as_float(keys[i]);
}

// Windowed runs: append one load window's survivors (pair, distance) to the
// pending chunk, and key a pending chunk by its position for the stable sort.
__global__ void gen_append_kernel(const int2* __restrict__ pairs, const float* __restrict__ dist,
                                  const uint32_t* __restrict__ surv, int64_t base, int64_t count,
                                  int2* __restrict__ acc_pairs, float* __restrict__ acc_dists) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t p = surv[base + i];
    acc_pairs[i] = pairs[p];
    acc_dists[i] = dist[p];
}

__global__ void gen_poskeys_kernel(const float* __restrict__ dist, int64_t count,
                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    keys[i] = __float_as_uint(dist[i]);
    vals[i] = (uint32_t)i;
}

// Band cells of one pair in O(1): rows i = 1..l2 hold columns
// max(1, i-kb)..min(l1, i+kb), non-empty for i <= min(l2, l1 + kb).
__host__ __device__ inline int64_t band_cells_of(int l1, int l2, int band) {
    const int64_t kb = band >= 2 ? (l1 + l2) / (2 * band) : (l1 > l2 ? l1 : l2);
    if (l1 <= 0 || l2 <= 0) return 0;
    const int64_t I = l2 < l1 + kb ? l2 : l1 + kb;
    int64_t a = l1 - kb > 0 ? l1 - kb : 0;
    a = a < I ? a : I;
    const int64_t sum_hi = a * (a + 1) / 2 + a * kb + (I - a) * l1;
    const int64_t b = kb + 1 < I ? kb + 1 : I;
    const int64_t sum_lo = b + (I * (I + 1) / 2 - b * (b + 1) / 2) - kb * (I - b);
    return sum_hi - sum_lo + I;
}


// Register-resident shapes (sub-group lanes G, band slots per lane C).
// Every one serves a pair with kBand + 1 <= G * C.
struct Shape {
    int g, c;
};
constexpr Shape kShapes[] = {{8, 1},  {8, 2},  {8, 4},  {16, 1}, {16, 2}, {16, 3}, {16, 4},
                             {16, 6}, {32, 1}, {32, 2}, {32, 3}, {32, 4}, {32, 6}, {32, 8},
                             {8, 5},  {8, 7},  {16, 5}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

// Pairs are binned by band slots; bin 0 is the wide-band kernel.  Bins are
// fine where bands are common (kBand 31-79 at band 10 on 300-800 nt reads)
// so that few slots of a pair sit outside its band.
constexpr int kBinSlots[] = {0, 8, 16, 32, 40, 48, 56, 64, 80, 96, 128, 192, 256};
constexpr int kNumBins = sizeof(kBinSlots) / sizeof(kBinSlots[0]);
__constant__ int c_bin_slots[kNumBins] = {0, 8, 16, 32, 40, 48, 56, 64, 80, 96, 128, 192, 256};
// the sort key holds the order-bin (up to 2 * kNumBins) in 5 bits
static_assert(2 * kNumBins < 32, "order-bins overflow the 18-bit sort key");

// Per-pair classification for the launch plan, on the device.  Order-bin
// ob: band-slot bin b (1..12) for a pair the 16-bit kernel takes (L1 + L2
// <= kGen16MaxSum), kNumBins + b for a longer pair (32-bit kernels), and
// 2 * kNumBins for the wide-band kernel (last).  Sort key: order-bin, then
// longer sweeps first (the anti-diagonal of the pair's last in-band cell of
// the last row or column, where the register kernels stop), so that the
// pairs of a warp, which runs until its longest sweep ends, end together.
// stats: [0] cells, [1] max kBand, [kStatBins + ob] pairs of order-bin ob,
// [kStatMaxSum16] the largest L1 + L2 of a pair the 16-bit kernel takes
// (it sizes that kernel's tag storage), [kStatWindows + 2w] widest band-slot
// bin of load window w (kNumBins = wide), [kStatWindows + 2w + 1] 1 when
// the window holds a pair beyond the 16-bit range.
constexpr int kStatBins = 2, kStatWindows = 32;
constexpr int kWideOrderBin = 2 * kNumBins;
constexpr int kStatMaxSum16 = kStatBins + kWideOrderBin + 1;
__global__ void gen_classify_kernel(const int2* __restrict__ pairs, int64_t count,
                                    const int32_t* __restrict__ len, int band, int nbins,
                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                    unsigned long long* __restrict__ stats) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool ok = p < count;
    unsigned long long cells = 0;
    int kb = 0, ob = -1, wb = -1, lng = 0;
    int sum_reg = 0;   // L1 + L2 of a pair for the register kernels' 16-bit form
    if (ok) {
        const int2 pr = pairs[p];
        const int l1 = len[pr.x], l2 = len[pr.y];
        kb = band >= 2 ? (l1 + l2) / (2 * band) : max(l1, l2);
        int bin = 0;
        for (int b = 1; b < nbins; ++b)
            if (c_bin_slots[b] >= kb + 1) { bin = b; break; }
        lng = l1 + l2 > kGen16MaxSum ? 1 : 0;
        if (bin != 0 && !lng) sum_reg = l1 + l2;
        wb = bin == 0 ? nbins : bin;
        ob = bin == 0 ? 2 * nbins : bin + lng * nbins;   // wide pairs sort last
        if (keys) {
            int se = 0;
            if (max(1, l2 - kb) <= min(l1, l2 + kb)) se = l2 + min(l1, l2 + kb);
            if (max(1, l1 - kb) <= min(l2, l1 + kb)) se = max(se, l1 + min(l2, l1 + kb));
            keys[p] = ((uint32_t)ob << 13) | (uint32_t)(8191 - min(se + (kb & 1), 8191));
            vals[p] = (uint32_t)p;
        }
        cells = (unsigned long long)band_cells_of(l1, l2, band);
    }
    // one atomic per warp and counter: the counters are few and shared by
    // every pair, so per-pair atomics would serialise
    cells = __reduce_add_sync(0xffffffffu, (unsigned)cells) + 0ull;   // cells < 2^32 per warp
    const unsigned kbw = __reduce_max_sync(0xffffffffu, (unsigned)kb);
    const unsigned sum16 = __reduce_max_sync(0xffffffffu, (unsigned)sum_reg);
    if (lane == 0) {
        if (cells) atomicAdd(&stats[0], cells);
        atomicMax(&stats[1], (unsigned long long)kbw);
        if (sum16) atomicMax(&stats[kStatMaxSum16], (unsigned long long)sum16);
    }
    const unsigned same_bin = __match_any_sync(0xffffffffu, ob);
    if (ok && lane == __ffs(same_bin) - 1) atomicAdd(&stats[kStatBins + ob], (unsigned long long)__popc(same_bin));
    const int64_t win = ok ? p / CRISPY_GEN_WINDOW : -1;
    const unsigned same_win = __match_any_sync(0xffffffffu, (unsigned long long)win);
    const int wbw = __reduce_max_sync(same_win, wb);   // max over the lanes of this window
    const int lw = __reduce_max_sync(same_win, lng);
    if (ok && lane == __ffs(same_win) - 1) {
        atomicMax(&stats[kStatWindows + 2 * win], (unsigned long long)wbw);
        if (lw) atomicMax(&stats[kStatWindows + 2 * win + 1], 1ull);
    }
}
// untuned 32-bit shape per bin (the plain form always uses it)
constexpr int kDefaultShape[kNumBins] = {-1, 0, 3, 4, 14, 5, 15, 6, 16, 7, 11, 12, 13};
static_assert(kStatMaxSum16 < kStatWindows, "per-bin counters overlap the window slots");

using WarpFn = void (*)(GenArgs);
WarpFn shape_fn(int shape) {
    switch (shape) {
        case 0: return gen_warp_kernel<8, 1>;
        case 1: return gen_warp_kernel<8, 2>;
        case 2: return gen_warp_kernel<8, 4>;
        case 3: return gen_warp_kernel<16, 1>;
        case 4: return gen_warp_kernel<16, 2>;
        case 5: return gen_warp_kernel<16, 3>;
        case 6: return gen_warp_kernel<16, 4>;
        case 7: return gen_warp_kernel<16, 6>;
        case 8: return gen_warp_kernel<32, 1>;
        case 9: return gen_warp_kernel<32, 2>;
        case 10: return gen_warp_kernel<32, 3>;
        case 11: return gen_warp_kernel<32, 4>;
        case 12: return gen_warp_kernel<32, 6>;
        case 13: return gen_warp_kernel<32, 8>;
        case 14: return gen_warp_kernel<8, 5>;
        case 15: return gen_warp_kernel<8, 7>;
        default: return gen_warp_kernel<16, 5>;
    }
}

// ---------------------------------------------------------------------------
// Autotuner: for each bin of a batched run, every shape that covers the bin
// without wasting more than half its slots is timed (CUDA events) on a
// strided sample of the bin's pairs; the fastest is cached per (band, bin,
// length bucket, SM count) for the life of the process.  Any shape gives the
// same bits, so tuning only picks speed.
// ---------------------------------------------------------------------------
struct TuneKey {
    int band, bin, len_bucket, sms;   // bin = order-bin (above kNumBins: pairs beyond the 16-bit range)
    bool operator<(const TuneKey& o) const {
        return std::tie(band, bin, len_bucket, sms) < std::tie(o.band, o.bin, o.len_bucket, o.sms);
    }
};
struct TuneEntry {
    int shape;
    float ms_best, ms_default;
    int64_t sample;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tuned;

bool autotune_enabled() {
    const char* e = std::getenv("CRISPY_AUTOTUNE");
    return !(e && e[0] == '0');
}

// Shape indices: 0..kNumShapes-1 the 32-bit kernel (kShapes), kNumShapes + i
// the 16-bit kernel's shape i (gen16.cu).
int num_shapes_all() { return kNumShapes + gen16_num_shapes(); }
bool is16(int shape) { return shape >= kNumShapes; }
int shape_slots(int shape) {
    if (is16(shape)) {
        const Shape16 h = gen16_shape(shape - kNumShapes);
        return 2 * h.g * h.r;
    }
    return kShapes[shape].g * kShapes[shape].c;
}
// untuned 16-bit shape per bin (index into gen16's shapes), -1 = none
constexpr int kDefault16[kNumBins] = {-1, 0, 1, 2, 4, 5, 7, 8, 9, 10, 11, 12, 13};
int default_shape(int order_bin) {
    if (order_bin >= 1 && order_bin < kNumBins && kDefault16[order_bin] >= 0)
        return kNumShapes + kDefault16[order_bin];
    return kDefaultShape[order_bin > kNumBins ? order_bin - kNumBins : order_bin];
}

// CRISPY_GEN_SHAPE=<index> makes the batched form run every bin the shape
// covers in that shape (tests reach each shape this way); unset or out of
// range: the autotuned shape.
int forced_shape() {
    const char* e = std::getenv("CRISPY_GEN_SHAPE");
    if (!e || !*e) return -1;
    const int v = std::atoi(e);
    return v >= 0 && v < num_shapes_all() ? v : -1;
}

int launch_shape(crispy_ctx* ctx, cudaStream_t s, int shape, GenArgs a, bool timed) {
    if (is16(shape)) return gen16_launch(ctx, s, shape - kNumShapes, a, timed);
    WarpFn fn = shape_fn(shape);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kGenThreads, 0);
    const int64_t per_block = (int64_t)kGenWarps * (32 / kShapes[shape].g);
    const int blocks = (int)std::min<int64_t>((int64_t)std::max(1, per_sm) * ctx->sm_count,
                                              (a.count + per_block - 1) / per_block);
    if (timed) ev_begin(ctx, ctx->ev_gen, s);
    fn<<<std::max(blocks, 1), kGenThreads, 0, s>>>(a);
    if (timed) ev_end(ctx, ctx->ev_gen, s);
    count_launch(ctx);
    return CRISPY_OK;
}

__global__ void gather_stride_kernel(const uint32_t* __restrict__ src, int64_t n, int64_t want,
                                     uint32_t* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < want) dst[i] = src[i * n / want];
}

// Status; the shape in *out.
int pick_shape(crispy_ctx* ctx, cudaStream_t s, int band, int bin, const GenArgs& a,
               const uint32_t* d_order, int64_t n_items, DevBuf& sample_buf, DevBuf& queue_buf,
               DevBuf& dirs_buf, int* out) {
    const int dflt = default_shape(bin);
    *out = dflt;
    if (!autotune_enabled() || n_items < 4096) return CRISPY_OK;
    const TuneKey key{band, bin, 0, ctx->sm_count};
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            *out = it->second.shape;
            return CRISPY_OK;
        }
    }
    // strided sample of the bin (keeps its length spread), taken on the device
    const int64_t want = std::min<int64_t>(n_items, 24576);
    CRISPY_TRY(ensure(ctx, sample_buf, (size_t)want * 4));
    CRISPY_TRY(ensure(ctx, queue_buf, 64 * 4));
    gather_stride_kernel<<<(unsigned)((want + 255) / 256), 256, 0, s>>>(d_order, n_items, want,
                                                                      sample_buf.as<uint32_t>());
    count_launch(ctx);
    const int need = kBinSlots[bin < kNumBins ? bin : bin - kNumBins];
    auto candidate = [&](int sh) {
        const int slots = shape_slots(sh);
        return slots >= need && slots <= 2 * need && !(is16(sh) && bin >= kNumBins);
    };
    int64_t dir_words = 0;   // tag storage of the 16-bit candidates
    for (int sh = 0; sh < num_shapes_all(); ++sh)
        if (candidate(sh) && is16(sh))
            dir_words = std::max(dir_words, gen16_dir_words(ctx, sh - kNumShapes, want, a.dir_blocks));
    if (dir_words) CRISPY_TRY(ensure(ctx, dirs_buf, (size_t)dir_words * 4));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = dflt;
    float best_ms = 1e30f, dflt_ms = 0;
    int qslot = 0;
    for (int sh = 0; sh < num_shapes_all(); ++sh) {
        if (!candidate(sh)) continue;
        float ms = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            GenArgs t = a;
            t.order = sample_buf.as<uint32_t>();
            t.count = want;
            t.dirs = dirs_buf.as<uint32_t>();
            t.dirs_words = dir_words;
            t.queue = queue_buf.as<unsigned int>() + (qslot++ % 64);
            CRISPY_CK(ctx, cudaMemsetAsync(t.queue, 0, 4, s));
            cudaEventRecord(e0, s);
            const int rc = launch_shape(ctx, s, sh, t, false);
            if (rc != CRISPY_OK) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return rc;
            }
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float m = 0;
            cudaEventElapsedTime(&m, e0, e1);
            ms = std::min(ms, m);
        }
        if (sh == dflt) dflt_ms = ms;
        if (ms < best_ms) { best_ms = ms; best = sh; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CRISPY_CK(ctx, cudaGetLastError());
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tuned[key] = TuneEntry{best, best_ms, dflt_ms, want};
    *out = best;
    return CRISPY_OK;
}

}  // namespace

// Launch plan for `count` pairs, computed on the device (no host pass over
// the pairs): PLAIN = the thread-per-pair kernel per 589,824-pair load
// window (as the reference launches per window, genCUDA.cu:156-209);
// STAGED = the warp kernel per window, in the untuned shape the window's
// widest pair needs; BATCHED = pairs sorted by band-slot bin and, inside a
// bin, longest first, one persistent launch per bin on a device work
// counter in the autotuned shape.
int gen_dispatch_impl(crispy_ctx* ctx, cudaStream_t s, const int2* d_pairs, int64_t count,
                      int band, int mode, float* d_dist, int32_t* d_score, int32_t* d_ml,
                      int32_t* d_al) {
    GenJob& g = ctx->gen;
    if (count <= 0) return CRISPY_OK;
    const int64_t nwin = (count + CRISPY_GEN_WINDOW - 1) / CRISPY_GEN_WINDOW;
    const int nstats = kStatWindows + 2 * (int)nwin;
    const bool sorted = mode == CRISPY_MODE_BATCHED;
    CRISPY_TRY(ensure(ctx, g.cstats, (size_t)nstats * 8));
    if (sorted) {
        CRISPY_TRY(ensure(ctx, g.ckeys, (size_t)count * 4));
        CRISPY_TRY(ensure(ctx, g.ckeys_alt, (size_t)count * 4));
        CRISPY_TRY(ensure(ctx, g.cvals, (size_t)count * 4));
        CRISPY_TRY(ensure(ctx, g.cvals_alt, (size_t)count * 4));
    }
    unsigned long long* d_stats = g.cstats.as<unsigned long long>();
    uint32_t* d_order = nullptr;
    auto classify = [&]() -> int {
        CRISPY_CK(ctx, cudaMemsetAsync(d_stats, 0, (size_t)nstats * 8, s));
        gen_classify_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(
            d_pairs, count, g.len.as<int32_t>(), band, kNumBins,
            sorted ? g.ckeys.as<uint32_t>() : nullptr, sorted ? g.cvals.as<uint32_t>() : nullptr, d_stats);
        count_launch(ctx);
        if (sorted) {
            uint32_t* sk = nullptr;
            CRISPY_TRY(sort_u32_payload(ctx, s, g.ckeys.as<uint32_t>(), g.ckeys_alt.as<uint32_t>(),
                                        g.cvals.as<uint32_t>(), g.cvals_alt.as<uint32_t>(), count, 18, &sk,
                                        &d_order, g.scan));
        }
        CRISPY_CK(ctx, cudaGetLastError());
        return CRISPY_OK;
    };
    if (sorted) {
        CRISPY_TRY(ensure(ctx, g.scan, sort_tmp_bytes(count)));
        const std::string key = "gclass," + key_of({(uint64_t)count, (uint64_t)band, (uint64_t)(uintptr_t)d_pairs,
            (uint64_t)(uintptr_t)g.len.ptr, (uint64_t)(uintptr_t)d_stats, (uint64_t)(uintptr_t)g.ckeys.ptr,
            (uint64_t)(uintptr_t)g.ckeys_alt.ptr, (uint64_t)(uintptr_t)g.cvals.ptr,
            (uint64_t)(uintptr_t)g.cvals_alt.ptr, (uint64_t)(uintptr_t)g.scan.ptr});
        CRISPY_TRY(graph_run(ctx, s, key, classify));
        // where the 3-pass (18-bit) sort leaves the payload: the alternate
        // buffer, or the input when there is nothing to sort
        d_order = count > 1 ? g.cvals_alt.as<uint32_t>() : g.cvals.as<uint32_t>();
    } else {
        CRISPY_TRY(classify());
    }
    std::vector<unsigned long long> st(nstats);
    CRISPY_CK(ctx, cudaMemcpyAsync(st.data(), d_stats, (size_t)nstats * 8, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    const int kbmax = (int)st[1];
    ctx->stats.gen_cells += (int64_t)st[0];
    ctx->stats.gen_pairs += count;
    GenArgs base{};
    for (int& o : base.one) o = 1;
    base.packed = g.packed.as<uint32_t>();
    base.woff = g.woff.as<int64_t>();
    base.len = g.len.as<int32_t>();
    base.pairs = d_pairs;
    base.band = band;
    base.dist = d_dist; base.score = d_score; base.ml = d_ml; base.al = d_al;
    base.dir_blocks = gen16_dir_blocks((int)st[kStatMaxSum16]);
    auto launch_wide = [&](const GenArgs& ga, const uint32_t* order, int64_t n_items, cudaStream_t ls,
                           bool timed) -> int {
        const int rs = 2 * kbmax + 3;
        const int threads = 128;
        const int64_t want_threads = std::min<int64_t>(n_items, (int64_t)ctx->sm_count * 4 * threads);
        const int blocks = (int)((want_threads + threads - 1) / threads);
        CRISPY_TRY(ensure(ctx, g.buckets, (size_t)blocks * threads * rs * 6 * sizeof(int)));
        WideArgs w{};
        w.g = ga; w.g.order = order; w.g.count = n_items;
        w.scratch = g.buckets.as<int>(); w.row_stride = rs;
        if (timed) ev_begin(ctx, ctx->ev_gen, ls);
        gen_wide_kernel<<<blocks, threads, 0, ls>>>(w);
        if (timed) ev_end(ctx, ctx->ev_gen, ls);
        count_launch(ctx);
        ctx->stats.gen_launches++;
        return CRISPY_OK;
    };
    if (mode == CRISPY_MODE_PLAIN || mode == CRISPY_MODE_STAGED) {
        // tag storage for the windows the 16-bit kernel takes (one at a time)
        int64_t dir_words = 0;
        for (int64_t w = 0; mode == CRISPY_MODE_STAGED && w < nwin; ++w) {
            const int wb = (int)st[kStatWindows + 2 * w];
            const int sh = wb >= kNumBins ? -1 : default_shape(st[kStatWindows + 2 * w + 1] ? wb + kNumBins : wb);
            if (sh >= 0 && is16(sh))
                dir_words = std::max(dir_words, gen16_dir_words(ctx, sh - kNumShapes,
                                                                std::min<int64_t>(CRISPY_GEN_WINDOW, count - w * CRISPY_GEN_WINDOW),
                                                                base.dir_blocks));
        }
        if (dir_words) {
            CRISPY_TRY(ensure(ctx, g.dirs, (size_t)dir_words * 4));
            base.dirs = g.dirs.as<uint32_t>();
            base.dirs_words = dir_words;
        }
        for (int64_t w = 0; w < nwin; ++w) {
            const int64_t w0 = w * CRISPY_GEN_WINDOW;
            const int64_t n_items = std::min<int64_t>(CRISPY_GEN_WINDOW, count - w0);
            GenArgs a = base;
            a.pairs = d_pairs + w0;
            a.count = n_items;
            a.dist = d_dist + w0;
            a.score = d_score ? d_score + w0 : nullptr;
            a.ml = d_ml ? d_ml + w0 : nullptr;
            a.al = d_al ? d_al + w0 : nullptr;
            const int wb = (int)st[kStatWindows + 2 * w];   // widest band-slot bin (kNumBins = wide)
            const bool lng = st[kStatWindows + 2 * w + 1] != 0;
            if (mode == CRISPY_MODE_PLAIN || wb >= kNumBins) {
                CRISPY_TRY(launch_wide(a, nullptr, n_items, s, true));
            } else {
                CRISPY_TRY(launch_shape(ctx, s, default_shape(lng ? wb + kNumBins : wb), a, true));
                ctx->stats.gen_launches++;
            }
        }
        CRISPY_CK(ctx, cudaGetLastError());
        return CRISPY_OK;
    }
    // BATCHED: bins in ascending width, wide last.  Every bin's shape is
    // picked first (the autotuner times its samples alone on s); then the
    // bins' persistent launches alternate between two side streams, so that
    // a bin's tail (its last, shortest pairs on a few SMs) overlaps the next
    // bin's start.  One event pair on s brackets them all.
    struct BinRun {
        int ob;
        int64_t at, n;
        int shape;
    };
    std::vector<BinRun> runs;
    int64_t at = 0;
    for (int ob = 1; ob <= kWideOrderBin; ++ob) {
        const int64_t n_items = (int64_t)st[kStatBins + ob];
        if (n_items == 0) continue;
        BinRun r{ob, at, n_items, -1};
        at += n_items;
        if (ob != kWideOrderBin) {
            GenArgs a = base;
            a.order = d_order + r.at;
            a.count = n_items;
            CRISPY_TRY(pick_shape(ctx, s, band, ob, a, a.order, n_items, g.tune_sample, g.tune_queue, g.dirs,
                                  &r.shape));
            const int forced = forced_shape();
            if (forced >= 0 && shape_slots(forced) >= kBinSlots[ob < kNumBins ? ob : ob - kNumBins] &&
                !(is16(forced) && ob >= kNumBins))
                r.shape = forced;
        }
        runs.push_back(r);
    }
    CRISPY_TRY(ensure(ctx, g.queue, 64 * 4));
    CRISPY_CK(ctx, cudaMemsetAsync(g.queue.ptr, 0, 64 * 4, s));   // one counter per order-bin (< 64)
    const bool fork = runs.size() > 1;
    // tag storage of the 16-bit launches: one half per side stream
    int64_t dir_words = 0;
    for (const BinRun& r : runs)
        if (r.shape >= 0 && is16(r.shape))
            dir_words = std::max(dir_words, gen16_dir_words(ctx, r.shape - kNumShapes, r.n, base.dir_blocks));
    if (dir_words) CRISPY_TRY(ensure(ctx, g.dirs, (size_t)dir_words * 4 * (fork ? 2 : 1)));
    ev_begin(ctx, ctx->ev_gen, s);
    if (fork) {
        CRISPY_CK(ctx, cudaEventRecord(ctx->fork_ev, s));
        for (int k = 0; k < 2; ++k) CRISPY_CK(ctx, cudaStreamWaitEvent(ctx->side[k], ctx->fork_ev, 0));
    }
    for (size_t i = 0; i < runs.size(); ++i) {
        const BinRun& r = runs[i];
        cudaStream_t ls = fork ? ctx->side[i & 1] : s;
        if (r.ob == kWideOrderBin) {
            CRISPY_TRY(launch_wide(base, d_order + r.at, r.n, ls, false));
            continue;
        }
        GenArgs a = base;
        a.order = d_order + r.at;
        a.count = r.n;
        a.queue = g.queue.as<unsigned int>() + r.ob;
        if (dir_words) {
            a.dirs = g.dirs.as<uint32_t>() + (fork ? (int64_t)(i & 1) * dir_words : 0);
            a.dirs_words = dir_words;
        }
        CRISPY_TRY(launch_shape(ctx, ls, r.shape, a, false));
        ctx->stats.gen_launches++;
    }
    if (fork) {
        for (int k = 0; k < 2; ++k) {
            CRISPY_CK(ctx, cudaEventRecord(ctx->join_ev[k], ctx->side[k]));
            CRISPY_CK(ctx, cudaStreamWaitEvent(s, ctx->join_ev[k], 0));
        }
    }
    ev_end(ctx, ctx->ev_gen, s);
    CRISPY_CK(ctx, cudaGetLastError());
    return CRISPY_OK;
}

}  // namespace crispy

using namespace crispy;

namespace {

int gen_check_pairs(crispy_ctx* ctx, const int32_t* pairs, int64_t npairs) {
    const int n = ctx->gen.n;
    for (int64_t p = 0; p < 2 * npairs; ++p)
        if (pairs[p] < 0 || pairs[p] >= n)
            return fail(ctx, CRISPY_E_INPUT, "pair %lld holds read index %d outside [0, %d)",
                        (long long)(p / 2), pairs[p], n);
    return CRISPY_OK;
}

// Threshold, windows, chunking, stable sort; delivers chunks to the sink.
// d_dist: the pairs' distances (default: the context's distance buffer);
// pair_base is subtracted from the output pairs (a cohort job's base).
int gen_finish(crispy_ctx* ctx, cudaStream_t s, const int2* d_pairs, int64_t npairs, float thr,
               crispy_sink sink, void* user, int64_t* nsurv, bool use_graph, const float* d_dist = nullptr,
               int pair_base = 0) {
    GenJob& g = ctx->gen;
    const float* dist = d_dist ? d_dist : g.dist.as<float>();
    *nsurv = 0;
    if (npairs == 0) return CRISPY_OK;
    CRISPY_TRY(ensure(ctx, g.flags, (size_t)npairs));
    CRISPY_TRY(ensure(ctx, g.surv_idx, (size_t)npairs * 4));
    const int64_t ntiles = (npairs + kScanTile - 1) / kScanTile;
    CRISPY_TRY(ensure(ctx, g.blocksum, (size_t)ntiles * 4));
    gen_flag_kernel<<<(unsigned)((npairs + 255) / 256), 256, 0, s>>>(dist, npairs, thr, g.flags.as<uint8_t>());
    count_launch(ctx);
    // the per-tile survivor counts give the chunk boundaries and the total:
    // one read-back
    CRISPY_TRY(compact_flags(ctx, s, g.flags.as<uint8_t>(), npairs, g.surv_idx.as<uint32_t>(),
                             g.blocksum.as<uint32_t>(), g.scan, nullptr));
    g.h_tiles.resize(ntiles);
    uint32_t* tile_counts = g.h_tiles.data();
    CRISPY_CK(ctx, cudaMemcpyAsync(tile_counts, g.blocksum.ptr, (size_t)ntiles * 4, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    int64_t total = 0;
    for (int64_t t = 0; t < ntiles; ++t) total += tile_counts[t];
    // chunk boundaries: genCUDA.cu:156-254 -- after each load window, flush
    // when the accumulated survivors reach the window size
    const int64_t tiles_per_window = CRISPY_GEN_WINDOW / kScanTile;
    std::vector<std::pair<int64_t, int64_t>> chunks;
    int64_t at = 0, pending = 0;
    for (int64_t t0 = 0; t0 < ntiles; t0 += tiles_per_window) {
        for (int64_t t = t0; t < std::min(ntiles, t0 + tiles_per_window); ++t) pending += tile_counts[t];
        if (pending >= CRISPY_GEN_WINDOW) {
            chunks.push_back({at, pending});
            at += pending;
            pending = 0;
        }
    }
    if (pending > 0) chunks.push_back({at, pending});
    int64_t maxc = 0;
    for (auto& c : chunks) maxc = std::max(maxc, c.second);
    CRISPY_TRY(ensure(ctx, g.keys, (size_t)std::max<int64_t>(maxc, 1) * 4));
    CRISPY_TRY(ensure(ctx, g.keys_alt, (size_t)std::max<int64_t>(maxc, 1) * 4));
    CRISPY_TRY(ensure(ctx, g.vals, (size_t)std::max<int64_t>(maxc, 1) * 4));
    CRISPY_TRY(ensure(ctx, g.vals_alt, (size_t)std::max<int64_t>(maxc, 1) * 4));
    CRISPY_TRY(ensure(ctx, g.out_pairs, (size_t)std::max<int64_t>(maxc, 1) * 8));
    CRISPY_TRY(ensure(ctx, g.out_dists, (size_t)std::max<int64_t>(maxc, 1) * 4));
    CRISPY_TRY(ensure_host(ctx, g.h_pairs, (size_t)std::max<int64_t>(maxc, 1) * 8));
    CRISPY_TRY(ensure_host(ctx, g.h_dists, (size_t)std::max<int64_t>(maxc, 1) * 4));
    for (size_t ci = 0; ci < chunks.size(); ++ci) {
        const int64_t b = chunks[ci].first, c = chunks[ci].second;
        const unsigned blocks = (unsigned)((c + 255) / 256);
        auto chunk_work = [&]() -> int {
            gen_keys_kernel<<<blocks, 256, 0, s>>>(dist, g.surv_idx.as<uint32_t>(), b, c,
                                                  g.keys.as<uint32_t>(), g.vals.as<uint32_t>());
            count_launch(ctx);
            uint32_t *sk = nullptr, *sv = nullptr;
            // distances lie in [0, 1]: sorted on their 32-bit patterns
            CRISPY_TRY(sort_u32_payload(ctx, s, g.keys.as<uint32_t>(), g.keys_alt.as<uint32_t>(),
                                        g.vals.as<uint32_t>(), g.vals_alt.as<uint32_t>(), c, 32, &sk,
                                        &sv, g.scan));
            gen_gather_kernel<<<blocks, 256, 0, s>>>(d_pairs, sk, sv, c, g.out_pairs.as<uint2>(),
                                                    g.out_dists.as<float>(), pair_base);
            count_launch(ctx);
            CRISPY_CK(ctx, cudaGetLastError());
            return CRISPY_OK;
        };
        if (use_graph) {
            CRISPY_TRY(ensure(ctx, g.scan, sort_tmp_bytes(c)));
            const std::string key = "gchunk," + key_of({(uint64_t)b, (uint64_t)c, (uint64_t)(uintptr_t)d_pairs,
                (uint64_t)(uintptr_t)dist, (uint64_t)(uintptr_t)g.surv_idx.ptr, (uint64_t)(uintptr_t)g.keys.ptr,
                (uint64_t)(uintptr_t)g.keys_alt.ptr, (uint64_t)(uintptr_t)g.vals.ptr, (uint64_t)(uintptr_t)g.vals_alt.ptr,
                (uint64_t)(uintptr_t)g.scan.ptr, (uint64_t)(uintptr_t)g.out_pairs.ptr, (uint64_t)(uintptr_t)g.out_dists.ptr});
            CRISPY_TRY(graph_run(ctx, s, key, chunk_work));
        } else {
            CRISPY_TRY(chunk_work());
        }
        if (sink) {
            CRISPY_CK(ctx, cudaMemcpyAsync(g.h_pairs.ptr, g.out_pairs.ptr, (size_t)c * 8, cudaMemcpyDeviceToHost, s));
            CRISPY_CK(ctx, cudaMemcpyAsync(g.h_dists.ptr, g.out_dists.ptr, (size_t)c * 4, cudaMemcpyDeviceToHost, s));
            CRISPY_CK(ctx, cudaStreamSynchronize(s));
            if (sink(user, (int)ci, g.h_pairs.ptr, g.h_dists.as<float>(), c) != 0)
                return fail(ctx, CRISPY_E_IO, "sink aborted at chunk %zu", ci);
        }
    }
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    *nsurv = total;
    return CRISPY_OK;
}

}  // namespace

extern "C" {

int crispy_gen_prepare(crispy_ctx* ctx, const char* seqbuf, const int64_t* offsets,
                       const int32_t* lengths, int n) {
    if (!ctx) return CRISPY_E_INPUT;
    if (!seqbuf || !offsets || !lengths || n <= 0)
        return fail(ctx, CRISPY_E_INPUT, "gen_prepare: empty or NULL read set");
    if (n > CRISPY_MAX_NUM_READS) return fail(ctx, CRISPY_E_UNSUPPORTED, "numReads %d > %d", n, CRISPY_MAX_NUM_READS);
    cudaSetDevice(ctx->device);
    GenJob& g = ctx->gen;
    g.ready = false;
    g.n = n;
    g.h_len.assign(lengths, lengths + n);
    g.h_woff.resize(n + 1);
    int64_t end = 0, words = 0;
    g.max_len = 0;
    for (int r = 0; r < n; ++r) {
        if (lengths[r] > CRISPY_MAX_READ_LEN)
            return fail(ctx, CRISPY_E_UNSUPPORTED, "read %d length %d > %d", r, lengths[r], CRISPY_MAX_READ_LEN);
        if (lengths[r] <= 0 || offsets[r] < 0) return fail(ctx, CRISPY_E_INPUT, "read %d is empty", r);
        g.h_woff[r] = words;
        words += (lengths[r] + 15) / 16;
        end = std::max(end, offsets[r] + lengths[r]);
        g.max_len = std::max(g.max_len, (int)lengths[r]);
    }
    g.h_woff[n] = words;
    cudaStream_t s = ctx->stream;
    CRISPY_TRY(ensure(ctx, g.seq, (size_t)end + 16));
    CRISPY_TRY(ensure(ctx, g.off, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, g.len, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, g.woff, (size_t)(n + 1) * 8));
    CRISPY_TRY(ensure(ctx, g.packed, (size_t)(words + 4) * 4));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.seq.ptr, seqbuf, end, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.off.ptr, offsets, (size_t)n * 8, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.len.ptr, lengths, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.woff.ptr, g.h_woff.data(), (size_t)(n + 1) * 8, cudaMemcpyHostToDevice, s));
    gen_pack_kernel<<<std::min(n, ctx->sm_count * 16), 128, 0, s>>>(
        g.seq.as<uint8_t>(), g.off.as<int64_t>(), g.len.as<int32_t>(), g.woff.as<int64_t>(), n,
        g.packed.as<uint32_t>());
    count_launch(ctx);
    CRISPY_CK(ctx, cudaGetLastError());
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    g.ready = true;
    return CRISPY_OK;
}

int crispy_gen_prepare_from_kmer(crispy_ctx* ctx) {
    if (!ctx) return CRISPY_E_INPUT;
    KmerJob& j = ctx->kmer;
    if (!j.ready) return fail(ctx, CRISPY_E_STATE, "gen_prepare_from_kmer before kmer_prepare");
    cudaSetDevice(ctx->device);
    GenJob& g = ctx->gen;
    g.ready = false;
    const int n = j.n;
    g.n = n;
    g.h_len.resize(n);
    g.h_woff.resize(n + 1);
    int64_t words = 0;
    g.max_len = 0;
    for (int r = 0; r < n; ++r) {
        const int L = j.h_t[r] + j.k - 1;
        if (L <= 0) return fail(ctx, CRISPY_E_INPUT, "read %d is empty", r);
        g.h_len[r] = L;
        g.h_woff[r] = words;
        words += (L + 15) / 16;
        g.max_len = std::max(g.max_len, L);
    }
    g.h_woff[n] = words;
    cudaStream_t s = ctx->stream;
    CRISPY_TRY(ensure(ctx, g.len, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, g.woff, (size_t)(n + 1) * 8));
    CRISPY_TRY(ensure(ctx, g.packed, (size_t)(words + 4) * 4));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.len.ptr, g.h_len.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.woff.ptr, g.h_woff.data(), (size_t)(n + 1) * 8, cudaMemcpyHostToDevice, s));
    gen_pack_kernel<<<std::min(n, ctx->sm_count * 16), 128, 0, s>>>(
        j.seq.as<uint8_t>(), j.off.as<int64_t>(), g.len.as<int32_t>(), g.woff.as<int64_t>(), n,
        g.packed.as<uint32_t>());
    count_launch(ctx);
    CRISPY_CK(ctx, cudaGetLastError());
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    g.ready = true;
    return CRISPY_OK;
}

// The reads the last crispy_preprocess kept, as genDist reads them back
// from the _Clean file: a device-to-device copy of the padded reads, then
// the same packing as gen_prepare.
int crispy_gen_prepare_from_pre(crispy_ctx* ctx, const crispy_raw* raw) {
    if (!ctx) return CRISPY_E_INPUT;
    cudaSetDevice(ctx->device);
    GenJob& g = ctx->gen;
    g.ready = false;
    const uint8_t* d_bytes;
    size_t bytes;
    const int64_t* d_off;
    std::vector<int32_t> len;
    CRISPY_TRY(pre_stage_reads(ctx, raw, 1, &d_bytes, &bytes, &d_off, len));
    const int n = (int)len.size();
    if (n <= 0) return fail(ctx, CRISPY_E_INPUT, "gen_prepare_from_pre: preprocess kept no read");
    if (n > CRISPY_MAX_NUM_READS) return fail(ctx, CRISPY_E_UNSUPPORTED, "numReads %d > %d", n, CRISPY_MAX_NUM_READS);
    g.n = n;
    g.h_len.assign(len.begin(), len.end());
    g.h_woff.resize(n + 1);
    int64_t words = 0;
    g.max_len = 0;
    for (int r = 0; r < n; ++r) {
        if (len[r] > CRISPY_MAX_READ_LEN)
            return fail(ctx, CRISPY_E_UNSUPPORTED, "read %d length %d > %d", r, len[r], CRISPY_MAX_READ_LEN);
        g.h_woff[r] = words;
        words += (len[r] + 15) / 16;
        g.max_len = std::max(g.max_len, len[r]);
    }
    g.h_woff[n] = words;
    cudaStream_t s = ctx->stream;
    CRISPY_TRY(ensure(ctx, g.seq, bytes + 16));
    CRISPY_TRY(ensure(ctx, g.off, (size_t)n * 8));
    CRISPY_TRY(ensure(ctx, g.len, (size_t)n * 4));
    CRISPY_TRY(ensure(ctx, g.woff, (size_t)(n + 1) * 8));
    CRISPY_TRY(ensure(ctx, g.packed, (size_t)(words + 4) * 4));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.seq.ptr, d_bytes, bytes, cudaMemcpyDeviceToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.off.ptr, d_off, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.len.ptr, len.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.woff.ptr, g.h_woff.data(), (size_t)(n + 1) * 8, cudaMemcpyHostToDevice, s));
    gen_pack_kernel<<<std::min(n, ctx->sm_count * 16), 128, 0, s>>>(
        g.seq.as<uint8_t>(), g.off.as<int64_t>(), g.len.as<int32_t>(), g.woff.as<int64_t>(), n,
        g.packed.as<uint32_t>());
    count_launch(ctx);
    CRISPY_CK(ctx, cudaGetLastError());
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    g.ready = true;
    return CRISPY_OK;
}

int crispy_gen_align(crispy_ctx* ctx, const int32_t* pairs, int64_t npairs, int band, int mode,
                     float* dist, int32_t* score, int32_t* ml, int32_t* al) {
    if (!ctx) return CRISPY_E_INPUT;
    GenJob& g = ctx->gen;
    if (!g.ready) return fail(ctx, CRISPY_E_STATE, "gen_align before gen_prepare");
    if (npairs < 0 || (npairs > 0 && !pairs)) return fail(ctx, CRISPY_E_INPUT, "bad pair list");
    if (band <= 0) band = 2;
    CRISPY_TRY(gen_check_pairs(ctx, pairs, npairs));
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    ctx->stats = crispy_stats{};
    ctx->ev_gen.used = 0;
    if (npairs == 0) return CRISPY_OK;
    CRISPY_TRY(ensure(ctx, g.pairs, (size_t)npairs * 8));
    CRISPY_TRY(ensure(ctx, g.dist, (size_t)npairs * 4));
    CRISPY_TRY(ensure(ctx, g.score, (size_t)npairs * 4));
    CRISPY_TRY(ensure(ctx, g.ml, (size_t)npairs * 4));
    CRISPY_TRY(ensure(ctx, g.al, (size_t)npairs * 4));
    CRISPY_CK(ctx, cudaMemcpyAsync(g.pairs.ptr, pairs, (size_t)npairs * 8, cudaMemcpyHostToDevice, s));
    CRISPY_TRY(gen_dispatch_impl(ctx, s, g.pairs.as<int2>(), npairs, band, mode, g.dist.as<float>(),
                                 g.score.as<int32_t>(), g.ml.as<int32_t>(), g.al.as<int32_t>()));
    if (dist) CRISPY_CK(ctx, cudaMemcpyAsync(dist, g.dist.ptr, (size_t)npairs * 4, cudaMemcpyDeviceToHost, s));
    if (score) CRISPY_CK(ctx, cudaMemcpyAsync(score, g.score.ptr, (size_t)npairs * 4, cudaMemcpyDeviceToHost, s));
    if (ml) CRISPY_CK(ctx, cudaMemcpyAsync(ml, g.ml.ptr, (size_t)npairs * 4, cudaMemcpyDeviceToHost, s));
    if (al) CRISPY_CK(ctx, cudaMemcpyAsync(al, g.al.ptr, (size_t)npairs * 4, cudaMemcpyDeviceToHost, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    ctx->stats.gen_kernel_ms = ev_sum_ms(ctx->ev_gen);
    return CRISPY_OK;
}

// Load windows per batch of a windowed run (CRISPY_GEN_BATCH_WINDOWS
// overrides, for tests).
int64_t gen_batch_windows() {
    if (const char* e = std::getenv("CRISPY_GEN_BATCH_WINDOWS")) {
        const long long v = std::atoll(e);
        if (v > 0) return v;
    }
    return 64;
}

// genDist over a host-resident pair list of any length, a batch of load
// windows at a time.  The survivors of each window join a pending chunk on
// the device, which is flushed (stably sorted by distance, sent to the sink)
// once it reaches the window size -- the reference's rule
// (genCUDA.cu:150-254) -- so chunks are those of a one-shot run, and the
// device holds one batch plus at most two windows of survivors.
int gen_run_windowed(crispy_ctx* ctx, cudaStream_t s, const int2* host_pairs, int64_t npairs, int band,
                     int mode, float thr, crispy_sink sink, void* user, int64_t* nsurv) {
    GenJob& g = ctx->gen;
    const int64_t W = CRISPY_GEN_WINDOW;
    const int64_t batch = gen_batch_windows() * W;
    const int64_t bmax = std::min(batch, npairs);
    CRISPY_TRY(ensure(ctx, g.pairs, (size_t)bmax * 8));
    CRISPY_TRY(ensure(ctx, g.dist, (size_t)bmax * 4));
    CRISPY_TRY(ensure(ctx, g.flags, (size_t)bmax));
    CRISPY_TRY(ensure(ctx, g.surv_idx, (size_t)bmax * 4));
    const int64_t ntiles_max = (bmax + kScanTile - 1) / kScanTile;
    CRISPY_TRY(ensure(ctx, g.blocksum, (size_t)ntiles_max * 4));
    CRISPY_TRY(ensure(ctx, g.acc_pairs, (size_t)2 * W * 8));
    CRISPY_TRY(ensure(ctx, g.acc_dists, (size_t)2 * W * 4));
    CRISPY_TRY(ensure(ctx, g.keys, (size_t)2 * W * 4));
    CRISPY_TRY(ensure(ctx, g.keys_alt, (size_t)2 * W * 4));
    CRISPY_TRY(ensure(ctx, g.vals, (size_t)2 * W * 4));
    CRISPY_TRY(ensure(ctx, g.vals_alt, (size_t)2 * W * 4));
    CRISPY_TRY(ensure(ctx, g.out_pairs, (size_t)2 * W * 8));
    CRISPY_TRY(ensure(ctx, g.out_dists, (size_t)2 * W * 4));
    CRISPY_TRY(ensure_host(ctx, g.h_pairs, (size_t)2 * W * 8));
    CRISPY_TRY(ensure_host(ctx, g.h_dists, (size_t)2 * W * 4));
    int64_t pending = 0, total = 0;
    int chunk = 0;
    auto flush = [&]() -> int {
        const int64_t c = pending;
        const unsigned blocks = (unsigned)((c + 255) / 256);
        gen_poskeys_kernel<<<blocks, 256, 0, s>>>(g.acc_dists.as<float>(), c, g.keys.as<uint32_t>(),
                                                 g.vals.as<uint32_t>());
        count_launch(ctx);
        uint32_t *sk = nullptr, *sv = nullptr;
        CRISPY_TRY(ensure(ctx, g.scan, sort_tmp_bytes(c)));
        CRISPY_TRY(sort_u32_payload(ctx, s, g.keys.as<uint32_t>(), g.keys_alt.as<uint32_t>(), g.vals.as<uint32_t>(),
                                    g.vals_alt.as<uint32_t>(), c, 32, &sk, &sv, g.scan));
        gen_gather_kernel<<<blocks, 256, 0, s>>>(g.acc_pairs.as<int2>(), sk, sv, c, g.out_pairs.as<uint2>(),
                                                g.out_dists.as<float>());
        count_launch(ctx);
        CRISPY_CK(ctx, cudaGetLastError());
        if (sink) {
            CRISPY_CK(ctx, cudaMemcpyAsync(g.h_pairs.ptr, g.out_pairs.ptr, (size_t)c * 8, cudaMemcpyDeviceToHost, s));
            CRISPY_CK(ctx, cudaMemcpyAsync(g.h_dists.ptr, g.out_dists.ptr, (size_t)c * 4, cudaMemcpyDeviceToHost, s));
            CRISPY_CK(ctx, cudaStreamSynchronize(s));
            if (sink(user, chunk, g.h_pairs.ptr, g.h_dists.as<float>(), c) != 0)
                return fail(ctx, CRISPY_E_IO, "sink aborted at chunk %d", chunk);
        }
        ++chunk;
        pending = 0;
        return CRISPY_OK;
    };
    for (int64_t b0 = 0; b0 < npairs; b0 += batch) {
        const int64_t nb = std::min(batch, npairs - b0);
        CRISPY_CK(ctx, cudaMemcpyAsync(g.pairs.ptr, host_pairs + b0, (size_t)nb * 8, cudaMemcpyHostToDevice, s));
        CRISPY_TRY(gen_dispatch_impl(ctx, s, g.pairs.as<int2>(), nb, band, mode, g.dist.as<float>(), nullptr,
                                     nullptr, nullptr));
        gen_flag_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(g.dist.as<float>(), nb, thr,
                                                                    g.flags.as<uint8_t>());
        count_launch(ctx);
        int64_t nsb = 0;
        CRISPY_TRY(compact_flags(ctx, s, g.flags.as<uint8_t>(), nb, g.surv_idx.as<uint32_t>(),
                                 g.blocksum.as<uint32_t>(), g.scan, &nsb));
        const int64_t ntiles = (nb + kScanTile - 1) / kScanTile;
        std::vector<uint32_t> tile_counts(ntiles);
        CRISPY_CK(ctx, cudaMemcpyAsync(tile_counts.data(), g.blocksum.ptr, (size_t)ntiles * 4,
                                       cudaMemcpyDeviceToHost, s));
        CRISPY_CK(ctx, cudaStreamSynchronize(s));
        const int64_t tiles_per_window = W / kScanTile;
        int64_t base = 0;
        for (int64_t t0 = 0; t0 < ntiles; t0 += tiles_per_window) {
            int64_t cw = 0;
            for (int64_t t = t0; t < std::min(ntiles, t0 + tiles_per_window); ++t) cw += tile_counts[t];
            if (cw > 0) {
                gen_append_kernel<<<(unsigned)((cw + 255) / 256), 256, 0, s>>>(
                    g.pairs.as<int2>(), g.dist.as<float>(), g.surv_idx.as<uint32_t>(), base, cw,
                    g.acc_pairs.as<int2>() + pending, g.acc_dists.as<float>() + pending);
                count_launch(ctx);
                pending += cw;
                base += cw;
                total += cw;
            }
            if (pending >= W) CRISPY_TRY(flush());
        }
    }
    if (pending > 0) CRISPY_TRY(flush());
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    *nsurv = total;
    return CRISPY_OK;
}

int crispy_gen_run(crispy_ctx* ctx, const int32_t* pairs, int64_t npairs, int band, float thr,
                   int mode, crispy_sink sink, void* user, int64_t* nsurvivors) {
    if (!ctx) return CRISPY_E_INPUT;
    GenJob& g = ctx->gen;
    if (!g.ready) return fail(ctx, CRISPY_E_STATE, "gen_run before gen_prepare");
    if (npairs < 0 || (npairs > 0 && !pairs)) return fail(ctx, CRISPY_E_INPUT, "bad pair list");
    if (band <= 0) band = 2;   // genMain.cpp:356-364
    CRISPY_TRY(gen_check_pairs(ctx, pairs, npairs));
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    ctx->stats = crispy_stats{};
    ctx->ev_gen.used = 0;
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_begin, s));
    int64_t ns = 0;
    if (npairs > gen_batch_windows() * CRISPY_GEN_WINDOW) {
        // longer than one batch of load windows: bounded device memory
        CRISPY_TRY(gen_run_windowed(ctx, s, reinterpret_cast<const int2*>(pairs), npairs, band, mode, thr, sink,
                                    user, &ns));
    } else if (npairs > 0) {
        CRISPY_TRY(ensure(ctx, g.pairs, (size_t)npairs * 8));
        CRISPY_TRY(ensure(ctx, g.dist, (size_t)npairs * 4));
        CRISPY_CK(ctx, cudaMemcpyAsync(g.pairs.ptr, pairs, (size_t)npairs * 8, cudaMemcpyHostToDevice, s));
        CRISPY_TRY(gen_dispatch_impl(ctx, s, g.pairs.as<int2>(), npairs, band, mode, g.dist.as<float>(),
                                     nullptr, nullptr, nullptr));
        CRISPY_TRY(gen_finish(ctx, s, g.pairs.as<int2>(), npairs, thr, sink, user, &ns,
                              mode == CRISPY_MODE_BATCHED));
    }
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_end, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    float tot = 0;
    cudaEventElapsedTime(&tot, ctx->t_begin, ctx->t_end);
    ctx->stats.total_ms = tot;
    ctx->stats.gen_kernel_ms = ev_sum_ms(ctx->ev_gen);
    ctx->stats.gen_survivors = ns;
    if (nsurvivors) *nsurvivors = ns;
    return CRISPY_OK;
}

int crispy_tune_report(char* buf, size_t len) {
    if (!buf || len == 0) return CRISPY_E_INPUT;
    std::string out = "[";
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        bool first = true;
        for (auto& kv : g_tuned) {
            char item[320];
            const int shp = kv.second.shape;
            int lanes, slots_lane, per_block;
            if (is16(shp)) {
                const Shape16 h = gen16_shape(shp - kNumShapes);
                lanes = h.g; slots_lane = 2 * h.r; per_block = gen16_pairs_per_block(shp - kNumShapes);
            } else {
                lanes = kShapes[shp].g; slots_lane = kShapes[shp].c; per_block = kGenWarps * (32 / lanes);
            }
            const int b = kv.first.bin;
            snprintf(item, sizeof item,
                     "%s{\"stage\": \"gen\", \"band\": %d, \"band_slots\": %d, \"len_bucket\": %d, "
                     "\"sms\": %d, \"kernel\": \"%s\", \"lanes_per_pair\": %d, \"slots_per_lane\": %d, "
                     "\"pairs_per_block\": %d, \"sample\": %lld, \"ms\": %.4f, \"default_ms\": %.4f}",
                     first ? "" : ", ", kv.first.band, kBinSlots[b < kNumBins ? b : b - kNumBins],
                     b < kNumBins ? 0 : 1, kv.first.sms, is16(shp) ? "gen16_kernel" : "gen_warp_kernel", lanes,
                     slots_lane, per_block, (long long)kv.second.sample, kv.second.ms_best, kv.second.ms_default);
            out += item;
            first = false;
        }
    }
    std::string km = kmer_tune_json();
    if (!km.empty()) out += out.size() > 1 ? km : km.substr(2);
    out += "]";
    std::strncpy(buf, out.c_str(), len - 1);
    buf[len - 1] = 0;
    return out.size() < len ? CRISPY_OK : CRISPY_E_INPUT;
}

int crispy_gen_run_from_kmer(crispy_ctx* ctx, int band, float thr, int mode, crispy_sink sink,
                             void* user, int64_t* nsurvivors) {
    if (!ctx) return CRISPY_E_INPUT;
    GenJob& g = ctx->gen;
    KmerJob& k = ctx->kmer;
    if (!g.ready || !k.ready) return fail(ctx, CRISPY_E_STATE, "gen_run_from_kmer needs kmer_run and gen_prepare");
    if (g.n != k.n) return fail(ctx, CRISPY_E_STATE, "kmer and gen read sets differ (%d vs %d reads)", k.n, g.n);
    if (band <= 0) band = 2;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    const int64_t npairs = k.nsurv;
    const crispy_stats kst = ctx->stats;
    ctx->stats = crispy_stats{};
    ctx->ev_gen.used = 0;
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_begin, s));
    int64_t ns = 0;
    if (k.spilled) {
        // the k-mer survivors sit in pinned host memory: windowed run
        CRISPY_TRY(gen_run_windowed(ctx, s, k.h_spill_pairs.as<int2>(), npairs, band, mode, thr, sink, user,
                                    &ns));
    } else if (npairs > 0) {
        CRISPY_TRY(ensure(ctx, g.dist, (size_t)npairs * 4));
        CRISPY_TRY(gen_dispatch_impl(ctx, s, k.pairs.as<int2>(), npairs, band, mode, g.dist.as<float>(),
                                     nullptr, nullptr, nullptr));
        CRISPY_TRY(gen_finish(ctx, s, k.pairs.as<int2>(), npairs, thr, sink, user, &ns,
                              mode == CRISPY_MODE_BATCHED));
    }
    CRISPY_CK(ctx, cudaEventRecord(ctx->t_end, s));
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    float tot = 0;
    cudaEventElapsedTime(&tot, ctx->t_begin, ctx->t_end);
    ctx->stats.total_ms = tot;
    ctx->stats.gen_kernel_ms = ev_sum_ms(ctx->ev_gen);
    ctx->stats.gen_survivors = ns;
    ctx->stats.kmer_kernel_ms = kst.kmer_kernel_ms;
    ctx->stats.kmer_pairs = kst.kmer_pairs;
    ctx->stats.kmer_survivors = kst.kmer_survivors;
    if (nsurvivors) *nsurvivors = ns;
    return CRISPY_OK;
}

}  // extern "C"

namespace crispy {

// genDist over a cohort after kmer_run_cohort (server cross-job batching):
// every job's survivors go through one classification and one set of
// persistent bin launches (the jobs share every launch); then each job's
// slice is thresholded, chunked and sorted on its own, with its own
// threshold, and its chunks (in its own read indices) go to its sink.
int gen_run_cohort(crispy_ctx* ctx, const std::vector<CohortJob>& jobs, const std::vector<int64_t>& counts,
                   int band, std::vector<int64_t>& gen_counts) {
    GenJob& g = ctx->gen;
    KmerJob& k = ctx->kmer;
    if (!g.ready || !k.ready) return fail(ctx, CRISPY_E_STATE, "gen cohort needs kmer_run_cohort and gen_prepare");
    if (counts.size() != jobs.size()) return fail(ctx, CRISPY_E_STATE, "gen cohort: %zu counts for %zu jobs",
                                                  counts.size(), jobs.size());
    int64_t total = 0;
    for (int64_t c : counts) total += c;
    if (total != k.nsurv || k.spilled) return fail(ctx, CRISPY_E_STATE, "gen cohort: survivor counts do not match");
    if (band <= 0) band = 2;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    ctx->stats = crispy_stats{};
    ctx->ev_gen.used = 0;
    gen_counts.assign(jobs.size(), 0);
    if (total > 0) {
        CRISPY_TRY(ensure(ctx, g.dist, (size_t)total * 4));
        CRISPY_TRY(gen_dispatch_impl(ctx, s, k.pairs.as<int2>(), total, band, CRISPY_MODE_BATCHED,
                                     g.dist.as<float>(), nullptr, nullptr, nullptr));
    }
    int64_t off = 0;
    for (size_t c = 0; c < jobs.size(); ++c) {
        int64_t ns = 0;
        if (counts[c] > 0)
            CRISPY_TRY(gen_finish(ctx, s, k.pairs.as<int2>() + off, counts[c], jobs[c].thr, jobs[c].sink,
                                  jobs[c].user, &ns, false, g.dist.as<float>() + off, jobs[c].base));
        gen_counts[c] = ns;
        off += counts[c];
    }
    CRISPY_CK(ctx, cudaStreamSynchronize(s));
    ctx->stats.gen_kernel_ms = ev_sum_ms(ctx->ev_gen);
    return CRISPY_OK;
}

}  // namespace crispy
