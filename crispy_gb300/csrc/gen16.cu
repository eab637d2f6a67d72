// gen16.cu -- genDist's banded Needleman-Wunsch with two cells per 32-bit
// register: the DP the batched and staged runs take for every pair with
// L1 + L2 <= kGen16MaxSum (3600) that fits a register band.
//
// Reference semantics are those of gen.cu (genCPU.cpp:290-466 restated by
// genKernel.cu:372-780): rows i over read2 = pair[1], columns j over read1 =
// pair[0], band |i - j| <= kBand = (L1 + L2) / (2 * band), boundary cells
// M = 0, up / left candidates penalised by the neighbour's own choice
// (GO = -10 after a diagonal, GE = -1 after the same gap, 0 after the other
// gap; genMain.h:32-35), ties diag > up > left, the last maximum of the last
// row and of the last column, (float)ML / (float)AL.
//
// Keys.  A cell on anti-diagonal s = i + j holds K = 4*M + t + 4*s + kBase,
// t its choice's tag: 3 diagonal, 1 up, 0 left.  A cell's three candidates
// carry distinct tags, so one unsigned three-way maximum of their keys gives
// the maximum and the reference's tie order at once: one __vimax3_u16x2 per
// two cells.  The winner's tag t and x2 = t & 2 give the two gap candidates
// it sends to the next anti-diagonal, already keyed, by multiply-adds:
//   up:    K + 5 - 5 t - 14 x2   = 4 (M + pen_up)   + 1 + 4 (s+1) + kBase
//   left:  K + 3 t - 24 x2       = 4 (M + pen_left) + 0 + 4 (s+1) + kBase
// (pen_up = -10 / -1 / 0 and pen_left = -10 / 0 / -1 after a diagonal / up /
// left choice), and the diagonal candidate two steps later is
// (K | 3) + 28 - 36 * mismatch; the cell stores its base K - t + 31 =
// (K | 3) + 28 in place of K (one three-input add).  Every cell the recurrence reaches has
// -4 min(i,j) <= M <= 5 min(i,j) (the diagonal candidate has no state and a
// gap never gains), so 4M + 4s lies in [-4s, 14s]: with kBase = 4 * 3632 +
// 128 every key of a pair with L1 + L2 <= 3600 -- and of the up to 32 steps
// a sweep runs past a pair's end -- lies in [128, 65507].  Cells outside the
// band, before the matrix or of a finished pair hold the key 8, below every
// candidate of an in-band cell.  No 16-bit half ever wraps, so plain 32-bit
// adds and multiply-adds act on both halves at once.
//
// ML and AL by a path walk.  Every cell's tag t (its choice) goes into a
// per-register word per parity, 2 bits per cell, stored every 16 steps to
// the pair's region of `dirs`.  After the sweep the pair's lanes walk the path
// back from the chosen last-row / last-column cell E to the boundary cell
// (i0, j0) it leaves, following the tags (the reference's tie-broken
// choices), and count A = diagonal moves and the gap penalties Gp (each gap
// move's penalty from the tag of the cell it leaves; a boundary cell's tag
// gives 0).  The score identity M(E) = 5 (A - mism) - 4 mism + Gp gives the
// mismatches, and AL = (iE + jE) - A, ML = (iE + jE) - 2A + mism - (i0 + j0)
// (genCPU.cpp:426-440: a diagonal adds 1 - hit to ML, a gap 1; AL counts
// every move from the boundary cell's own AL = i0 + j0).
//
// Layout.  G lanes per pair, R registers per lane: register r of lane l
// holds slot l*R + r in its low half and slot G*R + l*R + r in its high
// half.  Slot q hosts diagonal 2q - kBand + P at step parity P; its up /
// left neighbours are slots q + 1 / q - 1 of the previous step, i.e.
// registers r + 1 / r - 1 of the same lane, so only the lane's edge
// register crosses lanes (one shuffle of keys per step).
// Tags: step tau = s + (kBand & 1) (odd bands run one step late) lies in
// block b = tau / 16 at parity P = tau % 2; register r of lane l keeps the
// block's tags of parity P in word ((2b + P) * G + l) * R + r of the pair's
// region, the step's tag at bits 2 (7 - (tau % 16) / 2) of the half, so a
// diagonal (same slot, same parity) runs through consecutive fields.
// Symbols: two bit planes per read in shared memory, 32 symbols per word,
// behind a zero pad; every 32 steps a lane cuts its slots' 17-symbol
// windows out of four 32-symbol windows (consecutive slots of a lane read
// windows one symbol apart) and folds them into 16 one-bit mismatch flags
// per slot and parity.
// Border: a slot hosts one diagonal d per parity, so it enters the matrix
// once, at s = |d|, as a boundary cell (row 0 or column 0).  Every slot's cap
// starts closed (key 8); the two boundary cells of a step (d = s and d = -s)
// get their boundary values and open their slot's cap.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>

#include "gen_args.h"
#include "internal.h"

namespace crispy {
namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
// Blocks per SM for the register budget, counted in warps per SM
// sub-partition (16K registers each): 3 warps give a lane up to 168
// registers, 4 up to 128.
template <int R>
constexpr int min_blocks16() { return R <= 3 ? 6 : (R == 4 ? 5 : 3); }
// A read in shared memory: two bit planes (bit 0 and bit 1 of each symbol's
// code), 32 symbols per word, each behind kPlanePad zero words (positions
// down to -192) and before 2 zero tail words.
constexpr int kPlanePad = 6;
constexpr int kPlaneWords = kPlanePad + 64 + 2;
constexpr int kSmWords = 2 * kPlaneWords;
constexpr int kPairWords = 2 * kSmWords + 4;    // both reads of a pair, 4 words apart in banks
static_assert(kPairWords % 32 == 4 && kSmWords % 4 == 0, "shared layout");
constexpr int kSteps = 16;           // steps per block: 8 cells per slot and parity
constexpr int kSetupSteps = 32;      // steps per window set-up: 16 cells per slot and parity
constexpr int kSlack = 32;           // steps a sweep may run past a pair's end
constexpr int kBase = 4 * (kGen16MaxSum + kSlack) + 128;
constexpr uint32_t kLo = 0x00010001u;   // 1 in each half
constexpr uint32_t kOut = 8u;           // key of a cell outside the band / matrix
constexpr uint32_t kOut2 = kOut * kLo;
constexpr int kRefNegInf = -1000000;    // genCPU.cpp:350 initial last-row/column maximum
static_assert(18 * (kGen16MaxSum + kSlack) + 131 < 65536, "16-bit keys would wrap");
static_assert(kBase % 4 == 0, "the score is read back as (K - 4s - kBase) / 4");

constexpr int kClean = 0, kTrack = 1, kStart = 2;

__device__ __forceinline__ int kband16(int l1, int l2, int band) {
    return band >= 2 ? (l1 + l2) / (2 * band) : max(l1, l2);
}

// Runtime multipliers (all derived from GenArgs::one, whose values the
// compiler cannot see): products by them stay multiply-adds on the FMA pipe
// instead of turning into shift / add sequences on the ALU.
struct Mul {
    uint32_t one, four, n36, n5, n14, m3, n24, c5;
};

__device__ __forceinline__ Mul make_mul(const int* o) {
    Mul m;
    m.one = (uint32_t)o[0];
    m.four = 4u * (uint32_t)o[1];
    m.n36 = (uint32_t)(-36) * (uint32_t)o[2];
    m.n5 = (uint32_t)(-5) * (uint32_t)o[3];
    m.n14 = (uint32_t)(-14) * (uint32_t)o[4];
    m.m3 = 3u * (uint32_t)o[5];
    m.n24 = (uint32_t)(-24) * (uint32_t)o[0];
    m.c5 = 5u * kLo * (uint32_t)o[1];
    return m;
}

template <int R>
struct St {
    uint32_t K[2][R];    // diagonal bases (K | 3) + 28 by step parity, for two steps on
    uint32_t U[R], F[R]; // up / left candidates the last step sent
    uint32_t D[2][R];    // tags of the block by parity, 2 bits per cell, first step highest
    uint32_t MW[2][R];   // mismatch flags of the block by parity, 2 bits per step
    uint32_t CP[2][R];   // per half: 0xFFFF in band, kOut outside
};

struct Pair16 {
    int kb, l1, l2, shift;   // shift = kb & 1: odd bands run one step late
    // steps at which this lane may hold a last-row / last-column cell: four
    // windows of 2R steps (last row, then last column; low and high slots)
    int tw[4];
};

struct Best16 {
    int m;
    int at;
};

// 32 symbols starting at read position pos as their two bit planes (first
// symbol in bit 0; before the read and past it: zeros).
__device__ __forceinline__ void window32(const uint32_t* sm, int pos, uint32_t& p0, uint32_t& p1) {
    const int w = min(max(pos >> 5, -kPlanePad), 64) + kPlanePad;
    const int sh = pos & 31;
    p0 = __funnelshift_r(sm[w], sm[w + 1], sh);
    p1 = __funnelshift_r(sm[kPlaneWords + w], sm[kPlaneWords + w + 1], sh);
}

// Mismatch flags of 32 steps.  Parity-0 cells k = 0..15 of slot q compare
// read1[j0 - 1 + k] with read2[i0 - 1 + k], parity-1 cells read1[j0 - 1 + k]
// with read2[i0 + k], (i0, j0) = ((s0 + d0) / 2, (s0 - d0) / 2) the slot's
// parity-0 cell at the set-up, d0 = 2q - kb.  The lane's R slots of a half
// are consecutive, q = qb + r: read1 windows start at J - r, read2 windows
// at I + r, all inside one 32-symbol window per read.  A flag sits at bit k
// of its half (a mismatch: either plane differs).  A finished pair's caps
// close.
template <int G, int R>
__device__ __forceinline__ void block_setup(St<R>& st, const uint32_t* sm1, const uint32_t* sm2, int gl,
                                            int s0, const Pair16& pc, bool finished) {
    uint32_t f0[2][R], f1[2][R];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int qb = (h * G + gl) * R;
        const int d0 = 2 * qb - pc.kb;
        const int I = ((s0 + d0) >> 1) - 1, J = ((s0 - d0) >> 1) - 1;   // s0 + d0 is even
        uint32_t a0, a1, b0, b1;
        window32(sm1, J - (R - 1), a0, a1);   // read1 from J - (R-1): slot r at offset R-1-r
        window32(sm2, I, b0, b1);             // read2 from I: slot r at offset r
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t u0 = a0 >> (R - 1 - r), u1 = a1 >> (R - 1 - r);
            f0[h][r] = (u0 ^ (b0 >> r)) | (u1 ^ (b1 >> r));
            f1[h][r] = (u0 ^ (b0 >> (r + 1))) | (u1 ^ (b1 >> (r + 1)));   // read2 one symbol on
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        st.MW[0][r] = __byte_perm(f0[0][r], f0[1][r], 0x5410);
        st.MW[1][r] = __byte_perm(f1[0][r], f1[1][r], 0x5410);
        if (finished) { st.CP[0][r] = kOut2; st.CP[1][r] = kOut2; }
    }
}

// Even bits of x to its low half, odd bits to its high half, in order.
__device__ __forceinline__ uint32_t unzip_bits(uint32_t x) {
    uint32_t t;
    t = (x ^ (x >> 1)) & 0x22222222u; x ^= t ^ (t << 1);
    t = (x ^ (x >> 2)) & 0x0C0C0C0Cu; x ^= t ^ (t << 2);
    t = (x ^ (x >> 4)) & 0x00F000F0u; x ^= t ^ (t << 4);
    t = (x ^ (x >> 8)) & 0x0000FF00u; x ^= t ^ (t << 8);
    return x;
}

// Plane word k of a read (symbols 32 (k - kPlanePad) ..) from its packed
// words (16 symbols each, first symbol in the top bits): the bit reversal
// puts symbol q's code bits at 2q + 1 (bit 0) and 2q (bit 1).
__device__ __forceinline__ void plane_word(const uint32_t* g, int nw, int k, uint32_t& p0, uint32_t& p1) {
    const int w = 2 * (k - kPlanePad);
    const uint32_t x0 = w >= 0 && w < nw ? unzip_bits(__brev(g[w])) : 0u;
    const uint32_t x1 = w + 1 >= 0 && w + 1 < nw ? unzip_bits(__brev(g[w + 1])) : 0u;
    p0 = __byte_perm(x0, x1, 0x7632);   // code bit 0 of symbols 0..31
    p1 = __byte_perm(x0, x1, 0x5410);   // code bit 1
}

// Boundary events of a step: slot q = (d + kb - P) / 2 for d = s (column
// 0, j = 0, tag left) and d = -s (row 0, i = 0, tag up), when it lies in
// the band and in this lane: register *r (-1: none) and half *h.
template <int G, int R, int P>
__device__ __forceinline__ void boundary_slot(int d, const Pair16& pc, int gl, int* r, int* h) {
    *r = -1;
    *h = 0;
    if (pc.l1 <= 0 || d < -pc.kb || d > pc.kb) return;   // no pair, or outside the band
    const int q = (d + pc.kb - P) >> 1;
    const int rl = q - gl * R, rh = q - (G + gl) * R;
    if ((unsigned)rl < (unsigned)R) { *r = rl; *h = 0; }
    else if ((unsigned)rh < (unsigned)R) { *r = rh; *h = 1; }
}

// Sets one half to a boundary cell at step s (M = 0) and opens its cap.
__device__ __forceinline__ void boundary_set(uint32_t& K, uint32_t& CP, int h, int s, uint32_t tag) {
    const uint32_t key = tag + (uint32_t)(4 * s + kBase);
    if (h == 0) {
        K = (K & 0xFFFF0000u) | key;
        CP |= 0x0000FFFFu;
    } else {
        K = (K & 0x0000FFFFu) | (key << 16);
        CP |= 0xFFFF0000u;
    }
}

// The key of slot q (held by this lane) at the current parity.
template <int G, int R, int P>
__device__ __forceinline__ uint32_t take(const St<R>& st, int q, int gl) {
    const int rl = q - gl * R;
    const bool hi = (unsigned)rl >= (unsigned)R;
    const int rr = hi ? q - (G + gl) * R : rl;
    uint32_t kk = 0;
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (r == rr) kk = st.K[P][r];
    if (hi) kk >>= 16;
    return kk & 0xFFFFu;
}

__device__ __forceinline__ bool mine(int q, int gl, int G, int R) {
    return (unsigned)(q - gl * R) < (unsigned)R || (unsigned)(q - (G + gl) * R) < (unsigned)R;
}

// Last row (i = l2, tracked as `col`, ordered by j) and last column (j = l1,
// `row`, ordered by i): each holds at most one cell per step; the lane that
// holds it keeps the last maximum (>=), genCPU.cpp:442-464.
template <int G, int R, int P>
__device__ __forceinline__ void track16(const St<R>& st, int gl, int s, const Pair16& pc, Best16& col,
                                        Best16& row) {
    const int dr = 2 * pc.l2 - s, jr = s - pc.l2;
    const int qr = (dr + pc.kb - P) >> 1;
    const int dc = s - 2 * pc.l1, ic = s - pc.l1;
    const int qc = (dc + pc.kb - P) >> 1;
    const bool hr = jr >= 1 && jr <= pc.l1 && dr >= -pc.kb && dr <= pc.kb && mine(qr, gl, G, R);
    const bool hc = ic >= 1 && ic <= pc.l2 && dc >= -pc.kb && dc <= pc.kb && mine(qc, gl, G, R);
    if (hr) {
        const uint32_t key = take<G, R, P>(st, qr, gl);
        const int m = ((int)key - 31 - 4 * s - kBase) >> 2;
        if (m >= col.m) { col.m = m; col.at = jr; }
    }
    if (hc) {
        const uint32_t key = take<G, R, P>(st, qc, gl);
        const int m = ((int)key - 31 - 4 * s - kBase) >> 2;
        if (m >= row.m) { row.m = m; row.at = ic; }
    }
}

// One anti-diagonal step at parity P for the lane's 2R cells.  sel0 / sel1
// are the lane's byte selectors for the edge register's neighbour: identity,
// or (lane 0 at parity 0) its low half moved up over an empty slot, or (the
// last lane at parity 1) its high half moved down under an empty slot.
template <int G, int R, int P, int kMode>
__device__ __forceinline__ void step16(St<R>& st, int gl, int s, const Pair16& pc, const Mul& mu,
                                       uint32_t sel0, uint32_t sel1, Best16& col, Best16& row) {
    uint32_t nK;
    if (P == 0) {
        // left of register 0 = register R-1 of the previous lane
        const int src = (gl + G - 1) & (G - 1);
        nK = __byte_perm(__shfl_sync(0xffffffffu, st.F[R - 1], src, G), kOut2, sel0);
    } else {
        // up of register R-1 = register 0 of the next lane
        const int src = (gl + 1) & (G - 1);
        nK = __byte_perm(__shfl_sync(0xffffffffu, st.U[0], src, G), kOut2, sel1);
    }
    int ra = -1, ha = 0, rb = -1, hb = 0;
    if (kMode == kStart && s >= 0) {
        boundary_slot<G, R, P>(s, pc, gl, &ra, &ha);            // column 0
        if (s > 0) boundary_slot<G, R, P>(-s, pc, gl, &rb, &hb);   // row 0
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        // parity 0 reads register r-1 (runs downwards), parity 1 register
        // r+1 (runs upwards), so a neighbour is read before it is rewritten
        const int r = P == 0 ? R - 1 - k : k;
        uint32_t upK, lfK;
        if (P == 0) {
            upK = st.U[r];
            lfK = r > 0 ? st.F[r - 1] : nK;
        } else {
            lfK = st.F[r];
            upK = r < R - 1 ? st.U[r + 1] : nK;
        }
        const uint32_t mm = st.MW[P][r] & kLo;
        st.MW[P][r] >>= 1;
        const uint32_t kd = mm * mu.n36 + st.K[P][r];
        uint32_t K = __vimax3_u16x2(kd, upK, lfK);
        K = __vminu2(K, st.CP[P][r]);
        if (kMode == kStart && (r == ra || r == rb)) {
            // a boundary cell: its own key, not the recurrence's
            if (r == ra) boundary_set(K, st.CP[P][r], ha, s, 0u);
            if (r == rb) boundary_set(K, st.CP[P][r], hb, s, 1u);
        }
        const uint32_t t = K & (3u * kLo), x2 = K & (2u * kLo);
        st.U[r] = x2 * mu.n14 + (t * mu.n5 + (K * mu.one + mu.c5));
        st.F[r] = x2 * mu.n24 + (t * mu.m3 + K);
        st.D[P][r] = st.D[P][r] * mu.four + t;
        st.K[P][r] = K - t + 31u * kLo;
    }
    if (kMode != kClean) {
        const bool near = (unsigned)(s - pc.tw[0]) < 2u * R || (unsigned)(s - pc.tw[1]) < 2u * R ||
                          (unsigned)(s - pc.tw[2]) < 2u * R || (unsigned)(s - pc.tw[3]) < 2u * R;
        if (near) track16<G, R, P>(st, gl, s, pc, col, row);
    }
}

// A block of 16 steps, after which the lane's tag words go to `dst`
// (parity P at dst + P * G * R; nullptr: not stored).
template <int G, int R, int kMode>
__device__ __forceinline__ void block16(St<R>& st, int gl, int s0, const Pair16& pc, const Mul& mu,
                                        uint32_t sel0, uint32_t sel1, Best16& col, Best16& row,
                                        uint32_t* dst) {
#pragma unroll 1
    for (int t = 0; t < kSteps; t += 2) {
        step16<G, R, 0, kMode>(st, gl, s0 + t, pc, mu, sel0, sel1, col, row);
        step16<G, R, 1, kMode>(st, gl, s0 + t + 1, pc, mu, sel0, sel1, col, row);
    }
    if (dst) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            dst[r] = st.D[0][r];
            dst[G * R + r] = st.D[1][r];
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        st.D[0][r] = 0;
        st.D[1][r] = 0;
    }
}

// Largest m over a G-lane sub-group, ties to the largest index `at`.
template <int G>
__device__ __forceinline__ Best16 group_best16(Best16 b) {
    long long key = (long long)b.m * 4294967296LL + (long long)(unsigned)(b.at + 1);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const long long other = __shfl_xor_sync(0xffffffffu, key, o);
        key = other > key ? other : key;
    }
    Best16 r;
    r.m = (int)(key >> 32);
    r.at = (int)(unsigned)(key & 0xffffffffu) - 1;
    return r;
}

// Penalty of a gap move (g: 1 up, 0 left) out of a cell with tag t:
// GO after a diagonal, GE after the same gap, 0 after the other gap
// (genCPU.cpp:404-414; a boundary cell's tag gives 0).
__device__ __forceinline__ int gap_pen(int g, int t) { return t == 3 ? -10 : (t == g ? -1 : 0); }

// Asynchronous 16-byte global-to-shared copies (cp.async), grouped.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Walks the path back from cell (i, j) to the boundary over the tags the
// sweep stored in `region`, a window of kDepth 16-step blocks at a time in
// `stage` (the G lanes of the pair copy it together; every lane walks).
// The path leaves a window [lo, top] exactly at block lo - 1 (a move goes
// back at most one block), so the windows come in a fixed order: with
// room for two, the next one is copied (cp.async) while the current one is
// walked.  Returns the diagonal moves in *na, the gap penalties in *gp;
// (i, j) ends at the boundary cell.
template <int G, int R>
__device__ __forceinline__ void walk16(const uint32_t* region, uint32_t* stage, const Pair16& pc, int gl,
                                       bool walking, int& i, int& j, int* na, int* gp) {
    constexpr int kGR = G * R;
    constexpr int kBlockWords = 2 * kGR;   // a block: parity 0, parity 1
    constexpr int kBlock4 = kBlockWords / 4;
    constexpr bool kDouble = kSmWords / kBlockWords >= 1;   // two windows of at least a block
    constexpr int kRoom = kDouble ? kSmWords / kBlockWords : (2 * kSmWords) / kBlockWords;
    constexpr int kDepth = kRoom < 8 ? kRoom : 8;
    constexpr int kBuf4 = kSmWords / 4;   // uint4 per buffer (double-buffered)
    static_assert(kDepth >= 1 && kGR % 4 == 0, "tag staging");
    const uint4* region4 = reinterpret_cast<const uint4*>(region);
    uint4* stage4 = reinterpret_cast<uint4*>(stage);
    auto below = [](int top) { return top < 0 ? -1 : max(0, top - kDepth + 1) - 1; };
    // window [max(0, top - kDepth + 1), top] into buffer b, one copy group
    // (empty for top < 0)
    auto issue = [&](int top, int b) {
        if (top >= 0) {
            const int lo = max(0, top - kDepth + 1);
            const int n4 = (top + 1 - lo) * kBlock4;
            const uint4* src = region4 + (int64_t)lo * kBlock4;
            uint4* dst = stage4 + b * kBuf4;
            for (int k = gl; k < n4; k += G) cp_async16(dst + k, src + k);
        }
        cp_async_commit();
    };
    int wtop = walking && i > 0 && j > 0 ? (i + j + pc.shift) >> 4 : -1;   // window walked next
    int ntop = below(wtop);                                                   // the one after it
    int cur = 0, lo = INT_MAX;
    if (kDouble) {
        issue(wtop, 0);
        issue(ntop, 1);
    }
    int a = 0, g = 0, gprev = -1;
    while (__any_sync(0xffffffffu, walking)) {
        const bool need = walking && i > 0 && j > 0;
        if (need) {
            lo = max(0, wtop - kDepth + 1);
            if (kDouble) {
                cp_async_wait<1>();   // the current window (the next may be in flight)
            } else {
                const int n4 = (wtop + 1 - lo) * kBlock4;
                const uint4* src = region4 + (int64_t)lo * kBlock4;
                for (int k = gl; k < n4; k += G) stage4[k] = src[k];
            }
        }
        __syncwarp();
        const uint32_t* buf = stage + (kDouble ? cur * kSmWords : 0);
        while (walking) {
            if (i == 0 || j == 0) {
                if (gprev >= 0) g += gap_pen(gprev, j == 0 ? 0 : 1);   // column 0: tag left, row 0: up
                walking = false;
                break;
            }
            const int tau = i + j + pc.shift;
            const int blk = tau >> 4;
            if (blk < lo) break;   // the next window
            const int par = tau & 1;
            const int q = (i - j + pc.kb - par) >> 1;
            const int hi = q >= kGR ? 1 : 0;
            const int qq = min(max(q - hi * kGR, 0), kGR - 1);   // in range for every in-band cell
            // the half's tags of this parity at steps tau, tau - 2, ... from bit 0 up
            const uint32_t w = buf[(blk - lo) * kBlockWords + par * kGR + qq];
            const uint32_t x = ((w >> (16 * hi)) & 0xFFFFu) >> (2 * (7 - ((tau & 15) >> 1)));
            const int t = (int)(x & 3u);
            if (gprev >= 0) g += gap_pen(gprev, t);
            if (t == 3) {
                // a diagonal move keeps the slot and the parity: the run of
                // diagonal tags at steps tau, tau - 2, ... in this word
                const uint32_t z = ~(x & (x >> 1)) & 0x5555u;
                const int k = min(z ? (__ffs(z) - 1) >> 1 : 8, min(i, j));
                a += k; i -= k; j -= k; gprev = -1;
            } else if (t == 1) {
                --j; gprev = 1;
            } else {
                --i; gprev = 0;
            }
        }
        __syncwarp();
        if (need) {
            // the window is walked: its buffer takes the window after the next
            const int t2 = below(ntop);
            if (kDouble) issue(t2, cur);
            cur ^= 1;
            wtop = ntop;
            ntop = t2;
        }
    }
    if (kDouble) cp_async_wait<0>();   // no copy may land in the next pair's sequences
    __syncwarp();
    *na = a;
    *gp = g;
}

template <int G, int R>
__global__ void __launch_bounds__(kThreads, min_blocks16<R>()) gen16_kernel(GenArgs a) {
    constexpr int kPerWarp = 32 / G;
    static_assert(R <= 16, "a lane's slot windows must fit one 32-symbol window per read");
    // per pair: read1, read2; a stride of 4 words over 32 banks puts the
    // pairs of a warp, which read the same offsets, in different banks
    __shared__ __align__(16) uint32_t smem[kWarps][kPerWarp][kPairWords];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / G, gl = lane % G;
    uint32_t* sm1 = smem[warp][sub];
    uint32_t* sm2 = sm1 + kSmWords;
    const Mul mu = make_mul(a.one);
    const uint32_t sel0 = gl == 0 ? 0x1054u : 0x3210u;       // parity 0: lane 0's low half moves up
    const uint32_t sel1 = gl == G - 1 ? 0x7632u : 0x3210u;   // parity 1: last lane's high half moves down
    int64_t base = a.queue ? -1 : ((int64_t)blockIdx.x * kWarps + warp) * kPerWarp;
    const int64_t stride = (int64_t)gridDim.x * kWarps * kPerWarp;
    // this sub-group's tag region: [sub-block][lane][register] words
    const int64_t region_words = (int64_t)a.dir_blocks * 2 * G * R;
    uint32_t* region = a.dirs + (((int64_t)blockIdx.x * kWarps + warp) * kPerWarp + sub) * region_words;
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
        Pair16 pc{0, 0, 0, 0, {INT_MIN / 2, INT_MIN / 2, INT_MIN / 2, INT_MIN / 2}};
        int2 pr = make_int2(0, 0);
        if (valid) {
            p = a.order ? (int64_t)a.order[item] : item;
            pr = a.pairs[p];
            pc.l1 = a.len[pr.x];
            pc.l2 = a.len[pr.y];
            pc.kb = kband16(pc.l1, pc.l2, a.band);
        }
        pc.shift = pc.kb & 1;
        if (valid) {
            // last row i = l2: slot (2 l2 - s + kb - P) / 2 falls in [qa, qa + R) for
            // s in [2 l2 + kb - 2 qa - 2R + 1, 2 l2 + kb - 2 qa]; last column j = l1:
            // slot (s - 2 l1 + kb - P) / 2 for s in [2 l1 - kb + 2 qa, 2 l1 - kb + 2 qa + 2R - 1]
            const int qlo = gl * R, qhi = (G + gl) * R;
            pc.tw[0] = 2 * pc.l2 + pc.kb - 2 * qlo - 2 * R + 1;
            pc.tw[1] = 2 * pc.l2 + pc.kb - 2 * qhi - 2 * R + 1;
            pc.tw[2] = 2 * pc.l1 - pc.kb + 2 * qlo;
            pc.tw[3] = 2 * pc.l1 - pc.kb + 2 * qhi;
        }
        const int nw1 = (pc.l1 + 15) >> 4, nw2 = (pc.l2 + 15) >> 4;
        const uint32_t* g1 = a.packed + (valid ? a.woff[pr.x] : 0);
        const uint32_t* g2 = a.packed + (valid ? a.woff[pr.y] : 0);
        for (int k = gl; k < kPlaneWords; k += G) {
            plane_word(g1, nw1, k, sm1[k], sm1[kPlaneWords + k]);
            plane_word(g2, nw2, k, sm2[k], sm2[kPlaneWords + k]);
        }
        __syncwarp();
        St<R> st;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            // a closed cell (key 8) has the diagonal base (8 | 3) + 28 = 39
            st.K[0][r] = 39u * kLo; st.K[1][r] = 39u * kLo; st.U[r] = kOut2; st.F[r] = kOut2;
            st.D[0][r] = 0; st.D[1][r] = 0;
            st.MW[0][r] = 0; st.MW[1][r] = 0;
            // every cap starts closed; a slot's boundary cell opens it
            st.CP[0][r] = kOut2; st.CP[1][r] = kOut2;
        }
        Best16 col{kRefNegInf, -1}, row{kRefNegInf, -1};
        // the sweep ends at the last in-band cell of the last row or column
        int s_end = -1;
        if (valid) {
            if (max(1, pc.l2 - pc.kb) <= min(pc.l1, pc.l2 + pc.kb)) s_end = pc.l2 + min(pc.l1, pc.l2 + pc.kb);
            if (max(1, pc.l1 - pc.kb) <= min(pc.l2, pc.l1 + pc.kb))
                s_end = max(s_end, pc.l1 + min(pc.l2, pc.l1 + pc.kb));
        }
        const int t_end = (int)__reduce_max_sync(0xffffffffu, (unsigned)max(0, s_end + pc.shift));
        // the region holds dir_blocks blocks (sized on the host for the
        // launch's longest pair); a sweep that would not fit stores nothing
        // and reports ML = AL = -1
        const bool fits = (t_end >> 4) < a.dir_blocks;
        const int clean_hi = 2 * min(pc.l1, pc.l2) - pc.kb - 1;
        constexpr int kBlock = kSteps;
        for (int t0 = 0; t0 <= t_end; t0 += kBlock) {
            const int s0 = t0 - pc.shift;
            const bool finished = s0 > s_end;
            if ((t0 & (kSetupSteps - 1)) == 0) block_setup<G, R>(st, sm1, sm2, gl, s0, pc, finished);
            uint32_t* dst = fits && !finished ? region + ((int64_t)(t0 >> 4) * 2 * G + gl) * R : nullptr;
            const bool started = s0 > pc.kb;   // every boundary cell is behind (s = |d| <= kb)
            const bool clean = finished || (started && s0 + kBlock - 1 < clean_hi);
            if (__all_sync(0xffffffffu, clean))
                block16<G, R, kClean>(st, gl, s0, pc, mu, sel0, sel1, col, row, dst);
            else if (__all_sync(0xffffffffu, started || finished))
                block16<G, R, kTrack>(st, gl, s0, pc, mu, sel0, sel1, col, row, dst);
            else
                block16<G, R, kStart>(st, gl, s0, pc, mu, sel0, sel1, col, row, dst);
        }
        col = group_best16<G>(col);
        row = group_best16<G>(row);
        const bool use_col = col.m > row.m;   // genKernel.cu:765-768
        const Best16 b = use_col ? col : row;
        // end cell E: last row (l2, at) or last column (at, l1)
        int wi = use_col ? pc.l2 : b.at, wj = use_col ? b.at : pc.l1;
        int na = 0, gp = 0;
        __syncwarp();   // the sub-group's tag stores before its loads; the sequences are dead
        walk16<G, R>(region, sm1, pc, gl, fits && valid && b.at >= 0, wi, wj, &na, &gp);
        if (gl == 0 && valid) {
            int mlv = 0, alv = 0;
            if (!fits) {
                mlv = alv = -1;
            } else if (b.at >= 0) {
                const int ij = use_col ? pc.l2 + b.at : b.at + pc.l1;
                const int mism = (5 * na + gp - b.m) / 9;   // M(E) = 5 na - 9 mism + gp
                alv = ij - na;
                mlv = ij - 2 * na + mism - (wi + wj);
            }
            a.dist[p] = __fdiv_rn((float)mlv, (float)alv);
            if (a.score) a.score[p] = b.m;
            if (a.ml) a.ml[p] = mlv;
            if (a.al) a.al[p] = alv;
        }
        __syncwarp();
        if (!a.queue) base += stride;
    }
}

constexpr Shape16 kShapes16[] = {{4, 1}, {4, 2}, {4, 4}, {8, 2}, {4, 5}, {4, 6}, {8, 3},
                                 {4, 7}, {8, 4}, {8, 5}, {8, 6}, {16, 4}, {16, 6}, {32, 4}};
constexpr int kNumShapes16 = sizeof(kShapes16) / sizeof(kShapes16[0]);
constexpr bool shapes_within_max_r() {
    for (const Shape16& h : kShapes16)
        if (h.r > kGen16MaxR) return false;
    return true;
}
static_assert(shapes_within_max_r(), "kGen16MaxR bounds every shape's registers");

using Fn16 = void (*)(GenArgs);
Fn16 fn16(int i) {
    switch (i) {
        case 0: return gen16_kernel<4, 1>;
        case 1: return gen16_kernel<4, 2>;
        case 2: return gen16_kernel<4, 4>;
        case 3: return gen16_kernel<8, 2>;
        case 4: return gen16_kernel<4, 5>;
        case 5: return gen16_kernel<4, 6>;
        case 6: return gen16_kernel<8, 3>;
        case 7: return gen16_kernel<4, 7>;
        case 8: return gen16_kernel<8, 4>;
        case 9: return gen16_kernel<8, 5>;
        case 10: return gen16_kernel<8, 6>;
        case 11: return gen16_kernel<16, 4>;
        case 12: return gen16_kernel<16, 6>;
        default: return gen16_kernel<32, 4>;
    }
}

}  // namespace

int gen16_num_shapes() { return kNumShapes16; }
Shape16 gen16_shape(int i) { return kShapes16[i]; }
int gen16_pairs_per_block(int i) { return kWarps * (32 / kShapes16[i].g); }

namespace {
int gen16_grid(crispy_ctx* ctx, int shape, int64_t count) {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn16(shape), kThreads, 0);
    const int64_t per_block = gen16_pairs_per_block(shape);
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(1, per_sm) * ctx->sm_count,
                                                       (count + per_block - 1) / per_block));
}
}  // namespace

int64_t gen16_lane_regs_per_sm() {
    static const int64_t v = [] {
        int64_t best = 0;
        for (int i = 0; i < kNumShapes16; ++i) {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn16(i), kThreads, 0) != cudaSuccess) {
                cudaGetLastError();
                per_sm = 2048 / kThreads;
            }
            best = std::max<int64_t>(best, (int64_t)per_sm * kThreads * kShapes16[i].r);
        }
        return best;
    }();
    return v;
}

int64_t gen16_dir_words(crispy_ctx* ctx, int shape, int64_t count, int dir_blocks) {
    const Shape16 h = kShapes16[shape];
    // one region per pair slot of the grid: blocks x threads / G pairs
    return (int64_t)gen16_grid(ctx, shape, count) * kThreads / h.g * dir_blocks * 2 * h.g * h.r;
}

int gen16_launch(crispy_ctx* ctx, cudaStream_t s, int shape, const GenArgs& a, bool timed) {
    const int blocks = gen16_grid(ctx, shape, a.count);
    if (!a.dirs || a.dir_blocks < 1 || a.dirs_words < gen16_dir_words(ctx, shape, a.count, a.dir_blocks))
        return fail(ctx, CRISPY_E_STATE, "gen16: tag storage of %lld words for %lld pairs is too small",
                    (long long)a.dirs_words, (long long)a.count);
    if (timed) ev_begin(ctx, ctx->ev_gen, s);
    fn16(shape)<<<blocks, kThreads, 0, s>>>(a);
    if (timed) ev_end(ctx, ctx->ev_gen, s);
    count_launch(ctx);
    return CRISPY_OK;
}

}  // namespace crispy
