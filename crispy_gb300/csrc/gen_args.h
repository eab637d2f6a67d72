// gen_args.h -- launch arguments shared by the genDist DP kernels (gen.cu,
// gen16.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

struct crispy_ctx;

namespace crispy {

struct GenArgs {
    const uint32_t* packed;  // reads, 16 symbols per word, first symbol in the top bits
    const int64_t* woff;     // first packed word of each read
    const int32_t* len;
    const int2* pairs;
    const uint32_t* order;   // optional permutation (length buckets)
    int64_t count;
    int band;
    float* dist;
    int32_t* score;
    int32_t* ml;
    int32_t* al;
    unsigned int* queue;     // optional work counter (persistent launch)
    // 16-bit kernel only: every cell's choice, 2 bits, for the path walk
    // (gen16_dir_words words: one region per pair the grid holds at a
    // time, dir_blocks 16-step blocks long)
    uint32_t* dirs;
    int64_t dirs_words;
    int dir_blocks;
    // All 1.  Adds written as multiply-adds by these run on the FMA pipe;
    // distinct multipliers keep the compiler from factoring a common
    // product back into ALU adds.
    int one[6];
};

// The two-cells-per-register DP (gen16.cu) holds a cell as a 16-bit key
// whose range covers pairs with L1 + L2 <= kGen16MaxSum; longer pairs take
// the 32-bit kernels of gen.cu.
constexpr int kGen16MaxSum = 3600;

// Shapes of the 16-bit kernel: G lanes per pair, R registers per lane, so
// a pair with kBand + 1 <= 2 * G * R band slots fits.
struct Shape16 {
    int g, r;
};
int gen16_num_shapes();
Shape16 gen16_shape(int i);
// Pairs per block of a shape (all its warps).
int gen16_pairs_per_block(int i);
// Registers per lane of the widest shape (bounds the tag storage).
constexpr int kGen16MaxR = 7;
// 16-step blocks a pair's sweep runs at most, for pairs with L1 + L2 <= max_sum.
inline int gen16_dir_blocks(int max_sum) { return (max_sum + 1) / 16 + 1; }
// Words of choice storage a launch of shape i over `count` pairs needs.
int64_t gen16_dir_words(crispy_ctx* ctx, int shape, int64_t count, int dir_blocks);
// Largest resident threads x registers per lane of one SM over the shapes:
// a launch holds at most this many tag words per SM and sub-block.
int64_t gen16_lane_regs_per_sm();
// Launch shape i over a.count pairs: persistent grid sized by occupancy.
int gen16_launch(crispy_ctx* ctx, cudaStream_t s, int shape, const GenArgs& a, bool timed);

}  // namespace crispy
