// Test infrastructure (never part of the engine): orders genDist survivor
// records the way the reference orders each chunk before writing it --
// thrust::sort_by_key on the device over float distance keys carrying the
// (uint, uint) read pairs (genCUDA.cu:39-45).  The engine orders its chunks
// with its own stable radix sort; tests/test_thrust_order_gpu.py compares
// the two orders, so the library's ordering of equal distances is pinned by
// the library itself.
//
//   thrust_order <in> <out>
//   in:  int64 n, then n float32 distances, then n uint32 pairs (2n words)
//   out: the same layout, sorted by distance
#include <thrust/copy.h>
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>
#include <thrust/pair.h>
#include <thrust/sort.h>

#include <cstdint>
#include <cstdio>
#include <vector>

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: thrust_order <in> <out>\n");
        return 2;
    }
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int64_t n = 0;
    if (std::fread(&n, 8, 1, f) != 1 || n < 0) { std::fclose(f); return 4; }
    std::vector<float> dist((size_t)n);
    std::vector<uint32_t> pairs((size_t)n * 2);
    const bool ok = std::fread(dist.data(), 4, (size_t)n, f) == (size_t)n &&
                    std::fread(pairs.data(), 4, (size_t)n * 2, f) == (size_t)n * 2;
    std::fclose(f);
    if (!ok) return 5;
    thrust::host_vector<float> h_dist(dist.begin(), dist.end());
    thrust::host_vector<thrust::pair<unsigned int, unsigned int>> h_pair((size_t)n);
    for (int64_t i = 0; i < n; ++i) h_pair[(size_t)i] = thrust::make_pair(pairs[2 * i], pairs[2 * i + 1]);
    thrust::device_vector<float> d_dist = h_dist;
    thrust::device_vector<thrust::pair<unsigned int, unsigned int>> d_pair = h_pair;
    thrust::sort_by_key(d_dist.begin(), d_dist.end(), d_pair.begin());
    thrust::copy(d_dist.begin(), d_dist.end(), h_dist.begin());
    thrust::copy(d_pair.begin(), d_pair.end(), h_pair.begin());
    for (int64_t i = 0; i < n; ++i) {
        dist[(size_t)i] = h_dist[(size_t)i];
        pairs[2 * i] = h_pair[(size_t)i].first;
        pairs[2 * i + 1] = h_pair[(size_t)i].second;
    }
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 6;
    const bool wok = std::fwrite(&n, 8, 1, o) == 1 && std::fwrite(dist.data(), 4, (size_t)n, o) == (size_t)n &&
                     std::fwrite(pairs.data(), 4, (size_t)n * 2, o) == (size_t)n * 2;
    return std::fclose(o) == 0 && wok ? 0 : 7;
}
