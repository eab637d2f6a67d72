// aveclust -- drop-in for bin/aveclust (src/aveclust/aveclust.cpp), the
// step crispy.sh:24 runs after genDist.
//
//   aveclust -i <in> -n <numReads> -f <numFiles> [-e endLevel] [-o outFile] [-h]
//
// Same options and outputs as the reference (getOptions,
// aveclust.cpp:121-154; main, :663-1007): reads <in>.npair_<f> /
// <in>.ndist_<f> for f < numFiles, writes <in>_Merge, <in>.Cluster and
// <in>.Cluster_List, and with -o the edge lists outFile and
// outFile_Index1.  The clustering is crispy_aveclust.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "crispy_gb300.h"

namespace {

void help() {
    std::printf("-i <inFileName>\n-n <numReads>\n-f <numFiles>\n-h help description.\n");
}

bool read_all(const std::string& name, std::vector<char>& out) {
    FILE* f = std::fopen(name.c_str(), "rb");
    if (!f) return false;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) out.insert(out.end(), buf, buf + got);
    std::fclose(f);
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    std::string in, out;
    int num_reads = 0, num_files = 0;
    float end_level = -1.0f;
    for (int i = 0; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!std::strcmp(argv[i], "-i") && has) in = argv[i + 1];
        if (!std::strcmp(argv[i], "-n") && has) num_reads = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-f") && has) num_files = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-e") && has) end_level = (float)std::atof(argv[i + 1]);
        if (!std::strcmp(argv[i], "-o") && has) out = argv[i + 1];
        if (!std::strcmp(argv[i], "-h")) { help(); return 0; }
    }
    if (in.size() < 2 || num_reads < 1 || num_files < 1) { help(); return 0; }
    std::printf("\n----------------------------------------------------------------------\n");
    std::printf("                  AVERAGE CLUSTERING GENETIC DISTANCES                  \n");
    std::vector<std::vector<char>> pair_bytes(num_files), dist_bytes(num_files);
    std::vector<const uint32_t*> pairs(num_files);
    std::vector<const float*> dists(num_files);
    std::vector<int64_t> counts(num_files);
    for (int f = 0; f < num_files; ++f) {
        const std::string pn = in + ".npair_" + std::to_string(f), dn = in + ".ndist_" + std::to_string(f);
        if (!read_all(pn, pair_bytes[f])) { std::printf("Error: Cannot open file%s\n", pn.c_str()); return 255; }
        if (!read_all(dn, dist_bytes[f])) { std::printf("Error: Cannot open file%s\n", dn.c_str()); return 255; }
        // the reference takes the entry count from the distance file
        counts[f] = std::min<int64_t>((int64_t)dist_bytes[f].size() / 4, (int64_t)pair_bytes[f].size() / 8);
        pair_bytes[f].resize((size_t)counts[f] * 8 + 8);
        dist_bytes[f].resize((size_t)counts[f] * 4 + 4);
        pairs[f] = reinterpret_cast<const uint32_t*>(pair_bytes[f].data());
        dists[f] = reinterpret_cast<const float*>(dist_bytes[f].data());
    }
    std::printf("Use %d distance file(s).\n", num_files);
    crispy_clust_stats st{};
    const int rc = crispy_aveclust(pairs.data(), dists.data(), counts.data(), num_files, num_reads, end_level,
                                   in.c_str(), out.empty() ? nullptr : out.c_str(), &st);
    if (rc != CRISPY_OK) {
        std::fprintf(stderr, "aveclust: %s\n", crispy_last_error(nullptr));
        return 255;
    }
    std::printf("endLevel: %g\nDONE!\n\n%s\n", (double)st.end_level, st.report);
    std::printf("merges: %lld, clusters: %d, singletons: %d\n", (long long)st.merges, st.roots, st.singletons);
    std::printf("\n----------------------------------------------------------------------\n");
    return 0;
}
