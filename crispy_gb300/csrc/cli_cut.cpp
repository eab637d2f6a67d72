// sparsecut -- drop-in for bin/sparsecut (src/sparsecut/sparsecut.cpp), the
// last step of crispy.sh (crispy.sh:29), run with the cutoff file the
// changepoint step writes.
//
//   sparsecut -i <in> -n <numReads> -c <cutoffFile> [-h]
//
// Same options and outputs as the reference (getOptions,
// sparsecut.cpp:75-99; main, :317-410): reads the cutoffs (one number per
// line) and <in>_Merge, writes <in>.Cluster and <in>.Cluster_List with the
// clusters at each cutoff.  The cut is crispy_sparsecut.
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cli_common.h"
#include "crispy_gb300.h"

namespace {

void help() {
    std::printf("-i <inFileName>\n-c <cutoffFileName>\n-n <numReads>\n-h help description.\n");
}

double now_s() {
    timeval t;
    gettimeofday(&t, nullptr);
    return (double)t.tv_sec + 1e-6 * (double)t.tv_usec;
}

}  // namespace

int main(int argc, char** argv) {
    const double t0 = now_s();
    std::string in, cut_name;
    int num_reads = 0;
    std::printf("\n----------------------------------------------------------------------\n");
    std::printf("                  DENDROGRAM CUTTING GENETIC DISTANCES                  \n");
    for (int i = 0; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!std::strcmp(argv[i], "-i") && has) in = argv[i + 1];
        if (!std::strcmp(argv[i], "-c") && has) cut_name = argv[i + 1];
        if (!std::strcmp(argv[i], "-n") && has) num_reads = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-h")) { help(); return 0; }
    }
    if (in.size() < 2 || num_reads < 1) { help(); return 0; }
    std::vector<float> cutoffs;
    const std::string err = crispy_cli::read_cutoffs(cut_name, cutoffs, true);
    if (!err.empty()) {
        std::fprintf(stderr, "sparsecut: %s\n", err.c_str());
        return 255;
    }
    crispy_clust_stats st{};
    if (crispy_sparsecut(in.c_str(), num_reads, cutoffs.data(), (int)cutoffs.size(), &st) != CRISPY_OK) {
        std::fprintf(stderr, "sparsecut: %s\n", crispy_last_error(nullptr));
        return 255;
    }
    std::printf("DONE!\ncurrent node: %lld\n\n%s\n", (long long)num_reads + st.merges, st.report);
    std::printf("Time taken: %.3f s\n", now_s() - t0);
    std::printf("\n----------------------------------------------------------------------\n");
    return 0;
}
