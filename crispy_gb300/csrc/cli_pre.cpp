// preprocess -- drop-in for bin/preprocess (src/preprocess/preprocess.cpp),
// the step crispy.sh:18 runs before kmerDist.
//
//   preprocess -i <in> [-o <out>] [-f q] [-p <primer file>] [-m N] [-s SD] [-h]
//
// Same options, defaults and outputs as the reference (getCommandOptions,
// preprocess.cpp:613-684; main, :686-726): <out> (default <in>_Clean) holds
// the deduplicated reads ordered by (length, byte order), <out>.frq each
// kept read's label and merged frequency.  Records are parsed on the host;
// the length / N / primer filters and the duplicate merge run on the GPU
// (crispy_preprocess).  Like the reference, a run that finishes returns 1
// (main ends with `return 1`), and a failure returns 255 (exit(-1)).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "crispy_gb300.h"

namespace {

void help() {
    std::cout << "<-i inFileName>" << std::endl;
    std::cout << "[-f input format a(FASTA) q(FASTQ), default: a" << std::endl;
    std::cout << "[-p primerFileName]" << std::endl;
    std::cout << "[-m number of mismatches to primers allowed, default 2]" << std::endl;
    std::cout << "[-s standard deviation from average length allowed, default 1.0]" << std::endl;
    std::cout << "[-h  help]" << std::endl;
}

void trim_space(std::string& s) {   // deleteSpaces (preprocess.cpp:58-64)
    const size_t k = s.find_last_not_of("\n\r \t\v\f\b");
    if (k != std::string::npos) s.erase(k + 1);
}

}  // namespace

int main(int argc, char** argv) {
    const std::clock_t t0 = std::clock();
    std::string in, out, primer_file, primer = "$";
    bool fastq = false, primer_check = false, length_check = false;
    int max_mm = 2;
    double sd_allowed = 1.0;
    for (int i = 0; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!std::strcmp(argv[i], "-i") && has) {
            in = argv[i + 1];
            if (in.size() < 2) { help(); return 255; }
        }
        if (!std::strcmp(argv[i], "-o") && has) out = argv[i + 1];
        if (!std::strcmp(argv[i], "-f") && has && !std::strcmp(argv[i + 1], "q")) fastq = true;
        if (!std::strcmp(argv[i], "-p") && has) { primer_file = argv[i + 1]; primer_check = true; }
        if (!std::strcmp(argv[i], "-m") && has) max_mm = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-s") && has) { sd_allowed = std::atof(argv[i + 1]); length_check = true; }
        if (!std::strcmp(argv[i], "-h")) { help(); return 255; }
    }
    if (out.size() < 2) out = in + "_Clean";
    if (primer_check) {
        std::ifstream pf(primer_file.c_str());
        if (pf.fail()) {
            std::printf("Error: cannot open primer file. EXIT...");
            return 255;
        }
        std::getline(pf, primer);
        trim_space(primer);
    }
    std::printf("\n--------------------------------------------------------------------\n");
    std::printf("\n                            PREPROCESS\t               \t\t\t  \n");
    std::cout << (fastq ? "Format: FASTQ." : "Format: FASTA.") << std::endl;
    crispy_raw* raw = nullptr;
    int rc = crispy_raw_load(in.c_str(), fastq ? 1 : 0, &raw);
    if (rc == CRISPY_E_IO) {
        std::cout << "Can not open read file. Press any key to exit..." << std::endl;
        return 255;
    }
    if (rc != CRISPY_OK) {
        std::printf("Error: the read file is not in FASTA format. EXIT...\n");
        return 255;
    }
    const char* seq; const int64_t* off; const int32_t* len; const uint8_t* freq; int32_t n, records;
    crispy_raw_view(raw, &seq, &off, &len, &freq, &n, &records);
    std::printf("File name: %s.\n", in.c_str());

    crispy_ctx* ctx = nullptr;
    rc = crispy_ctx_create(0, &ctx);
    std::vector<int32_t> index((size_t)n), mult((size_t)n);
    crispy_pre_opts opts{length_check ? 1 : 0, sd_allowed, primer_check ? primer.c_str() : nullptr, max_mm};
    crispy_pre_stats st{};
    if (rc == CRISPY_OK) rc = crispy_preprocess(ctx, seq, off, len, freq, n, &opts, index.data(), mult.data(), &st);
    if (rc != CRISPY_OK) {
        std::fprintf(stderr, "preprocess: %s\n", crispy_last_error(ctx));
        crispy_ctx_destroy(ctx);
        crispy_raw_free(raw);
        return 255;
    }
    if (length_check) {   // processReadLength's report (preprocess.cpp:344-389)
        if (st.length_reads == 0) {
            std::cout << "Error in processReadLength" << std::endl;
        } else {
            std::cout << "minLen: " << st.min_len0 << "\t\tmaxLen: " << st.max_len0 << std::endl;
            std::cout << "aveLen: " << st.ave_len << "\t\tSD: " << st.sd << std::endl;
            std::cout << "minLen: " << st.min_len << "\t\tmaxLen: " << st.max_len << std::endl;
        }
    }
    const int deleted = st.length_discards + st.primer_discards + st.merges;
    std::printf("Total numReads: %d. Preprocessed numReads: %d\n", records, records - deleted);
    rc = crispy_pre_write(raw, index.data(), mult.data(), st.kept, out.c_str(), fastq ? 1 : 0);
    crispy_ctx_destroy(ctx);
    crispy_raw_free(raw);
    if (rc != CRISPY_OK) {
        std::printf("Error: cannot open output files. EXIT...");
        return 255;
    }
    std::printf("\nTime taken: %.3f secs\n", (double)(std::clock() - t0) / CLOCKS_PER_SEC);
    std::printf("\n--------------------------------------------------------------------\n");
    return 1;
}
