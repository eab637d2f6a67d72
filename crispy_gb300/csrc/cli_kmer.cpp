// kmerDist -- drop-in replacement for the reference's bin/kmerDist.
//
// Same command line (kmerMain.cpp:229-272): -i <fasta> (required), -k K
// (default 6), -t thr (used only inside [0,1]), -d (also write .kdist),
// -n threads and -c are accepted for compatibility; the GB300 engine is the
// only implementation (there is no CPU fallback).  Same files: <in>.kpair =
// int32 (row, col) pairs and, with -d, <in>.kdist = float32 distances, in
// the reference's stage order.  Progress lines mirror the reference's.
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "crispy_gb300.h"

namespace {

void help() {
    std::printf("<-i inFileName>: FASTA file \n");
    std::printf("[-t threshold] : value range: 0.0 to 1.0, default: 2/log2(numReads)\n");
    std::printf("[-k K]         : k-mer length 1..8, default: 6\n");
    std::printf("[-n numThreads]: accepted for compatibility\n");
    std::printf("[-d]           : output kmer distances \n");
    std::printf("[-c]           : accepted for compatibility (the GPU engine always runs)\n");
    std::printf("[-h]           : help\n");
}

struct Out {
    FILE* pair;
    FILE* dist;
};

int write_batch(void* user, int, const void* pairs, const float* dists, int64_t count) {
    Out* o = static_cast<Out*>(user);
    if (std::fwrite(pairs, sizeof(int32_t), (size_t)count * 2, o->pair) != (size_t)count * 2) return 1;
    if (o->dist && dists && std::fwrite(dists, sizeof(float), (size_t)count, o->dist) != (size_t)count)
        return 1;
    return 0;
}

double now() {
    timeval t;
    gettimeofday(&t, nullptr);
    return t.tv_sec + t.tv_usec * 1e-6;
}

}  // namespace

int main(int argc, char** argv) {
    const double t0 = now();
    std::string in;
    float thr = -1;
    int K = 6;
    bool dists = false;
    for (int i = 0; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!std::strcmp(argv[i], "-i") && has) {
            in = argv[i + 1];
            if (in.size() < 2) { help(); return 255; }
        }
        if (!std::strcmp(argv[i], "-t") && has) thr = (float)std::atof(argv[i + 1]);
        if (!std::strcmp(argv[i], "-k") && has) K = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-d")) dists = true;
        if (!std::strcmp(argv[i], "-h")) { help(); return 255; }
    }
    if (in.size() < 2) { help(); return 255; }
    crispy_reads* reads = nullptr;
    if (crispy_reads_load_fasta(in.c_str(), 0, &reads) != CRISPY_OK) {
        std::printf("Error: %s. Exit...\n", crispy_last_error(nullptr));
        return 255;
    }
    const char* seq; const int64_t* off; const int32_t* len; int32_t n, maxlen;
    crispy_reads_view(reads, &seq, &off, &len, &n, &maxlen);
    if (n > CRISPY_MAX_NUM_READS || maxlen > CRISPY_MAX_READ_LEN) {
        std::printf("Error: unsupported numReads: %d or maxLen: %d. Exit...", n, maxlen);
        return 255;
    }
    thr = crispy_default_threshold(n, thr, 0);
    std::printf("\n----------------------------------------------------------------------\n");
    std::printf("                       COMPUTE KMER DISTANCES                           \n");
    std::printf("File name: %s. K = %d\n\n", in.c_str(), K);
    std::printf("numReads: %d, maxLen: %d, threshold: %.2f\n  ", n, maxlen, thr);
    const char* mode_env = std::getenv("CRISPY_MODE");
    const int mode = !mode_env ? CRISPY_MODE_BATCHED
                     : !std::strcmp(mode_env, "plain") ? CRISPY_MODE_PLAIN
                     : !std::strcmp(mode_env, "staged") ? CRISPY_MODE_STAGED : CRISPY_MODE_BATCHED;
    std::printf("USE GPU (GB300 engine, %s)\n", mode == CRISPY_MODE_PLAIN ? "plain" : mode == CRISPY_MODE_STAGED ? "staged" : "batched");
    crispy_ctx* ctx = nullptr;
    int rc = crispy_ctx_create(0, &ctx);
    if (rc != CRISPY_OK) { std::fprintf(stderr, "kmerDist: %s\n", crispy_last_error(nullptr)); return 255; }
    int64_t total = 0;
    rc = crispy_kmer_prepare(ctx, seq, off, len, n, K);
    if (rc == CRISPY_OK) rc = crispy_kmer_run(ctx, thr, mode, dists ? 1 : 0, &total);
    if (rc == CRISPY_OK) {
        Out o{std::fopen((in + ".kpair").c_str(), "wb"), nullptr};
        if (dists) o.dist = std::fopen((in + ".kdist").c_str(), "wb");
        if (!o.pair || (dists && !o.dist)) {
            std::fprintf(stderr, "kmerDist: cannot open output files\n");
            rc = CRISPY_E_IO;
        } else {
            rc = crispy_kmer_stream(ctx, write_batch, &o);
        }
        if (o.pair) std::fclose(o.pair);
        if (o.dist) std::fclose(o.dist);
    }
    if (rc != CRISPY_OK) {
        std::fprintf(stderr, "kmerDist: %s\n", crispy_last_error(ctx));
        crispy_ctx_destroy(ctx);
        crispy_reads_free(reads);
        return 255;
    }
    std::printf("totalNumPairs: %llu\n", (unsigned long long)total);
    crispy_ctx_destroy(ctx);
    crispy_reads_free(reads);
    std::printf("Time taken: %.3f s\n", now() - t0);
    std::printf("\n----------------------------------------------------------------------\n");
    return 0;
}
