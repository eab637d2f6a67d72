// genDist -- drop-in replacement for the reference's bin/genDist.
//
// Same command line (genMain.cpp:334-373): -i <fasta> (required; reads
// <fasta>.kpair), -b band (default 2; <= 0 means 2; 1 = unbanded), -t thr
// (used only inside [0,1]); -n and -c are accepted for compatibility.  Same
// files: <fasta>.npair_<f> (uint32 pairs) and <fasta>.ndist_<f> (float32),
// chunked at 589,824 survivors per load window and sorted stably by
// distance inside each chunk, exactly as aveclust expects.  The last line
// printed before the timing is the survivor count, as in the reference.
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "crispy_gb300.h"

namespace {

void help() {
    std::printf("<-i inFileName>: FASTA file. Require: output from kmerDist (inFileName.kpair) \n");
    std::printf("[-t threshold] : value range: 0.0 to 1.0, default: 1/log2(numReads)\n");
    std::printf("[-n numThreads]: accepted for compatibility\n");
    std::printf("[-b]           : use banded alignment, 1/band band width (default 2)\n");
    std::printf("[-c]           : accepted for compatibility (the GPU engine always runs)\n");
    std::printf("[-h]           : help\n");
}

struct Sink {
    std::string base;
    int err = 0;
};

int write_chunk(void* user, int chunk, const void* pairs, const float* dists, int64_t count) {
    Sink* s = static_cast<Sink*>(user);
    char suf[32];
    std::snprintf(suf, sizeof suf, "_%d", chunk);
    FILE* fp = std::fopen((s->base + ".npair" + suf).c_str(), "wb");
    FILE* fd = std::fopen((s->base + ".ndist" + suf).c_str(), "wb");
    int bad = !fp || !fd;
    if (!bad) {
        bad |= std::fwrite(pairs, sizeof(uint32_t), (size_t)count * 2, fp) != (size_t)count * 2;
        bad |= std::fwrite(dists, sizeof(float), (size_t)count, fd) != (size_t)count;
    }
    if (fp) std::fclose(fp);
    if (fd) std::fclose(fd);
    if (bad) s->err = 1;
    return bad;
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
    int band = 2;
    for (int i = 0; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!std::strcmp(argv[i], "-i") && has) {
            in = argv[i + 1];
            if (in.size() < 2) { help(); return 0; }
        }
        if (!std::strcmp(argv[i], "-t") && has) thr = (float)std::atof(argv[i + 1]);
        if (!std::strcmp(argv[i], "-b") && has) {
            band = std::atoi(argv[i + 1]);
            if (band <= 0) {
                std::printf("Warning: invalid band (-b option). Set to 2.\n");
                band = 2;
            }
        }
        if (!std::strcmp(argv[i], "-h")) { help(); return 0; }
    }
    if (in.size() < 2) { help(); return 0; }
    crispy_reads* reads = nullptr;
    if (crispy_reads_load_fasta(in.c_str(), 1, &reads) != CRISPY_OK) {
        std::printf("Error: %s. EXIT...\n", crispy_last_error(nullptr));
        return 255;
    }
    const char* seq; const int64_t* off; const int32_t* len; int32_t n, maxlen;
    crispy_reads_view(reads, &seq, &off, &len, &n, &maxlen);
    if (n > CRISPY_MAX_NUM_READS || maxlen > CRISPY_MAX_READ_LEN) {
        std::printf("Error: unsupported numReads or maxLen. Exit...%d\t%d\n", n, maxlen);
        return 255;
    }
    thr = crispy_default_threshold(n, thr, 1);
    std::printf("\n----------------------------------------------------------------------\n");
    std::printf("                    COMPUTE GENETIC DISTANCES                          \n");
    std::printf("File name: %s.\n", in.c_str());
    std::printf("numReads: %d. band: %d. threshold: %f\n\n", n, band, thr);
    FILE* fk = std::fopen((in + ".kpair").c_str(), "rb");
    if (!fk) {
        std::printf("Error: cannot open pair file: %s.kpair. Exit...\n", in.c_str());
        return 255;
    }
    std::vector<int32_t> pairs;
    {
        std::vector<int32_t> buf(1 << 20);
        size_t got;
        while ((got = std::fread(buf.data(), sizeof(int32_t), buf.size(), fk)) > 0)
            pairs.insert(pairs.end(), buf.begin(), buf.begin() + got);
        std::fclose(fk);
    }
    const int64_t npairs = (int64_t)pairs.size() / 2;   // a trailing odd int is ignored, as fread/2 does
    const char* mode_env = std::getenv("CRISPY_MODE");
    const int mode = !mode_env ? CRISPY_MODE_BATCHED
                     : !std::strcmp(mode_env, "plain") ? CRISPY_MODE_PLAIN
                     : !std::strcmp(mode_env, "staged") ? CRISPY_MODE_STAGED : CRISPY_MODE_BATCHED;
    std::printf("USE GPU (GB300 engine, %s)\n", mode == CRISPY_MODE_PLAIN ? "plain" : mode == CRISPY_MODE_STAGED ? "staged" : "batched");
    crispy_ctx* ctx = nullptr;
    int rc = crispy_ctx_create(0, &ctx);
    if (rc != CRISPY_OK) { std::fprintf(stderr, "genDist: %s\n", crispy_last_error(nullptr)); return 255; }
    Sink sink{in};
    int64_t total = 0;
    rc = crispy_gen_prepare(ctx, seq, off, len, n);
    if (rc == CRISPY_OK)
        rc = crispy_gen_run(ctx, pairs.data(), npairs, band, thr, mode, write_chunk, &sink, &total);
    if (rc != CRISPY_OK) {
        std::fprintf(stderr, "genDist: %s\n", crispy_last_error(ctx));
        crispy_ctx_destroy(ctx);
        crispy_reads_free(reads);
        return 255;
    }
    std::printf("%llu\n", (unsigned long long)total);
    crispy_ctx_destroy(ctx);
    crispy_reads_free(reads);
    std::printf("Time taken: %.3f s\n", now() - t0);
    std::printf("\n----------------------------------------------------------------------\n");
    return 0;
}
