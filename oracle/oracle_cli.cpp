/*
 * oracle_cli.cpp -- command-line front end of the CPU restatement.
 *
 * TEST INFRASTRUCTURE ONLY.  `oracle_cli kmer ...` and `oracle_cli gen ...`
 * take the reference's kmerDist / genDist flags (kmerMain.cpp:229-272,
 * genMain.cpp:334-373) and write the same files in the GPU path's order
 * (.kpair/.kdist in stage order; .npair_<f>/.ndist_<f> chunked at 589,824
 * survivors).  Used by the tests to produce expected files and by bench.py
 * as the timed CPU baseline ("port").
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "oracle.h"

static double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

static int run_kmer(int argc, char** argv) {
    std::string in;
    float thr = -1;
    int K = 6, nthreads = 0;
    bool dists = false;
    for (int i = 0; i < argc; ++i) {
        if (!std::strcmp(argv[i], "-i") && i + 1 < argc) in = argv[i + 1];
        if (!std::strcmp(argv[i], "-t") && i + 1 < argc) thr = (float)std::atof(argv[i + 1]);
        if (!std::strcmp(argv[i], "-k") && i + 1 < argc) K = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-n") && i + 1 < argc) nthreads = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-d")) dists = true;
    }
    if (in.size() < 2 || K < 1 || K > 8) { std::fprintf(stderr, "usage: oracle_cli kmer -i <fasta> [-k K] [-t thr] [-d] [-n threads]\n"); return 2; }
    double t0 = now_s();
    oracle_fasta* f = nullptr;
    int n = oracle_fasta_read(in.c_str(), 0, &f);
    if (n < 0) { std::fprintf(stderr, "cannot read %s\n", in.c_str()); return 1; }
    const char* buf; const int64_t* off; const int32_t* len; int32_t maxlen;
    oracle_fasta_get(f, &buf, &off, &len, &maxlen);
    if (n > 1024 * 1024 || maxlen > 2048) { std::fprintf(stderr, "unsupported numReads %d or maxLen %d\n", n, maxlen); return 1; }
    float t = oracle_default_threshold(n, thr, 2);
    int A = oracle_array_dim(n);
    if (A <= 0) { std::fprintf(stderr, "fewer than 10 reads: no tile size\n"); return 1; }
    int64_t cap = 1 << 20;
    std::vector<int32_t> pairs;
    std::vector<float> d;
    int64_t total;
    for (;;) {
        pairs.resize(2 * cap); d.resize(cap);
        total = oracle_kmer_all(buf, off, len, n, K, t, A, nthreads, pairs.data(), d.data(), cap);
        if (total <= cap) break;
        cap = total;
    }
    if (total < 0) return 1;
    FILE* fp = std::fopen((in + ".kpair").c_str(), "wb");
    std::fwrite(pairs.data(), sizeof(int32_t), 2 * total, fp);
    std::fclose(fp);
    if (dists) {
        FILE* fd = std::fopen((in + ".kdist").c_str(), "wb");
        std::fwrite(d.data(), sizeof(float), total, fd);
        std::fclose(fd);
    }
    oracle_fasta_free(f);
    std::printf("numReads: %d, K: %d, threshold: %f, arrayDim: %d\ntotalNumPairs: %lld\nseconds: %.6f\n",
                n, K, t, A, (long long)total, now_s() - t0);
    return 0;
}

static int run_gen(int argc, char** argv) {
    std::string in;
    float thr = -1;
    int band = 2, nthreads = 0;
    for (int i = 0; i < argc; ++i) {
        if (!std::strcmp(argv[i], "-i") && i + 1 < argc) in = argv[i + 1];
        if (!std::strcmp(argv[i], "-t") && i + 1 < argc) thr = (float)std::atof(argv[i + 1]);
        if (!std::strcmp(argv[i], "-b") && i + 1 < argc) { band = std::atoi(argv[i + 1]); if (band <= 0) band = 2; }
        if (!std::strcmp(argv[i], "-n") && i + 1 < argc) nthreads = std::atoi(argv[i + 1]);
    }
    if (in.size() < 2) { std::fprintf(stderr, "usage: oracle_cli gen -i <fasta> [-b band] [-t thr] [-n threads]\n"); return 2; }
    double t0 = now_s();
    oracle_fasta* f = nullptr;
    int n = oracle_fasta_read(in.c_str(), 1, &f);
    if (n < 0) { std::fprintf(stderr, "cannot read %s\n", in.c_str()); return 1; }
    const char* buf; const int64_t* off; const int32_t* len; int32_t maxlen;
    oracle_fasta_get(f, &buf, &off, &len, &maxlen);
    if (n > 1024 * 1024 || maxlen > 2048) { std::fprintf(stderr, "unsupported numReads %d or maxLen %d\n", n, maxlen); return 1; }
    float t = oracle_default_threshold(n, thr, 1);
    FILE* fp = std::fopen((in + ".kpair").c_str(), "rb");
    if (!fp) { std::fprintf(stderr, "cannot open pair file\n"); return 1; }
    std::vector<int32_t> pairs;
    int32_t tmp[8192];
    size_t got;
    while ((got = std::fread(tmp, sizeof(int32_t), 8192, fp)) > 0) pairs.insert(pairs.end(), tmp, tmp + got);
    std::fclose(fp);
    int64_t np = (int64_t)pairs.size() / 2;
    for (int64_t p = 0; p < 2 * np; ++p)
        if (pairs[p] < 0 || pairs[p] >= n) { std::fprintf(stderr, "pair index out of range\n"); return 1; }
    std::vector<float> d(np);
    oracle_gen_all(buf, off, len, n, pairs.data(), np, band, nthreads, d.data(), nullptr, nullptr, nullptr);
    std::vector<uint32_t> op(2 * np + 2);
    std::vector<float> od(np + 1);
    std::vector<int64_t> sizes(np / 589824 + 4);
    int nc = oracle_gen_chunks(pairs.data(), d.data(), np, t, op.data(), od.data(), sizes.data(), (int)sizes.size());
    int64_t at = 0, total = 0;
    for (int c = 0; c < nc; ++c) {
        char suf[32];
        std::snprintf(suf, sizeof suf, "_%d", c);
        FILE* a = std::fopen((in + ".npair" + suf).c_str(), "wb");
        FILE* b = std::fopen((in + ".ndist" + suf).c_str(), "wb");
        std::fwrite(op.data() + 2 * at, sizeof(uint32_t), 2 * sizes[c], a);
        std::fwrite(od.data() + at, sizeof(float), sizes[c], b);
        std::fclose(a); std::fclose(b);
        at += sizes[c];
        total += sizes[c];
    }
    oracle_fasta_free(f);
    std::printf("numReads: %d, band: %d, threshold: %f\n%lld\nseconds: %.6f\n", n, band, t, (long long)total, now_s() - t0);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 2 && !std::strcmp(argv[1], "kmer")) return run_kmer(argc - 1, argv + 1);
    if (argc >= 2 && !std::strcmp(argv[1], "gen")) return run_gen(argc - 1, argv + 1);
    std::fprintf(stderr, "usage: oracle_cli kmer|gen ...\n");
    return 2;
}
