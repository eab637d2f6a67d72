// crispyDist -- kmerDist and genDist in one process.
//
// crispy.sh runs bin/kmerDist and then bin/genDist (crispy.sh:19-20); the two
// talk through <fasta>.kpair on disk.  This executable runs both stages on
// one device context:
//   - the k-mer survivors stay in HBM and feed genDist directly;
//   - the reads are uploaded once when both stages parse the FASTA alike.
//     kmerDist trims trailing non-ACGT letters, genDist keeps N/n
//     (kmerMain.cpp:289-295, genMain.cpp:175-181).
// The files it writes are byte-identical to the two programs':
//   <fasta>.npair_<f> / .ndist_<f> always;
//   <fasta>.kpair with -p, and <fasta>.kdist with -p -d.
//
//   crispyDist -i <fasta> [-k K] [-t kmerThr] [-b band] [-g genThr] [-p] [-d]
//
// K, thresholds and band follow the two programs' defaults and clamps
// (K = 6; thresholds 2/log2 n and 1/log2 n; band 2, <= 0 -> 2, 1 = unbanded).
// CRISPY_MODE selects the form as for the two programs.  No reference
// counterpart.
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "crispy_gb300.h"

namespace {

void help() {
    std::printf("<-i inFileName>: FASTA file\n");
    std::printf("[-k K]         : k-mer length 1..8, default: 6\n");
    std::printf("[-t threshold] : k-mer distance cut, 0.0 to 1.0, default: 2/log2(numReads)\n");
    std::printf("[-b band]      : banded alignment, 1/band band width (default 2; 1 = unbanded)\n");
    std::printf("[-g threshold] : genetic distance cut, 0.0 to 1.0, default: 1/log2(numReads)\n");
    std::printf("[-p]           : also write inFileName.kpair (as kmerDist does)\n");
    std::printf("[-d]           : with -p, also write inFileName.kdist\n");
    std::printf("[-h]           : help\n");
}

struct KOut {
    FILE* pair;
    FILE* dist;
};

int write_kmer(void* user, int, const void* pairs, const float* dists, int64_t count) {
    KOut* o = static_cast<KOut*>(user);
    if (std::fwrite(pairs, sizeof(int32_t), (size_t)count * 2, o->pair) != (size_t)count * 2) return 1;
    if (o->dist && dists && std::fwrite(dists, sizeof(float), (size_t)count, o->dist) != (size_t)count)
        return 1;
    return 0;
}

int write_chunk(void* user, int chunk, const void* pairs, const float* dists, int64_t count) {
    const std::string& base = *static_cast<const std::string*>(user);
    char suf[32];
    std::snprintf(suf, sizeof suf, "_%d", chunk);
    FILE* fp = std::fopen((base + ".npair" + suf).c_str(), "wb");
    FILE* fd = std::fopen((base + ".ndist" + suf).c_str(), "wb");
    int bad = !fp || !fd;
    if (!bad) {
        bad |= std::fwrite(pairs, sizeof(uint32_t), (size_t)count * 2, fp) != (size_t)count * 2;
        bad |= std::fwrite(dists, sizeof(float), (size_t)count, fd) != (size_t)count;
    }
    if (fp) std::fclose(fp);
    if (fd) std::fclose(fd);
    return bad;
}

double now() {
    timeval t;
    gettimeofday(&t, nullptr);
    return t.tv_sec + t.tv_usec * 1e-6;
}

bool same_reads(crispy_reads* a, crispy_reads* b) {
    const char *sa, *sb;
    const int64_t *oa, *ob;
    const int32_t *la, *lb;
    int32_t na, nb, ma, mb;
    crispy_reads_view(a, &sa, &oa, &la, &na, &ma);
    crispy_reads_view(b, &sb, &ob, &lb, &nb, &mb);
    if (na != nb) return false;
    for (int32_t r = 0; r < na; ++r)
        if (la[r] != lb[r] || std::memcmp(sa + oa[r], sb + ob[r], (size_t)la[r]) != 0) return false;
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    const double t0 = now();
    std::string in;
    float kthr = -1, gthr = -1;
    int K = 6, band = 2;
    bool write_kpair = false, dists = false;
    for (int i = 0; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!std::strcmp(argv[i], "-i") && has) in = argv[i + 1];
        if (!std::strcmp(argv[i], "-k") && has) K = std::atoi(argv[i + 1]);
        if (!std::strcmp(argv[i], "-t") && has) kthr = (float)std::atof(argv[i + 1]);
        if (!std::strcmp(argv[i], "-g") && has) gthr = (float)std::atof(argv[i + 1]);
        if (!std::strcmp(argv[i], "-b") && has) {
            band = std::atoi(argv[i + 1]);
            if (band <= 0) {
                std::printf("Warning: invalid band (-b option). Set to 2.\n");
                band = 2;
            }
        }
        if (!std::strcmp(argv[i], "-p")) write_kpair = true;
        if (!std::strcmp(argv[i], "-d")) dists = true;
        if (!std::strcmp(argv[i], "-h")) { help(); return 255; }
    }
    if (in.size() < 2) { help(); return 255; }
    crispy_reads *kreads = nullptr, *greads = nullptr;
    if (crispy_reads_load_fasta(in.c_str(), 0, &kreads) != CRISPY_OK ||
        crispy_reads_load_fasta(in.c_str(), 1, &greads) != CRISPY_OK) {
        std::printf("Error: %s. Exit...\n", crispy_last_error(nullptr));
        crispy_reads_free(kreads);
        return 255;
    }
    const char* seq; const int64_t* off; const int32_t* len; int32_t n, maxlen;
    crispy_reads_view(kreads, &seq, &off, &len, &n, &maxlen);
    if (n > CRISPY_MAX_NUM_READS || maxlen > CRISPY_MAX_READ_LEN) {
        std::printf("Error: unsupported numReads: %d or maxLen: %d. Exit...", n, maxlen);
        crispy_reads_free(kreads);
        crispy_reads_free(greads);
        return 255;
    }
    kthr = crispy_default_threshold(n, kthr, 0);
    gthr = crispy_default_threshold(n, gthr, 1);
    const char* mode_env = std::getenv("CRISPY_MODE");
    const int mode = !mode_env ? CRISPY_MODE_BATCHED
                     : !std::strcmp(mode_env, "plain") ? CRISPY_MODE_PLAIN
                     : !std::strcmp(mode_env, "staged") ? CRISPY_MODE_STAGED : CRISPY_MODE_BATCHED;
    std::printf("\n----------------------------------------------------------------------\n");
    std::printf("                 COMPUTE KMER AND GENETIC DISTANCES                     \n");
    std::printf("File name: %s. K = %d. band: %d\n\n", in.c_str(), K, band);
    std::printf("numReads: %d, maxLen: %d, kmer threshold: %.2f, genetic threshold: %f\n", n, maxlen,
                kthr, gthr);
    crispy_ctx* ctx = nullptr;
    int rc = crispy_ctx_create(0, &ctx);
    if (rc != CRISPY_OK) {
        std::fprintf(stderr, "crispyDist: %s\n", crispy_last_error(nullptr));
        crispy_reads_free(kreads);
        crispy_reads_free(greads);
        return 255;
    }
    int64_t kpairs = 0, total = 0;
    rc = crispy_kmer_prepare(ctx, seq, off, len, n, K);
    if (rc == CRISPY_OK) rc = crispy_kmer_run(ctx, kthr, mode, dists ? 1 : 0, &kpairs);
    if (rc == CRISPY_OK && write_kpair) {
        KOut o{std::fopen((in + ".kpair").c_str(), "wb"), nullptr};
        if (dists) o.dist = std::fopen((in + ".kdist").c_str(), "wb");
        if (!o.pair || (dists && !o.dist)) {
            std::fprintf(stderr, "crispyDist: cannot open the .kpair / .kdist files\n");
            rc = CRISPY_E_IO;
        } else {
            rc = crispy_kmer_stream(ctx, write_kmer, &o);
        }
        if (o.pair) std::fclose(o.pair);
        if (o.dist) std::fclose(o.dist);
    }
    if (rc == CRISPY_OK) std::printf("totalNumPairs: %llu\n", (unsigned long long)kpairs);
    if (rc == CRISPY_OK) {
        if (same_reads(kreads, greads)) {
            rc = crispy_gen_prepare_from_kmer(ctx);
        } else {
            const char* gs; const int64_t* go; const int32_t* gl; int32_t gn, gm;
            crispy_reads_view(greads, &gs, &go, &gl, &gn, &gm);
            rc = crispy_gen_prepare(ctx, gs, go, gl, gn);
        }
    }
    if (rc == CRISPY_OK) rc = crispy_gen_run_from_kmer(ctx, band, gthr, mode, write_chunk, &in, &total);
    if (rc != CRISPY_OK) {
        std::fprintf(stderr, "crispyDist: %s\n", crispy_last_error(ctx));
        crispy_ctx_destroy(ctx);
        crispy_reads_free(kreads);
        crispy_reads_free(greads);
        return 255;
    }
    std::printf("%llu\n", (unsigned long long)total);
    crispy_ctx_destroy(ctx);
    crispy_reads_free(kreads);
    crispy_reads_free(greads);
    std::printf("Time taken: %.3f s\n", now() - t0);
    std::printf("\n----------------------------------------------------------------------\n");
    return 0;
}
