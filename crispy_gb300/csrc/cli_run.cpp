// crispyRun -- crispy.sh in one process (the R changepoint step excepted).
//
// crispy.sh:18-24 runs
//     ./bin/preprocess -i $INPUT
//     ./bin/kmerDist  -i $INPUT"_Clean" -k $K
//     ./bin/genDist   -i $INPUT"_Clean" -b $B
//     NUM_READS=`grep '>' $INPUT"_Clean" | wc -l`;  NUM_FILES=`ls ...ndist* | wc -l`
//     ./bin/aveclust  -i $INPUT"_Clean" -n $NUM_READS -f $NUM_FILES
// and crispy.sh:26-29 then cuts the dendrogram at the changepoint's cutoffs
//     R ... crispy_changepoint.r --args $INPUT"_Clean_Merge"   (-> optimal_cutoff.txt)
//     ./bin/sparsecut -i $INPUT"_Clean" -n $NUM_READS -c optimal_cutoff.txt
// as separate programs that hand the reads over through the _Clean file, the
// k-mer survivors through the .kpair file and the genetic distances through
// the .npair_N / .ndist_N chunks.  This executable writes the same files
// (<in>_Clean, .frq, .kpair, .npair_<f> / .ndist_<f>, _Merge byte for byte;
// .Cluster / .Cluster_List with the same clusters, see crispy_aveclust)
// from one device context: the raw records go up once, preprocess keeps its
// kept reads on the device and both stages start from them
// (crispy_kmer_prepare_from_pre, crispy_gen_prepare_from_pre), the k-mer
// survivors feed genDist in HBM, and the chunks feed aveclust from memory.
// When a kept read would come back from the _Clean file split into several
// lines (whitespace inside a read, very long reads or headers), the stages
// read the written _Clean file instead, as the programs do.  NUM_FILES is
// the number of chunks this run wrote (crispy.sh's `ls` would also count
// chunk files an earlier, larger run left behind).
//
//   crispyRun <input file> [K (default 6)] [band (default 10)] [cutoff file]
//
// The first three arguments and their defaults are crispy.sh's
// (crispy.sh:1-16); the thresholds are the stages' defaults.  R is not part
// of this engine: given a cutoff file (as the changepoint step writes it),
// the sparsecut step runs on it and rewrites .Cluster / .Cluster_List with
// the clusters at those cutoffs (crispy_sparsecut).  CRISPY_MODE selects the form as for
// kmerDist / genDist.  No reference counterpart as a single program.
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cli_common.h"
#include "crispy_gb300.h"

namespace {

struct KOut {
    FILE* pair;
};

int write_kmer(void* user, int, const void* pairs, const float*, int64_t count) {
    KOut* o = static_cast<KOut*>(user);
    return std::fwrite(pairs, sizeof(int32_t), (size_t)count * 2, o->pair) != (size_t)count * 2;
}

struct Chunks {
    std::string base;
    std::vector<std::vector<uint32_t>> pairs;
    std::vector<std::vector<float>> dists;
};

int write_chunk(void* user, int chunk, const void* pairs, const float* dists, int64_t count) {
    Chunks& ck = *static_cast<Chunks*>(user);
    const std::string& base = ck.base;
    const uint32_t* pp = static_cast<const uint32_t*>(pairs);
    ck.pairs.emplace_back(pp, pp + 2 * count);
    ck.dists.emplace_back(dists, dists + count);
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

// The stage's reads from the written _Clean file (flavour 0 = kmerDist,
// 1 = genDist), for the cases the device hand-over declines.
int prepare_from_file(crispy_ctx* ctx, const std::string& clean, int flavour, int K, int32_t* nreads) {
    crispy_reads* rd = nullptr;
    int rc = crispy_reads_load_fasta(clean.c_str(), flavour, &rd);
    if (rc != CRISPY_OK) return rc;
    const char* seq; const int64_t* off; const int32_t* len; int32_t n, maxlen;
    crispy_reads_view(rd, &seq, &off, &len, &n, &maxlen);
    *nreads = n;
    rc = flavour == 0 ? crispy_kmer_prepare(ctx, seq, off, len, n, K) : crispy_gen_prepare(ctx, seq, off, len, n);
    crispy_reads_free(rd);
    return rc;
}

}  // namespace

int main(int argc, char** argv) {
    const double t0 = now();
    if (argc < 2 || !std::strcmp(argv[1], "-h")) {
        std::printf("Correct syntax: crispyRun <input file name> [k value] [band value] [cutoff file]\n");
        return 255;
    }
    const std::string in = argv[1];
    const int K = argc > 2 ? std::atoi(argv[2]) : 6;
    int band = argc > 3 ? std::atoi(argv[3]) : 10;
    if (band <= 0) band = 2;   // genMain.cpp:356-364
    const std::string clean = in + "_Clean";
    const char* mode_env = std::getenv("CRISPY_MODE");
    const int mode = !mode_env ? CRISPY_MODE_BATCHED
                     : !std::strcmp(mode_env, "plain") ? CRISPY_MODE_PLAIN
                     : !std::strcmp(mode_env, "staged") ? CRISPY_MODE_STAGED : CRISPY_MODE_BATCHED;

    crispy_raw* raw = nullptr;
    if (crispy_raw_load(in.c_str(), 0, &raw) != CRISPY_OK) {
        std::printf("Error: %s. Exit...\n", crispy_last_error(nullptr));
        return 255;
    }
    const char* seq; const int64_t* off; const int32_t* len; const uint8_t* freq; int32_t n, records;
    crispy_raw_view(raw, &seq, &off, &len, &freq, &n, &records);
    crispy_ctx* ctx = nullptr;
    int rc = crispy_ctx_create(0, &ctx);
    std::vector<int32_t> index((size_t)n + 1), mult((size_t)n + 1);
    crispy_pre_stats st{};
    if (rc == CRISPY_OK) rc = crispy_preprocess(ctx, seq, off, len, freq, n, nullptr, index.data(), mult.data(), &st);
    if (rc == CRISPY_OK) rc = crispy_pre_write(raw, index.data(), mult.data(), st.kept, clean.c_str(), 0);
    if (rc == CRISPY_OK)
        std::printf("Total numReads: %d. Preprocessed numReads: %d\n", records,
                    records - st.length_discards - st.primer_discards - st.merges);

    // kmerDist on the kept reads
    bool from_file = false;
    int64_t kpairs = 0, total = 0;
    int32_t nk = st.kept, ng = st.kept;   // reads each stage sees
    if (rc == CRISPY_OK) {
        rc = crispy_kmer_prepare_from_pre(ctx, raw, K);
        if (rc == CRISPY_E_UNSUPPORTED && st.kept > 0) {
            from_file = true;
            rc = prepare_from_file(ctx, clean, 0, K, &nk);
        }
    }
    const float kthr = crispy_default_threshold(nk, -1.0f, 0);
    if (rc == CRISPY_OK) rc = crispy_kmer_run(ctx, kthr, mode, 0, &kpairs);
    if (rc == CRISPY_OK) {
        KOut o{std::fopen((clean + ".kpair").c_str(), "wb")};
        if (!o.pair) rc = CRISPY_E_IO;
        else rc = crispy_kmer_stream(ctx, write_kmer, &o);
        if (o.pair && std::fclose(o.pair) != 0 && rc == CRISPY_OK) rc = CRISPY_E_IO;
    }
    if (rc == CRISPY_OK) std::printf("totalNumPairs: %llu\n", (unsigned long long)kpairs);

    // genDist on the survivors, still on the device
    if (rc == CRISPY_OK)
        rc = from_file ? prepare_from_file(ctx, clean, 1, K, &ng) : crispy_gen_prepare_from_pre(ctx, raw);
    const float gthr = crispy_default_threshold(ng, -1.0f, 1);
    Chunks ck{clean, {}, {}};
    if (rc == CRISPY_OK) rc = crispy_gen_run_from_kmer(ctx, band, gthr, mode, write_chunk, &ck, &total);
    if (rc != CRISPY_OK) {
        std::fprintf(stderr, "crispyRun: %s\n", crispy_last_error(ctx));
        crispy_ctx_destroy(ctx);
        crispy_raw_free(raw);
        return 255;
    }
    std::printf("%llu\n", (unsigned long long)total);

    // aveclust on the chunks, NUM_READS counted as `grep '>' | wc -l` does:
    // every header line, plus each line of a read that holds a '>'
    int64_t num_reads = st.kept;
    for (int32_t k = 0; k < st.kept; ++k) {
        const char* p = seq + off[index[k]];
        const char* e = p + len[index[k]];
        while (p < e) {
            const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(e - p)));
            const char* le = nl ? nl : e;
            if (std::memchr(p, '>', (size_t)(le - p))) ++num_reads;
            p = nl ? nl + 1 : e;
        }
    }
    std::vector<const uint32_t*> cp;
    std::vector<const float*> cd;
    std::vector<int64_t> cn;
    for (size_t c = 0; c < ck.pairs.size(); ++c) {
        cp.push_back(ck.pairs[c].data());
        cd.push_back(ck.dists[c].data());
        cn.push_back((int64_t)ck.dists[c].size());
    }
    crispy_clust_stats cs{};
    if (!cn.empty() && num_reads > 0) {
        rc = crispy_aveclust(cp.data(), cd.data(), cn.data(), (int)cn.size(), (int)num_reads, -1.0f,
                             clean.c_str(), nullptr, &cs);
        if (rc != CRISPY_OK) {
            std::fprintf(stderr, "crispyRun: %s\n", crispy_last_error(nullptr));
            crispy_ctx_destroy(ctx);
            crispy_raw_free(raw);
            return 255;
        }
        std::printf("aveclust: %lld merges, %d clusters, %d singletons\n", (long long)cs.merges, cs.roots,
                    cs.singletons);
    }
    if (argc > 4 && !cn.empty() && num_reads > 0) {
        // sparsecut on the _Merge file aveclust wrote (crispy.sh:29)
        std::vector<float> cutoffs;
        const std::string err = crispy_cli::read_cutoffs(argv[4], cutoffs, false);
        crispy_clust_stats ss{};
        if (!err.empty() || crispy_sparsecut(clean.c_str(), (int)num_reads, cutoffs.data(),
                                             (int)cutoffs.size(), &ss) != CRISPY_OK) {
            std::fprintf(stderr, "crispyRun: %s\n", err.empty() ? crispy_last_error(nullptr) : err.c_str());
            crispy_ctx_destroy(ctx);
            crispy_raw_free(raw);
            return 255;
        }
        std::printf("sparsecut: %d cutoffs\n%s", (int)cutoffs.size(), ss.report);
    }
    crispy_ctx_destroy(ctx);
    crispy_raw_free(raw);
    std::printf("Time taken: %.3f s\n", now() - t0);
    return 0;
}
