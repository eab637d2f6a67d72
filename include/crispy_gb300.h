/*
 * crispy_gb300.h -- C ABI of libcrispy_gb300.so, the GB300 (sm_103a) engine
 * behind CRiSPy's two pairwise-distance stages.
 *
 * The reference has no library API: its boundary is the bin/kmerDist and
 * bin/genDist command lines plus their binary files, and internally the C++
 * seams computeKmerDist_CUDA (src/kmerDist/kmerMain.h:73) and
 * computeGenDist_CUDA (src/genDist/genMain.h:77).  Each entry point below
 * replaces one part of those seams; the citation on each says which.  The
 * drop-in executables built from crispy_gb300/csrc/cli_*.cpp call only this
 * header.
 *
 * Conventions
 *   - Every function returns an int status: CRISPY_OK (0) or a CRISPY_E_*
 *     code.  Nothing calls exit(); crispy_last_error() describes the last
 *     failure on a context (or globally when ctx is NULL).
 *   - Plain pointers and sizes only.  Host buffers belong to the caller and
 *     are never retained past the call.  Device memory belongs to the
 *     context and is released by crispy_ctx_destroy().
 *   - One context per host thread.  A context drives one GPU (device index
 *     given at creation) on one CUDA stream.
 *   - Results are bit-exact to the reference: integer k-mer counts, DP
 *     scores, mismatch/alignment-length counts, FP32 distances evaluated in
 *     the reference's own expression order, and the reference's output
 *     order (stage order for .kpair, stable distance order per chunk for
 *     .npair_N/.ndist_N).
 */
#ifndef CRISPY_GB300_H
#define CRISPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference exits with -1 on every one of these,
 *      kmerKernel.h:17-26, genMain.cpp:117-126) ---- */
#define CRISPY_OK          0
#define CRISPY_E_INPUT     1   /* bad argument, malformed file, read index out of range */
#define CRISPY_E_OOM       2   /* device or pinned-host allocation failed */
#define CRISPY_E_DEVICE    3   /* CUDA error, no device, or missing sm_103a image */
#define CRISPY_E_TIMEOUT   4   /* a bounded device-side wait ran out */
#define CRISPY_E_STATE     5   /* call out of order (e.g. run before prepare) */
#define CRISPY_E_IO        6   /* file could not be opened, read or written */
#define CRISPY_E_UNSUPPORTED 7 /* limits of the reference: n > 1,048,576, length > 2048, K outside 1..8 */

/* ---- limits shared with the reference (kmerMain.h:28-30, genMain.h:29-30) ---- */
#define CRISPY_MAX_READ_LEN   2048
#define CRISPY_MAX_NUM_READS  (1024 * 1024)
#define CRISPY_GEN_WINDOW     589824   /* genMain.h:24-27: pairs per load window and chunk flush size */

/* ---- run modes (all three give identical bits) ----
 * PLAIN    the plain from-scratch kernels, one thread per pair: kmerDist with
 *          one block per row read holding its dense count table, genDist with
 *          band rows in global scratch; launched per reference stage (kmer)
 *          and per 589,824-pair load window (gen), like the reference.
 * STAGED   the GB300 kernels (bit-sliced k-mer tiles, warp-cooperative
 *          anti-diagonal DP) launched the plain way: per stage / per window,
 *          one fixed band-tile shape per window.
 * BATCHED  the GB300 kernels as persistent work-queue kernels: row-group
 *          queue for kmerDist, pairs bucketed by band width and length with
 *          autotuned lanes-per-pair and band-tile shape for genDist, launch
 *          sequences replayed as CUDA graphs. */
#define CRISPY_MODE_PLAIN    0
#define CRISPY_MODE_BATCHED  1
#define CRISPY_MODE_STAGED   2

typedef struct crispy_ctx crispy_ctx;

/* Receives output in the reference's order, in consecutive batches.
 * For kmer: pairs = int32[2*count] (row, col), dists = float[count].
 * For gen:  called once per chunk file (chunk_id = the _<f> suffix) with
 *           pairs = uint32[2*count], dists = float[count].
 * Return 0 to continue, non-zero to abort the run (status CRISPY_E_IO). */
typedef int (*crispy_sink)(void* user, int chunk_id, const void* pairs,
                           const float* dists, int64_t count);

/* Context lifetime.  Replaces the implicit device-0 setup and the
 * checkCudaErrors/exit(-1) error model of kmerKernel.h:17-26. */
int crispy_ctx_create(int device, crispy_ctx** out);
int crispy_ctx_destroy(crispy_ctx* ctx);
/* Run on a caller-owned cudaStream_t (pass NULL for the context's own). */
int crispy_ctx_set_stream(crispy_ctx* ctx, void* cuda_stream);
const char* crispy_last_error(const crispy_ctx* ctx);
const char* crispy_version(void);

/* ---- host helpers (no device work) ---- */

/* FASTA parse of readFile (kmerMain.cpp:298-397 when flavour = 0,
 * genMain.cpp:184-277 when flavour = 1): reads concatenated into one buffer.
 * The handle owns the memory; crispy_reads_free releases it. */
typedef struct crispy_reads crispy_reads;
int crispy_reads_load_fasta(const char* path, int flavour, crispy_reads** out);
int crispy_reads_view(const crispy_reads* r, const char** seqbuf,
                      const int64_t** offsets, const int32_t** lengths,
                      int32_t* n, int32_t* max_len);
void crispy_reads_free(crispy_reads* r);

/* Default cut threshold: kmerMain.cpp:43-48 (stage = 0, 2/log n) and
 * genMain.cpp:42-47 (stage = 1, 1/log n); user_thr in [0,1] wins. */
float crispy_default_threshold(int n, float user_thr, int stage);
/* Stage tile size arrayDim of kmerMain.cpp:50-53 (0 for n < 10). */
int crispy_array_dim(int n);

/* ---- kmerDist (replaces computeKmerDist_CUDA, kmerCUDA.cu:14-126) ---- */

/* Upload reads and build the per-read k-mer structures on the device
 * (replaces formTuples/sortTuples, kmerMain.cpp:117-159, and the texture
 * upload of kmerCUDA.cu:37-71).  seqbuf holds the reads back to back. */
int crispy_kmer_prepare(crispy_ctx* ctx, const char* seqbuf,
                        const int64_t* offsets, const int32_t* lengths,
                        int n, int k);

/* Re-run the device-side K-mer structure build from the reads uploaded by
 * the last crispy_kmer_prepare (no host transfer).  Part of formTuples in
 * the reference (kmerMain.cpp:117-159). */
int crispy_kmer_rebuild(crispy_ctx* ctx);

/* All-pairs k-mer distance with the cut threshold and sparse compaction
 * fused into the kernel (kmerKernel.cu:19-51 + writeToFile,
 * kmerMain.cpp:161-203).  Survivors stay on the device, already in the
 * reference's stage order; *npairs gets their count.  dists selects whether
 * distances are kept (the -d flag). */
int crispy_kmer_run(crispy_ctx* ctx, float thr, int mode, int dists,
                    int64_t* npairs);

/* Copy the survivors of the last crispy_kmer_run to host memory (pairs:
 * int32[2*cap], dists: float[cap] or NULL), or stream them to a sink in
 * batches.  *count receives the number copied. */
int crispy_kmer_fetch(crispy_ctx* ctx, int32_t* pairs, float* dists,
                      int64_t cap, int64_t* count);
int crispy_kmer_stream(crispy_ctx* ctx, crispy_sink sink, void* user);

/* ---- genDist (replaces computeGenDist_CUDA, genCUDA.cu:83-270) ---- */

/* Upload reads (genDist flavour: the same buffer layout) and 2-bit pack them
 * on the device (replaces convertToBinary, genMain.cpp:280-321, and the
 * texture upload of genCUDA.cu:130-142). */
int crispy_gen_prepare(crispy_ctx* ctx, const char* seqbuf,
                       const int64_t* offsets, const int32_t* lengths, int n);

/* The same from the reads the last crispy_kmer_prepare left on the device:
 * no second host upload when one process runs both stages (the reference
 * runs them as two programs that each parse the FASTA, genMain.cpp:184-277).
 * Fails with CRISPY_E_STATE without a prepared k-mer job and CRISPY_E_INPUT
 * for an empty read, as crispy_gen_prepare does. */
int crispy_gen_prepare_from_kmer(crispy_ctx* ctx);

/* Banded NW distance for every pair, threshold filter, 589,824-pair load
 * windows, chunk flush and stable per-chunk sort by distance
 * (genKernel.cu:707-780, genCUDA.cu:150-254, :17-81).  pairs is
 * int32[2*npairs] in .kpair order on the host; band <= 0 means 2
 * (genMain.cpp:356-364) and band == 1 is the unbanded alignment.  Each
 * chunk goes to the sink in file order; *nsurvivors gets the total. */
int crispy_gen_run(crispy_ctx* ctx, const int32_t* pairs, int64_t npairs,
                   int band, float thr, int mode, crispy_sink sink,
                   void* user, int64_t* nsurvivors);

/* The same, consuming the survivors of the last crispy_kmer_run directly
 * from device memory (no .kpair round trip).  Requires crispy_gen_prepare
 * on the same reads. */
int crispy_gen_run_from_kmer(crispy_ctx* ctx, int band, float thr, int mode,
                             crispy_sink sink, void* user,
                             int64_t* nsurvivors);

/* Per-pair alignment results without threshold or chunking (for parity
 * checks): dist[i], and when non-NULL score[i] (selected last-row/column
 * maximum), ml[i] (mismatches + gap columns) and al[i] (alignment length),
 * exactly the quantities of genKernel.cu:765-768. */
int crispy_gen_align(crispy_ctx* ctx, const int32_t* pairs, int64_t npairs,
                     int band, int mode, float* dist, int32_t* score,
                     int32_t* ml, int32_t* al);

/* Banded NW per pair (as crispy_gen_align) for callers that cannot allocate
 * device memory: an application that hands all device memory to its own
 * pool at start-up and forbids allocation later, or a runtime whose memory
 * accounting must not see foreign allocations.  No counterpart in the
 * reference.  The caller passes device buffers for everything: the reads as
 * ASCII bytes back to back (d_seq, d_offsets, d_lengths; n reads, none longer
 * than max_len <= 2048), the pairs (int32[2*npairs]) and the outputs
 * (d_dist required; d_score, d_ml, d_al may be NULL), and a cudaStream_t (or
 * NULL).  The DP rows live in a fixed 8 MiB array inside the library that
 * every GPU loading it holds until exit; nothing is allocated.  All calls
 * share that array: calls that overlap on the GPU race and must be
 * serialised by the caller.  Every call looks up the array's address in
 * the current device's context (a lookup, not an allocation).  The call is
 * synchronous: it waits for its kernel, which reports bad inputs, so it
 * cannot be made inside a stream capture.  Returns CRISPY_E_UNSUPPORTED
 * when max_len exceeds 2048 or the band needs more scratch than the array
 * holds, CRISPY_E_INPUT when a pair index is outside [0, n) or a read of a
 * pair is longer than max_len; such a pair gets dist NaN and score, ml and
 * al -1, and every other pair its result. */
int crispy_gen_align_noalloc(const char* d_seq, const int64_t* d_offsets,
                             const int32_t* d_lengths, int n, int max_len,
                             const int32_t* d_pairs, int64_t npairs, int band,
                             float* d_dist, int32_t* d_score, int32_t* d_ml,
                             int32_t* d_al, void* stream);

/* ---- preprocess (replaces bin/preprocess, src/preprocess/preprocess.cpp,
 *      the step crispy.sh:18 runs before kmerDist) ---- */

/* Records of a raw FASTA (fastq = 0, -f a) or FASTQ (fastq = 1, -f q) file
 * as readFile (preprocess.cpp:74-242) collects them, in file order: the
 * sequence (pieces of 4096-byte fgets reads, trailing whitespace and, for
 * FASTA, trailing characters outside "nNATGCatgc" trimmed per piece and per
 * read), the label (header line without any whitespace) and the frequency
 * (1, or 0 for a FASTQ record whose sequence line is empty).  `records` is
 * readIndex, the count the reference prints as "Total numReads" (it also
 * counts FASTA headers without a sequence). */
typedef struct crispy_raw crispy_raw;
int crispy_raw_load(const char* path, int fastq, crispy_raw** out);
int crispy_raw_view(const crispy_raw* r, const char** seqbuf, const int64_t** offsets,
                    const int32_t** lengths, const uint8_t** freq, int32_t* n,
                    int32_t* records);
int crispy_raw_label(const crispy_raw* r, int32_t i, const char** label, int32_t* len);
void crispy_raw_free(crispy_raw* r);

/* Options of preprocess's command line (getCommandOptions,
 * preprocess.cpp:613-684). */
typedef struct crispy_pre_opts {
    int length_check;      /* -s given: processReadLength (preprocess.cpp:322-392) */
    double sd_allowed;     /* -s value (default 1.0) */
    const char* primer;    /* -p: the primer (first line of the primer file, trailing
                              whitespace removed); NULL = no primer check */
    int max_mismatches;    /* -m (default 2): processPrimer (preprocess.cpp:530-560) */
} crispy_pre_opts;

typedef struct crispy_pre_stats {
    int32_t length_discards;   /* processReadLength's return */
    int32_t primer_discards;   /* processPrimer's return */
    int32_t merges;            /* mergeReads's return */
    int32_t kept;              /* reads written to the _Clean file */
    int32_t length_reads;      /* reads the length statistics cover (0: none) */
    int32_t min_len0, max_len0;   /* length range before the cut (printed first) */
    int32_t min_len, max_len;     /* the cut: lengths outside [min_len, max_len] go */
    double ave_len, sd;
} crispy_pre_stats;

/* The filters and the duplicate merge of preprocess on the device: length
 * cut and N/n check, primer check by Smith-Waterman (SWLocalAlignment,
 * preprocess.cpp:394-527), then mergeReads (preprocess.cpp:244-280): reads
 * sorted by (length, strcmp), stable, and each run of equal sequences
 * merged into its last read with the run's summed frequency.  Inputs are
 * the n records of a raw file (any buffer layout; freq 0 = not a read).
 * Writes the kept reads in _Clean order: out_index[k] = record index,
 * out_freq[k] = merged frequency (capacity n each). */
int crispy_preprocess(crispy_ctx* ctx, const char* seqbuf, const int64_t* offsets,
                      const int32_t* lengths, const uint8_t* freq, int32_t n,
                      const crispy_pre_opts* opts, int32_t* out_index, int32_t* out_freq,
                      crispy_pre_stats* stats);

/* writeToFile (preprocess.cpp:562-601): out_path gets "> <label>\n<seq>\n"
 * per kept read (FASTA labels lose their first character, the '>'), and
 * out_path.frq "<label> <freq>\n". */
int crispy_pre_write(const crispy_raw* r, const int32_t* index, const int32_t* freq,
                     int32_t kept, const char* out_path, int fastq);

/* The reads the last crispy_preprocess on this context kept, still on the
 * device, as the next two stages would parse them back from the _Clean file
 * (kmerDist: kmerMain.cpp:298-397, genDist: genMain.cpp:184-277): no file
 * round trip and no second upload, the hand-over crispy.sh:18-20 makes
 * through the file.  `raw` is the handle whose records went into that call.
 * CRISPY_E_UNSUPPORTED when a kept read holds a whitespace byte, a read is
 * longer than 4,094 bytes or a header line longer than 4,095: the file's
 * lines then split into several fgets pieces, and only parsing the written
 * _Clean file (crispy_reads_load_fasta) gives the stages' reads.
 * Otherwise equivalent to crispy_kmer_prepare / crispy_gen_prepare on the
 * parsed _Clean file. */
int crispy_kmer_prepare_from_pre(crispy_ctx* ctx, const crispy_raw* raw, int k);
int crispy_gen_prepare_from_pre(crispy_ctx* ctx, const crispy_raw* raw);

/* ---- aveclust (replaces bin/aveclust, src/aveclust/aveclust.cpp, the step
 *      crispy.sh:24 runs after genDist) ---- */
typedef struct crispy_clust_stats {
    int64_t pairs_read;   /* edges taken from the chunks */
    int64_t merges;       /* lines of the _Merge file */
    int32_t roots;        /* trees of two or more reads */
    int32_t singletons;   /* reads never merged */
    float end_level;      /* the final endLevel (lambda once the edge cap was hit) */
    char report[2048];    /* printClusters' "Dist: ... numOTUs ..." lines */
    /* aveclust only: host time (ms) in its phases -- taking edges from the
     * chunks and absorbing them into link maps, the per-round minimum
     * updates, the merges, cluster levels and file output */
    double ms_edges, ms_update, ms_merges, ms_output;
} crispy_clust_stats;

/* Sparse average-linkage clustering (aveclust's main loop,
 * aveclust.cpp:663-1007) over genDist's chunks: chunk c holds counts[c]
 * pairs (uint32 read indices, pairs[c][2k], pairs[c][2k+1]) and distances
 * (dists[c][k]) ascending, as <in>.npair_c / <in>.ndist_c.  end_level
 * outside [0, 1] selects the reference's default (1/log2 n above 500
 * reads, else 1/log10 n).  Writes <out_base>_Merge (byte-identical to the
 * reference), <out_base>.Cluster and <out_base>.Cluster_List (the same
 * clusters per level; the reference orders them by pointer hash, this
 * function by root ID), and with edge_out the -o files edge_out and
 * edge_out_Index1.  Host code: the clustering is sequential (each merge
 * decides the next); it runs in O(edges log n) where the reference scans
 * all nodes per merge. */
int crispy_aveclust(const uint32_t* const* pairs, const float* const* dists,
                    const int64_t* counts, int nchunks, int num_reads, float end_level,
                    const char* out_base, const char* edge_out, crispy_clust_stats* stats);

/* ---- sparsecut (replaces bin/sparsecut, src/sparsecut/sparsecut.cpp, the
 *      step crispy.sh:29 runs with the changepoint's cutoff file) ---- */
/* Reads the dendrogram <in_base>_Merge (as aveclust writes it: one
 * "idX idY dist" line per merge, 1-based node IDs) and writes
 * <in_base>.Cluster and <in_base>.Cluster_List with the clusters a cut at
 * each of the ncutoffs distances leaves (sparsecut.cpp:317-410; EPSILON
 * 1e-5).  Clusters are those of the reference; it orders them by pointer
 * hash, this function by root ID.  stats: merges read, roots, singletons,
 * and the "Dist: ... numOTUs ..." report lines.  A merge line that does not
 * join two current clusters is CRISPY_E_INPUT. */
int crispy_sparsecut(const char* in_base, int num_reads, const float* cutoffs, int ncutoffs,
                     crispy_clust_stats* stats);

/* ---- timing of the last run (CUDA events on the context's stream) ---- */
typedef struct crispy_stats {
    double kmer_kernel_ms;     /* summed duration of the k-mer tile kernel launches */
    int64_t kmer_launches;
    double gen_kernel_ms;      /* summed duration of the DP kernel launches */
    int64_t gen_launches;
    double total_ms;           /* whole call, device side */
    int64_t kmer_pairs;        /* all-pairs count n(n-1)/2 of the last kmer run */
    int64_t kmer_survivors;
    int64_t gen_pairs;         /* pairs aligned by the last gen run */
    int64_t gen_cells;         /* band cells of those pairs */
    int64_t gen_survivors;
    int64_t kernels_launched;  /* every kernel this library launched in the last run */
    int64_t graph_launches;    /* CUDA graph replays among them (batched form) */
    int64_t kmer_spilled;      /* 1 when the last kmer run's survivors outgrew the device
                                  share and were gathered in pinned host memory */
    /* bound pass of the batched 128-row tile kernel (K <= 6): level entries
     * gathered by bound passes (section 0) and by full passes, the (row
     * group, column) items counted in full and the full-pass rounds */
    int64_t kmer_bound_entries;
    int64_t kmer_full_entries;
    int64_t kmer_full_columns;
    int64_t kmer_rounds;
} crispy_stats;
int crispy_get_stats(const crispy_ctx* ctx, crispy_stats* out);
/* Enable per-launch event timing (adds events around the hot kernels). */
int crispy_set_timing(crispy_ctx* ctx, int enable);

/* The autotuner's choices so far, as a JSON array: one object per tuned
 * genDist bin (stage "gen": band, band slots, lanes per pair, slots per
 * lane, pairs per block, sample size, best and untuned times) and one per
 * read set whose k-mer bound-pass split was tuned (stage "kmer": reads, K,
 * split in 1/256, sampled row groups, best and default times).  Set
 * CRISPY_AUTOTUNE=0 in the environment to disable tuning.  No reference
 * counterpart. */
int crispy_tune_report(char* buf, size_t len);

/* Measured integer-pipe throughput of this GPU in Gop/s (32-bit add/xor
 * lane operations): the roofline denominator of both hot kernels, which
 * are integer-bound.  No reference counterpart (measurement utility). */
int crispy_probe_int32(crispy_ctx* ctx, double* gops);

/* Measured shared-memory gather throughput of this GPU in L1 wavefronts per
 * second (conflict-free 128-bit loads, one wavefront = one quarter-warp's 128
 * bytes): the roofline denominator of the k-mer tile kernels, whose bound is
 * the L1 data pipe.  No reference counterpart (measurement utility). */
int crispy_probe_lds128(crispy_ctx* ctx, double* wavefronts_per_s);

/* ---- memory cap of one context (device bytes); 0 = unlimited.  An
 *      allocation that would exceed it fails with CRISPY_E_OOM, exactly as
 *      an exhausted device would.  The server gives every slot a share of
 *      its HBM budget this way. ---- */
int crispy_ctx_set_mem_cap(crispy_ctx* ctx, size_t bytes);
int crispy_ctx_mem_in_use(const crispy_ctx* ctx, size_t* bytes);
/* Release every device buffer the context holds (its jobs stay valid only
 * until the next prepare). */
int crispy_ctx_trim(crispy_ctx* ctx);

/* ---- serving: continuous batching of whole clustering jobs ----
 *
 * No counterpart in the reference (each stage there is one process per data
 * set, crispy.sh:19-29).  A server owns `slots` contexts on one GPU, each
 * with its own stream.  Jobs (a read set plus k, band and thresholds) queue
 * in arrival order; a slot that frees up admits the next job whose memory
 * estimate fits the HBM budget left, so jobs arriving while others run are
 * admitted as slots and memory free up and their kernels overlap on the
 * device.  Each job runs kmerDist -> genDist with every intermediate
 * resident in HBM, and its result is the same chunk list a lone run gives.
 * Small jobs of the same K and band that are queued together run as one
 * cohort: one persistent k-mer launch over all their row groups (each over
 * its own columns, with its own threshold) and one set of genDist launches
 * over all their survivors, then per-job thresholds, chunks and sorts
 * (CRISPY_SERVE_COHORT=0 runs every job alone).
 * Submit, wait, result and cancel are thread-safe. */
#define CRISPY_JOB_QUEUED    0
#define CRISPY_JOB_RUNNING   1
#define CRISPY_JOB_DONE      2
#define CRISPY_JOB_FAILED    3
#define CRISPY_JOB_CANCELLED 4

typedef struct crispy_server crispy_server;
int crispy_server_create(int device, size_t hbm_budget_bytes, int slots,
                         crispy_server** out);
int crispy_server_destroy(crispy_server* srv);
/* Copies the reads; thresholds outside [0,1] select the stage defaults. */
int crispy_server_submit(crispy_server* srv, const char* seqbuf,
                         const int64_t* offsets, const int32_t* lengths,
                         int n, int k, int band, float kmer_thr, float gen_thr,
                         uint64_t* job_id);
/* Waits up to timeout_ms (< 0: forever) for the job to finish; *state gets
 * its CRISPY_JOB_* state.  CRISPY_E_TIMEOUT when it is still pending. */
int crispy_server_wait(crispy_server* srv, uint64_t job_id, int timeout_ms,
                       int* state);
/* Delivers a finished job's genDist chunks to the sink (chunk order), its
 * k-mer survivor and genetic survivor counts, then forgets the job.  A
 * failed job returns its error status. */
int crispy_server_result(crispy_server* srv, uint64_t job_id, crispy_sink sink,
                         void* user, int64_t* kmer_pairs, int64_t* gen_pairs);
/* Cancels a queued job (a running one finishes). */
int crispy_server_cancel(crispy_server* srv, uint64_t job_id);
/* Memory of the run that served a finished job (before its result is
 * taken): *reserved = device bytes the admission reserved for all the jobs
 * of that run (the job alone, or its cohort), *needed = device bytes the
 * run asked for at its peak, *cohort_size = jobs that shared the run. */
int crispy_server_job_memory(crispy_server* srv, uint64_t job_id, size_t* reserved,
                             size_t* needed, int* cohort_size);
/* The device bytes the server's admission reserves for a job of n reads of
 * these lengths at K = k (no device work). */
int crispy_server_job_bytes(const int32_t* lengths, int n, int k, size_t* bytes);
/* Submit-to-finish latency percentiles (ms) over finished jobs, finished
 * job count and pairs processed (sum of n(n-1)/2). */
int crispy_server_stats(crispy_server* srv, double* p50_ms, double* p99_ms,
                        int64_t* jobs_done, int64_t* pairs_done);
/* Forget the latency samples and pair count gathered so far. */
int crispy_server_stats_reset(crispy_server* srv);
const char* crispy_server_last_error(const crispy_server* srv);

#ifdef __cplusplus
}
#endif
#endif /* CRISPY_GB300_H */
