/*
 * oracle.h -- CPU restatement of CRiSPy's kmerDist and genDist semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the CUDA path
 * is compared against; nothing in the product (crispy_gb300/, include/) links
 * it, and the product fails loudly instead of falling back to it.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 *
 * Every function restates the reference's algorithm in plain C++ (no SIMD,
 * no tricks) and cites the reference file:line it follows.  Parity of this
 * restatement is pinned against the reference's own CPU code compiled from
 * source (oracle/build_ref.sh -> oracle/_ref/) on the sample FASTA and on
 * seeded synthetic sets (tests/golden/).
 */
#ifndef CRISPY_ORACLE_H
#define CRISPY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* FASTA parse.  flavour 0 = kmerDist (trailing trim set "ATGCatgc",
 * kmerMain.cpp:289-295), 1 = genDist (trim set "nNATGCatgc",
 * genMain.cpp:175-181).  Returns the number of reads (>= 0) or a negative
 * error: -1 cannot open, -2 not FASTA.  The reads are concatenated into an
 * internal buffer retrievable with oracle_fasta_get(); the handle is freed
 * by oracle_fasta_free(). */
typedef struct oracle_fasta oracle_fasta;
int oracle_fasta_read(const char* path, int flavour, oracle_fasta** out);
void oracle_fasta_get(const oracle_fasta* f, const char** seqbuf,
                      const int64_t** offsets, const int32_t** lengths,
                      int32_t* max_len);
void oracle_fasta_free(oracle_fasta* f);

/* Default cut thresholds: kmerMain.cpp:43-48 (num=2) and genMain.cpp:42-47
 * (num=1).  user_thr outside [0,1] selects the default. */
float oracle_default_threshold(int n, float user_thr, int num);

/* arrayDim = (int)(4 * 8^(floor(log10 n) - 1)) capped at 1536
 * (kmerMain.cpp:50-53). */
int oracle_array_dim(int n);

/* k-mer count between two reads by the reference's sorted merge
 * (kmerCPU.cpp:27-43 over tuples built by kmerMain.cpp:117-159). */
int oracle_kmer_matches(const char* a, int la, const char* b, int lb, int K);

/* All-pairs k-mer distance, threshold and compaction in the GPU path's
 * output order (stage order of kmerCUDA.cu:79-111, i-major then j inside a
 * stage, kmerMain.cpp:175-195).  Writes up to cap survivors; returns the
 * total survivor count (may exceed cap) or a negative error. */
int64_t oracle_kmer_all(const char* seqbuf, const int64_t* offsets,
                        const int32_t* lengths, int n, int K, float thr,
                        int array_dim, int nthreads, int32_t* out_pairs,
                        float* out_dists, int64_t cap);

/* Banded Needleman-Wunsch of genCPU.cpp:290-466 for one pair, with the
 * GPU path's 2-bit symbol comparison (genKernel.cu:437-447).  band <= 1
 * selects the unbanded semantics of genCPU.cpp:81-225.  Outputs the selected
 * score, mismatch+gap count (ML) and alignment length (AL); returns the
 * distance (float)ML/AL. */
float oracle_gen_pair(const char* r1, int l1, const char* r2, int l2, int band,
                      int32_t* score, int32_t* ml, int32_t* al);

/* The same over a pair list (OpenMP over pairs). */
void oracle_gen_all(const char* seqbuf, const int64_t* offsets,
                    const int32_t* lengths, int n, const int32_t* pairs,
                    int64_t npairs, int band, int nthreads, float* out_dist,
                    int32_t* out_score, int32_t* out_ml, int32_t* out_al);

/* Number of band cells of one pair (the GCUPS numerator). */
int64_t oracle_band_cells(int l1, int l2, int band);

/* Threshold filter, 589,824-pair load windows, chunk flush at >= 589,824
 * survivors and stable ascending sort by distance per chunk
 * (genCUDA.cu:150-254, :17-81).  pairs/dists are the per-input-pair arrays
 * in .kpair order.  Writes the concatenated chunk contents to out_pairs /
 * out_dists (capacity npairs) and the chunk sizes to chunk_sizes (capacity
 * max_chunks); returns the number of chunks. */
int oracle_gen_chunks(const int32_t* pairs, const float* dists,
                      int64_t npairs, float thr, uint32_t* out_pairs,
                      float* out_dists, int64_t* chunk_sizes, int max_chunks);

/* preprocess end to end (preprocess.cpp:686-726, oracle_pre.cpp): records
 * of in_path (fastq: -f q), the -s length filter (length_check, sd), the -p
 * primer check (primer = the primer sequence, NULL without -p; max_mm =
 * -m), the duplicate merge, and out_path / out_path.frq.  counts[5] gets
 * {records, length discards, primer discards, merges, kept}.  Returns 0,
 * -1 (cannot open input), -2 (not FASTA) or -3 (cannot write output). */
int oracle_preprocess(const char* in_path, const char* out_path, int fastq,
                      int length_check, double sd, const char* primer, int max_mm,
                      int64_t* counts);

/* aveclust's clustering (aveclust.cpp:663-1007, oracle_clust.cpp) over
 * genDist chunks (pairs[c]: uint32[2*counts[c]], dists[c]: float[counts[c]],
 * each ascending); writes the _Merge lines to merge_path.  end_level outside
 * [0,1] selects the default.  Returns 0, -1 (bad arguments) or -3 (cannot
 * write). */
int oracle_aveclust(const uint32_t* const* pairs, const float* const* dists,
                    const int64_t* counts, int nchunks, int num_reads, float end_level,
                    const char* merge_path, int64_t* merges_out);

/* Survivors of rows [row_lo, row_hi) against every later column, in (row,
 * col) order, with oracle_kmer_all's per-pair rule; returns the total (may
 * exceed cap) or a negative error. */
int64_t oracle_kmer_rows(const char* seqbuf, const int64_t* offsets, const int32_t* lengths,
                         int n, int K, float thr, int row_lo, int row_hi, int nthreads,
                         int32_t* out_pairs, float* out_dists, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
