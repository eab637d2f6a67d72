// internal.h -- host-side state shared by the translation units of
// libcrispy_gb300.so.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <new>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/crispy_gb300.h"

namespace crispy {

// Grow-only device allocation owned by a context.  need / epoch track the
// largest size requested during the context's current run (see
// crispy_ctx::run_need).
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    size_t need = 0;
    uint64_t epoch = 0;
    template <class T> T* as() const { return static_cast<T*>(ptr); }
};

// Grow-only pinned host allocation owned by a context.
struct HostBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    template <class T> T* as() const { return static_cast<T*>(ptr); }
};

// Allocator of page-locked host memory for per-read arrays that move
// between host and device every run (copies from or into pageable memory go
// through a staging buffer at a fraction of the link's rate).  Falls back to
// pageable memory when pinning fails; those blocks are recorded, so that a
// block is always freed by the call that matches its allocation.
void* pinned_or_pageable_alloc(size_t bytes);
void pinned_or_pageable_free(void* p);
template <class T>
struct PinnedAlloc {
    using value_type = T;
    PinnedAlloc() = default;
    template <class U> PinnedAlloc(const PinnedAlloc<U>&) {}
    T* allocate(size_t n) { return static_cast<T*>(pinned_or_pageable_alloc(n * sizeof(T))); }
    void deallocate(T* p, size_t) { pinned_or_pageable_free(p); }
    template <class U> bool operator==(const PinnedAlloc<U>&) const { return true; }
    template <class U> bool operator!=(const PinnedAlloc<U>&) const { return false; }
};
template <class T> using pinned_vector = std::vector<T, PinnedAlloc<T>>;

// Device-resident k-mer job: the reads of one kmerDist invocation.
struct KmerJob {
    bool ready = false;
    int n = 0, k = 0, max_len = 0, max_t = 0;
    int ngroups = 0;            // 32-read groups
    int64_t nent = 0;           // entries in the interleaved level-entry array
    pinned_vector<int32_t> h_t;   // tuples per read (L - K + 1)
    pinned_vector<int32_t> h_cntmax;   // largest k-mer multiplicity and high-level entries per read
    pinned_vector<int64_t> h_gstart;   // first entry of each group
    pinned_vector<int32_t> h_gent;     // entries per lane in each group (multiple of 16)
    pinned_vector<int64_t> h_tstart;   // tile stream: first entry of each group
    pinned_vector<int32_t> h_tgent;    // tile stream: steps per lane in each group
    int64_t ntent = 0;
    DevBuf seq, off, len, t, gstart, gent, ent, cntmax, hinfo, tstart, tgent, tent, bcnt;
    DevBuf tgentL, nsec;             // second-stream steps per group; per-read section counts
    // K <= 6: the split of every read's dense level entries into two
    // sections (a hash of the plane word below split / 256: section 0), 0:
    // one section; the tile kernel bounds each pair after section 0
    int split = 0;
    pinned_vector<int32_t> h_nsec;
    // K = 8 read order: per-read arrays above (t, cntmax, hinfo, entries)
    // are by position in it; perm maps position -> read ID, offp holds the
    // offsets by position, t0 the tuple counts by read ID
    DevBuf t0, offp, perm;
    pinned_vector<int32_t> h_perm;
    pinned_vector<int32_t> h_tpos;   // tuple counts by position
    // K = 8: H key per position and the run of equal keys holding it
    pinned_vector<uint32_t> h_hinfo;
    std::vector<int32_t> h_run_lo, h_run_hi;
    bool hkeys_ordered = false;
    // last run's survivors, in stage order: on the device, or (spilled) in
    // pinned host memory when they outgrow the device share
    int64_t nsurv = 0;
    bool have_dists = false;
    bool spilled = false;
    HostBuf h_spill_pairs, h_spill_dists;
    DevBuf keys, keys_alt, vals, vals_alt, pairs, dists, counter, mmin, smin, work;
    DevBuf sq;                       // K = 8 same-key pass: queued H sums per block and lane slot
    DevBuf sort_tmp;
};

// Device-resident genDist job: 2-bit packed reads.
struct GenJob {
    bool ready = false;
    int n = 0, max_len = 0;
    pinned_vector<int32_t> h_len;
    pinned_vector<int64_t> h_woff;     // first packed word of each read
    pinned_vector<uint32_t> h_tiles;   // survivors per compaction tile (chunk boundaries)
    DevBuf seq, off, len, woff, packed;
    DevBuf pairs, dist, score, ml, al, flags, scan, blocksum, surv_idx, keys, keys_alt,
        vals, vals_alt, out_pairs, out_dists, order, buckets, queue, err, tune_sample, tune_queue,
        cstats, ckeys, ckeys_alt, cvals, cvals_alt, acc_pairs, acc_dists;
    DevBuf dirs;   // the 16-bit DP's cell tags (two halves: one per concurrent bin launch)
    HostBuf h_pairs, h_dists;
};

// Device buffers of one preprocess call (raw records, their 16-byte
// aligned copy, filter flags, sort and merge lists).
struct PreJob {
    bool ready = false;   // out_idx holds the last call's kept reads
    int64_t kept = 0;
    int32_t n = 0;                 // records of the last call
    std::vector<int32_t> h_idx;    // kept record indices, _Clean order
    DevBuf seq, off, len, freq, woff, pad, alive, idx, idx_alt, flags, pos, tiles, out_idx,
        out_freq, counters, primer, tmp, stage_len, stage_off;
};

// An instantiated CUDA graph of one launch sequence and the number of
// kernels it holds.
struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
};

struct StreamEvents {
    std::vector<cudaEvent_t> start, stop;
    size_t used = 0;
};

}  // namespace crispy

struct crispy_ctx {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t side[8] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[2] = {};   // fork / join of side-stream launches
    bool timing = false;
    std::string err;
    crispy_stats stats{};
    crispy::KmerJob kmer;
    crispy::GenJob gen;
    crispy::PreJob pre;
    crispy::StreamEvents ev_kmer, ev_gen;
    std::map<std::string, crispy::GraphEntry> graphs;   // captured launch sequences
    bool use_graphs = true;
    // the batched k-mer run may tune its split per read set (off for the
    // server's contexts: every job is a new read set, and tuning one costs
    // more than it saves)
    bool kmer_tune = true;
    size_t mem_cap = 0;      // 0 = unlimited
    size_t mem_in_use = 0;   // bytes held by DevBuf allocations
    // device bytes the current run has asked for (each buffer's largest
    // request since the run began, summed): the run's own peak, whatever
    // larger buffers earlier runs left behind.  A new run bumps run_epoch.
    uint64_t run_epoch = 1;
    size_t run_need = 0;
    cudaEvent_t t_begin = nullptr, t_end = nullptr;
};

namespace crispy {

int fail(crispy_ctx* ctx, int code, const char* fmt, ...);
int cuda_fail(crispy_ctx* ctx, cudaError_t e, const char* what, const char* file, int line);
int ensure(crispy_ctx* ctx, DevBuf& b, size_t bytes);
int ensure_host(crispy_ctx* ctx, HostBuf& b, size_t bytes);
void release(DevBuf& b);
void release(crispy_ctx* ctx, DevBuf& b);
void release_host(HostBuf& b);

// Event pair around a launch, when timing is enabled.
cudaEvent_t ev_begin(crispy_ctx* ctx, StreamEvents& ev, cudaStream_t s);
void ev_end(crispy_ctx* ctx, StreamEvents& ev, cudaStream_t s);
double ev_sum_ms(StreamEvents& ev);

// kernel counter (every launch of this library increments it)
void count_launch(crispy_ctx* ctx, int n = 1);

// Run a launch sequence through a CUDA graph: the first call with a key
// captures `enqueue` (which must only enqueue work on s: no host syncs, no
// allocation) and instantiates it; later calls with the same key replay it.
// The key must name every size and device address the sequence bakes in.
int graph_run(crispy_ctx* ctx, cudaStream_t s, const std::string& key,
              const std::function<int()>& enqueue);
void graph_clear(crispy_ctx* ctx);

// The reads the last crispy_preprocess kept, in _Clean order, as the
// kmerDist (flavour 0) or genDist (flavour 1) FASTA parser reads them back
// from the _Clean file (pre.cu).  On success *d_bytes is the device buffer
// holding them, d_off their byte offsets there (device) and h_len their
// lengths (host).  CRISPY_E_UNSUPPORTED when a kept read holds a
// whitespace byte or is longer than 4,094 bytes: the file's lines then
// split differently and only the file itself gives the stage's reads.
int pre_stage_reads(crispy_ctx* ctx, const crispy_raw* raw, int flavour, const uint8_t** d_bytes,
                    size_t* bytes, const int64_t** d_off, std::vector<int32_t>& h_len);
// Read buffer of the FASTA scans: an anonymous mapping with transparent
// huge pages (pre_io.cpp).
struct FastaBuffer {
    char* p = nullptr;
    size_t n = 0;
    FastaBuffer() = default;
    FastaBuffer(const FastaBuffer&) = delete;
    FastaBuffer& operator=(const FastaBuffer&) = delete;
    ~FastaBuffer();
    bool alloc(size_t bytes);
};

// The reads of a FASTA file as kmerDist (flavour 0, kmerMain.cpp:298-397)
// or genDist (flavour 1, genMain.cpp:184-277) parse it, scanned in parallel
// chunks (pre_io.cpp): each read at buf.p + offsets[i], lengths[i] bytes.
int scan_stage_fasta(const char* path, int flavour, FastaBuffer& buf, std::vector<int64_t>& offsets,
                     std::vector<int32_t>& lengths);

// Records of a raw handle, and the length of the "> label" line
// writeToFile gives record i, newline excluded (pre_io.cpp).
int32_t raw_records(const crispy_raw* r);
int64_t raw_header_line(const crispy_raw* r, int32_t i);

// One job of a cohort run (server cross-job batching): its reads sit at
// positions [base, base + n) of the cohort's read set; thr is its k-mer
// (kmer_run_cohort) or genetic (gen_run_cohort) cut threshold.
struct CohortJob {
    int base = 0, n = 0;
    float thr = 0.0f;
    crispy_sink sink = nullptr;   // genDist chunks of this job (gen_run_cohort)
    void* user = nullptr;
};
int kmer_run_cohort(crispy_ctx* ctx, const std::vector<CohortJob>& jobs, std::vector<int64_t>& counts);
// The k-mer bound pass's tuned splits as JSON objects, each preceded by ", ".
std::string kmer_tune_json();
int gen_run_cohort(crispy_ctx* ctx, const std::vector<CohortJob>& jobs, const std::vector<int64_t>& counts,
                   int band, std::vector<int64_t>& gen_counts);

// radix sort / scan helpers (sort.cu)
size_t sort_tmp_bytes(int64_t n);   // scratch a sort of n items needs
int sort_u64_payload(crispy_ctx* ctx, cudaStream_t s, uint64_t* keys, uint64_t* keys_alt,
                     uint32_t* vals, uint32_t* vals_alt, int64_t n, int key_bits,
                     bool with_vals, uint64_t** sorted_keys, uint32_t** sorted_vals,
                     DevBuf& tmp);
int sort_u32_payload(crispy_ctx* ctx, cudaStream_t s, uint32_t* keys, uint32_t* keys_alt,
                     uint32_t* vals, uint32_t* vals_alt, int64_t n, int key_bits,
                     uint32_t** sorted_keys, uint32_t** sorted_vals, DevBuf& tmp);
// Stable compaction of indices with flag != 0; per-tile counts returned on
// the device in tile_counts (tile = kScanTile items).  With total != nullptr
// the call waits for the count and returns it; with nullptr it returns at
// once (the caller reads tile_counts).
constexpr int kScanTile = 4608;   // divides the 589,824-pair window (128 tiles)
int compact_flags(crispy_ctx* ctx, cudaStream_t s, const uint8_t* flags, int64_t n,
                  uint32_t* out_idx, uint32_t* tile_counts, DevBuf& tmp, int64_t* total);

}  // namespace crispy

inline std::string key_of(std::initializer_list<uint64_t> parts) {
    std::string k;
    for (uint64_t v : parts) {
        k += std::to_string(v);
        k += ',';
    }
    return k;
}

#define CRISPY_CK(ctx, call)                                                        \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) return crispy::cuda_fail(ctx, e_, #call, __FILE__, __LINE__); \
    } while (0)

#define CRISPY_TRY(call)                 \
    do {                                 \
        int rc_ = (call);                \
        if (rc_ != CRISPY_OK) return rc_; \
    } while (0)
