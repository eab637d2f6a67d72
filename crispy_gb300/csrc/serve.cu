// serve.cu -- continuous batching of clustering jobs on one GPU.
//
// The reference runs one process per data set and stage (crispy.sh:19-29);
// there is no server to mirror.  This one keeps `slots` contexts, each with
// its own stream and grow-only device buffers, and one worker thread per
// slot.  Jobs queue in arrival order.  A worker that is free takes the
// oldest queued job whose memory estimate fits the budget still unclaimed,
// so a large job at the head does not stall small ones behind it; a job
// larger than the whole budget fails at submit with CRISPY_E_OOM.
//
// Small jobs share the kernels: when the queue holds a backlog (at least as
// many jobs as slots), with the oldest fitting job the worker takes every
// other queued job of the same K and band that is small enough and fits the
// budget (a cohort, up to kCohortReads reads in all).  The
// cohort's reads go up as one read set, each job at a 128-aligned base; one
// persistent k-mer tile launch takes all their row groups from one queue,
// each over its own job's columns with its own threshold, and one set of
// genDist bin launches aligns all their survivors; each job is then cut,
// chunked and sorted on its own (kmer_run_cohort, gen_run_cohort).  A job
// alone runs prepare -> kmer_run -> gen_prepare -> gen_run_from_kmer.
// Everything stays in HBM until the chunks come back; jobs on different
// slots overlap on the device.  A job's result is the same alone, in a
// cohort and in a mix: per-pair work never depends on other jobs, and its
// thresholds, stage order and chunks are its own.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "gen_args.h"
#include "internal.h"

namespace {

using clock_type = std::chrono::steady_clock;

// Cohort limits: members of at most kCohortJobReads reads (larger jobs run
// alone), at most kCohortReads reads and kCohortJobs jobs per cohort.
constexpr int kCohortJobReads = 16384;
constexpr int kCohortReads = 32768;
constexpr int kCohortJobs = 64;

bool cohorts_enabled() {
    const char* e = std::getenv("CRISPY_SERVE_COHORT");
    return !(e && e[0] == '0');
}

struct Job {
    uint64_t id = 0;
    std::string bases;
    std::vector<int64_t> off;
    std::vector<int32_t> len;
    int n = 0, k = 6, band = 10;
    float kthr = -1, gthr = -1;
    int maxlen = 0;
    size_t mem_base = 0;   // estimate without the genDist cell tags
    size_t mem = 0;        // estimate of a lone run
    int state = CRISPY_JOB_QUEUED;
    int status = CRISPY_OK;
    std::string err;
    clock_type::time_point t_submit, t_done;
    int64_t kmer_pairs = 0, gen_pairs = 0;
    std::vector<int> chunk_id;
    std::vector<std::vector<uint32_t>> chunk_pairs;
    std::vector<std::vector<float>> chunk_dists;
    // memory of the run that served the job (alone or in a cohort): bytes
    // reserved at admission for all its jobs, bytes the run asked for
    size_t run_reserved = 0, run_needed = 0;
    int cohort_size = 1;
};

// Device bytes a job needs at its peak apart from the genDist cell tags
// (generous; the server only uses it for admission).
size_t estimate_base_bytes(const Job& j) {
    size_t reads = j.bases.size() + (size_t)j.n * 16;
    int64_t t = 0;
    for (int i = 0; i < j.n; ++i) t += std::max(0, j.len[i] - j.k + 1);
    // level entries + the scheduled tile stream (spare steps per group) +
    // per-read bank counts
    const size_t groups = (size_t)(j.n + 31) / 32;
    const size_t entries = (size_t)(2 * t + 32LL * (16 + 40) * groups) * 4 + (size_t)j.n * 136;
    const size_t survivors = (size_t)std::max<int64_t>(1 << 20, 16LL * j.n) * 24;
    const size_t gen = (size_t)std::max<int64_t>(1 << 20, 16LL * j.n) * 48 + reads;
    return 2 * reads + entries + survivors + gen + (8u << 20);
}

// Bytes of the 16-bit DP's cell tags a run over n reads of at most maxlen
// symbols may ask for: two launches in flight, each holding one word per
// resident lane, register and sub-block (two per 16-step block, for pairs
// of L1 + L2 <= min(2 maxlen, kGen16MaxSum)), and never more lanes than
// 32 per possible pair plus a block.  It depends on the run, not the job:
// a cohort counts it once.
size_t tag_bytes(int maxlen, int64_t n, int sms) {
    const int64_t pairs = n * (n - 1) / 2;
    const int64_t lane_regs = std::min<int64_t>((int64_t)sms * crispy::gen16_lane_regs_per_sm(),
                                                (32 * pairs + 128) * crispy::kGen16MaxR);
    const int64_t blocks = crispy::gen16_dir_blocks(std::min(2 * maxlen, crispy::kGen16MaxSum));
    return (size_t)(2 * lane_regs * 2 * blocks * 4);
}

// Estimate of one run over the jobs js (a lone job or a cohort).
size_t run_bytes(const std::vector<Job*>& js, int sms) {
    size_t base = 0;
    int maxlen = 0;
    int64_t n = 0;
    for (const Job* j : js) {
        base += j->mem_base;
        maxlen = std::max(maxlen, j->maxlen);
        n += j->n;
    }
    return base + tag_bytes(maxlen, n, sms);
}

// K = 8: the same-key pass's queue of H sums, per block (one per SM) and
// lane slot at most one item of up to 14 words per column group.
size_t k8_queue_bytes(const Job& j, int sms) {
    if (j.k != 8) return 0;
    return (size_t)sms * (size_t)((j.n + 31) / 32 + 1) * 14 * 32 * 4;
}

void set_estimate(Job& j, int sms) {
    j.maxlen = 0;
    for (int i = 0; i < j.n; ++i) j.maxlen = std::max(j.maxlen, j.len[i]);
    j.mem_base = estimate_base_bytes(j) + k8_queue_bytes(j, sms);
    j.mem = j.mem_base + tag_bytes(j.maxlen, j.n, sms);
}

// SMs of a device for the estimates (a GB300's 152 when it cannot be read).
int device_sms(int device) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        sms = 152;
    }
    return sms;
}

int sink_to_job(void* user, int chunk, const void* pairs, const float* dists, int64_t count) {
    Job* j = static_cast<Job*>(user);
    j->chunk_id.push_back(chunk);
    const uint32_t* p = static_cast<const uint32_t*>(pairs);
    j->chunk_pairs.emplace_back(p, p + 2 * count);
    j->chunk_dists.emplace_back(dists, dists + count);
    j->gen_pairs += count;
    return 0;
}

}  // namespace

struct crispy_server {
    int device = 0;
    int sms = 152;   // the device's SMs, for the estimates
    size_t budget = 0, claimed = 0;
    std::vector<crispy_ctx*> ctx;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable work_cv, done_cv;
    std::deque<Job*> queue;
    std::unordered_map<uint64_t, Job*> jobs;
    bool stopping = false;
    uint64_t next_id = 1;
    std::vector<double> latencies_ms;
    int64_t pairs_done = 0;
    std::string err;

    Job* take_fitting() {   // caller holds mu
        for (auto it = queue.begin(); it != queue.end(); ++it) {
            if (claimed + (*it)->mem <= budget) {
                Job* j = *it;
                queue.erase(it);
                return j;
            }
        }
        return nullptr;
    }

    bool cohort_member(const Job* j) const {
        return cohorts_enabled() && j->k >= 2 && j->k <= 6 && j->n >= 10 && j->n <= kCohortJobReads;
    }

    // With `first` taken: the other queued jobs that can share its run.
    // A cohort forms only under a backlog -- at least as many jobs still
    // queued as there are slots, so that every slot has work anyway -- since
    // a job that could start alone on an idle slot finishes sooner alone.
    std::vector<Job*> take_cohort(Job* first) {   // caller holds mu
        std::vector<Job*> c{first};
        if (!cohort_member(first) || queue.size() < ctx.size()) return c;
        auto aligned = [](int n) { return (n + 127) / 128 * 128; };
        int reads = aligned(first->n);
        for (auto it = queue.begin(); it != queue.end() && (int)c.size() < kCohortJobs;) {
            Job* j = *it;
            bool take = cohort_member(j) && j->k == first->k && j->band == first->band &&
                        reads + aligned(j->n) <= kCohortReads;
            if (take) {
                c.push_back(j);
                take = claimed + run_bytes(c, sms) <= budget;
                if (!take) c.pop_back();
            }
            if (take) {
                reads += aligned(j->n);
                it = queue.erase(it);
            } else {
                ++it;
            }
        }
        return c;
    }

    // Several jobs in one run: reads back to back at 128-aligned bases, with
    // reads of K - 1 symbols (no k-mer, no pair) filling the gaps.
    int run_cohort(crispy_ctx* c, const std::vector<Job*>& js) {
        const int k = js[0]->k;
        std::vector<crispy::CohortJob> kj(js.size()), gj(js.size());
        std::string bases;
        std::vector<int64_t> off;
        std::vector<int32_t> len;
        const std::string pad((size_t)(k - 1), 'A');
        for (size_t q = 0; q < js.size(); ++q) {
            const Job* j = js[q];
            kj[q].base = (int)len.size();
            kj[q].n = j->n;
            kj[q].thr = crispy_default_threshold(j->n, j->kthr, 0);
            gj[q] = kj[q];
            gj[q].thr = crispy_default_threshold(j->n, j->gthr, 1);
            gj[q].sink = sink_to_job;
            gj[q].user = js[q];
            for (int i = 0; i < j->n; ++i) {
                off.push_back((int64_t)bases.size());
                len.push_back(j->len[i]);
                bases.append(j->bases, (size_t)j->off[i], (size_t)j->len[i]);
            }
            while (len.size() % 128 != 0) {
                off.push_back((int64_t)bases.size());
                len.push_back(k - 1);
                bases += pad;
            }
        }
        int rc = crispy_kmer_prepare(c, bases.data(), off.data(), len.data(), (int)len.size(), k);
        std::vector<int64_t> kc, gc;
        if (rc == CRISPY_OK) rc = crispy::kmer_run_cohort(c, kj, kc);
        if (rc == CRISPY_OK) rc = crispy_gen_prepare_from_kmer(c);
        if (rc == CRISPY_OK) rc = crispy::gen_run_cohort(c, gj, kc, js[0]->band, gc);
        if (rc == CRISPY_OK)
            for (size_t q = 0; q < js.size(); ++q) js[q]->kmer_pairs = kc[q];
        return rc;
    }

    // Runs one job or a cohort on slot context c; fills each job's status.
    void run_jobs(crispy_ctx* c, const std::vector<Job*>& js) {
        c->run_epoch++;
        c->run_need = 0;
        const size_t reserved = run_bytes(js, sms);
        bool done = false;
        if (js.size() > 1) {
            const int rc = run_cohort(c, js);
            if (rc == CRISPY_OK) {
                for (Job* j : js) j->status = CRISPY_OK;
                done = true;
            } else {
                // the cohort form declined (or failed): every job alone, from scratch
                for (Job* j : js) {
                    j->chunk_id.clear(); j->chunk_pairs.clear(); j->chunk_dists.clear();
                    j->gen_pairs = 0; j->kmer_pairs = 0;
                }
            }
        }
        if (!done)
            for (Job* j : js) run_job(c, j);
        const size_t need = c->run_need;
        for (Job* j : js) {
            j->run_reserved = reserved;
            j->run_needed = need;
            j->cohort_size = done ? (int)js.size() : 1;
        }
    }

    void run_job(crispy_ctx* c, Job* j) {
        int rc = crispy_kmer_prepare(c, j->bases.data(), j->off.data(), j->len.data(), j->n, j->k);
        const float kt = crispy_default_threshold(j->n, j->kthr, 0);
        const float gt = crispy_default_threshold(j->n, j->gthr, 1);
        if (rc == CRISPY_OK) rc = crispy_kmer_run(c, kt, CRISPY_MODE_BATCHED, 0, &j->kmer_pairs);
        if (rc == CRISPY_OK) rc = crispy_gen_prepare_from_kmer(c);   // reads already on the device
        int64_t ns = 0;
        if (rc == CRISPY_OK)
            rc = crispy_gen_run_from_kmer(c, j->band, gt, CRISPY_MODE_BATCHED, sink_to_job, j, &ns);
        j->status = rc;
        if (rc != CRISPY_OK) j->err = crispy_last_error(c);
    }

    void worker(int slot) {
        crispy_ctx* c = ctx[slot];
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            Job* j = nullptr;
            work_cv.wait(lk, [&] { return stopping || (j = take_fitting()) != nullptr; });
            if (!j) return;   // stopping
            const std::vector<Job*> js = take_cohort(j);
            const size_t mem = run_bytes(js, sms);
            for (Job* x : js) x->state = CRISPY_JOB_RUNNING;
            claimed += mem;
            lk.unlock();
            run_jobs(c, js);
            // give memory back when this slot holds more than its share
            size_t in_use = 0;
            crispy_ctx_mem_in_use(c, &in_use);
            if (in_use > budget / ctx.size()) crispy_ctx_trim(c);
            lk.lock();
            claimed -= mem;
            const auto now = clock_type::now();
            for (Job* x : js) {
                x->t_done = now;
                x->state = x->status == CRISPY_OK ? CRISPY_JOB_DONE : CRISPY_JOB_FAILED;
                if (x->status == CRISPY_OK) {
                    latencies_ms.push_back(
                        std::chrono::duration<double, std::milli>(x->t_done - x->t_submit).count());
                    pairs_done += (int64_t)x->n * (x->n - 1) / 2;
                }
            }
            done_cv.notify_all();
            work_cv.notify_all();
        }
    }
};

extern "C" {

int crispy_server_create(int device, size_t hbm_budget_bytes, int slots, crispy_server** out) {
    if (!out || slots < 1 || slots > 64)
        return crispy::fail(nullptr, CRISPY_E_INPUT, "server: bad arguments");
    *out = nullptr;
    auto* s = new crispy_server();
    s->device = device;
    s->sms = device_sms(device);
    if (hbm_budget_bytes == 0) {
        size_t free_b = 0, total = 0;
        cudaSetDevice(device);
        cudaMemGetInfo(&free_b, &total);
        hbm_budget_bytes = free_b / 2;
    }
    s->budget = hbm_budget_bytes;
    for (int i = 0; i < slots; ++i) {
        crispy_ctx* c = nullptr;
        int rc = crispy_ctx_create(device, &c);
        if (rc != CRISPY_OK) {
            for (auto* x : s->ctx) crispy_ctx_destroy(x);
            delete s;
            return rc;
        }
        c->kmer_tune = false;
        s->ctx.push_back(c);
    }
    for (int i = 0; i < slots; ++i) s->workers.emplace_back(&crispy_server::worker, s, i);
    *out = s;
    return CRISPY_OK;
}

int crispy_server_destroy(crispy_server* s) {
    if (!s) return CRISPY_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stopping = true;
        for (Job* j : s->queue) j->state = CRISPY_JOB_CANCELLED;
        s->queue.clear();
    }
    s->work_cv.notify_all();
    for (auto& t : s->workers) t.join();
    for (auto* c : s->ctx) crispy_ctx_destroy(c);
    for (auto& kv : s->jobs) delete kv.second;
    delete s;
    return CRISPY_OK;
}

int crispy_server_submit(crispy_server* s, const char* seqbuf, const int64_t* offsets,
                         const int32_t* lengths, int n, int k, int band, float kmer_thr,
                         float gen_thr, uint64_t* job_id) {
    if (!s || !seqbuf || !offsets || !lengths || n <= 0 || !job_id) {
        if (s) s->err = "submit: NULL or empty read set";
        return CRISPY_E_INPUT;
    }
    auto* j = new Job();
    int64_t end = 0;
    for (int i = 0; i < n; ++i) end = std::max(end, offsets[i] + lengths[i]);
    j->bases.assign(seqbuf, seqbuf + end);
    j->off.assign(offsets, offsets + n);
    j->len.assign(lengths, lengths + n);
    j->n = n;
    j->k = k;
    j->band = band <= 0 ? 2 : band;
    j->kthr = kmer_thr;
    j->gthr = gen_thr;
    set_estimate(*j, s->sms);
    j->t_submit = clock_type::now();
    std::lock_guard<std::mutex> g(s->mu);
    if (j->mem > s->budget) {
        s->err = "job needs more device memory than the server budget";
        delete j;
        return CRISPY_E_OOM;
    }
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    *job_id = j->id;
    s->work_cv.notify_one();
    return CRISPY_OK;
}

int crispy_server_wait(crispy_server* s, uint64_t id, int timeout_ms, int* state) {
    if (!s) return CRISPY_E_INPUT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) {
        s->err = "unknown job id";
        return CRISPY_E_INPUT;
    }
    Job* j = it->second;
    auto finished = [&] { return j->state >= CRISPY_JOB_DONE; };
    if (timeout_ms < 0) {
        s->done_cv.wait(lk, finished);
    } else if (!s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished)) {
        if (state) *state = j->state;
        return CRISPY_E_TIMEOUT;
    }
    if (state) *state = j->state;
    return CRISPY_OK;
}

int crispy_server_result(crispy_server* s, uint64_t id, crispy_sink sink, void* user,
                         int64_t* kmer_pairs, int64_t* gen_pairs) {
    if (!s) return CRISPY_E_INPUT;
    Job* j = nullptr;
    {
        std::lock_guard<std::mutex> g(s->mu);
        auto it = s->jobs.find(id);
        if (it == s->jobs.end()) {
            s->err = "unknown job id";
            return CRISPY_E_INPUT;
        }
        j = it->second;
        if (j->state < CRISPY_JOB_DONE) {
            s->err = "job not finished";
            return CRISPY_E_STATE;
        }
        s->jobs.erase(it);
    }
    int rc = CRISPY_OK;
    if (j->state == CRISPY_JOB_CANCELLED) {
        rc = CRISPY_E_STATE;
        s->err = "job was cancelled";
    } else if (j->state == CRISPY_JOB_FAILED) {
        rc = j->status;
        s->err = j->err;
    } else {
        if (kmer_pairs) *kmer_pairs = j->kmer_pairs;
        if (gen_pairs) *gen_pairs = j->gen_pairs;
        for (size_t c = 0; c < j->chunk_id.size() && sink; ++c) {
            if (sink(user, j->chunk_id[c], j->chunk_pairs[c].data(), j->chunk_dists[c].data(),
                     (int64_t)j->chunk_dists[c].size()) != 0) {
                rc = CRISPY_E_IO;
                break;
            }
        }
    }
    delete j;
    return rc;
}

int crispy_server_job_memory(crispy_server* s, uint64_t id, size_t* reserved, size_t* needed,
                             int* cohort_size) {
    if (!s) return CRISPY_E_INPUT;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) {
        s->err = "unknown job id";
        return CRISPY_E_INPUT;
    }
    const Job* j = it->second;
    if (j->state != CRISPY_JOB_DONE) {
        s->err = "job not finished";
        return CRISPY_E_STATE;
    }
    if (reserved) *reserved = j->run_reserved;
    if (needed) *needed = j->run_needed;
    if (cohort_size) *cohort_size = j->cohort_size;
    return CRISPY_OK;
}

int crispy_server_job_bytes(const int32_t* lengths, int n, int k, size_t* bytes) {
    if (!lengths || n <= 0 || !bytes) return CRISPY_E_INPUT;
    Job j;
    j.n = n;
    j.k = k;
    j.len.assign(lengths, lengths + n);
    int64_t total = 0;
    for (int i = 0; i < n; ++i) total += std::max(0, lengths[i]);
    j.bases.assign((size_t)total, 'A');
    int dev = 0;
    cudaGetDevice(&dev);
    set_estimate(j, device_sms(dev));
    *bytes = j.mem;
    return CRISPY_OK;
}

int crispy_server_cancel(crispy_server* s, uint64_t id) {
    if (!s) return CRISPY_E_INPUT;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return CRISPY_E_INPUT;
    Job* j = it->second;
    auto q = std::find(s->queue.begin(), s->queue.end(), j);
    if (q == s->queue.end()) {
        s->err = "job already running or finished";
        return CRISPY_E_STATE;
    }
    s->queue.erase(q);
    j->state = CRISPY_JOB_CANCELLED;
    s->done_cv.notify_all();
    return CRISPY_OK;
}

int crispy_server_stats(crispy_server* s, double* p50, double* p99, int64_t* jobs_done,
                        int64_t* pairs_done) {
    if (!s) return CRISPY_E_INPUT;
    std::lock_guard<std::mutex> g(s->mu);
    std::vector<double> v(s->latencies_ms);
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) -> double {
        if (v.empty()) return 0.0;
        // nearest-rank percentile
        size_t r = (size_t)std::ceil(q * v.size());
        return v[std::min(v.size(), std::max<size_t>(r, 1)) - 1];
    };
    if (p50) *p50 = pct(0.50);
    if (p99) *p99 = pct(0.99);
    if (jobs_done) *jobs_done = (int64_t)v.size();
    if (pairs_done) *pairs_done = s->pairs_done;
    return CRISPY_OK;
}

int crispy_server_stats_reset(crispy_server* s) {
    if (!s) return CRISPY_E_INPUT;
    std::lock_guard<std::mutex> g(s->mu);
    s->latencies_ms.clear();
    s->pairs_done = 0;
    return CRISPY_OK;
}

const char* crispy_server_last_error(const crispy_server* s) { return s ? s->err.c_str() : ""; }

}  // extern "C"
