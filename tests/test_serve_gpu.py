"""Job server: each job's result is identical alone and in a mix; admission
by HBM budget; cancellation of queued jobs; a bad job fails alone."""
import threading

import numpy as np
import pytest

import crispy_gb300 as cg
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


def _job(n, seed, dist="normal", a=250, b=20, root=260):
    reads = synth.make_read_set(synth.ReadSetSpec(n, max(4, n // 50), root, dist, a, b, 6, seed))
    return synth.pack_reads(reads)


def _same(r1, r2):
    k1, c1 = r1
    k2, c2 = r2
    assert k1 == k2 and len(c1) == len(c2)
    for (i1, p1, d1), (i2, p2, d2) in zip(c1, c2):
        assert i1 == i2 and np.array_equal(p1, p2)
        assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


def test_alone_vs_mixed_bit_exact():
    jobs = [_job(n, 500 + n) for n in (600, 1500, 3000, 800, 2200, 5000)]
    jobs.append(_job(1200, 77, dist="uniform", a=300, b=500, root=520))
    alone = []
    with cg.Server(0, 0, 1) as srv:
        for buf, offs, lens in jobs:
            jid = srv.submit(buf, offs, lens)
            assert srv.wait(jid) == cg.JOB_DONE
            alone.append(srv.result(jid))
    with cg.Server(0, 0, 4) as srv:
        ids = []
        lock = threading.Lock()

        def submit(i):
            jid = srv.submit(*jobs[i])
            with lock:
                ids.append((i, jid))

        ts = [threading.Thread(target=submit, args=(i,)) for i in range(len(jobs))]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        for i, jid in sorted(ids):
            assert srv.wait(jid) == cg.JOB_DONE
            _same(srv.result(jid), alone[i])
        st = srv.stats()
        assert st["jobs"] == len(jobs) and st["p99_ms"] >= st["p50_ms"] > 0


def test_matches_engine_pipeline():
    buf, offs, lens = _job(2500, 9)
    n = len(lens)
    with cg.Engine(0) as eng:
        eng.kmer_prepare(buf, offs, lens, 6)
        kp = eng.kmer_run(cg.default_threshold(n, -1.0, 0), cg.MODE_BATCHED, False)
        eng.gen_prepare(buf, offs, lens)
        chunks = eng.gen_run_from_kmer(10, cg.default_threshold(n, -1.0, 1), cg.MODE_BATCHED)
    with cg.Server(0, 0, 2) as srv:
        jid = srv.submit(buf, offs, lens)
        srv.wait(jid)
        _same(srv.result(jid), (kp, chunks))


def test_budget_admission_and_cancel():
    small = _job(700, 31)
    big = _job(6000, 32)
    # a budget below one job's estimate is refused at submit
    with cg.Server(0, 4 << 20, 2) as srv:
        with pytest.raises(cg.CrispyError) as e:
            srv.submit(*small)
        assert e.value.code == cg.E_OOM
    # a budget that fits one job at a time still finishes every job, in order
    with cg.Server(0, 600 << 20, 4) as srv:
        ids = [srv.submit(*small) for _ in range(3)] + [srv.submit(*big)]
        victim = srv.submit(*small)
        try:
            srv.cancel(victim)
            cancelled = True
        except cg.CrispyError:
            cancelled = False   # it may already have started
        for jid in ids:
            assert srv.wait(jid) == cg.JOB_DONE
            srv.result(jid)
        st = srv.wait(victim)
        assert st == (cg.JOB_CANCELLED if cancelled else cg.JOB_DONE)


def test_failed_job_is_isolated():
    good = _job(900, 41)
    with cg.Server(0, 0, 2) as srv:
        bad_buf = np.frombuffer(b"ACG" * 1001, np.uint8).copy()   # 3003 bytes cover both reads
        bad = srv.submit(bad_buf, np.array([0, 3], np.int64), np.array([3, 3000], np.int32))
        ok = srv.submit(*good)
        assert srv.wait(bad) == cg.JOB_FAILED
        with pytest.raises(cg.CrispyError) as e:
            srv.result(bad)
        assert e.value.code in (cg.E_UNSUPPORTED, cg.E_INPUT)
        assert srv.wait(ok) == cg.JOB_DONE
        assert srv.result(ok)[0] > 0


def test_mixed_k_jobs(engine):
    # k = 8 jobs hold their reads in their own read order on their slot's
    # context; served alone, mixed with k = 6 jobs, and through the Engine,
    # they give the same chunks
    def job8(n, seed):
        reads = synth.make_read_set(synth.ReadSetSpec(n, max(4, n // 50), 260, "normal", 250, 30, 8, seed))
        return synth.pack_reads(reads)
    jobs = [(_job(1500, 901), 6, 10), (job8(2500, 902), 8, 5), (_job(900, 903), 6, 10),
            (job8(1200, 904), 8, 5), (job8(4000, 905), 8, 10)]
    alone = []
    with cg.Server(0, 0, 1) as srv:
        for (buf, offs, lens), k, band in jobs:
            jid = srv.submit(buf, offs, lens, k=k, band=band)
            assert srv.wait(jid) == cg.JOB_DONE
            alone.append(srv.result(jid))
    with cg.Server(0, 0, 3) as srv:
        ids = [srv.submit(buf, offs, lens, k=k, band=band) for (buf, offs, lens), k, band in jobs]
        for jid, want in zip(ids, alone):
            assert srv.wait(jid) == cg.JOB_DONE
            _same(srv.result(jid), want)
    (buf, offs, lens), k, band = jobs[1]
    n = len(lens)
    engine.kmer_prepare(buf, offs, lens, k)
    kp = engine.kmer_run(cg.default_threshold(n, -1.0, 0), cg.MODE_BATCHED, False)
    engine.gen_prepare_from_kmer()
    chunks = engine.gen_run_from_kmer(band, cg.default_threshold(n, -1.0, 1), cg.MODE_BATCHED)
    _same((kp, chunks), alone[1])
    assert kp > 0 and sum(len(c[2]) for c in chunks) > 0


def _engine_run(eng, buf, offs, lens, k=6, band=10):
    n = len(lens)
    eng.kmer_prepare(buf, offs, lens, k)
    kp = eng.kmer_run(cg.default_threshold(n, -1.0, 0), cg.MODE_BATCHED, False)
    eng.gen_prepare_from_kmer()
    return kp, eng.gen_run_from_kmer(band, cg.default_threshold(n, -1.0, 1), cg.MODE_BATCHED)


def test_cohort_jobs_bit_exact_and_within_reservation():
    """Jobs queued behind a running one share one run (a cohort: one k-mer
    launch over all their row groups, one set of genDist launches over all
    their survivors); each job's result equals a lone Engine run, and every
    run asks for no more device memory than admission reserved for it."""
    sizes = (3000, 500, 1200, 64, 2048, 777, 5000, 129, 16, 4096)
    jobs = [_job(n, 900 + i) for i, n in enumerate(sizes)]
    jobs.append(_job(1500, 77, dist="uniform", a=300, b=500, root=520))
    with cg.Engine(0) as eng:
        want = [_engine_run(eng, *j) for j in jobs]
    with cg.Server(0, 0, 1) as srv:
        ids = [srv.submit(*j) for j in jobs]   # all but the first queue behind it
        cohort = []
        for i, jid in enumerate(ids):
            assert srv.wait(jid) == cg.JOB_DONE
            mem = srv.job_memory(jid)
            assert 0 < mem["needed"] <= mem["reserved"], (i, mem)
            cohort.append(mem["cohort_size"])
            _same(srv.result(jid), want[i])
    assert max(cohort) > 1, "no cohort formed"


def test_admission_estimate_bounds_each_run():
    """A job alone: the device bytes its run asks for stay within the
    estimate the server admits it with (crispy_server_job_bytes)."""
    with cg.Server(0, 0, 1) as srv:
        for n, seed in ((500, 1), (6000, 2), (20000, 3), (48000, 4)):
            buf, offs, lens = _job(n, 4000 + seed)
            jid = srv.submit(buf, offs, lens)
            assert srv.wait(jid) == cg.JOB_DONE
            mem = srv.job_memory(jid)
            assert mem["cohort_size"] == 1
            assert mem["reserved"] == cg.server_job_bytes(lens, 6)
            assert 0 < mem["needed"] <= mem["reserved"], (n, mem)
            srv.result(jid)
