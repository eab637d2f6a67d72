"""Survivor lists beyond the device share: kmerDist gathers them stage row by
stage row in pinned host memory, genDist then runs over them a batch of load
windows at a time.  Both must reproduce the one-shot results exactly.

The limits are forced small through CRISPY_KMER_DEVICE_PAIRS and
CRISPY_GEN_BATCH_WINDOWS, read at every call.
"""
import os

import numpy as np
import pytest

import crispy_gb300 as cg
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


class _env:
    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update({k: str(v) for k, v in self.kv.items()})

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _same_chunks(a, b):
    assert [c[0] for c in a] == [c[0] for c in b]
    for (_, p, d), (_, wp, wd) in zip(a, b):
        assert np.array_equal(p, wp) and np.array_equal(d.view(np.uint32), wd.view(np.uint32))


@pytest.mark.parametrize("k", [6, 8])
def test_kmer_spill_matches_device(engine, k):
    reads = synth.make_read_set(synth.ReadSetSpec(2600, 40, 260, "normal", 250, 20, k, 501 + k))
    buf, offs, lens = synth.pack_reads(reads)
    thr = 0.6 if k == 6 else 0.75
    engine.kmer_prepare(buf, offs, lens, k)
    want_n = engine.kmer_run(thr, cg.MODE_BATCHED, True)
    want_p, want_d = engine.kmer_fetch(want_n, True)
    assert engine.stats()["kmer_spilled"] == 0 and want_n > 1000
    engine.gen_prepare_from_kmer()
    want_g = engine.gen_run_from_kmer(10, 0.3, cg.MODE_BATCHED)
    for mode in (cg.MODE_BATCHED, cg.MODE_STAGED):
        with _env(CRISPY_KMER_DEVICE_PAIRS=want_n // 5):
            got_n = engine.kmer_run(thr, mode, True)
            assert engine.stats()["kmer_spilled"] == 1
        got_p, got_d = engine.kmer_fetch(got_n, True)
        assert got_n == want_n
        assert np.array_equal(got_p, want_p) and np.array_equal(got_d.view(np.uint32), want_d.view(np.uint32))
        # genDist straight from the spilled host list (windowed run)
        _same_chunks(engine.gen_run_from_kmer(10, 0.3, cg.MODE_BATCHED), want_g)


def test_gen_windowed_matches_one_shot(engine):
    # more than two load windows, one window per batch: chunks flush across
    # batch boundaries with the pending survivors carried on the device
    reads = synth.make_read_set(synth.ReadSetSpec(500, 20, 260, "normal", 250, 15, 6, 77))
    buf, offs, lens = synth.pack_reads(reads)
    engine.gen_prepare(buf, offs, lens)
    rng = np.random.default_rng(9)
    pairs = np.stack([rng.integers(0, len(reads), 2 * cg.GEN_WINDOW + 54321),
                      rng.integers(0, len(reads), 2 * cg.GEN_WINDOW + 54321)], 1).astype(np.int32)
    for thr in (1.0, 0.35):
        want = engine.gen_run(pairs, 10, thr, cg.MODE_BATCHED)
        with _env(CRISPY_GEN_BATCH_WINDOWS=1):
            got = engine.gen_run(pairs, 10, thr, cg.MODE_BATCHED)
        assert sum(len(c[2]) for c in got) == sum(len(c[2]) for c in want) > 0
        _same_chunks(got, want)
