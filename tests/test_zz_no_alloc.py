"""crispy_gen_align_noalloc: the alignment entry point for callers that
cannot allocate device memory (their device memory belongs to a pool they
set up at start-up, or their memory accounting must not see foreign
allocations).  The test plays such a caller: it owns every device buffer,
calls the entry point through the C ABI twice in a row, and compares each
result bit for bit with the allocating entry point crispy_gen_align.

It sits in a file pytest collects last and must pass both alone in a fresh
process and after the other tests (the fixed scratch array keeps the last
call's contents between calls)."""
import ctypes as C

import numpy as np
import pytest

import crispy_gb300 as cg
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


def _call(lib, dev, n, max_len, pairs_t, band, stream):
    import torch

    npairs = pairs_t.shape[0]
    dist = torch.empty(npairs, dtype=torch.float32, device="cuda")
    score = torch.empty(npairs, dtype=torch.int32, device="cuda")
    ml = torch.empty(npairs, dtype=torch.int32, device="cuda")
    al = torch.empty(npairs, dtype=torch.int32, device="cuda")
    rc = lib.crispy_gen_align_noalloc(dev["seq"].data_ptr(), dev["off"].data_ptr(), dev["len"].data_ptr(),
                                      n, max_len, pairs_t.data_ptr(), npairs, band, dist.data_ptr(),
                                      score.data_ptr(), ml.data_ptr(), al.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc, dist.cpu().numpy(), score.cpu().numpy(), ml.cpu().numpy(), al.cpu().numpy()


def test_noalloc_matches_gen_align_twice():
    torch = pytest.importorskip("torch")
    lib = cg.load_library()
    reads = synth.make_read_set(synth.ReadSetSpec(300, 12, 520, "uniform", 250, 500, 6, 404))
    reads += [b"A", b"ACGT", b"GATTACA" * 40]
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    dev = {"seq": torch.from_numpy(buf).cuda(), "off": torch.from_numpy(offs).cuda(),
           "len": torch.from_numpy(lens).cuda()}
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    with cg.Engine(0) as eng:
        eng.gen_prepare(buf, offs, lens)
        for band, npairs in ((10, 3000), (2, 700)):
            pairs = rng.integers(0, n, size=(npairs, 2)).astype(np.int32)
            rc, d, s, ml, al = _call(lib, dev, n, int(lens.max()), torch.from_numpy(pairs).cuda(), band, stream)
            assert rc == cg.OK, lib.crispy_last_error(None)
            wd, ws, wml, wal = eng.gen_align(pairs, band, cg.MODE_BATCHED)
            assert np.array_equal(s, ws) and np.array_equal(ml, wml) and np.array_equal(al, wal)
            assert np.array_equal(d.view(np.uint32), wd.view(np.uint32))


def test_noalloc_rejects_out_of_range():
    torch = pytest.importorskip("torch")
    lib = cg.load_library()
    reads = synth.make_read_set(synth.ReadSetSpec(40, 4, 260, "normal", 250, 15, 6, 405))
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    dev = {"seq": torch.from_numpy(buf).cuda(), "off": torch.from_numpy(offs).cuda(),
           "len": torch.from_numpy(lens).cuda()}
    stream = torch.cuda.current_stream().cuda_stream
    good = torch.tensor([[0, 1], [2, 3]], dtype=torch.int32, device="cuda")
    rc, *_ = _call(lib, dev, n, 4096, good, 10, stream)
    assert rc == cg.E_UNSUPPORTED           # max_len beyond the reference limit
    bad = torch.tensor([[0, 1], [2, n]], dtype=torch.int32, device="cuda")
    rc, d, *_ = _call(lib, dev, n, int(lens.max()), bad, 10, stream)
    assert rc == cg.E_INPUT                 # index n is outside [0, n)
    rc, *_ = _call(lib, dev, n, int(lens.max()), good, 10, stream)
    assert rc == cg.OK                      # the error word is cleared per call
