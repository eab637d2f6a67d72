"""crispy_gen_align_noalloc: the alignment entry point for callers that
cannot allocate device memory (their device memory belongs to a pool they
set up at start-up, or their memory accounting must not see foreign
allocations).  The test plays such a caller: it owns every device buffer,
calls the entry point through the C ABI twice in a row, and compares each
result bit for bit with the allocating entry point crispy_gen_align and with
the oracle (bands 10, 2 and 1, reads of 1 to 2048 nt).

It sits in a file pytest collects last and must pass both alone in a fresh
process and after the other tests (the fixed scratch array keeps the last
call's contents between calls)."""
import ctypes as C

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


def _call(lib, dev, n, max_len, pairs_t, band, stream, outputs=True):
    """One call through the C ABI; with outputs=False only dist is passed
    (score, ml and al are NULL) and the others come back as None."""
    import torch

    npairs = pairs_t.shape[0]
    dist = torch.empty(npairs, dtype=torch.float32, device="cuda")
    score = torch.empty(npairs, dtype=torch.int32, device="cuda")
    ml = torch.empty(npairs, dtype=torch.int32, device="cuda")
    al = torch.empty(npairs, dtype=torch.int32, device="cuda")
    ptr = (lambda t: t.data_ptr()) if outputs else (lambda t: None)
    rc = lib.crispy_gen_align_noalloc(dev["seq"].data_ptr(), dev["off"].data_ptr(), dev["len"].data_ptr(),
                                      n, max_len, pairs_t.data_ptr(), npairs, band, dist.data_ptr(),
                                      ptr(score), ptr(ml), ptr(al), stream)
    torch.cuda.synchronize()
    if not outputs:
        return rc, dist.cpu().numpy(), None, None, None
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
        for band, npairs in ((10, 3000), (2, 700), (1, 200)):
            pairs = rng.integers(0, n, size=(npairs, 2)).astype(np.int32)
            od, os_, oml, oal = oracle.gen_all(buf, offs, lens, pairs, band)
            for _ in range(2):   # two calls in a row share the scratch array
                rc, d, s, ml, al = _call(lib, dev, n, int(lens.max()), torch.from_numpy(pairs).cuda(), band,
                                         stream)
                assert rc == cg.OK, lib.crispy_last_error(None)
                wd, ws, wml, wal = eng.gen_align(pairs, band, cg.MODE_BATCHED)
                assert np.array_equal(s, ws) and np.array_equal(ml, wml) and np.array_equal(al, wal)
                assert np.array_equal(d.view(np.uint32), wd.view(np.uint32))
                assert np.array_equal(s, os_) and np.array_equal(ml, oml) and np.array_equal(al, oal)
                assert np.array_equal(d.view(np.uint32), od.view(np.uint32))


def test_noalloc_max_length_reads_and_null_outputs():
    """Reads at the 2048-nt limit (band 10 and the unbanded band 1), with
    score / ml / al passed as NULL: dist alone, equal to the oracle's."""
    torch = pytest.importorskip("torch")
    lib = cg.load_library()
    rng = np.random.default_rng(21)
    base = rng.integers(0, 4, 2048)
    reads = []
    for sub in (0.0, 0.02, 0.05, 0.3):
        r = base.copy()
        hit = rng.random(2048) < sub
        r[hit] = (r[hit] + rng.integers(1, 4, hit.sum())) % 4
        reads.append(bytes(np.array(list(b"AGTC"), np.uint8)[r]))
    reads += [reads[1][:1500], b"ACGT" * 10]
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    assert int(lens.max()) == 2048
    dev = {"seq": torch.from_numpy(buf).cuda(), "off": torch.from_numpy(offs).cuda(),
           "len": torch.from_numpy(lens).cuda()}
    stream = torch.cuda.current_stream().cuda_stream
    pairs = np.array([[0, 1], [0, 2], [1, 3], [4, 0], [5, 2], [3, 3]], np.int32)
    for band in (10, 1):
        od, _, _, _ = oracle.gen_all(buf, offs, lens, pairs, band)
        for _ in range(2):
            rc, d, s, ml, al = _call(lib, dev, n, 2048, torch.from_numpy(pairs).cuda(), band, stream,
                                     outputs=False)
            assert rc == cg.OK, lib.crispy_last_error(None)
            assert s is None and np.array_equal(d.view(np.uint32), od.view(np.uint32))


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
    # a read longer than max_len: refused per pair, whatever its band width
    # (pair 1 holds the longest read, pair 0 two reads within the limit)
    order = np.argsort(lens)
    short_a, short_b, longest = int(order[0]), int(order[1]), int(order[-1])
    limit = int(lens[short_b])
    assert int(lens[longest]) > limit
    mixed = torch.tensor([[short_a, short_b], [short_a, longest]], dtype=torch.int32, device="cuda")
    rc, d, s, ml, al = _call(lib, dev, n, limit, mixed, 10, stream)
    assert rc == cg.E_INPUT
    assert np.isnan(d[1]) and s[1] == -1 and ml[1] == -1 and al[1] == -1
    od, os_, oml, oal = oracle.gen_all(buf, offs, lens, mixed.cpu().numpy()[:1], 10)
    assert d[0] == od[0] and s[0] == os_[0] and ml[0] == oml[0] and al[0] == oal[0]
