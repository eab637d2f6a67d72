"""Host-side checks that need no GPU: the C-ABI library loads and exports
every function include/crispy_gb300.h declares, its host helpers (FASTA
parser, default thresholds, tile size) agree with the oracle, and the
synthetic generator is deterministic and ordered like preprocess."""
import ctypes
import os
import re

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(crispy_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    lib = cg.load_library()
    decl = _declared()
    assert len(decl) >= 20
    missing = [n for n in decl if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the whole header
    assert decl <= set(cg.PROTOTYPES) | {"crispy_sink"}


def test_version_string():
    assert b"sm_103a" in cg.load_library().crispy_version()


@pytest.mark.parametrize("n", [1, 2, 9, 10, 99, 100, 500, 501, 585, 999, 1000, 20000, 100000, 1048576])
def test_thresholds_and_tile_size(n):
    for stage, num in ((0, 2), (1, 1)):
        for user in (-1.0, 0.0, 0.3, 1.0, 1.5):
            a = cg.default_threshold(n, user, stage)
            b = oracle.default_threshold(n, user, num)
            assert np.float32(a).view(np.uint32) == np.float32(b).view(np.uint32)
    assert cg.array_dim(n) == oracle.array_dim(n)


def _write(path, data: bytes):
    with open(path, "wb") as f:
        f.write(data)


FASTA_CASES = {
    "plain": b">a\nACGT\n>b\nGGCCA\n",
    "crlf": b">a\r\nACGTN\r\n>b x\r\nGG\r\nCC\r\n",
    "blank_inside": b">a\nACGT\n\nTTTT\n>b\nCC\n\n",
    "no_final_newline": b">a\nACGT\n>b\nACGTAC",
    "trailing_junk": b">a\nACGTNNN-\n>b\nacgtnn*\n",
    "empty_record": b">a\n>b\nACG\n>c\n\n>d\nT\n",
    "dollar_line": b">a\nACGT\n$stop\n>b\nCCCC\n",
    "long_line": b">a\n" + b"ACGT" * 1500 + b"\n>b\nAC\n",
    "long_header": b">" + b"h" * 5000 + b"\nACGT\n",
    "spaces": b">a\nAC GT \t\n>b\n  ACG\n",
}


def _reads_of(parsed):
    data, offs, lens = parsed
    return [data[o:o + l].tobytes() for o, l in zip(offs.tolist(), lens.tolist())]


@pytest.mark.parametrize("chunks", [None, "3", "9"])
@pytest.mark.parametrize("case", sorted(FASTA_CASES))
@pytest.mark.parametrize("flavour", [0, 1])
def test_fasta_parser_matches_oracle(tmp_path, monkeypatch, case, flavour, chunks):
    """Same reads as the oracle's parse, also when the file is scanned in
    several chunks (CRISPY_PARSE_CHUNKS) and the reads sit at chunk offsets."""
    p = str(tmp_path / case)
    _write(p, FASTA_CASES[case] * 7)
    if chunks:
        monkeypatch.setenv("CRISPY_PARSE_CHUNKS", chunks)
    a = cg.read_fasta(p, flavour)
    b = oracle.read_fasta(p, flavour)
    assert _reads_of(a) == _reads_of(b)


def test_fasta_not_fasta(tmp_path):
    p = str(tmp_path / "bad")
    _write(p, b"ACGT\n")
    with pytest.raises(cg.CrispyError) as e:
        cg.read_fasta(p, 0)
    assert e.value.code == cg.E_INPUT
    with pytest.raises(cg.CrispyError) as e:
        cg.read_fasta(str(tmp_path / "missing"), 0)
    assert e.value.code == cg.E_IO


def test_engine_without_gpu_fails_loudly():
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    with pytest.raises(cg.CrispyError) as e:
        cg.Engine(0)
    assert e.value.code == cg.E_DEVICE


def test_synth_deterministic_and_ordered():
    a = synth.make_read_set("small_1k")
    b = synth.make_read_set("small_1k")
    assert a == b
    assert len(set(a)) == len(a)
    assert all((len(x), x) < (len(y), y) for x, y in zip(a, a[1:]))
    assert all(set(s) <= set(b"ACGT") for s in a)
    lens = np.array([len(s) for s in a])
    assert 200 < lens.mean() < 265
