"""Preprocess checks that need no GPU.

* The oracle's preprocess (oracle/oracle_pre.cpp) reproduces the reference's
  own preprocess outputs byte for byte on every fixture of
  tests/golden/pre/ (made by tests/golden/pre/make_pre_golden.py from
  src/preprocess/preprocess.cpp compiled as it lies).
* The engine's host side -- crispy_raw_load (the record parser) and
  crispy_pre_write (the _Clean / .frq writer) -- reproduces the fixtures
  when the sort and merge between them are done here in Python (the device
  part runs in tests/test_pre_gpu.py).
"""
import json
import os
import shutil

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pre")
MANIFEST = json.load(open(os.path.join(GOLD, "MANIFEST.json")))


def _opts(args):
    sd = primer = None
    mm = 2
    fastq = False
    out = None
    for a, b in zip(args, args[1:] + [None]):
        if a == "-s":
            sd = float(b)
        elif a == "-m":
            mm = int(b)
        elif a == "-p":
            primer = b
        elif a == "-f" and b == "q":
            fastq = True
        elif a == "-o":
            out = b
    return sd, primer, mm, fastq, out


def _case_dir(tmp_path, name):
    d = tmp_path / name
    shutil.copytree(os.path.join(GOLD, name), d)
    return d


def _primer_text(d, primer_file):
    with open(os.path.join(d, primer_file), "rb") as f:
        line = f.readline().rstrip(b"\n")
    return line.rstrip(b"\r \t\v\f\b")


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_oracle_matches_reference_fixture(tmp_path, name):
    case = MANIFEST[name]
    d = _case_dir(tmp_path, name)
    sd, primer_file, mm, fastq, _ = _opts(case["args"])
    primer = _primer_text(d, primer_file) if primer_file else None
    out = str(d / ("oracle_" + case["output"]))
    c = oracle.preprocess(str(d / case["input"]), out, fastq=fastq, sd=sd, primer=primer, max_mm=mm)
    assert open(out, "rb").read() == open(d / case["output"], "rb").read()
    assert open(out + ".frq", "rb").read() == open(str(d / case["output"]) + ".frq", "rb").read()
    assert c["records"] == case["total"]
    deleted = c["length_discards"] + c["primer_discards"] + c["merges"]
    assert c["records"] - deleted == case["preprocessed"]


def _host_sort_merge(raw: cg.RawReads):
    """(length, bytes, record) order and the fold of equal runs into their
    last read -- the part crispy_preprocess does on the device."""
    live = [i for i in range(raw.n) if raw.freq[i]]
    seqs = {i: raw.seq(i) for i in live}
    live.sort(key=lambda i: (len(seqs[i]), seqs[i], i))
    index, freq = [], []
    for k, i in enumerate(live):
        if k + 1 < len(live) and seqs[live[k + 1]] == seqs[i]:
            continue
        run = 1
        while k - run >= 0 and seqs[live[k - run]] == seqs[i]:
            run += 1
        index.append(i)
        freq.append(run)
    return np.array(index, np.int32), np.array(freq, np.int32)


@pytest.mark.parametrize("name", sorted(n for n, c in MANIFEST.items()
                                        if "-s" not in c["args"] and "-p" not in c["args"]))
def test_engine_host_parse_and_write(tmp_path, name):
    case = MANIFEST[name]
    d = _case_dir(tmp_path, name)
    _, _, _, fastq, _ = _opts(case["args"])
    raw = cg.RawReads(str(d / case["input"]), fastq=fastq)
    assert raw.records == case["total"]
    index, freq = _host_sort_merge(raw)
    out = str(d / "engine_out")
    raw.write(index, freq, out)
    assert open(out, "rb").read() == open(d / case["output"], "rb").read()
    assert open(out + ".frq", "rb").read() == open(str(d / case["output"]) + ".frq", "rb").read()


@pytest.mark.parametrize("chunks", [2, 3, 7, 64])
@pytest.mark.parametrize("name", sorted(n for n, c in MANIFEST.items()
                                        if "-s" not in c["args"] and "-p" not in c["args"]
                                        and "-f" not in c["args"]))
def test_engine_parse_in_chunks(tmp_path, monkeypatch, name, chunks):
    """The FASTA parser cut into several chunks (parsed in parallel, then
    stitched) reads the same records as in one pass."""
    case = MANIFEST[name]
    d = _case_dir(tmp_path, name)
    monkeypatch.setenv("CRISPY_PARSE_CHUNKS", str(chunks))
    raw = cg.RawReads(str(d / case["input"]))
    monkeypatch.delenv("CRISPY_PARSE_CHUNKS")
    one = cg.RawReads(str(d / case["input"]))
    assert raw.records == one.records == case["total"] and raw.n == one.n
    for i in range(raw.n):
        assert raw.seq(i) == one.seq(i) and raw.label(i) == one.label(i)
    index, freq = _host_sort_merge(raw)
    out = str(d / "engine_out")
    raw.write(index, freq, out)
    assert open(out, "rb").read() == open(d / case["output"], "rb").read()


def _boundary_fasta(rng):
    """Records whose shapes meet chunk cuts: empty records, blank and
    whitespace lines, a header longer than one fgets piece, lines of
    exactly 4095 bytes, a '$' line late in the file."""
    out = bytearray()
    for i in range(400):
        kind = i % 9
        out += b">rec_%d some words\n" % i
        if kind == 1:
            continue                                   # header without sequence
        s = rng.choice(np.frombuffer(b"ACGTNacgt", np.uint8), size=int(rng.integers(1, 300))).tobytes()
        if kind == 2:
            out += s[:50] + b"\n\n" + s[50:] + b"\n"    # blank line inside
        elif kind == 3:
            out += s + b"  \t\n   \n"                  # trailing whitespace lines
        elif kind == 4:
            out += b"C" * 4095 + b"\n" + s + b"\n"      # a line of exactly one piece
        elif kind == 5 and i % 2:
            out = out[:-1] + b"H" * 4200 + b"\n" + s + b"\n"   # header beyond one piece
        else:
            out += s + b"XX\n"
    return bytes(out)


@pytest.mark.parametrize("chunks", [1, 2, 5, 13, 40])
def test_parse_chunk_boundaries_vs_oracle(tmp_path, monkeypatch, chunks):
    rng = np.random.default_rng(chunks)
    p = tmp_path / "b.fa"
    p.write_bytes(_boundary_fasta(rng))
    monkeypatch.setenv("CRISPY_PARSE_CHUNKS", str(chunks))
    raw = cg.RawReads(str(p))
    index, freq = _host_sort_merge(raw)
    raw.write(index, freq, str(tmp_path / "eng"))
    c = oracle.preprocess(str(p), str(tmp_path / "ora"))
    assert raw.records == c["records"]
    for e in ("", ".frq"):
        assert open(str(tmp_path / "eng") + e, "rb").read() == open(str(tmp_path / "ora") + e, "rb").read()
    # a '$' line ends the input in every chunking
    q = tmp_path / "d.fa"
    data = _boundary_fasta(rng)
    cut = data.index(b">rec_300 ")
    q.write_bytes(data[:cut] + b"$ stop\n" + data[cut:])
    raw = cg.RawReads(str(q))
    index, freq = _host_sort_merge(raw)
    raw.write(index, freq, str(tmp_path / "eng2"))
    c = oracle.preprocess(str(q), str(tmp_path / "ora2"))
    assert raw.records == c["records"]
    assert open(str(tmp_path / "eng2"), "rb").read() == open(str(tmp_path / "ora2"), "rb").read()


def test_raw_load_errors(tmp_path):
    with pytest.raises(cg.CrispyError):
        cg.RawReads(str(tmp_path / "missing.fa"))
    p = tmp_path / "notfasta.fa"
    p.write_bytes(b"ACGT\n>a\nACGT\n")
    with pytest.raises(cg.CrispyError):
        cg.RawReads(str(p))
    p.write_bytes(b"")
    with pytest.raises(cg.CrispyError):
        cg.RawReads(str(p))
