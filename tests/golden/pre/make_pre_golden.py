"""Regenerate the preprocess fixtures from the reference's own preprocess.

Needs the reference tree: `make -C oracle ref` compiles
src/preprocess/preprocess.cpp as it lies into oracle/_ref/preprocess.  Each
case is an input file (written here from a seed or by hand, to hit one
behaviour of preprocess.cpp) plus a command line; the reference's outputs
<input>_Clean and <input>_Clean.frq and its "Total numReads" line are kept
under tests/golden/pre/<case>/, and MANIFEST.json lists every case with the
SHA-256 of its files.

Run:  python tests/golden/pre/make_pre_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, ROOT)

from crispy_gb300 import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "preprocess")


def wrap_fasta(reads, labels, width=60, eol=b"\n"):
    out = bytearray()
    for lab, s in zip(labels, reads):
        out += lab + eol
        for a in range(0, len(s), width):
            out += s[a:a + width] + eol
    return bytes(out)


def dup_set(seed: int, n: int = 200):
    """Seeded 16S-like reads with planted duplicates, N's and lower case."""
    spec = synth.ReadSetSpec(n, 6, 260, "normal", 120, 6, 6, seed)
    reads = synth.generate(spec)
    rng = np.random.default_rng(seed)
    # a third of the reads again, at random places
    extra = [reads[i] for i in rng.integers(0, len(reads), size=n // 3)]
    reads = reads + extra
    order = rng.permutation(len(reads))
    reads = [bytearray(reads[i]) for i in order]
    for r in reads:
        u = rng.random()
        if u < 0.04:
            r[rng.integers(0, len(r))] = ord("N")
        elif u < 0.06:
            r[rng.integers(0, len(r))] = ord("n")
        elif u < 0.08:
            a = rng.integers(0, len(r))
            r[a:a + 5] = r[a:a + 5].lower()
    labels = [b">read_%d sample=%d\tpos %d" % (i, seed, i * 7) for i in range(len(reads))]
    primer = bytes(reads[0][:20]).upper()
    return [bytes(r) for r in reads], labels, primer


def edge_fasta() -> bytes:
    long_seq = (b"ACGT" * 1300)[:5000]
    parts = [
        b">first header with  spaces\r\n", b"ACGTACGTAC\r\n", b"GGTTAACC\n",
        b"\n",                                   # blank line inside a record
        b"TTGA\n",
        b">second\n", b"ACGTTTGA\n",
        b">empty_one\n",                         # no sequence: label kept from here
        b">empty_two\n",
        b"ACGTTTGA\n",                           # duplicate of 'second'
        b">trailing junk\n", b"ACGTXX12\n", b"CCGGNN??\n",
        b">only junk\n", b"XYZ\n",
        b">ws only line\n", b"ACG\n", b"   \n", b"TTT\n",
        b">long line\n", long_seq + b"\n",
        b">" + b"H" * 4200 + b"\n", b"GATTACA\n",  # header longer than one piece
        b">exact piece\n", b"C" * 4095 + b"\n",
        b">lower\n", b"acgtacgtNNac\n",
        b">tab\theader\n", b"ACGTTTGA\n",
        b">last no newline\n", b"GGGCCCAAATTT",
    ]
    return b"".join(parts)


def dollar_fasta() -> bytes:
    return b">a\nACGTACGT\n>b\nACGTACGA\n$stops here\n>c\nACGTACGT\n"


def fastq_text(seed: int) -> bytes:
    rng = np.random.default_rng(seed)
    out = bytearray()
    base = [bytes(rng.choice(list(b"ACGT"), size=rng.integers(30, 40))) for _ in range(25)]
    for i in range(80):
        s = base[rng.integers(0, len(base))]
        out += b"@q%d extra\n" % i + s + b"\n+\n" + b"I" * len(s) + b"\n"
    out += b"@tail\r\nACGTAC\r\n+\r\nIIIIII"   # CRLF, no final newline
    return bytes(out)


CASES = {
    # name: (input name, builder, argv after -i <input>, primer text or None)
    "dups": ("dups.fa", lambda: wrap_fasta(*dup_set(7)[:2]), [], None),
    "dups_s1": ("dups.fa", lambda: wrap_fasta(*dup_set(7)[:2]), ["-s", "1.0"], None),
    "dups_s05_p": ("dups.fa", lambda: wrap_fasta(*dup_set(7)[:2]), ["-s", "0.5", "-m", "2"], "primer"),
    "dups_p_m0": ("dups.fa", lambda: wrap_fasta(*dup_set(7)[:2]), ["-m", "0"], "primer"),
    "dups_neg_s": ("dups.fa", lambda: wrap_fasta(*dup_set(11)[:2]), ["-s", "-2"], None),
    "edge": ("edge.fa", edge_fasta, [], None),
    "edge_s": ("edge.fa", edge_fasta, ["-s", "3"], None),
    "dollar": ("dollar.fa", dollar_fasta, [], None),
    "fastq": ("reads.fq", lambda: fastq_text(5), ["-f", "q"], None),
    "out_name": ("dups.fa", lambda: wrap_fasta(*dup_set(3)[:2]), ["-o", "custom_out"], None),
}


def main():
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/preprocess is not built: make -C oracle ref (needs the reference tree)")
    manifest = {}
    for name, (inp, build, argv, primer) in CASES.items():
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        tmp = tempfile.mkdtemp()
        try:
            with open(os.path.join(tmp, inp), "wb") as f:
                f.write(build())
            args = ["-i", inp] + list(argv)
            if primer is not None:
                seed = 7
                with open(os.path.join(tmp, "primer.txt"), "wb") as f:
                    f.write(dup_set(seed)[2] + b"\n")
                args += ["-p", "primer.txt"]
            p = subprocess.run([REF] + args, cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if p.returncode != 1:   # preprocess ends with `return 1`
                raise RuntimeError(f"{name}: reference returned {p.returncode}\n{p.stdout!r}")
            m = re.search(rb"Total numReads: (-?\d+)\. Preprocessed numReads: (-?\d+)", p.stdout)
            out = "custom_out" if "-o" in argv else inp + "_Clean"
            files = [inp, out, out + ".frq"] + (["primer.txt"] if primer is not None else [])
            for fn in files:
                shutil.copy(os.path.join(tmp, fn), os.path.join(d, fn))
            manifest[name] = {
                "input": inp, "args": args, "output": out,
                "total": int(m.group(1)), "preprocessed": int(m.group(2)),
                "files": {fn: hashlib.sha256(open(os.path.join(d, fn), "rb").read()).hexdigest()
                          for fn in files},
            }
        finally:
            shutil.rmtree(tmp)
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("wrote", len(manifest), "cases")


if __name__ == "__main__":
    main()
