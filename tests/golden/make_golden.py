"""Regenerates tests/golden/golden.json from the reference programs (oracle/_ref, built by oracle/build_ref.sh).

For every case the input FASTQ is generated here (seeded synthetic read sets, or the edge-case set below),
the reference's genFastqIdx / genHistograms_metapart[min] / metapart[min] run on it with stage dumps on,
and the SHA-256 of every output (index files with padding masked, histogram, stage dumps, partition files)
is recorded together with the SHA-256 of the input.  The bundled reference fixture (data/reads.fastq) is
used when the reference tree is present; its bytes are not stored, only the digests of the outputs.

    python tests/golden/make_golden.py [REFERENCE_ROOT] [--only CASE ...]

With --only, the named cases are regenerated and the others kept as they are in golden.json.
"""
from __future__ import annotations

import hashlib
import os
import json
import random
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import pipeline_util as pu  # noqa: E402

CASES = {
    "se_k27": dict(gen=("plain_small", 4000, 5), p=dict(k=27, chunks=4, scans=1, threads=2)),
    "se_k31_s2": dict(gen=("plain_large", 6000, 5), p=dict(k=31, chunks=4, scans=2, threads=2)),
    "se_k25_s3_t3": dict(gen=("plain_small", 6000, 6), p=dict(k=25, chunks=6, scans=3, threads=3)),
    "min3_k31": dict(gen=("min3", 3000, 5), p=dict(k=31, chunks=4, scans=1, threads=2, min3=True)),
    "min3_k19": dict(gen=("plain_small", 4000, 8), p=dict(k=19, chunks=4, scans=1, threads=4, min3=True)),
    "il_k27": dict(gen=("interleaved_small", 4000, 5), p=dict(k=27, chunks=4, scans=1, threads=2, interleaved=True)),
    "il_k21_s2": dict(gen=("interleaved_small", 4000, 6), p=dict(k=21, chunks=8, scans=2, threads=4,
                                                                 interleaved=True)),
    "edge_k31": dict(gen=("edge", 2000, 9), p=dict(k=31, chunks=4, scans=1, threads=2)),
    "edge_k15_s2": dict(gen=("edge", 2000, 10), p=dict(k=15, chunks=4, scans=2, threads=2)),
    "edge_min3_k21": dict(gen=("edge", 2000, 11), p=dict(k=21, chunks=4, scans=1, threads=2, min3=True)),
    # the scan's first read is BAD and its last run is a thread range's first valid run (BAD_ANCHOR below)
    "bad_anchor_k27": dict(gen=("bad_anchor", 0, 0), p=dict(k=27, chunks=4, scans=1, threads=1)),
    "bad_anchor_k27_t2": dict(gen=("bad_anchor", 0, 0), p=dict(k=27, chunks=4, scans=1, threads=2)),
    "bad_anchor_k27_s2": dict(gen=("bad_anchor", 1, 0), p=dict(k=27, chunks=4, scans=2, threads=1)),
    "bad_anchor_k27_s2_t2": dict(gen=("bad_anchor", 1, 0), p=dict(k=27, chunks=4, scans=2, threads=2)),
    "bundled_k27": dict(gen=("bundled", 0, 0), p=dict(k=27, chunks=4, scans=1, threads=2, interleaved=True)),
    "bundled_min3_k27": dict(gen=("bundled", 0, 0), p=dict(k=27, chunks=4, scans=1, threads=2, interleaved=True,
                                                          min3=True)),
}


def edge_fastq(n: int, seed: int, k: int, min3: bool) -> bytes:
    """Reads that exercise the edges: lengths below/at/just above k and up to the longest read the
    reference handles (254 + k bases: at most 255 k-mers per read, the reference's 8-bit counter; 299 + k
    for the 3-minimizer variant, its lastKmerPos < 300 assert), N runs, poly-A and poly-T, palindromic
    segments, duplicated reads (long equal-k-mer runs), lowercase and IUPAC bytes."""
    rnd = random.Random(seed)
    genome = "".join(rnd.choice("ACGT") for _ in range(20000))
    recs = []
    top = 299 + k if min3 else 254 + k
    lengths = [L for L in (8, 14, 15, 16, 20, 21, 22, 30, 31, 32, 33, 60, 100, 150, 250, 268, 285, 300, 314, 329,
                           330) if L <= top] + [top]
    for i in range(n):
        kind = rnd.randrange(10)
        L = rnd.choice(lengths)
        if kind == 0:
            s = "A" * L
        elif kind == 1:
            s = "T" * (L // 2) + "A" * (L - L // 2)
        elif kind == 2:
            p = rnd.randrange(0, 19000)
            s = genome[p:p + L]
            s = s.ljust(L, "C")
        elif kind == 3:  # duplicates of one hot segment
            s = genome[5000:5000 + L].ljust(L, "G")
        elif kind == 4:  # N runs
            p = rnd.randrange(0, 19000)
            b = list(genome[p:p + L].ljust(L, "A"))
            for _ in range(rnd.randrange(1, 4)):
                b[rnd.randrange(L)] = "N"
            s = "".join(b)
        elif kind == 5:  # exotic bytes
            p = rnd.randrange(0, 19000)
            b = list(genome[p:p + L].ljust(L, "T"))
            for _ in range(rnd.randrange(1, 4)):
                b[rnd.randrange(L)] = rnd.choice("acgtnRYKMSWHBVD")
            s = "".join(b)
        elif kind == 6:  # palindrome
            h = genome[rnd.randrange(0, 19000):][: (L + 1) // 2]
            comp = {"A": "T", "C": "G", "G": "C", "T": "A"}
            s = (h + "".join(comp[c] for c in reversed(h)))[:L]
            s = s.ljust(L, "A")
        else:
            p = rnd.randrange(0, 19000)
            b = list(genome[p:p + L].ljust(L, "G"))
            for _ in range(rnd.randrange(0, 3)):
                b[rnd.randrange(L)] = rnd.choice("ACGT")
            s = "".join(b)
        q = "".join(rnd.choice("#$%&'()*,-./0123456789:;<=>?@ABCDEFGHIJ") for _ in range(L))
        recs.append(f"@e{i} x\n{s}\n+\n{q}\n")
    return "".join(recs).encode()


BAD_ANCHOR = ("first", "two_scans", "last")


def bad_anchor_fastq(variant: int) -> bytes:
    """A BAD read as the scan's first tuple's read while a thread range's first valid run is the scan's
    last run, so that the sweep's initial state unites that run with a BAD read.  Four poly-A reads end in
    C, G, T, C: their last all-A k-mer has another next base than the poly-A run's majority, which flags
    them BAD, and the first of them holds the scan's first tuple (the all-A k-mer).  Four poly-C reads hold
    the scan's last k-mer; every tuple before them has a BAD read or the k-mer 0, so the poly-C run is the
    first valid run of its range.  "two_scans" adds eight (GC)* reads, whose k-mers sort above poly-C and
    fill a second scan.  "last" puts the poly-C reads first, so that the BAD read's id is above the run's
    root."""
    L = 100
    bad = ["A" * (L - 1) + c for c in "CGTC"]
    poly_c = ["C" * L] * 4
    gc = [("GC" * L)[:L]] * 8
    reads = {"first": bad + poly_c, "two_scans": bad + poly_c + gc, "last": poly_c + bad}[BAD_ANCHOR[variant]]
    return "".join(f"@b{i}\n{s}\n+\n{'I' * len(s)}\n" for i, s in enumerate(reads)).encode()


def make_input(gen, ref_root: Path, k: int, min3: bool = False) -> bytes | None:
    from metapart_gb300 import synth
    name, n, seed = gen
    if name == "bundled":
        f = ref_root / "data" / "reads.fastq" if ref_root else None
        return f.read_bytes() if f and f.exists() else None
    if name == "edge":
        return edge_fastq(n, seed, k, min3)
    if name == "bad_anchor":
        return bad_anchor_fastq(n)
    return synth.fastq_bytes(synth.workload(name, n, seed=seed))


def params(d: dict) -> pu.Params:
    return pu.Params(**d)


def main():
    from metapart_gb300 import build
    build.build_synth()
    args = sys.argv[1:]
    only = args[args.index("--only") + 1:] if "--only" in args else None
    if only is not None:
        args = args[:args.index("--only")]
    if args:
        os.environ["MP_REFERENCE_ROOT"] = args[0]
    if not build.build_reference(force=bool(args)):
        raise SystemExit("reference sources not found: cannot regenerate golden digests")
    ref_root = build.reference_root()
    out = json.loads((HERE / "golden.json").read_text()) if only else {}
    for name, c in CASES.items():
        if only and name not in only:
            continue
        data = make_input(c["gen"], ref_root, c["p"]["k"], c["p"].get("min3", False))
        if data is None:
            continue
        p = params(c["p"])
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            fq = td / "in.fastq"
            fq.write_bytes(data)
            d = pu.run("ref", td, [fq], p)
            res = pu.outputs(d, p, "in.fastq")
        out[name] = {"gen": list(c["gen"]), "params": c["p"], "input_sha256": hashlib.sha256(data).hexdigest(),
                     "outputs": pu.digests(res)}
        print(name, len(res), "outputs")
    (HERE / "golden.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
