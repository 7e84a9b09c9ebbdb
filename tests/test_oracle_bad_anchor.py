"""A BAD read as a sweep's initial anchor, with the expected outputs written out.

A thread range's union sweep starts from the scan's last k-mer and the scan's first tuple's read
(metapart.c:2539-2545).  When that read is BAD and the range's first valid run is the scan's last run,
the reference unites the run with the BAD read: findRoot returns a BAD-parented read as its own root
(unionfind.h:25) and the hook goes below the larger id (metapart.c:2680-2700).  The inputs are
tests/golden/make_golden.py's bad_anchor_fastq (reads 0-3 poly-A with a branching last base, BAD; reads
4-7 poly-C, the scan's last k-mer; in "two_scans" reads 8-15 (GC)*, a second scan):

- "first", 1 or 2 threads: read 0 (the first tuple's read, BAD) is hooked below the poly-C component's
  root 7 and is a member from then on: after the scan the parents are 7 BAD BAD BAD 7 7 7 7; the mate
  union then pairs read 1 with read 0's component and reads 2, 3 together: 7 7 3 3 7 7 7 7.
- "two_scans": the first scan does the same; the second marks read 0 BAD again (it is flagged:
  metapart.c:2503-2516), so the mate union pairs it with read 1: 1 1 3 3 7 7 7 7 15 x 8.
- "last": the BAD read (4) is above the run's root (3), so the run's root goes below the BAD read, which
  keeps its BAD parent; the reference's edge replay then stops on its assertion (metapart.c:2772), and the
  oracle reports the same as an error.

The oracle is checked against these arrays; the reference itself (when oracle/_ref is built) gives the
same for the first two inputs (their digests are in golden.json) and aborts on the last.
"""
import importlib.util
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pipeline_util as pu

HERE = Path(__file__).resolve().parent
BADV = 0xBADBADBAD


def _mg():
    spec = importlib.util.spec_from_file_location("make_golden", HERE / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def parents(path: Path) -> list:
    """A parent dump (5 bytes per read: the quotient by 2^32 - 1, then the remainder) as values, BAD as "B"."""
    raw = np.fromfile(path, np.uint8).reshape(-1, 5)
    rem = raw[:, 1:].copy().view("<u4").ravel().astype(np.uint64)
    val = raw[:, 0].astype(np.uint64) * np.uint64(0xFFFFFFFF) + rem
    return ["B" if int(v) == BADV else int(v) for v in val]


B = "B"
EXPECT = {
    # variant, threads, scans -> {dump: parents}
    ("first", 1, 1): {"stats0_parent.bin": [7, B, B, B, 7, 7, 7, 7], "stats2_parent.bin": [7, 7, 3, 3, 7, 7, 7, 7]},
    ("first", 2, 1): {"stats0_parent.bin": [7, B, B, B, 7, 7, 7, 7], "stats2_parent.bin": [7, 7, 3, 3, 7, 7, 7, 7]},
    ("two_scans", 1, 2): {"stats0_parent.bin": [7, B, B, B, 7, 7, 7, 7] + list(range(8, 16)),
                          "stats1_parent.bin": [B, B, B, B, 7, 7, 7, 7] + [15] * 8,
                          "stats3_parent.bin": [1, 1, 3, 3, 7, 7, 7, 7] + [15] * 8},
    ("two_scans", 2, 2): {"stats0_parent.bin": [7, B, B, B, 7, 7, 7, 7] + list(range(8, 16)),
                          "stats1_parent.bin": [B, B, B, B, 7, 7, 7, 7] + [15] * 8,
                          "stats3_parent.bin": [1, 1, 3, 3, 7, 7, 7, 7] + [15] * 8},
}


def _run(impl, tmp_path, variant, threads, scans):
    mg = _mg()
    fq = tmp_path / "in.fastq"
    fq.write_bytes(mg.bad_anchor_fastq(mg.BAD_ANCHOR.index(variant)))
    p = pu.Params(k=27, chunks=4, scans=scans, threads=threads)
    return pu.run(impl, tmp_path, [fq], p, dump=True)


@pytest.mark.parametrize("variant,threads,scans", sorted(EXPECT))
def test_oracle_bad_anchor_outputs(tmp_path, built, variant, threads, scans):
    d = _run("oracle", tmp_path, variant, threads, scans)
    dumps = {f.name: f for f in d.rglob("stats*_parent.bin")}
    for name, want in EXPECT[(variant, threads, scans)].items():
        assert parents(dumps[name]) == want, name


def test_oracle_bad_anchor_above_root_is_the_reference_assertion(tmp_path, built):
    with pytest.raises(RuntimeError, match=r"metapart\.c:2772"):
        _run("oracle", tmp_path, "last", 1, 1)


def test_reference_aborts_on_bad_anchor_above_root(tmp_path, built):
    if not (pu.ROOT / "oracle" / "_ref" / "metapart_dump").exists():
        pytest.skip("the reference programs are not built on this machine")
    with pytest.raises(RuntimeError, match="Assertion"):
        _run("ref", tmp_path, "last", 1, 1)
