"""A BAD read as a sweep's initial anchor on the GPU (the case test_oracle_bad_anchor.py describes).

The whole-scan path is pinned to the reference by the golden digests (bad_anchor_* in golden.json); here
the same inputs go through the other union paths -- scans split into bucket-range pieces, and a batch of
samples -- which must give what the whole-scan job gives, and through the input on which the reference
stops on its replay assertion, where the GPU leaves the BAD read BAD (the edge is not taken) and finishes.
"""
import numpy as np
import pytest

import pipeline_util as pu
from metapart_gb300 import native, synth
from test_gpu_batch import _batched, _check
from test_oracle_bad_anchor import B, _mg, _run as _run_programs, parents

pytestmark = pytest.mark.gpu


def _data(variant):
    mg = _mg()
    return mg.bad_anchor_fastq(mg.BAD_ANCHOR.index(variant))


def _job(ctx, data, scans, threads, cap):
    fno, ofs = native.fastq_index(4, [data])
    starts = native.chunk_starts_of(fno, ofs, [len(data)])
    with native.Job(ctx) as job:
        job.set_scan_piece_tuples(cap)
        job.load(data)
        cnt = job.count(27, starts)
        bounds = job.partition(27, scans, threads, starts, cnt.chunk_first_read, cnt.hist)
        out, sizes = job.output()
        return dict(bounds=bounds.copy(), labels=job.labels(), out=bytes(out), sizes=sizes.copy(),
                    pieces=job.scan_pieces)


@pytest.mark.parametrize("variant,scans,threads", [("first", 1, 1), ("first", 1, 2), ("two_scans", 2, 1),
                                                   ("two_scans", 2, 2)])
def test_bad_anchor_in_pieces(built_gpu, variant, scans, threads):
    data = _data(variant)
    with native.Context(0) as ctx:
        whole = _job(ctx, data, scans, threads, 0)
        split = _job(ctx, data, scans, threads, 300)  # the poly-A and poly-C buckets hold 296 tuples each
    assert whole["pieces"] == scans and split["pieces"] > scans
    for key in ("bounds", "labels", "sizes"):
        assert np.array_equal(whole[key], split[key]), key
    assert whole["out"] == split["out"]
    # read 0 (BAD in the first scan) ends in the poly-C component with one scan, with its mate with two
    want = [7, 7, 3, 3, 7, 7, 7, 7] if scans == 1 else [1, 1, 3, 3, 7, 7, 7, 7] + [15] * 8
    assert whole["labels"].tolist() == want


def test_bad_anchor_in_a_batch(built_gpu):
    datas = [synth.fastq_bytes(synth.workload("plain_small", 6000, seed=4)), _data("first"), _data("first"),
             _data("two_scans")]
    shapes = [(4, 2), (4, 1), (4, 2), (4, 1)]
    with native.Context(0) as ctx:
        res, outs, fs, labs, groups = _batched(ctx, datas, shapes, 27)
        assert groups == 1
        _check(ctx, datas, shapes, 27, res, outs, fs, labs)
    assert labs[1][:8].tolist() == [7, 7, 3, 3, 7, 7, 7, 7]


def test_bad_anchor_above_root_leaves_it_bad(tmp_path, built_gpu):
    """The reference asserts on this input (metapart.c:2772); the GPU programs finish with the BAD read
    (4) left out of the poly-C component (reads 0-3, root 3); the mate union then pairs 4 with 5, 6 with 7."""
    d = _run_programs("gpu", tmp_path, "last", 1, 1)
    dumps = {f.name: f for f in d.rglob("stats*_parent.bin")}
    assert parents(dumps["stats0_parent.bin"]) == [3, 3, 3, 3, B, B, B, B]
    assert parents(dumps["stats2_parent.bin"]) == [3, 3, 3, 3, 5, 5, 7, 7]
