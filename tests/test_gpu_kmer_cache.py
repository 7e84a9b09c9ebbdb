"""The count pass's k-mer cache: a job that counts and partitions in one go (cache on) gives every stage
dump, label and partition file byte-identical to the same job with the cache off (k-mers recomputed from
the reads, the path the drop-in programs take and the parity tests pin to the oracle)."""
import numpy as np
import pytest

from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu

CASES = [
    ("plain_small", 20000, 27, 4, 1, 2, False),
    ("plain_large", 30000, 31, 8, 2, 4, False),
    ("plain_small", 12000, 25, 6, 3, 3, False),
    ("hotspot", 30000, 31, 4, 1, 2, False),
    ("interleaved_small", 20000, 27, 4, 2, 2, True),
    ("plain_small", 8000, 11, 4, 2, 2, False),
]


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


def _run(ctx, data, k, chunks, scans, threads, il, cache, d):
    d.mkdir()
    job, bounds, _ = native.run_pipeline(ctx, data, k, chunks, scans, threads, interleaved=il, dump_dir=str(d),
                                         kmer_cache=cache)
    try:
        out, sizes = job.output()
        return bytes(out), sizes.copy(), bounds.copy(), job.labels()
    finally:
        job.close()


@pytest.mark.parametrize("name,n,k,chunks,scans,threads,il", CASES,
                         ids=[f"{c[0]}-k{c[2]}-s{c[4]}" for c in CASES])
def test_cache_matches_recomputed(ctx, tmp_path, name, n, k, chunks, scans, threads, il):
    data = synth.fastq_bytes(synth.workload(name, n, seed=21))
    a = _run(ctx, data, k, chunks, scans, threads, il, True, tmp_path / "on")
    b = _run(ctx, data, k, chunks, scans, threads, il, False, tmp_path / "off")
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        assert np.array_equal(x, y)
    on = sorted(p.name for p in (tmp_path / "on").iterdir())
    off = sorted(p.name for p in (tmp_path / "off").iterdir())
    assert on == off and any(x.endswith("_enum.bin") for x in on)
    for f in on:
        assert (tmp_path / "on" / f).read_bytes() == (tmp_path / "off" / f).read_bytes(), f
