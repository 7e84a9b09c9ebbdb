"""Typed errors through the C ABI for inputs the reference would assert on or misread; after each failure the
context stays usable (no device fault is involved: every check is a host-visible status)."""
import numpy as np
import pytest

from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu

EARG, EFMT, ENOMEM, EUNSUP = -1, -3, -4, -5


def code(e: native.MetapartError) -> int:
    return int(str(e).split("(")[1].split(")")[0])


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


def small(n=400, seed=1):
    return synth.fastq_bytes(synth.workload("plain_small", n, seed=seed))


def test_quality_length_mismatch(ctx):
    bad = small().replace(b"\n+\nIIII", b"\n+\nIII", 1)
    with native.Job(ctx) as j, pytest.raises(native.MetapartError) as e:
        j.load(bad)
    assert code(e.value) == EFMT


def test_truncated_file(ctx):
    with native.Job(ctx) as j, pytest.raises(native.MetapartError) as e:
        j.load(small()[:-5])
    assert code(e.value) == EFMT


def test_chunk_offset_not_a_record_start(ctx):
    data = small()
    with native.Job(ctx) as j:
        j.load(data)
        with pytest.raises(native.MetapartError) as e:
            j.count(27, np.array([0, 17, len(data)], dtype=np.uint64))
        assert code(e.value) == EFMT


def test_k_out_of_range(ctx):
    data = small()
    with native.Job(ctx) as j:
        j.load(data)
        with pytest.raises(native.MetapartError) as e:
            j.count(32, np.array([0, len(data)], dtype=np.uint64))
        assert code(e.value) == EARG


def test_odd_read_count_and_min3_scans(ctx):
    data = small(401)
    fno, ofs = native.fastq_index(1, [data])
    st = native.chunk_starts_of(fno, ofs, [len(data)])
    with native.Job(ctx) as j:
        j.load(data)
        c = j.count(27, st)
        with pytest.raises(native.MetapartError) as e:
            j.partition(27, 1, 1, st, c.chunk_first_read, c.hist)
        assert code(e.value) == EUNSUP
    data = small(400)
    fno, ofs = native.fastq_index(2, [data])
    st = native.chunk_starts_of(fno, ofs, [len(data)])
    with native.Job(ctx) as j:
        j.load(data)
        c = j.count(27, st, min3=True)
        with pytest.raises(native.MetapartError) as e:
            j.partition(27, 2, 1, st, c.chunk_first_read, c.hist, min3=True)
        assert code(e.value) == EUNSUP
        with pytest.raises(native.MetapartError) as e:
            j.partition(27, 1, 3, st, c.chunk_first_read, c.hist, min3=True)   # 3 does not divide 2 chunks
        assert code(e.value) == EARG


def test_read_with_too_many_kmers(ctx):
    rec = b"@x\n" + b"ACGT" * 70 + b"\n+\n" + b"I" * 280 + b"\n"
    data = rec * 4
    st = np.array([0, len(data)], dtype=np.uint64)
    with native.Job(ctx) as j:
        j.load(data)
        c = j.count(21, st)
        with pytest.raises(native.MetapartError) as e:
            j.partition(21, 1, 1, st, c.chunk_first_read, c.hist)
        assert code(e.value) == EUNSUP


def test_hbm_budget_refusal(built_gpu):
    with native.Context(0, hbm_budget=1 << 20) as c, native.Job(c) as j:
        with pytest.raises(native.MetapartError) as e:
            j.load(small(20000))
        assert code(e.value) == ENOMEM


def test_context_usable_after_errors(ctx):
    data = small(2000, seed=9)
    job, bounds, cnt = native.run_pipeline(ctx, data, k=27, num_chunks=4, num_scans=1, num_threads=2)
    with job:
        assert int(bounds[16]) == 2000
        out, sizes = job.output()
        assert int(sizes.sum()) == len(data)


def test_no_kmers_at_all(ctx):
    # every read shorter than k: the reference's range planner crashes on the empty histogram; here it is a
    # typed error from the partition, after a count that reports an all-zero histogram
    recs = b"".join(b"@r%d\n%s\n+\n%s\n" % (i, b"ACGTACGTAC"[: 5 + i % 6], b"I" * (5 + i % 6)) for i in range(40))
    with native.Job(ctx) as j:
        j.load(recs)
        starts = np.array([0, len(recs)], dtype=np.uint64)
        cnt = j.count(27, starts)
        assert int(cnt.hist[-1]) == 0
        with pytest.raises(native.MetapartError) as e:
            j.partition(27, 1, 1, starts, cnt.chunk_first_read, cnt.hist)
        assert code(e.value) == EUNSUP


def test_empty_input(ctx):
    """No bytes at all: a typed error (the index finds no record), never a crash."""
    with native.Job(ctx) as j:
        with pytest.raises(native.MetapartError):
            j.load(b"")
            starts = np.array([0, 0], dtype=np.uint64)
            cnt = j.count(27, starts)
            j.partition(27, 1, 1, starts, cnt.chunk_first_read, cnt.hist)
