"""The overlapped load-and-count call (mp_job_load_count): pinned input goes up in segments of whole chunks
while the segments already in HBM are parsed and counted.  Its histogram, reads per chunk, stage dumps,
labels, bounds and partition files equal those of the load and count calls made one after the other, and
so do its errors; pageable input and the 3-minimizer variant take the one-after-the-other path."""
import re

import numpy as np
import pytest

from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu

# (workload, reads, k, chunks, scans, threads, interleaved)
CASES = [
    ("plain_small", 40000, 31, 16, 2, 2, False),
    ("plain_large", 60000, 27, 32, 2, 4, False),
    ("interleaved_small", 30000, 27, 16, 2, 2, True),
    ("hotspot", 30000, 25, 12, 1, 2, False),
]


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


def _pinned(data: bytes):
    import torch
    return torch.frombuffer(bytearray(data), dtype=torch.uint8).pin_memory()


def _starts(files, chunks, il):
    fno, ofs = native.fastq_index(chunks, files, il)
    return native.chunk_starts_of(fno, ofs, [len(f) for f in files])


def _run(ctx, files, k, chunks, scans, threads, il, how, dump=None, min3=False):
    data = b"".join(files)
    sizes = [len(f) for f in files]
    starts = _starts(files, chunks, il)
    job = native.Job(ctx)
    try:
        if dump:
            dump.mkdir()
            job.set_dump_dir(str(dump))
        if how == "steps":
            job.load(data, file_sizes=sizes, interleaved=il)
            cnt = job.count(k, starts, min3)
        else:
            buf = _pinned(data) if how == "pinned" else np.frombuffer(bytearray(data), dtype=np.uint8)
            ptr = buf.data_ptr() if how == "pinned" else buf.ctypes.data
            cnt = job.load_count(ptr, len(data), k, starts, min3=min3, interleaved=il, file_sizes=sizes)
        pieces = job.kmer_cache_pieces
        bounds = job.partition(k, scans, threads, starts, cnt.chunk_first_read, cnt.hist, min3)
        out, fsz = job.output()
        return dict(hist=cnt.hist.copy(), reads=cnt.chunk_reads.copy(), out=bytes(out), sizes=fsz.copy(),
                    bounds=bounds.copy(), labels=job.labels(), pieces=pieces)
    finally:
        job.close()


def _same(a, b):
    for key in ("hist", "reads", "sizes", "bounds", "labels"):
        assert np.array_equal(a[key], b[key]), key
    assert a["out"] == b["out"]


@pytest.mark.parametrize("name,n,k,chunks,scans,threads,il", CASES, ids=[f"{c[0]}-k{c[2]}" for c in CASES])
def test_overlapped_equals_steps(ctx, tmp_path, name, n, k, chunks, scans, threads, il):
    data = synth.fastq_bytes(synth.workload(name, n, seed=31))
    a = _run(ctx, [data], k, chunks, scans, threads, il, "pinned", tmp_path / "a")
    b = _run(ctx, [data], k, chunks, scans, threads, il, "steps", tmp_path / "b")
    assert a["pieces"] > 1 and b["pieces"] == 1  # the segmented path ran
    _same(a, b)
    da = sorted(p.name for p in (tmp_path / "a").iterdir())
    assert da == sorted(p.name for p in (tmp_path / "b").iterdir()) and da
    for f in da:
        assert (tmp_path / "a" / f).read_bytes() == (tmp_path / "b" / f).read_bytes(), f


def test_two_files(ctx):
    recs = synth.fastq_bytes(synth.workload("plain_small", 30000, seed=32)).split(b"\n")
    cut = 4 * 11000
    f1, f2 = b"\n".join(recs[:cut]) + b"\n", b"\n".join(recs[cut:])
    a = _run(ctx, [f1, f2], 29, 16, 2, 2, False, "pinned")
    b = _run(ctx, [f1, f2], 29, 16, 2, 2, False, "steps")
    assert a["pieces"] > 1
    _same(a, b)


def test_pageable_and_min3_take_the_steps(ctx):
    data = synth.fastq_bytes(synth.workload("plain_small", 20000, seed=33))
    a = _run(ctx, [data], 31, 8, 1, 2, False, "pageable")
    b = _run(ctx, [data], 31, 8, 1, 2, False, "steps")
    assert a["pieces"] == 1
    _same(a, b)
    m = _run(ctx, [data], 31, 8, 1, 2, False, "pinned", min3=True)
    s = _run(ctx, [data], 31, 8, 1, 2, False, "steps", min3=True)
    assert m["pieces"] == 0
    _same(m, s)


def _error(fn):
    with pytest.raises(native.MetapartError) as e:
        fn()
    return re.sub(r"^\w+ failed", "", str(e.value))


def _both_fail_alike(ctx, d, st):
    def steps():
        job = native.Job(ctx)
        try:
            job.load(d)
            job.count(31, st)
        finally:
            job.close()

    def overlapped():
        job = native.Job(ctx)
        h = _pinned(d)
        try:
            job.load_count(h.data_ptr(), len(d), 31, st)
        finally:
            job.close()

    assert _error(overlapped) == _error(steps)


def test_bad_record_in_a_later_segment(ctx):
    lines = synth.fastq_bytes(synth.workload("plain_small", 30000, seed=34)).split(b"\n")
    q = 4 * 20000 + 3  # a quality line two thirds in, one character short
    lines[q] = lines[q][:-1]
    bad = b"\n".join(lines)
    _both_fail_alike(ctx, bad, _starts([bad], 16, False))


def test_chunk_start_off_a_record(ctx):
    data = synth.fastq_bytes(synth.workload("plain_small", 30000, seed=35))
    st = _starts([data], 16, False)
    st[5] += 1
    _both_fail_alike(ctx, data, st)


def test_output_into_pinned_memory(ctx):
    """Partition files built batch by batch, each batch copied down while the next is built, equal those
    built whole and copied at once."""
    import torch
    data = synth.fastq_bytes(synth.workload("interleaved_small", 20000, seed=36))
    job, _, _ = native.run_pipeline(ctx, data, 27, 8, 2, 2, interleaved=True)
    try:
        sizes, total = job.output_plan()
        pinned = torch.zeros(total + 16, dtype=torch.uint8).pin_memory()
        assert job.output_to(pinned.data_ptr(), pinned.numel()) == total
        via_hbm, sizes2 = job.output()  # the files already in HBM: one copy
        assert bytes(pinned[:total].numpy()) == bytes(via_hbm) and np.array_equal(sizes, sizes2)
        job.prepare_output()
        again = torch.zeros(total + 16, dtype=torch.uint8).pin_memory()
        job.output_to(again.data_ptr(), again.numel())
        assert bytes(again[:total].numpy()) == bytes(via_hbm)
    finally:
        job.close()


def _edge_reads(n, seed, k):
    """The golden set's edge-case reads: lengths around k up to the longest read, N runs, poly-A/T,
    palindromes, duplicates, lowercase and IUPAC bytes."""
    import importlib.util
    from pathlib import Path
    spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).resolve().parent / "golden" /
                                                  "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.edge_fastq(n, seed, k, False)


@pytest.mark.parametrize("k", [31, 21])
def test_edge_reads(ctx, tmp_path, k):
    data = _edge_reads(6000, 40 + k, k)
    a = _run(ctx, [data], k, 16, 2, 2, False, "pinned", tmp_path / "a")
    b = _run(ctx, [data], k, 16, 2, 2, False, "steps", tmp_path / "b")
    assert a["pieces"] > 1
    _same(a, b)
    for f in sorted(p.name for p in (tmp_path / "a").iterdir()):
        assert (tmp_path / "a" / f).read_bytes() == (tmp_path / "b" / f).read_bytes(), f


def test_device_bytes_used_in_place(ctx):
    """Reads already in device memory used where they are give the results of an upload."""
    import torch
    data = synth.fastq_bytes(synth.workload("plain_small", 20000, seed=37))
    starts = _starts([data], 8, False)
    dev = torch.zeros(len(data) + 64, dtype=torch.uint8, device="cuda")
    dev[:len(data)].copy_(torch.frombuffer(bytearray(data), dtype=torch.uint8))
    res = []
    for inplace in (True, False):
        job = native.Job(ctx)
        try:
            if inplace:
                job.load_device_inplace(dev.data_ptr(), len(data))
            else:
                job.load(data)
            cnt = job.count(31, starts)
            bounds = job.partition(31, 2, 2, starts, cnt.chunk_first_read, cnt.hist)
            out, sizes = job.output()
            res.append((cnt.hist.copy(), bytes(out), sizes.copy(), bounds.copy(), job.labels()))
        finally:
            job.close()
    assert np.array_equal(res[0][0], res[1][0]) and res[0][1] == res[1][1]
    for x, y in zip(res[0][2:], res[1][2:]):
        assert np.array_equal(x, y)
    assert torch.count_nonzero(dev[len(data):]) == 0  # the caller's bytes are untouched
    job = native.Job(ctx)
    try:
        with pytest.raises(native.MetapartError):
            job.load_device_inplace(dev.data_ptr() + 1, len(data) - 1)  # not 16-byte aligned
    finally:
        job.close()
