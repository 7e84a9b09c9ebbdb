"""Batches (mp_batch_run): every sample of a batch gets exactly what it gets alone.

Each sample is partitioned alone through the job calls (mp_job_count + mp_job_partition with one scan +
mp_job_output, the path the parity tests pin to the oracle) and then in a batch with the others; its 16
bounds, every read's component label and every partition file must be equal byte for byte.  The mixes hold
samples of different sizes, read lengths and thread counts, an abundant one (oversized m-mer buckets, long
runs), and two samples made only of poly-C reads back to back, whose single k-mer is both the last tuple
of the first and the first tuple of the second (a run the sweeps must not carry across samples).  Batches
are also forced into several groups, and two samples' partition files are compared with the CPU oracle's
directly.  Errors name the sample.
"""
import os

import numpy as np
import pytest

import pipeline_util as pu
from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu


def _poly_c(n_reads, L=100):
    rec = b"".join(b"@c%d\n" % i + b"C" * L + b"\n+\n" + b"I" * L + b"\n" for i in range(n_reads))
    return rec


def _mix(seed):
    specs = synth.batch_mix(6, seed=seed, min_reads=4000, max_reads=60000)
    data = [synth.fastq_bytes(s) for s in specs]
    data.insert(2, _poly_c(3000))
    data.insert(3, _poly_c(2000, 120))
    data.append(synth.fastq_bytes(synth.workload("hotspot", 40000, seed=seed)))
    data.append(synth.fastq_bytes(synth.workload("plain_small", 20000, seed=seed)))
    shapes = [(8, 4), (4, 2), (4, 1), (6, 3), (16, 16), (8, 8), (4, 4), (12, 3), (4, 2), (8, 2)]
    return data, shapes[:len(data)]


def _alone(ctx, data, k, chunks, T):
    fno, ofs = native.fastq_index(chunks, [data])
    starts = native.chunk_starts_of(fno, ofs, [len(data)])
    with native.Job(ctx) as job:
        job.load(data)
        cnt = job.count(k, starts)
        bounds = job.partition(k, 1, T, starts, cnt.chunk_first_read, cnt.hist)
        labels = job.labels()
        buf, sizes = job.output()
        return bounds, labels, bytes(buf), sizes.copy()


def _batched(ctx, datas, shapes, k):
    hosts = [np.frombuffer(d, dtype=np.uint8).copy() for d in datas]
    outs = [np.zeros(len(d) + 64, dtype=np.uint8) for d in datas]
    fs = [np.zeros(16 * T, dtype=np.uint64) for _, T in shapes]
    labs = [np.zeros(len(d) // 20 + 8, dtype=np.uint32) for d in datas]
    samples = [native.SampleIn(h.ctypes.data, len(d), c, T, o.ctypes.data, len(o), f, lab)
               for h, d, (c, T), o, f, lab in zip(hosts, datas, shapes, outs, fs, labs)]
    with native.Batch(ctx) as b:
        res = b.run(k, samples)
        groups = b.groups
    return res, outs, fs, labs, groups


def _check(ctx, datas, shapes, k, res, outs, fs, labs):
    for i, (d, (c, T)) in enumerate(zip(datas, shapes)):
        bounds, labels, files, sizes = _alone(ctx, d, k, c, T)
        r = res[i]
        assert r["n_reads"] == len(labels), f"sample {i}: read count"
        assert np.array_equal(r["bounds"], bounds), f"sample {i}: partition bounds differ"
        assert np.array_equal(labs[i][:len(labels)], labels), f"sample {i}: component labels differ"
        assert np.array_equal(fs[i], sizes), f"sample {i}: file sizes differ"
        assert r["out_total"] == len(files) and bytes(outs[i][:len(files)]) == files, f"sample {i}: partition files differ"


@pytest.mark.parametrize("k", [31, 27])
def test_batch_equals_each_sample_alone(built_gpu, k):
    datas, shapes = _mix(5 + k)
    with native.Context(0) as ctx:
        res, outs, fs, labs, groups = _batched(ctx, datas, shapes, k)
        assert groups == 1
        _check(ctx, datas, shapes, k, res, outs, fs, labs)


def test_batch_in_several_groups(built_gpu, monkeypatch):
    datas, shapes = _mix(17)
    monkeypatch.setenv("MP_BATCH_GROUP_BYTES", str(300 << 20))
    with native.Context(0) as ctx:
        res, outs, fs, labs, groups = _batched(ctx, datas, shapes, 31)
        assert groups > 2
        _check(ctx, datas, shapes, 31, res, outs, fs, labs)


def test_batch_samples_match_the_oracle(tmp_path, built_gpu):
    specs = synth.batch_mix(3, seed=23, min_reads=20000, max_reads=40000)
    datas = [synth.fastq_bytes(s) for s in specs]
    shapes = [(8, 4), (4, 2), (16, 8)]
    with native.Context(0) as ctx:
        res, outs, fs, labs, _ = _batched(ctx, datas, shapes, 31)
    for i in (0, 2):
        c, T = shapes[i]
        d = tmp_path / f"s{i}"
        d.mkdir()
        fq = d / "in.fastq"
        fq.write_bytes(datas[i])
        p = pu.Params(k=31, chunks=c, scans=1, threads=T)
        ref = pu.outputs(pu.run("oracle", d, [fq], p, dump=False), p, "in.fastq")
        off = np.concatenate([[0], np.cumsum(fs[i])]).astype(np.int64)
        for part in range(16):
            for t in range(T):
                j = part * T + t
                name = f"part/FromTid{t}_ToRank{part}.paired.fastq"
                assert bytes(outs[i][off[j]:off[j + 1]]) == ref.get(name, b""), f"sample {i}: {name} differs"


def test_batch_errors_name_the_sample(built_gpu):
    good = synth.fastq_bytes(synth.batch_mix(1, seed=3, min_reads=4000, max_reads=5000)[0])
    short = b"".join(b"@s%d\nACGTACGTAC\n+\nIIIIIIIIII\n" % i for i in range(100))  # no k-mer at all
    with native.Context(0) as ctx:
        with pytest.raises(native.MetapartError, match="sample 1"):
            _batched(ctx, [good, short], [(4, 2), (4, 2)], 31)
        with pytest.raises(native.MetapartError, match="sample 0"):
            _batched(ctx, [good[:-7]], [(4, 2)], 31)  # a truncated last record
