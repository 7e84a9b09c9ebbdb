"""The sort's tuning table: rows chosen by k and scan size change the plan, never the result.

A table (MP_SORT_TUNING) that gives k = 31 narrow 5-bit unit-sort digits and byte bucket digits makes the
unit sort run more digit passes than one that gives 9-bit digits; every partition must give the same
labels, bounds and partition files as the defaults.  Rows of another k, or of a larger scan size than the
input's, must not apply.  The library reads the table once per process, so each table runs in a child
process.
"""
import json
import os
import subprocess
import sys
import textwrap

import pytest

from metapart_gb300 import synth

pytestmark = pytest.mark.gpu

KNOBS = ("MP_SORT_BUCKET_DIGITS", "MP_UNIT_SORT_MAX_BITS", "MP_ONESWEEP_PF_WAVES")


def test_tuning_rows_change_the_plan_not_the_result(tmp_path, built_gpu):
    data_path = tmp_path / "in.fastq"
    data_path.write_bytes(synth.fastq_bytes(synth.workload("plain_large", 40_000, seed=9)))
    script = textwrap.dedent(f"""
        import hashlib, json, sys
        sys.path.insert(0, {str(built_gpu.ROOT)!r})
        from metapart_gb300 import native
        data = open({str(data_path)!r}, "rb").read()
        fno, ofs = native.fastq_index(8, [data])
        starts = native.chunk_starts_of(fno, ofs, [len(data)])
        with native.Context(0) as ctx, native.Job(ctx) as job:
            job.load(data)
            cnt = job.count(31, starts)
            b = job.partition(31, 1, 4, starts, cnt.chunk_first_read, cnt.hist)
            buf, _ = job.output()
            print(json.dumps({{"bounds": b.tolist(), "labels": hashlib.sha256(job.labels().tobytes()).hexdigest(),
                              "files": hashlib.sha256(bytes(buf)).hexdigest(),
                              "unit_passes": job.sort_split()["unit_passes"]}}))
    """)

    def run(name, rows):
        env = {k: v for k, v in os.environ.items() if k not in KNOBS}
        t = tmp_path / f"{name}.tsv"
        t.write_text("# k min_tuples digits unit_bits pf_waves\n" + rows)
        env["MP_SORT_TUNING"] = str(t)
        r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        return json.loads(r.stdout.strip().splitlines()[-1])

    default = run("empty", "")
    narrow = run("narrow", "31 0 bytes 5 0\n")
    wide = run("wide", "31 0 balanced 9 2\n")
    other_k = run("other_k", "21 0 bytes 5 0\n31 0 balanced 9 1\n")
    too_big = run("too_big", "31 0 balanced 9 1\n31 999999999999 bytes 5 0\n")
    for r in (narrow, wide, other_k, too_big):
        assert r["bounds"] == default["bounds"] and r["labels"] == default["labels"] and r["files"] == default["files"]
    assert narrow["unit_passes"] > wide["unit_passes"]
    assert other_k["unit_passes"] == default["unit_passes"] == too_big["unit_passes"]
