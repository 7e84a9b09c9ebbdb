"""Autotuner of the bucket sort's plan knobs, keyed on k and scan size.

The bucket sort (csrc/k_sort.cu) has three knobs: the bucket digits ("balanced": the scan's varying bucket
bits in passes of near-equal width; "bytes": the bucket's bytes), the unit sort's widest digit (5..9 bits;
narrower digits mean more shared-memory passes over smaller histograms) and the digit pass's L2 prefetch
distance (SM waves of tiles ahead; 0 = none).  This script partitions synthetic read sets of the shape of
the 20M x 150 bp workload (plain_large) at several sizes and both k of the benchmarks on the GPU, times the sort
stage for every combination of the knobs (best of two runs, device time from the job's own events), and
writes the winners to sort_tuning.tsv beside this file, one row per (k, scan size class):

    k  min_tuples  digits  unit_bits  pf_waves

The library reads the table once per process and takes, for a sort of n tuples, the row of the nearest k
with the largest min_tuples not above n; the environment variables MP_SORT_BUCKET_DIGITS,
MP_UNIT_SORT_MAX_BITS and MP_ONESWEEP_PF_WAVES override it.

    python -m metapart_gb300.autotune            # on a GPU: measure and write sort_tuning.tsv
"""
from __future__ import annotations

import argparse
import itertools
import json
import math
import os
import time
from pathlib import Path

from . import build, native, synth

TABLE = Path(__file__).resolve().parent / "sort_tuning.tsv"
DIGITS = ("balanced", "bytes")
UNIT_BITS = (7, 8, 9)
PF_WAVES = (0, 1, 2)
ENV = ("MP_SORT_BUCKET_DIGITS", "MP_UNIT_SORT_MAX_BITS", "MP_ONESWEEP_PF_WAVES")


def _sort_ms(job: native.Job, k: int, starts, threads: int) -> tuple[float, int]:
    cnt = job.count(k, starts)
    job.partition(k, 1, threads, starts, cnt.chunk_first_read, cnt.hist)
    s = job.sort_split()
    return s["digit_pass_ms"] + s["unit_sort_ms"] + s["big_bucket_ms"], job.sort_stats()["tuples"]


def measure(ks=(27, 31), reads=(200_000, 2_000_000, 20_000_000), reps: int = 2, device: int = 0) -> list[dict]:
    build.build_gpu()
    saved = {e: os.environ.get(e) for e in ENV}
    rows = []
    try:
        with native.Context(device) as ctx:
            for n in reads:
                data = synth.fastq_bytes(synth.workload("plain_large", n, seed=13))
                fno, ofs = native.fastq_index(64, [data])
                starts = native.chunk_starts_of(fno, ofs, [len(data)])
                with native.Job(ctx) as job:
                    job.load(data)
                    for k in ks:
                        res = []
                        for dg, bits, pf in itertools.product(DIGITS, UNIT_BITS, PF_WAVES):
                            os.environ["MP_SORT_BUCKET_DIGITS"] = dg
                            os.environ["MP_UNIT_SORT_MAX_BITS"] = str(bits)
                            os.environ["MP_ONESWEEP_PF_WAVES"] = str(pf)
                            _sort_ms(job, k, starts, 16)  # warm-up
                            ms, tuples = min(_sort_ms(job, k, starts, 16) for _ in range(reps))
                            res.append((ms, dg, bits, pf, tuples))
                        res.sort()
                        ms, dg, bits, pf, tuples = res[0]
                        default = next(r[0] for r in res if r[1:4] == ("balanced", 9, 1))
                        rows.append({"k": k, "reads": n, "tuples": tuples, "digits": dg, "unit_bits": bits,
                                     "pf_waves": pf, "sort_ms": round(ms, 3), "default_ms": round(default, 3)})
    finally:
        for e, v in saved.items():
            if v is None:
                os.environ.pop(e, None)
            else:
                os.environ[e] = v
    return rows


def write_table(rows: list[dict], path: Path = TABLE, note: str = "") -> None:
    """One row per (k, size): min_tuples is the geometric midpoint between neighbouring measured sizes."""
    out = ["# k min_tuples digits unit_bits pf_waves   (written by metapart_gb300/autotune.py" +
           (f"; {note}" if note else "") + ")"]
    for k in sorted({r["k"] for r in rows}):
        rk = sorted((r for r in rows if r["k"] == k), key=lambda r: r["tuples"])
        for i, r in enumerate(rk):
            lo = 0 if i == 0 else int(math.sqrt(rk[i - 1]["tuples"] * r["tuples"]))
            out.append(f"{k} {lo} {r['digits']} {r['unit_bits']} {r['pf_waves']}"
                       f"   # {r['tuples']} tuples: {r['sort_ms']} ms (defaults {r['default_ms']} ms)")
    path.write_text("\n".join(out) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--reads", type=int, nargs="*", default=[200_000, 2_000_000, 20_000_000])
    ap.add_argument("--out", type=Path, default=TABLE)
    a = ap.parse_args()
    t0 = time.time()
    rows = measure(reads=tuple(a.reads), device=a.device)
    import torch
    note = f"{torch.cuda.get_device_name(a.device)}, {time.strftime('%Y-%m-%d')}"
    write_table(rows, a.out, note)
    print(json.dumps({"rows": rows, "seconds": round(time.time() - t0, 1)}))


if __name__ == "__main__":
    main()
