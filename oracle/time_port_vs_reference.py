"""Times the reference's own programs (oracle/_ref, built from the reference sources by oracle/build_ref.sh)
against the C restatement (oracle/_build/mpo_cli) on the same seeded inputs, every stage with all host
cores, so the CPU baseline the bench reports (which times the restatement: the reference sources exist only
where they were built) can be read against the reference itself.

Test infrastructure, like everything under oracle/: it times the two checkers, never the GPU path.

    python oracle/time_port_vs_reference.py [--reps 3]      # prints one JSON line per workload
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

BUF = 1 << 30  # fastqBufferSize: above the largest chunk (the reference allocates it per thread)

WORKLOADS = [
    # name, reads, k, scans
    ("plain_small", 100_000, 27, 1),    # the 100k x 100 bp workload at its full size
    ("plain_large", 400_000, 31, 2),    # the 20M x 150 bp workload's read set at the bench's CPU sample size
]


def _stages(impl: str, fq: str, k: int, scans: int, threads: int, chunks: int, out: str):
    if impl == "reference":
        b = ROOT / "oracle" / "_ref"
        return [[str(b / "genFastqIdx"), str(chunks), "0", "1", "0", fq],
                [str(b / "genHistograms_metapart"), str(k), "0", "1", "0", fq],
                [str(b / "metapart"), "-o", out, str(BUF), str(k), str(scans), str(threads), "0", "1", "0", fq]]
    c = str(ROOT / "oracle" / "_build" / "mpo_cli")
    return [[c, "genFastqIdx", str(chunks), "0", "1", "0", fq],
            [c, "genHistograms", str(k), "0", "1", "0", fq],
            [c, "metapart", "-o", out, str(BUF), str(k), str(scans), str(threads), "0", "1", "0", fq]]


def run_once(impl: str, d: Path, fq: Path, k: int, scans: int, threads: int, chunks: int) -> list[float]:
    work = d / impl
    (work / "out" / "Rank0").mkdir(parents=True, exist_ok=True)
    link = work / fq.name
    if not link.exists():
        link.symlink_to(fq)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_STACKSIZE="16M")
    secs = []
    for cmd in _stages(impl, fq.name, k, scans, threads, chunks, "./out"):
        t0 = time.perf_counter()
        r = subprocess.run(cmd, cwd=work, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        secs.append(time.perf_counter() - t0)
        if r.returncode:
            raise RuntimeError(f"{impl}: {' '.join(cmd)} failed\n{r.stdout[-2000:]}")
    return secs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    from metapart_gb300 import build, synth
    build.build_oracle()
    build.build_synth()
    if not build.build_reference():
        raise SystemExit("the reference sources are not present here: nothing to time against")
    cores = os.cpu_count() or 1
    chunks = cores * max(1, 64 // cores)
    for name, n, k, scans in WORKLOADS:
        with tempfile.TemporaryDirectory() as td:
            d = Path(td)
            fq = d / "in.fastq"
            spec = synth.workload(name, n, seed=7)
            synth.write_fastq(spec, fq)
            bases = n * spec.lengths[0]
            res = {}
            for impl in ("reference", "port"):
                run_once(impl, d, fq, k, scans, cores, chunks)  # warm-up (page cache, first-touch)
                runs = [run_once(impl, d, fq, k, scans, cores, chunks) for _ in range(a.reps)]
                tot = [sum(r) for r in runs]
                res[impl] = {"seconds": round(statistics.median(tot), 3),
                             "stage_seconds": [round(statistics.median(x), 3) for x in zip(*runs)],
                             "bases_per_s": round(bases / statistics.median(tot), 1)}
            print(json.dumps({"workload": f"{name}: {n} reads, k={k}, {scans} scan(s)", "cores": cores,
                              "threads": cores, "chunks": chunks, **res,
                              "port_over_reference": round(res["reference"]["seconds"] / res["port"]["seconds"], 3)}),
                  flush=True)


if __name__ == "__main__":
    main()
