"""Benchmark of the GB300 read-partitioning path (one JSON line on rank 0).

A step is one pass of the whole path over one read set: chunk index, GPU FASTQ parse, m-mer histogram,
then per scan tuple enumeration, onesweep radix sort, branching-k-mer filter and union-find, the mate
union, the 16 work partitions and the partition-FASTQ gather.

  value  -- bases/s with the FASTQ already in HBM (the step copies it into the job and runs every stage)
  e2e    -- the same through the C ABI from pinned host memory: FASTQ upload and partition-file download
            inside the timed region
  roofline -- the radix-sort digit passes (the dominant kernel): algorithmic bytes per pass over their
            CUDA-event time, against the measured HBM copy bandwidth
  cpu_baseline -- the CPU oracle (the reference's algorithm restated in C/OpenMP, all host cores) on a
            bounded sample of the same read set

Workload (default): 20M single-end 150 bp reads from 200 synthetic genomes (1-5 Mb, GC 0.3-0.7, log-normal
abundance sigma 1.5, 1 % substitutions, N at 1e-4, qualities '#'..'J'); k = 31, m = 10 (the only m the
reference supports), 2 scans, numThreads 16, 64 chunks.  Inputs are larger than L2 (no flush needed).
With --gpus N under torchrun every rank partitions its own replica (replicas only; weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bases/sec partitioned (k=31) batched vs plain on 1 GB300; p50/p99 job latency"
ROOFLINE_TRAFFIC_FILE = ROOT / "profiles" / "onesweep_traffic.json"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain_large")
    ap.add_argument("--reads", type=int, default=20_000_000)
    ap.add_argument("--k", type=int, default=31)
    ap.add_argument("--scans", type=int, default=2)
    ap.add_argument("--threads", type=int, default=16)
    ap.add_argument("--chunks", type=int, default=64)
    ap.add_argument("--cpu-reads", type=int, default=0, help="reads in the CPU sample (0: auto)")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines: list[str] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def traffic_per_tuple():
    """DRAM bytes per tuple of one onesweep pass from the committed ncu capture (null when absent)."""
    try:
        return float(json.loads(ROOFLINE_TRAFFIC_FILE.read_text())["dram_bytes_per_tuple_per_pass"])
    except Exception:
        return None


# ------------------------------------------------------------------ CPU oracle

def cpu_run(sample: Path, k: int, scans: int, threads: int, chunks: int, cores: int) -> float:
    """Times the oracle's three stages (genFastqIdx, genHistograms, metapart) on a FASTQ file; seconds."""
    from metapart_gb300 import build
    cli = str(build.ORACLE_BUILD / "mpo_cli")
    d = sample.parent
    out = d / "out"
    (out / "Rank0").mkdir(parents=True, exist_ok=True)
    env = dict(os.environ, OMP_NUM_THREADS=str(cores), OMP_STACKSIZE="16M")
    cmds = [[cli, "genFastqIdx", str(chunks), "0", "1", "0", sample.name],
            [cli, "genHistograms", str(k), "0", "1", "0", sample.name],
            [cli, "metapart", "-o", str(out), str(1 << 40), str(k), str(scans), str(threads), "0", "1", "0",
             sample.name]]
    t0 = time.perf_counter()
    for c in cmds:
        r = subprocess.run(c, cwd=d, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode:
            raise RuntimeError(f"oracle stage failed: {' '.join(c)}\n{r.stdout[-2000:]}")
    return time.perf_counter() - t0


def cpu_sample(args, n_reads: int, tmp: Path) -> tuple[Path, int]:
    from metapart_gb300 import synth
    spec = synth.workload(args.workload, n_reads, seed=7)
    fq = tmp / "sample.fastq"
    synth.write_fastq(spec, fq)
    bases = n_reads * spec.lengths[0]
    return fq, bases


# --------------------------------------------------------------------- main

def main():
    args = parse_args()
    from metapart_gb300.replicas import Replicas
    dist = Replicas()
    if args.impl == "reference":
        return reference_arm(args, dist)

    import numpy as np
    import torch
    from metapart_gb300 import build, native, synth

    if not (build.BUILD / "libmetapart_gpu.so").exists():
        build.build_all()
    dev = dist.local
    torch.cuda.set_device(dev)
    spec = synth.workload(args.workload, args.reads, seed=7)
    fq = synth.fastq_bytes(spec)
    nbytes = len(fq)
    bases = args.reads * spec.lengths[0]
    fno, ofs = native.fastq_index(args.chunks, [fq])
    starts = native.chunk_starts_of(fno, ofs, [nbytes])
    host_in = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    host_in.numpy()[:] = np.frombuffer(fq, dtype=np.uint8)
    dev_in = host_in.to(f"cuda:{dev}")
    del fq
    ctx = native.Context(dev)
    job = native.Job(ctx)
    stream = torch.cuda.ExternalStream(job.stream, device=dev)
    min3 = args.workload == "min3"

    def device_step():
        job.reset()
        job.load_device(dev_in.data_ptr(), nbytes)
        cnt = job.count(args.k, starts, min3)
        job.partition(args.k, args.scans, args.threads, starts, cnt.chunk_first_read, cnt.hist, min3)
        job.prepare_output()

    out_host = None

    def e2e_step():
        nonlocal out_host
        job.reset()
        f, o = native.fastq_index_ptr(args.chunks, host_in.data_ptr(), nbytes)
        st = native.chunk_starts_of(f, o, [nbytes])
        job.load_ptr(host_in.data_ptr(), nbytes)
        cnt = job.count(args.k, st, min3)
        job.partition(args.k, args.scans, args.threads, st, cnt.chunk_first_read, cnt.hist, min3)
        _, total = job.prepare_output()
        if out_host is None or out_host.numel() < total:
            out_host = torch.empty(total + 16, dtype=torch.uint8, pin_memory=True)
        return job.output_to(out_host.data_ptr(), out_host.numel())

    for _ in range(args.warmup):
        device_step()
    # ---- device-resident timed region
    sort_bytes = sort_ms = 0.0
    sort_passes = sort_tuples = 0
    stage = {}
    l0 = native.launch_count()
    dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(dev) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            device_step()
            s = job.sort_stats()
            sort_bytes += s["bytes"]
            sort_ms += s["pass_ms"]
            sort_passes += s["passes"]
            sort_tuples += s["tuples"]
            for kk, v in job.stage_ms().items():
                stage[kk] = stage.get(kk, 0.0) + v
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize(dev)
    dist.barrier()
    launches = native.launch_count() - l0
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = dist.max(ms)
    value = dist.world * bases / (ms / 1e3)
    # ---- end to end through the C ABI, host buffers
    e2e_step()
    dist.barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out_bytes = 0
    for _ in range(args.steps):
        out_bytes = e2e_step()
    e1.record(stream)
    e1.synchronize()
    dist.barrier()
    e2e_ms = dist.max(e0.elapsed_time(e1) / args.steps)
    e2e_value = dist.world * bases / (e2e_ms / 1e3)

    peak, peak_kind = measured_peak()
    achieved = (sort_bytes / 1e9) / (sort_ms / 1e3) if sort_ms > 0 else 0.0
    per_launch_bytes = sort_bytes / max(sort_passes, 1)
    elt = 13 if 2 * args.k + 8 > 64 else 12   # bytes of one tuple: key (8) + read id (4) [+ high k-mer byte]
    tuples_per_launch = sort_bytes / (2 * elt) / max(sort_passes, 1)
    tpt = traffic_per_tuple()
    traffic = tpt * tuples_per_launch if tpt else None
    line = {
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "bases/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (seeded generator, no real reads)",
        "config": {"workload": f"{args.workload}: {args.reads} SE x {spec.lengths[0]} bp, {spec.n_genomes} genomes, "
                               f"{spec.sub_rate * 100:.1f}% subs",
                   "k": args.k, "m": 10, "num_scans": args.scans, "num_threads": args.threads,
                   "chunks": args.chunks, "bases_per_step": bases, "fastq_bytes": nbytes,
                   "l2": "inputs larger than L2 (FASTQ and tuple arrays are GBs)", "parallelism": "replicas"},
        "e2e": {"value": round(e2e_value, 1), "unit": "bases/s", "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": int(out_bytes) + 8 * (1 << 20) + 8},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "kernel": "k_onesweep (radix digit pass)",
                     "bytes_per_launch": int(per_launch_bytes),
                     "launch_ms": round(sort_ms / max(sort_passes, 1), 4),
                     "traffic": (round(traffic) if traffic else None)},
        "gpu_launches": int(launches),
        "stage_ms": {kk: round(v / args.steps, 3) for kk, v in stage.items()},
        "tuples_sorted_per_s": round(sort_tuples / args.steps / (ms / 1e3), 1),
        "clocks": clk.summary(),
    }
    if dist.rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
    job.close()
    ctx.close()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def cpu_baseline(args) -> dict:
    cores = os.cpu_count() or 1
    n = args.cpu_reads or 400_000
    n -= n % 2
    with tempfile.TemporaryDirectory() as td:
        fq, bases = cpu_sample(args, n, Path(td))
        chunks = cores * max(1, 64 // cores) if cores <= 64 else cores
        sec = cpu_run(fq, args.k, args.scans, cores, chunks, cores)
    return {"value": round(bases / sec, 1), "unit": "bases/s", "cores": cores, "kind": "port",
            "sample": f"{n} reads of the same read set ({bases} bases), numThreads {cores}, {chunks} chunks, "
                      f"genFastqIdx+genHistograms+metapart wall {sec:.2f} s"}


def reference_arm(args, dist):
    """The reference's CPU path (the C oracle port: the reference sources are not present on the GPU host)."""
    if dist.rank != 0:
        dist.close()
        return
    from metapart_gb300 import build
    build.build_oracle()
    build.build_synth()
    cores = os.cpu_count() or 1
    n = args.cpu_reads or 400_000
    n -= n % 2
    times = []
    with tempfile.TemporaryDirectory() as td:
        fq, bases = cpu_sample(args, n, Path(td))
        chunks = cores * max(1, 64 // cores) if cores <= 64 else cores
        for i in range(args.warmup + args.steps):
            sec = cpu_run(fq, args.k, args.scans, cores, chunks, cores)
            if i >= args.warmup:
                times.append(sec)
    sec = statistics.mean(times)
    v = bases / sec
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(v, 1),
        "unit": "bases/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(sec * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (seeded generator, no real reads)",
        "config": {"workload": f"{args.workload}: bounded sample of {n} reads of the same read set",
                   "k": args.k, "m": 10, "num_scans": args.scans, "num_threads": cores, "chunks": chunks},
        "cpu_baseline": {"value": round(v, 1), "unit": "bases/s", "cores": cores, "kind": "port",
                         "sample": f"{n} reads ({bases} bases) per step; the C oracle (reference algorithm restated, "
                                   f"OpenMP on all host cores)"},
        "e2e": {"value": round(v, 1), "unit": "bases/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
