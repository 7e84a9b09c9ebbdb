"""Benchmark of the GB300 read-partitioning path (one JSON line on rank 0).

A step is one pass of the whole path over one read set: chunk index, GPU FASTQ parse, m-mer histogram,
then per scan tuple enumeration, onesweep radix sort, branching-k-mer filter and union-find, the mate
union, the 16 work partitions and the partition-FASTQ gather.

  value  -- bases/s with the FASTQ already in HBM (the step copies it into the job and runs every stage)
  e2e    -- the same through the C ABI from pinned host memory: FASTQ upload and partition-file download
            inside the timed region
  roofline -- the dominant kernel, the shared-memory unit sort (k_segsort: one launch per block shape and
            scan): algorithmic bytes (25 B per tuple read and written) over its CUDA-event time, against the
            measured HBM copy bandwidth; it is bound by shared memory, not HBM
  roofline_digit_pass -- the same for the bucket-digit radix passes (k_onesweep), the HBM-streaming kernel
  cpu_baseline -- the CPU oracle (the reference's algorithm restated in C/OpenMP, all host cores) on a
            bounded sample of the same read set; the GPU's partition files of that sample are compared with
            the oracle's ("parity")
  batch  -- the batch workload (64 samples of 50k-5M reads): the samples back to back through one
            job ("plain") against mp_batch_run ("batched"), both from pinned host FASTQ to partition files
  serve  -- Poisson arrivals of partition requests into the request loop: p50/p99 job latency

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
UNIT_SORT_TRAFFIC_FILE = ROOT / "profiles" / "unit_sort_traffic.json"


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
    ap.add_argument("--mode", default="plain", choices=["plain", "serve", "batch"],
                    help="plain: one read set per step; serve: Poisson request loop (p50/p99 latency); "
                         "batch: many samples, back to back vs queued together")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: mean arrivals per second")
    ap.add_argument("--slots", type=int, default=8, help="serve/batch: jobs in flight at most")
    ap.add_argument("--budget-gb", type=float, default=160.0, help="serve/batch: HBM admission budget")
    ap.add_argument("--pool", type=int, default=48, help="serve: distinct synthetic requests cycled")
    ap.add_argument("--samples", type=int, default=64, help="batch: samples")
    ap.add_argument("--sample-scale", type=float, default=1.0, help="batch: read-count scale")
    ap.add_argument("--serve-seconds", type=float, default=18.0,
                    help="plain mode: seconds of Poisson arrivals for the line's p50/p99 (0: none)")
    ap.add_argument("--no-batch", action="store_true", help="plain mode: leave out the batched-vs-plain run")
    ap.add_argument("--store", default="kmer_cache", choices=["kmer_cache", "packed", "fastq"],
                    help="plain mode: what the count pass keeps of the reads for the partition")
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


def traffic_per_tuple(path=ROOFLINE_TRAFFIC_FILE, key="dram_bytes_per_tuple_per_pass"):
    """DRAM bytes per tuple of one launch from a committed ncu capture (null when absent)."""
    try:
        return float(json.loads(path.read_text())[key])
    except Exception:
        return None


# ------------------------------------------------------------------ CPU oracle

def cpu_run(sample: Path, k: int, scans: int, threads: int, chunks: int, cores: int, min3: bool = False) -> float:
    """Times the oracle's three stages (genFastqIdx, genHistograms, metapart) on a FASTQ file; seconds."""
    from metapart_gb300 import build
    cli = str(build.ORACLE_BUILD / "mpo_cli")
    d = sample.parent
    out = d / "out"
    (out / "Rank0").mkdir(parents=True, exist_ok=True)
    env = dict(os.environ, OMP_NUM_THREADS=str(cores), OMP_STACKSIZE="16M")
    m3 = ["--min3"] if min3 else []
    cmds = [[cli, "genFastqIdx", str(chunks), "0", "1", "0", sample.name],
            [cli, "genHistograms", *m3, str(k), "0", "1", "0", sample.name],
            [cli, "metapart", *m3, "-o", str(out), str(1 << 40), str(k), str(scans), str(threads), "0", "1", "0",
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
    if args.mode == "serve":
        return serve_mode(args, dist)
    if args.mode == "batch":
        return batch_mode(args, dist)

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
    dev_in = torch.zeros(nbytes + 64, dtype=torch.uint8, device=f"cuda:{dev}")  # 64 readable bytes past the reads
    dev_in[:nbytes].copy_(host_in)
    del fq
    ctx = native.Context(dev)
    job = native.Job(ctx)
    job.set_read_store(args.store)
    stream = torch.cuda.ExternalStream(job.stream, device=dev)
    min3 = args.workload == "min3"

    def device_step():
        job.reset()
        job.load_device_inplace(dev_in.data_ptr(), nbytes)  # the reads already in HBM, used where they are
        cnt = job.count(args.k, starts, min3)
        job.partition(args.k, args.scans, args.threads, starts, cnt.chunk_first_read, cnt.hist, min3)
        job.prepare_output()

    out_host = None
    phase = {"index": 0.0, "load_count": 0.0, "partition": 0.0, "output_plan": 0.0, "download": 0.0}

    def e2e_step():
        nonlocal out_host
        t0 = time.perf_counter()
        job.reset()
        f, o = native.fastq_index_ptr(args.chunks, host_in.data_ptr(), nbytes)
        st = native.chunk_starts_of(f, o, [nbytes])
        t1 = time.perf_counter()
        cnt = job.load_count(host_in.data_ptr(), nbytes, args.k, st, min3)
        t2 = time.perf_counter()
        job.partition(args.k, args.scans, args.threads, st, cnt.chunk_first_read, cnt.hist, min3)
        t3 = time.perf_counter()
        _, total = job.output_plan()
        if out_host is None or out_host.numel() < total:
            out_host = torch.empty(total + 16, dtype=torch.uint8, pin_memory=True)
        t4 = time.perf_counter()
        n = job.output_to(out_host.data_ptr(), out_host.numel())
        t5 = time.perf_counter()
        for kk, a, b in (("index", t0, t1), ("load_count", t1, t2), ("partition", t2, t3), ("output_plan", t3, t4),
                         ("download", t4, t5)):
            phase[kk] += (b - a) * 1e3
        return n

    for _ in range(args.warmup):
        device_step()
    # ---- device-resident timed region
    sort_bytes = sort_ms = 0.0
    sort_passes = sort_tuples = 0
    stage = {}
    split = {}
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
            for kk, v in job.sort_split().items():
                if isinstance(v, dict):
                    d = split.setdefault(kk, {})
                    for k2, v2 in v.items():
                        d[k2] = d.get(k2, 0) + v2
                else:
                    split[kk] = split.get(kk, 0.0) + v
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
    for kk in phase:
        phase[kk] = 0.0
    dist.barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    out_bytes = 0
    with ClockSampler(dev) as clk_e2e:
        e0.record(stream)
        for _ in range(args.steps):
            out_bytes = e2e_step()
        e1.record(stream)
        e1.synchronize()
    dist.barrier()
    e2e_pieces = job.scan_pieces
    e2e_ms = dist.max(e0.elapsed_time(e1) / args.steps)
    e2e_value = dist.world * bases / (e2e_ms / 1e3)
    # the other stores of the reads (what the count pass keeps for the enumeration), device-resident, a few
    # steps each: their times and device bytes
    stores = {}
    reads_pos = args.reads * max(0, spec.lengths[0] - args.k + 1)
    rounds = args.reads * ((spec.lengths[0] + 31) // 32)
    store_bytes = {"kmer_cache": 9 * reads_pos + 8 * args.reads, "packed": 12 * rounds + 8 * args.reads, "fastq": 0}
    for other in [x for x in ("kmer_cache", "packed", "fastq") if x != args.store] if not min3 else []:
        job.set_read_store(other)
        device_step()
        e_a = torch.cuda.Event(enable_timing=True)
        e_b = torch.cuda.Event(enable_timing=True)
        e_a.record(stream)
        for _ in range(3):
            device_step()
        e_b.record(stream)
        e_b.synchronize()
        stores[other] = {"ms_per_step": round(e_a.elapsed_time(e_b) / 3, 3),
                         "enumerate_ms": round(job.stage_ms()["enumerate"], 3), "device_bytes": store_bytes[other]}
        job.set_read_store(args.store)
    stores[args.store] = {"ms_per_step": round(ms, 3), "enumerate_ms": round(stage.get("enumerate", 0) / args.steps, 3),
                          "device_bytes": store_bytes[args.store]}
    link = link_bandwidth(host_in, dev_in[:nbytes], out_host)

    peak, peak_kind = measured_peak()
    achieved = (sort_bytes / 1e9) / (sort_ms / 1e3) if sort_ms > 0 else 0.0
    per_launch_bytes = sort_bytes / max(sort_passes, 1)
    elt = 13 if 2 * args.k + 8 > 64 else 12   # bytes of one tuple: key (8) + read id (4) [+ high k-mer byte]
    tuples_per_launch = sort_bytes / (2 * elt) / max(sort_passes, 1)
    tpt = traffic_per_tuple()
    traffic = tpt * tuples_per_launch if tpt else None
    # the unit sort: every tuple outside the oversized buckets, read (key, high byte, id) and written (key, id)
    # once per scan; its time per scan covers both block shapes
    unit_tuples = (sort_tuples - split.get("big_tuples", 0)) / args.steps / max(args.scans, 1)
    unit_ms = split.get("unit_sort_ms", 0.0) / args.steps / max(args.scans, 1)
    unit_bytes = unit_tuples * (elt + 12)
    unit_achieved = (unit_bytes / 1e9) / (unit_ms / 1e3) if unit_ms > 0 else 0.0
    utpt = traffic_per_tuple(UNIT_SORT_TRAFFIC_FILE, "dram_bytes_per_tuple")
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
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": int(out_bytes) + 8 * (1 << 20) + 8,
                "scan_pieces": e2e_pieces,
                "phase_ms": {kk: round(v / args.steps, 2) for kk, v in phase.items()},
                "link_gbs": link, "host": host_placement(dev), "clocks": clk_e2e.summary()},
        "roofline": {"bound": "hbm", "achieved": round(unit_achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(unit_achieved / peak, 4), "peak_kind": peak_kind,
                     "kernel": "k_segsort (shared-memory unit sort, per scan)",
                     "limiter": "shared memory: the dependent gathers and scatters of its digit passes",
                     "bytes_per_launch": int(unit_bytes), "launch_ms": round(unit_ms, 4),
                     "traffic": (round(utpt * unit_tuples) if utpt else None)},
        "roofline_digit_pass": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                                "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                                "kernel": "k_onesweep (radix digit pass)",
                                "bytes_per_launch": int(per_launch_bytes),
                                "launch_ms": round(sort_ms / max(sort_passes, 1), 4),
                                "traffic": (round(traffic) if traffic else None)},
        "read_stores": stores,
        "gpu_launches": int(launches),
        "stage_ms": {kk: round(v / args.steps, 3) for kk, v in stage.items()},
        "sort_split": {kk: ({k2: int(v2 / args.steps) for k2, v2 in v.items()} if isinstance(v, dict) else
                             round(v / args.steps, 3) if kk.endswith("_ms") else int(v / args.steps))
                       for kk, v in split.items()},
        "tuples_sorted_per_s": round(sort_tuples / args.steps / (ms / 1e3), 1),
        "clocks": clk.summary(),
    }
    job.close()
    ctx.close()
    del dev_in
    torch.cuda.empty_cache()
    if dist.rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
        line["parity"] = line["cpu_baseline"]["gpu_parity"]["parity"]
    # the metric's other halves: batched against plain on the 64-sample batch workload, and job latency
    # under Poisson arrivals (rank 0 only: each is a single-GPU measurement)
    if dist.rank == 0 and not args.no_batch:
        b = batch_measure(args, dev, args.sample_scale)
        line["batch"] = b
        for kk in ("plain_bases_per_s", "batched_bases_per_s", "batched_over_plain"):
            line[kk] = b[kk]
    if dist.rank == 0 and args.serve_seconds > 0:
        r = serve_measure(args, dev, args.serve_seconds)
        line["serve"] = r
        line["p50_ms"] = r["p50_ms"]
        line["p99_ms"] = r["p99_ms"]
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def link_bandwidth(host_in, dev_buf, host_out, reps: int = 5) -> dict:
    """Host link rate of plain copies between the pinned buffers and HBM (GB/s): the best of `reps` and
    their harmonic mean (the host link has copies that run several times slower than the rest), for reading
    the e2e phases against.  Blocking copies: the pinned buffers carry no pending events into interpreter
    shutdown."""
    import torch
    n = min(host_in.numel(), dev_buf.numel(), host_out.numel())
    up, dn = [], []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        c = torch.cuda.Event(enable_timing=True)
        a.record()
        dev_buf[:n].copy_(host_in[:n])
        b.record()
        host_out[:n].copy_(dev_buf[:n])
        c.record()
        c.synchronize()
        up.append(a.elapsed_time(b))
        dn.append(b.elapsed_time(c))
    gbs = lambda ms: n / ms / 1e6
    return {"h2d": round(gbs(min(up)), 1), "d2h": round(gbs(min(dn)), 1),
            "h2d_mean": round(gbs(sum(up) / reps), 1), "d2h_mean": round(gbs(sum(dn) / reps), 1), "bytes": int(n)}


def host_placement(dev: int) -> dict:
    """Where the host side of the copies lives: the GPU's NUMA node (from its PCI device), the host's NUMA
    nodes with CPUs, and the nodes this process may allocate from (for reading the e2e phases)."""
    out = {}
    try:
        bus = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader", "-i", str(dev)],
                             stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=20).stdout.strip()
        if bus:
            bdf = bus.lower()[-12:] if len(bus) > 12 else bus.lower()  # 0000:xx:yy.z
            node = Path(f"/sys/bus/pci/devices/{bdf}/numa_node")
            if node.exists():
                out["gpu_numa_node"] = int(node.read_text().strip())
    except Exception:
        pass
    try:
        nodes = []
        for d in sorted(Path("/sys/devices/system/node").glob("node[0-9]*")):
            cpus = (d / "cpulist").read_text().strip()
            nodes.append({"node": int(d.name[4:]), "cpus": cpus or None})
        out["numa_nodes"] = nodes
    except Exception:
        pass
    try:
        for line in Path("/proc/self/status").read_text().splitlines():
            if line.startswith("Mems_allowed_list:"):
                out["mems_allowed"] = line.split(":", 1)[1].strip()
    except Exception:
        pass
    return out


# ------------------------------------------------- request loop and batches

def _pinned(n: int):
    import torch
    t = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    return t, t.data_ptr()


def _request_params(args, spec, chunks=None):
    from metapart_gb300 import serve
    return serve.RequestParams(args.k, 0, 1, args.threads, chunks or args.chunks, 0)


def serve_measure(args, dev: int, duration: float) -> dict:
    """Poisson arrivals of partition requests into the request loop (continuous admission by HBM footprint);
    p50/p99 submit-to-done latency and bases/s over the run."""
    import random

    import numpy as np
    import torch
    from metapart_gb300 import native, serve, synth
    specs = synth.serving_mix(args.pool, seed=11)
    pool = []
    for sp in specs:
        t = synth.fastq_to(sp, _pinned)
        out = torch.empty(t.numel() + 64, dtype=torch.uint8, pin_memory=True)
        pool.append((sp, t, out, sp.n_reads * sp.lengths[0]))
    budget = int(args.budget_gb * (1 << 30))
    ctx = native.Context(dev, hbm_budget=budget)
    srv = serve.Server(ctx, slots=args.slots, hbm_budget=budget)
    params = [_request_params(args, sp) for sp, *_ in pool]
    # warm-up: every slot once
    wt = [srv.submit(t.data_ptr(), t.numel(), params[i], o.data_ptr(), o.numel())
          for i, (sp, t, o, b) in enumerate(pool[:args.slots])]
    for x in wt:
        r = srv.result(x)
        if r.status:
            raise RuntimeError(f"warm-up request failed: {r.error}")
    rng = random.Random(3)
    arrivals, at = [], 0.0
    while True:
        at += rng.expovariate(args.rate)
        if at >= duration:
            break
        arrivals.append(at)
    free = list(range(len(pool)))
    rng.shuffle(free)
    inflight, results, stalls = {}, [], 0

    def reap(block_one=False):
        done = []
        for tk, i in inflight.items():
            r = srv.result(tk, wait=False)
            if r is not None:
                done.append((tk, i, r))
        if not done and block_one and inflight:
            tk = next(iter(inflight))
            done.append((tk, inflight[tk], srv.result(tk)))
        for tk, i, r in done:
            del inflight[tk]
            free.append(i)
            results.append((i, r))

    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        for at in arrivals:
            while True:
                reap()
                now = time.perf_counter() - t0
                if now >= at:
                    break
                time.sleep(min(0.002, at - now))
            if not free:
                stalls += 1
                reap(block_one=True)
            i = free.pop(0)
            sp, t, o, b = pool[i]
            tk = srv.submit(t.data_ptr(), t.numel(), params[i], o.data_ptr(), o.numel())
            inflight[tk] = i
        while inflight:
            reap(block_one=True)
    st = srv.stats()
    srv.close()
    ctx.close()
    bad = [r for _, r in results if r.status]
    if bad:
        raise RuntimeError(f"{len(bad)} requests failed, first: {bad[0].error}")
    lat = np.array([r.latency_ms for _, r in results])
    qms = np.array([r.queue_ms for _, r in results])
    # latency over the run (windows of a tenth of it) and by request size (thirds of the reads range, log scale)
    ts = np.array([r.t_submit_ms for _, r in results])
    ts = (ts - ts.min()) / 1e3
    win = max(duration / 10, 1e-9)
    dms = np.array([r.device_ms for _, r in results])
    # host share of a request's service time: admission to done, less the device stages (copies to and from
    # pinned memory, host indexing, launches)
    hms = np.array([r.t_done_ms - r.t_admit_ms - r.device_ms for _, r in results])
    by_time = []
    for w in range(10):
        m = (ts >= w * win) & (ts < (w + 1) * win)
        if m.any():
            by_time.append({"p50_ms": round(float(np.percentile(lat[m], 50)), 2),
                            "p99_ms": round(float(np.percentile(lat[m], 99)), 2),
                            "queue_mean_ms": round(float(qms[m].mean()), 2),
                            "device_mean_ms": round(float(dms[m].mean()), 2),
                            "host_mean_ms": round(float(hms[m].mean()), 2)})
    nr = np.array([r.n_reads for _, r in results], dtype=np.float64)
    edges = np.geomspace(max(nr.min(), 1), nr.max() + 1, 4)
    by_size = []
    for a, b in zip(edges[:-1], edges[1:]):
        m = (nr >= a) & (nr < b)
        if m.any():
            by_size.append({"reads": [int(a), int(b)], "jobs": int(m.sum()),
                            "p50_ms": round(float(np.percentile(lat[m], 50)), 2),
                            "p99_ms": round(float(np.percentile(lat[m], 99)), 2)})
    bases = sum(pool[i][3] for i, _ in results)
    span = (max(r.t_done_ms for _, r in results) - min(r.t_submit_ms for _, r in results)) / 1e3
    dev_ms = sum(r.device_ms for _, r in results)
    return {
        "workload": f"Poisson arrivals, mean {args.rate}/s for {duration:.0f} s; requests of 10k-2M SE x 150 bp reads "
                    f"(log-uniform) from 5-50 genomes, 1% subs; {len(pool)} distinct requests cycled; k={args.k}, "
                    f"1 scan, {args.threads} threads, {args.slots} slots, {args.budget_gb:.0f} GB admission budget",
        "bases_per_s": round(bases / span, 1), "jobs": len(results), "jobs_per_s": round(len(results) / span, 2),
        "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
        "mean_ms": round(float(lat.mean()), 2), "queue_p50_ms": round(float(np.percentile(qms, 50)), 2),
        "queue_p99_ms": round(float(np.percentile(qms, 99)), 2), "device_busy": round(dev_ms / 1e3 / span, 3),
        "peak_running": st["peak_running"], "peak_reserved_gb": round(st["peak_reserved"] / (1 << 30), 2),
        "pool_stalls": stalls, "warmup_jobs": len(wt), "by_tenth": by_time, "by_size": by_size,
        "clocks": clk.summary(),
    }


def serve_mode(args, dist):
    if dist.rank != 0:
        dist.close()
        return
    import torch
    torch.cuda.set_device(dist.local)
    r = serve_measure(args, dist.local, args.duration)
    line = {"metric": METRIC, "mode": "serve", "value": r["bases_per_s"], "unit": "bases/s", "n_gpus": 1,
            "steps": r["jobs"], "warmup": r["warmup_jobs"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded generator, no real reads)",
            "config": {"workload": r["workload"]}, **{kk: v for kk, v in r.items() if kk != "workload"}}
    print(json.dumps(line), flush=True)
    dist.close()


def _checksum(t, n: int) -> tuple:
    """Order-sensitive checksum of the first n bytes of a host tensor (sums of the 8-byte words and of the words
    times their index parity), enough to tell two runs' partition files apart."""
    import numpy as np
    a = t[:n].numpy()
    w = np.frombuffer(a[: n - n % 8].tobytes() if n % 8 else a, dtype=np.uint64) if n >= 8 else np.zeros(0, np.uint64)
    tail = bytes(a[n - n % 8:n]) if n % 8 else b""
    return int(w.sum()), int(w[::2].sum()), int(w[1::3].sum()), tail


def batch_measure(args, dev: int, scale: float) -> dict:
    """The batch workload: independent samples (read counts log-uniform 50k-5M x scale, lengths in
    {100, 150, 250}) from pinned host FASTQ to partition files in pinned host memory, (a) plain: one after
    another through one job, every stage per sample, (b) batched: all of them through mp_batch_run.  The two
    runs' partition files are compared, and two samples' files with the CPU oracle's."""
    import numpy as np
    import torch
    from metapart_gb300 import native, synth
    specs = synth.batch_mix(args.samples, seed=5, scale=scale)
    ins = [synth.fastq_to(sp, _pinned) for sp in specs]
    outs = [torch.empty(t.numel() + 64, dtype=torch.uint8, pin_memory=True) for t in ins]
    bases = sum(sp.n_reads * sp.lengths[0] for sp in specs)
    budget = int(args.budget_gb * (1 << 30))
    ctx = native.Context(dev, hbm_budget=budget)
    T, chunks = args.threads, args.chunks
    fsz = [np.zeros(16 * T, dtype=np.uint64) for _ in specs]

    def plain_all():
        res = []
        with native.Job(ctx) as job:
            for t, o in zip(ins, outs):
                job.reset()
                f, ofs = native.fastq_index_ptr(chunks, t.data_ptr(), t.numel())
                st = native.chunk_starts_of(f, ofs, [t.numel()])
                cnt = job.load_count(t.data_ptr(), t.numel(), args.k, st)
                bnd = job.partition(args.k, 1, T, st, cnt.chunk_first_read, cnt.hist)
                job.output_plan()
                res.append((job.output_to(o.data_ptr(), o.numel()), bnd.tolist()))
        return res

    batch = native.Batch(ctx)
    samples = [native.SampleIn(t.data_ptr(), t.numel(), chunks, T, o.data_ptr(), o.numel(), f)
               for t, o, f in zip(ins, outs, fsz)]

    def batched_all():
        return [(r["out_total"], r["bounds"].tolist()) for r in batch.run(args.k, samples)]

    with ClockSampler(dev) as clk:
        plain_all()  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        want = plain_all()
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
        digest_plain = [_checksum(o, n) for o, (n, _) in zip(outs, want)]
        batched_all()  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        got = batched_all()
        torch.cuda.synchronize()
        batched_s = time.perf_counter() - t0
    stage = batch.stage_ms()
    groups = batch.groups
    ss = batch.sort_stats()
    digest_batched = [_checksum(o, n) for o, (n, _) in zip(outs, got)]
    # two of the smallest samples against the CPU oracle, file by file
    oracle_ok = []
    order = sorted(range(len(specs)), key=lambda i: specs[i].n_reads)[:2]
    for i in order:
        with tempfile.TemporaryDirectory() as td:
            d = Path(td)
            fq = d / "sample.fastq"
            fq.write_bytes(ins[i].numpy().tobytes())
            cores = os.cpu_count() or 1
            cpu_run(fq, args.k, 1, T, chunks, cores)
            off = np.concatenate([[0], np.cumsum(fsz[i])]).astype(np.int64)
            ob = outs[i].numpy()
            same = True
            for part in range(16):
                for t in range(T):
                    j = part * T + t
                    f = d / "out" / "Rank0" / f"FromTid{t}_ToRank{part}.paired.fastq"
                    if ob[off[j]:off[j + 1]].tobytes() != (f.read_bytes() if f.exists() else b""):
                        same = False
            oracle_ok.append(same)
    batch.close()
    ctx.close()
    return {
        "workload": f"{len(specs)} samples, reads log-uniform 50k-5M x {scale} (even), lengths in {{100,150,250}}, "
                    f"10-100 genomes of 0.5-3 Mb, log-normal abundance sigma 1.5, 1% subs; k={args.k}, 1 scan, "
                    f"{T} threads, {chunks} chunks; pinned host FASTQ to pinned host partition files",
        "bases": bases, "reads": sum(sp.n_reads for sp in specs),
        "plain_bases_per_s": round(bases / plain_s, 1), "batched_bases_per_s": round(bases / batched_s, 1),
        "batched_over_plain": round(plain_s / batched_s, 3), "plain_s": round(plain_s, 3),
        "batched_s": round(batched_s, 3), "groups": groups,
        "identical_to_plain": bool(want == got and digest_plain == digest_batched),
        "oracle_samples_identical": oracle_ok,
        "batched_stage_ms": {kk: round(v, 2) for kk, v in stage.items()},
        "batched_sort": {"tuples": ss["tuples"], "digit_passes": ss["passes"], "digit_pass_ms": round(ss["pass_ms"], 2),
                         "digit_pass_gbs": round(ss["bytes"] / 1e9 / (ss["pass_ms"] / 1e3), 1) if ss["pass_ms"] else None},
        "clocks": clk.summary(),
    }


def batch_mode(args, dist):
    if dist.rank != 0:
        dist.close()
        return
    import torch
    torch.cuda.set_device(dist.local)
    r = batch_measure(args, dist.local, args.sample_scale)
    line = {"metric": METRIC, "mode": "batch", "value": r["batched_bases_per_s"], "unit": "bases/s", "n_gpus": 1,
            "steps": 1, "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (seeded generator, no real reads)",
            "config": {"workload": r["workload"]}, **{kk: v for kk, v in r.items() if kk != "workload"}}
    print(json.dumps(line), flush=True)
    dist.close()


def gpu_parity_on_sample(fq: Path, out_dir: Path, k: int, scans: int, threads: int, chunks: int,
                         min3: bool = False) -> dict:
    """Partitions the CPU sample on the GPU through the library with the oracle's parameters and compares
    every partition file (FromTid<t>_ToRank<p>.paired.fastq) with the oracle's, byte for byte."""
    import numpy as np
    from metapart_gb300 import native
    data = fq.read_bytes()
    with native.Context(0) as ctx:
        job, bounds, cnt = native.run_pipeline(ctx, data, k, chunks, scans, threads, min3=min3)
        try:
            buf, sizes = job.output()
        finally:
            job.close()
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    bad = []
    for p in range(16):
        for t in range(threads):
            j = p * threads + t
            f = out_dir / "Rank0" / f"FromTid{t}_ToRank{p}.paired.fastq"
            want = f.read_bytes() if f.exists() else b""
            if bytes(buf[off[j]:off[j + 1]]) != want:
                bad.append(f.name)
    return {"parity": not bad, "files": 16 * threads, "files_differing": bad[:8],
            "compared": "all partition files of the CPU sample, GPU (library) against the oracle, byte for byte"}


def cpu_baseline(args) -> dict:
    cores = os.cpu_count() or 1
    n = args.cpu_reads or 400_000
    n -= n % 2
    with tempfile.TemporaryDirectory() as td:
        fq, bases = cpu_sample(args, n, Path(td))
        chunks = cores * max(1, 64 // cores) if cores <= 64 else cores
        min3 = args.workload == "min3"
        sec = cpu_run(fq, args.k, args.scans, cores, chunks, cores, min3)
        par = gpu_parity_on_sample(fq, fq.parent / "out", args.k, args.scans, cores, chunks, min3)
    return {"value": round(bases / sec, 1), "unit": "bases/s", "cores": cores, "kind": "port",
            "sample": f"{n} reads of the same read set ({bases} bases), numThreads {cores}, {chunks} chunks, "
                      f"genFastqIdx+genHistograms+metapart wall {sec:.2f} s",
            "gpu_parity": par}


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
            sec = cpu_run(fq, args.k, args.scans, cores, chunks, cores, args.workload == "min3")
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
