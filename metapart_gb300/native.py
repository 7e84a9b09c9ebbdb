"""ctypes front end of libmetapart_gpu.so (include/metapart_gpu.h).

The stage functions mirror the reference programs' interfaces on in-memory data:
``fastq_index`` <-> genFastqIdx, ``Job.count`` <-> genHistograms (count module), ``Job.partition`` <->
metapart (enumerate, sort, filter, union-find, mate union), ``Job.output`` <-> writeOutput3.  Errors raise
``MetapartError`` with the library's message; there is no CPU fallback: without the CUDA library or a GPU
every call fails.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build

NB = 1 << 20
REC = 4194344
_lib = None


class MetapartError(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        path = build.BUILD / "libmetapart_gpu.so"
        if not path.exists():
            raise MetapartError(f"{path} is missing: run metapart_gb300.build.build_all() first")
        L = C.CDLL(str(path))
        u64p, u32p, i32p = C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_int32)
        L.mp_last_error.restype = C.c_char_p
        L.mp_ctx_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]
        L.mp_ctx_destroy.argtypes = [C.c_void_p]
        L.mp_ctx_hbm_in_use.argtypes = [C.c_void_p]
        L.mp_ctx_hbm_in_use.restype = C.c_uint64
        L.mp_fastq_index.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_char_p), u64p, i32p,
                                     u64p, C.POINTER(C.c_int)]
        L.mp_job_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.mp_job_destroy.argtypes = [C.c_void_p]
        L.mp_job_load_fastq.argtypes = [C.c_void_p, C.c_char_p, C.c_uint64, u64p, C.c_int, C.c_int]
        L.mp_job_load_fastq_device.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, u64p, C.c_int, C.c_int]
        L.mp_job_load_fastq_device_inplace.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, u64p, C.c_int, C.c_int]
        L.mp_job_reset.argtypes = [C.c_void_p]
        L.mp_job_stream.argtypes = [C.c_void_p]
        L.mp_job_stream.restype = C.c_void_p
        L.mp_launch_count.restype = C.c_uint64
        L.mp_job_num_reads.argtypes = [C.c_void_p]
        L.mp_job_num_reads.restype = C.c_uint64
        L.mp_job_count.argtypes = [C.c_void_p, C.c_int, C.c_int, u64p, C.c_int, u64p, u32p, u64p]
        L.mp_job_kmer_cache_pieces.argtypes = [C.c_void_p]
        L.mp_job_load_count.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, u64p, C.c_int, C.c_int, C.c_int, C.c_int,
                                        u64p, C.c_int, u64p, u64p]
        L.mp_job_partition.argtypes = [C.c_void_p, C.c_void_p, u64p, u64p, C.c_int, u64p, u64p]
        L.mp_job_labels.argtypes = [C.c_void_p, u32p]
        L.mp_job_output.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, u64p, u64p]
        L.mp_job_output_device.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), u64p, u64p]
        L.mp_job_set_dump_dir.argtypes = [C.c_void_p, C.c_char_p]
        L.mp_job_set_kmer_cache.argtypes = [C.c_void_p, C.c_int]
        L.mp_job_set_scan_piece_tuples.argtypes = [C.c_void_p, C.c_uint64]
        L.mp_job_set_read_store.argtypes = [C.c_void_p, C.c_int]
        L.mp_job_read_store.argtypes = [C.c_void_p]
        L.mp_job_set_wait_limits.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32]
        L.mp_job_set_checks.argtypes = [C.c_void_p, C.c_int]
        L.mp_count_unsorted.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                        C.POINTER(C.c_uint64)]
        L.mp_batch_set_wait_limits.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32]
        L.mp_job_scan_pieces.argtypes = [C.c_void_p]
        L.mp_job_stage_ms.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int]
        L.mp_job_sort_stats.argtypes = [C.c_void_p, u64p, C.POINTER(C.c_int), C.POINTER(C.c_double), u64p]
        L.mp_job_sort_split.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), u64p, u64p, u64p, u64p]
        L.mp_sort_tuples.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_uint64, C.c_void_p]
        L.mp_batch_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.mp_batch_destroy.argtypes = [C.c_void_p]
        L.mp_batch_run.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.mp_batch_stage_ms.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int]
        L.mp_batch_groups.argtypes = [C.c_void_p]
        L.mp_batch_sort_stats.argtypes = [C.c_void_p, u64p, C.POINTER(C.c_int), C.POINTER(C.c_double), u64p]
        _lib = L
    return _lib


def _check(rc: int, what: str):
    if rc != 0:
        msg = lib().mp_last_error().decode(errors="replace")
        raise MetapartError(f"{what} failed ({rc}): {msg}")


def _p64(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


class PartParams(C.Structure):
    _fields_ = [("k", C.c_int), ("min3", C.c_int), ("num_scans", C.c_int), ("num_threads", C.c_int)]


class Context:
    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.h = C.c_void_p()
        _check(lib().mp_ctx_create(device, hbm_budget, C.byref(self.h)), "mp_ctx_create")

    def hbm_in_use(self) -> int:
        return lib().mp_ctx_hbm_in_use(self.h)

    def close(self):
        if self.h:
            lib().mp_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def fastq_index(num_chunks: int, files: list[bytes], interleaved: bool = False):
    """genFastqIdx: (file_no, offset) of the num_chunks + 1 index records (fewer if files are short)."""
    n = len(files)
    arr = (C.c_char_p * n)(*files)
    sizes = np.array([len(f) for f in files], dtype=np.uint64)
    fno = np.zeros(num_chunks + 1, dtype=np.int32)
    ofs = np.zeros(num_chunks + 1, dtype=np.uint64)
    cnt = C.c_int()
    nse, nil = (0, n) if interleaved else (n, 0)
    _check(lib().mp_fastq_index(num_chunks, 0, nse, nil, n, arr, _p64(sizes),
                                fno.ctypes.data_as(C.POINTER(C.c_int32)), _p64(ofs), C.byref(cnt)), "mp_fastq_index")
    return fno[:cnt.value].copy(), ofs[:cnt.value].copy()


@dataclass
class CountResult:
    hist: np.ndarray          # 1048577 exclusive prefix sums (.kmerHist)
    chunk_reads: np.ndarray   # reads per chunk
    chunk_counts: np.ndarray | None  # [chunks, 1048576] u32 bucket counts

    @property
    def chunk_first_read(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum(self.chunk_reads)]).astype(np.uint64)


class Job:
    """One partition job: reads resident in HBM and the stage state, on its own CUDA stream."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = C.c_void_p()
        _check(lib().mp_job_create(ctx.h, C.byref(self.h)), "mp_job_create")

    def close(self):
        if self.h:
            lib().mp_job_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def load(self, data: bytes, file_sizes=None, interleaved: bool = False):
        fs = np.array(file_sizes if file_sizes is not None else [len(data)], dtype=np.uint64)
        _check(lib().mp_job_load_fastq(self.h, data, len(data), _p64(fs), len(fs), int(interleaved)), "load")

    def load_device(self, dev_ptr: int, nbytes: int, file_sizes=None, interleaved: bool = False):
        fs = np.array(file_sizes if file_sizes is not None else [nbytes], dtype=np.uint64)
        _check(lib().mp_job_load_fastq_device(self.h, C.c_void_p(dev_ptr), nbytes, _p64(fs), len(fs), int(interleaved)),
               "load_device")

    def load_device_inplace(self, dev_ptr: int, nbytes: int, file_sizes=None, interleaved: bool = False):
        """Uses FASTQ bytes already in device memory in place: 16-byte aligned, followed by 64 readable
        bytes, unchanged until the job is reset."""
        fs = np.array(file_sizes if file_sizes is not None else [nbytes], dtype=np.uint64)
        _check(lib().mp_job_load_fastq_device_inplace(self.h, C.c_void_p(dev_ptr), nbytes, _p64(fs), len(fs),
                                                      int(interleaved)), "load_device_inplace")

    def load_ptr(self, host_ptr: int, nbytes: int, interleaved: bool = False):
        """Upload from a host address (pinned memory for full copy bandwidth)."""
        fs = np.array([nbytes], dtype=np.uint64)
        _check(lib().mp_job_load_fastq(self.h, C.cast(C.c_void_p(host_ptr), C.c_char_p), nbytes, _p64(fs), 1,
                                       int(interleaved)), "load")

    def prepare_output(self):
        """Builds the partition files in device memory; returns (file sizes, total bytes)."""
        sizes = np.zeros(16 * self.num_threads, dtype=np.uint64)
        total = C.c_uint64()
        ptr = C.c_void_p()
        _check(lib().mp_job_output_device(self.h, C.byref(ptr), _p64(sizes), C.byref(total)), "output_device")
        return sizes, total.value

    def output_plan(self):
        """The partition files' sizes (file sizes, total bytes); no bytes move."""
        sizes = np.zeros(16 * self.num_threads, dtype=np.uint64)
        total = C.c_uint64()
        _check(lib().mp_job_output(self.h, None, 0, _p64(sizes), C.byref(total)), "output")
        return sizes, total.value

    def output_to(self, host_ptr: int, capacity: int) -> int:
        """Copies the partition files to a host address; returns the byte count."""
        total = C.c_uint64()
        _check(lib().mp_job_output(self.h, C.c_void_p(host_ptr), capacity, None, C.byref(total)), "output")
        return total.value

    def reset(self):
        _check(lib().mp_job_reset(self.h), "reset")

    @property
    def stream(self) -> int:
        return lib().mp_job_stream(self.h) or 0

    @property
    def num_reads(self) -> int:
        return lib().mp_job_num_reads(self.h)

    def set_kmer_cache(self, enable: bool):
        """Keep the count pass's k-mers for the next partition of the same k (default on)."""
        _check(lib().mp_job_set_kmer_cache(self.h, int(enable)), "set_kmer_cache")

    STORES = {"fastq": 0, "kmer_cache": 1, "packed": 2}

    def set_read_store(self, store: str):
        """What the count pass keeps of the reads for the partition: "kmer_cache" (default), "packed" or "fastq"."""
        _check(lib().mp_job_set_read_store(self.h, self.STORES[store]), "set_read_store")

    @property
    def read_store(self) -> str:
        v = lib().mp_job_read_store(self.h)
        return {b: a for a, b in self.STORES.items()}[v]

    def set_scan_piece_tuples(self, max_tuples: int):
        """Most tuples a scan holds in HBM at once (0: from the free device memory); a larger scan runs in
        bucket-range pieces with the same results."""
        _check(lib().mp_job_set_scan_piece_tuples(self.h, int(max_tuples)), "set_scan_piece_tuples")

    def set_checks(self, on: bool = True):
        """Self-checks of the sorted tuples and the final forest (mp_job_set_checks)."""
        _check(lib().mp_job_set_checks(self.h, int(bool(on))), "set_checks")

    def set_wait_limits(self, lookback_spins: int = 0, union_retries: int = 0, mate_rounds: int = 0):
        """Iteration limits of the bounded device waits (0: the default)."""
        _check(lib().mp_job_set_wait_limits(self.h, lookback_spins, union_retries, mate_rounds), "set_wait_limits")

    @property
    def scan_pieces(self) -> int:
        """Bucket-range pieces the last partition ran its scans in (numScans when none was split)."""
        return int(lib().mp_job_scan_pieces(self.h))

    def set_dump_dir(self, d: str | Path | None):
        _check(lib().mp_job_set_dump_dir(self.h, str(d).encode() if d else None), "set_dump_dir")

    def count(self, k: int, chunk_starts, min3: bool = False, want_chunk_counts: bool = False) -> CountResult:
        starts = np.ascontiguousarray(chunk_starts, dtype=np.uint64)
        nch = len(starts) - 1
        hist = np.zeros(NB + 1, dtype=np.uint64)
        reads = np.zeros(nch, dtype=np.uint64)
        cc = np.zeros((nch, NB), dtype=np.uint32) if want_chunk_counts else None
        ccp = cc.ctypes.data_as(C.POINTER(C.c_uint32)) if cc is not None else None
        _check(lib().mp_job_count(self.h, k, int(min3), _p64(starts), nch, _p64(hist), ccp, _p64(reads)), "count")
        return CountResult(hist, reads, cc)

    def load_count(self, host_ptr: int, nbytes: int, k: int, chunk_starts, min3: bool = False,
                   interleaved: bool = False, file_sizes=None) -> CountResult:
        """load_ptr followed by count, the upload overlapped with parsing and counting (pinned host bytes)."""
        fs = np.array(file_sizes if file_sizes is not None else [nbytes], dtype=np.uint64)
        starts = np.ascontiguousarray(chunk_starts, dtype=np.uint64)
        nch = len(starts) - 1
        hist = np.zeros(NB + 1, dtype=np.uint64)
        reads = np.zeros(nch, dtype=np.uint64)
        _check(lib().mp_job_load_count(self.h, C.c_void_p(host_ptr), nbytes, _p64(fs), len(fs), int(interleaved), k,
                                       int(min3), _p64(starts), nch, _p64(hist), _p64(reads)), "load_count")
        return CountResult(hist, reads, None)

    @property
    def kmer_cache_pieces(self) -> int:
        return int(lib().mp_job_kmer_cache_pieces(self.h))

    def partition(self, k: int, num_scans: int, num_threads: int, chunk_starts, chunk_first_read, hist,
                  min3: bool = False) -> np.ndarray:
        p = PartParams(k, int(min3), num_scans, num_threads)
        starts = np.ascontiguousarray(chunk_starts, dtype=np.uint64)
        first = np.ascontiguousarray(chunk_first_read, dtype=np.uint64)
        h = np.ascontiguousarray(hist, dtype=np.uint64)
        bounds = np.zeros(17, dtype=np.uint64)
        _check(lib().mp_job_partition(self.h, C.byref(p), _p64(starts), _p64(first), len(starts) - 1, _p64(h),
                                      _p64(bounds)), "partition")
        self.num_threads = num_threads
        return bounds

    def labels(self) -> np.ndarray:
        out = np.zeros(self.num_reads, dtype=np.uint32)
        _check(lib().mp_job_labels(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32))), "labels")
        return out

    def output(self, into: np.ndarray | None = None):
        """Partition file bytes (file j = partition * T + tid) and their sizes."""
        nf = 16 * self.num_threads
        sizes = np.zeros(nf, dtype=np.uint64)
        total = C.c_uint64()
        _check(lib().mp_job_output(self.h, None, 0, _p64(sizes), C.byref(total)), "output")
        buf = into if into is not None else np.empty(max(total.value, 1), dtype=np.uint8)
        _check(lib().mp_job_output(self.h, buf.ctypes.data_as(C.c_void_p), buf.nbytes, _p64(sizes), C.byref(total)),
               "output")
        return buf[:total.value], sizes

    def stage_ms(self) -> dict:
        a = (C.c_double * 8)()
        _check(lib().mp_job_stage_ms(self.h, a, 8), "stage_ms")
        names = ["parse", "count", "enumerate", "sort", "filter", "union_find", "mate_union_plan", "output"]
        return dict(zip(names, list(a)))

    def sort_stats(self) -> dict:
        t, b = C.c_uint64(), C.c_uint64()
        p, ms = C.c_int(), C.c_double()
        _check(lib().mp_job_sort_stats(self.h, C.byref(t), C.byref(p), C.byref(ms), C.byref(b)), "sort_stats")
        return {"tuples": t.value, "passes": p.value, "pass_ms": ms.value, "bytes": b.value}

    def sort_split(self) -> dict:
        a, u, g = C.c_double(), C.c_double(), C.c_double()
        nu, nb, nt = C.c_uint64(), C.c_uint64(), C.c_uint64()
        uc = (C.c_uint64 * 11)()
        _check(lib().mp_job_sort_split(self.h, C.byref(a), C.byref(u), C.byref(g), C.byref(nu), C.byref(nb),
                                       C.byref(nt), uc), "sort_split")
        return {"digit_pass_ms": a.value, "unit_sort_ms": u.value, "big_bucket_ms": g.value, "units": nu.value,
                "big_buckets": nb.value, "big_tuples": nt.value, "unit_passes": uc[0],
                "unit_cycles": {"load": uc[1], "passes": uc[2], "store": uc[3]},
                "pass_cycles": {"tile_id": uc[4], "load_rank": uc[5], "scan": uc[6], "order_lookback": uc[7],
                                "store": uc[8], "lookback_words": uc[9], "lookback_waits": uc[10]},
                "scan_pieces": self.scan_pieces}


def fastq_index_ptr(num_chunks: int, host_ptr: int, nbytes: int, interleaved: bool = False):
    """genFastqIdx on one FASTQ held at a host address."""
    arr = (C.c_char_p * 1)(C.cast(C.c_void_p(host_ptr), C.c_char_p))
    sizes = np.array([nbytes], dtype=np.uint64)
    fno = np.zeros(num_chunks + 1, dtype=np.int32)
    ofs = np.zeros(num_chunks + 1, dtype=np.uint64)
    cnt = C.c_int()
    nse, nil = (0, 1) if interleaved else (1, 0)
    _check(lib().mp_fastq_index(num_chunks, 0, nse, nil, 1, arr, _p64(sizes),
                                fno.ctypes.data_as(C.POINTER(C.c_int32)), _p64(ofs), C.byref(cnt)), "mp_fastq_index")
    return fno[:cnt.value].copy(), ofs[:cnt.value].copy()


def sort_tuples(ctx: Context, lo_in: int, hi_in: int | None, id_in: int, lo_out: int, hi_out: int | None,
                id_out: int, n: int, stream: int = 0):
    """mp_sort_tuples on device addresses (e.g. torch tensors' data_ptr())."""
    _check(lib().mp_sort_tuples(ctx.h, lo_in, hi_in, id_in, lo_out, hi_out, id_out, n, stream or None),
           "mp_sort_tuples")


def count_unsorted(ctx: Context, lo: int, hi: int | None, n: int, stream: int = 0) -> int:
    """mp_count_unsorted on device addresses: adjacent tuple pairs out of (k-mer, adjacency) order."""
    out = C.c_uint64(0)
    _check(lib().mp_count_unsorted(ctx.h, C.c_void_p(lo), C.c_void_p(hi) if hi else None, C.c_uint64(n),
                                   C.c_void_p(stream) if stream else None, C.byref(out)), "mp_count_unsorted")
    return int(out.value)


def launch_count() -> int:
    return lib().mp_launch_count()


def chunk_starts_of(fno: np.ndarray, ofs: np.ndarray, file_sizes) -> np.ndarray:
    base = np.concatenate([[0], np.cumsum(np.asarray(file_sizes, dtype=np.uint64))]).astype(np.uint64)
    return (base[fno.astype(np.int64)] + ofs).astype(np.uint64)


def run_pipeline(ctx: Context, fastq: bytes, k: int, num_chunks: int, num_scans: int, num_threads: int,
                 min3: bool = False, interleaved: bool = False, dump_dir=None, kmer_cache: bool = True,
                 store: str | None = None):
    """genFastqIdx -> genHistograms -> metapart on one in-memory FASTQ; returns (job, bounds, count).  store
    ("kmer_cache", "packed", "fastq") overrides kmer_cache."""
    fno, ofs = fastq_index(num_chunks, [fastq], interleaved)
    starts = chunk_starts_of(fno, ofs, [len(fastq)])
    job = Job(ctx)
    job.set_read_store(store or ("kmer_cache" if kmer_cache else "fastq"))
    if dump_dir:
        job.set_dump_dir(dump_dir)
    job.load(fastq, interleaved=interleaved)
    cnt = job.count(k, starts, min3)
    bounds = job.partition(k, num_scans, num_threads, starts, cnt.chunk_first_read, cnt.hist, min3)
    return job, bounds, cnt


class BatchParams(C.Structure):
    _fields_ = [("k", C.c_int), ("interleaved", C.c_int)]


class BatchSample(C.Structure):
    _fields_ = [("fastq", C.c_void_p), ("nbytes", C.c_uint64), ("num_chunks", C.c_int), ("num_threads", C.c_int),
                ("out", C.c_void_p), ("out_cap", C.c_uint64), ("file_sizes", C.POINTER(C.c_uint64)),
                ("labels", C.POINTER(C.c_uint32)), ("labels_cap", C.c_uint64)]


class BatchResult(C.Structure):
    _fields_ = [("status", C.c_int), ("error", C.c_char * 256), ("n_reads", C.c_uint64), ("out_total", C.c_uint64),
                ("bounds", C.c_uint64 * 17)]


@dataclass
class SampleIn:
    """One sample of a batch: its FASTQ at a host address (pinned memory for overlapped uploads), its chunk
    and thread counts, and where its partition files (and optionally labels) go."""
    fastq_ptr: int
    nbytes: int
    num_chunks: int
    num_threads: int
    out_ptr: int = 0
    out_cap: int = 0
    file_sizes: np.ndarray | None = None
    labels: np.ndarray | None = None


class Batch:
    """Many independent samples partitioned together (mp_batch_run): each gets the bounds, labels and
    partition files it gets alone with one scan."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = C.c_void_p()
        _check(lib().mp_batch_create(ctx.h, C.byref(self.h)), "mp_batch_create")

    def close(self):
        if self.h:
            lib().mp_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, k: int, samples: list, interleaved: bool = False) -> list:
        n = len(samples)
        arr = (BatchSample * n)()
        for i, s in enumerate(samples):
            arr[i].fastq = s.fastq_ptr
            arr[i].nbytes = s.nbytes
            arr[i].num_chunks = s.num_chunks
            arr[i].num_threads = s.num_threads
            arr[i].out = s.out_ptr or None
            arr[i].out_cap = s.out_cap
            if s.file_sizes is not None:
                arr[i].file_sizes = s.file_sizes.ctypes.data_as(C.POINTER(C.c_uint64))
            if s.labels is not None:
                arr[i].labels = s.labels.ctypes.data_as(C.POINTER(C.c_uint32))
                arr[i].labels_cap = len(s.labels)
        res = (BatchResult * n)()
        p = BatchParams(k, int(interleaved))
        _check(lib().mp_batch_run(self.h, C.byref(p), n, arr, res), "mp_batch_run")
        return [{"n_reads": r.n_reads, "out_total": r.out_total, "bounds": np.array(list(r.bounds), dtype=np.uint64)}
                for r in res]

    def stage_ms(self) -> dict:
        a = (C.c_double * 8)()
        _check(lib().mp_batch_stage_ms(self.h, a, 8), "mp_batch_stage_ms")
        names = ["parse", "count", "enumerate", "sort", "filter", "union_find", "mate_union_plan", "output"]
        return dict(zip(names, list(a)))

    @property
    def groups(self) -> int:
        return int(lib().mp_batch_groups(self.h))

    def sort_stats(self) -> dict:
        t, b = C.c_uint64(), C.c_uint64()
        p, ms = C.c_int(), C.c_double()
        _check(lib().mp_batch_sort_stats(self.h, C.byref(t), C.byref(p), C.byref(ms), C.byref(b)), "mp_batch_sort_stats")
        return {"tuples": t.value, "passes": p.value, "pass_ms": ms.value, "bytes": b.value}
