"""Request loop (mp_server_* in include/metapart_gpu.h): partition jobs admitted by HBM footprint.

``Server.submit`` queues one FASTQ held at a host address (pinned memory keeps the upload fast); the
library's worker threads admit requests in arrival order as slots and budget free up, run the whole
stage chain on their own CUDA streams and write the partition files into the caller's buffer.
``Server.result`` blocks until a request is done.  The caller keeps the input and output buffers alive
until then.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native


class RequestParams(C.Structure):
    """k, min3, num_scans, num_threads, num_chunks, interleaved, read_store (default: the packed reads, the
    smallest admission footprint)."""
    _fields_ = [("k", C.c_int), ("min3", C.c_int), ("num_scans", C.c_int), ("num_threads", C.c_int),
                ("num_chunks", C.c_int), ("interleaved", C.c_int), ("read_store", C.c_int)]

    def __init__(self, k=31, min3=0, num_scans=1, num_threads=16, num_chunks=64, interleaved=0, read_store=2):
        super().__init__(k, min3, num_scans, num_threads, num_chunks, interleaved, read_store)


class _Result(C.Structure):
    _fields_ = [("status", C.c_int), ("error", C.c_char * 256), ("n_reads", C.c_uint64), ("out_total", C.c_uint64),
                ("bounds", C.c_uint64 * 17), ("footprint", C.c_uint64), ("t_submit_ms", C.c_double),
                ("t_admit_ms", C.c_double), ("t_done_ms", C.c_double), ("device_ms", C.c_double)]


class _Stats(C.Structure):
    _fields_ = [("queued", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("reserved", C.c_uint64), ("peak_reserved", C.c_uint64), ("budget", C.c_uint64),
                ("running", C.c_int), ("peak_running", C.c_int)]


@dataclass
class Result:
    ticket: int
    status: int
    error: str
    n_reads: int
    out_total: int
    bounds: list
    footprint: int
    t_submit_ms: float
    t_admit_ms: float
    t_done_ms: float
    device_ms: float

    @property
    def latency_ms(self) -> float:
        return self.t_done_ms - self.t_submit_ms

    @property
    def queue_ms(self) -> float:
        return self.t_admit_ms - self.t_submit_ms


_bound = False


def _lib():
    global _bound
    L = native.lib()
    if not _bound:
        u64p = C.POINTER(C.c_uint64)
        L.mp_request_footprint.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(RequestParams)]
        L.mp_request_footprint.restype = C.c_uint64
        L.mp_server_create.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]
        L.mp_server_submit.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(RequestParams), C.c_void_p,
                                       C.c_uint64, u64p, C.c_void_p, C.c_uint64, u64p]
        L.mp_server_poll.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.POINTER(_Result)]
        L.mp_server_stats.argtypes = [C.c_void_p, C.POINTER(_Stats)]
        L.mp_server_destroy.argtypes = [C.c_void_p]
        _bound = True
    return L


def footprint(host_ptr: int, nbytes: int, params: RequestParams) -> int:
    """Estimated HBM bytes of one request (what admission reserves)."""
    return int(_lib().mp_request_footprint(host_ptr, nbytes, C.byref(params)))


class Server:
    def __init__(self, ctx: native.Context, slots: int = 4, hbm_budget: int = 0):
        self.h = C.c_void_p()
        rc = _lib().mp_server_create(ctx.h, slots, hbm_budget, C.byref(self.h))
        if rc:
            raise native.MetapartError(f"mp_server_create failed ({rc})")
        self.ctx = ctx

    def submit(self, host_ptr: int, nbytes: int, params: RequestParams, out_ptr: int, out_cap: int,
               file_sizes: np.ndarray | None = None, labels: np.ndarray | None = None) -> int:
        t = C.c_uint64()
        fs = file_sizes.ctypes.data_as(C.POINTER(C.c_uint64)) if file_sizes is not None else None
        lp = labels.ctypes.data if labels is not None else None
        lc = labels.size if labels is not None else 0
        rc = _lib().mp_server_submit(self.h, host_ptr, nbytes, C.byref(params), out_ptr, out_cap, fs, lp, lc,
                                     C.byref(t))
        if rc:
            raise native.MetapartError(f"mp_server_submit failed ({rc})")
        return t.value

    def result(self, ticket: int, wait: bool = True) -> Result | None:
        r = _Result()
        rc = _lib().mp_server_poll(self.h, ticket, 1 if wait else 0, C.byref(r))
        if rc < 0:
            raise native.MetapartError(f"mp_server_poll failed ({rc})")
        if rc == 0:
            return None
        return Result(ticket, r.status, r.error.decode(errors="replace"), r.n_reads, r.out_total, list(r.bounds),
                      r.footprint, r.t_submit_ms, r.t_admit_ms, r.t_done_ms, r.device_ms)

    def stats(self) -> dict:
        s = _Stats()
        _lib().mp_server_stats(self.h, C.byref(s))
        return {f: getattr(s, f) for f, _ in _Stats._fields_}

    def close(self):
        if self.h:
            _lib().mp_server_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
