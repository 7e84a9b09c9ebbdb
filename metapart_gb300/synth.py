"""Seeded synthetic read sets (ctypes front end of csrc/synth.c).

The named workloads restate the benchmark workloads by their shapes and
distributions; the reads themselves are generated here, never downloaded.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

from . import build

AB_UNIFORM, AB_LOGNORMAL, AB_ZIPF = 0, 1, 2


class _Spec(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("n_reads", C.c_uint64),
        ("len_choices", C.c_int * 4),
        ("n_len_choices", C.c_int),
        ("n_genomes", C.c_int),
        ("glen_lo", C.c_double),
        ("glen_hi", C.c_double),
        ("gc_lo", C.c_double),
        ("gc_hi", C.c_double),
        ("abundance", C.c_int),
        ("ab_param", C.c_double),
        ("repeat_frac", C.c_double),
        ("repeat_len", C.c_int),
        ("repeat_pool", C.c_int),
        ("sub_rate", C.c_double),
        ("n_rate", C.c_double),
        ("qual_char", C.c_char),
        ("qual_lo", C.c_char),
        ("qual_hi", C.c_char),
        ("interleaved", C.c_int),
        ("insert_len", C.c_int),
    ]


@dataclass
class ReadSpec:
    n_reads: int
    lengths: tuple = (100,)
    n_genomes: int = 20
    glen: tuple = (50_000, 50_000)
    gc: tuple = (0.5, 0.5)
    abundance: int = AB_UNIFORM
    ab_param: float = 0.0
    repeat_frac: float = 0.0
    repeat_len: int = 0
    repeat_pool: int = 0
    sub_rate: float = 0.005
    n_rate: float = 0.0
    qual: str = "I"             # one char, or "#J" for uniform in ['#', 'J']
    interleaved: bool = False
    insert_len: int = 0
    seed: int = 7
    extra: dict = field(default_factory=dict)

    def _c(self) -> _Spec:
        s = _Spec()
        s.seed = self.seed
        s.n_reads = self.n_reads
        for i, L in enumerate(self.lengths[:4]):
            s.len_choices[i] = L
        s.n_len_choices = len(self.lengths[:4])
        s.n_genomes = self.n_genomes
        s.glen_lo, s.glen_hi = float(self.glen[0]), float(self.glen[1])
        s.gc_lo, s.gc_hi = float(self.gc[0]), float(self.gc[1])
        s.abundance = self.abundance
        s.ab_param = self.ab_param
        s.repeat_frac = self.repeat_frac
        s.repeat_len = self.repeat_len
        s.repeat_pool = self.repeat_pool
        s.sub_rate = self.sub_rate
        s.n_rate = self.n_rate
        if len(self.qual) == 2:
            s.qual_lo, s.qual_hi = self.qual[0].encode(), self.qual[1].encode()
            s.qual_char = b"I"
        else:
            s.qual_char = self.qual.encode()
            s.qual_lo = s.qual_hi = b"\0"
        s.interleaved = int(self.interleaved)
        s.insert_len = self.insert_len
        return s


_lib = None


def _load():
    global _lib
    if _lib is None:
        build.build_synth()
        _lib = C.CDLL(str(build.BUILD / "libmp_synth.so"))
        _lib.mp_synth_fastq.argtypes = [C.POINTER(_Spec), C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
        _lib.mp_synth_fastq_file.argtypes = [C.POINTER(_Spec), C.c_char_p, C.POINTER(C.c_size_t)]
        _lib.mp_synth_free.argtypes = [C.c_void_p]
    return _lib


def fastq_bytes(spec: ReadSpec) -> bytes:
    lib = _load()
    p, n = C.c_void_p(), C.c_size_t()
    rc = lib.mp_synth_fastq(C.byref(spec._c()), C.byref(p), C.byref(n))
    if rc:
        raise RuntimeError(f"mp_synth_fastq failed: {rc}")
    try:
        # ctypes.string_at takes a C int size; copy through an array type for inputs above 2 GiB
        return bytes(memoryview((C.c_char * n.value).from_address(p.value)))
    finally:
        lib.mp_synth_free(p)


def fastq_to(spec: ReadSpec, alloc):
    """Generates into a caller buffer: alloc(nbytes) returns (buffer object, host address)."""
    lib = _load()
    p, n = C.c_void_p(), C.c_size_t()
    rc = lib.mp_synth_fastq(C.byref(spec._c()), C.byref(p), C.byref(n))
    if rc:
        raise RuntimeError(f"mp_synth_fastq failed: {rc}")
    try:
        obj, addr = alloc(n.value)
        C.memmove(addr, p.value, n.value)
        return obj
    finally:
        lib.mp_synth_free(p)


def write_fastq(spec: ReadSpec, path: str | Path) -> int:
    lib = _load()
    n = C.c_size_t()
    rc = lib.mp_synth_fastq_file(C.byref(spec._c()), str(path).encode(), C.byref(n))
    if rc:
        raise RuntimeError(f"mp_synth_fastq_file failed: {rc}")
    return n.value


def workload(name: str, n_reads: int | None = None, seed: int = 7) -> ReadSpec:
    """Named read sets with the benchmark shapes (n_reads may scale a set down for a test or a CPU sample)."""
    if name == "plain_small":   # 100k SE x 100 bp, 20 x 50 kb genomes, 0.5 % subs, no N, 'I', k=27
        return ReadSpec(n_reads=n_reads or 100_000, lengths=(100,), n_genomes=20, glen=(50_000, 50_000),
                        sub_rate=0.005, qual="I", seed=seed)
    if name == "plain_large":   # 20M SE x 150 bp, 200 genomes 1-5 Mb log-uniform, GC 0.3-0.7, lognormal 1.5
        return ReadSpec(n_reads=n_reads or 20_000_000, lengths=(150,), n_genomes=200, glen=(1e6, 5e6),
                        gc=(0.3, 0.7), abundance=AB_LOGNORMAL, ab_param=1.5, sub_rate=0.01, n_rate=1e-4,
                        qual="#J", seed=seed)
    if name == "min3":          # 5M SE x 250 bp, 100 x 2 Mb genomes, Zipf 1.1, 30 % shared 5 kb repeats
        return ReadSpec(n_reads=n_reads or 5_000_000, lengths=(250,), n_genomes=100, glen=(2e6, 2e6),
                        abundance=AB_ZIPF, ab_param=1.1, repeat_frac=0.3, repeat_len=5000, repeat_pool=200,
                        sub_rate=0.01, qual="I", seed=seed)
    if name == "hotspot":       # one 200 bp genome at very high coverage: oversized m-mer buckets, long runs
        return ReadSpec(n_reads=n_reads or 60_000, lengths=(100,), n_genomes=1, glen=(200, 200),
                        sub_rate=0.002, qual="I", seed=seed)
    if name == "interleaved_small":
        return ReadSpec(n_reads=n_reads or 20_000, lengths=(100,), n_genomes=10, glen=(40_000, 40_000),
                        sub_rate=0.005, qual="#J", interleaved=True, insert_len=300, seed=seed)
    raise KeyError(name)


def _loguniform_even(rng, lo: int, hi: int) -> int:
    import math
    n = int(math.exp(rng.uniform(math.log(lo), math.log(hi))))
    return max(2, n - (n % 2))


def serving_mix(n_jobs: int, seed: int = 11, min_reads: int = 10_000, max_reads: int = 2_000_000) -> list:
    """Partition requests: read counts log-uniform in [min_reads, max_reads] (even), 150 bp, 5-50 genomes of
    0.5-3 Mb each, log-normal abundance sigma 1.5, 1 % substitutions."""
    import random
    rng = random.Random(seed)
    return [ReadSpec(n_reads=_loguniform_even(rng, min_reads, max_reads), lengths=(150,),
                     n_genomes=rng.randint(5, 50), glen=(5e5, 3e6), gc=(0.35, 0.65), abundance=AB_LOGNORMAL,
                     ab_param=1.5, sub_rate=0.01, qual="I", seed=seed * 1000 + i) for i in range(n_jobs)]


def batch_mix(n_samples: int = 64, seed: int = 5, min_reads: int = 50_000, max_reads: int = 5_000_000,
              scale: float = 1.0) -> list:
    """Independent samples: read counts log-uniform in [min_reads, max_reads] (even; times scale), read
    length one of 100/150/250, 10-100 genomes of 0.5-3 Mb, log-normal abundance sigma 1.5, 1 % substitutions."""
    import random
    rng = random.Random(seed)
    out = []
    for i in range(n_samples):
        n = _loguniform_even(rng, min_reads, max_reads)
        n = max(2, int(n * scale) // 2 * 2)
        out.append(ReadSpec(n_reads=n, lengths=(rng.choice((100, 150, 250)),), n_genomes=rng.randint(10, 100),
                            glen=(5e5, 3e6), gc=(0.35, 0.65), abundance=AB_LOGNORMAL, ab_param=1.5, sub_rate=0.01,
                            qual="I", seed=seed * 1000 + i))
    return out
