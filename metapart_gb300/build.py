"""In-tree build of the native parts.

Products (git-ignored, rebuilt on every machine -- x86 here, aarch64 on the GPU host):
  metapart_gb300/_build/libmetapart_gpu.so   CUDA sm_103a kernels + C ABI (include/metapart_gpu.h)
  metapart_gb300/_build/libmp_synth.so       seeded synthetic FASTQ generator
  metapart_gb300/_build/bin/*                drop-in stage programs (genFastqIdx, genHistograms_metapart[min],
                                             metapart[min]) linked against libmetapart_gpu.so
Test infrastructure (also git-ignored):
  oracle/_build/libmpo.so, oracle/_build/mpo_cli   CPU oracle
  oracle/_ref/*                                    reference programs, only where the reference sources exist
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
CLI = PKG / "cli"
BUILD = PKG / "_build"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"
# Where oracle/build_ref.sh found the reference sources it built from (written by the recipe); the
# reference's own test fixture is read from there.
REFERENCE_ROOT_FILE = ORACLE / "_ref" / "REFERENCE_ROOT"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
CUDA_HOME = Path(NVCC).resolve().parent.parent

CU_SOURCES = ["mp_api.cu", "mp_batch.cu", "mp_server.cu", "k_reads.cu", "k_kmers.cu", "k_sort.cu", "k_graph.cu", "k_output.cu"]
CLI_PROGRAMS = {
    "genFastqIdx": ("genFastqIdx.c", []),
    "genHistograms_metapart": ("genHistograms.c", []),
    "genHistograms_metapartmin": ("genHistograms.c", ["-DMIN3"]),
    "metapart": ("metapart.c", []),
    "metapartmin": ("metapart.c", ["-DMIN3"]),
}


def _run(cmd: list[str], cwd: Path | None = None) -> None:
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build_oracle(force: bool = False) -> None:
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    deps = [ORACLE / "mp_oracle.c", ORACLE / "mp_oracle.h", ORACLE / "mpo_cli.c"]
    jobs = []
    lib = ORACLE_BUILD / "libmpo.so"
    cli = ORACLE_BUILD / "mpo_cli"
    if force or _stale(lib, deps):
        jobs.append(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-o", str(lib), str(ORACLE / "mp_oracle.c")])
    if force or _stale(cli, deps):
        jobs.append(["gcc", "-O3", "-fopenmp", "-o", str(cli), str(ORACLE / "mpo_cli.c"), str(ORACLE / "mp_oracle.c")])
    with ThreadPoolExecutor(4) as ex:
        list(ex.map(_run, jobs))


def build_reference(force: bool = False) -> bool:
    """Builds the reference programs into oracle/_ref when the reference sources are present (the recipe
    oracle/build_ref.sh knows where; MP_REFERENCE_ROOT overrides it).  False when they are absent."""
    marker = ORACLE / "_ref" / "metapart_dumpmin"
    deps = [ORACLE / "build_ref.sh", ORACLE / "ref_hooks.c", ORACLE / "mpi_shim" / "mpi.h"]
    if not (force or _stale(marker, deps)):
        return True
    root = os.environ.get("MP_REFERENCE_ROOT")
    r = subprocess.run(["bash", str(ORACLE / "build_ref.sh"), *([root] if root else [])], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    if r.returncode == 2:  # the recipe found no reference sources
        return False
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): oracle/build_ref.sh\n{r.stdout}")
    return True


def reference_root() -> Path | None:
    """The reference source tree oracle/_ref was built from, or None where it was not built."""
    try:
        p = Path(REFERENCE_ROOT_FILE.read_text().strip())
    except OSError:
        return None
    return p if (p / "src" / "metapart.c").exists() else None


def build_synth(force: bool = False) -> None:
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / "libmp_synth.so"
    if force or _stale(out, [CSRC / "synth.c", CSRC / "synth.h"]):
        _run(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-o", str(out), str(CSRC / "synth.c"), "-lm"])


def build_gpu(force: bool = False) -> None:
    BUILD.mkdir(parents=True, exist_ok=True)
    obj_dir = BUILD / "obj"
    obj_dir.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "metapart_gpu.h"]
    common = [NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-O3",
              "-I", str(ROOT / "include"), "-I", str(CSRC), "--expt-relaxed-constexpr"]
    jobs, objs = [], []
    for src in CU_SOURCES:
        o = obj_dir / (src + ".o")
        objs.append(o)
        if force or _stale(o, [CSRC / src, *headers]):
            jobs.append(common + ["-c", str(CSRC / src), "-o", str(o)])
    with ThreadPoolExecutor(len(CU_SOURCES)) as ex:
        list(ex.map(_run, jobs))
    lib = BUILD / "libmetapart_gpu.so"
    if force or jobs or _stale(lib, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    bindir = BUILD / "bin"
    bindir.mkdir(exist_ok=True)
    cli_jobs = []
    for name, (src, flags) in CLI_PROGRAMS.items():
        out = bindir / name
        deps = [CLI / src, CLI / "cli_common.h", ROOT / "include" / "metapart_gpu.h", lib]
        if force or _stale(out, deps):
            cli_jobs.append(["gcc", "-O2", "-Wall", *flags, "-I", str(ROOT / "include"), "-o", str(out), str(CLI / src),
                             "-L", str(BUILD), "-lmetapart_gpu", f"-Wl,-rpath,{BUILD}", "-Wl,-rpath,$ORIGIN/.."])
    with ThreadPoolExecutor(5) as ex:
        list(ex.map(_run, cli_jobs))


def build_all(force: bool = False, gpu: bool = True) -> None:
    with ThreadPoolExecutor(3) as ex:
        futs = [ex.submit(build_oracle, force), ex.submit(build_synth, force), ex.submit(build_reference, force)]
        if gpu:
            futs.append(ex.submit(build_gpu, force))
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("build ok")
