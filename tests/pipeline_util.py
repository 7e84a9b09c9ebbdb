"""Runs the three stage programs of one implementation in a directory and collects the outputs.

Implementations: "ref" (the reference programs built into oracle/_ref), "oracle" (the CPU restatement
oracle/_build/mpo_cli) and "gpu" (the drop-in programs in metapart_gb300/_build/bin).  All three write the
same files, so every comparison is a byte comparison (index padding masked).
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from dataclasses import dataclass
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
REC = 4194344


@dataclass
class Params:
    k: int = 27
    chunks: int = 4
    scans: int = 1
    threads: int = 2
    min3: bool = False
    interleaved: bool = False
    buffer: int = 1 << 30


def _cmds(impl: str, p: Params, files: list[str], out: str):
    kinds = ["0", "0", "1"] if p.interleaved else ["0", str(len(files)), "0"]
    kinds[2] = str(len(files)) if p.interleaved else "0"
    suffix = "min" if p.min3 else ""
    if impl == "ref":
        b = ROOT / "oracle" / "_ref"
        idx = [str(b / "genFastqIdx"), str(p.chunks), *kinds, *files]
        hist = [str(b / f"genHistograms_metapart{suffix}"), str(p.k), *kinds, *files]
        mp = [str(b / f"metapart_dump{suffix}"), "-o", out, str(p.buffer), str(p.k), str(p.scans), str(p.threads),
              *kinds, *files]
    elif impl == "oracle":
        c = str(ROOT / "oracle" / "_build" / "mpo_cli")
        m3 = ["--min3"] if p.min3 else []
        idx = [c, "genFastqIdx", str(p.chunks), *kinds, *files]
        hist = [c, "genHistograms", *m3, str(p.k), *kinds, *files]
        mp = [c, "metapart", *m3, "-o", out, str(p.buffer), str(p.k), str(p.scans), str(p.threads), *kinds, *files]
    elif impl == "gpu":
        b = ROOT / "metapart_gb300" / "_build" / "bin"
        idx = [str(b / "genFastqIdx"), str(p.chunks), *kinds, *files]
        hist = [str(b / f"genHistograms_metapart{suffix}"), str(p.k), *kinds, *files]
        mp = [str(b / f"metapart{suffix}"), "-o", out, str(p.buffer), str(p.k), str(p.scans), str(p.threads),
              *kinds, *files]
    else:
        raise ValueError(impl)
    return idx, hist, mp


def run(impl: str, workdir: Path, fastqs: list[Path], p: Params, dump: bool = True, env_extra=None) -> Path:
    """Copies the FASTQ files into workdir/impl and runs the three stages there.  Returns that directory."""
    d = workdir / impl
    if d.exists():
        shutil.rmtree(d)
    (d / "out" / "Rank0").mkdir(parents=True)
    (d / "dump").mkdir()
    files = []
    for f in fastqs:
        shutil.copyfile(f, d / f.name)
        files.append(f.name)
    env = dict(os.environ)
    env["OMP_STACKSIZE"] = "16M"
    env.setdefault("OMP_NUM_THREADS", "4")
    if dump:
        env["MP_DUMP_DIR"] = str(d / "dump")
    if env_extra:
        env.update(env_extra)
    idx, hist, mp = _cmds(impl, p, files, "./out")
    for cmd, extra in ((idx, {}), (hist, {"OMP_NUM_THREADS": "1"} if impl == "ref" else {}), (mp, {})):
        e = dict(env)
        e.update(extra)
        r = subprocess.run(cmd, cwd=d, env=e, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                           timeout=1800)
        (d / (Path(cmd[0]).name + ".log")).write_text(r.stdout[-200_000:])
        if r.returncode != 0:
            raise RuntimeError(f"{impl}: {' '.join(cmd)} exited {r.returncode}\n{r.stdout[-4000:]}")
    return d


def masked_index(path: Path) -> bytes:
    b = bytearray(path.read_bytes())
    for i in range(0, len(b), REC):
        b[i + 17:i + 20] = b"\0\0\0"
        b[i + REC - 4:i + REC] = b"\0\0\0\0"
    return bytes(b)


def outputs(d: Path, p: Params, fastq_name: str) -> dict[str, bytes]:
    """All comparable outputs of one run: index files (masked), histogram, partition files, stage dumps."""
    m = "_3min" if p.min3 else ""
    res = {
        "idx": masked_index(d / f"{fastq_name}.idx"),
        "kmeridx": masked_index(d / f"{fastq_name}.KmerIdx{m}{p.k}"),
        "kmerhist": (d / f"{fastq_name}.kmerHist{m}{p.k}").read_bytes(),
    }
    for f in sorted((d / "out" / "Rank0").iterdir()):
        res["part/" + f.name] = f.read_bytes()
    for f in sorted((d / "dump").iterdir()):
        res["dump/" + f.name] = f.read_bytes()
    return res


def digests(res: dict[str, bytes]) -> dict[str, str]:
    return {k: hashlib.sha256(v).hexdigest() for k, v in res.items()}


def diff_keys(a: dict, b: dict, keys=None) -> list[str]:
    ks = keys if keys is not None else sorted(set(a) | set(b))
    return [k for k in ks if a.get(k) != b.get(k)]
