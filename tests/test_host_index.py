"""Host-side chunk indexer of the library (mp_fastq_index, no GPU needed) against the oracle's genFastqIdx
and, where built, the reference's; the drop-in genFastqIdx program writes the same .idx bytes."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pipeline_util as pu
from metapart_gb300 import native, synth

ROOT = Path(__file__).resolve().parent.parent


def _idx_headers(path):
    b = Path(path).read_bytes()
    out = []
    for i in range(0, len(b), pu.REC):
        out.append((int.from_bytes(b[i + 24:i + 28], "little", signed=True), int.from_bytes(b[i:i + 8], "little")))
    return out


@pytest.mark.parametrize("name,n,chunks", [("plain_small", 5000, 4), ("plain_small", 5000, 7),
                                           ("interleaved_small", 6000, 5), ("plain_large", 3000, 16),
                                           ("min3", 1000, 3)])
def test_index_matches_oracle(tmp_path, built_gpu, name, n, chunks):
    data = synth.fastq_bytes(synth.workload(name, n, seed=4))
    il = name.startswith("interleaved")
    fno, ofs = native.fastq_index(chunks, [data], interleaved=il)
    fq = tmp_path / "in.fastq"
    fq.write_bytes(data)
    kinds = ["0", "0", "1"] if il else ["0", "1", "0"]
    subprocess.run([str(ROOT / "oracle" / "_build" / "mpo_cli"), "genFastqIdx", str(chunks), *kinds, "in.fastq"],
                   cwd=tmp_path, check=True, capture_output=True)
    want = _idx_headers(tmp_path / "in.fastq.idx")
    assert list(zip(fno.tolist(), ofs.tolist())) == want
    d2 = tmp_path / "gpu"
    d2.mkdir()
    (d2 / "in.fastq").write_bytes(data)
    subprocess.run([str(ROOT / "metapart_gb300" / "_build" / "bin" / "genFastqIdx"), str(chunks), *kinds,
                    "in.fastq"], cwd=d2, check=True, capture_output=True)
    assert pu.masked_index(d2 / "in.fastq.idx") == pu.masked_index(tmp_path / "in.fastq.idx")


def test_index_multi_file(tmp_path, built_gpu):
    a = synth.fastq_bytes(synth.workload("plain_small", 1500, seed=1))
    b = synth.fastq_bytes(synth.workload("plain_small", 2500, seed=2))
    fno, ofs = native.fastq_index(6, [a, b])
    (tmp_path / "a.fastq").write_bytes(a)
    (tmp_path / "b.fastq").write_bytes(b)
    subprocess.run([str(ROOT / "oracle" / "_build" / "mpo_cli"), "genFastqIdx", "6", "0", "2", "0", "a.fastq",
                    "b.fastq"], cwd=tmp_path, check=True, capture_output=True)
    assert list(zip(fno.tolist(), ofs.tolist())) == _idx_headers(tmp_path / "a.fastq.idx")


def test_index_rejects_two_file_paired_end(built_gpu):
    a = synth.fastq_bytes(synth.workload("plain_small", 100, seed=1))
    arr = (native.C.c_char_p * 2)(a, a)
    sizes = np.array([len(a), len(a)], dtype=np.uint64)
    fno = np.zeros(5, dtype=np.int32)
    ofs = np.zeros(5, dtype=np.uint64)
    cnt = native.C.c_int()
    rc = native.lib().mp_fastq_index(4, 1, 0, 0, 2, arr, native._p64(sizes),
                                     fno.ctypes.data_as(native.C.POINTER(native.C.c_int32)), native._p64(ofs),
                                     native.C.byref(cnt))
    assert rc == -5 and b"paired" in native.lib().mp_last_error()
