"""The GPU drop-in programs against the reference's golden digests directly (cases whose input regenerates
bit-identically on this machine)."""
import hashlib
import json
from pathlib import Path

import pytest

import pipeline_util as pu
from test_oracle_golden import _input

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent
GOLDEN = json.loads((HERE / "golden" / "golden.json").read_text())


def _comparable(key: str, scans: int) -> bool:
    if key.startswith("dump/pe_"):        # state inside the reference's sequential mate-union loop
        return False
    if key.startswith("dump/stats") and key.endswith("_sizes.bin"):
        return int(key[len("dump/stats"):-len("_sizes.bin")]) >= scans
    return True


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_gpu_matches_reference_digests(tmp_path, built_gpu, name):
    case = GOLDEN[name]
    data = _input(case)
    if data is None:
        pytest.skip("the reference's bundled fixture is not present on this machine")
    if hashlib.sha256(data).hexdigest() != case["input_sha256"]:
        pytest.skip("the regenerated input differs from the one the digests were taken on")
    fq = tmp_path / "in.fastq"
    fq.write_bytes(data)
    p = pu.Params(**case["params"])
    got = pu.digests(pu.outputs(pu.run("gpu", tmp_path, [fq], p), p, "in.fastq"))
    want = {k: v for k, v in case["outputs"].items() if _comparable(k, p.scans)}
    assert [k for k in want if got.get(k) != want[k]] == []
