"""Pins the CPU oracle to the reference: its outputs must have the digests the reference programs produced
(tests/golden/golden.json, written by tests/golden/make_golden.py from oracle/_ref runs)."""
import hashlib
import json
from pathlib import Path

import pytest

import pipeline_util as pu

HERE = Path(__file__).resolve().parent
GOLDEN = json.loads((HERE / "golden" / "golden.json").read_text())


def _input(case):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", HERE / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    from metapart_gb300 import build
    return mg.make_input(tuple(case["gen"]), build.reference_root(), case["params"]["k"],
                         case["params"].get("min3", False))


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_oracle_matches_reference_digests(tmp_path, built, name):
    case = GOLDEN[name]
    data = _input(case)
    if data is None:
        pytest.skip("the reference's bundled fixture is not present on this machine")
    if hashlib.sha256(data).hexdigest() != case["input_sha256"]:
        pytest.skip("the regenerated input differs from the one the digests were taken on (other libm)")
    fq = tmp_path / "in.fastq"
    fq.write_bytes(data)
    p = pu.Params(**case["params"])
    got = pu.digests(pu.outputs(pu.run("oracle", tmp_path, [fq], p), p, "in.fastq"))
    want = case["outputs"]
    assert sorted(got) == sorted(want)
    assert [k for k in want if got[k] != want[k]] == []
