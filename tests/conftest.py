import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger CPU cases")


@pytest.fixture(scope="session")
def built():
    from metapart_gb300 import build
    build.build_oracle()
    build.build_synth()
    build.build_reference()
    return build


@pytest.fixture(scope="session")
def built_gpu(built):
    built.build_gpu()
    return built
