"""The C ABI library loads and exports every entry point include/metapart_gpu.h declares; without a GPU
the context call fails with a typed error (there is no CPU fallback)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared():
    h = (ROOT / "include" / "metapart_gpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(mp_\w+)\s*\(", h, re.M)))


def test_header_declares_entry_points():
    names = declared()
    for n in ["mp_ctx_create", "mp_fastq_index", "mp_job_load_fastq", "mp_job_count", "mp_job_partition",
              "mp_job_output", "mp_job_labels", "mp_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol(built_gpu):
    lib = ctypes.CDLL(str(ROOT / "metapart_gb300" / "_build" / "libmetapart_gpu.so"))
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert missing == []


def test_no_gpu_is_an_error_not_a_fallback(built_gpu):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from metapart_gb300 import native
    with pytest.raises(native.MetapartError):
        native.Context(0)
