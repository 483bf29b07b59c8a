"""The C-ABI library builds, loads without a GPU, exports every function that
include/xcgpu.h declares, and fails loudly (no CPU fallback) when no device exists."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "xcgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xcgpu_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from serenity_gb300 import build
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (xcgpu_\w+)", out))
    missing = [s for s in declared() if s not in exported]
    assert not missing, missing
    L = ctypes.CDLL(lib)
    for s in declared():
        getattr(L, s)


def test_no_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from serenity_gb300 import xcgpu
    with pytest.raises(xcgpu.XcgpuError):
        xcgpu.Context()
