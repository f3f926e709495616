"""Shared test setup: import paths, the `gpu` marker, and skip rules.

`-m gpu` tests need a CUDA device and the sm_103a library; `-m "not gpu"` tests
run on the CPU (oracle known-answer tests, host logic, ABI surface).
"""
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
for p in (ROOT / "volumefluxes.jl_gb300", ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libvfsm103.so")


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        import ctypes
        try:
            lib = ctypes.CDLL("libcuda.so.1")
            n = ctypes.c_int()
            return lib.cuInit(0) == 0 and lib.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
        except OSError:
            return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
