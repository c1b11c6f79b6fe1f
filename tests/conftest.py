"""Test configuration: the `gpu` marker (tests that need a CUDA device) and shared helpers."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libsi_cuda)")


_GPU = None


def has_gpu():
    """True when the CUDA driver reports a device (asked through libcuda, no framework import)."""
    global _GPU
    if _GPU is None:
        import ctypes
        try:
            cu = ctypes.CDLL("libcuda.so.1")
            n = ctypes.c_int(0)
            _GPU = cu.cuInit(0) == 0 and cu.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
        except OSError:
            _GPU = False
    return _GPU


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def mulberry32(seed):
    """The reference test harness's PRNG (tests/harness.js:59-66)."""
    state = [seed & 0xFFFFFFFF]

    def imul(a, b):
        return ((a & 0xFFFFFFFF) * (b & 0xFFFFFFFF)) & 0xFFFFFFFF

    def r():
        s = (state[0] + 0x6D2B79F5) & 0xFFFFFFFF
        state[0] = s
        t = imul(s ^ (s >> 15), 1 | s)
        t = ((t + imul(t ^ (t >> 7), 61 | t)) & 0xFFFFFFFF) ^ t
        return ((t ^ (t >> 14)) & 0xFFFFFFFF) / 4294967296
    return r


@pytest.fixture
def rng():
    return np.random.default_rng(1234)
