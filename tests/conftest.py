"""Shared fixtures: the in-tree package path, the oracle, and the GPU marker.

Tests marked ``gpu`` run the sm_103a library on a GB300 and compare it with the CPU
oracle; everything else runs on CPU only.
"""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PACKAGE = ROOT / "monki-gpu_gb300"

for path in (str(ROOT), str(PACKAGE)):
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as module

    module.library()
    return module


@pytest.fixture(scope="session")
def native():
    """The CUDA library, built in-tree; GPU tests fail loudly when it is missing."""

    from monki.execution import native as binding

    return binding.load()


@pytest.fixture(scope="session")
def device(native):
    import ctypes

    import numpy as np

    out = np.zeros(1, dtype=np.float32)
    err = ctypes.create_string_buffer(256)
    status = native.monki_cuda_probe_uniforms(0, 0, 0, 0, 1, out.ctypes.data_as(binding_f32()), err, len(err))

    if status:
        pytest.fail(f"No usable CUDA device: {err.value.decode()}")

    return 0


def binding_f32():
    from monki.execution import native as binding

    return binding.F32P
