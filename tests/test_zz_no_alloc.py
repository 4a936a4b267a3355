"""The allocation-free entry point (monki_cuda_run_static) against the session path.

Callers that cannot call cudaMalloc (their host application owns all device memory, or
they must not allocate once running) use monki_cuda_run_static, whose device scratch is
a fixed 16 MiB array inside the library. Two consecutive calls must each reproduce what
monki_cuda_create + monki_cuda_run return for the same round group with the same kernel
(one FP32 tally bank), up to the order of floating-point atomic additions.

This file is collected last so that a run stopping at the first failure has already run
every other test.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 2e-5, 2e-5  # FP32 atomic summation order only


def _session_run(native, tables, controls):
    from monki.execution.native import F64P

    err = ctypes.create_string_buffer(1024)
    handle = native.monki_cuda_create(
        0, tables.ctypes.data_as(F64P), tables.size, int(controls[7]), b"precision=fp32,engine=megakernel,shards=1", err, len(err)
    )
    assert handle, err.value
    try:
        out = np.zeros(int(native.monki_cuda_tally_count(handle)) * int(controls[7]))
        ctl = (ctypes.c_uint32 * 8)(*controls)
        assert native.monki_cuda_run(handle, ctl, out.ctypes.data_as(F64P), err, len(err)) == 0, err.value
        return out
    finally:
        native.monki_cuda_close(handle)


def _static_run(native, tables, controls, size):
    from monki.execution.native import F64P

    err = ctypes.create_string_buffer(1024)
    out = np.full(size, np.nan)
    ctl = (ctypes.c_uint32 * 8)(*controls)
    status = native.monki_cuda_run_static(0, tables.ctypes.data_as(F64P), tables.size, ctl, out.ctypes.data_as(F64P), err, len(err))
    assert status == 0, err.value
    return out


def test_static_scratch_matches_session_on_consecutive_calls(native, device):
    import monki.scenes as scenes

    scene = scenes.layered_cloud(16, 2, nx=10, ny=8)
    tables = np.ascontiguousarray(scene.tables)
    nmat, nx, ny, nz, angles = scene.shape
    per_round = 16 * nx * ny
    first = [per_round, 0, 1, 7, 100000, 0, per_round, 1]
    second = [2 * per_round, 0, 2, 7, 100000, 0, per_round, 2]
    expected = [_session_run(native, tables, first), _session_run(native, tables, second)]
    actual = [_static_run(native, tables, first, expected[0].size), _static_run(native, tables, second, expected[1].size)]

    for got, want in zip(actual, expected, strict=True):
        assert np.all(np.isfinite(got))
        assert got[:nmat].sum() != 0
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=ATOL)


def test_static_scratch_rejects_oversized_scenes(native, device):
    import monki.scenes as scenes
    from monki.execution.native import F64P

    scene = scenes.layered_cloud(1, 1, nx=128, ny=96)
    tables = np.ascontiguousarray(scene.tables)
    per_round = 128 * 96
    ctl = (ctypes.c_uint32 * 8)(per_round, 0, 1, 0, 100000, 0, per_round, 1)
    out = np.zeros(8)
    err = ctypes.create_string_buffer(1024)
    status = native.monki_cuda_run_static(0, tables.ctypes.data_as(F64P), tables.size, ctl, out.ctypes.data_as(F64P), err, len(err))
    assert status == 1
    assert b"16 MiB" in err.value
