"""Device FP64 round statistics against the host driver's.

The same scene, seed and rounds through ``simulate`` twice: once with the round sums,
sums of squares and AMF moments folded on the GPU (``CUDA(device_statistics=True)``,
the default, which after the first check also runs the rounds the last check says are
still needed as one held group, folded and checked round by round) and once from each
round's tallies on the host (the reference driver's loop). FP64 transport keeps the per-round tallies equal up to the order of the device's
atomic sums, so the products agree to 1e-9 (the AMF standard error, a difference of
nearly equal moments, to 1e-6) and the stopping decisions match.
"""

from __future__ import annotations

import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ("radiance", "std_radiance", "DOP", "radiance_convergence", "AMF_layer", "std_AMF_layer")


def _simulate(tmp_path, tag, scene, convergence, device_statistics):
    from monki import simulate
    from monki.execution import CUDA

    backend = CUDA(precision="fp64", seed=77, device_statistics=device_statistics)
    result = simulate(scene, backend, tmp_path / f"{tag}.nc", convergence=convergence)
    receipt = json.loads((tmp_path / f"{tag}.run.json").read_text())
    return result, receipt


@pytest.mark.parametrize("kind", ["layered_amf", "box_radiance", "box_fixed"])
def test_device_statistics_equal_host_statistics(tmp_path, device, kind):
    import monki.scenes as scenes
    from monki import AMFConvergence, RadianceConvergence

    if kind == "layered_amf":
        scene = scenes.layered_cloud(40, 64, nx=10, ny=8)
        convergence = AMFConvergence(0.2, minimum_rounds=32, check_every=8, consecutive_checks=2)
    elif kind == "box_radiance":
        scene = scenes.box_cloud(40, 64, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
        convergence = RadianceConvergence(0.2, minimum_rounds=32, check_every=4, consecutive_checks=2)
    else:
        scene = scenes.box_cloud(20, 36, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
        convergence = None
    device, r_device = _simulate(tmp_path, "device", scene, convergence, True)
    host, r_host = _simulate(tmp_path, "host", scene, convergence, False)
    assert r_device["completed_rounds"] == r_host["completed_rounds"]
    assert r_device["status"] == r_host["status"]
    for key in ("amf_convergence", "radiance_convergence"):
        if key in r_host:
            a, b = r_device[key]["checks"], r_host[key]["checks"]
            assert [c["rounds"] for c in a] == [c["rounds"] for c in b]
            assert [c["below_target"] for c in a] == [c["below_target"] for c in b]
            np.testing.assert_allclose([c["max_relative_se"] for c in a], [c["max_relative_se"] for c in b], rtol=1e-9)
    for name in NAMES:
        if name in host.values:
            # The AMF standard error subtracts nearly equal moments, which magnifies the
            # last-bit differences of the two runs' atomic sums in thin upper layers.
            rtol = 1e-6 if name == "std_AMF_layer" else 1e-9
            np.testing.assert_allclose(device.values[name], host.values[name], rtol=rtol, atol=1e-15, err_msg=name)
    # The device path copied no per-round tallies: one dispatch per group, statistics on the GPU.
    assert r_device["gpu_dispatches"] <= r_host["gpu_dispatches"]


def test_statistics_accumulate_and_reset(device):
    import monki.scenes as scenes
    from monki.execution import CUDA, BatchControls

    scene = scenes.box_cloud(10, 4, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    with CUDA(precision="fp64", seed=5) as backend:
        backend.prepare(scene)
        rows = backend.accumulate([BatchControls(i, 10) for i in (1, 2, 3)])
        stats = backend.statistics()
        assert stats["rounds"] == 3 and rows.shape == (3, 3)
        # Per-round spatial sums add up to the summed normalized tallies.
        np.testing.assert_allclose(rows.sum(axis=0), stats["sum"].sum(axis=(1, 2, 3)), rtol=1e-12)
        np.testing.assert_allclose(stats["total"] / 10.0, stats["sum"], rtol=1e-12)
        backend.reset_statistics()
        assert backend.statistics()["rounds"] == 0 and not np.any(backend.statistics()["sum"])
        backend.accumulate([BatchControls(4, 10)])
        assert backend.statistics()["rounds"] == 1
