"""Scattering-order diagnostics on the GPU against the oracle and through simulate().

The reference computes them in calc_radiances_and_scats
(mc_routines_cartesian_mod.f90:405-836): single-scattering Stokes by pixel and the
contribution of every event location (layer 0 = the surface), all orders and single.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _box(ppc, rounds):
    import monki.scenes as scenes

    return scenes.box_cloud(ppc, rounds, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))


def test_fp64_order_tallies_reproduce_oracle(oracle, device):
    from monki.execution import CUDA, BatchControls

    scene = _box(8, 2)
    nmat, nx, ny, nz, angles = scene.shape
    per_round = 8 * nx * ny
    with CUDA(precision="fp64", seed=23274, orders=True) as backend:
        backend.prepare(scene)
        batches = backend.run_batches([BatchControls(i, 8) for i in (1, 2)])
    expected, _ = oracle.run(scene.tables, [per_round * 2, 0, 1, 23274, 100000, 0, per_round, 2], 8, orders=True)
    for batch, row in zip(batches, expected, strict=True):
        single, located, located_single = oracle.split_orders(scene.tables, row)
        for name, ref in (("single", single), ("locations", located), ("single_locations", located_single)):
            close = np.isclose(batch.orders[name], ref, rtol=1e-6, atol=1e-12)
            assert close.mean() == 1.0, (name, (~close).sum())


def test_simulate_writes_order_products(tmp_path, device):
    from monki import SimulationResult, simulate
    from monki.execution import CUDA

    scene = _box(50, 4)
    result = simulate(scene, CUDA(orders=True), tmp_path / "orders.nc")
    v = result.values
    np.testing.assert_allclose(v["radiance_sing"] + v["radiance_mult"], v["radiance"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(v["contrib_radiance_3D_sing"] + v["contrib_radiance_3D_mult"], v["contrib_radiance_3D"],
                               rtol=1e-12, atol=1e-15)
    # All contributions, by location, add up to all radiance, by pixel (FP32 tallies in
    # different records: equal to single-precision rounding).
    np.testing.assert_allclose(v["contrib_radiance_3D"].sum(axis=(1, 2, 3)), v["radiance"].sum(axis=(1, 2)), rtol=1e-5)
    assert v["contrib_radiance_3D"].shape[1] == scene.shape[3]  # surface + physical layers
    loaded = SimulationResult.load(tmp_path / "orders.nc")
    np.testing.assert_allclose(loaded.values["radiance_mult"], v["radiance_mult"])
