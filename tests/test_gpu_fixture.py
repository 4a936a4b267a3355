"""The reference's 2boxclouds fixture, prepared by monki.preparation (Mie phase matrices
with F12 != 0, Rayleigh with the computed depolarization, O3 absorption), on the GPU
against the oracle: FP64 histories exactly, FP32 within combined standard error."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _scene(ppc, rounds):
    from monki.scenes import TransportScene

    tables = np.load(GOLDEN / "prepared_2boxclouds.npz")["tables"]
    return TransportScene("2boxclouds", tables, None, ppc, rounds)


def _controls(scene, rounds, seed):
    nmat, nx, ny, nz, angles = scene.shape
    per_round = scene.photons_per_column * nx * ny
    return [per_round * rounds, 0, 1, seed, 100000, 0, per_round, rounds]


def _run(scene, rounds, seed, precision):
    from monki.execution import CUDA, BatchControls

    with CUDA(precision=precision, seed=seed) as backend:
        backend.prepare(scene)
        batches = backend.run_batches([BatchControls(i, scene.photons_per_column) for i in range(1, rounds + 1)])
        return np.stack([b.stokes.ravel(order="F") for b in batches]), dict(backend.provenance)


def test_fp64_transport_of_the_prepared_fixture_reproduces_oracle(oracle, device):
    scene = _scene(4, 2)
    actual, provenance = _run(scene, 2, 23274, "fp64")
    expected, counters = oracle.run(scene.tables, _controls(scene, 2, 23274), 8)
    assert provenance["scatters"] == counters["scatters"]
    close = np.isclose(actual, expected, rtol=1e-6, atol=1e-12)
    assert close.mean() >= 0.999, f"{(~close).sum()} of {close.size} tallies differ"


def test_fp32_transport_of_the_prepared_fixture_agrees_with_oracle(oracle, device):
    rounds = 32
    scene = _scene(10, rounds)
    gpu, _ = _run(scene, rounds, 881, "fp32")
    cpu, _ = oracle.run(scene.tables, _controls(scene, rounds, 23274), 16)
    se = np.hypot(gpu.std(0, ddof=1), cpu.std(0, ddof=1)) / np.sqrt(rounds)
    mask = se > 0
    z = (gpu.mean(0) - cpu.mean(0))[mask] / se[mask]
    assert np.mean(np.abs(z) < 3) >= 0.99, np.sort(np.abs(z))[-10:]
    assert abs(np.mean(z)) < 0.1
