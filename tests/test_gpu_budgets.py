"""The FP32 product at the workloads' own photon budgets against the oracle.

The oracle's per-entry round moments (tests/golden/budget_moments.npz, made by
make_golden.py with its own seed) for: the clear sky at 2,000 photons per column x 32
rounds, the layered cloud with layer paths at 20,000 (on a 6 x 4 grid), the box cloud at
2,000, and four config-3 scenes (seed 93's draws on a 128 x 128 grid, I only, I/Q/U, and a
grid under 32 x 32) at about 40 per column. The GPU runs seed 0, the workloads' seed.

Criteria, the reference's (python/monki/validation.py:146-253, the scientific suite's):
over every tally entry (Stokes, and layer paths and weights where the scene has them),
|z| < 3 in at least 99 % of entries and |mean z| < 0.1; and the product comparator
(monki.validation.compare, statistical, Bonferroni family error 1e-6 over the combined
standard errors) accepts the GPU product of simulate() against the oracle's.
"""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "budget_moments.npz"


NAMES = ("clear_sky", "layered_cloud", "box_cloud", "batched_largest", "batched_nmat1", "batched_nmat3",
         "batched_small")


def _moments(name):
    with np.load(GOLDEN) as data:
        return {key.split(".", 1)[1]: data[key] for key in data.files if key.startswith(name + ".")}


def _scene(m):
    import monki.scenes as scenes

    args, kwargs = json.loads(str(m["args"]))
    kwargs = {k: (tuple(v) if isinstance(v, list) else v) for k, v in kwargs.items()}
    scene = getattr(scenes, str(m["builder"]))(*args, **kwargs)
    # The builder still makes the fixture's tables (up to the last bits of numpy's
    # transcendental functions, which differ between x86 and Arm).
    t = np.asarray(scene.tables, dtype=np.float64)
    assert t.size == int(m["tables_size"]), "the scene builder no longer makes the fixture's tables"
    np.testing.assert_array_equal(t[:8], m["tables_head"][:8])  # version, grid and list sizes
    np.testing.assert_allclose(t[:16], m["tables_head"], rtol=1e-10)
    stride = max(1, -(-t.size // 4096))
    np.testing.assert_allclose(t[::stride], m["tables_sample"], rtol=1e-10, atol=1e-300)
    np.testing.assert_allclose([t.sum(), np.abs(t).sum(), (t * t).sum()], m["tables_sums"], rtol=1e-10)
    return scene


def _flat(batch):
    parts = [batch.stokes.ravel(order="F")]
    if batch.weighted_paths is not None:
        parts += [batch.weighted_paths.ravel(order="F"), batch.weights.ravel(order="F")]
    return np.concatenate(parts)


def _oracle_product(product, m, scene):
    """The GPU product with its statistics replaced by the oracle's (same case)."""

    from monki.output import SimulationResult

    nmat, nx, ny, nz, angles = scene.shape
    n, ppc = int(m["rounds"]), int(m["photons_per_column"])
    pixels = nmat * nx * ny * angles
    total, squares = m["sum"][:pixels], m["squares"][:pixels]
    shape = (nmat, nx, ny, angles)
    radiance = (total / n).reshape(shape, order="F")
    error = (np.sqrt(np.maximum(squares - total * total / n, 0.0) / (n - 1)) / np.sqrt(n)).reshape(shape, order="F")
    dop = np.divide(np.sqrt(np.sum(radiance[1:] ** 2, axis=0)), radiance[0], out=np.zeros_like(radiance[0]),
                    where=radiance[0] > 1e-16)
    values = {key: value.copy() for key, value in product.values.items()}
    values["radiance"] = radiance.transpose(3, 2, 1, 0)[..., None]
    values["std_radiance"] = error.transpose(3, 2, 1, 0)[..., None]
    values["DOP"] = dop.transpose(2, 1, 0)[..., None]
    running = np.cumsum(m["history"], axis=0) / np.arange(1, n + 1)[:, None]
    values["radiance_convergence"] = running[..., None]
    if "AMF_layer" in values:
        paths = (m["sum"][pixels : pixels + nx * ny * nz * angles] * ppc).reshape((nx, ny, nz, angles), order="F")
        weights = (m["sum"][pixels + nx * ny * nz * angles :] * ppc).reshape((nx, ny, angles), order="F")
        thickness = np.diff(values["alt"]) / 1000.0
        amf = paths[:, :, :-1, :] / weights[:, :, None, :] / thickness[None, None, :, None]
        values["AMF_layer"] = amf.transpose(3, 2, 1, 0)[..., None]
    return SimulationResult(None, values, dict(product.dimensions), dict(product.attributes))


@pytest.mark.parametrize("name", NAMES)
def test_fp32_product_at_the_workload_budget_agrees_with_the_oracle(device, tmp_path, name):
    from monki import simulate
    from monki.execution import CUDA, BatchControls
    from monki.validation import compare

    from dataclasses import replace

    m = _moments(name)
    n, ppc = int(m["rounds"]), int(m["photons_per_column"])
    scene = replace(_scene(m), rounds=n)
    assert scene.photons_per_column == ppc

    # Every tally entry, per round, from the backend (seed 0).
    with CUDA(seed=0) as backend:
        backend.prepare(scene)
        x = np.stack([_flat(b) for b in backend.run_batches([BatchControls(r, ppc) for r in range(1, n + 1)])]) / ppc
    mean_o = m["sum"] / n
    var_o = np.maximum(m["squares"] - m["sum"] ** 2 / n, 0.0) / (n - 1) / n
    se = np.sqrt(x.var(0, ddof=1) / n + var_o)
    mask = se > 0
    z = (x.mean(0) - mean_o)[mask] / se[mask]
    assert z.size > 1000
    assert np.mean(np.abs(z) < 3) >= 0.99, np.sort(np.abs(z))[-10:]
    assert abs(z.mean()) < 0.1, z.mean()

    # The reference's acceptance gate on the products (simulate through the public API).
    gpu = simulate(scene, CUDA(seed=0), tmp_path / "gpu.nc")
    verdict = compare(_oracle_product(gpu, m, scene), gpu)
    assert verdict.passed, verdict.details


def test_multi_scene_session_agrees_with_the_oracle_at_the_workload_budgets(device):
    """The four config-3 scenes of the fixtures in one multi-scene session (one launch
    sequence over a shared photon pool, FP32, seed 0), 32 rounds each at their own budgets:
    every tally entry by the same z-criteria against the oracle's round moments."""

    from monki.batched import run_persistent

    names = [name for name in NAMES if name.startswith("batched_")]
    moments = [_moments(name) for name in names]
    batch = [_scene(m) for m in moments]
    rounds = int(moments[0]["rounds"])
    assert all(int(m["rounds"]) == rounds for m in moments)
    results, summary = run_persistent(batch, seed=0, rounds=rounds)
    assert summary["scenes"] == len(batch)
    for name, m, (batches, _) in zip(names, moments, results, strict=True):
        ppc = int(m["photons_per_column"])
        x = np.stack([_flat(b) for b in batches]) / ppc
        n = x.shape[0]
        mean_o = m["sum"] / n
        var_o = np.maximum(m["squares"] - m["sum"] ** 2 / n, 0.0) / (n - 1) / n
        se = np.sqrt(x.var(0, ddof=1) / n + var_o)
        mask = se > 0
        z = (x.mean(0) - mean_o)[mask] / se[mask]
        assert z.size > 1000, name
        assert np.mean(np.abs(z) < 3) >= 0.99, (name, np.sort(np.abs(z))[-10:])
        assert abs(z.mean()) < 0.1, (name, z.mean())
