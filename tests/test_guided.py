"""Guided transport on the CPU oracle: unbiasedness, determinism and the importance tally.

The guided method (detector-directed sampling at particle scatters plus Russian
roulette, each with its exact weight correction) must keep the analog estimator's
expectation. These tests check that on small scenes against the analog method with
independent streams, and pin the bookkeeping the GPU kernels reproduce.
"""

from __future__ import annotations

import numpy as np
import pytest


def _controls(scene, rounds, seed, first_round=1):
    nmat, nx, ny, nz, angles = scene.shape
    per_round = scene.photons_per_column * nx * ny
    return [per_round * rounds, 0, first_round, seed, 100000, 0, per_round, rounds]


def _small_box(ppc=40, rounds=32):
    import monki.scenes as scenes

    return scenes.box_cloud(ppc, rounds, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))


def _stokes_rounds(oracle, scene, values):
    return np.stack([oracle.split(scene.tables, row)[0] for row in values])


def _z(a, b):
    n = a.shape[0]
    se = np.hypot(a.std(0, ddof=1), b.std(0, ddof=1)) / np.sqrt(n)
    mask = se > 0
    return (a.mean(0) - b.mean(0))[mask] / se[mask]


# Every case keeps the weights bounded (a DDIS cap): with epsilon > 0 and no cap, photons
# that keep the analog branch gain 1 / (1 - epsilon) per scatter and the estimator, still
# unbiased, has tails too heavy for a z-test.
@pytest.mark.parametrize("guide", [(0.0, 1.0, 0.0), (0.3, 0.5, 1.5), (0.5, 0.0, 1.2)])
def test_guided_estimates_agree_with_analog_within_combined_se(oracle, guide):
    scene = _small_box()
    plain, _ = oracle.run(scene.tables, _controls(scene, 32, 11), 8)
    guided, counters = oracle.run(scene.tables, _controls(scene, 32, 12), 8, guide=guide)
    z = _z(_stokes_rounds(oracle, scene, guided), _stokes_rounds(oracle, scene, plain))
    assert np.mean(np.abs(z) < 3) >= 0.98, np.sort(np.abs(z))[-8:]
    assert abs(z.mean()) < 0.3
    # Pooled over every pixel and view: the scene-mean intensity agrees tightly.
    gi = _stokes_rounds(oracle, scene, guided)[:, 0].sum(axis=(1, 2, 3))
    pi = _stokes_rounds(oracle, scene, plain)[:, 0].sum(axis=(1, 2, 3))
    pooled = (gi.mean() - pi.mean()) / np.hypot(gi.std(ddof=1), pi.std(ddof=1)) * np.sqrt(32)
    assert abs(pooled) < 4
    assert counters["scatters"] > 0


def test_roulette_cuts_the_cost_of_light_photons(oracle):
    scene = _small_box(ppc=20, rounds=4)
    _, plain = oracle.run(scene.tables, _controls(scene, 4, 5), 8)
    _, guided = oracle.run(scene.tables, _controls(scene, 4, 5), 8, guide=(0.0, 1.0, 0.0))
    assert guided["photons"] == plain["photons"]
    assert guided["scatters"] < 0.6 * plain["scatters"]


def test_unit_scale_map_equals_constant_roulette_and_zero_map_disables_it(oracle):
    scene = _small_box(ppc=10, rounds=2)
    nmat, nx, ny, nz, angles = scene.shape
    controls = _controls(scene, 2, 7)
    # One thread: the summation order, and so every bit, is then fixed.
    constant, c0 = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.7, 0.0))
    mapped, c1 = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.7, 0.0), scale=np.ones((nx, ny, nz)))
    np.testing.assert_array_equal(constant, mapped)
    assert c0 == c1
    plain, p0 = oracle.run(scene.tables, controls, 1)
    off, p1 = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.7, 0.0), scale=np.zeros((nx, ny, nz)))
    np.testing.assert_array_equal(plain, off)
    assert p0 == p1


def test_analog_guide_reproduces_the_analog_run(oracle):
    scene = _small_box(ppc=10, rounds=2)
    controls = _controls(scene, 2, 9)
    plain, _ = oracle.run(scene.tables, controls, 1)
    same, _ = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.0, 0.0))
    np.testing.assert_array_equal(plain, same)


def test_importance_tally_counts_every_event(oracle):
    scene = _small_box(ppc=10, rounds=2)
    nmat, nx, ny, nz, angles = scene.shape
    out, counters, importance = oracle.run(scene.tables, _controls(scene, 2, 3), 4, importance=True)
    assert importance.shape == (2, nx, ny, nz)
    assert importance[1].sum() == counters["scatters"]
    assert np.all(importance[0] >= 0) and np.all(np.isfinite(importance[0]))
    # The vacuum layer never hosts an event; the cloud's cells do.
    assert importance[1][:, :, nz - 1].sum() == 0
    assert importance[1][3:8, 2:6, :].sum() > 0
    # Every contribution is credited to its own event at least: the ring sum exceeds the
    # tallied Stokes-I (before the mu0/mu factor) of the first-order events alone.
    assert importance[0].sum() > 0


def test_guide_settings_are_validated(oracle):
    from monki import Guided

    scene = _small_box(ppc=2, rounds=1)
    for bad in ((1.0, 0.0, 0.0), (-0.1, 0.0, 0.0), (0.0, 1.5, 0.0)):
        with pytest.raises(RuntimeError, match="Invalid guide"):
            oracle.run(scene.tables, _controls(scene, 1, 1), 2, guide=bad)
    with pytest.raises(RuntimeError, match="split"):
        oracle.run(scene.tables, _controls(scene, 1, 1), 2, guide=(0.0, 0.5, 0.0, 0.5))
    for kwargs in ({"epsilon": 1.0}, {"roulette": -1.0}, {"roulette": 2.0}, {"cap": -1.0}, {"epsilon": float("nan")},
                   {"split": 0.5}, {"split": 2.0, "roulette": 0.0}):
        with pytest.raises(ValueError):
            Guided(**kwargs)
    assert Guided(0.25, 0.5, 1.5).oracle() == (0.25, 0.5, 1.5, 0.0)
    assert "epsilon=0.25" in Guided(0.25, 0.5, 1.5).config()
    assert "split" not in Guided(0.25, 0.5, 1.5).config() and "split=2.0" in Guided(0.0, 0.5, 0.0, 2.0).config()


def test_scattering_order_tallies_add_up(oracle):
    """Single scattering is part of the total; every contribution is booked once by its
    pixel and once by its event location (layer 0 = the surface)."""
    scene = _small_box(ppc=10, rounds=1)
    nmat, nx, ny, nz, angles = scene.shape
    out, _ = oracle.run(scene.tables, _controls(scene, 1, 13), 4, orders=True)
    plain, _ = oracle.run(scene.tables, _controls(scene, 1, 13), 4)
    stokes = oracle.split(scene.tables, out[0])[0]
    np.testing.assert_allclose(stokes, oracle.split(scene.tables, plain[0])[0], rtol=1e-12, atol=1e-15)
    single, located, located_single = oracle.split_orders(scene.tables, out[0])
    assert np.all(single[0] <= stokes[0] + 1e-15) and single[0].sum() > 0
    np.testing.assert_allclose(located.sum(axis=(1, 2, 3)), stokes.sum(axis=(1, 2)), rtol=1e-12)
    np.testing.assert_allclose(located_single.sum(axis=(1, 2, 3)), single.sum(axis=(1, 2)), rtol=1e-12)
    assert located[0][:, :, 0, :].sum() > 0  # surface reflections
    assert located.shape[3] == nz  # the surface and the nz - 1 physical layers


def _splitting_map(scene):
    """Roulette scale 4 outside the box cloud's columns and 0.25 inside them: photons
    gather weight outside and split when they scatter in the cloud."""

    nmat, nx, ny, nz, angles = scene.shape
    scale = np.full((nx, ny, nz), 4.0)
    scale[3:8, 2:6, :] = 0.25
    return scale


def test_splitting_keeps_the_analog_expectation(oracle):
    scene = _small_box()
    scale = _splitting_map(scene)
    plain, _ = oracle.run(scene.tables, _controls(scene, 32, 21), 8)
    split, counters = oracle.run(scene.tables, _controls(scene, 32, 22), 8, guide=(0.0, 0.5, 0.0, 2.0), scale=scale)
    z = _z(_stokes_rounds(oracle, scene, split), _stokes_rounds(oracle, scene, plain))
    assert np.mean(np.abs(z) < 3) >= 0.98, np.sort(np.abs(z))[-8:]
    assert abs(z.mean()) < 0.3
    gi = _stokes_rounds(oracle, scene, split)[:, 0].sum(axis=(1, 2, 3))
    pi = _stokes_rounds(oracle, scene, plain)[:, 0].sum(axis=(1, 2, 3))
    assert abs((gi.mean() - pi.mean()) / np.hypot(gi.std(ddof=1), pi.std(ddof=1)) * np.sqrt(32)) < 4


def test_splitting_spends_more_events_where_the_map_is_important(oracle):
    scene = _small_box(ppc=20, rounds=4)
    scale = _splitting_map(scene)
    controls = _controls(scene, 4, 5)
    _, without = oracle.run(scene.tables, controls, 8, guide=(0.0, 0.5, 0.0, 0.0), scale=scale)
    _, with_split = oracle.run(scene.tables, controls, 8, guide=(0.0, 0.5, 0.0, 2.0), scale=scale)
    assert with_split["photons"] == without["photons"]
    assert with_split["scatters"] > 1.2 * without["scatters"]


def test_splitting_is_deterministic_and_off_below_the_window(oracle):
    scene = _small_box(ppc=10, rounds=2)
    nmat, nx, ny, nz, angles = scene.shape
    controls = _controls(scene, 2, 9)
    scale = _splitting_map(scene)
    first, c0 = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.5, 0.0, 2.0), scale=scale)
    again, c1 = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.5, 0.0, 2.0), scale=scale)
    np.testing.assert_array_equal(first, again)
    assert c0 == c1
    # A uniform map keeps every weight at or below the roulette weight: nothing splits.
    flat, f0 = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.5, 0.0, 2.0))
    plain_roulette, f1 = oracle.run(scene.tables, controls, 1, guide=(0.0, 0.5, 0.0, 0.0))
    np.testing.assert_array_equal(flat, plain_roulette)
    assert f0 == f1


def test_splitting_rejects_paths_and_missing_roulette(oracle):
    import monki.scenes as scenes

    layered = scenes.layered_cloud(2, 1, nx=3, ny=2)
    with pytest.raises(RuntimeError, match="Splitting"):
        oracle.run(layered.tables, _controls(layered, 1, 1), 1, guide=(0.0, 0.5, 0.0, 2.0))
    box = _small_box(ppc=2, rounds=1)
    with pytest.raises(RuntimeError, match="Splitting"):
        oracle.run(box.tables, _controls(box, 1, 1), 1, guide=(0.0, 0.0, 0.0, 2.0))
