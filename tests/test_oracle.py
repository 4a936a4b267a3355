"""The CPU oracle against the golden vectors, and its physical invariants (no GPU)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_philox_matches_published_known_answer(oracle):
    kat = json.loads((GOLDEN / "philox_kat.json").read_text())
    np.testing.assert_array_equal(oracle.philox(kat["counter"], kat["key"]), kat["expected"])


def test_uniform_grid_is_open_and_float32_exact(oracle):
    values = oracle.uniforms(7, 3, 11, 4000)
    assert np.all(values > 0) and np.all(values < 1)
    # (w >> 9 + 0.5) * 2^-23: every draw is an odd multiple of 2^-24.
    scaled = values * 2.0**24
    np.testing.assert_array_equal(scaled, np.round(scaled))
    assert np.all(np.round(scaled).astype(np.int64) % 2 == 1)
    np.testing.assert_array_equal(values.astype(np.float32).astype(np.float64), values)


def test_streams_depend_only_on_photon_round_and_seed(oracle):
    a = oracle.uniforms(5, 2, 9, 12)
    np.testing.assert_array_equal(a, oracle.uniforms(5, 2, 9, 12))
    for other in (oracle.uniforms(6, 2, 9, 12), oracle.uniforms(5, 3, 9, 12), oracle.uniforms(5, 2, 10, 12)):
        assert not np.array_equal(a, other)


def test_polarization_probe_matches_golden(oracle):
    probe = json.loads((GOLDEN / "polarization_probe.json").read_text())
    for i in range(3):
        actual = oracle.scatter_stokes(
            probe["depol"], probe["incoming"][i], probe["outgoing"][i], probe["phi_in"][i], probe["phi_out"][i], probe["stokes"]
        )
        np.testing.assert_allclose(actual, probe["expected"][i], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize(
    "field,value",
    # version 4; nmat 2; nmat 4 with particles but no F34 / F44 tables (a v1 stream);
    # version 3 without its F34 / F44 tables (truncated); source and detector off the top
    [(0, 4), (4, 2), (4, 4), (0, 3), (7, 1), (8, 0)],
)
def test_unsupported_tables_are_rejected(oracle, field, value):
    import monki.scenes as scenes

    tables = scenes.clear_sky(2, 1, nx=3, ny=2).tables.copy()
    tables[field] = value
    assert oracle.validate(tables) is not None


def test_truncated_and_nonfinite_tables_are_rejected(oracle):
    import monki.scenes as scenes

    tables = scenes.clear_sky(2, 1, nx=3, ny=2).tables
    assert oracle.validate(tables) is None
    assert "Truncated" in oracle.validate(tables[:-5])
    bad = tables.copy()
    bad[40] = np.nan
    assert oracle.validate(bad) is not None


def _run(oracle, scene, rounds=1, seed=0, threads=4):
    nmat, nx, ny, nz, angles = scene.shape
    per_round = scene.photons_per_column * nx * ny
    out, counters = oracle.run(scene.tables, [per_round * rounds, 0, 1, seed, 100000, 0, per_round, rounds], threads)
    return out, counters


def test_thread_count_does_not_change_histories(oracle):
    import monki.scenes as scenes

    scene = scenes.layered_cloud(4, 1, nx=6, ny=4)
    a, ca = _run(oracle, scene, threads=1)
    b, cb = _run(oracle, scene, threads=7)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-15)
    assert ca == cb


def test_rounds_in_one_group_equal_rounds_run_alone(oracle):
    import monki.scenes as scenes

    scene = scenes.clear_sky(3, 3, nx=5, ny=4)
    nmat, nx, ny, nz, angles = scene.shape
    per_round = 3 * nx * ny
    grouped, _ = oracle.run(scene.tables, [per_round * 3, 0, 1, 5, 100000, 0, per_round, 3], 4)

    for r in range(3):
        alone, _ = oracle.run(scene.tables, [per_round, 0, 1 + r, 5, 100000, 0, per_round, 1], 4)
        np.testing.assert_allclose(grouped[r], alone[0], rtol=1e-12, atol=1e-15)


def test_step_limit_rejects_the_round(oracle):
    import monki.scenes as scenes

    scene = scenes.clear_sky(2, 1, nx=3, ny=2)
    per_round = 2 * 6
    with pytest.raises(RuntimeError, match="flag 16"):
        oracle.run(scene.tables, [per_round, 0, 1, 0, 1, 0, per_round, 1], 2)


def test_top_layer_amf_is_geometric(oracle):
    """Above a thin atmosphere the layer AMF tends to 1/mu0 + 1/mu (no scattering there)."""

    import monki.scenes as scenes

    scene = scenes.layered_cloud(20, 1, nx=4, ny=3)
    out, _ = _run(oracle, scene, threads=8)
    stokes, paths, weights = oracle.split(scene.tables, out[0])
    thickness = np.diff(scene.metadata.values["alt"]) / 1000.0
    amf = paths[:, :, :-1, :].sum(axis=(0, 1)) / weights.sum(axis=(0, 1))[None, :] / thickness[:, None]
    mu0 = np.cos(np.deg2rad(30.0))
    for ia, vza in enumerate((0.0, 30.0, 60.0)):
        expected = 1 / mu0 + 1 / np.cos(np.deg2rad(vza))
        np.testing.assert_allclose(amf[-1, ia], expected, rtol=2e-3)


def test_single_scattering_limit(oracle):
    """A thin non-absorbing Rayleigh layer over a black surface reproduces the analytic
    single-scattering radiance I = F11(Theta)/4 / mu * (1 - exp(-tau m)) / m, m = 1/mu0 + 1/mu.
    """

    import monki.scenes as scenes

    levels = scenes.layer_levels_km()
    layers = len(levels) - 1
    tau = np.zeros(layers)
    tau[10] = 3e-3  # one thin scattering layer at 5-5.5 km
    tables = scenes.build_tables(
        nx=1,
        ny=1,
        levels_km=levels,
        nmat=1,
        solar_zenith=30.0,
        solar_azimuth=0.0,
        view_zeniths=[0.0, 40.0],
        view_azimuths=[0.0, 120.0],
        albedo=0.0,
        save_path=False,
        gas_scattering=tau,
        gas_absorption=np.zeros(layers),
        particles=[],
        particle_optical_depth=np.zeros((0, 1, 1, layers)),
        depolarization=0.0,
        pixel_km=1000.0,
    )
    photons = 4_000_000
    out, counters = oracle.run(tables, [photons, 0, 1, 3, 100000, 0, photons, 1], 8)
    intensity = out[0, :2] / photons
    mu0 = np.cos(np.deg2rad(30.0))
    # About 1/sqrt(scatters) relative noise; allow four standard errors.
    tolerance = 4 / np.sqrt(counters["scatters"])

    for ia, (vza, raa) in enumerate(((0.0, 0.0), (40.0, 120.0))):
        mu = np.cos(np.deg2rad(vza))
        c = -mu0  # propagation direction of the sunlight is downward
        cos_sca = c * mu + np.sqrt(1 - c * c) * np.sqrt(1 - mu * mu) * np.cos(np.deg2rad(0.0 - raa))
        f11 = 0.75 * (1 + cos_sca**2) / 4
        m = 1 / mu0 + 1 / mu
        expected = f11 / mu * (1 - np.exp(-tau.sum() * m)) / m
        np.testing.assert_allclose(intensity[ia], expected, rtol=tolerance)
