"""Backward transport and the full Stokes vector (nmat 4) on the GPU against the oracle.

* FP64 transport against the FP64 oracle on the same Philox streams (every tally within
  rtol 1e-6, equal scatter counts): backward transport for nmat 1, 3 and 4, with and
  without layer paths and with the scattering-order tallies; forward transport with nmat 4
  and a particle whose F34 does not vanish;
* FP32 transport against the oracle with independent seeds, by the reference's
  statistical criterion (|z| < 3 in at least 99 % of entries, mean z within 0.1);
* simulate() reverses U of backward transport after accumulation, and the backward
  domain-mean Stokes vector of a horizontally uniform atmosphere matches the forward one
  (reciprocity) within the combined standard errors.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LEVELS = np.array([0.0, 0.5, 1.0, 1.5, 2.0, 3.0, 4.0, 6.0, 10.0, 20.0, 40.0, 60.0])


def _scene(nmat, *, backward, paths=False, box=True, ppc=8, rounds=2, nx=8, ny=6, polarizing=False,
           solar_zenith=40.0, solar_azimuth=0.0, views=((0.0, 0.0), (30.0, 90.0), (60.0, 180.0))):
    import monki.scenes as scenes
    from test_backward import polarizing_particle

    layers = len(LEVELS) - 1
    aerosol = np.broadcast_to(0.2 * scenes.layer_fraction(LEVELS, 0.0, 2.0) * np.diff(LEVELS) / 2.0, (nx, ny, layers))
    cloud = np.zeros((nx, ny, layers))
    profile = 8.0 * scenes.layer_fraction(LEVELS, 1.0, 2.0) * np.diff(LEVELS)
    if box:
        cloud[2:5, 1:4] = profile
    else:
        cloud[:] = profile
    particles = [scenes.AEROSOL, polarizing_particle() if polarizing else scenes.CLOUD]
    tables = scenes.build_tables(
        nx=nx, ny=ny, levels_km=LEVELS, nmat=nmat, solar_zenith=solar_zenith, solar_azimuth=solar_azimuth,
        view_zeniths=[v[0] for v in views], view_azimuths=[v[1] for v in views], albedo=0.1, save_path=paths,
        gas_scattering=scenes.rayleigh_layers(LEVELS), gas_absorption=scenes.ozone_layers(LEVELS),
        particles=particles, particle_optical_depth=np.stack([aerosol, cloud]), backward=backward,
    )
    metadata = scenes.scene_metadata(
        "backward" if backward else "forward", LEVELS, nx=nx, ny=ny, nmat=nmat, solar_zenith=solar_zenith,
        solar_azimuth=solar_azimuth, view_zeniths=[v[0] for v in views], view_azimuths=[v[1] for v in views],
        albedo=0.1, gas_scattering=scenes.rayleigh_layers(LEVELS), gas_absorption=scenes.ozone_layers(LEVELS),
        particle_optical_depth=np.stack([aerosol, cloud]), save_path=paths,
    )
    return scenes.TransportScene("backward" if backward else "forward", tables, metadata, ppc, rounds, backward)


def _native_run(native, scene, rounds, seed, config):
    import ctypes

    from monki.execution.native import F64P, U64P

    tables = np.ascontiguousarray(scene.tables)
    nmat, nx, ny, nz, angles = scene.shape
    per_round = scene.photons_per_column * nx * ny
    err = ctypes.create_string_buffer(2048)
    handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, rounds, config.encode(), err, len(err))
    assert handle, err.value
    try:
        count = int(native.monki_cuda_tally_count(handle))
        out = np.zeros(count * rounds)
        controls = (ctypes.c_uint32 * 8)(per_round * rounds, 0, 1, seed, 100000, 0, per_round, rounds)
        assert native.monki_cuda_run(handle, controls, out.ctypes.data_as(F64P), err, len(err)) == 0, err.value
        counters = np.zeros(6, dtype=np.uint64)
        native.monki_cuda_counters(handle, counters.ctypes.data_as(U64P))
        return out.reshape(rounds, count), int(counters[0])
    finally:
        native.monki_cuda_close(handle)


CASES = [
    # nmat, backward, paths, orders, polarizing particle
    (1, True, False, False, False),
    (3, True, False, False, False),
    (3, True, True, False, False),
    (3, True, False, True, False),
    (4, True, True, True, True),
    (4, False, False, False, True),
    (4, False, True, True, True),
]


@pytest.mark.parametrize("nmat,backward,paths,orders,polarizing", CASES)
def test_fp64_transport_reproduces_oracle(native, oracle, device, nmat, backward, paths, orders, polarizing):
    scene = _scene(nmat, backward=backward, paths=paths, polarizing=polarizing)
    nmat_, nx, ny, nz, angles = scene.shape
    per_round = scene.photons_per_column * nx * ny
    actual, scatters = _native_run(native, scene, 2, 23274, "precision=fp64" + (",orders=1" if orders else ""))
    expected, counters = oracle.run(scene.tables, [per_round * 2, 0, 1, 23274, 100000, 0, per_round, 2], 8, orders=orders)
    assert scatters == counters["scatters"]
    assert actual.shape == expected.shape
    close = np.isclose(actual, expected, rtol=1e-6, atol=1e-12)
    assert close.mean() == 1.0, f"{(~close).sum()} of {close.size} tallies differ"
    if nmat == 4:
        stokes = actual[:, : nmat * nx * ny * angles].reshape(2, angles, ny, nx, 4)
        assert np.abs(stokes[..., 3]).max() > 0.0


@pytest.mark.parametrize("nmat", [3, 4])
def test_fp32_backward_transport_agrees_with_oracle_statistically(native, oracle, device, nmat):
    # Enough independent pixels that the mean z of the (correlated) tallies is meaningful.
    scene = _scene(nmat, backward=True, paths=True, ppc=20, nx=16, ny=12, polarizing=nmat == 4)
    nmat_, nx, ny, nz, angles = scene.shape
    rounds = 16
    per_round = scene.photons_per_column * nx * ny
    actual, _ = _native_run(native, scene, rounds, 5, "precision=fp32")
    expected, _ = oracle.run(scene.tables, [per_round * rounds, 0, 1, 77, 100000, 0, per_round, rounds], 8)
    a, b = actual, expected
    se = np.hypot(a.std(0, ddof=1), b.std(0, ddof=1)) / np.sqrt(rounds)
    mask = se > 0
    z = (a.mean(0) - b.mean(0))[mask] / se[mask]
    assert np.mean(np.abs(z) < 3) >= 0.99
    assert abs(z.mean()) < 0.1


def test_simulate_backward_is_reciprocal_to_forward(tmp_path, device):
    from monki import simulate
    from monki.execution import CUDA

    sza, saa, vza, vaa = 40.0, 0.0, 25.0, 70.0
    # 40 rounds: the product reports standard errors from round 31 on (999 before).
    forward = _scene(3, backward=False, box=False, ppc=2000, rounds=40, nx=4, ny=4,
                     solar_zenith=sza, solar_azimuth=saa, views=((vza, vaa),))
    backward = _scene(3, backward=True, box=False, ppc=2000, rounds=40, nx=4, ny=4,
                      solar_zenith=vza, solar_azimuth=(vaa + 180.0) % 360.0, views=((sza, (saa + 180.0) % 360.0),))
    fw = simulate(forward, CUDA(seed=1), tmp_path / "forward.nc").values
    bw = simulate(backward, CUDA(seed=2), tmp_path / "backward.nc").values
    # radiance (views, ny, nx, nmat, wavelengths): domain means and their standard errors.
    mf, mb = fw["radiance"].mean(axis=(1, 2)), bw["radiance"].mean(axis=(1, 2))
    pixels = fw["radiance"].shape[1] * fw["radiance"].shape[2]
    sf = np.sqrt((fw["std_radiance"] ** 2).mean(axis=(1, 2)) / pixels)
    sb = np.sqrt((bw["std_radiance"] ** 2).mean(axis=(1, 2)) / pixels)
    assert np.all(sf < 0.01 * mf[:, :1]) and np.all(sb < 0.01 * mb[:, :1])
    z = (mf - mb) / np.hypot(sf, sb)
    assert np.all(np.abs(z) < 4.0), (mf, mb, z)
    assert abs(mf[0, 2, 0]) > 5.0 * np.hypot(sf, sb)[0, 2, 0]  # U is measured: a sign error would show


def test_simulate_writes_the_full_stokes_vector(tmp_path, device):
    from monki import SimulationResult, simulate
    from monki.execution import CUDA

    scene = _scene(4, backward=False, paths=True, ppc=200, rounds=4, polarizing=True)
    result = simulate(scene, CUDA(), tmp_path / "iquv.nc")
    radiance = result.values["radiance"]
    assert radiance.shape[3] == 4
    assert np.abs(radiance[..., 3, :]).max() > 0.0
    assert np.all(np.sqrt((radiance[..., 1:, :] ** 2).sum(axis=3)) <= radiance[..., 0, :] * 1.001)
    loaded = SimulationResult.load(tmp_path / "iquv.nc")
    np.testing.assert_allclose(loaded.values["radiance"], radiance)
