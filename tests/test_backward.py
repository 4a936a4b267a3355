"""Backward transport and the full Stokes vector in the oracle (CPU).

* nmat 4 with particles whose F34 vanishes (Rayleigh, Henyey-Greenstein): I, Q and U are
  the nmat 3 tallies exactly (V never couples back) and V stays zero;
* nmat 4 with a particle whose F34 does not vanish: V appears, and every pixel keeps
  Q^2 + U^2 + V^2 <= I^2 (to the tally tolerance);
* reciprocity: on a horizontally uniform atmosphere, backward transport along the reversed
  view with the views pointing back to the sun reproduces the forward domain-mean Stokes
  vector (with U reversed, as the reference's driver does after accumulation) within the
  combined standard errors, for nmat 1, 3 and 4.
"""

from __future__ import annotations

import numpy as np
import pytest

LEVELS = np.array([0.0, 0.5, 1.0, 1.5, 2.0, 3.0, 4.0, 6.0, 10.0, 20.0, 40.0, 60.0])


def _tables(nmat, *, solar_zenith, solar_azimuth, views, backward=False, particles=None, nx=2, ny=2, cloud=4.0):
    import monki.scenes as scenes

    layers = len(LEVELS) - 1
    tau_r = scenes.rayleigh_layers(LEVELS)
    tau_o3 = scenes.ozone_layers(LEVELS)
    aerosol = np.broadcast_to(0.2 * scenes.layer_fraction(LEVELS, 0.0, 2.0) * np.diff(LEVELS) / 2.0, (nx, ny, layers))
    cloud_tau = np.broadcast_to(cloud * scenes.layer_fraction(LEVELS, 1.0, 2.0) * np.diff(LEVELS), (nx, ny, layers))
    particles = particles or [scenes.AEROSOL, scenes.CLOUD]
    return scenes.build_tables(
        nx=nx, ny=ny, levels_km=LEVELS, nmat=nmat, solar_zenith=solar_zenith, solar_azimuth=solar_azimuth,
        view_zeniths=[v[0] for v in views], view_azimuths=[v[1] for v in views], albedo=0.1, save_path=False,
        gas_scattering=tau_r, gas_absorption=tau_o3, particles=particles,
        particle_optical_depth=np.stack([aerosol, cloud_tau]), backward=backward,
    )


def polarizing_particle(count=721, asymmetry=0.7, albedo=0.99):
    """A tabulated particle with F22 = F11, F44 = F33 and F12^2 + F33^2 + F34^2 = F11^2 (the
    structure of a single sphere's scattering matrix), with F34 != 0."""

    import monki.scenes as scenes

    cosines, cdf, f11, _, _, _ = scenes.henyey_greenstein_table(asymmetry, count)
    mu = cosines
    p = 0.5 * (1.0 - mu * mu) / (1.0 + mu * mu)
    delta = 0.6 * (1.0 - mu)
    f12 = -p * f11
    rest = np.sqrt(1.0 - p * p) * f11
    f33, f34 = rest * np.cos(delta), rest * np.sin(delta)
    bound = f11 + np.abs(f12)
    cdf = np.zeros_like(mu)
    for i in range(1, len(mu)):
        cdf[i] = cdf[i - 1] + (mu[i] - mu[i - 1]) * (bound[i] + bound[i - 1]) / 2.0
    cdf /= cdf[-1]
    return (cosines, cdf, f11, f11.copy(), f33, f12, albedo, f34, f33.copy())


def _controls(tables, ppc, rounds, seed):
    nx, ny = int(tables[1]), int(tables[2])
    per_round = ppc * nx * ny
    return [per_round * rounds, 0, 1, seed, 100000, 0, per_round, rounds]


def test_nmat4_without_f34_reproduces_nmat3_and_keeps_v_zero(oracle):
    kw = dict(solar_zenith=40.0, solar_azimuth=0.0, views=[(0.0, 0.0), (30.0, 90.0), (60.0, 180.0)])
    t3, t4 = _tables(3, **kw), _tables(4, **kw)
    assert int(t4[0]) == 3 and int(t4[4]) == 4
    out3, c3 = oracle.run(t3, _controls(t3, 50, 2, 5), 1)
    out4, c4 = oracle.run(t4, _controls(t4, 50, 2, 5), 1)
    assert {k: v for k, v in c3.items() if k != "tally_updates"} == {k: v for k, v in c4.items() if k != "tally_updates"}
    s3 = out3.reshape(2, -1, 3)
    s4 = out4.reshape(2, -1, 4)
    np.testing.assert_array_equal(s4[..., :3], s3)
    assert np.all(s4[..., 3] == 0.0)


def test_nmat4_with_circular_coupling_produces_bounded_v(oracle):
    import monki.scenes as scenes

    kw = dict(solar_zenith=40.0, solar_azimuth=0.0, views=[(0.0, 0.0), (30.0, 90.0), (60.0, 180.0)])
    t4 = _tables(4, particles=[scenes.AEROSOL, polarizing_particle()], **kw)
    out, _ = oracle.run(t4, _controls(t4, 400, 1, 3), 8)
    s = out.reshape(-1, 4)
    assert np.abs(s[:, 3]).max() > 1e-4 * s[:, 0].max()
    assert np.all(np.sqrt((s[:, 1:] ** 2).sum(axis=1)) <= s[:, 0] * 1.0001 + 1e-12)


def _domain_means(oracle, tables, ppc, rounds, seed):
    nmat, nx, ny, angles = int(tables[4]), int(tables[1]), int(tables[2]), int(tables[5])
    out, _ = oracle.run(tables, _controls(tables, ppc, rounds, seed), 8)
    per_round = out.reshape(rounds, angles, ny, nx, nmat).mean(axis=(2, 3)) / ppc  # rounds, angles, nmat
    return per_round.mean(axis=0), per_round.std(axis=0, ddof=1) / np.sqrt(rounds)


@pytest.mark.parametrize("nmat", [1, 3, 4])
def test_backward_transport_is_reciprocal_to_forward(oracle, nmat):
    import monki.scenes as scenes

    sza, saa, vza, vaa = 40.0, 0.0, 25.0, 70.0
    particles = [scenes.AEROSOL, polarizing_particle()] if nmat == 4 else None
    forward = _tables(nmat, solar_zenith=sza, solar_azimuth=saa, views=[(vza, vaa)], particles=particles)
    backward = _tables(nmat, solar_zenith=vza, solar_azimuth=(vaa + 180.0) % 360.0, views=[(sza, (saa + 180.0) % 360.0)],
                       backward=True, particles=particles)
    mf, sf = _domain_means(oracle, forward, 500, 24, 11)
    mb, sb = _domain_means(oracle, backward, 500, 24, 12)
    if nmat >= 3:
        mb[..., 2] *= -1.0  # the backward convention reverses U after accumulation
    z = (mf - mb) / np.hypot(sf, sb)
    assert np.all(np.abs(z) < 4.0), (mf, mb, z)
    # The comparison has power: the radiance is measured to better than 1 %.
    assert sf[0, 0] < 0.01 * mf[0, 0]
