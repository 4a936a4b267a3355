"""Scene preparation from the reference's INPUT fixtures (monki.preparation).

Where the reference's fixtures are mounted, the preparer reads them directly; the
prepared 2boxclouds tables are also kept in tests/golden/ (made by make_golden.py), so the
checks that need only the tables run everywhere.
"""

from __future__ import annotations

import os
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
HOME = Path(os.environ.get("MONKI_REFERENCE", "/root/reference")) / "fortran" / "monki" / "upstream"
needs_fixtures = pytest.mark.skipif(not (HOME / "INPUT").is_dir(), reason="reference fixtures not mounted")


@needs_fixtures
def test_fixture_input_is_parsed_like_rdinput():
    from monki.preparation import parse_input

    fx = parse_input(HOME / "INPUT" / "testrun" / "MONKI_MLS_2boxclouds_340_340_test.in")
    # nz = 33 in the file; rdsize adds the vacuum layer and rdinput reads all 34 level rows.
    assert (fx.nx, fx.ny, fx.levels, fx.nmat) == (30, 20, 34, 3)
    assert fx.x_dim / fx.nx == 4.0 and fx.y_dim / fx.ny == 4.0
    assert fx.wavelength_nm == 340.0 and fx.cloud_input == "baer"
    # Level 13 (11 km) carries two clouds: optical depth 10 over columns 4-11 x 8-12 and
    # 20 over 14-17 x 9-11 (1-based, inclusive), species 1.
    assert fx.clouds.sum() == pytest.approx(10 * 8 * 5 + 20 * 4 * 3)
    assert fx.clouds[0, 3, 7, 12] == 10 and fx.clouds[0, 13, 8, 12] == 20 and fx.clouds[0, 2, 7, 12] == 0
    assert fx.altitude_km[-1] == 100.0 and fx.altitude_km.size == 34


@needs_fixtures
def test_molecular_optics_are_physical():
    from monki.preparation import molecular_optics, parse_input

    fx = parse_input(HOME / "INPUT" / "testrun" / "MONKI_MLS_cloudfree_340_340_test.in")
    depol, bmsca, bmabs = molecular_optics(fx, HOME / "DATA" / "abs_data" / "O3T_BP.dat")
    # Rayleigh optical depth of a 1013 hPa atmosphere at 340 nm (about 0.71) and the air
    # depolarization factor there (about 0.031, King factor of Bodhaine et al. 1999).
    assert 0.69 < bmsca.sum() < 0.73
    assert 0.030 < depol < 0.032
    # The fixture integrates an exponential density (type 0); hydrostatic columns (type 1)
    # follow the pressure drop and give nearly the same total.
    from dataclasses import replace

    _, hydrostatic, _ = molecular_optics(replace(fx, gas_column_type=1), HOME / "DATA" / "abs_data" / "O3T_BP.dat")
    drop = -np.diff(fx.pressure_bar)
    np.testing.assert_allclose(hydrostatic / hydrostatic.sum(), drop / drop.sum(), rtol=1e-9)
    assert hydrostatic.sum() == pytest.approx(bmsca.sum(), rel=0.03)
    # Ozone absorption at 340 nm is weak (Huggins band tail) and peaks with the O3 layer.
    assert 0.002 < bmabs.sum() < 0.03
    assert np.argmax(bmabs / np.diff(fx.altitude_km)) in range(18, 30)


@needs_fixtures
def test_mie_table_is_read_and_normalized():
    from monki.preparation import mie_species

    sp = mie_species(HOME / "DATA" / "Mie_data", "Mie_nrvar_ni0/S.lu.", "Mie_nrvar_ni0/S.sc.", 340.0, 3)
    assert len(sp.cosines) == 3601 and np.all(np.diff(sp.cosines) > 0)
    assert sp.f11[-1] == pytest.approx(816.4533, rel=1e-6)  # forward peak, 0 degrees
    assert 0.5 * np.trapezoid(sp.f11, sp.cosines) == pytest.approx(1.0, rel=2e-3)
    assert sp.cdf[0] == 0 and sp.cdf[-1] == 1 and np.all(np.diff(sp.cdf) >= 0)
    assert sp.albedo == 1.0 and sp.extinction_efficiency == pytest.approx(2.1953542248964)
    assert np.any(sp.f12 != 0)  # a polarizing particle


@needs_fixtures
def test_prepared_fixture_matches_the_kept_tables(oracle):
    """A regression snapshot: the kept tables were made by this package's own preparer, so
    this test only detects changes. The independent evidence for the preparer is
    tests/test_archived.py, which finds the Fortran preparer's optical depths, altitudes and
    layer thicknesses (stored in the reference's archived outputs) equal to this package's."""

    from monki import ReferenceCase
    from monki.preparation import prepare_reference_case

    case = ReferenceCase("2boxclouds", "testrun/MONKI_MLS_2boxclouds_340_340_test.in", photons_per_column=100,
                         rounds=32, solar_zenith=45.0)
    scene = prepare_reference_case(case, HOME)
    kept = np.load(GOLDEN / "prepared_2boxclouds.npz")
    np.testing.assert_array_equal(scene.tables, kept["tables"])
    assert oracle.validate(scene.tables) is None


def test_prepared_tables_run_in_the_oracle(oracle):
    """The Mie (F12 != 0) 2boxclouds scene through the oracle: a valid round."""

    tables = np.load(GOLDEN / "prepared_2boxclouds.npz")["tables"]
    assert oracle.validate(tables) is None
    nx, ny = int(tables[1]), int(tables[2])
    per_round = 5 * nx * ny
    out, counters = oracle.run(tables, [per_round, 0, 1, 3, 100000, 0, per_round, 1], 4)
    stokes = oracle.split(tables, out[0])[0]
    assert counters["scatters"] > per_round and stokes[0].min() > 0
    assert np.abs(stokes[1]).max() > 0  # polarized radiance
