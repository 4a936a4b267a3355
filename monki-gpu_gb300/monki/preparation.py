"""Scene preparation from the reference's INPUT fixtures, without the Fortran preparer.

Restates, in NumPy, the steps the reference's Fortran worker runs before transport
(paths relative to the reference project):

* ``rdsize`` / ``rdinput`` (fortran/monki/upstream/PROGRAM/modules/
  main_routines_cartesian_mod.f90:32-487): grid, Monte Carlo, general and aerosol
  parameters, and the level table — altitude, pressure, temperature, O3 volume mixing
  ratio and, per cloud, its optical depth (or number column), species and column range,
  each assigned to the layer above its level; a synthetic top level 1e-6 m above the last
  makes the vacuum layer;
* ``molecules_earth`` (main_routines_general_mod.f90:33-321): molecular column per layer
  (hydrostatic or exponential-density integration), the air refractive index of Peck &
  Reeder, the King factor of N2, O2, Ar and CO2 (Bodhaine et al. 1999), the
  depolarization factor, the Rayleigh cross section and layer optical depth, and the O3
  absorption optical depth from temperature-dependent cross sections integrated over the
  layer;
* ``get_O3_crabs`` (modules/get_O3_crabs.f90): the O3 cross section at the wavelength from
  the three temperature coefficients of ``DATA/abs_data/O3T_BP.dat``;
* ``aerosols`` (main_routines_general_mod.f90:629-951): the Mie phase-matrix table
  (``S.lu``), reversed to ascending scattering cosine, its bound CDF by the trapezoid rule
  (F11 + |F12| with polarization, F11 without), and the single-scattering albedo, Qext and
  geometric cross section of ``S.sc``; layer optical depth from the cloud input (optical
  depth, or number column times Qext G);
* ``worker.f90:940-1029``: extinction per km and species fractions, via
  ``monki.scenes.build_tables``.

The geometry (solar and view angles, surface albedo) and the Monte Carlo sizes come from
the ``ReferenceCase``, as in the reference harness. Only what the transport supports is
accepted: TOA source, detector and output grid, one wavelength, O3 as the only absorber,
Earth.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .input import ReferenceCase
from .scenes import TransportScene, build_tables, scene_metadata

# Physical constants of the reference (PROGRAM/modules/physical_parameters_mod.f90).
AVOGADRO = 6.022137e23
LOSCHMIDT = 2.5468993e25
GAS_CONSTANT = 8.314510
GRAVITY = 9.807
# Air composition (percent) and molar masses (g/mol) of molecules_earth.
FRACTIONS = {"N2": 78.084, "O2": 20.9476, "Ar": 0.934, "CO2": 0.0375}
MOLAR_MASS = {"N2": 28.0134, "O2": 32.00, "Ar": 39.948, "CO2": 44.01}


@dataclass
class FixtureInput:
    nx: int
    ny: int
    levels: int  # number of level rows, nz + 1 (= physical layers plus the vacuum layer)
    x_dim: float
    y_dim: float
    k_source: int
    k_detector: int
    k_register: int
    photons_per_column: int
    rounds: int
    nmat: int
    wavelength_nm: float
    gas_column_type: int  # 1 hydrostatic equilibrium, 0 exponential density decay
    planet: str
    fixed_depolarization: bool
    depolarization: float
    cloud_input: str  # "baer" or "ncol"
    save_path: bool
    save_scats: bool
    species_sc: list[str]
    species_lu: list[str]
    altitude_km: np.ndarray  # (levels,)
    pressure_bar: np.ndarray
    temperature_k: np.ndarray
    o3_ppm: np.ndarray
    clouds: np.ndarray  # (species, nx, ny, levels) optical depth or number column per layer


def _value(line: str) -> str:
    return line.split(":", 1)[0].split()[0]


def parse_input(path) -> FixtureInput:
    """Read a MONKI ``.in`` fixture (the positional layout rdsize / rdinput read)."""

    lines = Path(path).read_text().splitlines()
    at = 0

    def next_value() -> str:
        nonlocal at
        while at < len(lines):
            line = lines[at]
            at += 1
            stripped = line.strip()
            if not stripped or stripped.startswith("~") or stripped.isupper() and ":" not in stripped:
                continue
            if ":" in line:
                return _value(line)
        raise ValueError(f"{path}: unexpected end of the input file")

    # rdsize reads nz and adds the vacuum layer (nz + 1, main_routines_cartesian_mod.f90:75-82);
    # rdinput then reads that many level rows (all nz + 1 of the file) and puts the vacuum
    # level 1e-6 m above the last (:392-459).
    nx, ny, levels = int(next_value()), int(next_value()), int(next_value()) + 1
    x_dim, y_dim = float(next_value()), float(next_value())
    k_source, k_detector, k_register = int(next_value()), int(next_value()), int(next_value())
    photons, rounds = int(next_value()), int(next_value())
    next_value()  # stop when converged
    next_value()  # maximum reflectance standard deviation
    nmat = int(next_value())
    wave_type = next_value()
    wave_min, wave_max = float(next_value()), float(next_value())
    next_value()  # wavelength step
    read_bmsca = next_value().lower() == ".true."
    next_value()  # bmsca file
    gas_column_type = int(next_value())
    planet = next_value()
    fixed_depol = next_value().lower() == ".true."
    depol = float(next_value())
    read_bmabs = next_value().lower() == ".true."
    next_value()  # bmabs file
    cloud_input = next_value()
    save_path = next_value().lower() == ".true."
    save_scats = next_value().lower() == ".true."
    species = int(next_value())
    species_sc, species_lu = [], []
    for _ in range(species):
        species_sc.append(next_value())
        species_lu.append(next_value())
        next_value()  # number of scattering angles
    gases = int(next_value())
    nclouds = int(next_value())

    if wave_type != "wl" or wave_min != wave_max:
        raise NotImplementedError("only one wavelength in nm is supported")
    if read_bmsca or read_bmabs:
        raise NotImplementedError("optical thickness files are not supported")
    if gases != 1:
        raise NotImplementedError("O3 must be the only absorbing gas")
    if planet.lower() != "earth":
        raise NotImplementedError("only the Earth atmosphere is supported")

    rows = []
    for line in lines[at:]:
        parts = line.split()
        if parts and parts[0].isdigit() and len(parts) >= 5 + 6 * nclouds:
            rows.append(parts)
    # Every level row is read; the layer above the last level is the vacuum layer.
    if len(rows) < levels:
        raise ValueError(f"{path}: expected {levels} level rows, found {len(rows)}")
    if len(rows) > levels:
        raise ValueError(f"{path}: more level rows than nz + 1 = {levels}")
    alt = np.array([float(r[1]) for r in rows])
    pres = np.array([float(r[2]) for r in rows])
    temp = np.array([float(r[3]) for r in rows])
    o3 = np.array([float(r[4]) for r in rows])
    clouds = np.zeros((species, nx, ny, levels))
    for k, r in enumerate(rows):
        for c in range(nclouds):
            value, iaer, x0, x1, y0, y1 = r[5 + 6 * c : 11 + 6 * c]
            value, iaer = float(value), int(iaer)
            if iaer < 0 or iaer > species:
                iaer = 0
            if value > 1e-16 and iaer > 0:
                x0, x1, y0, y1 = int(x0), int(x1), int(y0), int(y1)
                if not (1 <= x0 <= nx and 1 <= x1 <= nx and 1 <= y0 <= ny and 1 <= y1 <= ny):
                    raise ValueError(f"{path}: cloud columns outside the grid")
                clouds[iaer - 1, x0 - 1 : x1, y0 - 1 : y1, k] += value
    if np.any(pres <= 0) or np.any(temp <= 0):
        raise ValueError(f"{path}: pressure and temperature must be positive")
    return FixtureInput(nx, ny, levels, x_dim, y_dim, k_source, k_detector, k_register, photons, rounds, nmat,
                        wave_min, gas_column_type, planet, fixed_depol, depol, cloud_input, save_path, save_scats,
                        species_sc, species_lu, alt, pres, temp, o3, clouds)


def _linear(x, y, xp):
    """Linear interpolation of the bracketing nodes (interpol_sp.f linpol_dp_single)."""

    x, y = np.asarray(x, dtype=float), np.asarray(y, dtype=float)
    hi = int(np.clip(np.searchsorted(x, xp), 1, len(x) - 1))
    lo = hi - 1
    return (y[hi] - y[lo]) / (x[hi] - x[lo]) * (xp - x[lo]) + y[lo]


def o3_cross_section(path, wavelength_nm: float, temperature_k) -> np.ndarray:
    """O3 absorption cross section (cm^2) at each temperature: sum of the coefficients
    interpolated at the wavelength times (T - 273.15) ** power (get_O3_crabs)."""

    lines = Path(path).read_text().splitlines()
    comments = int(lines[0].split()[0])
    count = int(lines[1].split()[0])
    table = np.array([[float(v) for v in line.split()[:4]] for line in lines[2 + comments : 2 + comments + count]])
    coefficients = [_linear(table[:, 0], table[:, 1 + p], wavelength_nm) for p in range(3)]
    celsius = np.asarray(temperature_k, dtype=float) - 273.15
    return sum(c * celsius**p for p, c in enumerate(coefficients))


def molecular_optics(fixture: FixtureInput, o3_table) -> tuple[float, np.ndarray, np.ndarray]:
    """(depolarization factor, Rayleigh and O3 optical depth per physical layer)."""

    pres = fixture.pressure_bar * 1e5  # Pa
    temp = fixture.temperature_k
    alt = fixture.altitude_km * 1e3  # m
    layers = fixture.levels - 1
    if fixture.gas_column_type == 1:
        total = sum(FRACTIONS.values())
        molar = sum(MOLAR_MASS[g] * FRACTIONS[g] for g in FRACTIONS) / total * 1e-3 / AVOGADRO
        column = (pres[:-1] - pres[1:]) / (molar * GRAVITY)
    elif fixture.gas_column_type == 0:
        column = np.zeros(layers)
        for k in range(layers):
            p1, p2 = pres[k] / temp[k], pres[k + 1] / temp[k + 1]
            dz = alt[k + 1] - alt[k]
            pt = p1 * dz if abs(p1 - p2) < 1e-16 else (p2 - p1) * dz / (math.log(p2) - math.log(p1))
            column[k] = AVOGADRO / GAS_CONSTANT * pt
    else:
        raise ValueError("gas column type must be 0 or 1")
    micron = fixture.wavelength_nm / 1000.0
    w2 = 1.0 / (micron * micron)
    ri = 1.0 + 1e-8 * 8060.51 + 1e-8 * (2480990.0 / (132.274 - w2)) + 1e-8 * (17455.7 / (39.32957 - w2))
    rindex = (ri * ri - 1.0) ** 2 / (ri * ri + 2.0) ** 2
    sig = 1e3 / fixture.wavelength_nm
    king = {"N2": 1.034 + 3.17e-4 * sig**2, "O2": 1.096 + 1.385e-3 * sig**2 + 1.448e-4 * sig**4, "Ar": 1.0, "CO2": 1.15}
    dep = sum(FRACTIONS[g] * king[g] for g in FRACTIONS) / sum(FRACTIONS.values())
    depol = (6.0 * dep - 6.0) / (3.0 + 7.0 * dep)
    sigma_rayleigh = 24.0 * math.pi**3 * rindex * dep / (micron**4 * LOSCHMIDT**2 * 1e-24)
    bmsca = sigma_rayleigh * column
    sigma_o3 = o3_cross_section(o3_table, fixture.wavelength_nm, temp) / 100.0 / 100.0  # m^2
    bmabs = np.zeros(layers)
    for k in range(layers):
        p1, p2 = pres[k] / temp[k], pres[k + 1] / temp[k + 1]
        dz = alt[k + 1] - alt[k]
        s1 = fixture.o3_ppm[k] / 1e6 * sigma_o3[k]
        s2 = fixture.o3_ppm[k + 1] / 1e6 * sigma_o3[k + 1]
        if abs(p1 - p2) < 1e-16:
            integral = 0.5 * p1 * (s1 + s2) * dz
        else:
            lg = math.log(p2 / p1)
            integral = (p2 - p1) * dz * (s1 - s2) / lg**2 + p2 * dz * s2 / lg - p1 * dz * s1 / lg
        bmabs[k] = AVOGADRO / GAS_CONSTANT * integral
    if fixture.fixed_depolarization:
        depol = fixture.depolarization
    return depol, bmsca, bmabs


@dataclass
class MieSpecies:
    cosines: np.ndarray  # ascending
    cdf: np.ndarray
    f11: np.ndarray
    f22: np.ndarray
    f33: np.ndarray
    f12: np.ndarray
    albedo: float
    extinction_efficiency: float
    geometric_cross_section: float
    f34: np.ndarray | None = None
    f44: np.ndarray | None = None


def _suffix(wavelength_nm: float) -> str:
    if wavelength_nm % 1.0 != 0.0 or not 100.0 <= wavelength_nm < 10000.0:
        raise NotImplementedError("Mie tables exist for whole wavelengths in nm from 100 to 9999")
    text = f"{wavelength_nm / 1000.0:.3f}"
    return ("00" + text[1:]) if wavelength_nm < 1000.0 else ("0" + text)


def mie_species(mie_dir, lut_start: str, sc_start: str, wavelength_nm: float, nmat: int) -> MieSpecies:
    suffix = _suffix(wavelength_nm)
    table = np.loadtxt(Path(mie_dir) / f"{lut_start}{suffix}")
    angles = table[::-1, 0]
    cosines = np.cos(np.deg2rad(angles))
    # Columns: angle, F11, F22, F33, F44, F12, F34 (main_routines_general_mod.f90:790).
    f11, f22, f33, f44, f12, f34 = (table[::-1, c] for c in (1, 2, 3, 4, 5, 6))
    bound = f11 + np.abs(f12) if nmat > 1 else f11.copy()
    cdf = np.zeros_like(cosines)
    for i in range(1, len(cosines)):
        cdf[i] = cdf[i - 1] + (cosines[i] - cosines[i - 1]) * (bound[i] + bound[i - 1]) / 2.0
    cdf /= cdf[-1]
    lines = (Path(mie_dir) / f"{sc_start}{suffix}").read_text().splitlines()
    albedo = float(lines[7][32:57])
    q_ext = float(lines[9][32:57])
    geometric = float(lines[11][32:57])
    return MieSpecies(cosines, cdf, f11, f22, f33, f12, albedo, q_ext, geometric, f34, f44)


def prepare_reference_case(case: ReferenceCase, home) -> TransportScene:
    """The prepared scene of a reference fixture: ``home`` holds INPUT/ and DATA/."""

    home = Path(home)
    fixture = parse_input(home / "INPUT" / case.input_file)
    if (fixture.k_source, fixture.k_detector, fixture.k_register) != (1, 1, 1):
        raise NotImplementedError("only a TOA source, detector and output grid are supported")
    depol, bmsca, bmabs = molecular_optics(fixture, home / "DATA" / "abs_data" / "O3T_BP.dat")
    species = [mie_species(home / "DATA" / "Mie_data", lu, sc, fixture.wavelength_nm, fixture.nmat)
               for sc, lu in zip(fixture.species_sc, fixture.species_lu, strict=True)]
    layers = fixture.levels - 1
    clouds = fixture.clouds[:, :, :, :layers]
    if fixture.cloud_input == "ncol":
        clouds = clouds * np.array([s.extinction_efficiency * s.geometric_cross_section for s in species])[:, None, None, None]
    elif fixture.cloud_input != "baer":
        raise ValueError("cloud input must be baer or ncol")
    levels_km = fixture.altitude_km
    particles = [(s.cosines, s.cdf, s.f11, s.f22, s.f33, s.f12, s.albedo, s.f34, s.f44) for s in species]
    x_unit, y_unit = fixture.x_dim / fixture.nx, fixture.y_dim / fixture.ny
    tables = build_tables(
        nx=fixture.nx, ny=fixture.ny, levels_km=levels_km, nmat=fixture.nmat,
        solar_zenith=case.solar_zenith, solar_azimuth=case.solar_azimuth,
        view_zeniths=list(case.view_zeniths), view_azimuths=[case.view_azimuth] * len(case.view_zeniths),
        albedo=case.surface_albedo, save_path=fixture.save_path,
        gas_scattering=bmsca, gas_absorption=bmabs, particles=particles,
        particle_optical_depth=clouds, depolarization=depol, pixel_km=(x_unit, y_unit), backward=case.backward,
    )
    metadata = scene_metadata(
        case.name, levels_km, nx=fixture.nx, ny=fixture.ny, nmat=fixture.nmat,
        solar_zenith=case.solar_zenith, solar_azimuth=case.solar_azimuth,
        view_zeniths=list(case.view_zeniths), view_azimuths=[case.view_azimuth] * len(case.view_zeniths),
        albedo=case.surface_albedo, gas_scattering=bmsca, gas_absorption=bmabs, particle_optical_depth=clouds,
        save_path=fixture.save_path, pixel_km=(x_unit, y_unit), wavelength_nm=fixture.wavelength_nm,
        pressure_pa=fixture.pressure_bar * 1e5, temperature_k=fixture.temperature_k, vmr_ppm=fixture.o3_ppm,
    )
    return TransportScene(case.name, tables, metadata, case.photons_per_column, case.rounds, case.backward,
                          {"fixture": case.input_file, "depolarization": depol,
                           "rayleigh_optical_depth": float(bmsca.sum()), "o3_optical_depth": float(bmabs.sum())})


def scene_arrays(scene: TransportScene, fixture_description: dict) -> dict:
    """Arrays that rebuild a prepared fixture scene without the fixture files
    (``scene_from_arrays``): the table stream and the product metadata's inputs."""

    v = scene.metadata.values
    return {
        "tables": scene.tables,
        "levels_km": v["alt"] / 1000.0,
        "bmsca": v["bmsca"][:, 0],
        "bmabs": v["bmabs"][:, 0],
        "baer": v["baer"][..., 0].transpose(3, 2, 1, 0),
        "geometry": np.array([v["theta0"][0], v["phi0"][0], v["asurf"][0], v["x_unit"][0], v["y_unit"][0], v["wav"][0]]),
        "view_zeniths": v["theta"],
        "view_azimuths": np.broadcast_to(v["phi"], v["theta"].shape).copy(),
        "sizes": np.array([scene.photons_per_column, scene.rounds]),
        "name": np.array(scene.name),
        **({"pres": v["pres"], "temp": v["temp"], "vmrgas": v["vmrgas"]} if "pres" in v else {}),
    }


def scene_from_arrays(arrays) -> TransportScene:
    """The TransportScene of ``scene_arrays``."""

    tables = np.asarray(arrays["tables"])
    nx, ny, nz, nmat = (int(v) for v in tables[1:5])
    sza, saa, albedo, x_unit, y_unit, wavelength = (float(v) for v in arrays["geometry"])
    metadata = scene_metadata(
        str(arrays["name"]), np.asarray(arrays["levels_km"]), nx=nx, ny=ny, nmat=nmat, solar_zenith=sza,
        solar_azimuth=saa, view_zeniths=list(arrays["view_zeniths"]), view_azimuths=list(arrays["view_azimuths"]),
        albedo=albedo, gas_scattering=np.asarray(arrays["bmsca"]), gas_absorption=np.asarray(arrays["bmabs"]),
        particle_optical_depth=np.asarray(arrays["baer"]), save_path=bool(tables[10]), pixel_km=(x_unit, y_unit),
        wavelength_nm=wavelength,
        **({"pressure_pa": arrays["pres"], "temperature_k": arrays["temp"], "vmr_ppm": arrays["vmrgas"]}
           if "pres" in arrays else {}),
    )
    ppc, rounds = (int(v) for v in arrays["sizes"])
    return TransportScene(str(arrays["name"]), tables, metadata, ppc, rounds, False, {})
