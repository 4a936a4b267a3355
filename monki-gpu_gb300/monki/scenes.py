"""Synthetic prepared scenes for the benchmark configurations, in the transport table format.

The reference prepares optical tables in Fortran (kernels/cpu/worker.f90:940-1120) from a
fixture and exports ``transport.bin`` v1 (float64, Fortran order, layout at
worker.f90:1102-1120). This module builds the same stream directly from the synthetic
atmospheres of the workloads, as version 2: v1 plus one view azimuth per view, because
the workloads pair each view zenith with its own relative azimuth. Scenes with the full
Stokes vector (nmat 4) are written as version 3: version 2 plus the F34 and F44 tables of
each particle species, which the reference reads from its Mie files
(fortran/.../main_routines_general_mod.f90:790-817) but leaves out of its v1 export.

Stream layout (all float64):
  header   version, nx, ny, nz, nmat, angles, species, k_source, k_detector, k_register,
           save_path, backward
  geometry xunit, yunit, depol, solar propagation zenith (deg), solar azimuth (deg),
           view azimuth of the first view (deg)
  zunit(nz), view zeniths(angles), [v2] view azimuths(angles),
  surface type(nx,ny) = -1, albedo(nx,ny), elevation index(nx,ny) = 1,
  beta(nx,ny,nz), species fractions(species+1,nx,ny,nz), gas single-scattering albedo(nz)
  per particle species: LUT size, albedo, cosines, bound CDF, F11, F22, F33, F12, [v3] F34, F44

A backward scene (header backward = 1) injects photons along the sensor's line of sight:
its "solar" angles are those of the reversed view and its views point back to the sun
(fortran/.../worker.f90:650-702); the transport registers every contribution at the
injection column.

The layer ``nz`` is the vacuum layer above the top of the atmosphere; like the reference
input parser (fortran/.../main_routines_cartesian_mod.f90:455-460) it is one micrometre
thick and has zero extinction.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from math import erf, sqrt

import numpy as np

from .output import SimulationResult

VACUUM_KM = 1.0e-9
LUT_ANGLES = 3601  # 0.05 degree steps, as the reference Mie table


@dataclass(frozen=True)
class Particle:
    """A tabulated scattering species: Henyey-Greenstein F11, non-polarizing (F22 = F33 = F11)."""

    name: str
    asymmetry: float
    albedo: float


@dataclass
class TransportScene:
    """A prepared scene: the float64 table stream plus output metadata and run settings.

    ``simulate`` and every backend accept it wherever the reference accepts a
    ``ReferenceCase``: it carries ``photons_per_column``, ``rounds`` and ``backward``.
    """

    name: str
    tables: np.ndarray
    metadata: SimulationResult
    photons_per_column: int
    rounds: int
    backward: bool = False
    description: dict = field(default_factory=dict)

    @property
    def shape(self) -> tuple[int, int, int, int, int]:
        """(nmat, nx, ny, nz, angles) of the prepared tables."""

        nx, ny, nz, nmat, angles = (int(v) for v in self.tables[1:6])
        return nmat, nx, ny, nz, angles

    @property
    def save_path(self) -> bool:
        return bool(self.tables[10])


def layer_levels_km() -> np.ndarray:
    """The fixed 34-layer grid: 0-10 km by 0.5, 10-30 km by 2, 30-60 km by 7.5."""

    return np.concatenate(
        [np.arange(0.0, 10.0, 0.5), np.arange(10.0, 30.0, 2.0), np.arange(30.0, 60.01, 7.5)]
    )


def scaled_levels_km(layers: int) -> np.ndarray:
    """A grid of ``layers`` physical layers over 0-60 km with the same three-band shape.

    The lowest 3 km always resolve at 0.5 km so cloud placement stays layer-aligned.
    """

    if layers == 34:
        return layer_levels_km()

    if layers < 12:
        raise ValueError("at least 12 layers are required")

    low = np.arange(0.0, 3.0, 0.5)
    rest = layers - len(low)
    middle = max(1, int(round(rest * 0.6)))
    upper = rest - middle
    mid_levels = np.linspace(3.0, 20.0, middle + 1)[:-1]
    up_levels = np.linspace(20.0, 60.0, upper + 1)
    return np.concatenate([low, mid_levels, up_levels])


def henyey_greenstein_table(asymmetry: float, count: int = LUT_ANGLES):
    """F11 of Henyey-Greenstein on the reference angle grid, normalized to (1/2)int F11 dmu = 1.

    Returns ascending cosines (from 180 to 0 degrees) and F11, F22, F33, F12, with the
    bound-function CDF built by the trapezoid rule of
    fortran/.../main_routines_general_mod.f90:825-866.
    """

    if not -1 < asymmetry < 1:
        raise ValueError("asymmetry must be in (-1, 1)")

    angles = np.linspace(180.0, 0.0, count)
    cosines = np.cos(np.deg2rad(angles))
    g = asymmetry
    f11 = (1.0 - g * g) / (1.0 + g * g - 2.0 * g * cosines) ** 1.5
    f12 = np.zeros_like(f11)
    bound = f11 + np.abs(f12)
    cdf = np.zeros(count)

    for index in range(1, count):
        cdf[index] = cdf[index - 1] + (cosines[index] - cosines[index - 1]) * (
            bound[index] + bound[index - 1]
        ) / 2.0

    cdf /= cdf[-1]
    return cosines, cdf, f11, f11.copy(), f11.copy(), f12


def rayleigh_layers(levels: np.ndarray, total: float = 0.70, scale_km: float = 8.0) -> np.ndarray:
    top = levels[-1]
    norm = 1.0 - np.exp(-top / scale_km)
    return total * (np.exp(-levels[:-1] / scale_km) - np.exp(-levels[1:] / scale_km)) / norm


def ozone_layers(levels: np.ndarray, total: float = 0.30, peak_km: float = 22.0, width_km: float = 5.0):
    def cdf(z):
        return 0.5 * (1.0 + erf((z - peak_km) / (width_km * sqrt(2.0))))

    weights = np.array([cdf(b) - cdf(a) for a, b in zip(levels[:-1], levels[1:], strict=True)])
    return total * weights / (cdf(levels[-1]) - cdf(levels[0]))


def layer_fraction(levels: np.ndarray, bottom: float, top: float) -> np.ndarray:
    """Fraction of each layer's thickness that lies inside [bottom, top]."""

    lower = np.clip(levels[:-1], bottom, top)
    upper = np.clip(levels[1:], bottom, top)
    return (upper - lower) / (levels[1:] - levels[:-1])


def build_tables(
    *,
    nx: int,
    ny: int,
    levels_km: np.ndarray,
    nmat: int,
    solar_zenith: float,
    solar_azimuth: float,
    view_zeniths,
    view_azimuths,
    albedo,
    save_path: bool,
    gas_scattering: np.ndarray,
    gas_absorption: np.ndarray,
    particles: list[Particle],
    particle_optical_depth: np.ndarray,
    depolarization: float = 0.0279,
    pixel_km=1.0,
    backward: bool = False,
) -> np.ndarray:
    """Assemble a version-2 table stream (version 3 with F34 and F44 when nmat is 4).

    ``particle_optical_depth`` has shape (species, nx, ny, layers) in layer optical depth;
    gas optical depths have shape (layers,). Extinctions are per km, the species
    fractions are normalized by the total as worker.f90:985-1000 does.
    """

    levels = np.asarray(levels_km, dtype=float)
    layers = len(levels) - 1
    nz = layers + 1
    zunit = np.append(np.diff(levels), VACUUM_KM)
    views = np.asarray(view_zeniths, dtype=float)
    azimuths = np.asarray(view_azimuths, dtype=float)

    if views.shape != azimuths.shape or views.ndim != 1:
        raise ValueError("one azimuth per view zenith is required")

    species = len(particles)
    tau_p = np.asarray(particle_optical_depth, dtype=float).reshape(species, nx, ny, layers)
    gas = np.append(np.asarray(gas_scattering) + np.asarray(gas_absorption), 0.0)
    ext = np.zeros((species + 1, nx, ny, nz))

    for s in range(species):
        ext[s, :, :, :layers] = tau_p[s] / zunit[None, None, :layers]

    ext[species] = (gas / zunit)[None, None, :]
    beta = ext.sum(axis=0)
    fractions = np.divide(ext, beta[None], out=np.zeros_like(ext), where=beta[None] > 1e-16)
    ssalb = np.ones(nz)
    total_gas = np.asarray(gas_scattering) + np.asarray(gas_absorption)
    ssalb[:layers] = np.divide(
        gas_scattering, total_gas, out=np.ones(layers), where=total_gas > 1e-16
    )
    surface_albedo = np.broadcast_to(np.asarray(albedo, dtype=float), (nx, ny))
    if nmat not in (1, 3, 4):
        raise ValueError("nmat must be 1, 3 or 4")
    version = 3 if nmat == 4 else 2
    header = [version, nx, ny, nz, nmat, len(views), species, nz, nz, nz, int(save_path), int(bool(backward))]
    x_km, y_km = (pixel_km, pixel_km) if np.isscalar(pixel_km) else pixel_km
    geometry = [x_km, y_km, depolarization, 180.0 - solar_zenith, solar_azimuth, azimuths[0]]
    parts = [
        np.asarray(header, dtype=float),
        np.asarray(geometry, dtype=float),
        zunit,
        views,
        azimuths,
        -np.ones(nx * ny),
        surface_albedo.ravel(order="F"),
        np.ones(nx * ny),
        beta.ravel(order="F"),
        fractions.ravel(order="F"),
        ssalb,
    ]

    for particle in particles:
        if isinstance(particle, Particle):
            cosines, cdf, f11, f22, f33, f12 = henyey_greenstein_table(particle.asymmetry)
            # The non-polarizing particle: F44 = F11 and F34 = 0, like F22 = F33 = F11.
            f34, f44 = np.zeros_like(f11), f11.copy()
            albedo_p = particle.albedo
        else:  # tabulated: (cosines, cdf, F11, F22, F33, F12, albedo[, F34, F44])
            cosines, cdf, f11, f22, f33, f12, albedo_p = particle[:7]
            f34, f44 = particle[7:9] if len(particle) >= 9 else (None, None)
        parts += [np.array([len(cosines), albedo_p]), cosines, cdf, f11, f22, f33, f12]
        if version == 3:
            if f34 is None:
                raise ValueError("nmat 4 needs the F34 and F44 tables of every tabulated species")
            parts += [np.asarray(f34, dtype=float), np.asarray(f44, dtype=float)]

    return np.concatenate(parts).astype(np.float64)


def scene_metadata(
    name: str,
    levels_km: np.ndarray,
    *,
    nx: int,
    ny: int,
    nmat: int,
    solar_zenith: float,
    solar_azimuth: float,
    view_zeniths,
    view_azimuths,
    albedo: float,
    gas_scattering,
    gas_absorption,
    particle_optical_depth,
    save_path: bool,
    pixel_km=1.0,
    wavelength_nm: float = 340.0,
    pressure_pa=None,
    temperature_k=None,
    vmr_ppm=None,
) -> SimulationResult:
    """Labels and optical fields with the reference product's names, dimensions and
    attributes (long_name, units, plot_title; kernels/cpu/worker.f90:1272-1600). A fixture
    scene also carries its level profiles (pressure in Pa, temperature in K, absorbing-gas
    volume mixing ratios in ppm at every level). One view azimuth for all views is stored
    on the "single" dimension like the reference's; scenes that pair each view zenith with
    its own azimuth store one per view."""

    layers = len(levels_km) - 1
    alt = np.append(np.asarray(levels_km) * 1000.0, levels_km[-1] * 1000.0 + 1e-6)
    angles = len(view_zeniths)
    single_azimuth = np.all(np.asarray(view_azimuths, dtype=float) == float(view_azimuths[0]))
    tau_p = np.asarray(particle_optical_depth, dtype=float)
    species = tau_p.shape[0]
    values = {
        "asurf": np.array([float(np.mean(albedo))]),
        "n_photons_per_column": np.array([0], dtype=np.int32),
        "n_rounds": np.array([0], dtype=np.int32),
        "theta0": np.array([float(solar_zenith)]),
        "theta": np.asarray(view_zeniths, dtype=float),
        "phi0": np.array([float(solar_azimuth)]),
        "phi": np.asarray(view_azimuths, dtype=float)[:1] if single_azimuth else np.asarray(view_azimuths, dtype=float),
        "x_unit": np.array([pixel_km if np.isscalar(pixel_km) else pixel_km[0]]),
        "y_unit": np.array([pixel_km if np.isscalar(pixel_km) else pixel_km[1]]),
        "z_unit": np.diff(alt) / 1000.0,
        "alt": alt,
        "bmabs": np.append(gas_absorption, 0.0)[:, None],
        "bmsca": np.append(gas_scattering, 0.0)[:, None],
        "baer": np.concatenate([tau_p, np.zeros(tau_p.shape[:3] + (1,))], axis=3).transpose(3, 2, 1, 0)[..., None],
        "wav": np.array([wavelength_nm]),
    }
    dimensions = {
        "asurf": ("single",),
        "n_photons_per_column": ("single",),
        "n_rounds": ("single",),
        "theta0": ("single",),
        "theta": ("nvza",),
        "phi0": ("single",),
        "phi": ("single",) if single_azimuth else ("nvza",),
        "x_unit": ("single",),
        "y_unit": ("single",),
        "z_unit": ("nz",),
        "alt": ("nlev",),
        "bmabs": ("nz", "nwavs"),
        "bmsca": ("nz", "nwavs"),
        "baer": ("nz", "ny", "nx", "nscatt_types", "nwavs"),
        "wav": ("nwavs",),
        "radiance": ("nvza", "ny", "nx", "nmat", "nwavs"),
        "std_radiance": ("nvza", "ny", "nx", "nmat", "nwavs"),
        "DOP": ("nvza", "ny", "nx", "nwavs"),
        "radiance_convergence": ("nrounds", "nmat", "nwavs"),
    }
    # (long_name, units, plot_title) of worker.f90:1512-1596.
    labels = {
        "asurf": ("Surface albedo", "-", "asurf"),
        "n_photons_per_column": ("Number of photons used per column and per round", "-", "n_photons_per_column"),
        "n_rounds": ("Number of rounds used", "-", "n_rounds"),
        "theta0": ("Solar zenith angle", "deg", "solar_zenith_angle"),
        "theta": ("Viewing zenith angle", "deg", "viewing_zenith_angle"),
        "phi0": ("Solar azimuth angle", "deg", "solar_azimuth_angle"),
        "phi": ("Viewing azimuth angle", "deg", "viewing_azimuth_angle"),
        "x_unit": ("Spatial resolution in the x-direction", "km", "x_unit"),
        "y_unit": ("Spatial resolution in the y-direction", "km", "y_unit"),
        "z_unit": ("Spatial resolution in the z-direction (layer dependent)", "km", "z_unit"),
        "alt": ("Altitude", "m", "alt"),
        "bmabs": ("Molecular absorption optical thickness", "-", "bmabs"),
        "bmsca": ("Molecular scattering optical thickness", "-", "bmsca"),
        "baer": ("Aerosol total optical thickness (baerabs+baersca)", "-", "baer"),
        "wav": ("Wavelength of the light", "nm", "wav"),
        "radiance": ("TOA radiance", "-, assuming E0=pi", "radiance"),
        "std_radiance": ("Standard deviation of TOA radiance", "-", "std"),
        "DOP": ("Degree of polarization", "-", "DOP"),
        "radiance_convergence": ("radiance_convergence", "-", "radiance convergence history"),
        "AMF_layer": ("Layer AMF", "-", "AMF_layer"),
        "pres": ("Pressure", "Pa", "pres"),
        "temp": ("Temperature", "K", "temp"),
        "vmrgas": ("Volume mixing ratio of the absorbing gases", "ppm", "vmrgas"),
    }
    attributes = {name: {"long_name": long, "units": units, "plot_title": title}
                  for name, (long, units, title) in labels.items() if name in dimensions}
    if pressure_pa is not None:
        # Level profiles of a fixture (rdinput): every level row, without the vacuum level.
        values["pres"] = np.asarray(pressure_pa, dtype=float)[: layers + 1]
        values["temp"] = np.asarray(temperature_k, dtype=float)[: layers + 1]
        values["vmrgas"] = np.asarray(vmr_ppm, dtype=float).reshape(layers + 1, -1)
        dimensions.update({"pres": ("nlev",), "temp": ("nlev",), "vmrgas": ("nlev", "ngases")})
        for name in ("pres", "temp", "vmrgas"):
            long, units, title = labels[name]
            attributes[name] = {"long_name": long, "units": units, "plot_title": title}

    if save_path:
        dimensions["AMF_layer"] = ("nvza", "nz", "ny", "nx", "nwavs")
        attributes["AMF_layer"] = dict(zip(("long_name", "units", "plot_title"), labels["AMF_layer"], strict=True))
        values["AMF_layer"] = np.zeros((angles, layers, ny, nx, 1))

    # z_unit and the AMF layer axis exclude the vacuum layer in the public product.
    values["z_unit"] = values["z_unit"][:layers]
    values["alt"] = alt[: layers + 1]
    values["bmabs"] = values["bmabs"][:layers]
    values["bmsca"] = values["bmsca"][:layers]
    values["baer"] = values["baer"][:layers]
    _ = (name, nmat, species)
    return SimulationResult(None, values, dimensions, attributes)


def _atmosphere(levels):
    tau_r = rayleigh_layers(levels)
    tau_o3 = ozone_layers(levels)
    return tau_r, tau_o3


AEROSOL = Particle("aerosol", 0.70, 0.92)
CLOUD = Particle("cloud", 0.85, 0.9999)
VIEWS = ((0.0, 0.0), (30.0, 90.0), (60.0, 180.0))


def _scene(
    name,
    *,
    nx,
    ny,
    levels,
    nmat,
    save_path,
    solar_zenith,
    albedo,
    particles,
    tau_p,
    photons_per_column,
    rounds,
    views=VIEWS,
    description=None,
):
    tau_r, tau_o3 = _atmosphere(levels)
    zeniths = [v[0] for v in views]
    azimuths = [v[1] for v in views]
    tables = build_tables(
        nx=nx,
        ny=ny,
        levels_km=levels,
        nmat=nmat,
        solar_zenith=solar_zenith,
        solar_azimuth=0.0,
        view_zeniths=zeniths,
        view_azimuths=azimuths,
        albedo=albedo,
        save_path=save_path,
        gas_scattering=tau_r,
        gas_absorption=tau_o3,
        particles=particles,
        particle_optical_depth=tau_p,
    )
    metadata = scene_metadata(
        name,
        levels,
        nx=nx,
        ny=ny,
        nmat=nmat,
        solar_zenith=solar_zenith,
        solar_azimuth=0.0,
        view_zeniths=zeniths,
        view_azimuths=azimuths,
        albedo=albedo,
        gas_scattering=tau_r,
        gas_absorption=tau_o3,
        particle_optical_depth=tau_p,
        save_path=save_path,
    )
    return TransportScene(name, tables, metadata, photons_per_column, rounds, False, description or {})


def aerosol_depth(levels, nx, ny, total=0.20, top_km=2.0):
    per_layer = total * layer_fraction(levels, 0.0, top_km) * np.diff(levels) / top_km
    return np.broadcast_to(per_layer, (nx, ny, len(per_layer))).copy()


def clear_sky(photons_per_column: int = 2000, rounds: int = 32, *, nx: int = 30, ny: int = 20) -> TransportScene:
    """Plain method, clear sky at 340 nm: intensity only, one aerosol species."""

    levels = layer_levels_km()
    tau_p = aerosol_depth(levels, nx, ny)[None]
    return _scene(
        "clear-sky",
        nx=nx,
        ny=ny,
        levels=levels,
        nmat=1,
        save_path=False,
        solar_zenith=30.0,
        albedo=0.05,
        particles=[AEROSOL],
        tau_p=tau_p,
        photons_per_column=photons_per_column,
        rounds=rounds,
        description={"config": 0, "photons_per_column": photons_per_column, "rounds": rounds},
    )


def layered_cloud(photons_per_column: int = 20000, rounds: int = 128, *, nx: int = 30, ny: int = 20) -> TransportScene:
    """Layered cloud: polarized I/Q/U with AMF paths; uniform slab at 2-3 km, tau 10."""

    levels = layer_levels_km()
    layers = len(levels) - 1
    aerosol = aerosol_depth(levels, nx, ny)
    cloud_layers = layer_fraction(levels, 2.0, 3.0) * np.diff(levels)
    cloud = np.broadcast_to(10.0 * cloud_layers / cloud_layers.sum(), (nx, ny, layers)).copy()
    return _scene(
        "layered-cloud",
        nx=nx,
        ny=ny,
        levels=levels,
        nmat=3,
        save_path=True,
        solar_zenith=30.0,
        albedo=0.05,
        particles=[AEROSOL, CLOUD],
        tau_p=np.stack([aerosol, cloud]),
        photons_per_column=photons_per_column,
        rounds=rounds,
        description={"config": 1, "photons_per_column": photons_per_column, "rounds": rounds},
    )


def box_cloud(
    photons_per_column: int = 50000,
    rounds: int = 256,
    *,
    nx: int = 30,
    ny: int = 20,
    box_x=(10, 20),
    box_y=(7, 13),
    optical_depth: float = 20.0,
) -> TransportScene:
    """3-D box cloud: a 10 x 6-column block at 1-3 km, tau 20, SZA 60 degrees (I/Q/U)."""

    levels = layer_levels_km()
    layers = len(levels) - 1
    aerosol = aerosol_depth(levels, nx, ny)
    cloud_layers = layer_fraction(levels, 1.0, 3.0) * np.diff(levels)
    cloud = np.zeros((nx, ny, layers))
    cloud[box_x[0] : box_x[1], box_y[0] : box_y[1], :] = optical_depth * cloud_layers / cloud_layers.sum()
    return _scene(
        "box-cloud",
        nx=nx,
        ny=ny,
        levels=levels,
        nmat=3,
        save_path=False,
        solar_zenith=60.0,
        albedo=0.05,
        particles=[AEROSOL, CLOUD],
        tau_p=np.stack([aerosol, cloud]),
        photons_per_column=photons_per_column,
        rounds=rounds,
        description={"config": 2, "photons_per_column": photons_per_column, "rounds": rounds},
    )


def box_cloud_variant(seed: int, photons_per_column: int = 50000, rounds: int = 256) -> TransportScene:
    """A box cloud of the held-out family of the learned-importance workload: the box-cloud
    scene with a 10 x 6-column block placed at random and a log-uniform optical depth in
    [10, 40], drawn from ``numpy.random.default_rng(seed)``."""

    rng = np.random.default_rng(seed)
    x0 = int(rng.integers(0, 20))
    y0 = int(rng.integers(0, 14))
    depth = float(np.exp(rng.uniform(np.log(10.0), np.log(40.0))))
    scene = box_cloud(photons_per_column, rounds, box_x=(x0, x0 + 10), box_y=(y0, y0 + 6), optical_depth=depth)
    scene.name = f"box-cloud-{seed}"
    scene.description = {"config": 4, "seed": seed, "box": [x0, y0], "optical_depth": depth}
    return scene


def batched_scene(seed: int, *, photons_scale: float = 1.0, grid: tuple[int, int] | None = None) -> TransportScene:
    """One scene of the batched workload, drawn from ``numpy.random.default_rng(seed)``.

    Grids 8-128 columns a side, 20-60 layers, photons per column log-uniform in 1e3-1e5,
    SZA 0-70, albedo 0.02-0.30, lognormal cloud optical depth (median 5, sigma_ln 1)
    thresholded to 40 % cover in a 1-3 km layer (g 0.85), I or I/Q/U at random. ``grid``
    replaces the drawn (nx, ny); every other draw is unchanged.
    """

    rng = np.random.default_rng(seed)
    nx = int(rng.integers(8, 129))
    ny = int(rng.integers(8, 129))
    if grid is not None:
        nx, ny = (int(v) for v in grid)
    layers = int(rng.integers(20, 61))
    photons = int(round(10 ** rng.uniform(3, 5) * photons_scale))
    sza = float(rng.uniform(0, 70))
    albedo = float(rng.uniform(0.02, 0.30))
    cot = rng.lognormal(np.log(5.0), 1.0, size=(nx, ny))
    cot[cot < np.quantile(cot, 0.6)] = 0.0
    nmat = 3 if rng.uniform() < 0.5 else 1
    levels = scaled_levels_km(layers)
    aerosol = aerosol_depth(levels, nx, ny)
    cloud_layers = layer_fraction(levels, 1.0, 3.0) * np.diff(levels)
    cloud = cot[:, :, None] * (cloud_layers / cloud_layers.sum())[None, None, :]
    return _scene(
        f"batched-{seed}",
        nx=nx,
        ny=ny,
        levels=levels,
        nmat=nmat,
        save_path=False,
        solar_zenith=sza,
        albedo=albedo,
        particles=[AEROSOL, CLOUD],
        tau_p=np.stack([aerosol, cloud]),
        photons_per_column=max(1, photons),
        rounds=1,
        description={"config": 3, "seed": seed},
    )
