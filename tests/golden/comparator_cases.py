"""Seeded products and the comparator cases run on them.

Shared by make_golden.py, which records the reference comparator's verdicts on every case
(comparator_verdicts.json), and tests/test_validation.py, which runs monki.validation on the
same cases. A product is plain data — (values, dimensions, attributes) — so each side builds
its own SimulationResult from it.
"""

from __future__ import annotations

from statistics import NormalDist

import numpy as np

AXES = ("nvza", "ny", "nx", "nmat", "nwavs")


def product(seed: int = 0, views: int = 3, ny: int = 4, nx: int = 5, nmat: int = 3, rounds: int = 32):
    """A valid product: positive intensity, polarization below it, the DOP it implies,
    standard errors of a few per cent, forward views at 0, 30, 60 degrees."""

    rng = np.random.default_rng(seed)
    shape = (views, ny, nx, nmat, 1)
    radiance = np.empty(shape)
    radiance[..., 0, :] = rng.uniform(0.05, 0.3, size=(views, ny, nx, 1))
    for m in range(1, nmat):
        radiance[..., m, :] = radiance[..., 0, :] * rng.uniform(-0.4, 0.4, size=(views, ny, nx, 1))
    values = {
        "radiance": radiance,
        "std_radiance": np.abs(radiance) * rng.uniform(0.01, 0.03, size=shape) + 1e-4,
        "DOP": dop(radiance),
        "wav": np.array([340.0]),
        "theta": np.array([0.0, 30.0, 60.0][:views]),
        "n_rounds": np.array([rounds]),
        "n_photons_per_column": np.array([2000]),
        "alt": np.linspace(0.0, 60.0, 6),
    }
    dimensions = {
        "radiance": AXES,
        "std_radiance": AXES,
        "DOP": ("nvza", "ny", "nx", "nwavs"),
        "wav": ("nwavs",),
        "theta": ("nvza",),
        "n_rounds": ("single",),
        "n_photons_per_column": ("single",),
        "alt": ("nlev",),
    }
    attributes = {"radiance": {"units": "1"}, "std_radiance": {"units": "1"}}
    return values, dimensions, attributes


def dop(radiance: np.ndarray) -> np.ndarray:
    stokes = np.moveaxis(radiance, 3, -1)
    polarized = np.sqrt(np.sum(stokes[..., 1:] ** 2, axis=-1))
    out = np.zeros_like(stokes[..., 0])
    np.divide(polarized, stokes[..., 0], out=out, where=stokes[..., 0] > 0)
    return out


def _with(p, **changes):
    values, dimensions, attributes = p
    values = {k: v.copy() for k, v in values.items()}
    dimensions = dict(dimensions)
    attributes = {k: dict(v) for k, v in attributes.items()}
    for name, change in changes.items():
        if change is None:
            values.pop(name)
            dimensions.pop(name)
            continue
        value, *rest = change if isinstance(change, tuple) else (change,)
        values[name] = np.asarray(value)
        if rest:
            dimensions[name] = rest[0]
    return values, dimensions, attributes


def _radiance(p, radiance):
    return _with(p, radiance=radiance, DOP=dop(radiance))


def _threshold(p, factor):
    """One value moved to ``factor`` times the statistical bound of a default comparison."""

    values = p[0]
    n = values["radiance"].size
    z = NormalDist().inv_cdf(1.0 - 1e-6 / (2 * n))
    radiance = values["radiance"].copy()
    se = values["std_radiance"][1, 2, 3, 0, 0]
    radiance[1, 2, 3, 0, 0] += factor * (1e-10 + z * np.hypot(se, se))
    return _radiance(p, radiance)


def compare_cases():
    """(label, reference product, candidate product, keyword arguments of compare)."""

    base = product(0)
    rng = np.random.default_rng(7)
    noisy = base[0]["radiance"] + 0.5 * base[0]["std_radiance"] * rng.standard_normal(base[0]["radiance"].shape)
    relative = base[0]["radiance"] * (1 + 1e-9)
    tiny_se = _with(base, std_radiance=np.full(base[0]["radiance"].shape, 1e-12))
    shifted = tiny_se[0]["radiance"] + 1e-6
    history = (np.ones((32, 3, 1)), ("nrounds", "nmat", "nwavs"))
    with_history = _with(base, radiance_convergence=history)
    swapped = _with(base, radiance=(base[0]["radiance"].transpose(0, 2, 1, 3, 4).copy().reshape(base[0]["radiance"].shape),
                                    ("nvza", "nx", "ny", "nmat", "nwavs")))
    optics = _with(base, bmsca=(np.array([0.1, 0.2]), ("nz",)))
    units = _with(base)
    units[2]["radiance"] = {"units": "W m-2 sr-1"}
    nan = base[0]["radiance"].copy()
    nan[0, 0, 0, 0, 0] = np.nan
    return [
        ("identical statistical", base, base, {}),
        ("identical deterministic", base, base, {"mode": "deterministic"}),
        ("independent noise within errors", base, _radiance(base, noisy), {}),
        ("independent noise deterministic", base, _radiance(base, noisy), {"mode": "deterministic"}),
        ("wrong but physical x1.5", base, _radiance(base, base[0]["radiance"] * 1.5), {}),
        ("one value just above the bound", base, _threshold(base, 1.001), {}),
        ("one value just below the bound", base, _threshold(base, 0.999), {}),
        ("looser family error rate", base, _threshold(base, 0.999), {"family_error_rate": 1e-2}),
        ("relative change, deterministic", base, _radiance(base, relative), {"mode": "deterministic"}),
        ("relative change within tolerance", base, _radiance(base, relative),
         {"mode": "deterministic", "relative_tolerance": 1e-8}),
        ("absolute tolerance covers a shift", tiny_se, _radiance(tiny_se, shifted), {"absolute_tolerance": 1e-5}),
        ("shift beyond tiny errors", tiny_se, _radiance(tiny_se, shifted), {}),
        ("view zenith differs", base, _with(base, theta=np.array([0.0, 31.0, 60.0])), {}),
        ("wavelength differs", base, _with(base, wav=np.array([550.0])), {}),
        ("sentinel standard error", base, _with(base, std_radiance=np.full(base[0]["radiance"].shape, 999.0)), {}),
        ("negative standard error", base, _with(base, std_radiance=np.full(base[0]["radiance"].shape, -0.1)), {}),
        ("non-finite radiance", base, _with(base, radiance=nan), {}),
        ("thirty rounds", base, _with(base, n_rounds=np.array([30])), {}),
        ("thirty rounds deterministic", _with(base, n_rounds=np.array([30])), _with(base, n_rounds=np.array([30])),
         {"mode": "deterministic"}),
        ("inconsistent DOP", base, _with(base, DOP=np.full(base[0]["DOP"].shape, 0.9)), {}),
        ("axis names swapped", base, swapped, {}),
        ("units differ", base, units, {}),
        ("scene optics differ", optics, _with(optics, bmsca=np.array([0.1, 0.3])), {}),
        ("inventories differ", base, with_history, {}),
        ("history lengths differ, statistical", with_history,
         _with(with_history, radiance_convergence=np.ones((48, 3, 1))), {}),
        ("history lengths differ, deterministic", with_history,
         _with(with_history, radiance_convergence=np.ones((48, 3, 1))), {"mode": "deterministic"}),
        ("intensity only", product(3, nmat=1), _radiance(product(3, nmat=1), product(3, nmat=1)[0]["radiance"] * 1.001), {}),
        ("full Stokes vector", product(4, nmat=4), product(4, nmat=4), {"mode": "deterministic"}),
    ]


def check_cases():
    """(label, product, require_uncertainty) for check_result."""

    base = product(1)
    bad = base[0]["radiance"].copy()
    bad[0, 0, 0, 0, 0] = -0.1
    excess = base[0]["radiance"].copy()
    excess[1, 1, 1, 1, 0] = excess[1, 1, 1, 0, 0] + 0.5
    sing = base[0]["radiance"] * 0.4
    return [
        ("valid", base, True),
        ("valid without uncertainty", _with(base, n_rounds=np.array([12])), False),
        ("too few rounds", _with(base, n_rounds=np.array([12])), True),
        ("negative intensity and excess polarization", _with(base, radiance=bad), True),
        ("excess polarization", _with(base, radiance=excess), True),
        ("decomposition adds up", _with(base, radiance_sing=(sing, AXES), radiance_mult=(base[0]["radiance"] - sing, AXES)), True),
        ("decomposition does not add up", _with(base, radiance_sing=(sing, AXES), radiance_mult=(sing * 1.75, AXES)), True),
        ("incomplete decomposition", _with(base, radiance_sing=(sing, AXES)), True),
        ("no Stokes axis", _with(base, radiance=(base[0]["radiance"], ("nvza", "ny", "nx", "nstokes", "nwavs"))), True),
        ("two Stokes elements", _radiance(base, base[0]["radiance"][..., :2, :].copy()), True),
        ("missing DOP and wavelength", _with(base, DOP=None, wav=None), True),
        ("non-positive counts and wavelength",
         _with(base, wav=np.array([0.0]), n_photons_per_column=np.array([0])), False),
        ("misshapen standard error", _with(base, std_radiance=base[0]["std_radiance"][:2].copy()), True),
    ]


def view_cases():
    """(label, product, angles): select_views by coordinate."""

    return [
        ("two views reordered", product(2), (60.0, 0.0)),
        ("one view", product(2), (30.0,)),
        ("absent view", product(2), (45.0,)),
    ]
