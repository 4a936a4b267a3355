"""Checks of one MONKI product and comparisons of two.

Mirrors the reference's comparator (python/monki/validation.py:1-253), the gate its tests and
scientific suite use to accept one backend's product against another's:

* ``check_result`` lists what is wrong with a single product: required variables missing,
  non-finite values, a radiance without a Stokes axis or with a Stokes length other than
  1, 3 or 4, negative intensity, polarization beyond the intensity plus mc.f90's absolute
  1e-2 guard (``stokes_criterium_error``), a DOP inconsistent with the Stokes components,
  standard errors that are negative, misshapen, or not yet available (fewer than 31 rounds,
  or the 999 sentinel), non-positive wavelength or counts, and single + multiple scattering
  that does not add up to the total.
* ``compare`` first refuses products that are not the same case (failed checks, different
  variable inventories, axis names, shapes or units, coordinates or scene optics more than
  1e-12 apart), then compares the radiance statistically — |a - b| within
  ``absolute_tolerance`` + z * hypot(SE_a, SE_b), z the normal quantile of a Bonferroni tail
  ``family_error_rate`` / (2 n) over the n compared values — or, in deterministic mode, every
  numeric variable within ``absolute_tolerance`` + ``relative_tolerance`` * |a|.

The failure messages are the reference's, so callers that match on them keep working.
"""

from __future__ import annotations

from dataclasses import asdict, dataclass
from statistics import NormalDist

import numpy as np

from .output import SimulationResult

# Variables that fix the case: the geometry and spectral coordinates, and the scene optics.
COORDINATES = ("wav", "theta", "theta0", "phi", "phi0", "asurf", "x_unit", "y_unit", "z_unit")
SCENE_VARIABLES = ("pres", "temp", "alt", "bmabs", "bmsca", "baer", "vmrgas")

STOKES_PHYSICAL_TOLERANCE = 1e-2  # mc.f90: sqrt(Q^2 + U^2) may exceed I by this much
COORDINATE_TOLERANCE = 1e-12
UNCERTAINTY_SENTINEL = 999
MINIMUM_UNCERTAINTY_ROUNDS = 31

_REQUIRED = ("radiance", "std_radiance", "DOP", "wav", "n_rounds", "n_photons_per_column")


@dataclass(frozen=True)
class Comparison:
    """Outcome of ``compare``: the verdict, the counts, the largest errors and the reasons."""

    passed: bool
    mode: str
    compared_values: int
    failed_values: int
    max_absolute_error: float
    max_normalized_error: float
    details: tuple[str, ...]

    def to_dict(self):
        return asdict(self)


def select_views(result: SimulationResult, angles: tuple[float, ...]) -> SimulationResult:
    """The product restricted to the forward views whose zenith equals each of ``angles``
    (within 1e-12), in that order: views are chosen by coordinate, never by position."""

    if result.dimensions.get("theta") != ("nvza",) or "theta" not in result.values:
        raise ValueError("view selection requires forward theta(nvza)")

    theta = np.asarray(result.values["theta"])
    picked = []

    for angle in angles:
        found = np.flatnonzero(np.abs(theta - angle) <= 1e-12)

        if found.size != 1:
            raise ValueError(f"view {angle} is absent or ambiguous")

        picked.append(int(found[0]))

    values = {}

    for name, data in result.values.items():
        dims = result.dimensions[name]
        values[name] = np.take(data, picked, axis=dims.index("nvza")) if "nvza" in dims else data.copy()

    return SimulationResult(result.path, values, dict(result.dimensions), dict(result.attributes))


def _stokes_last(result: SimulationResult) -> np.ndarray:
    # The Stokes axis is found by name: the product's axis order is NetCDF's, not Fortran's.
    return np.moveaxis(result.radiance, result.dimensions["radiance"].index("nmat"), -1)


def check_result(result: SimulationResult, *, require_uncertainty: bool = True) -> list[str]:
    """Every reason the product is not a valid MONKI radiance product (empty when valid)."""

    values = result.values
    missing = [f"missing variable: {name}" for name in _REQUIRED if name not in values]

    if missing:
        return missing

    failures = [
        f"non-finite values: {name}"
        for name, data in values.items()
        if np.issubdtype(np.asarray(data).dtype, np.number) and not np.isfinite(data).all()
    ]

    if "nmat" not in result.dimensions["radiance"]:
        failures.append("radiance has no nmat dimension")
        return failures

    stokes = _stokes_last(result)

    if stokes.shape[-1] not in (1, 3, 4):
        failures.append("Stokes vector must contain 1, 3, or 4 elements")

    intensity = stokes[..., 0]
    polarized = np.sqrt(np.sum(stokes[..., 1:] ** 2, axis=-1))

    if (intensity < -1e-12).any():
        failures.append("negative intensity")

    if (polarized > intensity + STOKES_PHYSICAL_TOLERANCE).any():
        failures.append("polarized magnitude exceeds intensity")

    # The DOP is derived from the Stokes components; a product whose arrays each look
    # plausible can still disagree with itself here.
    dop = np.zeros_like(intensity)
    np.divide(polarized, intensity, out=dop, where=intensity > 0)
    stored = values["DOP"]

    if stored.shape != intensity.shape or not np.allclose(stored, dop, rtol=1e-9, atol=1e-10):
        failures.append("DOP is inconsistent with Stokes components")

    error = result.standard_error

    if error.shape != result.radiance.shape or result.dimensions["std_radiance"] != result.dimensions["radiance"]:
        failures.append("standard-error shape/dimensions differ from radiance")

    if (error < 0).any():
        failures.append("negative standard error")

    if require_uncertainty:
        too_few = int(np.asarray(values["n_rounds"]).item()) < MINIMUM_UNCERTAINTY_ROUNDS

        if too_few or (error == UNCERTAINTY_SENTINEL).any():
            failures.append("uncertainty unavailable: need more than 30 completed rounds")

    if (values["wav"] <= 0).any():
        failures.append("non-positive wavelength")

    failures += [f"non-positive {name}" for name in ("n_rounds", "n_photons_per_column") if (values[name] <= 0).any()]

    parts = [name for name in ("radiance_sing", "radiance_mult") if name in values]

    if len(parts) == 1:
        failures.append("incomplete scattering decomposition")
    elif parts and not np.allclose(result.radiance, values["radiance_sing"] + values["radiance_mult"], rtol=1e-9, atol=1e-10):
        failures.append("single + multiple scattering does not equal total radiance")

    return failures


def _misalignments(reference: SimulationResult, candidate: SimulationResult, mode: str) -> list[str]:
    """Reasons the two products are not the same case, before any numbers are compared."""

    statistical = mode == "statistical"
    problems = [f"reference: {item}" for item in check_result(reference, require_uncertainty=statistical)]
    problems += [f"candidate: {item}" for item in check_result(candidate, require_uncertainty=statistical)]

    if set(reference.values) != set(candidate.values):
        problems.append("variable inventories differ")

    for name in sorted(set(reference.values) & set(candidate.values)):
        a, b = reference.values[name], candidate.values[name]
        aligned = reference.dimensions[name] == candidate.dimensions[name] and a.shape == b.shape

        # Convergence histories of independent statistical runs may have different lengths.
        if not aligned and not (statistical and name == "radiance_convergence"):
            problems.append(f"shape/dimension mismatch: {name}")

        if reference.attributes.get(name, {}).get("units") != candidate.attributes.get(name, {}).get("units"):
            problems.append(f"units mismatch: {name}")

    for name in COORDINATES + SCENE_VARIABLES:
        if name in reference.values and name in candidate.values:
            a, b = reference.values[name], candidate.values[name]

            if a.shape != b.shape or not np.allclose(a, b, rtol=0, atol=COORDINATE_TOLERANCE):
                problems.append(f"coordinate mismatch: {name}")

    return problems


def compare(
    reference: SimulationResult,
    candidate: SimulationResult,
    *,
    mode: str = "statistical",
    absolute_tolerance: float = 1e-10,
    relative_tolerance: float = 1e-10,
    family_error_rate: float = 1e-6,
) -> Comparison:
    """Compare two products of the same case (module docstring). Statistical mode compares
    the radiance against the combined standard errors; deterministic mode compares every
    numeric variable of two runs of the same configuration."""

    if mode not in ("statistical", "deterministic"):
        raise ValueError("mode must be statistical or deterministic")

    if not all(np.isfinite(t) and t >= 0 for t in (absolute_tolerance, relative_tolerance)):
        raise ValueError("tolerances must be finite and non-negative")

    if not 0 < family_error_rate < 1:
        raise ValueError("family_error_rate must be in (0, 1)")

    problems = _misalignments(reference, candidate, mode)

    if problems:
        return Comparison(False, mode, 0, 0, 0.0, 0.0, tuple(problems))

    compared = failed = 0
    worst_absolute = worst_normalized = 0.0
    tiny = np.finfo(float).tiny

    for name in ["radiance"] if mode == "statistical" else sorted(reference.values):
        a, b = reference.values[name], candidate.values[name]

        if not np.issubdtype(a.dtype, np.number):
            if not np.array_equal(a, b):
                problems.append(f"non-numeric values differ: {name}")
            continue

        delta = np.abs(a.astype(float) - b.astype(float))

        if mode == "statistical":
            # Independent estimates add variances; the Bonferroni tail covers the many
            # pixels and components checked at once without assuming they are independent.
            tail = max(family_error_rate / (2 * a.size), np.finfo(float).eps)
            z = NormalDist().inv_cdf(1.0 - tail)
            bound = absolute_tolerance + z * np.hypot(reference.standard_error, candidate.standard_error)
        else:
            bound = absolute_tolerance + relative_tolerance * np.abs(a)

        over = delta > bound
        count = int(np.count_nonzero(over))
        compared += a.size
        failed += count
        worst_absolute = max(worst_absolute, float(np.max(delta, initial=0.0)))
        worst_normalized = max(worst_normalized, float(np.max(delta / np.maximum(bound, tiny), initial=0.0)))

        if count:
            problems.append(f"{name}: {count}/{a.size} values exceed tolerance")

    return Comparison(not problems, mode, compared, failed, worst_absolute, worst_normalized, tuple(problems))
