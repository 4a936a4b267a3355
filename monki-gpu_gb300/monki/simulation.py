"""Round statistics and the saved product, shared by every backend.

Follows the reference driver (python/monki/simulation.py:17-189): fixed or
convergence-scheduled rounds, FP64 sums of each round's normalized Stokes tallies and
their squares, the standard error of the mean with the 999 sentinel through round 30,
the U sign flip of backward transport, layer AMF = paths / weights / thickness without
the vacuum layer, an exclusive-create NetCDF product and a ``.run.json`` receipt.
"""

from __future__ import annotations

import hashlib
import json
from dataclasses import asdict
from pathlib import Path

import numpy as np

from .convergence import AMFConvergence, AMFStopping, RadianceConvergence, RadianceStopping
from .execution.backend import Backend
from .execution.tallies import BatchControls, RawTallies
from .output import SimulationResult


def file_hash(path: Path) -> str:
    return hashlib.sha256(Path(path).read_bytes()).hexdigest()


def _host_rounds(case, backend, stopping):
    """Round sums from each round's host tallies (the reference driver's loop)."""

    if stopping is not None:
        batches = stopping.batches(backend, case)
    else:
        requests = [BatchControls(i, case.photons_per_column) for i in range(1, case.rounds + 1)]
        batches = backend.run_batches(requests)

        if len(batches) != case.rounds:
            raise ValueError("Backend returned the wrong number of statistical rounds")

    total = rounds_sum = rounds_squared = paths = weights = None
    history = []
    orders = None

    for index, batch in enumerate(batches, start=1):
        if not isinstance(batch, RawTallies):
            raise TypeError("Backend must return RawTallies")

        if batch.controls != BatchControls(index, case.photons_per_column):
            raise ValueError("Backend returned tallies for a different round")

        if total is None:
            total = np.zeros_like(batch.stokes)
            rounds_sum = np.zeros_like(batch.stokes)
            rounds_squared = np.zeros_like(batch.stokes)

            if batch.weighted_paths is not None:
                paths = np.zeros_like(batch.weighted_paths)
                weights = np.zeros_like(batch.weights)

        total += batch.stokes
        normalized = batch.stokes / case.photons_per_column
        rounds_sum += normalized
        rounds_squared += normalized**2
        _, nx, ny, angles = total.shape
        # Successive spatial sums then divisions, all Stokes components kept.
        history.append(rounds_sum.sum(axis=1).sum(axis=1).sum(axis=1) / nx / ny / angles / index)

        if paths is not None:
            if batch.weighted_paths is None or batch.weights is None:
                raise ValueError("Backend dropped path diagnostics during a session")

            paths += batch.weighted_paths
            weights += batch.weights

        if getattr(batch, "orders", None) is not None:
            if orders is None:
                orders = {name: np.zeros_like(value) for name, value in batch.orders.items()}
            for name, value in batch.orders.items():
                orders[name] += value

    if orders is not None:
        backend.provenance["scattering_orders"] = orders  # summed over rounds, raw
    return total, rounds_sum, rounds_squared, history, paths, weights


def _lookahead(stopping, groups, g, backend, ppc) -> int:
    """How many checked groups, from ``g`` on, to run in one held dispatch: the rounds the last
    check says the target still needs, at least three, within one dispatch (0 when group ``g``
    alone exceeds a dispatch). A round past the stopping point costs its transport; one
    dispatch too few costs a wait for the slowest histories of a dispatch, worth about three
    rounds on the box cloud."""

    estimate = stopping.rounds_estimate()
    first = groups[g][0]
    capacity = backend.held_capacity(ppc)
    if groups[g][1] - first + 1 > capacity:
        return 0  # a group larger than one dispatch goes through accumulate
    if estimate is None:
        return 1
    wanted = max(3.0, estimate - (first - 1))
    count, rounds = 0, 0
    for f, e, _ in groups[g:]:
        size = e - f + 1
        if count and (rounds + size > capacity or rounds + size > wanted):
            break
        count, rounds = count + 1, rounds + size
    return count


def _device_rounds(case, backend, stopping):
    """Round sums folded on the device in FP64 (``backend.accumulate``): the same rounds,
    schedule and checks; only the per-round tallies stay on the GPU. The history is the
    running pixel sum of the device's per-round sums (equal to the host's to rounding).

    After the first check, backends with held groups (``run_held`` / ``fold_next``) run the
    rounds the last check says are still needed in one dispatch and fold them one at a time,
    checking where the schedule checks: the same rounds are folded and the same checks made
    as when each group is its own dispatch, rounds past the stopping point are computed and
    discarded, and a dispatch's straggling histories are waited for once per held group
    instead of once per check."""

    ppc = case.photons_per_column
    groups = list(stopping.groups(case.rounds)) if stopping is not None else [(1, case.rounds, False)]
    held = bool(getattr(backend, "lookahead", False)) and hasattr(backend, "run_held")
    rows = []
    g = 0

    while g < len(groups):
        first, end, checked = groups[g]
        ahead = _lookahead(stopping, groups, g, backend, ppc) if held and checked and stopping.history else 0
        if ahead:
            last = groups[g + ahead - 1][1]
            backend.run_held([BatchControls(i, ppc) for i in range(first, last + 1)])

            for f, e, c in groups[g : g + ahead]:
                rows.extend(backend.fold_next()[None, :] for _ in range(f, e + 1))

                if c:
                    stopping.load(backend.statistics())
                    stopping.check(e)

                    if stopping.converged:
                        break

            g += ahead
        else:
            rows.append(backend.accumulate([BatchControls(i, ppc) for i in range(first, end + 1)]))
            g += 1

            if checked:
                stopping.load(backend.statistics())
                stopping.check(end)

        if stopping is not None and stopping.converged:
            break

    statistics = backend.statistics()
    total = statistics["total"]
    _, nx, ny, angles = total.shape
    running = np.cumsum(np.concatenate(rows), axis=0)
    history = [running[r] / nx / ny / angles / (r + 1) for r in range(statistics["rounds"])]
    return (total, statistics["sum"], statistics["squares"], history, statistics.get("paths"),
            statistics.get("weights"))


def simulate(case, backend: Backend, output, *, convergence: AMFConvergence | None = None) -> SimulationResult:
    """Run equally sized rounds, save the product and its receipt, return the result.

    With a convergence policy, ``case.rounds`` is the hard round cap; the receipt tells
    convergence apart from exhausting the cap.
    """

    if convergence is not None and case.rounds < convergence.minimum_rounds:
        raise ValueError("round cap must be at least minimum_rounds")

    output = Path(output).resolve()
    receipt = output.with_suffix(".run.json")

    if output.exists() or receipt.exists():
        raise FileExistsError(f"Refusing to overwrite an existing result: {output}")

    with backend:
        backend.prepare(case)
        metadata = backend.metadata

        if metadata is None:
            raise RuntimeError("Backend did not supply prepared scene metadata")

        stopping = None

        if isinstance(convergence, RadianceConvergence):
            stopping = RadianceStopping(convergence, case.photons_per_column)
        elif convergence is not None:
            if "AMF_layer" not in metadata.values:
                raise ValueError("AMF stopping requires layer path diagnostics")

            stopping = AMFStopping(convergence, np.diff(metadata.values["alt"]) / 1000)

        device = getattr(backend, "device_statistics_available", None)

        if device is not None and device(case.photons_per_column):
            total, rounds_sum, rounds_squared, history, paths, weights = _device_rounds(case, backend, stopping)
        else:
            total, rounds_sum, rounds_squared, history, paths, weights = _host_rounds(case, backend, stopping)

        completed = len(history)
        _, nx, ny, angles = total.shape
        radiance = total / completed / case.photons_per_column
        uncertainty = np.full_like(radiance, 999.0)

        # 999 marks an unavailable uncertainty through round 30.
        if completed > 30:
            variance_sum = rounds_squared - (1.0 / completed) * rounds_sum**2
            tolerance = 64 * np.finfo(float).eps * np.maximum(rounds_squared, 1e-300)

            if np.any(variance_sum < -tolerance):
                raise ArithmeticError("Negative round variance exceeds floating-point roundoff")

            uncertainty = np.sqrt(np.maximum(variance_sum, 0) / (completed - 1)) / np.sqrt(completed)

        radiance_history = np.asarray(history)

        if case.backward and radiance.shape[0] >= 3:
            radiance[2] *= -1
            radiance_history[:, 2] *= -1

        intensity = radiance[0]
        polarization = np.sqrt(np.sum(radiance[1:] ** 2, axis=0))
        dop = np.divide(polarization, intensity, out=np.zeros_like(intensity), where=intensity > 1e-16)
        values = {name: value.copy() for name, value in metadata.values.items()}
        values["radiance"] = radiance.transpose(3, 2, 1, 0)[..., None]
        values["std_radiance"] = uncertainty.transpose(3, 2, 1, 0)[..., None]
        values["DOP"] = dop.transpose(2, 1, 0)[..., None]
        values["radiance_convergence"] = radiance_history[..., None]
        values["n_rounds"] = np.full_like(values["n_rounds"], completed)
        values["n_photons_per_column"] = np.full_like(values["n_photons_per_column"], case.photons_per_column)

        if paths is not None:
            if np.any(weights <= 0):
                raise ValueError("Layer AMF is undefined for a pixel with no detected weight")

            # Lengths are km; altitudes are m. The vacuum layer is dropped.
            thickness = np.diff(values["alt"]) / 1000.0
            amf = paths[:, :, :-1, :] / weights[:, :, None, :] / thickness[None, None, :, None]
            values["AMF_layer"] = amf.transpose(3, 2, 1, 0)[..., None]

        dimensions = dict(metadata.dimensions)
        attributes = dict(metadata.attributes)
        orders = backend.provenance.pop("scattering_orders", None) if hasattr(backend, "provenance") else None

        if orders is not None:
            # Scattering-order diagnostics with the reference product's names
            # (kernels/cpu/worker.f90:1462-1492): single and multiple scattering, and the
            # contribution of each event location (layer axis: surface, then the physical
            # layers), normalized like the radiance.
            scale = 1.0 / completed / case.photons_per_column
            single = orders["single"] * scale
            located = orders["locations"] * scale  # layer axis: surface + physical layers
            located_single = orders["single_locations"] * scale
            pixel_axes = (3, 2, 1, 0)
            location_axes = (4, 3, 2, 1, 0)
            values["radiance_sing"] = single.transpose(pixel_axes)[..., None]
            values["radiance_mult"] = (radiance - single).transpose(pixel_axes)[..., None]
            values["contrib_radiance_3D"] = located.transpose(location_axes)[..., None]
            values["contrib_radiance_3D_sing"] = located_single.transpose(location_axes)[..., None]
            values["contrib_radiance_3D_mult"] = (located - located_single).transpose(location_axes)[..., None]
            for name, label in (("radiance_sing", "single scattering"), ("radiance_mult", "multiple scattering")):
                dimensions[name] = ("nvza", "ny", "nx", "nmat", "nwavs")
                attributes[name] = {"long_name": f"TOA radiance, {label} only", "units": "-, assuming E0=pi"}
            for suffix, label in (("", ""), ("_sing", ", single scattering"), ("_mult", ", multiple scattering")):
                dimensions["contrib_radiance_3D" + suffix] = ("nvza", "nz_withsurf", "ny", "nx", "nmat", "nwavs")
                attributes["contrib_radiance_3D" + suffix] = {
                    "long_name": f"TOA radiance 3D contribution by event location{label}", "units": "-"}

        if isinstance(stopping, AMFStopping) and not isinstance(stopping, RadianceStopping):
            _, amf_error = stopping.moments.estimate(stopping.thickness)
            values["std_AMF_layer"] = amf_error.transpose(3, 2, 1, 0)[..., None]
            dimensions["std_AMF_layer"] = dimensions["AMF_layer"]
            attributes["std_AMF_layer"] = {"long_name": "Layer AMF standard error", "units": "-"}

        result = SimulationResult(output, values, dimensions, attributes)
        result.save()
        provenance = {
            **backend.provenance,
            "status": "complete",
            "completed_rounds": completed,
            "total_photons": completed * case.photons_per_column * nx * ny,
            "output_sha256": file_hash(output),
        }

        if stopping is not None:
            provenance["status"] = "converged" if stopping.converged else "max_rounds_reached"
            provenance["radiance_convergence" if isinstance(stopping, RadianceStopping) else "amf_convergence"] = {
                "policy": asdict(stopping.policy),
                "converged": stopping.converged,
                "checks": stopping.history,
                "uncertainty": "pointwise relative standard error",
            }

        with receipt.open("x") as stream:
            stream.write(json.dumps(provenance, indent=2) + "\n")

        return result
