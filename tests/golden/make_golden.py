"""Generate the golden fixtures of tests/golden from the reference project.

Run in a container where the reference is mounted (default /root/reference, or the
MONKI_REFERENCE environment variable); the fixtures it writes are committed, so the
tests never need the reference at run time.

What each fixture pins, and where it comes from:
  philox_kat.json        Random123 Philox4x32-10 known-answer vector, read from the
                         reference's device test (tests/integration/test_metal.py:43-59).
  polarization_probe.json
                         The probe geometries of tests/native/metal_probe.f90:10-16 with
                         expected L2 F L1 S from an independent numpy restatement of
                         ray_scat_matrix / stokes_rot_mat / matmul_stokes_rot
                         (mc_routines_general_mod.f90:74-136, 942-1242); the Fortran
                         itself cannot be compiled here (no gfortran).
  amf_moments.npz        The reference's own AMFMoments (python/monki/convergence.py)
                         on seeded synthetic rounds: inputs, AMF and its standard error.
  uniform_top.json       The reference's own pack_tables (python/monki/execution/
                         metal_tables.py) on version-1 streams built here: the first
                         uniform layer and the optical depth above each layer.
  driver_statistics.npz  The reference's own simulate() (python/monki/simulation.py)
                         driven by a fixed synthetic backend: radiance, standard error,
                         DOP, convergence history, layer AMF and its standard error.
  archived_*.npz         The reference's archived Fortran outputs of its three test runs
                         (fortran/monki/upstream/OUTPUT/testrun/*.nc, read by
                         hdf5_reader.py): radiance, standard error and settings, the
                         Fortran preparer's optical depths, and the tables that
                         monki.preparation builds for the same run.
  budget_moments.npz     The oracle's per-entry round moments (sums of tally / photons per
                         column and of its square over 32 rounds) for the workloads at their
                         own photon budgets and four config-3 scenes; the GPU parity test
                         compares against them.
  archived_amf_oracle.npz
                         The oracle's layer-path round moments for the archived clear-sky and
                         1-layer-cloud runs at their own budgets (10,000 and 20,000 photons per
                         column, 100 rounds, every view): per view and layer the sums over
                         rounds of the path tally p, of the weight tally w, and of p^2, w^2
                         and p w.
  comparator_verdicts.json
                         The reference's own check_result / compare / select_views
                         (python/monki/validation.py) on the seeded products and cases of
                         comparator_cases.py: each verdict, its counts and largest errors,
                         and its reasons.

``python tests/golden/make_golden.py [name ...]`` writes only the named fixtures (the stem
of each file name); with no names, all of them.
"""

from __future__ import annotations

import json
import os
import re
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("MONKI_REFERENCE", "/root/reference"))
REPO = HERE.parents[1]


def reference_package():
    """Import the reference's pure-Python package with a stand-in for netCDF4."""

    class Variable:
        def __init__(self, store, name):
            self.store, self.name = store, name

        def setncatts(self, attributes):
            self.store.setdefault("_attributes", {})[self.name] = dict(attributes)

        def __setitem__(self, key, value):
            self.store[self.name] = np.array(value, copy=True)

    class Dataset:
        written: dict = {}

        def __init__(self, path, mode="r", clobber=True):
            self.path = Path(path)
            self.store = {}
            Dataset.written[str(self.path)] = self.store
            self.path.write_bytes(b"golden-placeholder")

        def __enter__(self):
            return self

        def __exit__(self, *args):
            return False

        def createDimension(self, name, size):
            self.store.setdefault("_dimensions", {})[name] = size

        def createVariable(self, name, dtype, dimensions):
            return Variable(self.store, name)

    stub = types.ModuleType("netCDF4")
    stub.Dataset = Dataset
    sys.modules["netCDF4"] = stub
    sys.path.insert(0, str(REFERENCE / "python"))
    import monki  # the reference package
    import monki.convergence
    import monki.execution.metal_tables
    import monki.simulation

    return monki, Dataset


def philox_kat():
    text = (REFERENCE / "tests/integration/test_metal.py").read_text()
    words = re.search(r"assert_array_equal\(actual, \[([^\]]+)\]\)", text).group(1)
    return {
        "counter": [0, 0, 0, 0],
        "key": [0, 0],
        "expected": [int(w.strip(), 16) for w in words.split(",")],
        "source": "Random123 kat_vectors via tests/integration/test_metal.py:43-59",
    }


def _probe_geometry():
    text = (REFERENCE / "tests/native/metal_probe.f90").read_text()

    def vector(name):
        match = re.search(name + r"\s*=\s*\[([^\]]+)\]", text)
        return [float(v.split("_")[0]) for v in match.group(1).split(",")]

    return vector("incoming"), vector("outgoing"), vector("phi_in"), vector("phi_out"), vector("stokes")


def _numpy_probe(depol, uo, u1, phio, phi1, stokes):
    """L2 F L1 S for Rayleigh scattering, written from the Fortran formulas."""

    eps = 1e-16
    cs = uo * u1 + np.sqrt(1 - uo * uo) * np.sqrt(1 - u1 * u1) * np.cos(phio - phi1)
    sin2 = 0.0 if 1 - cs * cs < eps else 1 - cs * cs
    delta = (1 - depol) / (1 + depol / 2)
    F = np.zeros((3, 3))
    F[0, 0] = 0.75 * (1 + cs * cs)
    F[0, 1] = F[1, 0] = -0.75 * sin2
    F[1, 1] = 0.75 * (1 + cs * cs)
    F[2, 2] = 1.5 * cs
    F *= delta
    F[0, 0] += 1 - delta
    F /= 4
    L = []

    # Meridian rotation angles (general, vertical-incident and vertical-scattered cases).
    dphi = abs(phio - phi1)
    rem = dphi % np.pi

    if rem < eps or abs(rem - np.pi) < eps or (abs(uo) > 1 - eps and abs(u1) > 1 - eps):
        c1 = c2 = 1.0
        s1 = s2 = 0.0
    else:
        sino = 0.0 if 1 - uo * uo < eps else np.sqrt(1 - uo * uo)
        sin1 = 0.0 if 1 - u1 * u1 < eps else np.sqrt(1 - u1 * u1)
        wo = np.array([sino * np.cos(phio), sino * np.sin(phio)])
        w1 = np.array([sin1 * np.cos(phi1), sin1 * np.sin(phi1)])
        wophi = np.array([np.cos(phio), np.sin(phio)])
        w1phi = np.array([np.cos(phi1), np.sin(phi1)])

        if abs(u1) > 1 - eps:
            cosi1 = np.copysign(1.0, u1)
            cosi2 = -cosi1 * (w1phi @ wophi)
            q = wo[1] * w1phi[0] - wo[0] * w1phi[1]
        elif abs(uo) > 1 - eps:
            cosi2 = np.copysign(1.0, uo)
            cosi1 = -cosi2 * (w1phi @ wophi)
            q = wophi[1] * w1[0] - wophi[0] * w1[1]
        else:
            cosi1 = (u1 - uo * cs) / np.sqrt(max(eps, (1 - uo * uo) * (1 - cs * cs)))
            cosi2 = (uo - u1 * cs) / np.sqrt(max(eps, (1 - u1 * u1) * (1 - cs * cs)))
            q = wo[1] * w1[0] - wo[0] * w1[1]

        sini1 = 0.0 if 1 - cosi1**2 < eps else np.sqrt(1 - cosi1**2) * np.copysign(1.0, q)
        sini2 = 0.0 if 1 - cosi2**2 < eps else np.sqrt(1 - cosi2**2) * np.copysign(1.0, q)
        c1, s1 = cosi1**2 - sini1**2, 2 * sini1 * cosi1
        c2, s2 = cosi2**2 - sini2**2, 2 * sini2 * cosi2

    for c, s in ((c1, s1), (c2, s2)):
        L.append(np.array([[1, 0, 0], [0, c, -s], [0, s, c]]))

    P = L[1] @ F @ L[0]
    return P @ np.asarray(stokes)


def polarization_probe():
    uo, u1, phio, phi1, stokes = _probe_geometry()
    expected = [
        _numpy_probe(0.03, uo[i], u1[i], phio[i], phi1[i], stokes).tolist() for i in range(3)
    ]
    return {
        "depol": 0.03,
        "incoming": uo,
        "outgoing": u1,
        "phi_in": phio,
        "phi_out": phi1,
        "stokes": stokes,
        "expected": expected,
        "rtol": 1e-5,
        "atol": 1e-7,
        "source": "geometries of tests/native/metal_probe.f90; values from a numpy restatement",
    }


def amf_moments(ref):
    from monki.convergence import AMFMoments
    from monki.execution.tallies import BatchControls, RawTallies

    rng = np.random.default_rng(123)
    weights = rng.uniform(1, 4, (100, 2, 3, 2))
    paths = weights[:, :, :, None, :] * rng.uniform(1, 5, (100, 2, 3, 5, 2))
    moments = AMFMoments()

    for index in range(100):
        moments.add(RawTallies(BatchControls(index + 1, 100), np.zeros((3, 2, 3, 2)), paths[index], weights[index]))

    thickness = np.array([0.5, 2.0, 5.0, 1.0])
    amf, error = moments.estimate(thickness)
    return {"paths": paths, "weights": weights, "thickness": thickness, "amf": amf, "error": error}


def _v1_stream(varying: bool):
    """A version-1 stream (one species) for pack_tables, built without the product code."""

    nx, ny = 6, 4
    levels = np.concatenate([np.arange(0, 10, 0.5), np.arange(10, 30, 2.0), np.arange(30, 60.01, 7.5)])
    layers = len(levels) - 1
    nz = layers + 1
    zunit = np.append(np.diff(levels), 1e-9)
    tau_gas = 0.7 * (np.exp(-levels[:-1] / 8) - np.exp(-levels[1:] / 8)) / (1 - np.exp(-60 / 8))
    tau_aer = np.zeros((nx, ny, layers))
    tau_aer[:, :, :4] = 0.05

    if varying:
        tau_aer[2:4, 1:3, 2:6] += 3.0  # a box occupying layers 2..5

    ext = np.zeros((2, nx, ny, nz))
    ext[0, :, :, :layers] = tau_aer / zunit[:layers]
    ext[1, :, :, :layers] = (tau_gas / zunit[:layers])[None, None, :]
    beta = ext.sum(0)
    frac = np.divide(ext, beta[None], out=np.zeros_like(ext), where=beta[None] > 1e-16)
    n = 181
    cosines = np.cos(np.deg2rad(np.linspace(180, 0, n)))
    f11 = 0.51 / (1.49 - 1.4 * cosines) ** 1.5
    cdf = np.concatenate([[0], np.cumsum(np.diff(cosines) * (f11[1:] + f11[:-1]) / 2)])
    cdf /= cdf[-1]
    parts = [
        [1, nx, ny, nz, 3, 3, 1, nz, nz, nz, 1, 0],
        [1.0, 1.0, 0.0279, 150.0, 0.0, 40.0],
        zunit,
        [0.0, 30.0, 60.0],
        -np.ones(nx * ny),
        np.full(nx * ny, 0.05),
        np.ones(nx * ny),
        beta.ravel(order="F"),
        frac.ravel(order="F"),
        np.ones(nz),
        [n, 0.92],
        cosines,
        cdf,
        f11,
        f11,
        f11,
        np.zeros(n),
    ]
    return np.concatenate([np.asarray(p, dtype=float) for p in parts])


def uniform_top(ref):
    from monki.execution.metal_tables import pack_tables

    cases = {}

    for name, varying in (("uniform", False), ("box", True)):
        raw = _v1_stream(varying)
        packed, (nmat, nx, ny, nz, angles) = pack_tables(raw)
        cases[name] = {
            "tables": raw.tolist(),
            "uniform_top": int(packed[15]),
            "tau_above": packed[-nz:].astype(float).tolist(),
            "height_above": packed[-2 * nz : -nz].astype(float).tolist(),
        }

    return cases


def driver_statistics(ref, Dataset):
    from monki import AMFConvergence, simulate
    from monki.execution.backend import Backend
    from monki.execution.tallies import RawTallies
    from monki.output import SimulationResult

    nmat, nx, ny, nz, angles, ppc = 3, 3, 2, 5, 2, 40
    rng = np.random.default_rng(7)
    rounds = 64
    stokes = rng.uniform(0.5, 2.0, (rounds, nmat, nx, ny, angles))
    stokes[:, 1:] -= 1.25
    weights = rng.uniform(1.0, 3.0, (rounds, nx, ny, angles))
    paths = weights[:, :, :, None, :] * rng.uniform(0.5, 4.0, (rounds, nx, ny, nz, angles))
    alt = np.array([0.0, 500.0, 1500.0, 4000.0, 10000.0])
    metadata = SimulationResult(
        Path("scene.nc"),
        {
            "alt": alt,
            "n_rounds": np.array([0], dtype=np.int32),
            "n_photons_per_column": np.array([0], dtype=np.int32),
            "AMF_layer": np.zeros((angles, nz - 1, ny, nx, 1)),
        },
        {
            "alt": ("nlev",),
            "n_rounds": ("single",),
            "n_photons_per_column": ("single",),
            "AMF_layer": ("nvza", "nz", "ny", "nx", "nwavs"),
            "radiance": ("nvza", "ny", "nx", "nmat", "nwavs"),
            "std_radiance": ("nvza", "ny", "nx", "nmat", "nwavs"),
            "DOP": ("nvza", "ny", "nx", "nwavs"),
            "radiance_convergence": ("nrounds", "nmat", "nwavs"),
        },
        {},
    )

    class Fixed(Backend):
        def __init__(self):
            self.metadata = None
            self.provenance = {"backend": "fixed"}

        def prepare(self, scene):
            self.metadata = metadata

        def run_batch(self, controls):
            r = controls.round_index - 1
            return RawTallies(controls, stokes[r].copy(), paths[r].copy(), weights[r].copy())

        def close(self):
            pass

    Case = type("Case", (), {"photons_per_column": ppc, "rounds": rounds, "backward": False})

    results = {}

    with tempfile.TemporaryDirectory() as tmp:
        for label, convergence in (("fixed", None), ("amf", AMFConvergence(minimum_rounds=32, check_every=16))):
            out = Path(tmp) / f"{label}.nc"
            simulate(Case(), Fixed(), out, convergence=convergence)
            store = Dataset.written[str(out.resolve())]

            for name in ("radiance", "std_radiance", "DOP", "radiance_convergence", "AMF_layer", "std_AMF_layer"):
                if name in store:
                    results[f"{label}_{name}"] = store[name]

    results.update(
        {
            "stokes": stokes,
            "paths": paths,
            "weights": weights,
            "alt": alt,
            "photons_per_column": np.array(ppc),
        }
    )
    return results


def prepared_fixture():
    """The 2boxclouds fixture prepared by monki.preparation from the reference's INPUT and
    DATA files (Mie LUT with F12, Rayleigh with King factors, O3 absorption): the tables
    and the optical depths, so GPU tests can run the scene where the fixtures are absent."""

    sys.path.insert(0, str(REPO / "monki-gpu_gb300"))
    from monki import ReferenceCase
    from monki.preparation import prepare_reference_case

    case = ReferenceCase("2boxclouds", "testrun/MONKI_MLS_2boxclouds_340_340_test.in", photons_per_column=100,
                         rounds=32, solar_zenith=45.0)
    scene = prepare_reference_case(case, REFERENCE / "fortran" / "monki" / "upstream")
    return {"tables": scene.tables, "bmsca": scene.metadata.values["bmsca"], "bmabs": scene.metadata.values["bmabs"],
            "alt": scene.metadata.values["alt"], "depolarization": np.array(scene.description["depolarization"])}


def benchmark_scenes():
    """The two cases of the reference's time-to-AMF-precision benchmark
    (validation/benchmark_amf_convergence.py: validation/cases/{clear,layered-cloud}.json at
    8,000 photons per column and an 8,192-round cap), prepared by monki.preparation."""

    sys.path.insert(0, str(REPO / "monki-gpu_gb300"))
    from dataclasses import replace

    from monki import ReferenceCase
    from monki.preparation import prepare_reference_case, scene_arrays

    out = {}
    for name in ("clear", "layered-cloud"):
        spec = json.loads((REFERENCE / "validation" / "cases" / f"{name}.json").read_text())
        case = replace(ReferenceCase(**spec), photons_per_column=8000, rounds=8192)
        scene = prepare_reference_case(case, REFERENCE / "fortran" / "monki" / "upstream")
        out[name] = scene_arrays(scene, {})
    return out


ARCHIVED = {
    "cloudfree": "MONKI_MLS_cloudfree_340_340_test.in",
    "1layercloud": "MONKI_MLS_1layercloud_340_340_test.in",
    "2boxclouds": "MONKI_MLS_2boxclouds_340_340_test.in",
}
ARCHIVED_VIEWS = 15  # view zeniths per prepared scene (the device scene holds up to 16)
ARCHIVED_ARRAYS = ("radiance", "std_radiance", "DOP", "AMF_layer", "theta", "theta0", "phi0", "phi", "asurf",
                   "n_photons_per_column", "n_rounds", "bmsca", "bmabs", "baer", "alt", "z_unit", "x_unit", "y_unit",
                   "pres", "temp", "vmrgas", "wav")


def archived_schema(f) -> dict:
    """Dimensions (name: size) and, per variable, its dimension names and its long_name,
    units and plot_title, from the netCDF-4 bookkeeping of an archived file: dimensions are
    the datasets marked as dimension scales (_Netcdf4Dimid), a variable's dimensions its
    _Netcdf4Coordinates ids."""

    scales, variables = {}, {}
    for name in f.names():
        attributes = f.attributes(name)
        if attributes.get("CLASS") == "DIMENSION_SCALE":
            scales[int(attributes["_Netcdf4Dimid"][0])] = (name, int(f.dataset(name)["shape"][0]))
    for name in f.names():
        attributes = f.attributes(name)
        if "_Netcdf4Coordinates" in attributes:
            variables[name] = {
                "dimensions": [scales[int(i)][0] for i in attributes["_Netcdf4Coordinates"]],
                "attributes": {key: attributes[key] for key in ("long_name", "units", "plot_title") if key in attributes},
            }
    return {"dimensions": {name: size for name, size in scales.values()}, "variables": variables}


def archived_runs():
    """The reference's archived Fortran outputs (fortran/monki/upstream/OUTPUT/testrun/*.nc,
    NetCDF-4 read by hdf5_reader.py) with the scene this repository prepares for each: the
    radiance, its standard error and the run's settings, the Fortran preparer's optical
    depths, and the prepared table stream of the run's first view_group (later groups
    differ only in their view zeniths)."""

    sys.path.insert(0, str(REPO / "monki-gpu_gb300"))
    sys.path.insert(0, str(HERE))
    from hdf5_reader import HDF5File
    from monki import ReferenceCase
    from monki.preparation import prepare_reference_case

    home = REFERENCE / "fortran" / "monki" / "upstream"
    out = {}
    for name, input_file in ARCHIVED.items():
        path = next((home / "OUTPUT" / "testrun").glob(f"MONKI_MLS_{name}_340_340_*.nc"))
        with HDF5File(path) as f:
            arrays = {key: f.read(key) for key in ARCHIVED_ARRAYS if key in f.links()}
            schema = archived_schema(f)
        theta = np.asarray(arrays["theta"], dtype=float)
        groups = [np.arange(g, min(g + ARCHIVED_VIEWS, theta.size)) for g in range(0, theta.size, ARCHIVED_VIEWS)]
        case = ReferenceCase(name, f"testrun/{input_file}",
                             photons_per_column=int(arrays["n_photons_per_column"][0]),
                             rounds=int(arrays["n_rounds"][0]), surface_albedo=float(arrays["asurf"][0]),
                             solar_zenith=float(arrays["theta0"][0]), solar_azimuth=float(arrays["phi0"][0]),
                             view_azimuth=float(arrays["phi"][0]), view_zeniths=tuple(theta[groups[0]]))
        scene = prepare_reference_case(case, home)
        arrays = {key: np.asarray(value) for key, value in arrays.items()}
        arrays["tables"] = scene.tables
        arrays["view_groups"] = np.array([[g[0], g[-1] + 1] for g in groups])
        arrays["source"] = np.array(f"fortran/monki/upstream/OUTPUT/testrun/{path.name}")
        arrays["schema"] = np.array(json.dumps(schema, sort_keys=True))
        out[name] = arrays
    return out


# The workloads at their own photon budgets (32 rounds each), for the FP32 GPU parity test:
# builder of monki.scenes, its arguments, and the oracle's seed (independent of the GPU's).
# The layered cloud runs on a reduced 6 x 4 grid (its 20,000 photons per column on the full
# grid would take the oracle half an hour here); config-3 scenes at a tenth of their budgets.
BUDGETS = {
    "clear_sky": ("clear_sky", (2000, 32), {}),
    "layered_cloud": ("layered_cloud", (20000, 32), {"nx": 6, "ny": 4}),
    "box_cloud": ("box_cloud", (2000, 32), {}),
}
BATCHED_SCALE = 0.005  # config-3 photon budgets scaled so every pick gets about 40 per column
ORACLE_SEED = 1000003


def batched_picks():
    """Four config-3 scenes (seed, grid override): seed 93's draws on a 128 x 128 grid (the
    workload's largest), and the first seeds of 0-199 with I only, with I/Q/U, and with a
    grid under 32 x 32."""

    sys.path.insert(0, str(REPO / "monki-gpu_gb300"))
    import monki.scenes as scenes

    shapes = {seed: scenes.batched_scene(seed, photons_scale=BATCHED_SCALE).shape for seed in range(200)}
    nmat1 = next(s for s in shapes if shapes[s][0] == 1 and s != 93)
    nmat3 = next(s for s in shapes if shapes[s][0] == 3 and s not in (93, nmat1))
    small = next(s for s in shapes if shapes[s][1] * shapes[s][2] < 32 * 32 and s not in (93, nmat1, nmat3))
    picks = {"largest": (93, (128, 128)), "nmat1": (nmat1, None), "nmat3": (nmat3, None), "small": (small, None)}
    out = {}
    for label, (seed, grid) in picks.items():
        full = scenes.batched_scene(seed, grid=grid).photons_per_column
        out[label] = (seed, grid, min(1.0, 40.0 / full))
    return out


def table_fingerprint(tables):
    """Sums and an evenly strided sample (at most 4,096 entries, the header included) of a
    scene's tables. The scene builders call numpy's exp, log and trigonometry, whose last
    bits differ between x86 and Arm builds, so a consumer compares these within a relative
    1e-10 rather than byte for byte."""

    t = np.asarray(tables, dtype=np.float64)
    stride = max(1, -(-t.size // 4096))
    return {"tables_size": np.array(t.size), "tables_sums": np.array([t.sum(), np.abs(t).sum(), (t * t).sum()]),
            "tables_head": t[:16].copy(), "tables_sample": t[::stride].copy()}


def budget_moments():
    """Per-entry round moments of the oracle at the workloads' own budgets: for every tally
    entry (Stokes, and layer paths and weights when the scene has them) the sum over the
    rounds of tally / photons per column and of its square; the per-round domain means of
    the Stokes components (the convergence history); the scatters; a fingerprint of the
    tables (table_fingerprint)."""

    sys.path.insert(0, str(REPO / "monki-gpu_gb300"))
    sys.path.insert(0, str(REPO))
    import monki.scenes as scenes
    from oracle import oracle

    specs = dict(BUDGETS)
    for label, (seed, grid, scale) in batched_picks().items():
        specs[f"batched_{label}"] = ("batched_scene", (seed,), {"photons_scale": scale, "grid": grid})
    out = {}
    for name, (builder, args, kwargs) in specs.items():
        scene = getattr(scenes, builder)(*args, **kwargs)
        rounds = 32
        ppc = scene.photons_per_column
        nmat, nx, ny, nz, angles = scene.shape
        per_round = ppc * nx * ny
        tallies, counters = oracle.run(scene.tables, [per_round * rounds, 0, 1, ORACLE_SEED, 100000, 0, per_round, rounds],
                                       os.cpu_count() or 1)
        x = tallies / ppc
        stokes = np.stack([oracle.split(scene.tables, tallies[r])[0] for r in range(rounds)])
        out[name] = {
            "builder": np.array(builder), "args": np.array(json.dumps([list(args), kwargs])),
            "rounds": np.array(rounds), "photons_per_column": np.array(ppc), "seed": np.array(ORACLE_SEED),
            "sum": x.sum(0), "squares": (x * x).sum(0),
            "history": stokes.sum(axis=(2, 3, 4)) / (nx * ny * angles) / ppc,
            "scatters": np.array(counters["scatters"]),
            **table_fingerprint(scene.tables),
        }
        print(name, scene.shape, ppc, counters["scatters"], flush=True)
    return out


def archived_amf_oracle():
    """Layer-path round moments of the oracle for the archived runs that kept layer AMFs
    (the clear sky and the 1-layer cloud), at each run's photons and rounds, views in the
    archived order (about 12 minutes on 8 cores); keys "<run>.<moment>"."""

    sys.path.insert(0, str(HERE.parent))
    sys.path.insert(0, str(REPO))
    import archived_runs as ar
    from oracle import oracle

    out = {}
    for name in ("cloudfree", "1layercloud"):
        fixture = ar.load(name)
        ppc, rounds = int(fixture["n_photons_per_column"][0]), int(fixture["n_rounds"][0])
        layers = fixture["z_unit"].size
        views = fixture["theta"].size
        moments = {key: np.zeros((views, layers)) for key in ("p", "pp", "pw")}
        moments.update({key: np.zeros(views) for key in ("w", "ww")})
        for lo, hi in ar.view_groups(fixture):
            tables = ar.with_views(fixture["tables"], fixture["theta"][lo:hi])
            tallies, _ = oracle.run(tables, [ppc * rounds, 0, 1, ORACLE_SEED, 100000, 0, ppc, rounds],
                                    os.cpu_count() or 1)
            parts = [oracle.split(tables, tallies[r]) for r in range(rounds)]
            p = np.stack([q[1][0, 0, :layers, :] for q in parts])  # (round, layer, view), 1 x 1 column
            w = np.stack([q[2][0, 0, :] for q in parts])  # (round, view)
            moments["p"][lo:hi] = p.sum(0).T
            moments["pp"][lo:hi] = (p * p).sum(0).T
            moments["pw"][lo:hi] = (p * w[:, None, :]).sum(0).T
            moments["w"][lo:hi] = w.sum(0)
            moments["ww"][lo:hi] = (w * w).sum(0)
            print(name, "views", lo, hi, flush=True)
        moments.update({"photons_per_column": np.array(ppc), "rounds": np.array(rounds), "seed": np.array(ORACLE_SEED)})
        out.update({f"{name}.{key}": value for key, value in moments.items()})
    return out


def comparator_verdicts(ref):
    """The reference comparator's verdicts on the cases of comparator_cases.py."""

    import monki.output
    import monki.validation

    sys.path.insert(0, str(HERE))
    import comparator_cases as cases

    def result(p):
        return monki.output.SimulationResult(Path("synthetic.nc"), *p)

    def verdict(c):
        out = c.to_dict()
        out["details"] = sorted(out["details"])
        return out

    compare = [
        {"label": label, **verdict(monki.validation.compare(result(a), result(b), **kwargs))}
        for label, a, b, kwargs in cases.compare_cases()
    ]
    check = [
        {"label": label, "failures": sorted(monki.validation.check_result(result(p), require_uncertainty=req))}
        for label, p, req in cases.check_cases()
    ]
    views = []
    for label, p, angles in cases.view_cases():
        try:
            chosen = monki.validation.select_views(result(p), angles)
            views.append({"label": label, "theta": chosen.values["theta"].tolist(),
                          "radiance_sum": [float(chosen.values["radiance"][i].sum()) for i in range(len(angles))]})
        except ValueError as error:
            views.append({"label": label, "error": str(error)})
    return {"compare": compare, "check": check, "views": views}


def _forget_package():
    """Drop this repository's ``monki`` (and its path) so the reference's package, which has
    the same name, can be imported next."""

    for name in [m for m in sys.modules if m == "monki" or m.startswith("monki.")]:
        del sys.modules[name]
    ours = str(REPO / "monki-gpu_gb300")
    sys.path[:] = [p for p in sys.path if p != ours]


def main(names=()):
    wanted = set(names)

    def want(name):
        return not wanted or name in wanted

    # Fixtures prepared by this repository's package first, then the reference's package.
    if want("prepared_2boxclouds"):
        np.savez_compressed(HERE / "prepared_2boxclouds.npz", **prepared_fixture())
    for name, arrays in benchmark_scenes().items() if want("prepared_benchmark") else ():
        np.savez_compressed(HERE / f"prepared_{name.replace('-', '_')}.npz", **arrays)
    for name, arrays in archived_runs().items() if want("archived") else ():
        np.savez_compressed(HERE / f"archived_{name}.npz", **arrays)
    if want("budget_moments"):
        np.savez_compressed(HERE / "budget_moments.npz",
                            **{f"{name}.{key}": value for name, arrays in budget_moments().items()
                               for key, value in arrays.items()})
    if want("archived_amf_oracle"):
        np.savez_compressed(HERE / "archived_amf_oracle.npz", **archived_amf_oracle())
    _forget_package()
    ref, Dataset = reference_package()
    if want("philox_kat"):
        (HERE / "philox_kat.json").write_text(json.dumps(philox_kat(), indent=1) + "\n")
    if want("polarization_probe"):
        (HERE / "polarization_probe.json").write_text(json.dumps(polarization_probe(), indent=1) + "\n")
    if want("amf_moments"):
        np.savez_compressed(HERE / "amf_moments.npz", **amf_moments(ref))
    if want("uniform_top"):
        (HERE / "uniform_top.json").write_text(json.dumps(uniform_top(ref)) + "\n")
    if want("driver_statistics"):
        np.savez_compressed(HERE / "driver_statistics.npz", **driver_statistics(ref, Dataset))
    if want("comparator_verdicts"):
        (HERE / "comparator_verdicts.json").write_text(json.dumps(comparator_verdicts(ref), indent=1) + "\n")
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1:])
