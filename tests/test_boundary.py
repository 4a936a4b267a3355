"""The drop-in boundary without a GPU: the C ABI library, the host mirror of the
reference interface, and the driver statistics against the reference's own code."""

from __future__ import annotations

import ctypes
import json
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"


def header_symbols():
    text = "".join(path.read_text() for path in sorted((ROOT / "include").glob("*.h")))
    return sorted(set(re.findall(r"\b(monki_(?:cuda|mlp)_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native):
    from monki.execution import native as binding

    declared = header_symbols()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(native, name), name
    assert sorted(binding.EXPORTS) == declared
    assert native.monki_cuda_abi_version() == binding.ABI_VERSION


def test_stale_library_is_rejected(monkeypatch, tmp_path):
    from monki.execution import native as binding

    with pytest.raises(FileNotFoundError):
        binding.load(tmp_path / "missing.so")


@pytest.mark.parametrize("name", ["uniform", "box"])
@pytest.mark.parametrize("fp64", [0, 1])
def test_uniform_top_prefix_matches_reference_packer(native, name, fp64):
    """The packer's uniform-top layer and prefix optical depths equal metal_tables.pack_tables."""

    from monki.execution.native import F64P

    case = json.loads((GOLDEN / "uniform_top.json").read_text())[name]
    tables = np.asarray(case["tables"], dtype=np.float64)
    nz = int(tables[3])
    top = ctypes.c_int32(-1)
    tau = np.zeros(nz)
    err = ctypes.create_string_buffer(512)
    status = native.monki_cuda_inspect(tables.ctypes.data_as(F64P), tables.size, fp64, ctypes.byref(top), tau.ctypes.data_as(F64P), nz, err, len(err))
    assert status == 0, err.value
    assert top.value == case["uniform_top"]
    # pack_tables integrates float32 extinction in float64; fp32 sums round at 1e-7.
    np.testing.assert_allclose(tau, case["tau_above"], rtol=1e-6 if not fp64 else 1e-6, atol=1e-9)


def _rectangle_reach(native, scene, fp64):
    """(layers, reach[4, layers, ny, nx]) from the packer: cells before / after along x, y."""

    from monki.execution.native import F64P, U32P

    tables = np.ascontiguousarray(scene.tables)
    nmat, nx, ny, nz, angles = scene.shape
    extent = np.zeros(nx * ny * nz, dtype=np.uint32)
    written = ctypes.c_size_t(0)
    err = ctypes.create_string_buffer(512)
    status = native.monki_cuda_inspect_rectangles(tables.ctypes.data_as(F64P), tables.size, fp64, extent.ctypes.data_as(U32P),
                                                  extent.size, ctypes.byref(written), err, len(err))
    assert status == 0, err.value
    layers = written.value // (nx * ny)
    words = extent[: written.value].reshape((layers, ny, nx))
    return layers, np.stack([(words >> shift) & 0xFF for shift in (0, 8, 16, 24)]).astype(int)


@pytest.mark.parametrize("name", ["box_cloud", "layered_cloud", "clear_sky"])
@pytest.mark.parametrize("fp64", [0, 1])
def test_equal_extinction_rectangles_tile_each_band_layer(native, name, fp64):
    """Every band cell's rectangle holds it and lies inside the grid, all of its cells
    report the same rectangle (so the rectangles tile the layer), and it has a single
    extinction at transport precision, the only property a cell walk relies on."""

    import monki.scenes as scenes
    from monki.importance import parse_tables

    scene = getattr(scenes, name)(2, 1)
    nmat, nx, ny, nz, angles = scene.shape
    beta = parse_tables(scene.tables).beta.astype(np.float64 if fp64 else np.float32)
    layers, reach = _rectangle_reach(native, scene, fp64)
    rectangles = []
    for k in range(layers):
        seen = set()
        for j in range(ny):
            for i in range(nx):
                i0, i1 = i - reach[0, k, j, i], i + reach[1, k, j, i]
                j0, j1 = j - reach[2, k, j, i], j + reach[3, k, j, i]
                assert 0 <= i0 <= i1 < nx and 0 <= j0 <= j1 < ny
                for jj in range(j0, j1 + 1):
                    for ii in range(i0, i1 + 1):
                        r = reach[:, k, jj, ii]
                        assert (ii - r[0], ii + r[1], jj - r[2], jj + r[3]) == (i0, i1, j0, j1)
                assert np.all(beta[i0 : i1 + 1, j0 : j1 + 1, k] == beta[i, j, k])
                seen.add((i0, j0))
        rectangles.append(len(seen))
    if name == "box_cloud":
        # A cloud layer: the cloud block and four clear rectangles around it.
        assert max(rectangles) == 5
    if name == "clear_sky":
        assert layers == 0


# version 4; nmat 2; nmat 4 with particles but no F34 / F44 tables; version 3 without
# them (truncated); source off the top; four particle species
@pytest.mark.parametrize("field,value", [(0, 4), (4, 2), (4, 4), (0, 3), (7, 1), (6, 4)])
def test_packer_rejects_unsupported_tables(native, field, value):
    import monki.scenes as scenes
    from monki.execution.native import F64P

    tables = scenes.clear_sky(2, 1, nx=3, ny=2).tables.copy()
    tables[field] = value
    top = ctypes.c_int32()
    tau = np.zeros(64)
    err = ctypes.create_string_buffer(512)
    assert native.monki_cuda_inspect(tables.ctypes.data_as(F64P), tables.size, 0, ctypes.byref(top), tau.ctypes.data_as(F64P), 64, err, len(err)) == 1
    assert err.value


def test_backend_is_abstract_and_closes_on_failure():
    from monki.execution import Backend

    with pytest.raises(TypeError, match="abstract"):
        Backend()

    class Recording(Backend):
        def __init__(self):
            self.events = []

        def prepare(self, scene):
            self.events.append("prepare")

        def run_batch(self, controls):
            return controls

        def close(self):
            self.events.append("close")

    backend = Recording()
    with pytest.raises(RuntimeError, match="boom"), backend:
        raise RuntimeError("boom")
    assert backend.events == ["close"]


@pytest.mark.parametrize(
    "settings",
    [
        {"seed": -1},
        {"seed": True},
        {"seed": 2**32},
        {"photons_per_dispatch": 0},
        {"tally_shards": 0},
        {"tally_shards": 65},
        {"profile": "yes"},
        {"max_steps": 0},
        {"save_path": "yes"},
        {"precision": "bf16"},
        {"block": 48},
        {"device": -1},
        {"engine": "triton"},
        {"pool": 10},
    ],
)
def test_invalid_settings_fail_before_any_device_work(settings):
    from monki.execution import CUDA

    with pytest.raises(ValueError):
        CUDA(**settings)


@pytest.mark.parametrize(
    "scene,config,message",
    [
        ("box", "split=0.5", "split must be 0 or at least 1"),
        ("box", "roulette=0,split=2", "splitting needs a roulette weight"),
        ("layered", "roulette=0.5,split=2", "splitting needs a scene without layer paths"),
        ("box", "fused=2", "Invalid config value"),
        ("box", "tail=-1", "Invalid config value"),
        ("backward", "roulette=0.5", "guided transport and importance tallies need forward transport"),
        ("backward", "engine=megakernel", "backward transport and nmat 4 need engine=wavefront"),
        ("box", "engine=megakernel,orders=1", "need engine=wavefront"),
    ],
)
def test_session_settings_are_validated_before_any_device_work(native, scene, config, message):
    """The packer and the configuration parser reject unsupported combinations with the
    message the host reports, before looking for a device (so this runs on any machine)."""
    import monki.scenes as scenes
    from monki.execution.native import F64P

    if scene == "backward":
        tables = scenes.box_cloud(2, 1, nx=6, ny=4, box_x=(1, 3), box_y=(1, 2)).tables.copy()
        tables[11] = 1
    elif scene == "layered":
        tables = scenes.layered_cloud(2, 1, nx=3, ny=2).tables
    else:
        tables = scenes.box_cloud(2, 1, nx=6, ny=4, box_x=(1, 3), box_y=(1, 2)).tables
    tables = np.ascontiguousarray(tables)
    err = ctypes.create_string_buffer(512)
    handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, 1, config.encode(), err, len(err))
    assert not handle
    assert message in err.value.decode()


def test_cuda_rejects_cloud_and_unprepared_use():
    from monki.execution import CUDA, BatchControls

    with pytest.raises(TypeError):
        CUDA(provider="aws")

    with pytest.raises(RuntimeError, match="prepared"):
        CUDA().run_batch(BatchControls(1, 10))


def test_reference_case_needs_the_fixture_home(monkeypatch, tmp_path):
    from monki import ReferenceCase
    from monki.execution import CUDA

    monkeypatch.delenv("MONKI_HOME", raising=False)
    case = ReferenceCase("clear", "testrun/MONKI_MLS_cloudfree_340_340_test.in")
    with pytest.raises(ValueError, match="MONKI_HOME"):
        CUDA().prepare(case)
    # A home without the fixture fails before any device work.
    with pytest.raises(FileNotFoundError):
        CUDA(monki_home=tmp_path).prepare(case)


def test_amf_moments_match_reference_implementation():
    from monki.convergence import AMFMoments
    from monki.execution.tallies import BatchControls, RawTallies

    g = np.load(GOLDEN / "amf_moments.npz")
    moments = AMFMoments()
    for index in range(g["paths"].shape[0]):
        moments.add(RawTallies(BatchControls(index + 1, 100), np.zeros((3, 2, 3, 2)), g["paths"][index], g["weights"][index]))
    amf, error = moments.estimate(g["thickness"])
    np.testing.assert_allclose(amf, g["amf"], rtol=1e-12)
    np.testing.assert_allclose(error, g["error"], rtol=1e-12)


def _fixed_backend(golden):
    from monki.execution import Backend
    from monki.execution.tallies import RawTallies
    from monki.output import SimulationResult

    nz = golden["paths"].shape[3]
    angles = golden["stokes"].shape[-1]
    ny, nx = golden["stokes"].shape[3], golden["stokes"].shape[2]
    metadata = SimulationResult(
        None,
        {
            "alt": golden["alt"],
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
            return RawTallies(controls, golden["stokes"][r].copy(), golden["paths"][r].copy(), golden["weights"][r].copy())

        def close(self):
            pass

    return Fixed()


@pytest.mark.parametrize("label", ["fixed", "amf"])
def test_driver_statistics_match_reference_simulate(tmp_path, label):
    from monki import AMFConvergence, SimulationResult, simulate

    golden = dict(np.load(GOLDEN / "driver_statistics.npz"))
    case = type("Case", (), {"photons_per_column": int(golden["photons_per_column"]), "rounds": golden["stokes"].shape[0], "backward": False})
    convergence = AMFConvergence(minimum_rounds=32, check_every=16) if label == "amf" else None
    result = simulate(case(), _fixed_backend(golden), tmp_path / f"{label}.nc", convergence=convergence)
    loaded = SimulationResult.load(tmp_path / f"{label}.nc")

    for name in ("radiance", "std_radiance", "DOP", "radiance_convergence", "AMF_layer", "std_AMF_layer"):
        key = f"{label}_{name}"
        if key not in golden:
            continue
        np.testing.assert_allclose(result.values[name], golden[key], rtol=1e-12, atol=1e-15, err_msg=name)
        np.testing.assert_allclose(loaded.values[name], golden[key], rtol=1e-12, atol=1e-15, err_msg=name)

    receipt = json.loads((tmp_path / f"{label}.run.json").read_text())
    assert receipt["completed_rounds"] <= golden["stokes"].shape[0]
    with pytest.raises(FileExistsError):
        simulate(case(), _fixed_backend(golden), tmp_path / f"{label}.nc")


def test_late_outlier_resets_precision_streak():
    from monki import AMFConvergence
    from monki.convergence import AMFStopping
    from monki.execution.tallies import RawTallies

    class Synthetic:
        def run_batches(self, requests):
            return [
                RawTallies(r, np.ones((3, 1, 1, 1)), np.full((1, 1, 2, 1), 100.0 if r.round_index == 48 else 1.0), np.ones((1, 1, 1)))
                for r in requests
            ]

    case = type("Case", (), {"rounds": 64, "photons_per_column": 100})
    stopping = AMFStopping(AMFConvergence(minimum_rounds=32, check_every=16), np.array([1.0]))
    assert len(list(stopping.batches(Synthetic(), case()))) == 64
    assert not stopping.converged
    assert [h["streak"] for h in stopping.history][:2] == [1, 0]


def test_radiance_stopping_uses_intensity_relative_error():
    from monki import RadianceConvergence
    from monki.convergence import RadianceStopping
    from monki.execution.tallies import RawTallies

    rng = np.random.default_rng(0)

    class Synthetic:
        def run_batches(self, requests):
            return [RawTallies(r, 100 * (1 + 0.001 * rng.standard_normal((3, 2, 2, 1)))) for r in requests]

    case = type("Case", (), {"rounds": 256, "photons_per_column": 100})
    stopping = RadianceStopping(RadianceConvergence(0.01, minimum_rounds=32, check_every=32, consecutive_checks=2), 100)
    batches = list(stopping.batches(Synthetic(), case()))
    assert stopping.converged and len(batches) == 64


@pytest.mark.parametrize("minimum, every, rounds", [(32, 5, 60), (128, 32, 256), (32, 1, 40), (64, 16, 40)])
def test_rounds_before_the_first_check_run_as_one_group(minimum, every, rounds):
    """The first request covers every round up to the first check; the checks (rounds and
    values) are those of the reference schedule of groups of check_every."""
    from monki import AMFConvergence
    from monki.convergence import AMFStopping
    from monki.execution.tallies import RawTallies

    rng = np.random.default_rng(3)
    groups = []

    class Synthetic:
        def run_batches(self, requests):
            groups.append([r.round_index for r in requests])
            return [
                RawTallies(r, np.ones((3, 1, 1, 1)), 1 + 0.3 * rng.random((1, 1, 2, 1)), np.ones((1, 1, 1)))
                for r in requests
            ]

    case = type("Case", (), {"rounds": rounds, "photons_per_column": 100})
    policy = AMFConvergence(relative_error=0.5, minimum_rounds=minimum, check_every=every, consecutive_checks=100)
    stopping = AMFStopping(policy, np.array([1.0]))
    assert len(list(stopping.batches(Synthetic(), case()))) == rounds
    ends = [min(start + every - 1, rounds) for start in range(1, rounds + 1, every)]
    checked = [e for e in ends if e >= minimum]
    assert [h["rounds"] for h in stopping.history] == checked
    first = checked[0] if checked else rounds
    assert groups[0] == list(range(1, first + 1))
    assert [g[-1] for g in groups] == [first] + [e for e in ends if e > first]


@pytest.mark.parametrize("builder", ["clear_sky", "layered_cloud", "box_cloud"])
def test_scene_builders_produce_valid_tables(oracle, builder):
    import monki.scenes as scenes

    scene = getattr(scenes, builder)(10, 4)
    assert oracle.validate(scene.tables) is None
    nmat, nx, ny, nz, angles = scene.shape
    assert (nx, ny, nz, angles) == (30, 20, 35, 3)
    assert len(scene.metadata.values["alt"]) == nz  # physical levels only
    # Optical depths of the synthetic atmosphere.
    assert scene.metadata.values["bmsca"].sum() == pytest.approx(0.70)
    assert scene.metadata.values["bmabs"].sum() == pytest.approx(0.30)


def test_batched_scene_generator_is_seeded():
    import monki.scenes as scenes

    a, b = scenes.batched_scene(3), scenes.batched_scene(3)
    np.testing.assert_array_equal(a.tables, b.tables)
    assert not np.array_equal(a.tables, scenes.batched_scene(4).tables)
