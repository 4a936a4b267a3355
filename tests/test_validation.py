"""The product comparator (monki.validation) against the reference's own.

The reference accepts one backend's product against another's with check_result / compare
(python/monki/validation.py); its unit tests hold that plausible wrong results must not pass
(tests/unit/test_validation.py). Here every case of tests/golden/comparator_cases.py is run
through monki.validation and checked against the verdict, counts, largest errors and reasons
the reference's comparator gave on the same case (tests/golden/comparator_verdicts.json),
and the comparator then judges products of the oracle run through ``simulate``.
"""

from __future__ import annotations

import json
import sys
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import comparator_cases as cases  # noqa: E402

sys.path.insert(0, str(GOLDEN.parent))
from oracle_backend import oracle_backend  # noqa: E402


@pytest.fixture(scope="module")
def verdicts():
    return json.loads((GOLDEN / "comparator_verdicts.json").read_text())


def _result(p):
    from monki import SimulationResult

    return SimulationResult(Path("synthetic.nc"), *p)


def test_compare_verdicts_equal_the_reference_comparator(verdicts):
    from monki.validation import compare

    expected = {v["label"]: v for v in verdicts["compare"]}
    run = cases.compare_cases()
    assert [label for label, *_ in run] == [v["label"] for v in verdicts["compare"]]

    for label, a, b, kwargs in run:
        got = compare(_result(a), _result(b), **kwargs).to_dict()
        want = expected[label]
        assert got["passed"] == want["passed"], label
        assert got["mode"] == want["mode"], label
        assert got["compared_values"] == want["compared_values"], label
        assert got["failed_values"] == want["failed_values"], label
        assert got["max_absolute_error"] == pytest.approx(want["max_absolute_error"], rel=1e-12, abs=0), label
        assert got["max_normalized_error"] == pytest.approx(want["max_normalized_error"], rel=1e-9, abs=0), label
        assert sorted(got["details"]) == want["details"], label


def test_check_result_reasons_equal_the_reference(verdicts):
    from monki.validation import check_result

    expected = {v["label"]: v["failures"] for v in verdicts["check"]}

    for label, p, require in cases.check_cases():
        assert sorted(check_result(_result(p), require_uncertainty=require)) == expected[label], label


def test_views_are_selected_by_coordinate_like_the_reference(verdicts):
    from monki.validation import select_views

    expected = {v["label"]: v for v in verdicts["views"]}

    for label, p, angles in cases.view_cases():
        want = expected[label]

        if "error" in want:
            with pytest.raises(ValueError, match="absent or ambiguous"):
                select_views(_result(p), angles)
            continue

        chosen = select_views(_result(p), angles)
        assert chosen.values["theta"].tolist() == want["theta"]
        np.testing.assert_allclose([chosen.values["radiance"][i].sum() for i in range(len(angles))],
                                   want["radiance_sum"], rtol=1e-14)
        assert chosen.values["DOP"].shape[0] == len(angles)
        assert chosen.values["wav"].tolist() == [340.0]


def test_view_selection_needs_forward_view_zeniths():
    from monki.validation import select_views

    values, dimensions, attributes = cases.product(0)
    dimensions = {**dimensions, "theta": ("single",)}
    with pytest.raises(ValueError, match="forward theta"):
        select_views(_result((values, dimensions, attributes)), (0.0,))


@pytest.mark.parametrize("rate", [0.0, 1.0, -1.0, float("nan")])
def test_invalid_family_error_rate_is_rejected(rate):
    from monki.validation import compare

    p = _result(cases.product(0))
    with pytest.raises(ValueError, match="family_error_rate"):
        compare(p, p, family_error_rate=rate)


@pytest.mark.parametrize("kwargs,message", [
    ({"mode": "exact"}, "mode must be"),
    ({"absolute_tolerance": -1.0}, "tolerances"),
    ({"relative_tolerance": float("inf")}, "tolerances"),
])
def test_invalid_policy_is_rejected(kwargs, message):
    from monki.validation import compare

    p = _result(cases.product(0))
    with pytest.raises(ValueError, match=message):
        compare(p, p, **kwargs)


@pytest.fixture(scope="module")
def oracle_products(oracle, tmp_path_factory):
    from monki import scenes, simulate

    root = tmp_path_factory.mktemp("products")
    out = {}
    for name, scene in (("clear", scenes.clear_sky(200, 32, nx=6, ny=4)),
                        ("cloud", scenes.layered_cloud(40, 32, nx=6, ny=4))):
        for seed in (1, 2):
            out[name, seed] = simulate(scene, oracle_backend(oracle, seed), root / f"{name}_{seed}.nc")
        out[name, "again"] = simulate(scene, oracle_backend(oracle, 1), root / f"{name}_again.nc")
    return out


@pytest.mark.parametrize("name", ["clear", "cloud"])
def test_independent_oracle_runs_pass_the_statistical_gate(oracle_products, name):
    from monki.validation import check_result, compare

    a, b = oracle_products[name, 1], oracle_products[name, 2]
    assert check_result(a) == [] and check_result(b) == []
    report = compare(a, b)
    assert report.passed, report.details
    assert report.compared_values == a.radiance.size and report.max_normalized_error < 1


@pytest.mark.parametrize("name", ["clear", "cloud"])
def test_scaled_radiance_fails_and_replays_pass_deterministically(oracle_products, name):
    from monki.validation import compare

    a, again = oracle_products[name, 1], oracle_products[name, "again"]
    assert compare(a, again, mode="deterministic").passed
    assert not compare(a, oracle_products[name, 2], mode="deterministic").passed

    scaled = replace(a, values={**a.values, "radiance": a.radiance * 1.5})
    report = compare(oracle_products[name, 2], scaled)
    assert not report.passed and report.failed_values > 0 and report.max_normalized_error > 1
