"""The CUDA product against the oracle's through the reference's own acceptance gate.

``monki.validation.compare`` is the comparator the reference uses to accept one backend's
product against another's (python/monki/validation.py:146-253): the radiance of two
independent runs must agree within the Bonferroni bound of their combined standard errors
(family error rate 1e-6), after every coordinate, unit, shape and product check passes. Here
the FP32 product of ``simulate`` with the CUDA backend faces the FP64 oracle's (independent
seeds), and a radiance scaled by 1.5 must fail the same gate.
"""

from __future__ import annotations

import sys
from dataclasses import replace
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent))
from oracle_backend import oracle_backend  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["clear", "cloud"])
def test_cuda_product_passes_the_reference_gate_against_the_oracle(oracle, device, tmp_path, name):
    from monki import scenes, simulate
    from monki.execution import CUDA
    from monki.validation import check_result, compare

    scene = scenes.clear_sky(400, 32, nx=8, ny=6) if name == "clear" else scenes.layered_cloud(60, 32, nx=8, ny=6)
    expected = simulate(scene, oracle_backend(oracle, 5), tmp_path / "oracle.nc")
    product = simulate(scene, CUDA(seed=6), tmp_path / "cuda.nc")

    assert check_result(product) == []
    report = compare(expected, product)
    assert report.passed, report.details
    assert report.compared_values == product.radiance.size

    wrong = replace(product, values={**product.values, "radiance": product.radiance * 1.5})
    assert not compare(expected, wrong).passed
