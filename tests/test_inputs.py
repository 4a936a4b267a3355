"""``ReferenceCase`` validation, as the reference's own input tests hold it
(tests/unit/test_inputs.py:14-31): every malformed request fails at construction."""

from __future__ import annotations

import pytest

INPUT = "testrun/MONKI_MLS_cloudfree_340_340_test.in"


@pytest.mark.parametrize(
    "arguments",
    [
        {"rounds": 0},
        {"rounds": True},
        {"rounds": 2**31},
        {"photons_per_column": -1},
        {"photons_per_column": 1.5},
        {"view_zeniths": ()},
        {"view_zeniths": (90,)},
        {"view_zeniths": tuple(range(92))},
        {"surface_albedo": 1.1},
        {"surface_albedo": float("nan")},
        {"solar_zenith": float("nan")},
        {"solar_azimuth": 360.0},
        {"view_azimuth": -1.0},
        {"input_file": "../escape.in"},
        {"input_file": "/abs/escape.in"},
        {"name": "../escape"},
        {"name": ""},
        {"backward": 1},
    ],
)
def test_invalid_case_rejected(arguments):
    from monki import ReferenceCase

    with pytest.raises(ValueError):
        ReferenceCase(**({"name": "clear", "input_file": INPUT} | arguments))


def test_valid_case_keeps_the_reference_defaults():
    from monki import ReferenceCase

    case = ReferenceCase("clear", INPUT)
    assert (case.photons_per_column, case.rounds, case.surface_albedo, case.solar_zenith) == (200, 32, 0.05, 45.0)
    assert case.view_zeniths == (0.0, 30.0, 60.0) and case.backward is False
    assert ReferenceCase("layered-cloud_2", INPUT, backward=True, view_zeniths=(89.9,)).backward
