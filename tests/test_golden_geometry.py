"""Geometry packing and decoding pinned to the reference's executed Python.

tests/golden/reference_geometry.json holds the outputs of the reference's own
utils.angle / utils.param_set and config values (generated by
tests/golden/make_golden.py, which runs that code)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from fanbeamctrecon_tensorflowop_gb300 import config as cfg_mod
from fanbeamctrecon_tensorflowop_gb300.geometry import angle, decode, param_set

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_geometry.json").read_text())


def test_config_mirrors_reference():
    ours = cfg_mod.default_config()
    assert set(ours) == set(GOLDEN["config"])
    for k, v in GOLDEN["config"].items():
        assert ours[k] == v, k


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: c["label"])
def test_angle_and_param_set_bitwise(case):
    c = cfg_mod.default_config()
    c.StartAngle = case["start_angle"]
    if case["label"] == "alt_scanner_shift":
        c.SourceDetectorDistance = 1117.6
        c.SourceAxisDistance = 889
        c.ProjectionsPerRotation = 1081
        c.DetectorColumnNumber = 2001
        c.DetectorShift = 1.25
    a = angle(c.ProjectionsPerRotation, c.StartAngle)
    p = param_set(case["nimg"], c)
    assert a.dtype == np.float32 and p.dtype == np.float32
    np.testing.assert_array_equal(a, np.asarray(case["angle"], np.float32))
    np.testing.assert_array_equal(p, np.asarray(case["parameter"], np.float32))


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: c["label"])
def test_decode_matches_oracle(case, orc):
    p = np.asarray(case["parameter"], np.float32)
    ours = decode(p).as_dict()
    ref = orc.decode(p).as_dict()
    assert ours == ref
    # spot-check the reference constructor arithmetic (FP/transform.cc:59-76)
    PI = np.float32(3.14159265359)
    assert ours["n_views"] == int(p[2]) and ours["n_cols"] == int(p[4])
    assert np.float32(ours["dcol"]) == np.float32(np.float32(p[8] * PI) / np.float32(180))
    assert np.float32(ours["dx"]) == np.float32(np.float32(2 * p[7]) / np.float32(int(p[5])))
    assert ours["n_slices"] == case["nimg"]
