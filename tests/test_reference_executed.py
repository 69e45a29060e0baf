"""The oracle pinned to the reference's own ops.

tests/golden/reference_ops.npz was made by executing the reference's
TensorFlow ops (op wrapper + CUDA source, compiled against host stand-ins;
tests/golden/make_golden_reference_ops.py).  The kernels ran as written, with
the GPU texture unit's linear filter following oracle/texture_rule.h, a rule
measured on GB300 (tests/golden/texture_unit_gb300.npz).

Tolerances (relative L2 against the executed reference):

* the oracle with the texture-unit weights: FP 5e-6, BP 5e-6 (2.6e-5 on
  U[0,1) noise: 5e-5), FBP and FDK 1e-4.  What remains is fp32 rounding of
  the reference's sample coordinates and column indices moving a fetch across
  a 1/256 weight boundary.
* the exact-weight oracle (the discretisation the CUDA kernels implement):
  FP 5e-5, BP 2e-5 (noise 2e-4), FBP and FDK 3e-4: the reference's 8-bit
  texture weights themselves.

Two reference behaviours are reproduced here rather than in the library
(which fixes them): its FDK op reconstructs only the first slice, and its BP
and FBP grids cover floor(N/32)*32 pixels per axis.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2
from refgold import CASES, EXACT_TOL, GOLD, OPS, TEX_TOL, gold, reference_view, shapes


def oracle_outputs(orc, case: str) -> dict:
    p, a = gold(case, "parameter"), gold(case, "angle")
    g = orc.decode(p)
    fp = gold(case, "fp")
    return {"fp": orc.fp_fan(g, a, gold(case, "image")), "bp": orc.bp_fan(g, a, fp),
            "fbp": orc.fbp_fan(g, a, fp), "fdk": orc.fdk_bp(g, a, fp),
            "bp_noise": orc.bp_fan(g, a, gold(case, "noise"))}


@pytest.fixture(scope="module")
def with_texture_rule(orc):
    orc.set_texture_emulation(True)
    try:
        yield {c: oracle_outputs(orc, c) for c in CASES}
    finally:
        orc.set_texture_emulation(False)


@pytest.fixture(scope="module")
def exact(orc):
    orc.set_texture_emulation(False)
    return {c: oracle_outputs(orc, c) for c in CASES}


@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("case", CASES)
def test_oracle_with_texture_rule_matches_executed_reference(with_texture_rule, case, op):
    err = rel_l2(reference_view(case, op, with_texture_rule[case][op]), gold(case, op))
    assert err <= TEX_TOL[op], f"{case}/{op}: {err:.3e}"


@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("case", CASES)
def test_exact_oracle_within_texture_weight_gap(exact, case, op):
    err = rel_l2(reference_view(case, op, exact[case][op]), gold(case, op))
    assert err <= EXACT_TOL[op], f"{case}/{op}: {err:.3e}"


@pytest.mark.parametrize("case", CASES)
def test_reference_quirks_recorded(case):
    nx = int(gold(case, "vol_shape")[1])
    if nx % 32:
        cover = nx // 32 * 32
        assert np.all(gold(case, "bp")[:, cover:, :] == 0)
        assert np.all(gold(case, "bp")[:, :, cover:] == 0)
        assert np.any(gold(case, "fdk")[:, cover:, :] != 0)  # the FDK grid covers N
    if gold(case, "image").shape[0] > 1:
        assert np.all(gold(case, "fdk")[1:] == 0)
        assert np.any(gold(case, "fbp")[1] != 0)
    # the FDK library's one-row op and the FBP op agree (same filter, same 1/L^2 BP)
    k = nx // 32 * 32
    np.testing.assert_allclose(gold(case, "fdk")[0, :k, :k], gold(case, "fbp")[0, :k, :k],
                               rtol=0, atol=1e-6 * np.abs(gold(case, "fbp")).max())


@pytest.mark.parametrize("case", CASES)
def test_shape_functions(case):
    vs = tuple(int(v) for v in gold(case, "vol_shape"))
    ps = tuple(int(v) for v in gold(case, "proj_shape"))
    assert tuple(gold(case, "shape_fp").astype(int)) == ps
    for op in ("bp", "fbp", "fdk"):
        assert tuple(gold(case, f"shape_{op}").astype(int)) == vs


TEX = GOLD / "texture_unit_gb300.npz"


@pytest.mark.skipif(not TEX.exists(), reason="texture fixture not generated")
def test_texture_rule_matches_gb300_fetches(orc):
    t = np.load(TEX)
    sweep = orc.texture_fetch1d(np.array([0.0, 1.0], np.float32), t["sweep_x"])
    np.testing.assert_array_equal(sweep, t["sweep"])  # the weight itself: exact
    o1 = orc.texture_fetch1d(t["t1"], t["x1"])
    o2 = orc.texture_fetch2d(t["t2"], t["x2"], t["y2"])
    for got, hw in ((o1, t["o1"]), (o2, t["o2"])):
        assert np.mean(got == hw) >= 0.97
        assert np.abs(got.astype(np.float64) - hw).max() <= 6e-8


def test_executed_reference_reproduces_golden():
    """Where the reference's sources are present, re-executing it gives the
    committed vectors bit for bit (the cases whose FP runs in seconds)."""
    from oracle import reference
    if not reference.available():
        pytest.skip("the reference's sources are not present here")
    for case in ("small", "n48", "batch2"):
        p, a = gold(case, "parameter"), gold(case, "angle")
        vs, ps = shapes(case)
        np.testing.assert_array_equal(reference.run("fp", p, a, vs, ps, gold(case, "image")),
                                      gold(case, "fp"))
        for op in ("bp", "fbp", "fdk"):
            np.testing.assert_array_equal(reference.run(op, p, a, vs, ps, gold(case, "fp")),
                                          gold(case, op))
