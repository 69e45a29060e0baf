"""The tensor-core Toeplitz ramp filter (tcgen05, TF32 three-term split)
against the FP64 oracle and the direct FP32 filter.  Tolerance: relative L2
<= 1e-4 as for every operator."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
import geometries as G

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _np(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("geom", ["small", "config0", "config1"])
@pytest.mark.parametrize("window", [_lib.WINDOW_RAMLAK, _lib.WINDOW_SHEPP_LOGAN])
def test_tc_filter_matches_oracle(cuda, orc, geom, window):
    p, a = {"small": G.small, "config0": G.config0, "config1": G.config1}[geom]()
    tc = FanPlan(p, a, device=cuda, window=window, filter_algo=_lib.FILTER_TOEPLITZ_TC)
    direct = FanPlan(p, a, device=cuda, window=window, filter_algo=_lib.FILTER_DIRECT)
    g = orc.decode(p)
    # sinograms of phantoms (strong cancellation in the ramp) and of noise
    img = phantom.ellipse_phantom(g.nx, float(g.dx), seed=1)
    y = orc.fp_fan(g, a, img)
    y = np.concatenate([y, np.random.default_rng(0).uniform(0, 1, y.shape)]).astype(np.float32)
    yt = torch.from_numpy(y).to(cuda)
    got = _np(tc.ramp_filter(yt))
    ref = orc.ramp_filter(g, y, window)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    assert rel_l2(got, _np(direct.ramp_filter(yt))) <= TOL
    assert _lib.load().ct_plan_check(tc._h) == 0


def test_tc_fbp_matches_oracle(cuda, orc):
    p, a = G.config0()
    tc = FanPlan(p, a, device=cuda, filter_algo=_lib.FILTER_TOEPLITZ_TC)
    g = orc.decode(p)
    y = orc.fp_fan(g, a, phantom.ellipse_phantom(g.nx, float(g.dx), seed=2))
    got = _np(tc.fbp(torch.from_numpy(y.astype(np.float32)).to(cuda)))
    ref = orc.fbp_fan(g, a, y)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


def test_tc_filter_partial_tiles(cuda, orc):
    """Rows not a multiple of 128 and columns not a multiple of 224 or 32."""
    p, a = G.small(n=40, views=37, cols=100)
    tc = FanPlan(p, a, device=cuda, filter_algo=_lib.FILTER_TOEPLITZ_TC)
    g = orc.decode(p)
    y = np.random.default_rng(3).standard_normal((3, 37, 100)).astype(np.float32)
    got = _np(tc.ramp_filter(torch.from_numpy(y).to(cuda)))
    assert rel_l2(got, orc.ramp_filter(g, y)) <= TOL


def test_tc_filter_rejects_unsupported_widths(cuda):
    p, a = G.small(cols=98)  # 98 % 4 != 0: TMA rows must be 16-byte multiples
    with pytest.raises(_lib.CtError):
        FanPlan(p, a, device=cuda, filter_algo=_lib.FILTER_TOEPLITZ_TC)


def test_bounded_wait_timeout_is_reported_and_context_survives(cuda, orc):
    """The filter's bounded mbarrier wait, on a barrier nothing completes, gives
    up after its budget and raises the plan's flag; ct_plan_check reports it
    once, and the context keeps working."""
    p, a = G.small(n=40, views=36, cols=64)
    tc = FanPlan(p, a, device=cuda, filter_algo=_lib.FILTER_TOEPLITZ_TC)
    lib = _lib.load()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    assert lib.ct_plan_check(tc._h) == 0
    assert lib.ct_plan_selftest_wait_timeout(tc._h, 20000, stream) == 0  # 20 ms budget
    assert lib.ct_plan_check(tc._h) == 7  # CT_ERR_TIMEOUT
    assert b"gave up" in lib.ct_last_error()
    assert lib.ct_plan_check(tc._h) == 0  # reported once
    assert lib.ct_plan_selftest_wait_timeout(tc._h, 0, stream) == 1
    g = orc.decode(p)
    y = np.random.default_rng(4).uniform(0, 1, (2, 36, 64)).astype(np.float32)
    got = _np(tc.fbp(torch.from_numpy(y).to(cuda)))
    assert rel_l2(got, orc.fbp_fan(g, a, y)) <= TOL
    assert lib.ct_plan_check(tc._h) == 0
