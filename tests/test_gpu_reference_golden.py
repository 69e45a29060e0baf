"""The CUDA operators against the executed reference's golden vectors, and the
texture-unit rule against this GPU's own texture unit.

The reference interpolates through the texture unit (8-bit weights); the
kernels interpolate with exact fp32 weights.  Their distance from the
reference is therefore bounded by the exact-weight tolerances of
refgold.EXACT_TOL (FP 5e-5, BP 2e-5, FBP/FDK 3e-4 relative L2), the same
bounds the exact-weight FP64 oracle meets; each error is printed."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
from refgold import CASES, EXACT_TOL, gold, reference_view

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


@pytest.mark.parametrize("case", CASES)
def test_cuda_ops_match_executed_reference(cuda, case):
    p, a = gold(case, "parameter"), gold(case, "angle")
    plan = FanPlan(p, a, device=cuda)
    fp_in = _t(gold(case, "fp"), cuda)
    got = {"fp": plan.fp(_t(gold(case, "image"), cuda)), "bp": plan.bp(fp_in),
           "fbp": plan.fbp(fp_in), "fdk": plan.fdk_bp(fp_in),
           "bp_noise": plan.bp(_t(gold(case, "noise"), cuda))}
    torch.cuda.synchronize()
    errs = {}
    for op, y in got.items():
        errs[op] = rel_l2(reference_view(case, op, y.cpu().numpy()), gold(case, op))
    print(case, {k: f"{v:.2e}" for k, v in errs.items()})
    for op, e in errs.items():
        assert e <= EXACT_TOL[op], f"{case}/{op}: {e:.3e}"


def test_texture_rule_matches_this_gpu(cuda, orc):
    """Fetches through a real texture object with the reference's sampler
    state, against oracle/texture_rule.h."""
    rng = np.random.default_rng(7)
    sweep_x = (0.5 + np.arange(65537) / 65536.0).astype(np.float32)
    unit = np.array([0.0, 1.0], np.float32)
    np.testing.assert_array_equal(orc.texture_probe_fetch(unit, sweep_x),
                                  orc.texture_fetch1d(unit, sweep_x))
    t1 = rng.uniform(-1, 1, 777).astype(np.float32)
    x1 = rng.uniform(-3, 781, 20000).astype(np.float32)
    t2 = rng.uniform(-1, 1, (33, 70)).astype(np.float32)
    x2 = rng.uniform(-2, 73, 20000).astype(np.float32)
    y2 = rng.uniform(-2, 36, 20000).astype(np.float32)
    for hw, rule in ((orc.texture_probe_fetch(t1, x1), orc.texture_fetch1d(t1, x1)),
                     (orc.texture_probe_fetch(t2, x2, y2), orc.texture_fetch2d(t2, x2, y2))):
        exact = float(np.mean(hw == rule))
        worst = float(np.abs(hw.astype(np.float64) - rule).max())
        print(f"texture rule: {exact:.4f} bit-exact, worst {worst:.2e}")
        assert exact >= 0.97 and worst <= 6e-8
