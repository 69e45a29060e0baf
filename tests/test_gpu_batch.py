"""Uneven batches (ct_batch_run): per-item results equal the per-plan
operators, BF16 storage stays within BF16 rounding of the FP32 result, a
captured CUDA graph replays the same results, and bad batches are refused."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom
from fanbeamctrecon_tensorflowop_gb300.batch import UnevenBatch
from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan, FanPlan
import geometries as G

pytestmark = pytest.mark.gpu


def _tol(op):
    return 1e-6


def _np(t):
    torch.cuda.synchronize()
    return t.detach().float().cpu().numpy().astype(np.float64)


def _make(cuda, dtype, ops=("fp", "fbp", "fbp_adjoint", "bp"), n_items=8, scale=4):
    items, ref = [], []
    for k in range(n_items):
        p, a = G.uneven(k, scale=scale)
        plan = FanPlan(p, a, device=cuda)
        op = ops[k % len(ops)]
        g = plan.geom
        img = torch.from_numpy(phantom.ellipse_phantom(g.nx, float(g.dx), seed=k)).to(cuda)
        sino = plan.fp(img)[0]
        x = img if op in ("fp", "fbp_adjoint") else sino
        x = x.to(dtype).contiguous()
        out_shape = plan.sino_shape if op in ("fp", "fbp_adjoint") else plan.image_shape
        y = torch.full(out_shape, float("nan"), device=cuda, dtype=dtype)
        items.append((plan, op, x, y))
        xf = x.float()
        want = {"fp": plan.fp, "bp": plan.bp, "fbp": plan.fbp,
                "fbp_adjoint": plan.fbp_adjoint}[op](xf)[0]
        ref.append(want)
    return items, ref


def test_batch_f32_equals_per_plan_operators(cuda):
    items, ref = _make(cuda, torch.float32)
    UnevenBatch(items).run()
    for (plan, op, x, y), want in zip(items, ref):
        assert rel_l2(_np(y), _np(want)) <= _tol(op), op


def test_batch_bf16_storage(cuda, orc):
    items, ref = _make(cuda, torch.bfloat16)
    UnevenBatch(items).run()
    for (plan, op, x, y), want in zip(items, ref):
        # FP32 arithmetic on the BF16 input: only the output rounding differs
        assert rel_l2(_np(y), _np(want)) <= 8e-3, op
    # errors against the FP64 oracle of the BF16-rounded inputs
    for (plan, op, x, y), _ in zip(items[:4], ref[:4]):
        g = orc.decode(plan.param16)
        xin = _np(x)
        o = {"fp": lambda: orc.fp_fan(g, plan.angles, xin),
             "fbp": lambda: orc.fbp_fan(g, plan.angles, xin),
             "fbp_adjoint": lambda: orc.fbp_fan_adjoint(g, plan.angles, xin),
             "bp": lambda: orc.bp_fan(g, plan.angles, xin)}[op]()[0]
        assert rel_l2(_np(y), o) <= 8e-3, op


def test_batch_graph_replay(cuda):
    items, ref = _make(cuda, torch.float32, n_items=6)
    ub = UnevenBatch(items)
    ub.capture()
    for _, _, _, y in items:
        y.fill_(float("nan"))
    ub.replay()
    for (plan, op, x, y), want in zip(items, ref):
        assert rel_l2(_np(y), _np(want)) <= _tol(op), op
    # new inputs, same buffers: the graph recomputes
    for _, op, x, _ in items:
        x.mul_(2.0)
    ub.replay()
    for (plan, op, x, y), want in zip(items, ref):
        assert rel_l2(_np(y), 2.0 * _np(want)) <= _tol(op), op


def test_batch_validation(cuda):
    items, _ = _make(cuda, torch.float32, n_items=2)
    lib = _lib.load()
    arr = (_lib.CtBatchItem * 65)()
    n = __import__("ctypes").c_size_t()
    assert lib.ct_batch_workspace_size(arr, 65, n) == 1
    bad = (_lib.CtBatchItem * 1)()
    bad[0].plan = items[0][0]._h.value
    bad[0].op = 99
    bad[0].d_in, bad[0].d_out = items[0][2].data_ptr(), items[0][3].data_ptr()
    assert lib.ct_batch_workspace_size(bad, 1, n) == 1
    bad[0].op = _lib.OP_FP
    bad[0].d_in = None
    assert lib.ct_batch_workspace_size(bad, 1, n) == 2
    p, a, nr, nz = G.cone_small()
    cone = ConePlan(p, a, nr, nz, device=cuda)
    with pytest.raises(TypeError):
        UnevenBatch([(cone, "fp", torch.zeros(nz, 32, 32, device=cuda),
                      torch.zeros(48, 64, device=cuda))])
    with pytest.raises(TypeError):
        plan, op, x, y = items[0]
        UnevenBatch([(plan, op, x.to(torch.bfloat16), y)])


CONFIGS = [
    dict(fp_blocks_per_sm=1, fp_dynamic=1, bp_blocks_per_sm=2, bp_dynamic=1, bp_tile_rows=16),
    dict(fp_blocks_per_sm=8, fp_dynamic=0, bp_blocks_per_sm=12, bp_dynamic=0, bp_tile_rows=16),
    dict(fp_blocks_per_sm=2, fp_dynamic=1, bp_blocks_per_sm=6, bp_dynamic=1, bp_tile_rows=32),
]


def test_every_launch_shape_gives_the_same_result(cuda):
    """Each unit's arithmetic is independent of which warp or block takes it, so
    every launch shape reproduces the default's FP and BP outputs bit for bit."""
    items, _ = _make(cuda, torch.float32, ops=("fp", "fbp", "bp"), n_items=6)
    ub = UnevenBatch(items)
    ub.set_config(None)
    ub.run()
    base = [y.clone() for *_, y in items]
    for cfg in CONFIGS:
        ub.set_config(cfg)
        assert ub.config == ({**cfg}, True)
        for *_, y in items:
            y.fill_(float("nan"))
        ub.run()
        for (plan, op, x, y), want in zip(items, base):
            assert torch.equal(y, want), (cfg, op)
    ub.set_config(None)
    assert ub.config[1] is False


def test_tune_then_capture(cuda):
    items, ref = _make(cuda, torch.bfloat16, n_items=8)
    ub = UnevenBatch(items)
    cfg = ub.tune(reps=1)
    assert ub.config == (cfg, True)
    assert 1 <= cfg["fp_blocks_per_sm"] <= 8 and 2 <= cfg["bp_blocks_per_sm"] <= 12
    assert cfg["bp_tile_rows"] in (16, 32)
    ub.capture()
    for *_, y in items:
        y.fill_(float("nan"))
    ub.replay()
    for (plan, op, x, y), want in zip(items, ref):
        assert rel_l2(_np(y), _np(want)) <= 8e-3, op
    ub.set_config(None)


def test_config_validation(cuda):
    items, _ = _make(cuda, torch.float32, n_items=2)
    ub = UnevenBatch(items)
    for bad in (dict(fp_blocks_per_sm=0), dict(bp_tile_rows=24), dict(fp_dynamic=2),
                dict(bp_blocks_per_sm=17)):
        cfg = {**ub.config[0], **bad}
        with pytest.raises(RuntimeError):
            ub.set_config(cfg)
    assert ub.config[1] is False


def _make_groups(cuda, dtype):
    """Three shared plans with three items of every operator each (slice
    groups of three), plus two items whose plans appear once (the persistent
    launches)."""
    plans = [FanPlan(*G.uneven(k, scale=4), device=cuda) for k in range(3)]
    singles = [FanPlan(*G.uneven(k, scale=4), device=cuda) for k in (3, 4)]
    items, ref = [], []
    ops = ("fp", "bp", "fbp", "fbp_adjoint")
    seed = 0
    for plan in plans:
        for op in ops:
            for _ in range(3):
                seed += 1
                items.append(_item(cuda, plan, op, dtype, seed, ref))
    items.append(_item(cuda, singles[0], "fp", dtype, 99, ref))
    items.append(_item(cuda, singles[1], "fbp", dtype, 98, ref))
    return items, ref


def _item(cuda, plan, op, dtype, seed, ref):
    g = plan.geom
    img = torch.from_numpy(phantom.ellipse_phantom(g.nx, float(g.dx), seed=seed)).to(cuda)
    x = img if op in ("fp", "fbp_adjoint") else plan.fp(img)[0]
    x = x.to(dtype).contiguous()
    out_shape = plan.sino_shape if op in ("fp", "fbp_adjoint") else plan.image_shape
    y = torch.full(out_shape, float("nan"), device=cuda, dtype=dtype)
    ref.append({"fp": plan.fp, "bp": plan.bp, "fbp": plan.fbp,
                "fbp_adjoint": plan.fbp_adjoint}[op](x.float())[0])
    return plan, op, x, y


def test_batch_slice_groups_equal_per_plan_operators(cuda):
    items, ref = _make_groups(cuda, torch.float32)
    ub = UnevenBatch(items)
    ub.run()
    for (plan, op, x, y), want in zip(items, ref):
        if op == "fbp_adjoint":
            assert rel_l2(_np(y), _np(want)) <= _tol(op), op
        else:  # the same kernels on the same slices: identical bits
            np.testing.assert_array_equal(_np(y), _np(want), err_msg=op)
    # replayed from a graph, and after tuning (only the two persistent items
    # have launch shapes), the results stay the same
    ub.tune(reps=1)
    ub.capture()
    for _, _, _, y in items:
        y.fill_(float("nan"))
    ub.replay()
    for (plan, op, x, y), want in zip(items, ref):
        assert rel_l2(_np(y), _np(want)) <= _tol(op), op


def test_batch_slice_groups_bf16(cuda):
    items, ref = _make_groups(cuda, torch.bfloat16)
    UnevenBatch(items).run()
    for (plan, op, x, y), want in zip(items, ref):
        # FP32 arithmetic on the BF16 input, the result rounded to BF16 once
        if op != "fbp_adjoint":
            np.testing.assert_array_equal(_np(y), _np(want.to(torch.bfloat16)), err_msg=op)
        assert rel_l2(_np(y), _np(want)) <= 8e-3, op


def test_batch_all_grouped_tunes(cuda):
    plan = FanPlan(*G.uneven(1, scale=4), device=cuda)
    ref = []
    items = [_item(cuda, plan, "fp", torch.float32, s, ref) for s in range(4)]
    ub = UnevenBatch(items)
    cfg = ub.tune(reps=1)  # nothing persistent to time: the defaults come back
    assert cfg["fp_blocks_per_sm"] > 0
    ub.run()
    for (_, _, _, y), want in zip(items, ref):
        np.testing.assert_array_equal(_np(y), _np(want))


def test_batch_slice_groups_with_preweights(cuda):
    """Slice groups of short-scan (Parker) and cosine-weighted plans: the
    grouped FBP and FBP adjoint apply the pre-weights as ct_fbp_fan and
    ct_fbp_fan_adjoint do."""
    p, a = G.short_scan(n=96, views=160, cols=256)
    plans = [FanPlan(p, a, device=cuda, short_scan=True),
             FanPlan(p, a, device=cuda, cosine_weight=True)]
    items, ref = [], []
    seed = 100
    for plan in plans:
        for op in ("fbp", "fbp_adjoint"):
            for _ in range(3):
                seed += 1
                items.append(_item(cuda, plan, op, torch.float32, seed, ref))
    UnevenBatch(items).run()
    for (plan, op, x, y), want in zip(items, ref):
        if op == "fbp":
            np.testing.assert_array_equal(_np(y), _np(want), err_msg=op)
        else:
            assert rel_l2(_np(y), _np(want)) <= _tol(op), op
