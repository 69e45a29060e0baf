"""The debug build (-DCT_DEBUG): kernels that test every gather index
against the array they read and record a failure instead of reading.

In-range data must leave the flags clear (ct_plan_check returns CT_OK) and
give the release library's results; the release library must carry no
checks (ct_build_flags() == 0).  No test plants an out-of-range index on the
GPU: a failing check would only skip the access and set a flag, but the
checks are exercised here on valid work alone."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib
from fanbeamctrecon_tensorflowop_gb300.geometry import decode
from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan, FanPlan
import geometries as G


def test_release_build_has_no_index_checks(ctlib):
    assert ctlib.ct_build_flags() == 0


def _plan(lib, p, a, n_rows=None, nz=None):
    g = decode(p)
    a = np.ascontiguousarray(a, np.float32)
    h = ctypes.c_void_p()
    fp = ctypes.POINTER(ctypes.c_float)
    if n_rows is None:
        st = lib.ct_plan_create(ctypes.byref(g), a.ctypes.data_as(fp), len(a), None,
                                ctypes.byref(h))
    else:
        st = lib.ct_plan_create_cone(ctypes.byref(g), n_rows, nz, a.ctypes.data_as(fp), len(a),
                                     None, ctypes.byref(h))
    assert st == 0, lib.ct_last_error()
    return h


def _run(lib, h, name, op, x, out_shape, dev):
    out = torch.full(out_shape, float("nan"), device=dev)
    s = torch.cuda.current_stream(dev).cuda_stream
    fn = getattr(lib, name)
    if op is None:
        st = fn(h, x.data_ptr(), out.data_ptr(), x.shape[0], s)
    else:
        n = ctypes.c_size_t()
        assert lib.ct_workspace_size(h, op, x.shape[0], ctypes.byref(n)) == 0
        w = torch.empty(max(1, n.value), dtype=torch.uint8, device=dev)
        st = fn(h, x.data_ptr(), out.data_ptr(), x.shape[0], w.data_ptr(), n.value, s)
    assert st == 0, (name, lib.ct_last_error())
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("geom", ["small", "odd"])
def test_debug_build_fan_operators(cuda, geom):
    dlib = _lib.load_debug()
    assert dlib.ct_build_flags() & _lib.BUILD_INDEX_CHECKS
    p, a = G.small() if geom == "small" else G.small(n=45, views=37, cols=61, pixel=3.9)
    ref = FanPlan(p, a, device=cuda)
    h = _plan(dlib, p, a)
    gen = torch.Generator(device=cuda).manual_seed(1)
    for B in (1, 6, 20):
        img = torch.rand((B, *ref.image_shape), device=cuda, generator=gen)
        sino = torch.rand((B, *ref.sino_shape), device=cuda, generator=gen)
        cases = [("ct_fp_fan", _lib.OP_FP, img, ref.sino_shape, ref.fp),
                 ("ct_fp_fan_adjoint", _lib.OP_FP_ADJOINT, sino, ref.image_shape, ref.fp_adjoint),
                 ("ct_bp_fan", None, sino, ref.image_shape, ref.bp),
                 ("ct_bp_fan_adjoint", None, img, ref.sino_shape, ref.bp_adjoint),
                 ("ct_fbp_fan", _lib.OP_FBP, sino, ref.image_shape, ref.fbp),
                 ("ct_fbp_fan_adjoint", _lib.OP_FBP_ADJOINT, img, ref.sino_shape,
                  ref.fbp_adjoint)]
        for name, op, x, tail, rfn in cases:
            got = _run(dlib, h, name, op, x, (B, *tail), cuda)
            want = rfn(x)
            torch.cuda.synchronize()
            assert torch.isfinite(got).all(), name
            assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) <= 1e-6, (name, B)
        assert dlib.ct_plan_check(h) == 0, dlib.ct_last_error()
    assert dlib.ct_plan_destroy(h) == 0


@pytest.mark.gpu
def test_debug_build_cone_operators(cuda):
    dlib = _lib.load_debug()
    p, a, nr, nz = G.cone_small()
    ref = ConePlan(p, a, nr, nz, device=cuda)
    h = _plan(dlib, p, a, nr, nz)
    gen = torch.Generator(device=cuda).manual_seed(2)
    vol = torch.rand((2, *ref.volume_shape), device=cuda, generator=gen)
    proj = torch.rand((2, *ref.proj_shape), device=cuda, generator=gen)
    for name, op, x, tail, rfn in (
            ("ct_fp_cone", _lib.OP_FP_CONE, vol, ref.proj_shape, ref.fp_cone),
            ("ct_fdk_cone", _lib.OP_FDK_CONE, proj, ref.volume_shape, ref.fdk),
            ("ct_fdk_cone_adjoint", _lib.OP_FDK_CONE_ADJOINT, vol, ref.proj_shape,
             ref.fdk_adjoint),
            ("ct_cone_bp", None, proj, ref.volume_shape, ref.cone_bp)):
        got = _run(dlib, h, name, op, x, (2, *tail), cuda)
        want = rfn(x)
        torch.cuda.synchronize()
        assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) <= 1e-6, name
    assert dlib.ct_plan_check(h) == 0, dlib.ct_last_error()
    assert dlib.ct_plan_destroy(h) == 0
