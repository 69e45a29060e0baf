"""ct_fbp_fan_static_scratch: filtered backprojection for callers that cannot
allocate device memory (framework plugins handed only their input/output
buffers, real-time pipelines that forbid allocation after start-up).  It keeps
the filtered sinogram in a fixed array inside the library's device code.

Checked through the C ABI against ct_fbp_fan (same tolerance as the other
parity tests), on two calls in a row with different inputs, so a stale or
shared scratch array would show; plus the capacity check and that repeated
calls take no device memory.  This file sorts last so that a run stopping at
the first failure has already run every other test."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
import geometries as G

pytestmark = pytest.mark.gpu

TOL = 1e-4  # relative L2, as in test_gpu_parity.py


@pytest.mark.parametrize("B", [3, 6])
def test_static_scratch_fbp_matches_fbp(cuda, B):
    """3 slices: one per thread; 6: four per thread with a ragged group, read by
    gathers here and from tap images by ct_fbp_fan (the same values)."""
    p, a = G.config0()  # 256^2, 720 views x 512 channels
    plan = FanPlan(p, a, device=cuda)
    lib = _lib.load()
    gen = torch.Generator(device=cuda).manual_seed(0)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    outs = []
    for call in range(2):
        sino = torch.rand((B, *plan.sino_shape), device=cuda, generator=gen)
        ref = plan.fbp(sino)
        out = torch.full((B, *plan.image_shape), float("nan"), device=cuda)
        st = lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), B, stream)
        assert st == 0, lib.ct_last_error()
        torch.cuda.synchronize()
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, want) <= TOL, (call, rel_l2(got, want))
        outs.append(out)
    assert not torch.equal(outs[0], outs[1])


def test_static_scratch_repeats_take_no_device_memory(cuda):
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)
    lib = _lib.load()
    sino = torch.rand((2, *plan.sino_shape), device=cuda)
    out = torch.empty((2, *plan.image_shape), device=cuda)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    assert lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), 2, stream) == 0
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info(cuda)
    for _ in range(3):
        assert lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), 2,
                                             stream) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info(cuda)
    assert free_after >= free_before


def test_static_scratch_rejects_batches_beyond_capacity(cuda):
    p, a = G.config1()  # 984 x 888 floats per slice
    plan = FanPlan(p, a, device=cuda)
    lib = _lib.load()
    per_slice = plan.geom.n_views * plan.geom.n_cols
    fits = _lib.FBP_STATIC_SCRATCH_FLOATS // per_slice
    assert fits == 9
    dummy_in = torch.zeros(1, device=cuda)
    dummy_out = torch.zeros(1, device=cuda)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    st = lib.ct_fbp_fan_static_scratch(plan._h, dummy_in.data_ptr(), dummy_out.data_ptr(),
                                       fits + 1, stream)
    assert st == 3  # CT_ERR_WORKSPACE
    assert b"exceeds the static scratch" in lib.ct_last_error()
    assert lib.ct_fbp_fan_static_scratch(plan._h, None, None, 0, stream) == 0
