"""ct_fbp_fan_static_scratch: filtered backprojection for callers that cannot
allocate device memory (framework plugins handed only their input/output
buffers, real-time pipelines that forbid allocation after start-up).  It keeps
the filtered sinogram in a fixed array inside the library's device code.

Checked through the C ABI against ct_fbp_fan (same tolerance as the other
parity tests), on two calls in a row with different inputs, so a stale or
shared scratch array would show; plus the capacity check, a tensor-core plan
of the widest detector the filter takes, and that the calls make no device
allocation (the library's allocation counter) and, after the first call on a
device (its set-up), take no device memory.  This file sorts last so that a run stopping at
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


def test_static_scratch_calls_allocate_nothing(cuda):
    """Every device allocation of the library goes through one counted route
    (ct_device_alloc_count); the static-scratch calls leave the count, and
    the device's free memory, unchanged."""
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)
    lib = _lib.load()
    sino = torch.rand((2, *plan.sino_shape), device=cuda)
    out = torch.empty((2, *plan.image_shape), device=cuda)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    assert lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), 2, stream) == 0
    torch.cuda.synchronize()
    n0 = lib.ct_device_alloc_count()
    free_before, _ = torch.cuda.mem_get_info(cuda)
    for _ in range(3):
        assert lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), 2,
                                             stream) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info(cuda)
    assert lib.ct_device_alloc_count() == n0
    assert free_after == free_before
    # the counter does see the allocating entry point's scratch
    st = lib.ct_fbp_fan(plan._h, sino.data_ptr(), out.data_ptr(), 2, None, 0, stream)
    assert st == 0
    torch.cuda.synchronize()
    assert lib.ct_device_alloc_count() == n0 + 1


_FRESH = r"""
import json, sys
import torch
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
dev = torch.device("cuda", 0)
torch.cuda.init(); torch.zeros(1, device=dev); torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info(dev)[0]
from fanbeamctrecon_tensorflowop_gb300 import _lib
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
import geometries as G
lib = _lib.load()
p, a = G.small()
plan = FanPlan(p, a, device=dev)
sino = torch.rand((2, *plan.sino_shape), device=dev)
out = torch.empty((2, *plan.image_shape), device=dev)
torch.cuda.synchronize()
s = torch.cuda.current_stream(dev).cuda_stream
free1 = torch.cuda.mem_get_info(dev)[0]
n1 = lib.ct_device_alloc_count()
r = [lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), 2, s)]
torch.cuda.synchronize()
free2 = torch.cuda.mem_get_info(dev)[0]
n2 = lib.ct_device_alloc_count()
for _ in range(3):
    r.append(lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), 2, s))
torch.cuda.synchronize()
free3 = torch.cuda.mem_get_info(dev)[0]
n3 = lib.ct_device_alloc_count()
print(json.dumps(dict(r=r, free0=free0, free1=free1, free2=free2, free3=free3, n1=n1, n2=n2,
                      n3=n3)))
"""


def test_static_scratch_first_call_sets_up_then_nothing(cuda):
    """In a fresh process: once the first call on the device (its set-up) has
    returned, the array's 32 MiB are held; later calls take no memory and no
    allocation.  The library makes no allocation in either."""
    import json
    import os
    import subprocess
    import sys
    from pathlib import Path
    repo = Path(__file__).resolve().parent.parent
    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    res = subprocess.run([sys.executable, "-c", _FRESH, str(repo)], capture_output=True,
                         text=True, timeout=300, env=env)
    assert res.returncode == 0, res.stderr[-3000:]
    d = json.loads(res.stdout.strip().splitlines()[-1])
    assert d["r"] == [0, 0, 0, 0]
    mib = 1 << 20
    assert d["free0"] - d["free2"] >= 32 * mib - 2 * mib, d   # held after the set-up
    assert d["free3"] == d["free2"], d                        # later calls take nothing
    assert d["n2"] == d["n1"] and d["n3"] == d["n2"], d


def test_static_scratch_wide_tensor_core_plan(cuda):
    """A 4000-channel plan filters on the tensor cores; the static-scratch
    entry point takes every width ct_fbp_fan takes."""
    from fanbeamctrecon_tensorflowop_gb300.geometry import angle, fan_param16
    p = fan_param16(sdd=949.0, sid=541.0, n_views=48, n_cols=4000, n=64, pixel_mm=2.8,
                    dcol_rad=0.15 / 949.0)
    plan = FanPlan(p, angle(48, 0.0), device=cuda, filter_algo=_lib.FILTER_TOEPLITZ_TC)
    lib = _lib.load()
    gen = torch.Generator(device=cuda).manual_seed(3)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    for call in range(2):
        sino = torch.rand((2, *plan.sino_shape), device=cuda, generator=gen)
        ref = plan.fbp(sino)
        out = torch.full((2, *plan.image_shape), float("nan"), device=cuda)
        st = lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), out.data_ptr(), 2, stream)
        assert st == 0, lib.ct_last_error()
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) <= TOL, call


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
