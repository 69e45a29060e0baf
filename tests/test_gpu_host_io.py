"""Host callers of the forward projector: the sinogram is written by the
kernel straight into page-locked host memory (ct_host_mapped checks that the
buffer is mapped for the device before any kernel sees it).  The result must
equal the device-resident projection bit for bit."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom, utils
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
import geometries as G

pytestmark = pytest.mark.gpu

CT_ERR_INVALID_ARGUMENT, CT_ERR_NULL_POINTER = 1, 2


def test_host_mapped_query(cuda, ctlib):
    pinned = torch.empty(1024, dtype=torch.float32, pin_memory=True)
    dptr = ctypes.c_void_p()
    assert ctlib.ct_host_mapped(ctypes.c_void_p(pinned.data_ptr()), ctypes.byref(dptr)) == 0
    assert dptr.value  # the device's address of the buffer
    pageable = np.zeros(1024, np.float32)
    assert ctlib.ct_host_mapped(ctypes.c_void_p(pageable.ctypes.data),
                                ctypes.byref(dptr)) == CT_ERR_INVALID_ARGUMENT
    dev = torch.empty(16, device=cuda)
    assert ctlib.ct_host_mapped(ctypes.c_void_p(dev.data_ptr()),
                                ctypes.byref(dptr)) == CT_ERR_INVALID_ARGUMENT
    assert ctlib.ct_host_mapped(None, ctypes.byref(dptr)) == CT_ERR_NULL_POINTER
    torch.cuda.synchronize()  # the context is untouched


@pytest.mark.parametrize("geom", ["small", "config1"])
def test_fp_into_host_memory_equals_device_result(cuda, geom):
    p, a = G.small() if geom == "small" else G.config1()
    plan = FanPlan(p, a, device=cuda)
    n = plan.image_shape[0]
    B = 3 if geom == "small" else 17
    imgs = phantom.phantom_batch(B, n, float(plan.geom.dx), seed0=11)
    dev = plan.fp(torch.from_numpy(imgs).to(cuda)).cpu().numpy()
    host = plan.fp_to_host(torch.from_numpy(imgs).to(cuda))
    torch.cuda.synchronize()
    assert host.is_pinned() and host.device.type == "cpu"
    np.testing.assert_array_equal(host.numpy(), dev)
    out = utils.fp_fan_curve(volume=imgs, angle=a, parameter=p, vol_shape=list(imgs.shape),
                             proj_shape=[B, *plan.sino_shape])
    assert isinstance(out, np.ndarray)
    np.testing.assert_array_equal(out, dev)
    out_t = utils.fp_fan_curve(volume=torch.from_numpy(imgs), angle=a, parameter=p,
                               vol_shape=list(imgs.shape), proj_shape=[B, *plan.sino_shape])
    assert isinstance(out_t, torch.Tensor) and out_t.device.type == "cpu"
    np.testing.assert_array_equal(out_t.numpy(), dev)
