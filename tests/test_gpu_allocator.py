"""The device-allocation hook (ct_set_allocator) and its failure paths.

The reference malloc'ed its buffers inside every call and exited the process
when one failed (FP/transform.cu:198-217, checkCudaErrors).  Here every
device allocation of the library goes through one route that a caller can
replace; these tests install a fake allocator (torch tensors handed out by
ctypes callbacks) that counts, and one that fails on a chosen allocation,
and check that:
  - every allocation the library makes goes through the installed allocator
    and is counted by ct_device_alloc_count;
  - a plan whose table allocation fails returns CT_ERR_ALLOC, gives back
    what it had taken, and the next plan on the same context works;
  - an operator whose scratch allocation fails returns CT_ERR_ALLOC, leaves
    its output untouched, and the next call works.
Failures are made on the host (the callback returns NULL); nothing faults."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from fanbeamctrecon_tensorflowop_gb300 import _lib
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
import geometries as G

CT_ERR_ALLOC = 5


class FakeAllocator:
    """Device memory from torch's caching allocator, handed out through the
    ct_allocator callbacks; fail_at = k makes the k-th allocation (1-based)
    return NULL."""

    def __init__(self, device, fail_at: int | None = None):
        self.device = device
        self.fail_at = fail_at
        self.live: dict[int, torch.Tensor] = {}
        self.calls = 0
        self.freed = 0
        self.streams: list[int | None] = []
        self._alloc = _lib.ALLOC_FN(self._on_alloc)
        self._free = _lib.FREE_FN(self._on_free)
        self.struct = _lib.CtAllocator(None, self._alloc, self._free)

    def _on_alloc(self, ctx, nbytes, stream):
        self.calls += 1
        self.streams.append(stream)
        if self.fail_at is not None and self.calls == self.fail_at:
            return None
        t = torch.empty(max(1, int(nbytes)), dtype=torch.uint8, device=self.device)
        self.live[t.data_ptr()] = t
        return t.data_ptr()

    def _on_free(self, ctx, ptr, stream):
        self.freed += 1
        self.live.pop(ptr)


@pytest.fixture
def lib():
    lib = _lib.load()
    yield lib
    assert lib.ct_set_allocator(None) == 0  # back to the CUDA runtime


def test_cpu_setter_validates(lib):
    a = _lib.CtAllocator(None, _lib.ALLOC_FN(), _lib.FREE_FN())
    assert lib.ct_set_allocator(ctypes.byref(a)) == 2  # CT_ERR_NULL_POINTER


@pytest.mark.gpu
def test_every_allocation_goes_through_the_hook(cuda, lib):
    fake = FakeAllocator(cuda)
    assert lib.ct_set_allocator(ctypes.byref(fake.struct)) == 0
    n0 = lib.ct_device_alloc_count()
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)
    tables = fake.calls
    assert tables >= 5 and all(s is None for s in fake.streams)
    x = torch.rand((3, *plan.image_shape), device=cuda)
    out = torch.empty((3, *plan.sino_shape), device=cuda)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    assert lib.ct_fp_fan(plan._h, x.data_ptr(), out.data_ptr(), 3, None, 0, stream) == 0
    torch.cuda.synchronize()
    assert fake.calls == tables + 1            # the call's scratch
    assert (fake.streams[-1] or 0) == stream   # on the call's stream (0: the legacy default)
    assert fake.freed == 1 and len(fake.live) == tables
    assert lib.ct_device_alloc_count() - n0 == fake.calls
    # same result as with caller-provided scratch
    ref = plan.fp(x)
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    plan.close()                               # tables go back to the fake
    assert not fake.live and fake.freed == fake.calls


@pytest.mark.gpu
@pytest.mark.parametrize("fail_at", [1, 3, 6])
def test_plan_table_allocation_failure(cuda, lib, fail_at):
    fake = FakeAllocator(cuda, fail_at=fail_at)
    assert lib.ct_set_allocator(ctypes.byref(fake.struct)) == 0
    p, a = G.small()
    with pytest.raises(_lib.CtError) as ei:
        FanPlan(p, a, device=cuda)
    assert ei.value.status == CT_ERR_ALLOC
    assert b"plan table" in lib.ct_last_error()
    assert not fake.live                       # what it had taken was given back
    assert fake.freed == fail_at - 1
    assert lib.ct_set_allocator(None) == 0
    plan = FanPlan(p, a, device=cuda)          # the context is fine
    x = torch.rand((1, *plan.image_shape), device=cuda)
    assert torch.isfinite(plan.fp(x)).all()


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["ct_fp_fan", "ct_fbp_fan", "ct_fp_fan_adjoint"])
def test_workspace_allocation_failure(cuda, lib, op):
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)          # tables from the CUDA runtime
    fake = FakeAllocator(cuda, fail_at=1)
    img_in = op == "ct_fp_fan"
    x = torch.rand((4, *(plan.image_shape if img_in else plan.sino_shape)), device=cuda)
    out = torch.full((4, *(plan.sino_shape if img_in else plan.image_shape)), float("nan"),
                     device=cuda)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    fn = getattr(lib, op)
    assert lib.ct_set_allocator(ctypes.byref(fake.struct)) == 0
    assert fn(plan._h, x.data_ptr(), out.data_ptr(), 4, None, 0, stream) == CT_ERR_ALLOC
    torch.cuda.synchronize()
    assert torch.isnan(out).all()              # nothing was enqueued
    assert fake.calls == 1 and not fake.live
    assert lib.ct_set_allocator(None) == 0
    assert fn(plan._h, x.data_ptr(), out.data_ptr(), 4, None, 0, stream) == 0
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    plan.close()
