"""Drop-in for the reference's ``utils.py`` and its ``tf.load_op_library`` modules.

The reference's drivers call

    FP_module.fp_fan_curve(volume=img, angle=..., parameter=..., vol_shape=..., proj_shape=...)
    BP_module.bp_fan_curve(projection=sino, ...)
    FBP_module.fbp_fan_curve(projection=sino, ...)
    FBP_module.BackProjection(projection=sino, ...)        # FDK/FDK_test_training.py:111

(utils.py:10-12,25,35,45) and the convenience wrappers ForwardProjection /
BackProjection / FilteredBackProjection (utils.py:15-46).  This module keeps
those names, keyword arguments and shapes.  Inputs may be numpy arrays, CPU
tensors or CUDA tensors; the result has the kind of the input (numpy in ->
numpy out, a CUDA tensor stays on its device).  Host inputs are copied to
the current CUDA device; host results land in page-locked memory.  CUDA tensors that
require grad are differentiated through the library's exact adjoints.

Memory layout follows the reference kernels, not the TF shape attribute: an
image is read as [nimg][ny][nx] with x fastest and a sinogram as
[nimg][nview][ncol] (BP/transform.cu:87, FP/transform.cu:250); the result is
returned with the ``vol_shape`` / ``proj_shape`` the caller gave.
"""
from __future__ import annotations

import os
from types import SimpleNamespace

import numpy as np
import torch

from . import _lib, autograd
from .config import config
from .geometry import angle, param_set
from .ops import get_plan

__all__ = [
    "ForwardProjection", "BackProjection", "FilteredBackProjection", "angle", "param_set",
    "fp_fan_curve", "bp_fan_curve", "fbp_fan_curve", "back_projection", "load_op_library",
    "FP_module", "BP_module", "FBP_module", "FDK_module", "config",
]

def _prod(shape) -> int:
    n = 1
    for s in shape:
        n *= int(s)
    return n


def _to_device(x, tail: tuple[int, int], device):
    """(cuda tensor [B, *tail], kind) from numpy / CPU tensor / CUDA tensor."""
    per = _prod(tail)
    if isinstance(x, torch.Tensor) and x.is_cuda:
        t = x if x.dtype == torch.float32 else x.float()
        kind = "cuda"
    else:
        if isinstance(x, torch.Tensor):
            t = x.detach().to(torch.float32)
            kind = "cpu"
        else:
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float32)))
            kind = "numpy"
        t = t.contiguous().to(device)
    if t.numel() % per:
        raise ValueError(f"input of {t.numel()} elements is not a whole number of "
                         f"{tail} slices")
    return t.contiguous().reshape(-1, *tail), kind


def _from_device(t: torch.Tensor, kind: str, shape):
    if kind == "cuda":
        return t.reshape(shape)
    # page-locked destination from torch's caching host allocator; the
    # returned array views it directly (no second host copy)
    host = torch.empty(t.numel(), dtype=torch.float32, pin_memory=True)
    host.copy_(t.reshape(-1), non_blocking=True)
    torch.cuda.current_stream(t.device).synchronize()
    host = host.reshape(shape)
    return host.numpy() if kind == "numpy" else host


def _device_for(x):
    if isinstance(x, torch.Tensor) and x.is_cuda:
        return x.device
    if not torch.cuda.is_available():
        raise RuntimeError("the CT operators run on a CUDA device; none is available")
    return torch.device("cuda", torch.cuda.current_device())


def _run(op: str, x, angle_arr, parameter, vol_shape, proj_shape, window: int):
    device = _device_for(x)
    plan = get_plan(parameter, angle_arr, device=device, window=window)
    if op == "fp":
        xin, kind = _to_device(x, plan.image_shape, device)
        out_shape = tuple(int(s) for s in proj_shape)
    else:
        xin, kind = _to_device(x, plan.sino_shape, device)
        out_shape = tuple(int(s) for s in vol_shape)
    grad = kind == "cuda" and torch.is_grad_enabled() and x.requires_grad
    if op == "fp" and kind != "cuda":
        # host caller: the projector writes the sinogram into page-locked host
        # memory as it runs
        host = plan.fp_to_host(xin)
        if _prod(out_shape) != host.numel():
            raise ValueError(f"output shape {out_shape} does not hold {host.numel()} elements "
                             f"({host.shape[0]} slices)")
        torch.cuda.current_stream(device).synchronize()
        host = host.reshape(out_shape)
        return host.numpy() if kind == "numpy" else host
    if op == "fp":
        y = autograd.forward_project(xin, plan) if grad else plan.fp(xin)
    elif op == "bp":
        y = autograd.back_project(xin, plan) if grad else plan.bp(xin)
    elif op == "fbp":
        y = autograd.filtered_back_project(xin, plan) if grad else plan.fbp(xin)
    elif op == "fdk":
        y = autograd.fdk_back_project(xin, plan) if grad else plan.fdk_bp(xin)
    else:  # pragma: no cover
        raise ValueError(op)
    if _prod(out_shape) != y.numel():
        raise ValueError(f"output shape {out_shape} does not hold {y.numel()} elements "
                         f"({y.shape[0]} slices)")
    return _from_device(y, kind, out_shape)


# ---- the op-library functions (keyword names of the TF ops) ------------------

def fp_fan_curve(volume, angle, parameter, vol_shape, proj_shape, name=None):
    """FPFanCurve (FP/transform.cc:17-37)."""
    return _run("fp", volume, angle, parameter, vol_shape, proj_shape, _lib.WINDOW_RAMLAK)


def bp_fan_curve(projection, angle, parameter, vol_shape, proj_shape, name=None):
    """BPFanCurve (BP/transform.cc:17-36)."""
    return _run("bp", projection, angle, parameter, vol_shape, proj_shape, _lib.WINDOW_RAMLAK)


def fbp_fan_curve(projection, angle, parameter, vol_shape, proj_shape, name=None,
                  window: int = _lib.WINDOW_RAMLAK):
    """FBPFanCurve (FBP/transform.cc:17-36); the reference filter is Ram-Lak."""
    return _run("fbp", projection, angle, parameter, vol_shape, proj_shape, window)


def back_projection(projection, angle, parameter, vol_shape, proj_shape, name=None):
    """The FDK library's BackProjection op (FDK/FBP.cc:16-35)."""
    return _run("fdk", projection, angle, parameter, vol_shape, proj_shape, _lib.WINDOW_RAMLAK)


FP_module = SimpleNamespace(fp_fan_curve=fp_fan_curve, FPFanCurve=fp_fan_curve)
BP_module = SimpleNamespace(bp_fan_curve=bp_fan_curve, BPFanCurve=bp_fan_curve)
FBP_module = SimpleNamespace(fbp_fan_curve=fbp_fan_curve, FBPFanCurve=fbp_fan_curve)
FDK_module = SimpleNamespace(BackProjection=back_projection, back_projection=back_projection)

_MODULES = {"FP.so": FP_module, "BP.so": BP_module, "FBP.so": FBP_module,
            "FBP_op.so": FDK_module}


def load_op_library(path: str):
    """Stands in for tf.load_op_library on the reference's library names
    (utils.py:10-12: ./FP/FP.so, ./BP/BP.so, ./FBP/FBP.so;
    FDK/FDK_test_training.py:7: ./FBP_op.so)."""
    base = os.path.basename(path)
    if base not in _MODULES:
        raise ValueError(f"unknown op library {path!r}; expected one of {sorted(_MODULES)}")
    return _MODULES[base]


# ---- the convenience wrappers of utils.py:15-46 -------------------------------

def _geometry(nimg: int):
    nview = config.ProjectionsPerRotation
    ncol = config.DetectorColumnNumber
    nx, ny = config.NX, config.NY
    return (angle(nview, config.StartAngle), param_set(nimg),
            [nimg, nx, ny], [nimg, nview, ncol])


def ForwardProjection(img, nimg=1):
    """utils.py:15-26: FP with the geometry of ``config``."""
    ang, par, vs, ps = _geometry(nimg)
    return fp_fan_curve(volume=img, angle=ang, parameter=par, vol_shape=vs, proj_shape=ps)


def BackProjection(sino, nimg=1):
    """utils.py:28-36: unweighted BP with the geometry of ``config``."""
    ang, par, vs, ps = _geometry(nimg)
    return bp_fan_curve(projection=sino, angle=ang, parameter=par, vol_shape=vs, proj_shape=ps)


def FilteredBackProjection(sino, nimg=1):
    """utils.py:38-46: Ram-Lak FBP with the geometry of ``config``."""
    ang, par, vs, ps = _geometry(nimg)
    return fbp_fan_curve(projection=sino, angle=ang, parameter=par, vol_shape=vs, proj_shape=ps)
