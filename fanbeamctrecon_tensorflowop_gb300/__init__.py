"""GB300-native (sm_103a) fan-beam CT operators of FanBeamCTRecon_TensorflowOp.

The compute path is libctgb.so (hand-written CUDA kernels behind the C ABI in
include/ctgb.h); this package binds it to PyTorch and mirrors the reference's
Python interface (``utils``, ``config``).
"""
from . import _lib
from .geometry import angle, decode, fan_param16, param_set
from .ops import ConePlan, FanPlan, clear_plan_cache, get_plan
from .autograd import (back_project, fdk_back_project, fdk_cone, filtered_back_project,
                       forward_project, forward_project_adjoint)

__all__ = [
    "FanPlan", "ConePlan", "fdk_cone", "get_plan", "clear_plan_cache", "angle", "param_set", "decode", "fan_param16",
    "forward_project", "forward_project_adjoint", "back_project", "filtered_back_project",
    "fdk_back_project",
]


def load_library():
    """Loads (building in-tree if needed) libctgb.so and returns the ctypes handle."""
    return _lib.load()
