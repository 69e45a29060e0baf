"""ctypes binding of libctgb.so (declared in include/ctgb.h).

The library is the only compute path: if it is missing or fails to load, every
operator raises.  There is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import _build

CT_OK = 0
STATUS_NAMES = {
    0: "CT_OK", 1: "CT_ERR_INVALID_ARGUMENT", 2: "CT_ERR_NULL_POINTER", 3: "CT_ERR_WORKSPACE",
    4: "CT_ERR_CUDA", 5: "CT_ERR_ALLOC", 6: "CT_ERR_UNSUPPORTED", 7: "CT_ERR_TIMEOUT",
    8: "CT_ERR_DEVICE_CHECK",
}
BUILD_INDEX_CHECKS = 1  # ct_build_flags bit

# ct_filter_window / ct_filter_algo / ct_op
WINDOW_RAMLAK = 0
WINDOW_SHEPP_LOGAN = 1
FILTER_AUTO = 0
FILTER_DIRECT = 1
FILTER_TOEPLITZ_TC = 2
(OP_FP, OP_FP_ADJOINT, OP_BP, OP_FBP, OP_FBP_ADJOINT, OP_FDK_BP, OP_BP_ADJOINT, OP_FP_CONE,
 OP_FDK_CONE, OP_FDK_CONE_ADJOINT) = range(10)
FBP_STATIC_SCRATCH_FLOATS = 8 * 1024 * 1024  # CT_FBP_STATIC_SCRATCH_FLOATS


class CtError(RuntimeError):
    """A ct_status other than CT_OK, with the library's message."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        name = STATUS_NAMES.get(status, f"status {status}")
        msg = f"{where}: {name}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class CtFanGeom(ctypes.Structure):
    """Mirror of ct_fan_geom."""

    _fields_ = [
        ("sdd", ctypes.c_float), ("sid", ctypes.c_float), ("n_views", ctypes.c_int32),
        ("full_angle", ctypes.c_float), ("n_cols", ctypes.c_int32), ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32), ("rfov", ctypes.c_float), ("shift", ctypes.c_float),
        ("n_slices", ctypes.c_int32), ("det_bottom", ctypes.c_float), ("drow", ctypes.c_float),
        ("dz", ctypes.c_float), ("d_angle", ctypes.c_float), ("dx", ctypes.c_float),
        ("dy", ctypes.c_float), ("xmin", ctypes.c_float), ("ymin", ctypes.c_float),
        ("dcol", ctypes.c_float), ("left", ctypes.c_float), ("start_angle", ctypes.c_float),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class CtBatchItem(ctypes.Structure):
    """Mirror of ct_batch_item."""

    _fields_ = [("plan", ctypes.c_void_p), ("op", ctypes.c_int32), ("dtype", ctypes.c_int32),
                ("d_in", ctypes.c_void_p), ("d_out", ctypes.c_void_p)]


DTYPE_F32 = 0
DTYPE_BF16 = 1
BATCH_MAX_ITEMS = 64


class CtBatchConfig(ctypes.Structure):
    """Mirror of ct_batch_config."""

    _fields_ = [("fp_blocks_per_sm", ctypes.c_int32), ("fp_dynamic", ctypes.c_int32),
                ("bp_blocks_per_sm", ctypes.c_int32), ("bp_dynamic", ctypes.c_int32),
                ("bp_tile_rows", ctypes.c_int32), ("reserved", ctypes.c_int32 * 3)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


# ct_allocator: alloc(ctx, bytes, stream) -> ptr, free(ctx, ptr, stream)
ALLOC_FN = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p)
FREE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)


class CtAllocator(ctypes.Structure):
    """Mirror of ct_allocator."""

    _fields_ = [("ctx", ctypes.c_void_p), ("alloc", ALLOC_FN), ("free", FREE_FN)]


class CtPlanOpts(ctypes.Structure):
    _fields_ = [("filter_window", ctypes.c_int32), ("filter_algo", ctypes.c_int32),
                ("short_scan", ctypes.c_int32), ("cosine_weight", ctypes.c_int32),
                ("texture_weights", ctypes.c_int32), ("reserved", ctypes.c_int32 * 3)]


_vp = ctypes.c_void_p
_i = ctypes.c_int
_sz = ctypes.c_size_t
_P = ctypes.POINTER

# name -> (restype, argtypes); every function include/ctgb.h declares.
SIGNATURES = {
    "ct_status_string": (ctypes.c_char_p, [_i]),
    "ct_version": (ctypes.c_char_p, []),
    "ct_last_error": (ctypes.c_char_p, []),
    "ct_launch_count": (ctypes.c_uint64, []),
    "ct_build_flags": (ctypes.c_uint32, []),
    "ct_set_allocator": (_i, [_P(CtAllocator)]),
    "ct_device_alloc_count": (ctypes.c_uint64, []),
    "ct_host_mapped": (_i, [_vp, _P(_vp)]),
    "ct_geom_from_param16": (_i, [_P(ctypes.c_float), _P(CtFanGeom)]),
    "ct_fp_ray_table": (_i, [_P(CtFanGeom), _P(ctypes.c_float), _i, _P(ctypes.c_float),
                            _P(ctypes.c_int32)]),
    "ct_plan_create": (_i, [_P(CtFanGeom), _P(ctypes.c_float), _i, _P(CtPlanOpts), _P(_vp)]),
    "ct_plan_create_cone": (_i, [_P(CtFanGeom), _i, _i, _P(ctypes.c_float), _i, _P(CtPlanOpts),
                                 _P(_vp)]),
    "ct_plan_create_cone_ex": (_i, [_P(CtFanGeom), _i, _i, _P(ctypes.c_float),
                                    _P(ctypes.c_float), _i, _P(CtPlanOpts), _P(_vp)]),
    "ct_plan_destroy": (_i, [_vp]),
    "ct_plan_check": (_i, [_vp]),
    "ct_plan_selftest_wait_timeout": (_i, [_vp, ctypes.c_int32, _vp]),
    "ct_plan_geom": (_i, [_vp, _P(CtFanGeom)]),
    "ct_workspace_size": (_i, [_vp, _i, _i, _P(_sz)]),
    "ct_fp_fan": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_fp_fan_adjoint": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_bp_fan": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_bp_fan_adjoint": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_ramp_filter": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_fbp_fan": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_fbp_fan_adjoint": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_fdk_bp": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_cone_bp": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_fdk_cone": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_fdk_cone_adjoint": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_fp_cone": (_i, [_vp, _vp, _vp, _i, _vp, _sz, _vp]),
    "ct_batch_workspace_size": (_i, [_P(CtBatchItem), _i, _P(_sz)]),
    "ct_batch_run": (_i, [_P(CtBatchItem), _i, _vp, _sz, _vp]),
    "ct_batch_tune": (_i, [_P(CtBatchItem), _i, _vp, _sz, ctypes.c_int32, _vp,
                           _P(CtBatchConfig)]),
    "ct_batch_get_config": (_i, [_P(CtBatchItem), _i, _P(CtBatchConfig),
                                 _P(ctypes.c_int32)]),
    "ct_batch_set_config": (_i, [_P(CtBatchItem), _i, _P(CtBatchConfig)]),
    "ct_fbp_fan_static_scratch": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_plain_fp_fan": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_plain_fp_fan_adjoint": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_plain_bp_fan": (_i, [_vp, _vp, _vp, _i, _vp]),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> Path:
    return _build.LIB_PATH


def _bind(path) -> ctypes.CDLL:
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads libctgb.so (building it in-tree first if it is absent or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build_if_missing else _build.LIB_PATH
        if not Path(path).exists():
            raise RuntimeError(f"libctgb.so not found at {path}; run __graft_entry__.build()")
        _lib = _bind(path)
        return _lib


_debug_lib = None


def load_debug() -> ctypes.CDLL:
    """The debug build of the library (kernels with index checks, -DCT_DEBUG),
    built in-tree on first use into _build/debug/.  A separate library with
    its own plans: pass it only plans it created."""
    global _debug_lib
    with _lock:
        if _debug_lib is None:
            _debug_lib = _bind(_build.build(debug=True))
        return _debug_lib


def check(status: int, where: str) -> None:
    if status != CT_OK:
        detail = ""
        try:
            detail = load().ct_last_error().decode()
        except Exception:  # pragma: no cover - best effort message
            pass
        raise CtError(status, where, detail)


def launch_count() -> int:
    return int(load().ct_launch_count())
