"""The C ABI on the CPU: the library loads, exports every function
include/ctgb.h declares, and its host-only entry points validate input.
No kernel is launched here."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from fanbeamctrecon_tensorflowop_gb300 import _lib
from fanbeamctrecon_tensorflowop_gb300.geometry import decode, param_set
import geometries as G

HEADER = Path(__file__).resolve().parent.parent / "include" / "ctgb.h"


def declared_functions() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(ct_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(ctlib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(ctlib, n), f"{n} declared in ctgb.h but not exported"
    # and the Python binding types every one of them
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_library_is_in_tree(ctlib):
    p = _lib.lib_path()
    assert p.exists() and p.parent.name == "_build"


def test_status_strings(ctlib):
    for code, name in _lib.STATUS_NAMES.items():
        assert ctlib.ct_status_string(code).decode().startswith(name)
    assert b"unknown" in ctlib.ct_status_string(99)
    assert ctlib.ct_version().startswith(b"ctgb")


def _decode_status(ctlib, p):
    g = _lib.CtFanGeom()
    p = np.ascontiguousarray(p, dtype=np.float32)
    return ctlib.ct_geom_from_param16(p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                      ctypes.byref(g))


@pytest.mark.parametrize("idx,val", [
    (2, 0), (2, np.nan), (4, -3), (5, 0), (6, np.inf), (7, 0), (7, 600),  # rfov >= sid
    (1, np.nan), (8, 0), (8, -0.06), (3, np.inf),
])
def test_decode_rejects_invalid_geometry(ctlib, idx, val):
    p = param_set(1)
    p[idx] = val
    assert _decode_status(ctlib, p) == 1  # CT_ERR_INVALID_ARGUMENT


def test_null_pointers_and_null_plan(ctlib):
    g = _lib.CtFanGeom()
    assert ctlib.ct_geom_from_param16(None, ctypes.byref(g)) == 2
    # operator calls on a NULL plan fail before touching CUDA
    for name in ("ct_fp_fan", "ct_fp_fan_adjoint", "ct_fbp_fan", "ct_fbp_fan_adjoint",
                 "ct_fdk_bp"):
        assert getattr(ctlib, name)(None, None, None, 1, None, 0, None) == 2
    for name in ("ct_bp_fan", "ct_bp_fan_adjoint", "ct_ramp_filter", "ct_plain_fp_fan",
                 "ct_plain_fp_fan_adjoint", "ct_plain_bp_fan"):
        assert getattr(ctlib, name)(None, None, None, 1, None) == 2
    n = ctypes.c_size_t()
    assert ctlib.ct_workspace_size(None, 0, 1, ctypes.byref(n)) == 2
    assert ctlib.ct_plan_destroy(None) == 0


def test_plan_create_validates_before_cuda(ctlib):
    p, a = G.small()
    g = decode(p)
    h = ctypes.c_void_p()
    fptr = a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    # wrong angle count
    assert ctlib.ct_plan_create(ctypes.byref(g), fptr, len(a) - 1, None, ctypes.byref(h)) == 1
    # non-finite angle
    bad = a.copy()
    bad[3] = np.nan
    assert ctlib.ct_plan_create(ctypes.byref(g), bad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                len(a), None, ctypes.byref(h)) == 1
    # bad option values
    o = _lib.CtPlanOpts()
    o.filter_window = 7
    assert ctlib.ct_plan_create(ctypes.byref(g), fptr, len(a), ctypes.byref(o),
                                ctypes.byref(h)) == 1
    o = _lib.CtPlanOpts()
    o.reserved[2] = 1
    assert ctlib.ct_plan_create(ctypes.byref(g), fptr, len(a), ctypes.byref(o),
                                ctypes.byref(h)) == 1
    assert ctlib.ct_plan_create(None, fptr, len(a), None, ctypes.byref(h)) == 2


def test_ray_table_rejects_bad_input(ctlib):
    p, a = G.small()
    g = decode(p)
    ray = np.zeros(4 * g.n_views * g.n_cols, np.float32)
    ns = np.zeros(g.n_views * g.n_cols, np.int32)
    fp = lambda x: x.ctypes.data_as(ctypes.POINTER(ctypes.c_float))  # noqa: E731
    ip = ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    assert ctlib.ct_fp_ray_table(ctypes.byref(g), fp(a), g.n_views, fp(ray), ip) == 0
    assert ctlib.ct_fp_ray_table(ctypes.byref(g), fp(a), g.n_views + 1, fp(ray), ip) == 1
    assert ctlib.ct_fp_ray_table(ctypes.byref(g), None, g.n_views, fp(ray), ip) == 2
    assert ns.max() > 0
