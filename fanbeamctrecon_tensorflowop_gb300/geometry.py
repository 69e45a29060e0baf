"""Geometry packing: the reference's ``angle()`` / ``param_set()`` and decoding.

``angle`` and ``param_set`` reproduce utils.py:49-88 value for value (including
its quirks: the start angle is added in degrees to radian angles, utils.py:53,
and parameter[13:16] keep the 13, 14, 15 that ``np.arange(16)`` left there,
utils.py:73).  ``decode`` runs the library's ct_geom_from_param16, the float
arithmetic of the op constructors (FP/transform.cc:59-76).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from .config import config as _default_config


def angle(nview: int, fstartangle: float) -> np.ndarray:
    """float32[nview] view angles fstartangle + i*2*pi/nview (utils.py:49-54)."""
    d_angle = 2.0 * math.pi / nview
    return (float(fstartangle) + np.arange(nview, dtype=np.float64) * d_angle).astype(np.float32)


def param_set(nimg: int, cfg=None) -> np.ndarray:
    """The 16-float ``parameter`` attribute of utils.py:56-88."""
    c = _default_config if cfg is None else cfg
    sdd = c.SourceDetectorDistance
    sod = c.SourceAxisDistance
    nfan = c.FanAngle
    ncol = c.DetectorColumnNumber
    dcol = nfan / ncol
    dshift = c.DetectorShift
    d_left = -nfan / 2 - dshift * dcol
    p = np.arange(16, dtype=np.float32)
    p[0] = sdd
    p[1] = sod
    p[2] = c.ProjectionsPerRotation
    p[3] = c.FullAngle
    p[4] = ncol
    p[5] = c.NX
    p[6] = c.NY
    p[7] = c.FOVRadius
    p[8] = dcol
    p[9] = dshift
    p[10] = d_left
    p[11] = 1 * nimg
    p[12] = c.StartAngle
    return p


def fan_param16(*, sdd: float, sid: float, n_views: int, n_cols: int, n: int, pixel_mm: float,
                dcol_rad: float, full_angle: float = 360.0, shift: float = 0.0,
                left_rad: float | None = None, ny: int | None = None, batch: int = 1,
                det_bottom: float = 13.0, drow: float = 14.0, dz: float = 15.0) -> np.ndarray:
    """Packs a geometry given in physical units into the 16-float vector.

    rFOV = n * pixel / 2; the detector is centred (left = -n_cols*dcol/2) unless
    ``left_rad`` is given.
    """
    ny = n if ny is None else ny
    left = -n_cols * dcol_rad / 2.0 if left_rad is None else left_rad
    p = np.arange(16, dtype=np.float32)
    p[0] = sdd
    p[1] = sid
    p[2] = n_views
    p[3] = full_angle
    p[4] = n_cols
    p[5] = n
    p[6] = ny
    p[7] = n * pixel_mm / 2.0
    p[8] = math.degrees(dcol_rad)
    p[9] = shift
    p[10] = math.degrees(left)
    p[11] = batch
    p[12] = 0.0
    p[13] = det_bottom
    p[14] = drow
    p[15] = dz
    return p


def decode(param16) -> _lib.CtFanGeom:
    """ct_geom_from_param16 (host-only; raises CtError on invalid geometry)."""
    p = np.ascontiguousarray(np.asarray(param16, dtype=np.float32))
    if p.shape != (16,):
        raise ValueError(f"parameter must have 16 entries, got shape {p.shape}")
    g = _lib.CtFanGeom()
    st = _lib.load().ct_geom_from_param16(p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                         ctypes.byref(g))
    _lib.check(st, "ct_geom_from_param16")
    return g


def ray_table(param16, angles):
    """(ray [V, C, 4] float32, nsamp [V, C] int32): the forward projector's FP64
    ray table as plans build it (ct_fp_ray_table; host-only)."""
    g = decode(param16)
    a = np.ascontiguousarray(np.asarray(angles, dtype=np.float32))
    ray = np.zeros((g.n_views, g.n_cols, 4), np.float32)
    ns = np.zeros((g.n_views, g.n_cols), np.int32)
    st = _lib.load().ct_fp_ray_table(
        ctypes.byref(g), a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), int(a.shape[0]),
        ray.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
        ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    _lib.check(st, "ct_fp_ray_table")
    return ray, ns
