"""The executed reference: FanBeamCTRecon_TensorflowOp's own ops (the
TensorFlow op wrapper and its CUDA source), compiled by ``oracle/build_ref.py``
against host stand-ins and run on the CPU.  TEST INFRASTRUCTURE ONLY: the
golden-vector script and the tests call it as the checker; no product code
imports it.

It exists only where the reference's sources are present (it is built from
them in place); elsewhere ``available()`` is False and the committed golden
vectors it produced stand in for it.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build_ref

OP_NAMES = {op: name for op, (_, _, name) in build_ref.OPS.items()}
_LIBS: dict[str, ctypes.CDLL] = {}
_P = ctypes.POINTER


def available(ref: Path | None = None) -> bool:
    """Builds the libraries if the reference's sources are present."""
    try:
        return build_ref.build(ref) is not None
    except RuntimeError:
        raise
    except OSError:
        return False


def _lib(op: str) -> ctypes.CDLL:
    if op not in _LIBS:
        libs = build_ref.build()
        if libs is None:
            raise RuntimeError("the reference's sources are not present; the executed "
                               "reference cannot be built")
        lib = ctypes.CDLL(str(libs[op]))
        i64p, f32p = _P(ctypes.c_longlong), _P(ctypes.c_float)
        lib.ctref_run.argtypes = [ctypes.c_char_p, f32p, ctypes.c_longlong, f32p,
                                  ctypes.c_longlong, i64p, ctypes.c_int, i64p, ctypes.c_int,
                                  f32p, ctypes.c_longlong, f32p, ctypes.c_longlong,
                                  ctypes.c_char_p, ctypes.c_longlong]
        lib.ctref_run.restype = ctypes.c_int
        lib.ctref_shape.argtypes = [ctypes.c_char_p, i64p, ctypes.c_int, i64p, ctypes.c_int,
                                    i64p, ctypes.c_int, i64p, _P(ctypes.c_int),
                                    ctypes.c_char_p, ctypes.c_longlong]
        lib.ctref_shape.restype = ctypes.c_int
        _LIBS[op] = lib
    return _LIBS[op]


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _i64(s) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(list(s), dtype=np.int64))


def run(op: str, parameter, angle, vol_shape, proj_shape, x) -> np.ndarray:
    """Constructs the reference's op ``op`` ("fp", "bp", "fbp", "fdk") with
    these attributes and computes it on ``x``; returns the output shaped
    ``proj_shape`` (fp) or ``vol_shape``."""
    lib = _lib(op)
    p, a, xin = _f32(parameter), _f32(angle), _f32(x)
    vs, ps = _i64(vol_shape), _i64(proj_shape)
    out_shape = tuple(ps if op == "fp" else vs)
    out = np.zeros(out_shape, np.float32)
    err = ctypes.create_string_buffer(2048)
    f32p, i64p = _P(ctypes.c_float), _P(ctypes.c_longlong)
    rc = lib.ctref_run(OP_NAMES[op].encode(), p.ctypes.data_as(f32p), p.size,
                       a.ctypes.data_as(f32p), a.size, vs.ctypes.data_as(i64p), vs.size,
                       ps.ctypes.data_as(i64p), ps.size, xin.ctypes.data_as(f32p), xin.size,
                       out.ctypes.data_as(f32p), out.size, err, len(err))
    if rc != 0:
        raise RuntimeError(f"reference {OP_NAMES[op]}: {err.value.decode()}")
    return out


def shape(op: str, in_shape, vol_shape, proj_shape) -> tuple:
    """The reference op's registered shape function on an input shape."""
    lib = _lib(op)
    ins, vs, ps = _i64(in_shape), _i64(vol_shape), _i64(proj_shape)
    out = np.zeros(8, np.int64)
    rank = ctypes.c_int(0)
    err = ctypes.create_string_buffer(1024)
    i64p = _P(ctypes.c_longlong)
    rc = lib.ctref_shape(OP_NAMES[op].encode(), ins.ctypes.data_as(i64p), ins.size,
                         vs.ctypes.data_as(i64p), vs.size, ps.ctypes.data_as(i64p), ps.size,
                         out.ctypes.data_as(i64p), ctypes.byref(rank), err, len(err))
    if rc != 0:
        raise ValueError(err.value.decode())
    return tuple(int(v) for v in out[:rank.value])
