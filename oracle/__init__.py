"""FP64 CPU oracle of the reference's FP / BP / FBP / FDK operators.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` import this package, and only as the checker
or the timed CPU reference; the product path never calls it.

Parity status: pinned to the reference's own ops, executed.  Its TensorFlow op
wrappers and CUDA sources are compiled for the host against stand-ins
(``build_ref.py``, ``refexec/``) and run by ``reference.py``; their outputs are
the golden vectors in ``tests/golden/reference_ops.npz``.  With the GPU
texture unit's weights (``texture_rule.h``, measured on GB300) this oracle
meets them within 2e-6 (FP), 1e-6 (BP) and 5e-5 (FBP, FDK) relative L2.

The C restatement (``oracle.c``) is compiled with gcc + OpenMP into
``oracle/_build/liboracle.so`` on first use (``build()``).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
_SRC = _DIR / "oracle.c"
_BUILD = _DIR / "_build"
_LIB = _BUILD / "liboracle.so"
_CFLAGS = ["-O2", "-fopenmp", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra", "-shared"]

RAMLAK = 0
SHEPP_LOGAN = 1


class OrcGeom(ctypes.Structure):
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


def build(force: bool = False) -> Path:
    """Compiles liboracle.so (gcc, OpenMP) if missing or stale."""
    _BUILD.mkdir(parents=True, exist_ok=True)
    stamp = _BUILD / "stamp.txt"
    fp = hashlib.sha256(_SRC.read_bytes() + (_SRC.parent / "texture_rule.h").read_bytes()
                        + " ".join(_CFLAGS).encode()
                        + os.uname().machine.encode()).hexdigest()
    if not force and _LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return _LIB
    tmp = _BUILD / "liboracle.so.tmp"
    cmd = ["gcc", *_CFLAGS, str(_SRC), "-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{res.stderr}")
    os.replace(tmp, _LIB)
    stamp.write_text(fp)
    return _LIB


_lib = None


def _l():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        P = ctypes.POINTER
        dp, fp_, ip = P(ctypes.c_double), P(ctypes.c_float), P(ctypes.c_int32)
        g = P(OrcGeom)
        lib.orc_decode_param16.argtypes = [fp_, g]
        lib.orc_decode_param16.restype = ctypes.c_int
        lib.orc_set_texture_emulation.argtypes = [ctypes.c_int]
        lib.orc_tex_fetch1d.argtypes = [fp_, ctypes.c_int, fp_, fp_, ctypes.c_int]
        lib.orc_tex_fetch2d.argtypes = [fp_, ctypes.c_int, ctypes.c_int, fp_, fp_, fp_,
                                        ctypes.c_int]
        lib.orc_ray_table.argtypes = [g, fp_, dp, ip]
        lib.orc_fp_fan.argtypes = [g, fp_, dp, dp, ctypes.c_int]
        lib.orc_fp_fan_adjoint.argtypes = [g, fp_, dp, dp, ctypes.c_int]
        lib.orc_bp_fan.argtypes = [g, fp_, dp, dp, ctypes.c_int, ctypes.c_int]
        lib.orc_bp_fan_transpose.argtypes = [g, fp_, dp, dp, ctypes.c_int, ctypes.c_int]
        lib.orc_ramp_taps.argtypes = [g, ctypes.c_int, dp]
        lib.orc_ramp_filter.argtypes = [g, ctypes.c_int, dp, dp, ctypes.c_long]
        lib.orc_fbp_fan.argtypes = [g, fp_, ctypes.c_int, dp, dp, ctypes.c_int]
        lib.orc_fbp_fan_adjoint.argtypes = [g, fp_, ctypes.c_int, dp, dp, ctypes.c_int]
        lib.orc_fdk_bp.argtypes = [g, fp_, ctypes.c_int, dp, dp, ctypes.c_int]
        lib.orc_parker_weight.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.orc_parker_weight.restype = ctypes.c_double
        lib.orc_parker_weights.argtypes = [g, fp_, dp]
        lib.orc_cosine_weights.argtypes = [g, ctypes.c_int, ctypes.c_int, dp]
        ci = ctypes.c_int
        lib.orc_cone_bp_zs.argtypes = [g, ci, ci, fp_, fp_, dp, dp, ci]
        lib.orc_cone_bp_transpose_zs.argtypes = [g, ci, ci, fp_, fp_, dp, dp, ci]
        lib.orc_cone_fp_zs.argtypes = [g, ci, ci, fp_, fp_, dp, dp, ci]
        lib.orc_cone_bp.argtypes = [g, ci, ci, fp_, dp, dp, ci]
        lib.orc_cone_bp_transpose.argtypes = [g, ci, ci, fp_, dp, dp, ci]
        lib.orc_fdk_cone.argtypes = [g, ci, ci, fp_, ci, dp, dp, ci]
        lib.orc_fdk_cone_adjoint.argtypes = [g, ci, ci, fp_, ci, dp, dp, ci]
        lib.orc_cone_fp.argtypes = [g, ci, ci, fp_, dp, dp, ci]
        _lib = lib
    return _lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _angles(g: OrcGeom, angles) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(angles, dtype=np.float32))
    if a.shape != (g.n_views,):
        raise ValueError(f"angles must have shape ({g.n_views},), got {a.shape}")
    return a


def decode(param16) -> OrcGeom:
    p = np.ascontiguousarray(np.asarray(param16, dtype=np.float32))
    if p.shape != (16,):
        raise ValueError("parameter vector must have 16 entries")
    g = OrcGeom()
    if _l().orc_decode_param16(_fptr(p), ctypes.byref(g)) != 0:
        raise ValueError("invalid parameter vector")
    return g


def set_texture_emulation(on: bool) -> None:
    _l().orc_set_texture_emulation(1 if on else 0)


def texture_fetch1d(table, x) -> np.ndarray:
    """The GPU texture unit's linear filter (texture_rule.h) on a 1-D fp32 row."""
    t = np.ascontiguousarray(table, np.float32)
    xs = np.ascontiguousarray(x, np.float32)
    out = np.empty(xs.size, np.float32)
    _l().orc_tex_fetch1d(_fptr(t), t.size, _fptr(xs), _fptr(out), xs.size)
    return out


def texture_fetch2d(table, x, y) -> np.ndarray:
    """The GPU texture unit's linear filter on an h-by-w fp32 image (row = y)."""
    t = np.ascontiguousarray(table, np.float32)
    xs = np.ascontiguousarray(x, np.float32)
    ys = np.ascontiguousarray(y, np.float32)
    out = np.empty(xs.size, np.float32)
    _l().orc_tex_fetch2d(_fptr(t), t.shape[1], t.shape[0], _fptr(xs), _fptr(ys), _fptr(out),
                         xs.size)
    return out


def ray_table(g: OrcGeom, angles):
    a = _angles(g, angles)
    R = g.n_views * g.n_cols
    ray = np.zeros((R, 4), np.float64)
    ns = np.zeros(R, np.int32)
    _l().orc_ray_table(ctypes.byref(g), _fptr(a), _dptr(ray),
                       ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return ray.reshape(g.n_views, g.n_cols, 4), ns.reshape(g.n_views, g.n_cols)


def _batch_img(g, img):
    x = _f64(img)
    if x.ndim == 2:
        x = x[None]
    if x.shape[1:] != (g.ny, g.nx):
        raise ValueError(f"image must be [B,{g.ny},{g.nx}], got {x.shape}")
    return x


def _batch_sino(g, sino):
    y = _f64(sino)
    if y.ndim == 2:
        y = y[None]
    if y.shape[1:] != (g.n_views, g.n_cols):
        raise ValueError(f"sinogram must be [B,{g.n_views},{g.n_cols}], got {y.shape}")
    return y


def fp_fan(g, angles, img) -> np.ndarray:
    x = _batch_img(g, img)
    out = np.zeros((x.shape[0], g.n_views, g.n_cols), np.float64)
    _l().orc_fp_fan(ctypes.byref(g), _fptr(_angles(g, angles)), _dptr(x), _dptr(out), x.shape[0])
    return out


def fp_fan_adjoint(g, angles, sino) -> np.ndarray:
    y = _batch_sino(g, sino)
    out = np.zeros((y.shape[0], g.ny, g.nx), np.float64)
    _l().orc_fp_fan_adjoint(ctypes.byref(g), _fptr(_angles(g, angles)), _dptr(y), _dptr(out),
                            y.shape[0])
    return out


def bp_fan(g, angles, sino, weighted: bool = False) -> np.ndarray:
    y = _batch_sino(g, sino)
    out = np.zeros((y.shape[0], g.ny, g.nx), np.float64)
    _l().orc_bp_fan(ctypes.byref(g), _fptr(_angles(g, angles)), _dptr(y), _dptr(out), y.shape[0],
                    1 if weighted else 0)
    return out


def bp_fan_transpose(g, angles, img, weighted: bool = False) -> np.ndarray:
    x = _batch_img(g, img)
    out = np.zeros((x.shape[0], g.n_views, g.n_cols), np.float64)
    _l().orc_bp_fan_transpose(ctypes.byref(g), _fptr(_angles(g, angles)), _dptr(x), _dptr(out),
                              x.shape[0], 1 if weighted else 0)
    return out


def ramp_taps(g, window: int = RAMLAK) -> np.ndarray:
    t = np.zeros(2 * g.n_cols - 1, np.float64)
    _l().orc_ramp_taps(ctypes.byref(g), window, _dptr(t))
    return t


def ramp_filter(g, sino, window: int = RAMLAK) -> np.ndarray:
    y = _f64(sino)
    if y.shape[-1] != g.n_cols:
        raise ValueError("last axis must be n_cols")
    out = np.zeros_like(y)
    rows = y.size // g.n_cols
    _l().orc_ramp_filter(ctypes.byref(g), window, _dptr(y), _dptr(out), rows)
    return out


def parker_weight(beta: float, gamma: float, half_fan: float) -> float:
    """Parker's short-scan weight of the ray (beta, gamma), undoubled."""
    return _l().orc_parker_weight(float(beta), float(gamma), float(half_fan))


def parker_weights(g, angles) -> np.ndarray:
    """Doubled Parker weights [n_views, n_cols] of a short-scan plan."""
    w = np.zeros((g.n_views, g.n_cols), np.float64)
    _l().orc_parker_weights(ctypes.byref(g), _fptr(_angles(g, angles)), _dptr(w))
    return w


def cosine_weights(g, n_rows: int = 1, cone: bool = False) -> np.ndarray:
    """Feldkamp cosine pre-weights [n_rows, n_cols]."""
    w = np.zeros((n_rows, g.n_cols), np.float64)
    _l().orc_cosine_weights(ctypes.byref(g), n_rows, 1 if cone else 0, _dptr(w))
    return w


def _weighted(g, angles, y, short_scan, cosine=False, n_rows=1, cone=False):
    """Scales y [B, V, (rows,) C] by the Parker table [V, C] and the cosine
    table [rows, C], each when requested."""
    if short_scan:
        w = parker_weights(g, angles)
        y = y * (w[:, None, :] if y.ndim == 4 else w)
    if cosine:
        w = cosine_weights(g, n_rows, cone)
        y = y * (w if y.ndim == 4 else w[0])
    return y


def fbp_fan(g, angles, sino, window: int = RAMLAK, short_scan: bool = False,
            cosine: bool = False) -> np.ndarray:
    y = np.ascontiguousarray(_weighted(g, angles, _batch_sino(g, sino), short_scan, cosine))
    out = np.zeros((y.shape[0], g.ny, g.nx), np.float64)
    _l().orc_fbp_fan(ctypes.byref(g), _fptr(_angles(g, angles)), window, _dptr(y), _dptr(out),
                     y.shape[0])
    return out


def fbp_fan_adjoint(g, angles, img, window: int = RAMLAK, short_scan: bool = False,
                    cosine: bool = False) -> np.ndarray:
    x = _batch_img(g, img)
    out = np.zeros((x.shape[0], g.n_views, g.n_cols), np.float64)
    _l().orc_fbp_fan_adjoint(ctypes.byref(g), _fptr(_angles(g, angles)), window, _dptr(x),
                             _dptr(out), x.shape[0])
    return _weighted(g, angles, out, short_scan, cosine)


def fdk_bp(g, angles, sino, window: int = RAMLAK, short_scan: bool = False,
           cosine: bool = False) -> np.ndarray:
    y = np.ascontiguousarray(_weighted(g, angles, _batch_sino(g, sino), short_scan, cosine))
    out = np.zeros((y.shape[0], g.ny, g.nx), np.float64)
    _l().orc_fdk_bp(ctypes.byref(g), _fptr(_angles(g, angles)), window, _dptr(y), _dptr(out),
                    y.shape[0])
    return out


# ---- cone beam: volume [B][nz][ny][nx], projections [B][V][n_rows][C] ----------

def _batch_vol(g, nz, vol):
    x = _f64(vol)
    if x.ndim == 3:
        x = x[None]
    if x.shape[1:] != (nz, g.ny, g.nx):
        raise ValueError(f"volume must be [B,{nz},{g.ny},{g.nx}], got {x.shape}")
    return x


def _batch_proj(g, n_rows, proj):
    y = _f64(proj)
    if y.ndim == 3:
        y = y[None]
    if y.shape[1:] != (g.n_views, n_rows, g.n_cols):
        raise ValueError(f"projections must be [B,{g.n_views},{n_rows},{g.n_cols}], got {y.shape}")
    return y


def _zs(g, source_z):
    if source_z is None:
        return None
    z = np.ascontiguousarray(np.asarray(source_z, np.float32))
    if z.shape != (g.n_views,):
        raise ValueError(f"source_z must be [{g.n_views}]")
    return z


def cone_fp(g, n_rows, nz, angles, vol, source_z=None) -> np.ndarray:
    x = _batch_vol(g, nz, vol)
    out = np.zeros((x.shape[0], g.n_views, n_rows, g.n_cols), np.float64)
    zs = _zs(g, source_z)
    if zs is None:
        _l().orc_cone_fp(ctypes.byref(g), n_rows, nz, _fptr(_angles(g, angles)), _dptr(x),
                         _dptr(out), x.shape[0])
    else:
        _l().orc_cone_fp_zs(ctypes.byref(g), n_rows, nz, _fptr(_angles(g, angles)), _fptr(zs),
                            _dptr(x), _dptr(out), x.shape[0])
    return out


def cone_bp(g, n_rows, nz, angles, proj, source_z=None) -> np.ndarray:
    y = _batch_proj(g, n_rows, proj)
    out = np.zeros((y.shape[0], nz, g.ny, g.nx), np.float64)
    zs = _zs(g, source_z)
    if zs is None:
        _l().orc_cone_bp(ctypes.byref(g), n_rows, nz, _fptr(_angles(g, angles)), _dptr(y),
                         _dptr(out), y.shape[0])
    else:
        _l().orc_cone_bp_zs(ctypes.byref(g), n_rows, nz, _fptr(_angles(g, angles)), _fptr(zs),
                            _dptr(y), _dptr(out), y.shape[0])
    return out


def cone_bp_transpose(g, n_rows, nz, angles, vol, source_z=None) -> np.ndarray:
    x = _batch_vol(g, nz, vol)
    out = np.zeros((x.shape[0], g.n_views, n_rows, g.n_cols), np.float64)
    zs = _zs(g, source_z)
    if zs is None:
        _l().orc_cone_bp_transpose(ctypes.byref(g), n_rows, nz, _fptr(_angles(g, angles)),
                                   _dptr(x), _dptr(out), x.shape[0])
    else:
        _l().orc_cone_bp_transpose_zs(ctypes.byref(g), n_rows, nz, _fptr(_angles(g, angles)),
                                      _fptr(zs), _dptr(x), _dptr(out), x.shape[0])
    return out


def fdk_cone(g, n_rows, nz, angles, proj, window: int = RAMLAK, short_scan: bool = False,
             cosine: bool = False, source_z=None) -> np.ndarray:
    """FDK: pre-weights (each when requested), the ramp filter of every
    (view, row), then the CB_EA backprojection."""
    y = _weighted(g, angles, _batch_proj(g, n_rows, proj), short_scan, cosine, n_rows, True)
    return cone_bp(g, n_rows, nz, angles, ramp_filter(g, y, window), source_z)


def fdk_cone_adjoint(g, n_rows, nz, angles, vol, window: int = RAMLAK, short_scan: bool = False,
                     cosine: bool = False, source_z=None) -> np.ndarray:
    t = ramp_filter(g, cone_bp_transpose(g, n_rows, nz, angles, vol, source_z), window)
    return _weighted(g, angles, t, short_scan, cosine, n_rows, True)


# ---- the GPU texture probe (tests/golden/texture_probe.cu) -------------------

_PROBE_SRC = Path(__file__).resolve().parent.parent / "tests" / "golden" / "texture_probe.cu"
_PROBE_LIB = _BUILD / "libtexprobe.so"
_probe = None


def texture_probe_build(force: bool = False) -> Path:
    """Compiles the texture probe with nvcc for sm_103a (needs the CUDA toolkit)."""
    _BUILD.mkdir(parents=True, exist_ok=True)
    stamp = _BUILD / "texprobe.stamp"
    fp = hashlib.sha256(_PROBE_SRC.read_bytes() + os.uname().machine.encode()).hexdigest()
    if not force and _PROBE_LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return _PROBE_LIB
    tmp = _BUILD / "libtexprobe.so.tmp"
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared",
           "-Xcompiler", "-fPIC", str(_PROBE_SRC), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"texture probe build failed: {' '.join(cmd)}\n{res.stderr}")
    os.replace(tmp, _PROBE_LIB)
    stamp.write_text(fp)
    return _PROBE_LIB


def texture_probe_fetch(table, x, y=None) -> np.ndarray:
    """Fetches through a real texture object on the current GPU: a 1-D row
    when ``y`` is None, else an h-by-w image (row = y)."""
    global _probe
    if _probe is None:
        lib = ctypes.CDLL(str(texture_probe_build()))
        fp_ = ctypes.POINTER(ctypes.c_float)
        lib.texprobe_fetch.argtypes = [fp_, ctypes.c_int, ctypes.c_int, fp_, fp_, fp_,
                                       ctypes.c_int]
        lib.texprobe_fetch.restype = ctypes.c_int
        _probe = lib
    t = np.ascontiguousarray(table, np.float32)
    xs = np.ascontiguousarray(x, np.float32)
    ys = xs if y is None else np.ascontiguousarray(y, np.float32)
    w, h = (t.size, 0) if y is None else (t.shape[1], t.shape[0])
    out = np.empty(xs.size, np.float32)
    rc = _probe.texprobe_fetch(_fptr(t), w, h, _fptr(xs), _fptr(ys), _fptr(out), xs.size)
    if rc != 0:
        raise RuntimeError(f"texture probe failed with CUDA error {rc}")
    return out
