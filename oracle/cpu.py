"""FP32 OpenMP CPU transcription of the reference's operators (``cpu_fp32.c``):
the timed CPU baseline of ``bench.py`` (its ``cpu_baseline`` entries and its
``--impl reference`` arm).

MEASUREMENT INFRASTRUCTURE ONLY.  The parity checker is the FP64 oracle
(``oracle.c``); this module keeps the reference's single precision so that
its speed is the reference algorithm's on host cores.  Only ``bench.py`` and
``tests/`` import it.

Compiled with gcc ``-O3 -fopenmp`` into ``oracle/_build/libcpufp32.so`` on
first use.  ``OMP_NUM_THREADS`` sets the thread count (default: all cores).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import platform
import subprocess
import time
from pathlib import Path

import numpy as np

from . import OrcGeom, _angles

_DIR = Path(__file__).resolve().parent
_SRC = _DIR / "cpu_fp32.c"
_BUILD = _DIR / "_build"
_LIB = _BUILD / "libcpufp32.so"
_CFLAGS = ["-O3", "-fopenmp", "-fPIC", "-Wall", "-Wextra", "-shared"]

_lib = None


def build(force: bool = False) -> Path:
    """Compiles libcpufp32.so (gcc -O3, OpenMP) if missing or stale."""
    _BUILD.mkdir(parents=True, exist_ok=True)
    stamp = _BUILD / "cpufp32.stamp"
    fp = hashlib.sha256(_SRC.read_bytes() + " ".join(_CFLAGS).encode()
                        + os.uname().machine.encode()).hexdigest()
    if not force and _LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return _LIB
    tmp = _BUILD / "libcpufp32.so.tmp"
    cmd = ["gcc", *_CFLAGS, str(_SRC), "-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"CPU baseline build failed: {' '.join(cmd)}\n{res.stderr}")
    os.replace(tmp, _LIB)
    stamp.write_text(fp)
    return _LIB


def _l():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        P = ctypes.POINTER
        fp_ = P(ctypes.c_float)
        g = P(OrcGeom)
        ci = ctypes.c_int
        lib.cpu_threads.restype = ci
        lib.cpu_fp_fan.argtypes = [g, fp_, ci, ci, fp_, fp_, ci]
        lib.cpu_bp_fan.argtypes = [g, fp_, ci, ci, fp_, fp_, ci, ci]
        lib.cpu_ramp_taps.argtypes = [g, fp_]
        lib.cpu_ramp_filter.argtypes = [g, fp_, fp_, fp_, ctypes.c_long]
        lib.cpu_fbp_fan.argtypes = [g, fp_, ci, ci, fp_, fp_, ci, fp_]
        _lib = lib
    return _lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def threads() -> int:
    return int(_l().cpu_threads())


def cpu_model() -> str:
    """The host CPU's model name, as the OS reports it."""
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            k = line.split(":", 1)[0].strip().lower()
            if k in ("model name", "cpu model", "hardware"):
                return line.split(":", 1)[1].strip()
        # Arm kernels report implementer/part numbers, not a name
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("cpu part"):
                return f"{platform.machine()} (cpu part {line.split(':', 1)[1].strip()})"
    except OSError:
        pass
    return platform.machine()


def _views(g: OrcGeom, angles, view0: int, n_views: int):
    a = _angles(g, angles)
    if not (0 <= view0 and n_views >= 1 and view0 + n_views <= g.n_views):
        raise ValueError("view range outside the plan's views")
    return a


def fp_fan(g: OrcGeom, angles, img, view0: int = 0, n_views: int | None = None) -> np.ndarray:
    """FP32 forward projection of img [B, ny, nx] over views view0 .. view0+n_views-1."""
    n_views = g.n_views if n_views is None else n_views
    a = _views(g, angles, view0, n_views)
    x = _f32(img)
    if x.ndim == 2:
        x = x[None]
    out = np.zeros((x.shape[0], n_views, g.n_cols), np.float32)
    _l().cpu_fp_fan(ctypes.byref(g), _fptr(a), view0, n_views, _fptr(x), _fptr(out), x.shape[0])
    return out


def bp_fan(g: OrcGeom, angles, sino, view0: int = 0, weighted: bool = False) -> np.ndarray:
    """FP32 pixel-driven BP of sino [B, n_views, n_cols] (views view0 ..)."""
    y = _f32(sino)
    if y.ndim == 2:
        y = y[None]
    a = _views(g, angles, view0, y.shape[1])
    out = np.zeros((y.shape[0], g.ny, g.nx), np.float32)
    _l().cpu_bp_fan(ctypes.byref(g), _fptr(a), view0, y.shape[1], _fptr(y), _fptr(out),
                    y.shape[0], 1 if weighted else 0)
    return out


def ramp_filter(g: OrcGeom, sino) -> np.ndarray:
    """The reference's Ram-Lak row filter in FP32, direct O(C^2)."""
    y = _f32(sino)
    taps = np.zeros(2 * g.n_cols - 1, np.float32)
    _l().cpu_ramp_taps(ctypes.byref(g), _fptr(taps))
    out = np.zeros_like(y)
    _l().cpu_ramp_filter(ctypes.byref(g), _fptr(taps), _fptr(y), _fptr(out), y.size // g.n_cols)
    return out


def fbp_fan(g: OrcGeom, angles, sino, view0: int = 0) -> np.ndarray:
    """FP32 Ram-Lak FBP of sino [B, n_views, n_cols] (views view0 ..)."""
    y = _f32(sino)
    if y.ndim == 2:
        y = y[None]
    a = _views(g, angles, view0, y.shape[1])
    out = np.zeros((y.shape[0], g.ny, g.nx), np.float32)
    work = np.zeros_like(y)
    _l().cpu_fbp_fan(ctypes.byref(g), _fptr(a), view0, y.shape[1], _fptr(y), _fptr(out),
                     y.shape[0], _fptr(work))
    return out


def time_ops(g: OrcGeom, angles, img, sino, n_views: int, reps: int = 1) -> dict:
    """Times FP, BP and FBP of one slice over n_views views spread over the
    scan (every k-th view); returns the best of `reps` seconds each and the
    rates they give: FP rays/s, BP pixel-views/s (full grid), and FBP seconds
    per slice extrapolated to all views (the filter and the BP both scale
    with the view count)."""
    step = max(1, g.n_views // n_views)
    sel = np.arange(0, step * n_views, step)[:n_views]
    sub = OrcGeom.from_buffer_copy(g)
    sub.n_views = len(sel)
    a = _f32(np.asarray(angles, np.float32)[sel])
    s_sub = _f32(np.asarray(sino)[..., sel, :]) if np.asarray(sino).ndim == 3 else \
        _f32(np.asarray(sino)[sel])
    best = {"fp": float("inf"), "bp": float("inf"), "fbp": float("inf")}
    for _ in range(reps):
        t0 = time.perf_counter()
        fp_fan(sub, a, img)
        best["fp"] = min(best["fp"], time.perf_counter() - t0)
        t0 = time.perf_counter()
        bp_fan(sub, a, s_sub)
        best["bp"] = min(best["bp"], time.perf_counter() - t0)
        t0 = time.perf_counter()
        fbp_fan(sub, a, s_sub)
        best["fbp"] = min(best["fbp"], time.perf_counter() - t0)
    nv = len(sel)
    return {
        "views_timed": nv,
        "seconds": best,
        "fp_grays_per_s": nv * g.n_cols / best["fp"] / 1e9,
        "bp_gpix_views_per_s": nv * g.nx * g.ny / best["bp"] / 1e9,
        "fbp_ms_per_slice": 1e3 * best["fbp"] * g.n_views / nv,
        "threads": threads(),
        "cpu": cpu_model(),
    }
