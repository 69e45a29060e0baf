"""PyTorch-facing operators over the C ABI.

``FanPlan`` owns a ct_plan (geometry decoded from the reference's 16-float
parameter vector plus the view angles) on one CUDA device.  Its methods take
and return float32 CUDA tensors -- images [B, ny, nx], sinograms
[B, n_views, n_cols] -- and enqueue the library's kernels on the current
torch stream.  Scratch space comes from torch's caching allocator.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np
import torch

from . import _lib
from .geometry import decode

_plan_cache: dict = {}
_plan_lock = threading.Lock()


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


class FanPlan:
    """A fan-beam geometry bound to one CUDA device.

    ``texture_weights=True`` makes the backprojectors (BP, FBP, the FDK op and
    their adjoints) interpolate with the GPU texture unit's 8-bit weights, as
    the reference's texture fetches did; the default interpolates with exact
    FP32 weights.  The forward projector is exact either way."""

    n_rows = 1
    nz = 1

    def __init__(self, param16, angles, device=None, window: int = _lib.WINDOW_RAMLAK,
                 filter_algo: int = _lib.FILTER_AUTO, short_scan: bool = False,
                 cosine_weight: bool = False, texture_weights: bool = False):
        self._lib = _lib.load()
        self.param16 = np.ascontiguousarray(np.asarray(param16, dtype=np.float32)).copy()
        self.angles = np.ascontiguousarray(np.asarray(angles, dtype=np.float32)).copy()
        self.geom = decode(self.param16)
        self.window = int(window)
        self.short_scan = bool(short_scan)
        self.cosine_weight = bool(cosine_weight)
        self.texture_weights = bool(texture_weights)
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("FanPlan needs a CUDA device")
        opts = _lib.CtPlanOpts()
        opts.filter_window = int(window)
        opts.filter_algo = int(filter_algo)
        opts.short_scan = int(self.short_scan)
        opts.cosine_weight = int(self.cosine_weight)
        opts.texture_weights = int(self.texture_weights)
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            st = self._create(opts, handle)
        _lib.check(st, "ct_plan_create")
        self._h = handle

    def _create(self, opts, handle) -> int:
        return self._lib.ct_plan_create(
            ctypes.byref(self.geom), self.angles.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            int(self.angles.shape[0]), ctypes.byref(opts), ctypes.byref(handle))

    # -- lifetime ---------------------------------------------------------------
    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.ct_plan_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def total_samples(self) -> int:
        """Ray samples of one FP slice (sum of floor(chord/0.125) over rays)."""
        if getattr(self, "_total_samples", None) is None:
            from .geometry import ray_table
            _, ns = ray_table(self.param16, self.angles)
            self._total_samples = int(ns.astype(np.int64).sum())
        return self._total_samples

    # -- shapes -----------------------------------------------------------------
    @property
    def image_shape(self) -> tuple[int, int]:
        return (self.geom.ny, self.geom.nx)

    @property
    def sino_shape(self) -> tuple[int, int]:
        return (self.geom.n_views, self.geom.n_cols)

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def _check_in(self, t: torch.Tensor, tail: tuple[int, int], what: str) -> torch.Tensor:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{what} must be a torch.Tensor")
        if t.device != self.device:
            raise ValueError(f"{what} is on {t.device}, plan is on {self.device}")
        if t.dtype != torch.float32:
            raise TypeError(f"{what} must be float32, got {t.dtype}")
        if t.dim() == 2:
            t = t.unsqueeze(0)
        if t.dim() != 3 or tuple(t.shape[1:]) != tail:
            raise ValueError(f"{what} must be [B, {tail[0]}, {tail[1]}], got {tuple(t.shape)}")
        return t.contiguous()

    def workspace_bytes(self, op: int, batch: int) -> int:
        n = ctypes.c_size_t()
        _lib.check(self._lib.ct_workspace_size(self._h, op, batch, ctypes.byref(n)),
                   "ct_workspace_size")
        return int(n.value)

    def _work(self, op: int, batch: int):
        nbytes = self.workspace_bytes(op, batch)
        if nbytes == 0:
            return None, 0
        return torch.empty(nbytes, dtype=torch.uint8, device=self.device), nbytes

    def _run(self, name: str, op: int | None, x: torch.Tensor, out_tail: tuple[int, int],
             with_work: bool, out: torch.Tensor | None = None) -> torch.Tensor:
        B = x.shape[0]
        if out is None:
            out = torch.empty((B, *out_tail), dtype=torch.float32, device=self.device)
        fn = getattr(self._lib, name)
        with torch.cuda.device(self.device):
            if with_work:
                work, nbytes = self._work(op, B)
                st = fn(self._h, _ptr(x), _ptr(out), B, _ptr(work), nbytes, self._stream())
            else:
                st = fn(self._h, _ptr(x), _ptr(out), B, self._stream())
        _lib.check(st, name)
        return out

    # -- operators --------------------------------------------------------------
    def fp(self, img: torch.Tensor, out=None) -> torch.Tensor:
        """Ray-driven forward projection (FPFanCurve)."""
        x = self._check_in(img, self.image_shape, "image")
        return self._run("ct_fp_fan", _lib.OP_FP, x, self.sino_shape, True, out)

    def fp_to_host(self, img: torch.Tensor) -> torch.Tensor:
        """``fp`` with its sinogram written straight into page-locked host memory:
        the kernel's stores cross to the host while it runs and no device-to-host
        copy follows.  Returns a pinned CPU tensor, complete once the device's
        current stream has been synchronised."""
        x = self._check_in(img, self.image_shape, "image")
        host = torch.empty((x.shape[0], *self.sino_shape), dtype=torch.float32, pin_memory=True)
        dptr = ctypes.c_void_p()
        st = self._lib.ct_host_mapped(ctypes.c_void_p(host.data_ptr()), ctypes.byref(dptr))
        if st != 0:
            # page-locked memory that is not mapped for the device: copy back instead
            return self.fp(x).to("cpu")
        B = x.shape[0]
        with torch.cuda.device(self.device):
            work, nbytes = self._work(_lib.OP_FP, B)
            st = self._lib.ct_fp_fan(self._h, _ptr(x), dptr.value, B, _ptr(work), nbytes,
                                     self._stream())
        _lib.check(st, "ct_fp_fan")
        return host

    def fp_adjoint(self, sino: torch.Tensor, out=None) -> torch.Tensor:
        """Exact transpose of ``fp``."""
        y = self._check_in(sino, self.sino_shape, "sinogram")
        return self._run("ct_fp_fan_adjoint", _lib.OP_FP_ADJOINT, y, self.image_shape, True, out)

    def bp(self, sino: torch.Tensor, out=None) -> torch.Tensor:
        """Unweighted pixel-driven backprojection (BPFanCurve)."""
        y = self._check_in(sino, self.sino_shape, "sinogram")
        return self._run("ct_bp_fan", None, y, self.image_shape, False, out)

    def bp_adjoint(self, img: torch.Tensor, out=None) -> torch.Tensor:
        """Exact transpose of ``bp``."""
        x = self._check_in(img, self.image_shape, "image")
        return self._run("ct_bp_fan_adjoint", None, x, self.sino_shape, False, out)

    def ramp_filter(self, sino: torch.Tensor, out=None) -> torch.Tensor:
        """Row ramp filter with the plan's window."""
        y = self._check_in(sino, self.sino_shape, "sinogram")
        if out is None:
            out = torch.empty_like(y)
        with torch.cuda.device(self.device):
            st = self._lib.ct_ramp_filter(self._h, _ptr(y), _ptr(out), y.shape[0] * y.shape[1],
                                          self._stream())
        _lib.check(st, "ct_ramp_filter")
        return out

    def fbp(self, sino: torch.Tensor, out=None) -> torch.Tensor:
        """Filtered backprojection (FBPFanCurve)."""
        y = self._check_in(sino, self.sino_shape, "sinogram")
        return self._run("ct_fbp_fan", _lib.OP_FBP, y, self.image_shape, True, out)

    def fbp_adjoint(self, img: torch.Tensor, out=None) -> torch.Tensor:
        """Exact transpose of ``fbp``."""
        x = self._check_in(img, self.image_shape, "image")
        return self._run("ct_fbp_fan_adjoint", _lib.OP_FBP_ADJOINT, x, self.sino_shape, True, out)

    def fdk_bp(self, sino: torch.Tensor, out=None) -> torch.Tensor:
        """The reference FDK "BackProjection" op (one detector row, one slice)."""
        y = self._check_in(sino, self.sino_shape, "sinogram")
        return self._run("ct_fdk_bp", _lib.OP_FDK_BP, y, self.image_shape, True, out)

    # -- the plain per-view launch loop (measurement baseline) -------------------
    def plain_fp(self, img: torch.Tensor) -> torch.Tensor:
        x = self._check_in(img, self.image_shape, "image")
        return self._run("ct_plain_fp_fan", None, x, self.sino_shape, False)

    def plain_fp_adjoint(self, sino: torch.Tensor) -> torch.Tensor:
        y = self._check_in(sino, self.sino_shape, "sinogram")
        return self._run("ct_plain_fp_fan_adjoint", None, y, self.image_shape, False)

    def plain_bp(self, sino: torch.Tensor) -> torch.Tensor:
        y = self._check_in(sino, self.sino_shape, "sinogram")
        return self._run("ct_plain_bp_fan", None, y, self.image_shape, False)


class ConePlan(FanPlan):
    """A cone-beam geometry: the fan geometry of ``param16`` (parameter[13..15]
    = detector bottom, row height, slice thickness) with ``n_rows`` detector
    rows and ``nz`` slices.  Volumes are float32 [B, nz, ny, nx], projections
    float32 [B, n_views, n_rows, n_cols].  ``source_z`` (mm, one per view)
    puts the source of each view at that height: a z-offset orbit or a helix;
    ``cosine_weight`` adds Feldkamp's cos(gamma) cos(cone angle) pre-weight."""

    def __init__(self, param16, angles, n_rows: int, nz: int, device=None,
                 window: int = _lib.WINDOW_RAMLAK, short_scan: bool = False,
                 cosine_weight: bool = False, source_z=None, texture_weights: bool = False):
        self.n_rows = int(n_rows)
        self.nz = int(nz)
        self.source_z = (None if source_z is None else
                         np.ascontiguousarray(np.asarray(source_z, dtype=np.float32)).copy())
        super().__init__(param16, angles, device=device, window=window, short_scan=short_scan,
                         cosine_weight=cosine_weight, texture_weights=texture_weights)

    def _create(self, opts, handle) -> int:
        fptr = ctypes.POINTER(ctypes.c_float)
        if self.source_z is not None and self.source_z.shape != self.angles.shape:
            raise ValueError("source_z needs one height per view")
        zs = None if self.source_z is None else self.source_z.ctypes.data_as(fptr)
        return self._lib.ct_plan_create_cone_ex(
            ctypes.byref(self.geom), self.n_rows, self.nz, self.angles.ctypes.data_as(fptr), zs,
            int(self.angles.shape[0]), ctypes.byref(opts), ctypes.byref(handle))

    @property
    def volume_shape(self) -> tuple[int, int, int]:
        return (self.nz, self.geom.ny, self.geom.nx)

    @property
    def proj_shape(self) -> tuple[int, int, int]:
        return (self.geom.n_views, self.n_rows, self.geom.n_cols)

    def _check4(self, t: torch.Tensor, tail, what: str) -> torch.Tensor:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{what} must be a torch.Tensor")
        if t.device != self.device or t.dtype != torch.float32:
            raise ValueError(f"{what} must be float32 on {self.device}")
        if t.dim() == 3:
            t = t.unsqueeze(0)
        if t.dim() != 4 or tuple(t.shape[1:]) != tuple(tail):
            raise ValueError(f"{what} must be [B, {', '.join(map(str, tail))}], got "
                             f"{tuple(t.shape)}")
        return t.contiguous()

    def _run4(self, name, op, x, out_tail, out=None):
        B = x.shape[0]
        if out is None:
            out = torch.empty((B, *out_tail), dtype=torch.float32, device=self.device)
        fn = getattr(self._lib, name)
        with torch.cuda.device(self.device):
            if op is None:
                st = fn(self._h, _ptr(x), _ptr(out), B, self._stream())
            else:
                work, nbytes = self._work(op, B)
                st = fn(self._h, _ptr(x), _ptr(out), B, _ptr(work), nbytes, self._stream())
        _lib.check(st, name)
        return out

    def fp_cone(self, vol: torch.Tensor, out=None) -> torch.Tensor:
        """Cone-beam forward projection."""
        x = self._check4(vol, self.volume_shape, "volume")
        return self._run4("ct_fp_cone", _lib.OP_FP_CONE, x, self.proj_shape, out)

    def cone_bp(self, proj: torch.Tensor, out=None) -> torch.Tensor:
        """The reference's CB_EA backprojection (unfiltered)."""
        y = self._check4(proj, self.proj_shape, "projections")
        return self._run4("ct_cone_bp", None, y, self.volume_shape, out)

    def fdk(self, proj: torch.Tensor, out=None) -> torch.Tensor:
        """FDK: ramp filter per (view, row), then the CB_EA backprojection."""
        y = self._check4(proj, self.proj_shape, "projections")
        return self._run4("ct_fdk_cone", _lib.OP_FDK_CONE, y, self.volume_shape, out)

    def fdk_adjoint(self, vol: torch.Tensor, out=None) -> torch.Tensor:
        """Exact transpose of ``fdk``."""
        x = self._check4(vol, self.volume_shape, "volume")
        return self._run4("ct_fdk_cone_adjoint", _lib.OP_FDK_CONE_ADJOINT, x, self.proj_shape,
                          out)


def get_plan(param16, angles, device=None, window: int = _lib.WINDOW_RAMLAK,
             short_scan: bool = False) -> FanPlan:
    """A cached FanPlan for (parameter, angles, device, window, short scan)."""
    p = np.ascontiguousarray(np.asarray(param16, dtype=np.float32))
    a = np.ascontiguousarray(np.asarray(angles, dtype=np.float32))
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    device = torch.device(device)
    if device.type == "cuda" and device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    key = (p.tobytes(), a.tobytes(), str(device), int(window), bool(short_scan))
    with _plan_lock:
        plan = _plan_cache.get(key)
        if plan is None:
            plan = FanPlan(p, a, device=device, window=window, short_scan=short_scan)
            _plan_cache[key] = plan
        return plan


def clear_plan_cache() -> None:
    with _plan_lock:
        for p in _plan_cache.values():
            p.close()
        _plan_cache.clear()
