"""Uneven batches: slices of different geometries, operators and storage
types in one ``ct_batch_run`` call (one persistent FP launch, one persistent
BP launch), optionally captured once in a CUDA graph and replayed.

    ub = UnevenBatch([(plan_a, "fp", img_a, sino_a), (plan_b, "fbp", sino_b, img_b), ...])
    ub.tune()                # optional: pick the launch shapes for this batch
    ub.run()                 # eager
    ub.capture(); ub.replay()  # CUDA graph

Tensors are single slices (image [ny, nx], sinogram [n_views, n_cols]) of
dtype float32 or bfloat16 (BF16 storage, FP32 arithmetic); input and output
of one item share the dtype.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .ops import FanPlan

OPS = {"fp": _lib.OP_FP, "bp": _lib.OP_BP, "fbp": _lib.OP_FBP,
       "fbp_adjoint": _lib.OP_FBP_ADJOINT}
DTYPES = {torch.float32: _lib.DTYPE_F32, torch.bfloat16: _lib.DTYPE_BF16}


class UnevenBatch:
    def __init__(self, items):
        if not 0 < len(items) <= _lib.BATCH_MAX_ITEMS:
            raise ValueError(f"1..{_lib.BATCH_MAX_ITEMS} items per batch")
        self._lib = _lib.load()
        self.items = list(items)
        arr = (_lib.CtBatchItem * len(items))()
        self.device = None
        for k, (plan, op, x, y) in enumerate(items):
            if not isinstance(plan, FanPlan) or plan.n_rows != 1 or plan.nz != 1:
                raise TypeError("uneven batches take fan-beam plans")
            if op not in OPS:
                raise ValueError(f"op must be one of {sorted(OPS)}")
            if x.dtype not in DTYPES or y.dtype != x.dtype:
                raise TypeError("input and output must both be float32 or both bfloat16")
            img_t, sino_t = tuple(plan.image_shape), tuple(plan.sino_shape)
            want_in, want_out = (img_t, sino_t) if op in ("fp", "fbp_adjoint") else (sino_t, img_t)
            if tuple(x.shape) != want_in or tuple(y.shape) != want_out:
                raise ValueError(f"item {k}: {op} takes {want_in} -> {want_out}")
            if not (x.is_contiguous() and y.is_contiguous()):
                raise ValueError(f"item {k}: tensors must be contiguous")
            if x.device != plan.device or y.device != plan.device:
                raise ValueError(f"item {k}: tensors must be on the plan's device")
            self.device = plan.device
            arr[k].plan = plan._h.value
            arr[k].op = OPS[op]
            arr[k].dtype = DTYPES[x.dtype]
            arr[k].d_in = x.data_ptr()
            arr[k].d_out = y.data_ptr()
        self._arr = arr
        n = ctypes.c_size_t()
        _lib.check(self._lib.ct_batch_workspace_size(arr, len(items), ctypes.byref(n)),
                   "ct_batch_workspace_size")
        self.work = torch.empty(max(1, n.value), dtype=torch.uint8, device=self.device)
        self.graph = None

    def run(self) -> None:
        with torch.cuda.device(self.device):
            st = self._lib.ct_batch_run(self._arr, len(self.items), self.work.data_ptr(),
                                        self.work.numel(),
                                        torch.cuda.current_stream(self.device).cuda_stream)
        _lib.check(st, "ct_batch_run")

    def tune(self, reps: int = 3) -> dict:
        """Times every candidate launch shape of the two persistent launches on
        this batch (outputs are overwritten) and keeps the fastest for this
        batch shape; later run() / capture() calls use it.  Returns it."""
        cfg = _lib.CtBatchConfig()
        with torch.cuda.device(self.device):
            st = self._lib.ct_batch_tune(self._arr, len(self.items), self.work.data_ptr(),
                                         self.work.numel(), int(reps),
                                         torch.cuda.current_stream(self.device).cuda_stream,
                                         ctypes.byref(cfg))
        _lib.check(st, "ct_batch_tune")
        return cfg.as_dict()

    @property
    def config(self) -> tuple[dict, bool]:
        """(launch shape run() uses, whether it was tuned or set)."""
        cfg, tuned = _lib.CtBatchConfig(), ctypes.c_int32()
        _lib.check(self._lib.ct_batch_get_config(self._arr, len(self.items), ctypes.byref(cfg),
                                                 ctypes.byref(tuned)), "ct_batch_get_config")
        return cfg.as_dict(), bool(tuned.value)

    def set_config(self, cfg: dict | None) -> None:
        """Records a launch shape for this batch shape (None forgets it)."""
        if cfg is None:
            st = self._lib.ct_batch_set_config(self._arr, len(self.items), None)
        else:
            c = _lib.CtBatchConfig(**cfg)
            st = self._lib.ct_batch_set_config(self._arr, len(self.items), ctypes.byref(c))
        _lib.check(st, "ct_batch_set_config")

    def capture(self) -> "torch.cuda.CUDAGraph":
        """Records one run() into a CUDA graph (after an eager warm-up run)."""
        self.run()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.device(self.device):
            s = torch.cuda.Stream(self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self.run()
            torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return g

    def replay(self) -> None:
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()
