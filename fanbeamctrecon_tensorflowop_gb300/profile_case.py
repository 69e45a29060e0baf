"""Runs one operator on the clinical-scale geometry a few times, for profilers.

    python -m fanbeamctrecon_tensorflowop_gb300.profile_case --op fp --batch 8 --iters 3

Geometry: 512x512 at 0.7 mm, 984 views x 888 channels (1 mm pitch at the
detector), SID 541 / SDD 949 mm.  One untimed warm-up call precedes the
``iters`` profiled calls, so ``ncu -s <launches of one call>`` skips it.
Ops: fp, fp_adjoint, bp, bp_adjoint, filter, fbp, fbp_adjoint; cone_fp, fdk and
fdk_adjoint take ``--batch`` volumes of 512^2 x 64 voxels (0.7 x 0.7 x 0.625 mm) with
888 x 64 detector cells (1 mm rows) per view.
"""
from __future__ import annotations

import argparse

import numpy as np
import torch

from . import _lib, phantom
from .geometry import angle, fan_param16
from .ops import ConePlan, FanPlan


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="fp")
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--views", type=int, default=984)
    ap.add_argument("--cols", type=int, default=888)
    ap.add_argument("--pixel", type=float, default=0.7)
    ap.add_argument("--window", default="ramlak", choices=["ramlak", "shepp_logan"])
    args = ap.parse_args()
    dev = torch.device("cuda", 0)
    p = fan_param16(sdd=949.0, sid=541.0, n_views=args.views, n_cols=args.cols, n=args.n,
                    pixel_mm=args.pixel, dcol_rad=1.0 / 949.0)
    a = angle(args.views, 0.0)
    win = _lib.WINDOW_RAMLAK if args.window == "ramlak" else _lib.WINDOW_SHEPP_LOGAN
    if args.op in ("cone_fp", "fdk", "fdk_adjoint"):
        n_rows = nz = 64
        pc = fan_param16(sdd=949.0, sid=541.0, n_views=args.views, n_cols=args.cols, n=args.n,
                         pixel_mm=args.pixel, dcol_rad=1.0 / 949.0, det_bottom=-n_rows / 2.0,
                         drow=1.0, dz=0.625)
        cplan = ConePlan(pc, angle(args.views, 0.0), n_rows, nz, device=dev)
        vol = torch.rand((args.batch, nz, args.n, args.n), device=dev)
        proj = cplan.fp_cone(vol)
        fn = {"cone_fp": lambda: cplan.fp_cone(vol, out=proj),
              "fdk": lambda: cplan.fdk(proj),
              "fdk_adjoint": lambda: cplan.fdk_adjoint(vol)}[args.op]
        fn()
        torch.cuda.synchronize()
        for _ in range(args.iters):
            fn()
        torch.cuda.synchronize()
        print(f"profile_case {args.op} batch={args.batch} ok")
        return
    plan = FanPlan(p, a, device=dev, window=win)
    img = torch.from_numpy(np.stack([phantom.ellipse_phantom(args.n, args.pixel, seed=s)
                                     for s in range(args.batch)])).to(dev)
    sino = plan.fp(img)
    fns = {
        "fp": lambda: plan.fp(img),
        "fp_adjoint": lambda: plan.fp_adjoint(sino),
        "bp": lambda: plan.bp(sino),
        "bp_adjoint": lambda: plan.bp_adjoint(img),
        "filter": lambda: plan.ramp_filter(sino),
        "fbp": lambda: plan.fbp(sino),
        "fbp_adjoint": lambda: plan.fbp_adjoint(img),
    }
    fn = fns[args.op]
    fn()
    torch.cuda.synchronize()
    for _ in range(args.iters):
        fn()
    torch.cuda.synchronize()
    print(f"profile_case {args.op} batch={args.batch} ok")


if __name__ == "__main__":
    main()
