"""Generates tests/golden/reference_ops.npz by EXECUTING the reference's own
ops: each op's TensorFlow wrapper and CUDA source (FP/transform.{cc,cu},
BP/..., FBP/..., FDK/FBP.cc + FDK/GPURecon_GPU.cu), compiled from a checkout
of FanBeamCTRecon_TensorflowOp against host stand-ins by oracle/build_ref.py
and run on the CPU (oracle/reference.py).  The kernels run as written; the
texture unit's linear filter follows the rule measured on GB300
(oracle/texture_rule.h).

Cases (all inputs seeded; the phantom is the package's ellipse rasteriser):

* ``small``: 64^2 at 2.8 mm, 90 views x 96 channels of 4/949 rad.  FP of a
  phantom; BP, FBP and the FDK library's BackProjection of that FP output;
  BP of a U[0,1) sinogram.
* ``shift``: 64^2, 72 views x 100 channels, detector shift 1.5 channels.
* ``fdk_driver``: the FDK driver's geometry (FDK/FDK_test_training.py:20-77:
  888 channels, shift 1.125, left -27.50295 deg, rFOV 250) at 96 views and
  64^2.
* ``batch2``: ``small`` with two slices (parameter[11] = 2): the slice loops
  of FP, BP and FBP, and the FDK op's single-slice reconstruction (it copies
  and filters only the first nViews x nCols block,
  FDK/GPURecon_GPU.cu:177-179, and leaves the other output slices as
  allocated: zero here).
* ``n48``: 48^2: records that the reference's BP grid covers only
  floor(N/32)*32 pixels per axis (BP/transform.cu:103).

Every array is float32.  Keys: ``<case>/parameter``, ``/angle``,
``/vol_shape``, ``/proj_shape``, ``/image``, ``/fp``, ``/bp``, ``/fbp``,
``/fdk``, ``/noise``, ``/bp_noise``; ``<case>/shape_<op>`` holds the op's
registered shape function output for the case's input.

usage: python tests/golden/make_golden_reference_ops.py [/path/to/reference]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(HERE.parent))

import geometries as G  # noqa: E402
from fanbeamctrecon_tensorflowop_gb300 import phantom  # noqa: E402
from oracle import build_ref, reference  # noqa: E402
import oracle  # noqa: E402


def _phantoms(g, n, seed):
    out = []
    for b in range(n):
        ell = phantom.random_ellipses(float(g.rfov), seed + b)
        out.append(phantom.rasterize(ell, g.nx, g.ny, float(g.dx), float(g.dy)))
    return np.stack(out).astype(np.float32)


CASES = {
    "small": (lambda: G.small(), 1),
    "shift": (lambda: G.small(n=64, shift=1.5, views=72, cols=100), 1),
    "fdk_driver": (lambda: G.fdk_driver(nview=96, ncol=888, nimg=64), 1),
    "batch2": (lambda: G.small(batch=2), 2),
    "n48": (lambda: G.small(n=48, pixel=3.7), 1),
}


def make_case(name: str) -> dict:
    geom, batch = CASES[name]
    p, a = geom()
    g = oracle.decode(p)
    vs = [batch, g.nx, g.ny]
    ps = [batch, g.n_views, g.n_cols]
    img = _phantoms(g, batch, seed=0)
    fp = reference.run("fp", p, a, vs, ps, img)
    out = {"parameter": np.asarray(p, np.float32), "angle": np.asarray(a, np.float32),
           "vol_shape": np.asarray(vs, np.float32), "proj_shape": np.asarray(ps, np.float32),
           "image": img, "fp": fp}
    for op in ("bp", "fbp", "fdk"):
        out[op] = reference.run(op, p, a, vs, ps, fp)
    noise = np.random.default_rng(1).uniform(0, 1, ps).astype(np.float32)
    out["noise"] = noise
    out["bp_noise"] = reference.run("bp", p, a, vs, ps, noise)
    for op in ("fp", "bp", "fbp", "fdk"):
        ins = vs if op == "fp" else ps
        out[f"shape_{op}"] = np.asarray(reference.shape(op, ins, vs, ps), np.float32)
    return out


def main(ref: Path | None) -> None:
    if build_ref.build(ref) is None:
        raise SystemExit("the reference's sources were not found")
    oracle.build()
    arrays = {}
    for name in CASES:
        for k, v in make_case(name).items():
            arrays[f"{name}/{k}"] = v
        print("case", name, "done", flush=True)
    path = HERE / "reference_ops.npz"
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({path.stat().st_size} bytes)")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else None)
