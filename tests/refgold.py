"""The golden vectors of the executed reference (tests/golden/reference_ops.npz,
made by tests/golden/make_golden_reference_ops.py) and how the library's
outputs are compared with them."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLD = Path(__file__).resolve().parent / "golden"
Z = np.load(GOLD / "reference_ops.npz")
CASES = sorted({k.split("/")[0] for k in Z.files})
OPS = ("fp", "bp", "fbp", "fdk", "bp_noise")

# relative L2 against the executed reference: the oracle with the texture
# unit's weights, and any exact-weight implementation (the oracle's exact mode
# and the CUDA kernels), whose distance is the reference's 8-bit weights
TEX_TOL = {"fp": 5e-6, "bp": 5e-6, "bp_noise": 5e-5, "fbp": 1e-4, "fdk": 1e-4}
EXACT_TOL = {"fp": 5e-5, "bp": 2e-5, "bp_noise": 2e-4, "fbp": 3e-4, "fdk": 3e-4}


def gold(case, key):
    return Z[f"{case}/{key}"]


def shapes(case):
    vs = [int(v) for v in gold(case, "vol_shape")]
    ps = [int(v) for v in gold(case, "proj_shape")]
    return vs, ps


def reference_view(case: str, op: str, out) -> np.ndarray:
    """A full output as the reference would leave it: its BP and FBP grids
    cover floor(N/32)*32 pixels per axis (BP/transform.cu:103,
    FBP/transform.cu:97) and its FDK op reconstructs only the first slice
    (FDK/GPURecon_GPU.cu:177-179)."""
    out = np.array(out, dtype=np.float64, copy=True)
    nx = int(gold(case, "vol_shape")[1])
    if op in ("bp", "fbp", "bp_noise") and nx % 32:
        cover = nx // 32 * 32
        mask = np.zeros(out.shape[1:], bool)
        mask[:cover, :cover] = True
        out[:, ~mask] = 0.0
    if op == "fdk":
        out[1:] = 0.0
    return out
