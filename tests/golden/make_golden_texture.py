"""Generates tests/golden/texture_unit_gb300.npz: fetches through a real GPU
texture object with the reference's sampler state (texture_probe.cu), on a
GB300.  The CPU tests hold the texture-unit rule of oracle/texture_rule.h
against these measured values.

Fetches (seeded numpy default_rng(2024)):

* ``sweep``: a 1-D row {0, 1} sampled at x = 1/2 + k/65536, k = 0..65536,
  which returns the quantised weight itself (ties included);
* ``t1``/``x1``/``o1``: a 1-D row of 1024 texels in U[-1, 1), 8192 fetches
  at x in [-2, 1028) (both clamp zones included);
* ``t2``/``x2``/``y2``/``o2``: a 48 x 64 image in U[-1, 1), 8192 fetches at
  x in [-1, 65), y in [-1, 49).

usage (on a machine with the GPU): python tests/golden/make_golden_texture.py [out.npz]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402


def inputs() -> dict:
    rng = np.random.default_rng(2024)
    d = {}
    d["sweep_x"] = (0.5 + np.arange(65537) / 65536.0).astype(np.float32)
    d["t1"] = rng.uniform(-1, 1, 1024).astype(np.float32)
    d["x1"] = rng.uniform(-2, 1028, 8192).astype(np.float32)
    d["t2"] = rng.uniform(-1, 1, (48, 64)).astype(np.float32)
    d["x2"] = rng.uniform(-1, 65, 8192).astype(np.float32)
    d["y2"] = rng.uniform(-1, 49, 8192).astype(np.float32)
    return d


def measure(d: dict) -> dict:
    out = dict(d)
    out["sweep"] = oracle.texture_probe_fetch(np.array([0.0, 1.0], np.float32), d["sweep_x"])
    out["o1"] = oracle.texture_probe_fetch(d["t1"], d["x1"])
    out["o2"] = oracle.texture_probe_fetch(d["t2"], d["x2"], d["y2"])
    return out


def main(path: Path) -> None:
    out = measure(inputs())
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else HERE / "texture_unit_gb300.npz")
