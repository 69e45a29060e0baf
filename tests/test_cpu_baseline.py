"""The FP32 OpenMP transcription of the reference (oracle/cpu_fp32.c), which
the benchmark times as its CPU baseline, computes the same operators as the
FP64 oracle: FP (FP/transform.cu:64-146), pixel-driven BP
(BP/transform.cu:67-95) and Ram-Lak FBP (FBP/transform.cu:149-174, 61-89).
CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import phantom
import geometries as G


@pytest.fixture(scope="module")
def cpu():
    from oracle import cpu
    cpu.build()
    return cpu


@pytest.mark.parametrize("geom", ["small", "shifted", "config0"])
def test_fp32_transcription_matches_oracle(orc, cpu, geom):
    if geom == "small":
        p, a = G.small()
    elif geom == "shifted":
        p, a = G.small(n=48, views=60, cols=80, shift=1.25)
    else:
        p, a = G.config0()
    g = orc.decode(p)
    img = phantom.ellipse_phantom(g.nx, 2 * g.rfov / g.nx, seed=2)
    sino = np.random.default_rng(1).random((g.n_views, g.n_cols)).astype(np.float32)
    assert rel_l2(cpu.fp_fan(g, a, img)[0], orc.fp_fan(g, a, img)[0]) < 5e-5
    assert rel_l2(cpu.bp_fan(g, a, sino)[0], orc.bp_fan(g, a, sino)[0]) < 1e-5
    assert rel_l2(cpu.bp_fan(g, a, sino, weighted=True)[0],
                  orc.bp_fan(g, a, sino, weighted=True)[0]) < 1e-5
    assert rel_l2(cpu.fbp_fan(g, a, sino)[0], orc.fbp_fan(g, a, sino)[0]) < 1e-4


def test_view_subsets_and_timing(orc, cpu):
    """A run over every k-th view projects exactly those views; the timing
    helper reports positive rates."""
    p, a = G.small()
    g = orc.decode(p)
    img = phantom.ellipse_phantom(g.nx, 2 * g.rfov / g.nx, seed=0)
    full = cpu.fp_fan(g, a, img)[0]
    part = cpu.fp_fan(g, a, img, view0=30, n_views=20)[0]
    np.testing.assert_array_equal(part, full[30:50])
    r = cpu.time_ops(g, a, img, np.ones((g.n_views, g.n_cols), np.float32), 15)
    assert r["views_timed"] == 15 and r["threads"] >= 1
    assert r["fp_grays_per_s"] > 0 and r["bp_gpix_views_per_s"] > 0 and r["fbp_ms_per_slice"] > 0
