"""The reference's drivers end to end on the GPU: the test.py command line
(raw image file -> FP / BP / FBP raw files) and the batched FDK
data-generation driver, against per-slice operator calls and the oracle."""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import cli, fdk_driver, phantom, utils
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
from fanbeamctrecon_tensorflowop_gb300.rawio import read_binary_dataset, write_raw
from golden.make_golden_fdk_driver import synthetic

pytestmark = pytest.mark.gpu


def test_cli_reproduces_test_py(cuda, tmp_path):
    ang, par, _, _ = utils._geometry(1)
    plan = FanPlan(par, ang, device=cuda)
    n = plan.geom.nx
    img = np.stack([phantom.ellipse_phantom(n, float(plan.geom.dx), seed=s) for s in (0, 1)])
    src = tmp_path / "test.fbp"
    write_raw(src, img.astype(np.float32))
    out = tmp_path / "out"
    assert cli.main(["test", "--input", str(src), "--out-dir", str(out), "--quiet"]) == 0
    V, C = plan.geom.n_views, plan.geom.n_cols
    sino = read_binary_dataset(out / "test_prj.raw", [V, C])
    bp = read_binary_dataset(out / "test_img_BP.raw", [n, n])
    fbp = read_binary_dataset(out / "test_img_FBP.raw", [n, n])
    assert sino.shape == (2, V, C) and bp.shape == (2, n, n) and fbp.shape == (2, n, n)
    x = torch.from_numpy(img.astype(np.float32)).to(cuda)
    want = plan.fp(x)
    assert rel_l2(sino, want.cpu().numpy()) <= 1e-6
    s = torch.from_numpy(sino).to(cuda)
    assert rel_l2(bp, plan.bp(s).cpu().numpy()) <= 1e-6
    assert rel_l2(fbp, plan.fbp(s).cpu().numpy()) <= 1e-6


def test_fdk_generate_batched_equals_per_slice_op(cuda, orc, tmp_path):
    index, fstart, nview, nslice = 3, 56.4605480091944, 48, 3
    data = tmp_path / "data"
    for ch, path in fdk_driver.exam_paths(data, "Training", index).items():
        os.makedirs(os.path.dirname(path), exist_ok=True)
        # smooth, sinogram-like values
        raw = synthetic(path, nslice, nview, 888)
        write_raw(path, np.sin(raw / 300.0).astype(np.float32) + 1.0)
    out = fdk_driver.fdk_generate(index, fstart, nview, nslice, data_root=data,
                                  save_root=tmp_path / "npy", recon_dir=tmp_path / "rec",
                                  chunk=4)
    par = fdk_driver.fdk_parameters(nview, nview)
    ang = fdk_driver.fdk_angles(fstart, nview)
    shift = fdk_driver.view_shift(fstart, nview)
    paths = fdk_driver.exam_paths(data, "Training", index)
    high = fdk_driver.roll_views(read_binary_dataset(paths["high"], nslice, nview, 888), shift)
    m1 = fdk_driver.roll_views(read_binary_dataset(paths["m1"], nslice, nview, 888), shift)
    for i in range(nslice):
        # the reference's per-slice call: BackProjection on [1, nview, ncol]
        a = high[i].reshape(1, nview, 888) / 49000
        ref = utils.back_projection(projection=a, angle=ang, parameter=par,
                                    vol_shape=[1, 512, 512], proj_shape=[1, nview, 888])
        assert rel_l2(out["high_rcn"][i], ref[0]) <= 1e-6
        b = m1[i].reshape(1, nview, 888)
        ref = utils.back_projection(projection=b, angle=ang, parameter=par,
                                    vol_shape=[1, 512, 512], proj_shape=[1, nview, 888])
        assert rel_l2(out["m1_rcn"][i], ref[0]) <= 1e-6
    g = orc.decode(par)
    o = orc.fdk_bp(g, ang, (high[0] / 49000)[None])[0]
    assert rel_l2(out["high_rcn"][0], o) <= 1e-4
    raw0 = np.fromfile(tmp_path / "rec" / "recon_0.raw", np.float32).reshape(512, 512)
    np.testing.assert_array_equal(raw0, out["high_rcn"][0])
    m = np.load(tmp_path / "npy" / "Training" / f"m_rcn_{index}_2.npy")
    np.testing.assert_array_equal(m[0, :, :, 0], out["m1_rcn"][1])
    np.testing.assert_array_equal(m[0, :, :, 1], out["m2_rcn"][1])
