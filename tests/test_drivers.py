"""The reference's drivers on this package (CPU parts): raw-file I/O of
test.py and FDK/FDK_test_training.py, and the batched FDK data-generation
driver against the golden record of the reference driver executed with
recording stand-ins (tests/golden/make_golden_fdk_driver.py)."""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

from fanbeamctrecon_tensorflowop_gb300 import cli, fdk_driver
from fanbeamctrecon_tensorflowop_gb300.rawio import read_binary_dataset, write_raw
from golden.make_golden_fdk_driver import synthetic

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" /
                     "reference_fdk_driver.json").read_text())


def test_raw_round_trip_both_signatures(tmp_path):
    a = np.random.default_rng(0).standard_normal((3, 5, 7)).astype(np.float32)
    f = tmp_path / "x.raw"
    assert write_raw(f, a) == a.nbytes
    assert f.stat().st_size == a.nbytes
    np.testing.assert_array_equal(read_binary_dataset(f, [5, 7]), a)
    np.testing.assert_array_equal(read_binary_dataset(f, 3, 5, 7), a)
    # test.py's reshape (-1, H, W): the slice count comes from the file size
    assert read_binary_dataset(f, [7, 5]).shape == (3, 7, 5)
    with pytest.raises(ValueError):
        read_binary_dataset(f, [4, 4])
    with pytest.raises(ValueError):
        read_binary_dataset(f, 2, 5, 7)
    # bytearray(ndarray) of the drivers == C-order bytes
    assert bytes(bytearray(a)) == f.read_bytes()


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: str(c["fstart_angle"]))
def test_fdk_driver_geometry_matches_reference(case):
    nview = case["nview_full"]
    p = fdk_driver.fdk_parameters(nview, nview)
    np.testing.assert_array_equal(p, np.asarray(case["parameter"], np.float32))
    a = fdk_driver.fdk_angles(case["fstart_angle"], nview)
    np.testing.assert_array_equal(a, np.asarray(case["angle"], np.float32))
    assert fdk_driver.view_shift(case["fstart_angle"], nview) == int(case["printed_shift"])
    assert case["vol_shape"] == [1, 512, 512] and case["proj_shape"] == [1, nview, 888]


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: str(c["fstart_angle"]))
def test_fdk_generate_inputs_and_files_match_reference(case, tmp_path, monkeypatch):
    """Runs fdk_generate on the golden run's synthetic exam with the
    reconstruction replaced by zeros (the GPU part is checked in the gpu tests):
    the sinograms handed to the FDK op and every saved file agree."""
    nview, nslice, index = case["nview_full"], case["nslice"], case["index"]
    data = tmp_path / "data"
    for ch, path in fdk_driver.exam_paths(data, "Training", index).items():
        os.makedirs(os.path.dirname(path), exist_ok=True)
        write_raw(path, synthetic(path, nslice, nview, 888))
    seen = {}

    def fake_reconstruct(sinos, parameter, angles, device=None, chunk=96):
        seen["sinos"] = np.array(sinos, copy=True)
        seen["parameter"], seen["angles"] = parameter, angles
        return np.zeros((sinos.shape[0], 512, 512), np.float32)

    monkeypatch.setattr(fdk_driver, "fdk_reconstruct", fake_reconstruct)
    recon = tmp_path / "recon_images"
    out = fdk_driver.fdk_generate(index, case["fstart_angle"], nview, nslice, folder="Training",
                                  data_root=data, save_root=tmp_path / "npy", recon_dir=recon)
    s = seen["sinos"]
    assert s.shape == (3 * nslice, nview, 888)  # high, m1, m2 of every slice in one batch
    order = [int(round(float(x) * 49000.0)) for x in s[0, :, 0]]
    assert order == case["view_order"]
    assert float(s[0, 1, 1]) == case["high_first"]
    for i in range(nslice):
        got = [float(s[k * nslice + i].astype(np.float64).sum()) for k in range(3)]
        np.testing.assert_allclose(got, case["projection_sums"][i], rtol=1e-12)
    np.testing.assert_array_equal(seen["angles"], np.asarray(case["angle"], np.float32))
    assert out["index_data"] == [f"{index}_{i + 1}" for i in range(nslice)]
    saved = sorted(os.listdir(tmp_path / "npy" / "Training"))
    assert saved == sorted(r["name"] for r in case["saves"])
    for r in case["saves"]:
        arr = np.load(tmp_path / "npy" / "Training" / r["name"])
        assert list(arr.shape) == r["shape"] and str(arr.dtype) == r["dtype"], r["name"]
        assert float(arr.astype(np.float64).sum()) == pytest.approx(r["sum"], rel=1e-12)
    raws = sorted(os.listdir(recon))
    assert raws == sorted(os.path.basename(r["name"]) for r in case["raws"])
    assert all((recon / os.path.basename(r["name"])).stat().st_size == r["bytes"]
               for r in case["raws"])


def test_roll_views_is_a_rotation():
    x = np.arange(2 * 7 * 3, dtype=np.float32).reshape(2, 7, 3)
    for s in (-6, -1, 0, 1, 3, 6):
        np.testing.assert_array_equal(fdk_driver.roll_views(x, s), np.roll(x, -s, axis=1))


def test_cli_parser():
    ap = cli.build_parser()
    a = ap.parse_args(["test", "--input", "in.fbp", "--out-dir", "o", "--dim", "256", "256"])
    assert a.func is cli._cmd_test and a.dim == [256, 256] and a.out_dir == "o"
    a = ap.parse_args(["fdk-generate", "--index", "42", "--start-angle", "-12.5", "--nview",
                       "1968", "--nslice", "147"])
    assert a.func is cli._cmd_fdk and a.start_angle == -12.5 and a.folder == "Training"
    with pytest.raises(SystemExit):
        ap.parse_args(["fdk-generate", "--index", "1"])
