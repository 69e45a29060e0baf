"""Batched FDK data generation: the reference's per-slice driver as one call.

FDK/FDK_test_training.py:18-141 (``FDK_generate``) reads five projection
files of an exam ([nslice, nview, ncol] float32: high, m1, m2, energy, mask),
rolls their views so that view 0 sits at the start angle, then reconstructs
the high / m1 / m2 sinograms slice by slice, one ``tf.Session`` per slice,
with the FDK library's ``BackProjection`` op, and saves the projections and
reconstructions as .npy files plus one .raw image per slice.

Here the reconstruction of all slices of all three channels is one batched
``ct_fdk_bp`` call per chunk (``FanPlan.fdk_bp``), and the files are written
with the reference's names, shapes and dtypes.  The view-roll and start-angle
handling follow the driver exactly, including its quirk of adding the start
angle, in degrees, to radian view angles (FDK/FDK_test_training.py:42,85-89).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np
import torch

from .ops import FanPlan
from .rawio import read_binary_dataset, write_raw


@dataclass(frozen=True)
class FdkScanner:
    """The driver's scanner constants (FDK/FDK_test_training.py:21-34,50)."""
    sdd: float = 946.73233346
    sod: float = 538.52
    ncol: int = 888
    nfan: float = 55.0059     # degrees
    nimg: int = 512
    dz: float = 2.5
    shift: float = 1.125
    d_left: float = -27.50295  # degrees
    det_bottom: float = -35.16105
    drow: float = 1.0987828125
    rfov: float = 250.0


SCANNER = FdkScanner()
CHANNELS = ("high", "m1", "m2", "energy", "mask")
HIGH_SCALE = 49000  # FDK/FDK_test_training.py:101: the high sinogram is divided by it


def fdk_parameters(nview: int, nview_full: int, scanner: FdkScanner = SCANNER) -> np.ndarray:
    """The 16-float parameter vector of FDK/FDK_test_training.py:61-77."""
    p = np.arange(16, dtype=np.float32)
    p[0] = scanner.sdd
    p[1] = scanner.sod
    p[2] = nview
    p[3] = nview * 360 / nview_full
    p[4] = scanner.ncol
    p[5] = scanner.nimg
    p[6] = scanner.nimg
    p[7] = scanner.rfov
    p[8] = scanner.nfan / scanner.ncol
    p[9] = scanner.shift
    p[10] = scanner.d_left
    p[11] = 1
    p[12] = 0
    p[13] = scanner.det_bottom
    p[14] = scanner.drow
    p[15] = scanner.dz
    return p


def fdk_angles(fstart_angle: float, nview: int) -> np.ndarray:
    """float32 view angles -fstart_angle + i * 2 pi / nview
    (FDK/FDK_test_training.py:42,80-84; the degrees are added to radians)."""
    start = -fstart_angle
    d_angle = 2.0 * math.pi / nview
    a = np.arange(nview, dtype=np.float32)
    for i in range(nview):
        a[i] = start + i * d_angle
    return a


def view_shift(fstart_angle: float, nview: int) -> int:
    """int(round(-fstart_angle / (360 / nview))) (FDK/FDK_test_training.py:42-43);
    Python's round, so halves go to the even neighbour."""
    return int(round(-fstart_angle / (360 / nview)))


def roll_views(proj: np.ndarray, shift: int) -> np.ndarray:
    """concatenate(proj[:, shift:], proj[:, :shift]) along the view axis
    (FDK/FDK_test_training.py:88-92)."""
    return np.concatenate((proj[:, shift:proj.shape[1], :], proj[:, 0:shift, :]), axis=1)


def fdk_reconstruct(sinos: np.ndarray, parameter, angles, device=None,
                    chunk: int = 96) -> np.ndarray:
    """FDK-op reconstructions [S, nimg, nimg] of sinograms [S, nview, ncol],
    ``chunk`` slices per ct_fdk_bp call."""
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    plan = FanPlan(parameter, angles, device=device)
    try:
        s = sinos.shape[0]
        out = np.empty((s, *plan.image_shape), np.float32)
        host = torch.empty((min(chunk, s), *plan.image_shape), dtype=torch.float32,
                           pin_memory=True)
        for b0 in range(0, s, chunk):
            b1 = min(s, b0 + chunk)
            x = torch.from_numpy(np.ascontiguousarray(sinos[b0:b1], np.float32)).to(
                plan.device, non_blocking=True)
            y = plan.fdk_bp(x)
            h = host[: b1 - b0]
            h.copy_(y, non_blocking=True)
            torch.cuda.current_stream(plan.device).synchronize()
            out[b0:b1] = h.numpy()
        return out
    finally:
        plan.close()


def exam_paths(data_root, folder: str, index: int) -> dict:
    """{channel: path} of an exam's projection files (FDK/FDK_test_training.py:46-50)."""
    return {c: os.path.join(data_root, folder, f"exam{index}_{c}.prj") for c in CHANNELS}


def fdk_generate(index: int, fstart_angle: float, nview_full: int, nslice: int,
                 folder: str = "Training", data_root=".", save_root=".",
                 recon_dir="./recon_images", device=None, chunk: int = 96,
                 scanner: FdkScanner = SCANNER, save: bool = True) -> dict:
    """FDK_generate (FDK/FDK_test_training.py:18-141) with one batched
    reconstruction.  Returns {"high_rcn", "m1_rcn", "m2_rcn"} ([nslice, nimg,
    nimg] float32) and the list of slice ids; with ``save`` writes the
    reference's files:

      {save_root}/{folder}/{high,m1,m2,eff,mask}_prj_{index}_{i+1}.npy  [1, nview*ncol, 1]
      {save_root}/{folder}/high_rcn_{index}_{i+1}.npy                  [1, nimg, nimg, 1]
      {save_root}/{folder}/m_rcn_{index}_{i+1}.npy                     [1, nimg, nimg, 2]
      {recon_dir}/recon_{i}.raw                                        the high image
    """
    nview, ncol = nview_full, scanner.ncol
    shift = view_shift(fstart_angle, nview)
    parameter = fdk_parameters(nview, nview_full, scanner)
    angles = fdk_angles(fstart_angle, nview)
    paths = exam_paths(data_root, folder, index)
    proj = {c: roll_views(read_binary_dataset(paths[c], nslice, nview, ncol), shift)
            for c in CHANNELS}
    proj["high"] = proj["high"] / HIGH_SCALE
    # high, m1 and m2 of every slice in one batch
    stacked = np.concatenate([proj["high"], proj["m1"], proj["m2"]], axis=0)
    rec = fdk_reconstruct(stacked, parameter, angles, device=device, chunk=chunk)
    nimg = scanner.nimg
    out = {"high_rcn": rec[:nslice], "m1_rcn": rec[nslice:2 * nslice],
           "m2_rcn": rec[2 * nslice:]}
    ids = [f"{index}_{i + 1}" for i in range(nslice)]
    out["index_data"] = ids
    if save:
        savepath = os.path.join(save_root, folder)
        os.makedirs(savepath, exist_ok=True)
        prj_names = (("high", "high_prj_"), ("m1", "m1_prj_"), ("m2", "m2_prj_"),
                     ("energy", "eff_prj_"), ("mask", "mask_prj_"))
        for i, idx in enumerate(ids):
            for c, stem in prj_names:
                np.save(os.path.join(savepath, stem + idx + ".npy"),
                        proj[c][i].reshape(1, nview * ncol, 1))
            a_ = out["high_rcn"][i]
            np.save(os.path.join(savepath, "high_rcn_" + idx + ".npy"),
                    a_.reshape(1, nimg, nimg, 1))
            m_ = np.concatenate((out["m1_rcn"][i].reshape(1, nimg, nimg, 1),
                                 out["m2_rcn"][i].reshape(1, nimg, nimg, 1)), axis=-1)
            np.save(os.path.join(savepath, "m_rcn_" + idx + ".npy"), m_)
            write_raw(os.path.join(recon_dir, f"recon_{i}.raw"), a_)
    return out
