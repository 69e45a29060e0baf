"""Geometries of the parity tests, as 16-float parameter vectors + angles."""
from __future__ import annotations

import math

import numpy as np

from fanbeamctrecon_tensorflowop_gb300.geometry import angle, fan_param16

SID, SDD = 541.0, 949.0
DCOL = 1.0 / 949.0  # 1 mm channel pitch at the detector, in rad


def small(n=64, views=90, cols=96, pixel=2.8, shift=0.0, ny=None, full=360.0, batch=1):
    """A small fan geometry whose detector covers the FOV."""
    p = fan_param16(sdd=SDD, sid=SID, n_views=views, n_cols=cols, n=n, pixel_mm=pixel,
                    dcol_rad=4.0 * DCOL, shift=shift, ny=ny, full_angle=full, batch=batch)
    return p, angle(views, 0.0)


def config0():
    """256^2 at 1 mm, 720 views x 512 channels (the CPU-runnable workload)."""
    p = fan_param16(sdd=SDD, sid=SID, n_views=720, n_cols=512, n=256, pixel_mm=1.0,
                    dcol_rad=DCOL)
    return p, angle(720, 0.0)


def config1():
    """512^2 at 0.7 mm, 984 views x 888 channels (the clinical-scale workload)."""
    p = fan_param16(sdd=SDD, sid=SID, n_views=984, n_cols=888, n=512, pixel_mm=0.7,
                    dcol_rad=DCOL)
    return p, angle(984, 0.0)


def fdk_driver(nview=96, ncol=888, nimg=64):
    """The FDK driver's geometry (FDK/FDK_test_training.py:20-77) at reduced
    view count / image size: SDD 946.73233346, SAD 538.52, 888 channels of
    55.0059/888 deg, shift 1.125, left -27.50295 deg, rFOV 250, det_bottom
    -35.16105, drow 1.0987828125, dz 2.5."""
    p = np.arange(16, dtype=np.float32)
    p[0] = 946.73233346
    p[1] = 538.52
    p[2] = nview
    p[3] = nview * 360 / nview
    p[4] = ncol
    p[5] = nimg
    p[6] = nimg
    p[7] = 250
    p[8] = 55.0059 / ncol
    p[9] = 1.125
    p[10] = -27.50295
    p[11] = 1
    p[12] = 0
    p[13] = -35.16105
    p[14] = 1.0987828125
    p[15] = 2.5
    a = (np.arange(nview) * (2.0 * math.pi / nview)).astype(np.float32)
    return p, a


def cone_small(n=32, views=48, cols=64, n_rows=12, nz=10, pixel=5.6, dz=3.0, drow=6.0):
    """A small cone geometry whose detector covers the volume in z:
    |z| <= nz*dz/2 magnifies by at most D/(R - rFOV) onto rows of height drow."""
    p = fan_param16(sdd=SDD, sid=SID, n_views=views, n_cols=cols, n=n, pixel_mm=pixel,
                    dcol_rad=4.0 * DCOL, det_bottom=-n_rows * drow / 2.0, drow=drow, dz=dz)
    return p, angle(views, 0.0), n_rows, nz


def config4(views=984, cols=888, n_rows=64, nz=64, n=512):
    """Clinical cone geometry: 984 views, 888 x 64 detector (1 mm rows at the
    detector, bottom -32 mm), 512^2 x 64 voxels of 0.7 x 0.7 x 0.625 mm."""
    p = fan_param16(sdd=SDD, sid=SID, n_views=views, n_cols=cols, n=n, pixel_mm=0.7,
                    dcol_rad=DCOL, det_bottom=-n_rows / 2.0, drow=1.0, dz=0.625)
    return p, angle(views, 0.0), n_rows, nz


UNEVEN = [(256, 492, 512), (384, 720, 736), (512, 984, 888)]


def uneven(k, scale=1):
    """The k-th geometry of the uneven workload (cycling image 256^2 / 384^2 /
    512^2, views 492 / 720 / 984, channels 512 / 736 / 888), pixel pitch chosen
    so that rFOV = 179.2 mm for every size; scale > 1 shrinks all three sizes."""
    n, v, c = UNEVEN[k % 3]
    n, v, c = n // scale, v // scale, c // scale // 4 * 4
    pix = 358.4 / n
    dcol = DCOL * (888 / c) if scale > 1 else DCOL
    p = fan_param16(sdd=SDD, sid=SID, n_views=v, n_cols=c, n=n, pixel_mm=pix, dcol_rad=dcol)
    return p, angle(v, 0.0)


def short_scan(n=128, views=200, cols=320, pixel=2.0, dcol=1.5 * DCOL, start=0.3,
               reverse=False, shift=0.0, **kw):
    """A short scan: views evenly over pi + 2*Gamma (Gamma = the half fan
    angle to the outer channel edge), both ends included; parameter[3] makes
    the decoded angle step equal the view spacing."""
    half_fan = cols * dcol / 2.0 + abs(shift) * dcol
    step = (math.pi + 2.0 * half_fan) / (views - 1)
    p = fan_param16(sdd=SDD, sid=SID, n_views=views, n_cols=cols, n=n, pixel_mm=pixel,
                    dcol_rad=dcol, full_angle=math.degrees(step * views), shift=shift, **kw)
    a = (start + np.arange(views) * step).astype(np.float32)
    return p, (a[::-1].copy() if reverse else a)
