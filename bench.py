"""Benchmark of the fan-beam CT operators on GB300.

Headline (``value``): forward-projection throughput in G rays/s on the
clinical-scale geometry -- 512x512 slices at 0.7 mm, 984 views x 888
equiangular channels (1 mm pitch at the detector), SID 541 / SDD 949 mm --
one step = FP of a batch of 32 seeded ellipse phantoms resident in HBM.
Inputs rotate over 4 batches (576 MB of images + sinograms, > the 129 MB L2).

Also reported: ``e2e`` (the same FP through the reference-named Python entry
point ``utils.fp_fan_curve`` with host numpy buffers, host<->device copies
inside the timed region), BP throughput (G pixel-views/s, U[0,1)
sinograms), Shepp-Logan FBP time, the batch-32 FP + adjoint step against the
plain per-view launch loop on the same GPU, cone beam and uneven batches.

Roofline: the interpolation kernels are bound by the L1 data path (their
gathers hit L1), so ``roofline`` sets the forward projector's algorithmic L1
load bytes -- one 16-byte quad per (ray, cell) visit and slice -- against the
L1 load peak that ``csrc/peaks`` measures in this same run (the faster of
coalesced 16- and 32-byte loads); the compulsory and the measured DRAM
traffic are reported beside it.

``cpu_baseline`` and ``--impl reference`` time the reference's algorithms on
the host cores as an FP32 OpenMP transcription (oracle/cpu_fp32.c).  The
reference's ops cannot be built for the GPU (CUDA 13 rejects texture
references; TensorFlow and IPP are absent).  The same leg checks every
output against the FP64 oracle (``errors``), outside all timed regions.

``--profile-case OP`` runs one operator a few times for a profiler (see
``profile_case``).

Multi-GPU: ``torchrun --nproc-per-node N bench.py --gpus N``: every rank runs
its own batch (replicas, no collective on the data path); the step time is
the max over ranks and ``value`` counts the rays of all ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = ("FP Grays/s, BP Gpix-views/s @512²×984 views; "
          "batch-32 fwd+adjoint ms vs plain")
SID, SDD = 541.0, 949.0
N_PIX, PIXEL_MM, VIEWS, COLS = 512, 0.7, 984, 888
DCOL = 1.0 / 949.0
BATCH = 32
POOL = 4
WORKLOAD = ("fan-beam FP, batch of 32 seeded ellipse phantoms 512x512 @0.7 mm, "
            "984 views x 888 equiangular channels (1 mm pitch), SID 541 / SDD 949 mm")
QUAD_BYTES = 16      # FP: one float4 of four clamped taps per (ray, cell) visit and slice
TAP_BYTES = 8        # BP: two FP32 taps per pixel-view and slice (a 32-byte entry per 4 slices)
SINO_BYTES = 4       # FP adjoint: one FP32 sinogram value per (cell, ray) pair and slice
FMA_FLOP_PER_VISIT = 8  # FP: per visit and slice, two f32x2 FMAs (w . taps)
L1_PEAK_SOURCE = ("measured in this run (csrc/peaks): the larger of the coalesced 16-byte and "
                  "32-byte L1-hit load rates (peaks.l1_load_gbs, peaks.l1_load32_gbs)")


def c1_geometry():
    from fanbeamctrecon_tensorflowop_gb300.geometry import angle, fan_param16
    p = fan_param16(sdd=SDD, sid=SID, n_views=VIEWS, n_cols=COLS, n=N_PIX, pixel_mm=PIXEL_MM,
                    dcol_rad=DCOL)
    return p, angle(VIEWS, 0.0)


def measured_peaks() -> dict:
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profiled(kernel: str, key: str) -> float | None:
    """A per-launch figure of `kernel` at this workload from the ncu summary
    committed under profiles/ (lines 'kernel=<name> <key>=<value> ...')."""
    f = REPO / "profiles" / "traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("#"):
            continue
        parts = dict(kv.split("=", 1) for kv in line.split() if "=" in kv)
        if parts.get("kernel") == kernel and key in parts:
            return float(parts[key])
    return None


def fp_cell_visits(param16, angles) -> int:
    """(ray, cell) visits of one FP slice: for each ray, the bilinear cells its
    samples cross, 1 + |floor(u_last) - floor(u_first)| + |floor(v_last) -
    floor(v_first)| in cell coordinates (texture coordinates - 1/2), from the
    library's FP64 ray table.  The kernel gathers one quad per visit."""
    from fanbeamctrecon_tensorflowop_gb300.geometry import ray_table
    ray, ns = ray_table(param16, angles)
    r = ray.reshape(-1, 4).astype(np.float64)
    n = ns.reshape(-1).astype(np.float64)
    ok = n > 0
    u0, v0 = r[ok, 0] - 0.5, r[ok, 1] - 0.5
    u1 = u0 + (n[ok] - 1.0) * r[ok, 2]
    v1 = v0 + (n[ok] - 1.0) * r[ok, 3]
    return int(np.sum(1 + np.abs(np.floor(u1) - np.floor(u0)) + np.abs(np.floor(v1) - np.floor(v0))))


def fov_pixels(nx: int, ny: int, xmin: float, ymin: float, dx: float, dy: float, rfov: float) -> int:
    """Pixels whose centre lies inside the FOV disc (the backprojectors' own
    double-precision test)."""
    x = xmin + dx * (np.arange(nx) + 0.5)
    y = ymin + dy * (np.arange(ny) + 0.5)
    return int(np.count_nonzero(x[None, :] ** 2 + y[:, None] ** 2 <= float(rfov) * float(rfov)))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu_index: int):
        self.rows: list[list[str]] = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        for r in self.rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, val in zip(self.REASONS, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_index_for_smi(local_rank: int) -> int:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v.strip() for v in vis.split(",") if v.strip()]
    if ids and all(i.isdigit() for i in ids) and local_rank < len(ids):
        return int(ids[local_rank])
    return local_rank


# ---- peaks measured in this run (csrc/peaks) -----------------------------------------

def measure_peaks(gpu_index: int) -> dict:
    """L1 load bandwidth (16-byte read-only loads hitting L1, coalesced) and the
    FP32 FMA rate (scalar and f32x2), each the best of three launches on the
    current device, with the SM clock sampled meanwhile."""
    from fanbeamctrecon_tensorflowop_gb300 import _build
    _build.build()
    lib = ctypes.CDLL(str(_build.PEAKS_PATH))
    d = ctypes.c_double
    lib.ctpk_l1_load.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(d), ctypes.POINTER(d)]
    lib.ctpk_l1_load_v8.argtypes = lib.ctpk_l1_load.argtypes
    lib.ctpk_fma.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(d),
                             ctypes.POINTER(d)]
    lib.ctpk_sm_count.argtypes = [ctypes.POINTER(ctypes.c_int)]
    sms = ctypes.c_int()
    if lib.ctpk_sm_count(ctypes.byref(sms)):
        raise RuntimeError("ctpk_sm_count failed")
    out = {"sm_count": sms.value}
    with ClockSampler(gpu_index) as clk:
        for fn, key in ((lib.ctpk_l1_load, "l1_load_gbs"), (lib.ctpk_l1_load_v8, "l1_load32_gbs")):
            best = 0.0
            for _ in range(3):
                v, ms = d(), d()
                rc = fn(4, 2000, ctypes.byref(v), ctypes.byref(ms))
                if rc:
                    raise RuntimeError(f"L1 load peak failed: CUDA error {rc}")
                best = max(best, v.value)
            out[key] = best
        for packed, key in ((0, "fp32_tflops_scalar"), (1, "fp32_tflops_f32x2")):
            best = 0.0
            for _ in range(3):
                v, ms = d(), d()
                rc = lib.ctpk_fma(packed, 8, 4000, ctypes.byref(v), ctypes.byref(ms))
                if rc:
                    raise RuntimeError(f"ctpk_fma failed: CUDA error {rc}")
                best = max(best, v.value)
            out[key] = best
    c = clk.summary()
    out["fp32_tflops"] = max(out["fp32_tflops_scalar"], out["fp32_tflops_f32x2"])
    out["clocks"] = c
    if c.get("sm_mhz"):
        out["l1_bytes_per_clk_per_sm"] = out["l1_load_gbs"] * 1e9 / (c["sm_mhz"] * 1e6) / sms.value
        out["l1_32b_bytes_per_clk_per_sm"] = (out["l1_load32_gbs"] * 1e9 / (c["sm_mhz"] * 1e6)
                                              / sms.value)
    out["how"] = ("csrc/peaks: L1 = 16-byte (ld.global.nc.v4.f32) and 32-byte "
                  "(ld.global.nc.v8.f32) loads over a 32 KiB per-SM buffer, adjacent lanes on "
                  "adjacent addresses, 4 x 512 threads per SM; FP32 = 8 independent FMA chains "
                  "per thread, scalar and f32x2; best of 3 launches, CUDA events")
    return out


# ---- CPU baseline: FP32 OpenMP transcription of the reference --------------------------

def cpu_baseline(n_views_sample: int = 96) -> dict:
    """FP, BP and FBP of one clinical slice on the host cores with the FP32
    transcription, over n_views_sample views spread over the scan."""
    import oracle
    from oracle import cpu
    from fanbeamctrecon_tensorflowop_gb300 import phantom
    p, a = c1_geometry()
    g = oracle.decode(p)
    img = phantom.ellipse_phantom(N_PIX, PIXEL_MM, seed=0)
    sino = np.random.default_rng(0).random((VIEWS, COLS)).astype(np.float32)
    r = cpu.time_ops(g, a, img, sino, n_views_sample)
    return {
        "value": r["fp_grays_per_s"], "unit": "Grays/s", "cores": r["threads"], "kind": "port",
        "cpu": r["cpu"],
        "sample": (f"one clinical slice, {r['views_timed']} of 984 views (every "
                   f"{VIEWS // r['views_timed']}th) x 888 channels: FP, BP and Ram-Lak FBP, "
                   "FP32 OpenMP transcription of the reference (oracle/cpu_fp32.c)"),
        "bp_gpix_views_per_s": r["bp_gpix_views_per_s"],
        "fbp_ms_per_slice": r["fbp_ms_per_slice"],
        "seconds": r["seconds"],
    }


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from oracle import cpu
    from fanbeamctrecon_tensorflowop_gb300 import phantom
    cpu.build()
    p, a = c1_geometry()
    g = oracle.decode(p)
    img = phantom.ellipse_phantom(N_PIX, PIXEL_MM, seed=0)
    nv = 123  # views per step: one eighth of the scan, every 8th view
    sel = np.arange(0, VIEWS, VIEWS // nv)[:nv]
    sub = oracle.OrcGeom.from_buffer_copy(g)
    sub.n_views = nv
    sa = np.ascontiguousarray(a[sel])
    for _ in range(args.warmup):
        cpu.fp_fan(sub, sa, img)
    secs = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu.fp_fan(sub, sa, img)
        secs.append(time.perf_counter() - t0)
    total = sum(secs)
    v = args.steps * nv * COLS / total / 1e9
    others = cpu_baseline(96)
    sample = (f"FP of one clinical slice per step, {nv} of 984 views (every 8th) x 888 "
              f"channels ({nv * COLS} rays), FP32 OpenMP transcription of the reference "
              "(oracle/cpu_fp32.c)")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Grays/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded ellipse phantom (numpy default_rng seed 0)",
        "config": {"workload": WORKLOAD, "sample": sample,
                   "note": "the reference's CUDA/TF ops cannot be built for the GPU (CUDA 13 "
                           "rejects texture references; TF/IPP absent): its algorithms run "
                           "as an FP32 OpenMP transcription on the host cores"},
        "cpu_baseline": {"value": v, "unit": "Grays/s", "cores": cpu.threads(), "kind": "port",
                         "cpu": cpu.cpu_model(), "sample": sample,
                         "bp_gpix_views_per_s": others["bp_gpix_views_per_s"],
                         "fbp_ms_per_slice": others["fbp_ms_per_slice"]},
        "e2e": {"value": v, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---- output errors against the FP64 oracle (the checker), untimed ----------------------

def _rel(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_errors(dev, plan, plan_sl, imgs, usinos) -> dict:
    """Relative L2 of each output against the FP64 oracle on the same inputs,
    and the adjoints' dot-product mismatches, at each workload's own image
    and detector size (views subsampled where the oracle's cost needs it)."""
    import torch

    import oracle
    from fanbeamctrecon_tensorflowop_gb300 import _lib
    from fanbeamctrecon_tensorflowop_gb300.batch import UnevenBatch
    from fanbeamctrecon_tensorflowop_gb300.geometry import angle, fan_param16
    from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan, FanPlan

    t_start = time.perf_counter()
    out: dict = {"tolerance": 1e-4, "against": "FP64 oracle (oracle/oracle.c)"}
    p, a = c1_geometry()
    g = oracle.decode(p)
    every = 4
    sel = np.arange(0, VIEWS, every)
    sub = oracle.OrcGeom.from_buffer_copy(g)
    sub.n_views = len(sel)
    asub = np.ascontiguousarray(a[sel])

    x = imgs[0][:1]
    sino = plan.fp(x)
    c1 = {}
    c1["fp"] = _rel(sino[0].cpu().numpy()[sel], oracle.fp_fan(sub, asub, x[0].cpu().numpy())[0])
    u = usinos[0][:1]
    c1["bp"] = _rel(plan.bp(u)[0].cpu().numpy(), oracle.bp_fan(g, a, u[0].cpu().numpy())[0])
    c1["fbp_shepp_logan"] = _rel(plan_sl.fbp(sino)[0].cpu().numpy(),
                                 oracle.fbp_fan(g, a, sino[0].cpu().numpy(),
                                                window=oracle.SHEPP_LOGAN)[0])
    gen = torch.Generator(device=dev).manual_seed(7)
    y = torch.randn((1, VIEWS, COLS), device=dev, generator=gen)
    ymask = torch.zeros_like(y)
    ymask[:, sel] = y[:, sel]
    c1["fp_adjoint"] = _rel(plan.fp_adjoint(ymask)[0].cpu().numpy(),
                            oracle.fp_fan_adjoint(sub, asub, y[0].cpu().numpy()[sel])[0])
    c1["fbp_adjoint"] = _rel(plan_sl.fbp_adjoint(x)[0].cpu().numpy(),
                             oracle.fbp_fan_adjoint(g, a, x[0].cpu().numpy(),
                                                    window=oracle.SHEPP_LOGAN)[0])
    c1["views_compared"] = {"fp": f"every {every}th view", "fp_adjoint": f"sinogram nonzero on "
                            f"every {every}th view", "bp": "all", "fbp": "all"}
    out["clinical_512_984x888"] = c1

    # dot-product mismatches |<Ax, y> - <x, A^T y>| / |<Ax, y>| at batch 32
    xs = torch.randn((BATCH, N_PIX, N_PIX), device=dev, generator=gen)
    ys = torch.randn((BATCH, VIEWS, COLS), device=dev, generator=gen)

    def dot(u_, v_):
        return float((u_.double() * v_.double()).sum())

    def mismatch(ax, y_, x_, aty):
        """|<Ax, y> - <x, A^T y>| / (||Ax|| ||y||), as the tests define it."""
        return abs(dot(ax, y_) - dot(x_, aty)) / (float(ax.double().norm()) *
                                                  float(y_.double().norm()))

    dots = {"fp_batch32": mismatch(plan.fp(xs), ys, xs, plan.fp_adjoint(ys)),
            "fbp_batch32": mismatch(plan_sl.fbp_adjoint(xs), ys, xs, plan_sl.fbp(ys)),
            "bp_batch32": mismatch(plan.bp_adjoint(xs), ys, xs, plan.bp(ys))}
    del xs, ys

    # uneven BF16 batch: one slice of each of the three geometries, FP / FBP / FBP adjoint
    unev = {}
    for n_, v_, c_ in ((256, 492, 512), (384, 720, 736), (512, 984, 888)):
        up = fan_param16(sdd=SDD, sid=SID, n_views=v_, n_cols=c_, n=n_, pixel_mm=358.4 / n_,
                         dcol_rad=DCOL)
        ua = angle(v_, 0.0)
        pl = FanPlan(up, ua, device=dev)
        ug = oracle.decode(up)
        img16 = torch.rand((n_, n_), device=dev, generator=gen).to(torch.bfloat16)
        sino16 = torch.rand(pl.sino_shape, device=dev, generator=gen).to(torch.bfloat16)
        o_fp = torch.empty(pl.sino_shape, device=dev, dtype=torch.bfloat16)
        o_fbp = torch.empty(pl.image_shape, device=dev, dtype=torch.bfloat16)
        o_adj = torch.empty(pl.sino_shape, device=dev, dtype=torch.bfloat16)
        for it in ((pl, "fp", img16, o_fp), (pl, "fbp", sino16, o_fbp),
                   (pl, "fbp_adjoint", img16, o_adj)):
            UnevenBatch([it]).run()
        xi = img16.float().cpu().numpy()
        si = sino16.float().cpu().numpy()
        unev[f"{n_}^2_{v_}x{c_}"] = {
            "fp": _rel(o_fp.float().cpu().numpy(), oracle.fp_fan(ug, ua, xi)[0]),
            "fbp": _rel(o_fbp.float().cpu().numpy(), oracle.fbp_fan(ug, ua, si)[0]),
            "fbp_adjoint": _rel(o_adj.float().cpu().numpy(),
                                oracle.fbp_fan_adjoint(ug, ua, xi)[0]),
        }
        pl.close()
    unev["note"] = ("BF16 storage: the oracle runs on the BF16-rounded inputs, the outputs "
                    "are rounded to BF16 (2^-9 relative per value)")
    out["uneven_bf16"] = unev

    # cone beam at the clinical volume and detector (512^2 x 64, 888 x 64), 8 views
    nvc = 8
    csel = np.arange(0, VIEWS, VIEWS // nvc)[:nvc]
    cp = fan_param16(sdd=SDD, sid=SID, n_views=nvc, n_cols=COLS, n=N_PIX, pixel_mm=PIXEL_MM,
                     dcol_rad=DCOL, det_bottom=-32.0, drow=1.0, dz=0.625)
    ca = np.ascontiguousarray(a[csel])
    cplan = ConePlan(cp, ca, 64, 64, device=dev)
    cg = oracle.decode(cp)
    vol = torch.rand((1, 64, N_PIX, N_PIX), device=dev, generator=gen)
    proj = cplan.fp_cone(vol)
    rec = cplan.fdk(proj)
    cadj = cplan.fdk_adjoint(vol)
    vn, pn = vol[0].cpu().numpy(), proj[0].cpu().numpy()
    out["cone_512x512x64_888x64"] = {
        "fp_cone": _rel(pn, oracle.cone_fp(cg, 64, 64, ca, vn)[0]),
        "fdk": _rel(rec[0].cpu().numpy(), oracle.fdk_cone(cg, 64, 64, ca, pn)[0]),
        "fdk_adjoint": _rel(cadj[0].cpu().numpy(), oracle.fdk_cone_adjoint(cg, 64, 64, ca, vn)[0]),
        "views": f"{nvc} of 984 (every {VIEWS // nvc}th)",
    }
    yc = torch.randn((1, nvc, 64, COLS), device=dev, generator=gen)
    vr = torch.randn((1, 64, N_PIX, N_PIX), device=dev, generator=gen)
    dots["fdk_cone"] = mismatch(cplan.fdk_adjoint(vr), yc, vr, cplan.fdk(yc))
    cplan.close()
    out["dot_mismatch"] = dots
    f32 = [v for d in (c1, out["cone_512x512x64_888x64"]) for v in d.values()
           if isinstance(v, float)]
    bf16 = [v for d in unev.values() if isinstance(d, dict) for v in d.values()]
    out["worst_rel_l2_f32"] = max(f32)
    out["worst_rel_l2_bf16"] = max(bf16)
    out["worst_dot_mismatch"] = max(dots.values())
    out["seconds"] = time.perf_counter() - t_start
    return out


# ---- profiler driver -------------------------------------------------------------------

def profile_case(args) -> None:
    """Runs one operator on the clinical-scale geometry: one untimed warm-up
    call, then ``--iters`` calls, so ``ncu -s <launches of one call>`` skips the
    warm-up.  Ops: fp, fp_adjoint, bp, bp_adjoint, filter, fbp, fbp_adjoint
    (``--batch`` slices); cone_fp, fdk, fdk_adjoint (``--batch`` volumes of
    512^2 x 64 voxels at 0.7 x 0.7 x 0.625 mm, 888 x 64 detector cells of 1 mm
    rows per view)."""
    import torch

    from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom
    from fanbeamctrecon_tensorflowop_gb300.geometry import angle, fan_param16
    from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan, FanPlan

    dev = torch.device("cuda", 0)
    op = args.profile_case
    n, views, cols, pixel = args.n, args.views, COLS, PIXEL_MM
    a = angle(views, 0.0)
    if op in ("cone_fp", "fdk", "fdk_adjoint"):
        pc = fan_param16(sdd=SDD, sid=SID, n_views=views, n_cols=cols, n=n, pixel_mm=pixel,
                         dcol_rad=DCOL, det_bottom=-32.0, drow=1.0, dz=0.625)
        cplan = ConePlan(pc, a, 64, 64, device=dev)
        vol = torch.rand((args.batch, 64, n, n), device=dev)
        proj = cplan.fp_cone(vol)
        fn = {"cone_fp": lambda: cplan.fp_cone(vol, out=proj),
              "fdk": lambda: cplan.fdk(proj),
              "fdk_adjoint": lambda: cplan.fdk_adjoint(vol)}[op]
    else:
        p = fan_param16(sdd=SDD, sid=SID, n_views=views, n_cols=cols, n=n, pixel_mm=pixel,
                        dcol_rad=DCOL)
        win = _lib.WINDOW_SHEPP_LOGAN if args.window == "shepp_logan" else _lib.WINDOW_RAMLAK
        plan = FanPlan(p, a, device=dev, window=win)
        img = torch.from_numpy(np.stack([phantom.ellipse_phantom(n, pixel, seed=s)
                                         for s in range(args.batch)])).to(dev)
        sino = plan.fp(img)
        fn = {"fp": lambda: plan.fp(img), "fp_adjoint": lambda: plan.fp_adjoint(sino),
              "bp": lambda: plan.bp(sino), "bp_adjoint": lambda: plan.bp_adjoint(img),
              "filter": lambda: plan.ramp_filter(sino), "fbp": lambda: plan.fbp(sino),
              "fbp_adjoint": lambda: plan.fbp_adjoint(img)}[op]
    fn()
    torch.cuda.synchronize()
    for _ in range(args.iters):
        fn()
    torch.cuda.synchronize()
    print(f"profile_case {op} batch={args.batch} ok")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU baseline and the oracle error checks")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cone", action="store_true")
    ap.add_argument("--no-uneven", action="store_true")
    ap.add_argument("--profile-case", default=None,
                    help="run one operator for a profiler instead of the benchmark")
    ap.add_argument("--batch", type=int, default=8, help="--profile-case: slices or volumes")
    ap.add_argument("--iters", type=int, default=3, help="--profile-case: profiled calls")
    ap.add_argument("--views", type=int, default=VIEWS, help="--profile-case: views")
    ap.add_argument("--n", type=int, default=N_PIX, help="--profile-case: image size")
    ap.add_argument("--window", default="ramlak", choices=["ramlak", "shepp_logan"])
    ap.add_argument("--peaks-only", action="store_true",
                    help="measure and print the L1-load and FP32 peaks, then exit")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
        return
    if args.peaks_only:
        import torch
        torch.cuda.init()
        print(json.dumps(measure_peaks(gpu_index_for_smi(int(os.environ.get("LOCAL_RANK", "0"))))))
        return
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist

    from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom, utils
    from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    smi = gpu_index_for_smi(local)

    p, a = c1_geometry()
    plan = FanPlan(p, a, device=dev)
    plan_sl = FanPlan(p, a, device=dev, window=_lib.WINDOW_SHEPP_LOGAN)
    g = plan.geom
    stream = torch.cuda.current_stream(dev)

    # inputs: POOL batches of seeded phantoms (distinct per rank), resident in HBM
    base = np.stack([phantom.ellipse_phantom(N_PIX, PIXEL_MM, seed=rank * 1000 + s)
                     for s in range(8)])
    imgs = []
    for k in range(POOL):
        idx = [(k * BATCH + b) % len(base) for b in range(BATCH)]
        t = torch.from_numpy(base[idx]).to(dev)
        imgs.append(t * (1.0 + 0.01 * k))  # distinct buffers and values
    sinos = [torch.empty((BATCH, VIEWS, COLS), device=dev) for _ in range(POOL)]
    gen = torch.Generator(device=dev).manual_seed(1234 + rank)
    usinos = [torch.rand((BATCH, VIEWS, COLS), device=dev, generator=gen) for _ in range(POOL)]
    bimgs = [torch.empty((BATCH, N_PIX, N_PIX), device=dev) for _ in range(POOL)]

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def timed(fn, steps, warmup):
        """Event-timed loop: per-step events on the launching stream.  Returns
        (max-over-ranks seconds, per-step seconds, library launches inside)."""
        for k in range(warmup):
            fn(k)
        barrier()
        n0 = _lib.launch_count()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        t_all0 = torch.cuda.Event(enable_timing=True)
        t_all1 = torch.cuda.Event(enable_timing=True)
        t_all0.record(stream)
        for k in range(steps):
            evs[k][0].record(stream)
            fn(k)
            evs[k][1].record(stream)
        t_all1.record(stream)
        n1 = _lib.launch_count()
        barrier()
        total = t_all0.elapsed_time(t_all1) / 1e3
        per = [e0.elapsed_time(e1) / 1e3 for e0, e1 in evs]
        return max_over_ranks(total), per, n1 - n0

    # ---- peaks of this GPU, measured now (untimed) ----------------------------------
    pk = measure_peaks(smi)
    hbm = measured_peaks()
    # the L1 load path's peak: 32-byte loads move about twice the bytes of
    # 16-byte ones in the same time, so the larger of the two is the roofline
    l1_peak = max(pk["l1_load_gbs"], pk["l1_load32_gbs"])

    # ---- headline: FP throughput -----------------------------------------------
    def fp_step(k):
        plan.fp(imgs[k % POOL], out=sinos[k % POOL])

    with ClockSampler(smi) as clk:
        total_fp, per_fp, launches = timed(fp_step, args.steps, args.warmup)
    rays_per_step = BATCH * VIEWS * COLS
    value = world * rays_per_step * args.steps / total_fp / 1e9
    ms_per_step = 1e3 * total_fp / args.steps

    # roofline of the dominant kernel of the step, fp_fan_kernel (98% of the step:
    # build_quads_kernel + fp_fan_kernel; profiles/bench_launches_c1.md)
    visits = fp_cell_visits(p, a)
    mean_fp = sum(per_fp) / len(per_fp)
    share = profiled("fp_fan_kernel", "share_of_step") or 1.0
    kern_s = mean_fp * share
    l1_bytes = QUAD_BYTES * BATCH * visits
    achieved = l1_bytes / kern_s / 1e9
    traffic = profiled("fp_fan_kernel", "dram_bytes_per_launch")
    compulsory = 4.0 * (N_PIX * N_PIX + VIEWS * COLS) * BATCH
    roofline = {
        "bound": "l1", "achieved": achieved, "peak": l1_peak, "unit": "GB/s",
        "frac": achieved / l1_peak, "traffic": traffic,
        "peak_source": L1_PEAK_SOURCE,
        "frac_of_16b_load_peak": achieved / pk["l1_load_gbs"],
        "kernel": "fp_fan_kernel",
        "algorithmic": (f"{QUAD_BYTES} B (one float4 quad) per (ray, cell) visit and slice x "
                        f"{visits} visits per slice x {BATCH} slices = {l1_bytes:.4g} B per launch"),
        "timed": (f"per-step CUDA events x the kernel's share of the step ({share:.3f}, "
                  "profiles/traffic.txt)"),
        "kernel_ms": 1e3 * kern_s,
        "dram": {"compulsory_bytes": compulsory,
                 "compulsory_frac_of_hbm": compulsory / kern_s / 1e9 / hbm["hbm_gbs"],
                 "measured_bytes": traffic,
                 "measured_frac_of_hbm": (traffic / kern_s / 1e9 / hbm["hbm_gbs"]) if traffic
                 else None,
                 "hbm_peak_gbs": hbm["hbm_gbs"], "hbm_peak_source": hbm["source"]},
        "fp32": {"achieved_tflops": FMA_FLOP_PER_VISIT * BATCH * visits / kern_s / 1e12,
                 "peak_tflops": pk["fp32_tflops"],
                 "frac": FMA_FLOP_PER_VISIT * BATCH * visits / kern_s / 1e12 / pk["fp32_tflops"],
                 "algorithmic": f"{FMA_FLOP_PER_VISIT} FLOP (two f32x2 FMAs) per visit and slice",
                 "peak_source": "measured in this run (csrc/peaks FMA chains)"},
    }

    # ---- BP throughput ------------------------------------------------------------
    def bp_step(k):
        plan.bp(usinos[k % POOL], out=bimgs[k % POOL])

    total_bp, per_bp, _ = timed(bp_step, args.steps, args.warmup)
    bp_gpv = world * BATCH * N_PIX * N_PIX * VIEWS * args.steps / total_bp / 1e9
    fovpix = fov_pixels(g.nx, g.ny, g.xmin, g.ymin, g.dx, g.dy, g.rfov)
    bp_share = profiled("bp_fan_kernel", "share_of_step") or 1.0
    bp_s = sum(per_bp) / len(per_bp) * bp_share
    bp_bytes = TAP_BYTES * BATCH * fovpix * VIEWS
    bp_roof = {"bound": "l1", "kernel": "bp_fan_kernel", "achieved": bp_bytes / bp_s / 1e9,
               "peak": l1_peak, "unit": "GB/s",
               "frac": bp_bytes / bp_s / 1e9 / l1_peak, "peak_source": L1_PEAK_SOURCE,
               "algorithmic": (f"{TAP_BYTES} B (two FP32 taps) per in-FOV pixel-view and slice "
                               f"x {fovpix} pixels x {VIEWS} views x {BATCH} slices"),
               "share_of_step": bp_share,
               "dram_compulsory_frac_of_hbm": 4.0 * (N_PIX * N_PIX + VIEWS * COLS) * BATCH
               / bp_s / 1e9 / hbm["hbm_gbs"]}

    # ---- Shepp-Logan FBP of the FP sinograms ----------------------------------------
    def fbp_step(k):
        plan_sl.fbp(sinos[k % POOL], out=bimgs[k % POOL])

    total_fbp, _, _ = timed(fbp_step, max(5, args.steps // 3), args.warmup)
    fbp_ms_per_slice = 1e3 * total_fbp / max(5, args.steps // 3) / BATCH

    # ---- the Shepp-Logan ramp filter alone (tensor-core Toeplitz GEMM), 32 slices --------
    fbuf = torch.empty_like(sinos[0])

    def filter_step(k):
        plan_sl.ramp_filter(sinos[k % POOL], out=fbuf)

    n_f = max(5, args.steps // 3)
    total_filt, _, _ = timed(filter_step, n_f, args.warmup)
    filter_ms = 1e3 * total_filt / n_f
    filter_tflops = 2.0 * BATCH * VIEWS * COLS * COLS / (total_filt / n_f) / 1e12

    # ---- batch-32 differentiable step: FP, residual, adjoint ------------------------
    target = [plan.fp(imgs[(k + 1) % POOL]) for k in range(2)]
    grads = [torch.empty((BATCH, N_PIX, N_PIX), device=dev) for _ in range(2)]

    def fwd_adj_step(k):
        r = plan.fp(imgs[k % POOL])
        r.sub_(target[k % 2])
        plan.fp_adjoint(r, out=grads[k % 2])

    n_fa = max(5, args.steps // 3)
    total_fa, _, _ = timed(fwd_adj_step, n_fa, args.warmup)
    fa_ms = 1e3 * total_fa / n_fa

    def adj_step(k):
        plan.fp_adjoint(sinos[k % POOL], out=grads[k % 2])

    total_adj, per_adj, _ = timed(adj_step, n_fa, args.warmup)
    adj_ms = 1e3 * total_adj / n_fa
    adj_share = profiled("fp_adjoint_cells_kernel", "share_of_step") or 1.0
    adj_s = sum(per_adj) / len(per_adj) * adj_share
    adj_bytes = SINO_BYTES * BATCH * visits
    adj_roof = {"bound": "issue", "kernel": "fp_adjoint_cells_kernel",
                "achieved": adj_bytes / adj_s / 1e9, "peak": l1_peak, "unit": "GB/s",
                "frac": adj_bytes / adj_s / 1e9 / l1_peak, "peak_source": L1_PEAK_SOURCE,
                "algorithmic": (f"{SINO_BYTES} B (one FP32 sinogram value) per (cell, ray) pair "
                                f"and slice x {visits} pairs per slice x {BATCH} slices"),
                "share_of_step": adj_share}

    # ---- BP / FBP adjoints (transposes) -------------------------------------------
    def bpt_step(k):
        plan.bp_adjoint(imgs[k % POOL], out=sinos[k % POOL])

    total_bpt, _, _ = timed(bpt_step, n_fa, args.warmup)
    bpt_ms = 1e3 * total_bpt / n_fa

    def fbpt_step(k):
        plan_sl.fbp_adjoint(imgs[k % POOL], out=sinos[k % POOL])

    total_fbpt, _, _ = timed(fbpt_step, n_fa, args.warmup)
    fbpt_ms = 1e3 * total_fbpt / n_fa

    plain_ms = None
    if not args.no_plain:
        def plain_step(k):
            r = plan.plain_fp(imgs[k % POOL])
            r.sub_(target[k % 2])
            grads[k % 2].copy_(plan.plain_fp_adjoint(r))

        for k in range(1):
            plain_step(k)
        barrier()
        t0 = time.perf_counter()
        n_plain = 2
        for k in range(n_plain):
            plain_step(k)
        barrier()
        plain_ms = 1e3 * max_over_ranks(time.perf_counter() - t0) / n_plain

    # ---- cone beam, batch of 4 volumes (512^2 x 64 @0.7x0.7x0.625 mm, 984 views,
    #      888 x 64 detector): cone FP -> FDK -> FDK adjoint --------------------------------
    cone = None
    if not args.no_cone:
        from fanbeamctrecon_tensorflowop_gb300.geometry import fan_param16 as _f16
        from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan
        cp = _f16(sdd=SDD, sid=SID, n_views=VIEWS, n_cols=COLS, n=N_PIX, pixel_mm=PIXEL_MM,
                  dcol_rad=DCOL, det_bottom=-32.0, drow=1.0, dz=0.625)
        cplan = ConePlan(cp, a, 64, 64, device=dev)
        CB = 4
        cvol = torch.rand((CB, 64, N_PIX, N_PIX), device=dev, generator=gen)
        cproj = cplan.fp_cone(cvol)
        crec = cplan.fdk(cproj)
        cgrad = cplan.fdk_adjoint(crec)

        def cone_time(fn):
            fn()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            barrier()
            return max_over_ranks(e0.elapsed_time(e1)) / CB

        t_fp = cone_time(lambda: cplan.fp_cone(cvol, out=cproj))
        t_fdk = cone_time(lambda: cplan.fdk(cproj, out=crec))
        t_adj = cone_time(lambda: cplan.fdk_adjoint(crec, out=cgrad))
        cone = {"workload": "cone beam, 4 volumes 512x512x64 @0.7x0.7x0.625 mm, 984 views, "
                            "888 x 64 detector (1 mm rows), FP -> FDK -> FDK adjoint",
                "fp_cone_ms_per_volume": t_fp, "fdk_ms_per_volume": t_fdk,
                "fdk_adjoint_ms_per_volume": t_adj,
                "fdk_gvoxel_views_per_s": 512 * 512 * 64 * VIEWS / t_fdk / 1e6}
        # the cone FP's in-plane cells are the fan FP's (same rays): 8 FP32 taps per
        # (cell, detector row)
        cone_l1 = 32.0 * 64 * visits
        cone_ach = cone_l1 / (t_fp * 1e-3) / 1e9
        cone["fp_roofline"] = {
            "bound": "l1", "kernel": "cone_fp_seg_kernel", "achieved": cone_ach,
            "peak": l1_peak, "unit": "GB/s", "frac": cone_ach / l1_peak,
            "peak_source": L1_PEAK_SOURCE,
            "algorithmic": (f"32 B (eight FP32 trilinear taps) per (in-plane cell, detector row) x "
                            f"{visits} cells x 64 rows = {cone_l1:.4g} B per volume"),
            "timed": "per-volume CUDA events of ct_fp_cone (its column build included)"}
        del cvol, cproj, crec, cgrad
        cplan.close()

    # ---- uneven batches, BF16 storage; FP, FBP and FBP adjoint of all 48 slices as
    #      three ct_batch_run calls recorded in one CUDA graph:
    #      (a) 48 slices cycling 256^2/492 views/512 ch, 384^2/720/736, 512^2/984/888
    #          (rFOV 179.2 mm): three plans of 16 slices each, run as slice groups;
    #      (b) 48 slices of 48 different geometries: the persistent launches, with
    #          their launch shapes from the autotuner ----------------------------------
    uneven = uneven_distinct = None
    if not args.no_uneven:
        from fanbeamctrecon_tensorflowop_gb300.batch import UnevenBatch
        from fanbeamctrecon_tensorflowop_gb300.geometry import angle as _ang
        from fanbeamctrecon_tensorflowop_gb300.geometry import fan_param16 as _f16

        def uneven_run(sizes):
            """sizes: one (n, views, channels) per slice; equal sizes share a plan."""
            plans = {}
            for sz in sizes:
                if sz not in plans:
                    n_, v_, c_ = sz
                    up = _f16(sdd=SDD, sid=SID, n_views=v_, n_cols=c_, n=n_,
                              pixel_mm=358.4 / n_, dcol_rad=DCOL)
                    plans[sz] = FanPlan(up, _ang(v_, 0.0), device=dev)
            fp_items, fbp_items, adj_items = [], [], []
            rays = 0
            for sz in sizes:
                pl = plans[sz]
                n_ = pl.geom.nx
                img16 = torch.rand((n_, n_), device=dev, generator=gen).to(torch.bfloat16)
                sino16 = torch.rand(pl.sino_shape, device=dev, generator=gen).to(torch.bfloat16)
                fp_items.append((pl, "fp", img16, torch.empty(pl.sino_shape, device=dev,
                                                              dtype=torch.bfloat16)))
                fbp_items.append((pl, "fbp", sino16, torch.empty(pl.image_shape, device=dev,
                                                                 dtype=torch.bfloat16)))
                adj_items.append((pl, "fbp_adjoint", img16,
                                  torch.empty(pl.sino_shape, device=dev, dtype=torch.bfloat16)))
                rays += pl.geom.n_views * pl.geom.n_cols
            ubs = [UnevenBatch(fp_items), UnevenBatch(fbp_items), UnevenBatch(adj_items)]

            def graph_ms():
                for ub in ubs:
                    ub.run()
                torch.cuda.synchronize(dev)
                graph = torch.cuda.CUDAGraph()
                cap = torch.cuda.Stream(dev)
                cap.wait_stream(stream)
                with torch.cuda.stream(cap):
                    with torch.cuda.graph(graph, stream=cap):
                        for ub in ubs:
                            ub.run()
                stream.wait_stream(cap)
                for _ in range(args.warmup):
                    graph.replay()
                barrier()
                n_rep = max(3, args.steps // 3)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(n_rep):
                    graph.replay()
                e1.record(stream)
                barrier()
                return max_over_ranks(e0.elapsed_time(e1)) / n_rep

            for ub in ubs:
                ub.set_config(None)
            g_default = graph_ms()
            # the autotuner picks both persistent launches' shapes per batch
            t_tune = time.perf_counter()
            tuned = [ub.tune(reps=2) for ub in ubs]
            t_tune = time.perf_counter() - t_tune
            g_ms = graph_ms()
            out = {"graph_replay_ms": g_ms, "graph_replay_ms_default_shapes": g_default,
                   "tuned_shapes": {"fp": tuned[0], "fbp": tuned[1], "fbp_adjoint": tuned[2]},
                   "tune_seconds": t_tune, "slice_ops_per_replay": 3 * len(sizes),
                   "fp_rays_per_replay": rays, "plans": len(plans)}
            del ubs, fp_items, fbp_items, adj_items, plans
            return out

        cyc = [(256, 492, 512), (384, 720, 736), (512, 984, 888)]
        uneven = {"workload": "48 slices cycling 256^2/492x512, 384^2/720x736, 512^2/984x888 "
                              "(three plans, run as slice groups), BF16 storage: FP + FBP + "
                              "FBP adjoint of every slice, 3 ct_batch_run calls in one CUDA "
                              "graph"}
        uneven.update(uneven_run([cyc[k % 3] for k in range(48)]))
        # 48 geometries: image 256..512, views 492..962, channels 512..888 (multiples of 8)
        distinct = [(256 + 16 * (k % 17), 492 + 10 * k, 512 + 8 * k) for k in range(48)]
        uneven_distinct = {"workload": "48 slices of 48 different geometries (image "
                                       "256^2..512^2, 492..962 views, 512..888 channels), BF16 "
                                       "storage: FP + FBP + FBP adjoint, persistent launches, "
                                       "3 ct_batch_run calls in one CUDA graph"}
        uneven_distinct.update(uneven_run(distinct))

    # ---- e2e through the reference-named entry point with host buffers ---------------
    host_imgs = [imgs[k].cpu().numpy() for k in range(2)]
    vs, ps = [BATCH, N_PIX, N_PIX], [BATCH, VIEWS, COLS]
    # the warm-up holds each result while the next call runs, as the timed loop
    # does, so the page-locked result buffers it cycles through already exist
    out = None
    for k in range(max(args.warmup, 3)):
        out = utils.fp_fan_curve(volume=host_imgs[k % 2], angle=a, parameter=p, vol_shape=vs,
                                 proj_shape=ps)
    del out
    barrier()
    n_e2e = max(5, args.steps // 3)
    t0 = time.perf_counter()
    for k in range(n_e2e):
        out = utils.fp_fan_curve(volume=host_imgs[k % 2], angle=a, parameter=p, vol_shape=vs,
                                 proj_shape=ps)
        assert isinstance(out, np.ndarray)
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_val = world * rays_per_step * n_e2e / e2e_s / 1e9

    cpu = errors = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(96)
        cpu.pop("seconds", None)
        errors = oracle_errors(dev, plan, plan_sl, imgs, usinos)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Grays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded ellipse phantoms (numpy default_rng), U[0,1) sinograms",
            "config": {"workload": WORKLOAD, "global_batch": BATCH * world,
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs rotate over 4 batches (576 MB) > 129 MB L2"},
            "e2e": {"value": e2e_val, "unit": "Grays/s",
                    "h2d_bytes_per_step": BATCH * N_PIX * N_PIX * 4,
                    "d2h_bytes_per_step": BATCH * VIEWS * COLS * 4,
                    "path": "utils.fp_fan_curve(numpy) -> numpy"},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "peaks": pk,
            "errors": errors,
            "secondary": {
                "bp_gpix_views_per_s": bp_gpv,
                "bp_roofline": bp_roof,
                "fbp_shepp_logan_ms_per_slice": fbp_ms_per_slice,
                "filter_ms_batch32": filter_ms,
                "filter_algorithmic_tflops": filter_tflops,
                "batch32_fp_adjoint_ms": fa_ms,
                "batch32_adjoint_only_ms": adj_ms,
                "fp_adjoint_roofline": adj_roof,
                "batch32_bp_adjoint_ms": bpt_ms,
                "batch32_fbp_adjoint_ms": fbpt_ms,
                "plain_batch32_fp_adjoint_ms": plain_ms,
                "speedup_vs_plain": (plain_ms / fa_ms) if plain_ms else None,
                "fp_samples_per_slice": plan.total_samples,
                "fp_cell_visits_per_slice": visits,
                "cone": cone,
                "uneven_bf16": uneven,
                "uneven_distinct_bf16": uneven_distinct,
            },
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
