"""Benchmark of the fan-beam CT operators on GB300.

Headline (``value``): forward-projection throughput in G rays/s on the
clinical-scale geometry -- 512x512 slices at 0.7 mm, 984 views x 888
equiangular channels (1 mm pitch at the detector), SID 541 / SDD 949 mm --
one step = FP of a batch of 32 seeded ellipse phantoms resident in HBM.
Inputs rotate over 4 batches (576 MB of images + sinograms, > the 129 MB L2).

Also reported: ``e2e`` (the same FP through the reference-named Python entry
point ``utils.fp_fan_curve`` with host numpy buffers, host<->device copies
inside the timed region), BP throughput (G pixel-views/s, U[0,1)
sinograms), Shepp-Logan FBP time, and the batch-32 FP + adjoint step against
the plain per-view launch loop on the same GPU.

``--impl reference`` times the reference algorithm on the host CPU (the FP64
oracle restatement, all cores).  The reference's ops cannot be built for the
GPU, and their host-compiled form (oracle/build_ref.py, which runs each CUDA
thread as a fiber) exists only where the reference's sources are and is no
measure of its speed.

Multi-GPU: ``torchrun --nproc-per-node N bench.py --gpus N``: every rank runs
its own batch (replicas, no collective on the data path); the step time is
the max over ranks and ``value`` counts the rays of all ranks.
"""
from __future__ import annotations

import argparse
import json
import math
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
GATHER_BYTES_PER_SAMPLE = 16  # four FP32 bilinear taps per ray sample
FLOP_PER_SAMPLE = 16          # 2 FMA position, 2 fractions, 3 lerps, 1 add (FMA = 2)
# FP32 FMA peak, derived: 152 SMs x 128 lanes x 2 FLOP x 2.07 GHz (max SM clock)
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12


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


def profiled_traffic(kernel: str) -> float | None:
    """DRAM bytes per launch of `kernel` at this workload, from the ncu summary
    committed under profiles/ (a line 'kernel=<name> dram_bytes_per_launch=<B>')."""
    f = REPO / "profiles" / "traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = dict(kv.split("=", 1) for kv in line.split() if "=" in kv)
        if parts.get("kernel") == kernel and "dram_bytes_per_launch" in parts:
            return float(parts["dram_bytes_per_launch"])
    return None


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


def cpu_fp_sample(n_views_sample: int = 24, threads: int | None = None) -> dict:
    """The oracle's FP (the reference algorithm restated, FP64, OpenMP over all
    host cores) on a bounded sample: one phantom slice of the clinical
    geometry, the first n_views_sample views.  Returns G rays/s."""
    import oracle
    from fanbeamctrecon_tensorflowop_gb300 import phantom
    p, a = c1_geometry()
    ps = p.copy()
    ps[2] = n_views_sample
    g = oracle.decode(ps)
    img = phantom.ellipse_phantom(N_PIX, PIXEL_MM, seed=0)
    t0 = time.perf_counter()
    oracle.fp_fan(g, a[:n_views_sample], img)
    dt = time.perf_counter() - t0
    rays = n_views_sample * COLS
    return {"value": rays / dt / 1e9, "unit": "Grays/s",
            "cores": threads or os.cpu_count(), "seconds": dt,
            "sample": f"FP of 1 slice, {n_views_sample} of 984 views x 888 channels "
                      f"({rays} rays), FP64 oracle, OpenMP"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    for _ in range(args.warmup):
        cpu_fp_sample(8)
    vals, secs = [], 0.0
    res = None
    for _ in range(args.steps):
        res = cpu_fp_sample(24)
        vals.append(res["value"])
        secs += res["seconds"]
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Grays/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded ellipse phantom (numpy default_rng seed 0)",
        "config": {"workload": WORKLOAD, "sample": res["sample"],
                   "note": "the reference's CUDA/TF ops cannot be built for the GPU (CUDA 13 "
                           "rejects texture references; TF/IPP absent): its algorithm runs "
                           "as the FP64 oracle restatement on the host cores"},
        "cpu_baseline": {"value": v, "unit": "Grays/s", "cores": res["cores"], "kind": "port",
                         "sample": res["sample"]},
        "e2e": {"value": v, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cone", action="store_true")
    ap.add_argument("--no-uneven", action="store_true")
    args = ap.parse_args()
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

    # ---- headline: FP throughput -----------------------------------------------
    def fp_step(k):
        plan.fp(imgs[k % POOL], out=sinos[k % POOL])

    with ClockSampler(gpu_index_for_smi(local)) as clk:
        total_fp, per_fp, launches = timed(fp_step, args.steps, args.warmup)
    rays_per_step = BATCH * VIEWS * COLS
    value = world * rays_per_step * args.steps / total_fp / 1e9
    ms_per_step = 1e3 * total_fp / args.steps

    # roofline of the dominant (only) kernel of the step: fp_fan_kernel
    peaks = measured_peaks()
    samples_per_launch = BATCH * plan.total_samples
    mean_launch = sum(per_fp) / len(per_fp)
    achieved_gbs = GATHER_BYTES_PER_SAMPLE * samples_per_launch / mean_launch / 1e9
    traffic = profiled_traffic("fp_fan_kernel")
    fp32_tflops = FLOP_PER_SAMPLE * samples_per_launch / mean_launch / 1e12
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved_gbs / peaks["hbm_gbs"],
                "traffic": traffic, "peak_source": peaks["source"],
                "kernel": "fp_fan_kernel",
                "algorithmic": f"{GATHER_BYTES_PER_SAMPLE} B/sample x {samples_per_launch:.4g} "
                               "samples per launch (effective bilinear gather bytes)",
                "timed": "per-step CUDA events (the step is build_quads_kernel + "
                         "fp_fan_kernel; the quad build is ~3% of it)",
                "note": "the cell walk sums each cell's ~6 samples in closed form, so per-sample "
                        "work runs above the per-sample peaks; DRAM is far from the bound",
                "dram_gbs": (traffic / mean_launch / 1e9) if traffic else None,
                "fp32": {"achieved_tflops": fp32_tflops, "peak_tflops": FP32_PEAK_TFLOPS,
                         "frac": fp32_tflops / FP32_PEAK_TFLOPS,
                         "peak_source": "derived: 152 SMs x 128 x 2 FLOP x 2.07 GHz",
                         "algorithmic": f"{FLOP_PER_SAMPLE} FLOP/sample"}}

    # ---- BP throughput ------------------------------------------------------------
    def bp_step(k):
        plan.bp(usinos[k % POOL], out=bimgs[k % POOL])

    total_bp, _, _ = timed(bp_step, args.steps, args.warmup)
    bp_gpv = world * BATCH * N_PIX * N_PIX * VIEWS * args.steps / total_bp / 1e9

    # ---- Shepp-Logan FBP of the FP sinograms ----------------------------------------
    def fbp_step(k):
        plan_sl.fbp(sinos[k % POOL], out=bimgs[k % POOL])

    total_fbp, _, _ = timed(fbp_step, max(5, args.steps // 3), args.warmup)
    fbp_ms_per_slice = 1e3 * total_fbp / max(5, args.steps // 3) / BATCH

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
    adj_gather_gbs = GATHER_BYTES_PER_SAMPLE * samples_per_launch / (
        sum(per_adj) / len(per_adj)) / 1e9

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
        del cvol, cproj, crec, cgrad

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
    for k in range(args.warmup):
        utils.fp_fan_curve(volume=host_imgs[k % 2], angle=a, parameter=p, vol_shape=vs,
                           proj_shape=ps)
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

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_fp_sample(24)
        cpu.pop("seconds", None)

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
            "secondary": {
                "bp_gpix_views_per_s": bp_gpv,
                "fbp_shepp_logan_ms_per_slice": fbp_ms_per_slice,
                "batch32_fp_adjoint_ms": fa_ms,
                "batch32_adjoint_only_ms": adj_ms,
                "adjoint_effective_gather_gbs": adj_gather_gbs,
                "plain_batch32_fp_adjoint_ms": plain_ms,
                "speedup_vs_plain": (plain_ms / fa_ms) if plain_ms else None,
                "fp_samples_per_slice": plan.total_samples,
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
