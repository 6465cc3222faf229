"""Benchmark: W-projection grid + degrid throughput (Mvis/s) at 4096^2.

Workload (the W-projection dirty-image configuration): 27 antennas on a Y
with arms to 21 km, 8 h of 2 s dumps at 1.4 GHz (5,054,400 rows, one
channel), 200 seeded point sources 1 mJy - 1 Jy plus 5 mJy noise, a
4096 x 4096 image (grid 5000 x 5000), 128 w-planes with support growing
linearly with plane index from 8 to 64 pixels, oversampling 8.

One step = one pass of the hot path over the batch: the per-sample plan
(FP64 index selection, sort, deduplication; made once per step and shared by
gridding and degridding, as the reference's planned taps are), gridding of
PSF and dirty grids and degridding of a model grid, with inputs resident in
HBM.  Inputs are
larger than L2, so no flush is needed between steps.  `e2e` repeats the same
work through the reference-facing calls with host buffers (host -> device
copies, the dirty image and the model visibilities back to host).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "casa-rs_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Mvis/s grid+degrid (4096^2, W-proj)"
UNIT = "Mvis/s"
PLANES, SAMPLING, SUPPORT_LAW = 128, 8, (8, 64)
SEED = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rows-fraction", type=float, default=1.0,
                    help="use every k-th row (profiling runs only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cube", action="store_true",
                    help="skip the batched-cube versus per-channel-loop comparison")
    ap.add_argument("--cube-channels", type=int, default=256)
    ap.add_argument("--no-rows", action="store_true", help="skip the row-runs measurement")
    ap.add_argument("--no-feed", action="store_true",
                    help="skip the row-block read-ahead feed measurement")
    ap.add_argument("--feed-only", action="store_true",
                    help="run only the row-block feed measurement (profiling runs)")
    ap.add_argument("--fft-only", action="store_true",
                    help="run only the image-stage transform measurement (profiling runs)")
    ap.add_argument("--no-major-minor", action="store_true",
                    help="skip the device-resident major/minor CLEAN loop")
    ap.add_argument("--cube-only", action="store_true",
                    help="run only the cube comparison (profiling runs)")
    ap.add_argument("--cube-no-plain", action="store_true",
                    help="time only the batched cube path (profiling runs)")
    return ap.parse_args()


def max_over_ranks(x: float, device) -> float:
    """The slowest rank's time: all_reduce(MAX) over the process group (a
    no-op for one process)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mvis(world: int, accepted_per_rank: int, ms_per_step: float) -> float:
    """Replicas each process the full batch: all ranks' samples over the
    slowest rank's step time, in Mvis/s."""
    return world * accepted_per_rank / (ms_per_step * 1e-3) / 1e6


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(fraction=1.0):
    from casars_cuda import synthetic as S
    obs = S.wproj_4096_observation(SEED)
    if fraction < 1.0:
        k = max(1, int(round(1.0 / fraction)))
        obs.u, obs.v, obs.w = obs.u[::k].copy(), obs.v[::k].copy(), obs.w[::k].copy()
    return obs


def algorithmic_bytes(rows, grid_cells):
    """Compulsory bytes of one pass.  Grid: u,v,w f64 (24) + vis c64, weight
    f32 and flag u8 (13) per row, then 12 B per grid cell (dirty c64 + PSF
    f32) written once.  Degrid: u,v,w + flag per row, the model visibility
    written (8), the model grid (c64) read once."""
    grid = rows * (24 + 13) + grid_cells * 12
    degrid = rows * (24 + 1 + 8) + grid_cells * 8
    return grid, degrid


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons while timing."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": mx or None, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_rate(obs, kernels, norm, support, w_scale, model_grid, budget_s=12.0):
    """The reference CPU path restated in C (multi-threaded like the reference,
    in its Complex32 grid precision, gridder.rs:3680-3747) timed on host
    cores: grid + degrid of a bounded, evenly strided sample of the same rows,
    with the same kernels."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    geom = O.Geometry(obs.nx, obs.ny, obs.cell, obs.cell)
    og = O.StdGridder(geom, 100)
    wp = O.WProjector.from_arrays(geom, og, w_scale, support, kernels.astype(np.complex128),
                                  norm.astype(np.float64), SAMPLING)
    mg = np.asarray(model_grid, np.complex64)
    rng = np.random.default_rng(SEED)
    vis = (rng.normal(size=len(obs.u)) + 1j * rng.normal(size=len(obs.u))).astype(np.complex64)
    wt = np.ones(len(obs.u), np.float32)

    def run(stride):
        sl = slice(0, None, stride)
        u, v, w = obs.u[sl], obs.v[sl], obs.w[sl]
        t0 = time.perf_counter()
        _, _, acc = wp.grid_dirty_f32(u, v, w, wt[sl], vis[sl], threads=threads)
        wp.degrid_f32(mg, u, v, w, threads=threads)
        return acc.gridded, time.perf_counter() - t0

    # The reference scheme allocates, zeroes and merges one full grid pair per
    # thread, a fixed cost per call.  Two sample sizes give t = a + b * rows;
    # the figure reported is the rate of one call over the whole workload.
    n1, t1 = run(2048)
    stride = max(16, int(2048 * max(t1, 1e-3) / budget_s * 4))
    stride = min(stride, 512)
    n2, t2 = run(stride)
    b = max((t2 - t1) / max(n2 - n1, 1), 1e-12)
    a = max(t1 - b * n1, 0.0)
    rows = len(obs.u)
    rate = rows / (a + b * rows) / 1e6
    return rate, threads, (f"grid+degrid of every 2048th and every {stride}th row ({n1} and {n2} rows), "
                           f"{threads} threads; t = a + b*rows fit (a = {a:.3f} s, b = {b * 1e6:.3f} us/row) "
                           f"evaluated at {rows} rows")


def run_cube(args, ctx, dev, peak):
    """The 256-channel cube (1.0-2.0 GHz, 1024^2 image, 1,263,600 rows per
    channel, per-channel flag fraction uniform in 0-60 %, Briggs robust 0.5,
    PSWF support 3 at oversampling 128): the batched path (one plan of all
    channels, one gridding launch, one degridding launch) against the plain
    single-channel GPU path called channel by channel, both from inputs in
    HBM.  Mvis/s counts the gridded (unflagged, in-grid) samples."""
    import torch
    import casars_cuda as cc
    from casars_cuda import synthetic as S
    obs = S.cube_observation(channels=args.cube_channels)
    flags, vis = S.cube_device_inputs(obs, dev)
    C, R = obs.channels, obs.rows
    um = torch.as_tensor(obs.u_m, device=dev)
    vm = torch.as_tensor(obs.v_m, device=dev)
    wt = torch.ones((C, R), dtype=torch.float32, device=dev)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), 128)
    gs = (C,) + tuple(gg.grid_shape())
    model = torch.zeros(gs, dtype=torch.complex64, device=dev)
    model[:, gs[1] // 2, gs[2] // 2] = 1.0
    cube = cc.CubeBatch(um, vm, obs.lambda_scale, vis, wt, flags)
    torch.cuda.synchronize()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(steps):
            fn()
        e.record()
        torch.cuda.synchronize()
        return s.elapsed_time(e) / steps

    last = {}

    def batched_grid():
        _, _, last["sums"] = cc.cube_grid_dirty(gg, cube, "briggs", 0.5)
        last["t"] = ctx.last_timings()

    def batched_both():
        cc.cube_grid_degrid(gg, cube, model, "briggs", 0.5)
        last["t2"] = ctx.last_timings()

    steps = max(1, min(args.steps, 10))
    # a repeated all-device call runs eagerly once (tuning the gridding
    # chunk), is captured into a CUDA graph on the second and replayed after
    ms_grid = timed(batched_grid, steps, 3)
    ms_both = timed(batched_both, steps, 3)
    # the per-stage breakdown comes from eager calls (a replay is one stage)
    ctx.set_cube_graphs(False)
    ms_grid_eager = timed(batched_grid, steps, 1)
    t_grid = last["t"]
    ms_both_eager = timed(batched_both, steps, 1)
    t_both = last["t2"]
    ctx.set_cube_graphs(True)
    n_vis = sum(s.gridded_samples for s in last["sums"])

    # a resident plan (the cube CLEAN's major cycle): weighting and records
    # once, then per pass the batched residual refresh (degrid the model
    # grids, grid w (vis - pred)) and the image stage around it
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    plan = cc.CubePlan(gg, cube, "briggs", 0.5)
    ev1.record()
    torch.cuda.synchronize()
    ms_plan_create = ev0.elapsed_time(ev1)
    res_grids = torch.empty(gs, dtype=torch.complex64, device=dev)
    ms_refresh = timed(lambda: plan.grid_residual(model, out=res_grids), steps, 2)
    t_refresh = ctx.last_timings()
    pg = torch.empty(gs, dtype=torch.float32, device=dev)
    dg = torch.empty(gs, dtype=torch.complex64, device=dev)
    ms_plan_grid = timed(lambda: plan.grid_dirty(out=(pg, dg)), steps, 2)
    del pg, dg
    _, _, states = plan.dirty_images()
    models = torch.zeros((C, obs.nx, obs.nx), dtype=torch.float32, device=dev)
    models[:, obs.nx // 2, obs.nx // 2] = 1.0
    res_imgs = torch.empty_like(models)
    ms_refresh_img = timed(lambda: plan.residual_images(models, states, out=res_imgs), 2, 1)
    t_img = ctx.last_timings()
    # the same refresh with FP64 transforms, and how far the float32 images
    # are from it (peak-normalised, worst plane)
    plan.set_fft_precision(64)
    res64 = torch.empty_like(models)
    ms_refresh_img64 = timed(lambda: plan.residual_images(models, states, out=res64), 1, 1)
    t_img64 = ctx.last_timings()
    plan.set_fft_precision(32)
    img_err = float(torch.max(torch.amax(torch.abs(res_imgs - res64), dim=(1, 2)) /
                              torch.amax(torch.abs(res64), dim=(1, 2)).clamp_min(1e-30)))
    plan.close()
    del res_grids, res_imgs, res64, models

    # the cube CLEAN (run_standard_mfs_cube_clean): one persistent plan, the
    # PSF and residual planes, synchronized passes of per-plane Hogbom minor
    # cycles with one batched residual refresh per pass (PSF sidelobe level
    # fixed at 0.2 so that no beams are fitted; no restoration)
    clean_cfg = cc.CleanConfig(niter=C * 60, gain=0.1, minor_cycle_length=20)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cl = cc.run_cube_clean(gg, cube, clean_cfg, "briggs", 0.5, max_psf_sidelobe=0.2,
                           restore=False)
    torch.cuda.synchronize()
    clean_wall = time.perf_counter() - t0
    clean_out = {"wall_s": clean_wall, "passes": cl.major_cycles,
                 "minor_iterations": cl.minor_iterations,
                 "active_planes_per_pass": [len(a) for a in cl.active_planes],
                 "config": "niter 60 x channels, minor cycle length 20, gain 0.1, "
                           "Briggs 0.5, sidelobe 0.2"}
    del cl

    # the plain loop: per channel, the single-channel API on that channel's
    # batch (flagged samples carry gridable = 0 and weight 0)
    lsd = torch.as_tensor(obs.lambda_scale, device=dev)
    uc = [um * lsd[c] for c in range(C)]
    vc = [vm * lsd[c] for c in range(C)]
    wc = torch.where(flags.bool(), torch.zeros_like(wt), wt)
    gridable = (1 - flags).contiguous()

    def plain(degrid):
        for c in range(C):
            b = cc.VisibilityBatch(uc[c], vc[c], vis[c], wc[c], gridable=gridable[c])
            w1, _ = cc.apply_weighting(gg, b, "briggs", 0.5, per_plane=True)
            b1 = cc.VisibilityBatch(uc[c], vc[c], vis[c], w1, gridable=gridable[c])
            if degrid:
                p = cc.Plan(gg, b1)
                p.grid_dirty()
                p.degrid(model[c])
                p.close()
            else:
                cc.grid_dirty(gg, b1)

    psteps = 2
    if args.cube_no_plain:
        ms_plain = ms_plain_both = float("nan")
    else:
        ms_plain = timed(lambda: plain(False), psteps, 1)
        ms_plain_both = timed(lambda: plain(True), psteps, 1)
    cells = gs[1] * gs[2]
    S_all = C * R
    b_grid = R * 24 + S_all * 13 + C * cells * 12
    b_degrid = R * 24 + S_all * 9 + C * cells * 8
    gk = t_grid["grid_kernel_ms"]
    return {
        "workload": f"{C}-channel cube 1.0-2.0 GHz, 1024^2 image (grid {gs[1]}^2), "
                    f"{R} rows per channel, flag fraction U(0, 0.6) per channel, "
                    "Briggs robust 0.5, PSWF support 3 (7x7 taps), oversampling 128",
        "gridded_vis": n_vis, "samples": S_all,
        "batched": {"grid_ms": ms_grid, "grid_degrid_ms": ms_both, "graph_replay": True,
                    "eager_grid_ms": ms_grid_eager, "eager_grid_degrid_ms": ms_both_eager,
                    "grid_mvis_s": n_vis / (ms_grid * 1e-3) / 1e6,
                    "grid_degrid_mvis_s": n_vis / (ms_both * 1e-3) / 1e6,
                    "stages_ms": {"plan": t_grid["plan_ms"], "grid": t_grid["grid_ms"],
                                  "cube_grid_kernel": gk,
                                  "degrid": t_both["degrid_ms"],
                                  "cube_degrid_kernel": t_both["degrid_kernel_ms"]}},
        "resident_plan": {"create_ms": ms_plan_create, "grid_ms": ms_plan_grid,
                          "grid_mvis_s": n_vis / (ms_plan_grid * 1e-3) / 1e6,
                          "residual_refresh_ms": ms_refresh,
                          "residual_refresh_mvis_s": n_vis / (ms_refresh * 1e-3) / 1e6,
                          "refresh_kernels_ms": {"cube_degrid_kernel_residual":
                                                 t_refresh["degrid_kernel_ms"],
                                                 "cube_grid_kernel_residual":
                                                 t_refresh["grid_kernel_ms"]},
                          "residual_images_ms": ms_refresh_img,
                          "residual_images_fft_ms": t_img["fft_ms"],
                          "residual_images_fp64_ms": ms_refresh_img64,
                          "residual_images_fp64_fft_ms": t_img64["fft_ms"],
                          "float32_vs_fp64_image_err": img_err},
        "cube_clean": clean_out,
        "plain_loop": {"grid_ms": ms_plain, "grid_degrid_ms": ms_plain_both,
                       "grid_mvis_s": n_vis / (ms_plain * 1e-3) / 1e6,
                       "grid_degrid_mvis_s": n_vis / (ms_plain_both * 1e-3) / 1e6},
        "speedup_grid": ms_plain / ms_grid,
        "speedup_grid_degrid": ms_plain_both / ms_both,
        "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak,
                     "algorithmic_bytes_grid_pass": b_grid,
                     "algorithmic_bytes_degrid_pass": b_degrid,
                     "grid_pass_achieved": b_grid / (ms_grid * 1e-3) / 1e9,
                     "grid_pass_frac": b_grid / (ms_grid * 1e-3) / 1e9 / peak,
                     "grid_degrid_pass_achieved": (b_grid + b_degrid) / (ms_both * 1e-3) / 1e9,
                     "grid_degrid_pass_frac": (b_grid + b_degrid) / (ms_both * 1e-3) / 1e9 / peak},
    }


def run_rows(args, ctx, dev, peak):
    """Row runs to samples on the device (cr_row_runs_prepare): the cube's
    rows (1,263,600 of them, 27 antennas to 1 km, 10 h of 10 s dumps) with 64
    channels over 1.0-2.0 GHz and 4 correlations (XX, XY, YX, YY), 10 %
    flags, a weight spectrum, Stokes I (XX + YY collapsed).  Inputs in HBM;
    GB/s counts the bytes the kernels must move once: per (row, channel) the
    two used correlations' data, flags and spectrum weights, per row its
    uvw, and per kept sample the batch written (57 B)."""
    import torch
    import casars_cuda as cc
    from casars_cuda import synthetic as S
    obs = S.cube_observation(channels=64)
    R, C, K = obs.rows, obs.channels, 4
    g = torch.Generator(device=dev).manual_seed(11)
    data = torch.randn((R, C, K), dtype=torch.complex64, device=dev, generator=g)
    flag = (torch.rand((R, C, K), device=dev, generator=g) < 0.1).to(torch.uint8)
    spec = torch.rand((R, C, K), device=dev, generator=g) + 0.5
    uvw = torch.as_tensor(np.stack([obs.u_m, obs.v_m, np.zeros_like(obs.u_m)], 1), device=dev)
    runs = cc.RowRuns(uvw, obs.lambda_scale, data, flag, None, spec, None)
    pol = cc.Polarization.for_plane("I", [9, 10, 11, 12])
    for _ in range(2):
        b, _, _ = cc.prepare_row_runs(ctx, runs, pol)
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 10))
    t_ms = []
    for _ in range(steps):
        b, _, _ = cc.prepare_row_runs(ctx, runs, pol)
        t_ms.append(ctx.last_timings()["plan_ms"])
    ms = float(np.median(t_ms))
    kept = len(b)
    algo = R * C * 2 * (8 + 1 + 4) + R * 24 + kept * 57
    del data, flag, spec, b
    torch.cuda.empty_cache()
    return {"workload": f"{R} rows x {C} channels x {K} correlations, Stokes I from XX+YY, "
                        "10 % flags, weight spectrum",
            "samples": R * C, "kept": kept, "ms": ms, "msamples_s": R * C / (ms * 1e-3) / 1e6,
            "algorithmic_bytes": algo, "achieved_gbs": algo / (ms * 1e-3) / 1e9,
            "frac_of_measured_hbm": algo / (ms * 1e-3) / 1e9 / peak}


def run_feed(args, ctx, dev):
    """The row-block read-ahead feed (cr_row_feed_*): the cube's rows
    (1,263,600, 27 antennas to 1 km, 10 h of 10 s dumps) with 16 channels
    over 1.0-2.0 GHz and 4 correlations, 10 % flags, a weight spectrum,
    Stokes I into a 1024^2 image, natural weights.  A producer copies each
    block of 65,536 rows from host arrays (the reader's output) into the
    feed's page-locked slot; the feed uploads it and prepares and grids it
    on the device while the next block is filled.  Timed on the host clock
    from the first acquire to the images of finish(), against the same work
    with the whole input already on the device (one prepare, one
    accumulation, finish) and against a read-ahead depth of 1."""
    import time

    import torch
    import casars_cuda as cc
    from casars_cuda import synthetic as S
    obs = S.cube_observation(channels=16)
    R, C, K = obs.rows, obs.channels, 4
    rng = np.random.default_rng(31)
    data = rng.standard_normal((R, C, 2 * K), dtype=np.float32).view(np.complex64)
    flag = (rng.random((R, C, K), dtype=np.float32) < 0.1).astype(np.uint8)
    spec = rng.random((R, C, K), dtype=np.float32) + np.float32(0.5)
    uvw = np.stack([obs.u_m, obs.v_m, np.zeros_like(obs.u_m)], 1)
    weight = np.ones((R, K), np.float32)
    pol = cc.Polarization.for_plane("I", [9, 10, 11, 12])
    geom = cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell)
    block = 65536
    fill_s = [0.0]

    def producer():
        pos = [0]

        def produce(slot):
            r0 = pos[0]
            if r0 >= R:
                return None
            t0 = time.perf_counter()
            n = min(block, R - r0)
            sl = slice(r0, r0 + n)
            np.copyto(slot.uvw_m[:n], uvw[sl])
            np.copyto(slot.data[:n], data[sl])
            np.copyto(slot.flag[:n], flag[sl])
            np.copyto(slot.weight[:n], weight[sl])
            np.copyto(slot.weight_spectrum[:n], spec[sl])
            pos[0] = r0 + n
            fill_s[0] += time.perf_counter() - t0
            return n

        return produce

    def fed(live):
        gg = cc.StandardGridder(ctx, geom, 128)
        feed = cc.RowFeed(gg, obs.lambda_scale, pol, K, block, live, has_flag=True,
                          has_weight_spectrum=True)
        try:
            fill_s[0] = 0.0
            t0 = time.perf_counter()
            cc.stream_row_blocks(feed, producer())
            psf, res, _, sums, summary = feed.finish()
            return time.perf_counter() - t0, fill_s[0], sums, summary, res
        finally:
            feed.close()

    fed(2)                                   # warm-up: plans, workspaces
    runs = [fed(2) for _ in range(2)]
    wall, fill, sums, summary, res = min(runs, key=lambda r: r[0])
    wall1 = min(fed(1)[0] for _ in range(2))
    # the same work with the whole input resident in HBM
    tt = lambda a: torch.from_numpy(a).to(dev)
    rr = cc.RowRuns(tt(uvw), obs.lambda_scale, tt(data), tt(flag), tt(weight), tt(spec), None)
    gg = cc.StandardGridder(ctx, geom, 128)

    def resident():
        ctx.use_torch_stream()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b, _, _ = cc.prepare_row_runs(ctx, rr, pol)
        acc = cc.DirtyAccumulator(gg)
        acc.add(b)
        _, r_img, _, s = acc.finish()
        torch.cuda.synchronize()
        out = time.perf_counter() - t0
        acc.close()
        return out, r_img, s

    resident()
    res_runs = [resident() for _ in range(2)]
    t_res, r_img, s_res = min(res_runs, key=lambda r: r[0])
    ctx.use_own_stream()
    err = float(np.max(np.abs(res - r_img.cpu().numpy())) / max(np.max(np.abs(res)), 1e-30))
    del rr
    torch.cuda.empty_cache()
    return {"workload": f"{R} rows x {C} channels x {K} correlations in blocks of {block} rows, "
                        "Stokes I from XX+YY, 10 % flags, weight spectrum, 1024^2 image, "
                        "natural weights, host arrays copied into the feed's slots",
            "rows": R, "samples": R * C, "kept": summary.streamed_samples,
            "gridded": sums.gridded_samples, "source_bytes": summary.source_bytes,
            "wall_s": wall, "rows_per_s": R / wall, "source_gbs": summary.source_bytes / wall / 1e9,
            "read_ahead": 2, "wall_s_read_ahead_1": wall1,
            "producer_fill_s": fill, "consumer_elapsed_s": summary.consumer_elapsed_s,
            "producer_send_blocked_s": summary.producer_send_blocked_s,
            "consumer_recv_blocked_s": summary.consumer_recv_blocked_s,
            "producer_consumer_overlap_s": summary.producer_consumer_overlap_s,
            "live_row_block_high_water": summary.live_row_block_high_water,
            "row_blocks": summary.row_blocks,
            "device_resident_s": t_res, "residual_vs_device_resident": err,
            "gridded_equal": int(s_res.gridded_samples) == int(sums.gridded_samples)}


def run_image_stage(args, ctx, dev):
    """The FP64-grade image-stage transforms at the headline size: a random
    complex 5000^2 grid to the 4096^2 image (inverse transform, crop,
    correction) and a random 4096^2 model image to its grid (apodisation,
    forward transform), each timed with CUDA events on the context's
    stream, with the float-pair kernels (the default engine) and with cuFFT
    FP64."""
    import torch
    import casars_cuda as cc
    nx = 4096
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, 1.5e-6, 1.5e-6), 100)
    gs = gg.grid_shape()
    g = torch.Generator(device=dev).manual_seed(5)
    grid = torch.complex(torch.randn(gs, device=dev, generator=g),
                         torch.randn(gs, device=dev, generator=g))
    model = torch.randn((nx, nx), device=dev, generator=g)
    reps = max(1, min(args.steps, 10))
    out = {"workload": f"{nx}^2 image, {gs[0]}^2 grid, random complex grid and model image"}
    for engine in ("auto", "cufft"):
        ctx.set_image_fft_engine(engine)
        for name, fn in (("grid_to_image_ms", lambda: cc.grid_to_image(gg, grid, 1.0)),
                         ("image_to_grid_ms", lambda: cc.image_to_grid(gg, model))):
            for _ in range(max(args.warmup, 1)):
                fn()
            ts = []
            for _ in range(reps):
                stream = torch.cuda.current_stream(dev)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                torch.cuda.synchronize(dev)
                ts.append(a.elapsed_time(b))
            key = "float_pair" if engine == "auto" else "cufft_fp64"
            out.setdefault(key, {})[name] = float(np.median(ts))
    ctx.set_image_fft_engine("auto")
    del grid, model
    torch.cuda.empty_cache()
    return out


def run_major_minor(args, ctx, dev):
    """The device-resident major/minor loop: 2048^2 Stokes I, 10,108,800
    visibilities (21 km layout, 4 channels 1.3-1.5 GHz gridded together), 64
    w-planes (the reference's support search, sampling 4), 300 points + 5
    Gaussians, Hogbom gain 0.1, 2000 minor iterations per major cycle, 6
    major cycles, threshold 3 sigma with sigma the image-plane thermal noise
    of natural weighting, sigma_vis / sqrt(N).
    Wall time covers the dirty image, the plan and every cycle; the model
    visibilities are the model image's predicted visibilities plus 5 mJy
    noise."""
    import torch
    import casars_cuda as cc
    from casars_cuda import synthetic as S
    obs, model = S.major_minor_2048_observation(5)
    T = lambda a: torch.as_tensor(a, device=dev)
    u, v, w = T(obs.u), T(obs.v), T(obs.w)
    n = obs.rows
    wt = torch.ones(n, dtype=torch.float32, device=dev)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell))
    gw = cc.WProjector(gg, float(np.abs(obs.w).max()), planes=64)
    vis = cc.predict(gg, cc.VisibilityBatch(u, v, torch.zeros(n, dtype=torch.complex64,
                                                               device=dev), wt, w), T(model), gw)
    g = torch.Generator(device=dev)
    g.manual_seed(55)
    vis = vis + 5e-3 * torch.complex(torch.randn(n, generator=g, device=dev),
                                     torch.randn(n, generator=g, device=dev))
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    sigma = 5e-3 / math.sqrt(n)
    cfg = cc.CleanConfig(niter=12000, gain=0.1, threshold_jy_per_beam=3.0 * sigma,
                         minor_cycle_length=2000, cyclefactor=0.0, min_psf_fraction=0.0,
                         major_cycle_limit=6)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = cc.run_cotton_schwab(gg, b, cfg, wproj=gw, max_psf_sidelobe=0.0)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    support = gw.tables()[0]
    return {"workload": "2048^2, 10,108,800 vis (21 km, 4 ch 1.3-1.5 GHz MFS), "
                        f"64 w-planes (support {int(support.min())}-{int(support.max())}), "
                        "300 points + 5 Gaussians, Hogbom gain 0.1, 2000 minor x 6 major, "
                        "threshold 3 sigma",
            "wall_s": wall, "major_cycles": out.major_cycles,
            "minor_iterations": out.minor_iterations, "stop_reason": out.stop_reason,
            "threshold_jy": 3.0 * sigma,
            "final_residual_peak": float(torch.max(torch.abs(out.residual))),
            "model_flux_jy": float(torch.sum(out.model))}


def run_reference(args):
    """Reference arm: the reference's CPU path (restated in C; the Rust
    original cannot be built here) on the host cores, with W-kernels built by
    the FP64 oracle and gridded / degridded in the reference's Complex32
    precision, timed per step on a bounded sample of the same workload and
    extrapolated to all rows by t = a + b rows (the sample line says how)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    obs = workload(1.0)
    threads = os.cpu_count() or 1
    geom = O.Geometry(obs.nx, obs.ny, obs.cell, obs.cell)
    og = O.StdGridder(geom, 100)
    wp = O.WProjector(geom, og, float(np.abs(obs.w).max()), planes=PLANES, sampling=SAMPLING,
                      support_min=SUPPORT_LAW[0], support_max=SUPPORT_LAW[1], threads=threads)
    rng = np.random.default_rng(SEED)
    n_all = len(obs.u)
    vis = (rng.normal(size=n_all) + 1j * rng.normal(size=n_all)).astype(np.complex64)
    wt = np.ones(n_all, np.float32)
    mg = np.zeros((og.gnx, og.gny), np.complex64)
    mg[og.gnx // 2, og.gny // 2] = 1.0
    stride = 400  # ~12.6k rows per step

    def step(stride):
        sl = slice(0, None, stride)
        t0 = time.perf_counter()
        _, _, acc = wp.grid_dirty_f32(obs.u[sl], obs.v[sl], obs.w[sl], wt[sl], vis[sl],
                                      threads=threads)
        wp.degrid_f32(mg, obs.u[sl], obs.v[sl], obs.w[sl], threads=threads)
        return acc.gridded, time.perf_counter() - t0

    # The reference scheme's per-call cost has a fixed part (one full grid
    # pair per thread, zeroed and merged) and a per-row part.  The warm-up
    # measures the fixed part on a tiny sample; each step times a strided
    # sample, and the rate is that of one call over all rows:
    # rows / (a + b rows).
    a_fixed = min(step(n_all // 64)[1] for _ in range(max(args.warmup, 1)))
    n_tiny = len(range(0, n_all, n_all // 64))
    rates, ms, tot_n = [], [], 0
    for _ in range(args.steps):
        n, t = step(stride)
        tot_n += n
        b = max((t - a_fixed) / max(n - n_tiny, 1), 1e-12)
        rates.append(n_all / (a_fixed + b * n_all) / 1e6)
        ms.append(1e3 * t)
    value = float(np.median(rates))
    tot_t = sum(ms) / 1e3
    sample = (f"every {stride}th row ({tot_n // max(args.steps, 1)} rows) per step, grid+degrid; "
              f"rate of one call over all {n_all} rows from t = a + b*rows "
              f"(a = {a_fixed:.3f} s measured on every {n_all // 64}th row)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot_t / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 (the reference's Complex32 grids)",
            "data": "synthetic",
            "config": {"workload": "W-proj dirty 4096^2, 5,054,400 rows, 128 planes, "
                                   "support 8-64, oversampling 8", "rows": n_all,
                       "sample_rows_per_step": tot_n // max(args.steps, 1)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist

    import casars_cuda as cc
    from casars_cuda import synthetic as S

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    ctx = cc.Context(local)
    if args.feed_only:
        print(json.dumps({"row_feed": run_feed(args, ctx, dev)}), flush=True)
        return
    if args.fft_only:
        print(json.dumps({"image_stage": run_image_stage(args, ctx, dev)}), flush=True)
        return
    if args.cube_only:
        print(json.dumps({"cube": run_cube(args, ctx, dev, measured_peaks()[0])}), flush=True)
        return
    obs = workload(args.rows_fraction)
    n = obs.rows
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.ny, obs.cell, obs.cell), 100)
    gw = cc.WProjector(gg, float(np.abs(obs.w).max()), planes=PLANES, sampling=SAMPLING,
                       support_law=SUPPORT_LAW)
    u = torch.as_tensor(obs.u, device=dev)
    v = torch.as_tensor(obs.v, device=dev)
    w = torch.as_tensor(obs.w, device=dev)
    vis = S.visibilities_torch(obs.u, obs.v, obs.w, obs.sky, obs.nx, obs.ny, obs.cell, 5e-3,
                               SEED, device=dev)
    wt = torch.ones(n, dtype=torch.float32, device=dev)
    batch = cc.VisibilityBatch(u, v, vis, wt, w)
    model = torch.as_tensor(S.model_image(obs.sky, obs.nx, obs.ny), device=dev)
    model_grid = cc.image_to_grid(gg, model, gw)
    torch.cuda.synchronize()

    plan_ms, grid_ms, degrid_ms, gk_ms, dk_ms = [], [], [], [], []
    last = {}

    def step(record):
        # one pass over the batch: plan (FP64 indices, sort, deduplication),
        # grid PSF + dirty, degrid the model grid
        plan = cc.Plan(gg, batch, gw)
        tp = ctx.last_timings()
        psf, dirty = plan.grid_dirty()
        tg = ctx.last_timings()
        pred = plan.degrid(model_grid)
        td = ctx.last_timings()
        if record:
            plan_ms.append(tp["plan_ms"])
            grid_ms.append(tg["grid_ms"])
            degrid_ms.append(td["degrid_ms"])
            gk_ms.append(tg["grid_kernel_ms"])
            dk_ms.append(td["degrid_kernel_ms"])
        last["sums"] = plan.sums
        plan.close()
        return pred

    for _ in range(max(args.warmup, 0)):
        step(False)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    # the timed steps run with the library's per-call stage timings off (they
    # make every call wait for its events); the stage and kernel times come
    # from as many steps right after, with the timings on
    ctx.set_timings(False)
    launches0 = ctx.launch_count
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        start.record()
        for _ in range(args.steps):
            step(False)
        end.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(end) / args.steps
    launches = (ctx.launch_count - launches0)
    ctx.set_timings(True)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(args.steps):
        step(True)
    t1.record()
    torch.cuda.synchronize()
    ms_timed_stages = t0.elapsed_time(t1) / args.steps
    if world > 1:
        ms = max_over_ranks(ms, dev)
        dist.barrier()
    sums = last["sums"]
    accepted = sums.gridded_samples
    value = whole_job_mvis(world, accepted, ms)

    # dominant kernel roofline: wp_grid_kernel, timed alone with CUDA events
    # on the launching stream
    gcells = gg.grid_shape()[0] * gg.grid_shape()[1]
    b_grid, b_degrid = algorithmic_bytes(n, gcells)
    g_ms = statistics.mean(grid_ms)
    d_ms = statistics.mean(degrid_ms)
    gk = statistics.mean(gk_ms)
    dk = statistics.mean(dk_ms)
    peak, peak_kind = measured_peaks()
    achieved = b_grid / (gk * 1e-3) / 1e9

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 index selection and sums)", "data": "synthetic",
        "config": {"workload": "W-proj dirty 4096^2 (grid 5000^2), 5,054,400 rows, "
                               "1 channel, 128 w-planes, support 8-64 linear in plane, "
                               "oversampling 8, 200 points + 5 mJy noise",
                   "rows": n, "rows_fraction": args.rows_fraction,
                   "unique_records": sums.unique_records, "parallelism": f"replicas{world}",
                   "l2": "inputs (0.19 GB rows + 0.2 GB model grid + 0.4 GB output grids) exceed L2"},
        "gpu_launches": launches,
        "stages_ms": {"plan": statistics.mean(plan_ms), "grid": g_ms, "degrid": d_ms,
                      "wp_grid_kernel": gk, "wp_degrid_kernel": dk,
                      "measured": f"{args.steps} steps after the timed ones, with the per-call "
                                  f"stage timings on ({ms_timed_stages:.3f} ms per step)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "traffic_note": "DRAM bytes per launch come from an ncu capture, "
                                     "not from this run",
                     "kernel": "wp_grid_kernel", "peak_kind": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": b_grid,
                     "degrid": {"kernel": "wp_degrid_kernel", "algorithmic_bytes_per_launch":
                                b_degrid, "achieved": b_degrid / (dk * 1e-3) / 1e9,
                                "frac": b_degrid / (dk * 1e-3) / 1e9 / peak}},
        # the path's binding limit for W-projection: kernel taps per second
        "taps": {"per_pass": sums.taps, "grid_per_s": sums.taps / (gk * 1e-3),
                 "degrid_per_s": sums.taps / (dk * 1e-3)},
        "clocks": clk.summary(),
    }
    # the tap-rate ceiling: one L2-resident kernel value and three paired
    # FMAs per tap, nothing else (cr_probe_tap_rate), on a buffer the size of
    # this W-projector's kernel cube
    floor_rate, _ = cc.probe_tap_rate(ctx, int(gw.info.cube_elements) * 8, 256)
    result["roofline"]["tap_bound"] = {
        "unit": "taps/s", "ceiling": floor_rate,
        "grid_achieved": sums.taps / (gk * 1e-3), "grid_frac": sums.taps / (gk * 1e-3) / floor_rate,
        "degrid_achieved": sums.taps / (dk * 1e-3),
        "degrid_frac": sums.taps / (dk * 1e-3) / floor_rate,
        "ceiling_kernel": "tap_probe_kernel: per tap one float2 L2 load + 3 paired FP32 FMAs"}

    if not args.no_e2e:
        # the reference-facing calls with host (pinned) buffers
        hu, hv, hw = (torch.as_tensor(a).pin_memory() for a in (obs.u, obs.v, obs.w))
        hvis = vis.cpu().pin_memory()
        hwt = wt.cpu().pin_memory()
        hmodel = model.cpu().pin_memory()
        hb = cc.VisibilityBatch(hu, hv, hvis, hwt, hw)

        def e2e_step():
            cc.dirty_image(gg, hb, gw)
            cc.predict(gg, hb, hmodel, gw)

        e2e_steps = max(1, min(args.steps, 5))

        def e2e_ms():
            e2e_step()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                e2e_step()
            torch.cuda.synchronize()
            return (time.perf_counter() - t0) * 1e3 / e2e_steps

        e_ms = e2e_ms()
        # the dirty-product policy's F32 choice for the image stage (the
        # headline keeps the FP64 default)
        ctx.set_image_fft_precision("f32")
        e32_ms = e2e_ms()
        ctx.set_image_fft_precision("auto")
        row_bytes = 24 + 8 + 4
        result["e2e"] = {"value": world * accepted / (e_ms * 1e-3) / 1e6, "unit": UNIT,
                         "h2d_bytes_per_step": 2 * n * row_bytes + obs.nx * obs.ny * 4,
                         "d2h_bytes_per_step": 2 * obs.nx * obs.ny * 4 + n * 8,
                         "ms_per_step": e_ms, "calls": "cr_dirty_image + cr_predict",
                         "image_fft": "f64-grade (float-pair transform kernels)",
                         "f32_image_fft": {"value": world * accepted / (e32_ms * 1e-3) / 1e6,
                                           "ms_per_step": e32_ms}}

    if not args.no_cube:
        result["cube"] = run_cube(args, ctx, dev, peak)
    if not args.no_rows:
        result["row_runs"] = run_rows(args, ctx, dev, peak)
    if not args.no_feed:
        result["row_feed"] = run_feed(args, ctx, dev)
    result["image_stage"] = run_image_stage(args, ctx, dev)
    if not args.no_major_minor:
        result["major_minor"] = run_major_minor(args, ctx, dev)

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        support, kern, norm = gw.tables()
        rate, cores, sample = cpu_rate(obs, kern, norm, support, gw.w_scale,
                                       model_grid.cpu().numpy())
        result["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                  "sample": sample}
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
