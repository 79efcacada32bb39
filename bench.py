"""Benchmark of the VoxelEncoding hot path on one GB300 (or N replicas).

Default workload (--workload batch, the batched training step): 8 frames of
4-8 synthetic RGBD views each at uneven resolutions from {512, 768,
1024}^2, each frame its own seeded scene (12 capsules/ellipsoids, 5 mm depth
noise, 2 % dropout, uint16 depth) fused into its own 256^3 TSDF grid (2 m
cube, 3 cm truncation, 8^3 bricks); 16 target cameras of uneven sizes (256^2
to 1024^2, 7.4 M rays in all) with 32-128 adaptive samples per ray.  One
step = fusion + tree build of all frames, intersection, forward render
(density from the fused TSDF, colour = a linear head over a seeded
256^3 x 16 feature grid per frame), the gradient of an L2 colour loss, and
the backward (exact compositing adjoint; one 32-byte record per used sample,
then a segmented reduction over the sorted cell keys adds the feature and
TSDF gradients into the grids without atomics, bit-identical run to run)
-- one launch per stage over all frames and targets, replayed from a CUDA
graph.  value = rays of all targets / step time.  The plain per-frame
forward-only launch sequence (the reference's call order through the
drop-in API: integrate, build_multi_res_volumes, octree, and per target
traversal with 256-wide padded hit rows, coarse sampling, sort, field
gathers, compositing) runs on the same inputs for the ratio.

--workload plain: one frame of 4 views at 1024^2 fused into a 512^3 grid,
a 1024^2 target with up to 96 samples, forward only.

e2e = the same step through the public API from pinned host buffers (images,
cameras, rays and target colours copied in; the rendered colours read
back); the batched step's e2e goes through
BatchPipeline.train_steps_from_host, which copies each step's inputs and
outputs beside the neighbouring steps.  The per-step working set (> 10 GB)
is far larger than L2.

--workload diff | project | octree | nerf: the differentiation step, the
sample projection + 2D feature gather, the multi-level tree path and
FastNerf's occupancy network (each described at its run_* function).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                  [--workload batch|plain|diff|project|octree|nerf]
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rays/s fwd+bwd batched vs plain per-frame, ≤1e-5 err; TSDF Gvox/s; 1 GB300"
UNIT = "rays/s"
CFG = dict(views=4, res=1024, prims=24, D=512, rate=8, trunc=0.02, target=1024, S=96, color_D=256, seed=7)
BATCH = dict(frames=8, views=(4, 8), view_res=(512, 768, 1024), prims=12, D=256, rate=8, trunc=0.03, C=16,
             targets=16, target_res=(256, 1024), target_S=(32, 48, 64, 96, 128), W_hits=256, sdf_s=0.005,
             seed=11)
BATCH_SMALL = dict(BATCH, frames=3, views=(2, 4), view_res=(256, 384), D=128, targets=5, target_res=(128, 256))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="small configuration (256^3, 512^2) for profiling")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--workload", default="batch", choices=["batch", "plain", "project", "diff", "octree", "nerf"])
    ap.add_argument("--unfused", action="store_true",
                    help="render with four kernels (sample+sort, two field gathers, composite) instead of one")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the oracle parity check of the timed step (run after timing)")
    return ap.parse_args()



def dist_env():
    """(world size, rank, local rank) of a torchrun launch; (1, 0, 0) alone."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def whole_job(ms_per_step, units_per_rank, world, device):
    """Replicas: every rank processes its own units_per_rank per step; the
    job's step time is the slowest rank's (max over ranks), and the job's
    throughput is world * units_per_rank over that time.  Returns (ms_max,
    units per second)."""
    import torch
    t = torch.tensor([float(ms_per_step)], device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    return ms_max, world * units_per_rank / (ms_max / 1000.0)

def workload(cfg, rank=0):
    from sailor_gb300 import synthetic as syn
    seed = cfg["seed"] + 1000 * rank
    sc = syn.make_scene(seed=seed, n_views=cfg["views"], res=cfg["res"], n_prims=cfg["prims"], D=cfg["D"],
                        trunc=cfg["trunc"])
    ori, dirs = syn.target_rays(seed=seed, res=cfg["target"])
    rng = np.random.default_rng(seed)
    Dc = cfg["color_D"]
    color_grid = rng.random((1, Dc, Dc, Dc, 3), dtype=np.float32)
    color_vs = np.full((1, 1), np.float32(2.0) / np.float32(Dc - 1), np.float32)
    return sc, ori, dirs, color_grid, color_vs


def algorithmic_bytes(cfg, n_hits, n_rays, S, n_pix):
    """Per-launch algorithmic HBM bytes of each stage."""
    D = cfg["D"]
    V = D ** 3
    Vt = (D // cfg["rate"]) ** 3
    return dict(
        fusion=16 * V + 8 * n_pix,                      # 4 output volumes + depth/colour images
        tree=4 * V + 4 * Vt,                            # fine occupancy read + coarse write
        intersect=24 * n_rays + 12 * n_hits + 8 * n_rays,
        # fused render: hit rows + per-ray count/valid length + ray ori/dir in,
        # 24 B/ray out (field-grid taps are cache-resident and not counted)
        render=12 * n_hits + 8 * n_rays + 24 * n_rays + 24 * n_rays,
        # unfused render stages
        sample=12 * n_hits + 8 * n_rays + 8 * n_rays * S,
        gather=2 * 4 * n_rays * S + 4 * n_rays * S + 12 * n_rays * S,
        composite=20 * n_rays * S + 24 * n_rays,
    )


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100", "-i", str(int(os.environ.get("LOCAL_RANK", 0)))],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        try:
            rows = [r.split(", ") for r in open(self.path).read().strip().splitlines()]
        except OSError:
            return None
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(rows)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_fused_grid(sc, cfg):
    """Whole-grid fusion by the oracle (untimed set-up of the CPU baseline:
    the tree and render stages need the complete grid)."""
    from oracle import oracle as orc
    return orc.integrate(sc["K"], sc["RT"], sc["colors"], sc["depths"], cfg["D"], sc["vol_bbox"],
                         sc["voxel_size"], trunc_weight=sc["trunc_weight"])


def cpu_baseline(sc, ori, dirs, cfg, color_grid, color_vs, ray_sample=16384, fusion_slab=32, fz=None):
    """The oracle (a C port of the reference kernels, OpenMP on all host
    cores) on a bounded sample of the step: fusion of an x-slab of the grid
    and the render stages of a ray subset, both scaled to the full step."""
    from oracle import oracle as orc
    D, S = cfg["D"], cfg["S"]
    n_rays = ori.shape[1]
    t0 = time.perf_counter()
    orc.integrate_slab(sc["K"], sc["RT"], sc["colors"], sc["depths"], D, sc["vol_bbox"], sc["voxel_size"],
                       0, fusion_slab, trunc_weight=sc["trunc_weight"])
    t_fuse = (time.perf_counter() - t0) * D / fusion_slab
    if fz is None:
        fz = cpu_fused_grid(sc, cfg)
    t0 = time.perf_counter()
    top, _ = orc.merge(fz["occ"], cfg["rate"])
    tree = orc.build_tree(top, fz["occ"])
    t_tree = time.perf_counter() - t0
    sel = np.linspace(0, n_rays - 1, ray_sample).astype(np.int64)
    o, d = ori[:, sel], dirs[:, sel]
    t0 = time.perf_counter()
    hits = orc.voxel_traversal(tree, o, d, sc["voxel_size"], sc["vol_bbox"], W=1024)
    si, sz, _ = orc.sample_coarse(tree, hits, np.full((1, ray_sample, S), 0.5, np.float32), sc["voxel_size"], S)
    srt, sidx = orc.sort(sz)
    pts = (o[0][:, None, :] + d[0][:, None, :] * np.maximum(srt[0], 0)[..., None]).reshape(-1, 3)
    tsdf = orc.grid_gather(pts, fz["tsdf"][..., None], sc["vol_bbox"][:, :, 0], sc["voxel_size"][:, 0])
    sdf = tsdf[:, 0] * float(sc["voxel_size"][0, 0]) * sc["trunc_weight"]
    sigma = (1.0 / (1.0 + np.exp(sdf / 0.005)) / 0.005).astype(np.float32).reshape(1, ray_sample, S, 1)
    rgb = orc.grid_gather(pts, color_grid, np.full((1, 3), -1.0, np.float32), color_vs[:, 0])
    rgb = rgb.astype(np.float32).reshape(1, ray_sample, S, 3)
    orc.composite_fwd(srt, None, sigma, rgb, 1e-4, False)
    t_render = (time.perf_counter() - t0) * n_rays / ray_sample
    t_step = t_fuse + t_tree + t_render
    return dict(value=n_rays / t_step, unit=UNIT, cores=orc.num_threads(), kind="port",
                sample=(f"oracle (C port, OpenMP) on host cores: fusion of x-slab {fusion_slab}/{D} scaled x"
                        f"{D // fusion_slab}, full coarse occupancy + tree build, render stages on "
                        f"{ray_sample} of {n_rays} rays scaled x{n_rays // ray_sample}"),
                stage_s=dict(fusion=t_fuse, tree=t_tree, render=t_render))


def run_reference(args):
    """--impl reference: the reference's CPU implementation of the path (the
    oracle port of its kernels), all host threads, on a bounded sample of
    the same workload as this arm per step.  Rank 0 alone runs and prints."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "batch":
        bcfg = dict(BATCH_SMALL if args.small else BATCH)
        w = batch_workload(bcfg)
        R = sum(t["ori"].shape[0] for t in w["targets"])
        runs = cpu_baseline_isolated(w, bcfg, reps=args.warmup + args.steps)[args.warmup:]
        cb = summarize_cpu_baseline(runs)
        v = cb["value"]
        ms = 1000.0 * float(np.median([r["sample_wall_s"] for r in runs]))
        out = dict(metric=METRIC, value=v, unit=UNIT, impl="reference", n_gpus=args.gpus, steps=args.steps,
                   warmup=args.warmup, ms_per_step=ms, higher_is_better=True, scaling="weak", vs_baseline=None,
                   dtype="f32", data="synthetic",
                   config=dict(workload=("batched training step (CPU port): %d frames, %d targets (%d rays); each "
                                         "step a bounded sample scaled to the whole step (ms_per_step: the "
                                         "sample's wall time)" % (bcfg["frames"], bcfg["targets"], R)),
                               l2="inputs > L2"),
                   cpu_baseline=cb, e2e=dict(value=v, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(out), flush=True)
        return
    else:
        cfg = dict(CFG)
        if args.small:
            cfg.update(res=512, D=256, trunc=0.03, target=512, S=64, prims=12)
        sc, ori, dirs, color_grid, color_vs = workload(cfg)
        fz = cpu_fused_grid(sc, cfg)
        run = lambda: cpu_baseline(sc, ori, dirs, cfg, color_grid, color_vs, ray_sample=4096, fusion_slab=8,  # noqa
                                   fz=fz)
        R = ori.shape[1]
        workload = "full-resolution plain forward: 4x1024^2 views, 512^3 TSDF, 8^3 bricks, 1024^2 target, S=96"
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = run()
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.median(vals)) if vals else cb["value"]
    out = dict(metric=METRIC, value=v, unit=UNIT, impl="reference", n_gpus=args.gpus, steps=args.steps,
               warmup=args.warmup, ms_per_step=1000.0 * R / v, higher_is_better=True,
               scaling="weak", vs_baseline=None, dtype="f32", data="synthetic",
               config=dict(workload=workload, l2="inputs > L2"),
               cpu_baseline=dict(value=v, unit=UNIT, cores=cb["cores"], kind="port", sample=cb["sample"]),
               e2e=dict(value=v, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# batched training step (default workload)
# ---------------------------------------------------------------------------
def batch_workload(bcfg, rank=0):
    from sailor_gb300 import synthetic as syn
    return syn.make_batch_workload(seed=bcfg["seed"] + 1000 * rank, n_frames=bcfg["frames"], views=bcfg["views"],
                                   view_res=bcfg["view_res"], n_prims=bcfg["prims"], D=bcfg["D"],
                                   trunc=bcfg["trunc"], n_targets=bcfg["targets"], target_res=bcfg["target_res"],
                                   target_S=bcfg["target_S"], workers=min(8, os.cpu_count() or 1))


def batch_fields(bcfg, R, feat, rank=0):
    """Seeded feature grids ~ N(0, 0.1) written into feat [B, D, D, D, C] on
    the device; colour head [3, C] ~ N(0, 0.25); target colours U(0, 1)."""
    import torch
    gen = torch.Generator(device=feat.device)
    gen.manual_seed(bcfg["seed"] + 1000 * rank + 5)
    feat.normal_(0.0, 0.1, generator=gen)
    rng = np.random.default_rng(bcfg["seed"] + 1000 * rank + 5)
    head = rng.standard_normal((3, bcfg["C"]), dtype=np.float32) * np.float32(0.5)
    target = rng.random((R, 3), dtype=np.float32)
    return head, target


def padded_views(fr):
    """A frame's views zero-padded to its largest resolution (depth 0 =
    no measurement, so the padding changes nothing)."""
    hm = max(d.shape[0] for d in fr["depth"])
    nv = len(fr["depth"])
    dep = np.zeros((1, nv, hm, hm), np.float32)
    col = np.zeros((1, nv, hm, hm), np.float32)
    for v in range(nv):
        h, w_ = fr["depth"][v].shape
        dep[0, v, :h, :w_] = fr["depth"][v]
        col[0, v, :h, :w_] = fr["color"][v]
    return np.stack(fr["K"])[None], np.stack(fr["RT"])[None], dep, col


def near_node_bricks(bp):
    """Top bricks sg_zero_near_nodes clears for the pipeline's last gradient
    pass: the nodes' bricks and their 26-neighbourhoods."""
    import torch
    B, Dt = bp.B, bp.Dt
    m = (bp.grad_bricks >= 0).view(B, 1, Dt, Dt, Dt).float()
    return int(torch.nn.functional.max_pool3d(m, 3, stride=1, padding=1).sum().item())


def batch_algorithmic_bytes(bcfg, w, n_hits, R, n_samples, n_clear_bricks=None, n_touched=0):
    """Per-launch algorithmic HBM bytes of each batched stage.  n_touched:
    voxels whose feature cells the samples tap (read once: 4 C bytes of
    features and 4 of TSDF; the gradient written once: 4 C bytes)."""
    B, D, C = bcfg["frames"], bcfg["D"], bcfg["C"]
    V, Vt = B * D ** 3, B * (D // bcfg["rate"]) ** 3
    n_pix = sum(d.size for fr in w["frames"] for d in fr["depth"])
    return dict(
        fusion=16 * V + 8 * n_pix,
        tree=4 * V + 4 * Vt,
        # camera table, ray generation (24 B/ray written), intersection (rays
        # read back, hit rows + count + valid length written)
        intersect=24 * R + 24 * R + 12 * n_hits + 8 * R,
        forward=24 * R + 12 * n_hits + 8 * R + 24 * R,  # rays, hit rows, count + valid length in; 24 B/ray out
        # fused training pass: as forward, with the target colour in and the
        # per-ray loss out, plus the touched cells of the TSDF and feature
        # grids read once and the feature-gradient cells written once
        train=24 * R + 12 * n_hits + 8 * R + 12 * R + 24 * R + 4 * R + n_touched * (4 * C + 4 + 4 * C),
        # clear of the feature-gradient grid near the previous pass's nodes
        # (side stream, beside fusion): 4 C bytes per voxel of those bricks
        zero_grad=4 * C * bcfg["rate"] ** 3 * (n_clear_bricks if n_clear_bricks is not None else Vt),
    )


def cpu_batch_setup(w, bcfg):
    """Untimed set-up of the CPU baseline of the batched step: every frame
    fused by the oracle (the tree and render stages need complete grids), one
    seeded feature grid [1, D, D, D, C] ~ N(0, 0.1) shared by the frames (its
    values do not change the work) and a colour head ~ N(0, 0.5)."""
    from oracle import oracle as orc
    D, C = bcfg["D"], bcfg["C"]
    fz = []
    for b, fr in enumerate(w["frames"]):
        K, RT, dep, col = padded_views(fr)
        fz.append(orc.integrate(K, RT, col, dep, D, w["vol_bbox"][b:b + 1], w["voxel_size"][b:b + 1].reshape(1, 1),
                                trunc_weight=w["trunc_weight"]))
    rng = np.random.default_rng(bcfg["seed"] + 5)
    feat = rng.standard_normal((1, D, D, D, C), dtype=np.float32) * np.float32(0.1)
    head = rng.standard_normal((3, C), dtype=np.float32) * np.float32(0.5)
    return dict(fz=fz, feat=feat, head=head)


def cpu_baseline_batch(w, bcfg, setup, n_rays=4096, fusion_slab=8):
    """The oracle (a C port of the reference kernels, OpenMP on all host
    cores) on a bounded sample of the batched training step, scaled to the
    whole step: fusion of an x-slab of fusion_slab voxels of every frame
    (x D / fusion_slab), coarse occupancy + tree of every frame, and for
    every target a share of n_rays rays proportional to its rays x samples
    (evenly spaced over its rays, at least 8): traversal, coarse sampling,
    sort, TSDF and feature taps, colour head, compositing forward and
    backward, grid scatter -- each target's time scaled by its rays over the
    sampled ones.  Returns the rate, the stage times and the wall time of the
    sample itself."""
    from oracle import oracle as orc
    D, rate = bcfg["D"], bcfg["rate"]
    t_wall = time.perf_counter()
    t0 = time.perf_counter()
    for b, fr in enumerate(w["frames"]):
        K, RT, dep, col = padded_views(fr)
        orc.integrate_slab(K, RT, col, dep, D, w["vol_bbox"][b:b + 1], w["voxel_size"][b:b + 1].reshape(1, 1), 0,
                           fusion_slab, trunc_weight=w["trunc_weight"])
    t_fuse = (time.perf_counter() - t0) * (D / fusion_slab)
    t0 = time.perf_counter()
    trees = []
    for fz in setup["fz"]:
        top, _ = orc.merge(fz["occ"], rate)
        trees.append(orc.build_tree(top, fz["occ"]))
    t_tree = time.perf_counter() - t0
    tg_all = w["targets"]
    R = sum(t["ori"].shape[0] for t in tg_all)
    work = np.array([t["ori"].shape[0] * t["S"] for t in tg_all], np.float64)
    feat, head = setup["feat"], setup["head"]
    t_render = 0.0
    n_sampled = 0
    for t, tg in enumerate(tg_all):
        b, S, n = tg["frame"], tg["S"], tg["ori"].shape[0]
        ns = int(min(n, max(8, round(n_rays * work[t] / work.sum()))))
        sel = np.linspace(0, n - 1, ns).astype(np.int64)
        o, d = tg["ori"][sel][None], tg["dir"][sel][None]
        bb, vs = w["vol_bbox"][b:b + 1], w["voxel_size"][b:b + 1].reshape(1, 1)
        t0 = time.perf_counter()
        hits = orc.voxel_traversal(trees[b], o, d, vs, bb, W=bcfg["W_hits"])
        _, sz, _ = orc.sample_coarse(trees[b], hits, np.full((1, ns, S), 0.5, np.float32), vs, S)
        srt, _ = orc.sort(sz)
        pts = (o[0][:, None, :] + d[0][:, None, :] * np.maximum(srt[0], 0)[..., None]).reshape(-1, 3)
        tv = orc.grid_gather(pts, setup["fz"][b]["tsdf"][..., None], bb[:, :, 0], vs[:, 0])[:, 0]
        sdf = tv * float(vs[0, 0]) * w["trunc_weight"]
        sigma = (1.0 / (1.0 + np.exp(sdf / bcfg["sdf_s"])) / bcfg["sdf_s"]).astype(np.float32)
        fe = orc.grid_gather(pts, feat, bb[:, :, 0], vs[:, 0])
        rgb = (fe @ head.T.astype(np.float64)).astype(np.float32)
        sig4, rgb4 = sigma.reshape(1, ns, S, 1), rgb.reshape(1, ns, S, 3)
        fo = orc.composite_fwd(srt, None, sig4, rgb4, 1e-4, False)[:4]
        g = [np.ones(x.shape, np.float32) for x in fo]
        ident = np.broadcast_to(np.arange(S, dtype=np.int32), srt.shape)
        gf, _ = orc.composite_bwd_ref(*g, *fo, srt, ident, sig4, rgb4, 1e-4, False)
        gfe = (gf.reshape(-1, 3).astype(np.float64) @ head.astype(np.float64)).astype(np.float32)
        orc.grid_scatter(pts, gfe, 1, D, bb[:, :, 0], vs[:, 0])
        t_render += (time.perf_counter() - t0) * n / ns
        n_sampled += ns
    t_step = t_fuse + t_tree + t_render
    return dict(value=R / t_step, unit=UNIT, cores=orc.num_threads(), kind="port",
                sample=(f"oracle (C port, OpenMP) on host cores: fusion of x-slab {fusion_slab}/{D} of every frame "
                        f"(x{D // fusion_slab}), coarse occupancy + tree of every frame, traversal / sampling / "
                        f"sort / field taps / compositing forward and backward / grid scatter of {n_sampled} rays "
                        f"from all {len(tg_all)} targets (shares by rays x samples) scaled to {R} rays"),
                stage_s=dict(fusion=t_fuse, tree=t_tree, render=t_render),
                sample_wall_s=time.perf_counter() - t_wall)


def _cpu_baseline_job(w, bcfg, reps):
    """Child-process body of cpu_baseline_isolated."""
    setup = cpu_batch_setup(w, bcfg)
    return [cpu_baseline_batch(w, bcfg, setup) for _ in range(reps)]


def cpu_baseline_isolated(w, bcfg, reps=5):
    """reps timed samples of cpu_baseline_batch in a fresh spawned process
    (no GPU context or framework threads sharing its cores), after the
    untimed set-up there.  Returns the list of per-sample results."""
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as ex:
        return ex.submit(_cpu_baseline_job, w, bcfg, reps).result()


def summarize_cpu_baseline(runs):
    """Median of the samples' rates (the bench line's cpu_baseline)."""
    v = float(np.median([r["value"] for r in runs]))
    r0 = runs[0]
    return dict(value=v, unit=r0["unit"], cores=r0["cores"], kind=r0["kind"],
                sample=r0["sample"] + f"; median of {len(runs)} samples in a separate process",
                samples=[r["value"] for r in runs])


# ---------------------------------------------------------------------------
# parity of the batched step against the oracle (after timing; the oracle is
# the checker here, never part of a timed region)
# ---------------------------------------------------------------------------
def _oracle_frames(w, bcfg):
    """Oracle fusion + coarse occupancy + tree of every frame (C port)."""
    from oracle import oracle as orc
    out = []
    for b, fr in enumerate(w["frames"]):
        K, RT, dep, col = padded_views(fr)
        fz = orc.integrate(K, RT, col, dep, bcfg["D"], w["vol_bbox"][b:b + 1], w["voxel_size"][b:b + 1].reshape(1, 1),
                           trunc_weight=w["trunc_weight"])
        top, _ = orc.merge(fz["occ"], bcfg["rate"])
        out.append(dict(fusion=fz, tree=orc.build_tree(top, fz["occ"])))
    return out


def _pipeline_rows(bp, sel):
    """The pipeline's hit rows of rays sel as the oracle's padded rows
    (entries past each ray's count -1), with its valid lengths."""
    import torch
    st = torch.as_tensor(sel, device=bp.dev)
    cnt = bp.hit_count[st].cpu().numpy()
    idx, t0, t1 = (a[st].cpu().numpy().copy() for a in (bp.hit_idx, bp.hit_t0, bp.hit_t1))
    pad = np.arange(bp.W)[None, :] >= cnt[:, None]
    idx[pad], t0[pad], t1[pad] = -1, -1.0, -1.0
    return dict(idx=idx[None], t0=t0[None], t1=t1[None], valid_len=bp.valid_len[st].cpu().numpy()[None, :, None],
                max_hits=int(cnt.max(initial=0)), flags=np.zeros((1, len(sel)), np.int32))


def _pipeline_keys(bp):
    """Node ids of the pipeline's tree -> canonical (level, frame, x, y, z)."""
    return dict(Dt=bp.Dt, Db=bp.D, base_top=bp.B * bp.D ** 3, base_bot=0, top_key=bp.top_key.cpu().numpy(),
                bot_key=bp.bot_key.cpu().numpy())


def _check_rows(frame, w, b, o, d, rows, keys):
    """The oracle's traversal on its own tree of frame b against the
    pipeline's rows: (rays the oracle leaves unflagged, rows equal as
    canonical node sequences, max |t0/t1 difference| on equal rows)."""
    from oracle import oracle as orc
    W = rows["idx"].shape[-1]
    vs, bb = w["voxel_size"][b:b + 1].reshape(1, 1), w["vol_bbox"][b:b + 1]
    h = orc.voxel_traversal(frame["tree"], o[None], d[None], vs, bb, W=W)
    ko = orc.node_keys(frame["tree"], h["idx"][0])
    ko[..., 1] = np.where(h["idx"][0] >= 0, b, -1)
    kg = orc.node_keys(keys, rows["idx"][0])
    ok = (h["flags"][0] == 0) & (h["max_hits"] <= W)
    eq = np.all(ko == kg, axis=(1, 2))
    m = (h["idx"][0] >= 0) & eq[:, None]
    terr = max(float(np.abs(h["t0"][0][m] - rows["t0"][0][m]).max(initial=0.0)),
               float(np.abs(h["t1"][0][m] - rows["t1"][0][m]).max(initial=0.0)))
    return ok, eq, terr


def _samples_on_rows(bp, w, b, rows, S, rands):
    """The oracle's coarse sampling and sort of the pipeline's hit rows
    (sample depths [n, S], torch.sort order)."""
    from oracle import oracle as orc
    tree = {"Dt": bp.Dt, "Db": bp.D, "base_top": bp.B * bp.D ** 3}
    _, sz, _ = orc.sample_coarse(tree, rows, rands[None], w["voxel_size"][b:b + 1].reshape(1, 1), S)
    return orc.sort(sz)[0][0]


def _jitter(seed, r, S):
    """The render's jitter of rays r [n], samples 0..S-1: hashed with seed,
    the constant 0.5 when seed is 0."""
    from oracle import oracle as orc
    if not seed:
        return np.full((len(r), S), 0.5, np.float32)
    return orc.hash_uniform(seed, np.asarray(r)[:, None], np.arange(S)[None, :])


def _select_rays(hit_count, a, b, n_hit, n_all):
    """Evenly spaced rays of [a, b): n_hit among those with hits, n_all among all."""
    hc = hit_count[a:b]
    hit = np.nonzero(hc > 0)[0]
    sel = []
    if len(hit):
        sel.append(hit[np.linspace(0, len(hit) - 1, min(n_hit, len(hit))).astype(np.int64)])
    sel.append(np.linspace(0, b - a - 1, min(n_all, b - a)).astype(np.int64))
    return a + np.unique(np.concatenate(sel))


def _near_rays(bp, zs, b, vxyz, frame_of_ray):
    """Rays of frame b whose samples come within a voxel of voxel vxyz (a
    superset of the rays whose taps weight it)."""
    import torch
    near = torch.zeros(bp.R, dtype=torch.bool, device=bp.dev)
    bmin_t = bp.vol_bbox[b, :, 0]
    inv_vs = 1.0 / bp.voxel_size[b]
    v_t = torch.tensor(vxyz, dtype=torch.float32, device=bp.dev)
    for a in range(0, bp.R, 1 << 19):
        e = min(a + (1 << 19), bp.R)
        zz = zs[a:e]
        pts = bp.ori[a:e, None, :] + bp.dirs[a:e, None, :] * zz.clamp_min(0)[..., None]
        u = (pts - bmin_t) * inv_vs
        near[a:e] = (((u - v_t).abs() <= 1.5).all(-1) & (zz >= 0)).any(-1) & (frame_of_ray[a:e] == b)
    return torch.nonzero(near).view(-1).cpu().numpy()


def _perturbed_features(pts, feat, bmin, vs, vxyz, ch, dv):
    """float64 features at pts with feature (vxyz, ch) moved by dv (each
    sample's features change by dv times the voxel's trilinear weight)."""
    from oracle import oracle as orc
    fe = orc.grid_gather(pts, feat, bmin, vs)
    if dv != 0.0:
        i0, wt = orc.trilinear_cells(pts, bmin, vs)
        dlt = np.asarray(vxyz)[None, :] - i0
        inside = ((dlt >= 0) & (dlt <= 1)).all(-1)
        cr = np.clip((dlt[:, 0] << 2) | (dlt[:, 1] << 1) | dlt[:, 2], 0, 7)
        fe[:, ch] += np.where(inside, wt[np.arange(len(cr)), cr], 0.0) * dv
    return fe


def parity_batch(bp, w, bcfg, seed, frames=None, n_hit=192, n_all=64, n_fd_entries=48, h=1e-4):
    """Parity of the batched training step (its last outputs in bp) against
    the oracle, stage by stage:
    - fusion of every frame bit for bit (TSDF, weight, colour grids);
    - per target, n_hit rays with hits and n_all rays overall:
      * traversal: the oracle's rows on its own tree equal the pipeline's
        (canonical node sequences) on every ray the oracle does not flag as
        a near tie, t-intervals within 1e-5 (the GPU's approximate
        reciprocal moves them by ulps);
      * sampling: the oracle's coarse sampling (the step's jitter) and sort
        of the pipeline's rows equal the pipeline's samples bit for bit, on
        every ray;
      * compositing: the float64 render of those samples (float32 sample
        points, FP64 taps, density, colour head, compositing) against the
        training pass's colour, depth, weight sum and alpha -- max abs error
        per output on every ray but early-termination ties;
    - the feature-grid gradient of the step on n_fd_entries entries (the
      largest and random touched ones) against float64 central differences
      (step h) of the oracle's loss of every ray whose samples reach the
      entry (the feature at each affected sample moved by +-h times its
      trilinear weight, then re-composited).
    seed: the step's jitter seed (0: constant 0.5).  Returns the dict
    printed as the bench line's "parity"."""
    import torch
    from oracle import oracle as orc
    t_start = time.perf_counter()
    if frames is None:
        frames = _oracle_frames(w, bcfg)
    B, D, C = bcfg["frames"], bcfg["D"], bcfg["C"]
    fusion_exact = all(np.array_equal(bp.tsdf[b].cpu().numpy().view(np.uint32), f["fusion"]["tsdf"][0].view(np.uint32))
                       and np.array_equal(bp.weight[b].cpu().numpy(), f["fusion"]["weight"][0])
                       and np.array_equal(bp.colorv[b].cpu().numpy(), f["fusion"]["color"][0])
                       for b, f in enumerate(frames))
    trunc_m = float(w["voxel_size"][0]) * w["trunc_weight"]
    sdf_s = bcfg["sdf_s"]
    head = bp.head.cpu().numpy()
    hc = bp.hit_count.cpu().numpy()
    ori, dirs = bp.ori.cpu().numpy(), bp.dirs.cpu().numpy()
    outs = [t.cpu().numpy().reshape(bp.R, -1) for t in (bp.out_rgb, bp.out_depth, bp.out_ws, bp.out_alpha)]
    # the samples of every ray (the training pass samples as the forward)
    zs = torch.empty((bp.R, bp.S), device=bp.dev)
    nodes = torch.empty((bp.R, bp.S), dtype=torch.int32, device=bp.dev)
    bp.forward(zs, nodes)
    del nodes
    keys = _pipeline_keys(bp)
    feat = [bp.feat[b:b + 1].cpu().numpy() for b in range(B)]
    errs = dict(rgb=0.0, depth=0.0, ws=0.0, alpha=0.0)
    n_rays = rows_flagged = rows_mismatch = z_mismatch = comp_flagged = 0
    t_err = 0.0
    for t, (b, n, S) in enumerate(bp.targets):
        a, e = bp.ray_slices[t]
        sel = _select_rays(hc, a, e, n_hit, n_all)
        n_rays += len(sel)
        rows = _pipeline_rows(bp, sel)
        ok_rows, eq_rows, terr = _check_rows(frames[b], w, b, ori[sel], dirs[sel], rows, keys)
        rows_flagged += int((~ok_rows).sum())
        rows_mismatch += int((ok_rows & ~eq_rows).sum())
        t_err = max(t_err, terr)
        srt = _samples_on_rows(bp, w, b, rows, S, _jitter(seed, sel, S))
        zg = zs[torch.as_tensor(sel, device=bp.dev), :S].cpu().numpy()
        z_mismatch += int((~np.all(zg.view(np.uint32) == srt.view(np.uint32), axis=1)).sum())
        r = orc.render_fp64(ori[sel], dirs[sel], srt, frames[b]["fusion"]["tsdf"], w["vol_bbox"][b:b + 1, :, 0],
                            w["voxel_size"][b:b + 1], trunc_m, sdf_s, feat[b], head, 1e-4)
        ok = r["flags"] == 0
        comp_flagged += int((~ok).sum())
        for k, ref, got in (("rgb", r["rgb"], outs[0][sel]), ("depth", r["depth"], outs[1][sel, 0]),
                            ("ws", r["ws"], outs[2][sel, 0]), ("alpha", r["alpha"], outs[3][sel, 0])):
            if ok.any():
                errs[k] = max(errs[k], float(np.abs(got - ref)[ok].max()))
    # the feature-grid gradient against float64 central differences of the
    # loss of every ray that reaches the checked entries
    loss_scale = 2.0 / (3.0 * bp.R)
    tgt = bp.target_rgb.cpu().numpy().astype(np.float64)
    ray_frame = np.empty(bp.R, np.int64)
    ray_S = np.empty(bp.R, np.int64)
    for t, (b, n, S) in enumerate(bp.targets):
        a, e = bp.ray_slices[t]
        ray_frame[a:e] = b
        ray_S[a:e] = S

    def loss_of_rays(rays, b, vxyz, ch, dv):
        """float64 loss of rays (all of frame b) with feature (vxyz, ch)
        moved by dv; samples: the oracle's sampling of the pipeline's rows."""
        tot = 0.0
        for S in np.unique(ray_S[rays]):
            rr = rays[ray_S[rays] == S]
            srt = _samples_on_rows(bp, w, b, _pipeline_rows(bp, rr), int(S), _jitter(seed, rr, int(S)))
            bmin, vs = w["vol_bbox"][b:b + 1, :, 0], w["voxel_size"][b:b + 1]
            base = orc.render_fp64(ori[rr], dirs[rr], srt, frames[b]["fusion"]["tsdf"], bmin, vs, trunc_m, sdf_s,
                                   feat[b], head, 1e-4)
            pts = orc.sample_points(ori[rr], dirs[rr], srt).reshape(-1, 3)
            fe = _perturbed_features(pts, feat[b], bmin, vs, vxyz, ch, dv)
            rgb_s = np.where((srt >= 0)[..., None], (fe @ head.T.astype(np.float64)).reshape(len(rr), int(S), 3), 0)
            c = orc.composite_sorted_fp64(srt, base["sigma"], rgb_s, 1e-4)[0]
            tot += 0.5 * loss_scale * ((c - tgt[rr]) ** 2).sum()
            loss_of_rays.flagged += int((base["flags"] != 0).sum())
        return tot
    loss_of_rays.flagged = 0

    flat = bp.grad_feat.view(-1)
    top = torch.topk(flat.abs(), n_fd_entries // 2).indices
    nz = torch.nonzero(flat).view(-1)
    gen = torch.Generator(device="cpu").manual_seed(int(seed) + 1)
    rnd = nz[torch.randint(0, nz.numel(), (n_fd_entries - top.numel(),), generator=gen).to(nz.device)]
    entries = torch.unique(torch.cat([top, rnd])).cpu().numpy()
    g_gpu = flat[torch.as_tensor(entries, device=bp.dev)].double().cpu().numpy()
    rf = torch.as_tensor(ray_frame, device=bp.dev)
    g_fd = np.zeros(len(entries))
    n_rays_fd = 0
    for k, ent in enumerate(entries):
        b, rem = divmod(int(ent), D ** 3 * C)
        vox, ch = divmod(rem, C)
        vxyz = (vox // (D * D), (vox // D) % D, vox % D)
        rays = _near_rays(bp, zs, b, vxyz, rf)
        n_rays_fd += len(rays)
        g_fd[k] = (loss_of_rays(rays, b, vxyz, ch, h) - loss_of_rays(rays, b, vxyz, ch, -h)) / (2.0 * h)
    del zs
    gmax = float(np.abs(g_fd).max())
    gerr = float(np.abs(g_gpu - g_fd).max())
    return dict(fusion_frames_bit_exact=bool(fusion_exact), rays=n_rays,
                traversal=dict(rays_flagged=rows_flagged, unflagged_row_mismatches=rows_mismatch,
                               t_max_abs_err=t_err),
                sample_mismatches=z_mismatch,
                composite_max_abs_err=errs, composite_rays_flagged=comp_flagged, composite_atol=1e-5,
                composite_within_atol=all(v <= 1e-5 for v in errs.values()),
                grad_fd=dict(entries=len(entries), rays=n_rays_fd, h=h, max_abs_err=gerr, max_abs_fd=gmax,
                             rel_err=gerr / gmax if gmax > 0 else None,
                             ray_evaluations_flagged=loss_of_rays.flagged),
                seconds=time.perf_counter() - t_start)


def frame_tree(bp, b):
    """SgTree view of frame b of a BatchPipeline's tree (B = 1): the frame's
    brick map, masks, voxel size and box; node ids stay the pipeline's."""
    import ctypes as C

    from sailor_gb300 import _native as N
    t, Dt, mw = bp.tree, bp.Dt, N.mask_words(bp.rate)
    return N.SgTree(1, t.Dt, t.Db, t.rate, t.base_top, t.base_bot, t.cap_top, t.cap_bot,
                    bp.brick_node.data_ptr() + 4 * b * Dt ** 3, bp.brick_mask.data_ptr() + 4 * b * Dt ** 3 * mw,
                    t.top_key, t.top_child_base, t.bot_key, t.bot_parent, t.counts,
                    bp.voxel_size.data_ptr() + 4 * b, C.c_void_p(bp.vol_bbox.data_ptr() + 24 * b))


def sample_sort_ms(bp, steps):
    """Milliseconds per pass of sg_sample_sorted (coarse sampling + per-ray
    sort, S of each target, jitter 0.5) over every target's hit rows."""
    import ctypes as C

    import torch

    from sailor_gb300 import _native as N
    z = torch.empty((bp.R, bp.S), device=bp.dev)
    idx = torch.empty((bp.R, bp.S), dtype=torch.int32, device=bp.dev)
    trees = [frame_tree(bp, b) for b in range(bp.B)]
    W = bp.W
    vp = lambda t, a, size: C.c_void_p(t.data_ptr() + size * a)  # noqa: E731

    def one():
        for ti, (f, n, S) in enumerate(bp.targets):
            a, e = bp.ray_slices[ti]
            N.check(N.lib.sg_sample_sorted(C.byref(trees[f]), vp(bp.hit_idx, a, 4 * W), vp(bp.hit_t0, a, 4 * W),
                                           vp(bp.hit_t1, a, 4 * W), vp(bp.hit_count, a, 4), e - a, W, None, 0.5,
                                           vp(bp.valid_len, a, 4), S, 2, 0, vp(z, a, 4 * bp.S), vp(idx, a, 4 * bp.S),
                                           N.stream()), "sample_sorted")

    for _ in range(3):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        one()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def plain_per_frame_forward(VE, fields, w, bcfg, dev, feat, head_t, vbb, vvs, W_hits=256):
    """The reference's per-frame call order through the drop-in API, forward
    only: per frame integrate -> build_multi_res_volumes -> octree, then per
    target of the frame rays_calculating -> traversal (padded rows) -> coarse
    sampling -> sort -> TSDF density and feature gathers -> colour head ->
    compositing."""
    import torch
    D, rate = bcfg["D"], bcfg["rate"]
    Dt = D // rate
    trunc_m = float(w["voxel_size"][0]) * w["trunc_weight"]
    outs = []
    for b, fr in enumerate(w["frames"]):
        K, RT, dep, col = fr["_dev"]
        occ0 = torch.full((1, D, D, D), -1, dtype=torch.int32, device=dev)
        occ1 = torch.full((1, Dt, Dt, Dt), -1, dtype=torch.int32, device=dev)
        cnt0 = torch.zeros((1, 1), dtype=torch.int32, device=dev)
        cnt1 = torch.zeros((1, 1), dtype=torch.int32, device=dev)
        bb, vs = vbb[b:b + 1], vvs[b:b + 1]
        tsdf, _, _ = VE.integrate_in_box(occ0, cnt0, K, RT, col, dep, bb, vs, 1.0, w["trunc_weight"], 13.5, 13.5,
                                         dev.index or 0)
        VE.build_multi_res_volumes([occ0, occ1], [cnt0, cnt1], 2, rate, dev.index or 0)
        tot = [int(cnt0.sum()), int(cnt1.sum())]
        octree = VE.MultiLayerOctree(2, 1, rate, dev.index or 0)
        octree.init_octree([occ0, occ1], tot, [cnt0, cnt1], [0, tot[0]], vs, bb)
        octree.build_octree()
        for t in w["targets"]:
            if t["frame"] != b:
                continue
            Kt, Rt, Tt = t["_dev"]
            rays = VE.rays_calculating(Kt, Rt, Tt, t["res"], dev.index or 0).view(1, -1, 6)
            o, d = rays[..., :3].contiguous(), rays[..., 3:].contiguous()
            S = t["S"]
            n = o.shape[1]
            idx, t0, t1, vl = octree.voxel_traversal(o, d, W_hits, 0, -1, False, -1)
            rands = torch.full((1, n, S), 0.5, device=dev)
            _, sz = octree.ray_voxels_points_sampling_coarse(idx, t0, t1, rands, vl, 0, S)
            _, sidx = octree.sort_samplings(sz)
            sig = fields.tsdf_density(tsdf, o, d, sz, bb, vs, trunc_m, bcfg["sdf_s"])
            rgb = fields.grid_gather(feat[b:b + 1], o, d, sz, bb, vs) @ head_t
            outs.append(VE.volume_rendering_training_forward(sz, sidx, sig[..., None].contiguous(),
                                                             rgb.contiguous(), dev.index or 0, 1e-4, False))
    return outs


def run_batch(args):
    import torch
    import torch.distributed as dist

    from sailor_gb300 import fields
    from sailor_gb300.batch import BatchPipeline
    from sailor_gb300.dist import VoxelEncoding as VE

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    bcfg = dict(BATCH_SMALL if args.small else BATCH)
    w = batch_workload(bcfg, rank)
    view_hw = [[d.shape for d in fr["depth"]] for fr in w["frames"]]
    targets = [(t["frame"], t["ori"].shape[0], t["S"]) for t in w["targets"]]
    bp = BatchPipeline(view_hw, targets, D=bcfg["D"], rate=bcfg["rate"], C=bcfg["C"], W_hits=bcfg["W_hits"],
                       target_widths=[t["res"] for t in w["targets"]], device=dev)
    bp.load_views(w["frames"], w["vol_bbox"], w["voxel_size"], w["trunc_weight"])
    bp.load_cameras([t["K"] for t in w["targets"]], [t["R"] for t in w["targets"]], [t["T"] for t in w["targets"]])
    head, target = batch_fields(bcfg, bp.R, bp.feat, rank)
    bp.set_fields(head=torch.as_tensor(head).to(dev), target_rgb=torch.as_tensor(target).to(dev))
    trunc_m = float(w["voxel_size"][0]) * w["trunc_weight"]
    bp.render_args(trunc_m, sdf_s=bcfg["sdf_s"], t_thres=1e-4, rand_seed=bcfg["seed"] + 1)
    R = bp.R

    tuned = None
    bp.train_step()
    if not args.no_autotune:
        from sailor_gb300 import autotune
        autotune.set_knob("fuse_tiled", 1)
        tuned = autotune.tune({"isect_warp": bp.intersect, "isect_block": bp.intersect,
                               "render_warps": bp.train_step}, verbose=True)
        tuned.update(fuse_tiled=1)
    for _ in range(max(args.warmup - 1, 0)):
        bp.train_step()
    torch.cuda.synchronize()
    st = bp.status.tolist()
    if st[0] & 1:
        raise RuntimeError(f"hit rows overflowed: a ray has {st[1]} hits, rows hold {bp.W}")
    n_hits = int(bp.hit_count.sum().item())
    graph = bp.capture(warmup=1)
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    import tempfile
    clk = ClockSampler(os.path.join(tempfile.gettempdir(), f"sg_clocks_rank{rank}.csv"))
    with clk:
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            graph.replay()
        e1.record()
        barrier()
    ms_max, value = whole_job(e0.elapsed_time(e1) / args.steps, R, world, dev)
    ref_rgb = bp.out_rgb.cpu()  # the timed steps' image, for the e2e check below
    red_sizes = bp.reduction_sizes()  # of the last timed step

    # per-stage times (eager pass with events on the launching stream)
    stage_sum = {}
    for _ in range(args.steps):
        bp.events = []
        bp.train_step()
        for k, v in bp.stage_times().items():
            stage_sum[k] = stage_sum.get(k, 0.0) + v
    bp.events = None
    stages = {k: v / args.steps for k, v in stage_sum.items()}
    peak_mem = torch.cuda.max_memory_allocated(dev)

    # standalone sampling + per-ray sort (sg_sample_sorted) of every target's
    # hit rows, outside the graph: the sampler's own roofline
    samp_ms = sample_sort_ms(bp, args.steps)

    # plain per-frame forward-only launch sequence on the same inputs
    vbb = torch.as_tensor(w["vol_bbox"]).to(dev)
    vvs = torch.as_tensor(w["voxel_size"]).reshape(-1, 1).to(dev)
    for fr in w["frames"]:
        fr["_dev"] = [torch.as_tensor(a).to(dev) for a in padded_views(fr)]
    for t in w["targets"]:
        t["_dev"] = tuple(torch.as_tensor(t[k]).reshape(1, 1, *np.shape(t[k])).to(dev) for k in ("K", "R", "T"))
    feat_t, head_t = bp.feat, bp.head.T.contiguous()
    plain_forward = lambda: plain_per_frame_forward(VE, fields, w, bcfg, dev, feat_t, head_t, vbb, vvs)  # noqa
    for _ in range(2):
        plain_forward()
    barrier()
    p0 = time.perf_counter()
    n_plain = max(1, min(args.steps, 5))
    for _ in range(n_plain):
        plain_forward()
    barrier()
    plain_ms = (time.perf_counter() - p0) * 1000.0 / n_plain
    plain_value = R / (plain_ms / 1000.0)
    for fr in w["frames"]:
        fr.pop("_dev")
    for t in w["targets"]:
        t.pop("_dev")

    # e2e: the same step through the public API from pinned host buffers
    host = dict(depth=torch.as_tensor(np.concatenate([d.reshape(-1) for fr in w["frames"] for d in fr["depth"]])),
                color=torch.as_tensor(np.concatenate([c.reshape(-1) for fr in w["frames"] for c in fr["color"]])),
                K=torch.as_tensor(np.stack([k for fr in w["frames"] for k in fr["K"]])),
                RT=torch.as_tensor(np.stack([k for fr in w["frames"] for k in fr["RT"]])),
                # target cameras in the pipeline's segment order (what
                # load_cameras arranges; here once, outside the timed region)
                tK=torch.as_tensor(np.stack([w["targets"][t]["K"] for t in bp.order])),
                tR=torch.as_tensor(np.stack([w["targets"][t]["R"] for t in bp.order])),
                tT=torch.as_tensor(np.stack([w["targets"][t]["T"] for t in bp.order])),
                target_rgb=torch.as_tensor(target))
    host = {k: v.contiguous().pin_memory() for k, v in host.items()}
    out_host = torch.empty((R, 3), dtype=torch.float32).pin_memory()
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    d2h = out_host.numel() * 4
    # BatchPipeline.train_steps_from_host: every step's inputs go up and its
    # image comes back, the copies of neighbouring steps beside the step
    feed = [(host, {"out_rgb": out_host})]
    bp.train_steps_from_host(feed * 2, graph)
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record()
    bp.train_steps_from_host(feed * args.steps, graph)
    f1.record()
    barrier()
    _, e2e_value = whole_job(f0.elapsed_time(f1) / args.steps, R, world, dev)
    if not torch.equal(out_host, ref_rgb):
        raise RuntimeError("the e2e steps rendered a different image than the timed steps")

    if rank == 0:
        pk, pk_kind = peaks()
        S_all = sum(n * s for _, n, s in targets)
        n_touched = int((bp.grad_feat != 0).any(-1).sum().item())  # voxels the step's samples tap
        ab = batch_algorithmic_bytes(bcfg, w, n_hits, R, S_all, near_node_bricks(bp), n_touched)
        rl = {k: ab[k] / (stages[k] / 1000.0) / 1e9 for k in ab if stages.get(k)}
        dom = max(rl, key=lambda k: stages[k])
        # the standalone sampler (outside the step): hit rows, count and valid
        # length in, sorted depth and node id out per sample slot
        ab["sample_sort"] = 12 * n_hits + 8 * R + 8 * S_all
        rl["sample_sort"] = ab["sample_sort"] / (samp_ms / 1000.0) / 1e9
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath) and not args.small:  # figures scaled to the full batch
            traffic = json.load(open(tpath)).get("batch_" + dom)
        render_ms = sum(stages.get(k, 0.0) for k in ("intersect", "grad_prep", "train"))
        out = dict(
            metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
            ms_per_step=ms_max, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
            data="synthetic (seeded capsule/ellipsoid scenes per frame)",
            config=dict(workload=("batched training step: %d frames x 4-8 views at {512,768,1024}^2, 256^3 TSDF "
                                  "+ 256^3x16 feature grid per frame, 8^3 bricks, %d targets 256^2-1024^2 "
                                  "(%d rays), S 32-128, forward + adjoint, CUDA graph" %
                                  (bcfg["frames"], bcfg["targets"], R)) if not args.small else "batch small",
                        frames_per_rank=bcfg["frames"], rays_per_step=R, l2="per-step working set > 10 GB >> L2",
                        parallelism=f"replicas x{world}", launch_shapes=tuned),
            stages_ms=stages, sample_sort_ms=samp_ms,
            render_rays_s=R / (render_ms / 1000.0),
            plain_per_frame_fwd=dict(value=plain_value, unit=UNIT, ms_per_step=plain_ms,
                                     ratio_batched_fwd_bwd=value / plain_value),
            tsdf_gvox_s=bcfg["frames"] * bcfg["D"] ** 3 / (stages["fusion"] / 1000.0) / 1e9,
            hits_per_ray=n_hits / R, peak_hbm_bytes=peak_mem, touched_voxels=n_touched, reduction=red_sizes,
            roofline=dict(bound="hbm", kernel=dom, achieved=rl[dom], peak=pk["hbm_gbs"], unit="GB/s",
                          frac=rl[dom] / pk["hbm_gbs"], traffic=traffic, peak_kind=pk_kind,
                          algorithmic_bytes=ab[dom]),
            rooflines={k: dict(achieved=v, frac=v / pk["hbm_gbs"], algorithmic_bytes=ab[k]) for k, v in rl.items()},
            e2e=dict(value=e2e_value, unit=UNIT, h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h),
            # per step: gradient clear 1, depth blocks 1, fusion 1, coarse
            # occupancy 1, tree 5, camera table 1, ray generation 1,
            # intersection 1, and one training pass per sample-capacity group
            gpu_launches=(12 + len(bp._group_launch)) * args.steps,
            clocks=clk.summary(),
        )
        if not args.no_cpu_baseline:
            # the same samples as the reference arm's, in a process of their own
            out["cpu_baseline"] = summarize_cpu_baseline(cpu_baseline_isolated(w, bcfg, reps=5))
        if not args.no_parity:
            out["parity"] = parity_batch(bp, w, bcfg, bcfg["seed"] + 1)
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# differentiation workload: 2^20 random rays through the plain small volume,
# compositing forward + adjoint and the trilinear gathers + adjoint
# ---------------------------------------------------------------------------
DIFF = dict(views=4, res=512, prims=12, D=256, rate=8, trunc=0.03, rays=1 << 20, S=96, C=16, W=256, sdf_s=0.005,
            seed=17)


def diff_rays(seed, n, radius=3.0):
    """Seeded rays: origins uniform on a sphere of `radius` metres about the
    cube's centre, each aimed at a uniform point of the 2 m cube."""
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, 3))
    o = radius * v / np.linalg.norm(v, axis=1, keepdims=True)
    d = rng.uniform(-1.0, 1.0, (n, 3)) - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def diff_setup(cfg, dev):
    """The differentiation workload in a one-frame BatchPipeline: the fused
    volume, 2^20 rays (one segment of S samples), a seeded 256^3 x 16 feature
    grid ~ N(0, 0.1), a colour head ~ N(0, 0.5), upstream gradients ~ N(0, 1)
    on colour, depth and alpha (0 on the weight sum)."""
    import torch

    from sailor_gb300 import synthetic as syn
    from sailor_gb300.batch import BatchPipeline
    sc = syn.make_scene(seed=cfg["seed"], n_views=cfg["views"], res=cfg["res"], n_prims=cfg["prims"], D=cfg["D"],
                        trunc=cfg["trunc"])
    ori, dirs = diff_rays(cfg["seed"], cfg["rays"])
    frame = dict(K=list(sc["K"][0]), RT=list(sc["RT"][0]), depth=list(sc["depths"][0]), color=list(sc["colors"][0]))
    n, S = len(ori), cfg["S"]
    bp = BatchPipeline([[d.shape for d in frame["depth"]]], [(0, n, S)], D=cfg["D"], rate=cfg["rate"], C=cfg["C"],
                       W_hits=cfg["W"], train_tsdf=True, device=dev)
    bp.load_views([frame], sc["vol_bbox"], sc["voxel_size"].reshape(-1), sc["trunc_weight"])
    bp.load_rays([(ori, dirs)])
    gen = torch.Generator(device=dev)
    gen.manual_seed(cfg["seed"])
    bp.feat.normal_(0.0, 0.1, generator=gen)
    bp.set_fields(head=torch.randn((3, cfg["C"]), generator=gen, device=dev) * 0.5)
    trunc_m = float(sc["voxel_size"][0, 0]) * sc["trunc_weight"]
    bp.render_args(trunc_m, sdf_s=cfg["sdf_s"], t_thres=1e-4, rand_seed=cfg["seed"])
    g = dict(g_rgb=torch.randn((n, 3), generator=gen, device=dev), g_depth=torch.randn(n, generator=gen, device=dev),
             g_ws=torch.zeros(n, device=dev), g_alpha=torch.randn(n, generator=gen, device=dev))
    gs = torch.empty((n, S), device=dev)
    gr = torch.empty((n, S, 3), device=dev)
    w = dict(frames=[frame], vol_bbox=sc["vol_bbox"], voxel_size=sc["voxel_size"].reshape(-1),
             trunc_weight=sc["trunc_weight"])
    return dict(bp=bp, sc=sc, w=w, grads=g, grad_sigma=gs, grad_rgb=gr, trunc_m=trunc_m)


def diff_step(d):
    """One step: intersection, forward render, backward (per-sample sigma and
    colour gradients, and the feature and TSDF grid gradients)."""
    bp = d["bp"]
    bp.intersect()
    bp.forward()
    g = d["grads"]
    bp.backward(g["g_rgb"], g["g_depth"], g["g_ws"], g["g_alpha"], grad_sigma=d["grad_sigma"],
                grad_rgb=d["grad_rgb"], tsdf_grad=True, zero=True)


def parity_diff(d, cfg, n_rays=512, h=1e-4, n_entries=24, autograd_rays=None):
    """Checks of the differentiation step (after timing):
    - fusion bit for bit; on n_rays rays with hits: traversal rows against
      the oracle's (unflagged rays), samples against the oracle's sampling
      of the pipeline's rows (bit for bit), the forward outputs against the
      float64 oracle render of those samples, and the per-sample sigma and
      colour gradients against float64 central differences (step h) of L =
      g_rgb . rgb + g_depth depth + g_ws ws + g_alpha alpha;
    - on every ray (or the first autograd_rays): the per-sample gradients
      against float64 autograd of a plain PyTorch compositing (the kernel's
      semantics: sorted samples, last delta 1e10, early termination) fed with
      the modular chain's float32 sigma and colour at the same samples;
    - on n_entries feature- and TSDF-grid entries: the grid gradients against
      float64 central differences of L over every ray reaching the entry."""
    import torch

    from oracle import oracle as orc
    from sailor_gb300.fields import grid_gather, tsdf_density
    t_start = time.perf_counter()
    bp, w = d["bp"], d["w"]
    D, C, S = cfg["D"], cfg["C"], cfg["S"]
    frames = _oracle_frames(w, dict(D=D, rate=cfg["rate"]))
    fr = frames[0]
    fusion_exact = bool(np.array_equal(bp.tsdf[0].cpu().numpy().view(np.uint32), fr["fusion"]["tsdf"][0].view(
        np.uint32)))
    trunc_m, sdf_s, seed = d["trunc_m"], cfg["sdf_s"], cfg["seed"]
    head = bp.head.cpu().numpy().astype(np.float64)
    feat = bp.feat.cpu().numpy()
    ori, dirs = bp.ori.cpu().numpy(), bp.dirs.cpu().numpy()
    g = {k: v.cpu().numpy().astype(np.float64) for k, v in d["grads"].items()}
    bmin, vs = w["vol_bbox"][:, :, 0], w["voxel_size"]
    hc = bp.hit_count.cpu().numpy()
    sel = _select_rays(hc, 0, bp.R, n_rays, 0)
    outs = [t.cpu().numpy().reshape(bp.R, -1)[sel] for t in (bp.out_rgb, bp.out_depth, bp.out_ws, bp.out_alpha)]
    z = torch.empty((bp.R, S), device=bp.dev)
    node = torch.empty((bp.R, S), dtype=torch.int32, device=bp.dev)
    bp.forward(z, node)  # the same samples and outputs as the timed step's forward
    del node
    rows = _pipeline_rows(bp, sel)
    ok_rows, eq_rows, t_err = _check_rows(fr, w, 0, ori[sel], dirs[sel], rows, _pipeline_keys(bp))
    srt = _samples_on_rows(bp, w, 0, rows, S, _jitter(seed, sel, S))
    zg = z[torch.as_tensor(sel, device=bp.dev)].cpu().numpy()
    z_mismatch = int((~np.all(zg.view(np.uint32) == srt.view(np.uint32), axis=1)).sum())
    base = orc.render_fp64(ori[sel], dirs[sel], srt, fr["fusion"]["tsdf"], bmin, vs, trunc_m, sdf_s, feat, head,
                           1e-4)
    ok = base["flags"] == 0
    fwd_err = dict(rgb=float(np.abs(outs[0] - base["rgb"])[ok].max()),
                   depth=float(np.abs(outs[1][:, 0] - base["depth"])[ok].max()),
                   ws=float(np.abs(outs[2][:, 0] - base["ws"])[ok].max()),
                   alpha=float(np.abs(outs[3][:, 0] - base["alpha"])[ok].max()))

    def L(sig, rgb):
        c, dd, ws, a, _ = orc.composite_sorted_fp64(srt, sig, rgb, 1e-4)
        return ((c * g["g_rgb"][sel]).sum(1) + dd * g["g_depth"][sel] + ws * g["g_ws"][sel]
                + a * g["g_alpha"][sel])

    fs = np.zeros((len(sel), S))
    fr_ = np.zeros((len(sel), S, 3))
    for q in range(S):
        sp, sm = base["sigma"].copy(), base["sigma"].copy()
        sp[:, q] += h
        sm[:, q] -= h
        fs[:, q] = (L(sp, base["rgb_s"]) - L(sm, base["rgb_s"])) / (2 * h)
        for k in range(3):
            rp, rm = base["rgb_s"].copy(), base["rgb_s"].copy()
            rp[:, q, k] += h
            rm[:, q, k] -= h
            fr_[:, q, k] = (L(base["sigma"], rp) - L(base["sigma"], rm)) / (2 * h)
    gs = d["grad_sigma"].cpu().numpy()[sel]
    gr = d["grad_rgb"].cpu().numpy()[sel]
    sample_fd = dict(rays=int(ok.sum()), sigma_max_abs_err=float(np.abs(gs - fs)[ok].max()),
                     sigma_max_abs=float(np.abs(fs[ok]).max()), rgb_max_abs_err=float(np.abs(gr - fr_)[ok].max()),
                     rgb_max_abs=float(np.abs(fr_[ok]).max()))
    # autograd of a plain PyTorch compositing on the GPU in float64
    R = bp.R if autograd_rays is None else min(bp.R, autograd_rays)
    ag_err_s = ag_err_r = ag_max_s = ag_max_r = 0.0
    ag_checked = 0
    for a in range(0, R, 1 << 18):
        e = min(a + (1 << 18), R)
        zz = z[a:e][None].contiguous()
        o, dr = bp.ori[a:e][None], bp.dirs[a:e][None]
        with torch.no_grad():
            sig = tsdf_density(bp.tsdf[:1], o, dr, zz, bp.vol_bbox[:1], bp.voxel_size[:1], trunc_m, sdf_s)[0]
            rgb = grid_gather(bp.feat[:1], o, dr, zz, bp.vol_bbox[:1], bp.voxel_size[:1])[0] @ bp.head.T
        sd = sig.double().requires_grad_(True)
        rd = rgb.double().requires_grad_(True)
        z64 = zz[0].double()
        valid = z64 >= 0
        nxt = torch.cat([z64[:, 1:], torch.full_like(z64[:, :1], 1e10)], 1)
        delta = torch.where(torch.arange(S, device=z.device) == S - 1, torch.full_like(z64, 1e10), nxt - z64)
        alpha = torch.where(valid, 1 - torch.exp(-sd * delta), torch.zeros_like(sd))
        f = torch.where(valid, 1 - alpha, torch.ones_like(alpha))
        t_after = torch.cumprod(f, 1)
        t_before = torch.cat([torch.ones_like(f[:, :1]), t_after[:, :-1]], 1)
        below = valid & (t_after < 1e-4)
        first = torch.where(below.any(1), below.float().argmax(1), torch.full_like(below[:, 0], S, dtype=torch.long))
        used = valid & (torch.arange(S, device=z.device)[None, :] <= first[:, None])
        tie = (used & ((t_after - 1e-4).abs() <= 1e-4 * 1e-4)).any(1)
        wgt = torch.where(used, alpha * t_before, torch.zeros_like(alpha))
        loss = ((wgt[..., None] * rd).sum(1) * d["grads"]["g_rgb"][a:e].double()).sum() + \
            ((wgt * torch.where(valid, z64, torch.zeros_like(z64))).sum(1) * d["grads"]["g_depth"][a:e].double()).sum() \
            + (wgt.sum(1) * d["grads"]["g_ws"][a:e].double()).sum() + \
            ((wgt * alpha).sum(1) * d["grads"]["g_alpha"][a:e].double()).sum()
        loss.backward()
        m = ~tie
        ag_checked += int(m.sum())
        ag_err_s = max(ag_err_s, float((d["grad_sigma"][a:e].double() - sd.grad)[m].abs().max()))
        ag_err_r = max(ag_err_r, float((d["grad_rgb"][a:e].double() - rd.grad)[m].abs().max()))
        ag_max_s = max(ag_max_s, float(sd.grad[m].abs().max()))
        ag_max_r = max(ag_max_r, float(rd.grad[m].abs().max()))
    autograd = dict(rays=ag_checked, sigma_max_abs_err=ag_err_s, sigma_max_abs=ag_max_s, rgb_max_abs_err=ag_err_r,
                    rgb_max_abs=ag_max_r)

    # grid gradients against float64 central differences over the rays reaching each entry
    def loss_rays(rays, grid, vxyz, ch, dv):
        srt_r = _samples_on_rows(bp, w, 0, _pipeline_rows(bp, rays), S, _jitter(seed, rays, S))
        pts = orc.sample_points(ori[rays], dirs[rays], srt_r).reshape(-1, 3)
        tsdf4 = fr["fusion"]["tsdf"][..., None]
        if grid == "feat":
            t = orc.grid_gather(pts, tsdf4, bmin, vs)[:, 0]
            fe = _perturbed_features(pts, feat, bmin, vs, vxyz, ch, dv)
        else:
            t = _perturbed_features(pts, tsdf4, bmin, vs, vxyz, 0, dv)[:, 0]
            fe = orc.grid_gather(pts, feat, bmin, vs)
        n = len(rays)
        sig = np.where(srt_r >= 0, (1.0 / (1.0 + np.exp(t * (trunc_m / sdf_s))) / sdf_s).reshape(n, S), 0.0)
        rgb_s = np.where((srt_r >= 0)[..., None], (fe @ head.T).reshape(n, S, 3), 0.0)
        c, dd, ws, a, f2 = orc.composite_sorted_fp64(srt_r, sig, rgb_s, 1e-4)
        loss_rays.flagged += int((f2 != 0).sum())
        return float(((c * g["g_rgb"][rays]).sum(1) + dd * g["g_depth"][rays] + ws * g["g_ws"][rays]
                      + a * g["g_alpha"][rays]).sum())
    loss_rays.flagged = 0

    res = {}
    rf = torch.zeros(bp.R, dtype=torch.long, device=bp.dev)
    for grid, gt, nch in (("feat", bp.grad_feat, C), ("tsdf", bp.grad_tsdf, 1)):
        flat = gt.reshape(-1)
        top = torch.topk(flat.abs(), n_entries // 2).indices
        nz = torch.nonzero(flat).view(-1)
        gen = torch.Generator(device="cpu").manual_seed(seed)
        rnd = nz[torch.randint(0, nz.numel(), (n_entries - top.numel(),), generator=gen).to(nz.device)]
        entries = torch.unique(torch.cat([top, rnd])).cpu().numpy()
        g_gpu = flat[torch.as_tensor(entries, device=bp.dev)].double().cpu().numpy()
        g_fd = np.zeros(len(entries))
        n_fd_rays = 0
        for k, ent in enumerate(entries):
            vox, ch = divmod(int(ent), nch)
            vxyz = (vox // (D * D), (vox // D) % D, vox % D)
            rays = _near_rays(bp, z, 0, vxyz, rf)
            n_fd_rays += len(rays)
            g_fd[k] = (loss_rays(rays, grid, vxyz, ch, h) - loss_rays(rays, grid, vxyz, ch, -h)) / (2 * h)
        gmax = float(np.abs(g_fd).max())
        res[grid] = dict(entries=len(entries), rays=n_fd_rays, max_abs_err=float(np.abs(g_gpu - g_fd).max()),
                         max_abs_fd=gmax)
    return dict(fusion_bit_exact=fusion_exact, rays=len(sel),
                traversal=dict(rays_flagged=int((~ok_rows).sum()),
                               unflagged_row_mismatches=int((ok_rows & ~eq_rows).sum()), t_max_abs_err=t_err),
                sample_mismatches=z_mismatch, composite_rays_flagged=int((~ok).sum()),
                forward_max_abs_err=fwd_err, sample_grad_fd=sample_fd, sample_grad_autograd=autograd,
                grid_grad_fd=res, grid_fd_ray_evaluations_flagged=loss_rays.flagged,
                seconds=time.perf_counter() - t_start)


def run_diff(args):
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    cfg = dict(DIFF)
    if args.small:
        cfg.update(rays=1 << 16, D=128, res=256)
    d = diff_setup(cfg, dev)
    bp = d["bp"]
    bp.build()
    torch.cuda.synchronize()
    warm = max(args.warmup, 3)
    for _ in range(warm):
        diff_step(d)
    torch.cuda.synchronize()
    if bp.status[0].item() & 1:
        raise RuntimeError("hit rows overflowed")
    n_hits = int(bp.hit_count.sum().item())
    import tempfile
    clk = ClockSampler(os.path.join(tempfile.gettempdir(), "sg_clocks_diff.csv"))
    with clk:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            diff_step(d)
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    stage_sum = {}
    for _ in range(args.steps):
        bp.events = []
        diff_step(d)
        for k, v in bp.stage_times().items():
            stage_sum[k] = stage_sum.get(k, 0.0) + v
    bp.events = None
    stages = {k: v / args.steps for k, v in stage_sum.items()}
    R, S, C = bp.R, cfg["S"], cfg["C"]
    n_touched = int(((bp.grad_feat[0] != 0).any(-1) | (bp.grad_tsdf[0] != 0)).sum().item())
    n_samples = int((d["grad_rgb"].abs().sum(-1) != 0).sum().item())
    pk, pk_kind = peaks()
    # backward: rays (ori/dir, count, valid length, hit rows) and upstream
    # gradients in; per-sample sigma / colour gradients out (16 B x S per
    # ray); touched cells: features + TSDF read, their gradients written
    ab = dict(forward=24 * R + 8 * R + 12 * n_hits + 24 * R + n_touched * (4 * C + 4),
              backward=24 * R + 8 * R + 12 * n_hits + 16 * R + 16 * R * S + n_touched * 2 * (4 * C + 4),
              grad_prep=4 * (C + 1) * cfg["D"] ** 3)
    rl = {k: ab[k] / (stages[k] / 1000.0) / 1e9 for k in ab if stages.get(k)}
    dom = max(rl, key=lambda k: stages[k])
    out = dict(metric="rays/s differentiation step (2^20 random rays, S=96, 256^3x16 grid): fwd+bwd",
               value=R / (ms / 1000.0), unit="rays/s", n_gpus=1, steps=args.steps, warmup=warm, ms_per_step=ms,
               higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
               data="synthetic (seeded scene, random rays, N(0,0.1) features, N(0,1) upstream gradients)",
               config=dict(workload=f"{R} random rays through the {cfg['D']}^3 fused volume (8^3 bricks), S={S}, "
                                    f"{cfg['D']}^3x{C} feature grid + TSDF grid, intersection + fused forward + "
                                    f"exact adjoint with grid scatters", l2="grids 1.1 GB >> L2"),
               stages_ms=stages, hits_per_ray=n_hits / R, samples_with_gradient=n_samples, touched_voxels=n_touched,
               roofline=dict(bound="hbm", kernel=dom, achieved=rl[dom], peak=pk["hbm_gbs"], unit="GB/s",
                             frac=rl[dom] / pk["hbm_gbs"], traffic=None, peak_kind=pk_kind,
                             algorithmic_bytes=ab[dom]),
               rooflines={k: dict(achieved=v, frac=v / pk["hbm_gbs"], algorithmic_bytes=ab[k]) for k, v in rl.items()},
               gpu_launches=3 * args.steps, clocks=clk.summary())  # intersection, forward, backward
    if not args.no_parity:
        out["parity"] = parity_diff(d, cfg)
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------
# multi-level tree (four levels, rate 2): build, coarse DDA + depth-first
# descent and fine sampling through the drop-in MultiLayerOctree
# (octree_traversal / ray_voxels_points_sampling, the reference's
# only_voxel_traversal=False mode)
# --------------------------------------------------------------------------
OCTREE = dict(views=4, res=512, prims=12, D=256, rate=2, levels=4, trunc=0.03, target=512, start=1, S=64, Wf=512,
              seed=19)


def octree_setup(cfg, dev):
    """The fused 256^3 occupancy (drop-in integrate_in_box), its four-level
    pyramid (build_multi_res_volumes), a 512^2 target camera's rays and
    seeded rands.  Returns pristine volumes (the build rewrites its input
    volumes with node ids, so each step restores them first)."""
    import torch

    from sailor_gb300 import synthetic as syn
    from sailor_gb300.dist import VoxelEncoding as VE
    sc = syn.make_scene(seed=cfg["seed"], n_views=cfg["views"], res=cfg["res"], n_prims=cfg["prims"], D=cfg["D"],
                        trunc=cfg["trunc"])
    D, L, rate = cfg["D"], cfg["levels"], cfg["rate"]

    def T(a, dt=torch.float32):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(dev)
    occ = torch.full((1, D, D, D), -1, dtype=torch.int32, device=dev)
    cnt = torch.zeros((1, 1), dtype=torch.int32, device=dev)
    VE.integrate_in_box(occ, cnt, T(sc["K"]), T(sc["RT"]), T(sc["colors"]), T(sc["depths"]), T(sc["vol_bbox"]),
                        T(sc["voxel_size"]), 1.0, sc["trunc_weight"], 13.5, 13.5, 0)
    vols = [occ] + [torch.full((1,) + (D // rate ** l,) * 3, -1, dtype=torch.int32, device=dev)
                    for l in range(1, L)]
    cnts = [cnt] + [torch.zeros((1, 1), dtype=torch.int32, device=dev) for _ in range(1, L)]
    VE.build_multi_res_volumes(vols, cnts, L, rate, 0)
    ori, dirs = syn.target_rays(seed=cfg["seed"], res=cfg["target"])
    S = cfg["S"]
    rands = torch.rand((1, ori.shape[1], S), generator=torch.Generator(device=dev).manual_seed(cfg["seed"]),
                       device=dev)
    return dict(sc=sc, pristine=[v.clone() for v in vols], vols=vols, cnts=cnts, ori=ori, dirs=dirs, o=T(ori),
                d=T(dirs), rands=rands, vs=T(sc["voxel_size"]), bbox=T(sc["vol_bbox"]))


def octree_tree(d, cfg):
    from sailor_gb300.dist import VoxelEncoding as VE
    L = cfg["levels"]
    totals = [int(c.sum().item()) for c in d["cnts"]]
    index = [sum(totals[:l]) for l in range(L)]
    o = VE.MultiLayerOctree(L, 1, cfg["rate"], 0)
    o.init_octree(d["vols"], totals, d["cnts"], index, d["vs"], d["bbox"])
    return o


def octree_wc(cfg):
    # coarse rows: three cells per coarse-grid edge (voxel_encoding_helper.py:573)
    return cfg["D"] * 3 // cfg["rate"] ** (cfg["levels"] - cfg["start"] - 1)


def octree_step(o, d, cfg, events=None):
    """Restore the volumes, build, traverse, sample.  events: a list that
    receives (name, start, end) CUDA events per stage."""
    import torch

    def mark():
        if events is None:
            return None
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e
    e0 = mark()
    for a, b in zip(d["vols"], d["pristine"]):
        a.copy_(b)
    o.build_octree()
    e1 = mark()
    rows = o.octree_traversal(d["o"], d["d"], octree_wc(cfg), cfg["Wf"], cfg["start"], -1, -1)
    e2 = mark()
    idx, t0, t1, vl = rows[:4]
    si, sz = o.ray_voxels_points_sampling(idx, t0, t1, vl, d["rands"], cfg["start"], cfg["S"])
    e3 = mark()
    if events is not None:
        events += [("build", e0, e1), ("traversal", e1, e2), ("sampling", e2, e3)]
    return rows, si, sz


def _cpu_octree_job(cfg, occ0, ori, dirs, vs, bbox, reps, n_rays=None):
    """The oracle's C port on the host cores (spawned process): the
    multi-level build of the whole volume, and traversal + fine sampling of
    n_rays rays drawn from the target (all of them by default), scaled to
    all its rays."""
    import time

    from oracle import oracle as orc
    L, rate, S = cfg["levels"], cfg["rate"], cfg["S"]
    R = ori.shape[1]
    n_rays = R if n_rays is None else n_rays
    pick = np.sort(np.random.default_rng(5).choice(R, n_rays, replace=False))
    rd = np.random.default_rng(6).random((1, n_rays, S), dtype=np.float32)
    out = []
    for _ in range(reps):
        t0 = time.perf_counter()
        vols, _ = orc.merge_levels(occ0, (occ0 > -1).sum(), rate, L)
        t = orc.build_octree(vols, rate)
        t1 = time.perf_counter()
        ot = orc.octree_traversal(t, ori[:, pick], dirs[:, pick], vs, bbox, cfg["start"], octree_wc(cfg),
                                  cfg["Wf"])
        orc.sample_fine(t, ot["idx"], ot["t0"], ot["t1"], ot["valid_len"], rd, vs, S, cfg["start"])
        t2 = time.perf_counter()
        sec = (t1 - t0) + (t2 - t1) * R / n_rays
        out.append(dict(value=R / sec, sample_wall_s=t2 - t0))
    return out, orc.num_threads()


def cpu_baseline_octree(cfg, occ0, ori, dirs, vs, bbox, reps):
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as ex:
        runs, cores = ex.submit(_cpu_octree_job, cfg, occ0, ori, dirs, vs, bbox, reps).result()
    return dict(value=float(np.median([r["value"] for r in runs])), unit="rays/s", cores=cores, kind="port",
                sample="oracle (C port, OpenMP) on host cores: the whole step (merge + multi-level build of "
                       "the whole volume, traversal + fine sampling of every ray of the target); median of "
                       f"{len(runs)} runs in a separate process",
                samples=[r["value"] for r in runs], sample_wall_s=[r["sample_wall_s"] for r in runs])


def parity_octree(o, d, cfg, rows, si, sz, n_rays=4096):
    """After timing: the tree bit-exact, traversal rows of n_rays rays exact
    on the rays the oracle does not flag (depths within 1e-5 relative), fine
    samples bit-exact against the oracle run on the GPU's own rows."""
    import time

    from oracle import oracle as orc
    t_start = time.perf_counter()
    L, rate, S, st = cfg["levels"], cfg["rate"], cfg["S"], cfg["start"]
    vols = [v.cpu().numpy() for v in d["pristine"]]
    ref = orc.build_octree(vols, rate)
    tree_ok = all(np.array_equal(d["vols"][l].cpu().numpy(), ref["vols"][l]) for l in range(L))
    R = d["ori"].shape[1]
    pick = np.sort(np.random.default_rng(8).choice(R, n_rays, replace=False))
    vs = d["sc"]["voxel_size"].reshape(-1).astype(np.float32)
    bb = d["sc"]["vol_bbox"].astype(np.float32)
    ot = orc.octree_traversal(ref, d["ori"][:, pick], d["dirs"][:, pick], vs, bb, st, octree_wc(cfg), cfg["Wf"])
    g = [x.cpu().numpy()[:, pick] for x in rows]
    ok = ot["flags"][0] == 0
    mism = int(np.any(g[0][0][ok] != ot["idx"][0][ok], 1).sum() + np.any(g[4][0][ok] != ot["idx_c"][0][ok], 1).sum())
    terr = float(max(np.abs(g[1][0][ok] - ot["t0"][0][ok]).max(), np.abs(g[2][0][ok] - ot["t1"][0][ok]).max()))
    vrel = float((np.abs(g[3][0, :, 0] - ot["valid_len"][0, :, 0]) /
                  np.maximum(ot["valid_len"][0, :, 0], 1e-6))[ok].max())
    rd = d["rands"].cpu().numpy()[:, pick]
    ri, rz, _ = orc.sample_fine(ref, g[0], g[1], g[2], g[3], rd, vs, S, st)
    smis = int((si.cpu().numpy()[:, pick] != ri).sum() + (sz.cpu().numpy()[:, pick] != rz).sum())
    return dict(tree_bit_exact=bool(tree_ok), rays=int(n_rays), rays_flagged=int((~ok).sum()),
                unflagged_row_mismatches=mism, t_max_abs_err=terr, valid_len_max_rel_err=vrel,
                sample_mismatches=smis, seconds=time.perf_counter() - t_start)


def run_octree(args):
    import tempfile

    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    cfg = dict(OCTREE)
    if args.small:
        cfg.update(D=128, res=256, target=256)
    d = octree_setup(cfg, dev)
    o = octree_tree(d, cfg)
    warm = max(args.warmup, 3)
    for _ in range(warm):
        rows, si, sz = octree_step(o, d, cfg)
    torch.cuda.synchronize()
    st = o._ostatus.cpu().numpy()
    if st[0]:
        raise RuntimeError(f"octree status {st.tolist()}")
    clk = ClockSampler(os.path.join(tempfile.gettempdir(), "sg_clocks_octree.csv"))
    with clk:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            rows, si, sz = octree_step(o, d, cfg)
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    stage_sum = {}
    for _ in range(args.steps):
        ev = []
        rows, si, sz = octree_step(o, d, cfg, ev)
        torch.cuda.synchronize()
        for k, a, b in ev:
            stage_sum[k] = stage_sum.get(k, 0.0) + a.elapsed_time(b)
    stages = {k: v / args.steps for k, v in stage_sum.items()}
    R, S, L = d["ori"].shape[1], cfg["S"], cfg["levels"]
    Wc, Wf = octree_wc(cfg), cfg["Wf"]
    counts = o._obufs["counts"].cpu().numpy()
    n_fine = int((rows[0] >= 0).sum().item())
    n_coarse = int((rows[4] >= 0).sum().item())
    vox = sum(int(v.numel()) for v in d["vols"])
    # algorithmic bytes: the build reads every level's volume, writes the
    # node tables (key, parent, child base, count) and each node's volume
    # entry (the volume restore is a copy of the same size, counted too);
    # the traversal reads the rays and writes both padded row sets (the
    # reference's output contract) and the valid lengths; the sampler reads
    # the fine entries, valid lengths and rands and writes S samples a ray
    ab = dict(build=8 * vox + 4 * vox + 20 * int(counts.sum()),
              traversal=24 * R + 12 * R * (Wc + Wf) + 4 * R,
              sampling=12 * n_fine + 4 * R + 4 * R * S + 8 * R * S)
    pk, pk_kind = peaks()
    rl = {k: ab[k] / (stages[k] / 1000.0) / 1e9 for k in ab if stages.get(k)}
    dom = max(rl, key=lambda k: stages[k])
    # e2e through the drop-in API from pinned host buffers: the occupancy
    # pyramid and the rays up, the samples down
    host = dict(vols=[v.cpu().pin_memory() for v in d["pristine"]], o=torch.as_tensor(d["ori"]).pin_memory(),
                d=torch.as_tensor(d["dirs"]).pin_memory(), r=d["rands"].cpu().pin_memory())
    out_i = torch.empty((1, R, S), dtype=torch.int32).pin_memory()
    out_z = torch.empty((1, R, S), dtype=torch.float32).pin_memory()
    h2d = sum(v.numel() * 4 for v in host["vols"]) + host["o"].numel() * 4 * 2 + host["r"].numel() * 4
    d2h = 2 * out_i.numel() * 4

    def e2e_step():
        for a, b in zip(d["pristine"], host["vols"]):
            a.copy_(b, non_blocking=True)
        d["o"].copy_(host["o"], non_blocking=True)
        d["d"].copy_(host["d"], non_blocking=True)
        d["rands"].copy_(host["r"], non_blocking=True)
        _, a_i, a_z = octree_step(o, d, cfg)
        out_i.copy_(a_i, non_blocking=True)
        out_z.copy_(a_z, non_blocking=True)
    e2e_step()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        e2e_step()
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    n_scan = 3
    launches = (2 + n_scan + (L - 1) * (2 + n_scan)) + 3 + 1  # build, traversal + two row pads, sampler
    out = dict(metric=f"rays/s multi-level traversal + fine sampling ({cfg['D']}^3, rate {cfg['rate']}, {L} levels, "
                      f"S={S})",
               value=R / (ms / 1000.0), unit="rays/s", n_gpus=1, steps=args.steps, warmup=warm, ms_per_step=ms,
               higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32 / i32",
               data="synthetic (seeded capsule/ellipsoid scene)",
               config=dict(workload=f"{cfg['views']} views {cfg['res']}^2 fused into {cfg['D']}^3, {L}-level rate-"
                                    f"{cfg['rate']} tree built every step, {cfg['target']}^2 target ({R} rays) "
                                    f"traversed from start level {cfg['start']} (coarse rows {Wc}, fine rows {Wf}), "
                                    f"fine sampling S={S}", l2="padded rows > L2 (2.2 GB)"),
               stages_ms=stages, coarse_per_ray=n_coarse / R, fine_per_ray=n_fine / R,
               nodes_per_level=counts.tolist(), max_coarse=int(st[1]), max_fine=int(st[2]),
               roofline=dict(bound="hbm", kernel=dom, achieved=rl[dom], peak=pk["hbm_gbs"], unit="GB/s",
                             frac=rl[dom] / pk["hbm_gbs"], traffic=None, peak_kind=pk_kind,
                             algorithmic_bytes=ab[dom]),
               rooflines={k: dict(achieved=v, frac=v / pk["hbm_gbs"], algorithmic_bytes=ab[k]) for k, v in rl.items()},
               e2e=dict(value=R / (ms_e2e / 1000.0), unit="rays/s", h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h),
               gpu_launches=launches * args.steps, clocks=clk.summary())
    if not args.no_cpu_baseline:
        occ0 = d["pristine"][0].cpu().numpy()
        out["cpu_baseline"] = cpu_baseline_octree(cfg, occ0, d["ori"], d["dirs"],
                                                  d["sc"]["voxel_size"].reshape(-1).astype(np.float32),
                                                  d["sc"]["vol_bbox"].astype(np.float32), reps=5)
    if not args.no_parity:
        out["parity"] = parity_octree(o, d, cfg, rows, si, sz)
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------
# FastNerf's occupancy network (the consumer of the samples): the tensor-core
# sg_nerf_density over sampled point-views
# --------------------------------------------------------------------------
NERF = dict(points=1 << 22, views=3, scale=0.3, seed=29)


def nerf_inputs(cfg, dev):
    import torch
    gen = torch.Generator(device=dev).manual_seed(cfg["seed"])
    B, V, N = 1, cfg["views"], cfg["points"]
    from sailor_gb300 import _native as N_
    params = (torch.randn(int(N_.lib.sg_nerf_param_count()), generator=gen, device=dev) * cfg["scale"]).half()
    z = torch.rand((B, V, N, 1), generator=gen, device=dev) * 2.5 + 0.5
    tp = torch.rand((B, V, N, 1), generator=gen, device=dev) * 2.0 - 1.0
    g = torch.randn((B, V, N, 16), generator=gen, device=dev) * 0.5
    return params, z, tp, g


# float multiply-adds per point-view (feature + geometry MLPs) and per point (sigma MLP)
NERF_MACS_PV = 18 * 64 + 3 * 64 * 64 + 18 * 16 + 16 * 8
NERF_MACS_P = 2 * 64 * 64 + 64


def _cpu_nerf_job(cfg, n_points, reps):
    """The reference's float16 network restated in numpy (oracle/fastnerf.py)
    on n_points points x V views, in a spawned process."""
    import time

    from oracle import fastnerf as fn
    rng = np.random.default_rng(cfg["seed"])
    V = cfg["views"]
    params = (rng.normal(0, 1, fn.PARAM_COUNT) * cfg["scale"]).astype(np.float16)
    z = rng.uniform(0.5, 3.0, (1, V, n_points, 1)).astype(np.float32)
    tp = rng.uniform(-1.0, 1.0, (1, V, n_points, 1)).astype(np.float32)
    g = rng.normal(0, 0.5, (1, V, n_points, 16)).astype(np.float32)
    out = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn.infer_density(z, tp, g, params, 1, n_points, V)
        out.append(n_points / (time.perf_counter() - t0))
    return out


def run_nerf(args):
    import tempfile

    import torch

    from sailor_gb300 import _native as N_
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    cfg = dict(NERF)
    if args.small:
        cfg.update(points=1 << 18)
    params, z, tp, g = nerf_inputs(cfg, dev)
    B, V, Np = 1, cfg["views"], cfg["points"]
    dens = torch.empty((B, 1, Np), device=dev)
    geo = torch.empty((B, V, Np, 8), device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)

    def step():
        N_.check(N_.lib.sg_nerf_density(N_.ptr(params), N_.ptr(z), N_.ptr(tp), N_.ptr(g), B, Np, V, N_.ptr(dens),
                                        N_.ptr(geo), N_.ptr(err), N_.stream()), "nerf_density")
    warm = max(args.warmup, 3)
    for _ in range(warm):
        step()
    torch.cuda.synchronize()
    if err.item():
        raise RuntimeError("nerf_density wait timed out")
    clk = ClockSampler(os.path.join(tempfile.gettempdir(), "sg_clocks_nerf.csv"))
    with clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    flops = 2.0 * (NERF_MACS_PV * V * Np + NERF_MACS_P * Np)
    # algorithmic bytes: inputs (z, t_psdf, 16 features) per point-view, the
    # geometry features out per point-view, the density out per point, params
    nbytes = (18 * 4 + 8 * 4) * V * Np + 4 * Np + 2 * N_.lib.sg_nerf_param_count()
    pk, pk_kind = peaks()
    # e2e through the Python drop-in from pinned host buffers
    from sailor_gb300.nerf import infer_density
    host = [t.cpu().pin_memory() for t in (z, tp, g)]
    dev_in = [torch.empty_like(t) for t in (z, tp, g)]
    out_h = torch.empty((B, 1, Np)).pin_memory()

    def e2e_step():
        for a, b in zip(dev_in, host):
            a.copy_(b, non_blocking=True)
        d = infer_density(dev_in[0], dev_in[1], dev_in[2], params, B, Np, V, 0)
        out_h.copy_(d, non_blocking=True)
    e2e_step()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        e2e_step()
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    tf = flops / (ms / 1000.0) / 1e12
    out = dict(metric="points/s FastNerf occupancy network (3 views, feature + geometry + sigma MLPs, fp16 operands)",
               value=Np / (ms / 1000.0), unit="points/s", n_gpus=1, steps=args.steps, warmup=warm, ms_per_step=ms,
               higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f16 operands, f32 sums",
               data="synthetic (seeded inputs, N(0, 0.3) float16 parameters)",
               config=dict(workload=f"{Np} points x {V} views (z, t_psdf, 16 geometry features each) -> densities "
                                    f"and geometry features", l2=f"inputs {nbytes / 1e9:.2f} GB > L2"),
               tensor_tflops=tf, hbm_gbs=nbytes / (ms / 1000.0) / 1e9,
               roofline=dict(bound="hbm", kernel="nerf_density_kernel", achieved=nbytes / (ms / 1000.0) / 1e9,
                             peak=pk["hbm_gbs"], unit="GB/s", frac=nbytes / (ms / 1000.0) / 1e9 / pk["hbm_gbs"],
                             traffic=None, peak_kind=pk_kind, algorithmic_bytes=nbytes,
                             tensor=dict(achieved=tf, peak=pk.get("bf16_tflops"), unit="TFLOP/s",
                                         frac=(tf / pk["bf16_tflops"]) if pk.get("bf16_tflops") else None,
                                         flops=flops)),
               e2e=dict(value=Np / (ms_e2e / 1000.0), unit="points/s",
                        h2d_bytes_per_step=sum(t.numel() * 4 for t in host), d2h_bytes_per_step=out_h.numel() * 4),
               gpu_launches=args.steps, clocks=clk.summary())
    if not args.no_cpu_baseline:
        import concurrent.futures as cf
        import multiprocessing as mp
        n_cpu = 1 << 14
        with cf.ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as ex:
            vals = ex.submit(_cpu_nerf_job, cfg, n_cpu, 3).result()
        out["cpu_baseline"] = dict(value=float(np.median(vals)), unit="points/s", cores=1, kind="port",
                                   sample=f"oracle/fastnerf.py (numpy restatement of the reference's float16 "
                                          f"__hfma chains) on {n_cpu} points x {V} views; median of 3",
                                   samples=vals)
    print(json.dumps(out), flush=True)


def run_reference_nerf(args):
    """--impl reference --workload nerf: the reference's own CUDA kernels
    (density_feat_kernel, torch.mean, density_sigma_kernel, from the cubin
    that oracle/build.py --fastnerf compiles) on the same inputs and GPU."""
    import torch

    from oracle import ref_cubin as rc
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    cfg = dict(NERF)
    if args.small:
        cfg.update(points=1 << 18)
    if not rc.nerf_available():
        print(json.dumps({"impl": "reference", "unavailable": "FastNerf cubin not built (oracle/build.py --fastnerf)"}))
        return
    params, z, tp, g = nerf_inputs(cfg, dev)
    B, V, Np = 1, cfg["views"], cfg["points"]
    for _ in range(max(args.warmup, 1)):
        rc.infer_density_mlp(z, tp, g, params, B, Np, V)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        rc.infer_density_mlp(z, tp, g, params, B, Np, V)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    v = Np / (ms / 1000.0)
    print(json.dumps(dict(metric="points/s FastNerf occupancy network (3 views, feature + geometry + sigma MLPs, "
                                 "fp16 operands)", value=v, unit="points/s", impl="reference", n_gpus=1,
                          steps=args.steps, warmup=args.warmup, ms_per_step=ms, higher_is_better=True,
                          scaling="weak", vs_baseline=None, dtype="f16",
                          data="synthetic (seeded inputs, N(0, 0.3) float16 parameters)",
                          config=dict(workload=f"{Np} points x {V} views, the reference's two kernels and torch.mean "
                                               "on this GPU, inputs resident (CUDA events)"),
                          e2e=dict(value=v, unit="points/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))),
          flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        if args.workload == "nerf":
            return run_reference_nerf(args)
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "project":
        return run_project(args)
    if args.workload == "diff":
        return run_diff(args)
    if args.workload == "octree":
        return run_octree(args)
    if args.workload == "nerf":
        return run_nerf(args)
    return run_plain(args)


# --------------------------------------------------------------------------
# projection into the source views + 2D feature gather (SRONet's step after
# sampling): the fused sg_project_gather against the reference's torch
# sequence on the same GPU
# --------------------------------------------------------------------------
PROJ = dict(views=4, res=512, C_geo=32, C_rgb=32, target=512, S=64, seed=13)


def torch_proj_persp(points, K, R, T, p_depths, n_views, depth_thres=0.01, min_d=0.1, max_d=4.0, res=512):
    """The reference's proj_persp (utils_render/utils_render.py:380-414) as the
    torch calls it makes, for timing."""
    if p_depths is not None:
        invalid_d = (p_depths < min_d) | (p_depths > max_d)
        points = points[:, None].repeat(1, n_views, 1, 1).view(-1, *points.shape[-2:])
    pts = R @ points + T
    ori_pts = pts.clone()
    depth = pts[:, -1:, :].clone()
    invalid = depth < depth_thres
    depth_ = depth.clone()
    depth_[invalid] = 1
    if p_depths is not None:
        invalid_d = invalid_d[:, None].repeat(1, n_views, 1, 1).view(-1, 1, invalid_d.shape[-1])
        depth[invalid_d] = -2
    pts /= depth_
    pts_screen = (K @ pts)[:, :2, :]
    grids = (pts_screen - res // 2) / (res // 2)
    grids[invalid.repeat(1, 2, 1)] = -2
    if p_depths is not None:
        grids[invalid_d.repeat(1, 2, 1)] = -2
    return ori_pts, grids, depth


def torch_forward_sample_feature(feats_geo, depths, feats_rgb, rgbs_n, xy, z):
    """BasicRenNet.forward_sample_feature (SRONet/BasicRenNet.py:245-259)."""
    import torch
    import torch.nn.functional as F
    geo = F.grid_sample(feats_geo, xy, align_corners=True, mode="bilinear")[..., 0].permute(0, 2, 1).contiguous()
    sd = F.grid_sample(depths, xy, align_corners=True, mode="bilinear")[..., 0]
    psdf = (torch.clamp(z - sd, -0.01, 0.01) * (1.0 / 0.01)).permute(0, 2, 1).contiguous()
    rgbf = F.grid_sample(feats_rgb, xy, align_corners=True, mode="bilinear")[..., 0].permute(0, 2, 1).contiguous()
    rgbs = F.grid_sample(rgbs_n, xy, align_corners=True, mode="bilinear")[..., 0].permute(0, 2, 1).contiguous()
    return geo, rgbf, psdf, rgbs


def run_project(args):
    import torch

    from oracle import oracle as orc
    from sailor_gb300 import synthetic as syn
    from sailor_gb300 import views

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    cfg = dict(PROJ)
    if args.small:
        cfg.update(target=128)
    V, H, S = cfg["views"], cfg["res"], cfg["S"]
    rng = np.random.default_rng(cfg["seed"])
    cams = syn.ring_cameras(V)
    K = np.repeat(syn.intrinsics(H)[None], V, 0).astype(np.float32)
    R = np.stack([c[0] for c in cams]).astype(np.float32)
    T = np.stack([c[1] for c in cams]).astype(np.float32).reshape(V, 3, 1)
    ori, dirs = syn.target_rays(seed=cfg["seed"], res=cfg["target"])
    Nr = ori.shape[1]
    z = np.sort(rng.uniform(1.5, 3.5, (Nr, S)), -1).astype(np.float32)
    pts_rs = (ori[0, :, None, :] + dirs[0, :, None, :] * z[..., None]).astype(np.float32)  # [Nr, S, 3]
    Np = Nr * S
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    points = t(pts_rs.reshape(1, Np, 3)).permute(0, 2, 1)  # [1, 3, N], a view as SRONet makes it
    p_depths = t(z.reshape(1, 1, Np))
    Kt, Rt, Tt = t(K), t(R), t(T)
    maps = [torch.randn((V, cfg["C_geo"], H, H), device=dev), 1.0 + 2.0 * torch.rand((V, 1, H, H), device=dev),
            torch.randn((V, cfg["C_rgb"], H, H), device=dev), torch.rand((V, 3, H, H), device=dev)]
    maps_cl = [m.contiguous(memory_format=torch.channels_last) for m in maps]
    ch = sum(m.shape[1] for m in maps)

    def ours(mp):
        return views.project_sample_features(points, Kt, Rt, Tt, p_depths, V, *mp, res=H)

    # the torch sequence in chunks of points, as SRONet renders in ray chunks
    # (cuDNN's grid_sample takes at most 2^31 output elements); chunk
    # outputs are consumed as they come, not concatenated
    chunk = 1 << 21

    def plain():
        outs = []
        for c0 in range(0, Np, chunk):
            sl = slice(c0, min(c0 + chunk, Np))
            _, grids, depth = torch_proj_persp(points[:, :, sl], Kt, Rt, Tt, p_depths[:, :, sl], V, res=H)
            xy = grids.permute(0, 2, 1).reshape(V, -1, 1, 2)
            outs.append(torch_forward_sample_feature(*maps, xy, depth))
        return outs

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    # parity of the timed paths on the first chunk (features within 1e-5 of
    # torch's fp32 grid_sample)
    a, b_ = ours(maps_cl), plain()[0]
    c1 = min(chunk, Np)
    err = max((a[1][:, :c1] - b_[0]).abs().max().item(), (a[2][:, :c1] - b_[1]).abs().max().item(),
              (a[4][:, :c1] - b_[3]).abs().max().item())
    del a, b_
    warm = max(args.warmup, 3)
    import tempfile
    clk = ClockSampler(os.path.join(tempfile.gettempdir(), "sg_clocks_project.csv"))
    with clk:
        ms = timed(lambda: ours(maps_cl), args.steps, warm)
    ms_nchw = timed(lambda: ours(maps), args.steps, warm)
    ms_plain = timed(plain, args.steps, warm)
    vp = V * Np
    value = vp / (ms / 1000.0)
    map_bytes = sum(m.numel() for m in maps) * 4
    ab = vp * (4 * ch + 4) + Np * 16 + map_bytes  # outputs + point/p_depth reads + maps once
    pk, pk_kind = peaks()
    achieved = ab / (ms / 1000.0) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and args.small:  # captured on the small case (reads do not scale with points)
        traffic = json.load(open(tpath)).get("project_gather_small")
    out = dict(metric="view-points/s projected and gathered (proj_persp + 4x grid_sample + t_psdf)", value=value,
               unit="view-points/s", n_gpus=1, steps=args.steps, warmup=warm, ms_per_step=ms, higher_is_better=True,
               scaling="weak", vs_baseline=None, dtype="f32", data="synthetic (ring cameras, N(0,1) feature maps)",
               config=dict(workload=f"{V} views of {H}^2 maps ({cfg['C_geo']}+1+{cfg['C_rgb']}+3 ch), "
                                    f"{cfg['target']}^2 rays x {S} samples ({Np} points)",
                           maps="channels-last", l2=f"maps {map_bytes / 1e6:.0f} MB, outputs "
                                                    f"{vp * (4 * ch + 4) / 1e9:.1f} GB per step >> L2"),
               ms_nchw_maps=ms_nchw, plain_torch=dict(ms_per_step=ms_plain, value=vp / (ms_plain / 1000.0),
                                                      ratio=ms_plain / ms),
               max_abs_err_vs_torch=err,
               roofline=dict(bound="hbm", kernel="project_gather", achieved=achieved, peak=pk["hbm_gbs"],
                             unit="GB/s", frac=achieved / pk["hbm_gbs"], traffic=traffic, peak_kind=pk_kind,
                             algorithmic_bytes=ab),
               gpu_launches=args.steps, clocks=clk.summary())
    if not args.no_cpu_baseline:
        n_s = 8192
        sel = rng.choice(Np, n_s, replace=False)
        p_s = pts_rs.reshape(Np, 3)[sel].T[None]
        pd_s = z.reshape(Np)[sel][None, None]
        mcpu = [m.cpu().numpy() for m in maps]
        t0 = time.perf_counter()
        _, g_s, _ = orc.proj_persp(p_s, K, R, T, pd_s, V, res=H)
        gg = np.transpose(g_s, (0, 2, 1))
        for m in mcpu:
            orc.grid_sample(m, gg)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = dict(value=V * n_s / dt, unit="view-points/s", cores=1, kind="port",
                                   sample=f"oracle float64 numpy proj_persp + 4 grid_sample on {n_s} of {Np} points")
    print(json.dumps(out), flush=True)


def run_plain(args):
    import torch
    import torch.distributed as dist

    from sailor_gb300.pipeline import FramePipeline

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    cfg = dict(CFG)
    if args.small:
        cfg.update(res=512, D=256, trunc=0.03, target=512, S=64, prims=12)
    sc, ori, dirs, color_grid, color_vs = workload(cfg, rank)
    dev = torch.device("cuda", local)

    def T(a, dt=torch.float32):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(dev)

    K, RT, col, dep = T(sc["K"]), T(sc["RT"]), T(sc["colors"]), T(sc["depths"])
    bb, vs = T(sc["vol_bbox"]), T(sc["voxel_size"])
    o, d = T(ori), T(dirs)
    cg, cbb, cvs = T(color_grid), T(np.array([[[-1.0, 1.0]] * 3], np.float32)), T(color_vs)
    n_rays = ori.shape[1]
    trunc_m = float(sc["voxel_size"][0, 0]) * sc["trunc_weight"]
    pipe = FramePipeline(1, cfg["D"], cfg["rate"], n_rays, cfg["S"], W_hits=1024, device=dev)

    fused = not args.unfused

    def step():
        pipe.build(K, RT, col, dep, bb, vs, sc["trunc_weight"])
        return pipe.render(o, d, cg, cbb, cvs, trunc_m, fused=fused)

    tuned = None
    if not args.no_autotune:
        from sailor_gb300 import autotune
        step()
        tuned = autotune.tune_pipeline(
            pipe, lambda: pipe.build(K, RT, col, dep, bb, vs, sc["trunc_weight"]),
            lambda: pipe.render(o, d, cg, cbb, cvs, trunc_m, fused=fused), cache=False, verbose=True)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    n_hits = int(pipe.hit_count.sum().item())
    if pipe.status[0].item() & 1:
        raise RuntimeError("hit rows overflowed")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident steps (value) --------------------------------------
    import tempfile
    clk = ClockSampler(os.path.join(tempfile.gettempdir(), f"sg_clocks_rank{rank}.csv"))
    pipe.events = None
    with clk:
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        barrier()
    ms_total = e0.elapsed_time(e1)
    # per-stage times: one more pass of events per step (events are cheap)
    stage_sum = {}
    for _ in range(args.steps):
        pipe.events = []
        step()
        for k, v in pipe.stage_times().items():
            stage_sum[k] = stage_sum.get(k, 0.0) + v
    pipe.events = None
    stages = {k: v / args.steps for k, v in stage_sum.items()}
    ms_max, value = whole_job(ms_total / args.steps, n_rays, world, dev)

    # ---- e2e through the public pipeline API from pinned host buffers -------
    host = {k: torch.as_tensor(np.ascontiguousarray(v)).pin_memory() for k, v in
            dict(K=sc["K"], RT=sc["RT"], col=sc["colors"], dep=sc["depths"], o=ori, d=dirs).items()}
    dev_in = {k: torch.empty(v.shape, dtype=v.dtype, device=dev) for k, v in host.items()}
    out_host = torch.empty((n_rays, 6), dtype=torch.float32).pin_memory()
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    d2h = out_host.numel() * 4

    def e2e_step():
        for k in host:
            dev_in[k].copy_(host[k], non_blocking=True)
        pipe.build(dev_in["K"], dev_in["RT"], dev_in["col"], dev_in["dep"], bb, vs, sc["trunc_weight"])
        rgb, dep_, ws, al = pipe.render(dev_in["o"], dev_in["d"], cg, cbb, cvs, trunc_m, fused=fused)
        img = torch.cat([rgb.view(-1, 3), dep_.view(-1, 1), ws.view(-1, 1), al.view(-1, 1)], 1)
        out_host.copy_(img, non_blocking=True)

    for _ in range(2):
        e2e_step()
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(args.steps):
        e2e_step()
    f1.record()
    barrier()
    _, e2e_value = whole_job(f0.elapsed_time(f1) / args.steps, n_rays, world, dev)

    if rank == 0:
        pk, pk_kind = peaks()
        S = cfg["S"]
        n_pix = cfg["views"] * cfg["res"] ** 2
        ab = algorithmic_bytes(cfg, n_hits, n_rays, S, n_pix)
        dom = max(stages, key=lambda k: stages[k])
        achieved = ab[dom] / (stages[dom] / 1000.0) / 1e9
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            traffic = json.load(open(tpath)).get(dom)
        vox = cfg["D"] ** 3
        out = dict(
            metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
            ms_per_step=ms_max, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
            data="synthetic (seeded capsule/ellipsoid scenes)",
            config=dict(workload="full-resolution plain forward: 4x1024^2 views, 512^3 TSDF, 8^3 bricks, "
                                 "1024^2 target, S=96" if not args.small else
                        "small: 4x512^2 views, 256^3 TSDF, 8^3 bricks, 512^2 target, S=64",
                        frames_per_rank=1, rays_per_step=n_rays, l2="per-step working set > 10 GB >> L2",
                        parallelism=f"replicas x{world}", fused_render=fused, launch_shapes=tuned),
            stages_ms=stages, tsdf_gvox_s=vox / (stages.get("fusion", float("nan")) / 1000.0) / 1e9,
            render_rays_s=n_rays / (sum(stages.get(k, 0) for k in ("intersect", "render", "sample", "gather",
                                                                    "composite")) / 1000.0),
            hits_per_ray=n_hits / n_rays,
            roofline=dict(bound="hbm", kernel=dom, achieved=achieved, peak=pk["hbm_gbs"], unit="GB/s",
                          frac=achieved / pk["hbm_gbs"], traffic=traffic, peak_kind=pk_kind,
                          algorithmic_bytes=ab[dom]),
            rooflines={k: dict(achieved=ab[k] / (stages[k] / 1000.0) / 1e9,
                               frac=ab[k] / (stages[k] / 1000.0) / 1e9 / pk["hbm_gbs"], algorithmic_bytes=ab[k])
                       for k in ab if stages.get(k)},
            e2e=dict(value=e2e_value, unit=UNIT, h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h),
            gpu_launches=(9 if fused else 12) * args.steps,
            clocks=clk.summary(),
        )
        if not args.no_cpu_baseline and world >= 1:
            fzc = cpu_fused_grid(sc, cfg)  # untimed set-up, then a warm-up and the timed run
            cpu_baseline(sc, ori, dirs, cfg, color_grid, color_vs, fz=fzc)
            cb = cpu_baseline(sc, ori, dirs, cfg, color_grid, color_vs, fz=fzc)
            out["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
