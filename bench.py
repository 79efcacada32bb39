"""Benchmark of the VoxelEncoding hot path on one GB300 (or N replicas).

Workload (the full-resolution plain-forward configuration): one frame of 4
synthetic RGBD views at 1024x1024 (24 capsules/ellipsoids, 5 mm depth noise,
2 % dropout, uint16 depth), fused into a 512^3 TSDF grid (2 m cube, 2 cm
truncation), 8^3 bricks (64^3 top grid), then a 1024x1024 target view
rendered with up to 96 adaptive samples per ray: intersection, sampling and
per-ray sort, per-sample density (sigmoid of the fused TSDF, s = 5 mm) and
colour (trilinear from a seeded 256^3 x 3 grid), front-to-back compositing.

One step = fusion + tree build + rendering of the target view, all inputs
resident in HBM (value); e2e = the same step through the public pipeline API
from pinned host buffers (images, cameras, rays copied in; the rendered image
read back).  The per-step working set (>10 GB) is far larger than L2.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import math
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="small configuration (256^3, 512^2) for profiling")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--unfused", action="store_true",
                    help="render with four kernels (sample+sort, two field gathers, composite) instead of one")
    return ap.parse_args()


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
    oracle port of its kernels), all host threads, bounded sample per step."""
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return
    cfg = dict(CFG)
    if args.small:
        cfg.update(res=512, D=256, trunc=0.03, target=512, S=64, prims=12)
    sc, ori, dirs, color_grid, color_vs = workload(cfg)
    fz = cpu_fused_grid(sc, cfg)
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(sc, ori, dirs, cfg, color_grid, color_vs, ray_sample=4096, fusion_slab=8, fz=fz)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.median(vals)) if vals else cb["value"]
    out = dict(metric=METRIC, value=v, unit=UNIT, impl="reference", n_gpus=args.gpus, steps=args.steps,
               warmup=args.warmup, ms_per_step=1000.0 * ori.shape[1] / v, higher_is_better=True,
               scaling="weak", vs_baseline=None, dtype="f32", data="synthetic",
               config=dict(workload="full-resolution plain forward: 4x1024^2 views, 512^3 TSDF, 8^3 bricks, "
                                    "1024^2 target, S=96" if not args.small else "small", l2="inputs > L2"),
               cpu_baseline=dict(value=v, unit=UNIT, cores=cb["cores"], kind="port", sample=cb["sample"]),
               e2e=dict(value=v, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist

    from sailor_gb300.pipeline import FramePipeline

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
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
    ms = ms_total / args.steps
    t = torch.tensor([ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * n_rays / (ms_max / 1000.0)

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
    e2e_ms = f0.elapsed_time(f1) / args.steps
    t = torch.tensor([e2e_ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_value = world * n_rays / (float(t.item()) / 1000.0)

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
            data="synthetic (seeded capsule/ellipsoid scenes, see DESIGN.md)",
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
            e2e=dict(value=e2e_value, unit=UNIT, h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h),
            gpu_launches=(9 if fused else 12) * args.steps,
            clocks=clk.summary(),
        )
        if not args.no_cpu_baseline and world >= 1:
            cb = cpu_baseline(sc, ori, dirs, cfg, color_grid, color_vs)
            out["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
