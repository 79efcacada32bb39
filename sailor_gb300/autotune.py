"""Launch-shape autotuner for the sm_103a kernels.

The library's host wrappers read process-wide knobs (``sg_tune_set`` /
``sg_tune_get`` in include/sailor_gb300.h): voxels per thread and CTA size
of the fusion kernel, CTA size of the intersection kernel and the grid cap
of the warp-per-ray render kernel.  ``tune_pipeline`` times the candidate
values on the caller's own workload with CUDA events (best of a few repeats
per candidate, one knob at a time, the others held at their current best)
and leaves the fastest values set.  Results are cached per shape bucket in
a JSON file so later processes skip the search.
"""
import json
import os
import sys

import torch

from . import _native as N

KNOBS = {"fuse_vpt": 0, "fuse_block": 1, "isect_block": 2, "render_warps": 3, "fuse_tiled": 4, "isect_warp": 5}

CANDIDATES = {
    "fuse_vpt": (1, 2, 4),
    "fuse_block": (64, 128, 256),  # the kernel is built for <= 256 threads
    "isect_block": (64, 128, 256),
    "render_warps": (16, 32, 64),
    "fuse_tiled": (0, 1),  # 1: 16^3 voxel tiles; 0: linear runs shaped by fuse_vpt / fuse_block
    "isect_warp": (0, 1),  # 1: a warp tests each hit brick's children; 0: each ray's thread alone
}

CACHE = os.path.join(os.path.expanduser("~"), ".cache", "sailor_gb300", "tune.json")


def set_knob(name, value):
    N.check(N.lib.sg_tune_set(KNOBS[name], int(value)), f"tune {name}={value}")


def get_knob(name):
    return int(N.lib.sg_tune_get(KNOBS[name]))


def current():
    return {k: get_knob(k) for k in KNOBS}


def _time(fn, reps):
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune(stages, reps=3, cache_key=None, cache_path=CACHE, verbose=False):
    """stages: {knob name: callable running the work that knob affects}."""
    cached = {}
    if cache_key and os.path.exists(cache_path):
        try:
            cached = json.load(open(cache_path)).get(cache_key, {})
        except (OSError, ValueError):
            cached = {}
    if cached:
        for k, v in cached.items():
            set_knob(k, v)
        return dict(cached)
    chosen = {}
    for knob, fn in stages.items():
        fn()  # warm
        torch.cuda.synchronize()
        timings = {}
        for v in CANDIDATES[knob]:
            set_knob(knob, v)
            timings[v] = _time(fn, reps)
        best = min(timings, key=timings.get)
        set_knob(knob, best)
        chosen[knob] = best
        if verbose:
            print(f"autotune {knob}: {timings} -> {best}", file=sys.stderr, flush=True)
    if cache_key:
        try:
            os.makedirs(os.path.dirname(cache_path), exist_ok=True)
            data = json.load(open(cache_path)) if os.path.exists(cache_path) else {}
            data[cache_key] = chosen
            json.dump(data, open(cache_path, "w"), indent=1)
        except (OSError, ValueError):
            pass
    return chosen


def tune_pipeline(pipe, build_fn, render_fn, reps=3, cache=True, verbose=False):
    """Tune the knobs that a FramePipeline's build/render use."""
    key = None
    if cache:
        key = f"B{pipe.B}_D{pipe.D}_r{pipe.rate}_n{pipe.n_rays}_S{pipe.S}_{torch.cuda.get_device_name()}"
    if not (cache and key and _cached(key)):
        set_knob("fuse_tiled", 0)  # the linear shape knobs only act with tiling off
    return tune({"fuse_vpt": build_fn, "fuse_block": build_fn, "fuse_tiled": build_fn,
                 "isect_warp": render_fn, "isect_block": render_fn, "render_warps": render_fn}, reps=reps,
                cache_key=key, verbose=verbose)


def _cached(key, cache_path=CACHE):
    try:
        return key in json.load(open(cache_path))
    except (OSError, ValueError):
        return False
