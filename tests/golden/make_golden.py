"""Generate golden vectors by running the reference's own CUDA kernels.

Run on a GPU machine after ``oracle/build.py`` has compiled the reference
cubins into ``oracle/_ref/`` (they are compiled from the SAILOR sources where
they lie; this script only loads the cubins):

    python tests/golden/make_golden.py --out <dir>

It writes ``ref_chain_explicit.npz``, ``ref_chain_auto.npz``,
``ref_composite.npz``, ``ref_rays.npz`` and ``ref_project.npz`` (``--only rays`` or
``--only project``: that one alone; ``--only octree`` writes
``ref_octree.npz`` from the multi-level tree, its depth-first traversal
and the fine sampler; ``--only trilerp`` writes ``ref_trilerp.npz`` from the
node-corner trilinear gather and its adjoint (run with inputs laid out at
the kernels' own per-sample stride, so that they stay in bounds); ``--only density_mlp`` writes
``ref_density_mlp.npz`` from FastNerf's occupancy MLP, whose cubin
``oracle/build.py --fastnerf`` builds).  Each holds the seeded inputs
and the reference outputs of fusion, coarse occupancy, the two-level tree
(as canonical node keys, since the reference's node ids depend on atomic
ordering), the voxel traversal, the coarse sampling, the sort, compositing
forward/backward.  The reference's trilinear_aggregate_features kernels step
through their [B,C,N,S,8] input and gradient tensors with a per-sample
stride of MAX_LEAVES = 64 (sampling_kernel.cu:210-213, 272-275; octree.h:13),
past the end of those tensors; ``--only trilerp`` runs them on [B,C,N,S,64]
buffers holding the 8 values at the start of each block.  The committed
copies under tests/golden/ pin the CPU oracle in the CPU test suite.
"""
import argparse
import math
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_cubin as rc  # noqa: E402
from sailor_gb300 import synthetic as syn  # noqa: E402

RES, D, RATE, VIEWS, PRIMS, TRES, S = 96, 64, 4, 4, 12, 48, 32


def canonical(table, Dt, ids):
    """node id -> (level, b, x, y, z); level 1 = top brick, -2 = not a node."""
    ids = np.asarray(ids)
    out = np.full(ids.shape + (5,), -1, np.int32)
    m = ids >= 0
    g = ids[m]
    top_depth = int(round(math.log2(Dt)))
    valid = table["valid"][g] == 1
    lvl = np.where(table["depth"][g] == top_depth, 1, 0)
    lvl = np.where(valid, lvl, -2)
    out[m, 0] = lvl
    out[m, 1] = table["batch"][g]
    out[m, 2:] = table["xyz"][g]
    return out


def chain(scene, ori, dirs, rands_list, explicit, trunc_weight, th_bbox=0.025):
    res = {}
    f = rc.integrate(scene["K"], scene["RT"], scene["colors"], scene["depths"], D, 1.0, th_bbox,
                     trunc_weight, 13.5, 13.5,
                     vol_bbox=scene["vol_bbox"] if explicit else None,
                     voxel_size=scene["voxel_size"] if explicit else None)
    for k in ("tsdf", "weight", "color", "occ", "count", "vol_origin", "vol_bbox", "voxel_size"):
        res["fusion_" + k] = f[k].cpu().numpy()
    if not explicit:
        res["Kinv"], res["Rinv"] = f["Kinv"].cpu().numpy(), f["Rinv"].cpu().numpy()
    occ0, cnt0 = f["occ"], f["count"]
    occ1, cnt1 = rc.build_multi_res_volumes(occ0, cnt0, RATE)
    res["merge_occ"], res["merge_count"] = occ1.cpu().numpy(), cnt1.cpu().numpy()
    tree = rc.Octree(occ0, occ1, cnt0, cnt1, f["voxel_size"], f["vol_bbox"], RATE)
    table = tree.node_table()
    res["tree_queue"] = tree.queue.cpu().numpy()
    res["tree_totals"] = np.array(tree.totals, np.int32)
    n = tree.n_nodes
    res["tree_node_keys"] = canonical(table, tree.Dt, np.arange(n))
    res["tree_node_children"] = canonical(table, tree.Dt, table["children"])  # [n,64,5]
    res["tree_node_centre"] = table["centre"]
    res["tree_node_vs"] = table["voxel_size"]
    res["tree_node_valid"] = table["valid"].astype(np.int32)
    res["tree_occ_top"] = occ1.cpu().numpy()
    res["tree_occ_bot"] = occ0.cpu().numpy()
    W = 4 * tree.Dt * (RATE ** 3 + 1)
    idx, t0, t1, vl, q = tree.voxel_traversal(ori, dirs, W)
    mh = tree.max_hits
    res["trav_max_hits"] = np.array(mh, np.int32)
    res["trav_count"] = q.cpu().numpy()[..., 0]
    wk = max(mh, 1)
    res["trav_keys"] = canonical(table, tree.Dt, idx[..., :wk].cpu().numpy())
    res["trav_t0"] = t0[..., :wk].cpu().numpy()
    res["trav_t1"] = t1[..., :wk].cpu().numpy()
    res["trav_valid_len"] = vl.cpu().numpy()
    for j, rands in enumerate(rands_list):
        si, sd = tree.sample_coarse(idx, t0, t1, rands, vl, S)
        res[f"samp{j}_keys"] = canonical(table, tree.Dt, si.cpu().numpy())
        res[f"samp{j}_z"] = sd.cpu().numpy()
        srt, sidx = rc.sort_samplings(sd)
        res[f"samp{j}_sorted"] = srt.cpu().numpy()
        res[f"samp{j}_sort_idx"] = sidx.cpu().numpy()
        if j == 0:
            res["_si"], res["_sd"] = si, sd
    # training-mode traversal (parents only) and early-stop variants
    idx2, t02, t12, vl2, q2 = tree.voxel_traversal(ori, dirs, W, is_training=True)
    res["trav_train_keys"] = canonical(table, tree.Dt, idx2[..., :max(tree.max_hits, 1)].cpu().numpy())
    res["trav_train_t0"] = t02[..., :max(tree.max_hits, 1)].cpu().numpy()
    res["trav_train_valid_len"] = vl2.cpu().numpy()
    idx3, _, _, _, q3 = tree.voxel_traversal(ori, dirs, W, th_early_stop=3, opt_num=6)
    res["trav_stop_keys"] = canonical(table, tree.Dt, idx3[..., :max(tree.max_hits, 1)].cpu().numpy())
    res["trav_stop_count"] = q3.cpu().numpy()[..., 0]
    return res, tree


def rays(out_dir):
    """Ray generation: two frames of two cameras each (ring cameras with the
    synthetic pinhole, and cameras with an off-centre principal point, unequal
    focal lengths and skew), 48 x 48 pixels."""
    rng = np.random.default_rng(21)
    Ks, Rs, Ts = [], [], []
    for b in range(2):
        for v in range(2):
            if v == 0:
                K = syn.intrinsics(48)
                R, T = syn.ring_cameras(1, phase=rng.uniform(0, 2 * math.pi))[0]
            else:
                K = np.array([[rng.uniform(40, 70), rng.uniform(-2, 2), rng.uniform(18, 30)],
                              [0.0, rng.uniform(40, 70), rng.uniform(18, 30)], [0.0, 0.0, 1.0]])
                R, T = syn.look_at(rng.uniform(-3, 3, 3) + np.array([0.0, 0.0, 3.5]), rng.uniform(-0.3, 0.3, 3))
            Ks.append(K)
            Rs.append(R)
            Ts.append(T)
    K = np.array(Ks, np.float32).reshape(2, 2, 3, 3)
    R = np.array(Rs, np.float32).reshape(2, 2, 3, 3)
    T = np.array(Ts, np.float32).reshape(2, 2, 3)
    res = rc.rays_calculating(K, R, T, 48)
    np.savez_compressed(os.path.join(out_dir, "ref_rays.npz"), K=K, R=R, T=T, load_size=np.array(48),
                        rays=res["rays"].cpu().numpy(), Kinv=res["Kinv"].cpu().numpy(),
                        Rinv=res["Rinv"].cpu().numpy())
    print("rays done", flush=True)


def project(out_dir):
    """project_sampled_xyz on the reference's own tree and samples: 128 rays
    of 16 samples (rays without samples included), four views; with node
    corners at 640 x 480 (half sizes not powers of two) and without at
    512 x 512.  Node ids are remapped to the referenced nodes, whose corner
    table (read from the reference's node array) and canonical keys are
    stored."""
    Sp = 16
    scene = syn.make_scene(seed=13, n_views=VIEWS, res=RES, n_prims=PRIMS, D=D, trunc=0.03)
    ori, dirs = syn.target_rays(seed=13, res=TRES)
    f = rc.integrate(scene["K"], scene["RT"], scene["colors"], scene["depths"], D, 1.0, 0.025,
                     scene["trunc_weight"], 13.5, 13.5, vol_bbox=scene["vol_bbox"], voxel_size=scene["voxel_size"])
    occ1, cnt1 = rc.build_multi_res_volumes(f["occ"], f["count"], RATE)
    tree = rc.Octree(f["occ"], occ1, f["count"], cnt1, f["voxel_size"], f["vol_bbox"], RATE)
    table = tree.node_table()
    W = 4 * tree.Dt * (RATE ** 3 + 1)
    idx, t0, t1, vl, _ = tree.voxel_traversal(ori, dirs, W)
    si, sd = tree.sample_coarse(idx, t0, t1, np.full((1, ori.shape[1], Sp), 0.5, np.float32), vl, Sp)
    si, sd = si.cpu().numpy(), sd.cpu().numpy()
    rng = np.random.default_rng(17)
    hit = np.where((si[0] >= 0).any(-1))[0]
    miss = np.where(~(si[0] >= 0).any(-1))[0]
    rays = np.sort(np.concatenate([rng.choice(hit, 120, replace=False), rng.choice(miss, 8, replace=False)]))
    o, d = ori[:, rays], dirs[:, rays]
    sub_i, sub_z = si[:, rays], sd[:, rays]
    K = scene["K"].reshape(1, VIEWS, 3, 3)
    RT = scene["RT"].reshape(1, VIEWS, 3, 4)
    out = dict(ori=o, dirs=d, sampled_z=sub_z, K=K, RT=RT, vol_bbox=scene["vol_bbox"],
               voxel_size=scene["voxel_size"], rate=np.array(RATE), Dt=np.array(tree.Dt))
    used = np.unique(sub_i[sub_i >= 0])
    remap = np.full(int(sub_i.max()) + 1 if used.size else 1, -1, np.int32)
    remap[used] = np.arange(used.size, dtype=np.int32)
    out["sampled_idx"] = np.where(sub_i >= 0, remap[np.maximum(sub_i, 0)], -1).astype(np.int32)
    out["node_corners"] = table["corners"][used]
    out["node_keys"] = canonical(table, tree.Dt, used)
    for name, (w, h, rec) in (("corners", (640, 480, True)), ("point", (512, 512, False))):
        xy, pz = rc.project_sampled_xyz(tree, o, d, sub_z, sub_i, K, RT, w, h, rec)
        out[f"{name}_size"] = np.array([w, h], np.int32)
        out[f"{name}_xy"] = xy.cpu().numpy()
        out[f"{name}_z"] = pz.cpu().numpy()
    np.savez_compressed(os.path.join(out_dir, "ref_project.npz"), **out)
    print("project done: nodes", used.size, flush=True)


def density_mlp(out_dir):
    """FastNerf's occupancy MLP (infer_density_mlp) on seeded inputs and
    float16 weights -> ref_density_mlp.npz (needs oracle/build.py
    --fastnerf)."""
    assert rc.nerf_available(), "FastNerf cubin or GPU missing"
    rng = np.random.default_rng(23)
    B, V, N = 1, 3, 512
    from oracle import fastnerf as fn
    params = (rng.normal(0, 1, fn.PARAM_COUNT) * 0.15).astype(np.float16)
    z = rng.uniform(0.5, 3.0, (B, V, N, 1)).astype(np.float32)
    tp = rng.uniform(-1.0, 1.0, (B, V, N, 1)).astype(np.float32)
    g = rng.normal(0, 0.5, (B, V, N, 16)).astype(np.float32)
    dens, geo = rc.infer_density_mlp(z, tp, g, params, B, N, V)
    np.savez_compressed(os.path.join(out_dir, "ref_density_mlp.npz"), params=params, points_z=z, points_tpsdf=tp,
                        feats_geo=g, density=dens.cpu().numpy(), geo_feats=geo.cpu().numpy(),
                        shape=np.array([B, V, N], np.int32))
    print("density_mlp done", flush=True)


def octree(out_dir):
    """Rate-2 trees over a 64^3 fine grid -- two levels traversed from the
    top (start level 0) and three levels traversed from the middle (start
    level 1) -- their octree_traversal and ray_voxels_points_sampling with
    rands 0.5 -> ref_octree.npz.  Both descents go one level below the
    coarse node: deeper ones overflow the reference's 8-entry stack.  The
    scene seed is the first whose top grid has no isolated occupied voxel in
    either tree (so the reference's traversal reads only real nodes) and
    whose descents fit the 8-entry stack and list with a margin (checked on
    the oracle before any reference launch)."""
    from oracle import oracle as orc
    rate, Dm, tres = 2, 64, 40
    configs = ((2, 0, 32), (3, 1, 48))  # (levels, start level, samples)
    for seed in range(31, 60):
        scene = syn.make_scene(seed=seed, n_views=VIEWS, res=RES, n_prims=PRIMS, D=Dm, trunc=0.03)
        f = rc.integrate(scene["K"], scene["RT"], scene["colors"], scene["depths"], Dm, 1.0, 0.025,
                         scene["trunc_weight"], 13.5, 13.5, vol_bbox=scene["vol_bbox"],
                         voxel_size=scene["voxel_size"])
        ori, dirs = syn.target_rays(seed=seed, res=tres)
        vs, bb = scene["voxel_size"].reshape(-1), scene["vol_bbox"]
        good = True
        for L, st, _ in configs:
            vols, _ = rc.merge_levels(f["occ"], rate, L)
            occ_in = [v.cpu().numpy() for v in vols]
            t = orc.build_octree(occ_in, rate)
            s_ = L - 1 - st
            good = good and np.array_equal(t["counts"], [int((v > -1).sum()) for v in occ_in])
            good = good and orc.octree_traversal(t, ori, dirs, vs, bb, st, 4 * int(t["dims"][s_]),
                                                 32 * int(t["dims"][s_]))["need"].max() <= 7
        if good:
            break
    else:
        raise RuntimeError("no seed gives complete trees with bounded descents")
    out = dict(rate=np.array(rate), seed=np.array(seed), ori=ori, dirs=dirs, n_configs=np.array(len(configs)),
               voxel_size=f["voxel_size"].cpu().numpy(), vol_bbox=f["vol_bbox"].cpu().numpy())
    for c, (L, st, S) in enumerate(configs):
        k = f"c{c}_"
        vols, _ = rc.merge_levels(f["occ"].clone(), rate, L)
        occ_in = [v.cpu().numpy() for v in vols]
        tree = rc.OctreeML(vols, f["voxel_size"], f["vol_bbox"], rate)
        assert tree.complete
        table = tree.node_table()
        out[k + "L"], out[k + "start"], out[k + "S"] = np.array(L), np.array(st), np.array(S)
        for l in range(L):
            out[k + f"occ_in_{l}"] = occ_in[l]
            ids = np.arange(tree.index[l], tree.index[l] + tree.totals[l])
            out[k + f"nodes_{l}"] = tree.canonical(ids, table)[:, 1:].astype(np.int16)
        s_ = L - 1 - st
        Wc = 4 * tree.dims[s_]
        Wf = 8 * Wc
        r = tree.octree_traversal(ori, dirs, st, Wc, Wf)
        cnt = r["cnt"].cpu().numpy()[..., 0]
        wf = max(int(cnt.max()), 1)
        wc = max(int((r["idx_c"] >= 0).sum(-1).max().item()), 1)
        out[k + "Wc"], out[k + "Wf"] = np.array(wc), np.array(wf)
        out[k + "coarse_keys"] = tree.canonical(r["idx_c"][..., :wc].cpu().numpy(), table).astype(np.int16)
        out[k + "t0_c"] = r["t0_c"][..., :wc].cpu().numpy()
        out[k + "t1_c"] = r["t1_c"][..., :wc].cpu().numpy()
        out[k + "fine_keys"] = tree.canonical(r["idx"][..., :wf].cpu().numpy(), table).astype(np.int16)
        out[k + "t0"] = r["t0"][..., :wf].cpu().numpy()
        out[k + "t1"] = r["t1"][..., :wf].cpu().numpy()
        out[k + "valid_len"] = r["valid_len"].cpu().numpy()
        rands = np.full((1, ori.shape[1], S), 0.5, np.float32)
        si, sd = tree.sample_fine(r["idx"], r["t0"], r["t1"], r["valid_len"], rands, S, st)
        out[k + "sample_keys"] = tree.canonical(si.cpu().numpy(), table).astype(np.int16)
        out[k + "sample_z"] = sd.cpu().numpy()
        print("octree", L, "levels, start", st, "coarse", wc, "fine", wf, flush=True)
    np.savez_compressed(os.path.join(out_dir, "ref_octree.npz"), **out)
    print("octree done, seed", seed, flush=True)


def trilerp(out_dir):
    """The node-corner trilinear gather and its adjoint (trilinear_aggregate_
    features(_backward)) on the reference's own two-level tree and coarse
    samples (64^3, rate 4), 128 rays with hits, 2 channels -> ref_trilerp.npz
    with each sample's node corners from the reference's node array."""
    scene = syn.make_scene(seed=11, n_views=VIEWS, res=RES, n_prims=PRIMS, D=D, trunc=0.03)
    ori, dirs = syn.target_rays(seed=11, res=TRES)
    f = rc.integrate(scene["K"], scene["RT"], scene["colors"], scene["depths"], D, 1.0, 0.025,
                     scene["trunc_weight"], 13.5, 13.5, vol_bbox=scene["vol_bbox"], voxel_size=scene["voxel_size"])
    occ1, cnt1 = rc.build_multi_res_volumes(f["occ"], f["count"], RATE)
    tree = rc.Octree(f["occ"], occ1, f["count"], cnt1, f["voxel_size"], f["vol_bbox"], RATE)
    W = 4 * tree.Dt * (RATE ** 3 + 1)
    idx, t0, t1, vl, q = tree.voxel_traversal(ori, dirs, W)
    rands = np.full((1, ori.shape[1], S), 0.5, np.float32)
    si, sd = tree.sample_coarse(idx, t0, t1, rands, vl, S)
    hit = np.flatnonzero((si.cpu().numpy()[0] >= 0).sum(1) >= S // 2)
    pick = np.random.default_rng(3).choice(hit, 128, replace=False)
    pick.sort()
    o, dr = ori[:, pick], dirs[:, pick]
    z, ix = sd[:, pick].contiguous(), si[:, pick].contiguous()
    rng = np.random.default_rng(4)
    C = 2
    feats = rng.normal(size=(1, C, 128, S, 8)).astype(np.float32)
    gout = rng.normal(size=(1, C, 128, S)).astype(np.float32)
    out, grad = rc.trilerp_nodes(tree, o, dr, z, ix, feats, gout)
    table = tree.node_table()
    ixn = ix.cpu().numpy()
    corners = table["corners"][np.where(ixn >= 0, ixn, 0)]
    np.savez_compressed(os.path.join(out_dir, "ref_trilerp.npz"), ori=o, dirs=dr, sampled_z=z.cpu().numpy(),
                        valid=(ixn >= 0).astype(np.int8), corners=corners.astype(np.float32), feats=feats, gout=gout,
                        out=out.cpu().numpy(), grad=grad.cpu().numpy())
    print("trilerp done", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--only", choices=["rays", "project", "density_mlp", "octree", "trilerp"])
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    if args.only == "density_mlp":
        density_mlp(args.out)
        return
    if args.only == "octree":
        assert rc.available(), "reference cubins or GPU missing"
        octree(args.out)
        return
    if args.only == "trilerp":
        assert rc.available(), "reference cubins or GPU missing"
        trilerp(args.out)
        return
    assert rc.available(), "reference cubins or GPU missing"
    if args.only == "project":
        project(args.out)
        return
    rays(args.out)
    if args.only == "rays":
        return
    project(args.out)
    scene = syn.make_scene(seed=11, n_views=VIEWS, res=RES, n_prims=PRIMS, D=D, trunc=0.03)
    ori, dirs = syn.target_rays(seed=11, res=TRES)
    rng = np.random.default_rng(5)
    rands = [np.full((1, ori.shape[1], S), 0.5, np.float32),
             rng.random((1, ori.shape[1], S), dtype=np.float32)]
    inputs = dict(K=scene["K"], RT=scene["RT"], depths=scene["depths"], colors=scene["colors"],
                  vol_bbox=scene["vol_bbox"], voxel_size=scene["voxel_size"], ori=ori, dirs=dirs,
                  rands0=rands[0], rands1=rands[1])
    meta = dict(D=D, rate=RATE, S=S, res=RES, trunc_weight=scene["trunc_weight"])
    for name, explicit, tw in (("explicit", True, scene["trunc_weight"]), ("auto", False, 3.0)):
        res, tree = chain(scene, ori, dirs, rands, explicit, tw)
        res.pop("_si"), res.pop("_sd")
        out = dict(inputs)
        out.update(res)
        out.update({"meta_" + k: np.array(v) for k, v in meta.items()})
        out["meta_trunc_weight"] = np.array(tw, np.float32)
        np.savez_compressed(os.path.join(args.out, f"ref_chain_{name}.npz"), **out)
        print(name, "max_hits", res["trav_max_hits"], "nodes", res["tree_queue"], flush=True)

    # compositing: random sorted/unsorted samples with -1 padding
    R, Sc = 2048, 48
    z = rng.uniform(1.5, 3.5, (1, R, Sc)).astype(np.float32)
    npad = rng.integers(0, Sc, R)
    npad[:64] = Sc  # fully invalid rays
    npad[64:128] = 0
    for r in range(R):
        z[0, r, Sc - npad[r]:] = -1.0
    sigma = rng.gamma(0.8, 20.0, (1, R, Sc, 1)).astype(np.float32)
    occv = (1.0 / (1.0 + np.exp(-rng.normal(0, 3, (1, R, Sc, 1))))).astype(np.float32)
    feats = rng.random((1, R, Sc, 3), dtype=np.float32)
    zt = rc._dev(z, torch.float32)
    srt, sidx = rc.sort_samplings(zt)
    g = [rc._dev(rng.normal(size=s).astype(np.float32), torch.float32)
         for s in ((1, R, 3), (1, R, 1), (1, R, 1), (1, R, 1))]
    comp = dict(z=z, sigma=sigma, occ=occv, feats=feats, sort_idx=sidx.cpu().numpy(),
                sorted_z=srt.cpu().numpy(), g_feat=g[0].cpu().numpy(), g_depth=g[1].cpu().numpy(),
                g_ws=g[2].cpu().numpy(), g_alpha=g[3].cpu().numpy())
    for occ in (False, True):
        tag = "occ" if occ else "den"
        sg = rc._dev(occv if occ else sigma, torch.float32)
        ft = rc._dev(feats, torch.float32)
        outs = rc.volume_rendering_forward(zt, sidx, sg, ft, 1e-4, occ)
        gf, gs = rc.volume_rendering_backward(g, outs, zt, sidx, sg, ft, 1e-4, occ)
        for k, v in zip(("feat", "depth", "ws", "alpha"), outs):
            comp[f"{tag}_fwd_{k}"] = v.cpu().numpy()
        comp[f"{tag}_bwd_feat"], comp[f"{tag}_bwd_sigma"] = gf.cpu().numpy(), gs.cpu().numpy()
    # pre-sorted occupancy rendering on the sorted depths
    occ_sorted = np.take_along_axis(occv[..., 0], sidx.cpu().numpy().astype(np.int64), 2)[..., None]
    feats_sorted = np.take_along_axis(feats, sidx.cpu().numpy().astype(np.int64)[..., None], 2)
    outs = rc.volume_rendering_occ_forward(srt, rc._dev(occ_sorted, torch.float32),
                                           rc._dev(feats_sorted, torch.float32), 1e-4)
    comp["presorted_occ"], comp["presorted_feats"] = occ_sorted, feats_sorted
    for k, v in zip(("feat", "depth", "ws", "alpha"), outs):
        comp[f"presorted_fwd_{k}"] = v.cpu().numpy()
    np.savez_compressed(os.path.join(args.out, "ref_composite.npz"), **comp)
    print("done", flush=True)


if __name__ == "__main__":
    main()
