"""CPU checks of the multi-level tree oracle (oracle/octree_oracle.c):

* the build over two levels equals the two-level oracle (ids and rewritten
  volumes), and over three and four levels has the structure
  gen_root_octree_nodes + gen_higher_octree_nodes give (octree_kernel.cu:
  18-239): top nodes = occupied top voxels with an occupied neighbour, every
  occupied voxel under a node is its child, children in (x, y, z) order;
* the traversal's coarse rows equal the two-level traversal's top-node rows
  (the same DDA, ray_voxel_traversal :286-439), and its fine rows equal a
  pure-Python restatement of ray_octree_traversal's descent
  (intersection_kernel.cu:441-643) on the same coarse rows;
* the fine sampler equals a pure-Python restatement of
  ray_voxels_sampling_kernel + ray_voxels_further_sampling_kernel
  (sampling_kernel.cu:911-1068);
* the golden vectors of the reference's own kernels (tests/golden/
  ref_octree.npz, made by make_golden.py --only octree): node sets, coarse
  rows, fine-row multisets and fine samples set-wise.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def occ64():
    D = 64
    sc = syn.make_scene(seed=5, n_views=4, res=128, n_prims=10, D=D, trunc=0.03)
    fz = orc.integrate(sc["K"], sc["RT"], sc["colors"], sc["depths"], D, sc["vol_bbox"], sc["voxel_size"], 1.0,
                       sc["trunc_weight"], 13.5, 13.5)
    ori, dirs = syn.target_rays(seed=5, res=40)
    return dict(sc=sc, occ=fz["occ"], ori=ori, dirs=dirs)


def _tree(occ64, rate, L):
    occ = occ64["occ"]
    vols, _ = orc.merge_levels(occ, (occ > -1).reshape(occ.shape[0], -1).sum(1), rate, L)
    return vols, orc.build_octree(vols, rate)


def test_build_two_levels_matches_two_level_oracle(occ64):
    vols, t = _tree(occ64, 4, 2)
    t2 = orc.build_tree(vols[1], vols[0])
    assert t["counts"][1] == t2["ntop"] and t["counts"][0] == t2["nbot"]
    assert np.array_equal(t["vols"][1], t2["occ_top"]) and np.array_equal(t["vols"][0], t2["occ_bot"])
    assert np.array_equal(t["key"][t["cap"][0]:t["cap"][0] + t2["ntop"]], t2["top_key"][:t2["ntop"]])


@pytest.mark.parametrize("L", [3, 4])
def test_build_multi_level_structure(occ64, L):
    rate = 2
    vols, t = _tree(occ64, rate, L)
    B = vols[0].shape[0]
    coff = np.concatenate([[0], np.cumsum(t["cap"])[:-1]])
    # top: occupied with an occupied 26-neighbour, ascending linear order
    top = vols[L - 1] > -1
    Dt = top.shape[1]
    pad = np.pad(top, ((0, 0), (1, 1), (1, 1), (1, 1)))
    nb = sum(pad[:, 1 + a:1 + a + Dt, 1 + b:1 + b + Dt, 1 + c:1 + c + Dt]
             for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1) if (a, b, c) != (0, 0, 0))
    kept = np.flatnonzero((top & (nb > 0)).reshape(-1))
    nt = t["counts"][L - 1]
    assert nt == kept.size and np.array_equal(t["key"][coff[L - 1]:coff[L - 1] + nt], kept)
    for l in range(L - 1, 0, -1):
        D, Dc = vols[l].shape[1], vols[l - 1].shape[1]
        occ_c = vols[l - 1].reshape(B, -1) > -1
        expect = []
        for k in range(t["counts"][l]):
            key = int(t["key"][coff[l] + k])
            b, lin = divmod(key, D ** 3)
            X, Y, Z = lin // (D * D), (lin // D) % D, lin % D
            kids = [b * Dc ** 3 + ((X * rate + a) * Dc + (Y * rate + m)) * Dc + (Z * rate + n)
                    for a in range(rate) for m in range(rate) for n in range(rate)
                    if occ_c[b, ((X * rate + a) * Dc + (Y * rate + m)) * Dc + (Z * rate + n)]]
            assert t["child_base"][coff[l] + k] == len(expect)
            assert t["nchild"][coff[l] + k] == len(kids)
            expect += kids
            # the node's volume entry holds its id
            assert t["vols"][l].reshape(-1)[key] == t["base"][l] + k
        n = t["counts"][l - 1]
        assert n == len(expect)
        assert np.array_equal(t["key"][coff[l - 1]:coff[l - 1] + n], np.array(expect, np.int32))
        par = t["parent"][coff[l - 1]:coff[l - 1] + n]
        assert np.all(np.diff(par) >= 0) and np.all((par >= t["base"][l]) & (par < t["base"][l] + t["counts"][l]))
        got = t["vols"][l - 1].reshape(-1)[np.array(expect, np.int64)]
        assert np.array_equal(got, t["base"][l - 1] + np.arange(n))


def test_coarse_rows_equal_two_level_traversal(occ64):
    """only_voxel_traversal = false records the top nodes the DDA crosses;
    voxel_traversal in training mode records exactly those too."""
    vols, t = _tree(occ64, 4, 2)
    t2 = orc.build_tree(vols[1], vols[0])
    sc = occ64["sc"]
    vt = orc.voxel_traversal(t2, occ64["ori"], occ64["dirs"], sc["voxel_size"], sc["vol_bbox"], W=256,
                             is_training=True)
    ot = orc.octree_traversal(t, occ64["ori"], occ64["dirs"], sc["voxel_size"], sc["vol_bbox"], 0, 256, 1024)
    assert np.array_equal(ot["idx_c"], vt["idx"]) and np.array_equal(ot["t0_c"], vt["t0"])
    assert np.array_equal(ot["t1_c"], vt["t1"]) and np.array_equal(ot["cnt_c"], vt["nhit"])
    assert ot["max_coarse"] > 3
    # rate 4: the fine rows hold what the child listing of the inference
    # traversal holds, except parents merged into a child with equal depths
    vi = orc.voxel_traversal(t2, occ64["ori"], occ64["dirs"], sc["voxel_size"], sc["vol_bbox"], W=1024)
    for r in range(occ64["ori"].shape[1]):
        a = set(vi["idx"][0, r][vi["idx"][0, r] >= 0].tolist())
        b = set(ot["idx"][0, r][ot["idx"][0, r] >= 0].tolist())
        assert b <= a
        assert all(x >= t["base"][1] for x in a - b)  # only parents go missing


def _geom(t, vs, bbox, ids):
    lv = orc.octree_level_of(t, ids)
    keys = orc.octree_node_keys(t, ids)
    out = []
    for i, l in zip(ids, lv):
        k = keys[list(ids).index(i)]
        size = int(t["dims"][0] // t["dims"][l])
        c, nvs = orc.node_geometry(vs[k[1]], size, bbox[k[1], :, 0], k[2:])
        out.append((c, np.float32(nvs), int(l)))
    return out


def _slab(o, inv, c, vs):
    f_low, f_high = np.float32(0), np.float32(100000)
    h = np.float32(vs) / np.float32(2)
    for i in range(3):
        lo = (np.float32(c[i]) - h - o[i]) * inv[i]
        hi = (np.float32(c[i]) + h - o[i]) * inv[i]
        if lo > hi:
            lo, hi = hi, lo
        if hi < f_low or lo > f_high:
            return None
        f_low = lo if lo > f_low else f_low
        f_high = hi if hi < f_high else f_high
        if f_low > f_high:
            return None
    return np.float32(f_low), np.float32(f_high)


@pytest.mark.parametrize("L,start", [(3, 0), (3, 1), (4, 0)])
def test_descent_matches_python_restatement(occ64, L, start):
    rate = 2
    vols, t = _tree(occ64, rate, L)
    sc = occ64["sc"]
    vs, bbox = sc["voxel_size"].reshape(-1).astype(np.float32), sc["vol_bbox"].astype(np.float32)
    ot = orc.octree_traversal(t, occ64["ori"], occ64["dirs"], vs, bbox, start, 256, 2048)
    coff = np.concatenate([[0], np.cumsum(t["cap"])[:-1]])
    s = L - 1 - start
    rays = np.flatnonzero(ot["cnt_c"][0] > 0)[:120]
    assert rays.size > 50
    for r in rays:
        o = occ64["ori"][0, r].astype(np.float32)
        d = occ64["dirs"][0, r].astype(np.float32)
        inv = (np.float32(1) / d).astype(np.float32)
        fine, vlen = [], np.float32(0)
        for j in range(ot["cnt_c"][0, r]):
            cid = int(ot["idx_c"][0, r, j])
            ent = [[cid, ot["t0_c"][0, r, j], ot["t1_c"][0, r, j]]]
            (_, start_vs, _), = _geom(t, vs, bbox, [cid])

            def visit(l, k):
                if l == 0:
                    return
                cb, nc = t["child_base"][coff[l] + k], t["nchild"][coff[l] + k]
                for q in range(nc - 1, -1, -1):
                    kk = int(cb + q)
                    gid = int(t["base"][l - 1] + kk)
                    (c, cvs, _), = _geom(t, vs, bbox, [gid])
                    h = _slab(o, inv, c, cvs)
                    if h is None:
                        continue
                    for e in ent:
                        if e[1] == h[0] and e[2] == h[1]:
                            (_, evs, _), = _geom(t, vs, bbox, [e[0]])
                            if evs > cvs:
                                e[0] = gid
                            break
                    else:
                        ent.append([gid, h[0], h[1]])
                    visit(l - 1, kk)

            visit(s, cid - int(t["base"][s]))
            for e in ent:
                (_, evs, _), = _geom(t, vs, bbox, [e[0]])
                vlen = np.float32(vlen + np.float32((np.float32(e[2]) - np.float32(e[1])) * (start_vs / evs)))
            fine += ent
        n = ot["cnt"][0, r]
        assert n == len(fine)
        assert [e[0] for e in fine] == ot["idx"][0, r, :n].tolist()
        assert np.array_equal(np.array([e[1] for e in fine], np.float32), ot["t0"][0, r, :n])
        assert np.array_equal(np.array([e[2] for e in fine], np.float32), ot["t1"][0, r, :n])
        assert vlen == ot["valid_len"][0, r, 0]
    assert ot["need"].max() <= 8 or start == 0  # one level below the start fits the reference's 8 entries


def _sample_py(t, idx, t0, t1, vl, rd, vs, S, start):
    L = t["L"]
    lv = orc.octree_level_of(t, idx)
    start_vs = np.float32(vs * np.float32(2.0 ** (L - start - 1)))
    si = np.full(S, -1, np.int32)
    sz = np.full(S, -1, np.float32)
    has = 0
    nh = int(np.argmax(idx == -1)) if (idx == -1).any() else idx.size

    def z_of(mn, off, j, rv):
        base = np.float32(np.float64(off) * (j + 1) + np.float64(mn))
        return np.float32(np.float64(base) - np.float64(off) / 2.0 + np.float64(np.float32(off * rv)))

    for i in range(nh):
        nvs = np.float32(vs * np.float32(t["dims"][0] // t["dims"][lv[i]]))
        rt = np.float32(start_vs / nvs)
        q = np.float32(np.float32(np.float32(np.float32(t1[i] - t0[i]) * rt) * np.float32(S)) / vl)
        n = max(int(q), 1)
        off = np.float32(np.float32(t1[i] - t0[i]) / np.float32(n + 1))
        for j in range(n):
            if has >= S:
                break
            sz[has], si[has] = z_of(t0[i], off, j, rd[has]), idx[i]
            has += 1
    best = None
    for i in range(nh):
        nvs = np.float32(vs * np.float32(t["dims"][0] // t["dims"][lv[i]]))
        mid = np.float32(np.float32(t0[i] + t1[i]) / np.float32(2))
        if best is None or nvs < best[0] or (nvs == best[0] and mid < best[1]):
            best = (nvs, mid, t0[i], t1[i], idx[i])
    if best is not None and has < S:
        off = np.float32(np.float32(best[3] - best[2]) / np.float32(S - has + 1))
        for j, q in enumerate(range(has, S)):
            sz[q], si[q] = z_of(best[2], off, j, rd[q]), best[4]
    return si, sz


@pytest.mark.parametrize("L,start,S", [(3, 0, 48), (3, 1, 64), (2, 0, 32)])
def test_sample_fine_matches_python_restatement(occ64, L, start, S):
    rate = 2 if L > 2 else 4
    vols, t = _tree(occ64, rate, L)
    sc = occ64["sc"]
    vs, bbox = sc["voxel_size"].reshape(-1).astype(np.float32), sc["vol_bbox"].astype(np.float32)
    ot = orc.octree_traversal(t, occ64["ori"], occ64["dirs"], vs, bbox, start, 256, 2048)
    B, N = occ64["ori"].shape[:2]
    rd = np.random.default_rng(7).random((B, N, S), dtype=np.float32)
    si, sz, fl = orc.sample_fine(t, ot["idx"], ot["t0"], ot["t1"], ot["valid_len"], rd, vs, S, start)
    hit = ot["cnt"][0] > 0
    assert np.all((si[0][hit] >= 0).sum(1) == S) and np.all(si[0][~hit] == -1)
    rays = np.flatnonzero(hit)[:150]
    for r in rays:
        a, b = _sample_py(t, ot["idx"][0, r], ot["t0"][0, r], ot["t1"][0, r], ot["valid_len"][0, r, 0], rd[0, r],
                          vs[0], S, start)
        assert np.array_equal(a, si[0, r]) and np.array_equal(b, sz[0, r]), r
    # every sample lies inside its own entry's interval
    for r in rays[:40]:
        n = ot["cnt"][0, r]
        for q in range(S):
            e = np.flatnonzero(ot["idx"][0, r, :n] == si[0, r, q])
            assert any(ot["t0"][0, r, k] <= sz[0, r, q] <= ot["t1"][0, r, k] for k in e)


def _close(a, b, rel=1e-5):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return bool(np.all(np.abs(a - b) <= rel * np.maximum(np.abs(a), np.abs(b)) + 1e-6))


def vl_tol(ot, vl, max_scale):
    """Valid-length tolerance between the __fdividef reciprocal and 1/d:
    every entry's (t1 - t0) moves by a few ulps of its depths, times its
    scale (at most max_scale), on top of a relative 1e-5."""
    tmax = np.abs(ot["t1"][0]).max(1)
    return 1e-5 * np.abs(vl) + 8.0 * 2.0 ** -23 * tmax * ot["cnt"][0] * max_scale + 1e-7


def test_golden_octree():
    """The reference's kernels (rate 2: two levels from the top, three from
    the middle level; descents one level deep, so its 8-entry buffers
    suffice): the oracle's node sets, coarse rows, fine-row multisets
    (canonical keys with depths) and fine samples (rands 0.5, set-wise) equal
    them on every ray the oracle does not flag."""
    path = os.path.join(GOLDEN, "ref_octree.npz")
    if not os.path.exists(path):
        pytest.skip("ref_octree.npz not generated (tests/golden/make_golden.py --only octree)")
    g = np.load(path)
    rate = int(g["rate"])
    vs, bb = g["voxel_size"].reshape(-1), g["vol_bbox"]
    checked = 0
    for c in range(int(g["n_configs"])):
        key = f"c{c}_"
        L, start, S = int(g[key + "L"]), int(g[key + "start"]), int(g[key + "S"])
        t = orc.build_octree([g[key + f"occ_in_{l}"] for l in range(L)], rate)
        for l in range(L):
            ids = t["base"][l] + np.arange(t["counts"][l])
            mine = orc.octree_node_keys(t, ids)[:, 1:]
            assert sorted(map(tuple, mine.tolist())) == sorted(map(tuple, g[key + f"nodes_{l}"].tolist())), l
        ot = orc.octree_traversal(t, g["ori"], g["dirs"], vs, bb, start, int(g[key + "Wc"]), int(g[key + "Wf"]))
        ok = ot["flags"][0] == 0
        assert ok.mean() > 0.95 and ot["need"].max() <= 8
        # coarse rows: the reference's per-ray thread writes them in DDA order
        ck = orc.octree_node_keys(t, ot["idx_c"])
        assert np.array_equal(ck[0][ok], g[key + "coarse_keys"][0][ok])
        # depths: the reference multiplies by __fdividef(1, d), the oracle by 1/d
        assert _close(ot["t0_c"][0][ok], g[key + "t0_c"][0][ok])
        assert _close(ot["t1_c"][0][ok], g[key + "t1_c"][0][ok])
        # fine rows: the same entries (one per node), in an order set by the
        # reference's atomics
        fk = orc.octree_node_keys(t, ot["idx"])
        for r in np.flatnonzero(ok):
            n = ot["cnt"][0, r]
            mine = sorted(zip(map(tuple, fk[0, r, :n].tolist()), ot["t0"][0, r, :n], ot["t1"][0, r, :n]))
            m = g[key + "fine_keys"][0, r][:, 0] >= 0
            ref = sorted(zip(map(tuple, g[key + "fine_keys"][0, r][m].tolist()), g[key + "t0"][0, r][m],
                             g[key + "t1"][0, r][m]))
            assert [e[0] for e in mine] == [e[0] for e in ref], (c, r)
            assert _close(np.array([e[1:] for e in mine]), np.array([e[1:] for e in ref])), (c, r)
            checked += 1
        ref_vl = g[key + "valid_len"][0, :, 0]
        assert (np.abs(ot["valid_len"][0, :, 0] - ref_vl) <= vl_tol(ot, ref_vl, rate ** (L - 1 - start)))[ok].all()
        # fine samples on the reference's own rows (rands 0.5: depths do not
        # depend on the slot order), set-wise per ray
        lut = {tuple(k): i for i, k in enumerate(orc.octree_node_keys(t, np.arange(t["n_nodes"])).tolist())}
        fkr = g[key + "fine_keys"][0]
        idx_ref = np.full((1,) + fkr.shape[:2], -1, np.int32)
        for r in range(fkr.shape[0]):
            m = fkr[r, :, 0] >= 0
            idx_ref[0, r, :m.sum()] = [lut[tuple(k)] for k in fkr[r][m].tolist()]
        rd = np.full((1, fkr.shape[0], S), 0.5, np.float32)
        si, sz, fl = orc.sample_fine(t, idx_ref, g[key + "t0"], g[key + "t1"], g[key + "valid_len"], rd, vs, S,
                                     start)
        ok2 = fl[0] == 0
        assert ok2.mean() > 0.9
        sk = orc.octree_node_keys(t, si)
        for r in np.flatnonzero(ok2):
            mine = sorted(zip(map(tuple, sk[0, r].tolist()), sz[0, r].tolist()))
            ref = sorted(zip(map(tuple, g[key + "sample_keys"][0, r].tolist()), g[key + "sample_z"][0, r].tolist()))
            assert mine == ref, (c, r)
    assert checked > 500
