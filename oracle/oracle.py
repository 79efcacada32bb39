"""NumPy front end of the C oracle (test infrastructure only).

Each method restates one reference operation of SAILOR's VoxelEncoding path
(the C source cites the reference file:line it follows) on host arrays.
Inputs are converted to contiguous float32/int32; outputs are new arrays.
"""
import ctypes as C

import numpy as np

from . import build as _build

FLAG_TIE, FLAG_ALIAS, FLAG_OVERFLOW, FLAG_TRUNC = 1, 2, 4, 8

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_vp = C.c_void_p

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        i, f, l = C.c_int, C.c_float, C.c_long
        L.orc_inverse3x3.argtypes = [_f32p, i, _f32p]
        L.orc_rays.argtypes = [_f32p, _f32p, _f32p, i, i, i, i, _f32p]
        L.orc_origin_bbox.argtypes = [_f32p, _f32p, _f32p, _f32p, i, i, i, i, f, _f32p]
        L.orc_resized_bbox.argtypes = [_f32p, i, i, _f32p, _f32p]
        L.orc_integrate.argtypes = [i, i, i, i, i, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                    f, f, f, f, _f32p, _f32p, _f32p, _i32p, _i32p]
        L.orc_integrate.restype = l
        L.orc_integrate_slab.argtypes = [i, i, i, i, i, i, i, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                         f, f, f, f, _f32p, _f32p, _f32p, _i32p, _i32p]
        L.orc_integrate_slab.restype = l
        L.orc_merge.argtypes = [i, i, i, _i32p, _i32p, _i32p]
        L.orc_build_tree.argtypes = [i, i, i, _i32p, _i32p, i, i, i, i,
                                     _i32p, _i32p, _i32p, _i32p, _i32p, _i32p]
        L.orc_build_tree.restype = i
        L.orc_voxel_traversal.argtypes = [i, i, _f32p, _f32p, i, i, _i32p, i, i, i, i,
                                          _i32p, _i32p, _i32p, _i32p, _f32p, _f32p,
                                          i, i, i, i, _i32p, _f32p, _f32p, _f32p, _i32p, _i32p]
        L.orc_voxel_traversal.restype = i
        L.orc_sample_coarse.argtypes = [i, i, i, i, _i32p, _f32p, _f32p, _f32p, _f32p,
                                        i, i, i, i, i, i, _f32p, _i32p, _f32p, _i32p]
        L.orc_sort.argtypes = [i, i, _f32p, _f32p, _i32p]
        L.orc_composite_fwd.argtypes = [i, i, i, _f32p, _vp, _f32p, _f32p, f, i,
                                        _f64p, _f64p, _f64p, _f64p, _vp]
        L.orc_composite_bwd_ref.argtypes = [i, i, i] + [_f32p] * 8 + [_f32p, _i32p, _f32p, _f32p,
                                                                      f, i, _f64p, _f64p]
        L.orc_trilerp_nodes.argtypes = [l, i, _f32p, _f32p, _i32p, _vp, _vp, _vp, _vp]
        L.orc_grid_gather.argtypes = [l, i, i, _f32p, _vp, _f32p, _f32p, _f32p, _f64p]
        L.orc_grid_scatter.argtypes = [l, i, i, i, _f32p, _vp, _f32p, _f32p, _f32p, _f64p]
        L.orc_node_geometry.argtypes = [f, i, _f32p, _i32p, _f32p, _f32p]
        L.orc_project_xyz.argtypes = [i, i, i, i, _f32p, _f32p, _f32p, _i32p, _f32p, _f32p, i, i, _vp, i,
                                      _f32p, _f32p]
        L.orc_octree_build.argtypes = [i, i, i, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p]
        L.orc_octree_build.restype = i
        L.orc_octree_traversal.argtypes = ([i, i, i, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p,
                                            _f32p, _f32p, i, _f32p, _f32p, i, i, i, i, i]
                                           + [_i32p, _f32p, _f32p, _i32p] * 2 + [_f32p, _i32p, _i32p])
        L.orc_octree_traversal.restype = i
        L.orc_sample_fine.argtypes = [i, i, i, _i32p, _i32p, _i32p, i, i, i, _i32p, _f32p, _f32p, _f32p,
                                      _f32p, i, _f32p, _i32p, _f32p, _i32p]
        L.orc_num_threads.restype = i
        L.orc_set_threads.argtypes = [i]
        _lib = L
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def num_threads():
    return lib().orc_num_threads()


def set_threads(n):
    lib().orc_set_threads(int(n))


# --------------------------------------------------------------------------
# fusion (fusion_kernel.cu)
# --------------------------------------------------------------------------
def inverse3x3(M):
    M = _f(M)
    out = np.zeros_like(M)
    lib().orc_inverse3x3(M.reshape(-1), M.size // 9, out.reshape(-1))
    return out


def rays(K, R, T, H, W=None):
    """rays_calculating (sampling_kernel.cu:674-731): K, R [B,N,3,3], T
    [B,N,3] -> [B,N,H,W,6] (ori, dir) per pixel (h, w)."""
    W = H if W is None else W
    K, R, T = _f(K), _f(R), _f(np.reshape(T, np.shape(K)[:2] + (3,)))
    B, N = K.shape[:2]
    out = np.zeros((B, N, H, W, 6), np.float32)
    lib().orc_rays(K.reshape(-1), R.reshape(-1), T.reshape(-1), B, N, H, W, out.reshape(-1))
    return out


def auto_bbox(depths, K, R, T, D, th_bbox):
    """fusion_cuda_integrate's bbox steps (fusion_kernel.cu:655-708)."""
    B, N, H, W = depths.shape
    Kinv = inverse3x3(K)
    Rinv = inverse3x3(R)
    vol_origin = np.empty((B, 3, 2), np.float32)
    vol_origin[..., 0] = 99999.0
    vol_origin[..., 1] = -99999.0
    lib().orc_origin_bbox(_f(depths).reshape(-1), Kinv.reshape(-1), Rinv.reshape(-1),
                          _f(T).reshape(-1), B, N, H, W, float(th_bbox), vol_origin.reshape(-1))
    vol_bbox = np.empty((B, 3, 2), np.float32)
    voxel_size = np.empty((B, 1), np.float32)
    lib().orc_resized_bbox(vol_origin.reshape(-1), B, D, vol_bbox.reshape(-1), voxel_size.reshape(-1))
    return vol_origin, vol_bbox, voxel_size


def integrate(K, RT, colors, depths, D, vol_bbox, voxel_size, obs_weight=1.0,
              trunc_weight=3.0, th_low=13.5, th_high=13.5):
    """integrate_cuda (fusion_kernel.cu:236-340) over a given box."""
    B, N, H, W = depths.shape
    n = B * D ** 3
    tsdf = np.empty(n, np.float32)
    weight = np.empty(n, np.float32)
    color = np.empty(n, np.float32)
    occ = np.empty(n, np.int32)
    count = np.zeros(B, np.int32)
    ties = lib().orc_integrate(B, N, H, W, D, _f(vol_bbox).reshape(-1), _f(voxel_size).reshape(-1),
                               _f(K).reshape(-1), _f(RT).reshape(-1), _f(colors).reshape(-1),
                               _f(depths).reshape(-1), float(obs_weight), float(trunc_weight),
                               float(th_low), float(th_high), tsdf, weight, color, occ, count)
    shp = (B, D, D, D)
    return dict(tsdf=tsdf.reshape(shp), weight=weight.reshape(shp), color=color.reshape(shp),
                occ=occ.reshape(shp), count=count.reshape(B, 1), ties=int(ties))


def integrate_slab(K, RT, colors, depths, D, vol_bbox, voxel_size, x_begin, x_end, obs_weight=1.0,
                   trunc_weight=3.0, th_low=13.5, th_high=13.5):
    """integrate over the x-slab [x_begin, x_end) only (outputs sized for the slab)."""
    B, N, H, W = depths.shape
    n = B * D ** 3
    tsdf = np.empty(n, np.float32)
    weight = np.empty(n, np.float32)
    color = np.empty(n, np.float32)
    occ = np.empty(n, np.int32)
    count = np.zeros(B, np.int32)
    lib().orc_integrate_slab(B, N, H, W, D, int(x_begin), int(x_end), _f(vol_bbox).reshape(-1),
                             _f(voxel_size).reshape(-1), _f(K).reshape(-1), _f(RT).reshape(-1),
                             _f(colors).reshape(-1), _f(depths).reshape(-1), float(obs_weight),
                             float(trunc_weight), float(th_low), float(th_high), tsdf, weight, color, occ, count)
    shp = (B, D, D, D)
    return dict(tsdf=tsdf.reshape(shp), occ=occ.reshape(shp), count=count)


# --------------------------------------------------------------------------
# tree (octree_kernel.cu)
# --------------------------------------------------------------------------
def merge(occ_fine, rate):
    B, Df = occ_fine.shape[0], occ_fine.shape[1]
    Dc = Df // rate
    coarse = np.empty((B, Dc, Dc, Dc), np.int32)
    count = np.zeros(B, np.int32)
    lib().orc_merge(B, Dc, rate, _i(occ_fine).reshape(-1), coarse.reshape(-1), count)
    return coarse, count.reshape(B, 1)


def build_tree(occ_top, occ_bot, base_top=None, base_bot=0, cap_top=None, cap_bot=None):
    """gen_root_octree_nodes with sequential node order; rewrites copies."""
    occ_top = _i(occ_top).copy()
    occ_bot = _i(occ_bot).copy()
    B, Dt, Db = occ_top.shape[0], occ_top.shape[1], occ_bot.shape[1]
    n_top_occ = int((occ_top > -1).sum())
    n_bot_occ = int((occ_bot > -1).sum())
    if base_top is None:
        base_top = n_bot_occ
    cap_top = n_top_occ if cap_top is None else cap_top
    cap_bot = n_bot_occ if cap_bot is None else cap_bot
    top_key = np.full(max(cap_top, 1), -1, np.int32)
    top_cb = np.zeros(max(cap_top, 1), np.int32)
    top_nc = np.zeros(max(cap_top, 1), np.int32)
    bot_key = np.full(max(cap_bot, 1), -1, np.int32)
    bot_par = np.full(max(cap_bot, 1), -1, np.int32)
    q = np.zeros(2, np.int32)
    rc = lib().orc_build_tree(B, Dt, Db, occ_top.reshape(-1), occ_bot.reshape(-1), base_top, base_bot,
                              cap_top, cap_bot, top_key, top_cb, top_nc, bot_key, bot_par, q)
    if rc != 0:
        raise RuntimeError("oracle tree build: capacity exceeded")
    nt, nb = int(q[0]), int(q[1])
    return dict(occ_top=occ_top, occ_bot=occ_bot, base_top=base_top, base_bot=base_bot,
                ntop=nt, nbot=nb, top_key=top_key[:max(nt, 1)].copy(), top_child_base=top_cb[:max(nt, 1)].copy(),
                top_nchild=top_nc[:max(nt, 1)].copy(), bot_key=bot_key[:max(nb, 1)].copy(),
                bot_parent=bot_par[:max(nb, 1)].copy(), Dt=Dt, Db=Db, B=B)


def node_geometry(vs, size, bbox_min3, idx3):
    c = np.zeros(3, np.float32)
    nvs = np.zeros(1, np.float32)
    lib().orc_node_geometry(float(vs), int(size), _f(bbox_min3), _i(idx3), c, nvs)
    return c, float(nvs[0])


def node_keys(tree, gids):
    """Canonical (level, b, x, y, z) per node id (level 1 = top brick)."""
    gids = np.asarray(gids)
    out = np.full(gids.shape + (5,), -1, np.int64)
    Dt, Db = tree["Dt"], tree["Db"]
    top = gids >= tree["base_top"]
    k = gids[top] - tree["base_top"]
    key = tree["top_key"][k].astype(np.int64)
    vt = Dt ** 3
    out[top, 0] = 1
    out[top, 1] = key // vt
    l = key % vt
    out[top, 2], out[top, 3], out[top, 4] = l // (Dt * Dt), (l // Dt) % Dt, l % Dt
    bot = (gids >= 0) & ~top
    key = tree["bot_key"][gids[bot] - tree["base_bot"]].astype(np.int64)
    vb = Db ** 3
    out[bot, 0] = 0
    out[bot, 1] = key // vb
    l = key % vb
    out[bot, 2], out[bot, 3], out[bot, 4] = l // (Db * Db), (l // Db) % Db, l % Db
    return out


# --------------------------------------------------------------------------
# intersection (intersection_kernel.cu) and sampling (sampling_kernel.cu)
# --------------------------------------------------------------------------
def voxel_traversal(tree, ori, dirs, voxel_size, vol_bbox, W=1024, th_early_stop=-1,
                    opt_num=-1, is_training=False):
    B, N = ori.shape[0], ori.shape[1]
    idx = np.full((B, N, W), -1, np.int32)
    t0 = np.full((B, N, W), -1, np.float32)
    t1 = np.full((B, N, W), -1, np.float32)
    vlen = np.zeros((B, N), np.float32)
    nhit = np.zeros((B, N), np.int32)
    flags = np.zeros((B, N), np.int32)
    mx = lib().orc_voxel_traversal(
        B, N, _f(ori).reshape(-1), _f(dirs).reshape(-1), tree["Dt"], tree["Db"],
        tree["occ_top"].reshape(-1), tree["base_top"], tree["base_bot"], tree["ntop"], tree["nbot"],
        tree["top_key"], tree["top_child_base"], tree["top_nchild"], tree["bot_key"],
        _f(voxel_size).reshape(-1), _f(vol_bbox).reshape(-1), W, th_early_stop, opt_num,
        int(bool(is_training)), idx.reshape(-1), t0.reshape(-1), t1.reshape(-1), vlen.reshape(-1),
        nhit.reshape(-1), flags.reshape(-1))
    return dict(idx=idx, t0=t0, t1=t1, valid_len=vlen[..., None], nhit=nhit, flags=flags, max_hits=int(mx))


def sample_coarse(tree, hits, rands, voxel_size, S, num_levels=2, start_level=0):
    idx, t0, t1 = hits["idx"], hits["t0"], hits["t1"]
    B, N, W = idx.shape
    sidx = np.full((B, N, S), -1, np.int32)
    sz = np.full((B, N, S), -1, np.float32)
    flags = _i(hits["flags"]).copy()
    lib().orc_sample_coarse(B, N, W, S, _i(idx).reshape(-1), _f(t0).reshape(-1), _f(t1).reshape(-1),
                            _f(rands).reshape(-1), _f(hits["valid_len"]).reshape(-1),
                            int(hits["max_hits"]), num_levels, start_level, tree["Dt"], tree["Db"],
                            tree["base_top"], _f(voxel_size).reshape(-1), sidx.reshape(-1),
                            sz.reshape(-1), flags.reshape(-1))
    return sidx, sz, flags


def sort(z):
    z = _f(z)
    S = z.shape[-1]
    R = z.size // S
    out = np.empty_like(z)
    idx = np.empty(z.shape, np.int32)
    lib().orc_sort(R, S, z.reshape(-1), out.reshape(-1), idx.reshape(-1))
    return out, idx


# --------------------------------------------------------------------------
# compositing (volume_rendering.cu)
# --------------------------------------------------------------------------
def composite_fwd(z, sort_idx, sigma, feats, t_thres=1e-4, occ_mode=False):
    z = _f(z)
    S = z.shape[-1]
    R = z.size // S
    Cf = feats.shape[-1]
    sig = _f(sigma).reshape(-1)
    ft = _f(feats).reshape(-1)
    sidx = None if sort_idx is None else _i(sort_idx)
    of = np.zeros(R * Cf, np.float64)
    od = np.zeros(R, np.float64)
    ow = np.zeros(R, np.float64)
    oa = np.zeros(R, np.float64)
    flags = np.zeros(R, np.int32)
    lib().orc_composite_fwd(R, S, Cf, z.reshape(-1), None if sidx is None else sidx.ctypes.data, sig, ft,
                            float(t_thres), int(bool(occ_mode)), of, od, ow, oa, flags.ctypes.data)
    lead = z.shape[:-1]
    return (of.reshape(lead + (Cf,)), od.reshape(lead + (1,)), ow.reshape(lead + (1,)),
            oa.reshape(lead + (1,)), flags.reshape(lead))


def composite_bwd_ref(g_feat, g_depth, g_ws, g_alpha, o_feat, o_depth, o_ws, o_alpha,
                      z, sort_idx, sigma, feats, t_thres=1e-4, occ_mode=False):
    z = _f(z)
    S = z.shape[-1]
    R = z.size // S
    Cf = feats.shape[-1]
    gf = np.zeros(R * S * Cf, np.float64)
    gs = np.zeros(R * S, np.float64)
    lib().orc_composite_bwd_ref(R, S, Cf, *[_f(a).reshape(-1) for a in (g_feat, g_depth, g_ws, g_alpha,
                                                                         o_feat, o_depth, o_ws, o_alpha)],
                                z.reshape(-1), _i(sort_idx).reshape(-1), _f(sigma).reshape(-1),
                                _f(feats).reshape(-1), float(t_thres), int(bool(occ_mode)), gf, gs)
    lead = z.shape
    return gf.reshape(lead + (Cf,)), gs.reshape(lead + (1,))


# --------------------------------------------------------------------------
# trilinear gathers (sampling_kernel.cu:162-327 and the dense-grid extension)
# --------------------------------------------------------------------------
def trilerp_nodes(pts, corners, valid, feats=None, gout=None):
    """pts [M,3], corners [M,8,3], valid [M]; feats [C,M,8]; gout [C,M]."""
    pts, corners, valid = _f(pts), _f(corners), _i(valid)
    M = pts.shape[0]
    Cf = (feats if feats is not None else gout).shape[0]
    out = np.zeros((Cf, M), np.float64) if feats is not None else None
    gin = np.zeros((Cf, M, 8), np.float64) if gout is not None else None
    fe = _f(feats) if feats is not None else None
    go = _f(gout) if gout is not None else None
    lib().orc_trilerp_nodes(M, Cf, pts.reshape(-1), corners.reshape(-1), valid,
                            None if fe is None else fe.ctypes.data, None if go is None else go.ctypes.data,
                            None if out is None else out.ctypes.data, None if gin is None else gin.ctypes.data)
    return out, gin


def grid_gather(pts, grid, bbox_min, voxel_size, batch=None):
    """pts [P,3]; grid [B,D,D,D,C]; bbox_min [B,3]; voxel_size [B]."""
    pts, grid = _f(pts), _f(grid)
    P, D, Cf = pts.shape[0], grid.shape[1], grid.shape[-1]
    out = np.zeros((P, Cf), np.float64)
    bt = None if batch is None else _i(batch)
    lib().orc_grid_gather(P, Cf, D, pts.reshape(-1), None if bt is None else bt.ctypes.data,
                          _f(bbox_min).reshape(-1), _f(voxel_size).reshape(-1), grid.reshape(-1), out)
    return out


def grid_scatter(pts, gout, B, D, bbox_min, voxel_size, batch=None):
    pts, gout = _f(pts), _f(gout)
    P, Cf = pts.shape[0], gout.shape[-1]
    gg = np.zeros((B, D, D, D, Cf), np.float64)
    bt = None if batch is None else _i(batch)
    lib().orc_grid_scatter(P, Cf, D, B, pts.reshape(-1), None if bt is None else bt.ctypes.data,
                           _f(bbox_min).reshape(-1), _f(voxel_size).reshape(-1), gout.reshape(-1),
                           gg.reshape(-1))
    return gg


# --------------------------------------------------------------------------
# projection into the views (sampling_kernel.cu:55-159, utils_render.py:380)
# and the bilinear 2D feature gather (F.grid_sample, BasicRenNet.py:245-259)
# --------------------------------------------------------------------------
def node_corner_table(tree, voxel_size, vol_bbox):
    """[n_nodes, 8, 3] corners of every node id of an oracle tree, in the
    order of OcTree::calculate_xyz_corners (octree.h:109-129, x outermost):
    the node centre plus or minus half its edge, in float32."""
    n = tree["base_top"] + tree["ntop"]
    ids = np.concatenate([np.arange(tree["base_bot"], tree["base_bot"] + tree["nbot"]),
                          np.arange(tree["base_top"], tree["base_top"] + tree["ntop"])])
    keys = node_keys(tree, ids)
    out = np.full((n, 8, 3), -1.0, np.float32)  # ids that are no node stay -1
    vs = np.asarray(voxel_size, np.float32).reshape(-1)
    bb = np.asarray(vol_bbox, np.float32).reshape(-1, 3, 2)
    rate = tree["Db"] // tree["Dt"]
    for g, key in zip(ids, keys):
        lvl, b, x, y, z = (int(v) for v in key)
        c, nvs = node_geometry(vs[b], rate if lvl == 1 else 1, bb[b, :, 0].copy(), np.array([x, y, z], np.int32))
        h = np.float32(nvs) / np.float32(2.0)
        for i in range(8):
            sgn = np.array([1 if i & 4 else -1, 1 if i & 2 else -1, 1 if i & 1 else -1], np.float32)
            out[g, i] = c + sgn * h
    return out


def project_xyz(ori, dirs, z, idx, K, RT, ori_w, ori_h, corners=None):
    """ori/dirs [B,N,3], z/idx [B,N,S], K [B,V,3,3], RT [B,V,3,4] ->
    (proj_xy [B,V,N,S,P,2], proj_z [B,V,N,S,P]) with P = 9 when a node
    corner table is given (node_corner_table), else 1."""
    z = _f(z)
    B, N, S = z.shape
    V = np.asarray(K).shape[1]
    per = 9 if corners is not None else 1
    xy = np.empty((B, V, N, S, per, 2), np.float32)
    pz = np.empty((B, V, N, S, per), np.float32)
    ct = None if corners is None else np.ascontiguousarray(corners, np.float32)
    lib().orc_project_xyz(B, V, N, S, _f(ori).reshape(-1), _f(dirs).reshape(-1), z.reshape(-1),
                          _i(idx).reshape(-1), _f(K).reshape(-1), _f(RT).reshape(-1), int(ori_w), int(ori_h),
                          None if ct is None else ct.ctypes.data, 0 if ct is None else ct.shape[0],
                          xy.reshape(-1), pz.reshape(-1))
    return xy, pz


def proj_persp(points, K, R, T, p_depths, n_views, depth_thres=0.01, min_d=0.1, max_d=4.0, res=512):
    """float64 restatement of utils_render.proj_persp (utils_render.py:380-414):
    points [B', 3, N]; K, R [n, 3, 3]; T [n, 3, 1] -> (ori_pts, grids, depth)."""
    pts = np.asarray(points, np.float64)
    K, R, T = (np.asarray(a, np.float64) for a in (K, R, T))
    n = K.shape[0]
    if p_depths is not None:
        pd = np.asarray(p_depths, np.float64)
        invalid_d = (pd < min_d) | (pd > max_d)                      # [B', 1, N]
        pts = np.repeat(pts[:, None], n_views, 1).reshape(-1, *pts.shape[-2:])
        invalid_d = np.repeat(invalid_d[:, None], n_views, 1).reshape(-1, 1, invalid_d.shape[-1])
    elif pts.shape[0] != n:
        pts = np.broadcast_to(pts, (n,) + pts.shape[1:])
    p = R @ pts + T
    ori = p.copy()
    depth = p[:, 2:3].copy()
    invalid = depth < depth_thres
    d_ = np.where(invalid, 1.0, depth)
    if p_depths is not None:
        depth[invalid_d] = -2
    scr = (K @ (p / d_))[:, :2]
    half = int(res) // 2
    grids = (scr - half) / half
    grids[np.repeat(invalid, 2, 1)] = -2
    if p_depths is not None:
        grids[np.repeat(invalid_d, 2, 1)] = -2
    return ori, grids, depth


def grid_sample(img, grid):
    """float64 F.grid_sample(img [n, C, H, W], grid [n, N, 2], bilinear,
    align_corners=True, zero padding) -> [n, N, C]."""
    img = np.asarray(img, np.float64)
    g = np.asarray(grid, np.float64)
    n, C_, H, W = img.shape
    ix = (g[..., 0] + 1) / 2 * (W - 1)
    iy = (g[..., 1] + 1) / 2 * (H - 1)
    x0, y0 = np.floor(ix), np.floor(iy)
    out = np.zeros(g.shape[:2] + (C_,))
    bidx = np.arange(n)[:, None]
    for cx, cy, w in ((x0, y0, (x0 + 1 - ix) * (y0 + 1 - iy)), (x0 + 1, y0, (ix - x0) * (y0 + 1 - iy)),
                      (x0, y0 + 1, (x0 + 1 - ix) * (iy - y0)), (x0 + 1, y0 + 1, (ix - x0) * (iy - y0))):
        ok = (cx >= 0) & (cx <= W - 1) & (cy >= 0) & (cy <= H - 1)
        xi = np.where(ok, cx, 0).astype(np.int64)
        yi = np.where(ok, cy, 0).astype(np.int64)
        v = img[bidx, :, yi, xi]                                     # [n, N, C]
        out += np.where(ok, w, 0.0)[..., None] * v
    return out


# --------------------------------------------------------------------------
# whole chain, as SRONet's forward_build + forward_ray_intersect call it
# --------------------------------------------------------------------------
def chain(scene, D, rate, S, ori, dirs, rands, W=1024, obs_weight=1.0, trunc_weight=3.0,
          th_low=13.5, th_high=13.5, th_bbox=0.025, explicit_box=True):
    """Fusion -> merge -> tree -> traversal -> sampling -> sort, on host."""
    K, RT, colors, depths = scene["K"], scene["RT"], scene["colors"], scene["depths"]
    if explicit_box:
        vol_bbox, voxel_size = scene["vol_bbox"], scene["voxel_size"]
    else:
        R = RT[..., :3]
        T = RT[..., 3]
        _, vol_bbox, voxel_size = auto_bbox(depths, K, R, T, D, th_bbox)
    fz = integrate(K, RT, colors, depths, D, vol_bbox, voxel_size, obs_weight, trunc_weight, th_low, th_high)
    top, cnt_top = merge(fz["occ"], rate)
    tree = build_tree(top, fz["occ"])
    hits = voxel_traversal(tree, ori, dirs, voxel_size, vol_bbox, W=W)
    sidx, sz, flags = sample_coarse(tree, hits, rands, voxel_size, S)
    sorted_z, sort_idx = sort(sz)
    return dict(fusion=fz, top=top, cnt_top=cnt_top, tree=tree, hits=hits, sampled_idx=sidx,
                sampled_z=sz, flags=flags, sorted_z=sorted_z, sort_idx=sort_idx,
                vol_bbox=vol_bbox, voxel_size=voxel_size)


# --------------------------------------------------------------------------
# float64 render of sorted samples (the fused render's arithmetic in FP64)
# --------------------------------------------------------------------------
def sample_points(ori, dirs, z):
    """Sample points as the render kernels form them: fma(dir, z, ori) in
    float32 (one rounding; the float64 product of two floats is exact and
    its sum with ori is exact at these magnitudes), [R, S, 3] float32."""
    o = np.asarray(ori, np.float64)[:, None, :]
    d = np.asarray(dirs, np.float64)[:, None, :]
    zz = np.maximum(np.asarray(z, np.float64), 0.0)[..., None]
    return (d * zz + o).astype(np.float32)


def composite_sorted_fp64(z, sigma, rgb, t_thres=1e-4):
    """Density compositing of samples already sorted ascending (padding -1
    first, as torch.sort leaves it) in float64, with the semantics of
    volume_rendering_training_forward_kernel (volume_rendering.cu:17-126):
    delta = next sample's depth - depth (float32 depths, exact difference),
    the last 1e10; alpha = 1 - exp(-sigma delta); w = alpha T; the sample
    whose update takes T below t_thres is the last one composited; a ray
    without a valid sample renders 0.  sigma [R, S], rgb [R, S, C] float64.
    Returns (rgb [R, C], depth, ws, alpha [R], flags [R]): FLAG_TIE where a
    composited T lies within a relative 1e-4 of t_thres (the float32 chain
    may stop one sample earlier or later there)."""
    z = np.asarray(z, np.float32)
    R, S = z.shape
    valid = z >= 0
    z64 = z.astype(np.float64)
    delta = np.empty((R, S), np.float64)
    delta[:, :-1] = z64[:, 1:] - z64[:, :-1]
    delta[:, -1] = 1e10
    sig = np.where(valid, np.asarray(sigma, np.float64), 0.0)
    with np.errstate(over="ignore", invalid="ignore"):
        alpha = np.where(valid, 1.0 - np.exp(-sig * delta), 0.0)
    f = np.where(valid, 1.0 - alpha, 1.0)
    t_after = np.cumprod(f, axis=1)
    t_before = np.concatenate([np.ones((R, 1)), t_after[:, :-1]], 1)
    below = valid & (t_after < t_thres)
    first = np.where(below.any(1), below.argmax(1), S)
    used = valid & (np.arange(S)[None, :] <= first[:, None])
    w = np.where(used, alpha * t_before, 0.0)
    out_rgb = np.einsum("rs,rsc->rc", w, np.asarray(rgb, np.float64))
    flags = np.where((used & (np.abs(t_after - t_thres) <= 1e-4 * t_thres)).any(1), FLAG_TIE, 0).astype(np.int32)
    return out_rgb, (w * np.where(valid, z64, 0.0)).sum(1), w.sum(1), (w * alpha).sum(1), flags


def render_fp64(ori, dirs, z, tsdf, bbox_min, voxel_size, trunc_m, sdf_s, feat, head=None, t_thres=1e-4,
                batch=None, feat_bbox_min=None, feat_voxel_size=None):
    """The fused render (density from the TSDF grid, colour = head @ a
    trilinear tap of a feature grid, compositing) of sorted samples, in
    float64 from the float32 sample points: sigma = sigmoid(-t trunc_m /
    sdf_s) / sdf_s with t the trilinear TSDF; rgb = head @ f (f itself when
    head is None).  ori, dirs [R, 3]; z [R, S] sorted (-1 padding first);
    tsdf [B, D, D, D]; feat [B, Df, Df, Df, C]; head [3, C]; batch [R]
    frame per ray (None: frame 0); the feature grid shares the TSDF grid's
    box unless feat_bbox_min / feat_voxel_size are given.  Returns dict(rgb
    [R, 3], depth, ws, alpha [R], sigma [R, S], rgb_s [R, S, 3], flags [R])."""
    z = np.asarray(z, np.float32)
    R, S = z.shape
    pts = sample_points(ori, dirs, z).reshape(-1, 3)
    bt = None if batch is None else np.repeat(np.asarray(batch, np.int32), S)
    t = grid_gather(pts, np.asarray(tsdf, np.float32)[..., None], bbox_min, voxel_size, batch=bt)[:, 0]
    sig = (1.0 / (1.0 + np.exp(t * (float(trunc_m) / float(sdf_s)))) / float(sdf_s)).reshape(R, S)
    fb = bbox_min if feat_bbox_min is None else feat_bbox_min
    fv = voxel_size if feat_voxel_size is None else feat_voxel_size
    fe = grid_gather(pts, feat, fb, fv, batch=bt)
    rgb_s = (fe @ np.asarray(head, np.float64).T if head is not None else fe[:, :3]).reshape(R, S, 3)
    valid = z >= 0
    sig = np.where(valid, sig, 0.0)
    rgb_s = np.where(valid[..., None], rgb_s, 0.0)
    c, d, ws, a, flags = composite_sorted_fp64(z, sig, rgb_s, t_thres)
    return dict(rgb=c, depth=d, ws=ws, alpha=a, sigma=sig, rgb_s=rgb_s, flags=flags)


def hash_uniform(seed, r, q):
    """The render's hashed jitter for ray r, sample q (a splitmix64 finaliser
    of seed + r * golden-ratio constant + q, top 24 bits / 2^24), as float32
    in [0, 1); r and q broadcast."""
    with np.errstate(over="ignore"):
        x = (np.uint64(seed) + np.asarray(r).astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
             + np.asarray(q).astype(np.uint64))
        x ^= x >> np.uint64(30)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(27)
        x *= np.uint64(0x94D049BB133111EB)
        x ^= x >> np.uint64(31)
    return (x >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def trilinear_cells(pts, bbox_min, voxel_size, batch=None):
    """Cells and corner weights of trilinear taps in float64, as the gathers
    form them: u = (p - bbox_min) / voxel_size, lower corner floor(u),
    weights of corner (dx, dy, dz) = bits (2, 1, 0) of its index.  pts [P, 3]
    float32.  Returns (i0 [P, 3] int64, w [P, 8] float64)."""
    pts = np.asarray(pts, np.float32).astype(np.float64)
    b = np.zeros(len(pts), np.int64) if batch is None else np.asarray(batch, np.int64)
    bmin = np.asarray(bbox_min, np.float32).reshape(-1, 3).astype(np.float64)[b]
    vs = np.asarray(voxel_size, np.float32).reshape(-1).astype(np.float64)[b]
    u = (pts - bmin) / vs[:, None]
    i0 = np.floor(u)
    f = u - i0
    w = np.empty((len(pts), 8))
    for cr in range(8):
        dx, dy, dz = (cr >> 2) & 1, (cr >> 1) & 1, cr & 1
        w[:, cr] = ((f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1])
                    * (f[:, 2] if dz else 1 - f[:, 2]))
    return i0.astype(np.int64), w


# --------------------------------------------------------------------------
# multi-level tree, depth-first traversal, fine sampler (octree_oracle.c)
# --------------------------------------------------------------------------
def merge_levels(occ0, counts0, rate, L):
    """build_multi_res_volumes (octree_kernel.cu:367-411) for L levels:
    volumes [level 0 (given), 1, .., L-1] and occupied counts [B, 1] each."""
    vols, cnts = [_i(occ0).copy()], [np.asarray(counts0, np.int32).reshape(-1, 1)]
    for _ in range(L - 1):
        c, n = merge(vols[-1], rate)
        vols.append(c)
        cnts.append(n)
    return vols, cnts


def build_octree(vols, rate, caps=None):
    """Multi-level tree over volumes [level 0 .. L-1] (rewrites copies).
    Node ids: base[l] = sum of the lower levels' occupied voxel counts
    (octree_nodes_index), capacities = the levels' occupied counts."""
    L = len(vols)
    B = vols[0].shape[0]
    dims = np.array([v.shape[1] for v in vols], np.int32)
    occ = [int((np.asarray(v) > -1).sum()) for v in vols]
    cap = np.array(occ if caps is None else caps, np.int32)
    base = np.concatenate([[0], np.cumsum(occ)[:-1]]).astype(np.int32)
    vol = np.concatenate([_i(v).reshape(-1) for v in vols]).astype(np.int32)
    n = max(int(cap.sum()), 1)
    key = np.full(n, -1, np.int32)
    parent = np.full(n, -1, np.int32)
    cb = np.zeros(n, np.int32)
    nc = np.zeros(n, np.int32)
    counts = np.zeros(L, np.int32)
    rc = lib().orc_octree_build(B, L, int(rate), dims, vol, base, cap, key, parent, cb, nc, counts)
    if rc != 0:
        raise RuntimeError("oracle octree build: capacity exceeded")
    out_vols, off = [], 0
    for v in vols:
        m = v.size
        out_vols.append(vol[off:off + m].reshape(v.shape).copy())
        off += m
    return dict(B=B, L=L, rate=int(rate), dims=dims, base=base, cap=cap, counts=counts, vols=out_vols,
                vol=vol, key=key, parent=parent, child_base=cb, nchild=nc, n_nodes=int(sum(occ)))


def octree_level_of(tree, ids):
    ids = np.asarray(ids)
    lv = np.full(ids.shape, -1, np.int64)
    for l in range(tree["L"]):
        m = (ids >= tree["base"][l]) & (ids < tree["base"][l] + tree["cap"][l])
        lv[m] = l
    return lv


def octree_node_keys(tree, ids):
    """Canonical (level, b, x, y, z) per node id of the multi-level tree."""
    ids = np.asarray(ids)
    out = np.full(ids.shape + (5,), -1, np.int64)
    coff = np.concatenate([[0], np.cumsum(tree["cap"])[:-1]])
    lv = octree_level_of(tree, ids)
    for l in range(tree["L"]):
        m = lv == l
        if not m.any():
            continue
        D = int(tree["dims"][l])
        key = tree["key"][coff[l] + ids[m] - tree["base"][l]].astype(np.int64)
        out[m, 0] = l
        out[m, 1] = key // D ** 3
        r = key % D ** 3
        out[m, 2], out[m, 3], out[m, 4] = r // (D * D), (r // D) % D, r % D
    return out


def octree_traversal(tree, ori, dirs, voxel_size, vol_bbox, start_level=0, Wc=256, Wf=1024, th_early_stop=-1,
                     opt_num=-1):
    B, N = ori.shape[0], ori.shape[1]
    R = B * N
    out = dict(idx_c=np.full((B, N, Wc), -1, np.int32), t0_c=np.full((B, N, Wc), -1, np.float32),
               t1_c=np.full((B, N, Wc), -1, np.float32), cnt_c=np.zeros((B, N), np.int32),
               idx=np.full((B, N, Wf), -1, np.int32), t0=np.full((B, N, Wf), -1, np.float32),
               t1=np.full((B, N, Wf), -1, np.float32), cnt=np.zeros((B, N), np.int32),
               valid_len=np.zeros((B, N), np.float32), flags=np.zeros((B, N), np.int32),
               need=np.zeros((B, N), np.int32))
    mx = lib().orc_octree_traversal(
        tree["B"], tree["L"], tree["rate"], tree["dims"], tree["vol"], tree["base"], tree["cap"], tree["counts"],
        tree["key"], tree["child_base"], tree["nchild"], _f(voxel_size).reshape(-1), _f(vol_bbox).reshape(-1), N,
        _f(ori).reshape(-1), _f(dirs).reshape(-1), int(start_level), Wc, Wf, int(th_early_stop), int(opt_num),
        out["idx_c"].reshape(-1), out["t0_c"].reshape(-1), out["t1_c"].reshape(-1), out["cnt_c"].reshape(-1),
        out["idx"].reshape(-1), out["t0"].reshape(-1), out["t1"].reshape(-1), out["cnt"].reshape(-1),
        out["valid_len"].reshape(-1), out["flags"].reshape(-1), out["need"].reshape(-1))
    del R
    out["max_fine"] = int(mx)
    out["max_coarse"] = int(out["cnt_c"].max()) if out["cnt_c"].size else 0
    out["valid_len"] = out["valid_len"][..., None]
    return out


def sample_fine(tree, idx, t0, t1, valid_len, rands, voxel_size, S, start_level=0):
    """ray_voxels_points_sampling over fine rows: (sampled_idx, sampled_z,
    flags) with FLAG_TIE near count / midpoint ties and FLAG_TRUNC where the
    entries ask for more than S samples."""
    idx, t0, t1 = _i(idx), _f(t0), _f(t1)
    B, N, W = idx.shape
    sidx = np.full((B, N, S), -1, np.int32)
    sz = np.full((B, N, S), -1, np.float32)
    flags = np.zeros((B, N), np.int32)
    lib().orc_sample_fine(tree["B"], tree["L"], tree["rate"], tree["dims"], tree["base"], tree["cap"], N, W, S,
                          idx.reshape(-1), t0.reshape(-1), t1.reshape(-1), _f(valid_len).reshape(-1),
                          _f(rands).reshape(-1), int(start_level), _f(voxel_size).reshape(-1), sidx.reshape(-1),
                          sz.reshape(-1), flags.reshape(-1))
    return sidx, sz, flags
