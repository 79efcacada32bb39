"""Run the reference's own CUDA kernels from cubins (test infrastructure).

``oracle/build.py`` compiles SAILOR's kernel sources (read in place) into
sm_103a cubins under ``oracle/_ref/``.  This module loads them with the CUDA
driver API (ctypes on libcuda) and replays the reference's host wrappers --
allocation, pre-fill values, kernel order and arguments -- with torch tensors
as device memory:

  integrate               fusion_kernel.cu:600-727
  build_multi_res_volumes octree_kernel.cu:367-411
  init_octree/build_octree octree_kernel.cu:569-697 (two levels; OctreeML:
                          any depth, gen_root + gen_higher_octree_nodes)
  octree_traversal        intersection_kernel.cu:441-643, 722-826 (OctreeML)
  ray_voxels_points_sampling sampling_kernel.cu:911-1068, 1178-1248 (OctreeML)
  voxel_traversal         intersection_kernel.cu:828-895
  ray_voxels_points_sampling_coarse sampling_kernel.cu:1251-1304
  sort_samplings          sampling_kernel.cu:1308-1329 (torch.sort)
  volume_rendering_*      volume_rendering.cu:525-787
  rays_calculating        sampling_kernel.cu:674-731
  project_sampled_xyz     sampling_kernel.cu:1333-1381

It is used only to generate golden vectors (tests/golden/make_golden.py) and
by optional GPU tests that skip when the cubins are absent.

Safety: the reference traversal reads ``octree_nodes[v]`` with v a brick's
local id for occupied bricks that were not made nodes (no occupied
neighbour), and writes hit lists without a bound.  ``voxel_traversal`` below
refuses inputs where such a read could leave the node array, and the caller
sizes the hit rows to the largest count the grid allows, so every access of
the reference kernels stays in bounds.  ``OctreeML`` runs only on trees
where every occupied voxel became a node (no such reads), and its caller
runs the descent only where the oracle shows that every coarse node's
stack and list fit the reference's 8 entries (N_STACK_MAX_NODES), with
rows as wide as the DDA's step bound allows.
"""
import ctypes as C
import os

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
OCTREE_BYTES = 1100  # sizeof(OcTree) for octree.h:30-153 with MAX_LEAVES 64

_NAMES = {
    "inverse": ("fusion_kernel", "14inverse_mat3x3PKf"),
    "origin_bbox": ("fusion_kernel", "18obtain_origin_bbox"),
    "resized_bbox": ("fusion_kernel", "19obtain_resized_bbox"),
    "integrate": ("fusion_kernel", "14integrate_cuda"),
    "merge": ("octree_kernel", "21merge_non_empty_nodes"),
    "gen_root": ("octree_kernel", "21gen_root_octree_nodes"),
    "traversal": ("intersection_kernel", "19ray_voxel_traversal"),
    "sampling": ("sampling_kernel", "ray_voxels_sampling_uniform_kernel"),
    "vr_fwd": ("volume_rendering", "volume_rendering_training_forward_kernelIfE"),
    "vr_occ_fwd": ("volume_rendering", "volume_rendering_occ_training_forward_kernelIfE"),
    "vr_bwd": ("volume_rendering", "volume_rendering_training_backward_kernelIfE"),
    "vr_occ_bwd": ("volume_rendering", "volume_rendering_occ_training_backward_kernelIfE"),
    "vr_occ": ("volume_rendering", "volume_rendering_occ_kernelIfE"),
    "rays_inverse": ("sampling_kernel", "14inverse_mat3x3IfE"),
    "rays": ("sampling_kernel", "23rays_calculating_kernelIfE"),
    "project": ("sampling_kernel", "11project_xyz"),
    "trilerp_fwd": ("sampling_kernel", "35trilinear_aggregate_features_kernel"),
    "trilerp_bwd": ("sampling_kernel", "44trilinear_aggregate_features_backward_kernel"),
    "gen_higher": ("octree_kernel", "23gen_higher_octree_nodes"),
    "octree_traversal": ("intersection_kernel", "20ray_octree_traversal"),
    "sampling_fine": ("sampling_kernel", "26ray_voxels_sampling_kernel"),
    "sampling_further": ("sampling_kernel", "34ray_voxels_further_sampling_kernel"),
}


# FastNerf inference kernels (c_lib/FastNerf/src/infer_mlp.cu), built on
# request only (oracle/build.py --fastnerf): looked up apart from the
# VoxelEncoding kernels so that available() does not wait for them
_NERF_NAMES = {
    "nerf_density_feat": ("infer_mlp", "19density_feat_kernel"),
    "nerf_density_sigma": ("infer_mlp", "20density_sigma_kernel"),
}
_NAMES.update(_NERF_NAMES)


def nerf_available():
    return os.path.exists(os.path.join(REF_DIR, "infer_mlp.cubin")) and torch.cuda.is_available()


def available():
    return all(os.path.exists(os.path.join(REF_DIR, m + ".cubin"))
               for k, (m, _) in _NAMES.items() if k not in _NERF_NAMES) and torch.cuda.is_available()


class _Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        cu = self.cu
        cu.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        cu.cuModuleGetFunctionCount.argtypes = [C.POINTER(C.c_uint), C.c_void_p]
        cu.cuModuleEnumerateFunctions.argtypes = [C.POINTER(C.c_void_p), C.c_uint, C.c_void_p]
        cu.cuFuncGetName.argtypes = [C.POINTER(C.c_char_p), C.c_void_p]
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_uint, C.c_uint, C.c_void_p,
                                      C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        self.mods = {}
        self.funcs = {}

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"CUDA driver call {what} failed: {rc}")

    def module(self, name):
        if name not in self.mods:
            with open(os.path.join(REF_DIR, name + ".cubin"), "rb") as f:
                data = f.read()
            mod = C.c_void_p()
            self.check(self.cu.cuModuleLoadData(C.byref(mod), data), "cuModuleLoadData")
            n = C.c_uint()
            self.check(self.cu.cuModuleGetFunctionCount(C.byref(n), mod), "cuModuleGetFunctionCount")
            arr = (C.c_void_p * n.value)()
            self.check(self.cu.cuModuleEnumerateFunctions(arr, n, mod), "cuModuleEnumerateFunctions")
            names = {}
            for fptr in arr:
                nm = C.c_char_p()
                self.check(self.cu.cuFuncGetName(C.byref(nm), fptr), "cuFuncGetName")
                names[nm.value.decode()] = fptr
            self.mods[name] = (mod, names)
        return self.mods[name]

    def func(self, key):
        if key not in self.funcs:
            mod, sub = _NAMES[key]
            _, names = self.module(mod)
            hits = [v for k, v in names.items() if sub in k]
            if len(hits) != 1:
                raise RuntimeError(f"kernel {sub}: {len(hits)} matches in {mod}")
            self.funcs[key] = hits[0]
        return self.funcs[key]

    def launch(self, key, n_items, args, block=128):
        f = self.func(key)
        grid = max(1, min((int(n_items) + block - 1) // block, 1 << 20))
        vals = []
        for a in args:
            if isinstance(a, torch.Tensor):
                assert a.is_cuda and a.is_contiguous()
                vals.append(C.c_void_p(a.data_ptr()))
            else:
                vals.append(a)
        ptrs = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.check(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, stream, ptrs, None),
                   f"cuLaunchKernel({key})")


_drv = None


def driver():
    global _drv
    if _drv is None:
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        _drv = _Driver()
    return _drv


i32, f32, u32, sz, cb = C.c_int, C.c_float, C.c_uint32, C.c_size_t, C.c_bool


def _dev(a, dt):
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=dt).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt).cuda().contiguous()


# --------------------------------------------------------------------------
def integrate(K, RT, colors, depths, D, obs_weight, th_bbox, trunc_weight, th_low, th_high,
              vol_bbox=None, voxel_size=None):
    """fusion_cuda_integrate (fusion_kernel.cu:600-727).  With vol_bbox and
    voxel_size given, the bbox steps are skipped (explicit box)."""
    d = driver()
    B, N, H, W = depths.shape
    Kt, RTt = _dev(K, torch.float32), _dev(RT, torch.float32)
    Rt = _dev(np.ascontiguousarray(RT[..., :3]), torch.float32)
    Tt = _dev(np.ascontiguousarray(RT[..., 3]), torch.float32)
    col, dep = _dev(colors, torch.float32), _dev(depths, torch.float32)
    masks = _dev((depths > 0).astype(np.int32), torch.int32)
    occ = torch.full((B, D, D, D), -1, dtype=torch.int32, device="cuda")
    cnt = torch.zeros((B, 1), dtype=torch.int32, device="cuda")
    origin = torch.cat([torch.full((B, 3, 1), 99999.0, device="cuda"),
                        torch.full((B, 3, 1), -99999.0, device="cuda")], 2).contiguous()
    if vol_bbox is None:
        bbox = torch.empty((B, 3, 2), device="cuda")
        vsz = torch.empty((B, 1), device="cuda")
        kinv = torch.zeros((B, N, 3, 3), device="cuda")
        rinv = torch.zeros((B, N, 3, 3), device="cuda")
        d.launch("inverse", B * N, [Kt, i32(B), i32(N), kinv])
        d.launch("inverse", B * N, [Rt, i32(B), i32(N), rinv])
        d.launch("origin_bbox", B * N * H * W, [dep, kinv, rinv, Tt, sz(H), sz(W), i32(B), i32(N),
                                                origin, f32(th_bbox)])
        d.launch("resized_bbox", B, [origin, i32(B), i32(D), bbox, vsz])
    else:
        bbox = _dev(vol_bbox, torch.float32)
        vsz = _dev(voxel_size, torch.float32)
        kinv = rinv = None
    tsdf = torch.full((B, D, D, D), 1.0, device="cuda")
    weight = torch.zeros((B, D, D, D), device="cuda")
    color = torch.zeros((B, D, D, D), device="cuda")
    d.launch("integrate", B * D ** 3, [tsdf, weight, color, occ, cnt, bbox, Kt, RTt, col, dep, masks, vsz,
                                       f32(obs_weight), i32(H), i32(W), i32(B), i32(N), i32(D ** 3),
                                       f32(trunc_weight), f32(th_low), f32(th_high), i32(D), i32(D), i32(D)])
    torch.cuda.synchronize()
    out = dict(tsdf=tsdf, weight=weight, color=color, occ=occ, count=cnt, vol_origin=origin,
               vol_bbox=bbox, voxel_size=vsz)
    if kinv is not None:
        out["Kinv"], out["Rinv"] = kinv, rinv
    return out


def build_multi_res_volumes(occ0, cnt0, rate):
    """Two levels: merge_non_empty_nodes (octree_kernel.cu:242-303)."""
    d = driver()
    B, Db = occ0.shape[0], occ0.shape[1]
    Dt = Db // rate
    occ1 = torch.full((B, Dt, Dt, Dt), -1, dtype=torch.int32, device="cuda")
    cnt1 = torch.zeros((B, 1), dtype=torch.int32, device="cuda")
    d.launch("merge", B * Dt ** 3, [occ1, cnt1, occ0, i32(Dt), i32(Db), i32(B)])
    torch.cuda.synchronize()
    return occ1, cnt1


class Octree:
    """MultiLayerOctree for two levels (octree_kernel.cu:569-697)."""

    def __init__(self, occ0, occ1, cnt0, cnt1, voxel_size, vol_bbox, rate):
        d = driver()
        self.B, self.Db, self.Dt = occ0.shape[0], occ0.shape[1], occ1.shape[1]
        self.rate = rate
        # the reference's children_gindex[MAX_LEAVES=64] (octree.h:13,53)
        # holds rate**3 entries only for rate <= 4
        assert rate ** 3 <= 64, "reference node layout supports rate <= 4 only"
        tot0, tot1 = int(cnt0.sum()), int(cnt1.sum())
        self.totals = [tot0, tot1]
        self.index = [0, tot0]
        self.n_nodes = tot0 + tot1
        self.nodes = torch.zeros(max(self.n_nodes, 1) * OCTREE_BYTES, dtype=torch.uint8, device="cuda")
        self.queue = torch.zeros(2, dtype=torch.int32, device="cuda")
        self.occ0, self.occ1 = occ0, occ1
        self.voxel_size, self.vol_bbox = voxel_size, vol_bbox
        base = self.nodes.data_ptr()
        d.launch("gen_root", self.B * self.Dt ** 3,
                 [occ1, occ0, C.c_void_p(base + self.index[1] * OCTREE_BYTES),
                  C.c_void_p(base + self.index[0] * OCTREE_BYTES), i32(self.index[1]), i32(self.index[0]),
                  self.queue, voxel_size, vol_bbox, i32(self.Dt), i32(self.Db), i32(rate), i32(self.B)])
        torch.cuda.synchronize()

    def node_table(self):
        """Per node id: valid, depth, gindex, batch, xyz index (int3)."""
        raw = self.nodes.cpu().numpy().reshape(-1, OCTREE_BYTES)
        def col(off, dt, n=1):
            return np.frombuffer(raw[:, off:off + 4 * n].tobytes(), dtype=dt).reshape(-1, n)
        return dict(valid=np.frombuffer(raw[:, 0:2].tobytes(), np.uint16).copy(),
                    depth=col(4, np.int32)[:, 0], gindex=col(8, np.int32)[:, 0],
                    nleaves=col(16, np.int32)[:, 0], batch=col(28, np.int32)[:, 0],
                    voxel_size=col(32, np.float32)[:, 0], xyz=col(36, np.int32, 3),
                    centre=col(48, np.float32, 3), corners=col(72, np.float32, 24).reshape(-1, 8, 3),
                    father=col(840, np.int32)[:, 0],
                    children=col(844, np.int32, 64))

    def voxel_traversal(self, ori, dirs, W, th_early_stop=-1, is_training=False, opt_num=-1):
        d = driver()
        vt = self.Dt ** 3
        # bounds guard for the reference's read of octree_nodes[local id]
        local = self.occ1.view(self.B, -1)
        bogus = (local > -1) & ((local < self.index[1]) | (local >= self.index[1] + int(self.queue[0])))
        if bool(bogus.any()) and int(local[bogus].max()) >= self.n_nodes:
            raise RuntimeError("reference traversal would read past the node array")
        assert W >= 4 * self.Dt * (self.rate ** 3 + 1), "hit rows too narrow for a bounded run"
        B, N = ori.shape[0], ori.shape[1]
        o, dr = _dev(ori, torch.float32), _dev(dirs, torch.float32)
        idx = torch.full((B, N, W), -1, dtype=torch.int32, device="cuda")
        t0 = torch.full((B, N, W), -1.0, device="cuda")
        t1 = torch.full((B, N, W), -1.0, device="cuda")
        q = torch.zeros((B, N, 1), dtype=torch.int32, device="cuda")
        vl = torch.zeros((B, N, 1), device="cuda")
        mx = torch.zeros(1, dtype=torch.int32, device="cuda")
        del vt
        d.launch("traversal", B * N, [self.occ1, self.nodes, i32(self.index[1]), o, dr, idx, t0, t1, q, vl,
                                      self.vol_bbox, self.voxel_size, i32(N), i32(W), i32(self.totals[1]),
                                      i32(self.Db), i32(self.Dt), i32(self.B), mx, i32(th_early_stop),
                                      i32(opt_num), cb(True), cb(bool(is_training))])
        torch.cuda.synchronize()
        self.max_hits = int(mx.item())
        return idx, t0, t1, vl, q

    def sample_coarse(self, idx, t0, t1, rands, vl, S, start_level=0):
        d = driver()
        B, N, W = idx.shape
        si = torch.full((B, N, S), -1, dtype=torch.int32, device="cuda")
        sd = torch.full((B, N, S), -1.0, device="cuda")
        if self.max_hits == 0:
            return si, sd
        r = _dev(rands, torch.float32)
        d.launch("sampling", B * N, [self.nodes, idx, t0, t1, r, vl, si, sd, i32(B), i32(N), i32(W), i32(S),
                                     i32(self.max_hits), i32(start_level), i32(2), self.voxel_size])
        torch.cuda.synchronize()
        return si, sd


def trilerp_nodes(tree, ori, dirs, z, idx, feats, gout):
    """trilinear_aggregate_features and its backward (sampling_kernel.cu:
    162-327, host :1384-1462) on the tree's nodes.  Both kernels step
    through the per-sample corner values with the stride MAX_LEAVES = 64
    (octree.h:13) although the host hands them [B, C, N, S, 8] tensors;
    here the values sit in the first 8 entries of [B, C, N, S, 64] blocks, so
    every access stays inside the buffers.  feats [B, C, N, S, 8], gout
    [B, C, N, S] -> (out [B, C, N, S], grad [B, C, N, S, 8])."""
    d = driver()
    o, dr = _dev(ori, torch.float32), _dev(dirs, torch.float32)
    zt, it = _dev(z, torch.float32), _dev(idx, torch.int32)
    f8 = _dev(feats, torch.float32)
    B, C, N, S, _ = f8.shape
    f64 = torch.zeros((B, C, N, S, 64), device="cuda")
    f64[..., :8] = f8
    go = _dev(gout, torch.float32)
    out = torch.zeros((B, C, N, S), device="cuda")
    gd = torch.zeros((B, C, N, S, 64), device="cuda")
    n = B * N * S * C
    d.launch("trilerp_fwd", n, [tree.nodes, o, dr, it, zt, f64, out, i32(B), i32(N), i32(S), i32(C)])
    d.launch("trilerp_bwd", n, [tree.nodes, o, dr, it, zt, go, gd, i32(B), i32(N), i32(S), i32(C)])
    torch.cuda.synchronize()
    return out, gd[..., :8].contiguous()


def merge_levels(occ0, rate, L):
    """build_multi_res_volumes for L levels (octree_kernel.cu:367-411):
    merge_non_empty_nodes level by level."""
    d = driver()
    B = occ0.shape[0]
    vols, cnts = [occ0], []
    for _ in range(L - 1):
        Dn = vols[-1].shape[1]
        Dc = Dn // rate
        occ = torch.full((B, Dc, Dc, Dc), -1, dtype=torch.int32, device="cuda")
        cnt = torch.zeros((B, 1), dtype=torch.int32, device="cuda")
        d.launch("merge", B * Dc ** 3, [occ, cnt, vols[-1], i32(Dc), i32(Dn), i32(B)])
        vols.append(occ)
        cnts.append(cnt)
    torch.cuda.synchronize()
    return vols, cnts


class OctreeML:
    """MultiLayerOctree of any depth (octree_kernel.cu:654-697): node slots
    of level l at octree_nodes_index[l] = the lower levels' occupied counts;
    gen_root_octree_nodes makes the top two levels, gen_higher_octree_nodes
    each level below.  vols [level 0 .. L-1] are rewritten to node ids."""

    def __init__(self, vols, voxel_size, vol_bbox, rate):
        d = driver()
        assert rate ** 3 <= 64, "reference node layout supports rate <= 4 only"
        self.L = L = len(vols)
        self.B = vols[0].shape[0]
        self.dims = [int(v.shape[1]) for v in vols]
        self.rate = rate
        self.totals = [int((v > -1).sum()) for v in vols]
        self.index = [sum(self.totals[:l]) for l in range(L)]
        self.n_nodes = sum(self.totals)
        self.vols = vols
        self.voxel_size, self.vol_bbox = voxel_size, vol_bbox
        self.nodes = torch.zeros(max(self.n_nodes, 1) * OCTREE_BYTES, dtype=torch.uint8, device="cuda")
        self.queue = torch.zeros(L, dtype=torch.int32, device="cuda")
        base = self.nodes.data_ptr()
        T = L - 1
        d.launch("gen_root", self.B * self.dims[T] ** 3,
                 [vols[T], vols[T - 1], C.c_void_p(base + self.index[T] * OCTREE_BYTES),
                  C.c_void_p(base + self.index[T - 1] * OCTREE_BYTES), i32(self.index[T]), i32(self.index[T - 1]),
                  self.queue, voxel_size, vol_bbox, i32(self.dims[T]), i32(self.dims[0]), i32(rate), i32(self.B)])
        for k in range(L - 2, 0, -1):
            d.launch("gen_higher", self.totals[k],
                     [vols[k - 1], C.c_void_p(base + self.index[k] * OCTREE_BYTES),
                      C.c_void_p(base + self.index[k - 1] * OCTREE_BYTES), i32(self.index[k - 1]),
                      i32(self.totals[k]), vol_bbox, C.c_void_p(self.queue.data_ptr() + 4 * (L - k)), i32(rate)])
        torch.cuda.synchronize()
        # queue_control[i] counts the nodes of level L-1-i
        self.built = self.queue.cpu().numpy()[::-1].copy()
        self.complete = bool(np.array_equal(self.built, np.array(self.totals)))

    def node_table(self):
        raw = self.nodes.cpu().numpy().reshape(-1, OCTREE_BYTES)

        def col(off, dt, n=1):
            return np.frombuffer(raw[:, off:off + 4 * n].tobytes(), dtype=dt).reshape(-1, n)
        return dict(valid=np.frombuffer(raw[:, 0:2].tobytes(), np.uint16).copy(), vol_dim=col(24, np.int32)[:, 0],
                    batch=col(28, np.int32)[:, 0], voxel_size=col(32, np.float32)[:, 0],
                    xyz=col(36, np.int32, 3), nleaves=col(16, np.int32)[:, 0])

    def canonical(self, ids, table=None):
        """(level, b, x, y, z) per node id; -1 rows for -1 ids."""
        table = self.node_table() if table is None else table
        ids = np.asarray(ids)
        out = np.full(ids.shape + (5,), -1, np.int32)
        m = ids >= 0
        g = ids[m]
        lvl = np.full(g.shape, -2, np.int32)
        for l, D in enumerate(self.dims):
            lvl[table["vol_dim"][g] == D] = l
        lvl[table["valid"][g] != 1] = -2
        out[m, 0] = lvl
        out[m, 1] = table["batch"][g]
        out[m, 2:] = table["xyz"][g]
        return out

    def octree_traversal(self, ori, dirs, start_level, Wc, Wf):
        """octree_traversal (intersection_kernel.cu:722-826) with
        th_early_stop = opt_num = -1."""
        assert self.complete, "every occupied voxel must be a node"
        d = driver()
        s = self.L - 1 - start_level
        assert Wc >= 4 * self.dims[s] and Wf >= 8 * Wc, "rows narrower than the reference's bounds"
        B, N = ori.shape[0], ori.shape[1]
        o, dr = _dev(ori, torch.float32), _dev(dirs, torch.float32)
        vl = torch.zeros((B, N, 1), device="cuda")
        qc = torch.zeros((B, N, 1), dtype=torch.int32, device="cuda")
        idx_c = torch.full((B, N, Wc), -1, dtype=torch.int32, device="cuda")
        t0c = torch.full((B, N, Wc), -1.0, device="cuda")
        t1c = torch.full((B, N, Wc), -1.0, device="cuda")
        q = torch.zeros((B, N, 1), dtype=torch.int32, device="cuda")
        idx = torch.full((B, N, Wf), -1, dtype=torch.int32, device="cuda")
        t0 = torch.full((B, N, Wf), -1.0, device="cuda")
        t1 = torch.full((B, N, Wf), -1.0, device="cuda")
        mc = torch.zeros(1, dtype=torch.int32, device="cuda")
        mf = torch.zeros(1, dtype=torch.int32, device="cuda")
        d.launch("traversal", B * N, [self.vols[s], self.nodes, i32(self.index[s]), o, dr, idx_c, t0c, t1c, qc, vl,
                                      self.vol_bbox, self.voxel_size, i32(N), i32(Wc), i32(self.totals[s]),
                                      i32(self.dims[0]), i32(self.dims[s]), i32(B), mc, i32(-1), i32(-1), cb(False),
                                      cb(False)])
        torch.cuda.synchronize()
        ncoarse = int(mc.item())
        if ncoarse > 0:
            d.launch("octree_traversal", B * N * ncoarse,
                     [self.nodes, o, dr, idx_c, t0c, t1c, idx, t0, t1, q, vl, i32(N), i32(Wc), i32(Wf), mf,
                      i32(ncoarse), i32(B), i32(self.rate)])
            torch.cuda.synchronize()
        self.max_fine = int(mf.item())
        return dict(idx_c=idx_c, t0_c=t0c, t1_c=t1c, idx=idx, t0=t0, t1=t1, valid_len=vl, cnt=q)

    def sample_fine(self, idx, t0, t1, vl, rands, S, start_level):
        """ray_voxels_points_sampling (sampling_kernel.cu:1178-1248)."""
        d = driver()
        B, N, W = idx.shape
        si = torch.full((B, N, S), -1, dtype=torch.int32, device="cuda")
        sd = torch.full((B, N, S), -1.0, device="cuda")
        sq = torch.zeros((B, N, 1), dtype=torch.int32, device="cuda")
        if self.max_fine == 0:
            return si, sd
        r = _dev(rands, torch.float32)
        d.launch("sampling_fine", B * N * self.max_fine,
                 [self.nodes, idx, t0, t1, r, vl, si, sq, sd, i32(B), i32(N), i32(W), i32(S), i32(self.max_fine),
                  i32(start_level), i32(self.L), self.voxel_size])
        d.launch("sampling_further", B * N, [self.nodes, idx, t0, t1, r, si, sq, sd, i32(B), i32(N), i32(W), i32(S)])
        torch.cuda.synchronize()
        return si, sd


def project_sampled_xyz(tree, ori, dirs, z, idx, K, RT, ori_w, ori_h, record_corners):
    """MultiLayerOctree::project_sampled_xyz (sampling_kernel.cu:1333-1381):
    -1-filled outputs, then project_xyz (:55-159) over B*V*N*S items."""
    d = driver()
    zt, it = _dev(z, torch.float32), _dev(idx, torch.int32)
    B, N, S = zt.shape
    V = np.asarray(K).shape[1]
    shape = (B, V, N, S, 9) if record_corners else (B, V, N, S)
    xy = torch.full(shape + (2,), -1.0, device="cuda")
    pz = torch.full(shape + (1,), -1.0, device="cuda")
    d.launch("project", B * V * N * S, [tree.nodes, _dev(ori, torch.float32), _dev(dirs, torch.float32),
                                        _dev(K, torch.float32), _dev(RT, torch.float32), it, zt, xy, pz,
                                        i32(ori_w), i32(ori_h), i32(B), i32(N), i32(S), i32(V),
                                        cb(bool(record_corners))])
    torch.cuda.synchronize()
    return xy, pz


def sort_samplings(z):
    s, i = torch.sort(z, 2, False)
    return s, i.int()


def volume_rendering_forward(z, sort_idx, sigma, feats, t_thres, occ):
    d = driver()
    B, N, S = z.shape
    of = torch.empty((B, N, 3), device="cuda")
    od, ws, oa = (torch.empty((B, N, 1), device="cuda") for _ in range(3))
    d.launch("vr_occ_fwd" if occ else "vr_fwd", B * N,
             [z, sort_idx, sigma, feats, of, od, ws, oa, u32(B), u32(N), u32(S), f32(t_thres)])
    torch.cuda.synchronize()
    return of, od, ws, oa


def volume_rendering_backward(g, outs, z, sort_idx, sigma, feats, t_thres, occ):
    d = driver()
    B, N, S = z.shape
    gf = torch.zeros((B, N, S, 3), device="cuda")
    gs = torch.zeros((B, N, S, 1), device="cuda")
    d.launch("vr_occ_bwd" if occ else "vr_bwd", B * N,
             [*g, z, sort_idx, sigma, feats, *outs, gf, gs, u32(B), u32(N), u32(S), f32(t_thres)])
    torch.cuda.synchronize()
    return gf, gs


def volume_rendering_occ_forward(z, occ_, feats, t_thres):
    d = driver()
    B, N, S = z.shape
    of = torch.empty((B, N, 3), device="cuda")
    od, ws, oa = (torch.empty((B, N, 1), device="cuda") for _ in range(3))
    d.launch("vr_occ", B * N, [z, occ_, feats, of, od, ws, oa, u32(B), u32(N), u32(S), f32(t_thres)])
    torch.cuda.synchronize()
    return of, od, ws, oa


def rays_calculating(K, R, T, load_size):
    """rays_calculating (sampling_kernel.cu:674-731): inverse_mat3x3 of K and
    R, then rays_calculating_kernel (:411-486) -> [B, N, H, W, 6] (ori, dir)."""
    d = driver()
    B, N = K.shape[0], K.shape[1]
    Kt, Rt, Tt = _dev(K, torch.float32), _dev(R, torch.float32), _dev(np.reshape(T, (B, N, 3)), torch.float32)
    kinv = torch.zeros((B, N, 3, 3), device="cuda")
    rinv = torch.zeros((B, N, 3, 3), device="cuda")
    out = torch.zeros((B, N, load_size, load_size, 6), device="cuda")
    d.launch("rays_inverse", B * N, [Kt, u32(B), u32(N), kinv])
    d.launch("rays_inverse", B * N, [Rt, u32(B), u32(N), rinv])
    d.launch("rays", B * N * load_size * load_size, [kinv, rinv, Tt, out, u32(B), u32(N), u32(load_size),
                                                     u32(load_size)])
    torch.cuda.synchronize()
    return dict(rays=out, Kinv=kinv, Rinv=rinv)


def infer_density_mlp(points_z, points_tpsdf, feats_geo, params, batch_size, num_points, num_views):
    """infer_density_mlp (infer_mlp.cu:583-636): density_feat_kernel over
    the B*V*N point-views, the float32 mean of the 64 density features over
    the views, density_sigma_kernel over the B*N points (256-thread CTAs, as
    the reference launches them).  params: the float16 parameter vector.
    Returns (densities [B, 1, N], geometry features [B, V, N, 8])."""
    from . import fastnerf
    B, N, V = batch_size, num_points, num_views
    nv = B * V * N
    # the reference kernels read mlp_params up to PARAM_COUNT halves and the
    # point inputs by index up to n_points with no bound of their own
    def size(a):
        return a.numel() if isinstance(a, torch.Tensor) else np.size(a)
    if size(params) != fastnerf.PARAM_COUNT:
        raise ValueError(f"params holds {size(params)} float16 values, the network has {fastnerf.PARAM_COUNT}")
    if size(points_z) != nv or size(points_tpsdf) != nv:
        raise ValueError(f"points_z / points_tpsdf must hold B*V*N = {nv} values")
    if size(feats_geo) != nv * 16:
        raise ValueError(f"feats_geo must hold B*V*N x 16 = {nv * 16} values")
    d = driver()
    # device tensors are used in place; host arrays are copied up
    z = _dev(points_z, torch.float32).reshape(-1)
    tp = _dev(points_tpsdf, torch.float32).reshape(-1)
    g = _dev(feats_geo, torch.float32).reshape(-1, 16)
    w = _dev(params if isinstance(params, torch.Tensor) else np.asarray(params, np.float16).reshape(-1),
             torch.float16).reshape(-1)
    dens = torch.empty((nv, 64), device="cuda")
    geo = torch.empty((nv, 8), device="cuda")
    d.launch("nerf_density_feat", nv, [w, z, tp, g, i32(nv), dens, geo], block=256)
    mean = dens.view(B, V, N, 64).mean(1).reshape(B * N, 64).contiguous()
    out = torch.empty((B * N, 1), device="cuda")
    d.launch("nerf_density_sigma", B * N, [w, mean, i32(B * N), out], block=256)
    torch.cuda.synchronize()
    return out.view(B, 1, N), geo.view(B, V, N, 8)
