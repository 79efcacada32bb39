"""Batched fusion, tree build, intersection and render over many frames and
target cameras of uneven sizes, one launch per stage.

``BatchPipeline`` keeps every buffer resident in HBM, sized once for a fixed
layout of frames (views of uneven count and resolution) and target cameras
(uneven ray counts and sample counts).  Each stage is one persistent launch
over all frames / all rays, indexed by segment tables:

* fusion: ``sg_fuse_tsdf_views`` over the view table (per-view image offsets
  and sizes);
* coarse occupancy and tree: ``sg_brick_occupancy`` / ``sg_tree_build`` over
  the frame axis;
* intersection: ``sg_intersect_segments`` (each ray's frame from its target's
  segment); with ``target_widths`` the targets are cameras (``load_cameras``)
  whose rays are generated on the device each step (``sg_camera_params``,
  ``sg_segment_rays``), so no ray crosses from the host;
* render: ``sg_render_segments_fwd`` (per-ray outputs only) and
  ``sg_render_segments_bwd`` (recomputes each ray, exact compositing adjoint,
  gradients scattered into the per-frame feature and TSDF grids).

``train_step`` runs the whole step (build, intersect, forward, an L2 loss
gradient against target colours, backward) with no allocation, so it can be
captured once in a CUDA graph (``capture``) and replayed.

The colour model is a dense per-frame feature grid [B, D, D, D, C] with a
fixed linear head [3, C] (the stand-in for SRONet's MLP); density comes from
the fused TSDF grid.  No reference counterpart as one object: the reference
runs one frame and one target view per call sequence
(SRONet/BasicRenNet.py:170-318).
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N


def sample_capacity(S):
    """Samples per ray of the training kernel that holds S samples (32 per
    lane block: 32, 64 or 128)."""
    return 32 if S <= 32 else (64 if S <= 64 else 128)


def capacity_layout(targets):
    """Ray layout of the targets (frame, n_rays, S), grouped by sample
    capacity so that each group is one launch of the training kernel sized
    for it.  Returns (order, ray_begin, ray_slices, groups): order lists the
    targets in layout order (by capacity, then as given); ray_begin [T + 1]
    the first ray of each target in that order (int64) and the total;
    ray_slices[t] the (begin, end) rays of target t; groups the (first
    segment, end segment, largest S) of each capacity group."""
    T = len(targets)
    order = sorted(range(T), key=lambda t: (sample_capacity(targets[t][2]), t))
    seg_t = [targets[t] for t in order]
    rb = np.concatenate([[0], np.cumsum([n for _, n, _ in seg_t])]).astype(np.int64)
    if rb[-1] >= 2 ** 31:
        raise ValueError("at most 2^31 - 1 rays per launch")
    ray_slices = [None] * T
    for i, t in enumerate(order):
        ray_slices[t] = (int(rb[i]), int(rb[i + 1]))
    groups = []
    for i, (_, _, s_) in enumerate(seg_t):
        if groups and sample_capacity(seg_t[groups[-1][0]][2]) == sample_capacity(s_):
            g0, _, sm = groups[-1]
            groups[-1] = (g0, i + 1, max(sm, s_))
        else:
            groups.append((i, i + 1, s_))
    return order, rb, ray_slices, groups


class BatchPipeline:
    def __init__(self, view_hw, targets, D=256, rate=8, C=16, W_hits=64, train_tsdf=False, target_widths=None,
                 device="cuda", deterministic=True, record_capacity=None):
        """view_hw: per frame, a list of (H, W) per view.  targets: list of
        (frame, n_rays, S).  train_tsdf: train_step also scatters the gradient
        of the TSDF grid (the feature grid is always trained).  target_widths:
        per target the image width in pixels -- the targets are then cameras
        (n_rays = width x height, ray = pixel in row-major order) given by
        load_cameras instead of ray buffers given by load_rays.
        deterministic: train_step reduces the grid gradients by a sort over
        cell ids (sg_render_segments_train_det: bit-identical gradients on
        every run) instead of float atomics (sg_render_segments_train).
        record_capacity: gradient-record slots of that reduction (default:
        the sum of S over all rays, which always suffices)."""
        self.B = B = len(view_hw)
        self.D, self.rate, self.C, self.W = D, rate, C, W_hits
        self.train_tsdf = bool(train_tsdf)
        self.Dt = D // rate
        if self.Dt * rate != D or D % 4:
            raise ValueError("D must be a multiple of rate and of 4")
        self.dev = dev = torch.device(device)
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        # views
        nv = [len(v) for v in view_hw]
        if max(nv) > 32:
            raise ValueError("at most 32 views per frame")
        self.views_hw = [tuple(map(int, hw)) for v in view_hw for hw in v]
        V = len(self.views_hw)
        sizes = [h * w for h, w in self.views_hw]
        offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.view_pix = int(offs[-1])
        self.view_begin = torch.tensor(np.concatenate([[0], np.cumsum(nv)]), **i32)
        self.view_hw_t = torch.tensor(np.array(self.views_hw, np.int32).reshape(-1), **i32)
        self.view_off = torch.tensor(offs[:-1], dtype=torch.int64, device=dev)
        self._view_slices = [(int(offs[k]), int(offs[k + 1])) for k in range(V)]
        self.K = torch.zeros((V, 3, 3), **f32)
        self.RT = torch.zeros((V, 3, 4), **f32)
        self.depth = torch.zeros(self.view_pix, **f32)
        self.color = torch.zeros(self.view_pix, **f32)
        # per-view maps of 8 x 8 depth blocks: fusion culls tiles from them
        nblk = [((h + 7) // 8) * ((w + 7) // 8) for h, w in self.views_hw]
        boffs = np.concatenate([[0], np.cumsum(nblk)]).astype(np.int64)
        self.block_off = torch.tensor(boffs[:-1], dtype=torch.int64, device=dev)
        self.depth_blocks = torch.empty(max(int(boffs[-1]), 1), **f32)
        self.views = N.SgViews(max(nv), N.ptr(self.view_begin), N.ptr(self.view_hw_t), N.ptr(self.view_off),
                               N.ptr(self.K), N.ptr(self.RT), N.ptr(self.depth), N.ptr(self.color),
                               N.ptr(self.block_off), N.ptr(self.depth_blocks))
        # volumes and tree
        Vol, Vt = B * D ** 3, B * self.Dt ** 3
        self.vol_bbox = torch.zeros((B, 3, 2), **f32)
        self.voxel_size = torch.zeros(B, **f32)
        self.tsdf = torch.empty((B, D, D, D), **f32)
        self.weight = torch.empty((B, D, D, D), **f32)
        self.colorv = torch.empty((B, D, D, D), **f32)
        self.occ0 = torch.empty((B, D, D, D), **i32)
        self.occ1 = torch.empty((B, self.Dt, self.Dt, self.Dt), **i32)
        self.cnt = torch.zeros((2, B), **i32)
        mw = N.mask_words(rate)
        self.brick_node = torch.empty(Vt, **i32)
        self.brick_mask = torch.empty(Vt * mw, **i32)
        self.top_key = torch.empty(Vt, **i32)
        self.top_child_base = torch.empty(Vt, **i32)
        self.bot_key = torch.empty(Vol, **i32)
        self.bot_parent = torch.empty(Vol, **i32)
        self.counts = torch.zeros(2, **i32)
        self.brick_box = torch.empty(6 * B, **i32)
        self.scratch = torch.empty(int(N.lib.sg_tree_scratch_bytes(B, self.Dt)), dtype=torch.uint8, device=dev)
        self.status = torch.zeros(4, **i32)
        self.tree = N.SgTree(B, self.Dt, D, rate, Vol, 0, Vt, Vol, N.ptr(self.brick_node), N.ptr(self.brick_mask),
                             N.ptr(self.top_key), N.ptr(self.top_child_base), N.ptr(self.bot_key),
                             N.ptr(self.bot_parent), N.ptr(self.counts), N.ptr(self.voxel_size),
                             N.ptr(self.vol_bbox), N.ptr(self.brick_box))
        # rays and segments.  Targets are laid out grouped by the sample
        # capacity their S needs (32, 64 or 128 samples per ray), so each
        # group is one launch of the training kernel sized for it;
        # ray_slices[t] are the rays of target t in that layout, and the
        # segment tables list targets in the order self.order.
        self.targets = [(int(f), int(n), int(s)) for f, n, s in targets]
        T = len(self.targets)
        self.order, rb, self.ray_slices, self._groups = capacity_layout(self.targets)
        seg_t = [self.targets[t] for t in self.order]
        self.R = R = int(rb[-1])
        self.S = S = max(s for _, _, s in self.targets)
        self.seg_begin = torch.tensor(rb.astype(np.int32), **i32)
        self.seg_frame = torch.tensor([f for f, _, _ in seg_t], **i32)
        self.seg_samples = torch.tensor([s_ for _, _, s_ in seg_t], **i32)
        self.cameras = target_widths is not None
        if self.cameras:
            if len(target_widths) != T or any(n % int(w) for (_, n, _), w in zip(self.targets, target_widths)):
                raise ValueError("one width per target, dividing its ray count")
            self.tK = torch.zeros((T, 3, 3), **f32)
            self.tR = torch.zeros((T, 3, 3), **f32)
            self.tT = torch.zeros((T, 3), **f32)
            self.cams = torch.zeros((T, 21), **f32)
            self.cam_w = torch.tensor([int(target_widths[t]) for t in self.order], **i32)
            self.cam_seg = N.SgRaySegments(T, R, N.ptr(self.seg_begin), N.ptr(self.seg_frame),
                                           N.ptr(self.seg_samples), N.ptr(self.cams), N.ptr(self.cam_w))
        else:
            self.cams = self.cam_w = self.cam_seg = None
        # ray buffers: loaded (load_rays), or written from the cameras once per
        # step (sg_segment_rays) -- cheaper than generating each ray inside the
        # warp-per-ray render kernels
        self.ori = torch.zeros((R, 3), **f32)
        self.dirs = torch.zeros((R, 3), **f32)
        self.seg = N.SgRaySegments(T, R, N.ptr(self.seg_begin), N.ptr(self.seg_frame), N.ptr(self.seg_samples))
        self.hit_idx = torch.empty((R, W_hits), **i32)
        self.hit_t0 = torch.empty((R, W_hits), **f32)
        self.hit_t1 = torch.empty((R, W_hits), **f32)
        self.hit_count = torch.empty(R, **i32)
        self.valid_len = torch.empty(R, **f32)
        # fields, outputs, gradients
        self.feat = torch.zeros((B, D, D, D, C), **f32)
        self.head = torch.zeros((3, C), **f32)
        self.grad_feat = torch.zeros((B, D, D, D, C), **f32)
        self.grad_tsdf = torch.zeros((B, D, D, D), **f32)
        # brick map of the tree the gradients were last accumulated over (-1:
        # none): outside its nodes' bricks and their neighbours the gradient
        # grids are 0, so train_step clears only those (sg_zero_near_nodes)
        self.grad_bricks = torch.full((Vt,), -1, **i32)
        self.grad_tree = N.SgTree(B, self.Dt, D, rate, Vol, 0, Vt, Vol, N.ptr(self.grad_bricks), None, None, None,
                                  None, None, None, N.ptr(self.voxel_size), N.ptr(self.vol_bbox))
        self.out_rgb = torch.empty((R, 3), **f32)
        self.out_depth = torch.empty(R, **f32)
        self.out_ws = torch.empty(R, **f32)
        self.out_alpha = torch.empty(R, **f32)
        self.target_rgb = torch.zeros((R, 3), **f32)
        self.g_rgb = torch.empty((R, 3), **f32)
        self.out_loss = torch.empty(R, **f32)
        # workspace of the deterministic gradient reduction
        self.deterministic = bool(deterministic)
        self.record_capacity = int(record_capacity if record_capacity is not None
                                   else sum(n * s_ for _, n, s_ in self.targets))
        self.det_ws = None
        if self.deterministic:
            nbytes = int(N.lib.sg_train_det_workspace_bytes(R, T, C, self.record_capacity))
            self.det_ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self.args = None
        self.trunc_weight = None
        self.events = None
        self.side_events = None
        self.side = torch.cuda.Stream(device=dev)  # zeroing of the gradient grids beside fusion
        self._feed = None  # copy stream, staging buffers and events of train_steps_from_host

    # ------------------------------------------------------------------ inputs
    def load_views(self, frames, vol_bbox, voxel_size, trunc_weight):
        """frames: per frame dict(K, RT, depth, color) lists of per-view arrays
        in the layout given to the constructor."""
        k = 0
        for fr in frames:
            for v in range(len(fr["K"])):
                a, b = self._view_slices[k]
                h, w = self.views_hw[k]
                if fr["depth"][v].shape != (h, w):
                    raise ValueError("view resolution differs from the layout")
                self.K[k].copy_(torch.as_tensor(fr["K"][v]))
                self.RT[k].copy_(torch.as_tensor(fr["RT"][v]))
                self.depth[a:b].copy_(torch.as_tensor(fr["depth"][v]).reshape(-1))
                self.color[a:b].copy_(torch.as_tensor(fr["color"][v]).reshape(-1))
                k += 1
        self.vol_bbox.copy_(torch.as_tensor(vol_bbox))
        self.voxel_size.copy_(torch.as_tensor(voxel_size).reshape(-1))
        self.trunc_weight = float(trunc_weight)

    def load_rays(self, rays):
        """rays: per target (ori [n,3], dir [n,3])."""
        if self.cameras:
            raise RuntimeError("this pipeline takes target cameras (load_cameras)")
        for (a, b), (o, d) in zip(self.ray_slices, rays):
            self.ori[a:b].copy_(torch.as_tensor(o))
            self.dirs[a:b].copy_(torch.as_tensor(d))

    def load_cameras(self, K, R, T):
        """Target cameras (K [T,3,3], R [T,3,3], T [T,3]); rays follow
        rays_calculating (origin -R^-1 T, direction R^-1 K^-1 [w, h, 1])."""
        if not self.cameras:
            raise RuntimeError("this pipeline takes ray buffers (load_rays)")
        perm = self.order  # the segment tables' target order
        self.tK.copy_(torch.as_tensor(np.asarray(K, np.float32).reshape(self.tK.shape)[perm]))
        self.tR.copy_(torch.as_tensor(np.asarray(R, np.float32).reshape(self.tR.shape)[perm]))
        self.tT.copy_(torch.as_tensor(np.asarray(T, np.float32).reshape(self.tT.shape)[perm]))

    def set_fields(self, feat=None, head=None, target_rgb=None):
        if feat is not None:
            self.feat.copy_(feat)
        if head is not None:
            self.head.copy_(head)
        if target_rgb is not None:
            self.target_rgb.copy_(target_rgb)

    def render_args(self, trunc_metres, sdf_s=0.005, t_thres=1e-4, rand_seed=0, rand_const=0.5):
        """Fix the render's scalar parameters (trunc_metres: the truncation
        margin in metres; sdf_s: the density's length scale)."""
        def args(S):
            return N.SgRenderArgs(
                N.ptr(self.ori), N.ptr(self.dirs), N.ptr(self.hit_idx), N.ptr(self.hit_t0), N.ptr(self.hit_t1),
                N.ptr(self.hit_count), N.ptr(self.valid_len), self.W, S, None, float(rand_const),
                int(rand_seed), N.ptr(self.tsdf), self.D, float(trunc_metres), float(sdf_s), N.ptr(self.feat),
                self.D, self.C, N.ptr(self.vol_bbox), N.ptr(self.voxel_size),
                N.ptr(self.head) if self.C != 3 else None, float(t_thres))

        self.args = args(self.S)
        # one (segment sub-table, arguments) per capacity group: the training
        # pass runs each group through the kernel sized for its largest S
        rb = self.seg_begin.cpu().numpy()
        self._group_launch = []
        for g0, g1, sm in self._groups:
            seg = N.SgRaySegments(g1 - g0, int(rb[g1]), self.seg_begin.data_ptr() + 4 * g0,
                                  self.seg_frame.data_ptr() + 4 * g0, self.seg_samples.data_ptr() + 4 * g0)
            self._group_launch.append((seg, args(sm)))
        ng = len(self._groups)
        self._det_groups = (C.c_int * (ng + 1))(*([g0 for g0, _, _ in self._groups] + [len(self.targets)]))
        self._det_group_S = (C.c_int * ng)(*[sm for _, _, sm in self._groups])
        return self.args

    def _mark(self, name):
        if self.events is not None:
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            self.events.append((name, ev))

    def _side_event(self):
        if self.events is None:
            return None
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        return ev

    # ------------------------------------------------------------------ stages
    def build(self, obs_weight=1.0, th_low=13.5, th_high=13.5, before_tree=None):
        st = N.stream()
        self.cnt.zero_()
        self.status.zero_()
        self._mark("start")
        N.check(N.lib.sg_fuse_tsdf_views(C.byref(self.views), self.B, self.D, N.ptr(self.vol_bbox),
                                         N.ptr(self.voxel_size), float(obs_weight), self.trunc_weight,
                                         float(th_low), float(th_high), N.ptr(self.tsdf), N.ptr(self.weight),
                                         N.ptr(self.colorv), N.ptr(self.occ0), N.ptr(self.cnt[0]), st),
                "fuse_tsdf_views")
        self._mark("fusion")
        if before_tree is not None:
            before_tree()
        N.check(N.lib.sg_brick_occupancy(N.ptr(self.occ0), self.B, self.D, self.rate, N.ptr(self.occ1),
                                         N.ptr(self.cnt[1]), st), "brick_occupancy")
        N.check(N.lib.sg_tree_build(C.byref(self.tree), N.ptr(self.occ1), N.ptr(self.occ0), N.ptr(self.scratch),
                                    self.scratch.numel(), N.ptr(self.status), st), "tree_build")
        self._mark("tree")

    def intersect(self):
        if self.cameras:
            N.check(N.lib.sg_camera_params(N.ptr(self.tK), N.ptr(self.tR), N.ptr(self.tT), len(self.targets),
                                           N.ptr(self.cams), N.stream()), "camera_params")
            N.check(N.lib.sg_segment_rays(C.byref(self.cam_seg), N.ptr(self.ori), N.ptr(self.dirs), N.stream()),
                    "segment_rays")
        N.check(N.lib.sg_intersect_segments(C.byref(self.tree), C.byref(self.seg), N.ptr(self.ori),
                                            N.ptr(self.dirs), self.W, N.ptr(self.hit_idx), N.ptr(self.hit_t0),
                                            N.ptr(self.hit_t1), N.ptr(self.valid_len), N.ptr(self.hit_count),
                                            N.ptr(self.status), N.stream()), "intersect_segments")
        self._mark("intersect")

    def forward(self, out_z=None, out_node=None):
        N.check(N.lib.sg_render_segments_fwd(C.byref(self.tree), C.byref(self.seg), C.byref(self.args),
                                             N.ptr(self.out_rgb), N.ptr(self.out_depth), N.ptr(self.out_ws),
                                             N.ptr(self.out_alpha), N.ptr(out_z), N.ptr(out_node), N.stream()),
                "render_fwd")
        self._mark("forward")
        return self.out_rgb, self.out_depth, self.out_ws, self.out_alpha

    def backward(self, g_rgb=None, g_depth=None, g_ws=None, g_alpha=None, grad_sigma=None, grad_rgb=None,
                 tsdf_grad=True, zero=True):
        if zero:
            self.grad_feat.zero_()
            self.grad_tsdf.zero_()  # both, so one brick map describes both grids
        self._mark("grad_prep")
        N.check(N.lib.sg_render_segments_bwd(C.byref(self.tree), C.byref(self.seg), C.byref(self.args),
                                             N.ptr(g_rgb), N.ptr(g_depth), N.ptr(g_ws), N.ptr(g_alpha),
                                             N.ptr(self.grad_feat), N.ptr(self.grad_tsdf) if tsdf_grad else None,
                                             N.ptr(grad_sigma), N.ptr(grad_rgb), N.stream()), "render_bwd")
        self._mark("backward")
        if zero:
            self.grad_bricks.copy_(self.brick_node)
        else:
            self.grad_bricks.fill_(0)  # unknown region: the next train_step clears everything

    def train_step(self):
        """Build, intersect, then one fused pass per ray: forward, the mean
        squared colour error against target_rgb (per-ray terms in out_loss)
        and its backward into grad_feat (and grad_tsdf when train_tsdf).
        Allocates nothing.  The gradient grids are owned by the pipeline:
        read them, do not write them (zero_grads() after writing).  Before
        accumulating, train_step clears only the bricks the previous
        gradient pass could reach (sg_zero_near_nodes over its brick map),
        on a side stream beside fusion; the tree build waits for it, as it
        rewrites the brick map the clear reads."""
        main = torch.cuda.current_stream()
        self.side.wait_stream(main)  # the previous step's users of the grids come first
        with torch.cuda.stream(self.side):
            z0 = self._side_event()
            N.check(N.lib.sg_zero_near_nodes(C.byref(self.grad_tree), N.ptr(self.grad_feat), self.C, N.stream()),
                    "zero_near_nodes")
            if self.train_tsdf:
                N.check(N.lib.sg_zero_near_nodes(C.byref(self.grad_tree), N.ptr(self.grad_tsdf), 1, N.stream()),
                        "zero_near_nodes")
            if z0 is not None:
                self.side_events = (z0, self._side_event())
        self.build(before_tree=lambda: main.wait_stream(self.side))
        self.intersect()
        self._mark("grad_prep")
        loss_scale = 2.0 / (3.0 * self.R)
        tsdf = N.ptr(self.grad_tsdf) if self.train_tsdf else None
        if self.deterministic:
            N.check(N.lib.sg_render_segments_train_det(
                C.byref(self.tree), C.byref(self.seg), C.byref(self.args), len(self._groups), self._det_groups,
                self._det_group_S, N.ptr(self.target_rgb), loss_scale, N.ptr(self.out_rgb), N.ptr(self.out_depth),
                N.ptr(self.out_ws), N.ptr(self.out_alpha), N.ptr(self.out_loss), N.ptr(self.grad_feat), tsdf,
                N.ptr(self.det_ws), self.det_ws.numel(), self.record_capacity, N.ptr(self.status), N.stream()),
                "render_train_det")
        else:
            for seg, args in self._group_launch:
                N.check(N.lib.sg_render_segments_train(
                    C.byref(self.tree), C.byref(seg), C.byref(args), N.ptr(self.target_rgb), loss_scale,
                    N.ptr(self.out_rgb), N.ptr(self.out_depth), N.ptr(self.out_ws), N.ptr(self.out_alpha),
                    N.ptr(self.out_loss), N.ptr(self.grad_feat), tsdf, N.stream()), "render_train")
        self.grad_bricks.copy_(self.brick_node)
        self._mark("train")

    def reduction_sizes(self):
        """Sizes of the last deterministic gradient reduction (synchronizes):
        rays with hits, record slots needed and used, records with a cell,
        distinct cells summed."""
        if self.det_ws is None:
            raise RuntimeError("the pipeline reduces gradients with atomics (deterministic=False)")
        c = self.det_ws[:4 * N.SG_DET_COUNTERS].view(torch.int32).tolist()
        return dict(rays_with_hits=c[N.SG_DET_RAYS_WITH_HITS], slots_needed=c[N.SG_DET_SLOTS_NEEDED],
                    slots=c[N.SG_DET_SLOTS], records=c[N.SG_DET_RECORDS], cells=c[N.SG_DET_CELLS])

    def zero_grads(self):
        """Clear the gradient grids entirely (after writing into them)."""
        self.grad_feat.zero_()
        self.grad_tsdf.zero_()
        self.grad_bricks.fill_(-1)

    def train_step_unfused(self):
        """The same step with separate forward and backward launches (the
        backward recomputes each ray) and the loss gradient formed between
        them."""
        self.build()
        self.intersect()
        self.forward()
        torch.sub(self.out_rgb, self.target_rgb, out=self.g_rgb)
        self.g_rgb.mul_(2.0 / (3.0 * self.R))
        self.backward(self.g_rgb, tsdf_grad=self.train_tsdf)

    def capture(self, warmup=2):
        """CUDA graph of train_step (run it a few times first, then capture)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(warmup):
                self.train_step()
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.train_step()
        return g

    # step inputs a host may feed, and step outputs it may read back
    HOST_INPUTS = ("depth", "color", "K", "RT", "tK", "tR", "tT", "ori", "dirs", "target_rgb")
    HOST_OUTPUTS = ("out_rgb", "out_depth", "out_ws", "out_alpha", "out_loss")

    def train_steps_from_host(self, batches, graph=None):
        """Training steps fed from host memory, with the copies overlapped.

        batches: iterable of (inputs, outputs) per step; inputs maps names of
        HOST_INPUTS to pinned host tensors holding that step's values (the
        shape and dtype of the pipeline's buffer of that name; tK / tR / tT in
        the segment order, ``order``), outputs maps names of HOST_OUTPUTS to
        pinned host tensors that receive the step's results.  graph: a
        ``capture`` of this pipeline's train_step (else train_step runs).

        Step i+1's inputs are copied into device staging buffers on a copy
        stream while step i runs, then into the pipeline's buffers (a device
        copy) when step i+1 starts; step i's outputs go to staging buffers
        when it ends and reach the host while step i+1 runs.  Every step's
        inputs and outputs cross the link; the steps' results equal those of
        copy-in, train_step, copy-out in sequence.  Returns on the host at
        once: the outputs are complete when the current stream reaches the
        end of the enqueued work (synchronize before reading them)."""
        main = torch.cuda.current_stream(self.dev)
        if self._feed is None:
            self._feed = dict(stream=torch.cuda.Stream(device=self.dev), stage={},
                              ev={k: torch.cuda.Event() for k in ("in_ready", "in_free", "out_ready", "out_free")})
        f = self._feed
        cps, ev, stage = f["stream"], f["ev"], f["stage"]

        def checked(allowed, tensors):
            for k, t in tensors.items():
                if k not in allowed:
                    raise ValueError(f"{k}: not one of {allowed}")
                if k in (("ori", "dirs") if self.cameras else ("tK", "tR", "tT")):
                    raise ValueError(f"{k}: not an input of this pipeline (its targets are "
                                     f"{'cameras' if self.cameras else 'ray buffers'})")
                buf = getattr(self, k, None)
                if buf is None:
                    raise ValueError(f"{k}: this pipeline has no such buffer")
                if t.device.type != "cpu" or not t.is_pinned():
                    raise ValueError(f"{k}: host tensors must be pinned CPU tensors")
                if t.shape != buf.shape or t.dtype != buf.dtype or not t.is_contiguous():
                    raise ValueError(f"{k}: expected a contiguous {tuple(buf.shape)} {buf.dtype} tensor")
                if k not in stage:
                    stage[k] = torch.empty_like(buf)
            return tensors

        def upload(inputs):
            with torch.cuda.stream(cps):
                cps.wait_event(ev["in_free"])  # the previous step has taken its inputs
                for k, t in inputs.items():
                    stage[k].copy_(t, non_blocking=True)
                ev["in_ready"].record(cps)

        it = iter(batches)
        cur = next(it, None)
        if cur is None:
            return
        checked(self.HOST_INPUTS, cur[0])
        checked(self.HOST_OUTPUTS, cur[1])
        cps.wait_stream(main)
        upload(cur[0])
        while cur is not None:
            nxt = next(it, None)
            if nxt is not None:
                checked(self.HOST_INPUTS, nxt[0])
                checked(self.HOST_OUTPUTS, nxt[1])
            main.wait_event(ev["in_ready"])
            for k in cur[0]:
                getattr(self, k).copy_(stage[k], non_blocking=True)
            ev["in_free"].record(main)
            if nxt is not None:
                upload(nxt[0])
            if graph is not None:
                graph.replay()
            else:
                self.train_step()
            main.wait_event(ev["out_free"])  # the previous step's outputs have left
            for k in cur[1]:
                stage[k].copy_(getattr(self, k), non_blocking=True)
            ev["out_ready"].record(main)
            with torch.cuda.stream(cps):
                cps.wait_event(ev["out_ready"])
                for k, t in cur[1].items():
                    t.copy_(stage[k], non_blocking=True)
                ev["out_free"].record(cps)
            cur = nxt
        main.wait_stream(cps)

    def stage_times(self):
        torch.cuda.synchronize()
        out = {}
        prev = None
        for name, ev in self.events or []:
            if prev is not None:
                out[name] = out.get(name, 0.0) + prev.elapsed_time(ev)
            prev = ev
        if self.events and self.side_events is not None:
            # zeroing of the gradient grids, timed on the side stream where it
            # overlaps fusion, tree build and intersection
            out["zero_grad"] = self.side_events[0].elapsed_time(self.side_events[1])
        self.side_events = None
        return out

    def frame_rays(self, t):
        a, b = self.ray_slices[t]
        return slice(a, b)
