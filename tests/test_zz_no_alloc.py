"""sg_tree_build_static (the tree build that allocates nothing) against
sg_tree_build (caller-provided scratch), both called through the C ABI.

Two builds in a row on different scenes and sizes go through the shared
static scratch array; each must give the same node tables, brick map,
masks, counts and rewritten occupancy volumes as the scratch-buffer entry
point (integer outputs: bit-exact).  A top grid whose scratch would exceed
SG_TREE_STATIC_SCRATCH_BYTES is rejected with SG_ERR_CAPACITY.
"""
import ctypes as C

import pytest
import torch

from sailor_gb300 import _native as N
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

STATIC_SCRATCH_BYTES = 8 << 20  # SG_TREE_STATIC_SCRATCH_BYTES
SG_ERR_CAPACITY = 3


def _t(a, dt=torch.float32):
    return torch.as_tensor(a, dtype=dt, device="cuda").contiguous()


def _volumes(seed, batch, D, rate):
    """Fused fine occupancy and coarse occupancy of a seeded scene."""
    sc = syn.make_scene(seed=seed, n_views=4, res=256, n_prims=10, D=D, trunc=0.03, batch=batch)
    B, Dt = batch, D // rate
    f32 = dict(dtype=torch.float32, device="cuda")
    tsdf, weight, color = (torch.empty((B, D, D, D), **f32) for _ in range(3))
    occ0 = torch.empty((B, D, D, D), dtype=torch.int32, device="cuda")
    occ1 = torch.empty((B, Dt, Dt, Dt), dtype=torch.int32, device="cuda")
    cnt = torch.zeros((2, B), dtype=torch.int32, device="cuda")
    vol_bbox, voxel_size = _t(sc["vol_bbox"]), _t(sc["voxel_size"])
    st = N.stream()
    Nv, H, W = sc["depths"].shape[1:]
    K, RT, colors, depths = (_t(sc[k]) for k in ("K", "RT", "colors", "depths"))  # held until the sync below
    N.check(N.lib.sg_fuse_tsdf(N.ptr(K), N.ptr(RT), N.ptr(colors),
                               N.ptr(depths), B, Nv, H, W, D, D, D, N.ptr(vol_bbox), N.ptr(voxel_size),
                               1.0, float(sc["trunc_weight"]), 13.5, 13.5, N.ptr(tsdf), N.ptr(weight),
                               N.ptr(color), N.ptr(occ0), N.ptr(cnt[0]), st), "fuse_tsdf")
    N.check(N.lib.sg_brick_occupancy(N.ptr(occ0), B, D, rate, N.ptr(occ1), N.ptr(cnt[1]), st), "brick_occupancy")
    torch.cuda.synchronize()
    assert int(cnt[1].sum()) > 0
    return occ0, occ1, vol_bbox, voxel_size


def _tree_buffers(B, D, rate, vol_bbox, voxel_size):
    """Output tables of one build, pre-filled with a sentinel so unwritten
    entries compare too."""
    Dt = D // rate
    V, Vt = B * D ** 3, B * Dt ** 3
    mw = N.mask_words(rate)
    i32 = dict(dtype=torch.int32, device="cuda")
    buf = dict(brick_node=torch.full((Vt,), -7, **i32), brick_mask=torch.full((Vt * mw,), -7, **i32),
               top_key=torch.full((Vt,), -7, **i32), top_child_base=torch.full((Vt,), -7, **i32),
               bot_key=torch.full((V,), -7, **i32), bot_parent=torch.full((V,), -7, **i32),
               counts=torch.full((2,), -7, **i32), status=torch.zeros(4, **i32))
    tree = N.SgTree(B, Dt, D, rate, V, 0, Vt, V, N.ptr(buf["brick_node"]), N.ptr(buf["brick_mask"]),
                    N.ptr(buf["top_key"]), N.ptr(buf["top_child_base"]), N.ptr(buf["bot_key"]),
                    N.ptr(buf["bot_parent"]), N.ptr(buf["counts"]), N.ptr(voxel_size), N.ptr(vol_bbox))
    return tree, buf


def _build_both(seed, batch, D, rate):
    occ0, occ1, vol_bbox, voxel_size = _volumes(seed, batch, D, rate)
    Dt = D // rate
    st = N.stream()
    # existing entry point, scratch from the caller
    ref_tree, ref = _tree_buffers(batch, D, rate, vol_bbox, voxel_size)
    ref["occ_top"], ref["occ_bot"] = occ1.clone(), occ0.clone()
    scratch = torch.empty(int(N.lib.sg_tree_scratch_bytes(batch, Dt)), dtype=torch.uint8, device="cuda")
    N.check(N.lib.sg_tree_build(C.byref(ref_tree), N.ptr(ref["occ_top"]), N.ptr(ref["occ_bot"]), N.ptr(scratch),
                                scratch.numel(), N.ptr(ref["status"]), st), "tree_build")
    # no-allocation entry point, scratch from the library's static array
    new_tree, new = _tree_buffers(batch, D, rate, vol_bbox, voxel_size)
    new["occ_top"], new["occ_bot"] = occ1.clone(), occ0.clone()
    N.check(N.lib.sg_tree_build_static(C.byref(new_tree), N.ptr(new["occ_top"]), N.ptr(new["occ_bot"]),
                                       N.ptr(new["status"]), st), "tree_build_static")
    torch.cuda.synchronize()
    return ref, new


def test_static_tree_build_matches_scratch_build_two_calls():
    # call 1: two frames, 128^3, 4^3 bricks (Dt 32, 65536 bricks);
    # call 2: one frame, 128^3, 8^3 bricks (Dt 16, 4096 bricks) -- smaller, so
    # stale scratch from call 1 past its end would show up as a mismatch
    for seed, batch, D, rate in ((3, 2, 128, 4), (11, 1, 128, 8)):
        ref, new = _build_both(seed, batch, D, rate)
        assert int(ref["counts"][0]) > 0 and int(ref["counts"][1]) > 0
        assert int(new["status"][0]) == int(ref["status"][0]) == 0
        for k in ("counts", "brick_node", "brick_mask", "top_key", "top_child_base", "bot_key", "bot_parent",
                  "occ_top", "occ_bot"):
            assert torch.equal(new[k], ref[k]), f"{k} differs (seed {seed}, B {batch}, D {D}, rate {rate})"


def test_static_tree_build_rejects_oversize():
    # 128^3 top bricks need 16 MiB of scratch > 8 MiB.  The buffers are real
    # and full-size (all -1), so the call would stay in bounds even if it ran.
    B, Dt, rate = 1, 128, 2
    D = Dt * rate
    assert N.lib.sg_tree_scratch_bytes(B, Dt) > STATIC_SCRATCH_BYTES
    vol_bbox = _t([[[-1.0, 1.0]] * 3])
    voxel_size = _t([[2.0 / (D - 1)]])
    tree, buf = _tree_buffers(B, D, rate, vol_bbox, voxel_size)
    occ_top = torch.full((B, Dt, Dt, Dt), -1, dtype=torch.int32, device="cuda")
    occ_bot = torch.full((B, D, D, D), -1, dtype=torch.int32, device="cuda")
    rc = N.lib.sg_tree_build_static(C.byref(tree), N.ptr(occ_top), N.ptr(occ_bot), N.ptr(buf["status"]),
                                    N.stream())
    torch.cuda.synchronize()
    assert rc == SG_ERR_CAPACITY
    assert int(buf["counts"][0]) == -7  # nothing launched
