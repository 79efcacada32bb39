"""Seeded synthetic RGBD workloads for the VoxelEncoding path.

No public dataset is used by the reference for this path, so every workload
is generated: a union of capsules and ellipsoids inside a 2 m cube centred
at the origin, seen by pinhole cameras on a circle of radius 2.5 m at height
1.2 m that look at the origin.  Depth is ray-cast analytically in float64,
perturbed by N(0, 5 mm) noise and 2 % dropout to 0, and quantised to uint16
millimetre/10 units (metres x 10000, the reference's depth PNG format) before
conversion to float32 metres.  Colours are uniform uint8 noise packed as
b*65536 + g*256 + r (the packing of the reference's integrate_depths
preprocessing).

Camera convention (the reference's): x_cam = R x_world + T, pixel =
K x_cam / z_cam with the full 3x3 K, depth maps hold z_cam.  Rays follow
rays_calculating: origin -R^-1 T, direction normalise(R^-1 K^-1 [u, v, 1]).
"""
import math

import numpy as np


def look_at(cam_pos, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0)):
    """World->camera rotation R and translation T (OpenCV axes)."""
    c = np.asarray(cam_pos, np.float64)
    f = np.asarray(target, np.float64) - c
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    R = np.stack([r, d, f])
    T = -R @ c
    return R, T


def ring_cameras(n, radius=2.5, height=1.2, phase=0.0):
    out = []
    for k in range(n):
        a = phase + 2.0 * math.pi * k / n
        out.append(look_at((radius * math.cos(a), radius * math.sin(a), height)))
    return out


def intrinsics(res, f_at_512=550.0):
    f = f_at_512 * res / 512.0
    return np.array([[f, 0.0, res / 2.0], [0.0, f, res / 2.0], [0.0, 0.0, 1.0]])


def random_primitives(rng, n):
    prims = []
    for _ in range(n):
        kind = "capsule" if rng.random() < 0.5 else "ellipsoid"
        c = rng.uniform(-0.45, 0.45, 3)
        if kind == "capsule":
            axis = rng.normal(size=3)
            axis /= np.linalg.norm(axis)
            half = rng.uniform(0.05, 0.30)
            r = rng.uniform(0.05, 0.25)
            prims.append(("capsule", c - half * axis, c + half * axis, r))
        else:
            radii = rng.uniform(0.05, 0.25, 3)
            q = rng.normal(size=(3, 3))
            Q, _ = np.linalg.qr(q)
            prims.append(("ellipsoid", c, radii, Q))
    return prims


def _hit_sphere(o, d, c, r):
    oc = o - c
    b = np.einsum("ij,ij->i", oc, d)
    cc = np.einsum("ij,ij->i", oc, oc) - r * r
    a = np.einsum("ij,ij->i", d, d)
    disc = b * b - a * cc
    t = np.full(o.shape[0], np.inf)
    ok = disc >= 0
    s = np.sqrt(np.where(ok, disc, 0.0))
    t0 = (-b - s) / a
    t1 = (-b + s) / a
    tt = np.where(t0 > 1e-6, t0, np.where(t1 > 1e-6, t1, np.inf))
    t[ok] = tt[ok]
    return t


def _hit_capsule(o, d, a, b, r):
    ba = b - a
    oa = o - a
    baba = ba @ ba
    bard = d @ ba
    baoa = oa @ ba
    rdoa = np.einsum("ij,ij->i", d, oa)
    oaoa = np.einsum("ij,ij->i", oa, oa)
    dd = np.einsum("ij,ij->i", d, d)
    A = baba * dd - bard * bard
    Bq = baba * rdoa - baoa * bard
    Cq = baba * oaoa - baoa * baoa - r * r * baba
    h = Bq * Bq - A * Cq
    t = np.full(o.shape[0], np.inf)
    ok = (h >= 0) & (np.abs(A) > 1e-12)
    tb = np.where(ok, (-Bq - np.sqrt(np.where(ok, h, 0.0))) / np.where(ok, A, 1.0), np.inf)
    y = baoa + tb * bard
    body = ok & (y > 0) & (y < baba) & (tb > 1e-6)
    t[body] = tb[body]
    caps = np.minimum(_hit_sphere(o, d, a, r), _hit_sphere(o, d, b, r))
    return np.where(body, t, np.minimum(t, caps))


def _hit_ellipsoid(o, d, c, radii, Q):
    ol = (o - c) @ Q / radii
    dl = d @ Q / radii
    return _hit_sphere(ol, dl, np.zeros(3), 1.0)


def cast_depth(prims, K, R, T, res):
    """z-depth image (float64, 0 = miss) of the union of primitives."""
    v, u = np.mgrid[0:res, 0:res].astype(np.float64)
    pix = np.stack([u.ravel(), v.ravel(), np.ones(res * res)], 1)
    dcam = pix @ np.linalg.inv(K).T            # z component == 1
    dw = dcam @ R                              # R^T dcam
    ow = np.broadcast_to(-R.T @ T, dw.shape)
    t = np.full(dw.shape[0], np.inf)
    o0 = -R.T @ T
    dn = np.sqrt(np.einsum("ij,ij->i", dw, dw))
    for p in prims:
        # only rays that pass the primitive's bounding sphere can hit it
        if p[0] == "capsule":
            c, rb = 0.5 * (p[1] + p[2]), 0.5 * np.linalg.norm(p[2] - p[1]) + p[3]
        else:
            c, rb = p[1], float(np.max(p[2]))
        oc = c - o0
        cr = np.cross(dw, oc)
        near = np.sqrt(np.einsum("ij,ij->i", cr, cr)) <= (rb * 1.001 + 1e-6) * dn
        if not near.any():
            continue
        sel = np.nonzero(near)[0]
        if p[0] == "capsule":
            th = _hit_capsule(ow[sel], dw[sel], p[1], p[2], p[3])
        else:
            th = _hit_ellipsoid(ow[sel], dw[sel], p[1], p[2], p[3])
        t[sel] = np.minimum(t[sel], th)
    z = np.where(np.isfinite(t), t, 0.0)       # dcam.z == 1, so t is z-depth
    return z.reshape(res, res)


def make_scene(seed=0, n_views=4, res=512, n_prims=12, D=256, trunc=0.03,
               noise=0.005, dropout=0.02, batch=1):
    """Inputs of integrate_depths for `batch` frames (one scene per frame)."""
    Ks, RTs, depths, colors = [], [], [], []
    for b in range(batch):
        rng = np.random.default_rng(seed * 1000 + b)
        prims = random_primitives(rng, n_prims)
        cams = ring_cameras(n_views, phase=rng.uniform(0, 2 * math.pi))
        K = intrinsics(res)
        for R, T in cams:
            z = cast_depth(prims, K, R, T, res)
            hit = z > 0
            z = z + rng.normal(0.0, noise, z.shape) * hit
            z[rng.random(z.shape) < dropout] = 0.0
            u16 = np.clip(np.round(z * 10000.0), 0, 65535).astype(np.uint16)
            depths.append((u16 / 10000.0).astype(np.float32))
            rgb = rng.integers(0, 256, (res, res, 3))
            colors.append(np.floor(rgb[..., 2] * 65536.0 + rgb[..., 1] * 256.0 + rgb[..., 0]).astype(np.float32))
            Ks.append(K.astype(np.float32))
            RTs.append(np.concatenate([R, T[:, None]], 1).astype(np.float32))
    B, N = batch, n_views
    vs = np.float32(2.0) / np.float32(D - 1)
    scene = dict(
        K=np.stack(Ks).reshape(B, N, 3, 3),
        RT=np.stack(RTs).reshape(B, N, 3, 4),
        depths=np.stack(depths).reshape(B, N, res, res),
        colors=np.stack(colors).reshape(B, N, res, res),
        vol_bbox=np.tile(np.array([[-1.0, 1.0]] * 3, np.float32), (B, 1, 1)),
        voxel_size=np.full((B, 1), vs, np.float32),
        trunc_weight=float(np.float32(trunc) / vs),
        D=D, res=res,
    )
    scene["masks"] = (scene["depths"] > 0).astype(np.int32)
    scene["R"] = np.ascontiguousarray(scene["RT"][..., :3])
    scene["T"] = np.ascontiguousarray(scene["RT"][..., 3])
    return scene


def camera_rays(K, R, T, res, stride=1):
    """rays_calculating for one camera: origins/directions [res*res, 3] f32."""
    v, u = np.mgrid[0:res:stride, 0:res:stride].astype(np.float64)
    pix = np.stack([u.ravel(), v.ravel(), np.ones(u.size)], 1)
    dw = (pix @ np.linalg.inv(K).T) @ R
    dw /= np.linalg.norm(dw, axis=1, keepdims=True) + 1e-10
    o = np.broadcast_to(-R.T @ T, dw.shape)
    return np.ascontiguousarray(o, np.float32), np.ascontiguousarray(dw, np.float32)


def target_rays(seed=0, res=512, batch=1):
    """Rays of a fifth camera on the same ring, at a seeded angle: [B,N,3]."""
    oris, dirs = [], []
    for b in range(batch):
        rng = np.random.default_rng(seed * 1000 + 777 + b)
        R, T = look_at((2.5 * math.cos(a := rng.uniform(0, 2 * math.pi)), 2.5 * math.sin(a), 1.2))
        o, d = camera_rays(intrinsics(res), R, T, res)
        oris.append(o)
        dirs.append(d)
    return np.stack(oris), np.stack(dirs)


def random_rays(seed, n, radius=3.0):
    """Rays with origins on a sphere aimed at uniform points in the cube."""
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(n, 3))
    o *= radius / np.linalg.norm(o, axis=1, keepdims=True)
    tgt = rng.uniform(-1.0, 1.0, (n, 3))
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def _view_images(rng, prims, K, R, T, res, noise, dropout):
    z = cast_depth(prims, K, R, T, res)
    hit = z > 0
    z = z + rng.normal(0.0, noise, z.shape) * hit
    z[rng.random(z.shape) < dropout] = 0.0
    u16 = np.clip(np.round(z * 10000.0), 0, 65535).astype(np.uint16)
    depth = (u16 / 10000.0).astype(np.float32)
    rgb = rng.integers(0, 256, (res, res, 3))
    color = np.floor(rgb[..., 2] * 65536.0 + rgb[..., 1] * 256.0 + rgb[..., 0]).astype(np.float32)
    return depth, color


def _batch_frame(job):
    seed, b, n_prims, views, view_res, noise, dropout = job
    frng = np.random.default_rng(seed * 1000 + 17 * b + 1)
    prims = random_primitives(frng, n_prims)
    nv = int(frng.integers(views[0], views[1] + 1))
    cams = ring_cameras(nv, phase=frng.uniform(0, 2 * math.pi))
    fr = dict(K=[], RT=[], depth=[], color=[])
    for R, T in cams:
        res = int(frng.choice(view_res))
        K = intrinsics(res)
        depth, color = _view_images(frng, prims, K, R, T, res, noise, dropout)
        fr["K"].append(K.astype(np.float32))
        fr["RT"].append(np.concatenate([R, T[:, None]], 1).astype(np.float32))
        fr["depth"].append(depth)
        fr["color"].append(color)
    return fr


def make_batch_workload(seed=0, n_frames=8, views=(4, 8), view_res=(512, 768, 1024), n_prims=12, D=256,
                        trunc=0.03, n_targets=16, target_res=(256, 1024), target_S=(32, 48, 64, 96, 128),
                        noise=0.005, dropout=0.02, workers=1):
    """Frames of uneven view counts and resolutions, each with its own seeded
    scene, and target cameras of uneven sizes and sample counts.  workers > 1
    generates the frames in that many spawned processes (same result).

    Returns dict(frames=[dict(K, RT, depth, color) lists per view],
    vol_bbox [B,3,2], voxel_size [B], trunc_weight, D,
    targets=[dict(frame, res, S, ori [res*res,3], dir [res*res,3])])."""
    jobs = [(seed, b, n_prims, views, view_res, noise, dropout) for b in range(n_frames)]
    if workers > 1:
        import concurrent.futures as cf
        import multiprocessing as mp
        with cf.ProcessPoolExecutor(min(workers, n_frames), mp_context=mp.get_context("spawn")) as ex:
            frames = list(ex.map(_batch_frame, jobs))
    else:
        frames = [_batch_frame(j) for j in jobs]
    rng = np.random.default_rng(seed)
    lo, hi = target_res
    sizes = np.linspace(lo, hi, n_targets)
    sizes = (np.round(sizes / 32.0) * 32).astype(int)
    rng.shuffle(sizes)
    targets = []
    for t in range(n_targets):
        res = int(sizes[t])
        a = rng.uniform(0, 2 * math.pi)
        R, T = look_at((2.5 * math.cos(a), 2.5 * math.sin(a), rng.uniform(0.6, 1.6)))
        o, d = camera_rays(intrinsics(res), R, T, res)
        targets.append(dict(frame=t % n_frames, res=res, S=int(target_S[t % len(target_S)]), ori=o, dir=d,
                            K=intrinsics(res).astype(np.float32), R=R.astype(np.float32), T=T.astype(np.float32)))
    vs = np.float32(2.0) / np.float32(D - 1)
    return dict(frames=frames, D=D,
                vol_bbox=np.tile(np.array([[-1.0, 1.0]] * 3, np.float32), (n_frames, 1, 1)),
                voxel_size=np.full((n_frames,), vs, np.float32),
                trunc_weight=float(np.float32(trunc) / vs), targets=targets)
