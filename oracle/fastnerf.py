"""Oracle (test infrastructure) for the occupancy MLP of SAILOR's FastNerf
inference path: a numpy restatement of

  density_feat_kernel   c_lib/FastNerf/src/infer_mlp.cu:120-199
  density_sigma_kernel  infer_mlp.cu:202-240
  infer_density_mlp     infer_mlp.cu:583-636 (the two kernels around a
                        float32 mean over the views)

with the reference's float16 arithmetic reproduced step for step: every
layer starts from its bias and adds one weight x input product at a time
with __hfma (a fused multiply-add rounded once to float16, round to nearest
even), in the reference's loop order; ReLU is max(x, 0) on float16 values.
The occupancy compositing that consumes the densities
(volume_rendering_occ_kernel, infer_mlp.cu:508-580) is the pre-sorted
occupancy mode of ``oracle.composite_fwd`` with C channels.

Pinned: the reference kernels (compiled by ``oracle/build.py --fastnerf``
and run by ``tests/golden/make_golden.py --only density_mlp``) give
``tests/golden/ref_density_mlp.npz``, which this restatement reproduces bit
for bit (densities and geometry features); the CPU tests also pin the
float16 arithmetic (``hfma`` against exact rational arithmetic) and the
parameter layout.

Parameter layout of the density network (one float16 vector, per layer the
weights [out][in] row-major, then the bias [out]):
  [0, 13696)       feature MLP 18 -> 64 -> 64 -> 64 -> 64 (ReLU after each)
  [13696, 22081)   sigma MLP 64 -> 64 -> 64 -> 1 (ReLU, ReLU, sigmoid)
  [22081, 22521)   geometry MLP 18 -> 16 -> 8 (ReLU after each)
"""
import numpy as np

F16, F32, F64 = np.float16, np.float32, np.float64

FEAT_LAYERS = ((18, 64), (64, 64), (64, 64), (64, 64))
SIGMA_LAYERS = ((64, 64), (64, 64), (64, 1))
GEO_LAYERS = ((18, 16), (16, 8))
SIGMA_OFFSET = 13696  # infer_mlp.cu:125, 208
GEO_OFFSET = 22081    # infer_mlp.cu:127
PARAM_COUNT = GEO_OFFSET + 440


def layer_sizes(layers):
    return sum(i * o + o for i, o in layers)


def hfma(a, b, c):
    """a * b + c rounded once to float16 (__hfma), elementwise.

    The product p = a * b of two float16 values has at most 22 significant
    bits between 2^32 and 2^-48, so it is exact in float64.  The float64 sum
    s = fl64(p + c) is then the only extra rounding, and it never changes
    the float16 result:
    - If s is exact, rounding it to float16 is the fused operation.
    - s is inexact only when the exact x = p + c spans more than 53 bits.
      With |p| >= |c| that needs |p| >= 2^29 (c's last bit is >= 2^-24), and
      x overflows float16 either way.  With |c| > |p| it needs p's last bit
      (>= |p| 2^-21) below 2^-52 |c|, so |p| < 2^-30 |c|: x lies within
      2^-30 |c| of the float16 value c, while every float16 rounding
      midpoint is at least 2^-12 |c| from c (half an ulp of the binade below
      c's).  The float64 error, at most 2^-52 |c|, cannot carry x across a
      midpoint or onto one.
    So one rounding of s to float16 (nearest, ties to even) gives the fused
    operation's result, subnormal operands included."""
    a, b, c = np.broadcast_arrays(np.asarray(a, F16), np.asarray(b, F16), np.asarray(c, F16))
    with np.errstate(over="ignore", invalid="ignore"):
        return (a.astype(F64) * b.astype(F64) + c.astype(F64)).astype(F16)


def relu16(x):
    """relu (infer_mlp.cu:42-45): max(float(x), 0) back to float16; NaN -> 0
    as fmaxf gives."""
    return np.fmax(x, F16(0)).astype(F16)


def fc16(x, params, off, n_in, n_out):
    """fc_layer (infer_mlp.cu:80-100) for points x [P, n_in] float16 with the
    layer's parameters at params[off:]: out[i] = b[i], then
    out[i] = hfma(W[i][j], x[j], out[i]) for j = 0 .. n_in-1."""
    W = params[off:off + n_in * n_out].reshape(n_out, n_in)
    b = params[off + n_in * n_out:off + n_in * n_out + n_out]
    acc = np.broadcast_to(b, (x.shape[0], n_out)).astype(F16)
    for j in range(n_in):
        acc = hfma(W[None, :, j], x[:, j, None], acc)
    return acc


def _mlp(x, params, off, layers, last_relu=True):
    for k, (n_in, n_out) in enumerate(layers):
        x = fc16(x, params, off, n_in, n_out)
        off += n_in * n_out + n_out
        if last_relu or k + 1 < len(layers):
            x = relu16(x)
    return x


def density_feat(points_z, points_tpsdf, feats_geo, params):
    """density_feat_kernel: per point-view (z, t_psdf, 16 geometry features)
    -> (64 density features, 8 geometry features), float32 outputs of the
    float16 network.  Inputs [P], [P], [P, 16] float32."""
    params = np.asarray(params, F16)
    x = np.concatenate([np.asarray(points_z, F32).reshape(-1, 1), np.asarray(points_tpsdf, F32).reshape(-1, 1),
                        np.asarray(feats_geo, F32).reshape(-1, 16)], axis=1).astype(F16)
    dens = _mlp(x, params, 0, FEAT_LAYERS)
    geo = _mlp(x, params, GEO_OFFSET, GEO_LAYERS)
    return dens.astype(F32), geo.astype(F32)


def sigmoid16(x):
    """sigmoid (infer_mlp.cu:48-50): 1 / (1 + exp(-x)) in float32 from the
    float16 input, rounded to float16 (exp evaluated in float64 and rounded
    to float32; CUDA's expf is within 2 ulp of that)."""
    xf = np.asarray(x, F16).astype(F32)
    e = np.exp(-xf.astype(F64)).astype(F32)
    return (F32(1.0) / (F32(1.0) + e)).astype(F16)


def density_sigma(mean_feats, params):
    """density_sigma_kernel: 64 mean density features [P, 64] float32 ->
    density [P] float32 (the sigmoid of the float16 network's output)."""
    params = np.asarray(params, F16)
    x = np.asarray(mean_feats, F32).reshape(-1, 64).astype(F16)
    y = _mlp(x, params, SIGMA_OFFSET, SIGMA_LAYERS, last_relu=False)
    return sigmoid16(y[:, 0]).astype(F32)


def infer_density(points_z, points_tpsdf, feats_geo, params, batch_size, num_points, num_views):
    """infer_density_mlp: inputs [B, V, N, 1|16] (B batches, V views, N
    points) -> densities [B, 1, N] float32.  The mean over the views is
    taken as torch's float32 reduction does it for a short axis: a float32
    sum in view order, times float32(1 / V); another summation order moves
    a mean by a float32 ulp, which changes the float16 input of the sigma
    network only next to a float16 rounding boundary."""
    B, V, N = batch_size, num_views, num_points
    dens, geo = density_feat(points_z, points_tpsdf, feats_geo, params)
    per_view = dens.reshape(B, V, N, 64)
    acc = np.zeros((B, N, 64), F32)
    for v in range(V):
        acc = (acc + per_view[:, v]).astype(F32)
    mean = (acc * F32(1.0 / V)).astype(F32)
    return density_sigma(mean.reshape(-1, 64), params).reshape(B, 1, N), geo.reshape(B, V, N, 8)


def composite_occ(sorted_z, occ, feats, t_thres=1e-4):
    """volume_rendering_occ_kernel (infer_mlp.cu:508-580): pre-sorted depths
    [..., S], occupancies [..., S] used as alphas, features [..., S, C] ->
    (features [..., C], depth [..., 1]) in float64; a ray whose last raw
    depth is negative gives zeros.  The same restatement as the VoxelEncoding
    occupancy compositing (oracle.composite_fwd, pre-sorted, occupancy mode)
    with the features' own channel count (30 in FastNerf)."""
    from . import oracle as orc
    of, od, _, _, _ = orc.composite_fwd(sorted_z, None, occ, feats, t_thres, occ_mode=True)
    return of, od


# --------------------------------------------------------------------------
# float32-accumulating and float64 evaluations of the same network (the
# tolerance references of the tensor-core kernel)
# --------------------------------------------------------------------------
def _fc_acc(x16, params, off, n_in, n_out, dtype):
    W = np.asarray(params[off:off + n_in * n_out], F16).reshape(n_out, n_in).astype(F64)
    b = np.asarray(params[off + n_in * n_out:off + n_in * n_out + n_out], F16).astype(F64)
    acc = x16.astype(F64) @ W.T
    if dtype == F32:  # products summed in float32 precision, then the bias in float32
        return (acc.astype(F32) + b.astype(F32)).astype(F32)
    return acc + b


def _mlp_acc(x, params, off, layers, last_relu, dtype):
    for k, (n_in, n_out) in enumerate(layers):
        y = _fc_acc(x, params, off, n_in, n_out, dtype)
        off += n_in * n_out + n_out
        if dtype == F32:
            y = y.astype(F16)  # layer outputs rounded to float16 as the reference rounds them
        if last_relu or k + 1 < len(layers):
            y = np.maximum(y, 0).astype(y.dtype)
        x = y
    return x


def infer_density_acc(points_z, points_tpsdf, feats_geo, params, batch_size, num_points, num_views, dtype=F32):
    """infer_density with each layer's products summed at once instead of
    through a float16 __hfma chain.  dtype float32: layer sums in float32,
    layer outputs rounded to float16 where the reference rounds them (the
    arithmetic of a float32-accumulating implementation, up to the order of
    its float32 additions); float64: no rounding after the float16 inputs
    and weights (the network's exact value).  Returns (densities [B, 1, N],
    geometry features [B, V, N, 8]) as float64."""
    B, V, N = batch_size, num_views, num_points
    params = np.asarray(params, F16)
    x = np.concatenate([np.asarray(points_z, F32).reshape(-1, 1), np.asarray(points_tpsdf, F32).reshape(-1, 1),
                        np.asarray(feats_geo, F32).reshape(-1, 16)], axis=1).astype(F16)
    dens = _mlp_acc(x, params, 0, FEAT_LAYERS, True, dtype)
    geo = _mlp_acc(x, params, GEO_OFFSET, GEO_LAYERS, True, dtype)
    pv = dens.astype(F64 if dtype == F64 else F32).reshape(B, V, N, 64)
    if dtype == F32:
        acc = np.zeros((B, N, 64), F32)
        for v in range(V):
            acc = (acc + pv[:, v]).astype(F32)
        mean = (acc * F32(1.0 / V)).astype(F32).reshape(-1, 64).astype(F16)
    else:
        mean = pv.mean(1).reshape(-1, 64)
    h = _mlp_acc(mean, params, SIGMA_OFFSET, SIGMA_LAYERS[:2], True, dtype)
    w3 = params[SIGMA_OFFSET + 8320:SIGMA_OFFSET + 8384].astype(F64)
    b3 = F64(params[SIGMA_OFFSET + 8384])
    pre = h.astype(F64) @ w3 + b3
    if dtype == F32:
        pre = pre.astype(F32).astype(F16).astype(F64)
        d = (F32(1) / (F32(1) + np.exp(-pre).astype(F32))).astype(F16).astype(F64)
    else:
        d = 1.0 / (1.0 + np.exp(-pre))
    return d.reshape(B, 1, N), geo.astype(F64).reshape(B, V, N, 8)
