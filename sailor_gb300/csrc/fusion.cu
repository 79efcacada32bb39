// fusion.cu -- data-driven bounding box and TSDF fusion on sm_103a.
//
// Replaces fusion_kernel.cu (SAILOR c_lib/VoxelEncoding/src):
//   inverse_mat3x3 :105, obtain_origin_bbox :137, obtain_resized_bbox :51,
//   integrate_cuda :236 and the host wrapper fusion_cuda_integrate :600.
//
// fuse_tsdf: one thread per 4 consecutive z voxels, one CTA row of the grid
// per frame (blockIdx.y); CTAs take 16^3 voxel tiles (or, as a tuning
// alternative, linear runs of voxels).  Cameras (K, [R|T] of every view)
// sit in shared memory; tsdf/weight/colour live in registers across the view
// loop and are stored once with 16-byte vector stores (the reference pre-
// fills three full volumes with torch::full and then read-modify-writes them
// once per view).  Occupancy counts are warp-aggregated before one atomic
// per warp.  HBM traffic is the 16 bytes/voxel of the four outputs plus the
// depth/colour images (L2-resident gathers).
#include "common.cuh"

namespace sg {

constexpr int kMaxViews = 32;

// ---------------------------------------------------------------------------
// bounding box
// ---------------------------------------------------------------------------
__global__ void bbox_init_kernel(float *vol_origin, int B) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < B * 3) {
    vol_origin[2 * i] = 99999.0f;       // fusion_kernel.cu:655
    vol_origin[2 * i + 1] = -99999.0f;  // fusion_kernel.cu:656
  }
}

// float atomics for min / max that are exact (order-independent results)
__device__ __forceinline__ void atomic_min_f(float *a, float v) {
  if (v >= 0.0f) atomicMin((int *)a, __float_as_int(v));
  else atomicMax((unsigned *)a, __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float *a, float v) {
  if (v >= 0.0f) atomicMax((int *)a, __float_as_int(v));
  else atomicMin((unsigned *)a, __float_as_uint(v));
}

// Grid: (pixel tiles, B).  Each CTA inverts K and R of its frame's views
// into shared memory (the reference runs a separate inverse kernel), then
// back-projects its pixels and reduces the six extrema before one atomic
// each.
__global__ void __launch_bounds__(256) origin_bbox_kernel(
    const float *__restrict__ depth, const float *__restrict__ K, const float *__restrict__ R,
    const float *__restrict__ T, int N, int H, int W, float thres, float *vol_origin) {
  __shared__ float s_ki[kMaxViews][9], s_ri[kMaxViews][9], s_t[kMaxViews][3];
  __shared__ float s_red[6][8];
  int b = blockIdx.y;
  for (int v = threadIdx.x; v < N; v += blockDim.x) {
    inverse3x3(K + (size_t)(b * N + v) * 9, s_ki[v]);
    inverse3x3(R + (size_t)(b * N + v) * 9, s_ri[v]);
    for (int a = 0; a < 3; a++) s_t[v][a] = T[(size_t)(b * N + v) * 3 + a];
  }
  __syncthreads();
  float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  long npix = (long)N * H * W;
  const float *dm = depth + (size_t)b * npix;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (long)gridDim.x * blockDim.x) {
    float d = __ldg(dm + i);
    if (d < 0.1f || d > 5.0f) continue;
    int v = (int)(i / ((long)H * W));
    long p = i - (long)v * H * W;
    int y = (int)(p / W), x = (int)(p - (long)y * W);
    const float *ki = s_ki[v], *ri = s_ri[v];
    float px = (float)x, py = (float)y;
    float cx = (__fmaf_rn(ki[0], px, ki[1] * py) + ki[2]) * d;
    float cy = (__fmaf_rn(ki[3], px, ki[4] * py) + ki[5]) * d;
    float cz = (__fmaf_rn(ki[6], px, ki[7] * py) + ki[8]) * d;
    cx -= s_t[v][0];
    cy -= s_t[v][1];
    cz -= s_t[v][2];
    float q[3] = {dot3c(ri[0], ri[1], ri[2], cx, cy, cz), dot3c(ri[3], ri[4], ri[5], cx, cy, cz),
                  dot3c(ri[6], ri[7], ri[8], cx, cy, cz)};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      mn[a] = fminf(mn[a], q[a] - thres);
      mx[a] = fmaxf(mx[a], q[a] + thres);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; a++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(SG_FULL, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(SG_FULL, mx[a], o));
    }
  }
  int w = threadIdx.x >> 5;
  if (lane_id() == 0) {
    for (int a = 0; a < 3; a++) {
      s_red[2 * a][w] = mn[a];
      s_red[2 * a + 1][w] = mx[a];
    }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    int k = threadIdx.x;
    int nw = blockDim.x >> 5;
    float r = s_red[k][0];
    for (int j = 1; j < nw; j++) r = (k & 1) ? fmaxf(r, s_red[k][j]) : fminf(r, s_red[k][j]);
    if ((k & 1) == 0) {
      if (r < 3.0e38f) atomic_min_f(&vol_origin[b * 6 + k], r);
    } else {
      if (r > -3.0e38f) atomic_max_f(&vol_origin[b * 6 + k], r);
    }
  }
}

// obtain_resized_bbox (fusion_kernel.cu:51-103)
__global__ void resized_bbox_kernel(const float *vol_origin, int B, int D, float *vol_bbox,
                                    float *voxel_size) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const float *o = vol_origin + 6 * i;
  float x_min = o[0], x_max = o[1], y_min = o[2], y_max = o[3], z_min = o[4], z_max = o[5];
  float x_len = x_max - x_min, y_len = y_max - y_min, z_len = z_max - z_min;
  float max_len = fmaxf(x_len, fmaxf(y_len, z_len));
  float xc = (x_min + x_max) / 2.0f, yc = (y_min + y_max) / 2.0f, zc = (z_min + z_max) / 2.0f;
  voxel_size[i] = max_len / (float)(D - 1);
  float h = max_len / 2.0f;
  if (max_len == x_len) {
    y_min = yc - h; y_max = yc + h; z_min = zc - h; z_max = zc + h;
  } else if (max_len == y_len) {
    x_min = xc - h; x_max = xc + h; z_min = zc - h; z_max = zc + h;
  } else {
    x_min = xc - h; x_max = xc + h; y_min = yc - h; y_max = yc + h;
  }
  float *bb = vol_bbox + 6 * i;
  bb[0] = x_min; bb[1] = x_max; bb[2] = y_min; bb[3] = y_max; bb[4] = z_min; bb[5] = z_max;
}

// ---------------------------------------------------------------------------
// TSDF fusion
// ---------------------------------------------------------------------------
struct FuseParams {
  const float *K, *RT, *color, *depth, *vol_bbox, *voxel_size;
  float *tsdf, *weight, *colorv;
  int *occ, *count;
  int N, H, W, Dx, Dy, Dz;
  float obs_weight, trunc_weight, th_low, th_high;
  // view table (NULL: every frame has N views of H x W at [b, k] of K / RT / images)
  const int *view_begin, *view_hw;
  const long long *view_off;
  // per-view maps of 8 x 8 pixel blocks (deepest valid depth), or null
  const long long *block_off;
  float *blocks;
};

constexpr int kDepthBlock = 8;

// Cameras and images of one frame's views, staged in shared memory.
struct ViewSmem {
  float K[kMaxViews][9];
  float P[kMaxViews][12];
  long long off[kMaxViews];
  long long boff[kMaxViews];  // block map offsets (with FuseParams::blocks)
  int hw[kMaxViews][2];
  int n;
};

// Approximate reciprocal of the hardware (PTX rcp.approx.ftz.f32: at most
// 1 ulp relative error for normal inputs).
__device__ __forceinline__ float rcp_approx(float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return r;
}

// roundf(a / b) (half away from zero), exactly as the IEEE quotient would
// round, given r = rcp_approx(b).  q = a * r is within 1.5 * 2^-23 |q| of
// a / b, so q and a / b round to the same integer unless a half-integer lies
// within that distance; the test below keeps a margin of 4.8e-7 |q| + 6e-8
// (2.7x the bound, plus the rounding of q - floor(q) for -1 < q < 0).  Near a
// tie, for |q| >= 2^20, a non-finite q, or b outside [1e-30, 1e30] the IEEE
// quotient decides.
__device__ __forceinline__ float round_div(float a, float b, float r) {
  const float q = a * r;
  const float aq = fabsf(q), ab = fabsf(b);
  const float fl = floorf(q);
  const float d = q - fl;
  if (aq < 1048576.0f && ab >= 1.0e-30f && ab <= 1.0e30f && fabsf(d - 0.5f) > __fmaf_rn(aq, 4.8e-7f, 6.0e-8f))
    return copysignf(d > 0.5f ? fl + 1.0f : fl, q);
  return roundf(a / b);
}

// x / w: a product with the exact reciprocal when w is a power of two in
// [2^-126, 2^126] (x * 2^-e and x / 2^e are the same real number, rounded
// once), else the IEEE quotient.
__device__ __forceinline__ float div_weight(float x, float w) {
  const unsigned wb = __float_as_uint(w);
  if ((wb & 0x807fffffu) == 0u && wb - 0x00800000u <= 0x7e000000u) return x * __uint_as_float(0x7f000000u - wb);
  return x / w;
}

// Integrate one view into the running state of one voxel (the body of the
// view loop of integrate_cuda, fusion_kernel.cu:279-332).  Every value is
// the one the reference computes; the divisions take the exact shortcuts
// above (rounded quotients from the approximate reciprocal, power-of-two
// weights, and dist = 1 when diff >= trunc > 0, where diff / trunc >= 1).
__device__ __forceinline__ void integrate_view(const float *__restrict__ Kk, const float *__restrict__ P,
                                               float ax, float ay, float az, float pz,
                                               const float *__restrict__ dimg,
                                               const float *__restrict__ cimg, int H, int W,
                                               float trunc, float obs, float &ts, float &w,
                                               float &col) {
  // cam = [R|T] p: fma(P2, pz, fma(P0, px, P1*py)) + P3 with the inner
  // fma shared by the four voxels of the thread (ax/ay/az)
  float cx = __fmaf_rn(P[2], pz, ax) + P[3];
  float cy = __fmaf_rn(P[6], pz, ay) + P[7];
  float cz = __fmaf_rn(P[10], pz, az) + P[11];
  if (cz < 0.0f) return;  // rejected by the reference after the pixel test
  float ux = dot3c(Kk[0], Kk[1], Kk[2], cx, cy, cz);
  float uy = dot3c(Kk[3], Kk[4], Kk[5], cx, cy, cz);
  float uz = dot3c(Kk[6], Kk[7], Kk[8], cx, cy, cz);
  const float ru = rcp_approx(uz);
  int pxi = (int)round_div(ux, uz, ru), pyi = (int)round_div(uy, uz, ru);
  if (pxi < 0 || pxi >= W || pyi < 0 || pyi >= H) return;
  size_t pidx = (size_t)pyi * W + pxi;
  float dv = __ldg(dimg + pidx);
  if (dv < 0.1f || dv > 4.0f) return;
  float diff = dv - cz;
  if (diff < -trunc) return;
  float dist = (diff >= trunc && trunc > 0.0f) ? 1.0f : fminf(1.0f, diff / trunc);
  float w_old = w, w_new = w_old + obs;
  w = w_new;
  // (tsdf*w_old + obs*dist)/w_new: nvcc fuses the second product
  ts = div_weight(__fmaf_rn(obs, dist, ts * w_old), w_new);
  // packed colour b*65536 + g*256 + r: integer-valued floats, exact steps
  // (products with 2^-16 and 2^-8 are the reference's exact divisions)
  float old_b = floorf(col * (1.0f / 65536.0f));
  float old_g = floorf((col - old_b * 256.0f * 256.0f) * (1.0f / 256.0f));
  float old_r = col - old_b * 256.0f * 256.0f - old_g * 256.0f;
  float nc = __ldg(cimg + pidx);
  float nb = floorf(nc * (1.0f / 65536.0f));
  float ng = floorf((nc - nb * 256.0f * 256.0f) * (1.0f / 256.0f));
  float nr = nc - nb * 256.0f * 256.0f - ng * 256.0f;
  const float rw = rcp_approx(w_new);
  nb = fminf(round_div(__fmaf_rn(old_b, w_old, obs * nb), w_new, rw), 255.0f);
  ng = fminf(round_div(__fmaf_rn(old_g, w_old, obs * ng), w_new, rw), 255.0f);
  nr = fminf(round_div(__fmaf_rn(old_r, w_old, obs * nr), w_new, rw), 255.0f);
  col = nb * 256.0f * 256.0f + ng * 256.0f + nr;
}

// Common per-frame constants of the fusion kernels.
struct FuseFrame {
  int b;
  long vol;
  float vs, trunc, bx, by, bz, hi_th, lo_th;
};

__device__ __forceinline__ FuseFrame fuse_frame(const FuseParams &p, int b) {
  FuseFrame f;
  f.b = b;
  f.vol = (long)p.Dx * p.Dy * p.Dz;
  f.vs = p.voxel_size[b];
  f.trunc = f.vs * p.trunc_weight;
  f.bx = p.vol_bbox[b * 6 + 0];
  f.by = p.vol_bbox[b * 6 + 2];
  f.bz = p.vol_bbox[b * 6 + 4];
  f.hi_th = f.trunc * p.th_high;
  f.lo_th = -f.trunc * p.th_low;
  return f;
}

// Cameras and image placement of frame b's views into shared memory (all
// threads of the CTA take part).
__device__ __forceinline__ void load_views(const FuseParams &p, int b, ViewSmem &vw) {
  int v0, n;
  if (p.view_begin) {
    v0 = __ldg(p.view_begin + b);
    n = min(__ldg(p.view_begin + b + 1) - v0, kMaxViews);
  } else {
    v0 = b * p.N;
    n = p.N;
  }
  for (int i = threadIdx.x; i < n * 21; i += blockDim.x) {
    int v = i / 21, k = i - v * 21;
    if (k < 9) vw.K[v][k] = p.K[(size_t)(v0 + v) * 9 + k];
    else vw.P[v][k - 9] = p.RT[(size_t)(v0 + v) * 12 + (k - 9)];
  }
  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    if (p.blocks) vw.boff[v] = p.block_off[v0 + v];
    if (p.view_begin) {
      vw.off[v] = p.view_off[v0 + v];
      vw.hw[v][0] = p.view_hw[2 * (v0 + v)];
      vw.hw[v][1] = p.view_hw[2 * (v0 + v) + 1];
    } else {
      vw.off[v] = (long long)(v0 + v) * p.H * p.W;
      vw.hw[v][0] = p.H;
      vw.hw[v][1] = p.W;
    }
  }
  if (threadIdx.x == 0) vw.n = n;
  __syncthreads();
}

// Fuse the VPT z-consecutive voxels (x, y, z0 .. z0+VPT-1) over all views and
// store them; returns how many of them are occupied.  Views whose bit is set
// in skip are left out (none of these voxels passes their early returns).
template <int VPT>
__device__ __forceinline__ int fuse_group(const FuseParams &p, const FuseFrame &f, const ViewSmem &vw, int x,
                                          int y, int z0, unsigned skip) {
  const long v0 = ((long)x * p.Dy + y) * p.Dz + z0;
  float px = __fmaf_rn((float)x, f.vs, f.bx);
  float py = __fmaf_rn((float)y, f.vs, f.by);
  float pz[VPT], ts[VPT], w[VPT], col[VPT];
#pragma unroll
  for (int j = 0; j < VPT; j++) {
    pz[j] = __fmaf_rn((float)(z0 + j), f.vs, f.bz);
    ts[j] = 1.0f;
    w[j] = 0.0f;
    col[j] = 0.0f;
  }
  for (int k = 0; k < vw.n; k++) {
    if ((skip >> k) & 1u) continue;
    const float *P = vw.P[k];
    const float *Kk = vw.K[k];
    float ax = __fmaf_rn(P[0], px, P[1] * py);
    float ay = __fmaf_rn(P[4], px, P[5] * py);
    float az = __fmaf_rn(P[8], px, P[9] * py);
    const float *dimg = p.depth + vw.off[k];
    const float *cimg = p.color + vw.off[k];
    const int H = vw.hw[k][0], W = vw.hw[k][1];
#pragma unroll
    for (int j = 0; j < VPT; j++)
      integrate_view(Kk, P, ax, ay, az, pz[j], dimg, cimg, H, W, f.trunc, p.obs_weight, ts[j], w[j], col[j]);
  }
  int oc[VPT], cnt = 0;
#pragma unroll
  for (int j = 0; j < VPT; j++) {
    bool o = ts[j] < f.hi_th && ts[j] > f.lo_th;
    oc[j] = o ? (int)(v0 + j) : -1;
    cnt += o;
  }
  size_t o = (size_t)f.b * f.vol + v0;
  if constexpr (VPT == 4) {
    *reinterpret_cast<float4 *>(p.tsdf + o) = make_float4(ts[0], ts[1], ts[2], ts[3]);
    *reinterpret_cast<float4 *>(p.weight + o) = make_float4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<float4 *>(p.colorv + o) = make_float4(col[0], col[1], col[2], col[3]);
    *reinterpret_cast<int4 *>(p.occ + o) = make_int4(oc[0], oc[1], oc[2], oc[3]);
  } else if constexpr (VPT == 2) {
    *reinterpret_cast<float2 *>(p.tsdf + o) = make_float2(ts[0], ts[1]);
    *reinterpret_cast<float2 *>(p.weight + o) = make_float2(w[0], w[1]);
    *reinterpret_cast<float2 *>(p.colorv + o) = make_float2(col[0], col[1]);
    *reinterpret_cast<int2 *>(p.occ + o) = make_int2(oc[0], oc[1]);
  } else {
#pragma unroll
    for (int j = 0; j < VPT; j++) {
      p.tsdf[o + j] = ts[j];
      p.weight[o + j] = w[j];
      p.colorv[o + j] = col[j];
      p.occ[o + j] = oc[j];
    }
  }
  return cnt;
}

// Linear order: thread g takes voxels [g*VPT, g*VPT + VPT) of the frame.
template <int VPT>
__global__ void __launch_bounds__(256) fuse_tsdf_kernel(FuseParams p) {
  __shared__ ViewSmem vw;
  const int b = blockIdx.y;
  load_views(p, b, vw);
  const FuseFrame f = fuse_frame(p, b);
  const long groups = f.vol / VPT;
  int cnt = 0;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += (long)gridDim.x * blockDim.x) {
    long v0 = g * VPT;
    int x = (int)(v0 / ((long)p.Dy * p.Dz));
    long rem = v0 - (long)x * p.Dy * p.Dz;
    int y = (int)(rem / p.Dz);
    int z0 = (int)(rem - (long)y * p.Dz);
    cnt += fuse_group<VPT>(p, f, vw, x, y, z0, 0u);
  }
  cnt = warp_sum(cnt);
  if (lane_id() == 0 && cnt) atomicAdd(p.count + b, cnt);
}

// Deepest valid depth of every 8 x 8 pixel block of every view (block
// (by, bx) of view v at blocks[block_off[v] + by * ceil(W / 8) + bx]):
// -infinity when no pixel of the block is valid, +infinity when one is NaN
// (integrate_view takes NaN as valid).  Grid (CTAs per view, frame, view
// slot of the frame); thread per block.
__global__ void __launch_bounds__(256) depth_blocks_kernel(FuseParams p) {
  const int b = blockIdx.y;
  const int v = __ldg(p.view_begin + b) + (int)blockIdx.z;
  if (v >= __ldg(p.view_begin + b + 1)) return;
  const int H = __ldg(p.view_hw + 2 * v), W = __ldg(p.view_hw + 2 * v + 1);
  const int Wb = (W + kDepthBlock - 1) / kDepthBlock, Hb = (H + kDepthBlock - 1) / kDepthBlock;
  const float *img = p.depth + __ldg(p.view_off + v);
  float *out = p.blocks + __ldg(p.block_off + v);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < Hb * Wb; k += gridDim.x * blockDim.x) {
    const int by = k / Wb, bx = k - by * Wb;
    float m = -INFINITY;
    for (int y = by * kDepthBlock; y < min(H, by * kDepthBlock + kDepthBlock); y++)
      for (int x = bx * kDepthBlock; x < min(W, bx * kDepthBlock + kDepthBlock); x++) {
        const float dv = __ldg(img + (size_t)y * W + x);
        if (!(dv < 0.1f || dv > 4.0f)) m = dv != dv ? INFINITY : fmaxf(m, dv);
      }
    out[k] = m;
  }
}

// Per-view culling of a voxel tile.  A view is left out of a whole tile
// when every voxel of the tile would take one of integrate_view's early
// returns for it, so the tile's results are unchanged:
//   * every corner of the tile is behind the camera (cz < 0 for all voxels:
//     cz is affine in the voxel position, extreme at the corners), or
//   * the tile is in front of the camera (cz, uz > 0 at every corner) and
//     the pixel rectangle that holds the projections of all its voxels
//     (the projection of a box in front of the camera lies in the convex
//     hull of its corners' projections; widened by 2 pixels for rounding)
//     either misses the image, or holds no valid depth, or its deepest
//     valid depth is more than trunc in front of the tile's nearest corner
//     (diff < -trunc for every voxel).
// Margins of 1e-4 m (and 1e-5 relative) cover the rounding of the float
// camera coordinates; a NaN depth, which integrate_view takes as valid,
// keeps the view.  Rectangles above kCullMaxPixels keep the view unscanned.
constexpr float kCullEps = 1.0e-4f;
constexpr int kCullMaxPixels = 1 << 15;

struct CullSmem {
  int rect[kMaxViews][4];  // x0, x1, y0, y1 (clamped to the image)
  float czmin[kMaxViews];
  int state[kMaxViews];    // 0: keep, 1: leave out, 2: scan the rectangle
  int bskip[kMaxViews];    // block-map decision of a scanned view
  float wmax[2][8];
  int wnan[2][8];
  unsigned skip;
};

// The CTA (256 threads; every thread calls) finds the views to leave out of
// the tile of voxels lo .. hi (inclusive).  Result in cs.skip.
__device__ __forceinline__ void tile_cull(const FuseParams &p, const FuseFrame &f, const ViewSmem &vw,
                                          const int (&lo)[3], const int (&hi)[3], CullSmem &cs) {
  const int tid = threadIdx.x, n = vw.n;
  __syncthreads();  // the previous tile's readers of cs are done
  // corners: thread = (view tid / 8, corner tid % 8), kMaxViews * 8 == 256
  {
    const int k = tid >> 3, c = tid & 7;
    const int kv = k < n ? k : 0;
    const float px = __fmaf_rn((float)((c & 4) ? hi[0] : lo[0]), f.vs, f.bx);
    const float py = __fmaf_rn((float)((c & 2) ? hi[1] : lo[1]), f.vs, f.by);
    const float pz = __fmaf_rn((float)((c & 1) ? hi[2] : lo[2]), f.vs, f.bz);
    const float *P = vw.P[kv], *Kk = vw.K[kv];
    const float cx = __fmaf_rn(P[2], pz, __fmaf_rn(P[0], px, P[1] * py)) + P[3];
    const float cy = __fmaf_rn(P[6], pz, __fmaf_rn(P[4], px, P[5] * py)) + P[7];
    const float cz = __fmaf_rn(P[10], pz, __fmaf_rn(P[8], px, P[9] * py)) + P[11];
    const float ux = dot3c(Kk[0], Kk[1], Kk[2], cx, cy, cz);
    const float uy = dot3c(Kk[3], Kk[4], Kk[5], cx, cy, cz);
    const float uz = dot3c(Kk[6], Kk[7], Kk[8], cx, cy, cz);
    float qx0 = ux / uz, qx1 = qx0, qy0 = uy / uz, qy1 = qy0;
    float zmin = cz, zmax = cz, uzmin = uz;
    bool fin = isfinite(qx0) && isfinite(qy0);
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      qx0 = fminf(qx0, __shfl_xor_sync(SG_FULL, qx0, o));
      qx1 = fmaxf(qx1, __shfl_xor_sync(SG_FULL, qx1, o));
      qy0 = fminf(qy0, __shfl_xor_sync(SG_FULL, qy0, o));
      qy1 = fmaxf(qy1, __shfl_xor_sync(SG_FULL, qy1, o));
      zmin = fminf(zmin, __shfl_xor_sync(SG_FULL, zmin, o));
      zmax = fmaxf(zmax, __shfl_xor_sync(SG_FULL, zmax, o));
      uzmin = fminf(uzmin, __shfl_xor_sync(SG_FULL, uzmin, o));
      fin = __shfl_xor_sync(SG_FULL, (int)fin, o) && fin;
    }
    if (c == 0 && k < n) {
      int state = 0;
      if (zmax < -kCullEps) {
        state = 1;
      } else if (zmin > kCullEps && uzmin > kCullEps && fin && fabsf(qx0) < 1.0e6f && fabsf(qx1) < 1.0e6f &&
                 fabsf(qy0) < 1.0e6f && fabsf(qy1) < 1.0e6f) {
        const int H = vw.hw[k][0], W = vw.hw[k][1];
        const int x0 = max((int)floorf(qx0) - 2, 0), x1 = min((int)ceilf(qx1) + 2, W - 1);
        const int y0 = max((int)floorf(qy0) - 2, 0), y1 = min((int)ceilf(qy1) + 2, H - 1);
        if (x0 > x1 || y0 > y1) {
          state = 1;
        } else if ((long)(x1 - x0 + 1) * (y1 - y0 + 1) <= kCullMaxPixels) {
          state = 2;
          cs.rect[k][0] = x0;
          cs.rect[k][1] = x1;
          cs.rect[k][2] = y0;
          cs.rect[k][3] = y1;
          cs.czmin[k] = zmin;
        }
      }
      cs.state[k] = state;
    }
  }
  __syncthreads();
  unsigned skip = 0u;
  const int w8 = tid >> 5;
  if (p.blocks) {
    // the block map: warp w8 takes views w8, w8 + 8, ..., its lanes the 8 x 8
    // blocks covering the rectangle (a superset of its pixels, so the test
    // stays conservative)
    const int lane = tid & 31;
    for (int k = w8; k < n; k += 8) {
      if (cs.state[k] != 2) continue;
      const int bx0 = cs.rect[k][0] / kDepthBlock, bx1 = cs.rect[k][1] / kDepthBlock;
      const int by0 = cs.rect[k][2] / kDepthBlock, by1 = cs.rect[k][3] / kDepthBlock;
      const int Wb = (vw.hw[k][1] + kDepthBlock - 1) / kDepthBlock;
      const int nbx = bx1 - bx0 + 1, nb = nbx * (by1 - by0 + 1);
      const float *bm = p.blocks + vw.boff[k];
      float m = -INFINITY;
      for (int i = lane; i < nb; i += 32) {
        const int yy = i / nbx;
        m = fmaxf(m, __ldg(bm + (size_t)(by0 + yy) * Wb + bx0 + (i - yy * nbx)));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(SG_FULL, m, o));
      if (lane == 0)
        cs.bskip[k] = (m == -INFINITY || m - cs.czmin[k] < -f.trunc - kCullEps - 1.0e-5f * fabsf(m)) ? 1 : 0;
    }
    __syncthreads();
    for (int k = 0; k < n; k++) {
      const int state = cs.state[k];
      if (state == 1 || (state == 2 && cs.bskip[k])) skip |= 1u << k;
    }
    if (tid == 0) cs.skip = skip;
    __syncthreads();
    return;
  }
  int buf = 0;
  for (int k = 0; k < n; k++) {
    const int state = cs.state[k];
    if (state == 1) skip |= 1u << k;
    if (state != 2) continue;
    // deepest valid depth in the rectangle (16 x 16 threads over its pixels)
    const int x0 = cs.rect[k][0], x1 = cs.rect[k][1], y0 = cs.rect[k][2], y1 = cs.rect[k][3];
    const float *dimg = p.depth + vw.off[k];
    const int W = vw.hw[k][1];
    float m = -INFINITY;
    int nan = 0;
    for (int y = y0 + (tid >> 4); y <= y1; y += 16) {
      const float *row = dimg + (size_t)y * W;
      for (int x = x0 + (tid & 15); x <= x1; x += 16) {
        const float dv = __ldg(row + x);
        if (!(dv < 0.1f || dv > 4.0f)) {
          m = fmaxf(m, dv);
          nan |= dv != dv;
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      m = fmaxf(m, __shfl_xor_sync(SG_FULL, m, o));
      nan |= __shfl_xor_sync(SG_FULL, nan, o);
    }
    if ((tid & 31) == 0) {
      cs.wmax[buf][w8] = m;
      cs.wnan[buf][w8] = nan;
    }
    __syncthreads();
    float M = cs.wmax[buf][0];
    int anynan = cs.wnan[buf][0];
#pragma unroll
    for (int j = 1; j < 8; j++) {
      M = fmaxf(M, cs.wmax[buf][j]);
      anynan |= cs.wnan[buf][j];
    }
    buf ^= 1;  // the next view writes the other half, so no second barrier
    if (!anynan && (M == -INFINITY || M - cs.czmin[k] < -f.trunc - kCullEps - 1.0e-5f * fabsf(M))) skip |= 1u << k;
  }
  if (tid == 0) cs.skip = skip;
  __syncthreads();
}

// Tiled order: a CTA of 256 threads fuses a 16 x 16 x 16 voxel tile, as four
// passes of 4 (x) x 16 (y) x 16 (z) voxels, each thread 4 consecutive z.  The
// voxels of one tile project to one compact patch of every view, so the
// depth/colour gathers of the tile reuse L1 lines (a linear run of z voxels
// projects to a line of distinct pixels instead).  Tiles are taken z-fastest
// so CTAs resident at the same time work on neighbouring tiles.  Views that
// no voxel of the tile can pass are left out of the tile (tile_cull).
constexpr int kTileEdge = 16;

__global__ void __launch_bounds__(256) fuse_tsdf_tiled_kernel(FuseParams p, int tiles_y, int tiles_z,
                                                              long n_tiles) {
  static_assert(kMaxViews * 8 == 256, "one corner thread per (view, corner)");
  __shared__ ViewSmem vw;
  __shared__ CullSmem cs;
  const int b = blockIdx.y;
  load_views(p, b, vw);
  const FuseFrame f = fuse_frame(p, b);
  const int tz = threadIdx.x & 3, ty = (threadIdx.x >> 2) & 15, tx = threadIdx.x >> 6;
  int cnt = 0;
  for (long t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const int Tz = (int)(t % tiles_z);
    const long r = t / tiles_z;
    const int Ty = (int)(r % tiles_y), Tx = (int)(r / tiles_y);
    const int lo[3] = {Tx * kTileEdge, Ty * kTileEdge, Tz * kTileEdge};
    const int hi[3] = {min(lo[0] + kTileEdge - 1, p.Dx - 1), min(lo[1] + kTileEdge - 1, p.Dy - 1),
                       min(lo[2] + kTileEdge - 1, p.Dz - 1)};
    tile_cull(p, f, vw, lo, hi, cs);
    const unsigned skip = cs.skip;
    const int y = lo[1] + ty, z0 = lo[2] + tz * 4;
    if (y >= p.Dy || z0 >= p.Dz) continue;
#pragma unroll 1
    for (int pass = 0; pass < kTileEdge / 4; pass++) {
      const int x = lo[0] + pass * 4 + tx;
      if (x < p.Dx) cnt += fuse_group<4>(p, f, vw, x, y, z0, skip);
    }
  }
  cnt = warp_sum(cnt);
  if (lane_id() == 0 && cnt) atomicAdd(p.count + b, cnt);
}

}  // namespace sg

using namespace sg;

extern "C" int sg_auto_bbox(const float *depth, const float *K, const float *R, const float *T, int B,
                            int N, int H, int W, int vol_dim, float th_bbox, float *vol_origin,
                            float *vol_bbox, float *voxel_size, sg_stream_t stream) {
  if (!depth || !K || !R || !T || !vol_origin || !vol_bbox || !voxel_size) return SG_ERR_INVALID_ARG;
  if (B <= 0 || N <= 0 || N > kMaxViews || H <= 0 || W <= 0 || vol_dim < 2) return SG_ERR_INVALID_ARG;
  bbox_init_kernel<<<ceil_div(B * 3, 128), 128, 0, stream>>>(vol_origin, B);
  long npix = (long)N * H * W;
  int gx = ceil_div(npix, 256 * 8);
  if (gx > 4096) gx = 4096;
  origin_bbox_kernel<<<dim3(gx, B), 256, 0, stream>>>(depth, K, R, T, N, H, W, th_bbox, vol_origin);
  resized_bbox_kernel<<<ceil_div(B, 128), 128, 0, stream>>>(vol_origin, B, vol_dim, vol_bbox, voxel_size);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

static int launch_fuse(const FuseParams &p, int B, sg_stream_t stream) {
  const int Dx = p.Dx, Dy = p.Dy, Dz = p.Dz;
  long vol = (long)Dx * Dy * Dz;
  const uintptr_t ptrs = ((uintptr_t)p.tsdf) | ((uintptr_t)p.weight) | ((uintptr_t)p.colorv) | ((uintptr_t)p.occ);
  if (p.view_begin || (tune(SG_TUNE_FUSE_TILED) && Dz % 4 == 0 && ptrs % 16 == 0)) {
    const int ty = ceil_div(Dy, kTileEdge), tz = ceil_div(Dz, kTileEdge);
    const long n_tiles = (long)ceil_div(Dx, kTileEdge) * ty * tz;
    const int gx = n_tiles < 65535L * 16 ? (int)n_tiles : 65535 * 16;
    if (p.blocks) depth_blocks_kernel<<<dim3(16, B, kMaxViews), 256, 0, stream>>>(p);
    fuse_tsdf_tiled_kernel<<<dim3(gx, B), 256, 0, stream>>>(p, ty, tz, n_tiles);
    SG_LAUNCH_CHECK();
    return SG_OK;
  }
  int vpt = tune(SG_TUNE_FUSE_VPT);
  const int blk = tune(SG_TUNE_FUSE_BLOCK);
  while (vpt > 1 && (Dz % vpt != 0 || ptrs % (4 * vpt) != 0)) vpt >>= 1;
  const int gx = ceil_div(vol / vpt, blk);
  if (vpt == 4) fuse_tsdf_kernel<4><<<dim3(gx, B), blk, 0, stream>>>(p);
  else if (vpt == 2) fuse_tsdf_kernel<2><<<dim3(gx, B), blk, 0, stream>>>(p);
  else fuse_tsdf_kernel<1><<<dim3(gx, B), blk, 0, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_fuse_tsdf(const float *K, const float *RT, const float *color, const float *depth, int B,
                            int N, int H, int W, int Dx, int Dy, int Dz, const float *vol_bbox,
                            const float *voxel_size, float obs_weight, float trunc_weight, float th_low,
                            float th_high, float *tsdf, float *weight, float *colorv, int *occ,
                            int *count, sg_stream_t stream) {
  if (!K || !RT || !color || !depth || !vol_bbox || !voxel_size || !tsdf || !weight || !colorv || !occ ||
      !count)
    return SG_ERR_INVALID_ARG;
  if (B <= 0 || N <= 0 || N > kMaxViews || H <= 0 || W <= 0 || Dx <= 0 || Dy <= 0 || Dz <= 0)
    return SG_ERR_INVALID_ARG;
  FuseParams p{K, RT, color, depth, vol_bbox, voxel_size, tsdf, weight, colorv, occ, count,
               N, H, W, Dx, Dy, Dz, obs_weight, trunc_weight, th_low, th_high, nullptr, nullptr, nullptr};
  return launch_fuse(p, B, stream);
}

extern "C" int sg_fuse_tsdf_views(const SgViews *views, int B, int D, const float *vol_bbox,
                                  const float *voxel_size, float obs_weight, float trunc_weight, float th_low,
                                  float th_high, float *tsdf, float *weight, float *colorv, int *occ, int *count,
                                  sg_stream_t stream) {
  if (!views || !views->view_begin || !views->view_hw || !views->view_offset || !views->K || !views->RT ||
      !views->depth || !views->color || !vol_bbox || !voxel_size || !tsdf || !weight || !colorv || !occ || !count)
    return SG_ERR_INVALID_ARG;
  if (B <= 0 || D <= 0 || D % 4 != 0) return SG_ERR_INVALID_ARG;
  if (views->max_views > kMaxViews) return SG_ERR_UNSUPPORTED;
  if ((((uintptr_t)tsdf) | ((uintptr_t)weight) | ((uintptr_t)colorv) | ((uintptr_t)occ)) % 16 != 0)
    return SG_ERR_INVALID_ARG;
  if ((views->block_offset == nullptr) != (views->depth_blocks == nullptr)) return SG_ERR_INVALID_ARG;
  FuseParams p{views->K, views->RT, views->color, views->depth, vol_bbox, voxel_size, tsdf, weight, colorv, occ,
               count, 0, 0, 0, D, D, D, obs_weight, trunc_weight, th_low, th_high, views->view_begin,
               views->view_hw, views->view_offset, views->block_offset, views->depth_blocks};
  return launch_fuse(p, B, stream);
}
