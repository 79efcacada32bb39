// render.cu -- fused per-ray render and its adjoint: sampling -> sort -> field
// taps -> compositing, forward and backward in one kernel each.
//
// One warp per ray does, without leaving the SM:
//   the reference's coarse sampling (ray_voxels_sampling_uniform_kernel,
//   sampling_kernel.cu:1070-1177) into shared memory, the per-ray sort
//   (sort_samplings :1308-1329) in registers, per-sample density from the
//   fused TSDF grid and colour from a dense feature grid (trilinear taps and
//   a linear colour head; the stand-in for SRONet's MLP), and density
//   compositing of the sorted samples (volume_rendering_training_forward_
//   kernel, volume_rendering.cu:17-126, with the transmittance carried in
//   strict sample order).
// The forward writes 24 bytes per ray (rgb, depth, weight sum, alpha); the
// sorted depths / node ids only when requested.  With a 3-channel colour
// grid and no head its results equal the unfused chain sg_sample_sorted ->
// sg_grid_gather (x2) -> sg_composite_fwd on the same inputs.
//
// The backward saves nothing from the forward: it re-runs the same per-ray
// evaluation (same samples, taps, alpha and transmittance, bit for bit),
// forms the exact adjoint of compositing from in-warp prefix sums, chains
// it through the density transform and the colour head, and scatters the
// per-sample gradients into the TSDF and feature grids: lanes own (corner,
// channel) slots, consecutive samples in one trilinear cell accumulate in
// registers, and each cell change flushes one atomic add per slot.
//
// Launches are persistent grid-stride loops over the rays of all frames and
// target cameras; a segment table (SgRaySegments) gives each ray its frame
// and sample count.
#include <climits>

#include "ray_core.cuh"
#include "scatter.cuh"

namespace sg {

struct RenderParams {
  SampleParams sp;  // tree, hits, jitter, valid_len, N (rays per frame without segments), W, S (row stride)
  const int *hit_count;
  float rand_const;
  long R;
  int nseg;  // 0: frames of sp.N rays with sp.S samples each
  const int *seg_begin, *seg_frame, *seg_samples;
  const float *ori, *dir;
  const float *tsdf;
  int D;
  float sdf_scale, sdf_s;
  const float *feat;
  int Df;
  const float *fbbox, *fvs;
  const float *head;  // [3, C] or null (C == 3)
  float t_thres;
  float dk, inv_s;    // density constants: sdf_scale / sdf_s, 1 / sdf_s
  bool shared;        // feature grid on the TSDF grid's geometry (one tap cell)
  float *out_rgb, *out_depth, *out_ws, *out_alpha, *out_z;
  int *out_node;
  const float *g_rgb, *g_depth, *g_ws, *g_alpha;
  float *grad_feat, *grad_tsdf, *grad_sigma, *grad_rgb;
  // training step: upstream gradient of loss_scale / 2 * |rgb - target|^2
  const float *target_rgb;
  float loss_scale;
  float *out_loss;
  // gradient records instead of the scatter (deterministic reduction,
  // scatter.cu): the launch's rays are hit_ray[k], k in [*k_begin, *k_end);
  // ray k's used samples, in sorted position order, go to record slots
  // hit_slot[k], hit_slot[k] + 1, ... (below rec_cap), their count to
  // ray_nrec[k]
  const int *hit_ray, *hit_slot, *k_begin, *k_end;
  int *ray_nrec;
  uint32_t *rec_key;
  GradRecord *rec;
  float *ray_g;  // [k][C]: head^T (colour gradient of ray k)
  long rec_cap;
  RecordKeys keys;
};

__device__ __forceinline__ void ray_frame(const RenderParams &p, long r, int &b, int &S, int &s) {
  if (p.nseg > 0) {
    s = segment_of(p.seg_begin, p.nseg, r);
    b = __ldg(p.seg_frame + s);
    S = min(__ldg(p.seg_samples + s), p.sp.S);
  } else {
    s = 0;
    b = (int)(r / p.sp.N);
    S = p.sp.S;
  }
}

template <int E>
struct RayEval {
  float z[E], sg[E], s01[E], al[E], tb[E], dl[E], rgb[E][3];
  unsigned valid, proc, post;
  int done;
};

// Warp-private shared memory of the render kernels.
template <int E>
struct RenderSmem {
  float *z, *f;
  int *i, *p;
  SampleScratch *sc;
};

// Samples, sort, field taps, alpha and transmittance of ray r (frame b, S
// samples) into ev; sorted depths stay in sm.z, with POS the sorted
// positions in sm.p.
template <int E, int C, bool POS>
__device__ __forceinline__ void eval_ray(const RenderParams &p, long r, int b, int S, int sgm,
                                         const RenderSmem<E> &sm, RayEval<E> &ev) {
  const int lane = lane_id();
  const int nh = p.hit_count ? min(__ldg(p.hit_count + r), p.sp.W) : p.sp.W;
  ev.done = warp_sample_ray(p.sp, r, b, S, nh, p.rand_const, sm.z, sm.i, *sm.sc);
  ev.valid = ev.proc = ev.post = 0;
  if (ev.done == 0) return;
  warp_sort_samples<E, POS>(sm.z, sm.p, S, ev.done);
  const float *bb = p.sp.t.vol_bbox + 6 * b;
  const float bmin[3] = {bb[0], bb[2], bb[4]};
  const float vs = __ldg(p.sp.t.voxel_size + b), inv_vs = 1.0f / vs;
  const float *fb = p.fbbox + 6 * b;
  const float fmin[3] = {fb[0], fb[2], fb[4]};
  const float fvs = __ldg(p.fvs + b), inv_fvs = 1.0f / fvs;
  const float *tsdf = p.tsdf + (size_t)b * p.D * p.D * p.D;
  const float *feat = p.feat + (size_t)b * p.Df * p.Df * p.Df * C;
  const float o[3] = {__ldg(p.ori + r * 3), __ldg(p.ori + r * 3 + 1), __ldg(p.ori + r * 3 + 2)};
  const float dr[3] = {__ldg(p.dir + r * 3), __ldg(p.dir + r * 3 + 1), __ldg(p.dir + r * 3 + 2)};
#pragma unroll
  for (int e = 0; e < E; e++) {
    const int i = e * 32 + lane;
    ev.z[e] = (i < S) ? sm.z[i] : -1.0f;
    ev.sg[e] = ev.s01[e] = 0.0f;
    ev.rgb[e][0] = ev.rgb[e][1] = ev.rgb[e][2] = 0.0f;
    if (ev.z[e] >= 0.0f) {
      ev.valid |= 1u << e;
      const float pt[3] = {__fmaf_rn(dr[0], ev.z[e], o[0]), __fmaf_rn(dr[1], ev.z[e], o[1]),
                           __fmaf_rn(dr[2], ev.z[e], o[2])};
      int i0[3];
      float wc[8];
      tap_cell(bmin, vs, inv_vs, pt, i0, wc);
      float t1[1];
      grid_tap_cell<1>(tsdf, p.D, i0, wc, t1);
      ev.s01[e] = tsdf_sigmoid(t1[0], p.dk);  // kept for the adjoint
      ev.sg[e] = ev.s01[e] * p.inv_s;
      if (!p.shared) tap_cell(fmin, fvs, inv_fvs, pt, i0, wc);
      float fe[C];
      grid_tap_cell<C>(feat, p.Df, i0, wc, fe);
      if (p.head) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          float a = 0.0f;
#pragma unroll
          for (int c = 0; c < C; c++) a = __fmaf_rn(__ldg(p.head + k * C + c), fe[c], a);
          ev.rgb[e][k] = a;
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) ev.rgb[e][k] = fe[k < C ? k : 0];
      }
    }
  }
  ray_alpha<E>(ev.z, ev.sg, ev.valid, S, 0, sm.z, ev.al, ev.dl);
  ray_transmittance<E>(ev.al, ev.valid, S, p.t_thres, sm.f, ev.tb, ev.proc, ev.post);
}

#define SG_RENDER_SMEM(E)                         \
  __shared__ __align__(16) float s_zall[8][32 * E]; \
  __shared__ __align__(16) float s_fall[8][kTransScratch<E>]; \
  __shared__ int s_iall[8][32 * E];                 \
  __shared__ int s_pall[8][32 * E];                 \
  __shared__ SampleScratch s_sc[8];                 \
  const int w8 = threadIdx.x >> 5;                  \
  const RenderSmem<E> sm{s_zall[w8], s_fall[w8], s_iall[w8], s_pall[w8], &s_sc[w8]};

template <int E, int C>
__global__ void __launch_bounds__(256) render_fwd_kernel(RenderParams p) {
  SG_RENDER_SMEM(E)
  const int lane = lane_id();
  const int Smax = p.sp.S;
  // a segment table covers rays [ray_begin[0], total): a sub-table of
  // consecutive segments is a group of targets
  const long r0 = p.nseg > 0 ? (long)__ldg(p.seg_begin) : 0;
  for (long r = r0 + (((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < p.R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    int b, S, sgm;
    ray_frame(p, r, b, S, sgm);
    RayEval<E> ev;
    eval_ray<E, C, true>(p, r, b, S, sgm, sm, ev);
    float acc_r = 0.0f, acc_g = 0.0f, acc_b = 0.0f, d = 0.0f, ws = 0.0f, aa = 0.0f;
    if (p.out_z) {
      for (int i = lane; i < Smax; i += 32) {
        const bool has = ev.done > 0 && i < S;
        p.out_z[(size_t)r * Smax + i] = has ? sm.z[i] : -1.0f;
        p.out_node[(size_t)r * Smax + i] = has ? sm.i[sm.p[i]] : -1;
      }
    }
    if (ev.done > 0) {
      // a ray whose largest depth is < 0 renders 0 (no sample: done == 0)
#pragma unroll
      for (int e = 0; e < E; e++) {
        if (((ev.proc & ev.valid) >> e) & 1u) {
          const float w = ev.al[e] * ev.tb[e];
          acc_r += w * ev.rgb[e][0];
          acc_g += w * ev.rgb[e][1];
          acc_b += w * ev.rgb[e][2];
          d += w * ev.z[e];
          ws += w;
          aa += w * ev.al[e];
        }
      }
      acc_r = warp_sum(acc_r);
      acc_g = warp_sum(acc_g);
      acc_b = warp_sum(acc_b);
      d = warp_sum(d);
      ws = warp_sum(ws);
      aa = warp_sum(aa);
    }
    if (lane == 0) {
      p.out_rgb[r * 3 + 0] = acc_r;
      p.out_rgb[r * 3 + 1] = acc_g;
      p.out_rgb[r * 3 + 2] = acc_b;
      p.out_depth[r] = d;
      p.out_ws[r] = ws;
      p.out_alpha[r] = aa;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// backward
// ---------------------------------------------------------------------------
// Scatter layout of the backward.  Feature gradient: with C == 16, lane l
// owns corner l / 4, channels 4 (l % 4) .. 4 (l % 4) + 3 (one float4, flushed
// with one vector reduction); with C == 3, lane l < 24 owns corner l / 3,
// channel l % 3.  TSDF gradient: lane l owns corner l - kTsdfLane0<C> when
// that is in [0, 8).
// A trilinear cell (lower corner i0, each axis in [-1, D-1] when any corner
// is inside the grid) packed into one non-negative key of 21 bits per axis;
// -1 when no corner is inside (the sample contributes nothing).
__device__ __forceinline__ long long cell_key(const int (&i0)[3], int D) {
  if (i0[0] < -1 || i0[1] < -1 || i0[2] < -1 || i0[0] >= D || i0[1] >= D || i0[2] >= D) return -1;
  return ((long long)(i0[0] + 1) << 42) | ((long long)(i0[1] + 1) << 21) | (long long)(i0[2] + 1);
}

struct Cell3 {
  int v[3];
};
__device__ __forceinline__ Cell3 cell_of(long long k) {
  return Cell3{{(int)(k >> 42) - 1, (int)((k >> 21) & 0x1fffff) - 1, (int)(k & 0x1fffff) - 1}};
}

template <int C>
constexpr int kTsdfLane0 = (C == 3) ? 24 : 0;

template <int C>
__device__ __forceinline__ void flush_feat(const RenderParams &p, int b, const Cell3 &c3, float4 &acc) {
  const int(&cell)[3] = c3.v;
  const int lane = lane_id();
  size_t off;
  if constexpr (C == 16) {
    if ((acc.x != 0.0f || acc.y != 0.0f || acc.z != 0.0f || acc.w != 0.0f) && corner_inside(cell, lane >> 2, p.Df, off))
      red_add_f32x4(p.grad_feat + ((size_t)b * p.Df * p.Df * p.Df + off) * C + 4 * (lane & 3), acc.x, acc.y, acc.z,
                    acc.w);
  } else {
    if (lane < 8 * C && acc.x != 0.0f && corner_inside(cell, lane / C, p.Df, off))
      atomicAdd(p.grad_feat + ((size_t)b * p.Df * p.Df * p.Df + off) * C + lane % C, acc.x);
  }
  acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

template <int C>
__device__ __forceinline__ void flush_tsdf(const RenderParams &p, int b, const Cell3 &c3, float &acc) {
  const int(&cell)[3] = c3.v;
  const int cr = lane_id() - kTsdfLane0<C>;
  size_t off;
  if (cr >= 0 && cr < 8 && acc != 0.0f && corner_inside(cell, cr, p.D, off))
    atomicAdd(p.grad_tsdf + (size_t)b * p.D * p.D * p.D + off, acc);
  acc = 0.0f;
}

// Records of ray r (compact index k) for the deterministic reduction of the
// grid gradients.  The colour head is linear, so the feature gradient of
// the sample at sorted position i is w_i G with G = head^T g_c (g_c: the
// gradient of the ray's colour, w_i its compositing weight): G goes to
// ray_g[k] once per ray, and each used sample's record holds its cell (the
// key), its cell fractions and w_i, the ray and its TSDF gradient.  The
// records of the samples with a cell are packed, in sorted position order,
// at the front of the ray's slots (a warp scan over the positions); their
// count goes to ray_nrec[k].
template <int E, int C>
__device__ __forceinline__ void emit_records(const RenderParams &p, long k, long r, int b, int S,
                                             const RayEval<E> &ev, const float (&w)[E], const float (&gsig)[E],
                                             const float (&gc)[3]) {
  const int lane = lane_id();
  if (lane < C) {
    float g;
    if (p.head)
      g = __fmaf_rn(__ldg(p.head + 2 * C + lane), gc[2], __fmaf_rn(__ldg(p.head + C + lane), gc[1],
                                                                    __ldg(p.head + lane) * gc[0]));
    else
      g = lane < 3 ? gc[lane] : 0.0f;
    p.ray_g[k * C + lane] = g;
  }
  const long base = __ldg(p.hit_slot + k);
  const float *fb = p.fbbox + 6 * b;
  const float fmin[3] = {fb[0], fb[2], fb[4]};
  const float fvs = __ldg(p.fvs + b), inv_fvs = 1.0f / fvs;
  const float o[3] = {__ldg(p.ori + r * 3), __ldg(p.ori + r * 3 + 1), __ldg(p.ori + r * 3 + 2)};
  const float dr[3] = {__ldg(p.dir + r * 3), __ldg(p.dir + r * 3 + 1), __ldg(p.dir + r * 3 + 2)};
  const float dsdt_k = -p.dk * p.inv_s;
  const unsigned used = ev.proc & ev.valid;
  const unsigned below = (1u << lane) - 1u;
  int n = 0;  // records of the positions before this block
#pragma unroll
  for (int e = 0; e < E; e++) {
    const int i = e * 32 + lane;
    uint32_t key = p.keys.invalid;
    float f[3] = {0.0f, 0.0f, 0.0f};
    if (i < S && ((used >> e) & 1u)) {
      const float pt[3] = {__fmaf_rn(dr[0], ev.z[e], o[0]), __fmaf_rn(dr[1], ev.z[e], o[1]),
                           __fmaf_rn(dr[2], ev.z[e], o[2])};
      int i0[3];
      tap_frac(fmin, fvs, inv_fvs, pt, i0, f);
      key = record_key(p.keys, b, i0);
    }
    const bool has = key != p.keys.invalid;
    const unsigned m = __ballot_sync(SG_FULL, has);
    const long slot = base + n + __popc(m & below);
    if (has && slot < p.rec_cap) {
      const float gt = p.grad_tsdf ? gsig[e] * (ev.s01[e] * (1.0f - ev.s01[e]) * dsdt_k) : 0.0f;
      p.rec[slot].fw = make_float4(f[0], f[1], f[2], w[e]);
      p.rec[slot].kt = make_int4((int)k, __float_as_int(gt), 0, 0);
      p.rec_key[slot] = key;
    }
    n += __popc(m);
  }
  if (lane == 0) {
    // the ray's records within the slot capacity
    const long room = p.rec_cap - base;
    p.ray_nrec[k] = (int)(room <= 0 ? 0 : (n < room ? n : room));
  }
}

// TRAIN: the upstream gradient is formed in the kernel from the ray's own
// outputs (loss = loss_scale / 2 * |rgb - target|^2 per ray, so d loss /
// d rgb = loss_scale * (rgb - target)); the outputs and per-ray loss are
// written, and nothing is recomputed.
// Resident CTAs per SM the adjoint kernels' register budget is set for: the
// training pass of the smaller sample capacities has less live state, so
// more of its warps fit (64 and 80 registers, a few bytes spilled; 4 and 3
// CTAs measured 7 % faster over the batched step than 2 CTAs at 128).
// The record-mode pass (REC) carries no scatter state, so more of its CTAs
// fit: 4 / 4 / 3 at up to 32 / 64 / 128 samples (measured 0.27 ms faster on
// the batched step than 4 / 3 / 2; 5 / 4 / 3 and 6 / 4 / 2 were slower).
// Build-time settings SG_REC_MINB_E1/E2/E4.
#ifndef SG_REC_MINB_E1
#define SG_REC_MINB_E1 4
#endif
#ifndef SG_REC_MINB_E2
#define SG_REC_MINB_E2 4
#endif
#ifndef SG_REC_MINB_E4
#define SG_REC_MINB_E4 3
#endif
template <int E, bool TRAIN, bool REC = false>
constexpr int kBwdMinBlocks = !TRAIN ? 2
                              : (REC ? (E == 1 ? SG_REC_MINB_E1 : (E == 2 ? SG_REC_MINB_E2 : SG_REC_MINB_E4))
                                     : (E == 1 ? 4 : (E == 2 ? 3 : 2)));

// REC: the rays are the compact list of rays with hits and the grid
// gradients leave the kernel as per-sample records (emit_records) for the
// deterministic reduction, instead of the in-kernel scatter with atomics.
template <int E, int C, bool TRAIN, bool REC>
__global__ void __launch_bounds__(256, kBwdMinBlocks<E, TRAIN, REC>) render_bwd_kernel(RenderParams p) {
  static_assert(C == 3 || C == 16, "feature grids of 3 or 16 channels");
  SG_RENDER_SMEM(E)
  __shared__ float s_wf[REC ? 1 : 8][32][9], s_wt[REC ? 1 : 8][32][9];
  __shared__ __align__(16) float s_g[REC ? 1 : 8][32][C == 16 ? 20 : 4];
  __shared__ long long s_kf[REC ? 1 : 8][32], s_kt[REC ? 1 : 8][32];  // packed cell keys, -1: no contribution
  const int lane = lane_id();
  const int Smax = p.sp.S;
  // a segment table covers rays [ray_begin[0], total): a sub-table of
  // consecutive segments is a group of targets
  const long it0 = REC ? (long)__ldg(p.k_begin) : (p.nseg > 0 ? (long)__ldg(p.seg_begin) : 0);
  const long it1 = REC ? (long)__ldg(p.k_end) : p.R;
  for (long it = it0 + (((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5); it < it1;
       it += ((long)gridDim.x * blockDim.x) >> 5) {
    const long r = REC ? (long)__ldg(p.hit_ray + it) : it;
    int b, S, sgm;
    ray_frame(p, r, b, S, sgm);
    RayEval<E> ev;
    eval_ray<E, C, false>(p, r, b, S, sgm, sm, ev);
    if (ev.done == 0) {
      if (REC && lane == 0) p.ray_nrec[it] = 0;  // no sample: no record
      if (p.grad_sigma) {
        for (int i = lane; i < Smax; i += 32) {
          p.grad_sigma[(size_t)r * Smax + i] = 0.0f;
          for (int k = 0; k < 3; k++) p.grad_rgb[((size_t)r * Smax + i) * 3 + k] = 0.0f;
        }
      }
      if (TRAIN && lane == 0) {
        // no sample: zero outputs, loss of the target alone, no gradient
        float l = 0.0f;
        for (int k = 0; k < 3; k++) {
          const float t = __ldg(p.target_rgb + r * 3 + k);
          p.out_rgb[r * 3 + k] = 0.0f;
          l += t * t;
        }
        p.out_depth[r] = p.out_ws[r] = p.out_alpha[r] = 0.0f;
        if (p.out_loss) p.out_loss[r] = 0.5f * p.loss_scale * l;
      }
      __syncwarp();
      continue;
    }
    float gc[3] = {0.0f, 0.0f, 0.0f}, gd = 0.0f, gws = 0.0f, ga = 0.0f;
    if (!TRAIN) {
      if (p.g_rgb) {
        gc[0] = __ldg(p.g_rgb + r * 3);
        gc[1] = __ldg(p.g_rgb + r * 3 + 1);
        gc[2] = __ldg(p.g_rgb + r * 3 + 2);
      }
      gd = p.g_depth ? __ldg(p.g_depth + r) : 0.0f;
      gws = p.g_ws ? __ldg(p.g_ws + r) : 0.0f;
      ga = p.g_alpha ? __ldg(p.g_alpha + r) : 0.0f;
    }
    // weights and inclusive prefix sums over sorted positions of
    // w*rgb, w*z, w, w*alpha; totals by carries (the forward's outputs)
    float w[E], pf[E][3], pd[E], pw[E], pa[E];
    float cf[3] = {0.0f, 0.0f, 0.0f}, cd = 0.0f, cw = 0.0f, ca = 0.0f;
    const unsigned used = ev.proc & ev.valid;
#pragma unroll
    for (int e = 0; e < E; e++) {
      w[e] = ((used >> e) & 1u) ? ev.al[e] * ev.tb[e] : 0.0f;
      if (!__any_sync(SG_FULL, (used >> e) & 1u)) {
        // a block of positions no lane uses (past the ray's sample count or
        // its termination): zero weights, the running totals stand
#pragma unroll
        for (int k = 0; k < 3; k++) pf[e][k] = cf[k];
        pd[e] = cd;
        pw[e] = cw;
        pa[e] = ca;
        continue;
      }
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float v = warp_incl_scan_f(w[e] * ev.rgb[e][k]);
        pf[e][k] = cf[k] + v;
        cf[k] += __shfl_sync(SG_FULL, v, 31);
      }
      if (!TRAIN) {
        const float vd = warp_incl_scan_f(w[e] * ev.z[e]);
        const float vw = warp_incl_scan_f(w[e]);
        const float va = warp_incl_scan_f(w[e] * ev.al[e]);
        pd[e] = cd + vd;
        pw[e] = cw + vw;
        pa[e] = ca + va;
        cd += __shfl_sync(SG_FULL, vd, 31);
        cw += __shfl_sync(SG_FULL, vw, 31);
        ca += __shfl_sync(SG_FULL, va, 31);
      }
    }
    if (TRAIN) {
      // the loss reads only the colour: depth, weight sum and alpha sum are
      // outputs alone, summed as the forward kernel sums them
      float d = 0.0f, ws = 0.0f, aa = 0.0f;
#pragma unroll
      for (int e = 0; e < E; e++) {
        if ((used >> e) & 1u) {
          d += w[e] * ev.z[e];
          ws += w[e];
          aa += w[e] * ev.al[e];
        }
      }
      cd = warp_sum(d);
      cw = warp_sum(ws);
      ca = warp_sum(aa);
    }
    if (TRAIN) {
      // forward outputs = the totals; upstream gradient of the per-ray loss
      float l = 0.0f;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float d = cf[k] - __ldg(p.target_rgb + r * 3 + k);
        gc[k] = p.loss_scale * d;
        l += d * d;
      }
      if (lane == 0) {
        p.out_rgb[r * 3 + 0] = cf[0];
        p.out_rgb[r * 3 + 1] = cf[1];
        p.out_rgb[r * 3 + 2] = cf[2];
        p.out_depth[r] = cd;
        p.out_ws[r] = cw;
        p.out_alpha[r] = ca;
        if (p.out_loss) p.out_loss[r] = 0.5f * p.loss_scale * l;
      }
    }
    // exact adjoint per sorted position: d out / d sigma_i = delta_i *
    // (T_{i+1} v_i - sum_{j>i} w_j v_j) (v = rgb, z, 1; 2 alpha T_{i+1} for
    // the alpha sum); d out / d rgb_i = w_i
    float gsig[E], grgb[E][3];
#pragma unroll
    for (int e = 0; e < E; e++) {
      gsig[e] = 0.0f;
      grgb[e][0] = grgb[e][1] = grgb[e][2] = 0.0f;
      if (((ev.proc & ev.valid) >> e) & 1u) {
        const float Ta = ev.tb[e] * (1.0f - ev.al[e]);
        float acc = 0.0f;
        if (!TRAIN)
          acc = gws * (Ta - (cw - pw[e])) + gd * (Ta * ev.z[e] - (cd - pd[e])) +
                ga * (2.0f * ev.al[e] * Ta - (ca - pa[e]));
#pragma unroll
        for (int k = 0; k < 3; k++) acc += gc[k] * (Ta * ev.rgb[e][k] - (cf[k] - pf[e][k]));
        gsig[e] = ev.dl[e] * acc;
#pragma unroll
        for (int k = 0; k < 3; k++) grgb[e][k] = w[e] * gc[k];
      }
    }
    if (p.grad_sigma) {
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int i = e * 32 + lane;
        if (i < Smax) {
          p.grad_sigma[(size_t)r * Smax + i] = i < S ? gsig[e] : 0.0f;
#pragma unroll
          for (int k = 0; k < 3; k++) p.grad_rgb[((size_t)r * Smax + i) * 3 + k] = i < S ? grgb[e][k] : 0.0f;
        }
      }
      for (int i = 32 * E + lane; i < Smax; i += 32) {
        p.grad_sigma[(size_t)r * Smax + i] = 0.0f;
        for (int k = 0; k < 3; k++) p.grad_rgb[((size_t)r * Smax + i) * 3 + k] = 0.0f;
      }
    }
    if (REC) {
      emit_records<E, C>(p, it, r, b, S, ev, w, gsig, gc);
      __syncwarp();
      continue;
    }
    if (!p.grad_feat && !p.grad_tsdf) {
      __syncwarp();
      continue;
    }
    // scatter into the grids, samples in sorted order
    const float *bb = p.sp.t.vol_bbox + 6 * b;
    const float bmin[3] = {bb[0], bb[2], bb[4]};
    const float vs = __ldg(p.sp.t.voxel_size + b), inv_vs = 1.0f / vs;
    const float *fb = p.fbbox + 6 * b;
    const float fmin[3] = {fb[0], fb[2], fb[4]};
    const float fvs = __ldg(p.fvs + b), inv_fvs = 1.0f / fvs;
    const float o[3] = {__ldg(p.ori + r * 3), __ldg(p.ori + r * 3 + 1), __ldg(p.ori + r * 3 + 2)};
    const float dr[3] = {__ldg(p.dir + r * 3), __ldg(p.dir + r * 3 + 1), __ldg(p.dir + r * 3 + 2)};
    const float dsdt_k = -p.dk * p.inv_s;
    // lane-owned accumulators: feature (corner, channels) and TSDF corner
    float4 accf = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float acct = 0.0f;
    const int fcr = (C == 16) ? (lane >> 2) : (lane < 8 * C ? lane / C : 0);
    const int fch = (C == 16) ? 4 * (lane & 3) : (lane < 8 * C ? lane % C : 0);
    const int tcr = lane - kTsdfLane0<C>;
    const bool town = tcr >= 0 && tcr < 8;
    long long curf = -1, curt = -1;
    const bool want_t = p.grad_tsdf != nullptr, want_f = p.grad_feat != nullptr;
#pragma unroll
    for (int e = 0; e < E; e++) {
      const bool use = ((used >> e) & 1u) != 0;
      if (!__any_sync(SG_FULL, use)) continue;  // no sample of this block contributes
      long long kf = -1, kt = -1;
      if (use) {
        const float pt[3] = {__fmaf_rn(dr[0], ev.z[e], o[0]), __fmaf_rn(dr[1], ev.z[e], o[1]),
                             __fmaf_rn(dr[2], ev.z[e], o[2])};
        int i0[3];
        float wt[8];
        tap_cell(bmin, vs, inv_vs, pt, i0, wt);
        if (want_t) {
          kt = cell_key(i0, p.D);
#pragma unroll
          for (int cr = 0; cr < 8; cr++) s_wt[w8][lane][cr] = wt[cr];
          s_g[w8][lane][C == 16 ? 16 : 3] = gsig[e] * (ev.s01[e] * (1.0f - ev.s01[e]) * dsdt_k);
        }
        if (want_f) {
          if (!p.shared) tap_cell(fmin, fvs, inv_fvs, pt, i0, wt);
          kf = cell_key(i0, p.Df);
#pragma unroll
          for (int cr = 0; cr < 8; cr++) s_wf[w8][lane][cr] = wt[cr];
          // feature gradient: head^T d rgb
#pragma unroll
          for (int c = 0; c < C; c++) {
            float g;
            if (p.head)
              g = __fmaf_rn(__ldg(p.head + 2 * C + c), grgb[e][2],
                            __fmaf_rn(__ldg(p.head + C + c), grgb[e][1], __ldg(p.head + c) * grgb[e][0]));
            else
              g = c < 3 ? grgb[e][c] : 0.0f;
            s_g[w8][lane][c] = g;
          }
        }
      }
      s_kf[w8][lane] = kf;
      s_kt[w8][lane] = kt;
      __syncwarp();
      // samples with a cell, in sorted order (the same mask in every lane)
      const unsigned mf = __ballot_sync(SG_FULL, kf >= 0), mt = __ballot_sync(SG_FULL, kt >= 0);
      if (want_f) {
        for (unsigned m = mf; m; m &= m - 1) {
          const int j = __ffs(m) - 1;
          const long long k = s_kf[w8][j];
          if (k != curf) {
            if (curf >= 0) flush_feat<C>(p, b, cell_of(curf), accf);
            curf = k;
          }
          const float wf = s_wf[w8][j][fcr];
          if constexpr (C == 16) {
            const float4 g4 = *reinterpret_cast<const float4 *>(&s_g[w8][j][fch]);
            accf.x = __fmaf_rn(wf, g4.x, accf.x);
            accf.y = __fmaf_rn(wf, g4.y, accf.y);
            accf.z = __fmaf_rn(wf, g4.z, accf.z);
            accf.w = __fmaf_rn(wf, g4.w, accf.w);
          } else {
            accf.x = __fmaf_rn(wf, s_g[w8][j][fch], accf.x);
          }
        }
      }
      if (want_t) {
        for (unsigned m = mt; m; m &= m - 1) {
          const int j = __ffs(m) - 1;
          const long long k = s_kt[w8][j];
          if (k != curt) {
            if (curt >= 0) flush_tsdf<C>(p, b, cell_of(curt), acct);
            curt = k;
          }
          if (town) acct = __fmaf_rn(s_wt[w8][j][tcr], s_g[w8][j][C == 16 ? 16 : 3], acct);
        }
      }
      __syncwarp();
    }
    if (curf >= 0) flush_feat<C>(p, b, cell_of(curf), accf);
    if (curt >= 0) flush_tsdf<C>(p, b, cell_of(curt), acct);
    __syncwarp();
  }
}

static int render_grid(long R) {
  long g = (R * 32 + 255) / 256;
  const long cap = (long)num_sms() * tune(SG_TUNE_RENDER_WARPS);
  return (int)(g < cap ? g : cap);
}

// mode 0: forward, 1: backward, 2: training step (forward + loss + backward),
// 3: training step writing gradient records
template <int E, int C>
static void launch_render_e(const RenderParams &p, int mode, int g, sg_stream_t stream) {
  if (mode == 0) render_fwd_kernel<E, C><<<g, 256, 0, stream>>>(p);
  else if (mode == 1) render_bwd_kernel<E, C, false, false><<<g, 256, 0, stream>>>(p);
  else if (mode == 2) render_bwd_kernel<E, C, true, false><<<g, 256, 0, stream>>>(p);
  else render_bwd_kernel<E, C, true, true><<<g, 256, 0, stream>>>(p);
}

template <int C>
static int launch_render(const RenderParams &p, int mode, int g, sg_stream_t stream) {
  const int S = p.sp.S;
  if (S <= 32) launch_render_e<1, C>(p, mode, g, stream);
  else if (S <= 64) launch_render_e<2, C>(p, mode, g, stream);
  else if (S <= 128) launch_render_e<4, C>(p, mode, g, stream);
  else return SG_ERR_UNSUPPORTED;
  SG_LAUNCH_CHECK();
  return SG_OK;
}

static int launch_render_c(const RenderParams &p, int C, int mode, sg_stream_t stream) {
  if (p.R <= 0) return SG_OK;
  const int g = render_grid(p.R);
  if (C == 3) return launch_render<3>(p, mode, g, stream);
  if (C == 16) return launch_render<16>(p, mode, g, stream);
  return SG_ERR_UNSUPPORTED;
}

// RenderParams of the batched entry points.
static int segment_params(const SgTree *tree, const SgRaySegments *seg, const SgRenderArgs *a, RenderParams &p) {
  if (!tree || !seg || !a) return SG_ERR_INVALID_ARG;
  if (seg->count <= 0 || seg->total < 0 || !seg->ray_begin || !seg->frame || !seg->samples)
    return SG_ERR_INVALID_ARG;
  if (!a->hit_idx || !a->hit_t0 || !a->hit_t1 || !a->valid_len || !a->tsdf || !a->feat || !a->feat_bbox ||
      !a->feat_vs)
    return SG_ERR_INVALID_ARG;
  // the render reads ray buffers (for camera segments: sg_segment_rays)
  if (!a->ori || !a->dir) return SG_ERR_INVALID_ARG;
  if (a->W <= 0 || a->S <= 0 || a->D <= 0 || a->Df <= 0 || tree->B <= 0 || a->sdf_s == 0.0f)
    return SG_ERR_INVALID_ARG;
  if (!a->head && a->C != 3) return SG_ERR_INVALID_ARG;
  p = RenderParams{};
  p.sp = SampleParams{*tree, a->hit_idx, a->hit_t0, a->hit_t1, a->rands, a->valid_len, 1, a->W, a->S, 2, 0,
                      nullptr, nullptr, a->rand_seed};
  p.hit_count = a->hit_count;
  p.rand_const = a->rand_const;
  p.R = seg->total;
  p.nseg = seg->count;
  p.seg_begin = seg->ray_begin;
  p.seg_frame = seg->frame;
  p.seg_samples = seg->samples;
  p.ori = a->ori;
  p.dir = a->dir;
  p.tsdf = a->tsdf;
  p.D = a->D;
  p.sdf_scale = a->sdf_scale;
  p.sdf_s = a->sdf_s;
  p.feat = a->feat;
  p.Df = a->Df;
  p.fbbox = a->feat_bbox;
  p.fvs = a->feat_vs;
  p.head = a->head;
  p.t_thres = a->t_thres;
  p.dk = a->sdf_scale / a->sdf_s;
  p.inv_s = 1.0f / a->sdf_s;
  p.shared = a->Df == a->D && a->feat_bbox == tree->vol_bbox && a->feat_vs == tree->voxel_size;
  // float4 loads of the feature rows and of the colour head's rows
  if (a->C == 16 && (((uintptr_t)a->feat) % 16 != 0 || ((uintptr_t)a->head) % 16 != 0)) return SG_ERR_INVALID_ARG;
  return SG_OK;
}

}  // namespace sg

using namespace sg;

extern "C" int sg_render_fused(const SgTree *tree, const int *hit_idx, const float *hit_t0, const float *hit_t1,
                               const int *hit_count, int N, int W, const float *rands, float rand_const,
                               const float *valid_len, int S, int num_levels, int start_level,
                               const float *ori, const float *dir, const float *tsdf, int D, float sdf_scale,
                               float sdf_s, const float *color_grid, int Dc, const float *color_bbox,
                               const float *color_vs, float t_thres, float *out_rgb, float *out_depth,
                               float *out_ws, float *out_alpha, float *out_z, int *out_node,
                               sg_stream_t stream) {
  if (!tree || !hit_idx || !hit_t0 || !hit_t1 || !valid_len || !ori || !dir || !tsdf || !color_grid ||
      !color_bbox || !color_vs || !out_rgb || !out_depth || !out_ws || !out_alpha)
    return SG_ERR_INVALID_ARG;
  if ((out_z == nullptr) != (out_node == nullptr)) return SG_ERR_INVALID_ARG;
  if (N <= 0 || W <= 0 || S <= 0 || D <= 0 || Dc <= 0 || tree->B <= 0 || sdf_s == 0.0f)
    return SG_ERR_INVALID_ARG;
  RenderParams p{};
  p.sp = SampleParams{*tree, hit_idx, hit_t0, hit_t1, rands, valid_len, N, W, S, num_levels, start_level,
                      nullptr, nullptr, 0ull};
  p.hit_count = hit_count;
  p.rand_const = rand_const;
  p.R = (long)tree->B * N;
  p.nseg = 0;
  p.ori = ori;
  p.dir = dir;
  p.tsdf = tsdf;
  p.D = D;
  p.sdf_scale = sdf_scale;
  p.sdf_s = sdf_s;
  p.feat = color_grid;
  p.Df = Dc;
  p.fbbox = color_bbox;
  p.fvs = color_vs;
  p.head = nullptr;
  p.t_thres = t_thres;
  p.dk = sdf_scale / sdf_s;
  p.inv_s = 1.0f / sdf_s;
  p.shared = Dc == D && color_bbox == tree->vol_bbox && color_vs == tree->voxel_size;
  p.out_rgb = out_rgb;
  p.out_depth = out_depth;
  p.out_ws = out_ws;
  p.out_alpha = out_alpha;
  p.out_z = out_z;
  p.out_node = out_node;
  return launch_render_c(p, 3, 0, stream);
}

extern "C" int sg_render_segments_fwd(const SgTree *tree, const SgRaySegments *seg, const SgRenderArgs *args,
                                      float *out_rgb, float *out_depth, float *out_ws, float *out_alpha,
                                      float *out_z, int *out_node, sg_stream_t stream) {
  RenderParams p;
  int rc = segment_params(tree, seg, args, p);
  if (rc != SG_OK) return rc;
  if (!out_rgb || !out_depth || !out_ws || !out_alpha || (out_z == nullptr) != (out_node == nullptr))
    return SG_ERR_INVALID_ARG;
  p.out_rgb = out_rgb;
  p.out_depth = out_depth;
  p.out_ws = out_ws;
  p.out_alpha = out_alpha;
  p.out_z = out_z;
  p.out_node = out_node;
  return launch_render_c(p, args->C, 0, stream);
}

extern "C" int sg_render_segments_bwd(const SgTree *tree, const SgRaySegments *seg, const SgRenderArgs *args,
                                      const float *g_rgb, const float *g_depth, const float *g_ws,
                                      const float *g_alpha, float *grad_feat, float *grad_tsdf,
                                      float *grad_sigma, float *grad_rgb, sg_stream_t stream) {
  RenderParams p;
  int rc = segment_params(tree, seg, args, p);
  if (rc != SG_OK) return rc;
  if ((grad_sigma == nullptr) != (grad_rgb == nullptr)) return SG_ERR_INVALID_ARG;
  p.g_rgb = g_rgb;
  p.g_depth = g_depth;
  p.g_ws = g_ws;
  p.g_alpha = g_alpha;
  p.grad_feat = grad_feat;
  p.grad_tsdf = grad_tsdf;
  p.grad_sigma = grad_sigma;
  p.grad_rgb = grad_rgb;
  return launch_render_c(p, args->C, 1, stream);
}

extern "C" int sg_render_segments_train(const SgTree *tree, const SgRaySegments *seg, const SgRenderArgs *args,
                                        const float *target_rgb, float loss_scale, float *out_rgb,
                                        float *out_depth, float *out_ws, float *out_alpha, float *out_loss,
                                        float *grad_feat, float *grad_tsdf, sg_stream_t stream) {
  RenderParams p;
  int rc = segment_params(tree, seg, args, p);
  if (rc != SG_OK) return rc;
  if (!target_rgb || !out_rgb || !out_depth || !out_ws || !out_alpha) return SG_ERR_INVALID_ARG;
  p.target_rgb = target_rgb;
  p.loss_scale = loss_scale;
  p.out_loss = out_loss;
  p.out_rgb = out_rgb;
  p.out_depth = out_depth;
  p.out_ws = out_ws;
  p.out_alpha = out_alpha;
  p.grad_feat = grad_feat;
  p.grad_tsdf = grad_tsdf;
  return launch_render_c(p, args->C, 2, stream);
}

// ---------------------------------------------------------------------------
// training step with the deterministic gradient reduction (scatter.cu)
// ---------------------------------------------------------------------------
extern "C" size_t sg_train_det_workspace_bytes(long long R, int nseg, int C, long long capacity) {
  if (R < 0 || nseg < 0 || C <= 0 || capacity < 0) return 0;
  return det_layout((long)R, nseg, C, (long)(capacity > 0 ? capacity : 1), nullptr, nullptr);
}

extern "C" int sg_render_segments_train_det(const SgTree *tree, const SgRaySegments *seg, const SgRenderArgs *args,
                                            int ngroups, const int *groups, const int *group_S,
                                            const float *target_rgb, float loss_scale, float *out_rgb,
                                            float *out_depth, float *out_ws, float *out_alpha, float *out_loss,
                                            float *grad_feat, float *grad_tsdf, void *workspace,
                                            size_t workspace_bytes, long long capacity, SgStatus *status,
                                            sg_stream_t stream) {
  RenderParams p;
  int rc = segment_params(tree, seg, args, p);
  if (rc != SG_OK) return rc;
  if (!target_rgb || !out_rgb || !out_depth || !out_ws || !out_alpha || !grad_feat || !workspace) return SG_ERR_INVALID_ARG;
  if (ngroups <= 0 || !groups || !group_S || groups[0] != 0 || groups[ngroups] != seg->count) return SG_ERR_INVALID_ARG;
  for (int g = 0; g < ngroups; g++)
    if (groups[g + 1] <= groups[g] || group_S[g] <= 0 || group_S[g] > args->S) return SG_ERR_INVALID_ARG;
  if (capacity <= 0 || capacity >= (1ll << 31)) return SG_ERR_INVALID_ARG;
  if (grad_tsdf && !p.shared) return SG_ERR_UNSUPPORTED;
  if (args->C != 3 && args->C != 16) return SG_ERR_UNSUPPORTED;
  if (!record_keys_fit(tree->B, args->Df)) return SG_ERR_UNSUPPORTED;
  const long R = seg->total;
  if (workspace_bytes < det_layout(R, seg->count, args->C, (long)capacity, nullptr, nullptr))
    return SG_ERR_INVALID_ARG;
  if (((uintptr_t)workspace) % 256 != 0) return SG_ERR_INVALID_ARG;
  if (R == 0) return SG_OK;
  if (!args->hit_count) return SG_ERR_INVALID_ARG;  // the ray scan reads the hit counts
  DetWork w;
  det_layout(R, seg->count, args->C, (long)capacity, (char *)workspace, &w);
  DetTrainOut o{target_rgb, loss_scale, out_rgb, out_depth, out_ws, out_alpha, out_loss};
  rc = launch_det_prepare(w, *seg, args->S, args->hit_count, R, (long)capacity, o, status, stream);
  if (rc != SG_OK) return rc;
  p.target_rgb = target_rgb;
  p.loss_scale = loss_scale;
  p.out_loss = out_loss;
  p.out_rgb = out_rgb;
  p.out_depth = out_depth;
  p.out_ws = out_ws;
  p.out_alpha = out_alpha;
  p.grad_feat = grad_feat;
  p.grad_tsdf = grad_tsdf;
  p.hit_ray = w.hit_ray;
  p.hit_slot = w.hit_slot;
  p.ray_nrec = w.ray_nrec;
  p.rec_key = w.rec_key;
  p.rec = w.rec;
  p.ray_g = w.ray_g;
  p.rec_cap = (long)capacity;
  p.keys = make_record_keys(tree->B, args->Df);
  for (int g = 0; g < ngroups; g++) {
    RenderParams pg = p;
    pg.sp.S = group_S[g];
    pg.k_begin = w.seg_hit + groups[g];
    pg.k_end = w.seg_hit + groups[g + 1];
    // the group's count of rays with hits is on the device: the grid is the
    // persistent cap, its warps striding over the compact range
    const int gsz = render_grid(R);
    if (args->C == 3) rc = launch_render<3>(pg, 3, gsz, stream);
    else rc = launch_render<16>(pg, 3, gsz, stream);
    if (rc != SG_OK) return rc;
  }
  return launch_det_reduce(w, p.keys, R, (long)capacity, args->C, grad_feat, grad_tsdf, stream);
}
