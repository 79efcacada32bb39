// composite.cu -- volume-rendering compositing and its adjoints on sm_103a.
//
// Replaces volume_rendering.cu (SAILOR c_lib/VoxelEncoding/src):
//   volume_rendering_training_forward_kernel :17-126 (density),
//   volume_rendering_occ_training_forward_kernel :129-240 (occupancy),
//   volume_rendering_occ_kernel :666-745 (pre-sorted occupancy),
//   volume_rendering_training_backward_kernel :244-381 and the occupancy
//   backward :384-522.
//
// One warp per ray; lane l holds sorted positions l, l+32, ...  Loads are
// coalesced within the ray's rows (the reference walks one ray per thread,
// so a warp's loads touch 32 different rows).  Per-sample alpha is
// computed in parallel; transmittance is carried through the positions in
// strict sequential order (a broadcast of each lane's factor, multiplied
// into a warp-uniform running product) so it is bit-identical to the
// reference's serial T *= 1 - alpha, and so is the early-termination
// decision T < t_thres.  Weighted sums use warp reductions / scans.
//
// The backward recomputes alpha and transmittance from the inputs and the
// per-ray outputs (no per-sample state is saved).  exact == 0 reproduces the
// reference's gradient formula; exact == 1 is the true derivative of the
// forward (the reference adds g_ws*(1-ws) four extra times and drops the
// sample that triggers early termination).
#include "ray_core.cuh"

namespace sg {

constexpr int kMaxC = 32;     // forward: FastNerf composites 30 channels (infer_mlp.cu:508-580)
constexpr int kMaxCBwd = 16;  // adjoint (no inference-only caller needs more)

struct CompParams {
  const float *z;
  const int *sort_idx;
  const float *sigma, *feats;
  long R;
  int S, C;
  float t_thres;
  int mode;
  // forward outputs / backward saved outputs
  float *of, *od, *ows, *oa;
  // backward
  const float *g_feat, *g_depth, *g_ws, *g_alpha;
  int exact;
  float *grad_feats, *grad_sigma;
};

// Per-ray state shared by forward and backward: positions in sorted order.
template <int E>
struct RayState {
  float z[E], sg[E], al[E], tb[E];
  int s[E];
  unsigned valid;  // bit e: position e*32+lane holds a valid sample
  unsigned proc;   // bit e: position processed (before early termination)
  unsigned post;   // bit e: transmittance after the sample is >= t_thres
};

template <int E>
__device__ __forceinline__ bool load_ray(const CompParams &p, long r, float *s_z, float *s_f, RayState<E> &st) {
  const int lane = lane_id();
  const size_t rb = (size_t)r * p.S;
  const int S = p.S;
  int last = p.sort_idx ? __ldg(p.sort_idx + rb + S - 1) : S - 1;
  if (__ldg(p.z + rb + last) < 0) return false;  // invalid ray
  st.valid = 0;
#pragma unroll
  for (int e = 0; e < E; e++) {
    int i = e * 32 + lane;
    if (i < S) {
      int s = p.sort_idx ? __ldg(p.sort_idx + rb + i) : i;
      st.s[e] = s;
      st.z[e] = __ldg(p.z + rb + s);
      st.sg[e] = __ldg(p.sigma + rb + s);
      if (st.z[e] >= 0) st.valid |= 1u << e;
    } else {
      st.s[e] = -1;
      st.z[e] = -1.0f;
      st.sg[e] = 0.0f;
    }
    s_z[i] = st.z[e];
  }
  __syncwarp();
  float dl[E];
  ray_alpha<E>(st.z, st.sg, st.valid, S, p.mode, s_z, st.al, dl);
  ray_transmittance<E>(st.al, st.valid, S, p.t_thres, s_f, st.tb, st.proc, st.post);
  return true;
}

template <int E, int CT>
__global__ void __launch_bounds__(256) composite_fwd_kernel(CompParams p) {
  __shared__ float s_zall[8][32 * E];
  __shared__ __align__(16) float s_fall[8][kTransScratch<E>];
  const int lane = lane_id();
  float *s_z = s_zall[threadIdx.x >> 5];
  float *s_f = s_fall[threadIdx.x >> 5];
  const int C = CT > 0 ? CT : p.C;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < p.R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    RayState<E> st;
    float acc[CT > 0 ? CT : kMaxC];
#pragma unroll
    for (int c = 0; c < (CT > 0 ? CT : kMaxC); c++) acc[c] = 0.0f;
    float d = 0.0f, ws = 0.0f, aa = 0.0f;
    bool ok = load_ray<E>(p, r, s_z, s_f, st);
    if (ok) {
      const size_t rb = (size_t)r * p.S;
#pragma unroll
      for (int e = 0; e < E; e++) {
        if (((st.proc & st.valid) >> e) & 1u) {
          float w = st.al[e] * st.tb[e];
          const float *f = p.feats + (rb + st.s[e]) * C;
#pragma unroll
          for (int c = 0; c < (CT > 0 ? CT : kMaxC); c++)
            if (c < C) acc[c] += w * __ldg(f + c);
          d += w * st.z[e];
          ws += w;
          aa += w * st.al[e];
        }
      }
#pragma unroll
      for (int c = 0; c < (CT > 0 ? CT : kMaxC); c++)
        if (c < C) acc[c] = warp_sum(acc[c]);
      d = warp_sum(d);
      ws = warp_sum(ws);
      aa = warp_sum(aa);
    }
    if (lane == 0) {
      p.od[r] = d;
      p.ows[r] = ws;
      p.oa[r] = aa;
    }
    for (int c = lane; c < C; c += 32) {
      float v = 0.0f;
#pragma unroll
      for (int q = 0; q < (CT > 0 ? CT : kMaxC); q++)
        if (q == c) v = acc[q];
      p.of[(size_t)r * C + c] = v;
    }
    __syncwarp();
  }
}

template <int E, int CT>
__global__ void __launch_bounds__(256) composite_bwd_kernel(CompParams p) {
  __shared__ float s_zall[8][32 * E];
  __shared__ __align__(16) float s_fall[8][kTransScratch<E>];
  const int lane = lane_id();
  float *s_z = s_zall[threadIdx.x >> 5];
  float *s_f = s_fall[threadIdx.x >> 5];
  constexpr int CM = CT > 0 ? CT : kMaxCBwd;
  const int C = CT > 0 ? CT : p.C;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < p.R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    RayState<E> st;
    bool ok = load_ray<E>(p, r, s_z, s_f, st);
    const size_t rb = (size_t)r * p.S;
    if (!ok) {
      // invalid ray: no gradient (the reference leaves its zero fill)
      for (int i = lane; i < p.S; i += 32) {
        p.grad_sigma[rb + i] = 0.0f;
        for (int c = 0; c < C; c++) p.grad_feats[(rb + i) * C + c] = 0.0f;
      }
      __syncwarp();
      continue;
    }
    float gc[CM], ofe[CM];
#pragma unroll
    for (int c = 0; c < CM; c++) {
      gc[c] = c < C ? __ldg(p.g_feat + (size_t)r * C + c) : 0.0f;
      ofe[c] = (c < C && !p.exact) ? __ldg(p.of + (size_t)r * C + c) : 0.0f;
    }
    const float gws = __ldg(p.g_ws + r), gd = __ldg(p.g_depth + r), ga = __ldg(p.g_alpha + r);
    // per-position weighted terms and their inclusive prefix sums
    float fv[E][CM];
    float w[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      bool use = ((st.proc & st.valid) >> e) & 1u;
      w[e] = use ? st.al[e] * st.tb[e] : 0.0f;
      const float *f = p.feats + (rb + (st.s[e] >= 0 ? st.s[e] : 0)) * C;
#pragma unroll
      for (int c = 0; c < CM; c++) fv[e][c] = (c < C && st.s[e] >= 0) ? __ldg(f + c) : 0.0f;
    }
    float carry_f[CM], carry_d = 0.0f, carry_w = 0.0f, carry_a = 0.0f;
#pragma unroll
    for (int c = 0; c < CM; c++) carry_f[c] = 0.0f;
    float pf[E][CM], pd[E], pw[E], pa[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
#pragma unroll
      for (int c = 0; c < CM; c++) {
        float v = c < C ? warp_incl_scan_f(w[e] * fv[e][c]) : 0.0f;
        pf[e][c] = carry_f[c] + v;
        carry_f[c] += __shfl_sync(SG_FULL, v, 31);
      }
      float vd = warp_incl_scan_f(w[e] * st.z[e]);
      float vw = warp_incl_scan_f(w[e]);
      float va = warp_incl_scan_f(w[e] * st.al[e]);
      pd[e] = carry_d + vd;
      pw[e] = carry_w + vw;
      pa[e] = carry_a + va;
      carry_d += __shfl_sync(SG_FULL, vd, 31);
      carry_w += __shfl_sync(SG_FULL, vw, 31);
      carry_a += __shfl_sync(SG_FULL, va, 31);
    }
    // totals: saved outputs (reference formula) or recomputed (exact)
    float Ff[CM], Fd, Fw, Fa;
    if (p.exact) {
#pragma unroll
      for (int c = 0; c < CM; c++) Ff[c] = carry_f[c];
      Fd = carry_d;
      Fw = carry_w;
      Fa = carry_a;
    } else {
#pragma unroll
      for (int c = 0; c < CM; c++) Ff[c] = ofe[c];
      Fd = __ldg(p.od + r);
      Fw = __ldg(p.ows + r);
      Fa = __ldg(p.oa + r);
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
      int i = e * 32 + lane;
      if (i >= p.S) continue;
      const int s = st.s[e];
      const bool use = ((st.proc & st.valid) >> e) & 1u;
      const bool wr = p.exact ? use : (use && ((st.post >> e) & 1u));
      float gsig = 0.0f;
      const float al = st.al[e];
      const float Ta = st.tb[e] * (1.0f - al);  // transmittance after the sample
      if (wr) {
        if (!p.exact) {
          if (p.mode == 0) {
            // recover delta: alpha = 1 - exp(-sigma*delta) -> delta from s_z
            float delta = 1e10f;
            if (i != p.S - 1) {
              int m = p.S - 1;
              for (int q = i + 1; q < p.S; q++)
                if (s_z[q] > 0.0f) {
                  m = q;
                  break;
                }
              delta = s_z[m] - st.z[e];
            }
            float tmp = gws * (1.0f - Fw);
            float a = delta * (gws * (Ta * 1.0f - (Fw - pw[e])) + tmp);
            float b = delta * (gd * (Ta * st.z[e] - (Fd - pd[e])) + tmp);
            float c2 = delta * (ga * (2.0f * Ta * al - (Fa - pa[e])) + tmp);
            float f = 0.0f;
#pragma unroll
            for (int c = 0; c < CM; c++)
              if (c < C) f += gc[c] * (Ta * fv[e][c] - (Ff[c] - pf[e][c]));
            f = delta * (f + tmp);
            gsig = a + b + f + c2;
          } else {
            float tmp = (1.0f / (1.0f - al + 1e-7f) <= 15.0f) ? 1.0f / (1.0f - al) : 15.0f;
            float a = gws * (Ta * 1.0f - (Fw - pw[e])) * tmp;
            float b = gd * (Ta * st.z[e] - (Fd - pd[e])) * tmp;
            float c2 = ga * (2.0f * Ta * al - (Fa - pa[e])) * tmp;
            float f = 0.0f;
#pragma unroll
            for (int c = 0; c < CM; c++)
              if (c < C) f += gc[c] * (Ta * fv[e][c] - (Ff[c] - pf[e][c]));
            f *= tmp;
            gsig = a + b + f + c2;
          }
        } else {
          // true derivative; suffix sums after this sample
          float sw = Fw - pw[e], sd = Fd - pd[e], sa = Fa - pa[e];
          if (p.mode == 0) {
            float delta = 1e10f;
            if (i != p.S - 1) {
              int m = p.S - 1;
              for (int q = i + 1; q < p.S; q++)
                if (s_z[q] > 0.0f) {
                  m = q;
                  break;
                }
              delta = s_z[m] - st.z[e];
            }
            float acc = gws * (Ta - sw) + gd * (Ta * st.z[e] - sd) + ga * (2.0f * al * Ta - sa);
#pragma unroll
            for (int c = 0; c < CM; c++)
              if (c < C) acc += gc[c] * (Ta * fv[e][c] - (Ff[c] - pf[e][c]));
            gsig = delta * acc;
          } else {
            float om = 1.0f - al;
            float inv = om != 0.0f ? 1.0f / om : 0.0f;
            float Tb = st.tb[e];
            float acc = gws * (Tb - sw * inv) + gd * (Tb * st.z[e] - sd * inv) + ga * (2.0f * al * Tb - sa * inv);
#pragma unroll
            for (int c = 0; c < CM; c++)
              if (c < C) acc += gc[c] * (Tb * fv[e][c] - (Ff[c] - pf[e][c]) * inv);
            gsig = acc;
          }
        }
      }
      p.grad_sigma[rb + s] = gsig;
      float wv = wr ? w[e] : 0.0f;
      for (int c = 0; c < C; c++) {
        float g = 0.0f;
#pragma unroll
        for (int q = 0; q < CM; q++)
          if (q == c) g = gc[q];
        p.grad_feats[(rb + s) * C + c] = g * wv;
      }
    }
    __syncwarp();
  }
}

template <int CT>
int launch_comp(const CompParams &p, bool bwd, int E, sg_stream_t stream) {
  int g = ceil_div(p.R * 32, 256);
  if (g > num_sms() * 64) g = num_sms() * 64;
#define SG_CASE(EE)                                                              \
  case EE:                                                                       \
    if (bwd) composite_bwd_kernel<EE, CT><<<g, 256, 0, stream>>>(p);             \
    else composite_fwd_kernel<EE, CT><<<g, 256, 0, stream>>>(p);                 \
    break;
  switch (E) {
    SG_CASE(1)
    SG_CASE(2)
    SG_CASE(3)
    SG_CASE(4)
    default:
      return SG_ERR_UNSUPPORTED;
  }
#undef SG_CASE
  return SG_OK;
}

}  // namespace sg

using namespace sg;

static int comp_dispatch(const CompParams &p, bool bwd, sg_stream_t stream) {
  int E = (p.S + 31) / 32;
  if (E < 1 || E > 4) return SG_ERR_UNSUPPORTED;
  int rc = (p.C == 3) ? launch_comp<3>(p, bwd, E, stream) : launch_comp<0>(p, bwd, E, stream);
  if (rc != SG_OK) return rc;
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_composite_fwd(const float *z, const int *sort_idx, const float *sigma, const float *feats,
                                int R, int S, int C, float t_thres, int mode, float *out_feat,
                                float *out_depth, float *out_ws, float *out_alpha, sg_stream_t stream) {
  if (!z || !sigma || !feats || !out_feat || !out_depth || !out_ws || !out_alpha) return SG_ERR_INVALID_ARG;
  if (R < 0 || S <= 0 || C <= 0 || C > kMaxC || (mode != 0 && mode != 1)) return SG_ERR_INVALID_ARG;
  if (R == 0) return SG_OK;
  CompParams p{};
  p.z = z;
  p.sort_idx = sort_idx;
  p.sigma = sigma;
  p.feats = feats;
  p.R = R;
  p.S = S;
  p.C = C;
  p.t_thres = t_thres;
  p.mode = mode;
  p.of = out_feat;
  p.od = out_depth;
  p.ows = out_ws;
  p.oa = out_alpha;
  return comp_dispatch(p, false, stream);
}

extern "C" int sg_composite_bwd(const float *g_feat, const float *g_depth, const float *g_ws,
                                const float *g_alpha, const float *o_feat, const float *o_depth,
                                const float *o_ws, const float *o_alpha, const float *z, const int *sort_idx,
                                const float *sigma, const float *feats, int R, int S, int C, float t_thres,
                                int mode, int exact, float *grad_feats, float *grad_sigma,
                                sg_stream_t stream) {
  if (!g_feat || !g_depth || !g_ws || !g_alpha || !z || !sigma || !feats || !grad_feats || !grad_sigma)
    return SG_ERR_INVALID_ARG;
  if (!exact && (!o_feat || !o_depth || !o_ws || !o_alpha)) return SG_ERR_INVALID_ARG;
  if (R < 0 || S <= 0 || C <= 0 || C > kMaxCBwd || (mode != 0 && mode != 1)) return SG_ERR_INVALID_ARG;
  if (R == 0) return SG_OK;
  CompParams p{};
  p.z = z;
  p.sort_idx = sort_idx;
  p.sigma = sigma;
  p.feats = feats;
  p.R = R;
  p.S = S;
  p.C = C;
  p.t_thres = t_thres;
  p.mode = mode;
  p.of = const_cast<float *>(o_feat);
  p.od = const_cast<float *>(o_depth);
  p.ows = const_cast<float *>(o_ws);
  p.oa = const_cast<float *>(o_alpha);
  p.g_feat = g_feat;
  p.g_depth = g_depth;
  p.g_ws = g_ws;
  p.g_alpha = g_alpha;
  p.exact = exact;
  p.grad_feats = grad_feats;
  p.grad_sigma = grad_sigma;
  return comp_dispatch(p, true, stream);
}
