// render.cu -- fused per-ray render: sampling -> sort -> field taps -> compositing.
//
// One warp per ray does, without leaving the SM:
//   the reference's coarse sampling (ray_voxels_sampling_uniform_kernel,
//   sampling_kernel.cu:1070-1177) into shared memory, the per-ray sort
//   (sort_samplings :1308-1329) in registers, per-sample density from the
//   fused TSDF grid and colour from a dense RGB grid (trilinear taps; the
//   stand-in for SRONet's MLP), and density compositing of the sorted
//   samples (volume_rendering_training_forward_kernel, volume_rendering.cu:
//   17-126, with the transmittance carried in strict sample order).
// Only 24 bytes per ray are written (rgb, depth, weight sum, alpha); the
// sorted depths / node ids are written only when requested.  The results
// equal the unfused chain sg_sample_sorted -> sg_grid_gather (x2) ->
// sg_composite_fwd on the same inputs (same operations, same order).
#include "ray_core.cuh"

namespace sg {

struct RenderParams {
  SampleParams sp;
  const int *hit_count;
  float rand_const;
  const float *ori, *dir;
  const float *tsdf;
  int D;
  float sdf_scale, sdf_s;
  const float *cgrid;
  int Dc;
  const float *cbbox, *cvs;
  float t_thres;
  float *out_rgb, *out_depth, *out_ws, *out_alpha;
  float *out_z;
  int *out_node;
};

template <int E>
__global__ void __launch_bounds__(256) render_kernel(RenderParams p) {
  __shared__ __align__(16) float s_zall[8][32 * E];
  __shared__ __align__(16) float s_fall[8][32 * E];
  __shared__ int s_iall[8][32 * E];
  __shared__ int s_pall[8][32 * E];
  __shared__ SampleScratch s_sc[8];
  const int lane = lane_id(), w8 = threadIdx.x >> 5;
  float *s_z = s_zall[w8];
  int *s_i = s_iall[w8], *s_p = s_pall[w8];
  const SampleParams &sp = p.sp;
  const long R = (long)sp.t.B * sp.N;
  const int S = sp.S;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    const int b = (int)(r / sp.N);
    const int nh = p.hit_count ? min(p.hit_count[r], sp.W) : sp.W;
    const int done = warp_sample_ray(sp, r, nh, p.rand_const, s_z, s_i, s_sc[w8]);
    float acc_r = 0.0f, acc_g = 0.0f, acc_b = 0.0f, d = 0.0f, ws = 0.0f, aa = 0.0f;
    if (done == 0) {
      // no sample: a ray whose largest depth is < 0 renders 0
      if (p.out_z) {
        for (int i = lane; i < S; i += 32) {
          p.out_z[(size_t)r * S + i] = -1.0f;
          p.out_node[(size_t)r * S + i] = -1;
        }
      }
    } else {
      warp_sort_samples(s_z, s_p, S, done);
      float z[E];
      int node[E];
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int i = e * 32 + lane;
        z[e] = (i < S) ? s_z[i] : -1.0f;
        node[e] = (i < S) ? s_i[s_p[i]] : -1;
      }
      if (p.out_z) {
#pragma unroll
        for (int e = 0; e < E; e++) {
          const int i = e * 32 + lane;
          if (i < S) {
            p.out_z[(size_t)r * S + i] = z[e];
            p.out_node[(size_t)r * S + i] = node[e];
          }
        }
      }
      const float *bb = sp.t.vol_bbox + 6 * b;
      const float bmin[3] = {bb[0], bb[2], bb[4]};
      const float vs = __ldg(sp.t.voxel_size + b);
      const float *cb = p.cbbox + 6 * b;
      const float cmin[3] = {cb[0], cb[2], cb[4]};
      const float cvs = __ldg(p.cvs + b);
      const float *tsdf = p.tsdf + (size_t)b * p.D * p.D * p.D;
      const float *cgrid = p.cgrid + (size_t)b * p.Dc * p.Dc * p.Dc * 3;
      const float o[3] = {__ldg(p.ori + r * 3), __ldg(p.ori + r * 3 + 1), __ldg(p.ori + r * 3 + 2)};
      const float dr[3] = {__ldg(p.dir + r * 3), __ldg(p.dir + r * 3 + 1), __ldg(p.dir + r * 3 + 2)};
      unsigned valid = 0;
      float sg[E], rgb[E][3];
#pragma unroll
      for (int e = 0; e < E; e++) {
        sg[e] = 0.0f;
        rgb[e][0] = rgb[e][1] = rgb[e][2] = 0.0f;
        if (z[e] >= 0.0f) {
          valid |= 1u << e;
          const float pt[3] = {__fmaf_rn(dr[0], z[e], o[0]), __fmaf_rn(dr[1], z[e], o[1]),
                               __fmaf_rn(dr[2], z[e], o[2])};
          float t1[1];
          grid_tap<1>(tsdf, p.D, bmin, vs, pt, t1);
          sg[e] = tsdf_density(t1[0], p.sdf_scale, p.sdf_s);
          grid_tap<3>(cgrid, p.Dc, cmin, cvs, pt, rgb[e]);
        }
      }
      float al[E], tb[E];
      unsigned proc, post;
      ray_alpha<E>(z, sg, valid, S, 0, s_z, al);
      ray_transmittance<E>(al, valid, S, p.t_thres, s_fall[w8], tb, proc, post);
#pragma unroll
      for (int e = 0; e < E; e++) {
        if (((proc & valid) >> e) & 1u) {
          const float w = al[e] * tb[e];
          acc_r += w * rgb[e][0];
          acc_g += w * rgb[e][1];
          acc_b += w * rgb[e][2];
          d += w * z[e];
          ws += w;
          aa += w * al[e];
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
  RenderParams p;
  p.sp = SampleParams{*tree, hit_idx, hit_t0, hit_t1, rands, valid_len, N, W, S, num_levels, start_level,
                      nullptr, nullptr};
  p.hit_count = hit_count;
  p.rand_const = rand_const;
  p.ori = ori;
  p.dir = dir;
  p.tsdf = tsdf;
  p.D = D;
  p.sdf_scale = sdf_scale;
  p.sdf_s = sdf_s;
  p.cgrid = color_grid;
  p.Dc = Dc;
  p.cbbox = color_bbox;
  p.cvs = color_vs;
  p.t_thres = t_thres;
  p.out_rgb = out_rgb;
  p.out_depth = out_depth;
  p.out_ws = out_ws;
  p.out_alpha = out_alpha;
  p.out_z = out_z;
  p.out_node = out_node;
  long R = (long)tree->B * N;
  int g = ceil_div(R * 32, 256);
  if (g > 152 * tune(SG_TUNE_RENDER_WARPS)) g = 152 * tune(SG_TUNE_RENDER_WARPS);
  if (S <= 32) render_kernel<1><<<g, 256, 0, stream>>>(p);
  else if (S <= 64) render_kernel<2><<<g, 256, 0, stream>>>(p);
  else if (S <= 128) render_kernel<4><<<g, 256, 0, stream>>>(p);
  else return SG_ERR_UNSUPPORTED;
  SG_LAUNCH_CHECK();
  return SG_OK;
}
