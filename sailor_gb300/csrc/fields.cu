// fields.cu -- trilinear gathers from dense voxel grids at sampled points.
//
// The reference's trilinear aggregation (sampling_kernel.cu:162-327 of
// SAILOR c_lib/VoxelEncoding/src) interpolates per-node corner features; the
// spec extension gathers from a dense per-voxel grid instead: grid
// [B, D, D, D, C] channel-last, voxel (x, y, z) centred at
// bbox_min + (x, y, z) * voxel_size (the fusion grid's convention), corners
// outside the grid contribute zero.  Sample point = ori + z * dir of its ray;
// samples with z < 0 produce 0.
//
// grid_gather_kernel: one thread per sample; the eight corner reads of
// neighbouring samples of a ray hit the same few cache lines (samples are
// depth-sorted), so HBM traffic is about the touched grid bytes plus the
// 4*C output bytes and 4-byte depth per sample.
//
// mode 1 turns a gathered normalised TSDF t (C == 1) into a density
// sigma = sigmoid(-t * scale / s) / s  (scale = truncation margin in metres,
// s = the density's length scale), so the gather is fused with the field
// transform that feeds compositing.
#include "ray_core.cuh"

namespace sg {

struct GatherParams {
  const float *ori, *dir, *z;
  long R;
  int N, S;
  const float *grid;
  int D, C;
  const float *vol_bbox, *voxel_size;
  int mode;
  float scale, s;
  float *out;
};

template <int C>
__global__ void __launch_bounds__(256) grid_gather_kernel(GatherParams p) {
  const long n = p.R * p.S;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const long r = k / p.S;
    const int b = (int)(r / p.N);
    const float zz = __ldg(p.z + k);
    float acc[C];
#pragma unroll
    for (int c = 0; c < C; c++) acc[c] = 0.0f;
    if (zz >= 0.0f) {
      const float *bb = p.vol_bbox + 6 * b;
      const float bmin[3] = {bb[0], bb[2], bb[4]};
      float pt[3];
#pragma unroll
      for (int a = 0; a < 3; a++) pt[a] = __fmaf_rn(__ldg(p.dir + r * 3 + a), zz, __ldg(p.ori + r * 3 + a));
      grid_tap<C>(p.grid + (size_t)b * p.D * p.D * p.D * C, p.D, bmin, __ldg(p.voxel_size + b), pt, acc);
      if (p.mode == 1) acc[0] = tsdf_density(acc[0], p.scale, p.s);
    }
#pragma unroll
    for (int c = 0; c < C; c++) p.out[k * C + c] = acc[c];
  }
}

}  // namespace sg

using namespace sg;

extern "C" int sg_grid_gather(const float *ori, const float *dir, const float *z, int B, int N, int S,
                              const float *grid, int D, int C, const float *vol_bbox, const float *voxel_size,
                              int mode, float scale, float s, float *out, sg_stream_t stream) {
  if (!ori || !dir || !z || !grid || !vol_bbox || !voxel_size || !out) return SG_ERR_INVALID_ARG;
  if (B <= 0 || N <= 0 || S <= 0 || D <= 0 || C <= 0 || C > 16) return SG_ERR_INVALID_ARG;
  if (mode == 1 && (C != 1 || s == 0.0f)) return SG_ERR_INVALID_ARG;
  GatherParams p{ori, dir, z, (long)B * N, N, S, grid, D, C, vol_bbox, voxel_size, mode, scale, s, out};
  long n = (long)B * N * S;
  int g = ceil_div(n, 256);
  if (g > 152 * 64) g = 152 * 64;
  switch (C) {
    case 1: grid_gather_kernel<1><<<g, 256, 0, stream>>>(p); break;
    case 3: grid_gather_kernel<3><<<g, 256, 0, stream>>>(p); break;
    case 4: grid_gather_kernel<4><<<g, 256, 0, stream>>>(p); break;
    case 8: grid_gather_kernel<8><<<g, 256, 0, stream>>>(p); break;
    case 16: grid_gather_kernel<16><<<g, 256, 0, stream>>>(p); break;
    default: return SG_ERR_UNSUPPORTED;
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}
