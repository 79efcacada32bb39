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
// grid_scatter_kernel (the adjoint): one warp per ray walks the ray's
// samples in order; lane l owns the (corner, channel) slots l, l+32, ... of
// the 8*C values a trilinear cell receives.  While consecutive samples stay in
// one cell their contributions w_corner * g_channel accumulate in registers;
// at a cell change (and at the end of the ray) the slots are flushed with one
// atomic add each, C consecutive lanes covering one corner's C contiguous
// channels.  Samples of a ray are depth-sorted and cluster in the few hit
// voxels, so a flush carries many samples.
//
// mode 1 turns a gathered normalised TSDF t (C == 1) into a density
// sigma = sigmoid(-t * scale / s) / s  (scale = truncation margin in metres,
// s = the density's length scale), so the gather is fused with the field
// transform that feeds compositing.
#include <climits>

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
      grid_tap<C>(p.grid + (size_t)b * p.D * p.D * p.D * C, p.D, bmin, __ldg(p.voxel_size + b),
                  1.0f / __ldg(p.voxel_size + b), pt, acc);
      if (p.mode == 1) acc[0] = tsdf_density(acc[0], p.scale / p.s, 1.0f / p.s);
    }
#pragma unroll
    for (int c = 0; c < C; c++) p.out[k * C + c] = acc[c];
  }
}


struct ScatterParams {
  const float *ori, *dir, *z;
  long R;
  int N, S;
  const float *gout;   // [R, S, C]
  const float *grid;   // mode 1: the TSDF grid the forward gathered from
  int D;
  const float *vol_bbox, *voxel_size;
  int mode;
  float scale, s;
  float *ggrid;        // [B, D, D, D, C], accumulated
};

template <int C>
__device__ __forceinline__ void scatter_flush(const ScatterParams &p, int b, const int cell[3],
                                              const float (&acc)[(8 * C + 31) / 32]) {
  constexpr int NSLOT = (8 * C + 31) / 32;
  const int lane = lane_id();
#pragma unroll
  for (int q = 0; q < NSLOT; q++) {
    const int slot = lane + 32 * q;
    if (slot >= 8 * C || acc[q] == 0.0f) continue;
    const int cr = slot / C, ch = slot - cr * C;
    const int ix = cell[0] + ((cr >> 2) & 1), iy = cell[1] + ((cr >> 1) & 1), iz = cell[2] + (cr & 1);
    if (ix < 0 || iy < 0 || iz < 0 || ix >= p.D || iy >= p.D || iz >= p.D) continue;
    atomicAdd(p.ggrid + ((((size_t)b * p.D + ix) * p.D + iy) * p.D + iz) * C + ch, acc[q]);
  }
}

template <int C>
__global__ void __launch_bounds__(256) grid_scatter_kernel(ScatterParams p) {
  constexpr int NSLOT = (8 * C + 31) / 32;
  __shared__ float s_w[8][32][9];      // padded rows: conflict-free per-lane writes
  __shared__ float s_g[8][32][C + 1];
  __shared__ int s_cell[8][32][5];
  const int lane = lane_id(), w8 = threadIdx.x >> 5;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < p.R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    const int b = (int)(r / p.N);
    const float *bb = p.vol_bbox + 6 * b;
    const float bmin[3] = {bb[0], bb[2], bb[4]};
    const float vs = __ldg(p.voxel_size + b);
    const float inv_vs = 1.0f / vs;
    float acc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; q++) acc[q] = 0.0f;
    int cur[3] = {INT_MIN, 0, 0};
    for (int c0 = 0; c0 < p.S; c0 += 32) {
      // per sample: cell, corner weights (as the forward tap forms them) and gradient
      const int i = c0 + lane;
      const float zz = i < p.S ? __ldg(p.z + r * p.S + i) : -1.0f;
      int valid = 0;
      if (zz >= 0.0f) {
        float pt[3], wc[8];
        int i0[3];
#pragma unroll
        for (int a = 0; a < 3; a++) pt[a] = __fmaf_rn(__ldg(p.dir + r * 3 + a), zz, __ldg(p.ori + r * 3 + a));
        tap_cell(bmin, vs, inv_vs, pt, i0, wc);
#pragma unroll
        for (int cr = 0; cr < 8; cr++) s_w[w8][lane][cr] = wc[cr];
        s_cell[w8][lane][0] = i0[0];
        s_cell[w8][lane][1] = i0[1];
        s_cell[w8][lane][2] = i0[2];
        const float *g = p.gout + ((size_t)r * p.S + i) * C;
        if (p.mode == 1) {
          // d sigma / d t of sigma = sigmoid(-t scale / s) / s at the gathered t
          float t1[1];
          grid_tap_cell<1>(p.grid + (size_t)b * p.D * p.D * p.D, p.D, i0, wc, t1);
          const float k = p.scale / p.s;
          const float sg = tsdf_sigmoid(t1[0], k);
          s_g[w8][lane][0] = __ldg(g) * (-sg * (1.0f - sg) * (k * (1.0f / p.s)));
        } else {
#pragma unroll
          for (int c = 0; c < C; c++) s_g[w8][lane][c] = __ldg(g + c);
        }
        valid = 1;
      }
      s_cell[w8][lane][3] = valid;
      __syncwarp();
      const int n = min(32, p.S - c0);
      for (int j = 0; j < n; j++) {
        if (!s_cell[w8][j][3]) continue;
        const int cj[3] = {s_cell[w8][j][0], s_cell[w8][j][1], s_cell[w8][j][2]};
        if (cj[0] != cur[0] || cj[1] != cur[1] || cj[2] != cur[2]) {
          if (cur[0] != INT_MIN) scatter_flush<C>(p, b, cur, acc);
#pragma unroll
          for (int q = 0; q < NSLOT; q++) acc[q] = 0.0f;
          cur[0] = cj[0];
          cur[1] = cj[1];
          cur[2] = cj[2];
        }
#pragma unroll
        for (int q = 0; q < NSLOT; q++) {
          const int slot = lane + 32 * q;
          if (slot < 8 * C) {
            const int cr = slot / C, ch = slot - cr * C;
            acc[q] = __fmaf_rn(s_w[w8][j][cr], s_g[w8][j][ch], acc[q]);
          }
        }
      }
      __syncwarp();
    }
    if (cur[0] != INT_MIN) scatter_flush<C>(p, b, cur, acc);
  }
}

// Zero of the part of a gradient grid [B, Db, Db, Db, C] (the tree's fine
// geometry) that a training pass over the tree's nodes can write: a CTA per
// top brick tests the brick's 26-neighbourhood for a node and, if it finds
// one, clears the brick's rate^3 voxels (rate z-runs of rate * C floats).
__global__ void __launch_bounds__(256) zero_near_nodes_kernel(SgTree t, float *grid, int C, int vec4) {
  const int b = blockIdx.y, Dt = t.Dt;
  const long vt = (long)Dt * Dt * Dt;
  const long brick = blockIdx.x;
  const int X = (int)(brick / ((long)Dt * Dt)), Y = (int)((brick / Dt) % Dt), Z = (int)(brick % Dt);
  int near = 0;
  if (threadIdx.x < 27) {
    const int x = X + (int)threadIdx.x / 9 - 1, y = Y + ((int)threadIdx.x / 3) % 3 - 1, z = Z + (int)threadIdx.x % 3 - 1;
    if (x >= 0 && y >= 0 && z >= 0 && x < Dt && y < Dt && z < Dt)
      near = __ldg(t.brick_node + b * vt + ((long)x * Dt + y) * Dt + z) >= 0;
  }
  if (!__syncthreads_or(near)) return;
  const int r = t.rate, Db = t.Db;
  const int per_run = vec4 ? r * C / 4 : r * C;  // stores per z-run
  float *g = grid + (size_t)b * Db * Db * Db * C;
  for (int i = threadIdx.x; i < r * r * per_run; i += blockDim.x) {
    const int xy = i / per_run, k = i - xy * per_run;
    const int x = X * r + xy / r, y = Y * r + xy % r;
    const size_t off = (((size_t)x * Db + y) * Db + (size_t)Z * r) * C;
    if (vec4) reinterpret_cast<float4 *>(g + off)[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    else g[off + k] = 0.0f;
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
  if (g > num_sms() * 64) g = num_sms() * 64;
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

extern "C" int sg_grid_scatter(const float *ori, const float *dir, const float *z, int B, int N, int S,
                               const float *grad_out, const float *grid, int D, int C, const float *vol_bbox,
                               const float *voxel_size, int mode, float scale, float s, float *grad_grid,
                               sg_stream_t stream) {
  if (!ori || !dir || !z || !grad_out || !vol_bbox || !voxel_size || !grad_grid) return SG_ERR_INVALID_ARG;
  if (B <= 0 || N <= 0 || S <= 0 || D <= 0 || C <= 0 || C > 16) return SG_ERR_INVALID_ARG;
  if (mode == 1 && (C != 1 || s == 0.0f || !grid)) return SG_ERR_INVALID_ARG;
  if (mode != 0 && mode != 1) return SG_ERR_INVALID_ARG;
  ScatterParams p{ori, dir, z, (long)B * N, N, S, grad_out, grid, D, vol_bbox, voxel_size, mode, scale, s,
                  grad_grid};
  long R = (long)B * N;
  int g = ceil_div(R * 32, 256);
  if (g > num_sms() * 32) g = num_sms() * 32;
  switch (C) {
    case 1: grid_scatter_kernel<1><<<g, 256, 0, stream>>>(p); break;
    case 3: grid_scatter_kernel<3><<<g, 256, 0, stream>>>(p); break;
    case 4: grid_scatter_kernel<4><<<g, 256, 0, stream>>>(p); break;
    case 8: grid_scatter_kernel<8><<<g, 256, 0, stream>>>(p); break;
    case 16: grid_scatter_kernel<16><<<g, 256, 0, stream>>>(p); break;
    default: return SG_ERR_UNSUPPORTED;
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_zero_near_nodes(const SgTree *tree, float *grid, int C, sg_stream_t stream) {
  if (!tree || !tree->brick_node || !grid) return SG_ERR_INVALID_ARG;
  if (tree->B <= 0 || tree->Dt <= 0 || tree->rate <= 0 || tree->Db != tree->Dt * tree->rate || C <= 0)
    return SG_ERR_INVALID_ARG;
  const long vt = (long)tree->Dt * tree->Dt * tree->Dt;
  if (vt > INT_MAX || tree->B > 65535) return SG_ERR_UNSUPPORTED;
  const int vec4 = ((tree->rate * C) % 4 == 0 && ((uintptr_t)grid) % 16 == 0) ? 1 : 0;
  zero_near_nodes_kernel<<<dim3((unsigned)vt, tree->B), 256, 0, stream>>>(*tree, grid, C, vec4);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
