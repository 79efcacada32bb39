// trilerp.cu -- trilinear aggregation at sampled points on sm_103a.
//
// Node-corner aggregation replaces trilinear_aggregate_features_kernel and
// its backward (sampling_kernel.cu:162-327 of SAILOR
// c_lib/VoxelEncoding/src; hosts :1384-1462): the eight corners of the node
// that holds each sample are recomputed from the node key (the reference
// copies the whole ~1.1 KB node per (sample, channel) thread).  One thread
// per (frame, channel, ray, sample); the 8 corner features of a thread are
// two 16-byte loads.  The reference interpolates x then y then z with the
// y/z weights formed in double; here they are formed in float (the corner
// coordinates along an axis coincide pairwise, so every pair weight is the
// same per axis).
#include "common.cuh"

namespace sg {

struct TriParams {
  SgTree t;
  const float *ori, *dir, *z;
  const int *idx;
  const float *feats, *gout;
  float *out, *gin;
  int N, S, C;
};

// weights along x, y, z of a sample in the node's cube
__device__ __forceinline__ bool node_weights(const TriParams &p, int b, long rs, float &tx, float &ty,
                                             float &tz) {
  int id = p.idx[rs];
  if (id == -1) return false;
  const SgTree &t = p.t;
  const float *bb = t.vol_bbox + 6 * b;
  const float vs = t.voxel_size[b];
  int ix, iy, iz;
  LevelGeom g;
  if (id >= t.base_top) {
    long key = t.top_key[id - t.base_top];
    long vt = (long)t.Dt * t.Dt * t.Dt;
    long l = key % vt;
    ix = (int)(l / ((long)t.Dt * t.Dt));
    iy = (int)((l / t.Dt) % t.Dt);
    iz = (int)(l % t.Dt);
    g = level_geom(vs, t.Db / t.Dt);
  } else {
    long key = t.bot_key[id - t.base_bot];
    long vb = (long)t.Db * t.Db * t.Db;
    long l = key % vb;
    ix = (int)(l / ((long)t.Db * t.Db));
    iy = (int)((l / t.Db) % t.Db);
    iz = (int)(l % t.Db);
    g = level_geom(vs, 1);
  }
  float cx = node_coord(g, bb[0], ix), cy = node_coord(g, bb[2], iy), cz = node_coord(g, bb[4], iz);
  float h = g.vs / 2.0f;
  long r = rs / p.S;
  float zz = p.z[rs];
  float px = __fmaf_rn(p.dir[r * 3 + 0], zz, p.ori[r * 3 + 0]);
  float py = __fmaf_rn(p.dir[r * 3 + 1], zz, p.ori[r * 3 + 1]);
  float pz = __fmaf_rn(p.dir[r * 3 + 2], zz, p.ori[r * 3 + 2]);
  float x0 = cx - h, x1 = cx + h, y0 = cy - h, y1 = cy + h, z0 = cz - h, z1 = cz + h;
  tx = (px - x0) / (x1 - x0);
  ty = (py - y0) / (y1 - y0);
  tz = (pz - z0) / (z1 - z0);
  return true;
}

// feats [B,C,N,S,8] -> out [B,C,N,S]; corner order of calculate_xyz_corners
// (octree.h:120-129): c = kx*4 + ky*2 + kz
__global__ void trilerp_nodes_fwd_kernel(TriParams p) {
  long n = (long)p.t.B * p.C * p.N * p.S;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    long NS = (long)p.N * p.S;
    int b = (int)(k / ((long)p.C * NS));
    long rs = (long)b * NS + (k % NS);
    float tx, ty, tz;
    if (!node_weights(p, b, rs, tx, ty, tz)) continue;  // output left as given (reference: zeros)
    const float4 *f4 = reinterpret_cast<const float4 *>(p.feats + k * 8);
    float4 a = __ldg(f4), c = __ldg(f4 + 1);
    // a = f0..f3 (x-), c = f4..f7 (x+)
    float x04 = a.x * (1.0f - tx) + c.x * tx;
    float x15 = a.y * (1.0f - tx) + c.y * tx;
    float x26 = a.z * (1.0f - tx) + c.z * tx;
    float x37 = a.w * (1.0f - tx) + c.w * tx;
    float y0 = x04 * (1.0f - ty) + x26 * ty;
    float y1 = x15 * (1.0f - ty) + x37 * ty;
    p.out[k] = y0 * (1.0f - tz) + y1 * tz;
  }
}

__global__ void trilerp_nodes_bwd_kernel(TriParams p) {
  long n = (long)p.t.B * p.C * p.N * p.S;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    long NS = (long)p.N * p.S;
    int b = (int)(k / ((long)p.C * NS));
    long rs = (long)b * NS + (k % NS);
    float tx, ty, tz;
    float4 *g4 = reinterpret_cast<float4 *>(p.gin + k * 8);
    if (!node_weights(p, b, rs, tx, ty, tz)) {
      g4[0] = make_float4(0.f, 0.f, 0.f, 0.f);
      g4[1] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    float g = p.gout[k];
    float ux = 1.0f - tx, uy = 1.0f - ty, uz = 1.0f - tz;
    g4[0] = make_float4(g * (ux * uy * uz), g * (ux * uy * tz), g * (ux * ty * uz), g * (ux * ty * tz));
    g4[1] = make_float4(g * (tx * uy * uz), g * (tx * uy * tz), g * (tx * ty * uz), g * (tx * ty * tz));
  }
}

}  // namespace sg

using namespace sg;

static int tri_launch(const SgTree *tree, const float *ori, const float *dir, const float *z, const int *idx,
                      const float *feats, const float *gout, int N, int S, int C, float *out, float *gin,
                      bool bwd, sg_stream_t stream) {
  if (!tree || !ori || !dir || !z || !idx) return SG_ERR_INVALID_ARG;
  if (N <= 0 || S <= 0 || C <= 0 || tree->B <= 0) return SG_ERR_INVALID_ARG;
  TriParams p{*tree, ori, dir, z, idx, feats, gout, out, gin, N, S, C};
  long n = (long)tree->B * C * N * S;
  int g = ceil_div(n, 256);
  if (g > num_sms() * 64) g = num_sms() * 64;
  if (bwd) trilerp_nodes_bwd_kernel<<<g, 256, 0, stream>>>(p);
  else trilerp_nodes_fwd_kernel<<<g, 256, 0, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_trilerp_nodes_fwd(const SgTree *tree, const float *ori, const float *dir, const float *z,
                                    const int *idx, const float *feats, int N, int S, int C, float *out,
                                    sg_stream_t stream) {
  if (!feats || !out || ((uintptr_t)feats) % 16) return SG_ERR_INVALID_ARG;
  return tri_launch(tree, ori, dir, z, idx, feats, nullptr, N, S, C, out, nullptr, false, stream);
}

extern "C" int sg_trilerp_nodes_bwd(const SgTree *tree, const float *ori, const float *dir, const float *z,
                                    const int *idx, const float *gout, int N, int S, int C, float *gin,
                                    sg_stream_t stream) {
  if (!gout || !gin || ((uintptr_t)gin) % 16) return SG_ERR_INVALID_ARG;
  return tri_launch(tree, ori, dir, z, idx, nullptr, gout, N, S, C, nullptr, gin, true, stream);
}
