// project.cu -- projection of sample points into the source views and the
// bilinear gather of per-view 2D feature maps at the projections (the step
// after sampling in SRONet), on sm_103a.
//
// sg_project_sampled_xyz replaces project_xyz (c_lib/VoxelEncoding/src/
// sampling_kernel.cu:55-159) behind MultiLayerOctree::project_sampled_xyz
// (:1333-1381): every (frame, view, ray, sample) is projected, optionally
// with the eight corners of the sample's node; one thread per item, the
// -1 of samples without a node written by the same pass (the reference
// pre-fills the whole output with torch::full first).
//
// sg_project_gather replaces proj_persp (utils_render/utils_render.py:
// 380-414) and the four F.grid_sample calls plus the clamped depth
// difference of BasicRenNet.forward_sample_feature (SRONet/BasicRenNet.py:
// 245-259): one thread per (view image, point) projects the point, writes
// the projection outputs that are asked for, and gathers up to four feature
// maps bilinearly (align_corners=True, zero padding) straight into the
// channel-last [view image, point, C] layout the reference produces with
// permute + contiguous.  Maps are read through strides, so NCHW and
// channels-last tensors both work; channels-last maps with C % 4 == 0 are
// gathered by lane groups with 16-byte loads of whole texel rows and
// 16-byte stores of whole output rows (a warp covers 32 items, four at a
// time), the others item by item.
#include <climits>

#include "common.cuh"

namespace sg {

// ---------------------------------------------------------------------------
// project_xyz
// ---------------------------------------------------------------------------
struct ProjSampledParams {
  SgTree t;
  const float *ori, *dir, *z;
  const int *idx;
  const float *K, *RT;
  int B, Nv, N, S;
  float cw, ch;  // ori_w / 2, ori_h / 2
  int corners;
  float *xy, *pz;
};

// (x - c) / c as the reference evaluates it (in double precision, stored as
// float; c = size / 2 is exact): the difference as an exact float pair
// (two_sum), the quotient of its leading part, and one correction from the
// exact remainder of that quotient.  Equal to the reference's value except
// where the exact quotient lies within about 2^-29 ulp of a rounding
// boundary; with c a power of two the difference of two floats is exact
// after scaling and the result is the reference's exactly.
__device__ __forceinline__ float grid_coord(float x, float c) {
  float dh, dl;
  two_sum(x, -c, dh, dl);
  const float q = dh / c;
  const float r = __fmaf_rn(-q, c, dh);  // dh - q c, exact
  return q + (r + dl) / c;
}

// camera point and normalised pixel of world point p in view (K, RT): the
// reference's expressions with the operand order nvcc gives them
// (project_xyz, sampling_kernel.cu:103-116)
__device__ __forceinline__ void project_point(const float *__restrict__ K, const float *__restrict__ P, float px,
                                              float py, float pz, float cw, float ch, float &gx, float &gy,
                                              float &cz) {
  const float cx = __fmaf_rn(P[2], pz, __fmaf_rn(P[0], px, P[1] * py)) + P[3];
  const float cy = __fmaf_rn(P[6], pz, __fmaf_rn(P[4], px, P[5] * py)) + P[7];
  cz = __fmaf_rn(P[10], pz, __fmaf_rn(P[8], px, P[9] * py)) + P[11];
  const float ux = dot3c(K[0], K[1], K[2], cx, cy, cz);
  const float uy = dot3c(K[3], K[4], K[5], cx, cy, cz);
  const float uz = dot3c(K[6], K[7], K[8], cx, cy, cz);
  gx = grid_coord(ux / uz, cw);
  gy = grid_coord(uy / uz, ch);
}

// Centre and edge of node g (a top brick or a fine voxel of the tree), as
// OcTree::calculate_xyz_corners places it (octree.h:109-129); false when g is
// not a node.
__device__ __forceinline__ bool node_centre(const SgTree &t, int g, float c[3], float &vs) {
  int ix, iy, iz, b, size;
  if (g >= t.base_top && g < t.base_top + t.counts[0]) {
    const long key = t.top_key[g - t.base_top];
    const long vt = (long)t.Dt * t.Dt * t.Dt;
    b = (int)(key / vt);
    const long l = key - (long)b * vt;
    ix = (int)(l / ((long)t.Dt * t.Dt)), iy = (int)((l / t.Dt) % t.Dt), iz = (int)(l % t.Dt);
    size = t.Db / t.Dt;
  } else if (g >= t.base_bot && g < t.base_bot + t.counts[1]) {
    const long key = t.bot_key[g - t.base_bot];
    const long vb = (long)t.Db * t.Db * t.Db;
    b = (int)(key / vb);
    const long l = key - (long)b * vb;
    ix = (int)(l / ((long)t.Db * t.Db)), iy = (int)((l / t.Db) % t.Db), iz = (int)(l % t.Db);
    size = 1;
  } else {
    return false;
  }
  const LevelGeom lg = level_geom(t.voxel_size[b], size);
  const float *bb = t.vol_bbox + 6 * b;
  c[0] = node_coord(lg, bb[0], ix);
  c[1] = node_coord(lg, bb[2], iy);
  c[2] = node_coord(lg, bb[4], iz);
  vs = lg.vs;
  return true;
}

__global__ void __launch_bounds__(256) project_sampled_kernel(ProjSampledParams p) {
  const long total = (long)p.B * p.Nv * p.N * p.S;
  const int per = p.corners ? 9 : 1;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (long)gridDim.x * blockDim.x) {
    const long rs = k % ((long)p.N * p.S);  // ray * S + sample
    const long bv = k / ((long)p.N * p.S);  // frame * Nv + view
    const int b = (int)(bv / p.Nv);
    const long si = (long)b * p.N * p.S + rs;
    float *xy = p.xy + k * (2 * per);
    float *oz = p.pz + k * per;
    const int id = __ldg(p.idx + si);
    if (id == -1) {  // no node: the reference's -1 fill stays
      for (int i = 0; i < per; i++) {
        xy[2 * i] = -1.0f;
        xy[2 * i + 1] = -1.0f;
        oz[i] = -1.0f;
      }
      continue;
    }
    const long r = rs / p.S;
    const float zs = __ldg(p.z + si);
    const float *o = p.ori + ((long)b * p.N + r) * 3, *d = p.dir + ((long)b * p.N + r) * 3;
    const float px = __fmaf_rn(__ldg(d), zs, __ldg(o));
    const float py = __fmaf_rn(__ldg(d + 1), zs, __ldg(o + 1));
    const float pz = __fmaf_rn(__ldg(d + 2), zs, __ldg(o + 2));
    const float *K = p.K + bv * 9, *P = p.RT + bv * 12;
    float gx, gy, cz;
    project_point(K, P, px, py, pz, p.cw, p.ch, gx, gy, cz);
    xy[0] = gx;
    xy[1] = gy;
    oz[0] = cz;
    if (!p.corners) continue;
    float c[3], vs;
    if (!node_centre(p.t, id, c, vs)) {  // not a node of this tree
      for (int i = 1; i < 9; i++) {
        xy[2 * i] = -1.0f;
        xy[2 * i + 1] = -1.0f;
        oz[i] = -1.0f;
      }
      continue;
    }
    const float h = vs / 2.0f;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const float qx = c[0] + ((i & 4) ? h : -h), qy = c[1] + ((i & 2) ? h : -h), qz = c[2] + ((i & 1) ? h : -h);
      project_point(K, P, qx, qy, qz, p.cw, p.ch, gx, gy, cz);
      xy[2 * (i + 1)] = gx;
      xy[2 * (i + 1) + 1] = gy;
      oz[i + 1] = cz;
    }
  }
}

// ---------------------------------------------------------------------------
// proj_persp + grid_sample
// ---------------------------------------------------------------------------
constexpr int kMaxMaps = 4;

struct GatherMap {
  const float *data;
  long sn, sc, sy, sx;  // element strides of [view image, channel, y, x]
  int C, H, W, vec4;    // vec4: channels contiguous, C % 4 == 0, 16-byte aligned
  float *out;           // [view image, N, C]
};

struct ProjGatherParams {
  const float *gin, *din;  // given grids [BV, N, 2] and depths [BV, N] (gin null: project pts)
  const float *pts;
  long pb, pa, pn;  // element strides of points [batch, axis, point]
  int pt_div;       // point batch = view image / pt_div
  const float *pdep;
  long db, dn;      // p_depths [batch, 1, point] strides (pdep may be null)
  const float *K, *R, *T;
  int BV, N;
  float depth_thres, min_d, max_d, half_res;
  float *ori_pts, *grids, *depth;  // [BV, 3, N], [BV, 2, N], [BV, 1, N]; each may be null
  GatherMap maps[kMaxMaps];
  int n_maps;
  int groups;                      // channels-last maps share map 0's size: lane-group gathers
  int psdf_map;                    // map holding depth for psdf (-1: none)
  float psdf_clip, psdf_scale;
  float *psdf;                     // [BV, N, 1]
};

// Bilinear footprint of a grid point on an H x W image (F.grid_sample,
// align_corners=True, zero padding): the nw corner (x0, y0), the weights of
// the corners nw, ne, sw, se, and a 4-bit mask of the corners inside the
// image (NaN or far-out coordinates have none).
struct Foot {
  float w[4];
  int x0, y0, mask;
};

__device__ __forceinline__ Foot footprint(int H, int W, float gx, float gy) {
  Foot f;
  const float ix = ((gx + 1.0f) / 2.0f) * (float)(W - 1);
  const float iy = ((gy + 1.0f) / 2.0f) * (float)(H - 1);
  const float x0 = floorf(ix), y0 = floorf(iy);
  const float x1 = x0 + 1.0f, y1 = y0 + 1.0f;
  f.w[0] = (x1 - ix) * (y1 - iy);
  f.w[1] = (ix - x0) * (y1 - iy);
  f.w[2] = (x1 - ix) * (iy - y0);
  f.w[3] = (ix - x0) * (iy - y0);
  const bool xa = x0 >= 0.0f && x0 <= (float)(W - 1), xb = x1 >= 0.0f && x1 <= (float)(W - 1);
  const bool ya = y0 >= 0.0f && y0 <= (float)(H - 1), yb = y1 >= 0.0f && y1 <= (float)(H - 1);
  f.mask = (xa && ya ? 1 : 0) | (xb && ya ? 2 : 0) | (xa && yb ? 4 : 0) | (xb && yb ? 8 : 0);
  f.x0 = f.mask ? (int)x0 : 0;  // in [-1, W - 1] when any corner is inside
  f.y0 = f.mask ? (int)y0 : 0;
  return f;
}

// element offset of corner i (nw, ne, sw, se) of footprint (x0, y0) in image img
__device__ __forceinline__ long corner_off(const GatherMap &m, int img, int x0, int y0, int i) {
  return (long)img * m.sn + (long)(y0 + (i >> 1)) * m.sy + (long)(x0 + (i & 1)) * m.sx;
}

// Per-item gather of a map that is not read in lane groups: channel by
// channel through the channel stride.  Returns channel 0.
__device__ __forceinline__ float gather_map(const GatherMap &m, int img, long k, const Foot &f) {
  float *out = m.out + k * m.C;
  long off[4];
#pragma unroll
  for (int i = 0; i < 4; i++) off[i] = corner_off(m, img, f.x0, f.y0, i);
  float first = 0.0f;
  for (int c = 0; c < m.C; c++) {
    float a = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; i++)
      if ((f.mask >> i) & 1) a = __fmaf_rn(__ldg(m.data + off[i] + (long)c * m.sc), f.w[i], a);
    __stcs(out + c, a);
    if (c == 0) first = a;
  }
  return first;
}

// proj_persp for point n of view image img: writes the projection outputs
// that are asked for and returns the grid coordinates and depth.
__device__ __forceinline__ void persp_point(const ProjGatherParams &p, long img, long n, float &gx, float &gy,
                                           float &dep) {
  const long pb = img / p.pt_div;
  const float *pt = p.pts + pb * p.pb + n * p.pn;
  const float x = __ldg(pt), y = __ldg(pt + p.pa), z = __ldg(pt + 2 * p.pa);
  const float *R = p.R + img * 9, *T = p.T + img * 3, *K = p.K + img * 9;
  // pts = R @ points + T
  const float cx = __fmaf_rn(R[2], z, __fmaf_rn(R[1], y, R[0] * x)) + T[0];
  const float cy = __fmaf_rn(R[5], z, __fmaf_rn(R[4], y, R[3] * x)) + T[1];
  const float cz = __fmaf_rn(R[8], z, __fmaf_rn(R[7], y, R[6] * x)) + T[2];
  const bool invalid = cz < p.depth_thres;
  bool invalid_d = false;
  if (p.pdep) {
    const float pd = __ldg(p.pdep + pb * p.db + n * p.dn);
    invalid_d = pd < p.min_d || pd > p.max_d;
  }
  const float dz = invalid ? 1.0f : cz;
  const float qx = cx / dz, qy = cy / dz, qz = cz / dz;
  const float sx = __fmaf_rn(K[2], qz, __fmaf_rn(K[1], qy, K[0] * qx));
  const float sy = __fmaf_rn(K[5], qz, __fmaf_rn(K[4], qy, K[3] * qx));
  gx = (sx - p.half_res) / p.half_res;
  gy = (sy - p.half_res) / p.half_res;
  if (invalid || invalid_d) gx = gy = -2.0f;
  dep = invalid_d ? -2.0f : cz;
  if (p.ori_pts) {
    p.ori_pts[(img * 3 + 0) * p.N + n] = cx;
    p.ori_pts[(img * 3 + 1) * p.N + n] = cy;
    p.ori_pts[(img * 3 + 2) * p.N + n] = cz;
  }
  if (p.grids) {
    p.grids[(img * 2 + 0) * p.N + n] = gx;
    p.grids[(img * 2 + 1) * p.N + n] = gy;
  }
  if (p.depth) p.depth[img * p.N + n] = dep;
}

// Footprints of a warp's 32 items, for the lane groups.
struct WarpFoot {
  float4 w;
  int4 a;  // x0, y0, mask, image
};

// Gather of one channels-last map (vec4) for the 32 items of a warp: lane
// groups of 8 take the items four at a time, lane (group, q) the channel
// quads q, q + 8, ..., so each load reads whole 16-byte quads of one texel
// row and each store writes a contiguous part of the item's output row.
// The items' footprints come from the warp's shared array.
__device__ __forceinline__ void gather_rows(const GatherMap &m, long k0, long total, const WarpFoot *sf) {
  const int lane = lane_id(), grp = lane >> 3, q0 = lane & 7;
  const int nq = m.C >> 2;
  for (int r = 0; r < 8; r++) {
    const int src = r * 4 + grp;
    if (k0 + src >= total) break;  // items past the end are the warp's last ones
    const float4 w = sf[src].w;
    const int4 a = sf[src].a;
    const float wt[4] = {w.x, w.y, w.z, w.w};
    long off[4];
#pragma unroll
    for (int i = 0; i < 4; i++) off[i] = corner_off(m, a.w, a.x, a.y, i);
    float4 *out = reinterpret_cast<float4 *>(m.out + (k0 + src) * m.C);
    for (int q = q0; q < nq; q += 8) {
      float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        if (!((a.z >> i) & 1)) continue;
        const float4 v = __ldg(reinterpret_cast<const float4 *>(m.data + off[i]) + q);
        acc.x = __fmaf_rn(v.x, wt[i], acc.x);
        acc.y = __fmaf_rn(v.y, wt[i], acc.y);
        acc.z = __fmaf_rn(v.z, wt[i], acc.z);
        acc.w = __fmaf_rn(v.w, wt[i], acc.w);
      }
      __stcs(out + q, acc);  // streaming: the maps, not the output, should stay in L2
    }
  }
}

// Warp per 32 consecutive (image, point) items: lane = item for the
// projection, the bilinear footprint (once per item; maps of one size share
// it) and the maps that are not channels-last with C % 4 == 0; channels-last
// maps in lane groups (gather_rows).
__global__ void __launch_bounds__(256) project_gather_kernel(ProjGatherParams p) {
  __shared__ WarpFoot s_foot[8][32];
  const long total = (long)p.BV * p.N;
  const int lane = lane_id(), w8 = threadIdx.x >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  const bool small = total < (long)INT_MAX;
  for (long k0 = (((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; k0 < total; k0 += nwarps * 32) {
    const long k = k0 + lane;
    const bool live = k < total;
    float gx = -2.0f, gy = -2.0f, dep = 0.0f;
    int img = 0, n = 0;
    if (live) {
      img = small ? (int)k / p.N : (int)(k / p.N);
      n = (int)(k - (long)img * p.N);
      if (p.gin) {
        gx = __ldg(p.gin + 2 * k);
        gy = __ldg(p.gin + 2 * k + 1);
        dep = p.din ? __ldg(p.din + k) : 0.0f;
      } else {
        persp_point(p, img, n, gx, gy, dep);
      }
    }
    const Foot f0 = footprint(p.maps[0].H, p.maps[0].W, gx, gy);
    if (p.groups) {
      __syncwarp();  // the previous items' readers are done
      s_foot[w8][lane].w = make_float4(f0.w[0], f0.w[1], f0.w[2], f0.w[3]);
      s_foot[w8][lane].a = make_int4(f0.x0, f0.y0, live ? f0.mask : 0, img);
      __syncwarp();
    }
    for (int mi = 0; mi < p.n_maps; mi++) {
      const GatherMap &m = p.maps[mi];
      float first = 0.0f;
      if (m.vec4 && p.groups) {
        gather_rows(m, k0, total, s_foot[w8]);
        if (mi == p.psdf_map && live) {  // channel 0 for the depth difference
#pragma unroll
          for (int i = 0; i < 4; i++)
            if ((f0.mask >> i) & 1) first = __fmaf_rn(__ldg(m.data + corner_off(m, img, f0.x0, f0.y0, i)), f0.w[i],
                                                      first);
        }
      } else if (live) {
        first = gather_map(m, img, k, m.H == p.maps[0].H && m.W == p.maps[0].W ? f0 : footprint(m.H, m.W, gx, gy));
      }
      if (mi == p.psdf_map && live) {
        const float dd = fminf(fmaxf(dep - first, -p.psdf_clip), p.psdf_clip);
        p.psdf[k] = dd * p.psdf_scale;
      }
    }
  }
}

}  // namespace sg

using namespace sg;

extern "C" int sg_project_sampled_xyz(const SgTree *tree, const float *ray_ori, const float *ray_dir,
                                      const float *sampled_z, const int *sampled_idx, const float *K,
                                      const float *RT, int B, int num_views, int N, int S, int ori_w, int ori_h,
                                      int record_corners, float *proj_xy, float *proj_z, sg_stream_t stream) {
  if (!ray_ori || !ray_dir || !sampled_z || !sampled_idx || !K || !RT || !proj_xy || !proj_z)
    return SG_ERR_INVALID_ARG;
  if (record_corners && (!tree || !tree->counts || !tree->top_key || !tree->bot_key || !tree->voxel_size ||
                         !tree->vol_bbox || tree->Dt <= 0 || tree->Db != tree->Dt * tree->rate))
    return SG_ERR_INVALID_ARG;
  if (B <= 0 || num_views <= 0 || N < 0 || S <= 0 || ori_w <= 0 || ori_h <= 0) return SG_ERR_INVALID_ARG;
  const long total = (long)B * num_views * N * S;
  if (total == 0) return SG_OK;
  ProjSampledParams p{};
  if (tree) p.t = *tree;
  p.ori = ray_ori;
  p.dir = ray_dir;
  p.z = sampled_z;
  p.idx = sampled_idx;
  p.K = K;
  p.RT = RT;
  p.B = B;
  p.Nv = num_views;
  p.N = N;
  p.S = S;
  p.cw = (float)ori_w * 0.5f;
  p.ch = (float)ori_h * 0.5f;
  p.corners = record_corners ? 1 : 0;
  p.xy = proj_xy;
  p.pz = proj_z;
  long g = (total + 255) / 256;
  if (g > (long)num_sms() * 64) g = (long)num_sms() * 64;
  project_sampled_kernel<<<(int)g, 256, 0, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_project_gather(const SgProjGather *a, sg_stream_t stream) {
  if (!a) return SG_ERR_INVALID_ARG;
  if (!a->grids_in) {
    if (!a->points || !a->K || !a->R || !a->T || a->points_div <= 0 || a->n_images % a->points_div != 0 ||
        a->half_res == 0.0f)
      return SG_ERR_INVALID_ARG;
  } else if (a->psdf_map >= 0 && !a->depth_in) {
    return SG_ERR_INVALID_ARG;
  }
  if (a->n_images <= 0 || a->num_points < 0 || a->n_maps < 0 || a->n_maps > kMaxMaps) return SG_ERR_INVALID_ARG;
  if (a->psdf_map >= 0 && (a->psdf_map >= a->n_maps || !a->psdf || a->psdf_clip <= 0.0f)) return SG_ERR_INVALID_ARG;
  ProjGatherParams p{};
  p.gin = a->grids_in;
  p.din = a->depth_in;
  p.pts = a->points;
  p.pb = a->points_stride[0];
  p.pa = a->points_stride[1];
  p.pn = a->points_stride[2];
  p.pt_div = a->points_div;
  p.pdep = a->p_depths;
  p.db = a->p_depths_stride[0];
  p.dn = a->p_depths_stride[1];
  p.K = a->K;
  p.R = a->R;
  p.T = a->T;
  p.BV = a->n_images;
  p.N = a->num_points;
  p.depth_thres = a->depth_thres;
  p.min_d = a->min_d;
  p.max_d = a->max_d;
  p.half_res = a->half_res;
  p.ori_pts = a->ori_pts;
  p.grids = a->grids;
  p.depth = a->depth;
  p.n_maps = a->n_maps;
  for (int i = 0; i < a->n_maps; i++) {
    const SgFeatureMap &m = a->maps[i];
    if (!m.data || !m.out || m.C <= 0 || m.H <= 0 || m.W <= 0) return SG_ERR_INVALID_ARG;
    GatherMap &g = p.maps[i];
    g.data = m.data;
    g.sn = m.stride[0];
    g.sc = m.stride[1];
    g.sy = m.stride[2];
    g.sx = m.stride[3];
    g.C = m.C;
    g.H = m.H;
    g.W = m.W;
    g.out = m.out;
    g.vec4 = (m.stride[1] == 1 && m.C % 4 == 0 && m.stride[0] % 4 == 0 && m.stride[2] % 4 == 0 &&
              m.stride[3] % 4 == 0 && ((uintptr_t)m.data) % 16 == 0 && ((uintptr_t)m.out) % 16 == 0)
                 ? 1
                 : 0;
  }
  p.groups = a->n_maps > 0 ? 1 : 0;
  for (int i = 0; i < a->n_maps; i++)
    if (p.maps[i].vec4 && (p.maps[i].H != p.maps[0].H || p.maps[i].W != p.maps[0].W)) p.groups = 0;
  p.psdf_map = a->psdf_map;
  p.psdf_clip = a->psdf_clip;
  p.psdf_scale = a->psdf_scale;
  p.psdf = a->psdf;
  const long total = (long)a->n_images * a->num_points;
  if (total == 0) return SG_OK;
  if (total > (1L << 40)) return SG_ERR_UNSUPPORTED;
  long g = (total + 255) / 256;
  if (g > (long)num_sms() * 64) g = (long)num_sms() * 64;
  project_gather_kernel<<<(int)g, 256, 0, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
