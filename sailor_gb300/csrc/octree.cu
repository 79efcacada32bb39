// octree.cu -- multi-level tree (octree_level >= 2) on sm_103a: build, node
// table, coarse DDA + depth-first descent, fine adaptive sampling.
//
// Replaces (SAILOR c_lib/VoxelEncoding/src):
//   gen_root_octree_nodes / gen_higher_octree_nodes   octree_kernel.cu:18-239
//   MultiLayerOctree::build_octree                    octree_kernel.cu:654-697
//   output_all_nodes_tensor                           octree_kernel.cu:309-328, 699-717
//   MultiLayerOctree::octree_traversal                intersection_kernel.cu:722-826
//     ray_voxel_traversal (only_voxel_traversal = false) :286-439, :72-126
//     ray_octree_traversal                            :441-643
//   MultiLayerOctree::ray_voxels_points_sampling      sampling_kernel.cu:1178-1248
//     ray_voxels_sampling_kernel :911-985, ray_voxels_further_sampling_kernel :987-1068
//
// Build: the reference walks top voxels (one thread each) and then every
// node of each level, taking node slots from atomicAdd queues.  Here each
// level is a count pass, a device-wide exclusive scan and an emit pass, so a
// node's slot is fixed by (frame, linear index) at the top and by (parent,
// child order) below -- children of one node are a contiguous run of the
// next level.  All counts stay on the device; no host synchronisation.
//
// Traversal: one thread per ray.  The reference's coarse pass writes a row
// per ray and then runs one thread per (ray, coarse hit) that descends
// through an 8-entry stack and appends with atomicAdd.  Here the ray's thread
// descends each coarse node as soon as the DDA records it, with one cursor
// per level (no stack bound: a node's children are a contiguous run), in
// the reference's per-node order (children last to first), and writes the
// fine row in coarse order.  The comparison that merges a descendant into an
// entry with bit-identical depths reads the entries already in the row, and
// only when a 64-bit filter of the coarse node's entry depths says a match
// is possible.  Node keys decode with shifts where a level's edge is a power
// of two, each level's node geometry is set once per ray, a node's key and
// child run are loaded together, and each warp pads its 32 rows' tails
// itself (16-byte stores) once its rays are done.
//
// Fine sampling: one warp per ray; per chunk of 32 entries a warp scan turns
// the per-entry sample counts into slot ranges and the chunk's samples are
// generated slot-parallel (owner found by binary search over the chunk's
// starts); the fill step is a warp arg-min over (node edge, midpoint,
// position).
#include "common.cuh"
#include "ray_core.cuh"
#include "segsort.cuh"

namespace sg {

// Per-level metadata in shared memory (dynamic level indices into the
// by-value parameter struct would spill it to local memory).
struct OctMeta {
  int L;
  int dim[SG_MAX_LEVELS], base[SG_MAX_LEVELS], cap[SG_MAX_LEVELS], count[SG_MAX_LEVELS];
  int shift[SG_MAX_LEVELS];   // log2(dim) where dim is a power of two, else -1
  float size[SG_MAX_LEVELS];  // fine voxels per node edge, dim[0] / dim[l]
  const int *vol[SG_MAX_LEVELS], *key[SG_MAX_LEVELS], *child_base[SG_MAX_LEVELS], *nchild[SG_MAX_LEVELS];
};

__device__ __forceinline__ void load_meta(const SgOctree &t, OctMeta &m) {
  if (threadIdx.x == 0) {
    m.L = t.L;
#pragma unroll
    for (int l = 0; l < SG_MAX_LEVELS; l++) {
      m.dim[l] = t.dim[l];
      m.base[l] = t.base[l];
      m.cap[l] = t.cap[l];
      m.vol[l] = t.vol[l];
      m.key[l] = t.key[l];
      m.child_base[l] = t.child_base[l];
      m.nchild[l] = t.nchild[l];
      m.count[l] = (l < t.L && t.counts) ? min(t.counts[l], t.cap[l]) : 0;
      const int D = t.dim[l];
      m.shift[l] = (D > 0 && (D & (D - 1)) == 0) ? __ffs(D) - 1 : -1;
      m.size[l] = D > 0 ? (float)(t.dim[0] / D) : 0.0f;
    }
  }
}

__device__ __forceinline__ int meta_level_of(const OctMeta &m, int id) {
  for (int l = m.L - 1; l >= 0; l--)
    if (id >= m.base[l] && id < m.base[l] + m.cap[l]) return l;
  return -1;
}

// key = b * D^3 + (x * D + y) * D + z, 0 <= key < 2^31 (the volume sizes
// are checked on the host): 32-bit unsigned arithmetic
__device__ __forceinline__ void decode_key(int key, int D, int &b, int &x, int &y, int &z) {
  const unsigned u = (unsigned)key, d = (unsigned)D, d2 = d * d;
  const unsigned bu = u / (d2 * d);
  const unsigned l = u - bu * d2 * d;
  const unsigned xu = l / d2, rem = l - xu * d2;
  const unsigned yu = rem / d;
  b = (int)bu;
  x = (int)xu;
  y = (int)yu;
  z = (int)(rem - yu * d);
}

// the same for a node of level lv: shifts and masks where the level's
// edge is a power of two
__device__ __forceinline__ void decode_node(const OctMeta &m, int lv, int key, int &x, int &y, int &z) {
  const int sh = m.shift[lv];
  if (sh >= 0) {
    const unsigned u = (unsigned)key, mask = (1u << sh) - 1u;
    z = (int)(u & mask);
    y = (int)((u >> sh) & mask);
    x = (int)((u >> (2 * sh)) & mask);
  } else {
    int b;
    decode_key(key, m.dim[lv], b, x, y, z);
  }
}

// ---------------------------------------------------------------------------
// build
// ---------------------------------------------------------------------------

// top voxels that become nodes: occupied with an occupied 26-neighbour
// (gen_root_octree_nodes :150-157 with if_single_occ_in_neighbors :101-122)
__global__ void oct_top_flags_kernel(const int *__restrict__ vtop, int B, int Dt, int *__restrict__ flags) {
  const long vt = (long)Dt * Dt * Dt, n = (long)B * vt;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    int f = 0;
    if (vtop[i] > -1) {
      const int b = (int)(i / vt);
      const long l = i - (long)b * vt;
      const int x = (int)(l / ((long)Dt * Dt)), y = (int)((l / Dt) % Dt), z = (int)(l % Dt);
      for (int a = x - 1; a <= x + 1 && !f; a++)
        for (int c = y - 1; c <= y + 1 && !f; c++)
          for (int e = z - 1; e <= z + 1; e++) {
            if (a < 0 || a >= Dt || c < 0 || c >= Dt || e < 0 || e >= Dt || (a == x && c == y && e == z)) continue;
            if (vtop[(long)b * vt + ((long)a * Dt + c) * Dt + e] > -1) {
              f = 1;
              break;
            }
          }
    }
    flags[i] = f;
  }
}

__global__ void oct_top_emit_kernel(int *__restrict__ vtop, long n, const int *__restrict__ flags,
                                     const int *__restrict__ offs, int base, int cap, int *__restrict__ key,
                                     int *__restrict__ parent, SgOctreeStatus *st) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    if (!flags[i]) continue;
    const int k = offs[i];
    if (k < cap) {
      key[k] = (int)i;
      parent[k] = -1;
      vtop[i] = base + k;
    } else if (st) {
      atomicOr(&st->flags, SG_FLAG_TREE_CAPACITY);
    }
  }
}

// children of each node of level l in level l-1 (gen_higher_octree_nodes :33-98)
__global__ void oct_child_count_kernel(const int *__restrict__ n_dev, int cap, const int *__restrict__ key, int Dp,
                                       const int *__restrict__ vchild, int Dc, int rate, int *__restrict__ nchild) {
  const int n = min(*n_dev, cap);
  const long vc = (long)Dc * Dc * Dc;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int b, X, Y, Z;
    decode_key(key[k], Dp, b, X, Y, Z);
    const int *vb = vchild + (long)b * vc;
    int c = 0;
    for (int a = 0; a < rate; a++)
      for (int m = 0; m < rate; m++) {
        const long row = ((long)(X * rate + a) * Dc + (Y * rate + m)) * Dc + (long)Z * rate;
        for (int e = 0; e < rate; e++) c += vb[row + e] > -1;
      }
    nchild[k] = c;
  }
}

__global__ void oct_child_emit_kernel(const int *__restrict__ n_dev, int cap, const int *__restrict__ key, int Dp,
                                      const int *__restrict__ child_base, int base_p, int *__restrict__ vchild,
                                      int Dc, int rate, int base_c, int cap_c, int *__restrict__ key_c,
                                      int *__restrict__ parent_c, SgOctreeStatus *st) {
  const int n = min(*n_dev, cap);
  const long vc = (long)Dc * Dc * Dc;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int b, X, Y, Z;
    decode_key(key[k], Dp, b, X, Y, Z);
    int j = child_base[k];
    bool over = false;
    for (int a = 0; a < rate; a++)
      for (int m = 0; m < rate; m++) {
        const long row = (long)b * vc + ((long)(X * rate + a) * Dc + (Y * rate + m)) * Dc + (long)Z * rate;
        for (int e = 0; e < rate; e++) {
          if (vchild[row + e] > -1) {
            if (j < cap_c) {
              key_c[j] = (int)(row + e);
              parent_c[j] = base_p + k;
              vchild[row + e] = base_c + j;
            } else {
              over = true;
            }
            j++;
          }
        }
      }
    if (over && st) atomicOr(&st->flags, SG_FLAG_TREE_CAPACITY);
  }
}

__global__ void oct_nodes_kernel(SgOctree t, int n_nodes, float *out) {
  __shared__ OctMeta m;
  load_meta(t, m);
  __syncthreads();
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes; g += (long)gridDim.x * blockDim.x) {
    float *o = out + g * 6;
    const int l = meta_level_of(m, (int)g);
    const int k = l >= 0 ? (int)g - m.base[l] : -1;
    if (l >= 0 && k < m.count[l]) {
      int b, x, y, z;
      decode_key(m.key[l][k], m.dim[l], b, x, y, z);
      const LevelGeom lg = level_geom(t.voxel_size[b], m.dim[0] / m.dim[l]);
      const float *bb = t.vol_bbox + 6 * b;
      o[0] = node_coord(lg, bb[0], x);
      o[1] = node_coord(lg, bb[2], y);
      o[2] = node_coord(lg, bb[4], z);
      o[3] = lg.vs;
      o[4] = 1.0f;
      o[5] = (float)b;
    } else {
      for (int q = 0; q < 6; q++) o[q] = 0.0f;
    }
  }
}

// ---------------------------------------------------------------------------
// traversal
// ---------------------------------------------------------------------------
struct OctTravParams {
  SgOctree t;
  const float *ori, *dir;
  int N, s, Wc, Wf, th_early_stop, opt_num;
  int *idx_c;
  float *t0_c, *t1_c;
  int *cnt_c;
  int *idx;
  float *t0, *t1;
  int *cnt;
  float *vl;
  SgOctreeStatus *st;
  long R;
};

// node edge of level l in frame b's metres
__device__ __forceinline__ float level_edge(const OctMeta &m, float vs, int l) {
  return vs * m.size[l > 0 ? l : 0];
}

constexpr int kTravThreads = 128;

// one of 64 bits chosen by the bits of t (multiplicative hash)
__device__ __forceinline__ unsigned long long t0_bit(float t) {
  return 1ull << ((__float_as_uint(t + 0.0f) * 0x9E3779B1u) >> 26);
}

__global__ void __launch_bounds__(kTravThreads, 8) octree_traverse_kernel(OctTravParams p) {
  __shared__ OctMeta m;
  // the ray's frame's node geometry per level (edge, offset), one column
  // per thread: set once per ray instead of once per tested node
  __shared__ float g_vs[SG_MAX_LEVELS][kTravThreads], g_st[SG_MAX_LEVELS][kTravThreads];
  load_meta(p.t, m);
  __syncthreads();
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int tid = threadIdx.x;
  const int s = p.s;
  int cc = 0, fc = 0;
  if (r < p.R) {
    const SgOctree &t = p.t;
    const int b = (int)(r / p.N);
    const int Ds = m.dim[s];
    const float *bb = t.vol_bbox + 6 * b;
    const float bmin[3] = {bb[0], bb[2], bb[4]};
    const float xc = (bb[0] + bb[1]) / 2.0f, yc = (bb[2] + bb[3]) / 2.0f, zc = (bb[4] + bb[5]) / 2.0f;
    const float vs = t.voxel_size[b];
    const float vs_top = vs * (float)(m.dim[0] / Ds);
    const float bst[3] = {bb[0] - vs / 2.0f, bb[2] - vs / 2.0f, bb[4] - vs / 2.0f};
    const float o[3] = {p.ori[r * 3 + 0], p.ori[r * 3 + 1], p.ori[r * 3 + 2]};
    const float d[3] = {p.dir[r * 3 + 0], p.dir[r * 3 + 1], p.dir[r * 3 + 2]};
    const float inv[3] = {__fdividef(1.0f, d[0]), __fdividef(1.0f, d[1]), __fdividef(1.0f, d[2])};
    const LevelGeom gs = level_geom(vs, m.dim[0] / Ds);
    for (int l = 0; l < s; l++) {
      const LevelGeom g = level_geom(vs, m.dim[0] / m.dim[l]);
      g_vs[l][tid] = g.vs;
      g_st[l][tid] = g.start;
    }
    const long vt = (long)Ds * Ds * Ds;
    const int *vol_s = m.vol[s], *key_s = m.key[s];
    int *oic = p.idx_c + (size_t)r * p.Wc;
    float *o0c = p.t0_c + (size_t)r * p.Wc, *o1c = p.t1_c + (size_t)r * p.Wc;
    int *oif = p.idx + (size_t)r * p.Wf;
    float *o0f = p.t0 + (size_t)r * p.Wf, *o1f = p.t1 + (size_t)r * p.Wf;
    float vlen = 0.0f;
    float T0, T1;
    if (slab(o, inv, xc, yc, zc, vs_top * (float)Ds, T0, T1) && !(T0 < 0.0f || T1 < 0.0f)) {
      float so[3];
      int st[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        float sp = __fmaf_rn(T0, d[a], o[a]);
        so[a] = sp - bst[a];
        int q = (int)(so[a] / vs_top);
        q = q < 0 ? 0 : q;
        st[a] = q < Ds ? q : Ds - 1;
      }
      float step[3], tm[3], td[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        step[a] = (d[a] >= 0) ? 1.0f : -1.0f;
        float nb = (step[a] > 0) ? ((float)st[a] + step[a]) * vs_top : (float)st[a] * vs_top;
        tm[a] = (d[a] != 0) ? (nb - so[a]) / d[a] : 9999999.0f;
        td[a] = (d[a] != 0) ? vs_top / d[a] * step[a] : 9999999.0f;
      }
      const int J = 4 * Ds;
      bool pre_empty = false, has_valid = false;
      int nsucc = 0, nint = 0;
      int cbs[SG_MAX_LEVELS], cur[SG_MAX_LEVELS];
      for (int j = 0; j < J; j++) {
        int rid = -1;
        const long cell = (long)b * vt + ((long)st[0] * Ds + st[1]) * Ds + st[2];
        const int v = vol_s[cell];
        const int k0 = v - m.base[s];
        bool node = v > -1 && k0 >= 0 && k0 < m.count[s];
        int nc0 = 0, cb0 = 0;
        if (node) {
          // the node's key and child run, loaded together
          const int kv = key_s[k0];
          if (s > 0) {
            nc0 = m.nchild[s][k0];
            cb0 = m.child_base[s][k0];
          }
          node = kv == (int)cell;
        }
        if (node) {
          float p0, p1;
          if (slab(o, inv, node_coord(gs, bmin[0], st[0]), node_coord(gs, bmin[1], st[1]),
                   node_coord(gs, bmin[2], st[2]), gs.vs, p0, p1) &&
              !(p0 < 0.0f || p1 < 0.0f)) {
            rid = cc;
            if (cc < p.Wc) {
              oic[cc] = v;
              o0c[cc] = p0;
              o1c[cc] = p1;
            }
            cc++;
            // descent from this coarse node
            const int f0 = fc;
            // bit per hashed t0 of this coarse node's stored entries: a
            // depth whose bit is clear matches no entry (equal depths hash
            // alike; + 0.0f folds -0 into +0, which compare equal)
            unsigned long long seen = fc < p.Wf ? t0_bit(p0) : 0ull;
            if (fc < p.Wf) {
              oif[fc] = v;
              o0f[fc] = p0;
              o1f[fc] = p1;
            }
            fc++;
            int depth = -1;
            if (nc0 > 0) {
              depth = 0;
              cbs[0] = cb0;
              cur[0] = nc0 - 1;
            }
            while (depth >= 0) {
              if (cur[depth] < 0) {
                depth--;
                continue;
              }
              const int lv = s - 1 - depth;
              const int kk = cbs[depth] + cur[depth];
              cur[depth]--;
              if (kk >= m.count[lv]) continue;  // a level past its capacity (flagged by the build)
              // the node's key and child run, loaded together
              const int key = m.key[lv][kk];
              int nc = 0, cbn = 0;
              if (lv > 0) {
                nc = m.nchild[lv][kk];
                cbn = m.child_base[lv][kk];
              }
              int cx, cy, cz;
              decode_node(m, lv, key, cx, cy, cz);
              const LevelGeom gl{g_vs[lv][tid], g_st[lv][tid]};
              float c0, c1;
              if (!slab(o, inv, node_coord(gl, bmin[0], cx), node_coord(gl, bmin[1], cy),
                        node_coord(gl, bmin[2], cz), gl.vs, c0, c1))
                continue;
              const int cid = m.base[lv] + kk;
              bool found = false;
              const unsigned long long hb = t0_bit(c0);
              if (seen & hb) {
                const int fe = min(fc, p.Wf);
                for (int e = f0; e < fe; e++) {
                  if (o0f[e] == c0 && o1f[e] == c1) {
                    const int pid = oif[e];
                    if (level_edge(m, vs, meta_level_of(m, pid)) > gl.vs) oif[e] = cid;
                    found = true;
                    break;
                  }
                }
              }
              if (!found) {
                if (fc < p.Wf) {
                  oif[fc] = cid;
                  o0f[fc] = c0;
                  o1f[fc] = c1;
                  seen |= hb;
                }
                fc++;
              }
              if (nc > 0) {
                depth++;
                cbs[depth] = cbn;
                cur[depth] = nc - 1;
              }
            }
            const int fe = min(fc, p.Wf);
            for (int e = f0; e < fe; e++) {
              const float scale = gs.vs / level_edge(m, vs, meta_level_of(m, oif[e]));
              vlen = vlen + (o1f[e] - o0f[e]) * scale;
            }
          }
        }
        if (p.th_early_stop > -1) {
          if (rid == -1) {
            if (pre_empty && has_valid) nsucc++;
            pre_empty = true;
          } else {
            nsucc = 0;
            pre_empty = false;
            has_valid = true;
          }
          if ((nsucc + 1) >= p.th_early_stop) break;
        }
        if (p.opt_num > -1) {
          if (rid + 1 > 0) nint++;
          if (nint >= p.opt_num) break;
        }
        int ax;
        if (tm[0] < tm[1]) ax = (tm[0] < tm[2]) ? 0 : 2;
        else ax = (tm[1] < tm[2]) ? 1 : 2;
        st[ax] += (int)step[ax];
        tm[ax] += td[ax];
        if (st[0] < 0 || st[0] >= Ds || st[1] < 0 || st[1] >= Ds || st[2] < 0 || st[2] >= Ds) break;
      }
    }
    p.vl[r] = vlen;
    if (p.cnt_c) p.cnt_c[r] = cc;
    if (p.cnt) p.cnt[r] = fc;
    if (p.st) {
      if (cc > 0) atomicMax(&p.st->max_coarse, cc);
      if (fc > 0) atomicMax(&p.st->max_fine, fc);
      if (cc > p.Wc || fc > p.Wf) atomicOr(&p.st->flags, SG_FLAG_HIT_OVERFLOW);
    }
  }
  // -1 padding of the warp's 32 rows, each by the whole warp (16-byte
  // stores; the rays' own threads would write them one element at a time)
  const int lane = lane_id();
  const long r0 = r - lane;
  for (int i = 0; i < 32; i++) {
    const int ci = __shfl_sync(SG_FULL, cc, i), fi = __shfl_sync(SG_FULL, fc, i);
    const long ri = r0 + i;
    if (ri >= p.R) break;
    pad_row_tail(p.idx_c, p.t0_c, p.t1_c, (size_t)ri * p.Wc, min(ci, p.Wc), p.Wc, lane);
    pad_row_tail(p.idx, p.t0, p.t1, (size_t)ri * p.Wf, min(fi, p.Wf), p.Wf, lane);
  }
}

// ---------------------------------------------------------------------------
// fine sampling
// ---------------------------------------------------------------------------
struct FineParams {
  SgOctree t;
  const int *idx;
  const float *t0, *t1, *vl, *rands;
  int N, W, S, start_level;
  int *si;
  float *sz;
  long R;
};

constexpr int kFineWarps = 4;

__global__ void __launch_bounds__(kFineWarps * 32) sample_fine_kernel(FineParams p) {
  __shared__ OctMeta m;
  __shared__ int s_start[kFineWarps][33], s_id[kFineWarps][32];
  __shared__ float s_mn[kFineWarps][32], s_off[kFineWarps][32];
  load_meta(p.t, m);
  __syncthreads();
  const int lane = lane_id(), w = threadIdx.x >> 5;
  const int S = p.S;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < p.R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    const int b = (int)(r / p.N);
    const int *hi = p.idx + (size_t)r * p.W;
    const float *h0 = p.t0 + (size_t)r * p.W, *h1 = p.t1 + (size_t)r * p.W;
    const float *rd = p.rands + (size_t)r * S;
    int *osi = p.si + (size_t)r * S;
    float *osz = p.sz + (size_t)r * S;
    const float vsb = p.t.voxel_size[b];
    const float vl = p.vl[r];
    const float start_vs = vsb * ldexpf(1.0f, m.L - p.start_level - 1);
    int has = 0, nh = 0;
    // best entry for the fill step: (edge, midpoint, position) minimum
    float bvs = 3.0e38f, bmid = 3.0e38f, bz0 = -1.0f, bz1 = -1.0f;
    int bpos = 0x7fffffff, bid = -1;
    for (int c0 = 0; c0 < p.W; c0 += 32) {
      const int i = c0 + lane;
      int id = -1;
      float mn = 0.0f, mx = 0.0f;
      if (i < p.W) {
        id = __ldg(hi + i);
        mn = __ldg(h0 + i);
        mx = __ldg(h1 + i);
      }
      const unsigned bad = __ballot_sync(SG_FULL, id == -1);
      const int first_bad = bad ? __ffs(bad) - 1 : 32;
      const bool ok = lane < first_bad;
      nh += first_bad;
      int n = 0;
      float nvs = 0.0f;
      if (ok) {
        nvs = vsb * (float)(m.dim[0] / m.dim[max(meta_level_of(m, id), 0)]);
        const float rt = start_vs / nvs;
        n = (int)((mx - mn) * rt * (float)S / vl);
        n = n >= 1 ? n : 1;
        // fill candidate (ray_voxels_further_sampling_kernel :1017-1040)
        const float mid = __fadd_rn(mn, mx) * 0.5f;
        if (nvs < bvs || (nvs == bvs && mid < bmid)) {
          bvs = nvs;
          bmid = mid;
          bz0 = mn;
          bz1 = mx;
          bpos = i;
          bid = id;
        }
      }
      const int incl = warp_incl_scan(n);
      const int total = __shfl_sync(SG_FULL, incl, 31);
      if (has < S && total > 0) {
        s_start[w][lane] = has + incl - n + (ok ? 0 : total);  // invalid lanes start past the chunk
        s_id[w][lane] = id;
        s_mn[w][lane] = mn;
        s_off[w][lane] = ok ? (mx - mn) / (float)(n + 1) : 0.0f;
        __syncwarp();
        const int end = min(S, has + total);
        for (int q = has + lane; q < end; q += 32) {
          // owner: last lane whose start <= q (starts increase over valid lanes)
          int lo = 0, hi2 = first_bad - 1;
          while (lo < hi2) {
            const int mid = (lo + hi2 + 1) >> 1;
            if (s_start[w][mid] <= q) lo = mid;
            else hi2 = mid - 1;
          }
          const int jj = q - s_start[w][lo];
          osz[q] = sample_z(s_mn[w][lo], s_off[w][lo], jj, __ldg(rd + q));
          osi[q] = s_id[w][lo];
        }
        has = end;
        __syncwarp();
      }
      if (bad || has >= S) break;  // with S placed the fill step never runs
    }
    // warp arg-min of the fill candidates
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ovs = __shfl_xor_sync(SG_FULL, bvs, o), omid = __shfl_xor_sync(SG_FULL, bmid, o);
      const float oz0 = __shfl_xor_sync(SG_FULL, bz0, o), oz1 = __shfl_xor_sync(SG_FULL, bz1, o);
      const int opos = __shfl_xor_sync(SG_FULL, bpos, o), oid = __shfl_xor_sync(SG_FULL, bid, o);
      const bool take = ovs < bvs || (ovs == bvs && (omid < bmid || (omid == bmid && opos < bpos)));
      if (take) {
        bvs = ovs;
        bmid = omid;
        bz0 = oz0;
        bz1 = oz1;
        bpos = opos;
        bid = oid;
      }
    }
    int filled = has;
    if (nh > 0 && bid >= 0 && has < S) {
      const int nn = S - has;
      const float off = (bz1 - bz0) / (float)(nn + 1);
      for (int q = has + lane; q < S; q += 32) {
        osz[q] = sample_z(bz0, off, q - has, __ldg(rd + q));
        osi[q] = bid;
      }
      filled = S;
    }
    for (int q = filled + lane; q < S; q += 32) {
      osz[q] = -1.0f;
      osi[q] = -1;
    }
  }
}

}  // namespace sg

using namespace sg;

static bool octree_ok(const SgOctree *t) {
  if (!t || t->B <= 0 || t->L < 2 || t->L > SG_MAX_LEVELS) return false;
  if (t->rate != 2 && t->rate != 4 && t->rate != 8) return false;
  if (!t->counts || !t->voxel_size || !t->vol_bbox) return false;
  for (int l = 0; l < t->L; l++) {
    if (t->dim[l] <= 0 || !t->vol[l] || t->cap[l] < 0) return false;
    if (l > 0 && t->dim[l - 1] != t->dim[l] * t->rate) return false;
    if (t->cap[l] > 0 && (!t->key[l] || !t->parent[l])) return false;
    if (l > 0 && t->cap[l] > 0 && (!t->child_base[l] || !t->nchild[l])) return false;
    if ((long)t->B * t->dim[l] * t->dim[l] * t->dim[l] > 0x7fffffffL) return false;
  }
  return true;
}

static long octree_scan_items(const SgOctree *t) {
  const int T = t->L - 1;
  long n = (long)t->B * t->dim[T] * t->dim[T] * t->dim[T];
  for (int l = 0; l < t->L; l++) n = n > t->cap[l] ? n : t->cap[l];
  return n;
}

extern "C" size_t sg_octree_scratch_bytes(const SgOctree *tree) {
  if (!octree_ok(tree)) return 0;
  const int T = tree->L - 1;
  const long nt = (long)tree->B * tree->dim[T] * tree->dim[T] * tree->dim[T];
  return (size_t)(2 * nt + (long)scan_scratch_ints(octree_scan_items(tree)) + 64) * sizeof(int);
}

extern "C" int sg_octree_build(SgOctree *tree, void *scratch, size_t scratch_bytes, SgOctreeStatus *status,
                               sg_stream_t stream) {
  if (!octree_ok(tree) || !scratch) return SG_ERR_INVALID_ARG;
  if (scratch_bytes < sg_octree_scratch_bytes(tree)) return SG_ERR_INVALID_ARG;
  const int T = tree->L - 1;
  const long nt = (long)tree->B * tree->dim[T] * tree->dim[T] * tree->dim[T];
  int *flags = static_cast<int *>(scratch);
  int *offs = flags + nt;
  int *scan_scr = offs + nt;
  const int grid_cap = num_sms() * 8;
  auto grid = [&](long n) {
    int g = ceil_div(n > 0 ? n : 1, 256);
    return g < grid_cap ? g : grid_cap;
  };
  cudaMemsetAsync(tree->counts, 0, sizeof(int) * tree->L, stream);
  oct_top_flags_kernel<<<grid(nt), 256, 0, stream>>>(tree->vol[T], tree->B, tree->dim[T], flags);
  launch_excl_scan(flags, nt, offs, scan_scr, tree->counts + T, stream);
  if (tree->cap[T] > 0)
    oct_top_emit_kernel<<<grid(nt), 256, 0, stream>>>(tree->vol[T], nt, flags, offs, tree->base[T], tree->cap[T],
                                                       tree->key[T], tree->parent[T], status);
  else
    oct_top_emit_kernel<<<grid(nt), 256, 0, stream>>>(tree->vol[T], nt, flags, offs, tree->base[T], 0, nullptr,
                                                       nullptr, status);
  for (int l = T; l >= 1; l--) {
    if (tree->cap[l] == 0) continue;  // no nodes here, none below (counts stay 0)
    oct_child_count_kernel<<<grid(tree->cap[l]), 256, 0, stream>>>(tree->counts + l, tree->cap[l], tree->key[l],
                                                                   tree->dim[l], tree->vol[l - 1], tree->dim[l - 1],
                                                                   tree->rate, tree->nchild[l]);
    launch_excl_scan_dev(tree->nchild[l], tree->cap[l], tree->counts + l, tree->child_base[l], scan_scr,
                         tree->counts + (l - 1), stream);
    oct_child_emit_kernel<<<grid(tree->cap[l]), 256, 0, stream>>>(
        tree->counts + l, tree->cap[l], tree->key[l], tree->dim[l], tree->child_base[l], tree->base[l],
        tree->vol[l - 1], tree->dim[l - 1], tree->rate, tree->base[l - 1], tree->cap[l - 1], tree->key[l - 1],
        tree->parent[l - 1], status);
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_octree_nodes(const SgOctree *tree, int n_nodes, float *out, sg_stream_t stream) {
  if (!octree_ok(tree) || n_nodes < 0) return SG_ERR_INVALID_ARG;
  if (n_nodes == 0) return SG_OK;
  if (!out) return SG_ERR_INVALID_ARG;
  int g = ceil_div(n_nodes, 256);
  if (g > num_sms() * 32) g = num_sms() * 32;
  oct_nodes_kernel<<<g, 256, 0, stream>>>(*tree, n_nodes, out);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_octree_traversal(const SgOctree *tree, const float *ori, const float *dir, int N, int start_level,
                                   int Wc, int Wf, int th_early_stop, int opt_num, int *idx_c, float *t0_c,
                                   float *t1_c, int *cnt_c, int *idx, float *t0, float *t1, int *cnt,
                                   float *valid_len, SgOctreeStatus *status, sg_stream_t stream) {
  if (!octree_ok(tree) || !ori || !dir || !idx_c || !t0_c || !t1_c || !idx || !t0 || !t1 || !valid_len)
    return SG_ERR_INVALID_ARG;
  if (!cnt_c || !cnt) return SG_ERR_INVALID_ARG;  // the row padding reads the counts
  if (N <= 0 || Wc <= 0 || Wf <= 0 || start_level < 0 || start_level >= tree->L) return SG_ERR_INVALID_ARG;
  if ((((uintptr_t)idx_c) | ((uintptr_t)t0_c) | ((uintptr_t)t1_c) | ((uintptr_t)idx) | ((uintptr_t)t0) |
       ((uintptr_t)t1)) % 16 != 0)
    return SG_ERR_INVALID_ARG;
  const long R = (long)tree->B * N;
  OctTravParams p{*tree, ori, dir, N, tree->L - 1 - start_level, Wc, Wf, th_early_stop, opt_num,
                  idx_c, t0_c, t1_c, cnt_c, idx, t0, t1, cnt, valid_len, status, R};
  // rows padded in the kernel
  octree_traverse_kernel<<<ceil_div(R, kTravThreads), kTravThreads, 0, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_sample_fine(const SgOctree *tree, const int *hit_idx, const float *hit_t0, const float *hit_t1,
                              int N, int W, const float *valid_len, const float *rands, int S, int start_level,
                              int *sampled_idx, float *sampled_z, sg_stream_t stream) {
  if (!octree_ok(tree) || !hit_idx || !hit_t0 || !hit_t1 || !valid_len || !rands || !sampled_idx || !sampled_z)
    return SG_ERR_INVALID_ARG;
  if (N <= 0 || W <= 0 || S <= 0 || start_level < 0 || start_level >= tree->L) return SG_ERR_INVALID_ARG;
  const long R = (long)tree->B * N;
  FineParams p{*tree, hit_idx, hit_t0, hit_t1, valid_len, rands, N, W, S, start_level, sampled_idx, sampled_z, R};
  long g = ceil_div(R, kFineWarps);
  if (g > (long)num_sms() * 16) g = (long)num_sms() * 16;
  sample_fine_kernel<<<(int)g, kFineWarps * 32, 0, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
