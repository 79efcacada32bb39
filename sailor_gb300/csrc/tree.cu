// tree.cu -- coarse occupancy and the two-level brick tree on sm_103a.
//
// Replaces octree_kernel.cu (SAILOR c_lib/VoxelEncoding/src):
//   merge_non_empty_nodes :242-303 (+ build_multi_res_occupied_volumes :367)
//   gen_root_octree_nodes :126-239 with if_single_occ_in_neighbors :101-122
//   MultiLayerOctree::build_octree :656-697
//
// Layout: instead of the reference's ~1.1 KB array-of-structs OcTree node
// (xyz corners and 64 child ids inline), the tree is brick-major
// structure-of-arrays (SgTree): a dense brick -> node map, a fine-occupancy
// bitmask per brick, and compact key arrays for top and bottom nodes.  Node
// geometry is recomputed from keys with the reference's arithmetic.
//
// brick_occupancy: one CTA per (frame, X, Y) column of bricks; threads sweep
// the rate^2 fine rows of the column with 16-byte loads (fully coalesced row
// reads), OR-reduce per brick through shared memory, and aggregate the
// count per warp.  HBM-bound: 4 bytes read per fine voxel.
//
// tree_build: (1) warp per top brick: neighbour test and, for kept bricks,
// the fine-occupancy mask by warp ballots over the brick's voxels;
// (2) a two-level exclusive scan over bricks of (kept, #children);
// (3) per-tile scan, node-table writes and in-place id rewrite of the top
// volume; (4) warp per kept brick: children in lexicographic order (ballot
// ranks), bottom-node table and in-place rewrite of the fine volume.
// Node ids therefore follow a sequential execution of the reference loop
// instead of atomicAdd arrival order.
#include "common.cuh"

namespace sg {

// ---------------------------------------------------------------------------
// coarse occupancy
// ---------------------------------------------------------------------------
__global__ void brick_occupancy_kernel(const int *__restrict__ fine, int Df, int rate, int *coarse,
                                       int *count) {
  extern __shared__ unsigned char s_any[];  // [Df]
  const int Dc = Df / rate;
  const int b = blockIdx.z, X = blockIdx.y, Y = blockIdx.x;
  const size_t vf = (size_t)Df * Df * Df;
  const int n4 = Df / 4;
  for (int t = threadIdx.x; t < n4; t += blockDim.x) {
    int any = 0;
    for (int a = 0; a < rate; a++) {
      for (int c = 0; c < rate; c++) {
        const int4 *row = reinterpret_cast<const int4 *>(
            fine + (size_t)b * vf + ((size_t)(X * rate + a) * Df + (Y * rate + c)) * Df);
        int4 q = __ldg(row + t);
        any |= (q.x > -1) | ((q.y > -1) << 1) | ((q.z > -1) << 2) | ((q.w > -1) << 3);
      }
    }
    s_any[4 * t + 0] = any & 1;
    s_any[4 * t + 1] = (any >> 1) & 1;
    s_any[4 * t + 2] = (any >> 2) & 1;
    s_any[4 * t + 3] = (any >> 3) & 1;
  }
  __syncthreads();
  const size_t vc = (size_t)Dc * Dc * Dc;
  int cnt = 0;
  for (int Z0 = 0; Z0 < Dc; Z0 += blockDim.x) {
    int Z = Z0 + threadIdx.x;
    if (Z < Dc) {
      int any = 0;
      for (int e = 0; e < rate; e++) any |= s_any[Z * rate + e];
      int local = (X * Dc + Y) * Dc + Z;
      coarse[(size_t)b * vc + local] = any ? local : -1;
      cnt += any;
    }
  }
  cnt = warp_sum(cnt);
  if (lane_id() == 0 && cnt) atomicAdd(count + b, cnt);
}

// ---------------------------------------------------------------------------
// tree build
// ---------------------------------------------------------------------------
constexpr int kTile = 1024;  // bricks per scan tile (256 threads x 4)

struct TreeScratch {
  int *keep;     // [nb] 0/1
  int *nchild;   // [nb] children of kept bricks (0 otherwise)
  int2 *tile;    // [ntiles] tile totals -> exclusive tile offsets
};

__host__ __device__ inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

__host__ __device__ inline void scratch_layout(int B, int Dt, char *base, TreeScratch *s, size_t *total) {
  size_t nb = (size_t)B * Dt * Dt * Dt;
  size_t ntiles = (nb + kTile - 1) / kTile;
  size_t off = 0;
  if (s) s->keep = (int *)(base + off);
  off += align_up(nb * 4);
  if (s) s->nchild = (int *)(base + off);
  off += align_up(nb * 4);
  if (s) s->tile = (int2 *)(base + off);
  off += align_up(ntiles * 8);
  if (total) *total = off;
}

// (1) warp per top brick
__global__ void tree_classify_kernel(SgTree t, const int *__restrict__ occ_top,
                                     const int *__restrict__ occ_bot, TreeScratch s, int mw) {
  const int lane = lane_id();
  const long nb = (long)t.B * t.Dt * t.Dt * t.Dt;
  const long vt = (long)t.Dt * t.Dt * t.Dt;
  const size_t vb = (size_t)t.Db * t.Db * t.Db;
  const int r = t.rate, r3 = r * r * r;
  for (long i = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nb;
       i += ((long)gridDim.x * blockDim.x) >> 5) {
    int b = (int)(i / vt);
    long l = i - (long)b * vt;
    int x = (int)(l / ((long)t.Dt * t.Dt)), y = (int)((l / t.Dt) % t.Dt), z = (int)(l % t.Dt);
    bool occ = occ_top[i] > -1;
    bool found = false;
    if (occ) {
      // 26-neighbourhood (if_single_occ_in_neighbors, octree_kernel.cu:101-122)
      bool mine = false;
      if (lane < 27 && lane != 13) {
        int k = x - 1 + lane / 9, m = y - 1 + (lane / 3) % 3, n = z - 1 + lane % 3;
        if (k >= 0 && k < t.Dt && m >= 0 && m < t.Dt && n >= 0 && n < t.Dt)
          mine = occ_top[(size_t)b * vt + ((size_t)k * t.Dt + m) * t.Dt + n] > -1;
      }
      found = __ballot_sync(SG_FULL, mine) != 0;
    }
    int nc = 0;
    if (found) {
      // fine occupancy bits in lexicographic child order c = a*r^2 + c2*r + e
      for (int w = 0; w < mw; w++) {
        int c = w * 32 + lane;
        bool o = false;
        if (c < r3) {
          int a = c / (r * r), c2 = (c / r) % r, e = c % r;
          size_t f = (size_t)b * vb + ((size_t)(x * r + a) * t.Db + (y * r + c2)) * t.Db + (z * r + e);
          o = occ_bot[f] > -1;
        }
        unsigned bits = __ballot_sync(SG_FULL, o);
        if (lane == 0) t.brick_mask[(size_t)i * mw + w] = bits;
        nc += __popc(bits);
      }
    }
    if (lane == 0) {
      s.keep[i] = found ? 1 : 0;
      s.nchild[i] = nc;
    }
  }
}

// (2a) tile totals
__global__ void tree_tile_sum_kernel(TreeScratch s, long nb) {
  __shared__ int2 red[8];
  long base = (long)blockIdx.x * kTile;
  int k = 0, c = 0;
  for (int j = threadIdx.x; j < kTile; j += blockDim.x) {
    long i = base + j;
    if (i < nb) {
      k += s.keep[i];
      c += s.nchild[i];
    }
  }
  k = warp_sum(k);
  c = warp_sum(c);
  if (lane_id() == 0) red[threadIdx.x >> 5] = make_int2(k, c);
  __syncthreads();
  if (threadIdx.x == 0) {
    int2 a = make_int2(0, 0);
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      a.x += red[w].x;
      a.y += red[w].y;
    }
    s.tile[blockIdx.x] = a;
  }
}

// (2b) exclusive scan of tile totals by one CTA; writes the node counts
__global__ void tree_tile_scan_kernel(TreeScratch s, int ntiles, SgTree t, SgStatus *st) {
  __shared__ int2 carry;
  __shared__ int2 wsum[32];
  if (threadIdx.x == 0) carry = make_int2(0, 0);
  __syncthreads();
  for (int base = 0; base < ntiles; base += blockDim.x) {
    int i = base + threadIdx.x;
    int2 v = (i < ntiles) ? s.tile[i] : make_int2(0, 0);
    int ix = warp_incl_scan(v.x), iy = warp_incl_scan(v.y);
    int w = threadIdx.x >> 5, lane = lane_id();
    if (lane == 31) wsum[w] = make_int2(ix, iy);
    __syncthreads();
    if (w == 0) {
      int nw = blockDim.x >> 5;
      int2 q = lane < nw ? wsum[lane] : make_int2(0, 0);
      int qx = warp_incl_scan(q.x), qy = warp_incl_scan(q.y);
      if (lane < nw) wsum[lane] = make_int2(qx - q.x, qy - q.y);
    }
    __syncthreads();
    int2 c = carry;
    int ex = c.x + wsum[w].x + ix - v.x, ey = c.y + wsum[w].y + iy - v.y;
    if (i < ntiles) s.tile[i] = make_int2(ex, ey);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = make_int2(ex + v.x, ey + v.y);
    __syncthreads();
  }
  if (t.brick_box)  // empty bounds (lo > hi) before the kept bricks widen them
    for (int i = threadIdx.x; i < 6 * t.B; i += blockDim.x) t.brick_box[i] = (i % 6) < 3 ? t.Dt : -1;
  if (threadIdx.x == 0) {
    int nt = carry.x, nbt = carry.y;
    bool over = nt > t.cap_top || nbt > t.cap_bot;
    t.counts[0] = nt < t.cap_top ? nt : t.cap_top;
    t.counts[1] = nbt < t.cap_bot ? nbt : t.cap_bot;
    if (over && st) {
      atomicOr(&st->flags, SG_FLAG_TREE_CAPACITY);
      atomicMax(&st->need_top, nt);
      atomicMax(&st->need_bottom, nbt);
    }
  }
}

// (3) per-tile scan: top-node table, brick map, top-volume rewrite.
//     The child base of each kept brick goes to s.nchild (reused).
__global__ void __launch_bounds__(256) tree_emit_top_kernel(SgTree t, int *occ_top, TreeScratch s,
                                                              long nb) {
  __shared__ int2 wsum[8];
  long base = (long)blockIdx.x * kTile + (long)threadIdx.x * 4;
  int kk[4], cc[4];
  int tk = 0, tc = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    long i = base + j;
    kk[j] = i < nb ? s.keep[i] : 0;
    cc[j] = i < nb ? s.nchild[i] : 0;
    tk += kk[j];
    tc += cc[j];
  }
  int ik = warp_incl_scan(tk), ic = warp_incl_scan(tc);
  int w = threadIdx.x >> 5, lane = lane_id();
  if (lane == 31) wsum[w] = make_int2(ik, ic);
  __syncthreads();
  int2 off = s.tile[blockIdx.x];
  for (int q = 0; q < w; q++) {
    off.x += wsum[q].x;
    off.y += wsum[q].y;
  }
  int k = off.x + ik - tk, c = off.y + ic - tc;
  const long vt = (long)t.Dt * t.Dt * t.Dt;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    long i = base + j;
    if (i >= nb) break;
    if (kk[j] && k < t.cap_top) {
      t.brick_node[i] = k;
      t.top_key[k] = (int)i;
      t.top_child_base[k] = c;
      occ_top[i] = t.base_top + k;
      if (t.brick_box) {
        const int b = (int)(i / vt);
        const long l = i - (long)b * vt;
        const int x = (int)(l / ((long)t.Dt * t.Dt)), y = (int)((l / t.Dt) % t.Dt), z = (int)(l % t.Dt);
        int *bx = t.brick_box + 6 * b;
        atomicMin(bx + 0, x);
        atomicMin(bx + 1, y);
        atomicMin(bx + 2, z);
        atomicMax(bx + 3, x);
        atomicMax(bx + 4, y);
        atomicMax(bx + 5, z);
      }
    } else {
      t.brick_node[i] = -1;
    }
    s.nchild[i] = c;  // child base (only read for kept bricks)
    k += kk[j];
    c += cc[j];
  }
}

// (4) warp per kept brick: bottom nodes in lexicographic child order
__global__ void tree_emit_children_kernel(SgTree t, int *occ_bot, int mw) {
  const int lane = lane_id();
  const int ntop = t.counts[0];
  const long vt = (long)t.Dt * t.Dt * t.Dt;
  const size_t vb = (size_t)t.Db * t.Db * t.Db;
  const int r = t.rate;
  for (long k = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < ntop;
       k += ((long)gridDim.x * blockDim.x) >> 5) {
    long i = t.top_key[k];
    int b = (int)(i / vt);
    long l = i - (long)b * vt;
    int x = (int)(l / ((long)t.Dt * t.Dt)), y = (int)((l / t.Dt) % t.Dt), z = (int)(l % t.Dt);
    int j = t.top_child_base[k];
    for (int w = 0; w < mw; w++) {
      unsigned bits = t.brick_mask[(size_t)i * mw + w];
      if ((bits >> lane) & 1u) {
        int rank = __popc(bits & ((1u << lane) - 1u));
        int jj = j + rank;
        int c = w * 32 + lane;
        int a = c / (r * r), c2 = (c / r) % r, e = c % r;
        size_t f = ((size_t)(x * r + a) * t.Db + (y * r + c2)) * t.Db + (z * r + e);
        if (jj < t.cap_bot) {
          t.bot_key[jj] = (int)((size_t)b * vb + f);
          t.bot_parent[jj] = t.base_top + (int)k;
          occ_bot[(size_t)b * vb + f] = t.base_bot + jj;
        }
      }
      j += __popc(bits);
    }
  }
}

// node table as MultiLayerOctree::output_all_nodes_tensor writes it
// (octree_kernel.cu:309-328, 699-717): per node id [x, y, z, voxel_size,
// valid, batch]; ids without a node get valid 0 and zeros.
__global__ void tree_nodes_kernel(SgTree t, int n_nodes, float *out) {
  const int ntop = t.counts[0], nbot = t.counts[1];
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes; g += (long)gridDim.x * blockDim.x) {
    float *o = out + g * 6;
    int ix = 0, iy = 0, iz = 0, b = 0;
    bool valid = false;
    LevelGeom lg;
    if (g >= t.base_top && g < t.base_top + ntop) {
      long key = t.top_key[g - t.base_top];
      long vt = (long)t.Dt * t.Dt * t.Dt;
      b = (int)(key / vt);
      long l = key - (long)b * vt;
      ix = (int)(l / ((long)t.Dt * t.Dt)), iy = (int)((l / t.Dt) % t.Dt), iz = (int)(l % t.Dt);
      lg = level_geom(t.voxel_size[b], t.Db / t.Dt);
      valid = true;
    } else if (g >= t.base_bot && g < t.base_bot + nbot) {
      long key = t.bot_key[g - t.base_bot];
      long vb = (long)t.Db * t.Db * t.Db;
      b = (int)(key / vb);
      long l = key - (long)b * vb;
      ix = (int)(l / ((long)t.Db * t.Db)), iy = (int)((l / t.Db) % t.Db), iz = (int)(l % t.Db);
      lg = level_geom(t.voxel_size[b], 1);
      valid = true;
    }
    if (valid) {
      const float *bb = t.vol_bbox + 6 * b;
      o[0] = node_coord(lg, bb[0], ix);
      o[1] = node_coord(lg, bb[2], iy);
      o[2] = node_coord(lg, bb[4], iz);
      o[3] = lg.vs;
      o[4] = 1.0f;
      o[5] = (float)b;
    } else {
      for (int k = 0; k < 6; k++) o[k] = 0.0f;
    }
  }
}

}  // namespace sg

using namespace sg;

extern "C" int sg_tree_nodes(const SgTree *tree, int n_nodes, float *out, sg_stream_t stream) {
  if (!tree || n_nodes < 0) return SG_ERR_INVALID_ARG;
  if (n_nodes == 0) return SG_OK;  // an empty tree: nothing to write (out may be NULL)
  if (!out) return SG_ERR_INVALID_ARG;
  int g = ceil_div(n_nodes, 256);
  if (g > num_sms() * 32) g = num_sms() * 32;
  tree_nodes_kernel<<<g, 256, 0, stream>>>(*tree, n_nodes, out);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_mask_words(int rate) { return sg_mask_words_dev(rate); }

extern "C" int sg_brick_occupancy(const int *occ_fine, int B, int Df, int rate, int *occ_coarse, int *count,
                                  sg_stream_t stream) {
  if (!occ_fine || !occ_coarse || !count) return SG_ERR_INVALID_ARG;
  if (B <= 0 || rate <= 0 || Df <= 0 || Df % rate != 0 || Df % 4 != 0) return SG_ERR_INVALID_ARG;
  if (((uintptr_t)occ_fine) % 16 != 0) return SG_ERR_INVALID_ARG;
  int Dc = Df / rate;
  int threads = Df / 4;
  if (threads < Dc) threads = Dc;
  threads = ((threads + 31) / 32) * 32;
  if (threads > 1024) threads = 1024;
  brick_occupancy_kernel<<<dim3(Dc, Dc, B), threads, Df, stream>>>(occ_fine, Df, rate, occ_coarse, count);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" size_t sg_tree_scratch_bytes(int B, int Dt) {
  size_t total = 0;
  scratch_layout(B, Dt, nullptr, nullptr, &total);
  return total;
}

namespace sg {
// Argument checks shared by sg_tree_build and sg_tree_build_static.
static int check_tree_args(const SgTree *tree, const int *occ_top, const int *occ_bot) {
  if (!tree || !occ_top || !occ_bot) return SG_ERR_INVALID_ARG;
  const SgTree &t = *tree;
  if (t.B <= 0 || t.Dt <= 0 || t.rate <= 0 || t.Db != t.Dt * t.rate) return SG_ERR_INVALID_ARG;
  if (!t.brick_node || !t.brick_mask || !t.top_key || !t.top_child_base || !t.bot_key || !t.bot_parent ||
      !t.counts)
    return SG_ERR_INVALID_ARG;
  if (t.rate * t.rate * t.rate > 4096) return SG_ERR_UNSUPPORTED;
  return SG_OK;
}

// The five launches of a tree build (classify, tile sums, tile scan, top
// nodes, children) over scratch of at least sg_tree_scratch_bytes(B, Dt).
static int launch_tree_build(const SgTree &t, int *occ_top, int *occ_bot, char *scratch, SgStatus *status,
                             sg_stream_t stream) {
  TreeScratch s;
  scratch_layout(t.B, t.Dt, scratch, &s, nullptr);
  long nb = (long)t.B * t.Dt * t.Dt * t.Dt;
  int ntiles = ceil_div(nb, kTile);
  int mw = sg_mask_words(t.rate);
  int gw = ceil_div(nb * 32, 256);
  if (gw > num_sms() * 64) gw = num_sms() * 64;
  tree_classify_kernel<<<gw, 256, 0, stream>>>(t, occ_top, occ_bot, s, mw);
  tree_tile_sum_kernel<<<ntiles, 256, 0, stream>>>(s, nb);
  tree_tile_scan_kernel<<<1, 1024, 0, stream>>>(s, ntiles, t, status);
  tree_emit_top_kernel<<<ntiles, 256, 0, stream>>>(t, occ_top, s, nb);
  tree_emit_children_kernel<<<num_sms() * 8, 256, 0, stream>>>(t, occ_bot, mw);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
}  // namespace sg

extern "C" int sg_tree_build(SgTree *tree, int *occ_top, int *occ_bot, void *scratch, size_t scratch_bytes,
                             SgStatus *status, sg_stream_t stream) {
  const int rc = check_tree_args(tree, occ_top, occ_bot);
  if (rc != SG_OK) return rc;
  if (!scratch || scratch_bytes < sg_tree_scratch_bytes(tree->B, tree->Dt)) return SG_ERR_INVALID_ARG;
  return launch_tree_build(*tree, occ_top, occ_bot, (char *)scratch, status, stream);
}

// ---------------------------------------------------------------------------
// sg_tree_build_static: sg_tree_build without a caller-provided scratch
// buffer.
//
// Some callers cannot call cudaMalloc: a host process whose device memory is
// owned by another allocator (a framework's caching pool or a fixed memory
// budget, where an extra allocation can fail or fragment the pool), per-frame
// loops that cannot afford the device-wide synchronisation cudaFree may take,
// and plain-C callers through a foreign-function interface that have no device
// allocator of their own to size and own a buffer.  This variant takes its
// scratch (the per-brick keep flags and child counts and the per-tile scan
// totals) from a fixed array in the library's device memory instead.
//
// The array is SG_TREE_STATIC_SCRATCH_BYTES (8 MiB) of device memory that every
// GPU which loads the library holds until the process exits.  In host code
// g_tree_static_scratch is only a host-side stand-in for the device array, so
// its device address is looked up with cudaGetSymbolAddress on every call,
// with the caller's device and context current.  Nothing is cached: after a
// cudaDeviceReset, or under a context the caller created and made current
// itself, the lookup gives the array of the context that is current now
// (a pointer kept from an earlier context would name freed or foreign
// memory).  The first call in a context may load the library's device code
// into it; make that first call before any stream capture on the device.
//
// Every call shares the one array per context, and the array keeps what the
// last call left in it.  Nothing here needs zeroing first: every scratch word
// a call reads was written earlier in the same call.  Calls whose work
// overlaps on the GPU (different streams, no ordering between them) race on
// the array and produce wrong trees; order them on one stream or with events.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_tree_static_scratch[SG_TREE_STATIC_SCRATCH_BYTES];

extern "C" int sg_tree_build_static(SgTree *tree, int *occ_top, int *occ_bot, SgStatus *status,
                                    sg_stream_t stream) {
  const int rc = check_tree_args(tree, occ_top, occ_bot);
  if (rc != SG_OK) return rc;
  if (sg_tree_scratch_bytes(tree->B, tree->Dt) > (size_t)SG_TREE_STATIC_SCRATCH_BYTES) return SG_ERR_CAPACITY;
  void *base = nullptr;
  if (cudaGetSymbolAddress(&base, g_tree_static_scratch) != cudaSuccess || !base) return SG_ERR_CUDA;
  return launch_tree_build(*tree, occ_top, occ_bot, (char *)base, status, stream);
}
