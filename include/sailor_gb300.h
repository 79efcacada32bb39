/*
 * sailor_gb300.h -- C ABI of the GB300 (sm_103a) VoxelEncoding library.
 *
 * Plain pointers and sizes only; every pointer named d_* or documented as
 * device memory must be a CUDA device (or managed) address.  Every entry
 * point enqueues work on `stream` (NULL = legacy default stream) and returns
 * a status code without synchronising; conditions only the device can see
 * (capacity overflow) are reported through a caller-provided device status
 * block (SgStatus) that the caller reads after synchronising.  No entry
 * point calls exit(); the reference's CUDA_CHECK_ERRORS (include/cuda_helper.h:
 * 31-40 of the SAILOR project) prints and exits instead.
 *
 * Each function names the reference interface it replaces (paths relative to
 * the SAILOR project root).  Tensor layouts are the reference's.
 */
#ifndef SAILOR_GB300_H
#define SAILOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *sg_stream_t; /* == cudaStream_t */

enum {
  SG_OK = 0,
  SG_ERR_INVALID_ARG = 1, /* null pointer, bad size, misaligned pointer */
  SG_ERR_CUDA = 2,        /* a launch failed (cudaGetLastError)            */
  SG_ERR_CAPACITY = 3,    /* output capacity exceeded (see SgStatus)      */
  SG_ERR_UNSUPPORTED = 4  /* a configuration the library does not handle   */
};

/* Device-side status block written by kernels (atomicOr / atomicMax). */
typedef struct SgStatus {
  int flags;         /* bit 0: hit-list overflow, bit 1: tree capacity      */
  int max_hits;      /* largest per-ray hit count seen (traversal)          */
  int need_top;      /* required top-node capacity when bit 1 is set        */
  int need_bottom;   /* required bottom-node capacity when bit 1 is set     */
} SgStatus;

#define SG_FLAG_HIT_OVERFLOW 1
#define SG_FLAG_TREE_CAPACITY 2
#define SG_FLAG_RECORD_CAPACITY 4 /* gradient records exceeded the workspace's slots */

/* Two-level brick tree kept in device memory (replaces the AoS OcTree node
 * array of include/octree.h:30-153 and MultiLayerOctree's buffers
 * :274-302).  Node ids keep the reference's id space: fine voxels (level 0)
 * are base_bot + j, top bricks (level 1) base_top + k. */
typedef struct SgTree {
  int B;          /* frames (batch)                                      */
  int Dt;         /* top grid edge (bricks)                              */
  int Db;         /* fine grid edge (voxels), Db = Dt * rate             */
  int rate;       /* brick edge in voxels                                */
  int base_top;   /* id of top node 0 (octree_nodes_index[1])            */
  int base_bot;   /* id of bottom node 0 (octree_nodes_index[0])         */
  int cap_top;    /* capacity of top_key/top_child_base                  */
  int cap_bot;    /* capacity of bot_key/bot_parent                      */
  int *brick_node;        /* [B*Dt^3] top node index k, or -1           */
  uint32_t *brick_mask;   /* [B*Dt^3*mask_words] fine occupancy bits     */
  int *top_key;           /* [cap_top] b*Dt^3 + brick linear index       */
  int *top_child_base;    /* [cap_top] first child index j               */
  int *bot_key;           /* [cap_bot] b*Db^3 + voxel linear index       */
  int *bot_parent;        /* [cap_bot] parent node id                    */
  int *counts;            /* [2] {#top nodes, #bottom nodes}             */
  const float *voxel_size;/* [B]                                         */
  const float *vol_bbox;  /* [B,3,2] (min,max) per axis                  */
  int *brick_box;         /* [B*6] or NULL: per frame the bounds of its  */
                          /* kept bricks (lo x,y,z, hi x,y,z), written by */
                          /* the build; the intersection then stops a ray */
                          /* once its DDA has passed them on some axis    */
                          /* (no node can follow), which leaves every     */
                          /* output unchanged                             */
} SgTree;

/* 32-bit words per brick in SgTree.brick_mask: max(1, rate^3 / 32). */
int sg_mask_words(int rate);

const char *sg_status_string(int status);
int sg_version(void);

/* Launch-shape knobs read by the kernels' host wrappers (process-wide).
 * Values are validated; sg_tune_set returns SG_ERR_INVALID_ARG for a value
 * a knob does not accept.  Set by the autotuner (sailor_gb300/autotune.py);
 * no reference counterpart (the reference sizes every launch with
 * cudaOccupancyMaxPotentialBlockSize). */
enum {
  SG_TUNE_FUSE_VPT = 0,      /* voxels per thread in sg_fuse_tsdf: 1, 2, 4 */
  SG_TUNE_FUSE_BLOCK = 1,    /* threads per CTA in sg_fuse_tsdf: 32..256   */
  SG_TUNE_ISECT_BLOCK = 2,   /* threads per CTA in sg_intersect: 32..512   */
  SG_TUNE_RENDER_WARPS = 3,  /* CTAs per SM (x SM count) of warp-per-ray   */
                             /* kernels                                     */
  SG_TUNE_FUSE_TILED = 4,    /* sg_fuse_tsdf voxel order: 1 = 16^3 tiles,   */
                             /* 0 = linear runs (FUSE_VPT, FUSE_BLOCK)      */
  SG_TUNE_ISECT_WARP = 5,    /* intersection child tests: 0 = each ray's    */
                             /* thread, children it can reach (default);    */
                             /* 1 = a warp per hit brick, every child       */
  SG_TUNE_COUNT = 6
};
int sg_tune_set(int knob, int value);
int sg_tune_get(int knob);

/* ---- fusion ------------------------------------------------------------ */

/* Data-driven cubic box.  Replaces inverse_mat3x3 + obtain_origin_bbox +
 * obtain_resized_bbox as run by fusion_cuda_integrate
 * (c_lib/VoxelEncoding/src/fusion_kernel.cu:51-184, 683-708).
 * depth [B,N,H,W], K/R [B,N,3,3], T [B,N,3]; writes vol_origin [B,3,2],
 * vol_bbox [B,3,2], voxel_size [B]. */
int sg_auto_bbox(const float *depth, const float *K, const float *R,
                 const float *T, int B, int N, int H, int W, int vol_dim,
                 float th_bbox, float *vol_origin, float *vol_bbox,
                 float *voxel_size, sg_stream_t stream);

/* TSDF / weight / packed-colour fusion with occupancy.  Replaces
 * integrate_cuda (fusion_kernel.cu:236-340) and the three torch::full
 * pre-fills of fusion_cuda_integrate (:668-670): tsdf/weight/color are
 * written, not read.  occ [B,Dx,Dy,Dz] is written (local id or -1);
 * count [B] is incremented by the number of occupied voxels. */
int sg_fuse_tsdf(const float *K, const float *RT, const float *color,
                 const float *depth, int B, int N, int H, int W, int Dx,
                 int Dy, int Dz, const float *vol_bbox,
                 const float *voxel_size, float obs_weight,
                 float trunc_weight, float th_low, float th_high,
                 float *tsdf, float *weight, float *colorv, int *occ,
                 int *count, sg_stream_t stream);

/* ---- two-level tree -------------------------------------------------------- */

/* Coarse occupancy: a coarse voxel holds its local id if any of its rate^3
 * fine children is > -1, else -1; count [B] is incremented.  Replaces
 * merge_non_empty_nodes / build_multi_res_occupied_volumes
 * (octree_kernel.cu:242-303, 367-411). */
int sg_brick_occupancy(const int *occ_fine, int B, int Df, int rate,
                       int *occ_coarse, int *count, sg_stream_t stream);

/* Scratch bytes sg_tree_build needs for a B x Dt^3 top grid. */
size_t sg_tree_scratch_bytes(int B, int Dt);

/* Node tables: top bricks that are occupied and have an occupied
 * 26-neighbour, in ascending brick order, and their occupied fine voxels in
 * ascending lexicographic order.  Rewrites occ_top / occ_bot entries of the
 * nodes to node ids in place.  Replaces MultiLayerOctree::build_octree ->
 * gen_root_octree_nodes (octree_kernel.cu:101-239, 656-697), whose node ids
 * come from atomicAdd queues; here they are deterministic. */
int sg_tree_build(SgTree *tree, int *occ_top, int *occ_bot, void *scratch,
                  size_t scratch_bytes, SgStatus *status, sg_stream_t stream);

/* Size of the device scratch array that sg_tree_build_static uses: 8 MiB,
 * held on every GPU that loads the library until the process exits.  It
 * covers sg_tree_scratch_bytes(B, Dt) up to about one million top bricks
 * (B * Dt^3 <= 1,040,000), e.g. three 512^3 volumes with 8^3 bricks
 * (786,432 bricks) or sixteen 256^3 volumes. */
#define SG_TREE_STATIC_SCRATCH_BYTES (8u << 20)

/* sg_tree_build for callers that cannot allocate device memory (their
 * process's device memory belongs to another allocator, their per-frame loop
 * cannot take the synchronisation of cudaMalloc/cudaFree, or they reach this
 * library through a plain C foreign-function interface with no device
 * allocator).  Same inputs, outputs and results as sg_tree_build; the scratch
 * comes from the library's own fixed device array instead of the caller.
 * No counterpart in the reference: its tree build allocates through ATen
 * and thrust.
 * Returns SG_ERR_CAPACITY, and launches nothing, when
 * sg_tree_scratch_bytes(B, Dt) > SG_TREE_STATIC_SCRATCH_BYTES.  Allocates
 * nothing.  Every call looks up the array's device address
 * (cudaGetSymbolAddress) in the context current at the call, so a device
 * reset or a caller-made context never leaves it a stale address; the first
 * call in a context may load the library's device code, so make it before
 * any stream capture on the device.  All calls in a context share the array,
 * so calls that overlap on the GPU race; order them on one stream.  Nothing
 * in the array needs clearing between calls. */
int sg_tree_build_static(SgTree *tree, int *occ_top, int *occ_bot,
                         SgStatus *status, sg_stream_t stream);

/* Node table [n_nodes, 6] = (centre x, y, z, edge, valid, frame) per node
 * id.  Replaces MultiLayerOctree::output_all_nodes_tensor
 * (octree_kernel.cu:309-328, 699-717).  n_nodes == 0 (an empty tree) is a
 * no-op and out may then be NULL. */
int sg_tree_nodes(const SgTree *tree, int n_nodes, float *out,
                  sg_stream_t stream);

/* ---- multi-level tree (octree_level >= 2) ------------------------------ */

#define SG_MAX_LEVELS 12

/* Multi-level tree kept in device memory, one node table per level.
 * Replaces MultiLayerOctree with num_levels = L (octree.h:155-302) as built
 * by gen_root_octree_nodes + gen_higher_octree_nodes (octree_kernel.cu:
 * 18-99, 126-239, 654-697).  Level 0 is the finest grid (edge dim[0]),
 * level l has edge dim[l] = dim[0] / rate^l, level L-1 is the top.  Node ids
 * keep the reference's id space: node k of level l is base[l] + k, with
 * base[l] = octree_nodes_index[l] (the sum of the lower levels' occupied
 * counts).  Within a level, nodes are ordered deterministically: top nodes
 * by (frame, linear index); every other level's nodes by parent, and the
 * children of one parent in ascending (x, y, z) order -- the order in which
 * the reference inserts them (octree_kernel.cu:66-93) -- so a node's
 * children are the contiguous run child_base[l][k] .. + nchild[l][k] of
 * level l-1.  The reference's ids come from atomicAdd queues instead. */
typedef struct SgOctree {
  int B, L, rate;
  int dim[SG_MAX_LEVELS];        /* grid edge of each level                  */
  int base[SG_MAX_LEVELS];       /* node id of each level's node 0           */
  int cap[SG_MAX_LEVELS];        /* node capacity of each level's tables     */
  int *vol[SG_MAX_LEVELS];       /* [B*dim^3] occupancy (> -1 occupied);      */
                                 /* the build writes node ids into it         */
  int *key[SG_MAX_LEVELS];       /* [cap] frame * dim^3 + linear index       */
  int *parent[SG_MAX_LEVELS];    /* [cap] parent node id; -1 at the top      */
  int *child_base[SG_MAX_LEVELS];/* [cap] first child (index into level l-1) */
  int *nchild[SG_MAX_LEVELS];    /* [cap] number of children (levels >= 1)   */
  int *counts;                   /* [L] nodes built per level                */
  const float *voxel_size;       /* [B] finest voxel edge                    */
  const float *vol_bbox;         /* [B,3,2]                                   */
} SgOctree;

/* Device status of the multi-level tree calls (zeroed by the caller). */
typedef struct SgOctreeStatus {
  int flags;        /* SG_FLAG_HIT_OVERFLOW, SG_FLAG_TREE_CAPACITY            */
  int max_coarse;   /* largest coarse-row count (num_max_intersected_voxels)  */
  int max_fine;     /* largest fine-row count (num_max_intersected_voxels_fine)*/
  int reserved;
} SgOctreeStatus;

/* Bytes of device scratch sg_octree_build needs. */
size_t sg_octree_scratch_bytes(const SgOctree *tree);

/* Build every level's node table from the occupancy volumes (dense grids,
 * value > -1 = occupied, as integrate and build_multi_res_volumes leave
 * them).  Top voxels without an occupied neighbour in their 3x3x3
 * neighbourhood are not nodes (if_single_occ_in_neighbors,
 * octree_kernel.cu:101-122), and neither is anything under them.  Every
 * built node's entry in its level's volume is overwritten with its node id;
 * other entries are left as they are (as the reference does).  rate must be
 * 2, 4 or 8.  A level whose nodes exceed its capacity gets
 * SG_FLAG_TREE_CAPACITY (counts[] then hold the required numbers).
 * Runs on the stream without a host synchronisation. */
int sg_octree_build(SgOctree *tree, void *scratch, size_t scratch_bytes,
                    SgOctreeStatus *status, sg_stream_t stream);

/* Node table [n_nodes, 6] = (centre x, y, z, edge, valid, frame) per node
 * id of the multi-level tree (output_all_nodes_tensor,
 * octree_kernel.cu:309-328, 699-717).  Ids past a level's built nodes are
 * the reference's invalid placeholder nodes (valid 0). */
int sg_octree_nodes(const SgOctree *tree, int n_nodes, float *out,
                    sg_stream_t stream);

/* Coarse DDA plus depth-first descent.  Replaces
 * MultiLayerOctree::octree_traversal (intersection_kernel.cu:441-643,
 * 722-826): a DDA over the grid of level s = L-1-start_level records the
 * nodes of s the ray crosses (coarse rows, idx_c/t0_c/t1_c [B,N,Wc],
 * ray_voxel_traversal with only_voxel_traversal = false, :286-439 and
 * RayVoxelIntersectionNodeList :72-126; th_early_stop and opt_num as
 * there); each coarse node is then descended depth first, children last to
 * first, recording every descendant the ray hits (fine rows,
 * idx/t0/t1 [B,N,Wf]): a descendant whose (t0, t1) equals, bit for bit, an
 * entry already recorded under the same coarse node replaces that entry's
 * node when it is smaller, else is not recorded; the descent enters only
 * hit nodes.  valid_len [B,N] = sum over the fine entries of
 * (t1 - t0) * (edge of s / edge of the entry's node).  Rows are padded with
 * -1.  The reference runs one thread per (ray, coarse hit) and appends with
 * atomicAdd, so its fine rows hold the same entries in an order that
 * changes run to run, and its descent keeps an 8-entry stack and an
 * 8-entry list per coarse node (N_STACK_MAX_NODES, :15), which overflow for
 * rate 4 or a descent of more than one level; here fine rows are in coarse
 * order, each coarse node's entries in descent order, and neither limit
 * exists.  Rows wider than Wc / Wf keep their first entries and set
 * SG_FLAG_HIT_OVERFLOW; status->max_coarse / max_fine receive the largest
 * counts.  cnt_c / cnt_f [B,N] (nullable) receive the row counts. */
int sg_octree_traversal(const SgOctree *tree, const float *ori,
                        const float *dir, int N, int start_level, int Wc,
                        int Wf, int th_early_stop, int opt_num, int *idx_c,
                        float *t0_c, float *t1_c, int *cnt_c, int *idx,
                        float *t0, float *t1, int *cnt, float *valid_len,
                        SgOctreeStatus *status, sg_stream_t stream);

/* Adaptive sampling over fine rows.  Replaces
 * MultiLayerOctree::ray_voxels_points_sampling -> ray_voxels_sampling_kernel
 * + ray_voxels_further_sampling_kernel (sampling_kernel.cu:911-1068,
 * 1178-1248).  Each entry (rows are read up to their first -1) takes
 * max(1, (int)((t1 - t0) * r * S / valid_len)) samples, r = edge of the
 * level-(L-1-start_level) node (finest edge x 2^(L-1-start_level), as the
 * reference computes it) / the entry's node edge, placed at
 * t0 + off*(j+1) - off/2 + off*rand, off = (t1 - t0)/(n+1), until S are
 * placed; the slots left are then filled the same way in the entry with the
 * smallest node, the nearest midpoint among those (the first on a tie).
 * Slots take rands in entry order; the reference hands slots out with
 * atomicAdd across its entries, so its slot order (and, with rands that
 * differ, which jitter each sample takes) changes run to run.
 * rands / sampled_idx / sampled_z [B,N,S]; entries without a sample
 * are -1. */
int sg_sample_fine(const SgOctree *tree, const int *hit_idx,
                   const float *hit_t0, const float *hit_t1, int N, int W,
                   const float *valid_len, const float *rands, int S,
                   int start_level, int *sampled_idx, float *sampled_z,
                   sg_stream_t stream);

/* ---- ray / tree intersection ---------------------------------------- */

/* Per-ray DDA over the top grid with child slab tests.  Replaces
 * MultiLayerOctree::voxel_traversal -> ray_voxel_traversal
 * (intersection_kernel.cu:36-71, 128-439, 828-895).
 * ori/dir [B,N,3].  Rows of width W: hit_idx/hit_t0/hit_t1 [B,N,W].
 * padded != 0: entries past each ray's hits are set to -1 (the reference's
 * layout); padded == 0: entries past the hits are left untouched.
 * valid_len [B,N] and hit_count [B,N] (nullable) are written.  Rays with
 * more than W hits keep the first W and set SG_FLAG_HIT_OVERFLOW;
 * status->max_hits receives the largest count. */
int sg_intersect(const SgTree *tree, const float *ori, const float *dir,
                 int N, int W, int th_early_stop, int opt_num,
                 int is_training, int padded, int *hit_idx, float *hit_t0,
                 float *hit_t1, float *valid_len, int *hit_count,
                 SgStatus *status, sg_stream_t stream);

/* ---- sampling ------------------------------------------------------------ */

/* Adaptive coarse sampling over padded hit rows.  Replaces
 * ray_voxels_points_sampling_coarse -> ray_voxels_sampling_uniform_kernel
 * (sampling_kernel.cu:1070-1177, 1251-1304).  rands/sampled_* [B,N,S];
 * entries without a sample are -1. */
int sg_sample_coarse(const SgTree *tree, const int *hit_idx,
                     const float *hit_t0, const float *hit_t1, int N, int W,
                     const float *rands, const float *valid_len, int S,
                     int num_levels, int start_level, int *sampled_idx,
                     float *sampled_z, sg_stream_t stream);

/* Fused sampling + per-ray sort (no reference counterpart as one call: it
 * is ray_voxels_points_sampling_coarse followed by sort_samplings,
 * sampling_kernel.cu:1251-1329, producing only the sorted outputs).
 * hit_count NULL: rows are -1 terminated; else the first hit_count[r]
 * entries of row r are its hits.  rands NULL: all jitters = rand_const.
 * sorted_z / sorted_idx [B,N,S] (S <= 128): sample depths ascending (-1
 * padding first) and the node id of each. */
int sg_sample_sorted(const SgTree *tree, const int *hit_idx,
                     const float *hit_t0, const float *hit_t1,
                     const int *hit_count, int N, int W, const float *rands,
                     float rand_const, const float *valid_len, int S,
                     int num_levels, int start_level, float *sorted_z,
                     int *sorted_idx, sg_stream_t stream);

/* Per-row ascending sort of R rows of S floats (S <= 256); equal keys keep
 * their input order.  Replaces sort_samplings (sampling_kernel.cu:
 * 1308-1329, torch::sort along dim 2 + int cast).  R == 0 is a no-op and the
 * buffers may then be NULL. */
int sg_sort_samples(const float *z, int R, int S, float *sorted, int *idx,
                    sg_stream_t stream);

/* ---- compositing ------------------------------------------------------------ */

/* Front-to-back compositing of R rays x S samples (S <= 128), C <= 32
 * feature channels (C <= 16 for the adjoint).
 * mode 0: alpha = 1 - exp(-sigma * delta) (volume_rendering_training_
 * forward_kernel, volume_rendering.cu:17-126); mode 1: alpha = sigma
 * (volume_rendering_occ_training_forward_kernel :129-240).  sort_idx NULL:
 * samples are already in order (volume_rendering_occ_kernel :666-745).
 * out_feat [R,C], out_depth/out_ws/out_alpha [R]. */
int sg_composite_fwd(const float *z, const int *sort_idx, const float *sigma,
                     const float *feats, int R, int S, int C, float t_thres,
                     int mode, float *out_feat, float *out_depth,
                     float *out_ws, float *out_alpha, sg_stream_t stream);

/* Adjoint of sg_composite_fwd.  exact == 0 reproduces the reference
 * gradient formula of volume_rendering_training_backward_kernel
 * (volume_rendering.cu:244-381) and its occupancy variant (:384-522);
 * exact == 1 is the true derivative of the forward (transmittance and
 * prefix sums recomputed per ray; the saved outputs are not read).
 * grad_feats [R,S,C], grad_sigma [R,S] are fully written. */
int sg_composite_bwd(const float *g_feat, const float *g_depth,
                     const float *g_ws, const float *g_alpha,
                     const float *o_feat, const float *o_depth,
                     const float *o_ws, const float *o_alpha, const float *z,
                     const int *sort_idx, const float *sigma,
                     const float *feats, int R, int S, int C, float t_thres,
                     int mode, int exact, float *grad_feats,
                     float *grad_sigma, sg_stream_t stream);

/* ---- trilinear gathers ------------------------------------------------------ */

/* Dense-grid trilinear gather at sample points (no reference counterpart:
 * the dense-grid extension of trilinear_aggregate_features,
 * sampling_kernel.cu:162-234).  Point of sample (b, n, s) = ori[b,n] +
 * z[b,n,s] * dir[b,n]; grid [B,D,D,D,C] channel-last over each frame's
 * vol_bbox / voxel_size; out [B,N,S,C] (0 where z < 0).  mode 1 (C == 1):
 * out = sigmoid(-g * scale / s) / s, a density from a normalised TSDF. */
int sg_grid_gather(const float *ori, const float *dir, const float *z, int B,
                   int N, int S, const float *grid, int D, int C,
                   const float *vol_bbox, const float *voxel_size, int mode,
                   float scale, float s, float *out, sg_stream_t stream);

/* Adjoint of sg_grid_gather: grad_grid [B, D, D, D, C] += the sum over the
 * samples of the trilinear corner weights times grad_out [B*N, S, C]
 * (mode 0), or, for mode 1 (C == 1), times grad_out * d sigma / d t at the
 * TSDF value the forward gathered (grid is read again to recompute it).
 * grad_grid is accumulated into, not overwritten.  Per ray, consecutive
 * samples in one trilinear cell are summed first; the per-cell sums of all
 * rays then meet in atomic adds, whose order is not fixed, so the last bits
 * can differ between runs.  No counterpart in the reference: its trilinear
 * backward (c_lib/VoxelEncoding/src/sampling_kernel.cu:237-327) returns
 * per-corner gradients of per-node features and scatters into no grid. */
int sg_grid_scatter(const float *ori, const float *dir, const float *z, int B,
                    int N, int S, const float *grad_out, const float *grid,
                    int D, int C, const float *vol_bbox,
                    const float *voxel_size, int mode, float scale, float s,
                    float *grad_grid, sg_stream_t stream);

/* Zero of the part of a gradient grid a training pass can write.  grid
 * [B, Db, Db, Db, C] lies on the tree's fine geometry (voxel centres at
 * vol_bbox min + index * voxel_size); every top brick that is a node of the
 * tree or borders one (26-neighbourhood) is set to 0 -- a trilinear tap at a
 * sample inside a node (a brick, or a voxel of one) reaches at most one
 * voxel beyond the brick.  After a pass over this tree accumulated into a
 * grid that was 0 elsewhere, this restores an all-zero grid at a fraction
 * of a full clear.  Bricks are cleared with 16-byte stores when rate * C is
 * a multiple of 4 and grid is 16-byte aligned.  No counterpart in the
 * reference (its training step clears dense gradients with torch). */
int sg_zero_near_nodes(const SgTree *tree, float *grid, int C, sg_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Projection into the source views and 2D feature gather                   */
/* ------------------------------------------------------------------------ */

/* Projection of sampled points into every view.  Replaces
 * MultiLayerOctree::project_sampled_xyz (sampling_kernel.cu:1333-1381) and
 * its kernel project_xyz (:55-159).  ray_ori/ray_dir [B,N,3], sampled_z /
 * sampled_idx [B,N,S] (node ids of `tree`, -1: none), K [B,V,3,3], RT
 * [B,V,3,4] -> proj_xy [B,V,N,S,P,2] normalised to [-1,1] as
 * (pixel - size/2) / (size/2), proj_z [B,V,N,S,P] camera z, with P = 9
 * (the point, then its node's eight corners, x outermost) when
 * record_corners, else P = 1.  Items whose sample has node id -1 are -1
 * (the reference's fill); with record_corners, corners of an id that is not
 * a node of `tree` are -1 (the reference would read an arbitrary node).
 * Point and projection use the reference's float operations; the
 * normalisation, which the reference evaluates in double precision, equals
 * it exactly when size/2 is a power of two and otherwise except in rare
 * near-tie cases (then by 1 ulp).  tree may be NULL without record_corners. */
int sg_project_sampled_xyz(const SgTree *tree, const float *ray_ori, const float *ray_dir,
                           const float *sampled_z, const int *sampled_idx, const float *K,
                           const float *RT, int B, int num_views, int N, int S, int ori_w,
                           int ori_h, int record_corners, float *proj_xy, float *proj_z,
                           sg_stream_t stream);

/* A [n_images, C, H, W] feature map read through element strides
 * {image, channel, y, x} (NCHW or channels-last), and its gathered output
 * out [n_images, num_points, C] (channel-last, the layout F.grid_sample's
 * result has after .permute(0,2,1).contiguous()). */
typedef struct SgFeatureMap {
  const float *data;
  long long stride[4];
  int C, H, W;
  float *out;
} SgFeatureMap;

/* proj_persp + F.grid_sample of up to four maps + clamped depth difference.
 * Replaces utils_render.proj_persp (utils_render/utils_render.py:380-414)
 * and SRONet's forward_sample_feature (SRONet/BasicRenNet.py:245-259).
 * points [batch, 3, num_points] through element strides {batch, axis,
 * point}; view image i uses point batch i / points_div (points_div = V when
 * the points are shared by a frame's V views, as proj_persp repeats them).
 * K, R [n_images,3,3], T [n_images,3].  Per (image, point):
 *   pts = R p + T (ori_pts [n_images,3,N]), depth = pts.z; invalid = depth <
 *   depth_thres (divided by 1 instead); with p_depths ([batch, 1, N] through
 *   strides {batch, point}) a point whose p_depth is outside [min_d, max_d]
 *   gets depth -2; grids [n_images,2,N] = ((K pts/depth).xy - half_res) /
 *   half_res, -2 for invalid points (either test).
 * Each map is then sampled bilinearly at grids (align_corners=True, zero
 * padding), and with psdf_map >= 0, psdf [n_images, N] = clamp(depth -
 * sample of that map's channel 0, -psdf_clip, psdf_clip) * psdf_scale.
 * ori_pts, grids, depth may be NULL.  With grids_in [n_images, N, 2] (the
 * grid F.grid_sample takes) the projection is skipped: the maps are sampled
 * at grids_in and psdf uses depth_in [n_images, N] (points, K, R, T unused).
 * Float arithmetic of one thread per (image, point); torch's matrix
 * products may sum in another order, so results agree with the reference's
 * to float rounding. */
typedef struct SgProjGather {
  const float *grids_in, *depth_in;
  const float *points;
  long long points_stride[3];
  int points_div;
  const float *p_depths;
  long long p_depths_stride[2];
  const float *K, *R, *T;
  int n_images, num_points;
  float depth_thres, min_d, max_d, half_res;
  float *ori_pts, *grids, *depth;
  int n_maps;
  SgFeatureMap maps[4];
  int psdf_map;
  float psdf_clip, psdf_scale;
  float *psdf;
} SgProjGather;

int sg_project_gather(const SgProjGather *args, sg_stream_t stream);

/* Node-corner trilinear aggregation.  Replaces
 * MultiLayerOctree::trilinear_aggregate_features(_backward)
 * (sampling_kernel.cu:162-327, 1384-1462).  ori/dir [B,N,3],
 * z/idx [B,N,S], feats [B,C,N,S,8] -> out [B,C,N,S];
 * backward: gout [B,C,N,S] -> gin [B,C,N,S,8] (fully written). */
int sg_trilerp_nodes_fwd(const SgTree *tree, const float *ori,
                         const float *dir, const float *z, const int *idx,
                         const float *feats, int N, int S, int C, float *out,
                         sg_stream_t stream);
int sg_trilerp_nodes_bwd(const SgTree *tree, const float *ori,
                         const float *dir, const float *z, const int *idx,
                         const float *gout, int N, int S, int C, float *gin,
                         sg_stream_t stream);

/* ---- fused render ------------------------------------------------------------ */

/* One pass per ray: coarse sampling over the hit row (compact: hit_count
 * given; or -1 terminated), per-ray sort, density from the normalised TSDF
 * grid tsdf [B,D,D,D] (sigma = sigmoid(-t * sdf_scale / sdf_s) / sdf_s),
 * colour from color_grid [B,Dc,Dc,Dc,3] over color_bbox / color_vs, and
 * density compositing (t_thres early termination) into out_rgb [B,N,3],
 * out_depth/out_ws/out_alpha [B,N].  out_z/out_node [B,N,S] (both NULL or
 * both set) receive the sorted samples.  No reference counterpart as one
 * call: it is ray_voxels_points_sampling_coarse + sort_samplings
 * (sampling_kernel.cu:1251-1329) + the field queries + 
 * volume_rendering_training_forward (volume_rendering.cu:17-126). */
int sg_render_fused(const SgTree *tree, const int *hit_idx,
                    const float *hit_t0, const float *hit_t1,
                    const int *hit_count, int N, int W, const float *rands,
                    float rand_const, const float *valid_len, int S,
                    int num_levels, int start_level, const float *ori,
                    const float *dir, const float *tsdf, int D,
                    float sdf_scale, float sdf_s, const float *color_grid,
                    int Dc, const float *color_bbox, const float *color_vs,
                    float t_thres, float *out_rgb, float *out_depth,
                    float *out_ws, float *out_alpha, float *out_z,
                    int *out_node, sg_stream_t stream);

/* ---- rays ----------------------------------------------------------------- */

/* Camera table: per camera i, K^-1 (9), R^-1 (9) and the centre -R^-1 T (3)
 * into cams [n, 21], with the reference's inverse_mat3x3
 * (sampling_kernel.cu:18-48) and centre arithmetic (:441-447).
 * K, R [n, 3, 3], T [n, 3]. */
int sg_camera_params(const float *K, const float *R, const float *T, int n,
                     float *cams, sg_stream_t stream);

/* Per-pixel rays of B x N cameras: out [B, N, H, W, 6] = (origin -R^-1 T,
 * direction R^-1 K^-1 [w, h, 1] normalised).  Replaces rays_calculating
 * (sampling_kernel.cu:674-731, kernel :411-486; square H = W = load_size
 * there).  Origins are bit-identical to the reference; directions are
 * within one ulp (the reference normalises in double precision, this
 * library in single). */
int sg_rays_from_cameras(const float *K, const float *R, const float *T, int B,
                         int N, int H, int W, float *out, sg_stream_t stream);

/* ---- batched launches over segment tables -------------------------------- */
/* Many frames, views and target cameras of uneven sizes go through one
 * launch per stage.  No reference counterpart: the reference runs one frame
 * and one target view per call sequence (SRONet/BasicRenNet.py:170-318). */

/* Views of B frames with uneven counts and resolutions (device arrays).
 * Frame b owns views [view_begin[b], view_begin[b+1]) (at most 32); view v
 * has K [3,3] and RT [3,4] at K + 9v / RT + 12v and an H x W image
 * (view_hw[2v], view_hw[2v+1]) starting at element view_offset[v] of the
 * packed depth / colour buffers.  Optional (both NULL or both set):
 * depth_blocks, a float buffer of sum_v ceil(H/8) ceil(W/8) entries, and
 * block_offset [n_views], where view v's 8 x 8 pixel blocks start; fusion
 * then fills it with each block's deepest valid depth and answers its
 * per-tile view culling from it instead of reading every pixel of the
 * tile's footprint (the same results, faster). */
typedef struct SgViews {
  int max_views;                /* most views of one frame (host value, <= 32) */
  const int *view_begin;        /* [B+1]           */
  const int *view_hw;           /* [n_views, 2]    */
  const long long *view_offset; /* [n_views]       */
  const float *K;               /* [n_views, 3, 3] */
  const float *RT;              /* [n_views, 3, 4] */
  const float *depth;           /* packed images   */
  const float *color;           /* packed images   */
  const long long *block_offset;/* [n_views] or NULL */
  float *depth_blocks;          /* scratch or NULL */
} SgViews;

/* Ray segments (device arrays): segment s (one target camera) owns rays
 * [ray_begin[s], ray_begin[s+1]) of the packed ray buffers; they look into
 * frame frame[s] of the tree and grids and take samples[s] samples per ray
 * (at most the S of the launch).  The render entry points process rays
 * [ray_begin[0], total): a table whose arrays start at segment s0 of a
 * larger one (count and total set to match) renders just those segments,
 * so targets grouped by sample count can each go through the kernel sized
 * for them (SgRenderArgs.S = the group's largest samples). */
typedef struct SgRaySegments {
  int count;
  int total;            /* end of the last segment (= ray_begin[count]) */
  const int *ray_begin; /* [count+1] */
  const int *frame;     /* [count]   */
  const int *samples;   /* [count]   */
  /* Optional (both NULL or both set): each segment is a camera image of
   * widths[s] pixels per row; ray r of segment s is pixel p = r -
   * ray_begin[s] (row p / width, column p % width) of camera cameras[s]
   * (sg_camera_params).  sg_intersect_segments then generates each ray
   * itself instead of reading ori / dir; sg_segment_rays writes the rays
   * for the render entry points, which always read ori / dir. */
  const float *cameras; /* [count, 21] */
  const int *widths;    /* [count]     */
} SgRaySegments;

/* Inputs of the batched render.  Rays ori/dir [R,3]; hit rows [R,W] with
 * hit_count [R] and valid_len [R] from sg_intersect_segments; sample jitter
 * from rands [R,S] if given, else a hash of (rand_seed, ray, position) if
 * rand_seed != 0, else rand_const.  Density sigma = sigmoid(-t * sdf_scale /
 * sdf_s) / sdf_s of the trilinear TSDF t (tsdf [B,D,D,D] over the tree's
 * vol_bbox / voxel_size); colour = head [3,C] x trilinear features of feat
 * [B,Df,Df,Df,C] over feat_bbox / feat_vs (head NULL: C == 3 and colour =
 * features).  C is 3 or 16; with C == 16, feat and head are 16-byte
 * aligned (SG_ERR_INVALID_ARG otherwise). */
typedef struct SgRenderArgs {
  const float *ori, *dir;
  const int *hit_idx;
  const float *hit_t0, *hit_t1;
  const int *hit_count;
  const float *valid_len;
  int W;
  int S;
  const float *rands;
  float rand_const;
  unsigned long long rand_seed;
  const float *tsdf;
  int D;
  float sdf_scale, sdf_s;
  const float *feat;
  int Df, C;
  const float *feat_bbox, *feat_vs;
  const float *head;
  float t_thres;
} SgRenderArgs;

/* sg_fuse_tsdf over a view table: frame b fuses its own views into volume
 * b of tsdf / weight / colorv / occ [B,D,D,D]; count [B] += occupied. */
int sg_fuse_tsdf_views(const SgViews *views, int B, int D,
                       const float *vol_bbox, const float *voxel_size,
                       float obs_weight, float trunc_weight, float th_low,
                       float th_high, float *tsdf, float *weight,
                       float *colorv, int *occ, int *count,
                       sg_stream_t stream);

/* The rays of camera-defined segments (SgRaySegments.cameras / widths set)
 * written to ori / dir [total, 3]: one thread per ray, the same rays the
 * kernels generate from the cameras.  Cheaper than generating them inside
 * the warp-per-ray render, which repeats the camera arithmetic per warp. */
int sg_segment_rays(const SgRaySegments *seg, float *ori, float *dir,
                    sg_stream_t stream);

/* sg_intersect (compact rows, inference mode) over ray segments: ray r of
 * segment s traverses frame frame[s] of the tree. */
int sg_intersect_segments(const SgTree *tree, const SgRaySegments *seg,
                          const float *ori, const float *dir, int W,
                          int *hit_idx, float *hit_t0, float *hit_t1,
                          float *valid_len, int *hit_count,
                          SgStatus *status, sg_stream_t stream);

/* Forward of the batched render (as sg_render_fused, per segment):
 * out_rgb [R,3], out_depth / out_ws / out_alpha [R]; out_z / out_node
 * [R,S] (both NULL or both set) receive the sorted samples. */
int sg_render_segments_fwd(const SgTree *tree, const SgRaySegments *seg,
                           const SgRenderArgs *args, float *out_rgb,
                           float *out_depth, float *out_ws, float *out_alpha,
                           float *out_z, int *out_node, sg_stream_t stream);

/* Backward of the batched render.  Per ray it recomputes samples, sort,
 * field taps, alpha and transmittance from the same inputs (nothing is saved
 * by the forward), forms the exact adjoint of compositing for upstream
 * gradients g_rgb [R,3], g_depth / g_ws / g_alpha [R] (any may be NULL =
 * 0), and accumulates (+=) the gradient of the feature grid into grad_feat
 * [B,Df,Df,Df,C] and of the TSDF grid into grad_tsdf [B,D,D,D] (either may
 * be NULL) -- per ray, consecutive samples in one trilinear cell are summed
 * before one atomic add per cell corner and channel.  grad_sigma [R,S] /
 * grad_rgb [R,S,3] (both NULL or both set) receive the per-sample gradients
 * by sorted position. */
int sg_render_segments_bwd(const SgTree *tree, const SgRaySegments *seg,
                           const SgRenderArgs *args, const float *g_rgb,
                           const float *g_depth, const float *g_ws,
                           const float *g_alpha, float *grad_feat,
                           float *grad_tsdf, float *grad_sigma,
                           float *grad_rgb, sg_stream_t stream);

/* Training step of the batched render in one pass per ray: the forward
 * (outputs written as by sg_render_segments_fwd), the per-ray loss
 * loss_scale / 2 * |rgb - target_rgb|^2 (out_loss [R], may be NULL), and
 * the backward for the upstream gradient loss_scale * (rgb - target_rgb)
 * (as sg_render_segments_bwd: gradients accumulated into grad_feat and, if
 * not NULL, grad_tsdf).  Nothing is recomputed and nothing per sample is
 * stored.  With loss_scale = 2 / (3 R) the loss summed over rays is the mean
 * squared colour error. */
int sg_render_segments_train(const SgTree *tree, const SgRaySegments *seg,
                             const SgRenderArgs *args, const float *target_rgb,
                             float loss_scale, float *out_rgb, float *out_depth,
                             float *out_ws, float *out_alpha, float *out_loss,
                             float *grad_feat, float *grad_tsdf,
                             sg_stream_t stream);

/* ---- deterministic gradient reduction -------------------------------- */

/* Bytes of the workspace of sg_render_segments_train_det for R rays, nseg
 * segments, C feature channels and `capacity` gradient-record slots (one
 * slot per sample of every ray with hits: sum over those rays of their S;
 * the sum over all rays always suffices).  After a call the workspace
 * begins with SG_DET_COUNTERS ints: [SG_DET_RAYS_WITH_HITS] the rays with
 * hits, [SG_DET_SLOTS_NEEDED] the record slots they need, [SG_DET_SLOTS]
 * the slots used (at most `capacity`), [SG_DET_CELLS] the distinct cells
 * summed, [SG_DET_RECORDS] the records with a cell. */
#define SG_DET_COUNTERS 8
enum { SG_DET_RAYS_WITH_HITS = 0, SG_DET_SLOTS_NEEDED = 1, SG_DET_SLOTS = 2, SG_DET_CELLS = 3, SG_DET_RECORDS = 4 };
size_t sg_train_det_workspace_bytes(long long R, int nseg, int C, long long capacity);

/* The training step of sg_render_segments_train (same outputs and loss)
 * with grid gradients that are bit-identical from run to run: a segmented
 * reduction over sorted cell ids instead of float atomics.  The pass visits
 * only the rays with hits (a scan builds their list; the others get their
 * outputs directly) and writes one record per used sample -- trilinear cell,
 * cell fractions, compositing weight, ray, TSDF gradient -- plus, per ray,
 * head^T times its colour gradient; the records are sorted by cell (a
 * stable radix sort), and each cell's run is summed in order and added to
 * its 8 corners, one parity class of cells at a time (cells of a class
 * share no corner).  The sums are added (+=) into grad_feat [B,Df,Df,Df,C]
 * and grad_tsdf [B,D,D,D] (may be NULL; needs the feature grid on the TSDF
 * grid's geometry).  groups: ngroups + 1 host ints, the segment index where
 * each group of the table starts (one launch of the pass per group, sized
 * for its largest sample count group_S[g], host ints).  workspace:
 * sg_train_det_workspace_bytes(seg->total, seg->count, args->C, capacity)
 * bytes of device memory.  More records than `capacity` set
 * SG_FLAG_RECORD_CAPACITY in status and leave the gradient incomplete.
 * No counterpart in the reference: its training path differentiates
 * per-node corner features (sampling_kernel.cu:237-327), with no dense grid
 * and no reduction across rays. */
int sg_render_segments_train_det(const SgTree *tree, const SgRaySegments *seg,
                                 const SgRenderArgs *args, int ngroups,
                                 const int *groups, const int *group_S,
                                 const float *target_rgb, float loss_scale,
                                 float *out_rgb, float *out_depth, float *out_ws,
                                 float *out_alpha, float *out_loss,
                                 float *grad_feat, float *grad_tsdf,
                                 void *workspace, size_t workspace_bytes,
                                 long long capacity, SgStatus *status,
                                 sg_stream_t stream);

/* Stable sort of (keys[i], i), i < *count (a device int, at most capacity),
 * by the low key_bits bits of the keys: the sorted keys and the indices
 * into keys_out / vals_out ([capacity] each); keys_tmp / vals_tmp are
 * [capacity] scratch and scratch sg_sort_pairs_scratch_bytes(capacity)
 * bytes.  The radix sort of the deterministic gradient reduction, exported
 * for callers and tests; no counterpart in the reference (it sorts with
 * torch::sort, sampling_kernel.cu:1321, for the per-ray sample sort). */
size_t sg_sort_pairs_scratch_bytes(long long capacity);
int sg_sort_pairs(const uint32_t *keys, const int *count, long long capacity,
                  int key_bits, uint32_t *keys_out, uint32_t *vals_out,
                  uint32_t *keys_tmp, uint32_t *vals_tmp, void *scratch,
                  size_t scratch_bytes, sg_stream_t stream);

/* ---- FastNerf occupancy network (tensor cores) ------------------------- */

/* Number of float16 parameters of the density network: the feature MLP
 * 18->64->64->64->64 ([0, 13696)), the sigma MLP 64->64->64->1
 * ([13696, 22081)) and the geometry MLP 18->16->8 ([22081, 22521)), each
 * layer its weights [out][in] then its bias (infer_mlp.cu:120-240). */
size_t sg_nerf_param_count(void);

/* FastNerf's occupancy network on the tcgen05 tensor cores.  Replaces
 * infer_density_mlp (c_lib/FastNerf/src/infer_mlp.cu:583-636) with
 * density_feat_kernel (:120-199) and density_sigma_kernel (:202-240) and the
 * torch.mean over the views between them.  params: float16 bits
 * [sg_nerf_param_count()]; points_z / points_tpsdf [B,V,N], feats_geo
 * [B,V,N,16] float32 (16-byte aligned); density [B,N] out; geo_feats
 * [B,V,N,8] out (nullable; the reference computes and drops them).  V <= 128.
 * Layer outputs are rounded to float16 where the reference rounds them;
 * products within a layer are summed in float32 (the reference rounds every
 * partial sum to float16).  error (nullable, a device int) is set to 1 if a
 * tensor-core wait times out. */
int sg_nerf_density(const uint16_t *params, const float *points_z,
                    const float *points_tpsdf, const float *feats_geo, int B,
                    int N, int V, float *density, float *geo_feats,
                    int *error, sg_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* SAILOR_GB300_H */
