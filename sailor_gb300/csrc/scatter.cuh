// scatter.cuh -- keys of the gradient records of the deterministic grid
// gradient reduction (scatter.cu, written by the training pass in render.cu).
#pragma once

#include "common.cuh"

namespace sg {

// A record's key names the trilinear cell of a sample: lower corner i0 with
// every axis in [-1, D-1] (at least one corner inside a grid of edge D),
// frame b.  Keys are grouped by the cell's parity class ((i0 + 1) mod 2 per
// axis; cells of one class share no corner), so sorted keys list the cells
// class by class.
struct RecordKeys {
  int B, D;          // frames, grid edge (cells per axis: D + 1)
  uint32_t frame;    // (D + 1)^3: cells of a frame
  uint32_t cls;      // B (D + 1)^3: keys of a parity class
  uint32_t invalid;  // 8 B (D + 1)^3: no cell (sorted after every cell)
};

__host__ __device__ inline RecordKeys make_record_keys(int B, int D) {
  RecordKeys k;
  k.B = B;
  k.D = D;
  k.frame = (uint32_t)(D + 1) * (uint32_t)(D + 1) * (uint32_t)(D + 1);
  k.cls = (uint32_t)B * k.frame;
  k.invalid = 8u * k.cls;
  return k;
}

// 8 B (D + 1)^3 keys must fit below 2^32
__host__ inline bool record_keys_fit(int B, int D) {
  return (double)B * (double)(D + 1) * (double)(D + 1) * (double)(D + 1) * 8.0 < 4294967295.0;
}

// One gradient record (32 bytes, one memory sector): the sample's cell
// fractions and compositing weight, its compact ray and TSDF gradient (bits).
struct __align__(16) GradRecord {
  float4 fw;  // f0, f1, f2, w
  int4 kt;    // k, gt bits, 0, 0
};

__device__ __forceinline__ uint32_t record_key(const RecordKeys &k, int b, const int (&i0)[3]) {
  if (i0[0] < -1 || i0[1] < -1 || i0[2] < -1 || i0[0] >= k.D || i0[1] >= k.D || i0[2] >= k.D) return k.invalid;
  const uint32_t e = (uint32_t)(k.D + 1);
  const uint32_t x = (uint32_t)(i0[0] + 1), y = (uint32_t)(i0[1] + 1), z = (uint32_t)(i0[2] + 1);
  const uint32_t cls = ((x & 1u) << 2) | ((y & 1u) << 1) | (z & 1u);
  return cls * k.cls + (((uint32_t)b * e + x) * e + y) * e + z;
}

// Frame and lower corner of a valid key.
__device__ __forceinline__ void record_cell(const RecordKeys &k, uint32_t key, int &b, int (&i0)[3]) {
  const uint32_t e = (uint32_t)(k.D + 1);
  uint32_t c = key % k.cls;
  b = (int)(c / k.frame);
  c -= (uint32_t)b * k.frame;
  i0[2] = (int)(c % e) - 1;
  c /= e;
  i0[1] = (int)(c % e) - 1;
  i0[0] = (int)(c / e) - 1;
}

// ---------------------------------------------------------------------------
// workspace and launches of the deterministic reduction (scatter.cu)
// ---------------------------------------------------------------------------
// the workspace's leading counters (their indices are the header's SG_DET_*)
constexpr int kDetCounters = SG_DET_COUNTERS;
enum {
  kDetHits = SG_DET_RAYS_WITH_HITS,
  kDetSlotsNeeded = SG_DET_SLOTS_NEEDED,
  kDetSlots = SG_DET_SLOTS,
  kDetCells = SG_DET_CELLS,
  kDetValid = SG_DET_RECORDS
};

struct DetWork {
  int *cnt;                 // counters: rays with hits, slots needed, slots used, distinct cells,
                            // records with a cell
  int *hitb, *slotb;        // [R]: per ray -> exclusive counts of rays with hits / record slots
  int *hit_ray, *hit_slot;  // [R]: compact list of rays with hits, first slot of each
  int *seg_hit;             // [segments + 1]: compact index of each segment's first ray
  int *ray_nrec;            // [R]: per compact ray, its records (then their first position)
  float *ray_g;             // [R][C]: per compact ray, head^T (colour gradient)
  uint32_t *rec_key;        // [cap] cell key per slot (later: the distinct cells' keys)
  GradRecord *rec;          // [cap] record per slot
  GradRecord *pay;          // [cap] the records in sorted key order
  uint32_t *ka, *va, *kb, *vb;  // [cap] sort buffers
  void *sort_scratch;
  int *scan_scratch;
};

struct DetTrainOut {  // outputs of rays without hits (training step)
  const float *target_rgb;
  float loss_scale;
  float *out_rgb, *out_depth, *out_ws, *out_alpha, *out_loss;
};

struct DetReduceParams {
  RecordKeys keys;
  const int *cnt;
  const uint32_t *ukey;
  const int *ustart;
  const GradRecord *pay;
  const float *ray_g;
  float *grad_feat, *grad_tsdf;
};

// Byte size of the workspace for R rays, nseg segments, C channels and cap
// record slots; with base, the sub-buffers are laid out from it into w.
size_t det_layout(long R, int nseg, int C, long cap, char *base, DetWork *w);

// Compact list of rays with hits and their record slots; outputs of the
// rays without hits (o.out_rgb null: none written).
int launch_det_prepare(const DetWork &w, const SgRaySegments &seg, int S_max, const int *hit_count, long R,
                       long cap, const DetTrainOut &o, SgStatus *status, sg_stream_t stream);

// Sort the records, find the distinct cells and add their gradients into
// the grids (grad_tsdf may be null).
int launch_det_reduce(const DetWork &w, const RecordKeys &keys, long R, long cap, int C, float *grad_feat,
                      float *grad_tsdf,
                      sg_stream_t stream);

}  // namespace sg
