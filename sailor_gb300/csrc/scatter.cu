// scatter.cu -- deterministic reduction of the training pass's grid
// gradients: a segmented reduction over the sampled cells, sorted.
//
// The in-kernel scatter of the render backward adds each cell run's
// gradient into the grids with float atomics, so the summation order -- and
// the last bits of the gradient -- change from run to run.  Here the
// training pass (render.cu, record mode) writes one record per used sample
// instead: the sample's trilinear cell as a 32-bit key (frame and lower
// corner, grouped by parity class), and a 32-byte record of its cell
// fractions, its compositing weight, its ray and its TSDF gradient; the
// ray's colour-head factor of the feature gradient goes to a per-ray table.
// The pass packs each ray's records at the front of the ray's slots and
// writes their count.  Then
//   1. the records are compacted (slot order kept: a scan over the rays'
//      record counts, a warp per ray moving its keys) and their
//      keys sorted, stably, with the record slots as values (segsort.cu):
//      records of one cell become one run, in slot order (ray order, then
//      sorted sample order -- fixed by the ray layout); the records are
//      gathered into that order;
//   2. run heads are flagged and scanned into the list of distinct cells;
//   3. for each of the 8 parity classes in turn, one warp per cell sums its
//      run in order into the 8 corners x C channels it touches (lane = corner
//      x 4 channels) and adds the sums into the grids.  Cells of one class
//      share no corner, so every grid value is updated by one warp per
//      class, classes in a fixed order.
// Every grid value is therefore the same sum in the same order on every run:
// the gradients are bit-identical across runs, launch shapes and graph
// replays.
//
// Before the training pass, a scan over the rays (rays with hits, and their
// record slots: S per ray with hits) builds the compact list of rays the
// pass visits; rays without hits get their outputs (0, and the loss of the
// target alone) here.
#include "ray_core.cuh"
#include "scatter.cuh"
#include "segsort.cuh"

namespace sg {

__device__ __forceinline__ long ray_samples(const SgRaySegments &seg, int S_max, long r, int &s) {
  s = segment_of(seg.ray_begin, seg.count, r);
  const int S = __ldg(seg.samples + s);
  return S < S_max ? S : S_max;
}

// hit flag and record slots per ray
__global__ void det_ray_counts_kernel(SgRaySegments seg, int S_max, const int *__restrict__ hit_count, long R,
                                      int *__restrict__ hitb, int *__restrict__ slotb) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (long)gridDim.x * blockDim.x) {
    int s;
    const long S = ray_samples(seg, S_max, r, s);
    const bool h = __ldg(hit_count + r) > 0;
    hitb[r] = h ? 1 : 0;
    slotb[r] = h ? (int)S : 0;
  }
}

// compact ray list and slots; outputs of rays without hits
__global__ void det_ray_emit_kernel(long R, const int *__restrict__ hit_count, const int *__restrict__ hitb,
                                    const int *__restrict__ slotb, int *__restrict__ hit_ray,
                                    int *__restrict__ hit_slot, DetTrainOut o) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (long)gridDim.x * blockDim.x) {
    if (__ldg(hit_count + r) > 0) {
      const int k = hitb[r];
      hit_ray[k] = (int)r;
      hit_slot[k] = slotb[r];
    } else if (o.out_rgb) {
      float l = 0.0f;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float t = __ldg(o.target_rgb + r * 3 + c);
        o.out_rgb[r * 3 + c] = 0.0f;
        l += t * t;
      }
      o.out_depth[r] = o.out_ws[r] = o.out_alpha[r] = 0.0f;
      if (o.out_loss) o.out_loss[r] = 0.5f * o.loss_scale * l;
    }
  }
}

// compact index of each segment's first ray; slots used (clamped to the
// capacity) and the capacity flag
__global__ void det_seg_kernel(SgRaySegments seg, long R, const int *__restrict__ hitb, int *__restrict__ cnt,
                               int *__restrict__ seg_hit, long cap, SgStatus *st) {
  for (int s = threadIdx.x; s <= seg.count; s += blockDim.x) {
    const long rb = __ldg(seg.ray_begin + s);
    seg_hit[s] = rb < R ? hitb[rb] : cnt[kDetHits];
  }
  if (threadIdx.x == 0) {
    const int need = cnt[kDetSlotsNeeded];
    cnt[kDetSlots] = need < cap ? need : (int)cap;
    if (need > cap && st) {
      atomicOr(&st->flags, SG_FLAG_RECORD_CAPACITY);
    }
  }
}

// the records, compacted in slot order (ray order, then sorted position
// order: each ray's records lead its slots): key and slot, a warp per ray;
// first = the rays' exclusive record counts
__global__ void det_compact_kernel(const uint32_t *__restrict__ key, const int *__restrict__ cnt,
                                   const int *__restrict__ first, const int *__restrict__ hit_slot,
                                   uint32_t *__restrict__ ckey, uint32_t *__restrict__ cslot) {
  const long n = cnt[kDetHits];
  const int total = cnt[kDetValid];
  const int lane = lane_id();
  for (long k = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n;
       k += ((long)gridDim.x * blockDim.x) >> 5) {
    const int a = __ldg(first + k), e = k + 1 < n ? __ldg(first + k + 1) : total;
    const long base = __ldg(hit_slot + k);
    for (int i = lane; i < e - a; i += 32) {
      ckey[a + i] = __ldg(key + base + i);
      cslot[a + i] = (uint32_t)(base + i);
    }
  }
}

// head flags of the sorted keys' runs (cells)
__global__ void det_heads_kernel(const uint32_t *__restrict__ key, const int *__restrict__ cnt,
                                 int *__restrict__ head) {
  const long n = cnt[kDetValid];
  for (long j = (long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x)
    head[j] = (j == 0 || __ldg(key + j - 1) != __ldg(key + j)) ? 1 : 0;
}

// distinct cells: key and first sorted position; the end of the last run
__global__ void det_unique_kernel(const uint32_t *__restrict__ key, const int *__restrict__ head_scan,
                                  const int *__restrict__ cnt, uint32_t *__restrict__ ukey,
                                  int *__restrict__ ustart) {
  const long n = cnt[kDetValid];
  const int nu = cnt[kDetCells];
  for (long j = (long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
    const uint32_t k = __ldg(key + j);
    if (j == 0 || __ldg(key + j - 1) != k) {
      const int u = head_scan[j];
      ukey[u] = k;
      ustart[u] = (int)j;
    }
    if (j + 1 == n) ustart[nu] = (int)n;
  }
}

// the records in sorted key order (one gathered 32-byte sector per record);
// kGatherItems records a thread per step, their loads in flight together
constexpr int kGatherItems = 4;
__global__ void det_gather_kernel(const uint32_t *__restrict__ sorted_slot, const int *__restrict__ cnt,
                                  const GradRecord *__restrict__ rec, GradRecord *__restrict__ pay) {
  const long n = cnt[kDetValid];
  const long stride = (long)gridDim.x * blockDim.x;
  for (long j0 = (long)blockIdx.x * blockDim.x + threadIdx.x; j0 < n; j0 += stride * kGatherItems) {
    uint32_t slot[kGatherItems];
    float4 fw[kGatherItems];
    int4 kt[kGatherItems];
#pragma unroll
    for (int q = 0; q < kGatherItems; q++) {
      const long j = j0 + q * stride;
      slot[q] = j < n ? __ldg(sorted_slot + j) : 0u;
    }
#pragma unroll
    for (int q = 0; q < kGatherItems; q++) {
      if (j0 + q * stride < n) {
        fw[q] = __ldg(&rec[slot[q]].fw);
        kt[q] = __ldg(&rec[slot[q]].kt);
      }
    }
#pragma unroll
    for (int q = 0; q < kGatherItems; q++) {
      const long j = j0 + q * stride;
      if (j < n) {
        pay[j].fw = fw[q];
        pay[j].kt = kt[q];
      }
    }
  }
}

__device__ __forceinline__ int lower_bound_u32(const uint32_t *a, int n, uint32_t v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Cells of parity class cls: warp per cell, its run summed in order, the
// sums added into the 8 corner voxels of the feature grid (and TSDF grid).
// TSDF: the TSDF gradient is reduced too (q.grad_tsdf set); without it the
// kernel holds no TSDF staging, which leaves more of the SM's L1 to the G rows
template <int C, bool TSDF>
__global__ void __launch_bounds__(256, 4) det_class_kernel(DetReduceParams q, int cls) {
  // per warp: the current chunk of up to 32 records of a run -- per record
  // its 8 corner weights times its compositing weight (s_a), its 8 corner
  // weights (s_cw, for the TSDF gradient), its TSDF gradient (s_t) and its
  // ray's G row (s_g) -- staged by all lanes at once (lane j: record j) and
  // read back in run order
  __shared__ __align__(16) float4 s_g[8][32][4];
  __shared__ __align__(16) float s_a[8][32][8];
  __shared__ __align__(16) float s_cw[TSDF ? 8 : 1][32][8];
  __shared__ float s_t[TSDF ? 8 : 1][32];
  __shared__ int s_rng[2];
  const int nu = q.cnt[kDetCells];
  if (threadIdx.x == 0) {
    s_rng[0] = lower_bound_u32(q.ukey, nu, (uint32_t)cls * q.keys.cls);
    s_rng[1] = lower_bound_u32(q.ukey, nu, (uint32_t)(cls + 1) * q.keys.cls);
  }
  __syncthreads();
  const int lo = s_rng[0], hi = s_rng[1];
  const int lane = lane_id(), w8 = threadIdx.x >> 5;
  // lane -> (corner, channels): C == 16: corner lane / 4, channels 4 (lane % 4)..+3;
  // C == 3: lanes < 24, corner lane / 3, channel lane % 3.  TSDF: corner = lane (< 8).
  const int cr = C == 16 ? (lane >> 2) : (lane < 24 ? lane / 3 : 0);
  const int ch = C == 16 ? 4 * (lane & 3) : (lane < 24 ? lane % 3 : 0);
  const bool fown = C == 16 || lane < 24;
  const long D = q.keys.D;
  const long wstride = ((long)gridDim.x * blockDim.x) >> 5;
  long u = lo + (((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  // the cell's run bounds and key, and its first 32 records, are loaded one
  // cell ahead: while a cell is summed, the next one's loads are in flight
  int j0 = 0, j1 = 0;
  uint32_t ckey = 0;
  if (u < hi) {
    j0 = __ldg(q.ustart + u);
    j1 = __ldg(q.ustart + u + 1);
    ckey = __ldg(q.ukey + u);
  }
  float4 pf_fw = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  int4 pf_kt = make_int4(0, 0, 0, 0);
  if (u < hi && j0 + lane < j1) {
    pf_fw = __ldg(&q.pay[j0 + lane].fw);
    pf_kt = __ldg(&q.pay[j0 + lane].kt);
  }
  for (; u < hi; u += wstride) {
    const long un = u + wstride;
    int nj0 = 0, nj1 = 0;
    uint32_t nkey = 0;
    if (un < hi) {
      nj0 = __ldg(q.ustart + un);
      nj1 = __ldg(q.ustart + un + 1);
      nkey = __ldg(q.ukey + un);
    }
    // the cell's corner values are read before its run is summed, so the
    // read of the grid overlaps the run
    int b, i0[3];
    record_cell(q.keys, ckey, b, i0);
    const int vx = i0[0] + ((cr >> 2) & 1), vy = i0[1] + ((cr >> 1) & 1), vz = i0[2] + (cr & 1);
    const bool fin = fown && vx >= 0 && vy >= 0 && vz >= 0 && vx < D && vy < D && vz < D;
    float *gp = fin ? q.grad_feat + ((((size_t)b * D + vx) * D + vy) * D + vz) * C + ch : nullptr;
    float4 old = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (fin) {
      if (C == 16) old = *reinterpret_cast<const float4 *>(gp);
      else old.x = *gp;
    }
    const int tx = i0[0] + ((lane >> 2) & 1), ty = i0[1] + ((lane >> 1) & 1), tz = i0[2] + (lane & 1);
    const bool tin = TSDF && lane < 8 && tx >= 0 && ty >= 0 && tz >= 0 && tx < D && ty < D && tz < D;
    float *tp = tin ? q.grad_tsdf + (((size_t)b * D + tx) * D + ty) * D + tz : nullptr;
    const float told = tin ? *tp : 0.0f;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float acct = 0.0f;
    for (int c0 = j0; c0 < j1; c0 += 32) {
      // lane jj stages the run's record c0 + jj (sorted: one coalesced load)
      // and its ray's G row; then the samples are summed in run order
      if (c0 + lane < j1) {
        float4 fw;
        int4 kt;
        if (c0 == j0) {
          fw = pf_fw;
          kt = pf_kt;
        } else {
          fw = __ldg(&q.pay[c0 + lane].fw);
          kt = __ldg(&q.pay[c0 + lane].kt);
        }
        const float *g = q.ray_g + (size_t)kt.x * C;
        if (C == 16) {
#pragma unroll
          for (int v = 0; v < 4; v++) s_g[w8][lane][v] = __ldg(reinterpret_cast<const float4 *>(g) + v);
        } else {
          s_g[w8][lane][0] = make_float4(__ldg(g), __ldg(g + 1), __ldg(g + 2), 0.0f);
        }
        const float f[3] = {fw.x, fw.y, fw.z};
        float cw[8], a[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
          cw[c] = corner_weight(f, c);
          a[c] = cw[c] * fw.w;
        }
        reinterpret_cast<float4 *>(s_a[w8][lane])[0] = make_float4(a[0], a[1], a[2], a[3]);
        reinterpret_cast<float4 *>(s_a[w8][lane])[1] = make_float4(a[4], a[5], a[6], a[7]);
        if (TSDF) {
          reinterpret_cast<float4 *>(s_cw[w8][lane])[0] = make_float4(cw[0], cw[1], cw[2], cw[3]);
          reinterpret_cast<float4 *>(s_cw[w8][lane])[1] = make_float4(cw[4], cw[5], cw[6], cw[7]);
          s_t[w8][lane] = __int_as_float(kt.y);
        }
      }
      if (c0 == j0 && un < hi && nj0 + lane < nj1) {
        // the next cell's first records
        pf_fw = __ldg(&q.pay[nj0 + lane].fw);
        pf_kt = __ldg(&q.pay[nj0 + lane].kt);
      }
      __syncwarp();
      const int m = min(32, j1 - c0);
#pragma unroll 4
      for (int jj = 0; jj < m; jj++) {
        const float a = s_a[w8][jj][cr];
        if (C == 16) {
          const float4 g = s_g[w8][jj][lane & 3];
          acc.x = __fmaf_rn(a, g.x, acc.x);
          acc.y = __fmaf_rn(a, g.y, acc.y);
          acc.z = __fmaf_rn(a, g.z, acc.z);
          acc.w = __fmaf_rn(a, g.w, acc.w);
        } else if (fown) {
          const float4 g = s_g[w8][jj][0];
          acc.x = __fmaf_rn(a, ch == 0 ? g.x : (ch == 1 ? g.y : g.z), acc.x);
        }
        if (TSDF && lane < 8) acct = __fmaf_rn(s_cw[w8][jj][lane], s_t[w8][jj], acct);
      }
      __syncwarp();
    }
    if (fin) {
      if (C == 16)
        *reinterpret_cast<float4 *>(gp) = make_float4(old.x + acc.x, old.y + acc.y, old.z + acc.z, old.w + acc.w);
      else
        *gp = old.x + acc.x;
    }
    if (tin) *tp = told + acct;
    j0 = nj0;
    j1 = nj1;
    ckey = nkey;
  }
}

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t det_layout(long R, int nseg, int C, long cap, char *base, DetWork *w) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  DetWork d{};
  d.cnt = (int *)take(kDetCounters * sizeof(int));
  d.hitb = (int *)take((size_t)R * 4);
  d.slotb = (int *)take((size_t)R * 4);
  d.hit_ray = (int *)take((size_t)R * 4);
  d.hit_slot = (int *)take((size_t)R * 4);
  d.seg_hit = (int *)take((size_t)(nseg + 1) * 4);
  d.ray_nrec = (int *)take((size_t)R * 4);
  d.ray_g = (float *)take((size_t)R * C * 4);
  d.rec_key = (uint32_t *)take((size_t)cap * 4);
  d.rec = (GradRecord *)take((size_t)cap * sizeof(GradRecord));
  d.pay = (GradRecord *)take((size_t)cap * sizeof(GradRecord));
  // one more than cap: after the sort, one of the pairs holds the distinct
  // cells' first positions and the end of the last run
  d.ka = (uint32_t *)take((size_t)(cap + 1) * 4);
  d.va = (uint32_t *)take((size_t)(cap + 1) * 4);
  d.kb = (uint32_t *)take((size_t)(cap + 1) * 4);
  d.vb = (uint32_t *)take((size_t)(cap + 1) * 4);
  d.sort_scratch = take(radix_scratch_bytes(cap));
  const size_t sc = scan_scratch_ints(R) > scan_scratch_ints(cap) ? scan_scratch_ints(R) : scan_scratch_ints(cap);
  d.scan_scratch = (int *)take(sc * 4);
  if (w) *w = d;
  return off;
}

static int grid_for(long n, int per_sm = 8) {
  long g = (n + 255) / 256;
  const long cap = (long)num_sms() * per_sm;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

int launch_det_prepare(const DetWork &w, const SgRaySegments &seg, int S_max, const int *hit_count, long R,
                       long cap, const DetTrainOut &o, SgStatus *status, sg_stream_t stream) {
  det_ray_counts_kernel<<<grid_for(R), 256, 0, stream>>>(seg, S_max, hit_count, R, w.hitb, w.slotb);
  launch_excl_scan(w.hitb, R, w.hitb, w.scan_scratch, w.cnt + kDetHits, stream);
  launch_excl_scan(w.slotb, R, w.slotb, w.scan_scratch, w.cnt + kDetSlotsNeeded, stream);
  det_ray_emit_kernel<<<grid_for(R), 256, 0, stream>>>(R, hit_count, w.hitb, w.slotb, w.hit_ray, w.hit_slot, o);
  det_seg_kernel<<<1, 256, 0, stream>>>(seg, R, w.hitb, w.cnt, w.seg_hit, cap, status);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

int launch_det_reduce(const DetWork &w, const RecordKeys &keys, long R, long cap, int C, float *grad_feat,
                      float *grad_tsdf,
                      sg_stream_t stream) {
  int key_bits = 1;
  while (key_bits < 32 && ((uint64_t)1 << key_bits) <= (uint64_t)keys.invalid) key_bits++;
  const int g = grid_for(cap, 16);
  // the records, compacted into the b pair (slot order kept): the rays'
  // record counts scanned in place into their first positions
  launch_excl_scan_dev(w.ray_nrec, R, w.cnt + kDetHits, w.ray_nrec, w.scan_scratch, w.cnt + kDetValid, stream);
  det_compact_kernel<<<grid_for(R * 32, 16), 256, 0, stream>>>(w.rec_key, w.cnt, w.ray_nrec, w.hit_slot, w.kb,
                                                                w.vb);
  const int passes = launch_radix_sort(w.kb, w.vb, w.cnt + kDetValid, cap, key_bits, w.ka, w.va, w.kb, w.vb,
                                       w.sort_scratch, stream);
  const uint32_t *skey = (passes & 1) ? w.ka : w.kb;
  const uint32_t *sval = (passes & 1) ? w.va : w.vb;
  // the other pair is free now: head flags and their scan in one buffer,
  // the distinct cells' first positions in the other; their keys where the
  // unsorted keys were
  int *heads = (int *)((passes & 1) ? w.kb : w.ka);
  int *ustart = (int *)((passes & 1) ? w.vb : w.va);
  uint32_t *ukey = w.rec_key;
  det_heads_kernel<<<g, 256, 0, stream>>>(skey, w.cnt, heads);
  launch_excl_scan_dev(heads, cap, w.cnt + kDetValid, heads, w.scan_scratch, w.cnt + kDetCells, stream);
  det_unique_kernel<<<g, 256, 0, stream>>>(skey, heads, w.cnt, ukey, ustart);
  det_gather_kernel<<<g, 256, 0, stream>>>(sval, w.cnt, w.rec, w.pay);
  DetReduceParams q{keys, w.cnt, ukey, ustart, w.pay, w.ray_g, grad_feat, grad_tsdf};
  for (int cls = 0; cls < 8; cls++) {
    const dim3 g(num_sms() * 8), blk(256);
    if (C == 16) {
      if (grad_tsdf) det_class_kernel<16, true><<<g, blk, 0, stream>>>(q, cls);
      else det_class_kernel<16, false><<<g, blk, 0, stream>>>(q, cls);
    } else {
      if (grad_tsdf) det_class_kernel<3, true><<<g, blk, 0, stream>>>(q, cls);
      else det_class_kernel<3, false><<<g, blk, 0, stream>>>(q, cls);
    }
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}

}  // namespace sg
