// intersect.cu -- ray / two-level tree intersection on sm_103a.
//
// Replaces intersection_kernel.cu (SAILOR c_lib/VoxelEncoding/src):
//   RayVoxelIntersection :36-71, RayVoxelIntersectionNodeListNew :128-284,
//   ray_voxel_traversal :286-439, MultiLayerOctree::voxel_traversal :828-895.
//
// One thread per ray walks the top grid with the reference's Amanatides-Woo
// DDA (same float operations, so the same cells in the same order).  At a
// kept brick the brick's node index comes from the dense brick map and the
// set bits of the brick's fine-occupancy mask give its children in
// ascending order -- the reference's lexicographic children order -- each
// slab-tested with geometry recomputed from its index (the reference copies
// a ~1.1 KB node per test).  The default variant (intersect_kernel) tests
// them in the ray's own thread, visiting only the children the ray can
// reach: per x-slab of the brick (slabs without occupied cells skipped) the
// reachable y/z ranges, and in each (x, y) row of the range the set bits of
// the occupancy mask within the z range, in ascending order; the
// warp-cooperative variant (intersect_warp_kernel, tune knob
// SG_TUNE_ISECT_WARP) tests every occupied child of a hit brick with the
// whole warp, one brick at a time -- the same rows, but measured about 8x
// slower at 8^3 bricks, where the reach test leaves ~1/5 of the children.  Hits are appended to the
// ray's row; the reference's -1 padding of the row tail is written by a
// second, warp-per-row kernel with coalesced 16-byte stores.
//
// With the tree's kept-brick bounds (SgTree.brick_box) the walk stops once
// it has passed them on an axis -- every later cell is empty, so the rows,
// counts and valid lengths are those of the full walk.
//
// Isolated occupied bricks (no occupied neighbour, hence not nodes) are
// treated as empty.  The reference instead looks up node index == the
// brick's local id there, i.e. an unrelated node.
#include "common.cuh"

namespace sg {

struct IsectParams {
  SgTree t;
  const float *ori, *dir;
  int N, W, th_early_stop, opt_num, is_training;
  int *hit_idx;
  float *hit_t0, *hit_t1, *valid_len;
  int *hit_count;
  SgStatus *st;
  long R;                               // rays of the launch
  int nseg;                             // 0: frames of N rays; else ray segments
  const int *seg_begin, *seg_frame;
  const float *cams;                    // segments given as cameras (rays generated here)
  const int *cam_w;
};

__global__ void __launch_bounds__(512) intersect_kernel(IsectParams p) {
  const SgTree &t = p.t;
  const long R = p.R;
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int cnt = 0;
  bool over = false;
  if (r < R) {
    const int sgm = p.nseg > 0 ? segment_of(p.seg_begin, p.nseg, r) : 0;
    const int b = p.nseg > 0 ? __ldg(p.seg_frame + sgm) : (int)(r / p.N);
    const float *bb = t.vol_bbox + 6 * b;
    const float bmin[3] = {bb[0], bb[2], bb[4]};
    const float xc = (bb[0] + bb[1]) / 2.0f, yc = (bb[2] + bb[3]) / 2.0f, zc = (bb[4] + bb[5]) / 2.0f;
    const float vs = t.voxel_size[b];
    const float vs_top = vs * (float)(t.Db / t.Dt);
    const float bst[3] = {bb[0] - vs / 2.0f, bb[2] - vs / 2.0f, bb[4] - vs / 2.0f};
    float o[3], d[3];
    segment_ray(p.ori, p.dir, p.cams, p.cam_w, p.seg_begin, sgm, r, o, d);
    const float inv[3] = {__fdividef(1.0f, d[0]), __fdividef(1.0f, d[1]), __fdividef(1.0f, d[2])};
    const LevelGeom gt = level_geom(vs, t.Db / t.Dt);
    const LevelGeom gb = level_geom(vs, 1);
    const int mw = sg_mask_words_dev(t.rate);
    const long vt = (long)t.Dt * t.Dt * t.Dt;
    int *oi = p.hit_idx + (size_t)r * p.W;
    float *o0 = p.hit_t0 + (size_t)r * p.W, *o1 = p.hit_t1 + (size_t)r * p.W;
    float vlen = 0.0f;
    float T0, T1;
    if (slab(o, inv, xc, yc, zc, vs_top * (float)t.Dt, T0, T1) && !(T0 < 0.0f || T1 < 0.0f)) {
      float so[3];
      int st[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        float sp = __fmaf_rn(T0, d[a], o[a]);
        so[a] = sp - bst[a];
        int s = (int)(so[a] / vs_top);
        s = s < 0 ? 0 : s;
        st[a] = s < t.Dt ? s : t.Dt - 1;
      }
      float step[3], tm[3], td[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        step[a] = (d[a] >= 0) ? 1.0f : -1.0f;
        float nb = (step[a] > 0) ? ((float)st[a] + step[a]) * vs_top : (float)st[a] * vs_top;
        tm[a] = (d[a] != 0) ? (nb - so[a]) / d[a] : 9999999.0f;
        td[a] = (d[a] != 0) ? vs_top / d[a] * step[a] : 9999999.0f;
      }
      const int J = 4 * t.Dt;
      bool pre_empty = false, has_valid = false;
      int nsucc = 0, nint = 0;
      // the frame's kept-brick bounds: cells outside hold no node, and once
      // the walk has passed them on an axis no node can follow
      int blo[3] = {0, 0, 0}, bhi[3] = {t.Dt - 1, t.Dt - 1, t.Dt - 1};
      if (t.brick_box) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
          blo[a] = __ldg(t.brick_box + 6 * b + a);
          bhi[a] = __ldg(t.brick_box + 6 * b + 3 + a);
        }
      }
      for (int j = 0; j < J; j++) {
        int rid = -1;
        bool inside = true, past = false;
#pragma unroll
        for (int a = 0; a < 3; a++) {
          inside = inside && st[a] >= blo[a] && st[a] <= bhi[a];
          past = past || (step[a] > 0 ? st[a] > bhi[a] : st[a] < blo[a]);
        }
        if (past) break;
        long brick = (long)b * vt + ((long)st[0] * t.Dt + st[1]) * t.Dt + st[2];
        int k = inside ? t.brick_node[brick] : -1;
        if (k >= 0) {
          float p0, p1;
          if (slab(o, inv, node_coord(gt, bmin[0], st[0]), node_coord(gt, bmin[1], st[1]),
                   node_coord(gt, bmin[2], st[2]), gt.vs, p0, p1) &&
              !(p0 < 0.0f || p1 < 0.0f)) {
            if (!p.is_training) {
              // Children in lexicographic (x, y, z) order.  Only cells the
              // ray can touch are visited: per x-slab of the brick, the y/z
              // cell ranges of the ray segment inside the parent interval,
              // widened by kMargin voxels (float error of the reference slab
              // test is ~1e-6 of a voxel).  Each occupied candidate then
              // gets the reference slab test, so the hit set and its order
              // equal the reference's full scan over all children.
              const uint32_t *mask = t.brick_mask + (size_t)brick * mw;
              const int cb = t.base_bot + t.top_child_base[k];
              const int r = t.rate;
              const float e0 = node_coord(gb, bmin[0], st[0] * r) - gb.vs * 0.5f;
              const float e1 = node_coord(gb, bmin[1], st[1] * r) - gb.vs * 0.5f;
              const float e2 = node_coord(gb, bmin[2], st[2] * r) - gb.vs * 0.5f;
              const float ivs = 1.0f / gb.vs;
              const float u0 = (o[0] - e0) * ivs, u1 = (o[1] - e1) * ivs, u2 = (o[2] - e2) * ivs;
              const float du0 = d[0] * ivs, du1 = d[1] * ivs, du2 = d[2] * ivs;
              // the candidate ranges only need to contain the cells the
              // ray reaches: a reciprocal's few-ulp error is far inside
              // kMargin, and every candidate gets the exact slab test
              // (slopes too small for a finite reciprocal keep the division)
              const bool rcp = fabsf(du0) > 1e-20f;
              const float idu0 = rcp ? 1.0f / du0 : 0.0f;
              const float tm_ = 1e-4f * (p1 - p0) + 1e-5f * fabsf(p1) + 1e-6f;
              const float tlo = p0 - tm_, thi = p1 + tm_;
              constexpr float kMargin = 0.02f;
              int rword = 0, rbase = 0;  // set bits of mask words [0, rword)
              for (int a = 0; a < r; a++) {
                // an x-slab without occupied cells has no candidate
                const int sb = a * r * r;
                const uint32_t sw = r == 8 ? (__ldg(mask + 2 * a) | __ldg(mask + 2 * a + 1))
                                           : ((__ldg(mask + (sb >> 5)) >> (sb & 31)) & ((1u << (r * r)) - 1u));
                if (sw == 0u) continue;
                float ta, tb;
                if (du0 != 0.0f) {
                  const float n1 = (float)a - kMargin - u0, n2 = (float)a + 1.0f + kMargin - u0;
                  const float q1 = rcp ? n1 * idu0 : n1 / du0, q2 = rcp ? n2 * idu0 : n2 / du0;
                  ta = fminf(q1, q2);
                  tb = fmaxf(q1, q2);
                } else {
                  if (u0 < (float)a - kMargin || u0 > (float)a + 1.0f + kMargin) continue;
                  ta = tlo;
                  tb = thi;
                }
                ta = fmaxf(ta, tlo);
                tb = fminf(tb, thi);
                if (ta > tb) continue;
                float ya = u1 + ta * du1, yb = u1 + tb * du1;
                float za = u2 + ta * du2, zb = u2 + tb * du2;
                int y0 = max(0, (int)floorf(fminf(ya, yb) - kMargin));
                int y1 = min(r - 1, (int)floorf(fmaxf(ya, yb) + kMargin));
                int z0 = max(0, (int)floorf(fminf(za, zb) - kMargin));
                int z1 = min(r - 1, (int)floorf(fmaxf(za, zb) + kMargin));
                // occupied candidates only: row (a, y) of the mask is r
                // bits inside one word; its set bits in [z0, z1] in order
                const uint32_t zsel = ((2u << z1) - 1u) & ~((1u << z0) - 1u);
                for (int y = y0; y <= y1; y++) {
                  const int row = (a * r + y) * r;
                  const uint32_t word = __ldg(mask + (row >> 5));
                  uint32_t zbits = (word >> (row & 31)) & zsel;
                  while (zbits) {
                    const int z = __ffs(zbits) - 1;
                    zbits &= zbits - 1u;
                    const int c = row + z;
                    float c0, c1;
                    if (slab(o, inv, node_coord(gb, bmin[0], st[0] * r + a),
                             node_coord(gb, bmin[1], st[1] * r + y), node_coord(gb, bmin[2], st[2] * r + z),
                             gb.vs, c0, c1) &&
                        !(c0 < 0.0f || c1 < 0.0f)) {
                      // children are visited in ascending c: the set bits
                      // of the words below c's word are counted once each
                      while (rword < (c >> 5)) rbase += __popc(__ldg(mask + rword++));
                      const int rank = rbase + __popc(word & ((1u << (c & 31)) - 1u));
                      if (cnt < p.W) {
                        oi[cnt] = cb + rank;
                        o0[cnt] = c0;
                        o1[cnt] = c1;
                      } else {
                        over = true;
                      }
                      vlen = vlen + (c1 - c0) * 4.0f;
                      cnt++;
                    }
                  }
                }
              }
            }
            if (cnt < p.W) {
              oi[cnt] = t.base_top + k;
              o0[cnt] = p0;
              o1[cnt] = p1;
            } else {
              over = true;
            }
            vlen = vlen + (p1 - p0);
            cnt++;
            rid = cnt - 1;
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
        st[ax] = (int)((float)st[ax] + step[ax]);
        tm[ax] += td[ax];
        if (st[0] < 0 || st[0] >= t.Dt || st[1] < 0 || st[1] >= t.Dt || st[2] < 0 || st[2] >= t.Dt) break;
      }
    }
    p.valid_len[r] = vlen;
    if (p.hit_count) p.hit_count[r] = cnt;
  }
  // warp-aggregated status updates
  int m = cnt;
#pragma unroll
  for (int o2 = 16; o2 > 0; o2 >>= 1) m = max(m, __shfl_xor_sync(SG_FULL, m, o2));
  bool anyover = __any_sync(SG_FULL, over);
  if (lane_id() == 0 && p.st) {
    if (m > 0) atomicMax(&p.st->max_hits, m);
    if (anyover) atomicOr(&p.st->flags, SG_FLAG_HIT_OVERFLOW);
  }
}

// ---------------------------------------------------------------------------
// Warp-cooperative variant: each lane walks its own ray's DDA (the same
// float operations, hence the same cells), but the children of a hit brick
// are tested by the whole warp: lane l takes children 32 i + l (i over the
// brick's 32-bit mask words), so one warp instruction covers 32 children in
// lexicographic order; a ballot of the hits and a popcount of the lanes
// before give each hit its row position, and the mask bits before a child
// its node rank.  Hit bricks of different lanes in the same DDA step are
// served one after another in lane order, so every ray's row is in the
// reference's order (per brick: children in lexicographic order, then the
// brick).  The valid length is summed hit by hit in row order, as the
// reference sums it.  The DDA state stays in registers (per-axis selects).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) intersect_warp_kernel(IsectParams p) {
  const SgTree &t = p.t;
  const long R = p.R;
  const int lane = lane_id();
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = r < R;
  int cnt = 0;
  bool over = false;
  float vlen = 0.0f;
  int b = 0;
  float o[3] = {0.0f, 0.0f, 0.0f}, d[3] = {1.0f, 1.0f, 1.0f}, inv[3] = {1.0f, 1.0f, 1.0f};
  float bmin[3] = {0.0f, 0.0f, 0.0f};
  float vs = 1.0f;
  int st0 = 0, st1 = 0, st2 = 0;
  float tm0 = 0.0f, tm1 = 0.0f, tm2 = 0.0f, td0 = 0.0f, td1 = 0.0f, td2 = 0.0f;
  int sp0 = 1, sp1 = 1, sp2 = 1;
  bool active = false;
  const long vt = (long)t.Dt * t.Dt * t.Dt;
  if (in) {
    const int sgm = p.nseg > 0 ? segment_of(p.seg_begin, p.nseg, r) : 0;
    b = p.nseg > 0 ? __ldg(p.seg_frame + sgm) : (int)(r / p.N);
    const float *bb = t.vol_bbox + 6 * b;
    bmin[0] = bb[0];
    bmin[1] = bb[2];
    bmin[2] = bb[4];
    const float xc = (bb[0] + bb[1]) / 2.0f, yc = (bb[2] + bb[3]) / 2.0f, zc = (bb[4] + bb[5]) / 2.0f;
    vs = t.voxel_size[b];
    const float vs_top = vs * (float)(t.Db / t.Dt);
    const float bst[3] = {bb[0] - vs / 2.0f, bb[2] - vs / 2.0f, bb[4] - vs / 2.0f};
    segment_ray(p.ori, p.dir, p.cams, p.cam_w, p.seg_begin, sgm, r, o, d);
#pragma unroll
    for (int a = 0; a < 3; a++) inv[a] = __fdividef(1.0f, d[a]);
    float T0, T1;
    if (slab(o, inv, xc, yc, zc, vs_top * (float)t.Dt, T0, T1) && !(T0 < 0.0f || T1 < 0.0f)) {
      float so[3];
      int st[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        float spos = __fmaf_rn(T0, d[a], o[a]);
        so[a] = spos - bst[a];
        int s = (int)(so[a] / vs_top);
        s = s < 0 ? 0 : s;
        st[a] = s < t.Dt ? s : t.Dt - 1;
      }
      float step[3], tm[3], td[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        step[a] = (d[a] >= 0) ? 1.0f : -1.0f;
        float nb = (step[a] > 0) ? ((float)st[a] + step[a]) * vs_top : (float)st[a] * vs_top;
        tm[a] = (d[a] != 0) ? (nb - so[a]) / d[a] : 9999999.0f;
        td[a] = (d[a] != 0) ? vs_top / d[a] * step[a] : 9999999.0f;
      }
      st0 = st[0], st1 = st[1], st2 = st[2];
      tm0 = tm[0], tm1 = tm[1], tm2 = tm[2];
      td0 = td[0], td1 = td[1], td2 = td[2];
      sp0 = (int)step[0], sp1 = (int)step[1], sp2 = (int)step[2];
      active = true;
    }
  }
  int *oi = p.hit_idx + (size_t)(in ? r : 0) * p.W;
  float *o0 = p.hit_t0 + (size_t)(in ? r : 0) * p.W, *o1 = p.hit_t1 + (size_t)(in ? r : 0) * p.W;
  const int rate = t.rate, r3 = rate * rate * rate;
  const int mw = sg_mask_words_dev(rate);
  bool pre_empty = false, has_valid = false;
  int nsucc = 0, nint = 0;
  const int J = 4 * t.Dt;
  for (int j = 0; j < J; j++) {
    if (!__any_sync(SG_FULL, active)) break;
    // this step's brick of every active lane: a node whose box the ray enters
    bool pend = false;
    int k = -1;
    float p0 = 0.0f, p1 = 0.0f;
    if (active) {
      const long brick = (long)b * vt + ((long)st0 * t.Dt + st1) * t.Dt + st2;
      k = t.brick_node[brick];
      if (k >= 0) {
        const LevelGeom gt = level_geom(vs, t.Db / t.Dt);
        pend = slab(o, inv, node_coord(gt, bmin[0], st0), node_coord(gt, bmin[1], st1), node_coord(gt, bmin[2], st2),
                    gt.vs, p0, p1) &&
               !(p0 < 0.0f || p1 < 0.0f);
      }
    }
    int rid = -1;
    if (!p.is_training) {
      // children of the pending bricks, one brick at a time in lane order
      unsigned pm = __ballot_sync(SG_FULL, pend);
      while (pm) {
        const int L = __ffs(pm) - 1;
        pm &= pm - 1;
        const float oL[3] = {__shfl_sync(SG_FULL, o[0], L), __shfl_sync(SG_FULL, o[1], L),
                             __shfl_sync(SG_FULL, o[2], L)};
        const float iL[3] = {__shfl_sync(SG_FULL, inv[0], L), __shfl_sync(SG_FULL, inv[1], L),
                             __shfl_sync(SG_FULL, inv[2], L)};
        const float bL[3] = {__shfl_sync(SG_FULL, bmin[0], L), __shfl_sync(SG_FULL, bmin[1], L),
                             __shfl_sync(SG_FULL, bmin[2], L)};
        const int sx = __shfl_sync(SG_FULL, st0, L), sy = __shfl_sync(SG_FULL, st1, L),
                  sz = __shfl_sync(SG_FULL, st2, L);
        const int fL = __shfl_sync(SG_FULL, b, L);
        const int kL = __shfl_sync(SG_FULL, k, L);
        const long rL = __shfl_sync(SG_FULL, (long long)(in ? r : 0), L);
        int base = __shfl_sync(SG_FULL, cnt, L);
        float vl = __shfl_sync(SG_FULL, vlen, L);
        const LevelGeom gb = level_geom(__shfl_sync(SG_FULL, vs, L), 1);
        const long brickL = (long)fL * vt + ((long)sx * t.Dt + sy) * t.Dt + sz;
        const uint32_t *mask = t.brick_mask + (size_t)brickL * mw;
        const int cb = t.base_bot + t.top_child_base[kL];
        int *oiL = p.hit_idx + (size_t)rL * p.W;
        float *o0L = p.hit_t0 + (size_t)rL * p.W, *o1L = p.hit_t1 + (size_t)rL * p.W;
        const int x0 = sx * rate, y0 = sy * rate, z0 = sz * rate;
        int rank0 = 0;
        bool ovL = false;
        for (int i = 0; i < mw; i++) {
          const uint32_t word = __ldg(mask + i);
          const int c = 32 * i + lane;
          bool hit = false;
          float c0 = 0.0f, c1 = 0.0f;
          if (c < r3 && ((word >> lane) & 1u)) {
            const int a = c / (rate * rate), y = (c / rate) % rate, z = c % rate;
            hit = slab(oL, iL, node_coord(gb, bL[0], x0 + a), node_coord(gb, bL[1], y0 + y),
                       node_coord(gb, bL[2], z0 + z), gb.vs, c0, c1) &&
                  !(c0 < 0.0f || c1 < 0.0f);
          }
          const unsigned hb = __ballot_sync(SG_FULL, hit);
          if (hit) {
            const int pos = base + __popc(hb & ((1u << lane) - 1u));
            if (pos < p.W) {
              oiL[pos] = cb + rank0 + __popc(word & ((1u << lane) - 1u));
              o0L[pos] = c0;
              o1L[pos] = c1;
            }
          }
          // the ray's valid length, hit by hit in row order
          const float len4 = (c1 - c0) * 4.0f;
          for (unsigned m = hb; m; m &= m - 1) vl = vl + __shfl_sync(SG_FULL, len4, __ffs(m) - 1);
          if (base + __popc(hb) > p.W) ovL = true;
          base += __popc(hb);
          rank0 += __popc(word);
        }
        if (lane == L) {
          cnt = base;
          vlen = vl;
          over = over || ovL;
        }
      }
    }
    if (pend) {
      if (cnt < p.W) {
        oi[cnt] = t.base_top + k;
        o0[cnt] = p0;
        o1[cnt] = p1;
      } else {
        over = true;
      }
      vlen = vlen + (p1 - p0);
      cnt++;
      rid = cnt - 1;
    }
    if (active) {
      if (p.th_early_stop > -1) {
        if (rid == -1) {
          if (pre_empty && has_valid) nsucc++;
          pre_empty = true;
        } else {
          nsucc = 0;
          pre_empty = false;
          has_valid = true;
        }
        if ((nsucc + 1) >= p.th_early_stop) active = false;
      }
      if (p.opt_num > -1) {
        if (rid + 1 > 0) nint++;
        if (nint >= p.opt_num) active = false;
      }
    }
    if (active) {
      int ax;
      if (tm0 < tm1) ax = (tm0 < tm2) ? 0 : 2;
      else ax = (tm1 < tm2) ? 1 : 2;
      if (ax == 0) {
        st0 = (int)((float)st0 + (float)sp0);
        tm0 += td0;
      } else if (ax == 1) {
        st1 = (int)((float)st1 + (float)sp1);
        tm1 += td1;
      } else {
        st2 = (int)((float)st2 + (float)sp2);
        tm2 += td2;
      }
      if (st0 < 0 || st0 >= t.Dt || st1 < 0 || st1 >= t.Dt || st2 < 0 || st2 >= t.Dt) active = false;
    }
  }
  if (in) {
    p.valid_len[r] = vlen;
    if (p.hit_count) p.hit_count[r] = cnt;
  }
  int m = cnt;
#pragma unroll
  for (int o2 = 16; o2 > 0; o2 >>= 1) m = max(m, __shfl_xor_sync(SG_FULL, m, o2));
  const bool anyover = __any_sync(SG_FULL, over);
  if (lane == 0 && p.st) {
    if (m > 0) atomicMax(&p.st->max_hits, m);
    if (anyover) atomicOr(&p.st->flags, SG_FLAG_HIT_OVERFLOW);
  }
}

// -1 padding of row tails [count, W): warp per row
__global__ void pad_rows_kernel(long R, int W, const int *__restrict__ count, int *idx, float *t0,
                                float *t1) {
  const int lane = lane_id();
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    pad_row_tail(idx, t0, t1, (size_t)r * W, min(count[r], W), W, lane);
  }
}

void launch_pad_rows(long R, int W, const int *count, int *idx, float *t0, float *t1, sg_stream_t stream) {
  if (R <= 0 || W <= 0) return;
  int g = ceil_div(R * 32, 256);
  if (g > num_sms() * 64) g = num_sms() * 64;
  pad_rows_kernel<<<g, 256, 0, stream>>>(R, W, count, idx, t0, t1);
}

}  // namespace sg

using namespace sg;

extern "C" int sg_intersect(const SgTree *tree, const float *ori, const float *dir, int N, int W,
                            int th_early_stop, int opt_num, int is_training, int padded, int *hit_idx,
                            float *hit_t0, float *hit_t1, float *valid_len, int *hit_count,
                            SgStatus *status, sg_stream_t stream) {
  if (!tree || !ori || !dir || !hit_idx || !hit_t0 || !hit_t1 || !valid_len) return SG_ERR_INVALID_ARG;
  if (N <= 0 || W <= 0 || tree->B <= 0 || tree->Dt <= 0 || tree->Db != tree->Dt * tree->rate)
    return SG_ERR_INVALID_ARG;
  if (padded && !hit_count) return SG_ERR_INVALID_ARG;
  if (padded && (((uintptr_t)hit_idx) | ((uintptr_t)hit_t0) | ((uintptr_t)hit_t1)) % 16 != 0)
    return SG_ERR_INVALID_ARG;
  long R = (long)tree->B * N;
  IsectParams p{*tree, ori, dir, N, W, th_early_stop, opt_num, is_training,
                hit_idx, hit_t0, hit_t1, valid_len, hit_count, status, R, 0, nullptr, nullptr, nullptr, nullptr};
  if (tune(SG_TUNE_ISECT_WARP)) {
    intersect_warp_kernel<<<ceil_div(R, 256), 256, 0, stream>>>(p);
  } else {
    const int blk = tune(SG_TUNE_ISECT_BLOCK);
    intersect_kernel<<<ceil_div(R, blk), blk, 0, stream>>>(p);
  }
  if (padded) launch_pad_rows(R, W, hit_count, hit_idx, hit_t0, hit_t1, stream);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_intersect_segments(const SgTree *tree, const SgRaySegments *seg, const float *ori,
                                     const float *dir, int W, int *hit_idx, float *hit_t0, float *hit_t1,
                                     float *valid_len, int *hit_count, SgStatus *status, sg_stream_t stream) {
  if (!tree || !seg || !hit_idx || !hit_t0 || !hit_t1 || !valid_len || !hit_count) return SG_ERR_INVALID_ARG;
  if ((seg->cameras == nullptr) != (seg->widths == nullptr)) return SG_ERR_INVALID_ARG;
  if (!seg->cameras && (!ori || !dir)) return SG_ERR_INVALID_ARG;
  if (seg->count <= 0 || seg->total < 0 || !seg->ray_begin || !seg->frame) return SG_ERR_INVALID_ARG;
  if (W <= 0 || tree->B <= 0 || tree->Dt <= 0 || tree->Db != tree->Dt * tree->rate) return SG_ERR_INVALID_ARG;
  if (seg->total == 0) return SG_OK;
  IsectParams p{*tree, ori, dir, 1, W, -1, -1, 0, hit_idx, hit_t0, hit_t1, valid_len, hit_count, status,
                (long)seg->total, seg->count, seg->ray_begin, seg->frame, seg->cameras, seg->widths};
  if (tune(SG_TUNE_ISECT_WARP)) {
    intersect_warp_kernel<<<ceil_div((long)seg->total, 256), 256, 0, stream>>>(p);
  } else {
    const int blk = tune(SG_TUNE_ISECT_BLOCK);
    intersect_kernel<<<ceil_div((long)seg->total, blk), blk, 0, stream>>>(p);
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}
