/*
 * octree_oracle.c -- CPU restatement of SAILOR's multi-level tree, its
 * depth-first ray traversal and the fine adaptive sampler.
 *
 * TEST INFRASTRUCTURE ONLY (linked into oracle/liboracle.so with
 * sailor_oracle.c): tests and the smoke check call it as the checker; the
 * CUDA library never links or calls it.
 *
 *   orc_octree_build      gen_root_octree_nodes + gen_higher_octree_nodes
 *                         (c_lib/VoxelEncoding/src/octree_kernel.cu:18-99,
 *                         101-239; host MultiLayerOctree::build_octree
 *                         :654-697)
 *   orc_octree_traversal  MultiLayerOctree::octree_traversal
 *                         (intersection_kernel.cu:722-826): ray_voxel_
 *                         traversal with only_voxel_traversal = false
 *                         (:286-439, RayVoxelIntersectionNodeList :72-126),
 *                         then ray_octree_traversal (:441-643)
 *   orc_sample_fine       MultiLayerOctree::ray_voxels_points_sampling
 *                         (sampling_kernel.cu:1178-1248):
 *                         ray_voxels_sampling_kernel (:911-985) and
 *                         ray_voxels_further_sampling_kernel (:987-1068)
 *
 * Layout.  Levels l = 0 (finest, edge dims[0]) .. L-1 (top), dims[l] =
 * dims[0] / rate^l.  vol concatenates the L occupancy volumes, level l at
 * sum_{i<l} B*dims[i]^3.  The node tables (key = b*dims[l]^3 + linear index,
 * parent id, child_base, nchild) concatenate the levels, level l at
 * sum_{i<l} cap[i]; node k of level l has id base[l] + k.
 *
 * Order.  The reference hands out node ids, fine-row slots and sample slots
 * with atomicAdd, so all three change run to run.  This restatement takes
 * the order a sequential run of the same loops gives: top nodes by
 * (frame, linear index), children per parent in the reference's insertion
 * order (x, y, z ascending); fine rows coarse node by coarse node, each in
 * the reference's own per-thread order (its stack pops children last to
 * first); sample slots entry by entry.  Comparisons with the reference's
 * outputs are set-wise (per ray, multisets of canonical node keys with their
 * depths).
 *
 * The reference's descent keeps an 8-entry stack and an 8-entry list per
 * coarse node (N_STACK_MAX_NODES, intersection_kernel.cu:15) and writes past
 * them when a node has more than 8 children or the descent goes more than
 * one level below the coarse node; the restatement has no such limit and
 * reports, per ray, the largest stack and list the reference would need
 * (need[]) so that a caller runs the reference only where they fit.
 *
 * Near ties.  The reference's slab test multiplies by __fdividef(1, d); the
 * restatement uses the correctly rounded 1/d.  Decisions that an ulp of
 * difference can flip set FLAG_TIE on the ray: slab hit/miss margins, DDA
 * crossings and start cells, the bit-for-bit (t0, t1) comparison of the
 * descent (equal is robust only when both depths come from the same face
 * plane, with no near tie in choosing it), sample counts near an integer and
 * midpoint ties in the fill step.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define TIE_REL 1e-5
#define FLAG_TIE 1
#define FLAG_OVERFLOW 4
#define FLAG_TRUNC 8 /* entries ask for more than S samples: the reference's */
                     /* truncation then depends on atomic arrival order      */

/* node geometry (calculate_bbox_start + calculate_xyz_corners, octree.h:109-151) */
void orc_node_geometry(float vs_bottom, int size, const float *bbox_min3, const int *idx3, float *centre3,
                       float *node_vs);

static inline int near_eq(double a, double b) {
  if (!isfinite(a) || !isfinite(b)) return 0;
  double m = fabs(a) > fabs(b) ? fabs(a) : fabs(b);
  return fabs(a - b) <= TIE_REL * m + 1e-30;
}

static inline int dda_tie(float a, float b) {
  if (a == 9999999.0f && b == 9999999.0f) return 0;
  return near_eq(a, b);
}

typedef struct {
  int B, L, rate;
  const int *dims, *base, *cap, *counts;
  const int *key, *child_base, *nchild; /* concatenated */
  long coff[16];
  long voff[16];
  const float *voxel_size, *vol_bbox;
} oct_t;

static void oct_init(oct_t *t, int B, int L, int rate, const int *dims, const int *base, const int *cap,
                     const int *counts, const int *key, const int *child_base, const int *nchild,
                     const float *voxel_size, const float *vol_bbox) {
  t->B = B;
  t->L = L;
  t->rate = rate;
  t->dims = dims;
  t->base = base;
  t->cap = cap;
  t->counts = counts;
  t->key = key;
  t->child_base = child_base;
  t->nchild = nchild;
  t->voxel_size = voxel_size;
  t->vol_bbox = vol_bbox;
  long c = 0, v = 0;
  for (int l = 0; l < L; l++) {
    t->coff[l] = c;
    t->voff[l] = v;
    c += cap[l];
    v += (long)B * dims[l] * dims[l] * dims[l];
  }
}

static int level_of(const oct_t *t, int id) {
  for (int l = t->L - 1; l >= 0; l--)
    if (id >= t->base[l] && id < t->base[l] + t->cap[l]) return l;
  return -1;
}

/* centre and edge of node k of level l */
static void oct_geom(const oct_t *t, int l, int k, float c[3], float *nvs, int *frame) {
  long D = t->dims[l];
  long vt = D * D * D;
  long key = t->key[t->coff[l] + k];
  int b = (int)(key / vt);
  long lin = key - (long)b * vt;
  int idx[3] = {(int)(lin / (D * D)), (int)((lin / D) % D), (int)(lin % D)};
  float bmin[3] = {t->vol_bbox[b * 6 + 0], t->vol_bbox[b * 6 + 2], t->vol_bbox[b * 6 + 4]};
  orc_node_geometry(t->voxel_size[b], t->dims[0] / t->dims[l], bmin, idx, c, nvs);
  if (frame) *frame = b;
}

/* ------------------------------------------------------------------------ */
/* Tree build.  Returns 0, or -1 when a level's capacity is exceeded         */
/* (counts[] then hold what was built).                                      */
/* ------------------------------------------------------------------------ */
int orc_octree_build(int B, int L, int rate, const int *dims, int *vol, const int *base, const int *cap,
                     int *key, int *parent, int *child_base, int *nchild, int *counts) {
  long coff[16], voff[16];
  long c = 0, v = 0;
  for (int l = 0; l < L; l++) {
    coff[l] = c;
    voff[l] = v;
    c += cap[l];
    v += (long)B * dims[l] * dims[l] * dims[l];
    counts[l] = 0;
  }
  int T = L - 1;
  long Dt = dims[T], vt = Dt * Dt * Dt;
  int *vtop = vol + voff[T];
  unsigned char *keep = (unsigned char *)calloc((size_t)B * vt + 1, 1);
  for (long i = 0; i < (long)B * vt; i++) {
    if (vtop[i] <= -1) continue;
    int b = (int)(i / vt);
    long lin = i - (long)b * vt;
    int x = (int)(lin / (Dt * Dt)), y = (int)((lin / Dt) % Dt), z = (int)(lin % Dt);
    int found = 0;
    for (int a = x - 1; a <= x + 1 && !found; a++)
      for (int m = y - 1; m <= y + 1 && !found; m++)
        for (int n = z - 1; n <= z + 1; n++) {
          if (a < 0 || a >= Dt || m < 0 || m >= Dt || n < 0 || n >= Dt || (a == x && m == y && n == z)) continue;
          if (vtop[(long)b * vt + ((long)a * Dt + m) * Dt + n] > -1) { found = 1; break; }
        }
    keep[i] = (unsigned char)found;
  }
  int nt = 0;
  for (long i = 0; i < (long)B * vt; i++) {
    if (!keep[i]) continue;
    if (nt >= cap[T]) { free(keep); counts[T] = nt; return -1; }
    key[coff[T] + nt] = (int)i;
    parent[coff[T] + nt] = -1;
    vtop[i] = base[T] + nt;
    nt++;
  }
  free(keep);
  counts[T] = nt;
  for (int l = T; l >= 1; l--) {
    long Dp = dims[l], vp = Dp * Dp * Dp;
    long Dc = dims[l - 1], vc = Dc * Dc * Dc;
    int *vchild = vol + voff[l - 1];
    int nc_total = 0;
    for (int k = 0; k < counts[l]; k++) {
      long kk = key[coff[l] + k];
      int b = (int)(kk / vp);
      long lin = kk - (long)b * vp;
      int X = (int)(lin / (Dp * Dp)), Y = (int)((lin / Dp) % Dp), Z = (int)(lin % Dp);
      child_base[coff[l] + k] = nc_total;
      int nc = 0;
      for (int a = 0; a < rate; a++)
        for (int m = 0; m < rate; m++)
          for (int n = 0; n < rate; n++) {
            long cl = ((long)(X * rate + a) * Dc + (Y * rate + m)) * Dc + (Z * rate + n);
            long ci = (long)b * vc + cl;
            if (vchild[ci] > -1) {
              if (nc_total >= cap[l - 1]) { counts[l - 1] = nc_total; return -1; }
              key[coff[l - 1] + nc_total] = (int)ci;
              parent[coff[l - 1] + nc_total] = base[l] + k;
              vchild[ci] = base[l - 1] + nc_total;
              nc_total++;
              nc++;
            }
          }
      nchild[coff[l] + k] = nc;
    }
    counts[l - 1] = nc_total;
  }
  return 0;
}

/* Slab test (RayVoxelIntersection, intersection_kernel.cu:36-71) that also */
/* reports where t0 and t1 come from: the axis and the face coordinate     */
/* (centre -/+ half edge) that won, or axis -1 for the initial 0 / 1e5.    */
/* *tie: a hit/miss margin; *seltie: a near tie in choosing t0 or t1.       */
typedef struct {
  float t0, t1;
  int ax0, ax1;
  float pl0, pl1;
  int seltie;
} hit_t;

static int slab_src(const float o[3], const float inv[3], const float c[3], float vs, hit_t *h, int *tie) {
  float f_low = 0.0f, f_high = 100000.0f;
  int a0 = -1, a1 = -1;
  float p0 = 0.0f, p1 = 0.0f;
  float half = vs / 2.0f;
  int sel = 0;
  for (int i = 0; i < 3; i++) {
    float pl_lo = c[i] - half, pl_hi = c[i] + half;
    float lo = (pl_lo - o[i]) * inv[i];
    float hi = (pl_hi - o[i]) * inv[i];
    if (lo > hi) {
      float t = lo; lo = hi; hi = t;
      t = pl_lo; pl_lo = pl_hi; pl_hi = t;
    }
    if (near_eq(hi, f_low) || near_eq(lo, f_high)) *tie = 1;
    if (hi < f_low) return 0;
    if (lo > f_high) return 0;
    if (near_eq(lo, f_low) && a0 >= 0) sel = 1;
    if (near_eq(hi, f_high) && a1 >= 0) sel = 1;
    if (lo > f_low) { f_low = lo; a0 = i; p0 = pl_lo; }
    if (hi < f_high) { f_high = hi; a1 = i; p1 = pl_hi; }
    if (near_eq(f_low, f_high)) *tie = 1;
    if (f_low > f_high) return 0;
  }
  h->t0 = f_low;
  h->t1 = f_high;
  h->ax0 = a0;
  h->ax1 = a1;
  h->pl0 = p0;
  h->pl1 = p1;
  h->seltie = sel;
  return 1;
}

/* the descent's bit-for-bit depth comparison; *tie when an ulp could flip it */
static int same_depths(const hit_t *a, const hit_t *b, int *tie) {
  int eq = (a->t0 == b->t0 && a->t1 == b->t1);
  int near = near_eq(a->t0, b->t0) && near_eq(a->t1, b->t1);
  if (near) {
    int robust = eq && a->ax0 == b->ax0 && a->ax1 == b->ax1 && a->pl0 == b->pl0 && a->pl1 == b->pl1 &&
                 !a->seltie && !b->seltie;
    if (!robust) *tie = 1;
  }
  return eq;
}

typedef struct {
  int id;
  hit_t h;
  float vs;
} entry_t;

/* ------------------------------------------------------------------------ */
/* Traversal.  Outputs (prefilled -1 / 0 by the caller): idx_c/t0_c/t1_c     */
/* [R,Wc], cnt_c [R]; idx/t0/t1 [R,Wf], cnt [R]; valid_len [R]; flags [R];   */
/* need [R] = the largest of (stack entries, list entries) the reference's   */
/* descent would use for any coarse node of the ray.  Returns the largest   */
/* fine count.                                                               */
/* ------------------------------------------------------------------------ */
int orc_octree_traversal(int B, int L, int rate, const int *dims, const int *vol, const int *base, const int *cap,
                         const int *counts, const int *key, const int *child_base, const int *nchild,
                         const float *voxel_size, const float *vol_bbox, int N, const float *ori, const float *dir,
                         int start_level, int Wc, int Wf, int th_early_stop, int opt_num, int *idx_c, float *t0_c,
                         float *t1_c, int *cnt_c, int *idx, float *t0, float *t1, int *cnt, float *valid_len,
                         int *flags, int *need) {
  oct_t t;
  oct_init(&t, B, L, rate, dims, base, cap, counts, key, child_base, nchild, voxel_size, vol_bbox);
  const int s = L - 1 - start_level;
  const long Ds = dims[s], vs3 = Ds * Ds * Ds;
  const int *vols = vol + t.voff[s];
  int maxf = 0;
#pragma omp parallel for schedule(dynamic, 32) reduction(max : maxf)
  for (long r = 0; r < (long)B * N; r++) {
    int b = (int)(r / N);
    int fl = 0, cc = 0, fc = 0, nd = 0, tie = 0;
    float vlen = 0.0f;
    const float *bb = vol_bbox + b * 6;
    float cen[3] = {(bb[0] + bb[1]) / 2.0f, (bb[2] + bb[3]) / 2.0f, (bb[4] + bb[5]) / 2.0f};
    float vs = voxel_size[b];
    float vs_top = vs * (float)(dims[0] / dims[s]);
    float bst[3] = {bb[0] - vs / 2.0f, bb[2] - vs / 2.0f, bb[4] - vs / 2.0f};
    float o[3] = {ori[r * 3 + 0], ori[r * 3 + 1], ori[r * 3 + 2]};
    float d[3] = {dir[r * 3 + 0], dir[r * 3 + 1], dir[r * 3 + 2]};
    float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    int *oic = idx_c + (size_t)r * Wc, *oif = idx + (size_t)r * Wf;
    float *o0c = t0_c + (size_t)r * Wc, *o1c = t1_c + (size_t)r * Wc;
    float *o0f = t0 + (size_t)r * Wf, *o1f = t1 + (size_t)r * Wf;
    hit_t whole;
    int ok = slab_src(o, inv, cen, vs_top * (float)Ds, &whole, &tie);
    if (ok && !(whole.t0 < 0.0f || whole.t1 < 0.0f)) {
      float so[3];
      int st[3];
      for (int a = 0; a < 3; a++) {
        float sp = fmaf(whole.t0, d[a], o[a]);
        so[a] = sp - bst[a];
        float q = so[a] / vs_top;
        if (fabsf(q - roundf(q)) < 1e-4f && roundf(q) >= 1.0f && roundf(q) <= (float)(Ds - 1)) tie = 1;
        int sc = (int)q;
        sc = sc < 0 ? 0 : sc;
        st[a] = sc < Ds ? sc : (int)Ds - 1;
      }
      float step[3], tm[3], td[3];
      for (int a = 0; a < 3; a++) {
        step[a] = (d[a] >= 0) ? 1.0f : -1.0f;
        float nb = (step[a] > 0) ? ((float)st[a] + step[a]) * vs_top : (float)st[a] * vs_top;
        tm[a] = (d[a] != 0) ? (nb - so[a]) / d[a] : 9999999.0f;
        td[a] = (d[a] != 0) ? vs_top / d[a] * step[a] : 9999999.0f;
      }
      int J = 4 * (int)Ds;
      int pre_empty = 0, has_valid = 0, nsucc = 0, nint = 0;
      entry_t *list = (entry_t *)malloc(sizeof(entry_t) * 4096);
      int list_cap = 4096;
      for (int j = 0; j < J; j++) {
        int rid = -1;
        long cell = (long)b * vs3 + ((long)st[0] * Ds + st[1]) * Ds + st[2];
        int v = vols[cell];
        int k = v - base[s];
        if (v > -1 && k >= 0 && k < counts[s] && key[t.coff[s] + k] == (int)cell) {
          float c[3], nvs;
          oct_geom(&t, s, k, c, &nvs, NULL);
          hit_t hc;
          if (slab_src(o, inv, c, nvs, &hc, &tie) && !(hc.t0 < 0.0f || hc.t1 < 0.0f)) {
            rid = cc;
            if (cc < Wc) { oic[cc] = v; o0c[cc] = hc.t0; o1c[cc] = hc.t1; } else fl |= FLAG_OVERFLOW;
            cc++;
            /* descent from this coarse node (ray_octree_traversal :441-643) */
            int nl = 0;
            list[nl].id = v;
            list[nl].h = hc;
            list[nl].vs = nvs;
            nl++;
            /* the reference's stack: start pushed (1), popped, children pushed */
            int sp = 0, sp_max = 1;
            /* explicit DFS over (level, local) with children last to first */
            int stl[256], stk[256];
            int top = -1;
            if (s > 0) {
              int cb = child_base[t.coff[s] + k], ncd = nchild[t.coff[s] + k];
              for (int q = 0; q < ncd; q++) { ++top; stl[top] = s - 1; stk[top] = cb + q; }
              sp = ncd;
              if (sp > sp_max) sp_max = sp;
            }
            while (top >= 0) {
              int lv = stl[top], kk = stk[top];
              top--;
              sp--;
              float cc3[3], cvs;
              oct_geom(&t, lv, kk, cc3, &cvs, NULL);
              hit_t h;
              if (!slab_src(o, inv, cc3, cvs, &h, &tie)) continue;
              int found = 0;
              for (int e = 0; e < nl; e++) {
                if (same_depths(&list[e].h, &h, &tie)) {
                  if (list[e].vs > cvs) {
                    list[e].id = base[lv] + kk;
                    list[e].vs = cvs;
                    /* the entry keeps its depths (equal bit for bit) */
                  }
                  found = 1;
                  break;
                }
              }
              if (!found) {
                if (nl >= list_cap) {
                  list_cap *= 2;
                  list = (entry_t *)realloc(list, sizeof(entry_t) * list_cap);
                }
                list[nl].id = base[lv] + kk;
                list[nl].h = h;
                list[nl].vs = cvs;
                nl++;
              }
              if (lv > 0) {
                int ncd = nchild[t.coff[lv] + kk], cb = child_base[t.coff[lv] + kk];
                for (int q = 0; q < ncd; q++) { ++top; stl[top] = lv - 1; stk[top] = cb + q; }
                sp += ncd;
                if (sp > sp_max) sp_max = sp;
              }
            }
            if (sp_max > nd) nd = sp_max;
            if (nl > nd) nd = nl;
            float start_vs = nvs;
            for (int e = 0; e < nl; e++) {
              if (fc < Wf) { oif[fc] = list[e].id; o0f[fc] = list[e].h.t0; o1f[fc] = list[e].h.t1; }
              else fl |= FLAG_OVERFLOW;
              fc++;
              float scale = start_vs / list[e].vs;
              vlen = vlen + (list[e].h.t1 - list[e].h.t0) * scale;
            }
          }
        }
        if (th_early_stop > -1) {
          if (rid == -1) {
            if (pre_empty && has_valid) nsucc++;
            pre_empty = 1;
          } else {
            nsucc = 0;
            pre_empty = 0;
            has_valid = 1;
          }
          if ((nsucc + 1) >= th_early_stop) break;
        }
        if (opt_num > -1) {
          if (rid + 1 > 0) nint++;
          if (nint >= opt_num) break;
        }
        if (dda_tie(tm[0], tm[1]) || dda_tie(tm[0], tm[2]) || dda_tie(tm[1], tm[2])) tie = 1;
        int ax;
        if (tm[0] < tm[1]) ax = (tm[0] < tm[2]) ? 0 : 2;
        else ax = (tm[1] < tm[2]) ? 1 : 2;
        st[ax] += (int)step[ax];
        tm[ax] += td[ax];
        if (st[0] < 0 || st[0] >= Ds || st[1] < 0 || st[1] >= Ds || st[2] < 0 || st[2] >= Ds) break;
      }
      free(list);
    }
    cnt_c[r] = cc;
    cnt[r] = fc;
    valid_len[r] = vlen;
    if (tie) fl |= FLAG_TIE;
    flags[r] = fl;
    need[r] = nd;
    if (fc > maxf) maxf = fc;
  }
  return maxf;
}

/* ------------------------------------------------------------------------ */
/* Fine sampler.  Rows [R,W] read up to their first -1; outputs [R,S]        */
/* prefilled -1 by the caller.  flags[r] gains FLAG_TIE near a count or     */
/* midpoint tie, FLAG_TRUNC when the entries ask for more than S samples.    */
/* ------------------------------------------------------------------------ */
void orc_sample_fine(int B, int L, int rate, const int *dims, const int *base, const int *cap, int N, int W,
                     int S, const int *hit_idx, const float *hit_t0, const float *hit_t1, const float *valid_len,
                     const float *rands, int start_level, const float *voxel_size, int *sampled_idx,
                     float *sampled_z, int *flags) {
  oct_t t;
  oct_init(&t, B, L, rate, dims, base, cap, NULL, NULL, NULL, NULL, voxel_size, NULL);
#pragma omp parallel for schedule(dynamic, 64)
  for (long r = 0; r < (long)B * N; r++) {
    int b = (int)(r / N);
    const int *hi = hit_idx + (size_t)r * W;
    const float *h0 = hit_t0 + (size_t)r * W, *h1 = hit_t1 + (size_t)r * W;
    const float *rd = rands + (size_t)r * S;
    int *si = sampled_idx + (size_t)r * S;
    float *sz = sampled_z + (size_t)r * S;
    float vl = valid_len[r];
    float vsb = voxel_size[b];
    float start_vs = vsb * powf(2.0f, (float)(L - start_level - 1));
    int has = 0, want = 0;
    int nh = 0;
    while (nh < W && hi[nh] != -1) nh++;
    for (int i = 0; i < nh; i++) {
      int id = hi[i];
      float mn = h0[i], mx = h1[i];
      int lv = level_of(&t, id);
      float nvs = vsb * (float)(dims[0] / dims[lv]);
      float rt = start_vs / nvs;
      float q = (mx - mn) * rt * (float)S / vl;
      {
        float et = 8.0f * ldexpf(fabsf(mx), -23);
        float rel = 2.0f * et / fmaxf(mx - mn, 1e-30f) + (float)nh * 8.0f * et / fmaxf(vl, 1e-30f);
        if (q >= 0.5f && q != roundf(q) && fabsf(q - roundf(q)) <= rel * fabsf(q) + 1e-6f * fabsf(q))
          flags[r] |= FLAG_TIE;
      }
      int n = (int)q;
      n = n >= 1 ? n : 1;
      want += n;
      float off = (mx - mn) / (float)(n + 1);
      for (int j = 0; j < n; j++) {
        if (has >= S) break;
        float rv = rd[has];
        float basez = fmaf(off, (float)(j + 1), mn);
        sz[has] = (float)((double)basez - (double)off / 2.0 + (double)(off * rv));
        si[has] = id;
        has++;
      }
    }
    if (want > S) flags[r] |= FLAG_TRUNC;
    /* fill step (:1017-1066) */
    float min_mid = 99999.0f, min_vs = 99999.0f, z0s = -1.0f, z1s = -1.0f;
    int best = -1;
    for (int i = 0; i < nh; i++) {
      int id = hi[i];
      int lv = level_of(&t, id);
      float nvs = vsb * (float)(dims[0] / dims[lv]);
      if (nvs <= min_vs) {
        float a = h0[i], c = h1[i];
        float mid = (float)((double)(a + c) / 2.0);
        if (nvs == min_vs) {
          if (near_eq(mid, min_mid)) flags[r] |= FLAG_TIE;
          if (mid < min_mid) { min_mid = mid; z0s = a; z1s = c; best = id; }
        } else {
          min_mid = mid; z0s = a; z1s = c; best = id;
        }
        min_vs = nvs;
      }
    }
    if (best < 0) continue;
    int nn = S - has;
    if (nn <= 0) continue;
    float off = (z1s - z0s) / (float)(nn + 1);
    for (int j = 0, q = has; q < S; q++, j++) {
      float basez = fmaf(off, (float)(j + 1), z0s);
      float rv = rd[q];
      sz[q] = (float)((double)basez - (double)off / 2.0 + (double)(off * rv));
      si[q] = best;
    }
  }
}
