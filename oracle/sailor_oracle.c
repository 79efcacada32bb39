/*
 * sailor_oracle.c -- CPU restatement of SAILOR's VoxelEncoding hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests, the smoke check
 * and the CPU-baseline leg of the benchmark call it; the product (the CUDA
 * library under sailor_gb300/) never links or calls it.
 *
 * Every function restates one reference routine and cites it by file:line
 * (paths relative to the SAILOR project root).  Float arithmetic follows the
 * reference's float32 operation order.  Where nvcc contracts a multiply-add
 * into one fused multiply-add (its default -fmad=true), the contraction is
 * written out with fmaf() so that integer-deciding steps (pixel rounding,
 * slab tests, sample counts) are reproduced bit for bit; the file is built
 * with -ffp-contract=off so the C compiler adds no contraction of its own.
 *
 * Two reference steps cannot be reproduced bit for bit on a CPU:
 *   - __fdividef(1, d) in the ray/box slab test (a hardware approximate
 *     reciprocal): the oracle uses the correctly rounded 1/d and flags every
 *     ray whose decisions lie within a relative margin of a tie;
 *   - __expf in density compositing: the oracle uses exp() in double and
 *     flags rays whose transmittance comes within a margin of the threshold.
 * Accumulations that carry no integer decision run in double.
 *
 * Node ids: the reference assigns tree-node ids through atomicAdd queues
 * (octree_kernel.cu:171,206), so its ids are run-to-run nondeterministic.
 * The oracle assigns them in the order a sequential execution of the same
 * loop produces (bricks in ascending linear order, children in ascending
 * lexicographic order), which is the order the CUDA library also uses.
 * Comparisons with reference output go through canonical (level,b,x,y,z)
 * keys.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define TIE_REL 1e-5

/* flags written per ray */
#define FLAG_TIE 1      /* a decision lies within TIE_REL of flipping        */
#define FLAG_ALIAS 2    /* ray visits an occupied top brick that is not a node */
#define FLAG_OVERFLOW 4 /* more hits than the output row holds                 */

/* Near ties of finite values only: an infinite slab distance (a direction */
/* component of 0) is infinite on the GPU as well, so it decides the same.  */
static inline int near_eq(double a, double b) {
  if (!isfinite(a) || !isfinite(b)) return 0;
  double m = fabs(a) > fabs(b) ? fabs(a) : fabs(b);
  return fabs(a - b) <= TIE_REL * m + 1e-30;
}

/* A near tie between two DDA crossing times (the axis-parallel sentinel */
/* 9999999 excepted).                                                     */
static inline int dda_tie(float a, float b) {
  if (a == 9999999.0f && b == 9999999.0f) return 0;
  return near_eq(a, b);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* 3x3 inverse by adjugate / determinant: fusion_kernel.cu:105-135.           */
/* ------------------------------------------------------------------------ */
static inline float msub(float p, float q, float r, float s) {
  /* p*q - r*s  as nvcc contracts it: fma(p, q, -(r*s)) */
  return fmaf(p, q, -(r * s));
}

void orc_inverse3x3(const float *M, int n, float *inv) {
  for (int i = 0; i < n; i++) {
    const float *m = M + 9 * i;
    float *o = inv + 9 * i;
    float a1 = m[0], b1 = m[1], c1 = m[2];
    float a2 = m[3], b2 = m[4], c2 = m[5];
    float a3 = m[6], b3 = m[7], c3 = m[8];
    float X = msub(b2, c3, c2, b3);
    float Y = msub(b1, c3, c1, b3);
    float Z = msub(b1, c2, c1, b2);
    float det = fmaf(a3, Z, fmaf(a1, X, -(a2 * Y)));
    o[0] = X / det;
    o[1] = msub(b3, c1, c3, b1) / det;
    o[2] = Z / det;
    o[3] = msub(a3, c2, c3, a2) / det;
    o[4] = msub(a1, c3, c1, a3) / det;
    o[5] = msub(a2, c1, c2, a1) / det;
    o[6] = msub(a2, b3, b2, a3) / det;
    o[7] = msub(b1, a3, a1, b3) / det;
    o[8] = msub(b2, a1, a2, b1) / det;
  }
}

/* ------------------------------------------------------------------------ */
/* Ray generation: rays_calculating (sampling_kernel.cu:674-731) and           */
/* rays_calculating_kernel (:411-486).  K^-1 and R^-1 by inverse_mat3x3        */
/* (:18-48, the same arithmetic as orc_inverse3x3); per pixel (h, w):          */
/* ori = -R^-1 T, dir = R^-1 K^-1 [w, h, 1] / (|.| + 1e-10).  nvcc contracts   */
/* the sums as written below; the normalising division is in double (the       */
/* literal 1e-10 is a double) and rounded to float, as the reference computes. */
/* out [B, N, H, W, 6].                                                        */
/* ------------------------------------------------------------------------ */
void orc_rays(const float *K, const float *R, const float *T, int B, int N, int H, int W, float *out) {
  for (int bv = 0; bv < B * N; bv++) {
    float ki[9], ri[9], c[3];
    orc_inverse3x3(K + 9 * bv, 1, ki);
    orc_inverse3x3(R + 9 * bv, 1, ri);
    const float *t = T + 3 * bv;
    for (int k = 0; k < 3; k++)
      c[k] = fmaf(-ri[3 * k + 2], t[2], fmaf(-ri[3 * k + 1], t[1], -(ri[3 * k] * t[0])));
#pragma omp parallel for schedule(static)
    for (int h = 0; h < H; h++)
      for (int w = 0; w < W; w++) {
        float cd[3], wd[3];
        for (int k = 0; k < 3; k++) cd[k] = fmaf((float)w, ki[3 * k], (float)h * ki[3 * k + 1]) + ki[3 * k + 2];
        for (int k = 0; k < 3; k++)
          wd[k] = fmaf(cd[2], ri[3 * k + 2], fmaf(cd[0], ri[3 * k], cd[1] * ri[3 * k + 1]));
        const float nd = sqrtf(fmaf(wd[2], wd[2], fmaf(wd[0], wd[0], wd[1] * wd[1])));
        float *o = out + (((size_t)bv * H + h) * W + w) * 6;
        for (int k = 0; k < 3; k++) {
          o[k] = c[k];
          o[3 + k] = (float)((double)wd[k] / ((double)nd + 1e-10));
        }
      }
  }
}

/* ------------------------------------------------------------------------ */
/* Data-driven bounding box: obtain_origin_bbox fusion_kernel.cu:137-184.     */
/* vol_origin [B,3,2] must hold 99999 / -99999 on entry (reference host code  */
/* fusion_kernel.cu:655-662).                                                */
/* ------------------------------------------------------------------------ */
void orc_origin_bbox(const float *depth, const float *Kinv, const float *Rinv,
                     const float *T, int B, int N, int H, int W, float thres,
                     float *vol_origin) {
  for (int b = 0; b < B; b++) {
    float mn[3] = {vol_origin[b * 6 + 0], vol_origin[b * 6 + 2], vol_origin[b * 6 + 4]};
    float mx[3] = {vol_origin[b * 6 + 1], vol_origin[b * 6 + 3], vol_origin[b * 6 + 5]};
    for (int v = 0; v < N; v++) {
      const float *ki = Kinv + (size_t)(b * N + v) * 9;
      const float *ri = Rinv + (size_t)(b * N + v) * 9;
      const float *t = T + (size_t)(b * N + v) * 3;
      const float *dm = depth + (size_t)(b * N + v) * H * W;
      for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
          float d = dm[(size_t)y * W + x];
          if (d < 0.1f || d > 5.0f) continue;
          float px = (float)x, py = (float)y;
          float cx = (fmaf(ki[0], px, ki[1] * py) + ki[2]) * d;
          float cy = (fmaf(ki[3], px, ki[4] * py) + ki[5]) * d;
          float cz = (fmaf(ki[6], px, ki[7] * py) + ki[8]) * d;
          cx -= t[0];
          cy -= t[1];
          cz -= t[2];
          float p[3];
          p[0] = fmaf(ri[2], cz, fmaf(ri[0], cx, ri[1] * cy));
          p[1] = fmaf(ri[5], cz, fmaf(ri[3], cx, ri[4] * cy));
          p[2] = fmaf(ri[8], cz, fmaf(ri[6], cx, ri[7] * cy));
          for (int a = 0; a < 3; a++) {
            float lo = p[a] - thres, hi = p[a] + thres;
            if (lo < mn[a]) mn[a] = lo;
            if (hi > mx[a]) mx[a] = hi;
          }
        }
    }
    for (int a = 0; a < 3; a++) {
      vol_origin[b * 6 + 2 * a] = mn[a];
      vol_origin[b * 6 + 2 * a + 1] = mx[a];
    }
  }
}

/* Cubic box about the centre: obtain_resized_bbox fusion_kernel.cu:51-103. */
void orc_resized_bbox(const float *vol_origin, int B, int D, float *vol_bbox,
                      float *voxel_size) {
  for (int i = 0; i < B; i++) {
    const float *o = vol_origin + 6 * i;
    float x_min = o[0], x_max = o[1], y_min = o[2], y_max = o[3], z_min = o[4],
          z_max = o[5];
    float x_len = x_max - x_min, y_len = y_max - y_min, z_len = z_max - z_min;
    float max_len = fmaxf(x_len, fmaxf(y_len, z_len));
    float xc = (x_min + x_max) / 2.0f, yc = (y_min + y_max) / 2.0f,
          zc = (z_min + z_max) / 2.0f;
    voxel_size[i] = max_len / (float)(D - 1);
    float h = max_len / 2.0f;
    if (max_len == x_len) {
      y_min = yc - h; y_max = yc + h; z_min = zc - h; z_max = zc + h;
    } else if (max_len == y_len) {
      x_min = xc - h; x_max = xc + h; z_min = zc - h; z_max = zc + h;
    } else {
      x_min = xc - h; x_max = xc + h; y_min = yc - h; y_max = yc + h;
    }
    float *bb = vol_bbox + 6 * i;
    bb[0] = x_min; bb[1] = x_max; bb[2] = y_min; bb[3] = y_max; bb[4] = z_min;
    bb[5] = z_max;
  }
}

/* ------------------------------------------------------------------------ */
/* TSDF fusion: integrate_cuda fusion_kernel.cu:236-340.                      */
/* Voxel order x-major, z fastest (:265-268).  tsdf/weight/colour start at    */
/* 1/0/0 (:668-670).  Returns the number of pixel-rounding near-ties seen.    */
/* ------------------------------------------------------------------------ */
/* x-slab [x_begin, x_end) of the grid (the whole grid: 0, D); used to time
 * a bounded sample of the fusion on the host */
long orc_integrate_slab(int B, int N, int H, int W, int D, int x_begin, int x_end,
                        const float *vol_bbox, const float *voxel_size,
                        const float *K, const float *RT, const float *color_im,
                        const float *depth_im, float obs_weight,
                        float trunc_weight, float th_low, float th_high,
                        float *tsdf, float *weight, float *colorv, int *occ,
                        int *count) {
  long ties = 0;
  size_t vol = (size_t)D * D * D;
  for (int b = 0; b < B; b++) {
    long cnt = 0;
    float vs = voxel_size[b];
    float trunc = vs * trunc_weight;
    float bx = vol_bbox[b * 6 + 0], by = vol_bbox[b * 6 + 2], bz = vol_bbox[b * 6 + 4];
    long v_begin = (long)x_begin * D * D, v_end = (long)x_end * D * D;
#pragma omp parallel for reduction(+ : cnt, ties) schedule(static)
    for (long v = v_begin; v < v_end; v++) {
      int x = (int)(v / ((long)D * D));
      int y = (int)((v - (long)x * D * D) / D);
      int z = (int)(v - (long)x * D * D - (long)y * D);
      float px = fmaf((float)x, vs, bx);
      float py = fmaf((float)y, vs, by);
      float pz = fmaf((float)z, vs, bz);
      float ts = 1.0f, w = 0.0f, col = 0.0f;
      for (int k = 0; k < N; k++) {
        const float *P = RT + (size_t)(b * N + k) * 12;
        const float *Kk = K + (size_t)(b * N + k) * 9;
        float cx = fmaf(P[2], pz, fmaf(P[0], px, P[1] * py)) + P[3];
        float cy = fmaf(P[6], pz, fmaf(P[4], px, P[5] * py)) + P[7];
        float cz = fmaf(P[10], pz, fmaf(P[8], px, P[9] * py)) + P[11];
        float ux = fmaf(Kk[2], cz, fmaf(Kk[0], cx, Kk[1] * cy));
        float uy = fmaf(Kk[5], cz, fmaf(Kk[3], cx, Kk[4] * cy));
        float uz = fmaf(Kk[8], cz, fmaf(Kk[6], cx, Kk[7] * cy));
        ux = ux / uz;
        uy = uy / uz;
        {
          float fx = ux - floorf(ux), fy = uy - floorf(uy);
          if (fabsf(fx - 0.5f) < 1e-4f || fabsf(fy - 0.5f) < 1e-4f) ties++;
        }
        int pix_x = (int)roundf(ux), pix_y = (int)roundf(uy);
        if (pix_x < 0 || pix_x >= W || pix_y < 0 || pix_y >= H || cz < 0) continue;
        size_t pidx = (size_t)(b * N + k) * H * W + (size_t)pix_y * W + pix_x;
        float dv = depth_im[pidx];
        if (dv < 0.1f || dv > 4.0f) continue;
        float diff = dv - cz;
        if (diff < -trunc) continue;
        float dist = fminf(1.0f, diff / trunc);
        float w_old = w, w_new = w_old + obs_weight;
        w = w_new;
        /* nvcc fuses the second product here: fma(obs, dist, ts*w_old) */
        ts = fmaf(obs_weight, dist, ts * w_old) / w_new;
        float old_b = floorf(col / 65536.0f);
        float old_g = floorf((col - old_b * 256.0f * 256.0f) / 256.0f);
        float old_r = col - old_b * 256.0f * 256.0f - old_g * 256.0f;
        float nc = color_im[pidx];
        float nb = floorf(nc / 65536.0f);
        float ng = floorf((nc - nb * 256.0f * 256.0f) / 256.0f);
        float nr = nc - nb * 256.0f * 256.0f - ng * 256.0f;
        nb = fminf(roundf(fmaf(old_b, w_old, obs_weight * nb) / w_new), 255.0f);
        ng = fminf(roundf(fmaf(old_g, w_old, obs_weight * ng) / w_new), 255.0f);
        nr = fminf(roundf(fmaf(old_r, w_old, obs_weight * nr) / w_new), 255.0f);
        col = nb * 256.0f * 256.0f + ng * 256.0f + nr;
      }
      size_t o = (size_t)b * vol + v;
      tsdf[o] = ts;
      weight[o] = w;
      colorv[o] = col;
      if (ts < trunc * th_high && ts > -trunc * th_low) {
        occ[o] = (int)v;
        cnt++;
      } else {
        occ[o] = -1;
      }
    }
    count[b] = (int)cnt;
  }
  return ties;
}

long orc_integrate(int B, int N, int H, int W, int D, const float *vol_bbox,
                   const float *voxel_size, const float *K, const float *RT,
                   const float *color_im, const float *depth_im,
                   float obs_weight, float trunc_weight, float th_low,
                   float th_high, float *tsdf, float *weight, float *colorv,
                   int *occ, int *count) {
  return orc_integrate_slab(B, N, H, W, D, 0, D, vol_bbox, voxel_size, K, RT,
                            color_im, depth_im, obs_weight, trunc_weight, th_low,
                            th_high, tsdf, weight, colorv, occ, count);
}

/* ------------------------------------------------------------------------ */
/* Coarse occupancy: merge_non_empty_nodes octree_kernel.cu:242-303.          */
/* A coarse voxel is occupied iff any of its rate^3 fine children is > -1.    */
/* ------------------------------------------------------------------------ */
void orc_merge(int B, int Dc, int rate, const int *fine, int *coarse,
               int *count) {
  int Df = Dc * rate;
  size_t vc = (size_t)Dc * Dc * Dc, vf = (size_t)Df * Df * Df;
  for (int b = 0; b < B; b++) {
    long cnt = 0;
#pragma omp parallel for reduction(+ : cnt) schedule(static)
    for (long i = 0; i < (long)vc; i++) {
      int X = (int)(i / ((long)Dc * Dc)), Y = (int)((i / Dc) % Dc), Z = (int)(i % Dc);
      int any = 0;
      for (int a = 0; a < rate && !any; a++)
        for (int c = 0; c < rate && !any; c++)
          for (int e = 0; e < rate; e++) {
            size_t f = (size_t)b * vf + ((size_t)(X * rate + a) * Df + (Y * rate + c)) * Df + (Z * rate + e);
            if (fine[f] > -1) { any = 1; break; }
          }
      coarse[(size_t)b * vc + i] = any ? (int)i : -1;
      cnt += any;
    }
    count[b] = (int)cnt;
  }
}

/* ------------------------------------------------------------------------ */
/* Node geometry: OcTree::calculate_bbox_start / calculate_xyz_corners,       */
/* octree.h:109-151, as initialised by gen_root_octree_nodes                  */
/* octree_kernel.cu:157-217.                                                  */
/* level 1 = top brick (size = Dbot/Dtop), level 0 = fine voxel (size 1).     */
/* ------------------------------------------------------------------------ */
void orc_node_geometry(float vs_bottom, int size, const float *bbox_min3,
                       const int *idx3, float *centre3, float *node_vs) {
  float nvs = vs_bottom * (float)size; /* voxel_size * (Dbot / Dlevel) */
  float basic = nvs / (float)size;
  int rate_vol = (int)log2f((float)size);
  float off = 0.0f;
  for (int i = 0; i < rate_vol; i++) off = off + ldexpf(1.0f, i) * basic / 2.0f;
  for (int a = 0; a < 3; a++) {
    float bs = bbox_min3[a] + off;
    centre3[a] = fmaf(nvs, (float)idx3[a], bs);
  }
  *node_vs = nvs;
}

/* ------------------------------------------------------------------------ */
/* Two-level tree build: gen_root_octree_nodes octree_kernel.cu:126-239 with  */
/* if_single_occ_in_neighbors :101-122.  Only two levels (the shipped         */
/* configuration, RenTestOptions octree_level=2) are restated.                */
/*   occ_top [B,Dt^3], occ_bot [B,Db^3] are rewritten in place to node ids.   */
/*   Outputs, sized by the caller: top_key[cap_top] (b*Dt^3 + brick),         */
/*   top_child_base[cap_top], top_nchild[cap_top], bot_key[cap_bot]           */
/*   (b*Db^3 + voxel), bot_parent[cap_bot] (parent node id), q[2]={#top,#bot}. */
/* Returns 0, or -1 when a capacity would be exceeded.                        */
/* ------------------------------------------------------------------------ */
int orc_build_tree(int B, int Dt, int Db, int *occ_top, int *occ_bot,
                   int base_top, int base_bot, int cap_top, int cap_bot,
                   int *top_key, int *top_child_base, int *top_nchild,
                   int *bot_key, int *bot_parent, int *q) {
  int rate = Db / Dt;
  size_t vt = (size_t)Dt * Dt * Dt, vb = (size_t)Db * Db * Db;
  int nt = 0, nb = 0;
  /* decide kept bricks first (all neighbour reads see pre-build values:    */
  /* rewritten entries stay > -1, so the reference's in-place race does not */
  /* change any decision)                                                   */
  unsigned char *keep = (unsigned char *)calloc((size_t)B * vt, 1);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)(B * vt); i++) {
    if (occ_top[i] <= -1) continue;
    int b = (int)(i / vt);
    long l = i - (long)b * vt;
    int x = (int)(l / ((long)Dt * Dt)), y = (int)((l / Dt) % Dt), z = (int)(l % Dt);
    int found = 0;
    for (int k = x - 1; k < x + 2 && !found; k++)
      for (int m = y - 1; m < y + 2 && !found; m++)
        for (int n = z - 1; n < z + 2; n++) {
          if (k >= 0 && k < Dt && m >= 0 && m < Dt && n >= 0 && n < Dt && !(k == x && m == y && n == z)) {
            if (occ_top[(size_t)b * vt + ((size_t)k * Dt + m) * Dt + n] > -1) { found = 1; break; }
          }
        }
    keep[i] = (unsigned char)found;
  }
  for (long i = 0; i < (long)(B * vt); i++) {
    if (!keep[i]) continue;
    int b = (int)(i / vt);
    long l = i - (long)b * vt;
    int X = (int)(l / ((long)Dt * Dt)), Y = (int)((l / Dt) % Dt), Z = (int)(l % Dt);
    if (nt >= cap_top) { free(keep); return -1; }
    int k = nt++;
    top_key[k] = (int)i;
    top_child_base[k] = nb;
    int nc = 0;
    for (int a = 0; a < rate; a++)
      for (int c = 0; c < rate; c++)
        for (int e = 0; e < rate; e++) {
          size_t f = (size_t)b * vb + ((size_t)(X * rate + a) * Db + (Y * rate + c)) * Db + (Z * rate + e);
          if (occ_bot[f] > -1) {
            if (nb >= cap_bot) { free(keep); return -1; }
            bot_key[nb] = (int)f;
            bot_parent[nb] = base_top + k;
            occ_bot[f] = base_bot + nb;
            nb++;
            nc++;
          }
        }
    top_nchild[k] = nc;
    occ_top[i] = base_top + k;
  }
  q[0] = nt;
  q[1] = nb;
  free(keep);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Ray / axis-aligned cube slab test: RayVoxelIntersection                   */
/* intersection_kernel.cu:36-71.  Returns 1 on hit with t0,t1.  *tie is set   */
/* when any comparison lies within TIE_REL (the GPU uses __fdividef).         */
/* ------------------------------------------------------------------------ */
static int slab(const float o[3], const float inv[3], const float c[3], float vs,
                float *t0, float *t1, int *tie) {
  float f_low = 0.0f, f_high = 100000.0f;
  float h = vs / 2.0f;
  for (int i = 0; i < 3; i++) {
    float lo = (c[i] - h - o[i]) * inv[i];
    float hi = (c[i] + h - o[i]) * inv[i];
    if (lo > hi) { float t = lo; lo = hi; hi = t; }
    if (near_eq(hi, f_low) || near_eq(lo, f_high)) *tie = 1;
    if (hi < f_low) return 0;
    if (lo > f_high) return 0;
    f_low = (lo > f_low) ? lo : f_low;
    f_high = (hi < f_high) ? hi : f_high;
    if (near_eq(f_low, f_high)) *tie = 1;
    if (f_low > f_high) return 0;
  }
  *t0 = f_low;
  *t1 = f_high;
  return 1;
}

/* One node table for the traversal/sampling restatements. */
typedef struct {
  int B, Dt, Db, rate, base_top, base_bot, ntop, nbot;
  const int *top_key, *top_child_base, *top_nchild, *bot_key;
  const float *voxel_size, *vol_bbox;
} tree_t;

static void node_centre(const tree_t *t, int gid, float c[3], float *nvs) {
  int idx[3], b;
  int size;
  if (gid >= t->base_top) {
    int k = gid - t->base_top;
    long key = t->top_key[k];
    size_t vt = (size_t)t->Dt * t->Dt * t->Dt;
    b = (int)(key / vt);
    long l = key - (long)b * vt;
    idx[0] = (int)(l / ((long)t->Dt * t->Dt));
    idx[1] = (int)((l / t->Dt) % t->Dt);
    idx[2] = (int)(l % t->Dt);
    size = t->Db / t->Dt;
  } else {
    long key = t->bot_key[gid - t->base_bot];
    size_t vb = (size_t)t->Db * t->Db * t->Db;
    b = (int)(key / vb);
    long l = key - (long)b * vb;
    idx[0] = (int)(l / ((long)t->Db * t->Db));
    idx[1] = (int)((l / t->Db) % t->Db);
    idx[2] = (int)(l % t->Db);
    size = 1;
  }
  float bmin[3] = {t->vol_bbox[b * 6 + 0], t->vol_bbox[b * 6 + 2], t->vol_bbox[b * 6 + 4]};
  orc_node_geometry(t->voxel_size[b], size, bmin, idx, c, nvs);
}

/* ------------------------------------------------------------------------ */
/* Voxel traversal: MultiLayerOctree::voxel_traversal intersection_kernel.cu: */
/* 828-895 -> ray_voxel_traversal :286-439 -> RayVoxelIntersectionNodeListNew */
/* :128-284.  occ_top holds node ids after the build (kept bricks), the brick */
/* local id (occupied, not kept) or -1.  Bricks that are occupied but not a   */
/* node are treated as empty and the ray is flagged FLAG_ALIAS: the reference */
/* reads an unrelated node there (its local id used as a node id).            */
/* Outputs: idx/t0/t1 [B,N,W] prefilled -1 by the caller, valid_len [B,N]      */
/* prefilled 0, nhit [B,N], flags [B,N].  Returns the max hit count.          */
/* ------------------------------------------------------------------------ */
int orc_voxel_traversal(int B, int N, const float *ori, const float *dir,
                        int Dt, int Db, const int *occ_top, int base_top,
                        int base_bot, int ntop, int nbot, const int *top_key,
                        const int *top_child_base, const int *top_nchild,
                        const int *bot_key, const float *voxel_size,
                        const float *vol_bbox, int W, int th_early_stop,
                        int opt_num, int is_training, int *out_idx,
                        float *out_t0, float *out_t1, float *valid_len,
                        int *nhit, int *flags) {
  tree_t t = {B, Dt, Db, Db / Dt, base_top, base_bot, ntop, nbot, top_key,
              top_child_base, top_nchild, bot_key, voxel_size, vol_bbox};
  int maxhits = 0;
  size_t vt = (size_t)Dt * Dt * Dt;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : maxhits)
  for (long r = 0; r < (long)B * N; r++) {
    int b = (int)(r / N);
    int fl = 0, cnt = 0;
    float vlen = 0.0f;
    const float *bb = vol_bbox + b * 6;
    float xc = (bb[0] + bb[1]) / 2.0f, yc = (bb[2] + bb[3]) / 2.0f, zc = (bb[4] + bb[5]) / 2.0f;
    float vs = voxel_size[b];
    float vs_top = vs * (float)(Db / Dt);
    float bst[3] = {bb[0] - vs / 2.0f, bb[2] - vs / 2.0f, bb[4] - vs / 2.0f};
    float o[3] = {ori[r * 3 + 0], ori[r * 3 + 1], ori[r * 3 + 2]};
    float d[3] = {dir[r * 3 + 0], dir[r * 3 + 1], dir[r * 3 + 2]};
    float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    float cen[3] = {xc, yc, zc};
    float T0, T1;
    int tie = 0;
    int *oi = out_idx + (size_t)r * W;
    float *o0 = out_t0 + (size_t)r * W, *o1 = out_t1 + (size_t)r * W;
    if (!slab(o, inv, cen, vs_top * (float)Dt, &T0, &T1, &tie) || T0 < 0.0f || T1 < 0.0f) {
      nhit[r] = 0;
      flags[r] = tie ? FLAG_TIE : 0;
      continue;
    }
    float sp[3], so[3];
    int st[3];
    for (int a = 0; a < 3; a++) {
      sp[a] = fmaf(T0, d[a], o[a]);
      so[a] = sp[a] - bst[a];
      float q = so[a] / vs_top;
      /* a start cell decided by truncation next to an interior cell face; */
      /* faces 0 and Dt are harmless (truncation toward zero, clamping)    */
      if (fabsf(q - roundf(q)) < 1e-4f && roundf(q) >= 1.0f && roundf(q) <= (float)(Dt - 1)) tie = 1;
      int s = (int)q;
      s = s < 0 ? 0 : s;
      st[a] = s < Dt ? s : Dt - 1;
    }
    float step[3], tm[3], td[3];
    for (int a = 0; a < 3; a++) {
      step[a] = (d[a] >= 0) ? 1.0f : -1.0f;
      float nb = (step[a] > 0) ? ((float)st[a] + step[a]) * vs_top : (float)st[a] * vs_top;
      tm[a] = (d[a] != 0) ? (nb - so[a]) / d[a] : 9999999.0f;
      td[a] = (d[a] != 0) ? vs_top / d[a] * step[a] : 9999999.0f;
    }
    int J = 4 * Dt;
    int pre_empty = 0, has_valid = 0, nsucc = 0, nint = 0;
    for (int j = 0; j < J; j++) {
      int rid = -1;
      size_t cell = (size_t)b * vt + ((size_t)st[0] * Dt + st[1]) * Dt + st[2];
      int nid = occ_top[cell];
      if (nid > -1) {
        if (nid < base_top || nid >= base_top + ntop) {
          fl |= FLAG_ALIAS;
        } else {
          float c[3], nvs;
          node_centre(&t, nid, c, &nvs);
          float p0, p1;
          if (slab(o, inv, c, nvs, &p0, &p1, &tie) && !(p0 < 0.0f || p1 < 0.0f)) {
            int k = nid - base_top;
            if (!is_training) {
              int cb = top_child_base[k], nc = top_nchild[k];
              for (int ci = 0; ci < nc; ci++) {
                int cg = base_bot + cb + ci;
                float cc[3], cvs, c0, c1;
                node_centre(&t, cg, cc, &cvs);
                if (!slab(o, inv, cc, cvs, &c0, &c1, &tie) || c0 < 0.0f || c1 < 0.0f) continue;
                if (cnt < W) { oi[cnt] = cg; o0[cnt] = c0; o1[cnt] = c1; } else fl |= FLAG_OVERFLOW;
                vlen = vlen + (c1 - c0) * 4.0f;
                cnt++;
              }
            }
            if (cnt < W) { oi[cnt] = nid; o0[cnt] = p0; o1[cnt] = p1; } else fl |= FLAG_OVERFLOW;
            vlen = vlen + (p1 - p0);
            cnt++;
            rid = cnt - 1;
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
      int ax;
      /* exact equality counts too: the GPU reaches tm from a start point   */
      /* computed with its approximate reciprocal, so two crossings that    */
      /* coincide here can come out an ulp apart there and step the other  */
      /* axis first; only the 9999999 of a zero direction component is the  */
      /* same constant on both                                              */
      if (dda_tie(tm[0], tm[1]) || dda_tie(tm[0], tm[2]) || dda_tie(tm[1], tm[2])) tie = 1;
      if (tm[0] < tm[1]) ax = (tm[0] < tm[2]) ? 0 : 2;
      else ax = (tm[1] < tm[2]) ? 1 : 2;
      st[ax] += (int)step[ax];
      tm[ax] += td[ax];
      if (st[0] < 0 || st[0] >= Dt || st[1] < 0 || st[1] >= Dt || st[2] < 0 || st[2] >= Dt) break;
    }
    valid_len[r] = vlen;
    nhit[r] = cnt;
    if (tie) fl |= FLAG_TIE;
    flags[r] = fl;
    if (cnt > maxhits) maxhits = cnt;
  }
  return maxhits;
}

/* ------------------------------------------------------------------------ */
/* Adaptive sampling over hit intervals: ray_voxels_sampling_uniform_kernel   */
/* sampling_kernel.cu:1070-1177 (host :1251-1304).  Padded hit lists of width */
/* W.  Outputs sampled_idx/sampled_z [B,N,S] prefilled -1 by the caller.      */
/* flags[r] gains FLAG_TIE when a sample count lies within 1e-4 (relative) of */
/* an integer boundary.  The sampling sample position uses double arithmetic  */
/* exactly as the reference does (:1148,:1169 mix float with 2.0).            */
/* ------------------------------------------------------------------------ */
void orc_sample_coarse(int B, int N, int W, int S, const int *hit_idx,
                       const float *hit_t0, const float *hit_t1,
                       const float *rands, const float *valid_len,
                       int max_hits, int num_levels, int start_level,
                       int Dt, int Db, int base_top, const float *voxel_size,
                       int *sampled_idx, float *sampled_z, int *flags) {
#pragma omp parallel for schedule(dynamic, 64)
  for (long r = 0; r < (long)B * N; r++) {
    int b = (int)(r / N);
    const int *hi = hit_idx + (size_t)r * W;
    const float *h0 = hit_t0 + (size_t)r * W, *h1 = hit_t1 + (size_t)r * W;
    const float *rd = rands + (size_t)r * S;
    int *si = sampled_idx + (size_t)r * S;
    float *sz = sampled_z + (size_t)r * S;
    if (hi[0] < 0) continue;
    float vl = valid_len[r];
    float start_vs = voxel_size[b] * powf(4.0f, (float)(num_levels - start_level - 1));
    int has = 0;
    int lim = max_hits < W ? max_hits : W;
    for (int i = 0; i < lim; i++) {
      int id = hi[i];
      float mn = h0[i], mx = h1[i];
      if (id < 0 || mn < 0 || mx < 0) break;
      float nvs = (id >= base_top) ? voxel_size[b] * (float)(Db / Dt) : voxel_size[b];
      float rate = start_vs / nvs;
      float q = (mx - mn) * rate * (float)S / vl;
      /* q near an integer boundary of the (int) cast, within the error that */
      /* a few-ulp difference in t0/t1 (the GPU's approximate reciprocal)   */
      /* induces: |dq|/q <= 2*et/len + nh*2*et*4/vl, et = 8 ulp of t1.       */
      /* Exact integers come from exact cancellation (one hit: q == S) and  */
      /* are reproduced by any implementation with the same operation order */
      {
        float et = 8.0f * ldexpf(fabsf(mx), -23);
        float rel = 2.0f * et / fmaxf(mx - mn, 1e-30f) + (float)(i + 1) * 8.0f * et / fmaxf(vl, 1e-30f);
        if (q >= 0.5f && q != roundf(q) && fabsf(q - roundf(q)) <= rel * fabsf(q) + 1e-6f * fabsf(q))
          flags[r] |= FLAG_TIE;
      }
      int n = (int)q;
      n = n >= 1 ? n : 1;
      int left = S - has;
      if (left < n) n = left;
      float off = (mx - mn) / (float)(n + 1);
      for (int j = 0; j < n; j++) {
        if (has >= S) break;
        float rv = rd[has];
        float base = fmaf(off, (float)(j + 1), mn);
        float z = (float)((double)base - (double)off / 2.0 + (double)(off * rv));
        sz[has] = z;
        si[has] = id;
        ++has;
      }
    }
    int left = S - has;
    if (left > max_hits) left = max_hits;
    for (int i = 0; i < left; i++) {
      if (has >= S) break;
      if (i >= W) break;
      int id = hi[i];
      float mn = h0[i], mx = h1[i];
      if (id < 0 || mn < 0 || mx < 0) break;
      float off = (float)((double)(mx - mn) / 2.0);
      float rv = rd[has];
      float base = mn + off;
      float z = (float)((double)base - (double)off / 2.0 + (double)(off * rv));
      sz[has] = z;
      si[has] = id;
      ++has;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Per-ray ascending sort of sample depths: sort_samplings                    */
/* sampling_kernel.cu:1308-1329 (torch::sort along dim 2).  The order of      */
/* equal keys is taken stable (ascending original index).                     */
/* ------------------------------------------------------------------------ */
void orc_sort(int R, int S, const float *z, float *sorted, int *idx) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    const float *zr = z + (size_t)r * S;
    int *ir = idx + (size_t)r * S;
    float *sr = sorted + (size_t)r * S;
    for (int i = 0; i < S; i++) ir[i] = i;
    /* insertion sort: stable */
    for (int i = 1; i < S; i++) {
      int v = ir[i];
      float key = zr[v];
      int j = i - 1;
      while (j >= 0 && zr[ir[j]] > key) { ir[j + 1] = ir[j]; j--; }
      ir[j + 1] = v;
    }
    for (int i = 0; i < S; i++) sr[i] = zr[ir[i]];
  }
}

/* ------------------------------------------------------------------------ */
/* Compositing forward: volume_rendering_training_forward_kernel              */
/* volume_rendering.cu:17-126 (density, alpha = 1-exp(-sigma*delta)) and      */
/* volume_rendering_occ_training_forward_kernel :129-240 (alpha = sigma).     */
/* sort_idx may be NULL (pre-sorted input: volume_rendering_occ_kernel        */
/* :666-745, which also tests only the last raw entry for an invalid ray).   */
/* C feature channels (the reference fixes C=3, FEATS_DIM :13).               */
/* ------------------------------------------------------------------------ */
void orc_composite_fwd(int R, int S, int C, const float *z, const int *sort_idx,
                       const float *sigma, const float *feats, float t_thres,
                       int occ_mode, double *out_feat, double *out_depth,
                       double *out_ws, double *out_alpha, int *flags) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    const float *zr = z + (size_t)r * S;
    const int *ir = sort_idx ? sort_idx + (size_t)r * S : NULL;
    const float *sg = sigma + (size_t)r * S;
    const float *fr = feats + (size_t)r * S * C;
    double *of = out_feat + (size_t)r * C;
    for (int c = 0; c < C; c++) of[c] = 0;
    out_depth[r] = out_ws[r] = out_alpha[r] = 0;
    if (flags) flags[r] = 0;
    int last = ir ? ir[S - 1] : S - 1;
    if (zr[last] < 0) continue;
    double T = 1.0, ws = 0, d = 0, al = 0;
    for (int i = 0; i < S; i++) {
      int s = ir ? ir[i] : i;
      float zs = zr[s];
      if (zs < 0) continue;
      double alpha;
      if (occ_mode) {
        alpha = sg[s];
      } else {
        float delta;
        if (i < S - 1) {
          float zn = 0;
          for (int m = i + 1; m < S; m++) {
            zn = zr[ir ? ir[m] : m];
            if (zn > 0) break;
          }
          delta = zn - zs;
        } else {
          delta = 1e10f;
        }
        alpha = 1.0 - exp(-(double)sg[s] * (double)delta);
      }
      double w = alpha * T;
      for (int c = 0; c < C; c++) of[c] += w * fr[(size_t)s * C + c];
      d += w * zs;
      ws += w;
      al += w * alpha;
      T *= 1.0 - alpha;
      if (flags && fabs(T - t_thres) <= 1e-4 * t_thres) flags[r] |= FLAG_TIE;
      if (T < t_thres) break;
    }
    out_depth[r] = d;
    out_ws[r] = ws;
    out_alpha[r] = al;
  }
}

/* ------------------------------------------------------------------------ */
/* Compositing backward as the reference computes it:                         */
/* volume_rendering_training_backward_kernel volume_rendering.cu:244-381 and  */
/* the occupancy variant :384-522.  Recomputes the forward from the saved     */
/* final outputs; the sample that triggers early termination gets no         */
/* gradient (:346 breaks before :350-377).  grad arrays zeroed by the caller. */
/* ------------------------------------------------------------------------ */
void orc_composite_bwd_ref(int R, int S, int C, const float *g_feat,
                           const float *g_depth, const float *g_ws,
                           const float *g_alpha, const float *o_feat,
                           const float *o_depth, const float *o_ws,
                           const float *o_alpha, const float *z,
                           const int *sort_idx, const float *sigma,
                           const float *feats, float t_thres, int occ_mode,
                           double *grad_feats, double *grad_sigma) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    const float *zr = z + (size_t)r * S;
    const int *ir = sort_idx + (size_t)r * S;
    const float *sg = sigma + (size_t)r * S;
    const float *fr = feats + (size_t)r * S * C;
    if (zr[ir[S - 1]] < 0) continue;
    double T = 1.0, ws = 0, al = 0, d = 0;
    double facc[64] = {0};
    double gws = g_ws[r], gd = g_depth[r], ga = g_alpha[r];
    double wsf = o_ws[r], df = o_depth[r], af = o_alpha[r];
    for (int i = 0; i < S; i++) {
      int s = ir[i];
      float zs = zr[s];
      if (zs < 0) continue;
      double alpha, delta = 0;
      if (occ_mode) {
        alpha = sg[s];
      } else {
        float dl;
        if (i < S - 1) {
          float zn = 0;
          for (int m = i + 1; m < S; m++) {
            zn = zr[ir[m]];
            if (zn > 0) break;
          }
          dl = zn - zs;
        } else {
          dl = 1e10f;
        }
        delta = dl;
        alpha = 1.0 - exp(-(double)sg[s] * delta);
      }
      double w = alpha * T;
      for (int c = 0; c < C; c++) facc[c] += w * fr[(size_t)s * C + c];
      d += w * zs;
      ws += w;
      al += w * alpha;
      T *= 1.0 - alpha;
      if (T < t_thres) break;
      for (int c = 0; c < C; c++) grad_feats[((size_t)r * S + s) * C + c] = g_feat[r * C + c] * w;
      double gs;
      if (occ_mode) {
        double tmp = (1.0 / (1.0 - alpha + 1e-7) <= 15.0) ? 1.0 / (1.0 - alpha) : 15.0;
        double a = gws * (T - (wsf - ws)) * tmp;
        double b2 = gd * (T * zs - (df - d)) * tmp;
        double c2 = ga * (2 * T * alpha - (af - al)) * tmp;
        double f = 0;
        for (int c = 0; c < C; c++) f += g_feat[r * C + c] * (T * fr[(size_t)s * C + c] - (o_feat[r * C + c] - facc[c]));
        f *= tmp;
        gs = a + b2 + f + c2;
      } else {
        double tmp = gws * (1 - wsf);
        double a = delta * (gws * (T - (wsf - ws)) + tmp);
        double b2 = delta * (gd * (T * zs - (df - d)) + tmp);
        double c2 = delta * (ga * (2 * T * alpha - (af - al)) + tmp);
        double f = 0;
        for (int c = 0; c < C; c++) f += g_feat[r * C + c] * (T * fr[(size_t)s * C + c] - (o_feat[r * C + c] - facc[c]));
        f = delta * (f + tmp);
        gs = a + b2 + f + c2;
      }
      grad_sigma[(size_t)r * S + s] = gs;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Node-corner trilinear aggregation: trilinear_aggregate_features_kernel     */
/* sampling_kernel.cu:162-234 and its backward :237-327.  corners[R*S][8][3]  */
/* are the eight corners of each sample's node in the order of                */
/* OcTree::calculate_xyz_corners (octree.h:120-129: x outer, z inner).        */
/* feats [C][R*S][8] -> out [C][R*S]; backward writes [C][R*S][8].           */
/* ------------------------------------------------------------------------ */
void orc_trilerp_nodes(long RS, int C, const float *pts, const float *corners,
                       const int *valid, const float *feats, const float *gout,
                       double *out, double *gin) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < RS; k++) {
    if (!valid[k]) continue;
    const float *cx = corners + (size_t)k * 24;
    double px = pts[k * 3], py = pts[k * 3 + 1], pz = pts[k * 3 + 2];
#define CX(i) cx[(i) * 3 + 0]
#define CY(i) cx[(i) * 3 + 1]
#define CZ(i) cx[(i) * 3 + 2]
    double tx04 = (px - CX(0)) / (CX(4) - CX(0));
    double tx15 = (px - CX(1)) / (CX(5) - CX(1));
    double tx26 = (px - CX(2)) / (CX(6) - CX(2));
    double tx37 = (px - CX(3)) / (CX(7) - CX(3));
    double ya = (CY(0) + CY(4)) / 2.0, yb = (CY(2) + CY(6)) / 2.0;
    double yc = (CY(1) + CY(5)) / 2.0, yd = (CY(3) + CY(7)) / 2.0;
    double ty0 = (py - ya) / (yb - ya), ty1 = (py - yc) / (yd - yc);
    double za = (CZ(0) + CZ(4) + CZ(2) + CZ(6)) / 4.0, zb = (CZ(1) + CZ(5) + CZ(3) + CZ(7)) / 4.0;
    double tz = (pz - za) / (zb - za);
#undef CX
#undef CY
#undef CZ
    double w[8];
    w[0] = (1 - tx04) * (1 - ty0) * (1 - tz);
    w[4] = tx04 * (1 - ty0) * (1 - tz);
    w[2] = (1 - tx26) * ty0 * (1 - tz);
    w[6] = tx26 * ty0 * (1 - tz);
    w[1] = (1 - tx15) * (1 - ty1) * tz;
    w[5] = tx15 * (1 - ty1) * tz;
    w[3] = (1 - tx37) * ty1 * tz;
    w[7] = tx37 * ty1 * tz;
    for (int c = 0; c < C; c++) {
      if (feats) {
        const float *f = feats + ((size_t)c * RS + k) * 8;
        double s = 0;
        for (int i = 0; i < 8; i++) s += w[i] * f[i];
        out[(size_t)c * RS + k] = s;
      }
      if (gout) {
        double g = gout[(size_t)c * RS + k];
        for (int i = 0; i < 8; i++) gin[((size_t)c * RS + k) * 8 + i] = g * w[i];
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Dense-grid trilinear gather and its adjoint (the spec extension of   */
/* trilinear_aggregate_features to a dense per-voxel grid).  The grid is      */
/* [B][D][D][D][C] with voxel (x,y,z) centred at bbox_min + (x,y,z)*vs        */
/* (the fusion grid).  Out-of-range corners contribute zero.                  */
/* ------------------------------------------------------------------------ */
void orc_grid_gather(long P, int C, int D, const float *pts, const int *batch,
                     const float *bbox_min, const float *voxel_size,
                     const float *grid, double *out) {
#pragma omp parallel for schedule(static)
  for (long p = 0; p < P; p++) {
    int b = batch ? batch[p] : 0;
    double u[3];
    for (int a = 0; a < 3; a++) u[a] = ((double)pts[p * 3 + a] - bbox_min[b * 3 + a]) / voxel_size[b];
    int i0[3];
    double f[3];
    for (int a = 0; a < 3; a++) { i0[a] = (int)floor(u[a]); f[a] = u[a] - i0[a]; }
    for (int c = 0; c < C; c++) out[p * C + c] = 0;
    for (int cr = 0; cr < 8; cr++) {
      int ix = i0[0] + ((cr >> 2) & 1), iy = i0[1] + ((cr >> 1) & 1), iz = i0[2] + (cr & 1);
      if (ix < 0 || iy < 0 || iz < 0 || ix >= D || iy >= D || iz >= D) continue;
      double w = (((cr >> 2) & 1) ? f[0] : 1 - f[0]) * (((cr >> 1) & 1) ? f[1] : 1 - f[1]) * ((cr & 1) ? f[2] : 1 - f[2]);
      const float *g = grid + ((((size_t)b * D + ix) * D + iy) * D + iz) * C;
      for (int c = 0; c < C; c++) out[p * C + c] += w * g[c];
    }
  }
}

void orc_grid_scatter(long P, int C, int D, int B, const float *pts,
                      const int *batch, const float *bbox_min,
                      const float *voxel_size, const float *gout,
                      double *ggrid) {
  /* sequential: deterministic double accumulation */
  (void)B;
  for (long p = 0; p < P; p++) {
    int b = batch ? batch[p] : 0;
    double u[3];
    for (int a = 0; a < 3; a++) u[a] = ((double)pts[p * 3 + a] - bbox_min[b * 3 + a]) / voxel_size[b];
    int i0[3];
    double f[3];
    for (int a = 0; a < 3; a++) { i0[a] = (int)floor(u[a]); f[a] = u[a] - i0[a]; }
    for (int cr = 0; cr < 8; cr++) {
      int ix = i0[0] + ((cr >> 2) & 1), iy = i0[1] + ((cr >> 1) & 1), iz = i0[2] + (cr & 1);
      if (ix < 0 || iy < 0 || iz < 0 || ix >= D || iy >= D || iz >= D) continue;
      double w = (((cr >> 2) & 1) ? f[0] : 1 - f[0]) * (((cr >> 1) & 1) ? f[1] : 1 - f[1]) * ((cr & 1) ? f[2] : 1 - f[2]);
      double *g = ggrid + ((((size_t)b * D + ix) * D + iy) * D + iz) * C;
      for (int c = 0; c < C; c++) g[c] += w * gout[p * C + c];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Projection of sampled points into the views: project_xyz,                 */
/* sampling_kernel.cu:55-159 (host MultiLayerOctree::project_sampled_xyz     */
/* :1333-1381).  Items (b, v, r, s), s fastest.  The sample point is         */
/* ori + dir * z (:89-91, one fma as nvcc contracts it); camera point and    */
/* pixel use the operand order of integrate_cuda's projection (the same      */
/* expressions); pixel / pixel_z in float; the [-1, 1] normalisation in      */
/* double, as the reference's ori_w / 2.0 makes it (:113-114).  corners:     */
/* [n_nodes][8][3] corner table indexed by node id (NULL: record_corners     */
/* off); items with node id -1 keep the -1 fill, as do the corners of an     */
/* id outside the table.                                                     */
/* ------------------------------------------------------------------------ */
static void orc_proj_one(const float *K, const float *P, float x, float y, float z, int w, int h,
                         float *gx, float *gy, float *cz) {
  float cx = fmaf(P[2], z, fmaf(P[0], x, P[1] * y)) + P[3];
  float cy = fmaf(P[6], z, fmaf(P[4], x, P[5] * y)) + P[7];
  float c3 = fmaf(P[10], z, fmaf(P[8], x, P[9] * y)) + P[11];
  float ux = fmaf(K[2], c3, fmaf(K[0], cx, K[1] * cy));
  float uy = fmaf(K[5], c3, fmaf(K[3], cx, K[4] * cy));
  float uz = fmaf(K[8], c3, fmaf(K[6], cx, K[7] * cy));
  ux = ux / uz;
  uy = uy / uz;
  *gx = (float)(((double)ux - w / 2.0) / (w / 2.0));
  *gy = (float)(((double)uy - h / 2.0) / (h / 2.0));
  *cz = c3;
}

void orc_project_xyz(int B, int V, int N, int S, const float *ori, const float *dir, const float *z,
                     const int *idx, const float *K, const float *RT, int w, int h, const float *corners,
                     int n_nodes, float *xy, float *pz) {
  const int per = corners ? 9 : 1;
  long total = (long)B * V * N * S;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < total; k++) {
    long rs = k % ((long)N * S), bv = k / ((long)N * S);
    int b = (int)(bv / V);
    long si = (long)b * N * S + rs;
    long r = rs / S;
    float *oxy = xy + k * 2 * per, *oz = pz + k * per;
    for (int i = 0; i < per; i++) {
      oxy[2 * i] = -1.0f;
      oxy[2 * i + 1] = -1.0f;
      oz[i] = -1.0f;
    }
    int id = idx[si];
    if (id == -1) continue;
    const float *o = ori + ((long)b * N + r) * 3, *d = dir + ((long)b * N + r) * 3;
    float zs = z[si];
    float px = fmaf(d[0], zs, o[0]), py = fmaf(d[1], zs, o[1]), p3 = fmaf(d[2], zs, o[2]);
    const float *Kk = K + bv * 9, *P = RT + bv * 12;
    orc_proj_one(Kk, P, px, py, p3, w, h, &oxy[0], &oxy[1], &oz[0]);
    if (!corners || id < 0 || id >= n_nodes) continue;
    for (int i = 0; i < 8; i++) {
      const float *c = corners + ((size_t)id * 8 + i) * 3;
      orc_proj_one(Kk, P, c[0], c[1], c[2], w, h, &oxy[2 * (i + 1)], &oxy[2 * (i + 1) + 1], &oz[i + 1]);
    }
  }
}
