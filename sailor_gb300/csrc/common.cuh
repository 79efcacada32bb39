// common.cuh -- shared device helpers of the sm_103a VoxelEncoding kernels.
//
// The library is compiled with -fmad=false: no multiply-add is contracted
// unless written as __fmaf_rn.  Steps whose rounding decides an integer
// (pixel choice, slab tests, DDA steps, sample counts) are written with the
// operation order and fused multiply-adds that nvcc's default contraction
// gives the reference's source expressions, so those integers come out the
// same as the reference's.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sailor_gb300.h"

#define SG_FULL 0xffffffffu

namespace sg {

constexpr int kWarp = 32;

__host__ __device__ inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// 32-bit words of fine-occupancy bits per brick: max(1, rate^3 / 32)
__host__ __device__ inline int sg_mask_words_dev(int rate) {
  int r3 = rate * rate * rate;
  return r3 <= 32 ? 1 : (r3 + 31) / 32;
}

// ---------------------------------------------------------------------------
// reference arithmetic
// ---------------------------------------------------------------------------

// a0*x + a1*y + a2*z as nvcc contracts it: fma(a2, z, fma(a0, x, a1*y)).
__device__ __forceinline__ float dot3c(float a0, float a1, float a2, float x,
                                       float y, float z) {
  return __fmaf_rn(a2, z, __fmaf_rn(a0, x, __fmul_rn(a1, y)));
}

// p*q - r*s as nvcc contracts it: fma(p, q, -(r*s)).
__device__ __forceinline__ float msub(float p, float q, float r, float s) {
  return __fmaf_rn(p, q, -__fmul_rn(r, s));
}

// 3x3 inverse by adjugate / determinant (fusion_kernel.cu:105-135).
__device__ inline void inverse3x3(const float *m, float *o) {
  float a1 = m[0], b1 = m[1], c1 = m[2];
  float a2 = m[3], b2 = m[4], c2 = m[5];
  float a3 = m[6], b3 = m[7], c3 = m[8];
  float X = msub(b2, c3, c2, b3), Y = msub(b1, c3, c1, b3), Z = msub(b1, c2, c1, b2);
  float det = __fmaf_rn(a3, Z, __fmaf_rn(a1, X, -__fmul_rn(a2, Y)));
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

// Node centre and edge of a level: OcTree::calculate_bbox_start and
// calculate_xyz_corners (octree.h:109-151) as set up by
// gen_root_octree_nodes (octree_kernel.cu:157-217).  size = fine voxels per
// node edge (rate for a top brick, 1 for a fine voxel).
struct LevelGeom {
  float vs;      // node edge in metres
  float start;   // per-axis offset added to bbox_min
};

__device__ __forceinline__ LevelGeom level_geom(float vs_bottom, int size) {
  LevelGeom g;
  g.vs = vs_bottom * (float)size;
  float basic = g.vs / (float)size;
  int rate_vol = (int)log2f((float)size);
  float off = 0.0f;
  for (int i = 0; i < rate_vol; i++) off = off + ldexpf(1.0f, i) * basic / 2.0f;
  g.start = off;
  return g;
}

__device__ __forceinline__ float node_coord(const LevelGeom &g, float bbox_min, int idx) {
  return __fmaf_rn(g.vs, (float)idx, bbox_min + g.start);
}

// Ray / cube slab test (RayVoxelIntersection, intersection_kernel.cu:36-71).
// inv holds __fdividef(1, dir) per axis, as the reference computes it.
__device__ __forceinline__ bool slab(const float o[3], const float inv[3], float cx,
                                     float cy, float cz, float vs, float &t0, float &t1) {
  float f_low = 0.0f, f_high = 100000.0f;
  float h = vs / 2.0f;
  float c[3] = {cx, cy, cz};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    float lo = ((c[i] - h) - o[i]) * inv[i];
    float hi = ((c[i] + h) - o[i]) * inv[i];
    if (lo > hi) {
      float t = lo;
      lo = hi;
      hi = t;
    }
    if (hi < f_low) return false;
    if (lo > f_high) return false;
    f_low = (lo > f_low) ? lo : f_low;
    f_high = (hi < f_high) ? hi : f_high;
    if (f_low > f_high) return false;
  }
  t0 = f_low;
  t1 = f_high;
  return true;
}

// ---------------------------------------------------------------------------
// float-only reproduction of  (float)((double)a - (double)b/2.0 + (double)p)
// The reference forms sample depths in double (sampling_kernel.cu:1148,1169);
// production kernels use no FP64, so the correctly rounded float sum of
// three floats is formed with error-free transformations and rounding to
// odd (S. Boldo, G. Melquiond, "Emulation of FMA and correctly rounded sums:
// proved algorithms using rounding to odd", IEEE Trans. Computers 57(4),
// 2008).  It equals the reference whenever the double evaluation is exact
// before its final rounding, which holds unless the three magnitudes span
// more than ~29 binary orders.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ float add_round_odd(float a, float b) {
  float s, e;
  two_sum(a, b, s, e);
  uint32_t u = __float_as_uint(s);
  if (e != 0.0f && (u & 1u) == 0u) {
    bool up = (e > 0.0f) == (s > 0.0f);
    u = up ? u + 1u : u - 1u;
    s = __uint_as_float(u);
  }
  return s;
}

__device__ __forceinline__ float sum3_rn(float a, float b, float c) {
  float uh, ul, th, tl;
  two_sum(b, c, uh, ul);
  two_sum(a, uh, th, tl);
  float v = add_round_odd(tl, ul);
  return __fadd_rn(th, v);
}

// ---------------------------------------------------------------------------
// warp helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(SG_FULL, v, o);
  return v;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
  int lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int n = __shfl_up_sync(SG_FULL, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

__device__ __forceinline__ float warp_incl_scan_f(float v) {
  int lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    float n = __shfl_up_sync(SG_FULL, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

__device__ __forceinline__ void status_or(SgStatus *st, int f) {
  if (st) atomicOr(&st->flags, f);
}

// launch-shape knobs (sg_tune_set / sg_tune_get, capi.cu)
int tune(int knob);

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount,
// looked up once per device; capi.cu).  Grid caps of the grid-stride kernels
// are multiples of it.
int num_sms();

// -1 padding of one hit row's tail [c, W) by the calling warp: scalar
// stores up to a 4-element boundary, then 16-byte stores.  base = the row's
// first element (row index x W).
__device__ __forceinline__ void pad_row_tail(int *idx, float *t0, float *t1, size_t base, int c, int W, int lane) {
  int head = c;
  while (head < W && ((base + head) & 3)) {
    if (lane == 0) {
      idx[base + head] = -1;
      t0[base + head] = -1.0f;
      t1[base + head] = -1.0f;
    }
    head++;
  }
  const int nvec = (W - head) / 4;
  const int4 mi = make_int4(-1, -1, -1, -1);
  const float4 mf = make_float4(-1.f, -1.f, -1.f, -1.f);
  for (int q = lane; q < nvec; q += 32) {
    const size_t o = base + head + 4 * q;
    *reinterpret_cast<int4 *>(idx + o) = mi;
    *reinterpret_cast<float4 *>(t0 + o) = mf;
    *reinterpret_cast<float4 *>(t1 + o) = mf;
  }
  for (int q = head + 4 * nvec + lane; q < W; q += 32) {
    idx[base + q] = -1;
    t0[base + q] = -1.0f;
    t1[base + q] = -1.0f;
  }
}

// -1 padding of hit-row tails [count[r], W) of R rows (a warp per row, 16-byte
// stores where the row is aligned); defined in intersect.cu
void launch_pad_rows(long R, int W, const int *count, int *idx, float *t0, float *t1, sg_stream_t stream);

// ---------------------------------------------------------------------------
// ray generation (rays_calculating_kernel, sampling_kernel.cu:411-486)
// ---------------------------------------------------------------------------
constexpr int kCamFloats = 21;  // K^-1 (9), R^-1 (9), centre (3)

// Camera table entry from K, R, T: the reference's inverses and centre.
__device__ __forceinline__ void camera_params(const float *K, const float *R, const float *T, float *cam) {
  inverse3x3(K, cam);
  inverse3x3(R, cam + 9);
  const float *ri = cam + 9;
#pragma unroll
  for (int k = 0; k < 3; k++)
    cam[18 + k] = __fmaf_rn(-ri[3 * k + 2], T[2], __fmaf_rn(-ri[3 * k + 1], T[1], -(ri[3 * k] * T[0])));
}

// Ray of pixel (h, w): direction R^-1 K^-1 [w, h, 1] / (|.| + 1e-10), with the
// multiply-adds of the reference kernel; the reference divides in double,
// the single-precision quotient here is within one ulp of it.  cam: a
// camera table entry in shared memory or (GLOBAL) read-only global memory.
template <bool GLOBAL>
__device__ __forceinline__ void pixel_ray(const float *cam, int h, int w, float o[3], float d[3]) {
  auto c = [&](int k) { return GLOBAL ? __ldg(cam + k) : cam[k]; };
  float cd[3], wd[3];
#pragma unroll
  for (int k = 0; k < 3; k++) cd[k] = __fmaf_rn((float)w, c(3 * k), (float)h * c(3 * k + 1)) + c(3 * k + 2);
#pragma unroll
  for (int k = 0; k < 3; k++)
    wd[k] = __fmaf_rn(cd[2], c(9 + 3 * k + 2), __fmaf_rn(cd[0], c(9 + 3 * k), cd[1] * c(9 + 3 * k + 1)));
  const float nd = sqrtf(__fmaf_rn(wd[2], wd[2], __fmaf_rn(wd[0], wd[0], wd[1] * wd[1]))) + 1e-10f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    o[k] = c(18 + k);
    d[k] = wd[k] / nd;
  }
}

// Origin and direction of ray r of segment s: generated from the segment's
// camera (cams != NULL) or read from ori / dir.
__device__ __forceinline__ void segment_ray(const float *__restrict__ ori, const float *__restrict__ dir,
                                            const float *__restrict__ cams, const int *__restrict__ widths,
                                            const int *__restrict__ seg_begin, int s, long r, float o[3],
                                            float d[3]) {
  if (cams) {
    const int p = (int)(r - __ldg(seg_begin + s));
    const int W = __ldg(widths + s);
    const int h = p / W;
    pixel_ray<true>(cams + (size_t)s * kCamFloats, h, p - h * W, o, d);
  } else {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      o[k] = __ldg(ori + r * 3 + k);
      d[k] = __ldg(dir + r * 3 + k);
    }
  }
}

}  // namespace sg

// launch-error check used by every entry point
// Segment of ray r: the last s with begin[s] <= r (begin ascending, n >= 1).
__device__ __forceinline__ int segment_of(const int *__restrict__ begin, int n, long r) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((long)__ldg(begin + mid) <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Uniform [0, 1) jitter from (seed, ray, position): the SplitMix64
// finaliser (Steele, Lea and Flood, 2014) of a Weyl-sequence key; 24 bits.
__device__ __forceinline__ float hash_uniform(unsigned long long seed, long r, int q) {
  unsigned long long x = seed + (unsigned long long)r * 0x9E3779B97F4A7C15ull + (unsigned long long)q;
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (float)(x >> 40) * (1.0f / 16777216.0f);
}

// Fire-and-forget vector reduction of four consecutive floats (PTX
// red.global.add.v4.f32, sm_90 and later); addr must be 16-byte aligned.
__device__ __forceinline__ void red_add_f32x4(float *addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

#define SG_LAUNCH_CHECK()                           \
  do {                                              \
    cudaError_t _e = cudaGetLastError();            \
    if (_e != cudaSuccess) return SG_ERR_CUDA;      \
  } while (0)
