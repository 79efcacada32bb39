// sample.cu -- adaptive sampling in hit intervals and per-ray sort, sm_103a.
//
// Replaces sampling_kernel.cu (SAILOR c_lib/VoxelEncoding/src):
//   ray_voxels_sampling_uniform_kernel :1070-1177 (host :1251-1304) and
//   sort_samplings :1308-1329 (torch::sort along dim 2).
//
// sample_coarse_kernel: one warp per ray.  Lanes take 32 hits at a time
// (coalesced row reads), compute each hit's sample count exactly as the
// reference's serial loop does, and a warp prefix sum turns the serial
// "samples left" capping into per-hit output ranges, so each lane emits its
// hit's samples independently.  Sample depths reproduce the reference's
// double-precision expression with float-only error-free arithmetic.  Row
// entries without a sample are written -1 by the same kernel (the reference
// pre-fills with torch::full).
//
// sort_rows_kernel: one warp per row, a register bitonic network on
// (depth, index) keys -- a total order, so equal depths keep input order.
#include "common.cuh"

namespace sg {

struct SampleParams {
  SgTree t;
  const int *hit_idx;
  const float *hit_t0, *hit_t1, *rands, *valid_len;
  int N, W, S, num_levels, start_level;
  int *sampled_idx;
  float *sampled_z;
};

// depth of the j-th sample (0-based) of a hit with n samples:
// base = min + off*(j+1); z = base - off/2 + off*rand   (sampling_kernel.cu:1142-1148)
__device__ __forceinline__ float sample_z(float mn, float off, int j, float rnd) {
  float base = __fmaf_rn(off, (float)(j + 1), mn);
  return sum3_rn(base, -(off * 0.5f), off * rnd);
}

__global__ void __launch_bounds__(256) sample_coarse_kernel(SampleParams p) {
  const int lane = lane_id();
  const long R = (long)p.t.B * p.N;
  const int S = p.S;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    const int b = (int)(r / p.N);
    const int *hi = p.hit_idx + (size_t)r * p.W;
    const float *h0 = p.hit_t0 + (size_t)r * p.W, *h1 = p.hit_t1 + (size_t)r * p.W;
    const float *rd = p.rands + (size_t)r * S;
    int *si = p.sampled_idx + (size_t)r * S;
    float *sz = p.sampled_z + (size_t)r * S;
    int done = 0;  // samples written (positions [0, done) hold samples)
    if (__ldg(hi) >= 0) {
      const float vl = p.valid_len[r];
      const float vs = p.t.voxel_size[b];
      const float start_vs = vs * ldexpf(1.0f, 2 * (p.num_levels - p.start_level - 1));
      const float vs_top = vs * (float)(p.t.Db / p.t.Dt);
      int has = 0, nvalid = 0;
      bool stop = false;
      for (int c0 = 0; c0 < p.W && !stop; c0 += 32) {
        int i = c0 + lane;
        int id = -1;
        float mn = -1.0f, mx = -1.0f;
        if (i < p.W) {
          id = __ldg(hi + i);
          mn = __ldg(h0 + i);
          mx = __ldg(h1 + i);
        }
        bool ok = i < p.W && !(id < 0 || mn < 0 || mx < 0);
        unsigned bad = __ballot_sync(SG_FULL, !ok);
        int first_bad = bad ? __ffs(bad) - 1 : 32;
        ok = ok && lane < first_bad;
        if (bad) stop = true;
        int n = 0;
        if (ok) {
          float nvs = (id >= p.t.base_top) ? vs_top : vs;
          float rate = start_vs / nvs;
          n = (int)((mx - mn) * rate * (float)S / vl);
          n = n >= 1 ? n : 1;
          n = n < S ? n : S;
        }
        int incl = warp_incl_scan(n);
        int start = has + incl - n;
        int ne = S - start;
        ne = ne < 0 ? 0 : (ne < n ? ne : n);
        if (ne > 0) {
          float off = (mx - mn) / (float)(ne + 1);
          for (int j = 0; j < ne; j++) {
            int q = start + j;
            sz[q] = sample_z(mn, off, j, __ldg(rd + q));
            si[q] = id;
          }
        }
        int tot = __shfl_sync(SG_FULL, incl, 31);
        has = min(has + tot, S);
        nvalid += __popc(__ballot_sync(SG_FULL, ok));
      }
      // leftover: one more sample in each of the first hits (:1156-1174)
      int left = S - has;
      int cnt = left < nvalid ? left : nvalid;
      for (int i = lane; i < cnt; i += 32) {
        int id = __ldg(hi + i);
        float mn = __ldg(h0 + i), mx = __ldg(h1 + i);
        float off = (mx - mn) * 0.5f;
        float base = mn + off;
        int q = has + i;
        sz[q] = sum3_rn(base, -(off * 0.5f), off * __ldg(rd + q));
        si[q] = id;
      }
      done = has + cnt;
    }
    for (int q = done + lane; q < S; q += 32) {
      sz[q] = -1.0f;
      si[q] = -1;
    }
  }
}

// ---------------------------------------------------------------------------
// per-row sort
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ordered_bits(float f) {
  uint32_t u = __float_as_uint(f);
  return u ^ ((u >> 31) ? 0xffffffffu : 0x80000000u);
}
__device__ __forceinline__ float from_ordered(uint32_t k) {
  return __uint_as_float((k >> 31) ? (k ^ 0x80000000u) : ~k);
}

// E keys per lane, element i = e*32 + lane, P = 32*E (power of two)
template <int E>
__device__ __forceinline__ void bitonic_warp(unsigned long long (&key)[E]) {
  const int lane = lane_id();
  constexpr int P = 32 * E;
#pragma unroll
  for (int k = 2; k <= P; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int m = j >> 5;
#pragma unroll
        for (int e = 0; e < E; e++) {
          if ((e & m) == 0) {
            const int i = e * 32 + lane;
            const bool asc = (i & k) == 0;
            unsigned long long a = key[e], c = key[e ^ m];
            bool sw = asc ? (a > c) : (a < c);
            key[e] = sw ? c : a;
            key[e ^ m] = sw ? a : c;
          }
        }
      } else {
#pragma unroll
        for (int e = 0; e < E; e++) {
          const int i = e * 32 + lane;
          const bool asc = (i & k) == 0;
          unsigned long long other = __shfl_xor_sync(SG_FULL, key[e], j);
          const bool lower = (lane & j) == 0;
          unsigned long long mn = key[e] < other ? key[e] : other;
          unsigned long long mx = key[e] < other ? other : key[e];
          key[e] = (lower == asc) ? mn : mx;
        }
      }
    }
  }
}

template <int E>
__global__ void __launch_bounds__(256) sort_rows_kernel(const float *__restrict__ z, long R, int S,
                                                        float *sorted, int *idx) {
  const int lane = lane_id();
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    unsigned long long key[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      int i = e * 32 + lane;
      key[e] = (i < S) ? (((unsigned long long)ordered_bits(__ldg(z + (size_t)r * S + i)) << 32) | (unsigned)i)
                       : ~0ull;
    }
    bitonic_warp<E>(key);
#pragma unroll
    for (int e = 0; e < E; e++) {
      int i = e * 32 + lane;
      if (i < S) {
        sorted[(size_t)r * S + i] = from_ordered((uint32_t)(key[e] >> 32));
        idx[(size_t)r * S + i] = (int)(key[e] & 0xffffffffu);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// fused sampling + per-ray sort (pipeline path)
// ---------------------------------------------------------------------------
// Same per-ray sampling as sample_coarse_kernel, but the samples of a ray go
// to shared memory, are sorted there by (depth, position) with the register
// bitonic network, and only the sorted depths and node ids are written: one
// coalesced 8-byte-per-sample write instead of the reference's two
// write-then-sort passes.  Hit rows may be compact (hit_count given: the
// first hit_count[r] entries are the hits) or -1 terminated (hit_count
// NULL).  rands NULL: every jitter is rand_const (the inference setting).
template <int E>
__global__ void __launch_bounds__(256) sample_sorted_kernel(SampleParams p, const int *__restrict__ hit_count,
                                                            float rand_const, float *out_z, int *out_idx) {
  __shared__ float s_z[8][32 * E];
  __shared__ int s_i[8][32 * E];
  const int lane = lane_id();
  const int w8 = threadIdx.x >> 5;
  const long R = (long)p.t.B * p.N;
  const int S = p.S;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    const int b = (int)(r / p.N);
    const int *hi = p.hit_idx + (size_t)r * p.W;
    const float *h0 = p.hit_t0 + (size_t)r * p.W, *h1 = p.hit_t1 + (size_t)r * p.W;
    const float *rd = p.rands ? p.rands + (size_t)r * S : nullptr;
    const int nh = hit_count ? min(hit_count[r], p.W) : p.W;
    float *sz = s_z[w8];
    int *si = s_i[w8];
    int done = 0;
    if (nh > 0 && __ldg(hi) >= 0) {
      const float vl = p.valid_len[r];
      const float vs = p.t.voxel_size[b];
      const float start_vs = vs * ldexpf(1.0f, 2 * (p.num_levels - p.start_level - 1));
      const float vs_top = vs * (float)(p.t.Db / p.t.Dt);
      int has = 0, nvalid = 0;
      bool stop = false;
      for (int c0 = 0; c0 < nh && !stop; c0 += 32) {
        int i = c0 + lane;
        int id = -1;
        float mn = -1.0f, mx = -1.0f;
        if (i < nh) {
          id = __ldg(hi + i);
          mn = __ldg(h0 + i);
          mx = __ldg(h1 + i);
        }
        bool ok = i < nh && !(id < 0 || mn < 0 || mx < 0);
        unsigned bad = __ballot_sync(SG_FULL, !ok);
        int first_bad = bad ? __ffs(bad) - 1 : 32;
        ok = ok && lane < first_bad;
        if (bad) stop = true;
        int n = 0;
        if (ok) {
          float nvs = (id >= p.t.base_top) ? vs_top : vs;
          float rate = start_vs / nvs;
          n = (int)((mx - mn) * rate * (float)S / vl);
          n = n >= 1 ? n : 1;
          n = n < S ? n : S;
        }
        int incl = warp_incl_scan(n);
        int start = has + incl - n;
        int ne = S - start;
        ne = ne < 0 ? 0 : (ne < n ? ne : n);
        if (ne > 0) {
          float off = (mx - mn) / (float)(ne + 1);
          for (int j = 0; j < ne; j++) {
            int q = start + j;
            sz[q] = sample_z(mn, off, j, rd ? __ldg(rd + q) : rand_const);
            si[q] = id;
          }
        }
        int tot = __shfl_sync(SG_FULL, incl, 31);
        has = min(has + tot, S);
        nvalid += __popc(__ballot_sync(SG_FULL, ok));
      }
      int left = S - has;
      int cnt = left < nvalid ? left : nvalid;
      for (int i = lane; i < cnt; i += 32) {
        int id = __ldg(hi + i);
        float mn = __ldg(h0 + i), mx = __ldg(h1 + i);
        float off = (mx - mn) * 0.5f;
        float base = mn + off;
        int q = has + i;
        sz[q] = sum3_rn(base, -(off * 0.5f), off * (rd ? __ldg(rd + q) : rand_const));
        si[q] = id;
      }
      done = has + cnt;
    }
    for (int q = done + lane; q < S; q += 32) {
      sz[q] = -1.0f;
      si[q] = -1;
    }
    __syncwarp();
    unsigned long long key[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      int i = e * 32 + lane;
      key[e] = (i < S) ? (((unsigned long long)ordered_bits(sz[i]) << 32) | (unsigned)i) : ~0ull;
    }
    bitonic_warp<E>(key);
#pragma unroll
    for (int e = 0; e < E; e++) {
      int i = e * 32 + lane;
      if (i < S) {
        int pos = (int)(key[e] & 0xffffffffu);
        out_z[(size_t)r * S + i] = from_ordered((uint32_t)(key[e] >> 32));
        out_idx[(size_t)r * S + i] = si[pos];
      }
    }
    __syncwarp();
  }
}

}  // namespace sg

using namespace sg;

extern "C" int sg_sample_sorted(const SgTree *tree, const int *hit_idx, const float *hit_t0,
                                const float *hit_t1, const int *hit_count, int N, int W, const float *rands,
                                float rand_const, const float *valid_len, int S, int num_levels,
                                int start_level, float *sorted_z, int *sorted_idx, sg_stream_t stream) {
  if (!tree || !hit_idx || !hit_t0 || !hit_t1 || !valid_len || !sorted_z || !sorted_idx)
    return SG_ERR_INVALID_ARG;
  if (N <= 0 || W <= 0 || S <= 0 || tree->B <= 0) return SG_ERR_INVALID_ARG;
  SampleParams p{*tree, hit_idx, hit_t0, hit_t1, rands, valid_len, N, W, S, num_levels, start_level,
                 nullptr, nullptr};
  long R = (long)tree->B * N;
  int g = ceil_div(R * 32, 256);
  if (g > 152 * 64) g = 152 * 64;
  if (S <= 32) sample_sorted_kernel<1><<<g, 256, 0, stream>>>(p, hit_count, rand_const, sorted_z, sorted_idx);
  else if (S <= 64) sample_sorted_kernel<2><<<g, 256, 0, stream>>>(p, hit_count, rand_const, sorted_z, sorted_idx);
  else if (S <= 128) sample_sorted_kernel<4><<<g, 256, 0, stream>>>(p, hit_count, rand_const, sorted_z, sorted_idx);
  else return SG_ERR_UNSUPPORTED;
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_sample_coarse(const SgTree *tree, const int *hit_idx, const float *hit_t0,
                                const float *hit_t1, int N, int W, const float *rands,
                                const float *valid_len, int S, int num_levels, int start_level,
                                int *sampled_idx, float *sampled_z, sg_stream_t stream) {
  if (!tree || !hit_idx || !hit_t0 || !hit_t1 || !rands || !valid_len || !sampled_idx || !sampled_z)
    return SG_ERR_INVALID_ARG;
  if (N <= 0 || W <= 0 || S <= 0 || tree->B <= 0) return SG_ERR_INVALID_ARG;
  SampleParams p{*tree, hit_idx, hit_t0, hit_t1, rands, valid_len, N, W, S, num_levels, start_level,
                 sampled_idx, sampled_z};
  long R = (long)tree->B * N;
  int g = ceil_div(R * 32, 256);
  if (g > 152 * 64) g = 152 * 64;
  sample_coarse_kernel<<<g, 256, 0, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_sort_samples(const float *z, int R, int S, float *sorted, int *idx, sg_stream_t stream) {
  if (!z || !sorted || !idx || R < 0 || S <= 0) return SG_ERR_INVALID_ARG;
  if (R == 0) return SG_OK;
  int g = ceil_div((long)R * 32, 256);
  if (g > 152 * 64) g = 152 * 64;
  if (S <= 32) sort_rows_kernel<1><<<g, 256, 0, stream>>>(z, R, S, sorted, idx);
  else if (S <= 64) sort_rows_kernel<2><<<g, 256, 0, stream>>>(z, R, S, sorted, idx);
  else if (S <= 128) sort_rows_kernel<4><<<g, 256, 0, stream>>>(z, R, S, sorted, idx);
  else if (S <= 256) sort_rows_kernel<8><<<g, 256, 0, stream>>>(z, R, S, sorted, idx);
  else return SG_ERR_UNSUPPORTED;
  SG_LAUNCH_CHECK();
  return SG_OK;
}
