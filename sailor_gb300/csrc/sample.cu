// sample.cu -- adaptive sampling in hit intervals and per-ray sort, sm_103a.
//
// Replaces sampling_kernel.cu (SAILOR c_lib/VoxelEncoding/src):
//   ray_voxels_sampling_uniform_kernel :1070-1177 (host :1251-1304) and
//   sort_samplings :1308-1329 (torch::sort along dim 2).
//
// One warp per ray (warp_sample_ray in ray_core.cuh): hit counts per chunk
// of 32 hits, a warp prefix sum in place of the reference's serial "samples
// left" capping, position-parallel sample generation into shared memory,
// then one coalesced row write.  Sample depths reproduce the reference's
// double-precision expression with float-only error-free arithmetic.
//
// sort_rows_kernel / sample_sorted_kernel: the stable (depth, position)
// order of each row -- equal depths keep their input order -- from a
// register bitonic network on 32-bit depth keys and a ranking pass
// (warp_sort_ranked in ray_core.cuh).
#include "ray_core.cuh"

namespace sg {

template <int E>
__global__ void __launch_bounds__(256) sample_coarse_kernel(SampleParams p) {
  __shared__ float s_z[8][32 * E];
  __shared__ int s_i[8][32 * E];
  __shared__ SampleScratch s_sc[8];
  const int lane = lane_id(), w8 = threadIdx.x >> 5;
  const long R = (long)p.t.B * p.N;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    warp_sample_ray(p, r, (int)(r / p.N), p.S, p.W, 0.5f, s_z[w8], s_i[w8], s_sc[w8]);
    for (int q = lane; q < p.S; q += 32) {
      p.sampled_z[(size_t)r * p.S + q] = s_z[w8][q];
      p.sampled_idx[(size_t)r * p.S + q] = s_i[w8][q];
    }
    __syncwarp();
  }
}

// A warp per row: the row goes through shared memory into the ranked sort
// (warp_sort_ranked).  VEC: rows start 16-byte aligned and S is a multiple
// of 4, so each lane's run of E consecutive elements moves as float2 /
// float4 / int4 (a run of 8 as two quads, each within the row or wholly
// past its end).
template <int E, bool VEC>
__global__ void __launch_bounds__(256) sort_rows_kernel(const float *__restrict__ z, long R, int S,
                                                        float *sorted, int *idx) {
  constexpr int Q = E < 4 ? E : 4;  // elements per vector access
  __shared__ __align__(16) float s_v[8][32 * E];
  __shared__ __align__(16) int s_p[8][32 * E];
  const int lane = lane_id(), w8 = threadIdx.x >> 5;
  const int i0 = lane * E;
  float *sv = s_v[w8];
  int *sp = s_p[w8];
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    const float *zr = z + (size_t)r * S;
#pragma unroll
    for (int q = 0; q < E; q += Q) {
      float t[Q];
      if (VEC && Q > 1) {
        if (i0 + q < S) {
          load_run<Q>(zr + i0 + q, t);
        } else {
#pragma unroll
          for (int u = 0; u < Q; u++) t[u] = 0.0f;
        }
      } else {
#pragma unroll
        for (int u = 0; u < Q; u++) t[u] = (i0 + q + u < S) ? __ldg(zr + i0 + q + u) : 0.0f;
      }
      uint32_t w[Q];
#pragma unroll
      for (int u = 0; u < Q; u++) w[u] = __float_as_uint(t[u]);
      store_run<Q>(reinterpret_cast<uint32_t *>(sv + i0 + q), w);
    }
    __syncwarp();
    uint32_t key[E];
    int pos[E];
    warp_sort_ranked<E>(sv, sp, S, key, pos);
#pragma unroll
    for (int e = 0; e < E; e++)
      if (e * 32 + lane < S) sp[pos[e]] = e * 32 + lane;
    __syncwarp();
    float *sr = sorted + (size_t)r * S;
    int *ir = idx + (size_t)r * S;
#pragma unroll
    for (int q = 0; q < E; q += Q) {
      if (VEC && Q > 1) {
        if (i0 + q < S) {
          if constexpr (Q == 2) {
            *reinterpret_cast<float2 *>(sr + i0 + q) = make_float2(from_ordered(key[q]), from_ordered(key[q + 1]));
            *reinterpret_cast<int2 *>(ir + i0 + q) = *reinterpret_cast<const int2 *>(sp + i0 + q);
          } else if constexpr (Q == 4) {
            *reinterpret_cast<float4 *>(sr + i0 + q) = make_float4(from_ordered(key[q]), from_ordered(key[q + 1]),
                                                                   from_ordered(key[q + 2]), from_ordered(key[q + 3]));
            *reinterpret_cast<int4 *>(ir + i0 + q) = *reinterpret_cast<const int4 *>(sp + i0 + q);
          }
        }
      } else {
#pragma unroll
        for (int u = 0; u < Q; u++) {
          if (i0 + q + u < S) {
            sr[i0 + q + u] = from_ordered(key[q + u]);
            ir[i0 + q + u] = sp[i0 + q + u];
          }
        }
      }
    }
    __syncwarp();
  }
}

// Fused sampling + per-ray sort (pipeline path): only the sorted depths and
// node ids are written (8 bytes per sample, one coalesced pass).  Hit rows
// may be compact (hit_count given) or -1 terminated (hit_count NULL).
template <int E>
__global__ void __launch_bounds__(256) sample_sorted_kernel(SampleParams p, const int *__restrict__ hit_count,
                                                            float rand_const, float *out_z, int *out_idx) {
  __shared__ __align__(16) float s_z[8][32 * E];
  __shared__ int s_i[8][32 * E];
  __shared__ int s_p[8][32 * E];
  __shared__ SampleScratch s_sc[8];
  const int lane = lane_id(), w8 = threadIdx.x >> 5;
  const long R = (long)p.t.B * p.N;
  const int S = p.S;
  for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < R;
       r += ((long)gridDim.x * blockDim.x) >> 5) {
    const int nh = hit_count ? min(hit_count[r], p.W) : p.W;
    const int done = warp_sample_ray(p, r, (int)(r / p.N), S, nh, rand_const, s_z[w8], s_i[w8], s_sc[w8]);
    warp_sort_samples<E, true>(s_z[w8], s_p[w8], S, done);
    for (int i = lane; i < S; i += 32) {
      out_z[(size_t)r * S + i] = s_z[w8][i];
      out_idx[(size_t)r * S + i] = s_i[w8][s_p[w8][i]];
    }
    __syncwarp();
  }
}

template <int E>
static void launch_sample_coarse(const SampleParams &p, int g, sg_stream_t s) {
  sample_coarse_kernel<E><<<g, 256, 0, s>>>(p);
}

}  // namespace sg

using namespace sg;

static int grid_for(long R) {
  int g = ceil_div(R * 32, 256);
  return g > num_sms() * 64 ? num_sms() * 64 : g;
}

extern "C" int sg_sample_sorted(const SgTree *tree, const int *hit_idx, const float *hit_t0,
                                const float *hit_t1, const int *hit_count, int N, int W, const float *rands,
                                float rand_const, const float *valid_len, int S, int num_levels,
                                int start_level, float *sorted_z, int *sorted_idx, sg_stream_t stream) {
  if (!tree || !hit_idx || !hit_t0 || !hit_t1 || !valid_len || !sorted_z || !sorted_idx)
    return SG_ERR_INVALID_ARG;
  if (N <= 0 || W <= 0 || S <= 0 || tree->B <= 0) return SG_ERR_INVALID_ARG;
  SampleParams p{*tree, hit_idx, hit_t0, hit_t1, rands, valid_len, N, W, S, num_levels, start_level,
                 nullptr, nullptr, 0ull};
  int g = grid_for((long)tree->B * N);
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
                 sampled_idx, sampled_z, 0ull};
  int g = grid_for((long)tree->B * N);
  if (S <= 32) launch_sample_coarse<1>(p, g, stream);
  else if (S <= 64) launch_sample_coarse<2>(p, g, stream);
  else if (S <= 128) launch_sample_coarse<4>(p, g, stream);
  else if (S <= 256) launch_sample_coarse<8>(p, g, stream);
  else return SG_ERR_UNSUPPORTED;
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_sort_samples(const float *z, int R, int S, float *sorted, int *idx, sg_stream_t stream) {
  if (R < 0 || S <= 0) return SG_ERR_INVALID_ARG;
  if (R == 0) return SG_OK;  // no rows (the buffers may be NULL)
  if (!z || !sorted || !idx) return SG_ERR_INVALID_ARG;
  int g = grid_for(R);
  const bool vec = (S % 4 == 0) && ((((uintptr_t)z) | ((uintptr_t)sorted) | ((uintptr_t)idx)) & 15) == 0;
  auto go = [&](auto tag) {
    constexpr int E = decltype(tag)::value;
    if (vec) sort_rows_kernel<E, true><<<g, 256, 0, stream>>>(z, R, S, sorted, idx);
    else sort_rows_kernel<E, false><<<g, 256, 0, stream>>>(z, R, S, sorted, idx);
  };
  if (S <= 32) go(std::integral_constant<int, 1>());
  else if (S <= 64) go(std::integral_constant<int, 2>());
  else if (S <= 128) go(std::integral_constant<int, 4>());
  else if (S <= 256) go(std::integral_constant<int, 8>());
  else return SG_ERR_UNSUPPORTED;
  SG_LAUNCH_CHECK();
  return SG_OK;
}
