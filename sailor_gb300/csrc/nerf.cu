// nerf.cu -- FastNerf's occupancy (density) network on the sm_103a tensor
// cores (tcgen05.mma kind::f16, float32 accumulators in tensor memory).
//
// Replaces (SAILOR c_lib/FastNerf/src/infer_mlp.cu):
//   density_feat_kernel  :120-199  per point-view: feature MLP 18->64->64->64->64
//                                  and geometry MLP 18->16->8 (ReLU after each)
//   density_sigma_kernel :202-240  per point: 64->64->64->1, ReLU, ReLU, sigmoid
//   infer_density_mlp    :583-636  the two around a torch.mean over the views
//
// The reference runs one thread per point-view with scalar __hfma chains
// (float16 accumulation rounded at every product).  Here a persistent CTA of
// 128 threads takes tiles of 128 rows, P = floor(128 / V) points x V views
// (row v*P + p), so the view mean happens inside the CTA and no per-view
// feature reaches HBM:
//   inputs (z, t_psdf, 16 geometry features) -> float16 rows in shared memory
//   each layer: one elected thread issues tcgen05.mma (K-major float16 operands
//   in shared memory, the weights staged once per CTA) into tensor memory and
//   commits to an mbarrier; every thread then reads its own row back
//   (tcgen05.ld), adds the bias in float32, applies ReLU and rounds to float16
//   into the next layer's operand tile;
//   after the fourth feature layer the P point rows take the float32 mean of
//   their V view rows (view order, times 1/V, as torch's mean does here),
//   then the sigma layers; the last 64->1 layer is a per-row dot product in
//   the epilogue, rounded to float16 before the sigmoid as the reference
//   rounds it.
// Layer outputs are rounded to float16 at the same points as the reference;
// within a layer the products are summed in float32 instead of rounding each
// partial sum to float16, so results differ from the reference by the
// reference's own accumulation error (a few float16 ulps).
//
// Every mbarrier wait has an iteration limit: on expiry the kernel sets
// *error, stops taking tiles, frees its tensor memory and returns.
#include <cuda_fp16.h>

#include "common.cuh"
#include "tc05.cuh"

namespace sg {

constexpr int kNerfParamCount = 22521;
constexpr int kSigmaOff = 13696, kGeoOff = 22081;

struct NerfSmem {
  // weights [out][in] in the K-major float16 operand layout
  alignas(128) uint8_t w1[64 * 32 * 2];   // 18 -> 64, K padded to 32
  alignas(128) uint8_t w2[64 * 64 * 2];
  alignas(128) uint8_t w3[64 * 64 * 2];
  alignas(128) uint8_t w4[64 * 64 * 2];
  alignas(128) uint8_t ws1[64 * 64 * 2];
  alignas(128) uint8_t ws2[64 * 64 * 2];
  alignas(128) uint8_t wg1[16 * 32 * 2];  // 18 -> 16, K padded to 32
  alignas(128) uint8_t wg2[16 * 16 * 2];  // 16 -> 8, N padded to 16
  alignas(128) uint8_t a_in[128 * 32 * 2];  // layer-1 rows; then the geometry hidden rows (K = 16)
  alignas(128) uint8_t h[128 * 64 * 2];     // hidden rows; then the view means
  float b1[64], b2[64], b3[64], b4[64], bs1[64], bs2[64], ws3[64], bg1[16], bg2[8];
  float bs3;
  alignas(8) uint64_t mbar;
  uint32_t tmem_slot;
};

constexpr int kNerfThreads = 128;
constexpr uint32_t kNerfTmemCols = 128;  // feature accumulators 0..63, geometry 64..79
constexpr long kNerfWaitIters = 1L << 24;

__device__ __forceinline__ float h2f(__half h) { return __half2float(h); }

// W [n_out][n_in] float16 at params + off -> rows n < n_out_pad, k < K of
// the operand tile (zero padding)
__device__ void stage_weights(uint8_t *dst, const __half *params, int off, int n_in, int n_out, int n_rows, int K) {
  for (int i = threadIdx.x; i < n_rows * K; i += blockDim.x) {
    const int n = i / K, k = i % K;
    const __half v = (n < n_out && k < n_in) ? params[off + n * n_in + k] : __float2half(0.0f);
    *reinterpret_cast<__half *>(dst + tc::kmaj_offset(n, k, K)) = v;
  }
}

__device__ void stage_bias(float *dst, const __half *params, int off, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = h2f(params[off + i]);
}

// 16 float values -> float16, stored to row `row`, columns [k0, k0 + 16) of
// a K-major operand tile with K columns (two 16-byte stores)
__device__ __forceinline__ void store_row16(uint8_t *tile, int row, int k0, int K, const float v[16]) {
#pragma unroll
  for (int c = 0; c < 2; c++) {
    __align__(16) __half hv[8];
#pragma unroll
    for (int j = 0; j < 8; j++) hv[j] = __float2half_rn(v[c * 8 + j]);
    *reinterpret_cast<uint4 *>(tile + tc::kmaj_offset(row, k0 + c * 8, K)) = *reinterpret_cast<uint4 *>(hv);
  }
}

__device__ __forceinline__ float relu_f16(float x) {
  // the reference's relu: max(float(half), 0) back to half (NaN -> 0)
  return h2f(__float2half_rn(fmaxf(h2f(__float2half_rn(x)), 0.0f)));
}

struct NerfParams {
  const __half *params;
  const float *z, *tpsdf, *geo;
  int B, N, V;
  float *density, *geo_out;
  int *error;
};

// issue one M=128 layer: D[tmem + dcol] = A[a] * W^T, K columns in steps of 16
__device__ __forceinline__ void issue_layer(uint32_t tmem, int dcol, const uint8_t *a, const uint8_t *w, int K,
                                            int N) {
  const uint32_t ia = tc::smem_addr(a), iw = tc::smem_addr(w);
  const uint32_t idesc = tc::idesc_f16_f32(128, N);
  for (int kk = 0; kk < K / 16; kk++) {
    const uint64_t da = tc::smem_desc(ia + kk * 256, 128, K * 16);
    const uint64_t dw = tc::smem_desc(iw + kk * 256, 128, K * 16);
    tc::mma_f16(tmem + dcol, da, dw, idesc, kk > 0 ? 1u : 0u);
  }
}

__global__ void __launch_bounds__(kNerfThreads) nerf_density_kernel(NerfParams p) {
  extern __shared__ uint8_t smem_raw[];
  NerfSmem &sm = *reinterpret_cast<NerfSmem *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5;
  const __half *P = p.params;
  // weights and biases, once per CTA
  stage_weights(sm.w1, P, 0, 18, 64, 64, 32);
  stage_weights(sm.w2, P, 1216, 64, 64, 64, 64);
  stage_weights(sm.w3, P, 5376, 64, 64, 64, 64);
  stage_weights(sm.w4, P, 9536, 64, 64, 64, 64);
  stage_weights(sm.ws1, P, kSigmaOff, 64, 64, 64, 64);
  stage_weights(sm.ws2, P, kSigmaOff + 4160, 64, 64, 64, 64);
  stage_weights(sm.wg1, P, kGeoOff, 18, 16, 16, 32);
  stage_weights(sm.wg2, P, kGeoOff + 304, 16, 8, 16, 16);
  stage_bias(sm.b1, P, 1152, 64);
  stage_bias(sm.b2, P, 5312, 64);
  stage_bias(sm.b3, P, 9472, 64);
  stage_bias(sm.b4, P, 13632, 64);
  stage_bias(sm.bs1, P, kSigmaOff + 4096, 64);
  stage_bias(sm.bs2, P, kSigmaOff + 8256, 64);
  stage_bias(sm.ws3, P, kSigmaOff + 8320, 64);
  stage_bias(sm.bg1, P, kGeoOff + 288, 16);
  stage_bias(sm.bg2, P, kGeoOff + 432, 8);
  if (tid == 0) {
    sm.bs3 = h2f(P[kSigmaOff + 8384]);
    tc::mbar_init(tc::smem_addr(&sm.mbar), 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&sm.tmem_slot), kNerfTmemCols);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.tmem_slot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's lane quadrant
  const uint32_t mbar = tc::smem_addr(&sm.mbar);
  const int V = p.V, Pt = kNerfThreads / V;
  const long n_points = (long)p.B * p.N;
  const long n_tiles = (n_points + Pt - 1) / Pt;
  const int r = tid;  // this thread's row
  const int rv = r / Pt, rp = r % Pt;
  uint32_t phase = 0;
  bool failed = false;

  auto layer_done = [&]() -> bool {
    bool ok = tc::mbar_wait(mbar, phase, kNerfWaitIters);
    phase ^= 1u;
    tc::fence_after_sync();
    return __syncthreads_and(ok);
  };
  auto operands_ready = [&]() {
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
  };

  for (long tile = blockIdx.x; tile < n_tiles && !failed; tile += gridDim.x) {
    // ---- inputs: row r = (view rv, point rp) ------------------------------
    const long g = tile * Pt + rp;
    const bool row_ok = rv < V && g < n_points;
    long pv = 0;
    {
      float x[32];
#pragma unroll
      for (int j = 0; j < 32; j++) x[j] = 0.0f;
      if (row_ok) {
        const long b = g / p.N, n = g - b * p.N;
        pv = (b * V + rv) * p.N + n;
        x[0] = p.z[pv];
        x[1] = p.tpsdf[pv];
        const float4 *gf = reinterpret_cast<const float4 *>(p.geo + pv * 16);
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const float4 f = __ldg(gf + q);
          x[2 + 4 * q] = f.x;
          x[3 + 4 * q] = f.y;
          x[4 + 4 * q] = f.z;
          x[5 + 4 * q] = f.w;
        }
      }
      store_row16(sm.a_in, r, 0, 32, x);
      store_row16(sm.a_in, r, 16, 32, x + 16);
    }
    operands_ready();
    if (tid == 0) {
      tc::fence_after_sync();
      issue_layer(tmem, 0, sm.a_in, sm.w1, 32, 64);
      issue_layer(tmem, 64, sm.a_in, sm.wg1, 32, 16);
      tc::commit(mbar);
    }
    if (!layer_done()) { failed = true; break; }
    // ---- layer 1 epilogue (features -> h, geometry hidden -> a_in) -------
    {
      float v[16];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        tc::tmem_ld16(trow + c * 16, v);
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = relu_f16(v[j] + sm.b1[c * 16 + j]);
        store_row16(sm.h, r, c * 16, 64, v);
      }
      tc::tmem_ld16(trow + 64, v);
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = relu_f16(v[j] + sm.bg1[j]);
      store_row16(sm.a_in, r, 0, 16, v);
    }
    operands_ready();
    if (tid == 0) {
      tc::fence_after_sync();
      issue_layer(tmem, 0, sm.h, sm.w2, 64, 64);
      issue_layer(tmem, 64, sm.a_in, sm.wg2, 16, 16);
      tc::commit(mbar);
    }
    if (!layer_done()) { failed = true; break; }
    // ---- layer 2 epilogue; geometry output ---------------------------------
    {
      float v[16];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        tc::tmem_ld16(trow + c * 16, v);
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = relu_f16(v[j] + sm.b2[c * 16 + j]);
        store_row16(sm.h, r, c * 16, 64, v);
      }
      tc::tmem_ld16(trow + 64, v);
      if (row_ok && p.geo_out) {
        float4 *go = reinterpret_cast<float4 *>(p.geo_out + pv * 8);
        float o[8];
#pragma unroll
        for (int j = 0; j < 8; j++) o[j] = relu_f16(v[j] + sm.bg2[j]);
        go[0] = make_float4(o[0], o[1], o[2], o[3]);
        go[1] = make_float4(o[4], o[5], o[6], o[7]);
      }
    }
    // ---- layers 3 and 4 ------------------------------------------------------
#pragma unroll 1
    for (int L = 3; L <= 4; L++) {
      operands_ready();
      if (tid == 0) {
        tc::fence_after_sync();
        issue_layer(tmem, 0, sm.h, L == 3 ? sm.w3 : sm.w4, 64, 64);
        tc::commit(mbar);
      }
      if (!layer_done()) { failed = true; break; }
      const float *bias = L == 3 ? sm.b3 : sm.b4;
      float v[16];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        tc::tmem_ld16(trow + c * 16, v);
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = relu_f16(v[j] + bias[c * 16 + j]);
        store_row16(sm.h, r, c * 16, 64, v);
      }
    }
    if (failed) break;
    __syncthreads();
    // ---- view mean: rows rp < Pt take the mean of rows v * Pt + rp ---------
    if (r < Pt) {
      float m[64];
#pragma unroll
      for (int c = 0; c < 64; c++) m[c] = 0.0f;
      for (int v = 0; v < V; v++) {
        const int src = v * Pt + r;
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++) {
          const uint4 q = *reinterpret_cast<const uint4 *>(sm.h + tc::kmaj_offset(src, c8 * 8, 64));
          const __half *hq = reinterpret_cast<const __half *>(&q);
#pragma unroll
          for (int j = 0; j < 8; j++) m[c8 * 8 + j] += h2f(hq[j]);
        }
      }
      const float inv = 1.0f / (float)V;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = m[c * 16 + j] * inv;
        store_row16(sm.h, r, c * 16, 64, v);
      }
    }
    // ---- sigma layers ----------------------------------------------------------
#pragma unroll 1
    for (int L = 1; L <= 2; L++) {
      operands_ready();
      if (tid == 0) {
        tc::fence_after_sync();
        issue_layer(tmem, 0, sm.h, L == 1 ? sm.ws1 : sm.ws2, 64, 64);
        tc::commit(mbar);
      }
      if (!layer_done()) { failed = true; break; }
      const float *bias = L == 1 ? sm.bs1 : sm.bs2;
      float v[16];
      if (L == 1) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
          tc::tmem_ld16(trow + c * 16, v);
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = relu_f16(v[j] + bias[c * 16 + j]);
          store_row16(sm.h, r, c * 16, 64, v);
        }
      } else {
        float acc = 0.0f;
#pragma unroll
        for (int c = 0; c < 4; c++) {
          tc::tmem_ld16(trow + c * 16, v);
#pragma unroll
          for (int j = 0; j < 16; j++) acc = __fmaf_rn(relu_f16(v[j] + bias[c * 16 + j]), sm.ws3[c * 16 + j], acc);
        }
        const long gp = tile * Pt + r;
        if (r < Pt && gp < n_points) {
          const float pre = h2f(__float2half_rn(acc + sm.bs3));
          p.density[gp] = h2f(__float2half_rn(1.0f / (1.0f + expf(-pre))));
        }
      }
    }
    if (failed) break;
  }
  if (failed && tid == 0 && p.error) atomicExch(p.error, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kNerfTmemCols);
  }
}

}  // namespace sg

using namespace sg;

extern "C" size_t sg_nerf_param_count(void) { return kNerfParamCount; }

extern "C" int sg_nerf_density(const uint16_t *params, const float *points_z, const float *points_tpsdf,
                               const float *feats_geo, int B, int N, int V, float *density, float *geo_feats,
                               int *error, sg_stream_t stream) {
  if (!params || !points_z || !points_tpsdf || !feats_geo || !density) return SG_ERR_INVALID_ARG;
  if (B <= 0 || N <= 0 || V <= 0 || V > kNerfThreads) return SG_ERR_INVALID_ARG;
  if ((((uintptr_t)feats_geo) % 16) != 0 || (geo_feats && ((uintptr_t)geo_feats) % 16 != 0))
    return SG_ERR_INVALID_ARG;
  const size_t smem = sizeof(NerfSmem) + 1024;
  static bool attr_set = false;  // the attribute is per function, any device
  if (!attr_set) {
    if (cudaFuncSetAttribute(nerf_density_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return SG_ERR_CUDA;
    attr_set = true;
  }
  const long n_points = (long)B * N;
  const int Pt = kNerfThreads / V;
  const long n_tiles = (n_points + Pt - 1) / Pt;
  // at most 3 CTAs fit an SM (shared memory), 3 x 128 tensor-memory columns
  long grid = (long)num_sms() * 3;
  if (grid > n_tiles) grid = n_tiles;
  NerfParams p{reinterpret_cast<const __half *>(params), points_z, points_tpsdf, feats_geo, B, N, V, density,
               geo_feats, error};
  nerf_density_kernel<<<(int)grid, kNerfThreads, smem, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
