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
// 256 threads (two warpgroups) takes two tiles at a time; a tile is 128 rows,
// P = floor(128 / V) points x V views (row v*P + p), so the view mean happens
// inside the CTA and no per-view feature reaches HBM:
//   inputs (z, t_psdf, 16 geometry features) -> float16 rows in shared memory
//   (the next tiles' inputs are loaded into registers while the current ones
//   run through the layers);
//   each layer: one thread of the tile's warpgroup issues tcgen05.mma (K-major
//   float16 operands in shared memory, the weights staged once per CTA) into
//   tensor memory and commits to the warpgroup's mbarrier; the warpgroup then
//   reads its tile's rows back (tcgen05.ld, one row per thread), adds the bias in
//   float32, applies ReLU and rounds to float16 into the next operand tile;
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

constexpr int kNerfTiles = 2;                    // tiles in flight per CTA, one warpgroup each
constexpr int kNerfThreads = 128 * kNerfTiles;
constexpr uint32_t kNerfTmemCols = 128 * kNerfTiles;  // tile t: features 128t+[0,64), geometry 128t+[64,80)
constexpr long kNerfWaitIters = 1L << 24;

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
  alignas(128) uint8_t a_in[kNerfTiles][128 * 32 * 2];  // layer-1 rows; then the geometry hidden rows (K = 16)
  alignas(128) uint8_t h[kNerfTiles][128 * 64 * 2];     // hidden rows; then the view means
  float b1[64], b2[64], b3[64], b4[64], bs1[64], bs2[64], ws3[64], bg1[16], bg2[8];
  float bs3;
  alignas(8) uint64_t mbar[kNerfTiles];  // one per warpgroup
  int fail[kNerfTiles];
  uint32_t tmem_slot;
};

// barrier of one warpgroup (named barrier 1 + t, 128 threads; immediate ids)
__device__ __forceinline__ void wg_sync(int t) {
  if (t == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
  else asm volatile("bar.sync 2, 128;" ::: "memory");
}

__device__ __forceinline__ float h2f(__half h) { return __half2float(h); }

// W [n_out][n_in] float16 at params + off -> rows n < n_rows, k < K of the
// operand tile (zero padding)
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

__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);  // one cvt.rn.f16x2.f32
  return *reinterpret_cast<const uint32_t *>(&h);
}

// 16 float values -> float16, stored to row `row`, columns [k0, k0 + 16) of
// a K-major operand tile with K columns (two 16-byte stores)
__device__ __forceinline__ void store_row16(uint8_t *tile, int row, int k0, int K, const float *v) {
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const uint4 q = make_uint4(pack_half2(v[c * 8], v[c * 8 + 1]), pack_half2(v[c * 8 + 2], v[c * 8 + 3]),
                               pack_half2(v[c * 8 + 4], v[c * 8 + 5]), pack_half2(v[c * 8 + 6], v[c * 8 + 7]));
    *reinterpret_cast<uint4 *>(tile + tc::kmaj_offset(row, k0 + c * 8, K)) = q;
  }
}

// The reference's relu of a float16 value: max(float(half), 0) back to half
// (NaN -> 0).  Rounding is monotone and keeps 0, so ReLU before the rounding
// to float16 gives the same value: the callers round max(x, 0).
__device__ __forceinline__ float relu_f32(float x) { return fmaxf(x, 0.0f); }
__device__ __forceinline__ float relu_f16(float x) { return h2f(__float2half_rn(fmaxf(x, 0.0f))); }

// 64 accumulator columns of this thread's row -> bias, ReLU, float16 -> row
__device__ __forceinline__ void epilogue64(uint32_t taddr, const float *bias, uint8_t *tile, int row) {
#pragma unroll
  for (int half = 0; half < 2; half++) {
    float v[32];
    tc::tmem_ld32(taddr + 32 * half, v);
#pragma unroll
    for (int j = 0; j < 32; j++) v[j] = relu_f32(v[j] + bias[32 * half + j]);
    store_row16(tile, row, 32 * half, 64, v);
    store_row16(tile, row, 32 * half + 16, 64, v + 16);
  }
}

struct NerfParams {
  const __half *params;
  const float *z, *tpsdf, *geo;
  int B, N, V;
  float *density, *geo_out;
  int *error;
};

// one row's inputs (z, t_psdf, 16 geometry features), loaded ahead
struct NerfRow {
  float x[18];
  long pv;
  bool ok;
};

__device__ __forceinline__ void load_row(const NerfParams &p, long tile, int rv, int rp, int Pt, long n_points,
                                         NerfRow &row) {
  const long g = tile * Pt + rp;
  row.ok = rv < p.V && g < n_points;
  row.pv = 0;
#pragma unroll
  for (int j = 0; j < 18; j++) row.x[j] = 0.0f;
  if (row.ok) {
    const long b = g / p.N, n = g - b * p.N;
    row.pv = (b * p.V + rv) * p.N + n;
    row.x[0] = __ldg(p.z + row.pv);
    row.x[1] = __ldg(p.tpsdf + row.pv);
    const float4 *gf = reinterpret_cast<const float4 *>(p.geo + row.pv * 16);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float4 f = __ldg(gf + q);
      row.x[2 + 4 * q] = f.x;
      row.x[3 + 4 * q] = f.y;
      row.x[4 + 4 * q] = f.z;
      row.x[5 + 4 * q] = f.w;
    }
  }
}

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

__global__ void __launch_bounds__(kNerfThreads, 2) nerf_density_kernel(NerfParams p) {
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
    for (int q = 0; q < kNerfTiles; q++) {
      tc::mbar_init(tc::smem_addr(&sm.mbar[q]), 1);
      sm.fail[q] = 0;
    }
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&sm.tmem_slot), kNerfTmemCols);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.tmem_slot;
  const int t = tid >> 7;   // this thread's tile (warpgroup)
  const int r = tid & 127;  // its row
  // warp (tid >> 5) may read tensor-memory lanes 32 * (warp % 4) ..: its rows
  const uint32_t trow = tmem + ((uint32_t)(r & ~31) << 16) + 128u * t;
  const uint32_t mbar = tc::smem_addr(&sm.mbar[t]);
  const int V = p.V, Pt = 128 / V;
  const long n_points = (long)p.B * p.N;
  const long n_tiles = (n_points + Pt - 1) / Pt;
  const long n_pairs = (n_tiles + kNerfTiles - 1) / kNerfTiles;
  const int rv = r / Pt, rp = r % Pt;
  uint8_t *a_in = sm.a_in[t];
  uint8_t *hh = sm.h[t];
  uint32_t phase = 0;
  bool failed = false;

  // The two warpgroups run their tiles independently (own mbarrier, own
  // issuing thread, own named barrier), so one's MMAs overlap the other's
  // epilogue.
  const bool issuer = r == 0;
  auto layer_done = [&]() -> bool {
    const bool ok = tc::mbar_wait(mbar, phase, kNerfWaitIters);
    phase ^= 1u;
    if (!ok) sm.fail[t] = 1;
    tc::fence_after_sync();
    wg_sync(t);
    return *reinterpret_cast<volatile int *>(&sm.fail[t]) == 0;
  };
  auto operands_ready = [&]() {
    tc::fence_async_smem();
    tc::fence_before_sync();
    wg_sync(t);
  };

  NerfRow cur;
  long pair = blockIdx.x;
  if (pair < n_pairs) load_row(p, pair * kNerfTiles + t, rv, rp, Pt, n_points, cur);
  for (; pair < n_pairs && !failed; pair += gridDim.x) {
    const long tile = pair * kNerfTiles + t;
    {
      float x[32];
#pragma unroll
      for (int j = 0; j < 18; j++) x[j] = cur.x[j];
#pragma unroll
      for (int j = 18; j < 32; j++) x[j] = 0.0f;
      store_row16(a_in, r, 0, 32, x);
      store_row16(a_in, r, 16, 32, x + 16);
    }
    const bool row_ok = cur.ok;
    const long pv = cur.pv;
    // the next pair's inputs: loads in flight while this pair runs
    if (pair + gridDim.x < n_pairs) load_row(p, (pair + gridDim.x) * kNerfTiles + t, rv, rp, Pt, n_points, cur);
    operands_ready();
    if (issuer) {
      tc::fence_after_sync();
      issue_layer(tmem + 128u * t, 0, a_in, sm.w1, 32, 64);
      issue_layer(tmem + 128u * t, 64, a_in, sm.wg1, 32, 16);
      tc::commit(mbar);
    }
    if (!layer_done()) { failed = true; break; }
    // ---- layer 1 epilogue (features -> h, geometry hidden -> a_in) -------
    epilogue64(trow, sm.b1, hh, r);
    {
      float v[16];
      tc::tmem_ld16(trow + 64, v);
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = relu_f32(v[j] + sm.bg1[j]);
      store_row16(a_in, r, 0, 16, v);
    }
    operands_ready();
    if (issuer) {
      tc::fence_after_sync();
      issue_layer(tmem + 128u * t, 0, hh, sm.w2, 64, 64);
      issue_layer(tmem + 128u * t, 64, a_in, sm.wg2, 16, 16);
      tc::commit(mbar);
    }
    if (!layer_done()) { failed = true; break; }
    // ---- layer 2 epilogue; geometry output ---------------------------------
    epilogue64(trow, sm.b2, hh, r);
    {
      float v[16];
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
      if (issuer) {
        tc::fence_after_sync();
        issue_layer(tmem + 128u * t, 0, hh, L == 3 ? sm.w3 : sm.w4, 64, 64);
        tc::commit(mbar);
      }
      if (!layer_done()) { failed = true; break; }
      epilogue64(trow, L == 3 ? sm.b3 : sm.b4, hh, r);
    }
    if (failed) break;
    wg_sync(t);
    // ---- view mean: rows rp < Pt take the mean of rows v * Pt + rp ---------
    if (r < Pt) {
      const float inv = 1.0f / (float)V;
      // two halves of 32 channels (row r is read for a half before it is written)
#pragma unroll
      for (int half = 0; half < 2; half++) {
        float m[32];
#pragma unroll
        for (int c = 0; c < 32; c++) m[c] = 0.0f;
        for (int v = 0; v < V; v++) {
          const int src = v * Pt + r;
#pragma unroll
          for (int c8 = 0; c8 < 4; c8++) {
            const uint4 q = *reinterpret_cast<const uint4 *>(hh + tc::kmaj_offset(src, 32 * half + c8 * 8, 64));
            const __half2 *hq = reinterpret_cast<const __half2 *>(&q);
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const float2 f = __half22float2(hq[j]);
              m[c8 * 8 + 2 * j] += f.x;
              m[c8 * 8 + 2 * j + 1] += f.y;
            }
          }
        }
#pragma unroll
        for (int c = 0; c < 32; c++) m[c] *= inv;
        store_row16(hh, r, 32 * half, 64, m);
        store_row16(hh, r, 32 * half + 16, 64, m + 16);
      }
    }
    // ---- sigma layers ----------------------------------------------------------
    operands_ready();
    if (issuer) {
      tc::fence_after_sync();
      issue_layer(tmem + 128u * t, 0, hh, sm.ws1, 64, 64);
      tc::commit(mbar);
    }
    if (!layer_done()) { failed = true; break; }
    epilogue64(trow, sm.bs1, hh, r);
    operands_ready();
    if (issuer) {
      tc::fence_after_sync();
      issue_layer(tmem + 128u * t, 0, hh, sm.ws2, 64, 64);
      tc::commit(mbar);
    }
    if (!layer_done()) { failed = true; break; }
    {
      float acc = 0.0f;
#pragma unroll
      for (int half = 0; half < 2; half++) {
        float v[32];
        tc::tmem_ld32(trow + 32 * half, v);
#pragma unroll
        for (int j = 0; j < 32; j++) acc = __fmaf_rn(relu_f16(v[j] + sm.bs2[32 * half + j]), sm.ws3[32 * half + j], acc);
      }
      const long gp = tile * Pt + r;
      if (r < Pt && gp < n_points) {
        const float pre = h2f(__float2half_rn(acc + sm.bs3));
        p.density[gp] = h2f(__float2half_rn(1.0f / (1.0f + expf(-pre))));
      }
    }
  }
  if (failed && issuer && p.error) atomicExch(p.error, 1);
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
  if (B <= 0 || N <= 0 || V <= 0 || V > 128) return SG_ERR_INVALID_ARG;
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
  const int Pt = 128 / V;
  const long n_pairs = ((n_points + Pt - 1) / Pt + kNerfTiles - 1) / kNerfTiles;
  // at most 2 CTAs fit an SM (shared memory): 2 x 256 tensor-memory columns
  long grid = (long)num_sms() * 2;
  if (grid > n_pairs) grid = n_pairs;
  NerfParams p{reinterpret_cast<const __half *>(params), points_z, points_tpsdf, feats_geo, B, N, V, density,
               geo_feats, error};
  nerf_density_kernel<<<(int)grid, kNerfThreads, smem, stream>>>(p);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
