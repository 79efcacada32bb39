// rays.cu -- per-pixel camera rays on sm_103a.
//
// Replaces rays_calculating (SAILOR c_lib/VoxelEncoding/src/
// sampling_kernel.cu:674-731: two inverse_mat3x3 launches and
// rays_calculating_kernel :411-486, writing a [B, N, H, W, 6] tensor).
//
// camera_params_kernel: one thread per camera -> the 21-float camera table
// (K^-1, R^-1, centre) that the batched intersection and render also read
// to generate the rays of camera-defined segments on the fly.
// rays_kernel: a CTA of 256 pixels of one camera; the camera's table entry
// is formed once per CTA in shared memory; three float2 stores per pixel.
#include "common.cuh"

namespace sg {

__global__ void camera_params_kernel(const float *__restrict__ K, const float *__restrict__ R,
                                     const float *__restrict__ T, int n, float *cams) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float m[9], r[9], t[3], cam[kCamFloats];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    m[k] = K[(size_t)i * 9 + k];
    r[k] = R[(size_t)i * 9 + k];
  }
#pragma unroll
  for (int k = 0; k < 3; k++) t[k] = T[(size_t)i * 3 + k];
  camera_params(m, r, t, cam);
#pragma unroll
  for (int k = 0; k < kCamFloats; k++) cams[(size_t)i * kCamFloats + k] = cam[k];
}

__global__ void __launch_bounds__(256) rays_kernel(const float *__restrict__ K, const float *__restrict__ R,
                                                   const float *__restrict__ T, int H, int W, float *out) {
  __shared__ float s_cam[kCamFloats];
  const int v = blockIdx.y;
  if (threadIdx.x == 0) {
    float m[9], r[9], t[3];
    for (int k = 0; k < 9; k++) {
      m[k] = K[(size_t)v * 9 + k];
      r[k] = R[(size_t)v * 9 + k];
    }
    for (int k = 0; k < 3; k++) t[k] = T[(size_t)v * 3 + k];
    camera_params(m, r, t, s_cam);
  }
  __syncthreads();
  const long npx = (long)H * W;
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npx) return;
  const int h = (int)(p / W), w = (int)(p - (long)h * W);
  float o[3], d[3];
  pixel_ray<false>(s_cam, h, w, o, d);
  float2 *q = reinterpret_cast<float2 *>(out + ((size_t)v * npx + p) * 6);
  q[0] = make_float2(o[0], o[1]);
  q[1] = make_float2(o[2], d[0]);
  q[2] = make_float2(d[1], d[2]);
}

__global__ void segment_rays_kernel(int nseg, const int *__restrict__ begin, const float *__restrict__ cams,
                                    const int *__restrict__ widths, long R, float *ori, float *dir) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int s = segment_of(begin, nseg, r);
  float o[3], d[3];
  segment_ray(nullptr, nullptr, cams, widths, begin, s, r, o, d);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ori[r * 3 + k] = o[k];
    dir[r * 3 + k] = d[k];
  }
}

}  // namespace sg

using namespace sg;

extern "C" int sg_camera_params(const float *K, const float *R, const float *T, int n, float *cams,
                                sg_stream_t stream) {
  if (!K || !R || !T || !cams || n < 0) return SG_ERR_INVALID_ARG;
  if (n == 0) return SG_OK;
  camera_params_kernel<<<ceil_div(n, 128), 128, 0, stream>>>(K, R, T, n, cams);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_rays_from_cameras(const float *K, const float *R, const float *T, int B, int N, int H, int W,
                                    float *out, sg_stream_t stream) {
  if (!K || !R || !T || !out || B <= 0 || N <= 0 || H <= 0 || W <= 0) return SG_ERR_INVALID_ARG;
  if (((uintptr_t)out) % 8 != 0) return SG_ERR_INVALID_ARG;
  if ((long)B * N > 65535) return SG_ERR_UNSUPPORTED;
  const long npx = (long)H * W;
  rays_kernel<<<dim3(ceil_div(npx, 256), B * N), 256, 0, stream>>>(K, R, T, H, W, out);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_segment_rays(const SgRaySegments *seg, float *ori, float *dir, sg_stream_t stream) {
  if (!seg || !ori || !dir || !seg->ray_begin || !seg->cameras || !seg->widths || seg->count <= 0 || seg->total < 0)
    return SG_ERR_INVALID_ARG;
  if (seg->total == 0) return SG_OK;
  segment_rays_kernel<<<ceil_div((long)seg->total, 256), 256, 0, stream>>>(seg->count, seg->ray_begin, seg->cameras,
                                                                          seg->widths, (long)seg->total, ori, dir);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
