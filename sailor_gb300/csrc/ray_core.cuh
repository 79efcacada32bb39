// ray_core.cuh -- per-ray building blocks shared by the sampling, compositing
// and fused render kernels (one warp per ray, lane l owns positions l, l+32..).
#pragma once

#include <type_traits>

#include "common.cuh"

namespace sg {

// ---------------------------------------------------------------------------
// sampling (ray_voxels_sampling_uniform_kernel, sampling_kernel.cu:1070-1177)
// ---------------------------------------------------------------------------
struct SampleParams {
  SgTree t;
  const int *hit_idx;
  const float *hit_t0, *hit_t1, *rands, *valid_len;
  int N, W, S, num_levels, start_level;
  int *sampled_idx;
  float *sampled_z;
  unsigned long long seed;  // rands == NULL and seed != 0: hashed jitter
};

// Warp-private shared scratch of the sampler.
struct SampleScratch {
  int start[32];
  float mn[32], off[32];
  int id[32];
};

// depth of the j-th sample (0-based) of a hit with n samples:
// base = min + off*(j+1); z = base - off/2 + off*rand   (sampling_kernel.cu:1142-1148)
__device__ __forceinline__ float sample_z(float mn, float off, int j, float rnd) {
  float base = __fmaf_rn(off, (float)(j + 1), mn);
  return sum3_rn(base, -(off * 0.5f), off * rnd);
}

// Samples of ray r into shared sz/si[0, S) in the reference's output order,
// -1 where there is none.  The hit row holds nh entries (compact rows) or is
// -1 terminated (nh = W).  Per chunk of 32 hits, lanes compute the hits'
// sample counts exactly as the reference's serial loop, a warp scan turns
// the serial "samples left" capping into output ranges, and the chunk's
// samples are generated position-parallel: the owner of position q is the
// last hit whose range starts at or before q (starts are non-decreasing and
// strictly increasing over hits that get samples).  Returns #samples.
// b: the ray's frame; S: its sample count (<= p.S, the row stride of rands).
__device__ __forceinline__ int warp_sample_ray(const SampleParams &p, long r, int b, int S, int nh,
                                               float rand_const, float *sz, int *si, SampleScratch &sc) {
  const int lane = lane_id();
  const int *hi = p.hit_idx + (size_t)r * p.W;
  const float *h0 = p.hit_t0 + (size_t)r * p.W, *h1 = p.hit_t1 + (size_t)r * p.W;
  const float *rd = p.rands ? p.rands + (size_t)r * p.S : nullptr;
  const unsigned long long seed = p.seed;
  auto jitter = [&](int q) {
    return rd ? __ldg(rd + q) : (seed ? hash_uniform(seed, r, q) : rand_const);
  };
  int done = 0;
  if (nh > 0 && __ldg(hi) >= 0) {
    const float vl = p.valid_len[r];
    const float vs = p.t.voxel_size[b];
    const float start_vs = vs * ldexpf(1.0f, 2 * (p.num_levels - p.start_level - 1));
    const float vs_top = vs * (float)(p.t.Db / p.t.Dt);
    int has = 0, nvalid = 0;
    bool stop = false;
    for (int c0 = 0; c0 < nh && !stop && has < S; c0 += 32) {
      const int i = c0 + lane;
      int id = -1;
      float mn = -1.0f, mx = -1.0f;
      if (i < nh) {
        id = __ldg(hi + i);
        mn = __ldg(h0 + i);
        mx = __ldg(h1 + i);
      }
      bool ok = i < nh && !(id < 0 || mn < 0 || mx < 0);
      const unsigned bad = __ballot_sync(SG_FULL, !ok);
      const int first_bad = bad ? __ffs(bad) - 1 : 32;
      ok = ok && lane < first_bad;
      if (bad) stop = true;
      int n = 0;
      if (ok) {
        const float nvs = (id >= p.t.base_top) ? vs_top : vs;
        const float rate = start_vs / nvs;
        n = (int)((mx - mn) * rate * (float)S / vl);
        n = n >= 1 ? n : 1;
        n = n < S ? n : S;
      }
      const int incl = warp_incl_scan(n);
      const int start = has + incl - n;
      int ne = S - start;
      ne = ne < 0 ? 0 : (ne < n ? ne : n);
      sc.start[lane] = start;
      sc.mn[lane] = mn;
      sc.off[lane] = (mx - mn) / (float)(ne + 1);
      sc.id[lane] = id;
      __syncwarp();
      const int end = min(has + __shfl_sync(SG_FULL, incl, 31), S);
      // owners are among the lanes with samples; lanes past the last of
      // them start at or after end, so the search stops there
      const unsigned with_n = __ballot_sync(SG_FULL, n > 0);
      const int last = with_n ? 31 - __clz(with_n) : 0;
      for (int q = has + lane; q < end; q += 32) {
        int lo = 0, up = last;
        while (lo < up) {
          const int mid = (lo + up + 1) >> 1;
          if (sc.start[mid] <= q) lo = mid;
          else up = mid - 1;
        }
        sz[q] = sample_z(sc.mn[lo], sc.off[lo], q - sc.start[lo], jitter(q));
        si[q] = sc.id[lo];
      }
      __syncwarp();
      has = end;
      nvalid += __popc(__ballot_sync(SG_FULL, ok));
    }
    // leftover: one more sample in each of the first hits (:1156-1174)
    const int left = S - has;
    const int cnt = left < nvalid ? left : nvalid;
    for (int i = lane; i < cnt; i += 32) {
      const int id = __ldg(hi + i);
      const float mn = __ldg(h0 + i), mx = __ldg(h1 + i);
      const float off = (mx - mn) * 0.5f;
      const float base = mn + off;
      const int q = has + i;
      sz[q] = sum3_rn(base, -(off * 0.5f), off * jitter(q));
      si[q] = id;
    }
    done = has + cnt;
  }
  for (int q = done + lane; q < S; q += 32) {
    sz[q] = -1.0f;
    si[q] = -1;
  }
  __syncwarp();
  return done;
}

// ---------------------------------------------------------------------------
// per-ray sort: register bitonic network on 32-bit depth keys; input
// positions, where read, by ranking (warp_sort_ranked)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ordered_bits(float f) {
  uint32_t u = __float_as_uint(f);
  return u ^ ((u >> 31) ? 0xffffffffu : 0x80000000u);
}
__device__ __forceinline__ float from_ordered(uint32_t k) {
  return __uint_as_float((k >> 31) ? (k ^ 0x80000000u) : ~k);
}

// E keys per lane in blocked order, element i = lane*E + e, P = 32*E (a
// power of two); K is an unsigned key type (here the 32-bit ordered depth).
// Partner distances below E stay in the lane, so of the network's
// log2(P)(log2(P)+1)/2 steps only those with distance >= E exchange across
// lanes (15 of 28 at E = 4).
template <int E, typename K>
__device__ __forceinline__ void bitonic_warp(K (&key)[E]) {
  const int lane = lane_id();
  constexpr int P = 32 * E;
#pragma unroll
  for (int k = 2; k <= P; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j < E) {
#pragma unroll
        for (int e = 0; e < E; e++) {
          if ((e & j) == 0) {
            const bool asc = ((lane * E + e) & k) == 0;
            const K a = key[e], c = key[e + j];
            const bool sw = asc ? (a > c) : (a < c);
            key[e] = sw ? c : a;
            key[e + j] = sw ? a : c;
          }
        }
      } else {
        const int m = j / E;  // partner lane distance
        const bool lower = (lane & m) == 0;
#pragma unroll
        for (int e = 0; e < E; e++) {
          const bool asc = ((lane * E + e) & k) == 0;
          const K other = __shfl_xor_sync(SG_FULL, key[e], m);
          const K mn = key[e] < other ? key[e] : other;
          const K mx = key[e] < other ? other : key[e];
          key[e] = (lower == asc) ? mn : mx;
        }
      }
    }
  }
}

// E consecutive floats from a 4E-byte aligned address (E = 1, 2, 4, 8)
template <int E>
__device__ __forceinline__ void load_run(const float *src, float (&v)[E]) {
  if constexpr (E == 1) {
    v[0] = src[0];
  } else if constexpr (E == 2) {
    const float2 a = *reinterpret_cast<const float2 *>(src);
    v[0] = a.x;
    v[1] = a.y;
  } else {
#pragma unroll
    for (int q = 0; q < E; q += 4) {
      const float4 a = *reinterpret_cast<const float4 *>(src + q);
      v[q] = a.x;
      v[q + 1] = a.y;
      v[q + 2] = a.z;
      v[q + 3] = a.w;
    }
  }
}

// E consecutive 32-bit words to a 4E-byte aligned address (E = 1, 2, 4, 8)
template <int E>
__device__ __forceinline__ void store_run(uint32_t *dst, const uint32_t (&v)[E]) {
  if constexpr (E == 1) {
    dst[0] = v[0];
  } else if constexpr (E == 2) {
    *reinterpret_cast<uint2 *>(dst) = make_uint2(v[0], v[1]);
  } else {
#pragma unroll
    for (int q = 0; q < E; q += 4) *reinterpret_cast<uint4 *>(dst + q) = make_uint4(v[q], v[q + 1], v[q + 2], v[q + 3]);
  }
}

// Stable warp sort of n <= 32E values with their input positions, on 32-bit
// keys.  The (depth, position) order needs 64-bit compare-exchanges, and the
// network is bound by the integer pipe; here the network sorts the depth
// keys alone, and each input element finds its place afterwards: a binary
// search gives the number of smaller keys, and elements of equal keys (rare
// but for padding) count the equal ones before them in input order, slot
// by slot with __match_any_sync.
//   buf: shared, 16-byte aligned, 32E words; on entry buf[0, n) the values
//        in input order (overwritten: the sorted keys).
//   cnt: shared scratch of n ints.
//   key: on return the sorted keys, blocked (element j = lane*E + e; ~0u
//        past n).  pos: the sorted position of input element e*32 + lane.
template <int E>
__device__ __forceinline__ void warp_sort_ranked(float *buf, int *cnt, int n, uint32_t (&key)[E], int (&pos)[E]) {
  const int lane = lane_id();
  uint32_t *u = reinterpret_cast<uint32_t *>(buf);
  uint32_t x[E];
#pragma unroll
  for (int e = 0; e < E; e++) x[e] = (e * 32 + lane < n) ? ordered_bits(buf[e * 32 + lane]) : 0u;
  {
    float v[E];
    load_run<E>(buf + lane * E, v);
#pragma unroll
    for (int e = 0; e < E; e++) key[e] = (lane * E + e < n) ? ordered_bits(v[e]) : ~0u;
  }
  __syncwarp();
  bitonic_warp<E>(key);
  store_run<E>(u + lane * E, key);
  __syncwarp();
  int lb[E];
  bool tie[E];
  bool any = false;
#pragma unroll
  for (int e = 0; e < E; e++) {
    // lower bound of x among the 32E sorted keys (entries past n are ~0u,
    // never below an input key)
    int l = 0;
#pragma unroll
    for (int step = 16 * E; step >= 1; step >>= 1) l += (u[l + step - 1] < x[e]) ? step : 0;
    lb[e] = l;
    pos[e] = l;
    tie[e] = (e * 32 + lane < n) && l + 1 < n && u[l + 1] == x[e];
    any |= tie[e];
  }
  if (__any_sync(SG_FULL, any)) {
#pragma unroll
    for (int e = 0; e < E; e++)
      if (tie[e]) cnt[lb[e]] = 0;
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int e = 0; e < E; e++) {
      // slot e holds inputs 32e .. 32e+31: earlier slots are counted in
      // cnt, earlier lanes of this slot by the match mask
      const unsigned m = __match_any_sync(SG_FULL, tie[e] ? lb[e] : -1 - lane);
      int before = 0;
      if (tie[e]) before = cnt[lb[e]] + __popc(m & lt);
      __syncwarp();
      if (tie[e] && (m >> lane) == 1u) cnt[lb[e]] += __popc(m);
      __syncwarp();
      pos[e] += before;
    }
  }
  __syncwarp();
}

// Sort the samples of a ray in shared memory.  sz[0, done) hold the
// samples, sz[done, S) the -1 padding (warp_sample_ray's layout).  On
// return sz[i] holds the depth of sorted position i: the padding first, then
// the samples ascending by (depth, position); with POS, spos[i] holds the
// original position (padding stable: done, done+1, ...).  Only the samples
// are sorted, with the smallest register bitonic network that holds them;
// done <= 32 * EMAX.  Without POS the keys are the depths alone: samples of
// equal depth have equal bits, so the sorted depths are the same.
template <int EMAX, bool POS>
__device__ __forceinline__ void warp_sort_samples(float *sz, int *spos, int S, int done) {
  const int lane = lane_id();
  const int npad = S - done;
  if (done > 0) {
    auto run = [&](auto tag) {
      constexpr int E = decltype(tag)::value;
      if constexpr (POS) {
        uint32_t key[E];
        int pos[E];
        warp_sort_ranked<E>(sz, spos, done, key, pos);  // spos[0, done): scratch
#pragma unroll
        for (int e = 0; e < E; e++) {
          const int j = lane * E + e;
          if (j < done) sz[npad + j] = from_ordered(key[e]);
          const int i = e * 32 + lane;
          if (i < done) spos[npad + pos[e]] = i;
        }
      } else {
        uint32_t key[E];
        float v[E];
        load_run<E>(sz + lane * E, v);
#pragma unroll
        for (int e = 0; e < E; e++) key[e] = (lane * E + e < done) ? ordered_bits(v[e]) : ~0u;
        __syncwarp();
        bitonic_warp<E>(key);
#pragma unroll
        for (int e = 0; e < E; e++) {
          const int j = lane * E + e;
          if (j < done) sz[npad + j] = from_ordered(key[e]);
        }
      }
    };
    if (done <= 32) {
      run(std::integral_constant<int, 1>());
    } else if constexpr (EMAX >= 2) {
      if (done <= 64) {
        run(std::integral_constant<int, 2>());
      } else if constexpr (EMAX >= 4) {
        if (done <= 128) run(std::integral_constant<int, 4>());
        else if constexpr (EMAX >= 8) run(std::integral_constant<int, 8>());
      }
    }
  }
  __syncwarp();
  for (int q = lane; q < npad; q += 32) {
    sz[q] = -1.0f;
    if (POS) spos[q] = done + q;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// compositing (volume_rendering.cu:17-240)
// ---------------------------------------------------------------------------
// alpha per sorted position.  mode 0: 1 - exp(-sigma * delta) with delta to
// the next position holding z > 0 (else the last position; 1e10 for the
// last position itself, :87-97); mode 1: alpha = sigma.  s_z: depths by
// sorted position.  Invalid positions (z < 0) get alpha 0.
template <int E>
__device__ __forceinline__ void ray_alpha(const float (&z)[E], const float (&sg)[E], unsigned valid, int S,
                                          int mode, const float *s_z, float (&al)[E], float (&dl)[E]) {
  const int lane = lane_id();
  if (mode == 0) {
    unsigned gtz[E];
#pragma unroll
    for (int e = 0; e < E; e++) gtz[e] = __ballot_sync(SG_FULL, z[e] > 0.0f);
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int i = e * 32 + lane;
      al[e] = 0.0f;
      dl[e] = 0.0f;
      if ((valid >> e) & 1u) {
        float delta;
        if (i == S - 1) {
          delta = 1e10f;
        } else {
          int m = S - 1;
          const unsigned above = (lane == 31) ? 0u : (gtz[e] & (~0u << (lane + 1)));
          if (above) {
            m = e * 32 + __ffs(above) - 1;
          } else {
#pragma unroll
            for (int e2 = 0; e2 < E; e2++)
              if (e2 > e && gtz[e2] && m == S - 1) m = e2 * 32 + __ffs(gtz[e2]) - 1;
          }
          delta = s_z[m] - z[e];
        }
        dl[e] = delta;
        al[e] = 1.0f - expf(-sg[e] * delta);
      }
    }
  } else {
#pragma unroll
    for (int e = 0; e < E; e++) {
      al[e] = ((valid >> e) & 1u) ? sg[e] : 0.0f;
      dl[e] = 0.0f;
    }
  }
}

// Transmittance before each position, carried strictly sequentially over
// positions (bit-identical to the reference's serial T *= 1 - alpha, so is
// the early-termination decision T < t_thres, which the reference takes
// after each valid sample).  proc: position reached; post: transmittance
// after the position still >= t_thres.
//
// Every lane runs the same chain (warp-uniform), eight positions per step
// from a shared-memory factor array; lane 0 stores the transmittance before
// each position into a second array, which the owning lanes read back.
// When every factor is in [0, 1] the product never increases (rounding is
// monotonic), so one test of the step's last value finds the step where it
// first falls below t_thres; otherwise the step's lowest value is tested.
// The product changes only at valid positions.
// Positions before the first valid one are padding (factor 1) and are
// skipped.  s_f: kTransScratch<E> floats of warp-private shared scratch,
// 16-byte aligned.
template <int E>
constexpr int kTransScratch = 2 * (32 * E + 8);

template <int E>
__device__ __forceinline__ void ray_transmittance(const float (&al)[E], unsigned valid, int S, float t_thres,
                                                  float *s_f, float (&tb)[E], unsigned &proc, unsigned &post) {
  const int lane = lane_id();
  float *s_t = s_f + kTransScratch<E> / 2;
  int m0 = 32 * E;
#pragma unroll
  for (int e = E - 1; e >= 0; e--) {
    const unsigned vb = __ballot_sync(SG_FULL, (valid >> e) & 1u);
    if (vb) m0 = e * 32 + __ffs(vb) - 1;
  }
  bool unit = true;  // every factor in [0, 1] (false for NaN)
#pragma unroll
  for (int e = 0; e < E; e++) {
    const float f = ((valid >> e) & 1u) ? (1.0f - al[e]) : 1.0f;
    unit = unit && f >= 0.0f && f <= 1.0f;
    s_f[e * 32 + lane] = f;
  }
  if (lane < 8) s_f[32 * E + lane] = 1.0f;  // the last step may read past position 32 E - 1
  const bool mono = __all_sync(SG_FULL, unit);
  __syncwarp();
  int stop = 1 << 30;  // position whose update took T below t_thres
  int end = S;
  if (m0 < S) {
    float T = 1.0f;
    for (int i = m0 & ~3; i < S; i += 8) {
      const float4 f0 = *reinterpret_cast<const float4 *>(s_f + i);
      const float4 f1 = *reinterpret_cast<const float4 *>(s_f + i + 4);
      float Ta[9];
      Ta[0] = T;
      Ta[1] = Ta[0] * f0.x;
      Ta[2] = Ta[1] * f0.y;
      Ta[3] = Ta[2] * f0.z;
      Ta[4] = Ta[3] * f0.w;
      Ta[5] = Ta[4] * f1.x;
      Ta[6] = Ta[5] * f1.y;
      Ta[7] = Ta[6] * f1.z;
      Ta[8] = Ta[7] * f1.w;
      if (lane == 0) {
        *reinterpret_cast<float4 *>(s_t + i) = make_float4(Ta[0], Ta[1], Ta[2], Ta[3]);
        *reinterpret_cast<float4 *>(s_t + i + 4) = make_float4(Ta[4], Ta[5], Ta[6], Ta[7]);
      }
      // lowest transmittance of the step: the last when the product cannot rise
      float lo = Ta[8];
      if (!mono)
        lo = fminf(fminf(fminf(Ta[1], Ta[2]), fminf(Ta[3], Ta[4])), fminf(fminf(Ta[5], Ta[6]), fminf(Ta[7], Ta[8])));
      if (lo < t_thres) {
        // the first position q of [m0, S) in this step with T after it below
        // t_thres (outside [m0, S) the factors are 1)
        int k = 8;
#pragma unroll
        for (int q = 7; q >= 0; q--)
          if (Ta[q + 1] < t_thres && i + q >= m0 && i + q < S) k = q;
        if (k < 8) {
          stop = i + k;
          end = stop + 1;
          break;
        }
      }
      T = Ta[8];
    }
  } else {
    end = 0;
  }
  __syncwarp();
  proc = 0;
  post = 0;
#pragma unroll
  for (int e = 0; e < E; e++) {
    const int i = e * 32 + lane;
    tb[e] = 0.0f;
    if (i >= m0 && i < end) {
      tb[e] = s_t[i];
      proc |= 1u << e;
      if (i != stop) post |= 1u << e;
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// dense-grid trilinear tap (grid [D,D,D,C] channel-last of one frame, voxel
// (x,y,z) centred at bbox_min + (x,y,z) * vs, outside corners contribute 0)
// ---------------------------------------------------------------------------
// Cell (lower corner index) and the eight corner weights of a trilinear tap
// at pt, in voxel units u = (pt - bmin) / vs; corner cr = (dx, dy, dz) =
// bits (2, 1, 0) of cr.  The fraction of u is formed to about 1e-7 of a
// voxel: pt - bmin as an exact two-term sum (Knuth's two-sum), then the
// quotient's remainder from a fused multiply-add carried into the
// fraction.  A plain (pt - bmin) * inv_vs is off by up to ~3e-5 voxel at
// u ~ 250, which the steep density transform turns into density errors of
// ~1e-3 and composited errors above 1e-5.
__device__ __forceinline__ void tap_frac(const float bmin[3], float vs, float inv_vs, const float pt[3],
                                         int (&i0)[3], float (&f)[3]) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float nb = -bmin[a];
    const float dh = pt[a] + nb;                         // pt - bmin, rounded
    const float bv = dh - pt[a];
    const float dl = (pt[a] - (dh - bv)) + (nb - bv);    // its rounding error (two-sum)
    const float uh = dh * inv_vs;
    const float ul = (__fmaf_rn(-uh, vs, dh) + dl) * inv_vs;  // (pt - bmin) / vs - uh
    float fl = floorf(uh);
    float fr = (uh - fl) + ul;
    if (fr < 0.0f) {
      fl -= 1.0f;
      fr += 1.0f;
    } else if (fr >= 1.0f) {
      fl += 1.0f;
      fr -= 1.0f;
    }
    i0[a] = (int)fl;
    f[a] = fr;
  }
}

// Weight of corner cr = (dx, dy, dz) = bits (2, 1, 0) of cr at fractions f.
__device__ __forceinline__ float corner_weight(const float (&f)[3], int cr) {
  const int dx = (cr >> 2) & 1, dy = (cr >> 1) & 1, dz = cr & 1;
  return (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) * (dz ? f[2] : 1.0f - f[2]);
}

__device__ __forceinline__ void tap_cell(const float bmin[3], float vs, float inv_vs, const float pt[3],
                                         int (&i0)[3], float (&w)[8]) {
  float f[3];
  tap_frac(bmin, vs, inv_vs, pt, i0, f);
#pragma unroll
  for (int cr = 0; cr < 8; cr++) w[cr] = corner_weight(f, cr);
}

__device__ __forceinline__ bool corner_inside(const int (&i0)[3], int cr, int D, size_t &off) {
  const int ix = i0[0] + ((cr >> 2) & 1), iy = i0[1] + ((cr >> 1) & 1), iz = i0[2] + (cr & 1);
  if (ix < 0 || iy < 0 || iz < 0 || ix >= D || iy >= D || iz >= D) return false;
  off = ((size_t)ix * D + iy) * D + iz;
  return true;
}

// Trilinear interpolation of a channel-last grid [D, D, D, C] for a given
// cell and weights; corners outside the grid contribute 0.
template <int C>
__device__ __forceinline__ void grid_tap_cell(const float *__restrict__ grid, int D, const int (&i0)[3],
                                              const float (&w)[8], float (&acc)[C]) {
#pragma unroll
  for (int c = 0; c < C; c++) acc[c] = 0.0f;
#pragma unroll
  for (int cr = 0; cr < 8; cr++) {
    size_t off;
    if (!corner_inside(i0, cr, D, off)) continue;
    const float *g = grid + off * C;
    if constexpr (C % 4 == 0) {
#pragma unroll
      for (int c4 = 0; c4 < C / 4; c4++) {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(g) + c4);
        acc[4 * c4 + 0] = __fmaf_rn(w[cr], v.x, acc[4 * c4 + 0]);
        acc[4 * c4 + 1] = __fmaf_rn(w[cr], v.y, acc[4 * c4 + 1]);
        acc[4 * c4 + 2] = __fmaf_rn(w[cr], v.z, acc[4 * c4 + 2]);
        acc[4 * c4 + 3] = __fmaf_rn(w[cr], v.w, acc[4 * c4 + 3]);
      }
    } else {
#pragma unroll
      for (int c = 0; c < C; c++) acc[c] = __fmaf_rn(w[cr], __ldg(g + c), acc[c]);
    }
  }
}

template <int C>
__device__ __forceinline__ void grid_tap(const float *__restrict__ grid, int D, const float bmin[3], float vs,
                                         float inv_vs, const float pt[3], float (&acc)[C]) {
  int i0[3];
  float w[8];
  tap_cell(bmin, vs, inv_vs, pt, i0, w);
  grid_tap_cell<C>(grid, D, i0, w, acc);
}

// Density of a normalised TSDF value t: sigmoid(-t * scale / s) / s, with
// k = scale / s and inv_s = 1 / s folded by the caller.  tsdf_sigmoid is
// the sigmoid factor (kept by the adjoint: d sigma / d t = -k inv_s sg (1 - sg)).
__device__ __forceinline__ float tsdf_sigmoid(float t, float k) {
  return 1.0f / (1.0f + expf(t * k));
}
__device__ __forceinline__ float tsdf_density(float t, float k, float inv_s) { return tsdf_sigmoid(t, k) * inv_s; }

}  // namespace sg
