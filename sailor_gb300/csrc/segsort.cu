// segsort.cu -- device-wide exclusive scan and a stable LSD radix sort of
// (key, value) pairs, the building blocks of the deterministic gradient
// reduction (scatter.cu).  Both work on buffers sized for a host-known
// capacity while the live element count stays in device memory, so a whole
// training step can be captured in a CUDA graph with no host read-back.
//
// Scan: blocks of 1024 ints (256 threads x 4) reduce to block sums, one CTA
// scans the block sums, every block then scans itself from its offset; the
// blocks past the live count are skipped by fixed, SM-sized grids.
//
// Radix sort: 8-bit digits, least significant first.  A tile is 4096 items:
// 8 warps x 16 rounds x 32 lanes in index order.  Pass = per-tile digit
// histograms (digit-major table) -> exclusive scan of the table -> scatter,
// where an item's place is the table entry of (its digit, its tile) plus the
// number of equal digits before it in the tile: warp w counts its own
// rounds' digits with __match_any_sync (peers before the lane in a round,
// plus a running per-warp count), and warps before w add their totals.  The
// order of equal keys is therefore the input order (stable), and the result
// is the same on every run.
#include "common.cuh"
#include "segsort.cuh"

namespace sg {

constexpr int kScanBlock = 1024;  // ints per scan block
constexpr int kSortTile = 4096;   // items per sort tile (256 threads x 16)
constexpr int kDigits = 256;

// ---------------------------------------------------------------------------
// exclusive scan
// ---------------------------------------------------------------------------
__device__ __forceinline__ int block_excl_scan_256(int v, int *s_warp, int &total) {
  // exclusive scan of one int per thread over a 256-thread block
  const int lane = lane_id(), w = threadIdx.x >> 5;
  const int incl = warp_incl_scan(v);
  if (lane == 31) s_warp[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int x = lane < 8 ? s_warp[lane] : 0;
    const int xi = warp_incl_scan(x);
    if (lane < 8) s_warp[8 + lane] = xi - x;
    if (lane == 7) s_warp[16] = xi;
  }
  __syncthreads();
  const int out = s_warp[8 + w] + incl - v;
  total = s_warp[16];
  __syncthreads();
  return out;
}

// n_dev (may be null): the live count in device memory, at most n
__device__ __forceinline__ long live_count(long n, const int *n_dev) {
  if (!n_dev) return n;
  const long m = *n_dev;
  return m < n ? m : n;
}

// Blocks of kScanBlock elements up to the live count; a fixed grid strides
// over them, so a capacity far above the live count costs no launches.
__global__ void __launch_bounds__(256) scan_block_sums_kernel(const int *__restrict__ in, long n,
                                                              const int *__restrict__ n_dev,
                                                              int *__restrict__ bsum) {
  __shared__ int s_warp[17];
  n = live_count(n, n_dev);
  const long nb = (n + kScanBlock - 1) / kScanBlock;
  for (long blk = blockIdx.x; blk < nb; blk += gridDim.x) {
    const long base = blk * kScanBlock + threadIdx.x * 4;
    int v = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) v += (base + k < n) ? in[base + k] : 0;
    int total;
    block_excl_scan_256(v, s_warp, total);
    if (threadIdx.x == 0) bsum[blk] = total;
  }
}

// One CTA of 1024 threads: exclusive scan of the live block sums in place,
// total into *total.
__global__ void __launch_bounds__(1024) scan_sums_kernel(int *bsum, long n, const int *__restrict__ n_dev,
                                                         int *total) {
  __shared__ int s_w[33];
  n = live_count(n, n_dev);
  const int nb = (int)((n + kScanBlock - 1) / kScanBlock);
  const int lane = lane_id(), w = threadIdx.x >> 5;
  int carry = 0;
  for (int c0 = 0; c0 < nb; c0 += 1024) {
    const int i = c0 + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    const int incl = warp_incl_scan(v);
    if (lane == 31) s_w[w] = incl;
    __syncthreads();
    if (w == 0) {
      const int x = s_w[lane];
      const int xi = warp_incl_scan(x);
      s_w[lane] = xi - x;
      if (lane == 31) s_w[32] = xi;
    }
    __syncthreads();
    if (i < nb) bsum[i] = carry + s_w[w] + incl - v;
    carry += s_w[32];
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void __launch_bounds__(256) scan_apply_kernel(const int *__restrict__ in, long n,
                                                         const int *__restrict__ n_dev,
                                                         const int *__restrict__ bsum, int *__restrict__ out) {
  __shared__ int s_warp[17];
  n = live_count(n, n_dev);
  const long nb = (n + kScanBlock - 1) / kScanBlock;
  for (long blk = blockIdx.x; blk < nb; blk += gridDim.x) {
    const long base = blk * kScanBlock + threadIdx.x * 4;
    int v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k] = (base + k < n) ? in[base + k] : 0;
      s += v[k];
    }
    int total;
    int run = block_excl_scan_256(s, s_warp, total) + bsum[blk];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (base + k < n) out[base + k] = run;
      run += v[k];
    }
  }
}

size_t scan_scratch_ints(long n) { return (size_t)ceil_div(n, kScanBlock) + 1; }

void launch_excl_scan_dev(const int *in, long n, const int *n_dev, int *out, int *scratch, int *total,
                          sg_stream_t stream) {
  const long nb = ceil_div(n, kScanBlock);
  if (nb == 0) {
    // nothing to scan: a zero total (through a one-CTA launch, so that the
    // call stays a stream operation)
    scan_sums_kernel<<<1, 1024, 0, stream>>>(scratch, 0, nullptr, total);
    return;
  }
  const long cap = (long)num_sms() * 8;
  const int g = (int)(nb < cap ? nb : cap);
  scan_block_sums_kernel<<<g, 256, 0, stream>>>(in, n, n_dev, scratch);
  scan_sums_kernel<<<1, 1024, 0, stream>>>(scratch, n, n_dev, total);
  scan_apply_kernel<<<g, 256, 0, stream>>>(in, n, n_dev, scratch, out);
}

void launch_excl_scan(const int *in, long n, int *out, int *scratch, int *total, sg_stream_t stream) {
  launch_excl_scan_dev(in, n, nullptr, out, scratch, total, stream);
}

// ---------------------------------------------------------------------------
// radix sort
// ---------------------------------------------------------------------------
// meta[0]: live tiles ceil(n / kSortTile), meta[1]: live table entries
// (kDigits x live tiles).  The digit-major tables hold the live tiles only,
// so their scans cover the live items, not the capacity.
__global__ void radix_meta_kernel(const int *__restrict__ n_dev, int *__restrict__ meta) {
  const int ntl = (int)ceil_div(*n_dev, kSortTile);
  meta[0] = ntl;
  meta[1] = ntl * kDigits;
}

__global__ void __launch_bounds__(256) radix_hist_kernel(const uint32_t *__restrict__ keys,
                                                         const int *__restrict__ n_dev, int shift,
                                                         const int *__restrict__ meta, int *__restrict__ hist) {
  __shared__ int s_h[kDigits];
  const int ntiles = meta[0];
  const long n = *n_dev;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    s_h[threadIdx.x] = 0;
    __syncthreads();
    const long base = (long)tile * kSortTile;
    uint32_t kk[kSortTile / 256];
#pragma unroll
    for (int k = 0; k < kSortTile / 256; k++) {
      const long i = base + k * 256 + threadIdx.x;
      kk[k] = i < n ? __ldg(keys + i) : 0u;
    }
#pragma unroll
    for (int k = 0; k < kSortTile / 256; k++) {
      const long i = base + k * 256 + threadIdx.x;
      if (i < n) atomicAdd(&s_h[(kk[k] >> shift) & 0xff], 1);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + tile] = s_h[threadIdx.x];  // digit-major, live tiles
    __syncthreads();
  }
}

// vals == nullptr: the values are the item indices.  The tile's items are
// first placed in shared memory in their sorted order (digit runs in digit
// order), then written out with consecutive threads on consecutive
// destinations of each digit run.
__global__ void __launch_bounds__(256, 3) radix_scatter_kernel(const uint32_t *__restrict__ keys,
                                                            const uint32_t *__restrict__ vals,
                                                            const int *__restrict__ n_dev, int shift,
                                                            const int *__restrict__ meta,
                                                            const int *__restrict__ offs,
                                                            uint32_t *__restrict__ keys_out,
                                                            uint32_t *__restrict__ vals_out) {
  constexpr int R = kSortTile / 256;  // rounds per warp
  __shared__ int s_cnt[8][kDigits];   // per-warp running count per digit
  __shared__ int s_start[kDigits];    // first tile position of each digit
  __shared__ int s_warp[17];
  __shared__ uint32_t s_key[kSortTile], s_val[kSortTile];
  const int ntiles = meta[0];
  const int lane = lane_id(), w = threadIdx.x >> 5;
  const long n = *n_dev;
  const unsigned lt = (1u << lane) - 1u;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    for (int d = lane; d < kDigits; d += 32) s_cnt[w][d] = 0;
    __syncwarp();
    const long tbase = (long)tile * kSortTile;
    const long wbase = tbase + (long)w * (R * 32);
    uint32_t k[R], v[R];
    int rank[R];
    // all of the warp's loads first, so that they are in flight together
#pragma unroll
    for (int q = 0; q < R; q++) {
      const long i = wbase + q * 32 + lane;
      const bool live = i < n;
      k[q] = live ? __ldg(keys + i) : 0u;
      v[q] = live ? (vals ? __ldg(vals + i) : (uint32_t)i) : 0u;
    }
#pragma unroll
    for (int q = 0; q < R; q++) {
      const long i = wbase + q * 32 + lane;
      const bool live = i < n;
      // inactive lanes match each other on a digit value no live key has
      const unsigned dg = live ? ((k[q] >> shift) & 0xffu) : 0x100u;
      const unsigned peers = __match_any_sync(SG_FULL, dg);
      const int before = __popc(peers & lt);
      int c = 0;
      if (live) c = s_cnt[w][dg];
      __syncwarp();
      if (live && before == 0) s_cnt[w][dg] = c + __popc(peers);
      __syncwarp();
      rank[q] = c + before;
    }
    __syncthreads();
    // per digit: the counts of the warps before each warp, and the tile total
    {
      const int d = threadIdx.x;  // 256 threads, one digit each
      int run = 0;
#pragma unroll
      for (int ww = 0; ww < 8; ww++) {
        const int c = s_cnt[ww][d];
        s_cnt[ww][d] = run;
        run += c;
      }
      int total;
      s_start[d] = block_excl_scan_256(run, s_warp, total);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < R; q++) {
      const long i = wbase + q * 32 + lane;
      if (i < n) {
        const int dg = (k[q] >> shift) & 0xff;
        const int pos = s_start[dg] + s_cnt[w][dg] + rank[q];
        s_key[pos] = k[q];
        s_val[pos] = v[q];
      }
    }
    __syncthreads();
    const int live = (int)(n - tbase < kSortTile ? n - tbase : kSortTile);
    for (int i = threadIdx.x; i < live; i += 256) {
      const uint32_t key = s_key[i];
      const int dg = (key >> shift) & 0xff;
      const long dst = (long)offs[(size_t)dg * ntiles + tile] + (i - s_start[dg]);
      keys_out[dst] = key;
      vals_out[dst] = s_val[i];
    }
    __syncthreads();
  }
}

size_t radix_scratch_bytes(long cap) {
  const long ntiles = ceil_div(cap, kSortTile) > 0 ? ceil_div(cap, kSortTile) : 1;
  const long table = ntiles * kDigits;
  return (size_t)(2 * table + (long)scan_scratch_ints(table) + 8) * sizeof(int);
}

int launch_radix_sort(const uint32_t *keys_in, const uint32_t *vals_in, const int *n_dev, long cap, int key_bits,
                      uint32_t *keys_a, uint32_t *vals_a, uint32_t *keys_b, uint32_t *vals_b, void *scratch,
                      sg_stream_t stream) {
  const int ntiles = ceil_div(cap, kSortTile) > 0 ? ceil_div(cap, kSortTile) : 1;
  const int ghist = ntiles < num_sms() * 8 ? ntiles : num_sms() * 8;
  const int gscat = ntiles < num_sms() * 4 ? ntiles : num_sms() * 4;
  const long table = (long)ntiles * kDigits;
  int *hist = (int *)scratch;
  int *offs = hist + table;
  int *ss = offs + table;
  int *tot = ss + scan_scratch_ints(table);
  int *meta = tot + 2;
  const int passes = key_bits <= 0 ? 1 : (key_bits + 7) / 8;
  const uint32_t *ki = keys_in;
  const uint32_t *vi = vals_in;
  radix_meta_kernel<<<1, 1, 0, stream>>>(n_dev, meta);
  for (int p = 0; p < passes; p++) {
    uint32_t *ko = (p & 1) ? keys_b : keys_a;
    uint32_t *vo = (p & 1) ? vals_b : vals_a;
    radix_hist_kernel<<<ghist, 256, 0, stream>>>(ki, n_dev, 8 * p, meta, hist);
    launch_excl_scan_dev(hist, table, meta + 1, offs, ss, tot, stream);
    radix_scatter_kernel<<<gscat, 256, 0, stream>>>(ki, vi, n_dev, 8 * p, meta, offs, ko, vo);
    ki = ko;
    vi = vo;
  }
  return passes;
}

}  // namespace sg

using namespace sg;

extern "C" size_t sg_sort_pairs_scratch_bytes(long long capacity) { return radix_scratch_bytes((long)capacity); }

extern "C" int sg_sort_pairs(const uint32_t *keys, const int *count, long long capacity, int key_bits,
                             uint32_t *keys_out, uint32_t *vals_out, uint32_t *keys_tmp, uint32_t *vals_tmp,
                             void *scratch, size_t scratch_bytes, sg_stream_t stream) {
  if (!keys || !count || !keys_out || !vals_out || !keys_tmp || !vals_tmp || !scratch) return SG_ERR_INVALID_ARG;
  if (capacity <= 0 || capacity >= (1ll << 31) || key_bits < 1 || key_bits > 32) return SG_ERR_INVALID_ARG;
  if (scratch_bytes < radix_scratch_bytes((long)capacity)) return SG_ERR_INVALID_ARG;
  const int passes = launch_radix_sort(keys, nullptr, count, (long)capacity, key_bits, keys_out, vals_out,
                                       keys_tmp, vals_tmp, scratch, stream);
  if (passes % 2 == 0) {
    // the last pass wrote the second pair: copy it into the outputs
    cudaMemcpyAsync(keys_out, keys_tmp, (size_t)capacity * 4, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
    cudaMemcpyAsync(vals_out, vals_tmp, (size_t)capacity * 4, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}
