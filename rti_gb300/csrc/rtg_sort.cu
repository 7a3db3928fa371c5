// rtg_sort.cu -- stable LSD radix sort of (uint32 key, uint32 value) pairs and
// exclusive prefix sums, used by the LBVH build (Morton order) and by the
// neighbour-grid build (cell order).  Neither runs inside a trace.
//
// Radix sort: 8-bit digits; per pass a histogram kernel counts the digits of
// each 4096-element tile, one scan turns the [digit][tile] table into output
// offsets, and a scatter kernel writes every tile back in digit order, ranking
// equal digits by warp match masks so that the pass is stable.
#include <cstdint>

#include "rtg_internal.cuh"

namespace rtg {

namespace {

constexpr int kRsThreads = 256;
constexpr int kRsRounds = 16;
constexpr int kRsTile = kRsThreads * kRsRounds;
constexpr int kRsWarps = kRsThreads / 32;

__global__ void __launch_bounds__(kRsThreads) rs_hist(const uint32_t* __restrict__ keys, int64_t n,
                                                       int shift, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  const int tid = threadIdx.x;
  h[tid] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsRounds; ++r) {
    int64_t i = base + (int64_t)r * kRsThreads + tid;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(int64_t)tid * gridDim.x + blockIdx.x] = h[tid];
}

__global__ void __launch_bounds__(kRsThreads) rs_scatter(const uint32_t* __restrict__ kin,
                                                          const uint32_t* __restrict__ vin,
                                                          uint32_t* __restrict__ kout,
                                                          uint32_t* __restrict__ vout, int64_t n,
                                                          int shift,
                                                          const uint32_t* __restrict__ offs) {
  __shared__ uint32_t base_off[256];
  __shared__ uint32_t wcnt[kRsWarps][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  base_off[tid] = offs[(int64_t)tid * gridDim.x + blockIdx.x];
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kRsRounds; ++r) {
    for (int j = lane; j < 256; j += 32) wcnt[warp][j] = 0;
    __syncthreads();
    const int64_t i = base + (int64_t)r * kRsThreads + tid;
    const bool valid = i < n;
    const uint32_t k = valid ? kin[i] : 0u;
    const uint32_t d = valid ? ((k >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    const int rank = __popc(peers & lt_mask);
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) wcnt[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pre = 0;
      for (int w = 0; w < warp; ++w) pre += wcnt[w][d];
      const uint32_t pos = base_off[d] + pre + (uint32_t)rank;
      kout[pos] = k;
      vout[pos] = vin[i];
    }
    __syncthreads();
    uint32_t tot = 0;
    for (int w = 0; w < kRsWarps; ++w) tot += wcnt[w][tid];
    base_off[tid] += tot;
    __syncthreads();
  }
}

constexpr int kScanThreads = 1024;
constexpr int64_t kScanChunk = (int64_t)kScanThreads * 4;  // items one block scans in one step

// Exclusive scan of items [base, base + kScanChunk) of a, in place, after
// `carry`; returns the chunk's total.  All threads of the block call it.
template <typename T>
__device__ T scan_chunk(T* __restrict__ a, int64_t base, int64_t m, T carry, T* warp_sums) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = blockDim.x >> 5;
  T v[4];
  T s = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t i = base + (int64_t)tid * 4 + q;
    v[q] = i < m ? a[i] : (T)0;
    s += v[q];
  }
  // inclusive warp scan of the thread sums
  T x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? warp_sums[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) warp_sums[lane] = w;
  }
  __syncthreads();
  T excl = carry + (warp > 0 ? warp_sums[warp - 1] : (T)0) + (x - s);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t i = base + (int64_t)tid * 4 + q;
    if (i < m) a[i] = excl;
    excl += v[q];
  }
  const T chunk_total = warp_sums[nw - 1];
  __syncthreads();  // warp_sums is reused by the next call
  return chunk_total;
}

// Single-block exclusive scan, in place, chunk after chunk.
template <typename T>
__global__ void __launch_bounds__(kScanThreads) scan_excl_kernel(T* __restrict__ a, int64_t m, T* total) {
  __shared__ T warp_sums[32];
  T carry = 0;
  for (int64_t base = 0; base < m; base += kScanChunk) carry += scan_chunk(a, base, m, carry, warp_sums);
  if (threadIdx.x == 0 && total) *total = carry;
}

// Multi-block scan, pass 1: the total of every chunk.
template <typename T>
__global__ void __launch_bounds__(kScanThreads) chunk_sum_kernel(const T* __restrict__ a, int64_t m,
                                                                 T* __restrict__ sums) {
  __shared__ T warp_sums[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  T s = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t i = base + (int64_t)tid * 4 + q;
    if (i < m) s += a[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
  if (lane == 0) warp_sums[warp] = s;
  __syncthreads();
  if (warp == 0) {
    T w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : (T)0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xFFFFFFFFu, w, o);
    if (lane == 0) sums[blockIdx.x] = w;
  }
}

// Multi-block scan, pass 3: every chunk after its scanned offset (pass 2 is
// scan_excl_kernel over the chunk totals).
template <typename T>
__global__ void __launch_bounds__(kScanThreads) chunk_scan_kernel(T* __restrict__ a, int64_t m,
                                                                  const T* __restrict__ offsets) {
  __shared__ T warp_sums[32];
  scan_chunk(a, (int64_t)blockIdx.x * kScanChunk, m, offsets[blockIdx.x], warp_sums);
}

// Exclusive scan of m items in place (total into *d_total when given): one
// block for short arrays, three passes over chunks of kScanChunk otherwise.
template <typename T>
int exclusive_scan(rtg_context* ctx, T* d_a, int64_t m, T* d_total, cudaStream_t st) {
  if (m <= 0) return RTG_OK;
  if (m <= 4 * kScanChunk) {
    scan_excl_kernel<T><<<1, kScanThreads, 0, st>>>(d_a, m, d_total);
    RTG_CUDA(ctx, cudaGetLastError());
    return RTG_OK;
  }
  const int64_t nc = (m + kScanChunk - 1) / kScanChunk;
  DBuf<T> sums;
  RTG_TRY(talloc(ctx, sums, (size_t)nc, st, "scan chunk totals"));
  chunk_sum_kernel<T><<<(unsigned)nc, kScanThreads, 0, st>>>(d_a, m, sums.p);
  scan_excl_kernel<T><<<1, kScanThreads, 0, st>>>(sums.p, nc, d_total);
  chunk_scan_kernel<T><<<(unsigned)nc, kScanThreads, 0, st>>>(d_a, m, sums.p);
  const cudaError_t e = cudaGetLastError();
  tfree(sums, st);
  if (e != cudaSuccess) return check_cuda(ctx, e, "scan");
  return RTG_OK;
}

}  // namespace

int exclusive_scan_u32(rtg_context* ctx, uint32_t* d_a, int64_t m, uint32_t* d_total, cudaStream_t st) {
  return exclusive_scan<uint32_t>(ctx, d_a, m, d_total, st);
}

int exclusive_scan_i64(rtg_context* ctx, int64_t* d_a, int64_t m, int64_t* d_total, cudaStream_t st) {
  return exclusive_scan<long long>(ctx, (long long*)d_a, m, (long long*)d_total, st);
}

// Sorts (keys, vals) by the low `bits` bits of the keys, stably.  Results end
// in d_keys/d_vals; d_tmp_keys/d_tmp_vals are scratch of the same length.
int radix_sort_pairs(rtg_context* ctx, uint32_t* d_keys, uint32_t* d_vals, uint32_t* d_tmp_keys,
                     uint32_t* d_tmp_vals, int64_t n, int bits, cudaStream_t st) {
  if (n <= 1) return RTG_OK;
  const int64_t tiles = (n + kRsTile - 1) / kRsTile;
  DBuf<uint32_t> hist;
  RTG_TRY(talloc(ctx, hist, (size_t)(256 * tiles), st, "radix histogram"));
  uint32_t *kin = d_keys, *vin = d_vals, *kout = d_tmp_keys, *vout = d_tmp_vals;
  int passes = (bits + 7) / 8;
  int rc = RTG_OK;
  for (int p = 0; p < passes && rc == RTG_OK; ++p) {
    const int shift = 8 * p;
    rs_hist<<<(unsigned)tiles, kRsThreads, 0, st>>>(kin, n, shift, hist.p);
    rc = exclusive_scan_u32(ctx, hist.p, 256 * tiles, nullptr, st);
    if (rc != RTG_OK) break;
    rs_scatter<<<(unsigned)tiles, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, shift, hist.p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = check_cuda(ctx, e, "radix scatter");
    uint32_t* t = kin; kin = kout; kout = t;
    t = vin; vin = vout; vout = t;
  }
  if (rc == RTG_OK && kin != d_keys) {
    cudaError_t e1 = cudaMemcpyAsync(d_keys, kin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    cudaError_t e2 = cudaMemcpyAsync(d_vals, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    if (e1 != cudaSuccess) rc = check_cuda(ctx, e1, "radix copy keys");
    else if (e2 != cudaSuccess) rc = check_cuda(ctx, e2, "radix copy values");
  }
  cudaError_t es = cudaStreamSynchronize(st);
  tfree(hist, st);
  if (rc == RTG_OK && es != cudaSuccess) rc = check_cuda(ctx, es, "radix sort");
  return rc;
}

}  // namespace rtg
