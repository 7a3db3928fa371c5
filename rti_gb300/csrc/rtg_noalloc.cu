// rtg_noalloc.cu -- normalised, smoothed estimates without any device allocation.
//
// rtg_get_mc_estimates allocates a small device scratch buffer for the
// maximum on every call and frees it again; cudaFree synchronises the whole
// device.  Some callers cannot allocate device memory at that point: a
// process simulator that keeps every byte of the GPU under its own memory
// pool (and must not grow it behind the pool's back), or one that overlaps
// the next surface update with the flux finalisation and cannot afford the
// device-wide synchronisation of cudaFree.  rtg_get_mc_estimates_noalloc
// computes the same estimates (device.hpp:154-187) into a device buffer the
// caller owns, and keeps its scratch -- one maximum per 256-element block
// plus the overall maximum -- in the file-scope array below.
//
// The array lives in every GPU that loads the library until the process
// exits: 32,768 doubles (256 KiB), enough for 8,388,352 primitives; larger
// surfaces are rejected with RTG_ERR_INVALID_ARGUMENT.  All calls on a device
// share it and it keeps the last call's contents; every slot a call reads is
// written earlier in the same call, so nothing needs clearing, but two calls
// whose kernels overlap on the GPU (different streams, no ordering) race on
// it and must be serialised by the caller.
//
// Ordering: the kernels are enqueued on the caller's stream after a wait on
// the event the last trace recorded at its end, so the estimates never read
// accumulators or areas that the trace is still writing, whichever stream it
// ran on; the host does not block.
//
// The device address of the array is looked up with cudaGetSymbolAddress the
// first time a CUDA context calls in (the first call on each device, and the
// first call again after that device's context was destroyed and created
// anew, e.g. by cudaDeviceReset); that first call should come before any
// stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "rtg_internal.cuh"

namespace rtg {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaSlots = 32768;                  // [0] overall max, [1..] block maxima
constexpr int64_t kNaMaxBlocks = kNaSlots - 1;
constexpr int64_t kNaMaxPrimitives = kNaMaxBlocks * kNaThreads;  // 8,388,352

__device__ __align__(256) double g_na_scratch[kNaSlots];

constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
// per device: the address of the array in the context it was looked up in
struct NaAddr {
  unsigned long long ctx_id = 0;
  double* addr = nullptr;
};
NaAddr g_na_addr[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Process-unique id of the current CUDA context (0 if the driver cannot say);
// called with g_na_mutex held:
// a context created after cudaDeviceReset gets a new id, even where its
// handle value repeats.  The driver functions are found through the runtime,
// so the library needs no link against the driver library.
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
    cudaGetLastError();
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the scratch array on `device` (the current device), set
// up once per device and context.  Without a context id (a driver that cannot
// report one) the address is looked up on every call.
int scratch_address(rtg_context* ctx, int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "device index too large");
  std::lock_guard<std::mutex> lock(g_na_mutex);
  const unsigned long long cid = current_context_id();
  NaAddr& a = g_na_addr[device];
  if (cid == 0 || a.ctx_id != cid || !a.addr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess) return check_cuda(ctx, e, "cudaGetSymbolAddress(no-alloc scratch)");
    a.addr = static_cast<double*>(p);
    a.ctx_id = cid;
  }
  *out = a.addr;
  return RTG_OK;
}

// Same per-element arithmetic as smooth_kernel in rtg_surface.cu; the maximum
// is reduced per block into scratch[1 + block] instead of by a global atomic.
__global__ void __launch_bounds__(kNaThreads) na_smooth_kernel(const double* __restrict__ s1,
                                                                const float* __restrict__ areas, int64_t n, int64_t nd,
                                                                const int64_t* __restrict__ rp,
                                                                const int32_t* __restrict__ cols, float* __restrict__ est,
                                                                double* __restrict__ scratch) {
  __shared__ double warp_max[kNaThreads / 32];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double vv = 0.0;
  if (i < n) {
    vv = s1[i] / areas[i];
    int64_t deg = 0;
    if (rp && i < nd) {
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q) vv += s1[cols[q]] / areas[cols[q]];
      deg = rp[i + 1] - rp[i];
    }
    vv /= (double)(deg + 1);
    est[i] = (float)vv;
  }
  double m = (i < n && vv > 0.0) ? vv : 0.0;
  for (int o = 16; o > 0; o >>= 1) {
    const double y = __shfl_down_sync(0xFFFFFFFFu, m, o);
    if (y > m) m = y;
  }
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < kNaThreads / 32; ++w)
      if (warp_max[w] > b) b = warp_max[w];
    scratch[1 + blockIdx.x] = b;
  }
}

__global__ void __launch_bounds__(kNaThreads) na_reduce_kernel(double* __restrict__ scratch, int64_t nblocks) {
  __shared__ double warp_max[kNaThreads / 32];
  double m = 0.0;
  for (int64_t b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double y = scratch[1 + b];
    if (y > m) m = y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double y = __shfl_down_sync(0xFFFFFFFFu, m, o);
    if (y > m) m = y;
  }
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < kNaThreads / 32; ++w)
      if (warp_max[w] > b) b = warp_max[w];
    scratch[0] = b;
  }
}

__global__ void na_divide_kernel(float* __restrict__ est, int64_t n, const double* __restrict__ scratch) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  est[i] = (float)((double)est[i] / scratch[0]);
}

}  // namespace
}  // namespace rtg

using namespace rtg;

extern "C" RTG_API int rtg_get_mc_estimates_noalloc(rtg_context* ctx, float* d_out, void* stream) {
  if (!ctx || !d_out) return RTG_ERR_INVALID_ARGUMENT;
  if (!ctx->traced) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "no trace has run");
  const int64_t np = ctx->g.nd + ctx->g.nt;
  if (np > kNaMaxPrimitives)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT,
                     "rtg_get_mc_estimates_noalloc handles at most 8388352 primitives; use rtg_get_mc_estimates");
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  double* scratch = nullptr;
  RTG_TRY(scratch_address(ctx, ctx->device, &scratch));
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  const int64_t nblocks = (np + kNaThreads - 1) / kNaThreads;
  const Geometry& g = ctx->g;
  // after the trace's last kernel, on whichever stream the trace ran
  RTG_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev1, 0));
  na_smooth_kernel<<<(unsigned)nblocks, kNaThreads, 0, st>>>(ctx->acc.p, ctx->areas.p, np, g.nd,
                                                            g.nd > 0 ? g.nb_ptr.p : nullptr, g.nb_idx.p, d_out,
                                                            scratch);
  na_reduce_kernel<<<1, kNaThreads, 0, st>>>(scratch, nblocks);
  na_divide_kernel<<<(unsigned)nblocks, kNaThreads, 0, st>>>(d_out, np, scratch);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}
