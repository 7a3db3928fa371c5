// rtg_trace.cu -- launches of the path kernel for one context (forward trace
// and adjoint replays), and the explicit-ray closest-hit kernel.
#include <algorithm>

#include "rtg_path.cuh"

namespace rtg {

namespace {

__global__ void closest_hit_kernel(const SceneView s, const float* __restrict__ rays, int64_t n, float tnear,
                                   int32_t* __restrict__ prim, float* __restrict__ tout,
                                   unsigned long long* errors) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 6 * i;
  float t;
  int id;
  uint32_t ref;
  unsigned long long e = 0;
  if (closest_hit<256, false>(s, mk3(r[0], r[1], r[2]), mk3(r[3], r[4], r[5]), tnear, t, id, ref, e)) {
    prim[i] = id;
    tout[i] = t;
  } else {
    prim[i] = -1;
    tout[i] = 0.0f;
  }
  if (e) atomicAdd(errors, e);
}

template <int TPB, bool POSTPONE>
PathKernel forward_kernel(int stack, bool shared, bool wide) {
  if (stack <= 32) return kernel_for<kModeForward, false, TPB, 32, POSTPONE>(shared, wide);
  if (stack <= 64) return kernel_for<kModeForward, false, TPB, 64, POSTPONE>(shared, wide);
  return kernel_for<kModeForward, false, TPB, 256, POSTPONE>(shared, wide);
}

template <int TPB>
PathKernel forward_kernel(int stack, bool postpone, bool shared, bool wide) {
  return postpone ? forward_kernel<TPB, true>(stack, shared, wide) : forward_kernel<TPB, false>(stack, shared, wide);
}

// The adjoint replays run with 128 threads and a 64- or 256-entry stack.
PathKernel pick_kernel(int mode, int tpb, int stack, bool postpone, bool shared, bool wide, int& tpb_out) {
  if (mode == kModeAdjGlobal) {
    tpb_out = 128;
    if (stack <= 64) return kernel_for<kModeAdjGlobal, false, 128, 64, false>(shared, wide);
    return wide ? trace_paths_kernel<kModeAdjGlobal, false, 128, 256, false, false, true>
                : trace_paths_kernel<kModeAdjGlobal, false, 128, 256>;
  }
  if (mode == kModeAdjField) {
    tpb_out = 128;
    if (stack <= 64) return kernel_for<kModeAdjField, false, 128, 64, false>(shared, wide);
    return wide ? trace_paths_kernel<kModeAdjField, false, 128, 256, false, false, true>
                : trace_paths_kernel<kModeAdjField, false, 128, 256>;
  }
  if (mode == kModeLogged) {  // a debugging trace: one configuration, both trees
    tpb_out = 128;
    return trace_paths_kernel<kModeLogged, false, 128, 256, false, false, true>;
  }
  if (mode == kModeWindow) {
    tpb_out = 128;
    if (stack <= 64)
      return wide ? trace_paths_kernel<kModeWindow, false, 128, 64, false, false, true>
                  : trace_paths_kernel<kModeWindow, false, 128, 64>;
    return wide ? trace_paths_kernel<kModeWindow, false, 128, 256, false, false, true>
                : trace_paths_kernel<kModeWindow, false, 128, 256>;
  }
  tpb_out = tpb;
  if (tpb == 64) return forward_kernel<64>(stack, postpone, shared, wide);
  if (tpb == 256) return forward_kernel<256>(stack, postpone, shared, wide);
  tpb_out = 128;
  return forward_kernel<128>(stack, postpone, shared, wide);
}

}  // namespace

namespace {

__global__ void s1_fixed_kernel(double* s1, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) reinterpret_cast<long long*>(s1)[i] = __double2ll_rn(s1[i] * 4294967296.0);
}

__global__ void s1_double_kernel(double* s1, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) s1[i] = (double)reinterpret_cast<const long long*>(s1)[i] * (1.0 / 4294967296.0);
}

}  // namespace

int s1_to_fixed(rtg_context* ctx, double* s1, int64_t n, cudaStream_t st) {
  if (n <= 0) return RTG_OK;
  s1_fixed_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s1, n);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

int s1_to_double(rtg_context* ctx, double* s1, int64_t n, cudaStream_t st) {
  if (n <= 0) return RTG_OK;
  s1_double_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s1, n);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

// Whether the tree and the primitive records of ctx outgrow the L2 cache.
bool outgrows_l2(const rtg_context* ctx) {
  int l2 = 0;
  if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const Geometry& g = ctx->g;
  const size_t bytes = g.nodes.n * sizeof(Node) + (g.disc.n + g.tri.n) * sizeof(float4);
  return l2 > 0 && bytes > (size_t)l2;
}

bool shared_stack(rtg_context* ctx, const rtg_launch_config& lc) {
  if (lc.stack_memory == RTG_STACK_SHARED) return true;
  if (lc.stack_memory == RTG_STACK_LOCAL) return false;
  return outgrows_l2(ctx);
}

int stack_for(int requested, int tree_depth) {
  const int need = requested > tree_depth ? requested : tree_depth;
  if (need <= 32) return 32;
  if (need <= 64) return 64;
  return 256;
}

int check_launch_config(rtg_context* ctx, const rtg_launch_config& lc) {
  auto bad = [&](const char* m) { return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, m); };
  if (lc.threads_per_block != 64 && lc.threads_per_block != 128 && lc.threads_per_block != 256)
    return bad("threads_per_block must be 64, 128 or 256");
  if (lc.packet < 1 || lc.packet > 32) return bad("packet must be in 1..32");
  if (lc.stack_depth != 0 && lc.stack_depth != 32 && lc.stack_depth != 64 && lc.stack_depth != 256)
    return bad("stack_depth must be 0, 32, 64 or 256");
  if (lc.scheduling != RTG_SCHED_MEGAKERNEL && lc.scheduling != RTG_SCHED_WAVEFRONT &&
      lc.scheduling != RTG_SCHED_PLAIN)
    return bad("scheduling must be RTG_SCHED_MEGAKERNEL, RTG_SCHED_WAVEFRONT or RTG_SCHED_PLAIN");
  if (lc.leaf_tests != RTG_LEAF_IMMEDIATE && lc.leaf_tests != RTG_LEAF_POSTPONED)
    return bad("leaf_tests must be RTG_LEAF_IMMEDIATE or RTG_LEAF_POSTPONED");
  if (lc.stack_memory != RTG_STACK_AUTO && lc.stack_memory != RTG_STACK_LOCAL && lc.stack_memory != RTG_STACK_SHARED)
    return bad("stack_memory must be RTG_STACK_AUTO, RTG_STACK_LOCAL or RTG_STACK_SHARED");
  return RTG_OK;
}

bool use_wide(const rtg_context* ctx) {
  const Geometry& g = ctx->g;
  return g.wide_current && g.n_wnodes > 0 && g.wide_stack <= 256 && wants_wide(ctx);
}

int traversal_depth(const rtg_context* ctx) {
  return use_wide(ctx) ? std::max(ctx->g.depth, ctx->g.wide_stack) : ctx->g.depth;
}

SceneView scene_view(rtg_context* ctx) {
  const Geometry& g = ctx->g;
  SceneView s{};
  const bool wide = use_wide(ctx);
  s.wnodes = wide ? g.wnodes.p : nullptr;
  s.n_wnodes = wide ? g.n_wnodes : 0u;
  s.disc = g.disc.p;
  s.nd = (int32_t)g.nd;
  s.tri = g.tri.p;
  s.nt = (int32_t)g.nt;
  s.nodes = g.nodes.p;
  s.root = g.root;
  s.nb_ptr = g.nd > 0 ? g.nb_ptr.p : nullptr;
  s.nb_slot = g.nb_slot.p;
  s.sticking_field = ctx->sticking_field.p;
  // a valid query visits each node at most once (< 2 x primitives)
  const uint64_t automatic = std::min<uint64_t>(4 * (uint64_t)(g.nd + g.nt) + 64, 0xFFFFFFFFull);
  s.max_visits = (uint32_t)(ctx->visit_limit ? std::min<uint64_t>(ctx->visit_limit, automatic) : automatic);
  return s;
}

int launch_trace(rtg_context* ctx, const TraceParams& p_in, cudaStream_t st, int mode) {
  const rtg_launch_config& lc = ctx->lc;
  const int stack = stack_for(lc.stack_depth, traversal_depth(ctx));
  TraceParams p = p_in;
  p.packet = lc.packet;
  const uint64_t nrays = p.ray_end - p.ray_begin;
  // the window deposit has a kernel of its own (megakernel or plain schedule),
  // so has a trace that fills the segment log
  if (mode == kModeForward && p.window) mode = kModeWindow;
  if (mode == kModeForward && p.log.rec) mode = kModeLogged;
  if (mode == kModeForward && lc.scheduling == RTG_SCHED_WAVEFRONT) {
    // a job table of one entry
    Wavefront& wf = ctx->wf;
    RTG_TRY(dalloc(ctx, wf.one_job, 1, "wavefront job"));
    RTG_TRY(dalloc(ctx, wf.one_prefix, 2, "wavefront prefix"));
    const uint64_t pre[2] = {0, nrays};
    RTG_CUDA(ctx, cudaMemcpyAsync(wf.one_job.p, &p, sizeof p, cudaMemcpyHostToDevice, st));
    RTG_CUDA(ctx, cudaMemcpyAsync(wf.one_prefix.p, pre, sizeof pre, cudaMemcpyHostToDevice, st));
    RTG_CUDA(ctx, cudaStreamSynchronize(st));  // the host copies above are locals
    return launch_wavefront(ctx, p, wf.one_job.p, wf.one_prefix.p, 1, nrays, st, lc, traversal_depth(ctx));
  }
  int tpb = 128, sms = 0, per_sm = 0;
  PathKernel kern = pick_kernel(mode, lc.threads_per_block, stack, lc.leaf_tests == RTG_LEAF_POSTPONED,
                                shared_stack(ctx, lc), p.s.wnodes != nullptr, tpb);
  p.plain = (mode == kModeForward || mode == kModeWindow) && lc.scheduling == RTG_SCHED_PLAIN ? 1 : 0;
  RTG_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, 0));
  if (per_sm < 1) per_sm = 1;
  uint64_t blocks = (uint64_t)sms * per_sm;
  const uint64_t need = (nrays + tpb - 1) / tpb;
  if (need < blocks || p.plain) blocks = need > 0 ? need : 1;
  if (blocks > 0x7FFFFFFFull) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "too many rays for a plain launch");
  kern<<<(unsigned)blocks, tpb, 0, st>>>(p, nullptr, nullptr, 0);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

int launch_closest_hit(rtg_context* ctx, const float* d_rays, int64_t n, float tnear, int32_t* d_prim, float* d_t,
                       unsigned long long* d_errors, cudaStream_t st) {
  if (n <= 0) return RTG_OK;
  RTG_TRY(ensure_wide(ctx));
  SceneView s = scene_view(ctx);
  closest_hit_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(s, d_rays, n, tnear, d_prim, d_t, d_errors);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

}  // namespace rtg
