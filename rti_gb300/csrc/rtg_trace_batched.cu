// rtg_trace_batched.cu -- the path kernel over a job table (rtg_batch_run):
// lanes draw global ray ids over the concatenated ray ranges of all jobs.
#include "rtg_path.cuh"

namespace rtg {

namespace {

template <int TPB, bool POSTPONE>
PathKernel batched_kernel(int stack, bool shared, bool wide) {
  if (stack <= 32) return kernel_for<kModeForward, true, TPB, 32, POSTPONE>(shared, wide);
  if (stack <= 64) return kernel_for<kModeForward, true, TPB, 64, POSTPONE>(shared, wide);
  return kernel_for<kModeForward, true, TPB, 256, POSTPONE>(shared, wide);
}

template <int TPB>
PathKernel batched_kernel(int stack, bool postpone, bool shared, bool wide) {
  return postpone ? batched_kernel<TPB, true>(stack, shared, wide) : batched_kernel<TPB, false>(stack, shared, wide);
}

}  // namespace

int launch_trace_batched(rtg_context* ctx, const TraceParams& p0_in, const TraceParams* d_jobs,
                         const uint64_t* d_prefix, int njobs, uint64_t total_rays, cudaStream_t st,
                         const rtg_launch_config& lc, int tree_depth, bool wide) {
  if (lc.scheduling == RTG_SCHED_WAVEFRONT)
    return launch_wavefront(ctx, p0_in, d_jobs, d_prefix, njobs, total_rays, st, lc, tree_depth);
  const int stack = stack_for(lc.stack_depth, tree_depth);
  TraceParams p0 = p0_in;
  p0.packet = lc.packet;
  p0.plain = lc.scheduling == RTG_SCHED_PLAIN ? 1 : 0;
  int tpb = lc.threads_per_block, sms = 0, per_sm = 0;
  const bool pp = lc.leaf_tests == RTG_LEAF_POSTPONED;
  const bool sh = lc.stack_memory == RTG_STACK_SHARED;  // AUTO: local (the jobs' trees differ in size)
  PathKernel kern = tpb == 64    ? batched_kernel<64>(stack, pp, sh, wide)
                    : tpb == 256 ? batched_kernel<256>(stack, pp, sh, wide)
                                 : batched_kernel<128>(stack, pp, sh, wide);
  if (tpb != 64 && tpb != 256) tpb = 128;
  RTG_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, 0));
  if (per_sm < 1) per_sm = 1;
  uint64_t blocks = (uint64_t)sms * per_sm;
  const uint64_t need = (total_rays + tpb - 1) / tpb;
  if (need < blocks || p0.plain) blocks = need > 0 ? need : 1;
  if (blocks > 0x7FFFFFFFull) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "too many rays for a plain launch");
  kern<<<(unsigned)blocks, tpb, 0, st>>>(p0, d_jobs, d_prefix, njobs);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

}  // namespace rtg
