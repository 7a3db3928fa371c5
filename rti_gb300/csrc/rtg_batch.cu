// rtg_batch.cu -- many (surface, species) traces in one persistent launch.
//
// A batch holds jobs: a surface (an rtg_context with its LBVH, neighbour lists
// and sticking field), a configuration (sticking, source exponent, boundaries,
// re-emission, box) and a ray count and seed.  Each job has its own
// accumulators.  rtg_batch_run zeroes them, launches the batched path kernel
// once -- its lanes draw global ray ids over the concatenated ray ranges of
// all jobs, so the tail of one job overlaps the start of the next -- and
// computes each job's exposed areas; optionally the whole sequence is captured
// into a CUDA graph once and replayed.  rtg_batch_run_sequential traces the
// same jobs with one plain launch each (the comparison), with identical
// results: every job's paths use the job's own Philox stream (seed, job tag).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "rtg_internal.cuh"

namespace rtg {
namespace {

struct Job {
  rtg_context* scene = nullptr;
  rtg_config cfg{};
  uint64_t n_rays = 0, seed = 0;
  float box_lo[3] = {0, 0, 0}, box_hi[3] = {0, 0, 0};
  DBuf<double> acc;              // S1 | S2 | S3 | S4
  DBuf<unsigned long long> cnt;
  DBuf<float> areas;
  TraceParams p{};
  int64_t np = 0;        // primitives of the surface (the size of acc, cnt, areas)
  uint64_t version = 0;  // the context's version that p was made from
};

}  // namespace
}  // namespace rtg

struct rtg_batch {
  rtg_context aux;  // device, stream and error text of the batch (no geometry)
  std::vector<rtg::Job> jobs;
  rtg::DBuf<rtg::TraceParams> d_jobs;
  rtg::DBuf<uint64_t> d_prefix;
  uint64_t total_rays = 0;
  bool tables_ready = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int depth = 0;  // deepest LBVH among the jobs' surfaces
  bool wide = false;  // some job's context traces over its wide tree
};

using namespace rtg;

namespace {

void drop_graph(rtg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

int build_tables(rtg_batch* b) {
  rtg_context* ctx = &b->aux;
  const int n = (int)b->jobs.size();
  std::vector<TraceParams> h(n);
  std::vector<uint64_t> prefix(n + 1, 0);
  for (int j = 0; j < n; ++j) {
    h[j] = b->jobs[j].p;
    prefix[j + 1] = prefix[j] + b->jobs[j].n_rays;
  }
  b->total_rays = prefix[n];
  RTG_TRY(dalloc(ctx, b->d_jobs, (size_t)(n > 0 ? n : 1), "batch job table"));
  RTG_TRY(dalloc(ctx, b->d_prefix, (size_t)(n + 1), "batch prefix"));
  RTG_CUDA(ctx, cudaMemcpy(b->d_jobs.p, h.data(), n * sizeof(TraceParams), cudaMemcpyHostToDevice));
  RTG_CUDA(ctx, cudaMemcpy(b->d_prefix.p, prefix.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice));
  b->tables_ready = true;
  return RTG_OK;
}

// The batched sequence on stream st: zero, one launch over the ray ranges in
// `prefix` (total rays `total`), areas.
int enqueue_batched(rtg_batch* b, cudaStream_t st, const uint64_t* prefix, uint64_t total) {
  rtg_context* ctx = &b->aux;
  for (Job& j : b->jobs) {
    RTG_CUDA(ctx, cudaMemsetAsync(j.acc.p, 0, 4 * j.np * sizeof(double), st));
    RTG_CUDA(ctx, cudaMemsetAsync(j.cnt.p, 0, j.np * sizeof(unsigned long long), st));
  }
  RTG_CUDA(ctx, cudaMemsetAsync(ctx->d_tally, 0, sizeof(DevTally), st));
  TraceParams p0{};
  p0.tally = ctx->d_tally;
  p0.abort_flag = nullptr;
  if (total > 0)
    RTG_TRY(launch_trace_batched(ctx, p0, b->d_jobs.p, prefix, (int)b->jobs.size(), total, st, ctx->lc, b->depth,
                                 b->wide));
  for (Job& j : b->jobs) RTG_TRY(compute_areas_into(j.scene, st, j.box_lo, j.box_hi, j.areas.p));
  return RTG_OK;
}

// What a batch cannot trace (the batched kernel runs rti's neighbour deposit
// into FP64 accumulators only); nullptr when the context is fine.
const char* unsupported_mode(const rtg_context* scene) {
  if (scene->deposit_mode != RTG_DEPOSIT_NEIGHBORS) return "a batch traces the neighbour deposit only";
  if (scene->accum != RTG_ACCUM_FP64) return "a batch accumulates in FP64 only";
  return nullptr;
}

// The kernel parameters of job j from its context's current surface, into
// the job's own accumulators.
int prepare_job(rtg_batch* b, Job& j) {
  rtg_context* ctx = &b->aux;
  rtg_context* scene = j.scene;
  box_for(j.cfg, scene->g, j.box_lo, j.box_hi);
  TraceParams p;
  const int rc = prepare_trace_with(scene, j.cfg, j.box_lo, j.box_hi, 0, j.n_rays, j.seed, p);
  if (rc != RTG_OK) return set_error(ctx, rc, rtg_last_error(scene));
  p.s1 = j.acc.p;
  p.s2 = j.acc.p + j.np;
  p.s3 = j.acc.p + 2 * j.np;
  p.s4 = j.acc.p + 3 * j.np;
  p.cnt = j.cnt.p;
  p.tally = ctx->d_tally;
  p.abort_flag = nullptr;
  j.p = p;
  j.version = scene->version;
  return RTG_OK;
}

// Before a run: jobs whose context changed since their parameters were made
// (refit, new tree, sticking field, visit limit, a new upload) are prepared
// again, and the job table and the captured graph are rebuilt; a job whose
// surface no longer has the same number of primitives fails the run.
int refresh_jobs(rtg_batch* b) {
  rtg_context* ctx = &b->aux;
  bool changed = false;
  for (size_t i = 0; i < b->jobs.size(); ++i) {
    Job& j = b->jobs[i];
    const rtg_context* scene = j.scene;
    if (scene->version == j.version) continue;
    if (scene->g.nd + scene->g.nt != j.np || !scene->g.nodes.p)
      return set_error(ctx, RTG_ERR_INVALID_ARGUMENT,
                       "job " + std::to_string(i) + ": its surface no longer has the same number of primitives");
    if (const char* why = unsupported_mode(scene))
      return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "job " + std::to_string(i) + ": " + why);
    RTG_TRY(prepare_job(b, j));
    changed = true;
  }
  if (changed) {
    b->depth = 0;
    b->wide = false;
    for (const Job& j : b->jobs) {
      b->depth = std::max(b->depth, traversal_depth(j.scene));
      b->wide = b->wide || use_wide(j.scene);
    }
    b->tables_ready = false;
    drop_graph(b);
  }
  return RTG_OK;
}

}  // namespace

extern "C" {

static int rtg_batch_create_body(rtg_batch** out, int device);

int rtg_batch_create(rtg_batch** out, int device) {
  return rtg::host_guard(nullptr, [&] { return rtg_batch_create_body(out, device); });
}

static int rtg_batch_create_body(rtg_batch** out, int device) {
  if (!out) return RTG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return RTG_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return RTG_ERR_INVALID_ARGUMENT;
  rtg_batch* b = new rtg_batch();
  b->aux.device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->aux.stream, cudaStreamNonBlocking) !=
                                                  cudaSuccess ||
      cudaMalloc((void**)&b->aux.d_tally, sizeof(DevTally)) != cudaSuccess || cudaEventCreate(&b->ev0) != cudaSuccess ||
      cudaEventCreate(&b->ev1) != cudaSuccess) {
    cudaGetLastError();
    if (b->aux.d_tally) cudaFree(b->aux.d_tally);
    if (b->aux.stream) cudaStreamDestroy(b->aux.stream);
    delete b;
    return RTG_ERR_CUDA;
  }
  *out = b;
  return RTG_OK;
}

int rtg_batch_destroy(rtg_batch* b) {
  if (!b) return RTG_OK;
  cudaSetDevice(b->aux.device);
  if (b->aux.stream) cudaStreamSynchronize(b->aux.stream);
  drop_graph(b);
  for (Job& j : b->jobs) {
    dfree(j.acc);
    dfree(j.cnt);
    dfree(j.areas);
  }
  dfree(b->d_jobs);
  dfree(b->d_prefix);
  if (b->aux.d_tally) cudaFree(b->aux.d_tally);
  b->aux.d_tally = nullptr;
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->aux.stream) cudaStreamDestroy(b->aux.stream);
  b->aux.stream = nullptr;
  delete b;
  return RTG_OK;
}

const char* rtg_batch_last_error(const rtg_batch* b) { return b ? b->aux.err.c_str() : "null batch"; }

static int rtg_batch_add_body(rtg_batch* b, rtg_context* scene, const rtg_config* cfg, uint64_t n_rays, uint64_t seed,
                  int32_t* job_out);

int rtg_batch_add(rtg_batch* b, rtg_context* scene, const rtg_config* cfg, uint64_t n_rays, uint64_t seed,
                  int32_t* job_out) {
  return rtg::host_guard(b ? &b->aux : nullptr, [&] { return rtg_batch_add_body(b, scene, cfg, n_rays, seed, job_out); });
}

static int rtg_batch_add_body(rtg_batch* b, rtg_context* scene, const rtg_config* cfg, uint64_t n_rays, uint64_t seed,
                  int32_t* job_out) {
  if (!b || !scene) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = &b->aux;
  if (scene->device != ctx->device) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "scene is on another device");
  if (scene->g.nd + scene->g.nt == 0 || !scene->g.nodes.p)
    return set_error(ctx, RTG_ERR_NO_GEOMETRY, "scene has no geometry");
  if (const char* why = unsupported_mode(scene)) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, why);
  if (b->jobs.size() >= 0x7FFFFFFF) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "too many jobs");
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  Job j;
  j.scene = scene;
  j.cfg = cfg ? *cfg : scene->cfg;
  if (check_config(ctx, j.cfg) != RTG_OK) return RTG_ERR_INVALID_ARGUMENT;
  j.cfg.job = (uint32_t)b->jobs.size();  // a Philox stream of its own
  j.n_rays = n_rays;
  j.seed = seed;
  j.np = scene->g.nd + scene->g.nt;
  int rc = dalloc(ctx, j.acc, (size_t)(4 * j.np), "batch accumulators");
  if (rc == RTG_OK) rc = dalloc(ctx, j.cnt, (size_t)j.np, "batch counts");
  if (rc == RTG_OK) rc = dalloc(ctx, j.areas, (size_t)j.np, "batch areas");
  if (rc == RTG_OK) rc = prepare_job(b, j);
  if (rc != RTG_OK) {
    dfree(j.acc);
    dfree(j.cnt);
    dfree(j.areas);
    return rc;
  }
  b->jobs.push_back(j);
  if (traversal_depth(scene) > b->depth) b->depth = traversal_depth(scene);
  if (use_wide(scene)) b->wide = true;
  b->tables_ready = false;
  drop_graph(b);
  if (job_out) *job_out = (int32_t)(b->jobs.size() - 1);
  return RTG_OK;
}

int rtg_batch_num_jobs(const rtg_batch* b, int32_t* n) {
  if (!b || !n) return RTG_ERR_INVALID_ARGUMENT;
  *n = (int32_t)b->jobs.size();
  return RTG_OK;
}

int rtg_batch_run(rtg_batch* b, int use_graph, void* stream) {
  if (!b) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = &b->aux;
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  RTG_TRY(refresh_jobs(b));
  if (!b->tables_ready) RTG_TRY(build_tables(b));
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  RTG_CUDA(ctx, cudaEventRecord(b->ev0, st));
  if (!use_graph || ctx->lc.scheduling == RTG_SCHED_WAVEFRONT) {  // a host-driven wavefront is not captured
    RTG_TRY(enqueue_batched(b, st, b->d_prefix.p, b->total_rays));
  } else {
    if (!b->exec) {
      // capture on the batch's own stream, then replay on `st`
      cudaStream_t cs = ctx->stream;
      RTG_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue_batched(b, cs, b->d_prefix.p, b->total_rays);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(cs, &g);
      if (rc != RTG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (e != cudaSuccess) return check_cuda(ctx, e, "graph capture");
      b->graph = g;
      RTG_CUDA(ctx, cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    RTG_CUDA(ctx, cudaGraphLaunch(b->exec, st));
  }
  RTG_CUDA(ctx, cudaEventRecord(b->ev1, st));
  return RTG_OK;
}

static int rtg_batch_run_sequential_body(rtg_batch* b, void* stream);

int rtg_batch_run_sequential(rtg_batch* b, void* stream) {
  return rtg::host_guard(b ? &b->aux : nullptr, [&] { return rtg_batch_run_sequential_body(b, stream); });
}

static int rtg_batch_run_sequential_body(rtg_batch* b, void* stream) {
  if (!b) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = &b->aux;
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  RTG_TRY(refresh_jobs(b));
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  RTG_CUDA(ctx, cudaEventRecord(b->ev0, st));
  RTG_CUDA(ctx, cudaMemsetAsync(ctx->d_tally, 0, sizeof(DevTally), st));
  for (Job& j : b->jobs) {
    RTG_CUDA(ctx, cudaMemsetAsync(j.acc.p, 0, 4 * j.np * sizeof(double), st));
    RTG_CUDA(ctx, cudaMemsetAsync(j.cnt.p, 0, j.np * sizeof(unsigned long long), st));
    RTG_CUDA(ctx, cudaMemsetAsync(&ctx->d_tally->next_ray, 0, sizeof(unsigned long long), st));
    if (j.n_rays > 0) {
      const int rc = launch_trace(j.scene, j.p, st, kModeForward);
      if (rc != RTG_OK) return set_error(ctx, rc, std::string("job trace: ") + j.scene->err);
    }
    RTG_TRY(compute_areas_into(j.scene, st, j.box_lo, j.box_hi, j.areas.p));
  }
  RTG_CUDA(ctx, cudaEventRecord(b->ev1, st));
  return RTG_OK;
}

int rtg_batch_synchronize(rtg_batch* b, double* elapsed_ms) {
  if (!b) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = &b->aux;
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  RTG_CUDA(ctx, cudaEventSynchronize(b->ev1));
  float ms = 0.0f;
  RTG_CUDA(ctx, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  if (elapsed_ms) *elapsed_ms = ms;
  DevTally t;
  RTG_CUDA(ctx, cudaMemcpy(&t, ctx->d_tally, sizeof t, cudaMemcpyDeviceToHost));
  if (t.errors) return set_error(ctx, RTG_ERR_BUDGET, "a device-side traversal limit was reached");
  return RTG_OK;
}

int rtg_batch_get_results(rtg_batch* b, int32_t job, double* s1, uint64_t* counts, float* areas) {
  if (!b || job < 0 || job >= (int32_t)b->jobs.size()) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = &b->aux;
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  RTG_CUDA(ctx, cudaDeviceSynchronize());
  Job& j = b->jobs[(size_t)job];
  const int64_t np = j.np;
  if (s1) RTG_CUDA(ctx, cudaMemcpy(s1, j.acc.p, np * sizeof(double), cudaMemcpyDeviceToHost));
  if (counts) RTG_CUDA(ctx, cudaMemcpy(counts, j.cnt.p, np * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  if (areas) RTG_CUDA(ctx, cudaMemcpy(areas, j.areas.p, np * sizeof(float), cudaMemcpyDeviceToHost));
  return RTG_OK;
}

int rtg_batch_get_tally(rtg_batch* b, rtg_tally* out) {
  if (!b || !out) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = &b->aux;
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  RTG_CUDA(ctx, cudaDeviceSynchronize());
  DevTally t;
  RTG_CUDA(ctx, cudaMemcpy(&t, ctx->d_tally, sizeof t, cudaMemcpyDeviceToHost));
  std::memset(out, 0, sizeof *out);
  uint64_t rays = 0;
  for (const Job& j : b->jobs) rays += j.n_rays;
  out->num_rays = rays;
  out->hitc = t.hitc;
  out->nonhitc = t.nonhitc;
  out->total = t.total;
  out->segments = t.segments;
  out->truncated = t.truncated;
  out->nb_deposits = t.nb_deposits;
  out->errors = t.errors;
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, b->ev0, b->ev1) == cudaSuccess) out->trace_ms = ms;
  cudaGetLastError();
  return RTG_OK;
}

int rtg_batch_set_launch_config(rtg_batch* b, const rtg_launch_config* lc) {
  if (!b || !lc) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(check_launch_config(&b->aux, *lc));
  if (std::memcmp(lc, &b->aux.lc, sizeof *lc) != 0) drop_graph(b);
  b->aux.lc = *lc;
  return RTG_OK;
}

int rtg_batch_get_launch_config(const rtg_batch* b, rtg_launch_config* lc) {
  if (!b || !lc) return RTG_ERR_INVALID_ARGUMENT;
  *lc = b->aux.lc;
  return RTG_OK;
}

static int rtg_batch_autotune_body(rtg_batch* b, double fraction, rtg_launch_config* best, double* best_rays_per_s);

int rtg_batch_autotune(rtg_batch* b, double fraction, rtg_launch_config* best, double* best_rays_per_s) {
  return rtg::host_guard(b ? &b->aux : nullptr, [&] { return rtg_batch_autotune_body(b, fraction, best, best_rays_per_s); });
}

static int rtg_batch_autotune_body(rtg_batch* b, double fraction, rtg_launch_config* best, double* best_rays_per_s) {
  if (!b || !(fraction > 0.0 && fraction <= 1.0)) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = &b->aux;
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  RTG_TRY(refresh_jobs(b));
  if (!b->tables_ready) RTG_TRY(build_tables(b));
  const int n = (int)b->jobs.size();
  if (n == 0) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "empty batch");
  // the first fraction of every job's rays
  std::vector<uint64_t> prefix(n + 1, 0);
  for (int j = 0; j < n; ++j) {
    const uint64_t r = b->jobs[j].n_rays;
    uint64_t s = (uint64_t)(r * fraction);
    if (s == 0 && r > 0) s = 1;
    prefix[j + 1] = prefix[j] + s;
  }
  const uint64_t total = prefix[n];
  DBuf<uint64_t> dp;
  RTG_TRY(dalloc(ctx, dp, (size_t)(n + 1), "sample prefix"));
  cudaStream_t st = ctx->stream;
  int rc = check_cuda(ctx, cudaMemcpy(dp.p, prefix.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice),
                      "sample prefix");
  const rtg_launch_config keep = ctx->lc;
  auto run = [&](const rtg_launch_config& lc, float& ms) -> int {
    ctx->lc = lc;
    RTG_CUDA(ctx, cudaEventRecord(b->ev0, st));
    RTG_TRY(enqueue_batched(b, st, dp.p, total));
    RTG_CUDA(ctx, cudaEventRecord(b->ev1, st));
    RTG_CUDA(ctx, cudaEventSynchronize(b->ev1));
    RTG_CUDA(ctx, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    return RTG_OK;
  };
  std::vector<rtg_launch_config> cand;
  // no wavefront candidates (see rtg_autotune)
  for (int sched : {RTG_SCHED_MEGAKERNEL, RTG_SCHED_PLAIN})
    for (int tpb : {64, 128, 256})
      for (int packet : {1, 8, 32})
        for (int stack : {0, 256})
          for (int leaf : {RTG_LEAF_IMMEDIATE, RTG_LEAF_POSTPONED}) {
            if (sched == RTG_SCHED_PLAIN && (packet != 1 || tpb == 64 || stack != 0)) continue;
            if (stack == 256 && stack_for(0, b->depth) == 256) continue;
            if (leaf == RTG_LEAF_POSTPONED && packet == 32) continue;
            cand.push_back(rtg_launch_config{tpb, packet, stack, sched, leaf, RTG_STACK_AUTO});
          }
  std::vector<float> tms(cand.size(), 0.0f);
  float ms = 0.0f;
  for (size_t i = 0; i < cand.size() && rc == RTG_OK; ++i) {
    rc = run(cand[i], ms);
    if (rc == RTG_OK) rc = run(cand[i], tms[i]);
  }
  std::vector<size_t> order(cand.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return tms[x] < tms[y]; });
  for (int r = 0; r < 2 && rc == RTG_OK; ++r)
    for (size_t q = 0; q < order.size() && q < 3 && rc == RTG_OK; ++q) {
      rc = run(cand[order[q]], ms);
      if (rc == RTG_OK && ms < tms[order[q]]) tms[order[q]] = ms;
    }
  // the three fastest with their stacks in shared memory, best of two
  for (size_t q = 0; q < order.size() && q < 3 && rc == RTG_OK; ++q) {
    rtg_launch_config alt = cand[order[q]];
    if (alt.scheduling == RTG_SCHED_WAVEFRONT) continue;
    alt.stack_memory = RTG_STACK_SHARED;
    float m1 = 0.0f, m2 = 0.0f;
    rc = run(alt, m1);
    if (rc == RTG_OK) rc = run(alt, m2);
    if (rc == RTG_OK) {
      cand.push_back(alt);
      tms.push_back(std::min(m1, m2));
    }
  }
  dfree(dp);
  if (rc != RTG_OK) {
    ctx->lc = keep;
    return rc;
  }
  size_t bi = 0;
  for (size_t i = 1; i < cand.size(); ++i)
    if (tms[i] < tms[bi]) bi = i;
  if (std::memcmp(&cand[bi], &keep, sizeof keep) != 0) drop_graph(b);
  ctx->lc = cand[bi];
  if (best) *best = cand[bi];
  if (best_rays_per_s) *best_rays_per_s = tms[bi] > 0.0f ? total / (tms[bi] * 1e-3) : 0.0;
  return RTG_OK;
}

}  // extern "C"
