// rtg_api.cu -- the C ABI of librtg (declared in include/rtg.h).
//
// A context owns one GPU's copy of a surface: primitive data by id and in
// LBVH slot order, the LBVH, the neighbour lists, the sticking field and the
// per-primitive accumulators.  rtg_trace enqueues the zeroing of the
// accumulators, the persistent path kernel and the exposed-area kernel on one
// stream, the span that rti times in tracer::run (tracer.hpp:122-286).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "rtg_internal.cuh"

namespace rtg {

int set_error(rtg_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int check_cuda(rtg_context* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RTG_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();
  return set_error(ctx, e == cudaErrorMemoryAllocation ? RTG_ERR_OUT_OF_MEMORY : RTG_ERR_CUDA, m);
}

namespace {

int use_device(rtg_context* ctx) {
  RTG_CUDA(ctx, cudaSetDevice(ctx->device));
  return RTG_OK;
}

bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

int alloc_results(rtg_context* ctx) {
  const int64_t np = ctx->g.nd + ctx->g.nt;
  const size_t n = (size_t)(np > 0 ? np : 1);
  RTG_TRY(dalloc(ctx, ctx->acc, 4 * n, "accumulators"));
  RTG_TRY(dalloc(ctx, ctx->cnt, n, "hit counts"));
  RTG_TRY(dalloc(ctx, ctx->areas, n, "exposed areas"));
  RTG_TRY(dalloc(ctx, ctx->est, n, "estimates"));
  RTG_CUDA(ctx, cudaMemsetAsync(ctx->acc.p, 0, 4 * n * sizeof(double), ctx->stream));
  RTG_CUDA(ctx, cudaMemsetAsync(ctx->cnt.p, 0, n * sizeof(unsigned long long), ctx->stream));
  ctx->traced = false;
  ctx->finalized = false;
  return RTG_OK;
}

// The trace box: explicit, or rti's rule (device.hpp:86-92, 225-237,
// point_cloud_disc_geometry.hpp:83-87): x/y = centre extents, z from the
// lowest centre to the highest centre + 2 r_max (source plane).
}  // namespace

void box_for(const rtg_config& c, const Geometry& g, float* box_lo, float* box_hi) {
  if (c.box_mode == RTG_BOX_EXPLICIT) {
    for (int a = 0; a < 3; ++a) {
      box_lo[a] = c.box_lo[a];
      box_hi[a] = c.box_hi[a];
    }
    return;
  }
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  if (g.nd > 0)
    for (int a = 0; a < 3; ++a) {
      lo[a] = g.cmin[a];
      hi[a] = g.cmax[a];
    }
  if (g.nt > 0)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], g.tri_min[a]);
      hi[a] = std::max(hi[a], g.tri_max[a]);
    }
  float top = hi[2];
  if (g.nd > 0) top = (hi[2] + g.rmax) + g.rmax;
  for (int a = 0; a < 3; ++a) {
    box_lo[a] = lo[a];
    box_hi[a] = hi[a];
  }
  box_hi[2] = top;
}

namespace {

void resolve_box(rtg_context* ctx) { box_for(ctx->cfg, ctx->g, ctx->box_lo, ctx->box_hi); }

// ---- upload: the host arrays are copied as they are and checked and
// converted on the device; one small read-back carries the outcome ----

// Bounds and first offending index of an upload.
struct UploadCheck {
  float lo[3], hi[3];           // disc centres, or the vertices the triangles use
  float rmax;                   // largest disc radius
  unsigned long long bad;       // lowest disc / vertex index that fails its check, or ~0
  unsigned long long bad_tri;   // lowest triangle with an index out of range, or ~0
};

__device__ __forceinline__ void atomic_min_f(float* a, float v) {  // order of IEEE bits as integers
  if (__float_as_int(v) >= 0) atomicMin((int*)a, __float_as_int(v));
  else atomicMax((unsigned int*)a, __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* a, float v) {
  if (__float_as_int(v) >= 0) atomicMax((int*)a, __float_as_int(v));
  else atomicMin((unsigned int*)a, __float_as_uint(v));
}

// Warp minima/maxima of (x, y, z), then one atomic per warp.
__device__ __forceinline__ void bounds_add(UploadCheck* c, float x, float y, float z, bool valid) {
  float l[3] = {valid ? x : FLT_MAX, valid ? y : FLT_MAX, valid ? z : FLT_MAX};
  float h[3] = {valid ? x : -FLT_MAX, valid ? y : -FLT_MAX, valid ? z : -FLT_MAX};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      l[a] = fminf(l[a], __shfl_xor_sync(0xFFFFFFFFu, l[a], o));
      h[a] = fmaxf(h[a], __shfl_xor_sync(0xFFFFFFFFu, h[a], o));
    }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; ++a) {
      atomic_min_f(&c->lo[a], l[a]);
      atomic_max_f(&c->hi[a], h[a]);
    }
}

__global__ void check_init_kernel(UploadCheck* c) {
  for (int a = 0; a < 3; ++a) {
    c->lo[a] = FLT_MAX;
    c->hi[a] = -FLT_MAX;
  }
  c->rmax = 0.0f;
  c->bad = ~0ull;
  c->bad_tri = ~0ull;
}

__device__ __forceinline__ bool finite3_d(float x, float y, float z) {
  return isfinite(x) && isfinite(y) && isfinite(z);
}

// Disc i: finite centre, normal and radius, radius > 0, unit normal (within
// 1e-3); writes (centre, r) and (normal, 0).  Grid-stride; whole warps.
__global__ void disc_check_kernel(const float* __restrict__ pts, const float* __restrict__ nrm,
                                  const float* __restrict__ rad, int64_t n, float4* __restrict__ cr,
                                  float4* __restrict__ nn, UploadCheck* c) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t i = base + threadIdx.x;
    const bool in = i < n;
    float p[3] = {0, 0, 0}, q[3] = {0, 0, 1}, r = 1.0f;
    if (in)
      for (int a = 0; a < 3; ++a) {
        p[a] = pts[3 * i + a];
        q[a] = nrm[3 * i + a];
      }
    if (in) r = rad[i];
    bool ok = finite3_d(p[0], p[1], p[2]) && finite3_d(q[0], q[1], q[2]) && isfinite(r) && r > 0.0f;
    if (ok) {
      const float l2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
      ok = fabsf(sqrtf(l2) - 1.0f) <= 1e-3f;
    }
    if (in && !ok) atomicMin(&c->bad, (unsigned long long)i);
    if (in) {
      cr[i] = make_float4(p[0], p[1], p[2], r);
      nn[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    const bool v = in && ok;
    bounds_add(c, p[0], p[1], p[2], v);
    float rm = v ? r : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rm = fmaxf(rm, __shfl_xor_sync(0xFFFFFFFFu, rm, o));
    if ((threadIdx.x & 31) == 0) atomic_max_f(&c->rmax, rm);
  }
}

// Vertex i: finite; writes (x, y, z, 0).
__global__ void vertex_check_kernel(const float* __restrict__ v, int64_t nv, float4* __restrict__ out,
                                    UploadCheck* c) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
    const float x = v[3 * i], y = v[3 * i + 1], z = v[3 * i + 2];
    if (!finite3_d(x, y, z)) atomicMin(&c->bad, (unsigned long long)i);
    out[i] = make_float4(x, y, z, 0.0f);
  }
}

// Triangle t: its three indices below nv; bounds over the vertices it uses.
__global__ void triangle_check_kernel(const uint32_t* __restrict__ idx, int64_t nt, int64_t nv,
                                      const float4* __restrict__ vert, UploadCheck* c) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nt; base += stride) {
    const int64_t t = base + threadIdx.x;
    const bool in = t < nt;
    for (int k = 0; k < 3; ++k) {
      const uint32_t q = in ? idx[3 * t + k] : 0u;
      const bool ok = in && (int64_t)q < nv;
      if (in && !ok) atomicMin(&c->bad_tri, (unsigned long long)t);
      float4 p = make_float4(0, 0, 0, 0);
      if (ok) p = vert[q];
      bounds_add(c, p.x, p.y, p.z, ok);
    }
  }
}

unsigned grid_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 4096));
}

// An upload checked on the device and not yet part of the context.
struct Staged {
  int64_t nd = 0, nv = 0, nt = 0;
  bool discs = false, triangles = false;
  UploadCheck hd{}, ht{};
  DBuf<float4> cr, nn, v4;
  DBuf<uint32_t> ix;
};

void release(Staged& sg, cudaStream_t st) {
  tfree(sg.cr, st);
  tfree(sg.nn, st);
  tfree(sg.v4, st);
  tfree(sg.ix, st);
}

void check_reset(UploadCheck& h) {
  for (int a = 0; a < 3; ++a) {
    h.lo[a] = FLT_MAX;
    h.hi[a] = -FLT_MAX;
  }
  h.rmax = 0.0f;
  h.bad = ~0ull;
  h.bad_tri = ~0ull;
}

// Copies n discs to the device, converts and checks them; the outcome is
// read back (one synchronisation).  Leaves the context untouched.
int stage_discs(rtg_context* ctx, const float* pts, const float* nrm, const float* rad, int64_t n, Staged& sg) {
  if (n < 0 || (n > 0 && (!pts || !nrm || !rad)))
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "discs: null array or negative count");
  cudaStream_t st = ctx->stream;
  sg.discs = true;
  sg.nd = n;
  check_reset(sg.hd);
  if (n == 0) return RTG_OK;
  DBuf<float> raw;
  DBuf<UploadCheck> chk;
  int rc = talloc(ctx, raw, (size_t)(7 * n), st, "disc upload");
  if (rc == RTG_OK) rc = talloc(ctx, sg.cr, (size_t)n, st, "disc upload");
  if (rc == RTG_OK) rc = talloc(ctx, sg.nn, (size_t)n, st, "disc upload");
  if (rc == RTG_OK) rc = talloc(ctx, chk, 1, st, "disc upload");
  cudaError_t e = cudaSuccess;
  if (rc == RTG_OK) e = cudaMemcpyAsync(raw.p, pts, 3 * n * sizeof(float), cudaMemcpyHostToDevice, st);
  if (rc == RTG_OK && e == cudaSuccess)
    e = cudaMemcpyAsync(raw.p + 3 * n, nrm, 3 * n * sizeof(float), cudaMemcpyHostToDevice, st);
  if (rc == RTG_OK && e == cudaSuccess)
    e = cudaMemcpyAsync(raw.p + 6 * n, rad, n * sizeof(float), cudaMemcpyHostToDevice, st);
  if (rc == RTG_OK && e == cudaSuccess) {
    check_init_kernel<<<1, 1, 0, st>>>(chk.p);
    disc_check_kernel<<<grid_for(n), 256, 0, st>>>(raw.p, raw.p + 3 * n, raw.p + 6 * n, n, sg.cr.p, sg.nn.p,
                                                      chk.p);
    e = cudaGetLastError();
  }
  if (rc == RTG_OK && e == cudaSuccess) e = cudaMemcpyAsync(&sg.hd, chk.p, sizeof sg.hd, cudaMemcpyDeviceToHost, st);
  if (rc == RTG_OK && e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (rc == RTG_OK && e != cudaSuccess) rc = check_cuda(ctx, e, "disc upload");
  tfree(raw, st);
  tfree(chk, st);
  if (rc == RTG_OK && sg.hd.bad != ~0ull) {  // the message of the first offending disc, as the host sees it
    const int64_t i = (int64_t)sg.hd.bad;
    const float* q = nrm + 3 * i;
    const bool finite = finite3(pts + 3 * i) && finite3(q) && std::isfinite(rad[i]) && rad[i] > 0.0f;
    rc = set_error(ctx, RTG_ERR_INVALID_ARGUMENT,
                   "disc " + std::to_string(i) +
                       (finite ? ": normal is not unit length" : ": non-finite value or radius <= 0"));
  }
  return rc;
}

// The same for nv vertices and nt index triples.
int stage_triangles(rtg_context* ctx, const float* vertices, const uint32_t* indices, int64_t nv, int64_t nt,
                    Staged& sg) {
  if (nv < 0 || nt < 0 || (nt > 0 && (!vertices || !indices)) || (nv > 0 && !vertices))
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "triangles: null array or negative count");
  cudaStream_t st = ctx->stream;
  sg.triangles = true;
  sg.nv = nv;
  sg.nt = nt;
  check_reset(sg.ht);
  if (nv == 0 && nt == 0) return RTG_OK;
  DBuf<float> raw;
  DBuf<UploadCheck> chk;
  int rc = talloc(ctx, chk, 1, st, "triangle upload");
  if (rc == RTG_OK && nv > 0) rc = talloc(ctx, raw, (size_t)(3 * nv), st, "triangle upload");
  if (rc == RTG_OK && nv > 0) rc = talloc(ctx, sg.v4, (size_t)nv, st, "triangle upload");
  if (rc == RTG_OK && nt > 0) rc = talloc(ctx, sg.ix, (size_t)(3 * nt), st, "triangle upload");
  cudaError_t e = cudaSuccess;
  if (rc == RTG_OK && nv > 0) e = cudaMemcpyAsync(raw.p, vertices, 3 * nv * sizeof(float), cudaMemcpyHostToDevice, st);
  if (rc == RTG_OK && nt > 0 && e == cudaSuccess)
    e = cudaMemcpyAsync(sg.ix.p, indices, 3 * nt * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (rc == RTG_OK && e == cudaSuccess) {
    check_init_kernel<<<1, 1, 0, st>>>(chk.p);
    if (nv > 0) vertex_check_kernel<<<grid_for(nv), 256, 0, st>>>(raw.p, nv, sg.v4.p, chk.p);
    if (nt > 0) triangle_check_kernel<<<grid_for(nt), 256, 0, st>>>(sg.ix.p, nt, nv, sg.v4.p, chk.p);
    e = cudaGetLastError();
  }
  if (rc == RTG_OK && e == cudaSuccess) e = cudaMemcpyAsync(&sg.ht, chk.p, sizeof sg.ht, cudaMemcpyDeviceToHost, st);
  if (rc == RTG_OK && e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (rc == RTG_OK && e != cudaSuccess) rc = check_cuda(ctx, e, "triangle upload");
  tfree(raw, st);
  tfree(chk, st);
  if (rc == RTG_OK && sg.ht.bad != ~0ull)
    rc = set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "vertex " + std::to_string(sg.ht.bad) + " is not finite");
  else if (rc == RTG_OK && sg.ht.bad_tri != ~0ull)
    rc = set_error(ctx, RTG_ERR_INVALID_ARGUMENT,
                   "triangle " + std::to_string(sg.ht.bad_tri) + ": vertex index out of range");
  return rc;
}

// Makes a checked upload the context's surface data (by id).
int commit(rtg_context* ctx, const Staged& sg) {
  Geometry& g = ctx->g;
  cudaStream_t st = ctx->stream;
  if (sg.discs) {
    const int64_t n = sg.nd;
    g.nd = n;
    for (int a = 0; a < 3; ++a) {
      g.cmin[a] = sg.hd.lo[a];
      g.cmax[a] = sg.hd.hi[a];
    }
    g.rmax = sg.hd.rmax;
    RTG_TRY(dalloc(ctx, g.disc_cr_by_id, (size_t)(n > 0 ? n : 1), "discs"));
    RTG_TRY(dalloc(ctx, g.disc_n_by_id, (size_t)(n > 0 ? n : 1), "disc normals"));
    if (n > 0) {
      RTG_CUDA(ctx, cudaMemcpyAsync(g.disc_cr_by_id.p, sg.cr.p, n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
      RTG_CUDA(ctx, cudaMemcpyAsync(g.disc_n_by_id.p, sg.nn.p, n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    }
  }
  if (sg.triangles) {
    g.nt = sg.nt;
    g.nv = sg.nv;
    for (int a = 0; a < 3; ++a) {
      g.tri_min[a] = sg.ht.lo[a];
      g.tri_max[a] = sg.ht.hi[a];
    }
    RTG_TRY(dalloc(ctx, g.tri_v, (size_t)(sg.nv > 0 ? sg.nv : 1), "vertices"));
    RTG_TRY(dalloc(ctx, g.tri_idx, (size_t)(3 * (sg.nt > 0 ? sg.nt : 1)), "triangle indices"));
    if (sg.nv > 0)
      RTG_CUDA(ctx, cudaMemcpyAsync(g.tri_v.p, sg.v4.p, sg.nv * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    if (sg.nt > 0)
      RTG_CUDA(ctx, cudaMemcpyAsync(g.tri_idx.p, sg.ix.p, 3 * sg.nt * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  }
  return RTG_OK;
}

}  // namespace

void drop_surface(rtg_context* ctx) {
  cudaStreamSynchronize(ctx->stream);
  Geometry& g = ctx->g;
  dfree(g.disc_cr_by_id); dfree(g.disc_n_by_id); dfree(g.tri_v); dfree(g.tri_idx);
  dfree(g.disc); dfree(g.tri); dfree(g.nodes);
  dfree(g.leaf_ref); dfree(g.leaf_prim); dfree(g.parent); dfree(g.prim_lo); dfree(g.prim_hi);
  dfree(g.refit_flags); dfree(g.nb_ptr); dfree(g.nb_idx); dfree(g.nb_slot); dfree(g.disc_slot);
  dfree(g.wnodes);
  dfree(g.wnodes);
  g.n_wnodes = 0;
  g.wide_stack = 0;
  g.wide_current = false;
  dfree(ctx->sticking_field);
  g.nd = g.nt = g.nv = 0;
  g.nb_nnz = 0;
  g.root = 0;
  g.depth = 0;
  ctx->traced = false;
  ctx->finalized = false;
  ++ctx->version;
}

// Checks the context and fills the kernel parameters of a trace (or of its
// adjoint replay) of source rays [ray_begin, ray_end) under configuration c
// and trace box box_lo/box_hi; accumulators and counters are the context's.
int prepare_trace_with(rtg_context* ctx, const rtg_config& c, const float* box_lo, const float* box_hi,
                       uint64_t ray_begin, uint64_t ray_end, uint64_t seed, TraceParams& p) {
  if (ray_end < ray_begin) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "ray_end < ray_begin");
  const int64_t np = ctx->g.nd + ctx->g.nt;
  if (np == 0 || !ctx->g.nodes.p) return set_error(ctx, RTG_ERR_NO_GEOMETRY, "no geometry uploaded");
  RTG_TRY(use_device(ctx));
  for (int a = 0; a < 2; ++a)
    if (!(box_lo[a] < box_hi[a]))
      return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "degenerate x/y box (all discs on one line?)");
  *ctx->h_abort = 0;
  p = TraceParams{};
  RTG_TRY(ensure_wide(ctx));
  p.s = scene_view(ctx);
  p.s1 = ctx->acc.p;
  p.s2 = ctx->acc.p + np;
  p.s3 = ctx->acc.p + 2 * np;
  p.s4 = ctx->acc.p + 3 * np;
  p.cnt = ctx->cnt.p;
  p.tally = ctx->d_tally;
  p.abort_flag = ctx->d_abort;
  p.ray_begin = ray_begin;
  p.ray_end = ray_end;
  p.seed = seed;
  for (int a = 0; a < 3; ++a) {
    p.box_lo[a] = box_lo[a];
    p.box_hi[a] = box_hi[a];
  }
  p.src_lo[0] = box_lo[0];
  p.src_lo[1] = box_lo[1];
  p.src_hi[0] = box_hi[0];
  p.src_hi[1] = box_hi[1];
  p.tnear = c.tnear;
  p.sticking = c.sticking;
  p.source_exponent = c.source_exponent;
  p.source_ee = 2.0f / (c.source_exponent + 1.0f);
  p.specular_fraction = c.specular_fraction;
  p.roulette_threshold = c.roulette_threshold;
  p.roulette_weight = c.roulette_weight;
  p.x_periodic = c.x_bound == RTG_BOUND_PERIODIC;
  p.y_periodic = c.y_bound == RTG_BOUND_PERIODIC;
  p.reflection = c.reflection;
  p.max_segments = c.max_segments;
  p.job = c.job;
  p.adj_inv_n1 = 1.0 / ((double)c.source_exponent + 1.0);
  p.fixed_s1 = ctx->accum == RTG_ACCUM_FIXED ? 1 : 0;
  p.window = ctx->deposit_mode == RTG_DEPOSIT_WINDOW ? 1 : 0;
  p.window_factor = ctx->window_factor;
  return RTG_OK;
}

namespace {

int prepare_trace(rtg_context* ctx, uint64_t ray_begin, uint64_t ray_end, uint64_t seed, TraceParams& p) {
  return prepare_trace_with(ctx, ctx->cfg, ctx->box_lo, ctx->box_hi, ray_begin, ray_end, seed, p);
}

int rebuild_all(rtg_context* ctx) {
  RTG_TRY(build_lbvh(ctx));
  RTG_TRY(build_neighbors(ctx));
  RTG_TRY(alloc_results(ctx));
  resolve_box(ctx);
  return RTG_OK;
}

}  // namespace
}  // namespace rtg

using namespace rtg;

extern "C" {

int rtg_abi_version(void) { return RTG_ABI_VERSION; }

void rtg_config_default(rtg_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof *c);
  c->x_bound = RTG_BOUND_REFLECTIVE;
  c->y_bound = RTG_BOUND_REFLECTIVE;
  c->reflection = RTG_REFLECT_DIFFUSE;
  c->specular_fraction = 0.0f;
  c->sticking = 1.0f;
  c->source_exponent = 1.0f;
  c->box_mode = RTG_BOX_FROM_GEOMETRY;
  c->tnear = 1e-4f;
  c->roulette_threshold = 0.1;
  c->roulette_weight = 0.3;
  c->max_segments = 1u << 16;
  c->job = 0;
}

static int rtg_create_body(rtg_context** out, int device);

int rtg_create(rtg_context** out, int device) {
  return rtg::host_guard(nullptr, [&] { return rtg_create_body(out, device); });
}

static int rtg_create_body(rtg_context** out, int device) {
  if (!out) return RTG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return RTG_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return RTG_ERR_INVALID_ARGUMENT;
  rtg_context* ctx = new rtg_context();
  ctx->device = device;
  rtg_config_default(&ctx->cfg);
  int rc = RTG_OK;
  do {
    if ((rc = use_device(ctx)) != RTG_OK) break;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { rc = RTG_ERR_CUDA; break; }
    if (cudaMalloc((void**)&ctx->d_tally, sizeof(DevTally)) != cudaSuccess) { rc = RTG_ERR_OUT_OF_MEMORY; break; }
    if (cudaMalloc((void**)&ctx->d_tally_adj, sizeof(DevTally)) != cudaSuccess) {
      rc = RTG_ERR_OUT_OF_MEMORY;
      break;
    }
    if (cudaHostAlloc((void**)&ctx->h_abort, sizeof(uint32_t), cudaHostAllocMapped) != cudaSuccess) {
      rc = RTG_ERR_CUDA;
      break;
    }
    *ctx->h_abort = 0;
    if (cudaHostGetDevicePointer((void**)&ctx->d_abort, ctx->h_abort, 0) != cudaSuccess) { rc = RTG_ERR_CUDA; break; }
    if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        cudaEventCreate(&ctx->evk0) != cudaSuccess || cudaEventCreate(&ctx->evk1) != cudaSuccess) {
      rc = RTG_ERR_CUDA;
      break;
    }
    cudaMemset(ctx->d_tally, 0, sizeof(DevTally));
  } while (0);
  if (rc != RTG_OK) {
    cudaGetLastError();
    rtg_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return RTG_OK;
}

int rtg_destroy(rtg_context* ctx) {
  if (!ctx) return RTG_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  Geometry& g = ctx->g;
  dfree(g.disc_cr_by_id); dfree(g.disc_n_by_id); dfree(g.tri_v); dfree(g.tri_idx);
  dfree(g.disc); dfree(g.tri); dfree(g.nodes);
  dfree(g.leaf_ref); dfree(g.leaf_prim); dfree(g.parent); dfree(g.prim_lo); dfree(g.prim_hi);
  dfree(g.refit_flags); dfree(g.nb_ptr); dfree(g.nb_idx); dfree(g.nb_slot); dfree(g.disc_slot);
  dfree(ctx->sticking_field); dfree(ctx->acc); dfree(ctx->cnt); dfree(ctx->areas); dfree(ctx->est);
  dfree(ctx->stat_tmp);
  dfree(ctx->seglog);
  dfree(ctx->seglog_count);
  free_wavefront(ctx->wf);
  if (ctx->d_tally) cudaFree(ctx->d_tally);
  if (ctx->d_tally_adj) cudaFree(ctx->d_tally_adj);
  if (ctx->h_abort) cudaFreeHost(ctx->h_abort);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->evk0) cudaEventDestroy(ctx->evk0);
  if (ctx->evk1) cudaEventDestroy(ctx->evk1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return RTG_OK;
}

const char* rtg_last_error(const rtg_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int rtg_upload_mixed(rtg_context* ctx, const float* points, const float* normals, const float* radii, int64_t nd,
                     const float* vertices, const uint32_t* indices, int64_t nv, int64_t nt) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  NvtxRange range("rtg upload + LBVH build");
  RTG_TRY(use_device(ctx));
  // both halves are checked before either replaces the context's surface
  Staged sg;
  int rc = stage_discs(ctx, points, normals, radii, nd, sg);
  if (rc == RTG_OK) rc = stage_triangles(ctx, vertices, indices, nv, nt, sg);
  if (rc == RTG_OK && nd + nt == 0) rc = set_error(ctx, RTG_ERR_NO_GEOMETRY, "no primitives");
  const bool committing = rc == RTG_OK;
  if (committing) {
    ++ctx->version;
    rc = commit(ctx, sg);
  }
  release(sg, ctx->stream);
  if (committing) {
    dfree(ctx->sticking_field);
    if (rc == RTG_OK) rc = rebuild_all(ctx);
    if (rc != RTG_OK) drop_surface(ctx);
  }
  return rc;
}

int rtg_upload_discs(rtg_context* ctx, const float* points, const float* normals, const float* radii, int64_t n) {
  return rtg_upload_mixed(ctx, points, normals, radii, n, nullptr, nullptr, 0, 0);
}

int rtg_upload_triangles(rtg_context* ctx, const float* vertices, const uint32_t* indices, int64_t nv, int64_t nt) {
  return rtg_upload_mixed(ctx, nullptr, nullptr, nullptr, 0, vertices, indices, nv, nt);
}

int rtg_update_discs(rtg_context* ctx, const float* points, const float* normals, const float* radii, int64_t n) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (ctx->g.nd == 0 || !ctx->g.nodes.p) return set_error(ctx, RTG_ERR_NO_GEOMETRY, "no discs to update");
  RTG_TRY(use_device(ctx));
  if (n != ctx->g.nd)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "update_discs: the disc count must not change");
  Staged sg;
  int rc = stage_discs(ctx, points, normals, radii, n, sg);
  const bool committing = rc == RTG_OK;
  if (committing) {
    ++ctx->version;
    rc = commit(ctx, sg);
  }
  release(sg, ctx->stream);
  if (!committing) return rc;
  if (rc == RTG_OK) rc = refit_lbvh(ctx);
  if (rc == RTG_OK) rc = build_neighbors(ctx);
  if (rc == RTG_OK) rc = alloc_results(ctx);
  if (rc != RTG_OK) {
    drop_surface(ctx);
    return rc;
  }
  resolve_box(ctx);
  return RTG_OK;
}

static int rtg_update_vertices_body(rtg_context* ctx, const float* vertices, int64_t nv);

int rtg_update_vertices(rtg_context* ctx, const float* vertices, int64_t nv) {
  return rtg::host_guard(ctx, [&] { return rtg_update_vertices_body(ctx, vertices, nv); });
}

static int rtg_update_vertices_body(rtg_context* ctx, const float* vertices, int64_t nv) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  Geometry& g = ctx->g;
  if (g.nt == 0 || nv != g.nv || !vertices)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "update_vertices: vertex count must match the upload");
  RTG_TRY(use_device(ctx));
  std::vector<float4> v((size_t)nv);
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int64_t i = 0; i < nv; ++i) {
    if (!finite3(vertices + 3 * i)) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "vertex is not finite");
    v[(size_t)i] = make_float4(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2], 0.0f);
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], vertices[3 * i + a]);
      hi[a] = std::max(hi[a], vertices[3 * i + a]);
    }
  }
  for (int a = 0; a < 3; ++a) {
    g.tri_min[a] = lo[a];
    g.tri_max[a] = hi[a];
  }
  ++ctx->version;
  int rc = check_cuda(ctx, cudaMemcpyAsync(g.tri_v.p, v.data(), nv * sizeof(float4), cudaMemcpyHostToDevice,
                                           ctx->stream), "vertex update");
  if (rc == RTG_OK) rc = refit_lbvh(ctx);
  if (rc == RTG_OK) rc = alloc_results(ctx);
  if (rc != RTG_OK) {
    drop_surface(ctx);
    return rc;
  }
  resolve_box(ctx);
  return RTG_OK;
}

int rtg_set_config(rtg_context* ctx, const rtg_config* cfg) {
  if (!ctx || !cfg) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(check_config(ctx, *cfg));
  ctx->cfg = *cfg;
  resolve_box(ctx);
  return RTG_OK;
}

}  // extern "C"

namespace rtg {
int check_config(rtg_context* ctx, const rtg_config& c) {
  auto bad = [&](const char* m) { return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, m); };
  if ((c.x_bound != RTG_BOUND_REFLECTIVE && c.x_bound != RTG_BOUND_PERIODIC) ||
      (c.y_bound != RTG_BOUND_REFLECTIVE && c.y_bound != RTG_BOUND_PERIODIC))
    return bad("bound condition must be RTG_BOUND_REFLECTIVE or RTG_BOUND_PERIODIC");
  if (c.reflection < RTG_REFLECT_DIFFUSE || c.reflection > RTG_REFLECT_MIXED) return bad("unknown reflection");
  if (!(c.specular_fraction >= 0.0f && c.specular_fraction <= 1.0f)) return bad("specular_fraction not in [0,1]");
  if (!(c.sticking >= 0.0f && c.sticking <= 1.0f)) return bad("sticking not in [0,1]");
  if (!(c.source_exponent >= 0.0f) || !std::isfinite(c.source_exponent)) return bad("source_exponent must be >= 0");
  if (!(c.tnear >= 0.0f) || !std::isfinite(c.tnear)) return bad("tnear must be >= 0");
  if (!(c.roulette_threshold >= 0.0 && c.roulette_threshold <= c.roulette_weight && c.roulette_weight <= 1.0))
    return bad("roulette needs 0 <= threshold <= weight <= 1");
  if (c.max_segments == 0) return bad("max_segments must be > 0");
  if (c.box_mode != RTG_BOX_FROM_GEOMETRY && c.box_mode != RTG_BOX_EXPLICIT) return bad("unknown box_mode");
  if (c.box_mode == RTG_BOX_EXPLICIT) {
    for (int a = 0; a < 3; ++a)
      if (!(c.box_lo[a] < c.box_hi[a]) || !std::isfinite(c.box_lo[a]) || !std::isfinite(c.box_hi[a]))
        return bad("explicit box needs finite box_lo < box_hi");
  }
  return RTG_OK;
}
}  // namespace rtg

extern "C" {

int rtg_get_config(const rtg_context* ctx, rtg_config* cfg) {
  if (!ctx || !cfg) return RTG_ERR_INVALID_ARGUMENT;
  *cfg = ctx->cfg;
  return RTG_OK;
}

int rtg_get_box(const rtg_context* ctx, float* lo, float* hi) {
  if (!ctx || !lo || !hi) return RTG_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; ++a) {
    lo[a] = ctx->box_lo[a];
    hi[a] = ctx->box_hi[a];
  }
  return RTG_OK;
}

int rtg_set_sticking(rtg_context* ctx, float s) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (!(s >= 0.0f && s <= 1.0f)) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "sticking not in [0,1]");
  ctx->cfg.sticking = s;
  return RTG_OK;
}

int rtg_set_sticking_field(rtg_context* ctx, const float* s, int64_t n) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  ++ctx->version;
  if (!s) {
    dfree(ctx->sticking_field);
    return RTG_OK;
  }
  const int64_t np = ctx->g.nd + ctx->g.nt;
  if (n != np) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "sticking field length != number of primitives");
  for (int64_t i = 0; i < n; ++i)
    if (!(s[i] >= 0.0f && s[i] <= 1.0f))
      return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "sticking field value not in [0,1]");
  RTG_TRY(dalloc(ctx, ctx->sticking_field, (size_t)n, "sticking field"));
  RTG_CUDA(ctx, cudaMemcpyAsync(ctx->sticking_field.p, s, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return RTG_OK;
}

void rtg_launch_config_default(rtg_launch_config* lc) {
  if (!lc) return;
  lc->threads_per_block = 128;
  lc->packet = 1;
  lc->stack_depth = 0;
  lc->scheduling = RTG_SCHED_MEGAKERNEL;
  lc->leaf_tests = RTG_LEAF_IMMEDIATE;
  lc->stack_memory = RTG_STACK_AUTO;
}

int rtg_set_launch_config(rtg_context* ctx, const rtg_launch_config* lc) {
  if (!ctx || !lc) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(check_launch_config(ctx, *lc));
  ctx->lc = *lc;
  return RTG_OK;
}

int rtg_get_launch_config(const rtg_context* ctx, rtg_launch_config* lc) {
  if (!ctx || !lc) return RTG_ERR_INVALID_ARGUMENT;
  *lc = ctx->lc;
  return RTG_OK;
}

int rtg_get_tree_depth(const rtg_context* ctx, int32_t* depth) {
  if (!ctx || !depth) return RTG_ERR_INVALID_ARGUMENT;
  *depth = ctx->g.depth;
  return RTG_OK;
}

int rtg_set_tree_builder(rtg_context* ctx, int32_t builder) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (builder != RTG_TREE_KARRAS && builder != RTG_TREE_PLOC)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "builder must be RTG_TREE_KARRAS or RTG_TREE_PLOC");
  RTG_TRY(use_device(ctx));
  const int32_t keep = ctx->g.builder;
  ctx->g.builder = builder;
  if (ctx->g.nd + ctx->g.nt > 0 && ctx->g.nodes.p && builder != keep) {
    ++ctx->version;
    int rc = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "tree rebuild");
    if (rc == RTG_OK) rc = build_lbvh(ctx);
    if (rc == RTG_OK) rc = build_neighbors(ctx);  // neighbour columns are stored as slots of the new tree
    if (rc != RTG_OK) {
      drop_surface(ctx);
      return rc;
    }
    ctx->traced = false;
    ctx->finalized = false;
  }
  return RTG_OK;
}

int rtg_get_tree_builder(const rtg_context* ctx, int32_t* builder) {
  if (!ctx || !builder) return RTG_ERR_INVALID_ARGUMENT;
  *builder = ctx->g.builder;
  return RTG_OK;
}

int rtg_set_node_width(rtg_context* ctx, int32_t width) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (width != RTG_NODES_AUTO && width != RTG_NODES_BINARY && width != RTG_NODES_WIDE)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "node width must be RTG_NODES_AUTO, _BINARY or _WIDE");
  if (width != ctx->node_width) ++ctx->version;  // batch jobs hold scene views
  ctx->node_width = width;
  return RTG_OK;
}

int rtg_get_node_width(const rtg_context* ctx, int32_t* width) {
  if (!ctx || !width) return RTG_ERR_INVALID_ARGUMENT;
  *width = ctx->node_width;
  return RTG_OK;
}

int rtg_get_traversal_width(const rtg_context* ctx, int32_t* width) {
  if (!ctx || !width) return RTG_ERR_INVALID_ARGUMENT;
  const Geometry& g = ctx->g;
  // a wanted tree not collapsed yet is built before the next trace
  const bool usable = !g.wide_current || (g.n_wnodes > 0 && g.wide_stack <= 256);
  *width = wants_wide(ctx) && g.nd + g.nt > 0 && usable ? RTG_NODES_WIDE : RTG_NODES_BINARY;
  return RTG_OK;
}

int rtg_set_deposit_mode(rtg_context* ctx, int32_t mode, float window_factor) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (mode != RTG_DEPOSIT_NEIGHBORS && mode != RTG_DEPOSIT_WINDOW)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "mode must be RTG_DEPOSIT_NEIGHBORS or RTG_DEPOSIT_WINDOW");
  if (!(window_factor >= 0.0f && window_factor < 1e30f))
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "window_factor must be finite and >= 0");
  ctx->deposit_mode = mode;
  ctx->window_factor = window_factor;
  return RTG_OK;
}

int rtg_set_accumulation(rtg_context* ctx, int32_t mode) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (mode != RTG_ACCUM_FP64 && mode != RTG_ACCUM_FIXED)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "mode must be RTG_ACCUM_FP64 or RTG_ACCUM_FIXED");
  ctx->accum = mode;
  return RTG_OK;
}

int rtg_get_accumulation(const rtg_context* ctx, int32_t* mode) {
  if (!ctx || !mode) return RTG_ERR_INVALID_ARGUMENT;
  *mode = ctx->accum;
  return RTG_OK;
}

int rtg_set_visit_limit(rtg_context* ctx, uint64_t visits) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  ctx->visit_limit = visits;
  ++ctx->version;
  return RTG_OK;
}

int rtg_inject_alloc_failure(rtg_context* ctx, int64_t after) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  ctx->alloc_failure_in = after < 0 ? -1 : after;
  return RTG_OK;
}

int rtg_get_visit_limit(const rtg_context* ctx, uint64_t* visits) {
  if (!ctx || !visits) return RTG_ERR_INVALID_ARGUMENT;
  *visits = ctx->visit_limit;
  return RTG_OK;
}

int rtg_get_deposit_mode(const rtg_context* ctx, int32_t* mode, float* window_factor) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (mode) *mode = ctx->deposit_mode;
  if (window_factor) *window_factor = ctx->window_factor;
  return RTG_OK;
}

static int rtg_autotune_body(rtg_context* ctx, uint64_t sample_rays, uint64_t seed, rtg_launch_config* best,
                 double* best_rays_per_s);

int rtg_autotune(rtg_context* ctx, uint64_t sample_rays, uint64_t seed, rtg_launch_config* best,
                 double* best_rays_per_s) {
  return rtg::host_guard(ctx, [&] { return rtg_autotune_body(ctx, sample_rays, seed, best, best_rays_per_s); });
}

static int rtg_autotune_body(rtg_context* ctx, uint64_t sample_rays, uint64_t seed, rtg_launch_config* best,
                 double* best_rays_per_s) {
  if (!ctx || sample_rays == 0) return RTG_ERR_INVALID_ARGUMENT;
  TraceParams p{};
  RTG_TRY(prepare_trace(ctx, 0, sample_rays, seed, p));
  const int64_t np = ctx->g.nd + ctx->g.nt;
  cudaStream_t st = ctx->stream;
  const rtg_launch_config keep = ctx->lc;
  const int32_t keep_builder = ctx->g.builder;
  const int32_t keep_width = ctx->node_width;
  struct Cand {
    int32_t builder;
    int32_t width;  // RTG_NODES_BINARY or RTG_NODES_WIDE
    rtg_launch_config lc;
    float ms;
  };
  auto run = [&](const Cand& c, float& ms) -> int {
    ctx->lc = c.lc;
    ctx->node_width = c.width;
    RTG_TRY(ensure_wide(ctx));
    p.s = scene_view(ctx);
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->acc.p, 0, 4 * np * sizeof(double), st));
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->cnt.p, 0, np * sizeof(unsigned long long), st));
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->d_tally, 0, sizeof(DevTally), st));
    RTG_CUDA(ctx, cudaEventRecord(ctx->evk0, st));
    RTG_TRY(launch_trace(ctx, p, st));
    RTG_CUDA(ctx, cudaEventRecord(ctx->evk1, st));
    RTG_CUDA(ctx, cudaEventSynchronize(ctx->evk1));
    RTG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->evk0, ctx->evk1));
    return RTG_OK;
  };
  std::vector<Cand> cand;
  int rc = RTG_OK;
  for (int32_t builder : {RTG_TREE_KARRAS, RTG_TREE_PLOC}) {
    if (rc != RTG_OK) break;
    rc = rtg_set_tree_builder(ctx, builder);
    if (rc == RTG_OK) rc = prepare_trace(ctx, 0, sample_rays, seed, p);  // the tree changed
    if (rc != RTG_OK) break;
    const size_t first = cand.size();
    const int32_t width = outgrows_l2(ctx) ? RTG_NODES_WIDE : RTG_NODES_BINARY;  // the automatic choice
    // the wavefront schedule is not a candidate: its queue traffic lost to the
    // megakernel on every workload measured (it stays selectable by hand)
    for (int sched : {RTG_SCHED_MEGAKERNEL, RTG_SCHED_PLAIN})
      for (int tpb : {64, 128, 256})
        for (int packet : {1, 8, 32})
          for (int stack : {0, 256})
            for (int leaf : {RTG_LEAF_IMMEDIATE, RTG_LEAF_POSTPONED}) {
              if (sched == RTG_SCHED_PLAIN && (packet != 1 || tpb == 64 || stack != 0)) continue;
              if (stack == 256 && stack_for(0, traversal_depth(ctx)) == 256) continue;
              if (leaf == RTG_LEAF_POSTPONED && packet == 32) continue;
              cand.push_back(Cand{builder, width, rtg_launch_config{tpb, packet, stack, sched, leaf, RTG_STACK_AUTO}, 0.0f});
            }
    float ms = 0.0f;
    for (size_t i = first; i < cand.size() && rc == RTG_OK; ++i) {
      rc = run(cand[i], ms);  // warm-up
      if (rc == RTG_OK) rc = run(cand[i], cand[i].ms);
    }
    // the three fastest of this tree again, keep each one's best time
    std::vector<size_t> order;
    for (size_t i = first; i < cand.size(); ++i) order.push_back(i);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cand[a].ms < cand[b].ms; });
    for (size_t r = 0; r < 2 && rc == RTG_OK; ++r)
      for (size_t q = 0; q < order.size() && q < 3 && rc == RTG_OK; ++q) {
        rc = run(cand[order[q]], ms);
        if (rc == RTG_OK && ms < cand[order[q]].ms) cand[order[q]].ms = ms;
      }
    // the three fastest with their stacks in the other memory, best of two
    for (size_t q = 0; q < order.size() && q < 3 && rc == RTG_OK; ++q) {
      Cand alt = cand[order[q]];
      if (alt.lc.scheduling == RTG_SCHED_WAVEFRONT) continue;
      alt.lc.stack_memory = shared_stack(ctx, alt.lc) ? RTG_STACK_LOCAL : RTG_STACK_SHARED;
      float m2 = 0.0f;
      rc = run(alt, alt.ms);
      if (rc == RTG_OK) rc = run(alt, m2);
      if (rc == RTG_OK) {
        alt.ms = std::min(alt.ms, m2);
        cand.push_back(alt);
      }
    }
    // the three fastest over the other tree layout (binary / wide), best of two
    if (ctx->g.n_wnodes > 0)
      for (size_t q = 0; q < order.size() && q < 3 && rc == RTG_OK; ++q) {
        Cand alt = cand[order[q]];
        alt.width = alt.width == RTG_NODES_WIDE ? RTG_NODES_BINARY : RTG_NODES_WIDE;
        float m2 = 0.0f;
        rc = run(alt, alt.ms);
        if (rc == RTG_OK) rc = run(alt, m2);
        if (rc == RTG_OK) {
          alt.ms = std::min(alt.ms, m2);
          cand.push_back(alt);
        }
      }
  }
  ctx->traced = false;
  ctx->finalized = false;
  if (rc != RTG_OK || cand.empty()) {
    ctx->lc = keep;
    ctx->node_width = keep_width;
    rtg_set_tree_builder(ctx, keep_builder);
    return rc != RTG_OK ? rc : set_error(ctx, RTG_ERR_INTERNAL, "autotune found no candidate");
  }
  size_t bi = 0;
  for (size_t i = 1; i < cand.size(); ++i)
    if (cand[i].ms < cand[bi].ms) bi = i;
  RTG_TRY(rtg_set_tree_builder(ctx, cand[bi].builder));
  ctx->lc = cand[bi].lc;
  ctx->node_width = cand[bi].width;
  ++ctx->version;
  if (best) *best = cand[bi].lc;
  if (best_rays_per_s) *best_rays_per_s = cand[bi].ms > 0.0f ? sample_rays / (cand[bi].ms * 1e-3) : 0.0;
  return RTG_OK;
}

int rtg_trace_range(rtg_context* ctx, uint64_t ray_begin, uint64_t ray_end, uint64_t seed, int accumulate,
                    void* stream) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  NvtxRange range("rtg trace (enqueue)");
  TraceParams p{};
  RTG_TRY(prepare_trace(ctx, ray_begin, ray_end, seed, p));
  const int64_t np = ctx->g.nd + ctx->g.nt;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  ctx->traced = false;  // until this trace is enqueued in full
  RTG_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  if (!accumulate) {
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->acc.p, 0, 4 * np * sizeof(double), st));
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->cnt.p, 0, np * sizeof(unsigned long long), st));
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->d_tally, 0, sizeof(DevTally), st));
    ctx->last_rays = 0;
  } else {
    RTG_CUDA(ctx, cudaMemsetAsync(&ctx->d_tally->next_ray, 0, sizeof(unsigned long long), st));
  }
  if (ctx->seglog.p) {
    if (p.window) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "the segment log records neighbour-deposit traces only");
    p.log = SegmentLog{ctx->seglog.p, ctx->seglog.n, ctx->seglog_count.p, ctx->seglog_begin, ctx->seglog_end};
    if (!accumulate) RTG_CUDA(ctx, cudaMemsetAsync(ctx->seglog_count.p, 0, sizeof(unsigned long long), st));
  }
  const bool fixed = p.fixed_s1 != 0;
  if (fixed && accumulate) RTG_TRY(s1_to_fixed(ctx, ctx->acc.p, np, st));  // resume the integer sums
  RTG_CUDA(ctx, cudaEventRecord(ctx->evk0, st));
  if (ray_end > ray_begin) RTG_TRY(launch_trace(ctx, p, st));
  RTG_CUDA(ctx, cudaEventRecord(ctx->evk1, st));
  if (fixed) RTG_TRY(s1_to_double(ctx, ctx->acc.p, np, st));
  RTG_TRY(compute_areas(ctx, st, ctx->box_lo, ctx->box_hi));
  RTG_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  ctx->last_rays += ray_end - ray_begin;
  ctx->traced = true;
  ctx->finalized = false;
  return RTG_OK;
}

int rtg_set_segment_log(rtg_context* ctx, uint64_t ray_begin, uint64_t ray_end, uint64_t capacity) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  if (capacity == 0) {
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    dfree(ctx->seglog);
    dfree(ctx->seglog_count);
    return RTG_OK;
  }
  if (ray_end <= ray_begin) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "segment log: empty ray range");
  if (capacity > (1ull << 32)) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "segment log: at most 2^32 records");
  RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  RTG_TRY(dalloc(ctx, ctx->seglog, (size_t)capacity, "segment log"));
  RTG_TRY(dalloc(ctx, ctx->seglog_count, 1, "segment log counter"));
  RTG_CUDA(ctx, cudaMemsetAsync(ctx->seglog_count.p, 0, sizeof(unsigned long long), ctx->stream));
  ctx->seglog_begin = ray_begin;
  ctx->seglog_end = ray_end;
  return RTG_OK;
}

// The kept records, sorted by (ray, segment); *dropped = records that did not fit.
static int read_segment_log(rtg_context* ctx, std::vector<rtg_segment>& out, uint64_t* dropped) {
  out.clear();
  if (dropped) *dropped = 0;
  if (!ctx->seglog.p) return RTG_OK;
  RTG_TRY(use_device(ctx));
  RTG_CUDA(ctx, cudaDeviceSynchronize());
  unsigned long long count = 0;
  RTG_CUDA(ctx, cudaMemcpy(&count, ctx->seglog_count.p, sizeof count, cudaMemcpyDeviceToHost));
  const uint64_t kept = std::min<uint64_t>(count, ctx->seglog.n);
  out.resize(kept);
  if (kept) RTG_CUDA(ctx, cudaMemcpy(out.data(), ctx->seglog.p, kept * sizeof(rtg_segment), cudaMemcpyDeviceToHost));
  std::sort(out.begin(), out.end(), [](const rtg_segment& a, const rtg_segment& b) {
    return a.ray != b.ray ? a.ray < b.ray : a.segment < b.segment;
  });
  if (dropped) *dropped = count - kept;
  return RTG_OK;
}

static int rtg_get_segment_log_body(rtg_context* ctx, rtg_segment* out, uint64_t cap, uint64_t* n_kept, uint64_t* n_dropped);

int rtg_get_segment_log(rtg_context* ctx, rtg_segment* out, uint64_t cap, uint64_t* n_kept, uint64_t* n_dropped) {
  return rtg::host_guard(ctx, [&] { return rtg_get_segment_log_body(ctx, out, cap, n_kept, n_dropped); });
}

static int rtg_get_segment_log_body(rtg_context* ctx, rtg_segment* out, uint64_t cap, uint64_t* n_kept, uint64_t* n_dropped) {
  if (!ctx || (cap > 0 && !out)) return RTG_ERR_INVALID_ARGUMENT;
  std::vector<rtg_segment> v;
  uint64_t dropped = 0;
  RTG_TRY(read_segment_log(ctx, v, &dropped));
  if (!v.empty() && cap > 0) std::memcpy(out, v.data(), std::min<uint64_t>(cap, v.size()) * sizeof(rtg_segment));
  if (n_kept) *n_kept = v.size();
  if (n_dropped) *n_dropped = dropped;
  return RTG_OK;
}

static int rtg_write_segment_log_vtp_body(rtg_context* ctx, const char* path);

int rtg_write_segment_log_vtp(rtg_context* ctx, const char* path) {
  return rtg::host_guard(ctx, [&] { return rtg_write_segment_log_vtp_body(ctx, path); });
}

static int rtg_write_segment_log_vtp_body(rtg_context* ctx, const char* path) {
  if (!ctx || !path) return RTG_ERR_INVALID_ARGUMENT;
  if (!ctx->seglog.p) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "no segment log (rtg_set_segment_log)");
  std::vector<rtg_segment> v;
  RTG_TRY(read_segment_log(ctx, v, nullptr));
  const int rc = rtg_write_vtp_segments(path, v.data(), (int64_t)v.size());
  return rc == RTG_OK ? rc : set_error(ctx, rc, std::string("cannot write ") + path);
}

int rtg_set_sticking_field_device(rtg_context* ctx, const float* d_field, int64_t n, void* stream) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  ++ctx->version;
  if (!d_field) {
    dfree(ctx->sticking_field);
    return RTG_OK;
  }
  const int64_t np = ctx->g.nd + ctx->g.nt;
  if (n != np) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "sticking field length != number of primitives");
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  RTG_TRY(dalloc(ctx, ctx->sticking_field, (size_t)n, "sticking field"));
  RTG_CUDA(ctx, cudaMemcpyAsync(ctx->sticking_field.p, d_field, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
  return RTG_OK;
}

int rtg_adjoint(rtg_context* ctx, const double* d_g, uint64_t ray_begin, uint64_t ray_end, uint64_t seed, int estimator,
                double* d_field_grad, double* d_scalars, void* stream) {
  if (!ctx || !d_g || !d_scalars) return RTG_ERR_INVALID_ARGUMENT;
  NvtxRange range("rtg adjoint (enqueue)");
  const bool field = ctx->sticking_field.p != nullptr;
  if (field && !d_field_grad)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "a sticking field is set: d_field_grad is required");
  if (ctx->deposit_mode != RTG_DEPOSIT_NEIGHBORS)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "the adjoint replays the neighbour deposit only");
  TraceParams p{};
  RTG_TRY(prepare_trace(ctx, ray_begin, ray_end, seed, p));
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  p.tally = ctx->d_tally_adj;
  p.s1 = p.s2 = p.s3 = p.s4 = nullptr;
  p.cnt = nullptr;
  p.adj_g = d_g;
  p.adj_field = field ? d_field_grad : nullptr;
  p.adj_scalars = d_scalars;
  p.adj_unbiased = estimator == RTG_ADJ_UNBIASED ? 1 : 0;
  RTG_CUDA(ctx, cudaMemsetAsync(ctx->d_tally_adj, 0, sizeof(DevTally), st));
  if (ray_end > ray_begin) RTG_TRY(launch_trace(ctx, p, st, field ? kModeAdjField : kModeAdjGlobal));
  return RTG_OK;
}

int rtg_adjoint_host(rtg_context* ctx, const double* g, uint64_t n_rays, uint64_t seed, int estimator, double* field_grad,
                     double* d_sticking, double* d_exponent) {
  if (!ctx || !g) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  const int64_t np = ctx->g.nd + ctx->g.nt;
  const bool field = ctx->sticking_field.p != nullptr;
  if (field && !field_grad)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "a sticking field is set: field_grad is required");
  DBuf<double> dg, df, ds;
  int rc = dalloc(ctx, dg, (size_t)(np > 0 ? np : 1), "adjoint weights");
  if (rc == RTG_OK) rc = dalloc(ctx, df, (size_t)(field ? np : 1), "adjoint field");
  if (rc == RTG_OK) rc = dalloc(ctx, ds, 2, "adjoint scalars");
  cudaStream_t st = ctx->stream;
  if (rc == RTG_OK) {
    cudaError_t e = cudaMemcpyAsync(dg.p, g, np * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(df.p, 0, df.n * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ds.p, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess) rc = check_cuda(ctx, e, "adjoint upload");
  }
  if (rc == RTG_OK) rc = rtg_adjoint(ctx, dg.p, 0, n_rays, seed, estimator, field ? df.p : nullptr, ds.p, nullptr);
  double sc[2] = {0.0, 0.0};
  if (rc == RTG_OK) {
    cudaError_t e = cudaMemcpyAsync(sc, ds.p, sizeof sc, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && field) e = cudaMemcpyAsync(field_grad, df.p, np * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = check_cuda(ctx, e, "adjoint");
  }
  if (rc == RTG_OK) {
    DevTally t;
    if (cudaMemcpy(&t, ctx->d_tally_adj, sizeof t, cudaMemcpyDeviceToHost) == cudaSuccess) {
      if (t.abort_seen) rc = set_error(ctx, RTG_ERR_ABORTED, "adjoint aborted on request");
      else if (t.errors) rc = set_error(ctx, RTG_ERR_BUDGET, "a device-side traversal limit was reached");
    }
  }
  dfree(dg);
  dfree(df);
  dfree(ds);
  if (rc == RTG_OK) {
    if (d_sticking) *d_sticking = sc[0];
    if (d_exponent) *d_exponent = sc[1];
  }
  return rc;
}

int rtg_trace(rtg_context* ctx, uint64_t n_rays, uint64_t seed, void* stream) {
  return rtg_trace_range(ctx, 0, n_rays, seed, 0, stream);
}

int rtg_synchronize(rtg_context* ctx) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  RTG_CUDA(ctx, cudaDeviceSynchronize());
  return RTG_OK;
}

int rtg_request_abort(rtg_context* ctx) {
  if (!ctx || !ctx->h_abort) return RTG_ERR_INVALID_ARGUMENT;
  *(volatile uint32_t*)ctx->h_abort = 1u;
  return RTG_OK;
}

int rtg_trace_rays(rtg_context* ctx, const float* rays, int64_t n, float tnear, int32_t* prim_out, float* t_out) {
  if (!ctx || n < 0 || (n > 0 && (!rays || !prim_out || !t_out))) return RTG_ERR_INVALID_ARGUMENT;
  if (ctx->g.nd + ctx->g.nt == 0 || !ctx->g.nodes.p) return set_error(ctx, RTG_ERR_NO_GEOMETRY, "no geometry");
  if (n == 0) return RTG_OK;
  RTG_TRY(use_device(ctx));
  DBuf<float> dr, dt;
  DBuf<int32_t> dp;
  DBuf<unsigned long long> de;  // queries that hit a traversal limit (the trace tally stays untouched)
  int rc = dalloc(ctx, dr, (size_t)(6 * n), "rays");
  if (rc == RTG_OK) rc = dalloc(ctx, dt, (size_t)n, "ray t");
  if (rc == RTG_OK) rc = dalloc(ctx, dp, (size_t)n, "ray prim");
  if (rc == RTG_OK) rc = dalloc(ctx, de, 1, "ray errors");
  unsigned long long errors = 0;
  if (rc == RTG_OK) {
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(dr.p, rays, 6 * n * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(de.p, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) rc = check_cuda(ctx, e, "trace_rays upload");
    if (rc == RTG_OK) rc = launch_closest_hit(ctx, dr.p, n, tnear, dp.p, dt.p, de.p, st);
    if (rc == RTG_OK) {
      e = cudaMemcpyAsync(prim_out, dp.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(t_out, dt.p, n * sizeof(float), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&errors, de.p, sizeof errors, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) rc = check_cuda(ctx, e, "trace_rays");
    }
  }
  dfree(dr);
  dfree(dt);
  dfree(dp);
  dfree(de);
  if (rc == RTG_OK && errors)
    rc = set_error(ctx, RTG_ERR_BUDGET, "a device-side traversal limit was reached");
  return rc;
}

int rtg_num_primitives(const rtg_context* ctx, int64_t* n) {
  if (!ctx || !n) return RTG_ERR_INVALID_ARGUMENT;
  *n = ctx->g.nd + ctx->g.nt;
  return RTG_OK;
}

static int sync_trace(rtg_context* ctx) {
  RTG_TRY(use_device(ctx));
  RTG_CUDA(ctx, cudaDeviceSynchronize());
  DevTally t;
  RTG_CUDA(ctx, cudaMemcpy(&t, ctx->d_tally, sizeof t, cudaMemcpyDeviceToHost));
  if (t.abort_seen) return set_error(ctx, RTG_ERR_ABORTED, "trace aborted on request");
  if (t.errors) return set_error(ctx, RTG_ERR_BUDGET, "a device-side traversal limit was reached");
  return RTG_OK;
}

int rtg_get_mc_estimates(rtg_context* ctx, float* out) {
  if (!ctx || !out) return RTG_ERR_INVALID_ARGUMENT;
  if (!ctx->traced) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "no trace has run");
  RTG_TRY(sync_trace(ctx));
  if (!ctx->finalized) {
    RTG_TRY(finalize_estimates(ctx, ctx->stream));
    ctx->finalized = true;
  }
  const int64_t np = ctx->g.nd + ctx->g.nt;
  RTG_CUDA(ctx, cudaMemcpy(out, ctx->est.p, np * sizeof(float), cudaMemcpyDeviceToHost));
  return RTG_OK;
}

int rtg_get_hit_counts(rtg_context* ctx, uint64_t* out) {
  if (!ctx || !out) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(sync_trace(ctx));
  const int64_t np = ctx->g.nd + ctx->g.nt;
  RTG_CUDA(ctx, cudaMemcpy(out, ctx->cnt.p, np * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return RTG_OK;
}

int rtg_get_accumulators(rtg_context* ctx, double* s1, double* s2, double* s3, double* s4) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(sync_trace(ctx));
  const int64_t np = ctx->g.nd + ctx->g.nt;
  double* outs[4] = {s1, s2, s3, s4};
  for (int k = 0; k < 4; ++k)
    if (outs[k]) RTG_CUDA(ctx, cudaMemcpy(outs[k], ctx->acc.p + k * np, np * sizeof(double), cudaMemcpyDeviceToHost));
  return RTG_OK;
}

int rtg_get_exposed_areas(rtg_context* ctx, float* out) {
  if (!ctx || !out) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  const int64_t np = ctx->g.nd + ctx->g.nt;
  if (!ctx->traced) {
    RTG_TRY(compute_areas(ctx, ctx->stream, ctx->box_lo, ctx->box_hi));
  }
  RTG_CUDA(ctx, cudaDeviceSynchronize());
  RTG_CUDA(ctx, cudaMemcpy(out, ctx->areas.p, np * sizeof(float), cudaMemcpyDeviceToHost));
  return RTG_OK;
}

static int stats_to_host(rtg_context* ctx, double* out, bool vov) {
  RTG_TRY(sync_trace(ctx));
  const int64_t np = ctx->g.nd + ctx->g.nt;
  DevTally t;
  RTG_CUDA(ctx, cudaMemcpy(&t, ctx->d_tally, sizeof t, cudaMemcpyDeviceToHost));
  RTG_TRY(dalloc(ctx, ctx->stat_tmp, (size_t)(2 * np), "statistics"));
  RTG_TRY(compute_stats(ctx, ctx->stream, t.total, ctx->stat_tmp.p, ctx->stat_tmp.p + np));
  RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  RTG_CUDA(ctx, cudaMemcpy(out, ctx->stat_tmp.p + (vov ? np : 0), np * sizeof(double), cudaMemcpyDeviceToHost));
  return RTG_OK;
}

int rtg_get_relative_error(rtg_context* ctx, double* out) {
  if (!ctx || !out) return RTG_ERR_INVALID_ARGUMENT;
  return stats_to_host(ctx, out, false);
}

int rtg_get_vov(rtg_context* ctx, double* out) {
  if (!ctx || !out) return RTG_ERR_INVALID_ARGUMENT;
  return stats_to_host(ctx, out, true);
}

int rtg_get_tally(rtg_context* ctx, rtg_tally* out) {
  if (!ctx || !out) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  RTG_CUDA(ctx, cudaDeviceSynchronize());
  DevTally t;
  RTG_CUDA(ctx, cudaMemcpy(&t, ctx->d_tally, sizeof t, cudaMemcpyDeviceToHost));
  std::memset(out, 0, sizeof *out);
  out->num_rays = ctx->last_rays;
  out->hitc = t.hitc;
  out->nonhitc = t.nonhitc;
  out->total = t.total;
  out->segments = t.segments;
  out->truncated = t.truncated;
  out->nb_deposits = t.nb_deposits;
  out->errors = t.errors;
  float ms = 0.0f;
  if (ctx->traced && cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) out->trace_ms = ms;
  if (ctx->traced && cudaEventElapsedTime(&ms, ctx->evk0, ctx->evk1) == cudaSuccess) out->kernel_ms = ms;
  cudaGetLastError();
  return RTG_OK;
}

int rtg_set_accumulators(rtg_context* ctx, const double* s1, const double* s2, const double* s3, const double* s4,
                         const uint64_t* counts, const rtg_tally* tally) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  if (!s1 || !s2 || !s3 || !s4 || !counts || !tally)
    return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "set_accumulators: S1..S4, counts and tally are all needed");
  const int64_t np = ctx->g.nd + ctx->g.nt;
  if (np == 0 || !ctx->acc.p || !ctx->cnt.p) return set_error(ctx, RTG_ERR_NO_GEOMETRY, "no geometry uploaded");
  RTG_TRY(use_device(ctx));
  RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  RTG_CUDA(ctx, cudaDeviceSynchronize());  // no trace of this context may still write the accumulators
  const size_t bytes = (size_t)np * sizeof(double);
  const double* s[4] = {s1, s2, s3, s4};
  for (int k = 0; k < 4; ++k)
    RTG_CUDA(ctx, cudaMemcpy(ctx->acc.p + (size_t)k * np, s[k], bytes, cudaMemcpyHostToDevice));
  RTG_CUDA(ctx, cudaMemcpy(ctx->cnt.p, counts, (size_t)np * sizeof(unsigned long long), cudaMemcpyHostToDevice));
  DevTally t{};
  t.hitc = tally->hitc;
  t.nonhitc = tally->nonhitc;
  t.total = tally->total;
  t.segments = tally->segments;
  t.truncated = tally->truncated;
  t.nb_deposits = tally->nb_deposits;
  t.errors = tally->errors;
  RTG_CUDA(ctx, cudaMemcpy(ctx->d_tally, &t, sizeof t, cudaMemcpyHostToDevice));
  // the exposed areas of this surface, and zero-length timings for the getters
  RTG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  RTG_CUDA(ctx, cudaEventRecord(ctx->evk0, ctx->stream));
  RTG_CUDA(ctx, cudaEventRecord(ctx->evk1, ctx->stream));
  RTG_TRY(compute_areas(ctx, ctx->stream, ctx->box_lo, ctx->box_hi));
  RTG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->last_rays = tally->num_rays;
  ctx->traced = true;
  ctx->finalized = false;
  return RTG_OK;
}

int rtg_get_neighbors(rtg_context* ctx, int64_t* row_ptr, int32_t* cols, int64_t cap, int64_t* nnz) {
  if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
  RTG_TRY(use_device(ctx));
  const int64_t nd = ctx->g.nd;
  if (nnz) *nnz = ctx->g.nb_nnz;
  if (row_ptr && nd > 0)
    RTG_CUDA(ctx, cudaMemcpy(row_ptr, ctx->g.nb_ptr.p, (nd + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
  if (cols) {
    if (cap < ctx->g.nb_nnz) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "neighbour buffer too small");
    if (ctx->g.nb_nnz > 0)
      RTG_CUDA(ctx, cudaMemcpy(cols, ctx->g.nb_idx.p, ctx->g.nb_nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  return RTG_OK;
}

int rtg_get_device_view(rtg_context* ctx, rtg_device_view* v) {
  if (!ctx || !v) return RTG_ERR_INVALID_ARGUMENT;
  const int64_t np = ctx->g.nd + ctx->g.nt;
  v->s1 = ctx->acc.p;
  v->s2 = ctx->acc.p ? ctx->acc.p + np : nullptr;
  v->s3 = ctx->acc.p ? ctx->acc.p + 2 * np : nullptr;
  v->s4 = ctx->acc.p ? ctx->acc.p + 3 * np : nullptr;
  v->counts = (uint64_t*)ctx->cnt.p;
  v->areas = ctx->areas.p;
  v->estimates = ctx->est.p;
  v->n = np;
  return RTG_OK;
}

static int rtg_write_vtp_body(rtg_context* ctx, const char* path, const char* const* meta_keys, const char* const* meta_values,
                  int32_t n_meta);

int rtg_write_vtp(rtg_context* ctx, const char* path, const char* const* meta_keys, const char* const* meta_values,
                  int32_t n_meta) {
  return rtg::host_guard(ctx, [&] { return rtg_write_vtp_body(ctx, path, meta_keys, meta_values, n_meta); });
}

static int rtg_write_vtp_body(rtg_context* ctx, const char* path, const char* const* meta_keys, const char* const* meta_values,
                  int32_t n_meta) {
  if (!ctx || !path || (n_meta > 0 && (!meta_keys || !meta_values))) return RTG_ERR_INVALID_ARGUMENT;
  if (!ctx->traced) return set_error(ctx, RTG_ERR_NO_GEOMETRY, "write_vtp: no trace results yet");
  const Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  std::vector<double> s1((size_t)np), rel((size_t)np), vov((size_t)np);
  std::vector<uint64_t> cnt((size_t)np);
  std::vector<float> area((size_t)np);
  RTG_TRY(rtg_get_accumulators(ctx, s1.data(), nullptr, nullptr, nullptr));
  RTG_TRY(rtg_get_hit_counts(ctx, cnt.data()));
  RTG_TRY(rtg_get_exposed_areas(ctx, area.data()));
  RTG_TRY(rtg_get_relative_error(ctx, rel.data()));
  RTG_TRY(rtg_get_vov(ctx, vov.data()));
  std::vector<float4> cr((size_t)g.nd), nn((size_t)g.nd), v4((size_t)g.nv);
  std::vector<uint32_t> idx((size_t)(3 * g.nt));
  if (g.nd > 0) {
    RTG_CUDA(ctx, cudaMemcpy(cr.data(), g.disc_cr_by_id.p, g.nd * sizeof(float4), cudaMemcpyDeviceToHost));
    RTG_CUDA(ctx, cudaMemcpy(nn.data(), g.disc_n_by_id.p, g.nd * sizeof(float4), cudaMemcpyDeviceToHost));
  }
  if (g.nt > 0) {
    RTG_CUDA(ctx, cudaMemcpy(v4.data(), g.tri_v.p, g.nv * sizeof(float4), cudaMemcpyDeviceToHost));
    RTG_CUDA(ctx, cudaMemcpy(idx.data(), g.tri_idx.p, 3 * g.nt * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  }
  std::vector<float> pts((size_t)(3 * g.nd)), nrm((size_t)(3 * g.nd)), rad((size_t)g.nd), vtx((size_t)(3 * g.nv));
  for (int64_t i = 0; i < g.nd; ++i) {
    const float4 c = cr[(size_t)i], q = nn[(size_t)i];
    pts[3 * i] = c.x; pts[3 * i + 1] = c.y; pts[3 * i + 2] = c.z;
    nrm[3 * i] = q.x; nrm[3 * i + 1] = q.y; nrm[3 * i + 2] = q.z;
    rad[(size_t)i] = c.w;
  }
  for (int64_t i = 0; i < g.nv; ++i) {
    vtx[3 * i] = v4[(size_t)i].x; vtx[3 * i + 1] = v4[(size_t)i].y; vtx[3 * i + 2] = v4[(size_t)i].z;
  }
  const int rc = rtg_write_vtp_mixed(path, g.nd, pts.data(), nrm.data(), rad.data(), g.nt > 0 ? g.nv : 0, vtx.data(),
                                     g.nt, idx.data(), s1.data(), cnt.data(), area.data(), rel.data(), vov.data(),
                                     meta_keys, meta_values, n_meta);
  if (rc != RTG_OK) return set_error(ctx, rc, std::string("write_vtp: cannot write ") + path);
  return RTG_OK;
}

static int rtg_device_run_body(const float* points, const float* normals, const float* radii, int64_t n, const rtg_config* cfg,
                   const float* sticking_field, uint64_t n_rays, uint64_t seed, float* est_out, uint64_t* cnt_out,
                   int device);

int rtg_device_run(const float* points, const float* normals, const float* radii, int64_t n, const rtg_config* cfg,
                   const float* sticking_field, uint64_t n_rays, uint64_t seed, float* est_out, uint64_t* cnt_out,
                   int device) {
  return rtg::host_guard(nullptr, [&] { return rtg_device_run_body(points, normals, radii, n, cfg, sticking_field, n_rays, seed, est_out, cnt_out, device); });
}

static int rtg_device_run_body(const float* points, const float* normals, const float* radii, int64_t n, const rtg_config* cfg,
                   const float* sticking_field, uint64_t n_rays, uint64_t seed, float* est_out, uint64_t* cnt_out,
                   int device) {
  rtg_context* ctx = nullptr;
  int rc = rtg_create(&ctx, device);
  if (rc != RTG_OK) return rc;
  rtg_config c;
  if (cfg) c = *cfg;
  else rtg_config_default(&c);
  do {
    if ((rc = rtg_upload_discs(ctx, points, normals, radii, n)) != RTG_OK) break;
    if ((rc = rtg_set_config(ctx, &c)) != RTG_OK) break;
    if (sticking_field && (rc = rtg_set_sticking_field(ctx, sticking_field, n)) != RTG_OK) break;
    if ((rc = rtg_trace(ctx, n_rays, seed, nullptr)) != RTG_OK) break;
    if (est_out && (rc = rtg_get_mc_estimates(ctx, est_out)) != RTG_OK) break;
    if (cnt_out && (rc = rtg_get_hit_counts(ctx, cnt_out)) != RTG_OK) break;
  } while (0);
  rtg_destroy(ctx);
  return rc;
}

}  // extern "C"
