// rtg_internal.cuh -- context and cross-file declarations of librtg.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <new>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "rtg.h"

namespace rtg {

// A BVH child reference: bit 31 = leaf, bit 30 = triangle leaf, bits 0..29 =
// internal node index or primitive slot.
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kTriBit = 0x40000000u;
constexpr uint32_t kSlotMask = 0x3FFFFFFFu;
constexpr int kStackSize = 64;

// One internal node: the boxes of both children and their references (64 B).
//   a = (c0.lo.x, c0.hi.x, c1.lo.x, c1.hi.x)
//   b = (c0.lo.y, c0.hi.y, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (child0, child1, parent, unused) as uint32 bits
struct __align__(16) Node {
  float4 a, b, c;
  uint4 d;
};

// One node of the compressed 8-wide tree the closest-hit query traverses
// (collapsed from the binary LBVH after every build and refit; rtg_wide.cu).
// 96 bytes, read by three 256-bit loads:
//   w[0..2]  node origin p (float bits), an exact multiple of the axis quantum
//   w[3]     biased exponents e_x, e_y, e_z of the quanta 2^e (bytes 0..2) and
//            the leaf mask (byte 3: bit s set when child slot s is a
//            primitive or empty)
//   w[4..11] child references by slot (kLeafBit/kTriBit as in Node; an
//            internal child is a wide-node index; kNoChild = empty slot)
//   w[12..23] quantised child boxes, one byte per slot: lo.x (w12, w13),
//            lo.y, lo.z, hi.x, hi.y, hi.z; box = p + q * 2^e, conservative
//            (floor for lo, ceil for hi); an empty slot has lo = 255, hi = 0.
// Slot s holds the child that lies most towards the corner whose axis signs
// are the bits of s (set = +), so a ray whose direction signs form the octant
// code o visits the slots in the order i ^ o, i = 0..7, nearly front to back.
struct __align__(32) WideNode {
  uint32_t w[24];
};
constexpr int kWide = 8;
constexpr uint32_t kNoChild = 0xFFFFFFFFu;

// LBVH topology builders over the Morton-ordered leaves.
constexpr int32_t kBuilderKarras = 0;  // Karras 2012 radix tree (split at the highest differing key bit)
constexpr int32_t kBuilderPloc = 1;    // Meister and Bittner 2018 locally-ordered clustering

// Device status counters (accumulated over a trace).
struct DevTally {
  unsigned long long hitc, nonhitc, total, segments, truncated, nb_deposits, errors, next_ray;
  unsigned int abort_seen;
  unsigned int pad;
};

// Read-only view of a scene for the kernels.
struct SceneView {
  // discs in LBVH (slot) order, 32 B each: (centre, radius), (normal, original id bits)
  const float4* disc;
  int32_t nd;
  // triangles in slot order, 64 B each: (v0, original id bits), e1, e2, unit normal
  const float4* tri;
  int32_t nt;
  const Node* nodes;
  uint32_t root;        // child reference of the root (internal node 0 or a leaf)
  // the 8-wide compressed tree of the closest-hit query (root = wide node 0),
  // or nullptr: closest hits traverse the binary nodes
  const WideNode* wnodes;
  uint32_t n_wnodes;
  // neighbour CSR: rows by original disc id, columns as disc slots (the
  // neighbour's record in `disc` carries its original id)
  const int64_t* nb_ptr;
  const uint32_t* nb_slot;
  const float* sticking_field;  // by original id or nullptr
  // node visits after which one closest-hit (or interval) query ends and
  // counts as an error
  uint32_t max_visits;
};

// The segment log of a trace (rtg_set_segment_log): records of the source
// rays [ray_begin, ray_end), rec == nullptr when off.
struct SegmentLog {
  rtg_segment* rec;
  unsigned long long cap;
  unsigned long long* count;  // records asked for (kept: min(count, cap))
  uint64_t ray_begin, ray_end;
};

struct TraceParams {
  SceneView s;
  // accumulators by original primitive id
  double* s1;
  double* s2;
  double* s3;
  double* s4;
  unsigned long long* cnt;
  DevTally* tally;
  volatile uint32_t* abort_flag;  // host-mapped; nonzero asks the kernel to stop
  uint64_t ray_begin, ray_end;
  uint64_t seed;
  float box_lo[3], box_hi[3];
  float src_lo[2], src_hi[2];
  float tnear;
  float sticking;
  float source_exponent, source_ee;
  float specular_fraction;
  double roulette_threshold, roulette_weight;
  int32_t x_periodic, y_periodic;
  int32_t reflection;
  uint32_t max_segments;
  uint32_t job;
  int32_t packet;  // a warp takes new source rays when at least this many lanes are idle
  int32_t plain;   // 1: one source ray per thread, no refill (grid covers all rays)
  int32_t fixed_s1;       // 1: s1 holds int64 multiples of 2^-32 during the trace (RTG_ACCUM_FIXED)
  int32_t window;         // 1: multi-hit window deposit (RTG_DEPOSIT_WINDOW), traced by kModeWindow
  float window_factor;    // window length in radii of the disc that opens it
  // adjoint replay (unused by the forward trace)
  const double* adj_g;     // dL/dS1 by primitive id
  double* adj_field;       // dL/ds_j by primitive id (sticking-field mode) or nullptr
  double* adj_scalars;     // [0] dL/ds (global sticking), [1] dL/dn (source exponent)
  double adj_inv_n1;       // 1 / (n + 1)
  int32_t adj_unbiased;    // 0: roulette decisions held as drawn; 1: with their likelihood ratio
  SegmentLog log;          // forward traces (kModeLogged)
};

// Path-kernel modes: the forward trace, and two adjoint replays of the same
// paths (same Philox counters, same arithmetic).
constexpr int kModeForward = 0;
constexpr int kModeAdjGlobal = 1;  // dL/ds (one global sticking) and dL/dn
constexpr int kModeAdjField = 2;   // dL/ds_j (sticking field) and dL/dn
constexpr int kModeWindow = 3;     // forward trace with the multi-hit window deposit
constexpr int kModeLogged = 4;     // forward trace that also fills the segment log

// ---- device buffers owned by a context ----
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
};

struct Geometry {
  int64_t nd = 0, nt = 0, nv = 0;
  // inputs by original id
  DBuf<float4> disc_cr_by_id, disc_n_by_id;
  DBuf<float4> tri_v;      // nv vertices (xyz, 0)
  DBuf<uint32_t> tri_idx;  // nt*3
  // slot-ordered copies
  DBuf<float4> disc;       // 2 per slot: (centre, radius), (normal, id bits)
  DBuf<float4> tri;        // 4 per slot: (v0, id bits), e1, e2, unit normal
  DBuf<Node> nodes;
  DBuf<uint32_t> leaf_ref;    // per sorted leaf i: child reference
  DBuf<int32_t> leaf_prim;    // per sorted leaf i: original primitive id
  DBuf<uint32_t> parent;      // parent of internal nodes [0,n-1) and leaves [n-1, 2n-1)
  DBuf<float> prim_lo, prim_hi;  // per original id, 3 floats each (padded boxes)
  DBuf<unsigned int> refit_flags;
  uint32_t root = 0;
  // neighbours
  DBuf<int64_t> nb_ptr;
  DBuf<int32_t> nb_idx;       // columns as original ids
  DBuf<uint32_t> nb_slot;     // the same columns as disc slots (read by the trace)
  DBuf<uint32_t> disc_slot;   // by original disc id: its slot
  int64_t nb_nnz = 0;
  // centre extents and max radius (rti's box rule)
  float cmin[3] = {0, 0, 0}, cmax[3] = {0, 0, 0};
  float rmax = 0.0f;
  float tri_min[3] = {0, 0, 0}, tri_max[3] = {0, 0, 0};
  int32_t depth = 0;  // internal nodes on the longest root-to-leaf path
  int32_t builder = 0;  // kBuilderKarras or kBuilderPloc
  // 8-wide compressed tree (rtg_wide.cu)
  DBuf<WideNode> wnodes;
  uint32_t n_wnodes = 0;
  int32_t wide_stack = 0;  // traversal stack entries the wide tree can need
  bool wide_current = false;  // wnodes were collapsed from the current binary tree (n_wnodes 0: unusable)
};

// Wavefront scheduling state (device buffers, lazily allocated).
struct Wavefront {
  DBuf<float4> ow[2];           // per path slot: (o.xyz, w)
  DBuf<float4> dk[2];           // (d.xyz, bits of k)
  DBuf<uint4> meta[2];          // (id lo, id hi, job, nseg)
  DBuf<float> hit_t;
  DBuf<int32_t> hit_id;
  DBuf<uint32_t> hit_ref;
  DBuf<unsigned long long> ctl;  // see rtg_wavefront.cu
  DBuf<TraceParams> one_job;     // job table of a single (unbatched) trace
  DBuf<uint64_t> one_prefix;
  unsigned long long* h_ctl = nullptr;  // pinned copy of ctl
  uint32_t capacity = 0;
};

}  // namespace rtg

struct rtg_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  rtg_config cfg{};
  rtg::Geometry g;
  rtg::DBuf<float> sticking_field;
  // accumulators (one allocation: s1 | s2 | s3 | s4), counts, areas, estimates
  rtg::DBuf<double> acc;
  rtg::DBuf<unsigned long long> cnt;
  rtg::DBuf<float> areas;
  rtg::DBuf<float> est;
  rtg::DBuf<double> stat_tmp;
  // segment log (rtg_set_segment_log)
  rtg::DBuf<rtg_segment> seglog;
  rtg::DBuf<unsigned long long> seglog_count;
  uint64_t seglog_begin = 0, seglog_end = 0;
  rtg::DevTally* d_tally = nullptr;
  rtg::DevTally* d_tally_adj = nullptr;  // counters of adjoint replays
  uint32_t* h_abort = nullptr;  // host-mapped flag
  uint32_t* d_abort = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
  uint64_t last_rays = 0;
  bool traced = false;
  bool finalized = false;
  float box_lo[3] = {0, 0, 0}, box_hi[3] = {0, 0, 0};
  rtg_launch_config lc{128, 1, 0, RTG_SCHED_MEGAKERNEL, RTG_LEAF_IMMEDIATE, RTG_STACK_AUTO};
  int32_t node_width = 0;  // RTG_NODES_*: closest hits over the binary or the wide tree
  int32_t deposit_mode = RTG_DEPOSIT_NEIGHBORS;
  int32_t accum = RTG_ACCUM_FP64;
  float window_factor = 5.0f;  // point_cloud_context.hpp:163
  uint64_t visit_limit = 0;    // 0: 4 x primitives + 64, more than a valid tree needs
  // bumped whenever the surface's device buffers, its tree or a trace input
  // that a batch job captured (sticking field, visit limit) may have changed
  uint64_t version = 0;
  // fault injection: real device allocations left before one fails (-1: off)
  int64_t alloc_failure_in = -1;
  rtg::Wavefront wf;
  std::string err;
};

namespace rtg {

// A named range on the host timeline for profilers (NVTX; a no-op unless a
// profiling tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// sort.cu
int exclusive_scan_u32(rtg_context* ctx, uint32_t* d_a, int64_t m, uint32_t* d_total, cudaStream_t st);
int exclusive_scan_i64(rtg_context* ctx, int64_t* d_a, int64_t m, int64_t* d_total, cudaStream_t st);
int radix_sort_pairs(rtg_context* ctx, uint32_t* d_keys, uint32_t* d_vals, uint32_t* d_tmp_keys,
                     uint32_t* d_tmp_vals, int64_t n, int bits, cudaStream_t st);
// lbvh.cu
int build_lbvh(rtg_context* ctx);      // full build from the by-id primitive data
int refit_lbvh(rtg_context* ctx);      // recompute boxes, keep topology
// wide.cu: the 8-wide compressed tree from the binary one (after a build or
// refit when the context wants it, else before the first trace that does)
int build_wide(rtg_context* ctx, cudaStream_t st);
// whether the node width setting asks for the wide tree on this surface
bool wants_wide(const rtg_context* ctx);
// collapses the wide tree if it is wanted and not current (synchronises)
int ensure_wide(rtg_context* ctx);
// surface.cu
int build_neighbors(rtg_context* ctx);
int compute_areas(rtg_context* ctx, cudaStream_t st, const float* box_lo, const float* box_hi);
int finalize_estimates(rtg_context* ctx, cudaStream_t st);
int compute_stats(rtg_context* ctx, cudaStream_t st, uint64_t total, double* d_rel, double* d_vov);
// trace.cu: a single trace with the context's launch configuration
int launch_trace(rtg_context* ctx, const TraceParams& p, cudaStream_t st, int mode = kModeForward);
// closest hits of explicit rays; queries that reach a traversal limit are
// counted in *d_errors
int launch_closest_hit(rtg_context* ctx, const float* d_rays, int64_t n, float tnear, int32_t* d_prim,
                       float* d_t, unsigned long long* d_errors, cudaStream_t st);
SceneView scene_view(rtg_context* ctx);
// whether the binary tree and the primitive records of ctx outgrow the L2 cache
bool outgrows_l2(const rtg_context* ctx);
// whether closest hits of ctx traverse the wide tree (chosen, built, and its
// stack need within the largest stack)
bool use_wide(const rtg_context* ctx);
// the traversal stack depth a query of ctx can need (binary tree depth, or
// the wide tree's stack need when it is used)
int traversal_depth(const rtg_context* ctx);
// stack entries for a requested depth (0 = automatic) and a tree depth: 32, 64 or 256
int stack_for(int requested, int tree_depth);
// RTG_ACCUM_FIXED: s1 between double and int64 multiples of 2^-32, in place
int s1_to_fixed(rtg_context* ctx, double* s1, int64_t n, cudaStream_t st);
int s1_to_double(rtg_context* ctx, double* s1, int64_t n, cudaStream_t st);
// whether a trace of ctx under lc keeps its traversal stacks in shared memory
bool shared_stack(rtg_context* ctx, const rtg_launch_config& lc);
int check_launch_config(rtg_context* ctx, const rtg_launch_config& lc);
// trace_batched.cu: the megakernel over a job table (forward only)
// (wide: some job's scene view carries a wide tree)
int launch_trace_batched(rtg_context* ctx, const TraceParams& p0, const TraceParams* d_jobs, const uint64_t* d_prefix,
                         int njobs, uint64_t total_rays, cudaStream_t st, const rtg_launch_config& lc,
                         int tree_depth, bool wide);
// wavefront.cu: the same paths scheduled as extend/shade kernel pairs over a
// path queue (forward only; host-driven loop, not capturable)
int launch_wavefront(rtg_context* ctx, const TraceParams& p0, const TraceParams* d_jobs, const uint64_t* d_prefix,
                     int njobs, uint64_t total_rays, cudaStream_t st, const rtg_launch_config& lc, int tree_depth);
void free_wavefront(Wavefront& wf);
int compute_areas_into(rtg_context* ctx, cudaStream_t st, const float* box_lo, const float* box_hi, float* out);

// api.cu helpers
int check_config(rtg_context* ctx, const rtg_config& c);
// Frees the surface after a failed upload, update or rebuild (whose buffers
// may no longer agree with one another): later traces report
// RTG_ERR_NO_GEOMETRY until an upload succeeds.
void drop_surface(rtg_context* ctx);
void box_for(const rtg_config& c, const Geometry& g, float* box_lo, float* box_hi);
int prepare_trace_with(rtg_context* ctx, const rtg_config& c, const float* box_lo, const float* box_hi,
                       uint64_t ray_begin, uint64_t ray_end, uint64_t seed, TraceParams& p);
int set_error(rtg_context* ctx, int code, const std::string& msg);
int check_cuda(rtg_context* ctx, cudaError_t e, const char* what);
// Runs an entry point's body and turns a C++ exception (a failed host
// allocation, above all) into an error code, so that none crosses the C ABI.
template <typename F>
int host_guard(rtg_context* ctx, F&& f) noexcept {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    if (!ctx) return RTG_ERR_OUT_OF_MEMORY;
    try {
      return set_error(ctx, RTG_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (...) {
      return RTG_ERR_OUT_OF_MEMORY;
    }
  } catch (...) {
    if (!ctx) return RTG_ERR_INVALID_ARGUMENT;
    try {
      return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "unexpected host exception");
    } catch (...) {
      return RTG_ERR_INVALID_ARGUMENT;
    }
  }
}
// Fault injection (rtg_inject_alloc_failure): whether this allocation is the
// one chosen to fail.
inline bool injected_alloc_failure(rtg_context* ctx) {
  if (ctx->alloc_failure_in < 0) return false;
  return ctx->alloc_failure_in-- == 0;  // fails once, then -1 (off)
}
template <typename T>
int dalloc(rtg_context* ctx, DBuf<T>& b, size_t n, const char* what) {
  if (b.p && b.n >= n && n > 0) {
    b.n = n;
    return RTG_OK;
  }
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.n = 0;
  if (n == 0) return RTG_OK;
  if (injected_alloc_failure(ctx))
    return set_error(ctx, RTG_ERR_OUT_OF_MEMORY, std::string("cudaMalloc failed for ") + what + " (injected)");
  cudaError_t e = cudaMalloc((void**)&b.p, n * sizeof(T));
  if (e != cudaSuccess) {
    b.p = nullptr;
    cudaGetLastError();
    return set_error(ctx, RTG_ERR_OUT_OF_MEMORY, std::string("cudaMalloc failed for ") + what);
  }
  b.n = n;
  return RTG_OK;
}
template <typename T>
void dfree(DBuf<T>& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.n = 0;
}
// Temporaries of a build step: stream-ordered allocations from the device's
// memory pool, released on the same stream without the device-wide
// synchronisation of cudaFree.
template <typename T>
int talloc(rtg_context* ctx, DBuf<T>& b, size_t n, cudaStream_t st, const char* what) {
  b.p = nullptr;
  b.n = 0;
  if (n == 0) return RTG_OK;
  if (injected_alloc_failure(ctx))
    return set_error(ctx, RTG_ERR_OUT_OF_MEMORY, std::string("cudaMallocAsync failed for ") + what + " (injected)");
  cudaError_t e = cudaMallocAsync((void**)&b.p, n * sizeof(T), st);
  if (e != cudaSuccess) {
    b.p = nullptr;
    cudaGetLastError();
    return set_error(ctx, RTG_ERR_OUT_OF_MEMORY, std::string("cudaMallocAsync failed for ") + what);
  }
  b.n = n;
  return RTG_OK;
}
template <typename T>
void tfree(DBuf<T>& b, cudaStream_t st) {
  if (b.p) cudaFreeAsync(b.p, st);
  b.p = nullptr;
  b.n = 0;
}

// device helpers shared by the kernels
__host__ __device__ inline int num_sms_hint() { return 152; }

}  // namespace rtg

#define RTG_CUDA(ctx, call)                                              \
  do {                                                                   \
    cudaError_t e__ = (call);                                            \
    if (e__ != cudaSuccess) return rtg::check_cuda((ctx), e__, #call);   \
  } while (0)

#define RTG_TRY(expr)            \
  do {                           \
    int r__ = (expr);            \
    if (r__ != RTG_OK) return r__; \
  } while (0)
