/*
 * rtg.h -- C ABI of the GB300 flux engine (librtg.so).
 *
 * The engine computes Monte Carlo particle flux onto surfaces made of
 * oriented discs and/or triangles, the job of rti::device / rti::trace::tracer
 * in the rti library.  Every entry point takes plain pointers and sizes, returns
 * an int status (RTG_OK = 0) and never throws; rtg_last_error() describes the
 * last failure on a context.  One context belongs to one host thread at a
 * time.  Host arrays are read during the call and not retained.
 *
 * Reference interfaces replaced (paths within the rti project):
 *   rtg_create / rtg_destroy        device.hpp:42-45 (ctor), :84-85,:101 (Embree device)
 *   rtg_upload_discs                device.hpp:47-60 set_points/set_normals/set_grid_spacing,
 *                                   device.hpp:86-88, point_cloud_disc_geometry.hpp:119-232
 *   rtg_upload_triangles            triangle_geometry.hpp:56-99, i_triangle_reader.hpp:22-38
 *   rtg_upload_mixed                (no counterpart: discs and triangles in one scene)
 *   rtg_update_discs / _vertices    (no counterpart: bounding-box refit for moved surfaces)
 *   rtg_config_default/rtg_set_config  device.hpp:62-80 set_number_of_rays/set_x/set_y/set,
 *                                   tracer.hpp:179 (tnear), rejection_control.hpp:16,22
 *   rtg_set_sticking / _field       i_particle.hpp:14 get_sticking_probability
 *   rtg_trace                       tracer.hpp:66-330 tracer::run
 *   rtg_trace_rays                  tracer.hpp:181 rtcIntersect1 on caller-given rays
 *   rtg_get_mc_estimates            device.hpp:109-112, :154-187
 *   rtg_get_hit_counts              device.hpp:114-117, hit_accumulator.hpp:144-146
 *   rtg_get_accumulators            hit_accumulator.hpp:140-142 (values, S1..S4)
 *   rtg_get_exposed_areas           hit_accumulator.hpp:256-259, tracer.hpp:385-413
 *   rtg_get_relative_error/_vov     hit_accumulator.hpp:152-249
 *   rtg_get_tally                   result.hpp:11-33 (numRays, hitc, nonhitc, time)
 *   rtg_get_neighbors               point_cloud_disc_geometry.hpp:103-106
 *   rtg_device_run                  device.hpp:82-107 device::run in one call
 */
#ifndef RTG_H
#define RTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTG_ABI_VERSION 1

#if defined(__GNUC__)
#define RTG_API __attribute__((visibility("default")))
#else
#define RTG_API
#endif

/* status codes */
#define RTG_OK 0
#define RTG_ERR_INVALID_ARGUMENT 1
#define RTG_ERR_CUDA 2
#define RTG_ERR_OUT_OF_MEMORY 3
#define RTG_ERR_NO_GEOMETRY 4
#define RTG_ERR_BUDGET 5      /* a device-side iteration limit was reached */
#define RTG_ERR_ABORTED 6     /* rtg_request_abort() stopped a trace */
#define RTG_ERR_INTERNAL 7

/* boundary conditions: rti::geo::bound_condition (bound_condition.hpp:4-6) */
#define RTG_BOUND_REFLECTIVE 0
#define RTG_BOUND_PERIODIC 1

/* re-emission: diffuse.hpp, specular.hpp, or a mixture of both */
#define RTG_REFLECT_DIFFUSE 0
#define RTG_REFLECT_SPECULAR 1
#define RTG_REFLECT_MIXED 2

/* box_mode */
#define RTG_BOX_FROM_GEOMETRY 0 /* rti rule: x/y = centre extents, top = max z + 2 r_max */
#define RTG_BOX_EXPLICIT 1      /* box_lo/box_hi as given (box_hi[2] is the source plane) */

typedef struct rtg_context rtg_context;

typedef struct rtg_config {
  int32_t  x_bound;            /* RTG_BOUND_*; rti default REFLECTIVE (device.hpp:292) */
  int32_t  y_bound;
  int32_t  reflection;         /* RTG_REFLECT_* */
  float    specular_fraction;  /* probability of a specular bounce for RTG_REFLECT_MIXED */
  float    sticking;           /* global sticking probability (used when no field is set) */
  float    source_exponent;    /* cos^n source; 1 = rti's cosine_direction_z */
  int32_t  box_mode;           /* RTG_BOX_* */
  float    box_lo[3];
  float    box_hi[3];
  float    tnear;              /* 1e-4 (tracer.hpp:179, source.hpp:32) */
  double   roulette_threshold; /* 0.1 (rejection_control.hpp:16) */
  double   roulette_weight;    /* 0.3 (rejection_control.hpp:22) */
  uint32_t max_segments;       /* closest-hit queries per path before it is cut */
  uint32_t job;                /* random-stream tag; 0 for a plain trace */
} rtg_config;

typedef struct rtg_tally {
  uint64_t num_rays;     /* result.hpp numRays */
  uint64_t hitc;         /* front-face hits (tracer.hpp:229) */
  uint64_t nonhitc;      /* paths that left through the top/bottom (tracer.hpp:186) */
  uint64_t total;        /* accumulator uses (hit_accumulator mTotalCnts) */
  uint64_t segments;     /* closest-hit queries */
  uint64_t truncated;    /* paths cut at max_segments */
  uint64_t nb_deposits;  /* neighbour deposits (tracer.hpp:371) */
  uint64_t errors;       /* device-side guard trips (stack/iteration limits) */
  double   trace_ms;     /* device time of the last rtg_trace (zeroing + paths + areas) */
  double   kernel_ms;    /* device time of the path kernel alone in the last rtg_trace */
} rtg_tally;

/* How the paths are scheduled on the GPU (no counterpart in rti, whose
 * OpenMP loop has no such knobs).  None of these changes a result: every
 * path is the same Philox-indexed computation whichever lane runs it.
 *   RTG_SCHED_MEGAKERNEL: one persistent kernel carries every path to its end;
 *   RTG_SCHED_WAVEFRONT: paths wait in a queue in device memory and advance
 *     one segment per pair of kernels (closest hit, then shading), with the
 *     surviving paths compacted between segments (forward traces only; the
 *     adjoint replays always use the megakernel);
 *   RTG_SCHED_PLAIN: a non-persistent launch, one thread per source ray that
 *     traces its path to the end (the plain GPU baseline; forward traces). */
#define RTG_SCHED_MEGAKERNEL 0
#define RTG_SCHED_WAVEFRONT 1
#define RTG_SCHED_PLAIN 2
typedef struct rtg_launch_config {
  int32_t threads_per_block; /* 64, 128 or 256 */
  int32_t packet;            /* 1..32: a warp takes new source rays when at least this many lanes are idle */
  int32_t stack_depth;       /* traversal stack entries, 32, 64 or 256; 0 = the smallest that holds the
                                tree (a smaller request than the tree needs is raised to that) */
  int32_t scheduling;        /* RTG_SCHED_* */
  int32_t leaf_tests;        /* RTG_LEAF_*: when the primitives of a leaf the ray reaches are tested */
  int32_t stack_memory;      /* RTG_STACK_*: where the traversal stack of the path kernel lives */
} rtg_launch_config;
/* leaf_tests: on the spot, or postponed until every lane of the warp holds a
 * leaf (Aila and Laine's while-while traversal; megakernel and plain
 * schedules, forward traces) */
#define RTG_LEAF_IMMEDIATE 0
#define RTG_LEAF_POSTPONED 1
/* stack_memory: per-thread local memory (cached in L1 beside the tree), or
 * shared memory (one column per thread, conflict-free), which leaves L1 to
 * the tree but takes its share of the SM's L1/shared capacity.  Shared is
 * used where the stack fits 16 KB per block (stack entries x block size x 4 B)
 * and falls back to local otherwise (larger shared stacks starve L1).  AUTO:
 * shared when the tree and the primitive records outgrow the L2 cache
 * (measured: a 4.19 M-disc surface traces 6 % faster with it, a 200 k-triangle
 * surface 2 % slower). */
#define RTG_STACK_AUTO 0
#define RTG_STACK_LOCAL 1
#define RTG_STACK_SHARED 2

/* Fills *cfg with rti's defaults. */
RTG_API void rtg_config_default(rtg_config* cfg);
RTG_API int  rtg_abi_version(void);

RTG_API int  rtg_create(rtg_context** ctx, int device);
RTG_API int  rtg_destroy(rtg_context* ctx);
RTG_API const char* rtg_last_error(const rtg_context* ctx);

/* points: n x 3 centres, normals: n x 3 unit normals, radii: n (rti's "grid
 * spacing", used as the disc radius, device.hpp:213-216).  Builds the LBVH and
 * the neighbour lists.  Replaces any previous geometry; clears the sticking
 * field.  The arrays are checked on the device before anything is replaced:
 * a refused upload (non-finite value, radius <= 0, normal not of unit length,
 * index out of range) leaves the previous surface as it was.  An upload,
 * update (rtg_update_*) or tree rebuild (rtg_set_tree_builder) that fails
 * after that point -- RTG_ERR_OUT_OF_MEMORY while the tree is built, a CUDA
 * error -- leaves the context without a surface: traces report
 * RTG_ERR_NO_GEOMETRY until an upload succeeds. */
RTG_API int rtg_upload_discs(rtg_context* ctx, const float* points, const float* normals, const float* radii,
                     int64_t n);
/* vertices: nv x 3, indices: nt x 3 (uint32).  Replaces any previous geometry. */
RTG_API int rtg_upload_triangles(rtg_context* ctx, const float* vertices, const uint32_t* indices, int64_t nv,
                         int64_t nt);
/* Discs and triangles in one surface: primitive ids are the discs 0..nd-1,
 * then the triangles nd..nd+nt-1.  Either part may be empty. */
RTG_API int rtg_upload_mixed(rtg_context* ctx, const float* points, const float* normals, const float* radii, int64_t nd,
                     const float* vertices, const uint32_t* indices, int64_t nv, int64_t nt);
/* Moves the surface without changing its topology: refits the LBVH boxes and
 * rebuilds the neighbour lists; the tree itself is kept. */
RTG_API int rtg_update_discs(rtg_context* ctx, const float* points, const float* normals, const float* radii,
                     int64_t n);
RTG_API int rtg_update_vertices(rtg_context* ctx, const float* vertices, int64_t nv);

RTG_API int rtg_set_config(rtg_context* ctx, const rtg_config* cfg);
RTG_API int rtg_get_config(const rtg_context* ctx, rtg_config* cfg);
/* The box the trace uses (after RTG_BOX_FROM_GEOMETRY is resolved). */
RTG_API int rtg_get_box(const rtg_context* ctx, float* box_lo3, float* box_hi3);
RTG_API int rtg_set_sticking(rtg_context* ctx, float sticking);
/* per-primitive sticking (length = number of primitives); NULL clears it */
RTG_API int rtg_set_sticking_field(rtg_context* ctx, const float* sticking, int64_t n);

/* Launch configuration of the traces of a context (default: 128 threads,
 * packet 1, automatic stack, megakernel). */
RTG_API void rtg_launch_config_default(rtg_launch_config* lc);
RTG_API int rtg_set_launch_config(rtg_context* ctx, const rtg_launch_config* lc);
RTG_API int rtg_get_launch_config(const rtg_context* ctx, rtg_launch_config* lc);
/* Internal nodes on the longest root-to-leaf path of the context's LBVH. */
RTG_API int rtg_get_tree_depth(const rtg_context* ctx, int32_t* depth);
/* Topology of the tree over the Morton-sorted primitives (no counterpart in
 * rti, whose Embree build quality is fixed at HIGH, tracer.hpp:85):
 *   RTG_TREE_KARRAS: radix tree split at the highest differing key bit
 *     (Karras, HPG 2012); the fastest build; best on regular grids;
 *   RTG_TREE_PLOC: locally-ordered clustering by merged surface area (Meister
 *     and Bittner, TVCG 2018); 2-3x the build time, fewer node visits on
 *     irregular surfaces.
 * Setting it rebuilds the tree of the current geometry and applies to later
 * uploads.  Results do not depend on it.  rtg_autotune tries both. */
#define RTG_TREE_KARRAS 0
#define RTG_TREE_PLOC 1
RTG_API int rtg_set_tree_builder(rtg_context* ctx, int32_t builder);
RTG_API int rtg_get_tree_builder(const rtg_context* ctx, int32_t* builder);
/* Which tree the closest-hit queries traverse (no counterpart in rti; Embree
 * chooses its own):
 *   RTG_NODES_BINARY (2): the binary tree itself (64-byte nodes, both child
 *     boxes in float);
 *   RTG_NODES_WIDE (8): a compressed 8-wide tree collapsed from it after every
 *     build and refit (96-byte nodes, child boxes as bytes on a per-node
 *     power-of-two grid, children ordered by direction).  Its boxes contain
 *     the binary boxes, so results are the same bit for bit;
 *   RTG_NODES_AUTO (0, the default): wide when the binary nodes and the
 *     primitive records outgrow the L2 cache, else binary.  Measured: the wide
 *     tree moves a third less DRAM traffic and traces a 4.19 M-disc surface
 *     13-16 % faster, but costs more instructions per query and traces
 *     L2-resident surfaces (200 k triangles, 98 k discs) 3-10 % slower.
 * A scene with a node wider than 4080 units, or a wide tree whose traversal
 * stack would exceed 256 entries, is traced over the binary tree whatever this
 * says.  The postponed leaf tests (RTG_LEAF_POSTPONED) and the multi-hit
 * window's interval queries always use the binary tree.  rtg_autotune tries
 * both for its fastest candidates. */
#define RTG_NODES_AUTO 0
#define RTG_NODES_BINARY 2
#define RTG_NODES_WIDE 8
RTG_API int rtg_set_node_width(rtg_context* ctx, int32_t width);
RTG_API int rtg_get_node_width(const rtg_context* ctx, int32_t* width);
/* The tree the closest-hit queries of the next trace use: 2 (binary) or 8. */
RTG_API int rtg_get_traversal_width(const rtg_context* ctx, int32_t* width);
/* What a front-face disc hit deposits.  rti has two treatments of
 * overlapping discs:
 *   RTG_DEPOSIT_NEIGHBORS (default): w*s on the hit disc and on every
 *     overlapping neighbour disc the ray crosses, then w -= w*s -- rti's
 *     tracer (tracer.hpp:229-240,339-383);
 *   RTG_DEPOSIT_WINDOW: the multi-hit window of rti's point-cloud context
 *     (trace/point_cloud_context.hpp:132-173,265-286): the window opens at the
 *     closest front-face disc hit t0 (rti: whichever hit Embree's filter
 *     reports first) and reaches to t0 + window_factor * r0 (r0 that disc's
 *     radius; rti: 5), closed earlier by the first back-face disc hit beyond
 *     t0 or by the x/y box; every disc hit from the front within it receives
 *     w*s_j (s_j its own sticking), and w drops by the mean of those deposits.
 *     Forward traces of one context only: rtg_adjoint and rtg_batch_add
 *     refuse a context in this mode.  Triangles deposit on the hit triangle.
 * Applies to later traces; window_factor >= 0 is used by RTG_DEPOSIT_WINDOW. */
#define RTG_DEPOSIT_NEIGHBORS 0
#define RTG_DEPOSIT_WINDOW 1
RTG_API int rtg_set_deposit_mode(rtg_context* ctx, int32_t mode, float window_factor);
RTG_API int rtg_get_deposit_mode(const rtg_context* ctx, int32_t* mode, float* window_factor);
/* How the flux S1 is summed during a trace (S2..S4 are always FP64):
 *   RTG_ACCUM_FP64 (default): FP64 atomics, as rti's double accumulators; the
 *     last bits of a sum depend on the order of the atomics;
 *   RTG_ACCUM_FIXED: every deposit rounded to a multiple of 2^-32 and summed
 *     in 64-bit integers, converted to double when the trace ends: the sums do
 *     not depend on the order, so repeated traces (and sharded ones summed in
 *     any order) give the same S1 bit for bit.  Up to 2^31 per primitive.
 * Single traces of a context (a batch refuses a context in fixed mode). */
#define RTG_ACCUM_FP64 0
#define RTG_ACCUM_FIXED 1
RTG_API int rtg_set_accumulation(rtg_context* ctx, int32_t mode);
RTG_API int rtg_get_accumulation(const rtg_context* ctx, int32_t* mode);
/* Work limit of one closest-hit query: after `visits` tree nodes the query
 * ends and counts as an error (tally.errors), the getters of that trace then
 * return RTG_ERR_BUDGET.  0 (default) = 4 x primitives + 64, which a valid
 * tree never reaches; a larger value is capped there.  Bounds the work of a
 * trace on a damaged or adversarial tree.  Applies to later traces. */
RTG_API int rtg_set_visit_limit(rtg_context* ctx, uint64_t visits);
RTG_API int rtg_get_visit_limit(const rtg_context* ctx, uint64_t* visits);
/* Fault injection for tests of the error paths: after `after` further device
 * allocations of this context succeed, the next one fails as if the device
 * were out of memory (once); after < 0 cancels.  The call that meets it
 * returns RTG_ERR_OUT_OF_MEMORY; an upload, update or rebuild then leaves the
 * context without a surface (see rtg_upload_discs), any other call leaves the
 * context as it was. */
RTG_API int rtg_inject_alloc_failure(rtg_context* ctx, int64_t after);
/* Autotuner: for each tree builder (RTG_TREE_*), times each candidate launch
 * configuration (block size x packet x stack depth x leaf tests, megakernel
 * or plain; the wavefront schedule, slower on every workload measured, is
 * left to rtg_set_launch_config) on source
 * rays [0, sample_rays) with `seed` under the current surface and
 * configuration, over the node width RTG_NODES_AUTO picks; re-times the three
 * fastest of each tree with their stacks in the other memory and over the
 * other node width; keeps the fastest as the context's tree, node width and
 * launch configuration and returns the latter (best and best_rays_per_s may
 * be NULL; rtg_get_tree_builder and rtg_get_node_width tell the rest).  Leaves
 * no trace results behind (trace again afterwards). */
RTG_API int rtg_autotune(rtg_context* ctx, uint64_t sample_rays, uint64_t seed, rtg_launch_config* best,
                         double* best_rays_per_s);

/* Traces source rays [0, n_rays) with Philox seed `seed` on `stream`
 * (a cudaStream_t, NULL = the context's stream).  Zeroes the accumulators,
 * traces, computes the exposed areas; returns after enqueueing.  The results
 * are read with the getters below (which synchronise). */
RTG_API int rtg_trace(rtg_context* ctx, uint64_t n_rays, uint64_t seed, void* stream);
/* Same, for the ray range [ray_begin, ray_end) and accumulating into the
 * current totals when accumulate != 0 (used to shard rays across GPUs). */
RTG_API int rtg_trace_range(rtg_context* ctx, uint64_t ray_begin, uint64_t ray_end, uint64_t seed,
                    int accumulate, void* stream);
RTG_API int rtg_synchronize(rtg_context* ctx);
/* Asks a running trace to stop; it returns RTG_ERR_ABORTED. */
RTG_API int rtg_request_abort(rtg_context* ctx);

/* Per-primitive sticking from a device array (e.g. a torch tensor), copied
 * into the context on `stream` (the caller's array may be freed or reused
 * after that copy in stream order); NULL clears it.  The values are not
 * checked: each must lie in [0, 1]. */
RTG_API int rtg_set_sticking_field_device(rtg_context* ctx, const float* d_field, int64_t n, void* stream);

/* Adjoint of the trace (no counterpart in rti; the differentiation path).
 * With L = sum_i g_i * S1_i, replays source rays [ray_begin, ray_end) of the
 * trace with `seed` under the current surface and configuration and ADDS
 *   d_scalars[0] += dL/ds  (global sticking; 0 when a sticking field is set),
 *   d_scalars[1] += dL/dn  (source cosine exponent, score-function estimator),
 *   d_field_grad[j] += dL/ds_j (when a sticking field is set; required then).
 * estimator: RTG_ADJ_HELD holds the Russian-roulette decisions as drawn (what
 * central differences with common random numbers measure); RTG_ADJ_UNBIASED
 * adds the likelihood ratio of each roulette survival (an unbiased gradient of
 * the expected flux).  All pointers are device pointers; enqueued on `stream`.
 * Same paths as the forward trace (same Philox counters); no per-path memory. */
#define RTG_ADJ_HELD 0
#define RTG_ADJ_UNBIASED 1
RTG_API int rtg_adjoint(rtg_context* ctx, const double* d_g, uint64_t ray_begin, uint64_t ray_end, uint64_t seed,
                        int estimator, double* d_field_grad, double* d_scalars, void* stream);
/* Host-array form of rtg_adjoint for rays [0, n_rays); synchronous. */
RTG_API int rtg_adjoint_host(rtg_context* ctx, const double* g, uint64_t n_rays, uint64_t seed, int estimator,
                             double* field_grad, double* d_sticking, double* d_exponent);

/* Closest hit for explicit rays: rays = n x 6 floats (origin, direction),
 * host pointers.  prim_out = primitive id or -1, t_out = distance.
 * Synchronous; RTG_ERR_BUDGET when a query reached the visit limit (its
 * result is then the closest hit found before it stopped). */
RTG_API int rtg_trace_rays(rtg_context* ctx, const float* rays, int64_t n, float tnear, int32_t* prim_out,
                   float* t_out);

/* Results (host buffers of the number of primitives). */
RTG_API int rtg_num_primitives(const rtg_context* ctx, int64_t* n);
RTG_API int rtg_get_mc_estimates(rtg_context* ctx, float* out);
RTG_API int rtg_get_hit_counts(rtg_context* ctx, uint64_t* out);
RTG_API int rtg_get_accumulators(rtg_context* ctx, double* s1, double* s2, double* s3, double* s4);
RTG_API int rtg_get_exposed_areas(rtg_context* ctx, float* out);
RTG_API int rtg_get_relative_error(rtg_context* ctx, double* out);
RTG_API int rtg_get_vov(rtg_context* ctx, double* out);
RTG_API int rtg_get_tally(rtg_context* ctx, rtg_tally* out);
/* Checkpoint and resume (no counterpart in rti, whose trace is one OpenMP
 * loop; the state of hit_accumulator.hpp:271-290 plus result.hpp's counts):
 * rtg_get_accumulators, rtg_get_hit_counts and rtg_get_tally save a trace of
 * the ray range [0, k); rtg_set_accumulators puts that state back into a
 * context holding the same surface and configuration, and
 * rtg_trace_range(ctx, k, n, seed, 1, stream) continues it.  Paths depend only
 * on (seed, ray id), so the result equals the trace of [0, n) in one go: the
 * same hit counts and tallies, S1 bit for bit under RTG_ACCUM_FIXED (S2..S4
 * and plain S1 up to the order of the FP64 additions).  All five arrays hold
 * rtg_num_primitives values; the tally's timings are ignored.  The call waits
 * for the device to finish its work (a trace of this context may still be
 * writing the accumulators) before it replaces them. */
RTG_API int rtg_set_accumulators(rtg_context* ctx, const double* s1, const double* s2, const double* s3,
                                 const double* s4, const uint64_t* counts, const rtg_tally* tally);
/* Neighbour CSR of the discs: row_ptr (nd+1), cols (cap entries); *nnz gets the count. */
RTG_API int rtg_get_neighbors(rtg_context* ctx, int64_t* row_ptr, int32_t* cols, int64_t cap, int64_t* nnz);

/* The special-purpose VTU readers of rti (UnstructuredGrid point clouds and
 * meshes written by other simulators):
 *   RTG_VTU_AREA (io/christoph/vtu_point_cloud_reader.hpp:31-120): radius =
 *     sqrt(point data "area_around_vertex", else cell data "gridSpacing")
 *     x sqrt(3)/2 x 1.25; normals from cell data "Normals", else point data
 *     "normal_vector"; the z coordinates of points and normals inverted;
 *   RTG_VTU_SPACING (io/xaver/vtu_point_cloud_reader.hpp:30-110): radius =
 *     cell data "gridSpacing" x sqrt(3)/2 x 1.25, z kept.
 * Both leave out points of zero area (radius) or with the zero vector as
 * normal and normalise the others' normals (utils.hpp:77-93); *n gets the
 * number kept (all outputs NULL: count only).  rtg_read_triangles_vtu is
 * io/christoph/vtu_triangle_reader.hpp:29-105: every three-point cell with its
 * second and third vertex swapped and, in `normals` (may be NULL), the mean
 * of its vertices' "normal_vector" values, normalised -- (0, 0, 1) where
 * all three components are below 1e-5, as the reference tests them (signed).
 * Where the reference would dereference a missing array, these return
 * RTG_ERR_INVALID_ARGUMENT with a message in err. */
#define RTG_VTU_AREA 1
#define RTG_VTU_SPACING 2
RTG_API int rtg_read_point_cloud_vtu(const char* path, int32_t flavor, int64_t* n, float* points, float* normals,
                                     float* radii, char* err, int32_t err_len);
RTG_API int rtg_read_triangles_vtu(const char* path, int64_t* nv, float* vertices, int64_t* nt, uint32_t* indices,
                                   float* normals, char* err, int32_t err_len);

/* Segment log (rti's RAYLOG / RAYSRCLOG of util/ray_logger.hpp:23-71, written
 * at trace/tracer.hpp:166,183,294-305, which record every ray segment and
 * source point of a single-threaded run).  Here a bounded device buffer
 * records, for the source rays [ray_begin, ray_end) of later traces, one
 * rtg_segment per closest-hit query of their paths: the query's origin and
 * where it ended (the hit point, the point where the path left the x/y box
 * sideways, or where it left through the top or bottom plane; rti draws
 * at most 10 units instead), what happened there, the primitive and the
 * particle weight.  The source points are the origins of the segments with
 * segment == 0.  rtg_set_segment_log(ctx, b, e, capacity) allocates room for
 * `capacity` records (0 frees it and stops logging); every trace that does
 * not accumulate starts the log afresh; records beyond the capacity are
 * counted, not kept.  Logging traces run one kernel configuration of their
 * own (results unchanged; not with RTG_DEPOSIT_WINDOW, nor in batches).
 * rtg_get_segment_log copies up to `cap` records, sorted by (ray, segment),
 * and reports how many were kept and how many were dropped (synchronises). */
#define RTG_SEG_HIT 0       /* front-face primitive hit: deposit, roulette, re-emission */
#define RTG_SEG_BACKFACE 1  /* back face: the path passes through */
#define RTG_SEG_BOUNDARY 2  /* x/y box side: wrapped (periodic) or mirrored (reflective) */
#define RTG_SEG_ESCAPE 3    /* left through the top or bottom plane: the path ends */
typedef struct rtg_segment {
  uint64_t ray;        /* source ray id */
  uint32_t segment;    /* closest-hit query index on the path (0 = from the source plane) */
  int32_t  kind;       /* RTG_SEG_* */
  float    org[3];
  float    end[3];
  int32_t  primitive;  /* primitive id for RTG_SEG_HIT / _BACKFACE, else -1 */
  float    weight;     /* particle weight at the segment's origin */
} rtg_segment;
RTG_API int rtg_set_segment_log(rtg_context* ctx, uint64_t ray_begin, uint64_t ray_end, uint64_t capacity);
RTG_API int rtg_get_segment_log(rtg_context* ctx, rtg_segment* out, uint64_t cap, uint64_t* n_kept,
                                uint64_t* n_dropped);
/* The log as VTK XML PolyData: one line cell per segment (two points each),
 * cell arrays ray, segment, kind, primitive, weight; the _host form writes a
 * caller's array and needs no GPU. */
RTG_API int rtg_write_segment_log_vtp(rtg_context* ctx, const char* path);
RTG_API int rtg_write_vtp_segments(const char* path, const rtg_segment* seg, int64_t n);

/* No counterpart in the reference.  The estimates of rtg_get_mc_estimates,
 * written to a device buffer the caller owns (d_out, one float per primitive),
 * enqueued on `stream` (NULL = the context's stream) without allocating or
 * freeing any device memory -- for callers whose GPU memory belongs to their
 * own pool, or who cannot take the device-wide synchronisation that cudaFree
 * implies.  The kernels wait (on the GPU, the host does not block) for the end
 * of the last trace, whichever stream it was enqueued on.  Scratch is a fixed
 * 256 KiB array in the library (at most 8388352 primitives; larger surfaces
 * are rejected with RTG_ERR_INVALID_ARGUMENT).  The first call on a device
 * (and the first after its context was reset) looks that array up and should
 * come before any stream capture.  Calls share the array: calls that overlap
 * on the GPU race.  The trace's status is not checked here (see
 * rtg_get_tally). */
RTG_API int rtg_get_mc_estimates_noalloc(rtg_context* ctx, float* d_out, void* stream);

/* VTK XML output (rti io/vtp_writer.hpp:27-139, 392-413, without VTK): an
 * ASCII PolyData file in the layout of rti's writer -- discs as vertex cells
 * with cell arrays Normals, radius, value (S1), exposed-area, hitcnt,
 * relative-error, variance-of-variance; triangles as polygon cells with the
 * same result arrays; one string field array per metadata (key, value) pair.
 * Cell i is primitive i.  hitcnt is written as UInt64 (rti: UInt32).
 * rtg_write_vtp writes a traced context (synchronises; RTG_ERR_NO_GEOMETRY
 * before the first trace); the _discs/_triangles/_mixed forms write host
 * arrays (result arrays may be NULL to leave them out) and need no GPU. */
RTG_API int rtg_write_vtp(rtg_context* ctx, const char* path, const char* const* meta_keys,
                          const char* const* meta_values, int32_t n_meta);
RTG_API int rtg_write_vtp_discs(const char* path, int64_t n, const float* points, const float* normals,
                                const float* radii, const double* value, const uint64_t* hitcnt,
                                const float* exposed_area, const double* relative_error, const double* vov,
                                const char* const* meta_keys, const char* const* meta_values, int32_t n_meta);
RTG_API int rtg_write_vtp_triangles(const char* path, int64_t nv, const float* vertices, int64_t nt,
                                    const uint32_t* indices, const double* value, const uint64_t* hitcnt,
                                    const float* exposed_area, const double* relative_error, const double* vov,
                                    const char* const* meta_keys, const char* const* meta_values, int32_t n_meta);
RTG_API int rtg_write_vtp_mixed(const char* path, int64_t nd, const float* points, const float* normals,
                                const float* radii, int64_t nv, const float* vertices, int64_t nt,
                                const uint32_t* indices, const double* value, const uint64_t* hitcnt,
                                const float* exposed_area, const double* relative_error, const double* vov,
                                const char* const* meta_keys, const char* const* meta_values, int32_t n_meta);

/* VTK XML input (rti io/vtp_point_cloud_reader.hpp:23-95,
 * io/vtp_triangle_reader.hpp:19-68, without VTK): PolyData or UnstructuredGrid,
 * DataArrays in ascii, binary (base64) or appended (raw/base64) form,
 * uncompressed or zlib-compressed (zlib builds).  No GPU needed.  Call once with
 * NULL output arrays to get the sizes, then with arrays of those sizes.
 * Point cloud: centres (n x 3), unit normals (n x 3, normalised as rti does),
 * radii from the cell array "radius", else "sqrt-of-area" * sqrt(3)/2 * (1+1/32).
 * Triangles: vertices (nv x 3) and the three-point cells (nt x 3).
 * On failure `err` (err_len bytes, may be NULL) holds the reason. */
RTG_API int rtg_read_point_cloud(const char* path, int64_t* n, float* points, float* normals, float* radii,
                                 char* err, int32_t err_len);
RTG_API int rtg_read_triangles(const char* path, int64_t* nv, float* vertices, int64_t* nt, uint32_t* indices,
                               char* err, int32_t err_len);

/* Device-resident views (valid until the geometry changes). */
typedef struct rtg_device_view {
  double*   s1;        /* S1..S4 are consecutive arrays of n doubles */
  double*   s2;
  double*   s3;
  double*   s4;
  uint64_t* counts;
  float*    areas;
  float*    estimates;
  int64_t   n;
} rtg_device_view;
RTG_API int rtg_get_device_view(rtg_context* ctx, rtg_device_view* view);

/* Batches (no counterpart in rti, which traces one geometry per
 * tracer::run, tracer.hpp:66-330; a batch replaces back-to-back runs).
 * A batch is a list of jobs, each a surface (a context with geometry), a
 * configuration (NULL = the context's), a ray count and a seed.  Job j's paths
 * use the Philox stream (seed, job tag j), so its results do not depend on the
 * other jobs or on how the batch is run.  rtg_batch_run traces all jobs in ONE
 * persistent launch whose lanes draw ray ids over the concatenated ray ranges
 * (use_graph != 0: the zeroing, the launch and the area kernels are captured
 * into a CUDA graph on the first run and replayed afterwards);
 * rtg_batch_run_sequential issues one plain launch per job, with the same
 * results.  A job keeps its configuration, ray count and seed from
 * rtg_batch_add and reads its context's surface when the batch runs: refits
 * (rtg_update_*), a new tree, a sticking field set or cleared, a new visit
 * limit and a new upload of as many primitives are seen by later runs; a run
 * whose job's context now holds another number of primitives (or none), or is
 * in window deposit or fixed-point mode, fails with RTG_ERR_INVALID_ARGUMENT.
 * The contexts must outlive the batch and must not trace while it runs. */
typedef struct rtg_batch rtg_batch;
RTG_API int rtg_batch_create(rtg_batch** out, int device);
RTG_API int rtg_batch_destroy(rtg_batch* b);
RTG_API const char* rtg_batch_last_error(const rtg_batch* b);
RTG_API int rtg_batch_add(rtg_batch* b, rtg_context* scene, const rtg_config* cfg, uint64_t n_rays, uint64_t seed,
                          int32_t* job_out);
RTG_API int rtg_batch_num_jobs(const rtg_batch* b, int32_t* n);
/* Enqueue on `stream` (NULL = the batch's own stream); returns without waiting. */
RTG_API int rtg_batch_run(rtg_batch* b, int use_graph, void* stream);
RTG_API int rtg_batch_run_sequential(rtg_batch* b, void* stream);
/* Waits for the last run; *elapsed_ms = its device time (may be NULL). */
RTG_API int rtg_batch_synchronize(rtg_batch* b, double* elapsed_ms);
/* Job results (host buffers of the job's primitive count, its context's at
 * rtg_batch_add; any may be NULL):
 * S1 (hit_accumulator.hpp:140-142), hit counts (:144-146), exposed areas. */
RTG_API int rtg_batch_get_results(rtg_batch* b, int32_t job, double* s1, uint64_t* counts, float* areas);
/* Counters over all jobs of the last run. */
RTG_API int rtg_batch_get_tally(rtg_batch* b, rtg_tally* out);
/* Launch configuration of rtg_batch_run (rtg_batch_run_sequential uses each
 * job's context configuration).  RTG_SCHED_WAVEFRONT is driven from the host
 * and is never captured: with it, rtg_batch_run(use_graph != 0) runs uncaptured. */
RTG_API int rtg_batch_set_launch_config(rtg_batch* b, const rtg_launch_config* lc);
RTG_API int rtg_batch_get_launch_config(const rtg_batch* b, rtg_launch_config* lc);
/* Autotuner of the batched launch: times the candidates of rtg_autotune (no
 * wavefront, so the pick is always graph-captured) on the first
 * sample_fraction (0 < f <= 1) of every job's rays, keeps the fastest. */
RTG_API int rtg_batch_autotune(rtg_batch* b, double sample_fraction, rtg_launch_config* best,
                               double* best_rays_per_s);

/* device::run in one call (device.hpp:82-107): host arrays in, normalised
 * smoothed estimates and hit counts out.  sticking_field may be NULL. */
RTG_API int rtg_device_run(const float* points, const float* normals, const float* radii, int64_t n,
                   const rtg_config* cfg, const float* sticking_field, uint64_t n_rays, uint64_t seed,
                   float* mc_estimates_out, uint64_t* hit_counts_out, int device);

#ifdef __cplusplus
}
#endif
#endif
