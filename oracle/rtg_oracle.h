/*
 * rtg_oracle.h -- CPU oracle for the flux-tracing path (test infrastructure).
 *
 * THIS IS TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, the smoke
 * check in __graft_entry__.py and the CPU-baseline leg of bench.py may load
 * it.  It restates, in plain C, the reference's flux-tracing algorithm
 * (rti: src/rti/trace/tracer.hpp:66-413 and the files it calls) so that the
 * CUDA path in rti_gb300/csrc can be checked against it.
 *
 * Every float operation on a ray path is a single IEEE-754 binary32 operation
 * (the library is built with -ffp-contract=off); sin/cos and pow are this
 * project's own polynomial routines evaluated with explicit fmaf, so that the
 * CUDA kernels, which follow the same formulas, produce bit-identical paths.
 */
#ifndef RTG_ORACLE_H
#define RTG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

/* Tracing parameters; mirrors rtg_config of include/rtg.h field by field. */
typedef struct orc_config {
  int32_t  x_bound;            /* 0 reflective, 1 periodic (bound_condition.hpp:4-6) */
  int32_t  y_bound;
  int32_t  reflection;         /* 0 diffuse, 1 specular, 2 mixed */
  float    specular_fraction;  /* probability of a specular bounce when mixed */
  float    sticking;           /* global sticking probability */
  float    source_exponent;    /* cos^n source, n >= 0 */
  float    box_lo[3];          /* x/y: periodic/reflective box, z: lower end */
  float    box_hi[3];          /* box_hi[2] is the source plane */
  float    src_lo[2];          /* source rectangle (normally the box x/y) */
  float    src_hi[2];
  float    tnear;              /* 1e-4 (tracer.hpp:179) */
  double   roulette_threshold; /* 0.1 (rejection_control.hpp:16) */
  double   roulette_weight;    /* 0.3 (rejection_control.hpp:22) */
  uint32_t max_segments;       /* per-path cap on closest-hit queries */
  uint32_t job;                /* Philox stream tag (instance/species) */
  uint64_t seed;
  const float* sticking_field; /* per-primitive sticking, or NULL */
  int32_t  window;             /* 1: multi-hit window deposit (point_cloud_context.hpp) */
  float    window_factor;      /* window length in radii of the disc that opens it (rti: 5) */
  int32_t  accum_fixed;        /* 1: S1 summed as int64 multiples of 2^-32 (order-independent) */
} orc_config;

typedef struct orc_tally {
  uint64_t hitc;        /* front-face primitive hits (tracer.hpp:229) */
  uint64_t nonhitc;     /* paths that left the domain (tracer.hpp:186) */
  uint64_t total;       /* accumulator uses (hit_accumulator.hpp:132) */
  uint64_t segments;    /* closest-hit queries */
  uint64_t truncated;   /* paths stopped by max_segments */
  uint64_t nb_deposits; /* neighbour deposits (tracer.hpp:371) */
} orc_tally;

/* One segment of a path (the layout of the library's segment-log record):
 * kind 0 front-face hit, 1 back face passed, 2 x/y box side, 3 out through
 * the top or bottom plane; end = org + t dir as the path computes its next
 * origin. */
typedef struct orc_segment {
  uint64_t ray;
  uint32_t segment;
  int32_t kind;
  float org[3];
  float end[3];
  int32_t primitive;
  float weight;
} orc_segment;

orc_scene* orc_scene_create(const float* disc_xyzr, const float* disc_normals, int64_t n_discs,
                            const float* tri_vertices, const uint32_t* tri_indices,
                            int64_t n_vertices, int64_t n_triangles);
void    orc_scene_destroy(orc_scene* s);
int64_t orc_num_primitives(const orc_scene* s);
/* Neighbour lists (CSR, each row sorted ascending); returns nnz, or -1 if
 * cap is too small.  row_ptr has n_discs+1 entries. */
int64_t orc_neighbors(orc_scene* s, int64_t* row_ptr, int32_t* cols, int64_t cap);
/* Rebuild the neighbour lists of the scene with the brute-force pair test. */
int64_t orc_neighbors_bruteforce(orc_scene* s, int64_t* row_ptr, int32_t* cols, int64_t cap);

/* disc_bounding_box_intersector::area_inside for one disc. */
float orc_area_inside(float xmin, float ymin, float xmax, float ymax,
                      const float* disc_xyzr, const float* normal);
/* Exposed areas of all primitives (discs clipped to the box, triangle areas). */
void orc_areas(const orc_scene* s, float xmin, float ymin, float xmax, float ymax, float* out);

/* local_intersector::intersect (local_intersector.hpp:41-97). */
int orc_local_intersect(const float* org, const float* dir, const float* disc_xyzr,
                        const float* normal);

/* Closest hit over the primitives for explicit rays [ox oy oz dx dy dz] x n. */
void orc_closest_hit(const orc_scene* s, const float* rays, int64_t n, float tnear,
                     int32_t* prim_out, float* t_out);

/* Trace source rays [ray_begin, ray_end) with nthreads OpenMP threads.
 * Accumulators (length = number of primitives) are ADDED to. */
int orc_trace(const orc_scene* s, const orc_config* cf, uint64_t ray_begin, uint64_t ray_end,
              int nthreads, double* s1, double* s2, double* s3, double* s4, uint64_t* cnt,
              orc_tally* tally);

/* Adjoint replay of rays [ray_begin, ray_end): with L = sum_i g_i S1_i adds
 * dL/ds (global sticking) to scalars[0] and dL/dn (source exponent) to
 * scalars[1]; with a sticking field in cf adds dL/ds_j to field_grad.
 * unbiased = 0 holds the roulette decisions as drawn, 1 adds their likelihood ratio. */
int orc_adjoint(const orc_scene* s, const orc_config* cf, uint64_t ray_begin, uint64_t ray_end, int nthreads,
                const double* g, int unbiased, double* field_grad, double* scalars, uint64_t* segments);

/* Central differences of L = sum_i g_i S1_i at s +- h (global sticking, common
 * random numbers) for rays [ray_begin, ray_end), split by whether the roulette
 * decisions of the path differ between s - h, s and s + h; also the held
 * dL/ds along the path at s.  out[8]: see rtg_oracle.c (fd_pair_path). */
int orc_fd_pair(const orc_scene* s, const orc_config* cf, uint64_t ray_begin, uint64_t ray_end, int nthreads,
                const double* g, float h, double* out);

/* Every closest-hit query of source ray `id`'s path, in order (single
 * thread); writes at most `cap` records, returns how many the path has. */
int64_t orc_trace_log(const orc_scene* s, const orc_config* cf, uint64_t id, orc_segment* out, int64_t cap);

/* One source ray (origin, direction) for ray id; exposes the sampler. */
void orc_source_ray(const orc_config* cf, uint64_t id, float* org, float* dir);
/* Diffuse re-emission direction about a normal for two uniforms. */
void orc_diffuse_dir(const float* normal, uint32_t u_phi, uint32_t u_t, float* dir);
void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
void orc_sincos2pi(float u, float* s, float* c);
float orc_powf(float x, float e);

/* device.hpp:154-187: (S1_i/A_i + sum_nb S1_j/A_j)/(deg+1), then / max. */
void orc_normalize(int64_t n, const double* s1, const float* areas, const int64_t* row_ptr,
                   const int32_t* cols, float* out);
/* hit_accumulator.hpp:152-249 */
void orc_relative_error(int64_t n, const double* s1, const double* s2, uint64_t total, double* out);
void orc_vov(int64_t n, const double* s1, const double* s2, const double* s3, const double* s4,
             const uint64_t* cnt, uint64_t total, double* out);

#ifdef __cplusplus
}
#endif
#endif
