/*
 * rtg_oracle.c -- CPU oracle for the flux-tracing path.
 *
 * TEST INFRASTRUCTURE: a plain-C restatement of the reference's algorithm
 * used only to check the CUDA path (tests/, smoke check, bench CPU baseline).
 * It is never linked into, or called by, the product library.
 *
 * Reference files restated here (paths within the rti project):
 *   src/rti/trace/tracer.hpp:66-413            path loop, deposit, neighbours, areas
 *   src/rti/trace/local_intersector.hpp:41-97  neighbour (front-face) disc test
 *   src/rti/trace/hit_accumulator.hpp:128-249  S1..S4, counts, relative error, VOV
 *   src/rti/geo/boundary_x_y.hpp:92-143        periodic / reflective x-y box
 *   src/rti/geo/disc_neighborhood.hpp:20-220   overlapping-disc neighbourhood
 *   src/rti/geo/disc_bounding_box_intersector.hpp:43-441  exposed disc area
 *   src/rti/mc/rejection_control.hpp:28-61     Russian roulette
 *   src/rti/reflection/diffuse.hpp:13-27, src/rti/ray/cos_hemi.hpp:11-45,
 *   src/rti/util/utils.hpp:207-244             diffuse re-emission and basis
 *   src/rti/reflection/specular.hpp:16-40      specular re-emission
 *   src/rti/ray/source.hpp:20-58, rectangle_origin_z.hpp:23-37,
 *   cosine_direction_z.hpp:13-27, power_cosine_direction_z.hpp:13-32  source
 *   src/rti/device.hpp:154-187                 normalised, smoothed estimates
 *
 * Deliberate, documented differences from the reference (the reference's
 * behaviour here is either unreproducible or unpinned):
 *   - random numbers: Philox4x32-10 counters (Salmon et al., SC'11) keyed by
 *     (seed) with counter (ray id, collision index, stream tag) instead of
 *     per-thread mt19937_64 streams (tracer.hpp:136-143);
 *   - closest hit: this project's own oriented-disc and Moller-Trumbore
 *     triangle tests with ties broken by the lower primitive id, instead of
 *     Embree 3.11's rtcIntersect1 (tracer.hpp:181);
 *   - boundary: an analytic slab exit test instead of 8 Embree triangles;
 *   - a per-path cap on closest-hit queries (the reference has none).
 * Build: oracle/Makefile (-O2 -ffp-contract=off -fopenmp).
 */
#include "rtg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { float x, y, z; } v3;

static inline v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 sub3(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
/* util::normalize (utils.hpp:86-93) */
static inline v3 normalize3(v3 v) {
  float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
  return mk(v.x / l, v.y / l, v.z / l);
}
/* util::distance(a, b) (utils.hpp:141-147) */
static inline float dist3(v3 a, v3 b) {
  float d1 = a.x - b.x, d2 = a.y - b.y, d3 = a.z - b.z;
  return sqrtf(d1 * d1 + d2 * d2 + d3 * d3);
}
static inline float len3(v3 v) { return dist3(v, mk(0.0f, 0.0f, 0.0f)); }

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as   */
/* easy as 1, 2, 3", SC'11).                                                  */
/* ------------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline void draw4(uint64_t seed, uint64_t id, uint32_t event, uint32_t job, uint32_t* u) {
  uint32_t ctr[4] = {(uint32_t)id, (uint32_t)(id >> 32), event, job};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  orc_philox4x32_10(ctr, key, u);
}

/* uniform in [0,1) and (0,1] from the top 24 bits */
static inline float u01_co(uint32_t x) { return (float)(x >> 8) * 0x1p-24f; }
static inline float u01_oc(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1p-24f; }

/* ------------------------------------------------------------------------ */
/* sin/cos of 2*pi*u for u in [0,1]: exact quadrant reduction on u, then     */
/* Taylor polynomials on [0, pi/4] evaluated by Horner with fmaf.            */
/* ------------------------------------------------------------------------ */
static inline void sincos_quarter(float th, float* s, float* c) {
  float z = th * th;
  float ps = fmaf(z, -2.50521084e-08f, 2.75573192e-06f);  /* -1/11!, 1/9!  */
  ps = fmaf(z, ps, -1.98412698e-04f);                     /* -1/7!         */
  ps = fmaf(z, ps, 8.33333333e-03f);                      /*  1/5!         */
  ps = fmaf(z, ps, -1.66666667e-01f);                     /* -1/3!         */
  *s = fmaf(th * z, ps, th);
  float pc = fmaf(z, -2.75573192e-07f, 2.48015873e-05f);  /* -1/10!, 1/8!  */
  pc = fmaf(z, pc, -1.38888889e-03f);                     /* -1/6!         */
  pc = fmaf(z, pc, 4.16666667e-02f);                      /*  1/4!         */
  pc = fmaf(z, pc, -0.5f);                                /* -1/2!         */
  *c = fmaf(z, pc, 1.0f);
}

void orc_sincos2pi(float u, float* s, float* c) {
  float x = u * 4.0f;                /* exact */
  float qf = floorf(x);
  float f = x - qf;                  /* exact, in [0,1) */
  int q = ((int)qf) & 3;
  float ss, cc;
  if (f <= 0.5f) {
    sincos_quarter(f * 1.57079633f, &ss, &cc);
  } else {
    float sc, cs;
    sincos_quarter((1.0f - f) * 1.57079633f, &sc, &cs);
    ss = cs; cc = sc;
  }
  switch (q) {
    case 0: *s = ss; *c = cc; break;
    case 1: *s = cc; *c = -ss; break;
    case 2: *s = -ss; *c = -cc; break;
    default: *s = -cc; *c = ss; break;
  }
}

/* ------------------------------------------------------------------------ */
/* x^e for x in (0,1], e > 0: exp2(e*log2(x)) with an atanh series for log  */
/* and a Taylor series for exp, both evaluated with fmaf.                     */
/* ------------------------------------------------------------------------ */
static inline float as_float(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t as_bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static float own_log2(float x) {
  uint32_t b = as_bits(x);
  int k;
  if ((b >> 23) == 0) {            /* subnormal: scale up by 2^32 */
    x = x * 4294967296.0f;
    b = as_bits(x);
    k = (int)(b >> 23) - 127 - 32;
  } else {
    k = (int)(b >> 23) - 127;
  }
  float m = as_float((b & 0x007FFFFFu) | 0x3F800000u); /* [1,2) */
  if (m > 1.41421356f) { m = m * 0.5f; k += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float z = s * s;
  float p = fmaf(z, 0.0909090909f, 0.111111111f);     /* 1/11, 1/9 */
  p = fmaf(z, p, 0.142857143f);                        /* 1/7 */
  p = fmaf(z, p, 0.2f);                                /* 1/5 */
  p = fmaf(z, p, 0.333333333f);                        /* 1/3 */
  float ln_m = 2.0f * fmaf(s * z, p, s);
  return fmaf(ln_m, 1.44269504f, (float)k);           /* 1/ln 2 */
}

static float own_exp2(float y) {
  if (y < -149.0f) return 0.0f;
  float nf = floorf(y + 0.5f);
  float f = y - nf;                                     /* [-0.5, 0.5] */
  float z = f * 0.693147181f;                           /* ln 2 */
  float p = fmaf(z, 2.48015873e-05f, 1.98412698e-04f);  /* 1/8!, 1/7! */
  p = fmaf(z, p, 1.38888889e-03f);                      /* 1/6! */
  p = fmaf(z, p, 8.33333333e-03f);                      /* 1/5! */
  p = fmaf(z, p, 4.16666667e-02f);                      /* 1/4! */
  p = fmaf(z, p, 1.66666667e-01f);                      /* 1/3! */
  p = fmaf(z, p, 0.5f);
  p = fmaf(z, p, 1.0f);
  p = fmaf(z, p, 1.0f);
  int n = (int)nf;
  if (n < -126) { p = p * 0x1p-64f; n += 64; }
  if (n > 127) n = 127;
  return p * as_float((uint32_t)(n + 127) << 23);
}

float orc_powf(float x, float e) {
  if (x <= 0.0f) return 0.0f;
  if (x == 1.0f) return 1.0f;
  return own_exp2(e * own_log2(x));
}

/* ------------------------------------------------------------------------ */
/* Scene: primitives 0..nd-1 are discs, nd..nd+nt-1 are triangles.           */
/* ------------------------------------------------------------------------ */
typedef struct bnode {
  float lo[3], hi[3];
  int32_t left;   /* internal: child index; leaf: first slot in prim_order */
  int32_t count;  /* 0 for internal nodes */
  int32_t right;
} bnode;

struct orc_scene {
  int64_t nd, nt, np;
  float* dc;   /* nd*4 x y z r */
  float* dn;   /* nd*3 */
  float* tv0;  /* nt*3 */
  float* te1;  /* nt*3 */
  float* te2;  /* nt*3 */
  float* tn;   /* nt*3 normalised normal */
  float* blo;  /* np*3 primitive boxes */
  float* bhi;
  int32_t* order;
  bnode* nodes;
  int64_t nnodes, cap_nodes;
  int64_t* nb_ptr;  /* neighbour CSR (discs) */
  int32_t* nb_idx;
};

static inline v3 disc_c(const orc_scene* s, int64_t i) {
  return mk(s->dc[4 * i], s->dc[4 * i + 1], s->dc[4 * i + 2]);
}
static inline v3 disc_n(const orc_scene* s, int64_t i) {
  return mk(s->dn[3 * i], s->dn[3 * i + 1], s->dn[3 * i + 2]);
}
static inline v3 ld3(const float* p, int64_t i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

static v3 prim_normal(const orc_scene* s, int64_t p) {
  return p < s->nd ? disc_n(s, p) : ld3(s->tn, p - s->nd);
}

/* --------------------------- binned SAH BVH ----------------------------- */
#define NBINS 16
static float box_area(const float* lo, const float* hi) {
  float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  if (dx < 0 || dy < 0 || dz < 0) return 0.0f;
  return dx * dy + dy * dz + dz * dx;
}

static int64_t new_node(orc_scene* s) {
  if (s->nnodes == s->cap_nodes) {
    s->cap_nodes = s->cap_nodes ? 2 * s->cap_nodes : 1024;
    s->nodes = (bnode*)realloc(s->nodes, (size_t)s->cap_nodes * sizeof(bnode));
  }
  return s->nnodes++;
}

static void build_rec(orc_scene* s, int64_t ni, int64_t first, int64_t count) {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int64_t k = first; k < first + count; ++k) {
    int32_t p = s->order[k];
    for (int a = 0; a < 3; ++a) {
      float l = s->blo[3 * p + a], h = s->bhi[3 * p + a], c = 0.5f * (l + h);
      if (l < lo[a]) lo[a] = l;
      if (h > hi[a]) hi[a] = h;
      if (c < clo[a]) clo[a] = c;
      if (c > chi[a]) chi[a] = c;
    }
  }
  memcpy(s->nodes[ni].lo, lo, sizeof lo);
  memcpy(s->nodes[ni].hi, hi, sizeof hi);
  if (count <= 4) {
    s->nodes[ni].left = (int32_t)first;
    s->nodes[ni].count = (int32_t)count;
    s->nodes[ni].right = -1;
    return;
  }
  int best_axis = -1, best_bin = -1;
  float best_cost = FLT_MAX;
  for (int a = 0; a < 3; ++a) {
    float ext = chi[a] - clo[a];
    if (!(ext > 0.0f)) continue;
    int cnt[NBINS] = {0};
    float blo[NBINS][3], bhi[NBINS][3];
    for (int b = 0; b < NBINS; ++b)
      for (int q = 0; q < 3; ++q) { blo[b][q] = FLT_MAX; bhi[b][q] = -FLT_MAX; }
    for (int64_t k = first; k < first + count; ++k) {
      int32_t p = s->order[k];
      float c = 0.5f * (s->blo[3 * p + a] + s->bhi[3 * p + a]);
      int b = (int)((c - clo[a]) / ext * NBINS);
      if (b >= NBINS) b = NBINS - 1;
      if (b < 0) b = 0;
      cnt[b]++;
      for (int q = 0; q < 3; ++q) {
        if (s->blo[3 * p + q] < blo[b][q]) blo[b][q] = s->blo[3 * p + q];
        if (s->bhi[3 * p + q] > bhi[b][q]) bhi[b][q] = s->bhi[3 * p + q];
      }
    }
    float rarea[NBINS];
    int rcnt[NBINS];
    float rl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int rc = 0;
    for (int b = NBINS - 1; b > 0; --b) {
      rc += cnt[b];
      for (int q = 0; q < 3; ++q) {
        if (blo[b][q] < rl[q]) rl[q] = blo[b][q];
        if (bhi[b][q] > rh[q]) rh[q] = bhi[b][q];
      }
      rarea[b] = box_area(rl, rh);
      rcnt[b] = rc;
    }
    float ll[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int lc = 0;
    for (int b = 0; b < NBINS - 1; ++b) {
      lc += cnt[b];
      for (int q = 0; q < 3; ++q) {
        if (blo[b][q] < ll[q]) ll[q] = blo[b][q];
        if (bhi[b][q] > lh[q]) lh[q] = bhi[b][q];
      }
      if (lc == 0 || rcnt[b + 1] == 0) continue;
      float cost = box_area(ll, lh) * lc + rarea[b + 1] * rcnt[b + 1];
      if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = b; }
    }
  }
  int64_t mid;
  if (best_axis < 0) {
    mid = first + count / 2; /* all centroids equal: split in the middle */
  } else {
    float ext = chi[best_axis] - clo[best_axis];
    int64_t i = first, j = first + count - 1;
    while (i <= j) {
      int32_t p = s->order[i];
      float c = 0.5f * (s->blo[3 * p + best_axis] + s->bhi[3 * p + best_axis]);
      int b = (int)((c - clo[best_axis]) / ext * NBINS);
      if (b >= NBINS) b = NBINS - 1;
      if (b < 0) b = 0;
      if (b <= best_bin) { ++i; }
      else { int32_t t = s->order[i]; s->order[i] = s->order[j]; s->order[j] = t; --j; }
    }
    mid = i;
    if (mid == first || mid == first + count) mid = first + count / 2;
  }
  int64_t l = new_node(s);
  int64_t r = new_node(s);
  s->nodes[ni].left = (int32_t)l;
  s->nodes[ni].right = (int32_t)r;
  s->nodes[ni].count = 0;
  build_rec(s, l, first, mid - first);
  build_rec(s, r, mid, first + count - mid);
}

/* Conservative primitive boxes: exact extents padded so that any hit the
 * primitive test accepts lies inside the box. */
static void prim_boxes(orc_scene* s) {
  for (int64_t i = 0; i < s->nd; ++i) {
    float r = s->dc[4 * i + 3];
    for (int a = 0; a < 3; ++a) {
      float n = s->dn[3 * i + a];
      float c = s->dc[4 * i + a];
      float e = 1.0f - n * n;
      float ext = r * sqrtf(e > 0.0f ? e : 0.0f);
      float pad = 1e-5f * (fabsf(c) + r) + 1e-4f * r;
      s->blo[3 * i + a] = c - ext - pad;
      s->bhi[3 * i + a] = c + ext + pad;
    }
  }
  for (int64_t i = 0; i < s->nt; ++i) {
    int64_t p = s->nd + i;
    for (int a = 0; a < 3; ++a) {
      float v0 = s->tv0[3 * i + a];
      float v1 = v0 + s->te1[3 * i + a];
      float v2 = v0 + s->te2[3 * i + a];
      float lo = fminf(v0, fminf(v1, v2)), hi = fmaxf(v0, fmaxf(v1, v2));
      float pad = 1e-5f * (fabsf(lo) + fabsf(hi)) + 1e-6f * (hi - lo) + 1e-7f;
      s->blo[3 * p + a] = lo - pad;
      s->bhi[3 * p + a] = hi + pad;
    }
  }
}

orc_scene* orc_scene_create(const float* dxyzr, const float* dnrm, int64_t nd, const float* tverts,
                            const uint32_t* tidx, int64_t nv, int64_t nt) {
  (void)nv;
  orc_scene* s = (orc_scene*)calloc(1, sizeof(orc_scene));
  s->nd = nd;
  s->nt = nt;
  s->np = nd + nt;
  s->dc = (float*)malloc(sizeof(float) * 4 * (size_t)(nd ? nd : 1));
  s->dn = (float*)malloc(sizeof(float) * 3 * (size_t)(nd ? nd : 1));
  if (nd) {
    memcpy(s->dc, dxyzr, sizeof(float) * 4 * (size_t)nd);
    memcpy(s->dn, dnrm, sizeof(float) * 3 * (size_t)nd);
  }
  size_t tn3 = sizeof(float) * 3 * (size_t)(nt ? nt : 1);
  s->tv0 = (float*)malloc(tn3);
  s->te1 = (float*)malloc(tn3);
  s->te2 = (float*)malloc(tn3);
  s->tn = (float*)malloc(tn3);
  for (int64_t i = 0; i < nt; ++i) {
    v3 a = ld3(tverts, tidx[3 * i]), b = ld3(tverts, tidx[3 * i + 1]), c = ld3(tverts, tidx[3 * i + 2]);
    v3 e1 = sub3(b, a), e2 = sub3(c, a);
    /* util::compute_normal + normalize (i_triangle_reader.hpp:22-38) */
    v3 n = normalize3(cross3(e1, e2));
    s->tv0[3 * i] = a.x; s->tv0[3 * i + 1] = a.y; s->tv0[3 * i + 2] = a.z;
    s->te1[3 * i] = e1.x; s->te1[3 * i + 1] = e1.y; s->te1[3 * i + 2] = e1.z;
    s->te2[3 * i] = e2.x; s->te2[3 * i + 1] = e2.y; s->te2[3 * i + 2] = e2.z;
    s->tn[3 * i] = n.x; s->tn[3 * i + 1] = n.y; s->tn[3 * i + 2] = n.z;
  }
  s->blo = (float*)malloc(sizeof(float) * 3 * (size_t)(s->np ? s->np : 1));
  s->bhi = (float*)malloc(sizeof(float) * 3 * (size_t)(s->np ? s->np : 1));
  s->order = (int32_t*)malloc(sizeof(int32_t) * (size_t)(s->np ? s->np : 1));
  prim_boxes(s);
  for (int64_t i = 0; i < s->np; ++i) s->order[i] = (int32_t)i;
  if (s->np > 0) {
    int64_t root = new_node(s);
    build_rec(s, root, 0, s->np);
  }
  return s;
}

void orc_scene_destroy(orc_scene* s) {
  if (!s) return;
  free(s->dc); free(s->dn); free(s->tv0); free(s->te1); free(s->te2); free(s->tn);
  free(s->blo); free(s->bhi); free(s->order); free(s->nodes);
  free(s->nb_ptr); free(s->nb_idx);
  free(s);
}

int64_t orc_num_primitives(const orc_scene* s) { return s->np; }

/* ------------------------------------------------------------------------ */
/* Primitive tests                                                           */
/* ------------------------------------------------------------------------ */
/* Oriented disc, both faces: plane distance t, accepted when t > tnear and
 * the plane point lies within the radius. */
static inline int disc_test(v3 c, float r, v3 n, v3 o, v3 d, float tnear, float* tout) {
  float dn = d.x * n.x + d.y * n.y + d.z * n.z;
  if (dn == 0.0f) return 0;
  float num = (c.x - o.x) * n.x + (c.y - o.y) * n.y + (c.z - o.z) * n.z;
  float t = num / dn;
  if (!(t > tnear)) return 0;
  float qx = (o.x - c.x) + d.x * t;
  float qy = (o.y - c.y) + d.y * t;
  float qz = (o.z - c.z) + d.z * t;
  float q2 = qx * qx + qy * qy + qz * qz;
  if (!(q2 <= r * r)) return 0;
  *tout = t;
  return 1;
}

/* Moller-Trumbore, both faces, closed edges. */
static inline int tri_test(v3 v0, v3 e1, v3 e2, v3 o, v3 d, float tnear, float* tout) {
  v3 p = cross3(d, e2);
  float det = dot3(e1, p);
  if (det == 0.0f) return 0;
  float inv = 1.0f / det;
  v3 sv = sub3(o, v0);
  float u = dot3(sv, p) * inv;
  if (!(u >= 0.0f && u <= 1.0f)) return 0;
  v3 q = cross3(sv, e1);
  float v = dot3(d, q) * inv;
  if (!(v >= 0.0f && u + v <= 1.0f)) return 0;
  float t = dot3(e2, q) * inv;
  if (!(t > tnear)) return 0;
  *tout = t;
  return 1;
}

static inline int box_hit(const bnode* nd, v3 o, v3 idr, float tmax) {
  float t0x = (nd->lo[0] - o.x) * idr.x, t1x = (nd->hi[0] - o.x) * idr.x;
  float t0y = (nd->lo[1] - o.y) * idr.y, t1y = (nd->hi[1] - o.y) * idr.y;
  float t0z = (nd->lo[2] - o.z) * idr.z, t1z = (nd->hi[2] - o.z) * idr.z;
  float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), 0.0f));
  float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
  tf = tf * 1.0000005f;
  return tn <= tf && tn <= tmax * 1.0000005f + 1e-30f;
}

static inline float safe_inv(float d) {
  if (fabsf(d) < 1e-30f) d = d < 0.0f ? -1e-30f : 1e-30f;
  return 1.0f / d;
}

/* Closest primitive hit; ties in t go to the lower primitive id. */
static int closest(const orc_scene* s, v3 o, v3 d, float tnear, float* tbest, int32_t* pbest) {
  if (s->np == 0) return 0;
  v3 idr = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
  int32_t stack[256];
  int sp = 0;
  stack[sp++] = 0;
  float bt = FLT_MAX;
  int32_t bp = -1;
  while (sp) {
    const bnode* nd = &s->nodes[stack[--sp]];
    if (!box_hit(nd, o, idr, bt)) continue;
    if (nd->count) {
      for (int32_t k = nd->left; k < nd->left + nd->count; ++k) {
        int32_t p = s->order[k];
        float t;
        int h;
        if (p < s->nd) {
          h = disc_test(disc_c(s, p), s->dc[4 * p + 3], disc_n(s, p), o, d, tnear, &t);
        } else {
          int64_t q = p - s->nd;
          h = tri_test(ld3(s->tv0, q), ld3(s->te1, q), ld3(s->te2, q), o, d, tnear, &t);
        }
        if (h && (t < bt || (t == bt && p < bp))) { bt = t; bp = p; }
      }
    } else if (sp + 2 <= 256) {
      stack[sp++] = nd->right;
      stack[sp++] = nd->left;
    }
  }
  if (bp < 0) return 0;
  *tbest = bt;
  *pbest = bp;
  return 1;
}

void orc_closest_hit(const orc_scene* s, const float* rays, int64_t n, float tnear, int32_t* prim_out,
                     float* t_out) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    const float* r = rays + 6 * i;
    float t = 0.0f;
    int32_t p = -1;
    if (closest(s, mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), tnear, &t, &p)) {
      prim_out[i] = p;
      t_out[i] = t;
    } else {
      prim_out[i] = -1;
      t_out[i] = 0.0f;
    }
  }
}

/* local_intersector::intersect (local_intersector.hpp:41-97), front faces only. */
static inline int local_intersect(v3 o, v3 d, v3 c, float r, v3 n) {
  float prod = n.x * d.x + n.y * d.y + n.z * d.z;
  if (prod > 0.0f) return 0;
  if (fabsf(prod) < 1e-9f) return 0;
  float ddneg = c.x * n.x + c.y * n.y + c.z * n.z;
  float ttnom = (-(n.x * o.x + n.y * o.y + n.z * o.z)) + ddneg;
  float tt = ttnom / prod;
  if (tt <= 0.0f) return 0;
  v3 hp = mk(o.x + d.x * tt, o.y + d.y * tt, o.z + d.z * tt);
  v3 v = mk(hp.x + (-c.x), hp.y + (-c.y), hp.z + (-c.z));
  float dist = len3(v);
  return r > dist;
}

int orc_local_intersect(const float* org, const float* dir, const float* disc, const float* nrm) {
  return local_intersect(mk(org[0], org[1], org[2]), mk(dir[0], dir[1], dir[2]),
                         mk(disc[0], disc[1], disc[2]), disc[3], mk(nrm[0], nrm[1], nrm[2]));
}

/* ------------------------------------------------------------------------ */
/* Source and re-emission                                                    */
/* ------------------------------------------------------------------------ */
static void source_dir(float expo, float ee, uint32_t u_phi, uint32_t u_t, v3* d) {
  float rt = u01_oc(u_t);
  float t = (expo == 1.0f) ? rt : orc_powf(rt, ee);
  float zz = -sqrtf(t);
  float sq = sqrtf(1.0f - t);
  float sn, cs;
  orc_sincos2pi(u01_co(u_phi), &sn, &cs);
  *d = normalize3(mk(cs * sq, sn * sq, zz));
}

void orc_source_ray(const orc_config* cf, uint64_t id, float* org, float* dir) {
  uint32_t u[4];
  draw4(cf->seed, id, 0xFFFFFFFFu, cf->job, u);
  float r1 = u01_co(u[0]), r2 = u01_co(u[1]);
  org[0] = cf->src_lo[0] + (cf->src_hi[0] - cf->src_lo[0]) * r1;
  org[1] = cf->src_lo[1] + (cf->src_hi[1] - cf->src_lo[1]) * r2;
  org[2] = cf->box_hi[2];
  float ee = 2.0f / (cf->source_exponent + 1.0f);
  v3 d;
  source_dir(cf->source_exponent, ee, u[2], u[3], &d);
  dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
}

/* util::get_orthonormal_basis (utils.hpp:207-244) + cos_hemi::get (cos_hemi.hpp:11-45) */
static v3 diffuse_dir(v3 n, uint32_t u_phi, uint32_t u_t) {
  v3 c0 = mk(n.z, n.z, -(n.x + n.y));
  v3 c1 = mk(n.y, -(n.x + n.z), n.y);
  v3 c2 = mk(-(n.y + n.z), n.x, n.x);
  v3 b1 = c0;
  float best = c0.x + c0.y + c0.z;
  if (c1.x + c1.y + c1.z > best) { b1 = c1; best = c1.x + c1.y + c1.z; }
  if (c2.x + c2.y + c2.z > best) { b1 = c2; }
  v3 b2 = cross3(n, b1);
  v3 b0 = normalize3(n);
  b1 = normalize3(b1);
  b2 = normalize3(b2);
  float r2 = u01_oc(u_t);
  float cc1 = sqrtf(r2);
  float sq = sqrtf(1.0f - r2);
  float sn, cs;
  orc_sincos2pi(u01_co(u_phi), &sn, &cs);
  float cc2 = cs * sq, cc3 = sn * sq;
  return mk(b0.x * cc1 + b1.x * cc2 + b2.x * cc3, b0.y * cc1 + b1.y * cc2 + b2.y * cc3,
            b0.z * cc1 + b1.z * cc2 + b2.z * cc3);
}

void orc_diffuse_dir(const float* normal, uint32_t u_phi, uint32_t u_t, float* dir) {
  v3 d = diffuse_dir(mk(normal[0], normal[1], normal[2]), u_phi, u_t);
  dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
}

/* specular::use (specular.hpp:66-90): d' = n*(2 n.(-d)) + d */
static v3 specular_dir(v3 n, v3 d) {
  float k = 2.0f * (n.x * (-d.x) + n.y * (-d.y) + n.z * (-d.z));
  return mk(n.x * k + d.x, n.y * k + d.y, n.z * k + d.z);
}

/* Side-face exit of the x/y box: returns 0 (x face), 1 (y face) or -1 when
 * the ray leaves through the top or bottom first (a miss). */
static int boundary_exit(const orc_config* cf, v3 o, v3 d, float* tb) {
  float tx = FLT_MAX, ty = FLT_MAX, tz = FLT_MAX;
  if (d.x > 0.0f) tx = (cf->box_hi[0] - o.x) / d.x;
  else if (d.x < 0.0f) tx = (cf->box_lo[0] - o.x) / d.x;
  if (d.y > 0.0f) ty = (cf->box_hi[1] - o.y) / d.y;
  else if (d.y < 0.0f) ty = (cf->box_lo[1] - o.y) / d.y;
  if (d.z > 0.0f) tz = (cf->box_hi[2] - o.z) / d.z;
  else if (d.z < 0.0f) tz = (cf->box_lo[2] - o.z) / d.z;
  int axis = tx <= ty ? 0 : 1;
  float t = tx <= ty ? tx : ty;
  if (!(t < FLT_MAX)) return -1;
  if (!(t >= cf->tnear)) return -1;
  if (t > tz) return -1;
  *tb = t;
  return axis;
}

typedef struct {
  double *s1, *s2, *s3, *s4;
  uint64_t* cnt;
  orc_tally t;
  int fixed; /* s1 holds int64 multiples of 2^-32 */
  /* segment log of one path (orc_trace_log): counted when logging, kept up to log_cap */
  int logging;
  orc_segment* log;
  int64_t log_n, log_cap;
} acc_t;

static void log_seg(acc_t* a, uint64_t id, uint32_t seg, int kind, v3 o, v3 d, float t, int32_t prim, float w) {
  if (!a->logging) return;
  if (a->log && a->log_n < a->log_cap) {
    orc_segment* r = &a->log[a->log_n];
    r->ray = id;
    r->segment = seg;
    r->kind = kind;
    r->org[0] = o.x; r->org[1] = o.y; r->org[2] = o.z;
    r->end[0] = o.x + d.x * t; r->end[1] = o.y + d.y * t; r->end[2] = o.z + d.z * t;
    r->primitive = prim;
    r->weight = w;
  }
  a->log_n += 1;
}

/* hit_accumulator::use (hit_accumulator.hpp:128-138); fixed: the flux as an
 * int64 multiple of 2^-32, rounded to nearest even like the GPU */
static inline void acc_use(acc_t* a, int32_t p, float v) {
  double dv = (double)v;
  if (a->fixed) {
    int64_t q;
    memcpy(&q, &a->s1[p], 8);
    q += (int64_t)llrint(dv * 4294967296.0);
    memcpy(&a->s1[p], &q, 8);
  } else {
    a->s1[p] += dv;
  }
  a->s2[p] += dv * v;
  a->s3[p] += dv * v * v;
  a->s4[p] += dv * v * v * v;
  a->cnt[p] += 1;
  a->t.total += 1;
}

/* The multi-hit window of rti's point-cloud context (point_cloud_context.hpp:
 * 132-173 filter, 265-286 post-processing), restated with a defined order:
 * the window opens at the closest front-face hit t0, on disc p0, instead of at
 * whichever hit Embree's filter reports first.  It reaches to
 * t0 + window_factor * r0 (rti: 5 radii of the first disc, :163), cut at the
 * x/y box exit tbox (rti's boundary hit is accepted and ends the query) and at
 * the first back-face disc hit or triangle hit beyond t0 (rti accepts a
 * back-face hit once the window is open, :145-153).  Every disc hit from the
 * front within it receives w s_j (each disc once, :271-281); w then drops by
 * the mean of those deposits (:283-285).  Scans the BVH for every primitive
 * hit in [0, te]; returns the new weight. */
static float window_deposit(const orc_scene* s, const orc_config* cf, v3 o, v3 d, float t0, float tbox, int32_t p0,
                            float w, acc_t* a) {
  float te = t0 + cf->window_factor * s->dc[4 * p0 + 3];
  if (tbox < te) te = tbox;
  const v3 idr = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
  float tc = te;
  double sum = 0.0;
  uint64_t n = 0;
  for (int pass = 0; pass < 2; ++pass) { /* 0: where the window closes; 1: the deposits */
    int32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
      const bnode* nd = &s->nodes[stack[--sp]];
      if (!box_hit(nd, o, idr, tc)) continue;
      if (!nd->count) {
        if (sp + 2 <= 256) {
          stack[sp++] = nd->right;
          stack[sp++] = nd->left;
        }
        continue;
      }
      for (int32_t k = nd->left; k < nd->left + nd->count; ++k) {
        const int32_t p = s->order[k];
        float t;
        int h, closes;
        if (p < s->nd) {
          const v3 nrm = disc_n(s, p);
          h = disc_test(disc_c(s, p), s->dc[4 * p + 3], nrm, o, d, cf->tnear, &t);
          closes = d.x * nrm.x + d.y * nrm.y + d.z * nrm.z > 0.0f;
        } else {
          const int64_t q = p - s->nd;
          h = tri_test(ld3(s->tv0, q), ld3(s->te1, q), ld3(s->te2, q), o, d, cf->tnear, &t);
          closes = 1;
        }
        if (!h) continue;
        if (pass == 0) {
          if (closes && t > t0 && t < tc) tc = t;
        } else if (p < s->nd && !closes && t >= t0 && t <= tc) {
          const float st = cf->sticking_field ? cf->sticking_field[p] : cf->sticking;
          const float v = w * st;
          acc_use(a, p, v);
          sum += (double)v;
          n += 1;
        }
      }
    }
  }
  if (n > 1) a->t.nb_deposits += n - 1;
  return n > 0 ? (float)((double)w - sum / (double)n) : w;
}

/* One path of tracer::run (tracer.hpp:160-280). */
static void trace_path(const orc_scene* s, const orc_config* cf, uint64_t id, acc_t* a) {
  float w = 1.0f;
  const float w0 = 1.0f;
  float org[3], dir[3];
  orc_source_ray(cf, id, org, dir);
  v3 o = mk(org[0], org[1], org[2]), d = mk(dir[0], dir[1], dir[2]);
  uint32_t k = 0;
  uint32_t nseg = 0;
  const float tnear = cf->tnear;
  for (;;) {
    if (nseg == cf->max_segments) { a->t.truncated += 1; break; }
    nseg += 1;
    a->t.segments += 1;
    float th = 0.0f, tb = 0.0f;
    int32_t p = -1;
    int hit = closest(s, o, d, tnear, &th, &p);
    int axis = boundary_exit(cf, o, d, &tb);
    if (hit && (axis < 0 || th <= tb)) {
      v3 n = prim_normal(s, p);
      v3 hp = mk(o.x + d.x * th, o.y + d.y * th, o.z + d.z * th);
      if (d.x * n.x + d.y * n.y + d.z * n.z > 0.0f) { /* back face: pass through */
        log_seg(a, id, nseg - 1, 1, o, d, th, p, w);
        o = hp;
        continue;
      }
      log_seg(a, id, nseg - 1, 0, o, d, th, p, w);
      a->t.hitc += 1;
      float st = cf->sticking_field ? cf->sticking_field[p] : cf->sticking;
      float v = w * st;
      if (cf->window && p < s->nd) {
        w = window_deposit(s, cf, o, d, th, axis >= 0 ? tb : FLT_MAX, p, w, a);
      } else {
        acc_use(a, p, v);
        if (p < s->nd && s->nb_ptr) {
          for (int64_t q = s->nb_ptr[p]; q < s->nb_ptr[p + 1]; ++q) {
            int32_t nb = s->nb_idx[q];
            if (local_intersect(o, d, disc_c(s, nb), s->dc[4 * nb + 3], disc_n(s, nb))) {
              acc_use(a, nb, v);
              a->t.nb_deposits += 1;
            }
          }
        }
        w = w - v;
      }
      if (w == 0.0f) break;
      uint32_t u[4];
      draw4(cf->seed, id, k, cf->job, u);
      /* rejection_control::check_weight_reweight_or_kill */
      double lower = cf->roulette_threshold * w0;
      double renew = cf->roulette_weight * w0;
      if (!((double)w >= lower)) {
        double kill = 1.0f - (double)w / renew;
        if ((double)u[0] < kill * 4294967296.0) break;
        w = (float)renew;
      }
      int spec = cf->reflection == 1 ||
                 (cf->reflection == 2 && (double)u[3] < (double)cf->specular_fraction * 4294967296.0);
      d = spec ? specular_dir(n, d) : diffuse_dir(n, u[1], u[2]);
      o = hp;
      k += 1;
      continue;
    }
    if (axis >= 0) {
      log_seg(a, id, nseg - 1, 2, o, d, tb, -1, w);
      v3 hp = mk(o.x + d.x * tb, o.y + d.y * tb, o.z + d.z * tb);
      int periodic = axis == 0 ? cf->x_bound : cf->y_bound;
      if (periodic) {
        if (axis == 0) hp.x = d.x > 0.0f ? cf->box_lo[0] : cf->box_hi[0];
        else hp.y = d.y > 0.0f ? cf->box_lo[1] : cf->box_hi[1];
      } else {
        if (axis == 0) d.x = -d.x;
        else d.y = -d.y;
      }
      o = hp;
      continue;
    }
    if (a->logging) { /* out through the top or bottom plane */
      const float tz = d.z > 0.0f ? (cf->box_hi[2] - o.z) / d.z : (d.z < 0.0f ? (cf->box_lo[2] - o.z) / d.z : 0.0f);
      log_seg(a, id, nseg - 1, 3, o, d, tz, -1, w);
    }
    a->t.nonhitc += 1;
    break;
  }
}

/* Adjoint replay of one path: derivatives of L = sum_i g_i S1_i.  G_k is the
 * sum of g over the primitives that received deposit k, v_k = w_k s its
 * weight (s the sticking of the hit primitive), P_k = sum_{m<=k} G_m v_m.
 * Two estimators (cf->adj_unbiased):
 *  held (0): the Russian-roulette decisions are held as drawn, which is what
 *    central differences with common random numbers measure.  Within a
 *    stretch between roulette resets every weight carries the factors (1 - s_e)
 *    of the earlier deposits of the stretch, so
 *      dL/ds_j = sum over deposits k on j of G_k w_k - (T - P_k)/(1 - s_j),
 *    T the stretch total; one global s: v_k = w_k s, dv_k/ds = w_k + s w'_k,
 *    w'_{k+1} = w'_k - dv_k/ds, w' = 0 after a reset.
 *  unbiased (1): adds the likelihood ratio of each roulette survival
 *    (probability w/0.3), which extends T to the whole path total L_p:
 *      dL/ds_j = sum over deposits k on j of G_k w_k - (L_p - P_k)/(1 - s_j).
 * With a sticking field each deposit's term is split as G_k w_k + P_k/(1 - s_j),
 * added at the deposit, minus T/(1 - s_j), added at the end of the stretch
 * (the whole path for the unbiased estimator) from a list of the stretch's
 * (element, sticking) pairs of at most ORC_ADJ_LIST entries; a longer stretch
 * is traced again from a snapshot of its start to add them -- the same split
 * and the same replay decisions as the GPU kernel.  Both:
 *   dL/dn = sum over paths of (1/(n+1) + ln cos theta_0) L_p. */
typedef struct { double ds, dn; double* field; } adj_acc_t;

#define ORC_ADJ_LIST 32

/* the deferred terms -T/(1 - s_j) of a stretch whose deposits all fit the list */
static void adj_flush(adj_acc_t* a, const int32_t* id, const float* st, int n, double t) {
  for (int i = 0; i < n; ++i)
    if (st[i] < 1.0f) a->field[id[i]] += -t / (1.0 - (double)st[i]);
}

static void adjoint_path(const orc_scene* s, const orc_config* cf, uint64_t id, const double* g, int unbiased,
                         adj_acc_t* a, uint64_t* segs) {
  const int fieldmode = cf->sticking_field != NULL;
  float org[3], dir[3];
  orc_source_ray(cf, id, org, dir);
  v3 o = mk(org[0], org[1], org[2]), d = mk(dir[0], dir[1], dir[2]);
  float w = 1.0f;
  uint32_t k = 0, nseg = 0;
  const double score = 1.0 / ((double)cf->source_exponent + 1.0) + log(-(double)d.z);
  double wd = 0.0, lp = 0.0, seg_t = 0.0, pa = 0.0, psum = 0.0, ncoll = 0.0;
  int sub = 0;
  v3 so = o, sd = d;
  float sw = w;
  uint32_t sk = k, snseg = nseg;
  int32_t list_id[ORC_ADJ_LIST];
  float list_s[ORC_ADJ_LIST];
  int list_n = 0;
  const double lower = cf->roulette_threshold * 1.0f, renew = cf->roulette_weight * 1.0f;
  const float s_glob = cf->sticking;
  for (;;) {
    int ended = 0;
    if (nseg == cf->max_segments) {
      ended = 1;
    } else {
      nseg += 1;
      *segs += 1;
      float th = 0.0f, tb = 0.0f;
      int32_t p = -1;
      int hit = closest(s, o, d, cf->tnear, &th, &p);
      int axis = boundary_exit(cf, o, d, &tb);
      if (hit && (axis < 0 || th <= tb)) {
        v3 n = prim_normal(s, p);
        v3 hp = mk(o.x + d.x * th, o.y + d.y * th, o.z + d.z * th);
        if (d.x * n.x + d.y * n.y + d.z * n.z > 0.0f) {
          o = hp;
          continue;
        }
        float st = cf->sticking_field ? cf->sticking_field[p] : s_glob;
        float v = w * st;
        double G = g[p];
        if (p < s->nd && s->nb_ptr)
          for (int64_t q = s->nb_ptr[p]; q < s->nb_ptr[p + 1]; ++q) {
            int32_t nb = s->nb_idx[q];
            if (local_intersect(o, d, disc_c(s, nb), s->dc[4 * nb + 3], disc_n(s, nb))) G += g[nb];
          }
        const double gv = G * (double)v;
        if (!fieldmode) {
          lp += gv;
          if (unbiased) {
            pa += G * (double)w;
            psum += lp;
            ncoll += 1.0;
          } else {
            double dv = (double)w + (double)st * wd;
            a->ds += G * dv;
            wd -= dv;
          }
        } else if (sub == 0) {
          seg_t += gv; /* P_k */
          lp += gv;
          double ak = G * (double)w;
          if (st < 1.0f) ak += seg_t / (1.0 - (double)st);
          a->field[p] += ak;
          if (list_n < ORC_ADJ_LIST) {
            list_id[list_n] = p;
            list_s[list_n] = st;
          }
          list_n += 1;
        } else if (st < 1.0f) { /* replay of a long stretch: seg_t holds its total */
          a->field[p] += -seg_t / (1.0 - (double)st);
        }
        w = w - v;
        if (w == 0.0f) {
          ended = 1;
        } else {
          uint32_t u[4];
          draw4(cf->seed, id, k, cf->job, u);
          int reset = 0;
          if (!((double)w >= lower)) {
            double kill = 1.0f - (double)w / renew;
            if ((double)u[0] < kill * 4294967296.0) ended = 1;
            else {
              w = (float)renew;
              reset = 1;
              wd = 0.0;
            }
          }
          if (!ended) {
            int spec = cf->reflection == 1 ||
                       (cf->reflection == 2 && (double)u[3] < (double)cf->specular_fraction * 4294967296.0);
            d = spec ? specular_dir(n, d) : diffuse_dir(n, u[1], u[2]);
            o = hp;
            k += 1;
            if (fieldmode && reset && !unbiased) {
              if (sub == 0 && list_n > ORC_ADJ_LIST) {
                o = so; d = sd; w = sw; k = sk; nseg = snseg;
                sub = 1;
              } else {
                if (sub == 0) adj_flush(a, list_id, list_s, list_n, seg_t);
                so = o; sd = d; sw = w; sk = k; snseg = nseg;
                seg_t = 0.0; sub = 0; list_n = 0;
              }
            }
            continue;
          }
        }
      } else if (axis >= 0) {
        v3 hp = mk(o.x + d.x * tb, o.y + d.y * tb, o.z + d.z * tb);
        int periodic = axis == 0 ? cf->x_bound : cf->y_bound;
        if (periodic) {
          if (axis == 0) hp.x = d.x > 0.0f ? cf->box_lo[0] : cf->box_hi[0];
          else hp.y = d.y > 0.0f ? cf->box_lo[1] : cf->box_hi[1];
        } else {
          if (axis == 0) d.x = -d.x;
          else d.y = -d.y;
        }
        o = hp;
        continue;
      } else {
        ended = 1;
      }
    }
    if (ended) {
      if (fieldmode && sub == 0) {
        if (list_n <= ORC_ADJ_LIST) {
          adj_flush(a, list_id, list_s, list_n, seg_t);
        } else {
          o = so; d = sd; w = sw; k = sk; nseg = snseg;
          sub = 1;
          continue;
        }
      }
      if (!fieldmode && unbiased) {
        double ds = pa;
        if (s_glob < 1.0f) ds -= (ncoll * lp - psum) / (1.0 - (double)s_glob);
        a->ds += ds;
      }
      a->dn += score * lp;
      return;
    }
  }
}

int64_t orc_trace_log(const orc_scene* s, const orc_config* cf, uint64_t id, orc_segment* out, int64_t cap) {
  const int64_t np = s->np;
  acc_t a;
  memset(&a, 0, sizeof a);
  a.fixed = cf->accum_fixed != 0;
  a.s1 = (double*)calloc((size_t)np + 1, sizeof(double));
  a.s2 = (double*)calloc((size_t)np + 1, sizeof(double));
  a.s3 = (double*)calloc((size_t)np + 1, sizeof(double));
  a.s4 = (double*)calloc((size_t)np + 1, sizeof(double));
  a.cnt = (uint64_t*)calloc((size_t)np + 1, sizeof(uint64_t));
  a.logging = 1;
  a.log = out;
  a.log_cap = cap;
  trace_path(s, cf, id, &a);
  free(a.s1); free(a.s2); free(a.s3); free(a.s4); free(a.cnt);
  return a.log_n;
}

int orc_adjoint(const orc_scene* s, const orc_config* cf, uint64_t b, uint64_t e, int nthreads, const double* g,
                int unbiased, double* field_grad, double* scalars, uint64_t* segments) {
  int64_t np = s->np;
  if (cf->sticking_field && !field_grad) return 1;
  if (cf->window) return 1; /* the adjoint replays the neighbour deposit only */
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  double ds = 0.0, dn = 0.0;
  uint64_t segs = 0;
#pragma omp parallel num_threads(nthreads)
  {
    adj_acc_t a = {0.0, 0.0, NULL};
    uint64_t sg = 0;
    if (cf->sticking_field) a.field = (double*)calloc((size_t)np + 1, sizeof(double));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = (int64_t)b; i < (int64_t)e; ++i) adjoint_path(s, cf, (uint64_t)i, g, unbiased, &a, &sg);
#pragma omp critical
    {
      ds += a.ds;
      dn += a.dn;
      segs += sg;
      if (a.field)
        for (int64_t p = 0; p < np; ++p) field_grad[p] += a.field[p];
    }
    free(a.field);
  }
  scalars[0] += ds;
  scalars[1] += dn;
  if (segments) *segments = segs;
  return 0;
}

int orc_trace(const orc_scene* s, const orc_config* cf, uint64_t b, uint64_t e, int nthreads,
              double* s1, double* s2, double* s3, double* s4, uint64_t* cnt, orc_tally* tally) {
  int64_t np = s->np;
  memset(tally, 0, sizeof *tally);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
#pragma omp parallel num_threads(nthreads)
  {
    acc_t a;
    memset(&a, 0, sizeof a);
    a.fixed = cf->accum_fixed != 0;
    a.s1 = (double*)calloc((size_t)np + 1, sizeof(double));
    a.s2 = (double*)calloc((size_t)np + 1, sizeof(double));
    a.s3 = (double*)calloc((size_t)np + 1, sizeof(double));
    a.s4 = (double*)calloc((size_t)np + 1, sizeof(double));
    a.cnt = (uint64_t*)calloc((size_t)np + 1, sizeof(uint64_t));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = (int64_t)b; i < (int64_t)e; ++i) trace_path(s, cf, (uint64_t)i, &a);
#pragma omp critical
    {
      for (int64_t p = 0; p < np; ++p) {
        if (a.fixed) {  /* s1 of the caller holds the integer sums until the end */
          int64_t x, y;
          memcpy(&x, &s1[p], 8);
          memcpy(&y, &a.s1[p], 8);
          x += y;
          memcpy(&s1[p], &x, 8);
        } else {
          s1[p] += a.s1[p];
        }
        s2[p] += a.s2[p]; s3[p] += a.s3[p]; s4[p] += a.s4[p];
        cnt[p] += a.cnt[p];
      }
      tally->hitc += a.t.hitc;
      tally->nonhitc += a.t.nonhitc;
      tally->total += a.t.total;
      tally->segments += a.t.segments;
      tally->truncated += a.t.truncated;
      tally->nb_deposits += a.t.nb_deposits;
    }
    free(a.s1); free(a.s2); free(a.s3); free(a.s4); free(a.cnt);
  }
  if (cf->accum_fixed)
    for (int64_t p = 0; p < np; ++p) {
      int64_t x;
      memcpy(&x, &s1[p], 8);
      s1[p] = (double)x * (1.0 / 4294967296.0);
    }
  return 0;
}

/* Central differences with common random numbers, decomposed by roulette
 * decisions.  Every path is traced once while three weights ride on it: w at
 * the configured global sticking s, and w+/w- at s + h / s - h.  The path's
 * geometry (hits, directions) does not depend on s, only on the Russian
 * roulette decisions (rejection_control.hpp:28-61) that its weights meet, so
 * all three share it for as long as they are alive; a state that is killed
 * stops depositing.  At each collision a state's decision is 0 (w >= 0.1, no
 * roulette), 1 (roulette, survived, w := 0.3) or 2 (roulette, killed).  A path
 * is "flipped" when the three states do not make the same decisions all the way.
 * Along the s state the held derivative dL_p/ds is formed exactly as the GPU's
 * held replay forms it (dv = w + s w', w' -= dv, w' = 0 after a survival).
 * out[0] = sum over paths of L+ - L-        (divide by 2h: the difference quotient)
 * out[1] = the same over unflipped paths
 * out[2] = held dL/ds over all paths
 * out[3] = held dL/ds over unflipped paths
 * out[4] = flipped paths
 * out[5] = collisions at which the +h and -h states, both alive, decide differently
 * out[6] = paths on which any state met the roulette
 * out[7] = L at s (sum over paths) */
static void fd_pair_path(const orc_scene* s, const orc_config* cf, uint64_t id, const double* g, float h,
                         double* out) {
  float org[3], dir[3];
  orc_source_ray(cf, id, org, dir);
  v3 o = mk(org[0], org[1], org[2]), d = mk(dir[0], dir[1], dir[2]);
  const float st[3] = {cf->sticking - h, cf->sticking, cf->sticking + h};
  float w[3] = {1.0f, 1.0f, 1.0f};
  int alive[3] = {1, 1, 1};
  double L[3] = {0.0, 0.0, 0.0};
  double wd = 0.0, held = 0.0;
  int flipped = 0, met = 0;
  double flips = 0.0;
  uint32_t k = 0, nseg = 0;
  const double lower = cf->roulette_threshold * 1.0f, renew = cf->roulette_weight * 1.0f;
  while (alive[0] || alive[1] || alive[2]) {
    if (nseg == cf->max_segments) break;
    nseg += 1;
    float th = 0.0f, tb = 0.0f;
    int32_t p = -1;
    int hit = closest(s, o, d, cf->tnear, &th, &p);
    int axis = boundary_exit(cf, o, d, &tb);
    if (hit && (axis < 0 || th <= tb)) {
      v3 n = prim_normal(s, p);
      v3 hp = mk(o.x + d.x * th, o.y + d.y * th, o.z + d.z * th);
      if (d.x * n.x + d.y * n.y + d.z * n.z > 0.0f) {
        o = hp;
        continue;
      }
      double G = g[p];
      if (p < s->nd && s->nb_ptr)
        for (int64_t q = s->nb_ptr[p]; q < s->nb_ptr[p + 1]; ++q) {
          int32_t nb = s->nb_idx[q];
          if (local_intersect(o, d, disc_c(s, nb), s->dc[4 * nb + 3], disc_n(s, nb))) G += g[nb];
        }
      uint32_t u[4];
      draw4(cf->seed, id, k, cf->job, u);
      int dec[3] = {-1, -1, -1};
      for (int j = 0; j < 3; ++j) {
        if (!alive[j]) continue;
        const float v = w[j] * st[j];
        L[j] += G * (double)v;
        if (j == 1) {
          const double dv = (double)w[1] + (double)st[1] * wd;
          held += G * dv;
          wd -= dv;
        }
        w[j] = w[j] - v;
        if (w[j] == 0.0f) {
          dec[j] = 3;
          alive[j] = 0;
          continue;
        }
        dec[j] = 0;
        if (!((double)w[j] >= lower)) {
          const double kill = 1.0f - (double)w[j] / renew;
          met = 1;
          if ((double)u[0] < kill * 4294967296.0) {
            dec[j] = 2;
            alive[j] = 0;
          } else {
            dec[j] = 1;
            w[j] = (float)renew;
            if (j == 1) wd = 0.0;
          }
        }
      }
      if (dec[0] != dec[1] || dec[1] != dec[2]) flipped = 1;
      if (dec[0] >= 0 && dec[2] >= 0 && dec[0] != dec[2]) flips += 1.0;
      int spec = cf->reflection == 1 ||
                 (cf->reflection == 2 && (double)u[3] < (double)cf->specular_fraction * 4294967296.0);
      d = spec ? specular_dir(n, d) : diffuse_dir(n, u[1], u[2]);
      o = hp;
      k += 1;
      continue;
    }
    if (axis >= 0) {
      v3 hp = mk(o.x + d.x * tb, o.y + d.y * tb, o.z + d.z * tb);
      int periodic = axis == 0 ? cf->x_bound : cf->y_bound;
      if (periodic) {
        if (axis == 0) hp.x = d.x > 0.0f ? cf->box_lo[0] : cf->box_hi[0];
        else hp.y = d.y > 0.0f ? cf->box_lo[1] : cf->box_hi[1];
      } else {
        if (axis == 0) d.x = -d.x;
        else d.y = -d.y;
      }
      o = hp;
      continue;
    }
    break;
  }
  out[0] += L[2] - L[0];
  out[2] += held;
  if (!flipped) {
    out[1] += L[2] - L[0];
    out[3] += held;
  }
  out[4] += flipped;
  out[5] += flips;
  out[6] += met;
  out[7] += L[1];
}

int orc_fd_pair(const orc_scene* s, const orc_config* cf, uint64_t b, uint64_t e, int nthreads, const double* g,
                float h, double* out) {
  if (cf->sticking_field || cf->window) return 1; /* one global sticking, neighbour deposit */
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  for (int i = 0; i < 8; ++i) out[i] = 0.0;
#pragma omp parallel num_threads(nthreads)
  {
    double o[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = (int64_t)b; i < (int64_t)e; ++i) fd_pair_path(s, cf, (uint64_t)i, g, h, o);
#pragma omp critical
    for (int i = 0; i < 8; ++i) out[i] += o[i];
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Neighbourhood: disc_neighborhood.hpp:37-220 restated (divide and conquer  */
/* on the centre coordinates, strict distance test).                         */
/* ------------------------------------------------------------------------ */
typedef struct { int32_t* v; int64_t n, cap; } ivec;
static void ivec_push(ivec* a, int32_t x) {
  if (a->n == a->cap) {
    a->cap = a->cap ? 2 * a->cap : 8;
    a->v = (int32_t*)realloc(a->v, (size_t)a->cap * sizeof(int32_t));
  }
  a->v[a->n++] = x;
}

typedef struct { const float* pts; ivec* nbhd; } nbctx;

/* check_dist (disc_neighborhood.hpp:190-220) */
static int check_dist(const float* pts, int32_t i1, int32_t i2) {
  const float* p1 = pts + 4 * i1;
  const float* p2 = pts + 4 * i2;
  float sr = p1[3] + p2[3];
  for (int a = 0; a < 3; ++a)
    if (fabsf(p2[a] - p1[a]) >= sr) return 0;
  float dd = dist3(mk(p1[0], p1[1], p1[2]), mk(p2[0], p2[1], p2[2]));
  return dd < p1[3] + p2[3];
}

static void dac(nbctx* c, const ivec* s1, const ivec* s2, float s1maxrad, float s2maxrad,
                const float* mn, const float* mx, int diridx, float pivot) {
  if (s1->n + s2->n <= 1) return;
  if (pivot == mn[diridx] || pivot == mx[diridx]) {
    /* corner case: all remaining points become mutual neighbours */
    int64_t m = s1->n + s2->n;
    for (int64_t a = 0; a + 1 < m; ++a)
      for (int64_t b2 = a + 1; b2 < m; ++b2) {
        int32_t pa = a < s1->n ? s1->v[a] : s2->v[a - s1->n];
        int32_t pb = b2 < s1->n ? s1->v[b2] : s2->v[b2 - s1->n];
        ivec_push(&c->nbhd[pa], pb);
        ivec_push(&c->nbhd[pb], pa);
      }
    return;
  }
  ivec s1c = {0}, s2c = {0}, s1r1 = {0}, s1r2 = {0}, s2r1 = {0}, s2r2 = {0};
  int nd = (diridx + 1) % 3;
  float npv = (mx[nd] + mn[nd]) / 2;
  float s1r1m = 0, s1r2m = 0, s2r1m = 0, s2r2m = 0;
  for (int64_t i = 0; i < s1->n; ++i) {
    const float* e = c->pts + 4 * s1->v[i];
    float rad = e[3];
    if (e[nd] <= npv) { ivec_push(&s1r1, s1->v[i]); if (rad > s1r1m) s1r1m = rad; }
    else { ivec_push(&s1r2, s1->v[i]); if (rad > s1r2m) s1r2m = rad; }
    if (e[diridx] + rad + s2maxrad <= pivot) continue;
    ivec_push(&s1c, s1->v[i]);
  }
  for (int64_t i = 0; i < s2->n; ++i) {
    const float* e = c->pts + 4 * s2->v[i];
    float rad = e[3];
    if (e[nd] <= npv) { ivec_push(&s2r1, s2->v[i]); if (rad > s2r1m) s2r1m = rad; }
    else { ivec_push(&s2r2, s2->v[i]); if (rad > s2r2m) s2r2m = rad; }
    if (e[diridx] - rad - s1maxrad >= pivot) continue;
    ivec_push(&s2c, s2->v[i]);
  }
  for (int64_t a = 0; a < s1c.n; ++a)
    for (int64_t b2 = 0; b2 < s2c.n; ++b2)
      if (check_dist(c->pts, s1c.v[a], s2c.v[b2])) {
        ivec_push(&c->nbhd[s1c.v[a]], s2c.v[b2]);
        ivec_push(&c->nbhd[s2c.v[b2]], s1c.v[a]);
      }
  free(s1c.v); free(s2c.v);
  if (s1->n > 1) {
    float m2[3] = {mx[0], mx[1], mx[2]};
    m2[diridx] = pivot;
    dac(c, &s1r1, &s1r2, s1r1m, s1r2m, mn, m2, nd, npv);
  }
  free(s1r1.v); free(s1r2.v);
  if (s2->n > 1) {
    float m1[3] = {mn[0], mn[1], mn[2]};
    m1[diridx] = pivot;
    dac(c, &s2r1, &s2r2, s2r1m, s2r2m, m1, mx, nd, npv);
  }
  free(s2r1.v); free(s2r2.v);
}

static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

static int64_t store_csr(orc_scene* s, ivec* nb, int64_t* row_ptr, int32_t* cols, int64_t cap) {
  int64_t nnz = 0;
  for (int64_t i = 0; i < s->nd; ++i) nnz += nb[i].n;
  free(s->nb_ptr); free(s->nb_idx);
  s->nb_ptr = (int64_t*)malloc(sizeof(int64_t) * (size_t)(s->nd + 1));
  s->nb_idx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
  int64_t off = 0;
  for (int64_t i = 0; i < s->nd; ++i) {
    qsort(nb[i].v, (size_t)nb[i].n, sizeof(int32_t), cmp_i32);
    s->nb_ptr[i] = off;
    if (nb[i].n) memcpy(s->nb_idx + off, nb[i].v, sizeof(int32_t) * (size_t)nb[i].n);
    off += nb[i].n;
    free(nb[i].v);
  }
  s->nb_ptr[s->nd] = off;
  free(nb);
  if (row_ptr) memcpy(row_ptr, s->nb_ptr, sizeof(int64_t) * (size_t)(s->nd + 1));
  if (cols) {
    if (nnz > cap) return -1;
    memcpy(cols, s->nb_idx, sizeof(int32_t) * (size_t)nnz);
  }
  return nnz;
}

int64_t orc_neighbors(orc_scene* s, int64_t* row_ptr, int32_t* cols, int64_t cap) {
  ivec* nb = (ivec*)calloc((size_t)(s->nd ? s->nd : 1), sizeof(ivec));
  if (s->nd > 0) {
    /* construct_neighborhood (disc_neighborhood.hpp:37-64); min/max are the
     * centre extents (point_cloud_disc_geometry.hpp:200-205) */
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int64_t i = 0; i < s->nd; ++i)
      for (int a = 0; a < 3; ++a) {
        float v = s->dc[4 * i + a];
        if (v < mn[a]) mn[a] = v;
        if (v > mx[a]) mx[a] = v;
      }
    int diridx = 0;
    float pivot = (mx[diridx] + mn[diridx]) / 2;
    float m1 = 0, m2 = 0;
    ivec a1 = {0}, a2 = {0};
    for (int64_t i = 0; i < s->nd; ++i) {
      float r = s->dc[4 * i + 3];
      if (s->dc[4 * i + diridx] <= pivot) { ivec_push(&a1, (int32_t)i); if (r > m1) m1 = r; }
      else { ivec_push(&a2, (int32_t)i); if (r > m2) m2 = r; }
    }
    nbctx c = {s->dc, nb};
    dac(&c, &a1, &a2, m1, m2, mn, mx, diridx, pivot);
    free(a1.v); free(a2.v);
  }
  return store_csr(s, nb, row_ptr, cols, cap);
}

int64_t orc_neighbors_bruteforce(orc_scene* s, int64_t* row_ptr, int32_t* cols, int64_t cap) {
  ivec* nb = (ivec*)calloc((size_t)(s->nd ? s->nd : 1), sizeof(ivec));
  for (int64_t i = 0; i < s->nd; ++i)
    for (int64_t j = i + 1; j < s->nd; ++j)
      if (check_dist(s->dc, (int32_t)i, (int32_t)j)) {
        ivec_push(&nb[i], (int32_t)j);
        ivec_push(&nb[j], (int32_t)i);
      }
  return store_csr(s, nb, row_ptr, cols, cap);
}

/* ------------------------------------------------------------------------ */
/* Exposed area: disc_bounding_box_intersector.hpp:43-441 restated.          */
/* ------------------------------------------------------------------------ */
typedef struct { float lx, ly, hx, hy; } bb_t;
typedef struct { float approach; int swap_xy, reflect_x; } approach_t;
typedef struct { bb_t bb; bb_t t[2][2]; } dbbi_t;

static void swapf(float* a, float* b) { float t = *a; *a = *b; *b = t; }

static void dbbi_init(dbbi_t* g, float xmin, float ymin, float xmax, float ymax) {
  g->bb.lx = xmin; g->bb.ly = ymin; g->bb.hx = xmax; g->bb.hy = ymax;
  g->t[0][0] = g->bb;
  bb_t* c = &g->t[1][0];
  *c = g->bb;
  swapf(&c->lx, &c->ly); swapf(&c->hx, &c->hy);
  c->ly *= -1; c->hy *= -1;
  c = &g->t[0][1];
  *c = g->bb;
  c->lx *= -1; c->hx *= -1; c->ly *= -1; c->hy *= -1;
  c = &g->t[1][1];
  *c = g->bb;
  swapf(&c->lx, &c->ly); swapf(&c->hx, &c->hy);
  c->lx *= -1; c->hx *= -1;
  if (g->bb.lx > g->bb.hx) swapf(&g->bb.lx, &g->bb.hx);
  if (g->bb.ly > g->bb.hy) swapf(&g->bb.ly, &g->bb.hy);
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      bb_t* r = &g->t[i][j];
      if (r->lx > r->hx) swapf(&r->lx, &r->hx);
      if (r->ly > r->hy) swapf(&r->ly, &r->hy);
    }
}

static float closest_approach1(const dbbi_t* g, const float* disc, v3 n, int swp, int refl) {
  int xi = 0, yi = 1;
  if (swp) { xi = 1; yi = 0; }
  float nn[3] = {n.x, n.y, n.z};
  float xx = disc[xi];
  float radius = disc[3];
  float nx = nn[xi], ny = nn[yi], nz = nn[2];
  if (refl) { xx = -xx; nx = -nx; }
  (void)nx;
  const bb_t* bb = &g->t[swp][refl];
  float xterm = radius * sqrtf(nz * nz + ny * ny);
  float hi = xx + xterm;
  if (hi <= bb->hx) return FLT_MAX;
  float lo = xx - xterm;
  if (lo >= bb->hx) return -FLT_MAX;
  if (xterm <= 1e-9) return FLT_MAX;
  return (bb->hx - xx) * radius / xterm;
}

static void closest_approach(const dbbi_t* g, const float* disc, v3 n, approach_t* res) {
  static const int tup[4][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 0}};
  for (int i = 0; i < 4; ++i) { res[i].approach = 0.0f; res[i].swap_xy = 0; res[i].reflect_x = 0; }
  for (int i = 0; i < 4; ++i) {
    res[i].approach = closest_approach1(g, disc, n, tup[i][0], tup[i][1]);
    res[i].swap_xy = tup[i][0];
    res[i].reflect_x = tup[i][1];
    if (res[i].approach < -disc[3]) return;
  }
}

static v3 scl(float f, v3 v) { return mk(v.x * f, v.y * f, v.z * f); }
static v3 sum3(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 diff3(v3 a, v3 b) { return mk(a.x + (-b.x), a.y + (-b.y), a.z + (-b.z)); }
static v3 neg3(v3 a) { return mk(-a.x, -a.y, -a.z); }

static float area_outside(const dbbi_t* g, const float* disc, v3 dn, const approach_t* ao) {
  float radius = disc[3];
  float area = 0.0f;
  for (int i = 0; i < 4; ++i) {
    float dd = ao[i].approach;
    if (-radius < dd && dd < radius) {
      double angle = 2 * acos((double)dd / radius);
      double seg = (double)(radius * radius / 2) * (angle - sin(angle));
      area = (float)((double)area + seg);
    }
  }
  for (int i = 0; i < 4; ++i) {
    const approach_t* a1 = &ao[i];
    const approach_t* a2 = &ao[(i + 1) % 4];
    float d1 = a1->approach, d2 = a2->approach;
    const bb_t* t1 = &g->t[a1->swap_xy][a1->reflect_x];
    const bb_t* t2 = &g->t[a2->swap_xy][a2->reflect_x];
    if (!(-radius < d1 && d1 < radius && -radius < d2 && d2 < radius)) continue;
    v3 dp = mk(disc[0], disc[1], disc[2]);
    v3 p1 = mk(t1->hx, t1->hy, 0), p2 = mk(t2->hx, t2->hy, 0);
    v3 n1 = normalize3(cross3(sub3(mk(t1->hx, t1->hy, 0), mk(t1->hx, t1->hy, 1)),
                              sub3(mk(t1->hx, t1->ly, 0), mk(t1->hx, t1->hy, 1))));
    v3 n2 = normalize3(cross3(sub3(mk(t2->hx, t2->hy, 0), mk(t2->hx, t2->hy, 1)),
                              sub3(mk(t2->hx, t2->ly, 0), mk(t2->hx, t2->hy, 1))));
    if (a1->reflect_x) { p1.y *= -1; n1.y *= -1; p1.x *= -1; n1.x *= -1; }
    if (a2->reflect_x) { p2.y *= -1; n2.y *= -1; p2.x *= -1; n2.x *= -1; }
    if (a1->swap_xy) { p1.y *= -1; n1.y *= -1; swapf(&p1.x, &p1.y); swapf(&n1.x, &n1.y); }
    if (a2->swap_xy) { p2.y *= -1; n2.y *= -1; swapf(&p2.x, &p2.y); swapf(&n2.x, &n2.y); }
    v3 id1 = normalize3(cross3(dn, n1));
    v3 id2 = normalize3(cross3(dn, n2));
    if (dot3(id1, n2) >= 0) id1 = neg3(id1);
    if (dot3(id2, n1) >= 0) id2 = neg3(id2);
    float xi = p2.x, yi = p2.y;
    v3 ip = mk(xi, yi,
               (dn.x * dp.x + dn.y * dp.y + dn.z * dp.z - dn.x * xi - dn.y * yi) / dn.z);
    if (dist3(dp, ip) >= radius) continue;
    v3 ic1 = diff3(dp, ip);
    float ca1 = dot3(ic1, id1);
    v3 cp1 = sum3(ip, scl(ca1, id1));
    float thc1 = sqrtf(radius * radius - d1 * d1);
    v3 q1 = sum3(cp1, scl(thc1, id1));
    v3 ic2 = diff3(dp, ip);
    float ca2 = dot3(ic2, id2);
    v3 cp2 = sum3(ip, scl(ca2, id2));
    float thc2 = sqrtf(radius * radius - d2 * d2);
    v3 q2 = sum3(cp2, scl(thc2, id2));
    v3 cq1 = diff3(q1, dp), cq2 = diff3(q2, dp);
    float ang = acosf(dot3(cq1, cq2) / len3(cq1) / len3(cq2));
    float oseg = radius * radius / 2 * (ang - sinf(ang));
    v3 k1 = diff3(q1, ip), k2 = diff3(q2, ip);
    float otri = 0.5f * len3(cross3(k1, k2));
    area -= oseg + otri;
  }
  return area;
}

static float area_inside_g(const dbbi_t* g, const float* disc, const float* nrm) {
  v3 dn = normalize3(mk(nrm[0], nrm[1], nrm[2]));
  float xx = disc[0], yy = disc[1], r = disc[3];
  if (r <= 0) return 0.0f;
  float full = r * r * (float)3.14159265358979323846;
  const bb_t* b = &g->bb;
  if ((b->lx <= xx - r && xx + r <= b->hx) && (b->ly <= yy - r && yy + r <= b->hy)) return full;
  if ((xx + r <= b->lx || b->hx <= xx - r) || (yy + r <= b->ly || b->hy <= yy - r)) return 0.0f;
  approach_t ao[4];
  closest_approach(g, disc, dn, ao);
  for (int i = 0; i < 4; ++i)
    if (ao[i].approach < -r) return 0.0f;
  return full - area_outside(g, disc, dn, ao);
}

float orc_area_inside(float xmin, float ymin, float xmax, float ymax, const float* disc,
                      const float* normal) {
  dbbi_t g;
  dbbi_init(&g, xmin, ymin, xmax, ymax);
  return area_inside_g(&g, disc, normal);
}

void orc_areas(const orc_scene* s, float xmin, float ymin, float xmax, float ymax, float* out) {
  dbbi_t g;
  dbbi_init(&g, xmin, ymin, xmax, ymax);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < s->nd; ++i) out[i] = area_inside_g(&g, s->dc + 4 * i, s->dn + 3 * i);
  for (int64_t i = 0; i < s->nt; ++i) {
    /* util::area_of_triangle (utils.hpp:161-169) */
    v3 c = cross3(ld3(s->te1, i), ld3(s->te2, i));
    out[s->nd + i] = (float)(0.5 * len3(c));
  }
}

/* ------------------------------------------------------------------------ */
/* Results                                                                   */
/* ------------------------------------------------------------------------ */
void orc_normalize(int64_t n, const double* s1, const float* areas, const int64_t* rp,
                   const int32_t* cols, float* out) {
  double maxv = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double vv = s1[i] / areas[i];
    int64_t deg = 0;
    if (rp) {
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q) vv += s1[cols[q]] / areas[cols[q]];
      deg = rp[i + 1] - rp[i];
    }
    vv /= (double)(deg + 1);
    out[i] = (float)vv;
    if (maxv < vv) maxv = vv;
  }
  for (int64_t i = 0; i < n; ++i) out[i] = (float)((double)out[i] / maxv);
}

void orc_relative_error(int64_t n, const double* s1, const double* s2, uint64_t total, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    out[i] = DBL_MAX;
    if (total == 0) continue;
    double sq = s1[i] * s1[i];
    if (sq == 0) continue;
    out[i] = sqrt(s2[i] / sq - 1.0 / (double)total);
  }
}

void orc_vov(int64_t n, const double* s1, const double* s2, const double* s3, const double* s4,
             const uint64_t* cnt, uint64_t total, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    out[i] = DBL_MAX;
    if (cnt[i] == 0) continue;
    double a = s1[i], b = s2[i], c = s3[i], d = s4[i];
    double a2 = a * a, a4 = a2 * a2, b2 = b * b;
    uint64_t nn = total;
    uint64_t nn2 = nn * nn, nn3 = nn * nn * nn;
    double num = d - (4 * a * c / nn) + (8 * b * a2 / nn2) - (4 * a4 / nn3) - (b2 / nn);
    double dr2 = nn * b - a2;
    double den2 = dr2 * dr2;
    if (den2 == 0) { out[i] = DBL_MAX; continue; }
    out[i] = num / den2 * nn * nn;
  }
}
