// rtg_surface.cu -- per-element kernels around the trace:
//   * neighbour lists of overlapping discs (disc_neighborhood.hpp:20-220):
//     uniform grid of cell size 2*r_max, each disc tests the 27 surrounding
//     cells with the reference's predicate distance(c_i, c_j) < r_i + r_j;
//     rows are sorted by id (CSR);
//   * exposed disc area inside the x/y box (disc_bounding_box_intersector.hpp:
//     43-441) and triangle areas (utils.hpp:161-169), one thread per element;
//   * normalised, neighbourhood-smoothed estimates (device.hpp:154-187);
//   * relative error and variance of variance (hit_accumulator.hpp:152-249).
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "rtg_internal.cuh"
#include "rtg_math.cuh"

namespace rtg {

namespace {

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct Grid {
  float org[3];
  float h;
  int dim[3];
};

__device__ __forceinline__ int cell_coord(float v, float org, float h, int dim) {
  int c = (int)floor(((double)v - (double)org) / (double)h);
  return c < 0 ? 0 : (c >= dim ? dim - 1 : c);
}

__global__ void cell_key_kernel(const float4* __restrict__ dcr, int64_t nd, Grid g, uint32_t* __restrict__ keys,
                                uint32_t* __restrict__ vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nd) return;
  float4 c = dcr[i];
  int cx = cell_coord(c.x, g.org[0], g.h, g.dim[0]);
  int cy = cell_coord(c.y, g.org[1], g.h, g.dim[1]);
  int cz = cell_coord(c.z, g.org[2], g.h, g.dim[2]);
  keys[i] = (uint32_t)((cz * g.dim[1] + cy) * g.dim[0] + cx);
  vals[i] = (uint32_t)i;
}

__global__ void cell_range_kernel(const uint32_t* __restrict__ keys, int64_t nd, uint32_t* __restrict__ start,
                                  uint32_t* __restrict__ end) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nd) return;
  uint32_t k = keys[i];
  if (i == 0 || keys[i - 1] != k) start[k] = (uint32_t)i;
  if (i == nd - 1 || keys[i + 1] != k) end[k] = (uint32_t)(i + 1);
}

// check_dist (disc_neighborhood.hpp:190-220): the three axis pre-tests are
// implied by the distance test in IEEE arithmetic and are omitted.
__device__ __forceinline__ bool overlaps(float4 a, float4 b) {
  float d1 = a.x - b.x, d2 = a.y - b.y, d3 = a.z - b.z;
  float dist = sqrtf(d1 * d1 + d2 * d2 + d3 * d3);
  return dist < a.w + b.w;
}

template <bool kFill>
__global__ void neighbor_kernel(const float4* __restrict__ dcr, int64_t nd, Grid g,
                                const uint32_t* __restrict__ sorted_ids, const uint32_t* __restrict__ start,
                                const uint32_t* __restrict__ end, int64_t* __restrict__ counts,
                                const int64_t* __restrict__ row_ptr, int32_t* __restrict__ cols) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nd) return;
  const float4 ci = dcr[i];
  const int cx = cell_coord(ci.x, g.org[0], g.h, g.dim[0]);
  const int cy = cell_coord(ci.y, g.org[1], g.h, g.dim[1]);
  const int cz = cell_coord(ci.z, g.org[2], g.h, g.dim[2]);
  int64_t cnt = 0;
  int64_t out = kFill ? row_ptr[i] : 0;
  for (int z = cz - 1; z <= cz + 1; ++z) {
    if (z < 0 || z >= g.dim[2]) continue;
    for (int y = cy - 1; y <= cy + 1; ++y) {
      if (y < 0 || y >= g.dim[1]) continue;
      for (int x = cx - 1; x <= cx + 1; ++x) {
        if (x < 0 || x >= g.dim[0]) continue;
        const uint32_t cell = (uint32_t)((z * g.dim[1] + y) * g.dim[0] + x);
        const uint32_t b = start[cell];
        if (b == 0xFFFFFFFFu) continue;
        const uint32_t e = end[cell];
        for (uint32_t q = b; q < e; ++q) {
          const uint32_t j = sorted_ids[q];
          if (j == (uint32_t)i) continue;
          if (overlaps(ci, dcr[j])) {
            if (kFill) cols[out + cnt] = (int32_t)j;
            ++cnt;
          }
        }
      }
    }
  }
  if (kFill) {
    // insertion sort of the row by id
    for (int64_t a = out + 1; a < out + cnt; ++a) {
      int32_t v = cols[a];
      int64_t b = a - 1;
      while (b >= out && cols[b] > v) {
        cols[b + 1] = cols[b];
        --b;
      }
      cols[b + 1] = v;
    }
  } else {
    counts[i] = cnt;
  }
}

// ---------------- exposed area (disc_bounding_box_intersector.hpp) ----------
struct BB {
  float lx, ly, hx, hy;
};
struct DBBI {
  BB bb;
  BB t[2][2];
};

__host__ __device__ inline void swapf(float& a, float& b) {
  float t = a;
  a = b;
  b = t;
}

// fill_bboxtransforms / fix_bboxtransforms (lines 265-340)
inline DBBI make_dbbi(float xmin, float ymin, float xmax, float ymax) {
  DBBI g;
  g.bb = BB{xmin, ymin, xmax, ymax};
  g.t[0][0] = g.bb;
  BB c = g.bb;
  swapf(c.lx, c.ly);
  swapf(c.hx, c.hy);
  c.ly *= -1;
  c.hy *= -1;
  g.t[1][0] = c;
  c = g.bb;
  c.lx *= -1;
  c.hx *= -1;
  c.ly *= -1;
  c.hy *= -1;
  g.t[0][1] = c;
  c = g.bb;
  swapf(c.lx, c.ly);
  swapf(c.hx, c.hy);
  c.lx *= -1;
  c.hx *= -1;
  g.t[1][1] = c;
  if (g.bb.lx > g.bb.hx) swapf(g.bb.lx, g.bb.hx);
  if (g.bb.ly > g.bb.hy) swapf(g.bb.ly, g.bb.hy);
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      BB& r = g.t[i][j];
      if (r.lx > r.hx) swapf(r.lx, r.hx);
      if (r.ly > r.hy) swapf(r.ly, r.hy);
    }
  return g;
}

struct Approach {
  float approach;
  int swp, refl;
};

// compute_closest_approach(disc, normal, swapXY, reflectX) (lines 372-441)
__device__ float closest_approach1(const DBBI& g, float4 disc, f3 n, int swp, int refl) {
  float xx = swp ? disc.y : disc.x;
  float ny = swp ? n.x : n.y;
  float nz = n.z;
  if (refl) xx = -xx;
  const BB& bb = g.t[swp][refl];
  const float radius = disc.w;
  float xterm = radius * sqrtf(nz * nz + ny * ny);
  if (xx + xterm <= bb.hx) return FLT_MAX;
  if (xx - xterm >= bb.hx) return -FLT_MAX;
  if ((double)xterm <= 1e-9) return FLT_MAX;
  return (bb.hx - xx) * radius / xterm;
}

__device__ f3 neg3(f3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ f3 scl3(float f, f3 v) { return mk3(v.x * f, v.y * f, v.z * f); }
__device__ f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ f3 diff3(f3 a, f3 b) { return mk3(a.x + (-b.x), a.y + (-b.y), a.z + (-b.z)); }
__device__ float dist3(f3 a, f3 b) {
  float d1 = a.x - b.x, d2 = a.y - b.y, d3 = a.z - b.z;
  return sqrtf(d1 * d1 + d2 * d2 + d3 * d3);
}

// compute_area_outside_given_closest_approach (lines 108-263)
__device__ float area_outside(const DBBI& g, float4 disc, f3 dn, const Approach* ao) {
  const float radius = disc.w;
  float area = 0.0f;
  for (int i = 0; i < 4; ++i) {
    const float dd = ao[i].approach;
    if (-radius < dd && dd < radius) {
      double angle = 2 * acos((double)dd / radius);
      double seg = (double)(radius * radius / 2) * (angle - sin(angle));
      area = (float)((double)area + seg);
    }
  }
  for (int i = 0; i < 4; ++i) {
    const Approach& a1 = ao[i];
    const Approach& a2 = ao[(i + 1) % 4];
    const float d1 = a1.approach, d2 = a2.approach;
    const BB& t1 = g.t[a1.swp][a1.refl];
    const BB& t2 = g.t[a2.swp][a2.refl];
    if (!(-radius < d1 && d1 < radius && -radius < d2 && d2 < radius)) continue;
    f3 dp = mk3(disc.x, disc.y, disc.z);
    f3 p1 = mk3(t1.hx, t1.hy, 0), p2 = mk3(t2.hx, t2.hy, 0);
    f3 n1 = normalize3(cross3(sub3(mk3(t1.hx, t1.hy, 0), mk3(t1.hx, t1.hy, 1)),
                              sub3(mk3(t1.hx, t1.ly, 0), mk3(t1.hx, t1.hy, 1))));
    f3 n2 = normalize3(cross3(sub3(mk3(t2.hx, t2.hy, 0), mk3(t2.hx, t2.hy, 1)),
                              sub3(mk3(t2.hx, t2.ly, 0), mk3(t2.hx, t2.hy, 1))));
    if (a1.refl) { p1.y *= -1; n1.y *= -1; p1.x *= -1; n1.x *= -1; }
    if (a2.refl) { p2.y *= -1; n2.y *= -1; p2.x *= -1; n2.x *= -1; }
    if (a1.swp) { p1.y *= -1; n1.y *= -1; swapf(p1.x, p1.y); swapf(n1.x, n1.y); }
    if (a2.swp) { p2.y *= -1; n2.y *= -1; swapf(p2.x, p2.y); swapf(n2.x, n2.y); }
    f3 id1 = normalize3(cross3(dn, n1));
    f3 id2 = normalize3(cross3(dn, n2));
    if (dot3(id1, n2) >= 0) id1 = neg3(id1);
    if (dot3(id2, n1) >= 0) id2 = neg3(id2);
    const float xi = p2.x, yi = p2.y;
    f3 ip = mk3(xi, yi, (dn.x * dp.x + dn.y * dp.y + dn.z * dp.z - dn.x * xi - dn.y * yi) / dn.z);
    if (dist3(dp, ip) >= radius) continue;
    f3 ic1 = diff3(dp, ip);
    float ca1 = dot3(ic1, id1);
    f3 cp1 = add3(ip, scl3(ca1, id1));
    float thc1 = sqrtf(radius * radius - d1 * d1);
    f3 q1 = add3(cp1, scl3(thc1, id1));
    f3 ic2 = diff3(dp, ip);
    float ca2 = dot3(ic2, id2);
    f3 cp2 = add3(ip, scl3(ca2, id2));
    float thc2 = sqrtf(radius * radius - d2 * d2);
    f3 q2 = add3(cp2, scl3(thc2, id2));
    f3 cq1 = diff3(q1, dp), cq2 = diff3(q2, dp);
    float ang = acosf(dot3(cq1, cq2) / len3(cq1) / len3(cq2));
    float oseg = radius * radius / 2 * (ang - sinf(ang));
    f3 k1 = diff3(q1, ip), k2 = diff3(q2, ip);
    float otri = 0.5f * len3(cross3(k1, k2));
    area -= oseg + otri;
  }
  return area;
}

// area_inside (lines 42-76)
__device__ float area_inside(const DBBI& g, float4 disc, float4 nrm) {
  f3 dn = normalize3(mk3(nrm.x, nrm.y, nrm.z));
  const float xx = disc.x, yy = disc.y, r = disc.w;
  if (r <= 0) return 0.0f;
  const float full = r * r * (float)3.14159265358979323846;
  const BB& b = g.bb;
  if ((b.lx <= xx - r && xx + r <= b.hx) && (b.ly <= yy - r && yy + r <= b.hy)) return full;
  if ((xx + r <= b.lx || b.hx <= xx - r) || (yy + r <= b.ly || b.hy <= yy - r)) return 0.0f;
  // order right, bottom, left, top: (swap, reflect) = (0,0) (1,1) (0,1) (1,0)
  Approach ao[4];
  for (int i = 0; i < 4; ++i) ao[i] = Approach{0.0f, 0, 0};
  for (int i = 0; i < 4; ++i) {
    const int swp = (i == 1 || i == 3) ? 1 : 0, refl = (i == 1 || i == 2) ? 1 : 0;
    ao[i].approach = closest_approach1(g, disc, dn, swp, refl);
    ao[i].swp = swp;
    ao[i].refl = refl;
    if (ao[i].approach < -r) break;
  }
  for (int i = 0; i < 4; ++i)
    if (ao[i].approach < -r) return 0.0f;
  return full - area_outside(g, disc, dn, ao);
}

__global__ void area_kernel(const float4* __restrict__ dcr, const float4* __restrict__ dn, int64_t nd,
                            const float4* __restrict__ tv, const uint32_t* __restrict__ tidx, int64_t nt,
                            DBBI g, float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nd) {
    out[i] = area_inside(g, dcr[i], dn[i]);
  } else if (i < nd + nt) {
    int64_t t = i - nd;
    float4 a = tv[tidx[3 * t]], b = tv[tidx[3 * t + 1]], c = tv[tidx[3 * t + 2]];
    f3 v0 = mk3(a.x, a.y, a.z);
    f3 e1 = sub3(mk3(b.x, b.y, b.z), v0), e2 = sub3(mk3(c.x, c.y, c.z), v0);
    out[i] = (float)(0.5 * len3(cross3(e1, e2)));
  }
}

// ---------------- normalised smoothed estimates (device.hpp:154-187) --------
__global__ void smooth_kernel(const double* __restrict__ s1, const float* __restrict__ areas, int64_t n,
                              int64_t nd, const int64_t* __restrict__ rp, const int32_t* __restrict__ cols,
                              float* __restrict__ est, unsigned long long* __restrict__ maxbits) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
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
  // maxv tracks only values that compare greater than the running max (0 start)
  double m = (i < n && vv > 0.0) ? vv : 0.0;
  for (int o = 16; o > 0; o >>= 1) {
    double y = __shfl_down_sync(0xFFFFFFFFu, m, o);
    if (y > m) m = y;
  }
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
}

__global__ void divide_kernel(float* __restrict__ est, int64_t n, const unsigned long long* __restrict__ maxbits) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double maxv = __longlong_as_double((long long)*maxbits);
  est[i] = (float)((double)est[i] / maxv);
}

__global__ void stats_kernel(const double* __restrict__ s1, const double* __restrict__ s2,
                             const double* __restrict__ s3, const double* __restrict__ s4,
                             const unsigned long long* __restrict__ cnt, int64_t n, unsigned long long total,
                             double* __restrict__ rel, double* __restrict__ vov) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // get_relative_error (hit_accumulator.hpp:152-186)
  double r = DBL_MAX;
  if (total != 0) {
    double sq = s1[i] * s1[i];
    if (sq != 0) r = sqrt(s2[i] / sq - 1.0 / (double)total);
  }
  rel[i] = r;
  // get_vov (hit_accumulator.hpp:188-249)
  double v = DBL_MAX;
  if (cnt[i] != 0) {
    double a = s1[i], b = s2[i], c = s3[i], d = s4[i];
    double a2 = a * a, a4 = a2 * a2, b2 = b * b;
    unsigned long long nn = total, nn2 = nn * nn, nn3 = nn * nn * nn;
    double num = d - (4 * a * c / nn) + (8 * b * a2 / nn2) - (4 * a4 / nn3) - (b2 / nn);
    double dr2 = nn * b - a2;
    double den2 = dr2 * dr2;
    v = den2 == 0 ? DBL_MAX : num / den2 * nn * nn;
  }
  vov[i] = v;
}

}  // namespace

// Neighbour columns as disc slots, for the trace (one 256-bit record load per neighbour).
__global__ void nb_slot_kernel(const int32_t* __restrict__ nb_idx, int64_t nnz, const uint32_t* __restrict__ slot_of_id,
                               uint32_t* __restrict__ nb_slot) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nnz) nb_slot[q] = slot_of_id[nb_idx[q]];
}

int build_neighbors(rtg_context* ctx) {
  Geometry& g = ctx->g;
  cudaStream_t st = ctx->stream;
  const int64_t nd = g.nd;
  g.nb_nnz = 0;
  RTG_TRY(dalloc(ctx, g.nb_ptr, (size_t)(nd + 1), "neighbour row pointers"));
  if (nd == 0) return RTG_OK;
  if (nd == 1) {
    RTG_CUDA(ctx, cudaMemsetAsync(g.nb_ptr.p, 0, 2 * sizeof(int64_t), st));
    RTG_TRY(dalloc(ctx, g.nb_idx, 1, "neighbour columns"));
    RTG_TRY(dalloc(ctx, g.nb_slot, 1, "neighbour slots"));
    return RTG_OK;
  }
  Grid grid;
  float h = 2.0f * g.rmax * 1.000001f;
  if (!(h > 0.0f)) h = 1.0f;
  double ext[3];
  for (int a = 0; a < 3; ++a) ext[a] = (double)g.cmax[a] - (double)g.cmin[a];
  // cap the number of cells near 2 per disc; larger cells keep the test exact
  for (;;) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) cells *= std::floor(ext[a] / h) + 1.0;
    if (cells <= 2.0 * (double)nd + 64.0 && cells < 2.0e9) break;
    h *= 1.25f;
  }
  for (int a = 0; a < 3; ++a) {
    grid.org[a] = g.cmin[a];
    grid.dim[a] = (int)std::floor(ext[a] / h) + 1;
  }
  grid.h = h;
  const int64_t ncells = (int64_t)grid.dim[0] * grid.dim[1] * grid.dim[2];
  DBuf<uint32_t> keys, vals, tk, tv, cs, ce;
  DBuf<int64_t> counts;
  auto cleanup = [&]() { tfree(keys, st); tfree(vals, st); tfree(tk, st); tfree(tv, st); tfree(cs, st); tfree(ce, st); tfree(counts, st); };
  int rc = RTG_OK;
  do {
    if ((rc = talloc(ctx, keys, (size_t)nd, st, "grid keys")) != RTG_OK) break;
    if ((rc = talloc(ctx, vals, (size_t)nd, st, "grid ids")) != RTG_OK) break;
    if ((rc = talloc(ctx, tk, (size_t)nd, st, "sort scratch")) != RTG_OK) break;
    if ((rc = talloc(ctx, tv, (size_t)nd, st, "sort scratch")) != RTG_OK) break;
    if ((rc = talloc(ctx, cs, (size_t)ncells, st, "cell starts")) != RTG_OK) break;
    if ((rc = talloc(ctx, ce, (size_t)ncells, st, "cell ends")) != RTG_OK) break;
    if ((rc = talloc(ctx, counts, (size_t)(nd + 1), st, "neighbour counts")) != RTG_OK) break;
    cell_key_kernel<<<blocks_for(nd, 256), 256, 0, st>>>(g.disc_cr_by_id.p, nd, grid, keys.p, vals.p);
    int bits = 1;
    while (bits < 32 && ((int64_t)1 << bits) < ncells) ++bits;
    if ((rc = radix_sort_pairs(ctx, keys.p, vals.p, tk.p, tv.p, nd, bits, st)) != RTG_OK) break;
    cudaMemsetAsync(cs.p, 0xFF, ncells * sizeof(uint32_t), st);
    cudaMemsetAsync(ce.p, 0x00, ncells * sizeof(uint32_t), st);
    cell_range_kernel<<<blocks_for(nd, 256), 256, 0, st>>>(keys.p, nd, cs.p, ce.p);
    neighbor_kernel<false><<<blocks_for(nd, 128), 128, 0, st>>>(g.disc_cr_by_id.p, nd, grid, vals.p, cs.p, ce.p,
                                                                counts.p, nullptr, nullptr);
    cudaMemsetAsync(counts.p + nd, 0, sizeof(int64_t), st);
    int64_t* total = g.nb_ptr.p + nd;
    if ((rc = exclusive_scan_i64(ctx, counts.p, nd + 1, nullptr, st)) != RTG_OK) break;
    int64_t nnz = 0;
    cudaError_t cerr = cudaMemcpyAsync(g.nb_ptr.p, counts.p, (nd + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice, st);
    if (cerr == cudaSuccess) cerr = cudaMemcpyAsync(&nnz, total, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cerr == cudaSuccess) cerr = cudaStreamSynchronize(st);
    if (cerr != cudaSuccess) {
      rc = check_cuda(ctx, cerr, "neighbour counts");
      break;
    }
    g.nb_nnz = nnz;
    if ((rc = dalloc(ctx, g.nb_idx, (size_t)(nnz > 0 ? nnz : 1), "neighbour columns")) != RTG_OK) break;
    neighbor_kernel<true><<<blocks_for(nd, 128), 128, 0, st>>>(g.disc_cr_by_id.p, nd, grid, vals.p, cs.p, ce.p,
                                                               nullptr, g.nb_ptr.p, g.nb_idx.p);
    if ((rc = dalloc(ctx, g.nb_slot, (size_t)(nnz > 0 ? nnz : 1), "neighbour slots")) != RTG_OK) break;
    if (nnz > 0)
      nb_slot_kernel<<<blocks_for(nnz, 256), 256, 0, st>>>(g.nb_idx.p, nnz, g.disc_slot.p, g.nb_slot.p);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) rc = check_cuda(ctx, e, "neighbour lists");
  } while (0);
  cleanup();
  return rc;
}

int compute_areas_into(rtg_context* ctx, cudaStream_t st, const float* box_lo, const float* box_hi, float* out) {
  Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  DBBI dbbi = make_dbbi(box_lo[0], box_lo[1], box_hi[0], box_hi[1]);
  area_kernel<<<blocks_for(np, 256), 256, 0, st>>>(g.disc_cr_by_id.p, g.disc_n_by_id.p, g.nd, g.tri_v.p,
                                                   g.tri_idx.p, g.nt, dbbi, out);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

int compute_areas(rtg_context* ctx, cudaStream_t st, const float* box_lo, const float* box_hi) {
  return compute_areas_into(ctx, st, box_lo, box_hi, ctx->areas.p);
}

int finalize_estimates(rtg_context* ctx, cudaStream_t st) {
  Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  DBuf<unsigned long long> mx;
  RTG_TRY(dalloc(ctx, mx, 1, "max"));
  cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), st);
  smooth_kernel<<<blocks_for(np, 256), 256, 0, st>>>(ctx->acc.p, ctx->areas.p, np, g.nd,
                                                     g.nd > 0 ? g.nb_ptr.p : nullptr, g.nb_idx.p, ctx->est.p,
                                                     mx.p);
  divide_kernel<<<blocks_for(np, 256), 256, 0, st>>>(ctx->est.p, np, mx.p);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  dfree(mx);
  if (e != cudaSuccess) return check_cuda(ctx, e, "normalised estimates");
  return RTG_OK;
}

int compute_stats(rtg_context* ctx, cudaStream_t st, uint64_t total, double* d_rel, double* d_vov) {
  const int64_t np = ctx->g.nd + ctx->g.nt;
  const double* s = ctx->acc.p;
  stats_kernel<<<blocks_for(np, 256), 256, 0, st>>>(s, s + np, s + 2 * np, s + 3 * np, ctx->cnt.p, np, total,
                                                    d_rel, d_vov);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

}  // namespace rtg
