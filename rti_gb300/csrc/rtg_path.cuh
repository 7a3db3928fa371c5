// rtg_path.cuh -- the persistent path-tracing kernel (a template included by
// the translation units that instantiate it) and the closest-hit traversal.
//
// One thread carries one particle path at a time, as tracer::run does per
// OpenMP iteration (tracer.hpp:160-280): source ray, closest hit, periodic or
// reflective x/y box, back-face pass-through, sticking deposit on the hit
// primitive and on every crossed overlapping neighbour disc (kModeWindow: on
// every disc met in the multi-hit window instead), Russian roulette,
// diffuse/specular re-emission.  Threads are persistent: when at
// least `packet` lanes of a warp are idle, the warp takes that many next
// source-ray ids from a global counter (one atomic per warp), so long and
// short paths share the SIMD lanes.
//
// Closest hit = stack traversal of the two-box LBVH nodes; ties in t go to the
// lower primitive id, and the node boxes are conservative, so the chosen hit
// does not depend on the traversal order.  The stack holds STACK entries (in
// local memory, or in shared memory with one column per thread); a tree
// deeper than that would overflow it (counted as an error), so the host picks
// STACK from the tree depth.
#pragma once
#include <cfloat>
#include <climits>
#include <cstdint>

#include "rtg_internal.cuh"
#include "rtg_math.cuh"

namespace rtg {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

// A build with -DRTG_CHECKED verifies every node, slot, primitive and
// neighbour index read from device data before it is used, and counts a bad
// one as an error (tally.errors) instead of dereferencing it.
#ifdef RTG_CHECKED
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif

__device__ __forceinline__ bool node_in_range(const SceneView& s, uint32_t cur) {
  return cur < (s.nd + s.nt > 1 ? (uint32_t)(s.nd + s.nt - 1) : 1u);
}
__device__ __forceinline__ bool leaf_in_range(const SceneView& s, uint32_t ref) {
  return (ref & kTriBit) ? (ref & kSlotMask) < (uint32_t)s.nt : (ref & kSlotMask) < (uint32_t)s.nd;
}
constexpr uint32_t kNoLeaf = 0xFFFFFFFFu;  // no child reference: slots stay below kSlotMask

// Maximum and minimum of three floats in one instruction (sm_100+); exact,
// so the result equals the two-input forms'.
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

__device__ __forceinline__ float safe_inv(float d) {
  if (fabsf(d) < 1e-30f) d = d < 0.0f ? -1e-30f : 1e-30f;
  return 1.0f / d;
}

struct Ray {
  f3 o, d, idr;
};

// Slab test of one child box; returns the entry distance in tn.
__device__ __forceinline__ bool slab(float lx, float hx, float ly, float hy, float lz, float hz, const Ray& r,
                                     float tmax, float& tn) {
  float t0x = (lx - r.o.x) * r.idr.x, t1x = (hx - r.o.x) * r.idr.x;
  float t0y = (ly - r.o.y) * r.idr.y, t1y = (hy - r.o.y) * r.idr.y;
  float t0z = (lz - r.o.z) * r.idr.z, t1z = (hz - r.o.z) * r.idr.z;
  tn = max3f(fminf(t0x, t1x), fminf(t0y, t1y), fmaxf(fminf(t0z, t1z), 0.0f));
  float tf = min3f(fmaxf(t0x, t1x), fmaxf(t0y, t1y), fmaxf(t0z, t1z));
  return tn <= tf * 1.0000005f && tn <= tmax * 1.0000005f + 1e-30f;
}

// One 64-B node as two 256-bit read-only loads (sm_100+ vector width; the
// node array is 64-B aligned): fewer load instructions than four 128-bit ones.
__device__ __forceinline__ void load_node(const Node* nd, float4& a, float4& b, float4& c, uint4& d) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(nd));
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w), "=r"(d.x), "=r"(d.y), "=r"(d.z), "=r"(d.w)
      : "l"(reinterpret_cast<const char*>(nd) + 32));
}

__device__ __forceinline__ void test_leaf(const SceneView& s, uint32_t ref, const Ray& r, float tnear, float& bt,
                                          int& bid, uint32_t& bref) {
  const uint32_t slot = ref & kSlotMask;
  float t;
  int id;
  bool h;
  if (ref & kTriBit) {
    float4 a, b;  // (v0, id bits), e1 as one 256-bit load; e2 as one 128-bit load
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(s.tri + 4 * (int64_t)slot));
    const float4 c = __ldg(&s.tri[4 * (int64_t)slot + 2]);
    id = __float_as_int(a.w);
    h = tri_test(mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z), r.o, r.d, tnear, t);
  } else {
    float4 cr, nn;  // one 32-B record: (centre, radius), (normal, id bits)
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(cr.x), "=f"(cr.y), "=f"(cr.z), "=f"(cr.w), "=f"(nn.x), "=f"(nn.y), "=f"(nn.z), "=f"(nn.w)
        : "l"(s.disc + 2 * (int64_t)slot));
    id = __float_as_int(nn.w);
    h = disc_test(mk3(cr.x, cr.y, cr.z), cr.w, mk3(nn.x, nn.y, nn.z), r.o, r.d, tnear, t);
  }
  if (h && (t < bt || (t == bt && id < bid))) {
    bt = t;
    bid = id;
    bref = ref;
  }
}

// Child reference of slot c (0..7) from the eight references of a wide node,
// by selects rather than an indexed (local-memory) array.
__device__ __forceinline__ uint32_t pick8(const uint32_t* r, uint32_t c) {
  const bool b0 = c & 1u, b1 = c & 2u, b2 = c & 4u;
  const uint32_t a01 = b0 ? r[1] : r[0], a23 = b0 ? r[3] : r[2];
  const uint32_t a45 = b0 ? r[5] : r[4], a67 = b0 ? r[7] : r[6];
  const uint32_t lo = b1 ? a23 : a01, hi = b1 ? a67 : a45;
  return b2 ? hi : lo;
}

// Bit i of the result is bit (i ^ o) of m (an 8-bit mask): the slots of a
// wide node in the visiting order of a ray with octant code o.
__device__ __forceinline__ uint32_t xor_perm8(uint32_t m, uint32_t o) {
  if (o & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
  if (o & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
  if (o & 4u) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
  return m;
}

// Closest hit over the compressed 8-wide tree (WideNode, rtg_wide.cu).  One
// node = three 256-bit loads; its eight child boxes are tested with two
// instructions per slab plane: q as the float 2^23 + q by a byte permute, then
// t = (2^23 + q) a + c with a = 2^e / d (exact) and c = (p - o) / d - 2^23 a
// moved outwards by a margin m = 1.02 |a| + 2^-21 |(p - o) / d|, which bounds
// every rounding on the way (c, the shift, and the final FMA: |t| is at most
// 255 |a| + |(p - o) / d|), so the interval tested always contains the exact
// slab interval of the decoded box -- and the decoded box contains the binary
// tree's box of the same child.  A box the exact test misses holds no
// primitive hit (the primitive boxes are padded well beyond rounding), and
// the exact entry distance of a box holding a hit at t <= bt is <= bt, so the
// test is tn <= min(tf, bt) without a relative slack.  Hit primitives are tested on the spot; the
// internal children hit are visited in the ray's octant order (xor_perm8),
// the nearest-first one at once and the others from the stack.  The closest
// hit (ties to the lower id) is therefore the binary traversal's.
// lstack: the caller's local stack (SST = 0), else sstk: a shared column.
template <int STACK, int SST, typename Count>
__device__ __forceinline__ bool closest_hit_wide(const SceneView& s, const Ray& r, float tnear, float& bt, int& bid,
                                                 uint32_t& bref, Count& errs, uint32_t* lstack, uint32_t* sstk) {
  auto stack = [&](int i) -> uint32_t& { return SST ? sstk[i * SST] : lstack[i]; };
  int sp = 0;
  const uint32_t oct = (r.idr.x < 0.0f ? 1u : 0u) | (r.idr.y < 0.0f ? 2u : 0u) | (r.idr.z < 0.0f ? 4u : 0u);
  uint32_t cur = 0;
  const uint32_t max_iter = s.max_visits;
  for (uint32_t it = 0;; ++it) {
    if (it >= max_iter || (kChecked && cur >= s.n_wnodes)) {
      errs += 1;
      break;
    }
    uint32_t w[24];
    const uint32_t* np_ = s.wnodes[cur].w;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
          : "=r"(w[8 * k]), "=r"(w[8 * k + 1]), "=r"(w[8 * k + 2]), "=r"(w[8 * k + 3]), "=r"(w[8 * k + 4]),
            "=r"(w[8 * k + 5]), "=r"(w[8 * k + 6]), "=r"(w[8 * k + 7])
          : "l"(np_ + 8 * k));
    float a[3], cn[3], cf[3];
    uint32_t nw[3][2], fw[3][2];
    const float oo[3] = {r.o.x, r.o.y, r.o.z}, id[3] = {r.idr.x, r.idr.y, r.idr.z};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const float sc = __uint_as_float(((w[3] >> (8 * ax)) & 0xFFu) << 23);  // 2^e
      a[ax] = sc * id[ax];
      const float b = (__uint_as_float(w[ax]) - oo[ax]) * id[ax];
      const float c = fmaf(-8388608.0f, a[ax], b);
      const float m = fmaf(fabsf(b), 0x1p-21f, 1.02f * fabsf(a[ax]));
      cn[ax] = c - m;
      cf[ax] = c + m;
      const bool pos = id[ax] >= 0.0f;  // near plane = lo for a positive direction, else hi
      nw[ax][0] = pos ? w[12 + 2 * ax] : w[18 + 2 * ax];
      nw[ax][1] = pos ? w[13 + 2 * ax] : w[19 + 2 * ax];
      fw[ax][0] = pos ? w[18 + 2 * ax] : w[12 + 2 * ax];
      fw[ax][1] = pos ? w[19 + 2 * ax] : w[13 + 2 * ax];
    }
    uint32_t hit = 0u;
#pragma unroll
    for (int c = 0; c < kWide; ++c) {
      const uint32_t sel = 0x7540u | (uint32_t)(c & 3);  // byte c of the word, then 0x00, 0x00, 0x4B
      float tn[3], tf[3];
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        const float qn = __uint_as_float(__byte_perm(nw[ax][c >> 2], 0x4B000000u, sel));
        const float qf = __uint_as_float(__byte_perm(fw[ax][c >> 2], 0x4B000000u, sel));
        tn[ax] = fmaf(qn, a[ax], cn[ax]);
        tf[ax] = fmaf(qf, a[ax], cf[ax]);
      }
      if (max3f(tn[0], tn[1], fmaxf(tn[2], 0.0f)) <= min3f(tf[0], tf[1], fminf(tf[2], bt))) hit |= 1u << c;
    }
    const uint32_t lm = w[3] >> 24;
    uint32_t leaves = hit & lm;
    while (leaves) {
      const uint32_t c = (uint32_t)__ffs(leaves) - 1u;
      leaves &= leaves - 1u;
      const uint32_t lf = pick8(w + 4, c);
      if (lf == kNoChild) continue;
      if (!kChecked || leaf_in_range(s, lf)) test_leaf(s, lf, r, tnear, bt, bid, bref);
      else errs += 1;
    }
    uint32_t pm = xor_perm8(hit & ~lm, oct);
    if (pm) {
      const uint32_t first = (uint32_t)__ffs(pm) - 1u;
      pm &= pm - 1u;
      while (pm) {  // the others farthest first, so that the nearest is on top
        const uint32_t i = 31u - (uint32_t)__clz(pm);
        pm ^= 1u << i;
        if (sp < STACK) stack(sp++) = pick8(w + 4, i ^ oct);
        else errs += 1;
      }
      cur = pick8(w + 4, first ^ oct);
    } else {
      if (sp == 0) break;
      cur = stack(--sp);
    }
  }
  return bid != INT_MAX;
}

// Closest primitive hit; returns false when nothing is hit.  errs counts
// stack overflows and iteration-limit trips (both end the query).
// POSTPONE = false: a leaf child whose box the ray enters is tested on the
// spot.  POSTPONE = true (Aila and Laine, HPG 2009, "while-while"): a lane
// keeps one such leaf pending and walks on through inner nodes until every
// lane of the warp holds a pending leaf (or has no inner node left), then the
// warp tests the pending leaves together; the closest hit is the same, only
// the lanes that run the primitive tests together change.
// SST = 0: the stack is a per-thread local array; SST > 0: it is a column of
// shared memory, entry i at sstk[i * SST] (SST = the block size, so the lanes
// of a warp always hit distinct banks).
// WIDE = false: the binary tree only (the wide traversal is not compiled in,
// which keeps the binary kernels' registers); WIDE = true: the wide tree
// whenever the scene view carries one.
template <int STACK, bool POSTPONE, int SST = 0, bool WIDE = true, typename Count = unsigned long long>
__device__ bool closest_hit(const SceneView& s, f3 o, f3 d, float tnear, float& bt, int& bid, uint32_t& bref,
                            Count& errs, uint32_t* sstk = nullptr) {
  Ray r;
  r.o = o;
  r.d = d;
  r.idr = mk3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
  bt = FLT_MAX;
  bid = INT_MAX;
  bref = 0xFFFFFFFFu;
  uint32_t lstack[SST ? 1 : STACK];
  if constexpr (WIDE && !POSTPONE) {
    if (s.wnodes) return closest_hit_wide<STACK, SST>(s, r, tnear, bt, bid, bref, errs, lstack, sstk);
  }
  auto stack = [&](int i) -> uint32_t& { return SST ? sstk[i * SST] : lstack[i]; };
  int sp = 0;
  uint32_t cur = s.root;
  const uint32_t max_iter = s.max_visits;
  if (!POSTPONE) {
    for (uint32_t it = 0;; ++it) {
      if (it >= max_iter) {
        errs += 1;
        break;
      }
      if (kChecked && !node_in_range(s, cur)) {
        errs += 1;
        break;
      }
      float4 a, b, c;
      uint4 ch;
      load_node(s.nodes + cur, a, b, c, ch);
      float tn0, tn1;
      bool h0 = slab(a.x, a.y, b.x, b.y, c.x, c.y, r, bt, tn0);
      bool h1 = slab(a.z, a.w, b.z, b.w, c.z, c.w, r, bt, tn1);
      // The leaf children go through one code path, so the lanes with a leaf
      // at child 0 and those with one at child 1 test together (a warp runs
      // the test once per node step, twice only where a lane has two leaves).
      const bool l0 = h0 && (ch.x & kLeafBit), l1 = h1 && (ch.y & kLeafBit);
      uint32_t lf = l0 ? ch.x : (l1 ? ch.y : kNoLeaf);
      uint32_t lf2 = l0 && l1 ? ch.y : kNoLeaf;
      while (lf != kNoLeaf) {
        if (!kChecked || leaf_in_range(s, lf)) test_leaf(s, lf, r, tnear, bt, bid, bref);
        else errs += 1;
        lf = lf2;
        lf2 = kNoLeaf;
      }
      h0 = h0 && !l0;
      h1 = h1 && !l1;
      if (h0 && h1) {
        uint32_t nearc = tn0 <= tn1 ? ch.x : ch.y;
        uint32_t farc = tn0 <= tn1 ? ch.y : ch.x;
        if (sp < STACK) {
          stack(sp++) = farc;
        } else {
          errs += 1;
        }
        cur = nearc;
      } else if (h0) {
        cur = ch.x;
      } else if (h1) {
        cur = ch.y;
      } else {
        if (sp == 0) break;
        cur = stack(--sp);
      }
    }
    return bid != INT_MAX;
  }
  // while-while: leaves travel through `cur` and the stack like inner nodes
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  uint32_t leaf = kNone;
  uint32_t it = 0;
  auto pop = [&]() -> uint32_t { return sp > 0 ? stack(--sp) : kNone; };
  while (cur != kNone) {
    // inner nodes until every lane of the warp holds a pending leaf
    while (cur != kNone && !(cur & kLeafBit)) {
      if (it++ >= max_iter) {
        errs += 1;
        cur = kNone;
        break;
      }
      if (kChecked && !node_in_range(s, cur)) {
        errs += 1;
        cur = kNone;
        break;
      }
      float4 a, b, c;
      uint4 ch;
      load_node(s.nodes + cur, a, b, c, ch);
      float tn0, tn1;
      const bool h0 = slab(a.x, a.y, b.x, b.y, c.x, c.y, r, bt, tn0);
      const bool h1 = slab(a.z, a.w, b.z, b.w, c.z, c.w, r, bt, tn1);
      if (h0 && h1) {
        const bool first = tn0 <= tn1;
        if (sp < STACK) stack(sp++) = first ? ch.y : ch.x;
        else errs += 1;
        cur = first ? ch.x : ch.y;
      } else if (h0) {
        cur = ch.x;
      } else if (h1) {
        cur = ch.y;
      } else {
        cur = pop();
      }
      if (cur != kNone && (cur & kLeafBit) && leaf == kNone) {
        leaf = cur;
        cur = pop();
      }
      if (!__any_sync(__activemask(), leaf == kNone)) break;
    }
    // the pending leaf, and any leaf reached right after it
    while (leaf != kNone) {
      if (it++ >= max_iter) {
        errs += 1;
        cur = kNone;
        break;
      }
      if (!kChecked || leaf_in_range(s, leaf)) test_leaf(s, leaf, r, tnear, bt, bid, bref);
      else errs += 1;
      leaf = kNone;
      if (cur != kNone && (cur & kLeafBit)) {
        leaf = cur;
        cur = pop();
      }
    }
  }
  return bid != INT_MAX;
}

// hit_accumulator::use (hit_accumulator.hpp:128-138); with fixed_s1 the flux
// is added as an int64 multiple of 2^-32 (order-independent sums)
__device__ __forceinline__ void deposit(const TraceParams& p, int id, float v) {
  const double dv = (double)v;
  if (p.fixed_s1)
    atomicAdd(reinterpret_cast<unsigned long long*>(&p.s1[id]), (unsigned long long)__double2ll_rn(dv * 4294967296.0));
  else
    atomicAdd(&p.s1[id], dv);
  atomicAdd(&p.s2[id], dv * v);
  atomicAdd(&p.s3[id], dv * v * v);
  atomicAdd(&p.s4[id], dv * v * v * v);
  atomicAdd(&p.cnt[id], 1ull);
}

// Does the ray overlap the box within [tlo, thi]?  Padded like slab(), so a
// primitive hit in the interval is never outside an overlapping box.
__device__ __forceinline__ bool overlaps(float lx, float hx, float ly, float hy, float lz, float hz, const Ray& r,
                                         float tlo, float thi) {
  float t0x = (lx - r.o.x) * r.idr.x, t1x = (hx - r.o.x) * r.idr.x;
  float t0y = (ly - r.o.y) * r.idr.y, t1y = (hy - r.o.y) * r.idr.y;
  float t0z = (lz - r.o.z) * r.idr.z, t1z = (hz - r.o.z) * r.idr.z;
  const float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), 0.0f));
  const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z)) * 1.0000005f;
  return tn <= tf && tn <= thi * 1.0000005f + 1e-30f && tf >= tlo;
}

// Calls visit(ref) once for every leaf whose box the ray overlaps within
// [tlo, thi].  errs counts stack overflows and iteration-limit trips.
template <int STACK, typename Visit>
__device__ void leaves_in_interval(const SceneView& s, const Ray& r, float tlo, float thi, uint32_t& errs,
                                   Visit visit) {
  uint32_t stack[STACK];
  int sp = 0;
  uint32_t cur = s.root;
  const uint32_t max_iter = s.max_visits;
  for (uint32_t it = 0;; ++it) {
    if (it >= max_iter) {
      errs += 1;
      return;
    }
    if (kChecked && !node_in_range(s, cur)) {
      errs += 1;
      return;
    }
    float4 a, b, c;
    uint4 ch;
    load_node(s.nodes + cur, a, b, c, ch);
    bool h0 = overlaps(a.x, a.y, b.x, b.y, c.x, c.y, r, tlo, thi);
    // a one-primitive tree holds its leaf in both children of the root
    bool h1 = ch.y != ch.x && overlaps(a.z, a.w, b.z, b.w, c.z, c.w, r, tlo, thi);
    if (h0 && (ch.x & kLeafBit)) {
      visit(ch.x);
      h0 = false;
    }
    if (h1 && (ch.y & kLeafBit)) {
      visit(ch.y);
      h1 = false;
    }
    if (h0 && h1) {
      if (sp < STACK) stack[sp++] = ch.y;
      else errs += 1;
      cur = ch.x;
    } else if (h0) {
      cur = ch.x;
    } else if (h1) {
      cur = ch.y;
    } else {
      if (sp == 0) return;
      cur = stack[--sp];
    }
  }
}

// The multi-hit window of rti's point-cloud context (point_cloud_context.hpp:
// 132-173,265-286), opened by the closest front-face hit at t0 on the disc in
// slot `ref`: it reaches to t0 + window_factor * r0 (r0 that disc's radius),
// cut at the x/y box exit tbox and at the first back-face disc hit or triangle
// hit beyond t0.  Every disc hit from the front within it receives w s_j; the
// return value is w minus the mean of those deposits (float w, double mean,
// as rti).  The sum of the deposits is formed in double; it is exact, hence
// independent of the traversal order, while the deposits of one window lie
// within a factor 2^28 of each other (always for a global sticking).
template <int STACK>
__device__ float window_deposit(const TraceParams& p, f3 o, f3 d, float t0, float tbox, uint32_t ref, float w,
                                uint32_t& c_tot, uint32_t& c_nb, uint32_t& errs) {
  Ray r;
  r.o = o;
  r.d = d;
  r.idr = mk3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
  const float r0 = __ldg(&p.s.disc[2 * (int64_t)(ref & kSlotMask)]).w;
  float te = t0 + p.window_factor * r0;
  if (tbox < te) te = tbox;
  // hit of the leaf primitive in slot lr: t, id, and whether it closes the window
  auto leaf = [&](uint32_t lr, float& t, int& id, bool& closes) -> bool {
    if (kChecked && !leaf_in_range(p.s, lr)) {
      errs += 1;
      return false;
    }
    const uint32_t slot = lr & kSlotMask;
    if (lr & kTriBit) {
      const float4 a = __ldg(&p.s.tri[4 * (int64_t)slot]), b = __ldg(&p.s.tri[4 * (int64_t)slot + 1]);
      const float4 c = __ldg(&p.s.tri[4 * (int64_t)slot + 2]);
      id = __float_as_int(a.w);
      closes = true;
      return tri_test(mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z), r.o, r.d, p.tnear, t);
    }
    const float4 cr = __ldg(&p.s.disc[2 * (int64_t)slot]), nn = __ldg(&p.s.disc[2 * (int64_t)slot + 1]);
    id = __float_as_int(nn.w);
    closes = d.x * nn.x + d.y * nn.y + d.z * nn.z > 0.0f;
    return disc_test(mk3(cr.x, cr.y, cr.z), cr.w, mk3(nn.x, nn.y, nn.z), r.o, r.d, p.tnear, t);
  };
  float tc = te;
  leaves_in_interval<STACK>(p.s, r, t0, te, errs, [&](uint32_t lr) {
    float t;
    int id;
    bool closes;
    if (leaf(lr, t, id, closes) && closes && t > t0 && t < tc) tc = t;
  });
  double sum = 0.0;
  unsigned long long n = 0;
  leaves_in_interval<STACK>(p.s, r, t0, tc, errs, [&](uint32_t lr) {
    if (lr & kTriBit) return;
    float t;
    int id;
    bool closes;
    if (leaf(lr, t, id, closes) && !closes && t >= t0 && t <= tc) {
      const float st = p.s.sticking_field ? __ldg(&p.s.sticking_field[id]) : p.sticking;
      const float v = w * st;
      deposit(p, id, v);
      sum += (double)v;
      n += 1;
    }
  });
  c_tot += (uint32_t)n;
  c_nb += n > 0 ? (uint32_t)(n - 1) : 0u;
  return n > 0 ? (float)((double)w - sum / (double)n) : w;
}

// Side-face exit of the x/y box: 0 = x face, 1 = y face, -1 = the ray leaves
// through the top or bottom first (a miss).
__device__ __forceinline__ int boundary_exit(const TraceParams& p, f3 o, f3 d, float& tb) {
  float tx = FLT_MAX, ty = FLT_MAX, tz = FLT_MAX;
  if (d.x > 0.0f) tx = (p.box_hi[0] - o.x) / d.x;
  else if (d.x < 0.0f) tx = (p.box_lo[0] - o.x) / d.x;
  if (d.y > 0.0f) ty = (p.box_hi[1] - o.y) / d.y;
  else if (d.y < 0.0f) ty = (p.box_lo[1] - o.y) / d.y;
  if (d.z > 0.0f) tz = (p.box_hi[2] - o.z) / d.z;
  else if (d.z < 0.0f) tz = (p.box_lo[2] - o.z) / d.z;
  const int axis = tx <= ty ? 0 : 1;
  const float t = tx <= ty ? tx : ty;
  if (!(t < FLT_MAX)) return -1;
  if (!(t >= p.tnear)) return -1;
  if (t > tz) return -1;
  tb = t;
  return axis;
}

// One record of the segment log (rtg_set_segment_log) for a logged ray: the
// query from o along d that ended at distance t.  A full log counts the
// record without keeping it.
__device__ __noinline__ void log_segment(const SegmentLog& lg, uint64_t id, uint32_t seg, int kind, f3 o, f3 d,
                                         float t, int prim, float w) {
  if (id < lg.ray_begin || id >= lg.ray_end) return;
  const unsigned long long i = atomicAdd(lg.count, 1ull);
  if (i >= lg.cap) return;
  rtg_segment r;
  r.ray = id;
  r.segment = seg;
  r.kind = kind;
  r.org[0] = o.x;
  r.org[1] = o.y;
  r.org[2] = o.z;
  r.end[0] = o.x + d.x * t;  // as the path computes its next origin
  r.end[1] = o.y + d.y * t;
  r.end[2] = o.z + d.z * t;
  r.primitive = prim;
  r.weight = w;
  lg.rec[i] = r;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
  return v;
}

// kModeForward traces and deposits.  The adjoint modes replay the same paths
// and accumulate derivatives of L = sum_i g_i S1_i instead.  G_k = the sum of g
// over the primitives that received deposit k, v_k = w_k s its weight,
// P_k = sum_{m<=k} G_m v_m.
//   held (adj_unbiased = 0): the roulette decisions are held as drawn (what
//     central differences with common random numbers measure).  Within a
//     stretch between roulette resets the weight is a product of (1 - s_e)
//     factors, so dL/ds_j = sum over deposits k on j of G_k w_k - (T - P_k) /
//     (1 - s_j), T the stretch total.  One global s: dv_k/ds = w_k + s w'_k,
//     w'_{k+1} = w'_k - dv_k/ds, w' = 0 after a reset.
//   unbiased (adj_unbiased = 1): adds the likelihood ratio of each roulette
//     survival (probability w/0.3); T becomes the path total L_p.  One global
//     s: dL/ds = sum_k G_k w_k - (K L_p - sum_k P_k)/(1 - s) over K deposits.
//   kModeAdjField splits each deposit's term as G_k w_k + P_k/(1 - s_j) (known
//     at the deposit, scattered at once) minus T/(1 - s_j) (T known at the end
//     of the stretch -- the whole path for the unbiased estimator).  The
//     deferred part is scattered from a small per-lane list of the stretch's
//     (element, sticking) pairs; a stretch with more deposits than the list
//     holds is traced again from a snapshot of its start to scatter them, so
//     no per-path memory is kept.
//   Both: dL/dn = sum over paths of (1/(n+1) + ln cos theta_0) * L_p (score
//     function of the cos^n source).
// Batched = true: lanes take global ray ids over the concatenated ray ranges
// of `njobs` jobs (prefix[j] = first global id of job j) and trace each with
// its job's parameters (scene, configuration, accumulators); the counters and
// the abort flag are the batch's (p0).  TPB threads per block and 1024 / TPB
// resident blocks per SM as the register target (64 registers per thread);
// forward traces with 128 threads target 9 blocks (56 registers, a few spilled:
// the extra warps hide more latency than the spills cost).
// SHSTACK = true: the traversal stacks of the block live in shared memory
// (STACK x TPB entries, at most 16 KB).  WIDE = true: closest hits over the
// wide tree where a scene view carries one (see closest_hit).
template <int M, bool Batched, int TPB, int STACK, bool POSTPONE = false, bool SHSTACK = false, bool WIDE = false>
__global__ void __launch_bounds__(TPB, (M == kModeForward && TPB == 128 ? 1152 : 1024) / TPB)
    trace_paths_kernel(const __grid_constant__ TraceParams p0, const TraceParams* __restrict__ jobs,
                       const uint64_t* __restrict__ prefix, int njobs) {
  constexpr bool kAdj = M == kModeAdjGlobal || M == kModeAdjField;
  constexpr bool kLog = M == kModeLogged;  // a forward trace that also fills p0.log
  static_assert(!SHSTACK || STACK * TPB * 4 <= 16384, "a shared stack of at most 16 KB per block");
  constexpr int kSst = SHSTACK ? TPB : 0;
  uint32_t* sstk = nullptr;
  if constexpr (SHSTACK) {
    __shared__ uint32_t sstack[STACK * TPB];
    sstk = sstack + threadIdx.x;
  }
  const TraceParams* pp = &p0;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  // per-lane counters, summed over the warp at the end (32 bits: a lane traces
  // far fewer than 2^32 segments)
  uint32_t c_hit = 0, c_non = 0, c_tot = 0, c_seg = 0, c_nb = 0, c_err = 0;
  bool active = false, exhausted = false;
  uint64_t id = 0;
  f3 o = mk3(0, 0, 0), d = mk3(0, 0, 0);
  float w = 1.0f;
  uint32_t k = 0, nseg = 0;
  const uint64_t nrays = Batched ? prefix[njobs] : p0.ray_end - p0.ray_begin;
  // adjoint state
  double wd = 0.0, lp = 0.0, score = 0.0, acc_s = 0.0, acc_n = 0.0, seg_t = 0.0;
  double pa = 0.0, psum = 0.0, ncoll = 0.0;
  const bool unbiased = p0.adj_unbiased != 0;
  int sub = 0;
  f3 so = o, sd = d;
  float sw = 1.0f;
  uint32_t sk = 0, snseg = 0;
  constexpr int kAdjList = 32;  // deposits of a stretch whose deferred term is kept per lane
  uint32_t alist_id[M == kModeAdjField ? kAdjList : 1];
  float alist_s[M == kModeAdjField ? kAdjList : 1];
  int alist_n = 0;
  auto snapshot = [&]() {
    so = o; sd = d; sw = w; sk = k; snseg = nseg;
    seg_t = 0.0; sub = 0; alist_n = 0;
  };
  // the deferred terms -T/(1 - s_j) of a stretch whose deposits all fit the list
  auto flush = [&]() {
    for (int i = 0; i < alist_n; ++i)
      if (alist_s[i] < 1.0f) atomicAdd(&pp->adj_field[alist_id[i]], -seg_t / (1.0 - (double)alist_s[i]));
  };
  // end of a path; in the field replay a stretch too long for the list is
  // traced again to scatter its deferred terms
  auto path_end = [&]() -> bool {
    if (M == kModeAdjField && sub == 0) {
      if (alist_n <= kAdjList) {
        flush();
      } else {
        o = so; d = sd; w = sw; k = sk; nseg = snseg;
        sub = 1;
        return true;
      }
    }
    if (M == kModeAdjGlobal && unbiased) {
      double ds = pa;
      if (pp->sticking < 1.0f) ds -= (ncoll * lp - psum) / (1.0 - (double)pp->sticking);
      acc_s += ds;
    }
    if (kAdj) acc_n += score * lp;
    return false;
  };
  for (uint32_t iter = 0;; ++iter) {
    if (!exhausted) {
      const unsigned need = __ballot_sync(kFull, !active);
      if (need && __popc(need) >= p0.packet) {
        const int leader = __ffs(need) - 1;
        unsigned long long base = 0;
        if (p0.plain) {  // one source ray per thread (all lanes are idle on the first pass)
          base = (unsigned long long)blockIdx.x * TPB + (threadIdx.x & ~31u);
          exhausted = true;
        } else {
          if (lane == leader) base = atomicAdd(&p0.tally->next_ray, (unsigned long long)__popc(need));
          base = __shfl_sync(kFull, base, leader);
          if (base + __popc(need) >= nrays) exhausted = true;
        }
        if (!active) {
          const uint64_t j = base + (uint64_t)__popc(need & lt_mask);
          if (j < nrays) {
            if (Batched) {
              int lo = 0, hi = njobs - 1;  // last job whose first id <= j
              while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(&prefix[mid]) <= j) lo = mid;
                else hi = mid - 1;
              }
              pp = jobs + lo;
              id = pp->ray_begin + (j - __ldg(&prefix[lo]));
            } else {
              id = p0.ray_begin + j;
            }
            // source.hpp:20-58 with rectangle_origin_z / (power_)cosine_direction_z
            const uint4 u = draw4(pp->seed, id, 0xFFFFFFFFu, pp->job);
            const float r1 = u01_co(u.x), r2 = u01_co(u.y);
            o = mk3(pp->src_lo[0] + (pp->src_hi[0] - pp->src_lo[0]) * r1,
                    pp->src_lo[1] + (pp->src_hi[1] - pp->src_lo[1]) * r2, pp->box_hi[2]);
            d = source_dir(pp->source_exponent, pp->source_ee, u.z, u.w);
            w = 1.0f;
            k = 0;
            nseg = 0;
            active = true;
            if (kAdj) {
              score = pp->adj_inv_n1 + log(-(double)d.z);
              lp = 0.0;
              wd = 0.0;
              pa = 0.0;
              psum = 0.0;
              ncoll = 0.0;
              if (M == kModeAdjField) snapshot();
            }
          }
        }
      }
    }
    if (!__any_sync(kFull, active)) break;
    if ((iter & 255u) == 0u && p0.abort_flag) {
      unsigned stop = 0;
      if (lane == 0) stop = *p0.abort_flag;
      stop = __shfl_sync(kFull, stop, 0);
      if (stop) {
        if (lane == 0) atomicExch(&p0.tally->abort_seen, 1u);
        break;
      }
    }
    if (!active) continue;
    // ---- one segment (tracer.hpp:169-279) ----
    if (nseg == pp->max_segments) {
      atomicAdd(&p0.tally->truncated, 1ull);  // rare: no per-lane counter
      active = path_end();
      continue;
    }
    nseg += 1;
    c_seg += 1;
    float th, tb = 0.0f;
    int hid;
    uint32_t href;
    const bool hit = closest_hit<STACK, POSTPONE, kSst, WIDE>(pp->s, o, d, pp->tnear, th, hid, href, c_err, sstk);
    const int axis = boundary_exit(*pp, o, d, tb);
    if (kChecked && hit && (unsigned)hid >= (unsigned)(pp->s.nd + pp->s.nt)) {
      c_err += 1;
      active = path_end();
      continue;
    }
    if (hit && (axis < 0 || th <= tb)) {
      float4 nn;
      if (href & kTriBit) nn = __ldg(&pp->s.tri[4 * (int64_t)(href & kSlotMask) + 3]);
      else nn = __ldg(&pp->s.disc[2 * (int64_t)(href & kSlotMask) + 1]);
      const f3 n = mk3(nn.x, nn.y, nn.z);
      const f3 hp = mk3(o.x + d.x * th, o.y + d.y * th, o.z + d.z * th);
      if (d.x * n.x + d.y * n.y + d.z * n.z > 0.0f) {  // back face: pass through (tracer.hpp:216-227)
        if (kLog) log_segment(p0.log, id, nseg - 1, RTG_SEG_BACKFACE, o, d, th, hid, w);
        o = hp;
        continue;
      }
      if (kLog) log_segment(p0.log, id, nseg - 1, RTG_SEG_HIT, o, d, th, hid, w);
      c_hit += 1;
      const float st = pp->s.sticking_field ? __ldg(&pp->s.sticking_field[hid]) : pp->sticking;
      const float v = w * st;
      double G = 0.0;
      float w_win = 0.0f;
      if (M == kModeWindow && !(href & kTriBit)) {
        w_win = window_deposit<STACK>(*pp, o, d, th, axis >= 0 ? tb : FLT_MAX, href, w, c_tot, c_nb, c_err);
      } else {
        if (kAdj) G = __ldg(&pp->adj_g[hid]);
        else deposit(*pp, hid, v);
        if (M == kModeWindow) c_tot += 1;  // elsewhere total = hits + neighbour deposits
      }
      if (M != kModeWindow && !(href & kTriBit) && pp->s.nb_ptr) {  // tracer.hpp:339-383
        const int64_t q0 = __ldg(&pp->s.nb_ptr[hid]), q1 = __ldg(&pp->s.nb_ptr[hid + 1]);
        for (int64_t q = q0; q < q1; ++q) {
          const uint32_t ns = __ldg(&pp->s.nb_slot[q]);
          if (kChecked && ns >= (uint32_t)pp->s.nd) {
            c_err += 1;
            continue;
          }
          float4 cr, nv;  // the neighbour's slot record: (centre, radius), (normal, id bits)
          asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
              : "=f"(cr.x), "=f"(cr.y), "=f"(cr.z), "=f"(cr.w), "=f"(nv.x), "=f"(nv.y), "=f"(nv.z), "=f"(nv.w)
              : "l"(pp->s.disc + 2 * (int64_t)ns));
          const int nb = __float_as_int(nv.w);
          if (kChecked && (unsigned)nb >= (unsigned)pp->s.nd) {
            c_err += 1;
            continue;
          }
          if (local_intersect(o, d, mk3(cr.x, cr.y, cr.z), cr.w, mk3(nv.x, nv.y, nv.z))) {
            if (kAdj) G += __ldg(&pp->adj_g[nb]);
            else deposit(*pp, nb, v);
            c_nb += 1;
          }
        }
      }
      if (M == kModeAdjGlobal) {
        lp += G * (double)v;
        if (unbiased) {
          pa += G * (double)w;
          psum += lp;
          ncoll += 1.0;
        } else {
          const double dv = (double)w + (double)st * wd;
          acc_s += G * dv;
          wd -= dv;
        }
      } else if (M == kModeAdjField) {
        const double gv = G * (double)v;
        if (sub == 0) {
          seg_t += gv;  // P_k
          lp += gv;
          double a = G * (double)w;
          if (st < 1.0f) a += seg_t / (1.0 - (double)st);
          atomicAdd(&pp->adj_field[hid], a);
          if (alist_n < kAdjList) {
            alist_id[alist_n] = (uint32_t)hid;
            alist_s[alist_n] = st;
          }
          alist_n += 1;
        } else if (st < 1.0f) {  // replay of a long stretch: seg_t holds its total T
          atomicAdd(&pp->adj_field[hid], -seg_t / (1.0 - (double)st));
        }
      }
      if (M == kModeWindow && !(href & kTriBit)) w = w_win;
      else w = w - v;
      if (w == 0.0f) {
        active = path_end();
        continue;
      }
      const uint4 u = draw4(pp->seed, id, k, pp->job);
      // rejection_control::check_weight_reweight_or_kill (rejection_control.hpp:28-61)
      bool reset = false;
      const double lower = pp->roulette_threshold * 1.0f;
      const double renew = pp->roulette_weight * 1.0f;
      if (!((double)w >= lower)) {
        const double kill = 1.0f - (double)w / renew;
        if ((double)u.x < kill * 4294967296.0) {
          active = path_end();
          continue;
        }
        w = (float)renew;
        reset = true;
        if (M == kModeAdjGlobal) wd = 0.0;
      }
      const bool spec = pp->reflection == RTG_REFLECT_SPECULAR ||
                        (pp->reflection == RTG_REFLECT_MIXED &&
                         (double)u.w < (double)pp->specular_fraction * 4294967296.0);
      d = spec ? specular_dir(n, d) : diffuse_dir(n, u.y, u.z);
      o = hp;
      k += 1;
      if (M == kModeAdjField && reset && !unbiased) {
        if (sub == 0 && alist_n > kAdjList) {  // the stretch is complete: trace it again to scatter
          o = so; d = sd; w = sw; k = sk; nseg = snseg;
          sub = 1;
        } else {
          if (sub == 0) flush();
          snapshot();  // the next stretch starts after this re-emission
        }
      }
      continue;
    }
    if (axis >= 0) {  // boundary_x_y::process_hit (boundary_x_y.hpp:92-143)
      if (kLog) log_segment(p0.log, id, nseg - 1, RTG_SEG_BOUNDARY, o, d, tb, -1, w);
      f3 hp = mk3(o.x + d.x * tb, o.y + d.y * tb, o.z + d.z * tb);
      const int periodic = axis == 0 ? pp->x_periodic : pp->y_periodic;
      if (periodic) {
        if (axis == 0) hp.x = d.x > 0.0f ? pp->box_lo[0] : pp->box_hi[0];
        else hp.y = d.y > 0.0f ? pp->box_lo[1] : pp->box_hi[1];
      } else {
        if (axis == 0) d.x = -d.x;
        else d.y = -d.y;
      }
      o = hp;
      continue;
    }
    if (kLog) {  // out through the top or bottom plane
      const float tz = d.z > 0.0f ? (pp->box_hi[2] - o.z) / d.z : (d.z < 0.0f ? (pp->box_lo[2] - o.z) / d.z : 0.0f);
      log_segment(p0.log, id, nseg - 1, RTG_SEG_ESCAPE, o, d, tz, -1, w);
    }
    c_non += 1;
    active = path_end();
  }
  if (kAdj) {
    acc_s = warp_sum_d(acc_s);
    acc_n = warp_sum_d(acc_n);
    if (lane == 0) {
      atomicAdd(&pp->adj_scalars[0], acc_s);
      atomicAdd(&pp->adj_scalars[1], acc_n);
    }
  }
  const unsigned long long s_hit = warp_sum(c_hit), s_non = warp_sum(c_non);
  const unsigned long long s_seg = warp_sum(c_seg), s_nb = warp_sum(c_nb);
  const unsigned long long s_tot = M == kModeWindow ? warp_sum(c_tot) : s_hit + s_nb;
  const unsigned long long s_err = warp_sum(c_err);
  if (lane == 0) {
    atomicAdd(&p0.tally->hitc, s_hit);
    atomicAdd(&p0.tally->nonhitc, s_non);
    atomicAdd(&p0.tally->total, s_tot);
    atomicAdd(&p0.tally->segments, s_seg);
    atomicAdd(&p0.tally->nb_deposits, s_nb);
    atomicAdd(&p0.tally->errors, s_err);
  }
}

using PathKernel = void (*)(const TraceParams, const TraceParams*, const uint64_t*, int);

// The instantiation of trace_paths_kernel with its stack in shared memory
// when `shared` asks for it and it fits 16 KB per block (8 blocks then leave
// half of the SM's L1/shared capacity to L1), else in local memory; with the
// wide traversal compiled in when `wide` (postponed leaf tests use the binary
// tree only).
template <int M, bool Batched, int TPB, int STACK, bool POSTPONE, bool WIDE>
PathKernel kernel_for_width(bool shared) {
  if constexpr (STACK * TPB * 4 <= 16384) {
    if (shared) return trace_paths_kernel<M, Batched, TPB, STACK, POSTPONE, true, WIDE>;
  }
  return trace_paths_kernel<M, Batched, TPB, STACK, POSTPONE, false, WIDE>;
}

template <int M, bool Batched, int TPB, int STACK, bool POSTPONE>
PathKernel kernel_for(bool shared, bool wide) {
  if constexpr (!POSTPONE) {
    if (wide) return kernel_for_width<M, Batched, TPB, STACK, false, true>(shared);
  }
  return kernel_for_width<M, Batched, TPB, STACK, POSTPONE, false>(shared);
}

}  // namespace
}  // namespace rtg
