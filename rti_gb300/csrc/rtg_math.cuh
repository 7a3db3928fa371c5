// rtg_math.cuh -- device arithmetic of the flux path.
//
// Every float operation on a ray path is one IEEE-754 binary32 operation in
// source order: the library is compiled with -fmad=false, so a*b+c is a
// rounded multiply followed by a rounded add, and fused multiply-adds appear
// only where written as fmaf().  Division and sqrtf are the IEEE-rounded
// forms (nvcc's default -prec-div/-prec-sqrt).  sin/cos of 2*pi*u and x^e
// are this project's own polynomials (Taylor / atanh series, Horner with
// fmaf), so that a path traced here is bit-identical to the same path traced
// by the CPU restatement of the reference.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rtg {

struct f3 {
  float x, y, z;
};

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
// util::normalize (utils.hpp:86-93)
__device__ __forceinline__ f3 normalize3(f3 v) {
  float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
  return mk3(v.x / l, v.y / l, v.z / l);
}
// util::distance / length_of_vec (utils.hpp:141-159)
__device__ __forceinline__ float len3(f3 v) {
  float d1 = v.x - 0.0f, d2 = v.y - 0.0f, d3 = v.z - 0.0f;
  return sqrtf(d1 * d1 + d2 * d2 + d3 * d3);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// Counter = (ray id lo, ray id hi, event, job), key = (seed lo, seed hi).
// event 0xFFFFFFFF draws the source ray; event k draws collision k.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ uint4 draw4(uint64_t seed, uint64_t id, uint32_t event, uint32_t job) {
  return philox4x32_10(make_uint4((uint32_t)id, (uint32_t)(id >> 32), event, job), (uint32_t)seed,
                       (uint32_t)(seed >> 32));
}

// uniform in [0,1) and (0,1] from the top 24 bits
__device__ __forceinline__ float u01_co(uint32_t x) { return (float)(x >> 8) * 0x1p-24f; }
__device__ __forceinline__ float u01_oc(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1p-24f; }

// ---------------------------------------------------------------------------
// sin/cos of 2*pi*u, u in [0,1]: exact quadrant reduction on u, Taylor
// polynomials on [0, pi/4].
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sincos_quarter(float th, float& s, float& c) {
  float z = th * th;
  float ps = fmaf(z, -2.50521084e-08f, 2.75573192e-06f);  // -1/11!, 1/9!
  ps = fmaf(z, ps, -1.98412698e-04f);                     // -1/7!
  ps = fmaf(z, ps, 8.33333333e-03f);                      //  1/5!
  ps = fmaf(z, ps, -1.66666667e-01f);                     // -1/3!
  s = fmaf(th * z, ps, th);
  float pc = fmaf(z, -2.75573192e-07f, 2.48015873e-05f);  // -1/10!, 1/8!
  pc = fmaf(z, pc, -1.38888889e-03f);                     // -1/6!
  pc = fmaf(z, pc, 4.16666667e-02f);                      //  1/4!
  pc = fmaf(z, pc, -0.5f);                                // -1/2!
  c = fmaf(z, pc, 1.0f);
}

__device__ __forceinline__ void sincos2pi(float u, float& s, float& c) {
  float x = u * 4.0f;
  float qf = floorf(x);
  float f = x - qf;
  int q = ((int)qf) & 3;
  float ss, cc;
  if (f <= 0.5f) {
    sincos_quarter(f * 1.57079633f, ss, cc);
  } else {
    float sc, cs;
    sincos_quarter((1.0f - f) * 1.57079633f, sc, cs);
    ss = cs;
    cc = sc;
  }
  switch (q) {
    case 0: s = ss; c = cc; break;
    case 1: s = cc; c = -ss; break;
    case 2: s = -ss; c = -cc; break;
    default: s = -cc; c = ss; break;
  }
}

// x^e for x in (0,1], e > 0 as exp2(e * log2 x)
__device__ __forceinline__ float own_log2(float x) {
  uint32_t b = __float_as_uint(x);
  int k;
  if ((b >> 23) == 0) {
    x = x * 4294967296.0f;
    b = __float_as_uint(x);
    k = (int)(b >> 23) - 127 - 32;
  } else {
    k = (int)(b >> 23) - 127;
  }
  float m = __uint_as_float((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    k += 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float z = s * s;
  float p = fmaf(z, 0.0909090909f, 0.111111111f);
  p = fmaf(z, p, 0.142857143f);
  p = fmaf(z, p, 0.2f);
  p = fmaf(z, p, 0.333333333f);
  float ln_m = 2.0f * fmaf(s * z, p, s);
  return fmaf(ln_m, 1.44269504f, (float)k);
}

__device__ __forceinline__ float own_exp2(float y) {
  if (y < -149.0f) return 0.0f;
  float nf = floorf(y + 0.5f);
  float f = y - nf;
  float z = f * 0.693147181f;
  float p = fmaf(z, 2.48015873e-05f, 1.98412698e-04f);
  p = fmaf(z, p, 1.38888889e-03f);
  p = fmaf(z, p, 8.33333333e-03f);
  p = fmaf(z, p, 4.16666667e-02f);
  p = fmaf(z, p, 1.66666667e-01f);
  p = fmaf(z, p, 0.5f);
  p = fmaf(z, p, 1.0f);
  p = fmaf(z, p, 1.0f);
  int n = (int)nf;
  if (n < -126) {
    p = p * 0x1p-64f;
    n += 64;
  }
  if (n > 127) n = 127;
  return p * __uint_as_float((uint32_t)(n + 127) << 23);
}

__device__ __forceinline__ float own_powf(float x, float e) {
  if (x <= 0.0f) return 0.0f;
  if (x == 1.0f) return 1.0f;
  return own_exp2(e * own_log2(x));
}

// ---------------------------------------------------------------------------
// Source (source.hpp:20-58, rectangle_origin_z.hpp:23-37,
// cosine_direction_z.hpp:13-27, power_cosine_direction_z.hpp:13-32)
// ---------------------------------------------------------------------------
__device__ __forceinline__ f3 source_dir(float expo, float ee, uint32_t u_phi, uint32_t u_t) {
  float rt = u01_oc(u_t);
  float t = (expo == 1.0f) ? rt : own_powf(rt, ee);
  float zz = -sqrtf(t);
  float sq = sqrtf(1.0f - t);
  float sn, cs;
  sincos2pi(u01_co(u_phi), sn, cs);
  return normalize3(mk3(cs * sq, sn * sq, zz));
}

// util::get_orthonormal_basis (utils.hpp:207-244) + cos_hemi::get (cos_hemi.hpp:11-45)
__device__ __forceinline__ f3 diffuse_dir(f3 n, uint32_t u_phi, uint32_t u_t) {
  f3 c0 = mk3(n.z, n.z, -(n.x + n.y));
  f3 c1 = mk3(n.y, -(n.x + n.z), n.y);
  f3 c2 = mk3(-(n.y + n.z), n.x, n.x);
  f3 b1 = c0;
  float best = c0.x + c0.y + c0.z;
  if (c1.x + c1.y + c1.z > best) {
    b1 = c1;
    best = c1.x + c1.y + c1.z;
  }
  if (c2.x + c2.y + c2.z > best) b1 = c2;
  f3 b2 = cross3(n, b1);
  f3 b0 = normalize3(n);
  b1 = normalize3(b1);
  b2 = normalize3(b2);
  float r2 = u01_oc(u_t);
  float cc1 = sqrtf(r2);
  float sq = sqrtf(1.0f - r2);
  float sn, cs;
  sincos2pi(u01_co(u_phi), sn, cs);
  float cc2 = cs * sq, cc3 = sn * sq;
  return mk3(b0.x * cc1 + b1.x * cc2 + b2.x * cc3, b0.y * cc1 + b1.y * cc2 + b2.y * cc3,
             b0.z * cc1 + b1.z * cc2 + b2.z * cc3);
}

// specular::use (specular.hpp:66-90): d' = n * (2 n.(-d)) + d
__device__ __forceinline__ f3 specular_dir(f3 n, f3 d) {
  float k = 2.0f * (n.x * (-d.x) + n.y * (-d.y) + n.z * (-d.z));
  return mk3(n.x * k + d.x, n.y * k + d.y, n.z * k + d.z);
}

// ---------------------------------------------------------------------------
// Primitive tests
// ---------------------------------------------------------------------------
// Oriented disc, both faces; accepted when t > tnear and the plane point lies
// within the radius.
__device__ __forceinline__ bool disc_test(f3 c, float r, f3 n, f3 o, f3 d, float tnear, float& tout) {
  float dn = d.x * n.x + d.y * n.y + d.z * n.z;
  if (dn == 0.0f) return false;
  float num = (c.x - o.x) * n.x + (c.y - o.y) * n.y + (c.z - o.z) * n.z;
  float t = num / dn;
  if (!(t > tnear)) return false;
  float qx = (o.x - c.x) + d.x * t;
  float qy = (o.y - c.y) + d.y * t;
  float qz = (o.z - c.z) + d.z * t;
  float q2 = qx * qx + qy * qy + qz * qz;
  if (!(q2 <= r * r)) return false;
  tout = t;
  return true;
}

// Moller-Trumbore, both faces, closed edges.
__device__ __forceinline__ bool tri_test(f3 v0, f3 e1, f3 e2, f3 o, f3 d, float tnear, float& tout) {
  f3 p = cross3(d, e2);
  float det = dot3(e1, p);
  if (det == 0.0f) return false;
  float inv = 1.0f / det;
  f3 sv = sub3(o, v0);
  float u = dot3(sv, p) * inv;
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  f3 q = cross3(sv, e1);
  float v = dot3(d, q) * inv;
  if (!(v >= 0.0f && u + v <= 1.0f)) return false;
  float t = dot3(e2, q) * inv;
  if (!(t > tnear)) return false;
  tout = t;
  return true;
}

// local_intersector::intersect (local_intersector.hpp:41-97), front faces only
__device__ __forceinline__ bool local_intersect(f3 o, f3 d, f3 c, float r, f3 n) {
  float prod = n.x * d.x + n.y * d.y + n.z * d.z;
  if (prod > 0.0f) return false;
  if (fabsf(prod) < 1e-9f) return false;
  float ddneg = c.x * n.x + c.y * n.y + c.z * n.z;
  float ttnom = (-(n.x * o.x + n.y * o.y + n.z * o.z)) + ddneg;
  float tt = ttnom / prod;
  if (tt <= 0.0f) return false;
  f3 hp = mk3(o.x + d.x * tt, o.y + d.y * tt, o.z + d.z * tt);
  f3 v = mk3(hp.x + (-c.x), hp.y + (-c.y), hp.z + (-c.z));
  return r > len3(v);
}

}  // namespace rtg
