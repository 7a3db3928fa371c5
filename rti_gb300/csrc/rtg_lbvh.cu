// rtg_lbvh.cu -- GPU LBVH over oriented discs and triangles.
//
// Replaces the Embree scene build of the reference (tracer.hpp:75-100,
// point_cloud_disc_geometry.hpp:178-222, triangle_geometry.hpp:56-99):
//   1. padded primitive boxes and centroid bounds,
//   2. 30-bit Morton codes of the centroids,
//   3. stable radix sort (rtg_sort.cu),
//   4. Karras (HPG 2012) binary radix tree over the keys (morton << 32 | rank),
//   5. primitives copied to slot order (LBVH leaf order) for coherent access,
//   6. bottom-up box refit with per-node arrival counters.
// rtg_update_* reruns 1, 5 and 6 only (moved surface, same topology).
// Step 4 is by default replaced by PLOC clustering over the same sorted
// leaves (build_ploc), whose trees need fewer node visits per query.
//
// Leaves hold one primitive; each internal node stores the boxes of both
// children (64 bytes), so one node fetch decides both children.
#include <cfloat>
#include <cstdint>
#include <vector>

#include "rtg_internal.cuh"
#include "rtg_math.cuh"

namespace rtg {

namespace {

__device__ __forceinline__ uint32_t fenc(float f) {
  uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fdec(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Conservative boxes: the exact extent of the disc (r*sqrt(1-n_i^2)) or of the
// triangle, padded so that every hit the primitive test accepts lies inside.
__global__ void prim_bounds_kernel(const float4* __restrict__ dcr, const float4* __restrict__ dn, int64_t nd,
                                   const float4* __restrict__ tv, const uint32_t* __restrict__ tidx,
                                   int64_t nt, float* __restrict__ plo, float* __restrict__ phi,
                                   uint32_t* __restrict__ cbounds) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nd + nt) return;
  float lo[3], hi[3];
  if (p < nd) {
    float4 c = dcr[p], n = dn[p];
    float cc[3] = {c.x, c.y, c.z}, nn[3] = {n.x, n.y, n.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float e = 1.0f - nn[a] * nn[a];
      float ext = c.w * sqrtf(e > 0.0f ? e : 0.0f);
      float pad = 1e-5f * (fabsf(cc[a]) + c.w) + 1e-4f * c.w;
      lo[a] = cc[a] - ext - pad;
      hi[a] = cc[a] + ext + pad;
    }
  } else {
    int64_t t = p - nd;
    float4 v0 = tv[tidx[3 * t]], v1 = tv[tidx[3 * t + 1]], v2 = tv[tidx[3 * t + 2]];
    float a0[3] = {v0.x, v0.y, v0.z}, a1[3] = {v1.x, v1.y, v1.z}, a2[3] = {v2.x, v2.y, v2.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float l = fminf(a0[a], fminf(a1[a], a2[a])), h = fmaxf(a0[a], fmaxf(a1[a], a2[a]));
      float pad = 1e-5f * (fabsf(l) + fabsf(h)) + 1e-6f * (h - l) + 1e-7f;
      lo[a] = l - pad;
      hi[a] = h + pad;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    plo[3 * p + a] = lo[a];
    phi[3 * p + a] = hi[a];
    float c = 0.5f * (lo[a] + hi[a]);
    if (cbounds) {
      atomicMin(&cbounds[a], fenc(c));
      atomicMax(&cbounds[3 + a], fenc(c));
    }
  }
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void morton_kernel(const float* __restrict__ plo, const float* __restrict__ phi, int64_t np,
                              const uint32_t* __restrict__ cbounds, uint32_t* __restrict__ keys,
                              uint32_t* __restrict__ vals) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  uint32_t q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float mn = fdec(cbounds[a]), mx = fdec(cbounds[3 + a]);
    float c = 0.5f * (plo[3 * p + a] + phi[3 * p + a]);
    float ext = mx - mn;
    float u = ext > 0.0f ? (c - mn) / ext : 0.0f;
    float s = fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);
    q[a] = (uint32_t)s;
  }
  keys[p] = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
  vals[p] = (uint32_t)p;
}

// is-disc flag per sorted position (scanned into disc slots)
__global__ void disc_flag_kernel(const uint32_t* __restrict__ sorted_prim, int64_t np, int64_t nd,
                                 uint32_t* __restrict__ flag) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  flag[i] = sorted_prim[i] < (uint32_t)nd ? 1u : 0u;
}

// Leaf references and slot-ordered primitive data.
__global__ void slots_kernel(const uint32_t* __restrict__ sorted_prim, const uint32_t* __restrict__ disc_rank,
                             int64_t np, int64_t nd, const float4* __restrict__ dcr_id,
                             const float4* __restrict__ dn_id, const float4* __restrict__ tv,
                             const uint32_t* __restrict__ tidx, float4* __restrict__ disc,
                             uint32_t* __restrict__ disc_slot, float4* __restrict__ tri,
                             uint32_t* __restrict__ leaf_ref, int32_t* __restrict__ leaf_prim) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  uint32_t p = sorted_prim[i];
  uint32_t ds = disc_rank[i];
  leaf_prim[i] = (int32_t)p;
  if (p < (uint32_t)nd) {
    float4 n = dn_id[p];
    disc[2 * (int64_t)ds] = dcr_id[p];
    disc_slot[p] = ds;
    disc[2 * (int64_t)ds + 1] = make_float4(n.x, n.y, n.z, __int_as_float((int)p));
    leaf_ref[i] = kLeafBit | ds;
  } else {
    uint32_t ts = (uint32_t)i - ds;
    int64_t t = (int64_t)p - nd;
    float4 a = tv[tidx[3 * t]], b = tv[tidx[3 * t + 1]], c = tv[tidx[3 * t + 2]];
    f3 v0 = mk3(a.x, a.y, a.z);
    f3 e1 = sub3(mk3(b.x, b.y, b.z), v0);
    f3 e2 = sub3(mk3(c.x, c.y, c.z), v0);
    // util::compute_normal + normalize (i_triangle_reader.hpp:22-38)
    f3 n = normalize3(cross3(e1, e2));
    tri[4 * (int64_t)ts] = make_float4(v0.x, v0.y, v0.z, __int_as_float((int)p));
    tri[4 * (int64_t)ts + 1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
    tri[4 * (int64_t)ts + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
    tri[4 * (int64_t)ts + 3] = make_float4(n.x, n.y, n.z, 0.0f);
    leaf_ref[i] = kLeafBit | kTriBit | ts;
  }
}

__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ m, int64_t n, int64_t i, int64_t j) {
  if (j < 0 || j >= n) return -1;
  uint64_t ki = ((uint64_t)m[i] << 32) | (uint32_t)i;
  uint64_t kj = ((uint64_t)m[j] << 32) | (uint32_t)j;
  return __clzll(ki ^ kj);
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees,
// and k-d trees": internal node i covers a key range found from the sign of
// the prefix difference and splits at the highest differing bit.
__global__ void karras_kernel(const uint32_t* __restrict__ m, int64_t n, const uint32_t* __restrict__ leaf_ref,
                              Node* __restrict__ nodes, uint32_t* __restrict__ parent) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (kdelta(m, n, i, i + 1) - kdelta(m, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(m, n, i, i - d);
  int64_t lmax = 2;
  while (kdelta(m, n, i, i + lmax * d) > dmin) lmax *= 2;
  int64_t l = 0;
  for (int64_t t = lmax / 2; t >= 1; t /= 2)
    if (kdelta(m, n, i, i + (l + t) * d) > dmin) l += t;
  const int64_t j = i + l * d;
  const int dnode = kdelta(m, n, i, j);
  int64_t s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (kdelta(m, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
  const int64_t first = i < j ? i : j, last = i < j ? j : i;
  uint32_t left, right;
  if (first == gamma) {
    left = leaf_ref[gamma];
    parent[(n - 1) + gamma] = (uint32_t)i;
  } else {
    left = (uint32_t)gamma;
    parent[gamma] = (uint32_t)i;
  }
  if (last == gamma + 1) {
    right = leaf_ref[gamma + 1];
    parent[(n - 1) + gamma + 1] = (uint32_t)i;
  } else {
    right = (uint32_t)(gamma + 1);
    parent[gamma + 1] = (uint32_t)i;
  }
  nodes[i].d = make_uint4(left, right, 0u, 0u);
}


// ---- PLOC: parallel locally-ordered clustering (Meister and Bittner, TVCG
// 2018), an agglomerative build over the Morton-ordered leaves.  Each round,
// every cluster finds the neighbour within kPlocRadius positions whose merged
// box has the smallest surface area (ties: the lower position); mutual pairs
// merge into a new internal node; the survivors are compacted in order.
// Node indices are handed out from the top down, round by round and in
// position order, so the root is node 0 and the layout is deterministic.
constexpr int kPlocRadius = 16;
constexpr int kPlocThreads = 256;
constexpr uint32_t kClusterLeaf = 0x80000000u;  // cluster = sorted leaf index | bit 31, else a node index

__global__ void ploc_init_kernel(const uint32_t* __restrict__ sorted_prim, int64_t n, const float* __restrict__ plo,
                                 const float* __restrict__ phi, uint32_t* __restrict__ cid, float4* __restrict__ blo,
                                 float4* __restrict__ bhi) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t p = sorted_prim[i];
  cid[i] = kClusterLeaf | (uint32_t)i;
  blo[i] = make_float4(plo[3 * p], plo[3 * p + 1], plo[3 * p + 2], 0.0f);
  bhi[i] = make_float4(phi[3 * p], phi[3 * p + 1], phi[3 * p + 2], 0.0f);
}

__device__ __forceinline__ float merged_area(float4 al, float4 ah, float4 bl, float4 bh) {
  const float dx = fmaxf(ah.x, bh.x) - fminf(al.x, bl.x);
  const float dy = fmaxf(ah.y, bh.y) - fminf(al.y, bl.y);
  const float dz = fmaxf(ah.z, bh.z) - fminf(al.z, bl.z);
  return dx * dy + dy * dz + dz * dx;
}

__global__ void __launch_bounds__(kPlocThreads) ploc_nn_kernel(const float4* __restrict__ blo,
                                                               const float4* __restrict__ bhi,
                                                               const uint64_t* __restrict__ state,
                                                               uint32_t* __restrict__ nn) {
  __shared__ float4 slo[kPlocThreads + 2 * kPlocRadius], shi[kPlocThreads + 2 * kPlocRadius];
  const int64_t n = (int64_t)state[0];
  if (n < 2 || (int64_t)blockIdx.x * kPlocThreads >= n) return;
  const int64_t b0 = (int64_t)blockIdx.x * kPlocThreads;
  for (int k = threadIdx.x; k < kPlocThreads + 2 * kPlocRadius; k += kPlocThreads) {
    const int64_t j = b0 - kPlocRadius + k;
    if (j >= 0 && j < n) {
      slo[k] = blo[j];
      shi[k] = bhi[j];
    }
  }
  __syncthreads();
  const int64_t i = b0 + threadIdx.x;
  if (i >= n) return;
  const int li = threadIdx.x + kPlocRadius;
  const float4 al = slo[li], ah = shi[li];
  float best = INFINITY;
  int64_t bj = i > 0 ? i - 1 : i + 1;
  for (int d = -kPlocRadius; d <= kPlocRadius; ++d) {
    const int64_t j = i + d;
    if (d == 0 || j < 0 || j >= n) continue;
    const float a = merged_area(al, ah, slo[li + d], shi[li + d]);
    if (a < best) {
      best = a;
      bj = j;
    }
  }
  nn[i] = (uint32_t)bj;
}

// Per position: (survives << 32) | merges-with-its-higher-mutual-neighbour,
// zero beyond the current cluster count (the scan length is an upper bound).
// The higher member of a mutual pair is absorbed.
__global__ void ploc_flags_kernel(const uint32_t* __restrict__ nn, int64_t bound, const uint64_t* __restrict__ state,
                                  unsigned long long* __restrict__ packed) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= bound) return;
  const int64_t n = (int64_t)state[0];
  if (i >= n) {
    packed[i] = 0ull;
    return;
  }
  if (n < 2) {
    packed[i] = 1ull << 32;
    return;
  }
  const uint32_t j = nn[i];
  const bool mutual = nn[j] == (uint32_t)i;
  const unsigned long long merge = (mutual && (uint32_t)i < j) ? 1ull : 0ull;
  const unsigned long long keep = (mutual && (uint32_t)i > j) ? 0ull : 1ull;
  packed[i] = (keep << 32) | merge;
}

// After the scan: state[0] = surviving clusters, state[1] += merges; a round
// without a merge while clusters remain is recorded in state[2].
__global__ void ploc_update_kernel(const unsigned long long* __restrict__ total, uint64_t* __restrict__ state) {
  const unsigned long long t = *total;
  const uint64_t merges = t & 0xFFFFFFFFull, kept = t >> 32;
  if (merges == 0 && state[0] > 1) state[2] = 1;
  state[0] = kept;
  state[1] += merges;
}

__global__ void ploc_merge_kernel(const uint32_t* __restrict__ nn, int64_t bound,
                                  const uint64_t* __restrict__ state, const uint32_t* __restrict__ cid,
                                  const float4* __restrict__ blo, const float4* __restrict__ bhi,
                                  const unsigned long long* __restrict__ packed, uint32_t n_int,
                                  const uint32_t* __restrict__ leaf_ref, int64_t nleaves, Node* __restrict__ nodes,
                                  uint32_t* __restrict__ parent, uint32_t* __restrict__ cid_out,
                                  float4* __restrict__ blo_out, float4* __restrict__ bhi_out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)state[0];
  if (i >= bound || i >= n) return;
  if (n < 2) {  // the finished root cluster: carried over unchanged
    cid_out[0] = cid[0];
    blo_out[0] = blo[0];
    bhi_out[0] = bhi[0];
    return;
  }
  const uint32_t j = nn[i];
  const bool mutual = nn[j] == (uint32_t)i;
  if (mutual && (uint32_t)i > j) return;  // absorbed by j
  // positions after compaction (high word) and merge ranks (low word) come
  // from the exclusive scan; nodes are handed out downwards from node_top
  const uint32_t pos = (uint32_t)(packed[i] >> 32);
  const uint32_t rank = (uint32_t)(packed[i] & 0xFFFFFFFFull);
  const uint32_t node_top = n_int - 1u - (uint32_t)state[1];
  if (mutual) {
    const uint32_t idx = node_top - rank;
    const uint32_t a = cid[i], b = cid[j];
    const uint32_t ra = (a & kClusterLeaf) ? leaf_ref[a & ~kClusterLeaf] : a;
    const uint32_t rb = (b & kClusterLeaf) ? leaf_ref[b & ~kClusterLeaf] : b;
    nodes[idx].d = make_uint4(ra, rb, 0u, 0u);
    if (a & kClusterLeaf) parent[(nleaves - 1) + (a & ~kClusterLeaf)] = idx;
    else parent[a] = idx;
    if (b & kClusterLeaf) parent[(nleaves - 1) + (b & ~kClusterLeaf)] = idx;
    else parent[b] = idx;
    const float4 al = blo[i], ah = bhi[i], bl = blo[j], bh = bhi[j];
    cid_out[pos] = idx;
    blo_out[pos] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
    bhi_out[pos] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
  } else {
    cid_out[pos] = cid[i];
    blo_out[pos] = blo[i];
    bhi_out[pos] = bhi[i];
  }
}

// The last rounds of PLOC in one block: once at most kPlocTailMax clusters
// remain, the rounds are too small to fill the GPU and a launch sequence per
// round (neighbours, flags, scan, merge) costs more than the work.  One block
// of kPlocTailThreads runs every remaining round with the same rules as the
// kernels above -- nearest neighbour within kPlocRadius positions (ties to the
// lower position), mutual pairs merged by the lower member, survivors
// compacted in order, nodes handed out downwards in position order -- so the
// tree is the one the round-by-round launches would build.  Each round merges
// at least the pair of smallest merged area, so the loop ends after at most
// n - 1 rounds (n_int + 1 bounds it); a round without a merge sets state[2]
// and stops.
constexpr uint32_t kPlocTailMax = 8192;  // measured: 2 Ki-8 Ki fastest on the hole (200 k leaves)
constexpr int kPlocTailThreads = 1024;

__global__ void __launch_bounds__(kPlocTailThreads) ploc_tail_kernel(
    uint32_t* __restrict__ cid0, float4* __restrict__ blo0, float4* __restrict__ bhi0, uint32_t* __restrict__ cid1,
    float4* __restrict__ blo1, float4* __restrict__ bhi1, uint32_t* __restrict__ nn, uint64_t* __restrict__ state,
    uint32_t n_int, const uint32_t* __restrict__ leaf_ref, int64_t nleaves, Node* __restrict__ nodes,
    uint32_t* __restrict__ parent) {
  __shared__ uint32_t w_keep[kPlocTailThreads / 32], w_merge[kPlocTailThreads / 32];
  __shared__ uint32_t s_tot[2];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  uint32_t n = (uint32_t)state[0];
  uint32_t allocated = (uint32_t)state[1];
  uint32_t* cid_in = cid0;
  float4* blo_in = blo0;
  float4* bhi_in = bhi0;
  uint32_t* cid_out = cid1;
  float4* blo_out = blo1;
  float4* bhi_out = bhi1;
  bool stalled = false;
  for (uint32_t round = 0; n > 1 && round < n_int + 1u; ++round) {
    for (uint32_t i = tid; i < n; i += kPlocTailThreads) {
      const float4 al = blo_in[i], ah = bhi_in[i];
      float best = INFINITY;
      uint32_t bj = i > 0 ? i - 1 : i + 1;
      for (int d = -kPlocRadius; d <= kPlocRadius; ++d) {
        const int64_t j = (int64_t)i + d;
        if (d == 0 || j < 0 || j >= (int64_t)n) continue;
        const float a = merged_area(al, ah, blo_in[j], bhi_in[j]);
        if (a < best) {
          best = a;
          bj = (uint32_t)j;
        }
      }
      nn[i] = bj;
    }
    __syncthreads();
    // survivors and merges of this thread's run of positions, then their
    // exclusive prefix over the block (positions in order)
    const uint32_t per = (n + kPlocTailThreads - 1) / kPlocTailThreads;
    const uint32_t c0 = min(n, tid * per), c1 = min(n, c0 + per);
    uint32_t keep = 0, merge = 0;
    for (uint32_t i = c0; i < c1; ++i) {
      const uint32_t j = nn[i];
      const bool mutual = nn[j] == i;
      keep += (mutual && i > j) ? 0u : 1u;
      merge += (mutual && i < j) ? 1u : 0u;
    }
    uint32_t ik = keep, im = merge;  // inclusive warp scan
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t k2 = __shfl_up_sync(0xFFFFFFFFu, ik, o), m2 = __shfl_up_sync(0xFFFFFFFFu, im, o);
      if (lane >= (uint32_t)o) {
        ik += k2;
        im += m2;
      }
    }
    if (lane == 31) {
      w_keep[warp] = ik;
      w_merge[warp] = im;
    }
    __syncthreads();
    if (warp == 0) {
      uint32_t tk = lane < kPlocTailThreads / 32 ? w_keep[lane] : 0u, tm = lane < kPlocTailThreads / 32 ? w_merge[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t k2 = __shfl_up_sync(0xFFFFFFFFu, tk, o), m2 = __shfl_up_sync(0xFFFFFFFFu, tm, o);
        if (lane >= (uint32_t)o) {
          tk += k2;
          tm += m2;
        }
      }
      if (lane < kPlocTailThreads / 32) {  // inclusive prefix over the warps
        w_keep[lane] = tk;
        w_merge[lane] = tm;
      }
      if (lane == kPlocTailThreads / 32 - 1) {
        s_tot[0] = tk;
        s_tot[1] = tm;
      }
    }
    __syncthreads();
    uint32_t pos = (warp > 0 ? w_keep[warp - 1] : 0u) + ik - keep;
    uint32_t rank = (warp > 0 ? w_merge[warp - 1] : 0u) + im - merge;
    const uint32_t kept_total = s_tot[0], merged_total = s_tot[1];
    const uint32_t node_top = n_int - 1u - allocated;
    for (uint32_t i = c0; i < c1; ++i) {
      const uint32_t j = nn[i];
      const bool mutual = nn[j] == i;
      if (mutual && i > j) continue;  // absorbed by j
      if (mutual) {
        const uint32_t idx = node_top - rank++;
        const uint32_t a = cid_in[i], b = cid_in[j];
        const uint32_t ra = (a & kClusterLeaf) ? leaf_ref[a & ~kClusterLeaf] : a;
        const uint32_t rb = (b & kClusterLeaf) ? leaf_ref[b & ~kClusterLeaf] : b;
        nodes[idx].d = make_uint4(ra, rb, 0u, 0u);
        if (a & kClusterLeaf) parent[(nleaves - 1) + (a & ~kClusterLeaf)] = idx;
        else parent[a] = idx;
        if (b & kClusterLeaf) parent[(nleaves - 1) + (b & ~kClusterLeaf)] = idx;
        else parent[b] = idx;
        const float4 al = blo_in[i], ah = bhi_in[i], bl = blo_in[j], bh = bhi_in[j];
        cid_out[pos] = idx;
        blo_out[pos] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
        bhi_out[pos] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
      } else {
        cid_out[pos] = cid_in[i];
        blo_out[pos] = blo_in[i];
        bhi_out[pos] = bhi_in[i];
      }
      ++pos;
    }
    __syncthreads();  // the outputs are complete before they become the inputs
    if (merged_total == 0) {
      stalled = true;
      break;
    }
    allocated += merged_total;
    n = kept_total;
    uint32_t* tc = cid_in;
    cid_in = cid_out;
    cid_out = tc;
    float4* tl = blo_in;
    blo_in = blo_out;
    blo_out = tl;
    float4* th = bhi_in;
    bhi_in = bhi_out;
    bhi_out = th;
  }
  if (tid == 0) {
    state[0] = n;
    state[1] = allocated;
    if (stalled || n > 1) state[2] = 1;
  }
}

__device__ __forceinline__ void child_box(uint32_t ref, const float4* __restrict__ dn,
                                          const float4* __restrict__ tri, const float* __restrict__ plo,
                                          const float* __restrict__ phi, const float* node_box, float* lo,
                                          float* hi) {
  if (ref & kLeafBit) {
    uint32_t slot = ref & kSlotMask;
    int p = (ref & kTriBit) ? __float_as_int(tri[4 * (int64_t)slot].w) : __float_as_int(dn[2 * (int64_t)slot + 1].w);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lo[a] = plo[3 * (int64_t)p + a];
      hi[a] = phi[3 * (int64_t)p + a];
    }
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lo[a] = __ldcg(&node_box[6 * (int64_t)ref + a]);
      hi[a] = __ldcg(&node_box[6 * (int64_t)ref + 3 + a]);
    }
  }
}

// Bottom-up refit: the second thread to reach a node writes both child boxes.
__global__ void refit_kernel(int64_t n, const uint32_t* __restrict__ leaf_ref, const uint32_t* __restrict__ parent,
                             const float4* __restrict__ dn, const float4* __restrict__ tri,
                             const float* __restrict__ plo, const float* __restrict__ phi, Node* nodes,
                             float* node_box, unsigned int* flags, unsigned long long* errors) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t node = parent[(n - 1) + i];
  for (int iter = 0; iter < 256; ++iter) {
    if ((int64_t)node >= n - 1) break;  // a parent that was never written
    __threadfence();
    unsigned int old = atomicAdd(&flags[node], 1u);
    if (old == 0) return;
    uint4 r = __ldcg(&nodes[node].d);
    float l0[3], h0[3], l1[3], h1[3];
    child_box(r.x, dn, tri, plo, phi, node_box, l0, h0);
    child_box(r.y, dn, tri, plo, phi, node_box, l1, h1);
    nodes[node].a = make_float4(l0[0], h0[0], l1[0], h1[0]);
    nodes[node].b = make_float4(l0[1], h0[1], l1[1], h1[1]);
    nodes[node].c = make_float4(l0[2], h0[2], l1[2], h1[2]);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      node_box[6 * (int64_t)node + a] = fminf(l0[a], l1[a]);
      node_box[6 * (int64_t)node + 3 + a] = fmaxf(h0[a], h1[a]);
    }
    __threadfence();
    if (node == 0) return;
    node = parent[node];
  }
  atomicAdd(errors, 1ull);
}

// Structural check of the tree before any traversal: every child reference is
// in range, and every node except the root has exactly one parent.
__global__ void validate_kernel(const Node* __restrict__ nodes, int64_t n_internal, int64_t nd, int64_t nt,
                                unsigned int* __restrict__ parents_internal,
                                unsigned int* __restrict__ parents_disc, unsigned int* __restrict__ parents_tri,
                                unsigned long long* __restrict__ errors) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_internal) return;
  const uint4 d = nodes[i].d;
  const uint32_t ch[2] = {d.x, d.y};
  for (int k = 0; k < 2; ++k) {
    const uint32_t r = ch[k];
    const uint32_t slot = r & kSlotMask;
    if (r & kLeafBit) {
      if (r & kTriBit) {
        if ((int64_t)slot < nt) atomicAdd(&parents_tri[slot], 1u);
        else atomicAdd(errors, 1ull);
      } else {
        if ((int64_t)slot < nd) atomicAdd(&parents_disc[slot], 1u);
        else atomicAdd(errors, 1ull);
      }
    } else if (r & kTriBit) {
      atomicAdd(errors, 1ull);
    } else if (slot == 0 || (int64_t)slot >= n_internal) {
      atomicAdd(errors, 1ull);
    } else {
      atomicAdd(&parents_internal[slot], 1u);
    }
  }
}

__global__ void count_check_kernel(const unsigned int* __restrict__ c, int64_t n, unsigned int expect_first,
                                   unsigned long long* __restrict__ errors) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned int want = i == 0 ? expect_first : 1u;
  if (c[i] != want) atomicAdd(errors, 1ull);
}

__global__ void single_leaf_kernel(const uint32_t* __restrict__ leaf_ref, const float4* __restrict__ dn,
                                   const float4* __restrict__ tri, const float* __restrict__ plo,
                                   const float* __restrict__ phi, Node* nodes) {
  uint32_t r = leaf_ref[0];
  float l[3], h[3];
  child_box(r, dn, tri, plo, phi, nullptr, l, h);
  nodes[0].a = make_float4(l[0], h[0], l[0], h[0]);
  nodes[0].b = make_float4(l[1], h[1], l[1], h[1]);
  nodes[0].c = make_float4(l[2], h[2], l[2], h[2]);
  nodes[0].d = make_uint4(r, r, 0u, 0u);
}

// Internal nodes from each leaf up to the root (bounded walk); the maximum
// is the deepest stack a traversal can need.
__global__ void depth_kernel(int64_t n, const uint32_t* __restrict__ parent, unsigned int* __restrict__ depth) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t node = parent[(n - 1) + i];
  unsigned int d = 0;
  for (int iter = 0; iter < 512; ++iter) {
    if ((int64_t)node >= n - 1) {
      d = 0xFFFFFFFFu;  // a broken link (the structural check reports it)
      break;
    }
    d += 1;
    if (node == 0) break;
    node = parent[node];
  }
  atomicMax(depth, d);
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int tree_depth(rtg_context* ctx, cudaStream_t st) {
  Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  if (np < 2) {
    g.depth = 1;
    return RTG_OK;
  }
  DBuf<unsigned int> dd;
  RTG_TRY(talloc(ctx, dd, 1, st, "tree depth"));
  unsigned int h = 0;
  cudaMemsetAsync(dd.p, 0, sizeof(unsigned int), st);
  depth_kernel<<<blocks_for(np, 256), 256, 0, st>>>(np, g.parent.p, dd.p);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, dd.p, sizeof h, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  tfree(dd, st);
  if (e != cudaSuccess) return check_cuda(ctx, e, "tree depth");
  if (h > 256) return set_error(ctx, RTG_ERR_INTERNAL, "LBVH deeper than 256 levels");
  g.depth = (int32_t)h;
  return RTG_OK;
}

int validate_tree(rtg_context* ctx, cudaStream_t st) {
  Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  if (np < 2) return RTG_OK;
  const int64_t ni = np - 1;
  DBuf<unsigned int> pi, pd, pt;
  DBuf<unsigned long long> err;
  auto cleanup = [&]() { tfree(pi, st); tfree(pd, st); tfree(pt, st); tfree(err, st); };
  int rc = talloc(ctx, pi, (size_t)ni, st, "tree check");
  if (rc == RTG_OK) rc = talloc(ctx, pd, (size_t)(g.nd ? g.nd : 1), st, "tree check");
  if (rc == RTG_OK) rc = talloc(ctx, pt, (size_t)(g.nt ? g.nt : 1), st, "tree check");
  if (rc == RTG_OK) rc = talloc(ctx, err, 1, st, "tree check");
  if (rc != RTG_OK) { cleanup(); return rc; }
  cudaMemsetAsync(pi.p, 0, ni * sizeof(unsigned int), st);
  cudaMemsetAsync(pd.p, 0, pd.n * sizeof(unsigned int), st);
  cudaMemsetAsync(pt.p, 0, pt.n * sizeof(unsigned int), st);
  cudaMemsetAsync(err.p, 0, sizeof(unsigned long long), st);
  validate_kernel<<<blocks_for(ni, 256), 256, 0, st>>>(g.nodes.p, ni, g.nd, g.nt, pi.p, pd.p, pt.p, err.p);
  count_check_kernel<<<blocks_for(ni, 256), 256, 0, st>>>(pi.p, ni, 0u, err.p);
  if (g.nd) count_check_kernel<<<blocks_for(g.nd, 256), 256, 0, st>>>(pd.p, g.nd, 1u, err.p);
  if (g.nt) count_check_kernel<<<blocks_for(g.nt, 256), 256, 0, st>>>(pt.p, g.nt, 1u, err.p);
  unsigned long long h = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err.p, sizeof h, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return check_cuda(ctx, e, "LBVH check");
  if (h) return set_error(ctx, RTG_ERR_INTERNAL, "LBVH check failed: " + std::to_string(h) + " bad links");
  return RTG_OK;
}


// Binary tree over the np sorted leaves by PLOC (see ploc_* kernels): writes
// the child references of nodes [0, np-1) and the parent array; boxes come
// from the refit that follows.
int build_ploc(rtg_context* ctx, const uint32_t* d_sorted_prim, cudaStream_t st) {
  Geometry& g = ctx->g;
  const int64_t n = g.nd + g.nt;
  DBuf<uint32_t> cid[2], nn;
  DBuf<float4> blo[2], bhi[2];
  DBuf<int64_t> packed, total;
  DBuf<uint64_t> state;  // [0] clusters, [1] nodes allocated, [2] stall flag
  auto cleanup = [&]() {
    for (int q = 0; q < 2; ++q) {
      tfree(cid[q], st);
      tfree(blo[q], st);
      tfree(bhi[q], st);
    }
    tfree(nn, st);
    tfree(packed, st);
    tfree(total, st);
    tfree(state, st);
  };
  int rc = RTG_OK;
  for (int q = 0; q < 2 && rc == RTG_OK; ++q) {
    rc = talloc(ctx, cid[q], (size_t)n, st, "PLOC clusters");
    if (rc == RTG_OK) rc = talloc(ctx, blo[q], (size_t)n, st, "PLOC boxes");
    if (rc == RTG_OK) rc = talloc(ctx, bhi[q], (size_t)n, st, "PLOC boxes");
  }
  if (rc == RTG_OK) rc = talloc(ctx, nn, (size_t)n, st, "PLOC neighbours");
  if (rc == RTG_OK) rc = talloc(ctx, packed, (size_t)n, st, "PLOC scan");
  if (rc == RTG_OK) rc = talloc(ctx, total, 1, st, "PLOC totals");
  if (rc == RTG_OK) rc = talloc(ctx, state, 3, st, "PLOC state");
  if (rc != RTG_OK) {
    cleanup();
    return rc;
  }
  const uint64_t init[3] = {(uint64_t)n, 0, 0};
  cudaMemcpyAsync(state.p, init, sizeof init, cudaMemcpyHostToDevice, st);
  ploc_init_kernel<<<blocks_for(n, 256), 256, 0, st>>>(d_sorted_prim, n, g.prim_lo.p, g.prim_hi.p, cid[0].p,
                                                        blo[0].p, bhi[0].p);
  const uint32_t n_int = (uint32_t)(n - 1);
  int64_t bound = n;  // the cluster count is only read back between chunks of rounds
  int q = 0;
  uint64_t h[3] = {(uint64_t)n, 0, 0};
  for (int chunk = 0; h[0] > 1; ++chunk) {
    if (chunk > 10000) {
      rc = set_error(ctx, RTG_ERR_INTERNAL, "PLOC did not converge");
      break;
    }
    if (h[0] <= kPlocTailMax) {  // the remaining rounds in one block
      ploc_tail_kernel<<<1, kPlocTailThreads, 0, st>>>(cid[q].p, blo[q].p, bhi[q].p, cid[q ^ 1].p, blo[q ^ 1].p,
                                                        bhi[q ^ 1].p, nn.p, state.p, n_int, g.leaf_ref.p, n,
                                                        g.nodes.p, g.parent.p);
    }
    for (int r = 0; r < 4 && rc == RTG_OK && h[0] > kPlocTailMax; ++r) {
      const unsigned nb = (unsigned)((bound + kPlocThreads - 1) / kPlocThreads);
      ploc_nn_kernel<<<nb, kPlocThreads, 0, st>>>(blo[q].p, bhi[q].p, state.p, nn.p);
      ploc_flags_kernel<<<blocks_for(bound, 256), 256, 0, st>>>(nn.p, bound, state.p,
                                                                (unsigned long long*)packed.p);
      rc = exclusive_scan_i64(ctx, packed.p, bound, total.p, st);
      if (rc != RTG_OK) break;
      ploc_merge_kernel<<<blocks_for(bound, 256), 256, 0, st>>>(
          nn.p, bound, state.p, cid[q].p, blo[q].p, bhi[q].p, (const unsigned long long*)packed.p, n_int,
          g.leaf_ref.p, n, g.nodes.p, g.parent.p, cid[q ^ 1].p, blo[q ^ 1].p, bhi[q ^ 1].p);
      ploc_update_kernel<<<1, 1, 0, st>>>((const unsigned long long*)total.p, state.p);
      q ^= 1;
    }
    if (rc != RTG_OK) break;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, state.p, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      rc = check_cuda(ctx, e, "PLOC round");
      break;
    }
    if (h[2] != 0 || h[1] > n_int) {
      rc = set_error(ctx, RTG_ERR_INTERNAL, "PLOC round without progress");
      break;
    }
    bound = (int64_t)h[0];
  }
  if (rc == RTG_OK && h[1] != n_int) rc = set_error(ctx, RTG_ERR_INTERNAL, "PLOC node count mismatch");
  cudaStreamSynchronize(st);
  cleanup();
  return rc;
}

int run_bounds(rtg_context* ctx, uint32_t* d_cbounds, cudaStream_t st) {
  Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  RTG_TRY(dalloc(ctx, g.prim_lo, (size_t)(3 * np), "primitive boxes"));
  RTG_TRY(dalloc(ctx, g.prim_hi, (size_t)(3 * np), "primitive boxes"));
  prim_bounds_kernel<<<blocks_for(np, 256), 256, 0, st>>>(g.disc_cr_by_id.p, g.disc_n_by_id.p, g.nd,
                                                          g.tri_v.p, g.tri_idx.p, g.nt, g.prim_lo.p,
                                                          g.prim_hi.p, d_cbounds);
  RTG_CUDA(ctx, cudaGetLastError());
  return RTG_OK;
}

int run_slots_and_refit(rtg_context* ctx, const uint32_t* d_sorted_prim, const uint32_t* d_disc_rank,
                        cudaStream_t st) {
  Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  if (d_sorted_prim) {
    slots_kernel<<<blocks_for(np, 256), 256, 0, st>>>(d_sorted_prim, d_disc_rank, np, g.nd, g.disc_cr_by_id.p,
                                                      g.disc_n_by_id.p, g.tri_v.p, g.tri_idx.p, g.disc.p,
                                                      g.disc_slot.p, g.tri.p, g.leaf_ref.p,
                                                      g.leaf_prim.p);
    RTG_CUDA(ctx, cudaGetLastError());
  }
  if (np == 1) {
    single_leaf_kernel<<<1, 1, 0, st>>>(g.leaf_ref.p, g.disc.p, g.tri.p, g.prim_lo.p, g.prim_hi.p, g.nodes.p);
    RTG_CUDA(ctx, cudaGetLastError());
    g.wide_current = false;
    return wants_wide(ctx) ? build_wide(ctx, st) : RTG_OK;
  }
  DBuf<float> node_box;
  DBuf<unsigned long long> err;
  int rc = talloc(ctx, node_box, (size_t)(6 * (np - 1)), st, "node boxes");
  if (rc == RTG_OK) rc = talloc(ctx, err, 1, st, "refit status");
  if (rc == RTG_OK) rc = dalloc(ctx, g.refit_flags, (size_t)(np - 1), "refit flags");
  if (rc != RTG_OK) {
    tfree(node_box, st);
    tfree(err, st);
    return rc;
  }
  cudaMemsetAsync(g.refit_flags.p, 0, sizeof(unsigned int) * (np - 1), st);
  cudaMemsetAsync(err.p, 0, sizeof(unsigned long long), st);
  refit_kernel<<<blocks_for(np, 256), 256, 0, st>>>(np, g.leaf_ref.p, g.parent.p, g.disc.p, g.tri.p,
                                                    g.prim_lo.p, g.prim_hi.p, g.nodes.p, node_box.p,
                                                    g.refit_flags.p, err.p);
  cudaError_t e = cudaGetLastError();
  unsigned long long herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err.p, sizeof herr, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  tfree(node_box, st);
  tfree(err, st);
  if (e != cudaSuccess) return check_cuda(ctx, e, "LBVH refit");
  if (herr) return set_error(ctx, RTG_ERR_INTERNAL, "LBVH refit exceeded its depth limit");
  g.wide_current = false;  // the wide tree's boxes follow the binary ones: now, or before a trace that wants it
  return wants_wide(ctx) ? build_wide(ctx, st) : RTG_OK;
}

}  // namespace

int build_lbvh(rtg_context* ctx) {
  Geometry& g = ctx->g;
  cudaStream_t st = ctx->stream;
  const int64_t np = g.nd + g.nt;
  if (np <= 0) return set_error(ctx, RTG_ERR_NO_GEOMETRY, "no primitives");
  if (np > (int64_t)kSlotMask) return set_error(ctx, RTG_ERR_INVALID_ARGUMENT, "too many primitives");
  DBuf<uint32_t> cb, keys, vals, tk, tv, rank;
  auto cleanup = [&]() { tfree(cb, st); tfree(keys, st); tfree(vals, st); tfree(tk, st); tfree(tv, st); tfree(rank, st); };
  int rc = RTG_OK;
  do {
    if ((rc = talloc(ctx, cb, 6, st, "centroid bounds")) != RTG_OK) break;
    const uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    if (cudaMemcpyAsync(cb.p, init, sizeof init, cudaMemcpyHostToDevice, st) != cudaSuccess) {
      rc = check_cuda(ctx, cudaGetLastError(), "centroid bounds init");
      break;
    }
    if ((rc = run_bounds(ctx, cb.p, st)) != RTG_OK) break;
    if ((rc = talloc(ctx, keys, (size_t)np, st, "morton keys")) != RTG_OK) break;
    if ((rc = talloc(ctx, vals, (size_t)np, st, "morton values")) != RTG_OK) break;
    if ((rc = talloc(ctx, tk, (size_t)np, st, "sort scratch")) != RTG_OK) break;
    if ((rc = talloc(ctx, tv, (size_t)np, st, "sort scratch")) != RTG_OK) break;
    morton_kernel<<<blocks_for(np, 256), 256, 0, st>>>(g.prim_lo.p, g.prim_hi.p, np, cb.p, keys.p, vals.p);
    if (cudaGetLastError() != cudaSuccess) { rc = check_cuda(ctx, cudaGetLastError(), "morton"); break; }
    if ((rc = radix_sort_pairs(ctx, keys.p, vals.p, tk.p, tv.p, np, 30, st)) != RTG_OK) break;
    // disc slot = number of discs before this sorted position
    if ((rc = talloc(ctx, rank, (size_t)np, st, "disc ranks")) != RTG_OK) break;
    disc_flag_kernel<<<blocks_for(np, 256), 256, 0, st>>>(vals.p, np, g.nd, rank.p);
    if ((rc = exclusive_scan_u32(ctx, rank.p, np, nullptr, st)) != RTG_OK) break;
    if ((rc = dalloc(ctx, g.disc, (size_t)(2 * (g.nd ? g.nd : 1)), "disc slots")) != RTG_OK) break;
    if ((rc = dalloc(ctx, g.disc_slot, (size_t)(g.nd ? g.nd : 1), "disc slot map")) != RTG_OK) break;
    if ((rc = dalloc(ctx, g.tri, (size_t)(4 * (g.nt ? g.nt : 1)), "triangle slots")) != RTG_OK) break;
    if ((rc = dalloc(ctx, g.leaf_ref, (size_t)np, "leaf references")) != RTG_OK) break;
    if ((rc = dalloc(ctx, g.leaf_prim, (size_t)np, "leaf primitives")) != RTG_OK) break;
    const int64_t nn = np > 1 ? np - 1 : 1;
    if ((rc = dalloc(ctx, g.nodes, (size_t)nn, "LBVH nodes")) != RTG_OK) break;
    if ((rc = dalloc(ctx, g.parent, (size_t)(2 * np), "LBVH parents")) != RTG_OK) break;
    // slots first: the Karras kernel reads the leaf references
    slots_kernel<<<blocks_for(np, 256), 256, 0, st>>>(vals.p, rank.p, np, g.nd, g.disc_cr_by_id.p,
                                                      g.disc_n_by_id.p, g.tri_v.p, g.tri_idx.p, g.disc.p,
                                                      g.disc_slot.p, g.tri.p, g.leaf_ref.p,
                                                      g.leaf_prim.p);
    if (cudaGetLastError() != cudaSuccess) { rc = check_cuda(ctx, cudaGetLastError(), "slots"); break; }
    if (np > 1) {
      // PLOC first; a clustering deeper than the traversal stacks allow (possible
      // for degenerate inputs) falls back to the Karras tree, whose depth is
      // bounded by the key length
      bool karras = g.builder != kBuilderPloc;
      if (!karras) {
        cudaMemsetAsync(g.parent.p, 0xFF, 2 * np * sizeof(uint32_t), st);
        if ((rc = build_ploc(ctx, vals.p, st)) != RTG_OK) break;
        if ((rc = validate_tree(ctx, st)) != RTG_OK) break;
        const int drc = tree_depth(ctx, st);  // RTG_ERR_INTERNAL: too deep for the stacks
        if (drc != RTG_OK && drc != RTG_ERR_INTERNAL) {
          rc = drc;
          break;
        }
        karras = drc != RTG_OK;
      }
      if (karras) {
        cudaMemsetAsync(g.parent.p, 0xFF, 2 * np * sizeof(uint32_t), st);
        karras_kernel<<<blocks_for(np - 1, 256), 256, 0, st>>>(keys.p, np, g.leaf_ref.p, g.nodes.p, g.parent.p);
        if (cudaGetLastError() != cudaSuccess) { rc = check_cuda(ctx, cudaGetLastError(), "karras"); break; }
        if ((rc = validate_tree(ctx, st)) != RTG_OK) break;
      }
    }
    if ((rc = tree_depth(ctx, st)) != RTG_OK) break;
    rc = run_slots_and_refit(ctx, nullptr, nullptr, st);
  } while (0);
  cudaStreamSynchronize(st);
  cleanup();
  g.root = 0;
  return rc;
}

int refit_lbvh(rtg_context* ctx) {
  Geometry& g = ctx->g;
  cudaStream_t st = ctx->stream;
  RTG_TRY(run_bounds(ctx, nullptr, st));
  // keep the leaf order: recompute slot data from the sorted primitive order
  const int64_t np = g.nd + g.nt;
  DBuf<uint32_t> rank, order;
  int rc = talloc(ctx, rank, (size_t)np, st, "disc ranks");
  if (rc == RTG_OK) rc = talloc(ctx, order, (size_t)np, st, "leaf order");
  if (rc == RTG_OK) {
    cudaMemcpyAsync(order.p, g.leaf_prim.p, np * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    disc_flag_kernel<<<blocks_for(np, 256), 256, 0, st>>>(order.p, np, g.nd, rank.p);
    rc = exclusive_scan_u32(ctx, rank.p, np, nullptr, st);
  }
  if (rc == RTG_OK) rc = run_slots_and_refit(ctx, order.p, rank.p, st);
  cudaStreamSynchronize(st);
  tfree(rank, st);
  tfree(order, st);
  return rc;
}

}  // namespace rtg
