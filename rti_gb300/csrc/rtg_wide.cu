// rtg_wide.cu -- the compressed 8-wide tree of the closest-hit query.
//
// Collapses the binary LBVH (Karras or PLOC, after every build and refit) top
// down into nodes of up to eight children: a wide node starts from the two
// children of its binary node and repeatedly opens the internal child of
// largest surface area until it holds eight or only primitives remain (the
// greedy collapse of Ylitie, Karras and Laine, HPG 2017).  Each wide level is
// one launch; the children of a node get consecutive indices, so the nodes
// lie in breadth-first order with siblings side by side.
//
// Child boxes are stored as bytes on a per-node grid (WideNode in
// rtg_internal.cuh): the quantum of an axis is 2^e, the origin p an exact
// multiple of it with |p| / 2^e < 2^23, so p + q 2^e is a float exactly for
// every q <= 255 and the decoded box contains the binary tree's float box
// (floor for lo, ceil for hi).  The closest-hit traversal therefore tests
// boxes that contain the ones the binary traversal tests.
//
// Children are placed in slots by direction: slot s takes the child that lies
// most towards the corner whose signs are the bits of s, assigned greedily by
// the centre offset from the node centre (in units of the node extent).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "rtg_internal.cuh"

namespace rtg {

namespace {

struct WChild {
  uint32_t ref;
  float lo[3], hi[3];
};

// ctl: [0] first wide node of the level, [1] one past its last, [2] wide
// nodes allocated, [3] deepest traversal stack, [4] errors
constexpr int kCtlWords = 5;

__device__ __forceinline__ void children_of(const Node& n, WChild& c0, WChild& c1) {
  c0.ref = n.d.x;
  c0.lo[0] = n.a.x; c0.hi[0] = n.a.y; c0.lo[1] = n.b.x; c0.hi[1] = n.b.y; c0.lo[2] = n.c.x; c0.hi[2] = n.c.y;
  c1.ref = n.d.y;
  c1.lo[0] = n.a.z; c1.hi[0] = n.a.w; c1.lo[1] = n.b.z; c1.hi[1] = n.b.w; c1.lo[2] = n.c.z; c1.hi[2] = n.c.w;
}

__device__ __forceinline__ float half_area(const WChild& c) {
  const float x = c.hi[0] - c.lo[0], y = c.hi[1] - c.lo[1], z = c.hi[2] - c.lo[2];
  return x * y + y * z + z * x;
}

// The grid of one axis over [lo, hi]: quantum 2^e and origin p with
// p <= lo, hi <= p + 255 * 2^e and |p| / 2^e <= 2^22.  Returns false when the
// quantum would exceed 2^4: the traversal forms 2^23 * 2^e / d with 1/d up to
// 1e30 (an axis-parallel ray), which must stay finite; such a scene (a node
// wider than 4080 units) is traced over the binary tree instead.
__device__ bool axis_grid(float lo, float hi, int& e, double& p) {
  const double dl = lo, dh = hi;
  const double mag = fmax(fabs(dl), fabs(dh));
  int e0 = -100;
  if (mag > 0.0) e0 = max(e0, ilogb(mag) - 21);          // |p| / 2^e <= 2^22
  const double ext = dh - dl;
  if (ext > 0.0) e0 = max(e0, ilogb(ext / 255.0));        // within one step of fitting
  for (e = e0; e <= 4; ++e) {
    const double s = ldexp(1.0, e);
    p = floor(dl / s) * s;
    if ((dh - p) / s <= 255.0 && fabs(p) / s <= 4194304.0) return true;
  }
  return false;
}

__global__ void wide_level_kernel(const Node* __restrict__ bn, uint32_t n_bin, WideNode* __restrict__ wn,
                                  uint32_t* __restrict__ w2b, uint32_t* __restrict__ need, unsigned int* ctl,
                                  uint32_t cap) {
  const uint32_t begin = ctl[0], end = min(ctl[1], cap);  // a level never reaches past the buffers
  for (uint32_t w = begin + blockIdx.x * blockDim.x + threadIdx.x; w < end; w += gridDim.x * blockDim.x) {
    WChild ch[kWide];
    int n = 2;
    const uint32_t b = w2b[w];
    if (b >= n_bin) {
      atomicAdd(&ctl[4], 1u);
      continue;
    }
    children_of(bn[b], ch[0], ch[1]);
    if (ch[0].ref == ch[1].ref) n = 1;  // a one-primitive tree holds its leaf in both children of the root
    bool bad = false;
    while (n < kWide) {
      int best = -1;
      float ba = -1.0f;
      for (int i = 0; i < n; ++i)
        if (!(ch[i].ref & kLeafBit)) {
          const float a = half_area(ch[i]);
          if (a > ba) {
            ba = a;
            best = i;
          }
        }
      if (best < 0) break;
      const uint32_t r = ch[best].ref;
      if (r >= n_bin) {
        bad = true;
        break;
      }
      children_of(bn[r], ch[best], ch[n]);
      ++n;
    }
    // the node's grid
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = ch[0].lo[a];
      hi[a] = ch[0].hi[a];
      for (int i = 1; i < n; ++i) {
        lo[a] = fminf(lo[a], ch[i].lo[a]);
        hi[a] = fmaxf(hi[a], ch[i].hi[a]);
      }
    }
    int e[3];
    double p[3];
    for (int a = 0; a < 3; ++a)
      if (!axis_grid(lo[a], hi[a], e[a], p[a])) bad = true;
    if (bad) {
      atomicAdd(&ctl[4], 1u);
      continue;
    }
    // slots by direction: greedy over (child, slot) pairs, best score first
    float off[kWide][3];
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < 3; ++a) {
        const float ext = hi[a] - lo[a];
        const float c = 0.5f * (ch[i].lo[a] + ch[i].hi[a]) - 0.5f * (lo[a] + hi[a]);
        off[i][a] = ext > 0.0f ? c / ext : 0.0f;
      }
    int slot_of[kWide], child_in[kWide];
    for (int i = 0; i < kWide; ++i) {
      slot_of[i] = -1;
      child_in[i] = -1;
    }
    for (int round = 0; round < n; ++round) {
      float bs = -FLT_MAX;
      int bi = -1, bsl = -1;
      for (int i = 0; i < n; ++i) {
        if (slot_of[i] >= 0) continue;
        for (int sl = 0; sl < kWide; ++sl) {
          if (child_in[sl] >= 0) continue;
          const float sc = ((sl & 1) ? off[i][0] : -off[i][0]) + ((sl & 2) ? off[i][1] : -off[i][1]) +
                           ((sl & 4) ? off[i][2] : -off[i][2]);
          if (sc > bs) {
            bs = sc;
            bi = i;
            bsl = sl;
          }
        }
      }
      slot_of[bi] = bsl;
      child_in[bsl] = bi;
    }
    // wide indices for the internal children, in slot order
    int n_inner = 0;
    for (int i = 0; i < n; ++i) n_inner += (ch[i].ref & kLeafBit) ? 0 : 1;
    uint32_t base = 0;
    if (n_inner > 0) {
      base = atomicAdd(&ctl[2], (unsigned int)n_inner);
      if (base + (uint32_t)n_inner > cap) {
        atomicAdd(&ctl[4], 1u);
        continue;
      }
    }
    WideNode out;
    for (int k = 0; k < 24; ++k) out.w[k] = 0u;
    uint32_t leafmask = 0u;
    int j = 0;
    for (int sl = 0; sl < kWide; ++sl) {
      const int i = child_in[sl];
      uint32_t qlo[3] = {255u, 255u, 255u}, qhi[3] = {0u, 0u, 0u};
      uint32_t ref = kNoChild;
      if (i < 0) {
        leafmask |= 1u << sl;
      } else {
        ref = ch[i].ref;
        if (ref & kLeafBit) {
          leafmask |= 1u << sl;
        } else {
          const uint32_t wi = base + (uint32_t)j++;
          w2b[wi] = ref;
          const uint32_t nd = need[w] + (uint32_t)(n_inner - 1);
          need[wi] = nd;
          atomicMax(&ctl[3], nd);
          ref = wi;
        }
        for (int a = 0; a < 3; ++a) {
          const double s = ldexp(1.0, e[a]);
          const double ql = floor(((double)ch[i].lo[a] - p[a]) / s), qh = ceil(((double)ch[i].hi[a] - p[a]) / s);
          qlo[a] = (uint32_t)fmin(fmax(ql, 0.0), 255.0);
          qhi[a] = (uint32_t)fmin(fmax(qh, 0.0), 255.0);
        }
      }
      out.w[4 + sl] = ref;
      const int word = sl >> 2, sh = 8 * (sl & 3);
      for (int a = 0; a < 3; ++a) {
        out.w[12 + 2 * a + word] |= qlo[a] << sh;
        out.w[18 + 2 * a + word] |= qhi[a] << sh;
      }
    }
    for (int a = 0; a < 3; ++a) out.w[a] = __float_as_uint((float)p[a]);
    out.w[3] = (uint32_t)(e[0] + 127) | ((uint32_t)(e[1] + 127) << 8) | ((uint32_t)(e[2] + 127) << 16) |
               (leafmask << 24);
    wn[w] = out;
  }
}

__global__ void wide_advance_kernel(unsigned int* ctl) {
  ctl[0] = ctl[1];
  ctl[1] = ctl[2];
}

__global__ void wide_init_kernel(uint32_t* w2b, uint32_t* need, unsigned int* ctl) {
  w2b[0] = 0u;  // the binary root is internal node 0
  need[0] = 0u;
  ctl[0] = 0u;
  ctl[1] = 1u;
  ctl[2] = 1u;
  ctl[3] = 0u;
  ctl[4] = 0u;
}

}  // namespace

bool wants_wide(const rtg_context* ctx) {
  return ctx->node_width == RTG_NODES_WIDE || (ctx->node_width == RTG_NODES_AUTO && outgrows_l2(ctx));
}

int ensure_wide(rtg_context* ctx) {
  const Geometry& g = ctx->g;
  if (g.wide_current || g.nd + g.nt == 0 || !g.nodes.p || !wants_wide(ctx)) return RTG_OK;
  return build_wide(ctx, ctx->stream);
}

int build_wide(rtg_context* ctx, cudaStream_t st) {
  Geometry& g = ctx->g;
  const int64_t np = g.nd + g.nt;
  g.n_wnodes = 0;
  g.wide_stack = 0;
  g.wide_current = false;
  if (np <= 0) return RTG_OK;
  const uint32_t n_bin = (uint32_t)(np > 1 ? np - 1 : 1);  // binary internal nodes (one for a single primitive)
  RTG_TRY(dalloc(ctx, g.wnodes, (size_t)n_bin, "wide tree"));
  DBuf<uint32_t> w2b, need;
  DBuf<unsigned int> ctl;
  auto cleanup = [&]() { tfree(w2b, st); tfree(need, st); tfree(ctl, st); };
  int rc = talloc(ctx, w2b, n_bin, st, "wide collapse");
  if (rc == RTG_OK) rc = talloc(ctx, need, n_bin, st, "wide collapse");
  if (rc == RTG_OK) rc = talloc(ctx, ctl, kCtlWords, st, "wide collapse");
  if (rc != RTG_OK) {
    cleanup();
    return rc;
  }
  wide_init_kernel<<<1, 1, 0, st>>>(w2b.p, need.p, ctl.p);
  // every wide level descends at least one binary level
  const int levels = (g.depth > 0 ? g.depth : 1) + 1;
  const unsigned blocks = (unsigned)std::min<int64_t>((n_bin + 127) / 128, 152 * 8);
  for (int l = 0; l < levels; ++l) {
    wide_level_kernel<<<blocks, 128, 0, st>>>(g.nodes.p, n_bin, g.wnodes.p, w2b.p, need.p, ctl.p, n_bin);
    wide_advance_kernel<<<1, 1, 0, st>>>(ctl.p);
  }
  unsigned int h[kCtlWords] = {0, 0, 0, 0, 0};
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, ctl.p, sizeof h, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return check_cuda(ctx, e, "wide tree");
  if (h[0] != h[2]) return set_error(ctx, RTG_ERR_INTERNAL, "wide tree deeper than the binary tree");
  g.wide_current = true;
  if (h[4] != 0) return RTG_OK;  // a node too wide for the byte grid: closest hits use the binary tree
  g.n_wnodes = h[2];
  g.wide_stack = (int32_t)h[3];
  return RTG_OK;
}

}  // namespace rtg
