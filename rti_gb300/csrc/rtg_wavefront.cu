// rtg_wavefront.cu -- wavefront scheduling of the forward paths.
//
// The same paths as the megakernel (same Philox counters, same arithmetic,
// hence the same deposits), scheduled differently: up to `capacity` paths wait
// in a queue in device memory, and each wave advances every queued path by one
// segment with two kernels --
//   extend: new source rays fill the free queue slots, then one closest-hit
//           query per queued path (hits stored per slot);
//   shade:  boundary wrap/mirror, back-face pass-through, deposits, roulette and
//           re-emission (tracer.hpp:169-279); surviving paths are compacted into
//           the other queue buffer with one atomic per warp.
// The last block of each shade launch schedules the next wave (queue length,
// first ray id and count of new rays) in a small control array, so waves run
// back to back without the host; the host only checks for the end every few
// waves.  Queue slot layout (SoA, two buffers): float4 (o, w), float4 (d, k
// bits), uint4 (ray id lo, ray id hi, job, segments so far).
#include <algorithm>

#include "rtg_path.cuh"

namespace rtg {

namespace {

enum : int {
  kCtlCur = 0,       // paths queued for this wave (before new rays)
  kCtlNext = 1,      // compaction counter of the next queue
  kCtlGenBase = 2,   // first global ray index generated this wave
  kCtlGenCount = 3,  // new rays this wave
  kCtlDone = 4,      // finished shade blocks
  kCtlNextRay = 5,   // next global ray index to generate
  kCtlTotal = 6,     // total rays
  kCtlCap = 7,       // queue capacity
  kCtlWords = 8
};

struct WfBufs {
  float4* ow[2];
  float4* dk[2];
  uint4* meta[2];
  float* ht;
  int32_t* hid;
  uint32_t* href;
  unsigned long long* ctl;
};

__device__ __forceinline__ int find_job(const uint64_t* __restrict__ prefix, int njobs, uint64_t j) {
  int lo = 0, hi = njobs - 1;  // last job whose first id <= j
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&prefix[mid]) <= j) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void flush_counts(DevTally* t, unsigned long long c_hit, unsigned long long c_non,
                                             unsigned long long c_tot, unsigned long long c_seg,
                                             unsigned long long c_trunc, unsigned long long c_nb,
                                             unsigned long long c_err) {
  __syncwarp();
  c_hit = warp_sum(c_hit);
  c_non = warp_sum(c_non);
  c_tot = warp_sum(c_tot);
  c_seg = warp_sum(c_seg);
  c_trunc = warp_sum(c_trunc);
  c_nb = warp_sum(c_nb);
  c_err = warp_sum(c_err);
  if ((threadIdx.x & 31) == 0) {
    if (c_hit) atomicAdd(&t->hitc, c_hit);
    if (c_non) atomicAdd(&t->nonhitc, c_non);
    if (c_tot) atomicAdd(&t->total, c_tot);
    if (c_seg) atomicAdd(&t->segments, c_seg);
    if (c_trunc) atomicAdd(&t->truncated, c_trunc);
    if (c_nb) atomicAdd(&t->nb_deposits, c_nb);
    if (c_err) atomicAdd(&t->errors, c_err);
  }
}

template <int TPB, int STACK>
__global__ void __launch_bounds__(TPB) wf_extend_kernel(const TraceParams* __restrict__ jobs,
                                                        const uint64_t* __restrict__ prefix, int njobs, WfBufs b,
                                                        int cur, DevTally* tally) {
  const uint64_t n_cur = b.ctl[kCtlCur], gen = b.ctl[kCtlGenCount], base = b.ctl[kCtlGenBase];
  const uint64_t n = n_cur + gen;
  unsigned long long c_seg = 0, c_err = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * TPB + threadIdx.x; i < n; i += (uint64_t)gridDim.x * TPB) {
    f3 o, d;
    const TraceParams* pp;
    if (i >= n_cur) {
      // source.hpp:20-58 with rectangle_origin_z / (power_)cosine_direction_z
      const uint64_t j = base + (i - n_cur);
      const int job = find_job(prefix, njobs, j);
      pp = jobs + job;
      const uint64_t id = pp->ray_begin + (j - __ldg(&prefix[job]));
      const uint4 u = draw4(pp->seed, id, 0xFFFFFFFFu, pp->job);
      const float r1 = u01_co(u.x), r2 = u01_co(u.y);
      o = mk3(pp->src_lo[0] + (pp->src_hi[0] - pp->src_lo[0]) * r1,
              pp->src_lo[1] + (pp->src_hi[1] - pp->src_lo[1]) * r2, pp->box_hi[2]);
      d = source_dir(pp->source_exponent, pp->source_ee, u.z, u.w);
      b.ow[cur][i] = make_float4(o.x, o.y, o.z, 1.0f);
      b.dk[cur][i] = make_float4(d.x, d.y, d.z, __uint_as_float(0u));
      b.meta[cur][i] = make_uint4((uint32_t)id, (uint32_t)(id >> 32), (uint32_t)job, 1u);
    } else {
      const float4 a = b.ow[cur][i], c = b.dk[cur][i];
      o = mk3(a.x, a.y, a.z);
      d = mk3(c.x, c.y, c.z);
      pp = jobs + b.meta[cur][i].z;
    }
    c_seg += 1;
    float th;
    int hid;
    uint32_t href;
    const bool hit = closest_hit<STACK, false>(pp->s, o, d, pp->tnear, th, hid, href, c_err);
    b.ht[i] = th;
    b.hid[i] = hit ? hid : -1;
    b.href[i] = href;
  }
  flush_counts(tally, 0, 0, 0, c_seg, 0, 0, c_err);
}

template <int TPB>
__global__ void __launch_bounds__(TPB) wf_shade_kernel(const TraceParams* __restrict__ jobs, WfBufs b, int cur,
                                                       DevTally* tally) {
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int nxt = cur ^ 1;
  const uint64_t n = b.ctl[kCtlCur] + b.ctl[kCtlGenCount];
  unsigned long long c_hit = 0, c_non = 0, c_tot = 0, c_trunc = 0, c_nb = 0, c_err = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * TPB + threadIdx.x; i < n; i += (uint64_t)gridDim.x * TPB) {
    const float4 a = b.ow[cur][i], c = b.dk[cur][i];
    const uint4 m = b.meta[cur][i];
    f3 o = mk3(a.x, a.y, a.z), d = mk3(c.x, c.y, c.z);
    float w = a.w;
    uint32_t k = __float_as_uint(c.w), nseg = m.w;
    const uint64_t id = (uint64_t)m.x | ((uint64_t)m.y << 32);
    const TraceParams* pp = jobs + m.z;
    const float th = b.ht[i];
    const int hid = b.hid[i];
    const uint32_t href = b.href[i];
    bool cont = false;
    float tb = 0.0f;
    const int axis = boundary_exit(*pp, o, d, tb);
    if (kChecked && hid >= pp->s.nd + pp->s.nt) {  // a bad hit id ends the path, counted
      c_err += 1;
    } else if (hid >= 0 && (axis < 0 || th <= tb)) {
      float4 nn;
      if (href & kTriBit) nn = __ldg(&pp->s.tri[4 * (int64_t)(href & kSlotMask) + 3]);
      else nn = __ldg(&pp->s.disc[2 * (int64_t)(href & kSlotMask) + 1]);
      const f3 nv = mk3(nn.x, nn.y, nn.z);
      const f3 hp = mk3(o.x + d.x * th, o.y + d.y * th, o.z + d.z * th);
      if (d.x * nv.x + d.y * nv.y + d.z * nv.z > 0.0f) {  // back face: pass through (tracer.hpp:216-227)
        o = hp;
        cont = true;
      } else {
        c_hit += 1;
        const float st = pp->s.sticking_field ? __ldg(&pp->s.sticking_field[hid]) : pp->sticking;
        const float v = w * st;
        deposit(*pp, hid, v);
        c_tot += 1;
        if (!(href & kTriBit) && pp->s.nb_ptr) {  // tracer.hpp:339-383
          const int64_t q0 = __ldg(&pp->s.nb_ptr[hid]), q1 = __ldg(&pp->s.nb_ptr[hid + 1]);
          for (int64_t q = q0; q < q1; ++q) {
            const uint32_t ns = __ldg(&pp->s.nb_slot[q]);
            if (kChecked && ns >= (uint32_t)pp->s.nd) {
              c_err += 1;
              continue;
            }
            float4 cr, nb_n;  // the neighbour's slot record
            asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                : "=f"(cr.x), "=f"(cr.y), "=f"(cr.z), "=f"(cr.w), "=f"(nb_n.x), "=f"(nb_n.y), "=f"(nb_n.z),
                  "=f"(nb_n.w)
                : "l"(pp->s.disc + 2 * (int64_t)ns));
            const int nb = __float_as_int(nb_n.w);
            if (kChecked && (unsigned)nb >= (unsigned)pp->s.nd) {
              c_err += 1;
              continue;
            }
            if (local_intersect(o, d, mk3(cr.x, cr.y, cr.z), cr.w, mk3(nb_n.x, nb_n.y, nb_n.z))) {
              deposit(*pp, nb, v);
              c_tot += 1;
              c_nb += 1;
            }
          }
        }
        w = w - v;
        if (w != 0.0f) {
          const uint4 u = draw4(pp->seed, id, k, pp->job);
          // rejection_control::check_weight_reweight_or_kill (rejection_control.hpp:28-61)
          const double lower = pp->roulette_threshold * 1.0f;
          const double renew = pp->roulette_weight * 1.0f;
          bool killed = false;
          if (!((double)w >= lower)) {
            const double kill = 1.0f - (double)w / renew;
            if ((double)u.x < kill * 4294967296.0) killed = true;
            else w = (float)renew;
          }
          if (!killed) {
            const bool spec = pp->reflection == RTG_REFLECT_SPECULAR ||
                              (pp->reflection == RTG_REFLECT_MIXED &&
                               (double)u.w < (double)pp->specular_fraction * 4294967296.0);
            d = spec ? specular_dir(nv, d) : diffuse_dir(nv, u.y, u.z);
            o = hp;
            k += 1;
            cont = true;
          }
        }
      }
    } else if (axis >= 0) {  // boundary_x_y::process_hit (boundary_x_y.hpp:92-143)
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
      cont = true;
    } else {
      c_non += 1;
    }
    if (cont) {  // the next segment, unless the path has used its budget
      if (nseg == pp->max_segments) {
        c_trunc += 1;
        cont = false;
      } else {
        nseg += 1;
      }
    }
    const unsigned act = __activemask();
    const unsigned want = __ballot_sync(act, cont);
    const int leader = __ffs(act) - 1;
    unsigned long long slot = 0;
    if (lane == leader && want) slot = atomicAdd(&b.ctl[kCtlNext], (unsigned long long)__popc(want));
    slot = __shfl_sync(act, slot, leader);
    if (cont) {
      slot += (unsigned long long)__popc(want & lt_mask);
      b.ow[nxt][slot] = make_float4(o.x, o.y, o.z, w);
      b.dk[nxt][slot] = make_float4(d.x, d.y, d.z, __uint_as_float(k));
      b.meta[nxt][slot] = make_uint4(m.x, m.y, m.z, nseg);
    }
  }
  flush_counts(tally, c_hit, c_non, c_tot, 0, c_trunc, c_nb, c_err);
  // the last block to finish schedules the next wave
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long done = atomicAdd(&b.ctl[kCtlDone], 1ull);
    if (done == (unsigned long long)gridDim.x - 1) {
      __threadfence();
      volatile unsigned long long* ctl = b.ctl;
      const unsigned long long queued = ctl[kCtlNext];
      const unsigned long long room = ctl[kCtlCap] - queued;
      const unsigned long long next = ctl[kCtlNextRay], total = ctl[kCtlTotal];
      const unsigned long long gen = total - next < room ? total - next : room;
      ctl[kCtlCur] = queued;
      ctl[kCtlNext] = 0;
      ctl[kCtlGenBase] = next;
      ctl[kCtlGenCount] = gen;
      ctl[kCtlNextRay] = next + gen;
      ctl[kCtlDone] = 0;
      __threadfence();
    }
  }
}

__global__ void wf_mark_abort(DevTally* t) { t->abort_seen = 1u; }

using ExtendKernel = void (*)(const TraceParams*, const uint64_t*, int, WfBufs, int, DevTally*);
using ShadeKernel = void (*)(const TraceParams*, WfBufs, int, DevTally*);

template <int TPB>
ExtendKernel extend_for(int stack) {
  if (stack <= 32) return wf_extend_kernel<TPB, 32>;
  if (stack <= 64) return wf_extend_kernel<TPB, 64>;
  return wf_extend_kernel<TPB, 256>;
}

}  // namespace

void free_wavefront(Wavefront& wf) {
  for (int q = 0; q < 2; ++q) {
    dfree(wf.ow[q]);
    dfree(wf.dk[q]);
    dfree(wf.meta[q]);
  }
  dfree(wf.hit_t);
  dfree(wf.hit_id);
  dfree(wf.hit_ref);
  dfree(wf.ctl);
  dfree(wf.one_job);
  dfree(wf.one_prefix);
  if (wf.h_ctl) cudaFreeHost(wf.h_ctl);
  wf.h_ctl = nullptr;
  wf.capacity = 0;
}

int launch_wavefront(rtg_context* ctx, const TraceParams& p0, const TraceParams* d_jobs, const uint64_t* d_prefix,
                     int njobs, uint64_t total_rays, cudaStream_t st, const rtg_launch_config& lc,
                     int tree_depth) {
  if (total_rays == 0) return RTG_OK;
  Wavefront& wf = ctx->wf;
  constexpr uint64_t kMaxCapacity = 1u << 20;
  uint64_t cap = std::min<uint64_t>(kMaxCapacity, (total_rays + 1023) / 1024 * 1024);
  if (wf.capacity < cap) {
    wf.capacity = 0;  // until every queue has the new size (an allocation may fail half way)
    for (int q = 0; q < 2; ++q) {
      RTG_TRY(dalloc(ctx, wf.ow[q], (size_t)cap, "wavefront queue"));
      RTG_TRY(dalloc(ctx, wf.dk[q], (size_t)cap, "wavefront queue"));
      RTG_TRY(dalloc(ctx, wf.meta[q], (size_t)cap, "wavefront queue"));
    }
    RTG_TRY(dalloc(ctx, wf.hit_t, (size_t)cap, "wavefront hits"));
    RTG_TRY(dalloc(ctx, wf.hit_id, (size_t)cap, "wavefront hits"));
    RTG_TRY(dalloc(ctx, wf.hit_ref, (size_t)cap, "wavefront hits"));
    wf.capacity = (uint32_t)cap;
  } else {
    cap = wf.capacity;
  }
  RTG_TRY(dalloc(ctx, wf.ctl, kCtlWords, "wavefront control"));
  if (!wf.h_ctl && cudaMallocHost((void**)&wf.h_ctl, kCtlWords * sizeof(unsigned long long)) != cudaSuccess) {
    wf.h_ctl = nullptr;
    cudaGetLastError();
    return set_error(ctx, RTG_ERR_OUT_OF_MEMORY, "pinned wavefront control");
  }
  WfBufs b;
  for (int q = 0; q < 2; ++q) {
    b.ow[q] = wf.ow[q].p;
    b.dk[q] = wf.dk[q].p;
    b.meta[q] = wf.meta[q].p;
  }
  b.ht = wf.hit_t.p;
  b.hid = wf.hit_id.p;
  b.href = wf.hit_ref.p;
  b.ctl = wf.ctl.p;
  const uint64_t gen0 = std::min<uint64_t>(cap, total_rays);
  unsigned long long* h = wf.h_ctl;
  h[kCtlCur] = 0;
  h[kCtlNext] = 0;
  h[kCtlGenBase] = 0;
  h[kCtlGenCount] = gen0;
  h[kCtlDone] = 0;
  h[kCtlNextRay] = gen0;
  h[kCtlTotal] = total_rays;
  h[kCtlCap] = cap;
  RTG_CUDA(ctx, cudaMemcpyAsync(wf.ctl.p, h, kCtlWords * sizeof(unsigned long long), cudaMemcpyHostToDevice, st));

  const int stack = stack_for(lc.stack_depth, tree_depth);
  int tpb = lc.threads_per_block;
  ExtendKernel ext = tpb == 64 ? extend_for<64>(stack) : tpb == 256 ? extend_for<256>(stack) : extend_for<128>(stack);
  ShadeKernel shd = tpb == 64 ? wf_shade_kernel<64> : tpb == 256 ? wf_shade_kernel<256> : wf_shade_kernel<128>;
  if (tpb != 64 && tpb != 256) tpb = 128;
  int sms = 0, per_e = 0, per_s = 0;
  RTG_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_e, ext, tpb, 0));
  RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_s, shd, tpb, 0));
  const uint64_t max_blocks = (cap + tpb - 1) / tpb;
  const unsigned ge = (unsigned)std::min<uint64_t>(max_blocks, (uint64_t)sms * std::max(per_e, 1));
  const unsigned gs = (unsigned)std::min<uint64_t>(max_blocks, (uint64_t)sms * std::max(per_s, 1));
  // Every wave advances each queued path by one segment and a path has at most
  // max_segments segments, so the loop ends.
  int chunk = 4;
  int cur = 0;
  for (;;) {
    for (int c = 0; c < chunk; ++c) {
      ext<<<ge, tpb, 0, st>>>(d_jobs, d_prefix, njobs, b, cur, p0.tally);
      shd<<<gs, tpb, 0, st>>>(d_jobs, b, cur, p0.tally);
      cur ^= 1;
    }
    RTG_CUDA(ctx, cudaGetLastError());
    RTG_CUDA(ctx, cudaMemcpyAsync(h, wf.ctl.p, kCtlWords * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    RTG_CUDA(ctx, cudaStreamSynchronize(st));
    if (h[kCtlCur] + h[kCtlGenCount] == 0) break;
    if (ctx->h_abort && *(volatile uint32_t*)ctx->h_abort) {
      wf_mark_abort<<<1, 1, 0, st>>>(p0.tally);
      RTG_CUDA(ctx, cudaGetLastError());
      break;
    }
    if (chunk < 16) chunk *= 2;
  }
  return RTG_OK;
}

}  // namespace rtg
