"""Benchmark: traced source rays per second on the triangle-mesh cylindrical hole.

Workload (one "step" = one trace of the whole ray batch): cylindrical hole of
radius 0.5 and depth 10 in a 2 x 2 x/y-periodic cell, 200,192 float32
triangles from a seeded structured tessellation with +-1 % vertex jitter,
cosine source (exponent 1) on the plane z = 0.1, sticking 0.01, 10 % specular /
90 % diffuse re-emission, 1e7 source rays per step.  Inputs are synthetic.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours: librtg on the GPU.  `value` = rays / device time of the traces with the
geometry resident in HBM (L2 flushed between steps by a 256 MB write);
`e2e` = the same metric through the public API from host arrays (geometry
upload + LBVH build + trace + reading counts and S1 back) per step.
reference: the CPU restatement of rti's tracer (oracle/) on all host cores,
each step a bounded sample of the same workload.
Under torchrun each rank traces its own ray range (weak scaling) and the
per-primitive accumulators are summed across ranks with NCCL.

Extra blocks of the ours line: `flux_1pct` = one trace of 4e8 rays of the same
workload, its rays/s and the median per-triangle relative error it reaches
(<= 1 %, rti's get_relative_error), beside the CPU oracle's rays/s on the same
workload; (rank 0, 1 GPU) `plain_gpu` = the same trace as
a non-persistent launch (one thread per source ray); `adjoint` = the adjoint
replay of the same trace; `batch` = 64 ragged trench/hole disc surfaces x 3
species x 2e6 rays in one autotuned, graph-replayed launch against 192
sequential plain launches and 192 sequential persistent launches;
`rough_field` = 4.2 M discs with a per-disc sticking field, 1e8 rays, forward
trace and the adjoint of all per-disc sticking gradients.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "traced rays/s"
UNIT = "rays/s"
N_RAYS = 10_000_000
STICKING = 0.01
SPECULAR = 0.1


def workload():
    from rti_gb300 import scenes
    return scenes.hole_triangles(radius=0.5, depth=10.0, cell=2.0, n_theta=512, n_wall=160, n_top=24, n_bottom=12,
                                 jitter=0.01, seed=0, source_gap=0.1)


TREE = "ploc"  # --tree: PLOC clustering traces the hole 4 % faster than the radix tree and builds in 1.8 ms
NODE_WIDTH = 0   # --node-width: 0 automatic (binary for this L2-resident hole), 2 binary, 8 wide


def set_tree(name, node_width=0):
    global TREE, NODE_WIDTH
    TREE = name
    NODE_WIDTH = node_width


def config_dict(h, n_rays):
    return {"workload": "hole_triangles", "radius": 0.5, "depth": 10.0, "cell": "2x2 periodic", "tree": TREE,
            "node_width": {0: "automatic", 2: "binary", 8: "8-wide"}[NODE_WIDTH],
            "n_triangles": int(h.n), "n_rays_per_step": int(n_rays), "sticking": STICKING,
            "specular_fraction": SPECULAR, "source_exponent": 1.0, "source_plane_z": 0.1,
            "l2": "flushed between steps (256 MB write)", "parallelism": "rays sharded per rank (weak scaling)"}


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_profile_line(key):
    """A per-launch byte count of the path kernel from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "trace_paths_hole.md")
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except OSError:
        pass
    return None


def read_traffic():
    return read_profile_line("traffic_bytes_per_launch")


def l2_copy_gbs(dev):
    """Copy bandwidth of a buffer pair that stays in L2 (2 x 24 MiB), best of 5
    runs of 50 copies, CUDA events on the current stream: read + write bytes."""
    import torch
    a = torch.empty(24 << 20, dtype=torch.uint8, device=dev)
    b = torch.empty_like(a)
    for _ in range(10):
        b.copy_(a)
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(50):
            b.copy_(a)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * a.numel() * 50 / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return best


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = max(mx, float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(h, n_rays, nthreads, seed=0):
    """Times the oracle on `n_rays` rays of the workload; returns rays/s."""
    from oracle import oracle as O
    s = O.Scene(tri_vertices=h.vertices, tri_indices=h.indices)
    cfg = O.make_config(h.box_lo, h.box_hi, sticking=STICKING, reflection=2, specular_fraction=SPECULAR, seed=seed)
    t0 = time.perf_counter()
    r = s.trace(cfg, 0, n_rays, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return n_rays / dt, r


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    h = workload()
    cores = os.cpu_count() or 1
    sample = args.ref_rays
    s = O.Scene(tri_vertices=h.vertices, tri_indices=h.indices)
    cfg = O.make_config(h.box_lo, h.box_hi, sticking=STICKING, reflection=2, specular_fraction=SPECULAR)
    for w in range(args.warmup):
        cfg.seed = 1000 + w
        s.trace(cfg, 0, sample, nthreads=cores)
    times = []
    for k in range(args.steps):
        cfg.seed = k
        t0 = time.perf_counter()
        s.trace(cfg, 0, sample, nthreads=cores)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = sample * args.steps / total
    # the configuration of the GPU arm (the same workload); each step times a
    # bounded sample of its source rays (rays/s does not depend on the sample
    # size on the CPU: no tail, per-thread paths)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 paths, f64 accumulators", "data": "synthetic",
            "impl": "reference", "config": config_dict(h, args.rays),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sample} of the {args.rays} source rays of a step (rays [0, {sample}) "
                                       "with the step's seed), all host threads; C restatement of rti's tracer "
                                       "(rti's Embree path does not build here)",
                             "sample_rays_per_step": sample, "host": host_info()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def host_info() -> dict:
    """The host CPU the baseline ran on: model, ISA, logical cores."""
    import platform
    model = ""
    try:  # lscpu names Arm cores too ("Neoverse-V2"); /proc/cpuinfo has no model name there
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.lower().startswith("model name"):
                        model = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"cpu_model": model or "unknown", "isa": platform.machine(), "nproc": os.cpu_count(),
            "build": "gcc -O3 -ffp-contract=off, OpenMP (oracle/Makefile)",
            "note": "C restatement of rti's tracer; rti's Embree path does not build here "
                    "(Embree 3.11 / VTK absent, x86-only intrinsics)"}


def run_batch_block(args):
    """64 ragged surfaces x 3 species, 2e6 rays per job: one batched launch vs
    192 back-to-back launches (plain, and persistent)."""
    from rti_gb300 import Engine, scenes
    from rti_gb300 import _lib as L
    from rti_gb300.batch import Batch
    t0 = time.perf_counter()
    inst = scenes.batch_instances(n=64, seed=0)
    engines, b = [], Batch(0)
    for s in inst:
        e = Engine(0)
        e.upload_discs(s.points, s.normals, s.radii)
        e.configure(box=(s.box_lo, s.box_hi), x_bound=1, y_bound=1, reset=True)
        engines.append(e)
        for stick, expo in scenes.BATCH_SPECIES:
            c = e.config()
            c.sticking, c.source_exponent = stick, expo
            b.add(e, args.batch_rays, seed=0, config=c)
    setup_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    tuned, _ = b.autotune(0.02)
    tune_s = time.perf_counter() - t0
    rays = len(b) * args.batch_rays

    def timed(fn, reps):
        out = []
        for _ in range(reps + 1):
            fn()
            out.append(b.synchronize())
        return statistics.mean(out[1:])

    batched_ms = timed(lambda: b.run(use_graph=True), 2)
    tb = b.tally()
    seq_ms = timed(b.run_sequential, 1)
    for e in engines:
        e.set_launch_config(scheduling=L.RTG_SCHED_PLAIN)
    plain_ms = timed(b.run_sequential, 1)
    tp = b.tally()
    for e in engines:
        e.close()
    b.close()
    ok = tb.segments == tp.segments and tb.hitc == tp.hitc and tb.errors == 0
    return {"workload": "64 trench/hole disc surfaces (aspect U[2,20], discs U[1e4,5e5], seeded) x 3 species "
                        "(s, n) in {(0.01,1), (0.1,5), (1,50)}, 2e6 rays per job, x/y periodic",
            "jobs": 192, "discs_total": int(sum(s.n for s in inst)), "rays": rays,
            "segments": tb.segments, "launch_config": tuned, "autotune_s": tune_s, "setup_s": setup_s,
            "batched_graph_ms": batched_ms, "batched_rays_per_s": rays / batched_ms * 1e3,
            "sequential_plain_ms": plain_ms, "sequential_plain_rays_per_s": rays / plain_ms * 1e3,
            "sequential_persistent_ms": seq_ms, "sequential_persistent_rays_per_s": rays / seq_ms * 1e3,
            "speedup_vs_plain_launches": plain_ms / batched_ms,
            "speedup_vs_persistent_launches": seq_ms / batched_ms,
            "same_results": bool(ok)}


def run_rough_block(args):
    """2048 x 2048 discs on a Gaussian height field with a per-disc sticking
    field, 1e8 rays: forward trace and the adjoint dL/ds_j of the bottom-quarter
    flux (held estimator), both timed with CUDA events."""
    import torch

    from rti_gb300 import Engine, scenes
    from rti_gb300 import _lib as L
    r = scenes.rough_discs(n=2048, spacing=0.01, rms=0.05, corr=0.2, seed=0)
    rng = np.random.default_rng(1)
    field = (1.0 / (1.0 + np.exp(-rng.normal(-2.0, 0.5, r.n)))).astype(np.float32)
    dev = torch.device("cuda", 0)
    rays = args.rough_rays
    with Engine(0) as e:
        e.set_tree_builder(L.RTG_TREE_PLOC)
        e.set_node_width(NODE_WIDTH)
        t0 = time.perf_counter()
        e.upload_discs(r.points, r.normals, r.radii)
        build_s = time.perf_counter() - t0
        e.configure(box=(r.box_lo, r.box_hi), x_bound=1, y_bound=1, reset=True)
        cs = torch.cuda.current_stream(dev).cuda_stream  # the events below are recorded on this stream
        f_dev = torch.from_numpy(field).to(dev)
        e.set_sticking_field_device(f_dev.data_ptr(), r.n, cs)
        z = r.points[:, 2]
        g = torch.from_numpy((z < np.quantile(z, 0.25)).astype(np.float64)).to(dev)
        fg = torch.zeros(r.n, dtype=torch.float64, device=dev)
        sc = torch.zeros(2, dtype=torch.float64, device=dev)

        def timed(fn, reps=2):
            out = []
            for k in range(reps + 1):
                a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a0.record()
                fn(k)
                a1.record()
                torch.cuda.synchronize()
                if k > 0:
                    out.append(a0.elapsed_time(a1))
            return statistics.mean(out)

        fwd_ms = timed(lambda k: e.trace(rays, seed=k, stream=cs))
        t = e.tally()
        used_width = "8-wide" if NODE_WIDTH == 8 or (NODE_WIDTH == 0 and e.uses_wide_tree) else "binary"
        adj_ms = timed(lambda k: e.adjoint_device(g.data_ptr(), 0, rays, k, fg.data_ptr(), sc.data_ptr(),
                                                  unbiased=False, stream=cs))
    return {"workload": "2048^2 discs on a Gaussian height field (rms 0.05, corr 0.2, spacing 0.01), per-disc "
                        "sticking logistic(N(-2,0.5)), cosine source, x/y periodic; L = flux onto the lowest "
                        "quarter of the discs",
            "discs": int(r.n), "rays": rays, "tree": "PLOC", "node_width": used_width, "build_s": build_s,
            "forward_ms": fwd_ms, "rays_per_s": rays / fwd_ms * 1e3, "segments": t.segments,
            "adjoint_field_ms": adj_ms, "adjoint_over_forward": adj_ms / fwd_ms,
            "grad_evals_per_s": 1e3 / (fwd_ms + adj_ms), "errors": t.errors}


def run_ours(args):
    import torch
    import torch.distributed as dist

    from rti_gb300 import Engine
    from rti_gb300 import _lib as L

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    h = workload()
    R = args.rays
    eng = Engine(local)
    tree = L.RTG_TREE_PLOC if TREE == "ploc" else L.RTG_TREE_KARRAS
    eng.set_tree_builder(tree)
    eng.set_node_width(NODE_WIDTH)
    eng.upload_triangles(h.vertices, h.indices)
    eng.configure(box=(h.box_lo, h.box_hi), sticking=STICKING, reflection=2, specular_fraction=SPECULAR,
                  x_bound=1, y_bound=1, source_exponent=1.0)
    if args.sweep:
        return ray_sweep(eng, [int(float(x)) for x in args.sweep.split(",")])
    # one dedicated stream for the flush, the events and librtg's kernels
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    acc = cnt = None
    if world > 1:
        from rti_gb300.sharding import allreduce_results, device_accumulators, ray_range
        acc, cnt = device_accumulators(eng)  # in-place views of the device accumulators
        assert ray_range(rank, world, R) == (rank * R, (rank + 1) * R)

    def step(k):
        eng.trace(R, seed=k, stream=stream.cuda_stream, ray_begin=rank * R)
        if world > 1:
            allreduce_results(acc, cnt)  # the path's one exchange: the sum of the accumulators

    for w in range(args.warmup):
        flush.zero_()
        step(10_000 + w)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kernel_ms, segs, tallies = [], 0, []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            step(k)
            ev[k][1].record(stream)
            t = eng.tally()  # synchronises; read outside the event pair
            kernel_ms.append(t.kernel_ms)
            tallies.append(t)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        wall = time.perf_counter() - t0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_s = sum(step_ms) / 1e3
    if world > 1:
        tt = torch.tensor([dev_s], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        dev_s = float(tt.item())
    value = world * R * args.steps / dev_s
    clocks = clk.summary()

    # roofline of the path kernel: algorithmic bytes per launch / its event time
    seg = statistics.mean(t.segments for t in tallies)
    dep = statistics.mean(t.hitc + t.nb_deposits for t in tallies)
    levels = math.ceil(math.log2(max(h.n / 4, 2)))
    prim_bytes = 48
    alg_bytes = seg * (64 + 64 * levels + 4 * prim_bytes) + 16 * dep
    kms = statistics.mean(kernel_ms)
    achieved = alg_bytes / (kms / 1e3) / 1e9
    peak, peak_kind = read_peaks()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": read_traffic(), "peak_source": peak_kind, "kernel": "trace_paths_kernel",
            "kernel_ms": kms, "segments_per_launch": seg, "alg_bytes_per_launch": alg_bytes,
            "bytes_per_segment_model": f"64 + 64*{levels} + 4*{prim_bytes} (+16 per deposit)"}

    # the same launch against the L2 roof (the tree and triangles are L2-resident):
    # L2 bytes from ncu (lts__t_sectors.sum x 32 of a full-size launch) over the
    # kernel's event time, against a measured L2-resident copy
    l2_bytes = read_profile_line("l2_bytes_per_launch")
    l2_peak = l2_copy_gbs(dev)
    roof_l2 = {"bound": "l2", "peak": l2_peak, "peak_source": "measured here: 2 x 24 MiB device copy",
               "unit": "GB/s", "traffic": l2_bytes,
               "achieved": (l2_bytes / (kms / 1e3) / 1e9) if l2_bytes else None,
               "frac": (l2_bytes / (kms / 1e3) / 1e9 / l2_peak) if l2_bytes else None}

    # end to end through the public API from host arrays
    e2e = None
    if not args.no_e2e:
        pin_v = torch.from_numpy(h.vertices).pin_memory().numpy()
        pin_i = torch.from_numpy(h.indices.view(np.int32)).pin_memory().numpy().view(np.uint32)
        pin_c = torch.zeros(h.n, dtype=torch.int64).pin_memory().numpy().view(np.uint64)
        pin_s = torch.zeros(h.n, dtype=torch.float64).pin_memory().numpy()
        def e2e_step(e2, k):
            e2.set_tree_builder(tree)
            e2.set_node_width(NODE_WIDTH)
            e2.upload_triangles(pin_v, pin_i)
            e2.configure(box=(h.box_lo, h.box_hi), sticking=STICKING, reflection=2, specular_fraction=SPECULAR,
                         x_bound=1, y_bound=1)
            e2.trace(R, seed=k, ray_begin=rank * R)
            e2.hit_counts(out=pin_c)
            e2.values(out=pin_s)

        # a caller that keeps its context (a simulator tracing a new surface every time step) ...
        e2e_times = []
        with Engine(local) as e2:
            for k in range(args.e2e_steps + 1):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                e2e_step(e2, k)
                dt = time.perf_counter() - t0
                if k > 0:
                    e2e_times.append(dt)
        # ... and one that creates and destroys a context around every trace
        fresh_times = []
        for k in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            with Engine(local) as e2:
                e2e_step(e2, k)
            dt = time.perf_counter() - t0
            if k > 0:
                fresh_times.append(dt)
        np_ = h.n
        e2e = {"value": world * R / statistics.mean(e2e_times), "unit": UNIT,
               "h2d_bytes_per_step": int(12 * len(h.vertices) + 12 * h.n),
               "d2h_bytes_per_step": int(16 * np_),
               "includes": "per step: upload of the surface from pinned host arrays (checks, LBVH build), "
                           "configuration, trace, hit counts + S1 read back into pinned host arrays, on a "
                           "context kept across steps" + ("; per rank, without the cross-rank sum" if world > 1
                                                          else ""),
               "fresh_context_value": world * R / statistics.mean(fresh_times),
               "fresh_context_includes": "the same with a context created and destroyed every step"}

    # adjoint replay (d/d sticking and d/d exponent of the bottom-quarter flux)
    adj = None
    if not args.no_adjoint:
        V = h.vertices.astype(np.float64)
        zc = V[h.indices].mean(axis=1)[:, 2]
        g = torch.from_numpy((zc < -0.75 * h.meta["depth"]).astype(np.float64)).to(dev)
        sc = torch.zeros(2, dtype=torch.float64, device=dev)
        t_adj = []
        for k in range(args.warmup + 3):
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.zero_()
            a0.record(stream)
            eng.adjoint_device(g.data_ptr(), rank * R, (rank + 1) * R, k, 0, sc.data_ptr(), unbiased=True,
                               stream=stream.cuda_stream)
            a1.record(stream)
            torch.cuda.synchronize()
            if k >= args.warmup:
                t_adj.append(a0.elapsed_time(a1))
        fwd_ms = statistics.mean(step_ms)
        adj_ms = statistics.mean(t_adj)
        adj = {"workload": "bottom-quarter flux of the same hole, d/d sticking (unbiased) and d/d exponent",
               "adjoint_ms": adj_ms, "forward_ms": fwd_ms, "adjoint_over_forward": adj_ms / fwd_ms,
               "grad_evals_per_s": 1e3 / (fwd_ms + adj_ms), "rays_per_grad_eval": R}

    # Monte Carlo error of the timed trace (hit_accumulator::get_relative_error
    # per primitive): the metric is quoted at <= 1 % flux error, so report the
    # error reached and the rays a 1 % median error needs (error ~ 1/sqrt(rays))
    rel = eng.relative_error()
    hitm = eng.hit_counts() > 0
    med = float(np.median(rel[hitm])) if hitm.any() else None
    flux_err = {"median_relative_error": med,
                "p90_relative_error": float(np.quantile(rel[hitm], 0.9)) if hitm.any() else None,
                "primitives_hit": int(hitm.sum()), "primitives": int(len(rel)),
                "rays_for_1pct_median": int(R * (med / 0.01) ** 2) if med else None,
                "gpu_vs_cpu": "bit-identical hit counts and tallies (tests/test_gpu_parity.py)"}

    # the metric's "at <= 1 % flux error" point, measured: one trace of enough
    # rays that the median per-triangle relative error (rti's formula) is <= 1 %
    one_pct = None
    if not args.no_one_pct:
        r1 = args.rays_1pct
        o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.zero_()
        o0.record(stream)
        eng.trace(r1, seed=424242, stream=stream.cuda_stream, ray_begin=rank * r1)
        o1.record(stream)
        torch.cuda.synchronize()
        t1 = eng.tally()
        rel1 = eng.relative_error()
        hit1 = eng.hit_counts() > 0
        med1 = float(np.median(rel1[hit1])) if hit1.any() else None
        one_pct = {"rays": r1, "ms": o0.elapsed_time(o1), "rays_per_s": r1 / (o0.elapsed_time(o1) / 1e3),
                   "kernel_ms": t1.kernel_ms, "segments": t1.segments, "errors": t1.errors,
                   "median_relative_error": med1,
                   "p90_relative_error": float(np.quantile(rel1[hit1], 0.9)) if hit1.any() else None,
                   "primitives_hit": int(hit1.sum()), "primitives": int(len(rel1)),
                   "meets_1pct": bool(med1 is not None and med1 <= 0.01),
                   "error_formula": "hit_accumulator::get_relative_error per triangle, median over hit triangles"}

    # the plain GPU baseline: the same trace as a non-persistent launch
    plain = None
    if not args.no_plain:
        from rti_gb300 import _lib as L
        eng.set_launch_config(scheduling=L.RTG_SCHED_PLAIN)
        pm = []
        for k in range(args.warmup + 3):
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.zero_()
            p0.record(stream)
            eng.trace(R, seed=k, stream=stream.cuda_stream, ray_begin=rank * R)
            p1.record(stream)
            torch.cuda.synchronize()
            if k >= args.warmup:
                pm.append(p0.elapsed_time(p1))
        tp = eng.tally()
        eng.set_launch_config()
        plain = {"value": world * R / (statistics.mean(pm) / 1e3), "unit": UNIT, "ms_per_step": statistics.mean(pm),
                 "what": "one thread per source ray, non-persistent launch of the same path code",
                 "errors": tp.errors}

    batch = None
    if rank == 0 and world == 1 and not args.no_batch:
        batch = run_batch_block(args)
    rough = None
    if rank == 0 and world == 1 and not args.no_rough:
        rough = run_rough_block(args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rays_s, _ = cpu_sample(h, args.cpu_rays, os.cpu_count() or 1)
        cpu = {"value": rays_s, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{args.cpu_rays} source rays of the same workload, all host threads",
               "host": host_info()}
        if one_pct is not None:
            one_pct["cpu_rays_per_s"] = rays_s
            one_pct["cpu_seconds_for_the_same_rays"] = one_pct["rays"] / rays_s
            one_pct["gpu_over_cpu"] = one_pct["rays_per_s"] / rays_s
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 paths, f64 accumulators",
                "data": "synthetic", "config": config_dict(h, R), "clocks": clocks, "roofline": roof,
                "roofline_l2": roof_l2,
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 2 * args.steps, "adjoint": adj,
                "plain_gpu": plain, "batch": batch, "rough_field": rough, "flux_error": flux_err,
                "flux_1pct": one_pct,
                "wall_s_timed_region": wall,
                "tally_per_step": {"segments": seg, "hitc": statistics.mean(t.hitc for t in tallies),
                                   "truncated": max(t.truncated for t in tallies),
                                   "errors": max(t.errors for t in tallies)}}
        print(json.dumps(line))
    eng.close()
    if world > 1:
        dist.destroy_process_group()


def run_case(args):
    """Path-kernel time of one workload alone (the target of ncu captures):
    hole = the bench workload, trench = the 98,301-disc trench (width 1, depth
    5, 3 x 3 periodic cell, sticking 0.1, diffuse), rough = the 2048^2-disc
    height field with its per-disc sticking field (PLOC tree).  Two warm-up
    traces, then --steps traces of --rays rays; one JSON line."""
    from rti_gb300 import Engine, scenes
    from rti_gb300 import _lib as L
    if args.case == "batch":
        return run_batch_case(args)
    with Engine(0) as e:
        e.set_node_width(args.node_width)
        if args.case == "hole":
            h = workload()
            e.set_tree_builder(L.RTG_TREE_PLOC if TREE == "ploc" else L.RTG_TREE_KARRAS)
            e.upload_triangles(h.vertices, h.indices)
            e.configure(box=(h.box_lo, h.box_hi), sticking=STICKING, reflection=2, specular_fraction=SPECULAR,
                        x_bound=1, y_bound=1, reset=True)
        elif args.case == "trench":
            t = scenes.trench_discs()
            e.upload_discs(t.points, t.normals, t.radii)
            e.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
        else:
            r = scenes.rough_discs(n=2048, spacing=0.01, rms=0.05, corr=0.2, seed=0)
            e.set_tree_builder(L.RTG_TREE_PLOC)
            e.upload_discs(r.points, r.normals, r.radii)
            e.configure(box=(r.box_lo, r.box_hi), x_bound=1, y_bound=1, reset=True)
            rng = np.random.default_rng(1)
            e.set_sticking_field((1.0 / (1.0 + np.exp(-rng.normal(-2.0, 0.5, r.n)))).astype(np.float32))
        rows = []
        for k in range(2 + args.steps):
            e.trace(args.rays, seed=k)
            t_ = e.tally()
            if k >= 2:
                rows.append(t_)
        print(json.dumps({"case": args.case, "rays": args.rays, "node_width": args.node_width,
                          "kernel_ms": [round(t_.kernel_ms, 3) for t_ in rows], "segments": rows[-1].segments,
                          "hitc": rows[-1].hitc, "nb_deposits": rows[-1].nb_deposits, "errors": rows[-1].errors}))


def run_batch_case(args):
    """The batch block's 192 jobs (64 surfaces x 3 species, --batch-rays rays
    each) in one graph-replayed launch with the launch shape the autotuner
    picks for them (64 threads, 256-entry stack): two warm-up runs, then
    --steps timed runs; one JSON line.  The target of the batch's ncu captures."""
    from rti_gb300 import Engine, scenes
    from rti_gb300.batch import Batch
    inst = scenes.batch_instances(n=64, seed=0)
    engines, b = [], Batch(0)
    try:
        for s in inst:
            e = Engine(0)
            engines.append(e)
            e.set_node_width(args.node_width)
            e.upload_discs(s.points, s.normals, s.radii)
            e.configure(box=(s.box_lo, s.box_hi), x_bound=1, y_bound=1, reset=True)
            for stick, expo in scenes.BATCH_SPECIES:
                c = e.config()
                c.sticking, c.source_exponent = stick, expo
                b.add(e, args.batch_rays, seed=0, config=c)
        b.set_launch_config(threads_per_block=64, stack_depth=256)
        ms = []
        for k in range(2 + args.steps):
            b.run(use_graph=True)
            t = b.synchronize()
            if k >= 2:
                ms.append(t)
        tb = b.tally()
        print(json.dumps({"case": "batch", "jobs": len(b), "rays": len(b) * args.batch_rays,
                          "batched_ms": [round(x, 3) for x in ms], "segments": tb.segments, "hitc": tb.hitc,
                          "errors": tb.errors}))
    finally:
        b.close()
        for e in engines:
            e.close()


def ray_sweep(eng, sizes):
    """Path-kernel time (best of 3) against the number of rays on the bench
    workload, and the least-squares line T = tail + slope * rays: the intercept
    is the time the longest paths add after the throughput phase."""
    eng.trace(1_000_000, seed=0)
    rows = []
    for n in sizes:
        ks = []
        for k in range(3):
            eng.trace(n, seed=k + 1)
            ks.append(eng.tally().kernel_ms)
        rows.append((n, min(ks)))
    x = np.array([r[0] for r in rows], dtype=np.float64)
    y = np.array([r[1] for r in rows])
    slope, tail = np.polyfit(x, y, 1) if len(rows) > 1 else (float("nan"), float("nan"))
    print(json.dumps({"sweep": [{"rays": n, "kernel_ms": round(ms, 3)} for n, ms in rows],
                      "tail_ms": round(float(tail), 2), "ms_per_1e6_rays": round(float(slope) * 1e6, 4),
                      "rays_per_s_without_tail": 1e3 / float(slope) if slope > 0 else None}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rays", type=int, default=N_RAYS)
    ap.add_argument("--cpu-rays", type=int, default=2_000_000, help="CPU-baseline sample (ours arm)")
    ap.add_argument("--ref-rays", type=int, default=2_000_000,
                    help="source rays timed per step of the reference arm (a sample of the step's rays)")
    ap.add_argument("--e2e-steps", type=int, default=6)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-one-pct", action="store_true")
    ap.add_argument("--rays-1pct", type=int, default=400_000_000,
                    help="rays of the trace that measures the <= 1 %% flux-error point")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-rays", type=int, default=2_000_000, help="rays per job of the batch block")
    ap.add_argument("--no-rough", action="store_true")
    ap.add_argument("--tree", default=TREE, choices=["karras", "ploc"], help="tree builder of the hole")
    ap.add_argument("--sweep", default="", help="comma-separated ray counts: path-kernel time against rays "
                                                "(the tail analysis), printed instead of the bench line")
    ap.add_argument("--rough-rays", type=int, default=100_000_000, help="rays of the rough-surface block")
    ap.add_argument("--rough-only", action="store_true", help="run the rough-surface block alone and print it")
    ap.add_argument("--case", default="", choices=["", "hole", "trench", "rough", "batch"],
                    help="time the path kernel on one workload alone (--rays, --steps, --node-width)")
    ap.add_argument("--node-width", type=int, default=0, choices=[0, 2, 8],
                    help="tree of the closest-hit queries: 0 automatic, 2 binary, 8 compressed 8-wide")
    args = ap.parse_args()
    set_tree(args.tree, args.node_width)
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    from __graft_entry__ import build
    if args.impl == "reference":
        from oracle import oracle
        oracle.build()
        run_reference(args)
    elif args.case:
        build()
        run_case(args)
    elif args.rough_only:
        build()
        print(json.dumps(run_rough_block(args)))
    else:
        build()
        run_ours(args)


if __name__ == "__main__":
    main()
