#!/usr/bin/env python3
"""Benchmark of the GB300 VortonSim step.

Headline (one JSON line on rank 0): direct mollified Biot-Savart throughput in
G interactions/s on the direct-sum workload -- a seeded vortex ring of 4,096
vortons (major radius 1, tube radius 0.25, Gaussian core sigma 0.1, peak
vorticity 10, vorton radius 0.05); velocity by direct summation at every
vorton and at the 33^3 points of a 32^3-cell grid on [-1.5, 1.5]^3; vortons
advected by Euler at dt = 1/30; 65,536 tracers (uniform in [-1.5, 1.5)^3)
advected through the velocity grid.  A step is that whole pass; interactions
per step = 4,096 x (4,096 + 35,937).

Keys beyond the base contract:
  * "e2e": the same metric through the host-buffer C ABI (vg_step_advect: the
    step and PclOpEvolve on the reference's 96-byte Particle records, then the
    tracer records' advection, from pinned host memory, copies included; the
    same frame as two calls, vg_step_evolve + vg_advect, beside it);
  * "roofline": the direct-sum kernel against the FP32 pipe (2 flops x 128
    lanes x the device's SM count x the SM clock sampled during the run), 26 algorithmic
    flops per interaction;
  * "cpu_baseline": the reference's own direct sum (built from its sources,
    std::thread TBB stand-in, all host threads) on the same workload;
  * "poisson": the vector-potential solve to 1e-6 relative residual on the
    multigrid workload (262,144 puff vortons, 129^3 grid, dx = 1/32): plain
    multigrid ms per solve, cycles and residuals.

--impl reference times the reference's own CPU code for the same step
(oracle/_ref, or the C oracle when the reference was not built) on all host
threads; under torchrun only rank 0 runs it.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_VORTONS = 4096
GRID_POINTS = 33
N_TRACERS = 65536
DT = np.float32(1.0 / 30.0)
FLOPS_PER_INTERACTION = 26
METRIC = "Poisson ms @1e-6 resid: NN warm-start vs plain MG; direct Biot-Savart Gint/s"
WORKLOAD = ("direct-sum step: vortex ring, 4096 vortons, velocity at vortons + 33^3 gridpoints on [-1.5,1.5]^3, "
            "Euler advection of vortons and 65536 tracers, dt=1/30")


def interactions():
    return N_VORTONS * (N_VORTONS + GRID_POINTS ** 3)


def make_inputs():
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(N_VORTONS, seed=1)
    tr = workloads.tracers(N_TRACERS, seed=4, lo=-1.5, hi=1.5)
    return pos, w, s, tr


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.rows = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def max_over_ranks(x, world):
    """The largest x over the ranks (a step's time: the job waits for the slowest replica)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gint_per_s(interactions_per_rank, ms_per_step, world):
    """Replicas: every rank evaluates the same number of interactions per step;
    the job's throughput is their sum over the slowest rank's step time."""
    return world * interactions_per_rank / (ms_per_step * 1e-3) / 1e9


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- CPU legs

def reference_lib():
    """The reference's own code (multithreaded build) if it was built, else None."""
    import oracle
    os.environ.setdefault("NUMBER_OF_PROCESSORS", str(os.cpu_count() or 1))
    try:
        oracle.build()
    except Exception:
        pass
    if oracle.ref_available("mt"):
        L = oracle.ref("mt")
        L.vgref_set_threads(int(os.environ["NUMBER_OF_PROCESSORS"]))
        return L
    return None


def cpu_direct_rate(pos, w, s, q, budget_s=3.0):
    """Reference direct sum (vortonSim.cpp:1144-1158) on all host threads:
    returns (Gint/s, kind, cores, sample description)."""
    import oracle
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    L = reference_lib()
    out = np.zeros((len(q), 3), np.float32)
    reps, t0 = 0, time.perf_counter()
    if L is not None:
        cores = int(os.environ["NUMBER_OF_PROCESSORS"])
        kind = "reference"
        while True:
            L.vgref_direct(0, P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(q), ctypes.c_size_t(len(q)),
                           ctypes.c_float(1.0), ctypes.c_float(1.0), P(out))
            reps += 1
            if time.perf_counter() - t0 > budget_s:
                break
    else:
        cores, kind = 1, "port"
        qs = q[:2048]
        while True:
            oracle.direct(0, pos, w, s, qs)
            reps += 1
            if time.perf_counter() - t0 > budget_s:
                break
        q = qs
    dt = time.perf_counter() - t0
    rate = reps * len(pos) * len(q) / dt / 1e9
    return rate, kind, cores, f"{reps} x direct velocity, {len(pos)} sources x {len(q)} targets"


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    import oracle
    pos, w, s, tr = make_inputs()
    from vortegrid_gb300 import workloads
    q = np.concatenate([workloads.grid_points([-1.5] * 3, [3.0 / 32] * 3, [GRID_POINTS] * 3), pos]).astype(np.float32)
    L = reference_lib()
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    cores = int(os.environ.get("NUMBER_OF_PROCESSORS", "1")) if L is not None else 1
    kind = "reference" if L is not None else "port"
    g12 = np.array([-1.5, -1.5, -1.5, 3.0, 3.0, 3.0, 3.0 / 32, 3.0 / 32, 3.0 / 32, 32 / 3.0, 32 / 3.0, 32 / 3.0],
                   np.float32)
    np3 = np.array([GRID_POINTS] * 3, np.uint32)

    def step():
        vel = np.zeros((len(q), 3), np.float32)
        if L is not None:
            L.vgref_direct(0, P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(q), ctypes.c_size_t(len(q)),
                           ctypes.c_float(1.0), ctypes.c_float(1.0), P(vel))
            grid = np.ascontiguousarray(vel[: GRID_POINTS ** 3])
            p = pos + vel[GRID_POINTS ** 3:] * DT
            t = tr.copy()
            tv = np.zeros_like(t)
            L.vgref_advect(P(t), P(tv), ctypes.c_size_t(len(t)), P(g12), P(np3), P(grid), ctypes.c_float(DT))
        else:  # C oracle port, single thread, on a bounded sample of targets
            vel = oracle.direct(0, pos, w, s, q[:: max(1, len(q) // 4096)])
            p = pos
        return p

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    ms = el / args.steps * 1e3
    inter = interactions() if L is not None else N_VORTONS * len(q[:: max(1, len(q) // 4096)])
    value = inter / (ms * 1e-3) / 1e9
    sample = ("full step: direct velocity at 4096 vortons + 35937 gridpoints, tracer gather + Euler"
              if L is not None else "direct velocity on a 4096-target sample (C oracle, 1 thread)")
    line = {"metric": METRIC, "value": value, "unit": "Gint/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "l2": "n/a (CPU)"}, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "Gint/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "Gint/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm

def run_ours(args, world, rank, local):
    import torch

    import vortegrid_gb300 as vg

    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    pos, w, s, tr = make_inputs()
    grid = vg.GridGeom.make([-1.5] * 3, [3.0] * 3, [GRID_POINTS] * 3)
    cfg = vg.default_config(velocity_technique=vg.VELOCITY_DIRECT, fixed_grid=grid, enable_stretch=0,
                            enable_diffusion=0, device=local)
    cfg.stream = stream.cuda_stream
    ctx = vg.VortonSim(cfg=cfg)

    def f4(a, wv=None):
        o = np.zeros((len(a), 4), np.float32)
        o[:, :3] = a
        if wv is not None:
            o[:, 3] = wv
        return torch.from_numpy(o).cuda()

    ps0, w0, tr0 = f4(pos, s), f4(w), f4(tr)
    ps, ww, vel = ps0.clone(), w0.clone(), torch.zeros_like(ps0)
    trp, trv = tr0.clone(), torch.zeros_like(tr0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2

    def reset():  # the same inputs every step, restored before the step's events
        ps.copy_(ps0, non_blocking=True)
        ww.copy_(w0, non_blocking=True)
        trp.copy_(tr0, non_blocking=True)

    def step():  # the step with the vortons' Euler step, then the tracers' gather + Euler step
        ctx.UpdateAndEvolveDevice(ps, ww, vel, float(DT))
        ctx.AdvectDevice(trp, trv, float(DT))

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            reset()
            step()
        ctx.synchronize()
        stats = ctx.stats()
        launches_per_step = stats.kernels_launched + 1  # the step's kernels + the tracer advection
        barrier(world)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with ClockSampler(local) as clk:
            for k in range(args.steps):
                reset()
                flush.zero_()
                ev[k][0].record(stream)
                step()
                ev[k][1].record(stream)
            ctx.synchronize()
            torch.cuda.synchronize()
        barrier(world)
        ms_steps = [a.elapsed_time(b) for a, b in ev]
    ms_total = max_over_ranks(sum(ms_steps), world)
    ms_per_step = ms_total / args.steps
    value = whole_job_gint_per_s(interactions(), ms_per_step, world)

    result = {"metric": METRIC, "value": value, "unit": "Gint/s", "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
              "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
              "config": {"workload": WORKLOAD, "parallelism": "replicas" if world > 1 else "single GPU",
                         "l2": "flushed between timed steps (256 MB write, outside the per-step events)",
                         "numerics": "fast",
                         "parity": "FP64 direct-sum oracle, relative L2 ~1e-7 (tests/test_gpu_parity.py)"},
              "gpu_launches": launches_per_step * args.steps}
    if rank != 0:
        return
    result["clocks"] = clk.summary()

    # ---- roofline of the direct-sum kernel (events on the context stream): the step's own
    # velocity evaluation (vg_direct_grid_device: every gridpoint and vorton), then the same
    # kernel on arbitrary targets (vg_direct_device: 1M random points, no grid rows)
    lib = vg.lib()
    vgrid = torch.zeros((grid.capacity, 3), dtype=torch.float32, device="cuda")
    velv = torch.zeros_like(ps0)

    def time_launch(fn, reps=20):
        with torch.cuda.stream(stream):
            for _ in range(3):
                fn()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    kms = time_launch(lambda: ctx.check(lib.vg_direct_grid_device(ctx.h, ctypes.byref(grid), vg._ptr(ps0), vg._ptr(w0),
                                                                   N_VORTONS, vg._ptr(vgrid), vg._ptr(velv)),
                                        "vg_direct_grid_device"))
    achieved = FLOPS_PER_INTERACTION * interactions() / (kms * 1e-3) / 1e12
    clk_mhz = result["clocks"].get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    peak = 2 * 128 * sms * clk_mhz * 1e6 / 1e12
    result["roofline"] = {"bound": "fp32", "kernel": "k_direct_pair (grid-row and general CTAs) + k_reduce_pair, "
                                                     "as the step launches them (vg_direct_grid_device)",
                          "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                          "traffic": profiled_traffic("direct_pair_ring4096.md"), "ms_per_launch": kms,
                          "peak_basis": f"2 flops x 128 FP32 lanes x {sms} SMs (device attribute) x {clk_mhz:.0f} MHz "
                                        "(sampled median)",
                          "flops_per_interaction": FLOPS_PER_INTERACTION,
                          "gint_per_s_kernel": interactions() / (kms * 1e-3) / 1e9}
    m_arb = 1 << 20
    qa = f4(np.random.default_rng(9).uniform(-1.5, 1.5, (m_arb, 3)).astype(np.float32))
    oa = torch.zeros_like(qa)
    kms_a = time_launch(lambda: ctx.check(lib.vg_direct_device(ctx.h, 0, vg._ptr(ps0), vg._ptr(w0), N_VORTONS,
                                                               vg._ptr(qa), m_arb, 1.0, 1.0, vg._ptr(oa)),
                                          "vg_direct_device"), reps=5)
    ach_a = FLOPS_PER_INTERACTION * N_VORTONS * m_arb / (kms_a * 1e-3) / 1e12
    result["roofline_arbitrary_targets"] = {"targets": m_arb, "sources": N_VORTONS, "ms_per_launch": kms_a,
                                            "achieved": ach_a, "peak": peak, "unit": "TFLOP/s", "frac": ach_a / peak,
                                            "kernel": "k_direct_pair general CTAs (+ k_reduce_pair), "
                                                      "1M uniform random targets in [-1.5,1.5]^3"}

    # ---- e2e through the host-buffer ABI from pinned memory
    recs_t = torch.empty(N_VORTONS * 96, dtype=torch.uint8, pin_memory=True)
    recs = recs_t.numpy().view(vg.PARTICLE_DTYPE)
    recs0 = vg.make_particles(pos, w, s)
    trr_t = torch.empty(N_TRACERS * 96, dtype=torch.uint8, pin_memory=True)
    trr = trr_t.numpy().view(vg.PARTICLE_DTYPE)
    trr0 = vg.make_particles(tr)
    host = vg.VortonSim(cfg=cfg)

    def e2e_run(frame):
        ms = []
        for k in range(args.warmup + args.steps):
            recs[...] = recs0
            trr[...] = trr0
            t0 = time.perf_counter()
            frame(k)
            t1 = time.perf_counter()
            if k >= args.warmup:
                ms.append((t1 - t0) * 1e3)
        return statistics.mean(ms)
    # one frame of both groups through the public API: the vorton group's PclOpVortonSim + PclOpEvolve and
    # the tracer group's AssignVelocityFromField + Evolve (vg_step_advect: the tracer upload overlaps the step)
    e2e_step = e2e_run(lambda k: host.UpdateAndAdvect(recs, trr, float(DT), k, evolve=True))
    sep_step = e2e_run(lambda k: (host.UpdateAndEvolve(recs, float(DT), k), host.Advect(trr, float(DT))))
    result["e2e"] = {"value": interactions() / (e2e_step * 1e-3) / 1e9, "unit": "Gint/s",
                     # 96-byte records travel whole, one contiguous copy each way
                     "h2d_bytes_per_step": (N_VORTONS + N_TRACERS) * 96,
                     "d2h_bytes_per_step": (N_VORTONS + N_TRACERS) * 96, "ms_per_step": e2e_step,
                     "path": "vg_step_advect: the step and PclOpEvolve on the vorton records, then "
                             "AssignVelocityFromField + Evolve on the tracer records, pinned",
                     "separate_calls": {"value": interactions() / (sep_step * 1e-3) / 1e9, "ms_per_step": sep_step,
                                        "path": "vg_step_evolve, then vg_advect"}}

    # ---- CPU baseline (reference code, all host threads)
    from vortegrid_gb300 import workloads
    qc = np.concatenate([workloads.grid_points([-1.5] * 3, [3.0 / 32] * 3, [GRID_POINTS] * 3), pos]).astype(np.float32)
    rate, kind, cores, sample = cpu_direct_rate(pos, w, s, qc, budget_s=args.cpu_seconds)
    result["cpu_baseline"] = {"value": rate, "unit": "Gint/s", "cores": cores, "kind": kind, "sample": sample}

    # ---- Poisson solve to 1e-6 on the multigrid workload
    if not args.skip_poisson:
        result["poisson"] = poisson_section(vg, torch, stream, local)
        result["treecode"] = treecode_section(vg, torch, stream, local)
        result["batched"] = batched_section(torch, local)
        result["rows"] = rows_section(vg, torch, stream, local)
    print(json.dumps(result), flush=True)


def profiled_traffic(summary):
    """DRAM bytes (read + write) per launch recorded by the ncu summary under profiles/."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", summary)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def vg_grid_points(grid):
    import torch
    from vortegrid_gb300 import workloads
    p = workloads.grid_points(list(grid.min_corner), list(grid.cell_spacing), grid.points)
    o = np.zeros((len(p), 4), np.float32)
    o[:, :3] = p
    return torch.from_numpy(o).cuda()


def treecode_section(vg, torch, stream, local, steps=3):
    """Treecode workload: 65,536 vortons in 8 randomly placed, randomly oriented
    rings in [-2,2]^3; grid from the reference's bounding-box rule over vortons
    and tracers; velocity by the treecode at every gridpoint and every vorton;
    1,048,576 tracers advected.  Error against the GPU direct sum (itself within
    ~1e-7 of the FP64 direct sum, tests/test_gpu_parity.py)."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.rings(65536, count=8, seed=2, box=2.0)
    tr = np.random.default_rng(5).uniform(-1.8, 1.8, (1 << 20, 3)).astype(np.float32)
    cfg = vg.default_config(velocity_technique=vg.VELOCITY_TREE, enable_stretch=0, enable_diffusion=0, device=local)
    cfg.stream = stream.cuda_stream
    ctx = vg.VortonSim(cfg=cfg)

    def f4(a, wv=None):
        o = np.zeros((len(a), 4), np.float32)
        o[:, :3] = a
        if wv is not None:
            o[:, 3] = wv
        return torch.from_numpy(o).cuda()

    ps0, w0, tr0 = f4(pos, s), f4(w), f4(tr)
    ps, ww, vel = ps0.clone(), w0.clone(), torch.zeros_like(ps0)
    trp, trv = tr0.clone(), torch.zeros_like(tr0)
    box = np.array(list(tr.min(0)) + list(tr.max(0)), np.float32)
    ms = []
    with torch.cuda.stream(stream):
        for k in range(steps + 1):
            ps.copy_(ps0)
            ww.copy_(w0)
            trp.copy_(tr0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.UpdateDevice(ps, ww, vel, float(DT), extra_minmax=box)
            ctx.AdvectDevice(trp, trv, float(DT))
            b.record(stream)
            ctx.synchronize()
            if k > 0:
                ms.append(a.elapsed_time(b))
        st = ctx.stats()
        grid_np = tuple(int(v) for v in st.grid.num_points)
        # accuracy: direct sum at every vorton and at a sample of gridpoints
        ref = torch.zeros_like(ps0)
        lib = vg.lib()
        lib.vg_direct_device(ctx.h, 0, vg._ptr(ps0), vg._ptr(w0), ps0.shape[0], vg._ptr(ps0), ps0.shape[0], 1.0, 1.0,
                             vg._ptr(ref))
        vgrid, geom = ctx.GetVelocityGrid()
        idx = np.random.default_rng(7).integers(0, geom.capacity, 8192)
        gq = workloads.grid_points(list(geom.min_corner), list(geom.cell_spacing), geom.points)[idx]
        q = f4(gq)
        refg = torch.zeros_like(q)
        lib.vg_direct_device(ctx.h, 0, vg._ptr(ps0), vg._ptr(w0), ps0.shape[0], vg._ptr(q), q.shape[0], 1.0, 1.0,
                             vg._ptr(refg))
        ctx.synchronize()
        # the treecode alone (cell lists, tree build, walk) at every gridpoint and vorton, for its roofline
        gq = f4(workloads.grid_points(list(geom.min_corner), list(geom.cell_spacing), geom.points))
        qa = torch.cat([gq, ps0]).contiguous()
        outa = torch.zeros_like(qa)
        npts = ctypes.c_size_t()
        tms = []
        for k in range(4):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.check(lib.vg_tree_device(ctx.h, 0, ctypes.byref(geom), vg._ptr(ps0), vg._ptr(w0), ps0.shape[0],
                                         vg._ptr(qa), qa.shape[0], 1.0, 1.0, vg._ptr(outa), None, 0,
                                         ctypes.byref(npts)), "vg_tree_device")
            b.record(stream)
            ctx.synchronize()
            if k > 0:
                tms.append(a.elapsed_time(b))
    v = vel[:, :3].cpu().double()
    r = ref[:, :3].cpu().double()
    vg_s = torch.from_numpy(vgrid[idx].astype(np.float64))
    rg = refg[:, :3].cpu().double()
    t = statistics.median(ms)
    nq = geom.capacity + len(pos)
    qh = qa.cpu().numpy()[:, :3]
    per_query = tree_interactions(geom.points, list(geom.min_corner), list(geom.extent), qh) / len(qh)
    tree_ms = statistics.median(tms)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    peak = 2 * 128 * sms * 2070.0 * 1e6 / 1e12
    achieved = FLOPS_PER_INTERACTION * per_query * qa.shape[0] / (tree_ms * 1e-3) / 1e12
    out = {"workload": "8 rings, 65536 vortons in [-2,2]^3; treecode (NestedGrid, bit-exact binning) at every "
                       "gridpoint and vorton; 1048576 tracers gathered + Euler; stretch and diffusion off",
           "grid_points": grid_np, "tree_depth": st.tree_depth, "step_ms": t,
           "queries_per_s": nq / (t * 1e-3), "tracers_per_s": len(tr) / (t * 1e-3),
           "rel_l2_vs_direct_at_vortons": float((v - r).norm() / r.norm()),
           "rel_l2_vs_direct_at_gridpoints": float((vg_s - rg).norm() / rg.norm()),
           "note": "treecode error is the far-field monopole approximation plus the grid's auto-mollification "
                   "(the reference's own treecode has the same error: tests/test_gpu_config_parity.py)",
           "roofline": {"bound": "fp32 (issue: a dependent walk of few interactions per query)",
                        "kernel": "vg_tree_device: cell lists, tree build and walk at every gridpoint and vorton",
                        "ms_per_call": tree_ms, "interactions_per_query": per_query,
                        "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                        "peak_basis": f"2 flops x 128 FP32 lanes x {sms} SMs x 2070 MHz (maximum clock)"}}
    out["cpu_baseline"] = treecode_cpu_baseline(pos, w, s, geom, qh, tr, vgrid)
    return out


def tree_interactions(points, min_corner, extent, q):
    """Pair laws the NestedGrid walk (vortonSim.cpp:1650-1905) evaluates over
    the queries q.  From the root, each layer examines every child of the
    cells opened above it; a child containing the query (its cell widened by
    1e-4 spacings, vortonSim.cpp:1707-1719) is opened, the others add one
    pair law each, and the leaf's parent adds all its children.  The open test
    is a conjunction over axes, so the examined and opened sets are products
    of per-axis ranges; the test is evaluated in FP32 as the walk does.  The
    layer rule is NestedGrid's (nestedGrid.h:69-85, uniformGrid.h:398-412,
    794-809)."""
    f32 = np.float32
    q = np.ascontiguousarray(q, f32)
    layers = [np.array([int(v) for v in points], np.int64)]
    while np.prod(layers[-1]) > 8:
        layers.append(np.maximum(2, (layers[-1] - 1) // 2 + 1))
    depth = len(layers)
    if depth < 2:
        return 0
    mn = np.array(min_corner[:3], f32)
    ext = np.array(extent[:3], f32)
    cell = [(ext / (L - 1).astype(f32)).astype(f32) for L in layers]
    dec = [None] + [(layers[l - 1] - 1) // (layers[l] - 1) for l in range(1, depth)]
    lo = np.zeros((len(q), 3), np.int64)
    hi = np.zeros((len(q), 3), np.int64)
    alive = np.ones(len(q), bool)
    total = 0
    for layer in range(depth - 1, 0, -1):
        c_cell = cell[layer - 1]
        d = dec[layer]
        elo, ehi = lo * d, hi * d + d - 1
        examined = np.where(alive, np.prod(ehi - elo + 1, axis=1), 0)
        if layer == 1:
            total += int(examined.sum())
            break
        margin = (f32(0.0001) * c_cell).astype(f32)
        olo = np.full_like(lo, np.iinfo(np.int64).max)
        ohi = np.full_like(hi, -1)
        for k in range(int((ehi - elo).max()) + 1):
            c = elo + k
            cmin = (mn + (c.astype(f32) * c_cell).astype(f32)).astype(f32)
            cmax = (mn + ((c + 1).astype(f32) * c_cell).astype(f32)).astype(f32)
            inside = (c <= ehi) & (q >= (cmin - margin).astype(f32)) & (q < (cmax + margin).astype(f32))
            olo = np.where(inside & (c < olo), c, olo)
            ohi = np.where(inside & (c > ohi), c, ohi)
        nopen = np.prod(np.where(ohi >= olo, ohi - olo + 1, 0), axis=1)
        nopen = np.where(alive, nopen, 0)
        total += int((examined - nopen).sum())
        alive = alive & (nopen > 0)
        lo, hi = np.where(alive[:, None], olo, 0), np.where(alive[:, None], ohi, 0)
    return total


def treecode_cpu_baseline(pos, w, s, geom, q, tr, vgrid):
    """The reference's treecode (CreateInfluenceTree + ComputeVelocity_Tree at
    every gridpoint and vorton, vortonSim.cpp:1192-1905) and its tracer
    advection through the same velocity grid, on all host threads."""
    L = reference_lib()
    if L is None:
        return None
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    g12 = geom.as12()
    np3 = np.array(geom.points, np.uint32)
    q = np.ascontiguousarray(q, np.float32)
    out = np.zeros((len(q), 3), np.float32)
    t0 = time.perf_counter()
    L.vgref_tree(0, P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(g12), P(np3), P(q), ctypes.c_size_t(len(q)),
                 ctypes.c_float(1.0), ctypes.c_float(1.0), P(out))
    t1 = time.perf_counter()
    t = np.ascontiguousarray(tr, np.float32).copy()
    tv = np.zeros_like(t)
    vg3 = np.ascontiguousarray(vgrid, np.float32)
    t2 = time.perf_counter()
    L.vgref_advect(P(t), P(tv), ctypes.c_size_t(len(t)), P(g12), P(np3), P(vg3), ctypes.c_float(DT))
    t3 = time.perf_counter()
    return {"value": (t1 - t0 + t3 - t2) * 1e3, "unit": "ms per step (treecode at every query + tracer advection)",
            "cores": int(os.environ["NUMBER_OF_PROCESSORS"]), "kind": "reference", "tree_ms": (t1 - t0) * 1e3,
            "advect_ms": (t3 - t2) * 1e3, "queries_per_s": len(q) / (t1 - t0),
            "sample": f"one step: {len(q)} treecode queries, {len(t)} tracers"}


def batched_section(torch, local, n_sims=256, frames=6, seq_frames=2, dt=1.0 / 60.0):
    """256 independent effects (vorton counts log-uniform in [1k, 64k], grids
    of 16-96 cells per axis from each effect's extent, seeded ring / puff mix),
    each frame: treecode boundary, multigrid interior solve (network warm start
    where it fits and the autotuner keeps it), PSE diffusion, advection.  Frames
    replayed from captured CUDA graphs on parallel branches, the Poisson
    solves in one persistent launch (when the autotuner keeps it), vs the same
    frames stepped sequentially with per-level launches."""
    from vortegrid_gb300 import batch, warmstart
    effects = [batch.make_effect(1000 + i) for i in range(n_sims)]
    B = batch.Batch(effects, streams=8, device=local)
    if os.path.exists(warmstart.DEFAULT_WEIGHTS):
        B.load_network(warmstart.DEFAULT_WEIGHTS)
    t0 = time.perf_counter()
    streams, use_net, tuned_ms = B.autotune(dt, frames=2, candidates=(1, 2, 4, 8, 16, 32))
    tune_s = time.perf_counter() - t0
    B.step(dt)
    B.synchronize()
    t0 = time.perf_counter()
    for _ in range(frames):
        B.step(dt)
    B.synchronize()
    graph_ms = (time.perf_counter() - t0) / frames * 1e3
    t0 = time.perf_counter()
    for _ in range(seq_frames):
        B.step(dt, graph=False)
    B.synchronize()
    seq_ms = (time.perf_counter() - t0) / seq_frames * 1e3
    st = [B.stats(i) for i in range(len(B))]
    graphs, max_nodes, total_nodes = B.graph_info()
    p_sims, p_teams, p_ctas, p_graph = B.solver_info()
    left = sum(B.outside(i) for i in range(len(B)))
    # the alternative the autotuner weighed: the Poisson solves in one persistent
    # cooperative launch per frame (teams of 16 CTAs), the rest in the branch graphs
    persistent = None
    if p_sims == 0:
        B.set_solver(True, 16)
        B.step(dt)
        B.synchronize()
        t0 = time.perf_counter()
        for _ in range(frames):
            B.step(dt)
        B.synchronize()
        pers_ms = (time.perf_counter() - t0) / frames * 1e3
        n_in, teams, ctas, _ = B.solver_info()
        persistent = {"ms_per_frame": pers_ms, "simulations_in_launch": n_in, "teams": teams, "ctas_per_team": ctas,
                      "vs_branch_graphs": pers_ms / graph_ms}
        B.set_solver(False)
    cells = [int(e.grid.num_points[0]) - 1 for e in effects]
    nv = sum(e.n for e in effects)
    B.close()
    return {"workload": f"{n_sims} effects, {nv} vortons in total (1k-64k each), grids of 16-96 cells per axis; "
                        "per frame: treecode boundary, multigrid to 1e-6 on a calibrated fixed schedule, PSE "
                        "(viscosity 0.01), Euler advection",
            "grid_cells_histogram": {str(c): cells.count(c) for c in sorted(set(cells))},
            "autotuned": {"streams": streams, "network_warm_start": use_net, "graph_ms_at_best": tuned_ms,
                          "seconds": tune_s,
                          "persistent_solve": {"simulations": p_sims, "teams": p_teams, "ctas_per_team": p_ctas,
                                               "captured_as_graph": p_graph}},
            "graph_ms_per_frame": graph_ms, "sequential_ms_per_frame": seq_ms,
            "persistent_solve_alternative": persistent,
            "speedup_vs_sequential": seq_ms / graph_ms,
            "graphs_per_frame": graphs, "graph_nodes_max": max_nodes, "graph_nodes_total": total_nodes,
            "effect_steps_per_s": n_sims / (graph_ms * 1e-3), "vorton_steps_per_s": nv / (graph_ms * 1e-3),
            "max_relres": max(x.poisson_relres for x in st),
            "mean_cycles": float(np.mean([x.poisson_cycles for x in st])),
            "effects_with_vortons_outside_grid": left,
            "timing": "host wall clock over the frames plus one synchronisation (graph launches are asynchronous)"}


def body_record(shape, position, dims, hole=False, velocity=(0, 0, 0), angular_velocity=(0, 0, 0), rot=None,
                temperature=300.0, conductivity=0.0):
    """One rigid body in the library's 32-float layout (shape 0 sphere, 1 box)."""
    b = np.zeros(32, np.float32)
    b[0], b[1] = shape, 1.0 if hole else 0.0
    b[2:5], b[5:8], b[8:11] = position, velocity, angular_velocity
    b[11:20] = np.asarray(np.eye(3) if rot is None else rot, np.float32).ravel()
    d = np.atleast_1d(np.asarray(dims, np.float32))
    b[20:20 + len(d)] = d
    b[23], b[24] = temperature, conductivity
    return b


def rows_cpu_baseline(L, pos, s, dens, w, g12, np3, bodies, amb, grav, dt):
    """The reference's own code for the same operations on the host (single-threaded: these
    functions are serial loops in the reference), each on the full workload or a stated sample."""
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    out = {}

    def timed(fn):
        t0 = time.perf_counter()
        fn()
        return (time.perf_counter() - t0) * 1e3
    n = len(pos)
    wc = w.copy()
    out["baroclinic_ms"] = timed(lambda: L.vgref_baroclinic(P(pos), P(wc), P(s), P(dens), ctypes.c_size_t(n), P(g12),
                                                            P(np3), P(grav), ctypes.c_float(amb), ctypes.c_float(dt)))
    dg = np.zeros(int(np.prod(np3)), np.float32)
    out["density_grid_ms"] = timed(lambda: L.vgref_density_grid(P(pos), P(s), P(dens), ctypes.c_size_t(n), P(g12),
                                                                P(np3), ctypes.c_float(amb), P(dg)))
    sdf = np.zeros_like(dg)
    out["signed_distance_ms"] = timed(lambda: L.vgref_signed_distance(P(g12), P(np3), P(dg), ctypes.c_float(amb),
                                                                      P(sdf)))
    pp, vv, ww, dd = pos.copy(), np.zeros_like(pos), w.copy(), dens.copy()
    o9 = np.zeros((len(bodies), 9), np.float32)
    out["collide_vortons_ms"] = timed(lambda: L.vgref_collide_vortons(P(pp), P(vv), P(ww), P(s), P(dd),
                                                                      ctypes.c_size_t(n), P(bodies), len(bodies),
                                                                      ctypes.c_float(amb), ctypes.c_float(1.0), P(o9)))
    hd = dens.copy()
    out["heat_pse_ms"] = timed(lambda: L.vgref_heat_pse(P(pos), P(hd), P(s), ctypes.c_size_t(n), P(g12), P(np3),
                                                        ctypes.c_float(1e-3), ctypes.c_float(amb),
                                                        ctypes.c_float(dt)))
    # tracer seeding on a 16^3-cell sample of the tracer grid (512,000 particles), scaled per particle
    cells = 16
    sg = np.array([-2.0, -2.0, -2.0, 2.0, 2.0, 2.0, 0.25, 0.25, 0.25, 4.0, 4.0, 4.0], np.float32)
    snp = np.array([cells + 1] * 3, np.uint32)
    cap = cells ** 3 * 125
    ep, ed, es = np.zeros((cap, 3), np.float32), np.zeros(cap, np.float32), np.zeros(cap, np.float32)
    cnt = ctypes.c_size_t()
    t = timed(lambda: L.vgref_emit_grid(P(sg), P(snp), ctypes.c_uint(5), P(pos), P(s), P(dens), ctypes.c_size_t(0), 0,
                                        ctypes.c_uint(1), P(ep), P(ed), P(es), ctypes.c_size_t(cap),
                                        ctypes.byref(cnt)))
    out["emit_ns_per_particle"] = t * 1e6 / cap
    out["cores"] = int(os.environ.get("NUMBER_OF_PROCESSORS", "1"))
    out["kind"] = "reference"
    out["sample"] = ("the full workload per operation (262,144 vortons on 129^3, 3 bodies), the tracer seeding on "
                     "512,000 particles; the reference's code with its own threading where it has any (the "
                     "std::thread stand-in for TBB); particle records converted to the reference's Particle "
                     "vectors inside the timed call")
    return out


def rows_section(vg, torch, stream, local):
    """The operations around the step, at the multigrid workload's sizes (262,144 puff vortons on the
    129^3 grid of [-2, 2]^3, 4,194,304 tracers): emitters, wind and age kill, heat PSE, the density
    grid / gradient / baroclinic generation, signed distance and marching cubes, fluid-body
    collisions with three bodies.  GPU time per call (CUDA events on the context's stream, median of
    5 after 2 warm-ups), the bytes each call must move against the measured HBM peak, and the
    reference's own code on the host cores beside them."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.puff(262144, seed=3)
    n = len(pos)
    dens = (1.0 + 0.2 * np.exp(-(pos.astype(np.float64) ** 2).sum(1) / 0.2)).astype(np.float32)
    grid = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [129] * 3)
    pts = grid.capacity
    amb, dt = 1.0, 1.0 / 30.0
    grav = np.array([0.0, -9.8, 0.0], np.float32)
    c, sn = np.cos(0.3), np.sin(0.3)
    rot = np.array([[c, -sn, 0], [sn, c, 0], [0, 0, 1]], np.float32)
    bodies = np.stack([body_record(0, [0.2, 0, 0], [0.4], velocity=[0.5, 0, 0], angular_velocity=[0, 0, 1],
                                   temperature=350, conductivity=0.5),
                       body_record(1, [0, 0, 0], [3.6, 3.6, 3.2], hole=True, rot=rot, conductivity=0.1),
                       body_record(1, [0.0, 0.5, 0.3], [0.3, 0.4, 0.5], velocity=[0, 0.2, 0],
                                   angular_velocity=[0.3, 0, 0], rot=rot, temperature=320, conductivity=0.2)])
    cfg = vg.default_config(device=local)
    cfg.stream = stream.cuda_stream
    ctx = vg.Context(cfg)
    lib = vg.lib()
    P = vg._ptr

    def f4(a, wv=None):
        o = np.zeros((len(a), 4), np.float32)
        o[:, :3] = a
        if wv is not None:
            o[:, 3] = wv
        return torch.from_numpy(o).cuda()
    ps0, w0, d0 = f4(pos, s), f4(w), torch.from_numpy(dens).cuda()
    ps, ww, dd, vel = ps0.clone(), w0.clone(), d0.clone(), torch.zeros_like(ps0)
    dg = torch.zeros(pts, dtype=torch.float32, device="cuda")
    gr = torch.zeros(pts * 3, dtype=torch.float32, device="cuda")
    sdf = torch.zeros(pts, dtype=torch.float32, device="cuda")
    m_tr = N_TRACERS_POISSON
    tr0 = f4(np.random.default_rng(6).uniform(-1.9, 1.9, (m_tr, 3)).astype(np.float32), 0.01)
    trp, trv = tr0.clone(), torch.zeros_like(tr0)
    birth0 = torch.randint(0, 100, (m_tr,), dtype=torch.int32, device="cuda")
    birth = birth0.clone()
    applied = ctypes.c_int()
    out9 = np.zeros((len(bodies), 9), np.float32)
    hits = np.zeros(len(bodies), np.uint64)
    out6 = np.zeros((len(bodies), 6), np.float32)
    tris = ctypes.c_size_t()
    cap_tris = 4 * pts
    verts = torch.empty(cap_tris * 9, dtype=torch.float32, device="cuda")

    def timed(fn, reset=None, reps=5):
        ms = []
        with torch.cuda.stream(stream):
            for k in range(reps + 2):
                if reset:
                    reset()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                torch.cuda.synchronize()
                if k >= 2:
                    ms.append(a.elapsed_time(b))
        return statistics.median(ms)
    peaks = measured_peaks()
    res = {}

    def row(name, ms, nbytes, note):
        gbs = nbytes / (ms * 1e-3) / 1e9
        res[name] = {"ms": ms, "algorithmic_bytes": nbytes, "achieved_gbs": gbs, "frac_of_hbm": gbs / peaks["hbm_gbs"],
                     "bytes_basis": note}
    g = ctypes.byref(grid)
    # tracer seeding: 32^3 cells x 5^3 = 4,096,000 tracers, counter-based jitter
    tg = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [33] * 3)
    grp = vg.ParticleGroup(32 ** 3 * 125)
    row("emit_grid_4096000", timed(lambda: vg.PclOpEmit.Emit(ctx, grp, tg, 5, None, vg.JITTER_HASH, 1),
                                   reset=lambda: setattr(grp, "count", 0)),
        4096000 * 56, "pos_size, vel4, angvel4 (16 B each), density, birth (4 B each) written per tracer")
    del grp
    row("wind_4194304", timed(lambda: ctx.check(lib.vg_wind_device(ctx.h, P(trv), m_tr, P(np.array([1.0, 0, 0],
        np.float32)), 0.125, 0.875), "wind")), m_tr * 32, "vel4 read and written")
    alive = ctypes.c_size_t()
    row("kill_age_4194304", timed(lambda: ctx.check(lib.vg_kill_age_device(ctx.h, P(trp), P(trv), None, P(birth), m_tr,
        120, 60, ctypes.byref(alive)), "kill"), reset=lambda: (trp.copy_(tr0), birth.copy_(birth0))),
        m_tr * 4 * 2, "birth read for the flags and the scan (the moves of removed slots not counted)")
    row("heat_pse_262144", timed(lambda: ctx.check(lib.vg_heat_pse_device(ctx.h, g, P(ps0), P(dd), n, 1e-3, amb, dt),
                                                   "heat"), reset=lambda: dd.copy_(d0)),
        n * (16 + 4 + 4), "pos_size and density read, density written per vorton")
    row("density_grid_129", timed(lambda: ctx.check(lib.vg_density_grid_device(ctx.h, g, P(ps0), P(d0), n, amb, P(dg)),
                                                    "density")), n * 20 + pts * 4,
        "pos_size and density read per vorton, one float written per point")
    row("gradient_129", timed(lambda: ctx.check(lib.vg_gradient_device(ctx.h, g, P(dg), P(gr)), "gradient")),
        pts * 16, "4 B read and 12 B written per point")
    row("baroclinic_262144", timed(lambda: ctx.check(lib.vg_baroclinic_device(ctx.h, g, P(ps0), P(d0), P(ww), n,
        P(grav), amb, dt, ctypes.byref(applied)), "baroclinic"), reset=lambda: ww.copy_(w0)),
        n * 20 + pts * 20 + n * 32, "density grid, its gradient, then pos_size + angvel read and angvel written")
    row("signed_distance_129", timed(lambda: ctx.check(lib.vg_signed_distance_device(ctx.h, g, P(dg), amb, 0, P(sdf)),
                                                       "sdf")), pts * 8, "density read, distance written per point")
    row("marching_cubes_129", timed(lambda: ctx.check(lib.vg_marching_cubes_device(ctx.h, g, P(sdf), 0.0, P(verts),
        None, cap_tris, ctypes.byref(tris)), "mc")), pts * 4 * 2,
        "the field read twice (count, emit); triangles written not counted")
    res["marching_cubes_129"]["triangles"] = tris.value
    bods = np.ascontiguousarray(bodies, np.float32)
    row("collide_vortons_262144_3_bodies", timed(lambda: ctx.check(lib.vg_collide_vortons_device(ctx.h, P(bods),
        len(bods), P(ps), P(vel), P(ww), P(dd), n, amb, 1.0, P(out9), P(hits)), "collide"),
        reset=lambda: (ps.copy_(ps0), vel.zero_(), ww.copy_(w0), dd.copy_(d0))),
        n * 3 * 2 * 52, "pos_size, vel4, angvel4, density read and written per vorton and body")
    row("collide_tracers_4194304_3_bodies", timed(lambda: ctx.check(lib.vg_collide_tracers_device(ctx.h, P(bods),
        len(bods), P(trp), P(trv), None, m_tr, P(out6)), "collide tracers"), reset=lambda: trp.copy_(tr0)),
        m_tr * 3 * 2 * 32, "pos_size and vel4 read and written per tracer and body")
    res["workload"] = ("262,144 puff vortons (density 1 + 0.2 exp(-r^2/0.2)) on 129^3 over [-2,2]^3; 4,194,304 "
                       "tracers; three bodies (a moving, spinning, hot sphere, a rotated hole box holding the "
                       "fluid, a rotated solid box); emitted tracers 32^3 cells x 5^3")
    res["hbm_peak_gbs"] = peaks["hbm_gbs"]
    L = reference_lib()
    if L is not None:
        g12, np3 = grid.as12(), np.array(grid.points, np.uint32)
        res["cpu_baseline"] = rows_cpu_baseline(L, pos, s, dens, w, g12, np3, bods, amb, grav, dt)
    return res


MG_BYTES_PER_POINT_CYCLE = 250  # V(2,2) over the levels: smoothing, residual + restriction, prolongation + correction
ADVECT_BYTES_PER_TRACER = 48     # float4 position read and written, float4 velocity written
N_TRACERS_POISSON = 1 << 22


def measured_peaks():
    """HBM and BF16 peaks measured on this GPU type (MEASURED_PEAKS.json), else the stated fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]), "basis": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "basis": "fallback"}


def poisson_cpu_baseline(pos, w, s, g12, np3, tr):
    """The reference's own solve on the same problem, all host threads: its
    boundary vector potential (ComputeVectorPotentialAtGridpoints_Slice,
    boundaries only) and its multigrid cascade at its fixed work (16 SOR
    sweeps per level, vortonSim.cpp:2523-2608), with the relative residual it
    reaches; and its tracer advection (AssignVelocityFromField + Evolve,
    pclOpAdvect.cpp:42-81, pclOpEvolve.cpp:36-58) of the same tracers."""
    import oracle
    L = reference_lib()
    if L is None:
        return None
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    cores = int(os.environ["NUMBER_OF_PROCESSORS"])
    npts = int(np3[0]) * int(np3[1]) * int(np3[2])
    b = np.zeros((npts, 3), np.float32)
    L.vgref_splat(P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(g12), P(np3), ctypes.c_float(-1.0), P(b))
    a = np.zeros((npts, 3), np.float32)
    t0 = time.perf_counter()
    L.vgref_boundary_vecpot(P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(g12), P(np3), 1, P(a))
    t1 = time.perf_counter()
    L.vgref_cascade(P(g12), P(np3), P(a), P(b), 16)
    t2 = time.perf_counter()
    og = oracle.Geom.from12(g12, np3)
    relres = oracle.relres(og, a, b)
    vel = np.zeros((npts, 3), np.float32)
    jac = np.zeros((npts, 9), np.float32)
    L.vgref_jacobian_curl(P(g12), P(np3), P(a), P(jac), P(vel))
    t = np.ascontiguousarray(tr, np.float32).copy()
    tv = np.zeros_like(t)
    t3 = time.perf_counter()
    L.vgref_advect(P(t), P(tv), ctypes.c_size_t(len(t)), P(g12), P(np3), P(vel), ctypes.c_float(DT))
    t4 = time.perf_counter()
    return {"value": (t2 - t0) * 1e3, "unit": "ms per solve (boundary + cascade)", "cores": cores,
            "kind": "reference", "boundary_ms": (t1 - t0) * 1e3, "cascade_ms": (t2 - t1) * 1e3,
            "relres": relres, "advect_ms": (t4 - t3) * 1e3, "advect_tracers_per_s": len(t) / (t4 - t3),
            "sample": f"one solve of the same 129^3 problem; {len(t)} tracers advected once"}


def poisson_section(vg, torch, stream, local, steps=3):
    """128^3 vector-potential solve to 1e-6 on the puff workload through the
    library's own step, from three starts: zero (plain multigrid), the learned
    network (its guess is timed inside the solve) and the previous frame; the
    same zero-start solve on the fixed schedule (no host round trip); 4M
    tracers advected through the step's velocity grid; the reference's own
    solve and advection on the host cores beside it."""
    from vortegrid_gb300 import workloads, warmstart
    pos, w, s = workloads.puff(262144, seed=3)
    grid = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [129] * 3)
    o = np.zeros((len(pos), 4), np.float32)
    o[:, :3] = pos
    o[:, 3] = s
    ps0 = torch.from_numpy(o).cuda()
    o2 = np.zeros((len(pos), 4), np.float32)
    o2[:, :3] = w
    w0 = torch.from_numpy(o2).cuda()
    tr = np.random.default_rng(6).uniform(-1.9, 1.9, (N_TRACERS_POISSON, 3)).astype(np.float32)
    o3 = np.zeros((len(tr), 4), np.float32)
    o3[:, :3] = tr
    tr0 = torch.from_numpy(o3).cuda()

    def make_ctx(warm):
        cfg = vg.default_config(fixed_grid=grid, device=local)
        cfg.stream = stream.cuda_stream
        cfg.warm_start = warm
        return vg.VortonSim(cfg=cfg)

    def run(ctx, reset):
        ps, ww, vel = ps0.clone(), w0.clone(), torch.zeros_like(ps0)
        res = []
        with torch.cuda.stream(stream):
            for k in range(steps + 1):
                if reset:
                    ps.copy_(ps0)
                    ww.copy_(w0)
                ctx.UpdateDevice(ps, ww, vel, float(DT))
                st = ctx.stats()
                if k > 0:
                    res.append((st.ms_poisson, st.ms_total, st.poisson_cycles, st.poisson_relres0, st.poisson_relres,
                                st.warm_start_used))
        return res

    def summary(res):
        return {"ms": statistics.median(r[0] for r in res), "step_ms": statistics.median(r[1] for r in res),
                "cycles": res[-1][2], "relres0": res[-1][3], "relres": res[-1][4], "warm_start_used": res[-1][5]}

    def velocity(ctx):
        v, _ = ctx.GetVelocityGrid()
        return torch.from_numpy(np.ascontiguousarray(v, np.float64).reshape(-1))

    zero_ctx = make_ctx(0)
    zero = summary(run(zero_ctx, True))
    out = {"workload": "puff: 262144 vortons N(0,0.5^2), vorticity N(0,2^2), 129^3 grid on [-2,2]^3 (dx=1/32), "
                       "treecode boundary, FP32 V(2,2)-cycles (red-black SOR, omega 1.3) in FP64-class iterative "
                       "refinement to 1e-6; 4194304 tracers advected",
           "tolerance": 1e-6, "plain_mg_adaptive_ms": zero["ms"], "step_ms": zero["step_ms"], "cycles": zero["cycles"],
           "relres0": zero["relres0"], "relres": zero["relres"],
           "timing": "CUDA events around the solve inside the step.  plain_mg_ms is the zero-start solve on the "
                     "fixed schedule (the cycle counts the adaptive solve of the same problem chose, replayed with "
                     "no host round trip, as a simulation replays it frame after frame); plain_mg_adaptive_ms is "
                     "the adaptive solve, which reads a residual back to the host after every cycle"}
    # velocity error at 512 interior points against the FP64 direct sum (tests/golden/puff129_exact.npz)
    try:
        fx = np.load(os.path.join(ROOT, "tests", "golden", "puff129_exact.npz"))
        vz, _ = zero_ctx.GetVelocityGrid()
        got = vz[fx["flat"]].astype(np.float64)
        d = fx["direct"]
        out["velocity_rel_l2_vs_fp64_direct"] = float(np.linalg.norm(got - d) / np.linalg.norm(d))
        out["velocity_rel_l2_vs_exact_discrete"] = float(np.linalg.norm(got - fx["exact_vel"]) /
                                                         np.linalg.norm(fx["exact_vel"]))
        out["exact_discrete_rel_l2_vs_fp64_direct"] = float(np.linalg.norm(fx["exact_vel"] - d) / np.linalg.norm(d))
        out["velocity_note"] = ("512 interior gridpoints; the puff's vortons lie closer than dx, so the grid "
                                "discretisation error dominates (the exact discrete solution has the same)")
    except OSError:
        pass
    # the same solve on the fixed schedule the adaptive one used (no host round trip)
    k1, k2 = zero_ctx.poisson_schedule()
    zero_ctx.set_poisson_schedule(k1, k2)
    fixed = summary(run(zero_ctx, True))
    st_fixed = zero_ctx.stats()
    v32 = velocity(zero_ctx)
    # the same schedule with the coarsest level (33^3, sine transforms) solved in FP64
    zero_ctx.set_coarsest_fp64(True)
    c64 = summary(run(zero_ctx, True))
    st64 = zero_ctx.stats()
    v64 = velocity(zero_ctx)
    zero_ctx.set_coarsest_fp64(False)
    zero_ctx.set_poisson_schedule(0, 0)
    out["coarsest_fp64"] = {"ms": c64["ms"], "relres": st64.poisson_relres,
                            "velocity_rel_diff_vs_fp32_coarsest": float((v64 - v32).norm() / v32.norm()),
                            "note": "the fixed schedule with the coarsest solve's tables and arithmetic in FP64; "
                                    "the default solve keeps them in FP32"}
    out["fixed_schedule"] = {"ms": fixed["ms"], "fp32_cycles": k1, "refinement_cycles": k2,
                             "relres": st_fixed.poisson_relres}
    out["plain_mg_ms"] = fixed["ms"]
    peaks = measured_peaks()
    pts = grid.capacity
    best_ms = min(zero["ms"], fixed["ms"])
    achieved = MG_BYTES_PER_POINT_CYCLE * pts * zero["cycles"] / (best_ms * 1e-3) / 1e9
    out["roofline"] = {"bound": "hbm", "kernel": "multigrid solve (all its kernels)", "achieved": achieved,
                       "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                       "peak_basis": peaks["basis"], "traffic": None,
                       "algorithmic_bytes": f"{MG_BYTES_PER_POINT_CYCLE} B per fine point per V(2,2) cycle x "
                                            f"{pts} points x {zero['cycles']} cycles",
                       "note": "the level-0 fields (52 MB) stay in the 129 MB L2; the fraction is of HBM peak"}
    # 4M tracers through the step's velocity grid (AssignVelocityFromField + Evolve)
    trp, trv = tr0.clone(), torch.zeros_like(tr0)
    ams = []
    with torch.cuda.stream(stream):
        for k in range(4):
            trp.copy_(tr0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            zero_ctx.AdvectDevice(trp, trv, float(DT))
            b.record(stream)
            zero_ctx.synchronize()
            if k > 0:
                ams.append(a.elapsed_time(b))
    adv = statistics.median(ams)
    adv_bytes = ADVECT_BYTES_PER_TRACER * len(tr) + pts * 12
    out["tracers"] = {"count": len(tr), "advect_ms": adv, "tracers_per_s": len(tr) / (adv * 1e-3),
                      "roofline": {"bound": "hbm", "achieved": adv_bytes / (adv * 1e-3) / 1e9,
                                   "peak": peaks["hbm_gbs"], "unit": "GB/s",
                                   "frac": adv_bytes / (adv * 1e-3) / 1e9 / peaks["hbm_gbs"],
                                   "algorithmic_bytes": f"{ADVECT_BYTES_PER_TRACER} B per tracer + the grid once"}}
    out["step_with_tracers_ms"] = zero["step_ms"] + adv
    prev = summary(run(make_ctx(1), False))
    out["previous_frame"] = {"ms": prev["ms"], "cycles": prev["cycles"], "relres0": prev["relres0"],
                             "relres": prev["relres"], "note": "field evolving one step between solves"}
    if os.path.exists(warmstart.DEFAULT_WEIGHTS):
        net = warmstart.Network(warmstart.EDGE, local, stream)
        net.load(warmstart.DEFAULT_WEIGHTS)
        nn_ctx = make_ctx(2)
        nn_ctx.check(vg.lib().vg_set_network(nn_ctx.h, net.h), "vg_set_network")
        nn = summary(run(nn_ctx, True))
        v_zero, v_nn = velocity(zero_ctx), velocity(nn_ctx)
        out["nn_warm_start_ms"] = nn["ms"]
        out["nn"] = {"ms_including_guess": nn["ms"], "cycles": nn["cycles"], "relres0": nn["relres0"],
                     "relres": nn["relres"], "warm_start_used": nn["warm_start_used"],
                     "velocity_rel_diff_vs_plain": float((v_nn - v_zero).norm() / v_zero.norm()),
                     "speedup_vs_plain_mg": zero["ms"] / nn["ms"]}
    else:
        out["nn_warm_start_ms"] = None
        out["nn_note"] = "no trained weights at " + warmstart.DEFAULT_WEIGHTS
    g12 = grid.as12()
    np3 = np.array(grid.points, np.uint32)
    cpu = poisson_cpu_baseline(pos, w, s, g12, np3, tr)
    if cpu is not None:
        out["cpu_baseline"] = cpu
    return out


def run_section(name):
    """One workload section alone on cuda:0 (its own JSON object), for profiling."""
    import torch
    import vortegrid_gb300 as vg
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    if name == "poisson":
        out = poisson_section(vg, torch, stream, 0)
    elif name == "treecode":
        out = treecode_section(vg, torch, stream, 0)
    elif name == "rows":
        out = rows_section(vg, torch, stream, 0)
    else:
        out = batched_section(torch, 0)
    print(json.dumps({"section": name, name: out}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=3.0)
    ap.add_argument("--skip-poisson", action="store_true")
    ap.add_argument("--section", choices=["poisson", "treecode", "batched", "rows"],
                    help="run one workload section alone and print its JSON (for profiling)")
    args = ap.parse_args()
    if args.section:
        run_section(args.section)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world, rank, local = dist_setup() if args.impl == "ours" else (int(os.environ.get("WORLD_SIZE", "1")),
                                                                  int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
