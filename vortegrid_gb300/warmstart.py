"""Learned warm start for the vector-potential solve: network handle,
solver-generated training pairs, training loop and evaluation.

The network's forward and backward passes and its optimiser run in
libvortegrid (the vg_net_* functions of include/vortegrid.h); this module only
drives them.  Training pairs come from this library's own plain solver on the
fixed 129^3 grid over [-2, 2]^3 (dx = 1/32): the vortons of a seeded field are
splatted to the right-hand side (PopulateVorticityGridFromVortons with scale
-1, VortonFluid/vortonSim.cpp:2372-2436), the boundary vector potential comes
from the treecode (vortonSim.cpp:2055-2204) and multigrid solves the interior
to a 1e-6 relative residual.

Fields (seeded; half rings, half puffs):
  * rings -- 1..12 rings of 65,536 vortons in all, major radius U[0.3, 1.0],
    tube radius 0.25, Gaussian vorticity profile (sigma 0.1, peak 10), random
    centres and axes inside the box;
  * puff  -- 262,144 vortons, positions N(0, sigma^2) with sigma U[0.2, 0.8]
    (clipped to +-1.9), vorticity components N(0, 2^2).

Usage (on a GPU):  python -m vortegrid_gb300.warmstart train --pairs 4000 --epochs 3
"""
import argparse
import ctypes
import json
import math
import os
import sys
import time

import numpy as np

from . import OK, VgError, GridGeom, Context, default_config, lib

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "weights", "unet_edge128.vgnet")
EDGE = 128
VORTON_RADIUS = 0.05
# (ci, co) per layer, in the library's order (see vg_nn.cu)
LAYERS = [(16, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128), (192, 64), (64, 64),
          (96, 32), (32, 32), (48, 16), (16, 16), (16, 16)]
INPUT_CHANNELS = 6   # right-hand side xyz, boundary values xyz
SLOPE = 0.1          # leaky ReLU slope below zero
OUTPUT_CHANNELS = 3


def field_grid(points=EDGE + 1, half=2.0):
    return GridGeom.make([-half] * 3, [2 * half] * 3, [points] * 3)


def init_params(seed=0, zero_output=True):
    """He-normal weights (for the leaky ReLU) over the channels that carry
    data, zero biases; the input layer ignores the zero-padded channels, the
    output layer starts at zero (the first guess is the zero start) and its
    unused channels stay zero."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (ci, co) in enumerate(LAYERS):
        fan_ci = INPUT_CHANNELS if l == 0 else ci
        std = math.sqrt(2.0 / ((1.0 + SLOPE ** 2) * 27 * fan_ci))
        w = rng.normal(0.0, std, (27, co, ci)).astype(np.float32)
        if l == 0:
            w[:, :, INPUT_CHANNELS:] = 0.0
        if l == len(LAYERS) - 1:
            w[:] = 0.0 if zero_output else w * math.sqrt(0.5)
            w[:, OUTPUT_CHANNELS:, :] = 0.0
        parts += [w.ravel(), np.zeros(co, np.float32)]
    p = np.concatenate(parts)
    assert p.size == lib().vg_net_param_count()
    return p


class _Ordered:
    """Orders work that the library enqueues on `stream` after the caller's
    current torch stream, and the caller's later work after it (event waits
    both ways), so library calls and torch tensor operations never race."""

    def __init__(self, stream):
        self.stream = stream

    def __enter__(self):
        import torch
        self.stream.wait_stream(torch.cuda.current_stream())
        return self

    def __exit__(self, *exc):
        import torch
        torch.cuda.current_stream().wait_stream(self.stream)
        return False


def _torch_stream(stream):
    import torch
    return stream if stream is not None else torch.cuda.Stream()


class Network:
    """One vg_net: the warm-start U-Net on an edge^3 voxel grid ((edge+1)^3
    points).  Runs on its own torch stream (or `stream`), ordered against the
    caller's current stream on every call."""

    def __init__(self, edge=EDGE, device=0, stream=None):
        import torch
        self.edge = edge
        torch.cuda.set_device(device)
        self.stream = _torch_stream(stream)
        h = ctypes.c_void_p()
        st = lib().vg_net_create(device, ctypes.c_void_p(self.stream.cuda_stream), edge, ctypes.byref(h))
        if st != OK:
            raise VgError(st, "vg_net_create: " + lib().vg_last_error(None).decode())
        self.h = h
        self.count = lib().vg_net_param_count()

    def close(self):
        if getattr(self, "h", None):
            lib().vg_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st, what):
        if st != OK:
            raise VgError(st, f"{what}: {lib().vg_net_last_error(self.h).decode()}")

    def set_params(self, p, out_scale):
        p = np.ascontiguousarray(p, np.float32)
        self.check(lib().vg_net_set_params(self.h, p.ctypes.data_as(ctypes.c_void_p), p.size, float(out_scale)),
                   "vg_net_set_params")

    def params(self):
        p = np.empty(self.count, np.float32)
        k = ctypes.c_float()
        self.check(lib().vg_net_get_params(self.h, p.ctypes.data_as(ctypes.c_void_p), p.size, ctypes.byref(k)),
                   "vg_net_get_params")
        return p, k.value

    def save(self, path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        self.check(lib().vg_net_save(self.h, path.encode()), "vg_net_save")

    def load(self, path):
        self.check(lib().vg_net_load(self.h, path.encode()), "vg_net_load")

    def guess(self, grid, rhs, vecpot):
        """Interior of vecpot (device tensor, boundary set) <- the network's guess for rhs."""
        with _Ordered(self.stream):
            self.check(lib().vg_net_guess_device(self.h, ctypes.byref(grid), ctypes.c_void_p(rhs.data_ptr()),
                                                 ctypes.c_void_p(vecpot.data_ptr())), "vg_net_guess_device")

    def backward(self, grid, rhs, vecpot, want_loss=False, accumulate=False):
        """Forward + backward on one pair of device tensors (float32 or bfloat16);
        with accumulate the gradients add to the previous pass's."""
        import torch
        bf = 1 if rhs.dtype == torch.bfloat16 else 0
        loss = ctypes.c_float()
        with _Ordered(self.stream):
            self.check(lib().vg_net_backward_device(self.h, ctypes.byref(grid), bf, ctypes.c_void_p(rhs.data_ptr()),
                                                    ctypes.c_void_p(vecpot.data_ptr()), 1 if accumulate else 0,
                                                    ctypes.byref(loss) if want_loss else None),
                       "vg_net_backward_device")
        return loss.value if want_loss else None

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        with _Ordered(self.stream):
            self.check(lib().vg_net_adam_step(self.h, lr, beta1, beta2, eps), "vg_net_adam_step")

    def grads(self):
        g = np.empty(self.count, np.float32)
        self.check(lib().vg_net_get_grads(self.h, g.ctypes.data_as(ctypes.c_void_p), g.size), "vg_net_get_grads")
        return g

    def output(self):
        o = np.empty(self.edge ** 3 * 16, np.float32)
        self.check(lib().vg_net_get_output(self.h, o.ctypes.data_as(ctypes.c_void_p), o.size), "vg_net_get_output")
        return o.reshape(-1, 16)

    def activation(self, which, channels, level):
        e = self.edge >> level
        a = np.empty(e ** 3 * channels, np.float32)
        self.check(lib().vg_net_get_activation(self.h, which, a.ctypes.data_as(ctypes.c_void_p), a.size),
                   "vg_net_get_activation")
        return a.reshape(-1, channels)

    def gradient(self, layer, of_input, channels, level):
        e = self.edge >> level
        a = np.empty(e ** 3 * channels, np.float32)
        self.check(lib().vg_net_get_gradient(self.h, layer, of_input, a.ctypes.data_as(ctypes.c_void_p), a.size),
                   "vg_net_get_gradient")
        return a.reshape(-1, channels)

    def synchronize(self):
        self.check(lib().vg_net_synchronize(self.h), "vg_net_synchronize")


# ------------------------------------------------------------------ fields

def _ring_torch(torch, gen, n, major, center, axis, tube=0.25, sigma=0.1, peak=10.0):
    dev = gen.device
    u = torch.rand((3, n), generator=gen, device=dev, dtype=torch.float64)
    phi, theta = 2 * math.pi * u[0], 2 * math.pi * u[1]
    r = tube * torch.sqrt(u[2])
    rho = major + r * torch.cos(theta)
    local = torch.stack([rho * torch.cos(phi), rho * torch.sin(phi), r * torch.sin(theta)], 1)
    mag = peak * torch.exp(-r * r / (2 * sigma * sigma))
    vort = torch.stack([-torch.sin(phi) * mag, torch.cos(phi) * mag, torch.zeros_like(mag)], 1)
    a = axis / np.linalg.norm(axis)
    z = np.array([0.0, 0.0, 1.0])
    v = np.cross(z, a)
    s, c = np.linalg.norm(v), float(np.dot(z, a))
    if s < 1e-12:
        R = np.eye(3) if c > 0 else np.diag([1.0, -1.0, -1.0])
    else:
        vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
        R = np.eye(3) + vx + vx @ vx * ((1 - c) / (s * s))
    Rt = torch.from_numpy(R.T.copy()).to(dev)
    return local @ Rt + torch.from_numpy(np.asarray(center, np.float64)).to(dev), vort @ Rt


def make_field(kind, seed, device="cuda", n_rings=65536, n_puff=262144):
    """(pos_size [n,4] float32, angvel [n,4] float32) device tensors for one seeded field.

    angvel = vorticity / 2 and size = 2 x radius, the reference's storage convention."""
    import torch
    rs = np.random.default_rng(seed)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed) & 0x7fffffffffffffff)
    if kind == "rings":
        count = int(rs.integers(1, 13))
        sizes = np.full(count, n_rings // count)
        sizes[: n_rings - sizes.sum()] += 1
        P, W = [], []
        for k in range(count):
            major = rs.uniform(0.3, 1.0)
            lim = 2.0 - major - 0.25 - 0.1
            p, w = _ring_torch(torch, gen, int(sizes[k]), major, rs.uniform(-lim, lim, 3), rs.normal(size=3))
            P.append(p)
            W.append(w)
        pos, vort = torch.cat(P), torch.cat(W)
    elif kind == "puff":
        sigma = rs.uniform(0.2, 0.8)
        pos = torch.clamp(torch.randn((n_puff, 3), generator=gen, device=device, dtype=torch.float64) * sigma,
                          -1.9, 1.9)
        vort = torch.randn((n_puff, 3), generator=gen, device=device, dtype=torch.float64) * 2.0
    else:
        raise ValueError(kind)
    n = pos.shape[0]
    ps = torch.empty((n, 4), dtype=torch.float32, device=device)
    ps[:, :3] = pos.float()
    ps[:, 3] = 2 * VORTON_RADIUS
    w = torch.zeros((n, 4), dtype=torch.float32, device=device)
    w[:, :3] = (0.5 * vort).float()
    return ps, w


def field_kind(i):
    return "rings" if i % 2 == 0 else "puff"


class Solver:
    """The plain pipeline around the network: splat, treecode boundary, optional
    guess, multigrid -- through this library's stage entry points."""

    def __init__(self, device=0, stream=None, points=EDGE + 1, tol=1e-6, max_cycles=40):
        import torch
        self.grid = field_grid(points)
        torch.cuda.set_device(device)
        self.stream = _torch_stream(stream)
        cfg = default_config(device=device)
        cfg.stream = self.stream.cuda_stream
        self.ctx = Context(cfg)
        self.tol, self.max_cycles = tol, max_cycles

    def rhs(self, ps, w, out):
        c = self.ctx
        with _Ordered(self.stream):
            c.check(lib().vg_splat_device(c.h, ctypes.byref(self.grid), ctypes.c_void_p(ps.data_ptr()),
                                          ctypes.c_void_p(w.data_ptr()), ps.shape[0], -1.0,
                                          ctypes.c_void_p(out.data_ptr())), "vg_splat_device")

    def boundary(self, ps, w, vp):
        c = self.ctx
        vp.zero_()
        with _Ordered(self.stream):
            c.check(lib().vg_boundary_vecpot_device(c.h, ctypes.byref(self.grid), ctypes.c_void_p(ps.data_ptr()),
                                                    ctypes.c_void_p(w.data_ptr()), ps.shape[0], 0,
                                                    ctypes.c_void_p(vp.data_ptr())), "vg_boundary_vecpot_device")

    def multigrid(self, rhs, vp, tol=None):
        """(cycles, relres0, relres); synchronises (the cycle count is read on the host)."""
        c = self.ctx
        cyc, r0, r1 = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        with _Ordered(self.stream):
            st = lib().vg_multigrid_device(c.h, ctypes.byref(self.grid), ctypes.c_void_p(vp.data_ptr()),
                                           ctypes.c_void_p(rhs.data_ptr()), tol or self.tol, self.max_cycles,
                                           ctypes.byref(cyc), ctypes.byref(r0), ctypes.byref(r1))
        if st != OK and st != 8:  # VG_NOT_CONVERGED still leaves the best solution
            c.check(st, "vg_multigrid_device")
        return cyc.value, r0.value, r1.value

    def down(self, fine3, coarse, coarse3):
        """Full-weighting restriction of a field on this grid to `coarse` (DownSampleInto)."""
        c = self.ctx
        with _Ordered(self.stream):
            c.check(lib().vg_downsample_device(c.h, ctypes.byref(self.grid), ctypes.c_void_p(fine3.data_ptr()),
                                               ctypes.byref(coarse), 0, ctypes.c_void_p(coarse3.data_ptr())),
                    "vg_downsample_device")

    def up(self, coarse, coarse3, fine3):
        """Trilinear prolongation of a field on `coarse` to this grid's interior points (UpSampleFrom)."""
        c = self.ctx
        with _Ordered(self.stream):
            c.check(lib().vg_upsample_device(c.h, ctypes.byref(coarse), ctypes.c_void_p(coarse3.data_ptr()),
                                             ctypes.byref(self.grid), 1, ctypes.c_void_p(fine3.data_ptr())),
                    "vg_upsample_device")

    def direct(self, ps, w, q, out):
        """Direct-sum velocity of the vortons at q (float4 rows) into out."""
        c = self.ctx
        with _Ordered(self.stream):
            c.check(lib().vg_direct_device(c.h, 0, ctypes.c_void_p(ps.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                                           ps.shape[0], ctypes.c_void_p(q.data_ptr()), q.shape[0], 1.0, 1.0,
                                           ctypes.c_void_p(out.data_ptr())), "vg_direct_device")

    def solve(self, ps, w, rhs, vp):
        self.rhs(ps, w, rhs)
        self.boundary(ps, w, vp)
        return self.multigrid(rhs, vp)


def output_scale(rhs_list, vp_list, grid):
    """K such that the scaled solution vp / (s h^2 K) has unit RMS on average."""
    cell = np.asarray(list(grid.cell_spacing), np.float64)
    h2 = float(np.mean(cell ** 2))
    ratios = []
    for r, v in zip(rhs_list, vp_list):
        s = float(r.double().pow(2).mean().sqrt())
        ratios.append(float(v.double().pow(2).mean().sqrt()) / (s * h2))
    return float(np.mean(ratios))


# ------------------------------------------------------------------ training

def make_pairs(torch, solver, count, seed0, log=None):
    pts = solver.grid.capacity
    R = torch.empty((count, pts * 3), dtype=torch.bfloat16, device="cuda")
    V = torch.empty((count, pts * 3), dtype=torch.bfloat16, device="cuda")
    rhs = torch.empty(pts * 3, dtype=torch.float32, device="cuda")
    vp = torch.empty(pts * 3, dtype=torch.float32, device="cuda")
    t0 = time.time()
    for i in range(count):
        ps, w = make_field(field_kind(i), seed0 + i)
        solver.solve(ps, w, rhs, vp)
        with _Ordered(solver.stream):
            for src, dst in ((rhs, R[i]), (vp, V[i])):
                st = lib().vg_net_to_bf16_device(ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                                                 src.numel(), ctypes.c_void_p(solver.stream.cuda_stream))
                if st != OK:
                    raise VgError(st, "vg_net_to_bf16_device")
        if log and (i + 1) % 500 == 0:
            torch.cuda.synchronize()
            log(f"pairs {i + 1}/{count}  {time.time() - t0:.1f} s")
    torch.cuda.synchronize()
    return R, V


def train(pairs=4000, epochs=3, lr=3e-4, seed=0, out=DEFAULT_WEIGHTS, log=print, device=0, batch=4,
          log_every=50, max_seconds=None):
    """Generates `pairs` solver pairs (cached on the device in BF16) and trains
    the network for `epochs` passes over them with Adam on batches of `batch`
    fields (gradients accumulated in the library), warm-up then cosine decay."""
    import torch
    torch.cuda.set_device(device)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        return _train(torch, stream, pairs, epochs, lr, seed, out, log, device, batch, log_every, max_seconds)


def _train(torch, stream, pairs, epochs, lr, seed, out, log, device, batch, log_every, max_seconds):
    solver = Solver(device, stream)
    grid = solver.grid
    t0 = time.time()
    R, V = make_pairs(torch, solver, pairs, seed0=1_000_000 * (seed + 1), log=log)
    t_pairs = time.time() - t0
    K = output_scale([R[i].float() for i in range(min(64, pairs))], [V[i].float() for i in range(min(64, pairs))],
                     grid)
    log(f"{pairs} pairs in {t_pairs:.1f} s; output scale K = {K:.4g}")
    net = Network(EDGE, device, stream)
    net.set_params(init_params(seed), K)
    order = np.concatenate([np.random.default_rng(seed + ep).permutation(pairs) for ep in range(epochs)])
    total = len(order) // batch
    warm = max(1, min(100, total // 10))
    hist = []
    t1 = time.time()
    step = 0
    for step in range(total):
        frac = step / max(1, total - 1)
        lr_t = lr * min(1.0, (step + 1) / warm) * (0.05 + 0.95 * 0.5 * (1 + math.cos(math.pi * frac)))
        want = step % log_every == 0 or step == total - 1
        losses = []
        for b in range(batch):
            i = int(order[step * batch + b])
            losses.append(net.backward(grid, R[i], V[i], want_loss=want, accumulate=b > 0))
        net.adam_step(lr_t)  # Adam normalises the summed gradient
        if want:
            hist.append((step, float(np.mean(losses))))
            log(f"step {step}/{total} loss {hist[-1][1]:.4e} lr {lr_t:.2e} {time.time() - t1:.1f} s")
        if max_seconds and time.time() - t1 > max_seconds:
            log(f"stopping at the time limit after {step + 1} steps")
            break
    torch.cuda.synchronize()
    t_train = time.time() - t1
    steps = step + 1
    net.save(out)
    log(f"trained {steps} steps x {batch} fields in {t_train:.1f} s "
        f"({1e3 * t_train / max(1, steps * batch):.2f} ms/field); saved {out}")
    return {"pairs": pairs, "epochs": epochs, "batch": batch, "steps": steps, "seconds_pairs": t_pairs,
            "seconds_train": t_train, "ms_per_field": 1e3 * t_train / max(1, steps * batch), "out_scale": K,
            "loss": hist}


def evaluate(weights=DEFAULT_WEIGHTS, fields=200, seed=7, device=0, log=print, dt=1.0 / 30.0):
    """Cycles and solve time to 1e-6 from zero, previous-frame and network warm
    starts on held-out seeded fields (seeds disjoint from training)."""
    import torch
    torch.cuda.set_device(device)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        return _evaluate(torch, stream, weights, fields, seed, device, log, dt)


def _evaluate(torch, stream, weights, fields, seed, device, log, dt):
    solver = Solver(device, stream)
    net = Network(EDGE, device, stream)
    net.load(weights)
    pts = solver.grid.capacity
    rhs = torch.empty(pts * 3, dtype=torch.float32, device="cuda")
    vp0 = torch.empty_like(rhs)
    vp = torch.empty_like(rhs)
    prev = torch.empty_like(rhs)
    sol_full, solz, diff = torch.empty_like(rhs), torch.empty_like(rhs), torch.empty_like(rhs)
    g = solver.grid
    coarse = []
    for name, div in (("coarse65", 2), ("coarse33", 4)):
        pts_c = (int(g.num_points[0]) - 1) // div + 1
        cg = GridGeom.make(list(g.min_corner), list(g.extent), [pts_c] * 3)
        coarse.append((name, cg, torch.zeros(cg.capacity * 3, dtype=torch.float32, device="cuda")))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rows = []

    def timed(fn):
        e0.record(stream)
        r = fn()
        e1.record(stream)
        e1.synchronize()
        return r, e0.elapsed_time(e1)

    for f in range(fields):
        kind = field_kind(f)
        ps, w = make_field(kind, 9_000_000_000 + 1000 * seed + f)
        # previous frame: the same field one step earlier (vortons moved back along their direct-sum velocity)
        vel = torch.zeros_like(ps)
        solver.direct(ps, w, ps, vel)
        ps_prev = ps.clone()
        ps_prev[:, :3] -= dt * vel[:, :3]
        solver.solve(ps_prev, w, rhs, prev)
        solver.rhs(ps, w, rhs)
        solver.boundary(ps, w, vp0)
        row = {"kind": kind}
        bmask = boundary_mask(torch, pts_axis=solver.grid.num_points[0])
        interior = ~bmask
        vp.copy_(vp0)
        (row["zero_cycles"], row["zero_relres0"], row["zero_relres"]), row["zero_ms"] = timed(
            lambda: solver.multigrid(rhs, vp))
        sol = vp[interior].double()
        sol_norm = float(sol.norm())
        sol_full.copy_(vp)

        def start_error(start):
            return float((start[interior].double() - sol).norm()) / sol_norm

        # previous frame: this frame's boundary values, the interior of the previous frame's solution
        vp.copy_(prev)
        vp[bmask] = vp0[bmask]
        row["prev_err0"] = start_error(vp)
        (row["prev_cycles"], row["prev_relres0"], row["prev_relres"]), row["prev_ms"] = timed(
            lambda: solver.multigrid(rhs, vp))
        # ceilings of a warm start that predicts only the smooth part: the converged
        # solution restricted to a coarse grid and prolonged back (what an exact coarse
        # network could give), alone and on top of the previous frame
        solz.copy_(sol_full)
        for name, cg, cbuf in coarse:
            vp.copy_(vp0)
            solver.down(solz, cg, cbuf)
            solver.up(cg, cbuf, vp)
            row[name + "_err0"] = start_error(vp)
            (row[name + "_cycles"], row[name + "_relres0"], _), row[name + "_ms"] = timed(
                lambda: solver.multigrid(rhs, vp))
        name, cg, cbuf = coarse[0]
        diff.copy_(solz - prev)
        solver.down(diff, cg, cbuf)
        vp.zero_()
        solver.up(cg, cbuf, vp)
        vp += prev
        vp[bmask] = vp0[bmask]
        row["prev_coarse65_err0"] = start_error(vp)
        (row["prev_coarse65_cycles"], row["prev_coarse65_relres0"], _), row["prev_coarse65_ms"] = timed(
            lambda: solver.multigrid(rhs, vp))
        vp.copy_(vp0)
        _, row["nn_guess_ms"] = timed(lambda: net.guess(solver.grid, rhs, vp))
        row["nn_err0"] = start_error(vp)
        (row["nn_cycles"], row["nn_relres0"], row["nn_relres"]), row["nn_mg_ms"] = timed(
            lambda: solver.multigrid(rhs, vp))
        row["nn_ms"] = row["nn_guess_ms"] + row["nn_mg_ms"]
        # both solves end at the same tolerance: their solutions agree to about it
        row["nn_vs_zero_solution"] = float((vp[interior].double() - sol).norm()) / sol_norm
        rows.append(row)
        if log and (f + 1) % 20 == 0:
            log(f"eval {f + 1}/{fields}: " + json.dumps(summarise(rows)))
    return summarise(rows), rows


_BMASK = {}


def boundary_mask(torch, pts_axis):
    m = _BMASK.get(pts_axis)
    if m is None:
        i = torch.arange(pts_axis, device="cuda")
        b = (i == 0) | (i == pts_axis - 1)
        m = (b[:, None, None] | b[None, :, None] | b[None, None, :]).reshape(-1)
        m = m[:, None].expand(-1, 3).reshape(-1)
        _BMASK[pts_axis] = m
    return m


def summarise(rows):
    out = {"fields": len(rows)}
    for k in ("zero_cycles", "prev_cycles", "nn_cycles", "zero_ms", "prev_ms", "nn_guess_ms", "nn_mg_ms", "nn_ms",
              "zero_relres0", "prev_relres0", "nn_relres0", "prev_err0", "nn_err0", "nn_vs_zero_solution",
              "coarse65_cycles", "coarse65_ms", "coarse65_relres0", "coarse65_err0",
              "coarse33_cycles", "coarse33_ms", "coarse33_relres0", "coarse33_err0",
              "prev_coarse65_cycles", "prev_coarse65_ms", "prev_coarse65_relres0", "prev_coarse65_err0"):
        if not rows or k not in rows[0]:
            continue
        v = [r[k] for r in rows]
        out[k] = float(np.median(v))
        out[k + "_mean"] = float(np.mean(v))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=4000)
    t.add_argument("--epochs", type=int, default=3)
    t.add_argument("--lr", type=float, default=3e-4)
    t.add_argument("--batch", type=int, default=4)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--out", default=DEFAULT_WEIGHTS)
    t.add_argument("--max-seconds", type=float, default=None)
    t.add_argument("--report", default=None)
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=DEFAULT_WEIGHTS)
    e.add_argument("--fields", type=int, default=200)
    e.add_argument("--report", default=None)
    a = ap.parse_args(argv)
    log = lambda s: print(s, flush=True)  # noqa: E731
    if a.cmd == "train":
        rep = train(a.pairs, a.epochs, a.lr, a.seed, a.out, log, batch=a.batch, max_seconds=a.max_seconds)
    else:
        rep, rows = evaluate(a.weights, a.fields, log=log)
        rep = {"summary": rep, "rows": rows}
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
    print(json.dumps(rep if a.cmd == "train" else rep["summary"]))


if __name__ == "__main__":
    main(sys.argv[1:])
