"""Batched effects: many independent vorton simulations stepped per frame
through the library's batch API (vg_batch_* in include/vortegrid.h): each
frame replayed from CUDA graphs on parallel branches, multigrid schedules
fixed by a calibration step, the stream count chosen by the batch autotuner.

Effects (seeded): vorton counts log-uniform in [1,024, 65,536]; each a ring
field (1-4 rings, major radius U[0.3, 0.9] x half-box, a Gaussian tube
profile) or a puff (Gaussian positions, sigma U[0.2, 0.5] x half-box,
vorticity N(0, 2^2)); vorton half-box L ~ U[0.6, 2.8]; a fixed cubic grid of
half-width 1.6 L (room for the vortons to move for many frames; a vorton that
still leaves it stops and drops out of its simulation), with 16 to 96 cells
per axis chosen from the extent (spacing ~1/16, rounded to a multiple of 16).
"""
import ctypes
import math

import numpy as np

from . import OK, VgError, GridGeom, StepStats, default_config, lib, VELOCITY_POISSON

H0 = 1.0 / 16.0
GRID_MARGIN = 1.6


class Effect:
    def __init__(self, pos, vort, radius, grid):
        self.pos, self.vort, self.radius, self.grid = pos, vort, radius, grid

    @property
    def n(self):
        return len(self.pos)


def _rotation_to(ax):
    z = np.array([0.0, 0.0, 1.0])
    v = np.cross(z, ax)
    s, c = np.linalg.norm(v), float(ax[2])
    if s < 1e-9:
        return np.eye(3) if c > 0 else np.diag([1.0, -1.0, -1.0])
    vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + vx + vx @ vx * ((1 - c) / (s * s))


def make_effect(seed):
    rng = np.random.default_rng(seed)
    n = int(round(math.exp(rng.uniform(math.log(1024), math.log(65536)))))
    L = rng.uniform(0.6, 2.8)
    if rng.random() < 0.5:
        k = int(rng.integers(1, 5))
        sizes = np.full(k, n // k)
        sizes[: n - sizes.sum()] += 1
        P, W = [], []
        for m in sizes:
            R = rng.uniform(0.3, 0.9) * L * 0.5
            tube = 0.25 * R
            c = rng.uniform(-1, 1, 3) * max(L - R - tube, 0.0) * 0.8
            ax = rng.normal(size=3)
            ax /= np.linalg.norm(ax)
            phi, theta = rng.uniform(0, 2 * np.pi, (2, m))
            r = tube * np.sqrt(rng.uniform(0, 1, m))
            rho = R + r * np.cos(theta)
            local = np.stack([rho * np.cos(phi), rho * np.sin(phi), r * np.sin(theta)], 1)
            mag = 10.0 * np.exp(-r * r / (2 * (0.4 * tube) ** 2))
            vort = np.stack([-np.sin(phi) * mag, np.cos(phi) * mag, np.zeros(m)], 1)
            Rm = _rotation_to(ax)
            P.append(local @ Rm.T + c)
            W.append(vort @ Rm.T)
        pos, vort = np.concatenate(P), np.concatenate(W)
    else:
        sigma = rng.uniform(0.2, 0.5) * L
        pos = np.clip(rng.normal(0, sigma, (n, 3)), -0.95 * L, 0.95 * L)
        vort = rng.normal(0, 2.0, (n, 3))
    half = GRID_MARGIN * L
    cells = int(min(96, max(16, 16 * round(2 * half / H0 / 16))))
    grid = GridGeom.make([-half] * 3, [2 * half] * 3, [cells + 1] * 3)
    radius = 1.5 * (2 * half / cells)
    return Effect(pos.astype(np.float32), vort.astype(np.float32), radius, grid)


class Batch:
    """One vg_batch with its simulations' device arrays (torch tensors)."""

    def __init__(self, effects, streams=8, device=0, viscosity=0.01):
        import torch
        h = ctypes.c_void_p()
        st = lib().vg_batch_create(device, streams, ctypes.byref(h))
        if st != OK:
            raise VgError(st, "vg_batch_create: " + lib().vg_last_error(None).decode())
        self.h = h
        self.arrays = []
        for e in effects:
            ps = np.zeros((e.n, 4), np.float32)
            ps[:, :3] = e.pos
            ps[:, 3] = 2 * e.radius
            w = np.zeros((e.n, 4), np.float32)
            w[:, :3] = 0.5 * e.vort
            P, W = torch.from_numpy(ps).cuda(device), torch.from_numpy(w).cuda(device)
            V = torch.zeros_like(P)
            self.arrays.append((P, W, V))
            cfg = default_config(fixed_grid=e.grid, device=device, viscosity=viscosity)
            cfg.velocity_technique = VELOCITY_POISSON
            cfg.enable_stretch = 0
            self.check(lib().vg_batch_add(self.h, ctypes.byref(cfg), ctypes.c_void_p(P.data_ptr()),
                                          ctypes.c_void_p(W.data_ptr()), ctypes.c_void_p(V.data_ptr()), e.n, None),
                       "vg_batch_add")
        torch.cuda.synchronize(device)

    def check(self, st, what):
        if st != OK:
            raise VgError(st, f"{what}: {lib().vg_batch_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            lib().vg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_network(self, path):
        self.check(lib().vg_batch_load_network(self.h, path.encode()), "vg_batch_load_network")

    def configure(self, streams, use_network):
        self.check(lib().vg_batch_configure(self.h, streams, 1 if use_network else 0), "vg_batch_configure")

    def calibrate(self, dt):
        self.check(lib().vg_batch_calibrate(self.h, dt), "vg_batch_calibrate")

    def step(self, dt, graph=True):
        self.check(lib().vg_batch_step(self.h, dt, 0 if graph else 1), "vg_batch_step")

    def synchronize(self):
        self.check(lib().vg_batch_synchronize(self.h), "vg_batch_synchronize")

    def autotune(self, dt, frames=3, candidates=(1, 2, 4, 8, 16, 32)):
        c = (ctypes.c_int * len(candidates))(*candidates)
        bs, bn, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        self.check(lib().vg_batch_autotune(self.h, dt, frames, c, len(candidates), ctypes.byref(bs), ctypes.byref(bn),
                                           ctypes.byref(ms)), "vg_batch_autotune")
        return bs.value, bool(bn.value), ms.value

    def outside(self, i):
        """Whether vortons of simulation i left its grid since the last call
        (they stop and drop out of the solve)."""
        o = ctypes.c_int()
        self.check(lib().vg_batch_outside(self.h, i, ctypes.byref(o)), "vg_batch_outside")
        return bool(o.value)

    def stats(self, i):
        """Step statistics of simulation i (after synchronize())."""
        s = StepStats()
        ctx = lib().vg_batch_context(self.h, i)
        st = lib().vg_get_stats(ctx, ctypes.byref(s))
        if st != OK:
            raise VgError(st, "vg_get_stats: " + lib().vg_last_error(ctx).decode())
        return s

    def velocity_grid(self, i):
        """Simulation i's velocity grid from its last step (after synchronize()):
        (float32[points, 3], GridGeom)."""
        ctx = lib().vg_batch_context(self.h, i)
        g = GridGeom()
        st = lib().vg_get_velocity_grid(ctx, None, 0, ctypes.byref(g))
        if st != OK:
            raise VgError(st, "vg_get_velocity_grid: " + lib().vg_last_error(ctx).decode())
        out = np.zeros((g.capacity, 3), np.float32)
        st = lib().vg_get_velocity_grid(ctx, out.ctypes.data_as(ctypes.c_void_p), g.capacity, ctypes.byref(g))
        if st != OK:
            raise VgError(st, "vg_get_velocity_grid: " + lib().vg_last_error(ctx).decode())
        return out, g

    def graph_info(self):
        """(graphs launched per frame, largest graph's nodes, total nodes)."""
        g, mx, tot = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_size_t()
        self.check(lib().vg_batch_graph_info(self.h, ctypes.byref(g), ctypes.byref(mx), ctypes.byref(tot)),
                   "vg_batch_graph_info")
        return g.value, mx.value, tot.value

    def set_solver(self, persistent=True, team_ctas=0, max_points=0):
        """Poisson solves of qualifying simulations (grids of at most
        max_points points; 0 = any) in one persistent launch per frame (teams
        of team_ctas CTAs; 0 = automatic), or inside each simulation's branch
        graphs."""
        self.check(lib().vg_batch_set_solver(self.h, 1 if persistent else 0, team_ctas, max_points),
                   "vg_batch_set_solver")

    def solver_info(self):
        """(simulations in the persistent launch, teams, CTAs per team, launch captured as a graph)."""
        n, t, c, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.check(lib().vg_batch_solver_info(self.h, ctypes.byref(n), ctypes.byref(t), ctypes.byref(c),
                                              ctypes.byref(g)), "vg_batch_solver_info")
        return n.value, t.value, c.value, bool(g.value)

    def __len__(self):
        return lib().vg_batch_size(self.h)
