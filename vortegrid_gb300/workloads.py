"""Seeded synthetic vorton fields for the benchmark and parity workloads.

All fields are generated with numpy from a fixed seed, so every run and every
machine sees the same inputs.  Vortons are returned in the reference's
storage convention: ``angvel`` = vorticity / 2 and ``size`` = diameter
(Particles/particle.h:425-430, VortonFluid/vorton.h:316-332).

Workloads (sizes as stated; nothing here reads external data):
  * ``ring``   -- one vortex ring: major radius R, tube radius a, positions
    uniform in the tube cross-section, vorticity tangential to the ring with
    magnitude peak * exp(-r^2 / (2 sigma^2)).
  * ``rings``  -- several randomly placed, randomly oriented rings inside a box.
  * ``puff``   -- a turbulent puff: Gaussian positions, i.i.d. normal vorticity.
  * ``tracers``-- passive tracers uniform in a box.
"""
import numpy as np

VORTON_RADIUS = 0.05


def ring(n, seed=1, major=1.0, tube=0.25, sigma=0.1, peak=10.0, radius=VORTON_RADIUS, center=(0.0, 0.0, 0.0),
         axis=(0.0, 0.0, 1.0), rng=None):
    rng = rng if rng is not None else np.random.default_rng(seed)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    theta = rng.uniform(0.0, 2.0 * np.pi, n)
    r = tube * np.sqrt(rng.uniform(0.0, 1.0, n))
    rho = major + r * np.cos(theta)
    local = np.stack([rho * np.cos(phi), rho * np.sin(phi), r * np.sin(theta)], axis=1)
    mag = peak * np.exp(-r * r / (2.0 * sigma * sigma))
    vort = np.stack([-np.sin(phi) * mag, np.cos(phi) * mag, np.zeros(n)], axis=1)
    # rotate local z onto `axis`
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    z = np.array([0.0, 0.0, 1.0])
    v = np.cross(z, a)
    s, c = np.linalg.norm(v), float(np.dot(z, a))
    if s < 1e-12:
        R = np.eye(3) if c > 0 else np.diag([1.0, -1.0, -1.0])
    else:
        vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
        R = np.eye(3) + vx + vx @ vx * ((1 - c) / (s * s))
    pos = local @ R.T + np.asarray(center)
    vort = vort @ R.T
    return (pos.astype(np.float32), (0.5 * vort).astype(np.float32),
            np.full(n, 2.0 * radius, np.float32))


def rings(n, count=8, seed=2, box=2.0, major=(0.3, 1.0), tube=0.25, radius=VORTON_RADIUS):
    rng = np.random.default_rng(seed)
    sizes = np.full(count, n // count)
    sizes[: n - sizes.sum()] += 1
    P, W, S = [], [], []
    for k in range(count):
        R = rng.uniform(*major)
        lim = box - R - tube
        c = rng.uniform(-lim, lim, 3)
        ax = rng.normal(size=3)
        p, w, s = ring(int(sizes[k]), major=R, tube=tube, center=c, axis=ax, radius=radius, rng=rng)
        P.append(p); W.append(w); S.append(s)
    return np.concatenate(P), np.concatenate(W), np.concatenate(S)


def puff(n, seed=3, sigma=0.5, clip=1.9, vort_sigma=2.0, radius=VORTON_RADIUS):
    rng = np.random.default_rng(seed)
    pos = np.clip(rng.normal(0.0, sigma, (n, 3)), -clip, clip)
    vort = rng.normal(0.0, vort_sigma, (n, 3))
    return pos.astype(np.float32), (0.5 * vort).astype(np.float32), np.full(n, 2.0 * radius, np.float32)


def tracers(m, seed=4, lo=-1.5, hi=1.5):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, (m, 3)).astype(np.float32)


def grid_points(mn, cell, np3):
    """Gridpoint positions min + i * spacing, x fastest."""
    xs = [mn[a] + np.arange(np3[a], dtype=np.float32) * np.float32(cell[a]) for a in range(3)]
    z, y, x = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float32)
