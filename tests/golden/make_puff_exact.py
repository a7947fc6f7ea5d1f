#!/usr/bin/env python3
"""Golden fixture for the multigrid workload's velocity check
(tests/golden/puff129_exact.npz).

The workload: 262,144 puff vortons (positions N(0, 0.5^2) clipped to +-1.9,
vorticity N(0, 2^2), radius 0.05; vortegrid_gb300.workloads.puff, seed 3) on
the 129^3 grid of [-2, 2]^3 (dx = 1/32).  On the CPU, with the C oracle:
  * the right-hand side is the splat of -vorticity (PopulateVorticityGridFromVortons);
  * the boundary is the reference treecode's vector potential at every
    boundary point (ComputeVectorPotentialAtGridpoints_Slice, boundaries only,
    no odd-x copy);
  * `exact` solves the same discrete Dirichlet problem in FP64 (scipy CG on the
    7-point Laplacian to 1e-9);
  * `cascade` is the reference's own solver at its fixed work (16 SOR sweeps
    per level of its cascade, vortonSim.cpp:2523-2608), which stalls;
  * velocities are the curl of each (ComputeJacobian + ComputeCurlFromJacobian);
  * `direct` is the FP64 direct sum at the same points.
Saved at 512 interior points drawn with seed 11 from [8, 121)^3.

Run from the repository root: python tests/golden/make_puff_exact.py (about a minute).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

N = 129
H = 1.0 / 32.0


def sample_points():
    idx = np.random.default_rng(11).integers(8, N - 8, (512, 3))
    return idx[:, 0] + N * (idx[:, 1] + N * idx[:, 2])


def exact_solve(b, a0):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    def lap1(m):
        return sp.diags([np.ones(m - 1), -2 * np.ones(m), np.ones(m - 1)], [-1, 0, 1]) / (H * H)
    L = sp.kronsum(sp.kronsum(lap1(N - 2), lap1(N - 2)), lap1(N - 2)).tocsr()
    A = a0.reshape(N, N, N, 3).astype(np.float64).copy()
    B = b.reshape(N, N, N, 3)
    for c in range(3):
        rhs = B[1:-1, 1:-1, 1:-1, c].astype(np.float64).copy()
        Ac = A[..., c]
        rhs[:, :, 0] -= Ac[1:-1, 1:-1, 0] / H ** 2
        rhs[:, :, -1] -= Ac[1:-1, 1:-1, -1] / H ** 2
        rhs[:, 0, :] -= Ac[1:-1, 0, 1:-1] / H ** 2
        rhs[:, -1, :] -= Ac[1:-1, -1, 1:-1] / H ** 2
        rhs[0, :, :] -= Ac[0, 1:-1, 1:-1] / H ** 2
        rhs[-1, :, :] -= Ac[-1, 1:-1, 1:-1] / H ** 2
        x, info = spl.cg(L, rhs.ravel(), rtol=1e-9, maxiter=4000)
        assert info == 0, info
        A[1:-1, 1:-1, 1:-1, c] = x.reshape(N - 2, N - 2, N - 2)
    return A.reshape(-1, 3).astype(np.float32)


def main():
    import oracle
    from vortegrid_gb300 import workloads
    oracle.build()
    pos, w, s = workloads.puff(262144, seed=3)
    g = oracle.Geom.from12(np.array([-2, -2, -2, 4, 4, 4, H, H, H, 32, 32, 32], np.float32), (N, N, N))
    b = oracle.splat(pos, w, s, g, -1.0)
    a0 = oracle.boundary_vecpot(pos, w, s, g, True, False)
    flat = sample_points()
    pts = workloads.grid_points([-2.0] * 3, [H] * 3, [N] * 3)[flat]
    exact = exact_solve(b, a0)
    casc = oracle.cascade(g, oracle.boundary_vecpot(pos, w, s, g, True, True), b, 16)
    vel = {}
    for name, a in (("exact", exact), ("cascade", casc)):
        vel[name] = oracle.curl_from_jacobian(oracle.jacobian(g, a))[flat]
    direct = oracle.direct(0, pos, w, s, pts, f64=True)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "puff129_exact.npz")
    np.savez_compressed(out, flat=flat, exact_vel=vel["exact"], cascade_vel=vel["cascade"], direct=direct,
                        exact_relres=np.float64(oracle.relres(g, exact, b)),
                        cascade_relres=np.float64(oracle.relres(g, casc, b)))
    for name in ("exact", "cascade"):
        e = np.linalg.norm(vel[name] - direct) / np.linalg.norm(direct)
        print(f"{name}: velocity rel-L2 vs FP64 direct sum {e:.4f}")
    print("wrote", out)


if __name__ == "__main__":
    main()
