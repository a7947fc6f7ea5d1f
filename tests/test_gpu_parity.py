"""GPU parity of every stage of the VortonSim step, through the C ABI.

Each test runs one stage of libvortegrid on cuda:0 on the golden inputs and
compares it with the golden outputs that the reference's own code produced
(tests/golden/reference.npz) or with the C oracle:
  * REFERENCE numerics: bit-exact (uint32 view) for every FP32 stage whose
    summation order the reference fixes;
  * FAST numerics: stated relative-L2 tolerances against the FP64 oracle;
  * PSE (order-dependent in the reference): 1e-3 relative L2 on vorticity.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

DT = np.float32(1.0 / 30.0)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def f4(xyz, w=None):
    out = np.zeros((len(xyz), 4), np.float32)
    out[:, :3] = xyz
    if w is not None:
        out[:, 3] = w
    return out


@pytest.fixture(scope="module")
def vg():
    import vortegrid_gb300 as vg
    vg.lib()
    return vg


@pytest.fixture(scope="module")
def ref_ctx(vg):
    return vg.Context(numerics=vg.NUMERICS_REFERENCE)


@pytest.fixture(scope="module")
def fast_ctx(vg):
    return vg.Context(numerics=vg.NUMERICS_FAST)


def geom(vg, golden):
    return vg.GridGeom.from12(golden["geom"], golden["np"])


def vortons(golden):
    return dev(f4(golden["pos"], golden["size"])), dev(f4(golden["angvel"]))


def sync():
    torch.cuda.synchronize()


def test_binning_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    p = dev(f4(golden["bin_pos"]))
    idx = torch.zeros((len(golden["bin_pos"]), 3), dtype=torch.int32, device="cuda")
    off = torch.zeros(len(golden["bin_pos"]), dtype=torch.int32, device="cuda")
    ref_ctx.check(vg.lib().vg_bin_device(ref_ctx.h, ctypes.byref(g), vg._ptr(p), len(p), vg._ptr(idx), vg._ptr(off)),
                  "bin")
    sync()
    assert np.array_equal(idx.cpu().numpy().view(np.uint32), golden["bin_idx"])
    assert np.array_equal(off.cpu().numpy().view(np.uint32), golden["bin_off"])


@pytest.mark.parametrize("kind,name", [(0, "vel"), (1, "vecpot")])
def test_direct_reference_bit_exact(vg, ref_ctx, golden, kind, name):
    ps, w = vortons(golden)
    q = dev(f4(golden["q"]))
    out = torch.zeros((len(q), 4), dtype=torch.float32, device="cuda")
    ref_ctx.check(vg.lib().vg_direct_device(ref_ctx.h, kind, vg._ptr(ps), vg._ptr(w), len(ps), vg._ptr(q), len(q),
                                            1.0, 1.0, vg._ptr(out)), "direct")
    sync()
    assert np.array_equal(bits(out.cpu().numpy()[:, :3]), bits(golden[f"direct_{name}"]))


@pytest.mark.parametrize("kind", [0, 1])
def test_direct_fast_vs_fp64(vg, fast_ctx, oracle_lib, kind):
    """FAST direct sum vs the FP64 oracle: rel-L2 <= 1e-5 (FP32 accumulation)."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(4096, seed=1)
    q = np.concatenate([workloads.grid_points([-1.5] * 3, [3 / 32] * 3, [33] * 3)[::5], pos[::3]])
    ref = oracle_lib.direct(kind, pos, w, s, q, f64=True)
    ps, wd, qd = dev(f4(pos, s)), dev(f4(w)), dev(f4(q))
    out = torch.zeros((len(q), 4), dtype=torch.float32, device="cuda")
    fast_ctx.check(vg.lib().vg_direct_device(fast_ctx.h, kind, vg._ptr(ps), vg._ptr(wd), len(ps), vg._ptr(qd), len(q),
                                             1.0, 1.0, vg._ptr(out)), "direct")
    sync()
    got = out.cpu().numpy()[:, :3].astype(np.float64)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < 1e-5, rel


def test_direct_step_matches_fp64(vg, oracle_lib):
    """The direct-technique step (FAST numerics; the ring of the bench's direct
    workload on its 33^3 grid): the velocity grid and every vorton's velocity,
    which the multi-chunk reduction writes straight into the grid and the
    vortons' records, against the FP64 direct sum at the step's gridpoint
    positions (min + i x spacing x (1 - 2 FLT_EPSILON)): rel-L2 <= 1e-5."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(4096, seed=1)
    grid = vg.GridGeom.make([-1.5] * 3, [3.0] * 3, [33] * 3)
    cfg = vg.default_config(velocity_technique=vg.VELOCITY_DIRECT, fixed_grid=grid, enable_stretch=0,
                            enable_diffusion=0, device=0)
    ctx = vg.VortonSim(cfg=cfg)
    ps, wd = dev(f4(pos, s)), dev(f4(w))
    vel = torch.zeros_like(ps)
    ctx.UpdateDevice(ps, wd, vel, float(DT))
    vgrid, g = ctx.GetVelocityGrid()
    nudge = np.float32(1.0) - np.float32(2.0) * np.finfo(np.float32).eps
    axes = []
    for a in range(3):
        step = np.float32(g.cell_spacing[a]) * nudge
        axes.append(np.float32(g.min_corner[a]) + np.arange(g.num_points[a], dtype=np.float32) * step)
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    q = np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(np.float32)
    ref_grid = oracle_lib.direct(0, pos, w, s, q, f64=True)
    ref_vort = oracle_lib.direct(0, pos, w, s, pos, f64=True)
    got_v = vel.cpu().numpy()[:, :3].astype(np.float64)
    assert np.linalg.norm(vgrid - ref_grid) / np.linalg.norm(ref_grid) < 1e-5
    assert np.linalg.norm(got_v - ref_vort) / np.linalg.norm(ref_vort) < 1e-5
    assert np.all(vel.cpu().numpy()[:, 3] == 0.0)


@pytest.mark.parametrize("shape,n,with_vortons", [((33, 33, 33), 4096, True), ((24, 9, 5), 4096, True),
                                                  ((29, 17, 11), 300, True), ((5, 7, 9), 4096, True),
                                                  ((64, 20, 3), 2000, False), ((9, 2, 2), 40, False)])
def test_direct_grid_vs_fp64(vg, fast_ctx, oracle_lib, shape, n, with_vortons):
    """vg_direct_grid_device (FAST numerics): the velocity at every gridpoint
    of grid shapes whose rows split into whole 8-point segments (24), leave a
    remainder (33, 29, 9), or are shorter than a segment (5), with and without
    the vortons as targets, one source chunk (40 vortons) or many: rel-L2
    <= 1e-5 against the FP64 direct sum at the step's gridpoint positions."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(n, seed=3)
    mn = np.array([-1.4, -1.3, -1.2], np.float32)
    ext = np.array([2.8, 2.7, 2.6], np.float32)
    grid = vg.GridGeom.make(mn, ext, list(shape))
    nudge = np.float32(1.0) - np.float32(2.0) * np.finfo(np.float32).eps
    axes = [np.float32(grid.min_corner[a]) + np.arange(shape[a], dtype=np.float32) *
            (np.float32(grid.cell_spacing[a]) * nudge) for a in range(3)]
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    q = np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(np.float32)
    ps, wd = dev(f4(pos, s)), dev(f4(w))
    vgrid = torch.full((q.shape[0], 3), np.nan, dtype=torch.float32, device="cuda")
    vel = torch.full((n, 4), np.nan, dtype=torch.float32, device="cuda") if with_vortons else None
    fast_ctx.check(vg.lib().vg_direct_grid_device(fast_ctx.h, ctypes.byref(grid), vg._ptr(ps), vg._ptr(wd), n,
                                                  vg._ptr(vgrid), vg._ptr(vel)), "direct grid")
    sync()
    ref = oracle_lib.direct(0, pos, w, s, q, f64=True)
    got = vgrid.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
    if with_vortons:
        rv = oracle_lib.direct(0, pos, w, s, pos, f64=True)
        gv = vel.cpu().numpy()
        assert np.linalg.norm(gv[:, :3] - rv) / np.linalg.norm(rv) < 1e-5 and np.all(gv[:, 3] == 0.0)


def test_tree_reference_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    ps, w = vortons(golden)
    q = dev(f4(golden["q"]))
    npts = ctypes.c_size_t()
    lib = vg.lib()
    ref_ctx.check(lib.vg_tree_device(ref_ctx.h, 0, ctypes.byref(g), vg._ptr(ps), vg._ptr(w), len(ps), None, 0, 1.0,
                                     1.0, None, None, 0, ctypes.byref(npts)), "tree size")
    tree = torch.zeros((npts.value, 8), dtype=torch.float32, device="cuda")
    sr, sc = golden["spread"]
    for kind, name in ((0, "vel"), (1, "vecpot")):
        for (a, b, suffix) in ((1.0, 1.0, ""), (float(sr), float(sc), "_spread")):
            out = torch.zeros((len(q), 4), dtype=torch.float32, device="cuda")
            ref_ctx.check(lib.vg_tree_device(ref_ctx.h, kind, ctypes.byref(g), vg._ptr(ps), vg._ptr(w), len(ps),
                                             vg._ptr(q), len(q), a, b, vg._ptr(out), vg._ptr(tree), npts.value,
                                             ctypes.byref(npts)), "tree")
            sync()
            assert np.array_equal(bits(out.cpu().numpy()[:, :3]), bits(golden[f"tree_{name}{suffix}"])), (name, suffix)
    t = tree.cpu().numpy()
    gt = golden["tree"]  # pos xyz, angvel xyz, size
    mine = np.concatenate([t[:, 0:3], t[:, 4:7], t[:, 3:4]], axis=1)
    assert np.array_equal(bits(mine), bits(gt))


def test_tree_fast_close(vg, fast_ctx, golden):
    g = geom(vg, golden)
    ps, w = vortons(golden)
    q = dev(f4(golden["q"]))
    out = torch.zeros((len(q), 4), dtype=torch.float32, device="cuda")
    npts = ctypes.c_size_t()
    fast_ctx.check(vg.lib().vg_tree_device(fast_ctx.h, 0, ctypes.byref(g), vg._ptr(ps), vg._ptr(w), len(ps),
                                           vg._ptr(q), len(q), 1.0, 1.0, vg._ptr(out), None, 0, ctypes.byref(npts)),
                   "tree")
    sync()
    ref = golden["tree_vel"]
    got = out.cpu().numpy()[:, :3]
    # the reference's magic-constant rsqrt carries ~1.8e-3 relative error per pair
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 3e-3


def test_splat_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    ps, w = vortons(golden)
    out = torch.zeros((g.capacity, 3), dtype=torch.float32, device="cuda")
    ref_ctx.check(vg.lib().vg_splat_device(ref_ctx.h, ctypes.byref(g), vg._ptr(ps), vg._ptr(w), len(ps), -1.0,
                                           vg._ptr(out)), "splat")
    sync()
    assert np.array_equal(bits(out.cpu().numpy()), bits(golden["negvort"]))


def test_boundary_vecpot_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    ps, w = vortons(golden)
    out = torch.zeros((g.capacity, 3), dtype=torch.float32, device="cuda")
    ref_ctx.check(vg.lib().vg_boundary_vecpot_device(ref_ctx.h, ctypes.byref(g), vg._ptr(ps), vg._ptr(w), len(ps), 1,
                                                     vg._ptr(out)), "boundary")
    sync()
    assert np.array_equal(bits(out.cpu().numpy()), bits(golden["boundary_vecpot"]))


def test_sor_and_cascade_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    rhs = dev(golden["negvort"])
    a = dev(golden["boundary_vecpot"])
    ref_ctx.check(vg.lib().vg_sor_device(ref_ctx.h, ctypes.byref(g), vg._ptr(a), vg._ptr(rhs), 5), "sor")
    sync()
    assert np.array_equal(bits(a.cpu().numpy()), bits(golden["sor5"]))
    a = dev(golden["boundary_vecpot"])
    ref_ctx.check(vg.lib().vg_cascade_device(ref_ctx.h, ctypes.byref(g), vg._ptr(a), vg._ptr(rhs), 16), "cascade")
    sync()
    assert np.array_equal(bits(a.cpu().numpy()), bits(golden["cascade"]))


def test_restrict_prolong_bit_exact(vg, ref_ctx, golden, oracle_lib):
    g = geom(vg, golden)
    og = oracle_lib.Geom.from12(golden["geom"], golden["np"])
    layers, _ = oracle_lib.nested_shape(og)
    cg = vg.GridGeom.from12(layers[1].as12(), layers[1].points)
    fine = dev(golden["cascade"])
    for inject, name in ((1, "inject"), (0, "average")):
        c = torch.zeros((cg.capacity, 3), dtype=torch.float32, device="cuda")
        ref_ctx.check(vg.lib().vg_downsample_device(ref_ctx.h, ctypes.byref(g), vg._ptr(fine), ctypes.byref(cg),
                                                    inject, vg._ptr(c)), "down")
        sync()
        assert np.array_equal(bits(c.cpu().numpy()), bits(golden[f"down_{name}"])), name
        for interior, rname in ((1, "interior"), (0, "entire")):
            f = dev(golden["cascade"])
            ref_ctx.check(vg.lib().vg_upsample_device(ref_ctx.h, ctypes.byref(cg), vg._ptr(c), ctypes.byref(g),
                                                      interior, vg._ptr(f)), "up")
            sync()
            assert np.array_equal(bits(f.cpu().numpy()), bits(golden[f"up_{name}_{rname}"])), (name, rname)


def test_jacobian_curl_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    a = dev(golden["cascade"])
    jac = torch.zeros((g.capacity, 9), dtype=torch.float32, device="cuda")
    curl = torch.zeros((g.capacity, 3), dtype=torch.float32, device="cuda")
    ref_ctx.check(vg.lib().vg_jacobian_curl_device(ref_ctx.h, ctypes.byref(g), vg._ptr(a), vg._ptr(jac),
                                                   vg._ptr(curl)), "jac")
    sync()
    assert np.array_equal(bits(jac.cpu().numpy()), bits(golden["jacobian"]))
    assert np.array_equal(bits(curl.cpu().numpy()), bits(golden["curl"]))


def test_stretch_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    ps, w = vortons(golden)
    vel = dev(golden["curl"])
    ref_ctx.check(vg.lib().vg_stretch_device(ref_ctx.h, ctypes.byref(g), vg._ptr(vel), vg._ptr(ps), vg._ptr(w),
                                             len(ps), float(DT)), "stretch")
    sync()
    assert np.array_equal(bits(w.cpu().numpy()[:, :3]), bits(golden["stretched"]))


def test_pse_tolerance(vg, ref_ctx, golden, oracle_lib):
    g = geom(vg, golden)
    ps, w = vortons(golden)
    ref_ctx.check(vg.lib().vg_pse_device(ref_ctx.h, ctypes.byref(g), vg._ptr(ps), vg._ptr(w), len(ps), 0.01,
                                         float(DT)), "pse")
    sync()
    got = w.cpu().numpy()[:, :3]
    ref = golden["pse"]
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-3
    og = oracle_lib.Geom.from12(golden["geom"], golden["np"])
    sym = oracle_lib.pse(golden["pos"], golden["angvel"], golden["size"], og, 0.01, DT, symmetric=True)
    assert np.linalg.norm(got - sym) / np.linalg.norm(sym) < 1e-6


def test_heat_pse_tolerance(vg, ref_ctx, golden, oracle_lib):
    """Heat PSE on the golden vortons with seeded densities (tests/golden/heat.npz,
    made by the reference's DiffuseAndDissipateHeatPSE).  At diffusivity 0.01
    the order-independent form is within 1e-4 relative of the reference's
    in-place order (the forms differ by ~(neighbours x 2 kappa dt) of the
    change) and equals the symmetric oracle to 1e-6 (summation order and the
    fast exponential).  At diffusivity 1.8, dt 1/3 (both clamps saturated) the
    reference's result depends on its serial order, and only the oracle
    comparison is meaningful."""
    import os
    h = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "heat.npz")))
    g = geom(vg, golden)
    ps, _ = vortons(golden)
    og = oracle_lib.Geom.from12(golden["geom"], golden["np"])
    d0 = h["heat_density"]
    for i in range(int(h["heat_cases"])):
        kappa, ambient, dt = (float(v) for v in h[f"heat{i}_params"])
        d = dev(d0)
        ref_ctx.check(vg.lib().vg_heat_pse_device(ref_ctx.h, ctypes.byref(g), vg._ptr(ps), vg._ptr(d), len(d0), kappa,
                                                  ambient, dt), "heat pse")
        sync()
        got = d.cpu().numpy()
        sym = oracle_lib.heat_pse(golden["pos"], d0, golden["size"], og, np.float32(kappa), np.float32(ambient),
                                  np.float32(dt), symmetric=True)
        assert np.linalg.norm(got - sym) / np.linalg.norm(sym) < 1e-6, i
        if i == 0:
            ref = h["heat0_out"]
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-4
            assert np.linalg.norm((got - d0) - (ref - d0)) / np.linalg.norm(ref - d0) < 0.02


def test_gather_advect_bit_exact(vg, ref_ctx, golden):
    g = geom(vg, golden)
    vel = dev(golden["curl"])
    p = dev(f4(golden["tracers"]))
    v = torch.zeros_like(p)
    ref_ctx.check(vg.lib().vg_gather_advect_device(ref_ctx.h, ctypes.byref(g), vg._ptr(vel), vg._ptr(p), vg._ptr(v),
                                                   len(p), float(DT)), "advect")
    sync()
    assert np.array_equal(bits(v.cpu().numpy()[:, :3]), bits(golden["tracer_vel"]))
    assert np.array_equal(bits(p.cpu().numpy()[:, :3]), bits(golden["tracer_pos1"]))


def test_full_step_reference_numerics(vg, golden):
    """PclOpVortonSim::Operate on the reference's 96-byte records, REFERENCE
    numerics + the reference cascade: the velocity grid and vorton velocities
    are bit-identical to the reference; angular velocity within the PSE bound."""
    sim = vg.VortonSim(0.01, numerics=vg.NUMERICS_REFERENCE, poisson_solver=vg.POISSON_REFERENCE_CASCADE,
                       boundary_copy_odd_x=1)
    recs = np.frombuffer(golden["step_in"].tobytes(), dtype=vg.PARTICLE_DTYPE).copy()
    sim.Update(recs, DT, 0, golden["step_extra_min"], golden["step_extra_max"])
    vel, g = sim.GetVelocityGrid()
    assert np.array_equal(bits(g.as12()), bits(golden["step_geom"]))
    assert list(g.points) == list(golden["step_np"])
    assert np.array_equal(bits(vel), bits(golden["step_velgrid"]))
    ap, _ = sim.GetVectorPotential()
    assert np.array_equal(bits(ap), bits(golden["step_vecpot"]))
    out = np.frombuffer(golden["step_out"].tobytes(), dtype=vg.PARTICLE_DTYPE)
    assert np.array_equal(bits(recs["velocity"]), bits(out["velocity"]))
    w, wr = recs["angular_velocity"], out["angular_velocity"]
    assert np.linalg.norm(w - wr) / np.linalg.norm(wr) < 1e-3
    # untouched fields survive the round trip
    assert np.array_equal(recs["position"], out["position"])
    assert np.array_equal(recs["size"], out["size"])


def _exact_discrete_solve(g, b, bc):
    """Independent FP64 solve of the same discrete Dirichlet problem (scipy CG)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    nx, ny, nz = g.points
    h = [float(g.cell[0]), float(g.cell[1]), float(g.cell[2])]

    def lap1(m, hh):
        return sp.diags([np.ones(m - 1), -2 * np.ones(m), np.ones(m - 1)], [-1, 0, 1]) / (hh * hh)
    L = sp.kronsum(sp.kronsum(lap1(nx - 2, h[0]), lap1(ny - 2, h[1])), lap1(nz - 2, h[2])).tocsr()
    a = bc.copy().reshape(nz, ny, nx, 3).astype(np.float64)
    B = b.reshape(nz, ny, nx, 3)
    for c in range(3):
        rhs = B[1:-1, 1:-1, 1:-1, c].astype(np.float64).copy()
        A = a[..., c]
        rhs[:, :, 0] -= A[1:-1, 1:-1, 0] / h[0] ** 2
        rhs[:, :, -1] -= A[1:-1, 1:-1, -1] / h[0] ** 2
        rhs[:, 0, :] -= A[1:-1, 0, 1:-1] / h[1] ** 2
        rhs[:, -1, :] -= A[1:-1, -1, 1:-1] / h[1] ** 2
        rhs[0, :, :] -= A[0, 1:-1, 1:-1] / h[2] ** 2
        rhs[-1, :, :] -= A[-1, 1:-1, 1:-1] / h[2] ** 2
        x, _ = spl.cg(L, rhs.ravel(), rtol=1e-11, maxiter=5000)
        a[1:-1, 1:-1, 1:-1, c] = x.reshape(nz - 2, ny - 2, nx - 2)
    return a.reshape(-1, 3)


@pytest.mark.parametrize("field", ["ring", "puff"])
def test_multigrid_reaches_tolerance(vg, oracle_lib, field):
    """FAST numerics, multigrid to 1e-6 relative residual:
      * the FP64 residual of the returned field is checked on the CPU;
      * the vector potential matches an independent FP64 sparse solve of the
        same discrete problem (so the solver is right);
      * for the smooth ring, the velocity is within the grid method's
        discretisation error (dx = 1/16) of the FP64 direct sum.  The
        white-noise puff's discretisation error is ~35% at this spacing (the
        exact discrete solution has the same error), so only the solver
        checks apply to it."""
    pytest.importorskip("scipy")
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(20000, seed=5) if field == "ring" else workloads.puff(20000, seed=5)
    g = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [65] * 3)
    sim = vg.VortonSim(0.01, fixed_grid=g, enable_stretch=0, enable_diffusion=0)
    recs = vg.make_particles(pos, w, s)
    sim.Update(recs, DT, 0)
    st = sim.stats()
    assert st.poisson_relres <= 1e-6 and st.poisson_cycles >= 1, (st.poisson_relres, st.poisson_cycles)
    a, gg = sim.GetVectorPotential()
    og = oracle_lib.Geom.from12(gg.as12(), gg.points)
    b = oracle_lib.splat(pos, w, s, og, -1.0)
    assert oracle_lib.relres(og, a, b) < 1e-4  # FP32 copy of the FP64 iterate
    exact = _exact_discrete_solve(og, b, a)  # boundary values: the GPU's own (treecode) boundary
    assert np.linalg.norm(a - exact) / np.linalg.norm(exact) < 1e-5
    if field == "ring":
        vel, _ = sim.GetVelocityGrid()
        sl = (slice(8, -8, 4),) * 3
        pts = workloads.grid_points(og.mn, og.cell, og.points).reshape(65, 65, 65, 3)[sl].reshape(-1, 3)
        d = oracle_lib.direct(0, pos, w, s, pts, f64=True)
        v = vel.reshape(65, 65, 65, 3)[sl].reshape(-1, 3)
        assert np.linalg.norm(v - d) / np.linalg.norm(d) < 0.08  # measured 4.2%


def test_multigrid_anisotropic_box(vg, oracle_lib):
    """The multigrid stage on a non-cubic box with unequal spacings (33 x 65 x
    17 points; its coarsest level, 9 x 17 x 5, is solved exactly by sine
    transforms along each axis) reaches 1e-6 and matches an independent FP64
    sparse solve of the same discrete problem to 1e-5 relative."""
    pytest.importorskip("scipy")
    g = vg.GridGeom.make([-1.0, -1.5, -0.375], [2.0, 3.0, 0.75], [33, 65, 17])
    n = g.capacity
    rng = np.random.default_rng(7)
    b = rng.normal(size=(n, 3)).astype(np.float32)
    a0 = np.zeros((17, 65, 33, 3), np.float32)
    bnd = rng.normal(size=a0.shape).astype(np.float32) * 1e-3
    for sl in ((0,), (-1,)):
        a0[sl] = bnd[sl]
        a0[:, sl[0]] = bnd[:, sl[0]]
        a0[:, :, sl[0]] = bnd[:, :, sl[0]]
    a0 = a0.reshape(-1, 3)
    ctx = vg.Context(numerics=vg.NUMERICS_FAST)
    soln, rhs = dev(a0), dev(b)
    cyc, r0, r1 = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
    ctx.check(vg.lib().vg_multigrid_device(ctx.h, ctypes.byref(g), vg._ptr(soln), vg._ptr(rhs), 1e-6, 50,
                                           ctypes.byref(cyc), ctypes.byref(r0), ctypes.byref(r1)), "multigrid")
    sync()
    a = soln.cpu().numpy()
    assert r1.value <= 1e-6 and 1 <= cyc.value <= 12, (r1.value, cyc.value)
    og = oracle_lib.Geom.from12(g.as12(), g.points)
    assert oracle_lib.relres(og, a, b) < 1e-4  # the FP32 copy of the refined iterate
    exact = _exact_discrete_solve(og, b, a)
    assert np.linalg.norm(a - exact) / np.linalg.norm(exact) < 1e-5


def test_multigrid_coarsest_fp64_vs_fp32(vg, oracle_lib):
    """The coarsest solve (33^3 under a 65^3 grid: sine transforms over the
    whole GPU) in FP64 and in FP32: both solves reach 1e-6 in the same number
    of cycles, and their vector potentials agree to 1e-6 relative (the
    coarsest level only shapes the correction; the FP64-class residual
    decides the answer), against an independent FP64 sparse solve to 1e-5."""
    pytest.importorskip("scipy")
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.puff(20000, seed=8)
    g = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [65] * 3)
    og = oracle_lib.Geom.from12(g.as12(), g.points)
    b = oracle_lib.splat(pos, w, s, og, -1.0)
    out = []
    for fp64 in (False, True):
        ctx = vg.Context(numerics=vg.NUMERICS_FAST)
        ctx.set_coarsest_fp64(fp64)
        soln, rhs = dev(np.zeros_like(b)), dev(b)
        cyc, r0, r1 = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        ctx.check(vg.lib().vg_multigrid_device(ctx.h, ctypes.byref(g), vg._ptr(soln), vg._ptr(rhs), 1e-6, 50,
                                               ctypes.byref(cyc), ctypes.byref(r0), ctypes.byref(r1)), "multigrid")
        sync()
        assert r1.value <= 1e-6, (fp64, r1.value)
        out.append((soln.cpu().numpy().astype(np.float64), cyc.value, r1.value))
    (a32, c32, _), (a64, c64, _) = out
    assert c32 == c64
    assert np.linalg.norm(a64 - a32) / np.linalg.norm(a64) < 1e-6
    exact = _exact_discrete_solve(og, b, np.zeros_like(b))
    assert np.linalg.norm(a64 - exact) / np.linalg.norm(exact) < 1e-5


def test_pinned_records_match_pageable(vg):
    """Particle records in pinned host memory (whole-record copies run
    asynchronously) give field-for-field the same step and advection as
    pageable records."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(2000, seed=4)
    tr = (pos[::2] * np.float32(0.9)).astype(np.float32)  # tracers inside the vortons' grid
    out = []
    for pinned in (False, True):
        sim = vg.VortonSim(0.01)
        recs0, trs0 = vg.make_particles(pos, w, s), vg.make_particles(tr)
        if pinned:
            rt = torch.empty(recs0.nbytes, dtype=torch.uint8, pin_memory=True)
            tt = torch.empty(trs0.nbytes, dtype=torch.uint8, pin_memory=True)
            recs, trs = rt.numpy().view(vg.PARTICLE_DTYPE), tt.numpy().view(vg.PARTICLE_DTYPE)
            recs[...] = recs0
            trs[...] = trs0
        else:
            recs, trs = recs0.copy(), trs0.copy()
        for k in range(2):
            sim.Update(recs, DT, k)
            sim.Advect(trs, DT)
        out.append((recs.copy(), trs.copy()))
    # every field bit for bit (the records' padding bytes are not compared)
    for a, b in zip(out[0], out[1]):
        for f in vg.PARTICLE_DTYPE.names:
            assert np.array_equal(np.ascontiguousarray(a[f]).view(np.uint8), np.ascontiguousarray(b[f]).view(np.uint8)), f


def test_step_evolve_matches_step_then_evolve(vg):
    """vg_step_evolve (the step and PclOpEvolve on the same vorton records,
    fused) gives every field bit for bit what vg_step followed by the FP32
    Euler step on the host records gives (pclOpEvolve.cpp:36-58), over three
    frames, for 96-byte records (copied whole) and for wider ones (copied as
    their first 48 bytes)."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(3000, seed=9)
    dt = np.float32(DT)
    wide = np.dtype({"names": list(vg.PARTICLE_DTYPE.names) + ["extra"],
                     "formats": [vg.PARTICLE_DTYPE.fields[f][0] for f in vg.PARTICLE_DTYPE.names] + [(np.float32, 40)],
                     "offsets": [vg.PARTICLE_DTYPE.fields[f][1] for f in vg.PARTICLE_DTYPE.names] + [96],
                     "itemsize": 256})
    for dtype in (vg.PARTICLE_DTYPE, wide):
        recs0 = np.zeros(len(pos), dtype)
        base = vg.make_particles(pos, w, s)
        for f in vg.PARTICLE_DTYPE.names:
            recs0[f] = base[f]
        a, b = recs0.copy(), recs0.copy()
        sa, sb = vg.VortonSim(0.01), vg.VortonSim(0.01)
        for k in range(3):
            sa.Update(a, DT, k)
            for j in range(3):  # position += velocity dt, FP32
                a["position"][:, j] = (a["position"][:, j] + a["velocity"][:, j] * dt).astype(np.float32)
            sb.UpdateAndEvolve(b, DT, k)
        for f in vg.PARTICLE_DTYPE.names:
            assert np.array_equal(np.ascontiguousarray(a[f]).view(np.uint8),
                                  np.ascontiguousarray(b[f]).view(np.uint8)), (dtype.itemsize, f)
        assert np.abs(b["position"] - recs0["position"]).max() > 0  # the vortons moved


def test_step_advect_matches_the_separate_calls(vg):
    """vg_step_advect (both groups of a frame in one call, the tracer upload on
    a second stream during the step) gives every field of the vorton and
    tracer records bit for bit what vg_step_evolve (or vg_step) then vg_advect
    give, over three frames, with whole and wide tracer records."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(3000, seed=11)
    tr = (pos[::3] * np.float32(0.8)).astype(np.float32)
    wide = np.dtype({"names": ["position", "velocity", "extra"], "formats": [(np.float32, 3), (np.float32, 3),
                                                                           (np.float32, 30)],
                     "offsets": [0, 12, 24], "itemsize": 144})
    for evolve in (True, False):
        for tdtype in (vg.PARTICLE_DTYPE, wide):
            t0 = np.zeros(len(tr), tdtype)
            t0["position"] = tr
            v0 = vg.make_particles(pos, w, s)
            va, ta, vb, tb = v0.copy(), t0.copy(), v0.copy(), t0.copy()
            sa, sb = vg.VortonSim(0.01), vg.VortonSim(0.01)
            for k in range(3):
                (sa.UpdateAndEvolve if evolve else sa.Update)(va, DT, k)
                sa.Advect(ta, DT)
                sb.UpdateAndAdvect(vb, tb, DT, k, evolve=evolve)
            for a, b, names in ((va, vb, vg.PARTICLE_DTYPE.names), (ta, tb, tdtype.names)):
                for f in names:
                    assert np.array_equal(np.ascontiguousarray(a[f]).view(np.uint8),
                                          np.ascontiguousarray(b[f]).view(np.uint8)), (evolve, tdtype.itemsize, f)
            assert np.abs(tb["position"] - t0["position"]).max() > 0


def test_step_evolve_device_matches_step_then_evolve(vg):
    """vg_step_evolve_device gives positions, velocities and angular
    velocities bit for bit equal to vg_step_device then vg_evolve_device: the
    direct technique on a fixed grid (the Euler step folded into the
    reduction), the direct technique with stretch and diffusion (a separate
    Euler kernel after them), the treecode and the Poisson technique (the
    Euler step in the vortons' gather)."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(4096, seed=1)
    grid = vg.GridGeom.make([-1.5] * 3, [3.0] * 3, [33] * 3)
    cases = [dict(velocity_technique=vg.VELOCITY_DIRECT, fixed_grid=grid, enable_stretch=0, enable_diffusion=0),
             dict(velocity_technique=vg.VELOCITY_DIRECT, fixed_grid=grid),
             dict(velocity_technique=vg.VELOCITY_TREE, enable_stretch=0, enable_diffusion=0),
             dict(velocity_technique=vg.VELOCITY_POISSON)]

    def f4(a, wv=None):
        o = np.zeros((len(a), 4), np.float32)
        o[:, :3] = a
        if wv is not None:
            o[:, 3] = wv
        return torch.from_numpy(o).cuda()
    for kw in cases:
        out = []
        for fused in (False, True):
            sim = vg.VortonSim(cfg=vg.default_config(device=0, **kw))
            ps, ww, vel = f4(pos, s), f4(w), torch.zeros((len(pos), 4), device="cuda")
            for k in range(2):
                if fused:
                    sim.UpdateAndEvolveDevice(ps, ww, vel, DT, k)
                else:
                    sim.UpdateDevice(ps, ww, vel, DT, k)
                    sim.EvolveDevice(ps, vel, DT)
            sim.synchronize()
            out.append([t.cpu().numpy() for t in (ps, ww, vel)])
        for a, b in zip(*out):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), kw
        assert np.abs(out[1][0][:, :3] - pos).max() > 0


def test_host_record_graph_replay_matches_direct_runs(vg):
    """On a fixed grid with pinned records, repeated host-record calls run
    from a captured CUDA graph (second call captures, later ones replay):
    six frames of vg_step_advect and of vg_step_evolve + vg_advect give every
    record field bit for bit what the same calls give on pageable records
    (always run directly); a change of the vortons' size between frames is
    picked up (a new capture); direct and treecode techniques."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(2048, seed=5)
    # 600,000 tracers: over two per cell of the 65^3 grid, so vg_advect gathers from the grid arranged by cell
    tr = np.random.default_rng(3).uniform(-1.2, 1.2, (600000, 3)).astype(np.float32)
    grid = vg.GridGeom.make([-1.5] * 3, [3.0] * 3, [65] * 3)

    def pinned_copy(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        b = t.numpy().view(a.dtype)
        b[...] = a
        return b, t
    for tech in (vg.VELOCITY_DIRECT, vg.VELOCITY_TREE):
        for one_call in (True, False):
            results = []
            for pinned in (False, True):
                sim = vg.VortonSim(cfg=vg.default_config(velocity_technique=tech, fixed_grid=grid, enable_stretch=0,
                                                         enable_diffusion=0, device=0))
                v0, t0 = vg.make_particles(pos, w, s), vg.make_particles(tr)
                keep = []
                if pinned:
                    (v, tv), (t, tt) = pinned_copy(v0), pinned_copy(t0)
                    keep = [tv, tt]
                else:
                    v, t = v0.copy(), t0.copy()
                for k in range(6):
                    if k == 4:
                        v["size"] *= np.float32(1.1)  # the vortons grow: the graph's key changes
                    if one_call:
                        sim.UpdateAndAdvect(v, t, DT, k, evolve=True)
                    else:
                        sim.UpdateAndEvolve(v, DT, k)
                        sim.Advect(t, DT)
                results.append((v.copy(), t.copy()))
                del keep
            (va, ta), (vb, tb) = results
            for a, b in ((va, vb), (ta, tb)):
                for f in vg.PARTICLE_DTYPE.names:
                    assert np.array_equal(np.ascontiguousarray(a[f]).view(np.uint8),
                                          np.ascontiguousarray(b[f]).view(np.uint8)), (tech, one_call, f)


def test_tracer_gather_by_cell_matches_grid_gather(vg):
    """A tracer group of at least two per cell on a grid of at least 2^17
    cells (here 600,000 tracers on 65^3 points) is gathered from the step's
    velocity grid arranged by cell: positions and velocities bit for bit those
    of the same tracers gathered from the grid itself
    (vg_gather_advect_device), over three steps with the grid changing in
    between (the by-cell copy is remade for every step)."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(2048, seed=6)
    grid = vg.GridGeom.make([-1.5] * 3, [3.0] * 3, [65] * 3)
    sim = vg.VortonSim(cfg=vg.default_config(velocity_technique=vg.VELOCITY_DIRECT, fixed_grid=grid, enable_stretch=0,
                                             enable_diffusion=0, device=0))

    def f4(a, wv=None):
        o = np.zeros((len(a), 4), np.float32)
        o[:, :3] = a
        if wv is not None:
            o[:, 3] = wv
        return torch.from_numpy(o).cuda()
    ps, ww, vel = f4(pos, s), f4(w), torch.zeros((len(pos), 4), device="cuda")
    trp = f4(np.random.default_rng(8).uniform(-1.2, 1.2, (600000, 3)).astype(np.float32))
    trv = torch.zeros_like(trp)
    for k in range(3):
        sim.UpdateDevice(ps, ww, vel, DT, k)
        ref_p, ref_v = trp.clone(), torch.zeros_like(trv)
        vg3 = ctypes.c_void_p()
        geom = vg.GridGeom()
        sim.check(vg.lib().vg_get_velocity_grid_device(sim.h, ctypes.byref(vg3), ctypes.byref(geom)), "grid")
        sim.check(vg.lib().vg_gather_advect_device(sim.h, ctypes.byref(geom), vg3, vg._ptr(ref_p), vg._ptr(ref_v),
                                                   ref_p.shape[0], DT), "gather")
        sim.AdvectDevice(trp, trv, DT)
        sim.synchronize()
        assert torch.equal(trp, ref_p) and torch.equal(trv[:, :3], ref_v[:, :3]), k
        ps[:, 0] += 0.01  # the vortons move: the next step's grid differs


def test_advect_records_match_the_float4_path(vg):
    """vg_advect on host records (gathering in place on the staged records)
    moves and assigns every tracer bit for bit as vg_advect_device does on
    float4 arrays, for whole (96-byte) and wide records."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(2000, seed=12)
    tr = (pos[::2] * np.float32(0.85)).astype(np.float32)
    wide = np.dtype({"names": ["position", "velocity", "extra"], "formats": [(np.float32, 3), (np.float32, 3),
                                                                           (np.float32, 30)],
                     "offsets": [0, 12, 24], "itemsize": 144})
    for tdtype in (vg.PARTICLE_DTYPE, wide):
        sim = vg.VortonSim(0.01)
        v = vg.make_particles(pos, w, s)
        sim.Update(v, DT, 0)
        recs = np.zeros(len(tr), tdtype)
        recs["position"] = tr
        p4 = np.zeros((len(tr), 4), np.float32)
        p4[:, :3] = tr
        dp, dv = torch.from_numpy(p4).cuda(), torch.zeros((len(tr), 4), device="cuda")
        sim.Advect(recs, DT)
        sim.AdvectDevice(dp, dv, DT)
        sim.synchronize()
        assert np.array_equal(recs["position"].view(np.uint32), dp.cpu().numpy()[:, :3].copy().view(np.uint32))
        assert np.array_equal(recs["velocity"].view(np.uint32), dv.cpu().numpy()[:, :3].copy().view(np.uint32))


def test_status_paths(vg):
    sim = vg.VortonSim(0.01)
    empty = np.zeros(0, vg.PARTICLE_DTYPE)
    with pytest.raises(vg.VgError) as e:
        sim.Update(empty, DT, 0)
    assert e.value.status == vg.EMPTY
    with pytest.raises(vg.VgError) as e:
        sim.GetVelocityGrid()
    assert e.value.status == vg.EMPTY
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(500, seed=3)
    sim.Update(vg.make_particles(pos, w, s), DT, 0)
    far = vg.make_particles(np.full((4, 3), 50.0, np.float32))
    with pytest.raises(vg.VgError) as e:
        sim.Advect(far, DT)
    assert e.value.status == vg.OUT_OF_GRID
    # one to two cells below the minimum corner on one axis (truncation gives
    # cell -1 there) is outside too
    _, g = sim.GetVelocityGrid()
    mn = np.array(g.min_corner[:3], np.float32)
    cell = np.array(g.cell_spacing[:3], np.float32)
    below = np.stack([mn + np.float32(3.0) * cell] * 3)
    for a in range(3):
        below[a, a] = mn[a] - np.float32(1.5) * cell[a]
    with pytest.raises(vg.VgError) as e:
        sim.Advect(vg.make_particles(below.astype(np.float32)), DT)
    assert e.value.status == vg.OUT_OF_GRID
    # the context stays usable after a reported error
    inside = vg.make_particles(pos[:10])
    sim.Advect(inside, DT)
    nan = vg.make_particles(np.array([[np.nan, 0, 0]] * 3, np.float32), w[:3], s[:3])
    with pytest.raises(vg.VgError) as e:
        sim.Update(nan, DT, 0)
    assert e.value.status == vg.NONFINITE
