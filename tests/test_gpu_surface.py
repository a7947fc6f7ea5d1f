"""GPU density grid, gradient, baroclinic generation and signed distance grid,
through the C ABI, against the reference's own code (tests/golden/surface.npz,
made by tests/golden/make_golden.py surface) and the C oracle:
  * density grid (PopulateDensityAndMassFractionGrids), gradient
    (ComputeGradient) and the density-grid baroclinic update of angular
    velocity (GenerateBaroclinicVorticity): bit-exact;
  * signed distance grid (PopulateSignedDistanceGridFromDensityGrid): bit-exact
    with the reference's FP32 statistics; with the FP64 parallel statistics
    within 1e-5 of the field's largest distance;
  * the same at the multigrid workload's size (262,144 puff vortons, 129^3)
    against the oracle, bit for bit;
  * marching cubes (ExtractIsoLevel / PolygoniseCellWithNormal): vertex
    positions and face normals bit-exact against the oracle on a sphere's
    signed distance, the puff's 129^3 density grid and the golden signed
    distance grids; the sphere's mesh closed, outward, with its area and
    volume within 0.5%; a too-small buffer refused with the count.
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


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
def ctx(vg):
    return vg.Context(numerics=vg.NUMERICS_REFERENCE)


@pytest.fixture(scope="module")
def surf():
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "surface.npz")))


# Device inputs are held in named tensors until the stream is synchronised: a
# temporary's memory goes back to torch's caching allocator when the Python
# object dies, and the next temporary can be given the same block.

def density_grid(vg, ctx, g, pos, size, dens, ambient):
    out = torch.zeros(g.capacity, dtype=torch.float32, device="cuda")
    ps, d = dev(f4(pos, size)), dev(dens.astype(np.float32))
    ctx.check(vg.lib().vg_density_grid_device(ctx.h, ctypes.byref(g), vg._ptr(ps), vg._ptr(d), len(pos), ambient,
                                              vg._ptr(out)), "density grid")
    ctx.synchronize()
    return out.cpu().numpy()


def signed_distance(vg, ctx, g, dgrid, ambient, reference_stats):
    out = torch.zeros(g.capacity, dtype=torch.float32, device="cuda")
    d = dev(dgrid)
    ctx.check(vg.lib().vg_signed_distance_device(ctx.h, ctypes.byref(g), vg._ptr(d), ambient, reference_stats,
                                                 vg._ptr(out)), "signed distance")
    ctx.synchronize()
    return out.cpu().numpy()


def test_density_gradient_baroclinic_bit_exact(vg, ctx, surf):
    dt, ambient = (float(v) for v in surf["surface_params"])
    for i in range(int(surf["surface_cases"])):
        g = vg.GridGeom.from12(surf[f"s{i}_geom"], surf[f"s{i}_np"])
        pos, size, dens = surf[f"s{i}_pos"], surf[f"s{i}_size"], surf[f"s{i}_density"]
        dg = density_grid(vg, ctx, g, pos, size, dens, ambient)
        assert np.array_equal(bits(dg), bits(surf[f"s{i}_density_grid"])), i
        grad = torch.zeros((g.capacity, 3), dtype=torch.float32, device="cuda")
        dgd = dev(dg)
        ctx.check(vg.lib().vg_gradient_device(ctx.h, ctypes.byref(g), vg._ptr(dgd), vg._ptr(grad)), "gradient")
        ctx.synchronize()
        assert np.array_equal(bits(grad.cpu().numpy()), bits(surf[f"s{i}_gradient"])), i
        w = dev(f4(surf[f"s{i}_angvel"]))
        ps, dd = dev(f4(pos, size)), dev(dens)
        grav = np.ascontiguousarray(surf[f"s{i}_grav"], np.float32)
        applied = ctypes.c_int()
        ctx.check(vg.lib().vg_baroclinic_device(ctx.h, ctypes.byref(g), vg._ptr(ps), vg._ptr(dd), vg._ptr(w),
                                                len(pos), vg._ptr(grav), ambient, dt, ctypes.byref(applied)),
                  "baroclinic")
        ctx.synchronize()
        assert applied.value == int(surf[f"s{i}_applied"])
        assert np.array_equal(bits(w.cpu().numpy()[:, :3]), bits(surf[f"s{i}_baroclinic"])), i
    # no gravity along the grid: nothing changes (the reference's early return)
    g = vg.GridGeom.from12(surf["s0_geom"], surf["s0_np"])
    w = dev(f4(surf["s0_angvel"]))
    ps, dd = dev(f4(surf["s0_pos"], surf["s0_size"])), dev(surf["s0_density"])
    applied = ctypes.c_int(7)
    ctx.check(vg.lib().vg_baroclinic_device(ctx.h, ctypes.byref(g), vg._ptr(ps), vg._ptr(dd), vg._ptr(w),
                                            len(surf["s0_pos"]), vg._ptr(np.zeros(3, np.float32)), ambient, dt,
                                            ctypes.byref(applied)), "baroclinic")
    ctx.synchronize()
    assert applied.value == 0 and np.array_equal(w.cpu().numpy()[:, :3], surf["s0_angvel"])


def test_signed_distance(vg, ctx, surf, oracle_lib):
    ambient = float(surf["surface_params"][1])
    for i in range(int(surf["surface_cases"])):
        g = vg.GridGeom.from12(surf[f"s{i}_geom"], surf[f"s{i}_np"])
        dg = surf[f"s{i}_density_grid"]
        exact = signed_distance(vg, ctx, g, dg, ambient, 1)
        assert np.array_equal(bits(exact), bits(surf[f"s{i}_sdf"])), i
        fast = signed_distance(vg, ctx, g, dg, ambient, 0)
        ref = surf[f"s{i}_sdf"]
        assert np.array_equal(np.isnan(fast), np.isnan(ref))
        assert np.nanmax(np.abs(fast - ref)) <= 1e-5 * float(np.nanmax(np.abs(ref))), i


def test_puff_density_and_sdf_at_workload_size(vg, ctx, oracle_lib):
    """262,144 puff vortons (density 2 in ambient 1) on the 129^3 grid of
    [-2, 2]^3: density grid and signed distance bit-exact against the oracle."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.puff(262144, seed=3)
    dens = np.full(len(pos), 2.0, np.float32)
    g = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [129] * 3)
    og = oracle_lib.Geom.from12(g.as12(), g.points)
    dg = density_grid(vg, ctx, g, pos, s, dens, 1.0)
    odg = oracle_lib.density_grid(pos, s, dens, og, 1.0)
    assert np.array_equal(bits(dg), bits(odg))
    sdf = signed_distance(vg, ctx, g, dg, 1.0, 1)
    osdf = oracle_lib.signed_distance(og, odg, 1.0, 0)
    assert np.array_equal(bits(sdf), bits(osdf))
    inside = np.nanmin(sdf)
    assert inside < 0 and np.nanmax(sdf) > 0


def marching_cubes(vg, ctx, g, values, iso, cap=None):
    v = dev(np.ascontiguousarray(values, np.float32))
    n = ctypes.c_size_t()
    st = vg.lib().vg_marching_cubes_device(ctx.h, ctypes.byref(g), vg._ptr(v), iso, None, None, 0, ctypes.byref(n))
    assert st in (vg.OK, vg.TOO_LARGE)
    cap = n.value if cap is None else cap
    verts = torch.zeros((max(cap, 1), 3, 3), dtype=torch.float32, device="cuda")
    norms = torch.zeros_like(verts)
    st = vg.lib().vg_marching_cubes_device(ctx.h, ctypes.byref(g), vg._ptr(v), iso, vg._ptr(verts), vg._ptr(norms),
                                           cap, ctypes.byref(n))
    return st, n.value, verts.cpu().numpy()[:n.value], norms.cpu().numpy()[:n.value]


def test_marching_cubes_sphere(vg, ctx, oracle_lib):
    """A sphere's signed distance on 65^3: the GPU mesh equals the oracle's bit
    for bit (positions and normals), is closed (every edge in two
    triangles), has outward normals, and its area and volume are within
    0.5% of the sphere's."""
    from collections import Counter
    from vortegrid_gb300 import workloads
    n = 65
    g = vg.GridGeom.make([-1.0] * 3, [2.0] * 3, [n] * 3)
    pts = workloads.grid_points(list(g.min_corner), list(g.cell_spacing), g.points)
    r = 0.6
    sdf = (np.linalg.norm(pts.astype(np.float64), axis=1) - r).astype(np.float32)
    st, nt, V, N = marching_cubes(vg, ctx, g, sdf, 0.0)
    assert st == vg.OK and nt > 1000
    og = oracle_lib.Geom.from12(g.as12(), g.points)
    OV, ON = oracle_lib.marching_cubes(og, sdf, 0.0)
    assert np.array_equal(bits(V), bits(OV)) and np.array_equal(bits(N), bits(ON))
    area = 0.5 * np.linalg.norm(np.cross(V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]).astype(np.float64), axis=1).sum()
    vol = np.einsum("ij,ij->i", V[:, 0].astype(np.float64), np.cross(V[:, 1], V[:, 2]).astype(np.float64)).sum() / 6
    assert abs(area / (4 * np.pi * r * r) - 1) < 5e-3 and abs(vol / (4 / 3 * np.pi * r ** 3) - 1) < 5e-3
    assert np.all(np.einsum("ij,ij->i", N[:, 0], V.mean(1)) > 0)
    edges = Counter()
    for t in np.round(V.astype(np.float64), 5):
        k = [tuple(p) for p in t]
        for i in range(3):
            edges[tuple(sorted((k[i], k[(i + 1) % 3])))] += 1
    assert set(edges.values()) == {2}
    # too small a buffer: the count comes back, nothing is written
    st, nt2, _, _ = marching_cubes(vg, ctx, g, sdf, 0.0, cap=nt - 1)
    assert st == vg.TOO_LARGE and nt2 == nt


def test_marching_cubes_of_puff_density(vg, ctx, oracle_lib):
    """The 129^3 density grid of 262,144 puff vortons (density 2 in ambient 1)
    at iso level 1.5, and the golden cases' signed distance grids at 0: the
    GPU mesh equals the oracle's bit for bit."""
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.puff(262144, seed=3)
    g = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [129] * 3)
    og = oracle_lib.Geom.from12(g.as12(), g.points)
    dg = oracle_lib.density_grid(pos, s, np.full(len(pos), 2.0, np.float32), og, 1.0)
    st, nt, V, N = marching_cubes(vg, ctx, g, dg, 1.5)
    OV, ON = oracle_lib.marching_cubes(og, dg, 1.5)
    assert st == vg.OK and nt == len(OV) > 0
    assert np.array_equal(bits(V), bits(OV)) and np.array_equal(bits(N), bits(ON))
    surf = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "surface.npz")))
    for i in range(int(surf["surface_cases"])):
        g = vg.GridGeom.from12(surf[f"s{i}_geom"], surf[f"s{i}_np"])
        og = oracle_lib.Geom.from12(surf[f"s{i}_geom"], surf[f"s{i}_np"])
        st, nt, V, N = marching_cubes(vg, ctx, g, surf[f"s{i}_sdf"], 0.0)
        OV, ON = oracle_lib.marching_cubes(og, surf[f"s{i}_sdf"], 0.0)
        assert st == vg.OK and nt == len(OV)
        assert np.array_equal(bits(V), bits(OV)) and np.array_equal(bits(N), bits(ON))
