"""Pin the C oracle against golden vectors from the reference's own code.

Every comparison here is bit-exact (integer and float bit patterns), except
the order-independent PSE form, which is checked against the reference's
in-place order at a stated tolerance.
"""
import os

import numpy as np
import pytest


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def geom_of(O, golden, prefix=""):
    return O.Geom.from12(golden[prefix + "geom"], golden[prefix + "np"])


def test_define_shape(oracle_lib, golden):
    O = oracle_lib
    for k in range(len(golden["shape_n"])):
        g = O.define_shape(int(golden["shape_n"][k]), golden["shape_min"][k], golden["shape_max"][k])
        assert np.array_equal(bits(g.as12()), bits(golden["shape_geom"][k])), k
        assert list(g.points) == list(golden["shape_np"][k]), k


def test_nested_grid_shape(oracle_lib, golden):
    O = oracle_lib
    for k in range(len(golden["shape_n"])):
        g = O.Geom.from12(golden["shape_geom"][k], golden["shape_np"][k])
        layers, dec = O.nested_shape(g)
        d = int(golden["nested_depth"][k])
        assert len(layers) == d
        assert np.array_equal(np.array([l.points for l in layers]), golden["nested_np"][k][: 3 * d].reshape(d, 3))
        if d > 1:
            assert np.array_equal(dec[1:], golden["nested_decim"][k][3: 3 * d].reshape(d - 1, 3))
    # the reference's own NestedGrid unit test: 1024 elements in a 2x3x5 box -> depth 5
    # (Core/SpatialPartition/nestedGridDiagnostics.cpp:34)
    assert int(golden["nested_depth"][2]) == 5
    for k in range(len(golden["shape_n"])):
        d = int(golden["nested_depth"][k])
        dec = golden["nested_decim"][k][3: 3 * d].reshape(-1, 3)
        assert np.all((dec == 1) | (dec == 2))  # nestedGridDiagnostics.cpp:35-98


def test_binning_bit_exact(oracle_lib, golden):
    O = oracle_lib
    g = geom_of(O, golden)
    idx, off = O.indices_of_position(g, golden["bin_pos"])
    assert np.array_equal(idx, golden["bin_idx"])
    assert np.array_equal(off, golden["bin_off"])


def test_influence_tree_bit_exact(oracle_lib, golden):
    O = oracle_lib
    g = geom_of(O, golden)
    t = O.influence_tree(golden["pos"], golden["angvel"], golden["size"], g)
    assert np.array_equal(bits(t), bits(golden["tree"]))
    # circulation is conserved through every layer (vortonSim.cpp:1257-1273, 1514-1568)
    layers, _ = O.nested_shape(g)
    total = golden["angvel"].astype(np.float64).sum(0)
    k = 0
    for L in layers:
        c = L.capacity
        s = t[k:k + c, 3:6].astype(np.float64).sum(0)
        assert np.allclose(s, total, rtol=1e-4, atol=1e-3)
        k += c


@pytest.mark.parametrize("kind,name", [(0, "vel"), (1, "vecpot")])
def test_direct_and_tree_bit_exact(oracle_lib, golden, kind, name):
    O = oracle_lib
    g = geom_of(O, golden)
    a = (golden["pos"], golden["angvel"], golden["size"])
    assert np.array_equal(bits(O.direct(kind, *a, golden["q"])), bits(golden[f"direct_{name}"]))
    assert np.array_equal(bits(O.tree(kind, *a, g, golden["q"])), bits(golden[f"tree_{name}"]))
    sr, sc = golden["spread"]
    assert np.array_equal(bits(O.tree(kind, *a, g, golden["q"], sr, sc)), bits(golden[f"tree_{name}_spread"]))


def test_direct_f64_oracle_close_to_reference(oracle_lib, golden):
    """The reference's magic-constant rsqrt costs ~1e-3 relative error."""
    O = oracle_lib
    a = (golden["pos"], golden["angvel"], golden["size"])
    d64 = O.direct(0, *a, golden["q"], f64=True)
    ref = golden["direct_vel"].astype(np.float64)
    rel = np.linalg.norm(ref - d64) / np.linalg.norm(d64)
    assert rel < 3e-3


def test_grid_stages_bit_exact(oracle_lib, golden):
    O = oracle_lib
    g = geom_of(O, golden)
    a = (golden["pos"], golden["angvel"], golden["size"])
    assert np.array_equal(bits(O.splat(*a, g, -1.0)), bits(golden["negvort"]))
    bvp = O.boundary_vecpot(*a, g)
    assert np.array_equal(bits(bvp), bits(golden["boundary_vecpot"]))
    assert np.array_equal(bits(O.sor(g, bvp, golden["negvort"], 5)), bits(golden["sor5"]))
    casc = O.cascade(g, bvp, golden["negvort"], 16)
    assert np.array_equal(bits(casc), bits(golden["cascade"]))
    jac = O.jacobian(g, casc)
    assert np.array_equal(bits(jac), bits(golden["jacobian"]))
    assert np.array_equal(bits(O.curl_from_jacobian(jac)), bits(golden["curl"]))


def test_restrict_prolong_bit_exact(oracle_lib, golden):
    O = oracle_lib
    g = geom_of(O, golden)
    layers, _ = O.nested_shape(g)
    fine, coarse = layers[0], layers[1]
    a = golden["cascade"]
    for inject, name in ((True, "inject"), (False, "average")):
        c = O.downsample(fine, a, coarse, inject)
        assert np.array_equal(bits(c), bits(golden[f"down_{name}"]))
        for interior, rname in ((True, "interior"), (False, "entire")):
            f = O.upsample(coarse, c, fine, a, interior)
            assert np.array_equal(bits(f), bits(golden[f"up_{name}_{rname}"]))


def test_particle_stages_bit_exact(oracle_lib, golden):
    O = oracle_lib
    g = geom_of(O, golden)
    dt = np.float32(1.0 / 30.0)
    jv = O.jacobian(g, golden["curl"])
    assert np.array_equal(bits(O.stretch(golden["pos"], golden["angvel"], g, jv, dt)), bits(golden["stretched"]))
    w = O.pse(golden["pos"], golden["angvel"], golden["size"], g, 0.01, dt)
    assert np.array_equal(bits(w), bits(golden["pse"]))
    v = O.gather(g, golden["curl"], golden["tracers"])
    assert np.array_equal(bits(v), bits(golden["tracer_vel"]))
    assert np.array_equal(bits(O.evolve(golden["tracers"], v, dt)), bits(golden["tracer_pos1"]))
    mn, mx = np.zeros(3, np.float32), np.zeros(3, np.float32)
    b = golden["pos"]
    assert np.array_equal(b.min(0), golden["bbox_min"]) and np.array_equal(b.max(0), golden["bbox_max"])


def test_pse_symmetric_tolerance(oracle_lib, golden):
    """Order-independent PSE vs the reference's in-place order.  Each pair
    exchanges a fraction 2 * nu * dt * law <= 6.7e-4 of its difference; the
    in-place order lets a vorton's earlier exchanges feed its later ones, so
    the two forms differ by ~(neighbours * 6.7e-4) of the PSE increment.
    Stated tolerance: 1e-3 relative L2 on the vorticity after the step."""
    O = oracle_lib
    g = geom_of(O, golden)
    dt = np.float32(1.0 / 30.0)
    w = O.pse(golden["pos"], golden["angvel"], golden["size"], g, 0.01, dt, symmetric=True)
    ref = golden["pse"]
    assert np.linalg.norm(w - ref) / np.linalg.norm(ref) < 1e-3
    # and it captures the bulk of the reference's change
    d_ref = ref - golden["angvel"]
    assert np.linalg.norm((w - golden["angvel"]) - d_ref) / np.linalg.norm(d_ref) < 0.05


def test_full_step_bit_exact(oracle_lib, golden):
    """PclOpVortonSim::Operate on 96-byte Particle records vs the oracle's step."""
    O = oracle_lib
    rec = golden["step_in"]
    pos, w, s = rec[:, 0:3].copy(), rec[:, 9:12].copy(), rec[:, 13].copy()
    g = O.step_geometry(pos, float(s[0]) * 0.5, golden["step_extra_min"], golden["step_extra_max"])
    assert np.array_equal(bits(g.as12()), bits(golden["step_geom"]))
    assert list(g.points) == list(golden["step_np"])
    v, w1, vg, ap, nv = O.step_fields(pos, rec[:, 3:6], w, s, g, np.float32(1.0 / 30.0), 0.01, pse_mode=0)
    assert np.array_equal(bits(nv), bits(golden["step_negvort"]))
    assert np.array_equal(bits(ap), bits(golden["step_vecpot"]))
    assert np.array_equal(bits(vg), bits(golden["step_velgrid"]))
    out = golden["step_out"]
    assert np.array_equal(bits(v), bits(out[:, 3:6]))
    assert np.array_equal(bits(w1), bits(out[:, 9:12]))


@pytest.fixture(scope="module")
def lifecycle():
    """PclOpKillAge / PclOpWind outputs of the reference's own code (make_golden.py lifecycle)."""
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "lifecycle.npz")))


def test_kill_age_order_bit_exact(oracle_lib, lifecycle):
    """Survivors and their order after PclOpKillAge: none, all, the first, the
    last, alternate and random particles too old, birth -1, wrapped ages."""
    for i in range(int(lifecycle["kill_cases"])):
        frame, age_max = (int(v) for v in lifecycle[f"kill{i}_frame_agemax"])
        got = oracle_lib.kill_age(lifecycle[f"kill{i}_birth"], frame, age_max)
        assert np.array_equal(got, lifecycle[f"kill{i}_order"]), i


def test_wind_bit_exact(oracle_lib, lifecycle):
    for i in range(int(lifecycle["wind_cases"])):
        ww, sw = (float(v) for v in lifecycle[f"wind{i}_weights"])
        got = oracle_lib.wind(lifecycle["wind_in"], lifecycle["wind_vec"], ww, sw)
        assert np.array_equal(bits(got), bits(lifecycle[f"wind{i}_out"])), i


def test_heat_pse_sequential_bit_exact(oracle_lib, golden):
    """The oracle's heat PSE in the reference's in-place order reproduces the
    reference's DiffuseAndDissipateHeatPSE bit for bit (tests/golden/heat.npz),
    including a diffusivity that saturates both clamps."""
    h = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "heat.npz")))
    g = geom_of(oracle_lib, golden)
    for i in range(int(h["heat_cases"])):
        kappa, ambient, dt = (np.float32(v) for v in h[f"heat{i}_params"])
        got = oracle_lib.heat_pse(golden["pos"], h["heat_density"], golden["size"], g, kappa, ambient, dt)
        assert np.array_equal(bits(got), bits(h[f"heat{i}_out"])), i


def test_heat_pse_symmetric_tolerance(oracle_lib, golden):
    """The order-independent heat PSE (the GPU's form) against the reference's
    in-place order at diffusivity 0.01: each pair exchanges <= 6.7e-4 of its
    difference, so the forms differ by ~(neighbours x 6.7e-4) of the change.
    Stated tolerance: 1e-4 relative on the densities, 2% on their change."""
    h = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "heat.npz")))
    g = geom_of(oracle_lib, golden)
    kappa, ambient, dt = (np.float32(v) for v in h["heat0_params"])
    d0 = h["heat_density"]
    sym = oracle_lib.heat_pse(golden["pos"], d0, golden["size"], g, kappa, ambient, dt, symmetric=True)
    ref = h["heat0_out"]
    assert np.linalg.norm(sym - ref) / np.linalg.norm(ref) < 1e-4
    assert np.linalg.norm((sym - d0) - (ref - d0)) / np.linalg.norm(ref - d0) < 0.02


@pytest.mark.parametrize("n,seed", [(1, 0), (50, 1), (3001, 2)])
def test_kill_age_permutation_properties(oracle_lib, n, seed):
    """The kill's survivors are exactly the young particles; the survivors
    below the survivor count keep their slots; the removed slots there are
    filled, in ascending order, by the survivors above it taken from the end."""
    rng = np.random.default_rng(seed)
    birth = rng.integers(0, 100, n).astype(np.int32)
    frame, age_max = 100, int(rng.integers(0, 100))
    order = oracle_lib.kill_age(birth, frame, age_max)
    alive = (frame - birth) <= age_max
    m = int(alive.sum())
    assert len(order) == m and sorted(order.tolist()) == np.flatnonzero(alive).tolist()
    holes = [i for i in range(m) if not alive[i]]
    movers = [p for p in range(n - 1, m - 1, -1) if alive[p]]
    want = np.arange(m)
    for k, i in enumerate(holes):
        want[i] = movers[k]
    assert np.array_equal(order, want)


def test_partition_is_stable_index_order(oracle_lib, golden):
    """PartitionParticles (Particles/particle.cpp:398-437) appends indices in
    particle order, so each list is ascending: the oracle's lists equal a
    stable sort of the particles by OffsetOfPosition, with the extra list
    (index `points`) for positions outside the grid."""
    O = oracle_lib
    g = geom_of(O, golden)
    pos = np.concatenate([golden["bin_pos"], np.array([[1e6, 0, 0], [np.nan, 0, 0]], np.float32)])
    idx, off = O.indices_of_position(g, pos)
    inside = (idx < np.array(g.points, np.uint32)).all(1) & np.isfinite(pos).all(1)
    key = np.where(inside, off, g.capacity)
    start, items = O.partition(g, pos)
    assert np.array_equal(items, np.argsort(key, kind="stable"))
    assert np.array_equal(np.diff(start.astype(np.int64)), np.bincount(key, minlength=g.capacity + 1))
    assert start[-1] == len(pos) and key[-1] == key[-2] == g.capacity


def test_tree_matches_reference_at_treecode_workload_size(oracle_lib):
    """The oracle's influence tree and treecode walk equal the reference's own
    code on the treecode workload (65,536 vortons in 8 rings, 64^3 cells,
    depth-7 NestedGrid), bit for bit."""
    import ctypes
    O = oracle_lib
    if not O.ref_available("serial"):
        pytest.skip("reference code not built on this host")
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.rings(65536, count=8, seed=2, box=2.0)
    g = O.step_geometry(pos, float(s[0]) * 0.5)
    assert g.points == (65, 65, 65)
    L = O.ref("serial")
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    g12, np3 = g.as12(), np.array(g.points, np.uint32)
    n = L.vgref_influence_tree(P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(g12), P(np3), None, ctypes.c_size_t(0))
    rt = np.zeros((n, 7), np.float32)
    L.vgref_influence_tree(P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(g12), P(np3), P(rt), ctypes.c_size_t(n))
    assert np.array_equal(bits(O.influence_tree(pos, w, s, g)), bits(rt))
    q = np.concatenate([workloads.grid_points(list(g.mn), list(g.cell), g.points)[::97], pos[::31]]).astype(np.float32)
    for kind in (0, 1):
        out = np.zeros((len(q), 3), np.float32)
        L.vgref_tree(kind, P(pos), P(w), P(s), ctypes.c_size_t(len(pos)), P(g12), P(np3), P(q), ctypes.c_size_t(len(q)),
                     ctypes.c_float(2.5), ctypes.c_float(0.6), P(out))
        assert np.array_equal(bits(O.tree(kind, pos, w, s, g, q, 2.5, 0.6)), bits(out)), kind


def _surface():
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "surface.npz")))


def test_density_gradient_baroclinic_sdf_bit_exact(oracle_lib):
    """The oracle's density grid (PopulateDensityAndMassFractionGrids),
    gradient (ComputeGradient), density-grid baroclinic generation and signed
    distance grid (PopulateSignedDistanceGridFromDensityGrid, with the
    reference's float statistics) equal the reference's own code on a ring
    with varying densities and a heavy puff (tests/golden/surface.npz)."""
    O = oracle_lib
    h = _surface()
    dt, ambient = (float(v) for v in h["surface_params"])
    for i in range(int(h["surface_cases"])):
        g = O.Geom.from12(h[f"s{i}_geom"], h[f"s{i}_np"])
        pos, size, dens = h[f"s{i}_pos"], h[f"s{i}_size"], h[f"s{i}_density"]
        dg = O.density_grid(pos, size, dens, g, ambient)
        assert np.array_equal(bits(dg), bits(h[f"s{i}_density_grid"])), i
        assert np.array_equal(bits(O.gradient(g, dg)), bits(h[f"s{i}_gradient"])), i
        applied, w = O.baroclinic(pos, h[f"s{i}_angvel"], size, dens, g, h[f"s{i}_grav"], ambient, np.float32(dt))
        assert applied == bool(h[f"s{i}_applied"])
        assert np.array_equal(bits(w), bits(h[f"s{i}_baroclinic"])), i
        sdf = O.signed_distance(g, dg, ambient, sumstats=0)
        assert np.array_equal(bits(sdf), bits(h[f"s{i}_sdf"])), i
        # double-precision statistics (a parallel reduction's) move the pinned
        # values, and the distances swept from them, by ~1e-6 relative
        sdf1 = O.signed_distance(g, dg, ambient, sumstats=1)
        assert np.nanmax(np.abs(sdf1 - sdf)) <= 1e-5 * float(np.nanmax(np.abs(sdf)))
    # no gravity along the grid: the reference returns before any change
    g = O.Geom.from12(h["s0_geom"], h["s0_np"])
    applied, w = O.baroclinic(h["s0_pos"], h["s0_angvel"], h["s0_size"], h["s0_density"], g, [0, 0, 0], ambient,
                              np.float32(dt))
    assert not applied and np.array_equal(w, h["s0_angvel"])


def test_marching_cubes_table_is_closed(oracle_lib):
    """The generated triangulation: every case's triangles use exactly the
    edges whose end points lie on opposite sides of the iso level, each
    triangle edge between two crossing edges is used once in each direction
    within a case's loops (closed loops), at most 5 triangles per cell, and a
    sphere's surface on a 65^3 grid is closed with outward normals."""
    from collections import Counter
    from vortegrid_gb300 import workloads
    cnt, tri = oracle_lib.marching_cubes_table()
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    edge = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
    assert cnt.max() <= 5 and cnt[0] == 0 and cnt[255] == 0
    for m in range(256):
        crossing = {e for e, (a, b) in enumerate(edge) if ((m >> a) & 1) != ((m >> b) & 1)}
        used = set(tri[m][: 3 * cnt[m]].tolist())
        assert used == crossing, m
    n = 65
    g = oracle_lib.Geom.from12(np.array([-1, -1, -1, 2, 2, 2, 2 / 64, 2 / 64, 2 / 64, 32, 32, 32], np.float32),
                               (n, n, n))
    pts = workloads.grid_points([-1.0] * 3, [2 / 64] * 3, [n] * 3)
    sdf = (np.linalg.norm(pts.astype(np.float64), axis=1) - 0.6).astype(np.float32)
    V, N = oracle_lib.marching_cubes(g, sdf, 0.0)
    assert np.all(np.einsum("ij,ij->i", N[:, 0], V.mean(1)) > 0)
    edges = Counter()
    for t in np.round(V.astype(np.float64), 5):
        k = [tuple(p) for p in t]
        for i in range(3):
            edges[tuple(sorted((k[i], k[(i + 1) % 3])))] += 1
    assert set(edges.values()) == {2}
    assert corner[6] == (1, 1, 1)


def test_fluid_body_collisions_bit_exact(oracle_lib):
    """The oracle's CollideVortonsSlice, CollideTracersSlice (body by body)
    and RemoveEmbeddedParticles equal the reference's own code
    (tests/golden/bodies.npz): particles and body sums bit for bit, for a
    moving, spinning sphere, a hollow rotated box container and a rotated
    solid box."""
    O = oracle_lib
    h = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "bodies.npz")))
    p, v, w, d, out = O.collide_vortons(h["b_pos"], h["b_vel"], h["b_angvel"], h["b_size"], h["b_density"],
                                        h["b_bodies"])
    for got, key in ((p, "b_vort_pos"), (v, "b_vort_vel"), (w, "b_vort_angvel"), (d, "b_vort_density"),
                     (out, "b_vort_sums")):
        assert np.array_equal(bits(got), bits(h[key])), key
    moved = np.abs(p - h["b_pos"]).max(1) > 0
    assert 0 < moved.sum() < len(p)
    tp, tv, tout = O.collide_tracers(h["b_pos"], h["b_vel"], h["b_size"], h["b_density"], h["b_bodies"])
    for got, key in ((tp, "b_tr_pos"), (tv, "b_tr_vel"), (tout, "b_tr_sums")):
        assert np.array_equal(bits(got), bits(h[key])), key
    assert np.array_equal(O.remove_embedded(h["b_pos"], h["b_size"], h["b_bodies"]), h["b_survivors"])


def _emit_gold():
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "emit.npz")))


def _geom12(oracle_lib, g12, np3):
    g = oracle_lib.Geom()
    for a in range(3):
        g.mn[a], g.ext[a], g.cell[a], g.cpe[a], g.np[a] = g12[a], g12[3 + a], g12[6 + a], g12[9 + a], int(np3[a])
    return g


def test_emit_grid_bit_exact(oracle_lib):
    """PclOpEmit::Emit: the reference's tracer seeding (with and without the
    vortons' density-deviation mask, and the empty case) after srand(seed),
    bit for bit."""
    e = _emit_gold()
    for i in range(int(e["emit_cases"])):
        m, seed, masked = (int(v) for v in e[f"e{i}_params"])
        g = _geom12(oracle_lib, e[f"e{i}_geom"], e[f"e{i}_np"])
        oracle_lib.srand(seed)
        vort = (e[f"e{i}_vpos"], e[f"e{i}_vdens"]) if masked else None
        pos, dens, size = oracle_lib.emit_grid(g, m, vort)
        assert len(pos) == len(e[f"e{i}_pos"]), i
        for got, key in ((pos, "pos"), (dens, "density"), (size, "size")):
            assert np.array_equal(got.view(np.uint32), e[f"e{i}_{key}"].view(np.uint32)), (i, key)
    assert len(e["e3_pos"]) == 0  # vortons at the ambient density: nothing emitted


def test_emit_operate_bit_exact(oracle_lib):
    """PclOpEmit::Operate over five frames (remainder carried), template +
    RandomSpread of the spread in the reference's draw order, bit for bit."""
    e = _emit_gold()
    rate, frame0, seed = e["op_params"]
    oracle_lib.srand(int(seed))
    rec, rem = oracle_lib.emit_operate(e["op_tmpl"], e["op_spread"], float(rate), e["op_dts"], frame0=int(frame0))
    assert np.array_equal(rec.view(np.uint32), e["op_records"].view(np.uint32))
    assert np.array_equal(rem.view(np.uint32), e["op_remainders"].view(np.uint32))


def test_emit_hash_stream_properties(oracle_lib):
    """The device emitter's own jitter stream (no rand()): every draw in
    [0, RAND_MAX], seeds give different streams, each particle inside its own
    sub-cell, and the same count and sub-cell order as the rand() stream."""
    rmax = oracle_lib.rand_max()
    d = [oracle_lib.jitter_hash(7, k) for k in range(2000)] + [oracle_lib.jitter_hash(7, (1 << 32) + k)
                                                               for k in range(100)]
    assert min(d) >= 0 and max(d) <= rmax
    assert len(set(d)) > 2000
    assert d[:50] != [oracle_lib.jitter_hash(8, k) for k in range(50)]
    e = _emit_gold()
    g = _geom12(oracle_lib, e["e1_geom"], e["e1_np"])
    m = 5
    pos, dens, size = oracle_lib.emit_grid(g, m, None, host_rand=False, seed=3)
    assert len(pos) == len(e["e1_pos"])
    sub = np.array([g.cell[a] for a in range(3)], np.float64) / m
    mn = np.array([g.mn[a] for a in range(3)], np.float64)
    expect = np.floor((e["e1_pos"].astype(np.float64) - mn) / sub)  # sub-cell of the reference's particle
    got = np.floor((pos.astype(np.float64) - mn) / sub)
    assert np.array_equal(got, expect)
    assert np.array_equal(size, e["e1_size"]) and np.all(dens == 1.0)
