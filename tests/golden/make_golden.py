#!/usr/bin/env python3
"""Generate the golden vectors in tests/golden/ from the reference's own code.

Runs the reference's VortonSim functions (built from the reference sources by
oracle/ref_build, serial USE_TBB=0 build) on small seeded inputs and stores
inputs and outputs in reference.npz.  The inputs are stored too, so the tests
never depend on the random generator of the machine they run on.

Usage (needs the reference tree or a staged copy; run in this container):
    python tests/golden/make_golden.py              # reference.npz
    python tests/golden/make_golden.py lifecycle    # lifecycle.npz (PclOpKillAge, PclOpWind)
    python tests/golden/make_golden.py heat         # heat.npz (DiffuseAndDissipateHeatPSE)
    python tests/golden/make_golden.py surface      # surface.npz (density grid, gradient, baroclinic, SDF)
    python tests/golden/make_golden.py bodies       # bodies.npz (fluid-body collisions, embedded particles)
    python tests/golden/make_golden.py emit         # emit.npz (PclOpEmit::Emit and ::Operate)
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from vortegrid_gb300 import workloads  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference.npz")
OUT_LIFE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lifecycle.npz")
OUT_HEAT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "heat.npz")
OUT_SURF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "surface.npz")
OUT_BODY = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bodies.npz")
OUT_EMIT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "emit.npz")


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def main():
    oracle.build()
    R = oracle.ref("serial")
    g = {}
    # --- a7 DefineShape: ring box, degenerate z, one element, a long box
    shapes = [(1500, [-1.4, -1.4, -0.4], [1.4, 1.4, 0.4]), (4096, [-1.5, -1.5, -1.5], [1.5, 1.5, 1.5]),
              (1024, [0, 0, 0], [2, 3, 5]), (100, [-1, -1, 0.25], [1, 1, 0.25]), (1, [0, 0, 0], [1, 1, 1]),
              (262144, [-2.05, -2.05, -2.05], [2.05, 2.05, 2.05]), (77, [-3, 0.1, 2], [5, 0.3, 9])]
    g12s, nps = [], []
    for n, a, b in shapes:
        g12 = np.zeros(12, np.float32)
        np3 = np.zeros(3, np.uint32)
        R.vgref_define_shape(ctypes.c_size_t(n), P(np.array(a, np.float32)), P(np.array(b, np.float32)), 1, P(g12),
                             P(np3))
        g12s.append(g12)
        nps.append(np3)
    g["shape_n"] = np.array([s[0] for s in shapes], np.uint64)
    g["shape_min"] = np.array([s[1] for s in shapes], np.float32)
    g["shape_max"] = np.array([s[2] for s in shapes], np.float32)
    g["shape_geom"] = np.array(g12s)
    g["shape_np"] = np.array(nps)

    # --- a9 NestedGrid shape for every geometry above
    depth, layers, decims = [], [], []
    for g12, np3 in zip(g12s, nps):
        ln = np.zeros(96, np.uint32)
        dc = np.zeros(96, np.uint32)
        d = R.vgref_nested_grid_shape(P(g12), P(np3), P(ln), P(dc), 32)
        depth.append(d)
        layers.append(ln)
        decims.append(dc)
    g["nested_depth"] = np.array(depth, np.int32)
    g["nested_np"] = np.array(layers)
    g["nested_decim"] = np.array(decims)

    # --- vortons: a small ring, tilted, plus tracers
    pos, w, s = workloads.ring(1500, seed=11, axis=(0.3, 0.2, 1.0))
    n = len(pos)
    mn = pos.min(0) - 0.15
    mx = pos.max(0) + 0.15
    g12 = np.zeros(12, np.float32)
    np3 = np.zeros(3, np.uint32)
    R.vgref_define_shape(ctypes.c_size_t(n), P(mn.astype(np.float32)), P(mx.astype(np.float32)), 1, P(g12), P(np3))
    cap = int(np3.prod())
    g.update(pos=pos, angvel=w, size=s, geom=g12, np=np3)

    # --- a8 binning incl. points nudged to cell corners
    rng = np.random.default_rng(5)
    cell = g12[6:9]
    corner = (g12[0:3] + rng.integers(0, np3 - 1, (200, 3)).astype(np.float32) * cell).astype(np.float32)
    nudged = np.concatenate([corner, np.nextafter(corner, np.float32(-10)), np.nextafter(corner, np.float32(10)),
                             pos]).astype(np.float32)
    idx = np.zeros((len(nudged), 3), np.uint32)
    off = np.zeros(len(nudged), np.uint32)
    R.vgref_indices_of_position(P(g12), P(np3), P(nudged), ctypes.c_size_t(len(nudged)), P(idx), P(off))
    g.update(bin_pos=nudged, bin_idx=idx, bin_off=off)

    # --- a10/a11 influence tree
    tot = R.vgref_influence_tree(P(pos), P(w), P(s), ctypes.c_size_t(n), P(g12), P(np3), None, ctypes.c_size_t(0))
    tree = np.zeros((tot, 7), np.float32)
    R.vgref_influence_tree(P(pos), P(w), P(s), ctypes.c_size_t(n), P(g12), P(np3), P(tree), ctypes.c_size_t(tot))
    g["tree"] = tree

    # --- a2/a3/a5 direct and a12 treecode at queries (incl. one at a vorton, inside the core)
    q = np.concatenate([workloads.tracers(400, seed=6, lo=-1.3, hi=1.3), pos[:50] + 0.01]).astype(np.float32)
    g["q"] = q
    sr = np.float32(1.5)
    sc = np.float32(1.0) / (sr * sr * sr)
    g["spread"] = np.array([sr, sc], np.float32)
    for kind, name in ((0, "vel"), (1, "vecpot")):
        o = np.zeros((len(q), 3), np.float32)
        R.vgref_direct(kind, P(pos), P(w), P(s), ctypes.c_size_t(n), P(q), ctypes.c_size_t(len(q)), ctypes.c_float(1),
                       ctypes.c_float(1), P(o))
        g[f"direct_{name}"] = o
        o = np.zeros((len(q), 3), np.float32)
        R.vgref_tree(kind, P(pos), P(w), P(s), ctypes.c_size_t(n), P(g12), P(np3), P(q), ctypes.c_size_t(len(q)),
                     ctypes.c_float(1), ctypes.c_float(1), P(o))
        g[f"tree_{name}"] = o
        o = np.zeros((len(q), 3), np.float32)
        R.vgref_tree(kind, P(pos), P(w), P(s), ctypes.c_size_t(n), P(g12), P(np3), P(q), ctypes.c_size_t(len(q)),
                     ctypes.c_float(sr), ctypes.c_float(sc), P(o))
        g[f"tree_{name}_spread"] = o

    # --- a14 splat (scale -1)
    negvort = np.zeros((cap, 3), np.float32)
    R.vgref_splat(P(pos), P(w), P(s), ctypes.c_size_t(n), P(g12), P(np3), ctypes.c_float(-1.0), P(negvort))
    g["negvort"] = negvort
    # --- a13 boundary A
    bvp = np.zeros((cap, 3), np.float32)
    R.vgref_boundary_vecpot(P(pos), P(w), P(s), ctypes.c_size_t(n), P(g12), P(np3), 1, P(bvp))
    g["boundary_vecpot"] = bvp
    # --- a16 SOR (5 sweeps) and a15 cascade
    a = bvp.copy()
    R.vgref_sor(P(g12), P(np3), P(a), P(negvort), 5)
    g["sor5"] = a
    a = bvp.copy()
    R.vgref_cascade(P(g12), P(np3), P(a), P(negvort), 16)
    g["cascade"] = a
    # --- a17/a18 restriction (injection and averaging) and prolongation
    for acc, name in ((1, "inject"), (0, "average")):
        for reg, rname in ((1, "interior"), (0, "entire")):
            co = np.zeros((cap, 3), np.float32)
            cn = np.zeros(3, np.uint32)
            fo = np.zeros((cap, 3), np.float32)
            R.vgref_down_up(P(g12), P(np3), P(a), acc, reg, P(co), P(cn), P(fo))
            ccap = int(cn.prod())
            g[f"down_{name}"] = co[:ccap].copy()
            g["coarse_np"] = cn
            g[f"up_{name}_{rname}"] = fo
    # --- a19 Jacobian + curl of the cascade result
    jac = np.zeros((cap, 9), np.float32)
    curl = np.zeros((cap, 3), np.float32)
    R.vgref_jacobian_curl(P(g12), P(np3), P(a), P(jac), P(curl))
    g["jacobian"] = jac
    g["curl"] = curl
    # --- a20 stretch with that velocity grid
    ww = w.copy()
    dt = np.float32(1.0 / 30.0)
    R.vgref_stretch(P(pos), P(ww), P(s), ctypes.c_size_t(n), P(g12), P(np3), P(curl), ctypes.c_float(dt))
    g["stretched"] = ww
    # --- a22 PSE (serial, reference order)
    ww = w.copy()
    R.vgref_pse(P(pos), P(ww), P(s), ctypes.c_size_t(n), P(g12), P(np3), ctypes.c_float(0.01), ctypes.c_float(dt))
    g["pse"] = ww
    # --- a23/a24 gather + Euler of tracers inside the grid
    tr = (g12[0:3] + (g12[3:6] * 0.999) * np.random.default_rng(8).uniform(0, 1, (700, 3))).astype(np.float32)
    pp = tr.copy()
    vv = np.zeros_like(pp)
    R.vgref_advect(P(pp), P(vv), ctypes.c_size_t(len(pp)), P(g12), P(np3), P(curl), ctypes.c_float(dt))
    g.update(tracers=tr, tracer_vel=vv, tracer_pos1=pp)
    # --- a25 AABB
    bmn = np.zeros(3, np.float32)
    bmx = np.zeros(3, np.float32)
    R.vgref_find_bbox(P(pos), ctypes.c_size_t(n), P(bmn), P(bmx))
    g.update(bbox_min=bmn, bbox_max=bmx)

    # --- a26 full PclOpVortonSim::Operate on Particle records with a tracer box
    rec = np.zeros((n, 24), np.float32)  # 96-byte Particle records
    rec[:, 0:3] = pos
    rec[:, 9:12] = w
    rec[:, 12] = 1.0  # density
    rec[:, 13] = s
    rec_in = rec.copy()
    emin = np.array([-1.5, -1.5, -0.5], np.float32)
    emax = np.array([1.5, 1.5, 0.5], np.float32)
    sg = np.zeros(12, np.float32)
    sn = np.zeros(3, np.uint32)
    assert R.vgref_sizeof_particle() == 96
    R.vgref_step(P(rec), ctypes.c_size_t(n), P(emin), P(emax), ctypes.c_float(dt), ctypes.c_uint(0),
                 ctypes.c_float(0.01), P(sg), P(sn))
    scap = int(sn.prod())
    vel = np.zeros((scap, 3), np.float32)
    vp = np.zeros((scap, 3), np.float32)
    nv = np.zeros((scap, 3), np.float32)
    R.vgref_last_grids(P(vel), P(vp), P(nv))
    g.update(step_in=rec_in, step_out=rec, step_extra_min=emin, step_extra_max=emax, step_geom=sg, step_np=sn,
             step_velgrid=vel, step_vecpot=vp, step_negvort=nv)

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB, {len(g)} arrays)")


def lifecycle():
    """PclOpKillAge and PclOpWind from the reference on seeded inputs: birth
    times around the frame (none, all, the first, the last, alternate and
    random particles too old; birth -1; a frame past 2^31 where the age wraps
    negative), and velocities with signed zeros under several weight pairs
    (including the reference's do-nothing pair 0 / 1)."""
    oracle.build()
    R = oracle.ref("serial")
    rng = np.random.default_rng(20240611)
    g = {}
    cases = []
    n = 1000
    cases.append((np.full(n, 90, np.int32), 100, 20))                  # none too old
    cases.append((np.full(n, 10, np.int32), 100, 20))                  # all
    b = np.full(n, 90, np.int32); b[0] = 0; cases.append((b, 100, 20))  # the first
    b = np.full(n, 90, np.int32); b[-1] = 0; cases.append((b, 100, 20))  # the last
    b = np.where(np.arange(n) % 2 == 0, 0, 90).astype(np.int32); cases.append((b, 100, 20))  # alternate
    for m in (1, 2, 7, 4099):
        cases.append((rng.integers(50, 101, m).astype(np.int32), 100, int(rng.integers(0, 51))))
    cases.append((np.array([-1, 5, -1, 7, 99], np.int32), 30, 25))    # birth -1 (age frame + 1)
    cases.append((np.array([3, 0x7ffffff0, 5, 1], np.int32), 0x80000005, 10))  # ages wrap negative
    for i, (birth, frame, age_max) in enumerate(cases):
        order = np.zeros(len(birth), np.uint32)
        m = ctypes.c_size_t()
        R.vgref_kill_age(P(birth), ctypes.c_size_t(len(birth)), ctypes.c_uint(frame), ctypes.c_int(age_max), P(order),
                         ctypes.byref(m))
        g[f"kill{i}_birth"] = birth
        g[f"kill{i}_frame_agemax"] = np.array([frame, age_max], np.int64)
        g[f"kill{i}_order"] = order[: m.value].copy()
    g["kill_cases"] = np.array(len(cases))
    vel = rng.normal(0, 3, (777, 3)).astype(np.float32)
    vel[:5] = -0.0
    vel[5:9] = 0.0
    weights = [(0.125, 0.875), (0.0, 1.0), (1.0, 0.0), (0.3, 0.9), (0.0, 0.5)]
    wind = np.array([1.0, -2.5, 0.375], np.float32)
    for i, (ww, sw) in enumerate(weights):
        v = vel.copy()
        R.vgref_wind(P(v), ctypes.c_size_t(len(v)), P(wind), ctypes.c_float(ww), ctypes.c_float(sw))
        g[f"wind{i}_weights"] = np.array([ww, sw], np.float32)
        g[f"wind{i}_out"] = v
    g["wind_in"] = vel
    g["wind_vec"] = wind
    g["wind_cases"] = np.array(len(weights))
    np.savez_compressed(OUT_LIFE, **g)
    print(f"wrote {OUT_LIFE} ({os.path.getsize(OUT_LIFE) / 1e3:.1f} kB, {len(g)} arrays)")


def heat():
    """DiffuseAndDissipateHeatPSE from the reference on the vortons of
    reference.npz carrying seeded densities (ambient 1 + N(0, 0.2^2)), at a
    small and a large diffusivity (the second saturates both clamps)."""
    oracle.build()
    R = oracle.ref("serial")
    src = np.load(OUT)
    pos, s, g12, np3 = src["pos"], src["size"], src["geom"], src["np"]
    n = len(pos)
    rng = np.random.default_rng(77)
    d0 = (1.0 + rng.normal(0, 0.2, n)).astype(np.float32)
    g = {"heat_density": d0}
    cases = [(0.01, 1.0, 1.0 / 30.0), (1.8, 1.2, 1.0 / 3.0)]
    for i, (kappa, ambient, dt) in enumerate(cases):
        d = d0.copy()
        R.vgref_heat_pse(P(pos), P(d), P(s), ctypes.c_size_t(n), P(g12), P(np3), ctypes.c_float(kappa),
                         ctypes.c_float(ambient), ctypes.c_float(dt))
        g[f"heat{i}_params"] = np.array([kappa, ambient, dt], np.float32)
        g[f"heat{i}_out"] = d
    g["heat_cases"] = np.array(len(cases))
    np.savez_compressed(OUT_HEAT, **g)
    print(f"wrote {OUT_HEAT} ({os.path.getsize(OUT_HEAT) / 1e3:.1f} kB, {len(g)} arrays)")


def surface():
    """PopulateDensityAndMassFractionGrids (density), ComputeGradient, the
    density-grid baroclinic path of GenerateBaroclinicVorticity and
    PopulateSignedDistanceGridFromDensityGrid, from the reference's own code
    (oracle/ref_build/ref_harness.cpp), on two seeded fields: a ring with
    densities in [1, 1.5) and a heavy puff (density 2 in ambient 1)."""
    oracle.build()
    R = oracle.ref("serial")
    R.vgref_baroclinic.restype = ctypes.c_int
    g = {}
    rng = np.random.default_rng(41)
    ring = workloads.ring(3000, seed=7)
    puff = workloads.puff(3000, seed=8, sigma=0.3, clip=0.9)
    cases = [(ring, (1.0 + 0.5 * rng.random(3000)).astype(np.float32), [0.0, 0.0, -9.8]),
             (puff, np.full(3000, 2.0, np.float32), [1.0, -3.0, 2.0])]
    dt, ambient = np.float32(1.0 / 30.0), np.float32(1.0)
    for i, ((pos, w, s), dens, grav) in enumerate(cases):
        geo = oracle.step_geometry(pos, float(s[0]) * 0.5)
        g12, np3 = geo.as12(), np.array(geo.points, np.uint32)
        n, npts = len(pos), geo.capacity
        grav = np.array(grav, np.float32)
        dg = np.zeros(npts, np.float32)
        R.vgref_density_grid(P(pos), P(s), P(dens), ctypes.c_size_t(n), P(g12), P(np3), ctypes.c_float(ambient),
                             P(dg))
        gr = np.zeros((npts, 3), np.float32)
        R.vgref_gradient(P(g12), P(np3), P(dg), P(gr))
        wv = w.copy()
        applied = R.vgref_baroclinic(P(pos), P(wv), P(s), P(dens), ctypes.c_size_t(n), P(g12), P(np3), P(grav),
                                     ctypes.c_float(ambient), ctypes.c_float(dt))
        sdf = np.zeros(npts, np.float32)
        R.vgref_signed_distance(P(g12), P(np3), P(dg), ctypes.c_float(ambient), P(sdf))
        g.update({f"s{i}_pos": pos, f"s{i}_angvel": w, f"s{i}_size": s, f"s{i}_density": dens,
                  f"s{i}_geom": g12, f"s{i}_np": np3, f"s{i}_grav": grav, f"s{i}_density_grid": dg,
                  f"s{i}_gradient": gr, f"s{i}_baroclinic": wv, f"s{i}_applied": np.array(applied),
                  f"s{i}_sdf": sdf})
    g["surface_params"] = np.array([dt, ambient], np.float32)
    g["surface_cases"] = np.array(len(cases))
    np.savez_compressed(OUT_SURF, **g)
    print(f"wrote {OUT_SURF} ({os.path.getsize(OUT_SURF) / 1e3:.1f} kB, {len(g)} arrays)")


def bodies():
    """FluidBodySim::CollideVortonsSlice, CollideTracersSlice (per body in
    turn) and RemoveEmbeddedParticles from the reference's own code
    (oracle/ref_build/ref_harness.cpp) on a seeded puff of 2,000 particles
    with three bodies: a moving, spinning, hot sphere; a hollow rotated box
    that contains the fluid; a small moving, spinning, rotated solid box."""
    oracle.build()
    R = oracle.ref("serial")
    n = 2000
    pos, w, s = workloads.puff(n, seed=9, sigma=0.5, clip=1.2)
    rng = np.random.default_rng(2)
    vel = rng.normal(0.0, 0.5, (n, 3)).astype(np.float32)
    dens = (1.0 + 0.1 * rng.random(n)).astype(np.float32)
    c, sn = np.cos(0.3), np.sin(0.3)
    rot = np.array([[c, -sn, 0], [sn, c, 0], [0, 0, 1]], np.float32)
    B = np.stack([oracle.body(0, [0.2, 0, 0], [0.4], velocity=[0.5, 0, 0], angular_velocity=[0, 0, 1],
                              temperature=350, conductivity=0.5),
                  oracle.body(1, [0, 0, 0], [2.0, 2.0, 1.6], hole=True, orientation=rot, temperature=300,
                              conductivity=0.1),
                  oracle.body(1, [0.0, 0.5, 0.3], [0.3, 0.4, 0.5], velocity=[0, 0.2, 0], angular_velocity=[0.3, 0, 0],
                              orientation=rot, temperature=320, conductivity=0.2)]).astype(np.float32)
    g = {"b_pos": pos, "b_vel": vel, "b_angvel": w, "b_size": s, "b_density": dens, "b_bodies": B}
    p, v, a, d = pos.copy(), vel.copy(), w.copy(), dens.copy()
    out = np.zeros((len(B), 9), np.float32)
    R.vgref_collide_vortons(P(p), P(v), P(a), P(s), P(d), ctypes.c_size_t(n), P(B), len(B), ctypes.c_float(1.0),
                            ctypes.c_float(1.0), P(out))
    g.update({"b_vort_pos": p, "b_vort_vel": v, "b_vort_angvel": a, "b_vort_density": d, "b_vort_sums": out})
    p, v = pos.copy(), vel.copy()
    out6 = np.zeros((len(B), 6), np.float32)
    R.vgref_collide_tracers(P(p), P(v), P(s), P(dens), ctypes.c_size_t(n), P(B), len(B), P(out6))
    g.update({"b_tr_pos": p, "b_tr_vel": v, "b_tr_sums": out6})
    order = np.zeros(n, np.uint32)
    m = ctypes.c_size_t()
    R.vgref_remove_embedded(P(pos), P(s), ctypes.c_size_t(n), P(B), len(B), P(order), ctypes.byref(m))
    g["b_survivors"] = order[: m.value].copy()
    np.savez_compressed(OUT_BODY, **g)
    print(f"wrote {OUT_BODY} ({os.path.getsize(OUT_BODY) / 1e3:.1f} kB, {len(g)} arrays)")


def emit():
    """PclOpEmit::Emit (tracer seeding on a grid, without and with vortons)
    and PclOpEmit::Operate (rate emission over five frames) from the
    reference's own code after srand(seed): the jitter is the C library's
    rand() stream, the same on every glibc host."""
    oracle.build()
    R = oracle.ref("serial")

    def geom(mn, mx, np3):
        go = oracle.Geom()
        for a in range(3):
            go.mn[a], go.ext[a], go.np[a] = mn[a], mx[a] - mn[a], np3[a]
        oracle.lib().vgo_precompute_spacing(ctypes.byref(go))
        return (np.array(list(go.mn) + list(go.ext) + list(go.cell) + list(go.cpe), np.float32),
                np.array(np3, np.uint32))

    rng = np.random.default_rng(31)
    vpos, _, _ = workloads.puff(3000, seed=32, sigma=0.35, clip=0.9)
    r2 = (vpos.astype(np.float64) ** 2).sum(1)
    vdens = (1.0 + 0.6 * np.exp(-r2 / 0.4) - 0.4 * np.exp(-((vpos[:, 0] - 0.4) ** 2) / 0.02)
             + 0.02 * rng.standard_normal(3000)).astype(np.float32)
    cases = [  # grid, multiplier, seed, vortons
        (geom([-1.0, -1.2, -0.8], [1.1, 1.0, 0.9], [7, 6, 5]), 2, 5, None),
        (geom([-1.0, -1.2, -0.8], [1.1, 1.0, 0.9], [7, 6, 5]), 5, 11, None),
        (geom([-1.0, -1.0, -1.0], [1.0, 1.0, 1.0], [9, 9, 9]), 3, 21, (vpos, vdens)),
        (geom([-1.0, -1.0, -1.0], [1.0, 1.0, 1.0], [9, 9, 9]), 2, 23, (vpos, np.ones(3000, np.float32))),
    ]
    g = {}
    for i, ((g12, np3), m, seed, vort) in enumerate(cases):
        cap = int(np.prod(np3 - 1)) * m ** 3
        pos = np.zeros((cap, 3), np.float32)
        d = np.zeros(cap, np.float32)
        sz = np.zeros(cap, np.float32)
        cnt = ctypes.c_size_t()
        vp, vd = vort if vort is not None else (np.zeros((1, 3), np.float32), np.zeros(1, np.float32))
        vs = np.full(len(vd), 0.05, np.float32)
        R.vgref_emit_grid(P(g12), P(np3), ctypes.c_uint(m), P(vp), P(vs), P(vd),
                          ctypes.c_size_t(len(vd) if vort is not None else 0), ctypes.c_int(vort is not None),
                          ctypes.c_uint(seed), P(pos), P(d), P(sz), ctypes.c_size_t(cap), ctypes.byref(cnt))
        k = cnt.value
        g.update({f"e{i}_geom": g12, f"e{i}_np": np3, f"e{i}_params": np.array([m, seed, vort is not None], np.int64),
                  f"e{i}_pos": pos[:k].copy(), f"e{i}_density": d[:k].copy(), f"e{i}_size": sz[:k].copy()})
        if vort is not None:
            g.update({f"e{i}_vpos": vp, f"e{i}_vdens": vd})
    g["emit_cases"] = np.array(len(cases))
    tmpl = np.array([0.1, 0.2, 0.3, 1, 2, 3, 0.5, 0.6, 0.7, 4, 5, 6, 1.5, 0.2, 0.3, 0.4, 0.05], np.float32)
    spread = np.array([0.5, 0.4, 0.3, 0.1, 0.2, 0.3, 0.01, 0.02, 0.03, 1, 1, 1, 0.1, 0.05, 0.05, 0.05, 0.01],
                      np.float32)
    dts = np.array([1 / 60, 1 / 30, 0.1, 0.013, 0.5], np.float32)
    rate, frame0, seed = 60.0, 7, 9
    cap = 256
    rec = np.zeros((cap, 18), np.float32)
    cnt = ctypes.c_size_t()
    rem = np.zeros(len(dts), np.float32)
    R.vgref_emit_operate(P(tmpl), P(spread), ctypes.c_float(rate), P(dts), ctypes.c_int(len(dts)),
                         ctypes.c_uint(frame0), ctypes.c_uint(seed), P(rec), ctypes.c_size_t(cap), ctypes.byref(cnt),
                         P(rem))
    g.update({"op_tmpl": tmpl, "op_spread": spread, "op_dts": dts,
              "op_params": np.array([rate, frame0, seed], np.float64), "op_records": rec[: cnt.value].copy(),
              "op_remainders": rem})
    np.savez_compressed(OUT_EMIT, **g)
    print(f"wrote {OUT_EMIT} ({os.path.getsize(OUT_EMIT) / 1e3:.1f} kB, {len(g)} arrays)",
          [len(g[f"e{i}_pos"]) for i in range(len(cases))], len(g["op_records"]))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "lifecycle":
        lifecycle()
    elif len(sys.argv) > 1 and sys.argv[1] == "heat":
        heat()
    elif len(sys.argv) > 1 and sys.argv[1] == "surface":
        surface()
    elif len(sys.argv) > 1 and sys.argv[1] == "bodies":
        bodies()
    elif len(sys.argv) > 1 and sys.argv[1] == "emit":
        emit()
    else:
        main()
