"""GPU fluid-body boundary conditions through the C ABI, against the
reference's own code (tests/golden/bodies.npz, made by
tests/golden/make_golden.py bodies) and the C oracle: a moving, spinning,
hot sphere; a hollow rotated box containing the fluid; a rotated solid box.
  * CollideVortonsSlice body by body: every vorton's position, velocity,
    angular velocity and density bit-exact; the body sums (FP64 reductions in
    a fixed order, the reference adds in vorton order in FP32) within 1e-5 of
    their scale, collision counts exact;
  * CollideTracersSlice: tracers bit-exact, body impulses within 1e-5;
  * RemoveEmbeddedParticles: the survivors and their order exact;
  * 262,144 particles against the oracle, bit for bit.
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def f4(xyz, w=None):
    out = np.zeros((len(xyz), 4), np.float32)
    out[:, :3] = xyz
    if w is not None:
        out[:, 3] = w
    return torch.from_numpy(out).cuda()


@pytest.fixture(scope="module")
def vg():
    import vortegrid_gb300 as vg
    vg.lib()
    return vg


@pytest.fixture(scope="module")
def ctx(vg):
    return vg.Context()


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "bodies.npz")))


def collide_vortons(vg, ctx, pos, vel, angvel, size, dens, bodies):
    ps, v, w = f4(pos, size), f4(vel), f4(angvel)
    d = torch.from_numpy(np.ascontiguousarray(dens, np.float32)).cuda()
    b = np.ascontiguousarray(bodies, np.float32)
    out = np.zeros((len(b), 9), np.float32)
    cnt = np.zeros(len(b), np.uint64)
    ctx.check(vg.lib().vg_collide_vortons_device(ctx.h, vg._ptr(b), len(b), vg._ptr(ps), vg._ptr(v), vg._ptr(w),
                                                 vg._ptr(d), len(pos), 1.0, 1.0, vg._ptr(out), vg._ptr(cnt)),
              "collide vortons")
    return (ps.cpu().numpy()[:, :3], v.cpu().numpy()[:, :3], w.cpu().numpy()[:, :3], d.cpu().numpy(), out, cnt)


def collide_tracers(vg, ctx, pos, vel, size, dens, bodies):
    ps, v = f4(pos, size), f4(vel)
    d = torch.from_numpy(np.ascontiguousarray(dens, np.float32)).cuda()
    b = np.ascontiguousarray(bodies, np.float32)
    out = np.zeros((len(b), 6), np.float32)
    ctx.check(vg.lib().vg_collide_tracers_device(ctx.h, vg._ptr(b), len(b), vg._ptr(ps), vg._ptr(v), vg._ptr(d),
                                                 len(pos), vg._ptr(out)), "collide tracers")
    return ps.cpu().numpy()[:, :3], v.cpu().numpy()[:, :3], out


def close(got, ref, scale):
    return np.all(np.abs(np.asarray(got, np.float64) - ref) <= 1e-5 * scale)


def test_collide_vortons_matches_reference(vg, ctx, gold):
    p, v, w, d, out, cnt = collide_vortons(vg, ctx, gold["b_pos"], gold["b_vel"], gold["b_angvel"], gold["b_size"],
                                           gold["b_density"], gold["b_bodies"])
    for got, key in ((p, "b_vort_pos"), (v, "b_vort_vel"), (w, "b_vort_angvel"), (d, "b_vort_density")):
        assert np.array_equal(bits(got), bits(gold[key])), key
    ref = gold["b_vort_sums"].astype(np.float64)
    assert np.array_equal(cnt.astype(np.float64), ref[:, 8])
    assert np.all(out[:, :3] == 0.0)
    for k in range(len(ref)):
        assert close(out[k, 3:6], ref[k, 3:6], np.abs(ref[k, 3:6]).max()), k
        assert close(out[k, 6:8], ref[k, 6:8], np.abs(ref[k, 6:8])), k
        # the body's new temperature (SolveBoundaryConditions' rule) from the reference's sums
        t_body, n = float(gold["b_bodies"][k, 23]), ref[k, 8]
        expect = t_body
        if n:
            half = 0.5 * abs(ref[k, 7] / n - t_body)
            expect = t_body + np.clip(ref[k, 6], -half, half)
        assert abs(out[k, 8] - expect) <= 1e-5 * abs(expect), k


def test_collide_tracers_matches_reference(vg, ctx, gold):
    p, v, out = collide_tracers(vg, ctx, gold["b_pos"], gold["b_vel"], gold["b_size"], gold["b_density"],
                                gold["b_bodies"])
    assert np.array_equal(bits(p), bits(gold["b_tr_pos"]))
    assert np.array_equal(bits(v), bits(gold["b_tr_vel"]))
    ref = gold["b_tr_sums"].astype(np.float64)
    for k in range(len(ref)):
        assert close(out[k, :3], ref[k, :3], np.abs(ref[k, :3]).max()), k
        assert close(out[k, 3:], ref[k, 3:], np.abs(ref[k, 3:]).max()), k


def remove_embedded(vg, ctx, pos, size, bodies):
    ps = f4(pos, size)
    idx = torch.arange(len(pos), dtype=torch.float32, device="cuda")  # exact below 2^24
    b = np.ascontiguousarray(bodies, np.float32)
    m = ctypes.c_size_t()
    ctx.check(vg.lib().vg_remove_embedded_device(ctx.h, vg._ptr(b), len(b), vg._ptr(ps), None, None, vg._ptr(idx),
                                                 len(pos), ctypes.byref(m)), "remove embedded")
    return idx.cpu().numpy()[: m.value].astype(np.uint32)


def test_remove_embedded_matches_reference(vg, ctx, gold):
    got = remove_embedded(vg, ctx, gold["b_pos"], gold["b_size"], gold["b_bodies"])
    assert np.array_equal(got, gold["b_survivors"])


def test_bodies_at_scale_match_oracle(vg, ctx, gold, oracle_lib):
    """262,144 puff particles and the same three bodies: vortons, tracers and
    the embedded-particle removal against the oracle, bit for bit."""
    from vortegrid_gb300 import workloads
    n = 262144
    pos, w, s = workloads.puff(n, seed=12, sigma=0.5, clip=1.2)
    rng = np.random.default_rng(13)
    vel = rng.normal(0.0, 0.5, (n, 3)).astype(np.float32)
    dens = (1.0 + 0.1 * rng.random(n)).astype(np.float32)
    B = gold["b_bodies"]
    p, v, ww, d, out, cnt = collide_vortons(vg, ctx, pos, vel, w, s, dens, B)
    op, ov, ow, od, oout = oracle_lib.collide_vortons(pos, vel, w, s, dens, B)
    for got, exp in ((p, op), (v, ov), (ww, ow), (d, od)):
        assert np.array_equal(bits(got), bits(exp))
    assert np.array_equal(cnt.astype(np.float64), oout[:, 8].astype(np.float64))
    tp, tv, _ = collide_tracers(vg, ctx, pos, vel, s, dens, B)
    otp, otv, _ = oracle_lib.collide_tracers(pos, vel, s, dens, B)
    assert np.array_equal(bits(tp), bits(otp)) and np.array_equal(bits(tv), bits(otv))
    assert np.array_equal(remove_embedded(vg, ctx, pos, s, B), oracle_lib.remove_embedded(pos, s, B))
