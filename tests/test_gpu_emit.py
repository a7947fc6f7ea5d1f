"""GPU emitters through the C ABI, against the reference's own PclOpEmit
(tests/golden/emit.npz, made by tests/golden/make_golden.py emit) and the C
oracle:
  * PclOpEmit::Emit after srand(seed): the tracer seeding with and without
    the vortons' density-deviation mask, and the empty case, bit for bit,
    appended behind particles already live (left untouched);
  * PclOpEmit::Operate over five frames after srand(seed): records and the
    carried remainder bit for bit;
  * the device jitter stream against the oracle at the tracer workload's size
    (4,096,000 tracers: 32^3 cells, 5^3 per cell), unmasked and masked;
  * a full group is refused with nothing written.
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOO_LARGE = 9


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


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
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "emit.npz")))


def srand(seed):
    ctypes.CDLL(None).srand(ctypes.c_uint(seed))


def case_geom(vg, e, i):
    return vg.GridGeom.from12(e[f"e{i}_geom"], e[f"e{i}_np"])


def vortons_on_device(vpos, vdens):
    ps = np.zeros((len(vpos), 4), np.float32)
    ps[:, :3] = vpos
    ps[:, 3] = 0.05
    return torch.from_numpy(ps).cuda(), torch.from_numpy(np.ascontiguousarray(vdens, np.float32)).cuda()


def test_emit_grid_matches_reference(vg, ctx, gold):
    for i in range(int(gold["emit_cases"])):
        m, seed, masked = (int(v) for v in gold[f"e{i}_params"])
        ref_pos = gold[f"e{i}_pos"]
        live = 37
        grp = vg.ParticleGroup(live + max(len(ref_pos), 1) + 5, fire=True, orientation=True)
        grp.pos_size[:live] = 7.0
        grp.birth[:live] = 3
        grp.count = live
        vort = vortons_on_device(gold[f"e{i}_vpos"], gold[f"e{i}_vdens"]) if masked else None
        srand(seed)
        vg.PclOpEmit.Emit(ctx, grp, case_geom(vg, gold, i), m, vort)
        torch.cuda.synchronize()
        k = len(ref_pos)
        assert grp.count == live + k, i
        ps = grp.pos_size.cpu().numpy()
        assert np.all(ps[:live] == 7.0) and np.all(grp.birth[:live].cpu().numpy() == 3)
        out = slice(live, live + k)
        assert np.array_equal(bits(ps[out, :3]), bits(ref_pos)), i
        assert np.array_equal(bits(ps[out, 3]), bits(gold[f"e{i}_size"])), i
        assert np.array_equal(bits(grp.density.cpu().numpy()[out]), bits(gold[f"e{i}_density"])), i
        assert np.all(grp.vel4.cpu().numpy()[out] == 0) and np.all(grp.angvel4.cpu().numpy()[out] == 0)
        assert np.all(grp.orient4.cpu().numpy()[out] == 0) and np.all(grp.birth.cpu().numpy()[out] == 0)
        assert np.all(grp.fire4.cpu().numpy()[out] == np.array([0, 0, 1, 0], np.float32))


def test_emit_operate_matches_reference(vg, ctx, gold):
    t, s = gold["op_tmpl"], gold["op_spread"]
    rate, frame0, seed = gold["op_params"]
    names = [("position", 0, 3), ("velocity", 3, 3), ("orientation", 6, 3), ("angular_velocity", 9, 3),
             ("density", 12, 1), ("fuel_fraction", 13, 1), ("flame_fraction", 14, 1), ("smoke_fraction", 15, 1),
             ("size", 16, 1)]
    op = vg.PclOpEmit(ctx)
    op.mTemplate = {n: (t[a:a + k] if k > 1 else t[a]) for n, a, k in names}
    op.mSpread = {n: (s[a:a + k] if k > 1 else s[a]) for n, a, k in names}
    op.mEmitRate = float(rate)
    grp = vg.ParticleGroup(64, fire=True, orientation=True)
    srand(int(seed))
    rems = []
    for f, dt in enumerate(gold["op_dts"]):
        op.Operate(grp, float(dt), int(frame0) + f)
        rems.append(op.mRemainder)
    torch.cuda.synchronize()
    R = gold["op_records"]
    k = len(R)
    assert grp.count == k
    assert np.array_equal(bits(np.array(rems, np.float32)), bits(gold["op_remainders"]))
    ps, v, w = grp.pos_size.cpu().numpy(), grp.vel4.cpu().numpy(), grp.angvel4.cpu().numpy()
    o, fire = grp.orient4.cpu().numpy(), grp.fire4.cpu().numpy()
    assert np.array_equal(bits(ps[:k, :3]), bits(R[:, 0:3]))
    assert np.array_equal(bits(v[:k, :3]), bits(R[:, 3:6]))
    assert np.array_equal(bits(o[:k, :3]), bits(R[:, 6:9]))
    assert np.array_equal(bits(w[:k, :3]), bits(R[:, 9:12]))
    assert np.array_equal(bits(grp.density.cpu().numpy()[:k]), bits(R[:, 12]))
    assert np.array_equal(bits(fire[:k, :3]), bits(R[:, 13:16]))
    assert np.array_equal(bits(ps[:k, 3]), bits(R[:, 16]))
    assert np.array_equal(grp.birth.cpu().numpy()[:k], R[:, 17].astype(np.int32))


def test_emit_full_group_is_refused(vg, ctx, gold):
    g = case_geom(vg, gold, 0)
    grp = vg.ParticleGroup(100)
    grp.count = 10
    with pytest.raises(vg.VgError) as ex:
        vg.PclOpEmit.Emit(ctx, grp, g, 2)
    assert ex.value.status == TOO_LARGE and grp.count == 10
    assert float(grp.pos_size.abs().sum()) == 0.0
    op = vg.PclOpEmit(ctx)
    op.mEmitRate = 1000.0
    op.mRemainder = 0.25
    with pytest.raises(vg.VgError):
        op.Operate(grp, 1.0, 0)
    assert op.mRemainder == 0.25 and grp.count == 10


def test_emit_hash_stream_at_workload_size(vg, ctx, oracle_lib):
    """Tracer seeding at the workload's size from the device's own jitter
    stream: 32^3 cells x 5^3 = 4,096,000 tracers bit-identical to the oracle;
    then masked by 200,000 puff vortons."""
    g = vg.define_shape(32768, np.array([-1.0, -1.0, -1.0], np.float32), np.array([1.0, 1.0, 1.0], np.float32),
                        pow2=False)
    go = oracle_lib.Geom()
    for a in range(3):
        go.mn[a], go.ext[a], go.cell[a], go.cpe[a], go.np[a] = (g.min_corner[a], g.extent[a], g.cell_spacing[a],
                                                                g.cells_per_extent[a], g.num_points[a])
    cells = int(np.prod([g.num_points[a] - 1 for a in range(3)]))
    total = cells * 125
    grp = vg.ParticleGroup(total)
    vg.PclOpEmit.Emit(ctx, grp, g, 5, None, vg.JITTER_HASH, 77)
    torch.cuda.synchronize()
    pos, dens, size = oracle_lib.emit_grid(go, 5, None, host_rand=False, seed=77)
    assert grp.count == total == len(pos)
    ps = grp.pos_size.cpu().numpy()
    assert np.array_equal(bits(ps[:, :3]), bits(pos)) and np.array_equal(bits(ps[:, 3]), bits(size))
    del grp
    from vortegrid_gb300 import workloads
    vp, _, _ = workloads.puff(200000, seed=5, sigma=0.3, clip=0.9)
    vd = (1.0 + 0.5 * np.exp(-(vp.astype(np.float64) ** 2).sum(1) / 0.2)).astype(np.float32)
    vps, vds = vortons_on_device(vp, vd)
    grp = vg.ParticleGroup(total)
    vg.PclOpEmit.Emit(ctx, grp, g, 2, (vps, vds), vg.JITTER_HASH, 78)
    torch.cuda.synchronize()
    pos, dens, size = oracle_lib.emit_grid(go, 2, (vp, vd), host_rand=False, seed=78)
    k = grp.count
    assert k == len(pos) and k > 1000
    ps = grp.pos_size.cpu().numpy()
    assert np.array_equal(bits(ps[:k, :3]), bits(pos))
    assert np.array_equal(bits(grp.density.cpu().numpy()[:k]), bits(dens))
