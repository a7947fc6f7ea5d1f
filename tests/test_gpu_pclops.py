"""GPU parity of the device particle operations (vg_wind_device,
vg_kill_age_device) with the C oracle, itself pinned bit-exactly to the
reference's PclOpWind / PclOpKillAge (tests/test_oracle_golden.py): the same
golden inputs, then large seeded inputs.  Bit-exact: the wind's FP32
products and sums, and the survivors and their order after the kill."""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "lifecycle.npz")


@pytest.fixture(scope="module")
def env():
    import oracle
    import vortegrid_gb300 as vg
    oracle.build()
    L = vg.lib()
    cfg = vg.default_config(device=0)
    h = ctypes.c_void_p()
    assert L.vg_create(ctypes.byref(cfg), ctypes.byref(h)) == vg.OK
    yield vg, L, h, oracle
    L.vg_destroy(h)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def gpu_kill(env, birth, frame, age_max, with_arrays=True):
    vg, L, h, _ = env
    n = len(birth)
    ids = np.arange(n, dtype=np.float32)
    a = torch.from_numpy(np.stack([ids, -ids, ids + 0.5, 2 * ids], 1).astype(np.float32)).cuda() if with_arrays else None
    c = torch.from_numpy(np.stack([ids * 3, ids, ids, ids], 1).astype(np.float32)).cuda() if with_arrays else None
    b = torch.from_numpy(np.ascontiguousarray(birth, np.int32)).cuda()
    m = ctypes.c_size_t()
    assert L.vg_kill_age_device(h, ptr(a), None, ptr(c), ptr(b), n, frame, age_max, ctypes.byref(m)) == vg.OK
    m = m.value
    order = a[:m, 0].cpu().numpy().astype(np.int64) if with_arrays else None
    if with_arrays:
        assert torch.equal(a[:m, 1], -a[:m, 0]) and torch.equal(c[:m, 0], 3 * a[:m, 0])
        assert np.array_equal(b[:m].cpu().numpy(), np.asarray(birth, np.int32)[order])
    return m, order


def test_kill_age_matches_reference_goldens(env):
    g = dict(np.load(GOLD))
    for i in range(int(g["kill_cases"])):
        frame, age_max = (int(v) for v in g[f"kill{i}_frame_agemax"])
        m, order = gpu_kill(env, g[f"kill{i}_birth"], frame, age_max)
        assert m == len(g[f"kill{i}_order"]) and np.array_equal(order, g[f"kill{i}_order"]), i


@pytest.mark.parametrize("n,seed", [(1, 1), (33, 2), (100_000, 3), (1_000_003, 4)])
def test_kill_age_matches_oracle_large(env, n, seed):
    rng = np.random.default_rng(seed)
    birth = rng.integers(0, 200, n).astype(np.int32)
    frame, age_max = 200, int(rng.integers(0, 200))
    m, order = gpu_kill(env, birth, frame, age_max)
    want = env[3].kill_age(birth, frame, age_max)
    assert m == len(want) and np.array_equal(order, want)


def test_kill_age_birth_only_and_empty(env):
    vg, L, h, _ = env
    m, _ = gpu_kill(env, np.array([0, 9, 0, 9], np.int32), 10, 5, with_arrays=False)
    assert m == 2
    mm = ctypes.c_size_t(7)
    assert L.vg_kill_age_device(h, None, None, None, None, 0, 1, 0, ctypes.byref(mm)) == vg.OK and mm.value == 0


def test_wind_matches_reference_goldens_and_oracle(env):
    vg, L, h, O = env
    g = dict(np.load(GOLD))
    for i in range(int(g["wind_cases"])):
        ww, sw = (float(v) for v in g[f"wind{i}_weights"])
        v4 = np.zeros((len(g["wind_in"]), 4), np.float32)
        v4[:, :3] = g["wind_in"]
        v4[:, 3] = 7.0
        t = torch.from_numpy(v4).cuda()
        assert L.vg_wind_device(h, ptr(t), len(v4), g["wind_vec"].ctypes.data_as(ctypes.c_void_p), ww, sw) == vg.OK
        L.vg_synchronize(h)
        out = t.cpu().numpy()
        assert np.array_equal(out[:, :3].view(np.uint32), g[f"wind{i}_out"].view(np.uint32)), i
        assert np.all(out[:, 3] == 7.0)
    rng = np.random.default_rng(9)
    vel = rng.normal(0, 5, (500_000, 3)).astype(np.float32)
    want = O.wind(vel, [0.5, 1.5, -2.0], 0.2, 0.8)
    v4 = np.zeros((len(vel), 4), np.float32)
    v4[:, :3] = vel
    t = torch.from_numpy(v4).cuda()
    wv = np.array([0.5, 1.5, -2.0], np.float32)
    assert L.vg_wind_device(h, ptr(t), len(v4), wv.ctypes.data_as(ctypes.c_void_p), 0.2, 0.8) == vg.OK
    L.vg_synchronize(h)
    assert np.array_equal(t.cpu().numpy()[:, :3].view(np.uint32), want.view(np.uint32))
