"""vg_direct_noalloc: the direct sum for callers that cannot allocate device
memory (fixed memory budgets, real-time frames that must not stall on the
allocator, embeddings that forbid it).  Its scratch is a fixed 8 MiB array
inside the library; this checks it against vg_direct_device through the C
ABI, twice in a row (the second call reuses whatever the first left in the
shared array), and that oversize calls are refused.

Named to be collected last, so a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def f4(xyz, w=None):
    out = np.zeros((len(xyz), 4), np.float32)
    out[:, :3] = xyz
    if w is not None:
        out[:, 3] = w
    return torch.from_numpy(out).cuda()


def test_noalloc_matches_direct_device_twice():
    import vortegrid_gb300 as vg
    from vortegrid_gb300 import workloads
    lib = vg.lib()
    pos, w, s = workloads.ring(4096, seed=1)
    q = np.concatenate([workloads.grid_points([-1.5] * 3, [3 / 32] * 3, [33] * 3), pos]).astype(np.float32)
    ps, wd, qd = f4(pos, s), f4(w), f4(q)
    ctx = vg.Context()
    ref = torch.zeros((len(q), 4), dtype=torch.float32, device="cuda")
    ctx.check(lib.vg_direct_device(ctx.h, 0, vg._ptr(ps), vg._ptr(wd), len(ps), vg._ptr(qd), len(q), 1.0, 1.0,
                                   vg._ptr(ref)), "vg_direct_device")
    ctx.synchronize()
    r = ref.cpu().numpy()[:, :3]
    stream = torch.cuda.current_stream().cuda_stream
    for kind in (0, 1):
        if kind == 1:
            ctx.check(lib.vg_direct_device(ctx.h, 1, vg._ptr(ps), vg._ptr(wd), len(ps), vg._ptr(qd), len(q), 1.0,
                                           1.0, vg._ptr(ref)), "vg_direct_device")
            ctx.synchronize()
            r = ref.cpu().numpy()[:, :3]
        for call in range(2):
            out = torch.full((len(q), 4), float("nan"), dtype=torch.float32, device="cuda")
            st = lib.vg_direct_noalloc(ctypes.c_void_p(stream), kind, vg._ptr(ps), vg._ptr(wd), len(ps), vg._ptr(qd),
                                       len(q), 1.0, 1.0, vg._ptr(out))
            assert st == vg.OK, lib.vg_last_error(None)
            torch.cuda.synchronize()
            got = out.cpu().numpy()[:, :3]
            assert np.all(np.isfinite(got))
            # the direct-sum tolerance used throughout the tests (rel-L2 1e-5)
            assert np.linalg.norm(got - r) / np.linalg.norm(r) < 1e-5, (kind, call)


def test_noalloc_refuses_oversize():
    import vortegrid_gb300 as vg
    lib = vg.lib()
    big = torch.zeros((40000, 4), dtype=torch.float32, device="cuda")
    q = torch.zeros((8, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros_like(q)
    st = lib.vg_direct_noalloc(None, 0, vg._ptr(big), vg._ptr(big), 40000, vg._ptr(q), 8, 1.0, 1.0, vg._ptr(out))
    assert st == vg.TOO_LARGE
    assert b"32768" in lib.vg_last_error(None)
    many = torch.zeros((1_000_000, 4), dtype=torch.float32, device="cuda")
    st = lib.vg_direct_noalloc(None, 0, vg._ptr(q), vg._ptr(q), 8, vg._ptr(many), 1_000_000, 1.0, 1.0,
                               vg._ptr(many))
    assert st == vg.TOO_LARGE
