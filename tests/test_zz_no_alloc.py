"""vg_direct_noalloc: the direct sum for callers that cannot allocate device
memory when they need a velocity -- applications with a fixed memory budget,
real-time frames that must not stall on the allocator's implicit
synchronisation, embeddings that forbid the CUDA allocator.  Its scratch is a
fixed 8 MiB array inside the library.  Checked here through the C ABI:
  * twice in a row (the second call reuses whatever the first left in the
    shared array) against vg_direct_device -- bit for bit, since it runs the
    same kernels with the same source split -- and against the FP64 direct-sum
    oracle within the direct-sum tolerance of the other tests (rel-L2 1e-5);
  * at the size limit (32,768 sources, targets filling the array);
  * with no sources (zero output);
  * that a call leaves the device's free memory unchanged;
  * that oversize calls are refused.

Named to be collected last, so a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SCRATCH = 8 << 20


def f4(xyz, w=None):
    out = np.zeros((len(xyz), 4), np.float32)
    out[:, :3] = xyz
    if w is not None:
        out[:, 3] = w
    return torch.from_numpy(out).cuda()


def device_sum(vg, ctx, kind, ps, wd, qd):
    ref = torch.zeros((qd.shape[0], 4), dtype=torch.float32, device="cuda")
    ctx.check(vg.lib().vg_direct_device(ctx.h, kind, vg._ptr(ps), vg._ptr(wd), ps.shape[0], vg._ptr(qd), qd.shape[0],
                                        1.0, 1.0, vg._ptr(ref)), "vg_direct_device")
    ctx.synchronize()
    return ref.cpu().numpy()[:, :3]


def noalloc(vg, kind, ps, wd, n, qd, out):
    stream = torch.cuda.current_stream().cuda_stream
    st = vg.lib().vg_direct_noalloc(ctypes.c_void_p(stream), kind, vg._ptr(ps), vg._ptr(wd), n, vg._ptr(qd),
                                    qd.shape[0], 1.0, 1.0, vg._ptr(out))
    assert st == vg.OK, vg.lib().vg_last_error(None)
    torch.cuda.synchronize()
    return out.cpu().numpy()[:, :3]


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.parametrize("kind,n", [(0, 4096), (1, 4096), (1, 1024)])
def test_noalloc_matches_direct_device_and_fp64_twice(oracle_lib, kind, n):
    """The direct-sum workload's ring and targets (the 33^3 gridpoints and the
    vortons).  Where vg_direct_device's source split fits the 8 MiB array
    (velocity; vector potential from 1,024 sources) the sums are bit-identical
    to it; where the array caps the split (vector potential from 4,096
    sources: ~30 chunks x 40k targets x 12 B) the partial sums are grouped
    differently and equal within rounding."""
    import vortegrid_gb300 as vg
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(n, seed=1)
    q = np.concatenate([workloads.grid_points([-1.5] * 3, [3 / 32] * 3, [33] * 3), pos]).astype(np.float32)
    ps, wd, qd = f4(pos, s), f4(w), f4(q)
    ctx = vg.Context()
    r = device_sum(vg, ctx, kind, ps, wd, qd)
    exact = oracle_lib.direct(kind, pos, w, s, q, f64=True)
    capped = kind == 1 and n > 1024
    for call in range(2):
        out = torch.full((len(q), 4), float("nan"), dtype=torch.float32, device="cuda")
        got = noalloc(vg, kind, ps, wd, len(pos), qd, out)
        assert np.all(np.isfinite(got))
        if not capped:
            assert np.array_equal(got.view(np.uint32), r.view(np.uint32)), (kind, call)
        # the direct-sum tolerance used throughout the tests (rel-L2 1e-5)
        assert rel(got, r) < 1e-5, (kind, call)
        assert rel(got, exact) < 1e-5, (kind, call, rel(got, exact))


def test_noalloc_at_the_size_limit():
    """32,768 sources and as many targets as the array holds beside their
    constants ((8 MiB - 32 n) / 12): the same sums as vg_direct_device."""
    import vortegrid_gb300 as vg
    from vortegrid_gb300 import workloads
    n = 32768
    m = (SCRATCH - 32 * n) // 12
    pos, w, s = workloads.puff(n, seed=9)
    q = workloads.tracers(m, seed=10, lo=-1.5, hi=1.5)
    ps, wd, qd = f4(pos, s), f4(w), f4(q)
    ctx = vg.Context()
    for kind in (0, 1):
        r = device_sum(vg, ctx, kind, ps, wd, qd)
        out = torch.full((m, 4), float("nan"), dtype=torch.float32, device="cuda")
        got = noalloc(vg, kind, ps, wd, n, qd, out)
        assert np.all(np.isfinite(got))
        assert rel(got, r) < 1e-5, kind
    big = torch.zeros((m + 1, 4), dtype=torch.float32, device="cuda")
    st = vg.lib().vg_direct_noalloc(None, 0, vg._ptr(ps), vg._ptr(wd), n, vg._ptr(big), m + 1, 1.0, 1.0, vg._ptr(big))
    assert st == vg.TOO_LARGE


def test_noalloc_no_sources_gives_zero():
    import vortegrid_gb300 as vg
    q = f4(np.zeros((1000, 3), np.float32))
    out = torch.full((1000, 4), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = vg.lib().vg_direct_noalloc(ctypes.c_void_p(stream), 0, None, None, 0, vg._ptr(q), 1000, 1.0, 1.0,
                                    vg._ptr(out))
    assert st == vg.OK
    torch.cuda.synchronize()
    assert torch.count_nonzero(out).item() == 0


def test_noalloc_leaves_free_memory_unchanged():
    import vortegrid_gb300 as vg
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.ring(4096, seed=1)
    q = workloads.tracers(100000, seed=3, lo=-1.5, hi=1.5)
    ps, wd, qd = f4(pos, s), f4(w), f4(q)
    out = torch.zeros((len(q), 4), dtype=torch.float32, device="cuda")
    noalloc(vg, 0, ps, wd, len(pos), qd, out)  # warm-up: module and array already in place
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for kind in (0, 1, 0):
        noalloc(vg, kind, ps, wd, len(pos), qd, out)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


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
