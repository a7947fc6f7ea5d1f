"""GPU tests of the learned warm start (vg_net_*), through the C ABI.

  * every kernel of a forward + backward pass (convolutions, input and
    weight gradients, pooling, gradient routing, loss gradient) against the
    float64 CPU oracle (oracle/unet_ref.py) on the GPU's own inputs, and the
    whole pass end to end; tolerances are stated in each test;
  * the guess written into the vector potential against the oracle's;
  * weight file round trip; training steps that fit one pair;
  * the warm start inside vg_step and its fallback to a zero start.
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

EDGE = 32


@pytest.fixture(scope="module")
def ws():
    import vortegrid_gb300 as vg
    from vortegrid_gb300 import warmstart
    vg.lib()
    return warmstart


@pytest.fixture(scope="module")
def U():
    from oracle import unet_ref
    return unet_ref


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_param_layout_matches_oracle(ws, U):
    assert ws.lib().vg_net_param_count() == U.param_count()
    assert [(ci, co) for (_, ci, co, _, _) in U.LAYERS] == ws.LAYERS


def random_pair(n, seed):
    rng = np.random.default_rng(seed)
    np1 = n + 1
    # smooth-ish right-hand side plus noise, and a random "solution"
    z, y, x = np.meshgrid(*(np.linspace(-1, 1, np1),) * 3, indexing="ij")
    base = np.stack([np.sin(3 * x) * np.cos(2 * y), np.cos(2 * z) * y, x * z], -1).reshape(-1, 3)
    rhs = (base + 0.3 * rng.normal(size=base.shape)).astype(np.float32)
    vp = (0.5 * base[:, ::-1] + 0.1 * rng.normal(size=base.shape)).astype(np.float32)
    return rhs, vp


ACT_C = [16, 16, 16, 16, 32, 32, 32, 64, 64, 64, 128, 128, 64, 64, 32, 32, 16, 16]
ACT_L = [0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 2, 2, 1, 1, 0, 0]
IN1 = [0, 1, 3, 4, 6, 7, 9, 10, 11, 12, 13, 14, 15, 16, 17]
IN2 = [None] * 8 + [8, None, 5, None, 2, None, None]
OUT = [1, 2, 4, 5, 7, 8, 10, 11, 12, 13, 14, 15, 16, 17, None]


@pytest.fixture(scope="module")
def pass_data(ws, U):
    """One forward + backward pass at edge 32 with every tensor read back."""
    net = ws.Network(EDGE)
    grid = ws.field_grid(EDGE + 1)
    p = ws.init_params(seed=11, zero_output=False)
    rng = np.random.default_rng(5)
    o = 0
    for (ci, co) in ws.LAYERS:  # non-zero biases exercise the bias paths
        o += 27 * co * ci
        p[o:o + co] = rng.normal(0, 0.05, co)
        o += co
    K = 0.5
    net.set_params(p, K)
    rhs, vp = random_pair(EDGE, 3)
    loss = net.backward(grid, torch.from_numpy(rhs).cuda(), torch.from_numpy(vp).cuda(), want_loss=True)
    d = {"loss": loss, "grads": net.grads(), "out": net.output(), "params": net.params()[0], "rhs": rhs, "vp": vp,
         "hk": U.h2k(list(grid.cell_spacing), K)}
    d["acts"] = [net.activation(k, ACT_C[k], ACT_L[k]) for k in range(18)]
    d["g"] = [net.gradient(l, 0, co, U.LAYERS[l][0]) for l, (ci, co) in enumerate(ws.LAYERS)]
    d["gin"] = {l: net.gradient(l, 1, U.LAYERS[l][1], U.LAYERS[l][0]) for l in (2, 4, 6, 8, 10, 12)}
    return d


def layer_params(p, l, U):
    o = 0
    for k, (_, ci, co, _, _) in enumerate(U.LAYERS):
        if k == l:
            return p[o:o + 27 * co * ci].reshape(27, co, ci), p[o + 27 * co * ci:o + 27 * co * ci + co]
        o += 27 * co * ci + co


def test_each_kernel_matches_oracle(pass_data, U):
    """Every kernel of the pass against the oracle on the GPU's own inputs.

    Tolerances (relative L2): BF16 outputs 2e-3 (an FP32 and a float64 sum of
    the same products may round to neighbouring BF16 values), FP32 output 1e-5,
    weight and bias gradients 1e-4 (FP32 accumulation)."""
    d = pass_data
    A, p = d["acts"], d["params"]
    errs = {}
    for l, (level, ci, co, cup, relu) in enumerate(U.LAYERS):
        e = EDGE >> level
        x1 = A[IN1[l]]
        x2 = A[IN2[l]] if IN2[l] is not None else None
        y = U.layer_forward(l, p, x1, x2, e)
        got = A[OUT[l]] if OUT[l] is not None else d["out"]
        errs[f"fwd{l}"] = (rel(got, y), 1e-5 if OUT[l] is None else 2e-3)
        dw, db = U.layer_wgrad(l, x1, x2, d["g"][l], e)
        gw, gb = layer_params(d["grads"], l, U)
        errs[f"dW{l}"] = (rel(gw, dw), 1e-4)
        errs[f"db{l}"] = (rel(gb, db), 1e-4)
        if l == 0:
            continue
        if cup or l in (2, 4, 6):
            errs[f"dgrad{l}"] = (rel(d["gin"][l], U.layer_dgrad(l, p, d["g"][l], e)), 2e-3)
        else:
            errs[f"dgrad{l}"] = (rel(d["g"][l - 1], U.layer_dgrad(l, p, d["g"][l], e, mask=x1)), 2e-3)
    for src, dst in ((2, 3), (5, 6), (8, 9)):
        errs[f"pool{dst}"] = (rel(A[dst], U.pool(A[src], EDGE >> ACT_L[src])), 2e-3)
    for l, prod in ((8, 11), (10, 13), (12, 15)):
        e = EDGE >> U.LAYERS[l][0]
        errs[f"up{l}"] = (rel(d["g"][l - 1], U.up_grad(d["gin"][l], U.LAYERS[l][3], A[prod], e)), 2e-3)
    for l, user, skip in ((2, 12, 2), (4, 10, 5), (6, 8, 8)):
        e = EDGE >> ACT_L[skip]
        want = U.skip_grad(d["gin"][user], U.LAYERS[user][3], d["gin"][l], A[skip], e)
        errs[f"skip{l}"] = (rel(d["g"][l - 1], want), 2e-3)
    errs["loss_grad"] = (rel(d["g"][14], U.loss_grad(d["out"], d["rhs"], d["vp"], EDGE, d["hk"])), 2e-3)
    bad = {k: v for k, v in errs.items() if not v[0] < v[1]}
    assert not bad, bad


def test_pass_matches_oracle_end_to_end(pass_data, U):
    """The whole pass against the oracle run from the same parameters and pair.

    Rounding differences of single kernels (bounded above) compound through 15
    forward and 30 backward layer operations at random initialisation, so the
    bounds here are wider: activations and output 1e-2, loss 1e-2, parameter
    gradients 1e-1 per layer (measured: below 5e-3 forward, below 5e-2 backward)."""
    d = pass_data
    loss_ref, g_ref, out_ref, acts_ref = U.loss_and_grads(d["params"], d["hk"], d["rhs"], d["vp"], EDGE)
    errs = {U.ACT_NAMES[k]: rel(d["acts"][k], acts_ref[k]) for k in range(18)}
    errs["output"] = rel(d["out"][:, :3], out_ref[:, :3])
    assert max(errs.values()) < 1e-2, errs
    assert abs(d["loss"] - loss_ref) / loss_ref < 1e-2, (d["loss"], loss_ref)
    gerr = []
    o = 0
    for (_, ci, co, _, _) in U.LAYERS:
        nw = 27 * co * ci
        gerr.append((rel(d["grads"][o:o + nw], g_ref[o:o + nw]), rel(d["grads"][o + nw:o + nw + co],
                                                                     g_ref[o + nw:o + nw + co])))
        o += nw + co
    assert max(max(a, b) for a, b in gerr) < 1e-1, gerr


def test_guess_matches_oracle(ws, U):
    net = ws.Network(EDGE)
    grid = ws.field_grid(EDGE + 1)
    p = ws.init_params(seed=2, zero_output=False)
    net.set_params(p, 2.0)
    rhs, vp = random_pair(EDGE, 9)
    vp_dev = torch.from_numpy(vp).cuda()
    net.guess(grid, torch.from_numpy(rhs).cuda(), vp_dev)
    got = vp_dev.cpu().numpy().reshape(-1, 3)  # guess() orders torch's stream after the network's
    pw, K = net.params()
    want = U.guess(pw, U.h2k(list(grid.cell_spacing), K), rhs, vp, EDGE)
    np1 = EDGE + 1
    G, W = got.reshape(np1, np1, np1, 3), want.reshape(np1, np1, np1, 3)
    assert rel(G[1:EDGE, 1:EDGE, 1:EDGE], W[1:EDGE, 1:EDGE, 1:EDGE]) < 1e-2
    # boundary points are untouched
    bnd = np.ones((np1,) * 3, bool)
    bnd[1:EDGE, 1:EDGE, 1:EDGE] = False
    assert np.array_equal(G[bnd], vp.reshape(np1, np1, np1, 3)[bnd])


def test_weight_file_round_trip(ws, tmp_path):
    a = ws.Network(EDGE)
    p = ws.init_params(seed=4, zero_output=False)
    a.set_params(p, 3.5)
    path = str(tmp_path / "net.vgnet")
    a.save(path)
    b = ws.Network(EDGE)
    b.load(path)
    q, K = b.params()
    assert K == np.float32(3.5)
    want = torch.from_numpy(p).to(torch.bfloat16).float().numpy()
    # weights round to BF16 in the file, biases are stored exactly
    o = 0
    for (ci, co) in ws.LAYERS:
        nw = 27 * co * ci
        assert np.array_equal(q[o:o + nw], want[o:o + nw])
        assert np.array_equal(q[o + nw:o + nw + co], p[o + nw:o + nw + co])
        o += nw + co
    with open(path, "r+b") as f:
        f.seek(0)
        f.write(b"XXXX")
    with pytest.raises(Exception):
        b.load(path)


def test_training_fits_one_pair(ws):
    net = ws.Network(EDGE)
    grid = ws.field_grid(EDGE + 1)
    net.set_params(ws.init_params(seed=0), 1.0)
    rhs, vp = random_pair(EDGE, 1)
    R, V = torch.from_numpy(rhs).cuda(), torch.from_numpy(vp).cuda()
    first = net.backward(grid, R, V, want_loss=True)
    for _ in range(60):
        net.backward(grid, R, V)
        net.adam_step(3e-4)
    last = net.backward(grid, R, V, want_loss=True)
    assert last < 0.5 * first, (first, last)


def test_bf16_pairs_train_like_fp32(ws):
    net = ws.Network(EDGE)
    grid = ws.field_grid(EDGE + 1)
    net.set_params(ws.init_params(seed=0, zero_output=False), 1.0)
    rhs, vp = random_pair(EDGE, 1)
    R, V = torch.from_numpy(rhs).cuda(), torch.from_numpy(vp).cuda()
    l32 = net.backward(grid, R, V, want_loss=True)
    g32 = net.grads()
    l16 = net.backward(grid, R.to(torch.bfloat16), V.to(torch.bfloat16), want_loss=True)
    g16 = net.grads()
    assert abs(l16 - l32) / l32 < 2e-2
    assert rel(g16, g32) < 5e-2


def test_gradient_accumulation_adds(ws):
    net = ws.Network(EDGE)
    grid = ws.field_grid(EDGE + 1)
    net.set_params(ws.init_params(seed=3, zero_output=False), 1.0)
    pairs = [random_pair(EDGE, k) for k in (4, 5)]
    dev = [(torch.from_numpy(r).cuda(), torch.from_numpy(v).cuda()) for r, v in pairs]
    net.backward(grid, *dev[0])
    g0 = net.grads()
    net.backward(grid, *dev[1])
    g1 = net.grads()
    net.backward(grid, *dev[0])
    net.backward(grid, *dev[1], accumulate=True)
    assert rel(net.grads(), g0.astype(np.float64) + g1) < 1e-5


def test_step_uses_network_and_falls_back(ws):
    import vortegrid_gb300 as vg
    from vortegrid_gb300 import workloads
    net = ws.Network(EDGE)
    net.set_params(ws.init_params(seed=0), 1.0)
    pos, w, s = workloads.ring(2000, seed=1)
    ps = np.zeros((len(pos), 4), np.float32)
    ps[:, :3], ps[:, 3] = pos, s
    ww = np.zeros((len(pos), 4), np.float32)
    ww[:, :3] = w

    def run(points):
        grid = vg.GridGeom.make([-2.0] * 3, [4.0] * 3, [points] * 3)
        ctx = vg.VortonSim(fixed_grid=grid, warm_start=2, enable_diffusion=0, enable_stretch=0)
        assert vg.lib().vg_set_network(ctx.h, net.h) == 0
        P, Wt, Vl = torch.from_numpy(ps).cuda(), torch.from_numpy(ww).cuda(), torch.zeros(len(ps), 4).cuda()
        ctx.UpdateDevice(P, Wt, Vl, 1.0 / 30.0)
        ctx.synchronize()
        st = ctx.stats()
        return st

    st = run(EDGE + 1)
    assert st.warm_start_used == 2
    assert st.poisson_relres <= 1e-6
    st = run(EDGE + 9)   # grid does not fit the network: plain zero start
    assert st.warm_start_used == 0
    assert st.poisson_relres <= 1e-6


def test_trained_network_gains_over_zero_start(ws):
    """The committed network on held-out seeded fields (seeds disjoint from
    training): it starts far closer to the solution than the zero start (error
    below half of the zero start's), never needs more multigrid cycles to the
    same 1e-6 tolerance, and where both starts take the same number of cycles
    it ends at a lower residual; both end at the same solution.  (With the
    exact coarse-level solve the cycle counts are equal on these fields: the
    network's gain shows in the starting error and the final residual, not in
    solve time.)"""
    if not os.path.exists(ws.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights")
    summ, rows = ws.evaluate(ws.DEFAULT_WEIGHTS, fields=4, seed=11, log=None)
    for r in rows:
        assert r["zero_relres"] <= 1e-6 and r["nn_relres"] <= 1e-6, r
        assert r["nn_err0"] < 0.5, r           # the zero start's error is 1 by definition
        assert r["nn_cycles"] <= r["zero_cycles"], r
        if r["nn_cycles"] == r["zero_cycles"]:
            assert r["nn_relres"] < r["zero_relres"], r
        assert r["nn_vs_zero_solution"] < 1e-3, r


def test_network_start_keeps_velocity_error(ws):
    """Equal velocity error against the FP64 direct-sum oracle: the velocity
    grids of the zero-start and network-start solves (curl of the vector
    potential) differ from the FP64 direct sum at sampled interior grid points
    by the same relative L2 error, to 1e-4 of each other."""
    import vortegrid_gb300 as vg
    import oracle
    if not os.path.exists(ws.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights")
    oracle.build()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        solver = ws.Solver(0, s)
        net = ws.Network(ws.EDGE, 0, s)
        net.load(ws.DEFAULT_WEIGHTS)
        ps, w = ws.make_field("rings", 9_000_777_001)
        g = solver.grid
        n3 = g.capacity * 3
        rhs = torch.empty(n3, device="cuda")
        vp0 = torch.empty(n3, device="cuda")
        solver.rhs(ps, w, rhs)
        solver.boundary(ps, w, vp0)
        vels = []
        for use_net in (False, True):
            vp = vp0.clone()
            if use_net:
                net.guess(g, rhs, vp)
            cyc, r0, r1 = solver.multigrid(rhs, vp)
            assert r1 <= 1e-6
            vel = torch.empty(n3, device="cuda")
            c = solver.ctx
            with ws._Ordered(solver.stream):
                c.check(vg.lib().vg_jacobian_curl_device(c.h, ctypes.byref(g), ctypes.c_void_p(vp.data_ptr()), None,
                                                         ctypes.c_void_p(vel.data_ptr())), "vg_jacobian_curl_device")
            vels.append(vel.cpu().numpy().reshape(-1, 3))
        torch.cuda.synchronize()
    pos = ps[:, :3].cpu().numpy()
    angvel = w[:, :3].cpu().numpy()
    size = ps[:, 3].cpu().numpy()
    rng = np.random.default_rng(3)
    np1 = g.points[0]
    idx = rng.integers(8, np1 - 8, (256, 3))
    flat = (idx[:, 2] * np1 + idx[:, 1]) * np1 + idx[:, 0]
    cell = np.float32(g.cell_spacing[0])
    q = np.float32(g.min_corner[0]) + idx.astype(np.float32) * cell
    ref = oracle.direct(0, pos, angvel, size, q, f64=True)  # kind 0: velocity
    errs = [rel(v[flat], ref) for v in vels]
    assert abs(errs[0] - errs[1]) < 1e-4 * max(1.0, errs[0]) + 1e-6, errs
