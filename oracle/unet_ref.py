"""CPU oracle for the learned warm-start network -- test infrastructure only.

The network has no counterpart in the reference (it warms the reference's
vector-potential solve, VortonFluid/vortonSim.cpp:2480-2560), so this file
restates the network that libvortegrid's vg_net_* kernels run, in float64
PyTorch on the CPU, from the definition alone:

  * layers (level, Ci, Co, channels read through 2x nearest upsampling, ReLU):
    the 4-level U-Net with 16/32/64/128 channels, 3x3x3 convolutions with zero
    padding, leaky ReLU (slope 0.1; none on the output), 2x2x2 average
    pooling, skip connections by channel concatenation;
  * parameters flat FP32: per layer W[27][Co][Ci] (tap = 9(dz+1) + 3(dy+1) +
    dx+1, the input read at (z+dz, y+dy, x+dx)) then bias[Co];
  * input channels: rhs / s, boundary values / (s h^2 K) (low faces; voxels
    next to a high face take their outer neighbour's value), zeros up to 16,
    s = RMS of the right-hand side over all points and 3 components;
  * loss: sum over interior voxels (all indices >= 1) and channels 0..2 of
    (out - vecpot / (s h^2 K))^2, divided by the sum of (vecpot / (s h^2 K))^2
    over the same entries (a relative squared error per field).

Where the GPU stores a tensor in BF16 (input, every activation, the pooled
tensors, the weights) this oracle rounds it to BF16 too, and where the GPU
stores a gradient in BF16 (pre-activation gradients, the loss gradient, the
gradients of concatenated and pooled inputs) the oracle rounds that gradient
on its way back, so that forward and backward results differ from the GPU's
only by summation order.  Only tests/ import this module.
"""
import numpy as np
import torch

SLOPE = 0.1  # leaky ReLU: v > 0 ? v : SLOPE v

# (level, ci, co, cup, relu) -- cup: channels of the first input read through upsampling
LAYERS = [
    (0, 16, 16, 0, 1), (0, 16, 16, 0, 1), (1, 16, 32, 0, 1), (1, 32, 32, 0, 1), (2, 32, 64, 0, 1),
    (2, 64, 64, 0, 1), (3, 64, 128, 0, 1), (3, 128, 128, 0, 1), (2, 192, 64, 128, 1), (2, 64, 64, 0, 1),
    (1, 96, 32, 64, 1), (1, 32, 32, 0, 1), (0, 48, 16, 32, 1), (0, 16, 16, 0, 1), (0, 16, 16, 0, 0),
]
ACT_NAMES = ["input", "enc0a", "enc0b", "pool1", "enc1a", "enc1b", "pool2", "enc2a", "enc2b", "pool3",
             "enc3a", "enc3b", "dec2a", "dec2b", "dec1a", "dec1b", "dec0a", "dec0b"]


def param_count():
    return sum(27 * co * ci + co for (_, ci, co, _, _) in LAYERS)


def split_params(p):
    """Flat parameters -> list of (W[27][Co][Ci], b[Co]) numpy views."""
    out, o = [], 0
    for (_, ci, co, _, _) in LAYERS:
        w = p[o:o + 27 * co * ci].reshape(27, co, ci)
        o += 27 * co * ci
        b = p[o:o + co]
        o += co
        out.append((w, b))
    assert o == len(p)
    return out


class _RoundBF16(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        return x.to(torch.bfloat16).to(torch.float64)

    @staticmethod
    def backward(ctx, g):
        return g


def bf16(x):
    return _RoundBF16.apply(x)


class _RoundGradBF16(torch.autograd.Function):
    """Identity forward; the gradient is rounded to BF16 on its way back."""

    @staticmethod
    def forward(ctx, x):
        return x.view_as(x)

    @staticmethod
    def backward(ctx, g):
        return g.to(torch.bfloat16).to(torch.float64)


def gbf16(x):
    return _RoundGradBF16.apply(x)


def torch_weight(w):
    """W[27][Co][Ci] -> conv3d weight [Co][Ci][3 (z)][3 (y)][3 (x)]."""
    co, ci = w.shape[1], w.shape[2]
    return w.reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2)


def h2k(cell, out_scale):
    """(cx^2 + cy^2 + cz^2) / 3 * K, each operation rounded to FP32 as on the GPU."""
    c = np.asarray(cell, np.float32)
    h2 = (c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) / np.float32(3.0)
    return np.float32(np.float32(h2) * np.float32(out_scale))


def scales(rhs, hk):
    s = float(np.sqrt(np.mean(rhs.astype(np.float64) ** 2)))
    if not (s > 0.0) or not np.isfinite(s):
        s = 1.0
    hk = float(hk)
    return np.float32(1.0 / s), np.float32(1.0 / (s * hk)), np.float32(s * hk)


def pack_input(rhs, vp, n, s_in, s_bc):
    """rhs, vp: [(n+1)^3, 3] float arrays (x fastest) -> [1, 16, n, n, n] float64 (BF16-rounded)."""
    np1 = n + 1
    R = rhs.reshape(np1, np1, np1, 3)[:n, :n, :n].astype(np.float32) * s_in
    V = vp.reshape(np1, np1, np1, 3).astype(np.float32)
    bc = np.zeros((n, n, n, 3), np.float32)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    low = (i == 0) | (j == 0) | (k == 0)
    high = ~low & ((i == n - 1) | (j == n - 1) | (k == n - 1))
    bc[low] = V[:n, :n, :n][low] * s_bc
    bi, bj, bk = np.where(i == n - 1, n, i), np.where(j == n - 1, n, j), np.where(k == n - 1, n, k)
    bc[high] = V[bk[high], bj[high], bi[high]] * s_bc
    x = np.zeros((n, n, n, 16), np.float64)
    x[..., 0:3] = R
    x[..., 3:6] = bc
    t = torch.from_numpy(x).permute(3, 0, 1, 2).unsqueeze(0)
    return bf16(t)


def forward(params, x, n, keep=False):
    """Network output [1, 16, n, n, n] float64 for input x; optionally every activation."""
    Ws = split_params(params)
    wt = [(bf16(torch_weight(torch.from_numpy(w.astype(np.float64)))), torch.from_numpy(b.astype(np.float64)))
          for (w, b) in Ws]
    return _forward_t(wt, x, keep)


def _conv(l, wt, inp, up=None):
    level, ci, co, cup, relu = LAYERS[l]
    if up is not None:
        # the GPU stores the gradient of the concatenated input in BF16
        inp = gbf16(torch.cat([torch.nn.functional.interpolate(up, scale_factor=2, mode="nearest"), inp], dim=1))
    # ... and the gradient of every pre-activation (the loss gradient for the output layer)
    y = gbf16(torch.nn.functional.conv3d(inp, wt[l][0], wt[l][1], padding=1))
    if relu:
        y = torch.nn.functional.leaky_relu(y, SLOPE)
    return y if l == len(LAYERS) - 1 else bf16(y)


def _pool(x):
    # the gradient of a pooled tensor is stored in BF16 as well
    return gbf16(bf16(torch.nn.functional.avg_pool3d(x, 2)))


def _forward_t(wt, x, keep):
    e0a = _conv(0, wt, x)
    e0b = _conv(1, wt, e0a)
    p1 = _pool(e0b)
    e1a = _conv(2, wt, p1)
    e1b = _conv(3, wt, e1a)
    p2 = _pool(e1b)
    e2a = _conv(4, wt, p2)
    e2b = _conv(5, wt, e2a)
    p3 = _pool(e2b)
    e3a = _conv(6, wt, p3)
    e3b = _conv(7, wt, e3a)
    d2a = _conv(8, wt, e2b, up=e3b)
    d2b = _conv(9, wt, d2a)
    d1a = _conv(10, wt, e1b, up=d2b)
    d1b = _conv(11, wt, d1a)
    d0a = _conv(12, wt, e0b, up=d1b)
    d0b = _conv(13, wt, d0a)
    out = _conv(14, wt, d0b)
    if keep:
        acts = [x, e0a, e0b, p1, e1a, e1b, p2, e2a, e2b, p3, e3a, e3b, d2a, d2b, d1a, d1b, d0a, d0b]
        return out, acts
    return out


def loss_and_grads(params, hk, rhs, vp, n):
    """(loss, flat float64 gradient, output [n^3][16], activations channels-last) for one pair;
    hk = h2k(cell spacing, output scale)."""
    s_in, s_t, _ = scales(rhs, hk)
    x = pack_input(rhs, vp, n, s_in, s_t)
    Ws = split_params(params)
    leaves = []
    wt = []
    for (w, b) in Ws:
        W = torch.tensor(w.astype(np.float64), requires_grad=True)
        B = torch.tensor(b.astype(np.float64), requires_grad=True)
        leaves += [W, B]
        wt.append((bf16(torch_weight(W)), B))
    out, acts = _forward_t(wt, x, keep=True)
    np1 = n + 1
    T = torch.from_numpy(vp.reshape(np1, np1, np1, 3)[:n, :n, :n].astype(np.float32) * s_t).to(torch.float64)
    T = T.permute(3, 0, 1, 2)
    d = out[0, 0:3] - T
    d = d[:, 1:, 1:, 1:]
    Ti = T[:, 1:, 1:, 1:]
    loss = (d * d).sum() / float((Ti * Ti).sum())
    loss.backward()
    g = np.concatenate([t.grad.numpy().ravel() for t in leaves])
    out_cl = out[0].detach().permute(1, 2, 3, 0).reshape(-1, 16).numpy()
    acts_cl = [a[0].detach().permute(1, 2, 3, 0).reshape(-1, a.shape[1]).numpy() for a in acts]
    return float(loss.detach()), g, out_cl, acts_cl


def guess(params, hk, rhs, vp, n):
    """Vector potential with the network's interior guess (the boundary of vp kept)."""
    s_in, s_t, s_out = scales(rhs, hk)
    x = pack_input(rhs, vp, n, s_in, s_t)
    with torch.no_grad():
        out = forward(params, x, n)
    np1 = n + 1
    res = vp.reshape(np1, np1, np1, 3).astype(np.float32).copy()
    o = out[0, 0:3].permute(1, 2, 3, 0).numpy().astype(np.float32) * s_out
    res[1:n, 1:n, 1:n] = o[1:, 1:, 1:]
    return res.reshape(-1, 3)


# ------------------------------------------------------------------ single kernels
# Each function below restates one GPU kernel of the network on inputs the GPU
# itself produced (channels-last float arrays holding BF16 values), so that a
# test compares every kernel on identical inputs instead of through the whole
# network, where rounding differences compound.

def _ncdhw(a, e):
    return torch.from_numpy(np.asarray(a, np.float64).reshape(e, e, e, -1)).permute(3, 0, 1, 2).unsqueeze(0)


def _cl(t):
    return t[0].permute(1, 2, 3, 0).reshape(-1, t.shape[1]).numpy()


def _rb(t):
    return t.to(torch.bfloat16).to(torch.float64)


def layer_input(l, x1, x2, e):
    """The (possibly upsampled and concatenated) input of layer l at edge e."""
    level, ci, co, cup, relu = LAYERS[l]
    if cup:
        up = torch.nn.functional.interpolate(_ncdhw(x1, e // 2), scale_factor=2, mode="nearest")
        return torch.cat([up, _ncdhw(x2, e)], dim=1)
    return _ncdhw(x1, e)


def layer_forward(l, params, x1, x2, e):
    """Output of layer l (BF16-rounded except the FP32 output layer), channels-last."""
    level, ci, co, cup, relu = LAYERS[l]
    w, b = split_params(params)[l]
    W = _rb(torch_weight(torch.from_numpy(w.astype(np.float64))))
    y = torch.nn.functional.conv3d(layer_input(l, x1, x2, e), W, torch.from_numpy(b.astype(np.float64)), padding=1)
    if relu:
        y = torch.nn.functional.leaky_relu(y, SLOPE)
    return _cl(y if l == len(LAYERS) - 1 else _rb(y))


def layer_wgrad(l, x1, x2, g, e):
    """(dW[27][Co][Ci], db[Co]) of layer l from its input and pre-activation gradient g."""
    level, ci, co, cup, relu = LAYERS[l]
    G = _ncdhw(g, e)
    dw = torch.nn.grad.conv3d_weight(layer_input(l, x1, x2, e), (co, ci, 3, 3, 3), G, padding=1)
    dw = dw.permute(2, 3, 4, 0, 1).reshape(27, co, ci)
    return dw.numpy(), G.sum((0, 2, 3, 4)).numpy()


def _dact(m):
    """Derivative of the leaky ReLU read off its (sign-preserving) output m."""
    return torch.where(m > 0, torch.ones_like(m), torch.full_like(m, SLOPE))


def layer_dgrad(l, params, g, e, mask=None):
    """Gradient w.r.t. layer l's input from its pre-activation gradient g, times
    the activation's derivative at mask if given, BF16-rounded; channels-last
    with Ci channels."""
    level, ci, co, cup, relu = LAYERS[l]
    w, _ = split_params(params)[l]
    W = _rb(torch_weight(torch.from_numpy(w.astype(np.float64))))
    d = torch.nn.grad.conv3d_input((1, ci, e, e, e), W, _ncdhw(g, e), padding=1)
    if mask is not None:
        d = d * _dact(_ncdhw(mask, e))
    return _cl(_rb(d))


def pool(x, e):
    """2x2x2 average of a level with edge e, BF16-rounded."""
    return _cl(_rb(torch.nn.functional.avg_pool3d(_ncdhw(x, e), 2)))


def up_grad(gin, cup, y, e):
    """Coarse gradient of an upsampled input: act'(y) * sum of the 8 children of gin[:, :cup]."""
    G = _ncdhw(gin, e)[:, :cup]
    s = G.reshape(1, cup, e // 2, 2, e // 2, 2, e // 2, 2).sum((3, 5, 7))
    return _cl(_rb(s * _dact(_ncdhw(y, e // 2))))


def skip_grad(gcat, cup, gp, skip, e):
    """act'(skip) * (gcat[:, cup:] + upsampled gp / 8) at edge e."""
    G = _ncdhw(gcat, e)[:, cup:]
    P = torch.nn.functional.interpolate(_ncdhw(gp, e // 2), scale_factor=2, mode="nearest")
    return _cl(_rb((G + P / 8) * _dact(_ncdhw(skip, e))))


def loss_grad(out, rhs, vp, n, hk):
    """BF16 loss gradient [n^3][16] from the network's FP32 output (channels-last)."""
    _, s_t, _ = scales(rhs, hk)
    np1 = n + 1
    T = vp.reshape(np1, np1, np1, 3)[:n, :n, :n].astype(np.float32) * s_t
    O = np.asarray(out, np.float32).reshape(n, n, n, 16)
    d = np.zeros((n, n, n, 16), np.float64)
    d[1:, 1:, 1:, :3] = O[1:, 1:, 1:, :3].astype(np.float64) - T[1:, 1:, 1:].astype(np.float64)
    energy = float((T[1:, 1:, 1:].astype(np.float64) ** 2).sum())
    g = torch.from_numpy(d * (2.0 / energy))
    return _rb(g).numpy().reshape(-1, 16)
