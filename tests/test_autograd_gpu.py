"""GPU: gradients of the differentiable path (hand-written adjoints behind a
torch.autograd.Function) against (a) a torch-op-composed FP64 reference of
the same formulas (grid_sample bilinear/zeros for rotate, separable conv2d
for the zero-padded gaussian) and (b) FP64 central finite differences of the
oracle on small crops."""
import math

import numpy as np
import pytest

from oracle import oracle as O

from helpers import TOL

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
F = torch.nn.functional


def mp_pipeline(*a, **k):
    from millipyde_gb300.autograd import pipeline
    return pipeline(*a, **k)


# ------------------------------------------------------------ torch reference
def _interior(t):
    """clamp01 with gradient only strictly inside (0, 1)."""
    return torch.where((t > 0) & (t < 1), t, t.clamp(0, 1).detach())


def ref_rotate(x, theta):
    B, H, W, C = x.shape
    th = theta.reshape(-1, 1, 1) * O.DEG2RAD
    ys, xs = torch.meshgrid(torch.arange(H, dtype=x.dtype, device=x.device),
                            torch.arange(W, dtype=x.dtype, device=x.device), indexing="ij")
    dx, dy = xs - W / 2.0, ys - H / 2.0
    c, s = torch.cos(th), torch.sin(th)
    sx = c * dx - s * dy + W / 2.0
    sy = s * dx + c * dy + H / 2.0
    grid = torch.stack([2 * sx / (W - 1) - 1, 2 * sy / (H - 1) - 1], dim=-1)
    out = F.grid_sample(x.permute(0, 3, 1, 2), grid, mode="bilinear", padding_mode="zeros",
                        align_corners=True)
    return out.permute(0, 2, 3, 1)


def ref_gaussian(x, sigma):
    outs = []
    B, H, W, C = x.shape
    for b in range(B):
        sg = sigma.reshape(-1)[b] if sigma.numel() > 1 else sigma.reshape(-1)[0]
        r = int(math.ceil(3.0 * float(sg)))
        k = torch.arange(-r, r + 1, dtype=x.dtype, device=x.device)
        w = torch.exp(-(k * k) / (2 * sg * sg))
        w = w / w.sum()
        xb = x[b:b + 1].permute(0, 3, 1, 2)
        xb = F.conv2d(xb, w.view(1, 1, -1, 1).expand(C, 1, -1, 1), padding=(r, 0), groups=C)
        xb = F.conv2d(xb, w.view(1, 1, 1, -1).expand(C, 1, 1, -1), padding=(0, r), groups=C)
        outs.append(xb.permute(0, 2, 3, 1))
    return torch.cat(outs, 0)


def ref_gamma(x, gamma, gain=1.0):
    g = gamma.reshape(-1, 1, 1, 1)
    col = x[..., :3] if x.shape[-1] == 4 else x
    safe = torch.where(col > 0, col, torch.ones_like(col))
    t = torch.where(col > 0, gain * safe ** g, torch.zeros_like(col))
    y = _interior(t)
    return torch.cat([y, x[..., 3:]], -1) if x.shape[-1] == 4 else y


def ref_brightness(x, delta):
    d = delta.reshape(-1, 1, 1, 1)
    return _interior(x + d)


def ref_grey(x):
    s = 0.2125 * x[..., 0] + 0.7154 * x[..., 1] + 0.0721 * x[..., 2]
    return torch.where(s < 1, s, torch.ones_like(s))


def rel(a, b):
    a, b = a.double(), b.double()
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


# ------------------------------------------------------------------ tests
def test_config4_chain_vs_torch_reference(gpu):
    """rotate -> gaussian -> adjust_gamma -> rgb2grey, loss = sum(out * W)."""
    torch.manual_seed(0)
    B, H, W = 6, 96, 112
    x = torch.rand(B, H, W, 3, device="cuda")
    theta = (torch.rand(B, device="cuda", dtype=torch.float64) * 60 - 30).requires_grad_()
    sigma = (1 + 2 * torch.rand(B, device="cuda", dtype=torch.float64)).requires_grad_()
    gamma = (0.7 + 0.8 * torch.rand(B, device="cuda", dtype=torch.float64)).requires_grad_()
    Wt = torch.randn(B, H, W, device="cuda")
    xg = x.clone().requires_grad_()
    y = mp_pipeline(xg, [("rotate", theta), ("gaussian", sigma), ("adjust_gamma", gamma), ("rgb2grey",)])
    (y * Wt).sum().backward()

    x64 = x.double().clone().requires_grad_()
    th2, sg2, gm2 = (t.detach().clone().requires_grad_() for t in (theta, sigma, gamma))
    y64 = ref_grey(ref_gamma(ref_gaussian(ref_rotate(x64, th2), sg2), gm2))
    (y64 * Wt.double()).sum().backward()

    assert float((y.double() - y64).abs().max()) <= TOL
    assert rel(xg.grad, x64.grad) < 2e-4
    assert rel(theta.grad, th2.grad) < 2e-3
    assert rel(sigma.grad, sg2.grad) < 2e-3
    assert rel(gamma.grad, gm2.grad) < 2e-3


def test_config5_chain_vs_torch_reference(gpu):
    """gaussian(sigma 8, radius 24) -> rotate -> brightness, recomputed backward."""
    torch.manual_seed(1)
    B, H, W = 2, 160, 144
    x = torch.rand(B, H, W, 3, device="cuda")
    theta = (torch.rand(B, device="cuda", dtype=torch.float64) * 90 - 45).requires_grad_()
    delta = (torch.rand(B, device="cuda", dtype=torch.float64) * 0.2 - 0.1).requires_grad_()
    Wt = torch.randn(B, H, W, 3, device="cuda")
    xg = x.clone().requires_grad_()
    y = mp_pipeline(xg, [("gaussian", 8.0), ("rotate", theta), ("brightness", delta)])
    (y * Wt).sum().backward()
    x64 = x.double().clone().requires_grad_()
    th2, dl2 = theta.detach().clone().requires_grad_(), delta.detach().clone().requires_grad_()
    s8 = torch.tensor(8.0, dtype=torch.float64, device="cuda")
    y64 = ref_brightness(ref_rotate(ref_gaussian(x64, s8), th2), dl2)
    (y64 * Wt.double()).sum().backward()
    assert float((y.double() - y64).abs().max()) <= TOL
    assert rel(xg.grad, x64.grad) < 2e-4
    assert rel(theta.grad, th2.grad) < 2e-3
    assert rel(delta.grad, dl2.grad) < 2e-3


@pytest.mark.parametrize("C", [1, 3, 4])
def test_sigma_gradient_every_channel_count(gpu, C):
    """d sigma and dx of a lone gaussian on 1-, 3- and 4-channel batches:
    radii 3, 6, 11, 12 (the streaming kernels' dot mode), then a batch with
    radius 14 in it (the tile kernel's dot mode for the whole launch)."""
    torch.manual_seed(3 + C)
    B, H, W = 4, 40, 52
    for sigmas in ((0.7, 1.9, 3.6, 3.9), (4.6, 1.0, 2.0, 3.0)):
        x = torch.rand(B, H, W, C, device="cuda")
        sigma = torch.tensor(sigmas, dtype=torch.float64, device="cuda").requires_grad_()
        Wt = torch.randn(B, H, W, C, device="cuda")
        xg = x.clone().requires_grad_()
        y = mp_pipeline(xg, [("gaussian", sigma)])
        y = y.reshape(B, H, W, C)
        (y * Wt).sum().backward()
        x64 = x.double().clone().requires_grad_()
        sg2 = sigma.detach().clone().requires_grad_()
        y64 = ref_gaussian(x64, sg2)
        (y64 * Wt.double()).sum().backward()
        assert float((y.double() - y64).abs().max()) <= TOL
        assert rel(xg.grad, x64.grad) < 2e-4
        assert rel(sigma.grad, sg2.grad) < 2e-3


def test_pointwise_params_and_permutations(gpu):
    torch.manual_seed(2)
    B, H, W = 3, 40, 56
    x = torch.rand(B, H, W, 4, device="cuda")
    gain = torch.full((B,), 1.1, device="cuda", dtype=torch.float64, requires_grad=True)
    gm = torch.full((B,), 1.7, device="cuda", dtype=torch.float64, requires_grad=True)
    xg = x.clone().requires_grad_()
    y = mp_pipeline(xg, [("fliplr",), ("adjust_gamma", gm, gain), ("transpose",), ("brightness", 0.05)])
    Wt = torch.randn_like(y)
    (y * Wt).sum().backward()
    x64 = x.double().clone().requires_grad_()
    g2, k2 = gm.detach().clone().requires_grad_(), gain.detach().clone().requires_grad_()
    t = torch.flip(x64, dims=[2])
    t = ref_gamma(t, g2, k2.reshape(-1, 1, 1, 1))
    t = t.transpose(1, 2)
    col = _interior(t[..., :3] + 0.05)
    y64 = torch.cat([col, t[..., 3:]], -1)
    (y64 * Wt.double()).sum().backward()
    assert float((y.double() - y64).abs().max()) <= TOL
    assert rel(xg.grad, x64.grad) < 2e-4
    assert rel(gm.grad, g2.grad) < 2e-3
    assert rel(gain.grad, k2.grad) < 2e-3


def _oracle_loss(x, theta, sigma, gamma, Wt):
    y = O.rgb2grey(O.adjust_gamma(O.gaussian(O.rotate(x, theta), sigma), gamma))
    return float(np.sum(y * Wt))


def test_finite_differences_on_crop(gpu):
    """FP64 central differences of the oracle on a 64x64 crop."""
    rng = np.random.default_rng(3)
    x = rng.random((64, 64, 3)).astype(np.float32).astype(np.float64)
    Wt = rng.standard_normal((64, 64))
    theta, sigma, gamma = 12.3, 1.7, 1.25
    xt = torch.tensor(x[None], dtype=torch.float32, device="cuda", requires_grad=True)
    th = torch.tensor([theta], dtype=torch.float64, device="cuda", requires_grad=True)
    sg = torch.tensor([sigma], dtype=torch.float64, device="cuda", requires_grad=True)
    gm = torch.tensor([gamma], dtype=torch.float64, device="cuda", requires_grad=True)
    y = mp_pipeline(xt, [("rotate", th), ("gaussian", sg), ("adjust_gamma", gm), ("rgb2grey",)])
    (y * torch.tensor(Wt[None], dtype=torch.float32, device="cuda")).sum().backward()
    for name, val, g, h in (("theta", theta, th.grad, 1e-4), ("sigma", sigma, sg.grad, 1e-5),
                            ("gamma", gamma, gm.grad, 1e-5)):
        args = dict(theta=theta, sigma=sigma, gamma=gamma)
        args[name] = val + h
        lp = _oracle_loss(x, Wt=Wt, **args)
        args[name] = val - h
        lm = _oracle_loss(x, Wt=Wt, **args)
        fd = (lp - lm) / (2 * h)
        assert abs(float(g) - fd) <= 2e-3 * max(1.0, abs(fd)), (name, float(g), fd)
    gx = xt.grad[0].double().cpu().numpy()
    for (i, j, c) in [(10, 20, 0), (32, 32, 1), (50, 7, 2), (0, 0, 0)]:
        h = 1e-5
        xp, xm = x.copy(), x.copy()
        xp[i, j, c] += h
        xm[i, j, c] -= h
        fd = (_oracle_loss(xp, theta, sigma, gamma, Wt) - _oracle_loss(xm, theta, sigma, gamma, Wt)) / (2 * h)
        assert abs(gx[i, j, c] - fd) <= 1e-4 + 2e-3 * abs(fd), ((i, j, c), gx[i, j, c], fd)


def test_rotate_adjoint_is_transpose(gpu):
    """<R x, g> == <x, R^T g> for the library's own kernels."""
    torch.manual_seed(4)
    x = torch.rand(2, 50, 70, 3, device="cuda", requires_grad=True)
    th = torch.tensor([33.3, -71.0], device="cuda", dtype=torch.float64)
    y = mp_pipeline(x, [("rotate", th)])
    g = torch.randn_like(y)
    (gx,) = torch.autograd.grad((y * g).sum(), x)
    lhs = float((y.double() * g.double()).sum())
    rhs = float((x.detach().double() * gx.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs) + 1e-3


def test_channels_first_input(gpu):
    torch.manual_seed(5)
    x = torch.rand(2, 3, 32, 40, device="cuda", requires_grad=True)
    y = mp_pipeline(x, [("gaussian", 1.5), ("rgb2grey",)], channels_first=True)
    assert y.shape == (2, 32, 40)
    y.sum().backward()
    assert x.grad.shape == x.shape and torch.isfinite(x.grad).all()


@pytest.mark.parametrize("chain", [
    [("rotate", (-30, 30)), ("gaussian", (1.0, 3.0)), ("adjust_gamma", (0.7, 1.5)), ("rgb2grey", None)],
    [("gaussian", (2.0, 2.0)), ("rotate", (-45, 45)), ("brightness", (-0.1, 0.1))],
    [("rgb2grey", None), ("gaussian", (0.8, 1.6)), ("transpose", None), ("rotate", (-20, 20)),
     ("brightness", (-0.2, 0.2)), ("fliplr", None)],
    [("rotate", (5, 15)), ("rotate", (-40, -10)), ("gaussian", (0.5, 2.5)), ("adjust_gamma", (0.6, 1.4))],
    [("rotate", (-30, 30)), ("adjust_gamma", (0.6, 1.4)), ("brightness", (-0.3, 0.3))],
    [("transpose", None), ("gaussian", (1.0, 2.0)), ("brightness", (-0.4, 0.4))],
])
def test_saved_intermediates_match_recompute(gpu, chain):
    """The backward reading the forward's saved intermediates (and, for a
    final lone brightness, the output) gives the gradients of the backward
    that recomputes every intermediate."""
    import ctypes as C
    from millipyde_gb300 import _abi
    L = _abi.lib()
    codes = {"rotate": _abi.OP_ROTATE, "gaussian": _abi.OP_GAUSSIAN, "adjust_gamma": _abi.OP_ADJUST_GAMMA,
             "rgb2grey": _abi.OP_RGB2GREY, "brightness": _abi.OP_BRIGHTNESS, "transpose": _abi.OP_TRANSPOSE,
             "fliplr": _abi.OP_FLIPLR}
    rng = np.random.default_rng(len(chain))
    B, H, W, Cc = 5, 72, 88, 3
    nops = len(chain)
    ops = (C.c_int * nops)(*[codes[n] for n, _ in chain])
    P = np.zeros((B, nops, 3), np.float64)
    for k, (n, rg) in enumerate(chain):
        if rg is not None:
            P[:, k, 0] = rng.uniform(rg[0], rg[1], B)
        if n == "adjust_gamma":
            P[:, k, 1] = 1.0
    ho, wo, co = C.c_int(), C.c_int(), C.c_int()
    _abi.check(L.mpk_chain_shape(ops, nops, H, W, Cc, C.byref(ho), C.byref(wo), C.byref(co)))
    x = torch.rand(B, H, W, Cc, device="cuda")
    y = torch.empty(B, ho.value, wo.value, co.value, device="cuda")
    gy = torch.randn_like(y)
    cnt, nbytes = C.c_int(), C.c_size_t()
    idx, off = (C.c_int * nops)(), (C.c_size_t * nops)()
    _abi.check(L.mpk_chain_saved_layout(ops, nops, B, H, W, Cc, C.byref(cnt), idx, off, C.byref(nbytes)))
    assert (cnt.value == 0) == (nbytes.value == 0)
    saved = torch.full((max(1, nbytes.value // 4),), float("nan"), device="cuda")
    sp = saved.data_ptr() if nbytes.value else None
    stream = torch.cuda.current_stream().cuda_stream
    pp = P.ctypes.data
    _abi.check(L.mpk_chain_forward_saved(ops, nops, pp, x.data_ptr(), y.data_ptr(), sp, B, H, W, Cc, stream))
    mask = (C.c_int * nops)(*([1] * nops))
    res = []
    for use_saved in (True, False):
        dx = torch.empty_like(x)
        dP = torch.zeros(B, nops, 3, dtype=torch.float64, device="cuda")
        # the saved variant also hands over y (a final lone brightness
        # back-propagates from it); the reference recomputes everything
        _abi.check(L.mpk_chain_backward_saved(ops, nops, pp, x.data_ptr(),
                                              sp if use_saved else None,
                                              y.data_ptr() if use_saved else None, gy.data_ptr(),
                                              dx.data_ptr(), dP.data_ptr(), mask, B, H, W, Cc, stream))
        torch.cuda.synchronize()
        res.append((dx, dP))
    (dx1, dp1), (dx0, dp0) = res
    if nbytes.value:
        assert not torch.isnan(saved).any()      # every saved intermediate was written
    assert rel(dx1, dx0) <= 1e-5
    assert rel(dp1, dp0) <= 1e-5
    # and the forward with a saved block writes the same output as without
    y0 = torch.empty_like(y)
    _abi.check(L.mpk_chain_forward(ops, nops, pp, x.data_ptr(), y0.data_ptr(), B, H, W, Cc, stream))
    torch.cuda.synchronize()
    assert float((y0 - y).abs().max()) <= TOL
