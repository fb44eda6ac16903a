"""Differentiable band-sharpness path: the hand-written kernels (NLPAR average with the weights'
derivatives through lambda, the pair distances and the noise sigma; reflect-padded Gaussian
background blur with its adjoint and d/dsigma; Radon back-projection; LoG adjoint; soft-argmax
objective) against

* an independent float64 torch-autograd reference of the same objective in which every
  dependence is live -- NLPAR weights from the patterns' own pair distances, the noise sigma
  from the patterns' own 3x3 neighbourhoods (torch.min), dense Radon / LoG matrices -- and
* central finite differences of that reference (h = 1e-3), nothing held fixed.

Bars: relative error <= 1e-4 for d/dlambda, d/d(background sigma) and for d/dx with the
kernels in float64; with the kernels in float32, <= 1e-4 for the two scalars and <= 1e-3 in
norm for d/dx (float32 accumulation through the softmax and the adjoints).
"""
import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import diff, synthetic as syn

pytestmark = pytest.mark.gpu

NR, NC, H, W = 6, 6, 40, 40
SR, LAM, BGS, TAU = 2, 0.9, 3.0, 2.0


def _setup(cuda, dthresh=0.0):
    import torch
    bd = pg.BandDetect(nTheta=90, nRho=60, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=6)
    bd.band_detect_setup(patDim=(H, W), patternmask=syn.circular_mask(H, W))
    pats, _ = syn.voronoi_scan(NR, NC, ngrains=5, h=H, w=W, seed=21, peak_range=(50.0, 50.0))
    x = torch.from_numpy(pats.reshape(NR * NC, H * W).astype(np.float32)).to(cuda)
    obj = diff.BandSharpness(bd, NR, NC, searchradius=SR, tau=TAU, bg_radius=8, dthresh=dthresh)
    return bd, obj, x


def _windows(n_r, n_c, sr):
    from oracle.nlpar_oracle import window_bounds
    winsz = (2 * sr + 1) ** 2
    nbr = np.zeros((n_r * n_c, winsz), dtype=np.int64)
    for j in range(n_r):
        ys, ye = window_bounds(j, sr, n_r)
        for i in range(n_c):
            xs, xe = window_bounds(i, sr, n_c)
            c = 0
            for jn in range(ys, ye):
                for inn in range(xs, xe):
                    nbr[i + n_c * j, c] = inn + n_c * jn
                    c += 1
    return nbr


def _sigma2(x, ind, mxs):
    """Noise sigma^2 of sigma_numba (nn = 1), differentiable: min over the 3x3 neighbours of
    SSD / (2 (n + 1e-12)) for pairs with SSD >= 1e-3 (nlpar_cpu.py:753-796)."""
    import torch
    vals = []
    a = x[:, ind]
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            if dj == 0 and di == 0:
                continue
            nb = np.full(NR * NC, -1, dtype=np.int64)
            for j in range(NR):
                for i in range(NC):
                    jn, inn = j + dj, i + di
                    if 0 <= jn < NR and 0 <= inn < NC:
                        nb[i + NC * j] = inn + NC * jn
            nbt = torch.as_tensor(np.maximum(nb, 0), device=x.device)
            b = x[nbt][:, ind]
            ok = (a < mxs) & (b < mxs)
            d2 = (((a - b) ** 2) * ok).sum(-1)
            n2 = ok.sum(-1).to(x.dtype) + 1e-12
            good = torch.as_tensor(nb >= 0, device=x.device) & (d2 >= 1e-3)
            vals.append(torch.where(good, d2 / (2.0 * n2), torch.full_like(d2, 1e24)))
    return torch.stack(vals, 1).min(1).values


def _reference(obj, x, lam, bgs, sigma2=None, dthresh=0.0):
    """float64 torch autograd of the objective, every dependence live (weights and sigma from x)."""
    import torch
    import torch.nn.functional as F
    n = NR * NC
    ind = obj.ind.long()
    mx = x.detach().max()
    s2 = _sigma2(x, ind, mx * 0.9961) if sigma2 is None else sigma2
    nbr = torch.as_tensor(_windows(NR, NC, SR), device=x.device)
    a = x[:, ind].unsqueeze(1)
    b = x[nbr][:, :, ind]
    ok = (a < mx * 0.999) & (b < mx * 0.999)
    d2 = (((a - b) ** 2) * ok).sum(-1)
    n2 = ok.sum(-1).to(torch.float64)
    ss = s2.unsqueeze(1) + s2[nbr]
    d = (d2 - n2 * ss) / (ss * torch.sqrt(2.0 * n2))
    centre = nbr == torch.arange(n, device=x.device).unsqueeze(1)
    m = torch.where(centre, torch.zeros_like(d), torch.clamp(d - dthresh, min=0.0))
    e = torch.exp(-m / lam ** 2)
    w = e / e.sum(1, keepdim=True)
    y = (w.unsqueeze(-1) * x[nbr]).sum(1)
    img = y.reshape(n, 1, H, W)
    t = torch.arange(-obj.bg_radius, obj.bg_radius + 1, dtype=torch.float64, device=x.device)
    k = torch.exp(-0.5 * (t / bgs) ** 2)
    k = k / k.sum()
    r0 = obj.bg_radius
    pad = F.pad(img, (r0, r0, r0, r0), mode="reflect")
    blur = F.conv2d(F.conv2d(pad, k.reshape(1, 1, 1, -1)), k.reshape(1, 1, -1, 1))
    z = (img - blur).reshape(n, H * W)
    R = torch.as_tensor(obj.R.dense(), device=x.device)
    M = torch.as_tensor(obj.M.dense(), device=x.device)
    c = (z @ R.T) @ M.T
    cm = c[:, obj.rmask.bool()]
    s = torch.softmax(cm / TAU, dim=1)
    return (s * cm).sum(1).mean()


def _rel(a, b):
    return abs(float(a) - float(b)) / max(abs(float(b)), 1e-30)


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_gradients_match_fp64_autograd(cuda, dtype):
    import torch
    dt = getattr(torch, dtype)
    bd, obj, x = _setup(cuda)
    xg = x.to(dt).clone().requires_grad_(True)
    lam = torch.tensor(LAM, dtype=dt, device=cuda, requires_grad=True)
    bgs = torch.tensor(BGS, dtype=dt, device=cuda, requires_grad=True)
    J = obj(xg, lam, bgs)
    J.backward()
    x64 = x.to(torch.float64).clone().requires_grad_(True)
    lam64 = torch.tensor(LAM, dtype=torch.float64, device=cuda, requires_grad=True)
    bgs64 = torch.tensor(BGS, dtype=torch.float64, device=cuda, requires_grad=True)
    J64 = _reference(obj, x64, lam64, bgs64)
    J64.backward()
    print(dtype, float(J), float(J64), float(lam.grad), float(lam64.grad), float(bgs.grad), float(bgs64.grad))
    assert _rel(J.detach(), J64.detach()) <= 1e-4
    assert _rel(lam.grad, lam64.grad) <= 1e-4, (float(lam.grad), float(lam64.grad))
    assert _rel(bgs.grad, bgs64.grad) <= 1e-4, (float(bgs.grad), float(bgs64.grad))
    gx, gx64 = xg.grad.to(torch.float64), x64.grad
    err = float((gx - gx64).norm() / gx64.norm())
    print(dtype, "dJ/dx relative error", err)
    assert err <= (1e-4 if dtype == "float64" else 1e-3)
    # the weights' dependence on the patterns is a real part of dJ/dx, not a rounding-level one
    xs = x.to(torch.float64).clone().requires_grad_(True)
    _reference(obj, xs, lam64.detach(), bgs64.detach(), sigma2=_sigma2(xs.detach(), obj.ind.long(),
                                                                         xs.detach().max() * 0.9961)).backward()
    assert float((xs.grad - gx64).norm() / gx64.norm()) > 1e-3


def test_gradients_match_finite_differences(cuda):
    """Central differences (h = 1e-3) of the float64 reference with every dependence live,
    against the float64 kernels: lambda, background sigma, and x along the gradient."""
    import torch
    bd, obj, x = _setup(cuda)
    x64 = x.to(torch.float64)
    xg = x64.clone().requires_grad_(True)
    lam = torch.tensor(LAM, dtype=torch.float64, device=cuda, requires_grad=True)
    bgs = torch.tensor(BGS, dtype=torch.float64, device=cuda, requires_grad=True)
    obj(xg, lam, bgs).backward()
    h = 1e-3
    with torch.no_grad():
        f = lambda l, s, xx: float(_reference(obj, xx, torch.tensor(l, dtype=torch.float64, device=cuda),
                                              torch.tensor(s, dtype=torch.float64, device=cuda)))
        fd_lam = (f(LAM + h, BGS, x64) - f(LAM - h, BGS, x64)) / (2 * h)
        fd_bgs = (f(LAM, BGS + h, x64) - f(LAM, BGS - h, x64)) / (2 * h)
        u = xg.grad / xg.grad.norm()
        fd_x = (f(LAM, BGS, x64 + h * u) - f(LAM, BGS, x64 - h * u)) / (2 * h)
    print("fd", float(lam.grad), fd_lam, float(bgs.grad), fd_bgs, float((xg.grad * u).sum()), fd_x)
    assert _rel(lam.grad, fd_lam) <= 1e-4, (float(lam.grad), fd_lam)
    assert _rel(bgs.grad, fd_bgs) <= 1e-4, (float(bgs.grad), fd_bgs)
    assert _rel((xg.grad * u).sum(), fd_x) <= 1e-4, (float((xg.grad * u).sum()), fd_x)


def test_held_sigma_matches_reference_with_fixed_sigma(cuda):
    """A given noise sigma is held fixed: the kernels then match the reference with that sigma.
    With a distance threshold of 0.5: pairs of one grain have normalised distances near 0, at
    the max(d - dthresh, 0) kink, where the gradient jumps with the last bit of sigma (the
    reference itself moves by ~10% between sigma in float32 and in float64 there)."""
    import torch
    bd, obj, x = _setup(cuda, dthresh=0.5)
    sigma = obj.sigma_of(x)
    xg = x.to(torch.float64).clone().requires_grad_(True)
    lam = torch.tensor(LAM, dtype=torch.float64, device=cuda, requires_grad=True)
    bgs = torch.tensor(BGS, dtype=torch.float64, device=cuda, requires_grad=True)
    obj(xg, lam, bgs, sigma=sigma).backward()
    x64 = x.to(torch.float64).clone().requires_grad_(True)
    s2 = sigma.to(torch.float64) ** 2
    _reference(obj, x64, lam.detach(), bgs.detach(), sigma2=s2, dthresh=0.5).backward()
    assert float((xg.grad - x64.grad).norm() / x64.grad.norm()) <= 1e-4


def test_kernels_individually(cuda):
    """The blur adjoint is the transpose of the blur; the soft-argmax value and gradient equal
    torch's; the sigma kernel's sigma^2 equals the NLPAR sigma kernel's squared."""
    import torch
    bd, obj, x = _setup(cuda)
    lib = diff._bind()
    g = torch.Generator(device="cuda").manual_seed(3)
    for r, hh, ww in ((8, H, W), (3, 17, 23)):
        k, dk = diff.gaussian_taps(torch.tensor(2.5, dtype=torch.float64, device=cuda), r)
        v = torch.randn((3, hh * ww), dtype=torch.float64, device=cuda, generator=g)
        u = torch.randn((3, hh * ww), dtype=torch.float64, device=cuda, generator=g)
        for axis in (0, 1):
            bu = diff._blur(lib, u, k, r, hh, ww, axis)
            btv = diff._blur(lib, v, k, r, hh, ww, axis, adjoint=True)
            assert abs(float((bu * v).sum() - (u * btv).sum())) <= 1e-10 * float((bu * v).abs().sum())
        import torch.nn.functional as F
        ref = F.conv2d(F.conv2d(F.pad(u.reshape(3, 1, hh, ww), (r, r, r, r), mode="reflect"), k.reshape(1, 1, 1, -1)),
                       k.reshape(1, 1, -1, 1)).reshape(3, -1)
        got = diff._blur(lib, diff._blur(lib, u, k, r, hh, ww, 1), k, r, hh, ww, 0)
        assert float((got - ref).abs().max()) <= 1e-12
    c = torch.randn((5, obj.M.shape[0]), dtype=torch.float64, device=cuda, generator=g).requires_grad_(True)
    J = diff._softargmax_fn().apply(c, obj.cells, TAU)
    J.backward()
    cr = c.detach().clone().requires_grad_(True)
    cm = cr[:, obj.rmask.bool()]
    Jr = (torch.softmax(cm / TAU, 1) * cm).sum(1).mean()
    Jr.backward()
    assert _rel(J, Jr) <= 1e-12 and float((c.grad - cr.grad).abs().max()) <= 1e-12
    sig = obj.sigma_of(x)
    npix = NR * NC
    sig2 = torch.empty(npix, dtype=torch.float32, device=cuda)
    arg = torch.empty(npix, dtype=torch.int32, device=cuda)
    nsig = torch.empty(npix, dtype=torch.float32, device=cuda)
    import ctypes as C  # noqa: F401
    from pyebsdindex_gb300 import _lib
    _lib.check(lib.ebsd_nlpar_sigma_arg(x.data_ptr(), NR, NC, H * W, obj.ind.data_ptr(), obj.ind.numel(),
                                        float(x.max()), 1, sig2.data_ptr(), arg.data_ptr(), nsig.data_ptr(), 0))
    torch.cuda.synchronize()
    assert torch.equal(sig2, sig * sig)
    assert int((arg >= 0).sum()) == npix


def test_radon_adjoint_is_the_transpose_on_device(cuda):
    """<R x, g> == <x, R^T g> and <M r, g> == <r, M^T g> with the device kernels (float64)."""
    import torch
    bd, obj, x = _setup(cuda)
    g = torch.randn((3, obj.R.shape[0]), dtype=torch.float64, device=cuda)
    xx = torch.randn((3, obj.R.shape[1]), dtype=torch.float64, device=cuda)
    lhs = (obj.R(xx) * g).sum()
    rhs = (xx * obj.RT(g)).sum()
    assert abs(float(lhs - rhs)) <= 1e-10 * abs(float(lhs))
    r = torch.randn((3, obj.M.shape[1]), dtype=torch.float64, device=cuda)
    lhs = (obj.M(r) * g).sum()
    rhs = (r * obj.MT(g)).sum()
    assert abs(float(lhs - rhs)) <= 1e-10 * abs(float(lhs))


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_pattern_minor_operator_equals_pattern_major(cuda, dtype):
    """The sparse Radon / LoG operators with the patterns along the fast axis (what the
    objective runs) give the pattern-major kernel's products bit for bit, for a batch that is
    not a multiple of 32, a contiguous input and another operator's transposed output."""
    import torch
    _, obj, x = _setup(cuda)
    td = getattr(torch, dtype)
    g = torch.Generator(device="cpu").manual_seed(5)
    xb = torch.rand((45, x.shape[1]), generator=g, dtype=td).to(cuda) * 100.0
    for op in (obj.R, obj.RT):
        xin = xb if op is obj.R else torch.rand((45, obj.R.shape[0]), generator=g, dtype=td).to(cuda)
        a = op(xin)
        b = op.apply_rows(xin)
        assert a.shape == b.shape and torch.equal(a, b), op.shape
    r = obj.R(xb)  # a transposed view, read in place by the next operator
    assert not r.is_contiguous() and r.t().is_contiguous()
    assert torch.equal(obj.M(r), obj.M.apply_rows(r.contiguous()))
