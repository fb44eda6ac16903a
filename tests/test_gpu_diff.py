"""Differentiable band-sharpness path: gradients from the hand-written adjoint kernels (Radon
back-projection, LoG adjoint, NLPAR W^T g and lambda derivative) against

* an independent float64 torch-autograd reference of the same objective (NLPAR weights from
  the same distance formula in float64, dense Radon / LoG matrices), and
* central finite differences of that float64 reference (h = 1e-3).

Bar: relative error <= 1e-4 for d/dlambda and d/dsigma; for d/dx <= 1e-4 in norm with the
adjoints in float64 and <= 1e-3 with them in float32.
"""
import numpy as np
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import diff, synthetic as syn

pytestmark = pytest.mark.gpu

NR, NC, H, W = 6, 6, 40, 40
SR, LAM, BGS, TAU = 2, 0.9, 3.0, 2.0


def _setup(cuda):
    import torch
    bd = pg.BandDetect(nTheta=90, nRho=60, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=6)
    bd.band_detect_setup(patDim=(H, W), patternmask=syn.circular_mask(H, W))
    pats, _ = syn.voronoi_scan(NR, NC, ngrains=5, h=H, w=W, seed=21, peak_range=(50.0, 50.0))
    x = torch.from_numpy(pats.reshape(NR * NC, H * W).astype(np.float32)).to(cuda)
    obj = diff.BandSharpness(bd, NR, NC, searchradius=SR, tau=TAU, bg_radius=8)
    return bd, obj, x


def _reference(obj, x64, lam, bgs, sigma64, xw=None):
    """float64 torch autograd of the same objective; the NLPAR weights come from ``xw``
    (default: the input itself, detached), as in the device path."""
    import torch
    import torch.nn.functional as F
    n = NR * NC
    ind = obj.ind.long()
    xd = (x64 if xw is None else xw).detach()
    mx = xd.max() * 0.999
    winsz = (2 * SR + 1) ** 2
    nbr = np.zeros((n, winsz), dtype=np.int64)
    from oracle.nlpar_oracle import window_bounds
    for j in range(NR):
        ys, ye = window_bounds(j, SR, NR)
        for i in range(NC):
            xs, xe = window_bounds(i, SR, NC)
            c = 0
            for jn in range(ys, ye):
                for inn in range(xs, xe):
                    nbr[i + NC * j, c] = inn + NC * jn
                    c += 1
    nbr = torch.as_tensor(nbr, device=x64.device)
    a = xd[:, ind].unsqueeze(1)
    b = xd[nbr][:, :, ind]
    ok = (a < mx) & (b < mx)
    d2 = (((a - b) ** 2) * ok).sum(-1)
    n2 = ok.sum(-1).to(torch.float64)
    s2 = sigma64 ** 2
    ss = s2.unsqueeze(1) + s2[nbr]
    d = (d2 - n2 * ss) / (ss * torch.sqrt(2.0 * n2))
    centre = nbr == torch.arange(n, device=x64.device).unsqueeze(1)
    m = torch.where(centre, torch.zeros_like(d), torch.clamp(d, min=0.0))
    e = torch.exp(-m / lam ** 2)
    w = e / e.sum(1, keepdim=True)
    y = (w.unsqueeze(-1) * x64[nbr]).sum(1)
    img = y.reshape(n, 1, H, W)
    t = torch.arange(-obj.bg_radius, obj.bg_radius + 1, dtype=torch.float64, device=x64.device)
    k = torch.exp(-0.5 * (t / bgs) ** 2)
    k = k / k.sum()
    r0 = obj.bg_radius
    pad = F.pad(img, (r0, r0, r0, r0), mode="reflect")
    blur = F.conv2d(F.conv2d(pad, k.reshape(1, 1, 1, -1)), k.reshape(1, 1, -1, 1))
    z = (img - blur).reshape(n, H * W)
    R = torch.as_tensor(obj.R.dense(), device=x64.device)
    M = torch.as_tensor(obj.M.dense(), device=x64.device)
    c = (z @ R.T) @ M.T
    cm = c[:, obj.rmask.bool()]
    s = torch.softmax(cm / TAU, dim=1)
    return (s * cm).sum(1).mean()


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_gradients_match_fp64_autograd_and_finite_differences(cuda, dtype):
    """float64: the adjoint kernels in double precision must match autograd and finite
    differences to 1e-4 (they do to ~1e-7).  float32: the same kernels in single precision;
    lambda / sigma gradients within 1e-4, the pattern gradient within 1e-3 in norm (float32
    accumulation through the softmax, Radon and LoG adjoints)."""
    import torch
    dt = getattr(torch, dtype)
    bd, obj, x = _setup(cuda)
    sigma = obj.sigma_of(x)
    xg = x.to(dt).clone().requires_grad_(True)
    lam = torch.tensor(LAM, dtype=dt, device=cuda, requires_grad=True)
    bgs = torch.tensor(BGS, dtype=dt, device=cuda, requires_grad=True)
    J = obj(xg, lam, bgs, sigma=sigma)
    J.backward()

    x64 = x.to(torch.float64).clone().requires_grad_(True)
    lam64 = torch.tensor(LAM, dtype=torch.float64, device=cuda, requires_grad=True)
    bgs64 = torch.tensor(BGS, dtype=torch.float64, device=cuda, requires_grad=True)
    s64 = sigma.to(torch.float64)
    J64 = _reference(obj, x64, lam64, bgs64, s64)
    J64.backward()

    rel = lambda a, b: abs(float(a) - float(b)) / max(abs(float(b)), 1e-30)
    assert rel(J.detach(), J64.detach()) <= 1e-4
    assert rel(lam.grad, lam64.grad) <= 1e-4, (float(lam.grad), float(lam64.grad))
    assert rel(bgs.grad, bgs64.grad) <= 1e-4, (float(bgs.grad), float(bgs64.grad))
    gx, gx64 = xg.grad.to(torch.float64), x64.grad
    xtol = 1e-4 if dtype == "float64" else 1e-3
    assert float((gx - gx64).norm() / gx64.norm()) <= xtol

    # central finite differences of the float64 reference, h = 1e-3 (weights held at x0)
    h = 1e-3
    with torch.no_grad():
        x0 = x.to(torch.float64)
        f = lambda l, s, xx: float(_reference(obj, xx, torch.tensor(l, dtype=torch.float64, device=cuda),
                                              torch.tensor(s, dtype=torch.float64, device=cuda), s64, xw=x0))
        fd_lam = (f(LAM + h, BGS, x0) - f(LAM - h, BGS, x0)) / (2 * h)
        fd_bgs = (f(LAM, BGS + h, x0) - f(LAM, BGS - h, x0)) / (2 * h)
        u = gx64 / gx64.norm()  # a direction with a well-conditioned derivative
        fd_x = (f(LAM, BGS, x0 + h * u) - f(LAM, BGS, x0 - h * u)) / (2 * h)
    assert rel(lam.grad, fd_lam) <= 1e-4, (float(lam.grad), fd_lam)
    assert rel(bgs.grad, fd_bgs) <= 1e-4, (float(bgs.grad), fd_bgs)
    assert rel((gx * u).sum(), fd_x) <= xtol, (float((gx * u).sum()), fd_x)


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
