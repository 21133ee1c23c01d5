"""Derivatives of G_loc (dmftgpu_gloc_jvp / dmftgpu_gloc_vjp) through the C ABI: forward mode against central
finite differences of GreenFtn_w, reverse mode against forward mode (adjoint identity), and a
torch.autograd.Function built on them (test harness only) whose gradient of ||G_loc - G_imp||^2 with respect
to self-energy parameters and mu is checked against central finite differences (h = 1e-6)."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu


def _setup(ctx, name):
    import torch
    dev = torch.device("cuda:0")
    if name == "soc56":
        wl = models.soc56(k=2, nfreq=32, beta=10.0)
    elif name == "t2g_p":
        wl = models.t2g_p(k=3, nfreq=48, beta=10.0)
    else:
        wl = models.hubbard_2d(kx=6, ky=6, nfreq=48, beta=10.0)
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, wl.D)
    S = torch.from_numpy(wl.sigma).to(dev)
    return wl, Hd, lat, S, dev


def _gloc(ctx, lat, Hd, S, mu):
    return ctx.GreenFtn_w(lat, Hd, S, mu, with_gwhf=False)[0].clone()


@pytest.mark.parametrize("name", ["hubbard", "t2g_p", "soc56"])
def test_jvp_matches_central_differences(ctx, name):
    import torch
    wl, Hd, lat, S, dev = _setup(ctx, name)
    rng = np.random.default_rng(3)
    X = rng.normal(size=wl.sigma.shape) + 1j * rng.normal(size=wl.sigma.shape)
    Sd = torch.from_numpy(0.3 * X).to(dev)
    mu, mud, h = 0.2, 0.7, 1e-6
    jvp = ctx.GreenFtn_w_jvp(lat, Hd, S, mu, Sd, mud)
    fd = (_gloc(ctx, lat, Hd, S + h * Sd, mu + h * mud) - _gloc(ctx, lat, Hd, S - h * Sd, mu - h * mud)) / (2 * h)
    assert rel_err(jvp.cpu().numpy(), fd.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("name", ["t2g_p", "soc56"])
def test_vjp_is_the_adjoint_of_the_jvp(ctx, name):
    """Re <Gbar, J v> = Re <J^H Gbar, Sigma_dot> + mu_bar mu_dot for random cotangents and tangents."""
    import torch
    wl, Hd, lat, S, dev = _setup(ctx, name)
    rng = np.random.default_rng(5)
    shp = wl.sigma.shape
    Gb = torch.from_numpy(rng.normal(size=shp) + 1j * rng.normal(size=shp)).to(dev)
    Sd = torch.from_numpy(rng.normal(size=shp) + 1j * rng.normal(size=shp)).to(dev)
    mu, mud = -0.1, 0.4
    Jv = ctx.GreenFtn_w_jvp(lat, Hd, S, mu, Sd, mud)
    Sb, mub = ctx.GreenFtn_w_vjp(lat, Hd, S, mu, Gb)
    lhs = float(torch.sum(torch.conj(Gb) * Jv).real)
    rhs = float(torch.sum(torch.conj(Sb) * Sd).real) + mub * mud
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1.0)


class _GLoc:
    """torch.autograd.Function over GreenFtn_w (forward) and dmftgpu_gloc_vjp (backward)."""

    @staticmethod
    def make(dctx, lat, Hd):
        import torch

        class F(torch.autograd.Function):
            @staticmethod
            def forward(fctx, S, mu):
                fctx.save_for_backward(S, mu)
                return _gloc(dctx, lat, Hd, S.detach(), float(mu))

            @staticmethod
            def backward(fctx, gbar):
                S, mu = fctx.saved_tensors
                sb, mub = dctx.GreenFtn_w_vjp(lat, Hd, S.detach(), float(mu), gbar.contiguous())
                return sb.contiguous(), torch.tensor(mub, dtype=mu.dtype, device=mu.device)

        return F


def test_autograd_gradient_matches_finite_differences(ctx):
    """d||G_loc - G_imp||^2 / d(a, b, mu) for Sigma = a M0 + b M1/(iw) on the 56-orbital SOC model (dense 20 x 20
    Sigma), reverse mode against central differences with h = 1e-6."""
    import torch
    wl, Hd, lat, S, dev = _setup(ctx, "soc56")
    F = _GLoc.make(ctx, lat, Hd)
    wn = np.pi * (2 * np.arange(wl.nfreq) + 1) / wl.beta
    M0 = torch.from_numpy(wl.extra["M0"]).to(dev)
    M1w = torch.from_numpy(wl.extra["M1"][None] / (1j * wn[:, None, None])).to(dev)
    Gimp = (_gloc(ctx, lat, Hd, 1.1 * M0 + 0.9 * M1w, 0.35) + 0.01).detach()

    def loss(theta):
        Sg = theta[0] * M0 + theta[1] * M1w
        G = F.apply(Sg, theta[2])
        return torch.sum(torch.abs(G - Gimp) ** 2)

    theta = torch.tensor([1.0, 1.0, 0.3], dtype=torch.float64, device=dev, requires_grad=True)
    L = loss(theta)
    L.backward()
    grad = theta.grad.cpu().numpy()
    h = 1e-6
    fd = np.zeros(3)
    with torch.no_grad():
        for i in range(3):
            e = torch.zeros(3, dtype=torch.float64, device=dev)
            e[i] = h
            fd[i] = (float(loss(theta + e)) - float(loss(theta - e))) / (2 * h)
    assert np.allclose(grad, fd, rtol=1e-6, atol=1e-9 * abs(L.item())), (grad, fd)
