"""dmftgpu_greenftn_w_batched: a batch of ragged lattice problems against one dmftgpu_greenftn_w call per problem,
eager, replayed as a CUDA graph (including after the inputs change in place), and with the autotuner."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu


def _problems(ctx, nprob=7):
    import torch
    dev = torch.device("cuda:0")
    wls = models.batched_uneven(nprob=nprob, seed=11, kgrids=(3, 4, 5), nfreqs=(32, 64, 96), beta_range=(5.0, 20.0))
    tcm = lambda t: t.transpose(-1, -2).contiguous()
    probs = []
    for w in wls:
        Hd = ctx.Construct_Hk(w.n, w.rindex, w.hr, w.kgrid, device_out=dev)
        lat = lib.Lattice(w.n, w.nk, w.nfreq, w.beta, 1, w.D)
        S = torch.from_numpy(w.sigma).to(dev)
        probs.append(dict(w=w, lat=lat, H=Hd, Hcm=tcm(Hd), S=S, Scm=tcm(S), mu=0.1 * w.n - 0.2))
    return probs, dev


def _run_batched(ctx, probs, dev, **kw):
    import torch
    D = [p["w"].D for p in probs]
    gw = [torch.zeros((p["w"].nfreq, d, d), dtype=torch.complex128, device=dev) for p, d in zip(probs, D)]
    g0 = [torch.zeros_like(g) for g in gw]
    nm = [torch.zeros((d, d), dtype=torch.complex128, device=dev) for d in D]
    ctx.GreenFtn_w_batched([p["lat"] for p in probs], [p["Hcm"] for p in probs], [p["Scm"] for p in probs],
                           [p["mu"] for p in probs], gw, g0, nm, **kw)
    torch.cuda.synchronize()
    back = lambda t: t.transpose(-1, -2).cpu().numpy()
    return [back(g) for g in gw], [back(g) for g in g0], [back(n) for n in nm]


def _check(ctx, probs, res, mixed=False, tol=1e-12):
    for i, p in enumerate(probs):
        g, g0, nm = ctx.GreenFtn_w(p["lat"], p["H"], p["S"], p["mu"], mixed=mixed)
        assert rel_err(res[0][i], g.cpu().numpy()) < tol, i
        assert rel_err(res[1][i], g0.cpu().numpy()) < tol, i
        assert rel_err(res[2][i], nm.cpu().numpy()) < tol, i


@pytest.mark.parametrize("mixed", [False, True])
def test_batched_matches_single_calls(ctx, mixed):
    probs, dev = _problems(ctx)
    _check(ctx, probs, _run_batched(ctx, probs, dev, mixed=mixed), mixed)


def test_batched_graph_replay_follows_inputs(ctx):
    import torch
    probs, dev = _problems(ctx)
    c2 = lib.Context(0)
    try:
        for _ in range(3):                                  # eager (warm-up), capture, replay
            res = _run_batched(c2, probs, dev, graph=True)
        _check(ctx, probs, res)
        for p in probs:                                     # new Sigma in the same buffers: the replay reads them
            p["Scm"].mul_(1.3)
            p["S"] = p["Scm"].transpose(-1, -2).contiguous()
        res = _run_batched(c2, probs, dev, graph=True)
        _check(ctx, probs, res)
    finally:
        c2.close()
    torch.cuda.synchronize()


def test_batched_autotune(ctx):
    probs, dev = _problems(ctx)
    c2 = lib.Context(0)
    try:
        res = _run_batched(c2, probs, dev, autotune=True)
        _check(ctx, probs, res, tol=1e-11)
        res = _run_batched(c2, probs, dev, autotune=True)  # tuned choices reused
        _check(ctx, probs, res, tol=1e-11)
    finally:
        c2.close()


def test_batched_without_gwhf(ctx):
    import torch
    probs, dev = _problems(ctx, nprob=3)
    gw = [torch.zeros((p["w"].nfreq, p["w"].D, p["w"].D), dtype=torch.complex128, device=dev) for p in probs]
    nm = [torch.zeros((p["w"].D, p["w"].D), dtype=torch.complex128, device=dev) for p in probs]
    ctx.GreenFtn_w_batched([p["lat"] for p in probs], [p["Hcm"] for p in probs], [p["Scm"] for p in probs],
                           [p["mu"] for p in probs], gw, None, nm)
    torch.cuda.synchronize()
    for i, p in enumerate(probs):
        g, _, n = ctx.GreenFtn_w(p["lat"], p["H"], p["S"], p["mu"])
        assert rel_err(gw[i].transpose(-1, -2).cpu().numpy(), g.cpu().numpy()) < 1e-12
        assert rel_err(nm[i].transpose(-1, -2).cpu().numpy(), n.cpu().numpy()) < 1e-12
