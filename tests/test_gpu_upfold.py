"""GPU parity of upfolding_density (k_upfold_k, the three k -> R axis passes and the gather) against the oracle,
through the C ABI, on the chain the reference runs: the generalized eigensolve and downfolding, densityMatDFT of the
model Hamiltonian, then the upfolding."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu


def _hk(orc, wl):
    return orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))


def test_upfold_returns_the_hopping_table(ctx, orc):
    wl = models.t2g_p(k=6, nfreq=8)
    H = _hk(orc, wl)
    eye = np.broadcast_to(np.eye(wl.n, dtype=np.complex128), H.shape).copy()
    outs = ctx.upfolding_density(H, eye, eye, wl.kgrid, wl.rindex)
    for x in outs:
        assert np.abs(x - wl.hr).max() < 1e-12


@pytest.mark.parametrize("overlap", [False, True])
def test_upfold_chain_matches_oracle(ctx, orc, overlap):
    wl = models.dp28(k=3, nfreq=16, ntau=16, beta=20.0)
    H = _hk(orc, wl)
    S = None
    if overlap:
        rng = np.random.default_rng(9)
        B = 0.3 * (rng.normal(size=H.shape) + 1j * rng.normal(size=H.shape))
        S = np.eye(wl.n)[None] + B @ B.conj().transpose(0, 2, 1) / wl.n
    hartr = list(range(wl.D))
    _, hm, _, df, ev = ctx.downfolding_ftn(H, hartr, S, with_df=True)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, wl.D)
    dens = ctx.densityMatDFT(lat, hm, wl.sigma, 0.1)
    got = ctx.upfolding_density(dens, df, ev, wl.kgrid, wl.rindex, S)
    ref = orc.upfold(dens, df, ev, S, wl.kgrid, wl.rindex)
    for g, r in zip(got, ref):
        assert rel_err(g, r) < 1e-12


def test_upfold_device_pointers_and_bad_index(ctx, orc):
    import torch
    wl = models.t2g_p(k=6, nfreq=8)
    H = _hk(orc, wl)
    eye = np.broadcast_to(np.eye(wl.n, dtype=np.complex128), H.shape).copy()
    dev = torch.device("cuda:0")
    Hd, Id = torch.from_numpy(H).to(dev), torch.from_numpy(eye).to(dev)
    outs = ctx.upfolding_density(Hd, Id, Id, wl.kgrid, wl.rindex)
    torch.cuda.synchronize()
    assert np.abs(outs[2].cpu().numpy() - wl.hr).max() < 1e-12
    bad = np.array(wl.rindex, dtype=np.int32).copy()
    bad[0, 3] = wl.n
    with pytest.raises(lib.DmftGpuError) as e:
        ctx.upfolding_density(H, eye, eye, wl.kgrid, bad)
    assert e.value.code == lib.BADARG


def test_upfold_band_window_matches_oracle(ctx, orc):
    """upfolding_density after a windowed downfolding (src/upfolding.cpp:10-35): the Fermi diagonal outside the
    window, the model-basis block inside it, against the oracle's upfold_window on the same inputs."""
    wl = models.dp28(k=3, nfreq=16, ntau=16, beta=20.0)
    H = _hk(orc, wl)
    rng = np.random.default_rng(9)
    B = 0.3 * (rng.normal(size=H.shape) + 1j * rng.normal(size=H.shape))
    S = np.eye(wl.n)[None] + B @ B.conj().transpose(0, 2, 1) / wl.n
    hartr, D, mu = list(range(6)), 6, 0.1
    eps, hm, _, df, ev, nb, fvk = ctx.downfolding_ftn(H, hartr, S, with_df=True, window=(0.0, -6.0, 3.0))
    sig = wl.sigma[:, :D, :D].copy()
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, D)
    dens = ctx.densityMatDFT(lat, hm, sig, mu)
    for k in range(wl.nk):   # the padded bands carry no density
        assert np.abs(dens[k][nb[k]:, :]).max() < 1e-12 and np.abs(dens[k][:, nb[k]:]).max() < 1e-12
    got = ctx.upfolding_density(dens, df, ev, wl.kgrid, wl.rindex, S, window=(eps, nb, fvk, mu, wl.beta))
    ref = orc.upfold_window([dens[k][:nb[k], :nb[k]] for k in range(wl.nk)],
                            [df[k][:nb[k], :nb[k]] for k in range(wl.nk)], ev, S, eps, fvk, mu, wl.beta, wl.kgrid,
                            wl.rindex)
    for g, r in zip(got, ref):
        assert rel_err(g, r) < 1e-12
