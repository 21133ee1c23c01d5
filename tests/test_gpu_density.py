"""GPU parity of GreenFtn_w's per-k density matrix densityMatDFT (k_dens_sum + k_dens_finish, through the C ABI)
against the oracle's explicit n x n inversions."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu

TOL = 1e-10

CASES = {
    # name: (workload, HartrIndex or None)
    "t2g_p": (lambda: models.t2g_p(k=3, nfreq=40, beta=12.0), None),
    "t2g_p_k8": (lambda: models.t2g_p(k=8, nfreq=16, beta=12.0), None),
    "t2g_p_hartr": (lambda: models.t2g_p(k=3, nfreq=24, beta=12.0), [4, 1, 9]),
    "hubbard_single_orbital": (lambda: models.hubbard_2d(kx=6, ky=6, nfreq=32, beta=10.0), None),
    "dp28": (lambda: models.dp28(k=2, nfreq=24, ntau=16, beta=20.0), None),
    "soc56": (lambda: models.soc56(k=2, nfreq=16), None),
}


def _hk(orc, wl):
    return orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("case", list(CASES))
def test_density_dft_matches_oracle(ctx, orc, case, mixed):
    """FP64 at 1e-10 and double-float (DMFTGPU_MIXED) at 1e-9 against the oracle's explicit inversions."""
    make, hartr = CASES[case]
    wl = make()
    H = _hk(orc, wl)
    mu = 0.15
    ref = orc.density_dft(H, wl.sigma, mu, wl.beta, hartr)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, wl.ncl, wl.nh, hartr)
    got = ctx.densityMatDFT(lat, H, wl.sigma, mu, mixed=mixed)
    assert rel_err(got, ref) < (1e-9 if mixed else TOL)


def test_density_dft_correlated_block_is_nummatrix(ctx, orc):
    wl = models.dp28(k=3, nfreq=32, ntau=16, beta=20.0)
    H = _hk(orc, wl)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, wl.ncl, wl.nh)
    d = ctx.densityMatDFT(lat, H, wl.sigma, 0.1)
    _, _, num = ctx.GreenFtn_w(lat, H, wl.sigma, 0.1)
    D = wl.D
    assert rel_err(d[:, :D, :D].mean(0), num) < 1e-11
    assert np.abs(d - d.conj().transpose(0, 2, 1)).max() < 1e-12


def test_density_dft_device_pointers(ctx, orc):
    import torch
    wl = models.t2g_p(k=3, nfreq=24, beta=12.0)
    H = _hk(orc, wl)
    ref = orc.density_dft(H, wl.sigma, 0.2, wl.beta)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, wl.ncl, wl.nh)
    dev = torch.device("cuda:0")
    got = ctx.densityMatDFT(lat, torch.from_numpy(H).to(dev), torch.from_numpy(wl.sigma).to(dev), 0.2)
    torch.cuda.synchronize()
    assert rel_err(got.cpu().numpy(), ref) < TOL
