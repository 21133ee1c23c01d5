"""GPU parity of the model-Hamiltonian construction (generalized eigenproblem + downfolding_ftn, k_downfold) against
the oracle, through the C ABI.  The ligand rows of DF are fixed only up to a unitary rotation among themselves
(Householder and eigenvector-phase conventions), so the comparison is on the quantities that do not depend on it:
band energies, the correlated block of H_model, H_imp, H_PL H_LP, the ligand block's spectrum, DF's unitarity and
the local Green function GreenFtn_w builds from H_model."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _overlap(rng, nk, n, scale=0.3):
    B = scale * (rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n)))
    return np.eye(n)[None] + (B @ B.conj().transpose(0, 2, 1)) / n


def _model_hk(orc, wl):
    return orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))


def _check(eps_g, hm_g, hi_g, df_g, eps, Hm, himp, D):
    n = Hm.shape[1]
    sc = max(1.0, np.abs(eps).max())
    assert np.abs(eps_g - eps).max() < TOL * sc
    assert np.abs(hm_g[:, :D, :D] - Hm[:, :D, :D]).max() < TOL * sc
    assert np.abs(hi_g - himp).max() < TOL * sc
    assert np.abs(hm_g - hm_g.conj().transpose(0, 2, 1)).max() < TOL * sc
    assert np.abs(np.linalg.eigvalsh(hm_g) - eps).max() < TOL * sc
    pl = hm_g[:, :D, D:] @ hm_g[:, D:, :D]
    assert np.abs(pl - Hm[:, :D, D:] @ Hm[:, D:, :D]).max() < TOL * sc * sc
    if D < n:
        assert np.abs(np.linalg.eigvalsh(hm_g[:, D:, D:]) - np.linalg.eigvalsh(Hm[:, D:, D:])).max() < TOL * sc
    if df_g is not None:
        assert np.abs(df_g @ df_g.conj().transpose(0, 2, 1) - np.eye(n)[None]).max() < 1e-12


CASES = {
    # name: (workload, correlated orbitals, overlap)
    "t2g_p_ortho": (lambda: models.t2g_p(k=4, nfreq=8), [0, 1, 2], False),
    "t2g_p_overlap": (lambda: models.t2g_p(k=4, nfreq=8), [0, 1, 2], True),
    "dp28_overlap": (lambda: models.dp28(k=3, nfreq=8, ntau=16), list(range(10)), True),
    "dp28_scattered": (lambda: models.dp28(k=2, nfreq=8, ntau=16), [3, 0, 11, 27, 14, 5], True),
    "soc56_overlap": (lambda: models.soc56(k=2, nfreq=8), list(range(20)), True),
}


@pytest.mark.parametrize("case", list(CASES))
def test_downfold_matches_oracle(ctx, orc, case):
    make, hartr, overlap = CASES[case]
    wl = make()
    H = _model_hk(orc, wl)
    S = _overlap(np.random.default_rng(7), H.shape[0], wl.n) if overlap else None
    eps, Hm, DF, himp = orc.downfold(H, S, hartr)
    eps_g, hm_g, hi_g, df_g, ev_g = ctx.downfolding_ftn(H, hartr, S, with_df=True)
    _check(eps_g, hm_g, hi_g, df_g, eps, Hm, himp, len(hartr))
    # the eigenvectors solve H v = e S v with V^H S V = I
    Sm = np.eye(wl.n)[None] if S is None else S
    sc = max(1.0, np.abs(eps).max())
    assert np.abs(H @ ev_g - (Sm @ ev_g) * eps_g[:, None, :]).max() < TOL * sc
    assert np.abs(ev_g.conj().transpose(0, 2, 1) @ Sm @ ev_g - np.eye(wl.n)[None]).max() < 1e-11
    # the correlated rows of DF are fixed up to the eigenvector phases, which cancel in DF_P diag(e) DF_P^H
    D = len(hartr)
    assert np.abs(hm_g[:, :D, :D] - (df_g[:, :D] * eps_g[:, None, :]) @ df_g[:, :D].conj().transpose(0, 2, 1)).max() \
        < TOL * max(1.0, np.abs(eps).max())


def test_downfold_device_pointers(ctx, orc):
    import torch
    wl = models.t2g_p(k=3, nfreq=8)
    H = _model_hk(orc, wl)
    S = _overlap(np.random.default_rng(3), H.shape[0], wl.n)
    eps, Hm, DF, himp = orc.downfold(H, S, [0, 1, 2])
    dev = torch.device("cuda:0")
    eps_g, hm_g, hi_g = ctx.downfolding_ftn(torch.from_numpy(H).to(dev), [0, 1, 2], torch.from_numpy(S).to(dev))
    torch.cuda.synchronize()
    _check(eps_g.cpu().numpy(), hm_g.cpu().numpy(), hi_g.cpu().numpy(), None, eps, Hm, himp, 3)


def test_downfolded_local_green_function_is_gauge_free(ctx, orc):
    # G_loc from the kernel's H_model equals G_loc from the oracle's H_model although their ligand frames differ
    wl = models.t2g_p(k=4, nfreq=24, beta=10.0)
    H = _model_hk(orc, wl)
    S = _overlap(np.random.default_rng(5), H.shape[0], wl.n)
    _, Hm, _, _ = orc.downfold(H, S, [0, 1, 2])
    _, hm_g, _ = ctx.downfolding_ftn(H, [0, 1, 2], S)
    gw_o, _, num_o = orc.greenftn_w(Hm, wl.sigma, 0.2, wl.beta, 1, 3)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, 3)
    gw_g, _, num_g = ctx.GreenFtn_w(lat, hm_g, wl.sigma, 0.2)
    assert rel_err(gw_g, gw_o) < 1e-10
    assert rel_err(num_g, num_o) < 1e-10


def test_downfold_rejects_bad_input(ctx):
    n = 6
    H = np.zeros((2, n, n), np.complex128)
    H[:] = np.diag(np.arange(n, dtype=float))
    with pytest.raises(lib.DmftGpuError) as e:
        ctx.downfolding_ftn(H, [0, 0])
    assert e.value.code == lib.BADARG
    with pytest.raises(lib.DmftGpuError) as e:
        ctx.downfolding_ftn(H, [0, n])
    assert e.value.code == lib.BADARG
    with pytest.raises(lib.DmftGpuError) as e:
        ctx.downfolding_ftn(np.zeros((1, 57, 57), np.complex128), [0])
    assert e.value.code == lib.BADARG
    S = np.broadcast_to(np.eye(n, dtype=np.complex128), (2, n, n)).copy()
    S[1, 2, 2] = -1.0   # indefinite overlap: flagged, no fault
    with pytest.raises(lib.DmftGpuError) as e:
        ctx.downfolding_ftn(H, [0, 1], S)
    assert e.value.code == lib.SINGULAR
    # the context stays usable
    eps, hm, hi = ctx.downfolding_ftn(H, [0, 1])
    assert np.abs(eps - np.arange(n)[None]).max() < 1e-13


def _dp28_overlap(orc, k=3):
    wl = models.dp28(k=k, nfreq=16, ntau=16, beta=20.0)
    H = _model_hk(orc, wl)
    return wl, H, _overlap(np.random.default_rng(7), H.shape[0], wl.n)


def test_downfold_band_window_matches_oracle(ctx, orc):
    """The band window of low_energy_subspace_in_KS_basis (src/downfolding.cpp:130-187) selected on the device:
    NBAND[k] (8 .. 11 here, ragged) and FromValToKS equal the host selection on the oracle's band energies, and the
    windowed H_model (padded beyond NBAND[k]) matches the oracle's ragged one on every gauge-free quantity."""
    from dmftpack_gb300 import window
    wl, H, S = _dp28_overlap(orc)
    hartr, mu, lower, upper, epad = list(range(6)), 0.0, -6.0, 3.0, 1e4
    D = len(hartr)
    eps_g, hm_g, hi_g, df_g, ev_g, nb_g, fvk_g = ctx.downfolding_ftn(H, hartr, S, with_df=True,
                                                                     window=(mu, lower, upper), pad_energy=epad)
    eps_full = orc.downfold(H, S, hartr)[0]
    nb_o, fvk_o = window.low_energy_subspace_in_KS_basis(eps_full, mu, lower, upper, D)
    assert np.array_equal(nb_g, nb_o) and all(np.array_equal(a, b) for a, b in zip(fvk_g, fvk_o))
    assert len(set(nb_o.tolist())) > 1   # ragged
    eps, Hm, DF, V, himp = orc.downfold_window(H, S, hartr, fvk_o)
    sc = max(1.0, np.abs(eps_full).max())
    assert np.abs(eps_g - eps_full).max() < TOL * sc
    assert np.abs(hi_g - himp).max() < TOL * sc
    n = wl.n
    for k in range(H.shape[0]):
        nb = nb_o[k]
        blk = hm_g[k][:nb, :nb]
        assert np.abs(blk[:D, :D] - Hm[k][:D, :D]).max() < TOL * sc
        assert np.abs(np.linalg.eigvalsh(blk) - eps_full[k][fvk_o[k]]).max() < TOL * sc
        pl = blk[:D, D:] @ blk[D:, :D]
        assert np.abs(pl - Hm[k][:D, D:] @ Hm[k][D:, :D]).max() < TOL * sc * sc
        pad = hm_g[k].copy()
        pad[:nb, :nb] = 0
        assert np.abs(pad - np.diag(np.r_[np.zeros(nb), np.full(n - nb, epad)])).max() == 0
        assert np.abs(df_g[k] @ df_g[k].conj().T - np.eye(n)).max() < 1e-12


def test_downfold_band_window_lattice_sum_equals_ragged(ctx, orc):
    """GreenFtn_w on the padded H_model equals the lattice sum over the ragged NBAND[k] x NBAND[k] matrices (explicit
    numpy inversion per k), and N(mu) does not depend on the padding energy (the padded bands cancel)."""
    wl, H, S = _dp28_overlap(orc, k=2)
    hartr, D = list(range(6)), 6
    nf, beta, mu = 16, 20.0, 0.3
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    sig = np.zeros((nf, D, D), np.complex128)
    for d in range(D):
        sig[:, d, d] = 0.1 - 0.6j / (wn + 0.4)
    _, hm, _, nb, _ = ctx.downfolding_ftn(H, hartr, S, window=(0.0, -6.0, 3.0), pad_energy=1e4)
    nk, n = hm.shape[0], hm.shape[1]
    lat = lib.Lattice(n, nk, nf, beta, 1, D)
    gw, _, _ = ctx.GreenFtn_w(lat, hm, sig, mu)
    ref = np.zeros((nf, D, D), np.complex128)
    for k in range(nk):
        m = nb[k]
        for f in range(nf):
            A = (1j * wn[f] + mu) * np.eye(m) - hm[k][:m, :m]
            A[:D, :D] -= sig[f]
            ref[f] += np.linalg.inv(A)[:D, :D]
    assert rel_err(gw, ref / nk) < 1e-10
    _, hm2, _, _, _ = ctx.downfolding_ftn(H, hartr, S, window=(0.0, -6.0, 3.0), pad_energy=3e4)
    N1 = ctx.GiwToNele(lat, hm, sig, mu)
    N2 = ctx.GiwToNele(lat, hm2, sig, mu)
    assert abs(N1 - N2) < 1e-11 * abs(N1)


def test_downfold_band_window_rejects_too_few_bands(ctx, orc):
    wl, H, S = _dp28_overlap(orc, k=2)
    with pytest.raises(lib.DmftGpuError) as e:   # a window narrower than the 6 correlated orbitals at some k
        ctx.downfolding_ftn(H, list(range(6)), S, window=(0.0, -1.0, 1.0))
    assert e.value.code == lib.BADARG
    eps, hm, hi = ctx.downfolding_ftn(H, list(range(6)), S)   # the context stays usable
    assert np.isfinite(eps).all()
