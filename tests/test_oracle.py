"""CPU tests of the FP64 oracle: primitives against numpy/LAPACK, the lattice functions against an
independent literal numpy restatement (tests/ref_numpy.py), and analytic known answers."""
import numpy as np
import pytest

import ref_numpy as R
from conftest import rel_err
from dmftpack_gb300 import models


def _herm(rng, n):
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return a + a.conj().T


@pytest.mark.parametrize("n", [1, 2, 3, 5, 12, 28])
def test_inverse_matches_lapack(orc, n):
    rng = np.random.default_rng(n)
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    x, st = orc.inverse(a)
    assert st == 0
    assert rel_err(x, np.linalg.inv(a)) < 1e-12


@pytest.mark.parametrize("n", [1, 2, 4, 10, 20])
def test_hermitian_eig_matches_lapack(orc, n):
    rng = np.random.default_rng(100 + n)
    h = _herm(rng, n)
    w, v, st = orc.hermitian_eig(h)
    assert st == 0
    assert np.allclose(w, np.linalg.eigvalsh(h), rtol=0, atol=1e-12 * np.abs(w).max())
    assert np.allclose(v @ np.diag(w) @ v.conj().T, h, atol=1e-12 * np.abs(h).max())


def test_hermitian_eig_reads_lower_triangle(orc):
    rng = np.random.default_rng(7)
    h = _herm(rng, 5)
    junk = np.triu(rng.normal(size=(5, 5)) * 10, 1)  # garbage in the strict upper triangle
    w, _, _ = orc.hermitian_eig(np.tril(h) + junk)
    assert np.allclose(w, np.linalg.eigvalsh(h), atol=1e-12)


def test_kmesh_and_hk(orc):
    wl = models.t2g_p(k=3, nfreq=32)
    km = orc.kmesh(*wl.kgrid)
    assert np.abs(km - R.kmesh(*wl.kgrid)).max() == 0.0
    H = orc.hk(wl.n, wl.rindex, wl.hr, km)
    assert rel_err(H, R.hk(wl.n, wl.rindex, wl.hr, km)) < 1e-14
    assert np.abs(H - np.conj(np.swapaxes(H, 1, 2))).max() < 1e-12  # t(-R) = t(R)^H


def test_hubbard_dispersion(orc):
    wl = models.hubbard_2d(kx=8, ky=8, nfreq=16)
    km = orc.kmesh(*wl.kgrid)
    H = orc.hk(wl.n, wl.rindex, wl.hr, km)
    kxs, kys = np.pi * km[:, 0], np.pi * km[:, 1]
    e = -2 * (np.cos(kxs) + np.cos(kys)) + np.cos(kxs) * np.cos(kys)
    assert np.abs(H[:, 0, 0] - e).max() < 1e-13 and np.abs(H[:, 0, 1]).max() == 0


def _small_t2g(nfreq=48):
    wl = models.t2g_p(k=3, nfreq=nfreq, beta=10.0)
    return wl


def test_greenftn_w_matches_numpy(orc):
    wl = _small_t2g()
    km = orc.kmesh(*wl.kgrid)
    H = orc.hk(wl.n, wl.rindex, wl.hr, km)
    mom = orc.moments(wl.sigma, wl.beta)
    gw, gwhf, num = orc.greenftn_w(H, wl.sigma, 0.3, wl.beta, wl.ncl, wl.nh)
    gw2, gwhf2, num2 = R.greenftn_w(H, wl.sigma, mom, 0.3, wl.beta, np.arange(wl.D), wl.ncl, wl.nh)
    assert rel_err(gw, gw2) < 1e-12
    assert rel_err(gwhf, gwhf2) < 1e-12
    assert rel_err(num, num2) < 1e-12


def test_nele_trace_form_matches_eigenvalue_form(orc):
    """GiwToNele literally (numpy eigvals of H+Sigma) == the oracle's trace identity."""
    wl = _small_t2g()
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    mom = orc.moments(wl.sigma, wl.beta)
    for mu in (-1.0, 0.3):
        N = orc.nele(H, wl.sigma, mu, wl.beta, wl.ncl, wl.nh)
        N2 = R.nele_eig(H, wl.sigma, mom, mu, wl.beta, np.arange(wl.D), wl.ncl, wl.nh)
        assert abs(N - N2) < 1e-11 * max(1, abs(N2))


def test_dnele_matches_finite_difference(orc):
    wl = _small_t2g()
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    N, dN = orc.nele(H, wl.sigma, 0.1, wl.beta, wl.ncl, wl.nh, deriv=True)
    h = 1e-6
    fd = (orc.nele(H, wl.sigma, 0.1 + h, wl.beta, wl.ncl, wl.nh)
          - orc.nele(H, wl.sigma, 0.1 - h, wl.beta, wl.ncl, wl.nh)) / (2 * h)
    assert abs(dN - fd) < 1e-6 * abs(fd)


def test_newton_mu_refines_the_bisection_to_the_electron_count(orc):
    """The oracle's Newton polish after GreenFtn_w_adjust_mu's bisection (the mu the library's DMFTGPU_NEWTON search
    converges to): |N(mu) - target| below 1e-12, within the bisection's 1e-5 resolution of its mu."""
    wl = _small_t2g()
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    target = 7.3
    mu_b, _ = orc.adjust_mu(H, wl.sigma, 0.0, wl.beta, wl.ncl, wl.nh, target)
    mu_n = orc.newton_mu(H, wl.sigma, mu_b, wl.beta, wl.D, target)
    assert abs(orc.nele(H, wl.sigma, mu_n, wl.beta, wl.ncl, wl.nh) - target) < 1e-12
    assert abs(mu_n - mu_b) < 2e-5


def test_free_electron_known_answers(orc):
    """Sigma = 0, diagonal H(k): G_loc = (1/Nk) sum_k 1/(iw+mu-e_k)."""
    wl = models.hubbard_2d(kx=6, ky=6, nfreq=40, beta=8.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    sigma = np.zeros_like(wl.sigma)
    gw, gwhf, num = orc.greenftn_w(H, sigma, 0.2, wl.beta, 1, 2)
    iw = 1j * np.pi * (2 * np.arange(40) + 1) / wl.beta
    ek = H[:, 0, 0].real
    exact = (1.0 / (iw[:, None] + 0.2 - ek[None, :])).mean(1)
    assert np.abs(gw[:, 0, 0] - exact).max() < 1e-13
    assert np.abs(gwhf[:, 0, 0] - exact).max() < 1e-13
    # with Sigma = 0, NumMatrix is the Fermi sum
    f = 1 / (1 + np.exp(wl.beta * (ek - 0.2)))
    assert abs(num[0, 0].real - f.mean()) < 1e-12


def test_moments_recover_laurent_series(orc):
    rng = np.random.default_rng(3)
    beta, nf = 20.0, 400
    iw = 1j * np.pi * (2 * np.arange(nf) + 1) / beta
    m = [_herm(rng, 3) * 0.1 for _ in range(4)]
    m[1] = m[1] @ m[1] + np.eye(3)   # positive definite m1
    F = m[0][None] + m[1][None] / iw[:, None, None] + m[2][None] / iw[:, None, None] ** 2 + m[3][None] / iw[:, None, None] ** 3
    mom = orc.moments(F, beta)
    for i in range(4):
        assert np.abs(mom[i] - m[i]).max() < 1e-7 * max(1, np.abs(m[i]).max())


def test_fourier_round_trip_two_pole(orc):
    """iw -> tau -> iw on a two-pole G: the tail-corrected transform and the exact piecewise-linear inverse."""
    beta, nf, ntau = 10.0, 256, 2048
    iw = 1j * np.pi * (2 * np.arange(nf) + 1) / beta
    e = np.array([-0.7, 0.4])
    G = np.zeros((nf, 2, 2), complex)
    for i in range(2):
        G[:, i, i] = 1.0 / (iw - e[i])
    gt, fix = orc.fourier(G, beta, ntau, green_asym=True)
    tau = np.arange(ntau + 1) * beta / ntau
    exact = -np.exp(-np.outer(tau, e)) / (1 + np.exp(-beta * e))
    assert np.abs(gt[:, 0, 0] - exact[:, 0]).max() < 1e-6
    assert np.abs(gt[0, 0, 0] + gt[-1, 0, 0] + 1) < 1e-6   # G(0+) + G(beta-) = -1
    gw, st = orc.tau2w(gt, beta, 64)
    assert np.abs(gw[:, 1, 1] - G[:64, 1, 1]).max() < 1e-4


def test_sigma2_vanishes_without_interaction(orc):
    beta, ntau = 5.0, 64
    tau = np.arange(ntau + 1) * beta / ntau
    gt = np.zeros((ntau + 1, 2, 2), complex)
    gt[:, 0, 0] = gt[:, 1, 1] = -0.5
    uidx, ut = orc.gen_uijkl(2, 0.0, 0.0, 0.0, density_density=True)
    st, fix, status = orc.sigma2_tau(gt, uidx, ut * 0, beta)
    assert np.all(np.abs(st[1:-1]) <= 1e-10)


def test_sigma2_matches_a_dense_tensor_contraction(orc):
    """getStimp (src/SCGF2_fullLoop.cpp:603-690) restated independently: the U list scattered into a dense
    U_{iqmk} and the second-order diagram as one einsum over G(tau) and G(beta - tau),
    Sigma_ij(tau) = U_{iqmk} U_{lnpj} [G_kl G_mn - G_kn G_ml](tau) G_pq(beta - tau), against the oracle's loop over
    pairs of list entries.  G(tau) of a non-interacting 4-orbital model is negative definite, so the positivity
    fix-up does not fire."""
    rng = np.random.default_rng(7)
    d, ntau, beta = 4, 32, 6.0
    A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    eps, V = np.linalg.eigh(0.4 * (A + A.conj().T))
    tau = np.arange(ntau + 1) * beta / ntau
    occ = np.exp(-np.outer(tau, eps)) / (1 + np.exp(-beta * eps))[None]
    gt = -np.einsum("ia,ta,ja->tij", V, occ, V.conj())
    uidx, ut = orc.gen_uijkl(d, 3.0, 1.9, 0.55)
    U = np.zeros((d,) * 4, complex)
    for (i, q, m, k), u in zip(uidx, ut):
        U[i, q, m, k] += u
    gm = gt[::-1]
    want = (np.einsum("iqmk,lnpj,tkl,tmn,tpq->tij", U, U, gt, gt, gm, optimize=True)
            - np.einsum("iqmk,lnpj,tkn,tml,tpq->tij", U, U, gt, gt, gm, optimize=True))
    got, fix, status = orc.sigma2_tau(gt, uidx, ut, beta)
    assert fix == 0
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_hyb_delta_fock_and_dyson_match_dense_restatements(orc):
    """Construct_hyb_delta (src/Construct_hyb_delta.cpp:47-119) on a projected orbital subset, getFockOperator
    (src/SCGF2_fullLoop.cpp:583-597) as two einsums over a dense U, and getGwimp (src/SCGF2_fullLoop.cpp:551-578)
    as a batched inverse, each restated with numpy and compared with the oracle."""
    rng = np.random.default_rng(11)
    D, nf, beta, mu = 3, 24, 7.0, 0.3
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    A = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
    himp = (A + A.conj().T) / 4
    sig = 0.2 * (rng.normal(size=(nf, D, D)) + 1j * rng.normal(size=(nf, D, D)))
    gw = np.linalg.inv((1j * wn[:, None, None] + mu) * np.eye(D)[None] - himp[None] - sig - 0.5j * np.eye(D)[None])
    orb = np.array([2, 0])
    P = np.ix_(orb, orb)
    want = ((1j * wn[:, None, None] + mu) * np.eye(2)[None] - himp[P][None] - sig[(slice(None),) + P]
            - np.linalg.inv(gw[(slice(None),) + P]))
    assert np.abs(orc.hyb_delta(orb, sig, gw, himp, mu, beta) - want).max() <= 1e-12 * np.abs(want).max()
    d = 4
    uidx, ut = orc.gen_uijkl(d, 3.0, 1.9, 0.55)
    U = np.zeros((d,) * 4, complex)
    for (a, b_, c, e), u in zip(uidx, ut):
        U[a, b_, c, e] += u
    B = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    occ = B @ B.conj().T / (2 * d)
    want_f = np.einsum("abcd,ca->bd", U, occ) - np.einsum("abcd,da->bc", U, occ)
    fk = orc.fock(occ, uidx, ut)
    assert np.abs(fk - want_f).max() <= 1e-12 * np.abs(want_f).max()
    delta = 0.3 * np.eye(d)[None] / (1j * wn[:, None, None] - 0.2)
    s2 = 0.1 * (rng.normal(size=(nf, d, d)) + 1j * rng.normal(size=(nf, d, d)))
    h4 = np.diag([0.1, -0.2, 0.3, 0.0]).astype(complex)
    want_g = np.linalg.inv((1j * wn[:, None, None] + mu) * np.eye(d)[None] - h4[None] - delta - fk[None] - s2)
    got_g, _ = orc.dyson(h4, delta, fk, s2, mu, beta)
    assert np.abs(got_g[:nf] - want_g).max() <= 1e-12 * np.abs(want_g).max()


def test_gen_uijkl_counts(orc):
    uidx, ut = orc.gen_uijkl(10, 4.0, 2.6, 0.7)
    assert len(ut) == 180
    uidx, ut = orc.gen_uijkl(2, 2.0, 2.0, 0.0, density_density=True)
    assert len(ut) == 4


def test_oracle_tau2w_against_exact_integral(orc):
    """The oracle's FT_t_to_w (the reference's per-segment formula) against the 40-digit evaluation of the same
    integral in tests/golden/tau2w_exact.npz."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "tau2w_exact.npz"))
    got, _ = orc.tau2w(z["ft"], float(z["beta"]), int(z["nfreq"]))
    assert np.abs(got - z["w"]).max() / np.abs(z["w"]).max() < 1e-10


def test_oracle_scgf2_without_interaction_keeps_the_bare_green_function(orc):
    """U = 0: no Fock or second-order term, so SCGF2 stops after the minimum 10 loops with G_imp = the
    non-interacting G (src/SCGF2_fullLoop.cpp:477-523).  SE_out is not exactly zero: getStimp's positivity fix-up
    replaces every Sigma(tau) = 0 point (minimum eigenvalue >= 0) by -1e-10 I (src/SCGF2_fullLoop.cpp:657-688)."""
    d, nf, ntau, beta, mu = 2, 32, 128, 8.0, 0.1
    himp = np.array([[0.2, 0.05], [0.05, -0.1]], complex)
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    weiss = 0.3 * np.eye(d)[None] / (1j * wn[:, None, None] - 0.4)
    g0 = np.linalg.inv((1j * wn[:, None, None] + mu) * np.eye(d)[None] - himp[None] - weiss)
    uidx, ut = orc.gen_uijkl(d, 0.0, 0.0, 0.0, density_density=True)
    se, g, loops = orc.scgf2(himp, weiss, g0, uidx, ut, mu, beta, ntau, 0.5)
    assert loops == 10
    assert np.abs(se).max() < 1e-9
    assert np.abs(g[:nf] - g0).max() < 1e-9


def _overlap(rng, nk, n, scale=0.2):
    B = scale * (rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n)))
    return np.eye(n)[None] + (B @ B.conj().transpose(0, 2, 1)) / n


def test_downfold_orthogonal_basis_keeps_the_correlated_block(orc):
    # with S = I the eigenvectors are unitary, the projected rows are already orthonormal and the correlated block
    # of H_model is H's own; the ligand block is a unitary rotation of H's, so H_PL H_LP and its spectrum survive
    wl = models.t2g_p(k=3, nfreq=8)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    D = 3
    eps, Hm, DF, himp = orc.downfold(H, None, np.arange(D))
    assert np.abs(Hm[:, :D, :D] - H[:, :D, :D]).max() < 1e-12
    assert np.abs(Hm[:, :D, D:] @ Hm[:, D:, :D] - H[:, :D, D:] @ H[:, D:, :D]).max() < 1e-12
    assert np.abs(np.linalg.eigvalsh(Hm[:, D:, D:]) - np.linalg.eigvalsh(H[:, D:, D:])).max() < 1e-12
    assert np.abs(himp - H[:, :D, :D].mean(0)).max() < 1e-12


def test_downfold_generalized_eigenproblem_and_orthonormal_frame(orc):
    rng = np.random.default_rng(11)
    nk, n, hartr = 4, 9, [1, 4, 5, 7]
    H = rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n))
    H = (H + H.conj().transpose(0, 2, 1)) / 2
    S = _overlap(rng, nk, n)
    eps, Hm, DF, himp = orc.downfold(H, S, hartr)
    # eps solves det(H - e S) = 0: the eigenvalues of S^-1/2 H S^-1/2
    for k in range(nk):
        w, W = np.linalg.eigh(S[k])
        Si = (W * w ** -0.5) @ W.conj().T
        assert np.abs(np.linalg.eigvalsh(Si @ H[k] @ Si) - eps[k]).max() < 1e-12
    assert np.abs(DF @ DF.conj().transpose(0, 2, 1) - np.eye(n)[None]).max() < 1e-12
    assert np.abs(np.linalg.eigvalsh(Hm) - eps).max() < 1e-12
    assert np.abs(himp - Hm[:, :4, :4].mean(0)).max() < 1e-14


def test_density_dft_is_consistent_with_nummatrix_and_nele(orc):
    # the correlated block of densityMatDFT averaged over k is GreenFtn_w's NumMatrix, its mean trace N(mu)
    wl = models.t2g_p(k=3, nfreq=32, beta=10.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    d = orc.density_dft(H, wl.sigma, 0.2, wl.beta)
    _, _, num = orc.greenftn_w(H, wl.sigma, 0.2, wl.beta, wl.ncl, wl.nh)
    assert np.abs(d[:, :3, :3].mean(0) - num).max() < 1e-12
    N = orc.nele(H, wl.sigma, 0.2, wl.beta, wl.ncl, wl.nh)
    N = N[0] if isinstance(N, tuple) else N
    assert abs(np.trace(d, axis1=1, axis2=2).real.mean() - N) < 1e-11
    assert np.abs(d - d.conj().transpose(0, 2, 1)).max() < 1e-13


def test_density_dft_without_self_energy_is_the_fermi_function_of_h(orc):
    wl = models.t2g_p(k=2, nfreq=16, beta=8.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    d = orc.density_dft(H, np.zeros_like(wl.sigma), 0.1, wl.beta)
    e, U = np.linalg.eigh(H)
    f = (U / (1 + np.exp(wl.beta * (e - 0.1)))[:, None, :]) @ U.conj().transpose(0, 2, 1)
    assert np.abs(d - f).max() < 1e-12


def test_upfold_inverts_the_hk_fourier_sum(orc):
    # with DF = V = I and S = I the k -> R sum of H(k) returns the hopping table (k grid wider than the R range)
    wl = models.t2g_p(k=6, nfreq=8)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    eye = np.broadcast_to(np.eye(wl.n, dtype=np.complex128), H.shape)
    dd, d, direct = orc.upfold(H, eye, eye, None, wl.kgrid, wl.rindex)
    for x in (dd, d, direct):
        assert np.abs(x - wl.hr).max() < 1e-12


def test_band_window_selection():
    from dmftpack_gb300.window import low_energy_subspace_in_KS_basis as sel
    e = np.array([[-5.0, -1.0, 0.2, 0.9, 3.0], [-4.0, -2.5, -0.5, 1.5, 2.5]])
    nband, idx = sel(e, 0.1, -3.0, 2.0, n_corr=2)
    assert list(nband) == [3, 3] and list(idx[0]) == [1, 2, 3] and list(idx[1]) == [1, 2, 3]
    nband, idx = sel(e, 0.0, -10.0, 10.0, n_corr=2, downfolding=False)
    assert list(nband) == [5, 5] and list(idx[1]) == [0, 1, 2, 3, 4]
    with pytest.raises(ValueError):
        sel(e, 0.0, 5.0, 6.0, n_corr=1)      # empty window
    with pytest.raises(ValueError):
        sel(e, 0.1, -3.0, 2.0, n_corr=4)     # fewer bands than correlated orbitals


def test_windowed_downfold_and_upfold_reduce_to_the_full_window(orc):
    rng = np.random.default_rng(21)
    wl = models.t2g_p(k=3, nfreq=8)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    S = _overlap(rng, H.shape[0], wl.n)
    full = [np.arange(wl.n)] * H.shape[0]
    e_w, hm_w, df_w, v_w, himp_w = orc.downfold_window(H, S, [0, 1, 2], full)
    eps, Hm, DF, himp = orc.downfold(H, S, [0, 1, 2])
    assert np.abs(np.array(e_w) - eps).max() < 1e-12
    assert np.abs(np.array(hm_w)[:, :3, :3] - Hm[:, :3, :3]).max() < 1e-12
    assert np.abs(himp_w - himp).max() < 1e-12
    dens = [(d * 0.3 + d.conj().T * 0.3) for d in hm_w]
    got = orc.upfold_window(dens, df_w, np.array(v_w), S, e_w, full, 0.0, 10.0, wl.kgrid, wl.rindex)
    ref = orc.upfold(np.array(dens), np.array(df_w), np.array(v_w), S, wl.kgrid, wl.rindex)
    for g_, r_ in zip(got, ref):
        assert np.abs(g_ - r_).max() < 1e-12


def test_windowed_upfold_of_the_model_fermi_density_is_the_full_fermi_density(orc):
    # inside the window the model-basis density DF f(e) DF^H maps back to f(e) on the window's bands; outside,
    # upfolding_density fills in f(e), so the result is V f(e) V^H over every band
    from dmftpack_gb300.window import low_energy_subspace_in_KS_basis as sel
    rng = np.random.default_rng(22)
    wl = models.t2g_p(k=3, nfreq=8)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    S = _overlap(rng, H.shape[0], wl.n)
    beta, mu = 8.0, 0.0
    eps_all = np.array([np.linalg.eigvalsh(np.linalg.solve(np.linalg.cholesky(S[k]), H[k])
                                           @ np.linalg.inv(np.linalg.cholesky(S[k])).conj().T)
                        for k in range(H.shape[0])])
    lo, hi = np.quantile(eps_all, 0.2), np.quantile(eps_all, 0.95)
    nband, win = sel(eps_all, mu, lo, hi, n_corr=3)
    assert nband.min() < wl.n  # a genuine window
    e_w, hm_w, df_w, v_w, _ = orc.downfold_window(H, S, [0, 1, 2], win)
    fermi = lambda e: 1.0 / (1.0 + np.exp(beta * (e - mu)))
    dens = [df_w[k] @ np.diag(fermi(e_w[k][win[k]])) @ df_w[k].conj().T for k in range(H.shape[0])]
    got = orc.upfold_window(dens, df_w, np.array(v_w), S, e_w, win, mu, beta, wl.kgrid, wl.rindex)
    V = np.array(v_w)
    full = np.array([V[k] @ np.diag(fermi(e_w[k])) @ V[k].conj().T for k in range(H.shape[0])])
    eye = np.broadcast_to(np.eye(wl.n, dtype=np.complex128), full.shape)
    ref = orc.upfold(full, eye, eye, S, wl.kgrid, wl.rindex)
    for g_, r_ in zip(got, ref):
        assert np.abs(g_ - r_).max() < 1e-11


def test_weak_solver_hf_is_the_fock_term(orc):
    """on_shot_HF: Sigma = F at every frequency and in the static slot, no 1/iw tail; SC2PT adds a causal second-order
    part whose static slot is still F."""
    d, nf, beta = 4, 48, 8.0
    rng = np.random.default_rng(3)
    A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    h = 0.3 * (A + A.conj().T) / 2
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    g = np.linalg.inv(1j * wn[:, None, None] * np.eye(d)[None] - h[None])
    uidx, ut = orc.gen_uijkl(d, 2.0, 1.4, 0.3)
    F = orc.fock(orc.occ(g, beta), uidx, ut)
    se = orc.weak_solver("HF", g, None, uidx, ut, beta, 192)
    assert np.abs(se[:nf] - F[None]).max() < 1e-14 and np.abs(se[nf] - F).max() < 1e-14
    assert np.abs(se[nf + 1:]).max() < 1e-14
    se2 = orc.weak_solver("SC2PT", g, None, uidx, ut, beta, 192)
    assert np.abs(se2[nf] - F).max() < 1e-14
    # second-order part: Im Sigma^(2)(iw) <= 0 on the diagonal (causal)
    assert (np.einsum("nii->ni", se2[:nf] - F[None]).imag <= 1e-12).all()
