"""GPU parity of the impurity stage (FourierTransform, FT_t_to_w, getStimp, getFockOperator, getGwimp,
getoccMat, estimate_asymto, IPT) against the FP64 oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _two_pole(nf, beta, d=2, seed=0):
    rng = np.random.default_rng(seed)
    iw = 1j * np.pi * (2 * np.arange(nf) + 1) / beta
    A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    H = (A + A.conj().T) / 2
    B = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    Hb = (B + B.conj().T) / 2
    G = np.linalg.inv(iw[:, None, None] * np.eye(d) - H - 0.3 * np.linalg.inv(iw[:, None, None] * np.eye(d) - Hb))
    return G


@pytest.mark.parametrize("direct", [False, True])
@pytest.mark.parametrize("d,green,m1,ntau", [(2, True, False, 640), (2, False, True, 512), (3, False, False, 640),
                                             (4, True, False, 512)])
def test_fourier_w2tau(ctx, orc, d, green, m1, ntau, direct):
    """ntau = 512 runs the FFT path unless direct; 640 (not a power of two) always the direct sums."""
    beta, nf = 10.0, 160
    G = _two_pole(nf, beta, d, seed=d)
    M1 = np.eye(d) if m1 else None
    ref, _ = orc.fourier(G, beta, ntau, green_asym=green, m1=M1)
    got = ctx.FourierTransform(G, beta, ntau, greenFtnAsym=green, moments1=M1, direct=direct)
    assert rel_err(got, ref) < TOL


def test_fourier_positivity_fixup(ctx, orc):
    beta, nf, ntau = 8.0, 96, 256
    G = -_two_pole(nf, beta, 2, seed=5)          # wrong sign: G(tau) positive, every point gets fixed
    ref, fix = orc.fourier(G, beta, ntau, green_asym=True)
    assert fix > 0
    got = ctx.FourierTransform(G, beta, ntau, greenFtnAsym=True)
    assert rel_err(got, ref) < TOL


def test_fourier_with_given_moments(ctx, orc):
    beta, nf, ntau = 12.0, 128, 512
    G = _two_pole(nf, beta, 3, seed=9)
    mom = orc.moments(G, beta, green_asym=True)
    ref, _ = orc.w2tau(G, mom, beta, ntau)
    got = ctx.FourierTransform(G, beta, ntau, moments=mom)
    assert rel_err(got, ref) < TOL


@pytest.mark.parametrize("direct", [False, True])
def test_ft_t_to_w(ctx, orc, direct):
    beta, nf, ntau = 10.0, 128, 1024
    G = _two_pole(nf, beta, 3, seed=2)
    gt, _ = orc.fourier(G, beta, ntau, green_asym=True)
    ref, st = orc.tau2w(gt, beta, nf)
    got = ctx.FT_t_to_w(gt, beta, nf, direct=direct)
    assert st == 0 and rel_err(got, ref) < TOL


def test_ft_t_to_w_fft_against_exact_integral(ctx):
    """The FFT form of FT_t_to_w against the 40-digit evaluation in tests/golden/tau2w_exact.npz (white noise
    on 256 tau points): it reaches FP64 rounding (1e-14), while the per-segment form of the reference, run by
    the direct path, carries the cancellation error of its a/w^2 and tau/w terms."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "tau2w_exact.npz"))
    ft, beta, nf, exact = z["ft"], float(z["beta"]), int(z["nfreq"]), z["w"]
    fft = ctx.FT_t_to_w(ft, beta, nf, allow_causality=True)
    direct = ctx.FT_t_to_w(ft, beta, nf, allow_causality=True, direct=True)
    e_fft, e_dir = rel_err(fft, exact), rel_err(direct, exact)
    assert e_fft < 1e-14, e_fft
    assert e_dir < 1e-10, e_dir


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("kanamori", [False, True])
def test_getstimp(ctx, orc, kanamori, mixed):
    """FP64 and double-float (mixed) getStimp against the oracle; the double-float sums carry ~1e-14 relative
    rounding per term."""
    beta, nf, ntau = 10.0, 96, 128
    d = 6 if kanamori else 2
    G = _two_pole(nf, beta, d, seed=3)
    gt, _ = orc.fourier(G, beta, ntau, green_asym=True)
    gt = (gt + np.conj(np.swapaxes(gt, 1, 2))) / 2      # exactly Hermitian, as the reference asserts
    uidx, ut = orc.gen_uijkl(d, 4.0, 2.6, 0.7, density_density=not kanamori)
    ref, _, st = orc.sigma2_tau(gt, uidx, ut, beta)
    got = ctx.getStimp(gt, uidx, ut, beta, allow_hermiticity=(st != 0), mixed=mixed)
    assert rel_err(got, ref) < TOL


def test_fock_dyson_occ_asymto(ctx, orc):
    beta, nf, d = 10.0, 200, 3
    rng = np.random.default_rng(4)
    occ = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    occ = (occ + occ.conj().T) / 4 + 0.5 * np.eye(d)
    uidx, ut = orc.gen_uijkl(d, 3.0, 2.0, 0.5)
    assert rel_err(ctx.getFockOperator(occ, uidx, ut), orc.fock(occ, uidx, ut)) < TOL
    G = _two_pole(nf, beta, d, seed=6)
    delta = 0.2 * G
    himp = np.diag([0.1, -0.2, 0.3]).astype(complex)
    fk = orc.fock(occ, uidx, ut)
    s2 = 0.05 * G
    ref, st = orc.dyson(himp, delta, fk, s2, 0.4, beta)
    got = ctx.getGwimp(himp, delta, fk, s2, 0.4, beta, allow_causality=(st != 0))
    assert rel_err(got, ref) < TOL
    assert rel_err(ctx.getoccMat(ref, beta), orc.occ(ref, beta)) < TOL
    F = np.zeros((nf + 3, d, d), complex)
    F[:nf] = ref
    F[nf] = np.eye(d)
    for order in (1, 2, 3):
        r = orc.estimate_asymto(F, nf, beta, order)
        g = ctx.estimate_asymto(F, nf, beta, order)
        assert rel_err(g[nf + order - 1], r[nf + order - 1]) < TOL


def test_ipt_matches_oracle(ctx, orc):
    wl = models.hubbard_2d(kx=8, ky=8, nfreq=128, beta=10.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    mu, U = 0.0, wl.extra["U"]
    gw, _, num = orc.greenftn_w(H, wl.sigma, mu, wl.beta, 1, 2)
    himp = H.mean(0)
    delta = orc.hyb_delta([0, 1], wl.sigma, gw, himp, mu, wl.beta)
    uidx, ut = orc.gen_uijkl(2, U, U, 0.0, density_density=True)
    himp_dc = himp - 0.5 * U * np.eye(2)            # nominal double counting of the example input
    ntau = 4 * wl.nfreq
    se, gi, nm, st = orc.ipt(himp_dc, delta, num, uidx, ut, U, mu, wl.beta, ntau)
    assert st == 0
    g_se, g_gi, g_nm = ctx.IPT(himp_dc, delta, num, uidx, ut, U, mu, wl.beta, ntau)
    nf = wl.nfreq
    assert rel_err(g_se[:nf + 3], se[:nf + 3]) < TOL
    assert rel_err(g_gi[:nf], gi[:nf]) < TOL
    assert rel_err(g_gi[nf + 1:nf + 4], gi[nf + 1:nf + 4]) < 1e-9
    assert rel_err(g_nm, nm) < TOL


def _dmft_setup(orc, nfreq=64, kx=8, beta=10.0):
    wl = models.hubbard_2d(kx=kx, ky=kx, nfreq=nfreq, beta=beta)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    U = wl.extra["U"]
    uidx, ut = orc.gen_uijkl(2, U, U, 0.0, density_density=True)
    p = dict(ntau=4 * nfreq, n_electrons=1.0, U=U, Uprime=U, J=0.0, mixing=0.5, magnetism=0, dctype=1,
             nominal_charge=1.0, uidx=uidx, ut=ut)
    # the first TightBinding call of dmft_main (src/dmft_main.cpp:300)
    mu, _ = orc.adjust_mu(H, wl.sigma, 0.0, wl.beta, 1, 2, 1.0)
    gloc, _, num = orc.greenftn_w(H, wl.sigma, mu, wl.beta, 1, 2)
    weiss = orc.hyb_delta([0, 1], wl.sigma, gloc, H[:, :2, :2].mean(0), mu, wl.beta)
    state = dict(selfe=wl.sigma.copy(), weiss=weiss, nummat=num, mu=mu, beta=wl.beta, gloc=gloc)
    return wl, H, p, state


def test_dmft_iterations_match_oracle(ctx, orc):
    """Nine dmft_main iterations (IPT, Pulay with the DIIS step from iteration 8, bisection mu) on the device
    against the oracle composition."""
    import torch
    from dmftpack_gb300 import lib
    wl, H, p, state = _dmft_setup(orc)
    dev = torch.device("cuda:0")
    cm = lambda a: torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(dev)
    Hd, se, we, nm = cm(H), cm(state["selfe"]), cm(state["weiss"]), cm(state["nummat"][None])[0].contiguous()
    gloc_g = cm(state["gloc"])
    mu_g = state["mu"]
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, 2)
    pulay = orc.Pulay()
    for it in range(1, 10):
        state, gloc, gimp, res = orc.dmft_iteration(H, state, p, it, pulay)
        mu_g, gimp_g, res_g = ctx.DMFT_iteration(lat, Hd, p, it, se, we, nm, gloc_g, mu_g)
        torch.cuda.synchronize()
        back = lambda t: np.swapaxes(t.cpu().numpy(), -1, -2)
        assert abs(mu_g - state["mu"]) < 1e-12, it
        assert rel_err(back(se), state["selfe"]) < 1e-9, it
        assert rel_err(back(gloc_g), gloc) < 1e-9, it
        assert rel_err(back(we), state["weiss"]) < 1e-9, it
        assert np.allclose(res_g, res, rtol=1e-6, atol=1e-12), (it, res_g, res)


def _scgf_case(orc, d=4, nfreq=64, ntau=256, beta=10.0, seed=7):
    """A small d-spin-orbital impurity: random Hermitian H_imp, a causal hybridisation Delta(iw) =
    sum_l V_l V_l^H / (iw - e_l), G_imp initialised to the non-interacting G, Kanamori U."""
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    himp = 0.3 * (A + A.conj().T) / 2
    wn = np.pi * (2 * np.arange(nfreq) + 1) / beta
    poles = rng.uniform(-2, 2, size=6)
    weiss = np.zeros((nfreq, d, d), np.complex128)
    for e in poles:
        v = 0.4 * (rng.normal(size=d) + 1j * rng.normal(size=d))
        weiss += np.einsum("i,j->ij", v, v.conj())[None] / (1j * wn[:, None, None] - e)
    mu = 0.2
    g0 = np.linalg.inv((1j * wn[:, None, None] + mu) * np.eye(d)[None] - himp[None] - weiss)
    uidx, ut = orc.gen_uijkl(d, 2.0, 1.4, 0.3)
    return himp, weiss, g0, uidx, ut, mu, beta, ntau


@pytest.mark.parametrize("max_iter,mixed", [(12, False), (2000, False), (12, True), (130, True)])
def test_scgf2_matches_oracle(orc, max_iter, mixed):
    """SCGF2 loop (SC2PT solver) against the oracle composition: 12 loops, and the full run to the reference's
    stopping test (135 loops here, including the Pulay DIIS steps from loop 102).  Both sides start
    mixing_check_outer's memory from zero."""
    himp, weiss, g0, uidx, ut, mu, beta, ntau = _scgf_case(orc)
    se_o, g_o, loops_o = orc.scgf2(himp, weiss, g0, uidx, ut, mu, beta, ntau, 0.5, max_iter=max_iter,
                                   static={"prev": 0.0})
    c2 = lib.Context(0)
    try:
        se, g, loops = c2.SCGF2(himp, weiss, g0, uidx, ut, mu, beta, ntau, 0.5, max_iter=max_iter, mixed=mixed)
    finally:
        c2.close()
    assert loops == loops_o
    assert rel_err(se, se_o) < 1e-9
    assert rel_err(g, g_o) < 1e-9


def test_dmft_iterations_sc2pt_match_oracle(orc):
    """Three dmft_main iterations with the SC2PT solver (SCGF2 from the lattice G_loc, Kanamori U on 10
    spin-orbitals of a seeded 28-orbital d+p model) against the oracle composition."""
    import torch
    wl = models.dp28(k=3, nfreq=48, ntau=192, beta=10.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    D = wl.D
    uidx, ut = orc.gen_uijkl(D, 4.0, 2.6, 0.7)
    ne = wl.n_electrons
    p = dict(solver="SC2PT", ntau=wl.ntau, n_electrons=ne, U=4.0, Uprime=2.6, J=0.7, mixing=0.5, magnetism=0,
             dctype=1, nominal_charge=2.0, uidx=uidx, ut=ut, scgf_max_iter=40)
    mu, _ = orc.adjust_mu(H, wl.sigma, 0.0, wl.beta, 1, D, ne)
    gloc, _, num = orc.greenftn_w(H, wl.sigma, mu, wl.beta, 1, D)
    weiss = orc.hyb_delta(list(range(D)), wl.sigma, gloc, H[:, :D, :D].mean(0), mu, wl.beta)
    state = dict(selfe=wl.sigma.copy(), weiss=weiss, nummat=num, mu=mu, beta=wl.beta, gloc=gloc)
    dev = torch.device("cuda:0")
    cm = lambda a: torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(dev)
    back = lambda t: np.swapaxes(t.cpu().numpy(), -1, -2)
    Hd, se, we, gl = cm(H), cm(state["selfe"]), cm(state["weiss"]), cm(state["gloc"])
    nm = cm(state["nummat"][None])[0].contiguous()
    mu_g = mu
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, D)
    pulay = orc.Pulay()
    c2 = lib.Context(0)
    try:
        for it in range(1, 4):
            state, gloc, gimp, res = orc.dmft_iteration(H, state, p, it, pulay)
            mu_g, gimp_g, res_g = c2.DMFT_iteration(lat, Hd, p, it, se, we, nm, gl, mu_g)
            torch.cuda.synchronize()
            assert res_g[4] == res[4], it
            assert abs(mu_g - state["mu"]) < 1e-12, it
            assert rel_err(back(gimp_g)[:wl.nfreq], gimp[:wl.nfreq]) < 1e-9, it
            assert rel_err(back(se), state["selfe"]) < 1e-9, it
            assert rel_err(back(gl), gloc) < 1e-9, it
            assert rel_err(back(we), state["weiss"]) < 1e-9, it
            assert np.allclose(res_g, res, rtol=1e-6, atol=1e-12), (it, res_g, res)
    finally:
        c2.close()


@pytest.mark.parametrize("mixed,direct,tol", [(True, False, 1e-9), (False, True, 1e-10)])
def test_dmft_iterations_variants_match_oracle(orc, mixed, direct, tol):
    """Three IPT iterations with the double-float lattice sum and getStimp, and with the reference's direct
    transform sums, against the oracle."""
    import torch
    wl, H, p, state = _dmft_setup(orc)
    dev = torch.device("cuda:0")
    cm = lambda a: torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(dev)
    back = lambda t: np.swapaxes(t.cpu().numpy(), -1, -2)
    Hd, se, we, gl = cm(H), cm(state["selfe"]), cm(state["weiss"]), cm(state["gloc"])
    nm = cm(state["nummat"][None])[0].contiguous()
    mu_g = state["mu"]
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, 2)
    pulay = orc.Pulay()
    c2 = lib.Context(0)
    try:
        for it in range(1, 4):
            state, gloc, gimp, res = orc.dmft_iteration(H, state, p, it, pulay)
            mu_g, gimp_g, res_g = c2.DMFT_iteration(lat, Hd, p, it, se, we, nm, gl, mu_g, mixed=mixed, direct=direct)
            torch.cuda.synchronize()
            assert abs(mu_g - state["mu"]) < 1e-10, it
            assert rel_err(back(se), state["selfe"]) < tol, it
            assert rel_err(back(gl), gloc) < tol, it
            assert rel_err(back(we), state["weiss"]) < tol, it
    finally:
        c2.close()


def test_scgf2_density_density_two_orbitals(orc):
    """SCGF2 with the density-density interaction on 2 spin-orbitals (the IPT model's U list)."""
    himp, weiss, g0, _, _, mu, beta, ntau = _scgf_case(orc, d=2, nfreq=48, ntau=192, seed=3)
    uidx, ut = orc.gen_uijkl(2, 2.5, 2.5, 0.0, density_density=True)
    se_o, g_o, loops_o = orc.scgf2(himp, weiss, g0, uidx, ut, mu, beta, ntau, 0.5, max_iter=40,
                                   static={"prev": 0.0})
    c2 = lib.Context(0)
    try:
        se, g, loops = c2.SCGF2(himp, weiss, g0, uidx, ut, mu, beta, ntau, 0.5, max_iter=40)
    finally:
        c2.close()
    assert loops == loops_o
    assert rel_err(se, se_o) < 1e-9 and rel_err(g, g_o) < 1e-9


@pytest.mark.parametrize("solver", ["HF", "2PT", "SC2PT"])
@pytest.mark.parametrize("d,nfreq,ntau", [(6, 64, 256), (10, 200, 600)])
def test_weak_solver_matches_oracle(orc, solver, d, nfreq, ntau):
    """weak_solver (the low-level solver of the weakly correlated subspace): HF, 2PT (second order from GwHF) and
    SC2PT (from Gw) on a Kanamori U list, FFT (power-of-two N_tau) and direct transform paths."""
    himp, weiss, g0, uidx, ut, mu, beta, _ = _scgf_case(orc, d=d, nfreq=nfreq, seed=d + nfreq)
    rng = np.random.default_rng(d)
    wn = np.pi * (2 * np.arange(nfreq) + 1) / beta
    A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    h2 = 0.2 * (A + A.conj().T) / 2
    ghf = np.linalg.inv((1j * wn[:, None, None] + mu) * np.eye(d)[None] - h2[None] - weiss)
    se_o = orc.weak_solver(solver, g0, ghf, uidx, ut, beta, ntau)
    c2 = lib.Context(0)
    try:
        se = c2.weak_solver(solver, g0, ghf, uidx, ut, beta, ntau)
    finally:
        c2.close()
    assert rel_err(se[:nfreq + 3], se_o[:nfreq + 3]) < 1e-10


@pytest.mark.parametrize("dctype", ["fll", "amf", "nominal_Uprime"])
def test_dmft_iterations_double_counting_types(orc, dctype):
    """Three IPT iterations with the FLL, AMF and nominal-U' double counting (built from the NumMatrix each
    iteration starts from, as dc_for_dmft is in the reference's loop) against the oracle."""
    import torch
    wl, H, p, state = _dmft_setup(orc)
    p = dict(p, dctype={"fll": lib.DC_FLL, "amf": lib.DC_AMF, "nominal_Uprime": lib.DC_NOMINAL | lib.DC_UPRIME}[dctype],
             Uprime=0.8 * p["U"])
    dev = torch.device("cuda:0")
    cm = lambda a: torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(dev)
    back = lambda t: np.swapaxes(t.cpu().numpy(), -1, -2)
    Hd, se, we, gl = cm(H), cm(state["selfe"]), cm(state["weiss"]), cm(state["gloc"])
    nm = cm(state["nummat"][None])[0].contiguous()
    mu_g = state["mu"]
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, 2)
    pulay = orc.Pulay()
    c2 = lib.Context(0)
    try:
        for it in range(1, 4):
            state, gloc, gimp, res = orc.dmft_iteration(H, state, p, it, pulay)
            mu_g, gimp_g, res_g = c2.DMFT_iteration(lat, Hd, p, it, se, we, nm, gl, mu_g)
            torch.cuda.synchronize()
            assert abs(mu_g - state["mu"]) < 1e-12, it
            assert rel_err(back(se), state["selfe"]) < 1e-9, it
            assert rel_err(back(gl), gloc) < 1e-9, it
    finally:
        c2.close()


@pytest.mark.parametrize("solver", ["IPT", "SC2PT"])
def test_dmft_iterations_with_basis_switch(orc, solver):
    """impurityBasisSwitch: the impurity problem solved in the eigenbasis of Re[H_imp + Delta(i w_0)] and rotated
    back, IPT on the 2-spin-orbital model and SC2PT on a 4-spin-orbital block of a seeded lattice, against the oracle
    with the same basis gauge."""
    import torch
    if solver == "IPT":
        wl, H, p, state = _dmft_setup(orc)
        D = 2
    else:
        rng = np.random.default_rng(12)
        n, D, nk, nf, beta = 8, 4, 27, 48, 8.0
        A = rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n))
        H = (A + np.conj(np.swapaxes(A, 1, 2))) / 4
        wn = np.pi * (2 * np.arange(nf) + 1) / beta
        sig = np.zeros((nf, D, D), complex)
        for d in range(D):
            sig[:, d, d] = -0.4j / (wn + 0.6)
        uidx, ut = orc.gen_uijkl(D, 2.0, 1.4, 0.3)
        p = dict(solver="SC2PT", ntau=4 * nf, n_electrons=4.0, U=2.0, Uprime=1.4, J=0.3, mixing=0.5, magnetism=0,
                 dctype=1, nominal_charge=1.0, uidx=uidx, ut=ut, scgf_max_iter=30)
        mu, _ = orc.adjust_mu(H, sig, 0.0, beta, 1, D, 4.0)
        gloc, _, num = orc.greenftn_w(H, sig, mu, beta, 1, D)
        weiss = orc.hyb_delta(list(range(D)), sig, gloc, H[:, :D, :D].mean(0), mu, beta)
        state = dict(selfe=sig.copy(), weiss=weiss, nummat=num, mu=mu, beta=beta, gloc=gloc)

        class W:
            pass
        wl = W()
        wl.n, wl.nk, wl.nfreq, wl.beta = n, nk, nf, beta
    p = dict(p, basis_switch=True)
    dev = torch.device("cuda:0")
    cm = lambda a: torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(dev)
    back = lambda t: np.swapaxes(t.cpu().numpy(), -1, -2)
    Hd, se, we, gl = cm(H), cm(state["selfe"]), cm(state["weiss"]), cm(state["gloc"])
    nm = cm(state["nummat"][None])[0].contiguous()
    mu_g = state["mu"]
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, D)
    pulay = orc.Pulay()
    c2 = lib.Context(0)
    try:
        for it in range(1, 3):
            state, gloc, gimp, res = orc.dmft_iteration(H, state, p, it, pulay)
            mu_g, gimp_g, res_g = c2.DMFT_iteration(lat, Hd, p, it, se, we, nm, gl, mu_g)
            torch.cuda.synchronize()
            assert abs(mu_g - state["mu"]) < 1e-10, it
            assert rel_err(back(se), state["selfe"]) < 1e-9, it
            assert rel_err(back(gl), gloc) < 1e-9, it
            assert rel_err(back(gimp_g)[:wl.nfreq], gimp[:wl.nfreq]) < 1e-9, it
    finally:
        c2.close()
