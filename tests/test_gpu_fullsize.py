"""GPU parity against the FP64 oracle at the workloads' real frequency and tau sizes, and on the reference's
own example input (example/Hubb_model/primitive_Cell_ipt, via tests/golden/hubbard_example.json).

The toy-size tests elsewhere cover the edge cases; these exercise what only large grids reach: the moment-fit
window search with Nv = N_freq/20 (src/FourierTransform.cpp:289-316), the positivity fix-ups
(src/FourierTransform.cpp:145-175, src/SCGF2_fullLoop.cpp:657-688), the SCGF2 stopping test, and the
lattice sums at N_freq = 2048-4096.  k grids are full where the oracle finishes in seconds (the Hubbard lattice, the
example) and a k subset otherwise (the per-k work is independent of the other k points)."""
import json
import os

import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import hwr, lib, models

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-10        # FP64 path vs FP64 oracle (relative)
TOL_MIXED = 1e-9   # double-float path vs FP64 oracle (relative)


def _dev():
    import torch
    return torch.device("cuda:0")


def _cm(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(_dev())


def _back(t):
    return np.swapaxes(t.cpu().numpy(), -1, -2)


def _oracle_dmft(orc, H, p, state, iters):
    """`iters` dmft_main iterations in the oracle: the initial state and, per iteration, (state, gloc, gimp, res)."""
    pulay = orc.Pulay()
    out = []
    for it in range(1, iters + 1):
        state, gloc, gimp, res = orc.dmft_iteration(H, state, p, it, pulay)
        out.append((state, gloc, gimp, res))
    return out


def _gpu_dmft(H, n, beta, nfreq, p, init, ref, mixed=False, tol=1e-9, mu_tol=1e-12):
    """The same iterations on the device from the same initial state, each compared with the oracle's."""
    import torch
    D = init["selfe"].shape[1]
    Hd, se, we, gl = _cm(H), _cm(init["selfe"]), _cm(init["weiss"]), _cm(init["gloc"])
    nm = _cm(init["nummat"][None])[0].contiguous()
    mu_g = init["mu"]
    lat = lib.Lattice(n, H.shape[0], nfreq, beta, 1, D)
    c2 = lib.Context(0)
    try:
        for it, (state, gloc, gimp, res) in enumerate(ref, start=1):
            mu_g, gimp_g, res_g = c2.DMFT_iteration(lat, Hd, p, it, se, we, nm, gl, mu_g, mixed=mixed)
            torch.cuda.synchronize()
            assert abs(mu_g - state["mu"]) < mu_tol, (it, mu_g, state["mu"])
            assert rel_err(_back(gimp_g)[:nfreq], gimp[:nfreq]) < tol, it
            assert rel_err(_back(se), state["selfe"]) < tol, it
            assert rel_err(_back(gl), gloc) < tol, it
            assert rel_err(_back(we), state["weiss"]) < tol, it
            assert rel_err(_back(nm), state["nummat"]) < tol, it
            assert np.allclose(res_g[:4], res[:4], rtol=1e-6, atol=1e-12), (it, res_g, res)
    finally:
        c2.close()


def _initial_state(orc, H, sigma, beta, D, n_electrons):
    """The first TightBinding call of dmft_main (src/dmft_main.cpp:300): mu search, G_loc, Delta."""
    mu, _ = orc.adjust_mu(H, sigma, 0.0, beta, 1, D, n_electrons)
    gloc, _, num = orc.greenftn_w(H, sigma, mu, beta, 1, D)
    weiss = orc.hyb_delta(list(range(D)), sigma, gloc, H[:, :D, :D].mean(0), mu, beta)
    return dict(selfe=sigma.copy(), weiss=weiss, nummat=num, mu=mu, beta=beta, gloc=gloc)


def reference_example():
    """The reference's Hubbard example: Hk.HWR rows, 22 x 22 x 1 k, beta = 40, 400 Matsubara points, N_tau = 2400
    (not a power of two: the direct transform sums), U = U' = 10, J = 0, IPT, nominal DC with N_d = 1,
    N_ELECTRONS = 1, MIXING = 0.5, MAGNETISM = 0.  SelfEnergy_w starts at zero (ImgFreqFtn::Initialize)."""
    with open(os.path.join(GOLDEN, "hubbard_example.json")) as f:
        fx = json.load(f)
    text = "\n".join(["Norbital of Atom = %d" % m for m in fx["norbital_of_atom"]] +
                     ["%d %d %d %d %d %d %d %.17g %.17g" % tuple(r) for r in fx["hwr_rows"]])
    norb, rindex, hr = hwr.read_hr(text, num_atoms=len(fx["norbital_of_atom"]))
    return fx, sum(norb), rindex, hr


def test_reference_example_ipt_iterations(orc):
    fx, n, rindex, hr = reference_example()
    assert fx["solver_type"] == "IPT" and fx["dc_type"] == "nominal" and fx["magnetism"] == 0 and n == 2
    kx, ky, kz = fx["k_points"]
    beta, nf, ntau = fx["beta"], fx["n_matsubara"], fx["n_tau"]
    H = orc.hk(n, rindex, hr, orc.kmesh(kx, ky, kz))
    uidx, ut = orc.gen_uijkl(2, fx["U"], fx["Uprime"], fx["J"], density_density=True)
    p = dict(solver="IPT", ntau=ntau, n_electrons=fx["n_electrons"], U=fx["U"], Uprime=fx["Uprime"], J=fx["J"],
             mixing=fx["mixing"], magnetism=fx["magnetism"], dctype=1, nominal_charge=fx["n_d"], uidx=uidx, ut=ut)
    init = _initial_state(orc, H, np.zeros((nf, 2, 2), np.complex128), beta, 2, fx["n_electrons"])
    ref = _oracle_dmft(orc, H, p, init, iters=3)
    _gpu_dmft(H, n, beta, nf, p, init, ref)


@pytest.fixture(scope="module")
def hubbard64(orc):
    """Single-band Hubbard, 64 x 64 k, beta = 50, N_freq = 2048, N_tau = 8192 (FFT transforms), U = 2, IPT, Sigma
    seeded U^2/(4 iw): the oracle's initial TightBinding call and one complete DMFT iteration."""
    wl = models.hubbard_2d(kx=64, ky=64, beta=50.0, nfreq=2048, ntau=8192)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    U = wl.extra["U"]
    uidx, ut = orc.gen_uijkl(2, U, U, 0.0, density_density=True)
    p = dict(ntau=wl.ntau, n_electrons=1.0, U=U, Uprime=U, J=0.0, mixing=0.5, magnetism=0, dctype=1,
             nominal_charge=1.0, uidx=uidx, ut=ut)
    init = _initial_state(orc, H, wl.sigma, wl.beta, 2, 1.0)
    return wl, H, p, init, _oracle_dmft(orc, H, p, init, iters=1)


@pytest.mark.parametrize("mixed", [False, True])
def test_hubbard_64x64_full_size_ipt_iteration(hubbard64, mixed):
    """One complete config-1 DMFT iteration on the device, FP64 and double-float, against the oracle."""
    wl, H, p, init, ref = hubbard64
    _gpu_dmft(H, wl.n, wl.beta, wl.nfreq, p, init, ref, mixed=mixed, tol=TOL_MIXED if mixed else 1e-9,
              mu_tol=1e-10 if mixed else 1e-12)


def _k_subset(orc, wl, nsub, stride):
    km = orc.kmesh(*wl.kgrid)[::stride][:nsub]
    return orc.hk(wl.n, wl.rindex, wl.hr, km)


@pytest.mark.parametrize("mixed", [False, True])
def test_t2g_p_k_subset_full_frequencies(ctx, orc, mixed):
    """t2g + p (12 x 12), 64 k points of the 24^3 grid, beta = 40, N_freq = 4096 (8192 points in the sums):
    GreenFtn_w, N(mu) with dN/dmu, and the mu search (bisection: the reference's mu sequence)."""
    wl = models.t2g_p(k=24, nfreq=4096, beta=40.0)
    H = _k_subset(orc, wl, 64, 216)
    lat = lib.Lattice(wl.n, H.shape[0], wl.nfreq, wl.beta, wl.ncl, wl.nh)
    tol = TOL_MIXED if mixed else TOL
    gw, gwhf, num = orc.greenftn_w(H, wl.sigma, 0.1, wl.beta, wl.ncl, wl.nh)
    g, g0, nm = ctx.GreenFtn_w(lat, H, wl.sigma, 0.1, mixed=mixed)
    assert rel_err(g, gw) < tol and rel_err(g0, gwhf) < tol and rel_err(nm, num) < tol
    if not mixed:
        g, g0, nm = ctx.GreenFtn_w(lat, H, wl.sigma, 0.1, explicit=True)
        assert rel_err(g, gw) < TOL and rel_err(g0, gwhf) < TOL and rel_err(nm, num) < TOL
    N, dN = orc.nele(H, wl.sigma, 0.1, wl.beta, wl.ncl, wl.nh, deriv=True)
    gN, gdN = ctx.GiwToNele(lat, H, wl.sigma, 0.1, deriv=True, mixed=mixed)
    assert abs(gN - N) < tol * abs(N) and abs(gdN - dN) < 1e-7 * abs(dN)
    target = 8.0
    mu_o, ne_o = orc.adjust_mu(H, wl.sigma, 0.0, wl.beta, wl.ncl, wl.nh, target)
    mu_g, ne_g = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, target, mixed=mixed)
    if not mixed:
        assert ne_g == ne_o and abs(mu_g - mu_o) <= 1e-12
    else:
        assert abs(mu_g - mu_o) <= 1e-9
    mu_n, _ = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, target, newton=True, mixed=mixed)
    assert abs(orc.nele(H, wl.sigma, mu_n, wl.beta, wl.ncl, wl.nh) - target) < 1e-9


def test_soc56_k_subset_dense_sigma(ctx, orc):
    """56 x 56 SOC model with a dense 20 x 20 Sigma, 8 k points of the 16^3 grid, beta = 30, N_freq = 2048."""
    wl = models.soc56(k=16, nfreq=2048, beta=30.0)
    H = _k_subset(orc, wl, 8, 512)
    lat = lib.Lattice(wl.n, H.shape[0], wl.nfreq, wl.beta, 1, wl.D)
    gw, gwhf, num = orc.greenftn_w(H, wl.sigma, 0.0, wl.beta, 1, wl.D)
    for mixed, tol in ((False, TOL), (True, TOL_MIXED)):
        g, g0, nm = ctx.GreenFtn_w(lat, H, wl.sigma, 0.0, mixed=mixed)
        assert rel_err(g, gw) < tol and rel_err(g0, gwhf) < tol and rel_err(nm, num) < tol, mixed
    N, dN = orc.nele(H, wl.sigma, 0.0, wl.beta, 1, wl.D, deriv=True)
    gN, gdN = ctx.GiwToNele(lat, H, wl.sigma, 0.0, deriv=True)
    assert abs(gN - N) < 1e-11 * abs(N) and abs(gdN - dN) < 1e-9 * abs(dN)


def _kanamori_impurity(d=10, nfreq=4096, beta=40.0, seed=11):
    """A seeded d-spin-orbital impurity with the SC2PT workload's sizes: Hermitian H_imp, a causal
    hybridisation sum_l V_l V_l^H / (iw - e_l) over 8 poles, G_imp initialised to the non-interacting G."""
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    himp = 0.3 * (A + A.conj().T) / 2
    wn = np.pi * (2 * np.arange(nfreq) + 1) / beta
    weiss = np.zeros((nfreq, d, d), np.complex128)
    for e in rng.uniform(-3, 3, size=8):
        v = 0.4 * (rng.normal(size=d) + 1j * rng.normal(size=d))
        weiss += np.einsum("i,j->ij", v, v.conj())[None] / (1j * wn[:, None, None] - e)
    mu = 0.5
    g0 = np.linalg.inv((1j * wn[:, None, None] + mu) * np.eye(d)[None] - himp[None] - weiss)
    return himp, weiss, g0, mu


@pytest.fixture(scope="module")
def scgf2_d10(orc):
    himp, weiss, g0, mu = _kanamori_impurity()
    uidx, ut = orc.gen_uijkl(10, 4.0, 2.6, 0.7)
    ref = orc.scgf2(himp, weiss, g0, uidx, ut, mu, 40.0, 8192, 0.5, max_iter=3, static={"prev": 0.0})
    return (himp, weiss, g0, uidx, ut, mu), ref


@pytest.mark.parametrize("mixed", [False, True])
def test_kanamori_d10_impurity_scgf2_loops(scgf2_d10, mixed):
    """SCGF2 on the 10 spin-orbital Kanamori impurity (U = 4, J = 0.7, U' = 2.6, Nu = 180) at N_freq = 4096,
    N_tau = 8192, beta = 40: three loops, FP64 and double-float getStimp."""
    (himp, weiss, g0, uidx, ut, mu), (se_o, g_o, loops_o) = scgf2_d10
    c2 = lib.Context(0)
    try:
        se, g, loops = c2.SCGF2(himp, weiss, g0, uidx, ut, mu, 40.0, 8192, 0.5, max_iter=3, mixed=mixed)
    finally:
        c2.close()
    assert loops == loops_o == 3
    tol = TOL_MIXED if mixed else 1e-9
    assert rel_err(se, se_o) < tol and rel_err(g, g_o) < tol


@pytest.mark.parametrize("mixed", [False, True])
def test_ragged_batch_against_oracle(ctx, orc, mixed):
    """The ragged batch's shapes (n in {1,3,5,10,14,28}, N_freq in {512..4096}, beta in [10,100]) through the
    batched entry point, each problem against the oracle on 27 of its k points."""
    import torch
    dev = _dev()
    wls = models.batched_uneven(nprob=64)
    picked, seen = [], set()
    for w in wls:                                    # one problem per (n, N_freq) pair present in the batch
        if (w.n, w.nfreq) not in seen:
            seen.add((w.n, w.nfreq))
            picked.append(w)
    assert {w.n for w in picked} == {1, 3, 5, 10, 14, 28} and max(w.nfreq for w in picked) == 4096
    tcm = lambda t: t.transpose(-1, -2).contiguous()
    lats, Hs, Ss, G, G0, N, mus, Hn = [], [], [], [], [], [], [], []
    for w in picked:
        km = orc.kmesh(*w.kgrid)[::max(1, w.nk // 27)][:27]
        H = orc.hk(w.n, w.rindex, w.hr, km)
        Hn.append(H)
        lats.append(lib.Lattice(w.n, H.shape[0], w.nfreq, w.beta, 1, w.D))
        Hs.append(tcm(torch.from_numpy(H).to(dev)))
        Ss.append(tcm(torch.from_numpy(w.sigma).to(dev)))
        G.append(torch.zeros((w.nfreq, w.D, w.D), dtype=torch.complex128, device=dev))
        G0.append(torch.zeros_like(G[-1]))
        N.append(torch.zeros((w.D, w.D), dtype=torch.complex128, device=dev))
        mus.append(0.05 * w.n - 0.3)
    ctx.GreenFtn_w_batched(lats, Hs, Ss, mus, G, G0, N, mixed=mixed)
    torch.cuda.synchronize()
    tol = TOL_MIXED if mixed else TOL
    for i, w in enumerate(picked):
        gw, gwhf, num = orc.greenftn_w(Hn[i], w.sigma, mus[i], w.beta, 1, w.D)
        back = lambda t: t.transpose(-1, -2).cpu().numpy()
        assert rel_err(back(G[i]), gw) < tol, (i, w.n, w.nfreq)
        assert rel_err(back(G0[i]), gwhf) < tol, (i, w.n, w.nfreq)
        assert rel_err(back(N[i]), num) < tol, (i, w.n, w.nfreq)
