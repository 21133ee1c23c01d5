"""The Newton-Krylov self-energy mixer of dmftgpu_dmft_iteration (DMFTGPU_MIXER_NEWTON_KRYLOV): Newton steps on
the DMFT fixed-point residual F(Sigma) = SE_out(Sigma) - Sigma, solved by GMRES on Jacobian-vector products
whose lattice part comes from the tangent pass (dmftgpu_gloc_jvp).

It must reach the self-consistency test GwRD < 1e-6 (dmft_scf_check's measure, src/dmft_main.cpp:902-1014, with
its threshold tightened from 1e-5) in fewer DMFT iterations than the Pulay mixer (src/pulay.cpp:48-167), and
converge to the same fixed point: the Pulay loop's, on the device and in the oracle."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda:0")


def _cm(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(_dev())


def _back(t):
    return np.swapaxes(t.cpu().numpy(), -1, -2)


def _initial_state(orc, H, sigma, beta, D, n_electrons):
    """The first TightBinding call of dmft_main (src/dmft_main.cpp:300) with the Newton mu."""
    mu, _ = orc.adjust_mu(H, sigma, 0.0, beta, 1, D, n_electrons)
    mu = orc.newton_mu(H, sigma, mu, beta, D, n_electrons)
    gloc, _, num = orc.greenftn_w(H, sigma, mu, beta, 1, D)
    weiss = orc.hyb_delta(list(range(D)), sigma, gloc, H[:, :D, :D].mean(0), mu, beta)
    return dict(selfe=sigma.copy(), weiss=weiss, nummat=num, mu=mu, beta=beta, gloc=gloc)


def _loop(ctx, H, lat, p, init, stop, max_iter, mixed=True):
    """DMFT iterations on the device from `init` until GwRD < stop: (iterations, GwRD history, Jacobian-vector
    products, SelfEnergy_w, mu, G_loc)."""
    import torch
    Hd = _cm(H)
    se, we, gl = _cm(init["selfe"]), _cm(init["weiss"]), _cm(init["gloc"])
    nm = _cm(init["nummat"][None])[0].contiguous()
    mu, hist, jvps = init["mu"], [], 0
    for it in range(1, max_iter + 1):
        mu, _, res = ctx.DMFT_iteration(lat, Hd, p, it, se, we, nm, gl, mu, mixed=mixed, newton=True)
        k, relres, _ = ctx.mixer_stats()
        jvps += k
        if k:
            assert relres < 0.5, (it, k, relres)
        hist.append(float(res[0]))
        if res[0] < stop:
            break
    torch.cuda.synchronize()
    return it, hist, jvps, _back(se), mu, _back(gl)


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def hubbard64(orc):
    """Single-band Hubbard, 64 x 64 k, beta = 50, N_freq = 2048, N_tau = 8192, U = 2, IPT, Sigma seeded
    U^2/(4 iw), half filling."""
    wl = models.hubbard_2d(kx=64, ky=64, beta=50.0, nfreq=2048, ntau=8192)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    U = wl.extra["U"]
    uidx, ut = orc.gen_uijkl(2, U, U, 0.0, density_density=True)
    p = dict(ntau=wl.ntau, n_electrons=1.0, U=U, Uprime=U, J=0.0, mixing=0.5, magnetism=0, dctype=1,
             nominal_charge=1.0, uidx=uidx, ut=ut)
    return wl, H, p, _initial_state(orc, H, wl.sigma, wl.beta, 2, 1.0)


def test_newton_krylov_fewer_iterations_same_fixed_point(ctx, hubbard64):
    wl, H, p, init = hubbard64
    lat = lib.Lattice(wl.n, H.shape[0], wl.nfreq, wl.beta, 1, 2)
    pulay = dict(p, pulay_history=3, pulay_start=3)
    nk = dict(p, mixer="newton_krylov", newton_start=3, pulay_history=3, pulay_start=3)
    it_p, hist_p, jv_p, _, _, _ = _loop(ctx, H, lat, pulay, init, 1e-6, 40)
    it_n, hist_n, jv_n, _, _, _ = _loop(ctx, H, lat, nk, init, 1e-6, 40)
    assert hist_p[-1] < 1e-6 and hist_n[-1] < 1e-6, (hist_p[-3:], hist_n[-3:])
    assert jv_p == 0 and jv_n > 0
    assert it_n < it_p, (it_n, it_p, hist_n, hist_p)
    # both to the rounding floor: the fixed points agree
    _, hp, _, se_p, mu_p, gl_p = _loop(ctx, H, lat, pulay, init, 1e-11, 60)
    _, hn, _, se_n, mu_n, gl_n = _loop(ctx, H, lat, nk, init, 1e-11, 60)
    assert hp[-1] < 1e-11 and hn[-1] < 1e-11, (hp[-3:], hn[-3:])
    assert rel_err(se_n, se_p) < 1e-9 and rel_err(gl_n, gl_p) < 1e-9 and abs(mu_n - mu_p) < 1e-10


def test_newton_krylov_fixed_point_matches_oracle(ctx, orc):
    """FP64 Newton-Krylov on the device against the oracle's Pulay loop (history 3, Newton mu), both converged."""
    wl = models.hubbard_2d(kx=24, ky=24, beta=30.0, nfreq=512, ntau=2048, U=2.5)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    U = wl.extra["U"]
    uidx, ut = orc.gen_uijkl(2, U, U, 0.0, density_density=True)
    p = dict(ntau=wl.ntau, n_electrons=1.0, U=U, Uprime=U, J=0.0, mixing=0.5, magnetism=0, dctype=1,
             nominal_charge=1.0, uidx=uidx, ut=ut)
    init = _initial_state(orc, H, wl.sigma, wl.beta, 2, 1.0)
    state, pul = dict(init), orc.Pulay(3, 3)
    po = dict(p, newton_mu=True)
    for it in range(1, 61):
        state, gloc, gimp, res = orc.dmft_iteration(H, state, po, it, pul)
        if res[0] < 1e-11:
            break
    assert res[0] < 1e-11, res
    lat = lib.Lattice(wl.n, H.shape[0], wl.nfreq, wl.beta, 1, 2)
    nk = dict(p, mixer="newton_krylov", newton_start=3)
    _, hist, jvps, se, mu, gl = _loop(ctx, H, lat, nk, init, 1e-11, 40, mixed=False)
    assert hist[-1] < 1e-11 and jvps > 0, hist
    assert rel_err(se, state["selfe"]) < 1e-9 and rel_err(gl, state["gloc"]) < 1e-9, (rel_err(se, state["selfe"]),)
    assert abs(mu - state["mu"]) < 1e-10


def test_mixer_settings_checked(ctx, hubbard64):
    wl, H, p, init = hubbard64
    lat = lib.Lattice(wl.n, H.shape[0], wl.nfreq, wl.beta, 1, 2)
    Hd = _cm(H)
    se, we, gl = _cm(init["selfe"]), _cm(init["weiss"]), _cm(init["gloc"])
    nm = _cm(init["nummat"][None])[0].contiguous()
    ctx.MIXERS["bogus"] = 7
    try:
        for bad in (dict(p, mixer="bogus"), dict(p, mixer="newton_krylov", krylov_dim=65),
                    dict(p, mixer="newton_krylov", krylov_tol=-1.0)):
            with pytest.raises(lib.DmftGpuError) as e:
                ctx.DMFT_iteration(lat, Hd, bad, 1, se, we, nm, gl, init["mu"])
            assert e.value.code == lib.BADARG
    finally:
        del ctx.MIXERS["bogus"]
    # a rejected call leaves the state untouched
    assert rel_err(_back(se), init["selfe"]) == 0


def test_newton_krylov_sc2pt_dp_model(ctx):
    """The SC2PT workload's model (28-orbital d+p, 10 correlated spin-orbitals, Kanamori U = 4, J = 0.7) on a 4^3 k
    grid with 256 Matsubara points: the fixed-point residual |SE_out - Sigma| / |Sigma| below 1e-8 in fewer
    iterations than Pulay (history 3, Newton mu), at the same fixed point.  (GwRD itself has a floor on this model:
    with magnetism 0 the spin-averaged Sigma of the lattice and the unaveraged G_imp of the solver differ.)"""
    import torch
    wl = models.dp28(k=4, nfreq=256, ntau=1024, beta=40.0)
    D = wl.D
    uidx, ut = models.gen_Uijkl(D, 4.0, 2.6, 0.7)
    p = dict(solver="SC2PT", ntau=wl.ntau, n_electrons=wl.n_electrons, U=4.0, Uprime=2.6, J=0.7, mixing=0.5,
             magnetism=0, dctype=1, nominal_charge=2.0, uidx=uidx, ut=ut, pulay_history=3, pulay_start=3)
    dev = _dev()
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, D)
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
    Hcm = Hd.transpose(-1, -2).contiguous()
    sig = torch.from_numpy(wl.sigma).to(dev)
    mu0, _ = ctx.GreenFtn_w_adjust_mu(lat, Hd, sig, 0.0, 1.0, wl.n_electrons, newton=True)
    gl0, _, nm0 = ctx.GreenFtn_w(lat, Hd, sig, mu0, with_gwhf=False)
    we0 = ctx.Construct_hyb_delta(list(range(D)), sig, gl0, mu0, wl.beta, Hd[:, :D, :D].mean(0))
    t = lambda x: x.transpose(-1, -2).contiguous()
    init = [t(sig), t(we0), t(nm0), t(gl0)]

    def run(q, max_iter):
        se, we, nm, gl = (x.clone() for x in init)
        mu, hist, jv = mu0, [], 0
        for it in range(1, max_iter + 1):
            mu, _, res = ctx.DMFT_iteration(lat, Hcm, q, it, se, we, nm, gl, mu, mixed=True, newton=True)
            k, _, fres = ctx.mixer_stats()
            jv += k
            hist.append(fres)
            if fres < 1e-8:
                break
        torch.cuda.synchronize()
        return it, hist, jv, se.cpu().numpy(), mu

    it_p, h_p, _, se_p, mu_p = run(p, 40)
    it_n, h_n, jv, se_n, mu_n = run(dict(p, mixer="newton_krylov", newton_start=3), 40)
    assert h_p[-1] < 1e-8 and h_n[-1] < 1e-8 and jv > 0, (h_p[-3:], h_n[-3:])
    assert it_n < it_p, (it_n, it_p, h_n, h_p)
    assert rel_err(se_n, se_p) < 1e-7 and abs(mu_n - mu_p) < 1e-8
