"""GPU parity of the lattice stage (H(k), G_loc, N(mu), mu search, Delta, moments) against the FP64 oracle.
Every call goes through the C ABI (libdmftgpu.so via ctypes)."""
import numpy as np
import pytest

from conftest import rel_err
from dmftpack_gb300 import lib, models

pytestmark = pytest.mark.gpu

TOL = 1e-10   # relative, plain FP64 path vs FP64 oracle
TOL_MIXED = 1e-9   # double-float (split-precision) path vs FP64 oracle


def _setup(orc, wl):
    km = orc.kmesh(*wl.kgrid)
    H = orc.hk(wl.n, wl.rindex, wl.hr, km)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, wl.ncl, wl.nh)
    return H, lat


def test_hk_matches_oracle(ctx, orc):
    wl = models.t2g_p(k=5, nfreq=16)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    Hg = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid)
    assert rel_err(Hg, H) < 1e-13
    import torch
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=torch.device("cuda:0"))
    assert rel_err(Hd.cpu().numpy(), H) < 1e-13


@pytest.mark.parametrize("case", ["t2g_p", "dp28", "soc56", "hubbard"])
def test_hk_tensor_cores_match_oracle(ctx, orc, case):
    """H(k) as a tcgen05 GEMM (bf16 slices, exact level sums): k counts and 2 n^2 that are not multiples of the
    128 x 48 tile, N_R = 9 .. 729, against the FP64 oracle at the plain form's tolerance; a second call reuses
    the cached phase image."""
    wl = {"t2g_p": lambda: models.t2g_p(k=5, nfreq=8), "dp28": lambda: models.dp28(k=3, nfreq=8, ntau=16),
          "soc56": lambda: models.soc56(k=3, nfreq=8), "hubbard": lambda: models.hubbard_2d(kx=11, ky=13, nfreq=8)}[case]()
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    for _ in range(2):
        Ht = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, mixed=True)
        assert rel_err(Ht, H) < TOL


@pytest.mark.parametrize("green", [False, True])
def test_moments_match_oracle(ctx, orc, green):
    wl = models.t2g_p(k=2, nfreq=200, beta=20.0)
    F = wl.sigma if not green else np.linalg.inv(1j * wl.wn()[:, None, None] * np.eye(3)[None]
                                                   - 0.3 * np.eye(3)[None] - wl.sigma)
    m_o = orc.moments(F, wl.beta, green_asym=green)
    m_g = ctx.getAsymto_moments(F, wl.beta, greenFtnAsym=green)
    for i in range(4):
        assert np.abs(m_g[i] - m_o[i]).max() <= 1e-9 * max(1.0, np.abs(m_o[i]).max()), i


CASES = {
    "t2g_p": lambda: models.t2g_p(k=4, nfreq=40, beta=12.0),
    "hubbard": lambda: models.hubbard_2d(kx=8, ky=8, nfreq=48, beta=10.0),
}


@pytest.mark.parametrize("explicit", [False, True])
@pytest.mark.parametrize("case", list(CASES))
def test_greenftn_w_matches_oracle(ctx, orc, case, explicit):
    wl = CASES[case]()
    H, lat = _setup(orc, wl)
    mu = 0.25
    gw, gwhf, num = orc.greenftn_w(H, wl.sigma, mu, wl.beta, wl.ncl, wl.nh)
    g_gw, g_gwhf, g_num = ctx.GreenFtn_w(lat, H, wl.sigma, mu, explicit=explicit)
    assert rel_err(g_gw, gw) < TOL
    assert rel_err(g_gwhf, gwhf) < TOL
    assert rel_err(g_num, num) < TOL


def test_greenftn_w_device_pointers(ctx, orc):
    import torch
    wl = CASES["t2g_p"]()
    H, lat = _setup(orc, wl)
    gw, gwhf, num = orc.greenftn_w(H, wl.sigma, 0.1, wl.beta, wl.ncl, wl.nh)
    dev = torch.device("cuda:0")
    g_gw, g_gwhf, g_num = ctx.GreenFtn_w(lat, torch.from_numpy(H).to(dev), torch.from_numpy(wl.sigma).to(dev), 0.1)
    torch.cuda.synchronize()
    assert rel_err(g_gw.cpu().numpy(), gw) < TOL
    assert rel_err(g_num.cpu().numpy(), num) < TOL


@pytest.mark.parametrize("explicit", [False, True])
@pytest.mark.parametrize("n,D,hartr", [(5, 2, [3, 1]), (7, 3, None), (3, 1, [2]), (16, 5, None), (9, 9, None)])
def test_greenftn_w_padding_and_hartree_index(ctx, orc, n, D, hartr, explicit):
    """Odd sizes (identity padding to the next instantiated N) and a HartrIndex that is not the identity."""
    rng = np.random.default_rng(n * 10 + D)
    nk, nf, beta = 27, 32, 8.0
    A = rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n))
    H = (A + np.conj(np.swapaxes(A, 1, 2))) / 2
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    S = np.zeros((nf, D, D), complex)
    for d in range(D):
        S[:, d, d] = 0.2 - 0.7j / (wn + 0.5)
    h = np.arange(D) if hartr is None else np.array(hartr)
    lat = lib.Lattice(n, nk, nf, beta, 1, D, hartr=h)
    gw, gwhf, num = orc.greenftn_w(H, S, -0.3, beta, 1, D, hartr=h)
    g_gw, g_gwhf, g_num = ctx.GreenFtn_w(lat, H, S, -0.3, explicit=explicit)
    assert rel_err(g_gw, gw) < TOL and rel_err(g_gwhf, gwhf) < TOL and rel_err(g_num, num) < TOL
    N, dN = orc.nele(H, S, -0.3, beta, 1, D, hartr=h, deriv=True)
    gN, gdN = ctx.GiwToNele(lat, H, S, -0.3, deriv=True, explicit=explicit)
    assert abs(gN - N) < 1e-11 * max(1, abs(N)) and abs(gdN - dN) < 1e-9 * abs(dN)


@pytest.mark.parametrize("n,D,hartr", [(5, 2, [3, 1]), (7, 3, None), (12, 3, None), (16, 5, None), (9, 9, None),
                                        (28, 10, None)])
def test_explicit_mixed_matches_oracle(ctx, orc, n, D, hartr):
    """The reference's own algorithm (an explicit n x n inversion of every (k, iw) matrix, src/GreenFtn.cpp:245-261)
    in double-float on the FP32 pipe (DMFTGPU_EXPLICIT | DMFTGPU_MIXED): G_loc, GwHF, NumMatrix, N and dN/dmu."""
    rng = np.random.default_rng(n * 7 + D)
    nk, nf, beta = 27, 32, 8.0
    A = rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n))
    H = (A + np.conj(np.swapaxes(A, 1, 2))) / 2
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    S = np.zeros((nf, D, D), complex)
    for d in range(D):
        S[:, d, d] = 0.2 - 0.7j / (wn + 0.5)
    S[:, 0, D - 1] = S[:, D - 1, 0] = 0.05 if D > 1 else 0
    h = np.arange(D) if hartr is None else np.array(hartr)
    lat = lib.Lattice(n, nk, nf, beta, 1, D, hartr=h)
    gw, gwhf, num = orc.greenftn_w(H, S, -0.3, beta, 1, D, hartr=h)
    g_gw, g_gwhf, g_num = ctx.GreenFtn_w(lat, H, S, -0.3, explicit=True, mixed=True)
    assert rel_err(g_gw, gw) < TOL_MIXED and rel_err(g_gwhf, gwhf) < TOL_MIXED and rel_err(g_num, num) < TOL_MIXED
    N, dN = orc.nele(H, S, -0.3, beta, 1, D, hartr=h, deriv=True)
    gN, gdN = ctx.GiwToNele(lat, H, S, -0.3, deriv=True, explicit=True, mixed=True)
    assert abs(gN - N) < 1e-10 * max(1, abs(N)) and abs(gdN - dN) < 1e-9 * abs(dN)


def test_large_orbital_count_schur_only(ctx, orc):
    """n = 56 with a 20-orbital correlated block (beyond the explicit kernels' register budget)."""
    rng = np.random.default_rng(5)
    n, D, nk, nf, beta = 56, 20, 8, 24, 5.0
    A = rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n))
    H = (A + np.conj(np.swapaxes(A, 1, 2))) / 4
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    S = np.zeros((nf, D, D), complex)
    for d in range(D):
        S[:, d, d] = -0.4j / (wn + 0.7)
    lat = lib.Lattice(n, nk, nf, beta, 1, D)
    gw, gwhf, num = orc.greenftn_w(H, S, 0.1, beta, 1, D)
    g_gw, g_gwhf, g_num = ctx.GreenFtn_w(lat, H, S, 0.1)
    assert rel_err(g_gw, gw) < TOL and rel_err(g_gwhf, gwhf) < TOL and rel_err(g_num, num) < TOL


def test_two_clusters(ctx, orc):
    rng = np.random.default_rng(11)
    n, nk, nf, beta, ncl, nh = 8, 16, 32, 6.0, 2, 2
    A = rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n))
    H = (A + np.conj(np.swapaxes(A, 1, 2))) / 2
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    S = np.zeros((nf, 4, 4), complex)
    for d in range(4):
        S[:, d, d] = -0.3j / (wn + 1)
    lat = lib.Lattice(n, nk, nf, beta, ncl, nh)
    gw, gwhf, num = orc.greenftn_w(H, S, 0.0, beta, ncl, nh)
    for explicit in (False, True):
        g_gw, g_gwhf, g_num = ctx.GreenFtn_w(lat, H, S, 0.0, explicit=explicit)
        assert rel_err(g_gw, gw) < TOL and rel_err(g_num, num) < TOL
        N = orc.nele(H, S, 0.0, beta, ncl, nh)
        assert abs(ctx.GiwToNele(lat, H, S, 0.0, explicit=explicit) - N) < 1e-11 * abs(N)


@pytest.mark.parametrize("explicit", [False, True])
@pytest.mark.parametrize("case", list(CASES))
def test_nele_matches_oracle(ctx, orc, case, explicit):
    wl = CASES[case]()
    H, lat = _setup(orc, wl)
    for mu in (-0.5, 0.25):
        N, dN = orc.nele(H, wl.sigma, mu, wl.beta, wl.ncl, wl.nh, deriv=True)
        gN, gdN = ctx.GiwToNele(lat, H, wl.sigma, mu, deriv=True, explicit=explicit)
        assert abs(gN - N) < 1e-11 * max(1, abs(N))
        assert abs(gdN - dN) < 1e-9 * abs(dN)


def test_adjust_mu_bisection_matches_oracle_and_newton_converges(ctx, orc):
    wl = CASES["t2g_p"]()
    H, lat = _setup(orc, wl)
    target = 7.3
    mu_o, ne_o = orc.adjust_mu(H, wl.sigma, 0.0, wl.beta, wl.ncl, wl.nh, target)
    mu_g, ne_g = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, target)
    assert ne_g == ne_o and abs(mu_g - mu_o) <= 1e-12
    mu_x, ne_x = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, target, explicit=True)
    assert ne_x == ne_o and abs(mu_x - mu_o) <= 1e-12
    mu_n, ne_n = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, target, newton=True)
    assert abs(mu_n - mu_o) < 2e-5
    assert abs(orc.nele(H, wl.sigma, mu_n, wl.beta, wl.ncl, wl.nh) - target) < 1e-9
    assert ne_n < ne_o


@pytest.mark.parametrize("newton", [False, True])
def test_adjust_mu_reports_singular_inversion(ctx, newton):
    """A zero pivot inside the mu search is reported as SINGULAR by both search modes (the reference would
    carry inf/nan on silently).  Flat band H(k) = 0 and Sigma(i w_0) = mu0 + i w_0 make z - H - Sigma exactly
    zero at the first frequency for the first mu evaluated."""
    nk, nf, beta, mu0 = 8, 16, 10.0, 0.3
    H = np.zeros((nk, 1, 1), complex)
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    S = (-0.5j / (wn + 1.0)).reshape(nf, 1, 1).astype(complex)
    S[0, 0, 0] = complex(mu0, np.pi / beta)
    lat = lib.Lattice(1, nk, nf, beta, 1, 1)
    with pytest.raises(lib.DmftGpuError) as e:
        ctx.GreenFtn_w_adjust_mu(lat, H, S, mu0, 1.0, 0.5, newton=newton)
    assert e.value.code == lib.SINGULAR




@pytest.mark.parametrize("n,D,nf", [(12, 4, 40), (16, 6, 33), (20, 8, 48), (28, 10, 64), (19, 9, 40), (40, 10, 24),
                                    (11, 5, 16)])
def test_nele_tensor_cores_match_oracle(ctx, orc, n, D, nf):
    """N(mu) with the pole sums on the tensor cores (bf16 slices, exact top levels) and the inversions in
    double-float: block widths 4 .. 10 (padded ones included), m = n - D up to 30, frequency counts that leave a
    partial 32-frequency tile.  Against the FP64 oracle with a diagonal Sigma, and, with an off-diagonal Sigma
    element added, against the GPU's FP64 and CUDA-core double-float passes (the same tail moments on every path:
    for that Sigma the moment fit's window choice compares variances that are equal up to rounding, so the
    oracle may pick another window)."""
    rng = np.random.default_rng(100 * n + D)
    nk, beta = 27, 8.0
    A = rng.normal(size=(nk, n, n)) + 1j * rng.normal(size=(nk, n, n))
    H = (A + np.conj(np.swapaxes(A, 1, 2))) / 3
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    S = np.zeros((nf, D, D), complex)
    for d in range(D):
        S[:, d, d] = 0.1 * d - 0.6j / (wn + 0.4)
    lat = lib.Lattice(n, nk, nf, beta, 1, D)
    for mu in (-0.4, 0.3):
        N = orc.nele(H, S, mu, beta, 1, D)
        gN = ctx.GiwToNele(lat, H, S, mu, mixed=True)
        assert abs(gN - N) < TOL_MIXED * max(1.0, abs(N)), (gN, N)
    S[:, 0, 1] = S[:, 1, 0] = 0.05 / (1j * wn + 1.0)
    for mu in (-0.4, 0.3):
        gF = ctx.GiwToNele(lat, H, S, mu)
        gN = ctx.GiwToNele(lat, H, S, mu, mixed=True)
        gC = ctx.GiwToNele(lat, H, S, mu, mixed=True, tensor=False)
        assert abs(gN - gF) < 1e-11 * max(1.0, abs(gF)), (gN, gF)
        assert abs(gC - gF) < 1e-11 * max(1.0, abs(gF)), (gC, gF)


def test_newton_mu_through_tensor_core_passes(ctx, orc):
    """The mixed Newton mu search on the 28-orbital d+p model (D = 10): its secant passes run on the tensor cores;
    the mu it returns gives the target occupation in the FP64 oracle."""
    wl = models.dp28(k=3, nfreq=64, ntau=256, beta=10.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, wl.D)
    mu_n, ne = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, wl.n_electrons, newton=True, mixed=True)
    assert abs(orc.nele(H, wl.sigma, mu_n, wl.beta, 1, wl.D) - wl.n_electrons) < 1e-9
    mu_c, _ = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, wl.n_electrons, newton=True, mixed=True,
                                       tensor=False)
    assert abs(mu_n - mu_c) < 1e-9


@pytest.mark.parametrize("case", list(CASES))
def test_mixed_precision_lattice_sum(ctx, orc, case):
    wl = CASES[case]()
    H, lat = _setup(orc, wl)
    gw, gwhf, num = orc.greenftn_w(H, wl.sigma, 0.25, wl.beta, wl.ncl, wl.nh)
    m_gw, m_gwhf, m_num = ctx.GreenFtn_w(lat, H, wl.sigma, 0.25, mixed=True)
    assert rel_err(m_gw, gw) < TOL_MIXED and rel_err(m_gwhf, gwhf) < TOL_MIXED and rel_err(m_num, num) < TOL_MIXED
    N, dN = orc.nele(H, wl.sigma, 0.25, wl.beta, wl.ncl, wl.nh, deriv=True)
    gN, gdN = ctx.GiwToNele(lat, H, wl.sigma, 0.25, deriv=True, mixed=True)
    assert abs(gN - N) < TOL_MIXED * abs(N) and abs(gdN - dN) < 1e-7 * abs(dN)


def test_mixed_precision_newton_mu(ctx, orc):
    wl = CASES["t2g_p"]()
    H, lat = _setup(orc, wl)
    mu_n, ne = ctx.GreenFtn_w_adjust_mu(lat, H, wl.sigma, 0.0, 1.0, 7.3, newton=True, mixed=True)
    assert abs(orc.nele(H, wl.sigma, mu_n, wl.beta, wl.ncl, wl.nh) - 7.3) < 1e-9
    assert ne <= 8


def test_hyb_delta_matches_oracle(ctx, orc):
    wl = CASES["t2g_p"]()
    H, lat = _setup(orc, wl)
    gw, _, _ = orc.greenftn_w(H, wl.sigma, 0.2, wl.beta, wl.ncl, wl.nh)
    himp = H.mean(0)[:3, :3]
    orb = [0, 1, 2]
    d_o = orc.hyb_delta(orb, wl.sigma, gw, himp, 0.2, wl.beta)
    d_g = ctx.Construct_hyb_delta(orb, wl.sigma, gw, 0.2, wl.beta, himp)
    assert rel_err(d_g, d_o) < TOL


@pytest.mark.parametrize("case", ["t2g_p", "dp28", "soc_small"])
@pytest.mark.parametrize("mixed", [False, True])
def test_retarded_gloc_real_axis(ctx, orc, case, mixed):
    """Real-axis lattice sum (retarded_GreenFtn2 over a qs_spectra energy grid) against explicit inversion."""
    if case == "t2g_p":
        wl = models.t2g_p(k=3, nfreq=8, beta=10.0)
    elif case == "dp28":   # D = 10: the packed 10-lane groups
        wl = models.dp28(k=2, nfreq=8, ntau=16, beta=10.0)
    else:
        wl = models.soc56(k=2, nfreq=8, beta=10.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    lat = lib.Lattice(wl.n, wl.nk, 8, wl.beta, 1, wl.D)
    nE, e0, de, eta, mu = 40, -4.0, 0.2, 0.05, 0.3
    rng = np.random.default_rng(2)
    A = rng.normal(size=(wl.D, wl.D)) + 1j * rng.normal(size=(wl.D, wl.D))
    Es = e0 + de * np.arange(nE)
    # a causal self-energy on the grid: Hermitian static part - i Gamma(E) (PSD)
    sig = 0.1 * (A + A.conj().T)[None] - 1j * (0.2 + 0.05 * Es[:, None, None] ** 2) * np.eye(wl.D)[None]
    g_o, tr_o = orc.retarded_gloc(H, sig, e0, de, eta, mu, wl.D)
    g, tr = ctx.retarded_GreenFtn(lat, H, sig, e0, de, eta, mu, mixed=mixed)
    tol = 1e-9 if mixed else 1e-10
    assert rel_err(g, g_o) < tol
    assert rel_err(tr, tr_o) < tol
