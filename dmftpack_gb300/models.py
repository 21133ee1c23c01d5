"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Each builder returns a :class:`Workload`: the tight-binding table in read_HR form (rindex, hr), the k grid,
beta, N_freq, N_tau, the correlated-space layout and an initial self-energy SelfE_w[N_freq, D, D].
All randomness comes from numpy's PCG64 with a fixed seed per workload.
"""
from dataclasses import dataclass, field

import numpy as np

PI = 3.1415926535897932384626


@dataclass
class Workload:
    name: str
    n: int
    rindex: np.ndarray
    hr: np.ndarray
    kgrid: tuple
    beta: float
    nfreq: int
    ntau: int
    ncl: int
    nh: int
    sigma: np.ndarray
    n_electrons: float
    extra: dict = field(default_factory=dict)

    @property
    def nk(self):
        return self.kgrid[0] * self.kgrid[1] * self.kgrid[2]

    @property
    def D(self):
        return self.ncl * self.nh

    def wn(self):
        return PI * (2 * np.arange(self.nfreq) + 1) / self.beta


def _hermitian_hoppings(n, rvecs, draw, onsite):
    """t(R) for every R in rvecs with t(-R) = t(R)^H; draw(R) -> n x n complex for one of each +-R pair."""
    rows, vals = [], []
    seen = {}
    for R in rvecs:
        R = tuple(int(x) for x in R)
        if R in seen:
            continue
        mR = tuple(-x for x in R)
        if R == (0, 0, 0):
            t = draw(R)
            t = (t + t.conj().T) / 2 + np.diag(onsite)
            seen[R] = t
        else:
            t = draw(R)
            seen[R] = t
            seen[mR] = t.conj().T
    for R, t in seen.items():
        for i in range(n):
            for j in range(n):
                if t[i, j] != 0:
                    rows.append((R[0], R[1], R[2], i, j))
                    vals.append(t[i, j])
    return np.asarray(rows, np.int32), np.asarray(vals, np.complex128)


def hubbard_2d(kx=64, ky=64, beta=50.0, nfreq=2048, ntau=None, U=2.0, t=1.0, tp=-0.25):
    """Single-band Hubbard model on the square lattice, 2 spin-orbitals (Norbital of Atom = 2):
    H(k) = -2t(cos kx + cos ky) - 4t' cos kx cos ky, Sigma(iw) = U^2/(4 iw), half filling (N = 1)."""
    rows, vals = [], []
    for s in range(2):
        for R in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0)]:
            rows.append(R + (s, s))
            vals.append(-t)
        for R in [(1, 1, 0), (1, -1, 0), (-1, 1, 0), (-1, -1, 0)]:
            rows.append(R + (s, s))
            vals.append(-tp)
    wn = PI * (2 * np.arange(nfreq) + 1) / beta
    sigma = np.zeros((nfreq, 2, 2), np.complex128)
    for s in range(2):
        sigma[:, s, s] = U * U / (4 * 1j * wn)
    return Workload("hubbard2d", 2, np.asarray(rows, np.int32), np.asarray(vals, np.complex128), (kx, ky, 1), beta,
                    nfreq, ntau if ntau else 4 * nfreq, 1, 2, sigma, 1.0, {"U": U})


def t2g_p(k=24, beta=40.0, nfreq=4096, ntau=None, seed=20250102, rmax=2):
    """3 t2g (on-site 0 eV) + 9 O-p (on-site -3 eV) orbitals, 12 x 12 complex Hermitian H(k) with seeded
    hoppings t(R) ~ N(0,1)/|R|^2 (complex) for |R_i| <= 2 (125 R vectors); Sigma is a diagonal 3 x 3 block
    on the d orbitals with Im Sigma = -0.5/(w_n + 1)."""
    n = 12
    rng = np.random.default_rng(seed)
    rvecs = [(a, b, c) for a in range(-rmax, rmax + 1) for b in range(-rmax, rmax + 1) for c in range(-rmax, rmax + 1)]

    def draw(R):
        r2 = max(1, R[0] ** 2 + R[1] ** 2 + R[2] ** 2)
        return (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(2) / r2

    onsite = np.array([0.0] * 3 + [-3.0] * 9)
    rows, vals = _hermitian_hoppings(n, rvecs, draw, onsite)
    wn = PI * (2 * np.arange(nfreq) + 1) / beta
    sigma = np.zeros((nfreq, 3, 3), np.complex128)
    for d in range(3):
        sigma[:, d, d] = -0.5j / (wn + 1.0)
    return Workload("t2g_p", n, rows, vals, (k, k, k), beta, nfreq, ntau if ntau else 2 * nfreq, 1, 3, sigma, 8.0)


def dp28(k=32, beta=40.0, nfreq=4096, ntau=8192, seed=20250105, rmax=4, U=4.0, J=0.7):
    """d+p model of dimension 28 (5 d x 2 spins correlated + 18 ligand spin-orbitals), seeded t(R) over
    |R_i| <= 4 (729 R vectors) with 1/|R|^2 decay; Sigma is a diagonal 10 x 10 block.  Kanamori U=4, J=0.7,
    U' = U - 2J."""
    n = 28
    rng = np.random.default_rng(seed)
    rvecs = [(a, b, c) for a in range(-rmax, rmax + 1) for b in range(-rmax, rmax + 1) for c in range(-rmax, rmax + 1)]

    def draw(R):
        r2 = max(1, R[0] ** 2 + R[1] ** 2 + R[2] ** 2)
        return (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(2) / (2 * r2)

    onsite = np.array([0.0] * 10 + [-3.0] * 18)
    rows, vals = _hermitian_hoppings(n, rvecs, draw, onsite)
    wn = PI * (2 * np.arange(nfreq) + 1) / beta
    sigma = np.zeros((nfreq, 10, 10), np.complex128)
    for d in range(10):
        sigma[:, d, d] = -0.5j / (wn + 1.0)
    return Workload("dp28", n, rows, vals, (k, k, k), beta, nfreq, ntau, 1, 10, sigma, 20.0,
                    {"U": U, "J": J, "Up": U - 2 * J})


def _ls_d():
    """L.S for l = 2 on (m, spin) pairs ordered (m = -2..2) x (up, down), spin-orbital index 2*m_idx + spin."""
    ms = np.arange(-2, 3)
    Lz = np.diag(ms).astype(complex)
    Lp = np.zeros((5, 5), complex)
    for i, m in enumerate(ms[:-1]):
        Lp[i + 1, i] = np.sqrt(2 * 3 - m * (m + 1))  # <m+1|L+|m> = sqrt(l(l+1) - m(m+1)), l = 2
    Lm = Lp.conj().T
    sz = np.diag([0.5, -0.5]).astype(complex)
    sp = np.array([[0, 1], [0, 0]], complex)
    sm = sp.T.copy()
    return np.kron(Lz, sz) + 0.5 * (np.kron(Lp, sm) + np.kron(Lm, sp))


def soc56(k=16, beta=30.0, nfreq=2048, ntau=None, seed=20250103, rmax=3, lam=0.1):
    """Two correlated sites with spin-orbit coupling: 2 x 5 d + 6 x 3 p = 28 orbitals x 2 spins = 56 x 56
    complex Hermitian H(k) (spin-orbital index 2*orbital + spin, the d orbitals of both sites first), seeded
    spin-independent t(R) over |R_i| <= 3 (343 R vectors) with 1/|R|^2 decay, on-site d at 0 and p at -3 eV,
    SOC lam L.S on each site's d shell; Sigma is a dense 20 x 20 block M0 + M1/(iw) with random Hermitian M0 and
    positive semidefinite M1 (causal)."""
    norb = 28
    n = 2 * norb
    rng = np.random.default_rng(seed)
    rvecs = [(a, b, c) for a in range(-rmax, rmax + 1) for b in range(-rmax, rmax + 1) for c in range(-rmax, rmax + 1)]

    def draw(R):
        r2 = max(1, R[0] ** 2 + R[1] ** 2 + R[2] ** 2)
        t = (rng.normal(size=(norb, norb)) + 1j * rng.normal(size=(norb, norb))) / np.sqrt(2) / (2 * r2)
        return np.kron(t, np.eye(2))

    onsite = np.repeat(np.array([0.0] * 10 + [-3.0] * 18), 2)
    rows, vals = _hermitian_hoppings(n, rvecs, draw, onsite)
    soc = lam * _ls_d()
    extra_r, extra_v = [], []
    for site in range(2):
        o = 10 * site
        for i in range(10):
            for j in range(10):
                if soc[i, j] != 0:
                    extra_r.append((0, 0, 0, o + i, o + j))
                    extra_v.append(soc[i, j])
    rows = np.concatenate([rows, np.asarray(extra_r, np.int32)])
    vals = np.concatenate([vals, np.asarray(extra_v, np.complex128)])
    D = 20
    A = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
    M0 = 0.2 * (A + A.conj().T) / 2
    Bm = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
    M1 = 0.1 * Bm @ Bm.conj().T / D
    wn = PI * (2 * np.arange(nfreq) + 1) / beta
    sigma = M0[None] + M1[None] / (1j * wn[:, None, None])
    return Workload("soc56", n, rows, vals, (k, k, k), beta, nfreq, ntau if ntau else 2 * nfreq, 1, D, sigma, 40.0,
                    {"M0": M0, "M1": M1})


def batched_uneven(nprob=64, seed=20250104, dims=(1, 3, 5, 10, 14, 28), kgrids=(8, 12, 16, 24, 32),
                   nfreqs=(512, 1024, 2048, 4096), beta_range=(10.0, 100.0), dmax=10):
    """Independent lattice problems of ragged sizes: orbital dimension from `dims`, k grid k^3 from `kgrids`,
    beta uniform in `beta_range`, N_freq from `nfreqs`; seeded random Hermitian nearest-cell t(R) scaled to a
    bandwidth of ~4 eV; Sigma diagonal on the correlated block (the first min(n, dmax) orbitals, a d shell) with
    Im Sigma = -Gamma/(w_n + Gamma), Gamma ~ U(0.1, 1)."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(nprob):
        n = int(rng.choice(dims))
        k = int(rng.choice(kgrids))
        nf = int(rng.choice(nfreqs))
        beta = float(rng.uniform(*beta_range))
        rvecs = [(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)]
        scale = 4.0 / (2 * 27 * np.sqrt(n))

        def draw(R):
            return scale * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))

        rows, vals = _hermitian_hoppings(n, rvecs, draw, rng.uniform(-1, 1, size=n))
        D = min(n, dmax)
        gam = rng.uniform(0.1, 1.0, size=D)
        wn = PI * (2 * np.arange(nf) + 1) / beta
        sigma = np.zeros((nf, D, D), np.complex128)
        for d in range(D):
            sigma[:, d, d] = -1j * gam[d] / (wn + gam[d])
        out.append(Workload("uneven%d" % p, n, rows, vals, (k, k, k), beta, nf, 2 * nf, 1, D, sigma, n / 2.0))
    return out


def gen_Uijkl(n_spinorb, U, Uprime, JH, density_density=False):
    """Interaction list (U_index (nu, 4) int32, U_tensor (nu,) complex) for H_int = 1/2 sum U_ijkl c+_i c+_j c_l c_k
    on spin-orbitals ordered (orbital, spin) = (i // 2, i % 2): gen_Uijkl (Slater-Kanamori: density-density,
    spin-flip and pair-hopping terms, src/gen_Uijkl.cpp:9-58) or gen_Uijkl_density_density (all (n, m, n, m),
    src/gen_Uijkl.cpp:60-87).  Entries come in the reference's (i, j, k, l) loop order."""
    n = int(n_spinorb)
    if density_density:
        a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        a, b = a.ravel(), b.ravel()
        v = np.where(a // 2 == b // 2, U, Uprime) - np.where(a % 2 == b % 2, JH, 0.0)
        return np.stack([a, b, a, b], 1).astype(np.int32), v.astype(np.complex128)
    i, j, k, l = (x.ravel() for x in np.meshgrid(*(np.arange(n),) * 4, indexing="ij"))
    io, jo, ko, lo = i // 2, j // 2, k // 2, l // 2
    is_, js, ks, ls = i % 2, j % 2, k % 2, l % 2
    dd = (i == k) & (j == l)
    flip = (ko == io) & (lo == jo) & (ko != lo) & (ks != is_) & (ls != js) & (ks != ls)
    pair = (ko == lo) & (ko != io) & (io == jo) & (ks != ls) & (ks == is_) & (ls == js)
    c = np.where(dd, np.where(io == jo, U, Uprime) - np.where(is_ == js, JH, 0.0),
                 np.where(flip | pair, JH, 0.0))
    keep = c != 0
    return np.stack([i, j, k, l], 1)[keep].astype(np.int32), c[keep].astype(np.complex128)
