"""ctypes binding of the CPU FP64 oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg and
reference arm, always as the checker or the timed CPU baseline, never by the product package.

Parity status: unpinned against the reference program (see dmft_oracle.cpp's header).

All arrays are numpy complex128 stacks of column-major matrices: a numpy array of shape (count, n, n)
whose element [c, j, i] is matrix c's entry (i, j) -- i.e. the Fortran-ordered matrices stacked in C order.
Use :func:`to_cm` / :func:`from_cm` to convert from/to ordinary (count, i, j) arrays.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
# host threads of the k sums (GreenFtn_w, GiwToNele, H(k)) and of the transforms; ORACLE_THREADS overrides
NTHREADS = int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1))

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Lattice(C.Structure):
    _fields_ = [("n", C.c_int), ("nk", C.c_int), ("nfreq", C.c_int), ("beta", C.c_double),
                ("ncl", C.c_int), ("nh", C.c_int), ("hartr", _ip)]


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "dmft_oracle.cpp")):
            build()
        _lib = C.CDLL(_LIB_PATH)
        _lib.orc_nele.argtypes = [C.POINTER(Lattice), _dp, _dp, C.c_double, _dp, _dp, C.c_int]
        _lib.orc_greenftn_w.argtypes = [C.POINTER(Lattice), _dp, _dp, C.c_double, _dp, _dp, _dp, C.c_int]
        _lib.orc_adjust_mu.argtypes = [C.POINTER(Lattice), _dp, _dp, C.c_double, C.c_double, C.c_double,
                                       _dp, _ip, C.c_int]
        _lib.orc_w2tau_single.argtypes = [C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_double, _dp]
        _lib.orc_hyb_delta.argtypes = [C.c_int, _ip, C.c_int, C.c_double, C.c_int, _dp, _dp, _dp, C.c_double,
                                       _dp]
        _lib.orc_dyson.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp]
        _lib.orc_ipt.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp,
                                 C.c_int, _ip, _dp, _dp, _dp, _dp]
        _lib.orc_moments.argtypes = [C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp]
        _lib.orc_w2tau.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, _ip]
        _lib.orc_fourier.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp, _dp, _ip]
        _lib.orc_tau2w.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp]
        _lib.orc_sigma2_tau.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, _ip, _dp, _dp, _dp, _ip]
        _lib.orc_fock.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp, _dp]
        _lib.orc_estimate_asymto.argtypes = [C.c_int, C.c_int, C.c_double, _dp, C.c_int]
        _lib.orc_occ.argtypes = [C.c_int, C.c_int, C.c_double, _dp, _dp]
        _lib.orc_gen_uijkl.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _ip, _dp]
        _lib.orc_hk.argtypes = [C.c_int, C.c_int, _ip, _dp, C.c_int, _dp, _dp, C.c_int]
        _lib.orc_kmesh.argtypes = [C.c_int, C.c_int, C.c_int, _dp]
        _lib.orc_kmesh.restype = None
        _lib.orc_fock.restype = None
        _lib.orc_estimate_asymto.restype = None
        _lib.orc_hermitian_eig.argtypes = [C.c_int, _dp, _dp, _dp]
        _lib.orc_inverse.argtypes = [C.c_int, _dp, _dp]
        _lib.orc_set_threads.argtypes = [C.c_int]
        _lib.orc_set_threads.restype = None
        _lib.orc_set_threads(NTHREADS)
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def to_cm(a):
    """(count, i, j) complex -> column-major stack (count, j, i), contiguous complex128."""
    a = np.asarray(a, dtype=np.complex128)
    return np.ascontiguousarray(np.swapaxes(a, -1, -2))


def from_cm(a):
    return np.ascontiguousarray(np.swapaxes(a, -1, -2))


def _lat(n, nk, nfreq, beta, ncl, nh, hartr):
    h = np.ascontiguousarray(hartr, dtype=np.int32)
    L = Lattice(n, nk, nfreq, beta, ncl, nh, _i(h))
    L._keep = h
    return L


def _check(st, what, allowed=(0,)):
    if st not in allowed:
        raise RuntimeError(f"oracle {what} returned status {st}")
    return st


def kmesh(kx, ky, kz):
    out = np.zeros((kx * ky * kz, 3))
    lib().orc_kmesh(kx, ky, kz, _d(out))
    return out


def hk(n, rindex, hr, km, nthreads=None):
    """rindex: (nnz,5) int (Rx,Ry,Rz,i0,j0); hr: (nnz,) complex; returns (nk, n, n) H(k) (i,j order)."""
    nthreads = nthreads or NTHREADS
    rindex = np.ascontiguousarray(rindex, dtype=np.int32)
    hr = np.ascontiguousarray(hr, dtype=np.complex128)
    km = np.ascontiguousarray(km, dtype=np.float64)
    out = np.zeros((km.shape[0], n, n), np.complex128)
    _check(lib().orc_hk(n, rindex.shape[0], _i(rindex), _d(hr.view(np.float64)), km.shape[0], _d(km),
                        _d(out.view(np.float64)), nthreads), "hk")
    return from_cm(out)


def hermitian_eig(a):
    a = np.asarray(a, np.complex128)
    n = a.shape[0]
    w = np.zeros(n)
    v = np.zeros((n, n), np.complex128)
    am = to_cm(a)
    st = lib().orc_hermitian_eig(n, _d(am.view(np.float64)), _d(w), _d(v.view(np.float64)))
    return w, from_cm(v), st


def inverse(a):
    a = np.asarray(a, np.complex128)
    n = a.shape[0]
    out = np.zeros((n, n), np.complex128)
    st = lib().orc_inverse(n, _d(to_cm(a).view(np.float64)), _d(out.view(np.float64)))
    return from_cm(out), st


def moments(fw, beta, green_asym=False):
    fw = to_cm(fw)
    nf, dim = fw.shape[0], fw.shape[1]
    out = np.zeros((4, dim, dim), np.complex128)
    _check(lib().orc_moments(dim, nf, beta, _d(fw.view(np.float64)), int(green_asym), _d(out.view(np.float64))),
           "moments")
    return from_cm(out)


def greenftn_w(hk_, sigma, mu, beta, ncl, nh, hartr=None, nthreads=None):
    """GreenFtn_w: hk_ (nk,n,n), sigma (nfreq,D,D); returns (Gw, GwHF, NumMatrix)."""
    nthreads = nthreads or NTHREADS
    hk_c = to_cm(hk_)
    s_c = to_cm(sigma)
    nk, n = hk_c.shape[0], hk_c.shape[1]
    nf, D = s_c.shape[0], ncl * nh
    if hartr is None:
        hartr = np.arange(D)
    L = _lat(n, nk, nf, beta, ncl, nh, hartr)
    gw = np.zeros((nf, D, D), np.complex128)
    gwhf = np.zeros_like(gw)
    num = np.zeros((D, D), np.complex128)
    _check(lib().orc_greenftn_w(C.byref(L), _d(hk_c.view(np.float64)), _d(s_c.view(np.float64)), mu,
                                _d(gw.view(np.float64)), _d(gwhf.view(np.float64)), _d(num.view(np.float64)),
                                nthreads), "greenftn_w")
    return from_cm(gw), from_cm(gwhf), from_cm(num)


def nele(hk_, sigma, mu, beta, ncl, nh, hartr=None, nthreads=None, deriv=False):
    nthreads = nthreads or NTHREADS
    hk_c = to_cm(hk_)
    s_c = to_cm(sigma)
    nk, n = hk_c.shape[0], hk_c.shape[1]
    nf, D = s_c.shape[0], ncl * nh
    if hartr is None:
        hartr = np.arange(D)
    L = _lat(n, nk, nf, beta, ncl, nh, hartr)
    N = C.c_double()
    dN = C.c_double()
    _check(lib().orc_nele(C.byref(L), _d(hk_c.view(np.float64)), _d(s_c.view(np.float64)), mu, C.byref(N),
                          C.byref(dN) if deriv else None, nthreads), "nele")
    return (N.value, dN.value) if deriv else N.value


def adjust_mu(hk_, sigma, mu, beta, ncl, nh, n_target, dmu=1.0, hartr=None, nthreads=None):
    nthreads = nthreads or NTHREADS
    hk_c = to_cm(hk_)
    s_c = to_cm(sigma)
    nk, n = hk_c.shape[0], hk_c.shape[1]
    nf, D = s_c.shape[0], ncl * nh
    if hartr is None:
        hartr = np.arange(D)
    L = _lat(n, nk, nf, beta, ncl, nh, hartr)
    out = C.c_double()
    ne = C.c_int()
    _check(lib().orc_adjust_mu(C.byref(L), _d(hk_c.view(np.float64)), _d(s_c.view(np.float64)), mu, dmu,
                               n_target, C.byref(out), C.byref(ne), nthreads), "adjust_mu")
    return out.value, ne.value


def hyb_delta(orb, sigma, gw, himp, mu, beta):
    orb = np.ascontiguousarray(orb, np.int32)
    s_c, g_c, h_c = to_cm(sigma), to_cm(gw), to_cm(himp[None])[0]
    nf, D = s_c.shape[0], s_c.shape[1]
    dim = orb.shape[0]
    out = np.zeros((nf, dim, dim), np.complex128)
    _check(lib().orc_hyb_delta(dim, _i(orb), nf, beta, D, _d(s_c.view(np.float64)), _d(g_c.view(np.float64)),
                               _d(h_c.view(np.float64)), mu, _d(out.view(np.float64))), "hyb_delta")
    return from_cm(out)


def w2tau(fw, mom, beta, ntau):
    f_c, m_c = to_cm(fw), to_cm(mom)
    nf, dim = f_c.shape[0], f_c.shape[1]
    out = np.zeros((ntau + 1, dim, dim), np.complex128)
    fix = C.c_int()
    _check(lib().orc_w2tau(dim, nf, ntau, beta, _d(f_c.view(np.float64)), _d(m_c.view(np.float64)),
                           _d(out.view(np.float64)), C.byref(fix)), "w2tau")
    return from_cm(out), fix.value


def fourier(fw, beta, ntau, green_asym=False, m1=None):
    f_c = to_cm(fw)
    nf, dim = f_c.shape[0], f_c.shape[1]
    out = np.zeros((ntau + 1, dim, dim), np.complex128)
    fix = C.c_int()
    m1p = None
    if m1 is not None:
        m1c = to_cm(np.asarray(m1)[None])[0]
        m1p = _d(m1c.view(np.float64))
    _check(lib().orc_fourier(dim, nf, ntau, beta, _d(f_c.view(np.float64)), int(green_asym), m1p,
                             _d(out.view(np.float64)), C.byref(fix)), "fourier")
    return from_cm(out), fix.value


def tau2w(ft, beta, nfreq):
    t_c = to_cm(ft)
    ntau, dim = t_c.shape[0] - 1, t_c.shape[1]
    out = np.zeros((nfreq, dim, dim), np.complex128)
    st = lib().orc_tau2w(dim, nfreq, ntau, beta, _d(t_c.view(np.float64)), _d(out.view(np.float64)))
    return from_cm(out), st


def sigma2_tau(gt, uidx, ut, beta):
    g_c = to_cm(gt)
    ntau, dim = g_c.shape[0] - 1, g_c.shape[1]
    uidx = np.ascontiguousarray(uidx, np.int32)
    ut = np.ascontiguousarray(ut, np.complex128)
    out = np.zeros((ntau + 1, dim, dim), np.complex128)
    fix = C.c_int()
    st = lib().orc_sigma2_tau(dim, ntau, beta, uidx.shape[0], _i(uidx), _d(ut.view(np.float64)),
                              _d(g_c.view(np.float64)), _d(out.view(np.float64)), C.byref(fix))
    return from_cm(out), fix.value, st


def fock(occ, uidx, ut):
    dim = occ.shape[0]
    uidx = np.ascontiguousarray(uidx, np.int32)
    ut = np.ascontiguousarray(ut, np.complex128)
    out = np.zeros((dim, dim), np.complex128)
    lib().orc_fock(dim, uidx.shape[0], _i(uidx), _d(ut.view(np.float64)), _d(to_cm(occ[None])[0].view(np.float64)),
                   _d(out.view(np.float64)))
    return from_cm(out)


def dyson(himp, delta, fk, s2, mu, beta):
    d_c, s_c = to_cm(delta), to_cm(s2)
    nf, dim = d_c.shape[0], d_c.shape[1]
    out = np.zeros((nf, dim, dim), np.complex128)
    st = lib().orc_dyson(dim, nf, beta, mu, _d(to_cm(himp[None])[0].view(np.float64)), _d(d_c.view(np.float64)),
                         _d(to_cm(fk[None])[0].view(np.float64)), _d(s_c.view(np.float64)),
                         _d(out.view(np.float64)))
    return from_cm(out), st


def estimate_asymto(f, nfreq, beta, order):
    """f: (nfreq+3, dim, dim) stack; returns a copy with slot nfreq+order-1 written."""
    f_c = to_cm(f)
    dim = f_c.shape[1]
    lib().orc_estimate_asymto(dim, nfreq, beta, _d(f_c.view(np.float64)), order)
    return from_cm(f_c)


def occ(gw, beta):
    g_c = to_cm(gw)
    nf, dim = g_c.shape[0], g_c.shape[1]
    out = np.zeros((dim, dim), np.complex128)
    _check(lib().orc_occ(dim, nf, beta, _d(g_c.view(np.float64)), _d(out.view(np.float64))), "occ")
    return from_cm(out[None])[0]


def gen_uijkl(nso, U, Up, J, density_density=False):
    cap = nso ** 4
    uidx = np.zeros((cap, 4), np.int32)
    ut = np.zeros(cap, np.complex128)
    cnt = lib().orc_gen_uijkl(nso, U, Up, J, int(density_density), cap, _i(uidx), _d(ut.view(np.float64)))
    return uidx[:cnt].copy(), ut[:cnt].copy()


def ipt(himp, delta, nummat, uidx, ut, U, mu, beta, ntau):
    d_c = to_cm(delta)
    nf, dim = d_c.shape[0], d_c.shape[1]
    uidx = np.ascontiguousarray(uidx, np.int32)
    ut = np.ascontiguousarray(ut, np.complex128)
    se = np.zeros((nf + 5, dim, dim), np.complex128)
    gi = np.zeros((nf + 5, dim, dim), np.complex128)
    nm = np.zeros((dim, dim), np.complex128)
    st = lib().orc_ipt(dim, nf, ntau, beta, U, mu, _d(to_cm(himp[None])[0].view(np.float64)),
                       _d(d_c.view(np.float64)), _d(to_cm(nummat[None])[0].view(np.float64)), uidx.shape[0],
                       _i(uidx), _d(ut.view(np.float64)), _d(se.view(np.float64)), _d(gi.view(np.float64)),
                       _d(nm.view(np.float64)))
    return from_cm(se), from_cm(gi), from_cm(nm[None])[0], st


# ---------------------------------------------------------------------------------------------------------
# Pulay mixer and one DMFT iteration, composed from the functions above (numpy restatement of the glue)
# ---------------------------------------------------------------------------------------------------------
class Pulay:
    """pulayMixing(mixing_history, start_mixing, ...) with parallel_pulay (src/pulay.cpp:11-167)."""

    def __init__(self, hist=2, start=5):
        self.h, self.start = hist, start
        self.inp = None
        self.om = np.zeros((hist + 1, hist + 1))
        for k in range(hist):
            self.om[hist, k] = -1
            self.om[k, hist] = -1
            self.om[hist - 1, hist - 1] = -100.0
        self.om[hist, hist] = 0.0

    def mixing(self, inp, out, mix, it, step=1):
        h = self.h
        if self.inp is None:
            self.inp = [np.zeros_like(inp) for _ in range(h)]
            self.res = [np.zeros_like(inp) for _ in range(h)]
        rc = h - 1
        for k in range(rc, 0, -1):
            self.inp[k] = self.inp[k - 1].copy()
            self.res[k] = self.res[k - 1].copy()
        self.inp[0] = inp.copy()
        self.res[0] = out - inp
        if it > self.start:
            idx = [k if k < rc else k + 1 for k in range(h - 1)]
            tmp = self.om[np.ix_(idx, idx)].copy()
            self.om[1:h, 1:h] = tmp
            for k in range(h):
                g = float(np.sum(np.real(np.conj(self.res[0]) * self.res[k])))
                self.om[0, k] = g
                self.om[k, 0] = g
        use = False
        if it > h + self.start and it % step == 0:
            use = np.linalg.matrix_rank(self.om) == h + 1
        if use:
            rhs = np.zeros(h + 1)
            rhs[h] = -1
            beta = np.linalg.solve(self.om, rhs)
            opt = sum(beta[k] * self.inp[k] for k in range(h))
            optr = sum(beta[k] * self.res[k] for k in range(h))
        else:
            opt, optr = inp, self.res[0]
        return opt + mix * optr


def matsubara_norm2(f, beta):
    """MatsubaraFtnnorm squared (src/SCGF2_fullLoop.cpp:791-805): sum_n ||f_n||_F^2 / w_n."""
    wn = np.pi * (2 * np.arange(f.shape[0]) + 1) / beta
    return float(np.sum(np.sum(np.abs(f) ** 2, axis=(1, 2)) / wn))


def scgf2(himp, weiss, gimp_init, uidx, ut, mu, beta, ntau, mixing, max_iter=2000, static=None):
    """SCGF2 (src/SCGF2_fullLoop.cpp:392-533) composed from the functions above.  weiss, gimp_init: nfreq
    slots.  static: dict carrying mixing_check_outer's function-static previous residual across calls
    (:722-727).  Returns (SE_out[nfreq+5], Gwimp_out[nfreq+5], loops)."""
    if static is None:
        static = {"prev": 0.0}
    nf, d = weiss.shape[0], weiss.shape[1]
    eye = np.eye(d, dtype=np.complex128)
    G = np.array(gimp_init[:nf], np.complex128)
    occ_m = occ(G, beta)
    unit = np.sqrt(matsubara_norm2(G, beta))
    loop, n_out, n_occ, mix = 0, 0.0, 0.0, mixing / 10.0
    pul = Pulay(2, 100)
    s2 = np.zeros((nf + 3, d, d), np.complex128)
    F = np.zeros((d, d), np.complex128)
    while (loop < 10 or n_out > 1e-6 or n_occ > 1e-6) and loop < max_iter:
        Gin, occ_in = G.copy(), occ_m.copy()
        occ_m = occ(G, beta)
        F = fock(occ_m, uidx, ut)
        gt, _ = fourier(G, beta, ntau, True, eye)
        st, _, stat = sigma2_tau(gt, uidx, ut, beta)
        _check(stat, "sigma2_tau")
        s2w, stat = tau2w(st, beta, nf)
        _check(stat, "tau2w")
        s2[:nf] = s2w
        G, stat = dyson(himp, weiss, F, s2[:nf], mu, beta)
        _check(stat, "dyson")
        occ_m = occ(G, beta)
        n_occ = float(np.linalg.norm(occ_m - occ_in))
        n_out = np.sqrt(matsubara_norm2(Gin - G, beta)) / unit
        if loop % 500 == 0:
            mix /= 1.5
        if loop < 1500:
            G = pul.mixing(Gin, G, mix, loop)
        else:
            G = (1 - mix) * Gin + mix * G
        if loop % 10 == 0:
            if static["prev"] > n_out:
                mix = min(1.07 * mix, 0.5)
            elif static["prev"] < n_out:
                mix = max(mix / 1.09, 1e-3)
            static["prev"] = n_out
        loop += 1
    s2 = estimate_asymto(s2, nf, beta, 1)
    s2 = estimate_asymto(s2, nf, beta, 2)
    se = np.zeros((nf + 5, d, d), np.complex128)
    se[:nf] = s2[:nf] + F
    se[nf] = F
    se[nf + 1] = s2[nf]
    se[nf + 2] = s2[nf + 1]
    go = np.zeros((nf + 5, d, d), np.complex128)
    go[:nf] = G
    go[nf + 1] = eye
    return se, go, loop


DC_NONE, DC_NOMINAL, DC_FLL, DC_AMF, DC_SIGMA0, DC_UPRIME = 0, 1, 2, 3, 4, 0x100


def double_counting(dctype, natoms, nso, U, Up, J, nominal_charge, nummat=None, sigma0=None, initial=0, dc_prev=None):
    """dc_for_dmft (src/dmft_main.cpp:593-707): the (natoms nso) x (natoms nso) double-counting matrix.  dctype:
    DC_NOMINAL / DC_FLL (optionally | DC_UPRIME: averU = U'), DC_AMF, DC_SIGMA0 (with initial: the previous DC plus
    Re Tr Sigma(i w_0) / nso per atom, :606-618; else FLL)."""
    base, uprime = dctype & 0xFF, bool(dctype & DC_UPRIME)
    N = natoms * nso
    out = np.zeros((N, N), np.complex128)
    averU = (nso * U + nso * (nso - 1) * Up) / (nso * nso)
    for at in range(natoms):
        o = at * nso
        if nummat is not None:
            up = sum(nummat[o + n, o + n].real for n in range(0, nso, 2))
            down = sum(nummat[o + n + 1, o + n + 1].real for n in range(0, nso, 2) if n + 1 < nso)
        if base == DC_SIGMA0 and initial:
            temp = sum(sigma0[o + i, o + i].real for i in range(nso)) / nso
            out[o:o + nso, o:o + nso] = dc_prev[o:o + nso, o:o + nso] + temp * np.eye(nso)
        elif base in (DC_FLL, DC_SIGMA0):
            u = Up if uprime else averU
            for i in range(0, nso, 2):
                out[o + i, o + i] = u * (down + up - 0.5) - J * (up - 0.5)
                out[o + i + 1, o + i + 1] = u * (down + up - 0.5) - J * (down - 0.5)
        elif base == DC_AMF:
            n0 = (down + down) / nso  # as written at :653
            for i in range(nso):
                out[o + i, o + i] = averU * n0 * (nso - 1) - J * n0 * (nso // 2 - 1)
        elif base == DC_NOMINAL:
            u = Up if uprime else averU
            v = u * (nominal_charge - 0.5) - J * (nominal_charge / 2.0 - 0.5)
            for i in range(0, nso, 2):
                out[o + i, o + i] = v
                out[o + i + 1, o + i + 1] = v
    return out


def _eigh_gauged(a):
    """numpy eigh with eigenvalues ascending and each eigenvector's first component of largest modulus made real
    and positive."""
    w, v = np.linalg.eigh(a)
    for j in range(v.shape[1]):
        mags = np.abs(v[:, j]) ** 2
        big = 0
        for i in range(len(mags)):
            if mags[i] > mags[big] * (1 + 1e-12):
                big = i
        v[:, j] *= np.conj(v[big, j]) / abs(v[big, j])
    return w, v


def impurity_basis(himp, delta0, magnetism=0):
    """proj_to_site's solver basis for impurityBasisSwitch (src/SOLVER.cpp:541-586) from H_imp - DC and
    Delta(i w_0), with the eigenvector gauge of _eigh_gauged."""
    n = himp.shape[0]
    B = np.zeros((n, n), np.complex128)
    if np.linalg.norm(himp.imag) < 1e-5 and magnetism in (0, 1) and n % 2 == 0:
        M = 0.5 * (delta0[0::2, 0::2] + delta0[1::2, 1::2]) + 0.5 * (himp[0::2, 0::2] + himp[1::2, 1::2])
        M = 0.5 * (M + M.conj().T)
        _, v = _eigh_gauged(M.real.astype(np.complex128))
        B[0::2, 0::2] = v.real
        B[1::2, 1::2] = v.real
    else:
        _, V1 = _eigh_gauged(himp)
        X = himp + 0.5 * (delta0 + delta0.conj().T)
        T = (V1.conj().T @ X @ V1).real
        _, v = _eigh_gauged(T.astype(np.complex128))
        B = V1 @ v.real
    return B


def weak_solver(solver, gw, gwhf, uidx, ut, beta, ntau):
    """weak_solver (src/SOLVER.cpp:72-102): "HF" is on_shot_HF (src/SCGF2_fullLoop.cpp:218-250), "2PT" / "SC2PT" is
    SC2PT_weak (src/SCGF2_fullLoop.cpp:49-133) with G0 = gwhf / gw.  gw, gwhf: nfreq slots.  Returns
    SE_out[nfreq+5] (writeResults, src/SCGF2_fullLoop.cpp:696-720)."""
    nf, d = gw.shape[0], gw.shape[1]
    eye = np.eye(d, dtype=np.complex128)
    F = fock(occ(gw, beta), uidx, ut)
    s2 = np.zeros((nf + 3, d, d), np.complex128)
    if solver != "HF":
        g0 = gw if solver == "SC2PT" else gwhf
        gt, _ = fourier(g0, beta, ntau, True, eye)
        st, _, stat = sigma2_tau(gt, uidx, ut, beta)
        _check(stat, "sigma2_tau")
        s2w, stat = tau2w(st, beta, nf)
        _check(stat, "tau2w")
        s2[:nf] = s2w
    s2 = estimate_asymto(s2, nf, beta, 1)
    s2 = estimate_asymto(s2, nf, beta, 2)
    se = np.zeros((nf + 5, d, d), np.complex128)
    se[:nf] = s2[:nf] + F
    se[nf] = F
    se[nf + 1] = s2[nf]
    se[nf + 2] = s2[nf + 1]
    return se


def newton_mu(H, sigma, mu, beta, D, n_target, tol=1e-12, max_iter=50):
    """The root of N(mu) = n_target to |N - n_target| <= tol by Newton steps on dN/dmu from the derivative pass,
    started from mu (the bisection's result): the mu that the library's DMFTGPU_NEWTON search converges to, for the
    DMFT loop's fixed point without the bisection's |dmu| <= 1e-5 resolution (src/GreenFtn.cpp:66-139)."""
    for _ in range(max_iter):
        N, dN = nele(H, sigma, mu, beta, 1, D, deriv=True)
        if abs(N - n_target) <= tol or not dN > 0:
            break
        mu += (n_target - N) / dN
    return mu


def dmft_iteration(H, state, p, it, pulay):
    """The dmft_main loop body for one correlated cluster (the first D orbitals) with IPT (D = 2) or SC2PT
    (SCGF2) (src/dmft_main.cpp:343-570): state = dict(selfe, weiss, nummat, mu, beta, gloc, scgf_static);
    p = dict(solver, ntau, n_electrons, U, Uprime, J, mixing, uidx, ut, nominal_charge, scgf_max_iter, newton_mu).
    Returns (new state, gloc, gimp, residuals[5])."""
    beta = state["beta"]
    nf, D = state["selfe"].shape[0], state["selfe"].shape[1]
    himp = H[:, :D, :D].mean(0)
    dc = double_counting(p.get("dctype", DC_NOMINAL), 1, D, p["U"], p["Uprime"], p["J"], p["nominal_charge"],
                         nummat=state["nummat"])
    loops = 0
    hdc, wS, nS = himp - dc, state["weiss"], state["nummat"]
    B = None
    if p.get("basis_switch"):
        # impurityBasisSwitch (src/SOLVER.cpp:541-595); the results come back at w < N_freq (:426-434)
        B = impurity_basis(hdc, state["weiss"][0], p.get("magnetism", 0))
        hdc = B.conj().T @ hdc @ B
        wS = B.conj().T[None] @ wS @ B[None]
        nS = B.conj().T @ nS @ B
    if p.get("solver", "IPT") == "SC2PT":
        se, gi, loops = scgf2(hdc, wS, state["gloc"], p["uidx"], p["ut"], state["mu"], beta,
                              p["ntau"], p["mixing"], max_iter=p.get("scgf_max_iter", 0) or 2000,
                              static=state.setdefault("scgf_static", {"prev": 0.0}))
        nm = nS.copy()
    else:
        se, gi, nm, st = ipt(hdc, wS, nS, p["uidx"], p["ut"], p["U"], state["mu"], beta, p["ntau"])
        if st != 0:
            raise RuntimeError("oracle IPT status %d" % st)
    if B is not None:
        se[:nf] = B[None] @ se[:nf] @ B.conj().T[None]
        gi[:nf] = B[None] @ gi[:nf] @ B.conj().T[None]
        nm = B @ nm @ B.conj().T
    for M in list(se) + [nm]:
        for n in range(0, D, 2):
            avg = (M[n, n] + M[n + 1, n + 1]) / 2
            M[n, n] = M[n + 1, n + 1] = avg
            M[n, n + 1] = M[n + 1, n] = 0
    nm_imp = nm.copy()
    seout = se[:nf] - dc[None]
    selfe = pulay.mixing(state["selfe"], seout, p["mixing"], it)
    mu, nev = adjust_mu(H, selfe, state["mu"], beta, 1, D, p["n_electrons"])
    if p.get("newton_mu"):
        mu = newton_mu(H, selfe, mu, beta, D, p["n_electrons"])
    gloc, _, nummat = greenftn_w(H, selfe, mu, beta, 1, D)
    weiss = hyb_delta(list(range(D)), selfe, gloc, himp, mu, beta)
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    d2 = np.abs(gi[:nf] - gloc) ** 2
    n2 = np.abs(gloc) ** 2
    low = wn < min(p["U"], 3.0)
    rd_n = d2.sum((1, 2))
    nr_n = n2.sum((1, 2))
    res = [np.sqrt(rd_n.sum() / (1e-10 + nr_n.sum())), np.sqrt(rd_n[low].sum() / (1e-10 + nr_n[low].sum())),
           np.sqrt(np.max(np.concatenate([[0.0], rd_n / (1e-10 + nr_n)]))),
           np.linalg.norm(nummat - nm_imp) / np.linalg.norm(nummat), loops]
    new = dict(state, selfe=selfe, weiss=weiss, nummat=nummat, mu=mu, gloc=gloc)
    return new, gloc, gi, np.array(res)


def retarded_gloc(H, sigma_e, e0, de, eta, mu, D):
    """retarded_GreenFtn2 (src/GreenFtn.cpp:425-466) in the model basis (DF_CorrBase = I) summed over k as qs_spectra
    does: G(k, E_n) = (E_n + mu + i eta - H(k) - Sigma(E_n) on the first D orbitals)^-1 by explicit inversion.
    Returns ((1/N_k) sum_k G_PP, (1/N_k) sum_k Tr G)."""
    nk, n = H.shape[0], H.shape[1]
    nE = sigma_e.shape[0]
    g = np.zeros((nE, D, D), np.complex128)
    tr = np.zeros(nE, np.complex128)
    for i in range(nE):
        z = e0 + i * de + mu + 1j * eta
        A = z * np.eye(n)[None] - H
        A[:, :D, :D] -= sigma_e[i][None]
        Gk = np.linalg.inv(A)
        g[i] = Gk[:, :D, :D].mean(0)
        tr[i] = np.trace(Gk, axis1=1, axis2=2).mean()
    return g, tr


def downfold(H, S, hartr):
    """Construct_Hk_Sk's generalized eigenproblem (src/ConstructModelHamiltonian.cpp:103-111) and downfolding_ftn over
    the full band window (src/downfolding.cpp:20-63, NBAND = n, FromValToKS = identity), with the impurity level of
    src/downfolding.cpp:85-104.  H, S: (nk, n, n) ordinary (k, i, j) arrays (S None: identity); hartr: the D
    correlated orbitals (HartrIndex_inDFT).  Per k: H v = e S v with V^H S V = I (scipy.linalg.eigh), P = V[hartr],
    P <- S_d^-1/2 P (S_d = P P^H), DF = Q^H from the complete QR of P^H with rows 0..D-1 replaced by P,
    H_model = DF diag(e) DF^H.  Returns (eps (nk, n), H_model (nk, n, n), DF (nk, n, n), H_imp (D, D)).  LAPACK's
    Householder and eigenvector phase conventions differ from Eigen's, so only quantities invariant under a unitary
    rotation of DF's rows D..n-1 are comparable with the reference (and with the CUDA kernel)."""
    import scipy.linalg as sla
    H = np.asarray(H, np.complex128)
    nk, n = H.shape[0], H.shape[1]
    hartr = np.asarray(hartr, int)
    D = len(hartr)
    eps = np.zeros((nk, n))
    Hm = np.zeros((nk, n, n), np.complex128)
    DF = np.zeros((nk, n, n), np.complex128)
    for k in range(nk):
        Sk = np.eye(n) if S is None else np.asarray(S[k], np.complex128)
        e, V = sla.eigh(H[k], Sk)
        P = V[hartr, :]
        w, W = np.linalg.eigh(P @ P.conj().T)
        Pn = (W * w ** -0.5) @ W.conj().T @ P
        Q, _ = np.linalg.qr(Pn.conj().T, mode="complete")
        F = Q.conj().T
        F[:D] = Pn
        eps[k] = e
        DF[k] = F
        Hm[k] = (F * e) @ F.conj().T
    return eps, Hm, DF, Hm[:, :D, :D].mean(0)


def density_dft(H, sigma, mu, beta, hartr=None):
    """densityMatDFT of GreenFtn_w (src/GreenFtn.cpp:170-172, 197-215, 268-275, 311-319) by explicit n x n inversion
    of every (k, iw_n), n < 2 N_freq: sum_n [G + G^H - G0 - G0^H] / beta + U f(e0) U^H, with Sigma on the HartrIndex
    orbitals (its moment tail beyond N_freq), G0 the resolvent of H + m0 = U diag(e0) U^H (m0 added on the HartrIndex
    block, as GreenFtn_w's static Hamiltonian does for a downfolded layout) and the +-100 cut-offs of the Fermi
    factors.  H: (nk, n, n), sigma: (nfreq, D, D) ordinary arrays; returns (nk, n, n)."""
    H = np.asarray(H, np.complex128)
    sigma = np.asarray(sigma, np.complex128)
    nk, n = H.shape[0], H.shape[1]
    nf, D = sigma.shape[0], sigma.shape[1]
    hp = np.arange(D) if hartr is None else np.asarray(hartr, int)
    mom = moments(sigma, beta)
    Hs = H.copy()
    Hs[:, hp[:, None], hp[None, :]] += mom[0]
    e0, U = np.linalg.eigh(Hs)
    dens = np.zeros((nk, n, n), np.complex128)
    eye = np.eye(n)
    for f in range(2 * nf):
        iw = 1j * np.pi * (2 * f + 1) / beta
        sw = sigma[f] if f < nf else mom[0] + mom[1] / iw + mom[2] / iw ** 2 + mom[3] / iw ** 3
        A = (iw + mu) * eye[None] - H
        A[:, hp[:, None], hp[None, :]] -= sw
        G = np.linalg.inv(A)
        G0 = (U / (iw + mu - e0)[:, None, :]) @ U.conj().transpose(0, 2, 1)
        dens += G + G.conj().transpose(0, 2, 1) - G0 - G0.conj().transpose(0, 2, 1)
    x = beta * (e0 - mu)
    fr = np.where(x > 100.0, 0.0, np.where(x < -100.0, 1.0, 1.0 / (1.0 + np.exp(np.clip(x, -100, 100)))))
    return dens / beta + (U * fr[:, None, :]) @ U.conj().transpose(0, 2, 1)


def upfold(dens, DF, V, S, kgrid, rindex):
    """upfolding_density over the full band window (src/upfolding.cpp:10-35, 38-91): per k, D_DFT = V (DF^H D DF) V^H,
    then (1/N_k) sum_k M_k(i0, j0) exp(+i k.a R) at the rows (Rx, Ry, Rz, i0, j0) of rindex for M = S^-1 D_DFT S^-1,
    S^-1 D_DFT and D_DFT, with the k mesh of TightBinding (kmesh above) and a = pi.  Arrays (nk, n, n) ordinary;
    S None: identity.  Returns the three complex [nnz] vectors."""
    dens, DF, V = (np.asarray(x, np.complex128) for x in (dens, DF, V))
    X = DF.conj().transpose(0, 2, 1) @ dens @ DF
    Dd = V @ X @ V.conj().transpose(0, 2, 1)
    if S is None:
        Mdd = Md = Dd
    else:
        Si = np.linalg.inv(np.asarray(S, np.complex128))
        Mdd = Si @ Dd @ Si
        Md = Si @ Dd
    km = kmesh(*kgrid)
    ri = np.asarray(rindex)
    ph = np.exp(1j * np.pi * (km @ ri[:, :3].T.astype(float)))  # (nk, nnz): a = pi
    nk = km.shape[0]
    i0, j0 = ri[:, 3], ri[:, 4]
    return tuple((M[:, i0, j0] * ph).sum(0) / nk for M in (Mdd, Md, Dd))


def downfold_window(H, S, hartr, from_val_to_ks):
    """downfolding_ftn with a band window (src/downfolding.cpp:20-63): per k the model space is the NBAND[k] bands
    listed in from_val_to_ks[k]; P = V[hartr][:, window], P <- S_d^-1/2 P, DF = Q^H (complete QR of P^H, NBAND x
    NBAND) with rows 0..D-1 replaced by P, H_model = DF diag(e[window]) DF^H.  Returns lists (eps, H_model, DF, V)
    per k (ragged) and H_imp (D, D)."""
    import scipy.linalg as sla
    H = np.asarray(H, np.complex128)
    nk, n = H.shape[0], H.shape[1]
    hartr = np.asarray(hartr, int)
    D = len(hartr)
    out_e, out_h, out_df, out_v = [], [], [], []
    himp = np.zeros((D, D), np.complex128)
    for k in range(nk):
        Sk = np.eye(n) if S is None else np.asarray(S[k], np.complex128)
        e, V = sla.eigh(H[k], Sk)
        win = np.asarray(from_val_to_ks[k], int)
        P = V[hartr][:, win]
        w, W = np.linalg.eigh(P @ P.conj().T)
        Pn = (W * w ** -0.5) @ W.conj().T @ P
        Q, _ = np.linalg.qr(Pn.conj().T, mode="complete")
        F = Q.conj().T
        F[:D] = Pn
        Hm = (F * e[win]) @ F.conj().T
        out_e.append(e)
        out_h.append(Hm)
        out_df.append(F)
        out_v.append(V)
        himp += Hm[:D, :D]
    return out_e, out_h, out_df, out_v, himp / nk


def upfold_window(dens, DF, V, S, eps, from_val_to_ks, mu, beta, kgrid, rindex):
    """upfolding_density with a band window (src/upfolding.cpp:10-35, 38-91): per k, X = DF^H D DF in the window's
    KS bands; Matrix_KSBase = diag(f(e - mu)) (the +-100 cut-offs) with the window block replaced by X; D_DFT =
    V Matrix_KSBase V^H; then the three k -> R sums of :func:`upfold`.  dens, DF: ragged lists (NBAND[k] square);
    V, S, eps: (nk, n, n), (nk, n, n) or None, (nk, n)."""
    nk = len(dens)
    n = np.asarray(V).shape[1]
    Dd = np.zeros((nk, n, n), np.complex128)
    for k in range(nk):
        x = beta * (np.asarray(eps[k]) - mu)
        f = np.where(x > 100.0, 0.0, np.where(x < -100.0, 1.0, 1.0 / (1.0 + np.exp(np.clip(x, -100, 100)))))
        M = np.diag(f).astype(np.complex128)
        win = np.asarray(from_val_to_ks[k], int)
        M[np.ix_(win, win)] = DF[k].conj().T @ dens[k] @ DF[k]
        Dd[k] = V[k] @ M @ V[k].conj().T
    eye = np.broadcast_to(np.eye(n, dtype=np.complex128), (nk, n, n))
    return upfold(Dd, eye, eye, S, kgrid, rindex)
