"""Independent numpy restatement of selected reference functions, used only to cross-check the C++ oracle.

It follows the reference lines literally where the C++ oracle takes a documented shortcut:
  - GiwToNele (src/GreenFtn.cpp:513-635) with numpy.linalg.eigvals of H(k)+S(iw_n), as the reference
    does with Eigen::ComplexEigenSolver, instead of the oracle's trace identity;
  - GreenFtn_w (src/GreenFtn.cpp:142-422) with numpy.linalg.inv / eigh in place of Eigen.
Arrays are ordinary (count, i, j) complex128.
"""
import numpy as np

PI = 3.1415926535897932384626


def kmesh(kx, ky, kz):
    """src/TB.cpp:196-207 (ax = ay = az = pi)."""
    nk = kx * ky * kz
    k = np.arange(nk)
    ax = PI
    dx, dy, dz = 2 * PI / (ax * kx), 2 * PI / (ax * ky), 2 * PI / (ax * kz)
    out = np.empty((nk, 3))
    out[:, 0] = -PI / ax + dx / 2 + (k % kx) * dx
    out[:, 1] = -PI / ax + dy / 2 + ((k % (kx * ky)) // kx) * dy
    out[:, 2] = -PI / ax + dz / 2 + (k // (kx * ky)) * dz
    return out


def hk(n, rindex, hr, km):
    """src/ConstructModelHamiltonian.cpp:66-77."""
    H = np.zeros((km.shape[0], n, n), np.complex128)
    ph = np.exp(-1j * (km[:, 0:1] * PI * rindex[None, :, 0] + km[:, 1:2] * PI * rindex[None, :, 1]
                       + km[:, 2:3] * PI * rindex[None, :, 2]))
    for e in range(rindex.shape[0]):
        H[:, rindex[e, 3], rindex[e, 4]] += hr[e] * ph[:, e]
    return H


def _sigma_at(n, Nf, S, mom, beta):
    iw = 1j * PI * (2.0 * n + 1.0) / beta
    if n < Nf:
        return S[n]
    return mom[0] + mom[1] / iw + mom[2] / iw ** 2 + mom[3] / iw ** 3


def nele_eig(H, S, mom, mu, beta, hartr, ncl, nh):
    """GiwToNele literally: eigenvalues of H(k) + S(iw_n) (within-cluster blocks), then the sums."""
    nk, n, _ = H.shape
    Nf = S.shape[0]
    D = ncl * nh
    mask = np.zeros((D, D), bool)
    for c in range(ncl):
        mask[c * nh:(c + 1) * nh, c * nh:(c + 1) * nh] = True
    w0, dw = 1j * PI / beta, 1j * 2 * PI / beta
    hi = np.asarray(hartr)
    total = 0.0
    Hinf = H.copy()
    Hinf[:, hi[:, None], hi[None, :]] += np.where(mask, mom[0], 0)
    einf = np.linalg.eigvals(Hinf)
    for nn in range(2 * Nf):
        SW = np.where(mask, _sigma_at(nn, Nf, S, mom, beta), 0)
        M = H.copy()
        M[:, hi[:, None], hi[None, :]] += SW
        ev = np.linalg.eigvals(M)
        w = w0 + nn * dw
        total += np.sum(np.real(1.0 / (w - ev + mu) - 1.0 / (w - einf + mu)))
    total *= 2.0 / beta
    total += np.sum(1.0 / (1 + np.exp(beta * (np.real(einf) - mu))))
    return total / nk


def greenftn_w(H, S, mom, mu, beta, hartr, ncl, nh):
    """GreenFtn_w literally with numpy inv/eigh; returns (Gw, GwHF, NumMatrix)."""
    nk, n, _ = H.shape
    Nf = S.shape[0]
    D = ncl * nh
    hi = np.asarray(hartr)
    Hs = H.copy()
    Hs[:, hi[:, None], hi[None, :]] += mom[0]
    ev, U = np.linalg.eigh(Hs)
    gw = np.zeros((Nf, D, D), np.complex128)
    g0w = np.zeros_like(gw)
    num = np.zeros((D, D), np.complex128)
    num0 = np.zeros((D, D), np.complex128)
    for nn in range(2 * Nf):
        iw = 1j * PI * (2.0 * nn + 1.0) / beta
        SW = _sigma_at(nn, Nf, S, mom, beta)
        A = -H.copy()
        A[:, hi[:, None], hi[None, :]] -= SW
        A += (iw + mu) * np.eye(n)[None]
        G = np.linalg.inv(A)
        G0 = np.einsum("kil,kl,kjl->kij", U, 1.0 / (iw + mu - ev), U.conj())
        Gp = G[:, hi[:, None], hi[None, :]]
        G0p = G0[:, hi[:, None], hi[None, :]]
        if nn < Nf:
            for c in range(ncl):
                sl = slice(c * nh, (c + 1) * nh)
                gw[nn, sl, sl] = Gp[:, sl, sl].sum(0) / nk
                g0w[nn, sl, sl] = G0p[:, sl, sl].sum(0) / nk
        num += (Gp + np.conj(np.swapaxes(Gp, 1, 2))).sum(0)
        num0 += (G0p + np.conj(np.swapaxes(G0p, 1, 2))).sum(0)
    x = beta * (ev - mu)
    f = np.where(x > 100, 0.0, np.where(x < -100, 1.0, 1.0 / (1.0 + np.exp(np.clip(x, -100, 100)))))
    occ = np.einsum("kil,kl,kjl->ij", U[:, hi, :], f, U[:, hi, :].conj())
    num = num / beta + 0.5 * nk * np.eye(D) + occ
    num0 = num0 / beta + 0.5 * nk * np.eye(D)
    return gw, g0w, (num - num0) / nk
