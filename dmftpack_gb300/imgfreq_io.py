"""ImgFreqFtn's text files (Sw_SOLVER.full.dat, Gw_loc.full.dat, ...): the restart formats of DMFTpack.

A file holds one line "w m n Re Im" (printf "%d %d %d %+0.8f %+0.8f") per element with |F| > 1e-7 for w < N_freq,
then, for every (m, n), the tail slots N_freq .. N_freq+4 as w = -1 .. -5 (ImgFreqFtn::dataOut_full,
src/ImgTimeFtn.cpp:330-355).  Arrays here are (N_freq + 5, N, N) complex stacks in (slot, m, n) order, the
ImgFreqFtn slot layout (src/ImgTimeFtn.h:32-98).
"""
import numpy as np

TOL = 1e-7  # src/ImgTimeFtn.cpp:10
W_MAX = 1 << 24  # frequency indices at or above this mark a damaged file


def write_full(path, F):
    """dataOut_full: F is (N_freq + 5, N, N)."""
    F = np.asarray(F)
    nf = F.shape[0] - 5
    N = F.shape[1]
    lines = []
    for w in range(nf):
        for m in range(N):
            for n in range(N):
                v = F[w, m, n]
                if abs(v) > TOL:
                    lines.append("%d %d %d %+0.8f %+0.8f\n" % (w, m, n, v.real, v.imag))
    for m in range(N):
        for n in range(N):
            for k in range(5):
                v = F[nf + k, m, n]
                lines.append("%d %d %d %+0.8f %+0.8f\n" % (-(k + 1), m, n, v.real, v.imag))
    with open(path, "w") as f:
        f.writelines(lines)


def _rows(path):
    out = []
    with open(path) as f:
        for line in f:
            p = line.split()
            if len(p) < 5:
                continue
            out.append((int(p[0]), int(p[1]), int(p[2]), float(p[3]), float(p[4])))
            if out[-1][0] >= W_MAX:
                raise ValueError("%s: frequency index %d out of range" % (path, out[-1][0]))
    return out


def update_full(path, nfreq, norbit, into=None):
    """update_full (src/ImgTimeFtn.cpp:624-670): the w in [0, N_freq) entries of the file overwrite `into` (a
    (N_freq + 5, N, N) stack, zeros if None); other slots are kept.  An orbital index outside [0, N) is an error,
    as in the reference (which exits)."""
    F = np.zeros((nfreq + 5, norbit, norbit), np.complex128) if into is None else np.array(into, np.complex128)
    for w, m, n, re, im in _rows(path):
        if not (0 <= m < norbit and 0 <= n < norbit):
            raise ValueError("%s: orbital index (%d, %d) outside %d" % (path, m, n, norbit))
        if 0 <= w < nfreq:
            F[w, m, n] = re + 1j * im
    return F


def read_full(path, nfreq, norbit, beta, beta_prev):
    """read_full (src/ImgTimeFtn.cpp:673-751): a file written at inverse temperature beta_prev, re-gridded to the
    Matsubara frequencies of beta: linear interpolation in w_n between the file's points, linear extrapolation
    from its first two points below the first, and R + w_last J / w above the last, with R = (F + F^H)/2 and
    J = (F - F^H)/(2i) of the last point.  As in the reference (src/ImgTimeFtn.cpp:741-747), J enters without a
    factor i, so above the file's grid the anti-Hermitian part comes back as a Hermitian one.  Returns the
    (N_freq + 5, N, N) stack (tail slots zero)."""
    rows = _rows(path)
    wmax = max(r[0] for r in rows) + 1
    S = np.zeros((wmax, norbit, norbit), np.complex128)
    mats = np.zeros(wmax)  # as in the reference, a frequency with no line keeps grid point 0
    for w, m, n, re, im in rows:
        if w >= 0:
            S[w, m, n] = re + 1j * im
            mats[w] = (2 * w + 1) * np.pi / beta_prev
    F = np.zeros((nfreq + 5, norbit, norbit), np.complex128)
    dw_prev = 2 * np.pi / beta_prev
    # complex-by-real products and quotients act on the real and imaginary parts separately, as std::complex's
    # operators do (numpy's vectorised complex arithmetic can differ in the last bit)
    Sr, Si = S.real.copy(), S.imag.copy()

    def line(a, b, t):
        return ((Sr[b] - Sr[a]) / dw_prev * t + Sr[a]) + 1j * ((Si[b] - Si[a]) / dw_prev * t + Si[a])

    wp = 0
    for w in range(nfreq):
        x = (2 * w + 1) * np.pi / beta
        if x <= mats[0]:
            F[w] = line(0, 1, x - mats[0])
        elif x <= mats[wmax - 1]:
            while wp + 1 < wmax and not (mats[wp] < x <= mats[wp + 1]):
                wp += 1
            if wp + 1 >= wmax:
                raise ValueError("%s: no bracketing pair of Matsubara points for w_%d" % (path, w))
            F[w] = line(wp, wp + 1, x - mats[wp])
        else:
            lr, li = Sr[wmax - 1], Si[wmax - 1]
            rr, ri = (lr + lr.T) / 2.0, (li - li.T) / 2.0     # R = (F + F^H)/2
            jr, ji = (li + li.T) / 2.0, -((lr - lr.T) / 2.0)  # J = (F - F^H)/(2i)
            F[w] = (rr + mats[wmax - 1] * jr / x) + 1j * (ri + mats[wmax - 1] * ji / x)
    return F
