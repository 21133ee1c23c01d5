"""Generate tests/golden/tau2w_exact.npz: FT_t_to_w of a seeded, piecewise-linear F(tau) evaluated in 40-digit
arithmetic (mpmath), i.e. the exact integral sum_s int_{tau_s}^{tau_{s+1}} F(tau) e^{i w_n tau} dtau of the
linear interpolant that src/FourierTransform.cpp:521-561 integrates.  The data are white noise on the tau grid,
the worst case for the cancellation in the per-segment formula.

    python tests/golden/make_tau2w_exact.py
"""
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 40
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    rng = np.random.default_rng(20251203)
    d, ntau, nfreq, beta = 2, 256, 64, 10.0
    ft = rng.normal(size=(ntau + 1, d, d)) + 1j * rng.normal(size=(ntau + 1, d, d))
    dt = mp.mpf(beta) / ntau
    out = np.zeros((nfreq, d, d), np.complex128)
    for n in range(nfreq):
        w = mp.pi * (2 * n + 1) / beta
        ph = [mp.exp(1j * w * s * dt) for s in range(ntau + 1)]
        for a in range(d):
            for b in range(d):
                f = [mp.mpc(complex(x)) for x in ft[:, a, b]]
                acc = mp.mpc(0)
                for s in range(ntau):
                    t0, t1 = s * dt, (s + 1) * dt
                    sl = (f[s + 1] - f[s]) / dt
                    c0 = f[s] - sl * t0
                    # int (sl t + c0) e^{i w t} dt over [t0, t1]
                    acc += sl * ((t1 * ph[s + 1] - t0 * ph[s]) / (1j * w) + (ph[s + 1] - ph[s]) / w ** 2)
                    acc += c0 * (ph[s + 1] - ph[s]) / (1j * w)
                out[n, a, b] = complex(acc)
    np.savez(os.path.join(HERE, "tau2w_exact.npz"), ft=ft, beta=beta, nfreq=nfreq, w=out)


if __name__ == "__main__":
    main()
