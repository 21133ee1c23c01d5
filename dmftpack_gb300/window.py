"""The band window of the downfolding, low_energy_subspace_in_KS_basis (src/downfolding.cpp:130-187): per k point
the bands with lower < e - mu_DFT < upper (strict) form the model space, NBAND[k] of them, FromValToKS[k] their
indices in ascending band order.  Without downfolding every band is kept (:176-184).  The reference asserts
NBAND[k] != 0 and exits when NBAND[k] is below the number of correlated orbitals; both raise ValueError here."""
import numpy as np


def low_energy_subspace_in_KS_basis(KS_eigenEnergy, muDFT, lower_model_window, upper_model_window, n_corr,
                                    downfolding=True):
    """KS_eigenEnergy: (nk, n) band energies.  Returns (NBAND[nk] int array, FromValToKS list of int arrays)."""
    e = np.asarray(KS_eigenEnergy, dtype=float)
    nk, n = e.shape
    if not downfolding:
        return np.full(nk, n, dtype=int), [np.arange(n) for _ in range(nk)]
    d = e - muDFT
    inside = (lower_model_window < d) & (d < upper_model_window)
    nband = inside.sum(1).astype(int)
    if (nband == 0).any():
        raise ValueError("downfolding window holds no band at k point %d" % int(np.argmax(nband == 0)))
    low = np.nonzero(nband < n_corr)[0]
    if low.size:
        raise ValueError("NBAND at k point %d = %d < %d correlated orbitals" % (low[0], nband[low[0]], n_corr))
    return nband, [np.nonzero(inside[k])[0] for k in range(nk)]
