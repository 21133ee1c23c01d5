"""Hk.HWR tight-binding files (the input of read_HR, src/read_TB_parm.cpp:6-76).

Format: one header line ``Norbital of Atom = m`` per atom, then rows
``Rx Ry Rz atom1 atom2 i j Re Im`` (1-based atoms and orbitals, spin-orbital indices).
read_HR maps (atom, i) to the global orbital index accumulated_Num_SpinOrbital[atom-1] + i - 1 and
produces H_Rindex rows (Rx, Ry, Rz, i0, j0) and H_RMatrix values Re + i Im; these are exactly the
``rindex`` / ``hr`` arguments of dmftgpu_hk.
"""
import re

import numpy as np

_HDR = re.compile(r"^\s*Norbital of Atom\s*=\s*(\d+)\s*$")


def read_hr(path_or_text, num_atoms=None):
    """Parse an Hk.HWR file (path or its text).  Returns (norb_per_atom list, rindex[nnz,5] int32,
    hr[nnz] complex128)."""
    if "\n" in path_or_text or "Norbital" in path_or_text:
        text = path_or_text
    else:
        with open(path_or_text) as f:
            text = f.read()
    lines = [ln for ln in text.splitlines() if ln.strip()]
    norb = []
    i = 0
    while i < len(lines) and _HDR.match(lines[i]) and (num_atoms is None or len(norb) < num_atoms):
        norb.append(int(_HDR.match(lines[i]).group(1)))
        i += 1
    acc = np.concatenate([[0], np.cumsum(norb)]).astype(int)
    rows, vals = [], []
    for ln in lines[i:]:
        f = ln.split()
        rx, ry, rz, a1, a2, oi, oj = (int(x) for x in f[:7])
        re_, im_ = float(f[7]), float(f[8])
        rows.append((rx, ry, rz, acc[a1 - 1] + oi - 1, acc[a2 - 1] + oj - 1))
        vals.append(complex(re_, im_))
    return norb, np.asarray(rows, np.int32).reshape(-1, 5), np.asarray(vals, np.complex128)


def write_hr(norb, rindex, hr):
    """Inverse of :func:`read_hr` (orbitals are mapped back to (atom, i))."""
    acc = np.concatenate([[0], np.cumsum(norb)]).astype(int)
    out = ["Norbital of Atom = %d" % m for m in norb]
    for (rx, ry, rz, i0, j0), v in zip(np.asarray(rindex), np.asarray(hr)):
        a1 = int(np.searchsorted(acc, i0, side="right"))
        a2 = int(np.searchsorted(acc, j0, side="right"))
        out.append("%+d %+d %+d %d %d %d %d  %.17g %.17g" % (rx, ry, rz, a1, a2, i0 - acc[a1 - 1] + 1,
                                                           j0 - acc[a2 - 1] + 1, v.real, v.imag))
    return "\n".join(out) + "\n"


def write_density_hwr(norb, rindex, values):
    """The R-space density files of upfolding_density (DM_DFT_DMFT.HWR, dual_DM_direct.HWR, direct_DM_direct.HWR;
    src/upfolding.cpp:94-136): one row per H_Rindex entry, ``Rx Ry Rz atom1 atom2 i j Re Im`` with 1-based atoms
    and local orbitals and the values in C's ``%e``, no header.  norb: spin-orbitals per atom (the read_HR
    headers), rindex[nnz,5] and values[nnz] as dmftgpu_upfold takes and returns them."""
    acc = np.concatenate([[0], np.cumsum(norb)]).astype(int)
    out = []
    for (rx, ry, rz, i0, j0), v in zip(np.asarray(rindex), np.asarray(values)):
        a1 = int(np.searchsorted(acc, i0, side="right"))
        a2 = int(np.searchsorted(acc, j0, side="right"))
        out.append(" %+d %+d %+d %d %d %d %d      %e    %e  " % (rx, ry, rz, a1, a2, i0 - acc[a1 - 1] + 1,
                                                               j0 - acc[a2 - 1] + 1, v.real, v.imag))
    return "\n".join(out) + "\n"


def read_density_hwr(text, norb):
    """Inverse of :func:`write_density_hwr` (the rows read_DensityMat consumes): (rindex[nnz,5], values[nnz])."""
    acc = np.concatenate([[0], np.cumsum(norb)]).astype(int)
    rows, vals = [], []
    for ln in text.splitlines():
        f = ln.split()
        if len(f) < 9:
            continue
        rx, ry, rz, a1, a2, oi, oj = (int(x) for x in f[:7])
        rows.append((rx, ry, rz, acc[a1 - 1] + oi - 1, acc[a2 - 1] + oj - 1))
        vals.append(complex(float(f[7]), float(f[8])))
    return np.asarray(rows, np.int32).reshape(-1, 5), np.asarray(vals, np.complex128)
