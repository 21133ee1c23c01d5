"""CPU tests of the C ABI boundary: the library builds, loads and exports every symbol the header declares.
No compute call is made (there is no GPU here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    hdr = open(os.path.join(ROOT, "include", "dmftgpu.h")).read()
    return sorted(set(re.findall(r"\b(dmftgpu_[a-z0-9_]+)\s*\(", hdr)))


def test_header_declares_the_python_export_list():
    from dmftpack_gb300 import lib
    assert sorted(lib.EXPORTS) == _declared()


def test_library_exports_every_declared_symbol():
    from dmftpack_gb300 import build
    path = build.build()
    so = ctypes.CDLL(path)
    missing = [s for s in _declared() if not hasattr(so, s)]
    assert not missing, missing


def test_kmesh_is_host_only_and_matches_oracle(orc):
    from dmftpack_gb300 import lib
    import numpy as np
    assert np.array_equal(lib.kmesh(5, 4, 3), orc.kmesh(5, 4, 3))


def test_hwr_round_trip_and_reference_example():
    from dmftpack_gb300 import hwr, models
    wl = models.t2g_p(k=2, nfreq=8)
    text = hwr.write_hr([12], wl.rindex, wl.hr)
    norb, r2, h2 = hwr.read_hr(text)
    assert norb == [12]
    assert (r2 == wl.rindex).all() and (h2 == wl.hr).all()



def test_reference_example_fixture_parses_to_the_square_lattice_band(orc):
    """tests/golden/hubbard_example.json (made from the reference's Hubbard example by make_hubbard_example.py):
    its Hk.HWR rows, read by read_HR's restatement, give H(k) = -0.5 (cos kx + cos ky) on both spin-orbitals with
    the reference's e^{-ik.R} convention."""
    import test_gpu_fullsize as fs
    fx, n, rindex, hr = fs.reference_example()
    assert n == 2 and rindex.shape == (8, 5) and np.allclose(hr, -0.25)
    assert fx["k_points"] == [22, 22, 1] and fx["n_matsubara"] == 400 and fx["n_tau"] == 2400
    km = orc.kmesh(*fx["k_points"])
    H = orc.hk(n, rindex, hr, km)
    band = -0.5 * (np.cos(km[:, 0] * np.pi) + np.cos(km[:, 1] * np.pi))
    assert np.abs(H - band[:, None, None] * np.eye(2)[None]).max() < 1e-14


@pytest.mark.parametrize("nso,dd", [(2, True), (2, False), (6, False), (10, True), (10, False)])
def test_gen_uijkl_matches_oracle(orc, nso, dd):
    from dmftpack_gb300 import models
    ui, ut = models.gen_Uijkl(nso, 4.0, 2.6, 0.7, density_density=dd)
    oi, ot = orc.gen_uijkl(nso, 4.0, 2.6, 0.7, density_density=dd)
    assert np.array_equal(ui, oi) and np.array_equal(ut, ot)


def test_entry_points_reject_a_null_context_without_a_device():
    # argument validation happens before any CUDA call, so these run on a machine without a GPU
    from dmftpack_gb300 import lib
    L = lib.load()
    dummy = (ctypes.c_double * 8)()
    hartr = (ctypes.c_int * 1)(0)
    rindex = (ctypes.c_int * 5)(0, 0, 0, 0, 0)
    lat = lib.Lattice(2, 1, 4, 10.0)._c()
    p = ctypes.cast(dummy, ctypes.c_void_p)
    assert L.dmftgpu_downfold(None, 1, 2, 1, hartr, p, None, p, p, None, None, None, 0) == lib.BADARG
    assert L.dmftgpu_density_dft(None, ctypes.byref(lat), p, p, 0.0, p, 0) == lib.BADARG
    assert L.dmftgpu_upfold(None, 2, 1, 1, 1, p, p, p, None, 1, rindex, p, p, p, 0) == lib.BADARG
    assert L.dmftgpu_gloc_real(None, ctypes.byref(lat), p, p, 1, 0.0, 0.1, 0.05, 0.0, p, p, 0) == lib.BADARG
    ip = (ctypes.c_int * 4)()
    dp = (ctypes.c_double * 4)()
    assert L.dmftgpu_downfold_window(None, 1, 2, 1, hartr, p, None, 0.0, -1.0, 1.0, 1e4, ip, ip, p, p, p, p, p,
                                     0) == lib.BADARG
    assert L.dmftgpu_upfold_window(None, 2, 1, 1, 1, p, p, p, None, p, ip, ip, 0.0, 10.0, 1, rindex, p, p, p,
                                   0) == lib.BADARG
    assert L.dmftgpu_moments(None, 2, 16, 10.0, p, 1, p, 0) == lib.BADARG
    assert L.dmftgpu_ipt(None, 2, 16, 64, 10.0, 1.0, 0.0, p, p, p, 0, None, None, p, p, p, 0) == lib.BADARG
    assert L.dmftgpu_scgf2(None, 2, 16, 64, 10.0, 0.0, 0.5, p, p, p, 0, None, None, 10, p, ip, 0) == lib.BADARG
    assert L.dmftgpu_weak_solver(None, 0, 2, 16, 64, 10.0, p, p, 0, None, None, p, 0) == lib.BADARG
    params = lib.DmftParams()
    assert L.dmftgpu_dmft_iteration(None, ctypes.byref(lat), p, ctypes.byref(params), 1, p, p, p, dp, p, p, dp,
                                    0) == lib.BADARG
    assert L.dmftgpu_mixer_stats(None, ip, dp, dp) == lib.BADARG


def test_create_without_a_device_fails_cleanly():
    # on a machine without a usable GPU the context constructor returns the CUDA error and no handle
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from dmftpack_gb300 import lib
    L = lib.load()
    h = ctypes.c_void_p()
    assert L.dmftgpu_create(ctypes.byref(h), 0) == lib.CUDA_ERROR
    assert not h.value


def test_density_hwr_round_trip(orc):
    # the upfolded density of H(k) itself (DF = V = I) is the hopping table; written and read back at %e precision
    from dmftpack_gb300 import hwr, models
    wl = models.t2g_p(k=6, nfreq=8)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    eye = np.broadcast_to(np.eye(wl.n, dtype=np.complex128), H.shape)
    dd, _, _ = orc.upfold(H, eye, eye, None, wl.kgrid, wl.rindex)
    text = hwr.write_density_hwr([3, 9], wl.rindex, dd)
    first = text.splitlines()[0].split()
    assert len(first) == 9 and first[0][0] in "+-" and "e" in first[7]
    r, v = hwr.read_density_hwr(text, [3, 9])
    assert (r == wl.rindex).all()
    assert np.abs(v - wl.hr).max() <= 1e-6 * np.abs(wl.hr).max()


def test_ctypes_structs_match_the_header_layout(tmp_path):
    # the C compiler's sizeof / offsetof of the ABI structs against the ctypes mirrors the bindings pass
    import subprocess
    from dmftpack_gb300 import lib
    structs = {"dmftgpu_lattice": lib._Lat, "dmftgpu_dmft_params": lib.DmftParams}
    src = ['#include <stddef.h>', '#include <stdio.h>', '#include "dmftgpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        src.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            src.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    src.append("return 0; }")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)])
    got = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)], text=True).splitlines())
    for cname, py in structs.items():
        assert int(got["%s size" % cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got["%s %s" % (cname, fname)]) == getattr(py, fname).offset, (cname, fname)


@pytest.mark.parametrize("dctype", ["nominal", "nominal_Uprime", "fll", "fll_Uprime", "amf", "sigma0", "sigma0_step"])
def test_double_counting_matches_oracle(orc, dctype):
    """dc_for_dmft for every double-counting type, two correlated atoms of 6 spin-orbitals, as a host call of the
    library (no device needed) against the oracle."""
    from dmftpack_gb300 import lib
    code = {"nominal": lib.DC_NOMINAL, "nominal_Uprime": lib.DC_NOMINAL | lib.DC_UPRIME, "fll": lib.DC_FLL,
            "fll_Uprime": lib.DC_FLL | lib.DC_UPRIME, "amf": lib.DC_AMF, "sigma0": lib.DC_SIGMA0,
            "sigma0_step": lib.DC_SIGMA0}[dctype]
    initial = 1 if dctype == "sigma0_step" else 0
    natoms, nso = 2, 6
    rng = np.random.default_rng(4)
    A = rng.normal(size=(12, 12)) + 1j * rng.normal(size=(12, 12))
    nummat = 0.05 * (A + A.conj().T) + 0.4 * np.eye(12)
    sigma0 = 0.3 * (A + A.conj().T) - 0.2j * np.eye(12)
    prev = np.diag(rng.uniform(1, 3, size=12)).astype(complex)
    kw = dict(nummat=nummat, sigma0=sigma0, initial=initial, dc_prev=prev)
    got = lib.double_counting(code, natoms, nso, 4.0, 2.6, 0.7, 2.0, **kw)
    ref = orc.double_counting(code, natoms, nso, 4.0, 2.6, 0.7, 2.0, **kw)
    assert np.abs(got - ref).max() < 1e-14 and np.abs(ref).max() > 0.1


@pytest.mark.parametrize("branch", ["spin_averaged", "soc"])
def test_impurity_basis_matches_oracle(orc, branch):
    """impurityBasisSwitch's solver basis (host call of the library, no device) against the numpy restatement with the
    same eigenvector gauge: unitary, and for the spin-averaged branch it diagonalises the spin-pair average of
    Re[H_imp + Delta(i w_0)]."""
    from dmftpack_gb300 import lib
    d = 6
    rng = np.random.default_rng(8)
    if branch == "spin_averaged":
        h0 = rng.normal(size=(d // 2, d // 2))
        himp = np.kron(h0 + h0.T, np.eye(2)).astype(complex)
        w0 = rng.normal(size=(d // 2, d // 2)) + 1j * rng.normal(size=(d // 2, d // 2))
        delta0 = np.kron(w0 + w0.T.conj(), np.eye(2)) * 0.3 - 0.5j * np.eye(d)
    else:
        A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
        himp = A + A.conj().T
        W = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
        delta0 = 0.3 * W - 0.5j * np.eye(d)
    B = lib.impurity_basis(himp, delta0)
    Bo = orc.impurity_basis(himp, delta0)
    assert np.abs(B.conj().T @ B - np.eye(d)).max() < 1e-12
    assert np.abs(B - Bo).max() < 1e-10
    if branch == "spin_averaged":
        M = 0.5 * (delta0[0::2, 0::2] + delta0[1::2, 1::2] + himp[0::2, 0::2] + himp[1::2, 1::2])
        R = (0.5 * (M + M.conj().T)).real
        Ev = B[0::2, 0::2].real
        off = Ev.T @ R @ Ev
        assert np.abs(off - np.diag(np.diag(off))).max() < 1e-10
