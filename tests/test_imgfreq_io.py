"""Restart files in ImgFreqFtn's text format (dmftpack_gb300/imgfreq_io.py)."""
import numpy as np

from dmftpack_gb300 import imgfreq_io as io


def _sample(nf=16, N=3, beta=10.0, seed=0):
    rng = np.random.default_rng(seed)
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    A = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    M0 = (A + A.conj().T) / 2
    F = np.zeros((nf + 5, N, N), np.complex128)
    F[:nf] = M0[None] + np.eye(N)[None] / (1j * wn[:, None, None] - 0.5)
    F[nf] = M0
    F[nf + 1] = np.eye(N)
    F[0, 0, 2] = 3e-8   # below the writer's 1e-7 threshold: not written
    return F


def test_write_then_update_round_trip(tmp_path):
    F = _sample()
    p = tmp_path / "Sw_SOLVER.full.dat"
    io.write_full(p, F)
    lines = p.read_text().splitlines()
    assert lines[0].split()[:3] == ["0", "0", "0"]
    assert all(len(line.split()) == 5 for line in lines)
    assert sum(1 for line in lines if line.startswith("-")) == 5 * 9
    G = io.update_full(p, 16, 3)
    assert np.abs(G[:16] - np.where(np.abs(F[:16]) > 1e-7, F[:16], 0)).max() < 1e-8
    assert np.abs(G[16:]).max() == 0          # update_full leaves the tail slots alone
    assert G[0, 0, 2] == 0


def test_update_keeps_entries_missing_from_the_file(tmp_path):
    F = _sample()
    p = tmp_path / "Gw_loc.full.dat"
    io.write_full(p, F)
    base = np.full_like(F, 7.0 + 1.0j)
    G = io.update_full(p, 16, 3, into=base)
    assert G[0, 0, 2] == 7.0 + 1.0j


def test_read_full_regrids_to_a_new_temperature(tmp_path):
    """A function linear in w_n is reproduced exactly inside the file's grid and extrapolated linearly below it;
    above it the reference's rule R + w_last J / w applies (R, J: Hermitian and anti-Hermitian parts of the last
    point, J added without a factor i as src/ImgTimeFtn.cpp:741-747 does)."""
    nf, N, beta_prev, beta = 200, 2, 20.0, 25.0
    wn = np.pi * (2 * np.arange(nf) + 1) / beta_prev
    c = np.array([[0.3, 0.1], [0.1, -0.2]], complex)
    d = np.array([[0.01j, 0.002], [0.002, -0.03j]])
    F = np.zeros((nf + 5, N, N), np.complex128)
    F[:nf] = c[None] + d[None] * wn[:, None, None]
    p = tmp_path / "Sw.full.dat"
    io.write_full(p, F)
    G = io.read_full(p, 300, N, beta, beta_prev)
    wn_new = np.pi * (2 * np.arange(300) + 1) / beta
    lin = c[None] + d[None] * wn_new[:, None, None]
    below_or_inside = wn_new <= wn[-1]
    assert np.abs(G[:300][below_or_inside] - lin[below_or_inside]).max() < 1e-7
    last = F[nf - 1]
    R, J = (last + last.conj().T) / 2, (last - last.conj().T) / 2j
    for w in np.where(wn_new > wn[-1])[0]:
        assert np.abs(G[w] - (R + wn[-1] * J / wn_new[w])).max() < 1e-7


# ---- the same formats through the C ABI (dmftgpu_imgfreq_*: host code, no device), against this module ----

def test_c_abi_writes_the_same_bytes(tmp_path):
    from dmftpack_gb300 import lib
    F = _sample(nf=40, N=4, seed=3)
    a, b = tmp_path / "py.dat", tmp_path / "c.dat"
    io.write_full(a, F)
    lib.imgfreq_write(b, F)
    assert a.read_bytes() == b.read_bytes()


def test_c_abi_update_and_read_match_the_restatement(tmp_path):
    from dmftpack_gb300 import lib
    nf, N = 120, 3
    F = _sample(nf=nf, N=N, beta=15.0, seed=5)
    F[7] = 0   # a frequency with no line in the file
    p = tmp_path / "Sw_SOLVER.full.dat"
    io.write_full(p, F)
    base = np.full_like(F, 2.0 - 1.0j)
    assert np.array_equal(lib.imgfreq_update(p, nf, N, into=base), io.update_full(p, nf, N, into=base))
    for beta, beta_prev in ((15.0, 15.0), (20.0, 15.0), (11.0, 15.0)):
        assert np.array_equal(lib.imgfreq_read(p, 90, N, beta, beta_prev), io.read_full(p, 90, N, beta, beta_prev))


def test_c_abi_errors(tmp_path):
    import pytest
    from dmftpack_gb300 import lib
    with pytest.raises(lib.DmftGpuError) as e:
        lib.imgfreq_update(tmp_path / "missing.dat", 8, 2)
    assert e.value.code == lib.IO
    p = tmp_path / "bad.dat"
    p.write_text("0 0 5 +1.00000000 +0.00000000\n")
    with pytest.raises(lib.DmftGpuError) as e:
        lib.imgfreq_update(p, 8, 2)
    assert e.value.code == lib.BADARG
    with pytest.raises(ValueError):
        io.update_full(p, 8, 2)
    # a damaged frequency index is refused before anything is sized by it
    p.write_text("0 0 0 +1.00000000 +0.00000000\n99999999 0 0 +1.00000000 +0.00000000\n")
    for call in (lambda: lib.imgfreq_update(p, 8, 2), lambda: lib.imgfreq_read(p, 8, 2, 10.0, 10.0)):
        with pytest.raises(lib.DmftGpuError) as e:
            call()
        assert e.value.code == lib.BADARG
    with pytest.raises(ValueError):
        io.read_full(p, 8, 2, 10.0, 10.0)
