"""A compiled C++ caller of the C ABI in the reference's data layout (tests/cxx/reference_layout_client.cpp): the
shims GreenFtn_w_adjust_mu, GreenFtn_w and Construct_hyb_delta (src/TB.h:45-61) over std::vector of column-major
complex matrices.  It is compiled with g++ against include/dmftgpu.h and linked to libdmftgpu.so; on the GPU it runs
and its outputs are compared with the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_err

SRC = os.path.join(ROOT, "tests", "cxx", "reference_layout_client.cpp")


def _compile(tmp_path):
    from dmftpack_gb300 import build
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    if not os.path.exists(build.LIB):
        pytest.skip("libdmftgpu.so is not built")
    exe = str(tmp_path / "client")
    libdir = os.path.dirname(build.LIB)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir, "-ldmftgpu",
           "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_layout_client_compiles_and_links(tmp_path):
    assert os.access(_compile(tmp_path), os.X_OK)


def test_reference_layout_client_restart_files(tmp_path):
    """The compiled caller's ImgFreqFtn::read_full / dataOut_full shims (host only) against the module restatement:
    a file written at beta_prev, re-gridded to beta and written again, byte for byte."""
    from dmftpack_gb300 import imgfreq_io as io
    exe = _compile(tmp_path)
    nf, N, beta_prev, beta = 64, 3, 12.0, 16.0
    rng = np.random.default_rng(4)
    wn = np.pi * (2 * np.arange(nf) + 1) / beta_prev
    A = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    F = np.zeros((nf + 5, N, N), np.complex128)
    F[:nf] = (A + A.conj().T)[None] / 2 + 1.0 / (1j * wn[:, None, None] - rng.normal(size=(N, N))[None])
    src, out, ref = tmp_path / "Sw.full.dat", tmp_path / "client.dat", tmp_path / "module.dat"
    io.write_full(src, F)
    r = subprocess.run([exe, "restart", str(src), str(out), "80", str(N), str(beta), str(beta_prev)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    io.write_full(ref, io.read_full(src, 80, N, beta, beta_prev))
    assert out.read_bytes() == ref.read_bytes()


@pytest.mark.gpu
def test_reference_layout_client_matches_oracle(tmp_path, orc):
    from dmftpack_gb300 import models
    exe = _compile(tmp_path)
    wl = models.t2g_p(k=3, nfreq=40, beta=12.0)
    H = orc.hk(wl.n, wl.rindex, wl.hr, orc.kmesh(*wl.kgrid))
    cm = lambda a: np.ascontiguousarray(np.swapaxes(a, -1, -2)).astype(np.complex128)
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([wl.n, wl.nk, wl.nfreq, wl.D], np.int32).tofile(f)
        np.array([wl.beta, 0.0, 7.3], np.float64).tofile(f)
        cm(H).tofile(f)
        cm(wl.sigma).tofile(f)
    r = subprocess.run([exe, inp, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, np.float64)
    mu = raw[0]
    z = raw[1:].view(np.complex128)
    D, nf = wl.D, wl.nfreq
    gw = np.swapaxes(z[:nf * D * D].reshape(nf, D, D), -1, -2)
    nm = np.swapaxes(z[nf * D * D:nf * D * D + D * D].reshape(D, D), -1, -2)
    weiss = np.swapaxes(z[nf * D * D + D * D:].reshape(nf, D, D), -1, -2)
    mu_o, _ = orc.adjust_mu(H, wl.sigma, 0.0, wl.beta, 1, D, 7.3)
    assert abs(mu - mu_o) < 1e-12
    gw_o, _, nm_o = orc.greenftn_w(H, wl.sigma, mu, wl.beta, 1, D)
    assert rel_err(gw, gw_o) < 1e-10 and rel_err(nm, nm_o) < 1e-10
    we_o = orc.hyb_delta(list(range(D)), wl.sigma, gw_o, H[:, :D, :D].mean(0), mu, wl.beta)
    assert rel_err(weiss, we_o) < 1e-10
