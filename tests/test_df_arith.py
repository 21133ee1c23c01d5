"""The double-float arithmetic of the mixed-precision kernels (dmftpack_gb300/csrc/df.cuh, smallmat_df.cuh) held to
exact rational arithmetic.  The header's own functions are compiled for the host (tests/cxx/df_arith_check.cu, nvcc
with -ffp-contract=off, where each single-precision operation is the IEEE round-to-nearest operation of its device
intrinsic) and run on seeded inputs; every result is compared with the exact value of the operation on the same
double-float inputs.  Bounds are in units of the inputs' magnitudes, as the error analysis of each operation gives
them (~2^-47 per operation; 2^-44 leaves room for the few roundings a composite operation chains)."""
import os
import shutil
import subprocess
import zlib
from fractions import Fraction as Q

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cxx", "df_arith_check.cu")
EPS = Q(1, 2 ** 44)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("no nvcc")
    exe = str(tmp_path_factory.mktemp("df") / "df_arith_check")
    csrc = os.path.join(ROOT, "dmftpack_gb300", "csrc")
    cmd = [nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", csrc, SRC, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(lines):
        out = subprocess.run([exe], input="".join(lines), capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stderr
        return [[float.fromhex(t) for t in ln.split()] for ln in out.stdout.splitlines()]
    return run


def _df(rng, lo=-8.0, hi=8.0, positive=False):
    """A double-float (hi, lo) split of a random double of random sign and magnitude."""
    x = float(np.exp(rng.uniform(lo, hi))) * (1 if positive or rng.random() < 0.5 else -1)
    h = float(np.float32(x))
    return h, float(np.float32(x - h))


def _v(d):
    return Q(d[0]) + Q(d[1])


def _hex(*ds):
    return " ".join(float(t).hex() for d in ds for t in d)


def _close(got, want, scale):
    return abs(got - want) <= EPS * scale


def test_two_sum_is_exact(harness):
    rng = np.random.default_rng(1)
    cases = [(float(np.float32(rng.normal() * 10 ** rng.uniform(-6, 6))), float(np.float32(rng.normal())))
             for _ in range(400)]
    out = harness(["two_sum %s %s\n" % (a.hex(), b.hex()) for a, b in cases])
    for (a, b), (s, e) in zip(cases, out):
        assert Q(s) + Q(e) == Q(a) + Q(b)


@pytest.mark.parametrize("op", ["add", "mul", "fma", "dot2", "fma2", "rcp", "sqrt", "div"])
def test_real_operations(harness, op):
    rng = np.random.default_rng(zlib.crc32(op.encode()))
    nargs = {"add": 2, "mul": 2, "fma": 3, "dot2": 4, "fma2": 5, "rcp": 1, "sqrt": 1, "div": 2}[op]
    cases = [[_df(rng, positive=(op == "sqrt")) for _ in range(nargs)] for _ in range(300)]
    out = harness(["%s %s\n" % (op, _hex(*c)) for c in cases])
    for c, r in zip(cases, out):
        x = [_v(d) for d in c]
        got = Q(r[0]) + Q(r[1])
        if op == "add":
            want, scale = x[0] + x[1], abs(x[0]) + abs(x[1])
        elif op == "mul":
            want = x[0] * x[1]
            scale = abs(want)
        elif op == "fma":
            want, scale = x[2] + x[0] * x[1], abs(x[0] * x[1]) + abs(x[2])
        elif op == "dot2":
            want, scale = x[0] * x[1] + x[2] * x[3], abs(x[0] * x[1]) + abs(x[2] * x[3])
        elif op == "fma2":
            want = x[4] + x[0] * x[1] + x[2] * x[3]
            scale = abs(x[0] * x[1]) + abs(x[2] * x[3]) + abs(x[4])
        elif op == "rcp":
            want = 1 / x[0]
            scale = abs(want)
        elif op == "div":
            want = x[0] / x[1]
            scale = abs(want)
        else:  # sqrt: compare squares (exact rational square root is not available)
            want, got, scale = x[0], got * got, abs(x[0])
        assert _close(got, want, scale), (op, c, r)


def test_lazy_sum_of_products(harness):
    rng = np.random.default_rng(5)
    cases = [[_df(rng, -3, 3) for _ in range(2 * n)] for n in (1, 2, 5, 9, 16) for _ in range(40)]
    out = harness(["lazy %s\n" % _hex(*c) for c in cases])
    for c, r in zip(cases, out):
        x = [_v(d) for d in c]
        want = sum((x[2 * i] * x[2 * i + 1] for i in range(len(c) // 2)), Q(0))
        scale = sum((abs(x[2 * i] * x[2 * i + 1]) for i in range(len(c) // 2)), Q(0))
        assert _close(Q(r[0]) + Q(r[1]), want, 4 * scale)


@pytest.mark.parametrize("op", ["cmul", "cmulc", "cfma", "cfms", "crcp"])
def test_complex_operations(harness, op):
    rng = np.random.default_rng(zlib.crc32(op.encode()))
    nargs = {"cmul": 2, "cmulc": 2, "cfma": 3, "cfms": 3, "crcp": 1}[op]
    cases = [[(_df(rng, -4, 4), _df(rng, -4, 4)) for _ in range(nargs)] for _ in range(200)]
    out = harness(["%s %s\n" % (op, _hex(*[d for z in c for d in z])) for c in cases])

    def cv(z):
        return _v(z[0]), _v(z[1])

    def mag(a):
        return abs(a[0]) + abs(a[1])

    for c, r in zip(cases, out):
        z = [cv(t) for t in c]
        got = (Q(r[0]) + Q(r[1]), Q(r[2]) + Q(r[3]))
        a = z[0]
        if op in ("cmul", "cmulc", "cfma", "cfms"):
            b = (z[1][0], -z[1][1]) if op == "cmulc" else z[1]
            p = (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])
            scale = mag(a) * mag(b)
            if op == "cfma":
                want = (z[2][0] + p[0], z[2][1] + p[1])
                scale += mag(z[2])
            elif op == "cfms":
                want = (z[2][0] - p[0], z[2][1] - p[1])
                scale += mag(z[2])
            else:
                want = p
        else:
            n = a[0] * a[0] + a[1] * a[1]
            want = (a[0] / n, -a[1] / n)
            scale = 4 * mag(want)
        assert _close(got[0], want[0], scale) and _close(got[1], want[1], scale), (op, c, r)


def _cmul(a, b):
    return a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0]


def _csub(a, b):
    return a[0] - b[0], a[1] - b[1]


def _exact_inverse3(A):
    """The inverse of a 3 x 3 complex rational matrix (pairs of Fractions) by its adjugate."""
    def cof(r, c):
        rs = [i for i in range(3) if i != r]
        cs = [j for j in range(3) if j != c]
        m = _csub(_cmul(A[rs[0]][cs[0]], A[rs[1]][cs[1]]), _cmul(A[rs[0]][cs[1]], A[rs[1]][cs[0]]))
        return m if (r + c) % 2 == 0 else (-m[0], -m[1])
    C = [[cof(r, c) for c in range(3)] for r in range(3)]
    det = (Q(0), Q(0))
    for c in range(3):
        t = _cmul(A[0][c], C[0][c])
        det = (det[0] + t[0], det[1] + t[1])
    n = det[0] * det[0] + det[1] * det[1]
    idet = (det[0] / n, -det[1] / n)
    return [[_cmul(C[c][r], idet) for c in range(3)] for r in range(3)]


@pytest.mark.parametrize("form", ["inv3", "inv3d"])
def test_in_register_inverse(harness, form):
    """The thread-per-frequency Schur kernel's pivoted in-register Gauss-Jordan (schur.cuh thread_inverse) in
    double-float and FP64 against the exact inverse: matrices of the kernel's form (mu + i w) I - H with H Hermitian,
    and row-permuted ones whose leading entries are small, so that every pivot choice is taken."""
    rng = np.random.default_rng(17)
    cases = []
    for t in range(120):
        Hm = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
        Hm = (Hm + Hm.conj().T) / 2
        w = float(np.exp(rng.uniform(np.log(0.05), np.log(5.0))))
        M = (0.3 + 1j * w) * np.eye(3) - Hm
        if t % 3 == 1:
            M = M[[1, 2, 0]]
        elif t % 3 == 2:
            M = M[[2, 0, 1]]
            M[0, 0] *= 1e-3
        cases.append(M)

    def split(x):
        h = float(np.float32(x))
        return h, float(np.float32(x - h))

    lines = []
    for M in cases:
        lines.append("%s %s\n" % (form, _hex(*[d for z in M.ravel() for d in (split(z.real), split(z.imag))])))
    out = harness(lines)
    for M, r in zip(cases, out):
        A = [[(_v(split(M[i, j].real)), _v(split(M[i, j].imag))) for j in range(3)] for i in range(3)]
        X = _exact_inverse3(A)
        assert r[0] == 0
        vals = r[1:]
        kappa = np.linalg.cond(M)
        scale = max(abs(X[i][j][0]) + abs(X[i][j][1]) for i in range(3) for j in range(3))
        tol = (Q(1, 2 ** 44) if form == "inv3" else Q(1, 2 ** 48)) * Q(float(kappa)) * scale
        for k in range(9):
            i, j = divmod(k, 3)
            got = (Q(vals[4 * k]) + Q(vals[4 * k + 1]), Q(vals[4 * k + 2]) + Q(vals[4 * k + 3]))
            assert abs(got[0] - X[i][j][0]) <= tol and abs(got[1] - X[i][j][1]) <= tol, (form, M, k)


def test_in_register_inverse_flags_a_singular_matrix(harness):
    z = "0x0p+0 " * 4
    one = "0x1p+0 0x0p+0 0x0p+0 0x0p+0 "
    # rows 1 and 2 equal: singular
    row = one + one + z
    out = harness(["inv3 %s\n" % (one + z + z + row + row)])
    assert out[0][0] == 1


def _fp64_lines(op, mats):
    lines = []
    for A in mats:
        n = A.shape[0]
        flat = A.ravel(order="F")
        lines.append("%s %s %s\n" % (op, float(n).hex(), " ".join("%s %s" % (z.real.hex(), z.imag.hex())
                                                                   for z in flat)))
    return lines


def test_fp64_gauss_jordan_inverse(harness):
    """linalg.cuh thread_gj_inverse (the impurity and moment kernels' per-thread inverse) against LAPACK."""
    rng = np.random.default_rng(21)
    mats = []
    for n in (1, 2, 3, 5, 8, 10):
        for _ in range(10):
            A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)) + 1j * np.eye(n)
            mats.append(A[rng.permutation(n)])
    out = harness(_fp64_lines("gj", mats))
    for A, r in zip(mats, out):
        n = A.shape[0]
        assert r[0] == 0
        X = (np.array(r[1::2]) + 1j * np.array(r[2::2])).reshape(n, n, order="F")
        want = np.linalg.inv(A)
        assert np.abs(X - want).max() <= 1e-14 * np.linalg.cond(A) * np.abs(want).max()


def test_fp64_jacobi_eigensolver(harness):
    """linalg.cuh thread_heig (reads the lower triangle) against LAPACK eigenvalues, with A U = U diag(w)."""
    rng = np.random.default_rng(23)
    mats = []
    for n in (1, 2, 4, 7, 10):
        for _ in range(8):
            B = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
            mats.append((B + B.conj().T) / 2)
    out = harness(_fp64_lines("heig", mats))
    for A, r in zip(mats, out):
        n = A.shape[0]
        assert r[0] == 0
        w = np.array(r[1:1 + n])
        U = (np.array(r[1 + n::2]) + 1j * np.array(r[2 + n::2])).reshape(n, n, order="F")
        scale = np.abs(A).max()
        assert np.abs(w - np.linalg.eigvalsh(A)).max() <= 1e-13 * scale
        assert np.abs(A @ U - U * w[None]).max() <= 1e-12 * scale
        assert np.abs(U.conj().T @ U - np.eye(n)).max() <= 1e-13


def test_cholesky_sign_tests(harness):
    """smallmat.cuh posdef_tri: the strict and semidefinite tests the positivity fix-up and causality checks ask."""
    def line(A, strict):
        n = A.shape[0]
        tri = [A[i, j] for i in range(n) for j in range(i + 1)]
        return "posdef %s %s %s\n" % (float(strict).hex(), float(n).hex(),
                                       " ".join("%s %s" % (z.real.hex(), z.imag.hex()) for z in tri))
    rng = np.random.default_rng(29)
    B = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    pd = B @ B.conj().T + 0.1 * np.eye(4)
    indef = pd - (np.linalg.eigvalsh(pd)[0] + 0.5) * np.eye(4)
    psd = np.diag([1.0, 0.0, 2.0]).astype(complex)
    cases = [(pd, 1, 1), (pd, 0, 1), (indef, 1, 0), (indef, 0, 0), (psd, 1, 0), (psd, 0, 1), (-pd, 0, 0)]
    out = harness([line(A, s) for A, s, _ in cases])
    assert [int(r[0]) for r in out] == [want for _, _, want in cases]

