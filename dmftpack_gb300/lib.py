"""ctypes binding of libdmftgpu.so and the Python mirror of the reference's call surface for the hot path.

Function names follow DMFTpack (GreenFtn_w, GreenFtn_w_adjust_mu, GiwToNele, Construct_hyb_delta,
getAsymto_moments, Construct_Hk_Sk ...).  The reference's globals (beta, N_freq, HartrIndex, ...) are
passed explicitly through :class:`Lattice`.

Arrays are ordinary ``(count, i, j)`` complex stacks: numpy arrays (host; the library copies them to the
device and back) or CUDA ``torch`` tensors (device; the call is enqueued on torch's current stream).  The
library itself stores matrices column-major like Eigen; this module does the transposition.

There is no CPU fallback: if libdmftgpu.so is missing or no CUDA device is present, calls raise.
"""
import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

OK, SINGULAR, NONCONVERGED, NAN, BADARG, CAUSALITY, HERMITICITY, CUDA_ERROR, NOMEM, TIMEOUT, IO = range(11)
STATUS_NAMES = {0: "OK", 1: "SINGULAR", 2: "NONCONVERGED", 3: "NAN", 4: "BADARG", 5: "CAUSALITY",
                6: "HERMITICITY", 7: "CUDA_ERROR", 8: "NOMEM", 9: "TIMEOUT", 10: "IO"}
DEVICE_PTRS, MIXED, NEWTON, EXPLICIT, DIRECT_DFT, GRAPH, AUTOTUNE, NO_TENSOR = 0x1, 0x2, 0x4, 0x8, 0x10, 0x20, 0x40, 0x80

# every symbol include/dmftgpu.h declares
EXPORTS = ["dmftgpu_version", "dmftgpu_create", "dmftgpu_destroy", "dmftgpu_set_stream", "dmftgpu_get_stream",
           "dmftgpu_synchronize", "dmftgpu_last_error", "dmftgpu_launch_count", "dmftgpu_timing",
           "dmftgpu_kernel_time", "dmftgpu_kmesh", "dmftgpu_hk",
           "dmftgpu_moments", "dmftgpu_greenftn_w", "dmftgpu_greenftn_w_batched", "dmftgpu_gloc_real", "dmftgpu_density_dft", "dmftgpu_upfold", "dmftgpu_gloc_vjp", "dmftgpu_gloc_jvp", "dmftgpu_downfold", "dmftgpu_nele", "dmftgpu_adjust_mu", "dmftgpu_hyb_delta",
           "dmftgpu_fourier_w2tau", "dmftgpu_fourier_tau2w", "dmftgpu_sigma2_tau", "dmftgpu_fock", "dmftgpu_dyson",
           "dmftgpu_occupation", "dmftgpu_estimate_asymto", "dmftgpu_ipt", "dmftgpu_scgf2", "dmftgpu_dmft_iteration",
           "dmftgpu_hyb_delta_noalloc", "dmftgpu_weak_solver", "dmftgpu_double_counting", "dmftgpu_impurity_basis",
           "dmftgpu_mixer_stats", "dmftgpu_imgfreq_write", "dmftgpu_imgfreq_update", "dmftgpu_imgfreq_read",
           "dmftgpu_downfold_window", "dmftgpu_upfold_window"]


class DmftGpuError(RuntimeError):
    def __init__(self, what, code, detail=""):
        super().__init__("%s failed: %s%s" % (what, STATUS_NAMES.get(code, code), (" (%s)" % detail) if detail else ""))
        self.code = code


class DmftParams(C.Structure):
    """dmftgpu_dmft_params (include/dmftgpu.h)."""
    _fields_ = [("solver", C.c_int), ("ntau", C.c_int), ("n_electrons", C.c_double), ("U", C.c_double),
                ("Uprime", C.c_double), ("J", C.c_double), ("mixing", C.c_double), ("magnetism", C.c_int),
                ("dctype", C.c_int), ("nominal_charge", C.c_double), ("nu", C.c_int), ("uidx", _ip), ("ut", _dp),
                ("scgf_max_iter", C.c_int), ("basis_switch", C.c_int), ("pulay_history", C.c_int),
                ("pulay_start", C.c_int), ("mixer", C.c_int), ("newton_start", C.c_int), ("krylov_dim", C.c_int),
                ("krylov_tol", C.c_double)]


class _Lat(C.Structure):
    _fields_ = [("n", C.c_int), ("nk", C.c_int), ("nfreq", C.c_int), ("beta", C.c_double),
                ("ncl", C.c_int), ("nh", C.c_int), ("hartr", _ip)]


_lib = None


def library_path():
    return _build.LIB


def load(require_built=True):
    """Load libdmftgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if require_built:
            raise RuntimeError("libdmftgpu.so is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        _build.build()
    lib = C.CDLL(path)
    P = C.POINTER
    lib.dmftgpu_create.argtypes = [P(_vp), C.c_int]
    lib.dmftgpu_destroy.argtypes = [_vp]
    lib.dmftgpu_set_stream.argtypes = [_vp, _vp]
    lib.dmftgpu_get_stream.argtypes = [_vp]
    lib.dmftgpu_get_stream.restype = _vp
    lib.dmftgpu_synchronize.argtypes = [_vp]
    lib.dmftgpu_last_error.argtypes = [_vp]
    lib.dmftgpu_last_error.restype = C.c_char_p
    lib.dmftgpu_launch_count.argtypes = [_vp]
    lib.dmftgpu_launch_count.restype = C.c_longlong
    lib.dmftgpu_timing.argtypes = [_vp, C.c_int]
    lib.dmftgpu_kernel_time.argtypes = [_vp, C.c_char_p, _dp, _ip]
    lib.dmftgpu_kmesh.argtypes = [C.c_int, C.c_int, C.c_int, _dp]
    lib.dmftgpu_hk.argtypes = [_vp, C.c_int, C.c_int, _ip, _dp, C.c_int, C.c_int, C.c_int, _vp, C.c_int]
    lib.dmftgpu_moments.argtypes = [_vp, C.c_int, C.c_int, C.c_double, _vp, C.c_int, _vp, C.c_int]
    lib.dmftgpu_greenftn_w.argtypes = [_vp, P(_Lat), _vp, _vp, C.c_double, _vp, _vp, _vp, C.c_int]
    lib.dmftgpu_greenftn_w_batched.argtypes = [_vp, C.c_int, P(_Lat), P(_vp), P(_vp), _dp, P(_vp), P(_vp), P(_vp),
                                               C.c_int]
    lib.dmftgpu_gloc_real.argtypes = [_vp, P(_Lat), _vp, _vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                      _vp, _vp, C.c_int]
    lib.dmftgpu_density_dft.argtypes = [_vp, P(_Lat), _vp, _vp, C.c_double, _vp, C.c_int]
    lib.dmftgpu_upfold.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_int, _ip, _vp, _vp,
                                   _vp, C.c_int]
    lib.dmftgpu_gloc_vjp.argtypes = [_vp, P(_Lat), _vp, _vp, C.c_double, _vp, _vp, _dp, C.c_int]
    lib.dmftgpu_gloc_jvp.argtypes = [_vp, P(_Lat), _vp, _vp, C.c_double, _vp, C.c_double, _vp, C.c_int]
    lib.dmftgpu_downfold.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _ip, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int]
    lib.dmftgpu_downfold_window.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _ip, _vp, _vp, C.c_double, C.c_double,
                                            C.c_double, C.c_double, _ip, _ip, _vp, _vp, _vp, _vp, _vp, C.c_int]
    lib.dmftgpu_upfold_window.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _ip, _ip,
                                          C.c_double, C.c_double, C.c_int, _ip, _vp, _vp, _vp, C.c_int]
    lib.dmftgpu_nele.argtypes = [_vp, P(_Lat), _vp, _vp, C.c_double, _dp, _dp, C.c_int]
    lib.dmftgpu_adjust_mu.argtypes = [_vp, P(_Lat), _vp, _vp, C.c_double, C.c_double, C.c_double, _dp, _ip, C.c_int]
    lib.dmftgpu_hyb_delta.argtypes = [_vp, C.c_int, _ip, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp, C.c_double,
                                      _vp, C.c_int]
    lib.dmftgpu_fourier_w2tau.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_double, _vp, _vp, C.c_int, _vp, _vp,
                                          C.c_int]
    lib.dmftgpu_fourier_tau2w.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_double, _vp, _vp, C.c_int]
    lib.dmftgpu_sigma2_tau.argtypes = [_vp, C.c_int, C.c_int, C.c_double, C.c_int, _ip, _dp, _vp, _vp, C.c_int]
    lib.dmftgpu_fock.argtypes = [_vp, C.c_int, C.c_int, _ip, _dp, _vp, _vp, C.c_int]
    lib.dmftgpu_dyson.argtypes = [_vp, C.c_int, C.c_int, C.c_double, C.c_double, _vp, _vp, _vp, _vp, _vp, C.c_int]
    lib.dmftgpu_occupation.argtypes = [_vp, C.c_int, C.c_int, C.c_double, _vp, _vp, C.c_int]
    lib.dmftgpu_estimate_asymto.argtypes = [_vp, C.c_int, C.c_int, C.c_double, _vp, C.c_int, C.c_int]
    lib.dmftgpu_ipt.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _vp, _vp, _vp,
                                C.c_int, _ip, _dp, _vp, _vp, _vp, C.c_int]
    lib.dmftgpu_scgf2.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _vp, _vp, _vp,
                                  C.c_int, _ip, _dp, C.c_int, _vp, P(C.c_int), C.c_int]
    lib.dmftgpu_dmft_iteration.argtypes = [_vp, P(_Lat), _vp, P(DmftParams), C.c_int, _vp, _vp, _vp, _dp, _vp, _vp,
                                           _dp, C.c_int]
    lib.dmftgpu_impurity_basis.argtypes = [C.c_int, C.c_int, _vp, _vp, _vp]
    lib.dmftgpu_mixer_stats.argtypes = [_vp, _ip, _dp, _dp]
    lib.dmftgpu_imgfreq_write.argtypes = [C.c_char_p, C.c_int, C.c_int, _vp]
    lib.dmftgpu_imgfreq_update.argtypes = [C.c_char_p, C.c_int, C.c_int, _vp]
    lib.dmftgpu_imgfreq_read.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double, _vp]
    lib.dmftgpu_double_counting.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                            _vp, _vp, C.c_int, _vp]
    lib.dmftgpu_weak_solver.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _vp, _vp, C.c_int, _ip,
                                        _dp, _vp, C.c_int]
    lib.dmftgpu_hyb_delta_noalloc.argtypes = [C.c_int, _ip, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp,
                                              C.c_double, _vp, _vp]
    _lib = lib
    return lib


@dataclass
class Lattice:
    """The reference's lattice globals (NBAND, knum, N_freq, beta, NumCluster, NumHartrOrbit_per_cluster,
    HartrIndex)."""
    n: int
    nk: int
    nfreq: int
    beta: float
    ncl: int = 1
    nh: int = 1
    hartr: object = None

    @property
    def D(self):
        return self.ncl * self.nh

    def _c(self):
        h = None
        if self.hartr is not None:
            h = np.ascontiguousarray(self.hartr, dtype=np.int32)
        s = _Lat(self.n, self.nk, self.nfreq, float(self.beta), self.ncl, self.nh,
                 h.ctypes.data_as(_ip) if h is not None else None)
        s._keep = h
        return s


def _is_torch(x):
    return type(x).__module__.startswith("torch")


class _Arr:
    """A (count, i, j) complex stack converted to the library's column-major layout."""

    def __init__(self, x, device):
        self.device = device
        if device:
            import torch
            t = x.to(torch.complex128).transpose(-1, -2).contiguous()
            self.obj = t
            self.ptr = t.data_ptr()
        else:
            a = np.ascontiguousarray(np.swapaxes(np.asarray(x, dtype=np.complex128), -1, -2))
            self.obj = a
            self.ptr = a.ctypes.data

    @staticmethod
    def empty(shape, device, like=None):
        if device:
            import torch
            t = torch.empty(shape[:-2] + (shape[-1], shape[-2]), dtype=torch.complex128, device=like.device)
            o = _Arr.__new__(_Arr)
            o.device, o.obj, o.ptr = True, t, t.data_ptr()
            return o
        a = np.empty(shape[:-2] + (shape[-1], shape[-2]), np.complex128)
        o = _Arr.__new__(_Arr)
        o.device, o.obj, o.ptr = False, a, a.ctypes.data
        return o

    def result(self):
        if self.device:
            return self.obj.transpose(-1, -2)
        return np.ascontiguousarray(np.swapaxes(self.obj, -1, -2))


class Context:
    """One libdmftgpu context (CUDA device, stream, device workspaces)."""

    def __init__(self, device=0):
        self.lib = load()
        h = _vp()
        st = self.lib.dmftgpu_create(C.byref(h), device)
        if st != OK:
            raise DmftGpuError("dmftgpu_create", st)
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.dmftgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, what, st, allowed=(OK,)):
        if st not in allowed:
            raise DmftGpuError(what, st, self.lib.dmftgpu_last_error(self.h).decode(errors="replace"))
        return st

    def launches(self):
        return int(self.lib.dmftgpu_launch_count(self.h))

    def timing(self, enable=True):
        self._check("dmftgpu_timing", self.lib.dmftgpu_timing(self.h, int(bool(enable))))

    def kernel_time(self, name):
        """(total ms, launches) of kernel `name` since timing(True)."""
        ms, cnt = C.c_double(), C.c_int()
        self._check("dmftgpu_kernel_time", self.lib.dmftgpu_kernel_time(self.h, name.encode(), C.byref(ms),
                                                                           C.byref(cnt)))
        return ms.value, cnt.value

    def synchronize(self):
        self._check("dmftgpu_synchronize", self.lib.dmftgpu_synchronize(self.h))

    def _flags(self, device, extra=0):
        if device:
            import torch
            self.lib.dmftgpu_set_stream(self.h, _vp(torch.cuda.current_stream().cuda_stream))
            return DEVICE_PTRS | extra
        return extra

    # ------------------------------------------------------------------ lattice stage
    def Construct_Hk(self, n, rindex, hr, kgrid, device_out=None, mixed=False, tensor=True):
        """H(k) on the TightBinding mesh (Construct_Hk_Sk's Fourier sum); kgrid = (kx, ky, kz).
        mixed=True computes it on the tensor cores (bf16 slices, FP64-exact level sums); the default is FP64.
        Returns (nk, n, n): numpy, or a CUDA tensor when device_out is a torch device."""
        rindex = np.ascontiguousarray(rindex, np.int32)
        hr = np.ascontiguousarray(hr, np.complex128)
        kx, ky, kz = kgrid
        nk = kx * ky * kz
        dev = device_out is not None
        if dev:
            import torch
            out = torch.empty((nk, n, n), dtype=torch.complex128, device=device_out)
            ptr = out.data_ptr()
        else:
            out = np.empty((nk, n, n), np.complex128)
            ptr = out.ctypes.data
        st = self.lib.dmftgpu_hk(self.h, n, rindex.shape[0], rindex.ctypes.data_as(_ip),
                                 hr.view(np.float64).ctypes.data_as(_dp), kx, ky, kz, _vp(ptr),
                                 self._flags(dev, (MIXED if mixed else 0) | (0 if tensor else NO_TENSOR)))
        self._check("dmftgpu_hk", st)
        # stored column-major per k: reinterpret
        return out.transpose(-1, -2) if dev else np.ascontiguousarray(np.swapaxes(out, -1, -2))

    def getAsymto_moments(self, fw, beta, greenFtnAsym=False):
        dev = _is_torch(fw)
        a = _Arr(fw, dev)
        nf, dim = a.obj.shape[0], a.obj.shape[1]
        out = _Arr.empty((4, dim, dim), dev, like=a.obj)
        st = self.lib.dmftgpu_moments(self.h, dim, nf, float(beta), _vp(a.ptr), int(bool(greenFtnAsym)),
                                      _vp(out.ptr), self._flags(dev))
        self._check("dmftgpu_moments", st)
        return out.result()

    def GreenFtn_w(self, lat, H_k, SelfE_w, mu, mixed=False, with_gwhf=True, explicit=False):
        """GreenFtn_w: returns (Gw[nfreq,D,D], GwHF[nfreq,D,D] or None, NumMatrix[D,D]).
        explicit=True inverts every (k, iw) matrix in full as the reference does; the default computes the
        same correlated block through its exact Schur complement."""
        dev = _is_torch(H_k)
        h, s = _Arr(H_k, dev), _Arr(SelfE_w, dev)
        D = lat.D
        gw = _Arr.empty((lat.nfreq, D, D), dev, like=h.obj)
        g0 = _Arr.empty((lat.nfreq, D, D), dev, like=h.obj) if with_gwhf else None
        nm = _Arr.empty((D, D), dev, like=h.obj)
        L = lat._c()
        st = self.lib.dmftgpu_greenftn_w(self.h, C.byref(L), _vp(h.ptr), _vp(s.ptr), float(mu), _vp(gw.ptr),
                                         _vp(g0.ptr) if g0 else None, _vp(nm.ptr),
                                         self._flags(dev, (MIXED if mixed else 0) | (EXPLICIT if explicit else 0)))
        self._check("dmftgpu_greenftn_w", st)
        return gw.result(), (g0.result() if g0 else None), nm.result()

    def GreenFtn_w_batched(self, lats, Hk_cm, Sig_cm, mus, gw_cm, gwhf_cm, num_cm, mixed=False, graph=False,
                           autotune=False):
        """GreenFtn_w over a batch of problems; every array a CUDA tensor in the library's column-major layout,
        outputs written in place (gwhf_cm may be None)."""
        import torch  # noqa: F401
        n = len(lats)
        Ls = (_Lat * n)(*[lt._c() for lt in lats])
        ptr = lambda ts: (_vp * n)(*[_vp(t.data_ptr()) for t in ts])
        st = self.lib.dmftgpu_greenftn_w_batched(
            self.h, n, Ls, ptr(Hk_cm), ptr(Sig_cm), (C.c_double * n)(*[float(m) for m in mus]), ptr(gw_cm),
            ptr(gwhf_cm) if gwhf_cm is not None else None, ptr(num_cm),
            self._flags(True, (MIXED if mixed else 0) | (GRAPH if graph else 0) | (AUTOTUNE if autotune else 0)))
        self._check("dmftgpu_greenftn_w_batched", st)

    def retarded_GreenFtn(self, lat, H_k, SelfE_E, e0, de, eta, mu, mixed=False):
        """Real-axis lattice sum on E_n = e0 + n de (n < len(SelfE_E)): returns (G_loc(E)[nE,D,D], Tr G(E)[nE])."""
        dev = _is_torch(H_k)
        h, s = _Arr(H_k, dev), _Arr(SelfE_E, dev)
        nE, D = s.obj.shape[0], lat.D
        g = _Arr.empty((nE, D, D), dev, like=h.obj)
        if dev:
            import torch
            tr = torch.empty(nE, dtype=torch.complex128, device=h.obj.device)
            trp = tr.data_ptr()
        else:
            tr = np.empty(nE, np.complex128)
            trp = tr.ctypes.data
        L = lat._c()
        st = self.lib.dmftgpu_gloc_real(self.h, C.byref(L), _vp(h.ptr), _vp(s.ptr), int(nE), float(e0), float(de),
                                        float(eta), float(mu), _vp(g.ptr), _vp(trp),
                                        self._flags(dev, MIXED if mixed else 0))
        self._check("dmftgpu_gloc_real", st)
        return g.result(), tr

    def densityMatDFT(self, lat, H_k, SelfE_w, mu, mixed=False):
        """GreenFtn_w's per-k density matrix densityMatDFT[nk, n, n] (the full-model-space occupation at each k);
        mixed: the per-(k, iw) work in double-float on the FP32 pipe."""
        dev = _is_torch(H_k)
        h, s = _Arr(H_k, dev), _Arr(SelfE_w, dev)
        out = _Arr.empty((lat.nk, lat.n, lat.n), dev, like=h.obj)
        L = lat._c()
        st = self.lib.dmftgpu_density_dft(self.h, C.byref(L), _vp(h.ptr), _vp(s.ptr), float(mu), _vp(out.ptr),
                                          self._flags(dev, MIXED if mixed else 0))
        self._check("dmftgpu_density_dft", st)
        return out.result()

    def upfolding_density(self, densityMatDFT, DF_CorrBase, KS_eigenVectors, kgrid, H_Rindex, S_overlap=None,
                          window=None):
        """upfolding_density: returns (dual_DMR_dual, dual_DM_direct_DFTR, direct_DMR_direct), each complex [nnz] at
        the rows of H_Rindex [nnz, 5] = (Rx, Ry, Rz, i0, j0).  The (nk, n, n) inputs are numpy arrays or CUDA
        tensors; kgrid = (kx, ky, kz) of the k mesh.  window = (KS_eigenEnergy[nk, n], NBAND, FromValToKS, mu, beta)
        for a windowed downfolding (dens and DF padded beyond NBAND[k]); None: the full band window."""
        dev = _is_torch(densityMatDFT)
        d, f, v = _Arr(densityMatDFT, dev), _Arr(DF_CorrBase, dev), _Arr(KS_eigenVectors, dev)
        s = _Arr(S_overlap, dev) if S_overlap is not None else None
        n = d.obj.shape[1]
        ri = np.ascontiguousarray(H_Rindex, dtype=np.int32)
        nnz = ri.shape[0]
        if dev:
            import torch
            outs = [torch.empty(nnz, dtype=torch.complex128, device=d.obj.device) for _ in range(3)]
            ptrs = [o.data_ptr() for o in outs]
        else:
            outs = [np.empty(nnz, np.complex128) for _ in range(3)]
            ptrs = [o.ctypes.data for o in outs]
        kx, ky, kz = kgrid
        if window is None:
            st = self.lib.dmftgpu_upfold(self.h, int(n), int(kx), int(ky), int(kz), _vp(d.ptr), _vp(f.ptr),
                                         _vp(v.ptr), _vp(s.ptr) if s else None, int(nnz), ri.ctypes.data_as(_ip),
                                         _vp(ptrs[0]), _vp(ptrs[1]), _vp(ptrs[2]), self._flags(dev))
            self._check("dmftgpu_upfold", st)
        else:
            eps, nband, fvk, mu, beta = window
            if dev:
                import torch
                e_obj = torch.as_tensor(eps, dtype=torch.float64, device=d.obj.device).contiguous()
                e_ptr = e_obj.data_ptr()
            else:
                e_obj = np.ascontiguousarray(eps, dtype=np.float64)
                e_ptr = e_obj.ctypes.data
            nb = np.ascontiguousarray(nband, np.int32)
            nk = nb.shape[0]
            win = np.full((nk, n), -1, np.int32)
            for k in range(nk):
                win[k, :nb[k]] = fvk[k]
            st = self.lib.dmftgpu_upfold_window(self.h, int(n), int(kx), int(ky), int(kz), _vp(d.ptr), _vp(f.ptr),
                                                _vp(v.ptr), _vp(s.ptr) if s else None, _vp(e_ptr),
                                                nb.ctypes.data_as(_ip), win.ctypes.data_as(_ip), float(mu),
                                                float(beta), int(nnz), ri.ctypes.data_as(_ip), _vp(ptrs[0]),
                                                _vp(ptrs[1]), _vp(ptrs[2]), self._flags(dev))
            self._check("dmftgpu_upfold_window", st)
        return tuple(outs)

    def GreenFtn_w_vjp(self, lat, H_k, SelfE_w, mu, Gbar):
        """Reverse mode of G_loc = GreenFtn_w(...)[0]: returns (Sigma_bar[nfreq,D,D], mu_bar) for the cotangent
        Gbar[nfreq,D,D] (torch's complex-autograd convention: x_bar = J^H y_bar)."""
        dev = _is_torch(H_k)
        h, s, gb = _Arr(H_k, dev), _Arr(SelfE_w, dev), _Arr(Gbar, dev)
        D = lat.D
        out = _Arr.empty((lat.nfreq, D, D), dev, like=h.obj)
        mub = C.c_double()
        L = lat._c()
        st = self.lib.dmftgpu_gloc_vjp(self.h, C.byref(L), _vp(h.ptr), _vp(s.ptr), float(mu), _vp(gb.ptr),
                                       _vp(out.ptr), C.byref(mub), self._flags(dev))
        self._check("dmftgpu_gloc_vjp", st)
        return out.result(), mub.value

    def GreenFtn_w_jvp(self, lat, H_k, SelfE_w, mu, Sigma_dot, mu_dot=0.0):
        """Forward mode of G_loc = GreenFtn_w(...)[0] along (Sigma_dot, mu_dot): returns G_loc_dot."""
        dev = _is_torch(H_k)
        h, s, sd = _Arr(H_k, dev), _Arr(SelfE_w, dev), _Arr(Sigma_dot, dev)
        D = lat.D
        out = _Arr.empty((lat.nfreq, D, D), dev, like=h.obj)
        L = lat._c()
        st = self.lib.dmftgpu_gloc_jvp(self.h, C.byref(L), _vp(h.ptr), _vp(s.ptr), float(mu), _vp(sd.ptr),
                                       float(mu_dot), _vp(out.ptr), self._flags(dev))
        self._check("dmftgpu_gloc_jvp", st)
        return out.result()

    def downfolding_ftn(self, H_k, HartrIndex_inDFT, S_overlap=None, with_df=False, window=None, pad_energy=1e4):
        """Construct_Hk_Sk's generalized eigenproblem and downfolding_ftn, per k: returns (KS_eigenEnergy[nk,n],
        H_k_inModelSpace[nk,n,n], impurity_site_Hamiltonian[D,D]) and, with with_df, DF_CorrBase[nk,n,n] and
        KS_eigenVectors_orthoBasis[nk,n,n] as fourth and fifth items; with window = (muDFT, lower, upper) the band
        window of low_energy_subspace_in_KS_basis, and (NBAND[nk], FromValToKS list) follow as the last two items
        (H_model and DF padded beyond NBAND[k] as dmftgpu_downfold_window describes).  H_k, S_overlap: (nk, n, n)
        numpy arrays or CUDA tensors (S_overlap None: orthogonal basis); HartrIndex_inDFT: the D correlated orbitals."""
        dev = _is_torch(H_k)
        h = _Arr(H_k, dev)
        s = _Arr(S_overlap, dev) if S_overlap is not None else None
        nk, n = h.obj.shape[0], h.obj.shape[1]
        hartr = np.ascontiguousarray(HartrIndex_inDFT, dtype=np.int32)
        D = len(hartr)
        hm = _Arr.empty((nk, n, n), dev, like=h.obj)
        df = _Arr.empty((nk, n, n), dev, like=h.obj) if with_df else None
        ev = _Arr.empty((nk, n, n), dev, like=h.obj) if with_df else None
        hi = _Arr.empty((D, D), dev, like=h.obj)
        if dev:
            import torch
            eps = torch.empty((nk, n), dtype=torch.float64, device=h.obj.device)
            ep = eps.data_ptr()
        else:
            eps = np.empty((nk, n))
            ep = eps.ctypes.data
        if window is None:
            st = self.lib.dmftgpu_downfold(self.h, int(nk), int(n), int(D), hartr.ctypes.data_as(_ip), _vp(h.ptr),
                                           _vp(s.ptr) if s else None, _vp(ep), _vp(hm.ptr),
                                           _vp(df.ptr) if df else None, _vp(ev.ptr) if ev else None, _vp(hi.ptr),
                                           self._flags(dev))
            self._check("dmftgpu_downfold", st)
        else:
            nband = np.zeros(nk, np.int32)
            win = np.zeros((nk, n), np.int32)
            mu_dft, lower, upper = (float(x) for x in window)
            st = self.lib.dmftgpu_downfold_window(self.h, int(nk), int(n), int(D), hartr.ctypes.data_as(_ip),
                                                  _vp(h.ptr), _vp(s.ptr) if s else None, mu_dft, lower, upper,
                                                  float(pad_energy), nband.ctypes.data_as(_ip),
                                                  win.ctypes.data_as(_ip), _vp(ep), _vp(hm.ptr),
                                                  _vp(df.ptr) if df else None, _vp(ev.ptr) if ev else None,
                                                  _vp(hi.ptr), self._flags(dev))
            self._check("dmftgpu_downfold_window", st)
        out = (eps, hm.result(), hi.result())
        if with_df:
            out = out + (df.result(), ev.result())
        if window is not None:
            out = out + (nband, [win[k, :nband[k]].copy() for k in range(nk)])
        return out

    def GiwToNele(self, lat, H_k, SelfE_w, mu, deriv=False, mixed=False, explicit=False, tensor=True):
        """N(mu) (and dN/dmu with deriv).  In the mixed form the N(mu) pass of correlated blocks of 4 .. 10 orbitals
        runs its pole sums on the tensor cores unless tensor=False."""
        dev = _is_torch(H_k)
        h, s = _Arr(H_k, dev), _Arr(SelfE_w, dev)
        N, dN = C.c_double(), C.c_double()
        L = lat._c()
        st = self.lib.dmftgpu_nele(self.h, C.byref(L), _vp(h.ptr), _vp(s.ptr), float(mu), C.byref(N),
                                   C.byref(dN) if deriv else None,
                                   self._flags(dev, (MIXED if mixed else 0) | (EXPLICIT if explicit else 0)
                                               | (0 if tensor else NO_TENSOR)))
        self._check("dmftgpu_nele", st)
        return (N.value, dN.value) if deriv else N.value

    def GreenFtn_w_adjust_mu(self, lat, H_k, SelfE_w, mu, dmu, n_target, newton=False, mixed=False, explicit=False,
                             tensor=True):
        """Returns (mu, number of N(mu) passes)."""
        dev = _is_torch(H_k)
        h, s = _Arr(H_k, dev), _Arr(SelfE_w, dev)
        out, ne = C.c_double(), C.c_int()
        L = lat._c()
        fl = (NEWTON if newton else 0) | (MIXED if mixed else 0) | (EXPLICIT if explicit else 0) | (0 if tensor else NO_TENSOR)
        st = self.lib.dmftgpu_adjust_mu(self.h, C.byref(L), _vp(h.ptr), _vp(s.ptr), float(mu), float(dmu),
                                        float(n_target), C.byref(out), C.byref(ne), self._flags(dev, fl))
        self._check("dmftgpu_adjust_mu", st)
        return out.value, ne.value

    def Construct_hyb_delta(self, impurityOrbit, SelfE_w, Gw, mu, beta, impurity_site_Hamiltonian):
        dev = _is_torch(Gw)
        orb = np.ascontiguousarray(impurityOrbit, np.int32)
        s, g = _Arr(SelfE_w, dev), _Arr(Gw, dev)
        hi = _Arr(impurity_site_Hamiltonian[None] if not dev else impurity_site_Hamiltonian.unsqueeze(0), dev)
        nf, D = s.obj.shape[0], s.obj.shape[1]
        dim = orb.shape[0]
        out = _Arr.empty((nf, dim, dim), dev, like=s.obj)
        st = self.lib.dmftgpu_hyb_delta(self.h, dim, orb.ctypes.data_as(_ip), nf, float(beta), D, _vp(s.ptr),
                                        _vp(g.ptr), _vp(hi.ptr), float(mu), _vp(out.ptr), self._flags(dev))
        self._check("dmftgpu_hyb_delta", st)
        return out.result()

    # ------------------------------------------------------------------ impurity stage
    @staticmethod
    def _ulist(uidx, ut):
        uidx = np.ascontiguousarray(uidx, np.int32).reshape(-1, 4)
        ut = np.ascontiguousarray(ut, np.complex128).reshape(-1)
        return uidx, ut, uidx.shape[0]

    def FourierTransform(self, delta_w, beta, ntau, greenFtnAsym=False, moments1=None, moments=None, direct=False):
        """FourierTransform (iw -> tau grid, with tail and positivity fix-up): returns (ntau+1, d, d)."""
        dev = _is_torch(delta_w)
        a = _Arr(delta_w, dev)
        nf, d = a.obj.shape[0], a.obj.shape[1]
        m1 = _Arr(moments1[None] if not dev else moments1.unsqueeze(0), dev) if moments1 is not None else None
        mo = _Arr(moments, dev) if moments is not None else None
        out = _Arr.empty((ntau + 1, d, d), dev, like=a.obj)
        st = self.lib.dmftgpu_fourier_w2tau(self.h, d, nf, ntau, float(beta), _vp(a.ptr), _vp(mo.ptr) if mo else None,
                                            int(bool(greenFtnAsym)), _vp(m1.ptr) if m1 else None, _vp(out.ptr),
                                            self._flags(dev, DIRECT_DFT if direct else 0))
        self._check("dmftgpu_fourier_w2tau", st)
        return out.result()

    def FT_t_to_w(self, delta_t, beta, nfreq, allow_causality=False, direct=False):
        dev = _is_torch(delta_t)
        a = _Arr(delta_t, dev)
        ntau, d = a.obj.shape[0] - 1, a.obj.shape[1]
        out = _Arr.empty((nfreq, d, d), dev, like=a.obj)
        st = self.lib.dmftgpu_fourier_tau2w(self.h, d, nfreq, ntau, float(beta), _vp(a.ptr), _vp(out.ptr),
                                            self._flags(dev, DIRECT_DFT if direct else 0))
        self._check("dmftgpu_fourier_tau2w", st, (OK, CAUSALITY) if allow_causality else (OK,))
        return out.result()

    def getStimp(self, Gt, uidx, ut, beta, allow_hermiticity=False, mixed=False):
        dev = _is_torch(Gt)
        a = _Arr(Gt, dev)
        ntau, d = a.obj.shape[0] - 1, a.obj.shape[1]
        uidx, ut, nu = self._ulist(uidx, ut)
        out = _Arr.empty((ntau + 1, d, d), dev, like=a.obj)
        st = self.lib.dmftgpu_sigma2_tau(self.h, d, ntau, float(beta), nu, uidx.ctypes.data_as(_ip),
                                         ut.view(np.float64).ctypes.data_as(_dp), _vp(a.ptr), _vp(out.ptr),
                                         self._flags(dev, MIXED if mixed else 0))
        self._check("dmftgpu_sigma2_tau", st, (OK, HERMITICITY) if allow_hermiticity else (OK,))
        return out.result()

    def getFockOperator(self, occMat, uidx, ut):
        dev = _is_torch(occMat)
        a = _Arr(occMat[None] if not dev else occMat.unsqueeze(0), dev)
        d = a.obj.shape[1]
        uidx, ut, nu = self._ulist(uidx, ut)
        out = _Arr.empty((1, d, d), dev, like=a.obj)
        st = self.lib.dmftgpu_fock(self.h, d, nu, uidx.ctypes.data_as(_ip), ut.view(np.float64).ctypes.data_as(_dp),
                                   _vp(a.ptr), _vp(out.ptr), self._flags(dev))
        self._check("dmftgpu_fock", st)
        return out.result()[0]

    def getGwimp(self, himp, delta_w, fock, sigma2, mu, beta, allow_causality=False):
        dev = _is_torch(delta_w)
        one = (lambda x: x[None]) if not dev else (lambda x: x.unsqueeze(0))
        h, dl, fk, s2 = _Arr(one(himp), dev), _Arr(delta_w, dev), _Arr(one(fock), dev), _Arr(sigma2, dev)
        nf, d = dl.obj.shape[0], dl.obj.shape[1]
        out = _Arr.empty((nf, d, d), dev, like=dl.obj)
        st = self.lib.dmftgpu_dyson(self.h, d, nf, float(beta), float(mu), _vp(h.ptr), _vp(dl.ptr), _vp(fk.ptr),
                                    _vp(s2.ptr), _vp(out.ptr), self._flags(dev))
        self._check("dmftgpu_dyson", st, (OK, CAUSALITY) if allow_causality else (OK,))
        return out.result()

    def getoccMat(self, Gwimp, beta):
        dev = _is_torch(Gwimp)
        a = _Arr(Gwimp, dev)
        nf, d = a.obj.shape[0], a.obj.shape[1]
        out = _Arr.empty((1, d, d), dev, like=a.obj)
        st = self.lib.dmftgpu_occupation(self.h, d, nf, float(beta), _vp(a.ptr), _vp(out.ptr), self._flags(dev))
        self._check("dmftgpu_occupation", st)
        return out.result()[0]

    def estimate_asymto(self, F, nfreq, beta, order):
        """F: (nfreq+3, d, d); returns a copy with slot nfreq+order-1 written."""
        dev = _is_torch(F)
        a = _Arr(F, dev)
        d = a.obj.shape[1]
        st = self.lib.dmftgpu_estimate_asymto(self.h, d, nfreq, float(beta), _vp(a.ptr), int(order), self._flags(dev))
        self._check("dmftgpu_estimate_asymto", st)
        return a.result()

    def IPT(self, himp, weiss_field, projNumMatrix, uidx, ut, U, mu, beta, ntau, direct=False):
        """IPT solver: returns (SE_out[nfreq+5], Gwimp_out[nfreq+5], projNumMatrix)."""
        dev = _is_torch(weiss_field)
        one = (lambda x: x[None]) if not dev else (lambda x: x.unsqueeze(0))
        h, dl, nm = _Arr(one(himp), dev), _Arr(weiss_field, dev), _Arr(one(projNumMatrix), dev)
        nf, d = dl.obj.shape[0], dl.obj.shape[1]
        uidx, ut, nu = self._ulist(uidx, ut)
        se = _Arr.empty((nf + 5, d, d), dev, like=dl.obj)
        gi = _Arr.empty((nf + 5, d, d), dev, like=dl.obj)
        no = _Arr.empty((1, d, d), dev, like=dl.obj)
        st = self.lib.dmftgpu_ipt(self.h, d, nf, ntau, float(beta), float(U), float(mu), _vp(h.ptr), _vp(dl.ptr),
                                  _vp(nm.ptr), nu, uidx.ctypes.data_as(_ip), ut.view(np.float64).ctypes.data_as(_dp),
                                  _vp(se.ptr), _vp(gi.ptr), _vp(no.ptr), self._flags(dev, DIRECT_DFT if direct else 0))
        self._check("dmftgpu_ipt", st)
        return se.result(), gi.result(), no.result()[0]

    def SCGF2(self, himp, weiss_field, Gwimp, uidx, ut, mu, beta, ntau, mixing, max_iter=2000, direct=False,
              mixed=False):
        """SC2PT solver (SCGF2): Gwimp (nfreq slots) is the initial G_imp.  Returns (SE_out[nfreq+5],
        Gwimp_out[nfreq+5], loops)."""
        dev = _is_torch(weiss_field)
        one = (lambda x: x[None]) if not dev else (lambda x: x.unsqueeze(0))
        h, dl = _Arr(one(himp), dev), _Arr(weiss_field, dev)
        nf, d = dl.obj.shape[0], dl.obj.shape[1]
        g = _Arr.empty((nf + 5, d, d), dev, like=dl.obj)
        g.obj[:nf] = _Arr(Gwimp[:nf], dev).obj
        uidx, ut, nu = self._ulist(uidx, ut)
        se = _Arr.empty((nf + 5, d, d), dev, like=dl.obj)
        loops = C.c_int()
        st = self.lib.dmftgpu_scgf2(self.h, d, nf, ntau, float(beta), float(mu), float(mixing), _vp(h.ptr),
                                    _vp(dl.ptr), _vp(g.ptr), nu, uidx.ctypes.data_as(_ip),
                                    ut.view(np.float64).ctypes.data_as(_dp), int(max_iter), _vp(se.ptr),
                                    C.byref(loops),
                                    self._flags(dev, (DIRECT_DFT if direct else 0) | (MIXED if mixed else 0)))
        self._check("dmftgpu_scgf2", st)
        return se.result(), g.result(), loops.value

    WEAK_SOLVERS = {"HF": 0, "2PT": 1, "SC2PT": 2}

    def weak_solver(self, solver, gw, gwhf, uidx, ut, beta, ntau, direct=False, mixed=False):
        """weak_solver (Lowlevel_SOLVERTYPE "HF", "2PT" or "SC2PT") on Gw_weak (nfreq slots) and, for "2PT", GwHF_weak:
        returns SE_out[nfreq+5]."""
        dev = _is_torch(gw)
        g = _Arr(gw, dev)
        ghf = _Arr(gwhf, dev) if gwhf is not None else None
        nf, d = g.obj.shape[0], g.obj.shape[1]
        uidx, ut, nu = self._ulist(uidx, ut)
        se = _Arr.empty((nf + 5, d, d), dev, like=g.obj)
        st = self.lib.dmftgpu_weak_solver(self.h, self.WEAK_SOLVERS[solver], d, nf, int(ntau), float(beta), _vp(g.ptr),
                                          _vp(ghf.ptr) if ghf else None, nu, uidx.ctypes.data_as(_ip),
                                          ut.view(np.float64).ctypes.data_as(_dp), _vp(se.ptr),
                                          self._flags(dev, (DIRECT_DFT if direct else 0) | (MIXED if mixed else 0)))
        self._check("dmftgpu_weak_solver", st)
        return se.result()

    # ------------------------------------------------------------------ DMFT iteration
    def DMFT_iteration(self, lat, Hk_cm, params, iteration, selfe_cm, weiss_cm, nummat_cm, gloc_cm, mu,
                       mixed=False, newton=False, direct=False, tensor=True):
        """One dmft_main loop iteration on device state kept in the library's column-major layout (CUDA
        tensors, updated in place: SelfEnergy_w, weiss_fieldTB, NumMatrix, G_loc).  params: dict(solver ("IPT" or
        "SC2PT"), ntau, n_electrons, U, Uprime, J, mixing, magnetism, dctype, nominal_charge, uidx, ut,
        scgf_max_iter, basis_switch, pulay_history, pulay_start, mixer ("pulay" or "newton_krylov"), newton_start,
        krylov_dim, krylov_tol).  Returns (mu, gimp_cm[nfreq+5], residuals[5] = GwRD, GwRD_low, GwRD_max, NumMatRD,
        SCGF2 loops)."""
        import torch
        nf, D = lat.nfreq, lat.D
        uidx = np.ascontiguousarray(params["uidx"], np.int32).reshape(-1, 4)
        ut = np.ascontiguousarray(params["ut"], np.complex128).reshape(-1)
        solver = {"IPT": 0, "SC2PT": 1}[params.get("solver", "IPT")]
        P = DmftParams(solver, params["ntau"], params["n_electrons"], params["U"], params["Uprime"], params["J"],
                       params["mixing"], params.get("magnetism", 0), params.get("dctype", 1),
                       params.get("nominal_charge", 1.0), uidx.shape[0], uidx.ctypes.data_as(_ip),
                       ut.view(np.float64).ctypes.data_as(_dp), params.get("scgf_max_iter", 0),
                       int(bool(params.get("basis_switch", False))), int(params.get("pulay_history", 0)),
                       int(params.get("pulay_start", 0)), self.MIXERS[params.get("mixer", "pulay")],
                       int(params.get("newton_start", 0)), int(params.get("krylov_dim", 0)),
                       float(params.get("krylov_tol", 0.0)))
        gimp = torch.empty((nf + 5, D, D), dtype=torch.complex128, device=selfe_cm.device)
        m = C.c_double(mu)
        res = np.zeros(5)
        L = lat._c()
        fl = self._flags(True, (MIXED if mixed else 0) | (NEWTON if newton else 0) | (DIRECT_DFT if direct else 0)
                         | (0 if tensor else NO_TENSOR))
        st = self.lib.dmftgpu_dmft_iteration(self.h, C.byref(L), _vp(Hk_cm.data_ptr()), C.byref(P), int(iteration),
                                             _vp(selfe_cm.data_ptr()), _vp(weiss_cm.data_ptr()),
                                             _vp(nummat_cm.data_ptr()), C.byref(m), _vp(gloc_cm.data_ptr()),
                                             _vp(gimp.data_ptr()), res.ctypes.data_as(_dp), fl)
        self._check("dmftgpu_dmft_iteration", st)
        return m.value, gimp, res

    MIXERS = {"pulay": 0, "newton_krylov": 1}

    def mixer_stats(self):
        """(Jacobian-vector products, linear-solve relative residual, fixed-point residual |SE_out - Sigma| / |Sigma|)
        of the last DMFT_iteration's mixer; the first two are (0, 0.0) after a Pulay step."""
        k = C.c_int()
        r = C.c_double()
        f = C.c_double()
        self._check("dmftgpu_mixer_stats", self.lib.dmftgpu_mixer_stats(self.h, C.byref(k), C.byref(r), C.byref(f)))
        return k.value, r.value, f.value


DC_NONE, DC_NOMINAL, DC_FLL, DC_AMF, DC_SIGMA0, DC_UPRIME = 0, 1, 2, 3, 4, 0x100


def double_counting(dctype, natoms, nso, U, Uprime, J, nominal_charge, nummat=None, sigma0=None, initial=0,
                    dc_prev=None):
    """dc_for_dmft: the double-counting self-energy, (natoms nso) x (natoms nso) (host arithmetic; no device)."""
    N = natoms * nso
    cmo = lambda a: np.ascontiguousarray(np.asarray(a, np.complex128).T) if a is not None else None
    nm, s0 = cmo(nummat), cmo(sigma0)
    dc = cmo(dc_prev) if dc_prev is not None else np.zeros((N, N), np.complex128)
    dc = np.ascontiguousarray(dc)
    st = load().dmftgpu_double_counting(int(dctype), natoms, nso, float(U), float(Uprime), float(J),
                                        float(nominal_charge), _vp(nm.ctypes.data) if nm is not None else None,
                                        _vp(s0.ctypes.data) if s0 is not None else None, int(initial),
                                        _vp(dc.ctypes.data))
    if st != OK:
        raise DmftGpuError("dmftgpu_double_counting", st)
    return np.ascontiguousarray(dc.T)


def impurity_basis(himp, delta0, magnetism=0):
    """proj_to_site's solver basis (impurityBasisSwitch) for H_imp - DC and Delta(i w_0) (d x d): returns B (d x d)."""
    d = np.asarray(himp).shape[0]
    cmo = lambda a: np.ascontiguousarray(np.asarray(a, np.complex128).T)
    h, w0 = cmo(himp), cmo(delta0)
    out = np.zeros((d, d), np.complex128)
    st = load().dmftgpu_impurity_basis(d, int(magnetism), _vp(h.ctypes.data), _vp(w0.ctypes.data), _vp(out.ctypes.data))
    if st != OK:
        raise DmftGpuError("dmftgpu_impurity_basis", st)
    return np.ascontiguousarray(out.T)


def kmesh(kx, ky, kz):
    out = np.empty((kx * ky * kz, 3))
    st = load().dmftgpu_kmesh(kx, ky, kz, out.ctypes.data_as(_dp))
    if st != OK:
        raise DmftGpuError("dmftgpu_kmesh", st)
    return out


def _imgfreq_cm(F):
    return np.ascontiguousarray(np.swapaxes(np.asarray(F, np.complex128), -1, -2))


def imgfreq_write(path, F):
    """dataOut_full through the library: F is an (N_freq + 5, N, N) stack."""
    F = np.asarray(F, np.complex128)
    cm = _imgfreq_cm(F)
    st = load().dmftgpu_imgfreq_write(os.fsencode(path), F.shape[0] - 5, F.shape[1], _vp(cm.ctypes.data))
    if st:
        raise DmftGpuError("dmftgpu_imgfreq_write", st, path)


def imgfreq_update(path, nfreq, norbit, into=None):
    """update_full through the library: the file's w < N_freq entries overwrite `into` (zeros if None)."""
    F = np.zeros((nfreq + 5, norbit, norbit), np.complex128) if into is None else np.asarray(into, np.complex128)
    cm = _imgfreq_cm(F)
    st = load().dmftgpu_imgfreq_update(os.fsencode(path), nfreq, norbit, _vp(cm.ctypes.data))
    if st:
        raise DmftGpuError("dmftgpu_imgfreq_update", st, path)
    return np.swapaxes(cm, -1, -2).copy()


def imgfreq_read(path, nfreq, norbit, beta, beta_prev):
    """read_full through the library: the file re-gridded from beta_prev's Matsubara points to beta's."""
    cm = np.zeros((nfreq + 5, norbit, norbit), np.complex128)
    st = load().dmftgpu_imgfreq_read(os.fsencode(path), nfreq, norbit, float(beta), float(beta_prev),
                                     _vp(cm.ctypes.data))
    if st:
        raise DmftGpuError("dmftgpu_imgfreq_read", st, path)
    return np.swapaxes(cm, -1, -2).copy()
