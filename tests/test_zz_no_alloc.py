"""dmftgpu_hyb_delta_noalloc: the hybridisation entry point for callers that cannot allocate device memory
(pool-owned HBM, or code that must not stall the device with a cudaMalloc).  It is checked against the
regular dmftgpu_hyb_delta through the C ABI on two calls in a row, which also exercises the reuse of its
static scratch, and both against the FP64 oracle's Construct_hyb_delta.  This file is collected last on
purpose."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _inputs(seed, nf, D):
    rng = np.random.default_rng(seed)
    beta = 12.0
    wn = np.pi * (2 * np.arange(nf) + 1) / beta
    S = np.zeros((nf, D, D), complex)
    G = np.zeros((nf, D, D), complex)
    for d in range(D):
        S[:, d, d] = 0.1 * d - 0.5j / (wn + 1.0)
        G[:, d, d] = 1.0 / (1j * wn - 0.2 * d - S[:, d, d])
    G += 0.01 * (rng.normal(size=G.shape) + 1j * rng.normal(size=G.shape)) / (1 + wn[:, None, None])
    himp = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
    himp = (himp + himp.conj().T) / 2
    return beta, S, G, himp


def test_noalloc_matches_hyb_delta_on_two_calls(orc):
    import torch
    from dmftpack_gb300 import lib

    so = lib.load()
    ctx = lib.Context(0)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    try:
        for call, (seed, nf, D, orb, mu) in enumerate([(1, 256, 4, [0, 1, 2], 0.3), (2, 512, 5, [4, 0, 2, 1], -0.7)]):
            beta, S, G, himp = _inputs(seed, nf, D)
            ref = ctx.Construct_hyb_delta(orb, S, G, mu, beta, himp)
            assert rel_err(ref, orc.hyb_delta(orb, S, G, himp, mu, beta)) < TOL, call
            cm = lambda a: torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, -1, -2))).to(dev)
            dS, dG, dH = cm(S), cm(G), cm(himp[None])[0]
            dim = len(orb)
            out = torch.full((nf, dim, dim), complex("nan"), dtype=torch.complex128, device=dev)
            o = np.ascontiguousarray(orb, np.int32)
            st = so.dmftgpu_hyb_delta_noalloc(dim, o.ctypes.data_as(C.POINTER(C.c_int)), nf, beta, D,
                                              C.c_void_p(dS.data_ptr()), C.c_void_p(dG.data_ptr()),
                                              C.c_void_p(dH.data_ptr()), mu, C.c_void_p(out.data_ptr()),
                                              C.c_void_p(stream.cuda_stream))
            assert st == 0, (call, st)
            got = np.swapaxes(out.cpu().numpy(), -1, -2)
            assert rel_err(got, ref) < TOL, call
            assert rel_err(got, orc.hyb_delta(orb, S, G, himp, mu, beta)) < TOL, call
    finally:
        ctx.close()


def test_noalloc_rejects_requests_beyond_its_scratch():
    from dmftpack_gb300 import lib
    so = lib.load()
    o = np.arange(32, dtype=np.int32)
    # 1024 frequencies x 32 x 32 exceeds the 2^19 complex numbers of static scratch: rejected before any launch
    st = so.dmftgpu_hyb_delta_noalloc(32, o.ctypes.data_as(C.POINTER(C.c_int)), 1024, 10.0, 32, C.c_void_p(16),
                                      C.c_void_p(16), C.c_void_p(16), 0.0, C.c_void_p(16), None)
    assert st == lib.BADARG
