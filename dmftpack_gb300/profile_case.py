"""Run one named hot-path case on cuda:0 and print its device time; the command the ncu summaries under
profiles/ are taken with.

    python -m dmftpack_gb300.profile_case gloc  [--k 16 --nfreq 2048 --precision mixed|fp64 --algo schur|explicit]
    python -m dmftpack_gb300.profile_case scgf2 [--d 10 --nfreq 4096 --ntau 8192 --loops 2 --direct --mixed]
    python -m dmftpack_gb300.profile_case dmft  [--k 32 --nfreq 4096 --ntau 8192 --iters 2 --mixed --newton]
    python -m dmftpack_gb300.profile_case lattice [--k 16 --nfreq 4096 --mixed --newton]
    python -m dmftpack_gb300.profile_case batched [--nprob 64 --mixed --graph --autotune]
    python -m dmftpack_gb300.profile_case adjoint [--k 16 --nfreq 2048]
    python -m dmftpack_gb300.profile_case downfold [--k 16 --repeat 2]
    python -m dmftpack_gb300.profile_case density [--k 16 --nfreq 4096]

gloc:  one GreenFtn_w pass of the seeded t2g+p model (12 x 12 H(k), k^3 grid, beta = 40).
scgf2: `loops` SCGF2 loop iterations of a seeded d-spin-orbital impurity with Kanamori U = 4, J = 0.7,
       U' = 2.6 (the SC2PT workload's impurity sizes by default: d = 10, N_w = 4096, N_tau = 8192, beta = 40).
batched: GreenFtn_w over the ragged batch (64 seeded problems: n in {1,3,5,10,14,28}, k^3 with k in
       {8,12,16,24,32}, N_freq in {512..4096}, beta in [10, 100]) in one batched call, timed over repeats.
adjoint: one GreenFtn_w pass, one reverse-mode (VJP) and one forward-mode (JVP) pass of G_loc on the 56-orbital
       SOC model (20 x 20 correlated block, k^3 grid, beta = 30), FP64.
downfold: the model Hamiltonian of the 56-orbital SOC model (20 correlated orbitals, k^3 grid) with a seeded
       Hermitian positive-definite overlap S(k) = I + B B^H / 56: the generalized eigenproblem, the downfolding and
       H_imp, device pointers, timed over repeats.
density: densityMatDFT (the per-k density matrix, FP64), one FP64 GreenFtn_w pass for comparison, and the
       upfolding (k -> R sums onto the hopping table) of a k-resolved matrix, on the d+p model of the dmft case.
lattice: one mu search (GreenFtn_w_adjust_mu) and one GreenFtn_w pass on the d+p model of the dmft case.
dmft:  `iters` DMFT iterations with the SC2PT solver on the seeded 28-orbital d+p model (10 correlated
       spin-orbitals, Kanamori U = 4, J = 0.7, U' = 2.6, k^3 grid, beta = 40), H(k) rebuilt every iteration.
"""
import argparse
import json
import time

import numpy as np


def _impurity(d, nfreq, beta, seed=11):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    himp = 0.3 * (A + A.conj().T) / 2
    wn = np.pi * (2 * np.arange(nfreq) + 1) / beta
    weiss = np.zeros((nfreq, d, d), np.complex128)
    for e in rng.uniform(-3, 3, size=8):
        v = 0.4 * (rng.normal(size=d) + 1j * rng.normal(size=d))
        weiss += np.einsum("i,j->ij", v, v.conj())[None] / (1j * wn[:, None, None] - e)
    mu = 0.5
    g0 = np.linalg.inv((1j * wn[:, None, None] + mu) * np.eye(d)[None] - himp[None] - weiss)
    return himp, weiss, g0, mu


def run_batched(ctx, dev, a):
    import torch
    from dmftpack_gb300 import lib, models
    wls = models.batched_uneven(nprob=a.nprob)
    tcm = lambda t: t.transpose(-1, -2).contiguous()
    lats, H, S, G, G0, N, mus = [], [], [], [], [], [], []
    for w in wls:
        lats.append(lib.Lattice(w.n, w.nk, w.nfreq, w.beta, 1, w.D))
        H.append(tcm(ctx.Construct_Hk(w.n, w.rindex, w.hr, w.kgrid, device_out=dev)))
        S.append(tcm(torch.from_numpy(w.sigma).to(dev)))
        G.append(torch.empty((w.nfreq, w.D, w.D), dtype=torch.complex128, device=dev))
        G0.append(torch.empty_like(G[-1]))
        N.append(torch.empty((w.D, w.D), dtype=torch.complex128, device=dev))
        mus.append(0.0)
    times = []
    for _ in range(max(3, a.repeat)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.GreenFtn_w_batched(lats, H, S, mus, G, G0, N, mixed=a.mixed, graph=a.graph, autotune=a.autotune)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    units = sum(w.nk * 2 * w.nfreq for w in wls)
    return {"nprob": len(wls), "units": units, "mixed": a.mixed, "graph": a.graph, "autotune": a.autotune,
            "seconds_per_call": times, "units_per_s_last": units / times[-1]}


def run_adjoint(ctx, dev, a):
    import torch
    from dmftpack_gb300 import lib, models
    wl = models.soc56(k=a.k, nfreq=a.nfreq or 2048)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, wl.D)
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
    S = torch.from_numpy(wl.sigma).to(dev)
    rng = np.random.default_rng(1)
    X = torch.from_numpy(rng.normal(size=wl.sigma.shape) + 1j * rng.normal(size=wl.sigma.shape)).to(dev)
    out = {"nk": wl.nk, "n": wl.n, "D": wl.D, "nfreq": wl.nfreq}
    for name, fn in (("greenftn_w", lambda: ctx.GreenFtn_w(lat, Hd, S, 0.0, with_gwhf=False)),
                     ("vjp", lambda: ctx.GreenFtn_w_vjp(lat, Hd, S, 0.0, X)),
                     ("jvp", lambda: ctx.GreenFtn_w_jvp(lat, Hd, S, 0.0, X, 0.3))):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        out[name + "_seconds"] = time.perf_counter() - t0
    return out


def run_downfold(ctx, dev, a):
    import torch
    from dmftpack_gb300 import models
    wl = models.soc56(k=a.k, nfreq=8)
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
    g = torch.Generator(device=dev).manual_seed(7)
    B = 0.3 * torch.complex(torch.randn(wl.nk, wl.n, wl.n, device=dev, generator=g, dtype=torch.float64),
                            torch.randn(wl.nk, wl.n, wl.n, device=dev, generator=g, dtype=torch.float64))
    S = torch.eye(wl.n, dtype=torch.complex128, device=dev) + B @ B.conj().transpose(1, 2) / wl.n
    hartr = list(range(wl.D))
    times = []
    for _ in range(a.repeat + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.downfolding_ftn(Hd, hartr, S)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    return {"nk": wl.nk, "n": wl.n, "D": wl.D, "seconds": times[1:], "k_per_second": wl.nk / min(times[1:])}


def run_density(ctx, dev, a):
    import torch
    from dmftpack_gb300 import lib, models
    wl = models.dp28(k=a.k, nfreq=a.nfreq or 4096, ntau=a.ntau, beta=40.0)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, wl.D)
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
    sig = torch.from_numpy(wl.sigma).to(dev)
    out = {"nk": wl.nk, "n": wl.n, "D": wl.D, "nfreq": wl.nfreq, "nnz": len(wl.rindex)}
    eye = torch.eye(wl.n, dtype=torch.complex128, device=dev).expand(wl.nk, wl.n, wl.n).contiguous()
    for name, fn in (("density_dft", lambda: ctx.densityMatDFT(lat, Hd, sig, 0.0)),
                     ("greenftn_w_fp64", lambda: ctx.GreenFtn_w(lat, Hd, sig, 0.0)),
                     ("upfolding_density", lambda: ctx.upfolding_density(Hd, eye, eye, wl.kgrid, wl.rindex))):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        out[name + "_seconds"] = time.perf_counter() - t0
    return out


def run_lattice(ctx, dev, a):
    import torch
    from dmftpack_gb300 import lib, models
    wl = models.dp28(k=a.k, nfreq=a.nfreq or 4096, ntau=a.ntau, beta=40.0)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, wl.D)
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
    sig = torch.from_numpy(wl.sigma).to(dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mu, npass = ctx.GreenFtn_w_adjust_mu(lat, Hd, sig, 0.0, 1.0, wl.n_electrons, mixed=a.mixed, newton=a.newton)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ctx.GreenFtn_w(lat, Hd, sig, mu, mixed=a.mixed)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"nk": wl.nk, "n": wl.n, "D": wl.D, "nfreq": wl.nfreq, "mixed": a.mixed, "newton": a.newton, "mu": mu,
            "n_passes": npass, "mu_search_seconds": t1 - t0, "greenftn_w_seconds": t2 - t1}


def run_dmft(ctx, dev, a):
    """DMFT iterations (SC2PT) on the d+p model: returns per-iteration seconds, SCGF2 loops and residuals."""
    import torch
    from dmftpack_gb300 import lib, models
    wl = models.dp28(k=a.k, nfreq=a.nfreq or 4096, ntau=a.ntau, beta=40.0)
    D = wl.D
    uidx, ut = models.gen_Uijkl(D, 4.0, 2.6, 0.7)
    p = dict(solver="SC2PT", ntau=wl.ntau, n_electrons=wl.n_electrons, U=4.0, Uprime=2.6, J=0.7, mixing=0.5,
             magnetism=0, dctype=1, nominal_charge=2.0, uidx=uidx, ut=ut, scgf_max_iter=a.scgf_max)
    lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, 1, D)
    mixed = a.mixed
    tcm = lambda t: t.transpose(-1, -2).contiguous()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
    torch.cuda.synchronize()
    t_hk = time.perf_counter() - t0
    Hcm = tcm(Hd)
    sig = torch.from_numpy(wl.sigma).to(dev)
    mu, _ = ctx.GreenFtn_w_adjust_mu(lat, Hd, sig, 0.0, 1.0, wl.n_electrons, mixed=mixed, newton=a.newton)
    gl, _, nm = ctx.GreenFtn_w(lat, Hd, sig, mu, mixed=mixed, with_gwhf=False)
    we = ctx.Construct_hyb_delta(list(range(D)), sig, gl, mu, wl.beta, Hd[:, :D, :D].mean(0))
    se, we, nm, gl = tcm(sig), tcm(we), tcm(nm), tcm(gl)
    iters = []
    for it in range(1, a.iters + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)  # TightBinding rebuilds H(k)
        Hcm = tcm(Hd)
        mu, gi, res = ctx.DMFT_iteration(lat, Hcm, p, it, se, we, nm, gl, mu, mixed=mixed, newton=a.newton)
        torch.cuda.synchronize()
        iters.append({"seconds": time.perf_counter() - t0, "scgf_loops": int(res[4]), "mu": mu,
                      "GwRD": float(res[0]), "NumMatRD": float(res[3])})
    return {"nk": wl.nk, "n": wl.n, "D": D, "nfreq": wl.nfreq, "ntau": wl.ntau, "hk_seconds": t_hk,
            "mixed": mixed, "newton": a.newton, "iterations": iters}


def main():
    import torch
    from dmftpack_gb300 import lib, models
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["gloc", "scgf2", "dmft", "lattice", "batched", "adjoint", "downfold",
                                        "density"])
    ap.add_argument("--nprob", type=int, default=64)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--iters", type=int, default=2)
    ap.add_argument("--newton", action="store_true")
    ap.add_argument("--scgf-max", type=int, default=0)
    ap.add_argument("--k", type=int, default=16)
    ap.add_argument("--nfreq", type=int, default=None)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--algo", default="schur", choices=["schur", "explicit"])
    ap.add_argument("--d", type=int, default=10)
    ap.add_argument("--ntau", type=int, default=8192)
    ap.add_argument("--loops", type=int, default=2)
    ap.add_argument("--direct", action="store_true")
    ap.add_argument("--mixed", action="store_true", help="scgf2: double-float getStimp")
    ap.add_argument("--repeat", type=int, default=2)
    a = ap.parse_args()
    dev = torch.device("cuda:0")
    ctx = lib.Context(0)
    out = {"case": a.case}
    if a.case == "gloc":
        wl = models.t2g_p(k=a.k, nfreq=a.nfreq or 2048, beta=40.0)
        Hd = ctx.Construct_Hk(wl.n, wl.rindex, wl.hr, wl.kgrid, device_out=dev)
        S = torch.from_numpy(wl.sigma).to(dev)
        lat = lib.Lattice(wl.n, wl.nk, wl.nfreq, wl.beta, wl.ncl, wl.nh)

        def run():
            return ctx.GreenFtn_w(lat, Hd, S, 0.0, mixed=a.precision == "mixed", explicit=a.algo == "explicit")
        out.update(nk=wl.nk, nfreq=wl.nfreq, n=wl.n, D=wl.D, precision=a.precision, algo=a.algo)
    else:
        nfreq = a.nfreq or 4096
        himp, weiss, g0, mu = _impurity(a.d, nfreq, 40.0)
        uidx, ut = models.gen_Uijkl(a.d, 4.0, 2.6, 0.7)
        W, G0, Hi = (torch.from_numpy(x).to(dev) for x in (weiss, g0, himp))

        def run():
            return ctx.SCGF2(Hi, W, G0, uidx, ut, mu, 40.0, a.ntau, 0.5, max_iter=a.loops, direct=a.direct,
                             mixed=a.mixed)
        out.update(d=a.d, nfreq=nfreq, ntau=a.ntau, loops=a.loops, nu=int(uidx.shape[0]), direct=a.direct,
                   mixed=a.mixed)
    if a.case in ("dmft", "lattice", "batched", "adjoint", "downfold", "density"):
        out.update({"dmft": run_dmft, "lattice": run_lattice, "batched": run_batched,
                    "adjoint": run_adjoint, "downfold": run_downfold, "density": run_density}[a.case](ctx, dev, a))
        print(json.dumps(out), flush=True)
        ctx.close()
        return
    times = []
    for _ in range(a.repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    out["seconds"] = times
    print(json.dumps(out), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
