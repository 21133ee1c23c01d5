// downfold.cu -- the model Hamiltonian of a non-orthogonal tight-binding input, one thread block per k point:
//   * the generalized Hermitian eigenproblem H(k) v = e S(k) v of Construct_Hk_Sk
//     (src/ConstructModelHamiltonian.cpp:103-111, Eigen::GeneralizedSelfAdjointEigenSolver in its default
//     A x = lambda B x mode): S = L L^H (Cholesky), A = L^-1 H L^-H, A = U diag(e) U^H, V = L^-H U, so that
//     V^H S V = I;
//   * downfolding_ftn with the full band window (src/downfolding.cpp:20-63, NBAND = n, FromValToKS = identity):
//     P = V(HartrIndex_inDFT rows, :) (D x n), P <- S_d^-1/2 P with S_d = P P^H (Loewdin orthonormalisation of
//     the projected correlated orbitals), DF = Q^H from a Householder QR of P^H with its first D rows replaced
//     by P, H_model = DF diag(e) DF^H;
//   * the impurity level H_imp = (1/N_k) sum_k H_model(k)[0:D, 0:D] (src/downfolding.cpp:85-104 with the
//     correlated index reset to 0 .. D-1 by the downfolding).
// Rows D .. n-1 of DF (the ligand orbitals) are fixed only up to a unitary rotation among themselves: Eigen's
// eigenvector phases and Householder sign convention pick one, this kernel another.  H_model's correlated
// block, its spectrum, H_imp and every lattice Green function G_PP built from H_model are independent of that
// choice.
//
// Shared memory: four n x n complex tiles (A, L, U, X) reused stage by stage, 200 KB at n = 56.
#include <cmath>

#include "internal.h"
#include "smallmat.cuh"

namespace {

constexpr int DF_THREADS = 128, DF_NMAX = 56;

struct DfSmem {
    double2 *A, *L, *U, *X;  // n x n each, column-major
    double2 *vh;             // n: the current Householder vector
    double *e, *w;           // n: band energies; n: eigenvalues of the current block_heig call
    int *ord;
    DgRot *rot;
    double *red;
};

inline size_t df_smem_bytes(int n) {
    return (size_t)4 * n * n * sizeof(double2) + n * sizeof(double2) + 2 * DF_NMAX * sizeof(double) +
           DF_NMAX * sizeof(int) + (DF_NMAX / 2 + 2) * sizeof(DgRot) + DF_THREADS * sizeof(double) + 32;
}

__device__ DfSmem df_smem(double2 *sm, int n) {
    DfSmem s;
    const size_t nn = (size_t)n * n;
    s.A = sm;
    s.L = sm + nn;
    s.U = sm + 2 * nn;
    s.X = sm + 3 * nn;
    s.vh = sm + 4 * nn;
    s.e = (double *)(s.vh + n);
    s.w = s.e + DF_NMAX;
    s.ord = (int *)(s.w + DF_NMAX);
    s.rot = (DgRot *)(((size_t)(s.ord + DF_NMAX) + 15) & ~(size_t)15);
    s.red = (double *)(s.rot + DF_NMAX / 2 + 1);
    return s;
}

// The band window of low_energy_subspace_in_KS_basis (src/downfolding.cpp:130-187) when nband != nullptr: the model
// space of k is the bands with lower < e - mu_dft < upper (strict), which, the band energies being ascending, are
// the contiguous range lo .. lo + NBAND[k] - 1; nband[k] and win[k][j] = lo + j (FromValToKS) are written out.  A
// window with no band or fewer bands than correlated orbitals (where the reference exits) flags DG_BADARG.
struct DfWindow {
    int *nband, *win;  // outputs [nk], [nk][n]
    double mu, lower, upper, epad;
};

// H, S: [nk][n][n] column-major (S == nullptr: identity); eps: [nk][n] ascending; Hm, DF, EV: [nk][n][n].
// With a band window, H_model and DF fill their leading NBAND[k] x NBAND[k] block, and the rows/columns beyond it
// are a decoupled padding: H_model = epad on the diagonal, DF = identity.  A padded band adds nothing to G_PP (it
// couples to no orbital) and cancels between Tr G and Tr G0 in N(mu); with beta (epad - mu) > 100 its Fermi factor
// is zero, so the lattice sums of the padded H_model equal those of the ragged one.
__global__ void __launch_bounds__(DF_THREADS) k_downfold(int n, int D, const int *__restrict__ hartr,
                                                         const double2 *__restrict__ Hk, const double2 *__restrict__ Sk,
                                                         DfWindow wnd, double *eps, double2 *Hm, double2 *DF,
                                                         double2 *EV, int *status) {
    extern __shared__ double2 dsm[];
    const int k = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const size_t nn = (size_t)n * n;
    __shared__ int win_lo, win_nb;
    DfSmem s = df_smem(dsm, n);
    __shared__ int bad;
    if (tid == 0) bad = 0;
    for (int q = tid; q < (int)nn; q += nt) {
        s.A[q] = Hk[(size_t)k * nn + q];
        s.L[q] = Sk ? Sk[(size_t)k * nn + q] : cmk((q % n) == (q / n) ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    // 1. Cholesky S = L L^H in the lower triangle of L (the upper triangle is never read)
    for (int j = 0; j < n; j++) {
        if (tid == 0) {
            const double d = DG_AT(s.L, n, j, j).x;
            if (!(d > 0)) bad = 1;
            DG_AT(s.L, n, j, j) = cmk(d > 0 ? sqrt(d) : 1.0, 0.0);
        }
        __syncthreads();
        const double r = 1.0 / DG_AT(s.L, n, j, j).x;
        for (int i = j + 1 + tid; i < n; i += nt) DG_AT(s.L, n, i, j) = cscale(DG_AT(s.L, n, i, j), r);
        __syncthreads();
        const int t = n - j - 1;
        for (int x = tid; x < t * t; x += nt) {
            const int i = j + 1 + x % t, c = j + 1 + x / t;
            if (c <= i)
                DG_AT(s.L, n, i, c) = csub(DG_AT(s.L, n, i, c), cmulc(DG_AT(s.L, n, i, j), DG_AT(s.L, n, c, j)));
        }
        __syncthreads();
    }
    // 2. X = L^-1 H, U = L^-1 X^H, X = U^H = L^-1 H L^-H (forward substitutions, one column per thread)
    for (int c = tid; c < n; c += nt)
        for (int i = 0; i < n; i++) {
            double2 v = DG_AT(s.A, n, i, c);
            for (int l = 0; l < i; l++) v = csub(v, cmul(DG_AT(s.L, n, i, l), DG_AT(s.X, n, l, c)));
            DG_AT(s.X, n, i, c) = cscale(v, 1.0 / DG_AT(s.L, n, i, i).x);
        }
    __syncthreads();
    for (int c = tid; c < n; c += nt)
        for (int i = 0; i < n; i++) {
            double2 v = cconj(DG_AT(s.X, n, c, i));
            for (int l = 0; l < i; l++) v = csub(v, cmul(DG_AT(s.L, n, i, l), DG_AT(s.U, n, l, c)));
            DG_AT(s.U, n, i, c) = cscale(v, 1.0 / DG_AT(s.L, n, i, i).x);
        }
    __syncthreads();
    for (int q = tid; q < (int)nn; q += nt) s.X[q] = cconj(DG_AT(s.U, n, q / n, q % n));
    __syncthreads();
    // 3. A = U diag(e) U^H (U: eigenvectors, ascending e)
    int st = block_heig(n, s.X, s.A, s.U, s.w, s.ord, s.rot, s.red);
    for (int l = tid; l < n; l += nt) {
        s.e[l] = s.w[l];
        eps[(size_t)k * n + l] = s.w[l];
    }
    if (tid == 0) {
        int lo = 0, nb = n;
        if (wnd.nband) {
            lo = n;
            nb = 0;
            for (int l = 0; l < n; l++) {
                const double d = s.w[l] - wnd.mu;
                if (wnd.lower < d && d < wnd.upper) {
                    if (nb == 0) lo = l;
                    nb++;
                }
            }
            if (nb < D || nb < 1) {
                bad = 2;
                lo = 0;
                nb = n;
            }
            wnd.nband[k] = nb;
            for (int j = 0; j < n; j++) wnd.win[(size_t)k * n + j] = j < nb ? lo + j : -1;
        }
        win_lo = lo;
        win_nb = nb;
    }
    __syncthreads();
    const int nb = win_nb, lo = win_lo;                // bands in the window of k, the first of them
    auto wc = [&](int j) { return lo + j; };           // KS band of window column j
    // 4. V = L^-H U into A (back substitution, one column per thread)
    for (int c = tid; c < n; c += nt)
        for (int i = n - 1; i >= 0; i--) {
            double2 v = DG_AT(s.U, n, i, c);
            for (int l = i + 1; l < n; l++) v = csub(v, cmul(cconj(DG_AT(s.L, n, l, i)), DG_AT(s.A, n, l, c)));
            DG_AT(s.A, n, i, c) = cscale(v, 1.0 / DG_AT(s.L, n, i, i).x);
        }
    __syncthreads();
    if (EV)
        for (int q = tid; q < (int)nn; q += nt) EV[(size_t)k * nn + q] = s.A[q];
    // 5. P = V(hartr, window) into X (D x nb, ld D); S_d = P P^H into U (D x D, ld D)
    double2 *P = s.X, *Sd = s.U;
    for (int q = tid; q < D * nb; q += nt) P[q] = DG_AT(s.A, n, hartr[q % D], wc(q / D));
    __syncthreads();
    for (int q = tid; q < D * D; q += nt) {
        const int a = q % D, b = q / D;
        double2 v = cmk(0, 0);
        for (int i = 0; i < nb; i++) v = cfma(P[a + (size_t)i * D], cconj(P[b + (size_t)i * D]), v);
        Sd[q] = v;
    }
    __syncthreads();
    // 6. S_d = W diag(w) W^H (work in L, W in A), S_d^-1/2 = W diag(w^-1/2) W^H into U
    st |= block_heig(D, Sd, s.L, s.A, s.w, s.ord, s.rot, s.red);
    if (tid == 0 && !(s.w[0] > 0)) bad = 1;
    for (int q = tid; q < D * D; q += nt) {
        const int a = q % D, b = q / D;
        double2 v = cmk(0, 0);
        for (int l = 0; l < D; l++)
            v = cadd(v, cscale(cmulc(s.A[a + (size_t)l * D], s.A[b + (size_t)l * D]), s.w[l] > 0 ? rsqrt(s.w[l]) : 0.0));
        Sd[q] = v;
    }
    __syncthreads();
    // 7. P <- S_d^-1/2 P into rows 0..D-1 of DF (kept in L), M = P^H (nb x D, ld n) into A
    for (int q = tid; q < D * nb; q += nt) {
        const int a = q % D, i = q / D;
        double2 v = cmk(0, 0);
        for (int b = 0; b < D; b++) v = cfma(Sd[a + (size_t)b * D], P[b + (size_t)i * D], v);
        DG_AT(s.L, n, a, i) = v;
        DG_AT(s.A, n, i, a) = cconj(v);
    }
    __syncthreads();
    // 8. Householder QR of M: reflector j (I - 2 v v^H, |v| = 1, zero above row j) maps column j of the
    //    partially reduced M to alpha e_j, alpha = -phase(M_jj) |M(j:n, j)|; reflectors kept in the columns of U
    for (int j = 0; j < D; j++) {
        if (tid == 0) {
            double nx = 0;
            for (int i = j; i < nb; i++) nx += cabs2(DG_AT(s.A, n, i, j));
            nx = sqrt(nx);
            const double2 x0 = DG_AT(s.A, n, j, j);
            const double a0 = sqrt(cabs2(x0));
            const double2 alpha = a0 > 0 ? cscale(x0, -nx / a0) : cmk(-nx, 0.0);
            double nv = 0;
            for (int i = 0; i < nb; i++) {
                double2 v = i < j ? cmk(0, 0) : DG_AT(s.A, n, i, j);
                if (i == j) v = csub(v, alpha);
                s.vh[i] = v;
                nv += cabs2(v);
            }
            const double r = nv > 0 ? 1.0 / sqrt(nv) : 0.0;
            for (int i = 0; i < nb; i++) s.vh[i] = cscale(s.vh[i], r);
        }
        __syncthreads();
        for (int i = tid; i < nb; i += nt) DG_AT(s.U, n, i, j) = s.vh[i];
        for (int c = j + tid; c < D; c += nt) {
            double2 dot = cmk(0, 0);
            for (int i = j; i < nb; i++) dot = cfma(cconj(s.vh[i]), DG_AT(s.A, n, i, c), dot);
            dot = cscale(dot, 2.0);
            for (int i = j; i < nb; i++) DG_AT(s.A, n, i, c) = csub(DG_AT(s.A, n, i, c), cmul(s.vh[i], dot));
        }
        __syncthreads();
    }
    // 9. Q = H_0 H_1 ... H_{D-1} (applied to the identity, last reflector first) into X
    for (int q = tid; q < (int)nn; q += nt) s.X[q] = cmk((q % n) == (q / n) ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int j = D - 1; j >= 0; j--) {
        for (int c = tid; c < nb; c += nt) {
            double2 dot = cmk(0, 0);
            for (int i = j; i < nb; i++) dot = cfma(cconj(DG_AT(s.U, n, i, j)), DG_AT(s.X, n, i, c), dot);
            dot = cscale(dot, 2.0);
            for (int i = j; i < nb; i++) DG_AT(s.X, n, i, c) = csub(DG_AT(s.X, n, i, c), cmul(DG_AT(s.U, n, i, j), dot));
        }
        __syncthreads();
    }
    // 10. DF rows D..nb-1 = rows D..nb-1 of Q^H (the orthonormal complement of the correlated rows in the window);
    //     the identity on the padding
    for (int q = tid; q < (int)nn; q += nt) {
        const int i = q % n, c = q / n;
        if (i >= nb || c >= nb) DG_AT(s.L, n, i, c) = cmk(i == c ? 1.0 : 0.0, 0.0);
        else if (i >= D) DG_AT(s.L, n, i, c) = cconj(DG_AT(s.X, n, c, i));
    }
    __syncthreads();
    // 11. H_model = DF diag(e(window)) DF^H on the window block, epad on the padding's diagonal
    for (int q = tid; q < (int)nn; q += nt) {
        const int i = q % n, c = q / n;
        double2 v = cmk(0, 0);
        if (i < nb && c < nb) {
            for (int l = 0; l < nb; l++)
                v = cfma(cscale(DG_AT(s.L, n, i, l), s.e[wc(l)]), cconj(DG_AT(s.L, n, c, l)), v);
        } else if (i == c) {
            v = cmk(wnd.epad, 0.0);
        }
        Hm[(size_t)k * nn + q] = v;
        if (DF) DF[(size_t)k * nn + q] = s.L[q];
    }
    if (tid == 0 && (st || bad)) dg_flag(status, bad == 2 ? DG_BADARG : (bad ? DG_SINGULAR : DG_NONCONV));
}

// H_imp(a, b) = (1/nk) sum_k Hm(k)(a, b), summed in k order
__global__ void k_himp_avg(int nk, int n, int D, const double2 *__restrict__ Hm, double2 *himp) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D * D) return;
    const int a = q % D, b = q / D;
    double2 v = cmk(0, 0);
    for (int k = 0; k < nk; k++) v = cadd(v, Hm[(size_t)k * n * n + a + (size_t)b * n]);
    himp[q] = cscale(v, 1.0 / nk);
}

}  // namespace

namespace {

int downfold_impl(dmftgpu_ctx *ctx, int nk, int n, int D, const int *hartr, const double *hk, const double *sk,
                  const double *window, int *nband, int *from_val_to_ks, double *eps, double *hmodel, double *df,
                  double *evec, double *himp, int flags) {
    if (!ctx || nk < 1 || n < 1 || n > DF_NMAX || D < 1 || D > n || !hartr || !hk || !eps || !hmodel)
        return DMFTGPU_BADARG;
    for (int a = 0; a < D; a++) {
        if (hartr[a] < 0 || hartr[a] >= n) return dg_fail(ctx, DMFTGPU_BADARG, "downfold: HartrIndex out of range");
        for (int b = 0; b < a; b++)
            if (hartr[a] == hartr[b]) return dg_fail(ctx, DMFTGPU_BADARG, "downfold: repeated HartrIndex");
    }
    if (window && (!nband || !from_val_to_ks || !std::isfinite(window[0]) || !(window[1] < window[2]) ||
                   !std::isfinite(window[3])))
        return DMFTGPU_BADARG;
    DG_CUDA(cudaSetDevice(ctx->device));
    const size_t nn = (size_t)n * n, mb = (size_t)nk * nn * sizeof(double2);
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, mb, flags, "io.df_h", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sk, mb, flags, "io.df_s", &st);
    if (st) return st;
    double *dE = (double *)dg_out(ctx, eps, (size_t)nk * n * sizeof(double), flags, "io.df_e", &st);
    if (st) return st;
    double2 *dM = (double2 *)dg_out(ctx, hmodel, mb, flags, "io.df_hm", &st);
    if (st) return st;
    double2 *dF = (double2 *)dg_out(ctx, df, mb, flags, "io.df_df", &st);
    if (st) return st;
    double2 *dV = (double2 *)dg_out(ctx, evec, mb, flags, "io.df_ev", &st);
    if (st) return st;
    double2 *dI = (double2 *)dg_out(ctx, himp, (size_t)D * D * sizeof(double2), flags, "io.df_himp", &st);
    if (st) return st;
    int *dh = (int *)dg_buf(ctx, "df.hartr", D * sizeof(int));
    if (!dh) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemcpyAsync(dh, hartr, D * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    DfWindow wnd{nullptr, nullptr, 0.0, 0.0, 0.0, 0.0};
    if (window) {
        wnd.nband = (int *)dg_buf(ctx, "df.nband", (size_t)nk * sizeof(int));
        wnd.win = (int *)dg_buf(ctx, "df.win", (size_t)nk * n * sizeof(int));
        if (!wnd.nband || !wnd.win) return DMFTGPU_NOMEM;
        wnd.mu = window[0];
        wnd.lower = window[1];
        wnd.upper = window[2];
        wnd.epad = window[3];
    }
    DG_TRY(dg_status_reset(ctx));
    const size_t sm = df_smem_bytes(n);
    DG_CUDA(cudaFuncSetAttribute(k_downfold, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_downfold<<<nk, DF_THREADS, sm, ctx->stream>>>(n, D, dh, dH, dS, wnd, dE, dM, dF, dV, ctx->d_status);
    DG_LAUNCH(ctx, "k_downfold");
    if (dI) {
        k_himp_avg<<<dg_ceil_div(D * D, 128), 128, 0, ctx->stream>>>(nk, n, D, dM, dI);
        DG_LAUNCH(ctx, "k_himp_avg");
    }
    if (window) {
        DG_CUDA(cudaMemcpyAsync(nband, wnd.nband, (size_t)nk * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        DG_CUDA(cudaMemcpyAsync(from_val_to_ks, wnd.win, (size_t)nk * n * sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
    }
    DG_TRY(dg_out_done(ctx, eps, dE, (size_t)nk * n * sizeof(double), flags));
    DG_TRY(dg_out_done(ctx, hmodel, dM, mb, flags));
    DG_TRY(dg_out_done(ctx, df, dF, mb, flags));
    DG_TRY(dg_out_done(ctx, evec, dV, mb, flags));
    DG_TRY(dg_out_done(ctx, himp, dI, (size_t)D * D * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

}  // namespace

extern "C" int dmftgpu_downfold(dmftgpu_ctx *ctx, int nk, int n, int D, const int *hartr, const double *hk,
                                const double *sk, double *eps, double *hmodel, double *df, double *evec, double *himp,
                                int flags) {
    return downfold_impl(ctx, nk, n, D, hartr, hk, sk, nullptr, nullptr, nullptr, eps, hmodel, df, evec, himp, flags);
}

extern "C" int dmftgpu_downfold_window(dmftgpu_ctx *ctx, int nk, int n, int D, const int *hartr, const double *hk,
                                       const double *sk, double mu_dft, double lower, double upper,
                                       double pad_energy, int *nband, int *from_val_to_ks, double *eps,
                                       double *hmodel, double *df, double *evec, double *himp, int flags) {
    const double window[4] = {mu_dft, lower, upper, pad_energy};
    return downfold_impl(ctx, nk, n, D, hartr, hk, sk, window, nband, from_val_to_ks, eps, hmodel, df, evec, himp,
                         flags);
}
