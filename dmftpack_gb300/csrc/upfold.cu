// upfold.cu -- upfolding_density (src/upfolding.cpp:10-35, 38-91) over the full band window: the DMFT density
// matrix of every k point taken from the model basis back to the DFT orbital basis and Fourier-summed onto the
// hopping table's (R, i0, j0) entries.
//
//   per k (k_upfold_k, one block per k):   X = DF^H D DF                      (model -> KS basis, :13)
//                                           D_DFT = V X V^H                     (KS -> DFT basis, :33; V = the KS
//                                                                                eigenvectors in the DFT basis)
//                                           M_dd = S^-1 D_DFT S^-1, M_d = S^-1 D_DFT, M = D_DFT   (:48-49)
//   k -> R (k_axis_dft x 3 + k_upfold_gather):  DM(R)(i0, j0) = (1/N_k) sum_k M_k(i0, j0) exp(+i k.a R)  (:64-73)
//
// The k mesh is TightBinding's regular grid (k_x a = -pi + pi/N_x + 2 pi i_x / N_x, k = i_x + N_x (i_y + N_y i_z)),
// so the exponential factorises over the three axes and the k sum is three short DFTs restricted to the R range
// of the table: each pass reads its input once per output R value instead of the N_k x nnz exponentials of the
// reference.  With the full window the Fermi-diagonal part of Matrix_KSBase (:17-22) is overwritten entirely by
// the model-basis block (NBAND = n).
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"
#include "linalg.cuh"

namespace {

constexpr int UF_NMAX = 64;

// column-major n x n products in shared memory, all threads; C distinct from A and B.  ta / tb: use A^H / B^H
__device__ void sm_mm(int n, const double2 *A, bool ta, const double2 *B, bool tb, double2 *C) {
    for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
        const int i = q % n, j = q / n;
        double2 s = cmk(0, 0);
        for (int l = 0; l < n; l++) {
            const double2 a = ta ? cconj(A[l + (size_t)i * n]) : A[i + (size_t)l * n];
            const double2 b = tb ? cconj(B[j + (size_t)l * n]) : B[l + (size_t)j * n];
            s = cfma(a, b, s);
        }
        C[q] = s;
    }
    __syncthreads();
}

// Y = S^-1 X for the Cholesky factor L (lower triangle) of S: forward then back substitution, one column per thread
__device__ void sm_chol_solve(int n, const double2 *L, const double2 *X, bool tx, double2 *Y) {
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        for (int i = 0; i < n; i++) {
            double2 v = tx ? cconj(X[c + (size_t)i * n]) : X[i + (size_t)c * n];
            for (int l = 0; l < i; l++) v = csub(v, cmul(L[i + (size_t)l * n], Y[l + (size_t)c * n]));
            Y[i + (size_t)c * n] = cscale(v, 1.0 / L[i + (size_t)i * n].x);
        }
        for (int i = n - 1; i >= 0; i--) {
            double2 v = Y[i + (size_t)c * n];
            for (int l = i + 1; l < n; l++) v = csub(v, cmul(cconj(L[l + (size_t)i * n]), Y[l + (size_t)c * n]));
            Y[i + (size_t)c * n] = cscale(v, 1.0 / L[i + (size_t)i * n].x);
        }
    }
    __syncthreads();
}

// out: [3][nk][n][n] = (M_dd, M_d, M) per k.  Band window (nband != nullptr, src/upfolding.cpp:10-35): X lives in the
// leading nband[k] x nband[k] block (the padding of a windowed downfolding beyond it); Matrix_KSBase is the Fermi
// diagonal f(e - mu) of every band (the +-100 cut-offs of the reference) with the window's rows and columns
// win[k][0 .. nband[k]-1] replaced by X.
__global__ void __launch_bounds__(128) k_upfold_k(int nk, int n, const double2 *__restrict__ dens,
                                                  const double2 *__restrict__ DF, const double2 *__restrict__ EV,
                                                  const double2 *__restrict__ S, const int *__restrict__ nband,
                                                  const int *__restrict__ win, const double *__restrict__ eps,
                                                  double mu, double beta, double2 *out, int *status) {
    extern __shared__ double2 usm[];
    const int k = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const size_t nn = (size_t)n * n, ko = (size_t)k * nn;
    double2 *A = usm, *B = usm + nn, *C = usm + 2 * nn;
    for (int q = tid; q < (int)nn; q += nt) {
        A[q] = dens[ko + q];
        B[q] = DF[ko + q];
    }
    __syncthreads();
    sm_mm(n, A, false, B, false, C);  // D DF
    sm_mm(n, B, true, C, false, A);   // X = DF^H D DF
    if (nband) {
        const int nb = nband[k];
        for (int q = tid; q < (int)nn; q += nt) {  // Matrix_KSBase into C
            const int i = q % n, j = q / n;
            double f = 0;
            if (i == j) {
                const double x = beta * (eps[(size_t)k * n + i] - mu);
                f = x > 100.0 ? 0.0 : (x < -100.0 ? 1.0 : 1.0 / (1.0 + exp(x)));
            }
            C[q] = cmk(f, 0.0);
        }
        __syncthreads();
        for (int q = tid; q < nb * nb; q += nt) {
            const int a = q % nb, b = q / nb;
            C[win[(size_t)k * n + a] + (size_t)win[(size_t)k * n + b] * n] = A[a + (size_t)b * n];
        }
        __syncthreads();
        for (int q = tid; q < (int)nn; q += nt) A[q] = C[q];
        __syncthreads();
    }
    for (int q = tid; q < (int)nn; q += nt) B[q] = EV[ko + q];
    __syncthreads();
    sm_mm(n, A, false, B, true, C);   // X V^H
    sm_mm(n, B, false, C, false, A);  // D_DFT = V X V^H
    double2 *M = out + 2 * (size_t)nk * nn + ko, *Md = out + (size_t)nk * nn + ko, *Mdd = out + ko;
    for (int q = tid; q < (int)nn; q += nt) M[q] = A[q];
    if (!S) {
        for (int q = tid; q < (int)nn; q += nt) Md[q] = Mdd[q] = A[q];
        return;
    }
    // Cholesky of S into B (lower triangle)
    __shared__ int bad;
    if (tid == 0) bad = 0;
    for (int q = tid; q < (int)nn; q += nt) B[q] = S[ko + q];
    __syncthreads();
    for (int j = 0; j < n; j++) {
        if (tid == 0) {
            const double d = B[j + (size_t)j * n].x;
            if (!(d > 0)) bad = 1;
            B[j + (size_t)j * n] = cmk(d > 0 ? sqrt(d) : 1.0, 0.0);
        }
        __syncthreads();
        const double r = 1.0 / B[j + (size_t)j * n].x;
        for (int i = j + 1 + tid; i < n; i += nt) B[i + (size_t)j * n] = cscale(B[i + (size_t)j * n], r);
        __syncthreads();
        const int t = n - j - 1;
        for (int x = tid; x < t * t; x += nt) {
            const int i = j + 1 + x % t, c = j + 1 + x / t;
            if (c <= i) B[i + (size_t)c * n] = csub(B[i + (size_t)c * n], cmulc(B[i + (size_t)j * n], B[c + (size_t)j * n]));
        }
        __syncthreads();
    }
    sm_chol_solve(n, B, A, false, C);  // M_d = S^-1 D_DFT
    for (int q = tid; q < (int)nn; q += nt) Md[q] = C[q];
    sm_chol_solve(n, B, C, true, A);   // M_dd = S^-1 (S^-1 D_DFT)^H = S^-1 D_DFT S^-1 (D_DFT Hermitian)
    for (int q = tid; q < (int)nn; q += nt) Mdd[q] = A[q];
    if (tid == 0 && bad) dg_flag(status, DG_SINGULAR);
}

// one axis of the k -> R sum: out[o][r][i] = sum_j in[o][j][i] exp(i pi (R0 + r)(2 j + 1 - N) / N), the phase
// table of this block's r in shared memory
__global__ void k_axis_dft(long long outer, int N, int nR, int R0, long long inner, const double2 *__restrict__ in,
                           double2 *out) {
    __shared__ double2 ph[UF_NMAX * 4];
    const int r = blockIdx.y;
    const long long o = blockIdx.z;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const long long num = (long long)(R0 + r) * (2 * j + 1 - N);
        double s, c;
        sincospi((double)(num % (2LL * N)) / N, &s, &c);
        ph[j] = cmk(c, s);
    }
    __syncthreads();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < inner; i += (long long)gridDim.x * blockDim.x) {
        double2 acc = cmk(0, 0);
        const double2 *p = in + (size_t)o * N * inner + i;
        for (int j = 0; j < N; j++) acc = cfma(p[(size_t)j * inner], ph[j], acc);
        out[((size_t)o * nR + r) * inner + i] = acc;
    }
}

// the table's entries of the three R-space sums, divided by N_k
__global__ void k_upfold_gather(int nnz, int n, int nk, const int *__restrict__ rindex, int rx0, int ry0, int rz0, int nrx,
                                int nry, int nrz, const double2 *__restrict__ A3, double2 *o_dd, double2 *o_d,
                                double2 *o) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnz) return;
    const int *r = rindex + 5 * t;
    const size_t nn = (size_t)n * n, box = (size_t)nrx * nry * nrz;
    const size_t cell = (((size_t)(r[2] - rz0) * nry + (r[1] - ry0)) * nrx + (r[0] - rx0)) * nn + r[3] + (size_t)r[4] * n;
    const double s = 1.0 / nk;
    if (o_dd) o_dd[t] = cscale(A3[cell], s);
    if (o_d) o_d[t] = cscale(A3[box * nn + cell], s);
    if (o) o[t] = cscale(A3[2 * box * nn + cell], s);
}

}  // namespace

namespace {

int upfold_impl(dmftgpu_ctx *ctx, int n, int kx, int ky, int kz, const double *dens, const double *df,
                const double *evec, const double *sk, const double *eps, const int *nband, const int *win, double mu,
                double beta, int nnz, const int *rindex, double *dm_dual_dual, double *dm_dual_direct,
                double *dm_direct, int flags) {
    if (!ctx || n < 1 || n > UF_NMAX || kx < 1 || ky < 1 || kz < 1 || kx > UF_NMAX * 4 || ky > UF_NMAX * 4 ||
        kz > UF_NMAX * 4 || !dens || !df || !evec || nnz < 1 || !rindex)
        return DMFTGPU_BADARG;
    if (3LL * ky * kz > 65535) return dg_fail(ctx, DMFTGPU_BADARG, "upfold: ky * kz > 21845");
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int e = 0; e < nnz; e++) {
        const int *r = rindex + 5 * e;
        if (r[3] < 0 || r[3] >= n || r[4] < 0 || r[4] >= n)
            return dg_fail(ctx, DMFTGPU_BADARG, "upfold: orbital index out of range");
        for (int d = 0; d < 3; d++) {
            lo[d] = e ? std::min(lo[d], r[d]) : r[d];
            hi[d] = e ? std::max(hi[d], r[d]) : r[d];
        }
    }
    const int nr[3] = {hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1};
    if (nr[0] > 4096 || nr[1] > 4096 || nr[2] > 4096) return dg_fail(ctx, DMFTGPU_BADARG, "upfold: R range too wide");
    const int nk = kx * ky * kz;
    if (nband) {
        if (!eps || !win || !(beta > 0) || !std::isfinite(mu)) return DMFTGPU_BADARG;
        for (int k = 0; k < nk; k++) {
            if (nband[k] < 1 || nband[k] > n) return dg_fail(ctx, DMFTGPU_BADARG, "upfold: NBAND[k] outside [1, n]");
            for (int j = 0; j < nband[k]; j++) {
                const int b = win[(size_t)k * n + j];
                if (b < 0 || b >= n || (j > 0 && b <= win[(size_t)k * n + j - 1]))
                    return dg_fail(ctx, DMFTGPU_BADARG, "upfold: FromValToKS not ascending band indices");
            }
        }
    }
    DG_CUDA(cudaSetDevice(ctx->device));
    const size_t nn = (size_t)n * n, mb = (size_t)nk * nn * sizeof(double2);
    int st;
    const double2 *dD = (const double2 *)dg_in(ctx, dens, mb, flags, "io.uf_dens", &st);
    if (st) return st;
    const double2 *dF = (const double2 *)dg_in(ctx, df, mb, flags, "io.uf_df", &st);
    if (st) return st;
    const double2 *dV = (const double2 *)dg_in(ctx, evec, mb, flags, "io.uf_ev", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sk, mb, flags, "io.uf_s", &st);
    if (st) return st;
    double2 *o1 = (double2 *)dg_out(ctx, dm_dual_dual, nnz * sizeof(double2), flags, "io.uf_o1", &st);
    if (st) return st;
    double2 *o2 = (double2 *)dg_out(ctx, dm_dual_direct, nnz * sizeof(double2), flags, "io.uf_o2", &st);
    if (st) return st;
    double2 *o3 = (double2 *)dg_out(ctx, dm_direct, nnz * sizeof(double2), flags, "io.uf_o3", &st);
    if (st) return st;
    const size_t s1 = 3 * (size_t)kz * ky * nr[0] * nn, s2 = 3 * (size_t)kz * nr[1] * nr[0] * nn,
                 s3 = 3 * (size_t)nr[2] * nr[1] * nr[0] * nn;
    double2 *M = (double2 *)dg_buf(ctx, "uf.M", 3 * mb);
    double2 *A1 = (double2 *)dg_buf(ctx, "uf.A1", s1 * sizeof(double2));
    double2 *A2 = (double2 *)dg_buf(ctx, "uf.A2", s2 * sizeof(double2));
    double2 *A3 = (double2 *)dg_buf(ctx, "uf.A3", s3 * sizeof(double2));
    int *dR = (int *)dg_buf(ctx, "uf.rindex", (size_t)nnz * 5 * sizeof(int));
    if (!M || !A1 || !A2 || !A3 || !dR) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemcpyAsync(dR, rindex, (size_t)nnz * 5 * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    const double *dE = nullptr;
    int *dnb = nullptr, *dwin = nullptr;
    if (nband) {
        dE = (const double *)dg_in(ctx, eps, (size_t)nk * n * sizeof(double), flags, "io.uf_eps", &st);
        if (st) return st;
        dnb = (int *)dg_buf(ctx, "uf.nband", (size_t)nk * sizeof(int));
        dwin = (int *)dg_buf(ctx, "uf.win", (size_t)nk * n * sizeof(int));
        if (!dnb || !dwin) return DMFTGPU_NOMEM;
        DG_CUDA(cudaMemcpyAsync(dnb, nband, (size_t)nk * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        DG_CUDA(cudaMemcpyAsync(dwin, win, (size_t)nk * n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    }
    DG_TRY(dg_status_reset(ctx));
    const size_t sm = 3 * nn * sizeof(double2);
    DG_CUDA(cudaFuncSetAttribute(k_upfold_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_upfold_k<<<nk, 128, sm, ctx->stream>>>(nk, n, dD, dF, dV, dS, dnb, dwin, dE, mu, beta, M, ctx->d_status);
    DG_LAUNCH(ctx, "k_upfold_k");
    // x: [3 kz ky][kx][n n] -> [3 kz ky][nrx][n n]; y: [3 kz][ky][nrx n n] -> [3 kz][nry][nrx n n];
    // z: [3][kz][nry nrx n n] -> [3][nrz][nry nrx n n]
    struct Pass {
        long long outer;
        int N, nR, R0;
        long long inner;
        const double2 *in;
        double2 *out;
    } passes[3] = {{3LL * kz * ky, kx, nr[0], lo[0], (long long)nn, M, A1},
                   {3LL * kz, ky, nr[1], lo[1], (long long)nr[0] * nn, A1, A2},
                   {3LL, kz, nr[2], lo[2], (long long)nr[1] * nr[0] * nn, A2, A3}};
    for (const Pass &p : passes) {
        const int bx = (int)std::min<long long>(dg_ceil_div(p.inner, 128), 1024);
        dim3 grid(bx, p.nR, (unsigned)p.outer);
        k_axis_dft<<<grid, 128, 0, ctx->stream>>>(p.outer, p.N, p.nR, p.R0, p.inner, p.in, p.out);
        DG_LAUNCH(ctx, "k_axis_dft");
    }
    k_upfold_gather<<<dg_ceil_div(nnz, 128), 128, 0, ctx->stream>>>(nnz, n, nk, dR, lo[0], lo[1], lo[2], nr[0], nr[1],
                                                                     nr[2], A3, o1, o2, o3);
    DG_LAUNCH(ctx, "k_upfold_gather");
    DG_TRY(dg_out_done(ctx, dm_dual_dual, o1, nnz * sizeof(double2), flags));
    DG_TRY(dg_out_done(ctx, dm_dual_direct, o2, nnz * sizeof(double2), flags));
    DG_TRY(dg_out_done(ctx, dm_direct, o3, nnz * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

}  // namespace

extern "C" int dmftgpu_upfold(dmftgpu_ctx *ctx, int n, int kx, int ky, int kz, const double *dens, const double *df,
                              const double *evec, const double *sk, int nnz, const int *rindex, double *dm_dual_dual,
                              double *dm_dual_direct, double *dm_direct, int flags) {
    return upfold_impl(ctx, n, kx, ky, kz, dens, df, evec, sk, nullptr, nullptr, nullptr, 0.0, 1.0, nnz, rindex,
                       dm_dual_dual, dm_dual_direct, dm_direct, flags);
}

extern "C" int dmftgpu_upfold_window(dmftgpu_ctx *ctx, int n, int kx, int ky, int kz, const double *dens,
                                     const double *df, const double *evec, const double *sk, const double *eps,
                                     const int *nband, const int *from_val_to_ks, double mu, double beta, int nnz,
                                     const int *rindex, double *dm_dual_dual, double *dm_dual_direct,
                                     double *dm_direct, int flags) {
    if (!nband || !from_val_to_ks || !eps) return DMFTGPU_BADARG;
    return upfold_impl(ctx, n, kx, ky, kz, dens, df, evec, sk, eps, nband, from_val_to_ks, mu, beta, nnz, rindex,
                       dm_dual_dual, dm_dual_direct, dm_direct, flags);
}
