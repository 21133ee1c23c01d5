// lattice.cu -- the lattice stage of the DMFT iteration on the device:
//   H(k) from t(R)                       (Construct_Hk_Sk, src/ConstructModelHamiltonian.cpp:66-77)
//   G_loc(iw), GwHF(iw), NumMatrix       (GreenFtn_w, src/GreenFtn.cpp:142-422)
//   N(mu), dN/dmu                        (GiwToNele, src/GreenFtn.cpp:513-635, trace form)
//   the chemical-potential search        (GreenFtn_w_adjust_mu, src/GreenFtn.cpp:66-139)
//
// The hot kernel is k_gloc<N,W,MODE>: one CTA owns FPB Matsubara frequencies and sweeps every k point;
// inside, lane groups of W lanes each invert one N x N matrix (iw+mu) I - H(k) - Sigma(iw) held one
// column per lane (warp_gj_inverse) and add the correlated block of G, of G0 = U (iw+mu-e)^-1 U^H and the
// trace terms of N(mu) into per-group shared-memory accumulators.  The k sum is therefore a fixed-order
// in-CTA reduction: no atomics in global memory, no partial buffers, bit-reproducible results.
// Orbitals are permuted so that the correlated (Hartree) orbitals lead; matrices whose dimension is not
// an instantiated N are padded with an identity block (which leaves the leading block's inverse intact).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <type_traits>
#include <vector>

#include "gloc.cuh"
#include "schur.cuh"
#include "smallmat.cuh"
#include "smallmat_df.cuh"
#include "adjoint.cuh"
#include "density.cuh"
#include "trace_tc.h"

namespace {

// ---------------------------------------------------------------------------------------------------
// H(k)
// ---------------------------------------------------------------------------------------------------
// hk[k][e] = sum_R T[R][e] exp(-i (kx ax Rx + ky ay Ry + kz az Rz)), e = i + j n (column-major element)
constexpr int HK_KB = 4;     // k points per CTA
constexpr int HK_RB = 32;    // R vectors per smem tile
constexpr int HK_EB = 64;    // elements per CTA (threads = HK_KB * HK_EB)

__global__ void __launch_bounds__(HK_KB *HK_EB) k_hk(int nk, int nR, int ne, int kx, int ky, int kz,
                                                       const int *__restrict__ R, const double2 *__restrict__ T,
                                                       double2 *__restrict__ hk) {
    __shared__ double2 ph[HK_KB][HK_RB];
    __shared__ double2 tt[HK_RB][HK_EB];
    const int kl = threadIdx.x / HK_EB, el = threadIdx.x % HK_EB;
    const int k = blockIdx.x * HK_KB + kl, e = blockIdx.y * HK_EB + el;
    // k mesh (src/TB.cpp:196-207), ax = ay = az = pi
    const double ax = DG_PI;
    double2 acc = cmk(0, 0);
    for (int r0 = 0; r0 < nR; r0 += HK_RB) {
        __syncthreads();
        for (int t = threadIdx.x; t < HK_KB * HK_RB; t += blockDim.x) {
            int kk = t / HK_RB, rr = t % HK_RB, kg = blockIdx.x * HK_KB + kk;
            double2 v = cmk(0, 0);
            if (kg < nk && r0 + rr < nR) {
                const int kpxy = kx * ky;
                const double delx = 2. * DG_PI / (ax * double(kx)), dely = 2. * DG_PI / (ax * double(ky)),
                             delz = 2. * DG_PI / (ax * double(kz));
                double k0 = -DG_PI / ax + delx / 2. + (kg % kx) * delx;
                double k1 = -DG_PI / ax + dely / 2. + ((kg % kpxy) / kx) * dely;
                double k2 = -DG_PI / ax + delz / 2. + (kg / kpxy) * delz;
                const int *Rv = R + 3 * (r0 + rr);
                double ang = (k0 * ax * Rv[0]) + (k1 * ax * Rv[1]) + (k2 * ax * Rv[2]);
                double s, c;
                sincos(ang, &s, &c);
                v = cmk(c, -s);
            }
            ph[kk][rr] = v;
        }
        for (int t = threadIdx.x; t < HK_RB * HK_EB; t += blockDim.x) {
            int rr = t / HK_EB, ee = t % HK_EB, eg = blockIdx.y * HK_EB + ee;
            tt[rr][ee] = (r0 + rr < nR && eg < ne) ? T[(size_t)(r0 + rr) * ne + eg] : cmk(0, 0);
        }
        __syncthreads();
        const int rmax = min(HK_RB, nR - r0);
        for (int rr = 0; rr < rmax; rr++) acc = cfma(tt[rr][el], ph[kl][rr], acc);
    }
    if (k < nk && e < ne) hk[(size_t)k * ne + e] = acc;
}

// ---------------------------------------------------------------------------------------------------
// per-pass preparation
// ---------------------------------------------------------------------------------------------------
// H'(k) = H(k)[perm][perm] so that the correlated orbitals come first
__global__ void k_permute(int nk, int n, const int *__restrict__ perm, const double2 *__restrict__ H,
                          double2 *__restrict__ Hp) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long tot = (long long)nk * n * n;
    if (t >= tot) return;
    int e = (int)(t % ((long long)n * n));
    long long k = t / ((long long)n * n);
    int i = e % n, j = e / n;
    Hp[t] = H[k * n * n + perm[i] + (size_t)perm[j] * n];
}

// Sigma(iw_n) for n < 2 N_freq: data below N_freq, moment tail above (src/GreenFtn.cpp:224-240 and the
// valenceHAMILTONIAN macro :13-31); `mask` keeps only within-cluster blocks (GiwToNele's placement).
__global__ void k_sigall(int Nf, int D, int nh, int mask, double beta, const double2 *__restrict__ S,
                         const double2 *__restrict__ mom, double2 *__restrict__ sig, double2 *__restrict__ m0eff) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long DD = (long long)D * D;
    if (t < DD) {
        int a = (int)(t % D), b = (int)(t / D);
        m0eff[t] = (mask && (a / nh != b / nh)) ? cmk(0, 0) : mom[t];
    }
    if (t >= 2LL * Nf * DD) return;
    int n = (int)(t / DD), e = (int)(t % DD);
    int a = e % D, b = e / D;
    double2 v;
    if (mask && (a / nh != b / nh)) v = cmk(0, 0);
    else if (n < Nf) v = S[(size_t)n * DD + e];
    else {
        // m0 + m1/iw + m2/iw^2 + m3/iw^3 with iw = i w: 1/iw = -i/w, 1/iw^2 = -1/w^2, 1/iw^3 = i/w^3
        double w = DG_PI * (2. * n + 1.) / beta;
        double2 m0 = mom[e], m1 = mom[DD + e], m2 = mom[2 * DD + e], m3 = mom[3 * DD + e];
        double2 i1 = cmk(0, -1.0 / w), i2 = cmk(-1.0 / (w * w), 0), i3 = cmk(0, 1.0 / (w * w * w));
        v = cadd(cadd(m0, cmul(m1, i1)), cadd(cmul(m2, i2), cmul(m3, i3)));
    }
    sig[t] = v;
}

// static eigen-decomposition of H(k) + S_inf on the correlated block (src/GreenFtn.cpp:197-215): outputs
// eps[k][n], UP[k][l][a] = U(a,l) for a < D (correlated rows of the eigenvectors); and the per-k data of the
// Schur form: H_QQ = V diag(e) V^H, b_l = H_PQ V(:,l) (Q = orbitals D..n-1).
// One block per k, in shared memory (smallmat.cuh's block_heig): the static eigen-decomposition of H(k) + m0
// (same output as k_static_eig) and the Schur data (same output as k_schur_prep).  Shared-memory layout:
// three n x n complex matrices, then eigenvalues [64], order [64], rotations [33], reduction scratch [128].
constexpr int EIG_THREADS = 128, EIG_NMAX = 64;
inline size_t eig_blk_smem(int n) {
    return (size_t)3 * n * n * sizeof(double2) + EIG_NMAX * sizeof(double) + EIG_NMAX * sizeof(int) +
           (EIG_NMAX / 2 + 1) * sizeof(DgRot) + EIG_THREADS * sizeof(double);
}
struct EigSmem {
    double2 *A0, *A, *U;
    double *w;
    int *ord;
    DgRot *rot;
    double *red;
};
__device__ inline EigSmem eig_smem(double2 *sm, int n) {
    EigSmem e;
    const size_t nn = (size_t)n * n;
    e.A0 = sm;
    e.A = sm + nn;
    e.U = sm + 2 * nn;
    e.w = (double *)(sm + 3 * nn);
    e.ord = (int *)(e.w + EIG_NMAX);
    e.rot = (DgRot *)(e.ord + EIG_NMAX);
    e.red = (double *)(e.rot + EIG_NMAX / 2 + 1);
    return e;
}

__global__ void __launch_bounds__(EIG_THREADS) k_static_eig_blk(int n, int D, int nh, int mask,
                                                                const double2 *__restrict__ H,
                                                                const double2 *__restrict__ m0, double *eps,
                                                                double2 *UP, double2 *Uf, int *status) {
    extern __shared__ double2 esm[];
    const int k = blockIdx.x;
    const size_t nn = (size_t)n * n;
    EigSmem e = eig_smem(esm, n);
    const double2 *Hk = H + (size_t)k * nn;
    for (int q = threadIdx.x; q < (int)nn; q += blockDim.x) {
        const int a = q % n, b = q / n;
        double2 v = Hk[q];
        if (a < D && b < D && (!mask || a / nh == b / nh)) v = cadd(v, m0[a + b * D]);
        e.A0[q] = v;
    }
    __syncthreads();
    const int st = block_heig(n, e.A0, e.A, e.U, e.w, e.ord, e.rot, e.red);
    for (int l = threadIdx.x; l < n; l += blockDim.x) eps[(size_t)k * n + l] = e.w[l];
    for (int q = threadIdx.x; q < n * D; q += blockDim.x) {
        const int l = q / D, a = q % D;
        UP[((size_t)k * n + l) * D + a] = DG_AT(e.U, n, a, l);
    }
    if (Uf)
        for (int q = threadIdx.x; q < (int)nn; q += blockDim.x) Uf[(size_t)k * nn + q] = e.U[q];
    if (st && threadIdx.x == 0) dg_flag(status, DG_NONCONV);
}

__global__ void __launch_bounds__(EIG_THREADS) k_schur_prep_blk(int n, int D, const double2 *__restrict__ H,
                                                                double *epsQ, double2 *B, double2 *Vq, int *status) {
    extern __shared__ double2 esm[];
    const int k = blockIdx.x, m = n - D;
    EigSmem e = eig_smem(esm, m);
    const double2 *Hk = H + (size_t)k * n * n;
    for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
        const int i = q % m, j = q / m;
        e.A0[q] = Hk[(D + i) + (size_t)(D + j) * n];
    }
    __syncthreads();
    const int st = block_heig(m, e.A0, e.A, e.U, e.w, e.ord, e.rot, e.red);
    for (int l = threadIdx.x; l < m; l += blockDim.x) epsQ[(size_t)k * m + l] = e.w[l];
    for (int q = threadIdx.x; q < m * D; q += blockDim.x) {
        const int l = q / D, a = q % D;
        double2 s = cmk(0, 0);
        for (int j = 0; j < m; j++) s = cfma(Hk[a + (size_t)(D + j) * n], DG_AT(e.U, m, j, l), s);
        B[((size_t)k * m + l) * D + a] = s;
    }
    if (Vq)
        for (int q = threadIdx.x; q < m * m; q += blockDim.x) Vq[(size_t)k * m * m + q] = e.U[q];
    if (st && threadIdx.x == 0) dg_flag(status, DG_NONCONV);
}

// The same two decompositions with one warp per k point, four k points per CTA: for the matrix sizes up to 32 a
// block-wide Jacobi spends most of its time in block barriers with idle threads.  Ops = OpsD: warp_heig in FP64;
// OpsF (the DMFTGPU_MIXED passes): warp_heig_df, every step in double-float on the FP32 pipe.  Per-warp shared
// region: three n x n complex matrices (16-byte elements either way), eigenvalues [64], order [64], rotations [33].
constexpr int EIG_WPB = 4;
template <class Ops>
__device__ __forceinline__ int warp_heig_ops(int n, const typename Ops::C *A0, typename Ops::C *a,
                                             typename Ops::C *u, double *w, int *order, DgRot *rot) {
    if constexpr (std::is_same<Ops, OpsF>::value) return warp_heig_df(n, A0, a, u, w, order, rot, 1e-24f);
    else return warp_heig(n, A0, a, u, w, order, rot);
}
__host__ __device__ inline size_t warp_eig_bytes(int n) {
    const size_t b = (size_t)3 * n * n * sizeof(double2) + EIG_NMAX * sizeof(double) + EIG_NMAX * sizeof(int) + 16 +
                     (EIG_NMAX / 2 + 1) * sizeof(DgRot);
    return (b + 15) & ~(size_t)15;
}
__device__ inline EigSmem warp_eig_smem(double2 *sm, int n) {
    char *base = reinterpret_cast<char *>(sm) + (threadIdx.x >> 5) * warp_eig_bytes(n);
    EigSmem e;
    const size_t nn = (size_t)n * n;
    e.A0 = reinterpret_cast<double2 *>(base);
    e.A = e.A0 + nn;
    e.U = e.A + nn;
    e.w = (double *)(e.U + nn);
    e.ord = (int *)(e.w + EIG_NMAX);
    e.rot = (DgRot *)(((size_t)(e.ord + EIG_NMAX) + 15) & ~(size_t)15);
    e.red = nullptr;
    return e;
}

template <class Ops>
__global__ void __launch_bounds__(32 * EIG_WPB) k_static_eig_warp(int nk, int n, int D, int nh, int mask,
                                                                  const double2 *__restrict__ H,
                                                                  const double2 *__restrict__ m0, double *eps,
                                                                  double2 *UP, double2 *Uf, int *status) {
    extern __shared__ double2 esm[];
    const int lane = threadIdx.x & 31, k = blockIdx.x * EIG_WPB + (threadIdx.x >> 5);
    if (k >= nk) return;  // whole warps only
    const size_t nn = (size_t)n * n;
    EigSmem e = warp_eig_smem(esm, n);
    typedef typename Ops::C C;
    C *A0 = reinterpret_cast<C *>(e.A0), *A = reinterpret_cast<C *>(e.A), *U = reinterpret_cast<C *>(e.U);
    const double2 *Hk = H + (size_t)k * nn;
    for (int q = lane; q < (int)nn; q += 32) {
        const int a = q % n, b = q / n;
        double2 v = Hk[q];
        if (a < D && b < D && (!mask || a / nh == b / nh)) v = cadd(v, m0[a + b * D]);
        A0[q] = Ops::from(v);
    }
    __syncwarp();
    const int st = warp_heig_ops<Ops>(n, A0, A, U, e.w, e.ord, e.rot);
    for (int l = lane; l < n; l += 32) eps[(size_t)k * n + l] = e.w[l];
    for (int q = lane; q < n * D; q += 32) {
        const int l = q / D, a = q % D;
        UP[((size_t)k * n + l) * D + a] = Ops::to(DG_AT(U, n, a, l));
    }
    if (Uf)
        for (int q = lane; q < (int)nn; q += 32) Uf[(size_t)k * nn + q] = Ops::to(U[q]);
    if (st && lane == 0) dg_flag(status, DG_NONCONV);
}

template <class Ops>
__global__ void __launch_bounds__(32 * EIG_WPB) k_schur_prep_warp(int nk, int n, int D, const double2 *__restrict__ H,
                                                                  double *epsQ, double2 *B, double2 *Vq, int *status) {
    extern __shared__ double2 esm[];
    const int lane = threadIdx.x & 31, k = blockIdx.x * EIG_WPB + (threadIdx.x >> 5), m = n - D;
    if (k >= nk) return;  // whole warps only
    EigSmem e = warp_eig_smem(esm, m);
    typedef typename Ops::C C;
    C *A0 = reinterpret_cast<C *>(e.A0), *A = reinterpret_cast<C *>(e.A), *U = reinterpret_cast<C *>(e.U);
    const double2 *Hk = H + (size_t)k * n * n;
    for (int q = lane; q < m * m; q += 32) {
        const int i = q % m, j = q / m;
        A0[q] = Ops::from(Hk[(D + i) + (size_t)(D + j) * n]);
    }
    __syncwarp();
    const int st = warp_heig_ops<Ops>(m, A0, A, U, e.w, e.ord, e.rot);
    for (int l = lane; l < m; l += 32) epsQ[(size_t)k * m + l] = e.w[l];
    // b_l = H_PQ V(:, l): in the arithmetic of the decomposition, stored in FP64
    for (int q = lane; q < m * D; q += 32) {
        const int l = q / D, a = q % D;
        C s = Ops::zero();
        for (int j = 0; j < m; j++) s = Ops::fma(Ops::from(Hk[a + (size_t)(D + j) * n]), DG_AT(U, m, j, l), s);
        B[((size_t)k * m + l) * D + a] = Ops::to(s);
    }
    if (Vq)
        for (int q = lane; q < m * m; q += 32) Vq[(size_t)k * m * m + q] = Ops::to(U[q]);
    if (st && lane == 0) dg_flag(status, DG_NONCONV);
}

// the Schur data of every k point (H_QQ = V diag(e) V^H, b_l = H_PQ V(:, l)), by warps for m <= 32
int launch_schur_prep(dmftgpu_ctx *ctx, cudaStream_t s, int nk, int n, int D, const double2 *H, double *epsQ,
                      double2 *B, double2 *Vq, bool df = false) {
    const int m = n - D;
    if (m <= 32) {
        const size_t sm = EIG_WPB * warp_eig_bytes(m);
        auto kern = df ? k_schur_prep_warp<OpsF> : k_schur_prep_warp<OpsD>;
        DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        kern<<<dg_ceil_div(nk, EIG_WPB), 32 * EIG_WPB, sm, s>>>(nk, n, D, H, epsQ, B, Vq, ctx->d_status);
        DG_LAUNCH(ctx, "k_schur_prep_warp");
    } else {
        const size_t sm = eig_blk_smem(m);
        DG_CUDA(cudaFuncSetAttribute(k_schur_prep_blk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_schur_prep_blk<<<nk, EIG_THREADS, sm, s>>>(n, D, H, epsQ, B, Vq, ctx->d_status);
        DG_LAUNCH(ctx, "k_schur_prep_blk");
    }
    return DMFTGPU_OK;
}

// Fermi parts: occ_k = P U f U^H P (with the +-100 cut-offs of src/GreenFtn.cpp:314-316) for NumMatrix,
// and sum_l f, beta f (1-f) for N(mu) (src/GreenFtn.cpp:616-620, no cut-off there)
__global__ void k_fermi(int nk, int n, int D, double beta, double mu, const double *__restrict__ eps,
                        const double2 *__restrict__ UP, double2 *occ, double *fs) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    double fsum = 0, dfsum = 0;
    for (int l = 0; l < n; l++) {
        double e = eps[(size_t)k * n + l];
        double f = 1. / (1 + exp(beta * (e - mu)));
        fsum += f;
        dfsum += beta * f * (1 - f);
    }
    fs[2 * k] = fsum;
    fs[2 * k + 1] = dfsum;
    if (!occ) return;
    for (int b = 0; b < D; b++)
        for (int a = 0; a < D; a++) {
            double2 s = cmk(0, 0);
            for (int l = 0; l < n; l++) {
                double x = beta * (eps[(size_t)k * n + l] - mu);
                double f = x > 100.0 ? 0.0 : (x < -100.0 ? 1.0 : 1. / (1. + exp(x)));
                const double2 *u = UP + ((size_t)k * n + l) * D;
                s = cadd(s, cscale(cmulc(u[a], u[b]), f));
            }
            occ[(size_t)k * D * D + a + b * D] = s;
        }
}

// G_loc, GwHF (src/GreenFtn.cpp:298-305, 371-383): scale the per-frequency k sums, keep within-cluster blocks
__global__ void k_gloc_scale(int Nf, int nk, int D, int nh, const double2 *blk, const double2 *blk0, double2 *gw,
                             double2 *gwhf) {
    const long long DD = (long long)D * D;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)Nf * DD) return;
    int e = (int)(t % DD);
    int a = e % D, b = e / D;
    bool same = (a / nh == b / nh);
    gw[t] = same ? cmk(blk[t].x / nk, blk[t].y / nk) : cmk(0, 0);
    if (gwhf) gwhf[t] = same ? cmk(blk0[t].x / nk, blk0[t].y / nk) : cmk(0, 0);
}

// NumMatrix (src/GreenFtn.cpp:283-290, 322-354): one CTA per element, fixed-order tree reductions over the
// 2 N_freq frequency sums and the N_k Fermi terms
__global__ void k_nummat(int Nf, int nk, int D, double beta, const double2 *blk, const double2 *blk0,
                         const double2 *occ, double2 *nummat) {
    __shared__ double2 r0[256], r1[256], r2[256];
    const int DD = D * D, e = blockIdx.x;
    const int a = e % D, b = e / D, et = b + a * D;
    double2 s = cmk(0, 0), s0 = cmk(0, 0), o = cmk(0, 0);
    for (int f = threadIdx.x; f < 2 * Nf; f += blockDim.x) {
        s = cadd(s, cadd(blk[(size_t)f * DD + e], cconj(blk[(size_t)f * DD + et])));
        s0 = cadd(s0, cadd(blk0[(size_t)f * DD + e], cconj(blk0[(size_t)f * DD + et])));
    }
    for (int k = threadIdx.x; k < nk; k += blockDim.x) o = cadd(o, occ[(size_t)k * DD + e]);
    r0[threadIdx.x] = s;
    r1[threadIdx.x] = s0;
    r2[threadIdx.x] = o;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            r0[threadIdx.x] = cadd(r0[threadIdx.x], r0[threadIdx.x + h]);
            r1[threadIdx.x] = cadd(r1[threadIdx.x], r1[threadIdx.x + h]);
            r2[threadIdx.x] = cadd(r2[threadIdx.x], r2[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        s = cmk(r0[0].x / beta, r0[0].y / beta);
        s0 = cmk(r1[0].x / beta, r1[0].y / beta);
        if (a == b) {
            s.x += 0.5 * nk;
            s0.x += 0.5 * nk;
        }
        s = cadd(s, r2[0]);
        s = cmk(s.x / nk, s.y / nk);
        s0 = cmk(s0.x / nk, s0.y / nk);
        nummat[e] = csub(s, s0);
    }
}

// single CTA: N(mu) = (2/beta sum tr + sum f)/nk and dN/dmu
__global__ void k_nele_finalize(int nf2, int nk, double beta, const double *tr, const double *dtr, const double *fs,
                                int deriv, double *out) {
    __shared__ double red[4][256];
    double a = 0, b = 0, c = 0, d = 0;
    for (int f = threadIdx.x; f < nf2; f += blockDim.x) {
        a += tr[f];
        if (deriv) b += dtr[f];
    }
    for (int k = threadIdx.x; k < nk; k += blockDim.x) {
        c += fs[2 * k];
        d += fs[2 * k + 1];
    }
    red[0][threadIdx.x] = a;
    red[1][threadIdx.x] = b;
    red[2][threadIdx.x] = c;
    red[3][threadIdx.x] = d;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 4; q++) red[q][threadIdx.x] += red[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = (red[0][0] * 2. / beta + red[2][0]) / nk;
        out[1] = (red[1][0] * 2. / beta + red[3][0]) / nk;
    }
}

// ---------------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------------
using dg::GlocArgs;
using dg::GlocKernel;
using dg::M_BLOCK;
using dg::M_DERIV;
using dg::M_TRACE;

struct Inst {
    int N, W;
    GlocKernel (*get)(int, bool);
};
const Inst kInst[] = {
    {1, 1, dg::gloc_kernel_1},    {2, 2, dg::gloc_kernel_2},    {3, 4, dg::gloc_kernel_3},
    {4, 4, dg::gloc_kernel_4},    {6, 8, dg::gloc_kernel_6},    {8, 8, dg::gloc_kernel_8},
    {12, 16, dg::gloc_kernel_12}, {16, 16, dg::gloc_kernel_16}, {28, 32, dg::gloc_kernel_28},
};

const Inst *pick_inst(int n) {
    for (const auto &x : kInst)
        if (x.N >= n) return &x;
    return nullptr;
}

using dg::SchurArgs;
using dg::SchurKernel;

// DP: padded correlated-block width; W: lane-group width of the adjoint and density kernels; SW: that of k_schur
// (10-lane packed groups at DP = 10, three per warp)
struct SInst {
    int DP, W, SW;
    SchurKernel (*get)(int, bool);
};
const SInst kSInst[] = {
    {1, 1, 1, dg::schur_kernel_1},      {2, 2, 2, dg::schur_kernel_2},      {3, 4, 4, dg::schur_kernel_3},
    {4, 4, 4, dg::schur_kernel_4},      {6, 8, 8, dg::schur_kernel_6},      {8, 8, 8, dg::schur_kernel_8},
    {10, 16, 10, dg::schur_kernel_10},  {12, 16, 16, dg::schur_kernel_12}, {16, 16, 16, dg::schur_kernel_16},
    {20, 32, 32, dg::schur_kernel_20},
};
const SInst *pick_schur(int D) {
    for (const auto &x : kSInst)
        if (x.DP >= D) return &x;
    return nullptr;
}

// Everything a lattice pass needs, prepared once per (H, Sigma, placement) and reused by every
// N(mu) evaluation of the mu search.
struct Prepared {
    int n, nk, Nf, D, ncl, nh, mask;
    double beta;
    const double2 *H;  // permuted
    double2 *sig, *mom, *UP, *m0, *B;
    double *eps, *epsQ;
    cudaEvent_t static_ready = nullptr;  // recorded on the side stream after the static eigen-decomposition
    double e0 = 0, de = 0, eta = 0;      // real-axis grid (S_REAL passes)
    const int *perm = nullptr;           // device orbital permutation (nullptr: identity)
    double2 *Vq = nullptr, *Uf = nullptr;  // with `vectors`: V of H_QQ [nk][m][m], U of H + m0 [nk][n][n]
    mutable bool tc_ready = false;         // the tensor-core N(mu) pass's per-k operand images are built
};

// the per-k Schur data for a real-axis pass (no self-energy tail, no static spectrum): sig = Sigma(E) as given
int prepare_real(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double2 *dH, const double2 *dSE, int nE,
                 Prepared &P) {
    P.n = L->n;
    P.nk = L->nk;
    P.Nf = nE;
    P.ncl = L->ncl;
    P.nh = L->nh;
    P.D = L->ncl * L->nh;
    P.mask = 0;
    P.beta = L->beta;
    P.H = dH;
    P.sig = const_cast<double2 *>(dSE);
    const int n = P.n, nk = P.nk, D = P.D, m = n - D;
    if (n < 1 || nk < 1 || D < 1 || D > n || !pick_schur(D))
        return dg_fail(ctx, DMFTGPU_BADARG, "gloc_real: unsupported sizes (need 1 <= ncl*nh <= min(n, 20))");
    P.m0 = (double2 *)dg_buf(ctx, "real.m0", (size_t)D * D * sizeof(double2));
    P.epsQ = (double *)dg_buf(ctx, "lat.epsQ", (size_t)nk * (m + 1) * sizeof(double));
    P.B = (double2 *)dg_buf(ctx, "lat.B", (size_t)nk * (m + 1) * D * sizeof(double2));
    if (!P.m0 || !P.epsQ || !P.B) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemsetAsync(P.m0, 0, (size_t)D * D * sizeof(double2), ctx->stream));
    if (m > 0) DG_TRY(launch_schur_prep(ctx, ctx->stream, nk, n, D, P.H, P.epsQ, P.B, nullptr));
    return DMFTGPU_OK;
}

// df (the DMFTGPU_MIXED passes): the per-k eigendecompositions (n <= 32) in double-float on the FP32 pipe, and the
// static one on the main stream after the Schur data instead of on the side stream (the mixed lattice kernels fill
// the SMs; an eigendecomposition beside them slows them by more than it takes alone)
int prepare(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double2 *dH, const double2 *dS, int mask, Prepared &P,
            bool vectors = false, bool df = false) {
    P.n = L->n;
    P.nk = L->nk;
    P.Nf = L->nfreq;
    P.ncl = L->ncl;
    P.nh = L->nh;
    P.D = L->ncl * L->nh;
    P.mask = mask;
    P.beta = L->beta;
    const int n = P.n, nk = P.nk, D = P.D, Nf = P.Nf;
    if (n < 1 || nk < 1 || Nf < 1 || D < 1 || D > n || !pick_schur(D))
        return dg_fail(ctx, DMFTGPU_BADARG, "lattice: unsupported sizes (need 1 <= ncl*nh <= min(n, 20))");
    cudaStream_t s = ctx->stream;
    // orbital permutation: Hartree orbitals first, the rest in their order
    std::vector<int> perm;
    bool identity = true;
    if (L->hartr) {
        std::vector<char> used(n, 0);
        for (int i = 0; i < D; i++) {
            int h = L->hartr[i];
            if (h < 0 || h >= n || used[h]) return dg_fail(ctx, DMFTGPU_BADARG, "lattice: bad HartrIndex");
            used[h] = 1;
            perm.push_back(h);
            if (h != i) identity = false;
        }
        for (int i = 0; i < n; i++)
            if (!used[i]) perm.push_back(i);
    }
    if (identity) P.H = dH;
    else {
        int *dperm = (int *)dg_buf(ctx, "lat.perm", n * sizeof(int));
        double2 *Hp = (double2 *)dg_buf(ctx, "lat.Hperm", (size_t)nk * n * n * sizeof(double2));
        if (!dperm || !Hp) return DMFTGPU_NOMEM;
        DG_CUDA(cudaMemcpyAsync(dperm, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, s));
        long long tot = (long long)nk * n * n;
        k_permute<<<dg_ceil_div(tot, 256), 256, 0, s>>>(nk, n, dperm, dH, Hp);
        DG_LAUNCH(ctx, "k_permute");
        P.H = Hp;
        P.perm = dperm;
    }
    P.mom = (double2 *)dg_buf(ctx, "lat.mom", 4 * (size_t)D * D * sizeof(double2));
    P.sig = (double2 *)dg_buf(ctx, "lat.sig", 2 * (size_t)Nf * D * D * sizeof(double2));
    P.eps = (double *)dg_buf(ctx, "lat.eps", (size_t)nk * n * sizeof(double));
    P.UP = (double2 *)dg_buf(ctx, "lat.UP", (size_t)nk * n * D * sizeof(double2));
    P.m0 = (double2 *)dg_buf(ctx, "lat.m0", (size_t)D * D * sizeof(double2));
    const int m = n - D;
    P.epsQ = (double *)dg_buf(ctx, "lat.epsQ", (size_t)nk * (m + 1) * sizeof(double));
    P.B = (double2 *)dg_buf(ctx, "lat.B", (size_t)nk * (m + 1) * D * sizeof(double2));
    if (!P.m0 || !P.epsQ || !P.B) return DMFTGPU_NOMEM;
    if (n > EIG_NMAX) return dg_fail(ctx, DMFTGPU_BADARG, "lattice: n > 64");
    if (!P.mom || !P.sig || !P.eps || !P.UP) return DMFTGPU_NOMEM;
    if (vectors) {
        P.Vq = (double2 *)dg_buf(ctx, "lat.Vq", (size_t)nk * (m * m + 1) * sizeof(double2));
        P.Uf = (double2 *)dg_buf(ctx, "lat.Uf", (size_t)nk * n * n * sizeof(double2));
        if (!P.Vq || !P.Uf) return DMFTGPU_NOMEM;
    }
    DG_TRY(dg_moments_dev(ctx, D, Nf, P.beta, dS, 0, P.mom));
    long long tot = 2LL * Nf * D * D;
    k_sigall<<<dg_ceil_div(tot, 256), 256, 0, s>>>(Nf, D, P.nh, mask, P.beta, dS, P.mom, P.sig, P.m0);
    DG_LAUNCH(ctx, "k_sigall");
    // the Schur data (eigen-decomposition of H_QQ) is needed first, by k_schur, on the main stream; the
    // static eigen-decomposition of H + m0 feeds only the Fermi terms, so it runs on the side stream
    // (FP64-pipe work) while the lattice kernel (FP32 pipe in the mixed form) proceeds
    if (m > 0) DG_TRY(launch_schur_prep(ctx, s, nk, n, D, P.H, P.epsQ, P.B, P.Vq, df));
    DG_CUDA(cudaEventRecord(ctx->ev_fork, s));
    DG_CUDA(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    cudaStream_t es = df ? s : ctx->side;
    if (n <= 32) {
        const size_t sm = EIG_WPB * warp_eig_bytes(n);
        auto kern = df ? k_static_eig_warp<OpsF> : k_static_eig_warp<OpsD>;
        DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        kern<<<dg_ceil_div(nk, EIG_WPB), 32 * EIG_WPB, sm, es>>>(nk, n, D, P.nh, mask, P.H, P.m0, P.eps, P.UP, P.Uf,
                                                                 ctx->d_status);
        DG_LAUNCH(ctx, "k_static_eig_warp");
    } else {
        const size_t sm = eig_blk_smem(n);
        DG_CUDA(cudaFuncSetAttribute(k_static_eig_blk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_static_eig_blk<<<nk, EIG_THREADS, sm, es>>>(n, D, P.nh, mask, P.H, P.m0, P.eps, P.UP, P.Uf, ctx->d_status);
        DG_LAUNCH(ctx, "k_static_eig_blk");
    }
    DG_CUDA(cudaEventRecord(ctx->ev_join, ctx->side));
    P.static_ready = ctx->ev_join;
    return DMFTGPU_OK;
}

int run_gloc(dmftgpu_ctx *ctx, const Prepared &P, int mode, double mu, int wgrid, double2 *blk, double2 *blk0,
             double *tr, double *dtr, bool mixed) {
    const Inst *in = pick_inst(P.n);
    if (!in) return dg_fail(ctx, DMFTGPU_BADARG, "explicit inversion: n > 28 not instantiated");
    GlocKernel kern = in->get(mode, mixed);
    int fpb = 4;
    auto smem_for = [&](int f) {
        return dg::gloc_smem(in->N, in->W, mode, f, P.D, mixed ? sizeof(cdf) : sizeof(double2));
    };
    while (fpb > 1 && smem_for(fpb) > 160 * 1024) fpb--;
    size_t smem = smem_for(fpb);
    if (smem > 200 * 1024) return dg_fail(ctx, DMFTGPU_BADARG, "lattice: correlated block too large");
    DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    GlocArgs g;
    g.H = P.H;
    g.sig = P.sig;
    g.eps = P.eps;
    g.UP = P.UP;
    g.n = P.n;
    g.nk = P.nk;
    g.nf2 = 2 * P.Nf;
    g.D = P.D;
    g.fpb = fpb;
    g.wgrid = wgrid;
    g.beta = P.beta;
    g.mu = mu;
    g.blk = blk;
    g.blk0 = blk0;
    g.tr = tr;
    g.dtr = dtr;
    g.status = ctx->d_status;
    // every mode reads the static spectrum (e_l for Tr G0 and the G0 block, U for the G0 block), computed on the
    // side stream
    DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
    {
        DgTimer tm(ctx, "k_gloc");
        kern<<<dg_ceil_div(g.nf2, fpb), 128, smem, ctx->stream>>>(g);
    }
    DG_LAUNCH(ctx, "k_gloc");
    return DMFTGPU_OK;
}


// fixed-order sum of the per-chunk partial sums
__global__ void k_schur_reduce(int nchunk, int nf2, int DD, int mode, const double2 *pblk, const double2 *pblk0,
                               const double2 *ptr, double2 *blk, double2 *blk0, double *tr, double *dtr) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((mode & dg::S_BLOCK) && t < (long long)nf2 * DD) {
        double2 s = cmk(0, 0), s0 = cmk(0, 0);
        for (int q = 0; q < nchunk; q++) {
            s = cadd(s, pblk[(size_t)q * nf2 * DD + t]);
            s0 = cadd(s0, pblk0[(size_t)q * nf2 * DD + t]);
        }
        blk[t] = s;
        if (blk0) blk0[t] = s0;
    }
    if ((mode & dg::S_TRACE) && t < nf2) {
        double a = 0, b = 0;
        for (int q = 0; q < nchunk; q++) {
            a += ptr[(size_t)q * nf2 + t].x;
            b += ptr[(size_t)q * nf2 + t].y;
        }
        tr[t] = a;
        if (dtr) dtr[t] = b;
    }
}

// the Schur-form pass (default); mode: dg::S_BLOCK (GreenFtn_w) or S_TRACE[|S_DERIV] (N(mu))
int run_schur(dmftgpu_ctx *ctx, const Prepared &P, int mode, double mu, int wgrid, double2 *blk, double2 *blk0,
              double *tr, double *dtr, bool mixed) {
    const SInst *in = pick_schur(P.D);
    // BLOCK passes of correlated blocks up to 3 x 3: one thread per frequency (k_schur_tpi).  It stages the
    // Hermitian pole products of each staged k; prepare() caps n at 64 (the static eigensolver), so one k needs
    // at most 63 * (3 * 16 + 3 * 8 + 8) + 9 * 16 B = 5.2 KB and the 200 KB check below never rejects a tpi pass.
    const bool tpi = mode == dg::S_BLOCK && P.D <= 3;
    SchurKernel kern = tpi ? dg::schur_tpi_kernel(P.D, mixed) : in->get(mode, mixed);
    const int m = P.n - P.D, NG = tpi ? 128 : dg::schur_groups(in->SW), DD = P.D * P.D;
    const int nf2 = (mode & dg::S_REAL) ? P.Nf : 2 * P.Nf;  // the real axis has exactly the caller's points
    auto smem_of = [&](int kc_) {
        return tpi ? dg::schur_tpi_smem(kc_, P.D, m) : dg::schur_smem(in->DP, in->SW, mode, kc_, P.D, m, P.n);
    };
    int kc = 16;
    while (kc > 1 && smem_of(kc) > 96 * 1024) kc /= 2;
    const size_t smem = smem_of(kc);
    if (smem > 200 * 1024) return dg_fail(ctx, DMFTGPU_BADARG, "lattice: correlated block too large");
    DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // k chunks: enough CTAs for `cps` per SM (8 unless tuned), at least 64 k points per chunk
    const int fblocks = dg_ceil_div(nf2, NG);
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    auto chunks = [&](int cps, int *kchunk_out) {
        int nc = std::max(1, std::min(dg_ceil_div(P.nk, 64), dg_ceil_div(cps * nsm, fblocks)));
        const int kch = dg_ceil_div(P.nk, nc);
        *kchunk_out = kch;
        return dg_ceil_div(P.nk, kch);
    };
    const std::string key = std::string(tpi ? "schur_tpi/" : "schur/") + std::to_string(in->DP) + "/" + std::to_string(mode) + "/" +
                            std::to_string((int)mixed) + "/" + std::to_string(P.nk) + "/" + std::to_string(nf2);
    int kch_max;
    const int nchunk_max = chunks(16, &kch_max);
    double2 *pblk = nullptr, *pblk0 = nullptr, *ptr = nullptr;
    if (mode & dg::S_BLOCK) {
        pblk = (double2 *)dg_buf(ctx, "schur.pblk", (size_t)nchunk_max * nf2 * DD * sizeof(double2));
        pblk0 = (double2 *)dg_buf(ctx, "schur.pblk0", (size_t)nchunk_max * nf2 * DD * sizeof(double2));
        if (!pblk || !pblk0) return DMFTGPU_NOMEM;
    }
    if (mode & dg::S_TRACE) {
        ptr = (double2 *)dg_buf(ctx, "schur.ptr", (size_t)nchunk_max * nf2 * sizeof(double2));
        if (!ptr) return DMFTGPU_NOMEM;
    }
    int kchunk;
    int nchunk = chunks(8, &kchunk);
    dg::SchurArgs g;
    g.H = P.H;
    g.B = P.B;
    g.epsQ = P.epsQ;
    g.sig = P.sig;
    g.m0 = P.m0;
    g.eps0 = P.eps;
    g.UP = P.UP;
    g.n = P.n;
    g.m = m;
    g.nk = P.nk;
    g.nf2 = nf2;
    g.D = P.D;
    g.wgrid = wgrid;
    g.e0 = P.e0;
    g.de = P.de;
    g.eta = P.eta;
    g.kc = kc;
    g.kchunk = kchunk;
    g.beta = P.beta;
    g.mu = mu;
    g.pblk = pblk;
    g.pblk0 = pblk0;
    g.ptr = ptr;
    g.status = ctx->d_status;
    // the TRACE passes read the static eigenvalues (Tr G0), computed on the side stream
    if (!(mode & dg::S_REAL) && ((mode & dg::S_TRACE) || ((mode & dg::S_BLOCK) && in->DP >= 8)))
        DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
    // autotuning: time 4, 8 and 16 CTAs per SM once per (width, mode, precision, N_k, points) and keep the fastest
    auto tuned = ctx->tuned.find(key);
    if (tuned != ctx->tuned.end()) {
        nchunk = chunks(tuned->second, &kchunk);
        g.kchunk = kchunk;
    } else if (ctx->autotune && !ctx->capturing) {
        // the two timing events are released on every exit, an error return included
        struct EventPair {
            cudaEvent_t a = nullptr, b = nullptr;
            ~EventPair() {
                if (a) cudaEventDestroy(a);
                if (b) cudaEventDestroy(b);
            }
        } ev;
        DG_CUDA(cudaEventCreate(&ev.a));
        DG_CUDA(cudaEventCreate(&ev.b));
        float best = 1e30f;
        int best_cps = 8;
        for (int cps : {4, 8, 16}) {
            int kch;
            const int nc = chunks(cps, &kch);
            g.kchunk = kch;
            DG_CUDA(cudaEventRecord(ev.a, ctx->stream));
            kern<<<dim3(fblocks, nc), 128, smem, ctx->stream>>>(g);
            DG_LAUNCH(ctx, "k_schur (autotune)");
            DG_CUDA(cudaEventRecord(ev.b, ctx->stream));
            DG_CUDA(cudaEventSynchronize(ev.b));
            float ms = 0;
            DG_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
            if (ms < best) {
                best = ms;
                best_cps = cps;
            }
        }
        ctx->tuned[key] = best_cps;
        nchunk = chunks(best_cps, &kchunk);
        g.kchunk = kchunk;
    }
    {
        DgTimer tm(ctx, "k_schur");
        kern<<<dim3(fblocks, nchunk), 128, smem, ctx->stream>>>(g);
    }
    DG_LAUNCH(ctx, "k_schur");
    const long long nred = (mode & dg::S_BLOCK) ? std::max((long long)nf2 * DD, (long long)nf2) : nf2;
    k_schur_reduce<<<dg_ceil_div(nred, 256), 256, 0, ctx->stream>>>(nchunk, nf2, DD, mode, pblk, pblk0, ptr, blk, blk0,
                                                                     tr, dtr);
    DG_LAUNCH(ctx, "k_schur_reduce");
    return DMFTGPU_OK;
}

// one N(mu) evaluation on a prepared lattice; result (N, dN/dmu) in device out[2]
int nele_pass(dmftgpu_ctx *ctx, const Prepared &P, double mu, bool deriv, double *dout, bool explicit_inv,
              bool mixed) {
    const int nf2 = 2 * P.Nf;
    double *tr = (double *)dg_buf(ctx, "nele.tr", nf2 * sizeof(double));
    double *dtr = (double *)dg_buf(ctx, "nele.dtr", nf2 * sizeof(double));
    double *fs = (double *)dg_buf(ctx, "nele.fs", 2 * (size_t)P.nk * sizeof(double));
    if (!tr || !dtr || !fs) return DMFTGPU_NOMEM;
    if (explicit_inv) {
        DG_TRY(run_gloc(ctx, P, deriv ? (M_TRACE | M_DERIV) : M_TRACE, mu, 1, nullptr, nullptr, tr, dtr, mixed));
    } else if (mixed && !deriv && ctx->tensor && !ctx->capturing && dg_trace_tc_supported(P.n, P.D)) {
        // the pole sums on the tensor cores (trace_tc.cu)
        DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
        TraceTcArgs a;
        a.H = P.H;
        a.B = P.B;
        a.epsQ = P.epsQ;
        a.sig = P.sig;
        a.eps0 = P.eps;
        a.n = P.n;
        a.m = P.n - P.D;
        a.nk = P.nk;
        a.nf2 = nf2;
        a.D = P.D;
        a.wgrid = 1;
        a.beta = P.beta;
        a.mu = mu;
        DG_TRY(dg_trace_tc(ctx, a, &P.tc_ready, tr));
    } else {
        DG_TRY(run_schur(ctx, P, deriv ? (dg::S_TRACE | dg::S_DERIV) : dg::S_TRACE, mu, 1, nullptr, nullptr, tr, dtr,
                         mixed));
    }
    DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
    k_fermi<<<dg_ceil_div(P.nk, 128), 128, 0, ctx->stream>>>(P.nk, P.n, P.D, P.beta, mu, P.eps, P.UP, nullptr, fs);
    DG_LAUNCH(ctx, "k_fermi");
    k_nele_finalize<<<1, 256, 0, ctx->stream>>>(nf2, P.nk, P.beta, tr, dtr, fs, deriv ? 1 : 0, dout);
    DG_LAUNCH(ctx, "k_nele_finalize");
    return DMFTGPU_OK;
}

int nele_host(dmftgpu_ctx *ctx, const Prepared &P, double mu, bool deriv, double *N, double *dN, bool explicit_inv,
              bool mixed) {
    double *dout = (double *)dg_buf(ctx, "nele.out", 2 * sizeof(double));
    if (!dout) return DMFTGPU_NOMEM;
    DG_TRY(nele_pass(ctx, P, mu, deriv, dout, explicit_inv, mixed));
    double h[2];
    DG_CUDA(cudaMemcpyAsync(h, dout, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    *N = h[0];
    if (dN) *dN = h[1];
    return DMFTGPU_OK;
}

int check_lat(const dmftgpu_lattice *L) {
    if (!L || L->n < 1 || L->nk < 1 || L->nfreq < 1 || L->ncl < 1 || L->nh < 1 || !(L->beta > 0))
        return DMFTGPU_BADARG;
    return DMFTGPU_OK;
}


// fixed-order sums over chunks of the derivative kernel's partials, scaled
__global__ void k_ad_reduce(int nchunk, long long len, double scale, const double2 *p, double2 *out) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= len) return;
    double2 s = cmk(0, 0);
    for (int q = 0; q < nchunk; q++) s = cadd(s, p[(size_t)q * len + t]);
    out[t] = cscale(s, scale);
}
__global__ void k_ad_mu(int n, double scale, const double *p, double *out) {
    __shared__ double red[256];
    double s = 0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) s += p[t];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0] * scale;
}

struct AdInst {
    int DP, W;
    dg::AdKernel (*get)(int);
};
const AdInst kAdInst[] = {
    {1, 1, dg::ad_kernel_1},    {2, 2, dg::ad_kernel_2},    {3, 4, dg::ad_kernel_3},   {4, 4, dg::ad_kernel_4},
    {6, 8, dg::ad_kernel_6},    {8, 8, dg::ad_kernel_8},    {10, 16, dg::ad_kernel_10}, {12, 16, dg::ad_kernel_12},
    {16, 16, dg::ad_kernel_16}, {20, 32, dg::ad_kernel_20},
};

// one derivative pass: VJP (gin = Gbar; out = Sigma_bar; *dmu_out = mu_bar on the device) or JVP (gin =
// Sigma_dot, mu_dot; out = G_loc_dot)
int run_ad(dmftgpu_ctx *ctx, const Prepared &P, int mode, double mu, const double2 *gin, double mu_dot, double2 *out,
           double *dmu_out) {
    const AdInst *in = nullptr;
    for (const auto &x : kAdInst)
        if (x.DP >= P.D) {
            in = &x;
            break;
        }
    if (!in) return dg_fail(ctx, DMFTGPU_BADARG, "derivatives: correlated block larger than 20");
    dg::AdKernel kern = in->get(mode);
    const int m = P.n - P.D, NG = 128 / in->W, nf = P.Nf, DD = P.D * P.D;
    int kc = 16;
    while (kc > 1 && dg::ad_smem(in->DP, in->W, kc, P.D, m) > 96 * 1024) kc /= 2;
    const size_t smem = dg::ad_smem(in->DP, in->W, kc, P.D, m);
    DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int fblocks = dg_ceil_div(nf, NG);
    int nchunk = std::max(1, std::min(dg_ceil_div(P.nk, 64), dg_ceil_div(8 * 152, fblocks)));
    const int kchunk = dg_ceil_div(P.nk, nchunk);
    nchunk = dg_ceil_div(P.nk, kchunk);
    double2 *pout = (double2 *)dg_buf(ctx, "ad.pout", (size_t)nchunk * nf * DD * sizeof(double2));
    double *pmu = (double *)dg_buf(ctx, "ad.pmu", (size_t)nchunk * nf * sizeof(double));
    if (!pout || !pmu) return DMFTGPU_NOMEM;
    dg::AdArgs g;
    g.H = P.H;
    g.B = P.B;
    g.epsQ = P.epsQ;
    g.sig = P.sig;  // the first nf slots are the input Sigma(iw_n)
    g.gin = gin;
    g.mu_dot = mu_dot;
    g.n = P.n;
    g.m = m;
    g.nk = P.nk;
    g.nf = nf;
    g.D = P.D;
    g.kc = kc;
    g.kchunk = kchunk;
    g.beta = P.beta;
    g.mu = mu;
    g.pout = pout;
    g.pmu = pmu;
    g.status = ctx->d_status;
    {
        DgTimer tm(ctx, "k_gloc_ad");
        kern<<<dim3(fblocks, nchunk), 128, smem, ctx->stream>>>(g);
    }
    DG_LAUNCH(ctx, "k_gloc_ad");
    const long long len = (long long)nf * DD;
    k_ad_reduce<<<dg_ceil_div(len, 256), 256, 0, ctx->stream>>>(nchunk, len, 1.0 / P.nk, pout, out);
    DG_LAUNCH(ctx, "k_ad_reduce");
    if (mode == dg::AD_VJP) {
        k_ad_mu<<<1, 256, 0, ctx->stream>>>(nchunk * nf, -1.0 / P.nk, pmu, dmu_out);
        DG_LAUNCH(ctx, "k_ad_mu");
    }
    return DMFTGPU_OK;
}


// GreenFtn_w on device arrays, enqueue only (the body of dmftgpu_greenftn_w and of each batched problem)
int greenftn_w_dev(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double2 *dH, const double2 *dS, double mu,
                   double2 *dG, double2 *dG0, double2 *dN, int flags) {
    const int D = L->ncl * L->nh, Nf = L->nfreq;
    const size_t DD = (size_t)D * D;
    Prepared P;
    DG_TRY(prepare(ctx, L, dH, dS, 0, P, false, (flags & DMFTGPU_MIXED) != 0));
    double2 *blk = (double2 *)dg_buf(ctx, "gloc.blk", 2 * Nf * DD * sizeof(double2));
    double2 *blk0 = (double2 *)dg_buf(ctx, "gloc.blk0", 2 * Nf * DD * sizeof(double2));
    double2 *occ = (double2 *)dg_buf(ctx, "gloc.occ", (size_t)L->nk * DD * sizeof(double2));
    double *fs = (double *)dg_buf(ctx, "gloc.fs", 2 * (size_t)L->nk * sizeof(double));
    if (!blk || !blk0 || !occ || !fs) return DMFTGPU_NOMEM;
    if (flags & DMFTGPU_EXPLICIT)
        DG_TRY(run_gloc(ctx, P, M_BLOCK, mu, 0, blk, blk0, nullptr, nullptr, (flags & DMFTGPU_MIXED) != 0));
    else DG_TRY(run_schur(ctx, P, dg::S_BLOCK, mu, 0, blk, blk0, nullptr, nullptr, (flags & DMFTGPU_MIXED) != 0));
    DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
    k_fermi<<<dg_ceil_div(L->nk, 128), 128, 0, ctx->stream>>>(L->nk, L->n, D, L->beta, mu, P.eps, P.UP, occ, fs);
    DG_LAUNCH(ctx, "k_fermi");
    k_gloc_scale<<<dg_ceil_div((long long)Nf * DD, 256), 256, 0, ctx->stream>>>(Nf, L->nk, D, L->nh, blk, blk0, dG, dG0);
    DG_LAUNCH(ctx, "k_gloc_scale");
    k_nummat<<<(int)DD, 256, 0, ctx->stream>>>(Nf, L->nk, D, L->beta, blk, blk0, occ, dN);
    DG_LAUNCH(ctx, "k_nummat");
    return DMFTGPU_OK;
}


// densityMatDFT, the second half (src/GreenFtn.cpp:311-319): per k, X' = sum over splits of Y + Y^H (the P-Q block is
// already the Hermitian combination), X = T X' T^H with T = diag(I, V), then
// dens = X / beta + U diag(f(e0) - R / beta) U^H (Fermi factors with the +-100 cut-offs), stored in the caller's
// orbital order.  One block per k; two n x n tiles in shared memory.
__global__ void __launch_bounds__(128) k_dens_finish(int nk, int n, int D, int nsplit, double beta, double mu,
                                                     const double2 *__restrict__ Y, const double *__restrict__ R,
                                                     const double2 *__restrict__ Vq, const double2 *__restrict__ Uf,
                                                     const double *__restrict__ eps0, const int *__restrict__ perm,
                                                     double2 *dens) {
    extern __shared__ double2 fsm[];
    const int k = blockIdx.x, m = n - D, nn = n * n, tid = threadIdx.x, nt = blockDim.x;
    double2 *X = fsm, *T = fsm + nn;
    double *gw = (double *)(T + nn);
    for (int q = tid; q < nn; q += nt) {
        double2 v = cmk(0, 0);
        for (int sp = 0; sp < nsplit; sp++) v = cadd(v, Y[((size_t)sp * nk + k) * nn + q]);
        T[q] = v;
    }
    for (int j = tid; j < n; j += nt) {
        double r = 0;
        for (int sp = 0; sp < nsplit; sp++) r += R[((size_t)sp * nk + k) * n + j];
        const double x = beta * (eps0[(size_t)k * n + j] - mu);
        const double f = x > 100.0 ? 0.0 : (x < -100.0 ? 1.0 : 1. / (1. + exp(x)));
        gw[j] = f - r / beta;
    }
    __syncthreads();
    for (int q = tid; q < nn; q += nt) {
        const int i = q % n, j = q / n;
        if ((i < D) == (j < D)) X[q] = cadd(T[q], cconj(T[j + i * n]));
        else if (i < D) X[q] = T[q];
        else X[q] = cconj(T[j + i * n]);
    }
    __syncthreads();
    if (m > 0) {
        const double2 *V = Vq + (size_t)k * m * m;  // V(i, l) = V[i + l m]
        for (int q = tid; q < nn; q += nt) {
            const int i = q % n, j = q / n;
            if (j < D) T[q] = X[q];
            else {
                double2 v = cmk(0, 0);
                for (int l = 0; l < m; l++) v = cfma(X[i + (D + l) * n], cconj(V[(j - D) + (size_t)l * m]), v);
                T[q] = v;
            }
        }
        __syncthreads();
        for (int q = tid; q < nn; q += nt) {
            const int i = q % n, j = q / n;
            if (i < D) X[q] = T[q];
            else {
                double2 v = cmk(0, 0);
                for (int l = 0; l < m; l++) v = cfma(V[(i - D) + (size_t)l * m], T[(D + l) + j * n], v);
                X[q] = v;
            }
        }
        __syncthreads();
    }
    const double2 *U = Uf + (size_t)k * nn;
    for (int q = tid; q < nn; q += nt) {
        const int i = q % n, j = q / n;
        double2 v = cscale(X[q], 1.0 / beta);
        for (int l = 0; l < n; l++) v = cfma(cscale(U[i + (size_t)l * n], gw[l]), cconj(U[j + (size_t)l * n]), v);
        const int pi = perm ? perm[i] : i, pj = perm ? perm[j] : j;
        dens[(size_t)k * nn + pi + (size_t)pj * n] = v;
    }
}

using dg::DensArgs;
using dg::DensKernel;
DensKernel pick_dens(int DP, bool mixed) {
    switch (DP) {
        case 1: return dg::dens_kernel_1(mixed);
        case 2: return dg::dens_kernel_2(mixed);
        case 3: return dg::dens_kernel_3(mixed);
        case 4: return dg::dens_kernel_4(mixed);
        case 6: return dg::dens_kernel_6(mixed);
        case 8: return dg::dens_kernel_8(mixed);
        case 10: return dg::dens_kernel_10(mixed);
        case 12: return dg::dens_kernel_12(mixed);
        case 16: return dg::dens_kernel_16(mixed);
        case 20: return dg::dens_kernel_20(mixed);
    }
    return nullptr;
}

// densityMatDFT for a prepared lattice (prepare(..., vectors = true)): enqueue only; mixed: the per-(k, iw) work in
// double-float
int run_density(dmftgpu_ctx *ctx, const Prepared &P, double mu, double2 *dens, bool mixed) {
    const int n = P.n, D = P.D, m = n - D, nk = P.nk, nf2 = 2 * P.Nf;
    const SInst *si = pick_schur(D);
    DensKernel kern = si ? pick_dens(si->DP, mixed) : nullptr;
    if (!kern) return dg_fail(ctx, DMFTGPU_BADARG, "density: unsupported correlated block");
    const int DP = si->DP, W = si->W;
    // groups per CTA: the most resident warps per SM within 227 KB of shared memory per CTA
    const size_t smem_cap = 227 * 1024, sm_per_sm = 228 * 1024;
    int ng = 0, best = -1;
    for (int g = 1; g * W <= 128; g++) {
        const size_t sm = dg::dens_smem(DP, D, m, n, g);
        if (sm > smem_cap) break;
        const int ctas = std::min((int)(sm_per_sm / (sm + 1024)), 2048 / (g * W));
        const int warps = ctas * ((g * W + 31) / 32);
        if (warps >= best) {
            best = warps;
            ng = g;
        }
    }
    if (!ng) return dg_fail(ctx, DMFTGPU_BADARG, "density: model too large for one k point's shared memory");
    const size_t smem = dg::dens_smem(DP, D, m, n, ng);
    const int ctas_per_sm = std::max(1, (int)(sm_per_sm / (smem + 1024)));
    int nsplit = dg_ceil_div(2LL * 152 * ctas_per_sm, nk);
    nsplit = std::max(1, std::min(nsplit, std::max(1, nf2 / (4 * ng))));
    double2 *Y = (double2 *)dg_buf(ctx, "dens.Y", (size_t)nsplit * nk * n * n * sizeof(double2));
    double *R = (double *)dg_buf(ctx, "dens.R", (size_t)nsplit * nk * n * sizeof(double));
    if (!Y || !R) return DMFTGPU_NOMEM;
    DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
    DensArgs g;
    g.H = P.H;
    g.B = P.B;
    g.epsQ = P.epsQ;
    g.eps0 = P.eps;
    g.sig = P.sig;
    g.n = n;
    g.m = m;
    g.nk = nk;
    g.nf2 = nf2;
    g.D = D;
    g.ng = ng;
    g.beta = P.beta;
    g.mu = mu;
    g.Y = Y;
    g.R = R;
    g.status = ctx->d_status;
    DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    {
        DgTimer tm(ctx, "k_dens_sum");
        kern<<<dim3(nk, nsplit), ng * W, smem, ctx->stream>>>(g);
    }
    DG_LAUNCH(ctx, "k_dens_sum");
    const size_t fs = 2 * (size_t)n * n * sizeof(double2) + n * sizeof(double);
    DG_CUDA(cudaFuncSetAttribute(k_dens_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs));
    k_dens_finish<<<nk, 128, fs, ctx->stream>>>(nk, n, D, nsplit, P.beta, mu, Y, R, P.Vq, P.Uf, P.eps, P.perm, dens);
    DG_LAUNCH(ctx, "k_dens_finish");
    return DMFTGPU_OK;
}

// the real-axis sums divided by N_k: G_PP blocks, and Tr G as (re, im)
__global__ void k_real_finish(int nE, int DD, int nk, const double2 *blk, const double *tr, double2 *g, double2 *trace) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < (long long)nE * DD) g[t] = cscale(blk[t], 1.0 / nk);
    if (t < nE) trace[t] = cmk(tr[t] / nk, tr[nE + t] / nk);
}

}  // namespace

extern "C" {

int dmftgpu_hk(dmftgpu_ctx *ctx, int n, int nnz, const int *rindex, const double *hr, int kx, int ky, int kz,
               double *hk, int flags) {
    if (!ctx || n < 1 || nnz < 0 || !rindex || !hr || !hk || kx < 1 || ky < 1 || kz < 1) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    // group the read_HR rows by lattice vector into a dense [N_R][n*n] table (duplicates add up, as the
    // reference's += does)
    std::map<std::array<int, 3>, int> rid;
    std::vector<std::array<int, 3>> Rl;
    for (int e = 0; e < nnz; e++) {
        const int *r = rindex + 5 * e;
        if (r[3] < 0 || r[3] >= n || r[4] < 0 || r[4] >= n) return dg_fail(ctx, DMFTGPU_BADARG, "hk: orbital index");
        std::array<int, 3> key = {r[0], r[1], r[2]};
        if (!rid.count(key)) {
            rid[key] = (int)Rl.size();
            Rl.push_back(key);
        }
    }
    const int nR = std::max(1, (int)Rl.size()), ne = n * n, nk = kx * ky * kz;
    std::vector<double2> T((size_t)nR * ne, make_double2(0, 0));
    std::vector<int> Rv(3 * (size_t)nR, 0);
    for (size_t i = 0; i < Rl.size(); i++)
        for (int d = 0; d < 3; d++) Rv[3 * i + d] = Rl[i][d];
    for (int e = 0; e < nnz; e++) {
        const int *r = rindex + 5 * e;
        int q = rid[{r[0], r[1], r[2]}];
        double2 &t = T[(size_t)q * ne + r[3] + (size_t)r[4] * n];
        t.x += hr[2 * e];
        t.y += hr[2 * e + 1];
    }
    int *dR = (int *)dg_buf(ctx, "hk.R", Rv.size() * sizeof(int));
    double2 *dT = (double2 *)dg_buf(ctx, "hk.T", T.size() * sizeof(double2));
    if (!dR || !dT) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemcpyAsync(dR, Rv.data(), Rv.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    DG_CUDA(cudaMemcpyAsync(dT, T.data(), T.size() * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    int st;
    double2 *dH = (double2 *)dg_out(ctx, hk, (size_t)nk * ne * sizeof(double2), flags, "io.hk", &st);
    if (st) return st;
    if ((flags & DMFTGPU_MIXED) && !(flags & DMFTGPU_NO_TENSOR)) {
        // split precision on the tensor cores (hk_tc.cu); the phase image is keyed by the mesh and the R list
        std::string key = std::to_string(kx) + "x" + std::to_string(ky) + "x" + std::to_string(kz) + ":";
        unsigned long long h = 1469598103934665603ull;
        for (int v : Rv) h = (h ^ (unsigned long long)(unsigned)v) * 1099511628211ull;
        key += std::to_string(Rl.size()) + ":" + std::to_string(h);
        DG_TRY(dg_status_reset(ctx));
        DG_TRY(dg_hk_tensor(ctx, n, (int)Rl.size(), dR, dT, kx, ky, kz, dH, key));
    } else {
        dim3 grid(dg_ceil_div(nk, HK_KB), dg_ceil_div(ne, HK_EB));
        k_hk<<<grid, HK_KB * HK_EB, 0, ctx->stream>>>(nk, (int)Rl.size(), ne, kx, ky, kz, dR, dT, dH);
        DG_LAUNCH(ctx, "k_hk");
    }
    DG_TRY(dg_out_done(ctx, hk, dH, (size_t)nk * ne * sizeof(double2), flags));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    if ((flags & DMFTGPU_MIXED) && !(flags & DMFTGPU_NO_TENSOR)) {
        int code = 0;
        DG_TRY(dg_status_read(ctx, &code));
        return code;
    }
    return DMFTGPU_OK;
}

int dmftgpu_greenftn_w(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const double *sigma, double mu,
                       double *gw, double *gwhf, double *nummat, int flags) {
    if (!ctx || check_lat(L) || !hk || !sigma || !gw || !nummat) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    const int D = L->ncl * L->nh, Nf = L->nfreq;
    const size_t DD = (size_t)D * D;
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, (size_t)L->nk * L->n * L->n * sizeof(double2), flags, "io.hk_in", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma, Nf * DD * sizeof(double2), flags, "io.sigma", &st);
    if (st) return st;
    double2 *dG = (double2 *)dg_out(ctx, gw, Nf * DD * sizeof(double2), flags, "io.gw", &st);
    if (st) return st;
    double2 *dG0 = gwhf ? (double2 *)dg_out(ctx, gwhf, Nf * DD * sizeof(double2), flags, "io.gwhf", &st) : nullptr;
    if (st) return st;
    double2 *dN = (double2 *)dg_out(ctx, nummat, DD * sizeof(double2), flags, "io.nummat", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(greenftn_w_dev(ctx, L, dH, dS, mu, dG, dG0, dN, flags));
    DG_TRY(dg_out_done(ctx, gw, dG, Nf * DD * sizeof(double2), flags));
    if (gwhf) DG_TRY(dg_out_done(ctx, gwhf, dG0, Nf * DD * sizeof(double2), flags));
    DG_TRY(dg_out_done(ctx, nummat, dN, DD * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

// GreenFtn_w for a batch of independent lattice problems (ragged sizes): each problem has its own workspaces
// and runs on one of four stream pairs, so small problems overlap; DMFTGPU_GRAPH replays the whole batched pass
// as one CUDA graph (captured on the first call after a warm-up call with the same problem set);
// DMFTGPU_AUTOTUNE tunes each Schur kernel's chunking on first use.
int dmftgpu_greenftn_w_batched(dmftgpu_ctx *ctx, int nprob, const dmftgpu_lattice *lats, const double *const *hk,
                               const double *const *sigma, const double *mu, double *const *gw, double *const *gwhf,
                               double *const *nummat, int flags) {
    if (!ctx || nprob < 1 || !lats || !hk || !sigma || !mu || !gw || !nummat) return DMFTGPU_BADARG;
    if (!(flags & DMFTGPU_DEVICE_PTRS)) return dg_fail(ctx, DMFTGPU_BADARG, "greenftn_w_batched: device pointers only");
    if (flags & DMFTGPU_EXPLICIT) return dg_fail(ctx, DMFTGPU_BADARG, "greenftn_w_batched: Schur form only");
    for (int i = 0; i < nprob; i++)
        if (check_lat(&lats[i]) || lats[i].hartr || !hk[i] || !sigma[i] || !gw[i] || !nummat[i])
            return dg_fail(ctx, DMFTGPU_BADARG, "greenftn_w_batched: bad problem (HartrIndex must be the identity)");
    cudaSetDevice(ctx->device);
    const int NL = 4;
    if (ctx->lanes.empty()) {
        ctx->lanes.resize(NL);
        for (auto &l : ctx->lanes) {
            DG_CUDA(cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking));
            DG_CUDA(cudaStreamCreateWithFlags(&l.side, cudaStreamNonBlocking));
            DG_CUDA(cudaEventCreateWithFlags(&l.fork, cudaEventDisableTiming));
            DG_CUDA(cudaEventCreateWithFlags(&l.join, cudaEventDisableTiming));
            DG_CUDA(cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming));
        }
        DG_CUDA(cudaEventCreateWithFlags(&ctx->ev_batch, cudaEventDisableTiming));
        DG_CUDA(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
    }
    // identity of this batched call: sizes, pointers and flags (a graph replays exactly these)
    std::string key = std::to_string(flags);
    for (int i = 0; i < nprob; i++) {
        const dmftgpu_lattice &L = lats[i];
        char b[256];
        snprintf(b, sizeof(b), "|%d,%d,%d,%.17g,%d,%d,%p,%p,%.17g,%p,%p,%p", L.n, L.nk, L.nfreq, L.beta, L.ncl, L.nh,
                 (const void *)hk[i], (const void *)sigma[i], mu[i], (void *)gw[i], gwhf ? (void *)gwhf[i] : nullptr,
                 (void *)nummat[i]);
        key += b;
    }
    DG_TRY(dg_status_reset(ctx));
    if ((flags & DMFTGPU_GRAPH) && ctx->graph && ctx->graph_key == key) {
        DG_CUDA(cudaGraphLaunch(ctx->graph, ctx->stream));
    } else {
        const bool capture = (flags & DMFTGPU_GRAPH) && ctx->graph_key == "warm:" + key;
        cudaStream_t user = ctx->stream, side0 = ctx->side;
        cudaStream_t origin = capture ? ctx->cap_stream : user;
        cudaEvent_t fork0 = ctx->ev_fork, join0 = ctx->ev_join;
        ctx->autotune = (flags & DMFTGPU_AUTOTUNE) != 0 && !capture;
        if (capture) {
            DG_CUDA(cudaEventRecord(ctx->ev_batch, user));
            DG_CUDA(cudaStreamWaitEvent(origin, ctx->ev_batch, 0));
            DG_CUDA(cudaStreamBeginCapture(origin, cudaStreamCaptureModeRelaxed));
            ctx->capturing = true;
        }
        int rc = DMFTGPU_OK;
        if (cudaEventRecord(ctx->ev_batch, origin) != cudaSuccess) rc = DMFTGPU_CUDA_ERROR;
        for (int l = 0; l < NL && !rc; l++)
            if (cudaStreamWaitEvent(ctx->lanes[l].stream, ctx->ev_batch, 0) != cudaSuccess) rc = DMFTGPU_CUDA_ERROR;
        for (int i = 0; i < nprob && !rc; i++) {
            auto &ln = ctx->lanes[i % NL];
            ctx->stream = ln.stream;
            ctx->side = ln.side;
            ctx->ev_fork = ln.fork;
            ctx->ev_join = ln.join;
            ctx->buf_ns = "b" + std::to_string(i) + "/";
            rc = greenftn_w_dev(ctx, &lats[i], (const double2 *)hk[i], (const double2 *)sigma[i], mu[i],
                                (double2 *)gw[i], gwhf ? (double2 *)gwhf[i] : nullptr, (double2 *)nummat[i],
                                flags & ~DMFTGPU_EXPLICIT);
        }
        for (int l = 0; l < NL; l++) {
            cudaEventRecord(ctx->lanes[l].done, ctx->lanes[l].stream);
            cudaStreamWaitEvent(origin, ctx->lanes[l].done, 0);
        }
        ctx->stream = user;
        ctx->side = side0;
        ctx->ev_fork = fork0;
        ctx->ev_join = join0;
        ctx->buf_ns.clear();
        ctx->autotune = false;
        if (capture) {
            cudaGraph_t graph = nullptr;
            ctx->capturing = false;
            cudaError_t e = cudaStreamEndCapture(origin, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess) return dg_set_cuda_error(ctx, e, "greenftn_w_batched: capture");
            if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
            ctx->graph = nullptr;
            e = cudaGraphInstantiate(&ctx->graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return dg_set_cuda_error(ctx, e, "greenftn_w_batched: instantiate");
            ctx->graph_key = key;
            DG_CUDA(cudaGraphLaunch(ctx->graph, user));
        } else {
            if (rc) return rc;
            if (flags & DMFTGPU_GRAPH) ctx->graph_key = "warm:" + key;
        }
    }
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

// retarded lattice Green function on a real-energy grid (retarded_GreenFtn2, src/GreenFtn.cpp:425-466, as
// summed over k by qs_spectra, src/qs_spectra.cpp:99-130): gloc[nE] = (1/N_k) sum_k G_PP(k, E) and trace[nE] =
// (1/N_k) sum_k Tr G(k, E) over the whole model space, G = (E + mu + i eta - H - Sigma(E))^-1
int dmftgpu_gloc_real(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const double *sigma_e, int nE,
                      double e0, double de, double eta, double mu, double *gloc, double *trace, int flags) {
    if (!ctx || check_lat(L) || !hk || !sigma_e || !gloc || !trace || nE < 1 || !(eta > 0)) return DMFTGPU_BADARG;
    if (L->ncl != 1 || L->hartr) return dg_fail(ctx, DMFTGPU_BADARG, "gloc_real: one cluster, HartrIndex identity");
    cudaSetDevice(ctx->device);
    const int D = L->nh;
    const size_t DD = (size_t)D * D;
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, (size_t)L->nk * L->n * L->n * sizeof(double2), flags, "io.hk_in", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma_e, (size_t)nE * DD * sizeof(double2), flags, "io.sigma_e", &st);
    if (st) return st;
    double2 *dG = (double2 *)dg_out(ctx, gloc, (size_t)nE * DD * sizeof(double2), flags, "io.gloc_e", &st);
    if (st) return st;
    double2 *dT = (double2 *)dg_out(ctx, trace, (size_t)nE * sizeof(double2), flags, "io.trace_e", &st);
    if (st) return st;
    double2 *blk = (double2 *)dg_buf(ctx, "real.blk", (size_t)nE * DD * sizeof(double2));
    double *tr = (double *)dg_buf(ctx, "real.tr", 2 * (size_t)nE * sizeof(double));
    if (!blk || !tr) return DMFTGPU_NOMEM;
    DG_TRY(dg_status_reset(ctx));
    Prepared P;
    DG_TRY(prepare_real(ctx, L, dH, dS, nE, P));
    P.e0 = e0;
    P.de = de;
    P.eta = eta;
    DG_TRY(run_schur(ctx, P, dg::S_BLOCK | dg::S_TRACE | dg::S_REAL, mu, 0, blk, nullptr, tr, tr + nE,
                     (flags & DMFTGPU_MIXED) != 0));
    k_real_finish<<<dg_ceil_div((long long)nE * DD, 256), 256, 0, ctx->stream>>>(nE, (int)DD, L->nk, blk, tr, dG, dT);
    DG_LAUNCH(ctx, "k_real_finish");
    DG_TRY(dg_out_done(ctx, gloc, dG, (size_t)nE * DD * sizeof(double2), flags));
    DG_TRY(dg_out_done(ctx, trace, dT, (size_t)nE * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

// reverse mode: Sigma_bar = (1/N_k) sum_k G^H Gbar G^H, mu_bar = -(1/N_k) sum Re Tr[(G S' G)^H Gbar]
int dmftgpu_gloc_vjp(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const double *sigma, double mu,
                     const double *gbar, double *sigma_bar, double *mu_bar, int flags) {
    if (!ctx || check_lat(L) || !hk || !sigma || !gbar || !sigma_bar || !mu_bar) return DMFTGPU_BADARG;
    if (L->ncl != 1) return dg_fail(ctx, DMFTGPU_BADARG, "gloc_vjp: one correlated cluster");
    cudaSetDevice(ctx->device);
    const int D = L->nh, Nf = L->nfreq;
    const size_t DD = (size_t)D * D;
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, (size_t)L->nk * L->n * L->n * sizeof(double2), flags, "io.hk_in", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma, Nf * DD * sizeof(double2), flags, "io.sigma", &st);
    if (st) return st;
    const double2 *dGb = (const double2 *)dg_in(ctx, gbar, Nf * DD * sizeof(double2), flags, "io.gbar", &st);
    if (st) return st;
    double2 *dSb = (double2 *)dg_out(ctx, sigma_bar, Nf * DD * sizeof(double2), flags, "io.sigbar", &st);
    if (st) return st;
    double *dmu = (double *)dg_buf(ctx, "ad.mubar", sizeof(double));
    if (!dmu) return DMFTGPU_NOMEM;
    DG_TRY(dg_status_reset(ctx));
    Prepared P;
    DG_TRY(prepare(ctx, L, dH, dS, 0, P));
    DG_TRY(run_ad(ctx, P, dg::AD_VJP, mu, dGb, 0.0, dSb, dmu));
    DG_TRY(dg_out_done(ctx, sigma_bar, dSb, Nf * DD * sizeof(double2), flags));
    DG_CUDA(cudaMemcpyAsync(mu_bar, dmu, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

// densityMatDFT of GreenFtn_w: dens[nk][n][n]
int dmftgpu_density_dft(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const double *sigma, double mu,
                        double *dens, int flags) {
    if (!ctx || check_lat(L) || !hk || !sigma || !dens) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    const int D = L->ncl * L->nh, Nf = L->nfreq;
    const size_t DD = (size_t)D * D, nb = (size_t)L->nk * L->n * L->n * sizeof(double2);
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, nb, flags, "io.hk_in", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma, Nf * DD * sizeof(double2), flags, "io.sigma", &st);
    if (st) return st;
    double2 *dD = (double2 *)dg_out(ctx, dens, nb, flags, "io.dens", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    Prepared P;
    DG_TRY(prepare(ctx, L, dH, dS, 0, P, true));
    DG_TRY(run_density(ctx, P, mu, dD, (flags & DMFTGPU_MIXED) != 0));
    DG_TRY(dg_out_done(ctx, dens, dD, nb, flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

// forward mode: G_loc_dot = (1/N_k) sum_k G (Sigma_dot - mu_dot S') G
int dmftgpu_gloc_jvp(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const double *sigma, double mu,
                     const double *sigma_dot, double mu_dot, double *gloc_dot, int flags) {
    if (!ctx || check_lat(L) || !hk || !sigma || !sigma_dot || !gloc_dot) return DMFTGPU_BADARG;
    if (L->ncl != 1) return dg_fail(ctx, DMFTGPU_BADARG, "gloc_jvp: one correlated cluster");
    cudaSetDevice(ctx->device);
    const int D = L->nh, Nf = L->nfreq;
    const size_t DD = (size_t)D * D;
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, (size_t)L->nk * L->n * L->n * sizeof(double2), flags, "io.hk_in", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma, Nf * DD * sizeof(double2), flags, "io.sigma", &st);
    if (st) return st;
    const double2 *dSd = (const double2 *)dg_in(ctx, sigma_dot, Nf * DD * sizeof(double2), flags, "io.sigdot", &st);
    if (st) return st;
    double2 *dGd = (double2 *)dg_out(ctx, gloc_dot, Nf * DD * sizeof(double2), flags, "io.glocdot", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    Prepared P;
    DG_TRY(prepare(ctx, L, dH, dS, 0, P));
    DG_TRY(run_ad(ctx, P, dg::AD_JVP, mu, dSd, mu_dot, dGd, nullptr));
    DG_TRY(dg_out_done(ctx, gloc_dot, dGd, Nf * DD * sizeof(double2), flags));
    DG_CUDA(cudaStreamWaitEvent(ctx->stream, P.static_ready, 0));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

int dmftgpu_nele(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const double *sigma, double mu,
                 double *nele, double *dnele, int flags) {
    if (!ctx || check_lat(L) || !hk || !sigma || !nele) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgTensorMode tmode(ctx, flags);
    const size_t DD = (size_t)L->ncl * L->nh * L->ncl * L->nh;
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, (size_t)L->nk * L->n * L->n * sizeof(double2), flags, "io.hk_in", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma, L->nfreq * DD * sizeof(double2), flags, "io.sigma", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    Prepared P;
    DG_TRY(prepare(ctx, L, dH, dS, 1, P, false, (flags & DMFTGPU_MIXED) != 0));
    DG_TRY(nele_host(ctx, P, mu, dnele != nullptr, nele, dnele, (flags & DMFTGPU_EXPLICIT) != 0,
                     (flags & DMFTGPU_MIXED) != 0));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    if (code) return code;
    if (!std::isfinite(*nele)) return DMFTGPU_NAN;
    return DMFTGPU_OK;
}

int dmftgpu_adjust_mu(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const double *sigma, double mu,
                      double dmu, double n_target, double *mu_out, int *n_eval, int flags) {
    if (!ctx || check_lat(L) || !hk || !sigma || !mu_out) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgTensorMode tmode(ctx, flags);
    const size_t DD = (size_t)L->ncl * L->nh * L->ncl * L->nh;
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, hk, (size_t)L->nk * L->n * L->n * sizeof(double2), flags, "io.hk_in", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma, L->nfreq * DD * sizeof(double2), flags, "io.sigma", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    Prepared P;
    DG_TRY(prepare(ctx, L, dH, dS, 1, P, false, (flags & DMFTGPU_MIXED) != 0));
    int evals = 0;
    auto N = [&](double m, double *out, double *dout) {
        evals++;
        return nele_host(ctx, P, m, dout != nullptr, out, dout, (flags & DMFTGPU_EXPLICIT) != 0,
                         (flags & DMFTGPU_MIXED) != 0);
    };
    const double goal = n_target;
    // every exit reads the status word the N(mu) kernels raise (DG_SINGULAR for a zero pivot ...): a flagged
    // code takes precedence over the search's own outcome, so a singular inversion is never reported as OK.
    auto finish = [&](int ret, double mu_final) {
        *mu_out = mu_final;
        if (n_eval) *n_eval = evals;
        int code = 0;
        int rs = dg_status_read(ctx, &code);
        if (rs) return rs;
        return code ? code : ret;
    };
    if (flags & DMFTGPU_NEWTON) {
        // safeguarded Newton: keep a bracket [lo, hi] with N(lo) < goal < N(hi) once found.  The first step
        // uses dN/dmu from the derivative pass; later steps take the secant slope of the last two evaluations
        // (a plain N(mu) pass costs ~45% of a derivative pass), falling back to a derivative pass whenever
        // that slope is not positive.
        double lo = -1e300, hi = 1e300, Nv, dN;
        double pmu = 0, pN = 0;
        bool need_deriv = true;
        for (int it = 0; it < 100; it++) {
            if (need_deriv) {
                DG_TRY(N(mu, &Nv, &dN));
            } else {
                DG_TRY(N(mu, &Nv, nullptr));
                dN = (Nv - pN) / (mu - pmu);
            }
            if (!std::isfinite(Nv)) return finish(DMFTGPU_NAN, mu);
            need_deriv = !(dN > 0) || !std::isfinite(dN);
            pmu = mu;
            pN = Nv;
            double r = Nv - goal;
            if (r < 0) lo = std::max(lo, mu);
            else hi = std::min(hi, mu);
            if (std::fabs(r) <= 1e-11 * std::max(1.0, std::fabs(goal))) return finish(DMFTGPU_OK, mu);
            double step = (dN > 0) ? -r / dN : (r < 0 ? std::fabs(dmu) : -std::fabs(dmu));
            double next = mu + step;
            if (!(next > lo && next < hi)) {
                if (lo > -1e299 && hi < 1e299) next = 0.5 * (lo + hi);
                else next = mu + (r < 0 ? std::fabs(dmu) : -std::fabs(dmu));
            }
            if (std::fabs(next - mu) < 1e-15 * std::max(1.0, std::fabs(mu))) return finish(DMFTGPU_OK, next);
            mu = next;
        }
        return finish(DMFTGPU_NONCONVERGED, mu);
    }
    // the reference's bracket expansion + bisection (src/GreenFtn.cpp:81-121)
    double Nele[2] = {-1, -1};
    DG_TRY(N(mu, &Nele[0], nullptr));
    if (!std::isfinite(Nele[0])) return finish(DMFTGPU_NAN, mu);
    double muUB = 0, muLB = 0, mu_next;
    int nearAns = 0;
    if (Nele[0] > goal) mu -= (dmu - dmu);
    else if (Nele[0] < goal) mu -= (dmu + dmu);
    int guard = 0;
    while ((Nele[0] != goal) && std::abs(dmu) > 1e-5) {
        if (++guard > 10000) return finish(DMFTGPU_NONCONVERGED, mu);
        mu += dmu;
        Nele[1] = Nele[0];
        DG_TRY(N(mu, &Nele[0], nullptr));
        if (nearAns == 0) {
            if (Nele[0] < goal) {
                muLB = mu;
                if (Nele[1] > goal && Nele[1] > 0) nearAns = 1;
                else dmu = std::fabs(dmu);
            }
            if (Nele[0] > goal) {
                muUB = mu;
                if (Nele[1] < goal && Nele[1] > 0) nearAns = 1;
                else dmu = -1 * std::fabs(dmu);
            }
            if (Nele[0] == goal) break;
            if (!(std::abs(mu) < 600)) return finish(DMFTGPU_NONCONVERGED, mu);
        } else {
            if (Nele[0] > goal) muUB = mu;
            else if (Nele[0] < goal) muLB = mu;
            mu_next = (muUB + muLB) / 2.;
            dmu = mu_next - mu;
        }
    }
    return finish(DMFTGPU_OK, mu);
}

}  // extern "C"
