// impurity.cu -- impurity-side kernels of the DMFT iteration:
//   Construct_hyb_delta                  (src/Construct_hyb_delta.cpp:47-119)
//   FourierTransform_ / _tau (iw -> tau)  (src/FourierTransform.cpp:16-178) with the two-pole tail
//   FT_t_to_w (tau -> iw)                 (src/FourierTransform.cpp:521-561)
//   getStimp (second-order Sigma(tau))    (src/SCGF2_fullLoop.cpp:603-690)
//   getFockOperator, getGwimp, getoccMat, estimate_asymto  (src/SCGF2_fullLoop.cpp:539-597, 736-787)
// Matsubara phases are taken from an exact table of exp(-i pi q / N_tau), q = (2n+1) j mod 2 N_tau, instead
// of exp(-i w tau) of a rounded product (the reference's phase error grows to ~1e-12 at w tau ~ 1e4).
// Both transforms are discrete Fourier sums over the grids w_n = pi (2n+1)/beta, tau_j = j beta / N_tau:
//   iw -> tau:  S_j = sum_n D_n e^{-i w_n tau_j} = e^{-i pi j/N} X_{j mod N},  X = DFT_N of D (zero padded)
//   tau -> iw:  the exact integral of the piecewise-linear F(tau) against e^{i w tau} (FT_t_to_w) is, summed
//     over hat functions, W_n = dt K(t_n) (Y_n - F_0) + dt (F_0 E(t_n) - F_N conj E(t_n)), t_n = w_n dt,
//     Y_n = sum_{s<N} F_s e^{i w_n tau_s} (an inverse DFT_N of F_s e^{i pi s/N}), K(t) = (sin(t/2)/(t/2))^2,
//     E(t) = (e^{it} - 1 - it)/(it)^2
// so for N_tau a power of two <= 8192 both run as shared-memory radix-2 FFTs (O(N log N) per element instead of
// O(N_w N_tau)).  The FFT form is also free of the cancellation in the reference's per-segment formula, which
// loses ~1e-10 relative at the lowest frequencies; DMFTGPU_DIRECT_DFT selects the direct per-point sums that
// follow the reference's arithmetic.
#include <algorithm>
#include <vector>

#include "impurity.h"
#include "smallmat.cuh"
#include "df.cuh"

namespace {

// ---------------------------------------------------------------------------------------------------
// Construct_hyb_delta: one thread per Matsubara frequency (src/Construct_hyb_delta.cpp:98-113)
// ---------------------------------------------------------------------------------------------------
__global__ void k_hyb_delta(int dim, int nfreq, int D, double beta, double mu, const int *__restrict__ orb,
                            const double2 *__restrict__ S, const double2 *__restrict__ G,
                            const double2 *__restrict__ Himp, double2 *work, int *iwork, double2 *delta,
                            int *status) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nfreq) return;
    const size_t DD = (size_t)D * D, dd = (size_t)dim * dim;
    double2 *g = work + (size_t)n * dd;
    for (int h2 = 0; h2 < dim; h2++)
        for (int h1 = 0; h1 < dim; h1++) DG_AT(g, dim, h1, h2) = G[n * DD + orb[h1] + (size_t)orb[h2] * D];
    if (dim != 0 && thread_gj_inverse(dim, g, iwork + (size_t)n * dim)) dg_flag(status, DG_SINGULAR);
    const double2 iw = cmk(0.0, DG_PI * (2. * n + 1.) / beta);
    double2 *out = delta + (size_t)n * dd;
    for (int h1 = 0; h1 < dim; h1++) {
        for (int h2 = 0; h2 < dim; h2++) {
            double2 hs = Himp[orb[h1] + (size_t)orb[h2] * D], ss = S[n * DD + orb[h1] + (size_t)orb[h2] * D];
            DG_AT(out, dim, h1, h2) = csub(csub(cneg(hs), ss), DG_AT(g, dim, h1, h2));
        }
        double2 v = DG_AT(out, dim, h1, h1);
        v = cadd(v, iw);
        v.x += mu;
        DG_AT(out, dim, h1, h1) = v;
    }
}

// ---------------------------------------------------------------------------------------------------
// FourierTransform_tau: the tau-independent tail data (src/FourierTransform.cpp:22-44, 66-83)
// ---------------------------------------------------------------------------------------------------
// T layout (complex slots, d x d each): V, H, H2, UH, UH2, then eH, eH2 (d doubles each, in a slot), then
// W1 = UH^H V, W2 = UH2^H V (the tail term V^H G0_H(tau) V = W1^H diag(g(tau)) W1)
constexpr int TAIL_SLOTS = 9;
struct TailPtrs {
    double2 *V, *H, *H2, *UH, *UH2, *W1, *W2;
    double *eH, *eH2;
};
__device__ TailPtrs tail_ptrs(double2 *T, int d) {
    const size_t dd = (size_t)d * d;
    TailPtrs p;
    p.V = T;
    p.H = T + dd;
    p.H2 = T + 2 * dd;
    p.UH = T + 3 * dd;
    p.UH2 = T + 4 * dd;
    p.eH = (double *)(T + 5 * dd);
    p.eH2 = (double *)(T + 6 * dd);
    p.W1 = T + 7 * dd;
    p.W2 = T + 8 * dd;
    return p;
}

// FourierTransform_tau's tail data (src/FourierTransform.cpp:22-44, 66-83) by one block, the smallmat.cuh
// routines in shared memory: V = sqrt(m1); M2' = V^-H (2 m2) V^-1, M3' likewise; H = M2'/2 + sqrt(M3'/2 -
// M2'^2/4) (or M2'/2 if that is not positive), H2 = M2' - H; eigen-decompositions of H and H2.  V^-1 =
// U diag(ev^-1/2) U^H comes from the same eigen-decomposition as V = U diag(ev^1/2) U^H.
constexpr int TAIL_THREADS = 128;
__host__ __device__ inline size_t tail_smem_bytes(int d) {
    return (size_t)8 * d * d * sizeof(double2) + 32 * sizeof(double) + 32 * sizeof(int) + 17 * sizeof(DgRot) +
           TAIL_THREADS * sizeof(double);
}
__global__ void __launch_bounds__(TAIL_THREADS) k_tail_setup_blk(int d, const double2 *mom, double2 *T, int *status) {
    extern __shared__ double2 sm[];
    const int dd = d * d, tid = threadIdx.x, nt = blockDim.x;
    double2 *A = sm, *U = A + dd, *X = U + dd, *M2 = X + dd, *M3 = M2 + dd, *t1 = M3 + dd, *V = t1 + dd, *Vi = V + dd;
    double *ev = (double *)(Vi + dd);
    int *ord = (int *)(ev + 32);
    DgRot *rot = (DgRot *)(ord + 32);
    double *red = (double *)(rot + 17);
    TailPtrs p = tail_ptrs(T, d);
    const double2 *m1 = mom + dd, *m2 = mom + 2 * dd, *m3 = mom + 3 * dd;
    int st = block_heig(d, m1, A, U, ev, ord, rot, red);
    const bool pos = ev[0] > 0;
    if (pos) {
        for (int e = tid; e < dd; e += nt) {
            const int i = e % d, j = e / d;
            double2 sv = cmk(0, 0), si = cmk(0, 0);
            for (int l = 0; l < d; l++) {
                const double2 uu = cmul(DG_AT(U, d, i, l), cconj(DG_AT(U, d, j, l)));
                const double r = sqrt(ev[l]);
                sv = cadd(sv, cscale(uu, r));
                si = cadd(si, cscale(uu, 1.0 / r));
            }
            V[e] = sv;
            Vi[e] = si;
            X[e] = cscale(m2[e], 2.0);
        }
        __syncthreads();
        block_matmul(d, Vi, X, t1);
        block_matmul(d, t1, Vi, M2);                      // M2' = V^-H (2 m2) V^-1
        for (int e = tid; e < dd; e += nt) X[e] = cscale(m3[e], 2.0);
        __syncthreads();
        block_matmul(d, Vi, X, t1);
        block_matmul(d, t1, Vi, M3);                      // M3'
        block_matmul(d, M2, M2, t1);
        for (int e = tid; e < dd; e += nt) X[e] = csub(cscale(M3[e], 0.5), cscale(t1[e], 0.25));
        __syncthreads();
        st |= block_heig(d, X, A, U, ev, ord, rot, red);
        const bool pos2 = ev[0] > 0;
        for (int e = tid; e < dd; e += nt) {
            const int i = e % d, j = e / d;
            double2 h = cscale(M2[e], 0.5);
            if (pos2)
                for (int l = 0; l < d; l++)
                    h = cadd(h, cscale(cmul(DG_AT(U, d, i, l), cconj(DG_AT(U, d, j, l))), sqrt(ev[l])));
            p.H[e] = h;
            p.H2[e] = csub(M2[e], h);
            p.V[e] = V[e];
        }
    } else {
        for (int e = tid; e < dd; e += nt) {
            V[e] = cmk(0, 0);
            p.V[e] = p.H[e] = p.H2[e] = cmk(0, 0);
        }
    }
    __syncthreads();
    st |= block_heig(d, p.H, A, U, ev, ord, rot, red);
    for (int e = tid; e < dd; e += nt) {
        p.UH[e] = U[e];
        M3[e] = U[e];
    }
    for (int l = tid; l < d; l += nt) p.eH[l] = ev[l];
    __syncthreads();
    st |= block_heig(d, p.H2, A, U, ev, ord, rot, red);
    for (int e = tid; e < dd; e += nt) {
        p.UH2[e] = U[e];
        const int i = e % d, j = e / d;
        double2 w1 = cmk(0, 0), w2 = cmk(0, 0);
        for (int l = 0; l < d; l++) {
            w1 = cfma(cconj(DG_AT(M3, d, l, i)), DG_AT(V, d, l, j), w1);
            w2 = cfma(cconj(DG_AT(U, d, l, i)), DG_AT(V, d, l, j), w2);
        }
        p.W1[e] = w1;
        p.W2[e] = w2;
    }
    for (int l = tid; l < d; l += nt) p.eH2[l] = ev[l];
    if (st && tid == 0) dg_flag(status, DG_NONCONV);
}

// g(tau) of the two tail poles: G[t * 2d + l] = -1/(exp(e_l tau) + exp(e_l (tau - beta))), e = (eH, eH2)
__global__ void k_tail_g(int d, int ntau, double beta, const double2 *T, double *G) {
    long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= (long long)(ntau + 1) * 2 * d) return;
    const int t = (int)(x / (2 * d)), l = (int)(x % (2 * d));
    TailPtrs p = tail_ptrs(const_cast<double2 *>(T), d);
    const double e = l < d ? p.eH[l] : p.eH2[l - d];
    const double tau = t * beta / ntau;
    G[x] = -1.0 / (exp(e * tau) + exp(e * (tau - beta)));
}

// one thread per (tau, element): (S + S^H)/beta + V^H G0_H V/2 + V^H G0_H2 V/2, symmetrised
__global__ void k_ft_finish_el(int d, int ntau, double beta, const double2 *T, const double *G, const double2 *S,
                               double2 *out) {
    const int dd = d * d;
    long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= (long long)(ntau + 1) * dd) return;
    const int t = (int)(x / dd), e = (int)(x % dd), a = e % d, b = e / d;
    TailPtrs p = tail_ptrs(const_cast<double2 *>(T), d);
    const double2 *Sj = S + (size_t)t * dd;
    const double *g = G + (size_t)t * 2 * d;
    double2 tab = cmk(0, 0), tba = cmk(0, 0);
    for (int l = 0; l < d; l++) {
        const double2 w1a = DG_AT(p.W1, d, l, a), w1b = DG_AT(p.W1, d, l, b);
        const double2 w2a = DG_AT(p.W2, d, l, a), w2b = DG_AT(p.W2, d, l, b);
        tab = cadd(tab, cadd(cscale(cmul(cconj(w1a), w1b), g[l]), cscale(cmul(cconj(w2a), w2b), g[d + l])));
        tba = cadd(tba, cadd(cscale(cmul(cconj(w1b), w1a), g[l]), cscale(cmul(cconj(w2b), w2a), g[d + l])));
    }
    const double2 sab = cadd(DG_AT(Sj, d, a, b), cconj(DG_AT(Sj, d, b, a)));
    const double2 sba = cadd(DG_AT(Sj, d, b, a), cconj(DG_AT(Sj, d, a, b)));
    const double2 Aab = cadd(cscale(sab, 1.0 / beta), cscale(tab, 0.5));
    const double2 Aba = cadd(cscale(sba, 1.0 / beta), cscale(tba, 0.5));
    out[x] = cscale(cadd(Aab, cconj(Aba)), 0.5);
}

// Definiteness of nmat Hermitian d x d matrices, one thread each, lower triangles interleaved in shared memory.
// mode 0: sign * lower(M_t) - shift I; mode 1: sign * (W_t - W_t^H)/(2i).  flag[t] = +1 if positive definite
// (strict) or semidefinite (!strict), else -1; if status != nullptr, `code` is flagged when the answer is
// `when` (0: not definite, 1: definite).
__global__ void k_posdef(int d, int nmat, const double2 *M, int mode, double sign, double shift, int strict,
                         double *flag, int *status, int code, int when) {
    extern __shared__ double2 tri[];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmat) return;
    const int stride = blockDim.x;
    double2 *my = tri + threadIdx.x;
    const double2 *Mt = M + (size_t)t * d * d;
    for (int i = 0; i < d; i++)
        for (int j = 0; j <= i; j++) {
            double2 v;
            if (mode == 0) {
                v = DG_AT(Mt, d, i, j);
            } else {
                const double2 x = csub(DG_AT(Mt, d, i, j), cconj(DG_AT(Mt, d, j, i)));
                v = cmk(x.y / 2, -x.x / 2);
            }
            v = cscale(v, sign);
            if (i == j) v = cmk(v.x - shift, 0.0);
            my[(size_t)((i * (i + 1)) / 2 + j) * stride] = v;
        }
    const bool ok = posdef_tri(d, my, stride, strict != 0);
    if (flag) flag[t] = ok ? 1.0 : -1.0;
    if (status && (int)ok == when) dg_flag(status, code);
}


// one thread per (frequency, element): Dw_i = F_i - V^H [(iw - H)^-1 + (iw - H2)^-1] V / 2 (:55-60), the
// inverses through the eigen-decompositions of H and H2: V^H (iw - H)^-1 V = W1^H diag(1/(iw - eH)) W1
__global__ void k_ft_subtract_el(int d, int nfreq, double beta, const double2 *F, const double2 *T, double2 *Dw) {
    const int dd = d * d;
    long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= (long long)nfreq * dd) return;
    const int i = (int)(x / dd), e = (int)(x % dd), a = e % d, b = e / d;
    TailPtrs p = tail_ptrs(const_cast<double2 *>(T), d);
    const double w = (DG_PI / beta) + i * ((2 * DG_PI) / beta);
    double2 tl = cmk(0, 0);
    for (int l = 0; l < d; l++) {
        tl = cadd(tl, cmul(cmul(cconj(DG_AT(p.W1, d, l, a)), DG_AT(p.W1, d, l, b)), crcp(cmk(-p.eH[l], w))));
        tl = cadd(tl, cmul(cmul(cconj(DG_AT(p.W2, d, l, a)), DG_AT(p.W2, d, l, b)), crcp(cmk(-p.eH2[l], w))));
    }
    Dw[x] = csub(F[x], cscale(tl, 0.5));
}

// exact phase table: ph[q] = exp(-i pi q / ntau), q in [0, 2 ntau)
__global__ void k_phase_table(int ntau, double2 *ph) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 2 * ntau) return;
    double s, c;
    sincospi(-(double)q / ntau, &s, &c);
    ph[q] = cmk(c, s);
}

// S(tau_j) = sum_i Dw_i exp(-i w_i tau_j), w_i tau_j = pi (2i+1) j / ntau.  Block: TJ tau points x all
// elements, frequencies staged through shared memory.
constexpr int FT_TJ = 64;
constexpr int FT_IB = 32;
__global__ void __launch_bounds__(FT_TJ) k_ft_sum(int dd, int nfreq, int ntau, const double2 *__restrict__ Dw,
                                                   const double2 *__restrict__ ph, double2 *__restrict__ S) {
    extern __shared__ double2 sd[];  // [FT_IB][16]
    const int j = blockIdx.x * FT_TJ + threadIdx.x;
    const int e0 = blockIdx.y * 16, ne = min(16, dd - e0);
    double2 acc[16];
#pragma unroll
    for (int e = 0; e < 16; e++) acc[e] = cmk(0, 0);
    const long long twoN = 2LL * ntau;
    const int jj = min(j, ntau);
    const double2 r = ph[(2LL * jj) % twoN];  // exp(-i 2 pi j / ntau): frequency step
    for (int i0 = 0; i0 < nfreq; i0 += FT_IB) {
        __syncthreads();
        for (int t = threadIdx.x; t < FT_IB * ne; t += blockDim.x) {
            int ii = t / ne, e = t % ne;
            sd[ii * 16 + e] = (i0 + ii < nfreq) ? Dw[(size_t)(i0 + ii) * dd + e0 + e] : cmk(0, 0);
        }
        __syncthreads();
        if (j <= ntau) {
            const int imax = min(FT_IB, nfreq - i0);
            double2 p = ph[((long long)(2 * i0 + 1) * jj) % twoN];  // exact at the chunk start
            for (int ii = 0; ii < imax; ii++) {
#pragma unroll
                for (int e = 0; e < 16; e++)
                    if (e < ne) acc[e] = cfma(sd[ii * 16 + e], p, acc[e]);
                p = cmul(p, r);
            }
        }
    }
    if (j <= ntau)
        for (int e = 0; e < ne; e++) S[(size_t)j * dd + e0 + e] = acc[e];
}

// ---------------------------------------------------------------------------------------------------
// FFT path (N = 2^logn <= 8192): one CTA per matrix element, the whole sequence in shared memory
// ---------------------------------------------------------------------------------------------------
constexpr int FFT_MAX_LOG = 13;
constexpr int FFT_THREADS = 1024;

// in-place radix-2 decimation-in-time FFT (forward, omega = e^{-2 pi i / N}) of x, loaded in bit-reversed
// order; twiddles e^{-2 pi i k / len} = ph[2 k N / len] from the exact table ph[q] = e^{-i pi q / N}
__device__ void smem_fft(double2 *x, int logn, const double2 *__restrict__ ph) {
    const int N = 1 << logn;
    for (int ls = 1; ls <= logn; ls++) {
        const int half = 1 << (ls - 1), tstep = 2 * (N >> ls);
        for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
            const int k = b & (half - 1), i0 = ((b >> (ls - 1)) << ls) + k, i1 = i0 + half;
            const double2 t = cmul(ph[k * tstep], x[i1]);
            const double2 u = x[i0];
            x[i0] = cadd(u, t);
            x[i1] = csub(u, t);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int bitrev(int i, int logn) { return (int)(__brev((unsigned)i) >> (32 - logn)); }

// S_j = e^{-i pi j/N} X_{j mod N}, X = DFT_N of the Dw column folded modulo N; j = 0..N
__global__ void __launch_bounds__(FFT_THREADS) k_fft_w2tau(int dd, int nfreq, int logn, const double2 *__restrict__ Dw,
                                                           const double2 *__restrict__ ph, double2 *__restrict__ S) {
    extern __shared__ double2 x[];
    const int e = blockIdx.x, N = 1 << logn;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double2 v = cmk(0, 0);
        for (int i2 = i; i2 < nfreq; i2 += N) v = cadd(v, Dw[(size_t)i2 * dd + e]);
        x[bitrev(i, logn)] = v;
    }
    __syncthreads();
    smem_fft(x, logn, ph);
    for (int j = threadIdx.x; j <= N; j += blockDim.x) S[(size_t)j * dd + e] = cmul(ph[j], x[j & (N - 1)]);
}

// FT_t_to_w by hat functions: W_n = dt K (Y_n - F_0) + dt (F_0 E - F_N conj E)
__global__ void __launch_bounds__(FFT_THREADS) k_fft_tau2w(int dd, int nfreq, int logn, double beta,
                                                           const double2 *__restrict__ Ft,
                                                           const double2 *__restrict__ ph, double2 *__restrict__ W) {
    extern __shared__ double2 x[];
    const int e = blockIdx.x, N = 1 << logn;
    // conj(F_s e^{i pi s/N}) = conj(F_s) ph[s]: a forward FFT of it, conjugated, gives Y
    for (int s = threadIdx.x; s < N; s += blockDim.x) x[bitrev(s, logn)] = cmul(cconj(Ft[(size_t)s * dd + e]), ph[s]);
    __syncthreads();
    smem_fft(x, logn, ph);
    const double dt = beta / N;
    const double2 f0 = Ft[e], fN = Ft[(size_t)N * dd + e];
    for (int n = threadIdx.x; n < nfreq; n += blockDim.x) {
        const double2 Y = cconj(x[n & (N - 1)]);
        const double q = (2.0 * n + 1.0) / N;  // t_n / pi
        const double t = DG_PI * q;
        const double sh = sinpi(0.5 * q);
        const double K = (sh / (0.5 * t)) * (sh / (0.5 * t));
        double eim;  // (t - sin t) / t^2
        if (t < 1.0) {
            // sum_{k>=1} (-1)^{k+1} t^{2k-1} / (2k+1)!, nine terms (truncation < 1e-17 relative for t < 1)
            const double t2 = t * t;
            double term = t / 6.0, acc = 0.0;
            for (int k = 1; k <= 9; k++) {
                acc += term;
                term *= -t2 / ((2.0 * k + 2.0) * (2.0 * k + 3.0));
            }
            eim = acc;
        } else {
            eim = (t - sinpi(q)) / (t * t);
        }
        const double2 E = cmk(0.5 * K, eim);
        double2 w = cscale(csub(Y, f0), dt * K);
        w = cadd(w, cscale(csub(cmul(f0, E), cmul(fN, cconj(E))), dt));
        W[(size_t)n * dd + e] = w;
    }
}

__host__ bool fft_ok(dmftgpu_ctx *ctx, int ntau) {
    if (ctx->ft_direct || ntau < 2 || (ntau & (ntau - 1))) return false;
    return ntau <= (1 << FFT_MAX_LOG);
}
__host__ int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

// single thread: the sequential positivity fix-up (src/FourierTransform.cpp:145-175,
// src/SCGF2_fullLoop.cpp:657-688); eigenvalues of untouched points come precomputed in mineig
// One block.  Only points whose minimum eigenvalue is >= 0 are ever touched, and handling point t reads only
// M[t-1] (already final) and the untouched M[t1 > t], so the block first lists those points in order (a
// parallel compaction) and one thread then runs the reference's sequential scan over the list alone.
constexpr int FIX_THREADS = 1024;
__global__ void __launch_bounds__(FIX_THREADS) k_fixup_scan(int d, int ntau, double beta, double2 *M,
                                                            const double *mineig, double2 *work, int *iwork,
                                                            int *list, int *nfix) {
    __shared__ int cnt[FIX_THREADS];
    const int n1 = ntau + 1, per = (n1 + FIX_THREADS - 1) / FIX_THREADS;
    const int t0 = threadIdx.x * per, t1e = min(n1, t0 + per);
    int c = 0;
    for (int t = t0; t < t1e; t++) c += (mineig[t] >= 0);
    cnt[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int i = 0; i < FIX_THREADS; i++) {
            const int v = cnt[i];
            cnt[i] = acc;
            acc += v;
        }
        *nfix = acc;
    }
    __syncthreads();
    int o = cnt[threadIdx.x];
    for (int t = t0; t < t1e; t++)
        if (mineig[t] >= 0) list[o++] = t;
    __syncthreads();
    if (threadIdx.x != 0) return;
    const size_t dd = (size_t)d * d;
    double2 *A = work;
    double *ev = (double *)(work + 2 * dd);
    const int nl = *nfix;
    for (int li = 0; li < nl; li++) {
        const int t = list[li];
        const double tau = t * beta / ntau;
        double m11 = mineig[t];
        double2 *Mt = M + (size_t)t * dd;
        if (t != 0 && t != ntau) {
            for (int t1 = t + 1; t1 < ntau + 1; t1++) {
                const double tau1 = t1 * beta / ntau, tprev = (t - 1) * beta / ntau;
                const double2 *M1 = M + (size_t)t1 * dd, *M0 = M + (size_t)(t - 1) * dd;
                for (size_t q = 0; q < dd; q++) {
                    double2 v = csub(M1[q], M0[q]);
                    v = cmk(v.x / (tau1 - tprev) * (tau - tprev) + M0[q].x, v.y / (tau1 - tprev) * (tau - tprev) + M0[q].y);
                    Mt[q] = v;
                }
                thread_heig(d, Mt, A, nullptr, ev, iwork);
                m11 = ev[0];
                if (m11 < 0) break;
            }
        }
        if (m11 >= 0)
            for (int b = 0; b < d; b++)
                for (int a = 0; a < d; a++) DG_AT(Mt, d, a, b) = cmk(a == b ? -1e-10 : 0.0, 0.0);
    }
}

// ---------------------------------------------------------------------------------------------------
// FT_t_to_w (src/FourierTransform.cpp:521-561): one thread per (frequency, element)
// ---------------------------------------------------------------------------------------------------
__global__ void k_tau2w(int dd, int nfreq, int ntau, double beta, const double2 *__restrict__ Ft,
                        const double2 *__restrict__ ph, double2 *__restrict__ W) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nfreq * dd) return;
    const int n = (int)(t / dd), e = (int)(t % dd);
    const double wn = (2 * n + 1) * DG_PI / beta, dt = beta / ntau;
    const int twoN = 2 * ntau;
    const double2 iwn = cmk(0.0, wn);
    const double2 inv_iw = crcp(iwn);
    const double inv_w2 = 1.0 / (wn * wn);
    double2 acc = cmk(0, 0);
    double2 e0 = cmk(1.0, 0.0);  // exp(i w tau_0), tau_0 = 0
    const int step = (int)((2LL * n + 1) % twoN);
    int q = 0;
    for (int s = 0; s < ntau; s++) {
        const double tau0 = s * dt, tau1 = (s + 1) * dt;
        q += step;
        if (q >= twoN) q -= twoN;
        const double2 e1 = cconj(ph[q]);  // exp(+i pi (2n+1)(s+1)/ntau)
        const double2 pI = csub(e1, e0);
        const double2 pI2 = csub(cscale(e1, tau1), cscale(e0, tau0));
        const double2 ca = cadd(cscale(pI, inv_w2), cmul(pI2, inv_iw));
        const double2 cb = cmul(pI, inv_iw);
        const double2 f0 = Ft[(size_t)s * dd + e], f1 = Ft[(size_t)(s + 1) * dd + e];
        const double2 at = cscale(csub(f1, f0), 1.0 / (tau1 - tau0));
        const double2 bt = cadd(cscale(at, -tau0), f0);
        acc = cfma(at, ca, acc);
        acc = cfma(bt, cb, acc);
        e0 = e1;
    }
    W[t] = acc;
}

// ---------------------------------------------------------------------------------------------------
// getStimp (src/SCGF2_fullLoop.cpp:603-653): Sigma_ij(tau) = sum over U entries x1 = (i,q,m,k), x2 = (l,n,p,j)
// of U1 U2 (-G_pq(beta - tau)) (G_kn G_ml - G_kl G_mn).  One block per S2_TB tau points, one thread per output
// (i, j) for all of them; the U list is pre-sorted on the host by its first index (x1 role) and by its last
// index (x2 role).  Per (x1, x2) pair the thread forms the 2x2 minor G_kn G_ml - G_kl G_mn once per tau and
// accumulates U2 G'_pq times it; U1 multiplies the inner sum.
// ---------------------------------------------------------------------------------------------------
constexpr int S2_TB = 4;
__global__ void k_sigma2(int d, int ntau, const int *__restrict__ byI, const int *__restrict__ byIoff,
                         const int *__restrict__ byJ, const int *__restrict__ byJoff, const int *__restrict__ uidx,
                         const double2 *__restrict__ ut, const double2 *__restrict__ G, double2 *__restrict__ S,
                         int *status) {
    extern __shared__ double2 sg[];  // per tau point b: G(tau) [dd], G(beta - tau) [dd]
    const int t0 = blockIdx.x * S2_TB;
    const int dd = d * d;
    const int nb = min(S2_TB, ntau + 1 - t0);
    for (int x = threadIdx.x; x < nb * dd; x += blockDim.x) {
        const int b = x / dd, q = x % dd;
        sg[(size_t)b * 2 * dd + q] = G[(size_t)(t0 + b) * dd + q];
        sg[(size_t)b * 2 * dd + dd + q] = G[(size_t)(ntau - t0 - b) * dd + q];
    }
    __syncthreads();
    for (int o = threadIdx.x; o < dd; o += blockDim.x) {
        const int i = o % d, j = o / d;
        double2 acc[S2_TB];
#pragma unroll
        for (int b = 0; b < S2_TB; b++) acc[b] = cmk(0, 0);
        for (int a1 = byIoff[i]; a1 < byIoff[i + 1]; a1++) {
            const int x1 = byI[a1];
            const int qq = uidx[4 * x1 + 1], m = uidx[4 * x1 + 2], k = uidx[4 * x1 + 3];
            double2 in[S2_TB];
#pragma unroll
            for (int b = 0; b < S2_TB; b++) in[b] = cmk(0, 0);
            for (int a2 = byJoff[j]; a2 < byJoff[j + 1]; a2++) {
                const int x2 = byJ[a2];
                const int l = uidx[4 * x2], n = uidx[4 * x2 + 1], p = uidx[4 * x2 + 2];
                const double2 u2 = ut[x2];
                const int ikn = k + n * d, iml = m + l * d, ikl = k + l * d, imn = m + n * d, ipq = p + qq * d;
#pragma unroll
                for (int b = 0; b < S2_TB; b++) {
                    const double2 *Gt = sg + (size_t)b * 2 * dd, *Gm = Gt + dd;
                    // minor = G_kn G_ml - G_kl G_mn
                    double2 mn = cmul(Gt[ikn], Gt[iml]);
                    const double2 g1 = Gt[ikl], g2 = Gt[imn];
                    mn.x = fma(-g1.x, g2.x, fma(g1.y, g2.y, mn.x));
                    mn.y = fma(-g1.x, g2.y, fma(-g1.y, g2.x, mn.y));
                    // in -= U2 G'_pq minor
                    in[b] = cfms(u2, cmul(Gm[ipq], mn), in[b]);
                }
            }
            const double2 u1 = ut[x1];
#pragma unroll
            for (int b = 0; b < S2_TB; b++) acc[b] = cfma(u1, in[b], acc[b]);
        }
        for (int b = 0; b < nb; b++) S[(size_t)(t0 + b) * dd + o] = acc[b];
    }
    __syncthreads();
    // Hermiticity asserts of the reference (:641-651): ||(G - G^H)/2i|| > 1e-10, ||(S - S^H)/2i|| > 1e-5
    if (threadIdx.x < nb) {
        const int b = threadIdx.x;
        const double2 *Gt = sg + (size_t)b * 2 * dd;
        const double2 *St = S + (size_t)(t0 + b) * dd;
        double ng = 0, ns = 0;
        for (int c = 0; c < d; c++)
            for (int a = 0; a < d; a++) {
                double2 vg = csub(DG_AT(Gt, d, a, c), cconj(DG_AT(Gt, d, c, a)));
                double2 vs = csub(DG_AT(St, d, a, c), cconj(DG_AT(St, d, c, a)));
                ng += cabs2(vg) / 4;
                ns += cabs2(vs) / 4;
            }
        if (sqrt(ng) > 1e-10 || sqrt(ns) > 1e-5) dg_flag(status, DG_HERMIT);
    }
}

// getStimp in double-float (df.cuh) on the FP32 pipe: the same sums as k_sigma2 with every complex product
// and sum formed as an unevaluated pair of floats (~2^-47 relative per operation); selected by
// DMFTGPU_MIXED.  G enters from FP64 exactly split into hi + lo, S leaves as hi + lo in FP64.
__global__ void __launch_bounds__(128) k_sigma2_df(int d, int ntau, int nu, const int *__restrict__ byI,
                                                   const int *__restrict__ byIoff, const int *__restrict__ byJ,
                                                   const int *__restrict__ byJoff, const int *__restrict__ uidx,
                                                   const double2 *__restrict__ ut, const double2 *__restrict__ G,
                                                   double2 *__restrict__ S, int *status) {
    extern __shared__ cdf sgf[];  // per tau point b: G(tau) [dd], G(beta - tau) [dd]; then the U values [nu]
    typedef OpsF O;
    const int t0 = blockIdx.x * S2_TB;
    const int dd = d * d;
    const int nb = min(S2_TB, ntau + 1 - t0);
    for (int x = threadIdx.x; x < nb * dd; x += blockDim.x) {
        const int b = x / dd, q = x % dd;
        sgf[(size_t)b * 2 * dd + q] = O::from(G[(size_t)(t0 + b) * dd + q]);
        sgf[(size_t)b * 2 * dd + dd + q] = O::from(G[(size_t)(ntau - t0 - b) * dd + q]);
    }
    for (int x = nb * dd + threadIdx.x; x < S2_TB * dd; x += blockDim.x) {  // unused tau slots of the last block
        const int b = x / dd, q = x % dd;
        sgf[(size_t)b * 2 * dd + q] = O::zero();
        sgf[(size_t)b * 2 * dd + dd + q] = O::zero();
    }
    cdf *su = sgf + (size_t)S2_TB * 2 * dd;  // U values split once per block, not per (x1, x2) pair
    for (int x = threadIdx.x; x < nu; x += blockDim.x) su[x] = O::from(ut[x]);
    __syncthreads();
    for (int o = threadIdx.x; o < dd; o += blockDim.x) {
        const int i = o % d, j = o / d;
        cdf acc[S2_TB];
#pragma unroll
        for (int b = 0; b < S2_TB; b++) acc[b] = O::zero();
        for (int a1 = byIoff[i]; a1 < byIoff[i + 1]; a1++) {
            const int x1 = byI[a1];
            const int qq = uidx[4 * x1 + 1], m = uidx[4 * x1 + 2], k = uidx[4 * x1 + 3];
            cdf in[S2_TB];
#pragma unroll
            for (int b = 0; b < S2_TB; b++) in[b] = O::zero();
            for (int a2 = byJoff[j]; a2 < byJoff[j + 1]; a2++) {
                const int x2 = byJ[a2];
                const int l = uidx[4 * x2], n = uidx[4 * x2 + 1], p = uidx[4 * x2 + 2];
                const cdf u2 = su[x2];
                const int ikn = k + n * d, iml = m + l * d, ikl = k + l * d, imn = m + n * d, ipq = p + qq * d;
#pragma unroll
                for (int b = 0; b < S2_TB; b++) {
                    const cdf *Gt = sgf + (size_t)b * 2 * dd, *Gm = Gt + dd;
                    const cdf mn = O::fms(Gt[ikl], Gt[imn], O::mul(Gt[ikn], Gt[iml]));  // G_kn G_ml - G_kl G_mn
                    in[b] = O::fms(u2, O::mul(Gm[ipq], mn), in[b]);
                }
            }
            const cdf u1 = su[x1];
#pragma unroll
            for (int b = 0; b < S2_TB; b++) acc[b] = O::fma(u1, in[b], acc[b]);
        }
        for (int b = 0; b < nb; b++) S[(size_t)(t0 + b) * dd + o] = O::to(acc[b]);
    }
    __syncthreads();
    if (threadIdx.x < nb) {
        const int b = threadIdx.x;
        const double2 *Gt = G + (size_t)(t0 + b) * dd;
        const double2 *St = S + (size_t)(t0 + b) * dd;
        double ng = 0, ns = 0;
        for (int c = 0; c < d; c++)
            for (int a = 0; a < d; a++) {
                double2 vg = csub(DG_AT(Gt, d, a, c), cconj(DG_AT(Gt, d, c, a)));
                double2 vs = csub(DG_AT(St, d, a, c), cconj(DG_AT(St, d, c, a)));
                ng += cabs2(vg) / 4;
                ns += cabs2(vs) / 4;
            }
        if (sqrt(ng) > 1e-10 || sqrt(ns) > 1e-5) dg_flag(status, DG_HERMIT);
    }
}

// getFockOperator (:583-597), single thread
__global__ void k_fock(int d, int nu, const int *uidx, const double2 *ut, const double2 *occ, double2 *fock) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int q = 0; q < d * d; q++) fock[q] = cmk(0, 0);
    for (int x = 0; x < nu; x++) {
        const int a = uidx[4 * x], b = uidx[4 * x + 1], c = uidx[4 * x + 2], dd_ = uidx[4 * x + 3];
        DG_AT(fock, d, b, dd_) = cadd(DG_AT(fock, d, b, dd_), cmul(ut[x], DG_AT(occ, d, c, a)));
        DG_AT(fock, d, b, c) = csub(DG_AT(fock, d, b, c), cmul(ut[x], DG_AT(occ, d, dd_, a)));
    }
}

// getGwimp (:551-570): one thread per frequency
__global__ void k_dyson(int d, int nfreq, double beta, double mu, const double2 *himp, const double2 *delta,
                        const double2 *fock, const double2 *s2, double2 *gw, int *iwork, int *status) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nfreq) return;
    const size_t dd = (size_t)d * d;
    const double wn = (DG_PI * (2. * n + 1.)) / beta;
    double2 *G = gw + (size_t)n * dd;
    for (int b = 0; b < d; b++)
        for (int a = 0; a < d; a++) {
            double2 v = (a == b) ? cmk(mu, wn) : cmk(0, 0);
            v = csub(v, DG_AT(himp, d, a, b));
            v = csub(v, delta[(size_t)n * dd + a + b * d]);
            v = csub(v, DG_AT(fock, d, a, b));
            v = csub(v, s2[(size_t)n * dd + a + b * d]);
            DG_AT(G, d, a, b) = v;
        }
    if (thread_gj_inverse(d, G, iwork + (size_t)n * d)) dg_flag(status, DG_SINGULAR);
}

// estimate_asymto (:736-787), single thread; F holds nfreq+3 matrices
__global__ void k_estimate_asymto(int d, int Nf, double beta, double2 *F, int order) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const size_t dd = (size_t)d * d;
    auto wn = [&](int i) { return (2 * (Nf - 3 + i) + 1) * DG_PI / beta; };
    double w0, w1, w2;
    int p = (order == 1) ? 2 : (order == 2 ? 4 : 6);
    w0 = 1. / pow(wn(0), p);
    w1 = 1. / pow(wn(1), p);
    w2 = 1. / pow(wn(2), p);
    const double wsum = w0 + w1 + w2;
    double2 *dst = F + (size_t)(Nf + order - 1) * dd;
    for (int b = 0; b < d; b++)
        for (int a = 0; a < d; a++) {
            double2 acc = cmk(0, 0);
            for (int w = 0; w < 3; w++) {
                const double2 *T = F + (size_t)(Nf - 3 + w) * dd;
                double2 tab = DG_AT(T, d, a, b), tba = DG_AT(T, d, b, a);
                double2 v;
                if (order == 1) {
                    v = cscale(csub(cconj(tba), tab), 0.5);   // (t^H - t)/2
                    v = cmul(v, crcp(cmk(0, wn(w))));          // / (i w)
                } else if (order == 2) {
                    v = cscale(cadd(tab, cconj(tba)), 0.5);
                    v = cscale(v, -1.0 / pow(wn(w), 2));
                } else {
                    const double2 *F0 = F + (size_t)Nf * dd;
                    const double2 ir = crcp(cmk(0, wn(w)));
                    double2 xab = csub(tab, cmul(DG_AT(F0, d, a, b), ir));
                    double2 xba = csub(tba, cmul(DG_AT(F0, d, b, a), ir));
                    v = cscale(csub(cconj(xba), xab), 0.5);
                    v = cscale(cmul(cmk(0, 1), v), 1.0 / pow(wn(w), 3));
                }
                acc = cadd(acc, v);
            }
            DG_AT(dst, d, a, b) = cscale(acc, 1.0 / wsum);
        }
}

// Kajueter-Kotliar interpolation of the IPT self-energy on (0,0), (1,1) (:1033-1046)
__global__ void k_ipt_kk(int nfreq, double a0, double a1, double b0, double b1, double c0, double c1, double2 *s2) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nfreq) return;
    double2 *S = s2 + (size_t)n * 4;
    double2 x0 = S[0], x1 = S[3];
    S[0] = cdiv(cscale(x0, a0), csub(cmk(c0, 0), cscale(x0, b0)));
    S[3] = cdiv(cscale(x1, a1), csub(cmk(c1, 0), cscale(x1, b1)));
}

}  // namespace

// ===================================================================================================
// device-level building blocks (all pointers device; enqueue only)
// ===================================================================================================
int dg_phase_table(dmftgpu_ctx *ctx, int ntau, double2 **ph) {
    *ph = (double2 *)dg_buf(ctx, "imp.phase", 2 * (size_t)ntau * sizeof(double2));
    if (!*ph) return DMFTGPU_NOMEM;
    k_phase_table<<<dg_ceil_div(2 * ntau, 256), 256, 0, ctx->stream>>>(ntau, *ph);
    DG_LAUNCH(ctx, "k_phase_table");
    return DMFTGPU_OK;
}

int dg_tail_setup_dev(dmftgpu_ctx *ctx, int d, const double2 *mom, double2 *T) {
    const size_t sm = tail_smem_bytes(d);
    DG_CUDA(cudaFuncSetAttribute(k_tail_setup_blk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_tail_setup_blk<<<1, TAIL_THREADS, sm, ctx->stream>>>(d, mom, T, ctx->d_status);
    DG_LAUNCH(ctx, "k_tail_setup_blk");
    return DMFTGPU_OK;
}

// flags (and/or status) from the definiteness of nmat d x d matrices; the fix-up reads flag >= 0 as
// "minimum eigenvalue >= 0"
int dg_posdef_dev(dmftgpu_ctx *ctx, int d, int nmat, const double2 *M, int mode, double sign, double shift,
                  bool strict, double *flag, int code, int when) {
    const int nt = posdef_threads(d);
    const size_t sm = (size_t)nt * d * (d + 1) / 2 * sizeof(double2);
    DG_CUDA(cudaFuncSetAttribute(k_posdef, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_posdef<<<dg_ceil_div(nmat, nt), nt, sm, ctx->stream>>>(d, nmat, M, mode, sign, shift, strict ? 1 : 0, flag,
                                                             code ? ctx->d_status : nullptr, code, when);
    DG_LAUNCH(ctx, "k_posdef");
    return DMFTGPU_OK;
}

int dg_fixup_dev(dmftgpu_ctx *ctx, int d, int ntau, double beta, double2 *M, const double *mineig) {
    double2 *w = (double2 *)dg_buf(ctx, "imp.fixwork", 4 * (size_t)d * d * sizeof(double2) + 64);
    int *iw = (int *)dg_buf(ctx, "imp.fixiwork", (size_t)(d + 1) * sizeof(int));
    int *nfix = (int *)dg_buf(ctx, "imp.nfix", sizeof(int));
    int *list = (int *)dg_buf(ctx, "imp.fixlist", (size_t)(ntau + 1) * sizeof(int));
    if (!w || !iw || !nfix || !list) return DMFTGPU_NOMEM;
    k_fixup_scan<<<1, FIX_THREADS, 0, ctx->stream>>>(d, ntau, beta, M, mineig, w, iw, list, nfix);
    DG_LAUNCH(ctx, "k_fixup_scan");
    return DMFTGPU_OK;
}

// tail data and Dw = F - tail for moments `mom`: the part of FourierTransform shared by every tau
int dg_tail_prepare_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, const double2 *fw, const double2 *mom,
                        double2 *T, double2 *Dw) {
    const size_t dd = (size_t)d * d;
    DG_TRY(dg_tail_setup_dev(ctx, d, mom, T));
    k_ft_subtract_el<<<dg_ceil_div((long long)nfreq * dd, 256), 256, 0, ctx->stream>>>(d, nfreq, beta, fw, T, Dw);
    DG_LAUNCH(ctx, "k_ft_subtract_el");
    return DMFTGPU_OK;
}

// the tau grid from prepared tail data: Fourier sums, tail terms, symmetrisation, positivity fix-up
int dg_w2tau_tail_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *T, const double2 *Dw,
                      double2 *ft) {
    const size_t dd = (size_t)d * d;
    cudaStream_t s = ctx->stream;
    double *gtail = (double *)dg_buf(ctx, "imp.gtail", (size_t)(ntau + 1) * 2 * d * sizeof(double));
    double2 *S = (double2 *)dg_buf(ctx, "imp.Ssum", (size_t)(ntau + 1) * dd * sizeof(double2));
    double *mineig = (double *)dg_buf(ctx, "imp.mineig", (size_t)(ntau + 1) * sizeof(double));
    if (!gtail || !S || !mineig) return DMFTGPU_NOMEM;
    double2 *ph;
    DG_TRY(dg_phase_table(ctx, ntau, &ph));
    if (fft_ok(ctx, ntau)) {
        const size_t sm = (size_t)ntau * sizeof(double2);
        DG_CUDA(cudaFuncSetAttribute(k_fft_w2tau, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        {
            DgTimer tm(ctx, "k_fft_w2tau");
            k_fft_w2tau<<<(int)dd, FFT_THREADS, sm, s>>>((int)dd, nfreq, ilog2(ntau), Dw, ph, S);
        }
        DG_LAUNCH(ctx, "k_fft_w2tau");
    } else {
        dim3 grid(dg_ceil_div(ntau + 1, FT_TJ), dg_ceil_div((int)dd, 16));
        {
            DgTimer tm(ctx, "k_ft_sum");
            k_ft_sum<<<grid, FT_TJ, FT_IB * 16 * sizeof(double2), s>>>((int)dd, nfreq, ntau, Dw, ph, S);
        }
        DG_LAUNCH(ctx, "k_ft_sum");
    }
    k_tail_g<<<dg_ceil_div((long long)(ntau + 1) * 2 * d, 256), 256, 0, s>>>(d, ntau, beta, T, gtail);
    DG_LAUNCH(ctx, "k_tail_g");
    k_ft_finish_el<<<dg_ceil_div((long long)(ntau + 1) * dd, 256), 256, 0, s>>>(d, ntau, beta, T, gtail, S, ft);
    DG_LAUNCH(ctx, "k_ft_finish_el");
    DG_TRY(dg_posdef_dev(ctx, d, ntau + 1, ft, 0, 1.0, 0.0, false, mineig, 0, 0));
    return dg_fixup_dev(ctx, d, ntau, beta, ft, mineig);
}

int dg_w2tau_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *fw, const double2 *mom,
                 double2 *ft) {
    const size_t dd = (size_t)d * d;
    double2 *T = (double2 *)dg_buf(ctx, "imp.tail", TAIL_SLOTS * dd * sizeof(double2));
    double2 *Dw = (double2 *)dg_buf(ctx, "imp.Dw", (size_t)nfreq * dd * sizeof(double2));
    if (!T || !Dw) return DMFTGPU_NOMEM;
    DG_TRY(dg_tail_prepare_dev(ctx, d, nfreq, beta, fw, mom, T, Dw));
    return dg_w2tau_tail_dev(ctx, d, nfreq, ntau, beta, T, Dw, ft);
}

int dg_fourier_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *fw, int green,
                   const double2 *m1, double2 *ft) {
    const size_t dd = (size_t)d * d;
    double2 *mom = (double2 *)dg_buf(ctx, "imp.mom", 4 * dd * sizeof(double2));
    if (!mom) return DMFTGPU_NOMEM;
    DG_TRY(dg_moments_dev(ctx, d, nfreq, beta, fw, green, mom));
    if (m1) {
        DG_CUDA(cudaMemsetAsync(mom, 0, dd * sizeof(double2), ctx->stream));
        DG_CUDA(cudaMemcpyAsync(mom + dd, m1, dd * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return dg_w2tau_dev(ctx, d, nfreq, ntau, beta, fw, mom, ft);
}

int dg_tau2w_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *ft, double2 *fw,
                 bool check) {
    const size_t dd = (size_t)d * d;
    double2 *ph;
    DG_TRY(dg_phase_table(ctx, ntau, &ph));
    if (fft_ok(ctx, ntau)) {
        const size_t sm = (size_t)ntau * sizeof(double2);
        DG_CUDA(cudaFuncSetAttribute(k_fft_tau2w, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        {
            DgTimer tm(ctx, "k_fft_tau2w");
            k_fft_tau2w<<<(int)dd, FFT_THREADS, sm, ctx->stream>>>((int)dd, nfreq, ilog2(ntau), beta, ft, ph, fw);
        }
        DG_LAUNCH(ctx, "k_fft_tau2w");
    } else {
        {
            DgTimer tm(ctx, "k_tau2w");
            k_tau2w<<<dg_ceil_div((long long)nfreq * dd, 128), 128, 0, ctx->stream>>>((int)dd, nfreq, ntau, beta, ft,
                                                                                      ph, fw);
        }
        DG_LAUNCH(ctx, "k_tau2w");
    }
    if (check) {
        // FT_t_to_w asserts max eig of (W - W^H)/2i <= 0: -(W - W^H)/2i positive semidefinite
        DG_TRY(dg_posdef_dev(ctx, d, nfreq, fw, 1, -1.0, 0.0, false, nullptr, DG_CAUSAL, 0));
    }
    return DMFTGPU_OK;
}

int dg_sigma2_dev(dmftgpu_ctx *ctx, int d, int ntau, double beta, const DgUList &U, const double2 *gt, double2 *st) {
    const size_t dd = (size_t)d * d;
    {
        DgTimer tm(ctx, "k_sigma2");
        const size_t sm = S2_TB * 2 * dd * sizeof(double2);
        if (ctx->imp_mixed) {
            const size_t smf = sm + (size_t)U.nu * sizeof(double2);
            DG_CUDA(cudaFuncSetAttribute(k_sigma2_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smf));
            k_sigma2_df<<<dg_ceil_div(ntau + 1, S2_TB), 128, smf, ctx->stream>>>(
                d, ntau, U.nu, U.byI, U.byIoff, U.byJ, U.byJoff, U.uidx, U.ut, gt, st, ctx->d_status);
        } else {
            const int nt = std::min(1024, (int)((dd + 31) / 32 * 32));
            DG_CUDA(cudaFuncSetAttribute(k_sigma2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            k_sigma2<<<dg_ceil_div(ntau + 1, S2_TB), nt, sm, ctx->stream>>>(d, ntau, U.byI, U.byIoff, U.byJ,
                                                                               U.byJoff, U.uidx, U.ut, gt, st,
                                                                               ctx->d_status);
        }
    }
    DG_LAUNCH(ctx, "k_sigma2");
    double *mineig = (double *)dg_buf(ctx, "imp.s2mineig", (size_t)(ntau + 1) * sizeof(double));
    if (!mineig) return DMFTGPU_NOMEM;
    DG_TRY(dg_posdef_dev(ctx, d, ntau + 1, st, 0, 1.0, 0.0, false, mineig, 0, 0));
    return dg_fixup_dev(ctx, d, ntau, beta, st, mineig);
}

int dg_fock_dev(dmftgpu_ctx *ctx, int d, const DgUList &U, const double2 *occ, double2 *fock) {
    k_fock<<<1, 1, 0, ctx->stream>>>(d, U.nu, U.uidx, U.ut, occ, fock);
    DG_LAUNCH(ctx, "k_fock");
    return DMFTGPU_OK;
}

int dg_dyson_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, double mu, const double2 *himp,
                 const double2 *delta, const double2 *fock, const double2 *s2, double2 *gw, bool check) {
    const size_t dd = (size_t)d * d;
    int *iw = (int *)dg_buf(ctx, "imp.dysiwork", (size_t)nfreq * d * sizeof(int));
    if (!iw) return DMFTGPU_NOMEM;
    k_dyson<<<dg_ceil_div(nfreq, 64), 64, 0, ctx->stream>>>(d, nfreq, beta, mu, himp, delta, fock, s2, gw, iw,
                                                            ctx->d_status);
    DG_LAUNCH(ctx, "k_dyson");
    if (check) {
        // getGwimp asserts max eig of (G - G^H)/2i < 0: -(G - G^H)/2i positive definite
        DG_TRY(dg_posdef_dev(ctx, d, nfreq, gw, 1, -1.0, 0.0, true, nullptr, DG_CAUSAL, 0));
    }
    return DMFTGPU_OK;
}

int dg_estimate_asymto_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, double2 *f, int order) {
    k_estimate_asymto<<<1, 1, 0, ctx->stream>>>(d, nfreq, beta, f, order);
    DG_LAUNCH(ctx, "k_estimate_asymto");
    return DMFTGPU_OK;
}

// getoccMat: n = -G(tau = beta) with the m0 = 0, m1 = I green tail (src/SCGF2_fullLoop.cpp:539-549).
// S(beta) = sum_i Dw_i exp(-i w_i beta) = -sum_i Dw_i (exp(-i pi (2i+1)) = -1); one block: per element, P
// threads sum fixed frequency ranges and the ranges are combined in order; then the tail term per element
constexpr int OCC_THREADS = 1024;
__global__ void __launch_bounds__(OCC_THREADS) k_occ_finish_blk(int d, int nfreq, double beta, const double2 *T,
                                                                const double2 *Dw, double2 *occ) {
    extern __shared__ double2 sw[];  // dd sums, then dd * P partials
    const int dd = d * d, P = max(1, OCC_THREADS / dd), chunk = (nfreq + P - 1) / P;
    double2 *part = sw + dd;
    for (int x = threadIdx.x; x < dd * P; x += blockDim.x) {
        const int e = x % dd, pp = x / dd;
        double2 s = cmk(0, 0);
        const int i1 = min(nfreq, (pp + 1) * chunk);
        for (int i = pp * chunk; i < i1; i++) s = csub(s, Dw[(size_t)i * dd + e]);
        part[x] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < dd; e += blockDim.x) {
        double2 s = cmk(0, 0);
        for (int pp = 0; pp < P; pp++) s = cadd(s, part[pp * dd + e]);
        sw[e] = s;
    }
    __syncthreads();
    TailPtrs p = tail_ptrs(const_cast<double2 *>(T), d);
    for (int e = threadIdx.x; e < dd; e += blockDim.x) {
        const int a = e % d, b = e / d;
        double2 tab = cmk(0, 0), tba = cmk(0, 0);
        for (int l = 0; l < d; l++) {
            const double e1 = p.eH[l], e2 = p.eH2[l];
            const double g1 = -1.0 / (exp(e1 * beta) + exp(e1 * (beta - beta)));
            const double g2 = -1.0 / (exp(e2 * beta) + exp(e2 * (beta - beta)));
            const double2 w1a = DG_AT(p.W1, d, l, a), w1b = DG_AT(p.W1, d, l, b);
            const double2 w2a = DG_AT(p.W2, d, l, a), w2b = DG_AT(p.W2, d, l, b);
            tab = cadd(tab, cadd(cscale(cmul(cconj(w1a), w1b), g1), cscale(cmul(cconj(w2a), w2b), g2)));
            tba = cadd(tba, cadd(cscale(cmul(cconj(w1b), w1a), g1), cscale(cmul(cconj(w2b), w2a), g2)));
        }
        const double2 Aab = cadd(cscale(cadd(sw[a + b * d], cconj(sw[b + a * d])), 1.0 / beta), cscale(tab, 0.5));
        const double2 Aba = cadd(cscale(cadd(sw[b + a * d], cconj(sw[a + b * d])), 1.0 / beta), cscale(tba, 0.5));
        occ[e] = cscale(cadd(Aab, cconj(Aba)), -0.5);
    }
}

__global__ void k_set_identity_slot(int d, double2 *m1) {
    int q = threadIdx.x + blockIdx.x * blockDim.x;
    if (q < d * d) m1[q] = cmk((q % d) == (q / d) ? 1.0 : 0.0, 0.0);
}

// occupation from prepared green-tail data (T, Dw of G)
int dg_occ_tail_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, const double2 *T, const double2 *Dw,
                    double2 *occ) {
    const size_t dd = (size_t)d * d;
    const int P = std::max(1, OCC_THREADS / (int)dd);
    k_occ_finish_blk<<<1, OCC_THREADS, dd * (1 + P) * sizeof(double2), ctx->stream>>>(d, nfreq, beta, T, Dw, occ);
    DG_LAUNCH(ctx, "k_occ_finish_blk");
    return DMFTGPU_OK;
}

// green-tail moments of G (m0 = 0, m1 = I), tail data and Dw: what getoccMat and FourierTransform(G, ., I,
// true) share
int dg_green_tail_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, const double2 *gw, double2 *T, double2 *Dw) {
    const size_t dd = (size_t)d * d;
    double2 *mom = (double2 *)dg_buf(ctx, "occ.mom", 4 * dd * sizeof(double2));
    if (!mom) return DMFTGPU_NOMEM;
    DG_TRY(dg_moments_dev(ctx, d, nfreq, beta, gw, 1, mom));
    k_set_identity_slot<<<dg_ceil_div((int)dd, 64), 64, 0, ctx->stream>>>(d, mom + dd);  // m1 = I (m0 = 0 already)
    DG_LAUNCH(ctx, "k_set_identity_slot");
    return dg_tail_prepare_dev(ctx, d, nfreq, beta, gw, mom, T, Dw);
}

int dg_occ_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, const double2 *gw, double2 *occ) {
    const size_t dd = (size_t)d * d;
    double2 *T = (double2 *)dg_buf(ctx, "occ.tail", TAIL_SLOTS * dd * sizeof(double2));
    double2 *Dw = (double2 *)dg_buf(ctx, "occ.Dw", (size_t)nfreq * dd * sizeof(double2));
    if (!T || !Dw) return DMFTGPU_NOMEM;
    DG_TRY(dg_green_tail_dev(ctx, d, nfreq, beta, gw, T, Dw));
    return dg_occ_tail_dev(ctx, d, nfreq, beta, T, Dw, occ);
}

int dg_ipt_kk_dev(dmftgpu_ctx *ctx, int nfreq, const double *a, const double *b, const double *c, double2 *s2) {
    k_ipt_kk<<<dg_ceil_div(nfreq, 128), 128, 0, ctx->stream>>>(nfreq, a[0], a[1], b[0], b[1], c[0], c[1], s2);
    DG_LAUNCH(ctx, "k_ipt_kk");
    return DMFTGPU_OK;
}

// U list on the device with the two index orders getStimp's output-stationary kernel needs
int dg_ulist(dmftgpu_ctx *ctx, int d, int nu, const int *uidx, const double *ut, DgUList &U) {
    for (int x = 0; x < nu; x++)
        for (int q = 0; q < 4; q++)
            if (uidx[4 * x + q] < 0 || uidx[4 * x + q] >= d) return dg_fail(ctx, DMFTGPU_BADARG, "U list index");
    std::vector<int> byI, byJ, offI(d + 1, 0), offJ(d + 1, 0);
    for (int i = 0; i < d; i++) {
        offI[i] = (int)byI.size();
        for (int x = 0; x < nu; x++)
            if (uidx[4 * x] == i) byI.push_back(x);
    }
    offI[d] = (int)byI.size();
    for (int j = 0; j < d; j++) {
        offJ[j] = (int)byJ.size();
        for (int x = 0; x < nu; x++)
            if (uidx[4 * x + 3] == j) byJ.push_back(x);
    }
    offJ[d] = (int)byJ.size();
    const size_t nb = (size_t)std::max(nu, 1);
    int *dI = (int *)dg_buf(ctx, "u.byI", nb * sizeof(int)), *dJ = (int *)dg_buf(ctx, "u.byJ", nb * sizeof(int));
    int *dOI = (int *)dg_buf(ctx, "u.offI", (d + 1) * sizeof(int)), *dOJ = (int *)dg_buf(ctx, "u.offJ", (d + 1) * sizeof(int));
    int *dU = (int *)dg_buf(ctx, "u.idx", nb * 4 * sizeof(int));
    double2 *dT = (double2 *)dg_buf(ctx, "u.val", nb * sizeof(double2));
    if (!dI || !dJ || !dOI || !dOJ || !dU || !dT) return DMFTGPU_NOMEM;
    cudaStream_t s = ctx->stream;
    if (nu > 0) {
        DG_CUDA(cudaMemcpyAsync(dI, byI.data(), nu * sizeof(int), cudaMemcpyHostToDevice, s));
        DG_CUDA(cudaMemcpyAsync(dJ, byJ.data(), nu * sizeof(int), cudaMemcpyHostToDevice, s));
        DG_CUDA(cudaMemcpyAsync(dU, uidx, (size_t)nu * 4 * sizeof(int), cudaMemcpyHostToDevice, s));
        DG_CUDA(cudaMemcpyAsync(dT, ut, (size_t)nu * sizeof(double2), cudaMemcpyHostToDevice, s));
    }
    DG_CUDA(cudaMemcpyAsync(dOI, offI.data(), (d + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    DG_CUDA(cudaMemcpyAsync(dOJ, offJ.data(), (d + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    DG_CUDA(cudaStreamSynchronize(s));  // host vectors go out of scope
    U.nu = nu;
    U.byI = dI;
    U.byJ = dJ;
    U.byIoff = dOI;
    U.byJoff = dOJ;
    U.uidx = dU;
    U.ut = dT;
    return DMFTGPU_OK;
}

// ===================================================================================================
// C ABI
// ===================================================================================================
extern "C" {

int dmftgpu_hyb_delta(dmftgpu_ctx *ctx, int dim, const int *orb, int nfreq, double beta, int D, const double *sigma,
                      const double *gw, const double *himp, double mu, double *delta, int flags) {
    if (!ctx || dim < 1 || !orb || nfreq < 1 || D < 1 || !sigma || !gw || !himp || !delta || !(beta > 0))
        return DMFTGPU_BADARG;
    for (int i = 0; i < dim; i++)
        if (orb[i] < 0 || orb[i] >= D) return dg_fail(ctx, DMFTGPU_BADARG, "hyb_delta: orbital index");
    cudaSetDevice(ctx->device);
    const size_t DD = (size_t)D * D, dd = (size_t)dim * dim;
    int st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma, nfreq * DD * sizeof(double2), flags, "io.hyb_s", &st);
    if (st) return st;
    const double2 *dG = (const double2 *)dg_in(ctx, gw, nfreq * DD * sizeof(double2), flags, "io.hyb_g", &st);
    if (st) return st;
    const double2 *dH = (const double2 *)dg_in(ctx, himp, DD * sizeof(double2), flags, "io.hyb_h", &st);
    if (st) return st;
    double2 *dD = (double2 *)dg_out(ctx, delta, nfreq * dd * sizeof(double2), flags, "io.hyb_d", &st);
    if (st) return st;
    int *dorb = (int *)dg_buf(ctx, "hyb.orb", dim * sizeof(int));
    double2 *work = (double2 *)dg_buf(ctx, "hyb.work", nfreq * dd * sizeof(double2));
    int *iwork = (int *)dg_buf(ctx, "hyb.iwork", (size_t)nfreq * dim * sizeof(int));
    if (!dorb || !work || !iwork) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemcpyAsync(dorb, orb, dim * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    DG_TRY(dg_status_reset(ctx));
    k_hyb_delta<<<dg_ceil_div(nfreq, 128), 128, 0, ctx->stream>>>(dim, nfreq, D, beta, mu, dorb, dS, dG, dH, work, iwork,
                                                                  dD, ctx->d_status);
    DG_LAUNCH(ctx, "k_hyb_delta");
    DG_TRY(dg_out_done(ctx, delta, dD, nfreq * dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

int dmftgpu_fourier_w2tau(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, const double *fw,
                          const double *mom, int green_asym, const double *m1, double *ft, int flags) {
    if (!ctx || dim < 1 || nfreq < 1 || ntau < 1 || !fw || !ft || !(beta > 0)) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgFtMode ftm(ctx, flags);
    const size_t dd = (size_t)dim * dim;
    int st;
    const double2 *dF = (const double2 *)dg_in(ctx, fw, nfreq * dd * sizeof(double2), flags, "io.ft_fw", &st);
    if (st) return st;
    const double2 *dM = mom ? (const double2 *)dg_in(ctx, mom, 4 * dd * sizeof(double2), flags, "io.ft_mom", &st) : nullptr;
    if (st) return st;
    const double2 *dM1 = m1 ? (const double2 *)dg_in(ctx, m1, dd * sizeof(double2), flags, "io.ft_m1", &st) : nullptr;
    if (st) return st;
    double2 *dT = (double2 *)dg_out(ctx, ft, (ntau + 1) * dd * sizeof(double2), flags, "io.ft_out", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    if (dM) DG_TRY(dg_w2tau_dev(ctx, dim, nfreq, ntau, beta, dF, dM, dT));
    else DG_TRY(dg_fourier_dev(ctx, dim, nfreq, ntau, beta, dF, green_asym, dM1, dT));
    DG_TRY(dg_out_done(ctx, ft, dT, (ntau + 1) * dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

int dmftgpu_fourier_tau2w(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, const double *ft, double *fw,
                          int flags) {
    if (!ctx || dim < 1 || nfreq < 1 || ntau < 1 || !fw || !ft || !(beta > 0)) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgFtMode ftm(ctx, flags);
    const size_t dd = (size_t)dim * dim;
    int st;
    const double2 *dT = (const double2 *)dg_in(ctx, ft, (ntau + 1) * dd * sizeof(double2), flags, "io.t2w_ft", &st);
    if (st) return st;
    double2 *dW = (double2 *)dg_out(ctx, fw, nfreq * dd * sizeof(double2), flags, "io.t2w_fw", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_tau2w_dev(ctx, dim, nfreq, ntau, beta, dT, dW, true));
    DG_TRY(dg_out_done(ctx, fw, dW, nfreq * dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

int dmftgpu_sigma2_tau(dmftgpu_ctx *ctx, int dim, int ntau, double beta, int nu, const int *uidx, const double *ut,
                       const double *gt, double *st_out, int flags) {
    if (!ctx || dim < 1 || ntau < 1 || nu < 0 || !gt || !st_out || (nu > 0 && (!uidx || !ut))) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgFtMode ftm(ctx, flags);
    const size_t dd = (size_t)dim * dim;
    int st;
    DgUList U;
    DG_TRY(dg_ulist(ctx, dim, nu, uidx, ut, U));
    const double2 *dG = (const double2 *)dg_in(ctx, gt, (ntau + 1) * dd * sizeof(double2), flags, "io.s2_gt", &st);
    if (st) return st;
    double2 *dS = (double2 *)dg_out(ctx, st_out, (ntau + 1) * dd * sizeof(double2), flags, "io.s2_st", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_sigma2_dev(ctx, dim, ntau, beta, U, dG, dS));
    DG_TRY(dg_out_done(ctx, st_out, dS, (ntau + 1) * dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

int dmftgpu_fock(dmftgpu_ctx *ctx, int dim, int nu, const int *uidx, const double *ut, const double *occ, double *fock,
                 int flags) {
    if (!ctx || dim < 1 || nu < 0 || !occ || !fock) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    const size_t dd = (size_t)dim * dim;
    int st;
    DgUList U;
    DG_TRY(dg_ulist(ctx, dim, nu, uidx, ut, U));
    const double2 *dO = (const double2 *)dg_in(ctx, occ, dd * sizeof(double2), flags, "io.fk_occ", &st);
    if (st) return st;
    double2 *dF = (double2 *)dg_out(ctx, fock, dd * sizeof(double2), flags, "io.fk_out", &st);
    if (st) return st;
    DG_TRY(dg_fock_dev(ctx, dim, U, dO, dF));
    DG_TRY(dg_out_done(ctx, fock, dF, dd * sizeof(double2), flags));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    return DMFTGPU_OK;
}

int dmftgpu_dyson(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, double mu, const double *himp, const double *delta,
                  const double *fock, const double *sigma2, double *gw, int flags) {
    if (!ctx || dim < 1 || nfreq < 1 || !himp || !delta || !fock || !sigma2 || !gw) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    const size_t dd = (size_t)dim * dim;
    int st;
    const double2 *dH = (const double2 *)dg_in(ctx, himp, dd * sizeof(double2), flags, "io.dy_h", &st);
    if (st) return st;
    const double2 *dD = (const double2 *)dg_in(ctx, delta, nfreq * dd * sizeof(double2), flags, "io.dy_d", &st);
    if (st) return st;
    const double2 *dF = (const double2 *)dg_in(ctx, fock, dd * sizeof(double2), flags, "io.dy_f", &st);
    if (st) return st;
    const double2 *dS = (const double2 *)dg_in(ctx, sigma2, nfreq * dd * sizeof(double2), flags, "io.dy_s", &st);
    if (st) return st;
    double2 *dG = (double2 *)dg_out(ctx, gw, nfreq * dd * sizeof(double2), flags, "io.dy_g", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_dyson_dev(ctx, dim, nfreq, beta, mu, dH, dD, dF, dS, dG, true));
    DG_TRY(dg_out_done(ctx, gw, dG, nfreq * dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

int dmftgpu_occupation(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, const double *gw, double *occ, int flags) {
    if (!ctx || dim < 1 || nfreq < 1 || !gw || !occ) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    const size_t dd = (size_t)dim * dim;
    int st;
    const double2 *dG = (const double2 *)dg_in(ctx, gw, nfreq * dd * sizeof(double2), flags, "io.oc_g", &st);
    if (st) return st;
    double2 *dO = (double2 *)dg_out(ctx, occ, dd * sizeof(double2), flags, "io.oc_o", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_occ_dev(ctx, dim, nfreq, beta, dG, dO));
    DG_TRY(dg_out_done(ctx, occ, dO, dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

int dmftgpu_estimate_asymto(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, double *f, int order, int flags) {
    if (!ctx || dim < 1 || nfreq < 3 || !f || order < 1 || order > 3) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    const size_t dd = (size_t)dim * dim, bytes = (nfreq + 3) * dd * sizeof(double2);
    int st;
    double2 *dF = (double2 *)dg_in(ctx, f, bytes, flags, "io.ea_f", &st);
    if (st) return st;
    DG_TRY(dg_estimate_asymto_dev(ctx, dim, nfreq, beta, dF, order));
    DG_TRY(dg_out_done(ctx, f, dF, bytes, flags));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    return DMFTGPU_OK;
}

}  // extern "C"
