// adjoint.cuh -- reverse- and forward-mode derivatives of the lattice sum G_loc(iw) = (1/N_k) sum_k G_PP(k, iw)
// with respect to the self-energy and the chemical potential, k_gloc_ad<DP, W, MODE>.
//
// With G = (z - H - Sigma)^-1 on the full orbital space and Sigma acting on the correlated block P:
//   dG_PP = G_PP dSigma G_PP                      (dSigma lives on P, so only the P block of G enters)
//   dG_PP = -(G^2)_PP dmu = -G_PP S' G_PP dmu    (S' = I + sum_l w_l^2 b_l b_l^H, the Schur form's dS/dz)
// so for one frequency
//   JVP:  dG_loc = (1/N_k) sum_k G_PP (dSigma - dmu S') G_PP
//   VJP:  Sigma_bar = (1/N_k) sum_k G_PP^H Gbar G_PP^H,   mu_bar = -(1/N_k) sum_k Re Tr[(G_PP S' G_PP)^H Gbar]
// (the adjoint of the holomorphic map in the convention of torch's complex autograd: x_bar = J^H y_bar).  G_PP
// is recomputed for every (k, iw) from the per-k Schur data, as the forward pass does, and never stored: the
// memory is O(N_freq D^2) whatever N_k, N_freq and n are.
//
// Mapping as in k_schur (schur.cuh): a lane group of W lanes per frequency, lane c = column c, a CTA = 128/W
// frequencies x one chunk of k points staged in shared memory, FP64, per-chunk sums reduced in fixed order.
#pragma once
#include "schur.cuh"

namespace dg {

enum { AD_VJP = 1, AD_JVP = 2 };

struct AdArgs {
    const double2 *H, *B;  // as SchurArgs
    const double *epsQ;
    const double2 *sig;    // [nf][D][D] Sigma(iw_n), n < nf
    const double2 *gin;    // VJP: Gbar [nf][D][D]; JVP: Sigma_dot [nf][D][D]
    double mu_dot;         // JVP
    int n, m, nk, nf, D, kc, kchunk;
    double beta, mu;
    double2 *pout;         // [nchunk][nf][D][D] per-chunk sums (Sigma_bar or G_loc_dot, before the 1/N_k)
    double *pmu;           // [nchunk][nf] VJP: per-chunk Re Tr[(G S' G)^H Gbar]
    int *status;
};

template <int DP, int W, int MODE>
__global__ void __launch_bounds__(128) k_gloc_ad(AdArgs g) {
    typedef OpsD Ops;
    typedef double2 C;
    constexpr int NG = 128 / W;
    extern __shared__ double2 sm[];
    const int D = g.D, DD = D * D, m = g.m;
    C *sB = sm, *sE = sB + (size_t)g.kc * m * D, *sH = sE + (size_t)g.kc * m;
    C *wla = sH + (size_t)g.kc * DD;                  // [NG][m]
    C *tla = wla + (size_t)NG * m;                    // [NG][4][DP][DP]: S', G, input (Gbar or Sigma_dot), work
    const int c = threadIdx.x & (W - 1), grp = threadIdx.x / W;
    const int f_raw = blockIdx.x * NG + grp;
    const bool fvalid = f_raw < g.nf;
    const int f = fvalid ? f_raw : g.nf - 1;
    const int chunk = blockIdx.y;
    const int kbeg = chunk * g.kchunk, kend = min(g.nk, kbeg + g.kchunk);
    C *tS = tla + (size_t)grp * 4 * DP * DP, *tG = tS + DP * DP, *tX = tG + DP * DP, *tV = tX + DP * DP;
    C *wl = wla + (size_t)grp * m;
    const bool col = c < D;
    const double w = DG_PI * (2. * f + 1.) / g.beta;
    const C zc = cmk(g.mu, w), iwc = cmk(0.0, w);
    // the group's frequency data: Sigma(:, c) in registers, Gbar / Sigma_dot as a tile
    C sgc[DP];
#pragma unroll
    for (int a = 0; a < DP; a++) sgc[a] = (col && a < D) ? g.sig[(size_t)f * DD + a + (size_t)c * D] : cmk(0, 0);
    if (c < DP)
        for (int a = 0; a < DP; a++)
            tX[a + c * DP] = (col && a < D) ? g.gin[(size_t)f * DD + a + (size_t)c * D] : cmk(0, 0);
    C acc[DP];
#pragma unroll
    for (int a = 0; a < DP; a++) acc[a] = cmk(0, 0);
    double accmu = 0.0;
    bool sing = false;
    for (int k0 = kbeg; k0 < kend; k0 += g.kc) {
        const int nkc = min(g.kc, kend - k0);
        __syncthreads();
        for (int t = threadIdx.x; t < nkc * m * D; t += blockDim.x) sB[t] = g.B[(size_t)k0 * m * D + t];
        for (int t = threadIdx.x; t < nkc * m; t += blockDim.x) sE[t] = cmk(g.mu - g.epsQ[(size_t)k0 * m + t], 0.0);
        for (int t = threadIdx.x; t < nkc * DD; t += blockDim.x) {
            const int kk = t / DD, e = t % DD, a = e % D, b = e / D;
            sH[t] = cneg(g.H[(size_t)(k0 + kk) * g.n * g.n + a + (size_t)b * g.n]);
        }
        __syncthreads();
        for (int kk = 0; kk < nkc; kk++) {
            const C *bs = sB + (size_t)kk * m * D, *es = sE + (size_t)kk * m, *hp = sH + (size_t)kk * DD;
            __syncwarp();
            for (int l = c; l < m; l += W) wl[l] = crcp(cadd(es[l], iwc));
            __syncwarp();
            // column c of S(z) = z - H_PP - Sigma - sum_l w_l b_l b_l^H, and of S' = I + sum_l w_l^2 b_l b_l^H
            C s[DP], sp[DP];
#pragma unroll
            for (int a = 0; a < DP; a++) {
                if (col && a < D) s[a] = csub(hp[a + c * D], sgc[a]);
                else s[a] = (a == c) ? cmk(1, 0) : cmk(0, 0);
                if (a == c && col) s[a] = cadd(s[a], zc);
                sp[a] = (a == c && col) ? cmk(1, 0) : cmk(0, 0);
            }
            if (col)
                for (int l = 0; l < m; l++) {
                    const C q = cmulc(wl[l], bs[l * D + c]);
                    const C q2 = cmul(wl[l], q);
#pragma unroll
                    for (int a = 0; a < DP; a++)
                        if (a < D) {
                            s[a] = cfms(bs[l * D + a], q, s[a]);
                            sp[a] = cfma(bs[l * D + a], q2, sp[a]);
                        }
                }
            sing |= gj_inverse<Ops, DP, W>(s, c);  // s = G(:, c)
            __syncwarp();
            if (c < DP) {
#pragma unroll
                for (int a = 0; a < DP; a++) {
                    tG[a + c * DP] = s[a];
                    tS[a + c * DP] = sp[a];
                }
            }
            __syncwarp();
            // the intermediate column v goes through the group's work tile, so only G(:, c), S'(:, c), Sigma(:, c)
            // and the accumulator live in registers; the inner sums are rolled loops over shared memory
            if (MODE == AD_JVP) {
                // column c of G (Sigma_dot - mu_dot S') G: v = (Sigma_dot - mu_dot S') G(:, c), then G v
                if (c < DP)
                    for (int a = 0; a < DP; a++) {
                        C x = cmk(0, 0);
#pragma unroll 4
                        for (int b = 0; b < DP; b++)
                            x = cfma(csub(tX[a + b * DP], cscale(tS[a + b * DP], g.mu_dot)), tG[b + c * DP], x);
                        tV[a + c * DP] = x;
                    }
                __syncwarp();
#pragma unroll
                for (int a = 0; a < DP; a++) {
                    C x = cmk(0, 0);
                    if (c < DP)
#pragma unroll 4
                        for (int b = 0; b < DP; b++) x = cfma(tG[a + b * DP], tV[b + c * DP], x);
                    acc[a] = cadd(acc[a], x);
                }
                __syncwarp();
            } else {
                // column c of G^H Gbar G^H: v = Gbar conj(G(c, :))^T, then G^H v
                if (c < DP)
                    for (int a = 0; a < DP; a++) {
                        C x = cmk(0, 0);
#pragma unroll 4
                        for (int b = 0; b < DP; b++) x = cfma(tX[a + b * DP], cconj(tG[c + b * DP]), x);
                        tV[a + c * DP] = x;
                    }
                __syncwarp();
#pragma unroll
                for (int a = 0; a < DP; a++) {
                    C x = cmk(0, 0);
                    if (c < DP)
#pragma unroll 4
                        for (int b = 0; b < DP; b++) x = cfma(cconj(tG[b + a * DP]), tV[b + c * DP], x);
                    acc[a] = cadd(acc[a], x);
                }
                __syncwarp();
                // Re Tr[(G S' G)^H Gbar], column c: u = S' G(:, c) in the work tile, y = G u, sum_a Re(Gbar(a,c) conj(y_a))
                if (c < DP)
                    for (int a = 0; a < DP; a++) {
                        C x = cmk(0, 0);
#pragma unroll 4
                        for (int b = 0; b < DP; b++) x = cfma(tS[a + b * DP], tG[b + c * DP], x);
                        tV[a + c * DP] = x;
                    }
                __syncwarp();
                double t = 0.0;
                if (col)
                    for (int a = 0; a < D; a++) {
                        C y = cmk(0, 0);
#pragma unroll 4
                        for (int b = 0; b < DP; b++) y = cfma(tG[a + b * DP], tV[b + c * DP], y);
                        t += cmulc(tX[a + c * DP], y).x;
                    }
                accmu += group_sum<DP, W>(t, 0);
                __syncwarp();
            }
        }
    }
    if (sing && fvalid) dg_flag(g.status, DG_SINGULAR);
    if (!fvalid) return;
    if (col) {
        const size_t o = ((size_t)chunk * g.nf + f) * DD + (size_t)c * D;
#pragma unroll
        for (int a = 0; a < DP; a++)
            if (a < D) g.pout[o + a] = acc[a];
    }
    if (MODE == AD_VJP && c == 0) g.pmu[(size_t)chunk * g.nf + f] = accmu;
}

inline size_t ad_smem(int DP, int W, int kc, int D, int m) {
    const int NG = 128 / W;
    return ((size_t)kc * m * D + (size_t)kc * m + (size_t)kc * D * D + (size_t)NG * m + (size_t)NG * 4 * DP * DP) * 16;
}

typedef void (*AdKernel)(AdArgs);
#define DG_AD_DECL(DP) AdKernel ad_kernel_##DP(int mode);
DG_AD_DECL(1)
DG_AD_DECL(2)
DG_AD_DECL(3)
DG_AD_DECL(4)
DG_AD_DECL(6)
DG_AD_DECL(8)
DG_AD_DECL(10)
DG_AD_DECL(12)
DG_AD_DECL(16)
DG_AD_DECL(20)
#define DG_AD_INST(DP, W) \
    AdKernel ad_kernel_##DP(int mode) { return mode == AD_VJP ? k_gloc_ad<DP, W, AD_VJP> : k_gloc_ad<DP, W, AD_JVP>; }

}  // namespace dg
