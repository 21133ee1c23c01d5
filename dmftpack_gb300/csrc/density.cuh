// density.cuh -- GreenFtn_w's per-k density matrix in the model basis, densityMatDFT (src/GreenFtn.cpp:170-172,
// 268-275, 311-319), k_dens_sum<DP, W>:
//
//   densityMatDFT[k] = (1/beta) sum_{n < 2 N_freq} [G + G^H - G0 - G0^H](k, iw_n) + U f(e0) U^H
//
// with G = (iw_n + mu - H(k) - Sigma(iw_n))^-1 on the whole model space (Sigma on the correlated block, its moment
// tail beyond N_freq), G0 = U (iw_n + mu - e0)^-1 U^H from the static spectrum of H + m0, and the +-100 cut-offs of
// the Fermi factors.  In the basis T = diag(I_P, V) (H_QQ = V diag(e) V^H, b_l = H_PQ V(:, l), w_l = 1/(z - e_l))
// the full G follows from the correlated block alone:
//
//   G'_PP = S^-1,  G'_PQ = G'_PP B W,  G'_QP = W B^H G'_PP,  G'_QQ = W + W B^H G'_PP B W
//
// so one (k, iw) costs a D x D inversion and O(D^2 m + D m^2) products instead of an n x n inversion.  This kernel
// sums, per k point, Y_PP = sum G'_PP, X_PQ = sum (G'_PQ + G'_QP^H), Y_QQ = sum (W B^H G'_PP B W + W) and the G0
// terms R_j = sum 2 Re 1/(iw_n + mu - e0_j); k_dens_finish (lattice.cu) forms X' = Y + Y^H, rotates it back with T,
// adds U diag(f - R/beta) U^H and undoes the HartrIndex permutation.
//
// Mapping: one CTA per k point (and frequency split); a lane group of W lanes owns one frequency at a time, lane c
// holds column c of S and inverts it with gj_inverse (schur.cuh); the group's products and accumulators live in its
// own shared-memory tiles, reduced over groups in a fixed order at the end.  FP64 (Ops = OpsD) or double-float on
// the FP32 pipe (OpsF, DMFTGPU_MIXED), with 16-byte complex elements either way.
#pragma once
#include "schur.cuh"

namespace dg {

struct DensArgs {
    const double2 *H;    // [nk][n][n] column-major, correlated orbitals first
    const double2 *B;    // [nk][m][D]  b_l(a)
    const double *epsQ;  // [nk][m]
    const double *eps0;  // [nk][n] eigenvalues of H + m0
    const double2 *sig;  // [nf2][D][D] Sigma(iw_n) with its moment tail
    int n, m, nk, nf2, D, ng;
    double beta, mu;
    double2 *Y;  // [nsplit][nk][n][n] per-split sums in the T basis (rows >= D of columns < D unused)
    double *R;   // [nsplit][nk][n]
    int *status;
};

// complex slots of one group: w[m], G tile [DP][DP], Z3 = W B^H G [m][D], X_PQ [D][m], Y_QQ [m][m], sum w [m],
// R [n] (real parts)
__host__ __device__ inline size_t dens_group_elems(int DP, int D, int m, int n) {
    return (size_t)m + (size_t)DP * DP + 2 * (size_t)m * D + (size_t)m * m + m + n;
}
inline size_t dens_smem(int DP, int D, int m, int n, int ng) {
    return ((size_t)m * D + m + (size_t)D * D + n + (size_t)ng * dens_group_elems(DP, D, m, n)) * sizeof(double2);
}

template <class Ops, int DP, int W>
__global__ void __launch_bounds__(128) k_dens_sum(DensArgs g) {
    typedef typename Ops::C C;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int D = g.D, DD = D * D, m = g.m, n = g.n, NG = g.ng;
    const int k = blockIdx.x, split = blockIdx.y, nsplit = gridDim.y;
    const int c = threadIdx.x & (W - 1), grp = threadIdx.x / W;
    const size_t PG = dens_group_elems(DP, D, m, n);
    C *sB = sm, *sE = sB + (size_t)m * D, *sH = sE + m, *sE0 = sH + DD, *gbase = sE0 + n;
    C *wl = gbase + grp * PG, *tG = wl + m, *Z3 = tG + DP * DP, *Xpq = Z3 + (size_t)m * D, *Yqq = Xpq + (size_t)D * m,
      *sw = Yqq + (size_t)m * m, *sr = sw + m;
    for (int t = threadIdx.x; t < m * D; t += blockDim.x) sB[t] = Ops::from(g.B[(size_t)k * m * D + t]);
    for (int t = threadIdx.x; t < m; t += blockDim.x) sE[t] = Ops::from(cmk(g.mu - g.epsQ[(size_t)k * m + t], 0.0));
    for (int t = threadIdx.x; t < DD; t += blockDim.x)
        sH[t] = Ops::from(cneg(g.H[(size_t)k * n * n + t % D + (size_t)(t / D) * n]));
    for (int t = threadIdx.x; t < n; t += blockDim.x) sE0[t] = Ops::from(cmk(g.mu - g.eps0[(size_t)k * n + t], 0.0));
    for (int q = c; q < D * m; q += W) Xpq[q] = Ops::zero();
    for (int q = c; q < m * m; q += W) Yqq[q] = Ops::zero();
    for (int q = c; q < m; q += W) sw[q] = Ops::zero();
    for (int q = c; q < n; q += W) sr[q] = Ops::zero();
    __syncthreads();
    const bool col = c < D;
    C accP[DP];
#pragma unroll
    for (int a = 0; a < DP; a++) accP[a] = Ops::zero();
    bool sing = false;
    // every group of the CTA runs the same number of steps (the warp-collective inversion needs converged warps);
    // a step past the last frequency recomputes the last one and accumulates nothing
    const int stride = nsplit * NG, nstep = (g.nf2 + stride - 1) / stride;
    for (int it = 0; it < nstep; it++) {
        const int f_raw = it * stride + split * NG + grp;
        const bool valid = f_raw < g.nf2;
        const int f = valid ? f_raw : g.nf2 - 1;
        const double w = DG_PI * (2. * f + 1.) / g.beta;
        const C iwc = Ops::from(cmk(0.0, w)), zc = Ops::from(cmk(g.mu, w));
        const double2 *sg = g.sig + (size_t)f * DD;
        __syncwarp();
        for (int l = c; l < m; l += W) {
            const C x = Ops::rcp(Ops::add(sE[l], iwc));
            wl[l] = x;
            if (valid) sw[l] = Ops::add(sw[l], x);
        }
        if (valid)
            for (int j = c; j < n; j += W) {
                const C r = Ops::rcp(Ops::add(sE0[j], iwc));
                sr[j] = Ops::add(sr[j], Ops::add(r, r));  // 2 Re 1/(z - e0_j): the real part is read
            }
        __syncwarp();
        // column c of S = z - H_PP - Sigma - sum_l w_l b_l b_l^H (identity padding beyond D), inverted in place
        C s[DP];
#pragma unroll
        for (int a = 0; a < DP; a++) {
            if (col && a < D) s[a] = Ops::sub(sH[a + c * D], Ops::from(sg[a + (size_t)c * D]));
            else s[a] = (a == c) ? Ops::one() : Ops::zero();
            if (a == c && col) s[a] = Ops::add(s[a], zc);
        }
        if (col)
            for (int l = 0; l < m; l++) {
                const C q = Ops::mulc(wl[l], sB[l * D + c]);
#pragma unroll
                for (int a = 0; a < DP; a++)
                    if (a < D) s[a] = Ops::fms(sB[l * D + a], q, s[a]);
            }
        const bool sg_ = gj_inverse<Ops, DP, W>(s, c);
        sing |= valid && sg_;
        if (valid) {
#pragma unroll
            for (int a = 0; a < DP; a++) accP[a] = Ops::add(accP[a], s[a]);
        }
        if (c < DP) {
#pragma unroll
            for (int a = 0; a < DP; a++) tG[a + c * DP] = s[a];
        }
        __syncwarp();
        // entries (a, l) spread over the lanes: Z1(a, l) = w_l (G b_l)(a), Z3(l, a) = w_l (b_l^H G)(a);
        // X_PQ(a, l) += Z1(a, l) + conj(Z3(l, a))
        for (int q = c; q < D * m; q += W) {
            const int a = q % D, l = q / D;
            const C wv = wl[l];
            const C *bl = sB + (size_t)l * D;
            C z1 = Ops::zero(), z3 = Ops::zero();
            for (int b = 0; b < D; b++) {
                z1 = Ops::fma(tG[a + b * DP], bl[b], z1);
                z3 = Ops::fma(Ops::conj(bl[b]), tG[b + a * DP], z3);
            }
            z1 = Ops::mul(z1, wv);
            z3 = Ops::mul(z3, wv);
            Z3[l + (size_t)a * m] = z3;
            if (valid) Xpq[q] = Ops::add(Xpq[q], Ops::add(z1, Ops::conj(z3)));
        }
        __syncwarp();
        // entries (l, l') spread over the lanes: Y_QQ(l, l') += (Z3 b_l')(l) w_l'
        if (valid)
            for (int q = c; q < m * m; q += W) {
                const int l = q % m, lp = q / m;
                const C *bl = sB + (size_t)lp * D;
                C y = Ops::zero();
                for (int b = 0; b < D; b++) y = Ops::fma(Z3[l + (size_t)b * m], bl[b], y);
                Yqq[q] = Ops::fma(y, wl[lp], Yqq[q]);
            }
    }
    __syncwarp();
    if (c < DP) {
#pragma unroll
        for (int a = 0; a < DP; a++) tG[a + c * DP] = accP[a];
    }
    if (sing) dg_flag(g.status, DG_SINGULAR);
    __syncthreads();
    // fixed-order sum over the groups into this split's partial Y and R
    double2 *Yo = g.Y + ((size_t)split * g.nk + k) * n * n;
    for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
        const int i = q % n, j = q / n;
        double2 v = cmk(0, 0);
        for (int gg = 0; gg < NG; gg++) {
            const C *gb = gbase + gg * PG;
            const C *gG = gb + m, *gX = gG + DP * DP + (size_t)m * D, *gY = gX + (size_t)D * m, *gw = gY + (size_t)m * m;
            if (i < D && j < D) v = cadd(v, Ops::to(gG[i + j * DP]));
            else if (i < D) v = cadd(v, Ops::to(gX[i + (size_t)(j - D) * D]));
            else if (j >= D) {
                v = cadd(v, Ops::to(gY[(i - D) + (size_t)(j - D) * m]));
                if (i == j) v = cadd(v, Ops::to(gw[i - D]));
            }
        }
        Yo[q] = v;
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double r = 0;
        for (int gg = 0; gg < NG; gg++) {
            const C *gb = gbase + gg * PG;
            r += Ops::re((gb + m + DP * DP + 2 * (size_t)m * D + (size_t)m * m + m)[j]);
        }
        g.R[((size_t)split * g.nk + k) * n + j] = r;
    }
}

typedef void (*DensKernel)(DensArgs);
#define DG_DENS_DECL(DP) DensKernel dens_kernel_##DP(bool mixed);
DG_DENS_DECL(1)
DG_DENS_DECL(2)
DG_DENS_DECL(3)
DG_DENS_DECL(4)
DG_DENS_DECL(6)
DG_DENS_DECL(8)
DG_DENS_DECL(10)
DG_DENS_DECL(12)
DG_DENS_DECL(16)
DG_DENS_DECL(20)
#define DG_DENS_INST(DP, W) \
    DensKernel dens_kernel_##DP(bool mixed) { return mixed ? k_dens_sum<OpsF, DP, W> : k_dens_sum<OpsD, DP, W>; }

}  // namespace dg
