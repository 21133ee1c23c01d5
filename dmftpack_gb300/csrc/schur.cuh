// schur.cuh -- the correlated-block (Schur complement) form of the lattice sum, k_schur<DP,W,MODE>.
//
// The self-energy acts only on the correlated block P (the first D orbitals after the HartrIndex
// permutation), so with Q = the remaining m = n - D orbitals and H_QQ(k) = V diag(e) V^H (once per k):
//
//   G_PP(z)  = S(z)^-1,   S(z)  = z - H_PP - Sigma(z) - sum_l w_l b_l b_l^H,   w_l = 1/(z - e_l),
//   G0_PP(z) = S0(z)^-1,  S0(z) = S(z) + Sigma(z) - m0        (the reference's GwHF: Sigma -> its static
//                                                              moment m0, src/GreenFtn.cpp:197-262)
//   Tr G - Tr G0 = Tr (G_PP - G0_PP) + sum_l w_l^2 b_l^H (G_PP - G0_PP) b_l,
//
// with b_l = H_PQ V(:,l).  These are exact identities (block inversion), so G_loc, GwHF, NumMatrix and the
// occupation sum of GiwToNele are the reference's quantities; the work per (k, iw) drops from an n x n
// inversion to O(D^2 m + D^3).  d/dmu of the trace (Newton's dN/dmu, = -Tr G^2 + Tr G0^2) follows by
// differentiating the same expression: dG_PP/dz = -G S' G with S' = I + sum_l w_l^2 b_l b_l^H.
//
// Mapping: a lane group of W lanes handles one (k, iw) item at a time, lane c holding column c of S (and
// of S0), both inverted with warp_gj_inverse<DP,W> (DP >= D padded with identity).  A CTA owns fpb
// frequencies and sweeps all k; per-group shared-memory accumulators are reduced in a fixed order.
#pragma once
#include "linalg.cuh"

namespace dg {

enum { S_BLOCK = 1, S_TRACE = 2, S_DERIV = 4 };

struct SchurArgs {
    const double2 *H;     // [nk][n][n] column-major, correlated orbitals first
    const double2 *B;     // [nk][m][D]  b_l(a)
    const double *epsQ;   // [nk][m]
    const double2 *sig;   // [2 Nf][D][D]
    const double2 *m0;    // [D][D]
    int n, m, nk, nf2, D, fpb, wgrid;
    double beta, mu;
    double2 *blk, *blk0;  // [nf2][D][D]
    double *tr, *dtr;     // [nf2]
    int *status;
};

template <int DP, int W>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int off = W / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off, W);
    return v;
}

template <int DP, int W, int MODE>
__global__ void __launch_bounds__(128) k_schur(SchurArgs g) {
    constexpr int NG = 128 / W;
    extern __shared__ double2 sm[];
    const int D = g.D, DD = D * D, fpb = g.fpb, m = g.m, n = g.n;
    // shared: acc[NG][fpb][DD], acc0[NG][fpb][DD], acct[NG][fpb], bs[NG][m][D], wls[NG][m], es[NG][m] (double),
    //         tiles[NG][3][DP][DP] (DERIV)
    double2 *acc = sm;
    double2 *acc0 = acc + (size_t)NG * fpb * DD;
    double2 *acct = acc0 + (size_t)NG * fpb * DD;
    double2 *bsa = acct + (size_t)NG * fpb;
    double2 *wla = bsa + (size_t)NG * m * D;
    double2 *tla = wla + (size_t)NG * m;
    double *esa = (double *)(tla + ((MODE & S_DERIV) ? (size_t)NG * 3 * DP * DP : 0));
    for (int t = threadIdx.x; t < NG * fpb * DD; t += blockDim.x) acc[t] = acc0[t] = cmk(0, 0);
    for (int t = threadIdx.x; t < NG * fpb; t += blockDim.x) acct[t] = cmk(0, 0);
    __syncthreads();

    const int c = threadIdx.x & (W - 1);
    const int grp = threadIdx.x / W;
    const int f0 = blockIdx.x * fpb;
    const int nfl = min(fpb, g.nf2 - f0);
    double2 *myacc = acc + (size_t)grp * fpb * DD, *myacc0 = acc0 + (size_t)grp * fpb * DD;
    double2 *myacct = acct + (size_t)grp * fpb;
    double2 *bs = bsa + (size_t)grp * m * D, *wl = wla + (size_t)grp * m;
    double *es = esa + (size_t)grp * m;
    double2 *tS = tla + (size_t)grp * 3 * DP * DP, *tG = tS + DP * DP, *tG0 = tG + DP * DP;
    const bool col = c < D;
    bool sing = false;

    for (int base = 0; base < g.nk; base += NG) {
        const int k = base + grp;
        const bool valid = k < g.nk;
        const int kk = valid ? k : 0;
        __syncwarp();
        for (int t = c; t < m * D; t += W) bs[t] = g.B[(size_t)kk * m * D + t];
        for (int t = c; t < m; t += W) es[t] = g.epsQ[(size_t)kk * m + t];
        __syncwarp();
        // -H_PP(:, c) and the static moment column
        double2 hc[DP], mc[DP];
#pragma unroll
        for (int a = 0; a < DP; a++) {
            hc[a] = (col && a < D) ? cneg(g.H[(size_t)kk * n * n + a + (size_t)c * n]) : cmk(0, 0);
            mc[a] = (col && a < D) ? g.m0[a + c * D] : cmk(0, 0);
        }
        for (int fl = 0; fl < nfl; fl++) {
            const int f = f0 + fl;
            const double w = g.wgrid ? (DG_PI / g.beta + f * ((2 * DG_PI) / g.beta)) : (DG_PI * (2. * f + 1.) / g.beta);
            const double2 z = cmk(g.mu, w);
            __syncwarp();
            for (int l = c; l < m; l += W) wl[l] = crcp(cmk(g.mu - es[l], w));
            __syncwarp();
            const double2 *sg = g.sig + (size_t)f * DD + (size_t)c * D;
            double2 s[DP], s0[DP];
#pragma unroll
            for (int a = 0; a < DP; a++) {
                if (col && a < D) s[a] = csub(hc[a], sg[a]);
                else s[a] = cmk(a == c ? 1.0 : 0.0, 0.0);
                if (a == c && col) s[a] = cadd(s[a], z);
            }
            if (col) {
                for (int l = 0; l < m; l++) {
                    const double2 q = cmulc(wl[l], bs[l * D + c]);  // w_l conj(b_l(c))
#pragma unroll
                    for (int a = 0; a < DP; a++)
                        if (a < D) s[a] = cfms(bs[l * D + a], q, s[a]);
                }
            }
#pragma unroll
            for (int a = 0; a < DP; a++) s0[a] = (col && a < D) ? csub(cadd(s[a], sg[a]), mc[a]) : s[a];
            double2 sp[DP];  // S' = I + sum_l w_l^2 b_l b_l^H (DERIV only)
            if (MODE & S_DERIV) {
#pragma unroll
                for (int a = 0; a < DP; a++) sp[a] = cmk((a == c && col) ? 1.0 : 0.0, 0.0);
                if (col)
                    for (int l = 0; l < m; l++) {
                        const double2 q = cmulc(cmul(wl[l], wl[l]), bs[l * D + c]);
#pragma unroll
                        for (int a = 0; a < DP; a++)
                            if (a < D) sp[a] = cfma(bs[l * D + a], q, sp[a]);
                    }
            }
            sing |= warp_gj_inverse<DP, W>(s, c) && valid;
            sing |= warp_gj_inverse<DP, W>(s0, c) && valid;
            if (MODE & S_BLOCK) {
                if (valid && col) {
#pragma unroll
                    for (int a = 0; a < DP; a++)
                        if (a < D) {
                            const size_t o = (size_t)fl * DD + a + c * D;
                            myacc[o] = cadd(myacc[o], s[a]);
                            myacc0[o] = cadd(myacc0[o], s0[a]);
                        }
                }
            }
            if (MODE & S_TRACE) {
                // X = G - G0 (column c); t1 = Re[X(c,c) + sum_l w_l^2 b_l^H X b_l]
                double2 x[DP];
#pragma unroll
                for (int a = 0; a < DP; a++) x[a] = csub(s[a], s0[a]);
                double2 acc1 = cmk(0, 0), acc2 = cmk(0, 0);
#pragma unroll
                for (int a = 0; a < DP; a++)
                    if (a == c && col) acc1 = x[a];
                double2 y[DP];
                if (MODE & S_DERIV) {
                    // Y = G S' G - G0 S' G0 through the group's shared tiles
                    __syncwarp();
                    if (c < DP) {
#pragma unroll
                        for (int a = 0; a < DP; a++) {
                            tS[a + c * DP] = sp[a];
                            tG[a + c * DP] = s[a];
                            tG0[a + c * DP] = s0[a];
                        }
                    }
                    __syncwarp();
                    double2 u[DP], u0[DP];
#pragma unroll
                    for (int a = 0; a < DP; a++) {
                        u[a] = cmk(0, 0);
                        u0[a] = cmk(0, 0);
#pragma unroll
                        for (int b = 0; b < DP; b++) {
                            u[a] = cfma(tS[a + b * DP], s[b], u[a]);
                            u0[a] = cfma(tS[a + b * DP], s0[b], u0[a]);
                        }
                    }
#pragma unroll
                    for (int a = 0; a < DP; a++) {
                        double2 v = cmk(0, 0);
#pragma unroll
                        for (int b = 0; b < DP; b++) {
                            v = cfma(tG[a + b * DP], u[b], v);
                            v = cfms(tG0[a + b * DP], u0[b], v);
                        }
                        y[a] = v;
                    }
                    __syncwarp();
#pragma unroll
                    for (int a = 0; a < DP; a++)
                        if (a == c && col) acc2 = cneg(y[a]);  // -Tr Y
                }
                if (col) {
                    for (int l = 0; l < m; l++) {
                        const double2 bc = bs[l * D + c];
                        double2 px = cmk(0, 0), py = cmk(0, 0);
#pragma unroll
                        for (int a = 0; a < DP; a++)
                            if (a < D) {
                                const double2 ba = cconj(bs[l * D + a]);
                                px = cfma(ba, x[a], px);
                                if (MODE & S_DERIV) py = cfma(ba, y[a], py);
                            }
                        const double2 w2 = cmul(wl[l], wl[l]);
                        acc1 = cfma(w2, cmul(px, bc), acc1);
                        if (MODE & S_DERIV) {
                            const double2 w3 = cmul(w2, wl[l]);
                            acc2 = cfms(cscale(w3, 2.0), cmul(px, bc), acc2);
                            acc2 = cfms(w2, cmul(py, bc), acc2);
                        }
                    }
                }
                const double t1 = group_sum<DP, W>(col ? acc1.x : 0.0);
                const double t2 = (MODE & S_DERIV) ? group_sum<DP, W>(col ? acc2.x : 0.0) : 0.0;
                if (valid && c == 0) {
                    myacct[fl].x += t1;
                    myacct[fl].y += t2;
                }
            }
        }
    }
    if (sing) dg_flag(g.status, DG_SINGULAR);
    __syncthreads();
    for (int t = threadIdx.x; t < nfl * DD; t += blockDim.x) {
        const int fl = t / DD, e = t % DD;
        if (MODE & S_BLOCK) {
            double2 s = cmk(0, 0), s0 = cmk(0, 0);
            for (int q = 0; q < NG; q++) {
                s = cadd(s, acc[((size_t)q * fpb + fl) * DD + e]);
                s0 = cadd(s0, acc0[((size_t)q * fpb + fl) * DD + e]);
            }
            g.blk[(size_t)(f0 + fl) * DD + e] = s;
            g.blk0[(size_t)(f0 + fl) * DD + e] = s0;
        }
    }
    if (MODE & S_TRACE)
        for (int fl = threadIdx.x; fl < nfl; fl += blockDim.x) {
            double s = 0, s2 = 0;
            for (int q = 0; q < NG; q++) {
                s += acct[(size_t)q * fpb + fl].x;
                s2 += acct[(size_t)q * fpb + fl].y;
            }
            g.tr[f0 + fl] = s;
            if (MODE & S_DERIV) g.dtr[f0 + fl] = s2;
        }
}

// shared-memory bytes of one k_schur launch
inline size_t schur_smem(int DP, int W, int mode, int fpb, int D, int m) {
    const int NG = 128 / W;
    size_t s = (size_t)NG * fpb * D * D * 2 + (size_t)NG * fpb + (size_t)NG * m * D + (size_t)NG * m;
    if (mode & S_DERIV) s += (size_t)NG * 3 * DP * DP;
    return s * sizeof(double2) + (size_t)NG * m * sizeof(double);
}

typedef void (*SchurKernel)(SchurArgs);

template <int DP, int W>
SchurKernel schur_pick(int mode) {
    switch (mode) {
        case S_BLOCK: return k_schur<DP, W, S_BLOCK>;
        case S_TRACE: return k_schur<DP, W, S_TRACE>;
        case S_TRACE | S_DERIV: return k_schur<DP, W, S_TRACE | S_DERIV>;
        default: return nullptr;
    }
}

#define DG_SCHUR_INST(DP, W) \
    SchurKernel schur_kernel_##DP(int mode) { return schur_pick<DP, W>(mode); }
#define DG_SCHUR_DECL(DP) SchurKernel schur_kernel_##DP(int mode);
DG_SCHUR_DECL(1)
DG_SCHUR_DECL(2)
DG_SCHUR_DECL(3)
DG_SCHUR_DECL(4)
DG_SCHUR_DECL(6)
DG_SCHUR_DECL(8)
DG_SCHUR_DECL(10)
DG_SCHUR_DECL(12)
DG_SCHUR_DECL(16)
DG_SCHUR_DECL(20)

}  // namespace dg
