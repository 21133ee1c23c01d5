// gloc.cuh -- the fused lattice kernel k_gloc<N,W,MODE> (see lattice.cu) and its argument block.
#pragma once
#include "linalg.cuh"

namespace dg {

// ---------------------------------------------------------------------------------------------------
// the fused inversion / projection / k-reduction kernel
// ---------------------------------------------------------------------------------------------------
enum { M_BLOCK = 1, M_TRACE = 2, M_DERIV = 4 };

struct GlocArgs {
    const double2 *H;    // [nk][n][n], correlated orbitals first
    const double2 *sig;  // [2 Nf][D][D]
    const double *eps;   // [nk][n]
    const double2 *UP;   // [nk][n][D]
    int n, nk, nf2, D, fpb, wgrid;  // wgrid: 0 -> w = pi(2f+1)/beta, 1 -> w = pi/beta + f 2pi/beta
    double beta, mu;
    double2 *blk;   // [nf2][D][D]  sum_k G block
    double2 *blk0;  // [nf2][D][D]  sum_k G0 block
    double *tr;     // [nf2] sum_k Re[Tr G - sum_l 1/(z - e_l)]
    double *dtr;    // [nf2] sum_k Re[-Tr G^2 + sum_l 1/(z - e_l)^2]
    int *status;
};

template <int N, int W, int MODE>
__global__ void __launch_bounds__(128) k_gloc(GlocArgs g) {
    constexpr bool KEEP_H = (N <= 12);  // keep -H(k) columns in registers across the frequency loop
    constexpr int NG = 128 / W;  // lane groups per CTA
    extern __shared__ double2 sm[];
    const int D = g.D, DD = D * D, fpb = g.fpb;
    // shared layout: acc[NG][fpb][DD], acc0[NG][fpb][DD], up[NG][N][D], tile[NG][N][N] (DERIV),
    //                acct[NG][fpb][2] (as double2: x = tr, y = dtr)
    double2 *acc = sm;
    double2 *acc0 = acc + (size_t)NG * fpb * DD;
    double2 *ups = acc0 + (size_t)NG * fpb * DD;
    double2 *tile = ups + (size_t)NG * N * D;
    double2 *acct = tile + ((MODE & M_DERIV) ? (size_t)NG * N * N : 0);
    const int nacc = NG * fpb * (2 * DD + 1);
    for (int t = threadIdx.x; t < NG * fpb * DD; t += blockDim.x) acc[t] = acc0[t] = cmk(0, 0);
    for (int t = threadIdx.x; t < NG * fpb; t += blockDim.x) acct[t] = cmk(0, 0);
    (void)nacc;
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int c = lane & (W - 1);
    const int grp = threadIdx.x / W;
    const int f0 = blockIdx.x * fpb;
    const int nfl = min(fpb, g.nf2 - f0);
    const int n = g.n;
    double2 *myacc = acc + (size_t)grp * fpb * DD, *myacc0 = acc0 + (size_t)grp * fpb * DD;
    double2 *myup = ups + (size_t)grp * N * D, *mytile = tile + (size_t)grp * N * N;
    double2 *myacct = acct + (size_t)grp * fpb;
    bool sing = false;

    for (int base = 0; base < g.nk; base += NG) {
        const int k = base + grp;
        const bool valid = k < g.nk;
        const int kk = valid ? k : 0;
        const double2 *Hk = g.H + (size_t)kk * n * n;
        // this lane's column of -H (identity in the padding block)
        auto load_col = [&](double2 (&dst)[N]) {
#pragma unroll
            for (int i = 0; i < N; i++) {
                if (c < n) dst[i] = (i < n) ? cneg(Hk[i + (size_t)c * n]) : cmk(0, 0);
                else dst[i] = cmk(i == c ? 1.0 : 0.0, 0.0);
            }
        };
        double2 h[KEEP_H ? N : 1];
        if constexpr (KEEP_H) load_col(h);
        const double el = (c < n) ? g.eps[(size_t)kk * n + c] : 0.0;
        if (MODE & M_BLOCK) {
            __syncwarp();
            for (int t = c; t < n * D; t += W) myup[t] = g.UP[(size_t)kk * n * D + t];
            __syncwarp();
        }
        for (int fl = 0; fl < nfl; fl++) {
            const int f = f0 + fl;
            const double w = g.wgrid ? (DG_PI / g.beta + f * ((2 * DG_PI) / g.beta)) : (DG_PI * (2. * f + 1.) / g.beta);
            const double2 z = cmk(g.mu, w);
            double2 a[N];
            if constexpr (KEEP_H) {
#pragma unroll
                for (int i = 0; i < N; i++) a[i] = h[i];
            } else {
                load_col(a);
            }
            if (c < n) {
#pragma unroll
                for (int i = 0; i < N; i++)
                    if (i == c) a[i] = cadd(a[i], z);
            }
            if (c < D) {
                const double2 *sg = g.sig + (size_t)f * DD + (size_t)c * D;
#pragma unroll
                for (int i = 0; i < N; i++)
                    if (i < D) a[i] = csub(a[i], sg[i]);
            }
            sing |= warp_gj_inverse<N, W>(a, c) && valid;
            // dz_l = 1/(z - e_l) on lane l
            const double2 dz = (c < n) ? crcp(cmk(g.mu - el, w)) : cmk(0, 0);
            if (MODE & M_BLOCK) {
                // G block: lane c < D holds column c
                if (valid && c < D) {
#pragma unroll
                    for (int i = 0; i < N; i++)
                        if (i < D) myacc[(size_t)fl * DD + i + c * D] = cadd(myacc[(size_t)fl * DD + i + c * D], a[i]);
                }
                // G0 block: column b = c: sum_l U(a,l) dz_l conj(U(b,l))
                double2 s0[N];
#pragma unroll
                for (int i = 0; i < N; i++) s0[i] = cmk(0, 0);
                for (int l = 0; l < n; l++) {
                    const double2 dzl = shfl2(dz, l, W);
                    if (c < D) {
                        const double2 q = cmulc(dzl, myup[l * D + c]);
#pragma unroll
                        for (int i = 0; i < N; i++)
                            if (i < D) s0[i] = cfma(myup[l * D + i], q, s0[i]);
                    }
                }
                if (valid && c < D) {
#pragma unroll
                    for (int i = 0; i < N; i++)
                        if (i < D) myacc0[(size_t)fl * DD + i + c * D] = cadd(myacc0[(size_t)fl * DD + i + c * D], s0[i]);
                }
            }
            if (MODE & M_TRACE) {
                double2 diag = cmk(0, 0);
#pragma unroll
                for (int i = 0; i < N; i++)
                    if (i == c) diag = a[i];
                double t1 = (c < n) ? (diag.x - dz.x) : 0.0;
                double t2 = 0.0;
                if (MODE & M_DERIV) {
                    __syncwarp();
                    if (c < N) {
#pragma unroll
                        for (int i = 0; i < N; i++) mytile[i + c * N] = a[i];
                    }
                    __syncwarp();
                    double2 s2 = cmk(0, 0);
                    if (c < n) {
#pragma unroll
                        for (int i = 0; i < N; i++)
                            if (i < n) s2 = cfma(a[i], mytile[c + i * N], s2);  // G(i,c) G(c,i)
                    }
                    const double2 dz2 = cmul(dz, dz);
                    t2 = (c < n) ? (-s2.x + dz2.x) : 0.0;
                    __syncwarp();
                }
#pragma unroll
                for (int off = W / 2; off > 0; off >>= 1) {
                    t1 += __shfl_xor_sync(0xffffffffu, t1, off, W);
                    if (MODE & M_DERIV) t2 += __shfl_xor_sync(0xffffffffu, t2, off, W);
                }
                if (valid && c == 0) {
                    myacct[fl].x += t1;
                    myacct[fl].y += t2;
                }
            }
        }
    }
    if (sing) dg_flag(g.status, DG_SINGULAR);
    __syncthreads();
    // fixed-order reduction over the lane groups
    for (int t = threadIdx.x; t < nfl * DD; t += blockDim.x) {
        const int fl = t / DD, e = t % DD;
        if (MODE & M_BLOCK) {
            double2 s = cmk(0, 0), s0 = cmk(0, 0);
            for (int q = 0; q < NG; q++) {
                s = cadd(s, acc[((size_t)q * fpb + fl) * DD + e]);
                s0 = cadd(s0, acc0[((size_t)q * fpb + fl) * DD + e]);
            }
            g.blk[(size_t)(f0 + fl) * DD + e] = s;
            g.blk0[(size_t)(f0 + fl) * DD + e] = s0;
        }
    }
    if (MODE & M_TRACE)
        for (int fl = threadIdx.x; fl < nfl; fl += blockDim.x) {
            double s = 0, s2 = 0;
            for (int q = 0; q < NG; q++) {
                s += acct[(size_t)q * fpb + fl].x;
                s2 += acct[(size_t)q * fpb + fl].y;
            }
            g.tr[f0 + fl] = s;
            if (MODE & M_DERIV) g.dtr[f0 + fl] = s2;
        }
}


typedef void (*GlocKernel)(GlocArgs);

template <int N, int W>
GlocKernel gloc_pick(int mode) {
    switch (mode) {
        case M_BLOCK: return k_gloc<N, W, M_BLOCK>;
        case M_TRACE: return k_gloc<N, W, M_TRACE>;
        case M_TRACE | M_DERIV: return k_gloc<N, W, M_TRACE | M_DERIV>;
        default: return nullptr;
    }
}

// one instantiation unit per size (gloc_inst_*.cu) keeps the build parallel
#define DG_GLOC_INST(N, W) \
    GlocKernel gloc_kernel_##N(int mode) { return gloc_pick<N, W>(mode); }
#define DG_GLOC_DECL(N) GlocKernel gloc_kernel_##N(int mode);
DG_GLOC_DECL(1)
DG_GLOC_DECL(2)
DG_GLOC_DECL(3)
DG_GLOC_DECL(4)
DG_GLOC_DECL(6)
DG_GLOC_DECL(8)
DG_GLOC_DECL(12)
DG_GLOC_DECL(16)
DG_GLOC_DECL(28)

}  // namespace dg
