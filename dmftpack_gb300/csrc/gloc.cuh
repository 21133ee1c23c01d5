// gloc.cuh -- the fused lattice kernel k_gloc<N,W,MODE> (see lattice.cu) and its argument block.
#pragma once
#include <type_traits>

#include "df.cuh"
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

// smem bytes of one k_gloc launch: acc, acc0 [NG][fpb][DD], up [NG][N][D], tile [NG][N][N] (DERIV), all of the
// arithmetic's complex type; acct [NG][fpb] (double2: x = tr, y = dtr); sg [fpb][DD] and z [fpb] (complex type)
__host__ __device__ inline size_t gloc_smem(int N, int W, int mode, int fpb, int D, size_t csize) {
    const size_t NG = 128 / W, DD = (size_t)D * D;
    size_t c = NG * fpb * DD * 2 + NG * N * D + (size_t)fpb * DD + fpb;
    if (mode & M_DERIV) c += NG * (size_t)N * N;
    return c * csize + NG * fpb * sizeof(double2);
}

// Ops = OpsD: FP64 throughout.  Ops = OpsF: the inversion, the G0 block and the sums over this CTA's k points in
// double-float on the FP32 pipe (df.cuh); H, Sigma, the spectra and U are converted once per k (per CTA for Sigma)
// and the partial sums once at the end, so no FP64 instruction runs per (k, iw) point.
template <class Ops, int N, int W, int MODE>
__global__ void __launch_bounds__(128) k_gloc(GlocArgs g) {
    typedef typename Ops::C C;
    constexpr bool KEEP_H = (N <= 12);  // keep -H(k) columns in registers across the frequency loop
    // double-float Gauss-Jordan from N = 8 up in the rolled form: the unrolled one overflows the instruction cache
    constexpr bool ROLLED = !std::is_same<C, double2>::value && N >= 8;
    constexpr int NG = 128 / W;  // lane groups per CTA
    extern __shared__ __align__(16) unsigned char smraw[];
    const int D = g.D, DD = D * D, fpb = g.fpb;
    C *acc = reinterpret_cast<C *>(smraw);
    C *acc0 = acc + (size_t)NG * fpb * DD;
    C *ups = acc0 + (size_t)NG * fpb * DD;
    C *tile = ups + (size_t)NG * N * D;
    C *sgs = tile + ((MODE & M_DERIV) ? (size_t)NG * N * N : 0);
    C *zs = sgs + (size_t)fpb * DD;
    double2 *acct = reinterpret_cast<double2 *>(zs + fpb);
    const int f0 = blockIdx.x * fpb;
    const int nfl = min(fpb, g.nf2 - f0);
    for (int t = threadIdx.x; t < NG * fpb * DD; t += blockDim.x) acc[t] = acc0[t] = Ops::zero();
    for (int t = threadIdx.x; t < NG * fpb; t += blockDim.x) acct[t] = cmk(0, 0);
    for (int t = threadIdx.x; t < fpb * DD; t += blockDim.x)
        sgs[t] = (t < nfl * DD) ? Ops::from(g.sig[(size_t)f0 * DD + t]) : Ops::zero();
    for (int t = threadIdx.x; t < fpb; t += blockDim.x) {
        const int f = f0 + t;
        const double w = g.wgrid ? (DG_PI / g.beta + f * ((2 * DG_PI) / g.beta)) : (DG_PI * (2. * f + 1.) / g.beta);
        zs[t] = Ops::from(cmk(g.mu, w));
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int c = lane & (W - 1);
    const int grp = threadIdx.x / W;
    const int n = g.n;
    C *myacc = acc + (size_t)grp * fpb * DD, *myacc0 = acc0 + (size_t)grp * fpb * DD;
    C *myup = ups + (size_t)grp * N * D, *mytile = tile + (size_t)grp * N * N;
    double2 *myacct = acct + (size_t)grp * fpb;
    bool sing = false;

    for (int base = 0; base < g.nk; base += NG) {
        const int k = base + grp;
        const bool valid = k < g.nk;
        const int kk = valid ? k : 0;
        const double2 *Hk = g.H + (size_t)kk * n * n;
        // this lane's column of -H (identity in the padding block)
        auto load_col = [&](C (&dst)[N]) {
#pragma unroll
            for (int i = 0; i < N; i++) {
                if (c < n) dst[i] = (i < n) ? Ops::from(cneg(Hk[i + (size_t)c * n])) : Ops::zero();
                else dst[i] = (i == c) ? Ops::one() : Ops::zero();
            }
        };
        C h[KEEP_H ? N : 1];
        if constexpr (KEEP_H) load_col(h);
        const C el = Ops::from(cmk((c < n) ? g.eps[(size_t)kk * n + c] : 0.0, 0.0));
        if (MODE & M_BLOCK) {
            __syncwarp();
            for (int t = c; t < n * D; t += W) myup[t] = Ops::from(g.UP[(size_t)kk * n * D + t]);
            __syncwarp();
        }
        for (int fl = 0; fl < nfl; fl++) {
            const C z = zs[fl];
            C a[N];
            if constexpr (KEEP_H) {
#pragma unroll
                for (int i = 0; i < N; i++) a[i] = h[i];
            } else {
                load_col(a);
            }
            if (c < n) {
#pragma unroll
                for (int i = 0; i < N; i++)
                    if (i == c) a[i] = Ops::add(a[i], z);
            }
            if (c < D) {
                const C *sg = sgs + (size_t)fl * DD + (size_t)c * D;
#pragma unroll
                for (int i = 0; i < N; i++)
                    if (i < D) a[i] = Ops::sub(a[i], sg[i]);
            }
            if constexpr (ROLLED) sing |= warp_gj_inverse_rolled<Ops, N, W>(a, c) && valid;
            else sing |= warp_gj_inverse_t<Ops, N, W>(a, c) && valid;
            // dz_l = 1/(z - e_l) on lane l
            const C dz = (c < n) ? Ops::rcp(Ops::sub(z, el)) : Ops::zero();
            if (MODE & M_BLOCK) {
                // G block: lane c < D holds column c
                if (valid && c < D) {
#pragma unroll
                    for (int i = 0; i < N; i++)
                        if (i < D) myacc[(size_t)fl * DD + i + c * D] = Ops::add(myacc[(size_t)fl * DD + i + c * D], a[i]);
                }
                // G0 block: column b = c: sum_l U(a,l) dz_l conj(U(b,l))
                C s0[N];
#pragma unroll
                for (int i = 0; i < N; i++) s0[i] = Ops::zero();
                for (int l = 0; l < n; l++) {
                    const C dzl = Ops::shfl(dz, l, W);
                    if (c < D) {
                        const C q = Ops::mulc(dzl, myup[l * D + c]);
#pragma unroll
                        for (int i = 0; i < N; i++)
                            if (i < D) s0[i] = Ops::fma(myup[l * D + i], q, s0[i]);
                    }
                }
                if (valid && c < D) {
#pragma unroll
                    for (int i = 0; i < N; i++)
                        if (i < D) myacc0[(size_t)fl * DD + i + c * D] = Ops::add(myacc0[(size_t)fl * DD + i + c * D], s0[i]);
                }
            }
            if (MODE & M_TRACE) {
                C diag = Ops::zero();
#pragma unroll
                for (int i = 0; i < N; i++)
                    if (i == c) diag = a[i];
                C t1 = (c < n) ? Ops::sub(diag, dz) : Ops::zero();
                C t2 = Ops::zero();
                if (MODE & M_DERIV) {
                    __syncwarp();
                    if (c < N) {
#pragma unroll
                        for (int i = 0; i < N; i++) mytile[i + c * N] = a[i];
                    }
                    __syncwarp();
                    C s2 = Ops::zero();
                    if (c < n) {
#pragma unroll
                        for (int i = 0; i < N; i++)
                            if (i < n) s2 = Ops::fma(a[i], mytile[c + i * N], s2);  // G(i,c) G(c,i)
                    }
                    t2 = (c < n) ? Ops::sub(Ops::mul(dz, dz), s2) : Ops::zero();
                    __syncwarp();
                }
#pragma unroll
                for (int off = W / 2; off > 0; off >>= 1) {
                    t1 = Ops::add(t1, Ops::shfl(t1, c ^ off, W));
                    if (MODE & M_DERIV) t2 = Ops::add(t2, Ops::shfl(t2, c ^ off, W));
                }
                if (valid && c == 0) {
                    myacct[fl].x += Ops::re(t1);
                    myacct[fl].y += Ops::re(t2);
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
                s = cadd(s, Ops::to(acc[((size_t)q * fpb + fl) * DD + e]));
                s0 = cadd(s0, Ops::to(acc0[((size_t)q * fpb + fl) * DD + e]));
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

template <class Ops, int N, int W>
GlocKernel gloc_pick(int mode) {
    switch (mode) {
        case M_BLOCK: return k_gloc<Ops, N, W, M_BLOCK>;
        case M_TRACE: return k_gloc<Ops, N, W, M_TRACE>;
        case M_TRACE | M_DERIV: return k_gloc<Ops, N, W, M_TRACE | M_DERIV>;
        default: return nullptr;
    }
}

// one instantiation unit per size (gloc_inst_*.cu) keeps the build parallel
#define DG_GLOC_INST(N, W)                                                                      \
    GlocKernel gloc_kernel_##N(int mode, bool mixed) {                                          \
        return mixed ? gloc_pick<OpsF, N, W>(mode) : gloc_pick<OpsD, N, W>(mode);               \
    }
#define DG_GLOC_DECL(N) GlocKernel gloc_kernel_##N(int mode, bool mixed);
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
