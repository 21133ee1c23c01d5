// schur.cuh -- the correlated-block (Schur complement) form of the lattice sum, k_schur<DP,W,MODE>.
//
// The self-energy acts only on the correlated block P (the first D orbitals after the HartrIndex
// permutation), so with Q = the remaining m = n - D orbitals and H_QQ(k) = V diag(e) V^H (once per k):
//
//   G_PP(z)  = S(z)^-1,   S(z)  = z - H_PP - Sigma(z) - sum_l w_l b_l b_l^H,   w_l = 1/(z - e_l),
//   G0_PP(z) = S0(z)^-1,  S0(z) = S(z) + Sigma(z) - m0        (the reference's GwHF: Sigma -> its static
//                                                              moment m0, src/GreenFtn.cpp:197-262)
//   Tr G(z) = Tr G_PP + sum_l w_l + sum_l w_l^2 b_l^H G_PP b_l,      Tr G0(z) = sum_j 1/(z - e0_j),
//
// with b_l = H_PQ V(:,l) and e0_j the eigenvalues of H + m0 (the reference's static spectrum, whose
// resolvent U (z - e0)^-1 U^H is its G0, src/GreenFtn.cpp:197-262).  These are exact identities (block
// inversion), so G_loc, GwHF, NumMatrix and the occupation sum of GiwToNele are the reference's quantities;
// the work per (k, iw) drops from an n x n inversion to O(D^2 m + D^3).  d/dmu of the trace (Newton's
// dN/dmu) is d/dz of the same expression: dG_PP/dz = -G S' G with S' = I + sum_l w_l^2 b_l b_l^H, dw_l/dz =
// -w_l^2.  The TRACE passes of the mu search invert S only; the BLOCK pass (G_loc, GwHF) inverts S0 as well for
// small blocks, and for DP >= 8 forms GwHF as U (z - e0)^-1 U^H from the static eigen-decomposition (the
// reference's own formula), keeping one unrolled inversion per kernel (instruction-cache bound otherwise).
//
// Mapping: a lane group of W lanes owns one Matsubara frequency and sweeps a chunk of k points; lane c holds
// column c of S (and S0), inverted with gj_inverse<Ops,DP,W> (DP >= D padded with identity), and
// accumulates column c of the k sum in registers.  A CTA = 128/W frequencies x one k chunk; the per-k data
// (b_l, mu - e_l, -H_PP) of kc k points at a time is staged once in shared memory in the kernel's
// arithmetic type.  Per-chunk sums are reduced over chunks in a fixed order by a second kernel.
// Ops = OpsD (FP64) or OpsF (double-float on the FP32 pipe; FP64 appears only when staging and storing).
#pragma once
#include <type_traits>
#include "df.cuh"
#include "linalg.cuh"

namespace dg {

// S_REAL: the real-axis grid z = mu + (e0 + n de) + i eta of the spectra (retarded_GreenFtn2, src/GreenFtn.cpp:
// 425-466), with TRACE giving the complex Tr G(z) of the whole model space (no G0 term) and BLOCK G_PP only
enum { S_BLOCK = 1, S_TRACE = 2, S_DERIV = 4, S_REAL = 8 };

struct SchurArgs {
    const double2 *H;     // [nk][n][n] column-major, correlated orbitals first
    const double2 *B;     // [nk][m][D]  b_l(a)
    const double *epsQ;   // [nk][m]
    const double2 *sig;   // [2 Nf][D][D]
    const double2 *m0;    // [D][D]
    const double *eps0;   // [nk][n] eigenvalues of H + m0 (TRACE modes; BLOCK for DP >= 8)
    const double2 *UP;    // [nk][n][D] correlated rows of their eigenvectors (BLOCK for DP >= 8)
    int n, m, nk, nf2, D, wgrid, kc, kchunk;  // kc: k points staged per round; kchunk: k points per CTA
    double e0, de, eta;                        // S_REAL grid
    double beta, mu;
    double2 *pblk, *pblk0;  // [nchunk][nf2][D][D]  per-chunk k sums (BLOCK)
    double2 *ptr;           // [nchunk][nf2]         per-chunk trace sums (x = tr, y = dtr)
    int *status;
};

// the rolled Gauss-Jordan (df.cuh) for double-float at every width and for FP64 from 8 on (measured: double-float
// kernels are instruction-fetch bound, FP64 ones FP64-pipe bound), the unrolled one otherwise
template <class Ops, int DP, int W>
__device__ __forceinline__ bool gj_inverse(typename Ops::C (&a)[DP], int c) {
    if constexpr (DP >= 8 || (std::is_same<Ops, OpsF>::value && DP >= 2))
        return warp_gj_inverse_rolled<Ops, DP, W>(a, c);
    else
        return warp_gj_inverse_t<Ops, DP, W>(a, c);
}

template <int DP, int W>
__device__ __forceinline__ double group_sum(double v, int base) {
    if constexpr ((W & (W - 1)) != 0) {  // packed groups: the W lanes from base, in a fixed order
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < W; j++) s += __shfl_sync(0xffffffffu, v, (base + j) & 31, 32);
        return s;
    } else {
#pragma unroll
        for (int off = W / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off, W);
        return v;
    }
}

// staged per-k data in shared memory (arithmetic type C): B[kc][m][D], e[kc][m] (mu - e_l, real),
// hpp[kc][D][D] (-H_PP), e0[kc][n] (mu - e0_j, TRACE modes), then once m0[D][D]
template <class Ops>
__device__ __forceinline__ void schur_stage(const SchurArgs &g, int k0, int nkc, typename Ops::C *st, bool e0,
                                            bool up) {
    typedef typename Ops::C C;
    const int m = g.m, D = g.D, DD = D * D;
    C *sB = st, *sE = sB + (size_t)g.kc * m * D, *sH = sE + (size_t)g.kc * m;
    C *sE0 = sH + (size_t)g.kc * DD, *sU = sE0 + (e0 ? (size_t)g.kc * g.n : 0);
    if (e0)
        for (int t = threadIdx.x; t < nkc * g.n; t += blockDim.x)
            sE0[t] = Ops::from(cmk(g.mu - g.eps0[(size_t)k0 * g.n + t], 0.0));
    if (up)
        for (int t = threadIdx.x; t < nkc * g.n * D; t += blockDim.x) sU[t] = Ops::from(g.UP[(size_t)k0 * g.n * D + t]);
    for (int t = threadIdx.x; t < nkc * m * D; t += blockDim.x) sB[t] = Ops::from(g.B[(size_t)k0 * m * D + t]);
    for (int t = threadIdx.x; t < nkc * m; t += blockDim.x)
        sE[t] = Ops::from(cmk(g.mu - g.epsQ[(size_t)k0 * m + t], 0.0));
    for (int t = threadIdx.x; t < nkc * DD; t += blockDim.x) {
        const int kk = t / DD, e = t % DD, a = e % D, b = e / D;
        sH[t] = Ops::from(cneg(g.H[(size_t)(k0 + kk) * g.n * g.n + a + (size_t)b * g.n]));
    }
}

// lane groups per 128-thread CTA: W a power of two, 128 / W; otherwise (W = DP, "packed") 32 / W groups per warp,
// the warp's remaining lanes idle
__host__ __device__ constexpr int schur_groups(int W) { return (W & (W - 1)) ? 4 * (32 / W) : 128 / W; }

// Lane group = one Matsubara frequency; CTA = NG frequencies x one chunk of k points.  W a power of two: groups of
// W lanes, exchanges by shuffles of width W.  W not a power of two (W = DP = 10): 32 / W groups of W lanes per warp
// (three of ten at D = 10, where 16-lane groups leave six lanes of every group idle), exchanges by full-warp
// shuffles from absolute source lanes; the two lanes outside the groups compute values that are never written.
template <class Ops, int DP, int W, int MODE>
__global__ void __launch_bounds__(128) k_schur(SchurArgs g) {
    typedef typename Ops::C C;
    constexpr bool PACK = (W & (W - 1)) != 0;
    static_assert(!PACK || W == DP, "packed groups are one column per lane");
    constexpr int GPW = PACK ? 32 / W : 1;
    constexpr int NG = schur_groups(W);
    extern __shared__ double2 sm[];
    const int D = g.D, DD = D * D, m = g.m;
    constexpr bool TR = (MODE & S_TRACE) != 0;
    constexpr bool RE = (MODE & S_REAL) != 0;
    constexpr bool G0E = (MODE & S_BLOCK) && DP >= 8 && !RE;  // GwHF from the static eigen-decomposition
    constexpr bool E0 = (TR && !RE) || G0E;
    C *st = reinterpret_cast<C *>(sm);
    C *sB = st, *sE = sB + (size_t)g.kc * m * D, *sH = sE + (size_t)g.kc * m;
    C *sE0 = sH + (size_t)g.kc * DD;                                      // [kc][n] (E0)
    C *sU = sE0 + (E0 ? (size_t)g.kc * g.n : 0);                         // [kc][n][D] (G0E)
    C *sM0 = sU + (G0E ? (size_t)g.kc * g.n * D : 0);
    C *wla = sM0 + DD;                                                   // reciprocals [NG][m]
    C *rla = wla + (size_t)NG * m;                                        // static reciprocals [NG][n] (E0)
    C *tla = rla + (E0 ? (size_t)NG * g.n : 0);                           // DERIV tiles [NG][2][DP][DP]
    const int lane = threadIdx.x & 31, gw = PACK ? lane / W : 0;
    const bool active = !PACK || gw < GPW;  // a lane of a group (packed: lanes 30, 31 of each warp are not)
    const int c = PACK ? lane % W : (threadIdx.x & (W - 1));
    const int grp = PACK ? (active ? (threadIdx.x >> 5) * GPW + gw : 0) : threadIdx.x / W;
    const int base = PACK ? gw * W : 0;     // the group's first lane in its warp
    const int f_raw = blockIdx.x * NG + grp;
    const bool fvalid = active && f_raw < g.nf2;
    const int f = fvalid ? f_raw : g.nf2 - 1;
    const int chunk = blockIdx.y;
    const int kbeg = chunk * g.kchunk, kend = min(g.nk, kbeg + g.kchunk);
    C *tS = tla + (size_t)grp * 2 * DP * DP, *tG = tS + DP * DP;
    C *wl = wla + (size_t)grp * m;
    C *rl = rla + (size_t)grp * g.n;
    const bool col = c < D;
    for (int t = threadIdx.x; t < DD; t += blockDim.x) sM0[t] = Ops::from(g.m0[t]);
    // per-group frequency constants: iw (as a complex with zero real part), z = mu + iw, Sigma(:, c)
    const double w = g.wgrid ? (DG_PI / g.beta + f * ((2 * DG_PI) / g.beta)) : (DG_PI * (2. * f + 1.) / g.beta);
    // iwc: z - mu (i w_n, or E + i eta on the real axis); zc = z
    const C zc = RE ? Ops::from(cmk(g.mu + (g.e0 + f * g.de), g.eta)) : Ops::from(cmk(g.mu, w));
    const C iwc = RE ? Ops::from(cmk(g.e0 + f * g.de, g.eta)) : Ops::from(cmk(0.0, w));
    C sgc[DP];
#pragma unroll
    for (int a = 0; a < DP; a++) sgc[a] = (col && a < D) ? Ops::from(g.sig[(size_t)f * DD + a + (size_t)c * D]) : Ops::zero();
    C accG[DP], accG0[DP];
#pragma unroll
    for (int a = 0; a < DP; a++) accG[a] = accG0[a] = Ops::zero();
    double acct1 = 0.0, acct2 = 0.0;
    bool sing = false;

    for (int k0 = kbeg; k0 < kend; k0 += g.kc) {
        const int nkc = min(g.kc, kend - k0);
        __syncthreads();
        schur_stage<Ops>(g, k0, nkc, st, E0, G0E);
        __syncthreads();
        for (int kk = 0; kk < nkc; kk++) {
            const C *bs = sB + (size_t)kk * m * D, *es = sE + (size_t)kk * m, *hp = sH + (size_t)kk * DD;
            // w_l = 1/(z - e_l), shared by the group's lanes; TRACE: r_j = 1/(z - e0_j)
            __syncwarp();
            if (active) {
                for (int l = c; l < m; l += W) wl[l] = Ops::rcp(Ops::add(es[l], iwc));
                if (E0) {
                    const C *e0s = sE0 + (size_t)kk * g.n;
                    for (int j = c; j < g.n; j += W) rl[j] = Ops::rcp(Ops::add(e0s[j], iwc));
                }
            }
            __syncwarp();
            C s[DP], s0[DP];  // s0: BLOCK mode only
#pragma unroll
            for (int a = 0; a < DP; a++) {
                if (col && a < D) s[a] = Ops::sub(hp[a + c * D], sgc[a]);
                else s[a] = (a == c) ? Ops::one() : Ops::zero();
                if (a == c && col) s[a] = Ops::add(s[a], zc);
            }
            if (col) {
                for (int l = 0; l < m; l++) {
                    const C q = Ops::mulc(wl[l], bs[l * D + c]);     // w_l conj(b_l(c))
#pragma unroll
                    for (int a = 0; a < DP; a++)
                        if (a < D) s[a] = Ops::fms(bs[l * D + a], q, s[a]);
                }
            }
            if ((MODE & S_BLOCK) && !G0E && !RE) {
#pragma unroll
                for (int a = 0; a < DP; a++)
                    s0[a] = (col && a < D) ? Ops::sub(Ops::add(s[a], sgc[a]), sM0[a + c * D]) : s[a];
            }
            if (MODE & S_DERIV) {
                // S' = I + sum_l w_l^2 b_l b_l^H, column c, straight into the group's tile
                C sp[DP];
#pragma unroll
                for (int a = 0; a < DP; a++) sp[a] = (a == c && col) ? Ops::one() : Ops::zero();
                if (col)
                    for (int l = 0; l < m; l++) {
                        const C q = Ops::mulc(Ops::mul(wl[l], wl[l]), bs[l * D + c]);
#pragma unroll
                        for (int a = 0; a < DP; a++)
                            if (a < D) sp[a] = Ops::fma(bs[l * D + a], q, sp[a]);
                    }
                __syncwarp();
                if (active && c < DP) {
#pragma unroll
                    for (int a = 0; a < DP; a++) tS[a + c * DP] = sp[a];
                }
            }
            if constexpr (PACK) sing |= group_gj_inverse<Ops, DP>(s, c, base) && active;
            else sing |= gj_inverse<Ops, DP, W>(s, c);
            if (RE && (MODE & S_BLOCK)) {
#pragma unroll
                for (int a = 0; a < DP; a++) accG[a] = Ops::add(accG[a], s[a]);
            }
            if ((MODE & S_BLOCK) && !G0E && !RE) {
                if constexpr (PACK) sing |= group_gj_inverse<Ops, DP>(s0, c, base) && active;
                else sing |= gj_inverse<Ops, DP, W>(s0, c);
#pragma unroll
                for (int a = 0; a < DP; a++) {
                    accG[a] = Ops::add(accG[a], s[a]);
                    accG0[a] = Ops::add(accG0[a], s0[a]);
                }
            }
            if (G0E) {
                // G0(:, c) = sum_j U(:, j) r_j conj(U(c, j))
                const C *us = sU + (size_t)kk * g.n * D;
#pragma unroll
                for (int a = 0; a < DP; a++) accG[a] = Ops::add(accG[a], s[a]);
                if (col)
                    for (int j = 0; j < g.n; j++) {
                        const C q = Ops::mulc(rl[j], us[j * D + c]);
#pragma unroll
                        for (int a = 0; a < DP; a++)
                            if (a < D) accG0[a] = Ops::fma(us[j * D + a], q, accG0[a]);
                    }
            }
            if (MODE & S_TRACE) {
                // lane c: column c of G_PP in s.  acc1 -> Tr G - Tr G0, acc2 -> d/dz of it (summed over lanes)
                C acc1 = Ops::zero(), acc2 = Ops::zero();
#pragma unroll
                for (int a = 0; a < DP; a++)
                    if (a == c && col) acc1 = s[a];
                for (int l = c; l < m; l += W) {
                    acc1 = Ops::add(acc1, wl[l]);
                    if (MODE & S_DERIV) acc2 = Ops::sub(acc2, Ops::mul(wl[l], wl[l]));
                }
                if (!RE)
                    for (int j = c; j < g.n; j += W) {
                        acc1 = Ops::sub(acc1, rl[j]);
                        if (MODE & S_DERIV) acc2 = Ops::add(acc2, Ops::mul(rl[j], rl[j]));
                    }
                C y[DP];
                if (MODE & S_DERIV) {
                    // Y = G S' G, column c: u = S' G(:,c), y = G u
                    __syncwarp();
                    if (active && c < DP) {
#pragma unroll
                        for (int a = 0; a < DP; a++) tG[a + c * DP] = s[a];
                    }
                    __syncwarp();
                    C u[DP];
#pragma unroll
                    for (int a = 0; a < DP; a++) {
                        u[a] = Ops::zero();
#pragma unroll
                        for (int b = 0; b < DP; b++) u[a] = Ops::fma(tS[a + b * DP], s[b], u[a]);
                    }
#pragma unroll
                    for (int a = 0; a < DP; a++) {
                        C v = Ops::zero();
#pragma unroll
                        for (int b = 0; b < DP; b++) v = Ops::fma(tG[a + b * DP], u[b], v);
                        y[a] = v;
                    }
                    __syncwarp();
#pragma unroll
                    for (int a = 0; a < DP; a++)
                        if (a == c && col) acc2 = Ops::sub(acc2, y[a]);
                }
                if (col) {
                    for (int l = 0; l < m; l++) {
                        const C bc = bs[l * D + c];
                        C px = Ops::zero(), py = Ops::zero();
#pragma unroll
                        for (int a = 0; a < DP; a++)
                            if (a < D) {
                                px = Ops::add(px, Ops::mulc(s[a], bs[l * D + a]));
                                if (MODE & S_DERIV) py = Ops::add(py, Ops::mulc(y[a], bs[l * D + a]));
                            }
                        const C w2 = Ops::mul(wl[l], wl[l]);
                        acc1 = Ops::fma(w2, Ops::mul(px, bc), acc1);
                        if (MODE & S_DERIV) {
                            const C w3 = Ops::mul(w2, wl[l]);
                            acc2 = Ops::fms(Ops::add(w3, w3), Ops::mul(px, bc), acc2);
                            acc2 = Ops::fms(w2, Ops::mul(py, bc), acc2);
                        }
                    }
                }
                acct1 += group_sum<DP, W>(Ops::re(acc1), base);
                if (MODE & S_DERIV) acct2 += group_sum<DP, W>(Ops::re(acc2), base);
                if (RE) acct2 += group_sum<DP, W>(Ops::im(acc1), base);  // complex Tr G on the real axis
            }
        }
    }
    if (sing && fvalid) dg_flag(g.status, DG_SINGULAR);
    if (!fvalid) return;
    if (MODE & S_BLOCK) {
        if (col) {
            const size_t o = ((size_t)chunk * g.nf2 + f) * DD + (size_t)c * D;
#pragma unroll
            for (int a = 0; a < DP; a++)
                if (a < D) {
                    g.pblk[o + a] = Ops::to(accG[a]);
                    g.pblk0[o + a] = Ops::to(accG0[a]);
                }
        }
    }
    if ((MODE & S_TRACE) && c == 0) g.ptr[(size_t)chunk * g.nf2 + f] = cmk(acct1, acct2);
}

// In-place inverse of a D x D matrix held by one thread (D <= 3): Gauss-Jordan with partial pivoting whose row
// swaps are predicated moves between compile-time indices (no local memory), undone as column swaps at the end.
// Each step stores the pivot's reciprocal in place and updates only the other columns: row j becomes
// a_jc / a_jj, row r becomes a_rc - a_rj a_jc for c != j, and column j becomes -a_rj / a_jj (no products with the
// known 1 and 0 entries).
template <class Ops, int N>
DG_HD bool thread_inverse(typename Ops::C (&a)[N][N]) {
    typedef typename Ops::C C;
    typedef typename Ops::M M;
    bool sing = false;
    int perm[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        int p = j;
        M best = Ops::mag2(a[j][j]);
#pragma unroll
        for (int r = j + 1; r < N; r++) {
            const M v = Ops::mag2(a[r][j]);
            if (v > best) {
                best = v;
                p = r;
            }
        }
        perm[j] = p;
#pragma unroll
        for (int r = j + 1; r < N; r++) {
            const bool sw = (p == r);
#pragma unroll
            for (int c = 0; c < N; c++) {
                const C x = a[j][c], y = a[r][c];
                a[j][c] = sw ? y : x;
                a[r][c] = sw ? x : y;
            }
        }
        sing |= !(best > M(0));
        const C piv = Ops::rcp(a[j][j]);
        a[j][j] = piv;
#pragma unroll
        for (int c = 0; c < N; c++)
            if (c != j) a[j][c] = Ops::mul(a[j][c], piv);
#pragma unroll
        for (int r = 0; r < N; r++)
            if (r != j) {
                const C t = a[r][j];
#pragma unroll
                for (int c = 0; c < N; c++)
                    if (c != j) a[r][c] = Ops::fms(t, a[j][c], a[r][c]);
                a[r][j] = Ops::mul(Ops::neg(t), piv);
            }
    }
#pragma unroll
    for (int j = N - 1; j >= 0; j--)
#pragma unroll
        for (int c2 = j + 1; c2 < N; c2++) {
            const bool sw = (perm[j] == c2);
#pragma unroll
            for (int r = 0; r < N; r++) {
                const C x = a[r][j], y = a[r][c2];
                a[r][j] = sw ? y : x;
                a[r][c2] = sw ? x : y;
            }
        }
    return sing;
}

// BLOCK mode (G_loc and GwHF) for correlated blocks of D <= 3: one thread per Matsubara frequency, the whole
// D x D S(z) and S0(z) of that thread's (k, iw) in its registers, inverted by thread_inverse.  A lane-group
// k_schur at these widths leaves lanes idle (D < W) and spends its issue slots on the group's pivot broadcasts;
// here every lane does useful work and nothing is exchanged.  Per k point the CTA stages, for all its
// frequencies, the pole outer products P_l = b_l b_l^H (Hermitian: the real diagonal and the upper triangle), the
// shifted poles mu - e_l and -H_PP - m0; each thread forms S0 = z - H_PP - m0 - sum_l w_l P_l and
// S = S0 - (Sigma - m0), Sigma - m0 held in its registers.
//
// The pole sum in Hermitian parts: with w_l = 1/(z - e_l) = (x_l - i w)/(x_l^2 + w^2), x_l = mu - e_l,
// sum_l w_l P_l = A + i B with A = sum_l Re(w_l) P_l and B = sum_l Im(w_l) P_l both Hermitian, so only the
// diagonal (real) and the upper triangle of A and B are accumulated: 2 D + 4 D(D-1)/2 real multiply-adds per pole
// instead of 4 D^2, and the lower triangle follows as A_ba + i B_ba = conj(A_ab) + i conj(B_ab).
template <class Ops, int D>
__global__ void __launch_bounds__(128) k_schur_tpi(SchurArgs g) {
    typedef typename Ops::C C;
    typedef typename Ops::R R;
    extern __shared__ double2 sm[];
    constexpr int DD = D * D, NP = D * (D - 1) / 2;
    const int m = g.m;
    // staged per k: P_l off-diagonal pairs [m][NP] (C), -H_PP - m0 [DD] (C), P_l diagonal [m][D] (R), mu - e_l [m] (R)
    C *sPo = reinterpret_cast<C *>(sm);
    C *sH = sPo + (size_t)g.kc * m * NP;
    R *sPd = reinterpret_cast<R *>(sH + (size_t)g.kc * DD);
    R *sE = sPd + (size_t)g.kc * m * D;
    const int f_raw = blockIdx.x * blockDim.x + threadIdx.x;
    const bool fvalid = f_raw < g.nf2;
    const int f = fvalid ? f_raw : g.nf2 - 1;
    const int chunk = blockIdx.y;
    const int kbeg = chunk * g.kchunk, kend = min(g.nk, kbeg + g.kchunk);
    const double w = g.wgrid ? (DG_PI / g.beta + f * ((2 * DG_PI) / g.beta)) : (DG_PI * (2. * f + 1.) / g.beta);
    const C zc = Ops::from(cmk(g.mu, w));
    const R wr = Ops::rfrom(w), w2 = Ops::rmul(wr, wr);
    C sd[D][D], aG[D][D], aG0[D][D];  // sd = Sigma(iw) - m0
#pragma unroll
    for (int a = 0; a < D; a++)
#pragma unroll
        for (int b = 0; b < D; b++) {
            sd[a][b] = Ops::from(csub(g.sig[(size_t)f * DD + a + b * D], g.m0[a + b * D]));
            aG[a][b] = aG0[a][b] = Ops::zero();
        }
    bool sing = false;
    for (int k0 = kbeg; k0 < kend; k0 += g.kc) {
        const int nkc = min(g.kc, kend - k0);
        __syncthreads();
        for (int t = threadIdx.x; t < nkc * m * D; t += blockDim.x) {
            const double2 b = g.B[((size_t)k0 * m + t / D) * D + t % D];
            sPd[t] = Ops::rfrom(b.x * b.x + b.y * b.y);
        }
        if (NP > 0)
            for (int t = threadIdx.x; t < nkc * m * NP; t += blockDim.x) {
                int q = t % NP, a = 0;  // pair q in row-major order over the strict upper triangle
                while (q >= D - 1 - a) {
                    q -= D - 1 - a;
                    a++;
                }
                const double2 *bl = g.B + ((size_t)k0 * m + t / NP) * D;
                sPo[t] = Ops::from(cmulc(bl[a], bl[a + 1 + q]));
            }
        for (int t = threadIdx.x; t < nkc * m; t += blockDim.x) sE[t] = Ops::rfrom(g.mu - g.epsQ[(size_t)k0 * m + t]);
        for (int t = threadIdx.x; t < nkc * DD; t += blockDim.x) {
            const int kk = t / DD, e = t % DD, a = e % D, b = e / D;
            sH[t] = Ops::from(csub(cneg(g.H[(size_t)(k0 + kk) * g.n * g.n + a + (size_t)b * g.n]), g.m0[e]));
        }
        __syncthreads();
        for (int kk = 0; kk < nkc; kk++) {
            const C *po = sPo + (size_t)kk * m * NP, *hp = sH + (size_t)kk * DD;
            const R *pd = sPd + (size_t)kk * m * D, *es = sE + (size_t)kk * m;
            R Ad[D], Bd[D], Ar[NP ? NP : 1], Ai[NP ? NP : 1], Br[NP ? NP : 1], Bi[NP ? NP : 1];
#pragma unroll
            for (int a = 0; a < D; a++) Ad[a] = Bd[a] = Ops::rzero();
#pragma unroll
            for (int q = 0; q < NP; q++) Ar[q] = Ai[q] = Br[q] = Bi[q] = Ops::rzero();
            // the pole sums are lazy double-float sums, renormalised after every 16 poles and at the end
            auto renorm = [&]() {
#pragma unroll
                for (int a = 0; a < D; a++) {
                    Ad[a] = Ops::rnorm(Ad[a]);
                    Bd[a] = Ops::rnorm(Bd[a]);
                }
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    Ar[q] = Ops::rnorm(Ar[q]);
                    Ai[q] = Ops::rnorm(Ai[q]);
                    Br[q] = Ops::rnorm(Br[q]);
                    Bi[q] = Ops::rnorm(Bi[q]);
                }
            };
            for (int l = 0; l < m; l++) {
                if (l > 0 && (l & 15) == 0) renorm();
                const R x = es[l];
                const R r = Ops::rrcp(Ops::rfma(x, x, w2));
                const R re = Ops::rmul(x, r), im = Ops::rneg(Ops::rmul(wr, r));  // w_l
#pragma unroll
                for (int a = 0; a < D; a++) {
                    const R p = pd[(size_t)l * D + a];
                    Ad[a] = Ops::racc(re, p, Ad[a]);
                    Bd[a] = Ops::racc(im, p, Bd[a]);
                }
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    const C p = po[(size_t)l * NP + q];
                    Ar[q] = Ops::racc(re, Ops::cre(p), Ar[q]);
                    Ai[q] = Ops::racc(re, Ops::cim(p), Ai[q]);
                    Br[q] = Ops::racc(im, Ops::cre(p), Br[q]);
                    Bi[q] = Ops::racc(im, Ops::cim(p), Bi[q]);
                }
            }
            renorm();
            C s0[D][D];
#pragma unroll
            for (int a = 0; a < D; a++) {
                const C h = Ops::add(hp[a + a * D], zc);
                s0[a][a] = Ops::sub(h, Ops::mk(Ad[a], Bd[a]));
            }
            {
                int q = 0;
#pragma unroll
                for (int a = 0; a < D; a++)
#pragma unroll
                    for (int b = a + 1; b < D; b++, q++) {
                        // S_ab = (Ar - Bi) + i (Ai + Br), S_ba = (Ar + Bi) + i (Br - Ai)
                        s0[a][b] = Ops::sub(hp[a + b * D], Ops::mk(Ops::rsub(Ar[q], Bi[q]), Ops::radd(Ai[q], Br[q])));
                        s0[b][a] = Ops::sub(hp[b + a * D], Ops::mk(Ops::radd(Ar[q], Bi[q]), Ops::rsub(Br[q], Ai[q])));
                    }
            }
            C s[D][D];
#pragma unroll
            for (int a = 0; a < D; a++)
#pragma unroll
                for (int b = 0; b < D; b++) s[a][b] = Ops::sub(s0[a][b], sd[a][b]);
            sing |= thread_inverse<Ops, D>(s);
            sing |= thread_inverse<Ops, D>(s0);
#pragma unroll
            for (int a = 0; a < D; a++)
#pragma unroll
                for (int b = 0; b < D; b++) {
                    aG[a][b] = Ops::add(aG[a][b], s[a][b]);
                    aG0[a][b] = Ops::add(aG0[a][b], s0[a][b]);
                }
        }
    }
    if (sing && fvalid) dg_flag(g.status, DG_SINGULAR);
    if (!fvalid) return;
    const size_t o = ((size_t)chunk * g.nf2 + f) * DD;
#pragma unroll
    for (int a = 0; a < D; a++)
#pragma unroll
        for (int b = 0; b < D; b++) {
            g.pblk[o + a + b * D] = Ops::to(aG[a][b]);
            g.pblk0[o + a + b * D] = Ops::to(aG0[a][b]);
        }
}

// staged per k: P_l off-diagonal pairs [m][D(D-1)/2] and -H_PP - m0 [D][D] (16 B complex), P_l diagonal [m][D] and
// mu - e_l [m] (8 B real; double and double-float alike)
inline size_t schur_tpi_smem(int kc, int D, int m) {
    return ((size_t)kc * m * (D * (D - 1) / 2) + (size_t)kc * D * D) * 16 + ((size_t)kc * m * D + (size_t)kc * m) * 8;
}

// shared-memory bytes of one k_schur launch
inline size_t schur_smem(int DP, int W, int mode, int kc, int D, int m, int n) {
    const int NG = schur_groups(W);
    size_t s = (size_t)kc * m * D + (size_t)kc * m + (size_t)kc * D * D + (size_t)D * D + (size_t)NG * m;
    const bool g0e = (mode & S_BLOCK) && DP >= 8 && !(mode & S_REAL);
    if (((mode & S_TRACE) && !(mode & S_REAL)) || g0e) s += (size_t)kc * n + (size_t)NG * n;
    if (g0e) s += (size_t)kc * n * D;
    if (mode & S_DERIV) s += (size_t)NG * 2 * DP * DP;
    return s * 16;
}

typedef void (*SchurKernel)(SchurArgs);

template <class Ops, int DP, int W>
SchurKernel schur_pick_ops(int mode) {
    switch (mode) {
        case S_BLOCK: return k_schur<Ops, DP, W, S_BLOCK>;
        case S_TRACE: return k_schur<Ops, DP, W, S_TRACE>;
        case S_TRACE | S_DERIV: return k_schur<Ops, DP, W, S_TRACE | S_DERIV>;
        case S_BLOCK | S_TRACE | S_REAL: return k_schur<Ops, DP, W, S_BLOCK | S_TRACE | S_REAL>;
        default: return nullptr;
    }
}
// mixed = true selects the double-float arithmetic
template <int DP, int W>
SchurKernel schur_pick(int mode, bool mixed) {
    return mixed ? schur_pick_ops<OpsF, DP, W>(mode) : schur_pick_ops<OpsD, DP, W>(mode);
}

// the thread-per-frequency BLOCK kernels, D = 1 .. 3 (schur_tpi.cu)
SchurKernel schur_tpi_kernel(int D, bool mixed);

#define DG_SCHUR_INST(DP, W) \
    SchurKernel schur_kernel_##DP(int mode, bool mixed) { return schur_pick<DP, W>(mode, mixed); }
#define DG_SCHUR_DECL(DP) SchurKernel schur_kernel_##DP(int mode, bool mixed);
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
