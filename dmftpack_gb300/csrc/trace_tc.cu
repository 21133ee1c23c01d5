// trace_tc.cu -- the N(mu) lattice pass of the mu search (GiwToNele's occupation sum, src/GreenFtn.cpp:513-635,
// in the trace form) with the pole sums on the tensor cores, for correlated blocks of 4 .. 10 orbitals in the
// double-float (DMFTGPU_MIXED) arithmetic.
//
// Per (k, iw_f), with w_l = 1/(z - e_l), P_l = b_l b_l^H and M = z - H_PP - Sigma(iw_f) - S (schur.cuh):
//     S = sum_l w_l P_l,   R = sum_l w_l^2 P_l,   Tr G = Tr[M^-1 (I + R)] + sum_l w_l      (I + R = dM/dz)
// and the pass sums Re[Tr G - Tr G0] over k, Tr G0 = sum_j 1/(z - e0_j).  S and R are sums of a complex weight
// times Hermitian matrices: S = A + iB with A = sum_l Re(w_l) P_l and B = sum_l Im(w_l) P_l both Hermitian, so
// each is a real GEMM over the D^2 real degrees of freedom ("dofs") of the P_l: diagonal |b_a|^2, then Re and Im
// of b_a conj(b_c) for a < c.  For one k and a tile of 32 frequencies the GEMM has 128 rows (4 channels Re w,
// Im w, Re w^2, Im w^2 x 32 frequencies, channel-major), K = the m poles (padded to 32) and N = the dofs
// (padded to a multiple of 16): 128 x NP x 32 per k, on tcgen05 with the accumulators in TMEM.
//
// FP64-level accuracy from bf16: each row is scaled by a power of two to |x| <= 1 and split into 5 slices
// x = sum_s v_s 2^{-8s} (v_s integers, |v_1| <= 256, |v_s| <= 128 after), each stored pre-weighted
// (v_s 2^{-8s}, exact in bf16); the dof columns likewise (per k and column).  Products of slices (i, j) carry
// their true weight 2^{-8(i+j)}.  Levels i + j = 2, 3 and 4 (one, two and three products) accumulate exactly in
// their own FP32 accumulators (sums of at most 32 poles stay below 2^22 in their units); the 9 products of levels
// >= 5 share a fourth one, whose values are below 2^-23 of the row x column scale, so its FP32 rounding adds
// ~2^-42 of it.  (Merging level 4 as well would leave ~5e-10 of it: level 4 reaches 2^-16 of the scale.)  The
// residual of 5 slices is 2^-41.  Four accumulators x NP columns stay within TMEM's 512.
//
// The D x D inversion of M and the trace run on the FP32 pipe in double-float, one frequency per group of DP
// lanes (32/DP groups per warp, group_gj_inverse), after the drain has assembled S and R from the dofs.
#include <algorithm>

#include <cuda_bf16.h>

#include "df.cuh"
#include "internal.h"
#include "linalg.cuh"
#include "tc.cuh"
#include "trace_tc.h"

namespace {

constexpr int FT = 32;        // Matsubara frequencies per CTA
constexpr int ROWS = 4 * FT;  // MMA M = 128: row = channel * FT + frequency
constexpr int KP = 32;        // poles per k, padded: the GEMM's K (m <= 32)
constexpr int KSTEPS = KP / 16;
constexpr int NS = 5;         // slices per operand
constexpr int NE0 = 64;       // static-spectrum entries staged per k (n <= 64)
constexpr uint32_t WAIT_LIMIT = 1u << 22;

__host__ __device__ constexpr int np_of(int DP) { return ((DP * DP + 15) / 16) * 16; }
__host__ __device__ constexpr int pow2_at_least(int x) { return x <= 32 ? 32 : (x <= 64 ? 64 : (x <= 128 ? 128 : (x <= 256 ? 256 : 512))); }

// element offset in an operand image of R rows x KP: [slice][k step][row group][k group][8 rows][8 elements]
// (the canonical no-swizzle K-major layout of tc.cuh: LBO 128 B, SBO 256 B)
__host__ __device__ __forceinline__ int img_off(int R, int s, int kk, int r) {
    const int q = kk >> 4, k16 = kk & 15;
    return s * KSTEPS * R * 16 + q * R * 16 + (r >> 3) * 128 + (k16 >> 3) * 64 + (r & 7) * 8 + (k16 & 7);
}

// index of the pair (a, c), a < c, in row-major order over the strict upper triangle of a D x D matrix
__host__ __device__ __forceinline__ int pair_index(int a, int c, int D) { return a * D - a * (a + 1) / 2 + (c - a - 1); }

template <int DP>
struct TT {
    static constexpr int NP = np_of(DP);                 // MMA N: dofs padded to a multiple of 16
    static constexpr int NDOF = DP * DP;
    static constexpr int NDS = NDOF | 1;                 // dof stride per (channel, frequency): odd in 8-byte words,
                                                          // so 16 lanes' float2 accesses at this stride hit distinct banks
    static constexpr int GPW = 32 / DP;                  // frequency groups per warp
    static constexpr int NGW = (FT + GPW - 1) / GPW;     // inversion warps (the first 4 also drain TMEM)
    static constexpr int NW = (NGW > 4 ? NGW : 4) + 1;   // + the warp that issues the copies and the MMAs
    static constexpr int NT = NW * 32;
    static constexpr int A_EL = NS * KSTEPS * ROWS * 16;
    static constexpr int B_EL = NS * KSTEPS * NP * 16;
    static constexpr int NACC = 4;                       // TMEM accumulators: levels 2, 3, 4 exact, >= 5 merged
    static constexpr int TMEM = pow2_at_least(NACC * NP);
    // shared memory layout (bytes)
    static constexpr int O_A = 0;
    static constexpr int O_B = O_A + A_EL * 2;
    static constexpr int O_COL = O_B + B_EL * 2;                       // NP floats: dof column scales of k
    static constexpr int O_DOF = O_COL + NP * 4;                       // [4][FT][NDS] float2 (double-float)
    static constexpr int DOF_BYTES = 4 * FT * (NDS > KP ? NDS : KP) * 8;   // also the A build's [4][FT][KP]
    static constexpr int O_ROW = O_DOF + DOF_BYTES;                    // ROWS floats: row scales
    static constexpr int O_SUMW = O_ROW + ROWS * 4;                    // FT cdf: sum_l w_l
    static constexpr int O_H = O_SUMW + FT * 16;                       // DP x DP cdf: H_PP(a, c) at a + c DP
    static constexpr int O_E0 = O_H + DP * DP * 16;                    // NE0 float2: mu - e0_j
    static constexpr int O_EQ = O_E0 + NE0 * 8;                        // KP float2: mu - e_l
    static constexpr int O_WF = O_EQ + KP * 8;                         // FT float2: the CTA's Matsubara frequencies
    static constexpr int O_BAR = (O_WF + FT * 8 + 15) / 16 * 16;       // 2 mbarriers + the TMEM slot
    static constexpr int SMEM = O_BAR + 32;
    static_assert(NACC * NP <= 512, "accumulators exceed TMEM");
    static_assert(NP <= 256 && NP % 16 == 0, "MMA N");
    static_assert(O_B % 16 == 0 && O_COL % 16 == 0 && O_BAR % 16 == 0, "alignment");
};

// the dofs of P_l = b_l b_l^H (FP64): p < D: |b_p|^2; then for each pair (a < c): Re, Im of b_a conj(b_c)
__device__ __forceinline__ double pole_dof(const double2 *b, int p, int D) {
    if (p < D) return b[p].x * b[p].x + b[p].y * b[p].y;
    const int q = p - D, idx = q >> 1;
    if (idx >= D * (D - 1) / 2) return 0.0;
    int a = 0, rem = idx;
    while (rem >= D - 1 - a) {
        rem -= D - 1 - a;
        a++;
    }
    const int c = a + 1 + rem;
    const double2 v = cmulc(b[a], b[c]);
    return (q & 1) ? v.y : v.x;
}

// x in [-1, 1] -> NS pre-weighted bf16 slices v_s 2^{-8s} (exact FP64 steps)
__device__ __forceinline__ void slice_pw(double x, __nv_bfloat16 *out, int stride) {
    double wgt = 1.0 / 256.0;
#pragma unroll
    for (int s = 0; s < NS; s++) {
        x *= 256.0;
        const double v = rint(x);
        out[s * stride] = __float2bfloat16_rn((float)(v * wgt));
        x -= v;
        wgt *= 1.0 / 256.0;
    }
}

// per k: the B operand image (dofs of the m poles, sliced per dof column) and the column scales; built once per
// prepared lattice and reused by every N(mu) evaluation of the mu search
template <int DP>
__global__ void k_trace_tc_prep(int nk, int m, int D, const double2 *__restrict__ B, __nv_bfloat16 *__restrict__ img,
                                float *__restrict__ colscale) {
    using T = TT<DP>;
    const long long total = (long long)nk * T::NP;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t / T::NP), p = (int)(t % T::NP);
        __nv_bfloat16 *base = img + (size_t)k * T::B_EL;
        double mx = 0.0;
        if (p < D * D)
            for (int l = 0; l < m; l++) mx = fmax(mx, fabs(pole_dof(B + ((size_t)k * m + l) * D, p, D)));
        int ex = 0;
        frexp(mx, &ex);
        const double g = (mx > 0.0) ? ldexp(1.0, ex) : 1.0;
        colscale[(size_t)k * T::NP + p] = (float)g;
        for (int l = 0; l < KP; l++) {
            const double v = (p < D * D && l < m) ? pole_dof(B + ((size_t)k * m + l) * D, p, D) / g : 0.0;
            slice_pw(v, base + img_off(T::NP, 0, l, p), KSTEPS * T::NP * 16);
        }
    }
}

__device__ __forceinline__ dfl dfl_of(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ float2 f2_of(dfl v) { return make_float2(v.h, v.l); }

// Hermitian matrix entry (a, c) from one (channel, frequency) dof vector
__device__ __forceinline__ cdf herm_entry(const float2 *d, int a, int c, int D) {
    if (a == c) return {dfl_of(d[a]), {0.f, 0.f}};
    if (a < c) {
        const int i = D + 2 * pair_index(a, c, D);
        return {dfl_of(d[i]), dfl_of(d[i + 1])};
    }
    const int i = D + 2 * pair_index(c, a, D);
    return {dfl_of(d[i]), df_neg(dfl_of(d[i + 1]))};
}

// fixed-order sum over the k chunks: tr[f] = sum_q ptr[q][f].x
__global__ void k_trace_tc_reduce(int nchunk, int nf2, const double2 *__restrict__ ptr, double *__restrict__ tr) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf2) return;
    double s = 0.0;
    for (int q = 0; q < nchunk; q++) s += ptr[(size_t)q * nf2 + f].x;
    tr[f] = s;
}

}  // namespace

namespace {

struct TcKArgs {
    TraceTcArgs a;
    const __nv_bfloat16 *Bimg;  // [nk][B_EL]
    const float *colscale;      // [nk][NP]
    int kchunk;
    double2 *ptr;               // [nchunk][nf2]: x = sum over the chunk's k of Re[Tr G - Tr G0]
    int *status;
};

// CTA = 32 Matsubara frequencies x one chunk of k points.  Per k: stage H_PP, e_l, e0_j; build the A image
// (w_l and w_l^2 of the 32 frequencies, sliced per row); one thread issues the bulk copy of the k's B image and the
// 30 MMAs; warps 0-3 drain the four accumulators into the dofs of S and R (warp = channel, lane = frequency);
// every inversion warp forms M column by column, inverts it and adds Re[Tr M^-1 (I + R) + sum w - sum r0].
template <int DP>
__global__ void __launch_bounds__(TT<DP>::NT, 1) k_trace_tc(TcKArgs g) {
    using T = TT<DP>;
    typedef OpsF Ops;
    extern __shared__ __align__(1024) unsigned char sm[];
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(sm + T::O_A);
    __nv_bfloat16 *sB = reinterpret_cast<__nv_bfloat16 *>(sm + T::O_B);
    float *sCol = reinterpret_cast<float *>(sm + T::O_COL);
    float2 *dofs = reinterpret_cast<float2 *>(sm + T::O_DOF);   // [4][FT][NDS]
    float2 *vals = dofs;                                          // [4][FT][KP] during the A build (aliased)
    float *rowsc = reinterpret_cast<float *>(sm + T::O_ROW);
    cdf *sumw = reinterpret_cast<cdf *>(sm + T::O_SUMW);
    cdf *hH = reinterpret_cast<cdf *>(sm + T::O_H);
    float2 *sE0 = reinterpret_cast<float2 *>(sm + T::O_E0);
    float2 *sEq = reinterpret_cast<float2 *>(sm + T::O_EQ);
    float2 *sWf = reinterpret_cast<float2 *>(sm + T::O_WF);
    uint64_t *barB = reinterpret_cast<uint64_t *>(sm + T::O_BAR), *barM = barB + 1;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(barB + 2);
    const TraceTcArgs &a = g.a;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int issuer = (T::NW - 1) * 32;
    const int D = a.D, m = a.m, n = a.n;
    const int chunk = blockIdx.y;
    const int kbeg = chunk * g.kchunk, kend = min(a.nk, kbeg + g.kchunk);
    const int f0 = blockIdx.x * FT;
    if (warp == 0) {
        tc::tmem_alloc(tslot, T::TMEM);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(barB, 1);
        tc::mbar_init(barM, 1);
    }
    if (tid < FT) {
        // the tile's frequencies once, as double-float (the same FP64 expression as the lane-group kernels)
        const int ff = min(blockIdx.x * FT + tid, a.nf2 - 1);
        const double wv = a.wgrid ? (DG_PI / a.beta + ff * ((2 * DG_PI) / a.beta)) : (DG_PI * (2. * ff + 1.) / a.beta);
        sWf[tid] = f2_of(df_make(wv));
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;

    // frequency group of this lane (inversion warps): lanes base .. base+DP-1 of the warp, column c
    const int gw = lane / DP, c = lane % DP, base = gw * DP;
    const int gidx = warp * T::GPW + gw;
    const bool grp_lane = warp < T::NGW && gw < T::GPW && gidx < FT;
    const int fl = grp_lane ? gidx : FT - 1;
    const int f = f0 + fl;
    const bool fvalid = grp_lane && f < a.nf2;
    const int fc = min(f, a.nf2 - 1);
    auto wfreq = [&](int ff) {
        return a.wgrid ? (DG_PI / a.beta + ff * ((2 * DG_PI) / a.beta)) : (DG_PI * (2. * ff + 1.) / a.beta);
    };
    const double wf = wfreq(fc);
    const cdf zc = Ops::from(cmk(a.mu, wf)), iwc = Ops::from(cmk(0.0, wf));
    const size_t DD = (size_t)D * D;
    cdf sgc[DP];  // column c of Sigma(iw_f)
#pragma unroll
    for (int r = 0; r < DP; r++)
        sgc[r] = (r < D && c < D) ? Ops::from(a.sig[(size_t)fc * DD + r + (size_t)c * D]) : Ops::zero();
    double acc = 0.0;
    bool sing = false, ok = true;
    int it = 0;
    constexpr uint32_t IDESC = tc::idesc_bf16_f32(ROWS, T::NP);

    for (int k = kbeg; k < kend; k++, it++) {
        // 1. the k's B image and column scales, by the bulk-copy engine (the previous k's MMAs are complete)
        if (tid == issuer) {
            tc::mbar_arrive_expect_tx(barB, (uint32_t)(T::B_EL * 2 + T::NP * 4));
            tc::bulk_g2s(sB, g.Bimg + (size_t)k * T::B_EL, (uint32_t)(T::B_EL * 2), barB);
            tc::bulk_g2s(sCol, g.colscale + (size_t)k * T::NP, (uint32_t)(T::NP * 4), barB);
        }
        // 2. per-k scalars
        for (int t = tid; t < D * D; t += T::NT) {
            const int r = t % D, cc = t / D;
            hH[r + cc * DP] = Ops::from(a.H[(size_t)k * n * n + r + (size_t)cc * n]);
        }
        for (int t = tid; t < n; t += T::NT) sE0[t] = f2_of(df_make(a.mu - a.eps0[(size_t)k * n + t]));
        for (int t = tid; t < KP; t += T::NT)
            sEq[t] = t < m ? f2_of(df_make(a.mu - a.epsQ[(size_t)k * m + t])) : make_float2(0.f, 0.f);
        __syncthreads();
        // 3. A build: w_l and w_l^2 of the tile's frequencies, row scales, slices
        for (int t = tid; t < FT * KP; t += T::NT) {
            const int ff = t / KP, l = t % KP;
            cdf w = Ops::zero(), w2 = Ops::zero();
            if (l < m) {
                const cdf x = {dfl_of(sEq[l]), dfl_of(sWf[ff])};
                w = Ops::rcp(x);
                w2 = Ops::mul(w, w);
            }
            vals[(0 * FT + ff) * KP + l] = f2_of(w.re);
            vals[(1 * FT + ff) * KP + l] = f2_of(w.im);
            vals[(2 * FT + ff) * KP + l] = f2_of(w2.re);
            vals[(3 * FT + ff) * KP + l] = f2_of(w2.im);
        }
        __syncthreads();
        // row scales and sum_l w_l, one row per warp at a time with the lanes across the poles (KP = 32 = a warp):
        // consecutive lanes read consecutive values, and the reductions are shuffles
        for (int row = warp; row < ROWS + FT; row += T::NW) {
            if (row < ROWS) {
                float mx = (lane < m) ? fabsf(vals[row * KP + lane].x) : 0.f;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                if (lane == 0) {
                    int ex = 0;
                    frexpf(mx, &ex);
                    rowsc[row] = (mx > 0.f) ? ldexpf(1.f, ex) : 1.f;
                }
            } else {
                const int ff = row - ROWS;
                cdf sw = (lane < m) ? cdf{dfl_of(vals[ff * KP + lane]), dfl_of(vals[(FT + ff) * KP + lane])} : Ops::zero();
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sw = Ops::add(sw, Ops::shfl(sw, lane ^ o, 32));
                if (lane == 0) sumw[ff] = sw;
            }
        }
        __syncthreads();
        for (int t = tid; t < ROWS * KP; t += T::NT) {
            const int row = t / KP, l = t % KP;
            const float inv = 1.f / rowsc[row];  // a power of two: exact
            dfl u = {vals[row * KP + l].x * inv, vals[row * KP + l].y * inv};
            float wgt = 1.f / 256.f;
#pragma unroll
            for (int s = 0; s < NS; s++) {
                const float uh = u.h * 256.f, ul = u.l * 256.f;
                const float v = rintf(uh);
                u = two_sum(__fsub_rn(uh, v), ul);
                sA[img_off(ROWS, s, l, row)] = __float2bfloat16_rn(v * wgt);
                wgt *= 1.f / 256.f;
            }
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        // 4. MMAs: accumulators 0, 1, 2 <- levels 2, 3, 4; accumulator 3 <- levels >= 5
        if (tid == issuer) {
            if (tc::mbar_wait(barB, it & 1, WAIT_LIMIT)) {
                tc::fence_after_sync();
                const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
                int started = 0;
#pragma unroll 1
                for (int q = 0; q < KSTEPS; q++)
#pragma unroll 1
                    for (int i = 0; i < NS; i++)
#pragma unroll 1
                        for (int j = 0; j < NS - i; j++) {
                            const int L = min(i + j, 3);
                            const uint64_t ad = tc::smem_desc(a0 + (uint32_t)((i * KSTEPS + q) * ROWS * 16 * 2), 128, 256);
                            const uint64_t bd = tc::smem_desc(b0 + (uint32_t)((j * KSTEPS + q) * T::NP * 16 * 2), 128, 256);
                            tc::mma_bf16(tbase + (uint32_t)(L * T::NP), ad, bd, IDESC, (started >> L) & 1);
                            started |= 1 << L;
                        }
                tc::mma_commit(barM);
            }
        }
        ok = __syncthreads_and(tc::mbar_wait(barM, it & 1, WAIT_LIMIT)) != 0;
        if (!ok) break;
        tc::fence_after_sync();
        // 5. drain: TMEM lane quarter = channel (warp % 4), lane = frequency; the warps sharing a quarter split its
        // column groups.  dof p = a0 + a1 + a2 + a3, scaled back by the row and column scales
        if (warp < 4 * (T::NW / 4)) {
            const int ch = warp & 3, part = warp >> 2, nparts = T::NW / 4;
            const float rs = rowsc[ch * FT + lane];
            float2 *dst = dofs + (size_t)(ch * FT + lane) * T::NDS;
            const uint32_t la = tbase + ((uint32_t)(ch * 32) << 16);
#pragma unroll 1
            for (int qg = part; qg < T::NP / 16; qg += nparts) {
                float v0[16], v1[16], v2[16], v3[16];
                tc::tmem_ld16(la + (uint32_t)(0 * T::NP + qg * 16), v0);
                tc::tmem_ld16(la + (uint32_t)(1 * T::NP + qg * 16), v1);
                tc::tmem_ld16(la + (uint32_t)(2 * T::NP + qg * 16), v2);
                tc::tmem_ld16(la + (uint32_t)(3 * T::NP + qg * 16), v3);
#pragma unroll
                for (int cc = 0; cc < 16; cc++) {
                    const int p = qg * 16 + cc;
                    if (p < D * D) {
                        dfl s = two_sum(v0[cc], v1[cc]);
                        s = df_add(s, {v2[cc], 0.f});
                        s = df_add(s, {v3[cc], 0.f});
                        const float sc = rs * sCol[p];
                        dst[p] = make_float2(s.h * sc, s.l * sc);
                    }
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        // 6. inversion and trace (inversion warps; lanes outside a group compute unused values)
        if (warp < T::NGW) {
            const float2 *d0 = dofs + (size_t)(0 * FT + fl) * T::NDS, *d1 = dofs + (size_t)(1 * FT + fl) * T::NDS;
            const float2 *d2 = dofs + (size_t)(2 * FT + fl) * T::NDS, *d3 = dofs + (size_t)(3 * FT + fl) * T::NDS;
            cdf col[DP];
#pragma unroll
            for (int r = 0; r < DP; r++) {
                if (r < D && c < D) {
                    const cdf hA = herm_entry(d0, r, c, D), hB = herm_entry(d1, r, c, D);
                    const cdf Srv = {df_sub(hA.re, hB.im), df_add(hA.im, hB.re)};  // S = A + iB
                    cdf x = Ops::sub(Ops::neg(hH[r + c * DP]), Ops::add(sgc[r], Srv));
                    if (r == c) x = Ops::add(x, zc);
                    col[r] = x;
                } else {
                    col[r] = (r == c) ? Ops::one() : Ops::zero();
                }
            }
            sing |= group_gj_inverse<Ops, DP>(col, c, base) && fvalid && c < D;
            cdf t = Ops::zero();
            if (c < D) {
#pragma unroll
                for (int r = 0; r < DP; r++)
                    if (r < D) {
                        // (I + R)(c, r), R = A_R + i B_R from channels 2 and 3
                        const cdf hA = herm_entry(d2, c, r, D), hB = herm_entry(d3, c, r, D);
                        cdf x = {df_sub(hA.re, hB.im), df_add(hA.im, hB.re)};
                        if (r == c) x = Ops::add(x, Ops::one());
                        t = Ops::fma(col[r], x, t);
                    }
            }
            for (int j = c; j < n; j += DP) t = Ops::sub(t, Ops::rcp(Ops::add(cdf{dfl_of(sE0[j]), {0.f, 0.f}}, iwc)));
            if (c == 0) t = Ops::add(t, sumw[fl]);
            if (fvalid) acc += df_val(t.re);
        }
        __syncthreads();  // the dofs (and the A build's values aliased on them) are rewritten by the next k
    }
    // group sum over the DP lanes of each frequency (full-warp shuffles from absolute lanes)
    if (warp < T::NGW) {
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < DP; j++) s += __shfl_sync(0xffffffffu, acc, (base + j) & 31, 32);
        if (ok && fvalid && c == 0) g.ptr[(size_t)chunk * a.nf2 + f] = cmk(s, 0.0);
        if (sing) dg_flag(g.status, DG_SINGULAR);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !ok) atomicMax(g.status, (int)DMFTGPU_TIMEOUT);
    if (warp == 0) tc::tmem_dealloc(tbase, T::TMEM);
}

template <int DP>
int launch_trace_tc(dmftgpu_ctx *ctx, const TraceTcArgs &a, bool *ready, double *tr) {
    using T = TT<DP>;
    __nv_bfloat16 *Bimg = (__nv_bfloat16 *)dg_buf(ctx, "trace_tc.B", (size_t)a.nk * T::B_EL * 2);
    float *col = (float *)dg_buf(ctx, "trace_tc.col", (size_t)a.nk * T::NP * 4);
    if (!Bimg || !col) return DMFTGPU_NOMEM;
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    if (!*ready) {
        k_trace_tc_prep<DP><<<nsm * 4, 256, 0, ctx->stream>>>(a.nk, a.m, a.D, a.B, Bimg, col);
        DG_LAUNCH(ctx, "k_trace_tc_prep");
        *ready = true;
    }
    DG_CUDA(cudaFuncSetAttribute(k_trace_tc<DP>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM));
    int per_sm = 1;
    DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_tc<DP>, T::NT, T::SMEM));
    per_sm = std::max(1, per_sm);
    const int fblocks = dg_ceil_div(a.nf2, FT);
    // k chunks: about 8 waves of CTAs over the SMs, at least 16 k points per chunk
    int nchunk = std::max(1, std::min(dg_ceil_div(a.nk, 16), dg_ceil_div(8LL * nsm * per_sm, fblocks)));
    const int kchunk = dg_ceil_div(a.nk, nchunk);
    nchunk = dg_ceil_div(a.nk, kchunk);
    double2 *ptr = (double2 *)dg_buf(ctx, "trace_tc.ptr", (size_t)nchunk * a.nf2 * sizeof(double2));
    if (!ptr) return DMFTGPU_NOMEM;
    TcKArgs g;
    g.a = a;
    g.Bimg = Bimg;
    g.colscale = col;
    g.kchunk = kchunk;
    g.ptr = ptr;
    g.status = ctx->d_status;
    {
        DgTimer tm(ctx, "k_trace_tc");
        k_trace_tc<DP><<<dim3(fblocks, nchunk), T::NT, T::SMEM, ctx->stream>>>(g);
    }
    DG_LAUNCH(ctx, "k_trace_tc");
    k_trace_tc_reduce<<<dg_ceil_div(a.nf2, 256), 256, 0, ctx->stream>>>(nchunk, a.nf2, ptr, tr);
    DG_LAUNCH(ctx, "k_trace_tc_reduce");
    return DMFTGPU_OK;
}

}  // namespace

bool dg_trace_tc_supported(int n, int D) { return D >= 4 && D <= 10 && n - D <= KP && n <= NE0; }

int dg_trace_tc(dmftgpu_ctx *ctx, const TraceTcArgs &a, bool *ready, double *tr) {
    if (!dg_trace_tc_supported(a.n, a.D)) return dg_fail(ctx, DMFTGPU_BADARG, "trace_tc: unsupported sizes");
    if (a.D <= 4) return launch_trace_tc<4>(ctx, a, ready, tr);
    if (a.D <= 6) return launch_trace_tc<6>(ctx, a, ready, tr);
    if (a.D <= 8) return launch_trace_tc<8>(ctx, a, ready, tr);
    return launch_trace_tc<10>(ctx, a, ready, tr);
}
