// hk_tc.cu -- H(k) = sum_R T(R) e^{-i k.a R} (src/ConstructModelHamiltonian.cpp:66-77) as a tensor-core GEMM.
//
// Real form: H[k][c] = sum_q A[k][q] B[c][q] with q = 2r + {0: cos, 1: sin} over the N_R lattice vectors,
// A[k][2r] = cos(k.aR_r), A[k][2r+1] = sin(k.aR_r) and, for the output column c = 2e + {0: Re, 1: Im} of the
// column-major element e = i + j n,
//   B[2e][2r] = Re T_r(e),  B[2e][2r+1] = Im T_r(e),  B[2e+1][2r] = Im T_r(e),  B[2e+1][2r+1] = -Re T_r(e)
// (H = sum_r T_r (cos - i sin)).
//
// FP64 accuracy from bf16 tensor cores (exact slicing): every A entry (|a| <= 1) and every B entry divided by its
// column's power-of-two scale g_c is split into S = 5 integer slices, x = sum_s x_s 2^{-8s}, x_1 in [-256, 256]
// and x_s in [-128, 128] for s > 1 (each an integer, exact in bf16), leaving |x - sum| <= 2^-41.  A product of
// slices (i, j) is an exact integer of at most 16 bits with weight 2^{-8(i+j)}; the products of one "level"
// L = i + j (L <= S + 1 = 6: 15 products) accumulate in their own FP32 TMEM accumulator.  Per K index a level
// adds at most 2^16 (L = 2, 3), 1.25 x 2^16 (L = 4), 1.5 x 2^16 (L = 5) or 1.75 x 2^16 (L = 6), so over K = 128
// (two chunks of 64) every partial sum stays below 2^24 and each accumulator holds an exact integer.  Every two
// chunks the five accumulators are drained into double-float registers with their weights (exact power-of-two
// scalings); the result carries ~2^-41 of the operands' magnitude, well inside the 1e-10 relative bar of the
// plain FP64 form.
//
// Work per launch: 15 x 2 x N_k x 2n^2 x 2N_R bf16 flops; HBM: the N_k n^2 complex H(k) written once (the
// phase-slice image is built once per (k mesh, R list) and kept in the context's workspace).
#include <cmath>
#include <cstring>
#include <cuda_bf16.h>

#include "internal.h"
#include "linalg.cuh"
#include "tc.cuh"

namespace {

constexpr int TM = 128;       // k points per tile (TMEM lanes, MMA M)
constexpr int TN = 48;        // real output columns per tile (MMA N)
constexpr int KC = 64;        // K per chunk: 4 MMA steps of 16
constexpr int NS = 5;         // slices per operand
constexpr int NL = NS;        // levels L = 2 .. NS+1
constexpr int TMEM_COLS_PIPE = 512;  // two accumulator sets of NL * TN = 240 columns, a power of two
constexpr uint32_t WAIT_LIMIT = 1u << 22;

// element offset in the smem image of one operand chunk: [slice][k step][row group][k group][8 rows][8 elems]
__host__ __device__ constexpr size_t img_elems(int R) { return (size_t)NS * 4 * R * 16; }
__device__ __forceinline__ size_t img_off(int R, int s, int kk, int r) {
    const int q = kk >> 4, k16 = kk & 15;
    return (size_t)s * 4 * R * 16 + (size_t)q * R * 16 + (size_t)(r >> 3) * 128 + (k16 >> 3) * 64 + (r & 7) * 8 +
           (k16 & 7);
}

// x in [-1, 1] -> NS integer slices (exact FP64 arithmetic: every step is a power-of-two scaling or the
// difference of a value and its nearest integer)
__device__ __forceinline__ void slice(double x, __nv_bfloat16 *out, size_t stride) {
#pragma unroll
    for (int s = 0; s < NS; s++) {
        x *= 256.0;
        const double v = rint(x);
        out[s * stride] = __float2bfloat16_rn((float)v);
        x -= v;
    }
}

// the phase slices A[k][q] of every (M tile, K chunk), in the smem image layout
__global__ void k_hk_phase_img(int nk, int nR, int nchunk, int kx, int ky, int kz, const int *__restrict__ R,
                               __nv_bfloat16 *__restrict__ img) {
    const size_t per = (size_t)TM * KC;
    const size_t total = (size_t)((nk + TM - 1) / TM) * nchunk * per;
    const double ax = DG_PI;
    const int kpxy = kx * ky;
    const double delx = 2. * DG_PI / (ax * double(kx)), dely = 2. * DG_PI / (ax * double(ky)),
                 delz = 2. * DG_PI / (ax * double(kz));
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t blk = t / per;
        const int rem = (int)(t % per), r = rem / KC, kk = rem % KC;
        const int mt = (int)(blk / nchunk), kc = (int)(blk % nchunk);
        const int k = mt * TM + r, q = kc * KC + kk, rv = q >> 1;
        double a = 0.0;
        if (k < nk && rv < nR) {
            // k mesh of src/TB.cpp:196-207 (ax = ay = az = pi), the same arithmetic as the FP64 k_hk
            const double k0 = -DG_PI / ax + delx / 2. + (k % kx) * delx;
            const double k1 = -DG_PI / ax + dely / 2. + ((k % kpxy) / kx) * dely;
            const double k2 = -DG_PI / ax + delz / 2. + (k / kpxy) * delz;
            const int *Rv = R + 3 * rv;
            const double ang = (k0 * ax * Rv[0]) + (k1 * ax * Rv[1]) + (k2 * ax * Rv[2]);
            double s, c;
            sincos(ang, &s, &c);
            a = (q & 1) ? s : c;
        }
        __nv_bfloat16 *base = img + blk * img_elems(TM);
        slice(a, base + img_off(TM, 0, kk, r), (size_t)4 * TM * 16);
    }
}

// per output column pair (element e): the power of two g >= max_r max(|Re T_r(e)|, |Im T_r(e)|)
__global__ void k_hk_colscale(int nR, int ne, const double2 *__restrict__ T, double *__restrict__ g) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double m = 0.0;
    for (int r = 0; r < nR; r++) {
        const double2 t = T[(size_t)r * ne + e];
        m = fmax(m, fmax(fabs(t.x), fabs(t.y)));
    }
    int ex = 0;
    frexp(m, &ex);  // m = f 2^ex, f in [0.5, 1)
    g[e] = (m > 0.0) ? ldexp(1.0, ex) : 1.0;
}

// the hopping slices B[c][q] / g_c of every (N tile, K chunk), in the smem image layout
__global__ void k_hk_hop_img(int nR, int ne, int nchunk, const double2 *__restrict__ T, const double *__restrict__ g,
                             __nv_bfloat16 *__restrict__ img) {
    const size_t per = (size_t)TN * KC;
    const int ncol = 2 * ne;
    const size_t total = (size_t)((ncol + TN - 1) / TN) * nchunk * per;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t blk = t / per;
        const int rem = (int)(t % per), r = rem / KC, kk = rem % KC;
        const int nt = (int)(blk / nchunk), kc = (int)(blk % nchunk);
        const int c = nt * TN + r, q = kc * KC + kk, rv = q >> 1;
        double b = 0.0;
        if (c < ncol && rv < nR) {
            const int e = c >> 1;
            const double2 tv = T[(size_t)rv * ne + e];
            const bool im_out = (c & 1) != 0, sin_term = (q & 1) != 0;
            b = im_out ? (sin_term ? -tv.x : tv.y) : (sin_term ? tv.y : tv.x);
            b /= g[e];  // a power of two: exact
        }
        __nv_bfloat16 *base = img + blk * img_elems(TN);
        slice(b, base + img_off(TN, 0, kk, r), (size_t)4 * TN * 16);
    }
}

// double-float helpers for the drain (FP32 pipe): a + b with b a float, and the FP64 value of hi + lo
struct dfs {
    float h, l;
};
__device__ __forceinline__ dfs dfs_add(dfs a, float b) {
    const float s = __fadd_rn(a.h, b);
    const float bb = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b, bb)), a.l);
    const float t = __fadd_rn(s, e);
    return {t, __fsub_rn(e, __fsub_rn(t, s))};
}

constexpr int NSTAGE = 2;      // shared-memory ring of chunk images
constexpr int GROUP = 2;       // chunks accumulated in TMEM between drains: K = 128 keeps every level exact
constexpr int NBUF = 2;        // TMEM accumulator sets (NBUF * NL * TN <= 512 columns)
constexpr uint32_t A_BYTES = (uint32_t)(img_elems(TM) * 2), B_BYTES = (uint32_t)(img_elems(TN) * 2);
constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int NTHREADS = 192;  // warps 0-3: drain (TMEM lane quarters 0-3); warp 4: bulk copies; warp 5: MMA

struct TcBars {
    uint64_t full[NSTAGE], empty[NSTAGE], tfull[NBUF], tempty[NBUF];
    uint32_t tslot;
    int err;
};
// the shared error flag is written by one role and polled by the others: read it through a volatile access
__device__ __forceinline__ bool tc_failed(TcBars *b) { return *reinterpret_cast<volatile int *>(&b->err) != 0; }

// One (128 k points) x (48 real columns) tile of H(k), warp-specialised: warp 4 streams the chunk images
// into a two-stage shared-memory ring with 1-D bulk copies (mbarrier transaction counts); warp 5 issues the
// 4 x 15 MMAs of each chunk into one of two TMEM accumulator sets and hands a set over every GROUP chunks;
// warps 0-3 drain a set (their lane = k point) into double-float registers while the next set fills.
__global__ void __launch_bounds__(NTHREADS, 1) k_hk_tc(int nk, int ne, int nchunk,
                                                      const __nv_bfloat16 *__restrict__ Aimg,
                                                      const __nv_bfloat16 *__restrict__ Bimg,
                                                      const double *__restrict__ g, double2 *__restrict__ hk,
                                                      int *status) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    TcBars *bar = reinterpret_cast<TcBars *>(smraw + NSTAGE * STAGE_BYTES);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nt = blockIdx.x, mt = blockIdx.y;  // CTAs resident together share mt: its phase tiles stay in L2
    const int ngroup = (nchunk + GROUP - 1) / GROUP;
    if (warp == 0) {
        tc::tmem_alloc(&bar->tslot, TMEM_COLS_PIPE);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < NSTAGE; i++) {
            tc::mbar_init(&bar->full[i], 1);
            tc::mbar_init(&bar->empty[i], 1);
        }
        for (int i = 0; i < NBUF; i++) {
            tc::mbar_init(&bar->tfull[i], 1);
            tc::mbar_init(&bar->tempty[i], 128);
        }
        bar->err = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = bar->tslot;

    if (warp == 4) {
        if (lane == 0) {
            int issued = 0;
            for (int c = 0; c < nchunk; c++) {
                const int st = c & 1;
                if (c >= NSTAGE && !tc::mbar_wait(&bar->empty[st], ((c >> 1) - 1) & 1, WAIT_LIMIT)) {
                    atomicExch(&bar->err, 1);
                    break;
                }
                unsigned char *dst = smraw + st * STAGE_BYTES;
                tc::mbar_arrive_expect_tx(&bar->full[st], STAGE_BYTES);
                tc::bulk_g2s(dst, Aimg + ((size_t)mt * nchunk + c) * img_elems(TM), A_BYTES, &bar->full[st]);
                tc::bulk_g2s(dst + A_BYTES, Bimg + ((size_t)nt * nchunk + c) * img_elems(TN), B_BYTES,
                             &bar->full[st]);
                issued = c + 1;
            }
            if (tc_failed(bar)) {
                // let the copies already in flight land before the CTA's shared memory goes away
                for (int c = (issued > NSTAGE ? issued - NSTAGE : 0); c < issued; c++)
                    tc::mbar_wait(&bar->full[c & 1], (c >> 1) & 1, WAIT_LIMIT);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            constexpr uint32_t IDESC = tc::idesc_bf16_f32(TM, TN);
            for (int gi = 0; gi < ngroup && !tc_failed(bar); gi++) {
                const int b = gi & 1;
                if (gi >= NBUF && !tc::mbar_wait(&bar->tempty[b], ((gi >> 1) - 1) & 1, WAIT_LIMIT)) {
                    atomicExch(&bar->err, 1);
                    break;
                }
                tc::fence_after_sync();
                const uint32_t acc0 = tbase + (uint32_t)(b * NL * TN);
                int started = 0;  // bit L: level L of this set has been written in this group
                const int c1 = min(nchunk, (gi + 1) * GROUP);
                for (int c = gi * GROUP; c < c1; c++) {
                    const int st = c & 1;
                    if (!tc::mbar_wait(&bar->full[st], (c >> 1) & 1, WAIT_LIMIT)) {
                        atomicExch(&bar->err, 1);
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t a0 = tc::smem_u32(smraw + st * STAGE_BYTES), b0 = a0 + A_BYTES;
#pragma unroll 1
                    for (int q = 0; q < 4; q++)
#pragma unroll 1
                        for (int i = 0; i < NS; i++)
#pragma unroll 1
                            for (int j = 0; j < NS - i; j++) {
                                const int L = i + j;
                                const uint64_t ad = tc::smem_desc(a0 + (uint32_t)((i * 4 + q) * TM * 16 * 2), 128, 256);
                                const uint64_t bd = tc::smem_desc(b0 + (uint32_t)((j * 4 + q) * TN * 16 * 2), 128, 256);
                                tc::mma_bf16(acc0 + (uint32_t)(L * TN), ad, bd, IDESC, (started >> L) & 1);
                                started |= 1 << L;
                            }
                    tc::mma_commit(&bar->empty[st]);  // this stage's images may be overwritten once these finish
                }
                tc::mma_commit(&bar->tfull[b]);        // the set is complete once every MMA issued so far is
            }
        }
    } else {
        // drain: level L (slice levels summing to L + 2) weighs 2^{-8(L+2)}, an exact power-of-two scaling
        dfs acc[TN];
#pragma unroll
        for (int c = 0; c < TN; c++) acc[c] = {0.f, 0.f};
        const uint32_t lane_addr = tbase + ((uint32_t)(warp * 32) << 16);
        bool ok = true;
        for (int gi = 0; gi < ngroup; gi++) {
            const int b = gi & 1;
            if (!tc::mbar_wait(&bar->tfull[b], (gi >> 1) & 1, WAIT_LIMIT) || tc_failed(bar)) {
                ok = false;
                atomicExch(&bar->err, 1);
                break;
            }
            tc::fence_after_sync();
#pragma unroll
            for (int cg = 0; cg < TN / 16; cg++) {
#pragma unroll
                for (int L = 0; L < NL; L++) {
                    float v[16];
                    tc::tmem_ld16(lane_addr + (uint32_t)(b * NL * TN + L * TN + cg * 16), v);
                    const float w = __int_as_float((127 - 8 * (L + 2)) << 23);  // 2^{-8(L+2)}
#pragma unroll
                    for (int c = 0; c < 16; c++) acc[cg * 16 + c] = dfs_add(acc[cg * 16 + c], v[c] * w);
                }
            }
            tc::fence_before_sync();
            tc::mbar_arrive(&bar->tempty[b]);
        }
        const int k = mt * TM + threadIdx.x;
        if (ok && k < nk) {
#pragma unroll
            for (int c = 0; c < TN; c += 2) {
                const int e = (nt * TN + c) >> 1;
                if (e < ne) {
                    const double sc = g[e];
                    hk[(size_t)k * ne + e] = make_double2(((double)acc[c].h + (double)acc[c].l) * sc,
                                                          ((double)acc[c + 1].h + (double)acc[c + 1].l) * sc);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0 && tc_failed(bar)) atomicMax(status, (int)DMFTGPU_TIMEOUT);
    if (warp == 0) tc::tmem_dealloc(tbase, TMEM_COLS_PIPE);
}

size_t tc_smem_bytes() { return (size_t)NSTAGE * STAGE_BYTES + sizeof(TcBars); }

}  // namespace

// H(k) on the tensor cores (all pointers device): R [nR][3], T [nR][n*n] complex, hk [nk][n*n] complex.
// `mesh_key` identifies (k mesh, R list): the phase-slice image is rebuilt only when it changes.
int dg_hk_tensor(dmftgpu_ctx *ctx, int n, int nR, const int *dR, const double2 *dT, int kx, int ky, int kz,
                 double2 *dH, const std::string &mesh_key) {
    const int nk = kx * ky * kz, ne = n * n;
    const int nchunk = dg_ceil_div(2 * nR, KC);
    const int nmt = dg_ceil_div(nk, TM), nnt = dg_ceil_div(2 * ne, TN);
    const size_t abytes = (size_t)nmt * nchunk * img_elems(TM) * sizeof(__nv_bfloat16);
    const size_t bbytes = (size_t)nnt * nchunk * img_elems(TN) * sizeof(__nv_bfloat16);
    __nv_bfloat16 *Aimg = (__nv_bfloat16 *)dg_buf(ctx, "hk.tc.A", abytes);
    __nv_bfloat16 *Bimg = (__nv_bfloat16 *)dg_buf(ctx, "hk.tc.B", bbytes);
    double *g = (double *)dg_buf(ctx, "hk.tc.g", (size_t)ne * sizeof(double));
    if (!Aimg || !Bimg || !g) return DMFTGPU_NOMEM;
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    const std::string key = mesh_key + "/" + std::to_string(abytes);
    if (ctx->hk_phase_key != key) {
        k_hk_phase_img<<<nsm * 8, 256, 0, ctx->stream>>>(nk, nR, nchunk, kx, ky, kz, dR, Aimg);
        DG_LAUNCH(ctx, "k_hk_phase_img");
        ctx->hk_phase_key = key;
    }
    k_hk_colscale<<<dg_ceil_div(ne, 128), 128, 0, ctx->stream>>>(nR, ne, dT, g);
    DG_LAUNCH(ctx, "k_hk_colscale");
    k_hk_hop_img<<<nsm * 4, 256, 0, ctx->stream>>>(nR, ne, nchunk, dT, g, Bimg);
    DG_LAUNCH(ctx, "k_hk_hop_img");
    const size_t smem = tc_smem_bytes();
    DG_CUDA(cudaFuncSetAttribute(k_hk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    {
        DgTimer tm(ctx, "k_hk_tc");
        k_hk_tc<<<dim3(nnt, nmt), NTHREADS, smem, ctx->stream>>>(nk, ne, nchunk, Aimg, Bimg, g, dH, ctx->d_status);
    }
    DG_LAUNCH(ctx, "k_hk_tc");
    return DMFTGPU_OK;
}
