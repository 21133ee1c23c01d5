// solvers.cu -- weak-coupling impurity solvers driven from the host, every step on the device:
//   IPT (src/SCGF2_fullLoop.cpp:873-1065): Kajueter-Kotliar interpolated second-order self-energy on two
//   spin-orbitals.  The host only sequences kernels and reads back the two 2x2 occupation matrices the
//   interpolation coefficients need.
//   SCGF2 (src/SCGF2_fullLoop.cpp:392-533): the self-consistent second-order (SC2PT) loop on G_imp with Pulay
//   mixing.  The host reads back two residual norms and the status word per loop iteration (the loop's
//   stopping test).
//   weak_solver (src/SOLVER.cpp:72-102): the one-shot low-level solvers of the weakly correlated subspace,
//   HF (on_shot_HF, src/SCGF2_fullLoop.cpp:218-250) and 2PT / SC2PT (SC2PT_weak, src/SCGF2_fullLoop.cpp:49-133).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "impurity.h"

namespace {

__global__ void k_set_identity(int d, double2 *m) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < d * d) m[q] = cmk((q % d) == (q / d) ? 1.0 : 0.0, 0.0);
}

// writeResults (src/SCGF2_fullLoop.cpp:696-720): SE_out and Gwimp_out in ImgFreqFtn slot order
__global__ void k_write_results(int d, int nfreq, const double2 *s2, const double2 *fock, const double2 *gimp,
                                double2 *se_out, double2 *gimp_out) {
    const size_t dd = (size_t)d * d;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)(nfreq + 5) * dd) return;
    const int slot = (int)(t / dd), e = (int)(t % dd);
    double2 se = cmk(0, 0), g = cmk(0, 0);
    if (slot < nfreq) {
        se = cadd(s2[t], fock[e]);
        g = gimp[t];
    } else if (slot == nfreq) {
        se = fock[e];
    } else {
        const int k = slot - nfreq;  // 1..4
        if (k == 1) se = s2[(size_t)nfreq * dd + e];
        if (k == 2) se = s2[(size_t)(nfreq + 1) * dd + e];
        g = gimp[(size_t)(nfreq + k - 1) * dd + e];
    }
    se_out[t] = se;
    if (gimp_out) gimp_out[t] = g;
}

// MatsubaraFtnnorm (src/SCGF2_fullLoop.cpp:791-805) of g - gin (gin == nullptr: of g) squared, per frequency
__global__ void k_scgf_norm_terms(int d, int nfreq, double beta, const double2 *gin, const double2 *g, double *terms) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nfreq) return;
    const size_t dd = (size_t)d * d;
    const double wn = (2 * n + 1) * DG_PI / beta;
    double a = 0;
    for (size_t e = 0; e < dd; e++) {
        const double2 x = gin ? csub(gin[(size_t)n * dd + e], g[(size_t)n * dd + e]) : g[(size_t)n * dd + e];
        a += cabs2(x);
    }
    terms[n] = a / wn;
}

// fixed-order sum of the per-frequency terms, and ||occ - occ_in||_F^2; one block
__global__ void k_scgf_norms(int d, int nfreq, const double *terms, const double2 *occ_in, const double2 *occ,
                             double *out) {
    __shared__ double red[256];
    double s = 0;
    for (int n = threadIdx.x; n < nfreq; n += blockDim.x) s += terms[n];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double o = 0;
        if (occ_in)
            for (int e = 0; e < d * d; e++) o += cabs2(csub(occ[e], occ_in[e]));
        out[0] = red[0];
        out[1] = o;
    }
}

// (1 - a) x + a y over n elements (the linear mixing branch of SCGF2, :481-485)
__global__ void k_lin_mix(long long n, double a, const double2 *x, double2 *y) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) y[t] = cadd(cscale(x[t], 1.0 - a), cscale(y[t], a));
}

}  // namespace

// IPT on device pointers.  delta: nfreq slots; se_out, gimp_out: nfreq+5 slots; occ_in/occ_out: d x d.
int dg_ipt_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, double U, double mu, const double2 *himp,
               const double2 *delta, const double2 *occ_in, const DgUList &Ul, double2 *se_out, double2 *gimp_out,
               double2 *occ_out) {
    if (d != 2) return dg_fail(ctx, DMFTGPU_BADARG, "IPT is defined for two spin-orbitals");
    const size_t dd = (size_t)d * d;
    cudaStream_t s = ctx->stream;
    double2 *fock = (double2 *)dg_buf(ctx, "ipt.fock", dd * sizeof(double2));
    double2 *s2 = (double2 *)dg_buf(ctx, "ipt.s2", (size_t)(nfreq + 3) * dd * sizeof(double2));
    double2 *gw0 = (double2 *)dg_buf(ctx, "ipt.gw0", (size_t)(nfreq + 4) * dd * sizeof(double2));
    double2 *gimp = (double2 *)dg_buf(ctx, "ipt.gimp", (size_t)(nfreq + 4) * dd * sizeof(double2));
    double2 *gt = (double2 *)dg_buf(ctx, "ipt.gt", (size_t)(ntau + 1) * dd * sizeof(double2));
    double2 *st = (double2 *)dg_buf(ctx, "ipt.st", (size_t)(ntau + 1) * dd * sizeof(double2));
    if (!fock || !s2 || !gw0 || !gimp || !gt || !st) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemsetAsync(s2, 0, (size_t)(nfreq + 3) * dd * sizeof(double2), s));
    DG_CUDA(cudaMemsetAsync(gw0, 0, (size_t)(nfreq + 4) * dd * sizeof(double2), s));
    DG_CUDA(cudaMemsetAsync(gimp, 0, (size_t)(nfreq + 4) * dd * sizeof(double2), s));
    // the interpolation coefficients use the input occupation (src/SCGF2_fullLoop.cpp:932-945, 1036-1041)
    double2 occ_h[4];
    DG_CUDA(cudaMemcpyAsync(occ_h, occ_in, dd * sizeof(double2), cudaMemcpyDeviceToHost, s));
    // HF: Fock from the input occupation, Dyson with S2 = 0 at muHF = mu
    DG_TRY(dg_fock_dev(ctx, d, Ul, occ_in, fock));
    DG_TRY(dg_dyson_dev(ctx, d, nfreq, beta, mu, himp, delta, fock, s2, gw0, true));
    k_set_identity<<<1, 32, 0, s>>>(d, gw0 + (size_t)nfreq * dd);
    DG_LAUNCH(ctx, "k_set_identity");
    // FourierTransform(Gw0, Gt0, Gw0[N_freq]): non-Green fit, then m0 = 0, m1 = Gw0[N_freq] = I
    DG_TRY(dg_fourier_dev(ctx, d, nfreq, ntau, beta, gw0, 0, gw0 + (size_t)nfreq * dd, gt));
    DG_TRY(dg_sigma2_dev(ctx, d, ntau, beta, Ul, gt, st));
    DG_TRY(dg_tau2w_dev(ctx, d, nfreq, ntau, beta, st, s2, true));
    DG_CUDA(cudaStreamSynchronize(s));
    const double n11 = occ_h[3].x, n00 = occ_h[0].x;  // occMat(1,1), occMat(0,0) (real parts)
    const double muHF = mu;
    double a[2], b[2], c[2];
    a[0] = U * U * n11 * (1.0 - n11);
    a[1] = U * U * n00 * (1.0 - n00);
    b[0] = (muHF - mu + U * (1.0 - 2.0 * n11));
    b[1] = (muHF - mu + U * (1.0 - 2.0 * n00));
    c[0] = U * U * n11 * (1.0 - n11);  // occMatHF == occMat on entry
    c[1] = U * U * n00 * (1.0 - n00);
    DG_TRY(dg_ipt_kk_dev(ctx, nfreq, a, b, c, s2));
    DG_TRY(dg_dyson_dev(ctx, d, nfreq, beta, mu, himp, delta, fock, s2, gimp, true));
    k_set_identity<<<1, 32, 0, s>>>(d, gimp + (size_t)nfreq * dd);
    DG_LAUNCH(ctx, "k_set_identity");
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, gimp, 2));
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, gimp, 3));
    DG_TRY(dg_occ_dev(ctx, d, nfreq, beta, gimp, occ_out));
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, s2, 1));
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, s2, 2));
    k_write_results<<<dg_ceil_div((long long)(nfreq + 5) * dd, 128), 128, 0, s>>>(d, nfreq, s2, fock, gimp, se_out,
                                                                                  gimp_out);
    DG_LAUNCH(ctx, "k_write_results");
    return DMFTGPU_OK;
}

// SCGF2 on device pointers.  weiss: nfreq slots; gimp: in, nfreq slots (the initial G_imp); out, nfreq+5
// slots; se_out: nfreq+5 slots.  *loops receives the number of loop iterations run.
int dg_scgf2_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, double mu, double mixing,
                 const double2 *himp, const double2 *weiss, double2 *gimp, const DgUList &Ul, int max_iter,
                 double2 *se_out, int *loops) {
    const size_t dd = (size_t)d * d;
    const long long len = (long long)nfreq * dd;
    cudaStream_t s = ctx->stream;
    double2 *G = (double2 *)dg_buf(ctx, "scgf.g", (size_t)(nfreq + 4) * dd * sizeof(double2));
    double2 *Gin = (double2 *)dg_buf(ctx, "scgf.gin", (size_t)nfreq * dd * sizeof(double2));
    double2 *s2 = (double2 *)dg_buf(ctx, "scgf.s2", (size_t)(nfreq + 3) * dd * sizeof(double2));
    double2 *gt = (double2 *)dg_buf(ctx, "scgf.gt", (size_t)(ntau + 1) * dd * sizeof(double2));
    double2 *st = (double2 *)dg_buf(ctx, "scgf.st", (size_t)(ntau + 1) * dd * sizeof(double2));
    double2 *occ = (double2 *)dg_buf(ctx, "scgf.occ", 2 * dd * sizeof(double2));
    double2 *fock = (double2 *)dg_buf(ctx, "scgf.fock", dd * sizeof(double2));
    double *nrm = (double *)dg_buf(ctx, "scgf.norms", 2 * sizeof(double));
    double *nterm = (double *)dg_buf(ctx, "scgf.nterms", (size_t)nfreq * sizeof(double));
    double2 *gT = (double2 *)dg_buf(ctx, "scgf.tail", 9 * dd * sizeof(double2));
    double2 *gDw = (double2 *)dg_buf(ctx, "scgf.Dw", (size_t)nfreq * dd * sizeof(double2));
    if (!G || !Gin || !s2 || !gt || !st || !occ || !fock || !nrm || !nterm || !gT || !gDw) return DMFTGPU_NOMEM;
    double2 *occ_in = occ + dd;
    DG_CUDA(cudaMemsetAsync(G, 0, (size_t)(nfreq + 4) * dd * sizeof(double2), s));
    DG_CUDA(cudaMemsetAsync(s2, 0, (size_t)(nfreq + 3) * dd * sizeof(double2), s));
    DG_CUDA(cudaMemsetAsync(fock, 0, dd * sizeof(double2), s));
    DG_CUDA(cudaMemcpyAsync(G, gimp, len * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    double2 *Gtail = G + (size_t)nfreq * dd;  // Gwimp[N_freq] = I
    k_set_identity<<<1, 32 * (int)((dd + 31) / 32), 0, s>>>(d, Gtail);
    DG_LAUNCH(ctx, "k_set_identity");
    DG_TRY(dg_occ_dev(ctx, d, nfreq, beta, G, occ));
    k_scgf_norm_terms<<<dg_ceil_div(nfreq, 128), 128, 0, s>>>(d, nfreq, beta, nullptr, G, nterm);
    DG_LAUNCH(ctx, "k_scgf_norm_terms");
    k_scgf_norms<<<1, 256, 0, s>>>(d, nfreq, nterm, nullptr, occ, nrm);
    DG_LAUNCH(ctx, "k_scgf_norms");
    double hn[2];
    DG_CUDA(cudaMemcpyAsync(hn, nrm, sizeof(hn), cudaMemcpyDeviceToHost, s));
    DG_CUDA(cudaStreamSynchronize(s));
    const double normUnit = std::sqrt(hn[0]);
    int loop = 0;
    double normOuter = 0, normOcc = 0, mix = mixing / 10.;
    DgPulay P;
    P.hist = 2;
    P.start = 100;
    while ((loop < 10 || normOuter > 1e-6 || normOcc > 1e-6) && loop < max_iter) {
        DG_CUDA(cudaMemcpyAsync(Gin, G, len * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_CUDA(cudaMemcpyAsync(occ_in, occ, dd * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        // HF, then Sigma^(2): G(iw) -> G(tau) -> Sigma(tau) -> Sigma(iw).  getoccMat(G) and
        // FourierTransform(G, ., Gwimp[N_freq] = I, true) fit the same green-tail moments of the same G, so
        // the moments, tail data and F - tail are formed once for both.
        DG_TRY(dg_green_tail_dev(ctx, d, nfreq, beta, G, gT, gDw));
        DG_TRY(dg_occ_tail_dev(ctx, d, nfreq, beta, gT, gDw, occ));
        DG_TRY(dg_fock_dev(ctx, d, Ul, occ, fock));
        DG_TRY(dg_w2tau_tail_dev(ctx, d, nfreq, ntau, beta, gT, gDw, gt));
        DG_TRY(dg_sigma2_dev(ctx, d, ntau, beta, Ul, gt, st));
        DG_TRY(dg_tau2w_dev(ctx, d, nfreq, ntau, beta, st, s2, true));
        // G = [(iw + mu) - H_imp - Delta - F - Sigma^(2)]^-1
        DG_TRY(dg_dyson_dev(ctx, d, nfreq, beta, mu, himp, weiss, fock, s2, G, true));
        DG_TRY(dg_occ_dev(ctx, d, nfreq, beta, G, occ));
        k_scgf_norm_terms<<<dg_ceil_div(nfreq, 128), 128, 0, s>>>(d, nfreq, beta, Gin, G, nterm);
        DG_LAUNCH(ctx, "k_scgf_norm_terms");
        k_scgf_norms<<<1, 256, 0, s>>>(d, nfreq, nterm, occ_in, occ, nrm);
        DG_LAUNCH(ctx, "k_scgf_norms");
        DG_CUDA(cudaMemcpyAsync(hn, nrm, sizeof(hn), cudaMemcpyDeviceToHost, s));
        int code = 0;
        DG_TRY(dg_status_read(ctx, &code));  // synchronises the stream
        if (code) return code;
        normOcc = std::sqrt(hn[1]);
        normOuter = std::sqrt(hn[0]) / normUnit;
        if (loop % 500 == 0) mix /= 1.5;
        if (loop < 1500) {
            DG_TRY(dg_pulay_mixing(ctx, P, "scgf.pulay", len, Gin, G, mix, loop));
        } else {
            k_lin_mix<<<dg_ceil_div(len, 256), 256, 0, s>>>(len, mix, Gin, G);
            DG_LAUNCH(ctx, "k_lin_mix");
        }
        // mixing_check_outer (:722-727)
        if (loop % 10 == 0) {
            double &prev = ctx->scgf_prev_norm;
            if (prev > normOuter) mix = std::min(1.07 * mix, 0.5);
            else if (prev < normOuter) mix = std::max(1. / 1.09 * mix, 1e-3);
            prev = normOuter;
        }
        loop++;
    }
    *loops = loop;
    // writeResults (:696-720)
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, s2, 1));
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, s2, 2));
    k_write_results<<<dg_ceil_div((long long)(nfreq + 5) * dd, 128), 128, 0, s>>>(d, nfreq, s2, fock, G, se_out,
                                                                                  gimp);
    DG_LAUNCH(ctx, "k_write_results");
    return DMFTGPU_OK;
}

extern "C" int dmftgpu_scgf2(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, double mu, double mixing,
                             const double *himp, const double *weiss, double *gimp, int nu, const int *uidx,
                             const double *ut, int max_iter, double *se_out, int *loops, int flags) {
    if (!ctx || dim < 1 || dim > 32 || nfreq < 8 || ntau < 2 || !himp || !weiss || !gimp || !se_out || !loops ||
        nu < 0 || !(beta > 0) || max_iter < 1)
        return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgFtMode ftm(ctx, flags);
    const size_t dd = (size_t)dim * dim;
    int st;
    DgUList Ul;
    DG_TRY(dg_ulist(ctx, dim, nu, uidx, ut, Ul));
    const double2 *dH = (const double2 *)dg_in(ctx, himp, dd * sizeof(double2), flags, "io.scgf_h", &st);
    if (st) return st;
    const double2 *dW = (const double2 *)dg_in(ctx, weiss, nfreq * dd * sizeof(double2), flags, "io.scgf_w", &st);
    if (st) return st;
    double2 *dG = (double2 *)dg_out(ctx, gimp, (nfreq + 5) * dd * sizeof(double2), flags, "io.scgf_g", &st);
    if (st) return st;
    if (!(flags & DMFTGPU_DEVICE_PTRS))
        DG_CUDA(cudaMemcpyAsync(dG, gimp, nfreq * dd * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    double2 *dSE = (double2 *)dg_out(ctx, se_out, (nfreq + 5) * dd * sizeof(double2), flags, "io.scgf_se", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_scgf2_dev(ctx, dim, nfreq, ntau, beta, mu, mixing, dH, dW, dG, Ul, max_iter, dSE, loops));
    DG_TRY(dg_out_done(ctx, gimp, dG, (nfreq + 5) * dd * sizeof(double2), flags));
    DG_TRY(dg_out_done(ctx, se_out, dSE, (nfreq + 5) * dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

extern "C" int dmftgpu_ipt(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, double U, double mu,
                           const double *himp, const double *delta, const double *nummat_in, int nu, const int *uidx,
                           const double *ut, double *se_out, double *gimp_out, double *nummat_out, int flags) {
    if (!ctx || dim != 2 || nfreq < 8 || ntau < 2 || !himp || !delta || !nummat_in || !se_out || !nummat_out ||
        nu < 0 || !(beta > 0))
        return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgFtMode ftm(ctx, flags);
    const size_t dd = (size_t)dim * dim;
    int st;
    DgUList Ul;
    DG_TRY(dg_ulist(ctx, dim, nu, uidx, ut, Ul));
    const double2 *dH = (const double2 *)dg_in(ctx, himp, dd * sizeof(double2), flags, "io.ipt_h", &st);
    if (st) return st;
    const double2 *dD = (const double2 *)dg_in(ctx, delta, nfreq * dd * sizeof(double2), flags, "io.ipt_d", &st);
    if (st) return st;
    const double2 *dN = (const double2 *)dg_in(ctx, nummat_in, dd * sizeof(double2), flags, "io.ipt_n", &st);
    if (st) return st;
    double2 *dSE = (double2 *)dg_out(ctx, se_out, (nfreq + 5) * dd * sizeof(double2), flags, "io.ipt_se", &st);
    if (st) return st;
    double2 *dGI = gimp_out ? (double2 *)dg_out(ctx, gimp_out, (nfreq + 5) * dd * sizeof(double2), flags, "io.ipt_gi", &st)
                            : nullptr;
    if (st) return st;
    double2 *dNO = (double2 *)dg_out(ctx, nummat_out, dd * sizeof(double2), flags, "io.ipt_no", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_ipt_dev(ctx, dim, nfreq, ntau, beta, U, mu, dH, dD, dN, Ul, dSE, dGI, dNO));
    DG_TRY(dg_out_done(ctx, se_out, dSE, (nfreq + 5) * dd * sizeof(double2), flags));
    if (gimp_out) DG_TRY(dg_out_done(ctx, gimp_out, dGI, (nfreq + 5) * dd * sizeof(double2), flags));
    DG_TRY(dg_out_done(ctx, nummat_out, dNO, dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}

// weak_solver on device pointers.  gw: nfreq slots (Gw_weak); gwhf: nfreq slots (GwHF_weak, read by 2PT only);
// se_out: nfreq+5 slots (SE_out in ImgFreqFtn order).
//   HF:     occ = getoccMat(G), F = getFockOperator(occ), Sigma^(2) = 0
//   2PT:    as SC2PT with G0 = GwHF;  SC2PT: G0 = G
//   (SC)2PT: occ and F from G; G0(iw) -> G0(tau) (green tail, m1 = I); Sigma^(2)(tau) = getStimp(G0(tau));
//           Sigma^(2)(iw) = FT_t_to_w; the two tail estimates; writeResults
int dg_weak_solver_dev(dmftgpu_ctx *ctx, int solver, int d, int nfreq, int ntau, double beta, const double2 *gw,
                       const double2 *gwhf, const DgUList &Ul, double2 *se_out) {
    const size_t dd = (size_t)d * d;
    cudaStream_t s = ctx->stream;
    double2 *G = (double2 *)dg_buf(ctx, "weak.g", (size_t)(nfreq + 4) * dd * sizeof(double2));
    double2 *s2 = (double2 *)dg_buf(ctx, "weak.s2", (size_t)(nfreq + 3) * dd * sizeof(double2));
    double2 *occ = (double2 *)dg_buf(ctx, "weak.occ", dd * sizeof(double2));
    double2 *fock = (double2 *)dg_buf(ctx, "weak.fock", dd * sizeof(double2));
    if (!G || !s2 || !occ || !fock) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemsetAsync(G, 0, (size_t)(nfreq + 4) * dd * sizeof(double2), s));
    DG_CUDA(cudaMemsetAsync(s2, 0, (size_t)(nfreq + 3) * dd * sizeof(double2), s));
    DG_CUDA(cudaMemcpyAsync(G, gw, (size_t)nfreq * dd * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    k_set_identity<<<1, 32 * (int)((dd + 31) / 32), 0, s>>>(d, G + (size_t)nfreq * dd);  // Gwimp[N_freq] = I
    DG_LAUNCH(ctx, "k_set_identity");
    DG_TRY(dg_occ_dev(ctx, d, nfreq, beta, G, occ));
    DG_TRY(dg_fock_dev(ctx, d, Ul, occ, fock));
    if (solver != DMFTGPU_WEAK_HF) {
        double2 *gt = (double2 *)dg_buf(ctx, "weak.gt", (size_t)(ntau + 1) * dd * sizeof(double2));
        double2 *st = (double2 *)dg_buf(ctx, "weak.st", (size_t)(ntau + 1) * dd * sizeof(double2));
        double2 *T = (double2 *)dg_buf(ctx, "weak.tail", 9 * dd * sizeof(double2));
        double2 *Dw = (double2 *)dg_buf(ctx, "weak.Dw", (size_t)nfreq * dd * sizeof(double2));
        if (!gt || !st || !T || !Dw) return DMFTGPU_NOMEM;
        // FourierTransform(G0, Gt0, G0[N_freq] = I, true): the green-tail fit of G0
        const double2 *g0 = (solver == DMFTGPU_WEAK_SC2PT) ? G : gwhf;
        DG_TRY(dg_green_tail_dev(ctx, d, nfreq, beta, g0, T, Dw));
        DG_TRY(dg_w2tau_tail_dev(ctx, d, nfreq, ntau, beta, T, Dw, gt));
        DG_TRY(dg_sigma2_dev(ctx, d, ntau, beta, Ul, gt, st));
        DG_TRY(dg_tau2w_dev(ctx, d, nfreq, ntau, beta, st, s2, true));
    }
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, s2, 1));
    DG_TRY(dg_estimate_asymto_dev(ctx, d, nfreq, beta, s2, 2));
    k_write_results<<<dg_ceil_div((long long)(nfreq + 5) * dd, 128), 128, 0, s>>>(d, nfreq, s2, fock, G, se_out,
                                                                                  nullptr);
    DG_LAUNCH(ctx, "k_write_results");
    return DMFTGPU_OK;
}

extern "C" int dmftgpu_weak_solver(dmftgpu_ctx *ctx, int solver, int dim, int nfreq, int ntau, double beta,
                                   const double *gw, const double *gwhf, int nu, const int *uidx, const double *ut,
                                   double *se_out, int flags) {
    if (!ctx || dim < 1 || dim > 32 || nfreq < 8 || ntau < 2 || !gw || !se_out || nu < 0 || !(beta > 0) ||
        solver < DMFTGPU_WEAK_HF || solver > DMFTGPU_WEAK_SC2PT || (solver == DMFTGPU_WEAK_2PT && !gwhf))
        return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    DgFtMode ftm(ctx, flags);
    const size_t dd = (size_t)dim * dim;
    int st;
    DgUList Ul;
    DG_TRY(dg_ulist(ctx, dim, nu, uidx, ut, Ul));
    const double2 *dG = (const double2 *)dg_in(ctx, gw, nfreq * dd * sizeof(double2), flags, "io.weak_g", &st);
    if (st) return st;
    const double2 *dGHF = nullptr;
    if (solver == DMFTGPU_WEAK_2PT) {
        dGHF = (const double2 *)dg_in(ctx, gwhf, nfreq * dd * sizeof(double2), flags, "io.weak_ghf", &st);
        if (st) return st;
    }
    double2 *dSE = (double2 *)dg_out(ctx, se_out, (nfreq + 5) * dd * sizeof(double2), flags, "io.weak_se", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_weak_solver_dev(ctx, solver, dim, nfreq, ntau, beta, dG, dGHF, Ul, dSE));
    DG_TRY(dg_out_done(ctx, se_out, dSE, (nfreq + 5) * dd * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code;
}
