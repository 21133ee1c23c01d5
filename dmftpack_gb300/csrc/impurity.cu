// impurity.cu -- impurity-side kernels: the hybridisation function (Construct_hyb_delta).
#include "linalg.cuh"

namespace {

// one thread per Matsubara frequency (src/Construct_hyb_delta.cpp:98-113)
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

}  // namespace

extern "C" int dmftgpu_hyb_delta(dmftgpu_ctx *ctx, int dim, const int *orb, int nfreq, double beta, int D,
                                 const double *sigma, const double *gw, const double *himp, double mu, double *delta,
                                 int flags) {
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
