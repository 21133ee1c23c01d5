// dmft.cu -- one DMFT self-consistency iteration (the body of the loop in src/dmft_main.cpp:343-570) for a
// single correlated cluster/atom with the IPT or the SC2PT (SCGF2) impurity solver, every array on the device:
//   SOLVER (src/SOLVER.cpp:105-502): proj_to_site (H_imp - DC), IPT or SCGF2 (the latter started from the
//     lattice G_loc block, src/dmft_main.cpp:389-405), the magnetism == 0 spin average, NumMatrix update
//     (IPT's occupation; SCGF2 leaves projNumMatrix as proj_to_site copied it); SE_out = Sigma_imp - DC
//     (src/dmft_main.cpp:489-525)
//   Pulay mixing of SelfEnergy_w (pulayMixing(2, 5, N_freq, D, D), used at src/dmft_main.cpp:529-533;
//     mixing.cu)
//   TightBinding (src/TB.cpp:97-369): mu search, GreenFtn_w, Construct_hyb_delta, impurity_site_Hamiltonian
//     (k average of the correlated block, src/downfolding.cpp:86-121)
//   dmft_scf_check residuals (src/dmft_main.cpp:902-1014) on the in-memory G_imp and G_loc
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "impurity.h"

int dg_ipt_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, double U, double mu, const double2 *himp,
               const double2 *delta, const double2 *occ_in, const DgUList &Ul, double2 *se_out, double2 *gimp_out,
               double2 *occ_out);
int dg_scgf2_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, double mu, double mixing,
                 const double2 *himp, const double2 *weiss, double2 *gimp, const DgUList &Ul, int max_iter,
                 double2 *se_out, int *loops);

namespace {

// k average of the correlated block of H(k): rows/columns hartr[a], hartr[b]
__global__ void k_himp(int nk, int n, int D, const int *hartr, const double2 *H, double2 *himp) {
    __shared__ double2 red[256];
    const int e = blockIdx.x, a = hartr[e % D], b = hartr[e / D];
    double2 s = cmk(0, 0);
    for (int k = threadIdx.x; k < nk; k += blockDim.x) s = cadd(s, H[(size_t)k * n * n + a + (size_t)b * n]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) himp[e] = cmk(red[0].x / nk, red[0].y / nk);
}

// proj_to_site: H_imp - DC (src/SOLVER.cpp:514-521)
__global__ void k_sub(int n, const double2 *a, const double2 *b, double2 *out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = csub(a[t], b[t]);
}

// magnetism == 0 spin average of SE_out (all nfreq+5 slots) and projNumMatrix (src/SOLVER.cpp:440-456)
__global__ void k_spin_average(int d, int nslots, double2 *se, double2 *occ) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int npair = d / 2;
    if (t >= (long long)(nslots + 1) * npair) return;
    const int slot = (int)(t / npair), n = 2 * (int)(t % npair);
    double2 *M = (slot < nslots) ? se + (size_t)slot * d * d : occ;
    const double2 avg = cscale(cadd(DG_AT(M, d, n, n), DG_AT(M, d, n + 1, n + 1)), 0.5);
    DG_AT(M, d, n, n) = avg;
    DG_AT(M, d, n + 1, n + 1) = avg;
    DG_AT(M, d, n, n + 1) = cmk(0, 0);
    DG_AT(M, d, n + 1, n) = cmk(0, 0);
}

// SelfEnergy_w_out = SE_out - DC for w < N_freq (only these slots reach SelfEnergy_w, src/ImgTimeFtn.cpp:575-606)
__global__ void k_se_combine(int nfreq, int d, const double2 *se, const double2 *dc, double2 *out) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int dd = d * d;
    if (t >= (long long)nfreq * dd) return;
    out[t] = csub(se[t], dc[t % dd]);
}

// scf residual sums over n < N_freq (src/dmft_main.cpp:971-997): per frequency |Gimp - Gloc|^2, |Gloc|^2
__global__ void k_scf_terms(int nfreq, int d, const double2 *gimp, const double2 *gloc, double *rd, double *nrm) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nfreq) return;
    const int dd = d * d;
    double a = 0, b = 0;
    for (int e = 0; e < dd; e++) {
        double2 x = csub(gimp[(size_t)n * dd + e], gloc[(size_t)n * dd + e]);
        a += cabs2(x);
        b += cabs2(gloc[(size_t)n * dd + e]);
    }
    rd[n] = a;
    nrm[n] = b;
}

double2 *buf2(dmftgpu_ctx *ctx, const char *name, size_t count) {
    return (double2 *)dg_buf(ctx, name, count * sizeof(double2));
}

}  // namespace

extern "C" int dmftgpu_dmft_iteration(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk,
                                      const dmftgpu_dmft_params *p, int iteration, double *selfe, double *weiss,
                                      double *nummat, double *mu, double *gloc, double *gimp, double *resid,
                                      int flags) {
    if (!ctx || !L || !hk || !p || !selfe || !weiss || !nummat || !mu || !gloc || !gimp || !resid)
        return DMFTGPU_BADARG;
    if (!(flags & DMFTGPU_DEVICE_PTRS)) return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: device pointers only");
    if (p->solver != DMFTGPU_SOLVER_IPT && p->solver != DMFTGPU_SOLVER_SC2PT)
        return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: solver");
    const int D = L->ncl * L->nh, Nf = L->nfreq, DD = D * D;
    if (L->ncl != 1) return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: one correlated cluster");
    if (p->solver == DMFTGPU_SOLVER_IPT && D != 2)
        return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: IPT needs 2 spin-orbitals");
    if (D > 32 || (p->magnetism == 0 && D % 2))
        return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: correlated block must be <= 32 spin-orbital pairs");
    cudaSetDevice(ctx->device);
    DgFtMode ftm(ctx, flags);
    DgTensorMode tmode(ctx, flags);
    cudaStream_t s = ctx->stream;
    const int dflags = DMFTGPU_DEVICE_PTRS | (flags & (DMFTGPU_MIXED | DMFTGPU_NEWTON | DMFTGPU_NO_TENSOR));
    double2 *dSE = (double2 *)selfe, *dW = (double2 *)weiss, *dN = (double2 *)nummat, *dG = (double2 *)gloc,
            *dGI = (double2 *)gimp;
    DgUList Ul;
    DG_TRY(dg_ulist(ctx, D, p->nu, p->uidx, p->ut, Ul));
    double2 *himp = buf2(ctx, "dmft.himp", DD), *hdc = buf2(ctx, "dmft.hdc", DD), *dc = buf2(ctx, "dmft.dc", DD);
    double2 *seimp = buf2(ctx, "dmft.seimp", (size_t)(Nf + 5) * DD), *seout = buf2(ctx, "dmft.seout", (size_t)Nf * DD);
    double2 *occ = buf2(ctx, "dmft.occ", DD), *nm_imp = buf2(ctx, "dmft.nmimp", DD);
    double *rd = (double *)dg_buf(ctx, "dmft.rd", 2 * (size_t)Nf * sizeof(double));
    int *dhartr = (int *)dg_buf(ctx, "dmft.hartr", D * sizeof(int));
    if (!himp || !hdc || !dc || !seimp || !seout || !occ || !nm_imp || !rd || !dhartr) return DMFTGPU_NOMEM;
    {
        std::vector<int> h(D);
        for (int i = 0; i < D; i++) h[i] = L->hartr ? L->hartr[i] : i;
        for (int i = 0; i < D; i++)
            if (h[i] < 0 || h[i] >= L->n) return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: bad HartrIndex");
        DG_CUDA(cudaMemcpyAsync(dhartr, h.data(), D * sizeof(int), cudaMemcpyHostToDevice, s));
        DG_CUDA(cudaStreamSynchronize(s));
    }
    // impurity_site_Hamiltonian (k average of H_PP) and the double counting (dc_for_dmft, nominal)
    k_himp<<<DD, 256, 0, s>>>(L->nk, L->n, D, dhartr, (const double2 *)hk, himp);
    DG_LAUNCH(ctx, "k_himp");
    {
        const int Nh = D;  // N_peratom_HartrOrbit
        const double averU = (Nh * p->U + Nh * (Nh - 1) * p->Uprime) / (double)(Nh * Nh);
        const double v = averU * (p->nominal_charge - 0.5) - p->J * (p->nominal_charge / 2.0 - 0.5);
        std::vector<double2> h(DD, make_double2(0, 0));
        for (int i = 0; i < D; i++) h[i + i * D] = make_double2(p->dctype == DMFTGPU_DC_NOMINAL ? v : 0.0, 0.0);
        DG_CUDA(cudaMemcpyAsync(dc, h.data(), DD * sizeof(double2), cudaMemcpyHostToDevice, s));
        DG_CUDA(cudaStreamSynchronize(s));
    }
    // ---- SOLVER: proj_to_site, IPT or SCGF2, spin average, NumMatrix
    k_sub<<<dg_ceil_div(DD, 64), 64, 0, s>>>(DD, himp, dc, hdc);
    DG_LAUNCH(ctx, "k_sub");
    DG_TRY(dg_status_reset(ctx));
    int loops = 0;
    if (p->solver == DMFTGPU_SOLVER_IPT) {
        DG_TRY(dg_ipt_dev(ctx, D, Nf, p->ntau, L->beta, p->U, *mu, hdc, dW, dN, Ul, seimp, dGI, occ));
    } else {
        // Gw_strong: the lattice G_loc of the last TightBinding call starts the SCGF2 loop
        DG_CUDA(cudaMemcpyAsync(dGI, dG, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_TRY(dg_scgf2_dev(ctx, D, Nf, p->ntau, L->beta, *mu, p->mixing, hdc, dW, dGI, Ul,
                            p->scgf_max_iter > 0 ? p->scgf_max_iter : 2000, seimp, &loops));
        DG_CUDA(cudaMemcpyAsync(occ, dN, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    }
    if (p->magnetism == 0) {
        k_spin_average<<<dg_ceil_div((long long)(Nf + 6) * (D / 2), 128), 128, 0, s>>>(D, Nf + 5, seimp, occ);
        DG_LAUNCH(ctx, "k_spin_average");
    }
    DG_CUDA(cudaMemcpyAsync(dN, occ, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    DG_CUDA(cudaMemcpyAsync(nm_imp, occ, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    k_se_combine<<<dg_ceil_div((long long)Nf * DD, 256), 256, 0, s>>>(Nf, D, seimp, dc, seout);
    DG_LAUNCH(ctx, "k_se_combine");
    // ---- Pulay mixing of SelfEnergy_w (w < N_freq)
    if (!ctx->pulay) ctx->pulay = new DgPulay();
    if (iteration <= 1) *ctx->pulay = DgPulay();
    DG_TRY(dg_pulay_mixing(ctx, *ctx->pulay, "pulay", (long long)Nf * DD, dSE, seout, p->mixing, iteration));
    DG_CUDA(cudaMemcpyAsync(dSE, seout, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    if (code) return code;
    // ---- TightBinding: mu search, GreenFtn_w, Construct_hyb_delta
    double mu_new = *mu;
    int nev = 0;
    DG_TRY(dmftgpu_adjust_mu(ctx, L, hk, selfe, *mu, 1.0, p->n_electrons, &mu_new, &nev, dflags));
    *mu = mu_new;
    DG_TRY(dmftgpu_greenftn_w(ctx, L, hk, selfe, *mu, gloc, nullptr, nummat, dflags & ~DMFTGPU_NEWTON));
    std::vector<int> orb(D);
    for (int i = 0; i < D; i++) orb[i] = i;
    DG_TRY(dmftgpu_hyb_delta(ctx, D, orb.data(), Nf, L->beta, D, selfe, gloc, (const double *)himp, *mu, weiss,
                             DMFTGPU_DEVICE_PTRS));
    // ---- dmft_scf_check residuals
    k_scf_terms<<<dg_ceil_div(Nf, 128), 128, 0, s>>>(Nf, D, dGI, dG, rd, rd + Nf);
    DG_LAUNCH(ctx, "k_scf_terms");
    std::vector<double> h(2 * (size_t)Nf);
    std::vector<double2> nl(DD), ni(DD);
    DG_CUDA(cudaMemcpyAsync(h.data(), rd, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    DG_CUDA(cudaMemcpyAsync(nl.data(), dN, DD * sizeof(double2), cudaMemcpyDeviceToHost, s));
    DG_CUDA(cudaMemcpyAsync(ni.data(), nm_imp, DD * sizeof(double2), cudaMemcpyDeviceToHost, s));
    DG_CUDA(cudaStreamSynchronize(s));
    double GwNorm = 1e-10, GwlowNorm = 1e-10, GwRD = 0, GwRD_low = 0, GwRD_max = 0;
    const double wcut = std::min(p->U, 3.0);
    for (int n = 0; n < Nf; n++) {
        const double wn = DG_PI * (2. * n + 1) / L->beta;
        if (wn < wcut) {
            GwRD_low += h[n];
            GwlowNorm += h[Nf + n];
        }
        GwRD += h[n];
        GwNorm += h[Nf + n];
        const double r = h[n] / (h[Nf + n] + 1e-10);
        if (r > GwRD_max) GwRD_max = r;
    }
    double dn = 0, nn = 0;
    for (int e = 0; e < DD; e++) {
        dn += (nl[e].x - ni[e].x) * (nl[e].x - ni[e].x) + (nl[e].y - ni[e].y) * (nl[e].y - ni[e].y);
        nn += nl[e].x * nl[e].x + nl[e].y * nl[e].y;
    }
    resid[0] = std::sqrt(GwRD / GwNorm);
    resid[1] = std::sqrt(GwRD_low / GwlowNorm);
    resid[2] = std::sqrt(GwRD_max);
    resid[3] = std::sqrt(dn) / std::sqrt(nn);
    resid[4] = loops;
    return DMFTGPU_OK;
}
