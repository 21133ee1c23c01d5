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
#include <algorithm>
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

// out[n] = B^H X[n] B (to_solver) or B X[n] B^H (back), n < nmat, every D x D column-major; one thread per entry
__global__ void k_rotate(int nmat, int D, const double2 *__restrict__ B, const double2 *__restrict__ X,
                         double2 *__restrict__ out, int to_solver) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t DD = (size_t)D * D;
    if (t >= (long long)nmat * DD) return;
    const int n = (int)(t / DD), e = (int)(t % DD), i = e % D, j = e / D;
    const double2 *x = X + (size_t)n * DD;
    double2 acc = cmk(0, 0);
    for (int b = 0; b < D; b++) {
        double2 xb = cmk(0, 0);  // (X B)(:, j)_a or (X B^H)(:, j)_a, contracted with row i of the left factor below
        for (int a = 0; a < D; a++) {
            const double2 l = to_solver ? cconj(DG_AT(B, D, a, i)) : DG_AT(B, D, i, a);  // (B^H)_ia or B_ia
            xb = cfma(l, DG_AT(x, D, a, b), xb);
        }
        const double2 r = to_solver ? DG_AT(B, D, b, j) : cconj(DG_AT(B, D, j, b));  // B_bj or (B^H)_bj
        acc = cfma(xb, r, acc);
    }
    out[t] = acc;
}

// Hermitian eigen-decomposition of a small matrix on the host by cyclic Jacobi rotations: eigenvalues ascending
// (the order of Eigen's SelfAdjointEigenSolver), V column-major with a fixed gauge: each eigenvector's first
// component of largest modulus is made real and positive.
void host_heig(int n, std::vector<double2> A, std::vector<double> &w, std::vector<double2> &V) {
    auto at = [&](std::vector<double2> &M, int i, int j) -> double2 & { return M[i + (size_t)j * n]; };
    V.assign((size_t)n * n, make_double2(0, 0));
    for (int i = 0; i < n; i++) at(V, i, i) = make_double2(1, 0);
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += cabs2(at(A, p, q));
        if (off < 1e-30) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                const double2 apq = at(A, p, q);
                const double mag = std::sqrt(cabs2(apq));
                if (mag < 1e-300) continue;
                const double2 ph = cmk(apq.x / mag, apq.y / mag);  // e^{i phi}
                const double tau = (at(A, q, q).x - at(A, p, p).x) / (2 * mag);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
                const double c = 1 / std::sqrt(1 + t * t), sn = t * c;
                // J = [[c, s e^{i phi}], [-s e^{-i phi}, c]] on columns (p, q); A <- J^H A J, V <- V J
                for (int k = 0; k < n; k++) {  // columns p, q of A and V
                    const double2 akp = at(A, k, p), akq = at(A, k, q);
                    at(A, k, p) = csub(cscale(akp, c), cscale(cmul(akq, cconj(ph)), sn));
                    at(A, k, q) = cadd(cscale(akq, c), cscale(cmul(akp, ph), sn));
                    const double2 vkp = at(V, k, p), vkq = at(V, k, q);
                    at(V, k, p) = csub(cscale(vkp, c), cscale(cmul(vkq, cconj(ph)), sn));
                    at(V, k, q) = cadd(cscale(vkq, c), cscale(cmul(vkp, ph), sn));
                }
                for (int k = 0; k < n; k++) {  // rows p, q of A
                    const double2 apk = at(A, p, k), aqk = at(A, q, k);
                    at(A, p, k) = csub(cscale(apk, c), cscale(cmul(aqk, ph), sn));
                    at(A, q, k) = cadd(cscale(aqk, c), cscale(cmul(apk, cconj(ph)), sn));
                }
            }
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return at(A, x, x).x < at(A, y, y).x; });
    w.resize(n);
    std::vector<double2> Vs((size_t)n * n);
    for (int j = 0; j < n; j++) {
        w[j] = at(A, ord[j], ord[j]).x;
        int big = 0;
        double bm = -1;
        for (int i = 0; i < n; i++)
            if (cabs2(at(V, i, ord[j])) > bm * (1 + 1e-12)) {
                bm = cabs2(at(V, i, ord[j]));
                big = i;
            }
        const double2 v = at(V, big, ord[j]);
        const double m = std::sqrt(cabs2(v));
        const double2 g = cmk(v.x / m, -v.y / m);  // conj(v)/|v|
        for (int i = 0; i < n; i++) Vs[i + (size_t)j * n] = cmul(at(V, i, ord[j]), g);
    }
    V = Vs;
}

double2 *buf2(dmftgpu_ctx *ctx, const char *name, size_t count) {
    return (double2 *)dg_buf(ctx, name, count * sizeof(double2));
}

}  // namespace

namespace {

// What every SOLVER call of one iteration shares
struct DmftSolve {
    const dmftgpu_dmft_params *p;
    int D, Nf, DD;
    double beta;
    const DgUList *Ul;
    const double2 *himp;  // k average of the correlated block of H(k)
};

// SOLVER of the loop body (src/SOLVER.cpp:105-502, src/dmft_main.cpp:489-525) from (weiss, nm_in, mu): the double
// counting from nm_in (dc_for_dmft), proj_to_site (H_imp - DC and, with basis_switch, the rotation to the solver
// basis; the basis is computed when *basis_ready is false and reused otherwise), IPT or SCGF2 (started from gstart),
// the rotation back, the magnetism == 0 spin average.  Outputs: seout[Nf] = SE_out - DC, gimp[Nf+5], occ (IPT's
// occupation; nm_in for SCGF2), dc, *loops.
int dmft_solver(dmftgpu_ctx *ctx, const DmftSolve &S, const double2 *weiss, const double2 *nm_in, double mu,
                const double2 *gstart, double2 *seout, double2 *gimp, double2 *occ, double2 *dc, double2 *basis,
                bool *basis_ready, int *loops) {
    const dmftgpu_dmft_params *p = S.p;
    const int D = S.D, Nf = S.Nf, DD = S.DD;
    cudaStream_t s = ctx->stream;
    double2 *hdc = buf2(ctx, "dmft.hdc", DD), *seimp = buf2(ctx, "dmft.seimp", (size_t)(Nf + 5) * DD);
    if (!hdc || !seimp) return DMFTGPU_NOMEM;
    {
        // dc_for_dmft from the NumMatrix of the last TightBinding (the state this iteration starts from)
        if ((p->dctype & 0xff) == DMFTGPU_DC_SIGMA0)
            return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: sigma0 double counting needs dmftgpu_double_counting");
        std::vector<double2> nm(DD), h(DD, make_double2(0, 0));
        DG_CUDA(cudaMemcpyAsync(nm.data(), nm_in, DD * sizeof(double2), cudaMemcpyDeviceToHost, s));
        DG_CUDA(cudaStreamSynchronize(s));
        const int st = dmftgpu_double_counting(p->dctype, 1, D, p->U, p->Uprime, p->J, p->nominal_charge,
                                               (const double *)nm.data(), nullptr, 0, (double *)h.data());
        if (st) return dg_fail(ctx, st, "dmft_iteration: double counting");
        DG_CUDA(cudaMemcpyAsync(dc, h.data(), DD * sizeof(double2), cudaMemcpyHostToDevice, s));
        DG_CUDA(cudaStreamSynchronize(s));
    }
    k_sub<<<dg_ceil_div(DD, 64), 64, 0, s>>>(DD, S.himp, dc, hdc);
    DG_LAUNCH(ctx, "k_sub");
    // impurityBasisSwitch (proj_to_site, src/SOLVER.cpp:541-595): H_imp - DC, Delta and NumMatrix go to the solver
    // basis B; Sigma and G_imp (w < N_freq) and the occupation come back (src/SOLVER.cpp:426-434)
    const double2 *sH = hdc, *sW = weiss, *sN = nm_in;
    const int rgrid = 128;
    if (p->basis_switch) {
        if (!*basis_ready) {
            std::vector<double2> hh(DD), d0(DD), Bh(DD);
            DG_CUDA(cudaMemcpyAsync(hh.data(), hdc, DD * sizeof(double2), cudaMemcpyDeviceToHost, s));
            DG_CUDA(cudaMemcpyAsync(d0.data(), weiss, DD * sizeof(double2), cudaMemcpyDeviceToHost, s));
            DG_CUDA(cudaStreamSynchronize(s));
            DG_TRY(dmftgpu_impurity_basis(D, p->magnetism, (const double *)hh.data(), (const double *)d0.data(),
                                          (double *)Bh.data()));
            DG_CUDA(cudaMemcpyAsync(basis, Bh.data(), DD * sizeof(double2), cudaMemcpyHostToDevice, s));
            *basis_ready = true;
        }
        double2 *hR = buf2(ctx, "dmft.hrot", DD), *wR = buf2(ctx, "dmft.wrot", (size_t)Nf * DD);
        double2 *nR = buf2(ctx, "dmft.nrot", DD);
        if (!hR || !wR || !nR) return DMFTGPU_NOMEM;
        k_rotate<<<dg_ceil_div((long long)DD, rgrid), rgrid, 0, s>>>(1, D, basis, hdc, hR, 1);
        k_rotate<<<dg_ceil_div((long long)Nf * DD, rgrid), rgrid, 0, s>>>(Nf, D, basis, weiss, wR, 1);
        k_rotate<<<dg_ceil_div((long long)DD, rgrid), rgrid, 0, s>>>(1, D, basis, nm_in, nR, 1);
        DG_LAUNCH(ctx, "k_rotate");
        sH = hR;
        sW = wR;
        sN = nR;
    }
    *loops = 0;
    if (p->solver == DMFTGPU_SOLVER_IPT) {
        DG_TRY(dg_ipt_dev(ctx, D, Nf, p->ntau, S.beta, p->U, mu, sH, sW, sN, *S.Ul, seimp, gimp, occ));
    } else {
        // Gw_strong: SCGF2 starts from gstart (the lattice G_loc of the last TightBinding call, as given, unrotated)
        if (gstart != gimp)
            DG_CUDA(cudaMemcpyAsync(gimp, gstart, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_TRY(dg_scgf2_dev(ctx, D, Nf, p->ntau, S.beta, mu, p->mixing, sH, sW, gimp, *S.Ul,
                            p->scgf_max_iter > 0 ? p->scgf_max_iter : 2000, seimp, loops));
        DG_CUDA(cudaMemcpyAsync(occ, sN, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    }
    if (p->basis_switch) {
        double2 *tmp = buf2(ctx, "dmft.rtmp", (size_t)Nf * DD);
        if (!tmp) return DMFTGPU_NOMEM;
        k_rotate<<<dg_ceil_div((long long)Nf * DD, rgrid), rgrid, 0, s>>>(Nf, D, basis, seimp, tmp, 0);
        DG_CUDA(cudaMemcpyAsync(seimp, tmp, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        k_rotate<<<dg_ceil_div((long long)Nf * DD, rgrid), rgrid, 0, s>>>(Nf, D, basis, gimp, tmp, 0);
        DG_CUDA(cudaMemcpyAsync(gimp, tmp, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        k_rotate<<<dg_ceil_div((long long)DD, rgrid), rgrid, 0, s>>>(1, D, basis, occ, tmp, 0);
        DG_CUDA(cudaMemcpyAsync(occ, tmp, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_LAUNCH(ctx, "k_rotate");
    }
    if (p->magnetism == 0) {
        k_spin_average<<<dg_ceil_div((long long)(Nf + 6) * (D / 2), 128), 128, 0, s>>>(D, Nf + 5, seimp, occ);
        DG_LAUNCH(ctx, "k_spin_average");
    }
    k_se_combine<<<dg_ceil_div((long long)Nf * DD, 256), 256, 0, s>>>(Nf, D, seimp, dc, seout);
    DG_LAUNCH(ctx, "k_se_combine");
    return DMFTGPU_OK;
}

// NumMatrix moved along a G_loc tangent: out = nm + h (1/beta) sum_{n < Nf} (dG_n + dG_n^H), the Matsubara sum's
// first-order change without the tail beyond N_freq (one block per entry, fixed-order reduction)
__global__ void k_nummat_tangent(int nfreq, int D, double beta, double h, const double2 *__restrict__ dG,
                                 const double2 *__restrict__ nm, double2 *__restrict__ out) {
    __shared__ double2 red[128];
    const int e = blockIdx.x, a = e % D, b = e / D, DD = D * D;
    double2 s = cmk(0, 0);
    for (int n = threadIdx.x; n < nfreq; n += blockDim.x)
        s = cadd(s, cadd(dG[(size_t)n * DD + a + b * D], cconj(dG[(size_t)n * DD + b + a * D])));
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + k]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[e] = cadd(nm[e], cscale(red[0], h / beta));
}

// One Newton-Krylov step of the self-energy mixer: with x = SelfEnergy_w, Phi(x) = SE_out of SOLVER on the
// TightBinding state of x and F = Phi(x) - x, solve (J_Phi - I) dx = -F by GMRES and return x + dx in xnew.
// J_Phi v: the lattice part exactly, by the tangent kernel (dmftgpu_gloc_jvp at fixed mu) with mu's first-order
// change from the electron count (dN/dSigma.v by a directional difference of the N(mu) pass, dN/dmu from the
// derivative pass); NumMatrix along the same tangent; then the small D x D stages (Construct_hyb_delta and SOLVER)
// by a directional difference at the tangent point.  SCGF2's perturbed solves start from the unperturbed G_imp.
int dmft_newton_step(dmftgpu_ctx *ctx, const dmftgpu_lattice *L, const double *hk, const DmftSolve &S, int lflags,
                     const double2 *x, const double2 *seout0, const double2 *gimp0, const double2 *weiss,
                     const double2 *nm, const double2 *gloc, double mu, double2 *basis, bool basis_ready,
                     double2 *xnew, int *krylov, double *relres) {
    const dmftgpu_dmft_params *p = S.p;
    const int D = S.D, Nf = S.Nf, DD = S.DD;
    const long long n = (long long)Nf * DD;
    cudaStream_t s = ctx->stream;
    double2 *b = buf2(ctx, "nk.b", n), *xp = buf2(ctx, "nk.xp", n), *dG = buf2(ctx, "nk.dG", n);
    double2 *Gp = buf2(ctx, "nk.Gp", n), *Wp = buf2(ctx, "nk.Wp", n), *nmp = buf2(ctx, "nk.nmp", DD);
    double2 *sop = buf2(ctx, "nk.sop", n), *gip = buf2(ctx, "nk.gip", (size_t)(Nf + 5) * DD);
    double2 *occp = buf2(ctx, "nk.occp", DD), *dcp = buf2(ctx, "nk.dcp", DD), *dx = buf2(ctx, "nk.dx", n);
    if (!b || !xp || !dG || !Gp || !Wp || !nmp || !sop || !gip || !occp || !dcp || !dx) return DMFTGPU_NOMEM;
    // b = -F = x - Phi(x)
    DG_CUDA(cudaMemcpyAsync(b, x, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    DG_TRY(dg_vaxpby(ctx, n, -1.0, seout0, 1.0, b));
    double N0 = 0, dNdmu = 0, dummy = 0, xx = 0;
    // N0 from the same pass as the perturbed N(mu) below (the derivative pass may take another kernel path, whose
    // rounding would then enter the directional difference)
    DG_TRY(dmftgpu_nele(ctx, L, hk, (const double *)x, mu, &N0, nullptr, lflags));
    DG_TRY(dmftgpu_nele(ctx, L, hk, (const double *)x, mu, &dummy, &dNdmu, lflags));
    if (!(dNdmu > 0)) return dg_fail(ctx, DMFTGPU_NONCONVERGED, "dmft_iteration: dN/dmu <= 0 at the Newton point");
    DG_TRY(dg_vdot(ctx, n, x, x, &xx));
    // directional-difference step: SCGF2's own stopping test leaves ~1e-6 of noise in its solution
    const double eps = p->solver == DMFTGPU_SOLVER_SC2PT ? 1e-4 : 1e-6;
    const double scgf_prev = ctx->scgf_prev_norm;
    std::vector<int> orb(D);
    for (int i = 0; i < D; i++) orb[i] = i;
    auto apply = [&](const double2 *v, double2 *Av) -> int {
        double vv = 0;
        DG_TRY(dg_vdot(ctx, n, v, v, &vv));
        const double h = eps * std::max(1.0, std::sqrt(xx)) / std::sqrt(vv);
        DG_CUDA(cudaMemcpyAsync(xp, x, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_TRY(dg_vaxpby(ctx, n, h, v, 1.0, xp));
        double Np = 0;
        DG_TRY(dmftgpu_nele(ctx, L, hk, (const double *)xp, mu, &Np, nullptr, lflags));
        const double dmu = -(Np - N0) / h / dNdmu;
        DG_TRY(dmftgpu_gloc_jvp(ctx, L, hk, (const double *)x, mu, (const double *)v, dmu, (double *)dG,
                                DMFTGPU_DEVICE_PTRS));
        DG_CUDA(cudaMemcpyAsync(Gp, gloc, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_TRY(dg_vaxpby(ctx, n, h, dG, 1.0, Gp));
        k_nummat_tangent<<<DD, 128, 0, s>>>(Nf, D, S.beta, h, dG, nm, nmp);
        DG_LAUNCH(ctx, "k_nummat_tangent");
        const double mup = mu + h * dmu;
        DG_TRY(dmftgpu_hyb_delta(ctx, D, orb.data(), Nf, S.beta, D, (const double *)xp, (const double *)Gp,
                                 (const double *)S.himp, mup, (double *)Wp, DMFTGPU_DEVICE_PTRS));
        bool ready = basis_ready;
        int loops = 0;
        DG_TRY(dmft_solver(ctx, S, Wp, nmp, mup, gimp0, sop, gip, occp, dcp, basis, &ready, &loops));
        ctx->scgf_prev_norm = scgf_prev;
        int code = 0;
        DG_TRY(dg_status_read(ctx, &code));
        if (code) return code;
        // Av = (Phi(x + h v) - Phi(x)) / h - v
        DG_CUDA(cudaMemcpyAsync(Av, sop, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_TRY(dg_vaxpby(ctx, n, -1.0 / h, seout0, 1.0 / h, Av));
        DG_TRY(dg_vaxpby(ctx, n, -1.0, v, 1.0, Av));
        return DMFTGPU_OK;
    };
    const int m = p->krylov_dim > 0 ? p->krylov_dim : 8;
    const double tol = p->krylov_tol > 0 ? p->krylov_tol : 1e-3;
    DG_TRY(dg_gmres(ctx, n, b, m, tol, apply, dx, krylov, relres));
    DG_CUDA(cudaMemcpyAsync(xnew, x, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    DG_TRY(dg_vaxpby(ctx, n, 1.0, dx, 1.0, xnew));
    return DMFTGPU_OK;
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
    if (p->mixer != DMFTGPU_MIXER_PULAY && p->mixer != DMFTGPU_MIXER_NEWTON_KRYLOV)
        return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: mixer");
    if (p->krylov_dim < 0 || p->krylov_dim > 64 || p->krylov_tol < 0 || p->newton_start < 0)
        return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: Newton-Krylov settings");
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
    double2 *himp = buf2(ctx, "dmft.himp", DD), *dc = buf2(ctx, "dmft.dc", DD);
    double2 *seout = buf2(ctx, "dmft.seout", (size_t)Nf * DD);
    double2 *occ = buf2(ctx, "dmft.occ", DD), *nm_imp = buf2(ctx, "dmft.nmimp", DD);
    double2 *basis = buf2(ctx, "dmft.basis", DD);
    double *rd = (double *)dg_buf(ctx, "dmft.rd", 2 * (size_t)Nf * sizeof(double));
    int *dhartr = (int *)dg_buf(ctx, "dmft.hartr", D * sizeof(int));
    if (!himp || !dc || !seout || !occ || !nm_imp || !basis || !rd || !dhartr) return DMFTGPU_NOMEM;
    {
        std::vector<int> h(D);
        for (int i = 0; i < D; i++) h[i] = L->hartr ? L->hartr[i] : i;
        for (int i = 0; i < D; i++)
            if (h[i] < 0 || h[i] >= L->n) return dg_fail(ctx, DMFTGPU_BADARG, "dmft_iteration: bad HartrIndex");
        DG_CUDA(cudaMemcpyAsync(dhartr, h.data(), D * sizeof(int), cudaMemcpyHostToDevice, s));
        DG_CUDA(cudaStreamSynchronize(s));
    }
    // impurity_site_Hamiltonian (k average of H_PP)
    k_himp<<<DD, 256, 0, s>>>(L->nk, L->n, D, dhartr, (const double2 *)hk, himp);
    DG_LAUNCH(ctx, "k_himp");
    DG_TRY(dg_status_reset(ctx));
    // ---- SOLVER: proj_to_site, IPT or SCGF2, spin average
    const DmftSolve S{p, D, Nf, DD, L->beta, &Ul, himp};
    bool basis_ready = false;
    int loops = 0;
    DG_TRY(dmft_solver(ctx, S, dW, dN, *mu, dG, seout, dGI, occ, dc, basis, &basis_ready, &loops));
    DG_CUDA(cudaMemcpyAsync(nm_imp, occ, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    if (code) return code;
    // ---- the self-energy mixer: Pulay (src/dmft_main.cpp:529-533) or a Newton-Krylov step
    if (!ctx->pulay) ctx->pulay = new DgPulay();
    if (iteration <= 1) {
        *ctx->pulay = DgPulay();  // pulayMixing(2, 5, ...) of dmft_main (src/dmft_main.cpp:342) unless set
        if (p->pulay_history > 0) ctx->pulay->hist = p->pulay_history;
        if (p->pulay_start > 0) ctx->pulay->start = p->pulay_start;
    }
    ctx->nk_krylov = 0;
    ctx->nk_relres = 0;
    {
        // the fixed-point residual |SE_out - SelfEnergy_w| / |SelfEnergy_w| that both mixers reduce
        double2 *fr = buf2(ctx, "dmft.fres", (size_t)Nf * DD);
        if (!fr) return DMFTGPU_NOMEM;
        DG_CUDA(cudaMemcpyAsync(fr, seout, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        DG_TRY(dg_vaxpby(ctx, (long long)Nf * DD, -1.0, dSE, 1.0, fr));
        double ff = 0, xx = 0;
        DG_TRY(dg_vdot(ctx, (long long)Nf * DD, fr, fr, &ff));
        DG_TRY(dg_vdot(ctx, (long long)Nf * DD, dSE, dSE, &xx));
        ctx->mix_resid = xx > 0 ? std::sqrt(ff / xx) : std::sqrt(ff);
    }
    const int nstart = p->newton_start > 0 ? p->newton_start : 3;
    if (p->mixer == DMFTGPU_MIXER_NEWTON_KRYLOV && iteration >= nstart) {
        // the Jacobian is taken at the state this call starts from (NumMatrix of its TightBinding, not IPT's)
        double2 *nm_tb = buf2(ctx, "dmft.nmtb", DD), *xnew = buf2(ctx, "dmft.xnew", (size_t)Nf * DD);
        if (!nm_tb || !xnew) return DMFTGPU_NOMEM;
        DG_CUDA(cudaMemcpyAsync(nm_tb, dN, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        const int lflags = DMFTGPU_DEVICE_PTRS | (flags & (DMFTGPU_MIXED | DMFTGPU_NO_TENSOR));
        DG_TRY(dmft_newton_step(ctx, L, hk, S, lflags, dSE, seout, dGI, dW, nm_tb, dG, *mu, basis, basis_ready, xnew,
                                &ctx->nk_krylov, &ctx->nk_relres));
        DG_CUDA(cudaMemcpyAsync(dSE, xnew, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    } else {
        DG_TRY(dg_pulay_mixing(ctx, *ctx->pulay, "pulay", (long long)Nf * DD, dSE, seout, p->mixing, iteration));
        DG_CUDA(cudaMemcpyAsync(dSE, seout, (size_t)Nf * DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    }
    DG_CUDA(cudaMemcpyAsync(dN, occ, DD * sizeof(double2), cudaMemcpyDeviceToDevice, s));
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

// dc_for_dmft (src/dmft_main.cpp:593-707), host arithmetic; see include/dmftgpu.h
extern "C" int dmftgpu_double_counting(int dctype, int natoms, int nso, double U, double Uprime, double J,
                                       double nominal_charge, const double *nummat, const double *sigma0, int initial,
                                       double *dc) {
    const int base = dctype & 0xff;
    const bool uprime = (dctype & DMFTGPU_DC_UPRIME) != 0;
    if (natoms < 1 || nso < 1 || !dc || base < DMFTGPU_DC_NONE || base > DMFTGPU_DC_SIGMA0) return DMFTGPU_BADARG;
    const bool sigma0_step = base == DMFTGPU_DC_SIGMA0 && initial;
    if ((base == DMFTGPU_DC_FLL || base == DMFTGPU_DC_AMF || (base == DMFTGPU_DC_SIGMA0 && !initial)) && !nummat)
        return DMFTGPU_BADARG;
    if (sigma0_step && !sigma0) return DMFTGPU_BADARG;
    if ((base == DMFTGPU_DC_NOMINAL || base == DMFTGPU_DC_FLL || base == DMFTGPU_DC_SIGMA0) && (nso % 2))
        return DMFTGPU_BADARG;  // spin-orbital pairs (i, i+1)
    const int N = natoms * nso;
    auto at = [&](const double *m, int i, int j) { return make_double2(m[2 * (i + (size_t)j * N)], m[2 * (i + (size_t)j * N) + 1]); };
    std::vector<double2> out((size_t)N * N, make_double2(0, 0));
    double averU = (nso * U + nso * (nso - 1) * Uprime) / (double)(nso * nso);
    const double averJ = J;
    for (int a = 0; a < natoms; a++) {
        const int o = a * nso;
        double up = 0, down = 0;
        if (nummat)
            for (int n = 0; n < nso; n += 2) {
                up += at(nummat, o + n, o + n).x;
                if (n + 1 < nso) down += at(nummat, o + n + 1, o + n + 1).x;
            }
        auto set = [&](int i, int j, double2 v) { out[(o + i) + (size_t)(o + j) * N] = v; };
        if (sigma0_step) {
            double tr = 0;
            for (int i = 0; i < nso; i++) tr += at(sigma0, o + i, o + i).x;
            const double temp = tr / nso;
            for (int i = 0; i < nso; i++)
                for (int j = 0; j < nso; j++) {
                    double2 v = at(dc, o + i, o + j);
                    if (i == j) v.x += temp;
                    set(i, j, v);
                }
        } else if (base == DMFTGPU_DC_FLL || base == DMFTGPU_DC_SIGMA0) {
            const double u = uprime ? Uprime : averU;
            for (int i = 0; i < nso; i += 2) {
                set(i, i, make_double2(u * (down + up - 0.5) - averJ * (up - 0.5), 0));
                set(i + 1, i + 1, make_double2(u * (down + up - 0.5) - averJ * (down - 0.5), 0));
            }
        } else if (base == DMFTGPU_DC_AMF) {
            const double n0 = (down + down) / nso;  // the reference's expression (src/dmft_main.cpp:653)
            for (int i = 0; i < nso; i++)
                set(i, i, make_double2(averU * n0 * (nso - 1) - averJ * n0 * (nso / 2 - 1), 0));
        } else if (base == DMFTGPU_DC_NOMINAL) {
            const double u = uprime ? Uprime : averU;
            const double v = u * (nominal_charge - 0.5) - averJ * (nominal_charge / 2.0 - 0.5);
            for (int i = 0; i < nso; i += 2) {
                set(i, i, make_double2(v, 0));
                set(i + 1, i + 1, make_double2(v, 0));
            }
        }
    }
    std::memcpy(dc, out.data(), out.size() * sizeof(double2));
    return DMFTGPU_OK;
}

// proj_to_site's solver basis (src/SOLVER.cpp:541-586), host arithmetic; see include/dmftgpu.h
extern "C" int dmftgpu_impurity_basis(int dim, int magnetism, const double *himp, const double *delta0,
                                      double *basis) {
    if (dim < 1 || dim > 64 || !himp || !delta0 || !basis) return DMFTGPU_BADARG;
    const int n = dim;
    auto H = [&](int i, int j) { return make_double2(himp[2 * (i + (size_t)j * n)], himp[2 * (i + (size_t)j * n) + 1]); };
    auto W = [&](int i, int j) { return make_double2(delta0[2 * (i + (size_t)j * n)], delta0[2 * (i + (size_t)j * n) + 1]); };
    std::vector<double2> B((size_t)n * n, make_double2(0, 0));
    double imn = 0;
    for (int e = 0; e < n * n; e++) imn += himp[2 * e + 1] * himp[2 * e + 1];
    std::vector<double> w;
    std::vector<double2> V;
    if (std::sqrt(imn) < 1e-5 && (magnetism == 0 || magnetism == 1) && n % 2 == 0) {
        // the spin-averaged real problem: Re[(Delta(iw_0) + H_imp) averaged over the spin pair, Hermitian part]
        const int h = n / 2;
        std::vector<double2> M((size_t)h * h);
        for (int i = 0; i < n; i += 2)
            for (int j = 0; j < n; j += 2)
                M[i / 2 + (size_t)(j / 2) * h] = cscale(cadd(cadd(W(i, j), W(i + 1, j + 1)), cadd(H(i, j), H(i + 1, j + 1))), 0.5);
        std::vector<double2> R((size_t)h * h);
        for (int i = 0; i < h; i++)
            for (int j = 0; j < h; j++)
                R[i + (size_t)j * h] = make_double2(0.5 * (M[i + (size_t)j * h].x + M[j + (size_t)i * h].x), 0.0);
        host_heig(h, R, w, V);
        for (int i = 0; i < n; i += 2)
            for (int j = 0; j < n; j += 2) {
                const double v = V[i / 2 + (size_t)(j / 2) * h].x;
                B[i + (size_t)j * n] = make_double2(v, 0);
                B[(i + 1) + (size_t)(j + 1) * n] = make_double2(v, 0);
            }
    } else {
        // eigenbasis of H_imp, then of the real part of (H_imp + the Hermitian part of Delta(iw_0)) in it
        std::vector<double2> Hm((size_t)n * n);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) Hm[i + (size_t)j * n] = H(i, j);
        std::vector<double2> V1;
        host_heig(n, Hm, w, V1);
        std::vector<double2> X((size_t)n * n), T((size_t)n * n, make_double2(0, 0));
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                X[i + (size_t)j * n] = cadd(H(i, j), cscale(cadd(W(i, j), cconj(W(j, i))), 0.5));
        for (int i = 0; i < n; i++)  // T = V1^H X V1, real part
            for (int j = 0; j < n; j++) {
                double2 acc = make_double2(0, 0);
                for (int a = 0; a < n; a++)
                    for (int b = 0; b < n; b++)
                        acc = cadd(acc, cmul(cmul(cconj(V1[a + (size_t)i * n]), X[a + (size_t)b * n]), V1[b + (size_t)j * n]));
                T[i + (size_t)j * n] = make_double2(acc.x, 0.0);
            }
        host_heig(n, T, w, V);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double2 acc = make_double2(0, 0);
                for (int a = 0; a < n; a++) acc = cadd(acc, cmul(V1[i + (size_t)a * n], make_double2(V[a + (size_t)j * n].x, 0.0)));
                B[i + (size_t)j * n] = acc;
            }
    }
    std::memcpy(basis, B.data(), B.size() * sizeof(double2));
    return DMFTGPU_OK;
}

extern "C" int dmftgpu_mixer_stats(dmftgpu_ctx *ctx, int *krylov, double *relres, double *residual) {
    if (!ctx || !krylov || !relres || !residual) return DMFTGPU_BADARG;
    *krylov = ctx->nk_krylov;
    *relres = ctx->nk_relres;
    *residual = ctx->mix_resid;
    return DMFTGPU_OK;
}
