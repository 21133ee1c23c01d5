/*
 * dmftgpu.h -- C ABI of libdmftgpu, the GB300 (sm_103a) implementation of DMFTpack's DMFT
 * self-consistency hot path.  Plain pointers, sizes and an opaque context; no C++ or torch types.
 *
 * Data conventions (identical to the reference's in-memory Eigen data, so a shim can pass .data()):
 *   - complex numbers are interleaved doubles (re, im)  == std::complex<double> / Eigen::MatrixXcd;
 *   - matrices are column-major (element (i,j) at [i + j*rows]) == Eigen's default storage;
 *   - a std::vector<Eigen::MatrixXcd> of equal-size matrices becomes one contiguous stack;
 *   - index tables are row-major int32 ([row][col]).
 * Array arguments are host pointers unless DMFTGPU_DEVICE_PTRS is set in `flags`, in which case every
 * array argument (except the small int index tables, which are always host) is a device pointer and the
 * call only enqueues work on the context's stream.  Scalar outputs (nele, mu_out, counters) are always
 * host pointers.  Every entry point returns a DMFTGPU_* status; nothing aborts the process.
 *
 * Each entry point names the reference function (path within the DMFTpack repository, file:line) that it
 * replaces.  The globals the reference reads (beta, N_freq, N_tau, knum, NBAND, HartrIndex, ...) become
 * explicit arguments.
 */
#ifndef DMFTGPU_H
#define DMFTGPU_H
#ifdef __cplusplus
extern "C" {
#endif

enum {
    DMFTGPU_OK = 0,
    DMFTGPU_SINGULAR = 1,     /* a zero pivot (the reference would produce inf/nan silently) */
    DMFTGPU_NONCONVERGED = 2, /* iteration cap reached (mu search, Jacobi, SCGF2 loop) */
    DMFTGPU_NAN = 3,          /* NaN/Inf in a result the reference asserts finite */
    DMFTGPU_BADARG = 4,
    DMFTGPU_CAUSALITY = 5,    /* an eigenvalue of Im G or Im Delta has the wrong sign (reference: assert) */
    DMFTGPU_HERMITICITY = 6,  /* G(tau) or Sigma(tau) not Hermitian (reference: assert) */
    DMFTGPU_CUDA_ERROR = 7,
    DMFTGPU_NOMEM = 8,
    DMFTGPU_TIMEOUT = 9,      /* a bounded wait inside a tensor-core kernel ran out (the kernel freed its TMEM and
                                 returned; the context stays usable) */
    DMFTGPU_IO = 10           /* a restart file could not be opened, read or written */
};

#define DMFTGPU_DEVICE_PTRS 0x1 /* array arguments live in device memory */
#define DMFTGPU_MIXED 0x2       /* double-float (FP32-pair) arithmetic on the FP32 pipe: lattice sums and getStimp */
#define DMFTGPU_NEWTON 0x4      /* dmftgpu_adjust_mu: Newton steps on dN/dmu from the same pass */
#define DMFTGPU_EXPLICIT 0x8    /* lattice sums by explicit n x n inversion of every (k, iw) matrix, as the
                                   reference does (default: the exact correlated-block Schur form); FP64, or
                                   double-float with DMFTGPU_MIXED */
#define DMFTGPU_GRAPH 0x20     /* dmftgpu_greenftn_w_batched: replay the batched pass as one CUDA graph */
#define DMFTGPU_AUTOTUNE 0x40  /* dmftgpu_greenftn_w_batched: tune each Schur kernel's k chunking on first use */
#define DMFTGPU_NO_TENSOR 0x80 /* with DMFTGPU_MIXED: keep the contractions (H(k), the N(mu) pole sums) on the
                                  CUDA cores instead of the tensor cores */
#define DMFTGPU_DIRECT_DFT 0x10 /* iw <-> tau transforms by the reference's direct per-point sums (default: the
                                   same sums by FFT when N_tau is a power of two <= 8192) */

typedef struct dmftgpu_ctx dmftgpu_ctx;

/* The reference's lattice globals: NBAND (n), knum (nk), N_freq (nfreq), beta, NumCluster (ncl),
 * NumHartrOrbit_per_cluster (nh) and HartrIndex[ncl*nh] (src/tight_common.cpp:28-114, src/TB.h:7-35).
 * hartr is a host pointer; NULL means HartrIndex[i] = i (the layout downfolding_ftn leaves behind,
 * src/downfolding.cpp:69-79). */
typedef struct {
    int n;
    int nk;
    int nfreq;
    double beta;
    int ncl;
    int nh;
    const int *hartr;
} dmftgpu_lattice;

int dmftgpu_version(void);
/* Context: one CUDA device, one stream, grow-only device workspaces. */
int dmftgpu_create(dmftgpu_ctx **ctx, int device);
int dmftgpu_destroy(dmftgpu_ctx *ctx);
int dmftgpu_set_stream(dmftgpu_ctx *ctx, void *cuda_stream);
void *dmftgpu_get_stream(dmftgpu_ctx *ctx);
int dmftgpu_synchronize(dmftgpu_ctx *ctx);
const char *dmftgpu_last_error(dmftgpu_ctx *ctx);
/* Number of kernels this context has launched so far (for launch accounting in benchmarks). */
long long dmftgpu_launch_count(dmftgpu_ctx *ctx);
/* Kernel timing for benchmarks: while enabled, CUDA events on the context's stream bracket every launch of
 * the hot kernels ("k_gloc", ...); dmftgpu_kernel_time sums their durations since the last enable.
 * No counterpart in the reference (which prints clock() estimates, src/GreenFtn.cpp:306-307). */
int dmftgpu_timing(dmftgpu_ctx *ctx, int enable);
int dmftgpu_kernel_time(dmftgpu_ctx *ctx, const char *kernel, double *ms, int *count);

/* k mesh of TightBinding (src/TB.cpp:196-207): kmesh[nk][3], nk = kx*ky*kz, host output. */
int dmftgpu_kmesh(int kx, int ky, int kz, double *kmesh);

/* H(k) = sum_R t(R) exp(-i k.a R) (Construct_Hk_Sk, src/ConstructModelHamiltonian.cpp:66-77) on the
 * TightBinding k mesh.  rindex[nnz][5] = (Rx, Ry, Rz, i0, j0) and hr[nnz] complex are read_HR's H_Rindex
 * and H_RMatrix (src/read_TB_parm.cpp:6-76).  Output hk[nk][n][n]. */
int dmftgpu_hk(dmftgpu_ctx *ctx, int n, int nnz, const int *rindex, const double *hr, int kx, int ky, int kz,
               double *hk, int flags);

/* getAsymto_moments (src/FourierTransform.cpp:184-465): fw[nfreq][dim][dim] -> mom[4][dim][dim]
 * (m0 + m1/iw + m2/(iw)^2 + m3/(iw)^3), green_asym selects the m0=0, m1=I variant (:337-457). */
int dmftgpu_moments(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, const double *fw, int green_asym,
                    double *mom, int flags);

/* GreenFtn_w (src/GreenFtn.cpp:142-422, declared src/TB.h:59-61): hk[nk][n][n] = H_k_inModelSpace,
 * sigma[nfreq][D][D] = SelfE_w (D = ncl*nh), mu.  Outputs gw[nfreq][D][D] (Gw), gwhf[nfreq][D][D]
 * (GwHF, may be NULL) and nummat[D][D] (the global NumMatrix). */
int dmftgpu_greenftn_w(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk, const double *sigma,
                       double mu, double *gw, double *gwhf, double *nummat, int flags);

/* GiwToNele (src/GreenFtn.cpp:513-635) in trace form; dnele (may be NULL) = dN/dmu. */
int dmftgpu_nele(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk, const double *sigma, double mu,
                 double *nele, double *dnele, int flags);

/* GreenFtn_w_adjust_mu (src/GreenFtn.cpp:66-139, declared src/TB.h:58): the reference's bracket +
 * bisection to |dmu| <= 1e-5, or with DMFTGPU_NEWTON a safeguarded Newton iteration to |N-n_target| <=
 * 1e-11 using dN/dmu from the same pass.  *mu_out = mu; *n_eval = number of N(mu) passes. */
int dmftgpu_adjust_mu(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk, const double *sigma,
                      double mu, double dmu, double n_target, double *mu_out, int *n_eval, int flags);

/* GreenFtn_w over a batch of independent lattice problems of ragged sizes (no counterpart in the reference;
 * one call per DMFT iteration of many systems).  Device pointers only (flags must contain DMFTGPU_DEVICE_PTRS),
 * HartrIndex the identity; the Schur form, FP64 or DMFTGPU_MIXED.  Arrays of nprob entries: lats, hk[i], sigma[i],
 * mu[i], gw[i], gwhf[i] (gwhf may be NULL), nummat[i] (as dmftgpu_greenftn_w).  DMFTGPU_GRAPH: the first call
 * with a given problem set runs eagerly and sizes the workspaces, the second captures the pass into a CUDA graph
 * and every later call with the same set (same sizes, pointers, mu and flags) replays it; DMFTGPU_AUTOTUNE
 * chooses each Schur kernel's CTAs per SM by timing on first use.  Each problem keeps its own workspaces in the
 * context. */
int dmftgpu_greenftn_w_batched(dmftgpu_ctx *ctx, int nprob, const dmftgpu_lattice *lats, const double *const *hk,
                               const double *const *sigma, const double *mu, double *const *gw, double *const *gwhf,
                               double *const *nummat, int flags);

/* The retarded lattice Green function on a real-energy grid E_n = e0 + n de, n < nE (retarded_GreenFtn2,
 * src/GreenFtn.cpp:425-466, summed over k as qs_spectra does, src/qs_spectra.cpp:99-130): with G(k, E) =
 * (E + mu + i eta - H(k) - Sigma(E))^-1 and sigma_e[nE][D][D] the self-energy on the grid,
 * gloc[nE][D][D] = (1/N_k) sum_k G_PP(k, E) and trace[nE] (complex) = (1/N_k) sum_k Tr G(k, E) over the whole
 * model space, from which the spectral weights of qsdos follow (-Im/pi).  One cluster, HartrIndex the identity;
 * FP64 or DMFTGPU_MIXED. */
int dmftgpu_gloc_real(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk, const double *sigma_e, int nE,
                      double e0, double de, double eta, double mu, double *gloc, double *trace, int flags);

/* upfolding_density over the full band window (src/upfolding.cpp:10-35, 38-91): per k, D_DFT = V (DF^H dens DF) V^H
 * with dens[nk][n][n] the model-basis densityMatDFT, df[nk][n][n] DF_CorrBase and evec[nk][n][n] the KS eigenvectors
 * in the DFT basis ((transformMatrix_k^H)^-1 KS_eigenVectors_orthoBasis; KS_eigenVectors_orthoBasis itself for the
 * identity transform of the generalized-eigensolve path), then the k -> R sums
 * DM(R)(i0, j0) = (1/nk) sum_k M_k(i0, j0) exp(+i k.a R) at the rindex[nnz][5] = (Rx, Ry, Rz, i0, j0) entries for
 * M = S^-1 D_DFT S^-1 (dm_dual_dual, DM_DFT_DMFT.HWR), S^-1 D_DFT (dm_dual_direct) and D_DFT (dm_direct); sk NULL:
 * S = I.  The k mesh is TightBinding's kx x ky x kz grid; outputs nnz complex each (any may be NULL); rindex host.
 * n <= 64, kx, ky, kz <= 256.  FP64. */
int dmftgpu_upfold(dmftgpu_ctx *ctx, int n, int kx, int ky, int kz, const double *dens, const double *df,
                   const double *evec, const double *sk, int nnz, const int *rindex, double *dm_dual_dual,
                   double *dm_dual_direct, double *dm_direct, int flags);

/* dmftgpu_upfold with a band window (src/upfolding.cpp:10-35): dens and df as dmftgpu_downfold_window leaves them
 * (the window in the leading NBAND[k] x NBAND[k] block), eps[nk][n] the band energies, nband / from_val_to_ks (host)
 * its window; Matrix_KSBase is the Fermi diagonal f(e - mu) (beta, the reference's +-100 cut-offs) with the window's
 * rows and columns replaced by DF^H dens DF, then D_DFT = V Matrix_KSBase V^H and the three k -> R sums. */
int dmftgpu_upfold_window(dmftgpu_ctx *ctx, int n, int kx, int ky, int kz, const double *dens, const double *df,
                          const double *evec, const double *sk, const double *eps, const int *nband,
                          const int *from_val_to_ks, double mu, double beta, int nnz, const int *rindex,
                          double *dm_dual_dual, double *dm_dual_direct, double *dm_direct, int flags);

/* GreenFtn_w's per-k density matrix in the model basis, densityMatDFT (src/GreenFtn.cpp:170-172, 268-275,
 * 311-319): dens[nk][n][n] = (1/beta) sum_{n < 2 nfreq} [G + G^H - G0 - G0^H](k, iw_n) + U f(e0) U^H, with G the full
 * n x n lattice Green function (Sigma on the HartrIndex orbitals, its moment tail beyond nfreq), G0 the resolvent
 * of the static H + m0 = U diag(e0) U^H and f the Fermi factors with the reference's +-100 cut-offs.  Computed
 * from the correlated-block Schur form (no n x n inversion); rows and columns in the caller's orbital order.  FP64,
 * or double-float on the FP32 pipe with DMFTGPU_MIXED. */
int dmftgpu_density_dft(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk, const double *sigma, double mu,
                        double *dens, int flags);

/* Derivatives of GreenFtn_w's G_loc(iw_n) = (1/N_k) sum_k G_PP(k, iw_n), n < nfreq, for one correlated cluster
 * (no counterpart in the reference, which has no derivatives; they supply dN/dmu-style Newton steps and
 * Jacobian-vector products of the self-consistency residual).  dG_PP = G_PP dSigma G_PP - dmu (G^2)_PP, with G
 * recomputed per (k, iw) from the Schur data (never stored).
 * dmftgpu_gloc_vjp: gbar[nfreq][D][D] -> sigma_bar[nfreq][D][D] = (1/N_k) sum_k G^H gbar G^H and *mu_bar (host) =
 *   -(1/N_k) sum Re Tr[((G^2)_PP)^H gbar] (the adjoint x_bar = J^H y_bar of complex autograd).
 * dmftgpu_gloc_jvp: (sigma_dot[nfreq][D][D], mu_dot) -> gloc_dot[nfreq][D][D].  FP64. */
int dmftgpu_gloc_vjp(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk, const double *sigma, double mu,
                     const double *gbar, double *sigma_bar, double *mu_bar, int flags);
int dmftgpu_gloc_jvp(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk, const double *sigma, double mu,
                     const double *sigma_dot, double mu_dot, double *gloc_dot, int flags);

/* The model Hamiltonian of a non-orthogonal tight-binding input, per k point: the generalized eigenproblem
 * H(k) v = e S(k) v of Construct_Hk_Sk (src/ConstructModelHamiltonian.cpp:103-111) followed by downfolding_ftn
 * over the full band window (src/downfolding.cpp:20-63) and the k-averaged impurity level
 * (src/downfolding.cpp:85-104).  hk, sk: [nk][n][n] (sk NULL: identity overlap), hartr[D] the correlated rows
 * (HartrIndex_inDFT, distinct, always a host pointer), n <= 56.  Outputs: eps[nk][n] ascending band energies; hmodel[nk][n][n] =
 * DF diag(eps) DF^H with rows 0..D-1 the Loewdin-orthonormalised projected correlated orbitals; optional
 * df[nk][n][n] (DF_CorrBase), evec[nk][n][n] (KS_eigenVectors_orthoBasis: the S-orthonormal eigenvectors, column l
 * for eps[l]) and himp[D][D] = (1/nk) sum_k hmodel[k][0:D][0:D].  The ligand rows D..n-1 of DF
 * are an orthonormal complement whose in-subspace rotation differs from Eigen's (see the kernel's header);
 * FP64.  DMFTGPU_SINGULAR when S is not positive definite or the projected block is rank deficient. */
int dmftgpu_downfold(dmftgpu_ctx *ctx, int nk, int n, int D, const int *hartr, const double *hk, const double *sk,
                     double *eps, double *hmodel, double *df, double *evec, double *himp, int flags);

/* dmftgpu_downfold with the band window of low_energy_subspace_in_KS_basis (src/downfolding.cpp:130-187, used by
 * downfolding_ftn, src/downfolding.cpp:20-63): per k the model space is the NBAND[k] bands with
 * lower < e - mu_dft < upper (strict), FromValToKS[k] their indices (a contiguous ascending range, the band
 * energies being ascending).  Outputs (host arrays) nband[nk] and from_val_to_ks[nk][n] (entries beyond NBAND[k]:
 * -1); H_model and DF fill the leading NBAND[k] x NBAND[k] block of their n x n slots, the rest a decoupled padding
 * (pad_energy on H_model's diagonal, the identity in DF): a padded band couples to no orbital, so every lattice sum of
 * the padded H_model (G_loc, GwHF, NumMatrix, N(mu) with beta (pad_energy - mu) > 100) equals that of the ragged one.
 * A k point whose window holds no band or fewer than D bands (where the reference exits) gives DMFTGPU_BADARG. */
int dmftgpu_downfold_window(dmftgpu_ctx *ctx, int nk, int n, int D, const int *hartr, const double *hk,
                            const double *sk, double mu_dft, double lower, double upper, double pad_energy,
                            int *nband, int *from_val_to_ks, double *eps, double *hmodel, double *df, double *evec,
                            double *himp, int flags);

/* Construct_hyb_delta (src/Construct_hyb_delta.cpp:47-119, declared src/TB.h:45-47):
 * delta[nfreq][dim][dim] = (iw+mu) I - himp[orb] - sigma[orb] - (gw[orb])^-1, orb[dim] indexes D. */
int dmftgpu_hyb_delta(dmftgpu_ctx *ctx, int dim, const int *orb, int nfreq, double beta, int D,
                      const double *sigma, const double *gw, const double *himp, double mu, double *delta,
                      int flags);

/* ---------------------------------------------------------------------------------------------
 * Impurity stage.  Matrices are dim x dim; U lists are gen_Uijkl's (src/gen_Uijkl.cpp:9-87):
 * uidx[nu][4] = (i, j, k, l), ut[nu] complex; both always host pointers.
 * --------------------------------------------------------------------------------------------- */

/* FourierTransform (src/FourierTransform.cpp:470-488 -> FourierTransform_, :126-178): fw[nfreq] -> ft[ntau+1],
 * tau_j = j beta / ntau, including the positivity fix-up.  If mom[4] is given it is used as is; else the moments
 * are fitted (green_asym selects the m0=0, m1=I fit) and, if m1 is given, m0 = 0 and m1 = *m1 (the overload with
 * the AsymtoV argument). */
int dmftgpu_fourier_w2tau(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, const double *fw,
                          const double *mom, int green_asym, const double *m1, double *ft, int flags);
/* FT_t_to_w (src/FourierTransform.cpp:521-561): ft[ntau+1] -> fw[nfreq]; DMFTGPU_CAUSALITY where the
 * reference asserts. */
int dmftgpu_fourier_tau2w(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, const double *ft, double *fw,
                          int flags);
/* getStimp (src/SCGF2_fullLoop.cpp:603-690): gt[ntau+1] -> st[ntau+1] (non-skeleton form), with the
 * Hermiticity checks (DMFTGPU_HERMITICITY) and the positivity fix-up. */
int dmftgpu_sigma2_tau(dmftgpu_ctx *ctx, int dim, int ntau, double beta, int nu, const int *uidx, const double *ut,
                       const double *gt, double *st, int flags);
/* getFockOperator (src/SCGF2_fullLoop.cpp:583-597). */
int dmftgpu_fock(dmftgpu_ctx *ctx, int dim, int nu, const int *uidx, const double *ut, const double *occ, double *fock,
                 int flags);
/* getGwimp (src/SCGF2_fullLoop.cpp:551-578): gw[nfreq] = [(iw+mu) - himp - delta - fock - sigma2]^-1. */
int dmftgpu_dyson(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, double mu, const double *himp, const double *delta,
                  const double *fock, const double *sigma2, double *gw, int flags);
/* getoccMat (src/SCGF2_fullLoop.cpp:539-549): occ = -G(tau = beta^-). */
int dmftgpu_occupation(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, const double *gw, double *occ, int flags);
/* estimate_asymto (src/SCGF2_fullLoop.cpp:736-787): f holds nfreq+3 matrices; writes slot nfreq+order-1. */
int dmftgpu_estimate_asymto(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, double *f, int order, int flags);
/* IPT (src/SCGF2_fullLoop.cpp:873-1065, dispatched by SOLVER at src/SOLVER.cpp:411-414): dim = 2.
 * himp = projimpurity_site_Hamiltonian, delta[nfreq] = projweiss_field, nummat_in = projNumMatrix;
 * outputs in ImgFreqFtn slot order (src/ImgTimeFtn.cpp:177): se_out[nfreq+5] (SE_out), gimp_out[nfreq+5]
 * (Gwimp_out, may be NULL) and nummat_out (the updated projNumMatrix). */
int dmftgpu_ipt(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, double U, double mu, const double *himp,
                const double *delta, const double *nummat_in, int nu, const int *uidx, const double *ut,
                double *se_out, double *gimp_out, double *nummat_out, int flags);
/* SCGF2 (src/SCGF2_fullLoop.cpp:392-533, dispatched by SOLVER for SOLVER_TYPE = SC2PT at
 * src/SOLVER.cpp:393-399): the self-consistent second-order loop on G_imp with Pulay mixing (history 2, DIIS
 * from loop 101), run until the reference's stopping test (at least 10 loops, then until both the G_imp and
 * the occupation residual are <= 1e-6) or max_iter loops (the reference's 2000).  himp =
 * projimpurity_site_Hamiltonian, weiss[nfreq] = projweiss_field, mu = muTB, mixing = MIXING; gimp[nfreq+5] is
 * Gwimp_in_out: its first nfreq slots are read as the initial G_imp and all nfreq+5 are written;
 * se_out[nfreq+5] = SE_out; *loops = loop iterations run.  mixing_check_outer's residual memory (a function
 * static of the reference) lives in the context. */
int dmftgpu_scgf2(dmftgpu_ctx *ctx, int dim, int nfreq, int ntau, double beta, double mu, double mixing,
                  const double *himp, const double *weiss, double *gimp, int nu, const int *uidx, const double *ut,
                  int max_iter, double *se_out, int *loops, int flags);

/* dc_for_dmft (src/dmft_main.cpp:593-707): the double-counting self-energy of every correlated atom, host
 * arithmetic only (no device, no context).  natoms = NumCorrAtom, nso = N_peratom_HartrOrbit; nummat, sigma0 and
 * dc are (natoms nso) x (natoms nso) complex column-major host arrays: nummat the NumMatrix the DC is built from
 * (NelectronDFT), sigma0 = SelfEnergy_w at the first Matsubara frequency (read by DMFTGPU_DC_SIGMA0 with
 * initial != 0 only, may be NULL otherwise), dc: in, the previous Sw_doublecounting (SIGMA0, initial != 0); out,
 * the new one.  initial is the reference's initial_dc (0 on the first call, 1 in the DMFT loop). */
int dmftgpu_double_counting(int dctype, int natoms, int nso, double U, double Uprime, double J, double nominal_charge,
                            const double *nummat, const double *sigma0, int initial, double *dc);

/* proj_to_site's solver basis for impurityBasisSwitch (src/SOLVER.cpp:541-586), host arithmetic: with a real H_imp
 * and magnetism 0 or 1, the eigenvectors of the spin-pair-averaged real symmetric Re[H_imp + Delta(i w_0)] on both
 * spins of each pair; otherwise the eigenvectors of H_imp times those of the real part of (H_imp + the Hermitian part
 * of Delta(i w_0)) in that basis.  himp, delta0: dim x dim (H_imp - DC and Delta(i w_0)), basis: out, all complex
 * column-major host arrays.  Eigenvectors are ordered by ascending eigenvalue with each one's first component of
 * largest modulus made real and positive (the reference takes Eigen's phases; for the Kanamori and density-density
 * interactions, whose terms pair every index, a spin-pair-averaged basis gives the same self-energy whatever the
 * phases). */
int dmftgpu_impurity_basis(int dim, int magnetism, const double *himp, const double *delta0, double *basis);

/* weak_solver (src/SOLVER.cpp:72-102, Lowlevel_SOLVERTYPE): the one-shot solver of the weakly correlated
 * subspace (the Hartree orbitals beyond the correlated ones), run by dmft_main when NumHartrOrbit_per_cluster >
 * NSpinOrbit_per_atom (src/dmft_main.cpp:420-454).  DMFTGPU_WEAK_HF: on_shot_HF (src/SCGF2_fullLoop.cpp:218-250),
 * the Fock term of getoccMat(gw); DMFTGPU_WEAK_2PT / _SC2PT: SC2PT_weak (src/SCGF2_fullLoop.cpp:49-133), the Fock
 * term plus the second-order Sigma from G0 = gwhf (2PT) or G0 = gw (SC2PT).  gw, gwhf: nfreq slots (Gw_weak,
 * GwHF_weak; gwhf may be NULL except for 2PT); se_out[nfreq+5] in ImgFreqFtn order (writeResults). */
#define DMFTGPU_WEAK_HF 0
#define DMFTGPU_WEAK_2PT 1
#define DMFTGPU_WEAK_SC2PT 2
int dmftgpu_weak_solver(dmftgpu_ctx *ctx, int solver, int dim, int nfreq, int ntau, double beta, const double *gw,
                        const double *gwhf, int nu, const int *uidx, const double *ut, double *se_out, int flags);

/* ---------------------------------------------------------------------------------------------
 * One DMFT self-consistency iteration: the body of the loop of src/dmft_main.cpp:343-570 for one correlated
 * cluster solved by IPT (two spin-orbitals, the example model of the reference) or by SC2PT (SCGF2, up to 32
 * spin-orbitals).
 * --------------------------------------------------------------------------------------------- */
#define DMFTGPU_SOLVER_IPT 0
#define DMFTGPU_SOLVER_SC2PT 1 /* SCGF2 */
#define DMFTGPU_DC_NONE 0
#define DMFTGPU_DC_NOMINAL 1 /* dc_for_dmft "nominal" (src/dmft_main.cpp:665-677) */
#define DMFTGPU_DC_FLL 2     /* "fll" (src/dmft_main.cpp:621-640): from the spin-resolved occupation of NumMatrix */
#define DMFTGPU_DC_AMF 3     /* "amf" (src/dmft_main.cpp:641-660) */
#define DMFTGPU_DC_SIGMA0 4  /* "sigma0" (src/dmft_main.cpp:606-618): FLL on the first call, then the previous DC
                                plus Re Tr Sigma(i w_0) / N per atom (dmftgpu_double_counting only) */
#define DMFTGPU_DC_UPRIME 0x100 /* with NOMINAL or FLL: U' instead of the orbital-averaged U ("nominal_Uprime",
                                   "fll_Uprime") */
typedef struct {
    int solver;            /* DMFTGPU_SOLVER_IPT or DMFTGPU_SOLVER_SC2PT */
    int ntau;              /* N_TAU */
    double n_electrons;    /* N_ELECTRONS: target of the mu search */
    double U, Uprime, J;   /* U, U', J */
    double mixing;         /* MIXING (Pulay, history 2, start 5) */
    int magnetism;         /* MAGNETISM (0: spin-averaged self-energy and occupation) */
    int dctype;            /* DMFTGPU_DC_NONE, _NOMINAL, _FLL, _AMF, optionally | DMFTGPU_DC_UPRIME; FLL and AMF use
                              the nummat the iteration starts from (the NumMatrix of the last TightBinding) */
    double nominal_charge; /* N_d */
    int nu;                /* U_{ijkl} list of the correlated space (gen_Uijkl), host pointers */
    const int *uidx;
    const double *ut;
    int scgf_max_iter;     /* SCGF2 loop limit (0: the reference's 2000) */
    int basis_switch;      /* impurityBasisSwitch: solve in the basis of dmftgpu_impurity_basis (src/SOLVER.cpp:541-595) */
    int pulay_history;     /* Pulay (DIIS) history of the SelfEnergy_w mixer (0: the reference's 2) */
    int pulay_start;       /* first iteration of the DIIS step; simple mixing before it (0: the reference's 5) */
    int mixer;             /* DMFTGPU_MIXER_PULAY (the reference's) or DMFTGPU_MIXER_NEWTON_KRYLOV */
    int newton_start;      /* Newton-Krylov: first iteration of Newton steps, the Pulay mixer before it (0: 3) */
    int krylov_dim;        /* Newton-Krylov: Jacobian-vector products per step at most (0: 8, at most 64) */
    double krylov_tol;     /* Newton-Krylov: relative residual of each step's linear solve (0: 1e-3) */
} dmftgpu_dmft_params;

/* Self-energy mixers of dmftgpu_dmft_iteration.  NEWTON_KRYLOV (no counterpart in the reference): with x =
 * SelfEnergy_w and Phi(x) the SOLVER output on the TightBinding state of x, each step solves
 * (dPhi/dx - I) dx = x - Phi(x) by GMRES and sets x <- x + dx.  Its Jacobian-vector products take the lattice
 * part from the tangent pass of dmftgpu_gloc_jvp (mu's first-order change from the electron count) and the
 * D x D stages (Construct_hyb_delta, SOLVER) by directional differences; the fixed point is the Pulay mixer's. */
#define DMFTGPU_MIXER_PULAY 0
#define DMFTGPU_MIXER_NEWTON_KRYLOV 1

/* SOLVER (IPT or SCGF2) with proj_to_site and the magnetism == 0 averaging (src/SOLVER.cpp:105-502), the Pulay mixing
 * of SelfEnergy_w (src/dmft_main.cpp:529-533), TightBinding's mu search, GreenFtn_w and Construct_hyb_delta
 * (src/TB.cpp:297-331) and the dmft_scf_check residuals (src/dmft_main.cpp:902-1014), all on the device.
 * Device pointers only (flags must contain DMFTGPU_DEVICE_PTRS; DMFTGPU_MIXED / DMFTGPU_NEWTON select the
 * lattice-sum precision and the mu search).  State, updated in place: selfe[nfreq][D][D] (SelfEnergy_w),
 * weiss[nfreq][D][D] (weiss_fieldTB), nummat[D][D] (NumMatrix), *mu (host), gloc[nfreq][D][D] (G_loc of
 * the last TightBinding call: read as SCGF2's initial G_imp, then overwritten).  Outputs: gimp[nfreq+5][D][D]
 * and resid[5] (host) = GwRD, GwRD_low, GwRD_max, NumMatRD, SCGF2 loop count (0 for IPT).  `iteration` is the
 * reference's currentIt (1 on the first call restarts the mixer history). */
int dmftgpu_dmft_iteration(dmftgpu_ctx *ctx, const dmftgpu_lattice *lat, const double *hk,
                           const dmftgpu_dmft_params *params, int iteration, double *selfe, double *weiss,
                           double *nummat, double *mu, double *gloc, double *gimp, double *resid, int flags);

/* The last dmftgpu_dmft_iteration's mixer: *krylov = Jacobian-vector products of its Newton-Krylov step (0 when the
 * call used the Pulay mixer), *relres = the relative residual of that step's linear solve, *residual = the
 * fixed-point residual |SE_out - SelfEnergy_w| / |SelfEnergy_w| (w < N_freq) the mixer was given. */
int dmftgpu_mixer_stats(dmftgpu_ctx *ctx, int *krylov, double *relres, double *residual);

/* ---------------------------------------------------------------------------------------------
 * Restart files: ImgFreqFtn's text format ("w m n Re Im" lines, printf "%d %d %d %+0.8f %+0.8f"), host only (no
 * context, no device).  f: nfreq + 5 ImgFreqFtn slots of column-major norbit x norbit complex matrices.
 * dmftgpu_imgfreq_write: dataOut_full (src/ImgTimeFtn.cpp:330-355): elements with |F| > 1e-7 for w < nfreq, then
 *   every tail slot as w = -1 .. -5.
 * dmftgpu_imgfreq_update: update_full (src/ImgTimeFtn.cpp:624-670): the file's w in [0, nfreq) entries overwrite f,
 *   the rest of f is kept; DMFTGPU_BADARG for an orbital index outside [0, norbit) (the reference exits).
 * dmftgpu_imgfreq_read: read_full (src/ImgTimeFtn.cpp:673-751): a file written at beta_prev re-gridded to beta's
 *   Matsubara points (linear interpolation, linear extrapolation below the file's first point, R + w_last J / w
 *   above its last); the tail slots of f are zeroed.
 * DMFTGPU_IO when the file cannot be opened, read or written. */
int dmftgpu_imgfreq_write(const char *path, int nfreq, int norbit, const double *f);
int dmftgpu_imgfreq_update(const char *path, int nfreq, int norbit, double *f);
int dmftgpu_imgfreq_read(const char *path, int nfreq, int norbit, double beta, double beta_prev, double *f);

/* No counterpart in the reference.  Construct_hyb_delta for callers that cannot allocate device memory
 * (a driver whose HBM belongs to a pool allocator, or one that must not stall the device with a
 * non-stream-ordered cudaMalloc): no context, no allocation, every array argument a DEVICE pointer except
 * orb (host, dim <= 32); work is enqueued on cuda_stream (NULL: the legacy default stream), which must belong
 * to the current device (else DMFTGPU_BADARG).  The call is synchronous: it waits for cuda_stream to finish
 * and returns the status its kernel raised.  Scratch is a static device array of 2^19 complex numbers
 * (8 MiB) per GPU that loads the library, so nfreq*dim*dim must not exceed 524288 (else DMFTGPU_BADARG).
 * Being synchronous, the call must not be made on a stream under capture (the read-back and the wait would
 * invalidate the capture).  Calls that overlap on the GPU share the array and race. */
int dmftgpu_hyb_delta_noalloc(int dim, const int *orb, int nfreq, double beta, int D, const double *sigma,
                              const double *gw, const double *himp, double mu, double *delta, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
