/*
 * dmft_oracle.h -- C interface of the CPU FP64 oracle for the DMFT self-consistency hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, __graft_entry__.smoke() and the
 * CPU-baseline / reference arm of bench.py load it.  The product (dmftpack_gb300, libdmftgpu.so) never
 * links, loads or calls it.
 *
 * PARITY UNPINNED: the reference (KAIST-ELST/DMFTpack, src/) needs Eigen (not vendored, not installed,
 * version unpinned) and MPI, so it cannot be compiled here, and it ships no tests, golden vectors or
 * reference outputs.  Every function below restates the cited reference lines in plain C++ FP64 with its
 * own LU / Jacobi primitives; the restatement is cross-checked against an independent numpy restatement
 * (numpy/LAPACK eigvals, inv, eigh standing in for Eigen) and against analytic known answers in tests/.
 *
 * Conventions (shared with include/dmftgpu.h):
 *   - complex numbers are interleaved doubles (re, im);
 *   - every matrix is column-major, element (i,j) at [i + j*ld], ld = its row count;
 *   - a frequency- or tau-indexed function is a contiguous stack of such matrices;
 *   - integer index tables are row-major ([row][col]).
 * Return codes: 0 ok, 1 singular pivot, 2 no convergence, 3 NaN/Inf, 4 bad argument,
 *               5 causality violated (Im G or Im Delta eigenvalue > 0), 6 Hermiticity violated.
 */
#ifndef DMFT_ORACLE_H
#define DMFT_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Lattice description: replaces the reference's globals NBAND, knum, N_freq, beta, NumCluster,
 * NumHartrOrbit_per_cluster, HartrIndex (src/tight_common.cpp:28-114, src/TB.h:7-35). */
typedef struct {
    int n;              /* orbitals per k (NBAND) */
    int nk;             /* k points (knum == knum_mpiGlobal on one rank) */
    int nfreq;          /* positive Matsubara frequencies (N_freq) */
    double beta;
    int ncl;            /* NumCluster */
    int nh;             /* NumHartrOrbit_per_cluster */
    const int *hartr;   /* HartrIndex[ncl*nh]: correlated orbital -> orbital index in H(k) */
} orc_lattice;

int  orc_version(void);
/* threads for the transforms, the moment fit and getStimp (results do not depend on the count) */
void orc_set_threads(int n);
void orc_kmesh(int kx, int ky, int kz, double *kmesh);
int  orc_hk(int n, int nnz, const int *rindex, const double *hr, int nk, const double *kmesh,
            double *hk, int nthreads);
int  orc_hermitian_eig(int n, const double *a, double *w, double *v);
int  orc_inverse(int n, const double *a, double *ainv);
int  orc_moments(int dim, int nfreq, double beta, const double *fw, int green_asym, double *mom);
int  orc_greenftn_w(const orc_lattice *L, const double *hk, const double *sigma, double mu,
                    double *gw, double *gwhf, double *nummat, int nthreads);
int  orc_nele(const orc_lattice *L, const double *hk, const double *sigma, double mu,
              double *nele, double *dnele, int nthreads);
int  orc_adjust_mu(const orc_lattice *L, const double *hk, const double *sigma, double mu, double dmu,
                   double n_target, double *mu_out, int *n_eval, int nthreads);
int  orc_hyb_delta(int dim, const int *orb, int nfreq, double beta, int D, const double *sigma,
                   const double *gw, const double *himp, double mu, double *delta);
int  orc_w2tau(int dim, int nfreq, int ntau, double beta, const double *fw, const double *mom,
               double *ft, int *fixups);
int  orc_w2tau_single(int dim, int nfreq, double beta, const double *fw, const double *mom,
                      double tau, double *out);
int  orc_fourier(int dim, int nfreq, int ntau, double beta, const double *fw, int green_asym,
                 const double *m1, double *ft, int *fixups);
int  orc_tau2w(int dim, int nfreq, int ntau, double beta, const double *ft, double *fw);
int  orc_sigma2_tau(int dim, int ntau, double beta, int nu, const int *uidx, const double *ut,
                    const double *gt, double *st, int *fixups);
void orc_fock(int dim, int nu, const int *uidx, const double *ut, const double *occ, double *fock);
int  orc_dyson(int dim, int nfreq, double beta, double mu, const double *himp, const double *delta,
               const double *fock, const double *sigma2, double *gw);
void orc_estimate_asymto(int dim, int nfreq, double beta, double *f, int order);
int  orc_occ(int dim, int nfreq, double beta, const double *gw, double *occ);
int  orc_gen_uijkl(int nso, double U, double Up, double J, int density_density, int cap, int *uidx,
                   double *ut);
int  orc_ipt(int dim, int nfreq, int ntau, double beta, double U, double mu, const double *himp,
             const double *delta, const double *nummat_in, int nu, const int *uidx, const double *ut,
             double *se_out, double *gimp_out, double *nummat_out);

#ifdef __cplusplus
}
#endif
#endif
