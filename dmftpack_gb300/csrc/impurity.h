// impurity.h -- device-level building blocks of the impurity stage (impurity.cu), shared with the
// solver drivers (solvers.cu).  All pointers are device pointers; functions only enqueue work.
#pragma once
#include "linalg.cuh"

// U_{ijkl} list (gen_Uijkl, src/gen_Uijkl.cpp:9-87) on the device, with the entries grouped by their first
// index (byI) and by their last index (byJ) for the output-stationary getStimp kernel
struct DgUList {
    int nu = 0;
    const int *byI = nullptr, *byIoff = nullptr, *byJ = nullptr, *byJoff = nullptr, *uidx = nullptr;
    const double2 *ut = nullptr;
};

int dg_ulist(dmftgpu_ctx *ctx, int d, int nu, const int *uidx_host, const double *ut_host, DgUList &U);
int dg_phase_table(dmftgpu_ctx *ctx, int ntau, double2 **ph);
int dg_w2tau_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *fw, const double2 *mom,
                 double2 *ft);
int dg_fourier_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *fw, int green,
                   const double2 *m1, double2 *ft);
int dg_tau2w_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *ft, double2 *fw, bool check);
int dg_sigma2_dev(dmftgpu_ctx *ctx, int d, int ntau, double beta, const DgUList &U, const double2 *gt, double2 *st);
int dg_fock_dev(dmftgpu_ctx *ctx, int d, const DgUList &U, const double2 *occ, double2 *fock);
int dg_dyson_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, double mu, const double2 *himp,
                 const double2 *delta, const double2 *fock, const double2 *s2, double2 *gw, bool check);
int dg_estimate_asymto_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, double2 *f, int order);
int dg_occ_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, const double2 *gw, double2 *occ);
// the shared parts of getoccMat and FourierTransform: T = tail data (9 d x d slots), Dw = F - tail
int dg_green_tail_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, const double2 *gw, double2 *T, double2 *Dw);
int dg_occ_tail_dev(dmftgpu_ctx *ctx, int d, int nfreq, double beta, const double2 *T, const double2 *Dw,
                    double2 *occ);
int dg_w2tau_tail_dev(dmftgpu_ctx *ctx, int d, int nfreq, int ntau, double beta, const double2 *T, const double2 *Dw,
                      double2 *ft);
int dg_ipt_kk_dev(dmftgpu_ctx *ctx, int nfreq, const double *a, const double *b, const double *c, double2 *s2);
