// trace_tc.h -- arguments of the tensor-core N(mu) pass (trace_tc.cu) and its host entry.
#pragma once
#include <cuda_runtime.h>

struct dmftgpu_ctx;

struct TraceTcArgs {
    const double2 *H;      // [nk][n][n] column-major, correlated orbitals first
    const double2 *B;      // [nk][m][D]  b_l(a)
    const double *epsQ;    // [nk][m]     eigenvalues of H_QQ
    const double2 *sig;    // [nf2][D][D] Sigma(iw) with its moment tail beyond N_freq
    const double *eps0;    // [nk][n]     eigenvalues of H + m0
    int n, m, nk, nf2, D, wgrid;
    double beta, mu;
};

// true when the tensor-core pass covers this lattice (4 <= D <= 10, m <= 32, n <= 64)
bool dg_trace_tc_supported(int n, int D);
// prepare the per-k operand images once (*ready tracks it for the caller's prepared lattice), then run one pass:
// tr[f] = sum_k Re[Tr G(k, iw_f) - Tr G0(k, iw_f)] for f < nf2 (device)
int dg_trace_tc(dmftgpu_ctx *ctx, const TraceTcArgs &a, bool *ready, double *tr);
