// mixing.cu -- Pulay (DIIS) mixing, pulayMixing::mixing (src/pulay.cpp:48-167), with the history on the
// device: residuals and combinations are device kernels, the residual Gram matrix entries are fixed-order
// device reductions, and the (h+1) x (h+1) DIIS system is solved on the host with complete pivoting (Eigen's
// FullPivLU invertibility test of the reference).  Used for SelfEnergy_w at the DMFT level (pulayMixing(2, 5))
// and for G_imp inside SCGF2 (pulayMixing(2, 100), src/SCGF2_fullLoop.cpp:472).
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace {

std::string nm(const char *tag, const char *suffix) { return std::string(tag) + suffix; }

double2 *buf2(dmftgpu_ctx *ctx, const std::string &name, size_t count) {
    return (double2 *)dg_buf(ctx, name.c_str(), count * sizeof(double2));
}

// Pulay: Gram entry g = sum_w Re Tr(r0^H rk) = sum over all elements of Re(conj(r0) rk)
__global__ void k_dot_re(long long n, const double2 *a, const double2 *b, double *out) {
    __shared__ double red[256];
    double s = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        s += a[t].x * b[t].x + a[t].y * b[t].y;
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

__global__ void k_axpby(long long n, double a, const double2 *x, double b, const double2 *y, double2 *out) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = cadd(cscale(x[t], a), cscale(y[t], b));
}

// Eigen::FullPivLU(A).isInvertible() and A x = b for the small real DIIS matrix (complete pivoting)
bool solve_full_pivot(int n, std::vector<double> A, std::vector<double> b, std::vector<double> &x) {
    std::vector<int> cperm(n);
    for (int i = 0; i < n; i++) cperm[i] = i;
    double maxpiv = 0;
    std::vector<double> piv(n);
    for (int k = 0; k < n; k++) {
        int pr = k, pc = k;
        double best = -1;
        for (int j = k; j < n; j++)
            for (int i = k; i < n; i++)
                if (std::fabs(A[i + j * n]) > best) {
                    best = std::fabs(A[i + j * n]);
                    pr = i;
                    pc = j;
                }
        piv[k] = best;
        maxpiv = std::max(maxpiv, best);
        for (int j = 0; j < n; j++) std::swap(A[k + j * n], A[pr + j * n]);
        std::swap(b[k], b[pr]);
        for (int i = 0; i < n; i++) std::swap(A[i + k * n], A[i + pc * n]);
        std::swap(cperm[k], cperm[pc]);
        if (best == 0) continue;
        for (int i = k + 1; i < n; i++) {
            const double f = A[i + k * n] / A[k + k * n];
            for (int j = k; j < n; j++) A[i + j * n] -= f * A[k + j * n];
            b[i] -= f * b[k];
        }
    }
    const double thr = 2.220446049250313e-16 * n * maxpiv;  // Eigen's default rank threshold
    for (int k = 0; k < n; k++)
        if (!(piv[k] > thr)) return false;
    std::vector<double> y(n);
    for (int i = n - 1; i >= 0; i--) {
        double s = b[i];
        for (int j = i + 1; j < n; j++) s -= A[i + j * n] * y[j];
        y[i] = s / A[i + i * n];
    }
    x.assign(n, 0.0);
    for (int k = 0; k < n; k++) x[cperm[k]] = y[k];
    return true;
}

}  // namespace

int dg_pulay_mixing(dmftgpu_ctx *ctx, DgPulay &P, const char *tag, long long len, double2 *in, double2 *out,
                    double mixing, int it) {
    const int h = P.hist, H1 = h + 1;
    double2 *inh = buf2(ctx, nm(tag, ".in"), (size_t)h * len), *resh = buf2(ctx, nm(tag, ".res"), (size_t)h * len);
    double *part = (double *)dg_buf(ctx, nm(tag, ".part").c_str(), 256 * sizeof(double));
    if (!inh || !resh || !part) return DMFTGPU_NOMEM;
    cudaStream_t s = ctx->stream;
    if (P.len != len) {
        P.len = len;
        P.om.assign(H1 * H1, 0.0);
        for (int k = 0; k < h; k++) {
            P.om[h + k * H1] = -1;
            P.om[k + h * H1] = -1;
        }
        P.om[(h - 1) + (h - 1) * H1] = -100.;
        P.om[h + h * H1] = 0.;
        DG_CUDA(cudaMemsetAsync(inh, 0, (size_t)h * len * sizeof(double2), s));
        DG_CUDA(cudaMemsetAsync(resh, 0, (size_t)h * len * sizeof(double2), s));
    }
    const int removeComp = h - 1;
    for (int k = removeComp; k > 0; k--) {
        DG_CUDA(cudaMemcpyAsync(inh + (size_t)k * len, inh + (size_t)(k - 1) * len, len * sizeof(double2),
                                cudaMemcpyDeviceToDevice, s));
        DG_CUDA(cudaMemcpyAsync(resh + (size_t)k * len, resh + (size_t)(k - 1) * len, len * sizeof(double2),
                                cudaMemcpyDeviceToDevice, s));
    }
    DG_CUDA(cudaMemcpyAsync(inh, in, len * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    k_axpby<<<dg_ceil_div(len, 256), 256, 0, s>>>(len, 1.0, out, -1.0, in, resh);  // res = out - in
    DG_LAUNCH(ctx, "k_axpby");
    if (it > P.start) {
        std::vector<double> tmp((h - 1) * (h - 1));
        for (int k = 0; k < h - 1; k++)
            for (int l = 0; l < h - 1; l++) {
                int ik = k >= removeComp ? k + 1 : k, il = l >= removeComp ? l + 1 : l;
                tmp[k + l * (h - 1)] = P.om[ik + il * H1];
            }
        for (int k = 1; k < h; k++)
            for (int l = 1; l < h; l++) P.om[k + l * H1] = tmp[(k - 1) + (l - 1) * (h - 1)];
        for (int k = 0; k < h; k++) {
            k_dot_re<<<256, 256, 0, s>>>(len, resh, resh + (size_t)k * len, part);
            DG_LAUNCH(ctx, "k_dot_re");
            double hp[256];
            DG_CUDA(cudaMemcpyAsync(hp, part, sizeof(hp), cudaMemcpyDeviceToHost, s));
            DG_CUDA(cudaStreamSynchronize(s));
            double g = 0;
            for (int q = 0; q < 256; q++) g += hp[q];
            P.om[0 + k * H1] = g;
            P.om[k + 0 * H1] = g;
        }
    }
    std::vector<double> beta;
    std::vector<double> rhs(H1, 0.0);
    rhs[h] = -1;
    const bool use = it > h + P.start && solve_full_pivot(H1, P.om, rhs, beta);
    double2 *opt = buf2(ctx, nm(tag, ".opt"), len), *optr = buf2(ctx, nm(tag, ".optr"), len);
    if (!opt || !optr) return DMFTGPU_NOMEM;
    if (use) {
        DG_CUDA(cudaMemsetAsync(opt, 0, len * sizeof(double2), s));
        DG_CUDA(cudaMemsetAsync(optr, 0, len * sizeof(double2), s));
        for (int k = 0; k < h; k++) {
            k_axpby<<<dg_ceil_div(len, 256), 256, 0, s>>>(len, 1.0, opt, beta[k], inh + (size_t)k * len, opt);
            DG_LAUNCH(ctx, "k_axpby");
            k_axpby<<<dg_ceil_div(len, 256), 256, 0, s>>>(len, 1.0, optr, beta[k], resh + (size_t)k * len, optr);
            DG_LAUNCH(ctx, "k_axpby");
        }
        k_axpby<<<dg_ceil_div(len, 256), 256, 0, s>>>(len, 1.0, opt, mixing, optr, out);
    } else {
        k_axpby<<<dg_ceil_div(len, 256), 256, 0, s>>>(len, 1.0, in, mixing, resh, out);
    }
    DG_LAUNCH(ctx, "k_axpby");
    return DMFTGPU_OK;
}

