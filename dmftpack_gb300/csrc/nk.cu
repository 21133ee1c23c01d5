// nk.cu -- GMRES on device-resident vectors for the Newton-Krylov self-energy mixer of the DMFT iteration.
//
// The DMFT map Sigma -> Sigma_out is real-linearisable but not complex-analytic (Hermitian parts, spin averages,
// real moment fits), so its Jacobian is a real-linear operator: every vector here is an array of complex
// numbers read as 2n reals, with the real inner product <a, b> = sum Re(conj(a) b).  Arnoldi by modified
// Gram-Schmidt; the (m+1) x m Hessenberg least-squares problem by Givens rotations on the host.  The dot
// products are fixed-order two-stage reductions (per-block partials, then the host sums them in block order),
// so a run is bitwise reproducible.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace {

constexpr int DOT_BLOCKS = 304;  // 2 x 152 SMs
constexpr int DOT_THREADS = 256;

__global__ void k_vdot(long long n, const double2 *__restrict__ a, const double2 *__restrict__ b, double *part) {
    __shared__ double red[DOT_THREADS];
    double s = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        s += a[t].x * b[t].x + a[t].y * b[t].y;
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// y = a x + b y (x may be y: the scaling of a vector in place)
__global__ void k_vaxpby(long long n, double a, const double2 *x, double b, double2 *y) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) y[t] = cadd(cscale(x[t], a), cscale(y[t], b));
}

}  // namespace

int dg_vdot(dmftgpu_ctx *ctx, long long n, const double2 *a, const double2 *b, double *out) {
    double *part = (double *)dg_buf(ctx, "nk.dot", DOT_BLOCKS * sizeof(double));
    if (!part) return DMFTGPU_NOMEM;
    k_vdot<<<DOT_BLOCKS, DOT_THREADS, 0, ctx->stream>>>(n, a, b, part);
    DG_LAUNCH(ctx, "k_vdot");
    double h[DOT_BLOCKS];
    DG_CUDA(cudaMemcpyAsync(h, part, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    double s = 0;
    for (int i = 0; i < DOT_BLOCKS; i++) s += h[i];
    *out = s;
    return DMFTGPU_OK;
}

int dg_vaxpby(dmftgpu_ctx *ctx, long long n, double a, const double2 *x, double b, double2 *y) {
    if (n <= 0) return DMFTGPU_OK;
    k_vaxpby<<<dg_ceil_div(n, 256), 256, 0, ctx->stream>>>(n, a, x, b, y);
    DG_LAUNCH(ctx, "k_vaxpby");
    return DMFTGPU_OK;
}

int dg_gmres(dmftgpu_ctx *ctx, long long n, const double2 *b, int m, double tol,
             const std::function<int(const double2 *, double2 *)> &apply, double2 *x, int *iters, double *relres) {
    cudaStream_t s = ctx->stream;
    *iters = 0;
    *relres = 1;
    double2 *V = (double2 *)dg_buf(ctx, "nk.V", (size_t)(m + 1) * n * sizeof(double2));
    double2 *w = (double2 *)dg_buf(ctx, "nk.w", (size_t)n * sizeof(double2));
    if (!V || !w) return DMFTGPU_NOMEM;
    DG_CUDA(cudaMemsetAsync(x, 0, (size_t)n * sizeof(double2), s));
    double bb = 0;
    DG_TRY(dg_vdot(ctx, n, b, b, &bb));
    const double beta = std::sqrt(bb);
    if (!(beta > 0)) {
        *relres = 0;
        return std::isfinite(beta) ? DMFTGPU_OK : DMFTGPU_NONCONVERGED;
    }
    DG_CUDA(cudaMemcpyAsync(V, b, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    DG_TRY(dg_vaxpby(ctx, n, 0.0, V, 1.0 / beta, V));
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
    auto Hat = [&](int i, int j) -> double & { return H[i + (size_t)j * (m + 1)]; };
    g[0] = beta;
    int k = 0;
    for (int j = 0; j < m; j++) {
        DG_TRY(apply(V + (size_t)j * n, w));
        for (int i = 0; i <= j; i++) {
            double h = 0;
            DG_TRY(dg_vdot(ctx, n, w, V + (size_t)i * n, &h));
            Hat(i, j) = h;
            DG_TRY(dg_vaxpby(ctx, n, -h, V + (size_t)i * n, 1.0, w));
        }
        double ww = 0;
        DG_TRY(dg_vdot(ctx, n, w, w, &ww));
        const double hn = std::sqrt(ww);
        if (!std::isfinite(hn)) return DMFTGPU_NONCONVERGED;
        Hat(j + 1, j) = hn;
        for (int i = 0; i < j; i++) {  // the earlier rotations on the new column
            const double a = Hat(i, j), c = Hat(i + 1, j);
            Hat(i, j) = cs[i] * a + sn[i] * c;
            Hat(i + 1, j) = -sn[i] * a + cs[i] * c;
        }
        const double a = Hat(j, j), c = Hat(j + 1, j), r = std::hypot(a, c);
        cs[j] = r > 0 ? a / r : 1;
        sn[j] = r > 0 ? c / r : 0;
        Hat(j, j) = r;
        Hat(j + 1, j) = 0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        k = j + 1;
        *relres = std::fabs(g[j + 1]) / beta;
        const bool breakdown = !(hn > 1e-14 * beta);
        if (!breakdown) {
            double2 *vn = V + (size_t)(j + 1) * n;
            DG_CUDA(cudaMemcpyAsync(vn, w, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
            DG_TRY(dg_vaxpby(ctx, n, 0.0, vn, 1.0 / hn, vn));
        }
        if (*relres <= tol || breakdown) break;
    }
    // back substitution R y = g, x = V y
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; i--) {
        double t = g[i];
        for (int l = i + 1; l < k; l++) t -= Hat(i, l) * y[l];
        y[i] = Hat(i, i) != 0 ? t / Hat(i, i) : 0;
    }
    for (int i = 0; i < k; i++) DG_TRY(dg_vaxpby(ctx, n, y[i], V + (size_t)i * n, 1.0, x));
    *iters = k;
    return DMFTGPU_OK;
}
