// moments.cu -- getAsymto_moments (src/FourierTransform.cpp:184-465) on the device.
//
// The reference fits F(iw) ~ m0 + m1/iw + m2/(iw)^2 + m3/(iw)^3 by least squares on every suffix window
// [w, N_freq) of the Matsubara axis, with (K^T K)^-1 K^T G per window.  K has two non-zeros per row, so
// K^T G and K^T K are suffix sums of four (resp. six) weighted series: the device forms those sums with one
// backward scan per series (O(N_freq) instead of the reference's O(N_freq^2)), inverts each 4x4 K^T K with
// partial pivoting, and then reproduces the reference's window averaging (2Nv+1 windows, Nv = N_freq/20),
// the variance of the trace of each moment, the positivity gates on the averaged moments, the first-minimum
// window choice (sequential argmin started at the last window) and the final Hermitisation.
#include "smallmat.cuh"

namespace {

struct MomArgs {
    int D, Nf, R, C, Nv, ncol;
    double beta;
    int green;
    const double2 *fw;  // [Nf][D][D]
    double2 *S;         // [D*D][ncol][R]  suffix sums K^T G
    double *KS;         // [6][R]          suffix sums for K^T K
    double *kinv;       // [R][16]
    double2 *mt;        // [D*D][R][ncol]  fitted moments per window ("momentstest")
    double *tr;         // [ncol][R]
    double2 *avg;       // [ncol][C][D*D]
    double *var;        // [ncol][C]
    int *ok;            // [C]
    double2 *work;      // [C][8][D*D]
    int *iwork;         // [C][2*D]
    double2 *mom;       // [4][D][D]
    int *status;
};

__device__ __forceinline__ double zof(int wn, double beta) { return (2 * wn + 1) * DG_PI / beta; }

// weighted series term q of element ab at frequency wn (q < ncol: K^T G columns; q >= ncol: K^T K sums)
__device__ __forceinline__ double2 mom_term(const MomArgs &g, int series, int wn) {
    const int DD = g.D * g.D;
    const double z = zof(wn, g.beta), z2 = z * z, z3 = z2 * z;
    if (series < DD * g.ncol) {
        const int ab = series / g.ncol, c = series % g.ncol;
        const int a = ab / g.D, b = ab % g.D;  // momentstest index alp*Dim + bet
        const double2 fab = g.fw[(size_t)wn * DD + a + b * g.D], fba = g.fw[(size_t)wn * DD + b + a * g.D];
        const double2 re = cmk((fab.x + fba.x) / 2, (fab.y - fba.y) / 2);        // (F_ab + conj F_ba)/2
        double2 im = cmk((fab.y + fba.y) * 0.5, -(fab.x - fba.x) * 0.5);        // (F_ab - conj F_ba)/(2i)
        if (!g.green) {
            if (c == 0) return re;
            if (c == 1) return cscale(im, -1. / z);
            if (c == 2) return cscale(re, -1. / z2);
            return cscale(im, 1. / z3);
        }
        if (c == 0) return cscale(re, -1. / z2);
        if (a == b) im.x += 1.0 / z;
        return cscale(im, 1. / z3);
    }
    const int q = series - DD * g.ncol;
    double v;
    if (q == 0) v = 1.0;
    else if (q == 1) v = -1. / z2;                  // K(.,0) K(.,2) on Re rows
    else if (q == 2) v = (-1. / z2) * (-1. / z2);
    else if (q == 3) v = (-1. / z) * (-1. / z);
    else if (q == 4) v = (-1. / z) * (1. / z3);
    else v = (1. / z3) * (1. / z3);
    return cmk(v, 0.0);
}

// one warp per series: suffix sums S(w) = sum_{wn >= w} term(wn), lanes own contiguous chunks
__global__ void k_mom_suffix(MomArgs g) {
    const int DD = g.D * g.D;
    const int nseries = DD * g.ncol + 6;
    const int series = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (series >= nseries) return;  // warp-uniform
    const int chunk = (g.Nf + 31) / 32;
    const int lo = min(g.Nf, lane * chunk), hi = min(g.Nf, lo + chunk);
    double2 part = cmk(0, 0);
    for (int wn = hi - 1; wn >= lo; wn--) part = cadd(part, mom_term(g, series, wn));
    // carry = sum of the chunks of all higher lanes (inclusive suffix scan, then shift)
    double2 incl = part;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        double2 v = shfl2(incl, min(31, lane + off), 32);
        if (lane + off < 32) incl = cadd(incl, v);
    }
    double2 run = csub(incl, part);
    for (int wn = hi - 1; wn >= lo; wn--) {
        run = cadd(run, mom_term(g, series, wn));
        if (wn < g.R) {
            if (series < DD * g.ncol) {
                const int ab = series / g.ncol, c = series % g.ncol;
                g.S[((size_t)ab * g.ncol + c) * g.R + wn] = run;
            } else {
                g.KS[(size_t)(series - DD * g.ncol) * g.R + wn] = run.x;
            }
        }
    }
}

// one thread per window: (K^T K)^-1
__global__ void k_mom_kinv(MomArgs g) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= g.R) return;
    double2 K[16];
    int perm[4];
    for (int i = 0; i < 16; i++) K[i] = cmk(0, 0);
    const int n = g.ncol;
    if (!g.green) {
        K[0 + 0 * 4] = cmk(g.KS[0 * g.R + w], 0);
        K[0 + 2 * 4] = K[2 + 0 * 4] = cmk(g.KS[1 * g.R + w], 0);
        K[2 + 2 * 4] = cmk(g.KS[2 * g.R + w], 0);
        K[1 + 1 * 4] = cmk(g.KS[3 * g.R + w], 0);
        K[1 + 3 * 4] = K[3 + 1 * 4] = cmk(g.KS[4 * g.R + w], 0);
        K[3 + 3 * 4] = cmk(g.KS[5 * g.R + w], 0);
    } else {
        K[0 + 0 * 2] = cmk(g.KS[2 * g.R + w], 0);
        K[1 + 1 * 2] = cmk(g.KS[5 * g.R + w], 0);
    }
    if (thread_gj_inverse(n, K, perm)) dg_flag(g.status, DG_SINGULAR);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) g.kinv[(size_t)w * 16 + i + j * n] = K[i + j * n].x;
}

// one thread per (window, element): m_i = sum_c inv(i,c) (K^T G)_c, and the trace contributions
__global__ void k_mom_solve(MomArgs g) {
    const int DD = g.D * g.D;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.R * DD) return;
    int w = (int)(t / DD), ab = (int)(t % DD);
    const int n = g.ncol;
    const double *ki = g.kinv + (size_t)w * 16;
    for (int i = 0; i < n; i++) {
        double2 m = cmk(0, 0);
        for (int c = 0; c < n; c++) m = cadd(m, cscale(g.S[((size_t)ab * n + c) * g.R + w], ki[i + c * n]));
        g.mt[((size_t)ab * g.R + w) * n + i] = m;
    }
}

__global__ void k_mom_trace(MomArgs g) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.R * g.ncol) return;
    int w = t / g.ncol, i = t % g.ncol;
    double s = 0;
    for (int a = 0; a < g.D; a++) s += g.mt[((size_t)(a * g.D + a) * g.R + w) * g.ncol + i].x;
    g.tr[(size_t)i * g.R + w] = s;
}

// one thread per (centre, element, moment): window averages; one per (centre, moment): variance
// window averages of the fitted moments and variances of their traces over 2 Nv + 1 consecutive windows.
// One thread per run of AVG_RUN consecutive centres of one series: the first window is summed directly and
// the next ones by sliding (add the entering, drop the leaving term), restarting every AVG_RUN centres
constexpr int AVG_RUN = 32;
__global__ void k_mom_avg(MomArgs g) {
    const int DD = g.D * g.D, L = 2 * g.Nv + 1;
    const int nrun = (g.C + AVG_RUN - 1) / AVG_RUN;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long navg = (long long)nrun * DD * g.ncol;
    if (t < navg) {
        const int run = (int)(t % nrun);
        const long long r = t / nrun;
        const int i = (int)(r % g.ncol), ab = (int)(r / g.ncol);
        const int a = ab / g.D, b = ab % g.D;
        const double2 *x = g.mt + (size_t)ab * g.R * g.ncol + i;  // x[iw * ncol]
        const int c0 = run * AVG_RUN, c1 = min(g.C, c0 + AVG_RUN);
        double2 s = cmk(0, 0);
        for (int iw = c0; iw < c0 + L; iw++) s = cadd(s, x[(size_t)iw * g.ncol]);
        for (int ci = c0; ci < c1; ci++) {
            if (ci > c0) s = csub(cadd(s, x[(size_t)(ci + L - 1) * g.ncol]), x[(size_t)(ci - 1) * g.ncol]);
            // Eigen MatrixXcd(a,b) with ab = a*Dim + b; stored column-major
            g.avg[((size_t)i * g.C + ci) * DD + a + b * g.D] = cmk(s.x / L, s.y / L);
        }
    } else if (t < navg + (long long)g.C * g.ncol) {
        const long long u = t - navg;
        const int ci = (int)(u % g.C), i = (int)(u / g.C);
        const double *tr = g.tr + (size_t)i * g.R + ci;
        double mean = 0;
        for (int j = 0; j < L; j++) mean += tr[j];
        mean /= L;
        double ss = 0;
        for (int j = 0; j < L; j++) ss += (tr[j] - mean) * (tr[j] - mean);
        g.var[(size_t)i * g.C + ci] = sqrt(ss / L);
    }
}

// one thread per centre: the positivity gates of the window search
__global__ void k_mom_gate(MomArgs g) {
    int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= g.C) return;
    const int D = g.D, DD = D * D;
    double2 *W = g.work + (size_t)ci * 8 * DD;
    double2 *A = W, *U = W + DD, *T1 = W + 2 * DD, *T2 = W + 3 * DD, *T3 = W + 4 * DD, *X = W + 5 * DD;
    int *ord = g.iwork + (size_t)ci * 2 * D, *perm = ord + D;
    double *ev = (double *)(W + 6 * DD);  // D doubles fit in DD complex slots
    int okv = 0;
    if (!g.green) {
        const double2 *m1 = g.avg + ((size_t)1 * g.C + ci) * DD;
        const double2 *m2 = g.avg + ((size_t)2 * g.C + ci) * DD;
        const double2 *m3 = g.avg + ((size_t)3 * g.C + ci) * DD;
        thread_heig(D, m1, A, U, ev, ord);
        double a = ev[0];
        if (a > 0) {
            // V_inv = (U sqrt(ev) U^H)^-1
            for (int j = 0; j < D; j++)
                for (int i = 0; i < D; i++) {
                    double2 s = cmk(0, 0);
                    for (int l = 0; l < D; l++) s = cfma(cscale(DG_AT(U, D, i, l), sqrt(ev[l])), cconj(DG_AT(U, D, j, l)), s);
                    DG_AT(T1, D, i, j) = s;
                }
            thread_gj_inverse(D, T1, perm);                   // T1 = V_inv
            thread_matmul(D, T1, m2, T2);                     // V_inv m2
            thread_matmul(D, T2, T1, T3);                     // T3 = V_inv m2 V_inv
            thread_matmul(D, T1, m3, T2);                     // V_inv m3
            thread_matmul(D, T2, T1, X);                      // X = V_inv m3 V_inv
            thread_matmul(D, T3, T3, T2);                     // T2 = (V_inv m2 V_inv)^2
            for (int k = 0; k < DD; k++) X[k] = csub(X[k], T2[k]);
            thread_heig(D, X, A, nullptr, ev, ord);
            double b = ev[0];
            okv = (a > 0 && b > 0);
        }
    } else {
        const double2 *m0 = g.avg + ((size_t)0 * g.C + ci) * DD;
        const double2 *m1 = g.avg + ((size_t)1 * g.C + ci) * DD;
        thread_matmul(D, m0, m0, T1);
        for (int k = 0; k < DD; k++) X[k] = csub(m1[k], T1[k]);
        thread_heig(D, X, A, nullptr, ev, ord);
        okv = (ev[0] > 1);
    }
    g.ok[ci] = okv;
}

// the green-tail gate (m0 = 0, m1 = I fixed): min eig of (avg1 - avg0^2) > 1, i.e. (avg1 - avg0^2) - I positive
// definite, by a Cholesky factorisation of the lower triangle (the triangle the eigensolver would read)
__global__ void k_mom_gate_green(MomArgs g) {
    extern __shared__ double2 tri[];
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= g.C) return;
    const int D = g.D, DD = D * D, stride = blockDim.x;
    double2 *my = tri + threadIdx.x;
    const double2 *m0 = g.avg + ((size_t)0 * g.C + ci) * DD;
    const double2 *m1 = g.avg + ((size_t)1 * g.C + ci) * DD;
    for (int i = 0; i < D; i++)
        for (int j = 0; j <= i; j++) {
            double2 x = DG_AT(m1, D, i, j);
            for (int k = 0; k < D; k++) x = csub(x, cmul(DG_AT(m0, D, i, k), DG_AT(m0, D, k, j)));
            if (i == j) x = cmk(x.x - 1.0, 0.0);
            my[(size_t)((i * (i + 1)) / 2 + j) * stride] = x;
        }
    g.ok[ci] = posdef_tri(D, my, stride, true) ? 1 : 0;
}

// single block: window choice per moment and the final averaged, Hermitised moments
__global__ void k_mom_final(MomArgs g) {
    __shared__ int win[4];
    __shared__ double rv[256];
    __shared__ int ri[256];
    const int D = g.D, DD = D * D;
    // sequential argmin of the reference (minPos = C-1; minPos = i when ok[i] and var[i] < var[minPos]) as a
    // block reduction: the first index of the smallest var[i] among ok candidates with var[i] < var[C-1],
    // else C-1
    for (int m = 0; m < g.ncol; m++) {
        const double *var = g.var + (size_t)m * g.C;
        const double vlast = var[g.C - 1];
        double bv = 0;
        int bi = -1;
        for (int i = threadIdx.x; i < g.C; i += blockDim.x)
            if (g.ok[i] && var[i] < vlast && (bi < 0 || var[i] < bv)) {
                bv = var[i];
                bi = i;
            }
        rv[threadIdx.x] = bv;
        ri[threadIdx.x] = bi;
        __syncthreads();
        for (int h = blockDim.x / 2; h > 0; h >>= 1) {
            if (threadIdx.x < h) {
                const int oi = ri[threadIdx.x + h];
                const double ov = rv[threadIdx.x + h];
                const int mi = ri[threadIdx.x];
                if (oi >= 0 && (mi < 0 || ov < rv[threadIdx.x] || (ov == rv[threadIdx.x] && oi < mi))) {
                    rv[threadIdx.x] = ov;
                    ri[threadIdx.x] = oi;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) win[m] = ri[0] >= 0 ? ri[0] : g.C - 1;  // window iw in [win, win + 2 Nv]
        __syncthreads();
    }
    for (int t = threadIdx.x; t < 4 * DD; t += blockDim.x) {
        int mom = t / DD, e = t % DD;
        int a = e % D, b = e / D;  // column-major element (a, b)
        double2 val = cmk(0, 0);
        int src = g.green ? mom - 2 : mom;
        if (src >= 0) {
            int w0 = win[src];
            double2 s = cmk(0, 0);
            for (int w = w0; w <= w0 + 2 * g.Nv; w++) {
                double2 x = g.mt[((size_t)(a * D + b) * g.R + w) * g.ncol + src];
                double2 y = g.mt[((size_t)(b * D + a) * g.R + w) * g.ncol + src];
                s = cadd(s, cscale(cadd(x, cconj(y)), 0.5));
            }
            val = cmk(s.x / (2 * g.Nv + 1), s.y / (2 * g.Nv + 1));
        } else if (mom == 1) {
            val = cmk(a == b ? 1.0 : 0.0, 0.0);
        }
        g.mom[(size_t)mom * DD + a + b * D] = val;
    }
    __syncthreads();
    // (m + m^H)/2
    for (int t = threadIdx.x; t < 4 * DD; t += blockDim.x) {
        int mom = t / DD, e = t % DD;
        int a = e % D, b = e / D;
        if (a > b) continue;
        double2 x = g.mom[(size_t)mom * DD + a + b * D], y = g.mom[(size_t)mom * DD + b + a * D];
        double2 h = cscale(cadd(x, cconj(y)), 0.5);
        g.mom[(size_t)mom * DD + a + b * D] = h;
        g.mom[(size_t)mom * DD + b + a * D] = cconj(h);
    }
}

}  // namespace

int dg_moments_dev(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, const double2 *fw, int green,
                   double2 *mom) {
    MomArgs g;
    g.D = dim;
    g.Nf = nfreq;
    g.green = green ? 1 : 0;
    g.ncol = green ? 2 : 4;
    g.R = green ? nfreq - 1 : nfreq - 3;
    g.Nv = nfreq / 20;
    if (g.Nv == 0) g.Nv = 1;
    g.C = g.R - 2 * g.Nv;
    g.beta = beta;
    if (dim < 1 || g.R < 1 || g.C < 1) return dg_fail(ctx, DMFTGPU_BADARG, "moments: N_freq too small");
    const size_t DD = (size_t)dim * dim;
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    size_t oS = carve(DD * g.ncol * g.R * sizeof(double2)), oKS = carve(6 * g.R * sizeof(double)),
           oKi = carve((size_t)g.R * 16 * sizeof(double)), oMt = carve(DD * g.R * g.ncol * sizeof(double2)),
           oTr = carve((size_t)g.ncol * g.R * sizeof(double)), oAvg = carve((size_t)g.ncol * g.C * DD * sizeof(double2)),
           oVar = carve((size_t)g.ncol * g.C * sizeof(double)), oOk = carve((size_t)g.C * sizeof(int)),
           oW = carve((size_t)g.C * 8 * DD * sizeof(double2)), oIw = carve((size_t)g.C * 2 * dim * sizeof(int));
    char *base = (char *)dg_buf(ctx, "moments.work", off);
    if (!base) return DMFTGPU_NOMEM;
    g.fw = fw;
    g.S = (double2 *)(base + oS);
    g.KS = (double *)(base + oKS);
    g.kinv = (double *)(base + oKi);
    g.mt = (double2 *)(base + oMt);
    g.tr = (double *)(base + oTr);
    g.avg = (double2 *)(base + oAvg);
    g.var = (double *)(base + oVar);
    g.ok = (int *)(base + oOk);
    g.work = (double2 *)(base + oW);
    g.iwork = (int *)(base + oIw);
    g.mom = mom;
    g.status = ctx->d_status;
    cudaStream_t s = ctx->stream;
    int nseries = (int)(DD * g.ncol + 6);
    k_mom_suffix<<<dg_ceil_div(nseries, 4), 128, 0, s>>>(g);
    DG_LAUNCH(ctx, "k_mom_suffix");
    k_mom_kinv<<<dg_ceil_div(g.R, 128), 128, 0, s>>>(g);
    DG_LAUNCH(ctx, "k_mom_kinv");
    k_mom_solve<<<dg_ceil_div((long long)g.R * DD, 256), 256, 0, s>>>(g);
    DG_LAUNCH(ctx, "k_mom_solve");
    k_mom_trace<<<dg_ceil_div(g.R * g.ncol, 256), 256, 0, s>>>(g);
    DG_LAUNCH(ctx, "k_mom_trace");
    long long navg = (long long)((g.C + AVG_RUN - 1) / AVG_RUN) * DD * g.ncol + (long long)g.C * g.ncol;
    k_mom_avg<<<dg_ceil_div(navg, 256), 256, 0, s>>>(g);
    DG_LAUNCH(ctx, "k_mom_avg");
    if (g.green) {
        const int nt = posdef_threads(dim);
        const size_t sm = (size_t)nt * dim * (dim + 1) / 2 * sizeof(double2);
        DG_CUDA(cudaFuncSetAttribute(k_mom_gate_green, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_mom_gate_green<<<dg_ceil_div(g.C, nt), nt, sm, s>>>(g);
        DG_LAUNCH(ctx, "k_mom_gate_green");
    } else {
        k_mom_gate<<<dg_ceil_div(g.C, 64), 64, 0, s>>>(g);
        DG_LAUNCH(ctx, "k_mom_gate");
    }
    k_mom_final<<<1, 256, 0, s>>>(g);
    DG_LAUNCH(ctx, "k_mom_final");
    return DMFTGPU_OK;
}

extern "C" int dmftgpu_moments(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, const double *fw, int green_asym,
                               double *mom, int flags) {
    if (!ctx || !fw || !mom || dim < 1 || nfreq < 1) return DMFTGPU_BADARG;
    cudaSetDevice(ctx->device);
    int st;
    size_t DD = (size_t)dim * dim;
    const double2 *dfw = (const double2 *)dg_in(ctx, fw, nfreq * DD * sizeof(double2), flags, "io.fw", &st);
    if (st) return st;
    double2 *dmom = (double2 *)dg_out(ctx, mom, 4 * DD * sizeof(double2), flags, "io.mom", &st);
    if (st) return st;
    DG_TRY(dg_status_reset(ctx));
    DG_TRY(dg_moments_dev(ctx, dim, nfreq, beta, dfw, green_asym, dmom));
    DG_TRY(dg_out_done(ctx, mom, dmom, 4 * DD * sizeof(double2), flags));
    int code = 0;
    DG_TRY(dg_status_read(ctx, &code));
    return code ? code : DMFTGPU_OK;
}
