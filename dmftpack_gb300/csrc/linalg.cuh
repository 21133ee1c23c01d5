// linalg.cuh -- small dense complex linear algebra on the device.
//
// Every warp shuffle below is executed by all 32 lanes under warp-uniform control flow: several lane
// groups can share a warp, and their data-dependent choices (pivot rows) never gate a shuffle.
//
//  * warp_gj_inverse<N,W>: one lane group of W lanes (W = power of two >= N) inverts an N x N complex
//    matrix held one COLUMN PER LANE in registers: Gauss-Jordan with partial (row) pivoting, pivot search
//    inside the pivot column's lane, pivot row/column broadcast by warp shuffles, and the final column
//    un-permutation done as lane exchanges (shuffles take a runtime source lane, so no dynamic register
//    indexing is ever needed).  Pivot rule = largest |a_ij| in the column, as Eigen's PartialPivLU.
//  * thread_*: one thread works on matrices in global scratch (column-major, ld = n): Gauss-Jordan
//    inverse with partial pivoting and a cyclic complex Jacobi Hermitian eigensolver that, like
//    Eigen::SelfAdjointEigenSolver, reads only the lower triangle (diagonal taken real) and returns
//    ascending eigenvalues.  Used where matrices are few (per k point, per tau point, per fit window).
#pragma once
#include "common.cuh"

enum { DG_OK = 0, DG_SINGULAR = 1, DG_NONCONV = 2, DG_NAN = 3, DG_BADARG = 4, DG_CAUSAL = 5, DG_HERMIT = 6 };

template <int N, int W>
__device__ __forceinline__ bool warp_gj_inverse(double2 (&a)[N], const int c) {
    static_assert(N <= W && W <= 32 && (W & (W - 1)) == 0, "bad lane group");
    bool singular = false;
    int perm[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        // pivot search over rows j..N-1 of column j (lane j); every lane scans its own column and
        // then takes lane j's answer
        double best = -1.0;
        int p = j;
#pragma unroll
        for (int i = j; i < N; i++) {
            double v = cabs2(a[i]);
            if (v > best) { best = v; p = i; }
        }
        p = __shfl_sync(0xffffffffu, p, j, W);
        best = __shfl_sync(0xffffffffu, best, j, W);
        singular |= !(best > 0.0);
        perm[j] = p;
#pragma unroll
        for (int i = j + 1; i < N; i++)
            if (i == p) {
                double2 t = a[j];
                a[j] = a[i];
                a[i] = t;
            }
        const double2 piv = shfl2(a[j], j, W);
        const double2 ipiv = crcp(piv);
        const double2 t = cmul(a[j], ipiv);  // new row-j entry of this lane's column
        const bool is_piv_col = (c == j);
        const double2 tu = is_piv_col ? ipiv : t;  // the pivot column's entries become cfms(f, ipiv, 0) = -f ipiv
#pragma unroll
        for (int i = 0; i < N; i++) {
            if (i == j) continue;
            const double2 f = shfl2(a[i], j, W);  // a_ij before the update (lane j's register i)
            a[i] = cfms(f, tu, is_piv_col ? cmk(0.0, 0.0) : a[i]);
        }
        a[j] = is_piv_col ? ipiv : t;
    }
    // undo the row interchanges as column interchanges, last first.  The exchange is unconditional:
    // lane groups that share a warp have different pivot sequences, so a branch on p != j would diverge
    // around the full-mask shuffles.
#pragma unroll
    for (int j = N - 1; j >= 0; j--) {
        const int p = perm[j];
        const int src = (c == j) ? p : ((c == p) ? j : c);
#pragma unroll
        for (int i = 0; i < N; i++) a[i] = shfl2(a[i], src, W);
    }
    return singular;
}

// ---------------------------------------------------------------------------------------------------
// thread-level routines on global-memory scratch
// ---------------------------------------------------------------------------------------------------
#define DG_AT(A, n, i, j) (A)[(i) + (size_t)(j) * (n)]

__host__ __device__ inline int thread_gj_inverse(int n, double2 *a, int *perm) {
    int st = DG_OK;
    for (int j = 0; j < n; j++) {
        int p = j;
        double best = -1.0;
        for (int i = j; i < n; i++) {
            double v = cabs2(DG_AT(a, n, i, j));
            if (v > best) { best = v; p = i; }
        }
        if (!(best > 0.0)) st = DG_SINGULAR;
        perm[j] = p;
        if (p != j)
            for (int c = 0; c < n; c++) {
                double2 t = DG_AT(a, n, j, c);
                DG_AT(a, n, j, c) = DG_AT(a, n, p, c);
                DG_AT(a, n, p, c) = t;
            }
        double2 ip = crcp(DG_AT(a, n, j, j));
        for (int c = 0; c < n; c++) {
            if (c == j) continue;
            double2 t = cmul(DG_AT(a, n, j, c), ip);
            DG_AT(a, n, j, c) = t;
            for (int i = 0; i < n; i++)
                if (i != j) DG_AT(a, n, i, c) = cfms(DG_AT(a, n, i, j), t, DG_AT(a, n, i, c));
        }
        for (int i = 0; i < n; i++)
            if (i != j) DG_AT(a, n, i, j) = cneg(cmul(DG_AT(a, n, i, j), ip));
        DG_AT(a, n, j, j) = ip;
    }
    for (int j = n - 1; j >= 0; j--) {
        int p = perm[j];
        if (p != j)
            for (int i = 0; i < n; i++) {
                double2 t = DG_AT(a, n, i, j);
                DG_AT(a, n, i, j) = DG_AT(a, n, i, p);
                DG_AT(a, n, i, p) = t;
            }
    }
    return st;
}

// C = A * B   (all n x n, distinct buffers)
__host__ __device__ inline void thread_matmul(int n, const double2 *A, const double2 *B, double2 *C) {
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double2 s = cmk(0, 0);
            for (int k = 0; k < n; k++) s = cfma(DG_AT(A, n, i, k), DG_AT(B, n, k, j), s);
            DG_AT(C, n, i, j) = s;
        }
}

// Hermitian eigen-decomposition from the lower triangle of A0 (A0 untouched).  a, u: n x n scratch;
// w: n eigenvalues ascending; if u == nullptr only eigenvalues are produced (a still needed).
// Cyclic Jacobi: the rotation G = [[c, s], [-s conj(u), c conj(u)]] zeroes the (p,q) element of G^H A G.
__host__ __device__ inline int thread_heig(int n, const double2 *A0, double2 *a, double2 *u, double *w, int *order) {
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double2 v;
            if (i > j) v = DG_AT(A0, n, i, j);
            else if (i < j) v = cconj(DG_AT(A0, n, j, i));
            else v = cmk(DG_AT(A0, n, i, i).x, 0.0);
            DG_AT(a, n, i, j) = v;
            if (u) DG_AT(u, n, i, j) = cmk(i == j ? 1.0 : 0.0, 0.0);
        }
    int st = DG_NONCONV;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) {
                double v = cabs2(DG_AT(a, n, i, j));
                tot += v;
                if (i != j) off += v;
            }
        if (off == 0.0 || off <= 1e-28 * tot) {
            st = DG_OK;
            break;
        }
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double2 apq = DG_AT(a, n, p, q);
                double r = sqrt(cabs2(apq));
                if (r == 0.0) continue;
                double app = DG_AT(a, n, p, p).x, aqq = DG_AT(a, n, q, q).x;
                double theta = (aqq - app) / (2.0 * r);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
                double2 ph = cmk(apq.x / r, apq.y / r), phc = cconj(ph);
                for (int k = 0; k < n; k++) {
                    double2 akp = DG_AT(a, n, k, p), akq = DG_AT(a, n, k, q);
                    DG_AT(a, n, k, p) = csub(cscale(akp, cs), cscale(cmul(phc, akq), sn));
                    DG_AT(a, n, k, q) = cadd(cscale(akp, sn), cscale(cmul(phc, akq), cs));
                }
                for (int k = 0; k < n; k++) {
                    double2 apk = DG_AT(a, n, p, k), aqk = DG_AT(a, n, q, k);
                    DG_AT(a, n, p, k) = csub(cscale(apk, cs), cscale(cmul(ph, aqk), sn));
                    DG_AT(a, n, q, k) = cadd(cscale(apk, sn), cscale(cmul(ph, aqk), cs));
                }
                DG_AT(a, n, p, q) = cmk(0, 0);
                DG_AT(a, n, q, p) = cmk(0, 0);
                DG_AT(a, n, p, p).y = 0.0;
                DG_AT(a, n, q, q).y = 0.0;
                if (u)
                    for (int k = 0; k < n; k++) {
                        double2 ukp = DG_AT(u, n, k, p), ukq = DG_AT(u, n, k, q);
                        DG_AT(u, n, k, p) = csub(cscale(ukp, cs), cscale(cmul(phc, ukq), sn));
                        DG_AT(u, n, k, q) = cadd(cscale(ukp, sn), cscale(cmul(phc, ukq), cs));
                    }
            }
    }
    // ascending order (stable insertion sort on indices), eigenvectors permuted alongside
    for (int i = 0; i < n; i++) order[i] = i;
    for (int i = 1; i < n; i++) {
        int v = order[i];
        double key = DG_AT(a, n, v, v).x;
        int j = i - 1;
        while (j >= 0 && DG_AT(a, n, order[j], order[j]).x > key) {
            order[j + 1] = order[j];
            j--;
        }
        order[j + 1] = v;
    }
    for (int i = 0; i < n; i++) w[i] = DG_AT(a, n, order[i], order[i]).x;
    if (u) {
        // permute columns of u in place through a (a is free now): a <- u, u(:, i) = a(:, order[i])
        for (size_t k = 0; k < (size_t)n * n; k++) a[k] = u[k];
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) DG_AT(u, n, i, j) = DG_AT(a, n, i, order[j]);
    }
    return st;
}
