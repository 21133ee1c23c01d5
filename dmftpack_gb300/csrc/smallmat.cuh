// smallmat.cuh -- block- and thread-level routines for the few small (n <= 32) Hermitian matrices of the
// impurity stage, all working in SHARED memory (the thread_* routines of linalg.cuh work in global scratch
// and are latency-bound there).
//
//  * block_heig: Hermitian eigen-decomposition by one thread block.  Like thread_heig (and
//    Eigen::SelfAdjointEigenSolver) it reads only the lower triangle, takes the diagonal real and returns
//    ascending eigenvalues, with the same complex Jacobi rotation and the same stopping rule
//    (off-diagonal mass <= 1e-28 of the total); the rotations of one sweep are applied in round-robin
//    ("tournament") order, n/2 disjoint (p, q) pairs at a time, so a sweep takes n - 1 parallel steps.
//  * block_matmul: C = A B, one thread per element.
//  * posdef_lower: is the Hermitian matrix s * (lower triangle of M) - shift * I positive definite (strict)
//    or positive semidefinite?  A Cholesky factorisation answers the eigenvalue-sign questions of the
//    reference (min eigenvalue >= 0 in the positivity fix-up, max eigenvalue < 0 in the causality checks,
//    min eigenvalue > 1 in the moment gate) with ~n^3/6 operations instead of a full eigensolve.  The
//    semidefinite variant accepts an exactly zero pivot when the rest of its column is exactly zero.
#pragma once
#include "linalg.cuh"

struct DgRot {
    int p, q, on;
    double c, s;
    double2 ph;
};

// all threads of the block call it; a, u: n*n shared, w: n shared doubles, order: n shared ints,
// rot: n/2+1 shared DgRot, red: blockDim.x shared doubles.  Returns DG_OK or DG_NONCONV (block-uniform).
__device__ inline int block_heig(int n, const double2 *A0, double2 *a, double2 *u, double *w, int *order, DgRot *rot,
                                 double *red) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < n * n; e += nt) {
        const int i = e % n, j = e / n;
        double2 v;
        if (i > j) v = DG_AT(A0, n, i, j);
        else if (i < j) v = cconj(DG_AT(A0, n, j, i));
        else v = cmk(DG_AT(A0, n, i, i).x, 0.0);
        a[e] = v;
        if (u) u[e] = cmk(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    const int m = n + (n & 1), half = m / 2;
    __shared__ int conv;
    int st = DG_NONCONV;
    for (int sweep = 0; sweep < 100; sweep++) {
        // off-diagonal and total mass
        double off = 0, tot = 0;
        for (int e = tid; e < n * n; e += nt) {
            const double v = cabs2(a[e]);
            tot += v;
            if (e % n != e / n) off += v;
        }
        red[tid] = off;
        __syncthreads();
        for (int h = nt / 2; h > 0; h >>= 1) {
            if (tid < h) red[tid] += red[tid + h];
            __syncthreads();
        }
        const double offs = red[0];
        __syncthreads();
        red[tid] = tot;
        __syncthreads();
        for (int h = nt / 2; h > 0; h >>= 1) {
            if (tid < h) red[tid] += red[tid + h];
            __syncthreads();
        }
        if (tid == 0) conv = (offs == 0.0 || offs <= 1e-28 * red[0]);
        __syncthreads();
        if (conv) {
            st = DG_OK;
            break;
        }
        for (int r = 0; r < m - 1; r++) {
            // pairs of round r: (r, m-1) and ((r+k) mod (m-1), (r-k) mod (m-1)), k = 1 .. half-1
            if (tid < half) {
                int p, q;
                if (tid == 0) {
                    p = r;
                    q = m - 1;
                } else {
                    p = (r + tid) % (m - 1);
                    q = (r - tid + (m - 1)) % (m - 1);
                }
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                DgRot R;
                R.p = p;
                R.q = q;
                R.on = 0;
                R.c = 1.0;
                R.s = 0.0;
                R.ph = cmk(1, 0);
                if (q < n) {
                    const double2 apq = DG_AT(a, n, p, q);
                    const double rr = sqrt(cabs2(apq));
                    if (rr != 0.0) {
                        const double app = DG_AT(a, n, p, p).x, aqq = DG_AT(a, n, q, q).x;
                        const double theta = (aqq - app) / (2.0 * rr);
                        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        R.c = 1.0 / sqrt(t * t + 1.0);
                        R.s = t * R.c;
                        R.ph = cmk(apq.x / rr, apq.y / rr);
                        R.on = 1;
                    }
                }
                rot[tid] = R;
            }
            __syncthreads();
            // columns p, q of a (and u): a(:,p) = c a(:,p) - s conj(ph) a(:,q); a(:,q) = s a(:,p) + c conj(ph) a(:,q)
            for (int x = tid; x < half * n; x += nt) {
                const DgRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const double2 phc = cconj(R.ph);
                const double2 akp = DG_AT(a, n, k, R.p), akq = DG_AT(a, n, k, R.q);
                DG_AT(a, n, k, R.p) = csub(cscale(akp, R.c), cscale(cmul(phc, akq), R.s));
                DG_AT(a, n, k, R.q) = cadd(cscale(akp, R.s), cscale(cmul(phc, akq), R.c));
                if (u) {
                    const double2 ukp = DG_AT(u, n, k, R.p), ukq = DG_AT(u, n, k, R.q);
                    DG_AT(u, n, k, R.p) = csub(cscale(ukp, R.c), cscale(cmul(phc, ukq), R.s));
                    DG_AT(u, n, k, R.q) = cadd(cscale(ukp, R.s), cscale(cmul(phc, ukq), R.c));
                }
            }
            __syncthreads();
            // rows p, q: a(p,:) = c a(p,:) - s ph a(q,:); a(q,:) = s a(p,:) + c ph a(q,:)
            for (int x = tid; x < half * n; x += nt) {
                const DgRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const double2 apk = DG_AT(a, n, R.p, k), aqk = DG_AT(a, n, R.q, k);
                DG_AT(a, n, R.p, k) = csub(cscale(apk, R.c), cscale(cmul(R.ph, aqk), R.s));
                DG_AT(a, n, R.q, k) = cadd(cscale(apk, R.s), cscale(cmul(R.ph, aqk), R.c));
            }
            __syncthreads();
            if (tid < half) {
                const DgRot R = rot[tid];
                if (R.on) {
                    DG_AT(a, n, R.p, R.q) = cmk(0, 0);
                    DG_AT(a, n, R.q, R.p) = cmk(0, 0);
                    DG_AT(a, n, R.p, R.p).y = 0.0;
                    DG_AT(a, n, R.q, R.q).y = 0.0;
                }
            }
            __syncthreads();
        }
    }
    if (tid == 0) {
        for (int i = 0; i < n; i++) order[i] = i;
        for (int i = 1; i < n; i++) {
            const int v = order[i];
            const double key = DG_AT(a, n, v, v).x;
            int j = i - 1;
            while (j >= 0 && DG_AT(a, n, order[j], order[j]).x > key) {
                order[j + 1] = order[j];
                j--;
            }
            order[j + 1] = v;
        }
        for (int i = 0; i < n; i++) w[i] = DG_AT(a, n, order[i], order[i]).x;
    }
    __syncthreads();
    if (u) {
        for (int e = tid; e < n * n; e += nt) a[e] = u[e];
        __syncthreads();
        for (int e = tid; e < n * n; e += nt) {
            const int k = e % n, i = e / n;
            DG_AT(u, n, k, i) = DG_AT(a, n, k, order[i]);
        }
        __syncthreads();
    }
    return st;
}

// block_heig for one warp (n <= 64): the same rotations, order and stopping rule, synchronised with __syncwarp
// (a butterfly reduction of the off-diagonal mass, the stopping decision taken from lane 0), so several small
// matrices share a thread block without block-wide barriers.  All 32 lanes call it; a, u: n*n shared (this warp's),
// w: n doubles, order: n ints, rot: n/2+1 DgRot, all this warp's.  Returns DG_OK or DG_NONCONV (warp-uniform).
__device__ inline int warp_heig(int n, const double2 *A0, double2 *a, double2 *u, double *w, int *order, DgRot *rot) {
    const int lane = threadIdx.x & 31;
    for (int e = lane; e < n * n; e += 32) {
        const int i = e % n, j = e / n;
        double2 v;
        if (i > j) v = DG_AT(A0, n, i, j);
        else if (i < j) v = cconj(DG_AT(A0, n, j, i));
        else v = cmk(DG_AT(A0, n, i, i).x, 0.0);
        a[e] = v;
        u[e] = cmk(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncwarp();
    const int m = n + (n & 1), half = m / 2;
    int st = DG_NONCONV;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (int e = lane; e < n * n; e += 32) {
            const double v = cabs2(a[e]);
            tot += v;
            if (e % n != e / n) off += v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        const int conv = __shfl_sync(0xffffffffu, (int)(off == 0.0 || off <= 1e-28 * tot), 0);
        if (conv) {
            st = DG_OK;
            break;
        }
        for (int r = 0; r < m - 1; r++) {
            if (lane < half) {
                int p, q;
                if (lane == 0) {
                    p = r;
                    q = m - 1;
                } else {
                    p = (r + lane) % (m - 1);
                    q = (r - lane + (m - 1)) % (m - 1);
                }
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                DgRot R;
                R.p = p;
                R.q = q;
                R.on = 0;
                R.c = 1.0;
                R.s = 0.0;
                R.ph = cmk(1, 0);
                if (q < n) {
                    const double2 apq = DG_AT(a, n, p, q);
                    const double rr = sqrt(cabs2(apq));
                    if (rr != 0.0) {
                        const double app = DG_AT(a, n, p, p).x, aqq = DG_AT(a, n, q, q).x;
                        const double theta = (aqq - app) / (2.0 * rr);
                        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        R.c = 1.0 / sqrt(t * t + 1.0);
                        R.s = t * R.c;
                        R.ph = cmk(apq.x / rr, apq.y / rr);
                        R.on = 1;
                    }
                }
                rot[lane] = R;
            }
            __syncwarp();
            for (int x = lane; x < half * n; x += 32) {
                const DgRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const double2 phc = cconj(R.ph);
                const double2 akp = DG_AT(a, n, k, R.p), akq = DG_AT(a, n, k, R.q);
                DG_AT(a, n, k, R.p) = csub(cscale(akp, R.c), cscale(cmul(phc, akq), R.s));
                DG_AT(a, n, k, R.q) = cadd(cscale(akp, R.s), cscale(cmul(phc, akq), R.c));
                const double2 ukp = DG_AT(u, n, k, R.p), ukq = DG_AT(u, n, k, R.q);
                DG_AT(u, n, k, R.p) = csub(cscale(ukp, R.c), cscale(cmul(phc, ukq), R.s));
                DG_AT(u, n, k, R.q) = cadd(cscale(ukp, R.s), cscale(cmul(phc, ukq), R.c));
            }
            __syncwarp();
            for (int x = lane; x < half * n; x += 32) {
                const DgRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const double2 apk = DG_AT(a, n, R.p, k), aqk = DG_AT(a, n, R.q, k);
                DG_AT(a, n, R.p, k) = csub(cscale(apk, R.c), cscale(cmul(R.ph, aqk), R.s));
                DG_AT(a, n, R.q, k) = cadd(cscale(apk, R.s), cscale(cmul(R.ph, aqk), R.c));
            }
            __syncwarp();
            if (lane < half) {
                const DgRot R = rot[lane];
                if (R.on) {
                    DG_AT(a, n, R.p, R.q) = cmk(0, 0);
                    DG_AT(a, n, R.q, R.p) = cmk(0, 0);
                    DG_AT(a, n, R.p, R.p).y = 0.0;
                    DG_AT(a, n, R.q, R.q).y = 0.0;
                }
            }
            __syncwarp();
        }
    }
    if (lane == 0) {
        for (int i = 0; i < n; i++) order[i] = i;
        for (int i = 1; i < n; i++) {
            const int v = order[i];
            const double key = DG_AT(a, n, v, v).x;
            int j = i - 1;
            while (j >= 0 && DG_AT(a, n, order[j], order[j]).x > key) {
                order[j + 1] = order[j];
                j--;
            }
            order[j + 1] = v;
        }
        for (int i = 0; i < n; i++) w[i] = DG_AT(a, n, order[i], order[i]).x;
    }
    __syncwarp();
    for (int e = lane; e < n * n; e += 32) a[e] = u[e];
    __syncwarp();
    for (int e = lane; e < n * n; e += 32) {
        const int k = e % n, i = e / n;
        DG_AT(u, n, k, i) = DG_AT(a, n, k, order[i]);
    }
    __syncwarp();
    return st;
}

// C = A B (n x n, all shared or global, C distinct from A and B); all threads call it; ends with a barrier
__device__ inline void block_matmul(int n, const double2 *A, const double2 *B, double2 *C) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        double2 s = cmk(0, 0);
        for (int k = 0; k < n; k++) s = cfma(DG_AT(A, n, i, k), DG_AT(B, n, k, j), s);
        C[e] = s;
    }
    __syncthreads();
}

// Cholesky test of one n x n Hermitian matrix held as its lower triangle in t[idx(i, j)] (i >= j), with
// t[idx] = tri[(idx) * stride] (stride = threads sharing the interleaved shared array).  Destroys t.
// strict: positive definite; else positive semidefinite (an exactly zero pivot with an exactly zero
// remaining column is skipped).
__host__ __device__ inline bool posdef_tri(int n, double2 *t, int stride, bool strict) {
#define DG_TRI(i, j) t[(size_t)(((i) * ((i) + 1)) / 2 + (j)) * stride]
    for (int j = 0; j < n; j++) {
        const double p = DG_TRI(j, j).x;
        if (strict ? !(p > 0.0) : !(p >= 0.0)) return false;
        if (p == 0.0) {
            for (int i = j + 1; i < n; i++)
                if (DG_TRI(i, j).x != 0.0 || DG_TRI(i, j).y != 0.0) return false;
            continue;
        }
        const double r = 1.0 / sqrt(p);
        for (int i = j + 1; i < n; i++) DG_TRI(i, j) = cscale(DG_TRI(i, j), r);
        for (int k = j + 1; k < n; k++) {
            const double2 lkj = DG_TRI(k, j);
            for (int i = k; i < n; i++) DG_TRI(i, k) = csub(DG_TRI(i, k), cmul(DG_TRI(i, j), cconj(lkj)));
            DG_TRI(k, k).y = 0.0;
        }
    }
    return true;
#undef DG_TRI
}

// threads per block for one-matrix-per-thread Cholesky tests on d x d matrices, their lower triangles
// interleaved in shared memory (<= 96 KiB per block)
inline int posdef_threads(int d) {
    const size_t tri = (size_t)d * (d + 1) / 2 * sizeof(double2);
    int t = 64;
    while (t > 1 && (size_t)t * tri > 96 * 1024) t >>= 1;
    return t;
}
