// smallmat_df.cuh -- warp_heig (smallmat.cuh) for either arithmetic policy of df.cuh: the Jacobi rotations'
// parameters are computed in FP64 from the current entries (one lane per pair, as before), while the O(n^3)
// column and row updates of the matrix and of the eigenvectors run in the policy's arithmetic.  With OpsF the
// updates run in double-float on the FP32 pipe, several times the FP64 rate of GB300; the double-float rounding
// floor (~2^-47 of the entries) leaves an off-diagonal mass near 1e-27 of the total, so the caller passes a
// stopping tolerance that the arithmetic can reach (1e-28 for OpsD, as Eigen-level FP64; 1e-24 for OpsF).
#pragma once
#include "df.cuh"
#include "smallmat.cuh"

template <class Ops>
struct RotArith;
template <>
struct RotArith<OpsD> {
    typedef double R;
    static __device__ __forceinline__ R real(double x) { return x; }
    static __device__ __forceinline__ double2 scale(double2 a, R r) { return cscale(a, r); }
};
template <>
struct RotArith<OpsF> {
    typedef dfl R;
    static __device__ __forceinline__ R real(double x) { return df_make(x); }
    static __device__ __forceinline__ cdf scale(cdf a, R r) { return {df_mul(a.re, r), df_mul(a.im, r)}; }
};

// All 32 lanes call it; A0 (read-only), a, u: n*n of Ops::C in shared memory; w: n doubles; order: n ints;
// rot: n/2+1 DgRot.  Eigenvalues ascending in w, eigenvectors (columns) in u.  Returns DG_OK or DG_NONCONV.
template <class Ops>
__device__ inline int warp_heig_t(int n, const typename Ops::C *A0, typename Ops::C *a, typename Ops::C *u, double *w,
                                  int *order, DgRot *rot, double tol) {
    typedef typename Ops::C C;
    typedef RotArith<Ops> RA;
    const int lane = threadIdx.x & 31;
    for (int e = lane; e < n * n; e += 32) {
        const int i = e % n, j = e / n;
        C v;
        if (i > j) v = DG_AT(A0, n, i, j);
        else if (i < j) v = Ops::from(cconj(Ops::to(DG_AT(A0, n, j, i))));
        else v = Ops::from(cmk(Ops::to(DG_AT(A0, n, i, i)).x, 0.0));
        a[e] = v;
        u[e] = (i == j) ? Ops::one() : Ops::zero();
    }
    __syncwarp();
    const int m = n + (n & 1), half = m / 2;
    int st = DG_NONCONV;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (int e = lane; e < n * n; e += 32) {
            const double v = cabs2(Ops::to(a[e]));
            tot += v;
            if (e % n != e / n) off += v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        const int conv = __shfl_sync(0xffffffffu, (int)(off == 0.0 || off <= tol * tot), 0);
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
                    const double2 apq = Ops::to(DG_AT(a, n, p, q));
                    const double rr = sqrt(cabs2(apq));
                    if (rr != 0.0) {
                        const double app = Ops::to(DG_AT(a, n, p, p)).x, aqq = Ops::to(DG_AT(a, n, q, q)).x;
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
            // columns p, q: x(:,p) = c x(:,p) - s conj(ph) x(:,q); x(:,q) = s x(:,p) + c conj(ph) x(:,q)
            for (int x = lane; x < half * n; x += 32) {
                const DgRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const typename RA::R c = RA::real(R.c), s = RA::real(R.s);
                const C sphc = Ops::from(cscale(cconj(R.ph), R.s)), cphc = Ops::from(cscale(cconj(R.ph), R.c));
                const C akp = DG_AT(a, n, k, R.p), akq = DG_AT(a, n, k, R.q);
                DG_AT(a, n, k, R.p) = Ops::fms(sphc, akq, RA::scale(akp, c));
                DG_AT(a, n, k, R.q) = Ops::fma(cphc, akq, RA::scale(akp, s));
                const C ukp = DG_AT(u, n, k, R.p), ukq = DG_AT(u, n, k, R.q);
                DG_AT(u, n, k, R.p) = Ops::fms(sphc, ukq, RA::scale(ukp, c));
                DG_AT(u, n, k, R.q) = Ops::fma(cphc, ukq, RA::scale(ukp, s));
            }
            __syncwarp();
            // rows p, q: x(p,:) = c x(p,:) - s ph x(q,:); x(q,:) = s x(p,:) + c ph x(q,:)
            for (int x = lane; x < half * n; x += 32) {
                const DgRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const typename RA::R c = RA::real(R.c), s = RA::real(R.s);
                const C sph = Ops::from(cscale(R.ph, R.s)), cph = Ops::from(cscale(R.ph, R.c));
                const C apk = DG_AT(a, n, R.p, k), aqk = DG_AT(a, n, R.q, k);
                DG_AT(a, n, R.p, k) = Ops::fms(sph, aqk, RA::scale(apk, c));
                DG_AT(a, n, R.q, k) = Ops::fma(cph, aqk, RA::scale(apk, s));
            }
            __syncwarp();
            if (lane < half) {
                const DgRot R = rot[lane];
                if (R.on) {
                    DG_AT(a, n, R.p, R.q) = Ops::zero();
                    DG_AT(a, n, R.q, R.p) = Ops::zero();
                    DG_AT(a, n, R.p, R.p) = Ops::from(cmk(Ops::to(DG_AT(a, n, R.p, R.p)).x, 0.0));
                    DG_AT(a, n, R.q, R.q) = Ops::from(cmk(Ops::to(DG_AT(a, n, R.q, R.q)).x, 0.0));
                }
            }
            __syncwarp();
        }
    }
    if (lane == 0) {
        for (int i = 0; i < n; i++) order[i] = i;
        for (int i = 1; i < n; i++) {
            const int v = order[i];
            const double key = Ops::to(DG_AT(a, n, v, v)).x;
            int j = i - 1;
            while (j >= 0 && Ops::to(DG_AT(a, n, order[j], order[j])).x > key) {
                order[j + 1] = order[j];
                j--;
            }
            order[j + 1] = v;
        }
        for (int i = 0; i < n; i++) w[i] = Ops::to(DG_AT(a, n, order[i], order[i])).x;
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
