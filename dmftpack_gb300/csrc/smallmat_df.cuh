// smallmat_df.cuh -- the warp-per-matrix cyclic Jacobi eigensolver (warp_heig, smallmat.cuh) entirely in
// double-float arithmetic on the FP32 pipe: the rotation parameters as well as the row and column updates.
//
// On GB300 an FP64 warp instruction occupies the SM's FP64 unit for ~16 cycles whether one lane or 32 are active,
// so both the FP64 updates and the per-round rotation parameters (square roots and divisions computed by a few
// lanes) run at the FP64 rate; here every step is a double-float operation (~2^-47 relative), and the rotation
// stays unitary to that precision because c = 1/sqrt(1 + t^2), s = t c and the phase ph = a_pq/|a_pq| are
// formed in double-float from the entry scaled to [0.5, 1) (the angle itself only needs to be accurate enough to
// converge).  The convergence test compares FP32 sums of the leading parts (off <= tol * total), which is all a
// threshold needs.
#pragma once
#include "df.cuh"
#include "smallmat.cuh"

// sqrt(a), a >= 0: the FP32 root refined by one Newton step in double-float
DG_HD dfl df_sqrt(dfl a) {
    if (!(a.h > 0.f)) return {0.f, 0.f};
    const float s = sqrtf(a.h);
    const dfl e = df_sub(a, df_mul({s, 0.f}, {s, 0.f}));  // a - s^2
    return fast_two_sum(s, e.h / (2.f * s));
}
// a / b: the FP32 quotient corrected by the double-float remainder
DG_HD dfl df_div(dfl a, dfl b) {
    const float q1 = a.h / b.h;
    const dfl r = df_sub(a, df_mul(b, {q1, 0.f}));
    const float q2 = r.h / b.h;
    return fast_two_sum(q1, q2);
}

// one Jacobi rotation of the (p, q) plane in double-float
struct DfRot {
    int p, q, on;
    dfl c, s;
    cdf ph;
};
static_assert(sizeof(DfRot) <= sizeof(DgRot), "DfRot shares the DgRot slots");

// All 32 lanes call it; A0 (read-only), a, u: n*n cdf in shared memory (column-major); w: n doubles (ascending
// eigenvalues out); order: n ints; rot: n/2+1 rotation slots (DgRot-sized).  Eigenvectors (columns) in u.
// Returns DG_OK or DG_NONCONV.
__device__ inline int warp_heig_df(int n, const cdf *A0, cdf *a, cdf *u, double *w, int *order, DgRot *rot_slots,
                                   float tol) {
    DfRot *rot = reinterpret_cast<DfRot *>(rot_slots);
    const int lane = threadIdx.x & 31;
    const cdf zero = {{0.f, 0.f}, {0.f, 0.f}}, one = {{1.f, 0.f}, {0.f, 0.f}};
    for (int e = lane; e < n * n; e += 32) {
        const int i = e % n, j = e / n;
        cdf v;
        if (i > j) v = DG_AT(A0, n, i, j);
        else if (i < j) v = {DG_AT(A0, n, j, i).re, df_neg(DG_AT(A0, n, j, i).im)};  // conj of the lower triangle
        else v = {DG_AT(A0, n, i, i).re, {0.f, 0.f}};
        a[e] = v;
        u[e] = (i == j) ? one : zero;
    }
    __syncwarp();
    const int m = n + (n & 1), half = m / 2;
    int st = DG_NONCONV;
    for (int sweep = 0; sweep < 100; sweep++) {
        float off = 0.f, tot = 0.f;
        for (int e = lane; e < n * n; e += 32) {
            const float v = __fmaf_rn(a[e].re.h, a[e].re.h, __fmul_rn(a[e].im.h, a[e].im.h));
            tot += v;
            if (e % n != e / n) off += v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        const int conv = __shfl_sync(0xffffffffu, (int)(off == 0.f || off <= tol * tot), 0);
        if (conv) {
            st = DG_OK;
            break;
        }
        for (int r = 0; r < m - 1; r++) {
            if (lane < half) {
                // the round-robin pairing of warp_heig
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
                DfRot R;
                R.p = p;
                R.q = q;
                R.on = 0;
                R.c = {1.f, 0.f};
                R.s = {0.f, 0.f};
                R.ph = one;
                if (q < n) {
                    const cdf apq = DG_AT(a, n, p, q);
                    const float mx = fmaxf(fabsf(apq.re.h), fabsf(apq.im.h));
                    if (mx > 1e-37f) {
                        // |a_pq| and its phase from the entry scaled by a power of two to [0.5, 1): the squares of a
                        // small entry would otherwise lose their low parts to FP32 underflow (|a_pq|^2 < 1e-31), and
                        // a phase that is not unit to double-float precision breaks the rotation's unitarity
                        int ex = 0;
                        frexpf(mx, &ex);
                        const float sc = ldexpf(1.f, -ex);
                        const dfl ar = {apq.re.h * sc, apq.re.l * sc}, ai = {apq.im.h * sc, apq.im.l * sc};
                        const dfl rrs = df_sqrt(df_fma(ai, ai, df_mul(ar, ar)));  // |a_pq| sc
                        const dfl rr = {rrs.h / sc, rrs.l / sc};                  // exact: a power of two
                        const dfl app = DG_AT(a, n, p, p).re, aqq = DG_AT(a, n, q, q).re;
                        const dfl d = df_sub(aqq, app);
                        dfl t;
                        if (fabsf(d.h) > 2e15f * rr.h) {
                            t = df_div(rr, d);  // t ~ 1/(2 theta) = |a_pq| / (a_qq - a_pp): theta^2 would overflow
                        } else {
                            const dfl theta = df_div(d, {2.f * rr.h, 2.f * rr.l});
                            const dfl den = df_add({fabsf(theta.h), theta.h < 0.f ? -theta.l : theta.l},
                                                   df_sqrt(df_fma(theta, theta, {1.f, 0.f})));
                            t = df_div({theta.h < 0.f ? -1.f : 1.f, 0.f}, den);
                        }
                        R.c = df_div({1.f, 0.f}, df_sqrt(df_fma(t, t, {1.f, 0.f})));
                        R.s = df_mul(t, R.c);
                        const dfl ir = df_div({1.f, 0.f}, rrs);
                        R.ph = {df_mul(ar, ir), df_mul(ai, ir)};
                        R.on = 1;
                    }
                }
                rot[lane] = R;
            }
            __syncwarp();
            // columns p, q: x(:,p) = c x(:,p) - s conj(ph) x(:,q); x(:,q) = s x(:,p) + c conj(ph) x(:,q)
            for (int x = lane; x < half * n; x += 32) {
                const DfRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const cdf phc = {R.ph.re, df_neg(R.ph.im)};
                const cdf sphc = {df_mul(phc.re, R.s), df_mul(phc.im, R.s)};
                const cdf cphc = {df_mul(phc.re, R.c), df_mul(phc.im, R.c)};
                const cdf akp = DG_AT(a, n, k, R.p), akq = DG_AT(a, n, k, R.q);
                DG_AT(a, n, k, R.p) = OpsF::fms(sphc, akq, {df_mul(akp.re, R.c), df_mul(akp.im, R.c)});
                DG_AT(a, n, k, R.q) = OpsF::fma(cphc, akq, {df_mul(akp.re, R.s), df_mul(akp.im, R.s)});
                const cdf ukp = DG_AT(u, n, k, R.p), ukq = DG_AT(u, n, k, R.q);
                DG_AT(u, n, k, R.p) = OpsF::fms(sphc, ukq, {df_mul(ukp.re, R.c), df_mul(ukp.im, R.c)});
                DG_AT(u, n, k, R.q) = OpsF::fma(cphc, ukq, {df_mul(ukp.re, R.s), df_mul(ukp.im, R.s)});
            }
            __syncwarp();
            // rows p, q: x(p,:) = c x(p,:) - s ph x(q,:); x(q,:) = s x(p,:) + c ph x(q,:)
            for (int x = lane; x < half * n; x += 32) {
                const DfRot R = rot[x / n];
                if (!R.on) continue;
                const int k = x % n;
                const cdf sph = {df_mul(R.ph.re, R.s), df_mul(R.ph.im, R.s)};
                const cdf cph = {df_mul(R.ph.re, R.c), df_mul(R.ph.im, R.c)};
                const cdf apk = DG_AT(a, n, R.p, k), aqk = DG_AT(a, n, R.q, k);
                DG_AT(a, n, R.p, k) = OpsF::fms(sph, aqk, {df_mul(apk.re, R.c), df_mul(apk.im, R.c)});
                DG_AT(a, n, R.q, k) = OpsF::fma(cph, aqk, {df_mul(apk.re, R.s), df_mul(apk.im, R.s)});
            }
            __syncwarp();
            if (lane < half) {
                const DfRot R = rot[lane];
                if (R.on) {
                    DG_AT(a, n, R.p, R.q) = zero;
                    DG_AT(a, n, R.q, R.p) = zero;
                    DG_AT(a, n, R.p, R.p).im = {0.f, 0.f};
                    DG_AT(a, n, R.q, R.q).im = {0.f, 0.f};
                }
            }
            __syncwarp();
        }
    }
    if (lane == 0) {
        for (int i = 0; i < n; i++) order[i] = i;
        for (int i = 1; i < n; i++) {
            const int v = order[i];
            const double key = df_val(DG_AT(a, n, v, v).re);
            int j = i - 1;
            while (j >= 0 && df_val(DG_AT(a, n, order[j], order[j]).re) > key) {
                order[j + 1] = order[j];
                j--;
            }
            order[j + 1] = v;
        }
        for (int i = 0; i < n; i++) w[i] = df_val(DG_AT(a, n, order[i], order[i]).re);
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
