// df.cuh -- double-float ("split precision") complex arithmetic on the FP32 pipe.
//
// A real number is an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), giving a 48-bit mantissa;
// products use the FMA error-free transformation (p = a*b, e = fma(a, b, -p)), sums the two-sum
// transformation (Knuth), so every operation is accurate to ~2^-47 relative.  On GB300 the FP32 pipe issues
// ~70x the FP64 rate, so a double-float multiply-add (~18 FP32 instructions) is still several times cheaper
// than an FP64 one.  Values enter from FP64 memory exactly (hi = rn(x), lo = rn(x - hi)) and leave as
// hi + lo in FP64.
//
// Ops policies used by the templated lattice kernels:
//   OpsD: complex FP64 (double2)       OpsF: complex double-float (cdf)
#pragma once
#include <cmath>

#include "common.cuh"

#define DG_HD __host__ __device__ __forceinline__

// IEEE single-precision operations rounded to nearest: the device intrinsics (never contracted into FMAs), and the
// same operations on the host, so that the double-float arithmetic below can be checked on a CPU (host code that
// includes this header is built with -ffp-contract=off)
DG_HD float f_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
DG_HD float f_sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
DG_HD float f_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
DG_HD float f_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
DG_HD float f_rcp(float a) {
#ifdef __CUDA_ARCH__
    return __frcp_rn(a);
#else
    return 1.0f / a;
#endif
}
DG_HD float f_from_double(double x) {
#ifdef __CUDA_ARCH__
    return __double2float_rn(x);
#else
    return (float)x;
#endif
}

struct dfl {
    float h, l;
};
struct cdf {
    dfl re, im;
};

DG_HD dfl df_make(double x) {
    const float h = f_from_double(x);
    return {h, f_from_double(x - (double)h)};
}
DG_HD double df_val(dfl a) { return (double)a.h + (double)a.l; }
DG_HD dfl fast_two_sum(float a, float b) {
    const float s = f_add(a, b);
    return {s, f_sub(b, f_sub(s, a))};
}
DG_HD dfl two_sum(float a, float b) {
    const float s = f_add(a, b);
    const float bb = f_sub(s, a);
    return {s, f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb))};
}
DG_HD dfl df_add(dfl a, dfl b) {
    dfl s = two_sum(a.h, b.h);
    const float e = f_add(s.l, f_add(a.l, b.l));
    return fast_two_sum(s.h, e);
}
DG_HD dfl df_neg(dfl a) { return {-a.h, -a.l}; }
DG_HD dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
DG_HD dfl df_mul(dfl a, dfl b) {
    const float p = f_mul(a.h, b.h);
    float e = f_fma(a.h, b.h, -p);
    e = f_fma(a.h, b.l, e);
    e = f_fma(a.l, b.h, e);
    return fast_two_sum(p, e);
}
// c + a*b with one rounding of the product's error term
DG_HD dfl df_fma(dfl a, dfl b, dfl c) {
    const float p = f_mul(a.h, b.h);
    float e = f_fma(a.h, b.h, -p);
    e = f_fma(a.h, b.l, e);
    e = f_fma(a.l, b.h, e);
    dfl s = two_sum(c.h, p);
    const float t = f_add(s.l, f_add(c.l, e));
    return fast_two_sum(s.h, t);
}
// the product a*b as hi p plus the FP32 sum e of its error terms (p + e = a*b to ~2^-48 relative)
DG_HD float df_prod(dfl a, dfl b, float &e) {
    const float p = f_mul(a.h, b.h);
    e = f_fma(a.h, b.h, -p);
    e = f_fma(a.h, b.l, e);
    e = f_fma(a.l, b.h, e);
    return p;
}
// a*b + c*d with one renormalisation (the real or imaginary part of a complex product): the two hi products
// are added exactly (two-sum), the error terms in FP32, so the result is as accurate as two chained
// df_fma and takes 19 FP32 operations instead of 22
DG_HD dfl df_dot2(dfl a, dfl b, dfl c, dfl d) {
    float e1, e2;
    const float p1 = df_prod(a, b, e1), p2 = df_prod(c, d, e2);
    const dfl s = two_sum(p1, p2);
    return fast_two_sum(s.h, f_add(s.l, f_add(e1, e2)));
}
// acc + a*b + c*d with one renormalisation (27 FP32 operations instead of 30 for two chained df_fma)
DG_HD dfl df_fma2(dfl a, dfl b, dfl c, dfl d, dfl acc) {
    float e1, e2;
    const float p1 = df_prod(a, b, e1), p2 = df_prod(c, d, e2);
    const dfl s1 = two_sum(acc.h, p1);
    const dfl s2 = two_sum(s1.h, p2);
    const float t = f_add(f_add(s1.l, s2.l), f_add(acc.l, f_add(e1, e2)));
    return fast_two_sum(s2.h, t);
}
// Lazy accumulation for a running sum of products: acc + a*b with the hi parts added exactly (two-sum) and the
// low parts summed unnormalised in FP32 (12 FP32 operations instead of 15).  The low part of a lazy sum of n
// terms grows to ~n ulp of the hi part and its own rounding with it, so lazy sums are for short runs (the poles of
// one k point, n <= ~64) and pass through df_renorm before any other double-float operation reads them.
DG_HD dfl df_fma_lazy(dfl a, dfl b, dfl acc) {
    float e;
    const float p = df_prod(a, b, e);
    const dfl s = two_sum(acc.h, p);
    return {s.h, f_add(f_add(acc.l, e), s.l)};
}
DG_HD dfl df_renorm(dfl a) { return fast_two_sum(a.h, a.l); }
// 1/a: FP32 reciprocal refined by one Newton step in double-float (24 -> ~48 bits)
DG_HD dfl df_rcp(dfl a) {
    const float r = f_rcp(a.h);
    // e = 1 - a*r in double-float
    dfl ar = df_mul(a, {r, 0.0f});
    dfl e = df_sub({1.0f, 0.0f}, ar);
    // r + r*e
    return df_fma({r, 0.0f}, e, {r, 0.0f});
}

DG_HD cdf cdf_make(double2 z) { return {df_make(z.x), df_make(z.y)}; }
DG_HD double2 cdf_val(cdf z) { return make_double2(df_val(z.re), df_val(z.im)); }

struct OpsD {
    typedef double2 C;
    typedef double M;  // pivot magnitude type
    static DG_HD C zero() { return cmk(0, 0); }
    static DG_HD C one() { return cmk(1, 0); }
    static DG_HD C from(double2 z) { return z; }
    static DG_HD double2 to(C z) { return z; }
    static DG_HD C add(C a, C b) { return cadd(a, b); }
    static DG_HD C sub(C a, C b) { return csub(a, b); }
    static DG_HD C neg(C a) { return cneg(a); }
    static DG_HD C mul(C a, C b) { return cmul(a, b); }
    static DG_HD C mulc(C a, C b) { return cmulc(a, b); }  // a conj(b)
    static DG_HD C conj(C a) { return cconj(a); }
    static DG_HD C fma(C a, C b, C acc) { return cfma(a, b, acc); }
    static DG_HD C fms(C a, C b, C acc) { return cfms(a, b, acc); }
    static DG_HD C rcp(C a) { return crcp(a); }
    static DG_HD double re(C a) { return a.x; }
    static DG_HD double im(C a) { return a.y; }
    static DG_HD double mag2(C a) { return cabs2(a); }
    static __device__ __forceinline__ C shfl(C v, int src, int w) { return shfl2(v, src, w); }
    // real parts (R) for the Hermitian split of the pole sums
    typedef double R;
    static DG_HD R rzero() { return 0.0; }
    static DG_HD R rfrom(double x) { return x; }
    static DG_HD R rfma(R a, R b, R acc) { return ::fma(a, b, acc); }
    static DG_HD R rmul(R a, R b) { return a * b; }
    static DG_HD R radd(R a, R b) { return a + b; }
    static DG_HD R rsub(R a, R b) { return a - b; }
    static DG_HD R rneg(R a) { return -a; }
    static DG_HD R rrcp(R a) { return 1.0 / a; }
    // lazy running sums of a few terms (double-float: unnormalised low parts, read through rnorm)
    static DG_HD R racc(R a, R b, R acc) { return ::fma(a, b, acc); }
    static DG_HD R rnorm(R a) { return a; }
    static DG_HD C mk(R re, R im) { return cmk(re, im); }
    static DG_HD R cre(C a) { return a.x; }
    static DG_HD R cim(C a) { return a.y; }
};

struct OpsF {
    typedef cdf C;
    typedef float M;
    static DG_HD C zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }
    static DG_HD C one() { return {{1.f, 0.f}, {0.f, 0.f}}; }
    static DG_HD C from(double2 z) { return cdf_make(z); }
    static DG_HD double2 to(C z) { return cdf_val(z); }
    static DG_HD C add(C a, C b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
    static DG_HD C sub(C a, C b) { return {df_sub(a.re, b.re), df_sub(a.im, b.im)}; }
    static DG_HD C neg(C a) { return {df_neg(a.re), df_neg(a.im)}; }
    static DG_HD C mul(C a, C b) {
        return {df_dot2(a.re, b.re, df_neg(a.im), b.im), df_dot2(a.re, b.im, a.im, b.re)};
    }
    static DG_HD C conj(C a) { return {a.re, df_neg(a.im)}; }
    static DG_HD C mulc(C a, C b) {  // a conj(b)
        return {df_dot2(a.re, b.re, a.im, b.im), df_dot2(a.im, b.re, df_neg(a.re), b.im)};
    }
    static DG_HD C fma(C a, C b, C acc) {
        return {df_fma2(a.re, b.re, df_neg(a.im), b.im, acc.re), df_fma2(a.re, b.im, a.im, b.re, acc.im)};
    }
    static DG_HD C fms(C a, C b, C acc) {
        return {df_fma2(df_neg(a.re), b.re, a.im, b.im, acc.re),
                df_fma2(df_neg(a.re), b.im, df_neg(a.im), b.re, acc.im)};
    }
    static DG_HD C rcp(C a) {  // conj(a)/|a|^2
        const dfl n = df_dot2(a.re, a.re, a.im, a.im);
        const dfl r = df_rcp(n);
        return {df_mul(a.re, r), df_neg(df_mul(a.im, r))};
    }
    static DG_HD double re(C a) { return df_val(a.re); }
    static DG_HD double im(C a) { return df_val(a.im); }
    static DG_HD float mag2(C a) {  // pivot choice only: FP32 magnitude suffices
        return f_fma(a.re.h, a.re.h, f_mul(a.im.h, a.im.h));
    }
    typedef dfl R;
    static DG_HD R rzero() { return {0.f, 0.f}; }
    static DG_HD R rfrom(double x) { return df_make(x); }
    static DG_HD R rfma(R a, R b, R acc) { return df_fma(a, b, acc); }
    static DG_HD R rmul(R a, R b) { return df_mul(a, b); }
    static DG_HD R radd(R a, R b) { return df_add(a, b); }
    static DG_HD R rsub(R a, R b) { return df_sub(a, b); }
    static DG_HD R rneg(R a) { return df_neg(a); }
    static DG_HD R rrcp(R a) { return df_rcp(a); }
    static DG_HD R racc(R a, R b, R acc) { return df_fma_lazy(a, b, acc); }
    static DG_HD R rnorm(R a) { return df_renorm(a); }
    static DG_HD C mk(R re, R im) { return {re, im}; }
    static DG_HD R cre(C a) { return a.re; }
    static DG_HD R cim(C a) { return a.im; }
    static __device__ __forceinline__ C shfl(C v, int src, int w) {
        C o;
        o.re.h = __shfl_sync(0xffffffffu, v.re.h, src, w);
        o.re.l = __shfl_sync(0xffffffffu, v.re.l, src, w);
        o.im.h = __shfl_sync(0xffffffffu, v.im.h, src, w);
        o.im.l = __shfl_sync(0xffffffffu, v.im.l, src, w);
        return o;
    }
};

// warp_gj_inverse (linalg.cuh) for any Ops policy
template <class Ops, int N, int W>
__device__ __forceinline__ bool warp_gj_inverse_t(typename Ops::C (&a)[N], const int c) {
    typedef typename Ops::C C;
    typedef typename Ops::M M;
    static_assert(N <= W && W <= 32 && (W & (W - 1)) == 0, "bad lane group");
    bool singular = false;
    int perm[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        M best = M(-1);
        int p = j;
#pragma unroll
        for (int i = j; i < N; i++) {
            const M v = Ops::mag2(a[i]);
            if (v > best) {
                best = v;
                p = i;
            }
        }
        p = __shfl_sync(0xffffffffu, p, j, W);
        best = __shfl_sync(0xffffffffu, best, j, W);
        singular |= !(best > M(0));
        perm[j] = p;
#pragma unroll
        for (int i = j + 1; i < N; i++)
            if (i == p) {
                const C t = a[j];
                a[j] = a[i];
                a[i] = t;
            }
        const C piv = Ops::shfl(a[j], j, W);
        const C ipiv = Ops::rcp(piv);
        const C t = Ops::mul(a[j], ipiv);
        const bool is_piv_col = (c == j);
        // the pivot column's entries become -f ipiv = fms(f, ipiv, 0): one fms per entry on every lane
        const C tu = is_piv_col ? ipiv : t;
#pragma unroll
        for (int i = 0; i < N; i++) {
            if (i == j) continue;
            const C f = Ops::shfl(a[i], j, W);
            a[i] = Ops::fms(f, tu, is_piv_col ? Ops::zero() : a[i]);
        }
        a[j] = is_piv_col ? ipiv : t;
    }
#pragma unroll
    for (int j = N - 1; j >= 0; j--) {
        const int p = perm[j];
        const int src = (c == j) ? p : ((c == p) ? j : c);
#pragma unroll
        for (int i = 0; i < N; i++) a[i] = Ops::shfl(a[i], src, W);
    }
    return singular;
}

// warp_gj_inverse_t with the elimination steps in a rolled loop: the same arithmetic and pivot choices, but
// the rows of each lane's column are rotated by one after every step, so the current pivot row is always
// register a[0] and the loop body is the same for every step (no dynamic register indexing).  The code is N
// times shorter than the unrolled form, which matters for large N, where the kernels are bound by instruction
// fetch.  Row r of step j sits in register (r - j) mod N; after N steps every row is back in place.
template <class Ops, int N, int W>
__device__ __forceinline__ bool warp_gj_inverse_rolled(typename Ops::C (&a)[N], const int c) {
    typedef typename Ops::C C;
    typedef typename Ops::M M;
    static_assert(N <= W && W <= 32 && (W & (W - 1)) == 0, "bad lane group");
    bool singular = false;
    int perm[N];
#pragma unroll 1
    for (int j = 0; j < N; j++) {
        // pivot search over rows j..N-1 (registers 0..N-1-j) of column j (lane j)
        M best = M(-1);
        int pp = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const M v = Ops::mag2(a[i]);
            if (i <= N - 1 - j && v > best) {
                best = v;
                pp = i;
            }
        }
        pp = __shfl_sync(0xffffffffu, pp, j, W);
        best = __shfl_sync(0xffffffffu, best, j, W);
        singular |= !(best > M(0));
        perm[j] = pp + j;  // the row index of the pivot
#pragma unroll
        for (int i = 1; i < N; i++)
            if (i == pp) {
                const C t = a[0];
                a[0] = a[i];
                a[i] = t;
            }
        const C piv = Ops::shfl(a[0], j, W);
        const C ipiv = Ops::rcp(piv);
        const C t = Ops::mul(a[0], ipiv);
        const bool is_piv_col = (c == j);
        const C tu = is_piv_col ? ipiv : t;  // the pivot column's entries become fms(f, ipiv, 0) = -f ipiv
#pragma unroll
        for (int i = 1; i < N; i++) {
            const C f = Ops::shfl(a[i], j, W);
            a[i] = Ops::fms(f, tu, is_piv_col ? Ops::zero() : a[i]);
        }
        a[0] = is_piv_col ? ipiv : t;
        // rotate: the finished pivot row moves to the end
        const C r0 = a[0];
#pragma unroll
        for (int i = 0; i < N - 1; i++) a[i] = a[i + 1];
        a[N - 1] = r0;
    }
#pragma unroll 1
    for (int j = N - 1; j >= 0; j--) {
        const int p = perm[j];
        const int src = (c == j) ? p : ((c == p) ? j : c);
#pragma unroll
        for (int i = 0; i < N; i++) a[i] = Ops::shfl(a[i], src, W);
    }
    return singular;
}

// warp_gj_inverse_rolled for lane groups of any width N that need not divide 32: the group is lanes
// base .. base+N-1 of the warp (lane c of the group holds column c), so 32/N groups share a warp with no idle
// padding lanes inside a group.  Every shuffle names an absolute source lane (width 32) and runs with the
// full mask under warp-uniform control flow; lanes outside any group take part with base past the last
// group and compute values that are never used.
template <class Ops, int N>
__device__ __forceinline__ bool group_gj_inverse(typename Ops::C (&a)[N], const int c, const int base) {
    typedef typename Ops::C C;
    typedef typename Ops::M M;
    bool singular = false;
    int perm[N];
#pragma unroll 1
    for (int j = 0; j < N; j++) {
        M best = M(-1);
        int pp = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const M v = Ops::mag2(a[i]);
            if (i <= N - 1 - j && v > best) {
                best = v;
                pp = i;
            }
        }
        pp = __shfl_sync(0xffffffffu, pp, base + j, 32);
        best = __shfl_sync(0xffffffffu, best, base + j, 32);
        singular |= !(best > M(0));
        perm[j] = pp + j;
#pragma unroll
        for (int i = 1; i < N; i++)
            if (i == pp) {
                const C t = a[0];
                a[0] = a[i];
                a[i] = t;
            }
        const C piv = Ops::shfl(a[0], base + j, 32);
        const C ipiv = Ops::rcp(piv);
        const C t = Ops::mul(a[0], ipiv);
        const bool is_piv_col = (c == j);
        const C tu = is_piv_col ? ipiv : t;  // the pivot column's entries become fms(f, ipiv, 0) = -f ipiv
#pragma unroll
        for (int i = 1; i < N; i++) {
            const C f = Ops::shfl(a[i], base + j, 32);
            a[i] = Ops::fms(f, tu, is_piv_col ? Ops::zero() : a[i]);
        }
        a[0] = is_piv_col ? ipiv : t;
        const C r0 = a[0];
#pragma unroll
        for (int i = 0; i < N - 1; i++) a[i] = a[i + 1];
        a[N - 1] = r0;
    }
#pragma unroll 1
    for (int j = N - 1; j >= 0; j--) {
        const int p = perm[j];
        const int src = base + ((c == j) ? p : ((c == p) ? j : c));
#pragma unroll
        for (int i = 0; i < N; i++) a[i] = Ops::shfl(a[i], src, 32);
    }
    return singular;
}
