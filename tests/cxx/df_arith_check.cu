// df_arith_check.cu -- runs the double-float arithmetic of the lattice kernels (dmftpack_gb300/csrc/df.cuh, the
// square root / division of smallmat_df.cuh and the in-register 3 x 3 inverse of schur.cuh) and the per-thread FP64
// matrix routines of linalg.cuh / smallmat.cuh on the host, so that tests/test_df_arith.py can hold them to exact
// rational arithmetic (or to LAPACK) without a GPU.  Built by nvcc with -ffp-contract=off: every single-precision
// operation is then the IEEE round-to-nearest operation its device intrinsic performs.
//
// stdin: one case per line, "<op> <x1> <x2> ..." with every number in C99 hex notation (%a); stdout: the results of
// each case on one line, in the same notation.  A double-float value is two floats (hi lo), a complex one four
// (re.hi re.lo im.hi im.lo); the FP64 routines take and give complex doubles as (re im) pairs.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "df.cuh"
#include "linalg.cuh"
#include "schur.cuh"
#include "smallmat.cuh"
#include "smallmat_df.cuh"

namespace {

bool read_numbers(const char *s, std::vector<double> &v) {
    while (*s) {
        while (*s == ' ' || *s == '\t') s++;
        if (!*s || *s == '\n') break;
        char *end = nullptr;
        const double x = std::strtod(s, &end);
        if (end == s) return false;
        v.push_back(x);
        s = end;
    }
    return true;
}
dfl d_at(const std::vector<float> &v, int i) { return {v[2 * i], v[2 * i + 1]}; }
cdf c_at(const std::vector<float> &v, int i) { return {{v[4 * i], v[4 * i + 1]}, {v[4 * i + 2], v[4 * i + 3]}}; }
void put(dfl a) { std::printf("%a %a", a.h, a.l); }
void put(cdf a) {
    put(a.re);
    std::printf(" ");
    put(a.im);
}

}  // namespace

int main() {
    static char line[1 << 16];
    while (std::fgets(line, sizeof line, stdin)) {
        char op[32];
        int off = 0;
        if (std::sscanf(line, "%31s%n", op, &off) != 1) continue;
        std::vector<double> dv;
        if (!read_numbers(line + off, dv)) return 2;
        const std::vector<float> v(dv.begin(), dv.end());  // the float operands are exact floats in the input
        const std::string o(op);
        if (o == "two_sum") put(two_sum(v[0], v[1]));
        else if (o == "add") put(df_add(d_at(v, 0), d_at(v, 1)));
        else if (o == "mul") put(df_mul(d_at(v, 0), d_at(v, 1)));
        else if (o == "fma") put(df_fma(d_at(v, 0), d_at(v, 1), d_at(v, 2)));
        else if (o == "dot2") put(df_dot2(d_at(v, 0), d_at(v, 1), d_at(v, 2), d_at(v, 3)));
        else if (o == "fma2") put(df_fma2(d_at(v, 0), d_at(v, 1), d_at(v, 2), d_at(v, 3), d_at(v, 4)));
        else if (o == "lazy") {  // a lazy sum of the products of the pairs that follow, renormalised at the end
            dfl acc = {0.f, 0.f};
            for (size_t i = 0; i + 3 < v.size(); i += 4) acc = df_fma_lazy(d_at(v, i / 2), d_at(v, i / 2 + 1), acc);
            put(df_renorm(acc));
        } else if (o == "rcp") put(df_rcp(d_at(v, 0)));
        else if (o == "sqrt") put(df_sqrt(d_at(v, 0)));
        else if (o == "div") put(df_div(d_at(v, 0), d_at(v, 1)));
        else if (o == "cmul") put(OpsF::mul(c_at(v, 0), c_at(v, 1)));
        else if (o == "cmulc") put(OpsF::mulc(c_at(v, 0), c_at(v, 1)));
        else if (o == "cfma") put(OpsF::fma(c_at(v, 0), c_at(v, 1), c_at(v, 2)));
        else if (o == "cfms") put(OpsF::fms(c_at(v, 0), c_at(v, 1), c_at(v, 2)));
        else if (o == "crcp") put(OpsF::rcp(c_at(v, 0)));
        else if (o == "inv3" || o == "inv3d") {
            // the in-register Gauss-Jordan inverse of the thread-per-frequency Schur kernel, row-major input;
            // output: the singular flag, then the inverse row-major (double-float, or FP64 as hi 0 pairs)
            bool sing;
            if (o == "inv3") {
                cdf a[3][3];
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) a[r][c] = c_at(v, 3 * r + c);
                sing = dg::thread_inverse<OpsF, 3>(a);
                std::printf("%d", (int)sing);
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) {
                        std::printf(" ");
                        put(a[r][c]);
                    }
            } else {
                double2 a[3][3];
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) {
                        const cdf z = c_at(v, 3 * r + c);
                        a[r][c] = make_double2((double)z.re.h + (double)z.re.l, (double)z.im.h + (double)z.im.l);
                    }
                sing = dg::thread_inverse<OpsD, 3>(a);
                std::printf("%d", (int)sing);
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) std::printf(" %a 0x0p+0 %a 0x0p+0", a[r][c].x, a[r][c].y);
            }
        } else if (o == "gj" || o == "heig") {
            // FP64 per-thread routines of the impurity and moment kernels (linalg.cuh): the pivoted Gauss-Jordan
            // inverse and the cyclic Jacobi eigensolver on one column-major n x n matrix
            const int n = (int)dv[0];
            std::vector<double2> a(n * n), u(n * n), w2(n * n);
            for (int e = 0; e < n * n; e++) a[e] = make_double2(dv[1 + 2 * e], dv[2 + 2 * e]);
            std::vector<int> iw(n);
            if (o == "gj") {
                std::printf("%d", thread_gj_inverse(n, a.data(), iw.data()));
                for (int e = 0; e < n * n; e++) std::printf(" %a %a", a[e].x, a[e].y);
            } else {
                std::vector<double> w(n);
                std::printf("%d", thread_heig(n, a.data(), w2.data(), u.data(), w.data(), iw.data()));
                for (int i = 0; i < n; i++) std::printf(" %a", w[i]);
                for (int e = 0; e < n * n; e++) std::printf(" %a %a", u[e].x, u[e].y);
            }
        } else if (o == "posdef") {
            // smallmat.cuh's Cholesky sign test: strict, n, then the lower triangle row by row
            const bool strict = dv[0] != 0;
            const int n = (int)dv[1];
            std::vector<double2> t(n * (n + 1) / 2);
            for (size_t e = 0; e < t.size(); e++) t[e] = make_double2(dv[2 + 2 * e], dv[3 + 2 * e]);
            std::printf("%d", (int)posdef_tri(n, t.data(), 1, strict));
        } else return 3;
        std::printf("\n");
    }
    return 0;
}
