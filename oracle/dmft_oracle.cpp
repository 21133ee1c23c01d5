/*
 * dmft_oracle.cpp -- CPU FP64 restatement of DMFTpack's DMFT self-consistency hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Loaded by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg / reference arm; never by the product library.
 *
 * PARITY UNPINNED against the reference program itself: it needs Eigen (unvendored, uninstalled,
 * version unpinned) and MPI and cannot be compiled here, and it ships no golden outputs.  Each function
 * cites the reference lines (paths relative to the DMFTpack repository) it restates.  Eigen's
 * primitives are replaced by:
 *   - PartialPivLU inverse  -> lu_inverse(): row pivoting on max |a_ik|, then L U X = P I;
 *   - SelfAdjointEigenSolver -> heig(): cyclic complex Jacobi on the matrix rebuilt from its LOWER
 *     triangle with a real diagonal (Eigen reads only the lower triangle), ascending eigenvalues;
 *   - ComplexEigenSolver in GiwToNele -> the trace identity sum_l 1/(z-e_l) = Tr (z-H-S)^-1.
 * The MPI k/tau/omega splits of the reference collapse to one rank; nthreads splits k like para_range.
 */
#include "dmft_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <thread>
#include <vector>

namespace {

typedef std::complex<double> cd;
const double PI = 3.1415926535897932384626;  // src/dmft_common.h:43
const cd I1(0.0, 1.0);

enum { OK = 0, SINGULAR = 1, NONCONV = 2, NANINF = 3, BADARG = 4, CAUSAL = 5, HERMIT = 6 };

struct Mat {
    int r = 0, c = 0;
    std::vector<cd> a;
    Mat() {}
    Mat(int r_, int c_) : r(r_), c(c_), a((size_t)r_ * c_, cd(0.0, 0.0)) {}
    cd &operator()(int i, int j) { return a[i + (size_t)j * r]; }
    const cd &operator()(int i, int j) const { return a[i + (size_t)j * r]; }
    static Mat eye(int n) {
        Mat m(n, n);
        for (int i = 0; i < n; i++) m(i, i) = 1.0;
        return m;
    }
};

Mat load(const double *p, int r, int c) {
    Mat m(r, c);
    std::memcpy((void *)m.a.data(), p, sizeof(cd) * (size_t)r * c);
    return m;
}
void store(const Mat &m, double *p) { std::memcpy(p, (const void *)m.a.data(), sizeof(cd) * m.a.size()); }
std::vector<Mat> load_stack(const double *p, int count, int n) {
    std::vector<Mat> v(count);
    for (int i = 0; i < count; i++) v[i] = load(p + (size_t)2 * n * n * i, n, n);
    return v;
}
void store_stack(const std::vector<Mat> &v, int count, double *p) {
    for (int i = 0; i < count; i++) store(v[i], p + (size_t)2 * v[i].r * v[i].c * i);
}

Mat mul(const Mat &A, const Mat &B) {
    Mat C(A.r, B.c);
    for (int j = 0; j < B.c; j++)
        for (int k = 0; k < A.c; k++) {
            cd b = B(k, j);
            for (int i = 0; i < A.r; i++) C(i, j) += A(i, k) * b;
        }
    return C;
}
Mat adj(const Mat &A) {
    Mat B(A.c, A.r);
    for (int j = 0; j < A.c; j++)
        for (int i = 0; i < A.r; i++) B(j, i) = std::conj(A(i, j));
    return B;
}
Mat lin(const Mat &A, cd sa, const Mat &B, cd sb) {
    Mat C(A.r, A.c);
    for (size_t i = 0; i < A.a.size(); i++) C.a[i] = sa * A.a[i] + sb * B.a[i];
    return C;
}
Mat add(const Mat &A, const Mat &B) {
    Mat C = A;
    for (size_t i = 0; i < A.a.size(); i++) C.a[i] += B.a[i];
    return C;
}
Mat sub(const Mat &A, const Mat &B) {
    Mat C = A;
    for (size_t i = 0; i < A.a.size(); i++) C.a[i] -= B.a[i];
    return C;
}
Mat scal(const Mat &A, cd s) {
    Mat C = A;
    for (auto &x : C.a) x *= s;
    return C;
}
double fnorm(const Mat &A) {
    double s = 0;
    for (auto &x : A.a) s += std::norm(x);
    return std::sqrt(s);
}

/* Eigen::PartialPivLU<MatrixXcd>(A).inverse(): pivot = first row of max |a_ik| in column k. */
int lu_inverse(const Mat &A, Mat &X) {
    int n = A.r;
    Mat LU = A;
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    int st = OK;
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = std::abs(LU(k, k));
        for (int i = k + 1; i < n; i++) {
            double v = std::abs(LU(i, k));
            if (v > best) { best = v; p = i; }
        }
        if (best == 0.0) st = SINGULAR;
        if (p != k) {
            for (int j = 0; j < n; j++) std::swap(LU(k, j), LU(p, j));
            std::swap(perm[k], perm[p]);
        }
        if (best != 0.0) {
            cd piv = LU(k, k);
            for (int i = k + 1; i < n; i++) LU(i, k) /= piv;
        }
        for (int j = k + 1; j < n; j++) {
            cd u = LU(k, j);
            for (int i = k + 1; i < n; i++) LU(i, j) -= LU(i, k) * u;
        }
    }
    X = Mat(n, n);
    for (int col = 0; col < n; col++) {
        std::vector<cd> b(n);
        for (int i = 0; i < n; i++) b[i] = (perm[i] == col) ? cd(1.0) : cd(0.0);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < i; k++) b[i] -= LU(i, k) * b[k];
        for (int i = n - 1; i >= 0; i--) {
            for (int k = i + 1; k < n; k++) b[i] -= LU(i, k) * b[k];
            b[i] /= LU(i, i);
        }
        for (int i = 0; i < n; i++) X(i, col) = b[i];
    }
    return st;
}
Mat inv(const Mat &A) {
    Mat X;
    lu_inverse(A, X);
    return X;
}

/* Eigen::SelfAdjointEigenSolver<MatrixXcd>: lower triangle, real diagonal, ascending eigenvalues. */
int heig(const Mat &A0, std::vector<double> &w, Mat *V) {
    int n = A0.r;
    Mat A(n, n);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            if (i > j) A(i, j) = A0(i, j);
            else if (i < j) A(i, j) = std::conj(A0(j, i));
            else A(i, i) = std::real(A0(i, i));
        }
    Mat U = Mat::eye(n);
    int st = NONCONV;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) {
                double v = std::norm(A(i, j));
                tot += v;
                if (i != j) off += v;
            }
        if (off == 0.0 || off <= 1e-28 * tot) { st = OK; break; }
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                cd apq = A(p, q);
                double r = std::abs(apq);
                if (r == 0.0) continue;
                double app = std::real(A(p, p)), aqq = std::real(A(q, q));
                double theta = (aqq - app) / (2.0 * r);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                cd u = apq / r, uc = std::conj(u);
                for (int k = 0; k < n; k++) {
                    cd akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * uc * akq;
                    A(k, q) = s * akp + c * uc * akq;
                }
                for (int k = 0; k < n; k++) {
                    cd apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * u * aqk;
                    A(q, k) = s * apk + c * u * aqk;
                }
                A(p, q) = 0.0;
                A(q, p) = 0.0;
                A(p, p) = std::real(A(p, p));
                A(q, q) = std::real(A(q, q));
                for (int k = 0; k < n; k++) {
                    cd ukp = U(k, p), ukq = U(k, q);
                    U(k, p) = c * ukp - s * uc * ukq;
                    U(k, q) = s * ukp + c * uc * ukq;
                }
            }
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int x, int y) { return std::real(A(x, x)) < std::real(A(y, y)); });
    w.resize(n);
    for (int i = 0; i < n; i++) w[i] = std::real(A(idx[i], idx[i]));
    if (V) {
        *V = Mat(n, n);
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) (*V)(i, j) = U(i, idx[j]);
    }
    return st;
}
double min_eig(const Mat &A) {
    std::vector<double> w;
    heig(A, w, nullptr);
    return w.empty() ? 0.0 : w.front();
}
double max_eig(const Mat &A) {
    std::vector<double> w;
    heig(A, w, nullptr);
    return w.empty() ? 0.0 : w.back();
}
/* SelfAdjointEigenSolver::operatorSqrt(): V sqrt(w) V^H. */
Mat op_sqrt(const Mat &A) {
    std::vector<double> w;
    Mat V;
    heig(A, w, &V);
    int n = A.r;
    Mat D(n, n);
    for (int i = 0; i < n; i++) D(i, i) = std::sqrt(w[i]);
    return mul(mul(V, D), adj(V));
}

// threads for the per-frequency / per-tau / per-window loops of the transforms and the moment fit; every
// index is computed independently, so the results do not depend on the count (orc_set_threads)
int g_nthreads = 1;

template <class F>
void parallel_for(int n, int nthreads, F f) {
    if (nthreads <= 1 || n < 2) {
        f(0, n, 0);
        return;
    }
    nthreads = std::min(nthreads, n);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) {
        int b = (int)((long long)n * t / nthreads), e = (int)((long long)n * (t + 1) / nthreads);
        th.emplace_back(f, b, e, t);
    }
    for (auto &x : th) x.join();
}

/* src/FourierTransform.cpp:184-465  getAsymto_moments. */
int moments_fit(int Dim, int Nf, double beta, const std::vector<Mat> &F, bool green, std::vector<Mat> &mom) {
    mom.assign(4, Mat(Dim, Dim));
    const int ncol = green ? 2 : 4;
    const int R = green ? Nf - 1 : Nf - 3;  // w_Asymto_range = w_Asymto_end + 1
    int Nv = Nf / 20;
    if (Nv == 0) Nv = 1;
    const int C = R - 2 * Nv;  // number of averaging centres
    if (R < 1 || C < 1) return BADARG;
    const int DD = Dim * Dim;
    std::vector<cd> mt((size_t)DD * R * ncol);  // momentstest[ab][w][col]
    auto MT = [&](int ab, int w, int col) -> cd & { return mt[((size_t)ab * R + w) * ncol + col]; };
    std::vector<std::vector<double>> trace(ncol, std::vector<double>(R, 0.0));
    // window w costs ~ (Nf - w): threads take the windows round-robin to balance the triangle
    const int T = std::max(1, std::min(g_nthreads, R));
    parallel_for(T, T, [&](int tb, int te, int) {
    for (int t0 = tb; t0 < te; t0++)
    for (int w = t0; w < R; w += T) {
        int ASlen = Nf - w;
        Mat KtK(ncol, ncol);
        auto krow = [&](int jj, int im, double *kr) {
            double z = (2 * (w + jj) + 1) * PI / beta;
            for (int c = 0; c < ncol; c++) kr[c] = 0;
            if (!green) {
                if (im == 0) { kr[0] = 1.0; kr[2] = -1. / std::pow(z, 2); }
                else { kr[1] = -1. / std::pow(z, 1); kr[3] = 1. / std::pow(z, 3); }
            } else {
                if (im == 0) kr[0] = -1. / std::pow(z, 2);
                else kr[1] = 1. / std::pow(z, 3);
            }
        };
        double kr[4];
        for (int jj = 0; jj < ASlen; jj++)
            for (int im = 0; im < 2; im++) {
                krow(jj, im, kr);
                for (int j = 0; j < ncol; j++)
                    for (int i = 0; i < ncol; i++) KtK(i, j) += kr[i] * kr[j];
            }
        Mat Kinv = inv(KtK);
        std::vector<cd> acc((size_t)DD * ncol, cd(0.0));
        for (int jj = 0; jj < ASlen; jj++) {
            int wn = w + jj;
            double z = (2 * wn + 1) * PI / beta;
            for (int im = 0; im < 2; im++) {
                krow(jj, im, kr);
                cd solve[4];
                for (int i = 0; i < ncol; i++) {
                    cd s = 0.0;
                    for (int c = 0; c < ncol; c++) s += Kinv(i, c) * kr[c];
                    solve[i] = s;
                }
                for (int b = 0; b < Dim; b++)
                    for (int a = 0; a < Dim; a++) {
                        cd g;
                        if (im == 0) g = (F[wn](a, b) + std::conj(F[wn](b, a))) / 2.0;
                        else g = (F[wn](a, b) - std::conj(F[wn](b, a))) / (2.0 * I1);
                        if (green && im == 1 && a == b) g += 1.0 / z;
                        for (int i = 0; i < ncol; i++) acc[((size_t)(a * Dim + b)) * ncol + i] += solve[i] * g;
                    }
            }
        }
        for (int ab = 0; ab < DD; ab++)
            for (int i = 0; i < ncol; i++) MT(ab, w, i) = acc[(size_t)ab * ncol + i];
        for (int a = 0; a < Dim; a++)
            for (int i = 0; i < ncol; i++) trace[i][w] += std::real(MT(a * Dim + a, w, i));
    }
    });
    // window averages of the fitted moments (src/FourierTransform.cpp:259-283)
    std::vector<std::vector<Mat>> avg(ncol, std::vector<Mat>(C, Mat(Dim, Dim)));
    for (int ci = 0; ci < C; ci++) {
        int cen = ci + Nv;
        for (int iw = cen - Nv; iw <= cen + Nv; iw++)
            for (int a = 0; a < Dim; a++)
                for (int b = 0; b < Dim; b++)
                    for (int i = 0; i < ncol; i++) avg[i][ci](a, b) += MT(a * Dim + b, iw, i);
        for (int i = 0; i < ncol; i++) avg[i][ci] = scal(avg[i][ci], cd(1.0) / cd(2.0 * Nv + 1, 0.0));
    }
    // admissible windows (same test for every moment index; src/FourierTransform.cpp:296-315, 421-434)
    std::vector<char> ok(C, 0);
    for (int i = 0; i < C; i++) {
        if (!green) {
            double a = min_eig(avg[1][i]);
            if (a > 0) {
                Mat Vinv = inv(op_sqrt(avg[1][i]));
                Mat m2 = mul(mul(Vinv, avg[2][i]), Vinv);
                Mat X = sub(mul(mul(Vinv, avg[3][i]), Vinv), mul(m2, m2));
                double b = min_eig(X);
                ok[i] = (a > 0 && b > 0);
            }
        } else {
            double a = min_eig(sub(avg[1][i], mul(avg[0][i], avg[0][i])));
            ok[i] = (a > 1);
        }
    }
    for (int m = 0; m < ncol; m++) {
        std::vector<double> var(C);
        for (int ci = 0; ci < C; ci++) {
            int s0 = ci;  // segment(w_Asymto_center - Nv, 2Nv+1)
            double mean = 0;
            for (int j = 0; j < 2 * Nv + 1; j++) mean += trace[m][s0 + j];
            mean /= (2 * Nv + 1);
            double ss = 0;
            for (int j = 0; j < 2 * Nv + 1; j++) ss += (trace[m][s0 + j] - mean) * (trace[m][s0 + j] - mean);
            var[ci] = std::sqrt(ss / (2 * Nv + 1));
        }
        int minPos = C - 1;
        for (int i = 0; i < C; i++)
            if (ok[i] && var[i] < var[minPos]) minPos = i;
        int cen = minPos + Nv;
        int dst = green ? m + 2 : m;
        Mat M(Dim, Dim);
        for (int w = cen - Nv; w <= cen + Nv; w++)
            for (int a = 0; a < Dim; a++)
                for (int b = 0; b < Dim; b++)
                    M(a, b) += (MT(a * Dim + b, w, m) + std::conj(MT(b * Dim + a, w, m))) / 2.0;
        mom[dst] = scal(M, cd(1.0) / cd(2.0 * Nv + 1, 0.0));
    }
    if (green) {
        mom[0] = Mat(Dim, Dim);
        mom[1] = Mat::eye(Dim);
    }
    for (int i = 0; i < 4; i++) mom[i] = scal(add(mom[i], adj(mom[i])), 0.5);
    return OK;
}

/* src/FourierTransform.cpp:16-118  FourierTransform_tau: tail pieces that do not depend on tau. */
struct Tail {
    int Dim;
    Mat V, H, H2;
    std::vector<double> eH, eH2;
    Mat UH, UH2;
};
Tail make_tail(int Dim, const std::vector<Mat> &mom) {
    Tail T;
    T.Dim = Dim;
    double a = min_eig(mom[1]);
    if (a > 0) {
        T.V = op_sqrt(mom[1]);
        Mat Vai = inv(adj(T.V)), Vi = inv(T.V);
        Mat M2 = mul(mul(Vai, scal(mom[2], 2.0)), Vi);
        Mat M3 = mul(mul(Vai, scal(mom[3], 2.0)), Vi);
        Mat X = sub(scal(M3, 0.5), scal(mul(M2, M2), 0.25));
        if (min_eig(X) > 0) T.H = add(scal(M2, 0.5), op_sqrt(X));
        else T.H = scal(M2, 0.5);
        T.H2 = sub(M2, T.H);
    } else {
        T.V = Mat(Dim, Dim);
        T.H = Mat(Dim, Dim);
        T.H2 = Mat(Dim, Dim);
    }
    heig(T.H, T.eH, &T.UH);
    heig(T.H2, T.eH2, &T.UH2);
    return T;
}
Mat tail_w(const Tail &T, double w) {
    int Dim = T.Dim;
    Mat id = Mat::eye(Dim);
    Mat A = lin(id, I1 * w, T.H, -1.0), B = lin(id, I1 * w, T.H2, -1.0);
    Mat Va = adj(T.V);
    Mat t = add(mul(mul(Va, inv(A)), T.V), mul(mul(Va, inv(B)), T.V));
    return scal(t, 0.5);
}
Mat ft_tau(const std::vector<Mat> &F, const Tail &T, const std::vector<Mat> &tails, int Nf, double beta,
           double tau) {
    int Dim = T.Dim;
    double dwl = (2 * PI) / beta, w0l = (PI / beta);
    Mat S(Dim, Dim);
    for (int i = 0; i < Nf; i++) {
        double w = w0l + i * dwl;
        cd ph = std::exp(-I1 * w * tau);
        for (int k = 0; k < Dim * Dim; k++) S.a[k] += (F[i].a[k] - tails[i].a[k]) * ph;
    }
    S = add(S, adj(S));
    S = scal(S, 1.0 / beta);
    auto g0 = [&](const std::vector<double> &e, const Mat &U) {
        Mat D(Dim, Dim);
        for (int i = 0; i < Dim; i++) D(i, i) = -1.0 / (std::exp(e[i] * tau) + std::exp(e[i] * (tau - beta)));
        return mul(mul(U, D), adj(U));
    };
    Mat Va = adj(T.V);
    S = add(S, scal(mul(mul(Va, g0(T.eH, T.UH)), T.V), 0.5));
    S = add(S, scal(mul(mul(Va, g0(T.eH2, T.UH2)), T.V), 0.5));
    S = add(S, adj(S));
    return scal(S, 0.5);
}

/* positivity fix-up shared by FourierTransform_ (:145-175) and getStimp (SCGF2_fullLoop.cpp:657-688). */
int positivity_fixup(std::vector<Mat> &D, int Nt, double beta) {
    int fixed = 0;
    int Dim = D[0].r;
    for (int t = 0; t < Nt + 1; t++) {
        double tau = t * beta / Nt;
        double mineig = min_eig(D[t]);
        double m11 = mineig;
        bool touched = false;
        if (mineig >= 0 && (t != 0 && t != Nt)) {
            touched = true;
            for (int t1 = t + 1; t1 < Nt + 1; t1++) {
                double tau1 = t1 * beta / Nt, tprev = (t - 1) * beta / Nt;
                Mat X(Dim, Dim);
                for (size_t k = 0; k < X.a.size(); k++)
                    X.a[k] = (D[t1].a[k] - D[t - 1].a[k]) / (tau1 - tprev) * (tau - tprev) + D[t - 1].a[k];
                D[t] = X;
                m11 = min_eig(D[t]);
                if (m11 < 0) break;
            }
        }
        if (m11 >= 0) {
            touched = true;
            D[t] = scal(Mat::eye(Dim), -1e-10);
        }
        if (touched) fixed++;
    }
    return fixed;
}

/* the per-k static eigen-decomposition of H + S_inf used by GreenFtn_w (:197-215) and GiwToNele. */
void add_sigma_block(Mat &A, const Mat &S, const orc_lattice *L, bool within_cluster, cd sign) {
    int D = L->ncl * L->nh;
    for (int p = 0; p < D; p++)
        for (int q = 0; q < D; q++) {
            if (within_cluster && p / L->nh != q / L->nh) continue;
            A(L->hartr[p], L->hartr[q]) += sign * S(p, q);
        }
}

}  // namespace

extern "C" {

int orc_version(void) { return 1; }

void orc_set_threads(int n) { g_nthreads = n < 1 ? 1 : n; }

/* src/TB.cpp:196-207 with ax=ay=az=pi (src/dmft_common.h:37-39). */
void orc_kmesh(int kx, int ky, int kz, double *kmesh) {
    int kpxy = kx * ky, nk = kx * ky * kz;
    double ax = PI, ay = PI, az = PI;
    double delx = 2. * PI / (ax * double(kx)), dely = 2. * PI / (ay * double(ky)), delz = 2. * PI / (az * double(kz));
    for (int k = 0; k < nk; k++) {
        kmesh[3 * k + 0] = -PI / ax + delx / 2. + ((int)k % kx) * delx;
        kmesh[3 * k + 1] = -PI / ay + dely / 2. + ((int)((int)(k % kpxy)) / kx) * dely;
        kmesh[3 * k + 2] = -PI / az + delz / 2. + ((int)k / kpxy) * delz;
    }
}

/* src/ConstructModelHamiltonian.cpp:66-77: H(k)_{ij} += t * exp(-i (kx ax Rx + ky ay Ry + kz az Rz)).
 * rindex rows: (Rx, Ry, Rz, i0, j0) as built by read_HR (src/read_TB_parm.cpp:36-45). */
int orc_hk(int n, int nnz, const int *rindex, const double *hr, int nk, const double *kmesh, double *hk,
           int nthreads) {
    for (int e = 0; e < nnz; e++)
        if (rindex[5 * e + 3] < 0 || rindex[5 * e + 3] >= n || rindex[5 * e + 4] < 0 || rindex[5 * e + 4] >= n)
            return BADARG;
    const double ax = PI, ay = PI, az = PI;
    parallel_for(nk, nthreads, [&](int b, int e, int) {
        for (int k = b; k < e; k++) {
            Mat H(n, n);
            for (int x = 0; x < nnz; x++) {
                const int *R = rindex + 5 * x;
                cd t(hr[2 * x], hr[2 * x + 1]);
                H(R[3], R[4]) += t * std::exp(-I1 * ((kmesh[3 * k] * ax * R[0]) + (kmesh[3 * k + 1] * ay * R[1]) +
                                                     (kmesh[3 * k + 2] * az * R[2])));
            }
            store(H, hk + (size_t)2 * n * n * k);
        }
    });
    return OK;
}

int orc_hermitian_eig(int n, const double *a, double *w, double *v) {
    Mat A = load(a, n, n), V;
    std::vector<double> ww;
    int st = heig(A, ww, &V);
    for (int i = 0; i < n; i++) w[i] = ww[i];
    if (v) store(V, v);
    return st;
}

int orc_inverse(int n, const double *a, double *ainv) {
    Mat X;
    int st = lu_inverse(load(a, n, n), X);
    store(X, ainv);
    return st;
}

int orc_moments(int dim, int nfreq, double beta, const double *fw, int green_asym, double *mom) {
    std::vector<Mat> F = load_stack(fw, nfreq, dim), M;
    int st = moments_fit(dim, nfreq, beta, F, green_asym != 0, M);
    store_stack(M, 4, mom);
    return st;
}

/* src/GreenFtn.cpp:142-422  GreenFtn_w (k split over threads like para_range; one rank). */
int orc_greenftn_w(const orc_lattice *L, const double *hk, const double *sigma, double mu, double *gw,
                   double *gwhf, double *nummat, int nthreads) {
    const int n = L->n, nk = L->nk, Nf = L->nfreq, D = L->ncl * L->nh, nh = L->nh;
    const double beta = L->beta;
    std::vector<Mat> S = load_stack(sigma, Nf, D), mom;
    int st = moments_fit(D, Nf, beta, S, false, mom);
    if (st) return st;
    int T = std::max(1, std::min(nthreads, nk));
    std::vector<std::vector<cd>> g_p(T, std::vector<cd>((size_t)Nf * D * D)), g0_p = g_p;
    std::vector<Mat> num_p(T, Mat(D, D)), num0_p(T, Mat(D, D)), occ_p(T, Mat(D, D));
    std::vector<int> st_p(T, OK);
    parallel_for(nk, T, [&](int kb, int ke, int tid) {
        for (int k = kb; k < ke; k++) {
            Mat H = load(hk + (size_t)2 * n * n * k, n, n);
            Mat Hs = H;
            // staticHamiltonian_Model[k](i0,m0) += Swmoments[0](i0,m0) on Hartree rows/cols (:197-207)
            add_sigma_block(Hs, mom[0], L, false, 1.0);
            std::vector<double> ev;
            Mat U;
            heig(Hs, ev, &U);
            for (int nn = 0; nn < 2 * Nf; nn++) {
                cd iw = I1 * PI * (2. * nn + 1.) / beta;
                Mat SW(D, D);
                if (nn < Nf) SW = S[nn];
                else
                    for (int a = 0; a < D * D; a++)
                        SW.a[a] = mom[0].a[a] + mom[1].a[a] / iw + mom[2].a[a] / std::pow(iw, 2) +
                                  mom[3].a[a] / std::pow(iw, 3);
                Mat A = scal(H, -1.0);
                add_sigma_block(A, SW, L, false, -1.0);
                for (int i = 0; i < n; i++) A(i, i) += (iw + mu);
                Mat G;
                if (lu_inverse(A, G)) st_p[tid] = SINGULAR;
                // Gkw0 = U diag(1/(iw+mu-e)) U^H, needed only on the correlated block
                std::vector<cd> dz(n);
                for (int l = 0; l < n; l++) dz[l] = 1. / (-ev[l] + (iw + mu));
                auto g0 = [&](int p, int q) {
                    cd s = 0;
                    for (int l = 0; l < n; l++) s += U(p, l) * dz[l] * std::conj(U(q, l));
                    return s;
                };
                if (nn < Nf)
                    for (int cl = 0; cl < L->ncl; cl++)
                        for (int i0 = 0; i0 < nh; i0++)
                            for (int m0 = 0; m0 < nh; m0++) {
                                int p = L->hartr[cl * nh + i0], q = L->hartr[cl * nh + m0];
                                size_t o = (size_t)nn * D * D + (cl * nh + i0) + (size_t)(cl * nh + m0) * D;
                                g_p[tid][o] += G(p, q);
                                g0_p[tid][o] += g0(p, q);
                            }
                for (int l1 = 0; l1 < D; l1++)
                    for (int l2 = 0; l2 < D; l2++) {
                        int a = L->hartr[l1], b = L->hartr[l2];
                        num_p[tid](l1, l2) += G(a, b) + std::conj(G(b, a));
                        num0_p[tid](l1, l2) += g0(a, b) + std::conj(g0(b, a));
                    }
            }
            // Fermi part of the occupation (:311-340), with the +-100 cut-offs of :314-316
            Mat occ(D, D);
            std::vector<double> f(n);
            for (int l = 0; l < n; l++) {
                double x = beta * (ev[l] - mu);
                f[l] = x > 100.0 ? 0.0 : (x < -100.0 ? 1.0 : 1. / (1. + std::exp(x)));
            }
            for (int l0 = 0; l0 < D; l0++)
                for (int m0 = 0; m0 < D; m0++) {
                    cd s = 0;
                    int a = L->hartr[l0], b = L->hartr[m0];
                    for (int l = 0; l < n; l++) s += U(a, l) * f[l] * std::conj(U(b, l));
                    occ_p[tid](l0, m0) += s;
                }
        }
    });
    std::vector<cd> g((size_t)Nf * D * D), g0((size_t)Nf * D * D);
    Mat num(D, D), num0(D, D), occ(D, D);
    for (int t = 0; t < T; t++) {
        for (size_t i = 0; i < g.size(); i++) { g[i] += g_p[t][i]; g0[i] += g0_p[t][i]; }
        num = add(num, num_p[t]);
        num0 = add(num0, num0_p[t]);
        occ = add(occ, occ_p[t]);
        if (st_p[t]) st = st_p[t];
    }
    for (size_t i = 0; i < g.size(); i++) { g[i] /= (double)nk; g0[i] /= (double)nk; }
    std::memcpy(gw, g.data(), sizeof(cd) * g.size());
    if (gwhf) std::memcpy(gwhf, g0.data(), sizeof(cd) * g0.size());
    // occupation tails (:322-354)
    for (int l0 = 0; l0 < D; l0++) {
        for (int m0 = 0; m0 < D; m0++) { num(l0, m0) /= beta; num0(l0, m0) /= beta; }
        num(l0, l0) += 0.5 * nk;
        num0(l0, l0) += 0.5 * nk;
    }
    num = add(num, occ);
    for (auto &x : num.a) x /= (double)nk;
    for (auto &x : num0.a) x /= (double)nk;
    store(sub(num, num0), nummat);
    return st;
}

/* src/GreenFtn.cpp:513-635  GiwToNele, evaluated with the trace identity
 *   sum_l Re 1/(w - e_l + mu) = Re Tr [(w + mu) I - H - S(w)]^-1
 * (S placed on within-cluster blocks as in the valenceHAMILTONIAN macro, :9-56); the core-level term
 * vanishes for the full model window (NBAND == NumOrbit).  dnele (optional) = dN/dmu. */
int orc_nele(const orc_lattice *L, const double *hk, const double *sigma, double mu, double *nele,
             double *dnele, int nthreads) {
    const int n = L->n, nk = L->nk, Nf = L->nfreq, D = L->ncl * L->nh;
    const double beta = L->beta;
    std::vector<Mat> S = load_stack(sigma, Nf, D), mom;
    int st = moments_fit(D, Nf, beta, S, false, mom);
    if (st) return st;
    int T = std::max(1, std::min(nthreads, nk));
    std::vector<double> sum_p(T, 0.0), fermi_p(T, 0.0), dsum_p(T, 0.0), dfermi_p(T, 0.0);
    std::vector<int> st_p(T, OK);
    const cd w0 = I1 * PI / beta, dw = I1 * (2 * PI) / beta;  // src/tight_common.cpp:248-249
    parallel_for(nk, T, [&](int kb, int ke, int tid) {
        for (int k = kb; k < ke; k++) {
            Mat H = load(hk + (size_t)2 * n * n * k, n, n);
            Mat Hs = H;
            add_sigma_block(Hs, mom[0], L, true, 1.0);
            std::vector<double> einf;
            heig(Hs, einf, nullptr);
            for (int nn = 0; nn < 2 * Nf; nn++) {
                cd iw = I1 * PI * (2. * nn + 1.) / beta;
                Mat SW(D, D);
                if (nn < Nf) SW = S[nn];
                else
                    for (int a = 0; a < D * D; a++)
                        SW.a[a] = mom[0].a[a] + mom[1].a[a] / iw + mom[2].a[a] / std::pow(iw, 2) +
                                  mom[3].a[a] / std::pow(iw, 3);
                cd w = w0 + (double)nn * dw;
                Mat A = scal(H, -1.0);
                add_sigma_block(A, SW, L, true, -1.0);
                for (int i = 0; i < n; i++) A(i, i) += (w + mu);
                Mat G;
                if (lu_inverse(A, G)) st_p[tid] = SINGULAR;
                double tr = 0, tr2 = 0;
                for (int l = 0; l < n; l++) tr += std::real(G(l, l));
                if (dnele) {
                    cd s2 = 0;
                    for (int i = 0; i < n; i++)
                        for (int j = 0; j < n; j++) s2 += G(i, j) * G(j, i);
                    tr2 = std::real(s2);
                }
                double ti = 0, ti2 = 0;
                for (int l = 0; l < n; l++) {
                    cd x = 1. / (w - einf[l] + mu);
                    ti += std::real(x);
                    ti2 += std::real(x * x);
                }
                sum_p[tid] += tr - ti;
                dsum_p[tid] += -tr2 + ti2;
            }
            for (int l = 0; l < n; l++) {
                double f = 1. / (1 + std::exp(beta * (einf[l] - mu)));
                fermi_p[tid] += f;
                dfermi_p[tid] += beta * f * (1 - f);
            }
        }
    });
    double s = 0, fs = 0, ds = 0, dfs = 0;
    for (int t = 0; t < T; t++) {
        s += sum_p[t];
        fs += fermi_p[t];
        ds += dsum_p[t];
        dfs += dfermi_p[t];
        if (st_p[t]) st = st_p[t];
    }
    double N = s * 2. / beta + fs;
    *nele = N / nk;
    if (dnele) *dnele = (ds * 2. / beta + dfs) / nk;
    if (!std::isfinite(*nele)) return NANINF;
    return st;
}

/* src/GreenFtn.cpp:66-139  GreenFtn_w_adjust_mu: bracket expansion, then bisection to |dmu| <= 1e-5. */
int orc_adjust_mu(const orc_lattice *L, const double *hk, const double *sigma, double mu, double dmu,
                  double n_target, double *mu_out, int *n_eval, int nthreads) {
    int evals = 0;
    auto N = [&](double m, double *out) {
        evals++;
        return orc_nele(L, hk, sigma, m, out, nullptr, nthreads);
    };
    double Nele[2] = {-1, -1};
    int st = N(mu, &Nele[0]);
    if (st) return st;
    double muUB = 0, muLB = 0, mu_next;
    const double goal = n_target;
    int nearAns = 0;
    if (Nele[0] > goal) mu -= (dmu - dmu);
    else if (Nele[0] < goal) mu -= (dmu + dmu);
    int guard = 0;
    while ((Nele[0] != goal) && std::abs(dmu) > 1e-5) {
        if (++guard > 10000) return NONCONV;
        mu += dmu;
        Nele[1] = Nele[0];
        st = N(mu, &Nele[0]);
        if (st) return st;
        if (nearAns == 0) {
            if (Nele[0] < goal) {
                muLB = mu;
                if (Nele[1] > goal && Nele[1] > 0) nearAns = 1;
                else dmu = std::fabs(dmu);
            }
            if (Nele[0] > goal) {
                muUB = mu;
                if (Nele[1] < goal && Nele[1] > 0) nearAns = 1;
                else dmu = -1 * std::fabs(dmu);
            }
            if (Nele[0] == goal) break;
            if (!(std::abs(mu) < 600)) return NONCONV;
        } else {
            if (Nele[0] > goal) muUB = mu;
            else if (Nele[0] < goal) muLB = mu;
            mu_next = (muUB + muLB) / 2.;
            dmu = mu_next - mu;
        }
    }
    *mu_out = mu;
    if (n_eval) *n_eval = evals;
    return OK;
}

/* src/Construct_hyb_delta.cpp:47-119: Delta_n = (iw+mu) I - Himp[P] - S_n[P] - (G_n[P])^-1. */
int orc_hyb_delta(int dim, const int *orb, int nfreq, double beta, int D, const double *sigma, const double *gw,
                  const double *himp, double mu, double *delta) {
    for (int i = 0; i < dim; i++)
        if (orb[i] < 0 || orb[i] >= D) return BADARG;
    std::vector<Mat> S = load_stack(sigma, nfreq, D), G = load_stack(gw, nfreq, D);
    Mat Hi = load(himp, D, D);
    int st = OK;
    for (int nn = 0; nn < nfreq; nn++) {
        cd iw = I1 * PI * (2. * nn + 1.) / beta;
        Mat pS(dim, dim), pG(dim, dim), pH(dim, dim);
        for (int h1 = 0; h1 < dim; h1++)
            for (int h2 = 0; h2 < dim; h2++) {
                pS(h1, h2) = S[nn](orb[h1], orb[h2]);
                pG(h1, h2) = G[nn](orb[h1], orb[h2]);
                pH(h1, h2) = Hi(orb[h1], orb[h2]);
            }
        Mat Gi;
        if (dim != 0 && lu_inverse(pG, Gi)) st = SINGULAR;
        Mat Dl(dim, dim);
        for (int h1 = 0; h1 < dim; h1++) {
            for (int h2 = 0; h2 < dim; h2++) Dl(h1, h2) = -pH(h1, h2) - pS(h1, h2) - Gi(h1, h2);
            Dl(h1, h1) = Dl(h1, h1) + iw + mu;
        }
        store(Dl, delta + (size_t)2 * dim * dim * nn);
    }
    return st;
}

/* src/FourierTransform.cpp:126-178  FourierTransform_ with given moments (tau_j = j beta / N_tau). */
int orc_w2tau(int dim, int nfreq, int ntau, double beta, const double *fw, const double *mom, double *ft,
              int *fixups) {
    std::vector<Mat> F = load_stack(fw, nfreq, dim), M = load_stack(mom, 4, dim);
    Tail T = make_tail(dim, M);
    std::vector<Mat> tails(nfreq);
    double dwl = (2 * PI) / beta, w0l = (PI / beta);
    parallel_for(nfreq, g_nthreads, [&](int b, int e, int) {
        for (int i = b; i < e; i++) tails[i] = tail_w(T, w0l + i * dwl);
    });
    std::vector<Mat> out(ntau + 1);
    parallel_for(ntau + 1, g_nthreads, [&](int b, int e, int) {
        for (int j = b; j < e; j++) out[j] = ft_tau(F, T, tails, nfreq, beta, j * beta / ntau);
    });
    int nfix = positivity_fixup(out, ntau, beta);
    if (fixups) *fixups = nfix;
    store_stack(out, ntau + 1, ft);
    return OK;
}

int orc_w2tau_single(int dim, int nfreq, double beta, const double *fw, const double *mom, double tau,
                     double *out) {
    std::vector<Mat> F = load_stack(fw, nfreq, dim), M = load_stack(mom, 4, dim);
    Tail T = make_tail(dim, M);
    std::vector<Mat> tails(nfreq);
    double dwl = (2 * PI) / beta, w0l = (PI / beta);
    for (int i = 0; i < nfreq; i++) tails[i] = tail_w(T, w0l + i * dwl);
    store(ft_tau(F, T, tails, nfreq, beta, tau), out);
    return OK;
}

/* src/FourierTransform.cpp:470-488  FourierTransform(delta_w, delta_t[, moments1], greenFtnAsym):
 * fit the moments, optionally replace m0 = 0 and m1 = *m1, then FourierTransform_. */
int orc_fourier(int dim, int nfreq, int ntau, double beta, const double *fw, int green_asym, const double *m1,
                double *ft, int *fixups) {
    std::vector<Mat> F = load_stack(fw, nfreq, dim), M;
    int st = moments_fit(dim, nfreq, beta, F, green_asym != 0, M);
    if (st) return st;
    if (m1) {
        M[0] = Mat(dim, dim);
        M[1] = load(m1, dim, dim);
    }
    std::vector<double> mom((size_t)8 * dim * dim);
    store_stack(M, 4, mom.data());
    return orc_w2tau(dim, nfreq, ntau, beta, fw, mom.data(), ft, fixups);
}

/* src/FourierTransform.cpp:521-561  FT_t_to_w: exact integral of the piecewise-linear F(tau). */
int orc_tau2w(int dim, int nfreq, int ntau, double beta, const double *ft, double *fw) {
    std::vector<Mat> Dt = load_stack(ft, ntau + 1, dim);
    int Nseg = ntau;
    std::vector<Mat> at(Nseg), bt(Nseg);
    double dt = beta / Nseg;
    for (int t = 0; t < Nseg; t++) {
        double tau0 = t * dt, tau1 = (t + 1) * dt;
        at[t] = scal(sub(Dt[t + 1], Dt[t]), 1.0 / (tau1 - tau0));
        bt[t] = add(scal(at[t], -tau0), Dt[t]);
    }
    std::vector<char> causal(nfreq, 0);
    parallel_for(nfreq, g_nthreads, [&](int nb, int ne, int) {
    for (int nn = nb; nn < ne; nn++) {
        double wn = (2 * nn + 1) * PI / beta;
        Mat W(dim, dim);
        for (int t = 0; t < Nseg; t++) {
            double tau0 = t * dt, tau1 = (t + 1) * dt;
            cd e1 = std::exp(I1 * tau1 * wn), e0 = std::exp(I1 * tau0 * wn);
            cd pI = (e1 - e0);
            cd pI2 = (tau1 * e1 - tau0 * e0);
            cd ca = (pI / (std::pow(wn, 2)) + pI2 / (I1 * wn)), cb = pI / (I1 * wn);
            for (int k = 0; k < dim * dim; k++) W.a[k] += at[t].a[k] * ca + bt[t].a[k] * cb;
        }
        Mat test = scal(sub(W, adj(W)), 1.0 / (2.0 * I1));
        if (max_eig(test) > 0) causal[nn] = 1;
        store(W, fw + (size_t)2 * dim * dim * nn);
    }
    });
    for (int nn = 0; nn < nfreq; nn++)
        if (causal[nn]) return CAUSAL;
    return OK;
}

/* src/SCGF2_fullLoop.cpp:603-690  getStimp: second-order Sigma(tau) from G(tau), U_{ijkl} list. */
int orc_sigma2_tau(int dim, int ntau, double beta, int nu, const int *uidx, const double *ut, const double *gt,
                   double *st, int *fixups) {
    std::vector<Mat> G = load_stack(gt, ntau + 1, dim), S(ntau + 1);
    std::vector<cd> U(nu);
    for (int x = 0; x < nu; x++) U[x] = cd(ut[2 * x], ut[2 * x + 1]);
    std::vector<char> herm(ntau + 1, 0);
    parallel_for(ntau + 1, g_nthreads, [&](int tb, int te, int) {
    for (int t = tb; t < te; t++) {
        Mat Sn(dim, dim);
        const Mat &Gt = G[t], &Gm = G[ntau - t];
        for (int x1 = 0; x1 < nu; x1++) {
            int i = uidx[4 * x1], q = uidx[4 * x1 + 1], m = uidx[4 * x1 + 2], k = uidx[4 * x1 + 3];
            for (int x2 = 0; x2 < nu; x2++) {
                int l = uidx[4 * x2], n = uidx[4 * x2 + 1], p = uidx[4 * x2 + 2], j = uidx[4 * x2 + 3];
                Sn(i, j) += (-1.0) * Gt(k, l) * Gt(m, n) * (-Gm(p, q)) * U[x1] * U[x2];
                Sn(i, j) += Gt(k, n) * Gt(m, l) * (-Gm(p, q)) * U[x1] * U[x2];
            }
        }
        S[t] = Sn;
        if (fnorm(scal(sub(Gt, adj(Gt)), 1.0 / (2.0 * I1))) > 1e-10) herm[t] = 1;
        if (fnorm(scal(sub(Sn, adj(Sn)), 1.0 / (2.0 * I1))) > 1e-5) herm[t] = 1;
    }
    });
    int status = OK;
    for (int t = 0; t < ntau + 1; t++)
        if (herm[t]) status = HERMIT;
    int nfix = positivity_fixup(S, ntau, beta);
    if (fixups) *fixups = nfix;
    store_stack(S, ntau + 1, st);
    return status;
}

/* src/SCGF2_fullLoop.cpp:583-597  getFockOperator. */
void orc_fock(int dim, int nu, const int *uidx, const double *ut, const double *occ, double *fock) {
    Mat O = load(occ, dim, dim), F(dim, dim);
    for (int x = 0; x < nu; x++) {
        int a = uidx[4 * x], b = uidx[4 * x + 1], c = uidx[4 * x + 2], d = uidx[4 * x + 3];
        cd u(ut[2 * x], ut[2 * x + 1]);
        F(b, d) += u * O(c, a);
        F(b, c) -= u * O(d, a);
    }
    store(F, fock);
}

/* src/SCGF2_fullLoop.cpp:551-578  getGwimp: G_n = [(iw_n+mu) - Himp - Delta_n - F - S2_n]^-1. */
int orc_dyson(int dim, int nfreq, double beta, double mu, const double *himp, const double *delta,
              const double *fock, const double *sigma2, double *gw) {
    Mat Hi = load(himp, dim, dim), F = load(fock, dim, dim);
    int st = OK;
    for (int nn = 0; nn < nfreq; nn++) {
        double wn = (PI * (2. * nn + 1.)) / beta;
        Mat Dl = load(delta + (size_t)2 * dim * dim * nn, dim, dim);
        Mat S2 = load(sigma2 + (size_t)2 * dim * dim * nn, dim, dim);
        Mat A = scal(Mat::eye(dim), I1 * wn + mu);
        A = sub(sub(sub(sub(A, Hi), Dl), F), S2);
        Mat G;
        if (lu_inverse(A, G)) st = SINGULAR;
        Mat test = scal(sub(G, adj(G)), 1.0 / (2.0 * I1));
        if (!(max_eig(test) < 0) && st == OK) st = CAUSAL;
        store(G, gw + (size_t)2 * dim * dim * nn);
    }
    return st;
}

/* src/SCGF2_fullLoop.cpp:736-787  estimate_asymto: f holds nfreq+3 matrices; writes slot nfreq+order-1. */
void orc_estimate_asymto(int dim, int nfreq, double beta, double *f, int order) {
    int Nf = nfreq;
    std::vector<Mat> F = load_stack(f, Nf + 3, dim);
    Mat tail[3], coeff;
    double w0, w1, w2;
    auto wn = [&](int i) { return (2 * (Nf - 3 + i) + 1) * PI / beta; };
    if (order == 1) {
        w0 = 1. / std::pow((2 * (Nf - 3) + 1) * PI / beta, 2);
        w1 = 1. / std::pow((2 * (Nf - 2) + 1) * PI / beta, 2);
        w2 = 1. / std::pow((2 * (Nf - 1) + 1) * PI / beta, 2);
        for (int w = 0; w < 3; w++) {
            tail[w] = F[Nf - 3 + w];
            tail[w] = scal(sub(adj(tail[w]), tail[w]), 0.5);
            tail[w] = scal(tail[w], 1.0 / (I1 * wn(w)));
        }
        coeff = scal(add(add(tail[0], tail[1]), tail[2]), 1.0 / (w0 + w1 + w2));
        F[Nf + 0] = coeff;
    } else if (order == 2) {
        w0 = 1. / std::pow((2 * (Nf - 3) + 1) * PI / beta, 4);
        w1 = 1. / std::pow((2 * (Nf - 2) + 1) * PI / beta, 4);
        w2 = 1. / std::pow((2 * (Nf - 1) + 1) * PI / beta, 4);
        for (int w = 0; w < 3; w++) {
            tail[w] = F[Nf - 3 + w];
            tail[w] = scal(add(tail[w], adj(tail[w])), 0.5);
            tail[w] = scal(tail[w], -1.0 / std::pow(wn(w), 2));
        }
        coeff = scal(add(add(tail[0], tail[1]), tail[2]), 1.0 / (w0 + w1 + w2));
        F[Nf + 1] = coeff;
    } else if (order == 3) {
        w0 = 1. / std::pow((2 * (Nf - 3) + 1) * PI / beta, 6);
        w1 = 1. / std::pow((2 * (Nf - 2) + 1) * PI / beta, 6);
        w2 = 1. / std::pow((2 * (Nf - 1) + 1) * PI / beta, 6);
        for (int w = 0; w < 3; w++) {
            tail[w] = sub(F[Nf - 3 + w], scal(F[Nf], 1.0 / (I1 * wn(w))));
            tail[w] = scal(sub(adj(tail[w]), tail[w]), 0.5);
            tail[w] = scal(tail[w], I1 / std::pow(wn(w), 3));
        }
        coeff = scal(add(add(tail[0], tail[1]), tail[2]), 1.0 / (w0 + w1 + w2));
        F[Nf + 2] = coeff;
    }
    store_stack(F, Nf + 3, f);
}

/* src/SCGF2_fullLoop.cpp:539-549  getoccMat: n = -G(tau = beta^-) with the m0 = 0, m1 = I green tail. */
int orc_occ(int dim, int nfreq, double beta, const double *gw, double *occ) {
    std::vector<Mat> F = load_stack(gw, nfreq, dim), M;
    int st = moments_fit(dim, nfreq, beta, F, true, M);
    if (st) return st;
    M[0] = Mat(dim, dim);
    M[1] = Mat::eye(dim);
    std::vector<double> mom((size_t)8 * dim * dim);
    store_stack(M, 4, mom.data());
    std::vector<double> out((size_t)2 * dim * dim);
    orc_w2tau_single(dim, nfreq, beta, gw, mom.data(), beta, out.data());
    for (size_t i = 0; i < out.size(); i++) occ[i] = -out[i];
    return OK;
}

/* src/gen_Uijkl.cpp:9-58 (Kanamori) and :60-87 (density-density).  Returns the number of entries. */
int orc_gen_uijkl(int nso, double U, double Up, double J, int density_density, int cap, int *uidx, double *ut) {
    int cnt = 0;
    auto push = [&](int i, int j, int k, int l, double v) {
        if (cnt < cap) {
            uidx[4 * cnt] = i; uidx[4 * cnt + 1] = j; uidx[4 * cnt + 2] = k; uidx[4 * cnt + 3] = l;
            ut[2 * cnt] = v; ut[2 * cnt + 1] = 0.0;
        }
        cnt++;
    };
    if (density_density) {
        for (int n = 0; n < nso; n++)
            for (int m = 0; m < nso; m++) {
                double v = 0;
                if (n / 2 == m / 2) v = U;
                else if (n / 2 != m / 2) v = Up;
                if (n % 2 == m % 2) v -= J;
                push(n, m, n, m, v);
            }
        return cnt;
    }
    for (int i = 0; i < nso; i++)
        for (int j = 0; j < nso; j++)
            for (int k = 0; k < nso; k++)
                for (int l = 0; l < nso; l++) {
                    int io = i / 2, is = i % 2, jo = j / 2, js = j % 2, ko = k / 2, ks = k % 2, lo = l / 2, ls = l % 2;
                    double c = 0;
                    if (i == k && j == l) {
                        if (io == jo) c = U;
                        else if (io != jo) c = Up;
                        if (is == js) c -= J;
                    } else if (ko == io && lo == jo && ko != lo && ks != is && ls != js && ks != ls)
                        c = J;
                    else if (ko == lo && ko != io && io == jo && ks != ls && ks == is && ls == js)
                        c = J;
                    if (c != 0) push(i, j, k, l, c);
                }
    return cnt;
}

/* src/SCGF2_fullLoop.cpp:873-1065  IPT (Kajueter-Kotliar on 2 spin-orbitals).
 * Slots follow ImgFreqFtn (src/ImgTimeFtn.cpp:177): se_out and gimp_out hold nfreq+5 matrices;
 * delta holds nfreq matrices; nummat_in is projNumMatrix, nummat_out its update. */
int orc_ipt(int dim, int nfreq, int ntau, double beta, double U, double mu, const double *himp,
            const double *delta, const double *nummat_in, int nu, const int *uidx, const double *ut,
            double *se_out, double *gimp_out, double *nummat_out) {
    if (dim != 2) return BADARG;
    const int Nf = nfreq, DD = dim * dim;
    const size_t M = (size_t)2 * DD;
    std::vector<double> fock(M), occ(M), occHF(M), zero((size_t)2 * DD * (Nf + 3), 0.0);
    std::memcpy(occ.data(), nummat_in, sizeof(double) * M);
    occHF = occ;
    const double muHF = mu;
    orc_fock(dim, nu, uidx, ut, occHF.data(), fock.data());
    // Gw0: nfreq + 4 slots ([Nf] = I, [Nf+1..3] = 0)
    std::vector<double> gw0((size_t)2 * DD * (Nf + 4), 0.0), s2((size_t)2 * DD * (Nf + 3), 0.0);
    int st = orc_dyson(dim, Nf, beta, muHF, himp, delta, fock.data(), s2.data(), gw0.data());
    int stc = st;
    for (int i = 0; i < dim; i++) gw0[(size_t)2 * DD * Nf + 2 * (i + i * dim)] = 1.0;
    // FourierTransform(Gw0, Gt0, Gw0[N_freq]) : greenFtnAsym = false, m1 = Gw0[N_freq] = I
    std::vector<double> gt((size_t)2 * DD * (ntau + 1)), stt((size_t)2 * DD * (ntau + 1));
    st = orc_fourier(dim, Nf, ntau, beta, gw0.data(), 0, gw0.data() + (size_t)2 * DD * Nf, gt.data(), nullptr);
    if (st) return st;
    st = orc_sigma2_tau(dim, ntau, beta, nu, uidx, ut, gt.data(), stt.data(), nullptr);
    if (st) stc = st;
    st = orc_tau2w(dim, Nf, ntau, beta, stt.data(), s2.data());
    if (st && !stc) stc = st;
    // Kajueter-Kotliar interpolation on (0,0), (1,1)  (:1033-1046)
    auto re = [&](const std::vector<double> &m, int i, int j) { return m[2 * (i + j * dim)]; };
    double a[2], b[2], c[2];
    a[0] = U * U * re(occ, 1, 1) * (1.0 - re(occ, 1, 1));
    a[1] = U * U * re(occ, 0, 0) * (1.0 - re(occ, 0, 0));
    b[0] = (muHF - mu + U * (1.0 - 2.0 * re(occ, 1, 1)));
    b[1] = (muHF - mu + U * (1.0 - 2.0 * re(occ, 0, 0)));
    c[0] = U * U * re(occHF, 1, 1) * (1.0 - re(occHF, 1, 1));
    c[1] = U * U * re(occHF, 0, 0) * (1.0 - re(occHF, 0, 0));
    for (int nn = 0; nn < Nf; nn++)
        for (int d = 0; d < 2; d++) {
            cd *p = reinterpret_cast<cd *>(s2.data() + (size_t)2 * DD * nn) + (d + d * dim);
            cd x = *p;
            // the reference's std::complex arithmetic: a*S / (c - b*S); imag parts of a,b,c are 0
            *p = a[d] * x / (c[d] - b[d] * x);
        }
    std::vector<double> gimp((size_t)2 * DD * (Nf + 4), 0.0);
    st = orc_dyson(dim, Nf, beta, mu, himp, delta, fock.data(), s2.data(), gimp.data());
    if (st && !stc) stc = st;
    for (int i = 0; i < dim; i++) gimp[(size_t)2 * DD * Nf + 2 * (i + i * dim)] = 1.0;
    orc_estimate_asymto(dim, Nf, beta, gimp.data(), 2);
    orc_estimate_asymto(dim, Nf, beta, gimp.data(), 3);
    std::vector<double> occ_new(M);
    st = orc_occ(dim, Nf, beta, gimp.data(), occ_new.data());
    if (st) return st;
    std::memcpy(nummat_out, occ_new.data(), sizeof(double) * M);
    // writeResults (:696-720)
    orc_estimate_asymto(dim, Nf, beta, s2.data(), 1);
    orc_estimate_asymto(dim, Nf, beta, s2.data(), 2);
    std::memset(se_out, 0, sizeof(double) * (size_t)2 * DD * (Nf + 5));
    for (int nn = 0; nn < Nf; nn++)
        for (size_t k = 0; k < M; k++) {
            se_out[M * nn + k] = s2[M * nn + k] + fock[k];
            gimp_out[M * nn + k] = gimp[M * nn + k];
        }
    for (size_t k = 0; k < M; k++) {
        se_out[M * Nf + k] = fock[k];
        se_out[M * (Nf + 1) + k] = s2[M * Nf + k];
        se_out[M * (Nf + 2) + k] = s2[M * (Nf + 1) + k];
        gimp_out[M * Nf + k] = 0.0;
        for (int s = 1; s <= 4; s++) gimp_out[M * (Nf + s) + k] = gimp[M * (Nf + s - 1) + k];
    }
    return stc;
}

}  // extern "C"
