// reference_layout_client.cpp -- a C++ caller of libdmftgpu that keeps its data the way the reference's hot path
// does: std::vector of column-major complex matrices (one per k point or Matsubara frequency, as
// std::vector<Eigen::MatrixXcd> holds them), the lattice sizes as plain values (the reference's globals), and thin
// shims with the reference's names and argument order (src/TB.h:45-61) that pack the matrices into the library's
// contiguous stacks and unpack the results.  No Eigen: std::complex<double> has the same layout as Eigen's cmplx.
//
//   reference_layout_client IN OUT
//   IN : int32 n, nk, nfreq, D; float64 beta, mu0, n_target; then H_k (nk n x n, column-major complex) and
//        SelfE_w (nfreq D x D), both as interleaved re/im float64
//   OUT: float64 mu (adjusted), then Gw (nfreq D x D), NumMatrix (D x D), weiss_fieldTB (nfreq D x D)
//
//   reference_layout_client restart IN OUT N_freq Norbit beta beta_prev
//   an ImgFreqFtn restart file IN (written at beta_prev) read with read_full on beta's grid, written with
//   dataOut_full to OUT (host only: no device is touched)
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "dmftgpu.h"

typedef std::complex<double> cmplx;
typedef std::vector<cmplx> Mat;  // one column-major matrix, like Eigen::MatrixXcd::data()

struct Globals {  // the reference's globals the shims translate into arguments
    int NBAND, knum, N_freq, NumCluster, NumHartrOrbit_per_cluster;
    double beta;
};

static std::vector<cmplx> pack(const std::vector<Mat> &v) {
    std::vector<cmplx> out;
    for (const Mat &m : v) out.insert(out.end(), m.begin(), m.end());
    return out;
}
static void unpack(const std::vector<cmplx> &flat, int count, int dim, std::vector<Mat> &v) {
    v.assign(count, Mat((size_t)dim * dim));
    for (int c = 0; c < count; c++)
        for (int e = 0; e < dim * dim; e++) v[c][e] = flat[(size_t)c * dim * dim + e];
}
static dmftgpu_lattice lattice(const Globals &g) {
    dmftgpu_lattice L;
    L.n = g.NBAND;
    L.nk = g.knum;
    L.nfreq = g.N_freq;
    L.beta = g.beta;
    L.ncl = g.NumCluster;
    L.nh = g.NumHartrOrbit_per_cluster;
    L.hartr = nullptr;
    return L;
}
static void check(int st, const char *what, dmftgpu_ctx *ctx) {
    if (st != DMFTGPU_OK) {
        std::fprintf(stderr, "%s failed: %d (%s)\n", what, st, ctx ? dmftgpu_last_error(ctx) : "");
        std::exit(2);
    }
}

// double GreenFtn_w_adjust_mu(std::vector<MatrixXcd>& H_k, ImgFreqFtn& SelfE_w, double mu, double dmu, int mu_adjust)
static double GreenFtn_w_adjust_mu(dmftgpu_ctx *ctx, const Globals &g, const std::vector<Mat> &H_k,
                                   const std::vector<Mat> &SelfE_w, double mu, double dmu, double NumberOfElectron) {
    dmftgpu_lattice L = lattice(g);
    std::vector<cmplx> h = pack(H_k), s = pack(SelfE_w);
    double out = mu;
    int nev = 0;
    check(dmftgpu_adjust_mu(ctx, &L, (const double *)h.data(), (const double *)s.data(), mu, dmu, NumberOfElectron,
                            &out, &nev, 0),
          "dmftgpu_adjust_mu", ctx);
    return out;
}

// void GreenFtn_w(int NumCluster, int NumHartrOrbit_per_cluster, std::vector<MatrixXcd>& H_k, ImgFreqFtn& SelfE_w,
//                 std::vector<MatrixXcd>& Gw, double mu, ...) -- NumMatrix is the reference's global output
static void GreenFtn_w(dmftgpu_ctx *ctx, const Globals &g, const std::vector<Mat> &H_k, const std::vector<Mat> &SelfE_w,
                       std::vector<Mat> &Gw, double mu, Mat &NumMatrix) {
    dmftgpu_lattice L = lattice(g);
    const int D = g.NumCluster * g.NumHartrOrbit_per_cluster;
    std::vector<cmplx> h = pack(H_k), s = pack(SelfE_w), gw((size_t)g.N_freq * D * D), nm((size_t)D * D);
    check(dmftgpu_greenftn_w(ctx, &L, (const double *)h.data(), (const double *)s.data(), mu, (double *)gw.data(),
                             nullptr, (double *)nm.data(), 0),
          "dmftgpu_greenftn_w", ctx);
    unpack(gw, g.N_freq, D, Gw);
    NumMatrix = nm;
}

// void Construct_hyb_delta(int impurityDim, std::vector<int> impurityOrbit, ImgFreqFtn& SelfE_w,
//                          std::vector<MatrixXcd> Gw, double mu, ImgFreqFtn& weiss_fieldTB, int atom, ...)
static void Construct_hyb_delta(dmftgpu_ctx *ctx, const Globals &g, int impurityDim, const std::vector<int> &impurityOrbit,
                                const std::vector<Mat> &SelfE_w, const std::vector<Mat> &Gw, double mu,
                                const Mat &impurity_site_Hamiltonian, std::vector<Mat> &weiss_fieldTB) {
    const int D = g.NumCluster * g.NumHartrOrbit_per_cluster;
    std::vector<cmplx> s = pack(SelfE_w), gw = pack(Gw), out((size_t)g.N_freq * impurityDim * impurityDim);
    check(dmftgpu_hyb_delta(ctx, impurityDim, impurityOrbit.data(), g.N_freq, g.beta, D, (const double *)s.data(),
                            (const double *)gw.data(), (const double *)impurity_site_Hamiltonian.data(), mu,
                            (double *)out.data(), 0),
          "dmftgpu_hyb_delta", ctx);
    unpack(out, g.N_freq, impurityDim, weiss_fieldTB);
}

// ImgFreqFtn's restart-file methods (src/ImgTimeFtn.cpp:330-355, 624-670, 673-751) over the library's host calls:
// Ftn_ holds N_freq + 5 column-major Norbit x Norbit matrices
struct ImgFreqFtn {
    int Nfreq_, Norbit;
    std::vector<Mat> Ftn_;
    ImgFreqFtn(int nfreq, int norbit) : Nfreq_(nfreq), Norbit(norbit), Ftn_(nfreq + 5, Mat((size_t)norbit * norbit)) {}
    void dataOut_full(const char *filename) {
        std::vector<cmplx> flat = pack(Ftn_);
        check(dmftgpu_imgfreq_write(filename, Nfreq_, Norbit, (const double *)flat.data()), "dmftgpu_imgfreq_write",
              nullptr);
    }
    void update_full(const char *filename) {
        std::vector<cmplx> flat = pack(Ftn_);
        check(dmftgpu_imgfreq_update(filename, Nfreq_, Norbit, (double *)flat.data()), "dmftgpu_imgfreq_update",
              nullptr);
        unpack(flat, Nfreq_ + 5, Norbit, Ftn_);
    }
    void read_full(const char *filename, double beta, double beta_prev) {
        std::vector<cmplx> flat((size_t)(Nfreq_ + 5) * Norbit * Norbit);
        check(dmftgpu_imgfreq_read(filename, Nfreq_, Norbit, beta, beta_prev, (double *)flat.data()),
              "dmftgpu_imgfreq_read", nullptr);
        unpack(flat, Nfreq_ + 5, Norbit, Ftn_);
    }
};

int main(int argc, char **argv) {
    if (argc == 8 && std::string(argv[1]) == "restart") {
        ImgFreqFtn SelfE_w(std::atoi(argv[4]), std::atoi(argv[5]));
        SelfE_w.read_full(argv[2], std::atof(argv[6]), std::atof(argv[7]));
        SelfE_w.dataOut_full(argv[3]);
        return 0;
    }
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 1;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 1;
    int dims[4];
    double par[3];
    if (std::fread(dims, sizeof(int), 4, f) != 4 || std::fread(par, sizeof(double), 3, f) != 3) return 1;
    Globals g;
    g.NBAND = dims[0];
    g.knum = dims[1];
    g.N_freq = dims[2];
    g.NumCluster = 1;
    g.NumHartrOrbit_per_cluster = dims[3];
    g.beta = par[0];
    const int n = g.NBAND, D = dims[3];
    std::vector<Mat> H_k(g.knum, Mat((size_t)n * n)), SelfE_w(g.N_freq, Mat((size_t)D * D));
    for (Mat &m : H_k)
        if (std::fread(m.data(), sizeof(cmplx), m.size(), f) != m.size()) return 1;
    for (Mat &m : SelfE_w)
        if (std::fread(m.data(), sizeof(cmplx), m.size(), f) != m.size()) return 1;
    std::fclose(f);

    dmftgpu_ctx *ctx = nullptr;
    check(dmftgpu_create(&ctx, 0), "dmftgpu_create", nullptr);
    const double mu = GreenFtn_w_adjust_mu(ctx, g, H_k, SelfE_w, par[1], 1.0, par[2]);
    std::vector<Mat> Gw, weiss;
    Mat NumMatrix;
    GreenFtn_w(ctx, g, H_k, SelfE_w, Gw, mu, NumMatrix);
    // impurity_site_Hamiltonian: the k average of the correlated block (downfolding.cpp's model-Hamiltonian case)
    Mat himp((size_t)D * D, cmplx(0, 0));
    for (const Mat &h : H_k)
        for (int j = 0; j < D; j++)
            for (int i = 0; i < D; i++) himp[i + (size_t)j * D] += h[i + (size_t)j * n] / (double)g.knum;
    std::vector<int> orb(D);
    for (int i = 0; i < D; i++) orb[i] = i;
    Construct_hyb_delta(ctx, g, D, orb, SelfE_w, Gw, mu, himp, weiss);
    dmftgpu_destroy(ctx);

    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 1;
    std::fwrite(&mu, sizeof(double), 1, o);
    for (const Mat &m : Gw) std::fwrite(m.data(), sizeof(cmplx), m.size(), o);
    std::fwrite(NumMatrix.data(), sizeof(cmplx), NumMatrix.size(), o);
    for (const Mat &m : weiss) std::fwrite(m.data(), sizeof(cmplx), m.size(), o);
    std::fclose(o);
    return 0;
}
