// restart_io.cu -- ImgFreqFtn's text files (Sw_SOLVER.full.dat, Gw_loc.full.dat, delta_w.full.dat ...), the
// restart format of DMFTpack, on the host: dataOut_full, update_full and read_full (src/ImgTimeFtn.cpp:330-355,
// 624-670, 673-751).  Arrays are ImgFreqFtn stacks: nfreq + 5 slots (N_freq Matsubara points, then the five tail
// slots) of column-major norbit x norbit complex matrices, element (m, n) of slot w at 2 (w N^2 + m + n N).
#include <cmath>
#include <cstdio>
#include <new>
#include <vector>

#include "dmftgpu.h"

namespace {

constexpr double TOL = 1e-7;  // dataOut_full writes |F| > tol only (src/ImgTimeFtn.cpp:10)
constexpr int W_MAX = 1 << 24;  // frequency indices at or above this mark a damaged file (DMFTGPU_BADARG)

struct Row {
    int w, m, n;
    double re, im;
};

// the "%d %d %d %lf %lf" records of a file; lines that do not hold five fields are skipped
int read_rows(const char *path, std::vector<Row> &rows) {
    FILE *f = std::fopen(path, "r");
    if (!f) return DMFTGPU_IO;
    char line[512];
    int st = DMFTGPU_OK;
    try {
        while (std::fgets(line, sizeof line, f)) {
            Row r;
            if (std::sscanf(line, "%d %d %d %lf %lf", &r.w, &r.m, &r.n, &r.re, &r.im) == 5) {
                if (r.w >= W_MAX) st = DMFTGPU_BADARG;
                rows.push_back(r);
            }
        }
    } catch (const std::bad_alloc &) {
        st = DMFTGPU_NOMEM;
    }
    if (std::ferror(f) != 0 && st == DMFTGPU_OK) st = DMFTGPU_IO;
    std::fclose(f);
    return st;
}

}  // namespace

extern "C" int dmftgpu_imgfreq_write(const char *path, int nfreq, int norbit, const double *f) {
    if (!path || nfreq < 1 || norbit < 1 || !f) return DMFTGPU_BADARG;
    FILE *out = std::fopen(path, "w");
    if (!out) return DMFTGPU_IO;
    const size_t NN = (size_t)norbit * norbit;
    auto at = [&](int w, int m, int n) { return f + 2 * ((size_t)w * NN + m + (size_t)n * norbit); };
    bool ok = true;
    for (int w = 0; w < nfreq && ok; w++)
        for (int m = 0; m < norbit && ok; m++)
            for (int n = 0; n < norbit && ok; n++) {
                const double *v = at(w, m, n);
                if (std::hypot(v[0], v[1]) > TOL) ok = std::fprintf(out, "%d %d %d %+0.8f %+0.8f\n", w, m, n, v[0], v[1]) > 0;
            }
    for (int m = 0; m < norbit && ok; m++)
        for (int n = 0; n < norbit && ok; n++)
            for (int k = 0; k < 5 && ok; k++) {
                const double *v = at(nfreq + k, m, n);
                ok = std::fprintf(out, "%d %d %d %+0.8f %+0.8f\n", -(k + 1), m, n, v[0], v[1]) > 0;
            }
    if (std::fclose(out) != 0) ok = false;
    return ok ? DMFTGPU_OK : DMFTGPU_IO;
}

extern "C" int dmftgpu_imgfreq_update(const char *path, int nfreq, int norbit, double *f) {
    if (!path || nfreq < 1 || norbit < 1 || !f) return DMFTGPU_BADARG;
    std::vector<Row> rows;
    const int st = read_rows(path, rows);
    if (st) return st;
    for (const Row &r : rows)  // the reference exits on an orbital index outside [0, N) (src/ImgTimeFtn.cpp:650)
        if (r.m < 0 || r.n < 0 || r.m >= norbit || r.n >= norbit) return DMFTGPU_BADARG;
    const size_t NN = (size_t)norbit * norbit;
    for (const Row &r : rows)
        if (r.w >= 0 && r.w < nfreq) {
            double *v = f + 2 * ((size_t)r.w * NN + r.m + (size_t)r.n * norbit);
            v[0] = r.re;
            v[1] = r.im;
        }
    return DMFTGPU_OK;
}

extern "C" int dmftgpu_imgfreq_read(const char *path, int nfreq, int norbit, double beta, double beta_prev,
                                    double *f) {
    if (!path || nfreq < 1 || norbit < 1 || !f || !(beta > 0) || !(beta_prev > 0)) return DMFTGPU_BADARG;
    std::vector<Row> rows;
    const int st = read_rows(path, rows);
    if (st) return st;
    int wmax = 0;
    for (const Row &r : rows) {
        if (r.w >= 0 && (r.m < 0 || r.n < 0 || r.m >= norbit || r.n >= norbit)) return DMFTGPU_BADARG;
        if (r.w > wmax) wmax = r.w;
    }
    wmax++;
    if (wmax < 2) return DMFTGPU_BADARG;  // the extrapolation below the grid needs two points
    const size_t NN = (size_t)norbit * norbit;
    // the file's points; as in the reference, a frequency with no line (every element <= 1e-7) keeps grid point 0
    std::vector<double> S, mats;
    try {
        S.assign(2 * (size_t)wmax * NN, 0.0);
        mats.assign(wmax, 0.0);
    } catch (const std::bad_alloc &) {
        return DMFTGPU_NOMEM;
    }
    for (const Row &r : rows)
        if (r.w >= 0) {
            mats[r.w] = (2 * r.w + 1) * M_PI / beta_prev;
            S[2 * ((size_t)r.w * NN + r.m + (size_t)r.n * norbit)] = r.re;
            S[2 * ((size_t)r.w * NN + r.m + (size_t)r.n * norbit) + 1] = r.im;
        }
    const double dw_prev = 2 * M_PI / beta_prev;
    auto s = [&](int w, size_t e, int c) { return S[2 * ((size_t)w * NN + e) + c]; };
    for (size_t i = 0; i < 2 * (size_t)(nfreq + 5) * NN; i++) f[i] = 0;
    int wp = 0;
    for (int w = 0; w < nfreq; w++) {
        const double x = (2 * w + 1) * M_PI / beta;
        double *o = f + 2 * (size_t)w * NN;
        if (x <= mats[0]) {
            for (size_t e = 0; e < NN; e++)
                for (int c = 0; c < 2; c++) o[2 * e + c] = (s(1, e, c) - s(0, e, c)) / dw_prev * (x - mats[0]) + s(0, e, c);
        } else if (x <= mats[wmax - 1]) {
            while (wp + 1 < wmax && !(mats[wp] < x && x <= mats[wp + 1])) wp++;
            if (wp + 1 >= wmax) return DMFTGPU_BADARG;  // no bracketing pair (the reference runs off its grid)
            for (size_t e = 0; e < NN; e++)
                for (int c = 0; c < 2; c++)
                    o[2 * e + c] = (s(wp + 1, e, c) - s(wp, e, c)) / dw_prev * (x - mats[wp]) + s(wp, e, c);
        } else {
            // R + w_last J / x with R = (F + F^H)/2 and J = (F - F^H)/(2i) of the last point; J enters without a
            // factor i, as in the reference (src/ImgTimeFtn.cpp:741-747)
            const int L = wmax - 1;
            for (int m = 0; m < norbit; m++)
                for (int n = 0; n < norbit; n++) {
                    const size_t e = m + (size_t)n * norbit, et = n + (size_t)m * norbit;
                    const double fr = s(L, e, 0), fi = s(L, e, 1), tr = s(L, et, 0), ti = -s(L, et, 1);  // F, F^H
                    const double Rr = (fr + tr) / 2, Ri = (fi + ti) / 2;
                    const double Dr = (fr - tr) / 2, Di = (fi - ti) / 2;  // (F - F^H)/2; J = that / i
                    const double Jr = Di, Ji = -Dr;
                    o[2 * e] = Rr + mats[L] * Jr / x;
                    o[2 * e + 1] = Ri + mats[L] * Ji / x;
                }
        }
    }
    return DMFTGPU_OK;
}
