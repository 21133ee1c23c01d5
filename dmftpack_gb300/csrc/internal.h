// internal.h -- host-side context of libdmftgpu shared by the translation units.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "dmftgpu.h"

// DMFT-level Pulay mixer state (pulayMixing(2, 5, ...), src/pulay.cpp:11-46): history on the device, the
// (hist+1) x (hist+1) DIIS matrix on the host
struct DgPulay {
    int hist = 2, start = 5;
    long long len = 0;
    std::vector<double> om;
};

struct dmftgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    long long launches = 0;
    struct Buf {
        void *p = nullptr;
        size_t bytes = 0;
    };
    std::map<std::string, Buf> bufs;  // grow-only named device workspaces
    int *d_status = nullptr;          // device status word (max of kernel-reported codes)
    cudaStream_t side = nullptr;      // side stream for work that overlaps the main stream's kernels
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    DgPulay *pulay = nullptr;         // mixer state of dmftgpu_dmft_iteration
    double scgf_prev_norm = 0.0;      // mixing_check_outer's previous residual (a function static in the
                                      // reference, src/SCGF2_fullLoop.cpp:722-727): kept across SCGF2 calls
    bool ft_direct = false;           // DMFTGPU_DIRECT_DFT of the current call
    bool imp_mixed = false;           // DMFTGPU_MIXED of the current call, for the impurity kernels
    bool timing = false;              // record CUDA events around the named hot kernels
    std::string buf_ns;               // workspace namespace (one per problem of a batched call)
    bool autotune = false;            // time the CTA-per-SM candidates of each Schur kernel on first use
    bool capturing = false;           // a CUDA graph capture is in progress (no syncs, no tuning)
    std::map<std::string, int> tuned; // kernel key -> chosen CTAs per SM
    struct Lane {
        cudaStream_t stream = nullptr, side = nullptr;
        cudaEvent_t fork = nullptr, join = nullptr, done = nullptr;
    };
    std::vector<Lane> lanes;          // stream pairs of batched calls
    cudaEvent_t ev_batch = nullptr;
    cudaStream_t cap_stream = nullptr;  // batched graphs are captured here (the caller's stream may be legacy)
    cudaGraphExec_t graph = nullptr;  // the last captured batched pass
    std::string graph_key;
    std::map<std::string, std::vector<std::pair<cudaEvent_t, cudaEvent_t>>> events;
    std::string hk_phase_key;         // (k mesh, R list) of the phase-slice image in workspace "hk.tc.A"
    bool tensor = true;               // tensor-core contractions allowed in the mixed form (!DMFTGPU_NO_TENSOR)
    int nk_krylov = 0;                // Jacobian-vector products of the last Newton-Krylov mixer step (0: none)
    double nk_relres = 0.0;           // its linear solve's relative residual
    double mix_resid = 0.0;           // |SE_out - SelfEnergy_w| / |SelfEnergy_w| of the last DMFT iteration
};

// sets ctx->tensor from a call's flags for the call's duration
struct DgTensorMode {
    dmftgpu_ctx *ctx;
    bool saved;
    DgTensorMode(dmftgpu_ctx *c, int flags) : ctx(c), saved(c->tensor) { ctx->tensor = !(flags & DMFTGPU_NO_TENSOR); }
    ~DgTensorMode() { ctx->tensor = saved; }
};

// sets ctx->ft_direct and ctx->imp_mixed from a call's flags for the call's duration
struct DgFtMode {
    dmftgpu_ctx *ctx;
    bool saved, saved_mixed;
    DgFtMode(dmftgpu_ctx *c, int flags) : ctx(c), saved(c->ft_direct), saved_mixed(c->imp_mixed) {
        ctx->ft_direct = (flags & DMFTGPU_DIRECT_DFT) != 0;
        ctx->imp_mixed = (flags & DMFTGPU_MIXED) != 0;
    }
    ~DgFtMode() {
        ctx->ft_direct = saved;
        ctx->imp_mixed = saved_mixed;
    }
};

// event pair around one launch of `name` when ctx->timing is on (no-op otherwise)
struct DgTimer {
    dmftgpu_ctx *ctx;
    cudaEvent_t b = nullptr, e = nullptr;
    const char *name;
    DgTimer(dmftgpu_ctx *c, const char *n) : ctx(c), name(n) {
        if (ctx->timing) {
            cudaEventCreate(&b);
            cudaEventCreate(&e);
            cudaEventRecord(b, ctx->stream);
        }
    }
    ~DgTimer() {
        if (ctx->timing) {
            cudaEventRecord(e, ctx->stream);
            ctx->events[name].push_back({b, e});
        }
    }
};

int dg_set_cuda_error(dmftgpu_ctx *ctx, cudaError_t e, const char *what);
int dg_fail(dmftgpu_ctx *ctx, int code, const char *msg);
// device workspace `name` of at least `bytes` (contents undefined); nullptr + error text on failure
void *dg_buf(dmftgpu_ctx *ctx, const char *name, size_t bytes);
// checks the last launch, counts it
int dg_launched(dmftgpu_ctx *ctx, const char *what);
// zero the status word, read it back (synchronising the stream)
int dg_status_reset(dmftgpu_ctx *ctx);
int dg_status_read(dmftgpu_ctx *ctx, int *code);

// stage a caller array on the device: returns the caller's pointer if it is already a device pointer
// (flags & DMFTGPU_DEVICE_PTRS), else copies `bytes` into workspace `name`.
const void *dg_in(dmftgpu_ctx *ctx, const void *p, size_t bytes, int flags, const char *name, int *st);
// output staging: device pointer to write into, and the copy-back afterwards
void *dg_out(dmftgpu_ctx *ctx, void *p, size_t bytes, int flags, const char *name, int *st);
int dg_out_done(dmftgpu_ctx *ctx, void *host, const void *dev, size_t bytes, int flags);

// internal device-to-device entry points (all pointers device, enqueue only)
int dg_moments_dev(dmftgpu_ctx *ctx, int dim, int nfreq, double beta, const double2 *fw, int green,
                   double2 *mom);
// Pulay mixing (mixing.cu): on return `out` holds the mixed input for the next iteration; `tag` names the
// history workspaces of this mixer instance
int dg_pulay_mixing(dmftgpu_ctx *ctx, DgPulay &P, const char *tag, long long len, double2 *in, double2 *out,
                    double mixing, int it);

// H(k) on the tensor cores (hk_tc.cu); all pointers device
int dg_hk_tensor(dmftgpu_ctx *ctx, int n, int nR, const int *dR, const double2 *dT, int kx, int ky, int kz,
                 double2 *dH, const std::string &mesh_key);

// Newton-Krylov support (nk.cu): real inner product of complex device vectors (a synchronous fixed-order
// reduction), y = a x + b y, and GMRES with at most m Arnoldi vectors on `apply` (x = the solution of
// apply(x) = b, *relres = |b - apply(x)| / |b| of the Arnoldi least-squares problem)
int dg_vdot(dmftgpu_ctx *ctx, long long n, const double2 *a, const double2 *b, double *out);
int dg_vaxpby(dmftgpu_ctx *ctx, long long n, double a, const double2 *x, double b, double2 *y);
int dg_gmres(dmftgpu_ctx *ctx, long long n, const double2 *b, int m, double tol,
             const std::function<int(const double2 *, double2 *)> &apply, double2 *x, int *iters, double *relres);

#define DG_LAUNCH(ctx, what)                     \
    do {                                         \
        int s_ = dg_launched((ctx), (what));     \
        if (s_) return s_;                       \
    } while (0)
#define DG_TRY(expr)          \
    do {                      \
        int s_ = (expr);      \
        if (s_) return s_;    \
    } while (0)
