// context.cu -- context lifetime, workspaces, staging and error plumbing of the C ABI.
#include <cstdio>
#include <cstring>

#include "common.cuh"

static void dg_clear_events(dmftgpu_ctx *ctx) {
    for (auto &kv : ctx->events)
        for (auto &p : kv.second) {
            cudaEventDestroy(p.first);
            cudaEventDestroy(p.second);
        }
    ctx->events.clear();
}


int dg_set_cuda_error(dmftgpu_ctx *ctx, cudaError_t e, const char *what) {
    if (ctx) {
        ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
    }
    return (e == cudaErrorMemoryAllocation) ? DMFTGPU_NOMEM : DMFTGPU_CUDA_ERROR;
}

int dg_fail(dmftgpu_ctx *ctx, int code, const char *msg) {
    if (ctx) ctx->err = msg;
    return code;
}

void *dg_buf(dmftgpu_ctx *ctx, const char *name, size_t bytes) {
    if (bytes == 0) bytes = 16;
    auto &b = ctx->bufs[ctx->buf_ns.empty() ? std::string(name) : ctx->buf_ns + name];
    if (b.bytes < bytes && ctx->capturing) {
        dg_fail(ctx, DMFTGPU_BADARG, "workspace growth during graph capture");
        return nullptr;
    }
    if (b.bytes < bytes) {
        if (b.p) {
            cudaStreamSynchronize(ctx->stream);
            if (ctx->side) cudaStreamSynchronize(ctx->side);
            cudaFree(b.p);
            b.p = nullptr;
            b.bytes = 0;
        }
        size_t want = bytes + bytes / 8;
        cudaError_t e = cudaMalloc(&b.p, want);
        if (e != cudaSuccess) {
            dg_set_cuda_error(ctx, e, name);
            b.p = nullptr;
            return nullptr;
        }
        b.bytes = want;
    }
    return b.p;
}

int dg_launched(dmftgpu_ctx *ctx, const char *what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return dg_set_cuda_error(ctx, e, what);
    return DMFTGPU_OK;
}

int dg_status_reset(dmftgpu_ctx *ctx) {
    DG_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
    return DMFTGPU_OK;
}

int dg_status_read(dmftgpu_ctx *ctx, int *code) {
    int h = 0;
    DG_CUDA(cudaMemcpyAsync(&h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    *code = h;
    return DMFTGPU_OK;
}

const void *dg_in(dmftgpu_ctx *ctx, const void *p, size_t bytes, int flags, const char *name, int *st) {
    *st = DMFTGPU_OK;
    if (!p) return nullptr;
    if (flags & DMFTGPU_DEVICE_PTRS) return p;
    void *d = dg_buf(ctx, name, bytes);
    if (!d) {
        *st = DMFTGPU_NOMEM;
        return nullptr;
    }
    cudaError_t e = cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        *st = dg_set_cuda_error(ctx, e, name);
        return nullptr;
    }
    return d;
}

void *dg_out(dmftgpu_ctx *ctx, void *p, size_t bytes, int flags, const char *name, int *st) {
    *st = DMFTGPU_OK;
    if (!p) return nullptr;
    if (flags & DMFTGPU_DEVICE_PTRS) return p;
    void *d = dg_buf(ctx, name, bytes);
    if (!d) *st = DMFTGPU_NOMEM;
    return d;
}

int dg_out_done(dmftgpu_ctx *ctx, void *host, const void *dev, size_t bytes, int flags) {
    if (!host || (flags & DMFTGPU_DEVICE_PTRS)) return DMFTGPU_OK;
    DG_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return DMFTGPU_OK;
}

extern "C" {

int dmftgpu_version(void) { return 1; }

int dmftgpu_create(dmftgpu_ctx **out, int device) {
    if (!out) return DMFTGPU_BADARG;
    *out = nullptr;
    dmftgpu_ctx *ctx = new dmftgpu_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        int code = dg_set_cuda_error(ctx, e, "dmftgpu_create");
        // release whatever was created before the failing call
        if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
        if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
        if (ctx->side) cudaStreamDestroy(ctx->side);
        if (ctx->d_status) cudaFree(ctx->d_status);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return code;
    }
    ctx->own_stream = true;
    cudaMemset(ctx->d_status, 0, sizeof(int));
    *out = ctx;
    return DMFTGPU_OK;
}

int dmftgpu_destroy(dmftgpu_ctx *ctx) {
    if (!ctx) return DMFTGPU_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    dg_clear_events(ctx);
    delete ctx->pulay;
    for (auto &kv : ctx->bufs)
        if (kv.second.p) cudaFree(kv.second.p);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    for (auto &l : ctx->lanes) {
        if (l.stream) {
            cudaStreamSynchronize(l.stream);
            cudaStreamDestroy(l.stream);
        }
        if (l.side) {
            cudaStreamSynchronize(l.side);
            cudaStreamDestroy(l.side);
        }
        if (l.fork) cudaEventDestroy(l.fork);
        if (l.join) cudaEventDestroy(l.join);
        if (l.done) cudaEventDestroy(l.done);
    }
    if (ctx->ev_batch) cudaEventDestroy(ctx->ev_batch);
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return DMFTGPU_OK;
}

int dmftgpu_set_stream(dmftgpu_ctx *ctx, void *stream) {
    if (!ctx) return DMFTGPU_BADARG;
    if (ctx->own_stream && ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    ctx->stream = (cudaStream_t)stream;
    ctx->own_stream = false;
    return DMFTGPU_OK;
}

void *dmftgpu_get_stream(dmftgpu_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int dmftgpu_synchronize(dmftgpu_ctx *ctx) {
    if (!ctx) return DMFTGPU_BADARG;
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    return DMFTGPU_OK;
}

const char *dmftgpu_last_error(dmftgpu_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

long long dmftgpu_launch_count(dmftgpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

int dmftgpu_timing(dmftgpu_ctx *ctx, int enable) {
    if (!ctx) return DMFTGPU_BADARG;
    cudaStreamSynchronize(ctx->stream);
    dg_clear_events(ctx);
    ctx->timing = enable != 0;
    return DMFTGPU_OK;
}

int dmftgpu_kernel_time(dmftgpu_ctx *ctx, const char *kernel, double *ms, int *count) {
    if (!ctx || !kernel || !ms) return DMFTGPU_BADARG;
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
    double tot = 0;
    int cnt = 0;
    auto it = ctx->events.find(kernel);
    if (it != ctx->events.end())
        for (auto &p : it->second) {
            float t = 0;
            DG_CUDA(cudaEventElapsedTime(&t, p.first, p.second));
            tot += t;
            cnt++;
        }
    *ms = tot;
    if (count) *count = cnt;
    return DMFTGPU_OK;
}

int dmftgpu_kmesh(int kx, int ky, int kz, double *kmesh) {
    // src/TB.cpp:196-207 with ax = ay = az = pi (src/dmft_common.h:37-39)
    if (kx <= 0 || ky <= 0 || kz <= 0 || !kmesh) return DMFTGPU_BADARG;
    const double ax = DG_PI, ay = DG_PI, az = DG_PI;
    const int kpxy = kx * ky, nk = kx * ky * kz;
    const double delx = 2. * DG_PI / (ax * double(kx)), dely = 2. * DG_PI / (ay * double(ky)),
                 delz = 2. * DG_PI / (az * double(kz));
    for (int k = 0; k < nk; k++) {
        kmesh[3 * k + 0] = -DG_PI / ax + delx / 2. + (k % kx) * delx;
        kmesh[3 * k + 1] = -DG_PI / ay + dely / 2. + ((k % kpxy) / kx) * dely;
        kmesh[3 * k + 2] = -DG_PI / az + delz / 2. + (k / kpxy) * delz;
    }
    return DMFTGPU_OK;
}

}  // extern "C"
