// noalloc.cu -- dmftgpu_hyb_delta_noalloc: the hybridisation function with no device allocation at all.
//
// Who needs it: callers that must not call cudaMalloc -- e.g. a DMFT driver whose device memory is owned
// by a pool allocator (a PyTorch caching allocator, or an MPI application that reserves all HBM up front),
// or one that runs between stream-ordered work where cudaMalloc, which is not stream-ordered, could stall
// every stream on the device.  Such a caller passes device pointers for every input and output; the only
// scratch (one n_c x n_c matrix per Matsubara frequency for the inversion of the projected G_loc) lives in
// the file-scope array below, which every GPU that loads the library holds until the process exits.
//
// Limits and sharing: nfreq * dim * dim <= DG_NOALLOC_HYB_MAX complex numbers (8 MiB) and dim <= 32;
// larger requests are rejected with DMFTGPU_BADARG.  All calls share the one array, so calls that overlap
// on the GPU (different streams, or several host threads at once) race on it; serialise them.  The first
// call on each device resolves the device address of the array (cudaGetSymbolAddress).  No call may be made
// on a stream under capture: each one reads its status back and waits for the stream.  The arrays belong to the device that is current when the call is made,
// and cuda_stream must belong to that device too (else DMFTGPU_BADARG).  Every call is synchronous: it
// reads the status word back and waits for cuda_stream to finish before it returns.
#include <mutex>

#include "linalg.cuh"

#define DG_NOALLOC_HYB_MAX (1 << 19)  // complex numbers: 8 MiB
#define DG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double2 g_hyb_scratch[DG_NOALLOC_HYB_MAX];
static __device__ __align__(256) int g_hyb_status[1];

namespace {

struct OrbTable {
    int orb[32];
};

struct DevSymbols {
    double2 *scratch = nullptr;
    int *status = nullptr;
    bool ready = false;
};
DevSymbols g_sym[DG_NOALLOC_MAX_DEVICES];
std::mutex g_sym_mutex;

// the same arithmetic as dmftgpu_hyb_delta (src/Construct_hyb_delta.cpp:98-113), one thread per frequency,
// the pivot table in registers/local memory and the matrix in the static scratch
__global__ void k_hyb_delta_static(int dim, int nfreq, int D, double beta, double mu, OrbTable ot,
                                   const double2 *__restrict__ S, const double2 *__restrict__ G,
                                   const double2 *__restrict__ Himp, double2 *scratch, double2 *delta, int *status) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nfreq) return;
    const size_t DD = (size_t)D * D, dd = (size_t)dim * dim;
    double2 *g = scratch + (size_t)n * dd;
    int perm[32];
    for (int h2 = 0; h2 < dim; h2++)
        for (int h1 = 0; h1 < dim; h1++) DG_AT(g, dim, h1, h2) = G[n * DD + ot.orb[h1] + (size_t)ot.orb[h2] * D];
    if (thread_gj_inverse(dim, g, perm)) atomicMax(status, (int)DG_SINGULAR);
    const double2 iw = cmk(0.0, DG_PI * (2. * n + 1.) / beta);
    double2 *out = delta + (size_t)n * dd;
    for (int h1 = 0; h1 < dim; h1++) {
        for (int h2 = 0; h2 < dim; h2++) {
            double2 hs = Himp[ot.orb[h1] + (size_t)ot.orb[h2] * D], ss = S[n * DD + ot.orb[h1] + (size_t)ot.orb[h2] * D];
            DG_AT(out, dim, h1, h2) = csub(csub(cneg(hs), ss), DG_AT(g, dim, h1, h2));
        }
        double2 v = DG_AT(out, dim, h1, h1);
        v = cadd(v, iw);
        v.x += mu;
        DG_AT(out, dim, h1, h1) = v;
    }
}

int resolve_symbols(int dev, DevSymbols *&out) {
    if (dev < 0 || dev >= DG_NOALLOC_MAX_DEVICES) return DMFTGPU_BADARG;
    std::lock_guard<std::mutex> lk(g_sym_mutex);
    DevSymbols &d = g_sym[dev];
    if (!d.ready) {
        // host code must not use the arrays' names as addresses: ask the runtime for this device's copies
        if (cudaGetSymbolAddress((void **)&d.scratch, g_hyb_scratch) != cudaSuccess) return DMFTGPU_CUDA_ERROR;
        if (cudaGetSymbolAddress((void **)&d.status, g_hyb_status) != cudaSuccess) return DMFTGPU_CUDA_ERROR;
        d.ready = true;
    }
    out = &d;
    return DMFTGPU_OK;
}

}  // namespace

extern "C" int dmftgpu_hyb_delta_noalloc(int dim, const int *orb, int nfreq, double beta, int D, const double *sigma,
                                         const double *gw, const double *himp, double mu, double *delta,
                                         void *cuda_stream) {
    if (dim < 1 || dim > 32 || !orb || nfreq < 1 || D < 1 || !sigma || !gw || !himp || !delta || !(beta > 0))
        return DMFTGPU_BADARG;
    if ((long long)nfreq * dim * dim > DG_NOALLOC_HYB_MAX) return DMFTGPU_BADARG;  // beyond the static scratch
    OrbTable ot;
    for (int i = 0; i < 32; i++) ot.orb[i] = 0;
    for (int i = 0; i < dim; i++) {
        if (orb[i] < 0 || orb[i] >= D) return DMFTGPU_BADARG;
        ot.orb[i] = orb[i];
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DMFTGPU_CUDA_ERROR;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    if (s) {
        // the scratch address resolved below belongs to the current device: a stream created on another
        // device would run the kernel against the wrong device's array, so such a stream is rejected
        int sdev = -1;
        if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) return DMFTGPU_BADARG;
        if (sdev != dev) return DMFTGPU_BADARG;
    }
    DevSymbols *sym = nullptr;
    int st = resolve_symbols(dev, sym);
    if (st) return st;
    if (cudaMemsetAsync(sym->status, 0, sizeof(int), s) != cudaSuccess) return DMFTGPU_CUDA_ERROR;
    k_hyb_delta_static<<<(nfreq + 127) / 128, 128, 0, s>>>(dim, nfreq, D, beta, mu, ot, (const double2 *)sigma,
                                                           (const double2 *)gw, (const double2 *)himp, sym->scratch,
                                                           (double2 *)delta, sym->status);
    if (cudaGetLastError() != cudaSuccess) return DMFTGPU_CUDA_ERROR;
    int code = 0;
    if (cudaMemcpyAsync(&code, sym->status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return DMFTGPU_CUDA_ERROR;
    if (cudaStreamSynchronize(s) != cudaSuccess) return DMFTGPU_CUDA_ERROR;
    return code;
}
