// noalloc.cu — the OpenFOAM-normalised residual of one LDU system, computed
// without allocating anything.
//
// Some callers cannot allocate device memory at the point where they need a
// residual: a solver callback running inside another library's Krylov loop
// (PETSc / Hypre style), where a cudaMalloc would synchronise the device in the
// middle of that loop, or an embedded host that has handed all device memory
// to a pool it manages.  rt_residual (ctx.cu) copies host arrays into freshly allocated
// device buffers; rt_residual_noalloc takes device pointers and keeps its
// reduction scratch in the file-scope array below, so it calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// The scratch holds one partial sum per thread block of each of three
// reductions (sum of psi; normalisation sum; sum of |b - A psi|) plus the
// reduced values: kMaxBlocks blocks of 256 cells, so meshes of up to
// kMaxBlocks * 256 = 2,097,152 cells (3 * 8192 + 8 doubles, 192 KiB).  Larger
// meshes are rejected with RT_EINVAL.  The array lives in every GPU that loads
// the library until the process exits.  Every call overwrites every partial it
// reads, so nothing has to be cleared between calls; but all calls share the
// one array, so calls that overlap on the GPU (two host threads, two streams)
// race and must be serialised by the caller.
#include <mutex>

#include "rt_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 8192;
constexpr int kMaxDevices = 128;

static __device__ __align__(256) double g_rt_noalloc_scratch[3 * kMaxBlocks + 8];

std::mutex g_mutex;
double *g_scratch[kMaxDevices] = {};

// device address of the scratch array on the current device (first call per
// device resolves it; the symbol name in host code is only a host stand-in)
rt::Error scratch_on_device(int device, double **out) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (device < 0 || device >= kMaxDevices) return rt::Error{RT_EINVAL, "device index out of range"};
    if (!g_scratch[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_rt_noalloc_scratch);
        if (e != cudaSuccess)
            return rt::Error{RT_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)};
        g_scratch[device] = static_cast<double *>(p);
    }
    *out = g_scratch[device];
    return rt::Error{RT_OK, ""};
}

__device__ __forceinline__ double na_block_sum(double v) {
    __shared__ double sh[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kThreads / 32; ++i) s += sh[i];
    return s;
}

struct NaMesh {
    int N, nSlots;
    const int *__restrict__ face;
    const int *__restrict__ nbr;
};

// partial sums of psi, one per block
__global__ void k_na_sum(NaMesh m, const double *__restrict__ psi, double *part) {
    int c = blockIdx.x * kThreads + threadIdx.x;
    double v = c < m.N ? psi[c] : 0.0;
    double s = na_block_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// fixed-order sum of nb partials into *out (one block)
__global__ void k_na_reduce(int nb, const double *part, double *out) {
    double v = 0.0;
    for (int i = threadIdx.x; i < nb; i += kThreads) v += part[i];
    double s = na_block_sum(v);
    if (threadIdx.x == 0) *out = s;
}

// per block: sum(|A psi - xbar A1| + |b - xbar A1|) and sum(|b - A psi|)
__global__ void k_na_res(NaMesh m, const double *__restrict__ diag, const double *__restrict__ upper,
                         const double *__restrict__ lower, const double *__restrict__ b,
                         const double *__restrict__ psi, const double *psiSum, double *partNorm,
                         double *partRes) {
    int c = blockIdx.x * kThreads + threadIdx.x;
    double vn = 0.0, vr = 0.0;
    if (c < m.N) {
        const double xbar = *psiSum / m.N;
        double ax = diag[c] * psi[c], sa = diag[c];
        for (int s = 0; s < m.nSlots; ++s) {
            int nb = m.nbr[s * m.N + c];
            if (nb < 0) break;
            int f = m.face[s * m.N + c];
            double a = nb > c ? upper[f] : lower[f];
            ax += a * psi[nb];
            sa += a;
        }
        sa *= xbar;
        double bb = b[c];
        vn = fabs(ax - sa) + fabs(bb - sa);
        vr = fabs(bb - ax);
    }
    double sn = na_block_sum(vn);
    __syncthreads();
    double sr = na_block_sum(vr);
    if (threadIdx.x == 0) {
        partNorm[blockIdx.x] = sn;
        partRes[blockIdx.x] = sr;
    }
}

// residual = sum|b - A psi| / (normalisation + 1e-20)
__global__ void k_na_finish(int nb, const double *partNorm, const double *partRes, double *out) {
    double vn = 0.0, vr = 0.0;
    for (int i = threadIdx.x; i < nb; i += kThreads) {
        vn += partNorm[i];
        vr += partRes[i];
    }
    double sn = na_block_sum(vn);
    __syncthreads();
    double sr = na_block_sum(vr);
    if (threadIdx.x == 0) out[0] = sr / (sn + 1e-20);
}

}  // namespace

extern "C" rt_status rt_residual_noalloc(rt_ctx *ctx, const double *diag, const double *upper,
                                         const double *lower, const double *source, const double *psi,
                                         double *residual) {
    if (!ctx) return RT_EINVAL;
    if (!ctx->meshReady) {
        ctx->lastError = "rt_residual_noalloc: mesh not uploaded";
        return RT_ENOTREADY;
    }
    if (!diag || !upper || !lower || !source || !psi || !residual) {
        ctx->lastError = "rt_residual_noalloc: null argument";
        return RT_EINVAL;
    }
    const int N = ctx->mesh.N;
    const int nb = (N + kThreads - 1) / kThreads;
    if (nb > kMaxBlocks) {
        ctx->lastError = "rt_residual_noalloc: " + std::to_string(N) + " cells exceed the maximum of " +
                         std::to_string(kMaxBlocks * kThreads) + " (static scratch of " +
                         std::to_string(kMaxBlocks) + " blocks)";
        return RT_EINVAL;
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
        ctx->lastError = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return RT_ECUDA;
    }
    double *scr = nullptr;
    rt::Error se = scratch_on_device(ctx->device, &scr);
    if (se.status != RT_OK) {
        ctx->lastError = "rt_residual_noalloc: " + se.msg;
        return se.status;
    }
    double *partA = scr, *partB = scr + kMaxBlocks, *partC = scr + 2 * kMaxBlocks;
    double *vals = scr + 3 * kMaxBlocks;   // [0] sum psi, [1] residual
    NaMesh m{N, ctx->mesh.nSlots, ctx->mesh.ellFace.p, ctx->mesh.ellNbr.p};
    cudaStream_t s = ctx->stream;
    k_na_sum<<<nb, kThreads, 0, s>>>(m, psi, partA);
    k_na_reduce<<<1, kThreads, 0, s>>>(nb, partA, vals);
    k_na_res<<<nb, kThreads, 0, s>>>(m, diag, upper, lower, source, psi, vals, partB, partC);
    k_na_finish<<<1, kThreads, 0, s>>>(nb, partB, partC, vals + 1);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(residual, vals + 1, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        ctx->lastError = std::string("rt_residual_noalloc: ") + cudaGetErrorString(e);
        return RT_ECUDA;
    }
    ctx->kernelLaunches += 4;
    return RT_OK;
}
