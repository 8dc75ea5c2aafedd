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
//
// The kernels run on the context's stream.  Nothing orders that stream after
// the streams on which the caller wrote its inputs, so the caller completes
// that work before the call.  The five input pointers are checked with
// cudaPointerGetAttributes (which allocates nothing): host memory, or memory
// of another device, is refused with RT_EINVAL before any kernel runs.
#include "rt_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 8192;
static __device__ __align__(256) double g_rt_noalloc_scratch[3 * kMaxBlocks + 8];

// Device address of the scratch array on the context's device (current when
// this runs).  In host code the symbol's name is only a host-side stand-in;
// the address is resolved on the first call of each context and kept in it,
// so a context created after a device reset resolves it again.
rt::Error scratch_on_device(rt_ctx *ctx, double **out) {
    if (!ctx->noallocScratch) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_rt_noalloc_scratch);
        if (e != cudaSuccess)
            return rt::Error{RT_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)};
        ctx->noallocScratch = p;
    }
    *out = static_cast<double *>(ctx->noallocScratch);
    return rt::Error{RT_OK, ""};
}

// a caller's array must be device (or managed) memory of the context's device
rt::Error check_device_pointer(const rt_ctx *ctx, const void *p, const char *name) {
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return rt::Error{RT_EINVAL, std::string(name) + ": not a CUDA pointer (" + cudaGetErrorString(e) + ")"};
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
        return rt::Error{RT_EINVAL, std::string(name) + ": not device memory (host or unregistered pointer)"};
    if (at.device != ctx->device)
        return rt::Error{RT_EINVAL, std::string(name) + ": memory of device " + std::to_string(at.device) +
                                        ", the context is on device " + std::to_string(ctx->device)};
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
    if (N <= 0) {   // rt_mesh_upload refuses empty meshes; nothing to reduce
        *residual = 0.0;
        return RT_OK;
    }
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
    const void *args[5] = {diag, upper, lower, source, psi};
    const char *names[5] = {"diag", "upper", "lower", "source", "psi"};
    for (int i = 0; i < 5; ++i) {
        rt::Error pe = check_device_pointer(ctx, args[i], names[i]);
        if (pe.status != RT_OK) {
            ctx->lastError = "rt_residual_noalloc: " + pe.msg;
            return pe.status;
        }
    }
    double *scr = nullptr;
    rt::Error se = scratch_on_device(ctx, &scr);
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
