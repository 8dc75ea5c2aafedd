// sweep.cu — systolic triangular sweeps of DIC / DILU on structured meshes.
//
// A structured mesh is the active-cell subset of an nx x ny x nz box numbered
// lexicographically (i fastest), as blockMesh numbers a block.  Its lower
// neighbours are (i,j,k-1), (i,j-1,k), (i-1,j,k) in increasing face order, its
// upper neighbours (i+1,j,k), (i,j+1,k), (i,j,k+1).  The sequential D-ILU
// recurrences of OpenFOAM (rD, forward, backward; face-ordered accumulation)
// are evaluated here in exactly that order of operations, so the result equals
// the level-scheduled sweep (and the sequential one up to FMA contraction).
//
// Work decomposition: rows (j,k) are grouped in blocks of 32 consecutive j in
// one plane k.  A warp owns a block; at step t lane l updates cell i = t - l of
// row j = 32 jb + l.  The i-1 value is the lane's own previous result
// (register), the j-1 value is lane l-1's previous result (shuffle), lane 0
// reads it from the block below in j, and the k-1 value comes from the block
// of the previous plane; those two come through global memory behind
// per-block progress counters.  Blocks are claimed in dependency order through
// an atomic counter, so a warp only ever waits for a block that a running warp
// owns: no deadlock.  Every wait is bounded; a timeout sets an error flag,
// marks the block finished and the host reports RT_ETIMEOUT.
//
// Per-entry data live in a "skewed" layout, entry (block, step, lane), so the
// 32 lanes of a step touch 32 consecutive doubles.  The backward sweep walks
// the same layout in reverse (lanes mirrored).
#include <cuda/atomic>

#include "rt_internal.h"
#include "sweep.h"

namespace rt {

namespace {

__device__ __forceinline__ int load_acquire(const int *p) {
    cuda::atomic_ref<int, cuda::thread_scope_device> a(*const_cast<int *>(p));
    return a.load(cuda::memory_order_acquire);
}
__device__ __forceinline__ void store_release(int *p, int v) {
    cuda::atomic_ref<int, cuda::thread_scope_device> a(*p);
    a.store(v, cuda::memory_order_release);
}

// lane 0 waits until prog[dep] >= need (bounded); returns false on timeout
__device__ __forceinline__ bool wait_progress(int *sync, int dep, int need, int *seen, long long maxSpin) {
    bool ok = true;
    if ((threadIdx.x & 31) == 0) {
        int v = *seen;
        long long spins = 0;
        while (v < need) {
            v = load_acquire(sync + SYNC_PROGRESS + dep);
            if (v >= need) break;
            if (load_acquire(sync + SYNC_ERROR) != 0 || ++spins > maxSpin) {
                atomicExch(sync + SYNC_ERROR, 1);
                ok = false;
                break;
            }
            if (spins > 64) __nanosleep(64);
        }
        *seen = v;
    }
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    __threadfence();
    return ok;
}

__device__ __forceinline__ void publish(int *sync, int blk, int steps) {
    __threadfence();
    __syncwarp();
    if ((threadIdx.x & 31) == 0) store_release(sync + SYNC_PROGRESS + blk, steps);
}

constexpr int PUB = 4;   // steps between progress publications

}  // namespace

// MODE 0: forward application, 1: backward application, 2: rD recurrence
template <int MODE, int NC>
__global__ void k_systolic(SkewView g, unsigned mask, const double *__restrict__ r, double *__restrict__ w,
                           int N, int *sync, long long maxSpin) {
    const int lane = threadIdx.x & 31;
    const int nBlk = g.nz * g.nJB;
    const long long BS = (long long)g.T * 32;
    while (true) {
        int b = 0;
        if (lane == 0) b = atomicAdd(sync + SYNC_WORK, 1);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= nBlk) return;
        const int blk = (MODE == 1) ? nBlk - 1 - b : b;
        const int k = blk / g.nJB, jb = blk % g.nJB;
        int depK, depJ;
        if (MODE == 1) {
            depK = (k + 1 < g.nz) ? blk + g.nJB : -1;
            depJ = (jb + 1 < g.nJB) ? blk + 1 : -1;
        } else {
            depK = (k > 0) ? blk - g.nJB : -1;
            depJ = (jb > 0) ? blk - 1 : -1;
        }
        int seenK = 0, seenJ = 0;
        bool alive = load_acquire(sync + SYNC_ERROR) == 0;
        double yprev[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) yprev[q] = (MODE == 2) ? 1.0 : 0.0;
        for (int t = 0; t < g.T && alive; ++t) {
            // dependencies of this step: depK at the same step, depJ at t + 31
            if (depK >= 0 && (seenK < t + 1)) {
                int need = min(g.T, ((t + 1 + PUB - 1) / PUB) * PUB);
                alive = wait_progress(sync, depK, need, &seenK, maxSpin);
                seenK = __shfl_sync(0xffffffffu, seenK, 0);
                if (!alive) break;
            }
            if (depJ >= 0 && (seenJ < t + 32)) {
                int need = min(g.T, ((t + 32 + PUB - 1) / PUB) * PUB);
                alive = wait_progress(sync, depJ, need, &seenJ, maxSpin);
                seenJ = __shfl_sync(0xffffffffu, seenJ, 0);
                if (!alive) break;
            }
            const long long e = (MODE == 1) ? (long long)blk * BS + (long long)(g.T - 1 - t) * 32 + (31 - lane)
                                            : (long long)blk * BS + (long long)t * 32 + lane;
            const long long eK = (MODE == 1) ? e + (long long)g.nJB * BS : e - (long long)g.nJB * BS;
            long long eJ = 0;
            if (MODE == 1)
                eJ = (long long)(blk + 1) * BS + (long long)(g.T - 1 - (t + 31)) * 32 + 0;
            else
                eJ = (long long)(blk - 1) * BS + (long long)(t + 31) * 32 + 31;
            const int cell = g.cellOf[e];
            double yup[NC];
#pragma unroll
            for (int q = 0; q < NC; ++q) yup[q] = __shfl_up_sync(0xffffffffu, yprev[q], 1);
            if (MODE == 2) {
                double v = 1.0;
                if (cell >= 0) {
                    v = g.D[e];
                    if (depK >= 0) v -= g.Pz[e] / g.rDraw[eK];
                    double yj = (lane > 0) ? yup[0] : (depJ >= 0 && t + 31 < g.T ? g.rDraw[eJ] : 1.0);
                    v -= g.Py[e] / yj;
                    v -= g.Px[e] / yprev[0];
                }
                g.rDraw[e] = v;
                yprev[0] = v;
            } else {
                const double cz = (MODE == 0) ? g.Az[e] : g.Bz[e];
                const double cy = (MODE == 0) ? g.Ay[e] : g.By[e];
                const double cx = (MODE == 0) ? g.Ax[e] : g.Bx[e];
                const double rd = g.rDinv[e];
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    if (!((mask >> q) & 1u)) continue;
                    double *wS = g.wS + (long long)q * g.nSkew;
                    double acc = 0.0;
                    if (cell >= 0) {
                        acc = (MODE == 0) ? rd * r[(long long)q * N + cell] : wS[e];
                        if (depK >= 0) acc -= cz * wS[eK];
                        double yj = (lane > 0) ? yup[q] : (depJ >= 0 && t + 31 < g.T ? wS[eJ] : 0.0);
                        acc -= cy * yj;
                        acc -= cx * yprev[q];
                        if (MODE == 1) w[(long long)q * N + cell] = acc;
                    }
                    wS[e] = acc;
                    yprev[q] = acc;
                }
            }
            if (((t + 1) % PUB) == 0 || t + 1 == g.T) publish(sync, blk, t + 1);
        }
        if (!alive) {
            // let dependants finish quickly; the host reports the timeout
            publish(sync, blk, g.T);
        }
    }
}

// gather the skewed per-entry coefficients of one matrix
__global__ void k_skew_setup(SkewView g, const int *__restrict__ faceLo, const int *__restrict__ faceHi, int N,
                             const double *__restrict__ diag, const double *__restrict__ upper,
                             const double *__restrict__ lower) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    int c = g.cellOf[e];
    double d = 1.0, pz = 0.0, py = 0.0, px = 0.0;
    if (c >= 0) {
        d = diag[c];
        int fz = faceLo[c], fy = faceLo[N + c], fx = faceLo[2 * N + c];
        if (fz >= 0) pz = upper[fz] * lower[fz];
        if (fy >= 0) py = upper[fy] * lower[fy];
        if (fx >= 0) px = upper[fx] * lower[fx];
    }
    g.D[e] = d;
    g.Pz[e] = pz;
    g.Py[e] = py;
    g.Px[e] = px;
}

// rD -> 1/rD and the premultiplied sweep coefficients rD_c a_cf
__global__ void k_skew_premul(SkewView g, const int *__restrict__ faceLo, const int *__restrict__ faceHi, int N,
                              const double *__restrict__ upper, const double *__restrict__ lower) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    int c = g.cellOf[e];
    double rd = 0.0, az = 0.0, ay = 0.0, ax = 0.0, bz = 0.0, by = 0.0, bx = 0.0;
    if (c >= 0) {
        rd = 1.0 / g.rDraw[e];
        int fz = faceLo[c], fy = faceLo[N + c], fx = faceLo[2 * N + c];
        int gz = faceHi[c], gy = faceHi[N + c], gx = faceHi[2 * N + c];
        if (fz >= 0) az = rd * lower[fz];
        if (fy >= 0) ay = rd * lower[fy];
        if (fx >= 0) ax = rd * lower[fx];
        if (gz >= 0) bz = rd * upper[gz];
        if (gy >= 0) by = rd * upper[gy];
        if (gx >= 0) bx = rd * upper[gx];
    }
    g.rDinv[e] = rd;
    g.Az[e] = az; g.Ay[e] = ay; g.Ax[e] = ax;
    g.Bz[e] = bz; g.By[e] = by; g.Bx[e] = bx;
}

namespace {

int systolic_grid(rt_ctx *ctx, const SkewView &g) {
    int warps = g.nz * g.nJB;
    int perBlock = 4;   // warps per CTA
    return std::max(1, (warps + perBlock - 1) / perBlock);
}

void reset_sync(rt_ctx *ctx, const SkewView &g) {
    StructMesh &s = ctx->mesh.sm;
    RT_CUDA(cudaMemsetAsync(s.sync.p, 0, sizeof(int) * (SYNC_PROGRESS + g.nz * g.nJB), ctx->stream));
}

template <int MODE>
void launch_mode(rt_ctx *ctx, const SkewView &g, int nc, unsigned mask, const double *r, double *w) {
    StructMesh &s = ctx->mesh.sm;
    reset_sync(ctx, g);
    const long long maxSpin = 1ll << 24;
    dim3 grid(systolic_grid(ctx, g)), block(128);
    const int N = ctx->mesh.N;
    if (MODE == 2 || nc == 1)
        k_systolic<MODE, 1><<<grid, block, 0, ctx->stream>>>(g, mask, r, w, N, s.sync.p, maxSpin);
    else if (nc <= 3)
        k_systolic<MODE, 3><<<grid, block, 0, ctx->stream>>>(g, mask, r, w, N, s.sync.p, maxSpin);
    else
        k_systolic<MODE, 6><<<grid, block, 0, ctx->stream>>>(g, mask, r, w, N, s.sync.p, maxSpin);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 2);
    s.pendingCheck = true;
}

}  // namespace

void skew_prepare(rt_ctx *ctx, const double *diag, const double *upper, const double *lower) {
    StructMesh &s = ctx->mesh.sm;
    SkewView g = s.view();
    int nb = nblocks(g.nSkew);
    k_skew_setup<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, s.faceLo.p, s.faceHi.p, ctx->mesh.N, diag, upper, lower);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    launch_mode<2>(ctx, g, 1, 1u, nullptr, nullptr);
    k_skew_premul<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, s.faceLo.p, s.faceHi.p, ctx->mesh.N, upper, lower);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

void skew_precondition(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w) {
    SkewView g = ctx->mesh.sm.view();
    launch_mode<0>(ctx, g, nc, mask, r, w);
    launch_mode<1>(ctx, g, nc, mask, r, w);
}

rt_status skew_check(rt_ctx *ctx) {
    StructMesh &s = ctx->mesh.sm;
    if (!s.pendingCheck) return RT_OK;
    int err = 0;
    RT_CUDA(cudaMemcpyAsync(&err, s.sync.p + SYNC_ERROR, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RT_CUDA(cudaStreamSynchronize(ctx->stream));
    s.pendingCheck = false;
    return err ? RT_ETIMEOUT : RT_OK;
}

}  // namespace rt
