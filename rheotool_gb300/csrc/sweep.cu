// sweep.cu — systolic triangular sweeps of DIC / DILU on structured meshes.
//
// A structured mesh is the active-cell subset of an nx x ny x nz box numbered
// lexicographically (i fastest), as blockMesh numbers a block.  Its lower
// neighbours are (i,j,k-1), (i,j-1,k), (i-1,j,k) in increasing face order, its
// upper neighbours (i+1,j,k), (i,j+1,k), (i,j,k+1).  The sequential D-ILU
// recurrences of OpenFOAM (rD, forward, backward; face-ordered accumulation)
// are evaluated here in exactly that order of operations, so the result equals
// the level-scheduled sweep bit for bit (and the sequential sweep up to FMA
// contraction).
//
// Work decomposition: rows (j,k) are grouped in blocks of 32 consecutive j in
// one plane k.  A warp owns a block; at step t lane l updates cell i = t - l of
// row j = 32 jb + l.  The i-1 value is the lane's own previous result
// (register) and the j-1 value lane l-1's previous result (shuffle).  Lane 0
// reads j-1 from the j-block below (step t + 31) and every lane reads k-1 from
// the block of the previous plane (same step): those come through memory
// behind progress counters.  The steps are taken in chunks of P: a chunk
// waits once, issues all its loads at once (one memory latency per chunk) and
// publishes once.
//
// A CTA owns KC consecutive planes with all their j-blocks; waits inside the
// CTA use shared-memory counters and block-scope fences, only the first plane
// of a CTA waits on the previous CTA's last plane through a global counter
// (release / acquire).  CTAs take plane groups in dependency order from an
// atomic counter, so a CTA only waits on groups owned by running CTAs: no
// deadlock.  Every wait is bounded; a timeout sets an error flag, marks the
// block finished and the host reports RT_ETIMEOUT.
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
__device__ __forceinline__ void pf_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// lane 0 spins on a shared counter (bounded); returns the value seen, or
// -1 after a timeout (error flag set)
__device__ __forceinline__ int spin_shared(volatile int *c, int need, int *sync, long long maxSpin) {
    long long spins = 0;
    int v = *c;
    while (v < need) {
        if ((++spins & 1023) == 0 && (spins > maxSpin || load_acquire(sync + SYNC_ERROR))) {
            atomicExch(sync + SYNC_ERROR, 1);
            return -1;
        }
        v = *c;
    }
    return v;
}

__device__ __forceinline__ int spin_global(const int *c, int need, int *sync, long long maxSpin) {
    long long spins = 0;
    int v = load_acquire(c);
    while (v < need) {
        if (++spins > maxSpin || load_acquire(sync + SYNC_ERROR)) {
            atomicExch(sync + SYNC_ERROR, 1);
            return -1;
        }
        if (spins > 16) __nanosleep(32);
        v = load_acquire(c);
    }
    return v;
}

}  // namespace

// MODE 0: forward application, 1: backward application, 2: rD recurrence.
// Warp w = o * nJB + jo of a CTA handles plane position o, j-block jo.
template <int MODE, int NC, int P>
__global__ void __launch_bounds__(512) k_systolic(SkewView g, unsigned mask, double *__restrict__ w, int N,
                                                  int *sync, long long maxSpin, int KC) {
    __shared__ int s_grp;
    __shared__ volatile int s_prog[16];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_grp = atomicAdd(sync + SYNC_WORK, 1);
    if (threadIdx.x < 16) s_prog[threadIdx.x] = 0;
    __syncthreads();
    const int nGroups = (g.nz + KC - 1) / KC;
    const int grp = s_grp;
    if (grp >= nGroups) return;
    const int gi = (MODE == 1) ? nGroups - 1 - grp : grp;
    const int o = wid / g.nJB, jo = wid % g.nJB;
    const int k = (MODE == 1) ? gi * KC + (KC - 1 - o) : gi * KC + o;
    const int jb = (MODE == 1) ? g.nJB - 1 - jo : jo;
    const int T = g.T;
    int *gprog = sync + SYNC_PROGRESS;
    if (k < 0 || k >= g.nz) {
        // a plane beyond the mesh in a partial group: nothing to do
        if (lane == 0) s_prog[wid] = T;
        return;
    }
    const bool crossProducer = (o == KC - 1);
    const int blk = k * g.nJB + jb;
    const long long BS = (long long)T * 32;
    const long long KS = (long long)g.nJB * BS;
    const int depKw = (o > 0) ? wid - g.nJB : -1;
    const int kd = (MODE == 1) ? k + 1 : k - 1;
    const int depKg = (o == 0 && kd >= 0 && kd < g.nz) ? kd * g.nJB + jb : -1;
    const bool hasK = (MODE == 1) ? (k + 1 < g.nz) : (k > 0);
    const int depJw = (jo > 0) ? wid - 1 : -1;
    constexpr int PF = 4 * P;   // prefetch distance in steps
    int seenK = 0, seenJ = 0, fail = 0;
    double yprev[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) yprev[q] = (MODE == 2) ? 1.0 : 0.0;

    for (int t0 = 0; t0 < T; t0 += P) {
        const int te = min(T, t0 + P);          // chunk [t0, te)
        // ---- prefetch the coefficients of a later chunk into L1
        {
            const int tp = t0 + PF + (lane & (P - 1));
            if (tp < T) {
                const long long ep = (MODE == 1) ? (long long)blk * BS + (long long)(T - 1 - tp) * 32
                                                 : (long long)blk * BS + (long long)tp * 32;
                // lanes share out (array, step) pairs; a step line is 256 bytes
                for (int which = lane / P; which < 8; which += 32 / P) {
                    const void *pa = nullptr;
                    if (MODE == 2) {
                        switch (which) {
                        case 0: pa = g.D + ep; break;
                        case 1: pa = g.Pz + ep; break;
                        case 2: pa = g.Py + ep; break;
                        case 3: pa = g.Px + ep; break;
                        default: break;
                        }
                    } else {
                        switch (which) {
                        case 0: pa = (MODE == 0 ? g.Az : g.Bz) + ep; break;
                        case 1: pa = (MODE == 0 ? g.Ay : g.By) + ep; break;
                        case 2: pa = (MODE == 0 ? g.Ax : g.Bx) + ep; break;
                        case 3: pa = (MODE == 0 ? g.rDinv : g.wS) + ep; break;
                        case 4: pa = (MODE == 0 ? g.rS + ep : nullptr); break;
                        default: break;
                        }
                    }
                    if (pa) {
                        pf_l1(pa);
                        pf_l1((const double *)pa + 16);
                    }
                    if (which == 7) pf_l1(g.cellOf + ep);
                }
            }
        }
        // ---- wait: previous plane through step te, previous j-block through te + 31
        if (hasK && seenK < te) {
            int v = 0;
            if (lane == 0) {
                if (depKw >= 0) v = spin_shared(s_prog + depKw, te, sync, maxSpin);
                else v = spin_global(gprog + depKg, te, sync, maxSpin >> 6);
            }
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) { fail = 1; break; }
            seenK = v;
            __threadfence_block();
        }
        if (depJw >= 0 && seenJ < min(T, te + 31)) {
            int v = 0;
            if (lane == 0) v = spin_shared(s_prog + depJw, min(T, te + 31), sync, maxSpin);
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) { fail = 1; break; }
            seenJ = v;
            __threadfence_block();
        }
        // ---- loads of the chunk (independent of the recurrence)
        long long e[P];
        int cell[P];
        double c0[P], c1[P], c2[P], c3[P];
        double rk[P][NC], wk[P][NC], wj[P][NC];
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int t = t0 + s;
            const bool in = t < te;
            e[s] = (MODE == 1) ? (long long)blk * BS + (long long)(T - 1 - t) * 32 + (31 - lane)
                               : (long long)blk * BS + (long long)t * 32 + lane;
            cell[s] = in ? g.cellOf[e[s]] : -1;
            const bool jOK = (depJw >= 0) && (t + 31 < T) && lane == 0 && in;
            long long eJ = 0;
            if (jOK) eJ = (MODE == 1) ? (long long)(blk + 1) * BS + (long long)(T - 1 - (t + 31)) * 32
                                      : (long long)(blk - 1) * BS + (long long)(t + 31) * 32 + 31;
            if (MODE == 2) {
                c0[s] = in ? g.D[e[s]] : 1.0;
                c1[s] = in ? g.Pz[e[s]] : 0.0;
                c2[s] = in ? g.Py[e[s]] : 0.0;
                c3[s] = in ? g.Px[e[s]] : 0.0;
                wk[s][0] = (in && hasK) ? __ldcg(g.rDraw + e[s] - KS) : 1.0;
                wj[s][0] = jOK ? __ldcg(g.rDraw + eJ) : 1.0;
            } else {
                c0[s] = in ? ((MODE == 0) ? g.Az[e[s]] : g.Bz[e[s]]) : 0.0;
                c1[s] = in ? ((MODE == 0) ? g.Ay[e[s]] : g.By[e[s]]) : 0.0;
                c2[s] = in ? ((MODE == 0) ? g.Ax[e[s]] : g.Bx[e[s]]) : 0.0;
                c3[s] = (in && MODE == 0) ? g.rDinv[e[s]] : 0.0;
                const long long eK = (MODE == 1) ? e[s] + KS : e[s] - KS;
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    const long long oq = (long long)q * g.nSkew;
                    const bool on = in && ((mask >> q) & 1u);
                    rk[s][q] = on ? ((MODE == 0) ? g.rS[oq + e[s]] : g.wS[oq + e[s]]) : 0.0;
                    wk[s][q] = (on && hasK) ? __ldcg(g.wS + oq + eK) : 0.0;
                    wj[s][q] = (on && jOK) ? __ldcg(g.wS + oq + eJ) : 0.0;
                }
            }
        }
        // ---- the recurrence
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int t = t0 + s;
            double yup[NC];
#pragma unroll
            for (int q = 0; q < NC; ++q) yup[q] = __shfl_up_sync(0xffffffffu, yprev[q], 1);
            if (t >= te) break;
            const bool jOK = (depJw >= 0) && (t + 31 < T);
            if (MODE == 2) {
                double v = 1.0;
                if (cell[s] >= 0) {
                    v = c0[s];
                    if (hasK) v -= c1[s] / wk[s][0];
                    const double yj = (lane > 0) ? yup[0] : (jOK ? wj[s][0] : 1.0);
                    v -= c2[s] / yj;
                    v -= c3[s] / yprev[0];
                }
                g.rDraw[e[s]] = v;
                yprev[0] = v;
            } else {
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    if (!((mask >> q) & 1u)) continue;
                    double acc = 0.0;
                    if (cell[s] >= 0) {
                        acc = (MODE == 0) ? c3[s] * rk[s][q] : rk[s][q];
                        if (hasK) acc -= c0[s] * wk[s][q];
                        const double yj = (lane > 0) ? yup[q] : (jOK ? wj[s][q] : 0.0);
                        acc -= c1[s] * yj;
                        acc -= c2[s] * yprev[q];
                        if (MODE == 1) w[(long long)q * N + cell[s]] = acc;
                    }
                    g.wS[(long long)q * g.nSkew + e[s]] = acc;
                    yprev[q] = acc;
                }
            }
        }
        // ---- publish
        __threadfence_block();
        __syncwarp();
        if (lane == 0) s_prog[wid] = te;
        if (crossProducer && ((te % (2 * P)) == 0 || te == T)) {
            __threadfence();
            __syncwarp();
            if (lane == 0) store_release(gprog + blk, te);
        }
    }
    if (fail) {
        if (lane == 0) s_prog[wid] = T;
        if (crossProducer) {
            __threadfence();
            if (lane == 0) store_release(gprog + blk, T);
        }
    }
}

// rS = r gathered into the skewed layout (0 outside the mesh)
__global__ void k_skew_gather(SkewView g, unsigned mask, int nc, const double *__restrict__ r, int N) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    int c = g.cellOf[e];
    for (int q = 0; q < nc; ++q)
        if ((mask >> q) & 1u) g.rS[(long long)q * g.nSkew + e] = c >= 0 ? r[(long long)q * N + c] : 0.0;
}

// gather the skewed per-entry coefficients of one matrix
__global__ void k_skew_setup(SkewView g, const int *__restrict__ faceLo, int N, const double *__restrict__ diag,
                             const double *__restrict__ upper, const double *__restrict__ lower) {
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

template <int MODE>
void launch_mode(rt_ctx *ctx, const SkewView &g, int nc, unsigned mask, double *w) {
    StructMesh &s = ctx->mesh.sm;
    RT_CUDA(cudaMemsetAsync(s.sync.p, 0, sizeof(int) * (SYNC_PROGRESS + g.nz * g.nJB), ctx->stream));
    const long long maxSpin = 1ll << 26;
    const int KC = s.KC;
    const int nGroups = (g.nz + KC - 1) / KC;
    dim3 grid(nGroups), block(32 * KC * g.nJB);
    const int N = ctx->mesh.N;
    cudaStream_t st = ctx->stream;
    if (MODE == 2 || nc == 1)
        k_systolic<MODE, 1, 4><<<grid, block, 0, st>>>(g, mask, w, N, s.sync.p, maxSpin, KC);
    else if (nc <= 3)
        k_systolic<MODE, 3, 2><<<grid, block, 0, st>>>(g, mask, w, N, s.sync.p, maxSpin, KC);
    else
        k_systolic<MODE, 6, 1><<<grid, block, 0, st>>>(g, mask, w, N, s.sync.p, maxSpin, KC);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 2);
    s.pendingCheck = true;
}

}  // namespace

void skew_prepare(rt_ctx *ctx, const double *diag, const double *upper, const double *lower) {
    StructMesh &s = ctx->mesh.sm;
    SkewView g = s.view();
    int nb = nblocks(g.nSkew);
    k_skew_setup<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, s.faceLo.p, ctx->mesh.N, diag, upper, lower);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    launch_mode<2>(ctx, g, 1, 1u, nullptr);
    k_skew_premul<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, s.faceLo.p, s.faceHi.p, ctx->mesh.N, upper, lower);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

void skew_precondition(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w) {
    SkewView g = ctx->mesh.sm.view();
    k_skew_gather<<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    launch_mode<0>(ctx, g, nc, mask, w);
    launch_mode<1>(ctx, g, nc, mask, w);
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
