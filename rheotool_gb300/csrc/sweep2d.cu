// sweep2d.cu — DIC / DILU triangular sweeps of a batch of structured 2-D
// cases, one CTA per case.
//
// Each case is the active-cell subset of an nx x ny box, one cell thick,
// numbered lexicographically (i fastest): its lower neighbours are (i, j-1)
// and (i-1, j) in increasing face order, its upper neighbours (i+1, j) and
// (i, j+1).  As in the 3-D systolic sweeps (sweep.cu), a warp owns 32
// consecutive rows (a j-block), lane l updating cell i = t - l of row
// 32 jb + l at step t: the i-1 value is the lane's own previous result, the
// j-1 value lane l-1's (shuffle), and lane 0 reads row 32 jb - 1 from the
// j-block below through a shared-memory ring behind a progress counter.  The
// recurrences are evaluated in the order of operations of the sequential
// sweep (y face, then x face), so an FP64 application equals the
// level-scheduled one bit for bit; the FP32 applications of the mixed
// precision solvers use coefficients rounded from the FP64 factorisation.
//
// A case with nJB j-blocks runs nx + 31 + 32 (nJB - 1) steps; cases are
// independent, so the CTAs of a launch never wait on one another.  Every wait
// is bounded: a timeout sets the error flag, publishes the warp's progress as
// complete (so no other warp waits on it) and the host reports RT_ETIMEOUT.
#include "batch.h"
#include "real_ops.cuh"

namespace rt {

namespace {

constexpr int kRJ = 64;   // j-block ring depth (power of two); the consumer lags 32 + P steps

__device__ __forceinline__ int ld_acquire_cta(const int *p) {
    int v;
    asm volatile("ld.acquire.cta.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cta(int *p, int v) {
    asm volatile("st.release.cta.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// lane 0 of a warp waits until *c >= need (bounded); -1 after a timeout
__device__ __forceinline__ int spin_cta(const int *c, int need, int *err, long long maxSpin) {
    long long spins = 0;
    int v = ld_acquire_cta(c);
    while (v < need) {
        if ((++spins & 255) == 0 && (spins > maxSpin || *(volatile int *)err)) {
            atomicExch(err, 1);
            return -1;
        }
        v = ld_acquire_cta(c);
    }
    return v;
}

}  // namespace

// MODE 0: forward application (rS -> wS), 1: backward application (wS -> w),
// 2: rD recurrence (D, Py, Px -> rDraw).
template <class Real, int MODE, int NC, int P>
__global__ void __launch_bounds__(1024) k_sweep2d(Skew2D<Real> g, unsigned mask, Real *__restrict__ w, int N,
                                                  int *err, long long maxSpin) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sProg[32];
    const int cb = blockIdx.x, lane = threadIdx.x & 31, jo = threadIdx.x >> 5;
    const int nJB = g.JB[cb], T = g.T[cb];
    const long long off = g.off[cb];
    Real *ringJ = reinterpret_cast<Real *>(smem_raw);   // [maxJB][kRJ][NC]
    if (threadIdx.x < 32) sProg[threadIdx.x] = 0;
    __syncthreads();
    if (jo >= nJB) return;
    const int jb = (MODE == 1) ? nJB - 1 - jo : jo;
    const long long e0 = (MODE == 1) ? off + ((long long)jb * T + (T - 1)) * 32 + (31 - lane)
                                     : off + (long long)jb * T * 32 + lane;
    const long long st = (MODE == 1) ? -32 : 32;
    const int depJ = (jo > 0) ? jo - 1 : -1;
    const int consJ = (jo + 1 < nJB) ? jo + 1 : -1;
    const Real zk = (MODE == 2) ? Real(1) : Real(0);
    Real yprev[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) yprev[q] = zk;
    int seenJ = 0, seenCJ = 0;
    for (int t0 = 0; t0 < T; t0 += P) {
        const int te = t0 + P;   // T is a multiple of P
        // the consumer has read the ring slots this chunk overwrites
        if (consJ >= 0 && seenCJ < te - kRJ - 31) {
            int v = 0;
            if (lane == 0) v = spin_cta(sProg + consJ, te - kRJ - 31, err, maxSpin);
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) break;
            seenCJ = v;
        }
        // the j-block below has produced row 32 jb - 1 through step te + 31
        if (depJ >= 0 && seenJ < min(T, te + 31)) {
            int v = 0;
            if (lane == 0) v = spin_cta(sProg + depJ, min(T, te + 31), err, maxSpin);
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) break;
            seenJ = v;
        }
        __syncwarp();
        // loads of the chunk (independent of the recurrence)
        Real c0[P], cy[P], cx[P], rk[P][NC];
        int cell[P];
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const long long e = e0 + (long long)(t0 + s) * st;
            if (MODE == 2) {
                c0[s] = g.D[e]; cy[s] = g.Py[e]; cx[s] = g.Px[e];
            } else {
                c0[s] = (MODE == 0) ? g.rDinv[e] : Real(0);
                cy[s] = (MODE == 0) ? g.Ay[e] : g.By[e];
                cx[s] = (MODE == 0) ? g.Ax[e] : g.Bx[e];
#pragma unroll
                for (int q = 0; q < NC; ++q) rk[s][q] = ((MODE == 0) ? g.rS : g.wS)[(long long)q * g.nSkew + e];
            }
            cell[s] = (MODE == 1) ? g.cellOf[e] : 0;
        }
        Real out[P][NC];
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int t = t0 + s;
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const Real yup = __shfl_up_sync(0xffffffffu, yprev[q], 1);
                const Real yj = (lane > 0) ? yup
                                           : ((depJ >= 0 && t + 31 < T) ? ringJ[((size_t)depJ * kRJ + ((t + 31) & (kRJ - 1))) * NC + q]
                                                                         : zk);
                Real v;
                if (MODE == 2) {
                    v = r_sub(c0[s], r_div(cy[s], yj));
                    v = r_sub(v, r_div(cx[s], yprev[q]));
                } else {
                    const Real pre = (MODE == 0) ? r_mul(c0[s], rk[s][q]) : rk[s][q];
                    if (sizeof(Real) == 4) {   // FP32: the i term first (as the 3-D sweeps)
                        v = r_fma(-cx[s], yprev[q], pre);
                        v = r_fma(-cy[s], yj, v);
                    } else {
                        v = r_fma(-cy[s], yj, pre);
                        v = r_fma(-cx[s], yprev[q], v);
                    }
                }
                if (consJ >= 0 && lane == 31) ringJ[((size_t)jo * kRJ + (t & (kRJ - 1))) * NC + q] = v;
                out[s][q] = v;
                yprev[q] = v;
            }
        }
        __syncwarp();
        if (lane == 0 && (consJ >= 0 || depJ >= 0)) st_release_cta(sProg + jo, te);
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const long long e = e0 + (long long)(t0 + s) * st;
            if (MODE == 2) {
                g.rDraw[e] = out[s][0];
            } else {
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    if (!((mask >> q) & 1u)) continue;
                    if (MODE == 0) g.wS[(long long)q * g.nSkew + e] = out[s][q];
                    else if (cell[s] >= 0) w[(long long)q * N + cell[s]] = out[s][q];
                }
            }
        }
    }
    // a warp that gave up releases everything it owes
    if (*(volatile int *)err && lane == 0) st_release_cta(sProg + jo, T);
}

template <class Real>
__global__ void k_s2_gather(Skew2D<Real> g, unsigned mask, int nc, const Real *__restrict__ r, int N) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    int c = g.cellOf[e];
    for (int q = 0; q < nc; ++q)
        if ((mask >> q) & 1u) g.rS[(long long)q * g.nSkew + e] = c >= 0 ? r[(long long)q * N + c] : Real(0);
}

__global__ void k_s2_setup(Skew2D<double> g, const int *__restrict__ faceLo, int N, const double *__restrict__ diag,
                           const double *__restrict__ upper, const double *__restrict__ lower) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    int c = g.cellOf[e];
    double d = 1.0, py = 0.0, px = 0.0;
    if (c >= 0) {
        d = diag[c];
        int fy = faceLo[c], fx = faceLo[N + c];
        if (fy >= 0) py = __dmul_rn(upper[fy], lower[fy]);
        if (fx >= 0) px = __dmul_rn(upper[fx], lower[fx]);
    }
    g.D[e] = d;
    g.Py[e] = py;
    g.Px[e] = px;
}

__global__ void k_s2_premul(Skew2D<double> g, const int *__restrict__ faceLo, const int *__restrict__ faceHi, int N,
                            const double *__restrict__ upper, const double *__restrict__ lower) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    int c = g.cellOf[e];
    double rd = 0.0, ay = 0.0, ax = 0.0, by = 0.0, bx = 0.0;
    if (c >= 0) {
        rd = 1.0 / g.rDraw[e];
        int fy = faceLo[c], fx = faceLo[N + c], gy = faceHi[c], gx = faceHi[N + c];
        if (fy >= 0) ay = rd * lower[fy];
        if (fx >= 0) ax = rd * lower[fx];
        if (gy >= 0) by = rd * upper[gy];
        if (gx >= 0) bx = rd * upper[gx];
    }
    g.rDinv[e] = rd;
    g.Ay[e] = ay; g.Ax[e] = ax;
    g.By[e] = by; g.Bx[e] = bx;
}

__global__ void k_s2_to32(Skew2D<double> g, Skew2D<float> h) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    h.rDinv[e] = (float)g.rDinv[e];
    h.Ay[e] = (float)g.Ay[e]; h.Ax[e] = (float)g.Ax[e];
    h.By[e] = (float)g.By[e]; h.Bx[e] = (float)g.Bx[e];
}

namespace {

template <class Real>
Skew2D<Real> view2d(Batch &b);

template <>
Skew2D<double> view2d<double>(Batch &b) {
    Skew2D<double> g{};
    g.nCases = b.n; g.maxJB = b.maxJB; g.nSkew = b.nSkew;
    g.T = b.sT.p; g.JB = b.sJB.p; g.off = b.sOff.p; g.cellOf = b.sCell.p;
    if (b.sData64.n != (size_t)21 * b.nSkew) b.sData64.alloc((size_t)21 * b.nSkew);
    double *p = b.sData64.p;
    double **slots[] = {&g.D, &g.Py, &g.Px, &g.rDraw, &g.rDinv, &g.Ay, &g.Ax, &g.By, &g.Bx};
    for (int i = 0; i < 9; ++i) *slots[i] = p + (size_t)i * b.nSkew;
    g.wS = p + (size_t)9 * b.nSkew;
    g.rS = p + (size_t)15 * b.nSkew;
    return g;
}

template <>
Skew2D<float> view2d<float>(Batch &b) {
    Skew2D<float> g{};
    g.nCases = b.n; g.maxJB = b.maxJB; g.nSkew = b.nSkew;
    g.T = b.sT.p; g.JB = b.sJB.p; g.off = b.sOff.p; g.cellOf = b.sCell.p;
    if (b.sData32.n != (size_t)17 * b.nSkew) b.sData32.alloc((size_t)17 * b.nSkew);
    float *p = b.sData32.p;
    g.D = g.Py = g.Px = g.rDraw = nullptr;
    float **slots[] = {&g.rDinv, &g.Ay, &g.Ax, &g.By, &g.Bx};
    for (int i = 0; i < 5; ++i) *slots[i] = p + (size_t)i * b.nSkew;
    g.wS = p + (size_t)5 * b.nSkew;
    g.rS = p + (size_t)11 * b.nSkew;
    return g;
}

template <class Real, int MODE, int NC, int P>
void launch2d(rt_ctx *ctx, const Skew2D<Real> &g, unsigned mask, Real *w) {
    Batch &b = ctx->mesh.batch;
    const size_t shm = (size_t)b.maxJB * kRJ * NC * sizeof(Real);
    static size_t attr = 0;
    if (shm > attr && shm > 48 * 1024) {
        RT_CUDA(cudaFuncSetAttribute(k_sweep2d<Real, MODE, NC, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)shm));
        attr = shm;
    }
    k_sweep2d<Real, MODE, NC, P><<<b.n, 32 * b.maxJB, shm, ctx->stream>>>(g, mask, w, ctx->mesh.N, b.sErr.p,
                                                                          1ll << 22);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    b.sPending = true;
}

template <class Real, int MODE>
void launch2d_nc(rt_ctx *ctx, const Skew2D<Real> &g, int nc, unsigned mask, Real *w) {
    if (nc == 1) launch2d<Real, MODE, 1, 8>(ctx, g, mask, w);
    else if (nc <= 3) launch2d<Real, MODE, 3, 4>(ctx, g, mask, w);
    else launch2d<Real, MODE, 6, 2>(ctx, g, mask, w);
}

template <class Real>
void precondition2d(rt_ctx *ctx, int nc, unsigned mask, const Real *r, Real *w) {
    Batch &b = ctx->mesh.batch;
    Skew2D<Real> g = view2d<Real>(b);
    k_s2_gather<Real><<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    launch2d_nc<Real, 0>(ctx, g, nc, mask, w);
    launch2d_nc<Real, 1>(ctx, g, nc, mask, w);
}

}  // namespace

void sweep2d_prepare(rt_ctx *ctx, const double *diag, const double *upper, const double *lower, bool fp32) {
    Batch &b = ctx->mesh.batch;
    Skew2D<double> g = view2d<double>(b);
    const int nb = nblocks(g.nSkew);
    const int N = ctx->mesh.N;
    k_s2_setup<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, b.sFaceLo.p, N, diag, upper, lower);
    RT_CHECK_LAUNCH();
    launch2d<double, 2, 1, 8>(ctx, g, 1u, (double *)nullptr);
    k_s2_premul<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, b.sFaceLo.p, b.sFaceHi.p, N, upper, lower);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 2);
    if (fp32) {
        Skew2D<float> h = view2d<float>(b);
        k_s2_to32<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, h);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }
}

void sweep2d_precondition(rt_ctx *ctx, int nc, unsigned mask, const float *r, float *w) {
    precondition2d<float>(ctx, nc, mask, r, w);
}
void sweep2d_precondition(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w) {
    precondition2d<double>(ctx, nc, mask, r, w);
}

rt_status sweep2d_check(rt_ctx *ctx) {
    Batch &b = ctx->mesh.batch;
    if (!b.sPending) return RT_OK;
    int err = 0;
    RT_CUDA(cudaMemcpyAsync(&err, b.sErr.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RT_CUDA(cudaStreamSynchronize(ctx->stream));
    b.sPending = false;
    if (err) RT_CUDA(cudaMemsetAsync(b.sErr.p, 0, sizeof(int), ctx->stream));
    return err ? RT_ETIMEOUT : RT_OK;
}

}  // namespace rt
