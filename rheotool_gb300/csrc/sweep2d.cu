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
// j-block below through a shared-memory ring of tagged words (the value
// with its step, so the reader waits on the data itself; the reader's
// progress counter only bounds how far the writer runs ahead).  The
// recurrences are evaluated in the order of operations of the sequential
// sweep (y face, then x face), so an FP64 application equals the
// level-scheduled one bit for bit; the FP32 applications of the mixed
// precision solvers use coefficients rounded from the FP64 factorisation.
//
// A case with nJB j-blocks runs nx + 31 + 32 (nJB - 1) steps; cases are
// independent, so the CTAs of a launch never wait on one another.  Every wait
// is bounded: a timeout sets the error flag, every other wait gives up on
// seeing it, and the host reports RT_ETIMEOUT.
#include "batch.h"
#include "real_ops.cuh"
#include "sweep2d_cta.cuh"

namespace rt {

namespace {

// MAXT: 256 threads (up to 8 j-blocks, the register room for the prefetched
// chunk) or 1024 (up to 32, with a shallower j-block ring to fit the shared
// memory)
template <int MAXT>
__host__ __device__ constexpr int ring2d() { return MAXT <= 256 ? s2d::kRJ : 64; }
template <class Real, int MODE, int NC, int P, int MAXT>
__global__ void __launch_bounds__(MAXT) k_sweep2d(Skew2D<Real> g, const int *__restrict__ order, unsigned mask,
                                                  Real *__restrict__ w, int N, int *err, long long maxSpin) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sProg[32];
    constexpr int RJ = ring2d<MAXT>();
    s2d::u64 *ring = reinterpret_cast<s2d::u64 *>(smem_raw);
    const int cb = order[blockIdx.x];
    s2d::reset<Real, NC, RJ>(ring, g.JB[cb], sProg);
    __syncthreads();
    sweep2d_cta<Real, MODE, NC, P, (MAXT <= 256), RJ>(g, cb, mask, w, N, err, maxSpin, ring, sProg);
}

}  // namespace

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

template <class Real, int MODE, int NC, int P, int MAXT>
void launch2d_t(rt_ctx *ctx, const Skew2D<Real> &g, unsigned mask, Real *w) {
    Batch &b = ctx->mesh.batch;
    const size_t shm = (size_t)b.maxJB * ring2d<MAXT>() * NC * s2d::W<Real>::n * sizeof(s2d::u64);
    static size_t attr = 0;   // the dynamic shared memory this kernel was opened to
    if (shm > attr && shm + 1024 > 48 * 1024) {   // (beside its static counters)
        RT_CUDA(cudaFuncSetAttribute(k_sweep2d<Real, MODE, NC, P, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)shm));
        attr = shm;
    }
    k_sweep2d<Real, MODE, NC, P, MAXT><<<b.n, 32 * b.maxJB, shm, ctx->stream>>>(g, b.caseOrder.p, mask, w,
                                                                                ctx->mesh.N, b.sErr.p, 1ll << 22);
    RT_CHECK_LAUNCH();
}

template <class Real, int MODE, int NC, int P>
void launch2d(rt_ctx *ctx, const Skew2D<Real> &g, unsigned mask, Real *w) {
    Batch &b = ctx->mesh.batch;
    if (b.maxJB <= 8) launch2d_t<Real, MODE, NC, P, 256>(ctx, g, mask, w);
    else launch2d_t<Real, MODE, NC, P, 1024>(ctx, g, mask, w);
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

Skew2D<float> sweep2d_view32(rt_ctx *ctx) { return view2d<float>(ctx->mesh.batch); }
Skew2D<double> sweep2d_view64(rt_ctx *ctx) { return view2d<double>(ctx->mesh.batch); }

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
