// krylov.cu — OpenFOAM lduMatrix solvers on the device: PCG (+DIC) and
// PBiCGStab (+DILU), run for up to six right-hand sides that share one LDU
// matrix (the components of U or theta), in lock step, each component with
// its own scalars and its own stopping point.
//
// Semantics follow the published methods as OpenFOAM applies them (see the
// oracle for the sequential restatement):
//   * residual = sum|b - A x| / normFactor, normFactor = sum(|A x - xbar A1|
//     + |b - xbar A1|) + 1e-20 (rheoTool sparseSolver.C:129-180);
//   * converged when res < tolerance or res < relTol * res0, never before
//     minIter iterations, at most maxIter;
//   * D-ILU(0) / DIC: rD_u = a_uu - sum_l a_ul a_lu / rD_l in face order,
//     applied as w = rD r, forward w_u -= rD_u a_ul w_l (faces ascending),
//     backward w_l -= rD_l a_lu w_u (faces descending).
//
// The triangular recurrences are exact: cells are processed level by level
// (level = 1 + max level of the lower neighbours), and inside a cell the
// neighbour contributions are accumulated in face order, which reproduces the
// sequential sweep's arithmetic.  Reductions are two-stage block trees in a
// fixed order, so every solve is run-to-run bit-reproducible.
#include <cmath>
#include <cstring>

#include "rt_internal.h"
#include "sweep.h"

namespace rt {

// scalar slots (device array ctx->scal, [slot*8 + comp])
enum {
    S_NF = 0, S_INIT, S_FIN, S_XBAR, S_A, S_B, S_AOLD, S_ALPHA, S_OMEGA,
    S_R0R, S_R0ROLD, S_SING, S_T1, S_T2, S_NSLOT
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// block sum, valid in thread 0; safe to call repeatedly in one kernel
__device__ double block_sum(double v) {
    __shared__ double sh[32];
    v = warp_sum(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) v = warp_sum(v);
    return v;
}

// partial[(slot*6 + k)*nBlocks + block]
__device__ __forceinline__ void store_partial(double *partial, int nB, int slot, int k, double v) {
    double s = block_sum(v);
    if (threadIdx.x == 0) partial[(slot * 6 + k) * nB + blockIdx.x] = s;
}

// one block per (slot, k): fixed-order tree over the block partials
__global__ void k_finalize(int nB, int nSlotsUsed, unsigned mask, const double *__restrict__ partial,
                           double *__restrict__ result) {
    int slot = blockIdx.x / 6, k = blockIdx.x % 6;
    if (slot >= nSlotsUsed || !((mask >> k) & 1u)) return;
    double v = 0.0;
    for (int i = threadIdx.x; i < nB; i += blockDim.x) v += partial[(slot * 6 + k) * nB + i];
    v = block_sum(v);
    if (threadIdx.x == 0) result[slot * 6 + k] = v;
}

// --------------------------------------------------------------------------
// matrix-vector kernels
// --------------------------------------------------------------------------
struct Ell {
    int N, nSlots;
    const int *__restrict__ face;
    const int *__restrict__ nbr;
};

__device__ __forceinline__ double row_mul(const Ell &e, int c, const double *__restrict__ diag,
                                          const double *__restrict__ upper,
                                          const double *__restrict__ lower,
                                          const double *__restrict__ x) {
    double acc = diag[c] * x[c];
    for (int s = 0; s < e.nSlots; ++s) {
        int nb = e.nbr[s * e.N + c];
        if (nb < 0) break;
        int f = e.face[s * e.N + c];
        double a = nb > c ? upper[f] : lower[f];
        acc += a * x[nb];
    }
    return acc;
}

__device__ __forceinline__ double row_sum(const Ell &e, int c, const double *__restrict__ diag,
                                          const double *__restrict__ upper,
                                          const double *__restrict__ lower) {
    double acc = diag[c];
    for (int s = 0; s < e.nSlots; ++s) {
        int nb = e.nbr[s * e.N + c];
        if (nb < 0) break;
        int f = e.face[s * e.N + c];
        acc += nb > c ? upper[f] : lower[f];
    }
    return acc;
}

// partial sums of psi (slot 0) for xbar
__global__ void k_sum(int N, unsigned mask, const double *__restrict__ x, double *partial, int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        double v = 0.0;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x)
            v += x[(size_t)k * N + c];
        store_partial(partial, nB, 0, k, v);
    }
}

// wA = A psi, rA = b - wA; partial slot 0: |wA - xbar sumA| + |b - xbar sumA|,
// slot 1: |rA|
__global__ void k_init_res(Ell e, unsigned mask, const double *__restrict__ diag,
                           const double *__restrict__ upper, const double *__restrict__ lower,
                           const double *__restrict__ b, const double *__restrict__ x,
                           double *__restrict__ wA, double *__restrict__ rA,
                           const double *__restrict__ S, double *partial, int nB) {
    const int N = e.N;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double xbar = S[S_XBAR * 8 + k];
        double v0 = 0.0, v1 = 0.0;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            double ax = row_mul(e, c, diag, upper, lower, x + (size_t)k * N);
            double sa = row_sum(e, c, diag, upper, lower) * xbar;
            double bb = b[(size_t)k * N + c];
            double r = bb - ax;
            wA[(size_t)k * N + c] = ax;
            rA[(size_t)k * N + c] = r;
            v0 += fabs(ax - sa) + fabs(bb - sa);
            v1 += fabs(r);
        }
        store_partial(partial, nB, 0, k, v0);
        store_partial(partial, nB, 1, k, v1);
    }
}

// y = A x on the masked components
__global__ void k_amul(Ell e, unsigned mask, const double *__restrict__ diag,
                       const double *__restrict__ upper, const double *__restrict__ lower,
                       const double *__restrict__ x, double *__restrict__ y) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= e.N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        y[(size_t)k * e.N + c] = row_mul(e, c, diag, upper, lower, x + (size_t)k * e.N);
    }
}

// generic dot products: slot0 = a.b, optional slot1 = c.d
__global__ void k_dot(int N, unsigned mask, const double *__restrict__ a, const double *__restrict__ b,
                      const double *__restrict__ c2, const double *__restrict__ d2, double *partial,
                      int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        double v0 = 0.0, v1 = 0.0;
        size_t o = (size_t)k * N;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            v0 += a[o + c] * b[o + c];
            if (c2) v1 += c2[o + c] * d2[o + c];
        }
        store_partial(partial, nB, 0, k, v0);
        if (c2) store_partial(partial, nB, 1, k, v1);
    }
}

// --------------------------------------------------------------------------
// D-ILU / DIC, level scheduled
// --------------------------------------------------------------------------
__global__ void k_rd_level(Ell e, int l0, int l1, const int *__restrict__ cells,
                           const double *__restrict__ diag, const double *__restrict__ upper,
                           const double *__restrict__ lower, double *__restrict__ rD) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    double r = diag[c];
    for (int s = 0; s < e.nSlots; ++s) {
        int nb = e.nbr[s * e.N + c];
        if (nb < 0 || nb > c) break;          // lower neighbours come first
        int f = e.face[s * e.N + c];
        r = __dsub_rn(r, __ddiv_rn(__dmul_rn(upper[f], lower[f]), rD[nb]));
    }
    rD[c] = r;
}

__global__ void k_recip(int N, double *rD) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < N) rD[c] = 1.0 / rD[c];
}

__global__ void k_recip_diag(int N, const double *diag, double *rD) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < N) rD[c] = 1.0 / diag[c];
}

__global__ void k_fwd_level(Ell e, int l0, int l1, const int *__restrict__ cells, unsigned mask,
                            const double *__restrict__ rD, const double *__restrict__ lower,
                            const double *__restrict__ r, double *__restrict__ w) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    const int N = e.N;
    const double rd = rD[c];
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t o = (size_t)k * N;
        double acc = __dmul_rn(rd, r[o + c]);
        for (int s = 0; s < e.nSlots; ++s) {
            int nb = e.nbr[s * N + c];
            if (nb < 0 || nb > c) break;
            int f = e.face[s * N + c];
            acc = __fma_rn(-__dmul_rn(rd, lower[f]), w[o + nb], acc);
        }
        w[o + c] = acc;
    }
}

__global__ void k_bwd_level(Ell e, int l0, int l1, const int *__restrict__ cells, unsigned mask,
                            const double *__restrict__ rD, const double *__restrict__ upper,
                            double *__restrict__ w) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    const int N = e.N;
    const double rd = rD[c];
    // number of used slots
    int ns = 0;
    while (ns < e.nSlots && e.nbr[ns * N + c] >= 0) ++ns;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t o = (size_t)k * N;
        double acc = w[o + c];
        for (int s = ns - 1; s >= 0; --s) {
            int nb = e.nbr[s * N + c];
            if (nb < c) break;                // upper neighbours are the last slots
            int f = e.face[s * N + c];
            acc = __fma_rn(-__dmul_rn(rd, upper[f]), w[o + nb], acc);
        }
        w[o + c] = acc;
    }
}

__global__ void k_diag_apply(int N, unsigned mask, const double *__restrict__ rD,
                             const double *__restrict__ r, double *__restrict__ w) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) w[(size_t)k * N + c] = __dmul_rn(rD[c], r[(size_t)k * N + c]);
}

__global__ void k_copy(int N, unsigned mask, const double *__restrict__ r, double *__restrict__ w) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) w[(size_t)k * N + c] = r[(size_t)k * N + c];
}

// --------------------------------------------------------------------------
// scalar bookkeeping kernels (one thread per component)
// --------------------------------------------------------------------------
// res[slot*6+k] -> S
__global__ void k_sc_xbar(unsigned mask, int N, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) S[S_XBAR * 8 + k] = res[0 * 6 + k] / N;
}
__global__ void k_sc_init(unsigned mask, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) {
        double nf = res[0 * 6 + k] + 1e-20;
        S[S_NF * 8 + k] = nf;
        S[S_INIT * 8 + k] = res[1 * 6 + k] / nf;
        S[S_FIN * 8 + k] = res[1 * 6 + k] / nf;
        S[S_SING * 8 + k] = 0.0;
        S[S_A * 8 + k] = 1e20;     // wArA before the first iteration
        S[S_R0R * 8 + k] = 0.0;
        S[S_ALPHA * 8 + k] = 0.0;
        S[S_OMEGA * 8 + k] = 0.0;
    }
}
// PCG: wArAold = wArA; wArA = res0
__global__ void k_sc_pcg_a(unsigned mask, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) {
        S[S_AOLD * 8 + k] = S[S_A * 8 + k];
        S[S_A * 8 + k] = res[k];
    }
}
// PCG: alpha = wArA / wApA, singularity test
__global__ void k_sc_pcg_alpha(unsigned mask, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) {
        double wApA = res[k];
        if (fabs(wApA) / S[S_NF * 8 + k] < 1e-300) {
            S[S_SING * 8 + k] = 1.0;
            S[S_ALPHA * 8 + k] = 0.0;
        } else {
            S[S_ALPHA * 8 + k] = S[S_A * 8 + k] / wApA;
        }
    }
}
// residual slot -> S_FIN
__global__ void k_sc_fin(unsigned mask, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) S[S_FIN * 8 + k] = res[k] / S[S_NF * 8 + k];
}
// BiCGStab: rA0rAold = rA0rA; rA0rA = res; singularity tests, beta in S_B
__global__ void k_sc_bicg_r0r(unsigned mask, int iter, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) {
        double old = S[S_R0R * 8 + k];
        double r0r = res[k];
        S[S_R0ROLD * 8 + k] = old;
        S[S_R0R * 8 + k] = r0r;
        if (fabs(r0r) < 1e-300) { S[S_SING * 8 + k] = 1.0; return; }
        if (iter > 0) {
            double om = S[S_OMEGA * 8 + k];
            if (fabs(om) < 1e-300) { S[S_SING * 8 + k] = 1.0; return; }
            S[S_B * 8 + k] = (r0r / old) * (S[S_ALPHA * 8 + k] / om);
        }
    }
}
__global__ void k_sc_bicg_alpha(unsigned mask, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) S[S_ALPHA * 8 + k] = S[S_R0R * 8 + k] / res[k];
}
__global__ void k_sc_bicg_omega(unsigned mask, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) S[S_OMEGA * 8 + k] = res[6 + k] / res[k];
}

// --------------------------------------------------------------------------
// vector update kernels
// --------------------------------------------------------------------------
// PCG: pA = wA (+ beta pA)
__global__ void k_pcg_p(int N, unsigned mask, int first, const double *__restrict__ S,
                        const double *__restrict__ wA, double *__restrict__ pA) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t i = (size_t)k * N + c;
        if (first) pA[i] = wA[i];
        else {
            double beta = S[S_A * 8 + k] / S[S_AOLD * 8 + k];
            pA[i] = wA[i] + beta * pA[i];
        }
    }
}
// PCG: psi += alpha pA; rA -= alpha wA; partial |rA| (slot 0)
__global__ void k_pcg_update(int N, unsigned mask, const double *__restrict__ S,
                             const double *__restrict__ pA, const double *__restrict__ wA,
                             double *__restrict__ psi, double *__restrict__ rA, double *partial, int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const bool sing = S[S_SING * 8 + k] != 0.0;
        const double alpha = S[S_ALPHA * 8 + k];
        double v = 0.0;
        size_t o = (size_t)k * N;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            if (!sing) {
                psi[o + c] += alpha * pA[o + c];
                rA[o + c] -= alpha * wA[o + c];
            }
            v += fabs(rA[o + c]);
        }
        store_partial(partial, nB, 0, k, v);
    }
}
// BiCGStab: pA = rA (first) or rA + beta (pA - omega AyA)
__global__ void k_bicg_p(int N, unsigned mask, int first, const double *__restrict__ S,
                         const double *__restrict__ rA, const double *__restrict__ AyA,
                         double *__restrict__ pA) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        if (S[S_SING * 8 + k] != 0.0) continue;
        size_t i = (size_t)k * N + c;
        if (first) pA[i] = rA[i];
        else pA[i] = rA[i] + S[S_B * 8 + k] * (pA[i] - S[S_OMEGA * 8 + k] * AyA[i]);
    }
}
// BiCGStab: sA = rA - alpha AyA; partial |sA|
__global__ void k_bicg_s(int N, unsigned mask, const double *__restrict__ S,
                         const double *__restrict__ rA, const double *__restrict__ AyA,
                         double *__restrict__ sA, double *partial, int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double alpha = S[S_ALPHA * 8 + k];
        double v = 0.0;
        size_t o = (size_t)k * N;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            double s = rA[o + c] - alpha * AyA[o + c];
            sA[o + c] = s;
            v += fabs(s);
        }
        store_partial(partial, nB, 0, k, v);
    }
}
// psi += alpha yA
__global__ void k_axpy_alpha(int N, unsigned mask, const double *__restrict__ S,
                             const double *__restrict__ yA, double *__restrict__ psi) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) psi[(size_t)k * N + c] += S[S_ALPHA * 8 + k] * yA[(size_t)k * N + c];
}
// psi += alpha yA + omega zA; rA = sA - omega tA; partial |rA|
__global__ void k_bicg_update(int N, unsigned mask, const double *__restrict__ S,
                              const double *__restrict__ yA, const double *__restrict__ zA,
                              const double *__restrict__ sA, const double *__restrict__ tA,
                              double *__restrict__ psi, double *__restrict__ rA, double *partial, int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double alpha = S[S_ALPHA * 8 + k], omega = S[S_OMEGA * 8 + k];
        double v = 0.0;
        size_t o = (size_t)k * N;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            psi[o + c] += alpha * yA[o + c] + omega * zA[o + c];
            double r = sA[o + c] - omega * tA[o + c];
            rA[o + c] = r;
            v += fabs(r);
        }
        store_partial(partial, nB, 0, k, v);
    }
}

// --------------------------------------------------------------------------
// host orchestration
// --------------------------------------------------------------------------
void reduce_init(rt_ctx *ctx) {
    Reduce &r = ctx->red;
    r.nBlocks = ctx->numSMs * 4;
    r.partial.alloc((size_t)8 * 6 * r.nBlocks);
    r.result.alloc(8 * 6);
    RT_CUDA(cudaMallocHost(&r.hostResult, sizeof(double) * 32 * 8));   // one copy of ctx->scal
    ctx->scal.alloc(32 * 8);
    ctx->scal.zero(ctx->stream);
}

namespace {

struct Solver {
    rt_ctx *ctx;
    Ell e;
    int N;
    cudaStream_t st;
    const SolveArgs &a;
    double *S;
    int nB;

    Solver(rt_ctx *c, const SolveArgs &args) : ctx(c), a(args) {
        const DevMesh &m = ctx->mesh;
        N = m.N;
        e = Ell{m.N, m.nSlots, m.ellFace.p, m.ellNbr.p};
        st = ctx->stream;
        S = ctx->scal.p;
        nB = ctx->red.nBlocks;
    }

    int rblocks() const { return std::min(nB, nblocks(N)); }

    // finalize nSlots reduction slots of the masked comps into red.result
    void finalize(int nSlots, unsigned mask) {
        // blocks beyond rblocks() left stale partials: zero them by using only
        // the first rblocks() entries — the reduction kernels always launch
        // exactly nB blocks, so all entries are written.
        k_finalize<<<nSlots * 6, RT_BLOCK, 0, st>>>(nB, nSlots, mask, ctx->red.partial.p, ctx->red.result.p);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }

    void fetch(const double *dev, int count) {
        RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, dev, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
        RT_CUDA(cudaStreamSynchronize(st));
    }

    static int pop(unsigned m) { return __builtin_popcount(m); }

    void amul(unsigned mask, const double *x, double *y) {
        // algorithmic bytes per cell: diag 8, lower+upper 2*(F/N)*8, face
        // addressing 2*(F/N)*4, x and y 16 per component
        const double fpc = (double)ctx->mesh.F / N;
        ProfScope ps(ctx, "amul", (double)N * (8.0 + fpc * 24.0 + 16.0 * pop(mask)));
        k_amul<<<nblocks(N), RT_BLOCK, 0, st>>>(e, mask, a.diag, a.upper, a.lower, x, y);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }

    void dot(unsigned mask, const double *x, const double *y, const double *x2 = nullptr,
             const double *y2 = nullptr) {
        ProfScope ps(ctx, "dot", (double)N * 8.0 * (x2 ? 4 : 2) * pop(mask));
        k_dot<<<nB, RT_BLOCK, 0, st>>>(N, mask, x, y, x2, y2, ctx->red.partial.p, nB);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
        finalize(x2 ? 2 : 1, mask);
    }

    bool systolic() const {
        int pre = a.ctl.preconditioner;
        return ctx->mesh.sm.on && ctx->sweepMode != 1 && (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU);
    }

    void compute_rd(double *rD) {
        const DevMesh &m = ctx->mesh;
        int pre = a.ctl.preconditioner;
        if (systolic()) {
            const double fpc = (double)m.F / N;
            ProfScope ps(ctx, "dilu_rD", (double)N * (16.0 + fpc * 28.0));
            skew_prepare(ctx, a.diag, a.upper, a.lower);
        } else if (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU) {
            const double fpc = (double)m.F / N;
            ProfScope ps(ctx, "dilu_rD", (double)N * (16.0 + fpc * 28.0));
            for (int l = 0; l < m.nLevels; ++l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_rd_level<<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(e, l0, l1, m.levelCells.p, a.diag,
                                                                  a.upper, a.lower, rD);
            }
            RT_CHECK_LAUNCH();
            launch_count(ctx, m.nLevels);
            k_recip<<<nblocks(N), RT_BLOCK, 0, st>>>(N, rD);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        } else if (pre == RT_PRECOND_DIAGONAL) {
            k_recip_diag<<<nblocks(N), RT_BLOCK, 0, st>>>(N, a.diag, rD);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        }
    }

    void precondition(unsigned mask, const double *rD, const double *r, double *w) {
        const DevMesh &m = ctx->mesh;
        int pre = a.ctl.preconditioner;
        if (pre == RT_PRECOND_NONE) {
            k_copy<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, r, w);
            launch_count(ctx);
        } else if (pre == RT_PRECOND_DIAGONAL) {
            k_diag_apply<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, rD, r, w);
            launch_count(ctx);
        } else if (systolic()) {
            const double fpc = (double)m.F / N;
            ProfScope ps(ctx, "dilu_precondition", (double)N * (16.0 + fpc * 32.0 + 32.0 * pop(mask)));
            skew_precondition(ctx, a.nc, mask, r, w);
        } else {
            // per application (forward + backward): rD 16, coefficients
            // 2*(F/N)*8, addressing 2*(F/N)*8, r 8 + w 8 + w 16 per component
            const double fpc = (double)m.F / N;
            ProfScope ps(ctx, "dilu_precondition", (double)N * (16.0 + fpc * 32.0 + 32.0 * pop(mask)));
            for (int l = 0; l < m.nLevels; ++l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_fwd_level<<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(e, l0, l1, m.levelCells.p, mask, rD,
                                                                   a.lower, r, w);
            }
            for (int l = m.nLevels - 1; l >= 0; --l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_bwd_level<<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(e, l0, l1, m.levelCells.p, mask, rD,
                                                                   a.upper, w);
            }
            launch_count(ctx, 2 * m.nLevels);
        }
        RT_CHECK_LAUNCH();
    }

    // shared prologue: x̄, A psi, r, normFactor, initial residual
    void prologue(unsigned mask, double *wA, double *rA) {
        k_sum<<<nB, RT_BLOCK, 0, st>>>(N, mask, a.psi, ctx->red.partial.p, nB);
        RT_CHECK_LAUNCH();
        finalize(1, mask);
        k_sc_xbar<<<1, 32, 0, st>>>(mask, N, ctx->red.result.p, S);
        k_init_res<<<nB, RT_BLOCK, 0, st>>>(e, mask, a.diag, a.upper, a.lower, a.source, a.psi, wA, rA, S,
                                            ctx->red.partial.p, nB);
        RT_CHECK_LAUNCH();
        finalize(2, mask);
        k_sc_init<<<1, 32, 0, st>>>(mask, ctx->red.result.p, S);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 4);
    }

    bool conv(double fin, double init) const {
        return fin < a.ctl.tolerance || (a.ctl.relTol > 1e-20 && fin < a.ctl.relTol * init);
    }
};

rt_status run_pcg(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    Solver sv(ctx, a);
    const int N = sv.N;
    double *ws = ctx->kws.p;
    double *wA = ws, *rA = ws + 6 * (size_t)N, *pA = ws + 12 * (size_t)N, *rD = ws + 48 * (size_t)N;
    unsigned mask = a.validMask;
    sv.compute_rd(rD);
    sv.prologue(mask, wA, rA);
    double h[2 * 8];
    RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, sv.S, sizeof(double) * 3 * 8, cudaMemcpyDeviceToHost, sv.st));
    RT_CUDA(cudaStreamSynchronize(sv.st));
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        perf[k].initialResidual = ctx->red.hostResult[S_INIT * 8 + k];
        perf[k].finalResidual = ctx->red.hostResult[S_FIN * 8 + k];
        perf[k].nIterations = 0;
        perf[k].singular = 0;
    }
    unsigned active = 0;
    for (int k = 0; k < 6; ++k)
        if (((mask >> k) & 1u) && (a.ctl.minIter > 0 || !sv.conv(perf[k].finalResidual, perf[k].initialResidual)))
            active |= 1u << k;
    int iter = 0;
    while (active) {
        sv.precondition(active, rD, rA, wA);
        sv.dot(active, wA, rA);
        k_sc_pcg_a<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);
        k_pcg_p<<<nblocks(N), RT_BLOCK, 0, sv.st>>>(N, active, iter == 0, sv.S, wA, pA);
        sv.amul(active, pA, wA);
        sv.dot(active, wA, pA);
        k_sc_pcg_alpha<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);
        k_pcg_update<<<sv.nB, RT_BLOCK, 0, sv.st>>>(N, active, sv.S, pA, wA, a.psi, rA, ctx->red.partial.p, sv.nB);
        RT_CHECK_LAUNCH();
        sv.finalize(1, active);
        k_sc_fin<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 4);
        RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, sv.S, sizeof(double) * (S_SING + 1) * 8,
                                cudaMemcpyDeviceToHost, sv.st));
        RT_CUDA(cudaStreamSynchronize(sv.st));
        const double *H = ctx->red.hostResult;
        ++iter;
        for (int k = 0; k < 6; ++k) {
            if (!((active >> k) & 1u)) continue;
            if (H[S_SING * 8 + k] != 0.0) {
                perf[k].singular = 1;
                active &= ~(1u << k);
                continue;
            }
            perf[k].finalResidual = H[S_FIN * 8 + k];
            perf[k].nIterations = iter;
            bool more = (iter < a.ctl.maxIter && !sv.conv(perf[k].finalResidual, perf[k].initialResidual)) ||
                        iter < a.ctl.minIter;
            if (!more) active &= ~(1u << k);
        }
    }
    (void)h;
    return RT_OK;
}

rt_status run_pbicgstab(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    Solver sv(ctx, a);
    const int N = sv.N;
    const size_t V6 = 6 * (size_t)N;
    double *ws = ctx->kws.p;
    double *yA = ws, *rA = ws + V6, *pA = ws + 2 * V6, *AyA = ws + 3 * V6, *sA = ws + 4 * V6,
           *zA = ws + 5 * V6, *tA = ws + 6 * V6, *rA0 = ws + 7 * V6, *rD = ws + 8 * V6;
    unsigned mask = a.validMask;
    sv.compute_rd(rD);
    sv.prologue(mask, yA, rA);
    RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, sv.S, sizeof(double) * 3 * 8, cudaMemcpyDeviceToHost, sv.st));
    RT_CUDA(cudaStreamSynchronize(sv.st));
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        perf[k].initialResidual = ctx->red.hostResult[S_INIT * 8 + k];
        perf[k].finalResidual = ctx->red.hostResult[S_FIN * 8 + k];
        perf[k].nIterations = 0;
        perf[k].singular = 0;
    }
    unsigned active = 0;
    for (int k = 0; k < 6; ++k)
        if (((mask >> k) & 1u) && (a.ctl.minIter > 0 || !sv.conv(perf[k].finalResidual, perf[k].initialResidual)))
            active |= 1u << k;
    if (!active) return RT_OK;
    RT_CUDA(cudaMemcpyAsync(rA0, rA, sizeof(double) * V6, cudaMemcpyDeviceToDevice, sv.st));
    int iter = 0;
    while (active) {
        sv.dot(active, rA0, rA);
        k_sc_bicg_r0r<<<1, 32, 0, sv.st>>>(active, iter, ctx->red.result.p, sv.S);
        k_bicg_p<<<nblocks(N), RT_BLOCK, 0, sv.st>>>(N, active, iter == 0, sv.S, rA, AyA, pA);
        sv.precondition(active, rD, pA, yA);
        sv.amul(active, yA, AyA);
        sv.dot(active, rA0, AyA);
        k_sc_bicg_alpha<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);
        k_bicg_s<<<sv.nB, RT_BLOCK, 0, sv.st>>>(N, active, sv.S, rA, AyA, sA, ctx->red.partial.p, sv.nB);
        RT_CHECK_LAUNCH();
        sv.finalize(1, active);
        k_sc_fin<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 5);
        RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, sv.S, sizeof(double) * (S_SING + 1) * 8,
                                cudaMemcpyDeviceToHost, sv.st));
        RT_CUDA(cudaStreamSynchronize(sv.st));
        double H[(S_SING + 1) * 8];
        memcpy(H, ctx->red.hostResult, sizeof H);
        unsigned finish = 0, cont = 0;
        for (int k = 0; k < 6; ++k) {
            if (!((active >> k) & 1u)) continue;
            if (H[S_SING * 8 + k] != 0.0) {
                perf[k].singular = 1;
                continue;     // stops without an update
            }
            perf[k].finalResidual = H[S_FIN * 8 + k];
            if (sv.conv(perf[k].finalResidual, perf[k].initialResidual)) {
                finish |= 1u << k;
                perf[k].nIterations = iter + 1;
            } else {
                cont |= 1u << k;
            }
        }
        if (finish) {
            k_axpy_alpha<<<nblocks(N), RT_BLOCK, 0, sv.st>>>(N, finish, sv.S, yA, a.psi);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        }
        active = cont;
        if (!active) break;
        sv.precondition(active, rD, sA, zA);
        sv.amul(active, zA, tA);
        sv.dot(active, tA, tA, tA, sA);
        k_sc_bicg_omega<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);
        k_bicg_update<<<sv.nB, RT_BLOCK, 0, sv.st>>>(N, active, sv.S, yA, zA, sA, tA, a.psi, rA,
                                                     ctx->red.partial.p, sv.nB);
        RT_CHECK_LAUNCH();
        sv.finalize(1, active);
        k_sc_fin<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 3);
        RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, sv.S, sizeof(double) * (S_SING + 1) * 8,
                                cudaMemcpyDeviceToHost, sv.st));
        RT_CUDA(cudaStreamSynchronize(sv.st));
        const double *H2 = ctx->red.hostResult;
        ++iter;
        for (int k = 0; k < 6; ++k) {
            if (!((active >> k) & 1u)) continue;
            perf[k].finalResidual = H2[S_FIN * 8 + k];
            perf[k].nIterations = iter;
            bool more = (iter < a.ctl.maxIter && !sv.conv(perf[k].finalResidual, perf[k].initialResidual)) ||
                        iter < a.ctl.minIter;
            if (!more) active &= ~(1u << k);
        }
    }
    return RT_OK;
}

}  // namespace

rt_status ldu_solve_device(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    const int N = ctx->mesh.N;
    ctx->kws.alloc(48 * (size_t)N + 2 * (size_t)N + 64);
    for (int k = 0; k < a.nc; ++k) {
        perf[k] = rt_solver_perf{};
        if (!((a.validMask >> k) & 1u)) {
            perf[k].nIterations = -1;
            perf[k].converged = 1;
        }
    }
    unsigned mask = a.validMask & ((1u << a.nc) - 1u);
    SolveArgs b = a;
    b.validMask = mask;
    rt_status st = RT_OK;
    if (mask) st = (a.ctl.solver == RT_SOLVER_PCG) ? run_pcg(ctx, b, perf) : run_pbicgstab(ctx, b, perf);
    rt_status sw = skew_check(ctx);
    if (sw != RT_OK) return sw;
    for (int k = 0; k < a.nc; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double fin = perf[k].finalResidual, init = perf[k].initialResidual;
        perf[k].converged = (fin < a.ctl.tolerance || (a.ctl.relTol > 1e-20 && fin < a.ctl.relTol * init)) ? 1 : 0;
        if (!std::isfinite(fin)) st = RT_ENAN;
    }
    return st;
}

double residual_device(rt_ctx *ctx, const double *diag, const double *upper, const double *lower,
                       const double *b, const double *x) {
    SolveArgs a{diag, upper, lower, b, const_cast<double *>(x), 1, 1u, rt_solver_ctl{}};
    Solver sv(ctx, a);
    const int N = sv.N;
    ctx->kws.alloc(48 * (size_t)N + 2 * (size_t)N + 64);
    double *wA = ctx->kws.p, *rA = ctx->kws.p + 6 * (size_t)N;
    sv.prologue(1u, wA, rA);
    RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, sv.S, sizeof(double) * 3 * 8, cudaMemcpyDeviceToHost, sv.st));
    RT_CUDA(cudaStreamSynchronize(sv.st));
    return ctx->red.hostResult[S_INIT * 8 + 0];
}

}  // namespace rt
