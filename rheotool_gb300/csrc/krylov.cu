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

#include "batch.h"
#include "real_ops.cuh"
#include "rt_internal.h"
#include "sweep.h"

namespace rt {

// scalar slots (device array ctx->scal, [slot*8 + comp])
enum {
    S_NF = 0, S_INIT, S_FIN, S_XBAR, S_A, S_B, S_AOLD, S_ALPHA, S_OMEGA,
    S_R0R, S_R0ROLD, S_SING, S_T1, S_T2, S_RST, S_ITER, S_NSLOT
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

// The ELL slots of a row are read in groups of kSG: the neighbour and face
// indices of the group first (one round of independent loads), then the
// coefficients and neighbour values (a second), then the accumulation in slot
// order.  A row ends in -1 padding, which adds nothing (the same sum as
// stopping at the row's end).
constexpr int kSG = 6;

__device__ __forceinline__ void slot_group(const Ell &e, int c, int s0, int (&nb)[kSG], int (&f)[kSG]) {
#pragma unroll
    for (int j = 0; j < kSG; ++j) {
        const bool in = s0 + j < e.nSlots;
        nb[j] = in ? e.nbr[(s0 + j) * e.N + c] : -1;
        f[j] = in ? e.face[(s0 + j) * e.N + c] : -1;
    }
}

__device__ __forceinline__ double row_mul(const Ell &e, int c, const double *__restrict__ diag,
                                          const double *__restrict__ upper,
                                          const double *__restrict__ lower,
                                          const double *__restrict__ x) {
    double acc = diag[c] * x[c];
    for (int s0 = 0; s0 < e.nSlots; s0 += kSG) {
        int nb[kSG], f[kSG];
        slot_group(e, c, s0, nb, f);
        double a[kSG], xn[kSG];
#pragma unroll
        for (int j = 0; j < kSG; ++j) {
            a[j] = nb[j] >= 0 ? (nb[j] > c ? upper[f[j]] : lower[f[j]]) : 0.0;
            xn[j] = nb[j] >= 0 ? x[nb[j]] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < kSG; ++j)
            if (nb[j] >= 0) acc += a[j] * xn[j];
    }
    return acc;
}

__device__ __forceinline__ double row_sum(const Ell &e, int c, const double *__restrict__ diag,
                                          const double *__restrict__ upper,
                                          const double *__restrict__ lower) {
    double acc = diag[c];
    for (int s0 = 0; s0 < e.nSlots; s0 += kSG) {
        int nb[kSG], f[kSG];
        slot_group(e, c, s0, nb, f);
        double a[kSG];
#pragma unroll
        for (int j = 0; j < kSG; ++j) a[j] = nb[j] >= 0 ? (nb[j] > c ? upper[f[j]] : lower[f[j]]) : 0.0;
#pragma unroll
        for (int j = 0; j < kSG; ++j)
            if (nb[j] >= 0) acc += a[j];
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
        #pragma unroll 4
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

// (templated on the real type: FP64 for the plain solvers, FP32 inside the
// mixed-precision ones)
template <class Real>
__global__ void k_fwd_level(Ell e, int l0, int l1, const int *__restrict__ cells, unsigned mask,
                            const Real *__restrict__ rD, const Real *__restrict__ lower,
                            const Real *__restrict__ r, Real *__restrict__ w) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    const int N = e.N;
    const Real rd = rD[c];
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t o = (size_t)k * N;
        Real acc = r_mul(rd, r[o + c]);
        for (int s = 0; s < e.nSlots; ++s) {
            int nb = e.nbr[s * N + c];
            if (nb < 0 || nb > c) break;
            int f = e.face[s * N + c];
            acc = r_fma(-r_mul(rd, lower[f]), w[o + nb], acc);
        }
        w[o + c] = acc;
    }
}

template <class Real>
__global__ void k_bwd_level(Ell e, int l0, int l1, const int *__restrict__ cells, unsigned mask,
                            const Real *__restrict__ rD, const Real *__restrict__ upper,
                            Real *__restrict__ w) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    const int N = e.N;
    const Real rd = rD[c];
    // number of used slots
    int ns = 0;
    while (ns < e.nSlots && e.nbr[ns * N + c] >= 0) ++ns;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t o = (size_t)k * N;
        Real acc = w[o + c];
        for (int s = ns - 1; s >= 0; --s) {
            int nb = e.nbr[s * N + c];
            if (nb < c) break;                // upper neighbours are the last slots
            int f = e.face[s * N + c];
            acc = r_fma(-r_mul(rd, upper[f]), w[o + nb], acc);
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
        #pragma unroll 4
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
        #pragma unroll 4
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
        #pragma unroll 4
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
    r.active.alloc(1);
    r.active.zero(ctx->stream);
    r.counter.alloc(1);
    r.counter.zero(ctx->stream);
    void *hf = nullptr;
    RT_CUDA(cudaHostAlloc(&hf, sizeof(int) * 4, cudaHostAllocMapped));
    r.hostFlag = static_cast<volatile int *>(hf);
    r.hostFlag[0] = 0;
    RT_CUDA(cudaHostGetDevicePointer((void **)&r.devFlag, hf, 0));
    for (cudaEvent_t &e : r.poll) RT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

// ==========================================================================
// PCG stopping on the device.  One iteration is four kernels after the
// preconditioner: k_pcg_rho (w.r, and for the flexible form w.q_old), k_pcg_pq
// (p = w + beta p into the other p buffer, q = A p with the neighbours' p
// formed on the fly, p.q), k_pcg_step (psi += alpha p, r -= alpha q, |r|).
// Each reduction's last block to arrive sums the block partials in the fixed
// order of k_finalize (so the scalars have the same bits as the host-driven
// loop) and does the scalar work: beta, alpha and the singularity test, or
// the residual, the iteration count and the stopping rules of lduMatrix's
// PCG.  Components that stop leave the device word `active`; when none is
// left the kernels and sweeps return at once and the mapped host flag drops,
// which the host polls every few iterations instead of synchronising every
// iteration.
// ==========================================================================

// true in every thread of the block that arrives last at `counter` (all
// blocks' partials are then visible); the counter is re-armed
__device__ bool last_block(unsigned *counter) {
    __shared__ bool amLast;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(counter, 1u);
        amLast = (t == gridDim.x - 1);
        if (amLast) *counter = 0u;
    }
    __syncthreads();
    return amLast;
}

// fixed-order sum of one slot's block partials (k_finalize's order), valid
// in thread 0; read past L1, since other SMs wrote them
__device__ double partials_sum(const double *partial, int nB, int slot, int k) {
    double v = 0.0;
    for (int i = threadIdx.x; i < nB; i += blockDim.x) v += __ldcg(partial + (slot * 6 + k) * nB + i);
    return block_sum(v);
}

// rho = w.r (slot 0) and, in the flexible form after the first iteration,
// w.q_old (slot 1); the last block: wArAold = wArA, wArA = rho, flexible beta
template <bool FLEX>
__global__ void k_pcg_rho(int N, unsigned mask0, const unsigned *__restrict__ active, int first,
                          const double *__restrict__ w, const double *__restrict__ r, const double *__restrict__ qold,
                          double *S, double *partial, int nB, unsigned *counter) {
    const unsigned mask = mask0 & *active;
    if (!mask) return;
    const bool two = FLEX && !first;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        double v0 = 0.0, v1 = 0.0;
        size_t o = (size_t)k * N;
        #pragma unroll 4
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            v0 += w[o + c] * r[o + c];
            if (two) v1 += w[o + c] * qold[o + c];
        }
        store_partial(partial, nB, 0, k, v0);
        if (two) store_partial(partial, nB, 1, k, v1);
    }
    if (!last_block(counter)) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double rho = partials_sum(partial, nB, 0, k);
        const double wq = two ? partials_sum(partial, nB, 1, k) : 0.0;
        if (threadIdx.x == 0) {
            const double aold = S[S_A * 8 + k];
            S[S_AOLD * 8 + k] = aold;
            S[S_A * 8 + k] = rho;
            if (two) S[S_B * 8 + k] = -S[S_ALPHA * 8 + k] * wq / aold;
        }
    }
}

// p_new = w (+ beta p_old); q = A p_new, the neighbours' p_new formed from
// their w and p_old exactly as the cell's own; p.q; the last block: alpha =
// wArA / wApA or the singularity test
template <bool FLEX>
__global__ void k_pcg_pq(Ell e, unsigned mask0, const unsigned *__restrict__ active, int first,
                         const double *__restrict__ diag, const double *__restrict__ upper,
                         const double *__restrict__ lower, const double *__restrict__ w,
                         const double *__restrict__ pold, double *__restrict__ pnew, double *__restrict__ q, double *S,
                         double *partial, int nB, unsigned *counter) {
    const unsigned mask = mask0 & *active;
    if (!mask) return;
    const int N = e.N;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double beta = first ? 0.0 : (FLEX ? S[S_B * 8 + k] : S[S_A * 8 + k] / S[S_AOLD * 8 + k]);
        const size_t o = (size_t)k * N;
        const double *wk = w + o, *pk = pold + o;
        double v = 0.0;
#pragma unroll 2
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            const double pc = first ? wk[c] : fma(beta, pk[c], wk[c]);
            double acc = diag[c] * pc;
            for (int s0 = 0; s0 < e.nSlots; s0 += kSG) {
                int nb[kSG], f[kSG];
                slot_group(e, c, s0, nb, f);
                double a[kSG], wn[kSG], pn[kSG];
#pragma unroll
                for (int j = 0; j < kSG; ++j) {
                    a[j] = nb[j] >= 0 ? (nb[j] > c ? upper[f[j]] : lower[f[j]]) : 0.0;
                    wn[j] = nb[j] >= 0 ? wk[nb[j]] : 0.0;
                    pn[j] = (nb[j] >= 0 && !first) ? pk[nb[j]] : 0.0;
                }
#pragma unroll
                for (int j = 0; j < kSG; ++j)
                    if (nb[j] >= 0) acc = fma(a[j], first ? wn[j] : fma(beta, pn[j], wn[j]), acc);
            }
            pnew[o + c] = pc;
            q[o + c] = acc;
            v = fma(acc, pc, v);
        }
        store_partial(partial, nB, 0, k, v);
    }
    if (!last_block(counter)) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double wApA = partials_sum(partial, nB, 0, k);
        if (threadIdx.x == 0) {
            if (fabs(wApA) / S[S_NF * 8 + k] < 1e-300) {
                S[S_SING * 8 + k] = 1.0;
                S[S_ALPHA * 8 + k] = 0.0;
            } else {
                S[S_ALPHA * 8 + k] = S[S_A * 8 + k] / wApA;
            }
        }
    }
}

// psi += alpha p; r -= alpha q; |r|; the last block: residual, iteration
// count and lduMatrix's stopping rules per component (a singular component
// stops without an update, keeping its last residual and count)
__global__ void k_pcg_step(int N, unsigned mask0, unsigned *active, rt_solver_ctl ctl, const double *__restrict__ p,
                           const double *__restrict__ q, double *__restrict__ psi, double *__restrict__ r, double *S,
                           double *partial, int nB, unsigned *counter, int *hostFlag) {
    const unsigned mask = mask0 & *active;
    if (!mask) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const bool sing = S[S_SING * 8 + k] != 0.0;
        const double alpha = S[S_ALPHA * 8 + k];
        double v = 0.0;
        size_t o = (size_t)k * N;
        #pragma unroll 4
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            if (!sing) {
                psi[o + c] += alpha * p[o + c];
                r[o + c] -= alpha * q[o + c];
            }
            v += fabs(r[o + c]);
        }
        store_partial(partial, nB, 0, k, v);
    }
    if (!last_block(counter)) return;
    unsigned next = mask;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const double res = partials_sum(partial, nB, 0, k);
        if (threadIdx.x == 0) {
            if (S[S_SING * 8 + k] != 0.0) {
                next &= ~(1u << k);
            } else {
                const double fin = res / S[S_NF * 8 + k], init = S[S_INIT * 8 + k];
                const double it = S[S_ITER * 8 + k] + 1.0;
                S[S_FIN * 8 + k] = fin;
                S[S_ITER * 8 + k] = it;
                const bool conv = fin < ctl.tolerance || (ctl.relTol > 1e-20 && fin < ctl.relTol * init);
                const bool more = (it < ctl.maxIter && !conv) || it < ctl.minIter;
                if (!more || !isfinite(fin)) next &= ~(1u << k);
            }
        }
    }
    if (threadIdx.x == 0) {
        *active = (*active & ~mask0) | next;
        if (!*active) {
            *(volatile int *)hostFlag = 0;
            __threadfence_system();
        }
    }
}

// the loop's starting state: the components to iterate, zero iterations
__global__ void k_pcg_arm(unsigned act, unsigned *active, double *S) {
    const int k = threadIdx.x;
    if (k < 6) {
        S[S_ITER * 8 + k] = 0.0;
        S[S_SING * 8 + k] = 0.0;
    }
    if (k == 0) *active = act;
}

namespace {

struct Solver {
    rt_ctx *ctx;
    Ell e;    // the matrix (every internal face)
    Ell pe;   // the DIC/DILU factorisation and sweeps (coupled faces left out)
    int N;
    cudaStream_t st;
    const SolveArgs &a;
    double *S;
    int nB;

    Solver(rt_ctx *c, const SolveArgs &args) : ctx(c), a(args) {
        const DevMesh &m = ctx->mesh;
        N = m.N;
        e = Ell{m.N, m.nSlots, m.ellFace.p, m.ellNbr.p};
        pe = m.hasCoupled ? Ell{m.N, m.pnSlots, m.pellFace.p, m.pellNbr.p} : e;
        st = ctx->stream;
        S = ctx->scal.p;
        nB = ctx->red.nBlocks;
    }

    // finalize nSlots reduction slots of the masked comps into red.result
    void finalize(int nSlots, unsigned mask) {
        // blocks beyond rblocks() left stale partials: zero them by using only
        // the first rblocks() entries — the reduction kernels always launch
        // exactly nB blocks, so all entries are written.
        k_finalize<<<nSlots * 6, RT_BLOCK, 0, st>>>(nB, nSlots, mask, ctx->red.partial.p, ctx->red.result.p);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }

    static int pop(unsigned m) { return __builtin_popcount(m); }

    // y = A x, or with T the transposed product A^T x (coefficients exchanged)
    void amul(unsigned mask, const double *x, double *y, bool T = false) {
        // algorithmic bytes per cell: diag 8, lower+upper 2*(F/N)*8, face
        // addressing 2*(F/N)*4, x and y 16 per component
        const double fpc = (double)ctx->mesh.F / N;
        ProfScope ps(ctx, "amul", (double)N * (8.0 + fpc * 24.0 + 16.0 * pop(mask)));
        k_amul<<<nblocks(N), RT_BLOCK, 0, st>>>(e, mask, a.diag, T ? a.lower : a.upper, T ? a.upper : a.lower, x, y);
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
                k_rd_level<<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(pe, l0, l1, m.levelCells.p, a.diag,
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

    // w = M^-1 r, or with T the transposed preconditioner M^-T r (the same rD,
    // the lower and upper coefficients exchanged; PBiCG's shadow system)
    // (dmask: the device word of the components still iterating, or null;
    // the systolic sweeps return at once when it is empty)
    void precondition(unsigned mask, const double *rD, const double *r, double *w, bool T = false,
                      const unsigned *dmask = nullptr) {
        const DevMesh &m = ctx->mesh;
        int pre = a.ctl.preconditioner;
        const double *lower = T ? a.upper : a.lower, *upper = T ? a.lower : a.upper;
        if (pre == RT_PRECOND_NONE) {
            k_copy<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, r, w);
            launch_count(ctx);
        } else if (pre == RT_PRECOND_DIAGONAL) {
            k_diag_apply<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, rD, r, w);
            launch_count(ctx);
        } else if (systolic()) {
            // per application: rD 8, coefficients 2*(F/N)*8 (premultiplied,
            // no addressing), r 8 + w 8 + the forward result 16 per component
            const double fpc = (double)m.F / N;
            ProfScope ps(ctx, "dilu_precondition", (double)N * (8.0 + fpc * 16.0 + 32.0 * pop(mask)));
            if (T) skew_precondition_T(ctx, a.nc, mask, r, w);
            else skew_precondition(ctx, a.nc, mask, r, w, dmask);
        } else {
            // per application (forward + backward): rD 16, coefficients
            // 2*(F/N)*8, addressing 2*(F/N)*8, r 8 + w 8 + w 16 per component
            const double fpc = (double)m.F / N;
            ProfScope ps(ctx, "dilu_precondition", (double)N * (16.0 + fpc * 32.0 + 32.0 * pop(mask)));
            for (int l = 0; l < m.nLevels; ++l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_fwd_level<<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(pe, l0, l1, m.levelCells.p, mask, rD,
                                                                   lower, r, w);
            }
            for (int l = m.nLevels - 1; l >= 0; --l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_bwd_level<<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(pe, l0, l1, m.levelCells.p, mask, rD,
                                                                   upper, w);
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

// PCG (FLEX = false: FP64, DIC in FP64; FLEX = true: the mixed form's
// flexible PCG with the FP32 DIC of Mixed::precondition32d) with the stopping
// decisions on the device.  The host launches iterations ahead and polls the
// mapped flag every kPoll iterations, after waiting for the iterations
// launched kPoll earlier, so it stays at most 2 kPoll iterations ahead; the
// iterations launched after the last component stopped return at once.
constexpr int kPoll = 8;

template <bool FLEX, class Pre>
rt_status pcg_device_loop(rt_ctx *ctx, Solver &sv, const SolveArgs &a, rt_solver_perf *perf, Pre &&precondition) {
    const int N = sv.N;
    const size_t V6 = 6 * (size_t)N;
    double *ws = ctx->kws.p;
    double *q = ws, *rA = ws + V6, *pbuf[2] = {ws + 2 * V6, ws + 4 * V6}, *z = ws + 3 * V6;
    const unsigned mask = a.validMask;
    Reduce &red = ctx->red;
    RT_CUDA(cudaMemcpyAsync(red.hostResult, sv.S, sizeof(double) * 3 * 8, cudaMemcpyDeviceToHost, sv.st));
    RT_CUDA(cudaStreamSynchronize(sv.st));
    unsigned act = 0;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        perf[k].initialResidual = red.hostResult[S_INIT * 8 + k];
        perf[k].finalResidual = red.hostResult[S_FIN * 8 + k];
        perf[k].nIterations = 0;
        perf[k].singular = 0;
        if (a.ctl.minIter > 0 || !sv.conv(perf[k].finalResidual, perf[k].initialResidual)) act |= 1u << k;
    }
    if (!act) return RT_OK;
    k_pcg_arm<<<1, 32, 0, sv.st>>>(act, red.active.p, sv.S);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    red.hostFlag[0] = 1;
    const int maxIt = std::max(a.ctl.maxIter, a.ctl.minIter);
    const double fpc = (double)ctx->mesh.F / N;
    for (int it = 0; it < maxIt; ++it) {
        const int first = it == 0;
        double *pold = pbuf[it & 1], *pnew = pbuf[(it + 1) & 1];
        precondition(act, rA, z, red.active.p);
        {
            ProfScope ps(ctx, "dot", (double)N * 8.0 * ((FLEX && !first) ? 3 : 2) * sv.pop(act));
            k_pcg_rho<FLEX><<<sv.nB, RT_BLOCK, 0, sv.st>>>(N, act, red.active.p, first, z, rA, q, sv.S,
                                                             red.partial.p, sv.nB, red.counter.p);
            RT_CHECK_LAUNCH();
        }
        {
            // the amul's bytes, plus w and p_old read and p written per component
            ProfScope ps(ctx, "amul", (double)N * (8.0 + fpc * 24.0 + 40.0 * sv.pop(act)));
            k_pcg_pq<FLEX><<<sv.nB, RT_BLOCK, 0, sv.st>>>(sv.e, act, red.active.p, first, a.diag, a.upper, a.lower, z,
                                                            pold, pnew, q, sv.S, red.partial.p, sv.nB, red.counter.p);
            RT_CHECK_LAUNCH();
        }
        {
            ProfScope ps(ctx, "pcg_update", (double)N * 40.0 * sv.pop(act));
            k_pcg_step<<<sv.nB, RT_BLOCK, 0, sv.st>>>(N, act, red.active.p, a.ctl, pnew, q, a.psi, rA, sv.S,
                                                      red.partial.p, sv.nB, red.counter.p, red.devFlag);
            RT_CHECK_LAUNCH();
        }
        launch_count(ctx, 3);
        if ((it + 1) % kPoll == 0) {
            const int b = (it + 1) / kPoll;
            RT_CUDA(cudaEventRecord(red.poll[b & 1], sv.st));
            if (b >= 2) {
                RT_CUDA(cudaEventSynchronize(red.poll[(b - 1) & 1]));
                if (red.hostFlag[0] == 0) break;
            }
        }
    }
    RT_CUDA(cudaMemcpyAsync(red.hostResult, sv.S, sizeof(double) * (S_ITER + 1) * 8, cudaMemcpyDeviceToHost, sv.st));
    RT_CUDA(cudaStreamSynchronize(sv.st));
    const double *H = red.hostResult;
    for (int k = 0; k < 6; ++k) {
        if (!((act >> k) & 1u)) continue;
        perf[k].finalResidual = H[S_FIN * 8 + k];
        perf[k].nIterations = (int)H[S_ITER * 8 + k];
        perf[k].singular = H[S_SING * 8 + k] != 0.0 ? 1 : 0;
    }
    return RT_OK;
}

rt_status run_pcg(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    Solver sv(ctx, a);
    double *rD = ctx->kws.p + 48 * (size_t)sv.N;
    sv.compute_rd(rD);
    sv.prologue(a.validMask, ctx->kws.p, ctx->kws.p + 6 * (size_t)sv.N);
    return pcg_device_loop<false>(ctx, sv, a, perf, [&](unsigned act, const double *r, double *w, const unsigned *dm) {
        sv.precondition(act, rD, r, w, false, dm);
    });
}

// rT = b - A^T psi on the masked components
__global__ void k_sub(int N, unsigned mask, const double *__restrict__ b, const double *__restrict__ y,
                      double *__restrict__ r) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) r[(size_t)k * N + c] = b[(size_t)k * N + c] - y[(size_t)k * N + c];
}

// PBiCG: pA = wA (+ beta pA), pT = wT (+ beta pT), beta = wArT / wArTold
__global__ void k_pbicg_p(int N, unsigned mask, int first, const double *__restrict__ S,
                          const double *__restrict__ wA, const double *__restrict__ wT, double *__restrict__ pA,
                          double *__restrict__ pT) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t i = (size_t)k * N + c;
        if (first) {
            pA[i] = wA[i];
            pT[i] = wT[i];
        } else {
            double beta = S[S_A * 8 + k] / S[S_AOLD * 8 + k];
            pA[i] = wA[i] + beta * pA[i];
            pT[i] = wT[i] + beta * pT[i];
        }
    }
}

// PBiCG: psi += alpha pA; rA -= alpha wA; rT -= alpha wT; partial |rA|
__global__ void k_pbicg_update(int N, unsigned mask, const double *__restrict__ S, const double *__restrict__ pA,
                               const double *__restrict__ wA, const double *__restrict__ wT,
                               double *__restrict__ psi, double *__restrict__ rA, double *__restrict__ rT,
                               double *partial, int nB) {
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
                rT[o + c] -= alpha * wT[o + c];
            }
            v += fabs(rA[o + c]);
        }
        store_partial(partial, nB, 0, k, v);
    }
}

// Preconditioned bi-conjugate gradients, OpenFOAM's PBiCG (the U and theta
// solver of rheoTool's Contraction41 tutorials, fvSolution:32,47): the
// shadow system is the transposed one with the same source (rT = b - A^T
// psi), preconditioned by the transposed DILU factorisation; per iteration
// wA = M^-1 rA, wT = M^-T rT, wArT = wA.rT, pA/pT updates with beta =
// wArT/wArTold, wA = A pA, wT = A^T pT, alpha = wArT / (wA.pT).  Stopping
// and singularity rules as run_pcg.
rt_status run_pbicg(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    Solver sv(ctx, a);
    const int N = sv.N;
    const size_t V6 = 6 * (size_t)N;
    double *ws = ctx->kws.p;
    double *wA = ws, *rA = ws + V6, *pA = ws + 2 * V6, *wT = ws + 3 * V6, *rT = ws + 4 * V6, *pT = ws + 5 * V6,
           *rD = ws + 48 * (size_t)N;
    const unsigned mask = a.validMask;
    sv.compute_rd(rD);
    if (sv.systolic()) skew_prepare_T(ctx, a.upper, a.lower);
    sv.prologue(mask, wA, rA);
    sv.amul(mask, a.psi, wT, true);
    k_sub<<<nblocks(N), RT_BLOCK, 0, sv.st>>>(N, mask, a.source, wT, rT);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
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
        sv.precondition(active, rD, rT, wT, true);
        sv.dot(active, wA, rT);
        k_sc_pcg_a<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);   // wArTold, wArT
        k_pbicg_p<<<nblocks(N), RT_BLOCK, 0, sv.st>>>(N, active, iter == 0, sv.S, wA, wT, pA, pT);
        sv.amul(active, pA, wA);
        sv.amul(active, pT, wT, true);
        sv.dot(active, wA, pT);
        k_sc_pcg_alpha<<<1, 32, 0, sv.st>>>(active, ctx->red.result.p, sv.S);   // singularity, alpha
        k_pbicg_update<<<sv.nB, RT_BLOCK, 0, sv.st>>>(N, active, sv.S, pA, wA, wT, a.psi, rA, rT,
                                                      ctx->red.partial.p, sv.nB);
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
            if (!more || !std::isfinite(perf[k].finalResidual)) active &= ~(1u << k);
        }
    }
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
            } else if (!std::isfinite(perf[k].finalResidual)) {
                perf[k].nIterations = iter + 1;   // stops (RT_ENAN follows)
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
            if (!more || !std::isfinite(perf[k].finalResidual)) active &= ~(1u << k);
        }
    }
    return RT_OK;
}


// ==========================================================================
// Mixed precision (RT_PREC_MIXED).  PBiCGStab (momentum and theta): the
// Krylov vectors, the matrix copy used inside the iterations and the
// preconditioner application are FP32; the scalars, the dot-product
// accumulations, the solution and the normalised residual stay FP64.  The
// solution is kept as psi (FP64) + x32 (an FP32 correction accumulated since
// the last residual replacement).  Whenever the recursively updated FP32
// residual has dropped by kReplace since the last replacement, claims
// convergence, or the iteration budget ends, x32 is folded into psi and the
// residual is recomputed from the FP64 matrix as b - A psi (reliable updates,
// Sleijpen & van der Vorst 1996; van der Vorst & Ye 2000).  Convergence is
// only ever declared on that FP64 residual, with the normFactor of the FP64
// prologue.  PCG (pressure) keeps FP64 vectors and applies only the DIC
// preconditioner in FP32 (run_pcg_flex32): the pressure matrix is too
// ill-conditioned for FP32 Krylov vectors to keep their conjugacy.
// ==========================================================================
constexpr double kReplace = 0.1;

// FP32 copy of the matrix in the differences form: the off-diagonal
// coefficients rounded, and instead of the diagonal the FP64 row sum rounded
// once.  A x = rowsum_c x_c + sum_f a_f (x_nb - x_c) is the same product, but
// the rounding no longer breaks the (near-)zero row sums of an assembled
// OpenFOAM matrix (negSumDiag), which would move the near-null space of a
// pressure matrix by far more than its smallest eigenvalue.
__global__ void k_mx_mat32(Ell e, int F, const double *__restrict__ diag, const double *__restrict__ upper,
                           const double *__restrict__ lower, float *__restrict__ d32, float *__restrict__ u32,
                           float *__restrict__ l32) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < e.N) d32[i] = (float)row_sum(e, i, diag, upper, lower);
    if (i < F) {
        u32[i] = (float)upper[i];
        l32[i] = (float)lower[i];
    }
}

__global__ void k_mx_to32(int n, const double *__restrict__ a, float *__restrict__ b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// r32 = rA (FP64 prologue residual), x32 = 0, no restart pending
__global__ void k_mx_start(int N, unsigned mask, const double *__restrict__ rA, float *__restrict__ r32,
                           float *__restrict__ x32, double *S) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < 6 && ((mask >> c) & 1u)) S[S_RST * 8 + c] = 0.0;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        r32[(size_t)k * N + c] = (float)rA[(size_t)k * N + c];
        x32[(size_t)k * N + c] = 0.0f;
    }
}

// y_c = rowsum_c x_c + sum_f a_f (x_nb - x_c)   (differences form, see k_mx_mat32)
__device__ __forceinline__ float row_mul32(const Ell &e, int c, const float *__restrict__ rowsum,
                                           const float *__restrict__ upper, const float *__restrict__ lower,
                                           const float *__restrict__ x) {
    const float xc = x[c];
    float acc = rowsum[c] * xc;
    for (int s = 0; s < e.nSlots; ++s) {
        int nb = e.nbr[s * e.N + c];
        if (nb < 0) break;
        int f = e.face[s * e.N + c];
        acc = fmaf(nb > c ? upper[f] : lower[f], x[nb] - xc, acc);
    }
    return acc;
}

__global__ void k_mx_amul(Ell e, unsigned mask, const float *__restrict__ diag, const float *__restrict__ upper,
                          const float *__restrict__ lower, const float *__restrict__ x, float *__restrict__ y) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= e.N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        y[(size_t)k * e.N + c] = row_mul32(e, c, diag, upper, lower, x + (size_t)k * e.N);
    }
}

// dot products of FP32 vectors accumulated in FP64: slot0 = a.b, slot1 = c.d
__global__ void k_mx_dot(int N, unsigned mask, const float *__restrict__ a, const float *__restrict__ b,
                         const float *__restrict__ c2, const float *__restrict__ d2, double *partial, int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        double v0 = 0.0, v1 = 0.0;
        size_t o = (size_t)k * N;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            v0 += (double)a[o + c] * (double)b[o + c];
            if (c2) v1 += (double)c2[o + c] * (double)d2[o + c];
        }
        store_partial(partial, nB, 0, k, v0);
        if (c2) store_partial(partial, nB, 1, k, v1);
    }
}

__global__ void k_mx_copy(int N, unsigned mask, const float *__restrict__ r, float *__restrict__ w) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) w[(size_t)k * N + c] = r[(size_t)k * N + c];
}

__global__ void k_mx_diag_apply(int N, unsigned mask, const float *__restrict__ rD, const float *__restrict__ r,
                                float *__restrict__ w) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) w[(size_t)k * N + c] = rD[c] * r[(size_t)k * N + c];
}

// flexible PCG scalars: wArAold = wArA; wArA = w.r; beta = w.(r - r_old) /
// wArAold = -alpha_old w.q_old / wArAold, since r - r_old = -alpha_old q_old
// (Polak-Ribiere form; equal to wArA / wArAold in exact arithmetic, robust to
// the FP32 preconditioner, which is not exactly the same operator twice)
__global__ void k_mx_sc_pcg_a(unsigned mask, int first, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) {
        const double aold = S[S_A * 8 + k];
        S[S_AOLD * 8 + k] = aold;
        S[S_A * 8 + k] = res[k];
        if (!first) S[S_B * 8 + k] = -S[S_ALPHA * 8 + k] * res[6 + k] / aold;
    }
}

// flexible PCG: p = z (+ beta p), beta from k_mx_sc_pcg_a
__global__ void k_pcg_p_flex(int N, unsigned mask, int first, const double *__restrict__ S,
                             const double *__restrict__ z, double *__restrict__ p) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t i = (size_t)k * N + c;
        p[i] = first ? z[i] : fma(S[S_B * 8 + k], p[i], z[i]);
    }
}

// FP64 <-> FP32 copies of the masked components
__global__ void k_mx_d2f(int N, unsigned mask, const double *__restrict__ a, float *__restrict__ b) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) b[(size_t)k * N + c] = (float)a[(size_t)k * N + c];
}
__global__ void k_mx_f2d(int N, unsigned mask, const float *__restrict__ a, double *__restrict__ b) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) b[(size_t)k * N + c] = (double)a[(size_t)k * N + c];
}

// psi += x32; x32 = 0
__global__ void k_mx_fold(int N, unsigned mask, float *__restrict__ x32, double *__restrict__ psi) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        size_t i = (size_t)k * N + c;
        psi[i] += (double)x32[i];
        x32[i] = 0.0f;
    }
}

// r32 = b - A psi from the FP64 matrix; partial |b - A psi| (slot 0)
__global__ void k_mx_true_res(Ell e, unsigned mask, const double *__restrict__ diag,
                              const double *__restrict__ upper, const double *__restrict__ lower,
                              const double *__restrict__ b, const double *__restrict__ psi,
                              float *__restrict__ r32, double *partial, int nB) {
    const int N = e.N;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        double v = 0.0;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            const double r = b[(size_t)k * N + c] - row_mul(e, c, diag, upper, lower, psi + (size_t)k * N);
            r32[(size_t)k * N + c] = (float)r;
            v += fabs(r);
        }
        store_partial(partial, nB, 0, k, v);
    }
}

// BiCGStab: p = r (first iteration or restart) or r + beta (p - omega Ay)
__global__ void k_mx_bicg_p(int N, unsigned mask, int first, const double *__restrict__ S,
                            const float *__restrict__ r, const float *__restrict__ Ay, float *__restrict__ p) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        if (S[S_SING * 8 + k] != 0.0) continue;
        size_t i = (size_t)k * N + c;
        if (first || S[S_RST * 8 + k] != 0.0) p[i] = r[i];
        else {
            const float beta = (float)S[S_B * 8 + k], omega = (float)S[S_OMEGA * 8 + k];
            p[i] = fmaf(beta, fmaf(-omega, Ay[i], p[i]), r[i]);
        }
    }
}

// BiCGStab: alpha = r0r / (r0 . Ay); a pending restart is consumed
__global__ void k_mx_sc_bicg_alpha(unsigned mask, const double *res, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) {
        S[S_ALPHA * 8 + k] = S[S_R0R * 8 + k] / res[k];
        S[S_RST * 8 + k] = 0.0;
    }
}

__global__ void k_mx_set_rst(unsigned mask, double *S) {
    int k = threadIdx.x;
    if (k < 6 && ((mask >> k) & 1u)) S[S_RST * 8 + k] = 1.0;
}

// BiCGStab: s = r - alpha Ay; partial |s|
__global__ void k_mx_bicg_s(int N, unsigned mask, const double *__restrict__ S, const float *__restrict__ r,
                            const float *__restrict__ Ay, float *__restrict__ s, double *partial, int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const float alpha = (float)S[S_ALPHA * 8 + k];
        double v = 0.0;
        size_t o = (size_t)k * N;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            const float sv = fmaf(-alpha, Ay[o + c], r[o + c]);
            s[o + c] = sv;
            v += fabs((double)sv);
        }
        store_partial(partial, nB, 0, k, v);
    }
}

// x32 += alpha y
__global__ void k_mx_axpy_alpha(int N, unsigned mask, const double *__restrict__ S, const float *__restrict__ y,
                                float *__restrict__ x) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((mask >> k) & 1u) {
            size_t i = (size_t)k * N + c;
            x[i] = fmaf((float)S[S_ALPHA * 8 + k], y[i], x[i]);
        }
}

// x32 += alpha y + omega z; r = s - omega t; partial |r|
__global__ void k_mx_bicg_update(int N, unsigned mask, const double *__restrict__ S, const float *__restrict__ y,
                                 const float *__restrict__ z, const float *__restrict__ s,
                                 const float *__restrict__ t, float *__restrict__ x, float *__restrict__ r,
                                 double *partial, int nB) {
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const float alpha = (float)S[S_ALPHA * 8 + k], omega = (float)S[S_OMEGA * 8 + k];
        double v = 0.0;
        size_t o = (size_t)k * N;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
            x[o + c] = fmaf(alpha, y[o + c], fmaf(omega, z[o + c], x[o + c]));
            const float rv = fmaf(-omega, t[o + c], s[o + c]);
            r[o + c] = rv;
            v += fabs((double)rv);
        }
        store_partial(partial, nB, 0, k, v);
    }
}

// --------------------------------------------------------------------------
// DIC/DILU applied by Jacobi sweeps (RT_OPT_MIXED_PRECOND = m): the forward
// solve (I + rD L) y = rD r by m sweeps y <- rD r - rD L y from y = rD r,
// then the backward (I + rD U) z = y by m sweeps z <- y - rD U z from z = y;
// the truncated Neumann series of the same factorisation (Anzt, Chow and
// Dongarra 2015), symmetric positive definite for DIC.  FP32 vectors and
// premultiplied FP32 coefficients over the split lower / upper adjacency;
// one component (the pressure solve).
// --------------------------------------------------------------------------
// lo[j][c] = rD_c a (lower neighbour j), up[j][c] = rD_c a (upper neighbour j)
__global__ void k_jac_coef(int N, int nLo, int nUp, const int *__restrict__ plFace, const int *__restrict__ puFace,
                           const double *__restrict__ rDc, const double *__restrict__ upper,
                           const double *__restrict__ lower, float *__restrict__ rD32, float *__restrict__ lo,
                           float *__restrict__ up) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const double rd = rDc[c];
    rD32[c] = (float)rd;
    for (int j = 0; j < nLo; ++j) {
        const int f = plFace[(size_t)j * N + c];
        lo[(size_t)j * N + c] = f >= 0 ? (float)(rd * lower[f]) : 0.0f;
    }
    for (int j = 0; j < nUp; ++j) {
        const int f = puFace[(size_t)j * N + c];
        up[(size_t)j * N + c] = f >= 0 ? (float)(rd * upper[f]) : 0.0f;
    }
}

// the first forward sweep: y0 = rD r (kept) and y1 = y0 - rD L y0, the
// neighbours' y0 formed on the fly; m = 0: w = y0 (FP64 out)
__global__ void k_jac_first(int N, int nLo, const int *__restrict__ nbr, const float *__restrict__ lo,
                            const float *__restrict__ rD32, const double *__restrict__ r, float *__restrict__ y0,
                            float *__restrict__ y1, double *__restrict__ w, const unsigned *__restrict__ dmask) {
    if (dmask && !*dmask) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const float b = rD32[c] * (float)r[c];
    if (!y1) {
        w[c] = (double)b;
        return;
    }
    float acc = b;
    for (int j = 0; j < nLo; ++j) {
        const int nb = nbr[(size_t)j * N + c];
        if (nb < 0) break;
        acc = fmaf(-lo[(size_t)j * N + c], rD32[nb] * (float)r[nb], acc);
    }
    y0[c] = b;
    y1[c] = acc;
}

// one sweep: out = base - sum_j coef_j y_in(nb_j); FP64 out when w is set
__global__ void k_jac_sweep(int N, int nS, const int *__restrict__ nbr, const float *__restrict__ coef,
                            const float *__restrict__ base, const float *__restrict__ yin, float *__restrict__ yout,
                            double *__restrict__ w, const unsigned *__restrict__ dmask) {
    if (dmask && !*dmask) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float acc = base[c];
    for (int j = 0; j < nS; ++j) {
        const int nb = nbr[(size_t)j * N + c];
        if (nb < 0) break;
        acc = fmaf(-coef[(size_t)j * N + c], yin[nb], acc);
    }
    if (w) w[c] = (double)acc;
    else yout[c] = acc;
}

// --------------------------------------------------------------------------
// DIC of the two-colour (red-black) ordering of a structured mesh
// (RT_OPT_MIXED_PRECOND = -1).  Every neighbour of a red cell is black and
// comes after it, every neighbour of a black cell is red and comes before:
// rD is a_cc on red cells and a_cc - sum a_cn a_nc / a_nn on black ones, and
// an application is two parallel passes, FP32 arithmetic with an FP64 right-
// hand side and result: black cells w = (r - sum a w_red) / rD with w_red =
// r / rD formed on the fly, then red cells w = (r - sum a w_black) / rD.
// --------------------------------------------------------------------------
__global__ void k_rb_rd(Ell e, const unsigned char *__restrict__ colour, const double *__restrict__ diag,
                        const double *__restrict__ upper, const double *__restrict__ lower,
                        float *__restrict__ rDinv) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= e.N) return;
    double rd = diag[c];
    if (colour[c]) {
        for (int s = 0; s < e.nSlots; ++s) {
            const int nb = e.nbr[s * e.N + c];
            if (nb < 0) break;
            const int f = e.face[s * e.N + c];
            rd -= upper[f] * lower[f] / diag[nb];
        }
    }
    rDinv[c] = (float)(1.0 / rd);
}

// pass 1: the black cells (FP32 copy kept for pass 2, FP64 result)
__global__ void k_rb_black(Ell e, const unsigned char *__restrict__ colour, const float *__restrict__ rDinv,
                           const float *__restrict__ upper, const float *__restrict__ lower,
                           const double *__restrict__ r, float *__restrict__ wb, double *__restrict__ w,
                           const unsigned *__restrict__ dmask) {
    if (dmask && !*dmask) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= e.N || !colour[c]) return;
    float acc = (float)r[c];
    for (int s = 0; s < e.nSlots; ++s) {
        const int nb = e.nbr[s * e.N + c];
        if (nb < 0) break;
        const int f = e.face[s * e.N + c];
        acc = fmaf(-(nb > c ? upper[f] : lower[f]), rDinv[nb] * (float)r[nb], acc);
    }
    const float v = rDinv[c] * acc;
    wb[c] = v;
    w[c] = (double)v;
}

// pass 2: the red cells
__global__ void k_rb_red(Ell e, const unsigned char *__restrict__ colour, const float *__restrict__ rDinv,
                         const float *__restrict__ upper, const float *__restrict__ lower,
                         const double *__restrict__ r, const float *__restrict__ wb, double *__restrict__ w,
                         const unsigned *__restrict__ dmask) {
    if (dmask && !*dmask) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= e.N || colour[c]) return;
    float acc = (float)r[c];
    for (int s = 0; s < e.nSlots; ++s) {
        const int nb = e.nbr[s * e.N + c];
        if (nb < 0) break;
        const int f = e.face[s * e.N + c];
        acc = fmaf(-(nb > c ? upper[f] : lower[f]), wb[nb], acc);
    }
    w[c] = (double)(rDinv[c] * acc);
}

// FP32 state of one mixed solve
struct Mixed : Solver {
    float *d32, *u32, *l32, *rD32;   // matrix copy, preconditioner diagonal
    float *vec;                      // FP32 vectors, 6N each
    double *rD64;

    Mixed(rt_ctx *c, const SolveArgs &args, int nVec) : Solver(c, args) {
        const size_t V6 = 6 * (size_t)N, F = ctx->mesh.F;
        ctx->kws32.alloc(9 * V6 + 2 * (size_t)N + 2 * F + 256);
        float *p = ctx->kws32.p;
        vec = p;
        d32 = p + 9 * V6;
        rD32 = d32 + N;
        u32 = rD32 + N;
        l32 = u32 + F;
        rD64 = ctx->kws.p + 48 * (size_t)N;
        (void)nVec;
    }
    float *v(int i) const { return vec + (size_t)i * 6 * N; }

    // FP32 matrix copy and FP32 preconditioner from the FP64 factorisation
    void prepare() {
        const int F = ctx->mesh.F;
        {
            ProfScope ps(ctx, "mixed_convert", (double)N * 12.0 + (double)F * 24.0);
            k_mx_mat32<<<nblocks(std::max(N, F)), RT_BLOCK, 0, st>>>(e, F, a.diag, a.upper, a.lower, d32, u32, l32);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        }
        const int pre = a.ctl.preconditioner;
        if (multigrid()) {
            ProfScope ps(ctx, "mg_setup", (double)N * (8.0 + 3.0 * 8.0 + 16.0 + 12.0));
            mg_prepare(ctx, a.diag, a.upper, a.lower, true);
        } else if (multigridU()) {
            ProfScope ps(ctx, "mg_setup", (double)N * (8.0 + 6.0 * 8.0 + 28.0 + 24.0));
            mg_prepare(ctx, a.diag, a.upper, a.lower, false);
        } else if (redblack()) {
            if (ctx->jac.n < 2 * (size_t)N) ctx->jac.alloc(2 * (size_t)N);
            ProfScope ps(ctx, "dilu_rD", (double)N * (8.0 + 8.0 + 4.0) + (double)ctx->mesh.F * 16.0);
            k_rb_rd<<<nblocks(N), RT_BLOCK, 0, st>>>(pe, ctx->mesh.colour.p, a.diag, a.upper, a.lower, ctx->jac.p);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        } else if (jacobi()) {
            // the exact factorisation's 1/rD in cell order, then the FP32
            // premultiplied coefficients of the Jacobi sweeps
            const DevMesh &m = ctx->mesh;
            const double fpc = (double)m.F / N;
            {
                ProfScope ps(ctx, "dilu_rD", (double)N * (16.0 + fpc * 28.0));
                if (systolic()) {
                    skew_prepare(ctx, a.diag, a.upper, a.lower);
                    skew_rdinv_cells(ctx, rD64);
                } else {
                    compute_rd(rD64);
                }
            }
            const size_t need = (size_t)(m.pnLo + m.pnUp + 4) * N;
            if (ctx->jac.n < need) ctx->jac.alloc(need);
            k_jac_coef<<<nblocks(N), RT_BLOCK, 0, st>>>(N, m.pnLo, m.pnUp, m.plFace.p, m.puFace.p, rD64, a.upper,
                                                        a.lower, jrD(), jlo(), jup());
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        } else if (systolic()) {
            const double fpc = (double)ctx->mesh.F / N;
            ProfScope ps(ctx, "dilu_rD", (double)N * (16.0 + fpc * 28.0));
            skew_prepare32(ctx, a.diag, a.upper, a.lower);
        } else if (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU || pre == RT_PRECOND_DIAGONAL) {
            compute_rd(rD64);
            k_mx_to32<<<nblocks(N), RT_BLOCK, 0, st>>>(N, rD64, rD32);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        }
    }

    // FP64 r -> FP32 preconditioner -> FP64 w (the structured sweeps round on
    // the way in and out; otherwise through the FP32 vectors r32, w32)
    // the red-black DIC of the pressure solve (one component, structured mesh)
    bool redblack() const {
        return ctx->mixedJacobi == -1 && a.nc == 1 && a.ctl.preconditioner == RT_PRECOND_DIC &&
               ctx->mesh.colour.p != nullptr && !ctx->mesh.hasCoupled;
    }
    void redblack_apply(const double *r, double *w, const unsigned *dmask) {
        const double fpc = (double)ctx->mesh.F / N;
        // rDinv 4 + colour 1 + coefficients 2*(F/N)*4 + addressing 2*(F/N)*8 (both passes),
        // r 8 read twice, the black copy 4 + 4, w 8
        ProfScope ps(ctx, "dilu_redblack32", (double)N * (5.0 + fpc * 24.0 + 16.0 + 8.0 + 8.0));
        float *rDi = ctx->jac.p, *wb = ctx->jac.p + N;
        k_rb_black<<<nblocks(N), RT_BLOCK, 0, st>>>(pe, ctx->mesh.colour.p, rDi, u32, l32, r, wb, w, dmask);
        k_rb_red<<<nblocks(N), RT_BLOCK, 0, st>>>(pe, ctx->mesh.colour.p, rDi, u32, l32, r, wb, w, dmask);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 2);
    }

    // the aggregation multigrid V-cycle of the pressure solve (one component,
    // a symmetric matrix, structured mesh without coupled faces)
    bool multigrid() const {
        return ctx->mixedJacobi == -2 && a.nc == 1 && a.ctl.preconditioner == RT_PRECOND_DIC && mg_available(ctx);
    }
    // the same V-cycle for the momentum solve (up to three components, a
    // non-symmetric matrix)
    bool multigridU() const {
        return ctx->mixedPrecondU == -2 && a.nc <= 3 && (a.validMask & ~7u) == 0 &&
               a.ctl.preconditioner == RT_PRECOND_DILU && mg_available(ctx);
    }

    // the Jacobi-swept DIC/DILU of the pressure solve (one component)
    bool jacobi() const {
        const int pre = a.ctl.preconditioner;
        return ctx->mixedJacobi > 0 && a.nc == 1 && (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU);
    }
    float *jrD() const { return ctx->jac.p; }
    float *jlo() const { return ctx->jac.p + N; }
    float *jup() const { return ctx->jac.p + (size_t)(1 + ctx->mesh.pnLo) * N; }
    float *jvec(int i) const { return ctx->jac.p + (size_t)(1 + ctx->mesh.pnLo + ctx->mesh.pnUp + i) * N; }

    void jacobi_apply(const double *r, double *w, const unsigned *dmask) {
        const DevMesh &m = ctx->mesh;
        const int sweeps = ctx->mixedJacobi;
        // per sweep: coefficients 4 and addressing 4 per neighbour, base 4, y 4 read, 4 written
        ProfScope ps(ctx, "dilu_jacobi32", (double)N * (12.0 + 2.0 * sweeps * (12.0 + 4.0 * m.F / N)));
        float *y0 = jvec(0), *ya = jvec(1), *yb = jvec(2);
        k_jac_first<<<nblocks(N), RT_BLOCK, 0, st>>>(N, m.pnLo, m.plNbr.p, jlo(), jrD(), r, y0, ya, nullptr, dmask);
        // forward: y_k = y0 - rD L y_{k-1}
        float *cur = ya, *spare = yb;
        for (int k = 1; k < sweeps; ++k) {
            k_jac_sweep<<<nblocks(N), RT_BLOCK, 0, st>>>(N, m.pnLo, m.plNbr.p, jlo(), y0, cur, spare, nullptr, dmask);
            std::swap(cur, spare);
        }
        // backward from z = y_m: z_k = y_m - rD U z_{k-1}; the last writes FP64 w
        float *base = cur, *zin = cur, *zout = (cur == ya) ? y0 : ya;
        float *zalt = (cur == yb) ? y0 : yb;
        if (cur == y0) zalt = yb;
        for (int k = 0; k < sweeps; ++k) {
            const bool last = k == sweeps - 1;
            k_jac_sweep<<<nblocks(N), RT_BLOCK, 0, st>>>(N, m.pnUp, m.puNbr.p, jup(), base, zin, last ? nullptr : zout,
                                                         last ? w : nullptr, dmask);
            zin = zout;
            std::swap(zout, zalt);
        }
        RT_CHECK_LAUNCH();
        launch_count(ctx, 2 * sweeps);
    }

    void precondition32d(unsigned mask, const double *r, double *w, float *r32, float *w32,
                         const unsigned *dmask = nullptr) {
        if (multigrid()) {
            // level 0: the FP64 residual and result, five passes of the 7-point
            // stencil (7 x 4 bytes and x, b); the coarser levels add about 1/7
            ProfScope ps(ctx, "mg_vcycle32", (double)N * (16.0 + 5.0 * 36.0) * 8.0 / 7.0);
            mg_apply(ctx, r, w, dmask);
            return;
        }
        if (redblack()) {
            redblack_apply(r, w, dmask);
            return;
        }
        if (jacobi()) {
            jacobi_apply(r, w, dmask);
            return;
        }
        if (systolic() && a.ctl.preconditioner != RT_PRECOND_NONE && a.ctl.preconditioner != RT_PRECOND_DIAGONAL) {
            const double fpc = (double)ctx->mesh.F / N;
            // (FP32 coefficients: rD 4, 2*(F/N)*4; FP64 r and w, FP32 forward result)
            ProfScope ps(ctx, "dilu_precondition32", (double)N * (4.0 + fpc * 8.0 + 24.0 * pop(mask)));
            skew_precondition32d(ctx, a.nc, mask, r, w, dmask);
            return;
        }
        k_mx_d2f<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, r, r32);
        precondition32(mask, r32, w32);
        k_mx_f2d<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, w32, w);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 2);
    }

    void precondition32(unsigned mask, const float *r, float *w) {
        const DevMesh &m = ctx->mesh;
        const int pre = a.ctl.preconditioner;
        const double fpc = (double)m.F / N;
        if (multigridU()) {
            // level 0: r and w (4 + 4 a component), five passes of the 7-point
            // stencil (7 x 4 bytes, x and b a component); the coarser levels
            // add about 1/7
            const double nc = pop(mask);
            ProfScope ps(ctx, "mg_vcycle32", (double)N * (8.0 * nc + 5.0 * (28.0 + 12.0 * nc)) * 8.0 / 7.0);
            mg_apply32(ctx, mask, r, w);
            return;
        }
        if (pre == RT_PRECOND_NONE) {
            k_mx_copy<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, r, w);
            launch_count(ctx);
        } else if (pre == RT_PRECOND_DIAGONAL) {
            k_mx_diag_apply<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, rD32, r, w);
            launch_count(ctx);
        } else if (systolic()) {
            ProfScope ps(ctx, "dilu_precondition32", (double)N * (4.0 + fpc * 8.0 + 16.0 * pop(mask)));
            skew_precondition32(ctx, a.nc, mask, r, w);
        } else {
            ProfScope ps(ctx, "dilu_precondition32", (double)N * (8.0 + fpc * 24.0 + 16.0 * pop(mask)));
            for (int l = 0; l < m.nLevels; ++l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_fwd_level<float><<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(pe, l0, l1, m.levelCells.p, mask, rD32,
                                                                          l32, r, w);
            }
            for (int l = m.nLevels - 1; l >= 0; --l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_bwd_level<float><<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(pe, l0, l1, m.levelCells.p, mask, rD32,
                                                                          u32, w);
            }
            launch_count(ctx, 2 * m.nLevels);
        }
        RT_CHECK_LAUNCH();
    }

    void amul32(unsigned mask, const float *x, float *y) {
        const double fpc = (double)ctx->mesh.F / N;
        ProfScope ps(ctx, "amul32", (double)N * (4.0 + fpc * 16.0 + 8.0 * pop(mask)));
        k_mx_amul<<<nblocks(N), RT_BLOCK, 0, st>>>(e, mask, d32, u32, l32, x, y);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }

    void dot32(unsigned mask, const float *x, const float *y, const float *x2 = nullptr,
               const float *y2 = nullptr) {
        ProfScope ps(ctx, "dot32", (double)N * 4.0 * (x2 ? 4 : 2) * pop(mask));
        k_mx_dot<<<nB, RT_BLOCK, 0, st>>>(N, mask, x, y, x2, y2, ctx->red.partial.p, nB);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
        finalize(x2 ? 2 : 1, mask);
    }

    void sync_scalars() {
        RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, S, sizeof(double) * (S_SING + 1) * 8, cudaMemcpyDeviceToHost,
                                st));
        RT_CUDA(cudaStreamSynchronize(st));
    }

    // fold x32 into psi and replace r32 by b - A psi; S_FIN gets the
    // normalised FP64 residual of the masked components
    void replace(unsigned mask, float *x32, float *r32) {
        if (!mask) return;
        const double fpc = (double)ctx->mesh.F / N;
        ProfScope ps(ctx, "residual_replace", (double)N * (8.0 + fpc * 24.0 + 44.0 * pop(mask)));
        k_mx_fold<<<nblocks(N), RT_BLOCK, 0, st>>>(N, mask, x32, a.psi);
        k_mx_true_res<<<nB, RT_BLOCK, 0, st>>>(e, mask, a.diag, a.upper, a.lower, a.source, a.psi, r32,
                                               ctx->red.partial.p, nB);
        RT_CHECK_LAUNCH();
        finalize(1, mask);
        k_sc_fin<<<1, 32, 0, st>>>(mask, ctx->red.result.p, S);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 3);
    }
};

// prologue shared by the mixed solvers; returns the components to iterate
unsigned mixed_begin(Mixed &mx, const SolveArgs &a, rt_solver_perf *perf, float *r32, float *x32,
                     double *lastTrue) {
    rt_ctx *ctx = mx.ctx;
    const int N = mx.N;
    double *wA = ctx->kws.p, *rA = ctx->kws.p + 6 * (size_t)N;
    const unsigned mask = a.validMask;
    mx.prepare();
    mx.prologue(mask, wA, rA);
    k_mx_start<<<nblocks(N), RT_BLOCK, 0, mx.st>>>(N, mask, rA, r32, x32, mx.S);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    RT_CUDA(cudaMemcpyAsync(ctx->red.hostResult, mx.S, sizeof(double) * 3 * 8, cudaMemcpyDeviceToHost, mx.st));
    RT_CUDA(cudaStreamSynchronize(mx.st));
    unsigned active = 0;
    for (int k = 0; k < 6; ++k) {
        if (!((mask >> k) & 1u)) continue;
        perf[k].initialResidual = ctx->red.hostResult[S_INIT * 8 + k];
        perf[k].finalResidual = ctx->red.hostResult[S_FIN * 8 + k];
        perf[k].nIterations = 0;
        perf[k].singular = 0;
        lastTrue[k] = perf[k].finalResidual;
        if (a.ctl.minIter > 0 || !mx.conv(perf[k].finalResidual, perf[k].initialResidual)) active |= 1u << k;
    }
    return active;
}

// after an iteration: which components need a residual replacement
unsigned mixed_replace_set(const Mixed &mx, const SolveArgs &a, unsigned cand, const double *H, int iter,
                           const rt_solver_perf *perf, const double *lastTrue) {
    unsigned R = 0;
    for (int k = 0; k < 6; ++k) {
        if (!((cand >> k) & 1u)) continue;
        const double fin = H[S_FIN * 8 + k];
        if (fin < kReplace * lastTrue[k] || mx.conv(fin, perf[k].initialResidual) || iter >= a.ctl.maxIter ||
            !std::isfinite(fin))
            R |= 1u << k;
    }
    return R;
}

// Mixed form of the pressure solve: PCG with FP64 vectors and scalars and
// the DIC preconditioner applied in FP32.  The FP32 sweeps make the
// preconditioner a slightly different operator at every application, so beta
// takes the flexible (Polak-Ribiere) form; the iterates keep FP64
// conjugacy, which an ill-conditioned pressure matrix needs (FP32 Krylov
// vectors lose it and stall).  Stopping test and records as run_pcg.
rt_status run_pcg_flex32(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    Mixed mx(ctx, a, 2);
    float *r32 = mx.v(0), *z32 = mx.v(1);
    mx.prepare();
    mx.prologue(a.validMask, ctx->kws.p, ctx->kws.p + 6 * (size_t)mx.N);
    return pcg_device_loop<true>(ctx, mx, a, perf, [&](unsigned act, const double *r, double *w, const unsigned *dm) {
        mx.precondition32d(act, r, w, r32, z32, dm);
    });
}

rt_status run_pbicgstab_mixed(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    Mixed mx(ctx, a, 9);
    const int N = mx.N;
    float *r = mx.v(0), *r0 = mx.v(1), *p = mx.v(2), *y = mx.v(3), *Ay = mx.v(4), *s = mx.v(5), *z = mx.v(6),
          *t = mx.v(7), *x = mx.v(8);
    double lastTrue[6] = {};
    unsigned active = mixed_begin(mx, a, perf, r, x, lastTrue);
    if (!active) return RT_OK;
    RT_CUDA(cudaMemcpyAsync(r0, r, sizeof(float) * 6 * (size_t)N, cudaMemcpyDeviceToDevice, mx.st));
    int iter = 0;
    double H[(S_SING + 1) * 8];
    while (active) {
        mx.dot32(active, r0, r);
        k_sc_bicg_r0r<<<1, 32, 0, mx.st>>>(active, iter, ctx->red.result.p, mx.S);
        k_mx_bicg_p<<<nblocks(N), RT_BLOCK, 0, mx.st>>>(N, active, iter == 0, mx.S, r, Ay, p);
        mx.precondition32(active, p, y);
        mx.amul32(active, y, Ay);
        mx.dot32(active, r0, Ay);
        k_mx_sc_bicg_alpha<<<1, 32, 0, mx.st>>>(active, ctx->red.result.p, mx.S);
        k_mx_bicg_s<<<mx.nB, RT_BLOCK, 0, mx.st>>>(N, active, mx.S, r, Ay, s, ctx->red.partial.p, mx.nB);
        RT_CHECK_LAUNCH();
        mx.finalize(1, active);
        k_sc_fin<<<1, 32, 0, mx.st>>>(active, ctx->red.result.p, mx.S);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 5);
        mx.sync_scalars();
        memcpy(H, ctx->red.hostResult, sizeof H);
        // the half-step test: components whose s meets the tolerance take
        // x += alpha y and have their residual replaced; the FP64 residual
        // decides whether they stop or restart
        unsigned half = 0, cont = 0;
        for (int k = 0; k < 6; ++k) {
            if (!((active >> k) & 1u)) continue;
            if (H[S_SING * 8 + k] != 0.0) {
                perf[k].singular = 1;
                continue;
            }
            if (mx.conv(H[S_FIN * 8 + k], perf[k].initialResidual)) half |= 1u << k;
            else cont |= 1u << k;
        }
        unsigned restart = 0;
        if (half) {
            k_mx_axpy_alpha<<<nblocks(N), RT_BLOCK, 0, mx.st>>>(N, half, mx.S, y, x);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
            mx.replace(half, x, r);
            mx.sync_scalars();
            for (int k = 0; k < 6; ++k) {
                if (!((half >> k) & 1u)) continue;
                perf[k].finalResidual = ctx->red.hostResult[S_FIN * 8 + k];
                perf[k].nIterations = iter + 1;
                lastTrue[k] = perf[k].finalResidual;
                const bool conv = mx.conv(perf[k].finalResidual, perf[k].initialResidual);
                if ((!conv || iter + 1 < a.ctl.minIter) && iter + 1 < a.ctl.maxIter &&
                    std::isfinite(perf[k].finalResidual))
                    restart |= 1u << k;
            }
            if (restart) {
                k_mx_set_rst<<<1, 32, 0, mx.st>>>(restart, mx.S);
                RT_CHECK_LAUNCH();
                launch_count(ctx);
            }
        }
        unsigned next = restart;
        if (cont) {
            mx.precondition32(cont, s, z);
            mx.amul32(cont, z, t);
            mx.dot32(cont, t, t, t, s);
            k_sc_bicg_omega<<<1, 32, 0, mx.st>>>(cont, ctx->red.result.p, mx.S);
            k_mx_bicg_update<<<mx.nB, RT_BLOCK, 0, mx.st>>>(N, cont, mx.S, y, z, s, t, x, r, ctx->red.partial.p,
                                                            mx.nB);
            RT_CHECK_LAUNCH();
            mx.finalize(1, cont);
            k_sc_fin<<<1, 32, 0, mx.st>>>(cont, ctx->red.result.p, mx.S);
            RT_CHECK_LAUNCH();
            launch_count(ctx, 3);
            mx.sync_scalars();
            memcpy(H, ctx->red.hostResult, sizeof H);
            const unsigned R = mixed_replace_set(mx, a, cont, H, iter + 1, perf, lastTrue);
            mx.replace(R, x, r);
            if (R) {
                mx.sync_scalars();
                memcpy(H, ctx->red.hostResult, sizeof H);
            }
            for (int k = 0; k < 6; ++k) {
                if (!((cont >> k) & 1u)) continue;
                perf[k].finalResidual = H[S_FIN * 8 + k];
                perf[k].nIterations = iter + 1;
                if ((R >> k) & 1u) lastTrue[k] = perf[k].finalResidual;
                const bool conv = ((R >> k) & 1u) && mx.conv(perf[k].finalResidual, perf[k].initialResidual);
                const bool more = (iter + 1 < a.ctl.maxIter && !conv) || iter + 1 < a.ctl.minIter;
                if (more && std::isfinite(perf[k].finalResidual)) next |= 1u << k;
            }
        }
        ++iter;
        active = next;
    }
    k_mx_fold<<<nblocks(N), RT_BLOCK, 0, mx.st>>>(N, a.validMask, x, a.psi);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
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
    if (mask && ctx->mesh.batch.n > 1) {
        RT_REQUIRE(a.ctl.solver != RT_SOLVER_PBICG, RT_EINVAL, "the batched form runs PCG and PBiCGStab, not PBiCG");
        st = batch_solve(ctx, b, perf);
    } else if (mask) {
        const bool pcg = a.ctl.solver == RT_SOLVER_PCG;
        if (a.ctl.solver == RT_SOLVER_PBICG) {
            // (FP64 in both forms: the mixed form's FP32 iterations are built
            // for PCG and PBiCGStab)
            st = run_pbicg(ctx, b, perf);
        } else if (a.precision == RT_PREC_MIXED && (ctx->mixedParts & 1)) {
            SolveArgs t = b;
            t.ctl.tolerance *= ctx->mixedTighten;
            t.ctl.relTol *= ctx->mixedTighten;
            st = pcg ? run_pcg_flex32(ctx, t, perf) : run_pbicgstab_mixed(ctx, t, perf);
        }
        else st = pcg ? run_pcg(ctx, b, perf) : run_pbicgstab(ctx, b, perf);
    }
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
