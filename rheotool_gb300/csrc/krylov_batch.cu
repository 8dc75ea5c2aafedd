// krylov_batch.cu — PCG (+DIC) and PBiCGStab (+DILU) for a batch of
// independent cases that share one device mesh (their disjoint union).
//
// Every (case, component) pair is a segment with its own Krylov scalars,
// its own normFactor, iteration count and stopping point, exactly as if the
// case were solved alone: the matrix of a batch is block diagonal, and every
// inner product and norm is reduced per case (reduction blocks never straddle
// two cases; the blocks of a case are summed in a fixed order).  Segments
// iterate in lock step; a segment that has stopped takes no further updates.
// The stopping decisions are taken on the device (one thread per segment),
// so one iteration is a fixed launch sequence: it is captured once into a
// CUDA graph and replayed, and the host only polls the number of segments
// still iterating every few iterations.
//
// Structured 2-D cases in batches that fill the GPU take a second form
// (RT_OPT_BATCH_PERSISTENT): one persistent CTA per case runs every
// iteration of its case's pressure PCG (k_b_pcg_case) or momentum BiCGStab
// (k_b_bicg_case) in one launch, with the same scalar decisions, the case's
// sweeps inside the CTA (sweep2d_cta.cuh, chunks staged by cp.async) and its
// reductions as one pass of the CTA (FP32 vectors summed as float-float
// pairs).
//
// Precision: the vectors are FP32 (RT_PREC_MIXED) or FP64, the scalars and
// reductions FP64.  As in the single-case mixed solvers, the solution is
// psi (FP64) + x (a correction in the vector type), folded into psi with the
// residual recomputed from the FP64 matrix whenever the iterated residual has
// dropped tenfold, claims convergence or the iteration budget ends; the
// stopping test uses that FP64 residual.
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

#include "batch.h"
#include "real_ops.cuh"
#include "sweep2d_cta.cuh"

namespace rt {

namespace {

constexpr double kReplaceB = 0.1;

__device__ __forceinline__ double bsum(double v) {   // valid in thread 0
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

struct BEll {
    int N, nSlots;
    const int *__restrict__ face;
    const int *__restrict__ nbr;
};

template <class M, class X>
__device__ __forceinline__ double brow_mul(const BEll &e, int c, const M *__restrict__ diag, const M *__restrict__ upper,
                                           const M *__restrict__ lower, const X *__restrict__ x) {
    double acc = (double)diag[c] * (double)x[c];
    for (int s = 0; s < e.nSlots; ++s) {
        int nb = e.nbr[s * e.N + c];
        if (nb < 0) break;
        int f = e.face[s * e.N + c];
        acc += (double)(nb > c ? upper[f] : lower[f]) * (double)x[nb];
    }
    return acc;
}

__device__ __forceinline__ double brow_sum(const BEll &e, int c, const double *__restrict__ diag,
                                           const double *__restrict__ upper, const double *__restrict__ lower) {
    double acc = diag[c];
    for (int s = 0; s < e.nSlots; ++s) {
        int nb = e.nbr[s * e.N + c];
        if (nb < 0) break;
        int f = e.face[s * e.N + c];
        acc += nb > c ? upper[f] : lower[f];
    }
    return acc;
}

struct Ctl {
    double tol, relTol;
    int minIter, maxIter;
};
__device__ __forceinline__ bool bconv(const Ctl &c, double fin, double init) {
    return fin < c.tol || (c.relTol > 1e-20 && fin < c.relTol * init);
}

// ---- reductions ---------------------------------------------------------
// partial[(slot * 6 + k) * nBlk + blk]; res[slot * nSeg + case * 8 + k]
__global__ void k_b_fin(int nSlots, unsigned vm, BTab t, const double *__restrict__ partial, double *__restrict__ res) {
    const int cb = blockIdx.x, k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= 6 || !((vm >> k) & 1u)) return;
    const int b0 = t.caseBlk[cb], b1 = t.caseBlk[cb + 1];
    const int nSeg = 8 * t.nCases;
    for (int slot = 0; slot < nSlots; ++slot) {
        double v = 0.0;
        for (int i = b0 + lane; i < b1; i += 32) v += partial[(slot * 6 + k) * t.nBlk + i];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) res[slot * nSeg + cb * 8 + k] = v;
    }
}

__global__ void k_b_sumx(BTab t, unsigned vm, const double *__restrict__ x, double *partial) {
    const int blk = blockIdx.x, c = t.blkCell0[blk] + threadIdx.x;
    const bool in = c < t.blkCell1[blk];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        double s = bsum(in ? x[(size_t)k * t.N + c] : 0.0);
        if (threadIdx.x == 0) partial[(0 * 6 + k) * t.nBlk + blk] = s;
    }
}

// r = b - A psi (FP64) into the vector type; slot 0: normFactor sums, slot 1: |r|
template <class V>
__global__ void k_b_init_res(BTab t, BEll e, unsigned vm, const double *__restrict__ diag,
                             const double *__restrict__ upper, const double *__restrict__ lower,
                             const double *__restrict__ b, const double *__restrict__ psi,
                             const double *__restrict__ xsum, const int *__restrict__ caseCell0, V *__restrict__ r,
                             V *__restrict__ x, double *partial) {
    const int blk = blockIdx.x, cb = t.blkCase[blk], c = t.blkCell0[blk] + threadIdx.x;
    const bool in = c < t.blkCell1[blk];
    const int nSeg = 8 * t.nCases;
    const double nCell = (double)(caseCell0[cb + 1] - caseCell0[cb]);
    (void)nSeg;
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        double v0 = 0.0, v1 = 0.0;
        if (in) {
            const double xbar = xsum[cb * 8 + k] / nCell;
            const size_t o = (size_t)k * t.N;
            double ax = brow_mul(e, c, diag, upper, lower, psi + o);
            double sa = brow_sum(e, c, diag, upper, lower) * xbar;
            double bb = b[o + c];
            double rr = bb - ax;
            r[o + c] = (V)rr;
            x[o + c] = V(0);
            v0 = fabs(ax - sa) + fabs(bb - sa);
            v1 = fabs(rr);
        }
        double s0 = bsum(v0);
        if (threadIdx.x == 0) partial[(0 * 6 + k) * t.nBlk + blk] = s0;
        double s1 = bsum(v1);
        if (threadIdx.x == 0) partial[(1 * 6 + k) * t.nBlk + blk] = s1;
    }
}

template <class V>
__global__ void k_b_dot(BTab t, unsigned vm, const int *__restrict__ active, const V *__restrict__ a,
                        const V *__restrict__ b, const V *__restrict__ c2, const V *__restrict__ d2, double *partial) {
    const int blk = blockIdx.x, cb = t.blkCase[blk], c = t.blkCell0[blk] + threadIdx.x;
    const bool in = c < t.blkCell1[blk];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        if (!active[cb * 8 + k]) continue;   // uniform in the block
        const size_t o = (size_t)k * t.N;
        double v0 = in ? (double)a[o + c] * (double)b[o + c] : 0.0;
        double s0 = bsum(v0);
        if (threadIdx.x == 0) partial[(0 * 6 + k) * t.nBlk + blk] = s0;
        if (c2) {
            double v1 = in ? (double)c2[o + c] * (double)d2[o + c] : 0.0;
            double s1 = bsum(v1);
            if (threadIdx.x == 0) partial[(1 * 6 + k) * t.nBlk + blk] = s1;
        }
    }
}

// ---- vector kernels (one thread per cell) ----------------------------------
template <class V, class M>
__global__ void k_b_amul(BEll e, unsigned vm, const M *__restrict__ diag, const M *__restrict__ upper,
                         const M *__restrict__ lower, const V *__restrict__ x, V *__restrict__ y) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= e.N) return;
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        const size_t o = (size_t)k * e.N;
        const V xc = x[o + c];
        V acc = V(diag[c]) * xc;
        for (int s = 0; s < e.nSlots; ++s) {
            int nb = e.nbr[s * e.N + c];
            if (nb < 0) break;
            int f = e.face[s * e.N + c];
            // FP32: differences form (diag holds the row sums)
            acc = fma(V(nb > c ? upper[f] : lower[f]), sizeof(V) == 4 ? x[o + nb] - xc : x[o + nb], acc);
        }
        y[o + c] = acc;
    }
}

template <class V>
__global__ void k_b_pcg_p(int N, unsigned vm, const int *__restrict__ caseOf, BSeg S, const V *__restrict__ w,
                          V *__restrict__ p) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int cb = caseOf[c];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        const int sg = cb * 8 + k;
        if (!S.active[sg]) continue;
        const size_t i = (size_t)k * N + c;
        if (S.iter[sg] == 0) p[i] = w[i];
        else p[i] = fma(V(S.beta[sg]), p[i], w[i]);
    }
}

template <class V>
__global__ void k_b_pcg_update(BTab t, unsigned vm, BSeg S, const V *__restrict__ p, const V *__restrict__ q,
                               V *__restrict__ x, V *__restrict__ r, double *partial) {
    const int blk = blockIdx.x, cb = t.blkCase[blk], c = t.blkCell0[blk] + threadIdx.x;
    const bool in = c < t.blkCell1[blk];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        const int sg = cb * 8 + k;
        if (!S.active[sg]) continue;
        double v = 0.0;
        if (in) {
            const size_t i = (size_t)k * t.N + c;
            V rr = r[i];
            if (!S.sing[sg]) {
                const V alpha = V(S.alpha[sg]);
                x[i] = fma(alpha, p[i], x[i]);
                rr = fma(-alpha, q[i], rr);
                r[i] = rr;
            }
            v = fabs((double)rr);
        }
        double s = bsum(v);
        if (threadIdx.x == 0) partial[(0 * 6 + k) * t.nBlk + blk] = s;
    }
}

// psi += x; x = 0 on the segments flagged in flag[] (all when flag is null)
template <class V>
__global__ void k_b_fold(int N, unsigned vm, const int *__restrict__ caseOf, const int *__restrict__ flag,
                         V *__restrict__ x, double *__restrict__ psi) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int cb = caseOf[c];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u) || (flag && !flag[cb * 8 + k])) continue;
        const size_t i = (size_t)k * N + c;
        psi[i] += (double)x[i];
        x[i] = V(0);
    }
}

// r = b - A psi (FP64 matrix) on flagged segments; partial |r|
template <class V>
__global__ void k_b_true(BTab t, BEll e, unsigned vm, const int *__restrict__ flag, const double *__restrict__ diag,
                         const double *__restrict__ upper, const double *__restrict__ lower,
                         const double *__restrict__ b, const double *__restrict__ psi, V *__restrict__ r,
                         double *partial) {
    const int blk = blockIdx.x, cb = t.blkCase[blk], c = t.blkCell0[blk] + threadIdx.x;
    const bool in = c < t.blkCell1[blk];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u) || !flag[cb * 8 + k]) continue;
        double v = 0.0;
        if (in) {
            const size_t o = (size_t)k * t.N;
            const double rr = b[o + c] - brow_mul(e, c, diag, upper, lower, psi + o);
            r[o + c] = (V)rr;
            v = fabs(rr);
        }
        double s = bsum(v);
        if (threadIdx.x == 0) partial[(0 * 6 + k) * t.nBlk + blk] = s;
    }
}

template <class V>
__global__ void k_b_bicg_p(int N, unsigned vm, const int *__restrict__ caseOf, BSeg S, const V *__restrict__ r,
                           const V *__restrict__ Ay, V *__restrict__ p) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int cb = caseOf[c];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        const int sg = cb * 8 + k;
        if (!S.active[sg] || S.sing[sg]) continue;
        const size_t i = (size_t)k * N + c;
        if (S.iter[sg] == 0 || S.rst[sg]) p[i] = r[i];
        else p[i] = fma(V(S.beta[sg]), fma(-V(S.omega[sg]), Ay[i], p[i]), r[i]);
    }
}

template <class V>
__global__ void k_b_bicg_s(BTab t, unsigned vm, BSeg S, const V *__restrict__ r, const V *__restrict__ Ay,
                           V *__restrict__ s, double *partial) {
    const int blk = blockIdx.x, cb = t.blkCase[blk], c = t.blkCell0[blk] + threadIdx.x;
    const bool in = c < t.blkCell1[blk];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        const int sg = cb * 8 + k;
        if (!S.active[sg] || S.sing[sg]) continue;
        double v = 0.0;
        if (in) {
            const size_t i = (size_t)k * t.N + c;
            const V sv = fma(-V(S.alpha[sg]), Ay[i], r[i]);
            s[i] = sv;
            v = fabs((double)sv);
        }
        double sm = bsum(v);
        if (threadIdx.x == 0) partial[(0 * 6 + k) * t.nBlk + blk] = sm;
    }
}

// x += alpha y on the half-step segments (flag 'half' in S.repl == 2)
template <class V>
__global__ void k_b_axpy_half(int N, unsigned vm, const int *__restrict__ caseOf, BSeg S, const V *__restrict__ y,
                              V *__restrict__ x) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int cb = caseOf[c];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        const int sg = cb * 8 + k;
        if (S.conv[sg] != 2) continue;
        const size_t i = (size_t)k * N + c;
        x[i] = fma(V(S.alpha[sg]), y[i], x[i]);
    }
}

template <class V>
__global__ void k_b_bicg_update(BTab t, unsigned vm, BSeg S, const V *__restrict__ y, const V *__restrict__ z,
                                const V *__restrict__ s, const V *__restrict__ tt, V *__restrict__ x,
                                V *__restrict__ r, double *partial) {
    const int blk = blockIdx.x, cb = t.blkCase[blk], c = t.blkCell0[blk] + threadIdx.x;
    const bool in = c < t.blkCell1[blk];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        const int sg = cb * 8 + k;
        if (!S.active[sg] || S.sing[sg] || S.conv[sg] == 2) continue;
        double v = 0.0;
        if (in) {
            const size_t i = (size_t)k * t.N + c;
            const V alpha = V(S.alpha[sg]), omega = V(S.omega[sg]);
            x[i] = fma(alpha, y[i], fma(omega, z[i], x[i]));
            const V rv = fma(-omega, tt[i], s[i]);
            r[i] = rv;
            v = fabs((double)rv);
        }
        double sm = bsum(v);
        if (threadIdx.x == 0) partial[(0 * 6 + k) * t.nBlk + blk] = sm;
    }
}

// ---- per-segment logic (one block, threads stride over the segments) ------
// S.conv: 0 iterating, 1 converged (stopped), 2 half-step exit pending
__global__ void k_b_start(int nCases, unsigned vm, Ctl ctl, BSeg S, const double *__restrict__ res) {
    const int nSeg = 8 * nCases;
    int cnt = 0;
    for (int sg = threadIdx.x; sg < nSeg; sg += blockDim.x) {
        const int k = sg & 7;
        if (k >= 6 || !((vm >> k) & 1u)) {
            S.active[sg] = 0;
            continue;
        }
        const double nf = res[0 * nSeg + sg] + 1e-20;
        const double r0 = res[1 * nSeg + sg] / nf;
        S.nf[sg] = nf;
        S.init[sg] = r0;
        S.fin[sg] = r0;
        S.last[sg] = r0;
        S.iter[sg] = 0;
        S.sing[sg] = 0;
        S.repl[sg] = 0;
        S.rst[sg] = 0;
        S.A[sg] = 1e20;
        S.r0r[sg] = 0.0;
        S.alpha[sg] = 0.0;
        S.omega[sg] = 0.0;
        const bool c = bconv(ctl, r0, r0);
        S.conv[sg] = c ? 1 : 0;
        S.active[sg] = (ctl.minIter > 0 || !c) ? 1 : 0;
        cnt += S.active[sg];
    }
    __shared__ int sc[32];
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) sc[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sc[i];
        S.count[0] = t;
    }
}

// PCG scalars; FP32 vectors use the flexible (Polak-Ribiere) beta
// w.(r - r_old) / w_old.r_old = -alpha_old w.q_old / w_old.r_old
__global__ void k_b_pcg_a(int nSeg, BSeg S, const double *__restrict__ res, int mixed) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg]) continue;
        const double aold = S.A[sg];
        S.Aold[sg] = aold;
        S.A[sg] = res[sg];
        S.beta[sg] = mixed ? -S.alpha[sg] * res[nSeg + sg] / aold : res[sg] / aold;
    }
}

__global__ void k_b_pcg_alpha(int nSeg, BSeg S, const double *__restrict__ res) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg]) continue;
        const double wApA = res[sg];
        if (fabs(wApA) / S.nf[sg] < 1e-300) {
            S.sing[sg] = 1;
            S.alpha[sg] = 0.0;
        } else {
            S.alpha[sg] = S.A[sg] / wApA;
        }
    }
}

// after an iteration's residual: count the iteration, stop singular
// segments; mixed precision flags the residual replacements, FP64 applies the
// stopping test of the plain solvers to the iterated residual
__global__ void k_b_iter_fin(int nSeg, Ctl ctl, BSeg S, const double *__restrict__ res, int skipHalf, int mixed) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg]) continue;
        if (skipHalf && S.conv[sg] == 2) {   // restarted at the half step: counted, no update
            S.iter[sg] += 1;
            S.conv[sg] = 0;
            continue;
        }
        if (S.sing[sg]) {
            S.active[sg] = 0;
            continue;
        }
        const double fin = res[sg] / S.nf[sg];
        S.fin[sg] = fin;
        S.iter[sg] += 1;
        if (mixed) {
            S.repl[sg] = (fin < kReplaceB * S.last[sg] || bconv(ctl, fin, S.init[sg]) || S.iter[sg] >= ctl.maxIter ||
                          !isfinite(fin)) ? 1 : 0;
        } else {
            const bool c = bconv(ctl, fin, S.init[sg]);
            const bool more = (S.iter[sg] < ctl.maxIter && !c) || S.iter[sg] < ctl.minIter;
            S.conv[sg] = c ? 1 : 0;
            if (!more || !isfinite(fin)) S.active[sg] = 0;
        }
    }
}

// after a residual replacement: FP64 residual, stopping test, count
__global__ void k_b_after(int nCases, Ctl ctl, BSeg S, const double *__restrict__ res) {
    const int nSeg = 8 * nCases;
    int cnt = 0;
    for (int sg = threadIdx.x; sg < nSeg; sg += blockDim.x) {
        if (S.active[sg] && S.repl[sg]) {
            const double fin = res[sg] / S.nf[sg];
            S.fin[sg] = fin;
            S.last[sg] = fin;
            const bool c = bconv(ctl, fin, S.init[sg]);
            const bool more = (S.iter[sg] < ctl.maxIter && !c) || S.iter[sg] < ctl.minIter;
            S.conv[sg] = c ? 1 : 0;
            if (!more || !isfinite(fin)) S.active[sg] = 0;
        }
        S.repl[sg] = 0;
        cnt += S.active[sg];
    }
    __shared__ int sc[32];
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) sc[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sc[i];
        S.count[0] = t;
    }
}

// BiCGStab scalars
__global__ void k_b_bicg_r0r(int nSeg, BSeg S, const double *__restrict__ res) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg]) continue;
        const double old = S.r0r[sg], r0r = res[sg];
        S.r0rOld[sg] = old;
        S.r0r[sg] = r0r;
        if (fabs(r0r) < 1e-300) { S.sing[sg] = 1; continue; }
        if (S.iter[sg] > 0 && !S.rst[sg]) {
            const double om = S.omega[sg];
            if (fabs(om) < 1e-300) { S.sing[sg] = 1; continue; }
            S.beta[sg] = (r0r / old) * (S.alpha[sg] / om);
        }
    }
}
__global__ void k_b_bicg_alpha(int nSeg, BSeg S, const double *__restrict__ res) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg] || S.sing[sg]) continue;
        S.alpha[sg] = S.r0r[sg] / res[sg];
        S.rst[sg] = 0;
    }
}
// the half-step test on |s|; singular segments stop here
__global__ void k_b_bicg_half(int nSeg, Ctl ctl, BSeg S, const double *__restrict__ res, int mixed) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg]) continue;
        if (S.sing[sg]) {
            S.active[sg] = 0;
            continue;
        }
        const double fs = res[sg] / S.nf[sg];
        if (bconv(ctl, fs, S.init[sg])) {
            S.conv[sg] = 2;
            S.repl[sg] = mixed ? 1 : 0;
            if (!mixed) S.fin[sg] = fs;
        }
    }
}
// after the half step: mixed precision stops or restarts from the FP64
// residual of the replacement; FP64 stops (the plain solvers' early exit)
__global__ void k_b_half_after(int nSeg, Ctl ctl, BSeg S, const double *__restrict__ res, int mixed) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg] || S.conv[sg] != 2) continue;
        if (!mixed) {
            S.iter[sg] += 1;
            S.conv[sg] = 1;
            S.active[sg] = 0;
            continue;
        }
        const double fin = res[sg] / S.nf[sg];
        S.fin[sg] = fin;
        S.last[sg] = fin;
        S.repl[sg] = 0;
        const int it = S.iter[sg] + 1;
        const bool c = bconv(ctl, fin, S.init[sg]);
        if ((c && it >= ctl.minIter) || it >= ctl.maxIter || !isfinite(fin)) {
            S.iter[sg] = it;
            S.conv[sg] = c ? 1 : 0;
            S.active[sg] = 0;
        } else {
            S.rst[sg] = 1;   // conv stays 2: the second half is skipped, the iteration counted
        }
    }
}
__global__ void k_b_bicg_omega(int nSeg, BSeg S, const double *__restrict__ res) {
    for (int sg = threadIdx.x + blockIdx.x * blockDim.x; sg < nSeg; sg += blockDim.x * gridDim.x) {
        if (!S.active[sg] || S.sing[sg] || S.conv[sg] == 2) continue;
        S.omega[sg] = res[1 * nSeg + sg] / res[sg];
    }
}

// ---- level-scheduled sweeps over the union (cases without a 2-D layout) ---
template <class V>
__global__ void k_b_fwd_level(BEll e, int l0, int l1, const int *__restrict__ cells, unsigned vm,
                              const V *__restrict__ rD, const V *__restrict__ lower, const V *__restrict__ r,
                              V *__restrict__ w) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    const V rd = rD[c];
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        size_t o = (size_t)k * e.N;
        V acc = r_mul(rd, r[o + c]);
        for (int s = 0; s < e.nSlots; ++s) {
            int nb = e.nbr[s * e.N + c];
            if (nb < 0 || nb > c) break;
            acc = r_fma(-r_mul(rd, lower[e.face[s * e.N + c]]), w[o + nb], acc);
        }
        w[o + c] = acc;
    }
}
template <class V>
__global__ void k_b_bwd_level(BEll e, int l0, int l1, const int *__restrict__ cells, unsigned vm,
                              const V *__restrict__ rD, const V *__restrict__ upper, V *__restrict__ w) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    const V rd = rD[c];
    int ns = 0;
    while (ns < e.nSlots && e.nbr[ns * e.N + c] >= 0) ++ns;
    for (int k = 0; k < 6; ++k) {
        if (!((vm >> k) & 1u)) continue;
        size_t o = (size_t)k * e.N;
        V acc = w[o + c];
        for (int s = ns - 1; s >= 0; --s) {
            int nb = e.nbr[s * e.N + c];
            if (nb < c) break;
            acc = r_fma(-r_mul(rd, upper[e.face[s * e.N + c]]), w[o + nb], acc);
        }
        w[o + c] = acc;
    }
}
__global__ void k_b_rd_level(BEll e, int l0, int l1, const int *__restrict__ cells, const double *__restrict__ diag,
                             const double *__restrict__ upper, const double *__restrict__ lower,
                             double *__restrict__ rD) {
    int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= l1) return;
    int c = cells[t];
    double r = diag[c];
    for (int s = 0; s < e.nSlots; ++s) {
        int nb = e.nbr[s * e.N + c];
        if (nb < 0 || nb > c) break;
        int f = e.face[s * e.N + c];
        r = __dsub_rn(r, __ddiv_rn(__dmul_rn(upper[f], lower[f]), rD[nb]));
    }
    rD[c] = r;
}
template <class V>
__global__ void k_b_recip(int N, const double *__restrict__ rD, V *__restrict__ out, int diagOnly,
                          const double *__restrict__ diag) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < N) out[c] = (V)(1.0 / (diagOnly ? diag[c] : rD[c]));
}
// the matrix in the vector type; FP32 stores the row sums in place of the
// diagonal (differences form: rounding keeps the zero row sums of an
// assembled matrix), FP64 the diagonal itself
template <class M>
__global__ void k_b_mat(BEll e, int F, const double *__restrict__ diag, const double *__restrict__ upper,
                        const double *__restrict__ lower, M *__restrict__ d, M *__restrict__ u, M *__restrict__ l) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < e.N) d[i] = (M)(sizeof(M) == 4 ? brow_sum(e, i, diag, upper, lower) : diag[i]);
    if (i < F) {
        u[i] = (M)upper[i];
        l[i] = (M)lower[i];
    }
}
template <class V>
__global__ void k_b_copy(int N, unsigned vm, const V *__restrict__ r, V *__restrict__ w, const V *__restrict__ rD) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 6; ++k)
        if ((vm >> k) & 1u) w[(size_t)k * N + c] = rD ? rD[c] * r[(size_t)k * N + c] : r[(size_t)k * N + c];
}

// ---- the per-case multigrid V-cycle (mixed pressure and momentum solves) ---
// The multigrid preconditioner of mg.cu on one 2-D case by the CTA that owns
// it: the same aggregation (2 x 2 blocks, Galerkin 5-point coarse
// operators), red-black Gauss-Seidel smoothing (kBMgNu sweeps each way,
// coarse correction scaled by kBMgOver) and symmetric sweeps on the
// coarsest level, every phase a loop of the CTA over a level's box followed
// by a barrier.  A level holds the diagonal and each cell's couplings to and
// from its (i-1) and (j-1) neighbours: A[c][c-1] in xl, A[c-1][c] in xu (yl,
// yu likewise); the symmetric pressure matrix keeps one copy (xu aliases xl).
// With piecewise-constant prolongation P and restriction P^T, the coarse
// operator P^T A P of a non-symmetric matrix is again such a stencil, so the
// momentum matrix (convection makes it non-symmetric) takes the same cycle,
// its components sharing every coefficient load.
constexpr int kBMgNu = 3;
constexpr float kBMgOver = 1.3f;
constexpr int kBMgCoarseSweeps = 16;
// cells a thread smooths per round of loads: the pressure solve's one
// component 4; the momentum solve's kernel has no registers to spare for
// more than one cell at a time (0: the one-cell loop)
constexpr int kMgPcgB = 4;
constexpr int kMgBicgB = 0;

struct BMg {
    const int *__restrict__ dims;       // [case][level][2]: nx, ny
    const int *__restrict__ nl;         // [case]: levels
    const long long *__restrict__ off;  // [case][level]: the level's arrays in pool
    const int *__restrict__ cell;       // level 0's cell of each box position (-1 outside)
    const long long *__restrict__ cellOff;
    const int *__restrict__ faceLo;     // 2N: the face to the (y, x) lower neighbour
    float *pool;
    int on;
};

struct CL {
    int nx, ny, n;
    size_t np;   // the stride of the components' x and b
    float *dg, *xl, *yl, *xu, *yu, *x, *b;
};

__device__ __forceinline__ CL case_level(const BMg &mg, int cb, int l, bool sym) {
    const size_t k = (size_t)cb * kBatchMgLevels + l;
    CL L;
    L.nx = mg.dims[2 * k];
    L.ny = mg.dims[2 * k + 1];
    L.n = L.nx * L.ny;
    L.np = ((size_t)L.n + 3) / 4 * 4;
    float *p = mg.pool + mg.off[k];
    L.dg = p;
    L.xl = p + L.np;
    L.yl = p + 2 * L.np;
    L.xu = sym ? L.xl : p + 3 * L.np;
    L.yu = sym ? L.yl : p + 4 * L.np;
    L.x = p + 5 * L.np;
    L.b = p + 8 * L.np;
    return L;
}

// the couplings of box cell b = (i, j) to its four neighbours
struct CNb {
    float w, e, s, n;
};

__device__ __forceinline__ CNb cl_coeffs(const CL &L, int b, int i, int j) {
    CNb a;
    a.w = i > 0 ? L.xl[b] : 0.0f;
    a.e = i + 1 < L.nx ? L.xu[b + 1] : 0.0f;
    a.s = j > 0 ? L.yl[b] : 0.0f;
    a.n = j + 1 < L.ny ? L.yu[b + L.nx] : 0.0f;
    return a;
}

// sum over the four neighbours of a_nb x_nb (x: one component's array)
__device__ __forceinline__ float cl_nb(const CL &L, const CNb &a, const float *__restrict__ x, int b, int i,
                                       int j) {
    float s = 0.0f;
    if (i > 0) s += a.w * x[b - 1];
    if (i + 1 < L.nx) s += a.e * x[b + 1];
    if (j > 0) s += a.s * x[b - L.nx];
    if (j + 1 < L.ny) s += a.n * x[b + L.nx];
    return s;
}

// level 0 from the FP64 matrix, then the Galerkin coarse levels
__device__ void case_mg_build(const BMg &mg, int cb, int N, bool sym, const double *__restrict__ diag,
                              const double *__restrict__ upper, const double *__restrict__ lower) {
    const CL L0 = case_level(mg, cb, 0, sym);
    const int *cell = mg.cell + mg.cellOff[cb];
    for (int b = threadIdx.x; b < L0.n; b += blockDim.x) {
        const int c = cell[b];
        float dg = 0.0f, xl = 0.0f, yl = 0.0f, xu = 0.0f, yu = 0.0f;
        if (c >= 0) {
            dg = (float)diag[c];
            // the face to the lower neighbour c': A[c][c'] = lower, A[c'][c] = upper
            const int fy = mg.faceLo[c], fx = mg.faceLo[N + c];
            if (fy >= 0) {
                yl = (float)lower[fy];
                if (!sym) yu = (float)upper[fy];
            }
            if (fx >= 0) {
                xl = (float)lower[fx];
                if (!sym) xu = (float)upper[fx];
            }
        }
        L0.dg[b] = dg;
        L0.xl[b] = xl;
        L0.yl[b] = yl;
        if (!sym) {
            L0.xu[b] = xu;
            L0.yu[b] = yu;
        }
    }
    __syncthreads();
    const int nL = mg.nl[cb];
    for (int l = 1; l < nL; ++l) {
        const CL F = case_level(mg, cb, l - 1, sym), C = case_level(mg, cb, l, sym);
        const int fx = F.nx == C.nx ? 1 : 2, fy = F.ny == C.ny ? 1 : 2;
        for (int B = threadIdx.x; B < C.n; B += blockDim.x) {
            const int I = B % C.nx, J = B / C.nx;
            float dg = 0.0f, xl = 0.0f, yl = 0.0f, xu = 0.0f, yu = 0.0f;
            for (int dj = 0; dj < fy; ++dj)
                for (int di = 0; di < fx; ++di) {
                    const int i = I * fx + di, j = J * fy + dj;
                    if (i >= F.nx || j >= F.ny) continue;
                    const int b = i + F.nx * j;
                    const float d = F.dg[b];
                    if (d == 0.0f) continue;
                    dg += d;
                    // a coupling inside the aggregate adds both directions
                    // to the diagonal, one across its faces to the coupling
                    if (di == 1) {
                        dg += F.xl[b] + F.xu[b];
                    } else {
                        xl += F.xl[b];
                        xu += F.xu[b];
                    }
                    if (dj == 1) {
                        dg += F.yl[b] + F.yu[b];
                    } else {
                        yl += F.yl[b];
                        yu += F.yu[b];
                    }
                }
            C.dg[B] = dg;
            C.xl[B] = I > 0 ? xl : 0.0f;
            C.yl[B] = J > 0 ? yl : 0.0f;
            if (!sym) {
                C.xu[B] = I > 0 ? xu : 0.0f;
                C.yu[B] = J > 0 ? yu : 0.0f;
            }
        }
        __syncthreads();
    }
}

// one red-black half-sweep of a level (colour 0: i + j even), the
// components in m; the CTA's threads walk the colour's cells only (row j
// holds them at i = (colour + j) % 2, +2, ...)
template <int KB>
__device__ __forceinline__ void cl_smooth(const CL &L, int colour, unsigned m) {
    const int hx = (L.nx + 1) >> 1, nh = hx * L.ny;
    if constexpr (KB == 0) {   // one cell at a time (fewest registers)
        for (int t = threadIdx.x; t < nh; t += blockDim.x) {
            const int j = t / hx;
            const int i = 2 * (t - j * hx) + ((colour + j) & 1);
            if (i >= L.nx) continue;
            const int b = i + L.nx * j;
            const float d = L.dg[b];
            if (d == 0.0f) continue;
            const CNb a = cl_coeffs(L, b, i, j);
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if ((m >> k) & 1u) {
                    float *x = L.x + k * L.np;
                    x[b] = (L.b[k * L.np + b] - cl_nb(L, a, x, b, i, j)) / d;
                }
        }
        __syncthreads();
        return;
    } else {
        // KB cells a thread per round: every load of the round before its
        // stores (the colour's cells read only the other colour's x, so no store
        // of a round feeds a load of it), one memory latency a round instead of
        // one a cell
        for (int t0 = threadIdx.x; t0 < nh; t0 += KB * blockDim.x) {
            int bb[KB];
            float v[KB][3];
#pragma unroll
            for (int u = 0; u < KB; ++u) {
                const int t = t0 + u * (int)blockDim.x;
                bb[u] = -1;
                if (t >= nh) continue;
                const int j = t / hx;
                const int i = 2 * (t - j * hx) + ((colour + j) & 1);
                if (i >= L.nx) continue;
                const int b = i + L.nx * j;
                // the box arrays hold every position (zero outside the mesh), so
                // the loads need not wait for the diagonal's test
                const float d = L.dg[b];
                const CNb a = cl_coeffs(L, b, i, j);
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    if ((m >> k) & 1u) {
                        const float *x = L.x + k * L.np;
                        v[u][k] = L.b[k * L.np + b] - cl_nb(L, a, x, b, i, j);
                    }
                if (d != 0.0f) {
                    bb[u] = b;
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        if ((m >> k) & 1u) v[u][k] = v[u][k] / d;
                }
            }
#pragma unroll
            for (int u = 0; u < KB; ++u)
                if (bb[u] >= 0)
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        if ((m >> k) & 1u) L.x[k * L.np + bb[u]] = v[u][k];
        }
        __syncthreads();
    }
}

// w = V-cycle(r) on the case's cells for the components in m (FP32 vectors
// in cell order, component k at k N); KB: cells a thread smooths per round
template <class V, int KB>
__device__ void case_mg_apply(const BMg &mg, int cb, int N, bool sym, unsigned m, const V *__restrict__ r,
                              V *__restrict__ w) {
    const int nL = mg.nl[cb];
    const int *cell = mg.cell + mg.cellOff[cb];
    {   // level 0 from x = 0: b, then the red half-sweep
        const CL L = case_level(mg, cb, 0, sym);
        for (int b = threadIdx.x; b < L.n; b += blockDim.x) {
            const int c = cell[b];
            const float d = L.dg[b];
            const bool red = (((b % L.nx) + (b / L.nx)) & 1) == 0 && d != 0.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if ((m >> k) & 1u) {
                    const float rb = c >= 0 ? (float)r[(size_t)k * N + c] : 0.0f;
                    L.b[k * L.np + b] = rb;
                    L.x[k * L.np + b] = red ? rb / d : 0.0f;
                }
        }
        __syncthreads();
    }
    for (int l = 0; l + 1 < nL; ++l) {
        const CL F = case_level(mg, cb, l, sym), C = case_level(mg, cb, l + 1, sym);
        for (int nu = 0; nu < kBMgNu; ++nu) {
            if (l > 0 || nu > 0) cl_smooth<KB>(F, 0, m);
            cl_smooth<KB>(F, 1, m);
        }
        const int fx = F.nx == C.nx ? 1 : 2, fy = F.ny == C.ny ? 1 : 2;
        for (int B = threadIdx.x; B < C.n; B += blockDim.x) {   // restriction
            const int I = B % C.nx, J = B / C.nx;
            float s[3] = {0.0f, 0.0f, 0.0f};
            for (int dj = 0; dj < fy; ++dj)
                for (int di = 0; di < fx; ++di) {
                    const int i = I * fx + di, j = J * fy + dj;
                    if (i >= F.nx || j >= F.ny) continue;
                    const int b = i + F.nx * j;
                    const float d = F.dg[b];
                    if (d == 0.0f) continue;
                    const CNb a = cl_coeffs(F, b, i, j);
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        if ((m >> k) & 1u) {
                            const float *x = F.x + k * F.np;
                            s[k] += F.b[k * F.np + b] - d * x[b] - cl_nb(F, a, x, b, i, j);
                        }
                }
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if ((m >> k) & 1u) {
                    C.b[k * C.np + B] = s[k];
                    C.x[k * C.np + B] = 0.0f;
                }
        }
        __syncthreads();
    }
    {   // the coarsest level: symmetric sweeps (red, black, black, red)
        const CL L = case_level(mg, cb, nL - 1, sym);
        if (nL == 1) {
            for (int b = threadIdx.x; b < L.n; b += blockDim.x)
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    if ((m >> k) & 1u) L.x[k * L.np + b] = 0.0f;
            __syncthreads();
        }
        for (int s = 0; s < kBMgCoarseSweeps; ++s) {
            cl_smooth<KB>(L, 0, m);
            cl_smooth<KB>(L, 1, m);
            cl_smooth<KB>(L, 1, m);
            cl_smooth<KB>(L, 0, m);
        }
    }
    for (int l = nL - 2; l >= 0; --l) {
        const CL F = case_level(mg, cb, l, sym), C = case_level(mg, cb, l + 1, sym);
        for (int b = threadIdx.x; b < F.n; b += blockDim.x) {   // prolongation
            if (F.dg[b] == 0.0f) continue;
            const int i = b % F.nx, j = b / F.nx;
            const int I = F.nx == C.nx ? i : i / 2, J = F.ny == C.ny ? j : j / 2;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if ((m >> k) & 1u) F.x[k * F.np + b] += kBMgOver * C.x[k * C.np + I + C.nx * J];
        }
        __syncthreads();
        for (int nu = 0; nu < kBMgNu; ++nu) {
            cl_smooth<KB>(F, 1, m);
            cl_smooth<KB>(F, 0, m);
        }
    }
    {   // level 0's result to w (cell order)
        const CL L = case_level(mg, cb, 0, sym);
        for (int b = threadIdx.x; b < L.n; b += blockDim.x) {
            const int c = cell[b];
            if (c < 0) continue;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if ((m >> k) & 1u) w[(size_t)k * N + c] = (V)L.x[k * L.np + b];
        }
        __syncthreads();
    }
}

// ---- the persistent per-case PCG -------------------------------------------
// One CTA per case runs the case's whole pressure solve (one component,
// structured 2-D cases with at most 8 j-blocks): the operations of
// BSolver::pcg_iteration, replayed until the case stops, with __syncthreads
// between the phases instead of kernel boundaries, and every reduction of the
// case as one pass of the CTA (each thread sums its cells, then one block
// tree; the launch path sums 256-cell blocks first, so the two differ in the
// last bits).  Every scalar decision is the launch path's.
constexpr int kCaseThreads = 512;
template <class V>
constexpr int kCaseP = sizeof(V) == 4 ? 8 : 4;   // sweep chunk of the pressure solve
// the sweeps of the persistent solvers stage their chunks in shared memory
// (cp.async) NB - 1 chunks ahead; the momentum solve runs two components'
// sweeps side by side (16 warps), with shorter chunks
constexpr int kCaseNB = 4;
template <class V>
constexpr int kBicgP = sizeof(V) == 4 ? 8 : 4;
template <class V>
constexpr int kBicgNB = sizeof(V) == 4 ? 3 : 2;
template <class V, int NC, int P, int NB>
__host__ __device__ constexpr int case_stage_bytes() {   // one warp's staging area, the larger of the two sweeps
    return s2d::stage_bytes<V, 0, NC, P, NB>() > s2d::stage_bytes<V, 1, NC, P, NB>()
               ? s2d::stage_bytes<V, 0, NC, P, NB>()
               : s2d::stage_bytes<V, 1, NC, P, NB>();
}
constexpr int kU = 4;                            // cells per thread whose loads are issued together
constexpr int kUA = 4;                           // the same for q = A p
constexpr int kSlots = 4;                        // ELL width of the 2-D cases

// 16-byte packs of a vector: four FP32 or two FP64 values, one load or store
template <class V> struct Pack;
template <> struct Pack<float> { using T = float4; static constexpr int n = 4; };
template <> struct Pack<double> { using T = double2; static constexpr int n = 2; };
__device__ __forceinline__ void ldp(const float *p, float (&v)[4]) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ldp(const double *p, double (&v)[2]) {
    const double2 a = *reinterpret_cast<const double2 *>(p);
    v[0] = a.x; v[1] = a.y;
}
__device__ __forceinline__ void stp(float *p, const float (&v)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void stp(double *p, const double (&v)[2]) {
    *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
}
// the pack-aligned part [a, b) of the cell range [c0, c1) (the vectors are
// 128-byte aligned); the rest, at most a pack at each end, goes cell by cell
__device__ __forceinline__ void pack_bounds(int c0, int c1, int n, int &a, int &b) {
    a = min(c1, (c0 + n - 1) / n * n);
    b = max(a, c1 / n * n);
}

// the bounded-wait error flag as one value for the whole CTA (another CTA
// may set it at any time: every thread must take the same branch)
__device__ bool case_error(const int *err) {
    __shared__ int sv;
    __syncthreads();
    if (threadIdx.x == 0) sv = *(volatile const int *)err;
    __syncthreads();
    return sv != 0;
}

// the matrix coefficient of each ELL slot of the case's cells, in the
// vector type (0 past a row's end), so that A x reads it beside the slot's
// neighbour instead of through the face; ends with a barrier
template <class V>
__device__ void case_ell_coefficients(const BEll &e, int N, int c0, int c1, const V *__restrict__ u32,
                                      const V *__restrict__ l32, V *__restrict__ aEll) {
    for (int c = c0 + (int)threadIdx.x; c < c1; c += blockDim.x) {
#pragma unroll
        for (int s = 0; s < kSlots; ++s) {
            const int nb = s < e.nSlots ? __ldg(e.nbr + (size_t)s * N + c) : -1;
            const int f = s < e.nSlots ? __ldg(e.face + (size_t)s * N + c) : -1;
            aEll[(size_t)s * N + c] = nb >= 0 ? V(nb > c ? u32[f] : l32[f]) : V(0);
        }
    }
    __syncthreads();
}

// the CTA's sum, valid in every thread
__device__ double case_total(double v) {
    __shared__ double sv;
    const double t = bsum(v);
    if (threadIdx.x == 0) sv = t;
    __syncthreads();
    const double r = sv;
    __syncthreads();
    return r;
}

template <class V>
__global__ void __launch_bounds__(kCaseThreads, 1) k_b_pcg_case(BTab t, BEll e, Skew2D<V> g, BSeg S, Ctl ctl, int mixed,
                                                              const V *__restrict__ d32, const V *__restrict__ u32,
                                                              const V *__restrict__ l32,
                                                              const double *__restrict__ diag,
                                                              const double *__restrict__ upper,
                                                              const double *__restrict__ lower,
                                                              const double *__restrict__ b, double *__restrict__ psi,
                                                              V *__restrict__ r, V *__restrict__ w,
                                                              V *__restrict__ p, V *__restrict__ q,
                                                              V *__restrict__ x, const int *__restrict__ order,
                                                              V *__restrict__ aEll, BMg mg, int *err,
                                                              long long maxSpin, int cap) {
    using Acc = typename AccOf<V>::type;
    __shared__ s2d::u64 ring[8 * s2d::kRJ * s2d::W<V>::n];
    __shared__ int sProg[32];
    extern __shared__ __align__(16) unsigned char stageSmem[];   // 8 warps' sweep staging
    const int cb = order[blockIdx.x], sg = cb * 8, tid = threadIdx.x, nt = blockDim.x, N = t.N;
    const int c0 = t.blkCell0[t.caseBlk[cb]], c1 = t.blkCell1[t.caseBlk[cb + 1] - 1];
    const long long e0 = g.off[cb], e1 = e0 + (long long)g.JB[cb] * g.T[cb] * 32;
    case_ell_coefficients(e, N, c0, c1, u32, l32, aEll);
    // the FP32 form may take the multigrid V-cycle in place of the DIC sweeps
    const bool useMg = sizeof(V) == 4 && mg.on;
    if (useMg) case_mg_build(mg, cb, N, true, diag, upper, lower);
    for (int it = 0; it < cap; ++it) {
        __syncthreads();
        if (!S.active[sg]) break;
        if (useMg) {
            case_mg_apply<V, kMgPcgB>(mg, cb, N, true, 1u, r, w);
        } else {
        // ---- w = M^-1 r: gather, forward and backward sweeps of this case
        for (long long i0 = e0 + tid; i0 < e1; i0 += (long long)kU * nt) {
            int cc[kU];
            V v[kU];
#pragma unroll
            for (int k = 0; k < kU; ++k) {
                const long long i = i0 + (long long)k * nt;
                cc[k] = i < e1 ? __ldg(g.cellOf + i) : -1;
            }
#pragma unroll
            for (int k = 0; k < kU; ++k) v[k] = cc[k] >= 0 ? r[cc[k]] : V(0);
#pragma unroll
            for (int k = 0; k < kU; ++k)
                if (i0 + (long long)k * nt < e1) g.rS[i0 + (long long)k * nt] = v[k];
        }
        for (int mode = 0; mode < 2; ++mode) {
            s2d::reset<V, 1>(ring, 8, sProg);
            __syncthreads();
            if (mode == 0)
                sweep2d_cta<V, 0, 1, kCaseP<V>, true, s2d::kRJ, kCaseNB>(g, cb, 1u, nullptr, N, err, maxSpin, ring,
                                                                         sProg, 0, stageSmem);
            else
                sweep2d_cta<V, 1, 1, kCaseP<V>, true, s2d::kRJ, kCaseNB>(g, cb, 1u, w, N, err, maxSpin, ring, sProg,
                                                                         0, stageSmem);
            __syncthreads();
        }
        if (case_error(err)) break;
        }
        // ---- rho = w.r (and w.q_old in the flexible form)
        constexpr int PN = Pack<V>::n;
        int pa, pb;
        pack_bounds(c0, c1, PN, pa, pb);
        Acc a0, a1;
        {
            auto one = [&](int c) {
                const V wc = w[c];
                acc_dot(a0, wc, r[c]);
                if (mixed) acc_dot(a1, wc, q[c]);
            };
            for (int c = c0 + tid; c < pa; c += nt) one(c);
            for (int c = pb + tid; c < c1; c += nt) one(c);
#pragma unroll 2
            for (int g = pa + tid * PN; g < pb; g += nt * PN) {
                V wv[PN], rv[PN], qv[PN];
                ldp(w + g, wv);
                ldp(r + g, rv);
                if (mixed) ldp(q + g, qv);
#pragma unroll
                for (int j = 0; j < PN; ++j) {
                    acc_dot(a0, wv[j], rv[j]);
                    if (mixed) acc_dot(a1, wv[j], qv[j]);
                }
            }
        }
        const double rho = case_total(acc_value(a0));
        const double wq = mixed ? case_total(acc_value(a1)) : 0.0;
        if (tid == 0) {   // k_b_pcg_a
            const double aold = S.A[sg];
            S.Aold[sg] = aold;
            S.A[sg] = rho;
            S.beta[sg] = mixed ? -S.alpha[sg] * wq / aold : rho / aold;
        }
        __syncthreads();
        // ---- p = w (+ beta p)
        {
            const bool first = S.iter[sg] == 0;
            const V beta = V(S.beta[sg]);
            auto one = [&](int c) { p[c] = first ? w[c] : fma(beta, p[c], w[c]); };
            for (int c = c0 + tid; c < pa; c += nt) one(c);
            for (int c = pb + tid; c < c1; c += nt) one(c);
#pragma unroll 2
            for (int g = pa + tid * PN; g < pb; g += nt * PN) {
                V wv[PN], pv[PN];
                ldp(w + g, wv);
                if (!first) ldp(p + g, pv);
#pragma unroll
                for (int j = 0; j < PN; ++j) pv[j] = first ? wv[j] : fma(beta, pv[j], wv[j]);
                stp(p + g, pv);
            }
        }
        __syncthreads();
        // ---- q = A p (the vector type's matrix copy; FP32: differences form); p.q
        // two rounds of independent loads per kUA cells: the ELL slots (the
        // rows end in -1 padding, which adds nothing) with their coefficients
        // and the cells' own values, then the neighbours' values
        Acc aq;
        for (int ci = c0 + tid; ci < c1; ci += kUA * nt) {
            int nb[kUA][kSlots];
            V cf[kUA][kSlots], pc[kUA], dc[kUA];
#pragma unroll
            for (int k = 0; k < kUA; ++k) {
                const int c = ci + k * nt;
                const bool in = c < c1;
#pragma unroll
                for (int s = 0; s < kSlots; ++s) {
                    const bool sl = in && s < e.nSlots;
                    nb[k][s] = sl ? __ldg(e.nbr + (size_t)s * N + c) : -1;
                    cf[k][s] = sl ? aEll[(size_t)s * N + c] : V(0);
                }
                pc[k] = in ? p[c] : V(0);
                dc[k] = in ? V(d32[c]) : V(0);
            }
            V pn[kUA][kSlots];
#pragma unroll
            for (int k = 0; k < kUA; ++k)
#pragma unroll
                for (int s = 0; s < kSlots; ++s) pn[k][s] = nb[k][s] >= 0 ? p[nb[k][s]] : V(0);
#pragma unroll
            for (int k = 0; k < kUA; ++k) {
                const int c = ci + k * nt;
                if (c >= c1) continue;
                V acc = dc[k] * pc[k];
#pragma unroll
                for (int s = 0; s < kSlots; ++s)
                    if (nb[k][s] >= 0) acc = fma(cf[k][s], sizeof(V) == 4 ? pn[k][s] - pc[k] : pn[k][s], acc);
                q[c] = acc;
                acc_dot(aq, acc, pc[k]);
            }
        }
        const double wApA = case_total(acc_value(aq));
        if (tid == 0) {   // k_b_pcg_alpha
            if (fabs(wApA) / S.nf[sg] < 1e-300) {
                S.sing[sg] = 1;
                S.alpha[sg] = 0.0;
            } else {
                S.alpha[sg] = S.A[sg] / wApA;
            }
        }
        __syncthreads();
        // ---- x += alpha p; r -= alpha q; |r|
        Acc ar;
        {
            const bool sing = S.sing[sg] != 0;
            const V alpha = V(S.alpha[sg]);
            auto one = [&](int c) {
                V rr = r[c];
                if (!sing) {
                    x[c] = fma(alpha, p[c], x[c]);
                    rr = fma(-alpha, q[c], rr);
                    r[c] = rr;
                }
                acc_add(ar, fabs(rr));
            };
            for (int c = c0 + tid; c < pa; c += nt) one(c);
            for (int c = pb + tid; c < c1; c += nt) one(c);
#pragma unroll 2
            for (int g = pa + tid * PN; g < pb; g += nt * PN) {
                V rv[PN], xv[PN], pv[PN], qv[PN];
                ldp(r + g, rv);
                if (!sing) {
                    ldp(x + g, xv);
                    ldp(p + g, pv);
                    ldp(q + g, qv);
#pragma unroll
                    for (int j = 0; j < PN; ++j) {
                        xv[j] = fma(alpha, pv[j], xv[j]);
                        rv[j] = fma(-alpha, qv[j], rv[j]);
                    }
                    stp(x + g, xv);
                    stp(r + g, rv);
                }
#pragma unroll
                for (int j = 0; j < PN; ++j) acc_add(ar, fabs(rv[j]));
            }
        }
        const double rs = case_total(acc_value(ar));
        if (tid == 0) {   // k_b_iter_fin
            if (S.sing[sg]) {
                S.active[sg] = 0;
            } else {
                const double fin = rs / S.nf[sg];
                S.fin[sg] = fin;
                S.iter[sg] += 1;
                if (mixed) {
                    S.repl[sg] = (fin < kReplaceB * S.last[sg] || bconv(ctl, fin, S.init[sg]) ||
                                  S.iter[sg] >= ctl.maxIter || !isfinite(fin)) ? 1 : 0;
                } else {
                    const bool c = bconv(ctl, fin, S.init[sg]);
                    const bool more = (S.iter[sg] < ctl.maxIter && !c) || S.iter[sg] < ctl.minIter;
                    S.conv[sg] = c ? 1 : 0;
                    if (!more || !isfinite(fin)) S.active[sg] = 0;
                }
            }
        }
        __syncthreads();
        // ---- residual replacement (mixed): psi += x, x = 0, r = b - A psi
        if (S.repl[sg]) {
            for (int c = c0 + tid; c < c1; c += nt) {
                psi[c] += (double)x[c];
                x[c] = V(0);
            }
            __syncthreads();
            double vt = 0.0;
            for (int c = c0 + tid; c < c1; c += nt) {
                const double rr = b[c] - brow_mul(e, c, diag, upper, lower, psi);
                r[c] = (V)rr;
                vt += fabs(rr);
            }
            const double rt = case_total(vt);
            if (tid == 0 && S.active[sg]) {   // k_b_after
                const double fin = rt / S.nf[sg];
                S.fin[sg] = fin;
                S.last[sg] = fin;
                const bool c = bconv(ctl, fin, S.init[sg]);
                const bool more = (S.iter[sg] < ctl.maxIter && !c) || S.iter[sg] < ctl.minIter;
                S.conv[sg] = c ? 1 : 0;
                if (!more || !isfinite(fin)) S.active[sg] = 0;
            }
        }
        if (tid == 0) S.repl[sg] = 0;
    }
}

// ---- the persistent per-case BiCGStab -------------------------------------
// One CTA per case runs the momentum solve of its components (up to three,
// the valid ones of vm) through every iteration: the operations and scalar
// decisions of BSolver::bicg_iteration for each segment (case, component),
// including the half-step exit and the residual replacements of the mixed
// form, with one-pass reductions per case.

// the CTA's sums of n values, valid in every thread (each warp reduces the
// warp totals itself, so all warps agree)
template <int n>
__device__ void case_totals(double (&v)[n]) {
    __shared__ double sh[n][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < n; ++i)
        for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < n; ++i) sh[i][wid] = v[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < n; ++i) {
        double t = lane < nw ? sh[i][lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        v[i] = t;
    }
    __syncthreads();
}

// For every component k in m (up to three): one(k, i) for the cells of
// [k N + c0, k N + c1) outside its 16-byte-aligned part, pack(k, i) for each
// pack of PN cells starting at i inside it
template <int PN, class One, class PackFn>
__device__ __forceinline__ void comp_packs(int c0, int c1, int N, unsigned m, One one, PackFn pack) {
    const long long nt = blockDim.x;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (!((m >> k) & 1u)) continue;
        const long long lo = (long long)k * N + c0, hi = (long long)k * N + c1;
        const long long a = min(hi, (lo + PN - 1) / PN * PN), b = max(a, hi / PN * PN);
        for (long long i = lo + threadIdx.x; i < a; i += nt) one(k, i);
        for (long long i = b + threadIdx.x; i < hi; i += nt) one(k, i);
#pragma unroll 2
        for (long long i = a + (long long)threadIdx.x * PN; i < b; i += nt * PN) pack(k, i);
    }
}

// y = A x for the components in m (FP32: differences form over the row sums)
template <class V>
__device__ void case_amul(const BEll &e, int N, int c0, int c1, unsigned m, const V *__restrict__ d32,
                          const V *__restrict__ aEll, const V *__restrict__ x, V *__restrict__ y) {
    const int nt = blockDim.x;
#pragma unroll 2
    for (int c = c0 + (int)threadIdx.x; c < c1; c += nt) {
        int nb[kSlots];
        V cf[kSlots];
#pragma unroll
        for (int s = 0; s < kSlots; ++s) {
            const bool sl = s < e.nSlots;
            nb[s] = sl ? __ldg(e.nbr + (size_t)s * N + c) : -1;
            cf[s] = sl ? aEll[(size_t)s * N + c] : V(0);
        }
        const V dc = d32[c];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (!((m >> k) & 1u)) continue;
            const size_t o = (size_t)k * N;
            const V xc = x[o + c];
            V xn[kSlots];
#pragma unroll
            for (int s = 0; s < kSlots; ++s) xn[s] = nb[s] >= 0 ? x[o + nb[s]] : V(0);
            V acc = dc * xc;
#pragma unroll
            for (int s = 0; s < kSlots; ++s)
                if (nb[s] >= 0) acc = fma(cf[s], sizeof(V) == 4 ? xn[s] - xc : xn[s], acc);
            y[o + c] = acc;
        }
    }
}

// w = M^-1 r for the components in m (gather, forward and backward sweeps):
// the sweeps of two components at a time, each by its own half of the CTA
// (warps 0-7 and 8-15, one per j-block) with its own ring and counters
template <class V>
__device__ void case_precondition(const Skew2D<V> &g, int cb, int N, unsigned m, const V *__restrict__ r,
                                  V *__restrict__ w, int *err, long long maxSpin, s2d::u64 *ring, int *sProg,
                                  unsigned char *stage) {
    const long long e0 = g.off[cb], e1 = e0 + (long long)g.JB[cb] * g.T[cb] * 32;
    const int nt = blockDim.x;
    for (long long i0 = e0 + threadIdx.x; i0 < e1; i0 += (long long)kU * nt) {
        int cc[kU];
        V v[kU][3];
#pragma unroll
        for (int j = 0; j < kU; ++j) {
            const long long i = i0 + (long long)j * nt;
            cc[j] = i < e1 ? __ldg(g.cellOf + i) : -1;
        }
#pragma unroll
        for (int j = 0; j < kU; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) v[j][k] = (cc[j] >= 0 && ((m >> k) & 1u)) ? r[(size_t)k * N + cc[j]] : V(0);
#pragma unroll
        for (int j = 0; j < kU; ++j) {
            const long long i = i0 + (long long)j * nt;
            if (i >= e1) continue;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if ((m >> k) & 1u) g.rS[(long long)k * g.nSkew + i] = v[j][k];
        }
    }
    int comps[3], nComp = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if ((m >> k) & 1u) comps[nComp++] = k;
    for (int c0 = 0; c0 < nComp; c0 += 2) {
        const int grp = threadIdx.x >= 256 ? 1 : 0;   // the half of the CTA
        const int k = grp == 0 ? comps[c0] : (c0 + 1 < nComp ? comps[c0 + 1] : -1);
        Skew2D<V> gk = g;
        if (k >= 0) {
            gk.rS += (long long)k * g.nSkew;
            gk.wS += (long long)k * g.nSkew;
        }
        for (int mode = 0; mode < 2; ++mode) {
            s2d::reset<V, 1>(ring, 16, sProg);
            __syncthreads();
            if (k >= 0) {
                s2d::u64 *rg = ring + grp * 8 * s2d::kRJ * s2d::W<V>::n;
                unsigned char *sg = stage + (size_t)grp * 8 * case_stage_bytes<V, 1, kBicgP<V>, kBicgNB<V>>();
                if (mode == 0)
                    sweep2d_cta<V, 0, 1, kBicgP<V>, true, s2d::kRJ, kBicgNB<V>>(gk, cb, 1u, nullptr, N, err, maxSpin, rg,
                                                                             sProg + 8 * grp, 8 * grp, sg);
                else
                    sweep2d_cta<V, 1, 1, kBicgP<V>, true, s2d::kRJ, kBicgNB<V>>(gk, cb, 1u, w + (size_t)k * N, N, err,
                                                                             maxSpin, rg, sProg + 8 * grp, 8 * grp, sg);
            }
            __syncthreads();
        }
    }
}

template <class V>
__global__ void __launch_bounds__(kCaseThreads, 1) k_b_bicg_case(BTab t, BEll e, Skew2D<V> g, BSeg S, Ctl ctl,
                                                              unsigned vm, int mixed, const V *__restrict__ d32,
                                                              const V *__restrict__ u32, const V *__restrict__ l32,
                                                              const double *__restrict__ diag,
                                                              const double *__restrict__ upper,
                                                              const double *__restrict__ lower,
                                                              const double *__restrict__ b, double *__restrict__ psi,
                                                              V *__restrict__ r, const V *__restrict__ r0,
                                                              V *__restrict__ p, V *__restrict__ y,
                                                              V *__restrict__ Ay, V *__restrict__ sv,
                                                              V *__restrict__ z, V *__restrict__ tt,
                                                              V *__restrict__ x, const int *__restrict__ order,
                                                              V *__restrict__ aEll, BMg mg, int *err,
                                                              long long maxSpin, int cap) {
    using Acc = typename AccOf<V>::type;
    constexpr int PN = Pack<V>::n;
    __shared__ s2d::u64 ring[16 * s2d::kRJ * s2d::W<V>::n];   // two halves of the CTA, 8 j-blocks each
    extern __shared__ __align__(16) unsigned char stageSmem[];   // 16 warps' sweep staging
    __shared__ int sProg[32];
    // segment masks that thread 0 publishes, one slot per use, so that no
    // slot is rewritten in an iteration after threads have read it without a
    // barrier in between: [0] iterating, [1] half-step exits, [2] their
    // replacements, [3] full steps, [4] end-of-iteration replacements
    __shared__ unsigned sMask[5];
    const int cb = order[blockIdx.x], tid = threadIdx.x, nt = blockDim.x, N = t.N;
    const int c0 = t.blkCell0[t.caseBlk[cb]], c1 = t.blkCell1[t.caseBlk[cb + 1] - 1];
    const int s0 = cb * 8;
    case_ell_coefficients(e, N, c0, c1, u32, l32, aEll);
    // the FP32 form may take the multigrid V-cycle in place of the DILU sweeps
    const bool useMg = sizeof(V) == 4 && mg.on;
    if (useMg) case_mg_build(mg, cb, N, false, diag, upper, lower);
    // the segments (components) selected by a predicate on their state
    auto seg_mask = [&](auto pred) {
        unsigned mm = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (((vm >> k) & 1u) && pred(s0 + k)) mm |= 1u << k;
        return mm;
    };
    // psi += x, x = 0, r = b - A psi (FP64) on the segments in mr; |r| per segment
    auto replace = [&](unsigned mr, double (&tot)[3]) {
#pragma unroll
        for (int k = 0; k < 3; ++k) tot[k] = 0.0;
        if (!mr) return;
#pragma unroll 4
        for (int c = c0 + tid; c < c1; c += nt)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (!((mr >> k) & 1u)) continue;
                const size_t i = (size_t)k * N + c;
                psi[i] += (double)x[i];
                x[i] = V(0);
            }
        __syncthreads();
#pragma unroll 4
        for (int c = c0 + tid; c < c1; c += nt)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (!((mr >> k) & 1u)) continue;
                const size_t o = (size_t)k * N;
                const double rr = b[o + c] - brow_mul(e, c, diag, upper, lower, psi + o);
                r[o + c] = (V)rr;
                tot[k] += fabs(rr);
            }
        case_totals(tot);
    };
    for (int it = 0; it < cap; ++it) {
        __syncthreads();
        const unsigned act = seg_mask([&](int sg) { return S.active[sg] != 0; });
        if (!act) break;
        // ---- r0r = r0.r; beta, singular stops
        {
            Acc a[3];
            comp_packs<PN>(c0, c1, N, act, [&](int k, long long i) { acc_dot(a[k], r0[i], r[i]); },
                           [&](int k, long long i) {
                               V x[PN], y[PN];
                               ldp(r0 + i, x);
                               ldp(r + i, y);
#pragma unroll
                               for (int j = 0; j < PN; ++j) acc_dot(a[k], x[j], y[j]);
                           });
            double v[3] = {acc_value(a[0]), acc_value(a[1]), acc_value(a[2])};
            case_totals(v);
            if (tid == 0) {   // k_b_bicg_r0r
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    if (!((act >> k) & 1u)) continue;
                    const int sg = s0 + k;
                    const double old = S.r0r[sg], r0r = v[k];
                    S.r0rOld[sg] = old;
                    S.r0r[sg] = r0r;
                    if (fabs(r0r) < 1e-300) { S.sing[sg] = 1; continue; }
                    if (S.iter[sg] > 0 && !S.rst[sg]) {
                        const double om = S.omega[sg];
                        if (fabs(om) < 1e-300) { S.sing[sg] = 1; continue; }
                        S.beta[sg] = (r0r / old) * (S.alpha[sg] / om);
                    }
                }
                sMask[0] = seg_mask([&](int sg) { return S.active[sg] && !S.sing[sg]; });
            }
            __syncthreads();
        }
        const unsigned live = sMask[0];
        // ---- p = r + beta (p - omega Ay)
        {
            bool restart[3];
            V beta[3], omega[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int sg = s0 + k;
                restart[k] = ((live >> k) & 1u) && (S.iter[sg] == 0 || S.rst[sg]);
                beta[k] = V(S.beta[sg]);
                omega[k] = V(S.omega[sg]);
            }
            comp_packs<PN>(c0, c1, N, live,
                           [&](int k, long long i) {
                               p[i] = restart[k] ? r[i] : fma(beta[k], fma(-omega[k], Ay[i], p[i]), r[i]);
                           },
                           [&](int k, long long i) {
                               V rv[PN], av[PN], pv[PN];
                               ldp(r + i, rv);
                               if (!restart[k]) {
                                   ldp(Ay + i, av);
                                   ldp(p + i, pv);
#pragma unroll
                                   for (int j = 0; j < PN; ++j) rv[j] = fma(beta[k], fma(-omega[k], av[j], pv[j]), rv[j]);
                               }
                               stp(p + i, rv);
                           });
        }
        __syncthreads();
        // ---- y = M^-1 p, Ay = A y, alpha = r0r / r0.Ay
        if (useMg) {
            case_mg_apply<V, kMgBicgB>(mg, cb, N, false, vm, p, y);
        } else {
            case_precondition(g, cb, N, vm, p, y, err, maxSpin, ring, sProg, stageSmem);
            if (case_error(err)) break;
        }
        case_amul(e, N, c0, c1, vm, d32, aEll, y, Ay);
        __syncthreads();
        {
            Acc a[3];
            comp_packs<PN>(c0, c1, N, live, [&](int k, long long i) { acc_dot(a[k], r0[i], Ay[i]); },
                           [&](int k, long long i) {
                               V x[PN], y[PN];
                               ldp(r0 + i, x);
                               ldp(Ay + i, y);
#pragma unroll
                               for (int j = 0; j < PN; ++j) acc_dot(a[k], x[j], y[j]);
                           });
            double v[3] = {acc_value(a[0]), acc_value(a[1]), acc_value(a[2])};
            case_totals(v);
            if (tid == 0)   // k_b_bicg_alpha
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    if (!((live >> k) & 1u)) continue;
                    S.alpha[s0 + k] = S.r0r[s0 + k] / v[k];
                    S.rst[s0 + k] = 0;
                }
            __syncthreads();
        }
        // ---- s = r - alpha Ay; the half-step test on |s|
        {
            Acc a[3];
            V alpha[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) alpha[k] = V(S.alpha[s0 + k]);
            comp_packs<PN>(c0, c1, N, live,
                           [&](int k, long long i) {
                               const V sk = fma(-alpha[k], Ay[i], r[i]);
                               sv[i] = sk;
                               acc_add(a[k], fabs(sk));
                           },
                           [&](int k, long long i) {
                               V av[PN], rv[PN];
                               ldp(Ay + i, av);
                               ldp(r + i, rv);
#pragma unroll
                               for (int j = 0; j < PN; ++j) {
                                   rv[j] = fma(-alpha[k], av[j], rv[j]);
                                   acc_add(a[k], fabs(rv[j]));
                               }
                               stp(sv + i, rv);
                           });
            double v[3] = {acc_value(a[0]), acc_value(a[1]), acc_value(a[2])};
            case_totals(v);
            if (tid == 0) {   // k_b_bicg_half
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int sg = s0 + k;
                    if (!((vm >> k) & 1u) || !S.active[sg]) continue;
                    if (S.sing[sg]) {
                        S.active[sg] = 0;
                        continue;
                    }
                    const double fs = v[k] / S.nf[sg];
                    if (bconv(ctl, fs, S.init[sg])) {
                        S.conv[sg] = 2;
                        S.repl[sg] = mixed ? 1 : 0;
                        if (!mixed) S.fin[sg] = fs;
                    }
                }
                sMask[1] = seg_mask([&](int sg) { return S.conv[sg] == 2; });
                sMask[2] = seg_mask([&](int sg) { return S.repl[sg] != 0; });
            }
            __syncthreads();
        }
        // ---- half-step exit: x += alpha y; replacement; stop or restart
        {
            const unsigned half = sMask[1], mr = sMask[2];
            if (half) {
#pragma unroll 4
                for (int c = c0 + tid; c < c1; c += nt)
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        if (!((half >> k) & 1u)) continue;
                        const size_t i = (size_t)k * N + c;
                        x[i] = fma(V(S.alpha[s0 + k]), y[i], x[i]);
                    }
                __syncthreads();
            }
            double tot[3];
            replace(mr, tot);
            if (tid == 0) {   // k_b_half_after
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int sg = s0 + k;
                    if (!((vm >> k) & 1u) || !S.active[sg] || S.conv[sg] != 2) continue;
                    if (!mixed) {
                        S.iter[sg] += 1;
                        S.conv[sg] = 1;
                        S.active[sg] = 0;
                        continue;
                    }
                    const double fin = tot[k] / S.nf[sg];
                    S.fin[sg] = fin;
                    S.last[sg] = fin;
                    S.repl[sg] = 0;
                    const int itn = S.iter[sg] + 1;
                    const bool c = bconv(ctl, fin, S.init[sg]);
                    if ((c && itn >= ctl.minIter) || itn >= ctl.maxIter || !isfinite(fin)) {
                        S.iter[sg] = itn;
                        S.conv[sg] = c ? 1 : 0;
                        S.active[sg] = 0;
                    } else {
                        S.rst[sg] = 1;
                    }
                }
                sMask[3] = seg_mask([&](int sg) { return S.active[sg] && !S.sing[sg] && S.conv[sg] != 2; });
            }
            __syncthreads();
        }
        const unsigned full = sMask[3];
        // ---- z = M^-1 s, tt = A z, omega = tt.s / tt.tt
        if (useMg) {
            case_mg_apply<V, kMgBicgB>(mg, cb, N, false, vm, sv, z);
        } else {
            case_precondition(g, cb, N, vm, sv, z, err, maxSpin, ring, sProg, stageSmem);
            if (case_error(err)) break;
        }
        case_amul(e, N, c0, c1, vm, d32, aEll, z, tt);
        __syncthreads();
        {
            Acc a[6];
            const unsigned on = seg_mask([&](int sg) { return S.active[sg] != 0; });
            comp_packs<PN>(c0, c1, N, on,
                           [&](int k, long long i) {
                               const V tk = tt[i];
                               acc_dot(a[k], tk, tk);
                               acc_dot(a[3 + k], tk, sv[i]);
                           },
                           [&](int k, long long i) {
                               V tv[PN], svv[PN];
                               ldp(tt + i, tv);
                               ldp(sv + i, svv);
#pragma unroll
                               for (int j = 0; j < PN; ++j) {
                                   acc_dot(a[k], tv[j], tv[j]);
                                   acc_dot(a[3 + k], tv[j], svv[j]);
                               }
                           });
            double v[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) v[i] = acc_value(a[i]);
            case_totals(v);
            if (tid == 0)   // k_b_bicg_omega
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    if ((full >> k) & 1u) S.omega[s0 + k] = v[3 + k] / v[k];
            __syncthreads();
        }
        // ---- x += alpha y + omega z; r = s - omega tt; |r|; the stopping test
        {
            Acc a[3];
            V alpha[3], omega[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                alpha[k] = V(S.alpha[s0 + k]);
                omega[k] = V(S.omega[s0 + k]);
            }
            comp_packs<PN>(c0, c1, N, full,
                           [&](int k, long long i) {
                               x[i] = fma(alpha[k], y[i], fma(omega[k], z[i], x[i]));
                               const V rv = fma(-omega[k], tt[i], sv[i]);
                               r[i] = rv;
                               acc_add(a[k], fabs(rv));
                           },
                           [&](int k, long long i) {
                               V yv[PN], zv[PN], xv[PN], tv[PN], svv[PN];
                               ldp(y + i, yv);
                               ldp(z + i, zv);
                               ldp(x + i, xv);
                               ldp(tt + i, tv);
                               ldp(sv + i, svv);
#pragma unroll
                               for (int j = 0; j < PN; ++j) {
                                   xv[j] = fma(alpha[k], yv[j], fma(omega[k], zv[j], xv[j]));
                                   svv[j] = fma(-omega[k], tv[j], svv[j]);
                                   acc_add(a[k], fabs(svv[j]));
                               }
                               stp(x + i, xv);
                               stp(r + i, svv);
                           });
            double v[3] = {acc_value(a[0]), acc_value(a[1]), acc_value(a[2])};
            case_totals(v);
            if (tid == 0) {   // k_b_iter_fin (skipHalf)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int sg = s0 + k;
                    if (!((vm >> k) & 1u) || !S.active[sg]) continue;
                    if (S.conv[sg] == 2) {
                        S.iter[sg] += 1;
                        S.conv[sg] = 0;
                        continue;
                    }
                    if (S.sing[sg]) {
                        S.active[sg] = 0;
                        continue;
                    }
                    const double fin = v[k] / S.nf[sg];
                    S.fin[sg] = fin;
                    S.iter[sg] += 1;
                    if (mixed) {
                        S.repl[sg] = (fin < kReplaceB * S.last[sg] || bconv(ctl, fin, S.init[sg]) ||
                                      S.iter[sg] >= ctl.maxIter || !isfinite(fin)) ? 1 : 0;
                    } else {
                        const bool c = bconv(ctl, fin, S.init[sg]);
                        const bool more = (S.iter[sg] < ctl.maxIter && !c) || S.iter[sg] < ctl.minIter;
                        S.conv[sg] = c ? 1 : 0;
                        if (!more || !isfinite(fin)) S.active[sg] = 0;
                    }
                }
                sMask[4] = seg_mask([&](int sg) { return S.repl[sg] != 0; });
            }
            __syncthreads();
        }
        // ---- replacement; k_b_after
        {
            double tot[3];
            const unsigned mr = sMask[4];
            replace(mr, tot);
            if (tid == 0)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int sg = s0 + k;
                    if (!((vm >> k) & 1u)) continue;
                    if (S.active[sg] && S.repl[sg]) {
                        const double fin = tot[k] / S.nf[sg];
                        S.fin[sg] = fin;
                        S.last[sg] = fin;
                        const bool c = bconv(ctl, fin, S.init[sg]);
                        const bool more = (S.iter[sg] < ctl.maxIter && !c) || S.iter[sg] < ctl.minIter;
                        S.conv[sg] = c ? 1 : 0;
                        if (!more || !isfinite(fin)) S.active[sg] = 0;
                    }
                    S.repl[sg] = 0;
                }
        }
    }
}

// ---- host side --------------------------------------------------------------
template <class V>
struct BSolver {
    rt_ctx *ctx;
    const SolveArgs &a;
    Batch &bt;
    cudaStream_t st;
    BTab t;
    BEll e;
    BSeg S;
    Ctl ctl;
    int N, F, nSeg;
    int mixed = sizeof(V) == 4;   // FP32 vectors: residual replacement
    unsigned vm;
    V *vec, *d32, *u32, *l32, *rD, *aEll;
    double *rD64, *partial, *res;

    BSolver(rt_ctx *c, const SolveArgs &args) : ctx(c), a(args), bt(c->mesh.batch) {
        const DevMesh &m = ctx->mesh;
        st = ctx->stream;
        N = m.N;
        F = m.F;
        nSeg = 8 * bt.n;
        vm = a.validMask;
        t = BTab{N, bt.nBlk, bt.n, bt.blkCase.p, bt.blkCell0.p, bt.blkCell1.p, bt.caseBlk.p, bt.caseOf.p};
        e = BEll{N, m.nSlots, m.ellFace.p, m.ellNbr.p};
        ctl = Ctl{a.ctl.tolerance, a.ctl.relTol, a.ctl.minIter, a.ctl.maxIter};
        double *sd = bt.segD.p;
        int *si = bt.segI.p;
        double **dslots[] = {&S.nf, &S.init, &S.fin, &S.xbar, &S.A, &S.Aold, &S.alpha, &S.omega,
                             &S.r0r, &S.r0rOld, &S.beta, &S.last};
        for (int i = 0; i < 12; ++i) *dslots[i] = sd + (size_t)i * nSeg;
        int **islots[] = {&S.active, &S.iter, &S.sing, &S.repl, &S.rst, &S.conv};
        for (int i = 0; i < 6; ++i) *islots[i] = si + (size_t)i * nSeg;
        S.count = si + (size_t)6 * nSeg;
        // vectors: 9 x 6N of V, then the matrix copy and rD
        const size_t V6 = vstride(N);   // 6N rounded up: every vector 128-byte aligned
        const size_t bytes = sizeof(V) * (9 * V6 + 2 * (size_t)N + 2 * (size_t)F + (size_t)kSlots * N + 64);
        ctx->kws32.alloc((bytes + sizeof(float) - 1) / sizeof(float));
        vec = reinterpret_cast<V *>(ctx->kws32.p);
        d32 = vec + 9 * V6;
        rD = d32 + N;
        u32 = rD + N;
        l32 = u32 + F;
        aEll = l32 + F;   // kSlots x N: the persistent solvers' per-slot coefficients
        ctx->kws.alloc(48 * (size_t)N + 2 * (size_t)N + 64);
        rD64 = ctx->kws.p + 48 * (size_t)N;
        partial = bt.bPartial.p;
        res = bt.bRes.p;
    }
    static size_t vstride(int n) { return (6 * (size_t)n + 31) / 32 * 32; }
    V *v(int i) const { return vec + (size_t)i * vstride(N); }
    int gridSeg() const { return (nSeg + 255) / 256; }

    void fin(int nSlots, unsigned mask) {
        k_b_fin<<<bt.n, 192, 0, st>>>(nSlots, mask, t, partial, res);
        RT_CHECK_LAUNCH();
    }

    void prepare() {
        k_b_mat<V><<<nblocks(std::max(N, F)), RT_BLOCK, 0, st>>>(e, F, a.diag, a.upper, a.lower, d32, u32, l32);
        RT_CHECK_LAUNCH();
        const int pre = a.ctl.preconditioner;
        if ((pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU) && bt.sweep2d) {
            sweep2d_prepare(ctx, a.diag, a.upper, a.lower, sizeof(V) == 4);
        } else if (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU) {
            const DevMesh &m = ctx->mesh;
            for (int l = 0; l < m.nLevels; ++l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_b_rd_level<<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(e, l0, l1, m.levelCells.p, a.diag, a.upper,
                                                                     a.lower, rD64);
            }
            k_b_recip<V><<<nblocks(N), RT_BLOCK, 0, st>>>(N, rD64, rD, 0, a.diag);
            launch_count(ctx, m.nLevels + 1);
        } else if (pre == RT_PRECOND_DIAGONAL) {
            k_b_recip<V><<<nblocks(N), RT_BLOCK, 0, st>>>(N, rD64, rD, 1, a.diag);
            launch_count(ctx);
        }
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }

    void precondition(const V *r, V *w) {
        const int pre = a.ctl.preconditioner;
        if (pre == RT_PRECOND_NONE || pre == RT_PRECOND_DIAGONAL) {
            k_b_copy<V><<<nblocks(N), RT_BLOCK, 0, st>>>(N, vm, r, w, pre == RT_PRECOND_DIAGONAL ? rD : nullptr);
            launch_count(ctx);
        } else if (bt.sweep2d) {
            sweep2d_precondition(ctx, a.nc, vm, r, w);
        } else {
            const DevMesh &m = ctx->mesh;
            for (int l = 0; l < m.nLevels; ++l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_b_fwd_level<V><<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(e, l0, l1, m.levelCells.p, vm, rD, l32, r,
                                                                        w);
            }
            for (int l = m.nLevels - 1; l >= 0; --l) {
                int l0 = m.levelStartH[l], l1 = m.levelStartH[l + 1];
                k_b_bwd_level<V><<<nblocks(l1 - l0), RT_BLOCK, 0, st>>>(e, l0, l1, m.levelCells.p, vm, rD, u32, w);
            }
            launch_count(ctx, 2 * m.nLevels);
        }
        RT_CHECK_LAUNCH();
    }

    void amul(const V *x, V *y) {
        k_b_amul<V, V><<<nblocks(N), RT_BLOCK, 0, st>>>(e, vm, d32, u32, l32, x, y);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }
    void dot(const V *x, const V *y, const V *x2 = nullptr, const V *y2 = nullptr) {
        k_b_dot<V><<<bt.nBlk, RT_BLOCK, 0, st>>>(t, vm, S.active, x, y, x2, y2, partial);
        RT_CHECK_LAUNCH();
        fin(x2 ? 2 : 1, vm);
        launch_count(ctx, 2);
    }
    // residual replacement of the segments flagged in S.repl
    void replace(V *x, V *r) {
        k_b_fold<V><<<nblocks(N), RT_BLOCK, 0, st>>>(N, vm, bt.caseOf.p, S.repl, x, a.psi);
        k_b_true<V><<<bt.nBlk, RT_BLOCK, 0, st>>>(t, e, vm, S.repl, a.diag, a.upper, a.lower, a.source, a.psi, r,
                                                  partial);
        RT_CHECK_LAUNCH();
        fin(1, vm);
        launch_count(ctx, 3);
    }

    // x = 0, r = b - A psi, normFactor, initial residuals, active segments
    void prologue(V *r, V *x) {
        double *xs = res + 2 * (size_t)nSeg;   // after the two result slots
        k_b_sumx<<<bt.nBlk, RT_BLOCK, 0, st>>>(t, vm, a.psi, partial);
        RT_CHECK_LAUNCH();
        k_b_fin<<<bt.n, 192, 0, st>>>(1, vm, t, partial, xs);
        k_b_init_res<V><<<bt.nBlk, RT_BLOCK, 0, st>>>(t, e, vm, a.diag, a.upper, a.lower, a.source, a.psi, xs,
                                                      bt.cellStartD.p, r, x, partial);
        RT_CHECK_LAUNCH();
        fin(2, vm);
        k_b_start<<<1, 1024, 0, st>>>(bt.n, vm, ctl, S, res);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 5);
    }

    int poll() {
        RT_CUDA(cudaMemcpyAsync(bt.hostCount, S.count, sizeof(int), cudaMemcpyDeviceToHost, st));
        RT_CUDA(cudaStreamSynchronize(st));
        return *bt.hostCount;
    }

    void pcg_iteration(V *r, V *w, V *p, V *q, V *x) {
        precondition(r, w);
        if (mixed) dot(w, r, w, q);   // q = A p of the previous iteration (unused on the first)
        else dot(w, r);
        k_b_pcg_a<<<gridSeg(), 256, 0, st>>>(nSeg, S, res, mixed);
        k_b_pcg_p<V><<<nblocks(N), RT_BLOCK, 0, st>>>(N, vm, bt.caseOf.p, S, w, p);
        amul(p, q);
        dot(q, p);
        k_b_pcg_alpha<<<gridSeg(), 256, 0, st>>>(nSeg, S, res);
        k_b_pcg_update<V><<<bt.nBlk, RT_BLOCK, 0, st>>>(t, vm, S, p, q, x, r, partial);
        RT_CHECK_LAUNCH();
        fin(1, vm);
        k_b_iter_fin<<<gridSeg(), 256, 0, st>>>(nSeg, ctl, S, res, 0, mixed);
        RT_CHECK_LAUNCH();
        replace(x, r);
        k_b_after<<<1, 1024, 0, st>>>(bt.n, ctl, S, res);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 7);
    }

    void bicg_iteration(V *r, V *r0, V *p, V *y, V *Ay, V *s, V *z, V *tt, V *x) {
        dot(r0, r);
        k_b_bicg_r0r<<<gridSeg(), 256, 0, st>>>(nSeg, S, res);
        k_b_bicg_p<V><<<nblocks(N), RT_BLOCK, 0, st>>>(N, vm, bt.caseOf.p, S, r, Ay, p);
        precondition(p, y);
        amul(y, Ay);
        dot(r0, Ay);
        k_b_bicg_alpha<<<gridSeg(), 256, 0, st>>>(nSeg, S, res);
        k_b_bicg_s<V><<<bt.nBlk, RT_BLOCK, 0, st>>>(t, vm, S, r, Ay, s, partial);
        RT_CHECK_LAUNCH();
        fin(1, vm);
        k_b_bicg_half<<<gridSeg(), 256, 0, st>>>(nSeg, ctl, S, res, mixed);
        k_b_axpy_half<V><<<nblocks(N), RT_BLOCK, 0, st>>>(N, vm, bt.caseOf.p, S, y, x);
        RT_CHECK_LAUNCH();
        replace(x, r);
        k_b_half_after<<<gridSeg(), 256, 0, st>>>(nSeg, ctl, S, res, mixed);
        precondition(s, z);
        amul(z, tt);
        dot(tt, tt, tt, s);
        k_b_bicg_omega<<<gridSeg(), 256, 0, st>>>(nSeg, S, res);
        k_b_bicg_update<V><<<bt.nBlk, RT_BLOCK, 0, st>>>(t, vm, S, y, z, s, tt, x, r, partial);
        RT_CHECK_LAUNCH();
        fin(1, vm);
        k_b_iter_fin<<<gridSeg(), 256, 0, st>>>(nSeg, ctl, S, res, 1, mixed);
        RT_CHECK_LAUNCH();
        replace(x, r);
        k_b_after<<<1, 1024, 0, st>>>(bt.n, ctl, S, res);
        RT_CHECK_LAUNCH();
        launch_count(ctx, 12);
    }
};

// iterations between two polls of the active count
constexpr int kPoll = 4;

template <class V>
rt_status run_batch(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    BSolver<V> sv(ctx, a);
    const bool pcg = a.ctl.solver == RT_SOLVER_PCG;
    V *x = sv.v(8);
    V *r = sv.v(0);
    sv.prepare();
    sv.prologue(r, x);
    if (!pcg) RT_CUDA(cudaMemcpyAsync(sv.v(1), r, sizeof(V) * 6 * (size_t)sv.N, cudaMemcpyDeviceToDevice, sv.st));
    else RT_CUDA(cudaMemsetAsync(sv.v(3), 0, sizeof(V) * 6 * (size_t)sv.N, sv.st));   // q before the first A p
    int active = sv.poll();
    // one iteration as a CUDA graph, replayed kPoll times between polls
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto body = [&]() {
        if (pcg) sv.pcg_iteration(r, sv.v(1), sv.v(2), sv.v(3), x);
        else sv.bicg_iteration(r, sv.v(1), sv.v(2), sv.v(3), sv.v(4), sv.v(5), sv.v(6), sv.v(7), x);
    };
    int done = 0;
    const int cap = a.ctl.maxIter + 2;
    // the pressure solve of structured 2-D cases: one persistent CTA per case
    // runs every iteration of its case (RT_OPT_BATCH_PERSISTENT)
    const int pre = a.ctl.preconditioner;
    Batch &bt = ctx->mesh.batch;
    // one SM per case: worth it once the cases fill the GPU (a few large
    // cases iterate faster with their vector work spread over every SM)
    const bool persistent = ctx->batchPersistent == 2 || (ctx->batchPersistent == 1 && 2 * bt.n >= ctx->numSMs);
    if (active && pcg && persistent && bt.sweep2d && a.nc == 1 && bt.maxJB <= 8 && sv.e.nSlots <= kSlots &&
        (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU)) {
        Skew2D<V> g;
        if constexpr (sizeof(V) == 4) g = sweep2d_view32(ctx);
        else g = sweep2d_view64(ctx);
        {
            // the multigrid V-cycle for the FP32 form (RT_OPT_MIXED_PRECOND -2, DIC)
            BMg bmg{bt.mgDims.p, bt.mgNL.p, bt.mgOff.p, bt.mgCell.p, bt.mgCellOff.p, bt.sFaceLo.p, bt.mgPool.p,
                    (sizeof(V) == 4 && ctx->mixedJacobi == -2 && pre == RT_PRECOND_DIC && bt.mgPool.p) ? 1 : 0};
            ProfScope ps(ctx, "batch_pcg_persistent");
            const int shm = 8 * case_stage_bytes<V, 1, kCaseP<V>, kCaseNB>();
            RT_CUDA(cudaFuncSetAttribute(k_b_pcg_case<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, shm));
            k_b_pcg_case<V><<<bt.n, kCaseThreads, shm, sv.st>>>(sv.t, sv.e, g, sv.S, sv.ctl, sv.mixed, sv.d32, sv.u32,
                                                              sv.l32, a.diag, a.upper, a.lower, a.source, a.psi, r,
                                                              sv.v(1), sv.v(2), sv.v(3), x, bt.caseOrder.p,
                                                              sv.aEll, bmg, bt.sErr.p, 1ll << 22, cap);
            RT_CHECK_LAUNCH();
        }
        launch_count(ctx);
        bt.sPending = true;
        active = 0;
    }
    // the momentum solve of the same cases (up to three components)
    if (active && !pcg && persistent && bt.sweep2d && a.nc <= 3 && (sv.vm & ~7u) == 0 &&
        bt.maxJB <= 8 && sv.e.nSlots <= kSlots && (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU)) {
        Skew2D<V> g;
        if constexpr (sizeof(V) == 4) g = sweep2d_view32(ctx);
        else g = sweep2d_view64(ctx);
        {
            // the multigrid V-cycle for the FP32 form (RT_OPT_MIXED_PRECOND_U -2, DILU)
            BMg bmg{bt.mgDims.p, bt.mgNL.p, bt.mgOff.p, bt.mgCell.p, bt.mgCellOff.p, bt.sFaceLo.p, bt.mgPool.p,
                    (sizeof(V) == 4 && ctx->mixedPrecondU == -2 && pre == RT_PRECOND_DILU && bt.mgPool.p) ? 1 : 0};
            ProfScope ps(ctx, "batch_bicgstab_persistent");
            const int shm = 16 * case_stage_bytes<V, 1, kBicgP<V>, kBicgNB<V>>();
            RT_CUDA(cudaFuncSetAttribute(k_b_bicg_case<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, shm));
            k_b_bicg_case<V><<<bt.n, kCaseThreads, shm, sv.st>>>(
                sv.t, sv.e, g, sv.S, sv.ctl, sv.vm, sv.mixed, sv.d32, sv.u32, sv.l32, a.diag, a.upper, a.lower,
                a.source, a.psi, r, sv.v(1), sv.v(2), sv.v(3), sv.v(4), sv.v(5), sv.v(6), sv.v(7), x,
                bt.caseOrder.p, sv.aEll, bmg, bt.sErr.p, 1ll << 22, cap);
            RT_CHECK_LAUNCH();
        }
        launch_count(ctx);
        bt.sPending = true;
        active = 0;
    }
    if (active) {
        body();   // first iteration eagerly (sets kernel attributes outside any capture)
        ++done;
        active = sv.poll();
    }
    if (active) {
        RT_CUDA(cudaStreamBeginCapture(sv.st, cudaStreamCaptureModeThreadLocal));
        try {
            body();
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(sv.st, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        RT_CUDA(cudaStreamEndCapture(sv.st, &graph));
        RT_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    }
    size_t nodes = 0;
    if (graph) RT_CUDA(cudaGraphGetNodes(graph, nullptr, &nodes));
    while (active && done < cap) {
        for (int i = 0; i < kPoll && done < cap; ++i, ++done) {
            RT_CUDA(cudaGraphLaunch(exec, sv.st));
            ctx->kernelLaunches += (long long)nodes;
        }
        active = sv.poll();
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    // what is left in x (segments stopped as singular) goes to psi
    k_b_fold<V><<<nblocks(sv.N), RT_BLOCK, 0, sv.st>>>(sv.N, sv.vm, ctx->mesh.batch.caseOf.p, nullptr, x, a.psi);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    // records of every segment
    const int nSeg = sv.nSeg;
    bt.hostSegD.resize((size_t)12 * nSeg);
    bt.hostSegI.resize((size_t)6 * nSeg + 8);
    RT_CUDA(cudaMemcpyAsync(bt.hostSegD.data(), bt.segD.p, sizeof(double) * 12 * nSeg, cudaMemcpyDeviceToHost,
                            sv.st));
    RT_CUDA(cudaMemcpyAsync(bt.hostSegI.data(), bt.segI.p, sizeof(int) * (6 * nSeg + 8), cudaMemcpyDeviceToHost,
                            sv.st));
    RT_CUDA(cudaStreamSynchronize(sv.st));
    const double *init = bt.hostSegD.data() + (size_t)1 * nSeg, *fin = bt.hostSegD.data() + (size_t)2 * nSeg;
    const int *iter = bt.hostSegI.data() + (size_t)1 * nSeg, *sing = bt.hostSegI.data() + (size_t)2 * nSeg,
              *conv = bt.hostSegI.data() + (size_t)5 * nSeg;
    if ((int)ctx->batchPerf.size() != bt.n) ctx->batchPerf.assign(bt.n, rt_step_perf{});
    for (int k = 0; k < a.nc; ++k) {
        rt_solver_perf agg{};
        agg.converged = 1;
        if (!((a.validMask >> k) & 1u)) {
            agg.nIterations = -1;
            perf[k] = agg;
            continue;
        }
        for (int cb = 0; cb < bt.n; ++cb) {
            const int sg = cb * 8 + k;
            rt_solver_perf p{};
            p.initialResidual = init[sg];
            p.finalResidual = fin[sg];
            p.nIterations = iter[sg];
            p.singular = sing[sg];
            p.converged = (conv[sg] == 1) ? 1 : 0;
            agg.initialResidual = std::max(agg.initialResidual, p.initialResidual);
            agg.finalResidual = std::max(agg.finalResidual, p.finalResidual);
            agg.nIterations = std::max(agg.nIterations, p.nIterations);
            agg.singular |= p.singular;
            agg.converged &= p.converged;
            rt_step_perf &sp = ctx->batchPerf[cb];
            if (a.stage == 0 && k < 3) sp.U[k] = p;
            else if (a.stage == 1 && k == 0) sp.p = p;
            else if (a.stage == 2) sp.theta[k] = p;
        }
        perf[k] = agg;
    }
    if (a.stage == 2)
        for (int cb = 0; cb < bt.n; ++cb)
            for (int k = 0; k < 6; ++k)
                if (!((a.validMask >> k) & 1u)) ctx->batchPerf[cb].theta[k] = rt_solver_perf{0, 0, -1, 1, 0, 0};
    if (a.stage == 0)
        for (int cb = 0; cb < bt.n; ++cb)
            for (int k = 0; k < 3; ++k)
                if (!((a.validMask >> k) & 1u)) ctx->batchPerf[cb].U[k] = rt_solver_perf{0, 0, -1, 1, 0, 0};
    return sweep2d_check(ctx);
}

}  // namespace

rt_status batch_solve(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf) {
    ProfScope ps(ctx, a.stage == 1 ? "batch_solve_p" : a.stage == 0 ? "batch_solve_U" : "batch_solve_theta");
    if (a.precision == RT_PREC_MIXED && (ctx->mixedParts & 1)) {
        SolveArgs t = a;
        t.ctl.tolerance *= ctx->mixedTighten;
        t.ctl.relTol *= ctx->mixedTighten;
        return run_batch<float>(ctx, t, perf);
    }
    return run_batch<double>(ctx, a, perf);
}

}  // namespace rt
