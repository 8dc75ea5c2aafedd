// sweep2d_cta.cuh — the per-case DIC/DILU sweep of the batched 2-D cases, as
// a device function of the CTA that owns the case (used by the sweep kernels
// of sweep2d.cu and by the persistent per-case Krylov kernel of
// krylov_batch.cu).  See sweep2d.cu for the method.
#pragma once

#include "batch.h"
#include "real_ops.cuh"

namespace rt {

namespace s2d {

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

}  // namespace s2d

// the coefficients and inputs of one chunk of P steps of a lane
template <class Real, int NC, int P>
struct S2Chunk {
    Real c0[P], cy[P], cx[P];
    Real rk[P][NC];
    int cell[P];
};

// loads of the chunk starting at step t0 (independent of the recurrence):
// coefficients and cell numbers through the read-only path, the sweep input
// (written earlier in the same kernel by the persistent solver) plainly
template <class Real, int MODE, int NC, int P>
__device__ __forceinline__ void s2_load(const Skew2D<Real> &g, long long e0, long long st, int t0,
                                        S2Chunk<Real, NC, P> &k) {
#pragma unroll
    for (int s = 0; s < P; ++s) {
        const long long e = e0 + (long long)(t0 + s) * st;
        if (MODE == 2) {
            k.c0[s] = __ldg(g.D + e); k.cy[s] = __ldg(g.Py + e); k.cx[s] = __ldg(g.Px + e);
        } else {
            k.c0[s] = (MODE == 0) ? __ldg(g.rDinv + e) : Real(0);
            k.cy[s] = __ldg(((MODE == 0) ? g.Ay : g.By) + e);
            k.cx[s] = __ldg(((MODE == 0) ? g.Ax : g.Bx) + e);
#pragma unroll
            for (int q = 0; q < NC; ++q) k.rk[s][q] = ((MODE == 0) ? g.rS : g.wS)[(long long)q * g.nSkew + e];
        }
        k.cell[s] = (MODE == 1) ? __ldg(g.cellOf + e) : 0;
    }
}

// One case's sweep by the CTA that owns it (case cb; warps wbase .. wbase +
// nJB - 1 take the j-blocks, the others do nothing).  MODE 0: forward application (rS -> wS), 1: backward
// application (wS -> w), 2: rD recurrence (D, Py, Px -> rDraw).  ringJ: the
// j-block ring in shared memory ([maxJB][kRJ][NC]), sProg: 32 progress
// counters, zero on entry (the caller clears them and synchronises).  The
// loads of chunk k + 1 are issued before the waits and the recurrence of
// chunk k, so their latency hides behind the dependent chain (PF; without
// it, for launches of up to 1024 threads, each chunk loads just before use).
template <class Real, int MODE, int NC, int P, bool PF = true>
__device__ void sweep2d_cta(const Skew2D<Real> &g, int cb, unsigned mask, Real *__restrict__ w, int N, int *err,
                            long long maxSpin, Real *ringJ, int *sProg, int wbase = 0) {
    const int lane = threadIdx.x & 31, jo = (int)(threadIdx.x >> 5) - wbase;
    const int nJB = g.JB[cb], T = g.T[cb];
    const long long off = g.off[cb];
    if (jo < 0 || jo >= nJB) return;
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
    S2Chunk<Real, NC, P> cur, nxt;
    if (PF) s2_load<Real, MODE, NC, P>(g, e0, st, 0, cur);
    for (int t0 = 0; t0 < T; t0 += P) {
        const int te = t0 + P;   // T is a multiple of P
        if (PF && te < T) s2_load<Real, MODE, NC, P>(g, e0, st, te, nxt);
        // the consumer has read the ring slots this chunk overwrites
        if (consJ >= 0 && seenCJ < te - s2d::kRJ - 31) {
            int v = 0;
            if (lane == 0) v = s2d::spin_cta(sProg + consJ, te - s2d::kRJ - 31, err, maxSpin);
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) break;
            seenCJ = v;
        }
        // the j-block below has produced row 32 jb - 1 through step te + 31
        if (depJ >= 0 && seenJ < min(T, te + 31)) {
            int v = 0;
            if (lane == 0) v = s2d::spin_cta(sProg + depJ, min(T, te + 31), err, maxSpin);
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) break;
            seenJ = v;
        }
        __syncwarp();
        if (!PF) s2_load<Real, MODE, NC, P>(g, e0, st, t0, cur);
        Real out[P][NC];
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int t = t0 + s;
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const Real yup = __shfl_up_sync(0xffffffffu, yprev[q], 1);
                const Real yj = (lane > 0) ? yup
                                           : ((depJ >= 0 && t + 31 < T) ? ringJ[((size_t)depJ * s2d::kRJ + ((t + 31) & (s2d::kRJ - 1))) * NC + q]
                                                                         : zk);
                Real v;
                if (MODE == 2) {
                    v = r_sub(cur.c0[s], r_div(cur.cy[s], yj));
                    v = r_sub(v, r_div(cur.cx[s], yprev[q]));
                } else {
                    const Real pre = (MODE == 0) ? r_mul(cur.c0[s], cur.rk[s][q]) : cur.rk[s][q];
                    if (sizeof(Real) == 4) {   // FP32: the i term first (as the 3-D sweeps)
                        v = r_fma(-cur.cx[s], yprev[q], pre);
                        v = r_fma(-cur.cy[s], yj, v);
                    } else {
                        v = r_fma(-cur.cy[s], yj, pre);
                        v = r_fma(-cur.cx[s], yprev[q], v);
                    }
                }
                if (consJ >= 0 && lane == 31) ringJ[((size_t)jo * s2d::kRJ + (t & (s2d::kRJ - 1))) * NC + q] = v;
                out[s][q] = v;
                yprev[q] = v;
            }
        }
        __syncwarp();
        if (lane == 0 && (consJ >= 0 || depJ >= 0)) s2d::st_release_cta(sProg + jo, te);
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
                    else if (cur.cell[s] >= 0) w[(long long)q * N + cur.cell[s]] = out[s][q];
                }
            }
        }
        if (PF) cur = nxt;
    }
    // a warp that gave up releases everything it owes
    if (*(volatile int *)err && lane == 0) s2d::st_release_cta(sProg + jo, T);
}

}  // namespace rt
