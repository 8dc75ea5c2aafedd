// sweep2d_cta.cuh — the per-case DIC/DILU sweep of the batched 2-D cases, as
// a device function of the CTA that owns the case (used by the sweep kernels
// of sweep2d.cu and by the persistent per-case Krylov kernel of
// krylov_batch.cu).  See sweep2d.cu for the method.
#pragma once

#include "batch.h"
#include "real_ops.cuh"

namespace rt {

namespace s2d {

constexpr int kRJ = 128;   // j-block ring depth (power of two); the consumer lags 32 + P steps
typedef unsigned long long u64;

// words per value in the j-block ring: a value travels with its step as a
// tag in 64-bit words (payload in the low half, tag = step + 1 in the high
// half; an FP64 value as two words, its high and low halves, each tagged),
// written and read with single-copy-atomic 64-bit accesses, so the consumer
// waits on the data itself and no fence sits on the dependency chain
template <class Real> struct W;
template <> struct W<float> { static constexpr int n = 1; };
template <> struct W<double> { static constexpr int n = 2; };

__device__ __forceinline__ void put(u64 *w, float v, unsigned tag) {
    *(volatile u64 *)w = ((u64)tag << 32) | __float_as_uint(v);
}
__device__ __forceinline__ void put(u64 *w, double v, unsigned tag) {
    volatile u64 *p = w;
    p[0] = ((u64)tag << 32) | (unsigned)__double2hiint(v);
    p[1] = ((u64)tag << 32) | (unsigned)__double2loint(v);
}
__device__ __forceinline__ bool take(const u64 *w, unsigned tag, float &v) {
    const u64 a = *(const volatile u64 *)w;
    v = __uint_as_float((unsigned)a);
    return (unsigned)(a >> 32) == tag;
}
__device__ __forceinline__ bool take(const u64 *w, unsigned tag, double &v) {
    const volatile u64 *p = w;
    const u64 a = p[0], b = p[1];
    v = __hiloint2double((int)(unsigned)a, (int)(unsigned)b);
    return ((unsigned)(a >> 32) == tag) & ((unsigned)(b >> 32) == tag);
}

// lane 0 of a warp waits until the consumer's progress counter *c >= need
// (bounded); -1 after a timeout.  The counter only bounds how far a producer
// runs ahead (a slot is rewritten after its consumer has used the value), so
// plain volatile accesses serve.
__device__ __forceinline__ int spin_cta(const int *c, int need, int *err, long long maxSpin) {
    long long spins = 0;
    int v = *(const volatile int *)c;
    while (v < need) {
        if ((++spins & 255) == 0 && (spins > maxSpin || *(volatile int *)err)) {
            atomicExch(err, 1);
            return -1;
        }
        v = *(const volatile int *)c;
    }
    return v;
}

// asynchronous 16-byte copies global -> shared (L2 only: the sources may have
// been written earlier in the same kernel by other threads of the CTA)
__device__ __forceinline__ void cp16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// the arrays of a staged chunk: MODE 0 rDinv, Ay, Ax, rS (NC); MODE 1 By,
// Bx, wS (NC) and the cells; MODE 2 D, Py, Px
template <int MODE, int NC> struct StageArrays { static constexpr int n = (MODE == 2) ? 3 : (MODE == 0 ? 3 : 2) + NC; };

// bytes of one warp's NB staging buffers
template <class Real, int MODE, int NC, int P, int NB>
__host__ __device__ constexpr int stage_bytes() {
    return NB * P * 32 * (StageArrays<MODE, NC>::n * (int)sizeof(Real) + (MODE == 1 ? 4 : 0));
}

// clears the rings and counters of a sweep (all threads of the CTA, before
// the barrier that precedes the sweep): the tags of a sweep start from 1
template <class Real, int NC, int RJ = kRJ>
__device__ __forceinline__ void reset(u64 *ring, int nJB, int *sProg) {
    const int n = nJB * RJ * NC * W<Real>::n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) ring[i] = 0ull;
    if (threadIdx.x < 32) sProg[threadIdx.x] = 0;
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
// nJB - 1 take the j-blocks, the others do nothing).  MODE 0: forward
// application (rS -> wS), 1: backward application (wS -> w), 2: rD recurrence
// (D, Py, Px -> rDraw).  ringJ: the j-block ring in shared memory
// ([nJB][RJ][NC][W] tagged words), sProg: the consumers' progress counters;
// both cleared by s2d::reset before the sweep.  At the start of a chunk of P
// steps lanes 0 .. P-1 fetch the P words lane 0 will need from the j-block
// below (steps t0 + 31 .. t0 + P + 30) and the warp waits until every tag
// matches; lane 31 writes its value of every step into the warp's own ring.
// The loads of chunk k + 1 are issued before the waits and the recurrence of
// chunk k, so their latency hides behind the dependent chain (PF; without
// it, for launches of up to 1024 threads, each chunk loads just before use).
//
// NB > 0: the chunks are staged instead into shared memory with cp.async,
// NB - 1 chunks ahead (stage: the CTA's staging area, stage_bytes() per warp
// of the sweep), and each chunk's values are read from there.
template <class Real, int MODE, int NC, int P, bool PF = true, int RJ = s2d::kRJ, int NB = 0>
__device__ void sweep2d_cta(const Skew2D<Real> &g, int cb, unsigned mask, Real *__restrict__ w, int N, int *err,
                            long long maxSpin, s2d::u64 *ringJ, int *sProg, int wbase = 0,
                            unsigned char *stage = nullptr) {
    constexpr int WN = s2d::W<Real>::n;
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
    s2d::u64 *myRing = ringJ + (size_t)jo * RJ * NC * WN;
    const s2d::u64 *depRing = ringJ + (size_t)(depJ >= 0 ? depJ : 0) * RJ * NC * WN;
    Real yprev[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) yprev[q] = zk;
    int seenCJ = 0;
    bool failed = false;
    S2Chunk<Real, NC, P> cur, nxt;
    // ---- staging (NB > 0): chunk c of this warp, array a, into buffer c % NB
    constexpr int NA = s2d::StageArrays<MODE, NC>::n;
    constexpr int CH = P * 32;                                  // entries of one array in one chunk
    constexpr int BUF = s2d::stage_bytes<Real, MODE, NC, P, NB>() / (NB > 0 ? NB : 1);
    unsigned char *myStage = stage + (size_t)jo * (NB > 0 ? NB : 1) * BUF;
    auto stage_chunk = [&](int c) {
        const int tc = c * P;
        const long long base = (MODE == 1) ? off + ((long long)jb * T + (T - tc - P)) * 32
                                           : off + ((long long)jb * T + tc) * 32;
        unsigned char *buf = myStage + (size_t)(c % NB) * BUF;
        constexpr int PIECES = CH * (int)sizeof(Real) / 16;
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            const Real *src;
            if (MODE == 2) src = a == 0 ? g.D : a == 1 ? g.Py : g.Px;
            else if (MODE == 0) src = a == 0 ? g.rDinv : a == 1 ? g.Ay : a == 2 ? g.Ax : g.rS + (long long)(a - 3) * g.nSkew;
            else src = a == 0 ? g.By : a == 1 ? g.Bx : g.wS + (long long)(a - 2) * g.nSkew;
            for (int i = lane; i < PIECES; i += 32)
                s2d::cp16(buf + (size_t)a * CH * sizeof(Real) + (size_t)i * 16, src + base + (long long)i * (16 / sizeof(Real)));
        }
        if (MODE == 1)
            for (int i = lane; i < CH * 4 / 16; i += 32)
                s2d::cp16(buf + (size_t)NA * CH * sizeof(Real) + (size_t)i * 16, g.cellOf + base + (long long)i * 4);
    };
    auto read_chunk = [&](int c) {
        const unsigned char *buf = myStage + (size_t)(c % NB) * BUF;
        const Real *arr = reinterpret_cast<const Real *>(buf);
        const int *cel = reinterpret_cast<const int *>(buf + (size_t)NA * CH * sizeof(Real));
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int i = (MODE == 1) ? (P - 1 - s) * 32 + (31 - lane) : s * 32 + lane;
            if (MODE == 2) {
                cur.c0[s] = arr[i]; cur.cy[s] = arr[CH + i]; cur.cx[s] = arr[2 * CH + i];
            } else if (MODE == 0) {
                cur.c0[s] = arr[i]; cur.cy[s] = arr[CH + i]; cur.cx[s] = arr[2 * CH + i];
#pragma unroll
                for (int q = 0; q < NC; ++q) cur.rk[s][q] = arr[(3 + q) * CH + i];
            } else {
                cur.c0[s] = Real(0); cur.cy[s] = arr[i]; cur.cx[s] = arr[CH + i];
#pragma unroll
                for (int q = 0; q < NC; ++q) cur.rk[s][q] = arr[(2 + q) * CH + i];
                cur.cell[s] = cel[i];
            }
        }
    };
    const int nChunks = T / P;
    if (NB > 0) {
        for (int c = 0; c < NB - 1; ++c) {
            if (c < nChunks) stage_chunk(c);
            s2d::cp_commit();
        }
    } else if (PF) {
        s2_load<Real, MODE, NC, P>(g, e0, st, 0, cur);
    }
    for (int t0 = 0; t0 < T; t0 += P) {
        const int te = t0 + P;   // T is a multiple of P
        if (NB > 0) {
            const int c = t0 / P;
            if (c + NB - 1 < nChunks) stage_chunk(c + NB - 1);
            s2d::cp_commit();
            s2d::cp_wait<NB - 1>();
            __syncwarp();
            read_chunk(c);
            __syncwarp();   // buffer c % NB is free for chunk c + NB
        } else if (PF && te < T) {
            s2_load<Real, MODE, NC, P>(g, e0, st, te, nxt);
        }
        // the consumer has used the ring slots this chunk overwrites
        if (consJ >= 0 && seenCJ < te - RJ - 31) {
            int v = 0;
            if (lane == 0) v = s2d::spin_cta(sProg + consJ, te - RJ - 31, err, maxSpin);
            v = __shfl_sync(0xffffffffu, v, 0);
            if (v < 0) { failed = true; break; }
            seenCJ = v;
        }
        // the words of the j-block below for this chunk's steps (lane s holds step t0 + s + 31)
        Real jv[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) jv[q] = zk;
        if (depJ >= 0) {
            const int tw = t0 + lane + 31;
            const bool need = lane < P && tw < T;
            const s2d::u64 *slot = depRing + (size_t)(tw & (RJ - 1)) * NC * WN;
            long long spins = 0;
            for (;;) {
                bool ok = true;
                if (need) {
#pragma unroll
                    for (int q = 0; q < NC; ++q) ok &= s2d::take(slot + q * WN, (unsigned)(tw + 1), jv[q]);
                }
                if (__all_sync(0xffffffffu, ok)) break;
                const bool quit = (++spins > maxSpin) || *(volatile int *)err;
                if (__any_sync(0xffffffffu, quit)) {
                    if (lane == 0) atomicExch(err, 1);
                    failed = true;
                    break;
                }
            }
            if (failed) break;
        }
        if (NB == 0 && !PF) s2_load<Real, MODE, NC, P>(g, e0, st, t0, cur);
        Real out[P][NC];
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int t = t0 + s;
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const Real fromBelow = __shfl_sync(0xffffffffu, jv[q], s);
                const Real yup = __shfl_up_sync(0xffffffffu, yprev[q], 1);
                const Real yj = (lane > 0) ? yup : ((depJ >= 0 && t + 31 < T) ? fromBelow : zk);
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
                if (consJ >= 0 && lane == 31) s2d::put(myRing + ((size_t)(t & (RJ - 1)) * NC + q) * WN, v,
                                                       (unsigned)(t + 1));
                out[s][q] = v;
                yprev[q] = v;
            }
        }
        // this warp has used the words of the block below through step te + 30
        if (lane == 0 && depJ >= 0) *(volatile int *)(sProg + jo) = te;
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
        if (NB == 0 && PF) cur = nxt;
    }
    if (NB > 0) s2d::cp_wait<0>();   // no copy into the staging area outlives the sweep
    // a warp that gave up releases its producer
    if (failed && lane == 0) *(volatile int *)(sProg + jo) = T + RJ + 64;
}

}  // namespace rt
