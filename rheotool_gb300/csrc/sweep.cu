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
#include <cooperative_groups.h>
#include <cuda/atomic>

#include "rt_internal.h"
#include "sweep.h"

namespace rt {

namespace cg = cooperative_groups;

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

__device__ __forceinline__ int ld_acquire_cluster(const int *p) {
    int v;
    asm volatile("ld.acquire.cluster.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cluster(int *p, int v) {
    asm volatile("st.release.cluster.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void fence_cluster() { asm volatile("fence.acq_rel.cluster;" ::: "memory"); }

// bounded spin of lane 0 on a counter of this CTA's shared memory that other
// CTAs of the cluster (or warps of this CTA) advance; -1 after a timeout
__device__ __forceinline__ int spin_cluster(const int *c, int need, int *sync, long long maxSpin) {
    long long spins = 0;
    int v = ld_acquire_cluster(c);
    while (v < need) {
        if ((++spins & 255) == 0 && (spins > maxSpin || load_acquire(sync + SYNC_ERROR))) {
            atomicExch(sync + SYNC_ERROR, 1);
            return -1;
        }
        v = ld_acquire_cluster(c);
    }
    return v;
}

// Ring depths (steps) of the hand-offs for chunk size P.
template <int P> struct Ring {
    static constexpr int R = (P >= 8) ? 2 * P : (P >= 4) ? 4 * P : 4;   // plane ring, at least two chunks
    static constexpr int RJ = (P >= 8) ? 128 : 64;    // j-block ring (power of two): the consumer lags ~32 + P steps
};

// Per-warp staging of a chunk's coefficients (cp.async, two buffers): NA
// double arrays of P steps x 32 lanes, plus the cells of the backward sweep.
template <int MODE, int NC> struct Stage { static constexpr int NA = 4 + NC; };

constexpr size_t kMaxSmem = 227 * 1024;   // dynamic shared memory per CTA on sm_100-class parts

template <int MODE, int NC, int P>
size_t sweep_smem_bytes(int nJB) {
    const size_t rings = (size_t)nJB * (Ring<P>::R * 32 * NC + Ring<P>::RJ * NC) * sizeof(double);
    const size_t stage = (size_t)nJB * 3 * P * 32 * (Stage<MODE, NC>::NA * sizeof(double) + sizeof(int));
    return rings + stage;
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// MODE 0: forward application, 1: backward application, 2: rD recurrence.
//
// One CTA owns one plane (all its j-blocks, warp = j-block); a thread-block
// cluster owns CS consecutive planes in processing order, CTA rank r holding
// the r-th.  The plane-to-plane values move through distributed shared
// memory: the producer CTA stores each step's 32 lanes straight into the
// consumer CTA's ring and advances the consumer's counter with a
// cluster-scope release; the consumer reports its own progress back into the
// producer's memory, which bounds how far the producer may run ahead (so a
// ring slot is never overwritten before it is read, and the two waits can
// never close a cycle).  The j-block hand-off stays inside the CTA (lane 31 of
// the block below, through a shared ring).  The first plane of a cluster reads
// the previous cluster's last plane from the global skewed array wS behind a
// global release/acquire counter.  Clusters take plane groups in dependency
// order from an atomic counter; all CTAs of a cluster are co-scheduled, and
// none leaves before the final cluster barrier, so no CTA ever accesses the
// shared memory of a CTA that has exited.
//
// Latency: a chunk's coefficients are staged into shared memory with cp.async
// one chunk ahead, and a chunk's global stores are issued one chunk late, so
// the releases never wait for stores in flight.  The remaining per-step cost
// is the dependent FP64 chain (one multiply and three fused multiply-adds on
// a pipe that retires about two FP64 lanes per cycle per SM).
// Invalid entries (outside the mesh, padding) have zero coefficients and zero
// right-hand sides, so every lane runs the same branch-free recurrence.
template <int MODE, int NC, int P>
__global__ void __launch_bounds__(512) k_systolic(SkewView g, unsigned mask, double *__restrict__ w, int N,
                                                  int *sync, long long maxSpin) {
    constexpr int R = Ring<P>::R, RJ = Ring<P>::RJ, NA = Stage<MODE, NC>::NA;
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks(), r = (int)cluster.block_rank();
    extern __shared__ double smem[];
    __shared__ int s_grp;
    __shared__ int kIn[16], kBack[16], sProg[16];
    const int lane = threadIdx.x & 31, jo = threadIdx.x >> 5;
    const int nJB = g.nJB;
    double *ringK = smem;                                   // [nJB][R][32][NC], filled by the k-producer
    double *ringJ = ringK + (size_t)nJB * R * 32 * NC;      // [nJB][RJ][NC]
    double *stage = ringJ + (size_t)nJB * RJ * NC;          // [nJB][3][P][NA][32]
    int *cstage = (int *)(stage + (size_t)nJB * 3 * P * NA * 32);   // [nJB][3][P][32]
    double *myStage = stage + (size_t)jo * 3 * P * NA * 32;
    int *myCStage = cstage + (size_t)jo * 3 * P * 32;
    if (threadIdx.x < 16) { kIn[threadIdx.x] = 0; kBack[threadIdx.x] = 0; sProg[threadIdx.x] = 0; }
    if (r == 0 && threadIdx.x == 0) s_grp = atomicAdd(sync + SYNC_WORK, 1);
    cluster.sync();
    const int grp = *cluster.map_shared_rank(&s_grp, 0);
    const int nGroups = (g.nz + CS - 1) / CS;
    const int T = g.T;
    int *gprog = sync + SYNC_PROGRESS;
    const int gi = (MODE == 1) ? nGroups - 1 - grp : grp;
    const int k = (MODE == 1) ? gi * CS + (CS - 1 - r) : gi * CS + r;
    const bool exists = grp < nGroups && k >= 0 && k < g.nz;
    if (exists) {
        const int jb = (MODE == 1) ? nJB - 1 - jo : jo;
        const int blk = k * nJB + jb;
        const long long BS = (long long)T * 32;
        const long long KS = (long long)nJB * BS;
        const bool hasK = (MODE == 1) ? (k + 1 < g.nz) : (k > 0);
        const bool kLocalProd = hasK && r > 0;
        const int kGlob = (hasK && r == 0) ? ((MODE == 1) ? k + 1 : k - 1) * nJB + jb : -1;
        const bool consExists = (MODE == 1) ? (k - 1 >= 0) : (k + 1 < g.nz);
        const bool kLocalCons = consExists && r + 1 < CS;
        const bool crossProducer = consExists && r == CS - 1;
        const int depJ = (jo > 0) ? jo - 1 : -1;
        const int consJ = (jo + 1 < nJB) ? jo + 1 : -1;
        double *consRing = kLocalCons ? cluster.map_shared_rank(ringK, r + 1) : nullptr;
        int *consKin = kLocalCons ? cluster.map_shared_rank(kIn, r + 1) : nullptr;
        int *prodBack = kLocalProd ? cluster.map_shared_rank(kBack, r - 1) : nullptr;
        // entry of step t: e0 + t * st
        const long long e0 = (MODE == 1) ? (long long)blk * BS + (long long)(T - 1) * 32 + (31 - lane)
                                         : (long long)blk * BS + lane;
        const long long st = (MODE == 1) ? -32 : 32;
        // stage the coefficients of the chunk starting at step c0 into buffer b
        auto stage_chunk = [&](int tc, int b) {
#pragma unroll
            for (int s = 0; s < P; ++s) {
                const long long e = e0 + (tc + s) * st;
                double *d = myStage + ((size_t)(b * P + s) * NA) * 32 + lane;
                if (MODE == 2) {
                    cp_async8(d + 0 * 32, g.D + e); cp_async8(d + 1 * 32, g.Pz + e);
                    cp_async8(d + 2 * 32, g.Py + e); cp_async8(d + 3 * 32, g.Px + e);
                } else {
                    cp_async8(d + 0 * 32, (MODE == 0 ? g.Az : g.Bz) + e);
                    cp_async8(d + 1 * 32, (MODE == 0 ? g.Ay : g.By) + e);
                    cp_async8(d + 2 * 32, (MODE == 0 ? g.Ax : g.Bx) + e);
                    if (MODE == 0) cp_async8(d + 3 * 32, g.rDinv + e);
#pragma unroll
                    for (int q = 0; q < NC; ++q)
                        cp_async8(d + (4 + q) * 32, (MODE == 0 ? g.rS : g.wS) + (long long)q * g.nSkew + e);
                    if (MODE == 1) cp_async4(myCStage + (b * P + s) * 32 + lane, g.cellOf + e);
                }
            }
        };
        int seenK = 0, seenJ = 0, seenCK = 0, seenCJ = 0, fail = 0;
        double yprev[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) yprev[q] = (MODE == 2) ? 1.0 : 0.0;
        double prevOut[P][NC];
        int prevCell[P];
        int prevT0 = -1;
        // three staging buffers: chunk c is staged two chunks ahead, right
        // after the release of chunk c - 2, so no release waits for it
        stage_chunk(0, 0);
        cp_async_commit();
        if (P < T) stage_chunk(P, 1);
        cp_async_commit();

        for (int t0 = 0; t0 < T; t0 += P) {
            const int te = t0 + P;   // T is a multiple of P
            const int buf = (t0 / P) % 3;
            cp_async_wait<1>();      // this chunk's group is complete
            // ---- back-pressure: consumers have read what this chunk overwrites
            if (kLocalCons && seenCK < te - R) {
                int v = 0;
                if (lane == 0) v = spin_cluster(kBack + jo, te - R, sync, maxSpin);
                v = __shfl_sync(0xffffffffu, v, 0);
                if (v < 0) { fail = 1; break; }
                seenCK = v;
            }
            if (consJ >= 0 && seenCJ < te - RJ - 31) {
                int v = 0;
                if (lane == 0) v = spin_cluster(sProg + consJ, te - RJ - 31, sync, maxSpin);
                v = __shfl_sync(0xffffffffu, v, 0);
                if (v < 0) { fail = 1; break; }
                seenCJ = v;
            }
            // ---- dependencies: previous plane through te, j-block below through te + 31
            if (hasK && seenK < te) {
                int v = 0;
                if (lane == 0)
                    v = kLocalProd ? spin_cluster(kIn + jo, te, sync, maxSpin)
                                   : spin_global(gprog + kGlob, te, sync, maxSpin >> 6);
                v = __shfl_sync(0xffffffffu, v, 0);
                if (v < 0) { fail = 1; break; }
                seenK = v;
            }
            if (depJ >= 0 && seenJ < min(T, te + 31)) {
                int v = 0;
                if (lane == 0) v = spin_cluster(sProg + depJ, min(T, te + 31), sync, maxSpin);
                v = __shfl_sync(0xffffffffu, v, 0);
                if (v < 0) { fail = 1; break; }
                seenJ = v;
            }
            // (lane 0's acquire loads + the warp-wide shuffle order the ring
            // reads below after the producers' releases)
            // ---- the recurrence (order of operations of the sequential sweep)
            double out[P][NC];
            int cell[P];
            // the terms of a step that do not depend on the previous step (the
            // right-hand side and the k neighbour) are formed for the whole
            // chunk first, so only the j and i terms stay on the dependent chain
            double pre[P][NC], wjv[P][NC], cy[P], cx[P];
#pragma unroll
            for (int s = 0; s < P; ++s) {
                const int t = t0 + s;
                const double *d = myStage + ((size_t)(buf * P + s) * NA) * 32 + lane;
                // staged arrays: MODE 2: D, Pz, Py, Px; MODE 0/1: z, y, x
                // coefficients, then (MODE 0) 1/rD, then the right-hand sides
                const double c0 = d[0], c3 = (MODE == 0) ? d[96] : 0.0;
                cy[s] = (MODE == 2) ? d[64] : d[32];
                cx[s] = (MODE == 2) ? d[96] : d[64];
                cell[s] = (MODE == 1) ? myCStage[(buf * P + s) * 32 + lane] : 0;
                const double zk = (MODE == 2) ? 1.0 : 0.0;
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    double wk;
                    if (kLocalProd) wk = ringK[(((size_t)jo * R + (t & (R - 1))) * 32 + lane) * NC + q];
                    else if (kGlob >= 0) {
                        const long long e = e0 + t * st;
                        const double *kv = (MODE == 2) ? g.rDraw : g.wS + (long long)q * g.nSkew;
                        wk = __ldcg(kv + ((MODE == 1) ? e + KS : e - KS));
                    } else wk = zk;
                    wjv[s][q] = (depJ >= 0 && t + 31 < T)
                                    ? ringJ[((size_t)depJ * RJ + ((t + 31) & (RJ - 1))) * NC + q] : zk;
                    if (MODE == 2) {
                        pre[s][q] = __dsub_rn(c0, __ddiv_rn(d[32], wk));   // D - Pz / rD(k-1)
                    } else {
                        const double rk = d[(4 + q) * 32];
                        const double v0 = (MODE == 0) ? __dmul_rn(c3, rk) : rk;
                        pre[s][q] = __fma_rn(-c0, wk, v0);
                    }
                }
            }
#pragma unroll
            for (int s = 0; s < P; ++s) {
                const int t = t0 + s;
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    const double yup = __shfl_up_sync(0xffffffffu, yprev[q], 1);
                    const double yj = (lane > 0) ? yup : wjv[s][q];
                    double v;
                    if (MODE == 2) {
                        v = __dsub_rn(pre[s][q], __ddiv_rn(cy[s], yj));
                        v = __dsub_rn(v, __ddiv_rn(cx[s], yprev[q]));
                    } else {
                        v = __fma_rn(-cy[s], yj, pre[s][q]);
                        v = __fma_rn(-cx[s], yprev[q], v);
                    }
                    if (kLocalCons) consRing[(((size_t)jo * R + (t & (R - 1))) * 32 + lane) * NC + q] = v;
                    if (consJ >= 0 && lane == 31) ringJ[((size_t)jo * RJ + (t & (RJ - 1))) * NC + q] = v;
                    out[s][q] = v;
                    yprev[q] = v;
                }
            }
            // ---- publish the shared-memory hand-offs: the warp barrier orders
            // every lane's ring stores before lane 0's cluster-scope release
            __syncwarp();
            if (lane == 0) {
                if (consJ >= 0 || depJ >= 0) st_release_cluster(sProg + jo, te);
                if (kLocalCons) st_release_cluster(consKin + jo, te);
                if (kLocalProd) st_release_cluster(prodBack + jo, te);
            }
            // ---- stage chunk c + 2 (always commit a group, possibly empty)
            if (te + P < T) stage_chunk(te + P, ((t0 / P) + 2) % 3);
            cp_async_commit();
            // ---- the previous chunk's global stores (one chunk late)
            if (prevT0 >= 0) {
#pragma unroll
                for (int s = 0; s < P; ++s) {
                    const long long e = e0 + (prevT0 + s) * st;
                    if (MODE == 2) {
                        g.rDraw[e] = prevOut[s][0];
                    } else {
#pragma unroll
                        for (int q = 0; q < NC; ++q) {
                            if (!((mask >> q) & 1u)) continue;
                            g.wS[(long long)q * g.nSkew + e] = prevOut[s][q];
                            if (MODE == 1 && prevCell[s] >= 0) w[(long long)q * N + prevCell[s]] = prevOut[s][q];
                        }
                    }
                }
                if (crossProducer && ((t0 % (2 * P)) == 0)) {
                    __threadfence();
                    __syncwarp();
                    if (lane == 0) store_release(gprog + blk, t0);
                }
            }
#pragma unroll
            for (int s = 0; s < P; ++s) {
                prevCell[s] = cell[s];
#pragma unroll
                for (int q = 0; q < NC; ++q) prevOut[s][q] = out[s][q];
            }
            prevT0 = t0;
        }
        if (!fail && prevT0 >= 0) {
#pragma unroll
            for (int s = 0; s < P; ++s) {
                const long long e = e0 + (prevT0 + s) * st;
                if (MODE == 2) {
                    g.rDraw[e] = prevOut[s][0];
                } else {
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        if (!((mask >> q) & 1u)) continue;
                        g.wS[(long long)q * g.nSkew + e] = prevOut[s][q];
                        if (MODE == 1 && prevCell[s] >= 0) w[(long long)q * N + prevCell[s]] = prevOut[s][q];
                    }
                }
            }
            if (crossProducer) {
                __threadfence();
                __syncwarp();
                if (lane == 0) store_release(gprog + blk, T);
            }
        }
        cp_async_wait<0>();
        if (fail && lane == 0) {
            st_release_cluster(sProg + jo, T);
            if (kLocalCons) st_release_cluster(consKin + jo, T);
            if (kLocalProd) st_release_cluster(prodBack + jo, T);
            if (crossProducer) {
                __threadfence();
                store_release(gprog + blk, T);
            }
        }
    }
    // no CTA may leave while a neighbour can still access its shared memory
    cluster.sync();
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
        if (fz >= 0) pz = __dmul_rn(upper[fz], lower[fz]);
        if (fy >= 0) py = __dmul_rn(upper[fy], lower[fy]);
        if (fx >= 0) px = __dmul_rn(upper[fx], lower[fx]);
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

template <int MODE, int NC, int P>
void launch_one(rt_ctx *ctx, const SkewView &g, unsigned mask, double *w, int CS) {
    StructMesh &s = ctx->mesh.sm;
    const size_t shm = sweep_smem_bytes<MODE, NC, P>(g.nJB);
    static size_t attr = 0;   // per instantiation: dynamic shared memory opted in so far
    if (shm > attr) {
        RT_CUDA(cudaFuncSetAttribute(k_systolic<MODE, NC, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        RT_CUDA(cudaFuncSetAttribute(k_systolic<MODE, NC, P>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        attr = shm;
    }
    const int nGroups = (g.nz + CS - 1) / CS;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nGroups * CS);
    cfg.blockDim = dim3(32 * g.nJB);
    cfg.dynamicSmemBytes = shm;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    RT_CUDA(cudaLaunchKernelEx(&cfg, k_systolic<MODE, NC, P>, g, mask, w, ctx->mesh.N, s.sync.p, 1ll << 24));
}

template <int MODE>
void launch_mode(rt_ctx *ctx, const SkewView &g, int nc, unsigned mask, double *w) {
    StructMesh &s = ctx->mesh.sm;
    RT_CUDA(cudaMemsetAsync(s.sync.p, 0, sizeof(int) * (SYNC_PROGRESS + g.nz * g.nJB), ctx->stream));
    const int CS = s.KC;   // planes (CTAs) per cluster
    if (MODE == 2 || nc == 1) {
        // chunks of 8 steps when the staging fits in shared memory, else 4
        if (sweep_smem_bytes<MODE, 1, 8>(g.nJB) <= kMaxSmem) launch_one<MODE, 1, 8>(ctx, g, mask, w, CS);
        else launch_one<MODE, 1, 4>(ctx, g, mask, w, CS);
    }
    else if (nc <= 3) launch_one<MODE, 3, 2>(ctx, g, mask, w, CS);
    else launch_one<MODE, 6, 2>(ctx, g, mask, w, CS);
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
