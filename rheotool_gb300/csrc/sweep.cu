// sweep.cu — systolic triangular sweeps of DIC / DILU on structured meshes.
//
// A structured mesh is the active-cell subset of an nx x ny x nz box numbered
// lexicographically (i fastest), as blockMesh numbers a block.  Its lower
// neighbours are (i,j,k-1), (i,j-1,k), (i-1,j,k) in increasing face order, its
// upper neighbours (i+1,j,k), (i,j+1,k), (i,j,k+1).  The sequential D-ILU
// recurrences of OpenFOAM (rD, forward, backward; face-ordered accumulation)
// are evaluated here in exactly that order of operations, so the FP64 result
// equals the level-scheduled sweep bit for bit (and the sequential sweep up to
// FMA contraction).  The same kernel runs in FP32 for the mixed-precision
// solvers (coefficients rounded from the FP64 factorisation).
//
// Work decomposition: rows (j,k) are grouped in blocks of 32 consecutive j in
// one plane k.  A warp owns a block; at step t lane l updates cell i = t - l of
// row j = 32 jb + l.  The i-1 value is the lane's own previous result
// (register) and the j-1 value lane l-1's previous result (shuffle).  Lane 0
// reads j-1 from the j-block below (step t + 31) and every lane reads k-1 from
// the block of the previous plane (same step).  The steps are taken in chunks
// of P: a chunk waits once, reads its staged coefficients and publishes once.
//
// One CTA owns one plane (warp = j-block); a thread-block cluster owns CS
// consecutive planes.  Values handed to another warp (plane to plane through
// distributed shared memory, j-block to j-block through shared memory,
// cluster to cluster through global memory) travel as tagged 64-bit words, so
// a consumer waits on the data itself and no fence or release/acquire pair
// sits on the dependency chain.  Clusters take plane groups in dependency
// order from an atomic counter, so a cluster only waits on groups owned by
// running clusters: no deadlock.  Every wait is bounded; a timeout sets an
// error flag, every other wait gives up on seeing it, and the host reports
// RT_ETIMEOUT.
//
// Per-entry data live in a "skewed" layout, entry (block, step, lane), so the
// 32 lanes of a step touch 32 consecutive values.  The backward sweep walks
// the same layout in reverse (lanes mirrored).
#include <algorithm>

#include <cooperative_groups.h>

#include "real_ops.cuh"
#include "rt_internal.h"
#include "sweep.h"

namespace rt {

namespace cg = cooperative_groups;

// ---- tagged hand-off words ------------------------------------------------
// A value handed to another warp travels with the step it belongs to, packed
// into one 64-bit word (32-bit payload in the low half, 32-bit tag in the
// high half) that is written and read with single-copy-atomic 64-bit
// accesses: a reader sees either the old word (wrong tag) or the new one
// (value and tag together), so no fence, release or acquire is needed.  An
// FP64 value travels as two words (its high and low halves), each tagged.
// Ring slots inside a launch carry tag = step + 1 (the rings are cleared at
// launch); the global hand-off between clusters carries the launch's epoch,
// so words left by an earlier launch never match.
typedef unsigned long long u64;
template <class Real> struct Words;
template <> struct Words<float> { static constexpr int W = 1; };
template <> struct Words<double> { static constexpr int W = 2; };

__device__ __forceinline__ void put_word(volatile u64 *p, unsigned payload, unsigned tag) {
    *p = ((u64)tag << 32) | (u64)payload;
}
__device__ __forceinline__ void put(volatile u64 *p, float v, unsigned tag) { put_word(p, __float_as_uint(v), tag); }
__device__ __forceinline__ void put(volatile u64 *p, double v, unsigned tag) {
    put_word(p, (unsigned)__double2hiint(v), tag);
    put_word(p + 1, (unsigned)__double2loint(v), tag);
}
__device__ __forceinline__ bool get(const volatile u64 *p, unsigned tag, float &v) {
    const u64 a = *p;
    if ((unsigned)(a >> 32) != tag) return false;
    v = __uint_as_float((unsigned)a);
    return true;
}
__device__ __forceinline__ bool get(const volatile u64 *p, unsigned tag, double &v) {
    const u64 a = p[0], b = p[1];
    if ((unsigned)(a >> 32) != tag || (unsigned)(b >> 32) != tag) return false;
    v = __hiloint2double((int)(unsigned)a, (int)(unsigned)b);
    return true;
}

__device__ __forceinline__ bool unpack(const u64 *w, unsigned tag, float &v) {
    if ((unsigned)(w[0] >> 32) != tag) return false;
    v = __uint_as_float((unsigned)w[0]);
    return true;
}
__device__ __forceinline__ bool unpack(const u64 *w, unsigned tag, double &v) {
    if ((unsigned)(w[0] >> 32) != tag || (unsigned)(w[1] >> 32) != tag) return false;
    v = __hiloint2double((int)(unsigned)w[0], (int)(unsigned)w[1]);
    return true;
}

// prefetch bytes (a multiple of 16, 16-byte aligned) into L2
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// bounded wait of one lane for a tagged value; false after a timeout or when
// another warp has failed (the error flag is then set)
template <class Real>
__device__ __forceinline__ bool wait_get(const volatile u64 *p, unsigned tag, Real &v, int *sync, long long maxSpin,
                                         bool sleep) {
    long long spins = 0;
    while (!get(p, tag, v)) {
        if ((++spins & 63) == 0 && (spins > maxSpin || *(volatile int *)(sync + SYNC_ERROR))) {
            atomicExch(sync + SYNC_ERROR, 1);
            return false;
        }
        if (sleep) __nanosleep(64);
    }
    return true;
}

// bounded wait of lane 0 on a progress counter; -1 after a timeout
__device__ __forceinline__ int wait_count(const volatile int *c, int need, int *sync, long long maxSpin) {
    long long spins = 0;
    int v = *c;
    while (v < need) {
        if ((++spins & 255) == 0 && (spins > maxSpin || *(volatile int *)(sync + SYNC_ERROR))) {
            atomicExch(sync + SYNC_ERROR, 1);
            return -1;
        }
        v = *c;
    }
    return v;
}

// Ring depths (steps, powers of two) of the hand-offs for chunk size P.
template <int P> struct Ring {
    static constexpr int R = (P >= 16) ? 32 : (P >= 4) ? 16 : 8;   // plane ring: at least two chunks
    static constexpr int RJ = (P >= 8) ? 128 : 64;    // j-block ring: the consumer lags ~32 + P steps
};

// Per-warp staging of a chunk's coefficients (cp.async, three buffers): NA
// arrays of P steps x 32 lanes, plus the cells of the backward sweep.
template <int MODE, int NC> struct Stage { static constexpr int NA = 4 + NC; };

constexpr size_t kMaxSmem = 227 * 1024 - 1024;   // dynamic shared memory per CTA (static part kept free)
constexpr int kPre = 8;                   // L2 prefetch distance (chunks)

template <class Real, int MODE, int NC, int P, int NB = 3>
size_t sweep_smem_bytes(int nJB) {
    constexpr int VW = NC * Words<Real>::W;
    const size_t rings = (size_t)nJB * (Ring<P>::R * 32 + Ring<P>::RJ) * VW * sizeof(u64);
    const size_t stage = (size_t)nJB * NB * P * 32 * (Stage<MODE, NC>::NA * sizeof(Real) + sizeof(int));
    return rings + stage;
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem), "n"(BYTES));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// MODE 0: forward application, 1: backward application, 2: rD recurrence
// (FP64 only).
//
// The producer CTA of a plane writes each step's 32 lanes, tagged, straight
// into the consumer CTA's ring (distributed shared memory); each consumer lane
// waits on its own slot.  The consumer reports its progress back into the
// producer's shared memory after each chunk, which bounds how far the
// producer may run ahead (so a slot is never overwritten before it is read;
// the two waits can never close a cycle).  The j-block hand-off stays inside
// the CTA (lane 31 of the block below, through a tagged shared ring).  The
// first plane of a cluster reads the previous cluster's last plane from a
// tagged global array (one entry per boundary, block, step and lane, written
// once per launch).  All CTAs of a cluster are co-scheduled, and none leaves
// before the final cluster barrier, so no CTA ever touches the shared memory
// of a CTA that has exited.
//
// Latency: a chunk's coefficients are staged into shared memory with cp.async
// two chunks ahead; the terms of a step that do not depend on the previous
// step are formed for the whole chunk first, so only the j and i terms stay
// on the dependent chain.  Invalid entries (outside the mesh, padding) have
// zero coefficients and zero right-hand sides, so every lane runs the same
// branch-free recurrence.
template <class Real, int MODE, int NC, int P, int NB>
__global__ void __launch_bounds__(512) k_systolic(SkewT<Real> g, unsigned mask, Real *__restrict__ w, int N,
                                                  int *sync, u64 *__restrict__ xfer, unsigned epoch,
                                                  long long maxSpin) {
    constexpr int R = Ring<P>::R, RJ = Ring<P>::RJ, NA = Stage<MODE, NC>::NA, W = Words<Real>::W;
    constexpr int VW = NC * W;   // words per (step, lane)
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks(), r = (int)cluster.block_rank();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_grp;
    __shared__ int kBack[16], jProg[16];
    const int lane = threadIdx.x & 31, jo = threadIdx.x >> 5;
    const int nJB = g.nJB;
    u64 *ringK = reinterpret_cast<u64 *>(smem_raw);                 // [nJB][R][32][VW], written by the k-producer
    u64 *ringJ = ringK + (size_t)nJB * R * 32 * VW;                  // [nJB][RJ][VW]
    Real *stage = reinterpret_cast<Real *>(ringJ + (size_t)nJB * RJ * VW);   // [nJB][3][P][NA][32]
    int *cstage = (int *)(stage + (size_t)nJB * NB * P * NA * 32);   // [nJB][NB][P][32]
    Real *myStage = stage + (size_t)jo * NB * P * NA * 32;
    int *myCStage = cstage + (size_t)jo * NB * P * 32;
    for (size_t i = threadIdx.x; i < (size_t)nJB * (R * 32 + RJ) * VW; i += blockDim.x) ringK[i] = 0ull;
    if (threadIdx.x < 16) { kBack[threadIdx.x] = 0; jProg[threadIdx.x] = 0; }
    if (r == 0 && threadIdx.x == 0) s_grp = atomicAdd(sync + SYNC_WORK, 1);
    cluster.sync();
    const int grp = *cluster.map_shared_rank(&s_grp, 0);
    const int nGroups = (g.nz + CS - 1) / CS;
    const int T = g.T;
    const int gi = (MODE == 1) ? nGroups - 1 - grp : grp;
    const int k = (MODE == 1) ? gi * CS + (CS - 1 - r) : gi * CS + r;
    const bool exists = grp < nGroups && k >= 0 && k < g.nz;
    if (exists) {
        const int jb = (MODE == 1) ? nJB - 1 - jo : jo;
        const long long BS = (long long)T * 32;
        const int blk = k * nJB + jb;
        const bool hasK = (MODE == 1) ? (k + 1 < g.nz) : (k > 0);
        const bool kLocalProd = hasK && r > 0;
        const bool kGlob = hasK && r == 0;
        const bool consExists = (MODE == 1) ? (k - 1 >= 0) : (k + 1 < g.nz);
        const bool kLocalCons = consExists && r + 1 < CS;
        const bool crossProducer = consExists && r == CS - 1;
        // cluster boundaries: b separates plane groups b and b + 1
        const int bIn = (MODE == 1) ? gi : gi - 1, bOut = (MODE == 1) ? gi - 1 : gi;
        const int depJ = (jo > 0) ? jo - 1 : -1;
        const int consJ = (jo + 1 < nJB) ? jo + 1 : -1;
        u64 *consRing = kLocalCons ? cluster.map_shared_rank(ringK, r + 1) : nullptr;
        int *prodBack = kLocalProd ? cluster.map_shared_rank(kBack, r - 1) : nullptr;
        // entry of step t: e0 + t * st
        const long long e0 = (MODE == 1) ? (long long)blk * BS + (long long)(T - 1) * 32 + (31 - lane)
                                         : (long long)blk * BS + lane;
        const long long st = (MODE == 1) ? -32 : 32;
        auto xslot = [&](int b, int t, int q) -> u64 * {
            return xfer + ((((size_t)b * nJB + jb) * T + t) * 32 + lane) * VW + q * W;
        };
        // stage the coefficients of the chunk starting at step tc into buffer
        // b: the chunk's entries of one array are one contiguous block of
        // P x 32 (the backward sweep walks it mirrored), copied in 16-byte
        // pieces spread over the lanes; smem layout [buffer][array][P * 32]
        constexpr int EPC = 16 / (int)sizeof(Real);   // entries per 16-byte piece
        constexpr int PIECES = P * 32 / EPC;
        auto copy_block = [&](Real *dst, const Real *src) {
#pragma unroll
            for (int i = lane; i < PIECES; i += 32) cp_async<16>(dst + i * EPC, src + i * EPC);
        };
        auto stage_chunk = [&](int tc, int b) {
            const long long lo = (MODE == 1) ? (long long)blk * BS + (long long)(T - tc - P) * 32
                                             : (long long)blk * BS + (long long)tc * 32;
            Real *dst = myStage + (size_t)b * NA * P * 32;
            if (MODE == 2) {
                copy_block(dst + 0 * P * 32, g.D + lo); copy_block(dst + 1 * P * 32, g.Pz + lo);
                copy_block(dst + 2 * P * 32, g.Py + lo); copy_block(dst + 3 * P * 32, g.Px + lo);
            } else {
                copy_block(dst + 0 * P * 32, (MODE == 0 ? g.Az : g.Bz) + lo);
                copy_block(dst + 1 * P * 32, (MODE == 0 ? g.Ay : g.By) + lo);
                copy_block(dst + 2 * P * 32, (MODE == 0 ? g.Ax : g.Bx) + lo);
#pragma unroll
                for (int q = 0; q < NC; ++q)
                    copy_block(dst + (size_t)(4 + q) * P * 32, (MODE == 0 ? g.rS : g.wS) + (long long)q * g.nSkew + lo);
                if (MODE == 1) {
#pragma unroll
                    for (int i = lane; i < P * 8; i += 32)
                        cp_async<16>(myCStage + b * P * 32 + i * 4, g.cellOf + lo + i * 4);
                }
            }
        };
        int seenCK = 0, seenCJ = 0, fail = 0;
        Real yprev[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) yprev[q] = (MODE == 2) ? Real(1) : Real(0);
        // NB staging buffers: chunk c is staged NB - 1 chunks ahead
#pragma unroll
        for (int c = 0; c < NB - 1; ++c) {
            if (c * P < T) stage_chunk(c * P, c);
            cp_async_commit();
        }

        for (int t0 = 0; t0 < T; t0 += P) {
            const int te = t0 + P;   // T is a multiple of P
            const int buf = (t0 / P) % NB;
            cp_async_wait<NB - 2>();   // this chunk's group is complete
            // ---- back-pressure: consumers have read what this chunk overwrites
            if (kLocalCons && seenCK < te - R) {
                int v = 0;
                if (lane == 0) v = wait_count(kBack + jo, te - R, sync, maxSpin);
                v = __shfl_sync(0xffffffffu, v, 0);
                if (v < 0) { fail = 1; break; }
                seenCK = v;
            }
            if (consJ >= 0 && seenCJ < te - RJ - 31) {
                int v = 0;
                if (lane == 0) v = wait_count(jProg + consJ, te - RJ - 31, sync, maxSpin);
                v = __shfl_sync(0xffffffffu, v, 0);
                if (v < 0) { fail = 1; break; }
                seenCJ = v;
            }
            // ---- L2 prefetch of the chunk kPre chunks ahead (one lane, one
            // contiguous range per array)
            if (lane == 0 && t0 + kPre * P < T) {
                const int tp = t0 + kPre * P;
                const long long lo = (MODE == 1) ? e0 - 31 + (long long)(tp + P - 1) * st : e0 + (long long)tp * st;
                const unsigned bytes = (unsigned)(P * 32 * sizeof(Real));
                if (MODE == 2) {
                    prefetch_l2(g.D + lo, bytes); prefetch_l2(g.Pz + lo, bytes);
                    prefetch_l2(g.Py + lo, bytes); prefetch_l2(g.Px + lo, bytes);
                } else {
                    prefetch_l2((MODE == 0 ? g.Az : g.Bz) + lo, bytes);
                    prefetch_l2((MODE == 0 ? g.Ay : g.By) + lo, bytes);
                    prefetch_l2((MODE == 0 ? g.Ax : g.Bx) + lo, bytes);
#pragma unroll
                    for (int q = 0; q < NC; ++q)
                        prefetch_l2((MODE == 0 ? g.rS : g.wS) + (long long)q * g.nSkew + lo, bytes);
                    if (MODE == 1) prefetch_l2(g.cellOf + lo, (unsigned)(P * 32 * sizeof(int)));
                }
            }
            // ---- the hand-off values of the chunk: every load is issued
            // first, then the tags are checked (a word not there yet is waited for)
            Real wkv[P][NC], wjv[P][NC];
            bool ok = true;
            const Real zk = (MODE == 2) ? Real(1) : Real(0);
            if (kLocalProd || kGlob) {
                u64 kw[P][VW];
#pragma unroll
                for (int s = 0; s < P; ++s) {
                    const volatile u64 *src = kLocalProd
                        ? ringK + (((size_t)jo * R + ((t0 + s) & (R - 1))) * 32 + lane) * VW
                        : xslot(bIn, t0 + s, 0);
#pragma unroll
                    for (int j = 0; j < VW; ++j) kw[s][j] = src[j];
                }
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        const unsigned tag = kLocalProd ? (unsigned)(t0 + s + 1) : epoch;
                        if (!unpack(&kw[s][q * W], tag, wkv[s][q])) {
                            const volatile u64 *src = kLocalProd
                                ? ringK + (((size_t)jo * R + ((t0 + s) & (R - 1))) * 32 + lane) * VW + q * W
                                : xslot(bIn, t0 + s, q);
                            ok &= wait_get(src, tag, wkv[s][q], sync, kLocalProd ? maxSpin : maxSpin >> 4, kGlob);
                        }
                    }
            } else {
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int q = 0; q < NC; ++q) wkv[s][q] = zk;
            }
#pragma unroll
            for (int s = 0; s < P; ++s)
#pragma unroll
                for (int q = 0; q < NC; ++q) wjv[s][q] = zk;
            if (depJ >= 0 && lane == 0) {
                u64 jw[P][VW];
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int j = 0; j < VW; ++j)
                        jw[s][j] = (t0 + s + 31 < T) ? ringJ[((size_t)depJ * RJ + ((t0 + s + 31) & (RJ - 1))) * VW + j]
                                                     : 0ull;
#pragma unroll
                for (int s = 0; s < P; ++s)
                    if (t0 + s + 31 < T)
#pragma unroll
                        for (int q = 0; q < NC; ++q)
                            if (!unpack(&jw[s][q * W], (unsigned)(t0 + s + 32), wjv[s][q]))
                                ok &= wait_get(ringJ + ((size_t)depJ * RJ + ((t0 + s + 31) & (RJ - 1))) * VW + q * W,
                                               (unsigned)(t0 + s + 32), wjv[s][q], sync, maxSpin, false);
            }
            // ---- the terms that do not depend on the previous step
            Real out[P][NC];
            int cell[P];
            Real pre[P][NC], cy[P], cx[P];
            const Real *db = myStage + (size_t)buf * NA * P * 32;
#pragma unroll
            for (int s = 0; s < P; ++s) {
                // entry of (step s, lane) inside the chunk's blocks
                const int si = (MODE == 1) ? (P - 1 - s) * 32 + (31 - lane) : s * 32 + lane;
                const Real *d = db + si;
                const Real c0 = d[0];
                cy[s] = (MODE == 2) ? d[2 * P * 32] : d[P * 32];
                cx[s] = (MODE == 2) ? d[3 * P * 32] : d[2 * P * 32];
                cell[s] = (MODE == 1) ? myCStage[buf * P * 32 + si] : 0;
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    const Real wk = wkv[s][q];
                    if (MODE == 2) {
                        pre[s][q] = r_sub(c0, r_div(d[P * 32], wk));   // D - Pz / rD(k-1)
                    } else {
                        // MODE 0: rk = rD r (premultiplied by the gather, the
                        // sequential sweep's first product); MODE 1: rk = w
                        const Real rk = d[(size_t)(4 + q) * P * 32];
                        pre[s][q] = r_fma(-c0, wk, rk);
                    }
                }
            }
            if (__any_sync(0xffffffffu, !ok)) { fail = 1; break; }
            // ---- the recurrence (order of operations of the sequential sweep)
#pragma unroll
            for (int s = 0; s < P; ++s) {
                const int t = t0 + s;
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    const Real yup = __shfl_up_sync(0xffffffffu, yprev[q], 1);
                    const Real yj = (lane > 0) ? yup : wjv[s][q];
                    Real v;
                    if (MODE == 2) {
                        v = r_sub(pre[s][q], r_div(cy[s], yj));
                        v = r_sub(v, r_div(cx[s], yprev[q]));
                    } else {
                        v = r_fma(-cy[s], yj, pre[s][q]);
                        v = r_fma(-cx[s], yprev[q], v);
                    }
                    out[s][q] = v;
                    yprev[q] = v;
                }
                (void)t;
            }
            // ---- publish the chunk's hand-off words (the consumers read whole
            // chunks, so publishing per chunk costs them no latency and keeps
            // the addressing off the dependent chain; a chunk never wraps a
            // ring: R and RJ are multiples of P)
            if (kLocalCons) {
                u64 *base = consRing + (((size_t)jo * R + (t0 & (R - 1))) * 32 + lane) * VW;
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int q = 0; q < NC; ++q) put(base + s * 32 * VW + q * W, out[s][q], (unsigned)(t0 + s + 1));
            }
            if (consJ >= 0 && lane == 31) {
                u64 *base = ringJ + ((size_t)jo * RJ + (t0 & (RJ - 1))) * VW;
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int q = 0; q < NC; ++q) put(base + s * VW + q * W, out[s][q], (unsigned)(t0 + s + 1));
            }
            if (crossProducer) {
                u64 *base = xslot(bOut, t0, 0);
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int q = 0; q < NC; ++q) put(base + s * 32 * VW + q * W, out[s][q], epoch);
            }
            // ---- progress for the producers' back-pressure (after every lane
            // has consumed its hand-off values of this chunk)
            __syncwarp();
            if (lane == 0) {
                if (kLocalProd) *(volatile int *)(prodBack + jo) = te;
                if (depJ >= 0) *(volatile int *)(jProg + jo) = te;
            }
            // ---- stage chunk c + 2 (always commit a group, possibly empty)
            if (te + (NB - 2) * P < T) stage_chunk(te + (NB - 2) * P, ((t0 / P) + NB - 1) % NB);
            cp_async_commit();
            // ---- this chunk's results
#pragma unroll
            for (int s = 0; s < P; ++s) {
                const long long e = e0 + (t0 + s) * st;
                if (MODE == 2) {
                    g.rDraw[e] = out[s][0];
                } else {
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        if (!((mask >> q) & 1u)) continue;
                        g.wS[(long long)q * g.nSkew + e] = out[s][q];
                        if (MODE == 1 && cell[s] >= 0) w[(long long)q * N + cell[s]] = out[s][q];
                    }
                }
            }
        }
        cp_async_wait<0>();
        // a failed warp lets the producers that wait on its progress go
        if (fail && lane == 0) {
            if (kLocalProd) *(volatile int *)(prodBack + jo) = T;
            if (depJ >= 0) *(volatile int *)(jProg + jo) = T;
        }
    }
    // no CTA may leave while a neighbour can still access its shared memory
    cluster.sync();
}

// rS = rD r gathered into the skewed layout (0 outside the mesh): the first
// product of the forward recurrence, rounded as the sequential sweep rounds it
template <class Real>
__global__ void k_skew_gather(SkewT<Real> g, unsigned mask, int nc, const Real *__restrict__ r, int N) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    int c = g.cellOf[e];
    const Real rd = g.rDinv[e];
    for (int q = 0; q < nc; ++q)
        if ((mask >> q) & 1u)
            g.rS[(long long)q * g.nSkew + e] = c >= 0 ? r_mul(rd, r[(long long)q * N + c]) : Real(0);
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

// FP32 copies of the FP64 sweep coefficients
__global__ void k_skew_to32(SkewView g, SkewView32 h) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    h.rDinv[e] = (float)g.rDinv[e];
    h.Az[e] = (float)g.Az[e]; h.Ay[e] = (float)g.Ay[e]; h.Ax[e] = (float)g.Ax[e];
    h.Bz[e] = (float)g.Bz[e]; h.By[e] = (float)g.By[e]; h.Bx[e] = (float)g.Bx[e];
}

namespace {

template <class Real, int MODE, int NC, int P, int NB = 3>
void launch_one(rt_ctx *ctx, const SkewT<Real> &g, unsigned mask, Real *w, int CS) {
    StructMesh &s = ctx->mesh.sm;
    const size_t shm = sweep_smem_bytes<Real, MODE, NC, P, NB>(g.nJB);
    static size_t attr = 0;   // per instantiation: dynamic shared memory opted in so far
    if (shm > attr) {
        RT_CUDA(cudaFuncSetAttribute(k_systolic<Real, MODE, NC, P, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)shm));
        RT_CUDA(cudaFuncSetAttribute(k_systolic<Real, MODE, NC, P, NB>, cudaFuncAttributeNonPortableClusterSizeAllowed,
                                     1));
        attr = shm;
    }
    const int nGroups = (g.nz + CS - 1) / CS;
    // tagged hand-off between clusters: (boundaries) x blocks x steps x lanes x words
    const size_t words = (size_t)std::max(1, nGroups - 1) * g.nJB * g.T * 32 * NC * Words<Real>::W;
    if (s.xfer.n < words) {
        s.xfer.alloc(words);
        s.xfer.zero(ctx->stream);
    }
    if (++s.epoch == 0) s.epoch = 1;   // 0 marks a cleared word
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
    RT_CUDA(cudaLaunchKernelEx(&cfg, k_systolic<Real, MODE, NC, P, NB>, g, mask, w, ctx->mesh.N, s.sync.p, s.xfer.p,
                               s.epoch, 1ll << 24));
}

// Schedules of the one-component sweeps (the pressure solve): chunk size P
// (steps per wait) and staging depth NB (chunks in flight); the autotuner
// times the candidates that fit on the first application per mesh and
// precision and keeps the fastest.
constexpr int kTuneN = 5;
constexpr int kTuneP[kTuneN] = {8, 8, 16, 16, 4};
constexpr int kTuneNB[kTuneN] = {3, 5, 3, 4, 6};

template <class Real, int MODE, int K>
bool tune_fits(int nJB) {
    return sweep_smem_bytes<Real, MODE, 1, kTuneP[K], kTuneNB[K]>(nJB) <= kMaxSmem;
}
template <class Real, int MODE>
bool tune_fits_any(int k, int nJB) {
    switch (k) {
    case 0: return tune_fits<Real, MODE, 0>(nJB);
    case 1: return tune_fits<Real, MODE, 1>(nJB);
    case 2: return tune_fits<Real, MODE, 2>(nJB);
    case 3: return tune_fits<Real, MODE, 3>(nJB);
    default: return tune_fits<Real, MODE, 4>(nJB);
    }
}
template <class Real, int MODE>
void launch_tuned(rt_ctx *ctx, const SkewT<Real> &g, unsigned mask, Real *w, int CS, int k) {
    switch (k) {
    case 0: launch_one<Real, MODE, 1, kTuneP[0], kTuneNB[0]>(ctx, g, mask, w, CS); break;
    case 1: launch_one<Real, MODE, 1, kTuneP[1], kTuneNB[1]>(ctx, g, mask, w, CS); break;
    case 2: launch_one<Real, MODE, 1, kTuneP[2], kTuneNB[2]>(ctx, g, mask, w, CS); break;
    case 3: launch_one<Real, MODE, 1, kTuneP[3], kTuneNB[3]>(ctx, g, mask, w, CS); break;
    default: launch_one<Real, MODE, 1, kTuneP[4], kTuneNB[4]>(ctx, g, mask, w, CS); break;
    }
}

// chunk size: the largest of 8, 4, 2, 1 steps whose staging and rings fit
// (one component: the tuned schedule, if any)
template <class Real, int MODE, int NC>
void launch_fit(rt_ctx *ctx, const SkewT<Real> &g, unsigned mask, Real *w, int CS) {
    if constexpr (NC == 1 && MODE != 2) {
        const int k = ctx->mesh.sm.tune[sizeof(Real) == 4 ? 1 : 0];
        if (k >= 0 && tune_fits_any<Real, MODE>(k, g.nJB)) {
            launch_tuned<Real, MODE>(ctx, g, mask, w, CS, k);
            return;
        }
    }
    if constexpr (NC == 1) {
        if (sweep_smem_bytes<Real, MODE, NC, 8>(g.nJB) <= kMaxSmem) {
            launch_one<Real, MODE, NC, 8>(ctx, g, mask, w, CS);
            return;
        }
    }
    // (FP64 six-component chunks of 4 steps would spill registers)
    if (!(sizeof(Real) == 8 && NC == 6) && sweep_smem_bytes<Real, MODE, NC, 4>(g.nJB) <= kMaxSmem) {
        if constexpr (!(sizeof(Real) == 8 && NC == 6)) launch_one<Real, MODE, NC, 4>(ctx, g, mask, w, CS);
    } else if (sweep_smem_bytes<Real, MODE, NC, 2>(g.nJB) <= kMaxSmem) launch_one<Real, MODE, NC, 2>(ctx, g, mask, w, CS);
    else launch_one<Real, MODE, NC, 1>(ctx, g, mask, w, CS);
}

template <class Real, int MODE>
void launch_mode(rt_ctx *ctx, const SkewT<Real> &g, int nc, unsigned mask, Real *w) {
    StructMesh &s = ctx->mesh.sm;
    // the group counter restarts; the error flag stays until skew_check reads it
    RT_CUDA(cudaMemsetAsync(s.sync.p + SYNC_WORK, 0, sizeof(int), ctx->stream));
    const int CS = s.KC;   // planes (CTAs) per cluster
    if (MODE == 2 || nc == 1) launch_fit<Real, MODE, 1>(ctx, g, mask, w, CS);
    else if constexpr (MODE != 2) {
        if (nc <= 3) launch_fit<Real, MODE, 3>(ctx, g, mask, w, CS);
        else if (sweep_smem_bytes<Real, MODE, 6, 1>(g.nJB) <= kMaxSmem) launch_fit<Real, MODE, 6>(ctx, g, mask, w, CS);
        else {
            // six components do not fit one CTA's shared memory (many
            // j-blocks, FP64): two launches of three, on shifted views
            launch_fit<Real, MODE, 3>(ctx, g, mask & 7u, w, CS);
            SkewT<Real> h = g;
            h.rS += 3 * g.nSkew;
            h.wS += 3 * g.nSkew;
            RT_CUDA(cudaMemsetAsync(s.sync.p + SYNC_WORK, 0, sizeof(int), ctx->stream));
            launch_fit<Real, MODE, 3>(ctx, h, (mask >> 3) & 7u, w ? w + 3 * (size_t)ctx->mesh.N : w, CS);
        }
    }
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
    launch_mode<double, 2>(ctx, g, 1, 1u, (double *)nullptr);
    k_skew_premul<<<nb, RT_BLOCK, 0, ctx->stream>>>(g, s.faceLo.p, s.faceHi.p, ctx->mesh.N, upper, lower);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

namespace {

// time every fitting schedule of the one-component sweeps on the current
// right-hand side (two applications each, CUDA events) and keep the fastest
template <class Real>
void autotune(rt_ctx *ctx, const SkewT<Real> &g, unsigned mask, Real *w) {
    StructMesh &s = ctx->mesh.sm;
    int &choice = s.tune[sizeof(Real) == 4 ? 1 : 0];
    if (choice >= 0) return;
    if (ctx->sweepTune > 0) {   // forced (RT_OPT_SWEEP_TUNE)
        choice = ctx->sweepTune - 1;
        return;
    }
    cudaEvent_t a, b;
    RT_CUDA(cudaEventCreate(&a));
    RT_CUDA(cudaEventCreate(&b));
    float best = 1e30f;
    int bestK = 0;
    for (int k = 0; k < kTuneN; ++k) {
        if (!tune_fits_any<Real, 0>(k, g.nJB) || !tune_fits_any<Real, 1>(k, g.nJB)) continue;
        choice = k;
        for (int rep = 0; rep < 3; ++rep) {
            if (rep == 1) RT_CUDA(cudaEventRecord(a, ctx->stream));
            launch_mode<Real, 0>(ctx, g, 1, mask, w);
            launch_mode<Real, 1>(ctx, g, 1, mask, w);
        }
        RT_CUDA(cudaEventRecord(b, ctx->stream));
        RT_CUDA(cudaEventSynchronize(b));
        float ms = 0.f;
        RT_CUDA(cudaEventElapsedTime(&ms, a, b));
        if (ms < best) {
            best = ms;
            bestK = k;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    choice = bestK;
    s.tuneMs[sizeof(Real) == 4 ? 1 : 0] = best / 2;
}

}  // namespace

void skew_precondition(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w) {
    SkewView g = ctx->mesh.sm.view();
    k_skew_gather<double><<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    if (nc == 1) autotune<double>(ctx, g, mask, w);
    launch_mode<double, 0>(ctx, g, nc, mask, w);
    launch_mode<double, 1>(ctx, g, nc, mask, w);
}

void skew_prepare32(rt_ctx *ctx, const double *diag, const double *upper, const double *lower) {
    skew_prepare(ctx, diag, upper, lower);
    StructMesh &s = ctx->mesh.sm;
    SkewView g = s.view();
    SkewView32 h = s.view32();
    k_skew_to32<<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, h);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

void skew_precondition32(rt_ctx *ctx, int nc, unsigned mask, const float *r, float *w) {
    SkewView32 g = ctx->mesh.sm.view32();
    k_skew_gather<float><<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    if (nc == 1) autotune<float>(ctx, g, mask, w);
    launch_mode<float, 0>(ctx, g, nc, mask, w);
    launch_mode<float, 1>(ctx, g, nc, mask, w);
}

rt_status skew_check(rt_ctx *ctx) {
    StructMesh &s = ctx->mesh.sm;
    if (!s.pendingCheck) return RT_OK;
    int err = 0;
    RT_CUDA(cudaMemcpyAsync(&err, s.sync.p + SYNC_ERROR, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RT_CUDA(cudaStreamSynchronize(ctx->stream));
    s.pendingCheck = false;
    if (err) RT_CUDA(cudaMemsetAsync(s.sync.p + SYNC_ERROR, 0, sizeof(int), ctx->stream));
    return err ? RT_ETIMEOUT : RT_OK;
}

}  // namespace rt
