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
// of P: a chunk stages its coefficients and exchanges the j-block words once,
// and takes the previous plane's words and publishes its own to the next
// plane quad by quad (four steps), so the planes lag one another by a quad.
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
// Per-entry data live in a "skewed" layout of (block, step, lane) in which one
// lane's four consecutive steps are adjacent (a quad), so a lane reads and
// writes its coefficients, results and hand-off words as 16-byte vectors.
// The backward sweep walks the same layout in reverse (lanes mirrored).
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


// the value of a word pair, and whether it carries the tag (no branch)
__device__ __forceinline__ bool peek(const u64 *w, unsigned tag, float &v) {
    v = __uint_as_float((unsigned)w[0]);
    return (unsigned)(w[0] >> 32) == tag;
}
__device__ __forceinline__ bool peek(const u64 *w, unsigned tag, double &v) {
    v = __hiloint2double((int)(unsigned)w[0], (int)(unsigned)w[1]);
    return ((unsigned)(w[0] >> 32) == tag) & ((unsigned)(w[1] >> 32) == tag);
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

// Ring depths (steps, powers of two) of the hand-offs for chunk size P.  The
// plane ring is chosen per launch (at least R, at most kMaxRing): a producer
// may run at most one ring ahead of its consumer, and with a ring of only two
// chunks it waits one round trip (data forward, progress back) every chunk,
// so the launch takes the deepest ring that fits the shared memory.
template <int P> struct Ring {
    static constexpr int R = (P >= 16) ? 32 : (P >= 4) ? 16 : 8;   // plane ring: at least two chunks
    static constexpr int RJ = (P >= 8) ? 128 : 64;    // j-block ring: the consumer lags ~32 + P steps
};
constexpr int kMaxRing = 128;

// Per-warp staging of a chunk's coefficients (cp.async, NB buffers): NA
// arrays of P steps x 32 lanes (MODE 2: D, Pz, Py, Px; MODE 0/1: the z, y, x
// coefficients and the NC right-hand sides), plus the cells of the backward
// sweep.
template <int MODE, int NC> struct Stage { static constexpr int NA = (MODE == 2) ? 4 : 3 + NC; };

constexpr size_t kMaxSmem = 227 * 1024 - 1024;   // dynamic shared memory per CTA (static part kept free)

template <class Real, int MODE, int NC, int P, int NB = 3>
size_t sweep_smem_bytes(int nJB, int R = Ring<P>::R) {
    constexpr int VW = NC * Words<Real>::W;
    const size_t rings = (size_t)nJB * ((size_t)R * 32 + Ring<P>::RJ) * VW * sizeof(u64);
    const size_t stage =
        (size_t)nJB * NB * P * 32 * (Stage<MODE, NC>::NA * sizeof(Real) + (MODE == 1 ? sizeof(int) : 0));
    return rings + stage;
}

// the deepest plane ring (a power of two from Ring<P>::R up to cap, and no
// deeper than the sweep) that fits the shared memory
template <class Real, int MODE, int NC, int P, int NB = 3>
int ring_depth(int nJB, int T, int cap) {
    int R = Ring<P>::R;
    while (2 * R <= cap && R < T && sweep_smem_bytes<Real, MODE, NC, P, NB>(nJB, 2 * R) <= kMaxSmem) R *= 2;
    return R;
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem), "n"(BYTES));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// ---- pairs of tagged words (16-byte vector accesses; each 64-bit element is
// single-copy atomic on its own, which is all the tag protocol needs)
__device__ __forceinline__ void ld2_shared(unsigned a, u64 &x, u64 &y) {
    asm volatile("ld.volatile.shared.v2.u64 {%0, %1}, [%2];" : "=l"(x), "=l"(y) : "r"(a) : "memory");
}
__device__ __forceinline__ void st2_shared(unsigned a, u64 x, u64 y) {
    asm volatile("st.volatile.shared.v2.u64 [%0], {%1, %2};" ::"r"(a), "l"(x), "l"(y) : "memory");
}
__device__ __forceinline__ void st2_cluster(unsigned a, u64 x, u64 y) {
    asm volatile("st.volatile.shared::cluster.v2.u64 [%0], {%1, %2};" ::"r"(a), "l"(x), "l"(y) : "memory");
}
__device__ __forceinline__ void ld2_global(const u64 *p, u64 &x, u64 &y) {
    asm volatile("ld.volatile.global.v2.u64 {%0, %1}, [%2];" : "=l"(x), "=l"(y) : "l"(p) : "memory");
}
__device__ __forceinline__ void st2_global(u64 *p, u64 x, u64 y) {
    asm volatile("st.volatile.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(x), "l"(y) : "memory");
}
__device__ __forceinline__ unsigned map_cluster(unsigned a, unsigned rank) {
    unsigned m;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(m) : "r"(a), "r"(rank));
    return m;
}
__device__ __forceinline__ void pack(float v, unsigned tag, u64 *w) { w[0] = ((u64)tag << 32) | __float_as_uint(v); }
__device__ __forceinline__ void pack(double v, unsigned tag, u64 *w) {
    w[0] = ((u64)tag << 32) | (unsigned)__double2hiint(v);
    w[1] = ((u64)tag << 32) | (unsigned)__double2loint(v);
}

// ---- four consecutive steps of one lane (one quad of the skewed layout)
__device__ __forceinline__ void ld4(const float *p, float *v) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(const double *p, double *v) {
    const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void ld4(const int *p, int *v) {
    const int4 a = *reinterpret_cast<const int4 *>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void st4(float *p, const float *v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double *p, const double *v) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
}

// MODE 0: forward application, 1: backward application, 2: rD recurrence
// (FP64 only).
//
// Skewed layout: the entry of (block, step t, lane l) is
// block * 32 T + (t / 4) * 128 + l * 4 + t % 4, so one lane's four
// consecutive steps are one 16-byte (FP32) or 32-byte (FP64) vector and one
// chunk of P steps is one contiguous range of P x 32 entries.  The hand-off
// rings use the same quad order, so a chunk's words are written and read
// with 16-byte vector accesses.
//
// The producer CTA of a plane writes each quad (four steps) of its 32 lanes,
// tagged, straight into the consumer CTA's ring as soon as the quad is
// computed (distributed shared memory: remote stores do not wait, and the
// consumer's local loads are cheap); each consumer lane checks its own words
// quad by quad, so a plane lags the previous one by about a quad.  The consumer reports its progress back into the
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
// NB - 1 chunks ahead and read, with the j-block words, before the wait for
// the previous plane; the terms of a step that do not depend on the previous
// step are formed quad by quad ahead of the recurrence, so only the j and i
// terms stay on the dependent chain.  Invalid entries (outside the mesh, padding) have
// zero coefficients and zero right-hand sides, so every lane runs the same
// branch-free recurrence.
template <class Real, int MODE, int NC, int P, int NB>
__global__ void __launch_bounds__(256, 1) k_systolic(SkewT<Real> g, unsigned mask, Real *__restrict__ w, int N,
                                                  int *sync, u64 *__restrict__ xfer, unsigned epoch,
                                                  unsigned cepoch, long long maxSpin, int R, int ncc,
                                                  long long xstride) {
    static_assert(P % 4 == 0 && P <= 32, "a chunk is whole quads");
    // every component of the launch has stopped iterating (the same word for
    // every CTA, written by an earlier kernel): nothing to do
    if (g.dmask) {
        mask &= *g.dmask;
        if (!mask) return;
    }
    constexpr int RJ = Ring<P>::RJ, NA = Stage<MODE, NC>::NA, W = Words<Real>::W;
    constexpr int VW = NC * W;   // words per (step, lane)
    constexpr int QW = 4 * VW;   // words per (quad, lane)
    constexpr int PQ = P / 4;    // quads per chunk
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks(), r = (int)cluster.block_rank();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_grp;
    __shared__ int kBack[16], jProg[16];
    const int lane = threadIdx.x & 31, jo = threadIdx.x >> 5;
    const int nJB = g.nJB;
    u64 *ringK = reinterpret_cast<u64 *>(smem_raw);                 // [nJB][R/4][32][4][VW], written by the k-producer
    u64 *ringJ = ringK + (size_t)nJB * R * 32 * VW;                  // [nJB][RJ][VW]
    Real *stage = reinterpret_cast<Real *>(ringJ + (size_t)nJB * RJ * VW);   // [nJB][NB][NA][P * 32]
    int *cstage = (int *)(stage + (size_t)nJB * NB * P * NA * 32);   // [nJB][NB][P * 32] (MODE 1)
    Real *myStage = stage + (size_t)jo * NB * P * NA * 32;
    int *myCStage = cstage + (size_t)jo * NB * P * 32;
    for (size_t i = threadIdx.x; i < (size_t)nJB * (R * 32 + RJ) * VW; i += blockDim.x) ringK[i] = 0ull;
    if (threadIdx.x < 16) { kBack[threadIdx.x] = 0; jProg[threadIdx.x] = 0; }
    if (r == 0 && threadIdx.x == 0) s_grp = atomicAdd(sync + SYNC_WORK, 1);
    cluster.sync();
    // ncc > 1 (one-component kernels only): the launch sweeps ncc components
    // side by side; ticket t is plane group t / ncc of component t % ncc, so
    // every component's groups are taken in dependency order
    const int ticket = *cluster.map_shared_rank(&s_grp, 0);
    const int comp = ticket % ncc;
    const int grp = ticket / ncc;
    if (ncc > 1) {
        g.rS += (long long)comp * g.nSkew;
        g.wS += (long long)comp * g.nSkew;
        if (w) w += (long long)comp * N;
        if (g.w64) g.w64 += (long long)comp * N;
        xfer += (long long)comp * xstride;
        mask = (mask >> comp) & 1u;
    }
    const int nGroups = (g.nz + CS - 1) / CS;
    const int T = g.T;
    const int gi = (MODE == 1) ? nGroups - 1 - grp : grp;
    const int k = (MODE == 1) ? gi * CS + (CS - 1 - r) : gi * CS + r;
    const bool exists = grp < nGroups && k >= 0 && k < g.nz && mask != 0u;
    if (exists) {
        const int jb = (MODE == 1) ? nJB - 1 - jo : jo;
        const int lf = (MODE == 1) ? 31 - lane : lane;   // the lane's entry column in the forward layout
        const long long BS = (long long)T * 32;
        const int blk = k * nJB + jb;
        const long long blk0 = (long long)blk * BS;
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
        const unsigned ringKs = (unsigned)__cvta_generic_to_shared(ringK);
        const unsigned ringJs = (unsigned)__cvta_generic_to_shared(ringJ);
        // the consumer plane's ring, written through distributed shared memory
        const unsigned consRing = kLocalCons ? map_cluster(ringKs, (unsigned)(r + 1)) : 0u;
        int *prodBack = kLocalProd ? cluster.map_shared_rank(kBack, r - 1) : nullptr;
        // word index, in this warp's plane ring, of the quad holding step t of this lane
        auto kword = [&](int t) -> unsigned {
            return ((unsigned)(jo * (R >> 2) + ((t & (R - 1)) >> 2)) * 32u + (unsigned)lane) * QW;
        };
        // the same in the global hand-off at cluster boundary b
        auto xword = [&](int b, int t) -> u64 * {
            return xfer + ((((size_t)b * nJB + jb) * (T >> 2) + (t >> 2)) * 32 + lane) * QW;
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
            const long long lo = (MODE == 1) ? blk0 + (long long)(T - tc - P) * 32 : blk0 + (long long)tc * 32;
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
                    copy_block(dst + (size_t)(3 + q) * P * 32, (MODE == 0 ? g.rS : g.wS) + (long long)q * g.nSkew + lo);
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
            // ---- the chunk's inputs, in the order of their readiness: the
            // j-block words (the block below runs ahead) and the staged
            // coefficients first, then, quad by quad, the previous plane's
            // words, which the pipeline waits on
            Real wkv[P][NC], wjv[P][NC];
            bool ok = true;
            const Real zk = (MODE == 2) ? Real(1) : Real(0);
#pragma unroll
            for (int s = 0; s < P; ++s)
#pragma unroll
                for (int q = 0; q < NC; ++q) wjv[s][q] = zk;
            if (depJ >= 0) {
                // lane s < P fetches and checks the words of step t0 + 31 + s
                // of the block below (lanes past P repeat the last one), all
                // in parallel; lane 0 gathers them by shuffles
                const int ts = t0 + 31 + min(lane, P - 1);
                const bool live = ts < T;   // steps past the row end read as zero
                const volatile u64 *src = ringJ + ((size_t)depJ * RJ + (ts & (RJ - 1))) * VW;
                u64 jw[VW];
#pragma unroll
                for (int j = 0; j < VW; ++j) jw[j] = src[j];
                Real jv[NC];
                bool hit = true;
#pragma unroll
                for (int q = 0; q < NC; ++q) hit &= peek(&jw[q * W], (unsigned)(ts + 1), jv[q]);
                if (__any_sync(0xffffffffu, live && !hit)) {
                    if (live) {
#pragma unroll
                        for (int q = 0; q < NC; ++q)
                            ok &= wait_get(src + q * W, (unsigned)(ts + 1), jv[q], sync, maxSpin, false);
                    }
                    if (__any_sync(0xffffffffu, !ok)) { fail = 1; break; }
                }
#pragma unroll
                for (int q = 0; q < NC; ++q) jv[q] = live ? jv[q] : zk;
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        const Real v = __shfl_sync(0xffffffffu, jv[q], s);
                        if (lane == 0) wjv[s][q] = v;
                    }
            }
            // ---- the terms that do not depend on the previous step (the
            // staged quads of this lane, indexed by forward step offset)
            Real out[P][NC];
            int cell[P];   // MODE 1: the cells, by forward step offset
            Real pre[P][NC], cy[P], cx[P];
            const Real *db = myStage + (size_t)buf * NA * P * 32;
            Real va[NA][P];
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int qd = 0; qd < PQ; ++qd) ld4(db + (size_t)a * P * 32 + qd * 128 + lf * 4, &va[a][4 * qd]);
            if (MODE == 1) {
#pragma unroll
                for (int qd = 0; qd < PQ; ++qd) ld4(myCStage + buf * P * 32 + qd * 128 + lf * 4, &cell[4 * qd]);
            }
            // ---- quad by quad: the previous plane's words of four steps, the
            // terms that wait on them, the recurrence and the publication of
            // the quad's results to the next plane.  The next plane starts on a
            // quad as soon as it is published, so a plane lags the previous
            // one by about one quad of work plus the hand-off, not a chunk.
            // (Each word is checked in registers; one warp-uniform branch
            // leads to the rare bounded waits for words not there yet.  A
            // ring never wraps inside a chunk: R is a multiple of P.)
            // (cepoch, the tag a cluster's first plane expects from the
            // previous cluster, is the launch's epoch except in a
            // failure-detection test, where no producer writes it)
            const unsigned ktag = kLocalProd ? (unsigned)(t0 + 1) : cepoch;
            bool qfail = false;
            // across a cluster boundary the words come from global memory: the
            // whole chunk's words are loaded at once (one memory round trip),
            // and checked quad by quad
            u64 kwg[PQ][QW];
            if (kGlob) {
#pragma unroll
                for (int qd = 0; qd < PQ; ++qd)
#pragma unroll
                    for (int h = 0; h < QW / 2; ++h) ld2_global(xword(bIn, t0 + 4 * qd) + 2 * h, kwg[qd][2 * h], kwg[qd][2 * h + 1]);
            }
#pragma unroll
            for (int qd = 0; qd < PQ; ++qd) {
                if (kLocalProd || kGlob) {
                    u64 kw[QW];
#pragma unroll
                    for (int h = 0; h < QW / 2; ++h) {
                        if (kLocalProd) ld2_shared(ringKs + 8u * (kword(t0 + 4 * qd) + 2 * h), kw[2 * h], kw[2 * h + 1]);
                        else { kw[2 * h] = kwg[qd][2 * h]; kw[2 * h + 1] = kwg[qd][2 * h + 1]; }
                    }
                    bool hit = true;
#pragma unroll
                    for (int e = 0; e < 4; ++e)
#pragma unroll
                        for (int q = 0; q < NC; ++q)
                            hit &= peek(&kw[e * VW + q * W], kLocalProd ? ktag + 4 * qd + e : ktag, wkv[4 * qd + e][q]);
                    if (__any_sync(0xffffffffu, !hit)) {
#pragma unroll
                        for (int e = 0; e < 4; ++e)
#pragma unroll
                            for (int q = 0; q < NC; ++q) {
                                const int s = 4 * qd + e;
                                const int wi = e * VW + q * W;
                                const unsigned tag = kLocalProd ? ktag + s : ktag;
                                const volatile u64 *src = kLocalProd ? ringK + kword(t0 + s) + wi : xword(bIn, t0 + s) + wi;
                                ok &= wait_get(src, tag, wkv[s][q], sync, kLocalProd ? maxSpin : maxSpin >> 4, kGlob);
                            }
                        if (__any_sync(0xffffffffu, !ok)) { qfail = true; break; }
                    }
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
#pragma unroll
                        for (int q = 0; q < NC; ++q) wkv[4 * qd + e][q] = zk;
                }
                // the terms of the quad's steps that do not depend on the previous step
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int s = 4 * qd + e;
                    const int sf = (MODE == 1) ? P - 1 - s : s;
                    if (MODE == 2) {
                        cy[s] = va[2][sf];
                        cx[s] = va[3][sf];
                        pre[s][0] = r_sub(va[0][sf], r_div(va[1][sf], wkv[s][0]));   // D - Pz / rD(k-1)
                    } else {
                        const Real c0 = va[0][sf];
                        cy[s] = va[1][sf];
                        cx[s] = va[2][sf];
                        // MODE 0: rk = rD r (premultiplied by the gather, the
                        // sequential sweep's first product); MODE 1: rk = w
#pragma unroll
                        for (int q = 0; q < NC; ++q) pre[s][q] = r_fma(-c0, wkv[s][q], va[3 + q][sf]);
                    }
                }
                // the recurrence (order of operations of the sequential sweep)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int s = 4 * qd + e;
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        const Real yup = __shfl_up_sync(0xffffffffu, yprev[q], 1);
                        const Real yj = (lane > 0) ? yup : wjv[s][q];
                        Real v;
                        if (MODE == 2) {
                            v = r_sub(pre[s][q], r_div(cy[s], yj));
                            v = r_sub(v, r_div(cx[s], yprev[q]));
                        } else if (sizeof(Real) == 4) {
                            // FP32: the i term first, so only one product waits on the shuffle
                            v = r_fma(-cx[s], yprev[q], pre[s][q]);
                            v = r_fma(-cy[s], yj, v);
                        } else {
                            v = r_fma(-cy[s], yj, pre[s][q]);
                            v = r_fma(-cx[s], yprev[q], v);
                        }
                        out[s][q] = v;
                        yprev[q] = v;
                    }
                }
                // publish the quad to the next plane
                if (kLocalCons || crossProducer) {
                    u64 wd[QW];
#pragma unroll
                    for (int e = 0; e < 4; ++e)
#pragma unroll
                        for (int q = 0; q < NC; ++q)
                            pack(out[4 * qd + e][q], kLocalCons ? (unsigned)(t0 + 4 * qd + e + 1) : epoch,
                                 &wd[e * VW + q * W]);
#pragma unroll
                    for (int h = 0; h < QW / 2; ++h) {
                        if (kLocalCons) st2_cluster(consRing + 8u * (kword(t0 + 4 * qd) + 2 * h), wd[2 * h], wd[2 * h + 1]);
                        else st2_global(xword(bOut, t0 + 4 * qd) + 2 * h, wd[2 * h], wd[2 * h + 1]);
                    }
                }
            }
            if (qfail) { fail = 1; break; }
            // ---- the j-block hand-off words of the whole chunk (the block
            // above lags by more than a chunk)
            if (consJ >= 0 && lane == 31) {
                u64 wd[P * VW];
#pragma unroll
                for (int s = 0; s < P; ++s)
#pragma unroll
                    for (int q = 0; q < NC; ++q) pack(out[s][q], (unsigned)(t0 + s + 1), &wd[s * VW + q * W]);
                const unsigned base = ringJs + 8u * (unsigned)(((jo * RJ) + (t0 & (RJ - 1))) * VW);
#pragma unroll
                for (int h = 0; h < P * VW / 2; ++h) st2_shared(base + 16u * h, wd[2 * h], wd[2 * h + 1]);
            }
            // ---- progress for the producers' back-pressure (after every lane
            // has consumed its hand-off values of this chunk)
            __syncwarp();
            if (lane == 0) {
                if (kLocalProd) *(volatile int *)(prodBack + jo) = te;
                if (depJ >= 0) *(volatile int *)(jProg + jo) = te;
            }
            // ---- stage chunk c + NB - 1 (always commit a group, possibly empty)
            if (te + (NB - 2) * P < T) stage_chunk(te + (NB - 2) * P, ((t0 / P) + NB - 1) % NB);
            cp_async_commit();
            // ---- this chunk's results: the forward sweeps write whole quads
            // of the skewed layout, the backward sweep scatters to the cells
            if (MODE == 1) {
                if (g.w64) {
#pragma unroll
                    for (int s = 0; s < P; ++s)
#pragma unroll
                        for (int q = 0; q < NC; ++q)
                            if (((mask >> q) & 1u) && cell[P - 1 - s] >= 0)
                                g.w64[(long long)q * N + cell[P - 1 - s]] = (double)out[s][q];
                } else {
#pragma unroll
                    for (int s = 0; s < P; ++s)
#pragma unroll
                        for (int q = 0; q < NC; ++q)
                            if (((mask >> q) & 1u) && cell[P - 1 - s] >= 0) w[(long long)q * N + cell[P - 1 - s]] = out[s][q];
                }
            } else {
                const long long e = blk0 + (long long)(t0 >> 2) * 128 + lane * 4;
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    if (MODE == 0 && !((mask >> q) & 1u)) continue;
                    Real *dst = (MODE == 2) ? g.rDraw + e : g.wS + (long long)q * g.nSkew + e;
#pragma unroll
                    for (int qd = 0; qd < PQ; ++qd) {
                        Real v4[4];
#pragma unroll
                        for (int x = 0; x < 4; ++x) v4[x] = out[4 * qd + x][q];
                        st4(dst + qd * 128, v4);
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
// (an FP64 right-hand side of the FP32 sweeps is rounded first)
template <class Real, class In>
__global__ void k_skew_gather(SkewT<Real> g, unsigned mask, int nc, const In *__restrict__ r, int N) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    if (g.dmask) mask &= *g.dmask;
    int c = g.cellOf[e];
    const Real rd = g.rDinv[e];
    for (int q = 0; q < nc; ++q)
        if ((mask >> q) & 1u)
            g.rS[(long long)q * g.nSkew + e] = c >= 0 ? r_mul(rd, (Real)r[(long long)q * N + c]) : Real(0);
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
void launch_one(rt_ctx *ctx, const SkewT<Real> &g, unsigned mask, Real *w, int CS, int ncc = 1) {
    StructMesh &s = ctx->mesh.sm;
    const int R = ring_depth<Real, MODE, NC, P, NB>(g.nJB, g.T, ctx->sweepRing > 0 ? ctx->sweepRing : kMaxRing);
    const size_t shm = sweep_smem_bytes<Real, MODE, NC, P, NB>(g.nJB, R);
    static size_t attr = 0;   // per instantiation: dynamic shared memory opted in so far
    if (shm > attr) {
        RT_CUDA(cudaFuncSetAttribute(k_systolic<Real, MODE, NC, P, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)shm));
        RT_CUDA(cudaFuncSetAttribute(k_systolic<Real, MODE, NC, P, NB>, cudaFuncAttributeNonPortableClusterSizeAllowed,
                                     1));
        attr = shm;
    }
    // a cluster of more than 8 CTAs (non-portable) must fit one GPC with this
    // launch's shared memory; otherwise the portable 8 (checked once per
    // instantiation and cluster size)
    static int fits16 = -1;
    if (CS > 8) {
        if (fits16 < 0) {
            cudaLaunchConfig_t q = {};
            q.gridDim = dim3(CS);
            q.blockDim = dim3(32 * g.nJB);
            q.dynamicSmemBytes = shm;
            cudaLaunchAttribute qa[1];
            qa[0].id = cudaLaunchAttributeClusterDimension;
            qa[0].val.clusterDim.x = CS;
            qa[0].val.clusterDim.y = 1;
            qa[0].val.clusterDim.z = 1;
            q.attrs = qa;
            q.numAttrs = 1;
            int n = 0;
            cudaError_t e = cudaOccupancyMaxActiveClusters(&n, k_systolic<Real, MODE, NC, P, NB>, &q);
            if (e != cudaSuccess) (void)cudaGetLastError();
            fits16 = (e == cudaSuccess && n >= 1) ? 1 : 0;
        }
        if (!fits16) CS = 8;
    }
    const int nGroups = (g.nz + CS - 1) / CS;
    // tagged hand-off between clusters: (boundaries) x blocks x steps x lanes x words
    const size_t words = (size_t)std::max(1, nGroups - 1) * g.nJB * g.T * 32 * NC * Words<Real>::W;
    if (s.xfer.n < words * ncc) {
        s.xfer.alloc(words * ncc);
        s.xfer.zero(ctx->stream);
    }
    if (++s.epoch == 0) s.epoch = 1;   // 0 marks a cleared word
    // failure-detection test (RT_OPT_STALL_TEST): this launch's consumers of
    // the cluster-to-cluster hand-off wait for a tag that no launch writes
    // (epochs stay far below 2^31), so their bounded waits run out
    unsigned cepoch = s.epoch;
    if (ctx->stallTest > 0) {
        cepoch = s.epoch ^ 0x80000000u;
        --ctx->stallTest;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nGroups * CS * ncc);
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
                               s.epoch, cepoch, ctx->waitLimit, R, ncc, (long long)words));
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
void launch_tuned(rt_ctx *ctx, const SkewT<Real> &g, unsigned mask, Real *w, int CS, int k, int ncc = 1) {
    switch (k) {
    case 0: launch_one<Real, MODE, 1, kTuneP[0], kTuneNB[0]>(ctx, g, mask, w, CS, ncc); break;
    case 1: launch_one<Real, MODE, 1, kTuneP[1], kTuneNB[1]>(ctx, g, mask, w, CS, ncc); break;
    case 2: launch_one<Real, MODE, 1, kTuneP[2], kTuneNB[2]>(ctx, g, mask, w, CS, ncc); break;
    case 3: launch_one<Real, MODE, 1, kTuneP[3], kTuneNB[3]>(ctx, g, mask, w, CS, ncc); break;
    default: launch_one<Real, MODE, 1, kTuneP[4], kTuneNB[4]>(ctx, g, mask, w, CS, ncc); break;
    }
}

// the chunk schedule of an NC-component sweep: the tuned one (one
// component), else chunks of 8 (one component) or 4 steps with three staging
// buffers, else 4 steps with two; false when none fits
template <class Real, int MODE, int NC>
bool launch_fit(rt_ctx *ctx, const SkewT<Real> &g, unsigned mask, Real *w, int CS, int ncc = 1) {
    if constexpr (NC == 1 && MODE != 2) {
        const int k = ctx->mesh.sm.tune[sizeof(Real) == 4 ? 1 : 0];
        if (k >= 0 && tune_fits_any<Real, MODE>(k, g.nJB)) {
            launch_tuned<Real, MODE>(ctx, g, mask, w, CS, k, ncc);
            return true;
        }
    }
    if constexpr (NC == 1) {
        if (sweep_smem_bytes<Real, MODE, NC, 8>(g.nJB) <= kMaxSmem) {
            launch_one<Real, MODE, NC, 8>(ctx, g, mask, w, CS, ncc);
            return true;
        }
        if (ncc > 1) return false;
    }
    if (sweep_smem_bytes<Real, MODE, NC, 4>(g.nJB) <= kMaxSmem) {
        launch_one<Real, MODE, NC, 4>(ctx, g, mask, w, CS);
        return true;
    }
    if (sweep_smem_bytes<Real, MODE, NC, 4, 2>(g.nJB) <= kMaxSmem) {
        launch_one<Real, MODE, NC, 4, 2>(ctx, g, mask, w, CS);
        return true;
    }
    return false;
}

// the nc components of one sweep, in launches of as many components as fit
// one CTA's shared memory (six in FP32, three, or one), on shifted views
template <class Real, int MODE>
void launch_mode(rt_ctx *ctx, const SkewT<Real> &g, int nc, unsigned mask, Real *w) {
    StructMesh &s = ctx->mesh.sm;
    const int CS = s.KC;   // planes (CTAs) per cluster
    // components c0 .. c0 + n - 1 in one launch; false (nothing launched)
    // when they do not fit
    auto part = [&](int c0, int n) -> bool {
        const unsigned mc = (mask >> c0) & ((1u << n) - 1u);
        if (!mc) return true;
        SkewT<Real> h = g;
        h.rS += (size_t)c0 * g.nSkew;
        h.wS += (size_t)c0 * g.nSkew;
        if (h.w64) h.w64 += (size_t)c0 * ctx->mesh.N;
        Real *wc = w ? w + (size_t)c0 * ctx->mesh.N : w;
        // the group counter restarts; the error flag stays until skew_check reads it
        RT_CUDA(cudaMemsetAsync(s.sync.p + SYNC_WORK, 0, sizeof(int), ctx->stream));
        bool ok = false;
        if (n == 1) {
            ok = launch_fit<Real, MODE, 1>(ctx, h, mc, wc, CS);
        } else if (n <= 3 && ctx->sweepComponents == 1) {
            // the components side by side: one-component sweeps, one launch
            const int ncc = 32 - __builtin_clz(mc);
            ok = launch_fit<Real, MODE, 1>(ctx, h, mc, wc, CS, ncc);
        }
        if constexpr (MODE != 2) {
            if (!ok && n == 3) ok = launch_fit<Real, MODE, 3>(ctx, h, mc, wc, CS);
            else if (!ok && n == 6) {
                if constexpr (sizeof(Real) == 4) ok = launch_fit<Real, MODE, 6>(ctx, h, mc, wc, CS);
            }
        }
        if (ok) launch_count(ctx, 2);
        return ok;
    };
    auto singles = [&](int c0, int n) -> bool {
        bool ok = true;
        for (int c = c0; c < c0 + n && ok; ++c) ok = part(c, 1);
        return ok;
    };
    bool ok;
    if (MODE == 2 || nc == 1) ok = part(0, 1);
    else if (nc <= 3) ok = part(0, 3) || singles(0, nc);
    else ok = part(0, 6) || ((part(0, 3) || singles(0, 3)) && (part(3, 3) || singles(3, nc - 3)));
    RT_REQUIRE(ok, RT_EINVAL, "the systolic sweep does not fit one CTA's shared memory");
    RT_CHECK_LAUNCH();
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

void skew_precondition(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w, const unsigned *dmask) {
    SkewView g = ctx->mesh.sm.view();
    g.dmask = dmask;
    k_skew_gather<double, double><<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    if (nc == 1) autotune<double>(ctx, g, mask, w);
    launch_mode<double, 0>(ctx, g, nc, mask, w);
    launch_mode<double, 1>(ctx, g, nc, mask, w);
}

// 1/rD of the last skew_prepare, in cell order
__global__ void k_skew_rdinv_cells(SkewView g, double *__restrict__ rDc) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= g.nSkew) return;
    const int c = g.cellOf[e];
    if (c >= 0) rDc[c] = g.rDinv[e];
}

void skew_rdinv_cells(rt_ctx *ctx, double *rDc) {
    SkewView g = ctx->mesh.sm.view();
    k_skew_rdinv_cells<<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, rDc);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

void skew_prepare_T(rt_ctx *ctx, const double *upper, const double *lower) {
    StructMesh &s = ctx->mesh.sm;
    SkewView g = s.viewT();
    // the lower and upper coefficients exchanged: forward sweep rD_c a_fc,
    // backward rD_c a_cf (rDinv is rewritten with the same values)
    k_skew_premul<<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, s.faceLo.p, s.faceHi.p, ctx->mesh.N, lower,
                                                                  upper);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

void skew_precondition_T(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w) {
    SkewView g = ctx->mesh.sm.viewT();
    k_skew_gather<double, double><<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
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
    k_skew_gather<float, float><<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    if (nc == 1) autotune<float>(ctx, g, mask, w);
    launch_mode<float, 0>(ctx, g, nc, mask, w);
    launch_mode<float, 1>(ctx, g, nc, mask, w);
}

bool skew_fits(int nJB) {
    return nJB >= 1 && nJB <= 16 && sweep_smem_bytes<double, 2, 1, 4, 2>(nJB) <= kMaxSmem &&
           sweep_smem_bytes<double, 0, 1, 4, 2>(nJB) <= kMaxSmem && sweep_smem_bytes<double, 1, 1, 4, 2>(nJB) <= kMaxSmem;
}

void skew_precondition32d(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w, const unsigned *dmask) {
    SkewView32 g = ctx->mesh.sm.view32();
    g.w64 = w;
    g.dmask = dmask;
    k_skew_gather<float, double><<<nblocks(g.nSkew), RT_BLOCK, 0, ctx->stream>>>(g, mask, nc, r, ctx->mesh.N);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    if (nc == 1) autotune<float>(ctx, g, mask, (float *)nullptr);
    launch_mode<float, 0>(ctx, g, nc, mask, (float *)nullptr);
    launch_mode<float, 1>(ctx, g, nc, mask, (float *)nullptr);
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
