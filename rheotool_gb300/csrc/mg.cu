// mg.cu — an aggregation multigrid V-cycle as the preconditioner of the
// mixed form's pressure solve on structured meshes (RT_OPT_MIXED_PRECOND
// -2), in FP32.
//
// The pressure matrix of a structured mesh is a 7-point stencil on the
// box (nx x ny x nz, inactive box cells outside the mesh).  Level 0 holds
// its coefficients in box order: the diagonal and the couplings of every
// cell to its i-1, j-1 and k-1 neighbours (the matrix is symmetric, so the
// couplings to i+1, j+1, k+1 are the neighbours' own); a zero diagonal
// marks an inactive cell.  A coarse level aggregates 2 x 2 x 2 cells (a
// direction of one cell is not coarsened) with piecewise-constant
// prolongation, so its operator is the Galerkin product, again a 7-point
// stencil: the children's diagonals plus twice their couplings inside the
// aggregate, and the sums of their couplings across each aggregate face.
// Levels are added until the box has at most kCoarse cells; that last one
// is smoothed by one CTA.
//
// One application (a symmetric V-cycle from x = 0): on every level kNu
// red-black Gauss-Seidel sweeps (red then black), the residual restricted
// into the next level's right-hand side; on the coarsest level kCoarseSweeps
// symmetric sweeps; on the way up the correction prolongated (scaled by
// kOver, over-correction for the unsmoothed aggregation) and kNu sweeps in
// the reverse order (black then red).  kNu and kOver were chosen on the
// 1M-cell contraction: (1, 1.6) 331 pressure iterations, (2, 1.6) 185,
// (1, 1.9) 382, (2, 1.3) 162, (2, 1.0) 140, (3, 1.3) 108.  The smoother and its adjoint, and a
// constant scaling, keep the preconditioner symmetric, as PCG needs.  Every
// kernel is a plain pass over a level's box arrays: bandwidth-bound on the
// large levels, launch-bound on the small ones.
#include <algorithm>
#include <array>

#include "rt_internal.h"
#include "sweep.h"

namespace rt {

namespace {

constexpr int kCoarse = 512;        // cells of the level smoothed by one CTA
constexpr int kCoarseSweeps = 16;   // symmetric sweeps there
constexpr float kOver = 1.3f;       // coarse-correction scaling
constexpr int kNu = 3;              // red-black sweeps before and after the coarse correction

struct MgLev {
    int nx, ny, nz, n;
    float *dg, *cx, *cy, *cz, *x, *b;
};

__device__ __forceinline__ void box_ijk(const MgLev &L, int b, int &i, int &j, int &k) {
    i = b % L.nx;
    const int r = b / L.nx;
    j = r % L.ny;
    k = r / L.ny;
}

// sum over the six neighbours of a_nb x_nb
__device__ __forceinline__ float nb_sum(const MgLev &L, int b, int i, int j, int k, const float *__restrict__ x) {
    const int sy = L.nx, sz = L.nx * L.ny;
    float s = 0.0f;
    if (i > 0) s += L.cx[b] * x[b - 1];
    if (i + 1 < L.nx) s += L.cx[b + 1] * x[b + 1];
    if (j > 0) s += L.cy[b] * x[b - sy];
    if (j + 1 < L.ny) s += L.cy[b + sy] * x[b + sy];
    if (k > 0) s += L.cz[b] * x[b - sz];
    if (k + 1 < L.nz) s += L.cz[b + sz] * x[b + sz];
    return s;
}

// level 0 from the FP64 LDU matrix (box arrays zeroed before)
__global__ void k_mg_fine(int N, const int *__restrict__ boxOf, const int *__restrict__ faceLo,
                          const double *__restrict__ diag, const double *__restrict__ lower, MgLev L) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int b = boxOf[c];
    L.dg[b] = (float)diag[c];
    const int fz = faceLo[c], fy = faceLo[N + c], fx = faceLo[2 * N + c];
    L.cz[b] = fz >= 0 ? (float)lower[fz] : 0.0f;
    L.cy[b] = fy >= 0 ? (float)lower[fy] : 0.0f;
    L.cx[b] = fx >= 0 ? (float)lower[fx] : 0.0f;
}

// the Galerkin coarse operator of piecewise-constant aggregation
__global__ void k_mg_coarsen(MgLev F, MgLev C) {
    const int B = blockIdx.x * blockDim.x + threadIdx.x;
    if (B >= C.n) return;
    int I, J, K;
    box_ijk(C, B, I, J, K);
    const int fx = F.nx == C.nx ? 1 : 2, fy = F.ny == C.ny ? 1 : 2, fz = F.nz == C.nz ? 1 : 2;
    float dg = 0.0f, cx = 0.0f, cy = 0.0f, cz = 0.0f;
    for (int dk = 0; dk < fz; ++dk)
        for (int dj = 0; dj < fy; ++dj)
            for (int di = 0; di < fx; ++di) {
                const int i = I * fx + di, j = J * fy + dj, k = K * fz + dk;
                if (i >= F.nx || j >= F.ny || k >= F.nz) continue;
                const int b = i + F.nx * (j + F.ny * k);
                const float d = F.dg[b];
                if (d == 0.0f) continue;   // inactive
                dg += d;
                // a coupling to the lower neighbour inside the aggregate counts
                // twice in the diagonal (a_ij + a_ji), across it once in the face
                if (di == 1) dg += 2.0f * F.cx[b]; else cx += F.cx[b];
                if (dj == 1) dg += 2.0f * F.cy[b]; else cy += F.cy[b];
                if (dk == 1) dg += 2.0f * F.cz[b]; else cz += F.cz[b];
            }
    C.dg[B] = dg;
    C.cx[B] = I > 0 ? cx : 0.0f;
    C.cy[B] = J > 0 ? cy : 0.0f;
    C.cz[B] = K > 0 ? cz : 0.0f;
}

// level 0 from x = 0: the right-hand side from the FP64 residual (cell order),
// then the red half-sweep (x_red = b / dg; black x = 0)
__global__ void k_mg_first(MgLev L, const int *__restrict__ cellAt, const double *__restrict__ r, const unsigned *__restrict__ dm) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= L.n || (dm && !(*dm & 1u))) return;
    const int c = cellAt[b];
    const float rb = c >= 0 ? (float)r[c] : 0.0f;
    L.b[b] = rb;
    int i, j, k;
    box_ijk(L, b, i, j, k);
    const float d = L.dg[b];
    L.x[b] = (((i + j + k) & 1) == 0 && d != 0.0f) ? rb / d : 0.0f;
}

// one half-sweep of red-black Gauss-Seidel (colour 0: i + j + k even); with
// w set (level 0's last half-sweep) the updated x goes to w in cell order
__global__ void k_mg_smooth(MgLev L, int colour, const int *__restrict__ cellAt, double *__restrict__ w, const unsigned *__restrict__ dm) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= L.n || (dm && !(*dm & 1u))) return;
    int i, j, k;
    box_ijk(L, b, i, j, k);
    const float d = L.dg[b];
    float xv = L.x[b];
    if (((i + j + k) & 1) == colour && d != 0.0f) {
        xv = (L.b[b] - nb_sum(L, b, i, j, k, L.x)) / d;
        if (!w) L.x[b] = xv;
    }
    if (w) {
        const int c = cellAt[b];
        if (c >= 0) w[c] = (double)xv;
    }
}

// the residual b - A x of each aggregate's cells, summed into the coarse
// right-hand side; the coarse x starts at 0
__global__ void k_mg_restrict(MgLev F, MgLev C, const unsigned *__restrict__ dm) {
    const int B = blockIdx.x * blockDim.x + threadIdx.x;
    if (B >= C.n || (dm && !(*dm & 1u))) return;
    int I, J, K;
    box_ijk(C, B, I, J, K);
    const int fx = F.nx == C.nx ? 1 : 2, fy = F.ny == C.ny ? 1 : 2, fz = F.nz == C.nz ? 1 : 2;
    float s = 0.0f;
    for (int dk = 0; dk < fz; ++dk)
        for (int dj = 0; dj < fy; ++dj)
            for (int di = 0; di < fx; ++di) {
                const int i = I * fx + di, j = J * fy + dj, k = K * fz + dk;
                if (i >= F.nx || j >= F.ny || k >= F.nz) continue;
                const int b = i + F.nx * (j + F.ny * k);
                const float d = F.dg[b];
                if (d == 0.0f) continue;
                s += F.b[b] - d * F.x[b] - nb_sum(F, b, i, j, k, F.x);
            }
    C.b[B] = s;
    C.x[B] = 0.0f;
}

// x += kOver x_coarse(aggregate)
__global__ void k_mg_prolong(MgLev F, MgLev C, const unsigned *__restrict__ dm) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= F.n || (dm && !(*dm & 1u))) return;
    if (F.dg[b] == 0.0f) return;
    int i, j, k;
    box_ijk(F, b, i, j, k);
    const int I = F.nx == C.nx ? i : i / 2, J = F.ny == C.ny ? j : j / 2, K = F.nz == C.nz ? k : k / 2;
    F.x[b] += kOver * C.x[I + C.nx * (J + C.ny * K)];
}

// the coarsest level: symmetric Gauss-Seidel sweeps (red, black, black, red)
// from x = 0 by one CTA
__global__ void k_mg_coarsest(MgLev L, int sweeps, const unsigned *__restrict__ dm) {
    if (dm && !(*dm & 1u)) return;
    for (int b = threadIdx.x; b < L.n; b += blockDim.x) L.x[b] = 0.0f;
    __syncthreads();
    for (int s = 0; s < sweeps; ++s)
        for (int h = 0; h < 4; ++h) {
            const int colour = (h == 0 || h == 3) ? 0 : 1;
            for (int b = threadIdx.x; b < L.n; b += blockDim.x) {
                int i, j, k;
                box_ijk(L, b, i, j, k);
                const float d = L.dg[b];
                if (((i + j + k) & 1) == colour && d != 0.0f) L.x[b] = (L.b[b] - nb_sum(L, b, i, j, k, L.x)) / d;
            }
            __syncthreads();
        }
}

std::vector<MgLev> levels(rt_ctx *ctx) {
    StructMesh &s = ctx->mesh.sm;
    std::vector<MgLev> out;
    float *p = s.mgData.p;
    for (const auto &d : s.mgDims) {
        MgLev L{d[0], d[1], d[2], d[0] * d[1] * d[2], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
        float **a[] = {&L.dg, &L.cx, &L.cy, &L.cz, &L.x, &L.b};
        for (float **q : a) {
            *q = p;
            p += ((size_t)L.n + 31) / 32 * 32;
        }
        out.push_back(L);
    }
    return out;
}

}  // namespace

bool mg_available(rt_ctx *ctx) {
    const DevMesh &m = ctx->mesh;
    return m.sm.on && !m.hasCoupled && m.sm.boxOf.p != nullptr;
}

void mg_prepare(rt_ctx *ctx, const double *diag, const double *lower) {
    StructMesh &s = ctx->mesh.sm;
    const int N = ctx->mesh.N;
    if (s.mgDims.empty()) {   // the hierarchy's boxes, once per mesh
        int nx = s.nx, ny = s.ny, nz = s.nz;
        size_t total = 0;
        for (;;) {
            s.mgDims.push_back({nx, ny, nz});
            total += 6 * (((size_t)nx * ny * nz + 31) / 32 * 32);
            if ((long long)nx * ny * nz <= kCoarse || (nx == 1 && ny == 1 && nz == 1)) break;
            nx = (nx + 1) / 2;
            ny = (ny + 1) / 2;
            nz = (nz + 1) / 2;
        }
        s.mgData.alloc(total);
    }
    std::vector<MgLev> L = levels(ctx);
    RT_CUDA(cudaMemsetAsync(L[0].dg, 0, sizeof(float) * ((size_t)L[0].n + 31) / 32 * 32 * 4, ctx->stream));
    k_mg_fine<<<nblocks(N), RT_BLOCK, 0, ctx->stream>>>(N, s.boxOf.p, s.faceLo.p, diag, lower, L[0]);
    for (size_t l = 1; l < L.size(); ++l)
        k_mg_coarsen<<<nblocks(L[l].n), RT_BLOCK, 0, ctx->stream>>>(L[l - 1], L[l]);
    RT_CHECK_LAUNCH();
    launch_count(ctx, (int)L.size());
}

namespace {

// one V-cycle's launches on the stream; the number of kernels
int enqueue_vcycle(rt_ctx *ctx, const std::vector<MgLev> &L, const double *r, double *w, const unsigned *dm) {
    StructMesh &s = ctx->mesh.sm;
    cudaStream_t st = ctx->stream;
    const int nL = (int)L.size();
    int launches = 0;
    if (nL == 1) {   // a mesh no larger than the coarsest level
        k_mg_first<<<nblocks(L[0].n), RT_BLOCK, 0, st>>>(L[0], s.cellAt.p, r, dm);
        k_mg_coarsest<<<1, 1024, 0, st>>>(L[0], kCoarseSweeps, dm);
        k_mg_smooth<<<nblocks(L[0].n), RT_BLOCK, 0, st>>>(L[0], 1, s.cellAt.p, w, dm);
        RT_CHECK_LAUNCH();
        return 3;
    }
    // down: pre-smoothing (kNu sweeps, red then black) and restriction
    k_mg_first<<<nblocks(L[0].n), RT_BLOCK, 0, st>>>(L[0], s.cellAt.p, r, dm);
    ++launches;
    for (int l = 0; l + 1 < nL; ++l) {
        for (int nu = 0; nu < kNu; ++nu) {
            if (l > 0 || nu > 0) {
                k_mg_smooth<<<nblocks(L[l].n), RT_BLOCK, 0, st>>>(L[l], 0, nullptr, nullptr, dm);
                ++launches;
            }
            k_mg_smooth<<<nblocks(L[l].n), RT_BLOCK, 0, st>>>(L[l], 1, nullptr, nullptr, dm);
            ++launches;
        }
        k_mg_restrict<<<nblocks(L[l + 1].n), RT_BLOCK, 0, st>>>(L[l], L[l + 1], dm);
        ++launches;
    }
    k_mg_coarsest<<<1, 1024, 0, st>>>(L[nL - 1], kCoarseSweeps, dm);
    ++launches;
    // up: prolongation and post-smoothing (black, red); level 0's last half-sweep writes w
    for (int l = nL - 2; l >= 0; --l) {
        k_mg_prolong<<<nblocks(L[l].n), RT_BLOCK, 0, st>>>(L[l], L[l + 1], dm);
        ++launches;
        for (int nu = 0; nu < kNu; ++nu) {
            const bool last = l == 0 && nu == kNu - 1;
            k_mg_smooth<<<nblocks(L[l].n), RT_BLOCK, 0, st>>>(L[l], 1, nullptr, nullptr, dm);
            k_mg_smooth<<<nblocks(L[l].n), RT_BLOCK, 0, st>>>(L[l], 0, last ? s.cellAt.p : nullptr,
                                                              last ? w : nullptr, dm);
            launches += 2;
        }
    }
    RT_CHECK_LAUNCH();
    return launches;
}

}  // namespace

// The V-cycle's launches are captured once into a CUDA graph (per mesh and
// per r, w, dm buffers: a Krylov loop passes the same ones every iteration)
// and the graph is launched per application: most of the levels are small,
// and their launches, not their data, set the V-cycle's time.
void mg_apply(rt_ctx *ctx, const double *r, double *w, const unsigned *dm) {
    StructMesh &s = ctx->mesh.sm;
    MgGraph &gr = s.mgGraph;
    if (!gr.exec || gr.r != r || gr.w != w || gr.dm != dm) {
        gr.reset();
        std::vector<MgLev> L = levels(ctx);
        cudaGraph_t g = nullptr;
        RT_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int n = 0;
        try {
            n = enqueue_vcycle(ctx, L, r, w, dm);
        } catch (...) {
            cudaGraph_t dead = nullptr;
            cudaStreamEndCapture(ctx->stream, &dead);
            if (dead) cudaGraphDestroy(dead);
            throw;
        }
        RT_CUDA(cudaStreamEndCapture(ctx->stream, &g));
        cudaGraphExec_t exec = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        RT_CUDA(e);
        gr.exec = exec;
        gr.r = r;
        gr.w = w;
        gr.dm = dm;
        gr.launches = n;
    }
    RT_CUDA(cudaGraphLaunch(gr.exec, ctx->stream));
    launch_count(ctx, gr.launches);
}

}  // namespace rt
