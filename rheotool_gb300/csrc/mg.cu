// mg.cu — an aggregation multigrid V-cycle as the preconditioner of the
// mixed form's pressure solve (RT_OPT_MIXED_PRECOND -2) and momentum solve
// (RT_OPT_MIXED_PRECOND_U -2) on structured meshes, in FP32.
//
// The matrix of a structured mesh is a 7-point stencil on the box
// (nx x ny x nz, inactive box cells outside the mesh).  Level 0 holds its
// coefficients in box order: the diagonal and, for each of the i-1, j-1 and
// k-1 neighbours c' of a cell c, A[c][c'] (xl, yl, zl) and A[c'][c] (xu,
// yu, zu); a zero diagonal marks an inactive cell.  The symmetric pressure
// matrix keeps one copy (the u arrays alias the l arrays).  A coarse level
// aggregates 2 x 2 x 2 cells (a direction of one cell is not coarsened) with
// piecewise-constant prolongation P and restriction P^T, so its operator
// P^T A P is again a 7-point stencil: the children's diagonals plus both
// couplings of every child pair inside the aggregate, and the sums of the
// children's couplings across each aggregate face.  Levels are added until
// the box has at most kCoarse cells; that last one is smoothed by one CTA.
//
// One application (a V-cycle from x = 0): on every level kNu red-black
// Gauss-Seidel sweeps (red then black), the residual restricted into the
// next level's right-hand side; on the coarsest level kCoarseSweeps
// symmetric sweeps; on the way up the correction prolongated (scaled by
// kOver, over-correction for the unsmoothed aggregation) and kNu sweeps in
// the reverse order (black then red).  kNu and kOver were chosen on the
// 1M-cell contraction's pressure solve: (1, 1.6) 331 iterations, (2, 1.6)
// 185, (1, 1.9) 382, (2, 1.3) 162, (2, 1.0) 140, (3, 1.3) 108.  On a
// symmetric matrix the smoother and its adjoint, and a constant scaling,
// keep the preconditioner symmetric, as PCG needs; BiCGStab (the momentum
// solve) needs no symmetry, and the components of a vector solve go through
// one cycle together, sharing every coefficient load.  Every kernel is a
// plain pass over a level's box arrays: bandwidth-bound on the large
// levels, launch-bound on the small ones.
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
constexpr int kArrays = 13;         // arrays of a level: dg, xl, yl, zl, xu, yu, zu, x[3], b[3]
constexpr int kMaxLevels = 16;      // levels of a hierarchy, at most (a 2^16 box side)
constexpr int kTailCells = 4096;    // levels of at most this many box cells run in one CTA

struct MgLev {
    int nx, ny, nz, n;
    size_t np;   // the stride of the components' x and b
    float *dg, *xl, *yl, *zl, *xu, *yu, *zu, *x, *b;
};

__device__ __forceinline__ void box_ijk(const MgLev &L, int b, int &i, int &j, int &k) {
    i = b % L.nx;
    const int r = b / L.nx;
    j = r % L.ny;
    k = r / L.ny;
}

// the couplings of box cell b = (i, j, k) to its six neighbours
struct Nb6 {
    float c[6];
};

__device__ __forceinline__ Nb6 nb_coeffs(const MgLev &L, int b, int i, int j, int k) {
    const int sy = L.nx, sz = L.nx * L.ny;
    Nb6 a;
    a.c[0] = i > 0 ? L.xl[b] : 0.0f;
    a.c[1] = i + 1 < L.nx ? L.xu[b + 1] : 0.0f;
    a.c[2] = j > 0 ? L.yl[b] : 0.0f;
    a.c[3] = j + 1 < L.ny ? L.yu[b + sy] : 0.0f;
    a.c[4] = k > 0 ? L.zl[b] : 0.0f;
    a.c[5] = k + 1 < L.nz ? L.zu[b + sz] : 0.0f;
    return a;
}

// sum over the six neighbours of a_nb x_nb (x: one component's array)
__device__ __forceinline__ float nb_sum(const MgLev &L, const Nb6 &a, int b, int i, int j, int k,
                                        const float *__restrict__ x) {
    const int sy = L.nx, sz = L.nx * L.ny;
    float s = 0.0f;
    if (i > 0) s += a.c[0] * x[b - 1];
    if (i + 1 < L.nx) s += a.c[1] * x[b + 1];
    if (j > 0) s += a.c[2] * x[b - sy];
    if (j + 1 < L.ny) s += a.c[3] * x[b + sy];
    if (k > 0) s += a.c[4] * x[b - sz];
    if (k + 1 < L.nz) s += a.c[5] * x[b + sz];
    return s;
}

__device__ __forceinline__ bool skip(const unsigned *dm) { return dm && !(*dm & 1u); }

// level 0 from the FP64 LDU matrix (box arrays zeroed before): the face to
// the lower neighbour c' of cell c carries A[c][c'] = lower, A[c'][c] = upper
__global__ void k_mg_fine(int N, const int *__restrict__ boxOf, const int *__restrict__ faceLo,
                          const double *__restrict__ diag, const double *__restrict__ upper,
                          const double *__restrict__ lower, MgLev L, int sym) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int b = boxOf[c];
    L.dg[b] = (float)diag[c];
    const int fz = faceLo[c], fy = faceLo[N + c], fx = faceLo[2 * N + c];
    L.zl[b] = fz >= 0 ? (float)lower[fz] : 0.0f;
    L.yl[b] = fy >= 0 ? (float)lower[fy] : 0.0f;
    L.xl[b] = fx >= 0 ? (float)lower[fx] : 0.0f;
    if (!sym) {
        L.zu[b] = fz >= 0 ? (float)upper[fz] : 0.0f;
        L.yu[b] = fy >= 0 ? (float)upper[fy] : 0.0f;
        L.xu[b] = fx >= 0 ? (float)upper[fx] : 0.0f;
    }
}

// the Galerkin coarse operator of piecewise-constant aggregation
__global__ void k_mg_coarsen(MgLev F, MgLev C, int sym) {
    const int B = blockIdx.x * blockDim.x + threadIdx.x;
    if (B >= C.n) return;
    int I, J, K;
    box_ijk(C, B, I, J, K);
    const int fx = F.nx == C.nx ? 1 : 2, fy = F.ny == C.ny ? 1 : 2, fz = F.nz == C.nz ? 1 : 2;
    float dg = 0.0f, xl = 0.0f, yl = 0.0f, zl = 0.0f, xu = 0.0f, yu = 0.0f, zu = 0.0f;
    for (int dk = 0; dk < fz; ++dk)
        for (int dj = 0; dj < fy; ++dj)
            for (int di = 0; di < fx; ++di) {
                const int i = I * fx + di, j = J * fy + dj, k = K * fz + dk;
                if (i >= F.nx || j >= F.ny || k >= F.nz) continue;
                const int b = i + F.nx * (j + F.ny * k);
                const float d = F.dg[b];
                if (d == 0.0f) continue;   // inactive
                dg += d;
                // a coupling pair to the lower neighbour inside the aggregate
                // adds both directions to the diagonal (a_ij + a_ji), one
                // across it adds to the coarse couplings
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
                if (dk == 1) {
                    dg += F.zl[b] + F.zu[b];
                } else {
                    zl += F.zl[b];
                    zu += F.zu[b];
                }
            }
    C.dg[B] = dg;
    C.xl[B] = I > 0 ? xl : 0.0f;
    C.yl[B] = J > 0 ? yl : 0.0f;
    C.zl[B] = K > 0 ? zl : 0.0f;
    if (!sym) {
        C.xu[B] = I > 0 ? xu : 0.0f;
        C.yu[B] = J > 0 ? yu : 0.0f;
        C.zu[B] = K > 0 ? zu : 0.0f;
    }
}

// level 0 from x = 0: the right-hand side from the residual (cell order,
// component k at k N), then the red half-sweep (x_red = b / dg; black x = 0)
template <class T>
__global__ void k_mg_first(MgLev L, const int *__restrict__ cellAt, int N, unsigned m, const T *__restrict__ r,
                           const unsigned *__restrict__ dm) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= L.n || skip(dm)) return;
    const int c = cellAt[b];
    int i, j, k;
    box_ijk(L, b, i, j, k);
    const float d = L.dg[b];
    const bool red = ((i + j + k) & 1) == 0 && d != 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q)
        if ((m >> q) & 1u) {
            const float rb = c >= 0 ? (float)r[(size_t)q * N + c] : 0.0f;
            L.b[q * L.np + b] = rb;
            L.x[q * L.np + b] = red ? rb / d : 0.0f;
        }
}

// one half-sweep of red-black Gauss-Seidel (colour 0: i + j + k even); with
// w set (level 0's last half-sweep) the updated x goes to w in cell order
template <class T>
__global__ void k_mg_smooth(MgLev L, int colour, unsigned m, const int *__restrict__ cellAt, int N,
                            T *__restrict__ w, const unsigned *__restrict__ dm) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= L.n || skip(dm)) return;
    int i, j, k;
    box_ijk(L, b, i, j, k);
    const float d = L.dg[b];
    const bool mine = ((i + j + k) & 1) == colour && d != 0.0f;
    const int c = w ? cellAt[b] : -1;
    if (!mine && c < 0) return;
    Nb6 a;
    if (mine) a = nb_coeffs(L, b, i, j, k);
#pragma unroll
    for (int q = 0; q < 3; ++q)
        if ((m >> q) & 1u) {
            float *x = L.x + q * L.np;
            float xv = x[b];
            if (mine) {
                xv = (L.b[q * L.np + b] - nb_sum(L, a, b, i, j, k, x)) / d;
                if (!w) x[b] = xv;
            }
            if (c >= 0) w[(size_t)q * N + c] = (T)xv;
        }
}

// the same half-sweep without w, one thread per cell of the colour (row
// (j, k) holds them at i = (colour + j + k) % 2, +2, ...): the t-th cell
__device__ __forceinline__ void smooth_cell(const MgLev &L, int colour, unsigned m, int t) {
    const int hx = (L.nx + 1) >> 1;
    const int row = t / hx;
    const int j = row % L.ny, k = row / L.ny;
    const int i = 2 * (t - row * hx) + ((colour + j + k) & 1);
    if (i >= L.nx) return;
    const int b = i + L.nx * row;
    const float d = L.dg[b];
    if (d == 0.0f) return;
    const Nb6 a = nb_coeffs(L, b, i, j, k);
#pragma unroll
    for (int q = 0; q < 3; ++q)
        if ((m >> q) & 1u) {
            float *x = L.x + q * L.np;
            x[b] = (L.b[q * L.np + b] - nb_sum(L, a, b, i, j, k, x)) / d;
        }
}

// the threads of a one-colour half-sweep of a level
__host__ __device__ __forceinline__ int colour_cells(const MgLev &L) { return (L.nx + 1) / 2 * L.ny * L.nz; }

__global__ void k_mg_smooth_colour(MgLev L, int colour, unsigned m, const unsigned *__restrict__ dm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= colour_cells(L) || skip(dm)) return;
    smooth_cell(L, colour, m, t);
}

// the residual b - A x of each aggregate's cells, summed into the coarse
// right-hand side; the coarse x starts at 0 (coarse cell B)
__device__ __forceinline__ void restrict_cell(const MgLev &F, const MgLev &C, unsigned m, int B) {
    int I, J, K;
    box_ijk(C, B, I, J, K);
    const int fx = F.nx == C.nx ? 1 : 2, fy = F.ny == C.ny ? 1 : 2, fz = F.nz == C.nz ? 1 : 2;
    float s[3] = {0.0f, 0.0f, 0.0f};
    for (int dk = 0; dk < fz; ++dk)
        for (int dj = 0; dj < fy; ++dj)
            for (int di = 0; di < fx; ++di) {
                const int i = I * fx + di, j = J * fy + dj, k = K * fz + dk;
                if (i >= F.nx || j >= F.ny || k >= F.nz) continue;
                const int b = i + F.nx * (j + F.ny * k);
                const float d = F.dg[b];
                if (d == 0.0f) continue;
                const Nb6 a = nb_coeffs(F, b, i, j, k);
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    if ((m >> q) & 1u) {
                        const float *x = F.x + q * F.np;
                        s[q] += F.b[q * F.np + b] - d * x[b] - nb_sum(F, a, b, i, j, k, x);
                    }
            }
#pragma unroll
    for (int q = 0; q < 3; ++q)
        if ((m >> q) & 1u) {
            C.b[q * C.np + B] = s[q];
            C.x[q * C.np + B] = 0.0f;
        }
}

__global__ void k_mg_restrict(MgLev F, MgLev C, unsigned m, const unsigned *__restrict__ dm) {
    const int B = blockIdx.x * blockDim.x + threadIdx.x;
    if (B >= C.n || skip(dm)) return;
    restrict_cell(F, C, m, B);
}

// x += kOver x_coarse(aggregate) (fine cell b)
__device__ __forceinline__ void prolong_cell(const MgLev &F, const MgLev &C, unsigned m, int b) {
    if (F.dg[b] == 0.0f) return;
    int i, j, k;
    box_ijk(F, b, i, j, k);
    const int I = F.nx == C.nx ? i : i / 2, J = F.ny == C.ny ? j : j / 2, K = F.nz == C.nz ? k : k / 2;
    const int B = I + C.nx * (J + C.ny * K);
#pragma unroll
    for (int q = 0; q < 3; ++q)
        if ((m >> q) & 1u) F.x[q * F.np + b] += kOver * C.x[q * C.np + B];
}

__global__ void k_mg_prolong(MgLev F, MgLev C, unsigned m, const unsigned *__restrict__ dm) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= F.n || skip(dm)) return;
    prolong_cell(F, C, m, b);
}

// the coarsest level: symmetric Gauss-Seidel sweeps (red, black, black, red)
// from x = 0 by the calling CTA
__device__ void coarsest_cta(const MgLev &L, int sweeps, unsigned m) {
    for (int b = threadIdx.x; b < L.n; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            if ((m >> q) & 1u) L.x[q * L.np + b] = 0.0f;
    __syncthreads();
    for (int s = 0; s < sweeps; ++s)
        for (int h = 0; h < 4; ++h) {
            const int colour = (h == 0 || h == 3) ? 0 : 1;
            for (int b = threadIdx.x; b < L.n; b += blockDim.x) {
                int i, j, k;
                box_ijk(L, b, i, j, k);
                const float d = L.dg[b];
                if (((i + j + k) & 1) != colour || d == 0.0f) continue;
                const Nb6 a = nb_coeffs(L, b, i, j, k);
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    if ((m >> q) & 1u) {
                        float *x = L.x + q * L.np;
                        x[b] = (L.b[q * L.np + b] - nb_sum(L, a, b, i, j, k, x)) / d;
                    }
            }
            __syncthreads();
        }
}

__global__ void k_mg_coarsest(MgLev L, int sweeps, unsigned m, const unsigned *__restrict__ dm) {
    if (skip(dm)) return;
    coarsest_cta(L, sweeps, m);
}

// The small levels' part of the V-cycle in one CTA: from the right-hand side
// restricted onto level `first` down to the coarsest level and back up to the
// corrected, post-smoothed x of level `first` (the same passes and
// arithmetic as the per-level launches, a barrier between passes), so that
// those levels cost no launches.
struct MgTail {
    MgLev lev[kMaxLevels];
    int first, n;   // levels first .. n - 1
};

__global__ void __launch_bounds__(1024, 1) k_mg_tail(MgTail T, int sweeps, unsigned m,
                                                    const unsigned *__restrict__ dm) {
    if (skip(dm)) return;
    auto smooth = [&](const MgLev &L, int colour) {
        const int nc = colour_cells(L);
        for (int t = threadIdx.x; t < nc; t += blockDim.x) smooth_cell(L, colour, m, t);
        __syncthreads();
    };
    for (int l = T.first; l + 1 < T.n; ++l) {
        const MgLev &F = T.lev[l], &C = T.lev[l + 1];
        for (int nu = 0; nu < kNu; ++nu) {
            smooth(F, 0);
            smooth(F, 1);
        }
        for (int B = threadIdx.x; B < C.n; B += blockDim.x) restrict_cell(F, C, m, B);
        __syncthreads();
    }
    coarsest_cta(T.lev[T.n - 1], sweeps, m);
    for (int l = T.n - 2; l >= T.first; --l) {
        const MgLev &F = T.lev[l], &C = T.lev[l + 1];
        for (int b = threadIdx.x; b < F.n; b += blockDim.x) prolong_cell(F, C, m, b);
        __syncthreads();
        for (int nu = 0; nu < kNu; ++nu) {
            smooth(F, 1);
            smooth(F, 0);
        }
    }
}

std::vector<MgLev> levels(rt_ctx *ctx, bool sym) {
    StructMesh &s = ctx->mesh.sm;
    std::vector<MgLev> out;
    float *p = s.mgData.p;
    for (const auto &d : s.mgDims) {
        MgLev L{};
        L.nx = d[0];
        L.ny = d[1];
        L.nz = d[2];
        L.n = d[0] * d[1] * d[2];
        L.np = ((size_t)L.n + 31) / 32 * 32;
        float *q = p;
        L.dg = q;
        L.xl = q + L.np;
        L.yl = q + 2 * L.np;
        L.zl = q + 3 * L.np;
        L.xu = sym ? L.xl : q + 4 * L.np;
        L.yu = sym ? L.yl : q + 5 * L.np;
        L.zu = sym ? L.zl : q + 6 * L.np;
        L.x = q + 7 * L.np;
        L.b = q + 10 * L.np;
        p += kArrays * L.np;
        out.push_back(L);
    }
    return out;
}

}  // namespace

bool mg_available(rt_ctx *ctx) {
    const DevMesh &m = ctx->mesh;
    return m.sm.on && !m.hasCoupled && m.sm.boxOf.p != nullptr;
}

void mg_prepare(rt_ctx *ctx, const double *diag, const double *upper, const double *lower, bool sym) {
    StructMesh &s = ctx->mesh.sm;
    const int N = ctx->mesh.N;
    if (s.mgDims.empty()) {   // the hierarchy's boxes, once per mesh
        int nx = s.nx, ny = s.ny, nz = s.nz;
        size_t total = 0;
        for (;;) {
            s.mgDims.push_back({nx, ny, nz});
            total += kArrays * (((size_t)nx * ny * nz + 31) / 32 * 32);
            if ((long long)nx * ny * nz <= kCoarse || (nx == 1 && ny == 1 && nz == 1)) break;
            RT_REQUIRE((int)s.mgDims.size() < kMaxLevels, RT_EINVAL, "multigrid: too many levels");
            nx = (nx + 1) / 2;
            ny = (ny + 1) / 2;
            nz = (nz + 1) / 2;
        }
        s.mgData.alloc(total);
    }
    std::vector<MgLev> L = levels(ctx, sym);
    RT_CUDA(cudaMemsetAsync(L[0].dg, 0, sizeof(float) * L[0].np * 7, ctx->stream));
    k_mg_fine<<<nblocks(N), RT_BLOCK, 0, ctx->stream>>>(N, s.boxOf.p, s.faceLo.p, diag, upper, lower, L[0],
                                                       sym ? 1 : 0);
    for (size_t l = 1; l < L.size(); ++l)
        k_mg_coarsen<<<nblocks(L[l].n), RT_BLOCK, 0, ctx->stream>>>(L[l - 1], L[l], sym ? 1 : 0);
    RT_CHECK_LAUNCH();
    launch_count(ctx, (int)L.size());
}

namespace {

// the first level the one-CTA tail takes (at least 1: level 0's first and
// last passes read r and write w in cell order), or the level count for none
int tail_first(const std::vector<MgLev> &L) {
    const int nL = (int)L.size();
    for (int l = 1; l < nL; ++l)
        if (L[l].n <= kTailCells) return l;
    return nL;
}

// one V-cycle's launches on the stream; the number of kernels
template <class T>
int enqueue_vcycle(rt_ctx *ctx, const std::vector<MgLev> &L, unsigned m, const T *r, T *w, const unsigned *dm) {
    StructMesh &s = ctx->mesh.sm;
    cudaStream_t st = ctx->stream;
    const int N = ctx->mesh.N;
    const int nL = (int)L.size();
    int launches = 0;
    if (nL == 1) {   // a mesh no larger than the coarsest level
        k_mg_first<T><<<nblocks(L[0].n), RT_BLOCK, 0, st>>>(L[0], s.cellAt.p, N, m, r, dm);
        k_mg_coarsest<<<1, 1024, 0, st>>>(L[0], kCoarseSweeps, m, dm);
        k_mg_smooth<T><<<nblocks(L[0].n), RT_BLOCK, 0, st>>>(L[0], 1, m, s.cellAt.p, N, w, dm);
        RT_CHECK_LAUNCH();
        return 3;
    }
    // levels tf .. nL - 1 in one CTA (tf == nL: none)
    const int tf = tail_first(L);
    // down: pre-smoothing (kNu sweeps, red then black) and restriction
    k_mg_first<T><<<nblocks(L[0].n), RT_BLOCK, 0, st>>>(L[0], s.cellAt.p, N, m, r, dm);
    ++launches;
    for (int l = 0; l + 1 < nL && l < tf; ++l) {
        for (int nu = 0; nu < kNu; ++nu) {
            if (l > 0 || nu > 0) {
                k_mg_smooth_colour<<<nblocks(colour_cells(L[l])), RT_BLOCK, 0, st>>>(L[l], 0, m, dm);
                ++launches;
            }
            k_mg_smooth_colour<<<nblocks(colour_cells(L[l])), RT_BLOCK, 0, st>>>(L[l], 1, m, dm);
            ++launches;
        }
        k_mg_restrict<<<nblocks(L[l + 1].n), RT_BLOCK, 0, st>>>(L[l], L[l + 1], m, dm);
        ++launches;
    }
    if (tf < nL) {
        MgTail tail{};
        for (int l = 0; l < nL; ++l) tail.lev[l] = L[l];
        tail.first = tf;
        tail.n = nL;
        k_mg_tail<<<1, 1024, 0, st>>>(tail, kCoarseSweeps, m, dm);
    } else {
        k_mg_coarsest<<<1, 1024, 0, st>>>(L[nL - 1], kCoarseSweeps, m, dm);
    }
    ++launches;
    // up: prolongation and post-smoothing (black, red); level 0's last half-sweep writes w
    // (from the level the tail, or the coarsest level's sweeps, left corrected)
    const int top = tf < nL ? tf : nL - 1;
    for (int l = top - 1; l >= 0; --l) {
        k_mg_prolong<<<nblocks(L[l].n), RT_BLOCK, 0, st>>>(L[l], L[l + 1], m, dm);
        ++launches;
        for (int nu = 0; nu < kNu; ++nu) {
            const bool last = l == 0 && nu == kNu - 1;
            k_mg_smooth_colour<<<nblocks(colour_cells(L[l])), RT_BLOCK, 0, st>>>(L[l], 1, m, dm);
            if (last)   // level 0's last half-sweep writes every cell's x to w
                k_mg_smooth<T><<<nblocks(L[l].n), RT_BLOCK, 0, st>>>(L[l], 0, m, s.cellAt.p, N, w, dm);
            else
                k_mg_smooth_colour<<<nblocks(colour_cells(L[l])), RT_BLOCK, 0, st>>>(L[l], 0, m, dm);
            launches += 2;
        }
    }
    RT_CHECK_LAUNCH();
    return launches;
}

// The V-cycle's launches are captured once into a CUDA graph (per mesh,
// matrix kind and r, w, dm buffers and components: a Krylov loop passes the
// same few every iteration) and the graph is launched per application: most
// of the levels are small, and their launches, not their data, set the
// V-cycle's time.
template <class T>
void apply(rt_ctx *ctx, bool sym, unsigned m, const T *r, T *w, const unsigned *dm) {
    StructMesh &s = ctx->mesh.sm;
    MgGraph *gr = nullptr;
    for (MgGraph &g : s.mgGraph)
        if (g.exec && g.r == r && g.w == w && g.dm == dm && g.mask == m && g.sym == sym) gr = &g;
    if (!gr) {
        gr = &s.mgGraph[s.mgNext];
        s.mgNext = (s.mgNext + 1) % kMgGraphs;
        gr->reset();
        std::vector<MgLev> L = levels(ctx, sym);
        cudaGraph_t g = nullptr;
        RT_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int n = 0;
        try {
            n = enqueue_vcycle<T>(ctx, L, m, r, w, dm);
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
        gr->exec = exec;
        gr->r = r;
        gr->w = w;
        gr->dm = dm;
        gr->mask = m;
        gr->sym = sym;
        gr->launches = n;
    }
    RT_CUDA(cudaGraphLaunch(gr->exec, ctx->stream));
    launch_count(ctx, gr->launches);
}

}  // namespace

void mg_apply(rt_ctx *ctx, const double *r, double *w, const unsigned *dm) {
    apply<double>(ctx, true, 1u, r, w, dm);
}

void mg_apply32(rt_ctx *ctx, unsigned mask, const float *r, float *w) {
    apply<float>(ctx, false, mask, r, w, nullptr);
}

}  // namespace rt
