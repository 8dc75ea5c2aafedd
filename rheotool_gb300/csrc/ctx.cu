// ctx.cu — C-ABI entry points: context, mesh upload, case setup, field I/O.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "constitutive_cell.cuh"
#include "rt_internal.h"
#include "sweep.h"

using namespace rt;

namespace {

__global__ void k_aos2soa(int n, int nc, const double *__restrict__ in, double *__restrict__ out) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * nc) return;
    int i = (int)(t / nc), k = (int)(t % nc);
    out[(long long)k * n + i] = in[t];
}

__global__ void k_soa2aos(int n, int nc, const double *__restrict__ in, double *__restrict__ out) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * nc) return;
    int i = (int)(t / nc), k = (int)(t % nc);
    out[t] = in[(long long)k * n + i];
}

template <class F>
rt_status guarded(rt_ctx *ctx, F &&f) {
    if (!ctx) return RT_EINVAL;
    try {
        return f();
    } catch (const Error &e) {
        ctx->lastError = e.msg;
        return e.status;
    } catch (const std::exception &e) {
        ctx->lastError = e.what();
        return RT_EINVAL;
    }
}

// host AoS (n x nc) -> device SoA, through a staging buffer
void upload_soa(rt_ctx *ctx, const double *h, int n, int nc, DBuf<double> &dst) {
    dst.alloc((size_t)n * nc);
    if (n == 0) return;
    if (nc == 1) {
        RT_CUDA(cudaMemcpyAsync(dst.p, h, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        return;
    }
    size_t cnt = (size_t)n * nc;
    if (ctx->stage.n < cnt) ctx->stage.alloc(cnt);
    RT_CUDA(cudaMemcpyAsync(ctx->stage.p, h, sizeof(double) * cnt, cudaMemcpyHostToDevice, ctx->stream));
    k_aos2soa<<<nblocks((long long)cnt), RT_BLOCK, 0, ctx->stream>>>(n, nc, ctx->stage.p, dst.p);
    RT_CHECK_LAUNCH();
}

void download_aos(rt_ctx *ctx, const DBuf<double> &src, int n, int nc, double *h) {
    if (n == 0) return;
    if (nc == 1) {
        RT_CUDA(cudaMemcpyAsync(h, src.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        return;
    }
    size_t cnt = (size_t)n * nc;
    if (ctx->stage.n < cnt) ctx->stage.alloc(cnt);
    k_soa2aos<<<nblocks((long long)cnt), RT_BLOCK, 0, ctx->stream>>>(n, nc, src.p, ctx->stage.p);
    RT_CHECK_LAUNCH();
    RT_CUDA(cudaMemcpyAsync(h, ctx->stage.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, ctx->stream));
    RT_CUDA(cudaStreamSynchronize(ctx->stream));
}

template <class T>
void upload_vec(rt_ctx *ctx, const std::vector<T> &v, DBuf<T> &d) {
    d.upload(v.data(), v.size(), ctx->stream);
}

std::vector<double> aos_to_soa_host(const double *a, int n, int nc) {
    std::vector<double> o((size_t)n * nc);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < nc; ++k) o[(size_t)k * n + i] = a[(size_t)i * nc + k];
    return o;
}

// the parameter checks of one constitutive model (each mode of a multiMode one)
void validate_model(const rt_model_params *mp) {
    RT_REQUIRE(mp->model >= RT_MODEL_OLDROYDB_LOG && mp->model <= RT_MODEL_WHITEMETZNERCY_LOG, RT_EINVAL,
               "unknown constitutive model");
    RT_REQUIRE(mp->model != RT_MODEL_XPOMPOM_LOG || (mp->lambdaS > 0 && mp->q > 0), RT_EINVAL,
               "XPomPom needs lambdaS > 0 and q > 0");
    RT_REQUIRE(mp->model != RT_MODEL_WHITEMETZNERCY_LOG || mp->a > 0, RT_EINVAL, "WhiteMetznerCY needs a > 0");
    const bool pttGen = mp->model == RT_MODEL_PTT_LOG && mp->pttFunction == RT_PTT_GENERALIZED;
    RT_REQUIRE(mp->model != RT_MODEL_PTT_LOG || (mp->pttFunction >= RT_PTT_LINEAR &&
                                                 mp->pttFunction <= RT_PTT_GENERALIZED),
               RT_EINVAL, "unknown PTT destruction function");
    // PTTLog.C:147-152
    RT_REQUIRE(!pttGen || (mp->alpha > 0 && mp->beta > 0), RT_EINVAL,
               "Both alpha and beta should be positive values for the Mittag-Leffler function to converge.");
    RT_REQUIRE(!pttGen || mp->maxIterMittagLeffler >= 1, RT_EINVAL, "maxIterMittagLeffler must be positive");
    RT_REQUIRE(mp->lambda > 0 && mp->rho > 0, RT_EINVAL, "lambda and rho must be positive");
    RT_REQUIRE(mp->model != RT_MODEL_ROLIEPOLY_LOG || mp->lambdaR > 0, RT_EINVAL, "Rolie-Poly needs lambdaR > 0");
    RT_REQUIRE((mp->model != RT_MODEL_FENEP_LOG && mp->model != RT_MODEL_FENECR_LOG) || mp->L2 > 3.0, RT_EINVAL,
               "FENE-P and FENE-CR need L2 > 3");
}

}  // namespace

namespace rt {
void launch_count(rt_ctx *ctx, int n) { ctx->kernelLaunches += n; }
}  // namespace rt

extern "C" {

const char *rt_status_string(rt_status s) {
    switch (s) {
    case RT_OK: return "RT_OK";
    case RT_EINVAL: return "RT_EINVAL";
    case RT_ENOCONV: return "RT_ENOCONV";
    case RT_ENAN: return "RT_ENAN";
    case RT_ETIMEOUT: return "RT_ETIMEOUT";
    case RT_EOOM: return "RT_EOOM";
    case RT_ECUDA: return "RT_ECUDA";
    case RT_ENOTREADY: return "RT_ENOTREADY";
    default: return "unknown";
    }
}

rt_status rt_ctx_create(rt_ctx **out, int32_t device) {
    if (!out) return RT_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return RT_ECUDA;
    if (device < 0 || device >= n) return RT_EINVAL;
    rt_ctx *ctx = new rt_ctx();
    ctx->device = device;
    rt_status s = guarded(ctx, [&]() -> rt_status {
        RT_CUDA(cudaSetDevice(device));
        RT_CUDA(cudaDeviceGetAttribute(&ctx->numSMs, cudaDevAttrMultiProcessorCount, device));
        RT_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        reduce_init(ctx);
        return RT_OK;
    });
    if (s != RT_OK) {
        delete ctx;
        return s;
    }
    *out = ctx;
    return RT_OK;
}

rt_status rt_ctx_destroy(rt_ctx *ctx) {
    if (!ctx) return RT_EINVAL;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->red.hostResult) cudaFreeHost(ctx->red.hostResult);
    if (ctx->red.hostFlag) cudaFreeHost((void *)ctx->red.hostFlag);
    for (cudaEvent_t e : ctx->red.poll)
        if (e) cudaEventDestroy(e);
    if (ctx->mesh.batch.hostCount) cudaFreeHost(ctx->mesh.batch.hostCount);
    for (cudaEvent_t e : ctx->prof.pool) cudaEventDestroy(e);
    if (ctx->tStart) cudaEventDestroy(ctx->tStart);
    if (ctx->tStop) cudaEventDestroy(ctx->tStop);
    cudaStream_t st = ctx->stream;
    delete ctx;   // DBuf destructors free device memory
    if (st) cudaStreamDestroy(st);
    return RT_OK;
}

const char *rt_last_error(const rt_ctx *ctx) { return ctx ? ctx->lastError.c_str() : "null context"; }

rt_status rt_sync(rt_ctx *ctx) {
    return guarded(ctx, [&]() -> rt_status {
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        return RT_OK;
    });
}

rt_status rt_mesh_upload(rt_ctx *ctx, const rt_mesh_desc *md) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(md && md->nCells > 0 && md->nFaces >= 0 && md->nBFaces >= 0 && md->nPatches >= 0,
                   RT_EINVAL, "bad mesh sizes");
        RT_CUDA(cudaSetDevice(ctx->device));
        const int N = md->nCells, F = md->nFaces, NB = md->nBFaces;
        // ---- validate addressing -------------------------------------------
        for (int f = 0; f < F; ++f) {
            int o = md->owner[f], n = md->neighbour[f];
            RT_REQUIRE(o >= 0 && n < N && o < n, RT_EINVAL, "face " + std::to_string(f) + ": need 0 <= owner < neighbour < nCells");
            if (f > 0) {
                int po = md->owner[f - 1], pn = md->neighbour[f - 1];
                RT_REQUIRE(po < o || (po == o && pn < n), RT_EINVAL, "faces are not in upper-triangular order");
            }
        }
        for (int b = 0; b < NB; ++b)
            RT_REQUIRE(md->bCell[b] >= 0 && md->bCell[b] < N, RT_EINVAL, "bad boundary face cell");
        int acc = 0;
        for (int p = 0; p < md->nPatches; ++p) {
            RT_REQUIRE(md->patchStart[p] == acc && md->patchSize[p] >= 0, RT_EINVAL, "patches must tile the boundary faces in order");
            acc += md->patchSize[p];
        }
        RT_REQUIRE(acc == NB, RT_EINVAL, "patch sizes do not add up to nBFaces");

        DevMesh &m = ctx->mesh;
        m.sm.on = false;
        m.colour.release();
        m.nRed = 0;
        m.N = N; m.F = F; m.NB = NB; m.nPatches = md->nPatches;
        for (int k = 0; k < 3; ++k) m.solveDir[k] = md->solveDir[k];
        cudaStream_t s = ctx->stream;
        m.owner.upload(md->owner, F, s);
        m.neighbour.upload(md->neighbour, F, s);
        upload_vec(ctx, aos_to_soa_host(md->Sf, F, 3), m.Sf);
        m.magSf.upload(md->magSf, F, s);
        m.w.upload(md->weights, F, s);
        m.deltaCoeffs.upload(md->deltaCoeffs, F, s);
        upload_vec(ctx, aos_to_soa_host(md->C, N, 3), m.C);
        {
            // face delta vectors C_N - C_P (given, for cyclic faces)
            std::vector<double> dv((size_t)3 * F);
            for (int f = 0; f < F; ++f)
                for (int d = 0; d < 3; ++d)
                    dv[(size_t)d * F + f] = md->delta ? md->delta[3 * f + d]
                                                      : md->C[3 * md->neighbour[f] + d] - md->C[3 * md->owner[f] + d];
            upload_vec(ctx, dv, m.d);
        }
        m.coupledH.assign(F, 0);
        m.hasCoupled = false;
        if (md->coupled)
            for (int f = 0; f < F; ++f)
                if (md->coupled[f]) { m.coupledH[f] = 1; m.hasCoupled = true; }
        m.V.upload(md->V, N, s);
        m.bCell.upload(md->bCell, NB, s);
        upload_vec(ctx, aos_to_soa_host(md->bSf, NB, 3), m.bSf);
        m.bmagSf.upload(md->bmagSf, NB, s);
        m.bDelta.upload(md->bDeltaCoeffs, NB, s);
        {
            std::vector<double> ctf((size_t)3 * NB);
            for (int b = 0; b < NB; ++b)
                for (int d = 0; d < 3; ++d)
                    ctf[(size_t)d * NB + b] = md->bCf[3 * b + d] - md->C[3 * md->bCell[b] + d];
            upload_vec(ctx, ctf, m.bCtoF);
        }
        m.patchStartH.assign(md->patchStart, md->patchStart + md->nPatches);
        m.patchSizeH.assign(md->patchSize, md->patchSize + md->nPatches);
        {
            std::vector<int> bp(NB);
            for (int p = 0; p < md->nPatches; ++p)
                for (int i = 0; i < md->patchSize[p]; ++i) bp[md->patchStart[p] + i] = p;
            upload_vec(ctx, bp, m.bPatch);
        }
        // ---- ELL adjacency in face order ---------------------------------
        std::vector<int> cnt(N, 0);
        for (int f = 0; f < F; ++f) { cnt[md->owner[f]]++; cnt[md->neighbour[f]]++; }
        int ns = 0;
        for (int c = 0; c < N; ++c) ns = std::max(ns, cnt[c]);
        m.nSlots = ns;
        std::vector<int> ef((size_t)std::max(ns, 1) * N, -1), en((size_t)std::max(ns, 1) * N, -1);
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int f = 0; f < F; ++f) {
            int o = md->owner[f], n = md->neighbour[f];
            ef[(size_t)cnt[o] * N + o] = f; en[(size_t)cnt[o] * N + o] = n; cnt[o]++;
            ef[(size_t)cnt[n] * N + n] = f; en[(size_t)cnt[n] * N + n] = o; cnt[n]++;
        }
        upload_vec(ctx, ef, m.ellFace);
        upload_vec(ctx, en, m.ellNbr);
        // the preconditioner's ELL: the same slots without the coupled faces
        m.pellFace.release();
        m.pellNbr.release();
        m.pnSlots = ns;
        if (m.hasCoupled) {
            std::fill(cnt.begin(), cnt.end(), 0);
            for (int f = 0; f < F; ++f)
                if (!m.coupledH[f]) { cnt[md->owner[f]]++; cnt[md->neighbour[f]]++; }
            int pns = 0;
            for (int c = 0; c < N; ++c) pns = std::max(pns, cnt[c]);
            m.pnSlots = pns;
            std::vector<int> pf((size_t)std::max(pns, 1) * N, -1), pn((size_t)std::max(pns, 1) * N, -1);
            std::fill(cnt.begin(), cnt.end(), 0);
            for (int f = 0; f < F; ++f) {
                if (m.coupledH[f]) continue;
                int o = md->owner[f], n = md->neighbour[f];
                pf[(size_t)cnt[o] * N + o] = f; pn[(size_t)cnt[o] * N + o] = n; cnt[o]++;
                pf[(size_t)cnt[n] * N + n] = f; pn[(size_t)cnt[n] * N + n] = o; cnt[n]++;
            }
            upload_vec(ctx, pf, m.pellFace);
            upload_vec(ctx, pn, m.pellNbr);
        }
        // the preconditioner adjacency split into lower and upper neighbours
        {
            std::vector<int> nlo(N, 0), nup(N, 0);
            for (int f = 0; f < F; ++f) {
                if (m.hasCoupled && m.coupledH[f]) continue;
                nlo[md->neighbour[f]]++;
                nup[md->owner[f]]++;
            }
            int mlo = 0, mup = 0;
            for (int c = 0; c < N; ++c) { mlo = std::max(mlo, nlo[c]); mup = std::max(mup, nup[c]); }
            m.pnLo = mlo;
            m.pnUp = mup;
            std::vector<int> ln((size_t)std::max(mlo, 1) * N, -1), lf((size_t)std::max(mlo, 1) * N, -1);
            std::vector<int> un((size_t)std::max(mup, 1) * N, -1), uf((size_t)std::max(mup, 1) * N, -1);
            std::fill(nlo.begin(), nlo.end(), 0);
            std::fill(nup.begin(), nup.end(), 0);
            for (int f = 0; f < F; ++f) {   // faces ascending: each cell's slots in face order
                if (m.hasCoupled && m.coupledH[f]) continue;
                const int o = md->owner[f], n = md->neighbour[f];
                ln[(size_t)nlo[n] * N + n] = o; lf[(size_t)nlo[n] * N + n] = f; nlo[n]++;
                un[(size_t)nup[o] * N + o] = n; uf[(size_t)nup[o] * N + o] = f; nup[o]++;
            }
            upload_vec(ctx, ln, m.plNbr);
            upload_vec(ctx, lf, m.plFace);
            upload_vec(ctx, un, m.puNbr);
            upload_vec(ctx, uf, m.puFace);
        }
        // ---- boundary CSR ----------------------------------------------------
        std::vector<int> bs(N + 1, 0), bl(NB);
        for (int b = 0; b < NB; ++b) bs[md->bCell[b] + 1]++;
        for (int c = 0; c < N; ++c) bs[c + 1] += bs[c];
        {
            std::vector<int> pos(bs.begin(), bs.end() - 1);
            for (int b = 0; b < NB; ++b) bl[pos[md->bCell[b]]++] = b;
        }
        upload_vec(ctx, bs, m.bStart);
        upload_vec(ctx, bl, m.bList);
        std::vector<int> bc;
        for (int c = 0; c < N; ++c) if (bs[c + 1] > bs[c]) bc.push_back(c);
        m.nBCells = (int)bc.size();
        upload_vec(ctx, bc, m.bCells);
        // ---- level schedule ------------------------------------------------
        std::vector<int> lev(N, 0);
        for (int f = 0; f < F; ++f) {
            int o = md->owner[f], n = md->neighbour[f];
            lev[n] = std::max(lev[n], lev[o] + 1);
        }
        int nl = 0;
        for (int c = 0; c < N; ++c) nl = std::max(nl, lev[c] + 1);
        m.nLevels = nl;
        m.levelStartH.assign(nl + 1, 0);
        for (int c = 0; c < N; ++c) m.levelStartH[lev[c] + 1]++;
        for (int l = 0; l < nl; ++l) m.levelStartH[l + 1] += m.levelStartH[l];
        std::vector<int> lc(N), pos(m.levelStartH.begin(), m.levelStartH.end() - 1);
        for (int c = 0; c < N; ++c) lc[pos[lev[c]]++] = c;
        upload_vec(ctx, lc, m.levelCells);
        // ---- scratch ---------------------------------------------------------
        size_t need = (size_t)N * 160 + (size_t)F * 24 + (size_t)NB * 96 + 4096;
        ctx->work.a.alloc(need);
        ctx->work.used = 0;
        m.batch.n = 1;
        m.batch.sweep2d = false;
        RT_CUDA(cudaStreamSynchronize(s));
        ctx->meshReady = true;
        ctx->cs.ready = false;
        ctx->cs.thermoOn = false;
        return RT_OK;
    });
}

rt_status rt_mesh_set_ijk(rt_ctx *ctx, int32_t nx, int32_t ny, int32_t nz, const int32_t *cellIJK) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->meshReady, RT_ENOTREADY, "mesh not uploaded");
        RT_REQUIRE(nx > 0 && ny > 0 && nz > 0 && cellIJK, RT_EINVAL, "bad box dimensions");
        DevMesh &m = ctx->mesh;
        StructMesh &s = m.sm;
        s.on = false;
        const int N = m.N, F = m.F;
        const long long box = (long long)nx * ny * nz;
        std::vector<int> at((size_t)box, -1);
        long long prev = -1;
        for (int c = 0; c < N; ++c) {
            int i = cellIJK[3 * c], j = cellIJK[3 * c + 1], k = cellIJK[3 * c + 2];
            RT_REQUIRE(i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz, RT_EINVAL, "cell outside the box");
            long long key = ((long long)k * ny + j) * nx + i;
            RT_REQUIRE(key > prev, RT_EINVAL, "cells are not numbered lexicographically (i fastest)");
            prev = key;
            at[(size_t)key] = c;
        }
        // faces must join box neighbours; record the face of each direction
        std::vector<int> own(F), nei(F);
        RT_CUDA(cudaMemcpy(own.data(), m.owner.p, sizeof(int) * F, cudaMemcpyDeviceToHost));
        RT_CUDA(cudaMemcpy(nei.data(), m.neighbour.p, sizeof(int) * F, cudaMemcpyDeviceToHost));
        std::vector<int> lo((size_t)3 * N, -1), hi((size_t)3 * N, -1);
        for (int f = 0; f < F; ++f) {
            int o = own[f], n = nei[f];
            if (m.hasCoupled && m.coupledH[f]) continue;   // not part of the sweeps
            int di = cellIJK[3 * n] - cellIJK[3 * o], dj = cellIJK[3 * n + 1] - cellIJK[3 * o + 1],
                dk = cellIJK[3 * n + 2] - cellIJK[3 * o + 2];
            int dir = (di == 0 && dj == 0 && dk == 1) ? 0 : (di == 0 && dj == 1 && dk == 0) ? 1
                      : (di == 1 && dj == 0 && dk == 0) ? 2 : -1;   // 0 z, 1 y, 2 x
            RT_REQUIRE(dir >= 0, RT_EINVAL, "face " + std::to_string(f) + " does not join box neighbours");
            RT_REQUIRE(hi[(size_t)dir * N + o] < 0 && lo[(size_t)dir * N + n] < 0, RT_EINVAL, "duplicate face");
            hi[(size_t)dir * N + o] = f;
            lo[(size_t)dir * N + n] = f;
        }
        s.nx = nx; s.ny = ny; s.nz = nz;
        s.nJB = (ny + 31) / 32;
        s.T = ((nx + 31 + 15) / 16) * 16;   // steps per block, padded to whole chunks (P <= 16)
        s.nSkew = (long long)nz * s.nJB * s.T * 32;
        std::vector<int> cellOf((size_t)s.nSkew, -1);
        for (int k = 0; k < nz; ++k)
            for (int jb = 0; jb < s.nJB; ++jb)
                for (int t = 0; t < s.T; ++t)
                    for (int l = 0; l < 32; ++l) {
                        int i = t - l, j = jb * 32 + l;
                        if (i < 0 || i >= nx || j >= ny) continue;
                        // quad layout: one lane's four consecutive steps are adjacent
                        long long e = ((long long)k * s.nJB + jb) * s.T * 32 + (long long)(t >> 2) * 128 + l * 4 + (t & 3);
                        cellOf[(size_t)e] = at[((size_t)k * ny + j) * nx + i];
                    }
        upload_vec(ctx, cellOf, s.cellOf);
        upload_vec(ctx, lo, s.faceLo);
        upload_vec(ctx, hi, s.faceHi);
        {   // the box maps (the multigrid preconditioner's level 0)
            std::vector<int> boxOf(N);
            for (size_t b = 0; b < at.size(); ++b)
                if (at[b] >= 0) boxOf[at[b]] = (int)b;
            upload_vec(ctx, at, s.cellAt);
            upload_vec(ctx, boxOf, s.boxOf);
            s.mgDims.clear();
            for (MgGraph &g : s.mgGraph) g.reset();
            s.mgNext = 0;
        }
        RT_REQUIRE(s.nJB <= 8 && skew_fits(s.nJB), RT_EINVAL, "structured sweeps need ny <= 256");
        // planes (CTAs) per thread-block cluster: 16 (the non-portable maximum;
        // fewer hand-offs through global memory), 8 where 16 cannot be scheduled
        s.KC = std::max(1, std::min(nz, 16));
        s.sync.alloc(SYNC_PROGRESS + (size_t)nz * s.nJB);
        s.sync.zero(ctx->stream);
        s.data.alloc((size_t)(12 + 6 + 6) * s.nSkew);
        s.data.zero(ctx->stream);
        // the two colours of the box (red: i + j + k even)
        {
            std::vector<unsigned char> col(N);
            int red = 0;
            for (int c = 0; c < N; ++c) {
                col[c] = (unsigned char)((cellIJK[3 * c] + cellIJK[3 * c + 1] + cellIJK[3 * c + 2]) & 1);
                red += col[c] == 0;
            }
            upload_vec(ctx, col, m.colour);
            m.nRed = red;
        }
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        s.tune[0] = s.tune[1] = -1;
        s.on = true;
        return RT_OK;
    });
}

rt_status rt_set_option(rt_ctx *ctx, int32_t option, int64_t value) {
    return guarded(ctx, [&]() -> rt_status {
        switch (option) {
        case RT_OPT_SWEEP:
            RT_REQUIRE(value >= 0 && value <= 2, RT_EINVAL, "RT_OPT_SWEEP: 0 auto, 1 levels, 2 structured");
            ctx->sweepMode = (int)value;
            return RT_OK;
        case RT_OPT_SWEEP_PLANES: {
            StructMesh &s = ctx->mesh.sm;
            RT_REQUIRE(s.on, RT_ENOTREADY, "mesh is not structured");
            RT_REQUIRE(value >= 1 && value <= 16, RT_EINVAL, "planes per cluster: 1 .. 16");
            s.KC = (int)std::min<int64_t>(value, s.nz);
            s.tune[0] = s.tune[1] = -1;
            return RT_OK;
        }
        case RT_OPT_SWEEP_TUNE:
            RT_REQUIRE(value >= 0 && value <= 5, RT_EINVAL, "RT_OPT_SWEEP_TUNE: 0 autotune, 1 .. 5 a schedule");
            ctx->sweepTune = (int)value;
            ctx->mesh.sm.tune[0] = ctx->mesh.sm.tune[1] = -1;
            return RT_OK;
        case RT_OPT_SWEEP_RING:
            RT_REQUIRE(value == 0 || (value >= 8 && value <= 128 && (value & (value - 1)) == 0), RT_EINVAL,
                       "RT_OPT_SWEEP_RING: 0, or a power of two 8 .. 128");
            ctx->sweepRing = (int)value;
            ctx->mesh.sm.tune[0] = ctx->mesh.sm.tune[1] = -1;
            return RT_OK;
        case RT_OPT_WAIT_LIMIT:
            RT_REQUIRE(value >= 64 && value <= (1ll << 40), RT_EINVAL, "RT_OPT_WAIT_LIMIT: 64 .. 2^40 spins");
            ctx->waitLimit = value;
            return RT_OK;
        case RT_OPT_STALL_TEST:
            RT_REQUIRE(value >= 0 && value <= 1000, RT_EINVAL, "RT_OPT_STALL_TEST: 0 .. 1000 launches");
            ctx->stallTest = (int)value;
            return RT_OK;
        case RT_OPT_MIXED_TIGHTEN:
            RT_REQUIRE(value >= 0 && value <= 12, RT_EINVAL, "RT_OPT_MIXED_TIGHTEN: decades 0 .. 12");
            ctx->mixedTighten = std::pow(10.0, -(double)value);
            return RT_OK;
        case RT_OPT_MIXED_PRECOND:
            RT_REQUIRE(value >= -2 && value <= 64, RT_EINVAL,
                       "RT_OPT_MIXED_PRECOND: 0 exact sweeps, -1 red-black DIC, -2 aggregation multigrid, 1 .. 64 "
                       "Jacobi sweeps per triangular factor");
            ctx->mixedJacobi = (int)value;
            return RT_OK;
        case RT_OPT_MIXED_PRECOND_U:
            RT_REQUIRE(value == 0 || value == -2, RT_EINVAL,
                       "RT_OPT_MIXED_PRECOND_U: 0 exact DILU sweeps, -2 aggregation multigrid");
            ctx->mixedPrecondU = (int)value;
            return RT_OK;
        case RT_OPT_SWEEP_COMPONENTS:
            RT_REQUIRE(value == 0 || value == 1, RT_EINVAL, "RT_OPT_SWEEP_COMPONENTS: 0 or 1");
            ctx->sweepComponents = (int)value;
            return RT_OK;
        case RT_OPT_BATCH_PERSISTENT:
            RT_REQUIRE(value >= 0 && value <= 2, RT_EINVAL, "RT_OPT_BATCH_PERSISTENT: 0 never, 1 auto, 2 always");
            ctx->batchPersistent = (int)value;
            return RT_OK;
        case RT_OPT_MIXED_PARTS:
            RT_REQUIRE(value >= 0 && value <= 3, RT_EINVAL, "RT_OPT_MIXED_PARTS: bit 1 Krylov, bit 2 constitutive");
            ctx->mixedParts = (int)value;
            return RT_OK;
        case RT_OPT_PRECISION:
            RT_REQUIRE(value == RT_PREC_FP64 || value == RT_PREC_MIXED, RT_EINVAL,
                       "RT_OPT_PRECISION: RT_PREC_FP64 or RT_PREC_MIXED");
            ctx->precision = (int)value;
            return RT_OK;
        default:
            return RT_EINVAL;
        }
    });
}

rt_status rt_case_setup(rt_ctx *ctx, const rt_bc_desc *bc, const rt_model_params *mp,
                        const rt_case_ctl *ctl) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->meshReady, RT_ENOTREADY, "mesh not uploaded");
        RT_REQUIRE(bc && mp && ctl, RT_EINVAL, "null argument");
        validate_model(mp);
        const bool pttGen = mp->model == RT_MODEL_PTT_LOG && mp->pttFunction == RT_PTT_GENERALIZED;
        RT_REQUIRE(ctl->deltaT > 0, RT_EINVAL, "deltaT must be positive");
        RT_REQUIRE(ctl->nNonOrthCorr >= 0 && ctl->nNonOrthCorr <= 100, RT_EINVAL,
                   "nNonOrthogonalCorrectors: 0 .. 100");
        RT_REQUIRE(ctl->ddtScheme == RT_DDT_EULER ||
                       (ctl->ddtScheme == RT_DDT_CRANKNICOLSON && ctl->ddtPsi >= 0.0 && ctl->ddtPsi <= 1.0),
                   RT_EINVAL, "ddt scheme: Euler, or CrankNicolson with 0 <= psi <= 1");
        for (const rt_solver_ctl *sc : {&ctl->solverU, &ctl->solverP, &ctl->solverTheta}) {
            RT_REQUIRE(sc->solver >= RT_SOLVER_PCG && sc->solver <= RT_SOLVER_PBICG, RT_EINVAL, "unknown solver");
            RT_REQUIRE(sc->preconditioner >= RT_PRECOND_NONE && sc->preconditioner <= RT_PRECOND_DIAGONAL, RT_EINVAL,
                       "unknown preconditioner");
        }
        RT_REQUIRE(ctl->divU >= RT_LIM_NONE && ctl->divU <= RT_LIM_SUPERBEE &&
                       ctl->divTheta >= RT_LIM_NONE && ctl->divTheta <= RT_LIM_SUPERBEE,
                   RT_EINVAL, "unknown GaussDefCmpw limiter");
        DevMesh &m = ctx->mesh;
        DevCase &c = ctx->cs;
        RT_REQUIRE(ctl->pRefCell >= 0 && ctl->pRefCell < m.N, RT_EINVAL, "pRefCell out of range");
        c.mp = *mp;
        c.ctl = *ctl;
        c.thetaOldSaved = false;
        c.nModes = 1;            // rt_case_setup_modes adds the further modes
        c.modes.clear();
        c.tauTot.release();
        c.taubTot.release();
        c.thetaStep0.release();
        c.modePerf.clear();
        c.mpMom = *mp;
        // Crank-Nicolson state: no step taken yet, D = 0
        c.ddtSteps = c.ddtThSteps = 0;
        c.ddtC = c.ddtCth = 1.0;
        for (DBuf<double> *b : {&c.DU, &c.DUb, &c.Dphi, &c.Dphib, &c.Us, &c.Ubs, &c.phis, &c.phibs, &c.Dth, &c.ths})
            b->release();
        if (ctl->ddtScheme == RT_DDT_CRANKNICOLSON) {
            const size_t N = m.N, F = m.F, NB = m.NB;
            const std::pair<DBuf<double> *, size_t> bufs[] = {{&c.DU, 3 * N}, {&c.DUb, 3 * NB}, {&c.Dphi, F},
                                                              {&c.Dphib, NB}, {&c.Us, 3 * N}, {&c.Ubs, 3 * NB},
                                                              {&c.phis, F}, {&c.phibs, NB}, {&c.Dth, 6 * N},
                                                              {&c.ths, 6 * N}};
            for (const auto &b : bufs) {
                b.first->alloc(b.second);
                b.first->zero(ctx->stream);
            }
        }
        if (pttGen) {
            std::vector<double> g = ml_gamma_table(*mp);
            c.mlK = (int)g.size() - 1;
            RT_REQUIRE(c.mlK >= 1, RT_EINVAL, "Gamma(beta) overflows: no Mittag-Leffler term");
            upload_vec(ctx, g, c.mlGamma);
        } else {
            c.mlGamma.release();
            c.mlK = 0;
        }
        const int P = m.nPatches, NB = m.NB, N = m.N;
        c.kindU.assign(bc->U, bc->U + P);
        c.kindP.assign(bc->p, bc->p + P);
        c.kindTheta.assign(bc->theta, bc->theta + P);
        c.kindTau.assign(bc->tau, bc->tau + P);
        for (int p = 0; p < P; ++p) {
            RT_REQUIRE(c.kindU[p] == RT_BC_FIXED || c.kindU[p] == RT_BC_ZEROGRAD, RT_EINVAL, "U: unsupported BC");
            RT_REQUIRE(c.kindP[p] == RT_BC_FIXED || c.kindP[p] == RT_BC_ZEROGRAD, RT_EINVAL, "p: unsupported BC");
            RT_REQUIRE(c.kindTheta[p] == RT_BC_FIXED || c.kindTheta[p] == RT_BC_ZEROGRAD, RT_EINVAL, "theta: unsupported BC");
            RT_REQUIRE(c.kindTau[p] >= RT_BC_FIXED && c.kindTau[p] <= RT_BC_LINEXTRAP, RT_EINVAL, "tau: unsupported BC");
        }
        auto per_face = [&](const std::vector<int> &k, DBuf<int> &d) {
            std::vector<int> v(NB);
            for (int p = 0; p < P; ++p)
                for (int i = 0; i < m.patchSizeH[p]; ++i) v[m.patchStartH[p] + i] = k[p];
            upload_vec(ctx, v, d);
        };
        per_face(c.kindU, c.bkU);
        per_face(c.kindP, c.bkP);
        per_face(c.kindTheta, c.bkTh);
        per_face(c.kindTau, c.bkTau);
        c.tauWaveH.clear();
        c.tauWaveFace.release();
        if (m.batch.n > 1) {
            // patch order within each case: the k-th updating patch of a case
            // sees the values its earlier patches wrote (corner cells)
            const std::vector<int> &bs = m.batch.bStartH;
            std::vector<std::vector<int>> waves;
            std::vector<int> rank(m.batch.n, 0);
            for (int p = 0; p < P; ++p) {
                if (m.patchSizeH[p] == 0 || (c.kindTau[p] != RT_BC_ZEROGRAD && c.kindTau[p] != RT_BC_LINEXTRAP))
                    continue;
                const int k = (int)(std::upper_bound(bs.begin(), bs.end(), m.patchStartH[p]) - bs.begin()) - 1;
                const int wv = rank[k]++;
                if ((int)waves.size() <= wv) waves.resize(wv + 1);
                for (int i = 0; i < m.patchSizeH[p]; ++i) waves[wv].push_back(m.patchStartH[p] + i);
            }
            std::vector<int> faces;
            c.tauWaveH.push_back(0);
            for (auto &w : waves) {
                faces.insert(faces.end(), w.begin(), w.end());
                c.tauWaveH.push_back((int)faces.size());
            }
            if (!faces.empty()) upload_vec(ctx, faces, c.tauWaveFace);
        }
        upload_soa(ctx, bc->Ub, NB, 3, c.UbFixed);
        upload_soa(ctx, bc->pb, NB, 1, c.pbFixed);
        upload_soa(ctx, bc->thetab, NB, 6, c.thetabFixed);
        upload_soa(ctx, bc->taub, NB, 6, c.taubFixed);
        // state: U = p = theta = tau = 0, eigVals = eigVecs = I
        c.U.alloc(3 * (size_t)N); c.U.zero(ctx->stream);
        c.p.alloc(N); c.p.zero(ctx->stream);
        c.theta.alloc(6 * (size_t)N); c.theta.zero(ctx->stream);
        c.tau.alloc(6 * (size_t)N); c.tau.zero(ctx->stream);
        c.Ub.alloc(3 * (size_t)NB); c.pb.alloc(NB); c.thetab.alloc(6 * (size_t)NB); c.taub.alloc(6 * (size_t)NB);
        c.phi.alloc(m.F); c.phib.alloc(NB);
        c.eigVals.alloc(3 * (size_t)N);
        c.eigVecs.alloc(9 * (size_t)N);
        init_fields(ctx);
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        c.thermoOn = false;   // a new case is isothermal until rt_set_temperature
        c.ready = true;
        return RT_OK;
    });
}

static void field_info(rt_ctx *ctx, int field, DBuf<double> **in, DBuf<double> **bd, int *nc, int *nIn) {
    DevCase &c = ctx->cs;
    *nIn = ctx->mesh.N;
    switch (field) {
    case RT_FIELD_U: *in = &c.U; *bd = &c.Ub; *nc = 3; break;
    case RT_FIELD_P: *in = &c.p; *bd = &c.pb; *nc = 1; break;
    case RT_FIELD_PHI: *in = &c.phi; *bd = &c.phib; *nc = 1; *nIn = ctx->mesh.F; break;
    case RT_FIELD_THETA: *in = &c.theta; *bd = &c.thetab; *nc = 6; break;
    case RT_FIELD_TAU:   // multiMode: the modes' summed tau (multiMode::tau())
        *in = c.nModes > 1 ? &c.tauTot : &c.tau;
        *bd = c.nModes > 1 ? &c.taubTot : &c.taub;
        *nc = 6;
        break;
    case RT_FIELD_EIGVALS: *in = &c.eigVals; *bd = nullptr; *nc = 3; break;
    case RT_FIELD_EIGVECS: *in = &c.eigVecs; *bd = nullptr; *nc = 9; break;
    default: throw Error{RT_EINVAL, "unknown field id"};
    }
}

rt_status rt_field_set(rt_ctx *ctx, int32_t field, const double *internal, const double *boundary) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->cs.ready, RT_ENOTREADY, "case not set up");
        DBuf<double> *in, *bd;
        int nc, nIn;
        field_info(ctx, field, &in, &bd, &nc, &nIn);
        if (internal) upload_soa(ctx, internal, nIn, nc, *in);
        // a new theta starts a new time step for rt_constitutive_correct_iter
        if (field == RT_FIELD_THETA && internal) ctx->cs.thetaOldSaved = false;
        if (boundary) {
            RT_REQUIRE(bd != nullptr, RT_EINVAL, "field has no boundary values");
            upload_soa(ctx, boundary, ctx->mesh.NB, nc, *bd);
        }
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        return RT_OK;
    });
}

// one mode's theta / tau / eigVals / eigVecs of a multiMode case
static void mode_field_info(rt_ctx *ctx, int field, int mode, DBuf<double> **in, DBuf<double> **bd, int *nc) {
    DevCase &c = ctx->cs;
    RT_REQUIRE(mode >= 0 && mode < c.nModes, RT_EINVAL, "mode out of range");
    RT_REQUIRE(field == RT_FIELD_THETA || field == RT_FIELD_TAU || field == RT_FIELD_EIGVALS ||
                   field == RT_FIELD_EIGVECS,
               RT_EINVAL, "per-mode fields: theta, tau, eigVals, eigVecs");
    if (mode == 0 || c.nModes == 1) {
        switch (field) {
        case RT_FIELD_THETA: *in = &c.theta; *bd = &c.thetab; *nc = 6; return;
        case RT_FIELD_TAU: *in = &c.tau; *bd = &c.taub; *nc = 6; return;
        case RT_FIELD_EIGVALS: *in = &c.eigVals; *bd = nullptr; *nc = 3; return;
        default: *in = &c.eigVecs; *bd = nullptr; *nc = 9; return;
        }
    }
    ModeState &m = *c.modes[mode - 1];
    switch (field) {
    case RT_FIELD_THETA: *in = &m.theta; *bd = &m.thetab; *nc = 6; return;
    case RT_FIELD_TAU: *in = &m.tau; *bd = &m.taub; *nc = 6; return;
    case RT_FIELD_EIGVALS: *in = &m.eigVals; *bd = nullptr; *nc = 3; return;
    default: *in = &m.eigVecs; *bd = nullptr; *nc = 9; return;
    }
}

rt_status rt_field_set_mode(rt_ctx *ctx, int32_t field, int32_t mode, const double *internal,
                            const double *boundary) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->cs.ready, RT_ENOTREADY, "case not set up");
        DBuf<double> *in, *bd;
        int nc;
        mode_field_info(ctx, field, mode, &in, &bd, &nc);
        if (internal) upload_soa(ctx, internal, ctx->mesh.N, nc, *in);
        if (field == RT_FIELD_THETA && internal) {
            if (mode == 0) ctx->cs.thetaOldSaved = false;
            else ctx->cs.modes[mode - 1]->thetaOldSaved = false;
        }
        if (boundary) {
            RT_REQUIRE(bd != nullptr, RT_EINVAL, "field has no boundary values");
            upload_soa(ctx, boundary, ctx->mesh.NB, nc, *bd);
        }
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        return RT_OK;
    });
}

rt_status rt_field_get_mode(rt_ctx *ctx, int32_t field, int32_t mode, double *internal, double *boundary) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->cs.ready, RT_ENOTREADY, "case not set up");
        DBuf<double> *in, *bd;
        int nc;
        mode_field_info(ctx, field, mode, &in, &bd, &nc);
        if (internal) download_aos(ctx, *in, ctx->mesh.N, nc, internal);
        if (boundary) {
            RT_REQUIRE(bd != nullptr, RT_EINVAL, "field has no boundary values");
            download_aos(ctx, *bd, ctx->mesh.NB, nc, boundary);
        }
        return RT_OK;
    });
}

rt_status rt_mode_perf(rt_ctx *ctx, rt_solver_perf *thetaPerf) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(thetaPerf, RT_EINVAL, "null argument");
        DevCase &c = ctx->cs;
        RT_REQUIRE(c.ready, RT_ENOTREADY, "case not set up");
        RT_REQUIRE(c.nModes > 1 && c.modePerf.size() == 6 * (size_t)c.nModes, RT_ENOTREADY,
                   "no multiMode correct() has run");
        for (size_t i = 0; i < c.modePerf.size(); ++i) thetaPerf[i] = c.modePerf[i];
        return RT_OK;
    });
}

rt_status rt_case_setup_modes(rt_ctx *ctx, const rt_bc_desc *bc, const rt_model_params *models, int32_t nModes,
                              const rt_case_ctl *ctl) {
    {
        rt_status v = guarded(ctx, [&]() -> rt_status {
            RT_REQUIRE(models && nModes >= 1 && nModes <= RT_MAX_MODES, RT_EINVAL,
                       "multiMode: 1 .. " + std::to_string(RT_MAX_MODES) + " modes");
            RT_REQUIRE(ctx->mesh.batch.n <= 1, RT_EINVAL, "the batched form runs single-mode models");
            for (int i = 0; i < nModes; ++i) {
                validate_model(&models[i]);
                // one divTau with the summed tau and viscosities (multiMode.C:144-156)
                RT_REQUIRE(models[i].rho == models[0].rho && models[i].stabilization == models[0].stabilization,
                           RT_EINVAL, "multiMode: every mode needs the same rho and stabilization");
            }
            return RT_OK;
        });
        if (v != RT_OK) return v;
    }
    rt_status st = rt_case_setup(ctx, bc, &models[0], ctl);
    if (st != RT_OK || nModes == 1) return st;
    return guarded(ctx, [&]() -> rt_status {
        DevCase &c = ctx->cs;
        const int N = ctx->mesh.N, NB = ctx->mesh.NB;
        const size_t n6 = 6 * (size_t)N, b6 = 6 * (size_t)NB;
        cudaStream_t s = ctx->stream;
        c.ready = false;
        for (int i = 1; i < nModes; ++i) {
            std::unique_ptr<ModeState> m(new ModeState());
            m->mp = models[i];
            // every mode starts as mode 0 did: theta = tau = 0, A = I, the
            // boundary values of the theta and tau conditions
            m->theta.alloc(n6); m->theta.zero(s);
            m->tau.alloc(n6); m->tau.zero(s);
            m->thetab.alloc(b6); m->taub.alloc(b6);
            if (b6) {
                RT_CUDA(cudaMemcpyAsync(m->thetab.p, c.thetab.p, sizeof(double) * b6, cudaMemcpyDeviceToDevice, s));
                RT_CUDA(cudaMemcpyAsync(m->taub.p, c.taub.p, sizeof(double) * b6, cudaMemcpyDeviceToDevice, s));
            }
            m->eigVals.alloc(3 * (size_t)N);
            m->eigVecs.alloc(9 * (size_t)N);
            RT_CUDA(cudaMemcpyAsync(m->eigVals.p, c.eigVals.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
            RT_CUDA(cudaMemcpyAsync(m->eigVecs.p, c.eigVecs.p, sizeof(double) * 9 * N, cudaMemcpyDeviceToDevice, s));
            if (models[i].model == RT_MODEL_PTT_LOG && models[i].pttFunction == RT_PTT_GENERALIZED) {
                std::vector<double> g = ml_gamma_table(models[i]);
                m->mlK = (int)g.size() - 1;
                RT_REQUIRE(m->mlK >= 1, RT_EINVAL, "Gamma(beta) overflows: no Mittag-Leffler term");
                upload_vec(ctx, g, m->mlGamma);
            }
            if (ctl->ddtScheme == RT_DDT_CRANKNICOLSON) {
                m->Dth.alloc(n6); m->Dth.zero(s);
                m->ths.alloc(n6); m->ths.zero(s);
            }
            c.modes.push_back(std::move(m));
        }
        c.nModes = nModes;
        rt_model_params e = models[0];
        e.etaS = 0.0;
        e.etaP = 0.0;
        for (int i = 0; i < nModes; ++i) {
            e.etaS += models[i].etaS;
            e.etaP += models[i].etaP;
        }
        c.mpMom = e;
        // tau() of the initial state: the modes' sum
        c.tauTot.alloc(n6);
        c.tauTot.zero(s);
        c.taubTot.alloc(b6);
        c.taubTot.zero(s);
        for (int i = 0; i < nModes && b6; ++i) {
            const double *tb = i ? c.modes[i - 1]->taub.p : c.taub.p;
            // taubTot += taub_i (through the host: setup only)
            std::vector<double> h(b6), acc(b6);
            RT_CUDA(cudaMemcpyAsync(h.data(), tb, sizeof(double) * b6, cudaMemcpyDeviceToHost, s));
            RT_CUDA(cudaMemcpyAsync(acc.data(), c.taubTot.p, sizeof(double) * b6, cudaMemcpyDeviceToHost, s));
            RT_CUDA(cudaStreamSynchronize(s));
            for (size_t j = 0; j < b6; ++j) acc[j] += h[j];
            RT_CUDA(cudaMemcpyAsync(c.taubTot.p, acc.data(), sizeof(double) * b6, cudaMemcpyHostToDevice, s));
            RT_CUDA(cudaStreamSynchronize(s));
        }
        RT_CUDA(cudaStreamSynchronize(s));
        c.thermoOn = false;   // a new case is isothermal until rt_set_temperature
        c.ready = true;
        return RT_OK;
    });
}

rt_status rt_field_get(rt_ctx *ctx, int32_t field, double *internal, double *boundary) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->cs.ready, RT_ENOTREADY, "case not set up");
        DBuf<double> *in, *bd;
        int nc, nIn;
        field_info(ctx, field, &in, &bd, &nc, &nIn);
        if (internal) download_aos(ctx, *in, nIn, nc, internal);
        if (boundary) {
            RT_REQUIRE(bd != nullptr, RT_EINVAL, "field has no boundary values");
            download_aos(ctx, *bd, ctx->mesh.NB, nc, boundary);
        }
        return RT_OK;
    });
}

rt_status rt_ldu_solve(rt_ctx *ctx, const double *diag, const double *upper, const double *lower,
                       const double *source, double *psi, int32_t ncmpt, const rt_solver_ctl *ctl,
                       rt_solver_perf *perf) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->meshReady, RT_ENOTREADY, "mesh not uploaded");
        RT_REQUIRE(ncmpt >= 1 && ncmpt <= 6, RT_EINVAL, "ncmpt must be 1..6");
        RT_REQUIRE(diag && upper && lower && source && psi && ctl && perf, RT_EINVAL, "null argument");
        RT_REQUIRE(ctl->solver >= RT_SOLVER_PCG && ctl->solver <= RT_SOLVER_PBICG, RT_EINVAL, "unknown solver");
        RT_REQUIRE(ctl->preconditioner >= RT_PRECOND_NONE && ctl->preconditioner <= RT_PRECOND_DIAGONAL,
                   RT_EINVAL, "unknown preconditioner");
        const int N = ctx->mesh.N, F = ctx->mesh.F;
        DBuf<double> d, u, l, b, x;
        cudaStream_t s = ctx->stream;
        d.upload(diag, N, s);
        u.upload(upper, F, s);
        l.upload(lower, F, s);
        b.upload(source, (size_t)ncmpt * N, s);
        x.upload(psi, (size_t)ncmpt * N, s);
        SolveArgs a{d.p, u.p, l.p, b.p, x.p, ncmpt, (1u << ncmpt) - 1u, *ctl, ctx->precision};
        rt_status st = ldu_solve_device(ctx, a, perf);
        RT_CUDA(cudaMemcpyAsync(psi, x.p, sizeof(double) * ncmpt * N, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
        return st;
    });
}

rt_status rt_residual(rt_ctx *ctx, const double *diag, const double *upper, const double *lower,
                      const double *source, const double *psi, double *residual) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->meshReady, RT_ENOTREADY, "mesh not uploaded");
        RT_REQUIRE(diag && upper && lower && source && psi && residual, RT_EINVAL, "null argument");
        const int N = ctx->mesh.N, F = ctx->mesh.F;
        DBuf<double> d, u, l, b, x;
        cudaStream_t s = ctx->stream;
        d.upload(diag, N, s);
        u.upload(upper, F, s);
        l.upload(lower, F, s);
        b.upload(source, N, s);
        x.upload(psi, N, s);
        *residual = residual_device(ctx, d.p, u.p, l.p, b.p, x.p);
        return RT_OK;
    });
}

rt_status rt_op_grad(rt_ctx *ctx, const double *psi, const double *psib, double *grad) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->meshReady, RT_ENOTREADY, "mesh not uploaded");
        RT_REQUIRE(psi && psib && grad, RT_EINVAL, "null argument");
        const int N = ctx->mesh.N, NB = ctx->mesh.NB;
        DBuf<double> x, xb, g;
        x.upload(psi, N, ctx->stream);
        xb.upload(psib, NB, ctx->stream);
        g.alloc(3 * (size_t)N);
        grad_scalar(ctx, x.p, xb.p, g.p);
        download_aos(ctx, g, N, 3, grad);
        return RT_OK;
    });
}

rt_status rt_op_eig(rt_ctx *ctx, int32_t n, const double *theta, double *eigVals, double *eigVecs) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(n >= 0 && theta && eigVals && eigVecs, RT_EINVAL, "bad argument");
        if (n == 0) return RT_OK;
        DBuf<double> th, ev, vv;
        upload_soa(ctx, theta, n, 6, th);
        ev.alloc(3 * (size_t)n);
        vv.alloc(9 * (size_t)n);
        eig_cells(ctx, n, th.p, ev.p, vv.p);
        download_aos(ctx, ev, n, 3, eigVals);
        download_aos(ctx, vv, n, 9, eigVecs);
        return RT_OK;
    });
}

rt_status rt_constitutive_correct(rt_ctx *ctx, const double *gradU, rt_solver_perf *thetaPerf) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->cs.ready, RT_ENOTREADY, "case not set up");
        RT_REQUIRE(thetaPerf, RT_EINVAL, "null perf");
        DBuf<double> g;
        if (gradU) upload_soa(ctx, gradU, ctx->mesh.N, 9, g);
        // a completed time step: the old-time theta kept by
        // rt_constitutive_correct_iter belongs to an earlier step now
        ctx->cs.thetaOldSaved = false;
        ddt_begin_step(ctx, false);   // a time step of its own (Crank-Nicolson state)
        rt_status st = modes_correct(ctx, gradU ? g.p : nullptr, thetaPerf);
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        return st;
    });
}

rt_status rt_constitutive_correct_iter(rt_ctx *ctx, const double *gradU, int32_t newTimeStep,
                                       rt_solver_perf *thetaPerf) {
    return guarded(ctx, [&]() -> rt_status {
        DevCase &c = ctx->cs;
        RT_REQUIRE(c.ready, RT_ENOTREADY, "case not set up");
        RT_REQUIRE(thetaPerf, RT_EINVAL, "null perf");
        RT_REQUIRE(c.nModes == 1, RT_EINVAL,
                   "rt_constitutive_correct_iter runs single-mode models (a multiMode step's inner iterations "
                   "run inside rt_step)");
        const size_t n6 = 6 * (size_t)ctx->mesh.N;
        if (newTimeStep) {
            ddt_begin_step(ctx, false);   // Crank-Nicolson: the step's old-time derivative and theta
            c.thetaOld.alloc(n6);
            RT_CUDA(cudaMemcpyAsync(c.thetaOld.p, c.theta.p, sizeof(double) * n6, cudaMemcpyDeviceToDevice,
                                    ctx->stream));
            c.thetaOldSaved = true;
        }
        RT_REQUIRE(c.thetaOldSaved && c.thetaOld.p && c.thetaOld.n == n6, RT_ENOTREADY,
                   "no old-time theta: the first call of a time step needs newTimeStep = 1");
        DBuf<double> g;
        if (gradU) upload_soa(ctx, gradU, ctx->mesh.N, 9, g);
        rt_status st = constitutive_correct(ctx, gradU ? g.p : nullptr, thetaPerf, c.thetaOld.p);
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        return st;
    });
}

// rheoHeatFoam's constEq.correct() (rheoHeatFoam.C:144,189): the cell
// temperatures and each mode's thermoFunctions give per-cell factors of the
// relaxation times and etaP, computed here on the device; constitutive_correct
// applies them while thermoOn
rt_status rt_set_temperature(rt_ctx *ctx, const rt_thermo_desc *modes, const double *T) {
    return guarded(ctx, [&]() -> rt_status {
        DevCase &c = ctx->cs;
        RT_REQUIRE(c.ready, RT_ENOTREADY, "case not set up");
        if (!T) {
            c.thermoOn = false;
            return RT_OK;
        }
        RT_REQUIRE(modes, RT_EINVAL, "null thermoFunction descriptors");
        RT_REQUIRE(ctx->mesh.batch.n <= 1, RT_EINVAL, "temperature-dependent parameters: not in the batched form");
        const int N = ctx->mesh.N;
        for (int i = 0; i < c.nModes; ++i) {
            const rt_thermo_fn *fns[3] = {&modes[i].lambda, &modes[i].lambda2, &modes[i].eta};
            for (const rt_thermo_fn *f : fns) {
                RT_REQUIRE(f->type >= RT_THERMO_CONSTANT && f->type <= RT_THERMO_VFT, RT_EINVAL,
                           "unknown thermoFunction type " + std::to_string(f->type));
                RT_REQUIRE(f->type != RT_THERMO_ARRHENIUS || f->T0 > 0, RT_EINVAL, "Arrhenius needs T0 > 0");
            }
        }
        for (int cell = 0; cell < N; ++cell) {
            const double t = T[cell];
            RT_REQUIRE(std::isfinite(t), RT_EINVAL, "temperature of cell " + std::to_string(cell) + " is not finite");
            for (int i = 0; i < c.nModes; ++i) {
                const rt_thermo_fn *fns[3] = {&modes[i].lambda, &modes[i].lambda2, &modes[i].eta};
                for (const rt_thermo_fn *f : fns) {
                    const bool ok = (f->type == RT_THERMO_ARRHENIUS) ? t > 0
                                    : (f->type == RT_THERMO_WLF)     ? f->c2 + (t - f->T0) != 0.0
                                    : (f->type == RT_THERMO_VFT)     ? t - f->T0 != 0.0
                                                                     : true;
                    RT_REQUIRE(ok, RT_EINVAL,
                               "temperature of cell " + std::to_string(cell) + " outside a thermoFunction's domain");
                }
            }
        }
        c.Tcell.alloc((size_t)N);
        RT_CUDA(cudaMemcpyAsync(c.Tcell.p, T, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream));
        for (int i = 0; i < c.nModes; ++i) {
            DBuf<double> &out = i == 0 ? c.thermo : c.modes[i - 1]->thermo;
            out.alloc(3 * (size_t)N);
            thermo_factors(ctx, modes[i], c.Tcell.p, out.p);
        }
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        c.thermoOn = true;
        return RT_OK;
    });
}

rt_status rt_step(rt_ctx *ctx, int32_t nSteps, rt_step_perf *perf) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->cs.ready, RT_ENOTREADY, "case not set up");
        RT_REQUIRE(nSteps >= 0, RT_EINVAL, "nSteps must be >= 0");
        RT_REQUIRE(!ctx->cs.thermoOn, RT_EINVAL,
                   "a temperature is set: the momentum equation's temperature-dependent viscosities are not "
                   "built, so temperature-dependent parameters apply to rt_constitutive_correct only");
        rt_step_perf local{};
        rt_status st = RT_OK;
        // the steps advance theta: an old-time theta kept by
        // rt_constitutive_correct_iter no longer belongs to the current step
        if (nSteps > 0) ctx->cs.thetaOldSaved = false;
        for (int i = 0; i < nSteps && st == RT_OK; ++i) {
            local = rt_step_perf{};
            st = step_once(ctx, &local);
        }
        if (perf) *perf = local;
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        return st;
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batches of independent cases
// ---------------------------------------------------------------------------
rt_status rt_batch_layout(rt_ctx *ctx, int32_t nCases, const int32_t *cellStart, const int32_t *faceStart,
                          const int32_t *bFaceStart, const int32_t *dims, const int32_t *cellIJK) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(ctx->meshReady, RT_ENOTREADY, "mesh not uploaded");
        RT_REQUIRE(nCases >= 1 && cellStart && faceStart && bFaceStart, RT_EINVAL, "null argument");
        DevMesh &m = ctx->mesh;
        Batch &b = m.batch;
        const int N = m.N, F = m.F, NB = m.NB, n = nCases;
        RT_REQUIRE(!m.hasCoupled, RT_EINVAL, "batches of cases with coupled (cyclic) faces are not supported");
        RT_REQUIRE(cellStart[0] == 0 && cellStart[n] == N && faceStart[0] == 0 && faceStart[n] == F &&
                       bFaceStart[0] == 0 && bFaceStart[n] == NB,
                   RT_EINVAL, "case ranges must cover the cells, faces and boundary faces");
        for (int c = 0; c < n; ++c)
            RT_REQUIRE(cellStart[c + 1] > cellStart[c] && faceStart[c + 1] >= faceStart[c] &&
                           bFaceStart[c + 1] >= bFaceStart[c],
                       RT_EINVAL, "case ranges must increase (every case owns a cell)");
        // every face lies inside its case
        std::vector<int> own(F), nei(F), bc(NB);
        if (F) {
            RT_CUDA(cudaMemcpy(own.data(), m.owner.p, sizeof(int) * F, cudaMemcpyDeviceToHost));
            RT_CUDA(cudaMemcpy(nei.data(), m.neighbour.p, sizeof(int) * F, cudaMemcpyDeviceToHost));
        }
        if (NB) RT_CUDA(cudaMemcpy(bc.data(), m.bCell.p, sizeof(int) * NB, cudaMemcpyDeviceToHost));
        std::vector<int> caseOf(N);
        for (int c = 0; c < n; ++c)
            for (int i = cellStart[c]; i < cellStart[c + 1]; ++i) caseOf[i] = c;
        for (int c = 0; c < n; ++c) {
            for (int f = faceStart[c]; f < faceStart[c + 1]; ++f)
                RT_REQUIRE(caseOf[own[f]] == c && caseOf[nei[f]] == c, RT_EINVAL,
                           "face " + std::to_string(f) + " leaves its case");
            for (int f = bFaceStart[c]; f < bFaceStart[c + 1]; ++f)
                RT_REQUIRE(caseOf[bc[f]] == c, RT_EINVAL, "boundary face " + std::to_string(f) + " leaves its case");
        }
        b.n = 1;   // until the layout is complete
        b.cellStartH.assign(cellStart, cellStart + n + 1);
        b.faceStartH.assign(faceStart, faceStart + n + 1);
        b.bStartH.assign(bFaceStart, bFaceStart + n + 1);
        upload_vec(ctx, caseOf, b.caseOf);
        upload_vec(ctx, b.cellStartH, b.cellStartD);
        upload_vec(ctx, b.faceStartH, b.faceStartD);
        upload_vec(ctx, b.bStartH, b.bStartD);
        // reduction blocks of RT_BLOCK cells that never straddle two cases
        std::vector<int> bcase, bc0, bc1, cblk(n + 1, 0);
        for (int c = 0; c < n; ++c) {
            cblk[c] = (int)bcase.size();
            for (int i = cellStart[c]; i < cellStart[c + 1]; i += RT_BLOCK) {
                bcase.push_back(c);
                bc0.push_back(i);
                bc1.push_back(std::min(i + RT_BLOCK, cellStart[c + 1]));
            }
        }
        cblk[n] = (int)bcase.size();
        b.nBlk = (int)bcase.size();
        b.caseBlkH = cblk;
        upload_vec(ctx, bcase, b.blkCase);
        upload_vec(ctx, bc0, b.blkCell0);
        upload_vec(ctx, bc1, b.blkCell1);
        upload_vec(ctx, cblk, b.caseBlk);
        {   // the order one-CTA-per-case launches take the cases in: largest first
            std::vector<int> order(n);
            std::iota(order.begin(), order.end(), 0);
            std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
                return cellStart[a + 1] - cellStart[a] > cellStart[c + 1] - cellStart[c];
            });
            upload_vec(ctx, order, b.caseOrder);
        }
        // structured 2-D cases: the skewed layout of the batched sweeps
        b.sweep2d = false;
        bool structured = dims && cellIJK;
        for (int c = 0; structured && c < n; ++c)
            structured = dims[3 * c] > 0 && dims[3 * c + 1] > 0 && dims[3 * c + 1] <= 1024 && dims[3 * c + 2] == 1;
        if (structured) {
            std::vector<int> lo((size_t)2 * N, -1), hi((size_t)2 * N, -1);
            std::vector<int> sT(n), sJB(n);
            std::vector<long long> sOff(n);
            long long nSkew = 0;
            int maxJB = 0;
            for (int c = 0; c < n; ++c) {
                const int nx = dims[3 * c], ny = dims[3 * c + 1];
                sJB[c] = (ny + 31) / 32;
                sT[c] = ((nx + 31 + 7) / 8) * 8;
                sOff[c] = nSkew;
                nSkew += (long long)sJB[c] * sT[c] * 32;
                maxJB = std::max(maxJB, sJB[c]);
            }
            std::vector<int> cellOf((size_t)nSkew, -1);
            // the multigrid hierarchy of each case (the mixed pressure and
            // momentum solves): its boxes down to at most kBatchMgCoarse
            // cells, their offsets in one pool, and level 0's cell of each box
            // position
            std::vector<int> mgDims((size_t)n * kBatchMgLevels * 2, 0), mgNL(n, 0), mgCell;
            std::vector<long long> mgOff((size_t)n * kBatchMgLevels, 0), mgCellOff(n, 0);
            long long mgTotal = 0;
            for (int c = 0; c < n; ++c) {
                int nx = dims[3 * c], ny = dims[3 * c + 1];
                for (int l = 0; l < kBatchMgLevels; ++l) {
                    mgDims[((size_t)c * kBatchMgLevels + l) * 2] = nx;
                    mgDims[((size_t)c * kBatchMgLevels + l) * 2 + 1] = ny;
                    mgOff[(size_t)c * kBatchMgLevels + l] = mgTotal;
                    mgTotal += kBatchMgArrays * (((long long)nx * ny + 3) / 4 * 4);
                    mgNL[c] = l + 1;
                    if ((long long)nx * ny <= kBatchMgCoarse) break;
                    nx = (nx + 1) / 2;
                    ny = (ny + 1) / 2;
                }
            }
            for (int c = 0; structured && c < n; ++c) {
                const int nx = dims[3 * c], ny = dims[3 * c + 1];
                std::vector<int> at((size_t)nx * ny, -1);
                long long prev = -1;
                for (int i = cellStart[c]; i < cellStart[c + 1]; ++i) {
                    const int ci = cellIJK[3 * i], cj = cellIJK[3 * i + 1], ck = cellIJK[3 * i + 2];
                    if (ci < 0 || ci >= nx || cj < 0 || cj >= ny || ck != 0) { structured = false; break; }
                    const long long key = (long long)cj * nx + ci;
                    if (key <= prev) { structured = false; break; }
                    prev = key;
                    at[(size_t)key] = i;
                }
                for (int f = faceStart[c]; structured && f < faceStart[c + 1]; ++f) {
                    const int o = own[f], ne = nei[f];
                    const int di = cellIJK[3 * ne] - cellIJK[3 * o], dj = cellIJK[3 * ne + 1] - cellIJK[3 * o + 1];
                    const int dir = (di == 0 && dj == 1) ? 0 : (di == 1 && dj == 0) ? 1 : -1;   // 0 y, 1 x
                    if (dir < 0 || hi[(size_t)dir * N + o] >= 0 || lo[(size_t)dir * N + ne] >= 0) {
                        structured = false;
                        break;
                    }
                    hi[(size_t)dir * N + o] = f;
                    lo[(size_t)dir * N + ne] = f;
                }
                for (int jb = 0; structured && jb < sJB[c]; ++jb)
                    for (int t = 0; t < sT[c]; ++t)
                        for (int l = 0; l < 32; ++l) {
                            const int i = t - l, j = jb * 32 + l;
                            if (i < 0 || i >= nx || j >= ny) continue;
                            cellOf[(size_t)(sOff[c] + ((long long)jb * sT[c] + t) * 32 + l)] = at[(size_t)j * nx + i];
                        }
                mgCellOff[c] = (long long)mgCell.size();
                mgCell.insert(mgCell.end(), at.begin(), at.end());
            }
            if (structured) {
                b.nSkew = nSkew;
                b.maxJB = maxJB;
                upload_vec(ctx, sT, b.sT);
                upload_vec(ctx, sJB, b.sJB);
                upload_vec(ctx, sOff, b.sOff);
                upload_vec(ctx, cellOf, b.sCell);
                upload_vec(ctx, lo, b.sFaceLo);
                upload_vec(ctx, hi, b.sFaceHi);
                b.sData64.alloc((size_t)21 * nSkew);
                b.sData64.zero(ctx->stream);
                b.sData32.alloc((size_t)17 * nSkew);
                b.sData32.zero(ctx->stream);
                upload_vec(ctx, mgDims, b.mgDims);
                upload_vec(ctx, mgNL, b.mgNL);
                upload_vec(ctx, mgOff, b.mgOff);
                upload_vec(ctx, mgCellOff, b.mgCellOff);
                upload_vec(ctx, mgCell, b.mgCell);
                b.mgPool.alloc((size_t)mgTotal);
                b.sweep2d = true;
            }
        }
        b.sErr.alloc(1);
        b.sErr.zero(ctx->stream);
        const size_t nSeg = (size_t)8 * n;
        b.segD.alloc(12 * nSeg);
        b.segD.zero(ctx->stream);
        b.segI.alloc(6 * nSeg + 8);
        b.segI.zero(ctx->stream);
        b.bPartial.alloc((size_t)2 * 6 * b.nBlk);
        b.bRes.alloc(4 * nSeg);
        if (!b.hostCount) RT_CUDA(cudaMallocHost(&b.hostCount, sizeof(int)));
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        b.n = n;
        ctx->batchPerf.assign(n, rt_step_perf{});
        ctx->cs.ready = false;
        ctx->cs.thermoOn = false;
        return RT_OK;
    });
}

rt_status rt_batch_case_setup(rt_ctx *ctx, const rt_bc_desc *bcs, const rt_model_params *models,
                              const rt_case_ctl *ctl, const int32_t *pRefCell, const double *pRefValue) {
    rt_status st = RT_OK;
    {
        rt_status v = guarded(ctx, [&]() -> rt_status {
            RT_REQUIRE(ctx->meshReady && ctx->mesh.batch.n >= 1, RT_ENOTREADY, "mesh not uploaded");
            RT_REQUIRE(bcs && models && ctl && pRefCell && pRefValue, RT_EINVAL, "null argument");
            RT_REQUIRE(ctl->ddtScheme == RT_DDT_EULER, RT_EINVAL, "the batched form runs the Euler ddt scheme");
            const Batch &b = ctx->mesh.batch;
            for (int c = 0; c < b.n; ++c) {
                const rt_model_params &mp = models[c];
                RT_REQUIRE(mp.model >= RT_MODEL_OLDROYDB_LOG && mp.model <= RT_MODEL_WHITEMETZNERCY_LOG, RT_EINVAL,
                           "case " + std::to_string(c) + ": unknown constitutive model");
                RT_REQUIRE(mp.model != RT_MODEL_ROLIEPOLY_LOG || mp.lambdaR > 0, RT_EINVAL,
                           "case " + std::to_string(c) + ": Rolie-Poly needs lambdaR > 0");
                RT_REQUIRE(mp.model != RT_MODEL_XPOMPOM_LOG || (mp.lambdaS > 0 && mp.q > 0), RT_EINVAL,
                           "case " + std::to_string(c) + ": XPomPom needs lambdaS > 0 and q > 0");
                RT_REQUIRE(mp.model != RT_MODEL_WHITEMETZNERCY_LOG || mp.a > 0, RT_EINVAL,
                           "case " + std::to_string(c) + ": WhiteMetznerCY needs a > 0");
                RT_REQUIRE(mp.model != RT_MODEL_PTT_LOG || mp.pttFunction == RT_PTT_LINEAR ||
                               mp.pttFunction == RT_PTT_EXP,
                           RT_EINVAL, "case " + std::to_string(c) + ": the batched form runs the linear and "
                                      "exponential PTT functions");
                RT_REQUIRE(mp.lambda > 0 && mp.rho > 0, RT_EINVAL,
                           "case " + std::to_string(c) + ": lambda and rho must be positive");
                RT_REQUIRE((mp.model != RT_MODEL_FENEP_LOG && mp.model != RT_MODEL_FENECR_LOG) || mp.L2 > 3.0, RT_EINVAL,
                           "case " + std::to_string(c) + ": FENE-P and FENE-CR need L2 > 3");
                RT_REQUIRE(pRefCell[c] < 0 || (pRefCell[c] >= b.cellStartH[c] && pRefCell[c] < b.cellStartH[c + 1]),
                           RT_EINVAL, "case " + std::to_string(c) + ": pRefCell outside the case");
            }
            return RT_OK;
        });
        if (v != RT_OK) return v;
    }
    rt_case_ctl c1 = *ctl;
    c1.needReference = 0;
    c1.pRefCell = 0;
    if (ctx->mesh.batch.n == 1) {
        // a batch of one case runs the single-case path: its own pressure
        // reference goes through the case control
        c1.needReference = pRefCell[0] >= 0 ? 1 : 0;
        c1.pRefCell = pRefCell[0] >= 0 ? pRefCell[0] : 0;
        c1.pRefValue = pRefValue[0];
    }
    st = rt_case_setup(ctx, bcs, &models[0], &c1);
    if (st != RT_OK) return st;
    return guarded(ctx, [&]() -> rt_status {
        Batch &b = ctx->mesh.batch;
        std::vector<rt_model_params> mp(models, models + b.n);
        std::vector<int> rc(pRefCell, pRefCell + b.n);
        std::vector<double> rv(pRefValue, pRefValue + b.n);
        upload_vec(ctx, mp, b.params);
        upload_vec(ctx, rc, b.refCell);
        upload_vec(ctx, rv, b.refValue);
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->batchPerf.assign(b.n, rt_step_perf{});
        return RT_OK;
    });
}

rt_status rt_batch_step_perf(rt_ctx *ctx, rt_step_perf *perf) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(perf, RT_EINVAL, "null argument");
        RT_REQUIRE(ctx->mesh.batch.n > 1 && (int)ctx->batchPerf.size() == ctx->mesh.batch.n, RT_ENOTREADY,
                   "no batch layout");
        for (int c = 0; c < ctx->mesh.batch.n; ++c) perf[c] = ctx->batchPerf[c];
        return RT_OK;
    });
}

rt_status rt_device_bytes(int64_t *bytes) {
    if (!bytes) return RT_EINVAL;
    *bytes = (int64_t)device_bytes().load();
    return RT_OK;
}

rt_status rt_sweep_schedule(rt_ctx *ctx, int32_t *schedule) {
    return guarded(ctx, [&]() -> rt_status {
        RT_REQUIRE(schedule, RT_EINVAL, "null argument");
        const StructMesh &s = ctx->mesh.sm;
        static const int P[5] = {8, 8, 16, 16, 4}, NB[5] = {3, 5, 3, 4, 6};
        for (int i = 0; i < 2; ++i) {
            const int k = s.tune[i];
            schedule[3 * i] = k;
            schedule[3 * i + 1] = k >= 0 ? P[k] : 0;
            schedule[3 * i + 2] = k >= 0 ? NB[k] : 0;
        }
        return RT_OK;
    });
}
