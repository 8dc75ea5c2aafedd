// constitutive.cu — log-conformation constitutive update on the device:
// boilerLog.H (M = R^T L^T R, decomposeGradU), the Oldroyd-B / Giesekus /
// PTT / FENE-P sources, the theta equation (Euler + GaussDefCmpw, six
// components solved in lock step with PBiCGStab-DILU), calcEig (cyclic Jacobi,
// eigenvalues ascending, exp of the eigenvalues) and tau with its
// linearExtrapolation wall values.
//   rheoTool: constitutiveEq.C:323-428 (decomposeGradU, calcEig),
//             utils/boilerLog.H:1-36, Oldroyd_BLog.C:127-179,
//             GiesekusLog.C:128-176, PTTLog.C:176-268, FENE_PLog.C:128-182,
//             linearExtrapolationFvPatchField.C:102-150.
#include <cmath>

#include "fv_device.cuh"
#include "fv_ops.h"

namespace rt {

// ---------------------------------------------------------------------------
// 3x3 tensors in registers (row-major)
// ---------------------------------------------------------------------------
struct T3 {
    double a[9];
};

__device__ __forceinline__ T3 mul(const T3 &A, const T3 &B) {
    T3 C;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C.a[3 * i + j] = A.a[3 * i] * B.a[j] + A.a[3 * i + 1] * B.a[3 + j] + A.a[3 * i + 2] * B.a[6 + j];
    return C;
}
__device__ __forceinline__ T3 tr(const T3 &A) {
    T3 B;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B.a[3 * i + j] = A.a[3 * j + i];
    return B;
}
__device__ __forceinline__ T3 dg(double x, double y, double z) {
    T3 A;
#pragma unroll
    for (int i = 0; i < 9; ++i) A.a[i] = 0.0;
    A.a[0] = x; A.a[4] = y; A.a[8] = z;
    return A;
}
__device__ __forceinline__ T3 load9(const double *__restrict__ p, int n, int c) {
    T3 A;
#pragma unroll
    for (int i = 0; i < 9; ++i) A.a[i] = p[(size_t)i * n + c];
    return A;
}

// ---------------------------------------------------------------------------
// cyclic Jacobi on a symmetric 3x3 (same sweep order, skip rule and sort as
// the FP64 oracle)
// ---------------------------------------------------------------------------
template <int P, int Q>
__device__ __forceinline__ void jrot(double A[3][3], double R[3][3]) {
    constexpr int K = 3 - P - Q;
    double apq = A[P][Q];
    if (fabs(apq) <= 1e-18 * (fabs(A[P][P]) + fabs(A[Q][Q]))) {
        A[P][Q] = A[Q][P] = 0.0;
        return;
    }
    double th = (A[Q][Q] - A[P][P]) / (2.0 * apq);
    double t = 1.0 / (fabs(th) + sqrt(th * th + 1.0));
    if (th < 0.0) t = -t;
    double c = 1.0 / sqrt(t * t + 1.0);
    double s = t * c;
    double app = A[P][P], aqq = A[Q][Q];
    A[P][P] = app - t * apq;
    A[Q][Q] = aqq + t * apq;
    A[P][Q] = A[Q][P] = 0.0;
    double akp = A[K][P], akq = A[K][Q];
    A[K][P] = A[P][K] = c * akp - s * akq;
    A[K][Q] = A[Q][K] = s * akp + c * akq;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double rp = R[i][P], rq = R[i][Q];
        R[i][P] = c * rp - s * rq;
        R[i][Q] = s * rp + c * rq;
    }
}

__device__ __forceinline__ void eig3(const double s[6], double mu[3], double V[9]) {
    double A[3][3] = {{s[0], s[1], s[2]}, {s[1], s[3], s[4]}, {s[2], s[4], s[5]}};
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 12; ++sweep) {
        double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
        if (off == 0.0) break;
        jrot<0, 1>(A, R);
        jrot<0, 2>(A, R);
        jrot<1, 2>(A, R);
    }
    double e[3] = {A[0][0], A[1][1], A[2][2]};
    int i0 = 0, i1 = 1, i2 = 2, t;
    // bubble sort of three, strict comparisons (stable)
    if (e[i0] > e[i1]) { t = i0; i0 = i1; i1 = t; }
    if (e[i1] > e[i2]) { t = i1; i1 = i2; i2 = t; }
    if (e[i0] > e[i1]) { t = i0; i0 = i1; i1 = t; }
    int id[3] = {i0, i1, i2};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        int q = id[j];
        mu[j] = q == 0 ? e[0] : (q == 1 ? e[1] : e[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) V[3 * i + j] = q == 0 ? R[i][0] : (q == 1 ? R[i][1] : R[i][2]);
    }
}

__global__ void k_eig(int n, const double *__restrict__ theta, double *__restrict__ ev,
                      double *__restrict__ vec) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double s[6], mu[3], V[9];
#pragma unroll
    for (int q = 0; q < 6; ++q) s[q] = theta[(size_t)q * n + c];
    eig3(s, mu, V);
#pragma unroll
    for (int k = 0; k < 3; ++k) ev[(size_t)k * n + c] = exp(mu[k]);
#pragma unroll
    for (int i = 0; i < 9; ++i) vec[(size_t)i * n + c] = V[i];
}

void eig_cells(rt_ctx *ctx, int n, const double *theta, double *eigVals, double *eigVecs) {
    k_eig<<<nblocks(n), RT_BLOCK, 0, ctx->stream>>>(n, theta, eigVals, eigVecs);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

// ---------------------------------------------------------------------------
// theta source: rhs = symm(Omega theta - theta Omega + 2B + S_model)
// ---------------------------------------------------------------------------
__global__ void k_theta_rhs(int N, rt_model_params mp, const double *__restrict__ L,
                            const double *__restrict__ Rv, const double *__restrict__ evv,
                            const double *__restrict__ theta, double *__restrict__ rhs,
                            double *__restrict__ fP) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const double lambda = mp.lambda;
    const double zeta = (mp.model == RT_MODEL_PTT_LOG) ? mp.zeta : 0.0;
    T3 Lc = load9(L, N, c), R = load9(Rv, N, c);
    double e0 = evv[c], e1 = evv[N + c], e2 = evv[2 * N + c];
    T3 Lt = tr(Lc);
    if (mp.model == RT_MODEL_PTT_LOG) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                Lt.a[3 * i + j] = Lt.a[3 * i + j] - zeta * (0.5 * (Lc.a[3 * i + j] + Lc.a[3 * j + i]));
    }
    T3 Rt = tr(R);
    T3 M = mul(mul(Rt, Lt), R);
    T3 om = dg(0.0, 0.0, 0.0), Bt = dg(M.a[0], M.a[4], M.a[8]);
    om.a[1] = (e1 * M.a[1] + e0 * M.a[3]) / (e1 - e0 + 1e-16);
    om.a[2] = (e2 * M.a[2] + e0 * M.a[6]) / (e2 - e0 + 1e-16);
    om.a[5] = (e2 * M.a[5] + e1 * M.a[7]) / (e2 - e1 + 1e-16);
    om.a[3] = -om.a[1]; om.a[6] = -om.a[2]; om.a[7] = -om.a[5];
    T3 Om = mul(mul(R, om), Rt);
    T3 B = mul(mul(R, Bt), Rt);
    T3 invm1 = dg(1.0 / e0 - 1.0, 1.0 / e1 - 1.0, 1.0 / e2 - 1.0);
    T3 S;
    if (mp.model == RT_MODEL_OLDROYDB_LOG) {
        S = mul(mul(R, invm1), Rt);
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lambda) * S.a[i];
    } else if (mp.model == RT_MODEL_GIESEKUS_LOG) {
        T3 A = mul(mul(R, dg(e0, e1, e2)), Rt);
        T3 T = mul(mul(R, invm1), Rt);
        T3 ATT = mul(A, mul(T, T));
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lambda) * (T.a[i] - mp.alpha * ATT.a[i]);
    } else if (mp.model == RT_MODEL_PTT_LOG) {
        T3 A = mul(mul(R, dg(e0, e1, e2)), Rt);
        double trA = A.a[0] + A.a[4] + A.a[8];
        T3 T = mul(mul(R, invm1), Rt);
        double fac = (mp.pttFunction == RT_PTT_EXP) ? exp((mp.epsilon / (1.0 - zeta)) * (trA - 3.0))
                                                    : (1.0 + (mp.epsilon / (1.0 - zeta)) * (trA - 3.0));
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = ((1.0 / lambda) * T.a[i]) * fac;
    } else {
        T3 A = mul(mul(R, dg(e0, e1, e2)), Rt);
        double trA = A.a[0] + A.a[4] + A.a[8];
        double f = mp.L2 / (mp.L2 - trA);
        double a = mp.L2 / (mp.L2 - 3.0);
        fP[c] = f;
        T3 D = dg(a * (1.0 / e0) - f, a * (1.0 / e1) - f, a * (1.0 / e2) - f);
        S = mul(mul(R, D), Rt);
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lambda) * S.a[i];
    }
    double th[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) th[q] = theta[(size_t)q * N + c];
    T3 Th;
    Th.a[0] = th[0]; Th.a[1] = th[1]; Th.a[2] = th[2];
    Th.a[3] = th[1]; Th.a[4] = th[3]; Th.a[5] = th[4];
    Th.a[6] = th[2]; Th.a[7] = th[4]; Th.a[8] = th[5];
    T3 OT = mul(Om, Th), TO = mul(Th, Om);
    T3 Ts;
#pragma unroll
    for (int i = 0; i < 9; ++i) Ts.a[i] = OT.a[i] - TO.a[i] + 2.0 * B.a[i] + S.a[i];
    rhs[c] = Ts.a[0];
    rhs[(size_t)N + c] = 0.5 * (Ts.a[1] + Ts.a[3]);
    rhs[(size_t)2 * N + c] = 0.5 * (Ts.a[2] + Ts.a[6]);
    rhs[(size_t)3 * N + c] = Ts.a[4];
    rhs[(size_t)4 * N + c] = 0.5 * (Ts.a[5] + Ts.a[7]);
    rhs[(size_t)5 * N + c] = Ts.a[8];
}

// theta matrix: diag = rDeltaT V + diagC; source = rDeltaT theta0 V + srcC + V rhs;
// complete diagonal/source for the solve (boundary coefficients added)
__global__ void k_theta_assemble(MeshView m, double rDeltaT, const double *__restrict__ diagC,
                                 const double *__restrict__ srcC, const double *__restrict__ theta0,
                                 const double *__restrict__ rhs, const double *__restrict__ intC,
                                 const double *__restrict__ bouC, double *__restrict__ dSolve,
                                 double *__restrict__ bSolve) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const int N = m.N;
    double v = m.V[c];
    double d = (0.0 + rDeltaT * v) + diagC[c];
    double b[6];
#pragma unroll
    for (int k = 0; k < 6; ++k)
        b[k] = ((0.0 + rDeltaT * theta0[(size_t)k * N + c] * v) + srcC[(size_t)k * N + c]) +
               v * rhs[(size_t)k * N + c];
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int bf = m.bList[i];
        d += intC[bf];
#pragma unroll
        for (int k = 0; k < 6; ++k) b[k] += bouC[(size_t)k * m.NB + bf];
    }
    dSolve[c] = d;
#pragma unroll
    for (int k = 0; k < 6; ++k) bSolve[(size_t)k * N + c] = b[k];
}

// tau = c (R Lambda R^T - I)   (FENE-P: c (f R Lambda R^T - a I))
__global__ void k_tau(int N, rt_model_params mp, const double *__restrict__ Rv,
                      const double *__restrict__ evv, const double *__restrict__ fP,
                      double *__restrict__ tau) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    double zeta = (mp.model == RT_MODEL_PTT_LOG) ? mp.zeta : 0.0;
    double cP = mp.etaP / mp.lambda;
    if (mp.model == RT_MODEL_PTT_LOG) cP = mp.etaP / (mp.lambda * (1.0 - zeta));
    T3 R = load9(Rv, N, c);
    T3 A = mul(mul(R, dg(evv[c], evv[N + c], evv[2 * N + c])), tr(R));
    T3 T;
    if (mp.model == RT_MODEL_FENEP_LOG) {
        double a = mp.L2 / (mp.L2 - 3.0);
        double f = fP[c];
#pragma unroll
        for (int i = 0; i < 9; ++i) T.a[i] = f * A.a[i];
        T.a[0] -= a; T.a[4] -= a; T.a[8] -= a;
    } else {
        T = A;
        T.a[0] -= 1.0; T.a[4] -= 1.0; T.a[8] -= 1.0;
    }
    tau[c] = cP * T.a[0];
    tau[(size_t)N + c] = cP * (0.5 * (T.a[1] + T.a[3]));
    tau[(size_t)2 * N + c] = cP * (0.5 * (T.a[2] + T.a[6]));
    tau[(size_t)3 * N + c] = cP * T.a[4];
    tau[(size_t)4 * N + c] = cP * (0.5 * (T.a[5] + T.a[7]));
    tau[(size_t)5 * N + c] = cP * T.a[8];
}

// linearExtrapolation: val = tau_P + grad(tau)_P . (Cf - C_P) for the faces
// [st, st+sz) of one patch, gradient over the current boundary values
__global__ void k_linextrap(MeshView m, int st, int sz, const double *__restrict__ tau,
                            const double *__restrict__ taub, double *__restrict__ val) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sz) return;
    int b = st + i;
    int c = m.bCell[b];
    double ct0 = m.bCtoF[b], ct1 = m.bCtoF[m.NB + b], ct2 = m.bCtoF[2 * m.NB + b];
    for (int q = 0; q < 6; ++q) {
        double g[3];
        cell_grad(m, c, tau + (size_t)q * m.N, taub + (size_t)q * m.NB, g);
        val[(size_t)q * sz + i] = tau[(size_t)q * m.N + c] + (g[0] * ct0 + g[1] * ct1 + g[2] * ct2);
    }
}

__global__ void k_patch_store(int NB, int st, int sz, int nc, const double *__restrict__ val,
                              double *__restrict__ xb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sz) return;
    for (int q = 0; q < nc; ++q) xb[(size_t)q * NB + st + i] = val[(size_t)q * sz + i];
}

__global__ void k_patch_zerograd(int N, int NB, int st, int sz, int nc, const int *__restrict__ bCell,
                                 const double *__restrict__ x, double *__restrict__ xb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sz) return;
    int b = st + i, c = bCell[b];
    for (int q = 0; q < nc; ++q) xb[(size_t)q * NB + b] = x[(size_t)q * N + c];
}

void tau_correct_bc(rt_ctx *ctx, double *valTmp) {
    DevMesh &mesh = ctx->mesh;
    DevCase &cs = ctx->cs;
    MeshView m = view(mesh);
    for (int p = 0; p < mesh.nPatches; ++p) {
        int st = mesh.patchStartH[p], sz = mesh.patchSizeH[p];
        if (sz == 0) continue;
        int kind = cs.kindTau[p];
        if (kind == RT_BC_ZEROGRAD) {
            k_patch_zerograd<<<nblocks(sz), RT_BLOCK, 0, ctx->stream>>>(m.N, m.NB, st, sz, 6, mesh.bCell.p,
                                                                        cs.tau.p, cs.taub.p);
            launch_count(ctx);
        } else if (kind == RT_BC_LINEXTRAP) {
            k_linextrap<<<nblocks(sz), RT_BLOCK, 0, ctx->stream>>>(m, st, sz, cs.tau.p, cs.taub.p, valTmp);
            k_patch_store<<<nblocks(sz), RT_BLOCK, 0, ctx->stream>>>(m.NB, st, sz, 6, valTmp, cs.taub.p);
            launch_count(ctx, 2);
        }
        RT_CHECK_LAUNCH();
    }
}

unsigned theta_valid_mask(const DevMesh &m) {
    int v[3] = {m.solveDir[0] ? 1 : -1, m.solveDir[1] ? 1 : -1, m.solveDir[2] ? 1 : -1};
    const int ij[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    unsigned mask = 0;
    for (int q = 0; q < 6; ++q)
        if (v[ij[q][0]] * v[ij[q][1]] > 0) mask |= 1u << q;
    return mask;
}

rt_status constitutive_correct(rt_ctx *ctx, const double *gradU, rt_solver_perf *perf) {
    DevMesh &mesh = ctx->mesh;
    DevCase &cs = ctx->cs;
    const int N = mesh.N, F = mesh.F, NB = mesh.NB;
    cudaStream_t s = ctx->stream;
    Work &W = ctx->work;
    size_t mark = W.used;
    double *G = const_cast<double *>(gradU);
    if (!G) {
        G = W.take(9 * (size_t)N);
        grad_field(ctx, 3, cs.U.p, cs.Ub.p, G);
    }
    double *rhs = W.take(6 * (size_t)N), *fP = W.take(N), *theta0 = W.take(6 * (size_t)N);
    double *gth = W.take(18 * (size_t)N), *lower = W.take(F), *upper = W.take(F);
    double *diagC = W.take(N), *srcC = W.take(6 * (size_t)N), *intC = W.take(6 * (size_t)NB);
    double *bouC = W.take(6 * (size_t)NB), *flux = W.take(6 * (size_t)F);
    double *dS = W.take(N), *bS = W.take(6 * (size_t)N);
    double *val = W.take(6 * (size_t)NB + 6);

    {
        ProfScope ps(ctx, "theta_rhs", (double)N * (72.0 + 72.0 + 24.0 + 48.0 + 48.0));
        k_theta_rhs<<<nblocks(N), RT_BLOCK, 0, s>>>(N, cs.mp, G, cs.eigVecs.p, cs.eigVals.p, cs.theta.p, rhs, fP);
        RT_CHECK_LAUNCH();
    }
    RT_CUDA(cudaMemcpyAsync(theta0, cs.theta.p, sizeof(double) * 6 * N, cudaMemcpyDeviceToDevice, s));
    const double fpc = (double)F / N;
    {
        ProfScope ps(ctx, "grad", (double)N * (48.0 + fpc * 16.0 + 72.0 + 144.0));
        grad_field(ctx, 6, cs.theta.p, cs.thetab.p, gth);
    }
    {
        ProfScope ps(ctx, "convection", (double)N * (48.0 + 144.0 + 24.0 + fpc * (8.0 + 8.0 + 16.0 + 16.0 + 2 * 48.0) + 8.0 + 48.0));
        convection(ctx, cs.ctl.divTheta, 6, cs.phi.p, cs.phib.p, cs.theta.p, cs.thetab.p, cs.bkTh.p, gth, lower,
                   upper, diagC, srcC, intC, bouC, flux);
    }
    MeshView m = view(mesh);
    k_theta_assemble<<<nblocks(N), RT_BLOCK, 0, s>>>(m, 1.0 / cs.ctl.deltaT, diagC, srcC, theta0, rhs, intC, bouC,
                                                      dS, bS);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 2);
    SolveArgs a{dS, upper, lower, bS, cs.theta.p, 6, theta_valid_mask(mesh), cs.ctl.solverTheta};
    rt_status st;
    {
        ProfScope ps(ctx, "solve_theta");
        st = ldu_solve_device(ctx, a, perf);
    }
    correct_bc(ctx, cs.bkTh.p, 6, cs.theta.p, cs.thetab.p);
    {
        ProfScope ps(ctx, "eig", (double)N * (48.0 + 72.0 + 24.0));
        eig_cells(ctx, N, cs.theta.p, cs.eigVals.p, cs.eigVecs.p);
    }
    {
        ProfScope ps(ctx, "tau", (double)N * (72.0 + 24.0 + 48.0));
        k_tau<<<nblocks(N), RT_BLOCK, 0, s>>>(N, cs.mp, cs.eigVecs.p, cs.eigVals.p, fP, cs.tau.p);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
        tau_correct_bc(ctx, val);
    }
    W.used = mark;
    return st;
}

}  // namespace rt
