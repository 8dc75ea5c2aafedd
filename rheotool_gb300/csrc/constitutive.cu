// constitutive.cu — log-conformation constitutive update on the device:
// the per-cell sources and tau of constitutive_cell.cuh (decomposeGradU and
// the eight log models), the theta equation (Euler + GaussDefCmpw, six
// components solved in lock step with PBiCGStab-DILU), calcEig (cyclic Jacobi,
// eigenvalues ascending, exp of the eigenvalues) and tau with its
// linearExtrapolation wall values.
//   rheoTool: constitutiveEq.C:323-428 (decomposeGradU, calcEig),
//             utils/boilerLog.H:1-36, Oldroyd_BLog.C:127-179,
//             GiesekusLog.C:128-176, PTTLog.C:176-268, FENE_PLog.C:128-182,
//             linearExtrapolationFvPatchField.C:102-150.
#include <cmath>

#include "constitutive_cell.cuh"
#include "fv_device.cuh"
#include "fv_ops.h"

namespace rt {

// ---------------------------------------------------------------------------
// cyclic Jacobi on a symmetric 3x3 (same sweep order, skip rule and sort as
// the FP64 oracle).  FP32 instances (mixed precision) skip a rotation once
// |a_pq| is below 1e-10 of the diagonal pair, far below what FP32 resolves.
// ---------------------------------------------------------------------------
template <class Real> struct JacobiSkip;
template <> struct JacobiSkip<double> { static constexpr double v = 1e-18; };
template <> struct JacobiSkip<float> { static constexpr float v = 1e-10f; };

template <int P, int Q, class Real>
__device__ __forceinline__ void jrot(Real A[3][3], Real R[3][3]) {
    constexpr int K = 3 - P - Q;
    Real apq = A[P][Q];
    if (fabs(apq) <= JacobiSkip<Real>::v * (fabs(A[P][P]) + fabs(A[Q][Q]))) {
        A[P][Q] = A[Q][P] = Real(0);
        return;
    }
    Real th = (A[Q][Q] - A[P][P]) / (Real(2) * apq);
    Real t = Real(1) / (fabs(th) + sqrt(th * th + Real(1)));
    if (th < Real(0)) t = -t;
    Real c = Real(1) / sqrt(t * t + Real(1));
    Real s = t * c;
    Real app = A[P][P], aqq = A[Q][Q];
    A[P][P] = app - t * apq;
    A[Q][Q] = aqq + t * apq;
    A[P][Q] = A[Q][P] = Real(0);
    Real akp = A[K][P], akq = A[K][Q];
    A[K][P] = A[P][K] = c * akp - s * akq;
    A[K][Q] = A[Q][K] = s * akp + c * akq;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Real rp = R[i][P], rq = R[i][Q];
        R[i][P] = c * rp - s * rq;
        R[i][Q] = s * rp + c * rq;
    }
}

template <class Real>
__device__ __forceinline__ void eig3(const Real s[6], Real mu[3], Real V[9]) {
    Real A[3][3] = {{s[0], s[1], s[2]}, {s[1], s[3], s[4]}, {s[2], s[4], s[5]}};
    Real R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 12; ++sweep) {
        Real off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
        if (off == Real(0)) break;
        jrot<0, 1>(A, R);
        jrot<0, 2>(A, R);
        jrot<1, 2>(A, R);
    }
    Real e[3] = {A[0][0], A[1][1], A[2][2]};
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

// ---- temperature-dependent parameters (rt_set_temperature) ----------------
// The shift factor of a thermoFunction at temperature T (thermoFunctions/
// <type>/<type>.C, multiply()): Constant 1; Arrhenius exp(alpha (1/T -
// 1/T0)); ArrheniusModified exp(-alpha (T - T0)); WLF 10^(-c1 (T - T0) /
// (c2 + (T - T0))); VFT 10^(B + A / (T - T0)).
__device__ double thermo_factor(const rt_thermo_fn &f, double T) {
    switch (f.type) {
    case RT_THERMO_ARRHENIUS: return exp(f.alpha * (1.0 / T - 1.0 / f.T0));
    case RT_THERMO_ARRHENIUS_MODIFIED: return exp(-f.alpha * (T - f.T0));
    case RT_THERMO_WLF: return pow(10.0, -f.c1 * (T - f.T0) / (f.c2 + (T - f.T0)));
    case RT_THERMO_VFT: return pow(10.0, f.B + f.A / (T - f.T0));
    default: return 1.0;
    }
}

// one mode's factors: lambda, the second relaxation time, etaP (3 N)
__global__ void k_thermo_factors(int N, rt_thermo_desc d, const double *__restrict__ T, double *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const double t = T[c];
    out[c] = thermo_factor(d.lambda, t);
    out[(size_t)N + c] = thermo_factor(d.lambda2, t);
    out[(size_t)2 * N + c] = thermo_factor(d.eta, t);
}

// a cell's model with its relaxation times and etaP shifted (the Log
// models' createField(lambda_), createField(etaP_): Oldroyd_BLog.C:133-135;
// Rolie-Poly lambdaD / lambdaR, XPomPom lambdaB / lambdaS by their own
// functions: RoliePolyLog.C:139-141, XPomPomLog.C:140-142)
__device__ __forceinline__ void thermo_shift(rt_model_params &m, const double *__restrict__ th, int N, int c) {
    m.lambda = m.lambda * th[c];
    m.lambdaR = m.lambdaR * th[(size_t)N + c];
    m.lambdaS = m.lambdaS * th[(size_t)N + c];
    m.etaP = m.etaP * th[(size_t)2 * N + c];
}

void thermo_factors(rt_ctx *ctx, const rt_thermo_desc &d, const double *T, double *out) {
    const int N = ctx->mesh.N;
    k_thermo_factors<<<nblocks(N), RT_BLOCK, 0, ctx->stream>>>(N, d, T, out);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

// th: the shift factors (3 N) or null
__global__ void k_theta_rhs(int N, rt_model_params mp, const int *__restrict__ caseOf,
                            const rt_model_params *__restrict__ cp, const double *__restrict__ L,
                            const double *__restrict__ Rv, const double *__restrict__ evv,
                            const double *__restrict__ theta, double *__restrict__ rhs,
                            double *__restrict__ fP, const double *__restrict__ mlg, int mlK,
                            const double *__restrict__ th) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const rt_model_params &m0 = caseOf ? cp[caseOf[c]] : mp;
    if (th) {
        rt_model_params m = m0;
        thermo_shift(m, th, N, c);
        theta_rhs_cell(c, N, m, L, Rv, evv, theta, rhs, fP, mlg, mlK);
    } else {
        theta_rhs_cell(c, N, m0, L, Rv, evv, theta, rhs, fP, mlg, mlK);
    }
}

// theta matrix: diag = rDeltaT V + diagC; source = rDeltaT theta0 V + srcC + V rhs;
// complete diagonal/source for the solve (boundary coefficients added)
// (Dth non-null: Crank-Nicolson, rDeltaT = c/dt and the source ((c/dt)
// theta0 + psi Dth) V; else Euler)
__global__ void k_theta_assemble(MeshView m, double rDeltaT, const double *__restrict__ diagC,
                                 const double *__restrict__ srcC, const double *__restrict__ theta0,
                                 const double *__restrict__ rhs, const double *__restrict__ intC,
                                 const double *__restrict__ bouC, double *__restrict__ dSolve,
                                 double *__restrict__ bSolve, double psi, const double *__restrict__ Dth) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const int N = m.N;
    double v = m.V[c];
    double d = (0.0 + rDeltaT * v) + diagC[c];
    double b[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const size_t i = (size_t)k * N + c;
        const double ddtSrc = Dth ? (rDeltaT * theta0[i] + psi * Dth[i]) * v : rDeltaT * theta0[i] * v;
        b[k] = ((0.0 + ddtSrc) + srcC[i]) + v * rhs[i];
    }
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

__global__ void k_tau(int N, rt_model_params mp, const int *__restrict__ caseOf,
                      const rt_model_params *__restrict__ cp, const double *__restrict__ Rv,
                      const double *__restrict__ evv, const double *__restrict__ fP,
                      double *__restrict__ tau, const double *__restrict__ th) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const rt_model_params &m0 = caseOf ? cp[caseOf[c]] : mp;
    if (th) {
        rt_model_params m = m0;
        thermo_shift(m, th, N, c);
        tau_cell(c, N, m, Rv, evv, fP, tau);
    } else {
        tau_cell(c, N, m0, Rv, evv, fP, tau);
    }
}

// ---------------------------------------------------------------------------
// Mixed precision (RT_PREC_MIXED): the cell-local constitutive update with
// its 3x3 matrix algebra in FP32.  Kept in FP64: the scalar functions of the
// eigenvalues where FP32 would cancel (eigenvalue gaps, 1/e - 1, e - 1,
// tr A - 3 and the FENE-P factors, all from the FP64 exp of the eigenvalues),
// and whole cells whose log-conformation eigenvalues are near-degenerate
// (gap below kMixGap of their magnitude: decomposeGradU divides by the gap)
// or large (|mu| above kMixMuHi, high Wi: exp amplifies the FP32 error of mu);
// those cells run the FP64 code above, bit for bit.  The algebra is
// regrouped so that no FP32 difference of nearly equal numbers remains:
// R (Lambda^-1 - I) R^T and R (Lambda - I) R^T are formed from the FP64
// diagonal differences, which is the same tensor as the reference's
// R Lambda^-1 R^T - I (R is orthogonal) without its cancellation.
// ---------------------------------------------------------------------------
constexpr double kMixGap = 0.1, kMixMuHi = 4.0;

struct F3 {
    float a[9];
};
__device__ __forceinline__ F3 fmul3(const F3 &A, const F3 &B) {
    F3 C;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C.a[3 * i + j] = A.a[3 * i] * B.a[j] + A.a[3 * i + 1] * B.a[3 + j] + A.a[3 * i + 2] * B.a[6 + j];
    return C;
}
__device__ __forceinline__ F3 ftr3(const F3 &A) {
    F3 B;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B.a[3 * i + j] = A.a[3 * j + i];
    return B;
}
__device__ __forceinline__ F3 fload9(const double *__restrict__ p, int n, int c) {
    F3 A;
#pragma unroll
    for (int i = 0; i < 9; ++i) A.a[i] = (float)p[(size_t)i * n + c];
    return A;
}
// R diag(d) R^T
__device__ __forceinline__ F3 frdr(const F3 &R, float d0, float d1, float d2) {
    F3 C;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C.a[3 * i + j] = R.a[3 * i] * d0 * R.a[3 * j] + R.a[3 * i + 1] * d1 * R.a[3 * j + 1] +
                             R.a[3 * i + 2] * d2 * R.a[3 * j + 2];
    return C;
}

// log-conformation eigenvalues (ascending) that FP32 resolves well
__device__ __forceinline__ bool mix_fp32_ok(double m0, double m1, double m2) {
    const double scale = fmax(fabs(m0), fabs(m2));
    const double gap = fmin(m1 - m0, m2 - m1);
    return scale <= kMixMuHi && gap > kMixGap * scale && isfinite(scale);
}

// models whose cell algebra has no FP32 form here (Rolie-Poly, XPomPom,
// WhiteMetznerCY, the generalized PTT function): the mixed kernels run their
// FP64 code for every cell
__device__ __forceinline__ bool mixed_fp64_model(const rt_model_params &mp) {
    return mp.model == RT_MODEL_ROLIEPOLY_LOG || mp.model == RT_MODEL_XPOMPOM_LOG ||
           mp.model == RT_MODEL_WHITEMETZNERCY_LOG ||
           (mp.model == RT_MODEL_PTT_LOG && mp.pttFunction == RT_PTT_GENERALIZED);
}

__global__ void k_eig_mixed(int n, const double *__restrict__ theta, double *__restrict__ ev,
                            double *__restrict__ vec) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    float sf[6], muf[3], Vf[9];
#pragma unroll
    for (int q = 0; q < 6; ++q) sf[q] = (float)theta[(size_t)q * n + c];
    eig3(sf, muf, Vf);
    if (mix_fp32_ok(muf[0], muf[1], muf[2])) {
#pragma unroll
        for (int k = 0; k < 3; ++k) ev[(size_t)k * n + c] = exp((double)muf[k]);
#pragma unroll
        for (int i = 0; i < 9; ++i) vec[(size_t)i * n + c] = (double)Vf[i];
        return;
    }
    double s[6], mu[3], V[9];
#pragma unroll
    for (int q = 0; q < 6; ++q) s[q] = theta[(size_t)q * n + c];
    eig3(s, mu, V);
#pragma unroll
    for (int k = 0; k < 3; ++k) ev[(size_t)k * n + c] = exp(mu[k]);
#pragma unroll
    for (int i = 0; i < 9; ++i) vec[(size_t)i * n + c] = V[i];
}

__device__ __forceinline__ void theta_rhs_mixed_cell(int c, int N, const rt_model_params &mp,
                                                     const double *__restrict__ L, const double *__restrict__ Rv,
                                                     const double *__restrict__ evv,
                                                     const double *__restrict__ theta, double *__restrict__ rhs,
                                                     double *__restrict__ fP, const double *__restrict__ mlg,
                                                     int mlK) {
    const double e0 = evv[c], e1 = evv[N + c], e2 = evv[2 * N + c];
    if (mixed_fp64_model(mp) || !mix_fp32_ok(log(e0), log(e1), log(e2))) {
        theta_rhs_cell(c, N, mp, L, Rv, evv, theta, rhs, fP, mlg, mlK);
        return;
    }
    const float lambdaInv = (float)(1.0 / mp.lambda);
    const float zeta = (mp.model == RT_MODEL_PTT_LOG) ? (float)mp.zeta : 0.0f;
    F3 Lc = fload9(L, N, c), R = fload9(Rv, N, c);
    F3 Lt = ftr3(Lc);
    if (mp.model == RT_MODEL_PTT_LOG) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                Lt.a[3 * i + j] = Lt.a[3 * i + j] - zeta * (0.5f * (Lc.a[3 * i + j] + Lc.a[3 * j + i]));
    }
    const F3 Rt = ftr3(R);
    const F3 M = fmul3(fmul3(Rt, Lt), R);
    const float f0 = (float)e0, f1 = (float)e1, f2 = (float)e2;
    // omega in the eigenbasis; the gaps in FP64
    const float g01 = (float)(e1 - e0 + 1e-16), g02 = (float)(e2 - e0 + 1e-16), g12 = (float)(e2 - e1 + 1e-16);
    F3 om;
#pragma unroll
    for (int i = 0; i < 9; ++i) om.a[i] = 0.0f;
    om.a[1] = (f1 * M.a[1] + f0 * M.a[3]) / g01;
    om.a[2] = (f2 * M.a[2] + f0 * M.a[6]) / g02;
    om.a[5] = (f2 * M.a[5] + f1 * M.a[7]) / g12;
    om.a[3] = -om.a[1]; om.a[6] = -om.a[2]; om.a[7] = -om.a[5];
    const F3 Om = fmul3(fmul3(R, om), Rt);
    const F3 B = frdr(R, M.a[0], M.a[4], M.a[8]);
    // Lambda^-1 - I in FP64
    const float d0 = (float)(1.0 / e0 - 1.0), d1 = (float)(1.0 / e1 - 1.0), d2 = (float)(1.0 / e2 - 1.0);
    F3 S;
    if (mp.model == RT_MODEL_OLDROYDB_LOG) {
        S = frdr(R, d0, d1, d2);
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = lambdaInv * S.a[i];
    } else if (mp.model == RT_MODEL_GIESEKUS_LOG) {
        const F3 A = frdr(R, f0, f1, f2);
        const F3 T = frdr(R, d0, d1, d2);
        const F3 ATT = fmul3(A, fmul3(T, T));
        const float alpha = (float)mp.alpha;
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = lambdaInv * (T.a[i] - alpha * ATT.a[i]);
    } else if (mp.model == RT_MODEL_PTT_LOG) {
        const double trAm3 = (e0 - 1.0) + (e1 - 1.0) + (e2 - 1.0);
        const double x = (mp.epsilon / (1.0 - mp.zeta)) * trAm3;
        const float fac = (float)((mp.pttFunction == RT_PTT_EXP) ? exp(x) : 1.0 + x);
        const F3 T = frdr(R, d0, d1, d2);
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = (lambdaInv * T.a[i]) * fac;
    } else if (mp.model == RT_MODEL_FENECR_LOG) {
        const double trA = e0 + e1 + e2;
        const double f = mp.L2 / (mp.L2 - trA);
        fP[c] = f;
        const float lf = (float)((1.0 / mp.lambda) * f);
        S = frdr(R, d0, d1, d2);
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = lf * S.a[i];
    } else {
        const double trA = e0 + e1 + e2;
        const double f = mp.L2 / (mp.L2 - trA);
        const double a = mp.L2 / (mp.L2 - 3.0);
        fP[c] = f;
        // a / e - f in FP64
        S = frdr(R, (float)(a / e0 - f), (float)(a / e1 - f), (float)(a / e2 - f));
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = lambdaInv * S.a[i];
    }
    float th[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) th[q] = (float)theta[(size_t)q * N + c];
    F3 Th;
    Th.a[0] = th[0]; Th.a[1] = th[1]; Th.a[2] = th[2];
    Th.a[3] = th[1]; Th.a[4] = th[3]; Th.a[5] = th[4];
    Th.a[6] = th[2]; Th.a[7] = th[4]; Th.a[8] = th[5];
    const F3 OT = fmul3(Om, Th), TO = fmul3(Th, Om);
    F3 Ts;
#pragma unroll
    for (int i = 0; i < 9; ++i) Ts.a[i] = OT.a[i] - TO.a[i] + 2.0f * B.a[i] + S.a[i];
    rhs[c] = Ts.a[0];
    rhs[(size_t)N + c] = 0.5f * (Ts.a[1] + Ts.a[3]);
    rhs[(size_t)2 * N + c] = 0.5f * (Ts.a[2] + Ts.a[6]);
    rhs[(size_t)3 * N + c] = Ts.a[4];
    rhs[(size_t)4 * N + c] = 0.5f * (Ts.a[5] + Ts.a[7]);
    rhs[(size_t)5 * N + c] = Ts.a[8];
}

__global__ void k_theta_rhs_mixed(int N, rt_model_params mp0, const int *__restrict__ caseOf,
                                  const rt_model_params *__restrict__ cp, const double *__restrict__ L,
                                  const double *__restrict__ Rv, const double *__restrict__ evv,
                                  const double *__restrict__ theta, double *__restrict__ rhs,
                                  double *__restrict__ fP, const double *__restrict__ mlg, int mlK,
                                  const double *__restrict__ th) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const rt_model_params &m0 = caseOf ? cp[caseOf[c]] : mp0;
    if (th) {
        rt_model_params m = m0;
        thermo_shift(m, th, N, c);
        theta_rhs_mixed_cell(c, N, m, L, Rv, evv, theta, rhs, fP, mlg, mlK);
    } else {
        theta_rhs_mixed_cell(c, N, m0, L, Rv, evv, theta, rhs, fP, mlg, mlK);
    }
}

__device__ __forceinline__ void tau_mixed_cell(int c, int N, const rt_model_params &mp,
                                               const double *__restrict__ Rv, const double *__restrict__ evv,
                                               const double *__restrict__ fP, double *__restrict__ tau) {
    const double e0 = evv[c], e1 = evv[N + c], e2 = evv[2 * N + c];
    if (mixed_fp64_model(mp) || !mix_fp32_ok(log(e0), log(e1), log(e2))) {
        tau_cell(c, N, mp, Rv, evv, fP, tau);
        return;
    }
    double cP = mp.etaP / mp.lambda;
    if (mp.model == RT_MODEL_PTT_LOG) cP = mp.etaP / (mp.lambda * (1.0 - mp.zeta));
    if (mp.model == RT_MODEL_FENECR_LOG) cP = cP * fP[c];
    const F3 R = fload9(Rv, N, c);
    F3 T;
    if (mp.model == RT_MODEL_FENEP_LOG) {
        // f (R Lambda R^T) - a I = f R (Lambda - I) R^T + (f - a) I
        const double a = mp.L2 / (mp.L2 - 3.0);
        const double f = fP[c];
        T = frdr(R, (float)(f * (e0 - 1.0)), (float)(f * (e1 - 1.0)), (float)(f * (e2 - 1.0)));
        const float fa = (float)(f - a);
        T.a[0] += fa; T.a[4] += fa; T.a[8] += fa;
    } else {
        T = frdr(R, (float)(e0 - 1.0), (float)(e1 - 1.0), (float)(e2 - 1.0));
    }
    tau[c] = cP * (double)T.a[0];
    tau[(size_t)N + c] = cP * (double)(0.5f * (T.a[1] + T.a[3]));
    tau[(size_t)2 * N + c] = cP * (double)(0.5f * (T.a[2] + T.a[6]));
    tau[(size_t)3 * N + c] = cP * (double)T.a[4];
    tau[(size_t)4 * N + c] = cP * (double)(0.5f * (T.a[5] + T.a[7]));
    tau[(size_t)5 * N + c] = cP * (double)T.a[8];
}

__global__ void k_tau_mixed(int N, rt_model_params mp0, const int *__restrict__ caseOf,
                            const rt_model_params *__restrict__ cp, const double *__restrict__ Rv,
                            const double *__restrict__ evv, const double *__restrict__ fP,
                            double *__restrict__ tau, const double *__restrict__ th) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const rt_model_params &m0 = caseOf ? cp[caseOf[c]] : mp0;
    if (th) {
        rt_model_params m = m0;
        thermo_shift(m, th, N, c);
        tau_mixed_cell(c, N, m, Rv, evv, fP, tau);
    } else {
        tau_mixed_cell(c, N, m0, Rv, evv, fP, tau);
    }
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

// one wave of a batch: the faces' new values from the current boundary values
// (every face of a wave belongs to another patch than the wave's other faces
// of its case), then stored
__global__ void k_tau_wave(MeshView m, const int *__restrict__ faces, int nf, const int *__restrict__ bk,
                           const double *__restrict__ tau, const double *__restrict__ taub, double *__restrict__ val) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    int b = faces[i];
    int c = m.bCell[b];
    if (bk[b] == RT_BC_ZEROGRAD) {
        for (int q = 0; q < 6; ++q) val[(size_t)q * nf + i] = tau[(size_t)q * m.N + c];
        return;
    }
    double ct0 = m.bCtoF[b], ct1 = m.bCtoF[m.NB + b], ct2 = m.bCtoF[2 * m.NB + b];
    for (int q = 0; q < 6; ++q) {
        double g[3];
        cell_grad(m, c, tau + (size_t)q * m.N, taub + (size_t)q * m.NB, g);
        val[(size_t)q * nf + i] = tau[(size_t)q * m.N + c] + (g[0] * ct0 + g[1] * ct1 + g[2] * ct2);
    }
}

__global__ void k_tau_wave_store(int NB, const int *__restrict__ faces, int nf, const double *__restrict__ val,
                                 double *__restrict__ xb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    for (int q = 0; q < 6; ++q) xb[(size_t)q * NB + faces[i]] = val[(size_t)q * nf + i];
}

void tau_correct_bc(rt_ctx *ctx, double *valTmp) {
    DevMesh &mesh = ctx->mesh;
    DevCase &cs = ctx->cs;
    MeshView m = view(mesh);
    if (!cs.tauWaveH.empty()) {   // a batch: the cases' patches wave by wave
        for (size_t wv = 0; wv + 1 < cs.tauWaveH.size(); ++wv) {
            const int f0 = cs.tauWaveH[wv], nf = cs.tauWaveH[wv + 1] - f0;
            if (nf == 0) continue;
            const int *faces = cs.tauWaveFace.p + f0;
            k_tau_wave<<<nblocks(nf), RT_BLOCK, 0, ctx->stream>>>(m, faces, nf, cs.bkTau.p, cs.tau.p, cs.taub.p,
                                                                 valTmp);
            k_tau_wave_store<<<nblocks(nf), RT_BLOCK, 0, ctx->stream>>>(m.NB, faces, nf, valTmp, cs.taub.p);
            launch_count(ctx, 2);
            RT_CHECK_LAUNCH();
        }
        return;
    }
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

rt_status constitutive_correct(rt_ctx *ctx, const double *gradU, rt_solver_perf *perf, const double *thetaOld) {
    DevMesh &mesh = ctx->mesh;
    DevCase &cs = ctx->cs;
    const int N = mesh.N, F = mesh.F, NB = mesh.NB;
    cudaStream_t s = ctx->stream;
    Work &W = ctx->work;
    WorkMark wmark(W);
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
    const MeshView mv = view(mesh);
    // the shift factors of this mode (rt_set_temperature), or none
    const double *th = cs.thermoOn ? cs.thermo.p : nullptr;

    {
        ProfScope ps(ctx, "theta_rhs", (double)N * (72.0 + 72.0 + 24.0 + 48.0 + 48.0));
        if (cs.ctl.precision == RT_PREC_MIXED && (ctx->mixedParts & 2))
            k_theta_rhs_mixed<<<nblocks(N), RT_BLOCK, 0, s>>>(N, cs.mp, mv.caseOf, mv.caseParams, G, cs.eigVecs.p,
                                                              cs.eigVals.p, cs.theta.p, rhs, fP, cs.mlGamma.p,
                                                              cs.mlK, th);
        else
            k_theta_rhs<<<nblocks(N), RT_BLOCK, 0, s>>>(N, cs.mp, mv.caseOf, mv.caseParams, G, cs.eigVecs.p,
                                                        cs.eigVals.p, cs.theta.p, rhs, fP, cs.mlGamma.p, cs.mlK,
                                                        th);
        RT_CHECK_LAUNCH();
    }
    // (Crank-Nicolson: the old-time theta is the one taken at the step's start)
    const bool cn = cs.ctl.ddtScheme == RT_DDT_CRANKNICOLSON;
    RT_CUDA(cudaMemcpyAsync(theta0, cn ? cs.ths.p : (thetaOld ? thetaOld : cs.theta.p), sizeof(double) * 6 * N,
                            cudaMemcpyDeviceToDevice, s));
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
    k_theta_assemble<<<nblocks(N), RT_BLOCK, 0, s>>>(m, (cn ? cs.ddtCth : 1.0) * (1.0 / cs.ctl.deltaT), diagC, srcC, theta0,
                                                      rhs, intC, bouC, dS, bS, cn ? cs.ctl.ddtPsi : 0.0,
                                                      cn ? cs.Dth.p : nullptr);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 2);
    SolveArgs a{dS, upper, lower, bS, cs.theta.p, 6, theta_valid_mask(mesh), cs.ctl.solverTheta, cs.ctl.precision,
                2};
    rt_status st;
    {
        ProfScope ps(ctx, "solve_theta");
        st = ldu_solve_device(ctx, a, perf);
    }
    correct_bc(ctx, cs.bkTh.p, 6, cs.theta.p, cs.thetab.p);
    {
        ProfScope ps(ctx, "eig", (double)N * (48.0 + 72.0 + 24.0));
        if (cs.ctl.precision == RT_PREC_MIXED && (ctx->mixedParts & 2)) {
            k_eig_mixed<<<nblocks(N), RT_BLOCK, 0, s>>>(N, cs.theta.p, cs.eigVals.p, cs.eigVecs.p);
            RT_CHECK_LAUNCH();
            launch_count(ctx);
        } else {
            eig_cells(ctx, N, cs.theta.p, cs.eigVals.p, cs.eigVecs.p);
        }
    }
    {
        ProfScope ps(ctx, "tau", (double)N * (72.0 + 24.0 + 48.0));
        if (cs.ctl.precision == RT_PREC_MIXED && (ctx->mixedParts & 2))
            k_tau_mixed<<<nblocks(N), RT_BLOCK, 0, s>>>(N, cs.mp, mv.caseOf, mv.caseParams, cs.eigVecs.p,
                                                        cs.eigVals.p, fP, cs.tau.p, th);
        else
            k_tau<<<nblocks(N), RT_BLOCK, 0, s>>>(N, cs.mp, mv.caseOf, mv.caseParams, cs.eigVecs.p, cs.eigVals.p,
                                                  fP, cs.tau.p, th);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
        tau_correct_bc(ctx, val);
    }
    return st;
}

// tauTot = sum over the modes of tau (internal and boundary values)
__global__ void k_add_into(size_t n, const double *__restrict__ a, double *__restrict__ acc, int first) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) acc[i] = first ? a[i] : acc[i] + a[i];
}

// multiMode correct() (multiMode.C:247-256): every mode's correct() in
// turn on the common U and phi, each with its own model, theta, tau and eigen
// fields; then tau() = the sum of the modes' tau (multiMode.C:222)
rt_status modes_correct(rt_ctx *ctx, const double *gradU, rt_solver_perf *perf, const double *theta0s) {
    DevCase &cs = ctx->cs;
    if (cs.nModes <= 1) return constitutive_correct(ctx, gradU, perf, theta0s);
    const int N = ctx->mesh.N, NB = ctx->mesh.NB;
    const size_t n6 = 6 * (size_t)N, b6 = 6 * (size_t)NB;
    cs.modePerf.assign(6 * (size_t)cs.nModes, rt_solver_perf{});
    rt_status st = RT_OK;
    for (int i = 0; i < cs.nModes && st == RT_OK; ++i) {
        ModeSwap sw(cs, i > 0 ? cs.modes[i - 1].get() : nullptr);
        st = constitutive_correct(ctx, gradU, &cs.modePerf[6 * (size_t)i], theta0s ? theta0s + n6 * i : nullptr);
    }
    for (int k = 0; k < 6; ++k) perf[k] = cs.modePerf[6 * (size_t)(cs.nModes - 1) + k];
    cudaStream_t s = ctx->stream;
    for (int i = 0; i < cs.nModes; ++i) {
        const double *t = i ? cs.modes[i - 1]->tau.p : cs.tau.p, *tb = i ? cs.modes[i - 1]->taub.p : cs.taub.p;
        k_add_into<<<nblocks((long long)n6), RT_BLOCK, 0, s>>>(n6, t, cs.tauTot.p, i == 0);
        if (b6) k_add_into<<<nblocks((long long)b6), RT_BLOCK, 0, s>>>(b6, tb, cs.taubTot.p, i == 0);
        RT_CHECK_LAUNCH();
        launch_count(ctx, b6 ? 2 : 1);
    }
    return st;
}

}  // namespace rt
