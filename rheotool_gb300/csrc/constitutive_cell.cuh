// constitutive_cell.cuh — the per-cell FP64 algebra of the log-conformation
// models: decomposeGradU (boilerLog.H:1-36, constitutiveEq.C:323-358), the
// model sources of the theta equation and tau from the eigen-decomposition.
// The functions are host-and-device so that the same source can be compiled
// for the CPU and compared there with the oracle's restatement.
//   rheoTool: Oldroyd_BLog.C:127-179, GiesekusLog.C:128-176, PTTLog.C:176-268,
//             FENE_PLog.C:128-182, FENE_CRLog.C:127-180, RoliePolyLog.C:125-203,
//             XPomPomLog.C:133-198, WhiteMetznerCYLog.C:145-206.
#pragma once

#include <cmath>
#include <cstddef>
#include <vector>

#include "../../include/rheogpu.h"

#ifndef RT_HD
#define RT_HD __host__ __device__ __forceinline__
#endif
// the scalar functions of the less common models: inlined at the
// compiler's choice, which keeps them out of the register budget of the
// common models' code
#ifndef RT_HDI
#define RT_HDI __host__ __device__ inline
#endif

namespace rt {

// ---------------------------------------------------------------------------
// 3x3 tensors in registers (row-major)
// ---------------------------------------------------------------------------
struct T3 {
    double a[9];
};

RT_HD T3 mul(const T3 &A, const T3 &B) {
    T3 C;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C.a[3 * i + j] = A.a[3 * i] * B.a[j] + A.a[3 * i + 1] * B.a[3 + j] + A.a[3 * i + 2] * B.a[6 + j];
    return C;
}
RT_HD T3 tr(const T3 &A) {
    T3 B;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B.a[3 * i + j] = A.a[3 * j + i];
    return B;
}
RT_HD T3 dg(double x, double y, double z) {
    T3 A;
#pragma unroll
    for (int i = 0; i < 9; ++i) A.a[i] = 0.0;
    A.a[0] = x; A.a[4] = y; A.a[8] = z;
    return A;
}
RT_HD T3 load9(const double *__restrict__ p, int n, int c) {
    T3 A;
#pragma unroll
    for (int i = 0; i < 9; ++i) A.a[i] = p[(size_t)i * n + c];
    return A;
}

// Rolie-Poly stretch rate M1 = 2 (1 - sqrt(3/trA)) / lambdaR, times the
// finite-extensibility factor when chiMax > 1 (RoliePolyLog.C:143-156)
RT_HDI double roliepoly_chi(const rt_model_params &mp, double trA) {
    const double c2 = mp.chiMax * mp.chiMax;
    return ((3.0 - (trA / 3.0) / c2) * (1.0 - 1.0 / c2)) / ((1.0 - (trA / 3.0) / c2) * (3.0 - 1.0 / c2));
}
RT_HDI double roliepoly_m1(const rt_model_params &mp, double trA) {
    double M1 = 2.0 * (1.0 - sqrt(3.0 / trA)) / mp.lambdaR;
    if (mp.chiMax > 1.0) M1 *= roliepoly_chi(mp, trA);
    return M1;
}

// Generalized PTT (PTTLog.C:143-169): Gamma(beta) first, then
// Gamma(alpha k + beta) for k = 0, 1, ... while fewer than maxIterMittagLeffler
// and the last below 1e100.  Host only: computed once per case setup.
inline std::vector<double> ml_gamma_table(const rt_model_params &mp) {
    std::vector<double> g{std::tgamma(mp.beta)};
    int k = 0;
    while (k < mp.maxIterMittagLeffler && g.back() < 1e+100) {
        g.push_back(std::tgamma(mp.alpha * k + mp.beta));
        ++k;
    }
    return g;
}

// E_{alpha,beta}(z) = sum_k z^k / Gamma(alpha k + beta), summed term by term
// until the relative change of the sum is at most rTolMittagLeffler or mlK
// terms are taken (PTTLog.C:205-222); g is ml_gamma_table's table, mlK its
// size less one
RT_HDI double mittag_leffler(const rt_model_params &mp, const double *__restrict__ g, int mlK, double z) {
    double sum = 0.0, sumOld = 0.0, err = 1.0;
    for (int k = 0; k < mlK && err > mp.rTolMittagLeffler; ++k) {
        const double t = pow(z, (double)k) / g[k + 1];
        sumOld = sum;
        sum += t;
        err = fabs((sumOld - sum) / (sumOld + 1e-12));
    }
    return sum;
}

// XPomPom: f of the pre-solve conformation (XPomPomLog.C:148-163); the
// backbone stretch is sqrt(tr A / 3)
RT_HDI double xpompom_f(const rt_model_params &mp, double trA, double trAA) {
    const double lam = sqrt(trA / 3.0), al = mp.alpha;
    const double stretch = (mp.n == 0.0) ? (1.0 - 1.0 / lam) : (1.0 - 1.0 / pow(lam, mp.n + 1.0));
    return ((2.0 * (mp.lambda / mp.lambdaS)) * exp((2.0 / mp.q) * (lam - 1.0))) * stretch +
           (1.0 / (lam * lam)) * (1.0 - al - (al / 3.0) * (trAA - 2.0 * trA));
}

// WhiteMetznerCY: the Carreau-Yasuda factor (1 + (K gd)^a)^((n-1)/a) of etaP
// and lambda at the shear rate gd = sqrt(2) |symm(L)| (WhiteMetznerCYLog.C:
// 152-161; the log form has m = n, L = K and b = a, so the factor is shared)
RT_HDI double whitemetznercy_factor(const rt_model_params &mp, const double L[9]) {
    double d2 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double d = 0.5 * (L[3 * i + j] + L[3 * j + i]);
            d2 += d * d;
        }
    return pow(1.0 + pow((mp.K * sqrt(2.0)) * sqrt(d2), mp.a), (mp.n - 1.0) / mp.a);
}

// ---------------------------------------------------------------------------
// theta source: rhs = symm(Omega theta - theta Omega + 2B + S_model)
// ---------------------------------------------------------------------------
// mlg: the Gamma-function table of the generalized PTT function (mlK + 1
// values, ml_gamma_table), null for the other models
RT_HD void theta_rhs_cell(int c, int N, const rt_model_params &mp, const double *__restrict__ L,
                          const double *__restrict__ Rv, const double *__restrict__ evv,
                          const double *__restrict__ theta, double *__restrict__ rhs, double *__restrict__ fP,
                          const double *__restrict__ mlg = nullptr, int mlK = 0) {
    const double lambda = mp.lambda;
    const double zeta = (mp.model == RT_MODEL_PTT_LOG) ? mp.zeta : 0.0;
    T3 Lc = load9(L, N, c), R = load9(Rv, N, c);
    double e0 = evv[c], e1 = evv[N + c], e2 = evv[2 * N + c];
    T3 Lt = tr(Lc);
    // WhiteMetznerCY's shear-rate factor, taken while grad U is at hand
    const double wmF = (mp.model == RT_MODEL_WHITEMETZNERCY_LOG) ? whitemetznercy_factor(mp, Lc.a) : 1.0;
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
        const double z = (mp.epsilon / (1.0 - zeta)) * (trA - 3.0);
        double fac;
        if (mp.pttFunction == RT_PTT_EXP) fac = exp(z);
        else if (mp.pttFunction == RT_PTT_GENERALIZED) fac = (mlK > 0) ? mlg[0] * mittag_leffler(mp, mlg, mlK, z) : 0.0;
        else fac = 1.0 + z;
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = ((1.0 / lambda) * T.a[i]) * fac;
    } else if (mp.model == RT_MODEL_ROLIEPOLY_LOG) {
        // RoliePolyLog.C:140-179: -(1/lambdaD) A^-1 ((A - I) + M1 lambdaD (A + beta (trA/3)^delta (A - I)))
        T3 A = mul(mul(R, dg(e0, e1, e2)), Rt);
        T3 Ai = mul(mul(R, dg(1.0 / e0, 1.0 / e1, 1.0 / e2)), Rt);
        const double trA = A.a[0] + A.a[4] + A.a[8];
        const double lamD = lambda;
        const double M1 = roliepoly_m1(mp, trA);
        const double ccr = mp.beta * pow(trA / 3.0, mp.delta);
        T3 G;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const double AmI = A.a[i] - ((i % 4 == 0) ? 1.0 : 0.0);
            G.a[i] = AmI + (M1 * lamD) * (A.a[i] + ccr * AmI);
        }
        T3 AG = mul(Ai, G);
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = -((1.0 / lamD) * AG.a[i]);
    } else if (mp.model == RT_MODEL_XPOMPOM_LOG) {
        // XPomPomLog.C:165-185: -(1/lambdaB) A^-1 (A (f - 2 alpha) + alpha A.A + (alpha - 1) I),
        // formed in the eigenbasis of A, where it is diagonal:
        // -(1/lambdaB) ((f - 2 alpha) + alpha e_i + (alpha - 1)/e_i)
        const double al = mp.alpha;
        const double f = xpompom_f(mp, e0 + e1 + e2, e0 * e0 + e1 * e1 + e2 * e2);
        const double fa = f - 2.0 * al, am1 = al - 1.0, li = 1.0 / lambda;
        S = mul(mul(R, dg(-(li * ((fa + al * e0) + am1 / e0)), -(li * ((fa + al * e1) + am1 / e1)),
                          -(li * ((fa + al * e2) + am1 / e2)))),
                Rt);
    } else if (mp.model == RT_MODEL_WHITEMETZNERCY_LOG) {
        // WhiteMetznerCYLog.C:170-193, 203: (1/lambda(gd)) R (Lambda^-1 - I) R^T, and
        // etaP(gd)/lambda(gd) of the same pre-solve grad U kept for tau
        const double lamc = lambda * wmF;
        fP[c] = (mp.etaP * wmF) / lamc;
        S = mul(mul(R, invm1), Rt);
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lamc) * S.a[i];
    } else if (mp.model == RT_MODEL_FENECR_LOG) {
        // FENE_CRLog.C:140-163: (1/lambda) f R (Lambda^-1 - I) R^T, f from the pre-solve A
        T3 A = mul(mul(R, dg(e0, e1, e2)), Rt);
        double trA = A.a[0] + A.a[4] + A.a[8];
        double f = mp.L2 / (mp.L2 - trA);
        fP[c] = f;
        S = mul(mul(R, invm1), Rt);
        const double lf = (1.0 / lambda) * f;
#pragma unroll
        for (int i = 0; i < 9; ++i) S.a[i] = lf * S.a[i];
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

// tau = c (R Lambda R^T - I)   (FENE-P: c (f R Lambda R^T - a I); FENE-CR:
// (c f)(R Lambda R^T - I), FENE_CRLog.C:174, with the pre-solve f;
// XPomPom: c = etaP/lambdaB, XPomPomLog.C:195; WhiteMetznerCY: c =
// etaP(gd)/lambda(gd) of the pre-solve grad U, WhiteMetznerCYLog.C:203)
RT_HD void tau_cell(int c, int N, const rt_model_params &mp, const double *__restrict__ Rv,
                                         const double *__restrict__ evv, const double *__restrict__ fP,
                                         double *__restrict__ tau) {
    double zeta = (mp.model == RT_MODEL_PTT_LOG) ? mp.zeta : 0.0;
    double cP = mp.etaP / mp.lambda;
    if (mp.model == RT_MODEL_PTT_LOG) cP = mp.etaP / (mp.lambda * (1.0 - zeta));
    if (mp.model == RT_MODEL_FENECR_LOG) cP = cP * fP[c];
    if (mp.model == RT_MODEL_WHITEMETZNERCY_LOG) cP = fP[c];
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
    if (mp.model == RT_MODEL_ROLIEPOLY_LOG && mp.chiMax > 1.0)   // RoliePolyLog.C:189-199
        cP = cP * roliepoly_chi(mp, A.a[0] + A.a[4] + A.a[8]);
    tau[c] = cP * T.a[0];
    tau[(size_t)N + c] = cP * (0.5 * (T.a[1] + T.a[3]));
    tau[(size_t)2 * N + c] = cP * (0.5 * (T.a[2] + T.a[6]));
    tau[(size_t)3 * N + c] = cP * T.a[4];
    tau[(size_t)4 * N + c] = cP * (0.5 * (T.a[5] + T.a[7]));
    tau[(size_t)5 * N + c] = cP * T.a[8];
}

}  // namespace rt
