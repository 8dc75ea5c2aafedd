/*
 * oracle.c — FP64 CPU restatement of rheoFoam's segregated time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA library is
 * compared against (tests/, __graft_entry__.smoke(), bench.py's CPU baseline).
 * Nothing in the product links or calls it.
 *
 * It restates, from the discretisation mathematics and from rheoTool's own
 * sources (paths inside fppimenta/rheoTool, of90/src):
 *   - rheoFoam segregated step .......... solvers/rheoFoam/rheoFoam.C:147-154,
 *                                         UEqn.H:5-21, pEqn.H:1-65
 *   - divTau (none / BSD / coupling) .... libs/constitutiveEquations/
 *                                         constitutiveEqs/constitutiveEq/
 *                                         constitutiveEq.C:72-132
 *   - boilerLog / decomposeGradU ........ constitutiveEqs/utils/boilerLog.H:1-36,
 *                                         constitutiveEq.C:323-358, innerP :471-531
 *   - calcEig ........................... constitutiveEq.C:360-428 (Eigen's
 *                                         SelfAdjointEigenSolver is replaced by
 *                                         the cyclic Jacobi method, eigenvalues
 *                                         ascending as Eigen returns them)
 *   - Oldroyd-BLog / GiesekusLog / PTTLog / FENE-PLog / FENE-CRLog /
 *     Rolie-PolyLog / XPomPomLog / WhiteMetznerCYLog correct()
 *                                         Oldroyd_BLog.C:127-179, GiesekusLog.C:
 *                                         128-176, PTTLog.C:176-268, FENE_PLog.C:
 *                                         128-182, FENE_CRLog.C:127-180,
 *                                         RoliePolyLog.C:125-203, XPomPomLog.C:
 *                                         133-198, WhiteMetznerCYLog.C:145-206
 *   - GaussDefCmpw convection ........... libs/gaussDefCmpwConvectionScheme/
 *                                         gaussDefCmpwConvectionScheme.C:72-170,
 *                                         197-328; limiters.H:39-100
 *   - linearExtrapolation BC ............ libs/boundaryConditions/
 *                                         linearExtrapolation/
 *                                         linearExtrapolationFvPatchField.C:102-150
 *   - residual normalisation ............ libs/sparseMatrixSolvers/segregated/
 *                                         sparseSolver.C:129-180
 *   - adjustCorrPhi ..................... solvers/shared/singlePhase/
 *                                         adjustCorrPhi.H:32-158
 *   - multiMode ......................... libs/constitutiveEquations/
 *                                         constitutiveEqs/multiMode/multiMode.C:
 *                                         144-156 (divTau), 222 (tau), 247-256
 *                                         (correct)
 *   - nNonOrthogonalCorrectors .......... solvers/rheoFoam/pEqn.H:31-50
 *   - temperature-dependent parameters .. libs/thermo/thermoFunctions/{Constant,
 *                                         Arrhenius,ArrheniusModified,WLF,VFT}/<type>.C
 *                                         (multiply), as the Log models' correct()
 *                                         applies them (Oldroyd_BLog.C:133-135,
 *                                         RoliePolyLog.C:139-141, XPomPomLog.C:
 *                                         140-142, WhiteMetznerCYLog.C:166-167)
 * and OpenFOAM v9 behaviour that is not vendored in rheoTool (fvm::ddt Euler
 * and Crank-Nicolson, Gauss linear grad/div, orthogonal laplacian, fvMatrix
 * A/H/H1/flux, ddtCorr, setReference, PCG, PBiCGStab, PBiCG, DIC, DILU),
 * restated from the published methods:
 *   - Gauss gradient, linear interpolation, orthogonal snGrad, Euler implicit
 *     ddt, SIMPLEC with Rhie-Chow/ddtCorr flux (Jasak 1996 thesis; Van
 *     Doormaal & Raithby 1984 for SIMPLEC);
 *   - Crank-Nicolson ddt with off-centering psi as the trapezoidal rule on a
 *     stored old-time derivative (psi = 1: the trapezoidal rule, psi = 0:
 *     Euler implicit), the first step of a run Euler implicit;
 *   - CG (Hestenes & Stiefel 1952), BiCGStab (van der Vorst 1992), BiCG
 *     (Fletcher 1976) with the transposed preconditioner, D-ILU(0)
 *     with the diagonal chosen so that diag(M) = diag(A) (Pommerell 1992),
 *     applied as a forward and a backward substitution in face order;
 *   - cyclic Jacobi eigenvalue method with Rutishauser's rotation formulas;
 *   - cyclic (periodic) patches: each face pair is an internal face whose
 *     neighbour centre is translated by the period (weights, deltaCoeffs and
 *     C_N - C_P from the translated geometry); its coefficients act in A x
 *     and in the residual but not in the DIC/DILU factorisation or sweeps,
 *     which is how an lduInterface coupling enters OpenFOAM's solvers.
 *
 * Parity status: the reference needs OpenFOAM v9 and Eigen, neither of which
 * exists here, so this restatement is pinned only by closed-form solutions
 * (tests/test_oracle_kat.py) and by its own invariants; parity with the
 * reference's own rheoFoam fields is unpinned.
 *
 * Compile with -ffp-contract=off so that x86 and Arm give the same bits.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#include "../include/rheogpu.h"

#define OR_SMALL   1e-15
#define OR_VSMALL  1e-300
#define OR_SOLVER_SMALL 1e-20

typedef struct {
    double *U, *Ub;          /* 3N, 3nB */
    double *p, *pb;          /* N, nB */
    double *phi, *phib;      /* nF, nB */
    double *theta, *thetab;  /* 6N, 6nB */
    double *tau, *taub;      /* 6N, 6nB */
    double *eigVals;         /* 3N */
    double *eigVecs;         /* 9N */
} or_state;

/* Crank-Nicolson state kept between time steps (NULL or scheme Euler: the
 * implicit Euler ddt).  The scheme is the trapezoidal rule written with the
 * stored time derivative of the old time level D: the step from n to n+1
 * solves (c/dt)(x - x_n) - psi D_n = f(x), c = 1 + psi, psi the off-centering
 * coefficient (1: Crank-Nicolson, 0: Euler), with D_n = c_{n-1}(x_n -
 * x_{n-1})/dt - psi D_{n-1}; the first step is an implicit Euler step (c = 1,
 * D_0 = 0), so D_1 = (x_1 - x_0)/dt is the derivative that step implies.  D
 * is formed at the start of a step from the fields there and the fields at
 * the start of the previous step (xs), then xs takes the current fields.  The
 * flux correction ddtCorr takes the same old-time parts:
 * ddtCorr = coef (c/dt phi_n + psi D_phi - Sf.interp(c/dt U_n + psi D_U)). */
typedef struct {
    int scheme;          /* RT_DDT_EULER / RT_DDT_CRANKNICOLSON */
    double psi;
    int nSteps;          /* time steps of the flow (U, phi) started so far */
    int nThSteps;        /* time steps of the theta equations started so far */
    double *DU, *DUb;    /* 3N, 3nB */
    double *Dphi, *Dphib;/* nF, nB */
    double *Dth;         /* 6N per mode */
    double *Us, *Ubs, *phis, *phibs, *ths;   /* the fields at the start of the last step */
} or_ddt;

/* coefficient c of the step with index j (0-based) */
static double ddt_coef(const or_ddt *d, int j) { return j == 0 ? 1.0 : 1.0 + d->psi; }

static void *xcalloc(size_t n, size_t sz) {
    void *p = calloc(n ? n : 1, sz);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}
#define DALLOC(n) ((double *)xcalloc((size_t)(n), sizeof(double)))

static int nthreads_ = 1;
void or_set_threads(int n) { nthreads_ = n > 0 ? n : 1; }

/* ------------------------------------------------------------------------ */
/* boundary helpers                                                          */
/* ------------------------------------------------------------------------ */
static void bface_kinds(const rt_mesh_desc *m, const int32_t *patchKind, int *out) {
    for (int p = 0; p < m->nPatches; ++p)
        for (int i = 0; i < m->patchSize[p]; ++i)
            out[m->patchStart[p] + i] = patchKind[p];
}

/* zeroGradient boundary values = cell values (nc components AoS) */
static void correct_bc(const rt_mesh_desc *m, const int *kind, const double *x,
                       double *xb, int nc) {
    for (int b = 0; b < m->nBFaces; ++b)
        if (kind[b] == RT_BC_ZEROGRAD)
            for (int k = 0; k < nc; ++k) xb[nc * b + k] = x[nc * m->bCell[b] + k];
}

/* ------------------------------------------------------------------------ */
/* fvc operators                                                              */
/* ------------------------------------------------------------------------ */
static inline double lin_interp(double w, double vP, double vN) {
    return w * (vP - vN) + vN;
}

/* Gauss linear gradient of component k of an nc-component AoS field. */
static void gauss_grad(const rt_mesh_desc *m, const double *x, const double *xb,
                       int nc, int k, double *g /*3N*/) {
    const int N = m->nCells;
    memset(g, 0, sizeof(double) * 3 * (size_t)N);
    for (int f = 0; f < m->nFaces; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double xf = lin_interp(m->weights[f], x[nc * o + k], x[nc * n + k]);
        for (int d = 0; d < 3; ++d) {
            double s = m->Sf[3 * f + d] * xf;
            g[3 * o + d] += s;
            g[3 * n + d] -= s;
        }
    }
    for (int b = 0; b < m->nBFaces; ++b) {
        int c = m->bCell[b];
        double xf = xb[nc * b + k];
        for (int d = 0; d < 3; ++d) g[3 * c + d] += m->bSf[3 * b + d] * xf;
    }
    for (int c = 0; c < N; ++c)
        for (int d = 0; d < 3; ++d) g[3 * c + d] /= m->V[c];
}

void or_grad(const rt_mesh_desc *m, const double *psi, const double *psib, double *g) {
    gauss_grad(m, psi, psib, 1, 0, g);
}

/* Gauss linear gradient of a vector field: G_ij = d_i U_j (9 comps AoS). */
static void grad_vector(const rt_mesh_desc *m, const double *U, const double *Ub, double *G) {
    const int N = m->nCells;
    double *g = DALLOC(3 * (size_t)N);
    for (int j = 0; j < 3; ++j) {
        gauss_grad(m, U, Ub, 3, j, g);
        for (int c = 0; c < N; ++c)
            for (int i = 0; i < 3; ++i) G[9 * c + 3 * i + j] = g[3 * c + i];
    }
    free(g);
}

/* Boundary value of a Gauss gradient: the cell value with its normal part
 * replaced by the face-normal gradient, g_b = g_P + n (snGrad_b - n.g_P). */
static void grad_boundary(const rt_mesh_desc *m, const double *G, const double *U,
                          const double *Ub, double *Gb /*9 nB*/) {
    for (int b = 0; b < m->nBFaces; ++b) {
        int c = m->bCell[b];
        double n[3];
        for (int d = 0; d < 3; ++d) n[d] = m->bSf[3 * b + d] / m->bmagSf[b];
        for (int j = 0; j < 3; ++j) {
            double sn = m->bDeltaCoeffs[b] * (Ub[3 * b + j] - U[3 * c + j]);
            double ng = 0.0;
            for (int i = 0; i < 3; ++i) ng += n[i] * G[9 * c + 3 * i + j];
            for (int i = 0; i < 3; ++i)
                Gb[9 * b + 3 * i + j] = G[9 * c + 3 * i + j] + n[i] * (sn - ng);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* LDU algebra                                                                */
/* ------------------------------------------------------------------------ */
static void amul(const rt_mesh_desc *m, const double *diag, const double *upper,
                 const double *lower, const double *x, double *y) {
    const int N = m->nCells;
    for (int c = 0; c < N; ++c) y[c] = diag[c] * x[c];
    for (int f = 0; f < m->nFaces; ++f) {
        int l = m->owner[f], u = m->neighbour[f];
        y[u] += lower[f] * x[l];
        y[l] += upper[f] * x[u];
    }
}

static void sum_a(const rt_mesh_desc *m, const double *diag, const double *upper,
                  const double *lower, double *s) {
    for (int c = 0; c < m->nCells; ++c) s[c] = diag[c];
    for (int f = 0; f < m->nFaces; ++f) {
        s[m->neighbour[f]] += lower[f];
        s[m->owner[f]] += upper[f];
    }
}

static double sum_mag(const double *x, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += fabs(x[i]);
    return s;
}
static double sum_prod(const double *x, const double *y, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

/* Residual normalisation factor of sparseSolver.C:129-180:
 * sum(|A x - xbar A 1| + |b - xbar A 1|) + 1e-20. */
static double norm_factor(const rt_mesh_desc *m, const double *diag, const double *upper,
                          const double *lower, const double *b, const double *x,
                          const double *Ax) {
    const int N = m->nCells;
    double *pA = DALLOC(N);
    sum_a(m, diag, upper, lower, pA);
    double xbar = 0.0;
    for (int c = 0; c < N; ++c) xbar += x[c];
    xbar /= N;
    for (int c = 0; c < N; ++c) pA[c] *= xbar;
    double s = 0.0;
    for (int c = 0; c < N; ++c) s += fabs(Ax[c] - pA[c]) + fabs(b[c] - pA[c]);
    free(pA);
    return s + 1e-20;
}

double or_residual(const rt_mesh_desc *m, const double *diag, const double *upper,
                   const double *lower, const double *b, const double *x) {
    const int N = m->nCells;
    double *Ax = DALLOC(N), *r = DALLOC(N);
    amul(m, diag, upper, lower, x, Ax);
    for (int c = 0; c < N; ++c) r[c] = b[c] - Ax[c];
    double nf = norm_factor(m, diag, upper, lower, b, x, Ax);
    double res = sum_mag(r, N) / nf;
    free(Ax); free(r);
    return res;
}

/* D-ILU(0): rD_u = a_uu - sum_{l<u} a_ul a_lu / rD_l, accumulated in face
 * order, then inverted.  DIC is the symmetric case (lower == upper). */
static void dilu_rd(const rt_mesh_desc *m, const double *diag, const double *upper,
                    const double *lower, double *rD) {
    for (int c = 0; c < m->nCells; ++c) rD[c] = diag[c];
    for (int f = 0; f < m->nFaces; ++f) {
        if (m->coupled && m->coupled[f]) continue;   /* interface: not factorised */
        int l = m->owner[f], u = m->neighbour[f];
        rD[u] -= upper[f] * lower[f] / rD[l];
    }
    for (int c = 0; c < m->nCells; ++c) rD[c] = 1.0 / rD[c];
}

static void precondition(const rt_mesh_desc *m, int type, const double *rD,
                         const double *upper, const double *lower,
                         const double *r, double *w) {
    const int N = m->nCells;
    if (type == RT_PRECOND_NONE) { memcpy(w, r, sizeof(double) * N); return; }
    for (int c = 0; c < N; ++c) w[c] = rD[c] * r[c];
    if (type == RT_PRECOND_DIAGONAL) return;
    for (int f = 0; f < m->nFaces; ++f) {
        if (m->coupled && m->coupled[f]) continue;   /* interfaces stay out of the sweeps */
        int l = m->owner[f], u = m->neighbour[f];
        w[u] -= rD[u] * lower[f] * w[l];
    }
    for (int f = m->nFaces - 1; f >= 0; --f) {
        if (m->coupled && m->coupled[f]) continue;
        int l = m->owner[f], u = m->neighbour[f];
        w[l] -= rD[l] * upper[f] * w[u];
    }
}

static int conv_check(double fin, double init, const rt_solver_ctl *c) {
    return fin < c->tolerance || (c->relTol > OR_SOLVER_SMALL && fin < c->relTol * init);
}

static void pcg(const rt_mesh_desc *m, const double *diag, const double *upper,
                const double *lower, const double *b, double *x,
                const rt_solver_ctl *ctl, rt_solver_perf *perf) {
    const int N = m->nCells;
    double *wA = DALLOC(N), *rA = DALLOC(N), *pA = DALLOC(N), *rD = DALLOC(N);
    int pre = ctl->preconditioner;
    if (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU) dilu_rd(m, diag, upper, lower, rD);
    else if (pre == RT_PRECOND_DIAGONAL) for (int c = 0; c < N; ++c) rD[c] = 1.0 / diag[c];
    amul(m, diag, upper, lower, x, wA);
    for (int c = 0; c < N; ++c) rA[c] = b[c] - wA[c];
    double nf = norm_factor(m, diag, upper, lower, b, x, wA);
    perf->initialResidual = sum_mag(rA, N) / nf;
    perf->finalResidual = perf->initialResidual;
    perf->nIterations = 0;
    perf->singular = 0;
    if (ctl->minIter > 0 || !conv_check(perf->finalResidual, perf->initialResidual, ctl)) {
        double wArA = 1e20, wArAold;
        do {
            wArAold = wArA;
            precondition(m, pre, rD, upper, lower, rA, wA);
            wArA = sum_prod(wA, rA, N);
            if (perf->nIterations == 0) {
                for (int c = 0; c < N; ++c) pA[c] = wA[c];
            } else {
                double beta = wArA / wArAold;
                for (int c = 0; c < N; ++c) pA[c] = wA[c] + beta * pA[c];
            }
            amul(m, diag, upper, lower, pA, wA);
            double wApA = sum_prod(wA, pA, N);
            if (fabs(wApA) / nf < OR_VSMALL) { perf->singular = 1; break; }
            double alpha = wArA / wApA;
            for (int c = 0; c < N; ++c) {
                x[c] += alpha * pA[c];
                rA[c] -= alpha * wA[c];
            }
            perf->finalResidual = sum_mag(rA, N) / nf;
        } while ((++perf->nIterations < ctl->maxIter &&
                  !conv_check(perf->finalResidual, perf->initialResidual, ctl)) ||
                 perf->nIterations < ctl->minIter);
    }
    perf->converged = conv_check(perf->finalResidual, perf->initialResidual, ctl);
    free(wA); free(rA); free(pA); free(rD);
}

static void pbicgstab(const rt_mesh_desc *m, const double *diag, const double *upper,
                      const double *lower, const double *b, double *x,
                      const rt_solver_ctl *ctl, rt_solver_perf *perf) {
    const int N = m->nCells;
    double *yA = DALLOC(N), *rA = DALLOC(N), *rD = DALLOC(N);
    int pre = ctl->preconditioner;
    if (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU) dilu_rd(m, diag, upper, lower, rD);
    else if (pre == RT_PRECOND_DIAGONAL) for (int c = 0; c < N; ++c) rD[c] = 1.0 / diag[c];
    amul(m, diag, upper, lower, x, yA);
    for (int c = 0; c < N; ++c) rA[c] = b[c] - yA[c];
    double nf = norm_factor(m, diag, upper, lower, b, x, yA);
    perf->initialResidual = sum_mag(rA, N) / nf;
    perf->finalResidual = perf->initialResidual;
    perf->nIterations = 0;
    perf->singular = 0;
    if (ctl->minIter > 0 || !conv_check(perf->finalResidual, perf->initialResidual, ctl)) {
        double *pA = DALLOC(N), *AyA = DALLOC(N), *sA = DALLOC(N), *zA = DALLOC(N),
               *tA = DALLOC(N), *rA0 = DALLOC(N);
        memcpy(rA0, rA, sizeof(double) * N);
        double rA0rA = 0.0, alpha = 0.0, omega = 0.0;
        int done = 0;
        do {
            double rA0rAold = rA0rA;
            rA0rA = sum_prod(rA0, rA, N);
            if (fabs(rA0rA) < OR_VSMALL) { perf->singular = 1; break; }
            if (perf->nIterations == 0) {
                for (int c = 0; c < N; ++c) pA[c] = rA[c];
            } else {
                if (fabs(omega) < OR_VSMALL) { perf->singular = 1; break; }
                double beta = (rA0rA / rA0rAold) * (alpha / omega);
                for (int c = 0; c < N; ++c) pA[c] = rA[c] + beta * (pA[c] - omega * AyA[c]);
            }
            precondition(m, pre, rD, upper, lower, pA, yA);
            amul(m, diag, upper, lower, yA, AyA);
            double rA0AyA = sum_prod(rA0, AyA, N);
            alpha = rA0rA / rA0AyA;
            for (int c = 0; c < N; ++c) sA[c] = rA[c] - alpha * AyA[c];
            perf->finalResidual = sum_mag(sA, N) / nf;
            if (conv_check(perf->finalResidual, perf->initialResidual, ctl)) {
                for (int c = 0; c < N; ++c) x[c] += alpha * yA[c];
                perf->nIterations++;
                done = 1;
                break;
            }
            precondition(m, pre, rD, upper, lower, sA, zA);
            amul(m, diag, upper, lower, zA, tA);
            double tAtA = sum_prod(tA, tA, N);
            omega = sum_prod(tA, sA, N) / tAtA;
            for (int c = 0; c < N; ++c) {
                x[c] += alpha * yA[c] + omega * zA[c];
                rA[c] = sA[c] - omega * tA[c];
            }
            perf->finalResidual = sum_mag(rA, N) / nf;
        } while ((++perf->nIterations < ctl->maxIter &&
                  !conv_check(perf->finalResidual, perf->initialResidual, ctl)) ||
                 perf->nIterations < ctl->minIter);
        (void)done;
        free(pA); free(AyA); free(sA); free(zA); free(tA); free(rA0);
    }
    perf->converged = conv_check(perf->finalResidual, perf->initialResidual, ctl);
    free(yA); free(rA); free(rD);
}

/* Preconditioned bi-conjugate gradients (Fletcher 1976; the preconditioned
 * form of Barrett et al. 1994, "Templates", fig. 2.7) in OpenFOAM's lduMatrix
 * conventions, as the PBiCG solver of the Contraction41 tutorials' U and
 * theta equations runs it (of90/tutorials/rheoFoam/Contraction41/
 * Oldroyd-BLog/system/fvSolution:32,47): the shadow system is the transposed
 * one with the same right-hand side (rT = b - A^T psi), preconditioned by the
 * transpose of the DILU factorisation (the same rD, the lower and upper
 * coefficients exchanged).  Per iteration: w = M^-1 r, wT = M^-T rT, rho =
 * w.rT, p = w (+ beta p), pT = wT (+ beta pT), q = A p, qT = A^T pT, alpha =
 * rho / (q.pT); the singularity test and the stopping rules are those of
 * pcg() above. */
static void pbicg(const rt_mesh_desc *m, const double *diag, const double *upper,
                  const double *lower, const double *b, double *x,
                  const rt_solver_ctl *ctl, rt_solver_perf *perf) {
    const int N = m->nCells;
    double *wA = DALLOC(N), *rA = DALLOC(N), *pA = DALLOC(N), *rD = DALLOC(N);
    double *wT = DALLOC(N), *rT = DALLOC(N), *pT = DALLOC(N);
    int pre = ctl->preconditioner;
    if (pre == RT_PRECOND_DIC || pre == RT_PRECOND_DILU) dilu_rd(m, diag, upper, lower, rD);
    else if (pre == RT_PRECOND_DIAGONAL) for (int c = 0; c < N; ++c) rD[c] = 1.0 / diag[c];
    amul(m, diag, upper, lower, x, wA);
    amul(m, diag, lower, upper, x, wT);           /* A^T x: the coefficients exchanged */
    for (int c = 0; c < N; ++c) {
        rA[c] = b[c] - wA[c];
        rT[c] = b[c] - wT[c];
    }
    double nf = norm_factor(m, diag, upper, lower, b, x, wA);
    perf->initialResidual = sum_mag(rA, N) / nf;
    perf->finalResidual = perf->initialResidual;
    perf->nIterations = 0;
    perf->singular = 0;
    if (ctl->minIter > 0 || !conv_check(perf->finalResidual, perf->initialResidual, ctl)) {
        double wArT = 1e20, wArTold;
        do {
            wArTold = wArT;
            precondition(m, pre, rD, upper, lower, rA, wA);
            precondition(m, pre, rD, lower, upper, rT, wT);   /* M^-T */
            wArT = sum_prod(wA, rT, N);
            if (perf->nIterations == 0) {
                for (int c = 0; c < N; ++c) {
                    pA[c] = wA[c];
                    pT[c] = wT[c];
                }
            } else {
                double beta = wArT / wArTold;
                for (int c = 0; c < N; ++c) {
                    pA[c] = wA[c] + beta * pA[c];
                    pT[c] = wT[c] + beta * pT[c];
                }
            }
            amul(m, diag, upper, lower, pA, wA);
            amul(m, diag, lower, upper, pT, wT);
            double wApT = sum_prod(wA, pT, N);
            if (fabs(wApT) / nf < OR_VSMALL) { perf->singular = 1; break; }
            double alpha = wArT / wApT;
            for (int c = 0; c < N; ++c) {
                x[c] += alpha * pA[c];
                rA[c] -= alpha * wA[c];
                rT[c] -= alpha * wT[c];
            }
            perf->finalResidual = sum_mag(rA, N) / nf;
        } while ((++perf->nIterations < ctl->maxIter &&
                  !conv_check(perf->finalResidual, perf->initialResidual, ctl) &&
                  isfinite(perf->finalResidual)) ||
                 perf->nIterations < ctl->minIter);
    }
    perf->converged = conv_check(perf->finalResidual, perf->initialResidual, ctl);
    free(wA); free(rA); free(pA); free(rD); free(wT); free(rT); free(pT);
}

/* One component solve, lduMatrix::solver semantics. */
int or_ldu_solve(const rt_mesh_desc *m, const double *diag, const double *upper,
                 const double *lower, const double *b, double *x,
                 const rt_solver_ctl *ctl, rt_solver_perf *perf) {
    if (ctl->solver == RT_SOLVER_PCG) pcg(m, diag, upper, lower, b, x, ctl, perf);
    else if (ctl->solver == RT_SOLVER_PBICG) pbicg(m, diag, upper, lower, b, x, ctl, perf);
    else pbicgstab(m, diag, upper, lower, b, x, ctl, perf);
    return (isfinite(perf->finalResidual)) ? RT_OK : RT_ENAN;
}

/* ------------------------------------------------------------------------ */
/* 3x3 tensors (row-major) and the Jacobi eigensolver                        */
/* ------------------------------------------------------------------------ */
typedef struct { double a[9]; } t3;

static inline t3 t3_mul(t3 A, t3 B) {
    t3 C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            C.a[3 * i + j] = A.a[3 * i + 0] * B.a[0 + j] + A.a[3 * i + 1] * B.a[3 + j] +
                             A.a[3 * i + 2] * B.a[6 + j];
    return C;
}
static inline t3 t3_T(t3 A) {
    t3 B;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B.a[3 * i + j] = A.a[3 * j + i];
    return B;
}
static inline t3 t3_from_symm(const double *s) {
    t3 A;
    A.a[0] = s[0]; A.a[1] = s[1]; A.a[2] = s[2];
    A.a[3] = s[1]; A.a[4] = s[3]; A.a[5] = s[4];
    A.a[6] = s[2]; A.a[7] = s[4]; A.a[8] = s[5];
    return A;
}
static inline void t3_symm(t3 A, double *s) {
    s[0] = A.a[0];
    s[1] = 0.5 * (A.a[1] + A.a[3]);
    s[2] = 0.5 * (A.a[2] + A.a[6]);
    s[3] = A.a[4];
    s[4] = 0.5 * (A.a[5] + A.a[7]);
    s[5] = A.a[8];
}
static inline t3 t3_diag(double x, double y, double z) {
    t3 A;
    memset(&A, 0, sizeof A);
    A.a[0] = x; A.a[4] = y; A.a[8] = z;
    return A;
}

/* Symmetric 3x3 eigensolver: cyclic Jacobi sweeps over (0,1), (0,2), (1,2),
 * rotation angle from t = sgn(th)/(|th| + sqrt(th^2 + 1)),
 * th = (a_qq - a_pp)/(2 a_pq); a rotation is skipped when |a_pq| is below
 * 1e-18 (|a_pp| + |a_qq|) (it is then set to zero).  mu ascending, V columns. */
void or_eig3(const double *s, double *mu, double *V) {
    double A[3][3] = {{s[0], s[1], s[2]}, {s[1], s[3], s[4]}, {s[2], s[4], s[5]}};
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    static const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
    for (int sweep = 0; sweep < 12; ++sweep) {
        double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
        if (off == 0.0) break;
        for (int r = 0; r < 3; ++r) {
            int p = P[r], q = Q[r];
            double apq = A[p][q];
            if (fabs(apq) <= 1e-18 * (fabs(A[p][p]) + fabs(A[q][q]))) {
                A[p][q] = A[q][p] = 0.0;
                continue;
            }
            double th = (A[q][q] - A[p][p]) / (2.0 * apq);
            double t = 1.0 / (fabs(th) + sqrt(th * th + 1.0));
            if (th < 0.0) t = -t;
            double c = 1.0 / sqrt(t * t + 1.0);
            double sn = t * c;
            double app = A[p][p], aqq = A[q][q];
            A[p][p] = app - t * apq;
            A[q][q] = aqq + t * apq;
            A[p][q] = A[q][p] = 0.0;
            int k = 3 - p - q;
            double akp = A[k][p], akq = A[k][q];
            A[k][p] = A[p][k] = c * akp - sn * akq;
            A[k][q] = A[q][k] = sn * akp + c * akq;
            for (int i = 0; i < 3; ++i) {
                double rp = R[i][p], rq = R[i][q];
                R[i][p] = c * rp - sn * rq;
                R[i][q] = sn * rp + c * rq;
            }
        }
    }
    double ev[3] = {A[0][0], A[1][1], A[2][2]};
    int idx[3] = {0, 1, 2};
    /* stable ascending sort of three */
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2 - i; ++j)
            if (ev[idx[j]] > ev[idx[j + 1]]) { int t = idx[j]; idx[j] = idx[j + 1]; idx[j + 1] = t; }
    for (int j = 0; j < 3; ++j) {
        mu[j] = ev[idx[j]];
        for (int i = 0; i < 3; ++i) V[3 * i + j] = R[i][idx[j]];
    }
}

/* constitutiveEq::calcEig on n cells: eigVals = exp(mu) (diagonal), eigVecs. */
void or_eig(int n, const double *theta, double *eigVals, double *eigVecs) {
#pragma omp parallel for num_threads(nthreads_) schedule(static)
    for (int c = 0; c < n; ++c) {
        double mu[3];
        or_eig3(theta + 6 * (size_t)c, mu, eigVecs + 9 * (size_t)c);
        for (int k = 0; k < 3; ++k) eigVals[3 * (size_t)c + k] = exp(mu[k]);
    }
}

/* ------------------------------------------------------------------------ */
/* GaussDefCmpw convection (fvm::div(phi, psi)) for an nc-component field     */
/* ------------------------------------------------------------------------ */
static void lims(int scheme, double *al, double *be, double *bl) {
    switch (scheme) {
    case RT_LIM_CUBISTA:  al[0]=7./4.; al[1]=3./4.; al[2]=1./4.; be[0]=0.; be[1]=3./8.; be[2]=3./4.; bl[0]=3./8.; bl[1]=3./4.; break;
    case RT_LIM_MINMOD:   al[0]=1.5; al[1]=.5; al[2]=.5; be[0]=0.; be[1]=.5; be[2]=.5; bl[0]=.5; bl[1]=1.; break;
    case RT_LIM_SMART:    al[0]=3.; al[1]=3./4.; al[2]=0.; be[0]=0.; be[1]=3./8.; be[2]=1.; bl[0]=1./6.; bl[1]=5./6.; break;
    case RT_LIM_WACEB:    al[0]=2.; al[1]=3./4.; al[2]=0.; be[0]=0.; be[1]=3./8.; be[2]=1.; bl[0]=3./10.; bl[1]=5./6.; break;
    case RT_LIM_SUPERBEE: al[0]=0.5; al[1]=1.5; al[2]=0.; be[0]=0.5; be[1]=0.; be[2]=1.; bl[0]=1./2.; bl[1]=2./3.; break;
    default:              al[0]=al[1]=al[2]=1.; be[0]=be[1]=be[2]=0.; bl[0]=bl[1]=1.; break;
    }
}

typedef struct {
    int N, nF, nB, nc;
    double *diag, *lower, *upper;   /* N, nF, nF */
    double *source;                 /* nc*N AoS */
    double *intC, *bouC;            /* nc*nB AoS */
} or_matrix;

static void mat_alloc(or_matrix *M, const rt_mesh_desc *m, int nc) {
    M->N = m->nCells; M->nF = m->nFaces; M->nB = m->nBFaces; M->nc = nc;
    M->diag = DALLOC(M->N); M->lower = DALLOC(M->nF); M->upper = DALLOC(M->nF);
    M->source = DALLOC((size_t)nc * M->N);
    M->intC = DALLOC((size_t)nc * M->nB); M->bouC = DALLOC((size_t)nc * M->nB);
}
static void mat_free(or_matrix *M) {
    free(M->diag); free(M->lower); free(M->upper); free(M->source); free(M->intC); free(M->bouC);
}

/* upwind part + explicit deferred correction, gaussDefCmpwConvectionScheme.C */
static void defcmpw(const rt_mesh_desc *m, int scheme, const double *phi, const double *phib,
                    const double *x, const double *xb, const int *kind, int nc, or_matrix *M) {
    const int N = m->nCells, nF = m->nFaces;
    double *upw = DALLOC(nF);
    for (int f = 0; f < nF; ++f) upw[f] = phi[f] >= 0.0 ? 1.0 : 0.0;
    for (int f = 0; f < nF; ++f) {
        M->lower[f] = -upw[f] * phi[f];
        M->upper[f] = (1.0 - upw[f]) * phi[f];
    }
    for (int f = 0; f < nF; ++f) {
        M->diag[m->owner[f]] -= M->lower[f];
        M->diag[m->neighbour[f]] -= M->upper[f];
    }
    for (int b = 0; b < m->nBFaces; ++b) {
        for (int k = 0; k < nc; ++k) {
            if (kind[b] == RT_BC_ZEROGRAD) {
                M->intC[nc * b + k] = phib[b] * 1.0;
                M->bouC[nc * b + k] = -phib[b] * 0.0;
            } else {
                M->intC[nc * b + k] = phib[b] * 0.0;
                M->bouC[nc * b + k] = -phib[b] * xb[nc * b + k];
            }
        }
    }
    if (scheme == RT_LIM_UPWIND || scheme == RT_LIM_NONE) { free(upw); return; }
    double al[3], be[3], bl[3];
    lims(scheme, al, be, bl);
    double *g = DALLOC(3 * (size_t)N);
    double *souT = DALLOC((size_t)nc * N);
    double *tf = DALLOC(nF);
    for (int k = 0; k < nc; ++k) {
        gauss_grad(m, x, xb, nc, k, g);
        for (int f = 0; f < nF; ++f) {
            int o = m->owner[f], n = m->neighbour[f];
            double d[3];
            for (int i = 0; i < 3; ++i)   /* C_N - C_P; across a cyclic face, the translated one */
                d[i] = m->delta ? m->delta[3 * f + i] : m->C[3 * n + i] - m->C[3 * o + i];
            double u = upw[f];
            double gu[3];
            for (int i = 0; i < 3; ++i) gu[i] = g[3 * o + i] * u + (1.0 - u) * g[3 * n + i];
            double gud = gu[0] * d[0] + gu[1] * d[1] + gu[2] * d[2];
            double xo = x[nc * o + k], xn = x[nc * n + k];
            double phitc = 1.0 - (xn - xo) / (2.0 * gud + 1e-18);
            double a, bb;
            if (phitc <= 0.0 || phitc >= 1.0) { a = 1.0; bb = 0.0; }
            else if (phitc < bl[0]) { a = al[0]; bb = be[0]; }
            else if (phitc < bl[1]) { a = al[1]; bb = be[1]; }
            else { a = al[2]; bb = be[2]; }
            double god = g[3 * o] * d[0] + g[3 * o + 1] * d[1] + g[3 * o + 2] * d[2];
            double gnd = g[3 * n] * d[0] + g[3 * n + 1] * d[1] + g[3 * n + 2] * d[2];
            tf[f] = (1.0 - a - bb) * (xn - 2.0 * god) * u
                  + (1.0 - a - bb) * (xo + 2.0 * gnd) * (1.0 - u)
                  + ((a - 1.0) * u + bb * (1.0 - u)) * xo
                  + (bb * u + (a - 1.0) * (1.0 - u)) * xn;
        }
        for (int f = 0; f < nF; ++f) {
            double s = tf[f] * phi[f];
            souT[nc * m->owner[f] + k] += s;
            souT[nc * m->neighbour[f] + k] -= s;
        }
    }
    for (size_t i = 0; i < (size_t)nc * N; ++i) M->source[i] = -souT[i];
    free(g); free(souT); free(tf); free(upw);
}

/* Euler implicit ddt: diag += V/dt, source += U0 V/dt */
static void add_ddt(const rt_mesh_desc *m, double rDeltaT, const double *x0, int nc, or_matrix *M) {
    for (int c = 0; c < m->nCells; ++c) {
        M->diag[c] += rDeltaT * m->V[c];
        for (int k = 0; k < nc; ++k) M->source[nc * c + k] += rDeltaT * x0[nc * c + k] * m->V[c];
    }
}

/* Crank-Nicolson ddt (see or_ddt): diag += (c/dt) V, source += ((c/dt) x0
 * + psi D) V; D == NULL is add_ddt */
static void add_ddt_cn(const rt_mesh_desc *m, double rDeltaT, double c, double psi, const double *x0,
                       const double *D, int nc, or_matrix *M) {
    if (!D) { add_ddt(m, rDeltaT, x0, nc, M); return; }
    const double rDtCoef = c * rDeltaT;
    for (int cl = 0; cl < m->nCells; ++cl) {
        M->diag[cl] += rDtCoef * m->V[cl];
        for (int k = 0; k < nc; ++k)
            M->source[nc * cl + k] += (rDtCoef * x0[nc * cl + k] + psi * D[nc * cl + k]) * m->V[cl];
    }
}

/* Solve all valid components of an nc-component matrix, fvMatrix::solveSegregated. */
static void solve_segregated(const rt_mesh_desc *m, or_matrix *M, double *x,
                             const int *valid, const rt_solver_ctl *ctl, rt_solver_perf *perf) {
    const int N = m->nCells, nc = M->nc;
    double *d = DALLOC(N), *b = DALLOC(N), *xc = DALLOC(N);
    for (int k = 0; k < nc; ++k) {
        if (!valid[k]) { perf[k].nIterations = -1; perf[k].initialResidual = perf[k].finalResidual = 0; perf[k].converged = 1; continue; }
        for (int c = 0; c < N; ++c) { d[c] = M->diag[c]; b[c] = M->source[nc * c + k]; xc[c] = x[nc * c + k]; }
        for (int bf = 0; bf < m->nBFaces; ++bf) {
            d[m->bCell[bf]] += M->intC[nc * bf + k];
            b[m->bCell[bf]] += M->bouC[nc * bf + k];
        }
        or_ldu_solve(m, d, M->upper, M->lower, b, xc, ctl, &perf[k]);
        for (int c = 0; c < N; ++c) x[nc * c + k] = xc[c];
    }
    free(d); free(b); free(xc);
}

/* ------------------------------------------------------------------------ */
/* constitutive update (boilerLog.H + <Model>Log::correct)                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    const rt_mesh_desc *m;
    const rt_bc_desc *bc;
    const rt_model_params *mp;
    const rt_case_ctl *ctl;
    or_state *s;
    int *kU, *kP, *kTh, *kTau;
    /* multiMode (nModes > 1): the modes' models and states (theta, tau and
     * the eigen fields of each; U, p and phi are s's), and where each mode's
     * theta solve records go (6 per mode, or NULL); s->tau is then the sum
     * of the modes' tau and mp the summed-viscosity model of the momentum
     * equation */
    int nModes;
    const rt_model_params *models;
    or_state *modes;
    rt_solver_perf *modePerf;
    /* Crank-Nicolson: the state (NULL for Euler), the coefficient c of the
     * current step and, for the theta equation of each mode, its D */
    or_ddt *ddt;
    double ddtC, ddtCth;
    const double *Dth;
    /* temperature-dependent parameters: per mode, 3 nCells shift factors
     * (lambda, the second relaxation time, etaP; mode i at 3 nCells i), or
     * NULL for the isothermal case */
    const double *thermo;
} or_case;

static void case_init(or_case *k, const rt_mesh_desc *m, const rt_bc_desc *bc,
                      const rt_model_params *mp, const rt_case_ctl *ctl, or_state *s) {
    k->m = m; k->bc = bc; k->mp = mp; k->ctl = ctl; k->s = s;
    k->nModes = 1; k->models = NULL; k->modes = NULL; k->modePerf = NULL;
    k->ddt = NULL; k->ddtC = 1.0; k->ddtCth = 1.0; k->Dth = NULL;
    k->thermo = NULL;
    int nB = m->nBFaces;
    k->kU = (int *)xcalloc(nB, sizeof(int)); k->kP = (int *)xcalloc(nB, sizeof(int));
    k->kTh = (int *)xcalloc(nB, sizeof(int)); k->kTau = (int *)xcalloc(nB, sizeof(int));
    bface_kinds(m, bc->U, k->kU); bface_kinds(m, bc->p, k->kP);
    bface_kinds(m, bc->theta, k->kTh); bface_kinds(m, bc->tau, k->kTau);
}
static void case_free(or_case *k) { free(k->kU); free(k->kP); free(k->kTh); free(k->kTau); }

/* tau boundary update, patches evaluated in order (GeometricField::
 * correctBoundaryConditions); linearExtrapolation: tau_b = tau_P +
 * grad(tau)_P . (Cf - C_P) with the gradient over the current boundary values. */
static void tau_correct_bc(or_case *k) {
    const rt_mesh_desc *m = k->m;
    or_state *s = k->s;
    const int N = m->nCells;
    double *g = NULL;
    for (int p = 0; p < m->nPatches; ++p) {
        int kind = k->bc->tau[p], st = m->patchStart[p], sz = m->patchSize[p];
        if (kind == RT_BC_ZEROGRAD) {
            for (int b = st; b < st + sz; ++b)
                for (int q = 0; q < 6; ++q) s->taub[6 * b + q] = s->tau[6 * m->bCell[b] + q];
        } else if (kind == RT_BC_LINEXTRAP) {
            if (!g) g = DALLOC(3 * (size_t)N);
            double *val = DALLOC(6 * (size_t)sz);
            for (int q = 0; q < 6; ++q) {
                gauss_grad(m, s->tau, s->taub, 6, q, g);
                for (int b = st; b < st + sz; ++b) {
                    int c = m->bCell[b];
                    double ctf[3] = {m->bCf[3 * b] - m->C[3 * c], m->bCf[3 * b + 1] - m->C[3 * c + 1],
                                     m->bCf[3 * b + 2] - m->C[3 * c + 2]};
                    val[6 * (b - st) + q] = s->tau[6 * c + q] +
                        (g[3 * c] * ctf[0] + g[3 * c + 1] * ctf[1] + g[3 * c + 2] * ctf[2]);
                }
            }
            for (int b = st; b < st + sz; ++b)
                for (int q = 0; q < 6; ++q) s->taub[6 * b + q] = val[6 * (b - st) + q];
            free(val);
        }
        /* fixedValue: unchanged */
    }
    free(g);
}

static void theta_valid(const rt_mesh_desc *m, int *valid) {
    /* symmTensor components solved: product of the solution directions */
    const int *sd = m->solveDir;
    int v[3] = {sd[0] ? 1 : -1, sd[1] ? 1 : -1, sd[2] ? 1 : -1};
    int ij[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    for (int q = 0; q < 6; ++q) valid[q] = (v[ij[q][0]] * v[ij[q][1]]) > 0;
}


/* Rolie-Poly: finite-extensibility factor and stretch rate M1 (RoliePolyLog.C:143-156) */
static double rp_chi(const rt_model_params *mp, double trA) {
    double c2 = mp->chiMax * mp->chiMax;
    return ((3.0 - (trA / 3.0) / c2) * (1.0 - 1.0 / c2)) / ((1.0 - (trA / 3.0) / c2) * (3.0 - 1.0 / c2));
}
static double rp_m1(const rt_model_params *mp, double trA) {
    double M1 = 2.0 * (1.0 - sqrt(3.0 / trA)) / mp->lambdaR;
    if (mp->chiMax > 1.0) M1 *= rp_chi(mp, trA);
    return M1;
}

/* generalized PTT (PTTLog.C:143-169): g[0] = Gamma(beta), then
 * Gamma(alpha k + beta) while k < maxIterMittagLeffler and the last value is
 * below 1e100; returns the number of series terms available (g holds one
 * more value) */
static int ml_table(const rt_model_params *mp, double *g) {
    g[0] = tgamma(mp->beta);
    int k = 0;
    while (k < mp->maxIterMittagLeffler && g[k] < 1e+100) {
        g[k + 1] = tgamma(mp->alpha * k + mp->beta);
        ++k;
    }
    return k;
}
/* E_{alpha,beta}(z) summed term by term (PTTLog.C:205-222) */
static double ml_sum(const rt_model_params *mp, const double *g, int K, double z) {
    double sum = 0.0, sumOld = 0.0, err = 1.0;
    int k = 0;
    while (k < K && err > mp->rTolMittagLeffler) {
        double t = pow(z, (double)k) / g[k + 1];
        sumOld = sum;
        sum += t;
        err = fabs((sumOld - sum) / (sumOld + 1e-12));
        ++k;
    }
    return sum;
}

/* XPomPom: f of the pre-solve conformation (XPomPomLog.C:148-163) */
static double xpp_f(const rt_model_params *mp, double trA, double trAA) {
    const double lam = sqrt(trA / 3.0), al = mp->alpha;
    const double stretch = (mp->n == 0.0) ? (1.0 - 1.0 / lam) : (1.0 - 1.0 / pow(lam, mp->n + 1.0));
    return ((2.0 * (mp->lambda / mp->lambdaS)) * exp((2.0 / mp->q) * (lam - 1.0))) * stretch +
           (1.0 / (lam * lam)) * (1.0 - al - (al / 3.0) * (trAA - 2.0 * trA));
}
/* ------------------------------------------------------------------------ */
/* thermoFunctions: the temperature shift factor a(T) of a parameter        */
/* ------------------------------------------------------------------------ */
/* the factor each function multiplies its constant by at temperature T
 * (thermoFunctions/<type>/<type>.C, multiply()): Constant.C:58-73 a = 1;
 * Arrhenius.C:61-76 exp(alpha (1/T - 1/T0)); ArrheniusModified.C:61-76
 * exp(-alpha (T - T0)); WLF.C:61-76 10^(-c1 (T - T0) / (c2 + (T - T0)));
 * VFT.C:62-77 10^(B + A / (T - T0)) */
double or_thermo_factor(const rt_thermo_fn *f, double T) {
    switch (f->type) {
    case RT_THERMO_ARRHENIUS: return exp(f->alpha * (1.0 / T - 1.0 / f->T0));
    case RT_THERMO_ARRHENIUS_MODIFIED: return exp(-f->alpha * (T - f->T0));
    case RT_THERMO_WLF: return pow(10.0, -f->c1 * (T - f->T0) / (f->c2 + (T - f->T0)));
    case RT_THERMO_VFT: return pow(10.0, f->B + f->A / (T - f->T0));
    default: return 1.0;
    }
}

/* a mode's factors of n cells: lambda, the second relaxation time and etaP
 * (out: 3 n, one array after the other) */
void or_thermo_factors(const rt_thermo_desc *d, int n, const double *T, double *out) {
    for (int c = 0; c < n; ++c) {
        out[c] = or_thermo_factor(&d->lambda, T[c]);
        out[n + c] = or_thermo_factor(&d->lambda2, T[c]);
        out[2 * (size_t)n + c] = or_thermo_factor(&d->eta, T[c]);
    }
}

/* the model of one cell with its relaxation times and etaP shifted
 * (createField(lambda_) and createField(etaP_) of the Log models'
 * correct(), e.g. Oldroyd_BLog.C:133-135; Rolie-Poly lambdaD / lambdaR and
 * XPomPom lambdaB / lambdaS by their own functions, RoliePolyLog.C:139-141,
 * XPomPomLog.C:140-142) */
static void thermo_shift(rt_model_params *mc, const double *th, int N, int c) {
    mc->lambda = mc->lambda * th[c];
    mc->lambdaR = mc->lambdaR * th[N + c];
    mc->lambdaS = mc->lambdaS * th[N + c];
    mc->etaP = mc->etaP * th[2 * (size_t)N + c];
}

/* WhiteMetznerCY: the Carreau-Yasuda factor of etaP and lambda at the shear
 * rate sqrt(2) |symm(L)| (WhiteMetznerCYLog.C:152-161, m = n, L = K, b = a) */
static double wmcy_factor(const rt_model_params *mp, const double *L) {
    double d2 = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double d = 0.5 * (L[3 * i + j] + L[3 * j + i]);
            d2 += d * d;
        }
    return pow(1.0 + pow((mp->K * sqrt(2.0)) * sqrt(d2), mp->a), (mp->n - 1.0) / mp->a);
}

/* the cell-local right-hand side of the theta equation,
 * symm(Omega theta - theta Omega + 2B + S_model), for n cells (AoS: L and
 * eigVecs 9 a cell, eigVals 3, theta and rhs 6); fP receives the FENE-P/CR f
 * of the pre-solve conformation and WhiteMetznerCY's etaP/lambda */
static void theta_source(const rt_model_params *mp0, int N, const double *L, const double *eigVecs,
                         const double *eigVals, const double *theta, double *rhs, double *fP,
                         const double *th) {
    const rt_model_params *mp = mp0;
    const double zeta = (mp->model == RT_MODEL_PTT_LOG) ? mp->zeta : 0.0;
    const int gen = mp->model == RT_MODEL_PTT_LOG && mp->pttFunction == RT_PTT_GENERALIZED;
    double *mlg = gen ? DALLOC((size_t)mp->maxIterMittagLeffler + 1) : NULL;
    const int mlK = gen ? ml_table(mp, mlg) : 0;

#pragma omp parallel for num_threads(nthreads_) schedule(static)
    for (int c = 0; c < N; ++c) {
        /* this cell's model: the temperature-shifted parameters, if any */
        rt_model_params mc = *mp0;
        if (th) thermo_shift(&mc, th, N, c);
        const rt_model_params *mp = &mc;
        const double lambda = mp->lambda, etaP = mp->etaP;
        t3 Lc, R, Lt, M;
        memcpy(Lc.a, L + 9 * (size_t)c, sizeof Lc.a);
        memcpy(R.a, eigVecs + 9 * (size_t)c, sizeof R.a);
        const double *ev = eigVals + 3 * (size_t)c;
        Lt = t3_T(Lc);
        if (mp->model == RT_MODEL_PTT_LOG) {
            /* L^T - zeta symm(L) */
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    Lt.a[3 * i + j] = Lt.a[3 * i + j] - zeta * (0.5 * (Lc.a[3 * i + j] + Lc.a[3 * j + i]));
        }
        M = t3_mul(t3_mul(t3_T(R), Lt), R);
        /* decomposeGradU */
        t3 om = t3_diag(0, 0, 0), Bt = t3_diag(M.a[0], M.a[4], M.a[8]);
        om.a[1] = (ev[1] * M.a[1] + ev[0] * M.a[3]) / (ev[1] - ev[0] + 1e-16);
        om.a[2] = (ev[2] * M.a[2] + ev[0] * M.a[6]) / (ev[2] - ev[0] + 1e-16);
        om.a[5] = (ev[2] * M.a[5] + ev[1] * M.a[7]) / (ev[2] - ev[1] + 1e-16);
        om.a[3] = -om.a[1]; om.a[6] = -om.a[2]; om.a[7] = -om.a[5];
        t3 Rt = t3_T(R);
        t3 Om = t3_mul(t3_mul(R, om), Rt);
        t3 B = t3_mul(t3_mul(R, Bt), Rt);
        /* model source */
        t3 S;
        t3 invm1 = t3_diag(1.0 / ev[0] - 1.0, 1.0 / ev[1] - 1.0, 1.0 / ev[2] - 1.0);
        t3 A = t3_mul(t3_mul(R, t3_diag(ev[0], ev[1], ev[2])), Rt);
        double trA = A.a[0] + A.a[4] + A.a[8];
        if (mp->model == RT_MODEL_OLDROYDB_LOG) {
            S = t3_mul(t3_mul(R, invm1), Rt);
            for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lambda) * S.a[i];
        } else if (mp->model == RT_MODEL_GIESEKUS_LOG) {
            t3 T = t3_mul(t3_mul(R, invm1), Rt);
            t3 ATT = t3_mul(A, t3_mul(T, T));
            for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lambda) * (T.a[i] - mp->alpha * ATT.a[i]);
        } else if (mp->model == RT_MODEL_PTT_LOG) {
            t3 T = t3_mul(t3_mul(R, invm1), Rt);
            const double z = (mp->epsilon / (1.0 - zeta)) * (trA - 3.0);
            double fac;
            if (mp->pttFunction == RT_PTT_EXP) fac = exp(z);
            else if (gen) fac = mlg[0] * ml_sum(mp, mlg, mlK, z);   /* PTTLog.C:201-236 */
            else fac = 1.0 + z;
            for (int i = 0; i < 9; ++i) S.a[i] = ((1.0 / lambda) * T.a[i]) * fac;
        } else if (mp->model == RT_MODEL_ROLIEPOLY_LOG) {
            /* RoliePolyLog.C:140-179: -(1/lambdaD) A^-1 ((A - I) + M1 lambdaD (A + beta (trA/3)^delta (A - I))) */
            t3 Ai = t3_mul(t3_mul(R, t3_diag(1.0 / ev[0], 1.0 / ev[1], 1.0 / ev[2])), Rt);
            double M1 = rp_m1(mp, trA);
            double ccr = mp->beta * pow(trA / 3.0, mp->delta);
            t3 G;
            for (int i = 0; i < 9; ++i) {
                double AmI = A.a[i] - ((i % 4 == 0) ? 1.0 : 0.0);
                G.a[i] = AmI + (M1 * lambda) * (A.a[i] + ccr * AmI);
            }
            t3 AG = t3_mul(Ai, G);
            for (int i = 0; i < 9; ++i) S.a[i] = -((1.0 / lambda) * AG.a[i]);
        } else if (mp->model == RT_MODEL_XPOMPOM_LOG) {
            /* XPomPomLog.C:165-185: -(1/lambdaB) A^-1 (A (f - 2 alpha) + alpha A.A + (alpha - 1) I) */
            t3 Ai = t3_mul(t3_mul(R, t3_diag(1.0 / ev[0], 1.0 / ev[1], 1.0 / ev[2])), Rt);
            t3 AA = t3_mul(A, A);
            const double al = mp->alpha;
            const double f = xpp_f(mp, trA, AA.a[0] + AA.a[4] + AA.a[8]);
            t3 G;
            for (int i = 0; i < 9; ++i)
                G.a[i] = (A.a[i] * (f - 2.0 * al) + al * AA.a[i]) + ((i % 4 == 0) ? (al - 1.0) : 0.0);
            t3 AG = t3_mul(Ai, G);
            for (int i = 0; i < 9; ++i) S.a[i] = -((1.0 / lambda) * AG.a[i]);
        } else if (mp->model == RT_MODEL_WHITEMETZNERCY_LOG) {
            /* WhiteMetznerCYLog.C:170-193, 203: (1/lambda(gd)) R (Lambda^-1 - I) R^T;
             * tau with etaP(gd)/lambda(gd) of the same pre-solve grad U */
            const double F = wmcy_factor(mp, Lc.a);
            const double lamc = lambda * F;
            fP[c] = (etaP * F) / lamc;
            S = t3_mul(t3_mul(R, invm1), Rt);
            for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lamc) * S.a[i];
        } else if (mp->model == RT_MODEL_FENECR_LOG) {
            /* FENE_CRLog.C:140-163 */
            double f = mp->L2 / (mp->L2 - trA);
            fP[c] = f;
            S = t3_mul(t3_mul(R, invm1), Rt);
            double lf = (1.0 / lambda) * f;
            for (int i = 0; i < 9; ++i) S.a[i] = lf * S.a[i];
        } else {
            double f = mp->L2 / (mp->L2 - trA);
            double a = mp->L2 / (mp->L2 - 3.0);
            fP[c] = f;
            t3 D = t3_diag(a * (1.0 / ev[0]) - f, a * (1.0 / ev[1]) - f, a * (1.0 / ev[2]) - f);
            S = t3_mul(t3_mul(R, D), Rt);
            for (int i = 0; i < 9; ++i) S.a[i] = (1.0 / lambda) * S.a[i];
        }
        t3 Th = t3_from_symm(theta + 6 * (size_t)c);
        t3 OT = t3_mul(Om, Th), TO = t3_mul(Th, Om);
        t3 Tsum;
        for (int i = 0; i < 9; ++i) Tsum.a[i] = OT.a[i] - TO.a[i] + 2.0 * B.a[i] + S.a[i];
        t3_symm(Tsum, rhs + 6 * (size_t)c);
    }
    free(mlg);
}

void or_theta_source(const rt_model_params *mp, int N, const double *L, const double *eigVecs,
                     const double *eigVals, const double *theta, double *rhs, double *fP) {
    theta_source(mp, N, L, eigVecs, eigVals, theta, rhs, fP, NULL);
}

/* tau of n cells from the post-solve eigen-decomposition (AoS) */
static void tau_cells(const rt_model_params *mp, int N, const double *eigVecs, const double *eigVals,
                      const double *fP, double *tau, const double *th) {
    const double zeta = (mp->model == RT_MODEL_PTT_LOG) ? mp->zeta : 0.0;
#pragma omp parallel for num_threads(nthreads_) schedule(static)
    for (int c = 0; c < N; ++c) {
        double lambda = mp->lambda, etaP = mp->etaP;
        if (th) {
            rt_model_params mc = *mp;
            thermo_shift(&mc, th, N, c);
            lambda = mc.lambda;
            etaP = mc.etaP;
        }
        double cP = etaP / lambda;
        if (mp->model == RT_MODEL_PTT_LOG) cP = etaP / (lambda * (1.0 - zeta));
        t3 R, Rt;
        memcpy(R.a, eigVecs + 9 * (size_t)c, sizeof R.a);
        Rt = t3_T(R);
        const double *ev = eigVals + 3 * (size_t)c;
        t3 A = t3_mul(t3_mul(R, t3_diag(ev[0], ev[1], ev[2])), Rt);
        t3 T;
        if (mp->model == RT_MODEL_FENEP_LOG) {
            double a = mp->L2 / (mp->L2 - 3.0);
            for (int i = 0; i < 9; ++i) T.a[i] = fP[c] * A.a[i];
            T.a[0] -= a; T.a[4] -= a; T.a[8] -= a;
        } else {
            T = A;
            T.a[0] -= 1.0; T.a[4] -= 1.0; T.a[8] -= 1.0;
        }
        double sy[6];
        t3_symm(T, sy);
        /* FENE-CR: (etaP/lambda) f symm(A - I) with the pre-solve f (FENE_CRLog.C:174);
         * Rolie-Poly: times the finite-extensibility factor of the new trA (RoliePolyLog.C:189-199) */
        double cPc = (mp->model == RT_MODEL_FENECR_LOG) ? cP * fP[c] : cP;
        if (mp->model == RT_MODEL_WHITEMETZNERCY_LOG) cPc = fP[c];
        if (mp->model == RT_MODEL_ROLIEPOLY_LOG && mp->chiMax > 1.0) cPc = cP * rp_chi(mp, A.a[0] + A.a[4] + A.a[8]);
        for (int q = 0; q < 6; ++q) tau[6 * (size_t)c + q] = cPc * sy[q];
    }
}

void or_tau_cells(const rt_model_params *mp, int N, const double *eigVecs, const double *eigVals,
                  const double *fP, double *tau) {
    tau_cells(mp, N, eigVecs, eigVals, fP, tau, NULL);
}

/* thetaOld: theta at the start of the time step (the inner iterations of a
 * step share it); NULL = the current theta */

static int constitutive_correct(or_case *k, const double *gradUin, rt_solver_perf *perf,
                                const double *thetaOld) {
    const rt_mesh_desc *m = k->m;
    const rt_model_params *mp = k->mp;
    or_state *s = k->s;
    const int N = m->nCells;
    double *L = DALLOC(9 * (size_t)N);
    if (gradUin) memcpy(L, gradUin, sizeof(double) * 9 * N);
    else grad_vector(m, s->U, s->Ub, L);
    double *rhs = DALLOC(6 * (size_t)N);
    double *fP = DALLOC(N);   /* FENE-P/CR f of the pre-solve conformation; WhiteMetznerCY etaP/lambda */
    theta_source(mp, N, L, s->eigVecs, s->eigVals, s->theta, rhs, fP, k->thermo);

    /* theta equation: ddt + GaussDefCmpw == rhs */
    or_matrix Mx;
    mat_alloc(&Mx, m, 6);
    double *theta0 = DALLOC(6 * (size_t)N);
    memcpy(theta0, thetaOld ? thetaOld : s->theta, sizeof(double) * 6 * N);
    or_matrix Md;
    mat_alloc(&Md, m, 6);
    add_ddt_cn(m, 1.0 / k->ctl->deltaT, k->ddtCth, k->ddt ? k->ddt->psi : 0.0, theta0, k->Dth, 6, &Mx);
    defcmpw(m, k->ctl->divTheta, s->phi, s->phib, s->theta, s->thetab, k->kTh, 6, &Md);
    for (int c = 0; c < N; ++c) Mx.diag[c] += Md.diag[c];
    for (int f = 0; f < m->nFaces; ++f) { Mx.lower[f] = Md.lower[f]; Mx.upper[f] = Md.upper[f]; }
    for (size_t i = 0; i < 6 * (size_t)N; ++i) Mx.source[i] += Md.source[i];
    for (size_t i = 0; i < 6 * (size_t)m->nBFaces; ++i) { Mx.intC[i] = Md.intC[i]; Mx.bouC[i] = Md.bouC[i]; }
    for (int c = 0; c < N; ++c)
        for (int q = 0; q < 6; ++q) Mx.source[6 * c + q] += m->V[c] * rhs[6 * c + q];
    int valid[6];
    theta_valid(m, valid);
    solve_segregated(m, &Mx, s->theta, valid, &k->ctl->solverTheta, perf);
    correct_bc(m, k->kTh, s->theta, s->thetab, 6);

    /* calcEig and tau */
    or_eig(N, s->theta, s->eigVals, s->eigVecs);
    tau_cells(mp, N, s->eigVecs, s->eigVals, fP, s->tau, k->thermo);
    tau_correct_bc(k);

    int st = RT_OK;
    for (int q = 0; q < 6; ++q) if (valid[q] && !isfinite(perf[q].finalResidual)) st = RT_ENAN;
    mat_free(&Mx); mat_free(&Md);
    free(theta0); free(L); free(rhs); free(fP);
    return st;
}

int or_constitutive_correct(const rt_mesh_desc *m, const rt_bc_desc *bc,
                            const rt_model_params *mp, const rt_case_ctl *ctl,
                            or_state *s, const double *gradU, rt_solver_perf *perf) {
    or_case k;
    case_init(&k, m, bc, mp, ctl, s);
    int st = constitutive_correct(&k, gradU, perf, NULL);
    case_free(&k);
    return st;
}

/* the same with the theta equation's old-time field given (AoS 6 nCells):
 * an inner iteration of a time step that started from thetaOld */
int or_constitutive_correct_old(const rt_mesh_desc *m, const rt_bc_desc *bc,
                                const rt_model_params *mp, const rt_case_ctl *ctl,
                                or_state *s, const double *gradU, const double *thetaOld,
                                rt_solver_perf *perf) {
    or_case k;
    case_init(&k, m, bc, mp, ctl, s);
    int st = constitutive_correct(&k, gradU, perf, thetaOld);
    case_free(&k);
    return st;
}

/* ------------------------------------------------------------------------ */
/* explicit divergences used by divTau                                        */
/* ------------------------------------------------------------------------ */
/* sum over faces of Sf . T_f for a symmTensor field T (cells + boundary), then /V */
static void div_symm(const rt_mesh_desc *m, const double *T, const double *Tb, double scale,
                     double *out /*3N*/) {
    const int N = m->nCells;
    memset(out, 0, sizeof(double) * 3 * (size_t)N);
    for (int f = 0; f < m->nFaces; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double Tf[6];
        for (int q = 0; q < 6; ++q)
            Tf[q] = lin_interp(m->weights[f], T[6 * o + q] / scale, T[6 * n + q] / scale);
        const double *S = m->Sf + 3 * f;
        double v[3] = {S[0] * Tf[0] + S[1] * Tf[1] + S[2] * Tf[2],
                       S[0] * Tf[1] + S[1] * Tf[3] + S[2] * Tf[4],
                       S[0] * Tf[2] + S[1] * Tf[4] + S[2] * Tf[5]};
        for (int d = 0; d < 3; ++d) { out[3 * o + d] += v[d]; out[3 * n + d] -= v[d]; }
    }
    for (int b = 0; b < m->nBFaces; ++b) {
        int c = m->bCell[b];
        double Tf[6];
        for (int q = 0; q < 6; ++q) Tf[q] = Tb[6 * b + q] / scale;
        const double *S = m->bSf + 3 * b;
        out[3 * c + 0] += S[0] * Tf[0] + S[1] * Tf[1] + S[2] * Tf[2];
        out[3 * c + 1] += S[0] * Tf[1] + S[1] * Tf[3] + S[2] * Tf[4];
        out[3 * c + 2] += S[0] * Tf[2] + S[1] * Tf[4] + S[2] * Tf[5];
    }
    for (int c = 0; c < N; ++c)
        for (int d = 0; d < 3; ++d) out[3 * c + d] /= m->V[c];
}

/* div(k * G) for a full tensor field G (cells) with boundary values Gb */
static void div_tensor(const rt_mesh_desc *m, const double *G, const double *Gb, double k,
                       double *out) {
    const int N = m->nCells;
    memset(out, 0, sizeof(double) * 3 * (size_t)N);
    for (int f = 0; f < m->nFaces; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double Gf[9];
        for (int q = 0; q < 9; ++q) Gf[q] = lin_interp(m->weights[f], k * G[9 * o + q], k * G[9 * n + q]);
        const double *S = m->Sf + 3 * f;
        for (int j = 0; j < 3; ++j) {
            double v = S[0] * Gf[j] + S[1] * Gf[3 + j] + S[2] * Gf[6 + j];
            out[3 * o + j] += v; out[3 * n + j] -= v;
        }
    }
    for (int b = 0; b < m->nBFaces; ++b) {
        int c = m->bCell[b];
        const double *S = m->bSf + 3 * b;
        for (int j = 0; j < 3; ++j)
            out[3 * c + j] += S[0] * (k * Gb[9 * b + j]) + S[1] * (k * Gb[9 * b + 3 + j]) +
                              S[2] * (k * Gb[9 * b + 6 + j]);
    }
    for (int c = 0; c < N; ++c)
        for (int d = 0; d < 3; ++d) out[3 * c + d] /= m->V[c];
}

/* fvc::laplacian(k, U), Gauss linear orthogonal, per component */
static void fvc_laplacian(const rt_mesh_desc *m, const double *U, const double *Ub, double k,
                          double *out) {
    const int N = m->nCells;
    memset(out, 0, sizeof(double) * 3 * (size_t)N);
    for (int f = 0; f < m->nFaces; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double gm = k * m->magSf[f];
        for (int j = 0; j < 3; ++j) {
            double v = gm * (m->deltaCoeffs[f] * (U[3 * n + j] - U[3 * o + j]));
            out[3 * o + j] += v; out[3 * n + j] -= v;
        }
    }
    for (int b = 0; b < m->nBFaces; ++b) {
        int c = m->bCell[b];
        double gm = k * m->bmagSf[b];
        for (int j = 0; j < 3; ++j)
            out[3 * c + j] += gm * (m->bDeltaCoeffs[b] * (Ub[3 * b + j] - U[3 * c + j]));
    }
    for (int c = 0; c < N; ++c)
        for (int d = 0; d < 3; ++d) out[3 * c + d] /= m->V[c];
}

/* ------------------------------------------------------------------------ */
/* multiMode (multiMode.C:69-91, 144-156, 222, 247-256)                       */
/* ------------------------------------------------------------------------ */
/* correct() of every mode in turn, each with its own model and its own
 * theta, tau and eigen fields on the common U and phi; then tau() = the sum
 * of the modes' tau (internal and boundary values).  theta0s: the modes'
 * old-time theta, mode after mode (NULL: their current theta).  perf gets the
 * last mode's records, k->modePerf (if set) every mode's. */
static int modes_correct(or_case *k, const double *gradU, rt_solver_perf *perf, const double *theta0s) {
    const rt_mesh_desc *m = k->m;
    or_state *s = k->s;
    const size_t n6 = 6 * (size_t)m->nCells, b6 = 6 * (size_t)m->nBFaces;
    int st = RT_OK;
    for (int i = 0; i < k->nModes && st == RT_OK; ++i) {
        or_state si = k->modes[i];
        si.U = s->U; si.Ub = s->Ub; si.p = s->p; si.pb = s->pb; si.phi = s->phi; si.phib = s->phib;
        or_case ki = *k;
        ki.mp = &k->models[i];
        ki.s = &si;
        ki.nModes = 1;
        ki.Dth = k->Dth ? k->Dth + n6 * i : NULL;
        ki.thermo = k->thermo ? k->thermo + 3 * (size_t)m->nCells * i : NULL;
        rt_solver_perf *pi = k->modePerf ? k->modePerf + 6 * i : perf;
        st = constitutive_correct(&ki, gradU, pi, theta0s ? theta0s + n6 * i : NULL);
        if (pi != perf) memcpy(perf, pi, 6 * sizeof *perf);
    }
    memset(s->tau, 0, sizeof(double) * n6);
    memset(s->taub, 0, sizeof(double) * b6);
    for (int i = 0; i < k->nModes; ++i) {
        for (size_t j = 0; j < n6; ++j) s->tau[j] += k->modes[i].tau[j];
        for (size_t j = 0; j < b6; ++j) s->taub[j] += k->modes[i].taub[j];
    }
    return st;
}

/* The momentum equation of a multiMode model: the sum of the modes' divTau
 * (multiMode.C:144-156).  With a common rho and stabilization it is one
 * divTau with the summed tau (s->tau) and the summed etaS and etaP; mode 0's
 * model carries the rest. */
static rt_model_params modes_momentum_model(const rt_model_params *models, int nModes) {
    rt_model_params e = models[0];
    e.etaS = 0.0;
    e.etaP = 0.0;
    for (int i = 0; i < nModes; ++i) {
        e.etaS += models[i].etaS;
        e.etaP += models[i].etaP;
    }
    return e;
}

/* ------------------------------------------------------------------------ */
/* one segregated rheoFoam step                                               */
/* ------------------------------------------------------------------------ */
/* One inner iteration of a time step: UEqn, pEqn and constEq.correct() with
 * the old-time fields of the step (U, phi and theta at its start). */
static int step_inner(or_case *k, rt_step_perf *perf, const double *U0s, const double *U0bs,
                      const double *phi0s, const double *phi0bs, const double *theta0s) {
    const rt_mesh_desc *m = k->m;
    const rt_model_params *mp = k->mp;
    const rt_case_ctl *ctl = k->ctl;
    or_state *s = k->s;
    const int N = m->nCells, nF = m->nFaces, nB = m->nBFaces;
    const double rDeltaT = 1.0 / ctl->deltaT;
    const double rho = mp->rho;

    /* old-time fields */
    double *U0 = DALLOC(3 * (size_t)N), *U0b = DALLOC(3 * (size_t)nB);
    double *phi0 = DALLOC(nF), *phi0b = DALLOC(nB);
    memcpy(U0, U0s, sizeof(double) * 3 * N); memcpy(U0b, U0bs, sizeof(double) * 3 * nB);
    memcpy(phi0, phi0s, sizeof(double) * nF); memcpy(phi0b, phi0bs, sizeof(double) * nB);

    /* ---------------- UEqn ---------------- */
    double *G = DALLOC(9 * (size_t)N), *Gb = DALLOC(9 * (size_t)nB);
    grad_vector(m, s->U, s->Ub, G);
    or_matrix UE;
    mat_alloc(&UE, m, 3);
    add_ddt_cn(m, rDeltaT, k->ddtC, k->ddt ? k->ddt->psi : 0.0, U0, k->ddt ? k->ddt->DU : NULL, 3, &UE);
    or_matrix Cv;
    mat_alloc(&Cv, m, 3);
    defcmpw(m, ctl->divU, s->phi, s->phib, s->U, s->Ub, k->kU, 3, &Cv);
    for (int c = 0; c < N; ++c) UE.diag[c] += Cv.diag[c];
    for (int f = 0; f < nF; ++f) { UE.lower[f] = Cv.lower[f]; UE.upper[f] = Cv.upper[f]; }
    for (size_t i = 0; i < 3 * (size_t)N; ++i) UE.source[i] += Cv.source[i];
    for (size_t i = 0; i < 3 * (size_t)nB; ++i) { UE.intC[i] = Cv.intC[i]; UE.bouC[i] = Cv.bouC[i]; }

    /* divTau: explicit part and implicit laplacian coefficient */
    double gam;
    double *expl = DALLOC(3 * (size_t)N), *tmp = DALLOC(3 * (size_t)N);
    div_symm(m, s->tau, s->taub, rho, expl);            /* fvc::div(tau/rho) */
    if (mp->stabilization == RT_STAB_COUPLING) {
        grad_boundary(m, G, s->U, s->Ub, Gb);
        div_tensor(m, G, Gb, mp->etaP / rho, tmp);      /* fvc::div(etaP/rho grad U) */
        for (size_t i = 0; i < 3 * (size_t)N; ++i) expl[i] -= tmp[i];
        gam = (mp->etaP + mp->etaS) / rho;
    } else if (mp->stabilization == RT_STAB_BSD) {
        fvc_laplacian(m, s->U, s->Ub, mp->etaP / rho, tmp);
        for (size_t i = 0; i < 3 * (size_t)N; ++i) expl[i] -= tmp[i];
        gam = (mp->etaP + mp->etaS) / rho;
    } else {
        gam = mp->etaS / rho;
    }
    /* - fvm::laplacian(gam, U): orthogonal Gauss linear; the laplacian matrix
     * (upper = gam |Sf| deltaCoeffs, diag = -sum of upper) is built first and
     * then subtracted, as fvMatrix operator- does */
    {
        double *ld = DALLOC(N);
        for (int f = 0; f < nF; ++f) {
            double up = gam * m->magSf[f] * m->deltaCoeffs[f];
            ld[m->owner[f]] -= up;
            ld[m->neighbour[f]] -= up;
            UE.upper[f] -= up;
            UE.lower[f] -= up;
        }
        for (int c = 0; c < N; ++c) UE.diag[c] -= ld[c];
        free(ld);
    }
    for (int b = 0; b < nB; ++b) {
        if (k->kU[b] == RT_BC_FIXED) {
            double gm = gam * m->bmagSf[b];
            for (int j = 0; j < 3; ++j) {
                UE.intC[3 * b + j] -= gm * (-m->bDeltaCoeffs[b]);
                UE.bouC[3 * b + j] -= -gm * (m->bDeltaCoeffs[b] * s->Ub[3 * b + j]);
            }
        }
    }
    /* explicit divTau terms plus the uniform body force per unit mass (the
     * pressure-gradient source that drives a periodic channel) */
    for (int c = 0; c < N; ++c)
        for (int j = 0; j < 3; ++j) UE.source[3 * c + j] += m->V[c] * (expl[3 * c + j] + ctl->bodyForce[j]);

    /* solve(UEqn == -grad(p)) */
    double *gp = DALLOC(3 * (size_t)N);
    gauss_grad(m, s->p, s->pb, 1, 0, gp);
    or_matrix US = UE;  /* shares coefficient arrays; only the source differs */
    US.source = DALLOC(3 * (size_t)N);
    for (int c = 0; c < N; ++c)
        for (int j = 0; j < 3; ++j)
            US.source[3 * c + j] = UE.source[3 * c + j] + m->V[c] * (-gp[3 * c + j]);
    int validU[3] = {m->solveDir[0] != 0, m->solveDir[1] != 0, m->solveDir[2] != 0};
    solve_segregated(m, &US, s->U, validU, &ctl->solverU, perf->U);
    free(US.source);
    correct_bc(m, k->kU, s->U, s->Ub, 3);

    /* ---------------- pEqn ---------------- */
    double *rAU = DALLOC(N), *H = DALLOC(3 * (size_t)N), *H1 = DALLOC(N);
    double *HbyA = DALLOC(3 * (size_t)N), *HbyAb = DALLOC(3 * (size_t)nB);
    /* A = (diag + cmptAv(internalCoeffs))/V */
    for (int c = 0; c < N; ++c) rAU[c] = UE.diag[c];
    for (int b = 0; b < nB; ++b)
        rAU[m->bCell[b]] += (UE.intC[3 * b] + UE.intC[3 * b + 1] + UE.intC[3 * b + 2]) / 3.0;
    for (int c = 0; c < N; ++c) rAU[c] = 1.0 / (rAU[c] / m->V[c]);
    /* H: (D_avg - D_cmpt) U - sum_nb a_nb U_nb + b + boundary source, over V */
    for (int b = 0; b < nB; ++b) {
        int c = m->bCell[b];
        double av = (UE.intC[3 * b] + UE.intC[3 * b + 1] + UE.intC[3 * b + 2]) / 3.0;
        for (int j = 0; j < 3; ++j) H[3 * c + j] += (av - UE.intC[3 * b + j]) * s->U[3 * c + j];
    }
    for (int f = 0; f < nF; ++f) {
        int l = m->owner[f], u = m->neighbour[f];
        for (int j = 0; j < 3; ++j) {
            H[3 * u + j] -= UE.lower[f] * s->U[3 * l + j];
            H[3 * l + j] -= UE.upper[f] * s->U[3 * u + j];
        }
        H1[u] -= UE.lower[f];
        H1[l] -= UE.upper[f];
    }
    for (size_t i = 0; i < 3 * (size_t)N; ++i) H[i] += UE.source[i];
    for (int b = 0; b < nB; ++b)
        for (int j = 0; j < 3; ++j) H[3 * m->bCell[b] + j] += UE.bouC[3 * b + j];
    for (int c = 0; c < N; ++c) {
        for (int j = 0; j < 3; ++j) H[3 * c + j] /= m->V[c];
        H1[c] /= m->V[c];
    }
    for (int c = 0; c < N; ++c)
        for (int j = 0; j < 3; ++j) HbyA[3 * c + j] = rAU[c] * H[3 * c + j];
    for (int b = 0; b < nB; ++b) {
        int c = m->bCell[b];
        for (int j = 0; j < 3; ++j)
            HbyAb[3 * b + j] = (k->kU[b] == RT_BC_FIXED) ? s->Ub[3 * b + j] : rAU[c] * H[3 * c + j];
    }
    /* phiHbyA = flux(HbyA) + interpolate(rAU) ddtCorr(U, phi) */
    double *phiHbyA = DALLOC(nF), *phiHbyAb = DALLOC(nB);
    for (int f = 0; f < nF; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double w = m->weights[f];
        const double *S = m->Sf + 3 * f;
        double hf = 0.0, u0f = 0.0;
        for (int j = 0; j < 3; ++j) {
            hf += S[j] * lin_interp(w, HbyA[3 * o + j], HbyA[3 * n + j]);
            u0f += S[j] * lin_interp(w, U0[3 * o + j], U0[3 * n + j]);
        }
        double phiCorr = phi0[f] - u0f;
        double cc = 1.0 - fmin(fabs(phiCorr) / (fabs(phi0[f]) + OR_SMALL), 1.0);
        double ddtCorr = cc * rDeltaT * phiCorr;
        if (k->ddt) {
            /* Crank-Nicolson: the old-time parts c/dt x0 + psi D of phi and U */
            const or_ddt *d = k->ddt;
            const double rc = k->ddtC * rDeltaT;
            double uf = 0.0;
            for (int j = 0; j < 3; ++j)
                uf += S[j] * lin_interp(w, rc * U0[3 * o + j] + d->psi * d->DU[3 * o + j],
                                        rc * U0[3 * n + j] + d->psi * d->DU[3 * n + j]);
            ddtCorr = cc * ((rc * phi0[f] + d->psi * d->Dphi[f]) - uf);
        }
        phiHbyA[f] = hf + lin_interp(w, rAU[o], rAU[n]) * ddtCorr;
    }
    for (int b = 0; b < nB; ++b) {
        int c = m->bCell[b];
        const double *S = m->bSf + 3 * b;
        double hf = S[0] * HbyAb[3 * b] + S[1] * HbyAb[3 * b + 1] + S[2] * HbyAb[3 * b + 2];
        double u0f = S[0] * U0b[3 * b] + S[1] * U0b[3 * b + 1] + S[2] * U0b[3 * b + 2];
        double phiCorr = phi0b[b] - u0f;
        double cc = (k->kU[b] == RT_BC_FIXED) ? 0.0
                  : 1.0 - fmin(fabs(phiCorr) / (fabs(phi0b[b]) + OR_SMALL), 1.0);
        double ddtCorr = cc * rDeltaT * phiCorr;
        if (k->ddt) {
            const or_ddt *d = k->ddt;
            const double rc = k->ddtC * rDeltaT;
            double uf = 0.0;
            for (int j = 0; j < 3; ++j) uf += S[j] * (rc * U0b[3 * b + j] + d->psi * d->DUb[3 * b + j]);
            ddtCorr = cc * ((rc * phi0b[b] + d->psi * d->Dphib[b]) - uf);
        }
        phiHbyAb[b] = hf + rAU[c] * ddtCorr;
    }
    /* adjustCorrPhi when p needs a reference */
    if (ctl->needReference) {
        double massIn = 0, fixedOut = 0, adjOut = 0, total = 1e-300;
        for (int f = 0; f < nF; ++f) total += fabs(phiHbyA[f]);
        for (int b = 0; b < nB; ++b) {
            if (phiHbyAb[b] < 0.0) massIn -= phiHbyAb[b];
            else if (k->kU[b] == RT_BC_FIXED) fixedOut += phiHbyAb[b];
            else adjOut += phiHbyAb[b];
        }
        if (fabs(adjOut) > 1e-300 && fabs(adjOut) / total > OR_SMALL) {
            double corr = (massIn - fixedOut) / adjOut;
            for (int b = 0; b < nB; ++b)
                if (k->kU[b] != RT_BC_FIXED && phiHbyAb[b] > 0.0) phiHbyAb[b] *= corr;
        } else if (fabs(fixedOut - massIn) / total > 1e-8) {
            fprintf(stderr, "oracle: continuity error cannot be removed by adjusting the outflow\n");
        }
    }
    double *rAtU = DALLOC(N);
    for (int c = 0; c < N; ++c) rAtU[c] = 1.0 / (1.0 / rAU[c] - H1[c]);
    /* phiHbyA += interpolate(rAtU - rAU) snGrad(p) |Sf| */
    for (int f = 0; f < nF; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double dr = lin_interp(m->weights[f], rAtU[o] - rAU[o], rAtU[n] - rAU[n]);
        phiHbyA[f] += dr * (m->deltaCoeffs[f] * (s->p[n] - s->p[o])) * m->magSf[f];
    }
    for (int b = 0; b < nB; ++b) {
        int c = m->bCell[b];
        double sn = (k->kP[b] == RT_BC_FIXED) ? m->bDeltaCoeffs[b] * (s->pb[b] - s->p[c]) : 0.0;
        phiHbyAb[b] += (rAtU[c] - rAU[c]) * sn * m->bmagSf[b];
    }
    /* HbyA -= (rAU - rAtU) grad p */
    for (int c = 0; c < N; ++c)
        for (int j = 0; j < 3; ++j) HbyA[3 * c + j] -= (rAU[c] - rAtU[c]) * gp[3 * c + j];

    /* pEqn: laplacian(rAtU, p) == div(phiHbyA) */
    double *pd = DALLOC(N), *pu = DALLOC(nF), *ps = DALLOC(N);
    double *pIntC = DALLOC(nB), *pBouC = DALLOC(nB);
    for (int f = 0; f < nF; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double gm = lin_interp(m->weights[f], rAtU[o], rAtU[n]) * m->magSf[f];
        pu[f] = m->deltaCoeffs[f] * gm;
        pd[o] -= pu[f];
        pd[n] -= pu[f];
    }
    for (int b = 0; b < nB; ++b) {
        if (k->kP[b] == RT_BC_FIXED) {
            double gm = rAtU[m->bCell[b]] * m->bmagSf[b];
            pIntC[b] = gm * (-m->bDeltaCoeffs[b]);
            pBouC[b] = -gm * (m->bDeltaCoeffs[b] * s->pb[b]);
        }
    }
    {
        double *dv = DALLOC(N);
        for (int f = 0; f < nF; ++f) { dv[m->owner[f]] += phiHbyA[f]; dv[m->neighbour[f]] -= phiHbyA[f]; }
        for (int b = 0; b < nB; ++b) dv[m->bCell[b]] += phiHbyAb[b];
        for (int c = 0; c < N; ++c) ps[c] += m->V[c] * (dv[c] / m->V[c]);
        free(dv);
    }
    if (ctl->needReference) {
        int r = ctl->pRefCell;
        ps[r] += pd[r] * ctl->pRefValue;
        pd[r] += pd[r];
    }
    {
        double *d2 = DALLOC(N), *b2 = DALLOC(N);
        memcpy(d2, pd, sizeof(double) * N);
        memcpy(b2, ps, sizeof(double) * N);
        for (int b = 0; b < nB; ++b) { d2[m->bCell[b]] += pIntC[b]; b2[m->bCell[b]] += pBouC[b]; }
        /* the non-orthogonal corrector loop (pEqn.H:31-50): with the orthogonal
         * laplacian the equation is the same each time; every solve starts
         * from the last one's p, the flux follows the last */
        const int nCorr = ctl->nNonOrthCorr > 0 ? ctl->nNonOrthCorr : 0;
        for (int corr = 0; corr <= nCorr; ++corr) {
            or_ldu_solve(m, d2, pu, pu, b2, s->p, &ctl->solverP, &perf->p);
            correct_bc(m, k->kP, s->p, s->pb, 1);
        }
        free(d2); free(b2);
    }
    /* phi = phiHbyA - pEqn.flux() */
    for (int f = 0; f < nF; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        s->phi[f] = phiHbyA[f] - (pu[f] * s->p[n] - pu[f] * s->p[o]);
    }
    for (int b = 0; b < nB; ++b)
        s->phib[b] = phiHbyAb[b] - (pIntC[b] * s->p[m->bCell[b]] - pBouC[b]);
    /* continuity errors (diagnostic) */
    {
        double *dv = DALLOC(N);
        for (int f = 0; f < nF; ++f) { dv[m->owner[f]] += s->phi[f]; dv[m->neighbour[f]] -= s->phi[f]; }
        for (int b = 0; b < nB; ++b) dv[m->bCell[b]] += s->phib[b];
        double sl = 0, gl = 0, vt = 0;
        for (int c = 0; c < N; ++c) { sl += fabs(dv[c]); gl += dv[c]; vt += m->V[c]; }
        perf->contErrSumLocal = ctl->deltaT * sl / vt;
        perf->contErrGlobal = ctl->deltaT * gl / vt;
        free(dv);
    }
    /* U = HbyA - rAtU grad p */
    gauss_grad(m, s->p, s->pb, 1, 0, gp);
    for (int c = 0; c < N; ++c)
        for (int j = 0; j < 3; ++j) s->U[3 * c + j] = HbyA[3 * c + j] - rAtU[c] * gp[3 * c + j];
    correct_bc(m, k->kU, s->U, s->Ub, 3);

    free(pd); free(pu); free(ps); free(pIntC); free(pBouC);
    free(rAU); free(H); free(H1); free(HbyA); free(HbyAb); free(phiHbyA); free(phiHbyAb);
    free(rAtU); free(gp); free(expl); free(tmp);
    mat_free(&UE);
    mat_free(&Cv);
    free(G); free(Gb);
    free(U0); free(U0b); free(phi0); free(phi0b);

    /* ---------------- constEq.correct() ---------------- */
    if (k->nModes <= 1) return constitutive_correct(k, NULL, perf->theta, theta0s);
    return modes_correct(k, NULL, perf->theta, theta0s);
}

/* One time step: nInIter inner iterations (rheoFoam.C:96-150; createControls.H
 * nInIter, 0 meaning 1) on the old-time fields of the step. */
/* Start of a Crank-Nicolson time step (see or_ddt): the old-time
 * derivatives D of the step that ended, from the fields now and at that
 * step's start; then the start fields become the current ones.  flow: U and
 * phi too (rt_step), else the theta equations only (a correct() of its own). */
static void ddt_begin_step(or_case *k, int flow) {
    or_ddt *d = k->ddt;
    if (!d || d->scheme != RT_DDT_CRANKNICOLSON) return;
    const rt_mesh_desc *m = k->m;
    or_state *s = k->s;
    const size_t N = m->nCells, nF = m->nFaces, nB = m->nBFaces;
    const int nM = k->nModes > 1 ? k->nModes : 1;
    const double rDt = 1.0 / k->ctl->deltaT, psi = d->psi;
    if (flow) {
        if (d->nSteps >= 1) {
            const double r = ddt_coef(d, d->nSteps - 1) * rDt;
            for (size_t i = 0; i < 3 * N; ++i) d->DU[i] = r * (s->U[i] - d->Us[i]) - psi * d->DU[i];
            for (size_t i = 0; i < 3 * nB; ++i) d->DUb[i] = r * (s->Ub[i] - d->Ubs[i]) - psi * d->DUb[i];
            for (size_t i = 0; i < nF; ++i) d->Dphi[i] = r * (s->phi[i] - d->phis[i]) - psi * d->Dphi[i];
            for (size_t i = 0; i < nB; ++i) d->Dphib[i] = r * (s->phib[i] - d->phibs[i]) - psi * d->Dphib[i];
        }
        memcpy(d->Us, s->U, sizeof(double) * 3 * N);
        memcpy(d->Ubs, s->Ub, sizeof(double) * 3 * nB);
        memcpy(d->phis, s->phi, sizeof(double) * nF);
        memcpy(d->phibs, s->phib, sizeof(double) * nB);
        d->nSteps++;
        k->ddtC = ddt_coef(d, d->nSteps - 1);
    }
    for (int i = 0; i < nM; ++i) {
        const double *th = k->nModes > 1 ? k->modes[i].theta : s->theta;
        double *D = d->Dth + 6 * N * i, *ts = d->ths + 6 * N * i;
        if (d->nThSteps >= 1) {
            const double r = ddt_coef(d, d->nThSteps - 1) * rDt;
            for (size_t j = 0; j < 6 * N; ++j) D[j] = r * (th[j] - ts[j]) - psi * D[j];
        }
        memcpy(ts, th, sizeof(double) * 6 * N);
    }
    d->nThSteps++;
    k->ddtCth = ddt_coef(d, d->nThSteps - 1);
    k->Dth = d->Dth;
}

static int step_once(or_case *k, rt_step_perf *perf) {
    const rt_mesh_desc *m = k->m;
    or_state *s = k->s;
    const int N = m->nCells, nF = m->nFaces, nB = m->nBFaces;
    const int nM = k->nModes > 1 ? k->nModes : 1;
    ddt_begin_step(k, 1);
    double *U0 = DALLOC(3 * (size_t)N), *U0b = DALLOC(3 * (size_t)nB);
    double *phi0 = DALLOC(nF), *phi0b = DALLOC(nB), *theta0 = DALLOC(6 * (size_t)N * nM);
    memcpy(U0, s->U, sizeof(double) * 3 * N); memcpy(U0b, s->Ub, sizeof(double) * 3 * nB);
    memcpy(phi0, s->phi, sizeof(double) * nF); memcpy(phi0b, s->phib, sizeof(double) * nB);
    if (k->nModes > 1)
        for (int i = 0; i < nM; ++i) memcpy(theta0 + 6 * (size_t)N * i, k->modes[i].theta, sizeof(double) * 6 * N);
    else
        memcpy(theta0, s->theta, sizeof(double) * 6 * N);
    const int nIn = k->ctl->nInIter > 1 ? k->ctl->nInIter : 1;
    int st = RT_OK;
    for (int it = 0; it < nIn && st == RT_OK; ++it) {
        memset(perf, 0, sizeof *perf);
        st = step_inner(k, perf, U0, U0b, phi0, phi0b, theta0);
    }
    free(U0); free(U0b); free(phi0); free(phi0b); free(theta0);
    return st;
}

int or_step(const rt_mesh_desc *m, const rt_bc_desc *bc, const rt_model_params *mp,
            const rt_case_ctl *ctl, or_state *s, int nSteps, rt_step_perf *perf) {
    if (ctl->ddtScheme != RT_DDT_EULER) return RT_EINVAL;   /* Crank-Nicolson keeps state: or_step_ddt */
    or_case k;
    case_init(&k, m, bc, mp, ctl, s);
    rt_step_perf local;
    int st = RT_OK;
    for (int i = 0; i < nSteps && st == RT_OK; ++i) {
        memset(&local, 0, sizeof local);
        st = step_once(&k, &local);
        if (st == RT_OK) {
            if (!isfinite(local.p.finalResidual)) st = RT_ENAN;
            for (int j = 0; j < 3; ++j) if (local.U[j].nIterations >= 0 && !isfinite(local.U[j].finalResidual)) st = RT_ENAN;
        }
    }
    if (perf) *perf = local;
    case_free(&k);
    return st;
}

/* nSteps rheoFoam steps of a multiMode model: models[nModes] (a common rho
 * and stabilization), s the common fields (U, p, phi; tau and taub get the
 * summed tau), modes[i] each mode's theta, tau and eigen fields; modePerf
 * (6 per mode, or NULL) each mode's theta solve records of the last step. */
int or_step_ddt(const rt_mesh_desc *m, const rt_bc_desc *bc, const rt_model_params *models, int nModes,
                const rt_case_ctl *ctl, or_state *s, or_state *modes, int nSteps, rt_step_perf *perf,
                rt_solver_perf *modePerf, or_ddt *ddt);

int or_step_modes(const rt_mesh_desc *m, const rt_bc_desc *bc, const rt_model_params *models, int nModes,
                  const rt_case_ctl *ctl, or_state *s, or_state *modes, int nSteps, rt_step_perf *perf,
                  rt_solver_perf *modePerf) {
    if (ctl->ddtScheme != RT_DDT_EULER) return RT_EINVAL;
    return or_step_ddt(m, bc, models, nModes, ctl, s, modes, nSteps, perf, modePerf, NULL);
}

/* nSteps steps of a single- (nModes 1, modes NULL) or multiMode case with the
 * ddt scheme of ctl; ddt: the Crank-Nicolson state (required for it). */
int or_step_ddt(const rt_mesh_desc *m, const rt_bc_desc *bc, const rt_model_params *models, int nModes,
                const rt_case_ctl *ctl, or_state *s, or_state *modes, int nSteps, rt_step_perf *perf,
                rt_solver_perf *modePerf, or_ddt *ddt) {
    if (nModes < 1 || (nModes > 1 && !modes)) return RT_EINVAL;
    if (ctl->ddtScheme == RT_DDT_CRANKNICOLSON && !ddt) return RT_EINVAL;
    for (int i = 1; i < nModes; ++i)
        if (models[i].rho != models[0].rho || models[i].stabilization != models[0].stabilization) return RT_EINVAL;
    rt_model_params eff = modes_momentum_model(models, nModes);
    or_case k;
    case_init(&k, m, bc, &eff, ctl, s);
    if (nModes > 1) { k.nModes = nModes; k.models = models; k.modes = modes; k.modePerf = modePerf; }
    if (ctl->ddtScheme == RT_DDT_CRANKNICOLSON) { ddt->scheme = RT_DDT_CRANKNICOLSON; ddt->psi = ctl->ddtPsi; k.ddt = ddt; }
    rt_step_perf local;
    int st = RT_OK;
    for (int i = 0; i < nSteps && st == RT_OK; ++i) {
        memset(&local, 0, sizeof local);
        st = step_once(&k, &local);
        if (st == RT_OK) {
            if (!isfinite(local.p.finalResidual)) st = RT_ENAN;
            for (int j = 0; j < 3; ++j) if (local.U[j].nIterations >= 0 && !isfinite(local.U[j].finalResidual)) st = RT_ENAN;
        }
    }
    if (perf) *perf = local;
    case_free(&k);
    return st;
}

/* correct() of a single- or multiMode model as a time step of its own
 * (newTimeStep != 0) or as a further inner iteration of the current one, with
 * the ddt scheme of ctl (ddt: the Crank-Nicolson state, required for it; the
 * old-time theta is then the one kept at the start of the time step). */
int or_constitutive_correct_ddt(const rt_mesh_desc *m, const rt_bc_desc *bc, const rt_model_params *models,
                                int nModes, const rt_case_ctl *ctl, or_state *s, or_state *modes,
                                const double *gradU, int newTimeStep, rt_solver_perf *modePerf, or_ddt *ddt) {
    if (nModes < 1 || (nModes > 1 && !modes) || !ddt || ctl->ddtScheme != RT_DDT_CRANKNICOLSON) return RT_EINVAL;
    or_case k;
    case_init(&k, m, bc, &models[0], ctl, s);
    if (nModes > 1) { k.nModes = nModes; k.models = models; k.modes = modes; k.modePerf = modePerf; }
    ddt->scheme = RT_DDT_CRANKNICOLSON;
    ddt->psi = ctl->ddtPsi;
    k.ddt = ddt;
    if (newTimeStep || ddt->nThSteps == 0) ddt_begin_step(&k, 0);
    k.ddtCth = ddt_coef(ddt, ddt->nThSteps - 1);
    k.Dth = ddt->Dth;
    int st;
    if (nModes > 1) {
        rt_solver_perf last[6];
        st = modes_correct(&k, gradU, last, ddt->ths);
    } else {
        st = constitutive_correct(&k, gradU, modePerf, ddt->ths);
    }
    case_free(&k);
    return st;
}

/* correct() of a multiMode model on the common fields of s (the modes'
 * fields in modes[]); s->tau gets the summed tau. */
int or_constitutive_correct_modes(const rt_mesh_desc *m, const rt_bc_desc *bc, const rt_model_params *models,
                                  int nModes, const rt_case_ctl *ctl, or_state *s, or_state *modes,
                                  const double *gradU, rt_solver_perf *modePerf) {
    if (nModes < 1) return RT_EINVAL;
    or_case k;
    case_init(&k, m, bc, &models[0], ctl, s);
    k.nModes = nModes; k.models = models; k.modes = modes; k.modePerf = modePerf;
    rt_solver_perf last[6];
    int st = modes_correct(&k, gradU, last, NULL);
    case_free(&k);
    return st;
}

/* correct() of a single- or multiMode model with temperature-dependent
 * parameters: each mode's shift functions (thermo[nModes]) at the cell
 * temperatures T, as the non-isothermal solvers call constEq.correct()
 * (rheoHeatFoam.C:144,189); modes as or_constitutive_correct_modes. */
int or_constitutive_correct_thermo(const rt_mesh_desc *m, const rt_bc_desc *bc, const rt_model_params *models,
                                   int nModes, const rt_case_ctl *ctl, or_state *s, or_state *modes,
                                   const double *gradU, const rt_thermo_desc *thermo, const double *T,
                                   rt_solver_perf *modePerf) {
    if (nModes < 1 || (nModes > 1 && !modes) || !thermo || !T) return RT_EINVAL;
    const int N = m->nCells;
    double *fac = DALLOC(3 * (size_t)N * nModes);
    for (int i = 0; i < nModes; ++i) or_thermo_factors(&thermo[i], N, T, fac + 3 * (size_t)N * i);
    or_case k;
    case_init(&k, m, bc, &models[0], ctl, s);
    k.thermo = fac;
    int st;
    if (nModes > 1) {
        k.nModes = nModes; k.models = models; k.modes = modes; k.modePerf = modePerf;
        rt_solver_perf last[6];
        st = modes_correct(&k, gradU, last, NULL);
    } else {
        st = constitutive_correct(&k, gradU, modePerf, NULL);
    }
    case_free(&k);
    free(fac);
    return st;
}

/* Initial phi = flux(U) (createPhi) and boundary values of U/p/theta/tau. */
void or_init_fields(const rt_mesh_desc *m, const rt_bc_desc *bc, or_state *s) {
    int nB = m->nBFaces;
    int *kU = (int *)xcalloc(nB, sizeof(int)), *kP = (int *)xcalloc(nB, sizeof(int));
    int *kT = (int *)xcalloc(nB, sizeof(int)), *kTa = (int *)xcalloc(nB, sizeof(int));
    bface_kinds(m, bc->U, kU); bface_kinds(m, bc->p, kP);
    bface_kinds(m, bc->theta, kT); bface_kinds(m, bc->tau, kTa);
    for (int b = 0; b < nB; ++b) {
        if (kU[b] == RT_BC_FIXED) for (int j = 0; j < 3; ++j) s->Ub[3 * b + j] = bc->Ub[3 * b + j];
        if (kP[b] == RT_BC_FIXED) s->pb[b] = bc->pb[b];
        if (kT[b] == RT_BC_FIXED) for (int q = 0; q < 6; ++q) s->thetab[6 * b + q] = bc->thetab[6 * b + q];
        if (kTa[b] != RT_BC_ZEROGRAD) for (int q = 0; q < 6; ++q) s->taub[6 * b + q] = bc->taub[6 * b + q];
    }
    correct_bc(m, kU, s->U, s->Ub, 3);
    correct_bc(m, kP, s->p, s->pb, 1);
    correct_bc(m, kT, s->theta, s->thetab, 6);
    correct_bc(m, kTa, s->tau, s->taub, 6);
    for (int f = 0; f < m->nFaces; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        double v = 0.0;
        for (int j = 0; j < 3; ++j)
            v += m->Sf[3 * f + j] * lin_interp(m->weights[f], s->U[3 * o + j], s->U[3 * n + j]);
        s->phi[f] = v;
    }
    for (int b = 0; b < nB; ++b)
        s->phib[b] = m->bSf[3 * b] * s->Ub[3 * b] + m->bSf[3 * b + 1] * s->Ub[3 * b + 1] +
                     m->bSf[3 * b + 2] * s->Ub[3 * b + 2];
    free(kU); free(kP); free(kT); free(kTa);
}

/* sizes of the ABI structs as the C compiler lays them out (ctypes check) */
void or_abi_sizes(int *out) {
    out[0] = (int)sizeof(rt_mesh_desc);
    out[1] = (int)sizeof(rt_bc_desc);
    out[2] = (int)sizeof(rt_model_params);
    out[3] = (int)sizeof(rt_solver_ctl);
    out[4] = (int)sizeof(rt_solver_perf);
    out[5] = (int)sizeof(rt_case_ctl);
    out[6] = (int)sizeof(rt_step_perf);
    out[7] = (int)sizeof(rt_thermo_desc);
}
