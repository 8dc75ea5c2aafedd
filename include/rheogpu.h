/*
 * rheogpu.h — C ABI of the GB300 rheoFoam time-step library (librheogpu.so).
 *
 * One context owns one device mesh, one case (boundary conditions, model,
 * solver controls) and the device-resident fields of that case.  Host arrays
 * crossing this boundary are in OpenFOAM's own layout: cell fields are AoS
 * (vector x,y,z; symmTensor xx,xy,xz,yy,yz,zz; tensor xx..zz row-major),
 * surface fields are per internal face in upper-triangular face order, then
 * per boundary face patch by patch.  No pointer is retained past a call.
 *
 * Reference interfaces replaced (paths inside fppimenta/rheoTool, of90/src):
 *   rt_constitutive_correct  constitutiveEq::correct(alpha*, gradU*)
 *                            libs/constitutiveEquations/constitutiveEqs/
 *                            constitutiveEq/constitutiveEq.H:343-347, as done by
 *                            Oldroyd-B/Oldroyd-BLog/Oldroyd_BLog.C:127-179,
 *                            Giesekus/GiesekusLog/GiesekusLog.C:128-176,
 *                            PTT/PTTLog/PTTLog.C:176-268,
 *                            FENE-P/FENE-PLog/FENE_PLog.C:128-182,
 *                            FENE-CR/FENE-CRLog/FENE_CRLog.C:127-180,
 *                            Rolie-Poly/Rolie-PolyLog/RoliePolyLog.C:125-203,
 *                            XPomPom/XPomPomLog/XPomPomLog.C:133-198,
 *                            WhiteMetznerCY/WhiteMetznerCYLog/
 *                            WhiteMetznerCYLog.C:145-206
 *   rt_constitutive_correct_iter  the same, called nInIter times in one time
 *                            step (solvers/rheoFoam/rheoFoam.C:149-153)
 *   rt_set_temperature       the thermoFunction shifts of lambda and etaP that
 *                            the Log models' correct() applies in a
 *                            non-isothermal solver (libs/thermo/thermoFunctions/
 *                            thermoFunctions/thermoFunction.H, the types'
 *                            createField) with T in the mesh, as
 *                            solvers/rheoHeatFoam/rheoHeatFoam.C:144,189 call
 *                            constEq.correct()
 *   rt_ldu_solve             lduMatrix::solver::solve(psi, source, cmpt) of
 *                            OpenFOAM's PCG/DIC, PBiCGStab/DILU and PBiCG/DILU, reached
 *                            through sparseSolver<Type>::solve
 *                            (libs/sparseMatrixSolvers/segregated/sparseSolver.H:
 *                            200-205, openFoamSolver/openFoamSolver.C:46-53)
 *   rt_step                  one segregated time step of rheoFoam
 *                            (solvers/rheoFoam/rheoFoam.C:147-154: UEqn.H,
 *                            pEqn.H, constEq.correct())
 *   rt_residual              sparseSolver<Type>::getFoamResiduals
 *                            (libs/sparseMatrixSolvers/segregated/sparseSolver.C:
 *                            129-180)
 *   rt_mesh_upload           the fvMesh / lduAddressing a solver is built on
 *   rt_field_set / _get      GeometricField construction / write
 *
 * Errors are integer status codes; no C++ exception crosses this boundary.
 */
#ifndef RHEOGPU_H
#define RHEOGPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------- */
#define RT_OK        0
#define RT_EINVAL    1   /* bad argument, size or state                        */
#define RT_ENOCONV   2   /* a Krylov solve hit maxIter without converging      */
#define RT_ENAN      3   /* a NaN/Inf appeared in a residual or field          */
#define RT_ETIMEOUT  4   /* a bounded device-side wait ran out                 */
#define RT_EOOM      5   /* device allocation failed / admission refused       */
#define RT_ECUDA     6   /* a CUDA runtime call failed                          */
#define RT_ENOTREADY 7   /* mesh / case not uploaded yet                        */
typedef int32_t rt_status;

typedef struct rt_ctx rt_ctx;

/* ---- mesh --------------------------------------------------------------- */
typedef struct {
    int32_t nCells, nFaces, nBFaces, nPatches;
    const int32_t *owner, *neighbour;          /* nFaces, owner < neighbour   */
    const double *Sf;                           /* 3*nFaces face area vectors  */
    const double *magSf;                        /* nFaces                      */
    const double *Cf;                           /* 3*nFaces face centres       */
    const double *weights;                      /* nFaces owner weights        */
    const double *deltaCoeffs;                  /* nFaces 1/|C_N - C_P|        */
    const double *C;                            /* 3*nCells cell centres       */
    const double *V;                            /* nCells volumes              */
    const int32_t *bCell;                       /* nBFaces face cells          */
    const double *bSf, *bmagSf, *bCf;           /* 3*nB, nB, 3*nB              */
    const double *bDeltaCoeffs;                 /* nB 1/|Cf - C_P|             */
    const int32_t *patchStart, *patchSize;      /* nPatches                    */
    int32_t solveDir[3];                        /* 0 for an empty direction    */
    /* Cyclic (periodic) patch pairs.  OpenFOAM keeps a cyclic face pair as
     * boundary faces whose implicit coefficients act through an lduInterface
     * (cyclicFvPatch, cyclicLduInterface): they enter A x and the residual,
     * but not the DIC/DILU factorisation or sweeps.  Here each pair is one
     * internal face (owner < neighbour, in upper-triangular order like the
     * others) with coupled[f] = 1: every operator treats it as the internal
     * face across the periodic boundary, and the preconditioners skip it,
     * which is the interface treatment.  delta[3f..3f+2] is C_N - C_P across
     * each face, with the neighbour translated by the period for coupled
     * faces; NULL means C[N] - C[P].  coupled == NULL: no coupled faces.     */
    const double *delta;                        /* 3*nFaces or NULL            */
    const int32_t *coupled;                     /* nFaces flags or NULL        */
} rt_mesh_desc;

/* ---- boundary conditions (one kind per patch and field) ---------------- */
#define RT_BC_FIXED     0   /* fixedValue                                      */
#define RT_BC_ZEROGRAD  1   /* zeroGradient                                    */
#define RT_BC_LINEXTRAP 2   /* linearExtrapolation (rheoTool, tau only)        */

typedef struct {
    const int32_t *U, *p, *theta, *tau;   /* nPatches kinds each                */
    const double *Ub;                     /* 3*nBFaces values of fixed U faces  */
    const double *pb;                     /* nBFaces                            */
    const double *thetab;                 /* 6*nBFaces                          */
    const double *taub;                   /* 6*nBFaces                          */
} rt_bc_desc;

/* ---- constitutive model ----------------------------------------------- */
#define RT_MODEL_OLDROYDB_LOG 0   /* type Oldroyd-BLog                          */
#define RT_MODEL_GIESEKUS_LOG 1   /* type GiesekusLog                           */
#define RT_MODEL_PTT_LOG      2   /* type PTTLog                                */
#define RT_MODEL_FENEP_LOG    3   /* type FENE-PLog                             */
#define RT_MODEL_FENECR_LOG   4   /* type FENE-CRLog (FENE-CR/FENE-CRLog/FENE_CRLog.C:127-180) */
#define RT_MODEL_ROLIEPOLY_LOG 5  /* type Rolie-PolyLog (Rolie-Poly/Rolie-PolyLog/RoliePolyLog.C:125-203);
                                     lambda carries lambdaD */
#define RT_MODEL_XPOMPOM_LOG  6   /* type XPomPomLog (XPomPom/XPomPomLog/XPomPomLog.C:133-198);
                                     lambda carries lambdaB, alpha the anisotropy */
#define RT_MODEL_WHITEMETZNERCY_LOG 7 /* type WhiteMetznerCYLog (WhiteMetznerCY/WhiteMetznerCYLog/
                                     WhiteMetznerCYLog.C:145-206); the log form needs m = n,
                                     L = K and b = a, so n, K and a serve both the
                                     viscosity and the relaxation time */
#define RT_PTT_LINEAR 0
#define RT_PTT_EXP    1
#define RT_PTT_GENERALIZED 2   /* Gamma(beta) E_{alpha,beta}(z), the Mittag-Leffler function
                                  summed as in PTTLog.C:201-236 (alpha, beta > 0) */
#define RT_STAB_NONE     0
#define RT_STAB_BSD      1
#define RT_STAB_COUPLING 2

typedef struct {
    int32_t model, pttFunction, stabilization, pad_;
    double rho, etaS, etaP, lambda;
    double alpha;     /* Giesekus mobility; XPomPom anisotropy; PTT generalized: Mittag-Leffler alpha */
    double epsilon;   /* PTT extensibility                                    */
    double zeta;      /* PTT slip                                             */
    double L2;        /* FENE-P / FENE-CR squared extensibility               */
    double lambdaR;   /* Rolie-Poly stretch relaxation time (lambda = lambdaD) */
    double beta;      /* Rolie-Poly convective constraint release coefficient;
                         PTT generalized: Mittag-Leffler beta                  */
    double delta;     /* Rolie-Poly CCR exponent                              */
    double chiMax;    /* Rolie-Poly maximum stretch (finite extensibility when > 1) */
    double lambdaS;   /* XPomPom stretch relaxation time (lambda = lambdaB)   */
    double q;         /* XPomPom number of arms                               */
    double n;         /* XPomPom stretch exponent; WhiteMetznerCY power index */
    double K;         /* WhiteMetznerCY time constant (K = L)                 */
    double a;         /* WhiteMetznerCY Carreau-Yasuda exponent (a = b)       */
    double rTolMittagLeffler;       /* PTT generalized: series tolerance (1e-12)  */
    int32_t maxIterMittagLeffler;   /* PTT generalized: series terms at most (200) */
    int32_t pad2_;
} rt_model_params;

/* ---- linear solvers ----------------------------------------------------- */
#define RT_SOLVER_PCG       0
#define RT_SOLVER_PBICGSTAB 1
#define RT_SOLVER_PBICG     2   /* OpenFOAM PBiCG (the Contraction41 tutorials' U and theta
                                   solver, of90/tutorials/rheoFoam/Contraction41/Oldroyd-BLog/
                                   system/fvSolution:32,47); FP64 in both precision forms;
                                   not in the batched form */
#define RT_PRECOND_NONE     0
#define RT_PRECOND_DIC      1
#define RT_PRECOND_DILU     2
#define RT_PRECOND_DIAGONAL 3

typedef struct {
    int32_t solver, preconditioner;
    double tolerance, relTol;
    int32_t minIter, maxIter;
} rt_solver_ctl;

typedef struct {
    double initialResidual, finalResidual;
    int32_t nIterations, converged, singular, pad_;
} rt_solver_perf;

/* ---- case control ---------------------------------------------------- */
#define RT_LIM_NONE     -1
#define RT_LIM_UPWIND    0
#define RT_LIM_CUBISTA   1
#define RT_LIM_MINMOD    2
#define RT_LIM_SMART     3
#define RT_LIM_WACEB     4
#define RT_LIM_SUPERBEE  5

#define RT_PREC_FP64  0   /* plain form: FP64 throughout                       */
#define RT_PREC_MIXED 1   /* FP32 Krylov + FP64 refinement, FP32 constitutive  */

typedef struct {
    double deltaT;
    int32_t divU, divTheta;          /* RT_LIM_* for div(phi,U), div(phi,theta) */
    int32_t pRefCell, needReference; /* needReference: p has no fixed patch    */
    double pRefValue;
    rt_solver_ctl solverU, solverP, solverTheta;
    int32_t precision;
    int32_t nInIter;                 /* inner iterations of a step (UEqn, pEqn,
                                        constEq.correct() on the step's old-time
                                        fields; rheoFoam.C:96-150); 0 or 1: one */
    /* uniform body force per unit mass in the momentum equation (the source
     * an fvOptions meanVelocityForce / pressure-gradient source adds to UEqn
     * to drive a periodic channel); zero for the other cases                */
    double bodyForce[3];
    /* SIMPLE nNonOrthogonalCorrectors (pEqn.H:31-50): the pressure equation
     * is solved 1 + nNonOrthCorr times, each from the last solution, and the
     * flux is updated after the last solve.  The library's laplacian is the
     * orthogonal one ("Gauss linear orthogonal", the tutorials' choice), whose
     * explicit non-orthogonal correction is zero. */
    int32_t nNonOrthCorr;
    /* ddtSchemes default: RT_DDT_EULER, or RT_DDT_CRANKNICOLSON with the
     * off-centering coefficient ddtPsi ("CrankNicolson 1" is ddtPsi = 1;
     * 0 is Euler) for every ddt of the step: fvm::ddt(U), fvm::ddt(theta)
     * and the ddtCorr of the face flux */
    int32_t ddtScheme;
    double ddtPsi;
} rt_case_ctl;

#define RT_DDT_EULER          0
#define RT_DDT_CRANKNICOLSON  1

typedef struct {
    rt_solver_perf U[3], p, theta[6];
    double contErrSumLocal, contErrGlobal;
} rt_step_perf;

/* ---- field identifiers for rt_field_set / rt_field_get --------------- */
#define RT_FIELD_U       0   /* 3 comps, internal + boundary                   */
#define RT_FIELD_P       1   /* 1                                              */
#define RT_FIELD_PHI     2   /* surface: nFaces internal + nBFaces boundary     */
#define RT_FIELD_THETA   3   /* 6                                              */
#define RT_FIELD_TAU     4   /* 6                                              */
#define RT_FIELD_EIGVALS 5   /* 3: diagonal of eigVals (= exp of eigenvalues)  */
#define RT_FIELD_EIGVECS 6   /* 9: eigenvectors as columns, row-major tensor   */

/* ---- entry points ------------------------------------------------------- */
rt_status rt_ctx_create(rt_ctx **ctx, int32_t device);
rt_status rt_ctx_destroy(rt_ctx *ctx);
const char *rt_last_error(const rt_ctx *ctx);
const char *rt_status_string(rt_status s);

rt_status rt_mesh_upload(rt_ctx *ctx, const rt_mesh_desc *mesh);

/* Optional structure of the uploaded mesh (no reference counterpart: blockMesh
 * numbers the cells of a block this way but OpenFOAM does not record it).
 * cellIJK (3*nCells) gives each cell's position in an nx x ny x nz box; cells
 * must be numbered lexicographically (i fastest) and every internal face must
 * join box neighbours, else RT_EINVAL and the mesh stays unstructured.  A
 * structured mesh gets the systolic DIC/DILU sweeps. */
rt_status rt_mesh_set_ijk(rt_ctx *ctx, int32_t nx, int32_t ny, int32_t nz, const int32_t *cellIJK);

/* Options.  RT_OPT_SWEEP: 0 auto (systolic when structured), 1 level-scheduled
 * sweeps, 2 structured systolic sweeps.  RT_OPT_SWEEP_PLANES: planes per
 * thread-block cluster of the systolic sweeps, one CTA per plane (1 .. 16;
 * default 16, or 8 where a cluster of 16 cannot be scheduled).
 * RT_OPT_PRECISION: RT_PREC_FP64 or RT_PREC_MIXED for rt_ldu_solve (the time
 * step takes its precision from rt_case_ctl). */
#define RT_OPT_SWEEP 1
#define RT_OPT_SWEEP_PLANES 2
#define RT_OPT_PRECISION 3
/* RT_OPT_MIXED_PARTS: which parts of the mixed-precision form run in FP32
 * (bit 1 the Krylov iterations, bit 2 the constitutive algebra; default 3),
 * for accuracy studies of each part. */
#define RT_OPT_MIXED_PARTS 4
/* RT_OPT_MIXED_TIGHTEN: the mixed-precision solves stop when the FP64
 * residual is below tolerance x 10^-value (default 2): a solve that only just
 * meets the tolerance can differ from the FP64 iterate by far more than the
 * FP64 solve differs from the exact solution, so the mixed form iterates a
 * little further to keep its fields within 1e-6 of the FP64 form. */
#define RT_OPT_MIXED_TIGHTEN 5
/* RT_OPT_SWEEP_TUNE: schedule of the one-component systolic sweeps (chunk of
 * P steps, NB chunks staged ahead): 0 (default) times the candidates on the
 * first application per structured mesh and precision and keeps the fastest;
 * 1 .. 5 forces one (P, NB) of (8,3) (8,5) (16,3) (16,4) (4,6). */
#define RT_OPT_SWEEP_TUNE 6
/* RT_OPT_SWEEP_RING: deepest plane-to-plane ring of the systolic sweeps, in
 * steps (a power of two, 8 .. 128; 0 = default 128).  Each launch takes the
 * deepest ring up to this cap that fits the shared memory. */
#define RT_OPT_SWEEP_RING 7
/* RT_OPT_WAIT_LIMIT: spins a bounded device-side wait of the systolic sweeps
 * makes before it gives up (sets the sweep's error flag; the call returns
 * RT_ETIMEOUT and the context stays usable).  Default 2^24 (about a second
 * for a wait between thread-block clusters, which polls 16x less often);
 * 64 .. 2^40. */
#define RT_OPT_WAIT_LIMIT 8
/* RT_OPT_STALL_TEST: failure-detection tests only.  value > 0: in the next
 * `value` systolic sweep launches, the first plane of every thread-block
 * cluster after the first waits for a hand-off word that no plane writes, so
 * its bounded wait runs out and the call returns RT_ETIMEOUT (meshes with
 * more planes than one cluster holds; see RT_OPT_SWEEP_PLANES).  0 (default)
 * clears it. */
#define RT_OPT_STALL_TEST 9
/* RT_OPT_MIXED_PRECOND: the preconditioner of the mixed form's pressure
 * solve (DIC selected).  -2 (default): on structured meshes without coupled
 * faces, an aggregation multigrid V-cycle (FP32, red-black Gauss-Seidel
 * smoothing, Galerkin coarse operators of 2 x 2 x 2 aggregates; elsewhere
 * the exact DIC).  0: DIC with the exact triangular sweeps (FP32 systolic
 * sweeps on structured meshes).  -1: DIC of the two-colour (red-black)
 * ordering of a structured mesh, applied in two parallel, bandwidth-bound
 * passes.  k = 1 .. 64: DIC applied by k Jacobi sweeps per triangular factor
 * (a truncated Neumann series of the same factorisation; Anzt, Chow and
 * Dongarra 2015).  Every choice stops on the same FP64 residual test.  The
 * FP64 plain form always uses the exact sweeps. */
#define RT_OPT_MIXED_PRECOND 10
/* RT_OPT_BATCH_PERSISTENT: the batched form's pressure and momentum solves
 * on structured 2-D cases (up to 256 rows) as one persistent CTA per case,
 * each running all the iterations of its case in one launch, or as a
 * per-iteration launch sequence replayed for all cases.  0: the launch
 * sequence; 1 (default): persistent when the batch holds at least half as
 * many cases as the GPU has SMs (a CTA per case leaves a small batch's SMs
 * idle); 2: persistent whatever the batch.  Both take the same scalar
 * decisions; the persistent form sums each case's reductions in one pass of
 * its CTA, so the iterates agree to round-off, not bit for bit. */
#define RT_OPT_BATCH_PERSISTENT 11
/* RT_OPT_SWEEP_COMPONENTS: the systolic sweeps of a solve of two or three
 * components (the momentum solve).  1 (default): the components side by
 * side, one one-component sweep each in a single launch (each thread-block
 * cluster takes a plane group of one component); 0: one sweep carrying all
 * the components lane by lane.  Both give the same bits. */
#define RT_OPT_SWEEP_COMPONENTS 12
/* RT_OPT_MIXED_PRECOND_U: the preconditioner of the mixed form's momentum
 * solve (DILU selected, up to three components).  -2 (default): on
 * structured meshes without coupled faces (and in the batched form's
 * persistent solver on structured 2-D cases), the aggregation multigrid
 * V-cycle of RT_OPT_MIXED_PRECOND -2 built from the non-symmetric momentum
 * matrix, its components in one cycle; elsewhere the exact DILU.  0: DILU
 * with the exact triangular sweeps.  Both stop on the same FP64 residual
 * test; the FP64 plain form always uses the exact sweeps. */
#define RT_OPT_MIXED_PRECOND_U 13
rt_status rt_set_option(rt_ctx *ctx, int32_t option, int64_t value);
rt_status rt_case_setup(rt_ctx *ctx, const rt_bc_desc *bcs,
                        const rt_model_params *model, const rt_case_ctl *ctl);
/* internal: ncmpt*nCells AoS (may be NULL); boundary: ncmpt*nBFaces AoS (may
 * be NULL).  For RT_FIELD_PHI internal is nFaces long. */
rt_status rt_field_set(rt_ctx *ctx, int32_t field, const double *internal,
                       const double *boundary);
rt_status rt_field_get(rt_ctx *ctx, int32_t field, double *internal,
                       double *boundary);

/* Solve ncmpt systems that share one LDU matrix on the uploaded mesh's
 * addressing.  diag/source/psi are complete (boundary coefficients already
 * added, as lduMatrix::solver receives them).  source and psi hold ncmpt
 * blocks of nCells (component-major).  perf gets ncmpt entries. */
rt_status rt_ldu_solve(rt_ctx *ctx, const double *diag, const double *upper,
                       const double *lower, const double *source, double *psi,
                       int32_t ncmpt, const rt_solver_ctl *ctl,
                       rt_solver_perf *perf);

/* OpenFOAM-normalised residual of one component (sparseSolver.C:129-180). */
rt_status rt_residual(rt_ctx *ctx, const double *diag, const double *upper,
                      const double *lower, const double *source,
                      const double *psi, double *residual);

/* rt_residual for callers that cannot allocate device memory (a solver
 * callback inside another library's Krylov loop, where a cudaMalloc would
 * synchronise the device in the middle of that loop; a host whose device
 * memory all belongs to its own pool allocator).  No reference counterpart:
 * an addition of this library.  diag, upper, lower, source and psi are
 * DEVICE pointers (device or managed memory) on the context's device
 * (nCells / nFaces doubles); anything else is refused with RT_EINVAL before
 * any kernel runs.  residual is a host pointer.  The kernels run on the
 * context's stream, which is not ordered after the caller's streams: the
 * caller finishes the work that writes the inputs first (synchronises its
 * stream, or has that work complete before the call by other means).  The
 * reduction scratch is a static device array inside the library, so the call
 * allocates nothing; it limits meshes to 2,097,152 cells (RT_EINVAL beyond).
 * The first call on each context resolves that array's address on the
 * context's device, so make it before any stream capture.  All calls share
 * the one array: calls that overlap on the GPU race and must be serialised by
 * the caller. */
rt_status rt_residual_noalloc(rt_ctx *ctx, const double *diag, const double *upper,
                              const double *lower, const double *source,
                              const double *psi, double *residual);

/* ---- multiMode models (multiMode.C:69-91, 144-156, 222, 247-256) -------
 * A multiMode constitutive model is a list of modes, each a constitutive
 * model of its own with its own theta, tau and eigen fields on the common U
 * and phi.  rt_case_setup_modes sets up such a case: models[nModes] (every
 * mode with the same rho and stabilization, so that the momentum equation's
 * sum of the modes' divTau is one divTau with the summed tau and the summed
 * etaS and etaP); all modes take the theta and tau conditions of bcs.
 * rt_step and rt_constitutive_correct then correct every mode in turn
 * (rt_step_perf.theta holds the last mode's solves, rt_mode_perf every
 * mode's: 6 records per mode).  rt_field_get(RT_FIELD_TAU) gives the summed
 * tau (multiMode::tau()); RT_FIELD_THETA, EIGVALS and EIGVECS without a mode
 * are mode 0's; rt_field_set_mode / rt_field_get_mode address one mode's
 * theta, tau, eigVals or eigVecs (the summed tau is formed at the next
 * correct()).  nModes = 1 is rt_case_setup.  Not in the batched form;
 * rt_constitutive_correct_iter runs single-mode models. */
#define RT_MAX_MODES 16
rt_status rt_case_setup_modes(rt_ctx *ctx, const rt_bc_desc *bcs, const rt_model_params *models,
                              int32_t nModes, const rt_case_ctl *ctl);
rt_status rt_field_set_mode(rt_ctx *ctx, int32_t field, int32_t mode, const double *internal,
                            const double *boundary);
rt_status rt_field_get_mode(rt_ctx *ctx, int32_t field, int32_t mode, double *internal,
                            double *boundary);
rt_status rt_mode_perf(rt_ctx *ctx, rt_solver_perf *thetaPerf);

/* One constitutiveEq::correct() on the device-resident U, phi, theta, eig
 * fields; gradU (9*nCells AoS) may be NULL (then fvc::grad(U) is used).
 * thetaPerf gets 6 entries (components not solved have nIterations = -1). */
rt_status rt_constitutive_correct(rt_ctx *ctx, const double *gradU,
                                  rt_solver_perf *thetaPerf);

/* constitutiveEq::correct() as rheoFoam's inner iterations call it
 * (rheoFoam.C:149-153 with nInIter > 1): newTimeStep != 0 first keeps the
 * current theta as the time step's old-time field, OpenFOAM's
 * theta.oldTime() after the time increment; every call then solves fvm::ddt
 * against that field, so nInIter calls in one step iterate the update rather
 * than advance nInIter steps.  rt_constitutive_correct is the call with
 * newTimeStep = 1.  A call with newTimeStep = 0 returns RT_ENOTREADY unless
 * a call with 1 came after the last rt_case_setup, rt_step,
 * rt_constitutive_correct or rt_field_set of theta (each of those starts
 * another time step, or replaces theta). */
rt_status rt_constitutive_correct_iter(rt_ctx *ctx, const double *gradU, int32_t newTimeStep,
                                       rt_solver_perf *thetaPerf);

/* ---- temperature-dependent parameters (thermoFunctions) ---------------
 * The non-isothermal solvers (rheoHeatFoam) call the same
 * constitutiveEq::correct() with a temperature field T in the mesh.  Each
 * Log model then takes its relaxation times and polymeric viscosity as
 * fields, the constant times a shift factor of T:
 *   volScalarField lambda(thermoLambdaPtr_->createField(lambda_));
 *   volScalarField etaP(thermoEtaPtr_->createField(etaP_));
 * (Oldroyd-B/Oldroyd-BLog/Oldroyd_BLog.C:133-135; the other Log models
 * likewise).  Rolie-Poly shifts lambdaD and lambdaR by their own functions
 * (thermoLambdaD, thermoLambdaR: RoliePolyLog.C:139-141), XPomPom lambdaB
 * and lambdaS (thermoLambdaB, thermoLambdaS: XPomPomLog.C:140-142).  The
 * shift factors, thermoFunctions/<type>/<type>.C (a model dictionary without
 * the sub-dictionary selects Constant, newThermoFunction.C:41): */
#define RT_THERMO_CONSTANT           0   /* a = 1                                  (Constant.C:58-73) */
#define RT_THERMO_ARRHENIUS          1   /* a = exp(alpha (1/T - 1/T0))            (Arrhenius.C:61-76) */
#define RT_THERMO_ARRHENIUS_MODIFIED 2   /* a = exp(-alpha (T - T0))               (ArrheniusModified.C:61-76) */
#define RT_THERMO_WLF                3   /* a = 10^(-c1 (T - T0) / (c2 + T - T0))  (WLF.C:61-76) */
#define RT_THERMO_VFT                4   /* a = 10^(B + A / (T - T0))              (VFT.C:62-77) */

typedef struct {
    int32_t type, pad_;
    double alpha, T0;   /* Arrhenius, ArrheniusModified (T0 also WLF and VFT) */
    double c1, c2;      /* WLF                                                */
    double A, B;        /* VFT                                                */
} rt_thermo_fn;

typedef struct {
    rt_thermo_fn lambda;    /* thermoLambda (Rolie-Poly: thermoLambdaD; XPomPom: thermoLambdaB) */
    rt_thermo_fn lambda2;   /* Rolie-Poly thermoLambdaR; XPomPom thermoLambdaS; unused otherwise  */
    rt_thermo_fn eta;       /* thermoEta (etaP)                                                   */
} rt_thermo_desc;

/* Set the cell temperatures T (nCells, host) and each mode's shift
 * functions (modes: the case's nModes descriptors, in mode order); the
 * factors are computed on the device at once and every later
 * rt_constitutive_correct / rt_constitutive_correct_iter applies them.  T =
 * NULL returns to the isothermal case, as does another rt_case_setup.
 * RT_EINVAL: a temperature outside a function's domain (Arrhenius T <= 0 or
 * T0 <= 0, WLF c2 + T - T0 = 0, VFT T = T0), a non-finite T, an unknown type,
 * or a batched layout.  The momentum equation's temperature-dependent
 * viscosities (etaSThermo, etaPThermo in constitutiveEq.C:200-245) and the
 * energy equation are not built, so rt_step returns RT_EINVAL while a
 * temperature is set. */
rt_status rt_set_temperature(rt_ctx *ctx, const rt_thermo_desc *modes, const double *T);

/* nSteps segregated rheoFoam time steps; perf (may be NULL) gets the last. */
rt_status rt_step(rt_ctx *ctx, int32_t nSteps, rt_step_perf *perf);

/* Gauss-linear gradient of one scalar field with boundary values
 * (fvc::grad): psi nCells, psib nBFaces, grad 3*nCells AoS. */
rt_status rt_op_grad(rt_ctx *ctx, const double *psi, const double *psib,
                     double *grad);

/* Per-cell symmetric 3x3 eigendecomposition of theta (6*n AoS): eigVals gets
 * exp(eigenvalues) ascending (3*n), eigVecs the eigenvectors as columns (9*n)
 * (constitutiveEq::calcEig, constitutiveEq.C:360-428). */
rt_status rt_op_eig(rt_ctx *ctx, int32_t n, const double *theta,
                    double *eigVals, double *eigVecs);

/* ---- batches of independent cases -------------------------------------
 * No reference counterpart (rheoFoam runs one case per process): the batched
 * form steps many independent cases of uneven size as one device mesh, the
 * disjoint union of the case meshes, uploaded with rt_mesh_upload.
 *
 * rt_batch_layout: case c owns cells [cellStart[c], cellStart[c+1]), internal
 * faces [faceStart[c], faceStart[c+1]) and boundary faces
 * [bFaceStart[c], bFaceStart[c+1]) (nCases + 1 entries each; no face may join
 * two cases).  dims (3*nCases: nx, ny, nz) and cellIJK (3*nCells, positions
 * inside each case's box) are optional; when every case is a lexicographic
 * 2-D box (nz = 1, ny <= 1024) the DIC/DILU sweeps run one CTA per case.
 * rt_batch_case_setup: as rt_case_setup, with one model per case and each
 * case's pressure reference (pRefCell: a cell of that case, or -1 when the
 * case has a fixed-value pressure patch).  rt_step then steps every case;
 * rt_batch_step_perf returns each case's solver records of the last step.
 * Every Krylov solve of a batch is per case: each case has its own scalars
 * and its own stopping point, as if it were solved alone. */
rt_status rt_batch_layout(rt_ctx *ctx, int32_t nCases, const int32_t *cellStart,
                          const int32_t *faceStart, const int32_t *bFaceStart,
                          const int32_t *dims, const int32_t *cellIJK);
rt_status rt_batch_case_setup(rt_ctx *ctx, const rt_bc_desc *bcs,
                              const rt_model_params *models, const rt_case_ctl *ctl,
                              const int32_t *pRefCell, const double *pRefValue);
rt_status rt_batch_step_perf(rt_ctx *ctx, rt_step_perf *perf);

/* The sweep schedules in use: schedule[0..2] = candidate, P, NB of the FP64
 * one-component sweeps, schedule[3..5] of the FP32 ones (-1, 0, 0 before the
 * first application).  No reference counterpart. */
rt_status rt_sweep_schedule(rt_ctx *ctx, int32_t *schedule);

/* Device memory held by all contexts of this library in the process (bytes):
 * what an admission controller adds a new case's footprint to.  No reference
 * counterpart. */
rt_status rt_device_bytes(int64_t *bytes);

/* Wait for all work of the context. */
rt_status rt_sync(rt_ctx *ctx);

/* Timing on the context stream (no reference counterpart: instrumentation,
 * like the per-step ExecutionTime print of rheoFoam.C:166-168).
 * rt_timer_start/stop bracket a region with CUDA events; rt_profile_enable
 * turns on named per-operation event pairs, rt_profile_report writes one
 * line "name launches device_ms algorithmic_bytes" per operation and clears
 * them; rt_kernel_count returns the number of kernels launched so far. */
rt_status rt_timer_start(rt_ctx *ctx);
rt_status rt_timer_stop(rt_ctx *ctx, double *ms);
rt_status rt_profile_enable(rt_ctx *ctx, int32_t on);
rt_status rt_profile_report(rt_ctx *ctx, char *buf, int32_t len);
rt_status rt_kernel_count(rt_ctx *ctx, int64_t *n);

#ifdef __cplusplus
}
#endif
#endif /* RHEOGPU_H */
