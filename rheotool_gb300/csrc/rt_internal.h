// rt_internal.h — device-side data structures shared by the librheogpu
// translation units.  All device fields are structure-of-arrays: a field with
// nc components over n entries is one allocation laid out component-major
// (component k of entry i at [k*n + i]), so every kernel reads and writes
// contiguous, coalesced runs of doubles.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <memory>
#include <string>
#include <utility>
#include <array>
#include <vector>

#include "../../include/rheogpu.h"

#define RT_BLOCK 256

namespace rt {

// ---------------------------------------------------------------------------
// error plumbing: every CUDA call goes through RT_CUDA, which records the
// failing call in the context and returns RT_ECUDA to the C caller.
// ---------------------------------------------------------------------------
struct Error {
    rt_status status;
    std::string msg;
};

#define RT_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            throw ::rt::Error{RT_ECUDA, std::string(#call) + ": " +                \
                                            cudaGetErrorString(e_)};               \
    } while (0)

#define RT_CHECK_LAUNCH() RT_CUDA(cudaGetLastError())

#define RT_REQUIRE(cond, code, what)                                               \
    do {                                                                           \
        if (!(cond)) throw ::rt::Error{(code), (what)};                            \
    } while (0)

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
// bytes of device memory held by every DBuf of the process (admission control)
inline std::atomic<long long> &device_bytes() {
    static std::atomic<long long> v{0};
    return v;
}

template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) {
            cudaFree(p);
            device_bytes() -= (long long)(n * sizeof(T));
        }
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error{RT_EOOM, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
        }
        n = count;
        device_bytes() += (long long)(count * sizeof(T));
    }
    void zero(cudaStream_t s) {
        if (p) RT_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
    void upload(const T *h, size_t count, cudaStream_t s) {
        alloc(count);
        if (count) RT_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    operator T *() const { return p; }
};

constexpr int SYNC_WORK = 0, SYNC_ERROR = 1, SYNC_PROGRESS = 2;

// raw view passed to the kernels; every array has nSkew entries in the
// skewed (block, step / 4, lane, step % 4) layout, wS has 6 components of nSkew
template <class Real>
struct SkewT {
    int nx, ny, nz, nJB, T;
    long long nSkew;
    const int *cellOf;
    Real *D, *Pz, *Py, *Px, *rDraw;   // rD recurrence inputs / output (FP64 only)
    Real *rDinv, *Az, *Ay, *Ax, *Bz, *By, *Bx;
    Real *wS;   // 6 components
    Real *rS;   // 6 components
    double *w64;   // backward sweep of the FP32 coefficients: FP64 output (cell order) instead of w, or null
    // the components still iterating, on the device (a Krylov loop that stops
    // on the device), or null: a launch whose components have all stopped
    // returns at once
    const unsigned *dmask;
};
using SkewView = SkewT<double>;
using SkewView32 = SkewT<float>;

// a captured multigrid V-cycle and the buffers it was captured with
struct MgGraph {
    cudaGraphExec_t exec = nullptr;
    const void *r = nullptr, *w = nullptr, *dm = nullptr;
    unsigned mask = 0;   // the components it smooths
    bool sym = false;    // the symmetric (pressure) view of the hierarchy
    int launches = 0;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        r = w = dm = nullptr;
        mask = 0;
        sym = false;
    }
    MgGraph() = default;
    MgGraph(const MgGraph &) = delete;
    MgGraph &operator=(const MgGraph &) = delete;
    ~MgGraph() { reset(); }
};
constexpr int kMgGraphs = 8;   // captured V-cycles kept per mesh

struct StructMesh {
    bool on = false;
    int nx = 0, ny = 0, nz = 0, nJB = 0, T = 0;
    int KC = 1;                // planes per CTA of the systolic sweeps
    long long nSkew = 0;
    DBuf<int> cellOf;          // nSkew: cell of each skewed entry, -1 outside the mesh
    DBuf<int> faceLo, faceHi;  // 3*N: face to the (z, y, x) lower / upper neighbour, -1 if none
    DBuf<int> sync;            // work counter, error flag
    DBuf<unsigned long long> xfer;   // tagged hand-off words between clusters
    unsigned epoch = 0;        // tag of the current launch's hand-off words
    int tune[2] = {-1, -1};    // schedule of the one-component sweeps (FP64, FP32), -1 until tuned
    float tuneMs[2] = {0, 0};  // its time per application
    DBuf<double> data;         // 12 + 6 + 6 arrays of nSkew doubles
    bool pendingCheck = false;
    // the box: the cell of each box position (-1 outside the mesh) and the
    // box position of each cell; the multigrid hierarchy's boxes and arrays
    DBuf<int> cellAt, boxOf;
    std::vector<std::array<int, 3>> mgDims;
    DBuf<float> mgData;
    MgGraph mgGraph[kMgGraphs];   // the captured V-cycles, replaced round robin
    int mgNext = 0;

    SkewView view() {
        SkewView v;
        v.nx = nx; v.ny = ny; v.nz = nz; v.nJB = nJB; v.T = T; v.nSkew = nSkew;
        v.cellOf = cellOf.p;
        double *p = data.p;
        double **slots[] = {&v.D, &v.Pz, &v.Py, &v.Px, &v.rDraw, &v.rDinv, &v.Az, &v.Ay, &v.Ax,
                            &v.Bz, &v.By, &v.Bx};
        for (int i = 0; i < 12; ++i) *slots[i] = p + (size_t)i * nSkew;
        v.wS = p + (size_t)12 * nSkew;
        v.rS = p + (size_t)18 * nSkew;
        v.w64 = nullptr;
        v.dmask = nullptr;
        return v;
    }

    // the premultiplied coefficients of the transposed factorisation (the
    // lower and upper coefficients exchanged, the same rD): PBiCG's M^-T,
    // allocated on first use
    DBuf<double> dataT;
    SkewView viewT() {
        if (dataT.n != (size_t)6 * nSkew) dataT.alloc((size_t)6 * nSkew);
        SkewView v = view();
        double **slots[] = {&v.Az, &v.Ay, &v.Ax, &v.Bz, &v.By, &v.Bx};
        for (int i = 0; i < 6; ++i) *slots[i] = dataT.p + (size_t)i * nSkew;
        return v;
    }

    // FP32 copies of the sweep coefficients and right-hand sides (mixed
    // precision): 7 coefficient arrays + 6 + 6 component arrays, allocated
    // on first use
    DBuf<float> data32;
    SkewView32 view32() {
        if (data32.n != (size_t)19 * nSkew) data32.alloc((size_t)19 * nSkew);
        SkewView32 v;
        v.nx = nx; v.ny = ny; v.nz = nz; v.nJB = nJB; v.T = T; v.nSkew = nSkew;
        v.cellOf = cellOf.p;
        v.D = v.Pz = v.Py = v.Px = v.rDraw = nullptr;
        float *p = data32.p;
        float **slots[] = {&v.rDinv, &v.Az, &v.Ay, &v.Ax, &v.Bz, &v.By, &v.Bx};
        for (int i = 0; i < 7; ++i) *slots[i] = p + (size_t)i * nSkew;
        v.wS = p + (size_t)7 * nSkew;
        v.rS = p + (size_t)13 * nSkew;
        v.w64 = nullptr;
        v.dmask = nullptr;
        return v;
    }
};


// ---------------------------------------------------------------------------
// batch of independent cases: the uploaded mesh is the disjoint union of the
// case meshes, case b owning a contiguous range of cells, internal faces and
// boundary faces.  One case (n = 1, caseOf = nullptr) is the plain context.
// ---------------------------------------------------------------------------
constexpr int kBatchMgLevels = 8;     // levels of a batched case's multigrid hierarchy, at most
constexpr int kBatchMgCoarse = 64;    // cells of its coarsest level, at most
constexpr int kBatchMgArrays = 11;   // arrays of a level: dg, xl, yl, xu, yu, x[3], b[3]

struct Batch {
    int n = 1;
    std::vector<int> cellStartH, faceStartH, bStartH;   // n + 1 each
    DBuf<int> caseOf;                 // N: case of each cell (batch only)
    DBuf<int> cellStartD, faceStartD, bStartD;          // n + 1 each, on the device
    DBuf<rt_model_params> params;     // n: model of each case
    DBuf<int> refCell;                // n: pRefCell (global) of each case, -1 without reference
    DBuf<double> refValue;            // n
    // reduction blocks aligned to cases: block k covers cells
    // [blkCell0[k], blkCell0[k] + 256) of case blkCase[k] (clipped)
    int nBlk = 0;
    std::vector<int> caseBlkH;        // n + 1: first block of each case
    DBuf<int> blkCase, blkCell0, blkCell1, caseBlk;
    // structured 2-D cases: skewed layout for the batched sweeps
    bool sweep2d = false;
    int maxJB = 0;
    long long nSkew = 0;
    std::vector<int> nxH, nyH;
    DBuf<int> sx, sy, sT, sJB;        // n: box and layout of each case
    DBuf<long long> sOff;             // n: first skewed entry of each case
    DBuf<int> sCell;                  // nSkew: global cell, -1 outside the case mesh
    DBuf<int> sFaceLo, sFaceHi;       // 2*N: face to the (y, x) lower / upper neighbour
    DBuf<double> sData64;             // D, Py, Px, rDraw, rDinv, Ay, Ax, By, Bx, wS(6), rS(6)
    DBuf<float> sData32;              // rDinv, Ay, Ax, By, Bx, wS(6), rS(6)
    DBuf<int> sErr;                   // bounded-wait error flag of the batched sweeps
    DBuf<int> caseOrder;              // n: cases by decreasing cell count (the CTA order of one-CTA-per-case launches)
    // structured 2-D cases: each case's multigrid hierarchy (the mixed
    // pressure and momentum solves of the persistent solvers, one at a time):
    // per case and level the box (nx, ny) and its arrays' offset in mgPool
    // (kBatchMgArrays of them, each padded to 4), the level count, and level
    // 0's cell of each box position
    DBuf<int> mgDims, mgNL, mgCell;
    DBuf<long long> mgOff, mgCellOff;
    DBuf<float> mgPool;
    bool sPending = false;
    // batched Krylov state: per-segment scalars (segment = case * 8 + component),
    // case-aligned reduction partials and results
    DBuf<double> segD, bPartial, bRes;
    DBuf<int> segI;
    int *hostCount = nullptr;         // pinned
    std::vector<double> hostSegD;
    std::vector<int> hostSegI;
};

// ---------------------------------------------------------------------------
// mesh: LDU addressing + geometry + cell-centric adjacency
// ---------------------------------------------------------------------------
struct DevMesh {
    StructMesh sm;               // structured (box-lexicographic) description, optional
    int N = 0, F = 0, NB = 0, nPatches = 0;
    int nSlots = 0;          // max internal faces per cell (ELL width)
    int solveDir[3] = {1, 1, 1};
    // faces (F)
    DBuf<int> owner, neighbour;
    DBuf<double> Sf;         // 3F SoA
    DBuf<double> magSf, w, deltaCoeffs;
    DBuf<double> d;          // 3F SoA, C_N - C_P (coupled faces: neighbour translated by the period)
    // coupled (cyclic) faces: internal faces that the DIC/DILU factorisation
    // and sweeps skip; coupledH[f] != 0 on the host
    bool hasCoupled = false;
    std::vector<char> coupledH;
    // ELL adjacency of the preconditioner (the faces that are not coupled);
    // empty when the mesh has no coupled faces (the full ELL serves then)
    DBuf<int> pellFace, pellNbr;
    int pnSlots = 0;
    // the preconditioner's adjacency split by direction: each cell's lower
    // neighbours (nb < c) in slots 0 .. pnLo - 1 and its upper ones in
    // 0 .. pnUp - 1, face order, padding -1 (the Jacobi-iterated DIC/DILU)
    DBuf<int> plNbr, plFace, puNbr, puFace;
    int pnLo = 0, pnUp = 0;
    // two-colour (red-black) ordering of a structured mesh: colour of each
    // cell (i + j + k) % 2, and its cells listed red first (N, set by
    // rt_mesh_set_ijk; empty otherwise)
    DBuf<unsigned char> colour;
    int nRed = 0;
    // cells (N)
    DBuf<double> C;          // 3N SoA
    DBuf<double> V;
    // boundary faces (NB)
    DBuf<int> bCell;
    DBuf<double> bSf;        // 3NB SoA
    DBuf<double> bmagSf, bDelta;
    DBuf<double> bCtoF;      // 3NB SoA, Cf - C_P
    DBuf<int> bPatch;
    // ELL adjacency: slot s of cell c at [s*N + c], sorted by face index,
    // padding -1 at the end
    DBuf<int> ellFace, ellNbr;
    // boundary faces of each cell, CSR over cells in boundary-face order
    DBuf<int> bStart, bList;
    // cells that own at least one boundary face
    DBuf<int> bCells;
    int nBCells = 0;
    // level schedule for the triangular sweeps: cells sorted by level,
    // level(c) = 1 + max(level of lower neighbours)
    int nLevels = 0;
    std::vector<int> levelStartH;
    DBuf<int> levelCells;
    // host copies needed by the host-side orchestration
    std::vector<int> patchStartH, patchSizeH;
    Batch batch;
};

// ---------------------------------------------------------------------------
// case + device fields
// ---------------------------------------------------------------------------
struct DevCase {
    bool ready = false;
    rt_model_params mp{};
    rt_case_ctl ctl{};
    std::vector<int> kindU, kindP, kindTheta, kindTau;   // per patch
    DBuf<int> bkU, bkP, bkTh, bkTau;                      // per boundary face
    // batches: the boundary faces whose tau values follow the field (zero
    // gradient, linear extrapolation) in waves, wave k holding the k-th such
    // patch of every case (empty for a single case)
    std::vector<int> tauWaveH;                            // nWaves + 1 starts
    DBuf<int> tauWaveFace;
    DBuf<double> UbFixed, pbFixed, thetabFixed, taubFixed;
    // state (SoA)
    DBuf<double> U, Ub, p, pb, phi, phib, theta, thetab, tau, taub, eigVals, eigVecs;
    // the theta of the start of the time step, kept by rt_constitutive_correct_iter
    DBuf<double> thetaOld;
    bool thetaOldSaved = false;
    // generalized PTT: Gamma(beta), Gamma(alpha k + beta) for k < mlK (else empty, mlK = 0)
    DBuf<double> mlGamma;
    int mlK = 0;
    // multiMode (nModes > 1): mode 0 lives in the fields above, modes 1 ..
    // nModes - 1 in `modes`; a mode's correct() swaps its state in (ModeSwap).
    // The momentum equation reads the summed tau (tauTot, taubTot) and the
    // summed-viscosity model mpMom; thetaStep0 keeps every mode's theta at
    // the start of a step with inner iterations.
    int nModes = 1;
    std::vector<std::unique_ptr<struct ModeState>> modes;
    DBuf<double> tauTot, taubTot, thetaStep0;
    rt_model_params mpMom{};
    std::vector<rt_solver_perf> modePerf;   // 6 per mode: the last correct()'s theta solves
    // Crank-Nicolson ddt (rt_case_ctl.ddtScheme): the old-time derivatives D
    // and the fields at the start of the last time step (xs), of the flow (U
    // with boundary values, phi) and of theta (each mode: Dth, ths here and
    // in ModeState); the time steps started so far and the coefficient c of
    // the current step (1 for the first, 1 + psi after)
    int ddtSteps = 0, ddtThSteps = 0;
    double ddtC = 1.0, ddtCth = 1.0;
    DBuf<double> DU, DUb, Dphi, Dphib, Us, Ubs, phis, phibs, Dth, ths;
    // temperature-dependent parameters (rt_set_temperature): thermoOn, the
    // cell temperatures, and this mode's shift factors (3 nCells: lambda, the
    // second relaxation time, etaP; the other modes' in ModeState)
    bool thermoOn = false;
    DBuf<double> Tcell, thermo;
};

// one further mode of a multiMode model: the DevCase's per-mode members
struct ModeState {
    rt_model_params mp{};
    DBuf<double> theta, thetab, tau, taub, eigVals, eigVecs, thetaOld, mlGamma, Dth, ths, thermo;
    bool thetaOldSaved = false;
    int mlK = 0;
};

template <class T>
void swap_buf(DBuf<T> &a, DBuf<T> &b) {
    std::swap(a.p, b.p);
    std::swap(a.n, b.n);
}

// exchanges a mode's state with the DevCase's own per-mode members for the
// guard's lifetime (constitutive_correct then works on that mode)
struct ModeSwap {
    DevCase &cs;
    ModeState *ms;
    static void swap_all(DevCase &c, ModeState &m) {
        std::swap(c.mp, m.mp);
        swap_buf(c.theta, m.theta);
        swap_buf(c.thetab, m.thetab);
        swap_buf(c.tau, m.tau);
        swap_buf(c.taub, m.taub);
        swap_buf(c.eigVals, m.eigVals);
        swap_buf(c.eigVecs, m.eigVecs);
        swap_buf(c.thetaOld, m.thetaOld);
        swap_buf(c.mlGamma, m.mlGamma);
        swap_buf(c.Dth, m.Dth);
        swap_buf(c.ths, m.ths);
        swap_buf(c.thermo, m.thermo);
        std::swap(c.thetaOldSaved, m.thetaOldSaved);
        std::swap(c.mlK, m.mlK);
    }
    ModeSwap(DevCase &c, ModeState *m) : cs(c), ms(m) {
        if (ms) swap_all(cs, *ms);
    }
    ~ModeSwap() {
        if (ms) swap_all(cs, *ms);
    }
};

// scratch arrays of the step, allocated once per mesh
struct Work {
    DBuf<double> a;   // generic pool, carved by the step code
    size_t used = 0;
    double *take(size_t n) {
        size_t al = (n + 31) & ~size_t(31);
        if (used + al > a.n) throw Error{RT_EOOM, "work pool exhausted"};
        double *p = a.p + used;
        used += al;
        return p;
    }
};

// gives back everything taken from the pool in its scope, on every exit path
struct WorkMark {
    Work &w;
    size_t mark;
    explicit WorkMark(Work &x) : w(x), mark(x.used) {}
    ~WorkMark() { w.used = mark; }
};

// reduction buffers
struct Reduce {
    int nBlocks = 0;
    DBuf<double> partial;   // [8 slots][6 comps][nBlocks]
    DBuf<double> result;    // [8 slots][6 comps]
    double *hostResult = nullptr;  // pinned
    // Krylov loops that stop on the device: the components still iterating
    // (one word), the arrival counter of the last-block reductions, and a
    // pinned, device-mapped flag the host polls (nonzero while iterating)
    DBuf<unsigned> active, counter;
    volatile int *hostFlag = nullptr;
    int *devFlag = nullptr;
    cudaEvent_t poll[2] = {nullptr, nullptr};
};

// CUDA-event profiler: named scopes on the context stream, aggregated at
// report time (launches, device milliseconds, algorithmic bytes)
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t next = 0;
    struct Rec {
        const char *name;
        size_t a, b;
        double bytes;
    };
    std::vector<Rec> recs;
};

}  // namespace rt

struct rt_ctx {
    int sweepMode = 0;           // 0 auto, 1 level-scheduled, 2 structured systolic
    int sweepTune = 0;           // 0 autotune the sweep schedule, k > 0: candidate k - 1
    int sweepRing = 0;           // deepest plane ring of the systolic sweeps (steps; 0: the default cap)
    int device = 0;
    int numSMs = 0;
    cudaStream_t stream = nullptr;
    std::string lastError;
    rt::DevMesh mesh;
    rt::DevCase cs;
    rt::Reduce red;
    rt::Work work;
    rt::DBuf<double> kws;        // Krylov workspace: 8 vectors x 6 comps x N + rD
    rt::DBuf<float> kws32;       // mixed-precision Krylov: FP32 vectors + FP32 matrix
    int precision = RT_PREC_FP64;   // of standalone rt_ldu_solve calls
    int mixedParts = 3;             // RT_PREC_MIXED: 1 FP32 Krylov, 2 FP32 constitutive
    double mixedTighten = 1e-2;     // RT_PREC_MIXED: solves stop at tolerance x this factor
    // RT_PREC_MIXED pressure solve: DIC applied by this many Jacobi sweeps per
    // triangular factor (0: the exact sweeps); FP32 premultiplied split-ELL
    // coefficients and three FP32 vectors
    int mixedJacobi = -2;   // RT_OPT_MIXED_PRECOND (default: the multigrid V-cycle)
    int mixedPrecondU = -2;   // RT_OPT_MIXED_PRECOND_U (default: the multigrid V-cycle)
    rt::DBuf<float> jac;
    // batched form: the pressure solve of structured 2-D cases as one
    // persistent CTA per case (RT_OPT_BATCH_PERSISTENT; 0: the per-iteration
    // launch sequence)
    int batchPersistent = 1;
    int sweepComponents = 1;   // RT_OPT_SWEEP_COMPONENTS
    std::vector<rt_step_perf> batchPerf;   // per case: the last step's solver records
    rt::DBuf<double> scal;       // device scalars of the Krylov loops [32 slots][8]
    rt::DBuf<double> stage;      // staging for AoS <-> SoA field transfers
    rt::Prof prof;
    cudaEvent_t tStart = nullptr, tStop = nullptr;
    bool meshReady = false;
    long long kernelLaunches = 0;
    // rt_residual_noalloc: device address of its static scratch array on this
    // context's device, resolved on the context's first call
    void *noallocScratch = nullptr;
    // bounded waits of the systolic sweeps: spins before a wait gives up
    // (RT_OPT_WAIT_LIMIT); stallTest > 0: the next sweep launch's
    // cluster-to-cluster consumers expect a tag no producer writes
    // (RT_OPT_STALL_TEST, failure-detection tests)
    long long waitLimit = 1ll << 24;
    int stallTest = 0;
};

namespace rt {

// kernels and host helpers implemented across the .cu files -----------------
// krylov.cu
struct SolveArgs {
    const double *diag, *upper, *lower;   // complete matrix (device)
    const double *source;                 // nc*N component-major (device)
    double *psi;                          // nc*N (device)
    int nc;
    unsigned validMask;                   // components to solve
    rt_solver_ctl ctl;
    int precision = RT_PREC_FP64;         // RT_PREC_MIXED: FP32 iterations, FP64 refinement
    int stage = -1;                       // batch records: 0 U, 1 p, 2 theta, -1 none
};
rt_status ldu_solve_device(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf);
double residual_device(rt_ctx *ctx, const double *diag, const double *upper,
                       const double *lower, const double *b, const double *x);
void reduce_init(rt_ctx *ctx);

// fv.cu
void grad_scalar(rt_ctx *ctx, const double *x, const double *xb, double *g);
void launch_count(rt_ctx *ctx, int n = 1);

// constitutive.cu
void eig_cells(rt_ctx *ctx, int n, const double *theta, double *eigVals, double *eigVecs);
// one mode's shift factors of the relaxation times and etaP (3 N: lambda,
// the second relaxation time, etaP) at the device cell temperatures T
void thermo_factors(rt_ctx *ctx, const rt_thermo_desc &d, const double *T, double *out);
// thetaOld: theta at the start of the time step (shared by its inner
// iterations); null = the current theta
rt_status constitutive_correct(rt_ctx *ctx, const double *gradU, rt_solver_perf *perf,
                               const double *thetaOld = nullptr);

// correct() of every mode of a multiMode model (or the one mode), then the
// summed tau; theta0s: the modes' old-time theta, mode after mode (or null)
rt_status modes_correct(rt_ctx *ctx, const double *gradU, rt_solver_perf *perf, const double *theta0s = nullptr);

// step.cu
rt_status step_once(rt_ctx *ctx, rt_step_perf *perf);
// start of a Crank-Nicolson time step: the old-time derivatives of the step
// that ended and the new start fields, of the flow (flow != 0) and of theta
void ddt_begin_step(rt_ctx *ctx, bool flow);
void init_fields(rt_ctx *ctx);

inline int nblocks(long long n, int b = RT_BLOCK) { return (int)((n + b - 1) / b); }

// prof.cu
int prof_begin(rt_ctx *ctx, const char *name);
void prof_end(rt_ctx *ctx, int rec, double bytes);
struct ProfScope {
    rt_ctx *ctx;
    int rec;
    double bytes;
    ProfScope(rt_ctx *c, const char *name, double b = 0.0) : ctx(c), rec(prof_begin(c, name)), bytes(b) {}
    ~ProfScope() { prof_end(ctx, rec, bytes); }
};

}  // namespace rt
