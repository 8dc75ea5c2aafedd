// rheogpu.hpp — C++ host side above the C ABI (include/rheogpu.h).
//
// It mirrors, for a C++ caller, the two interfaces of rheoTool / OpenFOAM
// that the library replaces, with their names, argument meanings and error
// behaviour:
//
//   LduSolver::New(fieldName, matrix, controls) / solve(psi, source, cmpt)
//       OpenFOAM's lduMatrix::solver::New and solve (selected by the
//       `solver` and `preconditioner` keywords of an fvSolution entry;
//       PCG/DIC, PBiCGStab/DILU, diagonal or no preconditioner), returning a
//       SolverPerformance (initial and final residual, iterations,
//       converged, singular).  Reached in rheoTool through
//       sparseSolver<Type>::solve (libs/sparseMatrixSolvers/segregated/
//       sparseSolver.H:200-205, openFoamSolver/openFoamSolver.C:46-53).
//   SparseSolver::New(fieldName, controls) / solve(matrix, psi, source, nCmpt)
//       rheoTool's sparseSolver<Type> selection by `solverType`.
//   ConstitutiveEq::New(name, constitutiveProperties) / correct() / tau()
//       rheoTool's constitutiveEq run-time selection (constitutiveEq.H:250-262,
//       newConstitutiveEq.C:32-61) for the log-conformation models the
//       library implements.
//
// OpenFOAM is not needed: Dictionary reads the subset of the dictionary
// format these entries use ("keyword value;" and nested sub-dictionaries),
// and fields are plain arrays in OpenFOAM's layouts.  Errors throw
// FatalError, as the reference aborts through FatalError (an unknown model
// type lists the valid ones, newConstitutiveEq.C:47-58; a missing keyword
// names it); a solve that hits maxIter is not an error (converged = false).
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/rheogpu.h"

namespace rheogpu {

struct FatalError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// "keyword value;" entries and "name { ... }" sub-dictionaries; comments
// (// and /* */) are skipped
class Dictionary {
public:
    Dictionary() = default;
    explicit Dictionary(std::string name) : name_(std::move(name)) {}
    static Dictionary parse(const std::string &text, const std::string &name = "dictionary");

    bool found(const std::string &key) const;
    bool isDict(const std::string &key) const;
    const std::string &lookup(const std::string &key) const;     // the raw value
    double lookupScalar(const std::string &key) const;
    double lookupOrDefault(const std::string &key, double def) const;
    int lookupOrDefault(const std::string &key, int def) const;
    std::string lookupOrDefault(const std::string &key, const std::string &def) const;
    const Dictionary &subDict(const std::string &key) const;
    void set(const std::string &key, const std::string &value) { entries_[key] = value; }
    const std::string &name() const { return name_; }

private:
    static void parseInto(const std::string &t, size_t &i, Dictionary &d);
    std::string name_;
    std::map<std::string, std::string> entries_;
    std::map<std::string, Dictionary> dicts_;
};

struct SolverPerformance {
    std::string solverName, fieldName;
    double initialResidual = 0.0, finalResidual = 0.0;
    int nIterations = 0;
    bool converged = false, singular = false;
};

// one device context (rt_ctx); owns nothing of the caller's
class Context {
public:
    explicit Context(int device = 0);
    ~Context();
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    rt_ctx *get() const { return ctx_; }
    void uploadMesh(const rt_mesh_desc &mesh);
    void setupCase(const rt_bc_desc &bcs, const rt_model_params &model, const rt_case_ctl &ctl);
    // throws FatalError(what + the library's message) unless s == RT_OK
    void check(rt_status s, const std::string &what) const;

private:
    rt_ctx *ctx_ = nullptr;
};

// the LDU coefficients of one matrix, in OpenFOAM's face order (not owned)
struct LduMatrixView {
    const double *diag = nullptr, *upper = nullptr, *lower = nullptr;
};

class LduSolver {
public:
    static std::unique_ptr<LduSolver> New(const std::string &fieldName, Context &ctx, const LduMatrixView &matrix,
                                          const Dictionary &controls);
    // one component: psi (nCells) is updated in place
    SolverPerformance solve(double *psi, const double *source, int cmpt = 0) const;
    // nCmpt components sharing the matrix (component-major blocks of nCells),
    // solved together as fvMatrix::solveSegregated solves a vector or tensor
    std::vector<SolverPerformance> solveComponents(double *psi, const double *source, int nCmpt) const;
    const std::string &type() const { return type_; }
    static const std::vector<std::string> &solvers();
    static const std::vector<std::string> &preconditioners();
    // the controls of an fvSolution solver entry (lduMatrix::solver::readControls
    // defaults: tolerance 1e-6, relTol 0, maxIter 1000, minIter 0)
    static rt_solver_ctl readControls(const Dictionary &controls);

private:
    LduSolver(std::string field, std::string type, Context &ctx, const LduMatrixView &m, const rt_solver_ctl &c)
        : field_(std::move(field)), type_(std::move(type)), ctx_(ctx), m_(m), ctl_(c) {}
    std::string field_, type_;
    Context &ctx_;
    LduMatrixView m_;
    rt_solver_ctl ctl_;
};

// rheoTool's sparseSolver<Type> (libs/sparseMatrixSolvers/segregated/
// sparseSolver.H:134-212): the per-field solver of rheoFoam's U and p,
// selected by `solverType` (sparseSolver.C:41).  The library serves the
// `openFoam` type (openFoamSolver.C:46-75: the lduMatrix solver of each
// component); the external types (eigenSolver, petscSolver, hypreSolver)
// throw FatalError listing the valid ones.
class SparseSolver {
public:
    static std::unique_ptr<SparseSolver> New(const std::string &fieldName, Context &ctx,
                                             const Dictionary &controls);
    static const std::vector<std::string> &types();
    // the solverType and lduMatrix controls of an entry (FatalError if not served)
    static rt_solver_ctl readControls(const Dictionary &controls);
    // every component of the field (component-major blocks of nCells), as
    // fvMatrix<Type>::solveSegregated does
    std::vector<SolverPerformance> solve(const LduMatrixView &matrix, double *psi, const double *source,
                                         int nCmpt) const;
    bool isExternalSolver() const { return false; }

private:
    SparseSolver(std::string f, Context &c, Dictionary d) : field_(std::move(f)), ctx_(c), controls_(std::move(d)) {}
    std::string field_;
    Context &ctx_;
    Dictionary controls_;
};

class ConstitutiveEq {
public:
    // `type` selects the model; the other keywords are the model's (rho,
    // etaS, etaP, lambda, alpha, epsilon, zeta, L2, lambdaR/lambdaD, beta,
    // delta, chiMax, lambdaS/lambdaB, q, n, m, K, L, a, b,
    // destructionFunctionType, stabilization)
    static std::unique_ptr<ConstitutiveEq> New(const std::string &name, const Dictionary &constitutiveProperties);
    static const std::vector<std::string> &types();

    const rt_model_params &params() const { return mp_; }
    double rho() const { return mp_.rho; }
    double etaS() const { return mp_.etaS; }
    double etaP() const { return mp_.etaP; }
    bool isGNF() const { return false; }
    const std::string &type() const { return type_; }

    // one constitutiveEq::correct() on the device-resident case of ctx
    // (set up with these params); gradU (9 nCells, AoS) may be null
    std::vector<SolverPerformance> correct(Context &ctx, const double *gradU = nullptr) const;
    // the same as one of rheoFoam's nInIter calls in a time step: newTimeStep
    // keeps the current theta as the step's old-time field, later calls of the
    // step solve against it (rt_constitutive_correct_iter)
    std::vector<SolverPerformance> correctIter(Context &ctx, bool newTimeStep, const double *gradU = nullptr) const;
    // tau (6 nCells AoS) and its boundary values (6 nBFaces, may be null)
    void tau(Context &ctx, double *internal, double *boundary = nullptr) const;
    // the model's thermoFunctions (thermoLambda / thermoLambdaD / thermoLambdaB,
    // thermoLambdaR / thermoLambdaS, thermoEta sub-dictionaries; Constant
    // where a sub-dictionary is absent)
    const rt_thermo_desc &thermo() const { return thermo_; }
    // the cell temperatures (nCells) the next correct() calls shift the
    // relaxation times and etaP by, as in a non-isothermal solver; null:
    // isothermal (rt_set_temperature, single-mode models)
    void setTemperature(Context &ctx, const double *T) const;

private:
    std::string name_, type_;
    rt_model_params mp_{};
    rt_thermo_desc thermo_{};
};

}  // namespace rheogpu
