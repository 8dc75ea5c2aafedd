// rheogpu_host.cpp — the C++ host mirror of rheoTool/OpenFOAM's solver and
// constitutive-model selection above the C ABI (see rheogpu.hpp).
#include "rheogpu.hpp"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <sstream>

namespace rheogpu {

// ---------------------------------------------------------------------------
// Dictionary
// ---------------------------------------------------------------------------
namespace {

std::string strip_comments(const std::string &t) {
    std::string out;
    out.reserve(t.size());
    for (size_t i = 0; i < t.size();) {
        if (t.compare(i, 2, "//") == 0) {
            while (i < t.size() && t[i] != '\n') ++i;
        } else if (t.compare(i, 2, "/*") == 0) {
            size_t e = t.find("*/", i + 2);
            i = (e == std::string::npos) ? t.size() : e + 2;
            out.push_back(' ');
        } else {
            out.push_back(t[i++]);
        }
    }
    return out;
}

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

}  // namespace

Dictionary Dictionary::parse(const std::string &text, const std::string &name) {
    Dictionary d(name);
    const std::string t = strip_comments(text);
    size_t i = 0;
    parseInto(t, i, d);
    return d;
}

// the entries of one dictionary level, from t[i] to its closing '}' (or the end)
void Dictionary::parseInto(const std::string &t, size_t &i, Dictionary &d) {
    while (i < t.size()) {
        while (i < t.size() && std::isspace((unsigned char)t[i])) ++i;
        if (i >= t.size()) return;
        if (t[i] == '}') {
            ++i;
            return;
        }
        std::string key;
        if (t[i] == '"') {
            size_t e = t.find('"', i + 1);
            if (e == std::string::npos) throw FatalError("dictionary " + d.name_ + ": unterminated quoted keyword");
            key = t.substr(i + 1, e - i - 1);
            i = e + 1;
        } else {
            size_t s = i;
            while (i < t.size() && !std::isspace((unsigned char)t[i]) && t[i] != '{' && t[i] != ';') ++i;
            key = t.substr(s, i - s);
        }
        while (i < t.size() && std::isspace((unsigned char)t[i])) ++i;
        if (i < t.size() && t[i] == '{') {
            ++i;
            Dictionary sub(d.name_ + "." + key);
            parseInto(t, i, sub);
            d.dicts_[key] = sub;
            continue;
        }
        // the value runs to the ';' outside parentheses
        size_t s = i;
        int depth = 0;
        while (i < t.size() && !(t[i] == ';' && depth == 0)) {
            if (t[i] == '(') ++depth;
            if (t[i] == ')') --depth;
            ++i;
        }
        d.entries_[key] = trim(t.substr(s, i - s));
        if (i < t.size()) ++i;
    }
}

bool Dictionary::found(const std::string &key) const { return entries_.count(key) || dicts_.count(key); }
bool Dictionary::isDict(const std::string &key) const { return dicts_.count(key) > 0; }

const std::string &Dictionary::lookup(const std::string &key) const {
    auto it = entries_.find(key);
    if (it == entries_.end()) throw FatalError("keyword " + key + " is undefined in dictionary " + name_);
    return it->second;
}

double Dictionary::lookupScalar(const std::string &key) const {
    const std::string &v = lookup(key);
    char *end = nullptr;
    double x = std::strtod(v.c_str(), &end);
    if (end == v.c_str()) throw FatalError("keyword " + key + " in dictionary " + name_ + ": expected a number, got " + v);
    return x;
}

double Dictionary::lookupOrDefault(const std::string &key, double def) const {
    return entries_.count(key) ? lookupScalar(key) : def;
}
int Dictionary::lookupOrDefault(const std::string &key, int def) const {
    return entries_.count(key) ? (int)lookupScalar(key) : def;
}
std::string Dictionary::lookupOrDefault(const std::string &key, const std::string &def) const {
    auto it = entries_.find(key);
    return it == entries_.end() ? def : it->second;
}

const Dictionary &Dictionary::subDict(const std::string &key) const {
    auto it = dicts_.find(key);
    if (it == dicts_.end()) throw FatalError("sub-dictionary " + key + " is undefined in dictionary " + name_);
    return it->second;
}

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
Context::Context(int device) {
    rt_status s = rt_ctx_create(&ctx_, device);
    if (s != RT_OK) {
        ctx_ = nullptr;
        throw FatalError(std::string("rt_ctx_create(device ") + std::to_string(device) + "): " + rt_status_string(s));
    }
}

Context::~Context() {
    if (ctx_) rt_ctx_destroy(ctx_);
}

void Context::check(rt_status s, const std::string &what) const {
    if (s == RT_OK) return;
    std::string msg = what + ": " + rt_status_string(s);
    const char *e = ctx_ ? rt_last_error(ctx_) : nullptr;
    if (e && *e) msg += std::string(" (") + e + ")";
    throw FatalError(msg);
}

void Context::uploadMesh(const rt_mesh_desc &mesh) { check(rt_mesh_upload(ctx_, &mesh), "rt_mesh_upload"); }

void Context::setupCase(const rt_bc_desc &bcs, const rt_model_params &model, const rt_case_ctl &ctl) {
    check(rt_case_setup(ctx_, &bcs, &model, &ctl), "rt_case_setup");
}

// ---------------------------------------------------------------------------
// LduSolver (lduMatrix::solver)
// ---------------------------------------------------------------------------
const std::vector<std::string> &LduSolver::solvers() {
    static const std::vector<std::string> v{"PBiCG", "PBiCGStab", "PCG"};
    return v;
}
const std::vector<std::string> &LduSolver::preconditioners() {
    static const std::vector<std::string> v{"DIC", "DILU", "diagonal", "none"};
    return v;
}

namespace {
std::string valid_list(const std::string &what, const std::string &got, const std::vector<std::string> &v) {
    std::ostringstream os;
    os << "Unknown " << what << " " << got << "\n\nValid " << what << "s are :\n" << v.size() << "\n(\n";
    for (auto &s : v) os << s << "\n";
    os << ")\n";
    return os.str();
}
}  // namespace

std::unique_ptr<LduSolver> LduSolver::New(const std::string &fieldName, Context &ctx, const LduMatrixView &m,
                                          const Dictionary &c) {
    const rt_solver_ctl ctl = readControls(c);
    if (!m.diag || !m.upper || !m.lower) throw FatalError("LduSolver::New(" + fieldName + "): null matrix coefficients");
    return std::unique_ptr<LduSolver>(new LduSolver(fieldName, c.lookup("solver"), ctx, m, ctl));
}

rt_solver_ctl LduSolver::readControls(const Dictionary &c) {
    const std::string solver = c.lookup("solver");
    rt_solver_ctl ctl{};
    if (solver == "PCG") ctl.solver = RT_SOLVER_PCG;
    else if (solver == "PBiCGStab") ctl.solver = RT_SOLVER_PBICGSTAB;
    else if (solver == "PBiCG") ctl.solver = RT_SOLVER_PBICG;
    else throw FatalError(valid_list("lduMatrix::solver", solver, solvers()));
    // "preconditioner DIC;" or "preconditioner { preconditioner DIC; }"
    std::string pre = c.isDict("preconditioner") ? c.subDict("preconditioner").lookup("preconditioner")
                                                 : c.lookupOrDefault("preconditioner", std::string("none"));
    if (pre == "DIC") ctl.preconditioner = RT_PRECOND_DIC;
    else if (pre == "DILU") ctl.preconditioner = RT_PRECOND_DILU;
    else if (pre == "diagonal") ctl.preconditioner = RT_PRECOND_DIAGONAL;
    else if (pre == "none") ctl.preconditioner = RT_PRECOND_NONE;
    else throw FatalError(valid_list("lduMatrix::preconditioner", pre, preconditioners()));
    // lduMatrix::solver::readControls defaults
    ctl.tolerance = c.lookupOrDefault("tolerance", 1e-6);
    ctl.relTol = c.lookupOrDefault("relTol", 0.0);
    ctl.maxIter = c.lookupOrDefault("maxIter", 1000);
    ctl.minIter = c.lookupOrDefault("minIter", 0);
    return ctl;
}

std::vector<SolverPerformance> LduSolver::solveComponents(double *psi, const double *source, int nCmpt) const {
    std::vector<rt_solver_perf> perf((size_t)nCmpt);
    rt_status s = rt_ldu_solve(ctx_.get(), m_.diag, m_.upper, m_.lower, source, psi, nCmpt, &ctl_, perf.data());
    if (s != RT_ENOCONV) ctx_.check(s, "rt_ldu_solve(" + field_ + ")");
    std::vector<SolverPerformance> out((size_t)nCmpt);
    for (int k = 0; k < nCmpt; ++k) {
        SolverPerformance &p = out[(size_t)k];
        p.solverName = type_;
        p.fieldName = nCmpt > 1 ? field_ + std::to_string(k) : field_;
        p.initialResidual = perf[(size_t)k].initialResidual;
        p.finalResidual = perf[(size_t)k].finalResidual;
        p.nIterations = perf[(size_t)k].nIterations;
        p.converged = perf[(size_t)k].converged != 0;
        p.singular = perf[(size_t)k].singular != 0;
    }
    return out;
}

SolverPerformance LduSolver::solve(double *psi, const double *source, int cmpt) const {
    SolverPerformance p = solveComponents(psi, source, 1)[0];
    (void)cmpt;   // the component index only names the output, as in OpenFOAM
    return p;
}

// ---------------------------------------------------------------------------
// SparseSolver (rheoTool sparseSolver<Type>)
// ---------------------------------------------------------------------------
const std::vector<std::string> &SparseSolver::types() {
    static const std::vector<std::string> v{"openFoam"};
    return v;
}

rt_solver_ctl SparseSolver::readControls(const Dictionary &c) {
    const std::string t = c.lookupOrDefault("solverType", std::string("openFoam"));
    if (t != "openFoam") throw FatalError(valid_list("sparseSolver solverType", t, types()));
    return LduSolver::readControls(c);
}

std::unique_ptr<SparseSolver> SparseSolver::New(const std::string &fieldName, Context &ctx, const Dictionary &c) {
    readControls(c);
    return std::unique_ptr<SparseSolver>(new SparseSolver(fieldName, ctx, c));
}

std::vector<SolverPerformance> SparseSolver::solve(const LduMatrixView &m, double *psi, const double *source,
                                                   int nCmpt) const {
    return LduSolver::New(field_, ctx_, m, controls_)->solveComponents(psi, source, nCmpt);
}

// ---------------------------------------------------------------------------
// ConstitutiveEq (constitutiveEq run-time selection)
// ---------------------------------------------------------------------------
const std::vector<std::string> &ConstitutiveEq::types() {
    static const std::vector<std::string> v{"FENE-CRLog", "FENE-PLog",         "GiesekusLog",      "Oldroyd-BLog",
                                            "PTTLog",     "Rolie-PolyLog",     "WhiteMetznerCYLog", "XPomPomLog"};
    return v;
}

// thermoFunction::New (thermoFunctions/newThermoFunction.C:33-61): the
// sub-dictionary `name` of the model's dictionary selects the type; without
// it the function is Constant
static rt_thermo_fn thermo_function(const Dictionary &d, const std::string &name) {
    rt_thermo_fn f{};
    f.type = RT_THERMO_CONSTANT;
    if (!d.isDict(name)) return f;
    const Dictionary &t = d.subDict(name);
    const std::string type = t.lookup("type");
    if (type == "Constant") return f;
    if (type == "Arrhenius" || type == "ArrheniusModified") {
        f.type = type == "Arrhenius" ? RT_THERMO_ARRHENIUS : RT_THERMO_ARRHENIUS_MODIFIED;
        f.alpha = t.lookupScalar("alpha");
        f.T0 = t.lookupScalar("T0");
    } else if (type == "WLF") {
        f.type = RT_THERMO_WLF;
        f.c1 = t.lookupScalar("c1");
        f.c2 = t.lookupScalar("c2");
        f.T0 = t.lookupScalar("T0");
    } else if (type == "VFT") {
        f.type = RT_THERMO_VFT;
        f.A = t.lookupScalar("A");
        f.B = t.lookupScalar("B");
        f.T0 = t.lookupScalar("T0");
    } else {
        throw FatalError(valid_list("thermoFunction type", type,
                                    {"Arrhenius", "ArrheniusModified", "Constant", "VFT", "WLF"}));
    }
    return f;
}

std::unique_ptr<ConstitutiveEq> ConstitutiveEq::New(const std::string &name, const Dictionary &d) {
    const std::string type = d.lookup("type");
    std::unique_ptr<ConstitutiveEq> ce(new ConstitutiveEq());
    ce->name_ = name;
    ce->type_ = type;
    rt_model_params &mp = ce->mp_;
    if (type == "Oldroyd-BLog") mp.model = RT_MODEL_OLDROYDB_LOG;
    else if (type == "GiesekusLog") mp.model = RT_MODEL_GIESEKUS_LOG;
    else if (type == "PTTLog") mp.model = RT_MODEL_PTT_LOG;
    else if (type == "FENE-PLog") mp.model = RT_MODEL_FENEP_LOG;
    else if (type == "FENE-CRLog") mp.model = RT_MODEL_FENECR_LOG;
    else if (type == "Rolie-PolyLog") mp.model = RT_MODEL_ROLIEPOLY_LOG;
    else if (type == "XPomPomLog") mp.model = RT_MODEL_XPOMPOM_LOG;
    else if (type == "WhiteMetznerCYLog") mp.model = RT_MODEL_WHITEMETZNERCY_LOG;
    else throw FatalError(valid_list("constitutiveEq type", type, types()));
    mp.rho = d.lookupScalar("rho");
    mp.etaS = d.lookupScalar("etaS");
    mp.etaP = d.lookupScalar("etaP");
    if (mp.model == RT_MODEL_ROLIEPOLY_LOG) {
        mp.lambda = d.lookupScalar("lambdaD");
        mp.lambdaR = d.lookupScalar("lambdaR");
        mp.beta = d.lookupScalar("beta");
        mp.delta = d.lookupScalar("delta");
        mp.chiMax = d.lookupScalar("chiMax");
    } else if (mp.model == RT_MODEL_XPOMPOM_LOG) {
        // XPomPomLog.C:114-122
        mp.lambda = d.lookupScalar("lambdaB");
        mp.lambdaS = d.lookupScalar("lambdaS");
        mp.q = d.lookupScalar("q");
        mp.n = d.lookupScalar("n");
    } else {
        mp.lambda = d.lookupScalar("lambda");
    }
    if (mp.model == RT_MODEL_WHITEMETZNERCY_LOG) {
        // WhiteMetznerCYLog.C:118-141: the log form needs m = n, K = L, a = b
        mp.n = d.lookupScalar("n");
        mp.K = d.lookupScalar("K");
        mp.a = d.lookupScalar("a");
        if (d.lookupScalar("m") != mp.n || d.lookupScalar("L") != mp.K || d.lookupScalar("b") != mp.a)
            throw FatalError("The Log version of the WhiteMetznerCY model can only be used if:\n\n   m=n   and   K=L"
                             "   and   a=b\n\n Check if this is the case, otherwise use the stress version "
                             "(WhiteMetznerCY).");
    }
    if (mp.model == RT_MODEL_GIESEKUS_LOG || mp.model == RT_MODEL_XPOMPOM_LOG) mp.alpha = d.lookupScalar("alpha");
    if (mp.model == RT_MODEL_PTT_LOG) {
        mp.epsilon = d.lookupScalar("epsilon");
        mp.zeta = d.lookupScalar("zeta");
        mp.rTolMittagLeffler = d.lookupOrDefault("rTolMittagLeffler", 1e-12);
        mp.maxIterMittagLeffler = d.lookupOrDefault("maxIterMittagLeffler", 200);
        const std::string f = d.lookup("destructionFunctionType");
        if (f == "linear") mp.pttFunction = RT_PTT_LINEAR;
        else if (f == "exponential") mp.pttFunction = RT_PTT_EXP;
        else if (f == "generalized") mp.pttFunction = RT_PTT_GENERALIZED;
        else throw FatalError(valid_list("destructionFunctionType", f, {"exponential", "generalized", "linear"}));
        if (mp.pttFunction == RT_PTT_GENERALIZED) {
            // PTTLog.C:143-152
            mp.alpha = d.lookupScalar("alpha");
            mp.beta = d.lookupScalar("beta");
            if (mp.alpha <= 0 || mp.beta <= 0)
                throw FatalError("Both alpha and beta should be positive values for the Mittag-Leffler function "
                                 "to converge.");
        }
    }
    if (mp.model == RT_MODEL_FENEP_LOG || mp.model == RT_MODEL_FENECR_LOG) mp.L2 = d.lookupScalar("L2");
    // the thermoFunctions of the relaxation times and etaP, by the names each
    // Log model gives them (Oldroyd_BLog.C:118-119, RoliePolyLog.C:122-124,
    // XPomPomLog.C:123-125)
    if (mp.model == RT_MODEL_ROLIEPOLY_LOG) {
        ce->thermo_.lambda = thermo_function(d, "thermoLambdaD");
        ce->thermo_.lambda2 = thermo_function(d, "thermoLambdaR");
    } else if (mp.model == RT_MODEL_XPOMPOM_LOG) {
        ce->thermo_.lambda = thermo_function(d, "thermoLambdaB");
        ce->thermo_.lambda2 = thermo_function(d, "thermoLambdaS");
    } else {
        ce->thermo_.lambda = thermo_function(d, "thermoLambda");
    }
    ce->thermo_.eta = thermo_function(d, "thermoEta");
    // constitutiveEq::checkForStab
    const std::string stab = d.lookup("stabilization");
    if (stab == "none") mp.stabilization = RT_STAB_NONE;
    else if (stab == "BSD") mp.stabilization = RT_STAB_BSD;
    else if (stab == "coupling") mp.stabilization = RT_STAB_COUPLING;
    else throw FatalError(valid_list("stabilization", stab, {"none", "BSD", "coupling"}));
    return ce;
}

namespace {
std::vector<SolverPerformance> theta_performance(const rt_solver_perf perf[6]) {
    static const char *cmpt[6] = {"xx", "xy", "xz", "yy", "yz", "zz"};
    std::vector<SolverPerformance> out;
    for (int k = 0; k < 6; ++k) {
        if (perf[k].nIterations < 0) continue;   // component not solved (2-D)
        SolverPerformance p;
        p.solverName = "PBiCGStab";
        p.fieldName = std::string("theta.") + cmpt[k];
        p.initialResidual = perf[k].initialResidual;
        p.finalResidual = perf[k].finalResidual;
        p.nIterations = perf[k].nIterations;
        p.converged = perf[k].converged != 0;
        p.singular = perf[k].singular != 0;
        out.push_back(p);
    }
    return out;
}
}  // namespace

void ConstitutiveEq::setTemperature(Context &ctx, const double *T) const {
    ctx.check(rt_set_temperature(ctx.get(), T ? &thermo_ : nullptr, T), "thermoFunction (" + type_ + ")");
}

std::vector<SolverPerformance> ConstitutiveEq::correct(Context &ctx, const double *gradU) const {
    rt_solver_perf perf[6];
    ctx.check(rt_constitutive_correct(ctx.get(), gradU, perf), "constitutiveEq::correct (" + type_ + ")");
    return theta_performance(perf);
}

std::vector<SolverPerformance> ConstitutiveEq::correctIter(Context &ctx, bool newTimeStep, const double *gradU) const {
    rt_solver_perf perf[6];
    ctx.check(rt_constitutive_correct_iter(ctx.get(), gradU, newTimeStep ? 1 : 0, perf),
              "constitutiveEq::correct (" + type_ + ")");
    return theta_performance(perf);
}

void ConstitutiveEq::tau(Context &ctx, double *internal, double *boundary) const {
    ctx.check(rt_field_get(ctx.get(), RT_FIELD_TAU, internal, boundary), "tau");
}

}  // namespace rheogpu
