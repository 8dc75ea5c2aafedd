// test_host.cpp — checks of the C++ host mirror (rheotool_gb300/host).
//   --cpu : dictionary parsing, run-time selection and its errors, and the
//           error raised when no GPU can be opened (no compute call)
//   --gpu : LduSolver::New + solve on a chain of cells (PCG-DIC and
//           PBiCGStab-DILU) against a direct tridiagonal solve
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../rheotool_gb300/host/rheogpu.hpp"

using namespace rheogpu;

static int failures = 0;
#define CHECK(c)                                                              \
    do {                                                                      \
        if (!(c)) {                                                           \
            std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                                       \
        }                                                                     \
    } while (0)

template <class F>
static std::string throws(F f) {
    try {
        f();
    } catch (const FatalError &e) {
        return e.what();
    }
    return "";
}

static void cpu_checks() {
    const char *props =
        "/* constitutiveProperties */\n"
        "parameters\n{\n    type            GiesekusLog;\n    rho             rho [1 -3 0 0 0 0 0] 0.01;\n"
        "    etaS 0.111; etaP 0.889;  // comment\n    lambda 0.5;\n    alpha 0.1;\n"
        "    stabilization   coupling;\n    nested { a 1; b (0 0 1); }\n}\n";
    Dictionary d = Dictionary::parse(props, "constitutiveProperties");
    const Dictionary &p = d.subDict("parameters");
    CHECK(p.lookup("type") == "GiesekusLog");
    CHECK(p.subDict("nested").lookup("b") == "(0 0 1)");
    CHECK(std::fabs(p.lookupScalar("alpha") - 0.1) < 1e-15);
    CHECK(p.lookupOrDefault("missing", 7.0) == 7.0);
    CHECK(throws([&] { p.lookup("missing"); }).find("keyword missing is undefined") != std::string::npos);

    // rho carries OpenFOAM's dimensioned form in the reference dictionaries:
    // the plain-number form is what the mirror reads
    Dictionary q = Dictionary::parse("type GiesekusLog; rho 0.01; etaS 0.111; etaP 0.889; lambda 0.5; alpha 0.1;"
                                     " stabilization coupling;", "parameters");
    auto ce = ConstitutiveEq::New("ce", q);
    CHECK(ce->type() == "GiesekusLog" && ce->params().model == RT_MODEL_GIESEKUS_LOG);
    CHECK(ce->params().stabilization == RT_STAB_COUPLING && std::fabs(ce->etaP() - 0.889) < 1e-15);
    CHECK(!ce->isGNF());

    Dictionary rp = Dictionary::parse("type Rolie-PolyLog; rho 1; etaS 0.1; etaP 0.9; lambdaD 1.0; lambdaR 0.2;"
                                      " beta 0.5; delta -0.5; chiMax 5; stabilization none;");
    auto r = ConstitutiveEq::New("rp", rp);
    CHECK(r->params().model == RT_MODEL_ROLIEPOLY_LOG && r->params().lambda == 1.0 && r->params().lambdaR == 0.2);

    Dictionary bad = Dictionary::parse("type BoguerLog; rho 1; etaS 1; etaP 1; lambda 1; stabilization none;");
    std::string m = throws([&] { ConstitutiveEq::New("x", bad); });
    CHECK(m.find("Unknown constitutiveEq type BoguerLog") != std::string::npos);
    CHECK(m.find("Oldroyd-BLog") != std::string::npos && m.find("FENE-PLog") != std::string::npos);

    Dictionary ptt = Dictionary::parse("type PTTLog; rho 1; etaS 1; etaP 1; lambda 1; epsilon 0.25; zeta 0;"
                                       " destructionFunctionType exponential; stabilization BSD;");
    auto pt = ConstitutiveEq::New("p", ptt);
    CHECK(pt->params().pttFunction == RT_PTT_EXP && pt->params().stabilization == RT_STAB_BSD);
    Dictionary pttg = Dictionary::parse("type PTTLog; rho 1; etaS 1; etaP 1; lambda 1; epsilon 0.25; zeta 0;"
                                        " alpha 0.8; beta 1.2; destructionFunctionType generalized; stabilization BSD;");
    auto pg = ConstitutiveEq::New("p", pttg);
    CHECK(pg->params().pttFunction == RT_PTT_GENERALIZED && pg->params().alpha == 0.8 && pg->params().beta == 1.2);
    CHECK(pg->params().maxIterMittagLeffler == 200 && pg->params().rTolMittagLeffler == 1e-12);
    Dictionary pttb = Dictionary::parse("type PTTLog; rho 1; etaS 1; etaP 1; lambda 1; epsilon 0.25; zeta 0;"
                                        " alpha 0.8; beta 0; destructionFunctionType generalized; stabilization BSD;");
    CHECK(throws([&] { ConstitutiveEq::New("p", pttb); }).find("should be positive") != std::string::npos);
    Dictionary pttu = Dictionary::parse("type PTTLog; rho 1; etaS 1; etaP 1; lambda 1; epsilon 0.25; zeta 0;"
                                        " destructionFunctionType quadratic; stabilization BSD;");
    CHECK(throws([&] { ConstitutiveEq::New("p", pttu); }).find("Unknown destructionFunctionType quadratic") !=
          std::string::npos);

    Dictionary xpp = Dictionary::parse("type XPomPomLog; rho 1; etaS 0.1; etaP 0.9; lambdaB 1.0; lambdaS 0.25;"
                                       " alpha 0.15; q 2; n 0; stabilization coupling;");
    auto x = ConstitutiveEq::New("xpp", xpp);
    CHECK(x->params().model == RT_MODEL_XPOMPOM_LOG && x->params().lambda == 1.0 && x->params().lambdaS == 0.25);
    CHECK(x->params().alpha == 0.15 && x->params().q == 2.0 && x->params().n == 0.0);
    Dictionary wm = Dictionary::parse("type WhiteMetznerCYLog; rho 1; etaS 0.1; etaP 0.9; lambda 1; m 0.5; n 0.5;"
                                      " K 1; L 1; a 2; b 2; stabilization coupling;");
    auto w = ConstitutiveEq::New("wm", wm);
    CHECK(w->params().model == RT_MODEL_WHITEMETZNERCY_LOG && w->params().n == 0.5 && w->params().K == 1.0 &&
          w->params().a == 2.0);
    Dictionary wmbad = Dictionary::parse("type WhiteMetznerCYLog; rho 1; etaS 0.1; etaP 0.9; lambda 1; m 0.5;"
                                         " n 0.4; K 1; L 1; a 2; b 2; stabilization coupling;");
    CHECK(throws([&] { ConstitutiveEq::New("wm", wmbad); }).find("m=n") != std::string::npos);

    // thermoFunctions: the sub-dictionaries by each model's names, Constant where absent
    Dictionary th = Dictionary::parse("type GiesekusLog; rho 1; etaS 0.1; etaP 0.9; lambda 1; alpha 0.1;"
                                      " stabilization coupling; thermoLambda { type Arrhenius; alpha 3000; T0 320; }"
                                      " thermoEta { type WLF; c1 8.86; c2 101.6; T0 300; }");
    auto tg = ConstitutiveEq::New("g", th);
    CHECK(tg->thermo().lambda.type == RT_THERMO_ARRHENIUS && tg->thermo().lambda.alpha == 3000.0 &&
          tg->thermo().lambda.T0 == 320.0);
    CHECK(tg->thermo().eta.type == RT_THERMO_WLF && tg->thermo().eta.c1 == 8.86 && tg->thermo().eta.c2 == 101.6);
    CHECK(tg->thermo().lambda2.type == RT_THERMO_CONSTANT);
    Dictionary thrp = Dictionary::parse("type Rolie-PolyLog; rho 1; etaS 0.1; etaP 0.9; lambdaD 1; lambdaR 0.2;"
                                        " beta 0; delta -0.5; chiMax 5; stabilization coupling;"
                                        " thermoLambdaR { type VFT; A 500; B -1; T0 150; }"
                                        " thermoLambdaD { type ArrheniusModified; alpha 0.02; T0 300; }");
    auto tr = ConstitutiveEq::New("rp", thrp);
    CHECK(tr->thermo().lambda.type == RT_THERMO_ARRHENIUS_MODIFIED && tr->thermo().lambda.alpha == 0.02);
    CHECK(tr->thermo().lambda2.type == RT_THERMO_VFT && tr->thermo().lambda2.A == 500.0 &&
          tr->thermo().lambda2.B == -1.0 && tr->thermo().lambda2.T0 == 150.0);
    CHECK(tr->thermo().eta.type == RT_THERMO_CONSTANT);
    Dictionary thbad = Dictionary::parse("type Oldroyd-BLog; rho 1; etaS 1; etaP 1; lambda 1; stabilization none;"
                                         " thermoEta { type Eyring; }");
    CHECK(throws([&] { ConstitutiveEq::New("o", thbad); }).find("Unknown thermoFunction type Eyring") !=
          std::string::npos);

    Dictionary nostab = Dictionary::parse("type Oldroyd-BLog; rho 1; etaS 1; etaP 1; lambda 1;");
    CHECK(throws([&] { ConstitutiveEq::New("o", nostab); }).find("stabilization") != std::string::npos);

    Dictionary sol = Dictionary::parse("p { solver PCG; preconditioner DIC; tolerance 1e-8; relTol 0; }"
                                       " U { solver PBiCG; preconditioner DILU; }"
                                       " T { solver PBiCGStab; preconditioner { preconditioner DILU; } }"
                                       " V { solver GAMG; smoother GaussSeidel; }");
    rt_solver_ctl cp = LduSolver::readControls(sol.subDict("p"));
    CHECK(cp.solver == RT_SOLVER_PCG && cp.preconditioner == RT_PRECOND_DIC && cp.tolerance == 1e-8);
    CHECK(cp.maxIter == 1000 && cp.minIter == 0 && cp.relTol == 0.0);
    rt_solver_ctl ct = LduSolver::readControls(sol.subDict("T"));
    CHECK(ct.solver == RT_SOLVER_PBICGSTAB && ct.preconditioner == RT_PRECOND_DILU && ct.tolerance == 1e-6);
    rt_solver_ctl cu = LduSolver::readControls(sol.subDict("U"));
    CHECK(cu.solver == RT_SOLVER_PBICG && cu.preconditioner == RT_PRECOND_DILU);
    std::string e1 = throws([&] { LduSolver::readControls(sol.subDict("V")); });
    CHECK(e1.find("Unknown lduMatrix::solver GAMG") != std::string::npos);
    CHECK(e1.find("PBiCG\nPBiCGStab\nPCG") != std::string::npos);

    // sparseSolver selection by solverType: only the openFoam type is served
    Dictionary ext = Dictionary::parse("solverType eigenSolver; solver BiCGSTAB; tolerance 1e-12;");
    std::string e3 = throws([&] { SparseSolver::readControls(ext); });
    CHECK(e3.find("Unknown sparseSolver solverType eigenSolver") != std::string::npos);
    Dictionary of = Dictionary::parse("solverType openFoam; solver PCG; preconditioner DIC; tolerance 1e-9;");
    CHECK(SparseSolver::readControls(of).solver == RT_SOLVER_PCG);

    std::string e2 = throws([&] { Context ctx(0); });
    CHECK(e2.find("rt_ctx_create") != std::string::npos);
}

// chain of n cells (one face between neighbours), no boundary faces
struct Chain {
    int n;
    std::vector<int32_t> own, nei;
    std::vector<double> Sf, magSf, Cf, w, dc, C, V;
    rt_mesh_desc desc{};
    explicit Chain(int n_) : n(n_) {
        for (int f = 0; f + 1 < n; ++f) {
            own.push_back(f);
            nei.push_back(f + 1);
            Sf.insert(Sf.end(), {1.0, 0.0, 0.0});
            magSf.push_back(1.0);
            Cf.insert(Cf.end(), {f + 1.0, 0.0, 0.0});
            w.push_back(0.5);
            dc.push_back(1.0);
        }
        for (int c = 0; c < n; ++c) {
            C.insert(C.end(), {c + 0.5, 0.0, 0.0});
            V.push_back(1.0);
        }
        desc.nCells = n;
        desc.nFaces = n - 1;
        desc.owner = own.data();
        desc.neighbour = nei.data();
        desc.Sf = Sf.data();
        desc.magSf = magSf.data();
        desc.Cf = Cf.data();
        desc.weights = w.data();
        desc.deltaCoeffs = dc.data();
        desc.C = C.data();
        desc.V = V.data();
        desc.solveDir[0] = desc.solveDir[1] = desc.solveDir[2] = 1;
    }
};

// Thomas algorithm for the tridiagonal LDU system
static std::vector<double> thomas(const std::vector<double> &d, const std::vector<double> &up,
                                  const std::vector<double> &lo, const std::vector<double> &b) {
    const int n = (int)d.size();
    std::vector<double> c(n), x(n), dd(d), bb(b);
    for (int i = 1; i < n; ++i) {   // row i: lo[i-1] x[i-1] + d[i] x[i] + up[i] x[i+1]
        double m = lo[i - 1] / dd[i - 1];
        dd[i] -= m * up[i - 1];
        bb[i] -= m * bb[i - 1];
    }
    x[n - 1] = bb[n - 1] / dd[n - 1];
    for (int i = n - 2; i >= 0; --i) x[i] = (bb[i] - up[i] * x[i + 1]) / dd[i];
    return x;
}

static void gpu_checks() {
    const int n = 5000;
    Chain ch(n);
    Context ctx(0);
    ctx.uploadMesh(ch.desc);
    std::vector<double> b(n);
    unsigned s = 12345u;
    for (int i = 0; i < n; ++i) {
        s = s * 1664525u + 1013904223u;
        b[i] = (double)(s >> 8) / (double)(1u << 24) - 0.5;
    }
    Dictionary sol = Dictionary::parse("p { solver PCG; preconditioner DIC; tolerance 1e-12; maxIter 20000; }"
                                       " T { solver PBiCGStab; preconditioner { preconditioner DILU; }"
                                       " tolerance 1e-12; maxIter 20000; }");
    for (const char *field : {"p", "T"}) {
        const bool sym = std::string(field) == "p";
        std::vector<double> d(n, sym ? 2.01 : 2.05), up(n - 1, sym ? -1.0 : -1.2), lo(n - 1, sym ? -1.0 : -0.8);
        LduMatrixView mv{d.data(), up.data(), lo.data()};
        auto solver = LduSolver::New(field, ctx, mv, sol.subDict(field));
        std::vector<double> x(n, 0.0);
        SolverPerformance perf = solver->solve(x.data(), b.data());
        std::vector<double> ref = thomas(d, up, lo, b);
        double num = 0, den = 0;
        for (int i = 0; i < n; ++i) {
            num += (x[i] - ref[i]) * (x[i] - ref[i]);
            den += ref[i] * ref[i];
        }
        std::printf("%s: %s %d iterations, residual %.3e -> %.3e, rel error %.3e\n", field,
                    perf.solverName.c_str(), perf.nIterations, perf.initialResidual, perf.finalResidual,
                    std::sqrt(num / den));
        CHECK(perf.converged && perf.nIterations > 0);
        CHECK(std::sqrt(num / den) < 1e-8);
    }
}

int main(int argc, char **argv) {
    const bool gpu = argc > 1 && std::strcmp(argv[1], "--gpu") == 0;
    try {
        if (gpu) gpu_checks();
        else cpu_checks();
    } catch (const FatalError &e) {
        std::fprintf(stderr, "FatalError: %s\n", e.what());
        return 2;
    }
    if (failures) return 1;
    std::printf("host checks passed (%s)\n", gpu ? "gpu" : "cpu");
    return 0;
}
