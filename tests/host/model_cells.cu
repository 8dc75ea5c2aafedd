// model_cells.cu — a host build of the library's per-cell constitutive
// algebra (rheotool_gb300/csrc/constitutive_cell.cuh), the same source the
// theta-source and tau kernels inline, so that tests can compare it with the
// oracle's restatement on the CPU.  nvcc compiles it as host code; no kernel
// is launched.  Layouts are the device ones: structure of arrays, component
// k of cell c at k * n + c.
#include "../../rheotool_gb300/csrc/constitutive_cell.cuh"

extern "C" void mc_theta_source(const rt_model_params *mp, int n, const double *L, const double *eigVecs,
                                const double *eigVals, const double *theta, double *rhs, double *fP) {
    // the generalized PTT function's Gamma table, as the case setup makes it
    std::vector<double> g;
    if (mp->model == RT_MODEL_PTT_LOG && mp->pttFunction == RT_PTT_GENERALIZED) g = rt::ml_gamma_table(*mp);
    const int K = g.empty() ? 0 : (int)g.size() - 1;
    for (int c = 0; c < n; ++c)
        rt::theta_rhs_cell(c, n, *mp, L, eigVecs, eigVals, theta, rhs, fP, g.empty() ? nullptr : g.data(), K);
}

extern "C" void mc_tau(const rt_model_params *mp, int n, const double *eigVecs, const double *eigVals,
                       const double *fP, double *tau) {
    for (int c = 0; c < n; ++c) rt::tau_cell(c, n, *mp, eigVecs, eigVals, fP, tau);
}
