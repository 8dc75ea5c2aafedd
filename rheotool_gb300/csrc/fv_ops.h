// fv_ops.h — host-side launchers of the finite-volume kernels (fv.cu).
#pragma once

#include "rt_internal.h"

namespace rt {

// gradient of nc (1, 3 or 6) SoA components: g[(d*nc + k)*N + c]
void grad_field(rt_ctx *ctx, int nc, const double *x, const double *xb, double *g);

// GaussDefCmpw fvm::div(phi, x) for nc (3 or 6) components; g is grad_field(x).
// Writes the upwind lower/upper, the convective diagonal diagC (negSumDiag),
// the explicit source srcC (nc*N), and the boundary coefficients intC/bouC
// (nc*NB).  fluxTmp holds nc*F doubles.
void convection(rt_ctx *ctx, int scheme, int nc, const double *phi, const double *phib,
                const double *x, const double *xb, const int *bkind, const double *g,
                double *lower, double *upper, double *diagC, double *srcC, double *intC,
                double *bouC, double *fluxTmp);

// zeroGradient boundary values = cell values (nc SoA components)
void correct_bc(rt_ctx *ctx, const int *kind, int nc, const double *x, double *xb);

}  // namespace rt
