// sweep.h — structured-mesh data for the systolic DIC/DILU sweeps (sweep.cu).
#pragma once

#include "rt_internal.h"

namespace rt {

// per matrix: rD recurrence and the premultiplied sweep coefficients
void skew_prepare(rt_ctx *ctx, const double *diag, const double *upper, const double *lower);
// w = M^-1 r for the masked components (nc <= 6), forward then backward;
// dmask (device, or null): the components still iterating
void skew_precondition(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w,
                       const unsigned *dmask = nullptr);
// the transposed factorisation's coefficients (after skew_prepare of the
// same matrix) and w = M^-T r with them (PBiCG)
void skew_prepare_T(rt_ctx *ctx, const double *upper, const double *lower);
void skew_precondition_T(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w);
// 1/rD of the last skew_prepare in cell order (N doubles)
void skew_rdinv_cells(rt_ctx *ctx, double *rDc);
// mixed precision: skew_prepare, then FP32 copies of the sweep coefficients
void skew_prepare32(rt_ctx *ctx, const double *diag, const double *upper, const double *lower);
// FP32 w = M^-1 r with the coefficients of the last skew_prepare32
void skew_precondition32(rt_ctx *ctx, int nc, unsigned mask, const float *r, float *w);
// the same with an FP64 right-hand side and result (rounded on the way in and out)
void skew_precondition32d(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w,
                          const unsigned *dmask = nullptr);
// mg.cu: the aggregation multigrid V-cycle of the mixed pressure and
// momentum solves (FP32): the hierarchy of a matrix (sym: a symmetric one,
// its lower coefficients only), then w = V-cycle(r): mg_apply for the
// pressure (FP64 vectors; dm, device or null: component 0 still iterating),
// mg_apply32 for the momentum components in mask (FP32 vectors, component k
// at k N)
bool mg_available(rt_ctx *ctx);
void mg_prepare(rt_ctx *ctx, const double *diag, const double *upper, const double *lower, bool sym);
void mg_apply(rt_ctx *ctx, const double *r, double *w, const unsigned *dm = nullptr);
void mg_apply32(rt_ctx *ctx, unsigned mask, const float *r, float *w);
// whether the sweeps of a structured mesh with nJB j-blocks fit one CTA's shared memory
bool skew_fits(int nJB);
// RT_ETIMEOUT if a bounded wait of the last sweeps ran out
rt_status skew_check(rt_ctx *ctx);

}  // namespace rt
