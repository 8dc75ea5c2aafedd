// batch.h — Krylov solves and DIC/DILU sweeps of a batch of independent cases
// (krylov_batch.cu, sweep2d.cu).
#pragma once

#include "rt_internal.h"

namespace rt {

// per-segment state of the batched solvers (segment = case * 8 + component)
struct BSeg {
    double *nf, *init, *fin, *xbar, *A, *Aold, *alpha, *omega, *r0r, *r0rOld, *beta, *last;
    int *active, *iter, *sing, *repl, *rst, *conv;
    int *count;   // [0]: segments still iterating
};

// the case-aligned reduction blocks
struct BTab {
    int N, nBlk, nCases;
    const int *__restrict__ blkCase;
    const int *__restrict__ blkCell0;
    const int *__restrict__ blkCell1;
    const int *__restrict__ caseBlk;
    const int *__restrict__ caseOf;
};

// skewed layout of the structured 2-D cases (one CTA per case)
template <class Real>
struct Skew2D {
    int nCases, maxJB;
    long long nSkew;
    const int *__restrict__ T;
    const int *__restrict__ JB;
    const long long *__restrict__ off;
    const int *__restrict__ cellOf;
    Real *D, *Py, *Px, *rDraw;              // rD recurrence (FP64)
    Real *rDinv, *Ay, *Ax, *By, *Bx;        // premultiplied sweep coefficients
    Real *wS, *rS;                          // 6 components of nSkew each
};

rt_status batch_solve(rt_ctx *ctx, const SolveArgs &a, rt_solver_perf *perf);

// sweep2d.cu: rD of one matrix, then FP32 (or FP64) applications
void sweep2d_prepare(rt_ctx *ctx, const double *diag, const double *upper, const double *lower, bool fp32);
void sweep2d_precondition(rt_ctx *ctx, int nc, unsigned mask, const float *r, float *w);
void sweep2d_precondition(rt_ctx *ctx, int nc, unsigned mask, const double *r, double *w);
rt_status sweep2d_check(rt_ctx *ctx);
// the skewed layout of the batch (for the per-case persistent solver)
Skew2D<float> sweep2d_view32(rt_ctx *ctx);
Skew2D<double> sweep2d_view64(rt_ctx *ctx);

}  // namespace rt
