// fv_device.cuh — raw-pointer view of the device mesh and the per-cell
// finite-volume helpers shared by the kernels.
//
// Face loops are written cell-centric: a cell gathers the contributions of its
// faces in increasing face order (the ELL slots are sorted by face index), then
// its boundary faces in boundary-face order.  This is the order in which
// OpenFOAM's face-loop scatter (owner +=, neighbour -=) accumulates into each
// cell, so the gather is deterministic and free of atomics.
#pragma once

#include "rt_internal.h"

namespace rt {

struct MeshView {
    int N, F, NB, nSlots;
    const int *__restrict__ owner;
    const int *__restrict__ neighbour;
    const int *__restrict__ ellFace;
    const int *__restrict__ ellNbr;
    const int *__restrict__ bStart;
    const int *__restrict__ bList;
    const int *__restrict__ bCell;
    const double *__restrict__ Sf;      // 3F SoA
    const double *__restrict__ magSf;
    const double *__restrict__ w;
    const double *__restrict__ delta;
    const double *__restrict__ d;       // 3F SoA, C_N - C_P across each face
    const double *__restrict__ C;       // 3N SoA
    const double *__restrict__ V;
    const double *__restrict__ bSf;     // 3NB SoA
    const double *__restrict__ bmagSf;
    const double *__restrict__ bDelta;
    const double *__restrict__ bCtoF;   // 3NB SoA
    // batch of cases (null for one case): case of each cell, model of each case
    const int *__restrict__ caseOf;
    const rt_model_params *__restrict__ caseParams;
    const int *__restrict__ refCell;
    const double *__restrict__ refValue;
};

inline MeshView view(const DevMesh &m) {
    const bool b = m.batch.n > 1;
    return MeshView{m.N, m.F, m.NB, m.nSlots, m.owner.p, m.neighbour.p, m.ellFace.p, m.ellNbr.p,
                    m.bStart.p, m.bList.p, m.bCell.p, m.Sf.p, m.magSf.p, m.w.p, m.deltaCoeffs.p,
                    m.d.p, m.C.p, m.V.p, m.bSf.p, m.bmagSf.p, m.bDelta.p, m.bCtoF.p,
                    b ? m.batch.caseOf.p : nullptr, b ? m.batch.params.p : nullptr,
                    b ? m.batch.refCell.p : nullptr, b ? m.batch.refValue.p : nullptr};
}

// the model of cell c: the case's in a batch, else the context's
__device__ __forceinline__ const rt_model_params &model_of(const MeshView &m, const rt_model_params &mp, int c) {
    return m.caseOf ? m.caseParams[m.caseOf[c]] : mp;
}

// momentum-equation coefficients of a model (divTau, constitutiveEq.C:72-132):
// the implicit laplacian coefficient gam and the explicit one kG
struct MomCoef {
    int stab;
    double rho, gam, kG;
};
__host__ __device__ inline MomCoef mom_coef(const rt_model_params &mp) {
    MomCoef c;
    c.stab = mp.stabilization;
    c.rho = mp.rho;
    if (mp.stabilization == RT_STAB_COUPLING || mp.stabilization == RT_STAB_BSD) {
        c.gam = (mp.etaP + mp.etaS) / mp.rho;
        c.kG = mp.etaP / mp.rho;
    } else {
        c.gam = mp.etaS / mp.rho;
        c.kG = 0.0;
    }
    return c;
}

__device__ __forceinline__ double lin_interp(double w, double vP, double vN) {
    return w * (vP - vN) + vN;
}

// Gauss linear gradient of one scalar (stride-N SoA component) at cell c
__device__ __forceinline__ void cell_grad(const MeshView &m, int c, const double *__restrict__ x,
                                          const double *__restrict__ xb, double g[3]) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int s = 0; s < m.nSlots; ++s) {
        int nb = m.ellNbr[s * m.N + c];
        if (nb < 0) break;
        int f = m.ellFace[s * m.N + c];
        bool own = nb > c;
        double xf = own ? lin_interp(m.w[f], x[c], x[nb]) : lin_interp(m.w[f], x[nb], x[c]);
        double s0 = m.Sf[f] * xf, s1 = m.Sf[m.F + f] * xf, s2 = m.Sf[2 * m.F + f] * xf;
        if (own) { a0 += s0; a1 += s1; a2 += s2; }
        else     { a0 -= s0; a1 -= s1; a2 -= s2; }
    }
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int b = m.bList[i];
        double xf = xb[b];
        a0 += m.bSf[b] * xf;
        a1 += m.bSf[m.NB + b] * xf;
        a2 += m.bSf[2 * m.NB + b] * xf;
    }
    double v = m.V[c];
    g[0] = a0 / v; g[1] = a1 / v; g[2] = a2 / v;
}

// limiter table of gaussDefCmpwConvectionScheme lims() (limiters.H:39-100)
struct Lims {
    double al[3], be[3], bl[2];
};

inline Lims make_lims(int scheme) {
    Lims L;
    switch (scheme) {
    case RT_LIM_CUBISTA:  L = {{7. / 4., 3. / 4., 1. / 4.}, {0., 3. / 8., 3. / 4.}, {3. / 8., 3. / 4.}}; break;
    case RT_LIM_MINMOD:   L = {{1.5, .5, .5}, {0., .5, .5}, {.5, 1.}}; break;
    case RT_LIM_SMART:    L = {{3., 3. / 4., 0.}, {0., 3. / 8., 1.}, {1. / 6., 5. / 6.}}; break;
    case RT_LIM_WACEB:    L = {{2., 3. / 4., 0.}, {0., 3. / 8., 1.}, {3. / 10., 5. / 6.}}; break;
    case RT_LIM_SUPERBEE: L = {{0.5, 1.5, 0.}, {0.5, 0., 1.}, {1. / 2., 2. / 3.}}; break;
    default:              L = {{1., 1., 1.}, {0., 0., 0.}, {1., 1.}}; break;
    }
    return L;
}

}  // namespace rt
