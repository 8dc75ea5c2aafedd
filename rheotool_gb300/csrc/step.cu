// step.cu — one segregated rheoFoam time step on the device
// (rheoFoam.C:147-154): UEqn.H (momentum with constitutiveEq::divTau),
// pEqn.H (SIMPLEC with ddtCorr, PCG-DIC pressure solve, flux and velocity
// correction), then constitutiveEq::correct().
#include <cmath>

#include "fv_device.cuh"
#include "fv_ops.h"

namespace rt {

// ---------------------------------------------------------------------------
// initial fields: boundary values from the BCs, phi = flux(U), eig = I
// ---------------------------------------------------------------------------
__global__ void k_init_bnd(int NB, const int *__restrict__ kU, const int *__restrict__ kP,
                           const int *__restrict__ kT, const int *__restrict__ kTa,
                           const double *__restrict__ UbF, const double *__restrict__ pbF,
                           const double *__restrict__ thF, const double *__restrict__ taF,
                           double *Ub, double *pb, double *thb, double *tab) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= NB) return;
    for (int k = 0; k < 3; ++k) Ub[(size_t)k * NB + b] = (kU[b] == RT_BC_FIXED) ? UbF[(size_t)k * NB + b] : 0.0;
    pb[b] = (kP[b] == RT_BC_FIXED) ? pbF[b] : 0.0;
    for (int k = 0; k < 6; ++k) {
        thb[(size_t)k * NB + b] = (kT[b] == RT_BC_FIXED) ? thF[(size_t)k * NB + b] : 0.0;
        tab[(size_t)k * NB + b] = (kTa[b] != RT_BC_ZEROGRAD) ? taF[(size_t)k * NB + b] : 0.0;
    }
}

__global__ void k_flux_U(MeshView m, const double *__restrict__ U, const double *__restrict__ Ub,
                         double *__restrict__ phi, double *__restrict__ phib) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < m.F) {
        int o = m.owner[f], n = m.neighbour[f];
        double w = m.w[f], v = 0.0;
        for (int j = 0; j < 3; ++j) v += m.Sf[(size_t)j * m.F + f] * lin_interp(w, U[(size_t)j * m.N + o], U[(size_t)j * m.N + n]);
        phi[f] = v;
    }
    if (f < m.NB) {
        int b = f;
        phib[b] = m.bSf[b] * Ub[b] + m.bSf[m.NB + b] * Ub[m.NB + b] + m.bSf[2 * m.NB + b] * Ub[2 * m.NB + b];
    }
}

__global__ void k_eye(int N, double *ev, double *vec) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    for (int k = 0; k < 3; ++k) ev[(size_t)k * N + c] = 1.0;
    for (int i = 0; i < 9; ++i) vec[(size_t)i * N + c] = (i == 0 || i == 4 || i == 8) ? 1.0 : 0.0;
}

void init_fields(rt_ctx *ctx) {
    DevMesh &mesh = ctx->mesh;
    DevCase &cs = ctx->cs;
    MeshView m = view(mesh);
    cudaStream_t s = ctx->stream;
    if (m.NB > 0) {
        k_init_bnd<<<nblocks(m.NB), RT_BLOCK, 0, s>>>(m.NB, cs.bkU.p, cs.bkP.p, cs.bkTh.p, cs.bkTau.p, cs.UbFixed.p,
                                                      cs.pbFixed.p, cs.thetabFixed.p, cs.taubFixed.p, cs.Ub.p,
                                                      cs.pb.p, cs.thetab.p, cs.taub.p);
        RT_CHECK_LAUNCH();
    }
    correct_bc(ctx, cs.bkU.p, 3, cs.U.p, cs.Ub.p);
    correct_bc(ctx, cs.bkP.p, 1, cs.p.p, cs.pb.p);
    correct_bc(ctx, cs.bkTh.p, 6, cs.theta.p, cs.thetab.p);
    correct_bc(ctx, cs.bkTau.p, 6, cs.tau.p, cs.taub.p);
    int nf = std::max(m.F, m.NB);
    if (nf > 0) k_flux_U<<<nblocks(nf), RT_BLOCK, 0, s>>>(m, cs.U.p, cs.Ub.p, cs.phi.p, cs.phib.p);
    k_eye<<<nblocks(m.N), RT_BLOCK, 0, s>>>(m.N, cs.eigVals.p, cs.eigVecs.p);
    RT_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// momentum equation
// ---------------------------------------------------------------------------
// explicit part of divTau: div(tau/rho) - div(kG grad U) (coupling) or
// - laplacian(kG, U) (BSD), both Gauss linear
__global__ void k_divtau_expl(MeshView m, MomCoef mc0,
                              const double *__restrict__ tau, const double *__restrict__ taub,
                              const double *__restrict__ G, const double *__restrict__ U,
                              const double *__restrict__ Ub, double *__restrict__ expl) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const MomCoef mc = m.caseOf ? mom_coef(m.caseParams[m.caseOf[c]]) : mc0;
    const int stab = mc.stab;
    const double rho = mc.rho, kG = mc.kG;
    const int N = m.N, NB = m.NB, F = m.F;
    double dt0 = 0.0, dt1 = 0.0, dt2 = 0.0;     // div(tau/rho) sums
    double dg0 = 0.0, dg1 = 0.0, dg2 = 0.0;     // div(kG grad U) or laplacian sums
    for (int s = 0; s < m.nSlots; ++s) {
        int nb = m.ellNbr[s * N + c];
        if (nb < 0) break;
        int f = m.ellFace[s * N + c];
        bool own = nb > c;
        int o = own ? c : nb, n = own ? nb : c;
        double w = m.w[f];
        double S0 = m.Sf[f], S1 = m.Sf[F + f], S2 = m.Sf[2 * F + f];
        double Tf[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) Tf[q] = lin_interp(w, tau[(size_t)q * N + o] / rho, tau[(size_t)q * N + n] / rho);
        double v0 = S0 * Tf[0] + S1 * Tf[1] + S2 * Tf[2];
        double v1 = S0 * Tf[1] + S1 * Tf[3] + S2 * Tf[4];
        double v2 = S0 * Tf[2] + S1 * Tf[4] + S2 * Tf[5];
        if (own) { dt0 += v0; dt1 += v1; dt2 += v2; } else { dt0 -= v0; dt1 -= v1; dt2 -= v2; }
        if (stab == RT_STAB_COUPLING) {
            double Gf[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) Gf[q] = lin_interp(w, kG * G[(size_t)q * N + o], kG * G[(size_t)q * N + n]);
            double u0 = S0 * Gf[0] + S1 * Gf[3] + S2 * Gf[6];
            double u1 = S0 * Gf[1] + S1 * Gf[4] + S2 * Gf[7];
            double u2 = S0 * Gf[2] + S1 * Gf[5] + S2 * Gf[8];
            if (own) { dg0 += u0; dg1 += u1; dg2 += u2; } else { dg0 -= u0; dg1 -= u1; dg2 -= u2; }
        } else if (stab == RT_STAB_BSD) {
            double gm = kG * m.magSf[f], dl = m.delta[f];
            double u0 = gm * (dl * (U[n] - U[o]));
            double u1 = gm * (dl * (U[N + n] - U[N + o]));
            double u2 = gm * (dl * (U[2 * N + n] - U[2 * N + o]));
            if (own) { dg0 += u0; dg1 += u1; dg2 += u2; } else { dg0 -= u0; dg1 -= u1; dg2 -= u2; }
        }
    }
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int b = m.bList[i];
        double S0 = m.bSf[b], S1 = m.bSf[NB + b], S2 = m.bSf[2 * NB + b];
        double Tf[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) Tf[q] = taub[(size_t)q * NB + b] / rho;
        dt0 += S0 * Tf[0] + S1 * Tf[1] + S2 * Tf[2];
        dt1 += S0 * Tf[1] + S1 * Tf[3] + S2 * Tf[4];
        dt2 += S0 * Tf[2] + S1 * Tf[4] + S2 * Tf[5];
        if (stab == RT_STAB_COUPLING) {
            // boundary gradient: cell value with the normal part replaced by snGrad
            double mg = m.bmagSf[b];
            double n0 = S0 / mg, n1 = S1 / mg, n2 = S2 / mg;
            double Gb[9];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                double sn = m.bDelta[b] * (Ub[(size_t)j * NB + b] - U[(size_t)j * N + c]);
                double g0 = G[(size_t)(0 + j) * N + c], g1 = G[(size_t)(3 + j) * N + c], g2 = G[(size_t)(6 + j) * N + c];
                double ng = 0.0;
                ng += n0 * g0;
                ng += n1 * g1;
                ng += n2 * g2;
                Gb[0 + j] = g0 + n0 * (sn - ng);
                Gb[3 + j] = g1 + n1 * (sn - ng);
                Gb[6 + j] = g2 + n2 * (sn - ng);
            }
            dg0 += S0 * (kG * Gb[0]) + S1 * (kG * Gb[3]) + S2 * (kG * Gb[6]);
            dg1 += S0 * (kG * Gb[1]) + S1 * (kG * Gb[4]) + S2 * (kG * Gb[7]);
            dg2 += S0 * (kG * Gb[2]) + S1 * (kG * Gb[5]) + S2 * (kG * Gb[8]);
        } else if (stab == RT_STAB_BSD) {
            double gm = kG * m.bmagSf[b], dl = m.bDelta[b];
            dg0 += gm * (dl * (Ub[b] - U[c]));
            dg1 += gm * (dl * (Ub[NB + b] - U[N + c]));
            dg2 += gm * (dl * (Ub[2 * NB + b] - U[2 * N + c]));
        }
    }
    double v = m.V[c];
    double e0 = dt0 / v, e1 = dt1 / v, e2 = dt2 / v;
    if (stab != RT_STAB_NONE) {
        e0 -= dg0 / v;
        e1 -= dg1 / v;
        e2 -= dg2 / v;
    }
    expl[c] = e0;
    expl[(size_t)N + c] = e1;
    expl[(size_t)2 * N + c] = e2;
}

// lower/upper -= gam |Sf| deltaCoeffs (the laplacian subtracted)
__global__ void k_sub_lap(MeshView m, double gam0, double *__restrict__ lower, double *__restrict__ upper) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.F) return;
    const double gam = m.caseOf ? mom_coef(m.caseParams[m.caseOf[m.owner[f]]]).gam : gam0;
    double up = gam * m.magSf[f] * m.delta[f];
    upper[f] -= up;
    lower[f] -= up;
}

// UEqn diag and source
// (body: the uniform body force per unit mass, added to the explicit divTau
// terms before they are integrated over the cell)
// (DU non-null: Crank-Nicolson, diag (c/dt) V and source ((c/dt) U0 + psi DU) V
// with rDeltaT = c/dt; else Euler)
__global__ void k_mom_cell(MeshView m, double rDeltaT, double gam0, const double *__restrict__ diagC,
                           const double *__restrict__ srcC, const double *__restrict__ U0,
                           const double *__restrict__ expl, double3 body, double *__restrict__ diag,
                           double *__restrict__ src, double psi, const double *__restrict__ DU) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const double gam = m.caseOf ? mom_coef(m.caseParams[m.caseOf[c]]).gam : gam0;
    const int N = m.N;
    double ld = 0.0;
    for (int s = 0; s < m.nSlots; ++s) {
        int nb = m.ellNbr[s * N + c];
        if (nb < 0) break;
        int f = m.ellFace[s * N + c];
        ld -= gam * m.magSf[f] * m.delta[f];
    }
    double v = m.V[c];
    diag[c] = ((0.0 + rDeltaT * v) + diagC[c]) - ld;
    const double bf[3] = {body.x, body.y, body.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const size_t i = (size_t)k * N + c;
        const double ddtSrc = DU ? (rDeltaT * U0[i] + psi * DU[i]) * v : rDeltaT * U0[i] * v;
        src[i] = ((0.0 + ddtSrc) + srcC[i]) + v * (expl[i] + bf[k]);
    }
}

// boundary coefficients of UEqn: convection minus laplacian (fixedValue faces)
__global__ void k_mom_bnd(MeshView m, double gam0, const int *__restrict__ kU, const double *__restrict__ Ub,
                          double *__restrict__ intC, double *__restrict__ bouC) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int NB = m.NB;
    if (b >= NB) return;
    if (kU[b] != RT_BC_FIXED) return;
    const double gam = m.caseOf ? mom_coef(m.caseParams[m.caseOf[m.bCell[b]]]).gam : gam0;
    double gm = gam * m.bmagSf[b];
    for (int k = 0; k < 3; ++k) {
        intC[(size_t)k * NB + b] -= gm * (-m.bDelta[b]);
        bouC[(size_t)k * NB + b] -= -gm * (m.bDelta[b] * Ub[(size_t)k * NB + b]);
    }
}

// solve(UEqn == -grad p): complete diagonal and source
__global__ void k_mom_solve_prep(MeshView m, const double *__restrict__ diag, const double *__restrict__ src,
                                 const double *__restrict__ gp, const double *__restrict__ intC,
                                 const double *__restrict__ bouC, double *__restrict__ dS, double *__restrict__ bS) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const int N = m.N;
    double v = m.V[c];
    double d = diag[c];
    double b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) b[k] = src[(size_t)k * N + c] + v * (-gp[(size_t)k * N + c]);
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int bf = m.bList[i];
        d += intC[bf];
#pragma unroll
        for (int k = 0; k < 3; ++k) b[k] += bouC[(size_t)k * m.NB + bf];
    }
    dS[c] = d;
#pragma unroll
    for (int k = 0; k < 3; ++k) bS[(size_t)k * N + c] = b[k];
}

// ---------------------------------------------------------------------------
// pressure equation
// ---------------------------------------------------------------------------
// rAU = 1/A, H, H1, HbyA, rAtU
__global__ void k_AH(MeshView m, const double *__restrict__ diag, const double *__restrict__ lower,
                     const double *__restrict__ upper, const double *__restrict__ src,
                     const double *__restrict__ intC, const double *__restrict__ bouC,
                     const double *__restrict__ U, double *__restrict__ rAU, double *__restrict__ HbyA,
                     double *__restrict__ rAtU, double *__restrict__ Hout) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const int N = m.N, NB = m.NB;
    double A = diag[c];
    double H[3] = {0.0, 0.0, 0.0};
    double Uc[3] = {U[c], U[N + c], U[2 * N + c]};
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int b = m.bList[i];
        double i0 = intC[b], i1 = intC[NB + b], i2 = intC[2 * NB + b];
        double av = (i0 + i1 + i2) / 3.0;
        A += av;
        H[0] += (av - i0) * Uc[0];
        H[1] += (av - i1) * Uc[1];
        H[2] += (av - i2) * Uc[2];
    }
    double H1 = 0.0;
    for (int s = 0; s < m.nSlots; ++s) {
        int nb = m.ellNbr[s * N + c];
        if (nb < 0) break;
        int f = m.ellFace[s * N + c];
        double a = nb > c ? upper[f] : lower[f];
#pragma unroll
        for (int k = 0; k < 3; ++k) H[k] -= a * U[(size_t)k * N + nb];
        H1 -= a;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) H[k] += src[(size_t)k * N + c];
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int b = m.bList[i];
#pragma unroll
        for (int k = 0; k < 3; ++k) H[k] += bouC[(size_t)k * NB + b];
    }
    double v = m.V[c];
    double r = 1.0 / (A / v);
    H1 /= v;
    rAU[c] = r;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double h = H[k] / v;
        Hout[(size_t)k * N + c] = h;
        HbyA[(size_t)k * N + c] = r * h;
    }
    rAtU[c] = 1.0 / (1.0 / r - H1);
}

// HbyA boundary values: U_b on fixedValue patches, rAU_P H_P elsewhere
__global__ void k_HbyA_bnd(int NB, int N, const int *__restrict__ kU, const int *__restrict__ bCell,
                           const double *__restrict__ Ub, const double *__restrict__ rAU,
                           const double *__restrict__ H, double *__restrict__ HbyAb) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= NB) return;
    int c = bCell[b];
    for (int k = 0; k < 3; ++k)
        HbyAb[(size_t)k * NB + b] = (kU[b] == RT_BC_FIXED) ? Ub[(size_t)k * NB + b] : rAU[c] * H[(size_t)k * N + c];
}

// phiHbyA on internal faces: flux(HbyA) + interp(rAU) ddtCorr + interp(rAtU - rAU) snGrad(p) |Sf|
// (DU non-null: Crank-Nicolson ddtCorr with the old-time parts rc x0 + psi D
// of phi and U, rc = c/dt; else Euler with rDeltaT)
__global__ void k_phiHbyA(MeshView m, double rDeltaT, const double *__restrict__ HbyA,
                          const double *__restrict__ U0, const double *__restrict__ phi0,
                          const double *__restrict__ rAU, const double *__restrict__ rAtU,
                          const double *__restrict__ p, double *__restrict__ phiHbyA,
                          double *partial, int nBlk, double *__restrict__ absPreF, double rc, double psi,
                          const double *__restrict__ DU, const double *__restrict__ Dphi) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    double absPre = 0.0;
    if (f < m.F) {
        const int N = m.N, F = m.F;
        int o = m.owner[f], n = m.neighbour[f];
        double w = m.w[f];
        double hf = 0.0, u0f = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double S = m.Sf[(size_t)j * F + f];
            hf += S * lin_interp(w, HbyA[(size_t)j * N + o], HbyA[(size_t)j * N + n]);
            u0f += S * lin_interp(w, U0[(size_t)j * N + o], U0[(size_t)j * N + n]);
        }
        double phiCorr = phi0[f] - u0f;
        double cc = 1.0 - fmin(fabs(phiCorr) / (fabs(phi0[f]) + 1e-15), 1.0);
        double ddtCorr = cc * rDeltaT * phiCorr;
        if (DU) {
            double uf = 0.0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const size_t io = (size_t)j * N + o, in = (size_t)j * N + n;
                uf += m.Sf[(size_t)j * F + f] * lin_interp(w, rc * U0[io] + psi * DU[io], rc * U0[in] + psi * DU[in]);
            }
            ddtCorr = cc * ((rc * phi0[f] + psi * Dphi[f]) - uf);
        }
        double pre = hf + lin_interp(w, rAU[o], rAU[n]) * ddtCorr;
        absPre = fabs(pre);
        if (absPreF) absPreF[f] = absPre;
        double dr = lin_interp(w, rAtU[o] - rAU[o], rAtU[n] - rAU[n]);
        phiHbyA[f] = pre + dr * (m.delta[f] * (p[n] - p[o])) * m.magSf[f];
    }
    if (partial) {
        // sum |phiHbyA| before the snGrad term (adjustCorrPhi normalisation)
        __shared__ double sh[RT_BLOCK / 32];
        double v = absPre;
        for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int i = 0; i < RT_BLOCK / 32; ++i) t += sh[i];
            partial[blockIdx.x] = t;
        }
    }
}

// boundary phiHbyA before adjustCorrPhi
__global__ void k_phiHbyA_bnd_pre(MeshView m, double rDeltaT, const int *__restrict__ kU,
                                  const double *__restrict__ HbyAb, const double *__restrict__ U0b,
                                  const double *__restrict__ phi0b, const double *__restrict__ rAU,
                                  double *__restrict__ phiHbyAb, double rc, double psi,
                                  const double *__restrict__ DUb, const double *__restrict__ Dphib) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.NB) return;
    const int NB = m.NB;
    int c = m.bCell[b];
    double S0 = m.bSf[b], S1 = m.bSf[NB + b], S2 = m.bSf[2 * NB + b];
    double hf = S0 * HbyAb[b] + S1 * HbyAb[NB + b] + S2 * HbyAb[2 * NB + b];
    double u0f = S0 * U0b[b] + S1 * U0b[NB + b] + S2 * U0b[2 * NB + b];
    double phiCorr = phi0b[b] - u0f;
    double cc = (kU[b] == RT_BC_FIXED) ? 0.0 : 1.0 - fmin(fabs(phiCorr) / (fabs(phi0b[b]) + 1e-15), 1.0);
    double ddtCorr = cc * rDeltaT * phiCorr;
    if (DUb) {
        const double uf = S0 * (rc * U0b[b] + psi * DUb[b]) + S1 * (rc * U0b[NB + b] + psi * DUb[NB + b]) +
                          S2 * (rc * U0b[2 * NB + b] + psi * DUb[2 * NB + b]);
        ddtCorr = cc * ((rc * phi0b[b] + psi * Dphib[b]) - uf);
    }
    phiHbyAb[b] = hf + rAU[c] * ddtCorr;
}

// adjustCorrPhi: one block; sums over the boundary faces in a fixed order
__global__ void k_adjust_corr_phi(int NB, int nPartial, const int *__restrict__ kU,
                                  const double *__restrict__ partial, double *__restrict__ phiHbyAb,
                                  int *__restrict__ status) {
    __shared__ double sh[4][RT_BLOCK];
    double mi = 0.0, fo = 0.0, ao = 0.0, tot = 0.0;
    for (int b = threadIdx.x; b < NB; b += blockDim.x) {
        double v = phiHbyAb[b];
        if (v < 0.0) mi -= v;
        else if (kU[b] == RT_BC_FIXED) fo += v;
        else ao += v;
    }
    for (int i = threadIdx.x; i < nPartial; i += blockDim.x) tot += partial[i];
    sh[0][threadIdx.x] = mi; sh[1][threadIdx.x] = fo; sh[2][threadIdx.x] = ao; sh[3][threadIdx.x] = tot;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    double massIn = sh[0][0], fixedOut = sh[1][0], adjOut = sh[2][0], total = 1e-300 + sh[3][0];
    double corr = 1.0;
    bool doCorr = fabs(adjOut) > 1e-300 && fabs(adjOut) / total > 1e-15;
    if (doCorr) corr = (massIn - fixedOut) / adjOut;
    else if (fabs(fixedOut - massIn) / total > 1e-8 && threadIdx.x == 0 && status) *status = 1;
    if (doCorr)
        for (int b = threadIdx.x; b < NB; b += blockDim.x)
            if (kU[b] != RT_BC_FIXED && phiHbyAb[b] > 0.0) phiHbyAb[b] *= corr;
}

// adjustCorrPhi of a batch: block b treats case b (cases without a pressure
// reference are left alone), same sums in the same order as above over the
// case's own boundary faces and internal faces
__global__ void k_adjust_corr_phi_batch(const int *__restrict__ refCell, const int *__restrict__ bStart,
                                        const int *__restrict__ fStart, const int *__restrict__ kU,
                                        const double *__restrict__ absPreF, double *__restrict__ phiHbyAb,
                                        int *__restrict__ status) {
    const int cb = blockIdx.x;
    if (refCell[cb] < 0) return;
    const int b0 = bStart[cb], b1 = bStart[cb + 1], f0 = fStart[cb], f1 = fStart[cb + 1];
    __shared__ double sh[4][RT_BLOCK];
    double mi = 0.0, fo = 0.0, ao = 0.0, tot = 0.0;
    for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
        double v = phiHbyAb[b];
        if (v < 0.0) mi -= v;
        else if (kU[b] == RT_BC_FIXED) fo += v;
        else ao += v;
    }
    for (int f = f0 + threadIdx.x; f < f1; f += blockDim.x) tot += absPreF[f];
    sh[0][threadIdx.x] = mi; sh[1][threadIdx.x] = fo; sh[2][threadIdx.x] = ao; sh[3][threadIdx.x] = tot;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    double massIn = sh[0][0], fixedOut = sh[1][0], adjOut = sh[2][0], total = 1e-300 + sh[3][0];
    double corr = 1.0;
    bool doCorr = fabs(adjOut) > 1e-300 && fabs(adjOut) / total > 1e-15;
    if (doCorr) corr = (massIn - fixedOut) / adjOut;
    else if (fabs(fixedOut - massIn) / total > 1e-8 && threadIdx.x == 0 && status) *status = 1;
    if (doCorr)
        for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x)
            if (kU[b] != RT_BC_FIXED && phiHbyAb[b] > 0.0) phiHbyAb[b] *= corr;
}

// boundary phiHbyA += (rAtU - rAU)_P snGrad(p) |Sf|
__global__ void k_phiHbyA_bnd_post(MeshView m, const int *__restrict__ kP, const double *__restrict__ rAU,
                                   const double *__restrict__ rAtU, const double *__restrict__ p,
                                   const double *__restrict__ pb, double *__restrict__ phiHbyAb) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.NB) return;
    int c = m.bCell[b];
    double sn = (kP[b] == RT_BC_FIXED) ? m.bDelta[b] * (pb[b] - p[c]) : 0.0;
    phiHbyAb[b] += (rAtU[c] - rAU[c]) * sn * m.bmagSf[b];
}

// p-laplacian coefficients
__global__ void k_pmat_face(MeshView m, const double *__restrict__ rAtU, double *__restrict__ pu) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.F) return;
    int o = m.owner[f], n = m.neighbour[f];
    double gm = lin_interp(m.w[f], rAtU[o], rAtU[n]) * m.magSf[f];
    pu[f] = m.delta[f] * gm;
}

__global__ void k_pmat_bnd(MeshView m, const int *__restrict__ kP, const double *__restrict__ rAtU,
                           const double *__restrict__ pb, double *__restrict__ pIntC, double *__restrict__ pBouC) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.NB) return;
    if (kP[b] == RT_BC_FIXED) {
        double gm = rAtU[m.bCell[b]] * m.bmagSf[b];
        pIntC[b] = gm * (-m.bDelta[b]);
        pBouC[b] = -gm * (m.bDelta[b] * pb[b]);
    } else {
        pIntC[b] = 0.0;
        pBouC[b] = 0.0;
    }
}

// p diag (negSumDiag), source V div(phiHbyA), setReference, complete diag/source
__global__ void k_pmat_cell(MeshView m, const double *__restrict__ pu, const double *__restrict__ phiHbyA,
                            const double *__restrict__ phiHbyAb, const double *__restrict__ pIntC,
                            const double *__restrict__ pBouC, int needRef, int refCell, double refValue,
                            double *__restrict__ dS, double *__restrict__ bS) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const int N = m.N;
    double pd = 0.0, dv = 0.0;
    for (int s = 0; s < m.nSlots; ++s) {
        int nb = m.ellNbr[s * N + c];
        if (nb < 0) break;
        int f = m.ellFace[s * N + c];
        pd -= pu[f];
        if (nb > c) dv += phiHbyA[f]; else dv -= phiHbyA[f];
    }
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) dv += phiHbyAb[m.bList[i]];
    double v = m.V[c];
    double ps = 0.0 + v * (dv / v);
    if (m.caseOf) {
        const int b = m.caseOf[c];
        if (m.refCell[b] == c) {
            ps += pd * m.refValue[b];
            pd += pd;
        }
    } else if (needRef && c == refCell) {
        ps += pd * refValue;
        pd += pd;
    }
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int b = m.bList[i];
        pd += pIntC[b];
        ps += pBouC[b];
    }
    dS[c] = pd;
    bS[c] = ps;
}

// phi = phiHbyA - pEqn.flux()
__global__ void k_phi_update(MeshView m, const double *__restrict__ phiHbyA, const double *__restrict__ phiHbyAb,
                             const double *__restrict__ pu, const double *__restrict__ pIntC,
                             const double *__restrict__ pBouC, const double *__restrict__ p,
                             double *__restrict__ phi, double *__restrict__ phib) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < m.F) {
        int o = m.owner[f], n = m.neighbour[f];
        phi[f] = phiHbyA[f] - (pu[f] * p[n] - pu[f] * p[o]);
    }
    if (f < m.NB) phib[f] = phiHbyAb[f] - (pIntC[f] * p[m.bCell[f]] - pBouC[f]);
}

// U = (HbyA - (rAU - rAtU) grad p_old) - rAtU grad p_new
__global__ void k_U_correct(int N, const double *__restrict__ HbyA, const double *__restrict__ rAU,
                            const double *__restrict__ rAtU, const double *__restrict__ gpOld,
                            const double *__restrict__ gpNew, double *__restrict__ U) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    double ra = rAU[c], rt = rAtU[c];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        size_t i = (size_t)k * N + c;
        double h = HbyA[i] - (ra - rt) * gpOld[i];
        U[i] = h - rt * gpNew[i];
    }
}

// ---------------------------------------------------------------------------
// one inner iteration of a time step (UEqn, pEqn, constEq.correct()) on the
// step's old-time fields U0, U0b, phi0, phi0b and theta0 (null: the current theta)
static rt_status step_inner(rt_ctx *ctx, rt_step_perf *perf, const double *U0, const double *U0b,
                            const double *phi0, const double *phi0b, const double *theta0) {
    DevMesh &mesh = ctx->mesh;
    DevCase &cs = ctx->cs;
    const rt_case_ctl &ctl = cs.ctl;
    const rt_model_params &mp = cs.mp;
    const int N = mesh.N, F = mesh.F, NB = mesh.NB;
    const double rDeltaT = 1.0 / ctl.deltaT;
    cudaStream_t s = ctx->stream;
    MeshView m = view(mesh);
    Work &W = ctx->work;
    WorkMark wmark(W);
    const int gN = nblocks(N), gF = nblocks(F), gB = nblocks(std::max(NB, 1));

    // ---------------- UEqn ----------------
    double *G = W.take(9 * (size_t)N);
    const double fpc = (double)F / N;
    {
        ProfScope ps(ctx, "grad", (double)N * (24.0 + 72.0 + fpc * 16.0 + 72.0 + 72.0));
        grad_field(ctx, 3, cs.U.p, cs.Ub.p, G);
    }
    double *lower = W.take(F), *upper = W.take(F), *diagC = W.take(N), *srcC = W.take(3 * (size_t)N);
    double *intC = W.take(3 * (size_t)NB), *bouC = W.take(3 * (size_t)NB), *flux = W.take(3 * (size_t)F);
    {
        ProfScope ps(ctx, "convection", (double)N * (24.0 + 72.0 + 24.0 + fpc * (8.0 + 8.0 + 16.0 + 16.0 + 2 * 24.0) + 8.0 + 24.0));
        convection(ctx, ctl.divU, 3, cs.phi.p, cs.phib.p, cs.U.p, cs.Ub.p, cs.bkU.p, G, lower, upper, diagC, srcC,
                   intC, bouC, flux);
    }
    // (multiMode: the summed divTau of the modes, one divTau with the summed
    // tau and viscosities, multiMode.C:144-156)
    const bool multi = cs.nModes > 1;
    const MomCoef mc = mom_coef(multi ? cs.mpMom : mp);
    const double gam = mc.gam;
    double *expl = W.take(3 * (size_t)N);
    ProfScope psMom(ctx, "mom_assembly", (double)N * (48.0 + 72.0 + 24.0 + 24.0 + 8.0 + 24.0 + 24.0 + 24.0 + 8.0 + 24.0) + F * 32.0);
    k_divtau_expl<<<gN, RT_BLOCK, 0, s>>>(m, mc, multi ? cs.tauTot.p : cs.tau.p, multi ? cs.taubTot.p : cs.taub.p, G,
                                          cs.U.p, cs.Ub.p, expl);
    double *diag = W.take(N), *src = W.take(3 * (size_t)N);
    const double3 body = make_double3(ctl.bodyForce[0], ctl.bodyForce[1], ctl.bodyForce[2]);
    // Crank-Nicolson: the step's ddt coefficient c/dt and the old-time derivatives
    const bool cn = ctl.ddtScheme == RT_DDT_CRANKNICOLSON;
    const double rc = cs.ddtC * rDeltaT, psi = cn ? ctl.ddtPsi : 0.0;
    k_mom_cell<<<gN, RT_BLOCK, 0, s>>>(m, cn ? rc : rDeltaT, gam, diagC, srcC, U0, expl, body, diag, src, psi,
                                       cn ? cs.DU.p : nullptr);
    if (F) k_sub_lap<<<gF, RT_BLOCK, 0, s>>>(m, gam, lower, upper);
    if (NB) k_mom_bnd<<<gB, RT_BLOCK, 0, s>>>(m, gam, cs.bkU.p, cs.Ub.p, intC, bouC);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 4);
    double *gp = W.take(3 * (size_t)N);
    grad_field(ctx, 1, cs.p.p, cs.pb.p, gp);
    double *dS = W.take(N), *bS = W.take(3 * (size_t)N);
    k_mom_solve_prep<<<gN, RT_BLOCK, 0, s>>>(m, diag, src, gp, intC, bouC, dS, bS);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
    unsigned maskU = 0;
    for (int k = 0; k < 3; ++k)
        if (mesh.solveDir[k]) maskU |= 1u << k;
    SolveArgs ua{dS, upper, lower, bS, cs.U.p, 3, maskU, ctl.solverU, ctl.precision, 0};
    prof_end(ctx, psMom.rec, psMom.bytes);
    psMom.rec = -1;
    rt_status st;
    {
        ProfScope ps(ctx, "solve_U");
        st = ldu_solve_device(ctx, ua, perf->U);
    }
    if (st != RT_OK && st != RT_ENOCONV) return st;
    correct_bc(ctx, cs.bkU.p, 3, cs.U.p, cs.Ub.p);

    // ---------------- pEqn ----------------
    double *rAU = W.take(N), *rAtU = W.take(N), *HbyA = W.take(3 * (size_t)N), *H = W.take(3 * (size_t)N);
    ProfScope psP(ctx, "p_assembly", (double)N * (8.0 + 24.0 + 24.0 + 24.0 + 24.0 + 8.0 + 8.0 + 24.0) + F * 48.0);
    k_AH<<<gN, RT_BLOCK, 0, s>>>(m, diag, lower, upper, src, intC, bouC, cs.U.p, rAU, HbyA, rAtU, H);
    double *HbyAb = W.take(3 * (size_t)NB);
    if (NB) k_HbyA_bnd<<<gB, RT_BLOCK, 0, s>>>(NB, N, cs.bkU.p, mesh.bCell.p, cs.Ub.p, rAU, H, HbyAb);
    double *phiHbyA = W.take(F), *phiHbyAb = W.take(NB);
    const bool batched = mesh.batch.n > 1;
    double *partial = (ctl.needReference && !batched) ? W.take(gF + 1) : nullptr;
    double *absPreF = batched ? W.take(F + 1) : nullptr;
    if (F)
        k_phiHbyA<<<gF, RT_BLOCK, 0, s>>>(m, rDeltaT, HbyA, U0, phi0, rAU, rAtU, cs.p.p, phiHbyA, partial, gF,
                                          absPreF, rc, psi, cn ? cs.DU.p : nullptr, cn ? cs.Dphi.p : nullptr);
    if (NB)
        k_phiHbyA_bnd_pre<<<gB, RT_BLOCK, 0, s>>>(m, rDeltaT, cs.bkU.p, HbyAb, U0b, phi0b, rAU, phiHbyAb, rc, psi,
                                                  cn ? cs.DUb.p : nullptr, cn ? cs.Dphib.p : nullptr);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 4);
    if (batched) {
        const Batch &bt = mesh.batch;
        k_adjust_corr_phi_batch<<<bt.n, RT_BLOCK, 0, s>>>(bt.refCell.p, bt.bStartD.p, bt.faceStartD.p, cs.bkU.p,
                                                          absPreF, phiHbyAb, nullptr);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    } else if (ctl.needReference && NB) {
        k_adjust_corr_phi<<<1, RT_BLOCK, 0, s>>>(NB, F ? gF : 0, cs.bkU.p, partial, phiHbyAb, nullptr);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }
    if (NB) {
        k_phiHbyA_bnd_post<<<gB, RT_BLOCK, 0, s>>>(m, cs.bkP.p, rAU, rAtU, cs.p.p, cs.pb.p, phiHbyAb);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    }
    double *pu = W.take(F), *pIntC = W.take(NB), *pBouC = W.take(NB), *pd = W.take(N), *ps = W.take(N);
    if (F) k_pmat_face<<<gF, RT_BLOCK, 0, s>>>(m, rAtU, pu);
    if (NB) k_pmat_bnd<<<gB, RT_BLOCK, 0, s>>>(m, cs.bkP.p, rAtU, cs.pb.p, pIntC, pBouC);
    k_pmat_cell<<<gN, RT_BLOCK, 0, s>>>(m, pu, phiHbyA, phiHbyAb, pIntC, pBouC, ctl.needReference, ctl.pRefCell,
                                        ctl.pRefValue, pd, ps);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 3);
    SolveArgs pa{pd, pu, pu, ps, cs.p.p, 1, 1u, ctl.solverP, ctl.precision, 1};
    prof_end(ctx, psP.rec, psP.bytes);
    psP.rec = -1;
    // the non-orthogonal corrector loop (pEqn.H:31-50): the orthogonal
    // laplacian makes every corrector the same equation, solved from the last
    // corrector's p; the flux follows the last
    const int nCorr = ctl.nNonOrthCorr > 0 ? ctl.nNonOrthCorr : 0;
    for (int corr = 0; corr <= nCorr; ++corr) {
        rt_status sp;
        {
            ProfScope pss(ctx, "solve_p");
            sp = ldu_solve_device(ctx, pa, &perf->p);
        }
        if (sp != RT_OK && sp != RT_ENOCONV) return sp;
        correct_bc(ctx, cs.bkP.p, 1, cs.p.p, cs.pb.p);
    }
    ProfScope psC(ctx, "U_correction", (double)N * (24.0 + 16.0 + 48.0 + 24.0) + F * 40.0);
    k_phi_update<<<nblocks(std::max(F, NB)), RT_BLOCK, 0, s>>>(m, phiHbyA, phiHbyAb, pu, pIntC, pBouC, cs.p.p,
                                                                cs.phi.p, cs.phib.p);
    double *gp2 = W.take(3 * (size_t)N);
    grad_field(ctx, 1, cs.p.p, cs.pb.p, gp2);
    k_U_correct<<<gN, RT_BLOCK, 0, s>>>(N, HbyA, rAU, rAtU, gp, gp2, cs.U.p);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 2);
    correct_bc(ctx, cs.bkU.p, 3, cs.U.p, cs.Ub.p);
    prof_end(ctx, psC.rec, psC.bytes);
    psC.rec = -1;
    perf->contErrSumLocal = 0.0;
    perf->contErrGlobal = 0.0;

    // ---------------- constEq.correct() ----------------
    return modes_correct(ctx, nullptr, perf->theta, theta0);
}

// D = r (x - xs) - psi D (when `roll`), then xs = x
__global__ void k_ddt_roll(size_t n, int roll, double r, double psi, const double *__restrict__ x,
                           double *__restrict__ xs, double *__restrict__ D) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (roll) D[i] = r * (x[i] - xs[i]) - psi * D[i];
    xs[i] = x[i];
}

// Crank-Nicolson, restated from the time-integration method: the trapezoidal
// rule with the stored old-time derivative D, (c/dt)(x - x_n) - psi D_n =
// f(x), c = 1 + psi (psi the off-centering coefficient), D_n = c_{n-1}(x_n -
// x_{n-1})/dt - psi D_{n-1}; the first step is implicit Euler (c = 1, D_0 =
// 0).  At the start of a step, D of the step that ended is formed from the
// fields now and at that step's start, and the start fields are taken.
void ddt_begin_step(rt_ctx *ctx, bool flow) {
    DevCase &cs = ctx->cs;
    if (cs.ctl.ddtScheme != RT_DDT_CRANKNICOLSON) return;
    const DevMesh &mesh = ctx->mesh;
    const size_t N = mesh.N, F = mesh.F, NB = mesh.NB;
    const double rDt = 1.0 / cs.ctl.deltaT, psi = cs.ctl.ddtPsi;
    auto coef = [&](int j) { return j == 0 ? 1.0 : 1.0 + psi; };
    cudaStream_t s = ctx->stream;
    auto roll = [&](size_t n, int doRoll, double r, const double *x, double *xs, double *D) {
        if (!n) return;
        k_ddt_roll<<<nblocks((long long)n), RT_BLOCK, 0, s>>>(n, doRoll, r, psi, x, xs, D);
        RT_CHECK_LAUNCH();
        launch_count(ctx);
    };
    if (flow) {
        const double r = cs.ddtSteps >= 1 ? coef(cs.ddtSteps - 1) * rDt : 0.0;
        roll(3 * N, cs.ddtSteps >= 1, r, cs.U.p, cs.Us.p, cs.DU.p);
        roll(3 * NB, cs.ddtSteps >= 1, r, cs.Ub.p, cs.Ubs.p, cs.DUb.p);
        roll(F, cs.ddtSteps >= 1, r, cs.phi.p, cs.phis.p, cs.Dphi.p);
        roll(NB, cs.ddtSteps >= 1, r, cs.phib.p, cs.phibs.p, cs.Dphib.p);
        ++cs.ddtSteps;
        cs.ddtC = coef(cs.ddtSteps - 1);
    }
    const double rt = cs.ddtThSteps >= 1 ? coef(cs.ddtThSteps - 1) * rDt : 0.0;
    for (int i = 0; i < cs.nModes; ++i) {
        ModeSwap sw(cs, i > 0 ? cs.modes[i - 1].get() : nullptr);
        roll(6 * N, cs.ddtThSteps >= 1, rt, cs.theta.p, cs.ths.p, cs.Dth.p);
    }
    ++cs.ddtThSteps;
    cs.ddtCth = coef(cs.ddtThSteps - 1);
}

// one time step: nInIter inner iterations (rheoFoam.C:96-150; 0 means 1)
// on the old-time fields taken at its start
rt_status step_once(rt_ctx *ctx, rt_step_perf *perf) {
    DevMesh &mesh = ctx->mesh;
    DevCase &cs = ctx->cs;
    const int N = mesh.N, F = mesh.F, NB = mesh.NB;
    cudaStream_t s = ctx->stream;
    Work &W = ctx->work;
    WorkMark wmark(W);
    const int nIn = cs.ctl.nInIter > 1 ? cs.ctl.nInIter : 1;
    ddt_begin_step(ctx, true);
    double *U0 = W.take(3 * (size_t)N), *U0b = W.take(3 * (size_t)NB), *phi0 = W.take(F), *phi0b = W.take(NB);
    RT_CUDA(cudaMemcpyAsync(U0, cs.U.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
    if (NB) RT_CUDA(cudaMemcpyAsync(U0b, cs.Ub.p, sizeof(double) * 3 * NB, cudaMemcpyDeviceToDevice, s));
    if (F) RT_CUDA(cudaMemcpyAsync(phi0, cs.phi.p, sizeof(double) * F, cudaMemcpyDeviceToDevice, s));
    if (NB) RT_CUDA(cudaMemcpyAsync(phi0b, cs.phib.p, sizeof(double) * NB, cudaMemcpyDeviceToDevice, s));
    double *theta0 = nullptr;
    if (nIn > 1 && cs.nModes > 1) {
        // every mode's theta at the start of the step
        const size_t n6 = 6 * (size_t)N;
        cs.thetaStep0.alloc(n6 * cs.nModes);
        theta0 = cs.thetaStep0.p;
        for (int i = 0; i < cs.nModes; ++i)
            RT_CUDA(cudaMemcpyAsync(theta0 + n6 * i, i ? cs.modes[i - 1]->theta.p : cs.theta.p, sizeof(double) * n6,
                                    cudaMemcpyDeviceToDevice, s));
    } else if (nIn > 1) {
        theta0 = W.take(6 * (size_t)N);
        RT_CUDA(cudaMemcpyAsync(theta0, cs.theta.p, sizeof(double) * 6 * N, cudaMemcpyDeviceToDevice, s));
    }
    rt_status st = RT_OK;
    for (int it = 0; it < nIn && st == RT_OK; ++it) {
        *perf = rt_step_perf{};
        st = step_inner(ctx, perf, U0, U0b, phi0, phi0b, theta0);
    }
    return st;
}

}  // namespace rt
