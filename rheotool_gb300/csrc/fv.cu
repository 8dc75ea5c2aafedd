// fv.cu — finite-volume operators on the device: Gauss linear gradients and
// the GaussDefCmpw convection scheme (upwind implicit part + deferred
// high-resolution correction, rheoTool gaussDefCmpwConvectionScheme.C:72-328).
#include "fv_device.cuh"
#include "fv_ops.h"

namespace rt {

// ---------------------------------------------------------------------------
// gradient of NC components: g[(d*NC + k)*N + c] = d/dx_d of component k
// ---------------------------------------------------------------------------
template <int NC>
__global__ void k_grad(MeshView m, const double *__restrict__ x, const double *__restrict__ xb,
                       double *__restrict__ g) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    double a[NC][3];
#pragma unroll
    for (int k = 0; k < NC; ++k) a[k][0] = a[k][1] = a[k][2] = 0.0;
    for (int s = 0; s < m.nSlots; ++s) {
        int nb = m.ellNbr[s * m.N + c];
        if (nb < 0) break;
        int f = m.ellFace[s * m.N + c];
        bool own = nb > c;
        int o = own ? c : nb, n = own ? nb : c;
        double wf = m.w[f];
        double S0 = m.Sf[f], S1 = m.Sf[m.F + f], S2 = m.Sf[2 * m.F + f];
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            double xf = lin_interp(wf, x[(size_t)k * m.N + o], x[(size_t)k * m.N + n]);
            double s0 = S0 * xf, s1 = S1 * xf, s2 = S2 * xf;
            if (own) { a[k][0] += s0; a[k][1] += s1; a[k][2] += s2; }
            else     { a[k][0] -= s0; a[k][1] -= s1; a[k][2] -= s2; }
        }
    }
    for (int i = m.bStart[c]; i < m.bStart[c + 1]; ++i) {
        int b = m.bList[i];
        double S0 = m.bSf[b], S1 = m.bSf[m.NB + b], S2 = m.bSf[2 * m.NB + b];
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            double xf = xb[(size_t)k * m.NB + b];
            a[k][0] += S0 * xf; a[k][1] += S1 * xf; a[k][2] += S2 * xf;
        }
    }
    double v = m.V[c];
#pragma unroll
    for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) g[((size_t)d * NC + k) * m.N + c] = a[k][d] / v;
}

void grad_field(rt_ctx *ctx, int nc, const double *x, const double *xb, double *g) {
    MeshView m = view(ctx->mesh);
    int nb = nblocks(m.N);
    switch (nc) {
    case 1: k_grad<1><<<nb, RT_BLOCK, 0, ctx->stream>>>(m, x, xb, g); break;
    case 3: k_grad<3><<<nb, RT_BLOCK, 0, ctx->stream>>>(m, x, xb, g); break;
    case 6: k_grad<6><<<nb, RT_BLOCK, 0, ctx->stream>>>(m, x, xb, g); break;
    default: throw Error{RT_EINVAL, "grad_field: nc must be 1, 3 or 6"};
    }
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

void grad_scalar(rt_ctx *ctx, const double *x, const double *xb, double *g) {
    grad_field(ctx, 1, x, xb, g);
}

// ---------------------------------------------------------------------------
// GaussDefCmpw
// ---------------------------------------------------------------------------
// face pass: upwind coefficients and, per component, the deferred-correction
// flux phi_f (psi_f^HR - psi_f^UD)
template <int NC>
__global__ void k_defc_face(MeshView m, Lims L, int hr, const double *__restrict__ phi,
                            const double *__restrict__ x, const double *__restrict__ g,
                            double *__restrict__ lower, double *__restrict__ upper,
                            double *__restrict__ flux) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.F) return;
    const int N = m.N;
    double ph = phi[f];
    double u = ph >= 0.0 ? 1.0 : 0.0;
    lower[f] = -u * ph;
    upper[f] = (1.0 - u) * ph;
    if (!hr) return;
    int o = m.owner[f], n = m.neighbour[f];
    double d0 = m.d[f], d1 = m.d[m.F + f], d2 = m.d[2 * m.F + f];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        double go0 = g[((size_t)0 * NC + k) * N + o], go1 = g[((size_t)1 * NC + k) * N + o],
               go2 = g[((size_t)2 * NC + k) * N + o];
        double gn0 = g[((size_t)0 * NC + k) * N + n], gn1 = g[((size_t)1 * NC + k) * N + n],
               gn2 = g[((size_t)2 * NC + k) * N + n];
        double gu0 = go0 * u + (1.0 - u) * gn0, gu1 = go1 * u + (1.0 - u) * gn1,
               gu2 = go2 * u + (1.0 - u) * gn2;
        double gud = gu0 * d0 + gu1 * d1 + gu2 * d2;
        double xo = x[(size_t)k * N + o], xn = x[(size_t)k * N + n];
        double phitc = 1.0 - (xn - xo) / (2.0 * gud + 1e-18);
        double a, bb;
        if (phitc <= 0.0 || phitc >= 1.0) { a = 1.0; bb = 0.0; }
        else if (phitc < L.bl[0]) { a = L.al[0]; bb = L.be[0]; }
        else if (phitc < L.bl[1]) { a = L.al[1]; bb = L.be[1]; }
        else { a = L.al[2]; bb = L.be[2]; }
        double god = go0 * d0 + go1 * d1 + go2 * d2;
        double gnd = gn0 * d0 + gn1 * d1 + gn2 * d2;
        double tf = (1.0 - a - bb) * (xn - 2.0 * god) * u
                  + (1.0 - a - bb) * (xo + 2.0 * gnd) * (1.0 - u)
                  + ((a - 1.0) * u + bb * (1.0 - u)) * xo
                  + (bb * u + (a - 1.0) * (1.0 - u)) * xn;
        flux[(size_t)k * m.F + f] = tf * ph;
    }
}

// cell pass: negSumDiag of the upwind part and source = -sum(+-flux)
template <int NC>
__global__ void k_defc_cell(MeshView m, int hr, const double *__restrict__ lower,
                            const double *__restrict__ upper, const double *__restrict__ flux,
                            double *__restrict__ diagC, double *__restrict__ srcC) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    double dg = 0.0;
    double sou[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) sou[k] = 0.0;
    for (int s = 0; s < m.nSlots; ++s) {
        int nb = m.ellNbr[s * m.N + c];
        if (nb < 0) break;
        int f = m.ellFace[s * m.N + c];
        bool own = nb > c;
        dg -= own ? lower[f] : upper[f];
        if (hr) {
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                double fl = flux[(size_t)k * m.F + f];
                if (own) sou[k] += fl; else sou[k] -= fl;
            }
        }
    }
    diagC[c] = dg;
#pragma unroll
    for (int k = 0; k < NC; ++k) srcC[(size_t)k * m.N + c] = -sou[k];
}

// boundary coefficients of the upwind part: fixedValue -> (0, -phi_b psi_b),
// zeroGradient -> (phi_b, 0)
__global__ void k_defc_bnd(int NB, int nc, const double *__restrict__ phib, const int *__restrict__ kind,
                           const double *__restrict__ xb, double *__restrict__ intC,
                           double *__restrict__ bouC) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= NB) return;
    double ph = phib[b];
    bool zg = kind[b] == RT_BC_ZEROGRAD;
    for (int k = 0; k < nc; ++k) {
        intC[(size_t)k * NB + b] = zg ? ph * 1.0 : ph * 0.0;
        bouC[(size_t)k * NB + b] = zg ? -ph * 0.0 : -ph * xb[(size_t)k * NB + b];
    }
}

void convection(rt_ctx *ctx, int scheme, int nc, const double *phi, const double *phib,
                const double *x, const double *xb, const int *bkind, const double *g,
                double *lower, double *upper, double *diagC, double *srcC, double *intC,
                double *bouC, double *fluxTmp) {
    MeshView m = view(ctx->mesh);
    Lims L = make_lims(scheme);
    int hr = (scheme != RT_LIM_UPWIND && scheme != RT_LIM_NONE) ? 1 : 0;
    cudaStream_t s = ctx->stream;
    if (nc == 3) {
        k_defc_face<3><<<nblocks(m.F), RT_BLOCK, 0, s>>>(m, L, hr, phi, x, g, lower, upper, fluxTmp);
        k_defc_cell<3><<<nblocks(m.N), RT_BLOCK, 0, s>>>(m, hr, lower, upper, fluxTmp, diagC, srcC);
    } else if (nc == 6) {
        k_defc_face<6><<<nblocks(m.F), RT_BLOCK, 0, s>>>(m, L, hr, phi, x, g, lower, upper, fluxTmp);
        k_defc_cell<6><<<nblocks(m.N), RT_BLOCK, 0, s>>>(m, hr, lower, upper, fluxTmp, diagC, srcC);
    } else {
        throw Error{RT_EINVAL, "convection: nc must be 3 or 6"};
    }
    k_defc_bnd<<<nblocks(m.NB), RT_BLOCK, 0, s>>>(m.NB, nc, phib, bkind, xb, intC, bouC);
    RT_CHECK_LAUNCH();
    launch_count(ctx, 3);
}

// zeroGradient boundary values = cell values
__global__ void k_correct_bc(int NB, int N, int nc, const int *__restrict__ bCell,
                             const int *__restrict__ kind, const double *__restrict__ x,
                             double *__restrict__ xb) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= NB) return;
    if (kind[b] != RT_BC_ZEROGRAD) return;
    int c = bCell[b];
    for (int k = 0; k < nc; ++k) xb[(size_t)k * NB + b] = x[(size_t)k * N + c];
}

void correct_bc(rt_ctx *ctx, const int *kind, int nc, const double *x, double *xb) {
    const DevMesh &m = ctx->mesh;
    if (m.NB == 0) return;
    k_correct_bc<<<nblocks(m.NB), RT_BLOCK, 0, ctx->stream>>>(m.NB, m.N, nc, m.bCell.p, kind, x, xb);
    RT_CHECK_LAUNCH();
    launch_count(ctx);
}

}  // namespace rt
