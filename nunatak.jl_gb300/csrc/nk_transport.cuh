// nk_transport.cuh — the face reconstructions of the thickness transport, shared by the forward stage
// (nk_coefficients.cu) and its reverse (nk_time_adjoint.cu).
#pragma once

#include "nk_kernels.cuh"

namespace nk {

// The face thickness that u H carries through a face (UpwindBiased(order = 1 or 3) and WENO(order = 5) of the
// reference's advection, restated from their published algorithms).  s[m + 2], m = -2..2, is the stage thickness m
// cells from the upwind cell s[2] of the face, m > 0 towards and past the face.  A periodic stencil wraps as often as
// the grid is short; a Bounded one takes the edge cell (the zero-gradient halo).
__device__ __forceinline__ int wide_map(int i, int n, int periodic) {
    if (periodic) { int r = i % n; return r < 0 ? r + n : r; }
    return i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
}
__device__ __forceinline__ void stencil_x(const DevGrid<double>& g, const double* __restrict__ H, int f, int j, bool east, double* s) {
    int row = wide_map(j, g.Ny, g.py) * g.pitch;
#pragma unroll
    for (int m = -2; m <= 2; ++m) s[m + 2] = H[row + wide_map(east ? f - 1 + m : f - m, g.Nx, g.px)];
}
__device__ __forceinline__ void stencil_y(const DevGrid<double>& g, const double* __restrict__ H, int i, int f, bool north, double* s) {
    int col = wide_map(i, g.Nx, g.px);
#pragma unroll
    for (int m = -2; m <= 2; ++m) s[m + 2] = H[wide_map(north ? f - 1 + m : f - m, g.Ny, g.py) * g.pitch + col];
}
// WENO-5: the three third-order candidates, their Jiang-Shu smoothness indicators and the WENO-Z weights
// α_k = d_k (1 + τ / (β_k + ε)), τ = |β₀ - β₂|, ε = 1e-8, d = (1, 6, 3) / 10 (Jiang and Shu 1996; Borges et al. 2008,
// exponent 1).
__device__ __forceinline__ double weno5_face(const double* s) {
    const double a = s[0], b = s[1], c = s[2], d = s[3], e = s[4];
    const double sixth = 1.0 / 6;
    double q0 = (2 * a - 7 * b + 11 * c) * sixth;
    double q1 = (-b + 5 * c + 2 * d) * sixth;
    double q2 = (2 * c + 5 * d - e) * sixth;
    double b0 = 13.0 / 12 * (a - 2 * b + c) * (a - 2 * b + c) + 0.25 * (a - 4 * b + 3 * c) * (a - 4 * b + 3 * c);
    double b1 = 13.0 / 12 * (b - 2 * c + d) * (b - 2 * c + d) + 0.25 * (b - d) * (b - d);
    double b2 = 13.0 / 12 * (c - 2 * d + e) * (c - 2 * d + e) + 0.25 * (3 * c - 4 * d + e) * (3 * c - 4 * d + e);
    const double eps = 1e-8;
    double tau = fabs(b0 - b2);
    // αₖ = dₖ (1 + τ / (βₖ + ε)) over the common denominator Π(βₖ + ε): one FP64 division per face instead of four
    // (the weights' ratio is unchanged; the rounding differs from the separate quotients in the last bits)
    double e0 = b0 + eps, e1 = b1 + eps, e2 = b2 + eps;
    double a0 = 0.1 * (e0 + tau) * (e1 * e2), a1 = 0.6 * (e1 + tau) * (e0 * e2), a2 = 0.3 * (e2 + tau) * (e0 * e1);
    return (a0 * q0 + a1 * q1 + a2 * q2) / (a0 + a1 + a2);
}
__device__ __forceinline__ double face_value(const ThicknessView& v, const double* s) {
    if (v.scheme == NK_ADVECTION_WENO) return weno5_face(s);
    return v.order == 3 ? (-s[1] + 5 * s[2] + 2 * s[3]) / 6 : s[2];
}


// ∂(face value)/∂s[m], m = 0..4, of the reconstructions above, for the reverse of the stage.  WENO-5 by the chain rule
// through its candidates qₖ, smoothness indicators βₖ and weights: with αₖ = dₖ (1 + τ / (βₖ + ε)), S = Σ αₖ and
// q = Σ αₖ qₖ / S, ∂q = Σ (αₖ ∂qₖ + (qₖ - q) ∂αₖ) / S, ∂αₖ = dₖ (∂τ / (βₖ + ε) - τ ∂βₖ / (βₖ + ε)²) and
// ∂τ = sign(β₀ - β₂) (∂β₀ - ∂β₂).
__device__ __forceinline__ void weno5_face_gradient(const double* s, double* J) {
    const double a = s[0], b = s[1], c = s[2], d = s[3], e = s[4];
    const double sixth = 1.0 / 6;
    const double q[3] = {(2 * a - 7 * b + 11 * c) * sixth, (-b + 5 * c + 2 * d) * sixth, (2 * c + 5 * d - e) * sixth};
    const double dq[3][5] = {{2 * sixth, -7 * sixth, 11 * sixth, 0, 0}, {0, -sixth, 5 * sixth, 2 * sixth, 0},
                             {0, 0, 2 * sixth, 5 * sixth, -sixth}};
    const double A0 = a - 2 * b + c, B0 = a - 4 * b + 3 * c;
    const double A1 = b - 2 * c + d, B1 = b - d;
    const double A2 = c - 2 * d + e, B2 = 3 * c - 4 * d + e;
    const double beta[3] = {13.0 / 12 * A0 * A0 + 0.25 * B0 * B0, 13.0 / 12 * A1 * A1 + 0.25 * B1 * B1,
                            13.0 / 12 * A2 * A2 + 0.25 * B2 * B2};
    const double k13 = 13.0 / 6;
    const double db[3][5] = {{k13 * A0 + 0.5 * B0, -2 * k13 * A0 - 2 * B0, k13 * A0 + 1.5 * B0, 0, 0},
                             {0, k13 * A1 + 0.5 * B1, -2 * k13 * A1, k13 * A1 - 0.5 * B1, 0},
                             {0, 0, k13 * A2 + 1.5 * B2, -2 * k13 * A2 - 2 * B2, k13 * A2 + 0.5 * B2}};
    const double eps = 1e-8, dk[3] = {0.1, 0.6, 0.3};
    const double tau = fabs(beta[0] - beta[2]), sg = beta[0] >= beta[2] ? 1.0 : -1.0;
    double al[3], S = 0, num = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        al[k] = dk[k] * (1 + tau / (beta[k] + eps));
        S += al[k];
        num += al[k] * q[k];
    }
    const double val = num / S, rS = 1 / S;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        const double dtau = sg * (db[0][m] - db[2][m]);
        double acc = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double ek = beta[k] + eps;
            const double dal = dk[k] * (dtau / ek - tau * db[k][m] / (ek * ek));
            acc += al[k] * dq[k][m] + (q[k] - val) * dal;
        }
        J[m] = acc * rS;
    }
}
__device__ __forceinline__ void face_value_gradient(const ThicknessView& v, const double* s, double* J) {
    if (v.scheme == NK_ADVECTION_WENO) { weno5_face_gradient(s, J); return; }
    const double third[5] = {0, -1.0 / 6, 5.0 / 6, 2.0 / 6, 0}, first[5] = {0, 0, 1, 0, 0};
#pragma unroll
    for (int m = 0; m < 5; ++m) J[m] = v.order == 3 ? third[m] : first[m];
}

}  // namespace nk
