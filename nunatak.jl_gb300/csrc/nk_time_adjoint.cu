// nk_time_adjoint.cu — the reverse of one thickness stage, for the gradient through time steps.
//
// The forward stage (k_thickness_faces, k_thickness_limiter, k_thickness_stage in nk_coefficients.cu) is
//   H = max(0, H⁻ + Δτ (S - ∇⋅F(Hs, u))),  S = a - (1 - φ(Hs)) w m  on full cells,
// with F the face fluxes u H_face, H_face the scheme's upwind-biased reconstruction of Hs, limited for a bounded
// WENO by the upwind cell's θ (H̄ + θ (H_face - H̄)).  Its reverse runs as four gathers, each thread owning one cell or
// one face, so no two threads add into one value and the result does not depend on the order of the launch:
//   cells    the clip, the sources and the divergence: λ★ = [H > 0] λ, λH⁻ += λ★, λa += Δτ λ★, λm -= Δτ λ★ (1 - φ) w;
//   faces    λF = λ of each face flux, from the divergence of its two cells, and λu += Δy H_face λF;
//   limiter  per cell, the faces it is upwind of: λHs += (1 - θ) Δy u λF, λθ += (H_face - H̄) Δy u λF, then θ's own
//            derivative back to H̄ and to the cell's four reconstructions;
//   stencils per cell, every reconstruction whose stencil holds it (∂H_face/∂s by face_value_gradient) and every
//            centre grounded fraction that reads its flotation.
// Wherever the forward takes a min, a max or a clip, the reverse follows the branch the forward took.
#include <cmath>

#include "nk_kernels.cuh"
#include "nk_transport.cuh"

namespace nk {

__device__ __forceinline__ bool stage_full(const ThicknessView& v, int k) { return !v.mu || v.mu[k] > 0; }

// ---- cells: the clip, the sources, the divergence ----------------------------------------------------------------
__global__ void k_stage_adjoint_cells(StageAdjointView a) {
    const ThicknessView& v = a.t;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    double ls = a.Hout[c] > 0 ? a.lam_out[c] : 0.0;   // λ★
    a.lam_H0[c] += ls;
    a.dv[c] = -a.dtau * ls / g.Az_cc(i, j);
    double lp = 0.0;
    if (stage_full(v, c)) {
        double lS = a.dtau * ls;
        a.lam_smb[c] += lS;
        a.lam_melt[c] -= lS * (v.grounding ? 1 - v.phi[c] : 1.0) * a.melt_weight;
        if (v.grounding) lp = lS * v.melt[c];   // ∂S/∂φ = w m
    }
    a.lam_phi[c] = lp + (a.lam_phi_in ? a.lam_phi_in[c] : 0.0);
}

// The limited face thickness of a flux between two full cells (as k_thickness_stage evaluates it).
__device__ __forceinline__ double limited_face(const ThicknessView& v, double h0, int k) {
    const bool bounded = v.scheme == NK_ADVECTION_WENO && v.bounded;
    return bounded ? v.Hs[k] + v.theta[k] * (h0 - v.Hs[k]) : h0;
}

// ---- faces: λ of each flux, and the velocity adjoint ---------------------------------------------------------------
__global__ void k_stage_adjoint_faces(StageAdjointView a) {
    const ThicknessView& v = a.t;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    double2 lf = make_double2(0.0, 0.0);
    double2 lx = a.lam_x[k];
    const double* __restrict__ Hs = v.Hs;
    double s[5];
    // x face (i, j); on a periodic axis face Nx is face 0 and is done there
    if (j < g.Ny && (i < g.Nx || !g.px) && !g.peripheral_fc(i, j)) {
        int kw = g.c_idx(i - 1, j), ke = g.c_idx(i, j);
        double F = a.dv[kw] - a.dv[ke];
        double u = v.x[k].x, h;
        bool w = stage_full(v, kw), e = stage_full(v, ke);
        if (!(w && e)) {
            h = w ? (u > 0 ? Hs[kw] : 0.0) : (e ? (u < 0 ? Hs[ke] : 0.0) : 0.0);
        } else {
            bool east = u > 0;
            double h0;
            if (v.fx) {
                double2 r = v.fx[k];
                h0 = east ? r.x : r.y;
            } else {
                stencil_x(g, Hs, i, j, east, s);
                h0 = face_value(v, s);
            }
            h = limited_face(v, h0, east ? kw : ke);
        }
        lx.x += g.dyc[j] * h * F;
        lf.x = F;
    }
    if (i < g.Nx && (j < g.Ny || !g.py) && !g.peripheral_cf(i, j)) {
        int ks = g.c_idx(i, j - 1), kn = g.c_idx(i, j);
        double F = a.dv[ks] - a.dv[kn];
        double w = v.x[k].y, h;
        bool so = stage_full(v, ks), no = stage_full(v, kn);
        if (!(so && no)) {
            h = so ? (w > 0 ? Hs[ks] : 0.0) : (no ? (w < 0 ? Hs[kn] : 0.0) : 0.0);
        } else {
            bool north = w > 0;
            double h0;
            if (v.fy) {
                double2 r = v.fy[k];
                h0 = north ? r.x : r.y;
            } else {
                stencil_y(g, Hs, i, j, north, s);
                h0 = face_value(v, s);
            }
            h = limited_face(v, h0, north ? ks : kn);
        }
        lx.y += g.dxc[i] * h * F;
        lf.y = F;
    }
    a.lamF[k] = lf;
    a.lam_x[k] = lx;
}

// ---- limiter: the direct terms of the upwind cell, θ's derivative --------------------------------------------------
__global__ void k_stage_adjoint_limiter(StageAdjointView a) {
    const ThicknessView& v = a.t;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    const bool bounded = v.scheme == NK_ADVECTION_WENO && v.bounded;
    int c = g.idx(i, j);
    const double Hc = v.Hs[c];
    const double th = bounded ? v.theta[c] : 1.0;
    double lam = 0.0, lt = 0.0;
    // one face of the cell: q = Δ λF; `low` when the cell is the face's west (south) neighbour, upwind for u > 0
    auto face = [&](double F, double u, double q, int klo, int khi, bool low, const double2* rec, int kf) {
        if (F == 0.0) return;
        bool flo = stage_full(v, klo), fhi = stage_full(v, khi);
        if (!(flo && fhi)) {   // a front flux reads the full side's thickness
            if (low && flo) lam += fmax(u, 0.0) * q;
            if (!low && fhi && !flo) lam += fmin(u, 0.0) * q;
            return;
        }
        bool pos = u > 0;
        if (pos != low || !bounded) return;   // unbounded: the face value's whole adjoint goes through its stencil
        double lh = u * q;
        double2 r = rec[kf];
        lam += (1 - th) * lh;
        lt += ((pos ? r.x : r.y) - Hc) * lh;
    };
    if (!g.peripheral_fc(i + 1, j)) {
        int kf = g.u_idx(i + 1, j);
        face(a.lamF[kf].x, v.x[kf].x, g.dyc[j] * a.lamF[kf].x, c, g.c_idx(i + 1, j), true, v.fx, kf);
    }
    if (!g.peripheral_fc(i, j)) {
        int kf = g.u_idx(i, j);
        face(a.lamF[kf].x, v.x[kf].x, g.dyc[j] * a.lamF[kf].x, g.c_idx(i - 1, j), c, false, v.fx, kf);
    }
    if (!g.peripheral_cf(i, j + 1)) {
        int kf = g.v_idx(i, j + 1);
        face(a.lamF[kf].y, v.x[kf].y, g.dxc[i] * a.lamF[kf].y, c, g.c_idx(i, j + 1), true, v.fy, kf);
    }
    if (!g.peripheral_cf(i, j)) {
        int kf = g.v_idx(i, j);
        face(a.lamF[kf].y, v.x[kf].y, g.dxc[i] * a.lamF[kf].y, g.c_idx(i, j - 1), c, false, v.fy, kf);
    }
    double2 lwx = make_double2(0.0, 0.0), lwy = make_double2(0.0, 0.0);
    if (bounded && lt != 0.0) {
        // θ = min(1, |(upper - H̄) / (M - H̄ + ε)|, |(lower - H̄) / (m - H̄ - ε)|) of k_thickness_limiter
        double E = v.fx[g.idx(i + 1, j)].x, W = v.fx[g.idx(i, j)].y;
        double N = v.fy[g.idx(i, j + 1)].x, S = v.fy[g.idx(i, j)].y;
        const double w = 5.0 / 18, eps = 2 * 2.220446049250313e-16, r12 = 1 / (1 - 2 * w);
        double px = (Hc - w * W - w * E) / (1 - 2 * w);
        double py = (Hc - w * S - w * N) / (1 - 2 * w);
        const double val[6] = {px, py, W, E, S, N};
        double M = fmax(fmax(fmax(px, py), fmax(W, E)), fmax(S, N));
        double m = fmin(fmin(fmin(px, py), fmin(W, E)), fmin(S, N));
        double a1 = v.upper - Hc, b1 = M - Hc + eps, a2 = v.lower - Hc, b2 = m - Hc - eps;
        double t1 = fabs(a1 / b1), t2 = fabs(a2 / b2);
        double lHc = 0.0, lext = 0.0;
        int arg = -1;
        if (t1 < 1.0 || t2 < 1.0) {
            bool first = t1 <= t2;
            double an = first ? a1 : a2, bn = first ? b1 : b2;
            double sg = an / bn >= 0 ? 1.0 : -1.0;
            // r = an / bn with ∂an/∂H̄ = -1, ∂bn/∂H̄ = -1, ∂bn/∂(M or m) = 1
            lHc = lt * sg * (an - bn) / (bn * bn);
            lext = lt * sg * (-an / (bn * bn));
            double ext = first ? M : m;
            for (int q = 0; q < 6; ++q)
                if (val[q] == ext) { arg = q; break; }
        }
        double lW = 0.0, lE = 0.0, lS = 0.0, lN = 0.0;
        switch (arg) {
            case 0: lHc += lext * r12; lW -= lext * w * r12; lE -= lext * w * r12; break;
            case 1: lHc += lext * r12; lS -= lext * w * r12; lN -= lext * w * r12; break;
            case 2: lW += lext; break;
            case 3: lE += lext; break;
            case 4: lS += lext; break;
            case 5: lN += lext; break;
            default: break;
        }
        lam += lHc;
        lwx = make_double2(lW, lE);
        lwy = make_double2(lS, lN);
    }
    if (bounded) {
        a.lw_x[c] = lwx;
        a.lw_y[c] = lwy;
    }
    a.lam_Hs[c] = lam;
}

// ---- stencils: the reconstructions and the centre grounded fractions -----------------------------------------------
// λ of x face f's two reconstructions (.x from cell f-1, flow east; .y from cell f, flow west): through the flux it
// carries (between full cells) and through the limiters of the two cells whose own face value it is.
__device__ __forceinline__ double2 recon_adjoint_x(const StageAdjointView& a, int f, int j) {
    const ThicknessView& v = a.t;
    const DevGrid<double>& g = v.g;
    const bool bounded = v.scheme == NK_ADVECTION_WENO && v.bounded;
    double2 r = make_double2(0.0, 0.0);
    if (!g.peripheral_fc(f, j)) {
        int kf = g.u_idx(f, j);
        double F = a.lamF[kf].x;
        int kw = g.c_idx(f - 1, j), ke = g.c_idx(f, j);
        if (F != 0.0 && stage_full(v, kw) && stage_full(v, ke)) {
            double u = v.x[kf].x;
            bool east = u > 0;
            double lh = g.dyc[j] * u * F * (bounded ? v.theta[east ? kw : ke] : 1.0);
            if (east) r.x += lh; else r.y += lh;
        }
    }
    if (bounded) {
        if (g.px || f >= 1) r.x += a.lw_x[g.c_idx(f - 1, j)].y;      // E of cell f - 1
        if (g.px || f < g.Nx) r.y += a.lw_x[g.c_idx(f, j)].x;        // W of cell f
    }
    return r;
}
__device__ __forceinline__ double2 recon_adjoint_y(const StageAdjointView& a, int i, int f) {
    const ThicknessView& v = a.t;
    const DevGrid<double>& g = v.g;
    const bool bounded = v.scheme == NK_ADVECTION_WENO && v.bounded;
    double2 r = make_double2(0.0, 0.0);
    if (!g.peripheral_cf(i, f)) {
        int kf = g.v_idx(i, f);
        double F = a.lamF[kf].y;
        int ks = g.c_idx(i, f - 1), kn = g.c_idx(i, f);
        if (F != 0.0 && stage_full(v, ks) && stage_full(v, kn)) {
            double w = v.x[kf].y;
            bool north = w > 0;
            double lh = g.dxc[i] * w * F * (bounded ? v.theta[north ? ks : kn] : 1.0);
            if (north) r.x += lh; else r.y += lh;
        }
    }
    if (bounded) {
        if (g.py || f >= 1) r.x += a.lw_y[g.c_idx(i, f - 1)].y;      // N of cell f - 1
        if (g.py || f < g.Ny) r.y += a.lw_y[g.c_idx(i, f)].x;        // S of cell f
    }
    return r;
}

// The distinct faces (x faces when `n` is Nx) whose five-cell stencils can hold cell `i`: i-3 .. i+3, within 0..n on
// a Bounded axis, wrapped on a Periodic one (every face when the axis is shorter than the seven).
struct FaceRange { int lo, hi; bool all; };
__device__ __forceinline__ FaceRange stencil_faces(int i, int n, int periodic) {
    if (periodic) return n <= 7 ? FaceRange{0, n - 1, true} : FaceRange{i - 3, i + 3, false};
    return FaceRange{i - 3 < 0 ? 0 : i - 3, i + 3 > n ? n : i + 3, false};
}

// ∂/∂(f1, f2, f3) of triangle_fraction (nk_coefficients.cu): one floating corner 1 - a² / ((b - a)(c - a)),
// one grounded corner c² / ((c - a)(c - b)), a ≤ b ≤ c the sorted flotations; zero when all three agree in sign.
__device__ __forceinline__ void triangle_fraction_partials(double f1, double f2, double f3, double* d) {
    d[0] = d[1] = d[2] = 0.0;
    double a = fmin(fmin(f1, f2), f3), c = fmax(fmax(f1, f2), f3);
    if (a >= 0 || c <= 0) return;
    double b = f1 + f2 + f3 - a - c;
    int ia = f1 == a ? 0 : (f2 == a ? 1 : 2);
    int ic = f1 == c ? 0 : (f2 == c ? 1 : 2);
    int ib = 3 - ia - ic;
    double da, db, dc;
    if (b > 0) {
        double D = (b - a) * (c - a);
        if (D == 0.0) return;
        double D2 = D * D;
        da = -(2 * a * D + a * a * ((c - a) + (b - a))) / D2;
        db = a * a * (c - a) / D2;
        dc = a * a * (b - a) / D2;
    } else {
        double D = (c - a) * (c - b);
        if (D == 0.0) return;
        double D2 = D * D;
        dc = (2 * c * D - c * c * ((c - b) + (c - a))) / D2;
        da = c * c * (c - b) / D2;
        db = c * c * (c - a) / D2;
    }
    d[ia] = da;
    d[ib] = db;
    d[ic] = dc;
}

// ∂φ/∂f of the centre grounded fraction of k_geometry over the 3 x 3 flotations f[x][y] around the centre (f[1][1]):
// φ = Σ of eight triangle fractions / 8, each of the centre, an edge midpoint (fc + f_nb) / 2 and a corner (the
// mean of four).
__device__ __forceinline__ void centre_fraction_partials(const double f[3][3], double dphi[3][3]) {
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = 0; y < 3; ++y) dphi[x][y] = 0.0;
    const double fc = f[1][1];
    // (edge neighbour, corner x, corner y) of the eight triangles: e, n, n, w, w, s, s, e with corners ne, ne, nw,
    // nw, sw, sw, se, se
    const int ex[8] = {2, 1, 1, 0, 0, 1, 1, 2}, ey[8] = {1, 2, 2, 1, 1, 0, 0, 1};
    const int cx[8] = {2, 2, 0, 0, 0, 0, 2, 2}, cy[8] = {2, 2, 2, 2, 0, 0, 0, 0};
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        double fe = (fc + f[ex[t]][ey[t]]) / 2;
        double fk = (fc + f[cx[t]][1] + f[1][cy[t]] + f[cx[t]][cy[t]]) / 4;
        double d[3];
        triangle_fraction_partials(fc, fe, fk, d);
        dphi[1][1] += d[0] / 8 + d[1] / 16 + d[2] / 32;
        dphi[ex[t]][ey[t]] += d[1] / 16;
        dphi[cx[t]][1] += d[2] / 32;
        dphi[1][cy[t]] += d[2] / 32;
        dphi[cx[t]][cy[t]] += d[2] / 32;
    }
}

__global__ void k_stage_adjoint_stencils(StageAdjointView a) {
    const ThicknessView& v = a.t;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    const double* __restrict__ Hs = v.Hs;
    double acc = 0.0, s[5], J[5];
    int cols[5];
    FaceRange fr = stencil_faces(i, g.Nx, g.px);
    int row = g.cy(j) * g.pitch;
    for (int q = fr.lo; q <= fr.hi; ++q) {
        int f = (g.px && !fr.all) ? wide_map(q, g.Nx, 1) : q;
        double2 r = recon_adjoint_x(a, f, j);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            double lr = side == 0 ? r.x : r.y;
            if (lr == 0.0) continue;
            bool hit = false;
#pragma unroll
            for (int m = -2; m <= 2; ++m) {
                cols[m + 2] = wide_map(side == 0 ? f - 1 + m : f - m, g.Nx, g.px);
                hit |= cols[m + 2] == i;
            }
            if (!hit) continue;
#pragma unroll
            for (int m = 0; m < 5; ++m) s[m] = Hs[row + cols[m]];
            face_value_gradient(v, s, J);
#pragma unroll
            for (int m = 0; m < 5; ++m)
                if (cols[m] == i) acc += J[m] * lr;
        }
    }
    fr = stencil_faces(j, g.Ny, g.py);
    int col = g.cx(i);
    for (int q = fr.lo; q <= fr.hi; ++q) {
        int f = (g.py && !fr.all) ? wide_map(q, g.Ny, 1) : q;
        double2 r = recon_adjoint_y(a, i, f);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            double lr = side == 0 ? r.x : r.y;
            if (lr == 0.0) continue;
            bool hit = false;
#pragma unroll
            for (int m = -2; m <= 2; ++m) {
                cols[m + 2] = wide_map(side == 0 ? f - 1 + m : f - m, g.Ny, g.py);
                hit |= cols[m + 2] == j;
            }
            if (!hit) continue;
#pragma unroll
            for (int m = 0; m < 5; ++m) s[m] = Hs[cols[m] * g.pitch + col];
            face_value_gradient(v, s, J);
#pragma unroll
            for (int m = 0; m < 5; ++m)
                if (cols[m] == j) acc += J[m] * lr;
        }
    }
    // the centre grounded fractions whose 3 x 3 flotations read this cell (φ of the melt source)
    if (v.grounding) {
        const int me = g.idx(i, j);
        auto range = [](int k, int n, int periodic, int& lo, int& hi, bool& all) {
            all = periodic && n < 3;
            if (all) { lo = 0; hi = n - 1; }
            else if (periodic) { lo = k - 1; hi = k + 1; }
            else { lo = k - 1 < 0 ? 0 : k - 1; hi = k + 1 > n - 1 ? n - 1 : k + 1; }
        };
        int xlo, xhi, ylo, yhi;
        bool xall, yall;
        range(i, g.Nx, g.px, xlo, xhi, xall);
        range(j, g.Ny, g.py, ylo, yhi, yall);
        for (int qy = ylo; qy <= yhi; ++qy) {
            int cj = (g.py && !yall) ? g.wrap(qy, g.Ny) : qy;
            for (int qx = xlo; qx <= xhi; ++qx) {
                int ci = (g.px && !xall) ? g.wrap(qx, g.Nx) : qx;
                double lp = a.lam_phi[g.idx(ci, cj)];
                if (lp == 0.0) continue;
                double f[3][3], d[3][3];
                int kk[3][3];
                bool hit = false;
#pragma unroll
                for (int x = 0; x < 3; ++x)
#pragma unroll
                    for (int y = 0; y < 3; ++y) {
                        int k = g.c_idx(ci + x - 1, cj + y - 1);
                        kk[x][y] = k;
                        f[x][y] = Hs[k] + a.rw_ri * a.bed[k];
                        hit |= k == me;
                    }
                if (!hit) continue;
                centre_fraction_partials(f, d);
#pragma unroll
                for (int x = 0; x < 3; ++x)
#pragma unroll
                    for (int y = 0; y < 3; ++y)
                        if (kk[x][y] == me) acc += lp * d[x][y];
            }
        }
    }
    a.lam_Hs[g.idx(i, j)] += acc;
}

void launch_stage_adjoint(const StageAdjointView& a, cudaStream_t s) {
    const DevGrid<double>& g = a.t.g;
    LaunchDims dc = dims2d(g.Nx, g.Ny), df = dims2d(g.Nx + 1, g.Ny + 1);
    k_stage_adjoint_cells<<<dc.grid, dc.block, 0, s>>>(a); count_launch();
    k_stage_adjoint_faces<<<df.grid, df.block, 0, s>>>(a); count_launch();
    k_stage_adjoint_limiter<<<dc.grid, dc.block, 0, s>>>(a); count_launch();
    k_stage_adjoint_stencils<<<dc.grid, dc.block, 0, s>>>(a); count_launch();
}

// ---- plane arithmetic of the reverse sweep -----------------------------------------------------------------------
__global__ void k_add_planes(DevGrid<double> g, double* y, const double* x, int planes, size_t plane) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    for (int p = 0; p < planes; ++p) y[p * plane + g.idx(i, j)] += x[p * plane + g.idx(i, j)];
}
void launch_add_planes(const DevGrid<double>& g, double* y, const double* x, int planes, size_t plane, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_add_planes<<<d.grid, d.block, 0, s>>>(g, y, x, planes, plane); count_launch();
}
__global__ void k_add_pairs(DevGrid<double> g, double2* y, const double2* x) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    double2 a = y[k], b = x[k];
    y[k] = make_double2(a.x + b.x, a.y + b.y);
}
void launch_add_pairs(const DevGrid<double>& g, double2* y, const double2* x, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx + 1, g.Ny + 1);
    k_add_pairs<<<d.grid, d.block, 0, s>>>(g, y, x); count_launch();
}
__global__ void k_scale_plane(DevGrid<double> g, double* y, const double* x, double a) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    y[g.idx(i, j)] = a * x[g.idx(i, j)];
}
void launch_scale_plane(const DevGrid<double>& g, double* y, const double* x, double a, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_scale_plane<<<d.grid, d.block, 0, s>>>(g, y, x, a); count_launch();
}

}  // namespace nk
