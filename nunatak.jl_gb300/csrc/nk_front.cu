// nk_front.cu — the partial-cell calving front (PartialCellFront, src/Models/partial_cell_front.jl) and its calving
// laws (src/Models/calving.jl) as one thread per cell.
//
// μ is the prognostic 0/1 flag of full cells and Hʳ the ice thickness of a partial front cell, which covers the
// fraction H / Hʳ of its area.  A neighbour outside a Bounded direction is inactive (never full, empty or a donor);
// a periodic neighbour wraps.  Every kernel writes only its own cell.  Where a kernel reads neighbours that another
// thread of the same launch may rewrite (the overflow passes), it reads a snapshot taken before the launch.
#include "nk_kernels.cuh"

namespace nk {

namespace {

// the four neighbours in the reference's order: west, east, south, north
__device__ __forceinline__ int DI(int d) { return d == 0 ? -1 : (d == 1 ? 1 : 0); }
__device__ __forceinline__ int DJ(int d) { return d == 2 ? -1 : (d == 3 ? 1 : 0); }

__device__ __forceinline__ bool inactive(const DevGrid<double>& g, int i, int j) { return g.out_x(i) || g.out_y(j); }
__device__ __forceinline__ bool full_at(const double* mu, int k) { return mu[k] > 0; }
// full_neighbor (:102): full and active
__device__ __forceinline__ bool full_neighbor(const DevGrid<double>& g, const double* mu, int i, int j) {
    return !inactive(g, i, j) && full_at(mu, g.c_idx(i, j));
}
// empty_cell (:103): not full, no ice, active
__device__ __forceinline__ bool empty_at(const DevGrid<double>& g, const double* mu, const double* H, int i, int j) {
    if (inactive(g, i, j)) return false;
    int k = g.c_idx(i, j);
    return !full_at(mu, k) && H[k] <= 0;
}

// interior_u / interior_v with the front's flag as the ice mask (strain_rates.jl:5-6, smooth_ice_mask.jl:72-73)
__device__ __forceinline__ double mu_u(const FrontView& v, int i, int j) {
    const DevGrid<double>& g = v.g;
    if (g.peripheral_fc(i, j) || (v.mu[g.c_idx(i - 1, j)] + v.mu[g.c_idx(i, j)]) == 0.0) return 0.0;
    return v.x[g.u_idx(i, j)].x;
}
__device__ __forceinline__ double mu_v(const FrontView& v, int i, int j) {
    const DevGrid<double>& g = v.g;
    if (g.peripheral_cf(i, j) || (v.mu[g.c_idx(i, j - 1)] + v.mu[g.c_idx(i, j)]) == 0.0) return 0.0;
    return v.x[g.v_idx(i, j)].y;
}
// strain_rate_xy with the flag as the mask (strain_rates.jl:14-17)
__device__ __forceinline__ double mu_strain_xy(const FrontView& v, int i, int j) {
    const DevGrid<double>& g = v.g;
    double dudy = (mu_u(v, i, j) - mu_u(v, i, j - 1)) / g.dyf[j];
    double dvdx = (mu_v(v, i, j) - mu_v(v, i - 1, j)) / g.dxf[i];
    double e = (dudy + dvdx) / 2;
    return g.peripheral_ff(i, j) ? v.wall_factor * e : e;
}
// the wall-masked strain rates of the viscosity (no ice mask): effective_strain_rate² (strain_rates.jl:27-32)
__device__ __forceinline__ double wall_u(const FrontView& v, int i, int j) {
    return v.g.peripheral_fc(i, j) ? 0.0 : v.x[v.g.u_idx(i, j)].x;
}
__device__ __forceinline__ double wall_v(const FrontView& v, int i, int j) {
    return v.g.peripheral_cf(i, j) ? 0.0 : v.x[v.g.v_idx(i, j)].y;
}
__device__ __forceinline__ double wall_strain_xy2(const FrontView& v, int i, int j) {
    const DevGrid<double>& g = v.g;
    double dudy = (wall_u(v, i, j) - wall_u(v, i, j - 1)) / g.dyf[j];
    double dvdx = (wall_v(v, i, j) - wall_v(v, i - 1, j)) / g.dxf[i];
    double e = (dudy + dvdx) / 2;
    e = g.peripheral_ff(i, j) ? v.wall_factor * e : e;
    return e * e;
}
__device__ double effective_strain_rate2(const FrontView& v, int i, int j) {
    const DevGrid<double>& g = v.g;
    double exx = (wall_u(v, i + 1, j) - wall_u(v, i, j)) / g.dxc[i];
    double eyy = (wall_v(v, i, j + 1) - wall_v(v, i, j)) / g.dyc[j];
    double a = (wall_strain_xy2(v, i, j) + wall_strain_xy2(v, i + 1, j)) / 2;
    double b = (wall_strain_xy2(v, i, j + 1) + wall_strain_xy2(v, i + 1, j + 1)) / 2;
    return exx * exx + eyy * eyy + exx * eyy + (a + b) / 2;
}

// principal_strain_rates (calving.jl:144-152) with the velocities masked by the flag
__device__ void principal_strain_rates(const FrontView& v, int i, int j, double& e1, double& e2) {
    const DevGrid<double>& g = v.g;
    double exx = (mu_u(v, i + 1, j) - mu_u(v, i, j)) / g.dxc[i];
    double eyy = (mu_v(v, i, j + 1) - mu_v(v, i, j)) / g.dyc[j];
    double exy = ((mu_strain_xy(v, i, j) + mu_strain_xy(v, i + 1, j)) / 2 + (mu_strain_xy(v, i, j + 1) + mu_strain_xy(v, i + 1, j + 1)) / 2) / 2;
    double eb = (exx + eyy) / 2;
    double r = sqrt(((exx - eyy) / 2) * ((exx - eyy) / 2) + exy * exy + v.eps0 * v.eps0);
    e1 = eb + r;
    e2 = eb - r;
}

// front_flow_speed (calving.jl:176-181): the larger face speed along each axis
__device__ double front_flow_speed(const FrontView& v, int i, int j) {
    double ut = fmax(fabs(mu_u(v, i, j)), fabs(mu_u(v, i + 1, j)));
    double vt = fmax(fabs(mu_v(v, i, j)), fabs(mu_v(v, i, j + 1)));
    double e = v.eps0 * v.g.dxc[i];
    return sqrt(ut * ut + vt * vt + e * e);
}

// calving_rate of a full cell (calving.jl:154-190)
__device__ double calving_rate(const FrontView& v, int i, int j) {
    int k = v.g.c_idx(i, j);
    if (v.law == NK_CALVING_EIGEN) {
        double e1, e2;
        principal_strain_rates(v, i, j, e1, e2);
        return v.coefficient * fmax(e1, 0.0) * fmax(e2, 0.0);
    }
    if (v.law == NK_CALVING_VON_MISES) {
        double e1, e2;
        principal_strain_rates(v, i, j, e1, e2);
        double n = v.n, e0 = v.eps0;
        double et2 = (fmax(e1, 0.0) * fmax(e1, 0.0) + fmax(e2, 0.0) * fmax(e2, 0.0)) / 2;
        double ee2 = effective_strain_rate2(v, i, j) + e0 * e0;
        double Hi = v.H[k];
        double eta = v.coef[k].x / (Hi > 0 ? Hi : 1.0);
        double smax = v.phi[k] * v.stress_threshold + (1 - v.phi[k]) * v.floating_stress_threshold;
        double B = 2 * eta * pow(ee2, (n - 1) / (2 * n));
        double sig = sqrt(3.0) * B * et2 * pow(et2 + e0 * e0, (1 - 2 * n) / (2 * n));
        return front_flow_speed(v, i, j) * sig / smax;
    }
    if (v.law == NK_CALVING_FRONT_VELOCITY) {
        double c = fmax(front_flow_speed(v, i, j) - v.front_velocity, 0.0);
        return (1 - v.phi[k]) * c;
    }
    return 0.0;
}

// front_ice_thickness (:331): its own thickness when full or not yet given an Hʳ
__device__ __forceinline__ double front_ice_thickness(const FrontView& v, int k) {
    return (full_at(v.mu, k) || v.Hr[k] <= 0) ? v.H[k] : v.Hr[k];
}

// remove_front_fraction! (:353-368) on the calling thread's own cell; returns the part of g beyond its ice
__device__ double remove_front_fraction(const FrontView& v, int k, double gfrac) {
    double Hi = v.H[k], Hf = front_ice_thickness(v, k);
    bool calves = (gfrac > 0) && (Hi > 0);
    double Hn = fmax(Hi - gfrac * Hf, 0.0);
    double a = Hf > 0 ? Hi / (Hf > 0 ? Hf : 1.0) : 0.0;
    if (calves) {
        v.calved[k] += Hi - Hn;
        v.H[k] = Hn;
        v.Hr[k] = Hn > 0 ? Hf : 0.0;
        v.mu[k] = 0.0;
    }
    return calves ? fmax(gfrac - a, 0.0) : 0.0;
}

}  // namespace

// initialize_front! (:80-92)
__global__ void k_initialize_front(FrontView v) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= v.g.Nx || j >= v.g.Ny) return;
    int k = v.g.idx(i, j);
    v.mu[k] = v.H[k] > 0 ? 1.0 : 0.0;
    v.Hr[k] = 0.0;
}

// _empty_drained_cells! (:197-200)
__global__ void k_front_drained(FrontView v) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= v.g.Nx || j >= v.g.Ny) return;
    int k = v.g.idx(i, j);
    if (v.H[k] <= 0) v.mu[k] = 0.0;
}

// _compute_reference_thickness! (:206-230): the mean thickness of the full neighbours flowing in; otherwise the kept
// Hʳ, the mean of all full neighbours, or H.  Reads only its own Hʳ.
__global__ void k_front_reference(FrontView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    bool inflow[4] = {v.x[g.u_idx(i, j)].x > 0, v.x[g.u_idx(i + 1, j)].x < 0, v.x[g.v_idx(i, j)].y > 0, v.x[g.v_idx(i, j + 1)].y < 0};
    double Sin = 0, Sf = 0;
    int nin = 0, nf = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        int a = i + DI(d), b = j + DJ(d);
        if (!full_neighbor(g, v.mu, a, b)) continue;
        double Hn = v.H[g.c_idx(a, b)];
        Sf += Hn;
        ++nf;
        if (inflow[d]) { Sin += Hn; ++nin; }
    }
    // the reference sums the four neighbours in the order west, east, south, north with zeros for the others
    double Hi = v.H[k];
    double Hs = nf > 0 ? Sf / (double)(nf > 1 ? nf : 1) : Hi;
    double Hp = Hi > 0 ? (v.Hr[k] > 0 ? v.Hr[k] : Hs) : 0.0;
    double Hbar = nin > 0 ? Sin / (double)(nin > 1 ? nin : 1) : Hp;
    v.Hr[k] = full_at(v.mu, k) ? 0.0 : Hbar;
}

// _fill_front_cells! (:235-251) from the snapshots H_in, mu_in
__global__ void k_front_fill(FrontView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    int n = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) n += empty_at(g, v.mu_in, v.H_in, i + DI(d), j + DJ(d)) ? 1 : 0;
    double Hi = v.H_in[k], Hri = v.Hr[k];
    bool fills = !full_at(v.mu_in, k) && (Hri > 0) && (Hi >= Hri);
    bool spills = fills && n > 0;
    v.O[k] = spills ? (Hi - Hri) * g.Az_cc(i, j) / (double)(n > 1 ? n : 1) : 0.0;
    v.H[k] = spills ? Hri : Hi;
    if (fills) v.mu[k] = 1.0;
}

// _receive_overflow! (:257-268): every donor counted each of its empty neighbours; H_in is the thickness after the fill
__global__ void k_front_receive(FrontView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    bool receives = empty_at(g, v.mu, v.H_in, i, j);
    double V = 0, S = 0;
    int n = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        int a = i + DI(d), b = j + DJ(d);
        if (inactive(g, a, b)) continue;
        int c = g.c_idx(a, b);
        V += v.O[c];
        if (v.O[c] > 0) { S += v.H_in[c]; ++n; }
    }
    if (receives) v.H[k] = V / g.Az_cc(i, j);
    if (receives && n > 0) v.Hr[k] = S / (double)(n > 1 ? n : 1);
}

// _compute_retreat_fraction! (:311-322) with front_length (:334-343) and retreat_fraction (calving.jl:212-227), from
// the state before any cell retreats
__global__ void k_calve_fraction(FrontView v, double dt) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    double dx = g.dxc[i], dy = g.dyc[j];
    auto ocean = [&](int a, int b, double len) { return (empty_at(g, v.mu, v.H, a, b) && v.bed[g.c_idx(a, b)] < 0) ? len : 0.0; };
    double lw = ocean(i - 1, j, dy), le = ocean(i + 1, j, dy), ls = ocean(i, j - 1, dx), ln = ocean(i, j + 1, dx);
    double r = 0.0;
    if (v.H[k] > 0 && (lw + le + ls + ln > 0)) {
        double Hf = front_ice_thickness(v, k);
        if (v.law == NK_CALVING_THICKNESS_THRESHOLD) {
            r = Hf < v.thickness ? 1.0 : 0.0;
        } else if (v.law == NK_CALVING_MAXIMUM_EXTENT) {
            r = v.extent[k] > 0 ? 0.0 : 1.0;
        } else {
            double ub = fabs((mu_u(v, i, j) + mu_u(v, i + 1, j)) / 2);
            double vb = fabs((mu_v(v, i, j) + mu_v(v, i, j + 1)) / 2);
            double speed = sqrt(ub * ub + vb * vb);
            double l2 = (le - lw) * (le - lw) + (ln - ls) * (ln - ls);
            double lv = l2 > 0 ? sqrt(l2 > 0 ? l2 : 1.0) : lw + le + ls + ln;
            double lu = (ub * (lw + le) + vb * (ls + ln)) / (speed > 0 ? speed : 1.0);
            double l = speed > 0 ? lu : lv;
            // front_calving_rate (calving.jl:197-206): a partial cell takes the mean rate of its full neighbours
            double c;
            if (full_at(v.mu, k)) {
                c = calving_rate(v, i, j);
            } else {
                double S = 0;
                int n = 0;
#pragma unroll
                for (int d = 0; d < 4; ++d)
                    if (full_neighbor(g, v.mu, i + DI(d), j + DJ(d))) { S += calving_rate(v, i + DI(d), j + DJ(d)); ++n; }
                c = S / (double)(n > 1 ? n : 1);
            }
            r = fmin(1.0, c * dt * l / g.Az_cc(i, j));
        }
    }
    v.f[k] = r;
}

// _retreat_front_cells! (:371-375): f becomes the area of retreat left once the cell is empty (rate laws only)
__global__ void k_calve_retreat(FrontView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    double r = remove_front_fraction(v, k, v.f[k]);
    bool removal = v.law == NK_CALVING_THICKNESS_THRESHOLD || v.law == NK_CALVING_MAXIMUM_EXTENT;
    v.f[k] = (removal ? 0.0 : r) * g.Az_cc(i, j);
}

// _share_residual_retreat! (:379-385): among the neighbours that hold ice
__global__ void k_calve_share(FrontView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    int n = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        int a = i + DI(d), b = j + DJ(d);
        n += (!inactive(g, a, b) && v.H[g.c_idx(a, b)] > 0) ? 1 : 0;
    }
    v.share[k] = n > 0 ? v.f[k] / (double)(n > 1 ? n : 1) : 0.0;
}

// _receive_residual_retreat! (:390-397): what the receiving cell cannot take is not passed on
__global__ void k_calve_receive(FrontView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    double A = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        int a = i + DI(d), b = j + DJ(d);
        A += inactive(g, a, b) ? 0.0 : v.share[g.c_idx(a, b)];
    }
    remove_front_fraction(v, k, A / g.Az_cc(i, j));
}

// _force_front_cells! (:271-286): the sources of the step on partial cells and on cells that filled or calved
__global__ void k_front_force(FrontView v, double dt) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    double Hi = v.H[k], Hri = v.Hr[k];
    double m = v.grounding ? (1 - v.phi[k]) * v.melt[k] : v.melt[k];
    double S = v.smb[k] - m - (v.coupled ? v.gmelt[k] : 0.0);
    bool full = full_at(v.mu, k);
    bool forced = (Hi > 0) && (Hri > 0);
    double Hf = full ? Hi : Hri;
    bool melted = forced && (Hf + S * dt <= 0);
    double Hn = full ? Hi + S * dt : Hi / (Hri > 0 ? Hri : 1.0) * (Hri + S * dt);
    if (melted) v.clipped[k] += -Hn;
    v.H[k] = melted ? 0.0 : (forced ? Hn : Hi);
    v.Hr[k] = (melted || full) ? 0.0 : (forced ? Hri + S * dt : Hri);
    if (melted) v.mu[k] = 0.0;
}

void launch_initialize_front(const FrontView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.g.Nx, v.g.Ny);
    k_initialize_front<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// advance_front!(front, model, Δt), partial_cell_front.jl:167-195
void launch_advance_front(const FrontView& v, int passes, double dt, size_t plane, cudaStream_t s) {
    LaunchDims d = dims2d(v.g.Nx, v.g.Ny);
    const size_t bytes = plane * sizeof(double);
    k_front_drained<<<d.grid, d.block, 0, s>>>(v); count_launch();
    k_front_reference<<<d.grid, d.block, 0, s>>>(v); count_launch();
    for (int p = 0; p < passes; ++p) {
        cudaMemcpyAsync(v.H_in, v.H, bytes, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(v.mu_in, v.mu, bytes, cudaMemcpyDeviceToDevice, s);
        k_front_fill<<<d.grid, d.block, 0, s>>>(v); count_launch();
        cudaMemcpyAsync(v.H_in, v.H, bytes, cudaMemcpyDeviceToDevice, s);
        k_front_receive<<<d.grid, d.block, 0, s>>>(v); count_launch();
    }
    if (v.law != NK_CALVING_NONE) {
        k_calve_fraction<<<d.grid, d.block, 0, s>>>(v, dt); count_launch();
        k_calve_retreat<<<d.grid, d.block, 0, s>>>(v); count_launch();
        k_calve_share<<<d.grid, d.block, 0, s>>>(v); count_launch();
        k_calve_receive<<<d.grid, d.block, 0, s>>>(v); count_launch();
    }
    k_front_force<<<d.grid, d.block, 0, s>>>(v, dt); count_launch();
}

// ---- the reverse of advance_front! without calving (the gradient through time steps) ----------------------------
// The forward is recorded first (launch_front_record): the drain and the reference pass, then per overflow pass the
// state before its fill, after its fill and its overflow volumes, and the state before the forced sources.  The
// reverse runs the forced sources, the passes last first (receive, then fill) and the reference pass, each kernel
// writing only its own cell's adjoints and gathering its neighbours' shares.
namespace {
// full after _empty_drained_cells!: flagged, holding ice and active
__device__ __forceinline__ bool drained_full(const DevGrid<double>& g, const double* mu, const double* H, int a, int b) {
    if (inactive(g, a, b)) return false;
    int c = g.c_idx(a, b);
    return mu[c] > 0 && H[c] > 0;
}
// The reference pass of cell (i, j) after the drain (k_front_reference): its sums over the full neighbours and over
// those flowing in, and the branch its Hʳ took.
struct Reference {
    double Hi, Hr_old, Hbar, Sin, Sf;
    int nin, nf;
    bool full, inflow[4];
};
__device__ Reference reference_of(const FrontView& v, int i, int j) {
    const DevGrid<double>& g = v.g;
    Reference r;
    int k = g.idx(i, j);
    r.inflow[0] = v.x[g.u_idx(i, j)].x > 0;
    r.inflow[1] = v.x[g.u_idx(i + 1, j)].x < 0;
    r.inflow[2] = v.x[g.v_idx(i, j)].y > 0;
    r.inflow[3] = v.x[g.v_idx(i, j + 1)].y < 0;
    r.Sin = r.Sf = 0.0;
    r.nin = r.nf = 0;
    for (int d = 0; d < 4; ++d) {
        int a = i + DI(d), b = j + DJ(d);
        if (!drained_full(g, v.mu, v.H, a, b)) continue;
        double Hn = v.H[g.c_idx(a, b)];
        r.Sf += Hn;
        ++r.nf;
        if (r.inflow[d]) { r.Sin += Hn; ++r.nin; }
    }
    r.Hi = v.H[k];
    r.Hr_old = v.Hr[k];
    r.full = v.mu[k] > 0 && r.Hi > 0;
    double Hs = r.nf > 0 ? r.Sf / (double)(r.nf > 1 ? r.nf : 1) : r.Hi;
    double Hp = r.Hi > 0 ? (r.Hr_old > 0 ? r.Hr_old : Hs) : 0.0;
    r.Hbar = r.nin > 0 ? r.Sin / (double)(r.nin > 1 ? r.nin : 1) : Hp;
    return r;
}
// the recorded levels: before fill p (p = passes: before the forced sources) H, μ, Hʳ; per pass after its fill H, O
__device__ __forceinline__ const double* level(const FrontAdjointView& a, int p, int field) {
    return a.snaps + ((size_t)3 * p + field) * a.plane;
}
__device__ __forceinline__ const double* filled(const FrontAdjointView& a, int p, int field) {
    return a.snaps + ((size_t)3 * (a.passes + 1) + 2 * p + field) * a.plane;
}
// the calving block: 0 fraction, 1-3 H, μ, Hʳ after the retreat, 4 its residual, 5 the shares, 6-8 after the receive
__device__ __forceinline__ const double* calved(const FrontAdjointView& a, int field) {
    return a.snaps + ((size_t)3 * (a.passes + 1) + 2 * a.passes + field) * a.plane;
}
// the state the forced sources read: after the calving, else after the last pass
__device__ __forceinline__ const double* forced_level(const FrontAdjointView& a, int field) {
    return a.f.law != NK_CALVING_NONE ? calved(a, 6 + field) : level(a, a.passes, field);
}
// overflow donors among the active neighbours of (i, j) in pass p
__device__ __forceinline__ int donors_of(const FrontAdjointView& a, const double* O, int i, int j) {
    const DevGrid<double>& g = a.f.g;
    int n = 0;
    for (int d = 0; d < 4; ++d) {
        int x = i + DI(d), y = j + DJ(d);
        if (!inactive(g, x, y) && O[g.c_idx(x, y)] > 0) ++n;
    }
    return n;
}
}  // namespace

int front_record_planes(int passes, int law) { return 3 * (passes + 1) + 2 * passes + (law != NK_CALVING_NONE ? 9 : 0); }

void launch_front_record(const FrontView& v, int passes, size_t plane, double* snaps, double dt, cudaStream_t s) {
    LaunchDims d = dims2d(v.g.Nx, v.g.Ny);
    const size_t bytes = plane * sizeof(double);
    auto keep = [&](double* to, const double* from) { cudaMemcpyAsync(to, from, bytes, cudaMemcpyDeviceToDevice, s); };
    auto lev = [&](int p, int field) { return snaps + ((size_t)3 * p + field) * plane; };
    auto fil = [&](int p, int field) { return snaps + ((size_t)3 * (passes + 1) + 2 * p + field) * plane; };
    k_front_drained<<<d.grid, d.block, 0, s>>>(v); count_launch();
    k_front_reference<<<d.grid, d.block, 0, s>>>(v); count_launch();
    keep(lev(0, 0), v.H);
    keep(lev(0, 1), v.mu);
    keep(lev(0, 2), v.Hr);
    for (int p = 0; p < passes; ++p) {
        keep(v.H_in, v.H);
        keep(v.mu_in, v.mu);
        k_front_fill<<<d.grid, d.block, 0, s>>>(v); count_launch();
        keep(fil(p, 0), v.H);
        keep(fil(p, 1), v.O);
        keep(v.H_in, v.H);
        k_front_receive<<<d.grid, d.block, 0, s>>>(v); count_launch();
        keep(lev(p + 1, 0), v.H);
        keep(lev(p + 1, 1), v.mu);
        keep(lev(p + 1, 2), v.Hr);
    }
    if (v.law != NK_CALVING_NONE) {
        double* c = snaps + ((size_t)3 * (passes + 1) + 2 * passes) * plane;
        auto cal = [&](int field) { return c + (size_t)field * plane; };
        k_calve_fraction<<<d.grid, d.block, 0, s>>>(v, dt); count_launch();
        keep(cal(0), v.f);
        k_calve_retreat<<<d.grid, d.block, 0, s>>>(v); count_launch();
        keep(cal(1), v.H);
        keep(cal(2), v.mu);
        keep(cal(3), v.Hr);
        keep(cal(4), v.f);
        k_calve_share<<<d.grid, d.block, 0, s>>>(v); count_launch();
        keep(cal(5), v.share);
        k_calve_receive<<<d.grid, d.block, 0, s>>>(v); count_launch();
        keep(cal(6), v.H);
        keep(cal(7), v.mu);
        keep(cal(8), v.Hr);
    }
}

// The reverse of _force_front_cells! (:271-286) on the state before it: λ of H and Hʳ before, and of the sources.
__global__ void k_front_rev_force(FrontAdjointView a) {
    const FrontView& v = a.f;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    const double Hi = forced_level(a, 0)[k], Hr = forced_level(a, 2)[k];
    const bool full = forced_level(a, 1)[k] > 0;
    double m = v.grounding ? (1 - v.phi[k]) * v.melt[k] : v.melt[k];
    double S = v.smb[k] - m;
    double dt = a.dt;
    bool forced = (Hi > 0) && (Hr > 0);
    double Hf = full ? Hi : Hr;
    bool melted = forced && (Hf + S * dt <= 0);
    double lH = a.lam_H[k], lR = a.lam_Hr[k];
    double lHi = 0.0, lHr = 0.0, lS = 0.0;
    if (melted) {
        // H and Hʳ become zero: nothing flows back
    } else if (forced && !full) {   // a partial cell: H (Hʳ + S Δt) / Hʳ, Hʳ + S Δt
        lHi = lH * (Hr + S * dt) / Hr;
        lHr = lH * Hi * (-S * dt) / (Hr * Hr) + lR;
        lS = (lH * Hi / Hr + lR) * dt;
    } else if (forced) {            // a full cell that filled this step: H + S Δt, Hʳ zero
        lHi = lH;
        lS = lH * dt;
    } else {
        lHi = lH;
        lHr = full ? 0.0 : lR;
    }
    a.lam_smb[k] += lS;
    a.lam_melt[k] -= lS * (v.grounding ? 1 - v.phi[k] : 1.0) * a.melt_weight;
    a.lam_phi[k] = v.grounding ? lS * v.melt[k] : 0.0;
    a.lam_a[k] = lHi;
    a.lam_Hr[k] = lHr;
}

// The reverse of _receive_overflow! (:257-268) of pass p: λ of the thickness after the fill (own and as a donor's
// mean), of the overflow volumes (as every receiving neighbour's sum) and of Hʳ before the receive.
__global__ void k_front_rev_receive(FrontAdjointView a, int p) {
    const DevGrid<double>& g = a.f.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    const double* Hf = filled(a, p, 0);
    const double* O = filled(a, p, 1);
    const double* mu1 = level(a, p + 1, 1);
    auto receives = [&](int x, int y) { return empty_at(g, mu1, Hf, x, y); };
    bool rc = receives(i, j);
    int nc = donors_of(a, O, i, j);
    double lHf = rc ? 0.0 : a.lam_a[c];
    double lHr = (rc && nc > 0) ? 0.0 : a.lam_Hr[c];
    double lO = 0.0;
    int seen[4], ns = 0;
    for (int e = 0; e < 4; ++e) {
        int x = i + DI(e), y = j + DJ(e);
        if (inactive(g, x, y)) continue;
        int k = g.c_idx(x, y);
        bool dup = false;
        for (int q = 0; q < ns; ++q) dup |= seen[q] == k;
        if (dup) continue;
        seen[ns++] = k;
        int kx = g.cx(x), ky = g.cy(y);
        if (!receives(kx, ky)) continue;
        // how often k reads c among its four neighbours (a short periodic axis can repeat one)
        int reads = 0;
        for (int d = 0; d < 4; ++d) {
            int na = kx + DI(d), nb = ky + DJ(d);
            if (!inactive(g, na, nb) && g.c_idx(na, nb) == c) ++reads;
        }
        lO += reads * a.lam_a[k] / g.Az_cc(kx, ky);
        int nk = donors_of(a, O, kx, ky);
        if (nk > 0 && O[c] > 0) lHf += reads * a.lam_Hr[k] / (double)nk;
    }
    a.lam_b[c] = lHf;
    a.lam_c[c] = lO;
    a.lam_d[c] = lHr;
}

// The reverse of _fill_front_cells! (:235-251) of pass p on its own cell: λ of the thickness and Hʳ before it.
__global__ void k_front_rev_fill(FrontAdjointView a, int p) {
    const DevGrid<double>& g = a.f.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    const double* H = level(a, p, 0);
    const double* mu = level(a, p, 1);
    const double* Hr = level(a, p, 2);
    int n = 0;
    for (int d = 0; d < 4; ++d) n += empty_at(g, mu, H, i + DI(d), j + DJ(d)) ? 1 : 0;
    bool fills = !(mu[k] > 0) && (Hr[k] > 0) && (H[k] >= Hr[k]);
    bool spills = fills && n > 0;
    double lHf = a.lam_b[k], lO = a.lam_c[k];
    double w = g.Az_cc(i, j) / (double)(n > 1 ? n : 1);
    a.lam_a[k] = spills ? lO * w : lHf;
    a.lam_Hr[k] = a.lam_d[k] + (spills ? lHf - lO * w : 0.0);
}

// Per cell: the cell's own terms of the reference pass (k_front_reference), from λ of H and Hʳ after it.
__global__ void k_front_rev_reference(FrontAdjointView a) {
    const FrontView& v = a.f;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    Reference r = reference_of(v, i, j);
    double lHi = a.lam_a[k];
    // Hʳ = H̄ on a cell not full: the donors' and full neighbours' shares are gathered by k_front_rev_gather
    double lbar = r.full ? 0.0 : a.lam_Hr[k], lHr_old = 0.0;
    if (r.nin == 0 && r.Hi > 0) {
        if (r.Hr_old > 0) lHr_old = lbar;
        else if (r.nf == 0) lHi += lbar;   // Hˢ = H of the cell itself
    }
    a.lam_b[k] = lbar;
    a.lam_c[k] = lHi;
    a.lam_Hr[k] = lHr_old;
}

// Per cell c: its own part plus the shares of the reference thickness of the neighbours it is a full neighbour of
// (the donors' mean when any flows in, else the full neighbours' mean when the cell had no Hʳ).
__global__ void k_front_rev_gather(FrontAdjointView a) {
    const FrontView& v = a.f;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    double acc = a.lam_c[c];
    if (drained_full(g, v.mu, v.H, i, j)) {
        int seen[4], ns = 0;
        for (int e = 0; e < 4; ++e) {
            int ki = i + DI(e), kj = j + DJ(e);
            if (inactive(g, ki, kj)) continue;
            int kc = g.c_idx(ki, kj);
            bool dup = false;
            for (int q = 0; q < ns; ++q) dup |= seen[q] == kc;
            if (dup) continue;
            seen[ns++] = kc;
            double lbar = a.lam_b[kc];
            if (lbar == 0.0) continue;
            int ci = g.cx(ki), cj = g.cy(kj);
            Reference r = reference_of(v, ci, cj);
            for (int d = 0; d < 4; ++d) {
                int na = ci + DI(d), nb = cj + DJ(d);
                if (inactive(g, na, nb) || g.c_idx(na, nb) != c) continue;
                if (r.nin > 0) {
                    if (r.inflow[d]) acc += lbar / (double)r.nin;
                } else if (r.Hi > 0 && !(r.Hr_old > 0) && r.nf > 0) {
                    acc += lbar / (double)r.nf;
                }
            }
        }
    }
    a.lam_H3[c] = acc;
}

// ---- the reverse of the calving (calve_front!, :300-397) for the rate laws and the removal laws -------------------
namespace {
// a value and its derivative along one seeded face velocity
struct Dual {
    double v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator*(double s, Dual a) { return {s * a.v, s * a.d}; }
__device__ __forceinline__ Dual operator/(Dual a, double s) { return {a.v / s, a.d / s}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
__device__ __forceinline__ Dual dsqrt(Dual a) { double r = sqrt(a.v); return {r, r > 0 ? a.d / (2 * r) : 0.0}; }
__device__ __forceinline__ Dual dabs(Dual a) { return a.v >= 0 ? a : Dual{-a.v, -a.d}; }
__device__ __forceinline__ Dual dmax(Dual a, Dual b) { return fmax(a.v, b.v) == a.v ? a : b; }
__device__ __forceinline__ Dual dpos(Dual a) { return a.v > 0 ? a : Dual{0.0, 0.0}; }   // fmax(a, 0)
__device__ __forceinline__ Dual dpow(Dual a, double p) {
    double r = pow(a.v, p);
    return {r, a.d != 0.0 ? p * pow(a.v, p - 1) * a.d : 0.0};
}

// The flag-masked face velocities of mu_u / mu_v with the seed's derivative: seed_u / seed_v is the stored index of
// the seeded u / v face (-1: none).
struct Seed {
    int u, v;
};
__device__ __forceinline__ Dual dmu_u(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    if (g.peripheral_fc(i, j) || (v.mu[g.c_idx(i - 1, j)] + v.mu[g.c_idx(i, j)]) == 0.0) return {0.0, 0.0};
    int k = g.u_idx(i, j);
    return {v.x[k].x, k == sd.u ? 1.0 : 0.0};
}
__device__ __forceinline__ Dual dmu_v(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    if (g.peripheral_cf(i, j) || (v.mu[g.c_idx(i, j - 1)] + v.mu[g.c_idx(i, j)]) == 0.0) return {0.0, 0.0};
    int k = g.v_idx(i, j);
    return {v.x[k].y, k == sd.v ? 1.0 : 0.0};
}
__device__ __forceinline__ Dual dstrain_xy(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    Dual dudy = (dmu_u(v, i, j, sd) - dmu_u(v, i, j - 1, sd)) / g.dyf[j];
    Dual dvdx = (dmu_v(v, i, j, sd) - dmu_v(v, i - 1, j, sd)) / g.dxf[i];
    Dual e = (dudy + dvdx) / 2.0;
    return g.peripheral_ff(i, j) ? v.wall_factor * e : e;
}
// the wall-masked velocities and strain rates of effective_strain_rate2, with the seed's derivative
__device__ __forceinline__ Dual dwall_u(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    if (g.peripheral_fc(i, j)) return {0.0, 0.0};
    int k = g.u_idx(i, j);
    return {v.x[k].x, k == sd.u ? 1.0 : 0.0};
}
__device__ __forceinline__ Dual dwall_v(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    if (g.peripheral_cf(i, j)) return {0.0, 0.0};
    int k = g.v_idx(i, j);
    return {v.x[k].y, k == sd.v ? 1.0 : 0.0};
}
__device__ __forceinline__ Dual dwall_strain_xy2(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    Dual dudy = (dwall_u(v, i, j, sd) - dwall_u(v, i, j - 1, sd)) / g.dyf[j];
    Dual dvdx = (dwall_v(v, i, j, sd) - dwall_v(v, i - 1, j, sd)) / g.dxf[i];
    Dual e = (dudy + dvdx) / 2.0;
    e = g.peripheral_ff(i, j) ? v.wall_factor * e : e;
    return e * e;
}
__device__ Dual deffective_strain_rate2(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    Dual exx = (dwall_u(v, i + 1, j, sd) - dwall_u(v, i, j, sd)) / g.dxc[i];
    Dual eyy = (dwall_v(v, i, j + 1, sd) - dwall_v(v, i, j, sd)) / g.dyc[j];
    Dual a = (dwall_strain_xy2(v, i, j, sd) + dwall_strain_xy2(v, i + 1, j, sd)) / 2.0;
    Dual b = (dwall_strain_xy2(v, i, j + 1, sd) + dwall_strain_xy2(v, i + 1, j + 1, sd)) / 2.0;
    return exx * exx + eyy * eyy + exx * eyy + (a + b) / 2.0;
}
// principal_strain_rates (calving.jl:144-152) with the seed's derivative
__device__ __forceinline__ void dprincipal_strain_rates(const FrontView& v, int i, int j, Seed sd, Dual& e1, Dual& e2) {
    const DevGrid<double>& g = v.g;
    Dual exx = (dmu_u(v, i + 1, j, sd) - dmu_u(v, i, j, sd)) / g.dxc[i];
    Dual eyy = (dmu_v(v, i, j + 1, sd) - dmu_v(v, i, j, sd)) / g.dyc[j];
    Dual exy = ((dstrain_xy(v, i, j, sd) + dstrain_xy(v, i + 1, j, sd)) / 2.0 +
                (dstrain_xy(v, i, j + 1, sd) + dstrain_xy(v, i + 1, j + 1, sd)) / 2.0) / 2.0;
    Dual eb = (exx + eyy) / 2.0;
    Dual h = (exx - eyy) / 2.0;
    Dual r = dsqrt(h * h + exy * exy + Dual{v.eps0 * v.eps0, 0.0});
    e1 = eb + r;
    e2 = eb - r;
}
// The von Mises rate of a full cell (calving.jl:160-174) at viscosity eta, with the seed's derivative, in the order
// calving_rate evaluates it; the rate is linear in eta, so eta = 1 gives its derivative with respect to eta.
__device__ Dual dvon_mises_rate(const FrontView& v, int i, int j, Seed sd, double eta) {
    const DevGrid<double>& g = v.g;
    int k = g.c_idx(i, j);
    Dual e1, e2;
    dprincipal_strain_rates(v, i, j, sd, e1, e2);
    double n = v.n, e0 = v.eps0;
    Dual p1 = dpos(e1), p2 = dpos(e2);
    Dual et2 = (p1 * p1 + p2 * p2) / 2.0;
    Dual ee2 = deffective_strain_rate2(v, i, j, sd) + Dual{e0 * e0, 0.0};
    double smax = v.phi[k] * v.stress_threshold + (1 - v.phi[k]) * v.floating_stress_threshold;
    Dual B = (2 * eta) * dpow(ee2, (n - 1) / (2 * n));
    Dual sig = sqrt(3.0) * B * et2 * dpow(et2 + Dual{e0 * e0, 0.0}, (1 - 2 * n) / (2 * n));
    Dual ut = dmax(dabs(dmu_u(v, i, j, sd)), dabs(dmu_u(v, i + 1, j, sd)));
    Dual vt = dmax(dabs(dmu_v(v, i, j, sd)), dabs(dmu_v(v, i, j + 1, sd)));
    double e = e0 * g.dxc[i];
    Dual fs = dsqrt(ut * ut + vt * vt + Dual{e * e, 0.0});
    return fs * sig / smax;
}
// η = η̄H / H of cell k as the von Mises rate reads it
__device__ __forceinline__ double von_mises_eta(const FrontView& v, int k) {
    double Hi = v.H[k];
    return v.coef[k].x / (Hi > 0 ? Hi : 1.0);
}
// calving_rate of a full cell (calving.jl:154-190) for the rate laws, with the seed's derivative (principal_strain_rates
// and front_flow_speed as k_calve_fraction evaluates them)
__device__ Dual dcalving_rate(const FrontView& v, int i, int j, Seed sd) {
    const DevGrid<double>& g = v.g;
    if (v.law == NK_CALVING_VON_MISES) return dvon_mises_rate(v, i, j, sd, von_mises_eta(v, g.c_idx(i, j)));
    if (v.law == NK_CALVING_EIGEN) {
        Dual e1, e2;
        dprincipal_strain_rates(v, i, j, sd, e1, e2);
        return v.coefficient * (dpos(e1) * dpos(e2));
    }
    if (v.law == NK_CALVING_FRONT_VELOCITY) {
        Dual ut = dmax(dabs(dmu_u(v, i, j, sd)), dabs(dmu_u(v, i + 1, j, sd)));
        Dual vt = dmax(dabs(dmu_v(v, i, j, sd)), dabs(dmu_v(v, i, j + 1, sd)));
        double e = v.eps0 * g.dxc[i];
        Dual fs = dsqrt(ut * ut + vt * vt + Dual{e * e, 0.0});
        return (1 - v.phi[g.c_idx(i, j)]) * dpos(fs - Dual{v.front_velocity, 0.0});
    }
    return {0.0, 0.0};
}
// The ocean-facing lengths of cell (i, j) and its front length l (k_calve_fraction), with the seed's derivative
struct FrontLength {
    double lw, le, ls, ln;
    bool facing;
};
__device__ FrontLength front_lengths(const FrontView& v, int i, int j) {
    const DevGrid<double>& g = v.g;
    double dx = g.dxc[i], dy = g.dyc[j];
    auto ocean = [&](int a, int b, double len) { return (empty_at(g, v.mu, v.H, a, b) && v.bed[g.c_idx(a, b)] < 0) ? len : 0.0; };
    FrontLength f;
    f.lw = ocean(i - 1, j, dy);
    f.le = ocean(i + 1, j, dy);
    f.ls = ocean(i, j - 1, dx);
    f.ln = ocean(i, j + 1, dx);
    f.facing = f.lw + f.le + f.ls + f.ln > 0;
    return f;
}
__device__ Dual dfront_length(const FrontView& v, int i, int j, const FrontLength& f, Seed sd) {
    Dual ub = dabs((dmu_u(v, i, j, sd) + dmu_u(v, i + 1, j, sd)) / 2.0);
    Dual vb = dabs((dmu_v(v, i, j, sd) + dmu_v(v, i, j + 1, sd)) / 2.0);
    Dual speed = dsqrt(ub * ub + vb * vb);
    if (!(speed.v > 0)) {
        double l2 = (f.le - f.lw) * (f.le - f.lw) + (f.ln - f.ls) * (f.ln - f.ls);
        return {l2 > 0 ? sqrt(l2) : f.lw + f.le + f.ls + f.ln, 0.0};
    }
    return (Dual{f.lw + f.le, 0.0} * ub + Dual{f.ls + f.ln, 0.0} * vb) / speed;
}
__device__ __forceinline__ bool rate_law(int law) {
    return law == NK_CALVING_EIGEN || law == NK_CALVING_FRONT_VELOCITY || law == NK_CALVING_VON_MISES;
}
__device__ __forceinline__ bool removal_law(int law) {
    return law == NK_CALVING_THICKNESS_THRESHOLD || law == NK_CALVING_MAXIMUM_EXTENT;
}
// remove_front_fraction! (:353-368) of a cell with thickness H, flag mu and Hʳ Hr by the fraction g: the reverse from
// λ of H and Hʳ after it and of its residual (times w) to λ of H, Hʳ and g.
__device__ __forceinline__ void remove_fraction_reverse(double H, double mu, double Hr, double gfrac, double lH, double lR,
                                                        double lres, double w, double& oH, double& oR, double& og) {
    bool own = (mu > 0) || !(Hr > 0);      // front_ice_thickness: its own thickness, else Hʳ
    double Hf = own ? H : Hr;
    bool calves = (gfrac > 0) && (H > 0);
    oH = oR = og = 0.0;
    if (!calves) {
        oH = lH;
        oR = lR;
        return;
    }
    double lHf = 0.0;
    double Hn = H - gfrac * Hf;
    if (Hn > 0) {           // H = H - g Hf, Hʳ = Hf
        oH += lH;
        lHf += -gfrac * lH + lR;
        og += -Hf * lH;
    }
    double a = Hf > 0 ? H / Hf : 0.0;
    if (lres != 0.0 && Hf > 0 && gfrac - a > 0) {   // residual max(g - H / Hf, 0) w
        og += lres * w;
        double la = -lres * w;
        oH += la / Hf;
        lHf += -la * H / (Hf * Hf);
    }
    if (own) oH += lHf; else oR += lHf;
}
}  // namespace

// The reverse of _receive_residual_retreat! (:390-397): the received fraction A / Az removed from the cell after the
// retreat; its λ goes to each neighbour's share.
__global__ void k_calve_rev_receive(FrontAdjointView a) {
    const DevGrid<double>& g = a.f.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    const double* share = calved(a, 5);
    double A = 0;
    for (int d = 0; d < 4; ++d) {
        int x = i + DI(d), y = j + DJ(d);
        A += inactive(g, x, y) ? 0.0 : share[g.c_idx(x, y)];
    }
    double Az = g.Az_cc(i, j);
    double oH, oR, og;
    remove_fraction_reverse(calved(a, 1)[k], calved(a, 2)[k], calved(a, 3)[k], A / Az, a.lam_a[k], a.lam_Hr[k], 0.0, 0.0, oH, oR, og);
    a.lam_b[k] = oH;
    a.lam_d[k] = oR;
    a.lam_c[k] = og / Az;   // λ of the received A
}

// The reverse of _share_residual_retreat! (:379-385) and _retreat_front_cells! (:371-375) of cell c: λ of its residual
// from the neighbours that received its shares, then back through its retreat by its own fraction.
__global__ void k_calve_rev_retreat(FrontAdjointView a) {
    const DevGrid<double>& g = a.f.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    const double* H1 = calved(a, 1);
    int n = 0;
    double lshare = 0.0;
    int seen[4], ns = 0;
    for (int e = 0; e < 4; ++e) {
        int x = i + DI(e), y = j + DJ(e);
        if (inactive(g, x, y)) continue;
        int k = g.c_idx(x, y);
        n += H1[k] > 0 ? 1 : 0;
        bool dup = false;
        for (int q = 0; q < ns; ++q) dup |= seen[q] == k;
        if (dup) continue;
        seen[ns++] = k;
        int kx = g.cx(x), ky = g.cy(y), reads = 0;
        for (int d = 0; d < 4; ++d) {
            int na = kx + DI(d), nb = ky + DJ(d);
            if (!inactive(g, na, nb) && g.c_idx(na, nb) == c) ++reads;
        }
        lshare += reads * a.lam_c[k];
    }
    double lres = n > 0 ? lshare / (double)n : 0.0;   // share = residual / n over the neighbours holding ice
    double w = removal_law(a.f.law) ? 0.0 : g.Az_cc(i, j);
    double oH, oR, og;
    remove_fraction_reverse(level(a, a.passes, 0)[c], level(a, a.passes, 1)[c], level(a, a.passes, 2)[c], calved(a, 0)[c],
                            a.lam_b[c], a.lam_d[c], lres, w, oH, oR, og);
    a.lam_a[c] = oH;
    a.lam_Hr[c] = oR;
    a.lam_e[c] = og;   // λ of the retreat fraction
}

// The reverse of _compute_retreat_fraction! (:311-322) for the rate laws: r = min(1, c Δt l / Az) gives λ of the cell's
// rate as used (its own, or a partial cell's mean of its full neighbours') and of its front length.
__global__ void k_calve_rev_fraction(FrontAdjointView a) {
    FrontView v = a.f;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    v.H = const_cast<double*>(level(a, a.passes, 0));
    v.mu = const_cast<double*>(level(a, a.passes, 1));
    v.Hr = const_cast<double*>(level(a, a.passes, 2));
    double lc = 0.0, ll = 0.0;
    FrontLength f = front_lengths(v, i, j);
    double lr = a.lam_e[k];
    if (rate_law(v.law) && v.H[k] > 0 && f.facing && lr != 0.0) {
        Seed none{-1, -1};
        double c;
        if (v.mu[k] > 0) {
            c = dcalving_rate(v, i, j, none).v;
        } else {
            double S = 0;
            int n = 0;
            for (int d = 0; d < 4; ++d)
                if (full_neighbor(g, v.mu, i + DI(d), j + DJ(d))) { S += dcalving_rate(v, i + DI(d), j + DJ(d), none).v; ++n; }
            c = S / (double)(n > 1 ? n : 1);
        }
        double l = dfront_length(v, i, j, f, none).v;
        if (c * a.dt * l / g.Az_cc(i, j) < 1.0) {
            double lcl = lr * a.dt / g.Az_cc(i, j);
            lc = lcl * l;
            ll = lcl * c;
        }
    }
    a.lam_f[k] = lc;
    a.lam_h[k] = ll;
}

// λ of each cell's computed rate: its own use when full, and its share in the partial neighbours' means.
__global__ void k_calve_rev_rate(FrontAdjointView a) {
    const DevGrid<double>& g = a.f.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    const double* mu = level(a, a.passes, 1);
    double acc = 0.0;
    if (mu[k] > 0) {
        acc = a.lam_f[k];
        int seen[4], ns = 0;
        for (int e = 0; e < 4; ++e) {
            int x = i + DI(e), y = j + DJ(e);
            if (inactive(g, x, y)) continue;
            int p = g.c_idx(x, y);
            bool dup = false;
            for (int q = 0; q < ns; ++q) dup |= seen[q] == p;
            if (dup || mu[p] > 0 || a.lam_f[p] == 0.0) continue;
            seen[ns++] = p;
            int px = g.cx(x), py = g.cy(y), n = 0, reads = 0;
            for (int d = 0; d < 4; ++d) {
                int na = px + DI(d), nb = py + DJ(d);
                if (full_neighbor(g, mu, na, nb)) {
                    ++n;
                    if (g.c_idx(na, nb) == k) ++reads;
                }
            }
            if (n > 0) acc += reads * a.lam_f[p] / (double)n;
        }
    }
    a.lam_g[k] = acc;
}

// λ of the face velocities: per face, every cell whose rate or front length reads it (cells within one column and
// row of the face), each differentiated along that face.  The front-velocity law's (1 - φ) sends λ to φ too; the von
// Mises rate sends λ to the cell's own H and η̄H (through η = η̄H / H) and to φ (through σᵐᵃˣ).
__global__ void k_calve_rev_velocity(FrontAdjointView a) {
    FrontView v = a.f;
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    v.H = const_cast<double*>(level(a, a.passes, 0));
    v.mu = const_cast<double*>(level(a, a.passes, 1));
    v.Hr = const_cast<double*>(level(a, a.passes, 2));
    double2 out = a.lam_x[k];
    for (int comp = 0; comp < 2; ++comp) {
        bool has = comp == 0 ? (j < g.Ny && (i < g.Nx || !g.px)) : (i < g.Nx && (j < g.Ny || !g.py));
        if (!has) continue;
        Seed sd{comp == 0 ? k : -1, comp == 1 ? k : -1};
        int ilo = comp == 0 ? i - 1 : i - 1, ihi = comp == 0 ? i : i + 1;
        int jlo = comp == 0 ? j - 1 : j - 1, jhi = comp == 0 ? j + 1 : j;
        double acc = 0.0;
        int seen[9], ns = 0;
        for (int y = jlo; y <= jhi; ++y)
            for (int x = ilo; x <= ihi; ++x) {
                if (inactive(g, x, y)) continue;
                int c = g.c_idx(x, y);
                bool dup = false;
                for (int q = 0; q < ns; ++q) dup |= seen[q] == c;
                if (dup) continue;
                seen[ns++] = c;
                int cx = g.cx(x), cy = g.cy(y);
                if (a.lam_g[c] != 0.0) acc += a.lam_g[c] * dcalving_rate(v, cx, cy, sd).d;
                if (a.lam_h[c] != 0.0) {
                    FrontLength f = front_lengths(v, cx, cy);
                    acc += a.lam_h[c] * dfront_length(v, cx, cy, f, sd).d;
                }
            }
        if (comp == 0) out.x += acc; else out.y += acc;
    }
    a.lam_x[k] = out;
    // φ of the front-velocity law, per cell (each cell once)
    if (v.law == NK_CALVING_FRONT_VELOCITY && i < g.Nx && j < g.Ny && a.lam_g[k] != 0.0) {
        Seed none{-1, -1};
        double c1 = 1 - v.phi[k];
        double c = dcalving_rate(v, i, j, none).v;
        if (c1 > 0) a.lam_phi[k] += -a.lam_g[k] * c / c1;
        else {
            // (1 - φ) = 0: the rate's φ derivative is −max(fs − v_f, 0), recomputed
            Dual ut = dmax(dabs(dmu_u(v, i, j, none)), dabs(dmu_u(v, i + 1, j, none)));
            Dual vt = dmax(dabs(dmu_v(v, i, j, none)), dabs(dmu_v(v, i, j + 1, none)));
            double e = v.eps0 * g.dxc[i];
            double fs = sqrt(ut.v * ut.v + vt.v * vt.v + e * e);
            a.lam_phi[k] += -a.lam_g[k] * fmax(fs - v.front_velocity, 0.0);
        }
    }
    if (v.law == NK_CALVING_VON_MISES && i < g.Nx && j < g.Ny) {
        double lg = a.lam_g[k], le = 0.0;
        if (lg != 0.0) {
            Seed none{-1, -1};
            double Hi = v.H[k], etaH = v.coef[k].x;
            double unit = dvon_mises_rate(v, i, j, none, 1.0).v;   // ∂c/∂η
            double Hd = Hi > 0 ? Hi : 1.0;
            le = lg * unit / Hd;
            if (Hi > 0) a.lam_a[k] += -lg * unit * etaH / (Hi * Hi);
            double smax = v.phi[k] * v.stress_threshold + (1 - v.phi[k]) * v.floating_stress_threshold;
            double c = dvon_mises_rate(v, i, j, none, etaH / Hd).v;
            a.lam_phi[k] += -lg * c * (v.stress_threshold - v.floating_stress_threshold) / smax;
        }
        if (a.lam_eta) a.lam_eta[k] = le;
    }
}

void launch_front_adjoint(const FrontAdjointView& a, cudaStream_t s) {
    LaunchDims d = dims2d(a.f.g.Nx, a.f.g.Ny);
    k_front_rev_force<<<d.grid, d.block, 0, s>>>(a); count_launch();
    if (a.f.law != NK_CALVING_NONE) {
        LaunchDims df = dims2d(a.f.g.Nx + 1, a.f.g.Ny + 1);
        k_calve_rev_receive<<<d.grid, d.block, 0, s>>>(a); count_launch();
        k_calve_rev_retreat<<<d.grid, d.block, 0, s>>>(a); count_launch();
        k_calve_rev_fraction<<<d.grid, d.block, 0, s>>>(a); count_launch();
        k_calve_rev_rate<<<d.grid, d.block, 0, s>>>(a); count_launch();
        k_calve_rev_velocity<<<df.grid, df.block, 0, s>>>(a); count_launch();
    }
    for (int p = a.passes - 1; p >= 0; --p) {
        k_front_rev_receive<<<d.grid, d.block, 0, s>>>(a, p); count_launch();
        k_front_rev_fill<<<d.grid, d.block, 0, s>>>(a, p); count_launch();
    }
    k_front_rev_reference<<<d.grid, d.block, 0, s>>>(a); count_launch();
    k_front_rev_gather<<<d.grid, d.block, 0, s>>>(a); count_launch();
}

}  // namespace nk
