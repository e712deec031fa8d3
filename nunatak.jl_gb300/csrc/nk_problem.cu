// nk_problem.cu — host side of libnunatak_gb300: problem object, device memory, solver drivers and the
// C ABI of include/nunatak_gb300.h.
//
// One nk_problem owns one device arena (a single cudaMalloc) holding every field, coefficient record,
// solver vector and multigrid level of its grid, and one CUDA stream on which every call is ordered.
// Conjugate gradients run without host synchronisation inside a solve: the host issues steps in
// batches and reads the device stopping flag once per batch.  Picard reads two device norms per
// iteration.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "nk_kernels.cuh"

namespace nk {

// ---- error handling ---------------------------------------------------------------------------------------
struct Failure {
    nk_status status;
    std::string message;
};
#define NK_CUDA(call)                                                                                      \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            throw ::nk::Failure{e_ == cudaErrorMemoryAllocation ? NK_OOM : NK_CUDA_ERROR,                  \
                                std::string(#call) + ": " + cudaGetErrorString(e_)};                       \
    } while (0)
#define NK_CHECK_LAUNCH() NK_CUDA(cudaGetLastError())

static void bad(const std::string& m) { throw Failure{NK_BAD_ARGUMENT, m}; }

// Rows per warp of the column-marching kernels: NK_STRIP_ROWS (1, 2, 4 or 8) when set, else 2 for FP32
// (56 registers: the memory-bound sweeps want occupancy; the 2048x1024 sweep takes 36.9 us against 41.6 us at 4
// rows, and the serving stream is unchanged) and, for FP64, 4 from 2^18 cells (the FP64 kernels are bound by
// the FP64 pipe; the two extra rows of each walk are a smaller share at 4).
// Walk lengths measured by the strip autotuner, per (kernel kind, Nx, Ny, element bytes), shared by every
// problem of the process.
static std::mutex& tuned_mutex() {
    static std::mutex m;
    return m;
}
static std::map<std::tuple<int, int, int, int>, int>& tuned_rows() {
    static std::map<std::tuple<int, int, int, int>, int> t;
    return t;
}

int strip_rows(int nx, int ny, int elem_bytes, int kind) {
    static const int forced = [] {
        const char* e = std::getenv("NK_STRIP_ROWS");
        int r = e ? std::atoi(e) : 0;
        return (r == 1 || r == 2 || r == 4 || r == 8) ? r : 0;
    }();
    if (forced) return elem_bytes == 8 ? std::min(forced, 4) : forced;
    if (kind != STRIP_OPERATOR) {
        std::lock_guard<std::mutex> g(tuned_mutex());
        auto it = tuned_rows().find(std::make_tuple(kind, nx, ny, elem_bytes));
        if (it != tuned_rows().end()) return it->second;
    }
    long long cells = (long long)nx * ny;
    // FP64 multigrid sweeps and residuals: what the autotuner measured for one solve at a time on GB300 (one row
    // below 2^16 cells, two above; 1.48 -> 1.68 solves/s on the FP64 stream); FP32 and the FP64 operator kernels
    // keep two rows (four from 2^18 cells for the operator), which the concurrent mixed stream prefers
    if (elem_bytes == 8 && kind != STRIP_OPERATOR) return cells < (1 << 16) ? 1 : 2;
    if (elem_bytes == 8) return cells >= (1 << 18) ? 4 : 2;
    return 2;
}

// ---- grid axis: Oceananigans generate_coordinate with halo nodes ----------------------------------------------
// Regular axes use the single spacing L / N; face vectors extend the edge spacing into the halo (Bounded)
// or wrap (Periodic); centres are face midpoints; Δᶜ(i) = F(i+1) - F(i), Δᶠ(i) = C(i) - C(i-1).
struct HostAxis {
    int N = 0, H = 0;
    bool periodic = false, regular = true;
    double delta = 0;
    int lo = 0;
    std::vector<double> F, C, dC, dF;
    int at(int i) const { return i - lo; }
    double face(int i) const { return F[at(i)]; }

    void build_regular(int n, int h, bool per, double x0, double L) {
        N = n; H = h; periodic = per; regular = true; delta = L / n;
        lo = -H - 3;                     // two nodes beyond the halo: the metric arrays read indices -1 .. N + 3
        int count = N + 2 * H + 8;
        F.assign(count, 0); C.assign(count, 0); dC.assign(count, delta); dF.assign(count, delta);
        for (int i = lo; i < lo + count; ++i) {
            F[at(i)] = x0 + ((i - 1) * L) / N;
            C[at(i)] = x0 + ((i - 1) * L) / N + delta / 2;
        }
    }
    void build_faces(int n, int h, bool per, const double* faces) {
        N = n; H = h; periodic = per; regular = false; delta = 0;
        lo = -H - 3;
        int count = N + 2 * H + 8;
        F.assign(count, 0); C.assign(count, 0); dC.assign(count, 0); dF.assign(count, 0);
        for (int i = 1; i <= N + 1; ++i) F[at(i)] = faces[i - 1];
        if (per) {
            double L = faces[N] - faces[0];
            for (int m = 1; at(1 - m) >= 0; ++m) F[at(1 - m)] = F[at(N + 1 - m)] - L;
            for (int m = 1; at(N + 1 + m) < count; ++m) F[at(N + 1 + m)] = F[at(1 + m)] + L;
        } else {
            double dm = faces[1] - faces[0], dp = faces[N] - faces[N - 1];
            for (int m = 1; at(1 - m) >= 0; ++m) F[at(1 - m)] = faces[0] - m * dm;
            for (int m = 1; at(N + 1 + m) < count; ++m) F[at(N + 1 + m)] = faces[N] + m * dp;
        }
        for (int i = lo; i < lo + count - 1; ++i) {
            C[at(i)] = (F[at(i + 1)] + F[at(i)]) / 2;
            dC[at(i)] = F[at(i + 1)] - F[at(i)];
        }
        for (int i = lo + 1; i < lo + count - 1; ++i) dF[at(i)] = C[at(i)] - C[at(i - 1)];
    }
    // 1-based Oceananigans index ↔ 0-based device index i - 1
    double dc(int i1) const { return regular ? delta : dC[at(i1)]; }
    double df(int i1) const { return regular ? delta : dF[at(i1)]; }
};

// coarsening(N, H, minimum_coarse_size), multigrid_preconditioner.jl:86
static int coarsening(int N, int H, int minimum) { return ((N % 2 == 0) && (N / 2 >= std::max(minimum, H))) ? 2 : 1; }

constexpr int METRIC_PAD = 2;   // metric arrays hold device indices -2 .. N + 2

// ---- device arena -------------------------------------------------------------------------------------------
struct Arena {
    char* base = nullptr;
    size_t size = 0;
    std::vector<std::pair<void**, size_t>> pending;
    size_t reserve(size_t bytes) { size_t off = size; size = (size + bytes + 255) & ~size_t(255); return off; }
};

template <typename T>
struct Level {
    int Nx = 0, Ny = 0, pitch = 0, cx = 1, cy = 1;
    HostAxis ax, ay;
    T* metrics = nullptr;                // 8 arrays of (N + 2 METRIC_PAD + 2) each
    typename Vec4<T>::type* coef = nullptr;
    uint8_t* mask = nullptr;
    typename Vec2<T>::type* irs = nullptr;
    typename Vec2<T>::type *x = nullptr, *x2 = nullptr, *b = nullptr, *q = nullptr;
    T* t = nullptr;
    DevGrid<T> g{};
    size_t plane() const { return (size_t)(Ny + 1) * pitch; }
};

static int make_pitch(int Nx) { return ((Nx + 1 + 31) / 32) * 32; }

template <typename T>
static void metric_host(const HostAxis& ax, int n, std::vector<T>& out_c, std::vector<T>& out_f) {
    // device index d ∈ [-PAD, n + PAD] ↔ Oceananigans index d + 1
    int len = n + 2 * METRIC_PAD + 2;
    out_c.assign(len, T(0));
    out_f.assign(len, T(0));
    for (int d = -METRIC_PAD; d <= n + METRIC_PAD; ++d) {
        out_c[d + METRIC_PAD] = (T)ax.dc(d + 1);
        out_f[d + METRIC_PAD] = (T)ax.df(d + 1);
    }
}

}  // namespace nk

using namespace nk;

struct nk_problem {
    nk_context* ctx = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    nk_grid_desc gd{};
    nk_physics_desc pd{};
    nk_solver_desc sd{};
    int Nx = 0, Ny = 0, pitch = 0, Ns = 1;
    bool px = false, py = false;
    size_t plane = 0;
    bool mixed = false;
    int precond = NK_PRECONDITIONER_DIAGONAL;

    Arena arena;
    bool external_arena = false;              // arena.base sub-allocated by a server (not cudaMalloc'd here)
    bool external_pinned = false;             // sc_host sub-allocated from a server's pinned pool
    bool external_stream = false;             // `stream` belongs to a batch (nk_batch) shared by its slots
    // fine level (FP64)
    Level<double> fine;                         // metrics, coef, mask, irs (multigrid FP64), x2, q, t
    double *H = nullptr, *bed = nullptr, *s = nullptr, *N = nullptr, *mu = nullptr, *phi = nullptr, *C = nullptr, *F2 = nullptr, *A2 = nullptr;
    double *A3 = nullptr, *T = nullptr, *eta_sigma = nullptr;
    double2 *phi_uv = nullptr, *tau = nullptr, *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *xprev = nullptr,
            *zold = nullptr, *invd = nullptr, *bb = nullptr, *ub = nullptr, *usig = nullptr, *tmp_a = nullptr, *tmp_b = nullptr;
    double* staging = nullptr;
    size_t staging_count = 0;
    double2* partials = nullptr;
    SolverScalars* sc = nullptr;
    SolverScalars* sc_host = nullptr;          // pinned mirror
    double* sig_tables = nullptr;              // dz, w2, zc (Ns each) + w1 (Ns * Ns) + zf (Ns + 1)
    double* rate_params = nullptr;             // 9 (nk_compute_rate_factor) or 14 (nk_thermal_params)
    double* thermal = nullptr;                 // enthalpy then water fraction (Ns planes each), allocated on first use
    double* transport = nullptr;               // a, m, mᵍ, clipped thickness, then H at the step's and the stage's start
    double* energy = nullptr;                  // H_w, G, T_s, T_o, Hⁿ, s_b, qᵍ, then Φ and the step-start E (Ns planes each)
    // the thickness advection of nk_step_thickness: the reference's default for the SSA and the DIVA,
    // WENO(order = 5, bounds = (0, 1e5)) (default_thickness_advection, src/Models/ice_sheet_model.jl:123)
    nk_advection_desc advection{NK_ADVECTION_WENO, 5, 1, 0, 0.0, 1e5};
    // a partial-cell front (nk_set_front): its settings and planes (ensure_front)
    nk_front_desc front{0, 4, NK_CALVING_NONE, 0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double* front_buf = nullptr;
    // a till (nk_set_till): N from the basal water, and its drainage in the energy step
    nk_till_desc till{0, 0, 1000.0, 0.02, 0.69, 0.12, 2.0, 0.0};
    std::vector<double> sig_dz, sig_w2, sig_zc, sig_w1, sig_zf;

    // coarse levels
    std::vector<Level<double>> lv64;           // FP64 hierarchy: [0] is the fine grid view
    std::vector<Level<float>> lv32;            // FP32 hierarchy (mixed): [0] is a float copy of the fine grid
    int nlevels = 0;                           // coarse levels below the fine grid
    cudaGraph_t picard_graph = nullptr, linear_graph = nullptr;
    cudaGraphExec_t picard_exec = nullptr, linear_exec = nullptr;
    long long picard_kernels[3] = {0, 0, 0};   // kernel nodes: top level, Picard body, CG body
    long long linear_kernels[2] = {0, 0};      // kernel nodes: top level, CG body
    bool async_pending = false;                // nk_picard_solve_async issued, nk_problem_wait not yet called
    bool strips_tuned = false;                 // the strip autotuner has seen this problem's levels
    double instantiate_s = 0;                  // host seconds of the last graph instantiation
    // Picard adjoint scratch, allocated by the first nk_picard_adjoint: ∂J/∂x (pairs), the strain-rate adjoint
    // per centre and the log C gradient per cell
    void* adj_base = nullptr;
    double2* adj_xbar = nullptr;
    double* adj_g = nullptr;
    double* adj_grad = nullptr;
    double* adj_grad_A = nullptr;                // Nσ planes (the first alone for a 2-D rate factor)
    // DIVA adjoint scratch (first DIVA nk_picard_adjoint): 8 pair planes (cbar, bbar, txbar, σ βᵇ, Ū, ūᵇ part,
    // ℑF₂⁻ adjoint, β̄ᵇ), σ F₂ and σ ησ (Nσ planes)
    void* adj_diva = nullptr;
    double2* adj_hmu = nullptr;                  // DIVA thickness gradient: (∂J/∂H via η̄H and F₂, ∂J/∂μ) per centre
    // Prescribed velocities (u_D, v_D) per face, NaN where free; allocated by the first set of either prescribed
    // field.  Its faces become identity rows whose values enter their neighbours' strain rates.
    double2* ud = nullptr;

    // ---- views ---------------------------------------------------------------------------------------------
    OpView<double> fine_op() const {
        OpView<double> o;
        o.g = fine.g;
        o.coef = fine.coef;
        o.mask = fine.mask;
        o.wall_factor = pd.side_walls == NK_NO_SLIP ? 2.0 : 0.0;
        return o;
    }
    SigmaTable sigma_table() const {
        SigmaTable t;
        t.N = Ns;
        t.dz = sig_tables;
        t.w2 = sig_tables + Ns;
        t.zc = sig_tables + 2 * Ns;
        t.w1 = sig_tables + 3 * Ns;
        t.zf = sig_tables + 3 * Ns + (size_t)Ns * Ns;
        return t;
    }
    PhysView phys() const {
        PhysView ph;
        ph.g = fine.g;
        ph.sig = sigma_table();
        ph.n = pd.glen_exponent;
        ph.eps0 = pd.strain_rate_regularization;
        ph.wall_factor = pd.side_walls == NK_NO_SLIP ? 2.0 : 0.0;
        ph.friction = pd.friction;
        ph.m = pd.friction_exponent;
        ph.alpha2 = pd.coulomb_coefficient;
        ph.u0 = pd.velocity_regularization;
        ph.rate_sigma = pd.rate_factor_layout == NK_RATE_FACTOR_SIGMA;
        ph.plane = (int)plane;
        ph.A = ph.rate_sigma ? A3 : A2;
        ph.H = H;
        ph.C = C;
        ph.N = N;
        ph.mu = mu;
        ph.phi = phi_uv;
        ph.use_mask = pd.use_ice_mask;
        ph.use_N = pd.use_effective_pressure;
        ph.ud = ud;
        return ph;
    }
    template <typename TT>
    LevelView<TT> level_view(Level<TT>& L) const {
        LevelView<TT> v;
        v.o.g = L.g;
        v.o.coef = L.coef;
        v.o.mask = L.mask;
        v.o.wall_factor = pd.side_walls == NK_NO_SLIP ? TT(2) : TT(0);
        v.x = L.x; v.x2 = L.x2; v.b = L.b; v.q = L.q; v.t = L.t; v.irs = L.irs;
        v.cx = L.cx; v.cy = L.cy;
        return v;
    }
    CGView cg_view(const double2* b) const {
        CGView v;
        v.o = fine_op();
        v.x = x; v.b = b; v.r = r; v.z = z; v.p = p; v.q = q;
        v.zold = nullptr;
        v.invd = invd;
        v.precond = precond;
        v.sc = sc;
        v.partials = partials;
        v.cond = 0;
        bool fused = mixed && precond == NK_PRECONDITIONER_MULTIGRID;
        v.r32 = fused ? lv32[0].b : nullptr;
        v.z32 = fused ? lv32[0].x : nullptr;
        v.zold32 = fused ? reinterpret_cast<float2*>(zold) : nullptr;   // flexible CG: z_old in FP32
        return v;
    }
};

namespace nk {

// ---- construction ---------------------------------------------------------------------------------------------
template <typename T>
static void setup_level_grid(Level<T>& L) {
    L.pitch = make_pitch(L.Nx);
    L.g.Nx = L.Nx;
    L.g.Ny = L.Ny;
    L.g.pitch = L.pitch;
    L.g.px = L.ax.periodic;
    L.g.py = L.ay.periodic;
}

template <typename T>
static size_t metric_len(const Level<T>& L, int axis) { return (size_t)((axis == 0 ? L.Nx : L.Ny) + 2 * METRIC_PAD + 2); }

template <typename T>
static void reserve_level(Arena& A, Level<T>& L, std::vector<std::pair<void**, size_t>>& slots, bool own_coef, bool own_xb) {
    size_t pl = L.plane();
    size_t mlen = 4 * (metric_len(L, 0) + metric_len(L, 1));
    slots.push_back({(void**)&L.metrics, A.reserve(mlen * sizeof(T))});
    if (own_coef) {
        slots.push_back({(void**)&L.coef, A.reserve(pl * sizeof(typename Vec4<T>::type))});
        slots.push_back({(void**)&L.mask, A.reserve(pl)});
    }
    slots.push_back({(void**)&L.irs, A.reserve(pl * sizeof(typename Vec2<T>::type))});
    if (own_xb) {
        slots.push_back({(void**)&L.x, A.reserve(pl * sizeof(typename Vec2<T>::type))});
        slots.push_back({(void**)&L.b, A.reserve(pl * sizeof(typename Vec2<T>::type))});
    }
    slots.push_back({(void**)&L.x2, A.reserve(pl * sizeof(typename Vec2<T>::type))});
    slots.push_back({(void**)&L.q, A.reserve(pl * sizeof(typename Vec2<T>::type))});
    slots.push_back({(void**)&L.t, A.reserve(pl * sizeof(T))});
}

template <typename T>
static void upload_metrics(Level<T>& L, cudaStream_t s) {
    std::vector<T> xc, xf, yc, yf;
    metric_host<T>(L.ax, L.Nx, xc, xf);
    metric_host<T>(L.ay, L.Ny, yc, yf);
    size_t nx = xc.size(), ny = yc.size();
    std::vector<T> host;
    host.reserve(4 * (nx + ny));
    auto add = [&](const std::vector<T>& v) { host.insert(host.end(), v.begin(), v.end()); };
    auto inv = [](std::vector<T> v) { for (auto& e : v) e = T(1) / e; return v; };
    add(xc); add(xf); add(yc); add(yf); add(inv(xc)); add(inv(xf)); add(inv(yc)); add(inv(yf));
    NK_CUDA(cudaMemcpyAsync(L.metrics, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    NK_CUDA(cudaStreamSynchronize(s));   // host vector goes out of scope
    bool uniform = true;   // over the filled entries (metric_host leaves the last one of each array at zero)
    for (const auto* v : {&xc, &xf, &yc, &yf})
        for (size_t q = 0; q + 1 < v->size(); ++q) uniform = uniform && (*v)[q] == xc[0];
    L.g.h = uniform ? xc[0] : T(0);
    T* m = L.metrics;
    L.g.dxc = m + METRIC_PAD; m += nx;
    L.g.dxf = m + METRIC_PAD; m += nx;
    L.g.dyc = m + METRIC_PAD; m += ny;
    L.g.dyf = m + METRIC_PAD; m += ny;
    L.g.rdxc = m + METRIC_PAD; m += nx;
    L.g.rdxf = m + METRIC_PAD; m += nx;
    L.g.rdyc = m + METRIC_PAD; m += ny;
    L.g.rdyf = m + METRIC_PAD;
}

// Exact integral of (1 - ζ)^p, column_integrals.jl:1-2
static double ipow(double x, int n) { double r = x; for (int m = 1; m < n; ++m) r *= x; return r; }
static double power_integral(double zm, double zp, int p) { return (ipow(1 - zm, p + 1) - ipow(1 - zp, p + 1)) / (p + 1); }

static void build(nk_problem* P, bool dry = false) {
    const nk_grid_desc& gd = P->gd;
    P->Nx = gd.Nx; P->Ny = gd.Ny; P->Ns = gd.Nsigma;
    P->px = gd.topology_x == NK_PERIODIC; P->py = gd.topology_y == NK_PERIODIC;
    P->mixed = P->sd.precision == NK_PRECISION_MIXED;
    P->precond = P->sd.preconditioner;
    Level<double>& F = P->fine;
    F.Nx = P->Nx; F.Ny = P->Ny;
    if (gd.x_faces) F.ax.build_faces(gd.Nx, gd.halo_x, P->px, gd.x_faces); else F.ax.build_regular(gd.Nx, gd.halo_x, P->px, gd.x0, gd.Lx);
    if (gd.y_faces) F.ay.build_faces(gd.Ny, gd.halo_y, P->py, gd.y_faces); else F.ay.build_regular(gd.Ny, gd.halo_y, P->py, gd.y0, gd.Ly);
    setup_level_grid(F);
    P->pitch = F.pitch;
    P->plane = F.plane();

    // sigma tables
    std::vector<double> faces(P->Ns + 1);
    for (int k = 0; k <= P->Ns; ++k) faces[k] = gd.sigma_faces ? gd.sigma_faces[k] : std::pow((double)k / P->Ns, gd.bed_refinement);
    auto zf = [&](int k1) { return faces[k1 - 1]; };                      // znode(k, Face), 1-based
    auto zc = [&](int k1) { return (faces[k1 - 1] + faces[k1]) / 2; };   // znode(k, Center)
    P->sig_dz.resize(P->Ns); P->sig_w2.resize(P->Ns); P->sig_zc.resize(P->Ns); P->sig_w1.assign((size_t)P->Ns * P->Ns, 0.0);
    P->sig_zf = faces;
    for (int k = 1; k <= P->Ns; ++k) {
        P->sig_dz[k - 1] = zf(k + 1) - zf(k);
        P->sig_w2[k - 1] = power_integral(zf(k), zf(k + 1), 2);
        P->sig_zc[k - 1] = zc(k);
        for (int kp = 1; kp <= k; ++kp) {
            double zp = (kp == k) ? zc(k) : zf(kp + 1);
            P->sig_w1[(size_t)(k - 1) * P->Ns + (kp - 1)] = power_integral(zf(kp), zp, 1);
        }
    }

    // multigrid levels (coarse_levels, multigrid_preconditioner.jl:88-120)
    if (P->precond == NK_PRECONDITIONER_MULTIGRID) {
        int minimum = P->sd.minimum_coarse_size;
        const HostAxis* fax = &F.ax;
        const HostAxis* fay = &F.ay;
        int nx = F.Nx, ny = F.Ny;
        std::vector<std::pair<HostAxis, HostAxis>> axes;
        std::vector<std::pair<int, int>> factors;
        while (true) {
            int cx = coarsening(nx, fax->H, minimum), cy = coarsening(ny, fay->H, minimum);
            if (cx == 1 && cy == 1) break;
            std::vector<double> xf, yf;
            for (int i = 1; i <= nx + 1; i += cx) xf.push_back(fax->face(i));
            for (int j = 1; j <= ny + 1; j += cy) yf.push_back(fay->face(j));
            HostAxis a, b;
            a.build_faces(nx / cx, fax->H, fax->periodic, xf.data());
            b.build_faces(ny / cy, fay->H, fay->periodic, yf.data());
            axes.push_back({a, b});
            factors.push_back({cx, cy});
            nx /= cx; ny /= cy;
            fax = &axes.back().first;   // push_back may have moved the stored axes
            fay = &axes.back().second;
        }
        P->nlevels = (int)axes.size();
        auto fill_levels = [&](auto& lv) {
            using LT = typename std::decay<decltype(lv[0])>::type;
            lv.resize(P->nlevels + 1);
            LT& L0 = lv[0];
            L0.Nx = F.Nx; L0.Ny = F.Ny; L0.ax = F.ax; L0.ay = F.ay;
            setup_level_grid(L0);
            for (int l = 1; l <= P->nlevels; ++l) {
                LT& L = lv[l];
                L.ax = axes[l - 1].first; L.ay = axes[l - 1].second;
                L.Nx = L.ax.N; L.Ny = L.ay.N;
                L.cx = factors[l - 1].first; L.cy = factors[l - 1].second;
                setup_level_grid(L);
            }
        };
        if (P->mixed) fill_levels(P->lv32); else fill_levels(P->lv64);
    }

    // arena
    Arena& A = P->arena;
    std::vector<std::pair<void**, size_t>> slots;
    size_t pl = P->plane;
    size_t d1 = pl * sizeof(double), d2 = pl * sizeof(double2);
    size_t mlen = 4 * (metric_len(F, 0) + metric_len(F, 1));
    slots.push_back({(void**)&F.metrics, A.reserve(mlen * sizeof(double))});
    slots.push_back({(void**)&F.coef, A.reserve(pl * sizeof(double4))});
    slots.push_back({(void**)&F.mask, A.reserve(pl)});
    for (double** f : {&P->H, &P->bed, &P->s, &P->N, &P->mu, &P->phi, &P->C, &P->F2, &P->A2}) slots.push_back({(void**)f, A.reserve(d1)});
    for (double2** f : {&P->phi_uv, &P->tau, &P->x, &P->r, &P->z, &P->p, &P->q, &P->xprev, &P->zold, &P->invd, &P->bb, &P->ub,
                        &P->tmp_a, &P->tmp_b})
        slots.push_back({(void**)f, A.reserve(d2)});
    slots.push_back({(void**)&P->eta_sigma, A.reserve(d1 * P->Ns)});
    if (P->pd.rate_factor_layout == NK_RATE_FACTOR_SIGMA) {
        slots.push_back({(void**)&P->A3, A.reserve(d1 * P->Ns)});
        slots.push_back({(void**)&P->T, A.reserve(d1 * P->Ns)});
    }
    slots.push_back({(void**)&P->usig, A.reserve(d2 * P->Ns)});
    P->staging_count = (size_t)(P->Nx + 1) * (P->Ny + 1) * P->Ns;
    slots.push_back({(void**)&P->staging, A.reserve(P->staging_count * sizeof(double))});
    LaunchDims big = dims2d(P->Nx + 1, P->Ny + 1), strips = strip_dims(P->Nx, P->Ny, STRIP_MIN_ROWS);
    size_t nblocks = std::max((size_t)big.grid.x * big.grid.y, (size_t)strips.grid.x * strips.grid.y);
    slots.push_back({(void**)&P->partials, A.reserve(nblocks * sizeof(double2))});
    slots.push_back({(void**)&P->sc, A.reserve(sizeof(SolverScalars))});
    slots.push_back({(void**)&P->sig_tables, A.reserve((4 * P->Ns + 1 + (size_t)P->Ns * P->Ns) * sizeof(double))});
    slots.push_back({(void**)&P->rate_params, A.reserve(16 * sizeof(double))});
    if (P->precond == NK_PRECONDITIONER_MULTIGRID) {
        if (P->mixed) {
            for (int l = 0; l <= P->nlevels; ++l) reserve_level(A, P->lv32[l], slots, true, true);
        } else {
            // level 0 is the fine grid: coefficients, mask and vectors are the fine ones (x = z, b = r)
            reserve_level(A, P->lv64[0], slots, false, false);
            for (int l = 1; l <= P->nlevels; ++l) reserve_level(A, P->lv64[l], slots, true, true);
        }
    }
    if (dry) return;   // sizing only: A.size is the device footprint
    if (!P->external_arena) NK_CUDA(cudaMalloc((void**)&A.base, A.size));
    NK_CUDA(cudaMemsetAsync(A.base, 0, A.size, P->stream));
    for (auto& sl : slots) *sl.first = A.base + sl.second;

    upload_metrics(F, P->stream);
    std::vector<double> tables;
    tables.insert(tables.end(), P->sig_dz.begin(), P->sig_dz.end());
    tables.insert(tables.end(), P->sig_w2.begin(), P->sig_w2.end());
    tables.insert(tables.end(), P->sig_zc.begin(), P->sig_zc.end());
    tables.insert(tables.end(), P->sig_w1.begin(), P->sig_w1.end());
    tables.insert(tables.end(), P->sig_zf.begin(), P->sig_zf.end());
    NK_CUDA(cudaMemcpyAsync(P->sig_tables, tables.data(), tables.size() * sizeof(double), cudaMemcpyHostToDevice, P->stream));
    NK_CUDA(cudaStreamSynchronize(P->stream));
    if (P->precond == NK_PRECONDITIONER_MULTIGRID) {
        if (P->mixed) {
            for (int l = 0; l <= P->nlevels; ++l) upload_metrics(P->lv32[l], P->stream);
            P->lv32[0].mask = F.mask;   // level 0 shares the fine mask (computed from the FP64 η̄H)
        } else {
            Level<double>& L0 = P->lv64[0];
            L0.metrics = F.metrics; L0.g = F.g; L0.coef = F.coef; L0.mask = F.mask; L0.x = P->z; L0.b = P->r;
            for (int l = 1; l <= P->nlevels; ++l) upload_metrics(P->lv64[l], P->stream);
        }
    }
    if (!P->external_pinned) NK_CUDA(cudaHostAlloc((void**)&P->sc_host, sizeof(SolverScalars), cudaHostAllocDefault));
    std::memset(P->sc_host, 0, sizeof(SolverScalars));
}

// ---- coefficient preparation ----------------------------------------------------------------------------------
// Mask (and the Jacobi inverse diagonal) after η̄H, η̄Hᶠᶠ or β changed.
static void prepare_operator(nk_problem* P) {
    OpView<double> o = P->fine_op();
    launch_mask<double>(o, P->fine.mask, P->stream, P->ud);
    if (P->precond == NK_PRECONDITIONER_DIAGONAL) launch_inverse_diagonal(o, P->invd, P->stream);
    NK_CHECK_LAUNCH();
}

// update_preconditioner!: coarse coefficients from the current fine ones, masks and ℓ1 row sums per level.
static void update_preconditioner(nk_problem* P) {
    if (P->precond != NK_PRECONDITIONER_MULTIGRID) return;
    cudaStream_t s = P->stream;
    if (!P->mixed) {
        auto& lv = P->lv64;
        LevelView<double> v0 = P->level_view(lv[0]);
        launch_inverse_row_sum<double>(v0.o, lv[0].irs, s);
        for (int l = 1; l <= P->nlevels; ++l) {
            LevelView<double> v = P->level_view(lv[l]);
            launch_coarsen<double, double>(v, lv[l - 1].g, lv[l - 1].coef, lv[l].coef, s);
            launch_mask<double>(v.o, lv[l].mask, s);
            launch_inverse_row_sum<double>(v.o, lv[l].irs, s);
        }
    } else {
        auto& lv = P->lv32;
        launch_coef_to_float(P->fine.g, P->fine.coef, lv[0].coef, s);
        LevelView<float> v0 = P->level_view(lv[0]);
        launch_inverse_row_sum<float>(v0.o, lv[0].irs, s);
        for (int l = 1; l <= P->nlevels; ++l) {
            LevelView<float> v = P->level_view(lv[l]);
            if (l == 1) launch_coarsen<float, double>(v, P->fine.g, P->fine.coef, lv[1].coef, s);
            else launch_coarsen<float, float>(v, lv[l - 1].g, lv[l - 1].coef, lv[l].coef, s);
            launch_mask<float>(v.o, lv[l].mask, s);
            launch_inverse_row_sum<float>(v.o, lv[l].irs, s);
        }
    }
    NK_CHECK_LAUNCH();
}

// Levels of at most `coarse_cells` cells run inside one thread block (k_coarse_vcycle), FP32 only: one SM's
// FP64 rate is 1/152 of the chip's, so FP64 coarse levels always run as grid-wide kernels.  Tunable with
// NK_COARSE_CELLS (default 0, off: measured on GB300, one SM is slower than grid-wide launches even for the
// 32 x 32 coarsest level with its 20 sweeps).
static int coarse_cells_limit() {
    static int limit = [] {
        const char* e = std::getenv("NK_COARSE_CELLS");
        return e ? std::atoi(e) : 0;
    }();
    return limit;
}

// NK_COARSEST_SMEM=0 runs the coarsest level's sweeps as separate launches instead of one shared-memory block.
static bool coarsest_in_shared_memory() {
    static bool on = [] {
        const char* e = std::getenv("NK_COARSEST_SMEM");
        return !(e && std::atoi(e) == 0);
    }();
    return on;
}

template <typename T>
static int fused_level(const std::vector<Level<T>>& lv, int nlevels) {
    if (sizeof(T) == 8) return nlevels + 1;
    for (int l = 0; l <= nlevels; ++l)
        if ((long long)lv[l].Nx * lv[l].Ny <= coarse_cells_limit()) return l;
    return nlevels + 1;
}

// CUDA graphs are the solve path.  NK_SOLVER_HOST_LOOP in the solver flags (or NK_GRAPHS=0 for the whole
// process) issues the same kernel sequence from a host loop (steps in batches, one read of the device stopping
// flag per batch): profilers cannot see inside graphs with conditional nodes.
static bool use_graphs(const nk_problem* P) {
    static bool on = [] {
        const char* e = std::getenv("NK_GRAPHS");
        return !(e && e[0] == '0');
    }();
    return on && !(P->sd.flags & NK_SOLVER_HOST_LOOP);
}

// Buffer that receives the first of `sweeps` point sweeps started from zero, so that the last lands in L.x.
template <typename T>
static typename Vec2<T>::type* first_sweep_target(Level<T>& L, int sweeps) { return ((sweeps - 1) % 2 == 0) ? L.x : L.x2; }

// smooth!, multigrid_preconditioner.jl:165-174, leaving the result in L.x.  `first`: x starts at zero;
// `first_done`: the first sweep from zero was already written (by the restriction) into first_sweep_target.
template <typename T>
static void smooth(nk_problem* P, Level<T>& L, int sweeps, bool first, const int* done, bool first_done = false) {
    cudaStream_t s = P->stream;
    LevelView<T> v = P->level_view(L);
    if (sweeps <= 0) {
        if (first) launch_zero_vec<T>(L.g, L.x, done, s);
        return;
    }
    if (P->sd.smoother == NK_SMOOTHER_LINE_JACOBI) {
        for (int k = 0; k < sweeps; ++k) {
            bool f = first && k == 0;
            if (!f) launch_level_apply<T>(v, L.x, L.q, 0, done, s);
            launch_line_relax<T>(v, L.x, f ? 1 : 0, done, s);
        }
        return;
    }
    using V2 = typename Vec2<T>::type;
    const V2* in = L.x;
    int k0 = 0;
    if (first && first_done) {
        in = first_sweep_target(L, sweeps);
        k0 = 1;
    } else if (first && sweeps >= 2) {        // sweeps 1 and 2 from zero in one pass
        V2* out = ((sweeps - 2) % 2 == 0) ? L.x : L.x2;
        launch_smooth_first2<T>(v, out, done, s);
        in = out;
        k0 = 2;
    } else if (!first && sweeps % 2 == 1) {   // an odd number of ping-pong sweeps starting from L.x would write L.x in place
        if (batch_slots() > 1) launch_copy_plane<T>(L.g, L.x2, L.x, (int)L.plane(), done, s);
        else cudaMemcpyAsync(L.x2, L.x, L.plane() * sizeof(V2), cudaMemcpyDeviceToDevice, s);
        in = L.x2;
    }
    for (int k = k0; k < sweeps; ++k) {
        V2* out = ((sweeps - 1 - k) % 2 == 0) ? L.x : L.x2;
        launch_smooth_point<T>(v, in, out, (first && k == 0) ? 1 : 0, done, s);
        in = out;
    }
}

// v_cycle!, multigrid_preconditioner.jl:144-163 (x ≈ A⁻¹ b from a zero guess on level l).  Levels from
// `fused_level` down run in one k_coarse_vcycle launch; above it each phase is one grid-wide kernel, and the
// restriction also performs the coarse level's first sweep from zero.
template <typename T>
static void v_cycle(nk_problem* P, std::vector<Level<T>>& lv, int l, const int* done, bool first_done = false) {
    cudaStream_t s = P->stream;
    int lc = fused_level(lv, P->nlevels);
    if (l == lc) {
        CoarseLevels<T> C{};
        C.n = P->nlevels - l + 1;
        if (C.n > MAX_COARSE_LEVELS) bad("too many coarse multigrid levels");
        for (int k = 0; k < C.n; ++k) C.lv[k] = P->level_view(lv[l + k]);
        C.sweeps = P->sd.smoothing_sweeps;
        C.coarsest = P->sd.coarsest_sweeps;
        C.line = P->sd.smoother == NK_SMOOTHER_LINE_JACOBI;
        launch_coarse_vcycle<T>(C, done, s);
        return;
    }
    Level<T>& L = lv[l];
    if (l == P->nlevels) {
        int sweeps = P->sd.coarsest_sweeps;
        LevelView<T> v = P->level_view(L);
        int plane = (int)L.plane();
        if (coarsest_in_shared_memory() && P->sd.smoother == NK_SMOOTHER_POINT_JACOBI && sweeps > 0 &&
            coarsest_smem_fits<T>(v, plane)) {
            if (first_done) launch_coarsest_smem<T>(v, plane, first_sweep_target(L, sweeps), sweeps - 1, 0, L.x, done, s);
            else launch_coarsest_smem<T>(v, plane, nullptr, sweeps, 1, L.x, done, s);
            return;
        }
        smooth(P, L, sweeps, true, done, first_done);
        return;
    }
    smooth(P, L, P->sd.smoothing_sweeps, true, done, first_done);
    LevelView<T> v = P->level_view(L);
    launch_level_apply<T>(v, L.x, L.q, 1, done, s);
    Level<T>& N = lv[l + 1];
    LevelView<T> c = P->level_view(N);
    bool fuse_first = (l + 1 != lc) && P->sd.smoother == NK_SMOOTHER_POINT_JACOBI;
    int next_sweeps = (l + 1 == P->nlevels) ? P->sd.coarsest_sweeps : P->sd.smoothing_sweeps;
    fuse_first = fuse_first && next_sweeps > 0;
    launch_restrict<T>(c, v, L.q, N.b, fuse_first ? first_sweep_target(N, next_sweeps) : nullptr, done, s);
    v_cycle(P, lv, l + 1, done, fuse_first);
    launch_prolongate<T>(v, c, L.x, N.x, done, s);
    smooth(P, L, P->sd.smoothing_sweeps, false, done);
}

// z = M r with the multigrid preconditioner.  `fused`: inside conjugate gradients, where the FP32 copy of r
// and the FP64 copy of the result are made by the CG kernels themselves (CGView::r32 / z32).
static void precondition_mg(nk_problem* P, const int* done, bool fused = false) {
    cudaStream_t s = P->stream;
    if (!P->mixed) {
        v_cycle<double>(P, P->lv64, 0, done);
    } else {
        if (!fused) launch_to_float(P->fine.g, P->r, P->lv32[0].b, done, s);
        v_cycle<float>(P, P->lv32, 0, done);
        if (!fused) launch_to_double(P->fine.g, P->lv32[0].x, P->z, done, s);
    }
    NK_CHECK_LAUNCH();
}

// ---- conjugate gradients and Picard as CUDA graphs ------------------------------------------------------------
// A whole solve is one graph launch.  Picard and conjugate gradients are conditional WHILE nodes whose
// conditions the kernels set on the device (cudaGraphSetConditional) when they take the stopping decision,
// so a solve needs no host round trip until it has finished:
//
//   picard_begin ─► WHILE(picard) { x⁻ = x ─► coefficient update ─► coarse coefficients ─► CG start
//                                    ─► WHILE(cg) { apply ─► update ─► [V-cycle ─► dots] ─► xpby }
//                                    ─► picard_end (Δ, X, stopping test) }
static SolverScalars control_scalars(const nk_problem* P) {
    SolverScalars h{};
    const nk_iteration_control& c = P->sd.linear;
    h.reltol = c.reltol;
    h.abstol = c.abstol;
    h.fixed = c.kind == NK_FIXED_ITERATIONS;
    h.iterations = c.iterations;
    h.maxiter = c.maxiter;
    h.flexible = (P->mixed && P->precond == NK_PRECONDITIONER_MULTIGRID) ? 1 : 0;
    const nk_iteration_control& pc = P->sd.picard;
    h.p_reltol = pc.reltol;
    h.p_abstol = pc.abstol;
    h.p_fixed = pc.kind == NK_FIXED_ITERATIONS;
    h.p_iterations = pc.iterations;
    h.p_maxiter = pc.maxiter;
    return h;
}
static void set_control(nk_problem* P) {
    *P->sc_host = control_scalars(P);
    NK_CUDA(cudaMemcpyAsync(P->sc, P->sc_host, sizeof(SolverScalars), cudaMemcpyHostToDevice, P->stream));
}

static void cg_step(nk_problem* P, const CGView& v) {
    cudaStream_t s = P->stream;
    launch_cg_apply(v, s);
    launch_cg_update(v, s);
    if (P->precond == NK_PRECONDITIONER_MULTIGRID) {
        precondition_mg(P, &P->sc->done, true);
        launch_cg_dots_after_precondition(v, s);
    }
    launch_cg_xpby(v, s);
}

// conjugate_gradient!, conjugate_gradient.jl:165-171 (everything before the iteration loop)
static void cg_start(nk_problem* P, const CGView& v) {
    update_preconditioner(P);
    launch_cg_init(v, P->stream);
    if (P->precond == NK_PRECONDITIONER_MULTIGRID) {
        if (v.r32) launch_cg_scale_r32(v, P->stream);
        precondition_mg(P, nullptr, true);
        launch_cg_init_finish(v, P->stream);
    }
    NK_CHECK_LAUNCH();
}

static void read_scalars(nk_problem* P) {
    NK_CUDA(cudaMemcpyAsync(P->sc_host, P->sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, P->stream));
    NK_CUDA(cudaStreamSynchronize(P->stream));
}

static std::vector<cudaGraphNode_t> leaves(cudaGraph_t g) {
    size_t n = 0;
    NK_CUDA(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n), out;
    if (n) NK_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
    for (cudaGraphNode_t node : nodes) {
        size_t d = 0;
        NK_CUDA(cudaGraphNodeGetDependentNodes(node, nullptr, nullptr, &d));
        if (d == 0) out.push_back(node);
    }
    return out;
}

template <typename F>
static void capture_into(nk_problem* P, cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps, F&& body) {
    NK_CUDA(cudaStreamBeginCaptureToGraph(P->stream, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                          cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    try {
        body();
    } catch (...) {
        set_capturing(false);
        cudaGraph_t dropped;
        cudaStreamEndCapture(P->stream, &dropped);
        throw;
    }
    set_capturing(false);
    cudaGraph_t captured;
    NK_CUDA(cudaStreamEndCapture(P->stream, &captured));
}

static long long kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    NK_CUDA(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) NK_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
    long long k = 0;
    for (cudaGraphNode_t node : nodes) {
        cudaGraphNodeType t;
        NK_CUDA(cudaGraphNodeGetType(node, &t));
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

static cudaGraph_t add_while(cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps, cudaGraphConditionalHandle h) {
    cudaGraphNodeParams params = {};
    params.type = cudaGraphNodeTypeConditional;
    params.conditional.handle = h;
    params.conditional.type = cudaGraphCondTypeWhile;
    params.conditional.size = 1;
    cudaGraphNode_t node;
    NK_CUDA(cudaGraphAddNode(&node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &params));
    return params.conditional.phGraph_out[0];
}

// update_stress_balance_coefficients! / update_diva_coefficients!
static void update_coefficients(nk_problem* P);

// The strip autotuner: for every multigrid level whose shape the process has not timed yet, times the sweep and
// the residual with walks of 1, 2 and 4 rows (a warm-up and 5 launches each, on this problem's own scratch
// buffers, before any graph is captured) and records the fastest.  Those kernels write one value per cell with
// no reduction; the walk length still changes how the compiler contracts their multiply-adds, so a tuned walk
// moves results in the last bits, and a timing-dependent choice would make them depend on the run.  Tuning is
// therefore opt-in (NK_AUTOTUNE=1; NK_AUTOTUNE_REPORT=1 prints the choices) and the fixed rule of strip_rows
// carries what it found.
static bool autotune_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("NK_AUTOTUNE");
        return e && e[0] == '1';
    }();
    return on;
}
static bool autotune_report() {
    static const bool on = [] {
        const char* e = std::getenv("NK_AUTOTUNE_REPORT");
        return e && e[0] == '1';
    }();
    return on;
}
template <typename T>
static void autotune_levels(nk_problem* P, std::vector<Level<T>>& lv) {
    for (int l = 0; l <= P->nlevels; ++l) {
        LevelView<T> v = P->level_view(lv[l]);
        if (!v.x || !v.x2 || !v.q) continue;
        for (int kind : {STRIP_SMOOTH, STRIP_RESIDUAL}) {
            auto key = std::make_tuple(kind, v.o.g.Nx, v.o.g.Ny, (int)sizeof(T));
            {
                std::lock_guard<std::mutex> g(tuned_mutex());
                if (tuned_rows().count(key)) continue;
            }
            int best = 0;
            float best_ms = 0.f;
            for (int rows : {1, 2, 4}) {
                float ms = time_strip_kernel<T>(v, kind, rows, 5, P->stream);
                if (ms < 0.f) throw Failure{NK_CUDA_ERROR, "strip autotuner: a timing launch failed"};
                if (!best || ms < best_ms) { best = rows; best_ms = ms; }
            }
            std::lock_guard<std::mutex> g(tuned_mutex());
            tuned_rows().emplace(key, best);
            if (autotune_report())
                std::fprintf(stderr, "nk autotune: %s %dx%d fp%d -> %d rows (%.2f us)\n", kind == STRIP_SMOOTH ? "sweep" : "residual",
                             v.o.g.Nx, v.o.g.Ny, 8 * (int)sizeof(T), best, 1e3 * best_ms);
        }
    }
}
// FP64 hierarchies only.  Timed alone, the FP32 sweeps prefer shorter walks on the coarse levels, but with 32
// solves sharing the GPU those choices lowered the mixed serving stream from 11.26 to 10.83 solves/s: there the
// SM time of a launch counts, not its latency, so FP32 keeps the fixed two-row walk.  The FP64 solver runs one
// solve at a time, and the tuned walks raised it from 1.48 to 1.68 solves/s on the same box.
static void autotune_strips(nk_problem* P) {
    if (P->strips_tuned) return;
    P->strips_tuned = true;
    if (!autotune_enabled() || P->precond != NK_PRECONDITIONER_MULTIGRID || P->mixed) return;
    autotune_levels<double>(P, P->lv64);
}

// Picard's change measure and stopping test: the reference's velocity change, or the viscosity change of
// NK_VISCOSITY_CONVERGENCE, whose previous η̄H lives in tmp_a (free during a Picard solve).
static void picard_end(nk_problem* P, cudaGraphConditionalHandle h) {
    if (P->sd.picard.kind == NK_VISCOSITY_CONVERGENCE)
        launch_picard_end_viscosity(P->fine.g, P->fine.coef, (double*)P->tmp_a, P->sc, P->partials, h, P->stream);
    else
        launch_picard_end(P->fine.g, P->xprev, P->x, P->sc, P->partials, h, P->stream);
}

static void build_picard_graph(nk_problem* P) {
    autotune_strips(P);
    cudaGraph_t g;
    NK_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle hp;
    NK_CUDA(cudaGraphConditionalHandleCreate(&hp, g, 0, 0));
    capture_into(P, g, {}, [&] { launch_picard_begin(P->sc, hp, 0, P->stream); });
    cudaGraph_t body = add_while(g, leaves(g), hp);
    cudaGraphConditionalHandle hc;
    NK_CUDA(cudaGraphConditionalHandleCreate(&hc, body, 0, 0));
    CGView v = P->cg_view(P->tau);
    v.cond = hc;
    capture_into(P, body, {}, [&] {
        launch_copy_range(P->fine.g, P->xprev, P->x, P->stream);
        update_coefficients(P);
        cg_start(P, v);
    });
    cudaGraph_t cg_body = add_while(body, leaves(body), hc);
    capture_into(P, cg_body, {}, [&] { cg_step(P, v); });
    capture_into(P, body, leaves(body), [&] { picard_end(P, hp); });
    P->picard_kernels[0] = kernel_nodes(g);
    P->picard_kernels[1] = kernel_nodes(body);
    P->picard_kernels[2] = kernel_nodes(cg_body);
    auto ti0 = std::chrono::steady_clock::now();
    NK_CUDA(cudaGraphInstantiate(&P->picard_exec, g, 0));
    P->instantiate_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - ti0).count();
    P->picard_graph = g;
}

static void build_linear_graph(nk_problem* P) {
    autotune_strips(P);
    cudaGraph_t g;
    NK_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle hc;
    NK_CUDA(cudaGraphConditionalHandleCreate(&hc, g, 0, 0));
    CGView v = P->cg_view(P->tmp_b);
    v.cond = hc;
    capture_into(P, g, {}, [&] { cg_start(P, v); });
    cudaGraph_t cg_body = add_while(g, leaves(g), hc);
    capture_into(P, cg_body, {}, [&] { cg_step(P, v); });
    P->linear_kernels[0] = kernel_nodes(g);
    P->linear_kernels[1] = kernel_nodes(cg_body);
    NK_CUDA(cudaGraphInstantiate(&P->linear_exec, g, 0));
    P->linear_graph = g;
}

static void fill_stats_from(const SolverScalars& h, nk_solve_stats* st, bool picard) {
    st->linear_iterations_last = h.it;
    st->linear_iterations_total = picard ? h.it_total : h.it;
    st->residual_norm = h.rnorm;
    st->initial_residual_norm = h.r0;
    st->picard_iterations = picard ? h.p_it : 0;
    st->picard_change = picard ? h.p_D : 0.0;
    st->picard_norm = picard ? h.p_X : 0.0;
    st->status = NK_OK;
    if (h.status == NK_NONFINITE) st->status = NK_NONFINITE;
    else if (picard && !h.p_fixed && !(h.p_D <= std::max(h.p_reltol * h.p_X, h.p_abstol))) st->status = NK_NOT_CONVERGED;
    else if (!h.fixed && !(h.rnorm <= h.tol)) st->status = NK_NOT_CONVERGED;
    else if (h.status == NK_BREAKDOWN) st->status = NK_BREAKDOWN;
}

static void fill_stats(nk_problem* P, nk_solve_stats* st, bool picard) { fill_stats_from(*P->sc_host, st, picard); }

// The same solve issued from the host (NK_GRAPHS=0): CG steps in growing batches, the device `done` flag read
// after each batch; Picard reads its stopping decision after every iteration.
static void host_cg(nk_problem* P, const double2* b) {
    autotune_strips(P);
    CGView v = P->cg_view(b);
    cg_start(P, v);
    const nk_iteration_control& ctl = P->sd.linear;
    int limit = ctl.kind == NK_FIXED_ITERATIONS ? ctl.iterations : ctl.maxiter;
    int issued = 0, batch = 4;
    while (issued < limit) {
        int n = std::min(batch, limit - issued);
        for (int k = 0; k < n; ++k) cg_step(P, v);
        NK_CHECK_LAUNCH();
        issued += n;
        read_scalars(P);
        if (P->sc_host->done) break;
        batch = std::min(batch * 2, 64);
    }
}

static void host_picard(nk_problem* P) {
    launch_picard_begin(P->sc, 0, 0, P->stream);
    read_scalars(P);
    while (!P->sc_host->p_done) {
        launch_copy_range(P->fine.g, P->xprev, P->x, P->stream);
        update_coefficients(P);
        host_cg(P, P->tau);
        picard_end(P, 0);
        NK_CHECK_LAUNCH();
        read_scalars(P);
    }
}

// The warm start takes the prescribed values, so the identity rows start (and stay) solved: their residual is
// zero and the conjugate-gradient directions vanish there.
static void impose_prescribed(nk_problem* P, const double2* val) {
    if (!P->ud) return;
    launch_impose_prescribed(P->fine.g, P->x, P->ud, val, P->stream);
    NK_CHECK_LAUNCH();
}

// solve!(x, solver, b, ...) with b already on the device in tmp_b
static void linear_solve(nk_problem* P, nk_solve_stats* st) {
    impose_prescribed(P, P->tmp_b);   // an identity row's solution is its right-hand side
    if (!use_graphs(P)) {
        set_control(P);
        host_cg(P, P->tmp_b);
        read_scalars(P);
        fill_stats(P, st, false);
        return;
    }
    if (!P->linear_exec) build_linear_graph(P);
    set_control(P);
    NK_CUDA(cudaGraphLaunch(P->linear_exec, P->stream));
    read_scalars(P);
    fill_stats(P, st, false);
    count_launches(P->linear_kernels[0] + (long long)P->sc_host->it * P->linear_kernels[1]);
}

// picard_solve!, picard.jl:63-90
static void picard_solve(nk_problem* P, nk_solve_stats* st) {
    impose_prescribed(P, P->ud);
    if (!use_graphs(P)) {
        set_control(P);
        host_picard(P);
        read_scalars(P);
        fill_stats(P, st, true);
        return;
    }
    if (!P->picard_exec) build_picard_graph(P);
    set_control(P);
    NK_CUDA(cudaGraphLaunch(P->picard_exec, P->stream));
    read_scalars(P);
    fill_stats(P, st, true);
    const SolverScalars& h = *P->sc_host;
    count_launches(P->picard_kernels[0] + (long long)h.p_it * P->picard_kernels[1] + (long long)h.it_total * P->picard_kernels[2]);
}

static void update_coefficients(nk_problem* P) {
    cudaStream_t s = P->stream;
    PhysView ph = P->phys();
    if (P->pd.stress_balance == NK_DIVA) {
        launch_basal_velocity(ph, P->x, P->bb, P->F2, P->ub, s);
        launch_basal_drag(ph, P->ub, nullptr, P->bb, s);
        launch_viscosity_diva(ph, P->x, P->bb, P->ub, P->eta_sigma, P->fine.coef, P->F2, s);
        launch_corners<double>(P->fine.g, P->fine.coef, s);
        launch_effective_drag(ph, P->bb, P->F2, P->fine.coef, s);
    } else {
        launch_viscosity(ph, P->x, P->eta_sigma, P->fine.coef, P->F2, s);
        launch_corners<double>(P->fine.g, P->fine.coef, s);
        launch_basal_drag(ph, P->x, P->fine.coef, nullptr, s);
    }
    NK_CHECK_LAUNCH();
    prepare_operator(P);
}

// ---- fields in interior layout -----------------------------------------------------------------------------------
struct FieldLoc {
    double* base = nullptr;   // pitched device array (first plane)
    int stride = 1, offset = 0, nx = 0, ny = 0, planes = 1;
    bool coef = false;        // a coefficient: the operator mask and diagonal follow it
    bool prescribed = false;  // a prescribed velocity (allocated on first use)
    bool thermal = false;     // the enthalpy or the water fraction (allocated on first use, sigma layout only)
    bool transport = false;   // a source or the clip of the thickness step (allocated on first use)
    bool energy = false;      // a state field or diagnostic of the energy step (allocated on first use)
    bool front = false;       // a field of the partial-cell front (allocated on first use)
};

static const int ENERGY_PLANES_2D = 7;   // the energy step's Center-Center planes before Φ

static FieldLoc field_loc(nk_problem* P, int id) {
    FieldLoc f;
    int nfx = P->px ? P->Nx : P->Nx + 1, nfy = P->py ? P->Ny : P->Ny + 1;
    auto cc = [&](double* b) { f.base = b; f.nx = P->Nx; f.ny = P->Ny; };
    auto fu = [&](double2* b) { f.base = (double*)b; f.stride = 2; f.offset = 0; f.nx = nfx; f.ny = P->Ny; };
    auto fv = [&](double2* b) { f.base = (double*)b; f.stride = 2; f.offset = 1; f.nx = P->Nx; f.ny = nfy; };
    switch (id) {
        case NK_FIELD_U: fu(P->x); break;
        case NK_FIELD_V: fv(P->x); break;
        case NK_FIELD_H: cc(P->H); break;
        case NK_FIELD_BED: cc(P->bed); break;
        case NK_FIELD_SURFACE: cc(P->s); break;
        case NK_FIELD_ICE_MASK: cc(P->mu); break;
        case NK_FIELD_PHI: cc(P->phi); break;
        case NK_FIELD_PHI_U: fu(P->phi_uv); break;
        case NK_FIELD_PHI_V: fv(P->phi_uv); break;
        case NK_FIELD_EFFECTIVE_PRESSURE: cc(P->N); break;
        case NK_FIELD_TAU_U: fu(P->tau); break;
        case NK_FIELD_TAU_V: fv(P->tau); break;
        case NK_FIELD_RATE_FACTOR:
            if (P->pd.rate_factor_layout == NK_RATE_FACTOR_SIGMA) { cc(P->A3); f.planes = P->Ns; } else cc(P->A2);
            break;
        case NK_FIELD_FRICTION_COEFFICIENT: cc(P->C); break;
        case NK_FIELD_ETA_H: f.base = (double*)P->fine.coef; f.stride = 4; f.offset = 0; f.nx = P->Nx; f.ny = P->Ny; f.coef = true; break;
        case NK_FIELD_ETA_H_FF: f.base = (double*)P->fine.coef; f.stride = 4; f.offset = 1; f.nx = nfx; f.ny = nfy; f.coef = true; break;
        case NK_FIELD_BETA_U: f.base = (double*)P->fine.coef; f.stride = 4; f.offset = 2; f.nx = nfx; f.ny = P->Ny; f.coef = true; break;
        case NK_FIELD_BETA_V: f.base = (double*)P->fine.coef; f.stride = 4; f.offset = 3; f.nx = P->Nx; f.ny = nfy; f.coef = true; break;
        case NK_FIELD_ETA_SIGMA: cc(P->eta_sigma); f.planes = P->Ns; break;
        case NK_FIELD_F2: cc(P->F2); break;
        case NK_FIELD_BETA_B_U: fu(P->bb); break;
        case NK_FIELD_BETA_B_V: fv(P->bb); break;
        case NK_FIELD_U_B: fu(P->ub); break;
        case NK_FIELD_V_B: fv(P->ub); break;
        case NK_FIELD_U_SIGMA: fu(P->usig); f.planes = P->Ns; break;
        case NK_FIELD_V_SIGMA: fv(P->usig); f.planes = P->Ns; break;
        case NK_FIELD_TEMPERATURE: if (P->T) { cc(P->T); f.planes = P->Ns; } break;
        case NK_FIELD_U_PRESCRIBED: fu(P->ud); f.prescribed = true; break;
        case NK_FIELD_V_PRESCRIBED: fv(P->ud); f.prescribed = true; break;
        case NK_FIELD_ENTHALPY:
        case NK_FIELD_WATER_FRACTION:
            if (P->pd.rate_factor_layout == NK_RATE_FACTOR_SIGMA) {
                cc(P->thermal ? P->thermal + (id == NK_FIELD_WATER_FRACTION ? (size_t)P->Ns * P->plane : 0) : nullptr);
                f.planes = P->Ns;
                f.thermal = true;
            }
            break;
        case NK_FIELD_SURFACE_MASS_BALANCE:
        case NK_FIELD_BASAL_MELT_RATE:
        case NK_FIELD_GROUNDED_MELT_RATE:
        case NK_FIELD_CLIPPED_THICKNESS:
            cc(P->transport ? P->transport + (size_t)(id - NK_FIELD_SURFACE_MASS_BALANCE) * P->plane : nullptr);
            f.transport = true;
            break;
        case NK_FIELD_BASAL_WATER_THICKNESS:
        case NK_FIELD_GEOTHERMAL_FLUX:
        case NK_FIELD_SURFACE_TEMPERATURE:
        case NK_FIELD_OCEAN_TEMPERATURE:
        case NK_FIELD_THICKNESS_PREVIOUS:
        case NK_FIELD_BASAL_TEMPERATE_FRACTION:
        case NK_FIELD_BASAL_HEAT_FLUX:
            cc(P->energy ? P->energy + (size_t)(id - NK_FIELD_BASAL_WATER_THICKNESS) * P->plane : nullptr);
            f.energy = true;
            break;
        case NK_FIELD_STRAIN_HEATING:
            cc(P->energy ? P->energy + (size_t)ENERGY_PLANES_2D * P->plane : nullptr);
            f.planes = P->Ns;
            f.energy = true;
            break;
        case NK_FIELD_FRONT_THICKNESS:
        case NK_FIELD_CALVED_THICKNESS:
        case NK_FIELD_CALVING_EXTENT:
            cc(P->front_buf ? P->front_buf + (size_t)(id - NK_FIELD_FRONT_THICKNESS) * P->plane : nullptr);
            f.front = true;
            break;
        default: break;
    }
    return f;
}

// The enthalpy and water-fraction planes (zero at first).  No graph reads them, so none is rebuilt.
static void ensure_thermal(nk_problem* P) {
    if (P->thermal || P->pd.rate_factor_layout != NK_RATE_FACTOR_SIGMA) return;
    if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
    size_t bytes = 2 * (size_t)P->Ns * P->plane * sizeof(double);
    NK_CUDA(cudaMalloc((void**)&P->thermal, bytes));
    NK_CUDA(cudaMemsetAsync(P->thermal, 0, bytes, P->stream));
}

// The energy step's planes (zero at first): the seven fields NK_FIELD_BASAL_WATER_THICKNESS ..
// NK_FIELD_BASAL_HEAT_FLUX, the strain heating (Ns planes) and the enthalpy at the start of the step (Ns planes).
static void ensure_energy(nk_problem* P) {
    if (P->energy) return;
    if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
    size_t bytes = (ENERGY_PLANES_2D + 2 * (size_t)P->Ns) * P->plane * sizeof(double);
    NK_CUDA(cudaMalloc((void**)&P->energy, bytes));
    NK_CUDA(cudaMemsetAsync(P->energy, 0, bytes, P->stream));
}

// The thickness step's planes (zero at first): the four fields of NK_FIELD_SURFACE_MASS_BALANCE ..
// NK_FIELD_CLIPPED_THICKNESS, then the thickness at the start of the step and of the stage, and the bounds-preserving
// limiter of each cell.  No graph reads them.
static const int TRANSPORT_PLANES = 11;   // 7 fields, then the WENO face reconstructions (two double2 planes)
static void ensure_transport(nk_problem* P) {
    if (P->transport) return;
    if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
    size_t bytes = TRANSPORT_PLANES * P->plane * sizeof(double);
    NK_CUDA(cudaMalloc((void**)&P->transport, bytes));
    NK_CUDA(cudaMemsetAsync(P->transport, 0, bytes, P->stream));
}

// The partial-cell front's planes (zero at first): Hʳ, the calved thickness and the calving extent (the fields
// NK_FIELD_FRONT_THICKNESS .. NK_FIELD_CALVING_EXTENT), then the overflow, two snapshots of H and μ and the two
// calving scratch planes.  No graph reads them.
static const int FRONT_PLANES = 8;
static void ensure_front(nk_problem* P) {
    if (P->front_buf) return;
    if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
    size_t bytes = FRONT_PLANES * P->plane * sizeof(double);
    NK_CUDA(cudaMalloc((void**)&P->front_buf, bytes));
    NK_CUDA(cudaMemsetAsync(P->front_buf, 0, bytes, P->stream));
}

// The prescribed-velocity pairs, all NaN (free) at first.  Graphs captured before hold no pointer to them and
// are rebuilt.
static void ensure_prescribed(nk_problem* P) {
    if (P->ud) return;
    if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
    NK_CUDA(cudaStreamSynchronize(P->stream));   // no graph of this problem is still running when it is destroyed
    NK_CUDA(cudaMalloc((void**)&P->ud, P->plane * sizeof(double2)));
    launch_fill((double*)P->ud, (int)(2 * P->plane), std::nan(""), P->stream);
    NK_CHECK_LAUNCH();
    if (P->picard_exec) { cudaGraphExecDestroy(P->picard_exec); P->picard_exec = nullptr; }
    if (P->linear_exec) { cudaGraphExecDestroy(P->linear_exec); P->linear_exec = nullptr; }
    if (P->picard_graph) { cudaGraphDestroy(P->picard_graph); P->picard_graph = nullptr; }
    if (P->linear_graph) { cudaGraphDestroy(P->linear_graph); P->linear_graph = nullptr; }
}

static void copy_in(nk_problem* P, const FieldLoc& f, const double* host) {
    size_t n = (size_t)f.nx * f.ny * f.planes;
    NK_CUDA(cudaMemcpyAsync(P->staging, host, n * sizeof(double), cudaMemcpyDefault, P->stream));   // host or device source
    launch_pack(f.base, P->pitch, (int)P->plane, f.stride, f.offset, P->staging, f.nx, f.ny, f.planes, P->stream);
    NK_CHECK_LAUNCH();
}
// Oceananigans parent layout: the interior rows of each level are gathered into the dense staging array by
// pitched 2-D copies (host or device source), then packed as above; out, the reverse, halos untouched.
struct ParentLayout { size_t px, py; int hx, hy, hz; };
static ParentLayout parent_layout(const FieldLoc& f, int hx, int hy, int hz, int64_t count) {
    if (hx < 0 || hy < 0 || hz < 0) bad("negative halo");
    if (f.planes == 1 && hz != 0) bad("a 2-D field's parent has one level (hz = 0)");
    ParentLayout L{(size_t)f.nx + 2 * (size_t)hx, (size_t)f.ny + 2 * (size_t)hy, hx, hy, hz};
    if (count != (int64_t)(L.px * L.py * ((size_t)f.planes + 2 * (size_t)hz))) bad("parent array size mismatch");
    return L;
}
static size_t parent_offset(const ParentLayout& L, int level) {
    return (((size_t)level + L.hz) * L.py + L.hy) * L.px + L.hx;
}
static void copy_in_parent(nk_problem* P, const FieldLoc& f, const double* parent, const ParentLayout& L) {
    size_t n2 = (size_t)f.nx * f.ny;
    for (int k = 0; k < f.planes; ++k)
        NK_CUDA(cudaMemcpy2DAsync(P->staging + k * n2, f.nx * sizeof(double), parent + parent_offset(L, k), L.px * sizeof(double),
                                  f.nx * sizeof(double), f.ny, cudaMemcpyDefault, P->stream));
    launch_pack(f.base, P->pitch, (int)P->plane, f.stride, f.offset, P->staging, f.nx, f.ny, f.planes, P->stream);
    NK_CHECK_LAUNCH();
}
static void copy_out_parent(nk_problem* P, const FieldLoc& f, double* parent, const ParentLayout& L) {
    size_t n2 = (size_t)f.nx * f.ny;
    launch_unpack(P->staging, f.base, P->pitch, (int)P->plane, f.stride, f.offset, f.nx, f.ny, f.planes, P->stream);
    NK_CHECK_LAUNCH();
    for (int k = 0; k < f.planes; ++k)
        NK_CUDA(cudaMemcpy2DAsync(parent + parent_offset(L, k), L.px * sizeof(double), P->staging + k * n2, f.nx * sizeof(double),
                                  f.nx * sizeof(double), f.ny, cudaMemcpyDefault, P->stream));
    NK_CUDA(cudaStreamSynchronize(P->stream));
}
static void copy_out(nk_problem* P, const FieldLoc& f, double* host) {
    size_t n = (size_t)f.nx * f.ny * f.planes;
    launch_unpack(P->staging, f.base, P->pitch, (int)P->plane, f.stride, f.offset, f.nx, f.ny, f.planes, P->stream);
    NK_CHECK_LAUNCH();
    NK_CUDA(cudaMemcpyAsync(host, P->staging, n * sizeof(double), cudaMemcpyDefault, P->stream));   // host or device target
    NK_CUDA(cudaStreamSynchronize(P->stream));
}
// a velocity vector (u part, v part) from host arrays into a pair buffer
static void vector_in(nk_problem* P, double2* dst, const double* u, const double* v) {
    NK_CUDA(cudaMemsetAsync(dst, 0, P->plane * sizeof(double2), P->stream));
    FieldLoc fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
    fu.base = (double*)dst; fv.base = (double*)dst;
    copy_in(P, fu, u);
    copy_in(P, fv, v);
}
static void vector_out(nk_problem* P, const double2* src, double* u, double* v) {
    FieldLoc fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
    fu.base = (double*)src; fv.base = (double*)src;
    copy_out(P, fu, u);
    copy_out(P, fv, v);
}

}  // namespace nk

// =================================================================================================================
// C ABI
// =================================================================================================================
namespace {
template <typename F>
nk_status guarded(nk_context* ctx, F&& f) {
    try {
        if (ctx) {
            cudaError_t e = cudaSetDevice(ctx->device);
            if (e != cudaSuccess) throw Failure{NK_CUDA_ERROR, std::string("cudaSetDevice: ") + cudaGetErrorString(e)};
        }
        f();
        return NK_OK;
    } catch (const Failure& fl) {
        if (ctx) ctx->error = fl.message;
        return fl.status;
    } catch (const std::exception& e) {
        if (ctx) ctx->error = e.what();
        return NK_CUDA_ERROR;
    }
}
}  // namespace

extern "C" {

int32_t nk_api_version(void) { return NK_API_VERSION; }

int64_t nk_launch_count(void) { return (int64_t)nk::launch_count(); }

nk_status nk_context_create(int32_t device, nk_context** out) {
    if (!out) return NK_BAD_ARGUMENT;
    // Independent solves run on one stream each; with the default of 8 hardware work queues, streams beyond the
    // eighth share a queue and wait on each other's work.  Effective only if the process has no CUDA context yet
    // (hosts that create one first set CUDA_DEVICE_MAX_CONNECTIONS themselves).
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return NK_CUDA_ERROR;
    auto* c = new nk_context();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ref) != cudaSuccess || cudaEventRecord(c->ref, c->stream) != cudaSuccess ||
        cudaEventSynchronize(c->ref) != cudaSuccess) {
        delete c;
        return NK_CUDA_ERROR;
    }
    *out = c;
    return NK_OK;
}

nk_status nk_context_destroy(nk_context* ctx) {
    if (ctx) {
        cudaSetDevice(ctx->device);
        if (ctx->ref) cudaEventDestroy(ctx->ref);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
    return NK_OK;
}

const char* nk_last_error(const nk_context* ctx) { return ctx ? ctx->error.c_str() : "no context"; }

static nk_status problem_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics, const nk_solver_desc* solver,
                                nk_problem** out, char* device_arena, SolverScalars* pinned_scalars);

nk_status nk_problem_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics, const nk_solver_desc* solver,
                            nk_problem** out) {
    return problem_create(ctx, grid, physics, solver, out, nullptr, nullptr);
}

// A problem whose device arena (problem_bytes) and pinned scalar block are supplied by the caller (the server).
static nk_status problem_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics, const nk_solver_desc* solver,
                                nk_problem** out, char* device_arena, SolverScalars* pinned_scalars) {
    if (!ctx || !grid || !physics || !solver || !out) return NK_BAD_ARGUMENT;
    auto* P = new nk_problem();
    if (device_arena) {
        P->arena.base = device_arena;
        P->external_arena = true;
    }
    if (pinned_scalars) {
        P->sc_host = pinned_scalars;
        P->external_pinned = true;
    }
    nk_status st = guarded(ctx, [&] {
        if (grid->Nx < 1 || grid->Ny < 1 || grid->Nsigma < 1 || grid->Nsigma > MAX_SIGMA) bad("grid size or Nsigma out of range");
        if (grid->halo_x < 0 || grid->halo_y < 0) bad("negative halo");
        if (!grid->x_faces && !(grid->Lx > 0)) bad("regular x axis needs Lx > 0");
        if (!grid->y_faces && !(grid->Ly > 0)) bad("regular y axis needs Ly > 0");
        if (physics->side_walls != NK_FREE_SLIP && physics->side_walls != NK_NO_SLIP)
            bad("the coefficients must include the side walls, FreeSlipWalls() or NoSlipWalls()");
        if (physics->glen_exponent <= 0) bad("glen exponent must be positive");
        if (physics->use_ice_mask && !(physics->mask_transition_thickness > 0)) bad("transition_thickness must be positive");
        if (solver->preconditioner < NK_PRECONDITIONER_NONE || solver->preconditioner > NK_PRECONDITIONER_MULTIGRID) bad("unknown preconditioner");
        if (solver->linear.kind != NK_CONVERGENCE && solver->linear.kind != NK_FIXED_ITERATIONS) bad("unknown linear iteration control");
        if (solver->picard.kind < NK_CONVERGENCE || solver->picard.kind > NK_VISCOSITY_CONVERGENCE) bad("unknown Picard iteration control");
        if (solver->precision != NK_PRECISION_FP64 && solver->precision != NK_PRECISION_MIXED) bad("unknown precision");
        if (solver->precision == NK_PRECISION_MIXED && solver->preconditioner != NK_PRECONDITIONER_MULTIGRID)
            bad("mixed precision needs the multigrid preconditioner");
        if (solver->flags & ~NK_SOLVER_HOST_LOOP) bad("unknown solver flags");
        P->ctx = ctx;
        P->gd = *grid;             // build() reads the caller's face vectors during this call only
        P->pd = *physics;
        P->sd = *solver;
        NK_CUDA(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
        NK_CUDA(cudaEventCreate(&P->ev0));
        NK_CUDA(cudaEventCreate(&P->ev1));
        build(P);
        configure_coarsest_smem<float>();   // shared-memory limit of the coarsest-level kernel, once, outside any capture
        configure_coarsest_smem<double>();
        P->gd.x_faces = nullptr; P->gd.y_faces = nullptr; P->gd.sigma_faces = nullptr;   // no pointer kept after the call
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
    if (st != NK_OK) {
        nk_problem_destroy(P);
        return st;
    }
    *out = P;
    return NK_OK;
}

nk_status nk_problem_destroy(nk_problem* P) {
    if (!P) return NK_OK;
    if (P->ctx) cudaSetDevice(P->ctx->device);
    if (P->stream) cudaStreamSynchronize(P->stream);
    if (P->picard_exec) cudaGraphExecDestroy(P->picard_exec);
    if (P->linear_exec) cudaGraphExecDestroy(P->linear_exec);
    if (P->picard_graph) cudaGraphDestroy(P->picard_graph);
    if (P->linear_graph) cudaGraphDestroy(P->linear_graph);
    if (P->arena.base && !P->external_arena) cudaFree(P->arena.base);
    if (P->sc_host && !P->external_pinned) cudaFreeHost(P->sc_host);
    if (P->ev0) cudaEventDestroy(P->ev0);
    if (P->ev1) cudaEventDestroy(P->ev1);
    if (P->adj_base) cudaFree(P->adj_base);
    if (P->adj_diva) cudaFree(P->adj_diva);
    if (P->adj_hmu) cudaFree(P->adj_hmu);
    if (P->ud) cudaFree(P->ud);
    if (P->thermal) cudaFree(P->thermal);
    if (P->transport) cudaFree(P->transport);
    if (P->energy) cudaFree(P->energy);
    if (P->front_buf) cudaFree(P->front_buf);
    if (P->stream && !P->external_stream) cudaStreamDestroy(P->stream);
    delete P;
    return NK_OK;
}

int64_t nk_problem_field_size(const nk_problem* P, int32_t id) {
    if (!P) return 0;
    FieldLoc f = field_loc(const_cast<nk_problem*>(P), id);
    return (f.base || f.prescribed || f.thermal || f.transport || f.energy) ? (int64_t)f.nx * f.ny * f.planes : 0;
}

nk_status nk_problem_set_field(nk_problem* P, int32_t id, const double* host, int64_t count) {
    if (!P || !host) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        FieldLoc f = field_loc(P, id);
        if (f.prescribed) {
            if (count != (int64_t)f.nx * f.ny * f.planes) bad("field size mismatch");
            ensure_prescribed(P);
            f = field_loc(P, id);
        }
        if (f.thermal) {
            ensure_thermal(P);
            f = field_loc(P, id);
        }
        if (f.transport) {
            ensure_transport(P);
            f = field_loc(P, id);
        }
        if (f.energy) {
            ensure_energy(P);
            f = field_loc(P, id);
        }
        if (f.front) {
            ensure_front(P);
            f = field_loc(P, id);
        }
        if (!f.base) bad("unknown field id or field not held by this problem");
        if (count != (int64_t)f.nx * f.ny * f.planes) bad("field size mismatch");
        copy_in(P, f, host);
        if (f.coef || f.prescribed) prepare_operator(P);
        if (f.prescribed) {   // the right-hand side and the velocity of the identity rows
            launch_impose_prescribed(P->fine.g, P->tau, P->ud, P->ud, P->stream);
            launch_impose_prescribed(P->fine.g, P->x, P->ud, P->ud, P->stream);
            NK_CHECK_LAUNCH();
        }
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_problem_get_field(const nk_problem* Pc, int32_t id, double* host, int64_t count) {
    nk_problem* P = const_cast<nk_problem*>(Pc);
    if (!P || !host) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        FieldLoc f = field_loc(P, id);
        if (f.prescribed) {
            ensure_prescribed(P);
            f = field_loc(P, id);
        }
        if (f.thermal) {
            ensure_thermal(P);
            f = field_loc(P, id);
        }
        if (f.transport) {
            ensure_transport(P);
            f = field_loc(P, id);
        }
        if (f.energy) {
            ensure_energy(P);
            f = field_loc(P, id);
        }
        if (f.front) {
            ensure_front(P);
            f = field_loc(P, id);
        }
        if (!f.base) bad("unknown field id or field not held by this problem");
        if (count != (int64_t)f.nx * f.ny * f.planes) bad("field size mismatch");
        copy_out(P, f, host);
    });
}

// set! / interior copies on Oceananigans parent arrays: the same field handling as nk_problem_set_field /
// nk_problem_get_field, with the interior gathered from (scattered into) the halo-padded parent
nk_status nk_problem_set_field_parent(nk_problem* P, int32_t id, const double* parent, int32_t hx, int32_t hy, int32_t hz,
                                      int64_t count) {
    if (!P || !parent) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        FieldLoc f = field_loc(P, id);
        if (f.prescribed) {
            parent_layout(f, hx, hy, hz, count);
            ensure_prescribed(P);
            f = field_loc(P, id);
        }
        if (f.thermal) {
            ensure_thermal(P);
            f = field_loc(P, id);
        }
        if (f.transport) {
            ensure_transport(P);
            f = field_loc(P, id);
        }
        if (f.energy) {
            ensure_energy(P);
            f = field_loc(P, id);
        }
        if (f.front) {
            ensure_front(P);
            f = field_loc(P, id);
        }
        if (!f.base) bad("unknown field id or field not held by this problem");
        copy_in_parent(P, f, parent, parent_layout(f, hx, hy, hz, count));
        if (f.coef || f.prescribed) prepare_operator(P);
        if (f.prescribed) {
            launch_impose_prescribed(P->fine.g, P->tau, P->ud, P->ud, P->stream);
            launch_impose_prescribed(P->fine.g, P->x, P->ud, P->ud, P->stream);
            NK_CHECK_LAUNCH();
        }
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_problem_get_field_parent(const nk_problem* Pc, int32_t id, double* parent, int32_t hx, int32_t hy, int32_t hz,
                                      int64_t count) {
    nk_problem* P = const_cast<nk_problem*>(Pc);
    if (!P || !parent) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        FieldLoc f = field_loc(P, id);
        if (f.prescribed) {
            ensure_prescribed(P);
            f = field_loc(P, id);
        }
        if (f.thermal) {
            ensure_thermal(P);
            f = field_loc(P, id);
        }
        if (f.transport) {
            ensure_transport(P);
            f = field_loc(P, id);
        }
        if (f.energy) {
            ensure_energy(P);
            f = field_loc(P, id);
        }
        if (f.front) {
            ensure_front(P);
            f = field_loc(P, id);
        }
        if (!f.base) bad("unknown field id or field not held by this problem");
        copy_out_parent(P, f, parent, parent_layout(f, hx, hy, hz, count));
    });
}

// The geometry and the driving stress from H and the bed (update_state! without the velocity solve), on the
// problem's stream.
static GeometryView problem_geometry_view(nk_problem* P) {
    GeometryView v;
    v.g = P->fine.g;
    v.H = P->H; v.bed = P->bed; v.s = P->s; v.N = P->N; v.mu = P->mu; v.phi = P->phi; v.phi_uv = P->phi_uv; v.tau = P->tau;
    v.rho_i = P->pd.ice_density; v.rho_w = P->pd.ocean_density; v.gacc = P->pd.gravitational_acceleration;
    v.grounding = P->pd.grounding; v.gl_stress = P->pd.grounding_line_driving_stress; v.use_mask = P->pd.use_ice_mask;
    v.mask_min = P->pd.mask_minimum_thickness; v.mask_trans = P->pd.mask_transition_thickness;
    v.ud = P->ud;
    v.front = P->front.enabled;
    if (P->till.enabled) {   // nk_set_till allocated the energy planes, H_w first
        v.Hw = P->energy;
        v.till_N0 = P->till.reference_effective_pressure;
        v.till_delta = P->till.overburden_fraction;
        v.till_e0_Cc = P->till.reference_void_ratio / P->till.compressibility;
        v.till_Wmax = P->till.maximum_water_thickness;
    }
    return v;
}
static void launch_problem_geometry(nk_problem* P) { launch_geometry(problem_geometry_view(P), P->stream); }

nk_status nk_compute_geometry(nk_problem* P) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        launch_problem_geometry(P);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

}  // extern "C"

namespace nk {
// The energy step's view of the problem (its planes allocated first).
static EnergyView energy_view(nk_problem* P, const nk_energy_params* prm) {
    ensure_thermal(P);
    ensure_transport(P);
    ensure_energy(P);
    const size_t pl = P->plane;
    EnergyView v;
    v.g = P->fine.g;
    v.sig = P->sigma_table();
    v.plane = (long long)pl;
    v.q = {prm->thermal_conductivity, prm->heat_capacity, prm->latent_heat, prm->clausius_clapeyron, prm->melting_temperature,
           prm->reference_temperature, prm->temperate_diffusivity_ratio, prm->enthalpy_blend_width,
           prm->water_layer_blend_thickness, prm->minimum_thickness, prm->drainage_water_fraction, prm->maximum_drainage_rate,
           prm->grounded_melt_coupling != 0};
    v.rho_i = P->pd.ice_density; v.gacc = P->pd.gravitational_acceleration;
    v.wall_factor = P->pd.side_walls == NK_NO_SLIP ? 2.0 : 0.0;
    v.diva = P->pd.stress_balance == NK_DIVA; v.grounding = P->pd.grounding != 0;
    v.x = P->x; v.ud = P->ud; v.usig = P->usig; v.ub = P->ub; v.coef = P->fine.coef; v.bb = P->bb; v.eta_sigma = P->eta_sigma;
    v.H = P->H; v.phi = P->phi;
    double* en = P->energy;
    v.Hw = en; v.G = en + pl; v.Ts = en + 2 * pl; v.To = en + 3 * pl; v.Hn = en + 4 * pl; v.sb = en + 5 * pl; v.qg = en + 6 * pl;
    v.Phi = en + ENERGY_PLANES_2D * pl;
    v.E_old = en + (ENERGY_PLANES_2D + (size_t)P->Ns) * pl;
    v.melt = P->transport + pl; v.gmelt = P->transport + 2 * pl;
    v.E = P->thermal; v.omega = P->thermal + (size_t)P->Ns * pl; v.T = P->T;
    v.till = P->till.enabled;
    v.till_drain = P->till.drainage_rate;
    v.till_Wmax = P->till.maximum_water_thickness;
    return v;
}

// The thickness step's view of the problem with its advection scheme (its planes allocated first).
static ThicknessView thickness_view(nk_problem* P, bool coupled) {
    ensure_transport(P);
    const nk_advection_desc& adv = P->advection;
    ThicknessView v;
    v.g = P->fine.g;
    v.x = P->x; v.Hs = P->transport + 5 * P->plane; v.H0 = P->transport + 4 * P->plane;
    v.smb = P->transport; v.melt = P->transport + P->plane; v.gmelt = P->transport + 2 * P->plane; v.phi = P->phi;
    v.H = P->H; v.clipped = P->transport + 3 * P->plane;
    v.grounding = P->pd.grounding != 0; v.coupled = coupled;
    v.scheme = adv.scheme; v.order = adv.order; v.bounded = adv.bounded;
    v.lower = adv.lower; v.upper = adv.upper;
    v.theta = P->transport + 6 * P->plane;
    v.mu = P->front.enabled ? P->mu : nullptr;
    if (adv.scheme == NK_ADVECTION_WENO) {
        v.fx = reinterpret_cast<double2*>(P->transport + 7 * P->plane);
        v.fy = reinterpret_cast<double2*>(P->transport + 9 * P->plane);
    }
    return v;
}

// The partial-cell front's view of the problem (its planes and the thickness step's allocated first).
static FrontView front_view(nk_problem* P, bool coupled) {
    ensure_transport(P);
    ensure_front(P);
    const size_t pl = P->plane;
    FrontView v;
    v.g = P->fine.g;
    v.H = P->H; v.mu = P->mu;
    v.Hr = P->front_buf; v.calved = P->front_buf + pl; v.extent = P->front_buf + 2 * pl; v.O = P->front_buf + 3 * pl;
    v.H_in = P->front_buf + 4 * pl; v.mu_in = P->front_buf + 5 * pl; v.f = P->front_buf + 6 * pl; v.share = P->front_buf + 7 * pl;
    v.clipped = P->transport + 3 * pl;
    v.x = P->x; v.bed = P->bed; v.phi = P->phi; v.coef = P->fine.coef;
    v.smb = P->transport; v.melt = P->transport + pl; v.gmelt = P->transport + 2 * pl;
    v.grounding = P->pd.grounding != 0; v.coupled = coupled; v.law = P->front.calving;
    v.thickness = P->front.thickness; v.coefficient = P->front.coefficient; v.stress_threshold = P->front.stress_threshold;
    v.floating_stress_threshold = P->front.floating_stress_threshold; v.front_velocity = P->front.front_velocity;
    v.n = P->pd.glen_exponent; v.eps0 = P->pd.strain_rate_regularization;
    v.wall_factor = P->pd.side_walls == NK_NO_SLIP ? 2.0 : 0.0;
    return v;
}

// EnthalpyThermodynamics' defaults (src/Thermodynamics/enthalpy_thermodynamics.jl:92-104).
static nk_energy_params default_energy_params() {
    nk_energy_params q{};
    q.thermal_conductivity = 2.1; q.heat_capacity = 2009; q.latent_heat = 3.34e5; q.clausius_clapeyron = 7.9e-8;
    q.melting_temperature = 273.15; q.reference_temperature = 223.15; q.temperate_diffusivity_ratio = 1e-3;
    q.enthalpy_blend_width = 1; q.water_layer_blend_thickness = 1e-3; q.minimum_thickness = 1;
    q.drainage_water_fraction = 0.01; q.maximum_drainage_rate = 0.05 / 31556926.0; q.grounded_melt_coupling = 1;
    return q;
}
}  // namespace nk

extern "C" {

nk_status nk_step_enthalpy(nk_problem* P, const nk_energy_params* prm, double dt) {
    if (!P || !prm) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        static_assert(sizeof(nk_energy_params) == 12 * sizeof(double) + 2 * sizeof(int32_t), "nk_energy_params layout");
        if (!(dt > 0) || !std::isfinite(dt)) bad("the time step must be finite and positive");
        if (P->pd.rate_factor_layout != NK_RATE_FACTOR_SIGMA) bad("the energy step needs the sigma rate-factor layout");
        if (P->Ns > ENERGY_MAX_LAYERS) bad("the energy step takes at most NK_ENERGY_MAX_LAYERS layers");
        if (!(prm->heat_capacity > 0) || !(prm->latent_heat > 0) || !(prm->thermal_conductivity > 0) ||
            !(prm->enthalpy_blend_width > 0) || !(prm->water_layer_blend_thickness > 0) || !(prm->drainage_water_fraction > 0) ||
            !(prm->minimum_thickness > 0))
            bad("conductivity, heat capacity, latent heat, blend widths, minimum thickness and drainage fraction must be positive");
        if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
        static_assert(ENERGY_MAX_LAYERS == NK_ENERGY_MAX_LAYERS, "one layer limit");
        EnergyView v = energy_view(P, prm);
        const size_t pl = P->plane;
        NK_CUDA(cudaMemcpyAsync(const_cast<double*>(v.E_old), P->thermal, (size_t)P->Ns * pl * sizeof(double), cudaMemcpyDeviceToDevice, P->stream));
        launch_step_enthalpy(v, dt, P->stream);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaMemcpyAsync(P->energy + 4 * pl, P->H, pl * sizeof(double), cudaMemcpyDeviceToDevice, P->stream));   // Hⁿ = H
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

}  // extern "C"

namespace nk {
static void check_thickness_step(nk_problem* P, double dt) {
    if (!(dt > 0) || !std::isfinite(dt)) bad("the time step must be finite and positive");
    if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
    const nk_advection_desc& adv = P->advection;
    const bool bounded = adv.scheme == NK_ADVECTION_WENO && adv.bounded;
    int halo = std::min(P->gd.halo_x, P->gd.halo_y);
    if (bounded && halo < 4)   // check_advection_halo, src/Models/ice_sheet_model.jl:131-135
        bad("bounded WENO(order = 5) needs a horizontal halo of at least 4, got (" + std::to_string(P->gd.halo_x) + ", " +
            std::to_string(P->gd.halo_y) + ")");
    if ((adv.scheme == NK_ADVECTION_WENO || adv.order == 3) && halo < 3)
        bad("the advection scheme's stencil needs a horizontal halo of at least 3");
}

// Stage st (0, 1, 2) of one thickness step: the first caches the step's starting H; each recomputes the limiter from
// the stage's thickness, sets H = max(0, H_start + Δτ G(H)), the last adds its clip and advances a front; then the
// geometry (rk_substep! and update_state! without the velocity solve, time_stepping.jl:15-25).
static void thickness_stage(nk_problem* P, double dt, int st, int coupling) {
    const bool bounded = P->advection.scheme == NK_ADVECTION_WENO && P->advection.bounded;
    ThicknessView v = thickness_view(P, coupling != 0);
    if (st == 0) NK_CUDA(cudaMemcpyAsync((double*)v.H0, P->H, P->plane * sizeof(double), cudaMemcpyDeviceToDevice, P->stream));
    const double stages[3] = {1.0 / 3, 1.0 / 2, 1.0};     // SplitRungeKutta3 (Wicker-Skamarock) fractions
    NK_CUDA(cudaMemcpyAsync((double*)v.Hs, P->H, P->plane * sizeof(double), cudaMemcpyDeviceToDevice, P->stream));
    if (v.fx) launch_thickness_faces(v, P->stream);
    if (bounded) launch_thickness_limiter(v, P->stream);
    launch_thickness_stage(v, stages[st] * dt, st == 2, P->stream);
    if (st == 2 && P->front.enabled)   // rk_substep!: advance_front! after the final stage (time_stepping.jl:23)
        launch_advance_front(front_view(P, coupling != 0), P->front.passes, stages[st] * dt, P->plane, P->stream);
    launch_problem_geometry(P);
    NK_CHECK_LAUNCH();
}
}  // namespace nk

extern "C" {

nk_status nk_step_thickness(nk_problem* P, double dt, int32_t grounded_melt_coupling) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        check_thickness_step(P, dt);
        for (int st = 0; st < 3; ++st) thickness_stage(P, dt, st, grounded_melt_coupling);
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_step_thickness_stage(nk_problem* P, double dt, int32_t stage, int32_t grounded_melt_coupling) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        check_thickness_step(P, dt);
        if (stage < 1 || stage > 3) bad("stage must be 1, 2 or 3");
        thickness_stage(P, dt, stage - 1, grounded_melt_coupling);
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_set_front(nk_problem* P, const nk_front_desc* f) {
    if (!P || !f) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (f->enabled) {
            if (!P->pd.use_ice_mask) bad("a PartialCellFront masks the stress balance with its flag: create the problem with use_ice_mask = 1");
            if (f->passes < 0) bad("passes must be non-negative");
            if (f->calving < NK_CALVING_NONE || f->calving > NK_CALVING_MAXIMUM_EXTENT) bad("unknown calving law");
            ensure_front(P);
        }
        P->front = *f;
    });
}

nk_status nk_set_till(nk_problem* P, const nk_till_desc* t) {
    if (!P || !t) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (t->enabled != 0 && t->enabled != 1) bad("enabled is 0 or 1");
        if (t->enabled) {
            auto positive = [](double x) { return x > 0 && std::isfinite(x); };
            if (!positive(t->reference_effective_pressure) || !positive(t->overburden_fraction) ||
                !positive(t->compressibility) || !positive(t->maximum_water_thickness) || !std::isfinite(t->reference_void_ratio))
                bad("the till's parameters must be positive and finite");
            if (!(t->drainage_rate >= 0) || !std::isfinite(t->drainage_rate)) bad("the till's drainage rate must be finite and non-negative");
            ensure_energy(P);
        }
        P->till = *t;
    });
}

nk_status nk_initialize_front(nk_problem* P) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (!P->front.enabled) bad("the problem has no partial-cell front (nk_set_front)");
        if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
        launch_initialize_front(front_view(P, false), P->stream);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_advance_front(nk_problem* P, double dt) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (!P->front.enabled) bad("the problem has no partial-cell front (nk_set_front)");
        if (!(dt > 0) || !std::isfinite(dt)) bad("the time step must be finite and positive");
        if (P->async_pending) bad("an asynchronous solve is pending (nk_problem_wait first)");
        launch_advance_front(front_view(P, false), P->front.passes, dt, P->plane, P->stream);
        launch_problem_geometry(P);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_set_thickness_advection(nk_problem* P, const nk_advection_desc* adv) {
    if (!P || !adv) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        bool upwind = adv->scheme == NK_ADVECTION_UPWIND && (adv->order == 1 || adv->order == 3) && !adv->bounded;
        bool weno = adv->scheme == NK_ADVECTION_WENO && adv->order == 5 && (!adv->bounded || adv->lower < adv->upper);
        if (!upwind && !weno)
            bad("thickness advection: UpwindBiased(order = 1 or 3) or WENO(order = 5) with bounds lower < upper");
        P->advection = *adv;
    });
}

nk_status nk_compute_rate_factor(nk_problem* P, double cold_prefactor, double warm_prefactor, double cold_activation_energy,
                                 double warm_activation_energy, double transition_temperature, double transition_width,
                                 double gas_constant, double clausius_clapeyron, double melting_temperature) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (P->pd.rate_factor_layout != NK_RATE_FACTOR_SIGMA) bad("the rate factor from temperature needs the sigma layout");
        double prm[9] = {cold_prefactor, warm_prefactor, cold_activation_energy, warm_activation_energy, transition_temperature,
                         transition_width, gas_constant, clausius_clapeyron, melting_temperature};
        NK_CUDA(cudaMemcpyAsync(P->rate_params, prm, sizeof(prm), cudaMemcpyHostToDevice, P->stream));
        launch_rate_factor(P->fine.g, P->sigma_table(), (int)P->plane, P->H, P->T, P->A3, P->pd.ice_density,
                           P->pd.gravitational_acceleration, P->rate_params, P->stream);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_compute_thermal_diagnostics(nk_problem* P, const nk_thermal_params* prm) {
    if (!P || !prm) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        static_assert(sizeof(nk_thermal_params) == 14 * sizeof(double), "nk_thermal_params is 14 doubles");
        if (P->pd.rate_factor_layout != NK_RATE_FACTOR_SIGMA) bad("the rate factor from the enthalpy needs the sigma layout");
        if (!(prm->heat_capacity > 0) || !(prm->latent_heat > 0) || !(prm->gas_constant > 0) || !(prm->transition_width > 0))
            bad("heat capacity, latent heat, gas constant and transition width must be positive");
        ensure_thermal(P);
        NK_CUDA(cudaMemcpyAsync(P->rate_params, prm, sizeof(nk_thermal_params), cudaMemcpyHostToDevice, P->stream));
        launch_thermal_diagnostics(P->fine.g, P->sigma_table(), (int)P->plane, P->H, P->thermal, P->T,
                                   P->thermal + (size_t)P->Ns * P->plane, P->A3, P->pd.ice_density, P->pd.gravitational_acceleration,
                                   P->rate_params, P->stream);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_update_coefficients(nk_problem* P) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        update_coefficients(P);
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_apply_operator(nk_problem* P, const double* pu, const double* pv, double* qu, double* qv) {
    if (!P || !pu || !pv || !qu || !qv) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        vector_in(P, P->tmp_a, pu, pv);
        vector_in(P, P->tmp_b, qu, qv);
        launch_apply(P->fine_op(), P->tmp_a, P->tmp_b, P->stream);
        NK_CHECK_LAUNCH();
        vector_out(P, P->tmp_b, qu, qv);
    });
}

nk_status nk_precondition(nk_problem* P, const double* ru, const double* rv, double* zu, double* zv) {
    if (!P || !ru || !rv || !zu || !zv) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        vector_in(P, P->r, ru, rv);
        vector_in(P, P->z, zu, zv);
        DevGrid<double> g = P->fine.g;
        if (P->precond == NK_PRECONDITIONER_NONE) {
            launch_copy_range(g, P->z, P->r, P->stream);                      // copyto!(z, r) over Nx x Ny
        } else if (P->precond == NK_PRECONDITIONER_DIAGONAL) {
            // z = r / diag over size(z); the wall faces are unit rows (diagonal_preconditioner.jl:11-18)
            launch_inverse_diagonal(P->fine_op(), P->invd, P->stream);
            launch_precondition_diagonal(g, P->z, P->r, P->invd, P->stream);
        } else {
            update_preconditioner(P);
            launch_zero_vec<double>(g, P->z, nullptr, P->stream);             // fill!(x, 0) of v_cycle! covers the wall faces
            precondition_mg(P, nullptr);
        }
        NK_CHECK_LAUNCH();
        vector_out(P, P->z, zu, zv);
    });
}

// device_ms, device_start_ms, device_end_ms of the solve bracketed by ev0 and ev1 (both complete)
static void event_times(nk_problem* P, nk_solve_stats* st) {
    float ms = 0, a = 0, b = 0;
    NK_CUDA(cudaEventElapsedTime(&ms, P->ev0, P->ev1));
    NK_CUDA(cudaEventElapsedTime(&a, P->ctx->ref, P->ev0));
    NK_CUDA(cudaEventElapsedTime(&b, P->ctx->ref, P->ev1));
    st->device_ms = ms;
    st->device_start_ms = a;
    st->device_end_ms = b;
}

static nk_status linear_solve_impl(nk_problem* P, const double* bu, const double* bv, nk_solve_stats* stats) {
    return guarded(P->ctx, [&] {
        nk_solve_stats local{};
        nk_solve_stats* st = stats ? stats : &local;
        std::memset(st, 0, sizeof(*st));
        vector_in(P, P->tmp_b, bu, bv);
        NK_CUDA(cudaEventRecord(P->ev0, P->stream));
        linear_solve(P, st);
        NK_CUDA(cudaEventRecord(P->ev1, P->stream));
        NK_CUDA(cudaEventSynchronize(P->ev1));
        event_times(P, st);
        if (st->status == NK_NONFINITE) throw Failure{NK_NONFINITE, "non-finite residual"};
    });
}

nk_status nk_linear_solve(nk_problem* P, const double* bu, const double* bv, nk_solve_stats* stats) {
    if (!P || !bu || !bv) return NK_BAD_ARGUMENT;
    return linear_solve_impl(P, bu, bv, stats);
}

nk_status nk_adjoint_solve(nk_problem* P, const double* bu, const double* bv, nk_solve_stats* stats) {
    if (!P || !bu || !bv) return NK_BAD_ARGUMENT;
    if (P->ud) {   // identity rows with lifted neighbours are not symmetric
        if (P->ctx) P->ctx->error = "nk_adjoint_solve: not available for a problem with prescribed velocities";
        return NK_BAD_ARGUMENT;
    }
    return linear_solve_impl(P, bu, bv, stats);   // the operator is self-adjoint (conjugate_gradient.jl:45-48, 155-156)
}

// Fixed-point adjoint of a converged picard_solve! (ext/NunatakEnzymeExt.jl:167-240).  The Picard step maps x to
// A(c(x))⁻¹ b; at its fixed point x* the adjoint λ solves λ = A⁻ᵀ (x̄ - Nᵀ λ), N = ∂[A(c(x)) x*]/∂x, iterated
// from λ = 0 with the problem's preconditioned CG warm-started from the previous λ, until
// ‖λ⁺ - λ‖ ≤ max(reltol ‖λ⁺‖, abstol).  Then b̄ = λ and p̄ = -(∂[A(c(p)) x*]/∂p)ᵀ λ.
// DIVA's step also maps its lagged state s = (βᵇ, F₂, ησ) (the overwritten coefficients it reads, diva.jl:77-80);
// the adjoint σ of s is swept along with λ (ext/NunatakEnzymeExt.jl:204-214): each iteration runs the step's reverse with q̄ = -λ and
// the state adjoint σ, which yields r and the next σ.
static void ensure_adjoint(nk_problem* P, bool want_H) {
    const bool diva = P->pd.stress_balance == NK_DIVA;
    if (P->ud) bad("nk_picard_adjoint: not available for a problem with prescribed velocities");
    size_t pl = P->plane;
    if (!P->adj_base) {
        NK_CUDA(cudaMalloc(&P->adj_base, pl * (sizeof(double2) + (2 + (size_t)P->Ns) * sizeof(double))));
        P->adj_xbar = (double2*)P->adj_base;
        P->adj_g = (double*)(P->adj_xbar + pl);
        P->adj_grad = P->adj_g + pl;
        P->adj_grad_A = P->adj_grad + pl;
    }
    if (diva && !P->adj_diva) NK_CUDA(cudaMalloc(&P->adj_diva, pl * (8 * sizeof(double2) + (1 + (size_t)P->Ns) * sizeof(double))));
    if (diva && want_H && !P->adj_hmu) NK_CUDA(cudaMalloc((void**)&P->adj_hmu, pl * sizeof(double2)));
}

// The adjoint with x̄ already in P->adj_xbar (ensure_adjoint first): leaves λ in tmp_a, ∂J/∂log C in adj_grad,
// ∂J/∂log A in adj_grad_A (want_A) and ∂J/∂H in adj_g (want_H), and U, V = x* again.
// eta_bar_in: ∂J/∂η̄H per centre from outside the solve (NULL: none), carried through every pass
static void picard_adjoint_device(nk_problem* P, const nk_iteration_control& ctl, bool want_A, bool want_H, nk_solve_stats* st,
                                  const double* eta_bar_in = nullptr) {
    const bool diva = P->pd.stress_balance == NK_DIVA;
    cudaStream_t s = P->stream;
    size_t pl = P->plane;
    NK_CUDA(cudaMemcpyAsync(P->xprev, P->x, pl * sizeof(double2), cudaMemcpyDeviceToDevice, s));   // x*
    update_coefficients(P);                                                                         // c(x*)
    NK_CUDA(cudaMemsetAsync(P->adj_g, 0, pl * sizeof(double), s));
    NK_CUDA(cudaMemsetAsync(P->tmp_a, 0, pl * sizeof(double2), s));                                 // λ
    NK_CUDA(cudaMemsetAsync(P->x, 0, pl * sizeof(double2), s));                                     // CG iterate
    AdjointView v;
    v.ph = P->phys();
    v.o = P->fine_op();
    v.xs = P->xprev;
    v.lam = P->tmp_a;
    v.xbar = P->adj_xbar;
    if (diva) {   // uᵇ, βᵇ and F₂ are the step's state: the coefficient adjoints get their own planes
        double2* d2 = (double2*)P->adj_diva;
        v.cbar = d2;
        v.bbar = d2 + pl;
        v.txbar = d2 + 2 * pl;
        v.sig_bb = d2 + 3 * pl;
        v.Ubar = d2 + 4 * pl;
        v.ubp = d2 + 5 * pl;
        v.mbar = d2 + 6 * pl;
        v.bbt = d2 + 7 * pl;
        v.sig_F2 = (double*)(d2 + 8 * pl);
        v.sig_eta = v.sig_F2 + pl;
        v.ubs = P->ub;
        v.bbs = P->bb;
        v.F2s = P->F2;
        NK_CUDA(cudaMemsetAsync(v.sig_bb, 0, pl * sizeof(double2), s));
        NK_CUDA(cudaMemsetAsync(v.sig_F2, 0, pl * (1 + (size_t)P->Ns) * sizeof(double), s));
    } else {
        v.cbar = P->ub;
        v.bbar = P->bb;
    }
    v.gbar = P->adj_g;
    v.r = P->tmp_b;
    v.grad_log_C = P->adj_grad;
    v.eta_sigma = P->eta_sigma;
    v.grad_log_A = nullptr;   // only in the final pass
    v.eta_bar_in = eta_bar_in;
    bool fixed = ctl.kind == NK_FIXED_ITERATIONS;
    int limit = fixed ? ctl.iterations : ctl.maxiter;
    int it = 0, cg_total = 0, cg_last = 0;
    double D = INFINITY, M = 0.0, rnorm = 0.0;
    bool cg_failed = false;
    while (it < limit && (fixed || D > std::max(ctl.reltol * M, ctl.abstol))) {
        launch_adjoint_coefficients(v, s);
        if (diva) {
            launch_adjoint_diva(v, s);                       // tmp_b = x̄ + ȳ, σ of the lagged state
        } else {
            launch_adjoint_viscosity(v, s);
            launch_adjoint_velocity(v, s);                   // tmp_b = x̄ - Nᵀ λ
        }
        nk_solve_stats lst{};
        linear_solve(P, &lst);                               // x = A⁻¹ tmp_b, from x = λ
        cg_total += lst.linear_iterations_total;
        cg_last = lst.linear_iterations_last;
        rnorm = lst.residual_norm;
        if (lst.status == NK_NONFINITE || lst.status == NK_BREAKDOWN) cg_failed = true;
        launch_adjoint_change(P->fine.g, P->x, P->tmp_a, P->sc, P->partials, s);   // Δ, M; λ = x
        NK_CHECK_LAUNCH();
        read_scalars(P);
        D = P->sc_host->p_D;
        M = P->sc_host->p_X;
        ++it;
        if (!std::isfinite(D) || cg_failed) break;
    }
    launch_adjoint_coefficients(v, s);
    if (want_A) v.grad_log_A = P->adj_grad_A;
    if (diva) {
        if (want_H) v.hmu = P->adj_hmu;
        launch_adjoint_diva(v, s);
        launch_adjoint_diva_gradient(v, s);
        if (want_H) launch_adjoint_thickness(v, problem_geometry_view(P), 1, P->adj_g, s);   // gbar is free after the last pass
    } else {
        if (want_A) launch_adjoint_viscosity(v, s);
        launch_adjoint_gradient(v, s);
        if (want_H) launch_adjoint_thickness(v, problem_geometry_view(P), 0, P->adj_g, s);
    }
    NK_CHECK_LAUNCH();
    NK_CUDA(cudaMemcpyAsync(P->x, P->xprev, pl * sizeof(double2), cudaMemcpyDeviceToDevice, s));   // U, V = x*
    std::memset(st, 0, sizeof(*st));
    st->picard_iterations = it;
    st->linear_iterations_total = cg_total;
    st->linear_iterations_last = cg_last;
    st->residual_norm = rnorm;
    st->picard_change = D;
    st->picard_norm = M;
    st->status = NK_OK;
    if (!std::isfinite(D) || cg_failed) st->status = NK_NONFINITE;
    else if (!fixed && !(D <= std::max(ctl.reltol * M, ctl.abstol))) st->status = NK_NOT_CONVERGED;
}

static void picard_adjoint(nk_problem* P, const double* ubar, const double* vbar, const nk_iteration_control& ctl, double* lu,
                           double* lv, double* grad, double* grad_A, double* grad_H, nk_solve_stats* st) {
    ensure_adjoint(P, grad_H != nullptr);
    vector_in(P, P->adj_xbar, ubar, vbar);
    picard_adjoint_device(P, ctl, grad_A != nullptr, grad_H != nullptr, st);
    if (lu && lv) vector_out(P, P->tmp_a, lu, lv);
    if (grad) {
        FieldLoc f;
        f.base = P->adj_grad;
        f.nx = P->Nx;
        f.ny = P->Ny;
        copy_out(P, f, grad);
    }
    if (grad_H) {
        FieldLoc f;
        f.base = P->adj_g;
        f.nx = P->Nx;
        f.ny = P->Ny;
        copy_out(P, f, grad_H);
    }
    if (grad_A) {
        FieldLoc f;
        f.base = P->adj_grad_A;
        f.nx = P->Nx;
        f.ny = P->Ny;
        f.planes = P->pd.rate_factor_layout == NK_RATE_FACTOR_SIGMA ? P->Ns : 1;
        copy_out(P, f, grad_A);
    }
    NK_CUDA(cudaStreamSynchronize(P->stream));
}

nk_status nk_picard_adjoint_gradients(nk_problem* P, const double* ubar, const double* vbar, const nk_iteration_control* control,
                                      double* lambda_u, double* lambda_v, double* grad_log_C, double* grad_log_A, double* grad_H,
                                      nk_solve_stats* stats) {
    if (!P || !ubar || !vbar) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        nk_iteration_control ctl = control ? *control : P->sd.picard;
        if (ctl.kind == NK_FIXED_ITERATIONS ? ctl.iterations < 0 : ctl.maxiter < 0) bad("negative iteration count");
        if (ctl.kind != NK_CONVERGENCE && ctl.kind != NK_FIXED_ITERATIONS) bad("the adjoint takes Convergence or FixedIterations");
        nk_solve_stats local{};
        nk_solve_stats* st = stats ? stats : &local;
        NK_CUDA(cudaEventRecord(P->ev0, P->stream));
        picard_adjoint(P, ubar, vbar, ctl, lambda_u, lambda_v, grad_log_C, grad_log_A, grad_H, st);
        NK_CUDA(cudaEventRecord(P->ev1, P->stream));
        NK_CUDA(cudaEventSynchronize(P->ev1));
        event_times(P, st);
        if (st->status == NK_NONFINITE) throw Failure{NK_NONFINITE, "non-finite Picard adjoint"};
    });
}

nk_status nk_picard_adjoint(nk_problem* P, const double* ubar, const double* vbar, const nk_iteration_control* control,
                            double* lambda_u, double* lambda_v, double* grad_log_C, double* grad_log_A, nk_solve_stats* stats) {
    return nk_picard_adjoint_gradients(P, ubar, vbar, control, lambda_u, lambda_v, grad_log_C, grad_log_A, nullptr, stats);
}

}  // extern "C"

namespace nk {
// ---- the gradient through time steps (checkpointed_gradient!, ext/NunatakEnzymeExt.jl:245-263) ---------------------
// A stored state: H, (U, V), and for the DIVA the lagged beta_b, F2 and eta_sigma its next Picard step reads
// (diva.jl:77-80; the vertical shear of _compute_shear_viscosity! divides by the previous viscosity), so that a
// restored state re-runs bit for bit and the adjoint of a solve linearises where the solve ended.
// With a partial-cell front the flag μ and the front thickness Hʳ follow them (the step's last stage moves the front),
// and under von Mises calving the depth-averaged viscosity η̄H its rates read (the last Picard step's coefficient).
static bool von_mises_front(const nk_problem* P) { return P->front.enabled && P->front.calving == NK_CALVING_VON_MISES; }
static int time_state_base(const nk_problem* P, bool diva) { return diva ? 6 + P->Ns : 3; }
static int time_state_planes(const nk_problem* P, bool diva) {
    return time_state_base(P, diva) + (P->front.enabled ? 2 : 0) + (von_mises_front(P) ? 1 : 0);
}
static void save_time_state(nk_problem* P, double* rec, bool diva) {
    const size_t pl = P->plane;
    cudaStream_t s = P->stream;
    NK_CUDA(cudaMemcpyAsync(rec, P->H, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
    NK_CUDA(cudaMemcpyAsync(rec + pl, P->x, pl * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    if (P->front.enabled) {
        double* f = rec + (size_t)time_state_base(P, diva) * pl;
        NK_CUDA(cudaMemcpyAsync(f, P->mu, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(f + pl, P->front_buf, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (von_mises_front(P))   // η̄H = coef[].x, one double of every double4
            NK_CUDA(cudaMemcpy2DAsync(f + 2 * pl, sizeof(double), P->fine.coef, sizeof(double4), sizeof(double), pl,
                                      cudaMemcpyDeviceToDevice, s));
    }
    if (diva) {
        NK_CUDA(cudaMemcpyAsync(rec + 3 * pl, P->bb, pl * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(rec + 5 * pl, P->F2, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(rec + 6 * pl, P->eta_sigma, (size_t)P->Ns * pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
}
static void load_time_state(nk_problem* P, const double* rec, bool diva) {
    const size_t pl = P->plane;
    cudaStream_t s = P->stream;
    NK_CUDA(cudaMemcpyAsync(P->H, rec, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
    NK_CUDA(cudaMemcpyAsync(P->x, rec + pl, pl * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    if (P->front.enabled) {
        const double* f = rec + (size_t)time_state_base(P, diva) * pl;
        NK_CUDA(cudaMemcpyAsync(P->mu, f, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(P->front_buf, f + pl, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (von_mises_front(P))
            NK_CUDA(cudaMemcpy2DAsync(P->fine.coef, sizeof(double4), f + 2 * pl, sizeof(double), sizeof(double), pl,
                                      cudaMemcpyDeviceToDevice, s));
    }
    if (diva) {
        NK_CUDA(cudaMemcpyAsync(P->bb, rec + 3 * pl, pl * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(P->F2, rec + 5 * pl, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(P->eta_sigma, rec + 6 * pl, (size_t)P->Ns * pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    launch_problem_geometry(P);
    NK_CHECK_LAUNCH();
}

struct TimeGradient {
    nk_problem* P;
    nk_time_gradient_desc d;
    nk_iteration_control ctl;
    nk_cost_fn cost;
    void* user;
    nk_time_gradient_stats* st;
    bool solves, diva, front;
    int N, K, S, rp, a_planes;
    size_t pl;
    double* mem = nullptr;
    // scratch planes
    double *lamH, *lamHs, *lamH0, *dv, *lamphi, *g_smb, *g_melt, *base_melt, *clipped_end, *g_logC, *g_logA;
    double *h3pre, *lamHr, *lamphi_front, *lam_eta;          // the front's reverse (lam_eta: λ of η̄H, von Mises)
    double* fmem = nullptr;                                     // its record and scratch (front_planes())
    double2 *lamF, *lwx, *lwy, *lamx_stage, *lamx_carry, *lamu_held;
    std::vector<double> hH, hu, hv, hmask, gH, gu, gv;

    ~TimeGradient() {
        if (mem) cudaFree(mem);
        if (fmem) cudaFree(fmem);
    }
    // the front's reverse: 13 work and adjoint planes (the last two one pair plane), then launch_front_record's record
    int front_planes() const { return 13 + front_record_planes(P->front.passes, P->front.calving); }
    double2* front_lamx() const { return reinterpret_cast<double2*>(fplane(11)); }
    double* fplane(int k) const { return fmem + (size_t)k * pl; }
    double* ckpt(int s) const { return mem + (size_t)s * rp * pl; }
    double* tape(int t) const { return mem + (size_t)(S + t) * rp * pl; }
    double* final_rec() const { return mem + (size_t)(S + 3 * K + 1) * rp * pl; }
    double weight(int n) const { return d.melt_weights ? d.melt_weights[n] : 1.0; }
    double* melt() const { return P->transport + P->plane; }

    void worst(int status) {
        if (status > st->worst_solve_status) st->worst_solve_status = status;
    }
    void allocate() {
        const int scratch = 27 + a_planes;
        size_t planes = (size_t)(S + 3 * K + 2) * rp + scratch;
        NK_CUDA(cudaMalloc(&mem, planes * pl * sizeof(double)));
        double* b = mem + (size_t)(S + 3 * K + 2) * rp * pl;
        auto one = [&](int k) { return b + (size_t)k * pl; };
        auto two = [&](int k) { return reinterpret_cast<double2*>(b + (size_t)k * pl); };
        lamH = one(0); lamHs = one(1); lamH0 = one(2); dv = one(3); lamphi = one(4); g_smb = one(5); g_melt = one(6);
        base_melt = one(7); clipped_end = one(8); g_logC = one(9);
        lamF = two(10); lwx = two(12); lwy = two(14); lamx_stage = two(16); lamx_carry = two(18); lamu_held = two(20);
        h3pre = one(22); lamHr = one(23); lamphi_front = one(24); lam_eta = one(25);
        if (front) NK_CUDA(cudaMalloc(&fmem, (size_t)front_planes() * pl * sizeof(double)));
        g_logA = one(27);
    }
    void solve() {
        nk_solve_stats ss{};
        picard_solve(P, &ss);
        ++st->picard_solves;
        worst(ss.status);
        if (ss.status == NK_NONFINITE) throw Failure{NK_NONFINITE, "non-finite Picard solve in the time steps"};
    }
    // step n (0-based) from the problem's state; record: the state before each stage into tape(3k + stage)
    void step(int n, bool record, int k) {
        launch_scale_plane(P->fine.g, melt(), base_melt, weight(n), P->stream);
        for (int stg = 0; stg < 3; ++stg) {
            if (record) save_time_state(P, tape(3 * k + stg), diva);
            thickness_stage(P, d.dt, stg, 0);
            if (solves) solve();
        }
    }
    // the Picard adjoint of the solve that ended in the loaded state, for x̄ = xbar and, when set, the adjoint of the
    // viscosity η̄H it left (eta_bar): λ_H += ∂J/∂H, log C, log A
    void solve_adjoint(const double2* xbar, double* lam_H, const double* eta_bar = nullptr) {
        NK_CUDA(cudaMemcpyAsync(P->adj_xbar, xbar, pl * sizeof(double2), cudaMemcpyDeviceToDevice, P->stream));
        nk_solve_stats ss{};
        picard_adjoint_device(P, ctl, true, true, &ss, eta_bar);
        ++st->picard_adjoints;
        st->adjoint_iterations += ss.picard_iterations;
        worst(ss.status);
        if (ss.status == NK_NONFINITE) throw Failure{NK_NONFINITE, "non-finite Picard adjoint in the time steps"};
        const DevGrid<double>& g = P->fine.g;
        launch_add_planes(g, lam_H, P->adj_g, 1, pl, P->stream);
        launch_add_planes(g, g_logC, P->adj_grad, 1, pl, P->stream);
        launch_add_planes(g, g_logA, P->adj_grad_A, a_planes, pl, P->stream);
        NK_CHECK_LAUNCH();
    }
    // the host's cost after `step` steps on the loaded state: J, and its gradient into lamH and the velocity adjoint
    void cost_at(int step) {
        FieldLoc fH = field_loc(P, NK_FIELD_H), fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
        FieldLoc fm = field_loc(P, NK_FIELD_ICE_MASK);
        copy_out(P, fH, hH.data());
        copy_out(P, fu, hu.data());
        copy_out(P, fv, hv.data());
        copy_out(P, fm, hmask.data());
        std::fill(gH.begin(), gH.end(), 0.0);
        std::fill(gu.begin(), gu.end(), 0.0);
        std::fill(gv.begin(), gv.end(), 0.0);
        nk_cost_state cs{step, N, hH.data(), hu.data(), hv.data(), hmask.data()};
        double J = 0.0;
        if (cost(user, &cs, &J, gH.data(), gu.data(), gv.data()) != 0) bad("the cost callback failed at step " + std::to_string(step));
        st->J += J;
        FieldLoc t = fH;
        t.base = lamHs;   // free until the stage reverse writes it
        copy_in(P, t, gH.data());
        launch_add_planes(P->fine.g, lamH, lamHs, 1, pl, P->stream);
        vector_in(P, lamx_stage, gu.data(), gv.data());
        launch_add_pairs(P->fine.g, solves ? lamx_carry : lamu_held, lamx_stage, P->stream);
        NK_CHECK_LAUNCH();
    }
    // the reverse of stage stg of step n (local k) from the loaded state tape(3k + stg): λ of its output in lamH,
    // λ of its input into lamHs (and the step start into lamH0), the velocity adjoint into lamx_stage
    void stage_reverse(int n, int k, int stg, bool after_front) {
        static const double fractions[3] = {1.0 / 3, 1.0 / 2, 1.0};
        cudaStream_t s = P->stream;
        launch_scale_plane(P->fine.g, melt(), base_melt, weight(n), s);
        ThicknessView tv = thickness_view(P, false);
        NK_CUDA(cudaMemcpyAsync((double*)tv.Hs, P->H, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync((double*)tv.H0, tape(3 * k), pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (tv.fx) launch_thickness_faces(tv, s);
        if (P->advection.scheme == NK_ADVECTION_WENO && P->advection.bounded) launch_thickness_limiter(tv, s);
        NK_CUDA(cudaMemsetAsync(lamx_stage, 0, pl * sizeof(double2), s));
        StageAdjointView a;
        a.t = tv;
        a.Hout = after_front ? h3pre : tape(3 * k + stg + 1);
        a.lam_phi_in = after_front ? lamphi_front : nullptr;
        a.bed = P->bed;
        a.rw_ri = P->pd.ocean_density / P->pd.ice_density;
        a.dtau = fractions[stg] * d.dt;
        a.melt_weight = weight(n);
        a.lam_out = lamH;
        a.lam_H0 = lamH0;
        a.lam_Hs = lamHs;
        a.lam_x = lamx_stage;
        a.lam_smb = g_smb;
        a.lam_melt = g_melt;
        a.dv = dv;
        a.lam_phi = lamphi;
        a.lamF = lamF;
        a.lw_x = lwx;
        a.lw_y = lwy;
        launch_stage_adjoint(a, s);
        NK_CHECK_LAUNCH();
    }

    // The reverse of the front's advance after the last stage of step n (local k): the stage's output before the front is
    // recomputed from the stored stage input; λ of H after the front (lamH) becomes λ of that output (lam_out), λ of Hʳ
    // passes back through the step (lamHr), and the forced cells' melt leaves λ of φ for the stage's reverse.  Von Mises
    // rates read the viscosity η̄H the stage's solve left (restored with the state): its λ (lam_eta) joins that solve's
    // adjoint; with the velocities held η̄H is held too.
    void front_reverse(int n, int k, double* lam_out) {
        static const double last = 1.0;
        cudaStream_t s = P->stream;
        load_time_state(P, tape(3 * k + 2), diva);
        launch_scale_plane(P->fine.g, melt(), base_melt, weight(n), s);
        ThicknessView tv = thickness_view(P, false);
        NK_CUDA(cudaMemcpyAsync((double*)tv.Hs, P->H, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync((double*)tv.H0, tape(3 * k), pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (tv.fx) launch_thickness_faces(tv, s);
        if (P->advection.scheme == NK_ADVECTION_WENO && P->advection.bounded) launch_thickness_limiter(tv, s);
        launch_thickness_stage(tv, last * d.dt, 1, s);   // P->H = the output before the front (the clip is restored at the end)
        NK_CUDA(cudaMemcpyAsync(h3pre, P->H, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        // the advance again on copies, recorded pass by pass
        FrontView rec = front_view(P, false);
        rec.H = fplane(4);
        rec.mu = fplane(5);
        rec.Hr = fplane(6);
        NK_CUDA(cudaMemcpyAsync(rec.H, h3pre, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(rec.mu, P->mu, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(rec.Hr, P->front_buf, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        launch_front_record(rec, P->front.passes, pl, fplane(13), last * d.dt, s);
        FrontAdjointView fa;
        fa.f = front_view(P, false);
        fa.f.H = h3pre;
        fa.passes = P->front.passes;
        fa.snaps = fplane(13);
        fa.plane = pl;
        fa.dt = last * d.dt;
        fa.melt_weight = weight(n);
        fa.lam_H = lamH;
        fa.lam_Hr = lamHr;
        fa.lam_H3 = lam_out;
        fa.lam_smb = g_smb;
        fa.lam_melt = g_melt;
        fa.lam_phi = lamphi_front;
        fa.lam_a = fplane(0);
        fa.lam_b = fplane(1);
        fa.lam_c = fplane(2);
        fa.lam_d = fplane(3);
        fa.lam_e = fplane(7);
        fa.lam_f = fplane(8);
        fa.lam_g = fplane(9);
        fa.lam_h = fplane(10);
        fa.lam_x = front_lamx();
        fa.lam_eta = von_mises_front(P) && solves ? lam_eta : nullptr;
        NK_CUDA(cudaMemsetAsync(fa.lam_x, 0, pl * sizeof(double2), s));
        launch_front_adjoint(fa, s);
        NK_CHECK_LAUNCH();
    }

    void run(nk_time_gradient_stats* stats) {
        st = stats;
        cudaStream_t s = P->stream;
        const DevGrid<double>& g = P->fine.g;
        ensure_transport(P);
        if (solves) ensure_adjoint(P, true);
        allocate();
        // ---- forward: the checkpoints ----
        launch_problem_geometry(P);
        NK_CUDA(cudaMemcpyAsync(base_melt, melt(), pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        for (int sg = 0; sg < S; ++sg) {
            save_time_state(P, ckpt(sg), diva);
            for (int k = 0; k < std::min(K, N - sg * K); ++k) step(sg * K + k, false, k);
        }
        save_time_state(P, final_rec(), diva);
        NK_CUDA(cudaMemcpyAsync(clipped_end, P->transport + 3 * pl, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        // ---- reverse, one segment at a time ----
        for (double* z : {lamH, g_smb, g_melt, g_logC, lamHr}) NK_CUDA(cudaMemsetAsync(z, 0, pl * sizeof(double), s));
        NK_CUDA(cudaMemsetAsync(g_logA, 0, (size_t)a_planes * pl * sizeof(double), s));
        for (double2* z : {lamx_carry, lamu_held, lamF, lwx, lwy}) NK_CUDA(cudaMemsetAsync(z, 0, pl * sizeof(double2), s));
        double* lam = lamH;      // λ of the current thickness (the buffers swap roles as the sweep moves back)
        double* lam_in = lamHs;
        for (int sg = S - 1; sg >= 0; --sg) {
            const int n0 = sg * K, len = std::min(K, N - n0);
            load_time_state(P, ckpt(sg), diva);
            for (int k = 0; k < len; ++k) step(n0 + k, true, k);
            save_time_state(P, tape(3 * len), diva);
            for (int k = len - 1; k >= 0; --k) {
                const int n = n0 + k;
                load_time_state(P, tape(3 * k + 3), diva);
                lamH = lam;
                lamHs = lam_in;
                cost_at(n + 1);
                if (solves) {
                    solve_adjoint(lamx_carry, lam);
                    NK_CUDA(cudaMemsetAsync(lamx_carry, 0, pl * sizeof(double2), s));
                }
                NK_CUDA(cudaMemsetAsync(lamH0, 0, pl * sizeof(double), s));
                if (front) {
                    lamH = lam;
                    front_reverse(n, k, lam_in);
                    std::swap(lam, lam_in);
                }
                for (int stg = 2; stg >= 0; --stg) {
                    load_time_state(P, tape(3 * k + stg), diva);
                    lamH = lam;
                    lamHs = lam_in;
                    stage_reverse(n, k, stg, front && stg == 2);
                    if (front && stg == 2 && P->front.calving != NK_CALVING_NONE)   // the calving rates read the stage's velocities
                        launch_add_pairs(g, lamx_stage, front_lamx(), s);
                    if (stg > 0) {
                        // the solve that made x_t from H_t (and, before the front, η̄H)
                        if (solves) solve_adjoint(lamx_stage, lam_in, front && stg == 2 && von_mises_front(P) ? lam_eta : nullptr);
                        else launch_add_pairs(g, lamu_held, lamx_stage, s);
                    } else {
                        launch_add_planes(g, lam_in, lamH0, 1, pl, s);  // stage 1 reads H⁻ as its stage thickness
                        if (solves) NK_CUDA(cudaMemcpyAsync(lamx_carry, lamx_stage, pl * sizeof(double2), cudaMemcpyDeviceToDevice, s));
                        else launch_add_pairs(g, lamu_held, lamx_stage, s);
                    }
                    NK_CHECK_LAUNCH();
                    std::swap(lam, lam_in);
                }
            }
        }
        lamH = lam;
        lamHs = lam_in;
        // ---- back to the final state ----
        load_time_state(P, final_rec(), diva);
        NK_CUDA(cudaMemcpyAsync(P->transport + 3 * pl, clipped_end, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaMemcpyAsync(melt(), base_melt, pl * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NK_CUDA(cudaStreamSynchronize(s));
    }
    void copy_results(const nk_time_gradient* out) {
        FieldLoc f = field_loc(P, NK_FIELD_H);
        auto plane_out = [&](double* host, double* dev, int planes) {
            if (!host) return;
            FieldLoc t = f;
            t.base = dev;
            t.planes = planes;
            copy_out(P, t, host);
        };
        plane_out(out->grad_H, lamH, 1);
        plane_out(out->grad_smb, g_smb, 1);
        plane_out(out->grad_melt, g_melt, 1);
        plane_out(out->grad_log_C, g_logC, 1);
        plane_out(out->grad_log_A, g_logA, a_planes);
        if (out->grad_u && out->grad_v) vector_out(P, solves ? lamx_carry : lamu_held, out->grad_u, out->grad_v);
    }
};
}  // namespace nk

extern "C" {

nk_status nk_checkpointed_gradient(nk_problem* P, const nk_time_gradient_desc* desc, nk_cost_fn cost, void* user,
                                   const nk_time_gradient* out, nk_time_gradient_stats* stats) {
    if (!P || !desc || !cost) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        auto t0 = std::chrono::steady_clock::now();
        check_thickness_step(P, desc->dt);
        if (desc->steps < 1) bad("steps must be at least 1");
        if (desc->checkpoint_interval < 0) bad("checkpoint_interval must be non-negative");
        if (desc->velocity_solves != 0 && desc->velocity_solves != 1) bad("velocity_solves is 0 or 1");
        if (desc->velocity_solves && P->ud) bad("the gradient through velocity solves is not available with prescribed velocities");
        if (desc->melt_weights)
            for (int n = 0; n < desc->steps; ++n)
                if (!std::isfinite(desc->melt_weights[n])) bad("melt weights must be finite");
        TimeGradient tg;
        tg.P = P;
        tg.d = *desc;
        tg.ctl = desc->adjoint_control ? *desc->adjoint_control : P->sd.picard;
        if (tg.ctl.kind != NK_CONVERGENCE && tg.ctl.kind != NK_FIXED_ITERATIONS) bad("the adjoint takes Convergence or FixedIterations");
        if (tg.ctl.kind == NK_FIXED_ITERATIONS ? tg.ctl.iterations < 0 : tg.ctl.maxiter < 0) bad("negative iteration count");
        tg.cost = cost;
        tg.user = user;
        tg.solves = desc->velocity_solves != 0;
        tg.diva = P->pd.stress_balance == NK_DIVA;
        tg.front = P->front.enabled != 0;
        tg.N = desc->steps;
        tg.K = desc->checkpoint_interval > 0 ? std::min(desc->checkpoint_interval, tg.N)
                                             : (int)std::ceil(std::sqrt((double)tg.N) - 1e-12);
        tg.S = (tg.N + tg.K - 1) / tg.K;
        tg.rp = time_state_planes(P, tg.diva);
        tg.a_planes = P->pd.rate_factor_layout == NK_RATE_FACTOR_SIGMA ? P->Ns : 1;
        tg.pl = P->plane;
        auto count = [&](int id) { FieldLoc f = field_loc(P, id); return (size_t)f.nx * f.ny * f.planes; };
        tg.hH.resize(count(NK_FIELD_H));
        tg.gH.resize(tg.hH.size());
        tg.hmask.resize(count(NK_FIELD_ICE_MASK));
        tg.hu.resize(count(NK_FIELD_U));
        tg.gu.resize(tg.hu.size());
        tg.hv.resize(count(NK_FIELD_V));
        tg.gv.resize(tg.hv.size());
        nk_time_gradient_stats local{};
        nk_time_gradient_stats* st = stats ? stats : &local;
        std::memset(st, 0, sizeof(*st));
        st->segments = tg.S;
        tg.run(st);
        if (out) tg.copy_results(out);
        st->elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
}

nk_status nk_picard_solve(nk_problem* P, nk_solve_stats* stats) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        nk_solve_stats local{};
        nk_solve_stats* st = stats ? stats : &local;
        NK_CUDA(cudaEventRecord(P->ev0, P->stream));
        picard_solve(P, st);
        NK_CUDA(cudaEventRecord(P->ev1, P->stream));
        NK_CUDA(cudaEventSynchronize(P->ev1));
        event_times(P, st);
        if (st->status == NK_NONFINITE) throw Failure{NK_NONFINITE, "non-finite velocity change"};
    });
}

nk_status nk_picard_solve_async(nk_problem* P) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (!use_graphs(P)) bad("asynchronous solves need CUDA graphs (NK_SOLVER_HOST_LOOP or NK_GRAPHS=0 is set)");
        if (!P->picard_exec) build_picard_graph(P);
        set_control(P);
        NK_CUDA(cudaEventRecord(P->ev0, P->stream));
        impose_prescribed(P, P->ud);
        NK_CUDA(cudaGraphLaunch(P->picard_exec, P->stream));
        NK_CUDA(cudaMemcpyAsync(P->sc_host, P->sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, P->stream));
        NK_CUDA(cudaEventRecord(P->ev1, P->stream));
        P->async_pending = true;
    });
}

nk_status nk_problem_query(nk_problem* P, int32_t* done) {
    if (!P || !done) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (!P->async_pending) bad("no asynchronous solve pending");
        cudaError_t e = cudaEventQuery(P->ev1);
        if (e == cudaErrorNotReady) {
            *done = 0;
            return;
        }
        NK_CUDA(e);
        *done = 1;
    });
}

nk_status nk_problem_wait(nk_problem* P, nk_solve_stats* stats) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        if (!P->async_pending) bad("no asynchronous solve pending");
        NK_CUDA(cudaEventSynchronize(P->ev1));
        P->async_pending = false;
        nk_solve_stats local{};
        nk_solve_stats* st = stats ? stats : &local;
        fill_stats(P, st, true);
        const SolverScalars& h = *P->sc_host;
        count_launches(P->picard_kernels[0] + (long long)h.p_it * P->picard_kernels[1] + (long long)h.it_total * P->picard_kernels[2]);
        event_times(P, st);
        if (st->status == NK_NONFINITE) throw Failure{NK_NONFINITE, "non-finite velocity change"};
    });
}

nk_status nk_solve_velocities(nk_problem* P, double* u, double* v, nk_solve_stats* stats) {
    if (!P || !u || !v) return NK_BAD_ARGUMENT;
    nk_status st = guarded(P->ctx, [&] {
        FieldLoc fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
        copy_in(P, fu, u);
        copy_in(P, fv, v);
    });
    if (st != NK_OK) return st;
    st = nk_picard_solve(P, stats);
    if (st != NK_OK) return st;
    return guarded(P->ctx, [&] {
        FieldLoc fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
        copy_out(P, fu, u);
        copy_out(P, fv, v);
    });
}

nk_status nk_velocity_profile(nk_problem* P) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        launch_velocity_profile(P->phys(), P->pd.stress_balance == NK_DIVA, P->x, P->bb, P->F2, P->eta_sigma, P->ub, P->usig, P->stream);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_multigrid_levels(const nk_problem* P, int32_t* count, int32_t* nx, int32_t* ny, int32_t capacity) {
    if (!P || !count) return NK_BAD_ARGUMENT;
    *count = P->nlevels;
    for (int l = 0; l < P->nlevels && l < capacity; ++l) {
        nx[l] = P->mixed ? P->lv32[l + 1].Nx : P->lv64[l + 1].Nx;
        ny[l] = P->mixed ? P->lv32[l + 1].Ny : P->lv64[l + 1].Ny;
    }
    return NK_OK;
}

static nk_status transfer(nk_problem* P, int32_t level, const double* au, const double* av, double* bu, double* bv, bool restrict_) {
    return guarded(P->ctx, [&] {
        if (P->precond != NK_PRECONDITIONER_MULTIGRID || level < 0 || level >= P->nlevels) bad("no such multigrid level");
        if (P->mixed) bad("the standalone transfers use the FP64 hierarchy (precision = FP64)");
        update_preconditioner(P);
        Level<double>& Lf = P->lv64[level];
        Level<double>& Lc = P->lv64[level + 1];
        LevelView<double> vf = P->level_view(Lf), vc = P->level_view(Lc);
        int fnx = Lf.Nx, fny = Lf.Ny, cnx = Lc.Nx, cny = Lc.Ny;
        int ffx = P->px ? fnx : fnx + 1, ffy = P->py ? fny : fny + 1;
        int cfx = P->px ? cnx : cnx + 1, cfy = P->py ? cny : cny + 1;
        auto in = [&](double2* dst, int pitch, size_t plane, int nfx, int ny_u, int nx_v, int nfy, const double* u, const double* v) {
            NK_CUDA(cudaMemsetAsync(dst, 0, plane * sizeof(double2), P->stream));
            NK_CUDA(cudaMemcpyAsync(P->staging, u, (size_t)nfx * ny_u * sizeof(double), cudaMemcpyHostToDevice, P->stream));
            launch_pack((double*)dst, pitch, (int)plane, 2, 0, P->staging, nfx, ny_u, 1, P->stream);
            NK_CUDA(cudaStreamSynchronize(P->stream));
            NK_CUDA(cudaMemcpyAsync(P->staging, v, (size_t)nx_v * nfy * sizeof(double), cudaMemcpyHostToDevice, P->stream));
            launch_pack((double*)dst, pitch, (int)plane, 2, 1, P->staging, nx_v, nfy, 1, P->stream);
            NK_CUDA(cudaStreamSynchronize(P->stream));
        };
        auto out = [&](const double2* src, int pitch, size_t plane, int nfx, int ny_u, int nx_v, int nfy, double* u, double* v) {
            launch_unpack(P->staging, (const double*)src, pitch, (int)plane, 2, 0, nfx, ny_u, 1, P->stream);
            NK_CUDA(cudaMemcpyAsync(u, P->staging, (size_t)nfx * ny_u * sizeof(double), cudaMemcpyDeviceToHost, P->stream));
            NK_CUDA(cudaStreamSynchronize(P->stream));
            launch_unpack(P->staging, (const double*)src, pitch, (int)plane, 2, 1, nx_v, nfy, 1, P->stream);
            NK_CUDA(cudaMemcpyAsync(v, P->staging, (size_t)nx_v * nfy * sizeof(double), cudaMemcpyDeviceToHost, P->stream));
            NK_CUDA(cudaStreamSynchronize(P->stream));
        };
        double2* fbuf = Lf.q;   // scratch vectors of the two levels
        double2* cbuf = Lc.x2;
        if (restrict_) {
            in(fbuf, Lf.pitch, Lf.plane(), ffx, fny, fnx, ffy, au, av);
            NK_CUDA(cudaMemsetAsync(cbuf, 0, Lc.plane() * sizeof(double2), P->stream));
            launch_restrict<double>(vc, vf, fbuf, cbuf, nullptr, nullptr, P->stream);
            NK_CHECK_LAUNCH();
            out(cbuf, Lc.pitch, Lc.plane(), cfx, cny, cnx, cfy, bu, bv);
        } else {
            in(cbuf, Lc.pitch, Lc.plane(), cfx, cny, cnx, cfy, au, av);
            in(fbuf, Lf.pitch, Lf.plane(), ffx, fny, fnx, ffy, bu, bv);
            launch_prolongate<double>(vf, vc, fbuf, cbuf, nullptr, P->stream);
            NK_CHECK_LAUNCH();
            out(fbuf, Lf.pitch, Lf.plane(), ffx, fny, fnx, ffy, bu, bv);
        }
    });
}

nk_status nk_multigrid_restrict(nk_problem* P, int32_t level, const double* fine_u, const double* fine_v, double* coarse_u, double* coarse_v) {
    if (!P || !fine_u || !fine_v || !coarse_u || !coarse_v) return NK_BAD_ARGUMENT;
    return transfer(P, level, fine_u, fine_v, coarse_u, coarse_v, true);
}

nk_status nk_multigrid_prolongate(nk_problem* P, int32_t level, const double* coarse_u, const double* coarse_v, double* fine_u, double* fine_v) {
    if (!P || !coarse_u || !coarse_v || !fine_u || !fine_v) return NK_BAD_ARGUMENT;
    return transfer(P, level, coarse_u, coarse_v, fine_u, fine_v, false);
}

nk_status nk_time_kernel(nk_problem* P, int32_t kernel, int32_t repeats, int64_t flush_bytes, double* mean_ms, double* bytes_per_launch) {
    if (!P || !mean_ms || !bytes_per_launch || repeats < 1 || flush_bytes < 0) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        cudaStream_t s = P->stream;
        double cells = (double)P->Nx * P->Ny;
        char* flush = nullptr;
        if (flush_bytes > 0) NK_CUDA(cudaMalloc((void**)&flush, (size_t)flush_bytes));
        double total = 0.0;
        double bytes = 0.0;
        ThicknessView tv{};
        EnergyView ev{};
        auto launch = [&]() {
            if (kernel == NK_KERNEL_OPERATOR_FP64) {
                launch_apply(P->fine_op(), P->p, P->q, s);
            } else if (kernel == NK_KERNEL_SMOOTHER) {
                if (P->precond != NK_PRECONDITIONER_MULTIGRID) bad("the smoother needs the multigrid preconditioner");
                if (P->mixed) {
                    LevelView<float> v = P->level_view(P->lv32[0]);
                    launch_smooth_point<float>(v, v.x, v.x2, 0, nullptr, s);
                } else {
                    LevelView<double> v = P->level_view(P->lv64[0]);
                    launch_smooth_point<double>(v, v.x, v.x2, 0, nullptr, s);
                }
            } else if (kernel == NK_KERNEL_CG_UPDATE) {
                CGView v = P->cg_view(P->tau);
                launch_cg_update(v, s);
            } else if (kernel == NK_KERNEL_THICKNESS_STAGE) {
                launch_thickness_stage(tv, 1.0, 0, s);
            } else if (kernel == NK_KERNEL_THICKNESS_LIMITER) {
                launch_thickness_limiter(tv, s);
            } else if (kernel == NK_KERNEL_THICKNESS_FACES) {
                launch_thickness_faces(tv, s);
            } else if (kernel == NK_KERNEL_STEP_ENTHALPY) {
                launch_step_enthalpy(ev, 1.0, s);
            } else {
                bad("unknown kernel id");
            }
        };
        const bool bounded = P->advection.scheme == NK_ADVECTION_WENO && P->advection.bounded;
        const bool weno = P->advection.scheme == NK_ADVECTION_WENO;
        if (kernel == NK_KERNEL_OPERATOR_FP64) bytes = cells * (16 + 32 + 1 + 16);
        else if (kernel == NK_KERNEL_SMOOTHER) bytes = cells * (P->mixed ? (8 + 8 + 8 + 16 + 1 + 8) : (16 + 16 + 16 + 32 + 1 + 16));
        else if (kernel == NK_KERNEL_CG_UPDATE) bytes = cells * (64 + 32 + (P->precond == NK_PRECONDITIONER_DIAGONAL ? 16 + 16 : 0));
        // Hs, H⁻, a, m, (u, v), H written; φ with a grounding treatment; θ for a bounded WENO
        // (a WENO stage reads the face reconstructions, one pair per x and per y face of the cell, instead of the stencils)
        else if (kernel == NK_KERNEL_THICKNESS_STAGE)
            bytes = cells * (8 + 8 + 8 + 8 + 16 + 8 + (P->pd.grounding ? 8 : 0) + (bounded ? 8 : 0) + (weno ? 32 : 0));
        else if (kernel == NK_KERNEL_THICKNESS_LIMITER) bytes = cells * (8 + 8 + 32);
        else if (kernel == NK_KERNEL_THICKNESS_FACES) bytes = cells * (8 + 32);
        // per column: H, Hⁿ, φ, m, mᵍ, G, Tₛ, Tₒ, H_w, (u, v), (uᵇ, vᵇ) and the drag; per layer E_old, η, (uσ, vσ) read and E,
        // T, ω, Φ written
        else if (kernel == NK_KERNEL_STEP_ENTHALPY) bytes = cells * 8 * (11 + 8.0 * P->Ns);
        if (kernel == NK_KERNEL_THICKNESS_STAGE || kernel == NK_KERNEL_THICKNESS_LIMITER || kernel == NK_KERNEL_THICKNESS_FACES) {
            tv = thickness_view(P, false);
            if (kernel == NK_KERNEL_THICKNESS_FACES && !tv.fx) bad("the face reconstructions belong to the WENO schemes");
            NK_CUDA(cudaMemcpyAsync((double*)tv.Hs, P->H, P->plane * sizeof(double), cudaMemcpyDeviceToDevice, s));
            NK_CUDA(cudaMemcpyAsync((double*)tv.H0, P->H, P->plane * sizeof(double), cudaMemcpyDeviceToDevice, s));
            if (tv.fx) launch_thickness_faces(tv, s);
            if (kernel == NK_KERNEL_THICKNESS_STAGE && !bounded) tv.bounded = 0;
            if (kernel == NK_KERNEL_THICKNESS_STAGE && bounded) launch_thickness_limiter(tv, s);
        } else if (kernel == NK_KERNEL_STEP_ENTHALPY) {
            if (P->pd.rate_factor_layout != NK_RATE_FACTOR_SIGMA || P->Ns > ENERGY_MAX_LAYERS) bad("the energy step needs the sigma rate factor");
            nk_energy_params q = default_energy_params();
            ev = energy_view(P, &q);
            NK_CUDA(cudaMemcpyAsync(const_cast<double*>(ev.E_old), P->thermal, (size_t)P->Ns * P->plane * sizeof(double), cudaMemcpyDeviceToDevice, s));
        }
        if (kernel == NK_KERNEL_CG_UPDATE) {
            // run the update with done = 0 so it is not skipped
            P->sc_host->done = 0;
            NK_CUDA(cudaMemcpyAsync(&P->sc->done, &P->sc_host->done, sizeof(int), cudaMemcpyHostToDevice, s));
        }
        for (int rep = 0; rep < repeats; ++rep) {
            if (flush) NK_CUDA(cudaMemsetAsync(flush, rep & 0xff, (size_t)flush_bytes, s));
            NK_CUDA(cudaEventRecord(P->ev0, s));
            launch();
            NK_CUDA(cudaEventRecord(P->ev1, s));
            NK_CUDA(cudaEventSynchronize(P->ev1));
            NK_CHECK_LAUNCH();
            float ms = 0;
            NK_CUDA(cudaEventElapsedTime(&ms, P->ev0, P->ev1));
            total += ms;
        }
        if (flush) cudaFree(flush);
        *mean_ms = total / repeats;
        *bytes_per_launch = bytes;
    });
}

}  // extern "C"

// =================================================================================================================
// Batched solves: problems of one configuration in one allocation at a fixed stride, solved by one graph whose
// launches cover every slot (gridDim.z = slots, the kernels' NK_BATCH_ENTER moving each block to its slot).
// =================================================================================================================
struct nk_batch {
    nk_context* ctx = nullptr;
    int slots = 0;
    size_t stride = 0;                   // bytes between two slots' arenas (a multiple of 256)
    char* base = nullptr;                // slots * stride bytes of arenas, then the loop counters
    char* pinned = nullptr;              // the slots' own scalars, the control records, the results, the counters
    bool external = false;               // base and pinned belong to a server
    int* counters = nullptr;             // device: Picard and CG loop bodies run by the last solve
    SolverScalars* control = nullptr;    // pinned, one per slot: the solver settings, p_done = 1 for idle slots
    SolverScalars* results = nullptr;    // pinned, one per slot: the scalars after the solve
    int* counters_host = nullptr;        // pinned copy of `counters`
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<nk_problem*> P;
    std::vector<uint8_t> active;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels[3] = {0, 0, 0};    // kernel nodes: top level, Picard body, CG body
    bool pending = false;
};

namespace nk {

static_assert(sizeof(SolverScalars) <= 256, "a slot's pinned scalars take one 256-byte record");
static size_t batch_pinned_bytes(int slots) { return (size_t)slots * (256 + 2 * sizeof(SolverScalars)) + 256; }
static size_t batch_device_bytes(size_t stride, int slots) { return stride * (size_t)slots + 256; }

// Device footprint of one problem of this configuration, rounded up to 256 bytes: the slot stride.
static size_t batch_stride(const nk_grid_desc* g, const nk_physics_desc* p, const nk_solver_desc* s) {
    nk_problem probe;
    probe.gd = *g;
    probe.pd = *p;
    probe.sd = *s;
    build(&probe, true);
    return (probe.arena.size + 255) / 256 * 256;
}

// The slot stride and the address of slot 0's Picard flag in every grid of P's hierarchy (0 and null: unbatched).
static void set_batch_grids(nk_problem* P, long long stride) {
    const int* pd = stride ? &P->sc->p_done : nullptr;
    P->fine.g.slot_stride = stride;
    P->fine.g.p_done = pd;
    for (auto& L : P->lv64) { L.g.slot_stride = stride; L.g.p_done = pd; }
    for (auto& L : P->lv32) { L.g.slot_stride = stride; L.g.p_done = pd; }
}

// The graph of build_picard_graph over every slot, captured from slot 0's problem: the kernels' stopping decisions
// stay per slot (p_done, done), and the loop conditions come from k_batch_condition over all slots:
//   picard_begin ─► any(Picard) ─► WHILE { x⁻ = x ─► coefficients ─► CG start ─► any(CG)
//                                          ─► WHILE { CG step ─► any(CG) } ─► picard_end ─► any(Picard) }
static void build_batch_graph(nk_batch* B) {
    nk_problem* P = B->P[0];
    autotune_strips(P);
    long long stride = (long long)B->stride;
    int S = B->slots;
    int* cp = B->counters;
    int* cc = B->counters + 1;
    set_batch_grids(P, stride);
    try {
        BatchScope scope(S);
        cudaGraph_t g;
        NK_CUDA(cudaGraphCreate(&g, 0));
        B->graph = g;
        cudaGraphConditionalHandle hp;
        NK_CUDA(cudaGraphConditionalHandleCreate(&hp, g, 0, 0));
        capture_into(P, g, {}, [&] {
            launch_picard_begin(P->sc, 0, stride, P->stream);
            launch_batch_condition(P->sc, stride, S, 0, hp, cp, P->stream);
        });
        cudaGraph_t body = add_while(g, leaves(g), hp);
        cudaGraphConditionalHandle hc;
        NK_CUDA(cudaGraphConditionalHandleCreate(&hc, body, 0, 0));
        CGView v = P->cg_view(P->tau);   // its grids carry the stride (set above)
        v.cond = 0;
        capture_into(P, body, {}, [&] {
            launch_copy_range(P->fine.g, P->xprev, P->x, P->stream);
            update_coefficients(P);
            cg_start(P, v);
            launch_batch_condition(P->sc, stride, S, 1, hc, cc, P->stream);
        });
        cudaGraph_t cg_body = add_while(body, leaves(body), hc);
        capture_into(P, cg_body, {}, [&] {
            cg_step(P, v);
            launch_batch_condition(P->sc, stride, S, 1, hc, cc, P->stream);
        });
        capture_into(P, body, leaves(body), [&] {
            picard_end(P, 0);
            launch_batch_condition(P->sc, stride, S, 0, hp, cp, P->stream);
        });
        B->kernels[0] = kernel_nodes(g);
        B->kernels[1] = kernel_nodes(body);
        B->kernels[2] = kernel_nodes(cg_body);
        NK_CUDA(cudaGraphInstantiate(&B->exec, g, 0));
    } catch (...) {
        set_batch_grids(P, 0);
        throw;
    }
    set_batch_grids(P, 0);
}

// Offsets of the buffers the solve graph reaches, relative to the arena: equal in every slot by construction
// (build is deterministic), checked once because the batched kernels rely on it.
static std::vector<long long> arena_offsets(const nk_problem* P) {
    const char* b = P->arena.base;
    auto off = [&](const void* q) { return q ? (long long)((const char*)q - b) : -1ll; };
    std::vector<long long> o = {(long long)P->arena.size, off(P->sc), off(P->x), off(P->tau), off(P->partials), off(P->fine.coef),
                                off(P->fine.metrics), off(P->fine.mask), off(P->H), off(P->A2), off(P->A3), off(P->sig_tables)};
    for (const auto& L : P->lv64) { o.push_back(off(L.x)); o.push_back(off(L.metrics)); o.push_back(off(L.coef)); }
    for (const auto& L : P->lv32) { o.push_back(off(L.x)); o.push_back(off(L.metrics)); o.push_back(off(L.coef)); }
    return o;
}

static void batch_free(nk_batch* B) {
    if (!B) return;
    if (B->ctx) cudaSetDevice(B->ctx->device);
    if (B->stream) cudaStreamSynchronize(B->stream);
    for (nk_problem* P : B->P) nk_problem_destroy(P);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    if (B->ev0) cudaEventDestroy(B->ev0);
    if (B->ev1) cudaEventDestroy(B->ev1);
    if (B->stream) cudaStreamDestroy(B->stream);
    if (!B->external) {
        if (B->base) cudaFree(B->base);
        if (B->pinned) cudaFreeHost(B->pinned);
    }
    delete B;
}

// `device_base` (batch_device_bytes) and `pinned_base` (batch_pinned_bytes) from a server, or null to allocate.
static nk_status batch_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics, const nk_solver_desc* solver,
                              int slots, char* device_base, char* pinned_base, nk_batch** out) {
    if (!ctx || !grid || !physics || !solver || !out) return NK_BAD_ARGUMENT;
    auto* B = new nk_batch();
    B->ctx = ctx;
    B->slots = slots;
    nk_status st = guarded(ctx, [&] {
        if (slots < 1 || slots > NK_MAX_BATCH_SLOTS) bad("batch slots out of range (1 .. NK_MAX_BATCH_SLOTS)");
        if (solver->flags & NK_SOLVER_HOST_LOOP) bad("batched solves run as CUDA graphs: NK_SOLVER_HOST_LOOP is set");
        if (solver->precision == NK_PRECISION_MIXED && solver->preconditioner == NK_PRECONDITIONER_MULTIGRID && coarse_cells_limit() > 0)
            bad("fused coarse multigrid levels (NK_COARSE_CELLS > 0) are not batched");
        if (grid->Nx < 1 || grid->Ny < 1 || grid->Nsigma < 1 || grid->Nsigma > MAX_SIGMA) bad("grid size or Nsigma out of range");
        B->stride = batch_stride(grid, physics, solver);
        if (device_base) {
            B->base = device_base;
            B->pinned = pinned_base;
            B->external = true;
        } else {
            NK_CUDA(cudaMalloc((void**)&B->base, batch_device_bytes(B->stride, slots)));
            NK_CUDA(cudaHostAlloc((void**)&B->pinned, batch_pinned_bytes(slots), cudaHostAllocDefault));
        }
        B->counters = reinterpret_cast<int*>(B->base + B->stride * (size_t)slots);
        B->control = reinterpret_cast<SolverScalars*>(B->pinned + (size_t)slots * 256);
        B->results = B->control + slots;
        B->counters_host = reinterpret_cast<int*>(B->results + slots);
        B->active.assign(slots, 0);
        NK_CUDA(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
        NK_CUDA(cudaEventCreate(&B->ev0));
        NK_CUDA(cudaEventCreate(&B->ev1));
        for (int k = 0; k < slots; ++k) {
            nk_problem* P = nullptr;
            nk_status ps = problem_create(ctx, grid, physics, solver, &P, B->base + B->stride * (size_t)k,
                                          reinterpret_cast<SolverScalars*>(B->pinned + (size_t)k * 256));
            if (ps != NK_OK) throw Failure{ps, ctx->error};
            NK_CUDA(cudaStreamDestroy(P->stream));
            P->stream = B->stream;
            P->external_stream = true;
            B->P.push_back(P);
        }
        if (!use_graphs(B->P[0])) bad("batched solves run as CUDA graphs: NK_GRAPHS=0 is set");
        std::vector<long long> o0 = arena_offsets(B->P[0]);
        for (int k = 1; k < slots; ++k)
            if (arena_offsets(B->P[k]) != o0) bad("batch slots with different arena layouts");
        if ((size_t)o0[0] > B->stride) bad("batch slot larger than its stride");
        build_batch_graph(B);
        NK_CUDA(cudaStreamSynchronize(B->stream));
    });
    if (st != NK_OK) {
        batch_free(B);
        return st;
    }
    *out = B;
    return NK_OK;
}

// Scalars of every slot between pinned records (one SolverScalars each) and the slots' arenas.
static void batch_scalars(nk_batch* B, SolverScalars* host, bool to_device) {
    SolverScalars* dev = B->P[0]->sc;
    size_t w = sizeof(SolverScalars);
    if (B->stride <= (size_t)1 << 30) {   // one strided copy
        if (to_device) NK_CUDA(cudaMemcpy2DAsync(dev, B->stride, host, w, w, B->slots, cudaMemcpyHostToDevice, B->stream));
        else NK_CUDA(cudaMemcpy2DAsync(host, w, dev, B->stride, w, B->slots, cudaMemcpyDeviceToHost, B->stream));
        return;
    }
    for (int k = 0; k < B->slots; ++k) {   // slots too far apart for a pitched copy
        SolverScalars* d = B->P[k]->sc;
        if (to_device) NK_CUDA(cudaMemcpyAsync(d, host + k, w, cudaMemcpyHostToDevice, B->stream));
        else NK_CUDA(cudaMemcpyAsync(host + k, d, w, cudaMemcpyDeviceToHost, B->stream));
    }
}

static void batch_solve_async(nk_batch* B, const uint8_t* active) {
    if (B->pending) bad("a batched solve is pending (nk_batch_wait first)");
    SolverScalars h = control_scalars(B->P[0]);
    for (int k = 0; k < B->slots; ++k) {
        uint8_t a = active ? (active[k] != 0) : 1;
        if (a && B->P[k]->ud) bad("batch slot " + std::to_string(k) + " has prescribed velocities, which batched solves do not take");
        B->active[k] = a;
        B->control[k] = h;
        B->control[k].p_done = !a;
    }
    batch_scalars(B, B->control, true);
    NK_CUDA(cudaMemsetAsync(B->counters, 0, 2 * sizeof(int), B->stream));
    NK_CUDA(cudaEventRecord(B->ev0, B->stream));
    NK_CUDA(cudaGraphLaunch(B->exec, B->stream));
    NK_CUDA(cudaEventRecord(B->ev1, B->stream));
    batch_scalars(B, B->results, false);
    NK_CUDA(cudaMemcpyAsync(B->counters_host, B->counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, B->stream));
    B->pending = true;
}

// Statistics of every slot after the pending solve has finished (the caller has waited on the stream).
static bool batch_finish(nk_batch* B, nk_solve_stats* stats) {
    B->pending = false;
    float ms = 0, a = 0, b = 0;
    NK_CUDA(cudaEventElapsedTime(&ms, B->ev0, B->ev1));
    NK_CUDA(cudaEventElapsedTime(&a, B->ctx->ref, B->ev0));
    NK_CUDA(cudaEventElapsedTime(&b, B->ctx->ref, B->ev1));
    bool nonfinite = false;
    for (int k = 0; k < B->slots; ++k) {
        nk_solve_stats st{};
        if (B->active[k]) {
            fill_stats_from(B->results[k], &st, true);
            st.device_ms = ms;
            st.device_start_ms = a;
            st.device_end_ms = b;
            nonfinite = nonfinite || st.status == NK_NONFINITE;
        }
        if (stats) stats[k] = st;
    }
    count_launches(B->kernels[0] + (long long)B->counters_host[0] * B->kernels[1] + (long long)B->counters_host[1] * B->kernels[2]);
    return !nonfinite;
}

}  // namespace nk

extern "C" {

nk_status nk_batch_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics, const nk_solver_desc* solver,
                          int32_t slots, nk_batch** out) {
    return batch_create(ctx, grid, physics, solver, slots, nullptr, nullptr, out);
}

nk_status nk_batch_destroy(nk_batch* B) {
    batch_free(B);
    return NK_OK;
}

int32_t nk_batch_slots(const nk_batch* B) { return B ? B->slots : 0; }

nk_problem* nk_batch_problem(nk_batch* B, int32_t slot) {
    if (!B || slot < 0 || slot >= B->slots) return nullptr;
    return B->P[slot];
}

nk_status nk_batch_picard_solve_async(nk_batch* B, const uint8_t* active) {
    if (!B) return NK_BAD_ARGUMENT;
    return guarded(B->ctx, [&] { batch_solve_async(B, active); });
}

nk_status nk_batch_query(nk_batch* B, int32_t* done) {
    if (!B || !done) return NK_BAD_ARGUMENT;
    return guarded(B->ctx, [&] {
        if (!B->pending) bad("no batched solve pending");
        cudaError_t e = cudaEventQuery(B->ev1);
        if (e == cudaErrorNotReady) {
            *done = 0;
            return;
        }
        NK_CUDA(e);
        *done = 1;
    });
}

nk_status nk_batch_wait(nk_batch* B, nk_solve_stats* stats) {
    if (!B) return NK_BAD_ARGUMENT;
    return guarded(B->ctx, [&] {
        if (!B->pending) bad("no batched solve pending");
        NK_CUDA(cudaStreamSynchronize(B->stream));
        if (!batch_finish(B, stats)) throw Failure{NK_NONFINITE, "non-finite velocity change in a batch slot"};
    });
}

}  // extern "C"

// =================================================================================================================
// Serving: a request loop over resident problems, one stream per in-flight request.
// =================================================================================================================
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace {

// First-fit sub-allocator over one reserved range, with coalescing of freed blocks (256-byte granules).
struct SubAllocator {
    size_t cap = 0;
    std::map<size_t, size_t> free_blocks;   // offset -> size
    void init(size_t bytes) {
        cap = bytes;
        free_blocks.clear();
        free_blocks[0] = bytes;
    }
    static size_t round(size_t b) { return (b + 255) & ~size_t(255); }
    bool alloc(size_t bytes, size_t& off) {
        bytes = round(bytes);
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            size_t rest = it->second - bytes;
            free_blocks.erase(it);
            if (rest) free_blocks[off + bytes] = rest;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = round(bytes);
        auto it = free_blocks.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_blocks.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_blocks.erase(next);
        }
        if (it != free_blocks.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_blocks.erase(it);
            }
        }
    }
};

struct ServerRequest {
    int64_t ticket = 0;
    nk_grid_desc grid{};
    nk_physics_desc physics{};
    nk_solver_desc solver{};
    std::vector<double> xf, yf, sf, H, bed, C, A, u0, v0;
    double* u_out = nullptr;
    double* v_out = nullptr;
    std::string key;
    double t_submit = 0, t_admit = 0, t_done = 0;
    nk_solve_stats stats{};
    int state = 0;   // 0 queued, 1 on the device, 2 finished
    nk_status status = NK_OK;
};

struct Resident {
    nk_problem* P = nullptr;
    nk_batch* B = nullptr;            // a batch resident (nk_server_desc.batch_slots > 1): P is its slot 0
    std::vector<int64_t> tickets;     // batch resident: the request in each slot (0: none)
    std::string key;
    bool busy = false;
    int64_t ticket = 0;
    size_t bytes = 0;                // device bytes sub-allocated at dev_off
    size_t dev_off = 0, pin_off = 0, pin_bytes = 0;
    double last_used = 0;
    double* pin = nullptr;          // pinned staging: H, bed, C, A, u0, v0 in; u, v out (one block per slot)
    size_t pin_count = 0;
    size_t pin_slot = 0;            // doubles between two slots' staging blocks
    SolverScalars* sc_out = nullptr; // pinned copy of the solver scalars at completion
    cudaEvent_t done = nullptr;
};

void append_bytes(std::string& k, const void* p, size_t n) { k.append(reinterpret_cast<const char*>(p), n); }

// Identity of a problem shape: grid (with face vectors), physics and solver, without pointers.
std::string request_key(const ServerRequest& R) {
    std::string k;
    nk_grid_desc g = R.grid;
    g.x_faces = g.y_faces = g.sigma_faces = nullptr;
    append_bytes(k, &g, sizeof(g));
    append_bytes(k, &R.physics, sizeof(R.physics));
    append_bytes(k, &R.solver, sizeof(R.solver));
    for (const auto* v : {&R.xf, &R.yf, &R.sf}) {
        size_t n = v->size();
        append_bytes(k, &n, sizeof(n));
        if (n) append_bytes(k, v->data(), n * sizeof(double));
    }
    return k;
}

nk_grid_desc grid_with_vectors(ServerRequest& R) {
    nk_grid_desc g = R.grid;
    g.x_faces = R.xf.empty() ? nullptr : R.xf.data();
    g.y_faces = R.yf.empty() ? nullptr : R.yf.data();
    g.sigma_faces = R.sf.empty() ? nullptr : R.sf.data();
    return g;
}

}  // namespace

struct nk_server {
    nk_context* ctx = nullptr;
    nk_server_desc desc{};
    // host seconds spent creating problems, starting and finishing requests (NK_SERVER_TRACE=1 prints them)
    double t_create = 0, t_start = 0, t_finish = 0, t_graph = 0;
    int created = 0;
    std::chrono::steady_clock::time_point t0;
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, std::unique_ptr<ServerRequest>> requests;
    std::vector<std::unique_ptr<Resident>> residents;
    int64_t next_ticket = 1;
    int64_t device_bytes = 0;
    int in_flight = 0, peak = 0;
    // the HBM budget and a pinned staging pool, reserved once when the server is created, so that no
    // allocation call (which can wait on running work) happens while requests are on the device
    char* dev_base = nullptr;
    char* pin_base = nullptr;
    SubAllocator dev, pin;
    // NK_SERVER_ADMISSION_THREAD: the loop runs on `worker`; every API call holds `mu`
    bool threaded = false, stop = false;
    std::thread worker;
    mutable std::mutex mu;
    std::condition_variable work_cv, done_cv;
    nk_status worker_status = NK_OK;
    std::string worker_error;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    // the lock of an API call: held in threaded mode, a no-op otherwise
    std::unique_lock<std::mutex> lock() const {
        return threaded ? std::unique_lock<std::mutex>(mu) : std::unique_lock<std::mutex>();
    }
};

namespace nk {

static int batch_slots_of(const nk_server* S) { return std::max(1, (int)S->desc.batch_slots); }

static size_t problem_bytes(ServerRequest& R) {
    nk_problem probe;
    probe.gd = grid_with_vectors(R);
    probe.pd = R.physics;
    probe.sd = R.solver;
    build(&probe, true);
    return probe.arena.size;
}

static void destroy_resident(nk_server* S, size_t idx) {
    Resident* r = S->residents[idx].get();
    S->device_bytes -= (int64_t)r->bytes;
    if (r->done) cudaEventDestroy(r->done);
    if (r->B) batch_free(r->B);
    else nk_problem_destroy(r->P);
    S->dev.release(r->dev_off, r->bytes);
    S->pin.release(r->pin_off, r->pin_bytes);
    S->residents.erase(S->residents.begin() + idx);
}

static size_t staging_doubles(const ServerRequest& R) {
    size_t cells = (size_t)R.grid.Nx * R.grid.Ny, faces = (size_t)(R.grid.Nx + 1) * (R.grid.Ny + 1);
    return 4 * cells + 4 * faces;
}
static size_t pinned_bytes(const ServerRequest& R) {
    return staging_doubles(R) * sizeof(double) + 2 * 256 + 2 * sizeof(SolverScalars);
}
// A batch resident's pinned block: the batch's own records, then one 256-byte-aligned staging block per slot.
static size_t batch_slot_doubles(const ServerRequest& R) { return (staging_doubles(R) * sizeof(double) + 255) / 256 * 256 / sizeof(double); }
static size_t batch_resident_pinned(const ServerRequest& R, int slots) {
    return (batch_pinned_bytes(slots) + 255) / 256 * 256 + (size_t)slots * batch_slot_doubles(R) * sizeof(double);
}

// A resident problem for R: an idle one of the same shape, else a new one carved out of the server's
// reserved HBM and pinned pool (evicting idle problems of other shapes, least recently used first).
// nullptr: wait until running requests release memory.
static Resident* acquire(nk_server* S, ServerRequest& R) {
    for (auto& r : S->residents)
        if (!r->busy && r->key == R.key) return r.get();
    int slots = batch_slots_of(S);
    size_t stride = 0;
    if (slots > 1) {
        nk_grid_desc g = grid_with_vectors(R);
        stride = batch_stride(&g, &R.physics, &R.solver);
    }
    size_t need = slots > 1 ? batch_device_bytes(stride, slots) : problem_bytes(R);
    size_t pneed = slots > 1 ? batch_resident_pinned(R, slots) : pinned_bytes(R);
    size_t off = 0, poff = 0;
    auto fits = [&] {
        if (!S->dev.alloc(need, off)) return false;
        if (!S->pin.alloc(pneed, poff)) {
            S->dev.release(off, need);
            return false;
        }
        return true;
    };
    while (!fits()) {
        int victim = -1;
        for (size_t i = 0; i < S->residents.size(); ++i)
            if (!S->residents[i]->busy && (victim < 0 || S->residents[i]->last_used < S->residents[victim]->last_used)) victim = (int)i;
        if (victim < 0) {
            if (S->in_flight > 0) return nullptr;
            throw Failure{NK_OOM, "a request needs more device or pinned memory than the server reserved"};
        }
        destroy_resident(S, victim);
    }
    double tc0 = S->now();
    auto r = std::make_unique<Resident>();
    r->dev_off = off;
    r->bytes = need;
    r->pin_off = poff;
    r->pin_bytes = pneed;
    char* pin = S->pin_base + poff;
    if (slots > 1) {
        nk_grid_desc g = grid_with_vectors(R);
        nk_status st = batch_create(S->ctx, &g, &R.physics, &R.solver, slots, S->dev_base + off, pin, &r->B);
        if (st != NK_OK) {
            S->dev.release(off, need);
            S->pin.release(poff, pneed);
            throw Failure{st, S->ctx->error};
        }
        r->P = r->B->P[0];
        r->key = R.key;
        r->tickets.assign(slots, 0);
        r->pin_slot = batch_slot_doubles(R);
        r->pin = reinterpret_cast<double*>(pin + (batch_pinned_bytes(slots) + 255) / 256 * 256);
        r->pin_count = staging_doubles(R);
        NK_CUDA(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming));
        S->device_bytes += (int64_t)r->bytes;
        S->residents.push_back(std::move(r));
        S->created += 1;
        S->t_create += S->now() - tc0;
        return S->residents.back().get();
    }
    r->sc_out = reinterpret_cast<SolverScalars*>(pin);
    SolverScalars* sc_host = reinterpret_cast<SolverScalars*>(pin + 256);
    r->pin = reinterpret_cast<double*>(pin + 512);
    nk_grid_desc g = grid_with_vectors(R);
    nk_status st = problem_create(S->ctx, &g, &R.physics, &R.solver, &r->P, S->dev_base + off, sc_host);
    if (st != NK_OK) {
        S->dev.release(off, need);
        S->pin.release(poff, pneed);
        throw Failure{st, S->ctx->error};
    }
    r->key = R.key;
    nk_problem* P = r->P;
    size_t cells = (size_t)P->Nx * P->Ny, faces = (size_t)(P->Nx + 1) * (P->Ny + 1);
    r->pin_count = 4 * cells + 4 * faces;
    NK_CUDA(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming));
    double tg0 = S->now();
    if (use_graphs(P)) build_picard_graph(P);
    S->t_graph += S->now() - tg0;
    if (const char* e = std::getenv("NK_SERVER_TRACE"))
        if (e[0] == '1')
            std::fprintf(stderr, "nk_server: problem %d: setup %.1f ms, graph %.1f ms (instantiate %.1f ms), %d in flight\n", S->created + 1,
                         1e3 * (tg0 - tc0), 1e3 * (S->now() - tg0), 1e3 * P->instantiate_s, S->in_flight);
    S->device_bytes += (int64_t)r->bytes;
    S->residents.push_back(std::move(r));
    S->created += 1;
    S->t_create += S->now() - tc0;
    return S->residents.back().get();
}

// Enqueue on P's stream: the request's inputs from the pinned block `pin` into P, the warm start, the geometry.
static void stage_request(const ServerRequest& R, nk_problem* P, double* pin) {
    cudaStream_t s = P->stream;
    size_t cells = (size_t)P->Nx * P->Ny;
    FieldLoc fu = field_loc(P, NK_FIELD_U);
    size_t nu = (size_t)fu.nx * fu.ny;
    auto stage = [&](int id, const std::vector<double>& src, double* at) {
        FieldLoc f = field_loc(P, id);
        std::memcpy(at, src.data(), src.size() * sizeof(double));
        size_t n = (size_t)f.nx * f.ny * f.planes;
        NK_CUDA(cudaMemcpyAsync(P->staging, at, n * sizeof(double), cudaMemcpyHostToDevice, s));
        launch_pack(f.base, P->pitch, (int)P->plane, f.stride, f.offset, P->staging, f.nx, f.ny, f.planes, s);
    };
    stage(NK_FIELD_H, R.H, pin);
    stage(NK_FIELD_BED, R.bed, pin + cells);
    if (!R.C.empty()) stage(NK_FIELD_FRICTION_COEFFICIENT, R.C, pin + 2 * cells);
    stage(NK_FIELD_RATE_FACTOR, R.A, pin + 3 * cells);
    double* uin = pin + 4 * cells;
    NK_CUDA(cudaMemsetAsync(P->x, 0, P->plane * sizeof(double2), s));
    if (!R.u0.empty()) stage(NK_FIELD_U, R.u0, uin);
    if (!R.v0.empty()) stage(NK_FIELD_V, R.v0, uin + nu);
    GeometryView gv;
    gv.g = P->fine.g;
    gv.H = P->H; gv.bed = P->bed; gv.s = P->s; gv.N = P->N; gv.mu = P->mu; gv.phi = P->phi; gv.phi_uv = P->phi_uv; gv.tau = P->tau;
    gv.rho_i = P->pd.ice_density; gv.rho_w = P->pd.ocean_density; gv.gacc = P->pd.gravitational_acceleration;
    gv.grounding = P->pd.grounding; gv.gl_stress = P->pd.grounding_line_driving_stress; gv.use_mask = P->pd.use_ice_mask;
    gv.mask_min = P->pd.mask_minimum_thickness; gv.mask_trans = P->pd.mask_transition_thickness;
    gv.ud = P->ud;
    launch_geometry(gv, s);
}

// Enqueue on P's stream: u and v of P's solution into the output part of the pinned block `pin`.
static void read_back(nk_problem* P, double* pin) {
    cudaStream_t s = P->stream;
    size_t cells = (size_t)P->Nx * P->Ny;
    FieldLoc fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
    size_t nu = (size_t)fu.nx * fu.ny, nv = (size_t)fv.nx * fv.ny;
    double* uout = pin + 4 * cells + nu + nv;
    launch_unpack(P->staging, (const double*)P->x, P->pitch, (int)P->plane, 2, 0, fu.nx, fu.ny, 1, s);
    NK_CUDA(cudaMemcpyAsync(uout, P->staging, nu * sizeof(double), cudaMemcpyDeviceToHost, s));
    launch_unpack(P->staging, (const double*)P->x, P->pitch, (int)P->plane, 2, 1, fv.nx, fv.ny, 1, s);
    NK_CUDA(cudaMemcpyAsync(uout + nu, P->staging, nv * sizeof(double), cudaMemcpyDeviceToHost, s));
}

static void admitted(nk_server* S, ServerRequest& R) {
    R.state = 1;
    R.t_admit = S->now();
    S->in_flight += 1;
    S->peak = std::max(S->peak, S->in_flight);
}

// Stage the request's inputs and enqueue its whole solve on the resident problem's stream.
static void start(nk_server* S, ServerRequest& R, Resident& r) {
    nk_problem* P = r.P;
    cudaStream_t s = P->stream;
    stage_request(R, P, r.pin);
    set_control(P);
    if (use_graphs(P)) {
        NK_CUDA(cudaGraphLaunch(P->picard_exec, s));
    } else {
        host_picard(P);
    }
    read_back(P, r.pin);
    NK_CUDA(cudaMemcpyAsync(r.sc_out, P->sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s));
    NK_CUDA(cudaEventRecord(r.done, s));
    NK_CHECK_LAUNCH();
    r.busy = true;
    r.ticket = R.ticket;
    admitted(S, R);
}

// The requests `reqs` (of one shape, at most the batch's slots) into slots 0, 1, ... of a batch resident and one
// batched solve of those slots.
static void start_batch(nk_server* S, const std::vector<ServerRequest*>& reqs, Resident& r) {
    nk_batch* B = r.B;
    std::vector<uint8_t> active(B->slots, 0);
    for (size_t k = 0; k < reqs.size(); ++k) {
        stage_request(*reqs[k], B->P[k], r.pin + k * r.pin_slot);
        active[k] = 1;
    }
    batch_solve_async(B, active.data());
    for (size_t k = 0; k < reqs.size(); ++k) read_back(B->P[k], r.pin + k * r.pin_slot);
    NK_CUDA(cudaEventRecord(r.done, B->stream));
    NK_CHECK_LAUNCH();
    r.busy = true;
    std::fill(r.tickets.begin(), r.tickets.end(), 0);
    for (size_t k = 0; k < reqs.size(); ++k) {
        r.tickets[k] = reqs[k]->ticket;
        admitted(S, *reqs[k]);
    }
}

// A batch resident's requests after its solve: each slot's results and statistics.
static void finish_batch(nk_server* S, Resident& r) {
    nk_batch* B = r.B;
    std::vector<nk_solve_stats> stats(B->slots);
    batch_finish(B, stats.data());
    double t = S->now();
    for (int k = 0; k < B->slots; ++k) {
        if (!r.tickets[k]) continue;
        ServerRequest& R = *S->requests.at(r.tickets[k]);
        nk_problem* P = B->P[k];
        FieldLoc fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
        size_t nu = (size_t)fu.nx * fu.ny, nv = (size_t)fv.nx * fv.ny;
        size_t cells = (size_t)P->Nx * P->Ny;
        const double* uout = r.pin + k * r.pin_slot + 4 * cells + nu + nv;
        if (R.u_out) std::memcpy(R.u_out, uout, nu * sizeof(double));
        if (R.v_out) std::memcpy(R.v_out, uout + nu, nv * sizeof(double));
        R.stats = stats[k];
        R.status = R.stats.status == NK_NONFINITE ? NK_NONFINITE : NK_OK;
        R.state = 2;
        R.t_done = t;
        S->in_flight -= 1;
        r.tickets[k] = 0;
    }
    r.busy = false;
    r.last_used = t;
}

static void finish(nk_server* S, Resident& r) {
    if (r.B) {
        finish_batch(S, r);
        return;
    }
    ServerRequest& R = *S->requests.at(r.ticket);
    nk_problem* P = r.P;
    FieldLoc fu = field_loc(P, NK_FIELD_U), fv = field_loc(P, NK_FIELD_V);
    size_t nu = (size_t)fu.nx * fu.ny, nv = (size_t)fv.nx * fv.ny;
    size_t cells = (size_t)P->Nx * P->Ny;
    const double* uout = r.pin + 4 * cells + nu + nv;
    if (R.u_out) std::memcpy(R.u_out, uout, nu * sizeof(double));
    if (R.v_out) std::memcpy(R.v_out, uout + nu, nv * sizeof(double));
    fill_stats_from(*r.sc_out, &R.stats, true);
    const SolverScalars& h = *r.sc_out;
    if (use_graphs(P))
        count_launches(P->picard_kernels[0] + (long long)h.p_it * P->picard_kernels[1] + (long long)h.it_total * P->picard_kernels[2]);
    R.status = R.stats.status == NK_NONFINITE ? NK_NONFINITE : NK_OK;
    R.state = 2;
    R.t_done = S->now();
    r.busy = false;
    r.last_used = R.t_done;
    S->in_flight -= 1;
}

static void progress(nk_server* S) {
    for (auto& r : S->residents) {
        if (!r->busy) continue;
        cudaError_t e = cudaEventQuery(r->done);
        if (e == cudaSuccess) {
            double tf0 = S->now();
            finish(S, *r);
            S->t_finish += S->now() - tf0;
        }
        else if (e != cudaErrorNotReady) NK_CUDA(e);
    }
    while (!S->queue.empty() && S->in_flight < S->desc.max_in_flight) {
        ServerRequest& R = *S->requests.at(S->queue.front());
        Resident* r = nullptr;
        try {
            r = acquire(S, R);
        } catch (const Failure& f) {
            R.status = f.status;
            R.state = 2;
            R.t_done = S->now();
            S->queue.pop_front();
            continue;
        }
        if (!r) break;   // wait for memory
        double ts0 = S->now();
        if (r->B) {
            // this request and the next queued ones of its shape, up to the slots and the requests allowed in flight
            size_t room = (size_t)std::min(r->B->slots, S->desc.max_in_flight - S->in_flight);
            std::vector<ServerRequest*> batch;
            for (auto it = S->queue.begin(); it != S->queue.end() && batch.size() < room;) {
                ServerRequest& Q = *S->requests.at(*it);
                if (Q.key == R.key) {
                    batch.push_back(&Q);
                    it = S->queue.erase(it);
                } else {
                    ++it;
                }
            }
            start_batch(S, batch, *r);
        } else {
            S->queue.pop_front();
            start(S, R, *r);
        }
        S->t_start += S->now() - ts0;
    }
}

// The admission thread: retire and admit while requests are queued or on the device (polling their events every
// 20 us, with the lock released), sleep on work_cv otherwise.  A CUDA failure is kept for the waiting calls and ends the loop.
static void admission_loop(nk_server* S) {
    cudaSetDevice(S->ctx->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (!S->stop) {
        try {
            progress(S);
        } catch (const Failure& f) {
            S->worker_status = f.status;
            S->worker_error = f.message;
            S->done_cv.notify_all();
            break;
        }
        S->done_cv.notify_all();
        if (S->in_flight > 0 || !S->queue.empty()) {   // requests to retire, or queued ones waiting for a slot
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        } else {
            S->work_cv.wait(lk, [&] { return S->stop || !S->queue.empty(); });
        }
    }
}

}  // namespace nk

extern "C" {

nk_status nk_server_create(nk_context* ctx, const nk_server_desc* desc, nk_server** out) {
    if (!ctx || !desc || !out || desc->max_in_flight < 1 || desc->memory_cap_bytes <= 0) return NK_BAD_ARGUMENT;
    if (desc->batch_slots < 0 || desc->batch_slots > NK_MAX_BATCH_SLOTS) return NK_BAD_ARGUMENT;
    auto* S = new nk_server();
    S->ctx = ctx;
    S->desc = *desc;
    S->t0 = std::chrono::steady_clock::now();
    // pinned staging: inputs and outputs of the requests in flight (a thirty-second of the device budget, >= 64 MiB)
    size_t pin_cap = std::max<size_t>(64ull << 20, (size_t)desc->memory_cap_bytes / 32);
    nk_status st = guarded(ctx, [&] {
        NK_CUDA(cudaMalloc((void**)&S->dev_base, (size_t)desc->memory_cap_bytes));
        NK_CUDA(cudaHostAlloc((void**)&S->pin_base, pin_cap, cudaHostAllocDefault));
    });
    if (st != NK_OK) {
        if (S->dev_base) cudaFree(S->dev_base);
        delete S;
        return st;
    }
    S->dev.init((size_t)desc->memory_cap_bytes);
    S->pin.init(pin_cap);
    if (desc->flags & NK_SERVER_ADMISSION_THREAD) {
        S->threaded = true;
        S->worker = std::thread(admission_loop, S);
    }
    *out = S;
    return NK_OK;
}

nk_status nk_server_destroy(nk_server* S) {
    if (!S) return NK_OK;
    if (S->threaded) {
        {
            std::lock_guard<std::mutex> g(S->mu);
            S->stop = true;
        }
        S->work_cv.notify_all();
        S->worker.join();
        S->threaded = false;
    }
    if (const char* e = std::getenv("NK_SERVER_TRACE"))
        if (e[0] == '1')
            std::fprintf(stderr, "nk_server: %d problems created in %.3f s (graph capture %.3f s); host time starting requests %.3f s, "
                                 "finishing %.3f s; peak in flight %d\n", S->created, S->t_create, S->t_graph, S->t_start, S->t_finish, S->peak);
    guarded(S->ctx, [&] {
        for (auto& r : S->residents)
            if (r->busy) cudaEventSynchronize(r->done);
        while (!S->residents.empty()) destroy_resident(S, S->residents.size() - 1);
        if (S->dev_base) cudaFree(S->dev_base);
        if (S->pin_base) cudaFreeHost(S->pin_base);
    });
    delete S;
    return NK_OK;
}

double nk_server_clock(const nk_server* S) { return S ? S->now() : 0.0; }

nk_status nk_server_submit(nk_server* S, const nk_request* q, int64_t* ticket) {
    if (!S || !q || !ticket || !q->H || !q->bed || !q->rate_factor) return NK_BAD_ARGUMENT;
    return guarded(S->ctx, [&] {
        if (q->physics.rate_factor_layout != NK_RATE_FACTOR_2D) bad("served requests take a 2-D rate factor");
        if (q->grid.Nx < 1 || q->grid.Ny < 1) bad("empty grid");
        auto R = std::make_unique<ServerRequest>();
        R->grid = q->grid;
        R->physics = q->physics;
        R->solver = q->solver;
        int Nx = q->grid.Nx, Ny = q->grid.Ny;
        if (q->grid.x_faces) R->xf.assign(q->grid.x_faces, q->grid.x_faces + Nx + 1);
        if (q->grid.y_faces) R->yf.assign(q->grid.y_faces, q->grid.y_faces + Ny + 1);
        if (q->grid.sigma_faces) R->sf.assign(q->grid.sigma_faces, q->grid.sigma_faces + q->grid.Nsigma + 1);
        size_t cells = (size_t)Nx * Ny;
        int nfx = q->grid.topology_x == NK_PERIODIC ? Nx : Nx + 1, nfy = q->grid.topology_y == NK_PERIODIC ? Ny : Ny + 1;
        R->H.assign(q->H, q->H + cells);
        R->bed.assign(q->bed, q->bed + cells);
        if (q->friction_coefficient) R->C.assign(q->friction_coefficient, q->friction_coefficient + cells);
        R->A.assign(q->rate_factor, q->rate_factor + cells);
        if (q->u_init) R->u0.assign(q->u_init, q->u_init + (size_t)nfx * Ny);
        if (q->v_init) R->v0.assign(q->v_init, q->v_init + (size_t)Nx * nfy);
        R->u_out = q->u_out;
        R->v_out = q->v_out;
        R->key = request_key(*R);
        R->t_submit = S->now();
        auto lk = S->lock();
        R->ticket = S->next_ticket++;
        *ticket = R->ticket;
        S->queue.push_back(R->ticket);
        S->requests[R->ticket] = std::move(R);
        if (S->threaded) {
            lk.unlock();
            S->work_cv.notify_one();
        } else {
            progress(S);
        }
    });
}

nk_status nk_server_progress(nk_server* S, int32_t* pending) {
    if (!S) return NK_BAD_ARGUMENT;
    return guarded(S->ctx, [&] {
        auto lk = S->lock();
        if (S->threaded) {
            if (S->worker_status != NK_OK) throw Failure{S->worker_status, S->worker_error};
        } else {
            progress(S);
        }
        if (pending) {
            int32_t n = 0;
            for (auto& kv : S->requests) n += kv.second->state != 2;
            *pending = n;
        }
    });
}

nk_status nk_server_wait(nk_server* S, int64_t ticket, nk_solve_stats* stats, double* t_submit, double* t_admit, double* t_done) {
    if (!S) return NK_BAD_ARGUMENT;
    auto lk = S->lock();
    auto it = S->requests.find(ticket);
    if (it == S->requests.end()) return NK_BAD_ARGUMENT;
    nk_status st = guarded(S->ctx, [&] {
        if (S->threaded) {
            S->done_cv.wait(lk, [&] { return it->second->state == 2 || S->worker_status != NK_OK; });
            if (it->second->state != 2) throw Failure{S->worker_status, S->worker_error};
            return;
        }
        while (it->second->state != 2) {
            progress(S);
            if (it->second->state != 2) std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    });
    if (st != NK_OK) return st;
    ServerRequest& R = *it->second;
    if (stats) *stats = R.stats;
    if (t_submit) *t_submit = R.t_submit;
    if (t_admit) *t_admit = R.t_admit;
    if (t_done) *t_done = R.t_done;
    return R.status;
}

nk_status nk_server_wait_all(nk_server* S) {
    if (!S) return NK_BAD_ARGUMENT;
    return guarded(S->ctx, [&] {
        auto lk = S->lock();
        auto all_done = [&] {
            for (auto& kv : S->requests)
                if (kv.second->state != 2) return false;
            return true;
        };
        if (S->threaded) {
            S->done_cv.wait(lk, [&] { return all_done() || S->worker_status != NK_OK; });
            if (!all_done()) throw Failure{S->worker_status, S->worker_error};
            return;
        }
        while (true) {
            progress(S);
            if (all_done()) break;
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    });
}

nk_status nk_server_info(const nk_server* S, int32_t* resident, int64_t* device_bytes, int32_t* peak_in_flight) {
    if (!S) return NK_BAD_ARGUMENT;
    auto lk = S->lock();
    if (resident) *resident = (int32_t)S->residents.size();
    if (device_bytes) *device_bytes = S->device_bytes;
    if (peak_in_flight) *peak_in_flight = S->peak;
    return NK_OK;
}

}  // extern "C"
