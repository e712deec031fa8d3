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
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "nk_kernels.cuh"

struct nk_context {
    int device = 0;
    std::string error;
};

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
    double* sig_tables = nullptr;              // dz, w2, zc (Ns each) + w1 (Ns * Ns)
    double* rate_params = nullptr;             // 9
    std::vector<double> sig_dz, sig_w2, sig_zc, sig_w1;

    // coarse levels
    std::vector<Level<double>> lv64;           // FP64 hierarchy: [0] is the fine grid view
    std::vector<Level<float>> lv32;            // FP32 hierarchy (mixed): [0] is a float copy of the fine grid
    int nlevels = 0;                           // coarse levels below the fine grid

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
        v.zold = mixed && precond == NK_PRECONDITIONER_MULTIGRID ? zold : nullptr;
        v.invd = invd;
        v.precond = precond;
        v.sc = sc;
        v.partials = partials;
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

// Exact integral of (1 - ζ)^p, column_integrals.jl:31
static double ipow(double x, int n) { double r = x; for (int m = 1; m < n; ++m) r *= x; return r; }
static double power_integral(double zm, double zp, int p) { return (ipow(1 - zm, p + 1) - ipow(1 - zp, p + 1)) / (p + 1); }

static void build(nk_problem* P) {
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
    LaunchDims big = dims2d(P->Nx + 1, P->Ny + 1);
    size_t nblocks = (size_t)big.grid.x * big.grid.y;
    slots.push_back({(void**)&P->partials, A.reserve(nblocks * sizeof(double2))});
    slots.push_back({(void**)&P->sc, A.reserve(sizeof(SolverScalars))});
    slots.push_back({(void**)&P->sig_tables, A.reserve((3 * P->Ns + (size_t)P->Ns * P->Ns) * sizeof(double))});
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
    NK_CUDA(cudaMalloc((void**)&A.base, A.size));
    NK_CUDA(cudaMemsetAsync(A.base, 0, A.size, P->stream));
    for (auto& sl : slots) *sl.first = A.base + sl.second;

    upload_metrics(F, P->stream);
    std::vector<double> tables;
    tables.insert(tables.end(), P->sig_dz.begin(), P->sig_dz.end());
    tables.insert(tables.end(), P->sig_w2.begin(), P->sig_w2.end());
    tables.insert(tables.end(), P->sig_zc.begin(), P->sig_zc.end());
    tables.insert(tables.end(), P->sig_w1.begin(), P->sig_w1.end());
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
    NK_CUDA(cudaHostAlloc((void**)&P->sc_host, sizeof(SolverScalars), cudaHostAllocDefault));
    std::memset(P->sc_host, 0, sizeof(SolverScalars));
}

// ---- coefficient preparation ----------------------------------------------------------------------------------
// Mask (and the Jacobi inverse diagonal) after η̄H, η̄Hᶠᶠ or β changed.
static void prepare_operator(nk_problem* P) {
    OpView<double> o = P->fine_op();
    launch_mask<double>(o, P->fine.mask, P->stream);
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

// smooth!, multigrid_preconditioner.jl:165-174, leaving the result in L.x
template <typename T>
static void smooth(nk_problem* P, Level<T>& L, int sweeps, bool first, const int* done) {
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
    if (!first && sweeps % 2 == 1) {   // an odd number of ping-pong sweeps starting from L.x would write L.x in place
        cudaMemcpyAsync(L.x2, L.x, L.plane() * sizeof(V2), cudaMemcpyDeviceToDevice, s);
        in = L.x2;
    }
    for (int k = 0; k < sweeps; ++k) {
        V2* out = ((sweeps - 1 - k) % 2 == 0) ? L.x : L.x2;
        launch_smooth_point<T>(v, in, out, (first && k == 0) ? 1 : 0, done, s);
        in = out;
    }
}

// v_cycle!, multigrid_preconditioner.jl:144-163 (x ≈ A⁻¹ b from a zero guess on level l)
template <typename T>
static void v_cycle(nk_problem* P, std::vector<Level<T>>& lv, int l, const int* done) {
    cudaStream_t s = P->stream;
    Level<T>& L = lv[l];
    if (l == P->nlevels) {
        smooth(P, L, P->sd.coarsest_sweeps, true, done);
        return;
    }
    smooth(P, L, P->sd.smoothing_sweeps, true, done);
    LevelView<T> v = P->level_view(L);
    launch_level_apply<T>(v, L.x, L.q, 1, done, s);
    LevelView<T> c = P->level_view(lv[l + 1]);
    // the restriction reads the residual in L.q through the fine mask
    launch_restrict<T>(c, v, L.q, lv[l + 1].b, done, s);
    v_cycle(P, lv, l + 1, done);
    launch_prolongate<T>(v, c, L.x, lv[l + 1].x, done, s);
    smooth(P, L, P->sd.smoothing_sweeps, false, done);
}

// z = M r with the configured preconditioner (inside conjugate gradients, predicated on `done`)
static void precondition_mg(nk_problem* P, const int* done) {
    cudaStream_t s = P->stream;
    if (!P->mixed) {
        v_cycle<double>(P, P->lv64, 0, done);
    } else {
        launch_to_float(P->fine.g, P->r, P->lv32[0].b, done, s);
        v_cycle<float>(P, P->lv32, 0, done);
        launch_to_double(P->fine.g, P->lv32[0].x, P->z, done, s);
    }
    NK_CHECK_LAUNCH();
}

// ---- conjugate gradients ----------------------------------------------------------------------------------------
static void set_control(nk_problem* P, const nk_iteration_control& c) {
    SolverScalars h{};
    h.reltol = c.reltol;
    h.abstol = c.abstol;
    h.fixed = c.kind == NK_FIXED_ITERATIONS;
    h.iterations = c.iterations;
    h.maxiter = c.maxiter;
    h.flexible = (P->mixed && P->precond == NK_PRECONDITIONER_MULTIGRID) ? 1 : 0;
    *P->sc_host = h;
    NK_CUDA(cudaMemcpyAsync(P->sc, P->sc_host, sizeof(SolverScalars), cudaMemcpyHostToDevice, P->stream));
}

static void cg_step(nk_problem* P, const CGView& v) {
    cudaStream_t s = P->stream;
    launch_cg_apply(v, s);
    launch_cg_update(v, s);
    if (P->precond == NK_PRECONDITIONER_MULTIGRID) {
        precondition_mg(P, &P->sc->done);
        launch_cg_dots_after_precondition(v, s);
    }
    launch_cg_xpby(v, s);
}

static void read_scalars(nk_problem* P) {
    NK_CUDA(cudaMemcpyAsync(P->sc_host, P->sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, P->stream));
    NK_CUDA(cudaStreamSynchronize(P->stream));
}

// conjugate_gradient!, conjugate_gradient.jl:299-341, on x (warm start) with right-hand side b
static void cg_solve(nk_problem* P, const double2* b, nk_solve_stats* st) {
    const nk_iteration_control& ctl = P->sd.linear;
    set_control(P, ctl);
    update_preconditioner(P);
    CGView v = P->cg_view(b);
    launch_cg_init(v, P->stream);
    if (P->precond == NK_PRECONDITIONER_MULTIGRID) {
        precondition_mg(P, nullptr);
        launch_cg_init_finish(v, P->stream);
    }
    NK_CHECK_LAUNCH();
    int limit = ctl.kind == NK_FIXED_ITERATIONS ? ctl.iterations : ctl.maxiter;
    int issued = 0;
    int batch = 4;
    while (issued < limit) {
        int n = std::min(batch, limit - issued);
        for (int k = 0; k < n; ++k) cg_step(P, v);
        NK_CHECK_LAUNCH();
        issued += n;
        if (ctl.kind == NK_FIXED_ITERATIONS) continue;
        read_scalars(P);
        if (P->sc_host->done) break;
        batch = std::min(batch * 2, 64);
    }
    read_scalars(P);
    const SolverScalars& h = *P->sc_host;
    if (st) {
        st->linear_iterations_last = h.it;
        st->linear_iterations_total += h.it;
        st->residual_norm = h.rnorm;
        st->initial_residual_norm = h.r0;
        if (h.status == NK_NONFINITE) st->status = NK_NONFINITE;
        else if (ctl.kind == NK_CONVERGENCE && h.rnorm > h.tol && st->status == NK_OK) st->status = NK_NOT_CONVERGED;
    }
}

// update_stress_balance_coefficients! / update_diva_coefficients!
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

// picard_solve!, picard.jl:63-90
static void picard_solve(nk_problem* P, nk_solve_stats* st) {
    const nk_iteration_control& ctl = P->sd.picard;
    std::memset(st, 0, sizeof(*st));
    int it = 0;
    if (ctl.kind == NK_FIXED_ITERATIONS) {
        for (int k = 0; k < ctl.iterations; ++k) {
            update_coefficients(P);
            cg_solve(P, P->tau, st);
        }
        it = ctl.iterations;
    } else {
        double D = INFINITY, X = 0.0;
        while (D > std::max(ctl.reltol * X, ctl.abstol) && it < ctl.maxiter) {
            launch_copy_range(P->fine.g, P->xprev, P->x, P->stream);
            update_coefficients(P);
            cg_solve(P, P->tau, st);
            launch_picard_delta(P->fine.g, P->xprev, P->x, P->sc, P->partials, P->stream);
            NK_CHECK_LAUNCH();
            read_scalars(P);
            D = std::sqrt(P->sc_host->picard_dd);
            X = std::sqrt(P->sc_host->picard_xx);
            ++it;
            if (!std::isfinite(D)) { st->status = NK_NONFINITE; break; }
        }
        st->picard_change = D;
        st->picard_norm = X;
        if (st->status == NK_OK && D > std::max(ctl.reltol * X, ctl.abstol)) st->status = NK_NOT_CONVERGED;
    }
    st->picard_iterations = it;
}

// ---- fields in interior layout -----------------------------------------------------------------------------------
struct FieldLoc {
    double* base = nullptr;   // pitched device array (first plane)
    int stride = 1, offset = 0, nx = 0, ny = 0, planes = 1;
    bool coef = false;        // a coefficient: the operator mask and diagonal follow it
};

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
        default: break;
    }
    return f;
}

static void copy_in(nk_problem* P, const FieldLoc& f, const double* host) {
    size_t n = (size_t)f.nx * f.ny * f.planes;
    NK_CUDA(cudaMemcpyAsync(P->staging, host, n * sizeof(double), cudaMemcpyHostToDevice, P->stream));
    launch_pack(f.base, P->pitch, (int)P->plane, f.stride, f.offset, P->staging, f.nx, f.ny, f.planes, P->stream);
    NK_CHECK_LAUNCH();
}
static void copy_out(nk_problem* P, const FieldLoc& f, double* host) {
    size_t n = (size_t)f.nx * f.ny * f.planes;
    launch_unpack(P->staging, f.base, P->pitch, (int)P->plane, f.stride, f.offset, f.nx, f.ny, f.planes, P->stream);
    NK_CHECK_LAUNCH();
    NK_CUDA(cudaMemcpyAsync(host, P->staging, n * sizeof(double), cudaMemcpyDeviceToHost, P->stream));
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

nk_status nk_context_create(int32_t device, nk_context** out) {
    if (!out) return NK_BAD_ARGUMENT;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return NK_CUDA_ERROR;
    auto* c = new nk_context();
    c->device = device;
    *out = c;
    return NK_OK;
}

nk_status nk_context_destroy(nk_context* ctx) {
    delete ctx;
    return NK_OK;
}

const char* nk_last_error(const nk_context* ctx) { return ctx ? ctx->error.c_str() : "no context"; }

nk_status nk_problem_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics, const nk_solver_desc* solver,
                            nk_problem** out) {
    if (!ctx || !grid || !physics || !solver || !out) return NK_BAD_ARGUMENT;
    auto* P = new nk_problem();
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
        if (solver->precision == NK_PRECISION_MIXED && solver->preconditioner != NK_PRECONDITIONER_MULTIGRID)
            bad("mixed precision needs the multigrid preconditioner");
        P->ctx = ctx;
        P->gd = *grid;             // build() reads the caller's face vectors during this call only
        P->pd = *physics;
        P->sd = *solver;
        NK_CUDA(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
        NK_CUDA(cudaEventCreate(&P->ev0));
        NK_CUDA(cudaEventCreate(&P->ev1));
        build(P);
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
    if (P->arena.base) cudaFree(P->arena.base);
    if (P->sc_host) cudaFreeHost(P->sc_host);
    if (P->ev0) cudaEventDestroy(P->ev0);
    if (P->ev1) cudaEventDestroy(P->ev1);
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
    return NK_OK;
}

int64_t nk_problem_field_size(const nk_problem* P, int32_t id) {
    if (!P) return 0;
    FieldLoc f = field_loc(const_cast<nk_problem*>(P), id);
    return f.base ? (int64_t)f.nx * f.ny * f.planes : 0;
}

nk_status nk_problem_set_field(nk_problem* P, int32_t id, const double* host, int64_t count) {
    if (!P || !host) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        FieldLoc f = field_loc(P, id);
        if (!f.base) bad("unknown field id or field not held by this problem");
        if (count != (int64_t)f.nx * f.ny * f.planes) bad("field size mismatch");
        copy_in(P, f, host);
        if (f.coef) prepare_operator(P);
        NK_CUDA(cudaStreamSynchronize(P->stream));
    });
}

nk_status nk_problem_get_field(const nk_problem* Pc, int32_t id, double* host, int64_t count) {
    nk_problem* P = const_cast<nk_problem*>(Pc);
    if (!P || !host) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        FieldLoc f = field_loc(P, id);
        if (!f.base) bad("unknown field id or field not held by this problem");
        if (count != (int64_t)f.nx * f.ny * f.planes) bad("field size mismatch");
        copy_out(P, f, host);
    });
}

nk_status nk_compute_geometry(nk_problem* P) {
    if (!P) return NK_BAD_ARGUMENT;
    return guarded(P->ctx, [&] {
        GeometryView v;
        v.g = P->fine.g;
        v.H = P->H; v.bed = P->bed; v.s = P->s; v.N = P->N; v.mu = P->mu; v.phi = P->phi; v.phi_uv = P->phi_uv; v.tau = P->tau;
        v.rho_i = P->pd.ice_density; v.rho_w = P->pd.ocean_density; v.gacc = P->pd.gravitational_acceleration;
        v.grounding = P->pd.grounding; v.gl_stress = P->pd.grounding_line_driving_stress; v.use_mask = P->pd.use_ice_mask;
        v.mask_min = P->pd.mask_minimum_thickness; v.mask_trans = P->pd.mask_transition_thickness;
        launch_geometry(v, P->stream);
        NK_CHECK_LAUNCH();
        NK_CUDA(cudaStreamSynchronize(P->stream));
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
            // z = r / diag over size(z); the wall faces are unit rows (diagonal_preconditioner.jl:132-139)
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

static nk_status linear_solve_impl(nk_problem* P, const double* bu, const double* bv, nk_solve_stats* stats) {
    return guarded(P->ctx, [&] {
        nk_solve_stats local{};
        nk_solve_stats* st = stats ? stats : &local;
        std::memset(st, 0, sizeof(*st));
        vector_in(P, P->tmp_b, bu, bv);
        NK_CUDA(cudaEventRecord(P->ev0, P->stream));
        cg_solve(P, P->tmp_b, st);
        NK_CUDA(cudaEventRecord(P->ev1, P->stream));
        NK_CUDA(cudaEventSynchronize(P->ev1));
        float ms = 0;
        cudaEventElapsedTime(&ms, P->ev0, P->ev1);
        st->device_ms = ms;
        if (st->status == NK_NONFINITE) throw Failure{NK_NONFINITE, "non-finite residual"};
    });
}

nk_status nk_linear_solve(nk_problem* P, const double* bu, const double* bv, nk_solve_stats* stats) {
    if (!P || !bu || !bv) return NK_BAD_ARGUMENT;
    return linear_solve_impl(P, bu, bv, stats);
}

nk_status nk_adjoint_solve(nk_problem* P, const double* bu, const double* bv, nk_solve_stats* stats) {
    if (!P || !bu || !bv) return NK_BAD_ARGUMENT;
    return linear_solve_impl(P, bu, bv, stats);   // the operator is self-adjoint (conjugate_gradient.jl:186-189)
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
        float ms = 0;
        cudaEventElapsedTime(&ms, P->ev0, P->ev1);
        st->device_ms = ms;
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
            launch_restrict<double>(vc, vf, fbuf, cbuf, nullptr, P->stream);
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

}  // extern "C"
