"""The seeded workloads of the golden solve fixtures (tests/golden/oracle_solves.npz), shared by the script that
writes them and by the test that checks both backends against them.  Every case runs Picard and CG with fixed
iteration counts, so two implementations differ only by rounding."""
from nunatak_gb300 import model as M
from nunatak_gb300 import workloads


def _fixed(picard, cg, preconditioner):
    return M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(cg), picard_iteration_control=M.FixedIterations(picard),
                                 preconditioner=preconditioner)


def channel_shelf():
    """84 x 40 floating channel shelf, no-slip walls, calving front at 80 km: Picard(3) x Jacobi-PCG(40)."""
    return workloads.channel_shelf(velocity_solver=_fixed(3, 40, M.StressBalanceDiagonalPreconditioner()))


def channel_shelf_inflow():
    """The channel shelf with 100 m/yr prescribed on the west faces: Picard(3) x Jacobi-PCG(40)."""
    return workloads.channel_shelf(inflow=100.0, velocity_solver=_fixed(3, 40, M.StressBalanceDiagonalPreconditioner()))


def marine_sheet():
    """40 x 20 marine sheet (seed 2), Weertman drag, free-slip walls: Picard(3) x multigrid-PCG(25)."""
    return workloads.marine_sheet(40, 20, seed=2, velocity_solver=_fixed(3, 25, M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4)))


def marine_sheet_line_jacobi():
    """The 40 x 20 marine sheet with the y-line smoother: Picard(3) x multigrid-PCG(25)."""
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4, smoother=M.LineJacobi())
    return workloads.marine_sheet(40, 20, seed=2, velocity_solver=_fixed(3, 25, mg))


def diva_sheet():
    """24 x 12 DIVA sheet (32 km cells, Nσ = 4, Arrhenius rate factor, regularised Coulomb drag):
    Picard(3) x multigrid-PCG(30), then the velocity profile."""
    return workloads.diva_sheet(24, 12, dx=32e3, Nsigma=4,
                                velocity_solver=_fixed(3, 30, M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4)))


CASES = {
    "channel_shelf": (channel_shelf, ("u", "v")),
    "channel_shelf_inflow": (channel_shelf_inflow, ("u", "v")),
    "marine_sheet": (marine_sheet, ("u", "v", "eta_H", "beta_u")),
    "marine_sheet_line_jacobi": (marine_sheet_line_jacobi, ("u", "v")),
    "diva_sheet": (diva_sheet, ("u", "v", "u_sigma", "v_sigma", "u_b", "eta_sigma")),
}


def solve(name, cls):
    """Run case `name` on backend `cls`; the fields it records, by name."""
    make, fields = CASES[name]
    P = make().problem(cls)
    P.picard_solve()
    P.velocity_profile()
    out = {k: P.get(k) for k in fields}
    P.close()
    return out
