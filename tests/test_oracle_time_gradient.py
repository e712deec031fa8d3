"""The oracle's restatement of the gradient through time steps (nko_checkpointed_gradient) against centred differences
of its own forward steps, on the CPU.  With the velocities held: the transport case of test/test_enzyme.jl:447-488
(16 x 4, sources a and m, eight steps; the default bounded WENO-5 and first-order upwinding) at the reference's cells
to 1e-6, the floating melt across a grounding line (the centre grounded fraction) at the partially grounded cells
to 1e-5, and a partial-cell front (its advance reversed through a numerical Jacobian) with and without overflow passes
and under eigencalving and von Mises calving, at the reference's cells (test/test_enzyme.jl:490-536) to 1e-5.  With a
Picard solve after every stage: the reference's ridge (:421-445) and von Mises calving on a confined shelf to 1e-5,
the DIVA ridge to 1e-4 (the DIVA with von Mises calving is refused).  The
library's gradient is held to this one over the whole field in test_gpu_time_gradient."""
import numpy as np
import pytest

from nunatak_gb300 import model as M
from test_gpu_time_gradient import (_close, calving_case, channel_front_case, fd_extrapolated, fd_final_thickness, gradient,
                                    grounding_line_case, ridge_case, shelf_case, transport_case)


@pytest.mark.parametrize("advection", [None, M.UpwindBiased(order=1)], ids=["bounded_weno5", "upwind1"])
def test_oracle_transport_gradient_matches_differences(oracle_cls, advection):
    case = transport_case(advection)
    _, g = gradient(case, oracle_cls)
    for field, key, idx, val in (("surface_mass_balance", "smb", (1, 4), 1e-8), ("basal_melt_rate", "melt", (2, 8), 1e-9 * 8.5 / 16)):
        _close(g[key][idx], fd_final_thickness(case, oracle_cls, field, idx, 1e-6 * val), 1e-6)
    P = case.build(oracle_cls)
    u0, H0 = P.get("u"), P.get("H")
    for idx in ((0, 5), (3, 10)):
        _close(g["u"][idx], fd_final_thickness(case, oracle_cls, "u", idx, 1e-6 * abs(u0[idx])), 1e-6)
    for idx in ((1, 3), (2, 8)):
        _close(g["H"][idx], fd_final_thickness(case, oracle_cls, "H", idx, 1e-6 * H0[idx]), 1e-6)


def test_oracle_floating_melt_gradient(oracle_cls):
    case = grounding_line_case(None)
    P0 = case.build(oracle_cls)
    phi, H0 = P0.get("phi"), P0.get("H")
    _, g = gradient(case, oracle_cls)
    partial = [tuple(ix) for ix in np.argwhere((phi > 0.05) & (phi < 0.95))]
    assert len(partial) >= 3
    for idx in partial[:3]:
        _close(g["H"][idx], fd_final_thickness(case, oracle_cls, "H", idx, 1e-6 * H0[idx]), 1e-5)


@pytest.mark.parametrize("passes", [4, 0])
def test_oracle_front_gradient(oracle_cls, passes):
    case = channel_front_case(passes)
    _, g = gradient(case, oracle_cls)
    for idx in ((1, 2), (2, 4)):
        _close(g["smb"][idx], fd_final_thickness(case, oracle_cls, "surface_mass_balance", idx, 1e-9), 1e-5)
    H0 = case.build(oracle_cls).get("H")
    _close(g["H"][2, 3], fd_final_thickness(case, oracle_cls, "H", (2, 3), 1e-6 * H0[2, 3]), 1e-5)


def test_oracle_eigencalving_gradient(oracle_cls):
    case = calving_case(M.EigenCalving(coefficient=1e13))
    _, g = gradient(case, oracle_cls)
    for idx in ((1, 3), (2, 3)):
        _close(g["u"][idx], fd_final_thickness(case, oracle_cls, "u", idx, 1e-12), 1e-5)


def test_oracle_von_mises_gradient(oracle_cls):
    """Von Mises calving with the velocities and the viscosity η̄H held: ∂J/∂u through the strain rates and the front
    speed, ∂J/∂H₀ through η = η̄H / H as well."""
    case = calving_case(M.VonMisesCalving(stress_threshold=1e6, floating_stress_threshold=2e5), grounding=M.SubgridGroundedFraction())
    _, g = gradient(case, oracle_cls)
    for idx in ((1, 3), (2, 3)):
        _close(g["u"][idx], fd_final_thickness(case, oracle_cls, "u", idx, 1e-12), 1e-5)
    H0 = case.build(oracle_cls).get("H")
    _close(g["H"][2, 3], fd_final_thickness(case, oracle_cls, "H", (2, 3), 1e-6 * H0[2, 3]), 1e-5)
    assert np.sum(case.forward(oracle_cls).get("calved_thickness")) > 0


def test_oracle_picard_time_steps_gradient(oracle_cls):
    """The reference's ridge (SSA, Weertman) with a Picard solve after every stage, two steps: the oracle's gradient
    (its Picard adjoint of every solve, the thickness part by differences of the residual τ − A(c(x*, H)) x*) against
    Richardson-extrapolated differences of its own forward steps, ∂J/∂H₀ at two cells, ∂J/∂log C and ∂J/∂a at one,
    to 1e-5 (test/test_enzyme.jl:421-445)."""
    case = ridge_case(oracle_cls, steps=2)
    _, g = gradient(case, oracle_cls)
    assert g["stats"]["picard_adjoints"] == 3 * case.steps and g["stats"]["worst_solve_status"] == 0
    H0 = case.build(oracle_cls).get("H")
    for idx in ((1, 5), (2, 9)):
        _close(g["H"][idx], fd_extrapolated(case, oracle_cls, "H", idx, 1e-3 * H0[idx]), 1e-5)
    C = case.build(oracle_cls).get("C")
    _close(g["log_C"][1, 6] / C[1, 6], fd_extrapolated(case, oracle_cls, "C", (1, 6), 1e-3 * C[1, 6]), 1e-5)
    _close(g["smb"][2, 8], fd_extrapolated(case, oracle_cls, "surface_mass_balance", (2, 8), 1e-2 * 1e-8), 1e-5)


def test_oracle_von_mises_gradient_with_solves(oracle_cls):
    """Von Mises calving on the confined shelf with a Picard solve after every stage: the front's η̄H column of the
    numerical Jacobian enters the oracle's Picard adjoint of the solve before the front as the coefficient's shadow;
    ∂J/∂H₀ at a shelf cell and at the front column and ∂J/∂log A near the front against Richardson differences, 1e-5."""
    case = shelf_case(False)
    P0 = case.build(oracle_cls)
    H0, A0 = P0.get("H"), P0.get("A")
    _, g = gradient(case, oracle_cls)
    assert g["stats"]["worst_solve_status"] == 0
    for idx in ((1, 4), (2, 9)):
        _close(g["H"][idx], fd_extrapolated(case, oracle_cls, "H", idx, 1e-5 * H0[idx]), 1e-5)
    idx = (1, 8)
    _close(g["log_A"][idx], A0[idx] * fd_extrapolated(case, oracle_cls, "A", idx, 1e-4 * A0[idx]), 1e-5)


def test_oracle_diva_picard_time_steps_gradient(oracle_cls):
    """The ridge under the DIVA (Nσ = 6) with a Picard solve after every stage, two steps: the thickness part of each
    solve's adjoint adds the lagged state's σᵀ ∂S/∂H (βᵇ, F₂, ησ of the state update at the fixed point) to λᵀ ∂r/∂H.
    The lagged state's adjoint settles more slowly than λ, whose change stops a Convergence control, so 3000 fixed
    adjoint iterations: ∂J/∂H₀ at two cells then meets Richardson differences to 1e-6 (the state's term is 3e-5 to 4e-5
    of it there), ∂J/∂log C at one to 1e-5."""
    case = ridge_case(oracle_cls, diva=True, steps=2)
    _, g = gradient(case, oracle_cls, adjoint_control=M.FixedIterations(3000))
    assert g["stats"]["picard_adjoints"] == 3 * case.steps
    H0 = case.build(oracle_cls).get("H")
    for idx in ((1, 5), (2, 9)):
        _close(g["H"][idx], fd_extrapolated(case, oracle_cls, "H", idx, 1e-3 * H0[idx]), 1e-6)
    C = case.build(oracle_cls).get("C")
    _close(g["log_C"][1, 6] / C[1, 6], fd_extrapolated(case, oracle_cls, "C", (1, 6), 1e-3 * C[1, 6]), 1e-5)


def test_oracle_refuses_solves_it_does_not_restate(oracle_cls):
    case = shelf_case(True)   # the DIVA under von Mises calving: its sweep takes no viscosity shadow
    P = case.build(oracle_cls)
    with pytest.raises(Exception):
        P.checkpointed_gradient(lambda *a: None, case.dt, 1, velocity_solves=True)
