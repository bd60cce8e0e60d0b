"""Known answer held by the reference: the thick-walled Mooney-Rivlin cylinder
under inflation and extension (FiniteElasticity_CylinderAnalyticCalculate,
finite_elasticity_routines.f90:491-602, with the boundary conditions of
FiniteElasticity_BoundaryConditionsAnalyticCalculate, :132-484).

The tube (inner radius 0.5, outer 1, height 1; c1 = 2, c2 = 6) is stretched
to lambda = 1.1 and loaded by an inner pressure of 1 over 4 load increments
(the reference's incremented pressure rule).  The finite-element solution
(triquadratic displacement / trilinear pressure, nodes on exact circles)
must converge to the analytic deformed coordinates and pressure as the mesh
is refined: this pins the oracle's restatement of the element residual,
Jacobian and surface-pressure load, and the CUDA path through it, to an
answer the reference itself states.

Measured on the oracle: nodal position errors 2.6e-5 (2 x 8 x 1 elements,
radial x circumferential x axial) and 1.8e-6 (4 x 16 x 1); pressure errors
(largest at the loaded inner surface) 6.6e-3 and 2.6e-3, against p ~ 1.87.
"""
import warnings

import numpy as np
import pytest
import torch

from cm_gb300 import mesh as M
from cm_gb300 import newton as N

warnings.filterwarnings("ignore", message="Sparse")

LAM, PIN, POUT, C1, C2, A_IN, A_OUT, H = 1.1, 1.0, 0.0, 2.0, 6.0, 0.5, 1.0, 1.0
INCREMENTS = 4


@pytest.fixture(scope="module")
def analytic():
    import cylinder_analytic as CA  # oracle/cylinder_analytic.py
    sol = CA.CylinderSolution(PIN, POUT, LAM, A_OUT, A_IN, C1, C2)
    assert abs(CA.residual_function(sol.mu1, PIN, POUT, LAM, 0.0, A_OUT, A_IN, C1, C2)) < 1e-12
    return sol


def tube(nr, nt, nz=1):
    return M.thick_cylinder(nr, nt, nz, A_IN, A_OUT, H, materials=(C1, C2))


def errors(m, x, sol):
    z = x[:3 * m.nu].reshape(3, m.nu)
    pn = m.pressure_node_u()
    R = np.hypot(m.X[0, pn], m.X[1, pn])
    p = x[3 * m.nu:]
    return float(np.abs(z - sol.deformed(m.X)).max()), float(np.abs(p - sol.library_pressure(R)).max())


def solve(es, m, device, **opt):
    s = N.LoadStepSolver(es, N.cylinder_conditions(m, LAM), N.NewtonOptions(**opt), device=device)
    x0 = torch.from_numpy(N.initial_state(m)).to(device)
    x, reps = s.solve(x0, INCREMENTS, pressure=N.PressureIncrements(N.cylinder_pressure(m, PIN, POUT)))
    assert all(r.converged for r in reps) and len(reps) == INCREMENTS
    return x.cpu().numpy(), reps


def test_analytic_restatement_is_consistent(analytic):
    """Incompressibility of the analytic map (det F = 1 through r dr/dR =
    R / lambda), the axial stretch, and the inflation direction."""
    R = np.linspace(A_IN, A_OUT, 7)
    r = analytic.mu(R) * R
    assert np.allclose(r ** 2 - r[0] ** 2, (R ** 2 - R[0] ** 2) / LAM, rtol=0, atol=1e-14)
    assert r[0] > A_IN / np.sqrt(LAM)  # the inner pressure opens the tube beyond the pure-stretch radius
    X = np.array([[0.7], [0.0], [0.4]])
    assert abs(analytic.deformed(X)[2, 0] - LAM * 0.4) < 1e-15


def test_oracle_converges_to_the_cylinder_solution(oracle, analytic):
    errs = []
    for nr, nt in ((2, 8), (4, 16)):
        m = tube(nr, nt)
        x, _ = solve(oracle.EquationsSet(m), m, "cpu", linear="dense")
        errs.append(errors(m, x, analytic))
    (dz0, dp0), (dz1, dp1) = errs
    assert dz0 < 4e-5 and dz1 < 3e-6 and dz1 < dz0 / 8
    assert dp0 < 1e-2 and dp1 < 4e-3 and dp1 < dp0 / 2


@pytest.mark.gpu
def test_gpu_newton_converges_to_the_cylinder_solution(oracle, analytic):
    """The CUDA path (FP64 Jacobian and residual, the Newton driver on the
    device) solves the tube to the oracle's solution (1e-9) and to the
    analytic one at the finer refinement, and the native C-ABI load step
    reaches the same state."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cm_gb300 import FiniteElasticityEquationsSet
    m = tube(4, 16)
    xo, ro = solve(oracle.EquationsSet(m), m, "cpu", linear="dense")
    es = FiniteElasticityEquationsSet(m)
    xg, rg = solve(es, m, "cuda", linear="dense")
    assert float(np.abs(xg - xo).max()) < 1e-9
    assert [r.iterations for r in rg] == [r.iterations for r in ro]
    dz, dp = errors(m, xg, analytic)
    assert dz < 3e-6 and dp < 4e-3
    # the native load step, the caller applying the increment rules
    bc = N.cylinder_conditions(m, LAM)
    pinc = N.PressureIncrements(N.cylinder_pressure(m, PIN, POUT))
    x = torch.from_numpy(N.initial_state(m)).cuda()
    for i in range(1, INCREMENTS + 1):
        cur = x[bc.dofs].cpu().numpy()
        new = bc.full.copy() if i == INCREMENTS else \
            np.where(bc.incremented, cur + (bc.full - cur) / (INCREMENTS - i + 1), bc.full)
        es.set_surface_pressure(pinc.step(i, INCREMENTS))
        rep = es.newton_load_step(x, bc.dofs, new, ksp_rtol=1e-10, ksp_max_iterations=4000)
        assert rep["converged"] == 1 and rep["residual_norm"] <= 1e-10
    assert float(np.abs(x.cpu().numpy() - xo).max()) < 1e-8


@pytest.mark.gpu
def test_gpu_refined_cylinder(analytic):
    """A finer tube (8 x 32 x 1 elements, 10k dofs) on the device only: the
    position error keeps falling with the mesh (1.5e-7 and a pressure error
    of 8.0e-4 measured on the oracle)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cm_gb300 import FiniteElasticityEquationsSet
    m = tube(8, 32)
    x, _ = solve(FiniteElasticityEquationsSet(m), m, "cuda", linear="dense")
    dz, dp = errors(m, x, analytic)
    assert dz < 3e-7 and dp < 1.2e-3
