"""Load-stepped Newton (the caller of the assembly path).

CPU tests run the driver on the oracle's equations set: the load-increment
rule of EQUATIONS_SET_BOUNDARY_CONDITIONS_INCREMENT
(equations_set_routines.f90:6560-6595), Newton's quadratic convergence to
||r_free||_2 <= 1e-10, the exact discrete solution of homogeneous uniaxial
stretch on the 4x4x4 trilinear cube, and GMRES against the dense solve.
GPU tests run the same driver on the CUDA path (FP64 and mixed Jacobian)
and compare every increment with the oracle run.
"""
import warnings

import numpy as np
import pytest
import torch

from cm_gb300 import mesh as M
from cm_gb300 import newton as N

warnings.filterwarnings("ignore", message="Sparse")


def cube_cfg1():
    return M.regular_box(4, 4, 4, nxi_u=2, pressure="element", law=M.MR, materials=(2.0, 6.0))


def quad_small():
    return M.regular_box(3, 2, 2, lengths=(1.5, 1.0, 1.0), nxi_u=3, pressure="node", law=M.MR,
                         materials=(2.0, 6.0), perturb=0.1, seed=11)


def oracle_solve(oracle, m, bc, increments, **opt):
    es = oracle.EquationsSet(m)
    s = N.LoadStepSolver(es, bc, N.NewtonOptions(**opt), device="cpu")
    return s.solve(torch.from_numpy(N.initial_state(m)), increments)


def test_increment_rule_reference_formula():
    # NEW = CUR + (FULL - CUR)/(N - i + 1), FULL on the last increment
    m = cube_cfg1()
    bc = N.DirichletConditions(m.ndofs).fix([3, 7], [2.0, -1.0], incremented=True).fix([11], 0.5)

    class _ES:
        mesh, ndofs, nnz = m, m.ndofs, m.ndofs

        def csr_pattern(self, base=0):
            return np.arange(m.ndofs + 1, dtype=np.int32), np.arange(m.ndofs, dtype=np.int32)

    s = N.LoadStepSolver(_ES(), bc, device="cpu")
    x = torch.zeros(m.ndofs, dtype=torch.float64)
    x[3] = 0.4  # not on the equal-step path: the rule still closes the gap in equal parts
    seen = []
    for i in range(1, 5):
        x = s.apply_increment(x, i, 4)
        seen.append((float(x[3]), float(x[7]), float(x[11])))
    cur3 = [0.4]
    for i in range(1, 5):
        cur3.append(cur3[-1] + (2.0 - cur3[-1]) / (4 - i + 1))
    assert np.allclose([v[0] for v in seen], cur3[1:], rtol=0, atol=1e-15)
    assert np.allclose([v[1] for v in seen], [-0.25, -0.5, -0.75, -1.0], rtol=0, atol=1e-15)
    assert all(v[2] == 0.5 for v in seen)   # fixed (not incremented) values hold from the start
    assert seen[-1][0] == 2.0


def test_config1_uniaxial_exact_solution(oracle):
    """4x4x4 trilinear cube, Mooney-Rivlin (2, 6), stretch 1.1 in 5 increments:
    Newton reaches ||r|| <= 1e-10 quadratically at every increment and the
    converged field is the homogeneous incompressible stretch, with the
    pressure that makes the lateral faces traction-free."""
    m = cube_cfg1()
    lam = 1.1
    es = oracle.EquationsSet(m)
    s = N.LoadStepSolver(es, N.uniaxial_symmetry_conditions(m, lam), N.NewtonOptions(linear="dense"), device="cpu")
    seen = []
    x, reps = s.solve(torch.from_numpy(N.initial_state(m)), 5, progress=lambda i, r: seen.append((i, r)))
    assert len(reps) == 5 and all(r.converged for r in reps)
    assert [i for i, _ in seen] == [1, 2, 3, 4, 5] and [r for _, r in seen] == reps
    for r in reps:
        assert r.iterations <= 5
        rn = r.residual_norms
        assert rn[-1] <= 1e-10
        assert rn[-2] <= 1e-3 * rn[-3] or rn[-2] <= 1e-6   # superlinear tail
    z = x[:3 * m.nu].numpy().reshape(3, -1)
    assert np.abs(z[0] - lam * m.X[0]).max() < 1e-11
    assert np.abs(z[1] - m.X[1] / np.sqrt(lam)).max() < 1e-11
    assert np.abs(z[2] - m.X[2] / np.sqrt(lam)).max() < 1e-11
    # sigma = dev(2 c1 B - 2 c2 B^-1) + p I with sigma_yy = 0
    B = np.array([lam ** 2, 1 / lam, 1 / lam])
    sb = 2 * 2.0 * B - 2 * 6.0 / B
    p_exact = -(sb[1] - sb.mean())
    p = x[3 * m.nu:].numpy()
    assert np.abs(p - p_exact).max() < 1e-10


def test_gmres_matches_dense(oracle):
    m = quad_small()
    bc = N.clamped_stretch_shear_conditions(m, 1.15, 0.05)
    xd, rd = oracle_solve(oracle, m, bc, 2, linear="dense")
    xg, rg = oracle_solve(oracle, m, bc, 2, linear="gmres", gmres_rtol=1e-8)
    assert all(r.converged for r in rd + rg)
    assert [r.iterations for r in rd] == [r.iterations for r in rg]
    assert float((xd - xg).abs().max()) < 1e-9
    assert all(max(r.linear_iterations) > 1 for r in rg)


def _cpu_sparse_products():
    """Whether this PyTorch build multiplies sparse CSR matrices on the CPU
    (builds without MKL do not; the multigrid set-up needs it on the CPU)."""
    a = torch.eye(2, dtype=torch.float64).to_sparse_csr()
    try:
        torch.sparse.mm(a, a)
        return True
    except RuntimeError:
        return False


def test_multigrid_preconditioned_gmres(oracle):
    """Block-triangular preconditioner (multigrid V-cycle on the displacement
    block, scaled pressure mass matrix on the Schur complement): same Newton
    iterates as the dense solve, and far fewer Krylov iterations than the
    block-Jacobi preconditioner."""
    if not _cpu_sparse_products():
        pytest.skip("this PyTorch build has no CPU sparse CSR products")
    m = M.regular_box(4, 4, 4, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=1)
    bc = N.clamped_stretch_shear_conditions(m, 1.05, 0.02)
    xd, rd = oracle_solve(oracle, m, bc, 1, linear="dense")
    xm, rm = oracle_solve(oracle, m, bc, 1, linear="mg", gmres_rtol=1e-8)
    assert rm[0].converged and rm[0].iterations == rd[0].iterations
    assert float((xd - xm).abs().max()) < 1e-9
    es = oracle.EquationsSet(m)
    sj = N.LoadStepSolver(es, bc, N.NewtonOptions(linear="gmres", max_iterations=1), device="cpu")
    _, rj = sj.solve(torch.from_numpy(N.initial_state(m)), 1)
    assert max(rm[0].linear_iterations) * 3 < rj[0].linear_iterations[0]


def test_multigrid_vertex_coarse_operator(oracle):
    """The first coarse operator by rediscretisation on the vertex mesh: the
    vertex mesh carries the fine vertices' coordinates and the injected state
    (nodal pressure included), and multigrid-preconditioned GMRES reaches the
    same Newton iterates as with the Galerkin coarse operator, in a similar
    number of Krylov iterations."""
    if not _cpu_sparse_products():
        pytest.skip("this PyTorch build has no CPU sparse CSR products")
    from cm_gb300 import multigrid as MG
    m = M.regular_box(4, 3, 2, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=5)
    cm, inj = MG.vertex_mesh(m)
    assert cm.nxi_u == 2 and cm.ne == m.ne and cm.grid_u == (5, 4, 3)
    i, j, k = m.node_ijk()
    vert = (i % 2 == 0) & (j % 2 == 0) & (k % 2 == 0)
    assert np.array_equal(np.sort(inj[:cm.nu]), np.nonzero(vert)[0])
    assert np.array_equal(cm.X, m.X[:, inj[:cm.nu]])
    assert np.array_equal(inj[3 * cm.nu:], 3 * m.nu + np.arange(cm.n_pressure))
    assert np.array_equal(m.pressure_node_u(), inj[:cm.nu])  # pressure nodes are the vertices, numbered alike
    bc = N.clamped_stretch_shear_conditions(m, 1.05, 0.02)
    xv, rv = oracle_solve(oracle, m, bc, 1, linear="mg", gmres_rtol=1e-8, mg_coarse="vertex")
    xg, rg = oracle_solve(oracle, m, bc, 1, linear="mg", gmres_rtol=1e-8, mg_coarse="galerkin")
    assert rv[0].converged and rg[0].converged and rv[0].iterations == rg[0].iterations
    assert float((xv - xg).abs().max()) < 1e-9
    assert max(rv[0].linear_iterations) <= 2 * max(rg[0].linear_iterations)


@pytest.mark.parametrize("kind", ["element_pressure", "guccione_fibres"])
def test_vertex_mesh_carries_the_fine_data(kind):
    """vertex_mesh for element-based pressure (one pressure dof per element,
    injected element by element) and for a Guccione slab (fibre angles and
    per-law materials taken at the vertices)."""
    from cm_gb300 import multigrid as MG
    if kind == "element_pressure":
        m = M.regular_box(3, 2, 2, nxi_u=3, pressure="element", law=M.MR, materials=(1.0, 4.0), perturb=0.1, seed=2)
    else:
        m = M.guccione_slab(4, 3, 2, seed=1)
    cm, inj = MG.vertex_mesh(m)
    assert cm.p_mode == m.p_mode and cm.law == m.law and np.array_equal(cm.materials, m.materials)
    assert cm.ne == m.ne and cm.ndofs == len(inj)
    vid = inj[:cm.nu]
    assert np.array_equal(cm.X, m.X[:, vid])
    if m.fibre is not None:
        assert np.array_equal(cm.fibre, m.fibre[:, vid])
    # the corner nodes of every fine element are the coarse element's nodes, in the same order
    corners = [a * 2 + b * 2 * 3 + c * 2 * 9 for c in (0, 1) for b in (0, 1) for a in (0, 1)]
    assert np.array_equal(vid[cm.elem_u], m.elem_u[:, corners])
    x = M.deformed_state(m, stretch=1.05, shear=0.02, noise=0.01, pressure=-0.5, seed=3)
    xc = x[inj]
    assert np.array_equal(xc[3 * cm.nu:], x[3 * m.nu:3 * m.nu + cm.n_pressure])


def test_multigrid_prolongation_is_exact_for_linear_fields():
    """The tensor-product prolongations reproduce linear fields on every level
    (Q1 functions are in the Q2 space, and coarse Q1 in fine Q1)."""
    from cm_gb300 import multigrid as MG
    m = M.regular_box(4, 2, 6, nxi_u=3, pressure="node")
    free = np.ones(3 * m.nu, dtype=bool)
    mg = MG.BoxMultigrid(m.grid_u, m.nxi_u, free, "cpu", torch.float64, min_dofs=10)
    levels = mg.levels
    assert levels[0] == (9, 5, 13) and levels[1] == (5, 3, 7)
    for lvl, (lf, lc) in enumerate(zip(levels[:-1], levels[1:])):
        def lin(shape):
            idx = np.arange(int(np.prod(shape)))
            i, j, k = idx % shape[0], (idx // shape[0]) % shape[1], idx // (shape[0] * shape[1])
            x, y, z = i / (shape[0] - 1), j / (shape[1] - 1), k / (shape[2] - 1)
            return np.concatenate([1 + 2 * x - y, 3 * z + 0.5 * x, x + y + z])
        fine = mg.P[lvl] @ torch.from_numpy(lin(lc))
        assert np.abs(fine.numpy() - lin(lf)).max() < 1e-12


def test_line_search_backtracks_on_a_large_step(oracle):
    """One increment straight to stretch 1.3 / shear 0.1 on the triquadratic
    mesh: the full Newton step fails the sufficient-decrease test at least
    once, the cubic backtracking shortens it, and Newton still ends at
    ||r|| <= 1e-10 with full steps in its quadratic tail."""
    m = quad_small()
    x, reps = oracle_solve(oracle, m, N.clamped_stretch_shear_conditions(m, 1.3, 0.1), 1, linear="dense")
    r = reps[0]
    assert r.converged
    assert min(r.line_search_lambdas) < 1.0
    for f0, f1 in zip(r.residual_norms[:-1], r.residual_norms[1:]):
        assert f1 < f0   # every accepted step decreases ||r||
    assert r.line_search_lambdas[-1] == 1.0


def test_failed_line_search_keeps_the_previous_state(oracle):
    """A line search that finds no step with sufficient decrease rejects the
    step.  The step is capped at max_step = 1e-9, so along it f = 1/2 ||r||^2
    changes by lam * slope to first order (slope = r . (J d), the directional
    derivative, whatever the accuracy of the linear solve), and with
    alpha = 1.5 the sufficient-decrease bound f0 + 1.5 lam slope lies below
    that for every descent direction: no trial passes, and min_lambda = 0.6
    stops the backtracking after its second trial.  The state must be the
    one before the step and the report must say so (PETSc's bt line search
    leaves X unchanged on a failed reduction)."""
    m = quad_small()
    bc = N.clamped_stretch_shear_conditions(m, 1.3, 0.1)
    es = oracle.EquationsSet(m)
    s = N.LoadStepSolver(es, bc, N.NewtonOptions(linear="dense", alpha=1.5, min_lambda=0.6, max_step=1e-9), device="cpu")
    x0 = s.apply_increment(torch.from_numpy(N.initial_state(m)), 1, 1)
    x, rep = s.newton(x0.clone())
    assert rep.line_search_failed and not rep.converged
    assert rep.iterations == 1 and len(rep.residual_norms) == 1
    assert torch.equal(x, x0)


def test_mixed_split_positions_cover_the_pattern():
    """Host logic of the mixed path: the uu and coupling positions partition
    the full pattern (checked on the layout arithmetic alone)."""
    class FakeSet:  # 3 u rows (nu = 1) + 1 p row, the layout fe_mixed_layout reports
        ndofs = 4

        class mesh:
            nu = 1

        @staticmethod
        def csr_pattern():
            return np.array([0, 5, 9, 13, 15]), None

        @staticmethod
        def mixed_layout():
            return np.array([0, 4, 7, 10]), np.array([0, 1, 2, 3, 5])

    uu_pos, cp_pos = N.mixed_positions(FakeSet())
    assert sorted(np.concatenate([uu_pos, cp_pos]).tolist()) == list(range(15))
    # each displacement row: its uu entries first, then its coupling entries
    assert uu_pos.tolist() == [0, 1, 2, 3, 5, 6, 7, 9, 10, 11]
    assert cp_pos.tolist() == [4, 8, 12, 13, 14]


# ------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cm_gb300 import _lib
    _lib.load()
    return torch.device("cuda")


def gpu_solve(m, bc, increments, **opt):
    from cm_gb300 import FiniteElasticityEquationsSet
    es = FiniteElasticityEquationsSet(m)
    s = N.LoadStepSolver(es, bc, N.NewtonOptions(**opt), device="cuda")
    x, reps = s.solve(torch.from_numpy(N.initial_state(m)).cuda(), increments)
    return x.cpu(), reps, es


@pytest.mark.gpu
def test_gpu_config1_matches_oracle_newton(cuda, oracle):
    m = cube_cfg1()
    bc = N.uniaxial_symmetry_conditions(m, 1.1)
    xo, ro = oracle_solve(oracle, m, bc, 5, linear="dense")
    xg, rg, es = gpu_solve(m, bc, 5, linear="dense")
    assert [r.iterations for r in rg] == [r.iterations for r in ro]
    for a, b in zip(rg, ro):
        assert a.converged
        assert np.allclose(a.residual_norms[:-1], b.residual_norms[:-1], rtol=1e-8)
    assert float((xg - xo).abs().max()) < 1e-11
    assert es.launch_count() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("hp", ["fp64", "double_float"])
def test_gpu_mixed_jacobian_converges_to_fp64_solution(cuda, oracle, hp):
    """FP32 Jacobian (BF16x3 tensor cores on the displacement blocks), FP64 or
    double-float residual: the converged solution meets the same
    ||r||_2 <= 1e-10 and agrees with the FP64 oracle run."""
    m = quad_small()
    bc = N.clamped_stretch_shear_conditions(m, 1.2, 0.1)
    xo, ro = oracle_solve(oracle, m, bc, 3, linear="dense")
    xm, rm, _ = gpu_solve(m, bc, 3, linear="dense", precision="mixed", high_precision=hp)
    assert all(r.converged for r in rm)
    assert all(r.residual_norms[-1] <= 1e-10 for r in rm)
    for a, b in zip(rm, ro):
        assert a.iterations <= b.iterations + 2
    assert float((xm - xo).abs().max()) < 1e-9


@pytest.mark.gpu
def test_gpu_gmres_path(cuda, oracle):
    m = quad_small()
    bc = N.clamped_stretch_shear_conditions(m, 1.15, 0.05)
    xo, ro = oracle_solve(oracle, m, bc, 2, linear="dense")
    xg, rg, _ = gpu_solve(m, bc, 2, linear="gmres", gmres_rtol=1e-8)
    assert all(r.converged for r in rg)
    assert float((xg - xo).abs().max()) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("coarse", ["vertex", "galerkin"])
def test_gpu_multigrid_newton(cuda, oracle, precision, coarse):
    m = M.regular_box(4, 4, 4, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=1)
    bc = N.clamped_stretch_shear_conditions(m, 1.1, 0.05)
    xo, ro = oracle_solve(oracle, m, bc, 2, linear="dense")
    xg, rg, _ = gpu_solve(m, bc, 2, linear="mg", precision=precision, gmres_rtol=1e-8, mg_coarse=coarse)
    assert all(r.converged for r in rg)
    assert all(max(r.linear_iterations) < 80 for r in rg)
    assert float((xg - xo).abs().max()) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("precision,coarse", [("mixed", "vertex"), ("fp64", "galerkin")])
def test_gpu_csr_int32_matches_int64(cuda, precision, coarse):
    """32-bit CSR indices for the Krylov operator and the multigrid's fine
    level: the same Newton iterates as with 64-bit indices."""
    m = M.regular_box(4, 4, 4, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=1)
    bc = N.clamped_stretch_shear_conditions(m, 1.1, 0.05)
    opt = dict(linear="mg", precision=precision, gmres_rtol=1e-8, mg_coarse=coarse)
    x64, r64, _ = gpu_solve(m, bc, 2, **opt)
    x32, r32, es = gpu_solve(m, bc, 2, csr_index="int32", **opt)
    assert all(r.converged for r in r32)
    assert [r.iterations for r in r32] == [r.iterations for r in r64]
    assert float((x32 - x64).abs().max()) < 1e-9


def test_pressure_increment_rule():
    # increment 1: FULL/N; then NEW = CUR + (CUR - PREV): a linear ramp to FULL
    full = np.array([[0.0, 2.0], [1.0, -3.0]])
    inc = N.PressureIncrements(full)
    vals = [inc.step(i, 8).copy() for i in range(1, 9)]
    for i, v in enumerate(vals, start=1):
        assert np.allclose(v, full * i / 8, rtol=0, atol=1e-15)


def slab_small():
    return M.guccione_slab(3, 3, 2, lengths=(4.0, 4.0, 1.0), seed=3)


def test_guccione_slab_pressure_newton(oracle):
    """Guccione slab with through-thickness fibres, lateral faces clamped,
    bottom-face pressure raised over 4 increments by the reference rule:
    Newton converges quadratically and the slab bulges along +z."""
    m = slab_small()
    es = oracle.EquationsSet(m)
    s = N.LoadStepSolver(es, N.clamped_lateral_conditions(m), N.NewtonOptions(linear="dense"), device="cpu")
    x, reps = s.solve(torch.from_numpy(N.initial_state(m)), 4,
                      pressure=N.PressureIncrements(N.bottom_face_pressure(m, 0.5)))
    assert all(r.converged for r in reps) and all(r.iterations <= 8 for r in reps)
    uz = x[2 * m.nu:3 * m.nu].numpy() - m.X[2]
    assert uz.max() > 0.1 and uz.min() > -1e-9   # pushed along +z, nowhere pulled down


@pytest.mark.gpu
def test_gpu_guccione_slab_matches_oracle_newton(cuda, oracle):
    m = slab_small()
    bc = N.clamped_lateral_conditions(m)
    es_o = oracle.EquationsSet(m)
    so = N.LoadStepSolver(es_o, bc, N.NewtonOptions(linear="dense"), device="cpu")
    xo, ro = so.solve(torch.from_numpy(N.initial_state(m)), 4,
                      pressure=N.PressureIncrements(N.bottom_face_pressure(m, 0.5)))
    from cm_gb300 import FiniteElasticityEquationsSet
    es = FiniteElasticityEquationsSet(m)
    for prec in ("fp64", "mixed"):
        sg = N.LoadStepSolver(es, bc, N.NewtonOptions(linear="dense", precision=prec), device="cuda")
        xg, rg = sg.solve(torch.from_numpy(N.initial_state(m)).cuda(), 4,
                          pressure=N.PressureIncrements(N.bottom_face_pressure(m, 0.5)))
        assert all(r.converged for r in rg)
        if prec == "fp64":
            assert [r.iterations for r in rg] == [r.iterations for r in ro]
        assert float((xg.cpu() - xo).abs().max()) < 1e-9


# ------------------------------------------- native Newton (fe_newton_load_step)
def native_solve(m, bc, increments, on_device=True, **opt):
    """Load increments through the C ABI's Newton load step, the caller
    applying the reference's increment rule to the Dirichlet values."""
    from cm_gb300 import FiniteElasticityEquationsSet
    es = FiniteElasticityEquationsSet(m)
    x = N.initial_state(m)
    reports = []
    for i in range(1, increments + 1):
        cur = x[bc.dofs]
        new = bc.full.copy() if i == increments else \
            np.where(bc.incremented, cur + (bc.full - cur) / (increments - i + 1), bc.full)
        if on_device:
            xd = torch.from_numpy(x).cuda()
            rep = es.newton_load_step(xd, bc.dofs, new, **opt)
            x = xd.cpu().numpy()
        else:
            rep = es.newton_load_step(x, bc.dofs, new, **opt)
        reports.append(rep)
    return x, reports


@pytest.mark.gpu
def test_native_newton_matches_oracle_config1(cuda, oracle):
    """fe_newton_load_step on the 4x4x4 trilinear cube (element pressure),
    5 increments: converges at every increment to the oracle's solution."""
    m = cube_cfg1()
    bc = N.uniaxial_symmetry_conditions(m, 1.1)
    xo, ro = oracle_solve(oracle, m, bc, 5, linear="dense")
    xn, rn = native_solve(m, bc, 5, ksp_rtol=1e-10, ksp_max_iterations=2000)
    for a, b in zip(rn, ro):
        assert a["converged"] == 1 and a["residual_norm"] <= 1e-10
        assert a["iterations"] <= b.iterations + 1
    assert float(np.abs(xn - xo.numpy()).max()) < 1e-9


@pytest.mark.gpu
def test_native_newton_matches_oracle_triquadratic(cuda, oracle):
    """Triquadratic / nodal pressure, clamped stretch and shear, 2 increments:
    the native load step reaches ||r_free||_2 <= 1e-10 and the oracle's
    solution; host and device state buffers give bit-identical results."""
    m = quad_small()
    bc = N.clamped_stretch_shear_conditions(m, 1.15, 0.05)
    xo, ro = oracle_solve(oracle, m, bc, 2, linear="dense")
    xn, rn = native_solve(m, bc, 2, ksp_rtol=1e-8)
    assert all(r["converged"] == 1 and r["residual_norm"] <= 1e-10 for r in rn)
    assert all(r["linear_iterations"] > 0 for r in rn)
    assert float(np.abs(xn - xo.numpy()).max()) < 1e-9
    xh, rh = native_solve(m, bc, 2, on_device=False, ksp_rtol=1e-8)
    assert np.array_equal(xh, xn)
    assert [r["iterations"] for r in rh] == [r["iterations"] for r in rn]


@pytest.mark.gpu
def test_native_newton_rejects_inverted_initial_state(cuda):
    from cm_gb300 import FEError, FiniteElasticityEquationsSet
    m = quad_small()
    es = FiniteElasticityEquationsSet(m)
    x = N.initial_state(m)
    x[:m.nu] *= -1.0  # mirror x: every element inverted
    bc = N.clamped_stretch_shear_conditions(m, 1.1, 0.0)
    with pytest.raises(FEError) as e:
        es.newton_load_step(x, bc.dofs, x[bc.dofs])
    assert e.value.code == -5


@pytest.mark.gpu
@pytest.mark.parametrize("on_device", [True, False])
def test_native_newton_failed_line_search_keeps_state(cuda, on_device):
    """fe_newton_load_step with alpha = 1.5, min_lambda = 0.6 and
    max_step = 1e-9 (see the CPU test above): the first line search fails
    after two trials, x comes back as the state before the step (the
    Dirichlet values applied), line_search_failed is set and the step is not
    converged."""
    from cm_gb300 import FiniteElasticityEquationsSet
    m = quad_small()
    bc = N.clamped_stretch_shear_conditions(m, 1.3, 0.1)
    es = FiniteElasticityEquationsSet(m)
    x0 = N.initial_state(m)
    x0[bc.dofs] = bc.full
    x = torch.from_numpy(x0.copy()).cuda() if on_device else x0.copy()
    rep = es.newton_load_step(x, bc.dofs, bc.full, alpha=1.5, min_lambda=0.6, max_step=1e-9, ksp_rtol=1e-8)
    xr = x.cpu().numpy() if on_device else x
    assert rep["line_search_failed"] == 1 and rep["converged"] == 0
    assert rep["iterations"] == 1 and rep["residual_norm"] == rep["residual_norm_initial"]
    assert np.array_equal(xr, x0)


@pytest.mark.gpu
def test_native_newton_slab_with_cavity_pressure(cuda, oracle):
    """The native load step on the Guccione slab with the bottom-face pressure
    raised by the reference's pressure-increment rule (the caller sets the
    surface load of each increment): the oracle's solution at every
    increment's end state."""
    from cm_gb300 import FiniteElasticityEquationsSet
    m = slab_small()
    bc = N.clamped_lateral_conditions(m)
    so = N.LoadStepSolver(oracle.EquationsSet(m), bc, N.NewtonOptions(linear="dense"), device="cpu")
    xo, ro = so.solve(torch.from_numpy(N.initial_state(m)), 4,
                      pressure=N.PressureIncrements(N.bottom_face_pressure(m, 0.5)))
    es = FiniteElasticityEquationsSet(m)
    pinc = N.PressureIncrements(N.bottom_face_pressure(m, 0.5))
    x = torch.from_numpy(N.initial_state(m)).cuda()
    for i in range(1, 5):
        es.set_surface_pressure(pinc.step(i, 4))
        rep = es.newton_load_step(x, bc.dofs, bc.full, ksp_rtol=1e-10, ksp_max_iterations=3000)
        assert rep["converged"] == 1 and rep["residual_norm"] <= 1e-10
    assert float((x.cpu() - xo).abs().max()) < 1e-9
