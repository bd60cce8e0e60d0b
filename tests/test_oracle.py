"""CPU tests: pin the oracle with the reference's own known answers and
closed forms, and check the product's host-side logic against it.

Known answers used (the reference ships no golden vectors for this path):
  * Gauss-Legendre self-check, basis_routines.f90:5886-5895
  * finite-difference element Jacobian rule, equations_set_routines.f90:
    3086-3130 (delta = (1+||x||_2)*1e-7)
  * homogeneous uniaxial stretch of incompressible Mooney-Rivlin with the
    reference's sigma = dev(sigma_bar) + p I split
    (finite_elasticity_routines.f90:4386-4414)
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cm_gb300 import mesh as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def small_meshes():
    return [
        ("lin_elem", M.regular_box(2, 2, 2, nxi_u=2, pressure="element", law=M.MR, materials=(2.0, 6.0))),
        ("quad_node", M.regular_box(2, 2, 2, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0),
                                    perturb=0.1, seed=3)),
        ("quad_node_guccione", M.regular_box(2, 2, 1, lengths=(4.0, 4.0, 1.0), nxi_u=3, pressure="node",
                                             law=M.GUCCIONE, materials=(0.88, 18.5, 3.58, 1.63),
                                             fibre=np.array([[0.3], [0.1], [-0.2]]), perturb=0.05, seed=5)),
    ]


def test_gauss_legendre_self_check(oracle):
    # basis_routines.f90:5886-5895: integrate y = x + 1 over [0, 1]
    _, w, xi = oracle.basis_tables(2)
    x1 = xi[:3, 0]
    w1 = w[:3] / (w[0] / (2.5 / 9.0))  # recover the 1-D weights of the first xi line
    t1 = np.sum((x1 + 1.0) * w1)
    assert abs(t1 - 1.5) < 1e-15
    # 3-point rule on [0,1]^3 integrates every monomial of degree <= 5 per direction exactly
    for p in range(6):
        for q in range(6):
            val = np.sum(w * xi[:, 0] ** p * xi[:, 1] ** q)
            assert abs(val - 1.0 / ((p + 1) * (q + 1))) < 1e-14
    assert abs(w.sum() - 1.0) < 1e-15


@pytest.mark.parametrize("nxi", [2, 3])
def test_basis_partition_of_unity(oracle, nxi):
    g, _, _ = oracle.basis_tables(nxi)
    assert np.allclose(g[:, 0, :].sum(axis=1), 1.0, atol=1e-15)
    assert np.allclose(g[:, 1:, :].sum(axis=2), 0.0, atol=1e-13)


@pytest.mark.parametrize("dims", [(2, 3, 4), (4, 4, 4), (1, 2, 1)])
@pytest.mark.parametrize("nxi,pmode", [(2, "element"), (3, "node"), (2, "node")])
def test_mesh_numbering_matches_reference_restatement(oracle, dims, nxi, pmode):
    m = M.regular_box(*dims, nxi_u=nxi, pressure=pmode)
    eu, ep, npn = oracle.regular_mesh(*dims, nxi, pmode == "node")
    assert np.array_equal(m.elem_u, eu)
    if pmode == "node":
        assert np.array_equal(m.elem_p, ep)
        assert m.np == npn


def test_stress_uniaxial_closed_form(oracle):
    c1, c2 = 2.0, 6.0
    for lam in (1.0, 1.05, 1.2, 0.9):
        F = np.diag([lam, lam ** -0.5, lam ** -0.5])
        S, _ = oracle.point_stress(M.MR, [c1, c2], F, 0.0)
        # sigma_xx - sigma_yy = 2 (lam^2 - 1/lam)(c1 + c2/lam), independent of p
        assert abs((S[0] - S[1]) - 2.0 * (lam ** 2 - 1.0 / lam) * (c1 + c2 / lam)) < 1e-12 * (1 + abs(S[0]))
        assert abs(S[1] - S[2]) < 1e-13 and np.all(np.abs(S[3:]) < 1e-13)
        assert abs(S[0] + S[1] + S[2]) < 1e-12 * (1 + abs(S[0]))  # p = 0: deviatoric


def test_stress_simple_shear_closed_form(oracle):
    """Mooney-Rivlin under simple shear F = I + gamma e1 (x) e2 (J = 1): the
    classical results sigma_12 = 2 (c1 + c2) gamma,
    sigma_11 - sigma_22 = 2 (c1 + c2) gamma^2 and
    sigma_22 - sigma_33 = -2 c2 gamma^2, whatever the pressure."""
    c1, c2 = 2.0, 6.0
    for gamma in (0.0, 0.05, 0.3, -0.2):
        F = np.eye(3)
        F[0, 1] = gamma
        S, _ = oracle.point_stress(M.MR, [c1, c2], F, 0.7)
        tol = 1e-12 * (1.0 + abs(c1 + c2))
        assert abs(S[3] - 2.0 * (c1 + c2) * gamma) < tol
        assert abs((S[0] - S[1]) - 2.0 * (c1 + c2) * gamma ** 2) < tol
        assert abs((S[1] - S[2]) + 2.0 * c2 * gamma ** 2) < tol
        assert abs(S[4]) < tol and abs(S[5]) < tol
        assert abs((S[0] + S[1] + S[2]) / 3.0 - 0.7) < tol  # the deviator carries no pressure


def test_guccione_stress_uniaxial_closed_form(oracle):
    """Guccione law (finite_elasticity_routines.f90:4419-4424) under isochoric
    uniaxial stretch along the fibre: E = (C - I)/2 is diagonal,
    Q = bf E11^2 + bt (E22^2 + E33^2), S_ii = C e^Q B_i E_i with
    B = (bf, bt, bt), sigma_bar = F S F^T, and the deviator keeps
    sigma_xx - sigma_yy = lam^2 S_11 - S_22 / lam."""
    c = [0.88, 18.5, 3.58, 1.63]
    for lam in (1.0, 1.03, 1.1, 0.95):
        F = np.diag([lam, lam ** -0.5, lam ** -0.5])
        S, _ = oracle.point_stress(M.GUCCIONE, c, F, 0.0)
        e11, e22 = 0.5 * (lam ** 2 - 1.0), 0.5 * (1.0 / lam - 1.0)
        q = c[1] * e11 ** 2 + 2.0 * c[2] * e22 ** 2
        s11, s22 = c[0] * np.exp(q) * c[1] * e11, c[0] * np.exp(q) * c[2] * e22
        expect = lam ** 2 * s11 - s22 / lam
        assert abs((S[0] - S[1]) - expect) < 1e-12 * (1 + abs(expect))
        assert abs(S[1] - S[2]) < 1e-13 and np.all(np.abs(S[3:]) < 1e-13)
        assert abs(S[0] + S[1] + S[2]) < 1e-12 * (1 + abs(S[0]))


@pytest.mark.parametrize("nxi,pmode", [(2, "element"), (3, "node")])
def test_hydrostatic_pressure_traction(oracle, nxi, pmode):
    """Undeformed box (z = X) with a uniform pressure p0: sigma = p0 I, so by
    the divergence theorem the interior displacement rows vanish and each
    face's rows add up to p0 times the face area along its outward normal;
    the incompressibility rows vanish (J = 1)."""
    p0 = -1.7
    L = (1.5, 1.0, 0.5)
    m = M.regular_box(2, 3, 2, lengths=L, nxi_u=nxi, pressure=pmode, law=M.MR, materials=(2.0, 6.0))
    x = np.concatenate([m.X.ravel(), np.full(m.n_pressure, p0)])
    P = oracle.Problem(m)
    rp, col = P.pattern()
    _, r = P.assemble(x, rp, col, jacobian=False)
    nu = m.nu
    i, j, k = m.node_ijk()
    n1, n2, n3 = m.grid_u
    idx = (i, j, k)
    top = (n1 - 1, n2 - 1, n3 - 1)
    area = (L[1] * L[2], L[0] * L[2], L[0] * L[1])
    inner = (i > 0) & (i < n1 - 1) & (j > 0) & (j < n2 - 1) & (k > 0) & (k < n3 - 1)
    for c in range(3):
        rc = r[c * nu:(c + 1) * nu]
        assert np.abs(rc[inner]).max(initial=0.0) < 1e-13
        assert abs(rc[idx[c] == top[c]].sum() - p0 * area[c]) < 1e-12
        assert abs(rc[idx[c] == 0].sum() + p0 * area[c]) < 1e-12
    assert np.abs(r[3 * nu:]).max() < 1e-13


def _strain_energy(law, c, Cb):
    """Strain energy of the isochoric right Cauchy-Green tensor: Mooney-Rivlin
    c1 (I1 - 3) + c2 (I2 - 3), or Guccione (C/2)(e^Q - 1) with E = (Cb - I)/2 and
    Q = bf E11^2 + bt (E22^2 + E33^2 + 2 E23^2) + 2 bfs (E12^2 + E13^2)."""
    if law == M.MR:
        I1 = np.trace(Cb)
        I2 = 0.5 * (I1 ** 2 - np.trace(Cb @ Cb))
        return c[0] * (I1 - 3.0) + c[1] * (I2 - 3.0)
    E = 0.5 * (Cb - np.eye(3))
    Q = (c[1] * E[0, 0] ** 2 + c[2] * (E[1, 1] ** 2 + E[2, 2] ** 2 + 2.0 * E[1, 2] ** 2)
         + 2.0 * c[3] * (E[0, 1] ** 2 + E[0, 2] ** 2))
    return 0.5 * c[0] * (np.exp(Q) - 1.0)


def _material_frame(dX, angles):
    """dX/dnu of the material frame at a point (coordinate_routines.f90:
    4042-4149): the orthonormal frame f = dX/dxi1, h = dX/dxi1 x dX/dxi2,
    g = h x f, rotated by the fibre angle about its third axis, then the
    imbrication angle about its second, then the sheet angle about its first."""
    f = dX[:, 0]
    h = np.cross(dX[:, 0], dX[:, 1])
    g = np.cross(h, f)
    R = np.stack([f / np.linalg.norm(f), g / np.linalg.norm(g), h / np.linalg.norm(h)], axis=1)
    a, b, c = angles
    Rz = np.array([[np.cos(a), -np.sin(a), 0.0], [np.sin(a), np.cos(a), 0.0], [0.0, 0.0, 1.0]])
    Ry = np.array([[np.cos(b), 0.0, np.sin(b)], [0.0, 1.0, 0.0], [-np.sin(b), 0.0, np.cos(b)]])
    Rx = np.array([[1.0, 0.0, 0.0], [0.0, np.cos(c), -np.sin(c)], [0.0, np.sin(c), np.cos(c)]])
    return R @ Rz @ Ry @ Rx


def _energy(oracle, m, x, law, c):
    """The discrete potential the residual is the gradient of:
    Pi = sum_e sum_g w_g J_x [W(C_bar) + p (J - 1)], restated directly from
    the strain energy (numpy, independent of the stress and residual code),
    with C_bar in the material frame of the fibre field when the mesh has one
    (angles interpolated from the nodes with the displacement basis)."""
    gu, w, _ = oracle.basis_tables(m.nxi_u)
    gp, _, _ = oracle.basis_tables(2)
    nu = m.nu
    z = x[:3 * nu].reshape(3, nu)
    pr = x[3 * nu:]
    total = 0.0
    for e in range(m.ne):
        nodes = m.elem_u[e]
        Xe, ze = m.X[:, nodes], z[:, nodes]
        for g in range(27):
            dN = gu[g, 1:4, :]              # [xi_k][a]
            dX, dz = Xe @ dN.T, ze @ dN.T   # [i][k]
            F = dz @ np.linalg.inv(dX)
            J = np.linalg.det(F)
            if getattr(m, "fibre", None) is not None:
                Q = _material_frame(dX, m.fibre[:, nodes] @ gu[g, 0, :])
                F = F @ Q
            Cb = J ** (-2.0 / 3.0) * (F.T @ F)
            pg = pr[m.elem_p[e]] @ gp[g, 0, :] if m.elem_p is not None else pr[e]
            total += w[g] * np.linalg.det(dX) * (_strain_energy(law, c, Cb) + pg * (J - 1.0))
    return total


def test_guccione_fibre_residual_is_the_gradient_of_the_energy(oracle):
    """Variational consistency with a fibre field: the Guccione energy of
    C_bar in the material frame (fibre angles varying through the
    thickness, plus constant imbrication and sheet angles) has the assembled
    residual as its gradient."""
    c = (0.88, 18.5, 3.58, 1.63)
    m = M.guccione_slab(1, 1, 2, lengths=(1.0, 0.8, 1.2), seed=2)
    m.fibre = m.fibre + np.array([[0.0], [0.2], [-0.15]])
    x = M.deformed_state(m, stretch=1.06, shear=0.05, noise=0.02, pressure=-0.4, seed=5)
    P = oracle.Problem(m)
    rp, col = P.pattern()
    _, r = P.assemble(x, rp, col, jacobian=False)
    h = 1e-6
    fd = np.zeros_like(x)
    for i in range(x.size):
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fd[i] = (_energy(oracle, m, xp, M.GUCCIONE, c) - _energy(oracle, m, xm, M.GUCCIONE, c)) / (2.0 * h)
    assert np.abs(fd - r).max() < 1e-7 * np.abs(r).max()


@pytest.mark.parametrize("law", ["mr", "guccione"])
@pytest.mark.parametrize("nxi,pmode", [(2, "element"), (3, "node")])
def test_residual_is_the_gradient_of_the_energy(oracle, nxi, pmode, law):
    """Variational consistency: the assembled residual equals the
    central-difference gradient of the discrete potential (strain energy of
    the isochoric right Cauchy-Green tensor plus p (J - 1)) at a general
    deformed state, for the MR and the Guccione law."""
    lw, c = (M.MR, (2.0, 6.0)) if law == "mr" else (M.GUCCIONE, (0.88, 18.5, 3.58, 1.63))
    m = M.regular_box(1, 1, 2, lengths=(1.0, 0.8, 1.2), nxi_u=nxi, pressure=pmode, law=lw,
                      materials=c, perturb=0.1, seed=2)
    x = M.deformed_state(m, stretch=1.08, shear=0.06, noise=0.02, pressure=-1.3, seed=5)
    P = oracle.Problem(m)
    rp, col = P.pattern()
    _, r = P.assemble(x, rp, col, jacobian=False)
    h = 1e-6
    fd = np.zeros_like(x)
    for i in range(x.size):
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fd[i] = (_energy(oracle, m, xp, lw, c) - _energy(oracle, m, xm, lw, c)) / (2.0 * h)
    assert np.abs(fd - r).max() < 1e-7 * np.abs(r).max()


@pytest.mark.parametrize("law", ["mr", "guccione"])
def test_rigid_motion_leaves_no_residual(oracle, law):
    """Objectivity: a rigid rotation and translation of the undeformed body
    (p = 0) gives C = I, so no stress and a zero residual, for the MR law and
    for the Guccione law with a fibre field (its stress vanishes at E = 0)."""
    if law == "mr":
        m = M.regular_box(2, 2, 2, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=5)
    else:
        m = M.guccione_slab(2, 2, 2, lengths=(2.0, 2.0, 1.0), seed=5)
    rng = np.random.default_rng(7)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1.0
    x = np.concatenate([(q @ m.X + rng.normal(size=(3, 1))).ravel(), np.zeros(m.n_pressure)])
    P = oracle.Problem(m)
    rp, col = P.pattern()
    _, r = P.assemble(x, rp, col, jacobian=False)
    assert np.abs(r).max() < 1e-12


@pytest.mark.parametrize("nxi,pmode", [(2, "element"), (3, "node")])
def test_patch_uniaxial_residual(oracle, nxi, pmode):
    """Homogeneous uniaxial stretch: interior and pressure rows vanish, the
    x = 1 face carries sigma_xx times the deformed face area."""
    c1, c2, lam = 2.0, 6.0, 1.1
    m = M.regular_box(2, 2, 2, nxi_u=nxi, pressure=pmode, materials=(c1, c2))
    F = np.diag([lam, lam ** -0.5, lam ** -0.5])
    S0, _ = oracle.point_stress(M.MR, [c1, c2], F, 0.0)
    p_star = -S0[1]  # lateral traction free
    x = np.concatenate([(F @ m.X).ravel(), np.full(m.n_pressure, p_star)])
    P = oracle.Problem(m)
    rp, col = P.pattern()
    _, r = P.assemble(x, rp, col, jacobian=False)
    nu = m.nu
    i, j, k = m.node_ijk()
    n1, n2, n3 = m.grid_u
    sxx = 2.0 * (lam ** 2 - 1.0 / lam) * (c1 + c2 / lam)
    scale = abs(sxx)
    inner = (i > 0) & (i < n1 - 1) & (j > 0) & (j < n2 - 1) & (k > 0) & (k < n3 - 1)
    for c in range(3):
        assert np.all(np.abs(r[c * nu:(c + 1) * nu][inner]) < 1e-12 * scale)
    assert np.all(np.abs(r[3 * nu:]) < 1e-13)
    face = i == n1 - 1
    assert abs(r[:nu][face].sum() - sxx / lam) < 1e-12 * scale
    assert abs(r[:nu][i == 0].sum() + sxx / lam) < 1e-12 * scale
    for c in (1, 2):
        for sel in (face, i == 0):
            assert abs(r[c * nu:(c + 1) * nu][sel].sum()) < 1e-12 * scale


@pytest.mark.parametrize("name,mesh", small_meshes())
def test_element_jacobian_matches_fd(oracle, name, mesh):
    """Analytic element Jacobian vs the reference's one-sided FD rule."""
    x = M.deformed_state(mesh, stretch=1.08, shear=0.04, noise=0.05, pressure=-1.5, seed=11)
    P = oracle.Problem(mesh)
    for e in (0, mesh.ne - 1):
        K = P.element_jacobian(e, x)
        Kfd = P.element_jacobian_fd(e, x)
        assert np.array_equal(K, K.T)
        err = np.abs(K - Kfd).max() / np.abs(K).max()
        assert err < 1e-4, (name, e, err)  # one-sided rule: O(delta) truncation error
        # central differences converge as O(h^2): the analytic tangent is the
        # exact derivative of the residual, not just close to the FD rule
        dofs = P.element_dofs(e)
        h = 1e-5
        Kc = np.zeros_like(K)
        for j, d in enumerate(dofs):
            xp, xm = x.copy(), x.copy()
            xp[d] += h
            xm[d] -= h
            Kc[:, j] = (P.element_residual(e, xp) - P.element_residual(e, xm)) / (2 * h)
        assert np.abs(K - Kc).max() / np.abs(K).max() < 1e-7, name


def test_pattern_closed_form_counts(oracle):
    # 9(3e+1)^3 + 2*3*(2e)^3 + e^3 for trilinear u / element-based p
    for e in (1, 2, 4):
        m = M.regular_box(e, e, e, nxi_u=2, pressure="element")
        rp, col = oracle.Problem(m).pattern()
        assert rp[-1] - 1 == 9 * (3 * e + 1) ** 3 + 2 * 3 * (2 * e) ** 3 + e ** 3
    # 9(8e+1)^3 + 2*3*(5e+1)^3 + (3e+1)^3 for triquadratic u / trilinear p
    for e in (1, 2, 3):
        m = M.regular_box(e, e, e, nxi_u=3, pressure="node")
        rp, col = oracle.Problem(m).pattern()
        assert rp[-1] - 1 == 9 * (8 * e + 1) ** 3 + 2 * 3 * (5 * e + 1) ** 3 + (3 * e + 1) ** 3
    m = M.regular_box(4, 4, 4, nxi_u=2, pressure="element")
    assert oracle.Problem(m).pattern()[0][-1] - 1 == 22909


def _desc(m, keep):
    from cm_gb300 import _lib

    def arr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data
    d = _lib.FEMeshDesc()
    mats = np.asarray(m.materials, dtype=np.float64)
    d.num_elements, d.num_nodes_u, d.num_nodes_p = m.ne, m.nu, m.np
    d.nodes_per_xi_u, d.pressure_interpolation, d.law = m.nxi_u, m.p_mode, m.law
    d.num_material_components = mats.shape[-1]
    d.materials_per_element = 1 if mats.ndim == 2 else 0
    d.element_nodes_u = arr(m.elem_u, np.int32)
    d.element_nodes_p = arr(m.elem_p, np.int32)
    d.geometry = arr(m.X, np.float64)
    d.materials = arr(mats, np.float64)
    d.fibre_angles = arr(m.fibre, np.float64)
    return d


def _shuffled(m, seed=7):
    """The mesh with its elements in a seeded random order."""
    import dataclasses
    perm = np.random.default_rng(seed).permutation(m.ne)
    return dataclasses.replace(m, elem_u=np.ascontiguousarray(m.elem_u[perm]),
                               elem_p=None if m.elem_p is None else np.ascontiguousarray(m.elem_p[perm]))


def product_pattern(m, base=1):
    from cm_gb300 import _lib
    L = _lib.load()
    keep = []
    d = _desc(m, keep)
    nd, nnz = C.c_int64(), C.c_int64()
    _lib.check(L.fe_structure_calculate(C.byref(d), base, C.byref(nd), C.byref(nnz), None, None))
    rp = np.zeros(nd.value + 1, dtype=np.int32)
    col = np.zeros(nnz.value, dtype=np.int32)
    _lib.check(L.fe_structure_calculate(C.byref(d), base, C.byref(nd), C.byref(nnz), rp.ctypes.data,
                                        col.ctypes.data))
    return rp, col


@pytest.mark.parametrize("name,mesh", small_meshes() + [
    ("lin_elem_4", M.regular_box(4, 4, 4, nxi_u=2, pressure="element")),
    ("quad_node_3x2x4", M.regular_box(3, 2, 4, nxi_u=3, pressure="node", perturb=0.1)),
    ("lin_node", M.regular_box(3, 3, 2, nxi_u=2, pressure="node")),
    ("quad_elem", M.regular_box(2, 3, 2, nxi_u=3, pressure="element")),
    ("cylinder", M.thick_cylinder(2, 8, 2, 0.5, 1.0, 1.0)),
    ("quad_node_shuffled", _shuffled(M.regular_box(3, 2, 2, nxi_u=3, pressure="node", perturb=0.1))),
])
def test_product_pattern_bit_exact(oracle, name, mesh):
    rp_o, col_o = oracle.Problem(mesh).pattern()
    rp_p, col_p = product_pattern(mesh, base=1)
    assert np.array_equal(rp_o, rp_p), name
    assert np.array_equal(col_o, col_p), name
    rp0, col0 = product_pattern(mesh, base=0)
    assert np.array_equal(rp0 + 1, rp_p) and np.array_equal(col0 + 1, col_p)


def test_product_rejects_bad_mesh():
    from cm_gb300 import _lib
    L = _lib.load()
    m = M.regular_box(2, 2, 2, nxi_u=2)
    keep = []
    d = _desc(m, keep)
    d.nodes_per_xi_u = 4
    nd, nnz = C.c_int64(), C.c_int64()
    assert L.fe_structure_calculate(C.byref(d), 1, C.byref(nd), C.byref(nnz), None, None) == _lib.FE_ERR_INVALID_ARGUMENT
    assert "nodes_per_xi_u" in _lib.last_error()
    d = _desc(m, keep)
    bad = np.array(m.elem_u, dtype=np.int32)
    bad[0, 0] = m.nu + 5
    keep.append(bad)
    d.element_nodes_u = bad.ctypes.data
    assert L.fe_structure_calculate(C.byref(d), 1, C.byref(nd), C.byref(nnz), None, None) == _lib.FE_ERR_INVALID_ARGUMENT
    d = _desc(m, keep)
    d.law = 7
    assert L.fe_structure_calculate(C.byref(d), 1, C.byref(nd), C.byref(nnz), None, None) == _lib.FE_ERR_INVALID_ARGUMENT


def test_threaded_assembly_matches_serial(oracle):
    m = M.regular_box(3, 3, 3, nxi_u=3, pressure="node", perturb=0.1, seed=2)
    x = M.deformed_state(m, noise=0.05)
    P = oracle.Problem(m)
    rp, col = P.pattern()
    v1, r1 = P.assemble(x, rp, col, nthreads=1)
    v4, r4 = P.assemble(x, rp, col, nthreads=4)
    assert np.allclose(v1, v4, rtol=1e-13, atol=1e-13 * np.abs(v1).max())
    assert np.allclose(r1, r4, rtol=1e-13, atol=1e-13 * np.abs(r1).max())


def test_assembled_jacobian_is_symmetric(oracle):
    m = M.regular_box(2, 2, 2, nxi_u=3, pressure="node", perturb=0.1)
    x = M.deformed_state(m, noise=0.05)
    P = oracle.Problem(m)
    rp, col = P.pattern()
    v, _ = P.assemble(x, rp, col, residual=False)
    import scipy.sparse as sp
    A = sp.csr_matrix((v, col - 1, rp - 1), shape=(P.ndofs, P.ndofs))
    assert abs(A - A.T).max() == 0.0


def test_abi_exports_every_declared_symbol():
    """libcm_fe.so loads and exports every function include/*.h declares."""
    from cm_gb300 import _lib
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        header = open(os.path.join(ROOT, "include", h)).read()
        names += re.findall(r"^(?:int|void) (\w+)\(", header, flags=re.M)
    names = sorted(set(names))
    assert len(names) >= 22
    L = _lib.load()
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.SIGNATURES, n


def _pressure_mesh(nxi, pmode, p0=1.5):
    m = M.regular_box(2, 2, 1, lengths=(2.0, 2.0, 1.0), nxi_u=nxi, pressure=pmode, law=M.MR,
                      materials=(2.0, 6.0), perturb=0.05, seed=4)
    sp = np.zeros((3, m.nu))
    i, j, k = m.node_ijk()
    sp[2, k == 0] = p0 * (1.0 + 0.2 * i[k == 0] / i.max())  # load on the z = 0 faces (normal xi3)
    return m, sp


@pytest.mark.parametrize("nxi,pmode", [(2, "element"), (3, "node")])
def test_surface_pressure_total_force(oracle, nxi, pmode):
    """Uniform pressure p on the flat z = 0 face of the undeformed box: the
    surface part of the residual sums to p times the face area along the
    outward normal (-z), and has no in-plane resultant."""
    m = M.regular_box(2, 2, 1, lengths=(2.0, 3.0, 1.0), nxi_u=nxi, pressure=pmode)
    x = np.concatenate([m.X.ravel(), np.zeros(m.n_pressure)])
    P = oracle.Problem(m)
    rp, col = P.pattern()
    _, r0 = P.assemble(x, rp, col, jacobian=False)
    sp = np.zeros((3, m.nu))
    i, j, k = m.node_ijk()
    sp[2, k == 0] = 0.7  # faces normal to xi3 with nonzero nodal pressure: the z = 0 faces only
    P.set_surface_pressure(sp)
    _, r1 = P.assemble(x, rp, col, jacobian=False)
    d = r1 - r0
    nu = m.nu
    assert abs(d[2 * nu:3 * nu].sum() - (-0.7 * 6.0)) < 1e-12
    assert abs(d[:nu].sum()) < 1e-12 and abs(d[nu:2 * nu].sum()) < 1e-12
    assert np.all(d[2 * nu:3 * nu][k > 0] == 0.0)


@pytest.mark.parametrize("nxi,pmode", [(2, "element"), (3, "node")])
def test_surface_pressure_tangent_matches_fd_on_lower_blocks(oracle, nxi, pmode):
    """The follower-load tangent is computed for the lower displacement blocks
    and mirrored (finite_elasticity_routines.f90:1075-1078, :1149-1153), so the
    analytic element Jacobian equals the central-difference derivative of the
    residual on every entry except the mirrored upper off-diagonal blocks."""
    m, sp = _pressure_mesh(nxi, pmode)
    x = M.deformed_state(m, stretch=1.05, shear=0.03, noise=0.03, pressure=-1.0, seed=8)
    P = oracle.Problem(m)
    P.set_surface_pressure(sp)
    npe = nxi ** 3
    for e in range(m.ne):
        K = P.element_jacobian(e, x)
        dofs = P.element_dofs(e)
        Kc = np.zeros_like(K)
        h = 1e-6
        for jj, d in enumerate(dofs):
            xp, xm = x.copy(), x.copy()
            xp[d] += h
            xm[d] -= h
            Kc[:, jj] = (P.element_residual(e, xp) - P.element_residual(e, xm)) / (2 * h)
        n = K.shape[0]
        comp = np.minimum(np.arange(n) // npe, 3)
        mask = ~((comp[:, None] < comp[None, :]) & (comp[:, None] < 3) & (comp[None, :] < 3))
        err = np.abs(K - Kc)[mask].max() / np.abs(K).max()
        assert err < 1e-7, (e, err)
    # the surface term is present: the element Jacobian changes with the load
    P2 = oracle.Problem(m)
    assert np.abs(P.element_jacobian(0, x) - P2.element_jacobian(0, x)).max() > 1e-3


def test_sampled_oracle_assembly_adds_up_to_the_full_assembly(oracle):
    """or_assemble_range (the reference arm's timing sample) over windows that
    cover the mesh gives the full or_assemble result (same colour order)."""
    m = M.regular_box(3, 2, 2, nxi_u=3, pressure="node", perturb=0.1, seed=2)
    x = M.deformed_state(m, stretch=1.05, shear=0.02, noise=0.02, seed=3)
    P = oracle.Problem(m)
    rp, col = P.pattern()
    full_v, full_r = P.assemble(x, rp, col, nthreads=2)
    v = np.zeros_like(full_v)
    r = np.zeros_like(full_r)
    L = oracle.lib()
    for first in range(0, m.ne, 5):
        n = min(5, m.ne - first)
        assert L.or_assemble_range(P.ref, x.ctypes.data, rp.ctypes.data, col.ctypes.data, v.ctypes.data,
                                   r.ctypes.data, first, n, 2) == 0
    S = np.abs(full_v).max()
    assert np.abs(v - full_v).max() <= 1e-13 * S
    assert np.abs(r - full_r).max() <= 1e-13 * np.abs(full_r).max()
