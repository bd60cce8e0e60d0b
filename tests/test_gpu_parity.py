"""GPU parity tests: the CUDA path through the C ABI against the FP64 oracle.

Tolerance (FP64 path, per entry): |gpu - oracle| <= 1e-12 |oracle| + 1e-13 S,
where S is the largest magnitude of the element matrix / vector (element
level) or of the assembled array (global level).  The absolute floor covers
entries that cancel to (near) zero, whose rounding noise is set by the size
of the terms, not by the entry.  The CSR pattern must match bit for bit.
The FP32 block of the mixed path (tensor-core contraction) is checked at
MIXED_UU_TOL relative to S.
"""
import dataclasses

import numpy as np
import pytest

from cm_gb300 import FEError, FiniteElasticityEquationsSet, _lib
from cm_gb300 import mesh as M

pytestmark = pytest.mark.gpu

REL, FLOOR = 1e-12, 1e-13


@pytest.fixture(scope="module")
def torch():
    import torch as _torch
    if not _torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.load()
    return _torch


def assert_entrywise(gpu, ref, rel=REL, floor=FLOOR, scale=None, what=""):
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert gpu.shape == ref.shape, what
    S = np.abs(ref).max() if scale is None else scale
    err = np.abs(gpu - ref)
    bound = rel * np.abs(ref) + floor * S
    bad = err > bound
    assert not bad.any(), "%s: %d entries off, worst %.3e (bound %.3e, scale %.3e)" % (
        what, bad.sum(), err.max(), bound[np.argmax(err - bound)], S)


def meshes():
    return {
        "cfg1_lin_elem_mr": M.regular_box(4, 4, 4, nxi_u=2, pressure="element", law=M.MR, materials=(2.0, 6.0)),
        "quad_node_mr_perturbed": M.regular_box(3, 2, 2, nxi_u=3, pressure="node", law=M.MR,
                                                materials=(2.0, 6.0), perturb=0.1, seed=7),
        "quad_node_guccione_fibres": M.regular_box(2, 2, 2, lengths=(4.0, 4.0, 1.0), nxi_u=3, pressure="node",
                                                   law=M.GUCCIONE, materials=(0.88, 18.5, 3.58, 1.63),
                                                   fibre=np.array([[0.4], [0.1], [-0.3]]), perturb=0.05, seed=9),
        "lin_node_mr": M.regular_box(3, 3, 2, nxi_u=2, pressure="node", law=M.MR, materials=(1.0, 3.0)),
        "quad_elem_mr": M.regular_box(2, 1, 2, nxi_u=3, pressure="element", law=M.MR, materials=(0.5, 9.0)),
    }


def state(m, seed=3):
    return M.deformed_state(m, stretch=1.07, shear=0.05, noise=0.04, pressure=-2.0, seed=seed)


@pytest.mark.parametrize("name", list(meshes()))
def test_element_parity(torch, oracle, name):
    m = meshes()[name]
    x = state(m)
    es = FiniteElasticityEquationsSet(m)
    P = oracle.Problem(m)
    xd = torch.from_numpy(x).cuda()
    K = es.element_jacobians(xd).cpu().numpy()
    R = es.element_residuals(xd).cpu().numpy()
    es.check_status(xd)
    for e in range(m.ne):
        Ko = P.element_jacobian(e, x)
        Ro = P.element_residual(e, x)
        assert_entrywise(K[e], Ko, what="%s K_e[%d]" % (name, e))
        assert_entrywise(R[e], Ro, what="%s r_e[%d]" % (name, e))


@pytest.mark.parametrize("name", list(meshes()))
def test_assembled_parity_and_pattern(torch, oracle, name):
    m = meshes()[name]
    x = state(m)
    es = FiniteElasticityEquationsSet(m)
    P = oracle.Problem(m)
    rp_o, col_o = P.pattern()
    rp, col = es.csr_pattern(base=1)
    assert np.array_equal(rp, rp_o) and np.array_equal(col, col_o)
    vo, ro = P.assemble(x, rp_o, col_o, nthreads=1)
    xd = torch.from_numpy(x).cuda()
    r = torch.empty_like(xd)
    v = es.jacobian_evaluate(xd, r=r)
    r2 = es.residual_evaluate(xd)
    es.check_status(xd)
    assert_entrywise(v.cpu().numpy(), vo, what=name + " CSR values")
    assert_entrywise(r.cpu().numpy(), ro, what=name + " residual (Jacobian pass)")
    assert_entrywise(r2.cpu().numpy(), ro, what=name + " residual")


def test_host_and_device_pointers_agree(torch):
    m = meshes()["quad_node_mr_perturbed"]
    x = state(m)
    es = FiniteElasticityEquationsSet(m)
    vh = es.jacobian_evaluate(x)                 # numpy in, numpy out
    rh = es.residual_evaluate(x)
    xd = torch.from_numpy(x).cuda()
    vd = es.jacobian_evaluate(xd).cpu().numpy()
    rd = es.residual_evaluate(xd).cpu().numpy()
    assert np.array_equal(vh, vd) and np.array_equal(rh, rd)


@pytest.mark.parametrize("order", ["staged", "coloured"])
def test_mixed_outputs_in_pinned_pageable_and_device_memory(torch, order):
    """The mixed assembly gives the same bits whether its outputs are device
    memory, page-locked host memory (written in place by the row gather in
    the staged order) or ordinary host memory (staged through the device),
    and a call given host outputs returns only after they are written."""
    m = meshes()["quad_node_mr_perturbed"]
    x = state(m)
    es = FiniteElasticityEquationsSet(m)
    es.set_assembly_order(order)
    xd = torch.from_numpy(x).cuda()
    rd = torch.empty_like(xd)
    ud, cd = es.jacobian_evaluate_mixed(xd, r=rd)
    ref = [t.cpu().numpy() for t in (ud, cd, rd)]
    for pinned in (True, False):
        bufs = [torch.full((es.nnz_uu,), float("nan"), dtype=torch.float32),
                torch.full((es.nnz_coupling,), float("nan"), dtype=torch.float64),
                torch.full((es.ndofs,), float("nan"), dtype=torch.float64)]
        if pinned:
            bufs = [b.pin_memory() for b in bufs]
        hu, hc, hr = (b.numpy() for b in bufs)
        es.jacobian_evaluate_mixed(x, hu, hc, hr)
        for a, b in zip((hu, hc, hr), ref):  # no synchronisation: the call has waited
            assert np.array_equal(a, b), (order, pinned)


@pytest.mark.parametrize("case", ["box", "shuffled_elements", "element_pressure"])
def test_streamed_host_outputs(torch, case):
    """Host outputs delivered chunk by chunk while the remaining elements
    assemble (fe_set_host_output streamed, 1..16 launches), written in place
    or copied after the assembly: the same bits as device outputs, in
    page-locked and pageable memory, for a call without the residual and with
    one output in device memory, and for an element order unrelated to the
    node numbering (rows then complete late; the last chunk copies them)."""
    if case == "element_pressure":
        m = M.regular_box(7, 6, 5, nxi_u=2, pressure="element", perturb=0.1, seed=3)
    else:
        m = M.regular_box(9, 7, 6, nxi_u=3, pressure="node", perturb=0.1, seed=3)
        if case == "shuffled_elements":
            perm = np.random.default_rng(5).permutation(m.ne)
            m = dataclasses.replace(m, elem_u=np.ascontiguousarray(m.elem_u[perm]),
                                    elem_p=np.ascontiguousarray(m.elem_p[perm]))
    x = state(m)
    es = FiniteElasticityEquationsSet(m)
    xd = torch.from_numpy(x).cuda()
    rd = torch.empty_like(xd)
    ud, cd = es.jacobian_evaluate_mixed(xd, r=rd)
    ref = [t.cpu().numpy() for t in (ud, cd, rd)]
    l0 = es.launch_count()
    es.set_host_output("streamed", 5)
    es.jacobian_evaluate_mixed(x, *(np.empty_like(a) for a in ref))
    assert es.launch_count() - l0 == 5
    for mode, chunks in (("streamed", 0), ("streamed", 1), ("streamed", 3), ("streamed", 16),
                         ("in_place", 0), ("after", 0)):
        es.set_host_output(mode, chunks)
        for pinned in (True, False):
            bufs = [torch.full((es.nnz_uu,), float("nan"), dtype=torch.float32),
                    torch.full((es.nnz_coupling,), float("nan"), dtype=torch.float64),
                    torch.full((es.ndofs,), float("nan"), dtype=torch.float64)]
            if pinned:
                bufs = [b.pin_memory() for b in bufs]
            hu, hc, hr = (b.numpy() for b in bufs)
            es.jacobian_evaluate_mixed(x, hu, hc, hr)
            for a, b in zip((hu, hc, hr), ref):  # no synchronisation: the call has waited
                assert np.array_equal(a, b), (case, mode, chunks, pinned)
        hu = np.full(es.nnz_uu, np.nan, dtype=np.float32)
        cdev = torch.full((es.nnz_coupling,), float("nan"), dtype=torch.float64, device="cuda")
        es.jacobian_evaluate_mixed(x, hu, cdev, None)
        assert np.array_equal(hu, ref[0]) and np.array_equal(cdev.cpu().numpy(), ref[1]), (case, mode, chunks)
    with pytest.raises(FEError):
        es.set_host_output("streamed", 17)


def test_deterministic(torch):
    m = M.regular_box(6, 5, 4, nxi_u=3, pressure="node", perturb=0.1, seed=1)
    x = torch.from_numpy(state(m)).cuda()
    es = FiniteElasticityEquationsSet(m)
    a = es.jacobian_evaluate(x).clone()
    b = es.jacobian_evaluate(x).clone()
    assert torch.equal(a, b)
    for order in ("staged", "coloured"):
        es.set_assembly_order(order)
        ra, rb = torch.empty_like(x), torch.empty_like(x)
        ua, ca = es.jacobian_evaluate_mixed(x, r=ra)
        ua, ca = ua.clone(), ca.clone()
        ub, cb = es.jacobian_evaluate_mixed(x, r=rb)
        assert torch.equal(ua, ub) and torch.equal(ca, cb) and torch.equal(ra, rb), order


MIXED_UU_TOL = 1e-4  # BF16x3 tensor-core products, FP32 accumulation, relative to the largest entry
# Double-float (FP32 pair, ~48-bit) high-precision phases: per-entry tolerance
# 1e-11 relative with a 1e-12 S floor (FP64 mode uses the FP64 tolerance).
REL_DD, FLOOR_DD = 1e-11, 1e-12


@pytest.mark.parametrize("order", ["staged", "coloured"])
@pytest.mark.parametrize("mode", ["fp64", "double_float"])
@pytest.mark.parametrize("name", list(meshes()))
def test_mixed_precision(torch, oracle, name, mode, order):
    """High-precision parts of the mixed path (coupling blocks, residual)
    match the oracle at the FP64 tolerance (fp64 mode) or the double-float
    tolerance; the FP32 displacement block matches it to MIXED_UU_TOL of the
    largest entry; for both assembly orders (per-element records and a row
    gather, or colour-ordered adds into the CSR arrays)."""
    m = meshes()[name]
    x = state(m)
    P = oracle.Problem(m)
    rp_o, col_o = P.pattern()
    vo, ro = P.assemble(x, rp_o, col_o, nthreads=1)
    es = FiniteElasticityEquationsSet(m)
    es.set_high_precision(mode)
    es.set_assembly_order(order)
    rel, floor = (REL, FLOOR) if mode == "fp64" else (REL_DD, FLOOR_DD)
    xd = torch.from_numpy(x).cuda()
    rm = torch.empty_like(xd)
    vu, vc = es.jacobian_evaluate_mixed(xd, r=rm)
    es.check_status(xd)
    full = es.mixed_to_full(vu.cpu().numpy(), vc.cpu().numpy())
    uu_rp, cp_rp = es.mixed_layout()
    rp, _ = es.csr_pattern()
    is_uu = np.zeros(es.nnz, dtype=bool)
    for r in range(3 * m.nu):
        is_uu[rp[r]:rp[r] + (uu_rp[r + 1] - uu_rp[r])] = True
    assert_entrywise(full[~is_uu], vo[~is_uu], rel, floor, what=name + " mixed coupling blocks")
    assert_entrywise(rm.cpu().numpy(), ro, rel, floor, what=name + " mixed residual")
    r_only = es.residual_evaluate(xd)  # colour-ordered: the same sums as the coloured mixed assembly
    if order == "coloured":
        assert torch.equal(r_only, rm)
    else:
        assert_entrywise(r_only.cpu().numpy(), ro, rel, floor, what=name + " residual-only")
    S = np.abs(vo).max()
    err = np.abs(full[is_uu] - vo[is_uu]).max() / S
    assert err < MIXED_UU_TOL, (name, err)
    # exact symmetry of the assembled FP32 block (mirrored like the reference)
    import scipy.sparse as sp
    A = sp.csr_matrix((full, col_o - 1, rp_o - 1), shape=(es.ndofs, es.ndofs))
    assert abs(A - A.T).max() == 0.0


@pytest.mark.parametrize("name", ["quad_node_mr_perturbed", "quad_node_guccione_fibres", "cfg1_lin_elem_mr"])
def test_rigid_motion_leaves_no_residual(torch, name):
    """Known answer on the CUDA path: a rigid rotation and translation of the
    undeformed body with p = 0 has C = I, hence no stress and a zero
    residual, for the FP64 and the mixed path alike."""
    m = meshes()[name]
    rng = np.random.default_rng(11)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1.0
    x = np.concatenate([(q @ m.X + rng.normal(size=(3, 1))).ravel(), np.zeros(m.n_pressure)])
    es = FiniteElasticityEquationsSet(m)
    xd = torch.from_numpy(x).cuda()
    r = es.residual_evaluate(xd)
    es.check_status(xd)
    assert float(r.abs().max()) < 1e-11
    rm = torch.empty_like(xd)
    es.jacobian_evaluate_mixed(xd, r=rm)
    es.check_status(xd)
    assert float(rm.abs().max()) < 1e-11
    v = es.jacobian_evaluate(xd)
    rf = torch.empty_like(xd)
    es.jacobian_evaluate(xd, v, rf)
    es.check_status(xd)
    assert float(rf.abs().max()) < 1e-11


def test_inverted_element_reports_numerical_error(torch):
    """A host-made fault: an element turned inside out gives FE_ERR_NUMERICAL
    (the kernel flags it, it does not trap)."""
    m = M.regular_box(2, 2, 2, nxi_u=2, pressure="element")
    x = state(m)
    nu = m.nu
    n0 = m.elem_u[0, 0]
    x[n0] += 3.0 * m.lengths[0] / m.dims[0]  # push a corner through the element
    es = FiniteElasticityEquationsSet(m)
    with pytest.raises(FEError) as ei:
        es.residual_evaluate(x)
    assert ei.value.code == _lib.FE_ERR_NUMERICAL
    # the context stays usable
    r = es.residual_evaluate(state(m))
    assert np.isfinite(r).all()
    assert nu > 0


def _csr_matvec(torch, rp, col, vals, v):
    n = rp.numel() - 1
    rows = torch.repeat_interleave(torch.arange(n, device=v.device), rp[1:] - rp[:-1])
    y = torch.zeros(n, dtype=torch.float64, device=v.device)
    y.index_add_(0, rows, vals.to(torch.float64) * v[col.long()])
    return y


def test_full_size_config2_properties(torch, oracle):
    """32^3 triquadratic / trilinear-pressure box (824k u dofs, 178.7M nnz):
    size-independent checks of the FP64 and mixed paths — element-sampled
    parity against the oracle, symmetry u^T J v = v^T J u, and J v against a
    central difference of the residual."""
    m = M.regular_box(32, 32, 32, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=2)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-2.0, seed=4)
    es = FiniteElasticityEquationsSet(m)
    assert es.nnz == 178723696 and es.ndofs == 859812
    xd = torch.from_numpy(x).cuda()
    sample = [0, 1, 777, 16383, 20000, m.ne - 1]
    P = oracle.Problem(m)
    for e in sample:
        Ke = es.element_jacobians(xd, e, 1).cpu().numpy()[0]
        assert_entrywise(Ke, P.element_jacobian(e, x), what="cfg2 K_e[%d]" % e)
    rp, col = es.csr_pattern()
    rp_d = torch.from_numpy(rp.astype(np.int64)).cuda()
    col_d = torch.from_numpy(col).cuda()
    r = torch.empty_like(xd)
    vals = es.jacobian_evaluate(xd, r=r)
    es.check_status(xd)
    g = torch.Generator(device="cuda").manual_seed(0)
    u = torch.randn(es.ndofs, dtype=torch.float64, device="cuda", generator=g)
    v = torch.randn(es.ndofs, dtype=torch.float64, device="cuda", generator=g)
    Jv = _csr_matvec(torch, rp_d, col_d, vals, v)
    Ju = _csr_matvec(torch, rp_d, col_d, vals, u)
    a, b = float(u @ Jv), float(v @ Ju)
    assert abs(a - b) <= 1e-10 * (abs(a) + 1e-30)
    h = 1e-6
    rp_ = es.residual_evaluate(xd + h * v)
    rm_ = es.residual_evaluate(xd - h * v)
    fd = (rp_ - rm_) / (2 * h)
    assert float((fd - Jv).norm() / Jv.norm()) < 1e-6
    # mixed path on the same state
    vu, vc = es.jacobian_evaluate_mixed(xd)
    uu_rp, cp_rp = es.mixed_layout()
    nu3 = 3 * m.nu
    uu_idx = np.concatenate([np.arange(rp[i], rp[i] + uu_rp[i + 1] - uu_rp[i]) for i in range(0, nu3, 997)])
    uu_pos = np.concatenate([np.arange(uu_rp[i], uu_rp[i + 1]) for i in range(0, nu3, 997)])
    d64 = vals[torch.from_numpy(uu_idx).cuda()]
    d32 = vu[torch.from_numpy(uu_pos).cuda()].double()
    assert float((d64 - d32).abs().max()) < MIXED_UU_TOL * float(vals.abs().max())


def test_native_library_launches(torch):
    m = meshes()["cfg1_lin_elem_mr"]
    es = FiniteElasticityEquationsSet(m)
    before = es.launch_count()
    es.jacobian_evaluate(torch.from_numpy(state(m)).cuda())
    torch.cuda.synchronize()
    assert es.launch_count() - before >= 8  # one launch per element colour


def pressure_meshes():
    out = {}
    for name, nxi, pm, law, mats, fib in [
            ("quad_node_mr", 3, "node", M.MR, (2.0, 6.0), None),
            ("lin_elem_mr", 2, "element", M.MR, (2.0, 6.0), None),
            ("quad_node_guccione_fibres", 3, "node", M.GUCCIONE, (0.88, 18.5, 3.58, 1.63),
             np.array([[-0.5], [0.0], [0.0]]))]:
        m = M.regular_box(3, 2, 2, lengths=(4.0, 3.0, 2.0), nxi_u=nxi, pressure=pm, law=law, materials=mats,
                          perturb=0.05, seed=6, fibre=fib)
        sp = np.zeros((3, m.nu))
        i, j, k = m.node_ijk()
        sp[2, k == 0] = 1.2 * (1.0 + 0.3 * i[k == 0] / i.max())   # z = 0 faces (normal xi3)
        sp[0, i == i.max()] = -0.4                                 # x = max faces (normal xi1)
        out[name] = (m, sp)
    return out


@pytest.mark.parametrize("name", list(pressure_meshes()))
def test_surface_pressure_parity(torch, oracle, name):
    m, sp = pressure_meshes()[name]
    x = state(m)
    P = oracle.Problem(m)
    P.set_surface_pressure(sp)
    rp_o, col_o = P.pattern()
    vo, ro = P.assemble(x, rp_o, col_o, nthreads=1)
    es = FiniteElasticityEquationsSet(m)
    es.set_surface_pressure(sp)
    xd = torch.from_numpy(x).cuda()
    # element level
    K = es.element_jacobians(xd).cpu().numpy()
    R = es.element_residuals(xd).cpu().numpy()
    for e in range(m.ne):
        assert_entrywise(K[e], P.element_jacobian(e, x), what="%s K_e[%d]" % (name, e))
        assert_entrywise(R[e], P.element_residual(e, x), what="%s r_e[%d]" % (name, e))
    # assembled, FP64
    r = torch.empty_like(xd)
    v = es.jacobian_evaluate(xd, r=r)
    assert_entrywise(v.cpu().numpy(), vo, what=name + " CSR values")
    assert_entrywise(r.cpu().numpy(), ro, what=name + " residual")
    assert_entrywise(es.residual_evaluate(xd).cpu().numpy(), ro, what=name + " residual-only")
    # assembled, mixed
    rm = torch.empty_like(xd)
    vu, vc = es.jacobian_evaluate_mixed(xd, r=rm)
    es.check_status(xd)
    full = es.mixed_to_full(vu.cpu().numpy(), vc.cpu().numpy())
    assert np.abs(full - vo).max() < MIXED_UU_TOL * np.abs(vo).max()
    assert_entrywise(rm.cpu().numpy(), ro, what=name + " mixed residual")
    # removing the load restores the unloaded result
    es.set_surface_pressure(None)
    P0 = oracle.Problem(m)
    _, r0 = P0.assemble(x, rp_o, col_o, jacobian=False)
    assert_entrywise(es.residual_evaluate(xd).cpu().numpy(), r0, what=name + " unloaded")


@pytest.mark.parametrize("name", ["cfg1_lin_elem_mr", "quad_node_mr_perturbed", "lin_node_mr", "quad_elem_mr"])
def test_device_structure_calculation_bit_exact(torch, oracle, name):
    """fe_structure_calculate_device builds the same CSR pattern as the host
    set-up and as the oracle's restatement of the reference rule."""
    from cm_gb300.equations_set import structure_calculate
    m = meshes()[name]
    rp_h, col_h = structure_calculate(m, base=1)
    rp_d, col_d = structure_calculate(m, base=1, on_device=True)
    rp_o, col_o = oracle.Problem(m).pattern()
    assert np.array_equal(rp_d, rp_h) and np.array_equal(col_d, col_h)
    assert np.array_equal(rp_d, rp_o) and np.array_equal(col_d, col_o)


def test_device_structure_calculation_large(torch):
    """32^3 triquadratic box and a trilinear box: device pattern equals the
    host pattern (0-based)."""
    from cm_gb300.equations_set import structure_calculate
    for m in (M.regular_box(32, 32, 32, nxi_u=3, pressure="node"),
              M.regular_box(24, 17, 9, nxi_u=2, pressure="element")):
        rp_h, col_h = structure_calculate(m)
        rp_d, col_d = structure_calculate(m, on_device=True)
        assert np.array_equal(rp_d, rp_h) and np.array_equal(col_d, col_h)


def test_clone_shares_the_mesh_and_keeps_its_own_materials(torch):
    """fe_clone: a clone with other materials (and a surface load) gives bit
    for bit what a handle created from scratch for those materials gives,
    and keeps working after the source handle is destroyed."""
    m = meshes()["quad_node_guccione_fibres"]
    x = torch.from_numpy(state(m)).cuda()
    src = FiniteElasticityEquationsSet(m)
    mats = np.array([1.3, 12.0, 2.5, 1.1])
    cl = src.clone(mats)
    sp = np.zeros((3, m.nu))
    sp[2, m.node_ijk()[2] == 0] = 0.7
    cl.set_surface_pressure(sp)
    import copy
    m2 = copy.copy(m)
    m2.materials = mats
    fresh = FiniteElasticityEquationsSet(m2)
    fresh.set_surface_pressure(sp)
    src.close()
    for es in (cl, fresh):
        es.r = torch.empty_like(x)
    a = [t.clone() for t in cl.jacobian_evaluate_mixed(x, r=cl.r)] + [cl.r.clone()]
    b = [t.clone() for t in fresh.jacobian_evaluate_mixed(x, r=fresh.r)] + [fresh.r.clone()]
    cl.check_status(x)
    assert all(torch.equal(u, v) for u, v in zip(a, b))
    assert torch.equal(cl.jacobian_evaluate(x), fresh.jacobian_evaluate(x))
