"""Per-entry parity at the benchmark configurations' full sizes.

Every entry of the assembled Jacobian and residual of the CUDA path is
checked against the FP64 oracle at the FP64 bar
|gpu - oracle| <= 1e-12 |oracle| + f S (S = largest magnitude of the array;
f = 1e-13 for Jacobian values, 1e-12 for the residual, whose entries are
sums of hundreds of Gauss-point terms of size up to S that cancel to far
below S: over 10^5-10^6 entries the difference between the CUDA kernels'
and the oracle's rounding of those sums reaches about 2e-13 S), on

* the 32x32x32 triquadratic / trilinear-pressure Mooney-Rivlin box
  (32,768 elements, 178.7 M nonzeros): the FP64 path, and the FP64 parts
  (coupling blocks, residual) of the mixed path, whose FP32 displacement
  block is held to 1e-4 S per entry;
* the 64x64x16 Guccione slab with its through-thickness fibre field and the
  cavity pressure on the z = 0 face (65,536 elements, 357.4 M nonzeros),
  FP64 and mixed paths, with the CSR pattern compared bit for bit;
* every member of a seeded 16-mesh batch of the batched configuration
  (per-edge element counts 4..24, trilinear or triquadratic), as written by
  the one persistent launch, compared with the oracle directly.

The oracle assembles with all host threads (seconds at these sizes).
"""
import os

import numpy as np
import pytest

from cm_gb300 import FiniteElasticityEquationsSet, _lib
from cm_gb300 import mesh as M
from cm_gb300 import newton as N

pytestmark = pytest.mark.gpu

REL, FLOOR, FLOOR_RES, UU_TOL = 1e-12, 1e-13, 1e-12, 1e-4
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def torch():
    import torch as _torch
    if not _torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.load()
    return _torch


def entrywise(gpu, ref, rel, floor, what, chunk=1 << 24):
    """|gpu - ref| <= rel |ref| + floor S per entry, in chunks (arrays of
    hundreds of millions of entries)."""
    assert gpu.shape == ref.shape, what
    S = float(np.abs(ref).max())
    bad, worst = 0, 0.0
    for a in range(0, ref.size, chunk):
        g = np.asarray(gpu[a:a + chunk], dtype=np.float64)
        r = ref[a:a + chunk]
        err = np.abs(g - r)
        over = err > rel * np.abs(r) + floor * S
        bad += int(over.sum())
        worst = max(worst, float(err.max()))
    assert bad == 0, "%s: %d of %d entries off (worst |diff| %.3e, S %.3e)" % (what, bad, ref.size, worst, S)


def check_mixed(es, vu, vc, rm, vo, ro, what):
    uu_pos, cp_pos = N.mixed_positions(es)
    entrywise(vc, vo[cp_pos], REL, FLOOR, what + " mixed coupling blocks")
    entrywise(rm, ro, REL, FLOOR_RES, what + " mixed residual")
    S = float(np.abs(vo).max())
    err = float(np.abs(vu.astype(np.float64) - vo[uu_pos]).max())
    assert err <= UU_TOL * S, "%s mixed FP32 block: %.3e of the largest entry" % (what, err / S)


def test_config2_box_every_entry(torch, oracle):
    m = M.regular_box(32, 32, 32, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=2)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-2.0, seed=4)
    es = FiniteElasticityEquationsSet(m)
    assert es.nnz == 178723696
    xd = torch.from_numpy(x).cuda()
    r = torch.empty_like(xd)
    vals = es.jacobian_evaluate(xd, r=r)
    es.check_status(xd)
    vg, rg = vals.cpu().numpy(), r.cpu().numpy()
    del vals
    rp, col = es.csr_pattern(base=1)
    vo, ro = oracle.Problem(m).assemble(x, rp, col, nthreads=THREADS)
    del col
    entrywise(vg, vo, REL, FLOOR, "32^3 FP64 Jacobian")
    entrywise(rg, ro, REL, FLOOR_RES, "32^3 FP64 residual")
    del vg
    rm = torch.empty_like(xd)
    vu, vc = es.jacobian_evaluate_mixed(xd, r=rm)
    es.check_status(xd)
    check_mixed(es, vu.cpu().numpy(), vc.cpu().numpy(), rm.cpu().numpy(), vo, ro, "32^3")


def test_guccione_slab_every_entry(torch, oracle):
    m = M.guccione_slab(64, 64, 16, seed=3)
    sp = N.bottom_face_pressure(m, 2.0)
    x = M.deformed_state(m, stretch=1.03, shear=0.02, noise=0.01, pressure=-1.0, seed=6)
    P = oracle.Problem(m)
    P.set_surface_pressure(sp)
    rp_o, col_o = P.pattern()
    es = FiniteElasticityEquationsSet(m)
    es.set_surface_pressure(sp)
    assert es.nnz == 357442336
    rp, col = es.csr_pattern(base=1)
    assert np.array_equal(rp, rp_o) and np.array_equal(col, col_o)
    del col
    xd = torch.from_numpy(x).cuda()
    r = torch.empty_like(xd)
    vals = es.jacobian_evaluate(xd, r=r)
    es.check_status(xd)
    vg, rg = vals.cpu().numpy(), r.cpu().numpy()
    del vals
    vo, ro = P.assemble(x, rp_o, col_o, nthreads=THREADS)
    del col_o
    entrywise(vg, vo, REL, FLOOR, "slab FP64 Jacobian")
    entrywise(rg, ro, REL, FLOOR_RES, "slab FP64 residual")
    del vg
    rm = torch.empty_like(xd)
    vu, vc = es.jacobian_evaluate_mixed(xd, r=rm)
    es.check_status(xd)
    check_mixed(es, vu.cpu().numpy(), vc.cpu().numpy(), rm.cpu().numpy(), vo, ro, "slab")


def test_batch_members_every_entry(torch, oracle):
    from cm_gb300 import EquationsSetBatch
    meshes, stretches = M.batch_meshes(16, seed=21)
    sets = [FiniteElasticityEquationsSet(m) for m in meshes]
    xs_h = [M.deformed_state(m, stretch=s, shear=0.02, noise=0.02, pressure=-1.0, seed=i)
            for i, (m, s) in enumerate(zip(meshes, stretches))]
    xs = [torch.from_numpy(x).cuda() for x in xs_h]
    b = EquationsSetBatch(sets)
    b.set_config(0, 2, 1)  # the persistent launch (not the per-member variant)
    vus, vcs, rs = b.allocate(xs[0].device)
    b.jacobian_evaluate_mixed(xs, vus, vcs, rs)
    b.check(xs[0])
    for i, (m, es, x) in enumerate(zip(meshes, sets, xs_h)):
        rp, col = es.csr_pattern(base=1)
        vo, ro = oracle.Problem(m).assemble(x, rp, col, nthreads=THREADS)
        check_mixed(es, vus[i].cpu().numpy(), vcs[i].cpu().numpy(), rs[i].cpu().numpy(), vo, ro,
                    "batch member %d (%d elements)" % (i, m.ne))
    b.close()
