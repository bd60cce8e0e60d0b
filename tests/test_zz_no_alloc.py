"""fe_residual_evaluate_noalloc: the allocation-free residual entry point.

Collected last (file name) so that it also runs after every other GPU test.
It must give the same residual as fe_residual_evaluate bit for bit (the same
kernels run in the same colour order, and the colour order fixes every sum)
on two calls in a row, leave the device's free memory unchanged from before
its first call (the handle's creation commits the static array), and reject
a problem above FE_NOALLOC_MAX_DOFS with an error instead of running.
"""
import numpy as np
import pytest

from cm_gb300 import FEError, FiniteElasticityEquationsSet, _lib
from cm_gb300 import mesh as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as _torch
    if not _torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.load()
    return _torch


@pytest.mark.parametrize("host", [True, False])
def test_noalloc_matches_residual_evaluate_twice(torch, host):
    m = M.regular_box(3, 3, 2, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=8)
    x = M.deformed_state(m, stretch=1.08, shear=0.04, noise=0.03, pressure=-1.5, seed=9)
    es = FiniteElasticityEquationsSet(m)
    ref = es.residual_evaluate(x)
    xin = x if host else torch.from_numpy(x).cuda()
    bufs = [np.zeros(es.ndofs) if host else torch.empty_like(xin) for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for out in bufs:
        es.residual_evaluate_noalloc(xin, out)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    outs = [b if host else b.cpu().numpy() for b in bufs]
    for o in outs:
        assert np.array_equal(o, ref)


def test_noalloc_rejects_too_many_dofs(torch):
    m = M.regular_box(35, 35, 35, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0))
    assert m.ndofs > _lib.FE_NOALLOC_MAX_DOFS
    es = FiniteElasticityEquationsSet(m)
    x = np.concatenate([m.X.ravel(), np.zeros(m.n_pressure)])
    with pytest.raises(FEError, match="FE_NOALLOC_MAX_DOFS"):
        es.residual_evaluate_noalloc(x)
