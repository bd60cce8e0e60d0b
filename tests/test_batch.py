"""Batched assembly: many equations sets in one persistent launch.

Every launch configuration the autotuner can choose, and the captured CUDA
graph, must agree with one single-set mixed evaluation per member: the FP64
residual and coupling blocks to 1e-12 of the array's largest entry, the FP32
displacement block to 1e-5 of its largest entry (the batched kernel is a
separate compilation of the same device code, so the compiler may fuse a
few multiply-adds differently).  Repeated launches of one configuration must
be bit-identical (colour order fixes the order of every CSR slot's sum).
"""
import numpy as np
import pytest

from cm_gb300 import mesh as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as _torch
    if not _torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cm_gb300 import _lib
    _lib.load()
    return _torch


def members():
    out = [
        M.regular_box(3, 2, 2, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=1),
        M.regular_box(4, 3, 2, nxi_u=2, pressure="element", law=M.MR, materials=(1.0, 3.0), perturb=0.1, seed=2),
        M.regular_box(2, 2, 3, nxi_u=3, pressure="element", law=M.MR, materials=(0.7, 5.0)),
        M.regular_box(3, 3, 3, nxi_u=2, pressure="node", law=M.MR, materials=(4.0, 1.0), perturb=0.05, seed=3),
        M.regular_box(2, 3, 2, lengths=(2.0, 1.0, 0.5), nxi_u=3, pressure="node", law=M.GUCCIONE,
                      materials=(0.88, 18.5, 3.58, 1.63), fibre=np.array([[0.3], [0.1], [-0.2]])),
    ]
    meshes, _ = M.batch_meshes(6, seed=5, edge_range=(1, 5))
    return out + meshes


def _setup(torch):
    from cm_gb300 import EquationsSetBatch, FiniteElasticityEquationsSet
    ms = members()
    sets = [FiniteElasticityEquationsSet(m) for m in ms]
    xs = [torch.from_numpy(M.deformed_state(m, stretch=1.05 + 0.01 * i, shear=0.03, noise=0.02, seed=i)).cuda()
          for i, m in enumerate(ms)]
    refs = []
    for s, x in zip(sets, xs):
        r = torch.empty_like(x)
        vu, vc = s.jacobian_evaluate_mixed(x, r=r)
        s.check_status(x)
        refs.append((vu.clone(), vc.clone(), r.clone()))
    return sets, xs, refs, EquationsSetBatch(sets)


def _close(torch, refs, vus, vcs, rs):
    for i, ((a, b, c), u, v, w) in enumerate(zip(refs, vus, vcs, rs)):
        for ref, got, tol in ((a, u, 1e-5), (b, v, 1e-12), (c, w, 1e-12)):
            assert not torch.isnan(got).any(), "member %d: entries not written" % i
            err = float((got.double() - ref.double()).abs().max())
            assert err <= tol * float(ref.double().abs().max()), "member %d: %.3e" % (i, err)


def test_batch_matches_single_set_bitwise(torch):
    sets, xs, refs, batch = _setup(torch)
    vus, vcs, rs = batch.allocate("cuda")
    for variant in range(5):
        for cps in (1, 2):
            for bg in (1, 3):
                batch.set_config(variant, cps, bg)
                for t in vus + vcs + rs:
                    t.fill_(float("nan"))
                batch.jacobian_evaluate_mixed(xs, vus, vcs, rs)
                batch.check(xs[0])
                _close(torch, refs, vus, vcs, rs)
                first = [t.clone() for t in vus + vcs + rs]
                batch.jacobian_evaluate_mixed(xs, vus, vcs, rs)
                batch.check(xs[0])
                assert all(torch.equal(a, b) for a, b in zip(first, vus + vcs + rs))
    assert batch.launch_count() == 40


def test_autotune_and_graph_replay(torch):
    sets, xs, refs, batch = _setup(torch)
    vus, vcs, rs = batch.allocate("cuda")
    cfg = batch.autotune(xs, vus, vcs, rs, repeats=2)
    assert 0 <= cfg["variant"] <= 5 and cfg["tuned_ms"] > 0
    batch.capture(xs, vus, vcs, rs)
    for t in vus + vcs + rs:
        t.zero_()
    batch.replay(xs[0])
    batch.check(xs[0])
    _close(torch, refs, vus, vcs, rs)
    # new inputs in the same buffers: the replay sees them
    xs[0].mul_(1.01)
    r = torch.empty_like(xs[0])
    vu0, vc0 = sets[0].jacobian_evaluate_mixed(xs[0], r=r)
    batch.replay(xs[0])
    batch.check(xs[0])
    _close(torch, [(vu0, vc0, r)], vus[:1], vcs[:1], rs[:1])


def test_batch_rejects_host_pointers(torch):
    from cm_gb300 import FEError
    sets, xs, refs, batch = _setup(torch)
    vus, vcs, rs = batch.allocate("cuda")
    xs_host = [x.cpu() for x in xs]
    with pytest.raises(FEError):
        batch.jacobian_evaluate_mixed(xs_host, vus, vcs, rs)


def test_batch_with_surface_pressure(torch):
    """Members carrying a follower surface-pressure load (and members without
    one) in one batch: agrees with the single-set mixed evaluation, which
    applies each colour's boundary faces after its volume work."""
    from cm_gb300 import EquationsSetBatch, FiniteElasticityEquationsSet
    ms = [M.guccione_slab(3, 3, 2, lengths=(4.0, 4.0, 1.0), seed=3),
          M.regular_box(3, 2, 2, nxi_u=2, pressure="element", law=M.MR, materials=(2.0, 6.0), perturb=0.05, seed=4),
          M.regular_box(2, 2, 2, nxi_u=3, pressure="node", law=M.MR, materials=(1.0, 4.0))]
    sets = [FiniteElasticityEquationsSet(m) for m in ms]
    for m, s in zip(ms[:2], sets[:2]):
        sp = np.zeros((3, m.nu))
        i, j, k = m.node_ijk()
        sp[2, k == 0] = 1.5
        sp[0, i == i.max()] = -0.3
        s.set_surface_pressure(sp)
    xs = [torch.from_numpy(M.deformed_state(m, stretch=1.04, shear=0.02, noise=0.02, seed=i + 7)).cuda()
          for i, m in enumerate(ms)]
    refs = []
    for s, x in zip(sets, xs):
        r = torch.empty_like(x)
        vu, vc = s.jacobian_evaluate_mixed(x, r=r)
        s.check_status(x)
        refs.append((vu.clone(), vc.clone(), r.clone()))
    batch = EquationsSetBatch(sets)
    vus, vcs, rs = batch.allocate("cuda")
    for variant in (1, 4):
        batch.set_config(variant, 2, 1)
        batch.jacobian_evaluate_mixed(xs, vus, vcs, rs)
        batch.check(xs[0])
        _close(torch, refs, vus, vcs, rs)
    # removing the load from a member is seen by the next batched call
    sets[0].set_surface_pressure(None)
    r0 = torch.empty_like(xs[0])
    vu0, vc0 = sets[0].jacobian_evaluate_mixed(xs[0], r=r0)
    batch.jacobian_evaluate_mixed(xs, vus, vcs, rs)
    batch.check(xs[0])
    _close(torch, [(vu0, vc0, r0)], vus[:1], vcs[:1], rs[:1])


@pytest.mark.parametrize("nxi_u,pressure", [(2, "element"), (2, "node"), (3, "element"), (3, "node")])
def test_single_type_batches(torch, nxi_u, pressure):
    """Batches whose members all have one element type run the kernel
    compiled for that type alone: every launch variant agrees with the
    single-set evaluation, with and without surface loads."""
    from cm_gb300 import EquationsSetBatch, FiniteElasticityEquationsSet
    ms = [M.regular_box(3, 2, 2, nxi_u=nxi_u, pressure=pressure, law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=1),
          M.regular_box(2, 2, 3, nxi_u=nxi_u, pressure=pressure, law=M.MR, materials=(0.7, 5.0)),
          M.regular_box(2, 3, 2, lengths=(2.0, 1.0, 0.5), nxi_u=nxi_u, pressure=pressure, law=M.GUCCIONE,
                        materials=(0.88, 18.5, 3.58, 1.63), fibre=np.array([[0.3], [0.1], [-0.2]]))]
    sets = [FiniteElasticityEquationsSet(m) for m in ms]
    sp = np.zeros((3, ms[2].nu))
    sp[2, ms[2].node_ijk()[2] == 0] = 0.8
    sets[2].set_surface_pressure(sp)
    xs = [torch.from_numpy(M.deformed_state(m, stretch=1.03, shear=0.02, noise=0.02, seed=i + 3)).cuda()
          for i, m in enumerate(ms)]
    refs = []
    for s, x in zip(sets, xs):
        r = torch.empty_like(x)
        vu, vc = s.jacobian_evaluate_mixed(x, r=r)
        s.check_status(x)
        refs.append((vu.clone(), vc.clone(), r.clone()))
    batch = EquationsSetBatch(sets)
    vus, vcs, rs = batch.allocate("cuda")
    for variant in range(6):
        for cps in (1, 3):
            batch.set_config(variant, cps, 2)
            for t in vus + vcs + rs:
                t.fill_(float("nan"))
            batch.jacobian_evaluate_mixed(xs, vus, vcs, rs)
            batch.check(xs[0])
            _close(torch, refs, vus, vcs, rs)


def test_batch_member_limit(torch):
    from cm_gb300 import EquationsSetBatch, FEError, FiniteElasticityEquationsSet
    es = FiniteElasticityEquationsSet(M.regular_box(1, 1, 1, nxi_u=2, pressure="element", law=M.MR,
                                                    materials=(2.0, 6.0)))
    EquationsSetBatch([es] * 256).close()
    with pytest.raises(FEError):
        EquationsSetBatch([es] * 257)


def test_per_member_variant_is_the_single_set_path(torch):
    """Variant 5 launches the single-set kernels member by member: bit-identical
    to one fe_jacobian_evaluate_mixed call per member (at least one launch per
    member), also from a captured graph."""
    sets, xs, refs, batch = _setup(torch)
    vus, vcs, rs = batch.allocate("cuda")
    batch.set_config(5, 1, 1)
    l0 = batch.launch_count()
    m0 = [s.launch_count() for s in sets]
    batch.jacobian_evaluate_mixed(xs, vus, vcs, rs)
    batch.check(xs[0])
    for (a, b, c), u, v, w in zip(refs, vus, vcs, rs):
        assert torch.equal(a, u) and torch.equal(b, v) and torch.equal(c, w)
    assert batch.launch_count() - l0 == sum(s.launch_count() - c for s, c in zip(sets, m0)) >= len(sets)
    batch.capture(xs, vus, vcs, rs)
    for t in vus + vcs + rs:
        t.zero_()
    batch.replay(xs[0])
    batch.check(xs[0])
    for (a, b, c), u, v, w in zip(refs, vus, vcs, rs):
        assert torch.equal(a, u) and torch.equal(b, v) and torch.equal(c, w)


def test_grid_barrier_gives_up_and_reports(torch):
    """The bounded grid-barrier wait of the persistent launch: with one
    arrival more than the grid can give, every barrier gives up after 16
    polls, the kernel still returns, and fe_batch_check reports the failure
    instead of the launch hanging; after restoring the default limits the
    same batch gives its normal, checked result again."""
    from cm_gb300 import FEError
    sets, xs, refs, b = _setup(torch)
    b.set_config(0, 1, 1)  # a persistent variant (not the per-member launches)
    vus, vcs, rs = b.allocate(xs[0].device)
    b.set_barrier_limits(16, 1)
    b.jacobian_evaluate_mixed(xs, vus, vcs, rs)
    with pytest.raises(FEError, match="grid barrier gave up"):
        b.check(xs[0])
    b.set_barrier_limits(0, 0)
    for t in vus + vcs + rs:
        t.fill_(float("nan"))
    b.jacobian_evaluate_mixed(xs, vus, vcs, rs)
    b.check(xs[0])
    _close(torch, refs, vus, vcs, rs)
    with pytest.raises(FEError):
        b.set_barrier_limits(0, 1)  # an unreachable barrier needs a small poll limit


def test_concurrent_creation_matches_serial(torch):
    """create_equations_sets builds the members' set-ups on several host
    threads: the same patterns and the same assembled values as handles
    created one after another."""
    from cm_gb300 import FiniteElasticityEquationsSet, create_equations_sets
    ms = members()
    par = create_equations_sets(ms, threads=8)
    for m, es in zip(ms, par):
        ref = FiniteElasticityEquationsSet(m)
        a, b = ref.csr_pattern(), es.csr_pattern()
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        x = torch.from_numpy(M.deformed_state(m, stretch=1.04, shear=0.02, noise=0.02, seed=3)).cuda()
        ua, ca = ref.jacobian_evaluate_mixed(x)
        ub, cb = es.jacobian_evaluate_mixed(x)
        assert torch.equal(ua, ub) and torch.equal(ca, cb)
