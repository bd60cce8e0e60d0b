"""Learned warm start: the MLP kernels against the FP64 numpy oracle, the POD,
and the gain of the trained network over Newton from the reference guess.

Tolerances: FP32 kernels vs the FP64 oracle at 2e-5 relative to the largest
entry of each array (FP32 rounding over sums of at most 256 terms of
O(1) size); BF16 inference at 2e-2 (8-bit mantissa weights and activations
with FP32 accumulation).
"""
import warnings

import numpy as np
import pytest
import torch

from cm_gb300 import mesh as M
from cm_gb300 import newton as N
from cm_gb300 import warmstart as W

warnings.filterwarnings("ignore", message="Sparse")


def test_oracle_mlp_backward_matches_finite_differences():
    import mlp_oracle as O
    rng = np.random.default_rng(0)
    widths = [4, 7, 5, 3]
    params = [(rng.normal(size=(o, i)) * 0.5, rng.normal(size=o) * 0.1) for i, o in zip(widths[:-1], widths[1:])]
    x = rng.normal(size=(6, 4))
    t = rng.normal(size=(6, 3))

    def loss(ps):
        return O.mse(O.forward(ps, x)[-1], t)[0]

    hs = O.forward(params, x)
    _, dy = O.mse(hs[-1], t)
    grads = O.backward(params, hs, dy)
    h = 1e-6
    for l, (Wl, bl) in enumerate(params):
        for arr, g in ((Wl, grads[l][0]), (bl, grads[l][1])):
            it = np.nditer(arr, flags=["multi_index"])
            for _ in it:
                idx = it.multi_index
                old = arr[idx]
                arr[idx] = old + h
                fp = loss(params)
                arr[idx] = old - h
                fm = loss(params)
                arr[idx] = old
                assert abs((fp - fm) / (2 * h) - g[idx]) < 1e-8


def test_pod_reconstructs_its_span():
    g = torch.Generator().manual_seed(0)
    basis = torch.randn(200, 5, generator=g, dtype=torch.float64)
    coef = torch.randn(30, 5, generator=g, dtype=torch.float64)
    S = coef @ basis.T + 0.3
    pod = W.POD().fit(S, 5)
    assert abs(pod.energy - 1.0) < 1e-12
    rec = pod.reconstruct(pod.coefficients(S))
    assert float((rec - S).abs().max()) < 1e-10
    Q = pod.modes.T @ pod.modes
    assert float((Q - torch.eye(5, dtype=torch.float64)).abs().max()) < 1e-10


def test_parameter_sampling_is_seeded_and_in_range():
    a = W.sample_parameters(500, 3)
    b = W.sample_parameters(500, 3)
    assert np.array_equal(a, b)
    assert a[:, 0].min() >= 1.0 and a[:, 0].max() <= 1.3
    assert a[:, 1].min() >= 0.0 and a[:, 1].max() <= 0.2
    assert a[:, 2:].min() >= 0.5 and a[:, 2:].max() <= 10.0


# ------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cm_gb300 import _lib
    _lib.load()
    return torch.device("cuda")


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.mark.gpu
def test_mlp_forward_backward_adam_match_oracle(cuda):
    import mlp_oracle as O
    net = W.MLP((4, 48, 40, 24), seed=5, device=cuda)
    rng = np.random.default_rng(1)
    x = rng.normal(size=(70, 4)).astype(np.float32)
    t = rng.normal(size=(70, 24)).astype(np.float32)
    params = [(net.W(l).cpu().numpy().astype(np.float64), net.b(l).cpu().numpy().astype(np.float64))
              for l in range(net.layers)]
    hs_o = O.forward(params, x.astype(np.float64))
    loss_o, dy_o = O.mse(hs_o[-1], t.astype(np.float64))
    grads_o = O.backward(params, hs_o, dy_o)
    loss = net.loss_and_grad(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
    hs = net.forward(torch.from_numpy(x).cuda())
    for a, b in zip(hs[1:], hs_o[1:]):
        assert _rel(a.cpu().numpy(), b) < 2e-5
    assert abs(float(loss) - loss_o) < 2e-5 * loss_o
    for l in range(net.layers):
        assert _rel(net.W(l, net.grad).cpu().numpy(), grads_o[l][0]) < 2e-5
        assert _rel(net.b(l, net.grad).cpu().numpy(), grads_o[l][1]) < 2e-5
    # one Adam step
    flat0 = net.flat.cpu().numpy().astype(np.float64)
    g0 = net.grad.cpu().numpy().astype(np.float64)
    net.adam_step(1e-3)
    p1, _, _ = O.adam(flat0, g0, np.zeros_like(flat0), np.zeros_like(flat0), 1, 1e-3)
    assert np.abs(net.flat.cpu().numpy() - p1).max() < 1e-6


@pytest.mark.gpu
def test_bf16_tensor_core_inference_matches_fp32(cuda):
    import mlp_oracle as O
    net = W.MLP((4, 256, 256, 256, 64), seed=2, device=cuda)
    x = torch.from_numpy(np.random.default_rng(4).normal(size=(37, 4)).astype(np.float32)).cuda()
    y = net.infer_bf16(x).cpu().numpy()
    params = [(net.W(l).cpu().numpy().astype(np.float64), net.b(l).cpu().numpy().astype(np.float64))
              for l in range(net.layers)]
    ref = O.forward(params, x.cpu().numpy().astype(np.float64))[-1]
    assert y.shape == ref.shape
    assert _rel(y, ref) < 2e-2


@pytest.mark.gpu
def test_mlp_training_reduces_loss(cuda):
    g = torch.Generator().manual_seed(0)
    x = torch.rand(512, 4, generator=g) * 2 - 1
    y = torch.stack([torch.sin(2 * x[:, 0]) * x[:, 1], x[:, 2] ** 2 - x[:, 3], x.sum(1)], 1)
    net = W.MLP((4, 64, 64, 3), seed=0, device=cuda)
    hs = net.forward(x.cuda())
    l0 = float(((hs[-1].cpu() - y) ** 2).mean())
    l1 = net.fit(x.cuda(), y.cuda(), steps=800, lr=3e-3, batch=128)
    assert l1 < 0.02 * l0


@pytest.mark.gpu
def test_learned_warm_start_beats_reference_guess(cuda):
    """Train on plain-method solves of a 3x3x3 triquadratic box over
    (stretch, shear, c1, c2); on held-out parameters, Newton from the
    network's prediction (one full-load increment, mixed-precision Jacobian)
    reaches ||r||_2 <= 1e-10 with fewer iterations than the plain method
    (FP64 Jacobian, reference guess, load increments)."""
    from cm_gb300 import FiniteElasticityEquationsSet
    m = M.regular_box(3, 3, 3, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=3)
    es = FiniteElasticityEquationsSet(m)
    plain = W.ParametricProblem(es, N.NewtonOptions(linear="dense"), device=cuda)
    fast = W.ParametricProblem(es, N.NewtonOptions(linear="dense", precision="mixed"), device=cuda)
    incs = 4
    train = W.sample_parameters(160, seed=11)
    test = W.sample_parameters(12, seed=12)
    states, _ = W.generate_solves(plain, train, incs)
    ws = W.LearnedWarmStart(plain.n_pressure, modes=32, hidden=(128, 128, 128), seed=0, device=cuda)
    rep = ws.fit(train, states, steps=1500, lr=2e-3, batch=128)
    assert rep.modes == 32 and rep.energy > 0.999
    guess = ws.predict(test)
    it_plain, it_learned, accepted = [], [], 0
    for p, gs in zip(test, guess):
        xr, rr, _ = plain.solve_reference(p, incs)
        xl, rl, _, ok = fast.solve_from_state(p, gs, incs)
        assert all(r.converged for r in rr) and rl[-1].converged
        assert rl[-1].residual_norms[-1] <= 1e-10
        assert float((xl - xr).abs().max()) < 1e-8
        it_plain.append(sum(r.iterations for r in rr))
        it_learned.append(sum(r.iterations for r in rl))
        accepted += ok
    assert accepted == len(test)
    assert np.mean(it_learned) < 0.6 * np.mean(it_plain)


def test_slab_problem_from_converged_state(oracle):
    """SlabProblem on the oracle: the reference path converges, and starting
    from its converged state the full-load Newton needs no iteration."""
    m = M.guccione_slab(3, 3, 2, lengths=(4.0, 4.0, 1.0), seed=3)
    es = oracle.EquationsSet(m)
    pb = W.SlabProblem(es, N.NewtonOptions(linear="dense"), device="cpu")
    p = W.sample_slab_parameters(1, seed=4)[0]
    x, reps, _ = pb.solve_reference(p, 4)
    assert all(r.converged for r in reps)
    x2, reps2, _, ok = pb.solve_from_state(p, pb.state(x), 4)
    assert ok and reps2[0].iterations == 0
    assert float((x2 - x).abs().max()) == 0.0
    f = W.slab_features(W.sample_slab_parameters(5, seed=1))
    assert f.shape == (5, 2)


@pytest.mark.gpu
def test_learned_warm_start_on_the_slab(cuda):
    """Guccione slab over (cavity pressure, C): trained on plain-method solves,
    Newton from the prediction at the full pressure needs fewer iterations
    than the pressure-increment path, at the same ||r||_2 <= 1e-10."""
    from cm_gb300 import FiniteElasticityEquationsSet
    m = M.guccione_slab(3, 3, 2, lengths=(4.0, 4.0, 1.0), seed=3)
    es = FiniteElasticityEquationsSet(m)
    plain = W.SlabProblem(es, N.NewtonOptions(linear="dense"), device=cuda)
    fast = W.SlabProblem(es, N.NewtonOptions(linear="dense", precision="mixed"), device=cuda)
    train = W.sample_slab_parameters(64, seed=31)
    test = W.sample_slab_parameters(6, seed=32)
    states, _ = W.generate_solves(plain, train, 4)
    ws = W.LearnedWarmStart(plain.n_pressure, modes=24, hidden=(128, 128, 128), seed=0, device=cuda,
                            featurize=W.slab_features)
    ws.fit(train, states, steps=1500, lr=2e-3, batch=64)
    guess = ws.predict(test)
    it_plain, it_learned = [], []
    for p, g in zip(test, guess):
        xr, rr, _ = plain.solve_reference(p, 4)
        xl, rl, _, ok = fast.solve_from_state(p, g, 4)
        assert ok and rl[-1].converged and rl[-1].residual_norms[-1] <= 1e-10
        assert float((xl - xr).abs().max()) < 1e-8
        it_plain.append(sum(r.iterations for r in rr))
        it_learned.append(sum(r.iterations for r in rl))
    assert np.mean(it_learned) < 0.6 * np.mean(it_plain)
