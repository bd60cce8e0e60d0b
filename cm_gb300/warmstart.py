"""Learned Newton warm start: POD of converged fields + an MLP trained on the GPU.

The reference starts every Newton solve from the current field
(SOLUTION_INITIALISE_CURRENT_FIELD, solver_routines.f90:17812) and reaches
the full load through load increments (equations_set_routines.f90:6560-6595).
Here a small network maps the load and material parameters
(stretch, shear, log c1, log c2) to the coefficients of a proper orthogonal
decomposition (POD) of converged solutions, and the field it predicts is the
Newton initial guess of a single full-load increment.  Newton from the
reference guess stays the fallback: a warm-started solve that does not reach
the tolerance is redone the reference way, so every accepted solution meets
the same ||r||_2 <= atol.

The network (default 4 -> 256 -> 256 -> 256 -> 64, tanh) is trained in FP32
by the hand-written kernels of include/cm_warmstart.h (GEMM, bias+tanh,
tanh backward, column sums, MSE, Adam) and evaluated with BF16 weights on the
tensor cores in one launch (ws_mlp_forward_bf16).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import WS_ACT_IDENTITY, WS_ACT_TANH, check


def _p(t):
    return C.c_void_p(t.data_ptr())


def _s(t):
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


class MLP:
    """Fully connected tanh network with a linear output layer; all parameters
    in one flat FP32 device buffer (so one Adam launch updates them all)."""

    def __init__(self, widths=(4, 256, 256, 256, 64), seed=0, device="cuda"):
        self.widths = tuple(int(w) for w in widths)
        self.device = torch.device(device)
        self.L = _lib.load()
        sizes = []
        for i, o in zip(self.widths[:-1], self.widths[1:]):
            sizes += [o * i, o]
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.flat = torch.zeros(int(self.offsets[-1]), dtype=torch.float32, device=self.device)
        self.grad = torch.zeros_like(self.flat)
        self.m = torch.zeros_like(self.flat)
        self.v = torch.zeros_like(self.flat)
        self.step = 0
        g = torch.Generator().manual_seed(seed)
        for l, (i, o) in enumerate(zip(self.widths[:-1], self.widths[1:])):
            bound = math.sqrt(6.0 / (i + o))  # Glorot uniform
            self.W(l).copy_((torch.rand(o, i, generator=g, dtype=torch.float32) * 2 - 1) * bound)
        self._bf16 = None

    @property
    def layers(self):
        return len(self.widths) - 1

    def _view(self, buf, k, shape):
        a, b = int(self.offsets[k]), int(self.offsets[k + 1])
        return buf[a:b].view(*shape)

    def W(self, l, buf=None):
        return self._view(self.flat if buf is None else buf, 2 * l, (self.widths[l + 1], self.widths[l]))

    def b(self, l, buf=None):
        return self._view(self.flat if buf is None else buf, 2 * l + 1, (self.widths[l + 1],))

    # ------------------------------------------------------------- training
    def forward(self, x):
        """FP32 forward; returns every layer output (h_0 = x .. h_L)."""
        hs = [x.contiguous()]
        n = x.shape[0]
        for l in range(self.layers):
            i, o = self.widths[l], self.widths[l + 1]
            h = torch.empty(n, o, dtype=torch.float32, device=self.device)
            W = self.W(l)
            check(self.L.ws_gemm_f32(n, o, i, _p(hs[-1]), i, 1, _p(W), 1, i, _p(h), o, 0.0, _s(h)))
            act = WS_ACT_TANH if l + 1 < self.layers else WS_ACT_IDENTITY
            check(self.L.ws_bias_act(_p(h), _p(self.b(l)), n, o, act, _s(h)))
            hs.append(h)
        return hs

    def backward(self, hs, dy):
        """Fills self.grad from the output gradient dy."""
        n = dy.shape[0]
        dh = dy.contiguous()
        for l in range(self.layers - 1, -1, -1):
            i, o = self.widths[l], self.widths[l + 1]
            act = WS_ACT_TANH if l + 1 < self.layers else WS_ACT_IDENTITY
            dz = torch.empty_like(dh)
            check(self.L.ws_act_backward(_p(hs[l + 1]), _p(dh), _p(dz), dz.numel(), act, _s(dz)))
            gW, gb = self.W(l, self.grad), self.b(l, self.grad)
            check(self.L.ws_gemm_f32(o, i, n, _p(dz), 1, o, _p(hs[l]), i, 1, _p(gW), i, 0.0, _s(dz)))
            check(self.L.ws_column_sum(_p(dz), _p(gb), n, o, _s(dz)))
            if l > 0:
                dprev = torch.empty(n, i, dtype=torch.float32, device=self.device)
                check(self.L.ws_gemm_f32(n, i, o, _p(dz), o, 1, _p(self.W(l)), i, 1, _p(dprev), i, 0.0, _s(dz)))
                dh = dprev

    def loss_and_grad(self, x, y):
        hs = self.forward(x)
        dy = torch.empty_like(hs[-1])
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        check(self.L.ws_mse(_p(hs[-1]), _p(y.contiguous()), _p(dy), _p(loss), dy.numel(), _s(dy)))
        self.backward(hs, dy)
        return loss

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        check(self.L.ws_adam(_p(self.flat), _p(self.grad), _p(self.m), _p(self.v), self.flat.numel(), lr, beta1,
                             beta2, eps, self.step, _s(self.flat)))
        self._bf16 = None

    def fit(self, x, y, steps=3000, lr=2e-3, batch=256, seed=0, lr_final=1e-5):
        """Adam on minibatches with a cosine learning-rate schedule; returns
        the final full-batch training loss."""
        g = torch.Generator(device="cpu").manual_seed(seed)
        n = x.shape[0]
        for s in range(steps):
            idx = torch.randint(0, n, (min(batch, n),), generator=g).to(self.device)
            lr_s = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * s / steps))
            self.loss_and_grad(x[idx], y[idx])
            self.adam_step(lr_s)
        hs = self.forward(x)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        check(self.L.ws_mse(_p(hs[-1]), _p(y.contiguous()), None, _p(loss), hs[-1].numel(), _s(loss)))
        return float(loss)

    # ------------------------------------------------------------ inference
    def _prepare_bf16(self):
        """BF16 weights, the input width padded to a multiple of 16."""
        ws, bs = [], []
        widths = [((w + 15) // 16) * 16 for w in self.widths]
        for l in range(self.layers):
            W = self.W(l)
            Wp = torch.zeros(widths[l + 1], widths[l], dtype=torch.float32, device=self.device)
            Wp[:W.shape[0], :W.shape[1]] = W
            Wb = torch.empty(Wp.shape, dtype=torch.int16, device=self.device)
            check(self.L.ws_to_bf16(_p(Wp), _p(Wb), Wp.numel(), _s(Wp)))
            bp = torch.zeros(widths[l + 1], dtype=torch.float32, device=self.device)
            bp[:self.widths[l + 1]] = self.b(l)
            ws.append(Wb)
            bs.append(bp)
        self._bf16 = (widths, ws, bs)

    def infer_bf16(self, x):
        if self._bf16 is None:
            self._prepare_bf16()
        widths, ws, bs = self._bf16
        n = x.shape[0]
        xp = torch.zeros(n, widths[0], dtype=torch.float32, device=self.device)
        xp[:, :x.shape[1]] = x
        y = torch.empty(n, widths[-1], dtype=torch.float32, device=self.device)
        W = (C.c_int32 * len(widths))(*widths)
        Wp = (C.c_void_p * self.layers)(*[w.data_ptr() for w in ws])
        Bp = (C.c_void_p * self.layers)(*[b.data_ptr() for b in bs])
        check(self.L.ws_mlp_forward_bf16(n, self.layers, W, Wp, Bp, _p(xp), _p(y), WS_ACT_TANH, _s(y)))
        return y[:, :self.widths[-1]]


class POD:
    """Proper orthogonal decomposition of snapshot rows (method of snapshots:
    eigenvectors of the Gram matrix)."""

    def fit(self, S, r):
        S = S.to(torch.float64)
        self.mean = S.mean(0)
        D = S - self.mean
        G = D @ D.T
        lam, V = torch.linalg.eigh(G)
        lam, V = lam.flip(0)[:r], V.flip(1)[:, :r]
        lam = torch.clamp(lam, min=1e-300)
        self.sigma = torch.sqrt(lam)                  # singular values
        self.modes = (D.T @ V) / self.sigma           # (n_dof, r), orthonormal columns
        self.energy = float(lam.sum() / torch.clamp(torch.trace(G), min=1e-300))
        return self

    def coefficients(self, S):
        return (S.to(torch.float64) - self.mean) @ self.modes

    def reconstruct(self, c):
        return self.mean + c.to(torch.float64) @ self.modes.T


def features(params):
    """(stretch, shear, c1, c2) -> (stretch, shear, log c1, log c2)."""
    p = np.asarray(params, dtype=np.float64)
    return np.stack([p[:, 0], p[:, 1], np.log(p[:, 2]), np.log(p[:, 3])], axis=1)


@dataclass
class TrainReport:
    samples: int
    modes: int
    energy: float
    train_loss: float
    seconds: float
    pod_relative_error: float


class LearnedWarmStart:
    """Maps (stretch, shear, c1, c2) to the free-dof state [z - X; p]."""

    def __init__(self, n_pressure, modes=64, hidden=(256, 256, 256), seed=0, device="cuda", featurize=None):
        self.n_p = int(n_pressure)   # trailing pressure entries of a state
        self.featurize = featurize or features  # parameters -> network inputs
        self.r = modes
        self.hidden = hidden
        self.seed = seed
        self.device = torch.device(device)

    def fit(self, params, states, steps=3000, lr=2e-3, batch=256):
        """params: (n, 4) host array; states: (n, n_free) device tensor of
        converged free-dof states (displacement z - X and pressure)."""
        t0 = time.perf_counter()
        states = states.to(self.device, torch.float64)
        nu_part = states.shape[1] - self.n_p
        # balance displacement and pressure magnitudes before the decomposition
        su = float(states[:, :nu_part].std()) or 1.0
        sp = float(states[:, nu_part:].std()) if nu_part < states.shape[1] else 1.0
        self.scale = torch.ones(states.shape[1], dtype=torch.float64, device=self.device)
        if nu_part < states.shape[1] and sp > 0:
            self.scale[nu_part:] = sp / su
        S = states / self.scale
        r = min(self.r, S.shape[0] - 1)
        self.pod = POD().fit(S, r)
        coef = self.pod.coefficients(S)
        rec = self.pod.reconstruct(coef) * self.scale
        pod_err = float(((rec - states).norm(dim=1) / states.norm(dim=1).clamp(min=1e-300)).max())
        f = self.featurize(params)
        self.f_mean, self.f_std = f.mean(0), f.std(0) + 1e-12
        x = torch.from_numpy((f - self.f_mean) / self.f_std).to(self.device, torch.float32)
        self.c_std = coef.std(0).clamp(min=1e-300)
        y = (coef / self.c_std).to(torch.float32)
        self.net = MLP((f.shape[1],) + tuple(self.hidden) + (r,), seed=self.seed, device=self.device)
        loss = self.net.fit(x, y, steps=steps, lr=lr, batch=batch, seed=self.seed)
        torch.cuda.synchronize(self.device)
        return TrainReport(samples=S.shape[0], modes=r, energy=self.pod.energy, train_loss=loss,
                           seconds=time.perf_counter() - t0, pod_relative_error=pod_err)

    def predict(self, params, bf16=True):
        f = self.featurize(params)
        x = torch.from_numpy((f - self.f_mean) / self.f_std).to(self.device, torch.float32)
        y = self.net.infer_bf16(x) if bf16 else self.net.forward(x)[-1]
        coef = y.to(torch.float64) * self.c_std
        return self.pod.reconstruct(coef) * self.scale


class ParametricProblem:
    """The clamped stretch/shear box problem over (stretch, shear, c1, c2):
    one equations set and one load-stepping solver reused for every sample
    (materials and Dirichlet values change, the dof sets do not)."""

    def __init__(self, es, options, device="cuda"):
        from . import newton as N
        self.N = N
        self.es = es
        self.mesh = es.mesh
        self.device = torch.device(device)
        self.solver = N.LoadStepSolver(es, N.clamped_stretch_shear_conditions(self.mesh, 1.0, 0.0), options,
                                       device=self.device)
        self.x_init = torch.from_numpy(N.initial_state(self.mesh)).to(self.device)
        self.free = self.solver.sys.free
        self.n_pressure = self.solver.sys.nfp

    def set_parameters(self, p):
        lam, gam, c1, c2 = (float(v) for v in p)
        self.es.set_materials(np.array([c1, c2]))
        self.solver.update_conditions(self.N.clamped_stretch_shear_conditions(self.mesh, lam, gam))

    def state(self, x):
        """Free-dof state: displacement z - X and pressure."""
        return x[self.free] - self.x_init[self.free]

    def solve_reference(self, p, increments):
        """The plain method: reference initial guess, load increments."""
        self.set_parameters(p)
        t0 = time.perf_counter()
        x, reps = self.solver.solve(self.x_init, increments)
        torch.cuda.synchronize(self.device) if self.device.type == "cuda" else None
        return x, reps, time.perf_counter() - t0

    def newton_from_state(self, p, state):
        """Newton at the full load of parameters p from the free-dof state
        `state`, without a fallback: (x, report)."""
        self.set_parameters(p)
        x = self.solver.apply_increment(self.x_init.clone(), 1, 1)
        x[self.free] = self.x_init[self.free] + state
        return self.solver.newton(x)

    def solve_from_state(self, p, state, fallback_increments):
        """One full-load increment from a predicted state; the reference
        method if that does not converge.  Returns (x, reports, seconds,
        accepted_guess)."""
        self.set_parameters(p)
        t0 = time.perf_counter()
        x = self.solver.apply_increment(self.x_init.clone(), 1, 1)
        x[self.free] = self.x_init[self.free] + state
        x, rep = self.solver.newton(x)
        if rep.converged:
            torch.cuda.synchronize(self.device) if self.device.type == "cuda" else None
            return x, [rep], time.perf_counter() - t0, True
        x, reps = self.solver.solve(self.x_init, fallback_increments)
        torch.cuda.synchronize(self.device) if self.device.type == "cuda" else None
        return x, [rep] + reps, time.perf_counter() - t0, False


def sample_parameters(n, seed, stretch=(1.0, 1.3), shear=(0.0, 0.2), c_range=(0.5, 10.0)):
    """Seeded (stretch, shear, c1, c2): uniform stretch and shear, c1 and c2
    log-uniform."""
    rng = np.random.default_rng(seed)
    lam = rng.uniform(*stretch, size=n)
    gam = rng.uniform(*shear, size=n)
    lc = np.log(c_range)
    c1 = np.exp(rng.uniform(*lc, size=n))
    c2 = np.exp(rng.uniform(*lc, size=n))
    return np.stack([lam, gam, c1, c2], axis=1)


def _interpolate_parameters(a, b, t):
    """(stretch, shear, c1, c2) between a and b: stretch and shear linearly,
    the moduli geometrically."""
    return np.array([a[0] + t * (b[0] - a[0]), a[1] + t * (b[1] - a[1]),
                     a[2] * (b[2] / a[2]) ** t, a[3] * (b[3] / a[3]) ** t])


def generate_solves(problem, params, increments, continuation=False, steps=1, progress=None):
    """Converged free-dof states for every parameter row.

    Without continuation every row is solved by the plain method (reference
    guess, load increments).  With continuation the rows are visited along a
    greedy nearest-neighbour path in feature space and each solve starts from
    the previous converged state, walking to the new parameters in `steps`
    full-load Newton solves at parameters interpolated between the two (the
    plain method where one of them does not converge); the converged states
    are the same (||r||_2 <= atol), only cheaper to reach.  Returns (states in
    the order of params, Newton iterations per row).  progress (optional) is
    called after every row with (rows done, row index, Newton iterations of
    the row, seconds of the row)."""
    n = len(params)
    order = list(range(n))
    if continuation and n > 1:
        f = features(params)
        f = (f - f.mean(0)) / (f.std(0) + 1e-12)
        left = np.ones(n, dtype=bool)
        left[0] = False
        order = [0]
        for _ in range(n - 1):
            d = ((f - f[order[-1]]) ** 2).sum(axis=1)
            d[~left] = np.inf
            nxt = int(np.argmin(d))
            order.append(nxt)
            left[nxt] = False
    states = [None] * n
    iters = np.zeros(n, dtype=np.int64)
    prev = None
    prev_p = None
    for done, i in enumerate(order, start=1):
        t_row = time.perf_counter()
        p = params[i]
        if prev is not None and steps > 1 and hasattr(problem, "newton_from_state"):
            reps, st, ok = [], prev, True
            for k in range(1, steps + 1):
                x, rep = problem.newton_from_state(_interpolate_parameters(prev_p, p, k / steps), st)
                reps.append(rep)
                if not rep.converged:
                    ok = False
                    break
                st = problem.state(x)
            if not ok:
                x, more, _ = problem.solve_reference(p, increments)
                reps += more
        elif prev is not None:
            x, reps, _, _ = problem.solve_from_state(p, prev, increments)
        else:
            x, reps, _ = problem.solve_reference(p, increments)
        if not reps[-1].converged:
            raise RuntimeError("a training solve did not converge: parameters %s" % (p,))
        states[i] = problem.state(x)
        iters[i] = sum(r.iterations for r in reps)
        prev = states[i] if continuation else None
        prev_p = p
        if progress is not None:
            progress(done, i, int(iters[i]), time.perf_counter() - t_row)
    return torch.stack(states), iters


def slab_features(params):
    """(surface pressure, Guccione C) -> (pressure, log C)."""
    p = np.asarray(params, dtype=np.float64)
    return np.stack([p[:, 0], np.log(p[:, 1])], axis=1)


def sample_slab_parameters(n, seed, pressure=(0.25, 2.0), c_range=(0.5, 2.0)):
    """Seeded (cavity pressure in kPa, Guccione C in kPa): pressure uniform,
    C log-uniform."""
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(*pressure, size=n), np.exp(rng.uniform(*np.log(c_range), size=n))], axis=1)


class SlabProblem:
    """The cardiac-style slab over (cavity pressure, Guccione C): lateral faces
    clamped, the pressure on z = 0 raised over the increments by the
    reference's pressure-increment rule; one equations set and solver reused
    for every sample (the other Guccione constants stay those of the mesh)."""

    def __init__(self, es, options, device="cuda"):
        from . import newton as N
        self.N = N
        self.es = es
        self.mesh = es.mesh
        self.device = torch.device(device)
        self.base_materials = np.asarray(self.mesh.materials, dtype=np.float64).copy()
        self.solver = N.LoadStepSolver(es, N.clamped_lateral_conditions(self.mesh), options, device=self.device)
        self.x_init = torch.from_numpy(N.initial_state(self.mesh)).to(self.device)
        self.free = self.solver.sys.free
        self.n_pressure = self.solver.sys.nfp

    def set_parameters(self, p):
        mats = self.base_materials.copy()
        mats[0] = float(p[1])
        self.es.set_materials(mats)

    def state(self, x):
        return x[self.free] - self.x_init[self.free]

    def _sync(self):
        if self.device.type == "cuda":
            torch.cuda.synchronize(self.device)

    def solve_reference(self, p, increments):
        self.set_parameters(p)
        t0 = time.perf_counter()
        full = self.N.bottom_face_pressure(self.mesh, float(p[0]))
        x, reps = self.solver.solve(self.x_init, increments, pressure=self.N.PressureIncrements(full))
        self._sync()
        return x, reps, time.perf_counter() - t0

    def solve_from_state(self, p, state, fallback_increments):
        """The full pressure at once from a predicted state; the reference
        method if that does not converge."""
        self.set_parameters(p)
        t0 = time.perf_counter()
        self.es.set_surface_pressure(self.N.bottom_face_pressure(self.mesh, float(p[0])))
        x = self.x_init.clone()
        x[self.free] = self.x_init[self.free] + state
        x, rep = self.solver.newton(x)
        if rep.converged:
            self._sync()
            return x, [rep], time.perf_counter() - t0, True
        full = self.N.bottom_face_pressure(self.mesh, float(p[0]))
        x, reps = self.solver.solve(self.x_init, fallback_increments, pressure=self.N.PressureIncrements(full))
        self._sync()
        return x, [rep] + reps, time.perf_counter() - t0, False
