"""Load-stepped Newton solve on the GPU around the assembly library.

Restates the reference's solve path for the static finite-elasticity problem
(the control loop and SNES settings the assembly path is called from):

* load increments — PROBLEM_CONTROL_LOAD_INCREMENT_LOOP (problem_routines.f90:
  643-691) with EQUATIONS_SET_BOUNDARY_CONDITIONS_INCREMENT
  (equations_set_routines.f90:6491-6590): every fixed-incremented Dirichlet
  value moves as NEW = CUR + (FULL - CUR)/(N - i + 1), and takes exactly FULL
  on the last increment;
* Newton — SOLVER_NEWTON_LINESEARCH defaults (solver_routines.f90:17803-17812,
  18772-18775): initial guess = the current field, at most 50 iterations,
  cubic backtracking line search with alpha = 1e-4 and maximum step 1e8, and
  the absolute residual tolerance 1e-10 (the convergence test here is
  ||r||_2 <= atol on the free dofs);
* solver mapping — rows and columns of Dirichlet dofs are removed from the
  linear system (solver_mapping_routines.f90:1420,1592).

PETSc is not part of this build: the cubic backtracking step follows the
published Dennis-Schnabel algorithm that PETSc's "bt" line search implements,
and the linear solve is a dense LU (small systems) or restarted GMRES with a
block-diagonal (Jacobi / Schur-diagonal) preconditioner, both on the GPU.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import torch


@dataclass
class NewtonOptions:
    atol: float = 1e-10          # ||r_free||_2 stopping tolerance
    max_iterations: int = 50
    alpha: float = 1e-4          # sufficient-decrease constant of the line search
    max_step: float = 1e8
    min_lambda: float = 1e-10
    precision: str = "fp64"      # "fp64" Jacobian, or "mixed" (FP32 displacement block)
    high_precision: str = "fp64"  # residual/coupling arithmetic of the mixed path
    linear: str = "auto"         # "dense", "gmres" (block-Jacobi), "mg" (multigrid block preconditioner)
    #                              or "auto" (dense up to dense_limit free dofs)
    dense_limit: int = 12000
    gmres_rtol: float = 1e-5     # reference KSP defaults (solver_routines.f90:10979-10987):
    gmres_restart: int = 30      # GMRES(30), relative tolerance 1e-5
    gmres_max_iterations: int = 600
    forcing: str = "constant"    # "constant" (gmres_rtol) or "ew" (Eisenstat-Walker choice 2)
    mg_coarse: str = "vertex"    # first coarse operator of a triquadratic mesh: "vertex" (the trilinear
    #                              vertex mesh assembled at the injected state) or "galerkin" (P^T A P)
    mg_graph: bool = True        # record the whole preconditioner application (V-cycle, pressure-mass
    #                              solve, coupling SpMV) in one CUDA graph per Newton iteration
    csr_index: str = "int64"     # index type of the free-dof CSR operators ("int32" reads 4 bytes
    #                              fewer per entry in every SpMV of the Krylov operator and the fine level)


@dataclass
class StepReport:
    iterations: int = 0
    converged: bool = False
    residual_norms: list = field(default_factory=list)
    linear_iterations: list = field(default_factory=list)
    line_search_lambdas: list = field(default_factory=list)
    line_search_failed: bool = False
    seconds: float = 0.0
    assembly_seconds: float = 0.0
    linear_seconds: float = 0.0
    preconditioner_seconds: float = 0.0  # part of linear_seconds: multigrid set-up


class DirichletConditions:
    """Fixed and fixed-incremented Dirichlet values on dofs (BOUNDARY_CONDITION_FIXED and
    BOUNDARY_CONDITION_FIXED_INCREMENTED, boundary_condition_routines.f90:100-108)."""

    def __init__(self, ndofs: int):
        self.ndofs = ndofs
        self.dofs = np.zeros(0, dtype=np.int64)
        self.full = np.zeros(0)
        self.incremented = np.zeros(0, dtype=bool)

    def fix(self, dofs, values, incremented=False):
        dofs = np.asarray(dofs, dtype=np.int64).ravel()
        values = np.broadcast_to(np.asarray(values, dtype=np.float64), dofs.shape).copy()
        keep = ~np.isin(dofs, self.dofs)
        self.dofs = np.concatenate([self.dofs, dofs[keep]])
        self.full = np.concatenate([self.full, values[keep]])
        self.incremented = np.concatenate([self.incremented, np.full(int(keep.sum()), bool(incremented))])
        return self

    def free_mask(self):
        m = np.ones(self.ndofs, dtype=bool)
        m[self.dofs] = False
        return m


class PressureIncrements:
    """Surface pressure raised over the load increments by the reference's
    BOUNDARY_CONDITION_PRESSURE_INCREMENTED rule
    (equations_set_routines.f90:6652-6720): on increment 1 the applied
    pressure is FULL / N and the previous one 0; afterwards
    NEW = CURRENT + (CURRENT - PREVIOUS), PREVIOUS = CURRENT."""

    def __init__(self, full):
        self.full = np.asarray(full, dtype=np.float64)
        self.current = None
        self.previous = None

    def step(self, i, n):
        if i == 1:
            self.current, self.previous = self.full / n, np.zeros_like(self.full)
        else:
            self.current, self.previous = self.current + (self.current - self.previous), self.current
        return self.current


class FreeDofSystem:
    """Index maps from the full CSR pattern to the free-dof submatrix."""

    def __init__(self, es, free_mask, device, index_dtype=torch.int64):
        rp, col = es.csr_pattern(base=0)
        n = es.ndofs
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
        keep = free_mask[rows] & free_mask[col]
        new_index = -np.ones(n, dtype=np.int64)
        new_index[free_mask] = np.arange(int(free_mask.sum()))
        self.nf = int(free_mask.sum())
        self.sel = torch.from_numpy(np.nonzero(keep)[0]).to(device)
        r = new_index[rows[keep]]
        c = new_index[col[keep]]
        counts = np.bincount(r, minlength=self.nf)
        if index_dtype == torch.int32 and int(keep.sum()) >= 2 ** 31:
            index_dtype = torch.int64
        ix = np.int32 if index_dtype == torch.int32 else np.int64
        self.crow = torch.from_numpy(np.concatenate([[0], np.cumsum(counts)]).astype(ix)).to(device)
        self.col = torch.from_numpy(c.astype(ix)).to(device)
        self.row = torch.from_numpy(r.astype(np.int64)).to(device)
        self.free = torch.from_numpy(np.nonzero(free_mask)[0]).to(device)
        self.is_p = torch.from_numpy(np.nonzero(free_mask)[0] >= 3 * es.mesh.nu).to(device)
        self.is_diag = (self.row == self.col)
        self.device = device
        # displacement block A (free u x free u) and coupling block B (p x free u):
        # free u dofs come first, and in every row the u columns precede the p columns
        nfu = int((np.nonzero(free_mask)[0] < 3 * es.mesh.nu).sum())
        self.nfu, self.nfp = nfu, self.nf - nfu
        am = (r < nfu) & (c < nfu)
        bm = (r >= nfu) & (c < nfu)
        self.a_sel = torch.from_numpy(np.nonzero(am)[0]).to(device)
        self.a_crow = torch.from_numpy(
            np.concatenate([[0], np.cumsum(np.bincount(r[am], minlength=nfu))]).astype(ix)).to(device)
        self.a_col = torch.from_numpy(c[am].astype(ix)).to(device)
        self.b_sel = torch.from_numpy(np.nonzero(bm)[0]).to(device)
        self.b_crow = torch.from_numpy(
            np.concatenate([[0], np.cumsum(np.bincount(r[bm] - nfu, minlength=self.nfp))]).astype(ix)).to(device)
        self.b_col = torch.from_numpy(c[bm].astype(ix)).to(device)

    def matrix(self, vals_full):
        v = vals_full[self.sel]
        return torch.sparse_csr_tensor(self.crow, self.col, v, size=(self.nf, self.nf))

    def blocks(self, J, dtype_a=torch.float64):
        v = J.values()
        A = torch.sparse_csr_tensor(self.a_crow, self.a_col, v[self.a_sel].to(dtype_a), size=(self.nfu, self.nfu))
        B = torch.sparse_csr_tensor(self.b_crow, self.b_col, v[self.b_sel], size=(self.nfp, self.nfu))
        return A, B


def _graphed(f, n, device):
    """f (a function of one FP64 vector of length n that launches only device
    work) recorded in a CUDA graph with a static input and output; f itself
    if the capture is refused.  The returned function holds f, and so every
    tensor f reads: the graph replays their device addresses."""
    w_in = torch.zeros(n, dtype=torch.float64, device=device)
    cur = torch.cuda.current_stream(device)
    side = torch.cuda.Stream(device)
    side.wait_stream(cur)
    with torch.cuda.stream(side):
        for _ in range(2):  # warm-up outside the capture (library handles, workspaces)
            f(w_in)
    cur.wait_stream(side)
    g = torch.cuda.CUDAGraph()
    try:
        with torch.cuda.graph(g):
            out = f(w_in)
    except RuntimeError:
        torch.cuda.synchronize(device)
        return f

    def replay(w, _source=f):
        w_in.copy_(w)
        g.replay()
        return out.clone()
    return replay


def _gmres(A, b, M, rtol, restart, max_it, check_every=6):
    """Right-preconditioned restarted GMRES (FP64); M(v) applies the preconditioner.

    The Arnoldi process (classical Gram-Schmidt with one re-orthogonalisation)
    stays on the device; the small least-squares problem min ||beta e1 - H y||
    is solved on the host every `check_every` iterations to test convergence,
    so the host waits for the device only at those points."""
    n = b.numel()
    x = torch.zeros_like(b)
    bnorm = float(b.norm())
    if bnorm == 0.0:
        return x, 0
    total = 0
    r = b.clone()
    tiny = torch.finfo(b.dtype).tiny
    V = torch.zeros(restart + 1, n, dtype=b.dtype, device=b.device)
    Z = torch.zeros(restart, n, dtype=b.dtype, device=b.device)
    while total < max_it:
        beta = float(r.norm())
        if beta <= rtol * bnorm:
            break
        H = torch.zeros(restart + 1, restart, dtype=b.dtype, device=b.device)
        V[0] = r / beta
        k = 0
        y = None
        while k < restart and total < max_it:
            Z[k] = M(V[k])
            w = A @ Z[k]
            h = V[:k + 1] @ w
            w = w - V[:k + 1].T @ h
            h2 = V[:k + 1] @ w
            w = w - V[:k + 1].T @ h2
            hn = w.norm()
            H[:k + 1, k] = h + h2
            H[k + 1, k] = hn
            V[k + 1] = w / torch.clamp(hn, min=tiny)
            k += 1
            total += 1
            if k % check_every == 0 or k == restart or total >= max_it:
                Hh = H[:k + 1, :k].double().cpu()
                rhs = torch.zeros(k + 1, dtype=torch.float64)
                rhs[0] = beta
                y = torch.linalg.lstsq(Hh, rhs.unsqueeze(1)).solution.squeeze(1)
                res = float((rhs - Hh @ y).norm())
                if res <= rtol * bnorm or float(Hh[k, k - 1]) <= 1e-14 * beta:
                    break
        if y is None or y.numel() != k:
            Hh = H[:k + 1, :k].double().cpu()
            rhs = torch.zeros(k + 1, dtype=torch.float64)
            rhs[0] = beta
            y = torch.linalg.lstsq(Hh, rhs.unsqueeze(1)).solution.squeeze(1)
        x = x + Z[:k].T @ y.to(b.device, b.dtype)
        r = b - A @ x
    return x, total


def mixed_positions(es):
    """Positions in the full CSR pattern (0-based) of the entries of the
    mixed split (fe_mixed_layout): each displacement row holds its uu
    entries first, then its coupling entries; pressure rows hold coupling
    entries only."""
    uu_rp, cp_rp = (a.astype(np.int64) for a in es.mixed_layout())
    rp = es.csr_pattern()[0].astype(np.int64)
    nu3 = 3 * es.mesh.nu
    ku = np.zeros(es.ndofs, dtype=np.int64)
    ku[:nu3] = np.diff(uu_rp)
    ru = np.repeat(np.arange(nu3), ku[:nu3])
    uu_pos = rp[ru] + (np.arange(uu_rp[-1]) - uu_rp[ru])
    rc = np.repeat(np.arange(es.ndofs), np.diff(cp_rp))
    cp_pos = rp[rc] + ku[rc] + (np.arange(cp_rp[-1]) - cp_rp[rc])
    return uu_pos, cp_pos


class LoadStepSolver:
    """Load-stepped Newton for one equations set on the GPU."""

    def __init__(self, es, bc: DirichletConditions, options: NewtonOptions | None = None, device="cuda"):
        self.es = es
        self.bc = bc
        self.opt = options or NewtonOptions()
        self.device = torch.device(device)
        self.free_mask = bc.free_mask()
        self.sys = FreeDofSystem(es, self.free_mask, self.device,
                                 torch.int32 if self.opt.csr_index == "int32" else torch.int64)
        self.bc_dofs = torch.from_numpy(bc.dofs).to(self.device)
        if self.opt.precision == "mixed":
            es.set_high_precision(self.opt.high_precision)
            uu_pos, cp_pos = mixed_positions(es)
            self.uu_pos = torch.from_numpy(uu_pos).to(self.device)
            self.cp_pos = torch.from_numpy(cp_pos).to(self.device)
            self.vu = torch.empty(es.nnz_uu, dtype=torch.float32, device=self.device)
            self.vc = torch.empty(es.nnz_coupling, dtype=torch.float64, device=self.device)
        if self.opt.linear == "mg":
            from .multigrid import BoxMultigrid, MassSolver, pressure_mass_matrix
            m = es.mesh
            self.mg = BoxMultigrid(m.grid_u, m.nxi_u, self.free_mask[:3 * m.nu], self.device,
                                   torch.float32 if self.opt.precision == "mixed" else torch.float64,
                                   use_graph=not self.opt.mg_graph)
            self.coarse = None
            if self.opt.mg_coarse == "vertex" and m.nxi_u == 3 and len(self.mg.free) > 1:
                from .multigrid import VertexOperator, vertex_mesh
                cm, _ = vertex_mesh(m)
                self.coarse = VertexOperator(m, type(es)(cm), self.mg.free[1], self.device)
                self.coarse_materials = None
            fp = self.free_mask[3 * m.nu:]
            Mp = pressure_mass_matrix(m)[fp][:, fp]
            self.mass_p = torch.from_numpy(Mp.diagonal().copy()).to(self.device)
            self.mass_solver = MassSolver(Mp, self.device)
        self.vals = torch.empty(es.nnz, dtype=torch.float64, device=self.device)
        self.r = torch.empty(es.ndofs, dtype=torch.float64, device=self.device)
        self.setup_seconds = 0.0

    def _sync(self):
        if self.device.type == "cuda":
            torch.cuda.synchronize(self.device)

    def update_conditions(self, bc: DirichletConditions):
        """New Dirichlet values on the same set of dofs (the free-dof system,
        its index maps and the multigrid hierarchy are kept)."""
        if not np.array_equal(bc.dofs, self.bc.dofs):
            raise ValueError("the Dirichlet dof set must not change")
        self.bc = bc

    # -------------------------------------------------------------- pieces
    def apply_increment(self, x, i, n):
        """Dirichlet values for increment i of n (1-based), the reference's rule."""
        cur = x[self.bc_dofs]
        full = torch.from_numpy(self.bc.full).to(x)
        inc = torch.from_numpy(self.bc.incremented).to(self.device)
        new = full.clone() if i == n else torch.where(inc, cur + (full - cur) / (n - i + 1), full)
        x[self.bc_dofs] = new
        return x

    def residual(self, x):
        """Residual on the free dofs, or None when the state has an element
        with det F <= 0 or a non-finite stress (the kernels' status word)."""
        self.es.residual_evaluate(x, self.r)
        check = getattr(self.es, "check_status", None)
        if check is not None:
            try:
                check(x)
            except Exception as e:  # FEError(FE_ERR_NUMERICAL)
                if getattr(e, "code", None) == -5:
                    return None
                raise
        return self.r[self.sys.free]

    def jacobian(self, x):
        self._x_jac = x  # the state of the Jacobian (the multigrid's coarse operator is assembled there)
        if self.opt.precision == "mixed":
            self.es.jacobian_evaluate_mixed(x, self.vu, self.vc, self.r)
            self.vals[self.uu_pos] = self.vu.double()
            self.vals[self.cp_pos] = self.vc
        else:
            self.es.jacobian_evaluate(x, self.vals, self.r)
        return self.sys.matrix(self.vals), self.r[self.sys.free]

    def _preconditioner(self, A):
        """Block-diagonal preconditioner: Jacobi on displacement rows, the
        diagonal of B diag(A)^-1 B^T on pressure rows."""
        S = self.sys
        v = A.values()
        diag = torch.zeros(S.nf, dtype=torch.float64, device=self.device)
        diag.index_add_(0, S.row[S.is_diag], v[S.is_diag])
        inv = torch.zeros_like(diag)
        u = ~S.is_p
        inv[u] = 1.0 / diag[u]
        # Schur diagonal for pressure rows: sum_j B_ij^2 / A_jj over displacement columns
        pr = S.is_p[S.row] & ~S.is_p[S.col]
        sd = torch.zeros_like(diag)
        sd.index_add_(0, S.row[pr], v[pr] ** 2 * inv[S.col[pr]])
        p = S.is_p
        inv[p] = -1.0 / torch.where(sd[p] != 0, sd[p], torch.ones_like(sd[p]))
        return lambda w: inv * w

    def _mg_preconditioner(self, J):
        """Block lower-triangular preconditioner [A 0; B -S]^-1 with a multigrid
        V-cycle for A and the scaled lumped pressure mass for S."""
        S = self.sys
        t0 = time.perf_counter()
        mg_dtype = torch.float32 if self.opt.precision == "mixed" else torch.float64
        A, B = S.blocks(J, mg_dtype)
        A1 = None
        if self.coarse is not None:
            mats = getattr(self.es, "materials", None)
            mats = self.es.mesh.materials if mats is None else mats
            if self.coarse_materials is None or not np.array_equal(mats, self.coarse_materials):
                self.coarse.es.set_materials(mats)
                self.coarse_materials = np.array(mats, copy=True)
            A1 = self.coarse.assemble(self._x_jac, mg_dtype)
        self.mg.setup(A, A1)
        dA = self.mg.dinv[0].to(torch.float64)
        sd = torch.zeros(S.nfp, dtype=torch.float64, device=self.device)
        bv = B.values()
        bcrow = B.crow_indices().long()
        brow = torch.repeat_interleave(torch.arange(S.nfp, device=self.device), bcrow[1:] - bcrow[:-1])
        sd.index_add_(0, brow, bv * bv * dA[B.col_indices().long()])
        scale = float(torch.median(sd / self.mass_p))
        nfu = S.nfu
        self.setup_seconds += time.perf_counter() - t0

        def apply(w):
            zu = self.mg.vcycle(w[:nfu].to(mg_dtype)).to(torch.float64)
            zp = self.mass_solver.solve(B @ zu - w[nfu:]) / scale
            return torch.cat([zu, zp])
        if self.device.type == "cuda" and self.opt.mg_graph:
            return _graphed(apply, S.nf, self.device)
        return apply

    def linear_solve(self, A, b, rtol=None):
        if self.opt.linear == "dense" or (self.opt.linear == "auto" and self.sys.nf <= self.opt.dense_limit):
            D = A.to_dense()
            return torch.linalg.solve(D, b), 1
        rtol = self.opt.gmres_rtol if rtol is None else rtol
        if self.opt.linear == "mg":
            M = self._mg_preconditioner(A)
            return _gmres(A, b, M, rtol, self.opt.gmres_restart, self.opt.gmres_max_iterations)
        M = self._preconditioner(A)
        return _gmres(A, b, M, rtol, self.opt.gmres_restart, self.opt.gmres_max_iterations)

    # -------------------------------------------------------------- Newton
    def newton(self, x, report: StepReport | None = None):
        """Newton iterations at the current Dirichlet values (x is updated in place)."""
        o = self.opt
        rep = report or StepReport()
        t_start = time.perf_counter()
        free = self.sys.free
        r = self.residual(x)
        if r is None:
            rep.residual_norms.append(float("inf"))
            rep.iterations, rep.converged = 0, False
            rep.seconds = time.perf_counter() - t_start
            return x, rep
        r = r.clone()
        fnorm = float(r.norm())
        rep.residual_norms.append(fnorm)
        it = 0
        prev_eta = None
        while fnorm > o.atol and it < o.max_iterations:
            self._sync()
            ta = time.perf_counter()
            A, _ = self.jacobian(x)
            self._sync()
            tb = time.perf_counter()
            eta = o.gmres_rtol
            if o.forcing == "ew":
                # Eisenstat & Walker (1996), choice 2 with gamma = 0.9, alpha = 2 and their safeguard
                eta = 0.5 if len(rep.residual_norms) < 2 else \
                    0.9 * (rep.residual_norms[-1] / rep.residual_norms[-2]) ** 2
                if prev_eta is not None and 0.9 * prev_eta ** 2 > 0.1:
                    eta = max(eta, 0.9 * prev_eta ** 2)
                eta = min(max(eta, o.gmres_rtol), 0.5)
                prev_eta = eta
            self.setup_seconds = 0.0
            d, lin_it = self.linear_solve(A, -r, eta)
            self._sync()
            rep.assembly_seconds += tb - ta
            rep.linear_seconds += time.perf_counter() - tb
            rep.preconditioner_seconds += self.setup_seconds
            rep.linear_iterations.append(int(lin_it))
            dn = float(d.norm())
            if dn > o.max_step:
                d = d * (o.max_step / dn)
            # cubic backtracking (Dennis & Schnabel): f = 1/2 ||r||^2
            f0 = 0.5 * fnorm * fnorm
            slope = float(r @ (A @ d))
            if slope > 0:
                slope = -slope
            lam, lam_prev, f_prev = 1.0, None, None
            accepted = False
            x0 = x[free].clone()
            while True:
                x[free] = x0 + lam * d
                rn = self.residual(x)
                if rn is None:          # a step into inverted elements counts as a failed step
                    rn = torch.full_like(r, float("inf"))
                else:
                    rn = rn.clone()
                f1 = 0.5 * float(rn @ rn)
                if np.isfinite(f1) and f1 <= f0 + o.alpha * lam * slope:
                    accepted = True
                    break
                if lam < o.min_lambda:
                    break
                if lam_prev is None or not np.isfinite(f1):
                    lt = -slope / (2.0 * (f1 - f0 - slope)) if np.isfinite(f1) else 0.1 * lam
                else:
                    a1 = f1 - f0 - lam * slope
                    a2 = f_prev - f0 - lam_prev * slope
                    den = lam - lam_prev
                    a = (a1 / lam ** 2 - a2 / lam_prev ** 2) / den
                    b = (-lam_prev * a1 / lam ** 2 + lam * a2 / lam_prev ** 2) / den
                    if a == 0.0:
                        lt = -slope / (2.0 * b)
                    else:
                        disc = max(b * b - 3.0 * a * slope, 0.0)
                        lt = (-b + np.sqrt(disc)) / (3.0 * a)
                lam_prev, f_prev = lam, f1
                lam = float(min(max(lt, 0.1 * lam), 0.5 * lam))
            rep.line_search_lambdas.append(lam)
            it += 1
            if not accepted:
                # no step with sufficient decrease: keep the state from before
                # the step (PETSc's bt line search leaves X on a failed
                # reduction) and stop unconverged
                x[free] = x0
                rep.line_search_failed = True
                break
            r = rn
            fnorm = float(r.norm())
            rep.residual_norms.append(fnorm)
        rep.iterations = it
        rep.converged = fnorm <= o.atol
        self._sync()
        rep.seconds = time.perf_counter() - t_start
        return x, rep

    def solve(self, x0, increments: int, guesses=None, pressure: PressureIncrements | None = None,
              progress=None):
        """All load increments from state x0; guesses (optional) maps the
        increment number to a Newton initial guess for the free dofs;
        pressure (optional) raises a surface-pressure load with the
        increments; progress (optional) is called with (increment, report)
        after each increment."""
        x = x0.clone()
        reports = []
        for i in range(1, increments + 1):
            x = self.apply_increment(x, i, increments)
            if pressure is not None:
                self.es.set_surface_pressure(pressure.step(i, increments))
            if guesses is not None and i in guesses:
                x[self.sys.free] = guesses[i][self.sys.free]
            x, rep = self.newton(x)
            reports.append(rep)
            if progress is not None:
                progress(i, rep)
            if not rep.converged:
                break
        return x, reports


# ----------------------------------------------------------------- set-ups
def uniaxial_symmetry_conditions(mesh, stretch):
    """Config-1 style uniaxial extension of a box: symmetry planes x=0 (u_x),
    y=0 (u_y), z=0 (u_z) fixed, the x = L face moved to stretch * L in x
    (fixed-incremented).  The symmetry planes remove the rigid rotation that
    'x=0 face fixed in x, one corner pinned' alone would leave."""
    nu = mesh.nu
    bc = DirichletConditions(mesh.ndofs)
    i, j, k = mesh.node_ijk()
    n1, n2, n3 = mesh.grid_u
    X = mesh.X
    bc.fix(np.nonzero(i == 0)[0], X[0, i == 0])
    bc.fix(nu + np.nonzero(j == 0)[0], X[1, j == 0])
    bc.fix(2 * nu + np.nonzero(k == 0)[0], X[2, k == 0])
    right = np.nonzero(i == n1 - 1)[0]
    bc.fix(right, stretch * X[0, right], incremented=True)
    return bc


def clamped_stretch_shear_conditions(mesh, stretch, shear):
    """Config-2 style loading: the x = 0 face clamped (z = X), the x = L face
    moved to z_x = stretch * L, z_y = Y + shear * L, z_z = Z (fixed-incremented)."""
    nu = mesh.nu
    bc = DirichletConditions(mesh.ndofs)
    i, j, k = mesh.node_ijk()
    n1 = mesh.grid_u[0]
    X = mesh.X
    left = np.nonzero(i == 0)[0]
    right = np.nonzero(i == n1 - 1)[0]
    for c in range(3):
        bc.fix(c * nu + left, X[c, left])
    L = X[0, right]
    bc.fix(right, stretch * L, incremented=True)
    bc.fix(nu + right, X[1, right] + shear * L, incremented=True)
    bc.fix(2 * nu + right, X[2, right], incremented=True)
    return bc


def initial_state(mesh):
    """The reference's initial dependent field: z = X, p = 0."""
    return np.concatenate([mesh.X.ravel(), np.zeros(mesh.n_pressure)])


def clamped_lateral_conditions(mesh):
    """Slab loading: the four lateral faces (x = 0, x = Lx, y = 0, y = Ly)
    clamped in every component, the z faces free."""
    i, j, k = mesh.node_ijk()
    n1, n2, _ = mesh.grid_u
    side = np.nonzero((i == 0) | (i == n1 - 1) | (j == 0) | (j == n2 - 1))[0]
    bc = DirichletConditions(mesh.ndofs)
    for c in range(3):
        bc.fix(c * mesh.nu + side, mesh.X[c, side])
    return bc


def bottom_face_pressure(mesh, value):
    """[3][nu] nodal surface pressure `value` on the z = 0 faces (faces
    normal to xi3), zero elsewhere."""
    i, j, k = mesh.node_ijk()
    sp = np.zeros((3, mesh.nu))
    sp[2, k == 0] = value
    return sp


def cylinder_conditions(mesh, stretch):
    """Dirichlet conditions of the reference's cylinder inflation-extension
    problem (FiniteElasticity_BoundaryConditionsAnalyticCalculate,
    finite_elasticity_routines.f90:132-484) on a `mesh.thick_cylinder` mesh:
    z fixed to 0 on the bottom and to stretch * Z on the top (here raised with
    the load increments, fixed-incremented), and on the bottom the x (y)
    component fixed to 0 at the nodes with |X| < 1e-7 (|Y| < 1e-7), which
    removes the rigid rotation and translation."""
    _, _, k = mesh.node_ijk()
    nz = mesh.grid_u[2]
    X = mesh.X
    nu = mesh.nu
    bc = DirichletConditions(mesh.ndofs)
    bottom = np.nonzero(k == 0)[0]
    top = np.nonzero(k == nz - 1)[0]
    bc.fix(2 * nu + bottom, 0.0)
    bc.fix(2 * nu + top, stretch * X[2, top], incremented=True)
    bx = bottom[np.abs(X[0, bottom]) < 1e-7]
    by = bottom[np.abs(X[1, bottom]) < 1e-7]
    bc.fix(bx, 0.0)
    bc.fix(nu + by, 0.0)
    return bc


def cylinder_pressure(mesh, p_inner, p_outer):
    """[3][nu] surface pressure of the cylinder problem: p_inner on the inner
    surface and p_outer on the outer surface, both on faces normal to xi1
    (the reference stores them on component |normal xi| = 1 of the DELUDELN
    variable, finite_elasticity_routines.f90:196-223)."""
    i, _, _ = mesh.node_ijk()
    sp = np.zeros((3, mesh.nu))
    sp[0, i == 0] = p_inner
    sp[0, i == mesh.grid_u[0] - 1] = p_outer
    return sp
