"""Geometric multigrid preconditioner for the Newton linear systems on box meshes.

The linear system of a Newton step (Dirichlet dofs removed) is the saddle point
problem

    [ A  B^T ] [du]   [r_u]
    [ B  0   ] [dp] = [r_p]

(the pressure-pressure block of the reference's Jacobian is zero,
finite_elasticity_routines.f90:1075-1153).  It is preconditioned by the block
lower-triangular operator [A 0; B -S] with

* A^-1 ~ one V-cycle of geometric multigrid on the displacement block:
  coarse operators on a hierarchy of regular grids (triquadratic -> trilinear
  on the element vertices, then trilinear with the element count halved per
  direction), Chebyshev smoothing on the Jacobi-scaled operator, the inverse
  of the coarsest operator (dense); on the GPU one V-cycle is recorded in a
  CUDA graph and replayed.  The first coarse operator of a triquadratic mesh
  is either the Galerkin product P^T A P or, cheaper at large sizes, the
  displacement block of the trilinear mesh on the element vertices assembled
  at the injected state (rediscretisation; `vertex_mesh`); the further
  levels are Galerkin products;
* S ~ the consistent pressure mass matrix times a scale taken from
  diag(B diag(A)^-1 B^T) of the current Jacobian (the mass matrix is
  spectrally equivalent to the Schur complement for inf-sup stable pairs),
  applied by a fixed Chebyshev-Jacobi polynomial.

The operator hierarchy lives on the device in CSR form; prolongations are
tensor products of 1-D linear interpolation, built once on the host.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch


def _interp1d(nf: int, nc: int) -> sp.csr_matrix:
    """Linear interpolation from nc equally spaced coarse nodes to nf fine
    nodes on the same segment (nf x nc)."""
    if nc == nf:
        return sp.identity(nf, format="csr")
    rows, cols, vals = [], [], []
    for i in range(nf):
        t = i * (nc - 1) / (nf - 1)
        j = min(int(np.floor(t + 1e-12)), nc - 2)
        w = t - j
        if w < 1e-12:
            rows.append(i); cols.append(j); vals.append(1.0)
        elif w > 1.0 - 1e-12:
            rows.append(i); cols.append(j + 1); vals.append(1.0)
        else:
            rows += [i, i]; cols += [j, j + 1]; vals += [1.0 - w, w]
    return sp.csr_matrix((vals, (rows, cols)), shape=(nf, nc))


def _nearest_fine(nf: int, nc: int) -> np.ndarray:
    return np.rint(np.arange(nc) * (nf - 1) / max(nc - 1, 1)).astype(np.int64)


def _to_torch_csr(M: sp.spmatrix, device, dtype):
    M = M.tocsr()
    M.sort_indices()
    return torch.sparse_csr_tensor(torch.from_numpy(M.indptr.astype(np.int64)),
                                   torch.from_numpy(M.indices.astype(np.int64)),
                                   torch.from_numpy(M.data.astype(np.float64)),
                                   size=M.shape).to(device=device, dtype=dtype)


def grid_hierarchy(grid_u, nxi_u, min_dofs=1500):
    """Node counts per direction for every level, finest first."""
    levels = [tuple(grid_u)]
    elems = [(n - 1) // (nxi_u - 1) for n in grid_u]
    if nxi_u == 3:
        levels.append(tuple(e + 1 for e in elems))
    while True:
        cur = levels[-1]
        if 3 * int(np.prod(cur)) <= min_dofs or all(n <= 2 for n in cur):
            break
        nxt = tuple(max(2, (n - 1 + 1) // 2 + 1) if n > 2 else n for n in cur)
        if nxt == cur:
            break
        levels.append(nxt)
    return levels


def vertex_mesh(mesh):
    """The trilinear box mesh on the element vertices of a triquadratic box
    mesh: the same elements (same numbering), the vertex coordinates and
    fibre angles of the fine mesh, the same materials and pressure
    interpolation.  Returns the mesh and, per coarse dof, the fine dof it
    takes its value from (injection; nodal pressure lives on the vertices in
    both meshes, numbered alike)."""
    import dataclasses

    from .mesh import FE_PRESSURE_NODE_BASED, regular_box
    if mesh.nxi_u != 3 or not mesh.grid_u:
        raise ValueError("vertex_mesh needs a triquadratic box mesh")
    ex, ey, ez = mesh.dims
    n1, n2, _ = mesh.grid_u
    node = mesh.p_mode == FE_PRESSURE_NODE_BASED
    cm = regular_box(ex, ey, ez, lengths=mesh.lengths, nxi_u=2, pressure="node" if node else "element",
                     law=mesh.law, materials=mesh.materials)
    ci = np.arange(cm.nu)
    cx, cy, cz = ci % (ex + 1), (ci // (ex + 1)) % (ey + 1), ci // ((ex + 1) * (ey + 1))
    vid = 2 * cx + n1 * (2 * cy + n2 * 2 * cz)
    fib = None if mesh.fibre is None else np.ascontiguousarray(mesh.fibre[:, vid])
    cm = dataclasses.replace(cm, X=np.ascontiguousarray(mesh.X[:, vid]), fibre=fib,
                             materials=np.array(mesh.materials, dtype=np.float64, copy=True))
    nuf = mesh.nu
    inj = [c * nuf + vid for c in range(3)]
    inj.append(3 * nuf + np.arange(cm.n_pressure))
    return cm, np.concatenate(inj).astype(np.int64)


class VertexOperator:
    """The first coarse operator of a triquadratic box mesh by
    rediscretisation: the free displacement block of the Jacobian of
    `vertex_mesh(mesh)`, assembled by `coarse_es` (an equations set of that
    mesh) at the state injected from the fine one.  free_c is the mask of
    free coarse displacement dofs (the multigrid's level-1 mask).  A
    surface-pressure load of the fine set is not carried over: its follower
    stiffness is left out of this preconditioning operator, not of the
    Newton system."""

    def __init__(self, mesh, coarse_es, free_c, device):
        self.es = coarse_es
        self.device = torch.device(device)
        cm = coarse_es.mesh
        self.inj = torch.from_numpy(vertex_mesh(mesh)[1]).to(self.device)
        rp, col = coarse_es.csr_pattern()
        rp, col = rp.astype(np.int64), col.astype(np.int64)
        nu3 = 3 * cm.nu
        free = np.zeros(cm.ndofs, dtype=bool)
        free[:nu3] = free_c
        row = np.repeat(np.arange(cm.ndofs), np.diff(rp))
        keep = free[row] & free[col]
        new = np.cumsum(free) - 1
        counts = np.bincount(new[row[keep]], minlength=int(free.sum()))
        self.sel = torch.from_numpy(np.nonzero(keep)[0]).to(self.device)
        self.crow = torch.from_numpy(np.concatenate([[0], np.cumsum(counts)])).to(self.device)
        self.col = torch.from_numpy(new[col[keep]]).to(self.device)
        self.n = int(free.sum())
        self.vals = torch.empty(coarse_es.nnz, dtype=torch.float64, device=self.device)

    def assemble(self, x, dtype):
        """The coarse operator at the fine state x (full dof vector)."""
        self.es.jacobian_evaluate(x[self.inj].contiguous(), self.vals)
        return torch.sparse_csr_tensor(self.crow, self.col, self.vals[self.sel].to(dtype), size=(self.n, self.n))


class BoxMultigrid:
    """V-cycle for the free displacement block of a regular box mesh.

    free_u: boolean mask over the 3*nu displacement dofs (component-major)."""

    def __init__(self, grid_u, nxi_u, free_u, device, dtype=torch.float64, degree=3, min_dofs=1500, use_graph=True):
        self.device, self.dtype, self.degree = torch.device(device), dtype, degree
        self.use_graph = use_graph
        self.levels = grid_hierarchy(grid_u, nxi_u, min_dofs)
        self.P, self.R = [], []
        free = np.asarray(free_u, dtype=bool)
        self.free = [free]
        for lf, lc in zip(self.levels[:-1], self.levels[1:]):
            p1 = [_interp1d(nf, nc) for nf, nc in zip(lf, lc)]
            P3 = sp.kron(p1[2], sp.kron(p1[1], p1[0], format="csr"), format="csr")
            P = sp.block_diag([P3, P3, P3], format="csr")
            # a coarse dof is Dirichlet when the fine dof at its nearest fine node is
            near = [_nearest_fine(nf, nc) for nf, nc in zip(lf, lc)]
            ci = np.arange(int(np.prod(lc)))
            cx, cy, cz = ci % lc[0], (ci // lc[0]) % lc[1], ci // (lc[0] * lc[1])
            fnode = near[0][cx] + lf[0] * (near[1][cy] + lf[1] * near[2][cz])
            nf_nodes = int(np.prod(lf))
            cfree = np.concatenate([free[c * nf_nodes + fnode] for c in range(3)])
            Pf = P[free][:, cfree]
            self.P.append(_to_torch_csr(Pf, device, dtype))
            self.R.append(_to_torch_csr(Pf.T, device, dtype))
            free = cfree
            self.free.append(free)
        self.n_coarse = int(free.sum())

    # ------------------------------------------------------------------ setup
    def setup(self, A, A1=None):
        """A: free displacement block, torch CSR on the device (any float
        dtype); A1 (optional): the first coarse operator, else the Galerkin
        product."""
        A = A.to(self.dtype)
        self.A = [A]
        for lvl, (P, R) in enumerate(zip(self.P, self.R)):
            if lvl == 0 and A1 is not None:
                self.A.append(A1.to(self.dtype))
                continue
            Ac = torch.sparse.mm(R, torch.sparse.mm(self.A[-1], P))
            self.A.append(Ac.to_sparse_csr())
        self.dinv, self.lmax = [], []
        g = torch.Generator(device="cpu").manual_seed(1234)
        for Al in self.A[:-1]:
            d = self._diag(Al)
            dinv = torch.where(d != 0, 1.0 / d, torch.zeros_like(d))
            self.dinv.append(dinv)
            v = torch.rand(Al.shape[0], generator=g, dtype=torch.float64).to(self.device, self.dtype)
            lam = 1.0
            for _ in range(12):
                w = dinv * (Al @ v)
                lam = float(w.norm() / v.norm())
                v = w / w.norm()
            self.lmax.append(1.1 * lam)
        Ac = self.A[-1].to_dense().to(torch.float64)
        self.coarse_inv = torch.linalg.inv(Ac).to(self.dtype)  # small: the coarse solve is one GEMV
        self.graph = None
        if self.device.type == "cuda" and self.use_graph:
            self._capture()
        return self

    def _capture(self):
        """Records one V-cycle in a CUDA graph (static input/output buffers);
        falls back to eager launches if the capture is refused."""
        n = self.A[0].shape[0]
        self.g_in = torch.zeros(n, dtype=self.dtype, device=self.device)
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for _ in range(2):
                self.g_out = self._vcycle(self.g_in, 0)
        torch.cuda.current_stream(self.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.graph(g):
                self.g_out = self._vcycle(self.g_in, 0)
            self.graph = g
        except RuntimeError:
            self.graph = None
            torch.cuda.synchronize(self.device)

    @staticmethod
    def _diag(A):
        crow, col, val = A.crow_indices().long(), A.col_indices().long(), A.values()
        rows = torch.repeat_interleave(torch.arange(A.shape[0], device=val.device), crow[1:] - crow[:-1])
        d = torch.zeros(A.shape[0], dtype=val.dtype, device=val.device)
        m = rows == col
        d.index_add_(0, rows[m], val[m])
        return d

    def _cheby(self, lvl, b, x):
        """Chebyshev smoothing of A x = b on the interval [0.1, 1] * lmax of
        the Jacobi-scaled operator (degree self.degree)."""
        A, dinv = self.A[lvl], self.dinv[lvl]
        hi = self.lmax[lvl]
        lo = 0.1 * hi
        theta, delta = 0.5 * (hi + lo), 0.5 * (hi - lo)
        r = b - A @ x if x is not None else b.clone()
        x = torch.zeros_like(b) if x is None else x
        sigma = theta / delta
        rho = 1.0 / sigma
        d = dinv * r / theta
        for k in range(self.degree):
            x = x + d
            if k + 1 == self.degree:
                break
            r = r - A @ d
            rho_new = 1.0 / (2.0 * sigma - rho)
            d = (rho_new * rho) * d + (2.0 * rho_new / delta) * (dinv * r)
            rho = rho_new
        return x

    def vcycle(self, b):
        if self.graph is not None:
            self.g_in.copy_(b)
            self.graph.replay()
            return self.g_out.clone()
        return self._vcycle(b, 0)

    def _vcycle(self, b, lvl):
        if lvl == len(self.A) - 1:
            return self.coarse_inv @ b
        A = self.A[lvl]
        x = self._cheby(lvl, b, None)
        r = b - A @ x
        x = x + self.P[lvl] @ self._vcycle(self.R[lvl] @ r, lvl + 1)
        return self._cheby(lvl, b, x)


def lumped_pressure_mass(mesh):
    """Row sums of the pressure mass matrix: element volume (corner-node
    hexahedron, one-point rule) shared equally by the element's pressure
    parameters."""
    n1 = mesh.nxi_u
    c = [(a * (n1 - 1)) + (b * (n1 - 1)) * n1 + (cc * (n1 - 1)) * n1 * n1
         for cc in (0, 1) for b in (0, 1) for a in (0, 1)]
    X = mesh.X[:, mesh.elem_u[:, c]]          # (3, ne, 8) corners, x fastest
    e1 = 0.25 * ((X[:, :, 1] - X[:, :, 0]) + (X[:, :, 3] - X[:, :, 2]) + (X[:, :, 5] - X[:, :, 4]) + (X[:, :, 7] - X[:, :, 6]))
    e2 = 0.25 * ((X[:, :, 2] - X[:, :, 0]) + (X[:, :, 3] - X[:, :, 1]) + (X[:, :, 6] - X[:, :, 4]) + (X[:, :, 7] - X[:, :, 5]))
    e3 = 0.25 * ((X[:, :, 4] - X[:, :, 0]) + (X[:, :, 5] - X[:, :, 1]) + (X[:, :, 6] - X[:, :, 2]) + (X[:, :, 7] - X[:, :, 3]))
    vol = np.abs(np.einsum("ie,ie->e", e1, np.cross(e2.T, e3.T).T))
    if mesh.p_mode == 0:
        return vol
    m = np.zeros(mesh.np)
    np.add.at(m, mesh.elem_p.ravel(), np.repeat(vol / 8.0, 8))
    return m


def pressure_mass_matrix(mesh):
    """Consistent pressure mass matrix M(q, q') = sum_e int psi_q psi_q' dV
    (trilinear nodal pressure), integrated with the 2x2x2 Gauss rule on the
    trilinear map through the element's corner nodes; element-based pressure
    gives the diagonal of element volumes."""
    if mesh.p_mode == 0:
        return sp.diags(lumped_pressure_mass(mesh)).tocsr()
    n1 = mesh.nxi_u
    c = [(a * (n1 - 1)) + (b * (n1 - 1)) * n1 + (cc * (n1 - 1)) * n1 * n1
         for cc in (0, 1) for b in (0, 1) for a in (0, 1)]
    X = mesh.X[:, mesh.elem_u[:, c]]          # (3, ne, 8)
    gp = np.array([0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)])
    ne = mesh.ne
    Me = np.zeros((ne, 8, 8))
    for g3 in gp:
        for g2 in gp:
            for g1 in gp:
                t = (g1, g2, g3)
                psi = np.array([(t[0] if a else 1 - t[0]) * (t[1] if b else 1 - t[1]) * (t[2] if cc else 1 - t[2])
                                for cc in (0, 1) for b in (0, 1) for a in (0, 1)])
                dpsi = np.zeros((3, 8))
                for q, (a, b, cc) in enumerate([(a, b, cc) for cc in (0, 1) for b in (0, 1) for a in (0, 1)]):
                    f = [(t[k] if v else 1 - t[k]) for k, v in enumerate((a, b, cc))]
                    d = [(1.0 if v else -1.0) for v in (a, b, cc)]
                    dpsi[0, q] = d[0] * f[1] * f[2]
                    dpsi[1, q] = f[0] * d[1] * f[2]
                    dpsi[2, q] = f[0] * f[1] * d[2]
                Jm = np.einsum("ieq,kq->eik", X, dpsi)      # (ne, 3, 3) dX_i/dxi_k
                det = np.abs(np.linalg.det(Jm))
                Me += (0.125 * det)[:, None, None] * np.outer(psi, psi)[None]
    rows = np.repeat(mesh.elem_p, 8, axis=1).ravel()
    cols = np.tile(mesh.elem_p, (1, 8)).ravel()
    return sp.csr_matrix((Me.ravel(), (rows, cols)), shape=(mesh.np, mesh.np))


class MassSolver:
    """Fixed-step Chebyshev-Jacobi approximation of M^-1 for an SPD mass
    matrix (a linear operator, so plain GMRES stays valid)."""

    def __init__(self, M, device, steps=8):
        self.M = _to_torch_csr(M, device, torch.float64)
        d = torch.from_numpy(M.diagonal().copy()).to(device)
        self.dinv = 1.0 / d
        v = torch.linspace(0.3, 1.0, M.shape[0], dtype=torch.float64, device=device)
        lam = 1.0
        for _ in range(20):
            w = self.dinv * (self.M @ v)
            lam = float(w.norm() / v.norm())
            v = w / w.norm()
        self.hi = 1.05 * lam
        self.lo = self.hi / 30.0
        self.steps = steps

    def solve(self, b):
        theta, delta = 0.5 * (self.hi + self.lo), 0.5 * (self.hi - self.lo)
        sigma = theta / delta
        rho = 1.0 / sigma
        x = torch.zeros_like(b)
        r = b.clone()
        d = self.dinv * r / theta
        for k in range(self.steps):
            x = x + d
            if k + 1 == self.steps:
                break
            r = r - self.M @ d
            rho_new = 1.0 / (2.0 * sigma - rho)
            d = (rho_new * rho) * d + (2.0 * rho_new / delta) * (self.dinv * r)
            rho = rho_new
        return x
