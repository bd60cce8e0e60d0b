"""ctypes front end of the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker.  The shipped library never
does.  Every function mirrors one routine of ``fe_oracle.cpp``; see that file
for the reference routines (file:line) each one restates.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build as _build  # noqa: E402

MR = 1          # EQUATIONS_SET_MOONEY_RIVLIN_SUBTYPE (equations_set_constants.f90:121)
GUCCIONE = 15   # EQUATIONS_SET_TRANSVERSE_ISOTROPIC_GUCCIONE_SUBTYPE (:135)


class OrProblem(C.Structure):
    _fields_ = [
        ("ne", C.c_int32), ("nu", C.c_int32), ("np", C.c_int32), ("nxi_u", C.c_int32),
        ("p_mode", C.c_int32), ("law", C.c_int32), ("nmat", C.c_int32), ("mat_per_element", C.c_int32),
        ("elem_u", C.c_void_p), ("elem_p", C.c_void_p), ("X", C.c_void_p), ("mat", C.c_void_p),
        ("fibre", C.c_void_p), ("surf_p", C.c_void_p), ("bface", C.c_void_p),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.POINTER(OrProblem)
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        L.or_element_size.argtypes = [P]; L.or_element_size.restype = C.c_int
        L.or_num_dofs.argtypes = [P]; L.or_num_dofs.restype = i64
        L.or_element_residual.argtypes = [P, C.c_int, vp, vp]
        L.or_element_jacobian.argtypes = [P, C.c_int, vp, vp]
        L.or_element_jacobian_fd.argtypes = [P, C.c_int, vp, vp]
        L.or_element_dofs.argtypes = [P, C.c_int, vp]
        L.or_pattern.argtypes = [P, vp, vp]; L.or_pattern.restype = i64
        L.or_assemble.argtypes = [P, vp, vp, vp, vp, vp, C.c_int]; L.or_assemble.restype = C.c_int
        L.or_assemble_range.argtypes = [P, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int]
        L.or_assemble_range.restype = C.c_int
        L.or_regular_mesh.argtypes = [C.c_int] * 4 + [vp, vp]; L.or_regular_mesh.restype = C.c_int
        L.or_basis_tables.argtypes = [C.c_int, vp, vp, vp]
        L.or_point_stress.argtypes = [C.c_int, vp, vp, C.c_double, C.c_double, vp, vp]
        L.or_boundary_faces.argtypes = [P, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class Problem:
    """Holds numpy arrays alive and exposes the oracle routines.

    ``mesh`` is any object with the attributes of ``cm_gb300.mesh.Mesh``
    (elem_u, elem_p, X, nxi_u, p_mode, law, materials, fibre, ...)."""

    def __init__(self, mesh):
        self.m = mesh
        self.elem_u = np.ascontiguousarray(mesh.elem_u, dtype=np.int32)
        self.elem_p = None if mesh.elem_p is None else np.ascontiguousarray(mesh.elem_p, dtype=np.int32)
        self.X = np.ascontiguousarray(mesh.X, dtype=np.float64)
        self.mat = np.ascontiguousarray(mesh.materials, dtype=np.float64)
        self.fibre = None if mesh.fibre is None else np.ascontiguousarray(mesh.fibre, dtype=np.float64)
        s = OrProblem()
        s.ne, s.nu, s.np = mesh.ne, mesh.nu, mesh.np
        s.nxi_u, s.p_mode, s.law = mesh.nxi_u, mesh.p_mode, mesh.law
        s.nmat = self.mat.shape[-1]
        s.mat_per_element = 1 if self.mat.ndim == 2 else 0
        s.elem_u, s.elem_p, s.X, s.mat, s.fibre = (_p(self.elem_u), _p(self.elem_p), _p(self.X),
                                                  _p(self.mat), _p(self.fibre))
        self.s = s
        self.ref = C.byref(s)
        self.surf_p = None
        self.bface = None
        sp = getattr(mesh, "surface_pressure", None)
        if sp is not None:
            self.set_surface_pressure(sp)

    def set_surface_pressure(self, values):
        """values: [3][nu] nodal pressure (component n loads faces normal to xi_n), or None."""
        if values is None:
            self.surf_p = None
            self.s.surf_p = None
            return
        self.surf_p = np.ascontiguousarray(values, dtype=np.float64).reshape(3, self.m.nu)
        if self.bface is None:
            self.bface = np.zeros((self.m.ne, 6), dtype=np.uint8)
            lib().or_boundary_faces(self.ref, self.bface.ctypes.data)
        self.s.surf_p = self.surf_p.ctypes.data
        self.s.bface = self.bface.ctypes.data

    @property
    def nrow(self):
        return lib().or_element_size(self.ref)

    @property
    def ndofs(self):
        return lib().or_num_dofs(self.ref)

    def element_residual(self, e, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        r = np.zeros(self.nrow)
        lib().or_element_residual(self.ref, e, x.ctypes.data, r.ctypes.data)
        return r

    def element_jacobian(self, e, x):
        """Element Jacobian as a (row, col) numpy array."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = self.nrow
        k = np.zeros((n, n))
        lib().or_element_jacobian(self.ref, e, x.ctypes.data, k.ctypes.data)
        return k.T.copy()  # stored column-major

    def element_jacobian_fd(self, e, x):
        x = np.array(x, dtype=np.float64, copy=True)
        n = self.nrow
        k = np.zeros((n, n))
        lib().or_element_jacobian_fd(self.ref, e, x.ctypes.data, k.ctypes.data)
        return k.T.copy()

    def element_dofs(self, e):
        d = np.zeros(self.nrow, dtype=np.int32)
        lib().or_element_dofs(self.ref, e, d.ctypes.data)
        return d

    def pattern(self):
        """1-based (row_ptr, col) exactly as JacobianMatrix_StructureCalculate builds them."""
        nd = self.ndofs
        rp = np.zeros(nd + 1, dtype=np.int32)
        nnz = lib().or_pattern(self.ref, rp.ctypes.data, None)
        col = np.zeros(nnz, dtype=np.int32)
        lib().or_pattern(self.ref, rp.ctypes.data, col.ctypes.data)
        return rp, col

    def assemble(self, x, rp, col, jacobian=True, residual=True, nthreads=1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        vals = np.zeros(int(rp[-1]) - 1) if jacobian else None
        res = np.zeros(self.ndofs) if residual else None
        rc = lib().or_assemble(self.ref, x.ctypes.data, rp.ctypes.data, col.ctypes.data, _p(vals), _p(res), nthreads)
        if rc != 0:
            raise RuntimeError("oracle assembly: element entry missing from the CSR pattern")
        return vals, res


def regular_mesh(ex, ey, ez, nxi_u, nodal_p):
    npe = nxi_u ** 3
    ne = ex * ey * ez
    eu = np.zeros((ne, npe), dtype=np.int32)
    ep = np.zeros((ne, 8), dtype=np.int32) if nodal_p else None
    np_ = lib().or_regular_mesh(ex, ey, ez, nxi_u, eu.ctypes.data, _p(ep))
    return eu, ep, np_


def basis_tables(nxi):
    nn = nxi ** 3
    g = np.zeros((27, 4, nn)); w = np.zeros(27); xi = np.zeros((27, 3))
    lib().or_basis_tables(nxi, g.ctypes.data, w.ctypes.data, xi.ctypes.data)
    return g, w, xi


def point_stress(law, c, F, p):
    c = np.ascontiguousarray(c, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.float64)
    S = np.zeros(6); Cm = np.zeros((6, 6))
    lib().or_point_stress(law, c.ctypes.data, F.ctypes.data, float(np.linalg.det(F)), float(p),
                          S.ctypes.data, Cm.ctypes.data)
    return S, Cm


class EquationsSet:
    """CPU equations set with the call surface of
    ``cm_gb300.equations_set.FiniteElasticityEquationsSet`` that the Newton
    driver uses (``csr_pattern``, ``residual_evaluate``, ``jacobian_evaluate``),
    evaluated by the oracle.  Test infrastructure: it lets the same
    load-stepping code run on the CPU as the checker of the GPU run."""

    def __init__(self, mesh, nthreads=4):
        self.mesh = mesh
        self.materials = np.asarray(mesh.materials, dtype=np.float64)
        self.prob = Problem(mesh)
        self.rp1, self.col1 = self.prob.pattern()
        self.ndofs = int(self.prob.ndofs)
        self.nnz = int(self.rp1[-1]) - 1
        self.nthreads = nthreads

    def csr_pattern(self, base=0):
        return (self.rp1 - 1 + base).astype(np.int32), (self.col1 - 1 + base).astype(np.int32)

    def set_surface_pressure(self, values):
        self.prob.set_surface_pressure(None if values is None else np.asarray(values))

    def set_materials(self, materials):
        import copy
        m = copy.copy(self.mesh)
        m.materials = np.asarray(materials, dtype=np.float64)
        self.materials = m.materials
        sp = self.prob.surf_p
        self.prob = Problem(m)
        if sp is not None:
            self.prob.set_surface_pressure(sp)

    def residual_evaluate(self, x, r):
        _, res = self.prob.assemble(np.asarray(x), self.rp1, self.col1, jacobian=False, residual=True,
                                    nthreads=self.nthreads)
        r.copy_(r.new_tensor(res)) if hasattr(r, "copy_") else np.copyto(r, res)
        return r

    def jacobian_evaluate(self, x, values, r=None):
        vals, res = self.prob.assemble(np.asarray(x), self.rp1, self.col1, jacobian=True, residual=r is not None,
                                       nthreads=self.nthreads)
        for dst, src in ((values, vals), (r, res)):
            if dst is None:
                continue
            dst.copy_(dst.new_tensor(src)) if hasattr(dst, "copy_") else np.copyto(dst, src)
        return values
