"""Host-side mirror of the reference's finite-elasticity equations-set call
surface for the assembly path, on top of the C ABI (include/cm_fe.h).

Reference call surface mirrored (OpenCMISS-Iron):
  * EQUATIONS_SET_RESIDUAL_EVALUATE (equations_set_routines.f90:5184) ->
    :meth:`FiniteElasticityEquationsSet.residual_evaluate`
  * EQUATIONS_SET_JACOBIAN_EVALUATE (:4694) ->
    :meth:`FiniteElasticityEquationsSet.jacobian_evaluate`
  * FiniteElasticity_FiniteElement{Residual,Jacobian}Evaluate
    (finite_elasticity_routines.f90:1260, :842) ->
    :meth:`element_residuals`, :meth:`element_jacobians`
  * the Jacobian's CSR structure (JacobianMatrix_StructureCalculate,
    equations_matrices_routines.f90:5048) -> :meth:`csr_pattern`

Arrays may be numpy arrays (host memory: the call copies in and out and
returns when done) or CUDA torch tensors (device memory: the call is
asynchronous on the current torch stream).  Failures raise
:class:`cm_gb300._lib.FEError`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FEError, check  # noqa: F401
from .mesh import Mesh


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    # torch tensor
    if not a.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return a.data_ptr()


def _stream(a):
    if isinstance(a, np.ndarray) or a is None or not getattr(a, "is_cuda", False):
        return None
    import torch
    return C.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)


def mesh_desc(mesh: Mesh, keep: list):
    """fe_mesh_desc for a mesh; the arrays it points to are appended to keep
    (they must stay alive while the descriptor is used)."""
    def arr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    mats = np.asarray(mesh.materials, dtype=np.float64)
    d = _lib.FEMeshDesc()
    d.num_elements = mesh.ne
    d.num_nodes_u = mesh.nu
    d.num_nodes_p = mesh.np
    d.nodes_per_xi_u = mesh.nxi_u
    d.pressure_interpolation = mesh.p_mode
    d.law = mesh.law
    d.num_material_components = mats.shape[-1]
    d.materials_per_element = 1 if mats.ndim == 2 else 0
    d.element_nodes_u = arr(mesh.elem_u, np.int32)
    d.element_nodes_p = arr(mesh.elem_p, np.int32)
    d.geometry = arr(mesh.X, np.float64)
    d.materials = arr(mats, np.float64)
    d.fibre_angles = arr(mesh.fibre, np.float64)
    return d


def structure_calculate(mesh: Mesh, base: int = 0, on_device: bool = False):
    """The Jacobian's CSR pattern of a mesh without creating an equations set:
    fe_structure_calculate (host) or fe_structure_calculate_device (GPU).
    Returns host (row_ptr, col) arrays."""
    L = _lib.load()
    keep = []
    d = mesh_desc(mesh, keep)
    nd, nnz = C.c_int64(), C.c_int64()
    if on_device:
        check(L.fe_structure_calculate_device(C.byref(d), base, C.byref(nd), C.byref(nnz), None, None, None))
    else:
        check(L.fe_structure_calculate(C.byref(d), base, C.byref(nd), C.byref(nnz), None, None))
    rp = np.zeros(nd.value + 1, dtype=np.int32)
    col = np.zeros(nnz.value, dtype=np.int32)
    if on_device:
        check(L.fe_structure_calculate_device(C.byref(d), base, None, None, rp.ctypes.data, col.ctypes.data, None))
    else:
        check(L.fe_structure_calculate(C.byref(d), base, None, None, rp.ctypes.data, col.ctypes.data))
    return rp, col


class FiniteElasticityEquationsSet:
    """One finite-elasticity equations set (mesh + law + materials) on the
    current CUDA device."""

    def __init__(self, mesh: Mesh):
        self.mesh = mesh
        L = _lib.load()
        self._keep = []
        d = mesh_desc(mesh, self._keep)
        h = C.c_void_p()
        check(L.fe_create(C.byref(d), C.byref(h)))
        self._keep = []
        self._h = h
        nd, nnz = C.c_int64(), C.c_int64()
        check(L.fe_sizes(h, C.byref(nd), C.byref(nnz)))
        self.ndofs, self.nnz = nd.value, nnz.value
        n = C.c_int32()
        check(L.fe_element_size(h, C.byref(n)))
        self.element_size = n.value
        nuu, ncp = C.c_int64(), C.c_int64()
        check(L.fe_mixed_layout(h, C.byref(nuu), C.byref(ncp), None, None))
        self.nnz_uu, self.nnz_coupling = nuu.value, ncp.value

    def clone(self, materials=None):
        """fe_clone: another equations set on the same mesh, sharing its
        mesh-only device arrays; optionally with new materials."""
        out = object.__new__(FiniteElasticityEquationsSet)
        h = C.c_void_p()
        check(_lib.load().fe_clone(self._h, C.byref(h)))
        out.__dict__.update({k: v for k, v in self.__dict__.items() if k != "_h"})
        out._h = h
        if materials is not None:
            out.set_materials(materials)
        return out

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().fe_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -------------------------------------------------------------- pattern
    def csr_pattern(self, base: int = 0):
        rp = np.zeros(self.ndofs + 1, dtype=np.int32)
        col = np.zeros(self.nnz, dtype=np.int32)
        check(_lib.load().fe_csr_pattern(self._h, base, rp.ctypes.data, col.ctypes.data))
        return rp, col

    def mixed_layout(self):
        uu = np.zeros(3 * self.mesh.nu + 1, dtype=np.int32)
        cp = np.zeros(self.ndofs + 1, dtype=np.int32)
        check(_lib.load().fe_mixed_layout(self._h, None, None, uu.ctypes.data, cp.ctypes.data))
        return uu, cp

    # ----------------------------------------------------------- evaluation
    def _alloc_like(self, x, n, dtype):
        if isinstance(x, np.ndarray):
            return np.zeros(n, dtype=dtype)
        import torch
        return torch.empty(n, dtype={np.float64: torch.float64, np.float32: torch.float32}[dtype], device=x.device)

    def residual_evaluate(self, x, r=None):
        r = self._alloc_like(x, self.ndofs, np.float64) if r is None else r
        check(_lib.load().fe_residual_evaluate(self._h, _ptr(x), _ptr(r), _stream(x)))
        return r

    def residual_evaluate_noalloc(self, x, r=None):
        """fe_residual_evaluate_noalloc: the residual without any device
        allocation (static staging array; at most FE_NOALLOC_MAX_DOFS dofs)."""
        r = np.zeros(self.ndofs) if r is None else r
        check(_lib.load().fe_residual_evaluate_noalloc(self._h, _ptr(x), _ptr(r), _stream(x)))
        return r

    def jacobian_evaluate(self, x, values=None, r=None):
        values = self._alloc_like(x, self.nnz, np.float64) if values is None else values
        check(_lib.load().fe_jacobian_evaluate(self._h, _ptr(x), _ptr(values), _ptr(r), _stream(x)))
        return values

    def jacobian_evaluate_mixed(self, x, values_uu=None, values_coupling=None, r=None):
        values_uu = self._alloc_like(x, self.nnz_uu, np.float32) if values_uu is None else values_uu
        values_coupling = (self._alloc_like(x, self.nnz_coupling, np.float64)
                           if values_coupling is None else values_coupling)
        check(_lib.load().fe_jacobian_evaluate_mixed(self._h, _ptr(x), _ptr(values_uu), _ptr(values_coupling),
                                                     _ptr(r), _stream(x)))
        return values_uu, values_coupling

    def element_residuals(self, x, first=0, count=None):
        count = self.mesh.ne - first if count is None else count
        out = self._alloc_like(x, count * self.element_size, np.float64)
        check(_lib.load().fe_element_residuals(self._h, _ptr(x), first, count, _ptr(out), _stream(x)))
        return out.reshape(count, self.element_size)

    def element_jacobians(self, x, first=0, count=None):
        """Element Jacobians as (count, row, col) arrays (the C ABI writes
        them column-major, like ELEMENT_JACOBIAN%MATRIX)."""
        count = self.mesh.ne - first if count is None else count
        n = self.element_size
        out = self._alloc_like(x, count * n * n, np.float64)
        check(_lib.load().fe_element_jacobians(self._h, _ptr(x), first, count, _ptr(out), _stream(x)))
        return out.reshape(count, n, n).transpose(1, 2) if not isinstance(out, np.ndarray) else \
            out.reshape(count, n, n).transpose(0, 2, 1)

    def set_surface_pressure(self, values):
        """Nodal surface pressure [3][nu] (component n loads the boundary faces
        normal to xi_n), as numpy or CUDA tensor; None removes the load."""
        if values is None:
            check(_lib.load().fe_set_surface_pressure(self._h, None))
            return
        if isinstance(values, np.ndarray):
            values = np.ascontiguousarray(values, dtype=np.float64)
        check(_lib.load().fe_set_surface_pressure(self._h, _ptr(values)))

    def set_materials(self, materials):
        """New material parameters, same layout as the mesh's (host array)."""
        mats = np.ascontiguousarray(materials, dtype=np.float64)
        if mats.shape != np.shape(self.mesh.materials):
            raise ValueError("materials must have shape %s" % (np.shape(self.mesh.materials),))
        check(_lib.load().fe_set_materials(self._h, mats.ctypes.data))
        self.materials = mats

    def set_high_precision(self, mode: str):
        """'fp64' (IEEE binary64, default) or 'double_float' (FP32 pairs, about
        48 significant bits) for the residual and pressure-coupling parts of
        residual_evaluate and jacobian_evaluate_mixed."""
        code = {"fp64": _lib.FE_HIGH_PRECISION_FP64, "double_float": _lib.FE_HIGH_PRECISION_DOUBLE_FLOAT}[mode]
        check(_lib.load().fe_set_high_precision(self._h, code))
        self.high_precision = mode

    def set_assembly_order(self, order):
        """fe_set_assembly_order: "staged" (per-element records and a row
        gather, the default) or "coloured" (element colours adding into the
        CSR arrays) for jacobian_evaluate_mixed."""
        code = {"staged": _lib.FE_ASSEMBLY_STAGED, "coloured": _lib.FE_ASSEMBLY_COLOURED}[order]
        check(_lib.load().fe_set_assembly_order(self._h, code))
        self.assembly_order = order

    def set_host_output(self, mode, chunks=0):
        """fe_set_host_output: how jacobian_evaluate_mixed delivers outputs in
        host memory -- "streamed" (the default: rows copied to the host chunk
        by chunk while the rest assembles; `chunks` equal launches, or 0 for
        launches on whole waves of the kernel's resident blocks),
        "in_place" (page-locked outputs written by the row gather over the
        host link) or "after" (one copy after the assembly).  The values are
        identical in every mode."""
        code = {"streamed": _lib.FE_HOST_OUTPUT_STREAMED, "in_place": _lib.FE_HOST_OUTPUT_IN_PLACE,
                "after": _lib.FE_HOST_OUTPUT_AFTER}[mode]
        check(_lib.load().fe_set_host_output(self._h, code, chunks))
        self.host_output = mode

    def newton_load_step(self, x, fixed_dofs, fixed_values, **options):
        """fe_newton_load_step: one load increment by Newton on the device
        (FP64 Jacobian, block-diagonal-preconditioned GMRES, cubic
        backtracking).  x (numpy array or CUDA tensor of all dofs) is the
        initial guess and receives the converged state; fixed_dofs take
        fixed_values.  Options are the fields of fe_newton_options
        (max_iterations, atol, alpha, max_step, min_lambda, ksp_rtol,
        ksp_restart, ksp_max_iterations, forcing).  Returns the report as a
        dict."""
        L = _lib.load()
        o = _lib.FENewtonOptions()
        L.fe_newton_options_default(C.byref(o))
        for k, v in options.items():
            if not hasattr(o, k):
                raise ValueError("unknown Newton option " + k)
            setattr(o, k, v)
        dofs = np.ascontiguousarray(fixed_dofs, dtype=np.int32)
        vals = np.ascontiguousarray(np.broadcast_to(np.asarray(fixed_values, dtype=np.float64), dofs.shape))
        rep = _lib.FENewtonReport()
        check(L.fe_newton_load_step(self._h, dofs.ctypes.data, vals.ctypes.data, int(dofs.size), _ptr(x),
                                    C.byref(o), C.byref(rep), _stream(x)))
        return {k: getattr(rep, k) for k, _ in rep._fields_}

    def check_status(self, x=None):
        check(_lib.load().fe_check(self._h, _stream(x)))

    def launch_count(self):
        c = C.c_int64()
        check(_lib.load().fe_launch_count(self._h, C.byref(c)))
        return c.value

    # ------------------------------------------------------------- helpers
    def mixed_to_full(self, values_uu, values_coupling):
        """Merges the mixed split back into one FP64 array in pattern order
        (host numpy; for checking)."""
        uu_rp, cp_rp = self.mixed_layout()
        rp, _ = self.csr_pattern()
        vu = np.asarray(values_uu, dtype=np.float64)
        vc = np.asarray(values_coupling, dtype=np.float64)
        out = np.empty(self.nnz)
        nu3 = 3 * self.mesh.nu
        for r in range(self.ndofs):
            a, b = rp[r], rp[r + 1]
            if r < nu3:
                k = uu_rp[r + 1] - uu_rp[r]
                out[a:a + k] = vu[uu_rp[r]:uu_rp[r + 1]]
                out[a + k:b] = vc[cp_rp[r]:cp_rp[r + 1]]
            else:
                out[a:b] = vc[cp_rp[r]:cp_rp[r + 1]]
        return out


def create_equations_sets(meshes, threads=None):
    """One FiniteElasticityEquationsSet per mesh, created concurrently: each
    fe_create builds its mesh's set-up (pattern, rank tables, colouring,
    geometry cache) on the host and uploads it, and the C call releases the
    interpreter, so many small meshes set up in parallel on the host cores.
    Returns the sets in the order of `meshes`."""
    import concurrent.futures as cf
    import os
    meshes = list(meshes)
    if threads is None:
        threads = min(len(meshes), os.cpu_count() or 1)
    if threads <= 1:
        return [FiniteElasticityEquationsSet(m) for m in meshes]
    with cf.ThreadPoolExecutor(threads) as ex:
        return list(ex.map(FiniteElasticityEquationsSet, meshes))


class EquationsSetBatch:
    """Many independent equations sets assembled in one persistent launch
    (fe_batch_* of include/cm_fe.h).  Buffers are CUDA tensors."""

    def __init__(self, sets):
        self.sets = list(sets)
        arr = (C.c_void_p * len(self.sets))(*[s.handle for s in self.sets])
        b = C.c_void_p()
        check(_lib.load().fe_batch_create(arr, len(self.sets), C.byref(b)))
        self._b = b

    def close(self):
        if getattr(self, "_b", None):
            _lib.load().fe_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arrays(self, xs, vus, vcs, rs):
        n = len(self.sets)
        if not (len(xs) == len(vus) == len(vcs) == n) or (rs is not None and len(rs) != n):
            raise ValueError("one buffer per member is required")
        P = C.c_void_p * n
        a = [P(*[t.data_ptr() for t in lst]) for lst in (xs, vus, vcs)]
        r = P(*[t.data_ptr() for t in rs]) if rs is not None else None
        return a[0], a[1], a[2], r

    def allocate(self, device):
        """Output buffers (values_uu, values_coupling, r) for every member."""
        import torch
        vus = [torch.empty(s.nnz_uu, dtype=torch.float32, device=device) for s in self.sets]
        vcs = [torch.empty(s.nnz_coupling, dtype=torch.float64, device=device) for s in self.sets]
        rs = [torch.empty(s.ndofs, dtype=torch.float64, device=device) for s in self.sets]
        return vus, vcs, rs

    def jacobian_evaluate_mixed(self, xs, vus, vcs, rs=None):
        x, u, c, r = self._arrays(xs, vus, vcs, rs)
        check(_lib.load().fe_batch_jacobian_evaluate_mixed(self._b, x, u, c, r, _stream(xs[0])))

    def check(self, like=None):
        check(_lib.load().fe_batch_check(self._b, _stream(like)))

    def set_config(self, variant, ctas_per_sm, block_groups):
        check(_lib.load().fe_batch_set_config(self._b, variant, ctas_per_sm, block_groups))

    def set_barrier_limits(self, polls=0, extra_arrivals=0):
        """fe_batch_set_barrier_limits: diagnostic of the grid barrier's
        failure path (extra_arrivals=1 makes every barrier give up after
        `polls` polls; (0, 0) restores the default)."""
        check(_lib.load().fe_batch_set_barrier_limits(self._b, polls, extra_arrivals))

    def config(self):
        v, c, g, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double()
        check(_lib.load().fe_batch_get_config(self._b, C.byref(v), C.byref(c), C.byref(g), C.byref(ms)))
        return {"variant": v.value, "ctas_per_sm": c.value, "block_groups": g.value, "tuned_ms": ms.value}

    def autotune(self, xs, vus, vcs, rs=None, repeats=3):
        x, u, c, r = self._arrays(xs, vus, vcs, rs)
        check(_lib.load().fe_batch_autotune(self._b, x, u, c, r, repeats, _stream(xs[0])))
        return self.config()

    def capture(self, xs, vus, vcs, rs=None):
        x, u, c, r = self._arrays(xs, vus, vcs, rs)
        check(_lib.load().fe_batch_capture(self._b, x, u, c, r, _stream(xs[0])))

    def replay(self, like):
        check(_lib.load().fe_batch_replay(self._b, _stream(like)))

    def launch_count(self):
        n = C.c_int64()
        check(_lib.load().fe_batch_launch_count(self._b, C.byref(n)))
        return n.value
