"""The reference's own exnode and exelem writers, driven the way the
reference drives them (test infrastructure: the field-export tests compare
the library's writer, cm_gb300/field_export.py, with this output; nothing in
the library imports it).

``oracle/_ref/libfieldexport.so`` is the reference's src/FieldExport.c,
compiled unchanged by ``oracle/build.py``.  This module restates, for the two
fields of one finite-elasticity equations set, the calls the reference's
Fortran makes into it when it exports nodes:

* FIELD_IO_EXPORT_NODES_INTO_LOCAL_FILE (field_IO_routines.f90:5355-5520):
  open a session, write the group name, then for every node of the sorted
  nodal information set a header when the node's component set differs from
  the previous node's, and one FieldExport_NodeValues call per component
  (no derivatives, one version: one value per call);
* FIELD_IO_EXPORT_NODAL_GROUP_HEADER_FORTRAN (:5101-5354): the field count,
  per variable its coordinate / general variable line, and per component its
  value index, with a padding entry for a component the node does not carry
  (whose padding value the node loop never writes: the padding counter sits
  at the position after the node's last component);
* FIELD_IO_NODAL_INFO_SET_SORT (:4452-4520): nodes with the same component
  set are brought together by its swap loop.

For elements it restates:

* FIELD_IO_EXPORT_ELEMENTS_INTO_LOCAL_FILE (field_IO_routines.f90:3533-3853):
  group name and mesh dimensions once, then per element (in element order:
  FIELD_IO_ELEMENTAL_INFO_SET_SORT, :3860-4061, keeps it, all elements sharing
  their bases) the header when the element's header differs from the last,
  the element index, the values of element-based components, the element's
  nodes on the basis with the most nodes, and its scale factors
  (FIELD_IO_EXPORT_ELEMENT_SCALE_FACTORS, :3418-3526: one set per distinct
  basis, in component order; Lagrange bases have unit factors);
* FieldIO_ExportElementalGroupHeaderFortran (:2519-3412, non-collapsed
  branch): scale-factor sets (one per distinct basis and scaling type; the
  default scaling, arithmetic mean), node count, field count, and per
  component its interpolation line followed by either the grid size
  (element-based: constant) or the node / value / scale-factor indices --
  with the reference's first scale index of a later set,
  SUM(set sizes up to and including that set) - 1 (:2826-2830).

The fields: the geometric field (label "Geometry", rectangular cartesian
coordinates, three components on mesh component 1) and the dependent field
(label "Dependent", FIELD_GEOMETRIC_GENERAL_TYPE, variable U, four
components: the deformed position on mesh component 1 and the hydrostatic
pressure on mesh component 2, nodal on the corner nodes; element-based
pressure is not a node-based component and is not in the exnode file).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libfieldexport.so")

EXPORT_TYPE_FILE = 1
FIELD_GEOMETRIC_TYPE, FIELD_GEOMETRIC_GENERAL_TYPE = 1, 5
FIELD_U_VARIABLE_TYPE = 1
COORDINATE_RECTANGULAR_CARTESIAN_TYPE = 1
NO_PART_DERIV = 1

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise FileNotFoundError(LIB)
        _lib = C.CDLL(LIB)
    return _lib


def node_components(mesh):
    """Per node (0-based), the node-based components it carries, in field and
    component order: ('G', 1..3) and ('D', 1..4)."""
    has_p = np.zeros(mesh.nu, dtype=bool)
    if mesh.p_mode == 1:
        has_p[mesh.pressure_node_u()] = True
    base = [("G", 1), ("G", 2), ("G", 3), ("D", 1), ("D", 2), ("D", 3)]
    return [tuple(base + ([("D", 4)] if has_p[n] else [])) for n in range(mesh.nu)]


def sort_nodes(comps):
    """FIELD_IO_NODAL_INFO_SET_SORT: the order of the nodes (0-based) and the
    SAME_HEADER flag of each position."""
    n = len(comps)
    order = list(range(n))
    same = [False] * n
    nn1 = 0
    while nn1 < n - 1:
        c1 = comps[order[nn1]]
        for nn2 in range(nn1 + 1, n):  # the Fortran DO bounds are fixed at loop entry
            if comps[order[nn2]] == c1:
                order[nn2], order[nn1 + 1] = order[nn1 + 1], order[nn2]
                same[nn2] = False
                same[nn1 + 1] = True
                nn1 += 1
        nn1 += 1
    return order, same


def write_exnode(path, mesh, x, group="Region"):
    """The exnode file of the state x (the library's dof order) through the
    reference's C writer."""
    L = lib()
    nu = mesh.nu
    z = np.asarray(x[:3 * nu], dtype=np.float64).reshape(3, nu)
    pval = np.zeros(nu)
    if mesh.p_mode == 1:
        pval[mesh.pressure_node_u()] = np.asarray(x[3 * nu:], dtype=np.float64)
    comps = node_components(mesh)
    order, same = sort_nodes(comps)
    h = C.c_int()
    assert L.FieldExport_OpenSession(EXPORT_TYPE_FILE, path.encode(), C.byref(h)) == 0
    hd = h.value
    L.FieldExport_Group(hd, group.encode())
    deriv = (C.c_int * 1)(NO_PART_DERIV)
    one = (C.c_double * 1)()
    for pos, n in enumerate(order):
        cs = comps[n]
        if not same[pos]:
            L.FieldExport_FieldCount(hd, 2)
            value_idx, comp_idx1 = 1, 0
            L.FieldExport_CoordinateVariable(hd, b"Geometry", 1, COORDINATE_RECTANGULAR_CARTESIAN_TYPE, 3)
            for c in (1, 2, 3):
                L.FieldExport_CoordinateDerivativeIndices(hd, c, COORDINATE_RECTANGULAR_CARTESIAN_TYPE, 1, deriv,
                                                          value_idx)
                L.FieldExport_VersionInfo(hd, 1)
                L.FieldExport_EndComponent(hd)
                comp_idx1 += 1
                value_idx += 1
            L.FieldExport_Variable(hd, b"Dependent", 2, FIELD_GEOMETRIC_GENERAL_TYPE, FIELD_U_VARIABLE_TYPE, 4)
            for c in (1, 2, 3, 4):
                present = comp_idx1 < len(cs) and cs[comp_idx1] == ("D", c)
                L.FieldExport_DerivativeIndices(hd, c, FIELD_GEOMETRIC_GENERAL_TYPE, FIELD_U_VARIABLE_TYPE, 1, deriv,
                                                value_idx)
                if present:
                    L.FieldExport_VersionInfo(hd, 1)
                    comp_idx1 += 1
                L.FieldExport_EndComponent(hd)
                value_idx += 1
        for kind, c in cs:
            one[0] = mesh.X[c - 1, n] if kind == "G" else (z[c - 1, n] if c < 4 else pval[n])
            L.FieldExport_NodeValues(hd, n + 1, 1, one)
    assert L.FieldExport_CloseSession(hd) == 0


BASIS_LAGRANGE_HERMITE_TP_TYPE = 1
LINEAR_LAGRANGE, QUADRATIC_LAGRANGE = 1, 2
INTERP_ELEMENT_BASED, INTERP_NODE_BASED = 2, 3


def _components(mesh):
    """The element components in field order: (field, component number,
    interpolation type, basis) with basis = (name, interpolation per xi,
    element nodes as u-node numbers per element)."""
    nxi = mesh.nxi_u
    u_basis = ("u", [QUADRATIC_LAGRANGE if nxi == 3 else LINEAR_LAGRANGE] * 3, mesh.elem_u)
    comps = [("G", c, INTERP_NODE_BASED, u_basis) for c in (1, 2, 3)]
    comps += [("D", c, INTERP_NODE_BASED, u_basis) for c in (1, 2, 3)]
    if mesh.p_mode == 1:
        corners = [(a * (nxi - 1)) + (b * (nxi - 1)) * nxi + (c * (nxi - 1)) * nxi * nxi
                   for c in (0, 1) for b in (0, 1) for a in (0, 1)]
        comps.append(("D", 4, INTERP_NODE_BASED, ("p", [LINEAR_LAGRANGE] * 3, mesh.elem_u[:, corners])))
    else:
        comps.append(("D", 4, INTERP_ELEMENT_BASED, u_basis))
    return comps


def write_exelem(path, mesh, x, group="Region"):
    """The exelem file of the state x (element-based pressure values from x)
    through the reference's C writer."""
    L = lib()
    comps = _components(mesh)
    nu = mesh.nu
    h = C.c_int()
    assert L.FieldExport_OpenSession(EXPORT_TYPE_FILE, path.encode(), C.byref(h)) == 0
    hd = h.value
    L.FieldExport_Group(hd, group.encode())
    L.FieldExport_MeshDimensions(hd, 3, BASIS_LAGRANGE_HERMITE_TP_TYPE)
    # scale-factor sets: one per distinct basis (all fields use the same scaling type)
    sets, comp_set = [], []
    for comp in comps:
        name = comp[3][0]
        if name not in [b[0] for b in sets]:
            sets.append(comp[3])
        comp_set.append([b[0] for b in sets].index(name) + 1)
    set_sizes = [int(np.prod([3 if t == QUADRATIC_LAGRANGE else 2 for t in b[1]])) for b in sets]
    nmax = max(b[2].shape[1] for b in sets)
    max_basis = next(c[3] for c in comps if c[3][2].shape[1] == nmax)
    for e in range(mesh.ne):
        if e == 0:  # every element has the first element's header
            L.FieldExport_ScalingFactorCount(hd, len(sets))
            for b, n in zip(sets, set_sizes):
                L.FieldExport_ScaleFactors(hd, 3, (C.c_int * 3)(*b[1]), n)
            L.FieldExport_NodeCount(hd, nmax)
            L.FieldExport_FieldCount(hd, 2)
            prev = None
            for (field, cn, interp, basis), sidx in zip(comps, comp_set):
                if field != prev:
                    prev = field
                    if field == "G":
                        L.FieldExport_CoordinateVariable(hd, b"Geometry", 1, COORDINATE_RECTANGULAR_CARTESIAN_TYPE, 3)
                    else:
                        L.FieldExport_Variable(hd, b"Dependent", 2, FIELD_GEOMETRIC_GENERAL_TYPE, FIELD_U_VARIABLE_TYPE,
                                               4)
                xi = (C.c_int * 3)(*basis[1])
                if field == "G":
                    L.FieldExport_CoordinateComponent(hd, COORDINATE_RECTANGULAR_CARTESIAN_TYPE, cn, interp, 3, xi)
                else:
                    L.FieldExport_Component(hd, cn, interp, 3, xi)
                if interp != INTERP_NODE_BASED:
                    L.FieldExport_ElementGridSize(hd, interp, 3, xi)
                    continue
                first = 0 if sidx == 1 else sum(set_sizes[:sidx]) - 1
                nn = basis[2].shape[1]
                nodes = basis[2][e]
                pos = [int(np.nonzero(max_basis[2][e] == n)[0][0]) + 1 for n in nodes]
                L.FieldExport_NodeScaleIndexes(hd, nn, (C.c_int * nn)(*([1] * nn)), (C.c_int * nn)(*([1] * nn)),
                                               (C.c_int * nn)(*pos),
                                               (C.c_int * nn)(*range(first + 1, first + 1 + nn)))
        L.FieldExport_ElementIndex(hd, 3, e + 1)
        first_value = 1
        for field, cn, interp, basis in comps:
            if interp == INTERP_ELEMENT_BASED:
                L.FieldExport_ElementGridValues(hd, first_value, 1, C.c_double(float(x[3 * nu + e])))
                first_value = 0
        nodes = max_basis[2][e] + 1
        L.FieldExport_ElementNodeIndices(hd, len(nodes), (C.c_int * len(nodes))(*nodes.tolist()))
        first_set, want = 1, 1
        for (field, cn, interp, basis), sidx in zip(comps, comp_set):
            if sidx == want:
                want += 1
                n = basis[2].shape[1]
                L.FieldExport_ElementNodeScales(hd, first_set, n, (C.c_double * n)(*([1.0] * n)))
                first_set = 0
    assert L.FieldExport_CloseSession(hd) == 0

