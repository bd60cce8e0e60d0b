"""The reference's own exnode writer, driven the way the reference drives it
(test infrastructure: the field-export tests compare the library's writer,
cm_gb300/field_export.py, with this output; nothing in the library imports
it).

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
