"""Export of the geometric and dependent fields in the CMISS exnode/exelem text format.

The reference writes its fields with FIELD_IO_NODES_EXPORT / FIELD_IO_ELEMENTS_EXPORT
(field_IO_routines.f90:6158-6245) through the C writer in src/FieldExport.c
(group header :233, "Shape.  Dimension" :243, "#Scale factor sets" :263,
interpolation labels "l.Lagrange" / "q.Lagrange" and ", no modify, standard
node based." :300-375, "coordinate, rectangular cartesian" :593, "#Nodes" /
"#Fields" :641-647, " Node:" :1029, " Element: e 0 0" :814, "Nodes:" :833).
This module writes the same layout for the fields of one equations set, so a
converged state can be compared with, or loaded next to, output of the
reference: the undeformed geometry, the deformed geometry z (the dependent
field's displacement components) and the hydrostatic pressure (nodal on the
element corners, or element-constant).  Lagrange bases carry no derivatives
and no scale factors.
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh


def _basis_label(nxi):
    lab = {2: "l.Lagrange", 3: "q.Lagrange"}[nxi]
    return "*".join([lab] * 3)


def _node_components(mesh: Mesh):
    """Node-based components carried by every node, in field order: the
    geometric field's x, y, z, then the dependent field's three position
    components and, on the pressure (corner) nodes of a nodal pressure, its
    fourth (pressure) component."""
    has_p = np.zeros(mesh.nu, dtype=bool)
    if mesh.p_mode == 1:
        has_p[mesh.pressure_node_u()] = True
    return [7 if has_p[n] else 6 for n in range(mesh.nu)]


def _group_nodes(ncomp):
    """Node order of the reference's nodal information set sort
    (FIELD_IO_NODAL_INFO_SET_SORT, field_IO_routines.f90:4452-4520): each
    node's later namesakes (same component set) are swapped in right behind
    it; returns the order and whether each position repeats the previous
    header."""
    n = len(ncomp)
    order = list(range(n))
    repeat = [False] * n
    i = 0
    while i < n - 1:
        key = ncomp[order[i]]
        for j in range(i + 1, n):
            if ncomp[order[j]] == key:
                order[j], order[i + 1] = order[i + 1], order[j]
                repeat[j] = False
                repeat[i + 1] = True
                i += 1
        i += 1
    return order, repeat


def write_exnode(path, mesh: Mesh, x, group="Region", geometry="Geometry", dependent="Dependent"):
    """Nodal values of the geometric field and of the dependent field
    (deformed position and, for nodal pressure, the hydrostatic pressure on
    the pressure nodes) in the layout the reference's FieldExport.c writes
    when FIELD_IO_NODES_EXPORT exports these two fields: one header per run
    of nodes with the same component set (the dependent variable lists four
    components on every node; nodes without pressure carry six values, as in
    the reference's output), then one value per line in %.16E."""
    nu = mesh.nu
    z = np.asarray(x[:3 * nu], dtype=np.float64).reshape(3, nu)
    p = np.zeros(nu)
    if mesh.p_mode == 1:
        p[mesh.pressure_node_u()] = np.asarray(x[3 * nu:], dtype=np.float64)
    ncomp = _node_components(mesh)
    order, repeat = _group_nodes(ncomp)
    header = [" #Fields=2",
              " 1) %s, coordinate, rectangular cartesian, #Components=3" % geometry,
              "   x.  Value index= 1, #Derivatives= 0",
              "   y.  Value index= 2, #Derivatives= 0",
              "   z.  Value index= 3, #Derivatives= 0",
              " 2) %s, field,  rectangular cartesian, #Components=4" % dependent]
    header += ["   %d.  Value index= %d, #Derivatives= 0" % (c, 3 + c) for c in (1, 2, 3, 4)]
    lines = [" Group name: %s" % group]
    for pos, n in enumerate(order):
        if not repeat[pos]:
            lines += header
        lines.append(" Node:            %d" % (n + 1))
        vals = [mesh.X[0, n], mesh.X[1, n], mesh.X[2, n], z[0, n], z[1, n], z[2, n]]
        if ncomp[n] == 7:
            vals.append(p[n])
        lines += ["  %.16E" % v for v in vals]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_exelem(path, mesh: Mesh, x=None, group="Region"):
    """Element topology with the node-based interpolation of the two
    geometric fields; element-constant pressure (when x is given and the
    pressure is element based) as a constant, grid-based field."""
    npe = mesh.nxi_u ** 3
    label = _basis_label(mesh.nxi_u)
    names = [("Geometry", "coordinate, rectangular cartesian"), ("DeformedGeometry", "field, rectangular cartesian")]
    lines = [" Group name: %s" % group, " Shape.  Dimension=3", " #Scale factor sets= 0",
             " #Nodes=           %d" % npe, " #Fields=%d" % len(names)]
    for i, (name, kind) in enumerate(names, start=1):
        lines.append(" %d) %s, %s, #Components=3" % (i, name, kind))
        for c in ("x", "y", "z"):
            lines.append("   %s.  %s, no modify, standard node based." % (c, label))
            lines.append("     #Nodes= %d" % npe)
            for a in range(npe):
                lines.append("     %d.  #Values=1" % (a + 1))
                lines.append("      Value indices:     1")
                lines.append("      Scale factor indices:   0")
    for e in range(mesh.ne):
        lines.append(" Element:            %d 0 0" % (e + 1))
        lines.append("   Nodes:")
        lines.append("   " + " ".join("%d" % (n + 1) for n in mesh.elem_u[e]))
    if x is not None and mesh.p_mode == 0:
        p = np.asarray(x[3 * mesh.nu:], dtype=np.float64)
        lines.append(" Shape.  Dimension=3")
        lines.append(" #Scale factor sets= 0")
        lines.append(" #Nodes=           0")
        lines.append(" #Fields=1")
        lines.append(" 1) HydrostaticPressure, field, rectangular cartesian, #Components=1")
        lines.append("   1.  l.Lagrange*l.Lagrange*l.Lagrange, no modify, grid based.")
        lines.append("     #xi1=0, #xi2=0, #xi3=0")
        for e in range(mesh.ne):
            lines.append(" Element:            %d 0 0" % (e + 1))
            lines.append("   Values:")
            lines.append("   %.17e" % p[e])
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def export(prefix, mesh: Mesh, x, group="Region"):
    """Writes prefix.exnode and prefix.exelem for the state x (host array or
    tensor in the library's dof order)."""
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    write_exnode(prefix + ".exnode", mesh, x, group)
    write_exelem(prefix + ".exelem", mesh, x, group)
    return prefix + ".exnode", prefix + ".exelem"


def read_exnode_values(path):
    """Parses a file written by write_exnode: {node number: values} (six or
    seven per node) for checking round trips."""
    out, node = {}, None
    with open(path) as f:
        for ln in f:
            s = ln.strip()
            if s.startswith("Node:"):
                node = int(s.split()[1])
                out[node] = []
            elif s.startswith("#Fields=") or s.startswith("Group"):
                node = None
            elif node is not None and s and s[0] in "-0123456789":
                out[node] += [float(v) for v in s.split()]
    return out


def read_exelem_nodes(path):
    """Element number -> node numbers of the node-based element blocks."""
    elems, cur, want = {}, None, False
    with open(path) as f:
        for ln in f:
            s = ln.strip()
            if s.startswith("Element:"):
                cur = int(s.split()[1])
                want = False
            elif s == "Nodes:":
                want = True
            elif want and cur is not None:
                elems[cur] = [int(v) for v in s.split()]
                want = False
    return elems
