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


def _node_fields(mesh: Mesh, x):
    nu = mesh.nu
    z = np.asarray(x[:3 * nu], dtype=np.float64).reshape(3, nu)
    fields = [("Geometry", "coordinate, rectangular cartesian", ("x", "y", "z"), mesh.X),
              ("DeformedGeometry", "field, rectangular cartesian", ("x", "y", "z"), z)]
    return fields


def write_exnode(path, mesh: Mesh, x, group="FiniteElasticity"):
    """Nodal values of the geometry and the deformed geometry (one value per
    node and component), plus the nodal pressure on the pressure nodes."""
    fields = _node_fields(mesh, x)
    nu = mesh.nu
    lines = [" Group name: %s" % group, " #Fields=%d" % len(fields)]
    for i, (name, kind, comps, _) in enumerate(fields, start=1):
        lines.append(" %d) %s, %s, #Components=%d" % (i, name, kind, len(comps)))
        for j, c in enumerate(comps):
            lines.append("   %s.  Value index=%d, #Derivatives=0" % (c, 1 + j))
    for n in range(nu):
        lines.append(" Node:            %d" % (n + 1))
        for _, _, _, vals in fields:
            lines.append("   " + "  ".join("%.17e" % vals[c, n] for c in range(3)))
    if mesh.p_mode == 1:
        p = np.asarray(x[3 * nu:], dtype=np.float64)
        pnode = mesh.pressure_node_u()
        lines.append(" #Fields=1")
        lines.append(" 1) HydrostaticPressure, field, rectangular cartesian, #Components=1")
        lines.append("   1.  Value index=1, #Derivatives=0")
        order = np.argsort(pnode)
        for q in order:
            lines.append(" Node:            %d" % (pnode[q] + 1))
            lines.append("   %.17e" % p[q])
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_exelem(path, mesh: Mesh, x=None, group="FiniteElasticity"):
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


def export(prefix, mesh: Mesh, x, group="FiniteElasticity"):
    """Writes prefix.exnode and prefix.exelem for the state x (host array or
    tensor in the library's dof order)."""
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    write_exnode(prefix + ".exnode", mesh, x, group)
    write_exelem(prefix + ".exelem", mesh, x, group)
    return prefix + ".exnode", prefix + ".exelem"


def read_exnode_values(path):
    """Parses the node blocks of a file written by write_exnode: returns
    {field group index: {node number: values}} for checking round trips."""
    out, block = {}, -1
    node = None
    with open(path) as f:
        for ln in f:
            s = ln.strip()
            if s.startswith("#Fields="):
                block += 1
                out[block] = {}
                node = None
            elif s.startswith("Node:"):
                node = int(s.split()[1])
                out[block][node] = []
            elif node is not None and s and s[0] in "-0123456789":
                out[block][node] += [float(v) for v in s.split()]
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
