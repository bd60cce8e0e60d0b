"""Export of the geometric and dependent fields in the CMISS exnode/exelem text format.

The reference writes its fields with FIELD_IO_NODES_EXPORT / FIELD_IO_ELEMENTS_EXPORT
(field_IO_routines.f90:6158-6245) through the C writer in src/FieldExport.c
(group header :233, "Shape.  Dimension" :243, "#Scale factor sets" :263,
interpolation labels "l.Lagrange" / "q.Lagrange" and ", no modify, standard
node based." :300-375, "coordinate, rectangular cartesian" :593, "#Nodes" /
"#Fields" :641-647, " Node:" :1029, " Element: e 0 0" :814, "Nodes:" :833).
This module writes the same files for the fields of one equations set, so a
converged state can be compared with, or loaded next to, output of the
reference: the geometric field and the dependent field (deformed position and
hydrostatic pressure, nodal on the element corners or element-constant).
Both files are byte-identical to the reference writer's for the same state.
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


def _element_bases(mesh: Mesh):
    """The element components in field order (geometric x, y, z; dependent
    1-4) as (field label, component label, basis key or None for an
    element-constant component) and the bases by key: (per-xi label, local
    u-node positions of the basis' nodes within the element)."""
    n1 = mesh.nxi_u
    bases = {"u": (_basis_label(n1), list(range(n1 ** 3)))}
    comps = [("G", c, "u") for c in ("x", "y", "z")] + [("D", str(c), "u") for c in (1, 2, 3)]
    if mesh.p_mode == 1:
        corners = [(a * (n1 - 1)) + (b * (n1 - 1)) * n1 + (c * (n1 - 1)) * n1 * n1
                   for c in (0, 1) for b in (0, 1) for a in (0, 1)]
        bases["p"] = (_basis_label(2), corners)
        comps.append(("D", "4", "p"))
    else:
        comps.append(("D", "4", None))
    return comps, bases


def write_exelem(path, mesh: Mesh, x=None, group="Region"):
    """Element file of the two fields, in the layout the reference's element
    export writes (FIELD_IO_EXPORT_ELEMENTS_INTO_LOCAL_FILE and its header,
    field_IO_routines.f90:2519-3853, through src/FieldExport.c): every element
    of a mesh shares one header, written before the first element; one
    scale-factor set per distinct basis (the default arithmetic-mean scaling:
    unit factors for Lagrange bases), numbered in component order, the first
    index of a later set being the reference's sum of the set sizes up to and
    including it, minus one; per node-based component its nodes as positions in
    the element's node list (the u basis), per element-constant component a
    grid-based line; per element its number, the element-constant values
    (element-based pressure from x), the u nodes and the scale factors of
    every set."""
    comps, bases = _element_bases(mesh)
    keys = []
    for _, _, k in comps:
        if k is not None and k not in keys:
            keys.append(k)
    size = {k: len(bases[k][1]) for k in keys}
    lines = [" Group name: %s" % group, " Shape.  Dimension=3", " #Scale factor sets= %d" % len(keys)]
    lines += [" %s, #Scale factors=%d" % (bases[k][0], size[k]) for k in keys]
    lines += [" #Nodes=           %d" % len(bases["u"][1]), " #Fields=2"]
    names = {"G": " 1) Geometry, coordinate, rectangular cartesian, #Components=3",
             "D": " 2) Dependent, field,  rectangular cartesian, #Components=4"}
    prev = None
    for field, label, k in comps:
        if field != prev:
            lines.append(names[field])
            prev = field
        if k is None:
            lines.append("   %s.   %s, no modify, grid based." % (label, "*".join(["constant"] * 3)))
            lines.append("     #xi1=0, #xi2=0, #xi3=0")
            continue
        lines.append("   %s.   %s, no modify, standard node based." % (label, bases[k][0]))
        nodes = bases[k][1]
        set_no = keys.index(k) + 1
        first = 0 if set_no == 1 else sum(size[q] for q in keys[:set_no]) - 1
        lines.append("     #Nodes= %d" % len(nodes))
        for i, a in enumerate(nodes):
            lines.append(" %5d.  #Values=1" % (a + 1))
            lines.append("      Value indices:     1")
            lines.append("      Scale factor indices: %4d" % (first + 1 + i))
    p = None
    if mesh.p_mode == 0 and x is not None:
        p = np.asarray(x[3 * mesh.nu:], dtype=np.float64)
    ones = {k: "  " + "   %.16E" % 1.0 * size[k] for k in keys}
    for e in range(mesh.ne):
        lines.append(" Element:            %d 0 0" % (e + 1))
        if p is not None:
            lines.append("   Values:")
            lines.append("     %.16E" % p[e])
        lines.append("   Nodes:")
        lines.append("".join("  %10d" % (n + 1) for n in mesh.elem_u[e]))
        lines.append("   Scale factors:")
        lines += [ones[k] for k in keys]
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
