"""Seeded box meshes with the reference's regular-mesh numbering.

``regular_box`` restates the numbering of GENERATED_MESH_REGULAR_CREATE_FINISH
for tensor-product Lagrange bases (generated_mesh_routines.f90:1480-1600):
elements x fastest, nodes x fastest, a trilinear pressure mesh component on
the corner nodes of the displacement mesh (its user numbers taken from the
first basis, GeneratedMesh_RegularComponentNodesToUserNumbers :5043-5200, and
numbered in sorted order, MeshTopologyNodesCalculate mesh_routines.f90:
9006-9119).  The reference has no public dataset for this path: all inputs are
synthetic, from a seeded generator.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from ._lib import FE_LAW_GUCCIONE, FE_LAW_MOONEY_RIVLIN, FE_PRESSURE_ELEMENT_BASED, FE_PRESSURE_NODE_BASED

MR = FE_LAW_MOONEY_RIVLIN
GUCCIONE = FE_LAW_GUCCIONE


@dataclass
class Mesh:
    dims: tuple            # elements per direction (ex, ey, ez)
    lengths: tuple         # box edge lengths
    nxi_u: int             # 2 trilinear, 3 triquadratic displacement/geometry
    p_mode: int            # FE_PRESSURE_ELEMENT_BASED or FE_PRESSURE_NODE_BASED
    law: int
    elem_u: np.ndarray     # (ne, nxi_u**3) int32
    elem_p: np.ndarray | None  # (ne, 8) int32 for node-based pressure
    X: np.ndarray          # (3, nu) geometric field, component-major
    materials: np.ndarray  # (nmat,) or (ne, nmat)
    fibre: np.ndarray | None = None  # (3, nu) fibre/imbrication/sheet angles, radians
    grid_u: tuple = field(default=())  # nodes per direction of the u mesh

    @property
    def ne(self):
        return int(self.elem_u.shape[0])

    @property
    def nu(self):
        return int(self.X.shape[1])

    @property
    def np(self):
        return 0 if self.elem_p is None else int(self.elem_p.max()) + 1

    @property
    def n_pressure(self):
        return self.ne if self.p_mode == FE_PRESSURE_ELEMENT_BASED else self.np

    @property
    def ndofs(self):
        return 3 * self.nu + self.n_pressure

    def node_ijk(self):
        """Integer grid coordinates (i, j, k) of every u node."""
        n1, n2, _ = self.grid_u
        idx = np.arange(self.nu)
        return idx % n1, (idx // n1) % n2, idx // (n1 * n2)

    def pressure_node_u(self):
        """u node number of every pressure node (node-based pressure)."""
        out = np.zeros(self.np, dtype=np.int64)
        npe = self.nxi_u ** 3
        n1 = self.nxi_u
        corners = [(a * (n1 - 1)) + (b * (n1 - 1)) * n1 + (c * (n1 - 1)) * n1 * n1
                   for c in (0, 1) for b in (0, 1) for a in (0, 1)]
        for k, loc in enumerate(corners):
            out[self.elem_p[:, k]] = self.elem_u[:, loc]
        assert npe >= 8
        return out


def regular_box(ex, ey, ez, lengths=(1.0, 1.0, 1.0), nxi_u=2, pressure="element", law=MR,
                materials=(2.0, 6.0), perturb=0.0, seed=0, fibre=None) -> Mesh:
    """Regular box mesh.  ``perturb`` moves every node strictly inside the box
    by seeded uniform noise of +-perturb*h per coordinate (h = element edge)."""
    n1 = nxi_u
    TN = [(n1 - 1) * e + 1 for e in (ex, ey, ez)]
    ne = ex * ey * ez
    npe = n1 ** 3
    # element -> node connectivity, numbering of the reference
    e1, e2, e3 = np.meshgrid(np.arange(ex), np.arange(ey), np.arange(ez), indexing="ij")
    e1, e2, e3 = (a.transpose(2, 1, 0).ravel() for a in (e1, e2, e3))  # x fastest
    base = e1 * (n1 - 1) + e2 * (n1 - 1) * TN[0] + e3 * (n1 - 1) * TN[0] * TN[1]
    a1, a2, a3 = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    a1, a2, a3 = (a.transpose(2, 1, 0).ravel() for a in (a1, a2, a3))
    offs = a1 + a2 * TN[0] + a3 * TN[0] * TN[1]
    elem_u = (base[:, None] + offs[None, :]).astype(np.int32)
    # coordinates
    nu = TN[0] * TN[1] * TN[2]
    idx = np.arange(nu)
    ijk = [idx % TN[0], (idx // TN[0]) % TN[1], idx // (TN[0] * TN[1])]
    X = np.zeros((3, nu))
    for c in range(3):
        X[c] = ijk[c] * (lengths[c] / (TN[c] - 1))
    if perturb:
        rng = np.random.default_rng(seed)
        inner = np.ones(nu, dtype=bool)
        for c in range(3):
            inner &= (ijk[c] > 0) & (ijk[c] < TN[c] - 1)
        h = [lengths[c] / (ex, ey, ez)[c] for c in range(3)]
        for c in range(3):
            X[c, inner] += rng.uniform(-perturb * h[c], perturb * h[c], size=int(inner.sum()))
    # pressure
    elem_p = None
    p_mode = FE_PRESSURE_ELEMENT_BASED
    if pressure == "node":
        p_mode = FE_PRESSURE_NODE_BASED
        corners = [(a * (n1 - 1)) + (b * (n1 - 1)) * n1 + (c * (n1 - 1)) * n1 * n1
                   for c in (0, 1) for b in (0, 1) for a in (0, 1)]
        users = elem_u[:, corners]
        uniq = np.unique(users)
        elem_p = np.searchsorted(uniq, users).astype(np.int32)
    mats = np.asarray(materials, dtype=np.float64)
    fib = None
    if fibre is not None:
        fib = np.ascontiguousarray(np.broadcast_to(np.asarray(fibre, dtype=np.float64), (3, nu)).copy())
    return Mesh(dims=(ex, ey, ez), lengths=tuple(lengths), nxi_u=n1, p_mode=p_mode, law=law,
                elem_u=elem_u, elem_p=elem_p, X=X, materials=mats, fibre=fib, grid_u=tuple(TN))


def deformed_state(mesh: Mesh, stretch=1.1, shear=0.05, noise=0.0, pressure=-1.0, seed=1):
    """Dof vector [z_x, z_y, z_z, p] of a smooth deformation of the box:
    uniaxial stretch along x with incompressible lateral contraction, a simple
    shear in the x-y plane, optional seeded nodal noise (fraction of the node
    spacing) and a pressure field with a seeded perturbation."""
    X = mesh.X
    lat = 1.0 / np.sqrt(stretch)
    z = np.empty_like(X)
    z[0] = stretch * X[0] + shear * X[1]
    z[1] = lat * X[1]
    z[2] = lat * X[2]
    rng = np.random.default_rng(seed)
    if noise:
        hmin = min(mesh.lengths[c] / mesh.dims[c] for c in range(3)) / (mesh.nxi_u - 1)
        z += rng.uniform(-noise * hmin, noise * hmin, size=z.shape)
    p = pressure * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, size=mesh.n_pressure))
    return np.concatenate([z.ravel(), p])


def batch_meshes(n=256, seed=0, edge_range=(4, 24), length_range=(0.5, 2.0), c_range=(0.5, 10.0),
                 stretch_range=(1.0, 1.3)):
    """Seeded batch of independent box problems: per-edge element counts
    uniform in edge_range, edge lengths uniform in length_range, trilinear
    (element-constant pressure) or triquadratic (trilinear nodal pressure)
    elements with probability 1/2 each, Mooney-Rivlin c1, c2 log-uniform in
    c_range, and a uniaxial stretch uniform in stretch_range.  Returns
    (meshes, stretches)."""
    rng = np.random.default_rng(seed)
    meshes, stretches = [], []
    lc = np.log(c_range)
    for _ in range(n):
        dims = tuple(int(v) for v in rng.integers(edge_range[0], edge_range[1] + 1, size=3))
        lengths = tuple(float(v) for v in rng.uniform(*length_range, size=3))
        quad = bool(rng.integers(0, 2))
        c = np.exp(rng.uniform(*lc, size=2))
        meshes.append(regular_box(*dims, lengths=lengths, nxi_u=3 if quad else 2,
                                  pressure="node" if quad else "element", law=MR, materials=tuple(c)))
        stretches.append(float(rng.uniform(*stretch_range)))
    return meshes, stretches


def guccione_slab(ex=64, ey=64, ez=16, lengths=(40.0, 40.0, 10.0), angle_range_deg=(-60.0, 60.0), noise_deg=5.0,
                  materials=(0.88, 18.5, 3.58, 1.63), seed=0) -> Mesh:
    """Cardiac-style slab: triquadratic displacement / trilinear nodal pressure,
    transversely isotropic Guccione law (C, bf, bt, bfs), fibre angle varying
    linearly through the thickness over angle_range_deg with seeded uniform
    noise of +-noise_deg per node (imbrication and sheet angles zero)."""
    m = regular_box(ex, ey, ez, lengths=lengths, nxi_u=3, pressure="node", law=GUCCIONE, materials=materials)
    rng = np.random.default_rng(seed)
    z = m.X[2] / lengths[2]
    ang = np.deg2rad(angle_range_deg[0] + (angle_range_deg[1] - angle_range_deg[0]) * z)
    ang = ang + np.deg2rad(rng.uniform(-noise_deg, noise_deg, size=m.nu))
    m.fibre = np.stack([ang, np.zeros(m.nu), np.zeros(m.nu)])
    return m


def thick_cylinder(n_r=2, n_theta=8, n_z=1, r_in=0.5, r_out=1.0, height=1.0, law=MR, materials=(2.0, 6.0)) -> Mesh:
    """Thick-walled cylinder (tube) of triquadratic displacement / trilinear
    nodal pressure elements, the geometry of the reference's cylinder
    generated mesh (GENERATED_MESH_CYLINDER_MESH_TYPE) on which its analytic
    inflation-extension solution is posed: xi1 radial (inner surface normal
    -xi1, outer +xi1), xi2 circumferential, xi3 axial (bottom -xi3, top +xi3),
    generated_mesh_routines.f90:4193-4280.  Nodes lie on exact circles; the
    circumferential direction wraps around (the last element shares the
    nodes at theta = 0).  Nodes are numbered radial fastest, then
    circumferential, then axial (this generator's own numbering); grid_u
    holds the node counts (radial, circumferential, axial)."""
    n1 = 3
    NR, NT, NZ = 2 * n_r + 1, 2 * n_theta, 2 * n_z + 1
    nu = NR * NT * NZ
    idx = np.arange(nu)
    i, j, k = idx % NR, (idx // NR) % NT, idx // (NR * NT)
    r = r_in + (r_out - r_in) * i / (NR - 1)
    th = 2.0 * np.pi * j / NT
    X = np.stack([r * np.cos(th), r * np.sin(th), height * k / (NZ - 1)])
    er, et, ez = np.meshgrid(np.arange(n_r), np.arange(n_theta), np.arange(n_z), indexing="ij")
    er, et, ez = (a.transpose(2, 1, 0).ravel() for a in (er, et, ez))  # radial fastest
    a1, a2, a3 = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    a1, a2, a3 = (a.transpose(2, 1, 0).ravel() for a in (a1, a2, a3))
    gi = 2 * er[:, None] + a1[None, :]
    gj = (2 * et[:, None] + a2[None, :]) % NT
    gk = 2 * ez[:, None] + a3[None, :]
    elem_u = (gi + NR * gj + NR * NT * gk).astype(np.int32)
    corners = [(a * (n1 - 1)) + (b * (n1 - 1)) * n1 + (c * (n1 - 1)) * n1 * n1
               for c in (0, 1) for b in (0, 1) for a in (0, 1)]
    users = elem_u[:, corners]
    uniq = np.unique(users)
    elem_p = np.searchsorted(uniq, users).astype(np.int32)
    return Mesh(dims=(n_r, n_theta, n_z), lengths=(r_out - r_in, 2.0 * np.pi * r_in, height), nxi_u=n1,
                p_mode=FE_PRESSURE_NODE_BASED, law=law, elem_u=elem_u, elem_p=elem_p, X=X,
                materials=np.asarray(materials, dtype=np.float64), fibre=None, grid_u=(NR, NT, NZ))
