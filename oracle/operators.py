"""Sparse TensorMesh operators restated from their definitions (oracle only).

The reference calls these ``discretize`` operators (a third-party package,
``discretize>=0.12``, ``pyproject.toml:25``; not vendored in the reference):

* ``nodal_gradient``               (``resistivity/simulation.py:532,562``)
* ``get_edge_inner_product(sigma)`` and its derivative (``base/pde_simulation.py:150-162,296-321``)
* ``boundary_faces``, ``boundary_face_outward_normals``, ``project_face_to_boundary_face``,
  ``average_node_to_face``, ``average_cell_to_face``, ``face_areas``
  (``resistivity/simulation.py:588-644``)
* ``get_interpolation_matrix(loc, "N")`` (``sources.py:84``, ``receivers.py:414,493``)
* cell-centred formulation (``resistivity/simulation.py:321-480``): ``face_divergence``,
  ``get_face_inner_product(rho, invert_matrix=True)``, ``cell_gradient_weak_form_robin``,
  ``closest_points_index(loc, "CC")`` (``sources.py:79-81``) and
  ``get_interpolation_matrix(loc, "CC")`` (``receivers.py:414``)

Definitions used (3D, Fortran ordering, edges x|y|z, faces x|y|z):

* G: x-edge (i,j,k) -> (phi[i+1,j,k] - phi[i,j,k]) / hx[i]; likewise y, z.
* Me(sigma) is diagonal: Me_e = sum over cells c touching edge e of sigma_c V_c / 4
  (mid-point corner quadrature; each cell edge touches two of the eight corners).
* Boundary faces: x-faces with i in {0, nx} (the side index fastest), then y, then z.
* average_node_to_face: 1/4 on each of the face's 4 nodes.
* average_cell_to_face on a boundary face: weight 1 on the adjacent cell.
* Trilinear interpolation to a point: in each axis pick the nearest node, take
  the bracketing pair on the side of the point, clamp to the grid; a point on
  the last node gets 0.5 + 0.5 on that node.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _ddx(n):
    """(n, n+1) forward difference."""
    return sp.diags([-np.ones(n), np.ones(n)], [0, 1], shape=(n, n + 1), format="csr")


def _adj(n):
    """(n+1, n) node-from-cell adjacency: row i has ones on cells i-1, i that exist."""
    return sp.diags([np.ones(n), np.ones(n)], [0, -1], shape=(n + 1, n), format="csr")


def _kron3(a, b, c):
    """Operator acting on a Fortran-ordered 3D array: a on z, b on y, c on x."""
    return sp.kron(a, sp.kron(b, c, format="csr"), format="csr")


class MeshOps:
    """All operators of one 3D tensor mesh (widths hx, hy, hz; origin x0)."""

    def __init__(self, h, origin):
        self.hx, self.hy, self.hz = [np.asarray(w, dtype=np.float64) for w in h]
        self.origin = np.asarray(origin, dtype=np.float64)
        self.nx, self.ny, self.nz = len(self.hx), len(self.hy), len(self.hz)
        nx, ny, nz = self.nx, self.ny, self.nz
        self.nN = (nx + 1) * (ny + 1) * (nz + 1)
        self.nC = nx * ny * nz
        self.nodes_x = self.origin[0] + np.r_[0.0, np.cumsum(self.hx)]
        self.nodes_y = self.origin[1] + np.r_[0.0, np.cumsum(self.hy)]
        self.nodes_z = self.origin[2] + np.r_[0.0, np.cumsum(self.hz)]
        self.ccx = 0.5 * (self.nodes_x[1:] + self.nodes_x[:-1])
        self.ccy = 0.5 * (self.nodes_y[1:] + self.nodes_y[:-1])
        self.ccz = 0.5 * (self.nodes_z[1:] + self.nodes_z[:-1])
        self.vol = np.kron(self.hz, np.kron(self.hy, self.hx))

    @staticmethod
    def ndgrid(x, y, z):
        X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
        return np.c_[X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F")]

    @property
    def nodes(self):
        return self.ndgrid(self.nodes_x, self.nodes_y, self.nodes_z)

    # ---- gradient and edge inner product -------------------------------
    def nodal_gradient(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        Ix, Iy, Iz = sp.eye(nx + 1), sp.eye(ny + 1), sp.eye(nz + 1)
        Dx = sp.diags(1.0 / self.hx) @ _ddx(nx)
        Dy = sp.diags(1.0 / self.hy) @ _ddx(ny)
        Dz = sp.diags(1.0 / self.hz) @ _ddx(nz)
        Gx = _kron3(Iz, Iy, Dx)
        Gy = _kron3(Iz, Dy, Ix)
        Gz = _kron3(Dz, Iy, Ix)
        return sp.vstack([Gx, Gy, Gz], format="csr")

    def edge_cell_matrix(self):
        """E (nE, nC): E[e, c] = V_c / 4 if edge e belongs to cell c.

        Me(sigma) = diag(E sigma); E = d(Me u)/d sigma at u = 1.
        """
        nx, ny, nz = self.nx, self.ny, self.nz
        Ex = _kron3(_adj(nz), _adj(ny), sp.eye(nx))
        Ey = _kron3(_adj(nz), sp.eye(ny), _adj(nx))
        Ez = _kron3(sp.eye(nz), _adj(ny), _adj(nx))
        return (sp.vstack([Ex, Ey, Ez], format="csr") @ sp.diags(self.vol / 4.0)).tocsr()

    def average_node_to_cell(self):
        """(nC, nN): the mean of each cell's 8 corner nodes (discretize ``aveN2CC`` on a tensor mesh)."""
        nx, ny, nz = self.nx, self.ny, self.nz

        def av(n):
            return sp.diags([0.5, 0.5], [0, 1], shape=(n, n + 1))

        return _kron3(av(nz), av(ny), av(nx)).tocsr()

    # ---- boundary ------------------------------------------------------
    def boundary_faces(self):
        """Centres, outward normals, areas, adjacent cell and 4 nodes of every boundary face."""
        nx, ny, nz = self.nx, self.ny, self.nz
        Nx, Ny = nx + 1, ny + 1
        cents, norms, areas, cells, nodes4, kind = [], [], [], [], [], []

        def node(i, j, k):
            return i + Nx * (j + Ny * k)

        def cell(i, j, k):
            return i + nx * (j + ny * k)

        # x-faces: (side, j, k), side fastest
        for k in range(nz):
            for j in range(ny):
                for s, i in ((0, 0), (1, nx)):
                    cents.append((self.nodes_x[i], self.ccy[j], self.ccz[k]))
                    norms.append((-1.0 if s == 0 else 1.0, 0.0, 0.0))
                    areas.append(self.hy[j] * self.hz[k])
                    cells.append(cell(0 if s == 0 else nx - 1, j, k))
                    nodes4.append([node(i, j, k), node(i, j + 1, k), node(i, j, k + 1), node(i, j + 1, k + 1)])
                    kind.append(("x", s))
        # y-faces: (i, side, k)
        for k in range(nz):
            for s, j in ((0, 0), (1, ny)):
                for i in range(nx):
                    cents.append((self.ccx[i], self.nodes_y[j], self.ccz[k]))
                    norms.append((0.0, -1.0 if s == 0 else 1.0, 0.0))
                    areas.append(self.hx[i] * self.hz[k])
                    cells.append(cell(i, 0 if s == 0 else ny - 1, k))
                    nodes4.append([node(i, j, k), node(i + 1, j, k), node(i, j, k + 1), node(i + 1, j, k + 1)])
                    kind.append(("y", s))
        # z-faces: (i, j, side)
        for s, k in ((0, 0), (1, nz)):
            for j in range(ny):
                for i in range(nx):
                    cents.append((self.ccx[i], self.ccy[j], self.nodes_z[k]))
                    norms.append((0.0, 0.0, -1.0 if s == 0 else 1.0))
                    areas.append(self.hx[i] * self.hy[j])
                    cells.append(cell(i, j, 0 if s == 0 else nz - 1))
                    nodes4.append([node(i, j, k), node(i + 1, j, k), node(i, j + 1, k), node(i + 1, j + 1, k)])
                    kind.append(("z", s))
        return dict(
            centers=np.array(cents), normals=np.array(norms), areas=np.array(areas),
            cells=np.array(cells), nodes=np.array(nodes4), kind=kind,
        )

    # ---- faces (cell-centred formulation) --------------------------------
    @property
    def n_faces(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        return ((nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1))

    def face_areas(self):
        """Areas of the x-, y- and z-faces (Fortran order within each)."""
        nx, ny, nz = self.nx, self.ny, self.nz
        ax = np.kron(self.hz, np.kron(self.hy, np.ones(nx + 1)))
        ay = np.kron(self.hz, np.kron(np.ones(ny + 1), self.hx))
        az = np.kron(np.ones(nz + 1), np.kron(self.hy, self.hx))
        return np.r_[ax, ay, az]

    def face_divergence_raw(self):
        """D (nC, nF) = V * face_divergence: D[c, f] = +A_f on the cell's + side, -A_f on its - side."""
        nx, ny, nz = self.nx, self.ny, self.nz
        Dx = _kron3(sp.eye(nz), sp.eye(ny), _ddx(nx))
        Dy = _kron3(sp.eye(nz), _ddx(ny), sp.eye(nx))
        Dz = _kron3(_ddx(nz), sp.eye(ny), sp.eye(nx))
        return (sp.hstack([Dx, Dy, Dz], format="csr") @ sp.diags(self.face_areas())).tocsr()

    def face_cell_matrix(self):
        """F (nF, nC): F[f, c] = V_c / 2 for the (one or two) cells holding face f.

        The face inner product of an isotropic property p on a tensor mesh is diagonal:
        Mf(p) = diag(F p) (each face gets V_c/8 from each of the 4 cell corners it touches)."""
        nx, ny, nz = self.nx, self.ny, self.nz
        Fx = _kron3(sp.eye(nz), sp.eye(ny), _adj(nx))
        Fy = _kron3(sp.eye(nz), _adj(ny), sp.eye(nx))
        Fz = _kron3(_adj(nz), sp.eye(ny), sp.eye(nx))
        return (sp.vstack([Fx, Fy, Fz], format="csr") @ sp.diags(self.vol / 2.0)).tocsr()

    def boundary_face_index(self):
        """Global face index of every boundary face, in the order of :meth:`boundary_faces`."""
        nx, ny, nz = self.nx, self.ny, self.nz
        nfx, nfy, _ = self.n_faces
        out = []
        for k in range(nz):
            for j in range(ny):
                for i in (0, nx):
                    out.append(i + (nx + 1) * (j + ny * k))
        for k in range(nz):
            for j in (0, ny):
                for i in range(nx):
                    out.append(nfx + i + nx * (j + (ny + 1) * k))
        for k in (0, nz):
            for j in range(ny):
                for i in range(nx):
                    out.append(nfx + nfy + i + nx * (j + ny * k))
        return np.array(out, dtype=np.int64)

    @property
    def cell_centers(self):
        return self.ndgrid(self.ccx, self.ccy, self.ccz)

    def closest_cell(self, locs):
        """Index of the nearest cell centre of each point (the first one on ties)."""
        locs = np.atleast_2d(np.asarray(locs, dtype=np.float64))
        cc = self.cell_centers
        return np.array([int(np.argmin(((cc - p) ** 2).sum(axis=1))) for p in locs], dtype=np.int64)

    def interpolation_matrix_cc(self, locs):
        """Trilinear interpolation from the cell centres (same per-axis rule as the nodes: outside
        the outermost centres the nearest centre gets weights 0.5 + 0.5); points outside the mesh
        raise."""
        locs = np.atleast_2d(np.asarray(locs, dtype=np.float64))
        tol = 1e-10
        for d, nd in enumerate((self.nodes_x, self.nodes_y, self.nodes_z)):
            if np.any(locs[:, d] < nd[0] - tol) or np.any(locs[:, d] > nd[-1] + tol):
                raise ValueError("Points outside of mesh")
        nx, ny = self.nx, self.ny
        rows, cols, vals = [], [], []
        for r, p in enumerate(locs):
            ix = self._interp1(self.ccx, p[0])
            iy = self._interp1(self.ccy, p[1])
            iz = self._interp1(self.ccz, p[2])
            for a, wa in ((ix[0], ix[2]), (ix[1], ix[3])):
                for b, wb in ((iy[0], iy[2]), (iy[1], iy[3])):
                    for c, wc in ((iz[0], iz[2]), (iz[1], iz[3])):
                        rows.append(r)
                        cols.append(a + nx * (b + ny * c))
                        vals.append(wa * wb * wc)
        return sp.csr_matrix((vals, (rows, cols)), shape=(locs.shape[0], self.nC))

    # ---- interpolation -------------------------------------------------
    @staticmethod
    def _interp1(nodes, x):
        im = int(np.argmin(np.abs(nodes - x)))
        if x - nodes[im] >= 0:
            i1, i2 = im, im + 1
        else:
            i1, i2 = im - 1, im
        n = nodes.size
        i1 = max(min(i1, n - 1), 0)
        i2 = max(min(i2, n - 1), 0)
        if i1 == i2:
            return i1, i2, 0.5, 0.5
        h = nodes[i2] - nodes[i1]
        return i1, i2, 1.0 - (x - nodes[i1]) / h, 1.0 - (nodes[i2] - x) / h

    def interpolation_matrix(self, locs):
        locs = np.atleast_2d(np.asarray(locs, dtype=np.float64))
        tol = 1e-10
        for d, nd in enumerate((self.nodes_x, self.nodes_y, self.nodes_z)):
            if np.any(locs[:, d] < nd[0] - tol) or np.any(locs[:, d] > nd[-1] + tol):
                raise ValueError("Points outside of mesh")
        Nx, Ny = self.nx + 1, self.ny + 1
        rows, cols, vals = [], [], []
        for r, p in enumerate(locs):
            ix = self._interp1(self.nodes_x, p[0])
            iy = self._interp1(self.nodes_y, p[1])
            iz = self._interp1(self.nodes_z, p[2])
            for a, wa in ((ix[0], ix[2]), (ix[1], ix[3])):
                for b, wb in ((iy[0], iy[2]), (iy[1], iy[3])):
                    for c, wc in ((iz[0], iz[2]), (iz[1], iz[3])):
                        rows.append(r)
                        cols.append(a + Nx * (b + Ny * c))
                        vals.append(wa * wb * wc)
        return sp.csr_matrix((vals, (rows, cols)), shape=(locs.shape[0], self.nN))
