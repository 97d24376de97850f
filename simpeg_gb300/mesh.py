"""Host-side 3D tensor-mesh geometry for the nodal DC path.

The reference simulation takes a ``discretize.TensorMesh``
(``simpeg/electromagnetics/static/resistivity/simulation.py:483-501``).  The
GPU path never assembles discretize's sparse operators; it only needs the cell
widths, the origin and the node/cell/face ordering, which follow discretize's
conventions:

* nodes and cells are numbered in Fortran order (x fastest, then y, then z);
* a cell-width spec is either an int ``n`` (``n`` cells of width ``1/n``), an
  array of widths, or a list of ``(h, n)`` / ``(h, n, factor)`` tuples, where a
  factor ``f`` gives ``h*|f|**1 .. h*|f|**n`` (reversed when ``f < 0``);
* ``origin`` may be an array or a string of ``"C"`` (centred), ``"N"``
  (negative: the mesh ends at 0) and ``"0"`` per axis.

Any object with ``h`` (three width arrays) and ``origin`` (three floats) is
accepted by :class:`simpeg_gb300.resistivity.Simulation3DNodal`, so a real
``discretize.TensorMesh`` works as well as this one.
"""

from __future__ import annotations

import numpy as np

__all__ = ["TensorMesh", "unpack_widths"]


def unpack_widths(spec) -> np.ndarray:
    """Expand a discretize-style cell-width spec to a float64 array."""
    if isinstance(spec, (int, np.integer)):
        n = int(spec)
        if n <= 0:
            raise ValueError("number of cells must be positive")
        return np.full(n, 1.0 / n)
    if isinstance(spec, np.ndarray):
        return np.asarray(spec, dtype=np.float64).ravel().copy()
    out = []
    for item in spec:
        if isinstance(item, (tuple, list)):
            if len(item) == 2:
                h, n = item
                out.append(np.full(int(round(n)), float(h)))
            elif len(item) == 3:
                h, n, f = item
                n = int(round(n))
                w = float(h) * np.abs(float(f)) ** np.arange(1, n + 1)
                if f < 0:
                    w = w[::-1]
                out.append(w)
            else:
                raise ValueError(f"bad width tuple {item!r}")
        else:
            out.append(np.array([float(item)]))
    return np.concatenate(out).astype(np.float64)


class TensorMesh:
    """Minimal 3D tensor mesh with discretize's naming and ordering."""

    _meshType = "TENSOR"
    dim = 3

    def __init__(self, h, origin=None):
        if len(h) != 3:
            raise ValueError("only 3D tensor meshes are supported")
        self.h = [unpack_widths(s) for s in h]
        for w in self.h:
            if np.any(w <= 0) or not np.all(np.isfinite(w)):
                raise ValueError("cell widths must be positive and finite")
        if origin is None:
            origin = "000"
        if isinstance(origin, str):
            if len(origin) != 3:
                raise ValueError("origin string must have one letter per axis")
            o = []
            for c, w in zip(origin.upper(), self.h):
                if c == "C":
                    o.append(-w.sum() / 2.0)
                elif c == "N":
                    o.append(-w.sum())
                elif c == "0":
                    o.append(0.0)
                else:
                    raise ValueError(f"unknown origin code {c!r}")
            origin = o
        self.origin = np.asarray(origin, dtype=np.float64).reshape(3)

    # --- sizes -----------------------------------------------------------
    @property
    def shape_cells(self):
        return tuple(len(w) for w in self.h)

    @property
    def shape_nodes(self):
        return tuple(len(w) + 1 for w in self.h)

    @property
    def n_cells(self):
        nx, ny, nz = self.shape_cells
        return nx * ny * nz

    nC = n_cells

    def __len__(self):
        return self.n_cells

    @property
    def n_nodes(self):
        a, b, c = self.shape_nodes
        return a * b * c

    nN = n_nodes

    @property
    def n_edges(self):
        nx, ny, nz = self.shape_cells
        return nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz

    # --- 1D coordinates --------------------------------------------------
    def _nodes_1d(self, d):
        return self.origin[d] + np.r_[0.0, np.cumsum(self.h[d])]

    @property
    def nodes_x(self):
        return self._nodes_1d(0)

    @property
    def nodes_y(self):
        return self._nodes_1d(1)

    @property
    def nodes_z(self):
        return self._nodes_1d(2)

    def _cc_1d(self, d):
        n = self._nodes_1d(d)
        return 0.5 * (n[1:] + n[:-1])

    @property
    def cell_centers_x(self):
        return self._cc_1d(0)

    @property
    def cell_centers_y(self):
        return self._cc_1d(1)

    @property
    def cell_centers_z(self):
        return self._cc_1d(2)

    # --- full grids (Fortran order) --------------------------------------
    @staticmethod
    def _ndgrid(x, y, z):
        X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
        return np.c_[X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F")]

    @property
    def nodes(self):
        return self._ndgrid(self.nodes_x, self.nodes_y, self.nodes_z)

    gridN = nodes

    @property
    def cell_centers(self):
        return self._ndgrid(self.cell_centers_x, self.cell_centers_y, self.cell_centers_z)

    gridCC = cell_centers

    @property
    def cell_volumes(self):
        hx, hy, hz = self.h
        return np.outer(np.outer(hx, hy).ravel(order="F"), hz).ravel(order="F")

    def is_inside(self, pts, tol=1e-10):
        pts = np.atleast_2d(np.asarray(pts, dtype=np.float64))
        ok = np.ones(pts.shape[0], dtype=bool)
        for d in range(3):
            n = self._nodes_1d(d)
            ok &= (pts[:, d] >= n[0] - tol) & (pts[:, d] <= n[-1] + tol)
        return ok

    def __repr__(self):
        nx, ny, nz = self.shape_cells
        return f"TensorMesh({nx}x{ny}x{nz} cells, origin={self.origin.tolist()})"
