"""Electrode -> node tables for sources and receivers (host, integer-exact).

``BaseSrc.eval`` (``sources.py:64-88``) and ``Rx.getP`` (``receivers.py:379-424,
461-498``) both use ``mesh.get_interpolation_matrix(loc, "N")``: trilinear
weights of the eight nodes around a point.  Per axis the rule is: take the
node nearest to the coordinate (first one on ties); the bracketing pair is
that node and the next one if the point is at or above it, else the previous
one and it; clamp both to the grid; if they coincide (point on the last node)
each gets weight 0.5; otherwise w1 = 1 - (x - x1)/h, w2 = 1 - (x2 - x)/h.
Points outside the mesh raise ``ValueError`` as discretize does.

The GPU never sees a dense ``(n_loc, nN)`` row: it gets CSR tables of
(node index, weight) that the kernels in ``include/dcgpu.h`` gather/scatter.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import receivers as Rx
from . import sources as Src


def _axis_interp(nodes, x):
    x = np.asarray(x, dtype=np.float64)
    n = nodes.size
    im = np.argmin(np.abs(nodes[None, :] - x[:, None]), axis=1)
    up = (x - nodes[im]) >= 0
    i1 = np.where(up, im, im - 1)
    i2 = np.where(up, im + 1, im)
    i1 = np.clip(i1, 0, n - 1)
    i2 = np.clip(i2, 0, n - 1)
    same = i1 == i2
    h = np.where(same, 1.0, nodes[i2] - nodes[i1])
    w1 = np.where(same, 0.5, 1.0 - (x - nodes[i1]) / h)
    w2 = np.where(same, 0.5, 1.0 - (nodes[i2] - x) / h)
    return i1, i2, w1, w2


def node_coords(mesh):
    o = np.asarray(mesh.origin, dtype=np.float64)
    return [o[d] + np.r_[0.0, np.cumsum(np.asarray(mesh.h[d], dtype=np.float64))] for d in range(3)]


def interp_weights(mesh, locs, tol=1e-10):
    """(n, 8) node indices and (n, 8) weights of the trilinear interpolation to ``locs``."""
    locs = np.atleast_2d(np.asarray(locs, dtype=np.float64))
    if locs.shape[1] != 3:
        raise ValueError("electrode locations must be (n, 3)")
    nodes = node_coords(mesh)
    for d in range(3):
        if np.any(locs[:, d] < nodes[d][0] - tol) or np.any(locs[:, d] > nodes[d][-1] + tol):
            raise ValueError("Points outside of mesh")
    Nx, Ny = nodes[0].size, nodes[1].size
    ax = [_axis_interp(nodes[d], locs[:, d]) for d in range(3)]
    idx = np.empty((locs.shape[0], 8), dtype=np.int64)
    w = np.empty((locs.shape[0], 8), dtype=np.float64)
    c = 0
    for a in (0, 1):
        for b in (0, 1):
            for e in (0, 1):
                ii, jj, kk = ax[0][a], ax[1][b], ax[2][e]
                idx[:, c] = ii + Nx * (jj + Ny * kk)
                w[:, c] = ax[0][2 + a] * ax[1][2 + b] * ax[2][2 + e]
                c += 1
    return idx, w


def cc_coords(mesh):
    return [0.5 * (n[1:] + n[:-1]) for n in node_coords(mesh)]


def cc_interp_weights(mesh, locs, tol=1e-10):
    """(n, 8) cell indices and weights of the interpolation from the cell centres to ``locs``
    (``get_interpolation_matrix(loc, "CC")``): the per-axis rule of :func:`interp_weights` on the
    cell-centre coordinates, so beyond the outermost centre the nearest one takes the value; points
    outside the mesh raise."""
    locs = np.atleast_2d(np.asarray(locs, dtype=np.float64))
    if locs.shape[1] != 3:
        raise ValueError("electrode locations must be (n, 3)")
    nodes = node_coords(mesh)
    for d in range(3):
        if np.any(locs[:, d] < nodes[d][0] - tol) or np.any(locs[:, d] > nodes[d][-1] + tol):
            raise ValueError("Points outside of mesh")
    cc = cc_coords(mesh)
    nx, ny = cc[0].size, cc[1].size
    ax = [_axis_interp(cc[d], locs[:, d]) for d in range(3)]
    idx = np.empty((locs.shape[0], 8), dtype=np.int64)
    w = np.empty((locs.shape[0], 8), dtype=np.float64)
    c = 0
    for a in (0, 1):
        for b in (0, 1):
            for e in (0, 1):
                idx[:, c] = ax[0][a] + nx * (ax[1][b] + ny * ax[2][e])
                w[:, c] = ax[0][2 + a] * ax[1][2 + b] * ax[2][2 + e]
                c += 1
    return idx, w


def closest_cells(mesh, locs):
    """Index of the cell centre nearest to each point (``closest_points_index(loc, "CC")``; ties go
    to the lowest index, which on a tensor grid is the per-axis nearest centre, lowest first)."""
    locs = np.atleast_2d(np.asarray(locs, dtype=np.float64))
    cc = cc_coords(mesh)
    ijk = [np.argmin(np.abs(cc[d][None, :] - locs[:, d][:, None]), axis=1) for d in range(3)]
    return (ijk[0] + cc[0].size * (ijk[1] + cc[1].size * ijk[2])).astype(np.int64)


def interpolation_matrix(mesh, locs):
    idx, w = interp_weights(mesh, locs)
    n = idx.shape[0]
    nN = int(np.prod([len(h) + 1 for h in mesh.h]))
    return sp.csr_matrix((w.ravel(), (np.repeat(np.arange(n), 8), idx.ravel())), shape=(n, nN))


def rx_projection(mesh, rx):
    """P of one receiver: interp(M) - interp(N) (Dipole) or interp(M) (Pole)."""
    if isinstance(rx, Rx.Dipole) or isinstance(getattr(rx, "locations", None), (list, tuple)):
        return (interpolation_matrix(mesh, rx.locations[0]) - interpolation_matrix(mesh, rx.locations[1])).tocsr()
    return interpolation_matrix(mesh, rx.locations).tocsr()


class SurveyTables:
    """All index tables of one survey on one mesh.

    * ``q_idx, q_val``: unique flat indices ``s*nN + node`` of the source term
      (column-major (nN, nSrc)) and their values ``sum_e I_e w_e``.
    * ``P``: CSR (nD, nSrc*nN) -- datum d gathers ``sum w * u[s(d)*nN + node]``,
      apparent-resistivity scaling folded in.
    * ``PT``: the transpose restricted to its nonzero rows: ``PT_out`` are the
      flat target indices, ``PT_ptr``/``PT_idx``/``PT_w`` the CSR over data.
    """

    def __init__(self, mesh, source_list, nN, grid="N"):
        """``grid`` "N": nodal unknowns (trilinear electrodes); "CC": cell-centred unknowns (sources
        at the nearest cell centre, ``sources.py:79-81``; receivers interpolated from the centres)."""
        self.nN = int(nN)
        self.nSrc = len(source_list)
        if grid not in ("N", "CC"):
            raise ValueError("grid must be 'N' or 'CC'")
        interp = interp_weights if grid == "N" else cc_interp_weights
        # source term: every electrode of every source in one interpolation
        locs, curs, sidx = [], [], []
        for s, src in enumerate(source_list):
            L = np.atleast_2d(np.asarray(src.location, dtype=np.float64))
            cur = np.asarray(src.electrode_currents() if hasattr(src, "electrode_currents") else src.current,
                             dtype=np.float64).ravel()
            if cur.size == 1 and L.shape[0] > 1:
                cur = np.full(L.shape[0], cur[0])
            locs.append(L)
            curs.append(cur)
            sidx.append(np.full(L.shape[0], s, dtype=np.int64))
        if locs and grid == "CC":
            # q[closest cell] = current: an assignment, so a later electrode in the same cell wins
            cells = closest_cells(mesh, np.concatenate(locs))
            keys = np.concatenate(sidx) * self.nN + cells
            vals = np.concatenate(curs)
            last = {}
            for kk, vv in zip(keys.tolist(), vals.tolist()):
                last[kk] = vv
            qi = np.fromiter(last.keys(), dtype=np.int64, count=len(last))
            qv = np.fromiter(last.values(), dtype=np.float64, count=len(last))
        elif locs:
            idx, w = interp_weights(mesh, np.concatenate(locs))
            qi = (idx + (np.concatenate(sidx) * self.nN)[:, None]).ravel()
            qv = (np.concatenate(curs)[:, None] * w).ravel()
        else:
            qi, qv = np.zeros(0, np.int64), np.zeros(0)
        Q = sp.csr_matrix((qv, (np.zeros_like(qi), qi)), shape=(1, self.nN * max(self.nSrc, 1)))
        Q.sum_duplicates()
        self.q_idx = Q.indices.astype(np.int64)
        self.q_val = Q.data.astype(np.float64)

        # receivers: all M electrodes in one interpolation, all N electrodes in another; a datum's
        # row is interp(M) - interp(N) (duplicates summed), then scaled by 1/geometric factor for
        # apparent resistivity
        m_locs, m_rows, m_src, n_locs, n_rows, n_src, fac, owner = [], [], [], [], [], [], [], []
        d0 = 0
        for s, src in enumerate(source_list):
            for rx in src.receiver_list:
                dipole = isinstance(rx, Rx.Dipole) or isinstance(getattr(rx, "locations", None), (list, tuple))
                M = np.atleast_2d(np.asarray(rx.locations[0] if dipole else rx.locations, dtype=np.float64))
                n = M.shape[0]
                rows = np.arange(d0, d0 + n, dtype=np.int64)
                m_locs.append(M)
                m_rows.append(rows)
                m_src.append(np.full(n, s, dtype=np.int64))
                if dipole:
                    n_locs.append(np.atleast_2d(np.asarray(rx.locations[1], dtype=np.float64)))
                    n_rows.append(rows)
                    n_src.append(np.full(n, s, dtype=np.int64))
                f = np.ones(n)
                if rx.data_type == "apparent_resistivity":
                    try:
                        f = 1.0 / np.asarray(rx.geometric_factor[src], dtype=np.float64)
                    except KeyError:
                        raise KeyError(
                            "Receiver geometric factor has not been set, please execute survey.set_geometric_factor()"
                        )
                fac.append(f)
                owner.append(np.full(n, s, dtype=np.int64))
                d0 += n
        self.owner = np.concatenate(owner) if owner else np.zeros(0, np.int64)
        ncol = self.nN * max(self.nSrc, 1)
        if d0:
            parts_r, parts_c, parts_v = [], [], []
            for locs_, rows_, src_, sign in ((m_locs, m_rows, m_src, 1.0), (n_locs, n_rows, n_src, -1.0)):
                if not locs_:
                    continue
                idx, w = interp(mesh, np.concatenate(locs_))
                parts_r.append(np.repeat(np.concatenate(rows_), 8))
                parts_c.append((idx + (np.concatenate(src_) * self.nN)[:, None]).ravel())
                parts_v.append(sign * w.ravel())
            P = sp.csr_matrix((np.concatenate(parts_v), (np.concatenate(parts_r), np.concatenate(parts_c))),
                              shape=(d0, ncol))
            P.sum_duplicates()
            P.eliminate_zeros()
            P.data = P.data * np.concatenate(fac)[np.repeat(np.arange(d0), np.diff(P.indptr))]
            self.P = P
        else:
            self.P = sp.csr_matrix((0, ncol))
        self.nD = self.P.shape[0]
        # transpose restricted to its nonzero rows, built from P's entries (sorted by
        # column, then datum) without materialising the nSrc*nN-row CSR
        Pc = self.P.tocoo()
        order = np.lexsort((Pc.row, Pc.col))
        cols, data_idx, vals = Pc.col[order].astype(np.int64), Pc.row[order].astype(np.int64), Pc.data[order]
        self.PT_out, starts = np.unique(cols, return_index=True)
        self.PT_out = self.PT_out.astype(np.int64)
        self.PT_ptr = np.r_[starts, cols.size].astype(np.int64)
        self.PT_idx = data_idx
        self.PT_w = vals.astype(np.float64)
        self.P_ptr = self.P.indptr.astype(np.int64)
        self.P_idx = self.P.indices.astype(np.int64)
        self.P_w = self.P.data.astype(np.float64)
