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

    def __init__(self, mesh, source_list, nN):
        self.nN = int(nN)
        self.nSrc = len(source_list)
        q_idx, q_val = [], []
        for s, src in enumerate(source_list):
            idx, w = interp_weights(mesh, src.location)
            cur = np.asarray(src.electrode_currents() if hasattr(src, "electrode_currents") else src.current,
                             dtype=np.float64)
            if cur.size == 1 and idx.shape[0] > 1:
                cur = np.full(idx.shape[0], cur[0])
            q_idx.append(idx.ravel() + s * self.nN)
            q_val.append((cur[:, None] * w).ravel())
        qi = np.concatenate(q_idx) if q_idx else np.zeros(0, np.int64)
        qv = np.concatenate(q_val) if q_val else np.zeros(0)
        Q = sp.csr_matrix((qv, (np.zeros_like(qi), qi)), shape=(1, self.nN * max(self.nSrc, 1)))
        Q.sum_duplicates()
        self.q_idx = Q.indices.astype(np.int64)
        self.q_val = Q.data.astype(np.float64)

        rows = []
        owner = []
        for s, src in enumerate(source_list):
            for rx in src.receiver_list:
                P = rx_projection(mesh, rx).tocoo()
                fac = None
                if rx.data_type == "apparent_resistivity":
                    try:
                        fac = 1.0 / np.asarray(rx.geometric_factor[src], dtype=np.float64)
                    except KeyError:
                        raise KeyError(
                            "Receiver geometric factor has not been set, please execute survey.set_geometric_factor()"
                        )
                data = P.data * (fac[P.row] if fac is not None else 1.0)
                rows.append(sp.csr_matrix((data, (P.row, P.col + s * self.nN)), shape=(P.shape[0], self.nN * self.nSrc)))
                owner.append(np.full(P.shape[0], s, dtype=np.int64))
        self.owner = np.concatenate(owner) if owner else np.zeros(0, np.int64)
        self.P = sp.vstack(rows, format="csr") if rows else sp.csr_matrix((0, self.nN * max(self.nSrc, 1)))
        self.P.sum_duplicates()
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
