"""Robin boundary weights of the nodal DC operator.

Restates ``Simulation3DNodal.setBC`` (``simpeg/electromagnetics/static/
resistivity/simulation.py:573-644``) in the packed per-side form the CUDA
engine consumes.  For every boundary face f (outward normal n_f, centre c_f,
area A_f) that is not a surface face:

    alpha_f = (r_hat . n_f) / r,   r = c_f - p,
    p = (median node x, median node y, max node z)

and alpha_f = 0 on surface faces (by default the top z-faces).  The Robin
term of A is ``AvgBC @ sigma`` with ``AvgBC = AvgN2Fb^T diag(alpha*A) AvgCC2Fb``:
each boundary face adds ``0.25 * alpha_f * A_f * sigma(cell adjacent to f)`` to
each of its four nodes.  This module returns ``0.25 * alpha_f * A_f`` per face,
packed as [x-lo (ny*nz), x-hi, y-lo (nx*nz), y-hi, z-lo (nx*ny), z-hi], each side
in Fortran order of its two in-plane cell indices.

``surface_faces`` (optional) is a bool array over discretize's boundary-face
order: x-faces (side fastest, then y, then z cell index), then y-faces
(x index, side, z), then z-faces (x, y, side).
"""

from __future__ import annotations

import numpy as np


def _geom(mesh):
    h = [np.asarray(w, dtype=np.float64) for w in mesh.h]
    o = np.asarray(mesh.origin, dtype=np.float64)
    nodes = [o[d] + np.r_[0.0, np.cumsum(h[d])] for d in range(3)]
    cc = [0.5 * (n[1:] + n[:-1]) for n in nodes]
    return h, nodes, cc


def source_point(mesh):
    _, nodes, _ = _geom(mesh)
    return np.array([np.median(nodes[0]), np.median(nodes[1]), nodes[2].max()])


def _side_faces(mesh):
    """Per side: (centres (m,3), normal (3,), areas (m,)) in packed order."""
    h, nodes, cc = _geom(mesh)
    hx, hy, hz = h
    out = []
    # x sides: in-plane indices (j, k), j fastest
    for s, x in ((0, nodes[0][0]), (1, nodes[0][-1])):
        J, K = np.meshgrid(np.arange(len(hy)), np.arange(len(hz)), indexing="ij")
        J, K = J.ravel(order="F"), K.ravel(order="F")
        c = np.c_[np.full(J.size, x), cc[1][J], cc[2][K]]
        out.append((c, np.array([-1.0 if s == 0 else 1.0, 0, 0]), hy[J] * hz[K]))
    for s, y in ((0, nodes[1][0]), (1, nodes[1][-1])):
        I, K = np.meshgrid(np.arange(len(hx)), np.arange(len(hz)), indexing="ij")
        I, K = I.ravel(order="F"), K.ravel(order="F")
        c = np.c_[cc[0][I], np.full(I.size, y), cc[2][K]]
        out.append((c, np.array([0, -1.0 if s == 0 else 1.0, 0]), hx[I] * hz[K]))
    for s, z in ((0, nodes[2][0]), (1, nodes[2][-1])):
        I, J = np.meshgrid(np.arange(len(hx)), np.arange(len(hy)), indexing="ij")
        I, J = I.ravel(order="F"), J.ravel(order="F")
        c = np.c_[cc[0][I], cc[1][J], np.full(I.size, z)]
        out.append((c, np.array([0, 0, -1.0 if s == 0 else 1.0]), hx[I] * hy[J]))
    return out


def surface_mask_by_side(mesh, surface_faces=None):
    """Bool mask per packed side; default marks the top (z-hi) side."""
    nx, ny, nz = (len(w) for w in mesh.h)
    sizes = [ny * nz, ny * nz, nx * nz, nx * nz, nx * ny, nx * ny]
    if surface_faces is None:
        return [np.zeros(n, bool) if s != 5 else np.ones(n, bool) for s, n in enumerate(sizes)]
    sf = np.asarray(surface_faces)
    n_bf = sum(sizes)
    if sf.dtype != bool:
        b = np.zeros(n_bf, bool)
        b[sf.astype(int)] = True
        sf = b
    if sf.shape != (n_bf,):
        raise ValueError(f"surface_faces must have one entry per boundary face ({n_bf})")
    # discretize order -> packed sides
    nxf = 2 * ny * nz
    nyf = 2 * nx * nz
    fx = sf[:nxf].reshape(2, ny, nz, order="F")
    fy = sf[nxf:nxf + nyf].reshape(nx, 2, nz, order="F")
    fz = sf[nxf + nyf:].reshape(nx, ny, 2, order="F")
    return [
        fx[0].ravel(order="F"), fx[1].ravel(order="F"),
        fy[:, 0].ravel(order="F"), fy[:, 1].ravel(order="F"),
        fz[:, :, 0].ravel(order="F"), fz[:, :, 1].ravel(order="F"),
    ]


def robin_face_weights(mesh, surface_faces=None):
    """Packed 0.25*alpha*area over the six sides (float64)."""
    p = source_point(mesh)
    masks = surface_mask_by_side(mesh, surface_faces)
    parts = []
    for (c, n, a), surf in zip(_side_faces(mesh), masks):
        r_vec = c - p
        r = np.linalg.norm(r_vec, axis=1)
        alpha = np.zeros(r.size)
        ok = ~surf
        alpha[ok] = (r_vec[ok] @ n) / r[ok] ** 2
        parts.append(0.25 * alpha * a)
    return np.concatenate(parts)


# ---------------------------------------------------------------- cell-centred formulation
def cc_boundary_weights(mesh, bc_type="Robin", surface_faces=None):
    """Boundary terms of the cell-centred operator ``Div MfRhoI (Div^T - B)``
    (``resistivity/simulation.py:421-480`` with ``cell_gradient_weak_form_robin``), packed
    per side like :func:`robin_face_weights`: ``bw_f = (1 - a_f) A_f^2 / (V_c / 2)``, so that
    boundary face f adds ``bw_f / rho_c`` to the diagonal of its cell c.

    ``a_f = (1 / h_f) / (alpha_f + 1 / h_f)`` is the ghost-point factor of the Robin condition
    ``alpha phi + d phi / dn = 0`` (beta = 1, gamma = 0), h_f the distance from the cell centre
    to the face (half the cell's width normal to it), alpha_f as in :func:`robin_face_weights`
    (zero on the surface faces).  Dirichlet (phi = 0 on the boundary, the formulation's natural
    condition): a_f = 0.  Neumann: None (no boundary term)."""
    if bc_type == "Mixed":
        bc_type = "Robin"
    if bc_type == "Neumann":
        return None
    h, _, _ = _geom(mesh)
    hn = [h[0][0], h[0][-1], h[1][0], h[1][-1], h[2][0], h[2][-1]]  # normal width of the boundary cells
    p = source_point(mesh)
    masks = surface_mask_by_side(mesh, surface_faces)
    parts = []
    for side, ((c, n, a), surf) in enumerate(zip(_side_faces(mesh), masks)):
        if bc_type == "Dirichlet":
            one_minus_a = np.ones(a.size)
        elif bc_type == "Robin":
            r_vec = c - p
            r = np.linalg.norm(r_vec, axis=1)
            alpha = np.zeros(r.size)
            ok = ~surf
            alpha[ok] = (r_vec[ok] @ n) / r[ok] ** 2
            hf = 0.5 * hn[side]
            one_minus_a = alpha * hf / (alpha * hf + 1.0)
        else:
            raise ValueError(f"bc_type must be Dirichlet, Neumann, Robin or Mixed, not {bc_type!r}")
        parts.append(one_minus_a * 2.0 * a / hn[side])  # A^2 / (V/2) = 2 A / h_n
    return np.concatenate(parts)


def cell_centre_grid(mesh):
    """The tensor mesh whose nodes are the cell centres of ``mesh`` (widths: the distances
    between neighbouring centres), on which the cell-centred unknowns are solved."""
    from ..mesh import TensorMesh

    h, _, cc = _geom(mesh)
    if min(len(w) for w in h) < 2:
        raise ValueError("the cell-centred simulation needs at least 2 cells per axis")
    return TensorMesh([0.5 * (w[1:] + w[:-1]) for w in h], origin=[c[0] for c in cc])


def cc_grid_face_weights(mesh, bc_type="Robin"):
    """Robin face weights of the cell-centre grid for the coarse multigrid levels (None for
    Neumann): the nodal Robin weights of that grid, or for Dirichlet a Robin condition of
    alpha = 2 / h_n (phi = 0 half a boundary cell beyond the outermost centres) on every side."""
    if bc_type == "Mixed":
        bc_type = "Robin"
    if bc_type == "Neumann":
        return None
    grid = cell_centre_grid(mesh)
    if bc_type == "Robin":
        return robin_face_weights(grid)
    h, _, _ = _geom(mesh)
    hn = [h[0][0], h[0][-1], h[1][0], h[1][-1], h[2][0], h[2][-1]]
    return np.concatenate([0.25 * (2.0 / hn[s]) * a for s, (_, _, a) in enumerate(_side_faces(grid))])
