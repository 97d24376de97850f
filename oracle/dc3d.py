"""CPU restatement of ``Simulation3DNodal`` (oracle only -- test infrastructure).

Follows, function by function:

* ``setBC`` (Robin)          ``simpeg/electromagnetics/static/resistivity/simulation.py:573-644``
* ``getA``                   ``simulation.py:523-555`` (Neumann row-0 pin at ``:535-540``)
* ``getADeriv``              ``simulation.py:557-571`` with ``MeSigmaDeriv``
                             (``simpeg/base/pde_simulation.py:296-321``) and
                             ``_inner_mat_mul_op`` (``pde_simulation.py:15-83``)
* ``getSourceTerm``          ``simulation.py:265-289`` / ``sources.py:64-88``
* ``fields``                 ``simulation.py:100-113`` (solver = SuperLU as ``SolverLU``)
* ``dpred``                  ``simpeg/simulation.py:161-196`` / ``receivers.py:156-192``
* ``Jvec``                   ``simulation.py:156-187``
* ``Jtvec`` / ``_Jtvec``     ``simulation.py:189-263``
* ``getJ``/``getJtJdiag``    ``simulation.py:115-121,137-154``
* ``Fields3DNodal`` e, j, charge, charge_density
                             ``resistivity/fields.py:214-253``

The per-source loops are vectorised over sources (one multi-RHS solve), which
changes only the floating-point summation order.  ``solver="cg"`` swaps the
direct factorisation for SciPy CG with a Jacobi preconditioner (what a
``pymatsolver`` iterative plug-in would do), used where SuperLU's fill does
not fit in host memory.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .operators import MeshOps


def _rx_projection(ops, rx):
    """P for one receiver: interp(M) - interp(N) (Dipole) or interp(M) (Pole)."""
    if isinstance(rx.locations, (list, tuple)):
        return (ops.interpolation_matrix(rx.locations[0]) - ops.interpolation_matrix(rx.locations[1])).tocsr()
    return ops.interpolation_matrix(rx.locations).tocsr()


class OracleDC3DNodal:
    """Dense-solver CPU path of the nodal DC simulation.

    ``mesh`` needs ``h`` and ``origin``; ``survey`` needs ``source_list`` with
    ``location``/``current``/``receiver_list`` and receivers with ``locations``,
    ``data_type`` and ``geometric_factor``.  ``sigma_map`` (optional) needs
    ``_transform``-style ``map * m`` and ``diag_deriv(m)``.
    """

    def __init__(self, mesh, survey, sigma_map=None, sigma=None, bc_type="Robin",
                 surface_faces=None, solver="lu", cg_rtol=1e-12, cg_maxiter=200000):
        self.ops = MeshOps(mesh.h, mesh.origin)
        self.survey = survey
        self.sigma_map = sigma_map
        self._sigma_fixed = None if sigma is None else np.asarray(sigma, dtype=np.float64)
        if bc_type == "Mixed":
            bc_type = "Robin"
        if bc_type not in ("Robin", "Neumann"):
            raise ValueError("bc_type must be Robin/Mixed or Neumann")
        self.bc_type = bc_type
        self.surface_faces = surface_faces
        self.solver = solver
        self.cg_rtol = cg_rtol
        self.cg_maxiter = cg_maxiter
        self.G = self.ops.nodal_gradient()
        self.E = self.ops.edge_cell_matrix()
        self.AvgBC = self._set_bc() if bc_type == "Robin" else None
        self.model = None
        self._factor = None

    # ------------------------------------------------------------ BC
    def robin_alpha(self):
        """alpha per boundary face (discretize boundary-face order); top faces 0."""
        ops = self.ops
        bf = ops.boundary_faces()
        nodes = ops.nodes
        middle = np.median(nodes, axis=0)
        top_v = np.max(nodes[:, -1])
        src_pt = np.r_[middle[:-1], top_v]
        n_bf = bf["centers"].shape[0]
        if self.surface_faces is None:
            is_top = np.array([k == ("z", 1) for k in bf["kind"]])
        else:
            is_top = np.asarray(self.surface_faces, dtype=bool)
            if is_top.shape != (n_bf,):
                raise ValueError("surface_faces must be a bool array over boundary faces")
        not_top = ~is_top
        alpha = np.zeros(n_bf)
        r_vec = bf["centers"][not_top] - src_pt
        r = np.linalg.norm(r_vec, axis=-1)
        r_hat = r_vec / r[:, None]
        r_dot_n = np.einsum("ij,ij->i", r_hat, bf["normals"][not_top])
        alpha[not_top] = r_dot_n / r
        return alpha, bf

    def _set_bc(self):
        alpha, bf = self.robin_alpha()
        n_bf = alpha.size
        # AvgN2Fb (n_bf, nN): 1/4 on the face's nodes; AvgCC2Fb (n_bf, nC): 1 on the adjacent cell
        rows = np.repeat(np.arange(n_bf), 4)
        avn = sp.csr_matrix((np.full(4 * n_bf, 0.25), (rows, bf["nodes"].ravel())), shape=(n_bf, self.ops.nN))
        avc = sp.csr_matrix((np.ones(n_bf), (np.arange(n_bf), bf["cells"])), shape=(n_bf, self.ops.nC))
        avc = sp.diags(alpha * bf["areas"]) @ avc
        return (avn.T @ avc).tocsr()

    # ------------------------------------------------------------ model
    def set_model(self, m):
        self.model = None if m is None else np.asarray(m, dtype=np.float64).ravel()
        self._factor = None

    @property
    def sigma(self):
        if self.sigma_map is None:
            if self._sigma_fixed is None:
                raise AttributeError("no sigma")
            return self._sigma_fixed
        return self.sigma_map * self.model

    def sigma_deriv_diag(self):
        return self.sigma_map.diag_deriv(self.model)

    def _sigma_deriv(self):
        """d sigma / d m: its diagonal (array) for elementwise maps, else the map's sparse derivative
        (``props.py:135-171``: sigmaDeriv = sigmaMap.deriv(model))."""
        if self.sigma_map is None or getattr(self.sigma_map, "is_diagonal", True):
            return self.sigma_deriv_diag()
        return sp.csr_matrix(self.sigma_map.deriv(self.model))

    def _dsig(self, v):
        d = self._sigma_deriv()
        return d * v if isinstance(d, np.ndarray) else np.asarray(d @ v).ravel()

    def _dsigT(self, g):
        d = self._sigma_deriv()
        return d * g if isinstance(d, np.ndarray) else np.asarray(d.T @ g).ravel()

    # ------------------------------------------------------------ operators
    def getA(self, sigma=None):
        s = self.sigma if sigma is None else sigma
        Me = sp.diags(self.E @ s)
        A = (self.G.T @ Me @ self.G).tocsr()
        if self.bc_type == "Neumann":
            A = A.tolil()
            A[0, :] = 0.0
            A[0, 0] = 1.0
            A = A.tocsr()
        else:
            A = A + sp.diags(self.AvgBC @ s, format="csr")
        return A

    def getADeriv(self, u, v, adjoint=False):
        """dA/dm products; u, v may be (nN,) or (nN, k) (k sources, adjoint sums over k)."""
        G = self.G
        Gu = G @ u
        if not adjoint:
            # Grad.T @ (Gu * (E sigma' v))  +  u * (AvgBC sigma' v)
            dv = self._dsig(v)
            w = self.E @ dv
            out = G.T @ (Gu * (w[:, None] if Gu.ndim == 2 else w))
            if self.bc_type != "Neumann":
                b = self.AvgBC @ dv
                out = out + u * (b[:, None] if np.ndim(u) == 2 else b)
            return out
        Gv = G @ v
        prod = Gu * Gv
        if prod.ndim == 2:
            prod = prod.sum(axis=1)
        out = self.E.T @ prod
        if self.bc_type != "Neumann":
            uv = u * v
            if uv.ndim == 2:
                uv = uv.sum(axis=1)
            out = out + self.AvgBC.T @ uv
        return self._dsigT(out)

    def getRHS(self):
        cols = []
        for src in self.survey.source_list:
            P = self.ops.interpolation_matrix(src.location)
            cur = np.asarray(src.current, dtype=np.float64)
            if cur.size == 1 and src.location.shape[0] > 1:
                cur = np.full(src.location.shape[0], cur[0])
            cols.append(np.asarray(P.T @ cur).ravel())
        return np.column_stack(cols)

    # ------------------------------------------------------------ solve
    def _solve(self, rhs):
        if self.solver == "lu":
            if self._factor is None:
                self._factor = spla.splu(self.getA().tocsc())
            return self._factor.solve(np.asarray(rhs, dtype=np.float64))
        A = self.getA()
        M = sp.diags(1.0 / A.diagonal())
        rhs2 = rhs if rhs.ndim == 2 else rhs[:, None]
        out = np.zeros_like(rhs2)
        for j in range(rhs2.shape[1]):
            x, info = spla.cg(A, rhs2[:, j], rtol=self.cg_rtol, atol=0.0, M=M, maxiter=self.cg_maxiter)
            if info != 0:
                raise RuntimeError(f"oracle CG did not converge (info={info})")
            out[:, j] = x
        return out if rhs.ndim == 2 else out[:, 0]

    def fields(self, m=None):
        if m is not None:
            self.set_model(m)
        self._factor = None
        return self._solve(self.getRHS())

    # ------------------------------------------------------------ data
    def _projections(self):
        """[(src_index, P (nD_rx, nN), factor or None)] in survey data order."""
        out = []
        for i, src in enumerate(self.survey.source_list):
            for rx in src.receiver_list:
                P = _rx_projection(self.ops, rx)
                fac = None
                if rx.data_type == "apparent_resistivity":
                    fac = 1.0 / np.asarray(rx.geometric_factor[src])
                out.append((i, P, fac))
        return out

    def dpred(self, m=None, f=None):
        if f is None:
            f = self.fields(m)
        d = []
        for i, P, fac in self._projections():
            v = P @ f[:, i]
            d.append(v * fac if fac is not None else v)
        return np.hstack(d)

    def Jvec(self, m, v, f=None):
        if f is None:
            f = self.fields(m)
        rhs = -self.getADeriv(f, np.asarray(v, dtype=np.float64))
        du = self._solve(rhs)
        out = []
        for i, P, fac in self._projections():
            w = P @ du[:, i]
            out.append(w * fac if fac is not None else w)
        return np.hstack(out)

    def Jtvec(self, m, v, f=None):
        if f is None:
            f = self.fields(m)
        v = np.asarray(v, dtype=np.float64)
        nsrc = len(self.survey.source_list)
        ptv = np.zeros((self.ops.nN, nsrc))
        start = 0
        for i, P, fac in self._projections():
            k = P.shape[0]
            vs = v[start:start + k]
            if fac is not None:
                vs = fac * vs
            ptv[:, i] += P.T @ vs
            start += k
        lam = self._solve(ptv)
        return -self.getADeriv(f, lam, adjoint=True)

    def derived_fields(self, phi, eps0):
        """e = -G phi, j = MeI MeSigma e, charge = -eps0 G^T Me(1) e, charge_density =
        aveN2CC charge / V (``fields.py:214-253``) for phi (nN,) or (nN, k)."""
        E1 = self.E @ np.ones(self.ops.nC)
        e = -(self.G @ phi)
        ratio = (self.E @ self.sigma) / E1
        j = e * (ratio[:, None] if e.ndim == 2 else ratio)
        me1e = e * (E1[:, None] if e.ndim == 2 else E1)
        charge = -eps0 * (self.G.T @ me1e)
        vol = self.ops.vol
        dens = (self.ops.average_node_to_cell() @ charge) / (vol[:, None] if charge.ndim == 2 else vol)
        return e, j, charge, dens

    def getJ(self, m, f=None):
        """Full J (nD, nP): one adjoint solve per datum (``_Jtvec(v=None)``)."""
        if f is None:
            f = self.fields(m)
        cols, owner = [], []
        for i, P, fac in self._projections():
            Pd = P.toarray()
            if fac is not None:
                Pd = fac[:, None] * Pd
            cols.append(Pd.T)
            owner.extend([i] * Pd.shape[0])
        PT = np.hstack(cols)
        lam = self._solve(PT)
        owner = np.array(owner)
        rows = [-self.getADeriv(f[:, owner[dcol]], lam[:, dcol], adjoint=True) for dcol in range(PT.shape[1])]
        J = np.array(rows).reshape(PT.shape[1], -1)  # (nD, nP): nP = the model's size under any map
        return J

    def getJtJdiag(self, m, W=None, f=None):
        J = self.getJ(m, f=f)
        w = np.ones(J.shape[0]) if W is None else np.asarray(W.diagonal()) ** 2
        return (w[:, None] * J * J).sum(axis=0)
