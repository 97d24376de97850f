"""CPU restatement of ``Simulation3DCellCentered`` (oracle only -- test infrastructure).

Follows, function by function:

* ``setBC``                 ``simpeg/electromagnetics/static/resistivity/simulation.py:421-480``:
  ``Div = V face_divergence``, ``Grad = Div^T - B`` with B from
  ``cell_gradient_weak_form_robin(alpha, beta=1, gamma=0)``; Robin alpha =
  (r_hat . n) / r on every boundary face but the top (the same source point and
  top-face rule as the nodal simulation), Neumann alpha = 0, Dirichlet no B
* ``getA``                  ``simulation.py:355-378``: ``A = Div MfRhoI Grad``; Neumann pins row 0
* ``getADeriv``             ``simulation.py:380-391``: ``Div MfRhoIDeriv(Grad u, v)`` and its adjoint
* ``getSourceTerm``         ``sources.py:79-81``: ``q[closest cell centre] = current``
* ``dpred`` / ``Jvec`` / ``Jtvec`` as the nodal oracle (``simulation.py:100-263``), receivers
  interpolating from the cell centres (``receivers.py:414``)
* ``Fields3DCellCentered``  ``resistivity/fields.py:75-185``: ``j = MfRhoI Grad phi``,
  ``e = MfI Grad phi``

The discretize operators (a third-party package, not vendored in the reference) are
restated from their definitions in :mod:`oracle.operators`:

* ``get_face_inner_product(rho)`` on a tensor mesh is diagonal, ``Mf_f = sum over the cells
  c holding face f of V_c rho_c / 2``; ``MfRhoI`` is its inverse.
* ``cell_gradient_weak_form_robin``: on boundary face f (area A_f, adjacent cell c, distance
  h_f = half the cell's width normal to f) the ghost-point value is
  ``phi_f = a_f phi_c`` with ``a_f = (beta / h_f) / (alpha_f + beta / h_f)``, and
  ``B[f, c] = s_f A_f a_f`` with s_f = +1 on the + side of the mesh, -1 on the - side.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .operators import MeshOps


class OracleDC3DCellCentered:
    """Direct-solver CPU path of the cell-centred DC simulation.

    ``rho_map`` (model -> resistivity) or ``sigma_map`` (model -> conductivity;
    rho = 1 / sigma) with ``diag_deriv``; or a fixed ``sigma`` / ``rho``.
    """

    def __init__(self, mesh, survey, sigma_map=None, rho_map=None, sigma=None, rho=None, bc_type="Robin",
                 surface_faces=None, solver="lu", cg_rtol=1e-12):
        self.ops = MeshOps(mesh.h, mesh.origin)
        self.survey = survey
        self.sigma_map, self.rho_map = sigma_map, rho_map
        self._rho_fixed = None
        if rho is not None:
            self._rho_fixed = np.asarray(rho, dtype=np.float64)
        elif sigma is not None:
            self._rho_fixed = 1.0 / np.asarray(sigma, dtype=np.float64)
        if bc_type == "Mixed":
            bc_type = "Robin"
        if bc_type not in ("Robin", "Neumann", "Dirichlet"):
            raise ValueError("bc_type must be Dirichlet, Neumann or Robin/Mixed")
        self.bc_type = bc_type
        self.surface_faces = surface_faces
        self.solver = solver
        self.cg_rtol = cg_rtol
        ops = self.ops
        self.D = ops.face_divergence_raw()     # Div = V face_divergence
        self.F = ops.face_cell_matrix()        # Mf(rho) = diag(F rho)
        self.B = self._robin_B()
        self.G = (self.D.T - self.B).tocsr() if self.B is not None else self.D.T.tocsr()
        self.model = None
        self._factor = None

    # ------------------------------------------------------------ BC
    def _robin_B(self):
        if self.bc_type == "Dirichlet":
            return None
        ops = self.ops
        bf = ops.boundary_faces()
        n_bf = bf["areas"].size
        alpha = np.zeros(n_bf)
        if self.bc_type == "Robin":
            middle = np.median(ops.nodes, axis=0)
            top_v = np.max(ops.nodes[:, -1])
            src_pt = np.r_[middle[:-1], top_v]
            if self.surface_faces is None:
                is_top = np.array([k == ("z", 1) for k in bf["kind"]])
            else:
                is_top = np.asarray(self.surface_faces, dtype=bool)
            not_top = ~is_top
            r_vec = bf["centers"] - src_pt
            r = np.linalg.norm(r_vec, axis=-1)
            with np.errstate(invalid="ignore", divide="ignore"):  # r = 0 only on a top face
                r_dot_n = np.einsum("ij,ij->i", r_vec / r[:, None], bf["normals"])
            alpha[not_top] = (r_dot_n / r)[not_top]
        # distance from the adjacent cell centre to the face centre
        h = np.linalg.norm(bf["centers"] - ops.cell_centers[bf["cells"]], axis=-1)
        beta = 1.0
        a = (beta / h) / (alpha + beta / h)
        sgn = np.array([1.0 if s == 1 else -1.0 for _, s in bf["kind"]])
        rows = ops.boundary_face_index()
        nF = int(sum(ops.n_faces))
        return sp.csr_matrix((sgn * bf["areas"] * a, (rows, bf["cells"])), shape=(nF, ops.nC))

    # ------------------------------------------------------------ model
    def set_model(self, m):
        self.model = None if m is None else np.asarray(m, dtype=np.float64).ravel()
        self._factor = None

    @property
    def rho(self):
        if self.rho_map is not None:
            return self.rho_map * self.model
        if self.sigma_map is not None:
            return 1.0 / (self.sigma_map * self.model)
        if self._rho_fixed is None:
            raise AttributeError("no resistivity")
        return self._rho_fixed

    def rho_deriv_diag(self):
        """d rho / d m (diagonal maps): rhoMap's derivative, or -sigma' / sigma^2 through sigmaMap."""
        if self.rho_map is not None:
            return self.rho_map.diag_deriv(self.model)
        s = self.sigma_map * self.model
        return -self.sigma_map.diag_deriv(self.model) / s**2

    def MfRhoI(self, rho=None):
        return sp.diags(1.0 / (self.F @ (self.rho if rho is None else rho)))

    # ------------------------------------------------------------ operators
    def getA(self, rho=None):
        A = (self.D @ self.MfRhoI(rho) @ self.G).tocsr()
        if self.bc_type == "Neumann":
            A = A.tolil()
            A[0, :] = 0.0
            A[0, 0] = 1.0
            A = A.tocsr()
        return A

    def getADeriv(self, u, v, adjoint=False):
        """Div MfRhoIDeriv(Grad u, v) (``simulation.py:380-391``); u (nC,) or (nC, k); the adjoint
        sums over the k columns."""
        mf = self.F @ self.rho
        dr = self.rho_deriv_diag()
        Gu = self.G @ u
        w = -1.0 / mf**2  # d(1/Mf)/dMf
        if not adjoint:
            dmf = self.F @ (dr * v)
            t = Gu * ((w * dmf)[:, None] if Gu.ndim == 2 else w * dmf)
            return self.D @ t
        Dv = self.D.T @ v
        prod = Gu * Dv
        if prod.ndim == 2:
            prod = prod.sum(axis=1)
        return dr * (self.F.T @ (w * prod))

    def getRHS(self):
        ops = self.ops
        cols = []
        for src in self.survey.source_list:
            loc = np.atleast_2d(np.asarray(src.location, dtype=np.float64))
            cur = np.asarray(src.current, dtype=np.float64).ravel()
            if cur.size == 1 and loc.shape[0] > 1:
                cur = np.full(loc.shape[0], cur[0])
            q = np.zeros(ops.nC)
            q[ops.closest_cell(loc)] = cur  # assignment, as the reference (a later electrode wins a shared cell)
            cols.append(q)
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
            x, info = spla.cg(A, rhs2[:, j], rtol=self.cg_rtol, atol=0.0, M=M, maxiter=200000)
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
        out = []
        ops = self.ops
        for i, src in enumerate(self.survey.source_list):
            for rx in src.receiver_list:
                if isinstance(rx.locations, (list, tuple)):
                    P = (ops.interpolation_matrix_cc(rx.locations[0]) -
                         ops.interpolation_matrix_cc(rx.locations[1])).tocsr()
                else:
                    P = ops.interpolation_matrix_cc(rx.locations).tocsr()
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
        du = self._solve(-self.getADeriv(f, np.asarray(v, dtype=np.float64)))
        out = []
        for i, P, fac in self._projections():
            w = P @ du[:, i]
            out.append(w * fac if fac is not None else w)
        return np.hstack(out)

    def Jtvec(self, m, v, f=None):
        if f is None:
            f = self.fields(m)
        v = np.asarray(v, dtype=np.float64)
        ptv = np.zeros((self.ops.nC, len(self.survey.source_list)))
        start = 0
        for i, P, fac in self._projections():
            k = P.shape[0]
            vs = v[start:start + k]
            if fac is not None:
                vs = fac * vs
            ptv[:, i] += P.T @ vs
            start += k
        lam = self._solve(ptv)  # the reference applies Ainv to the adjoint right-hand side too
        return -self.getADeriv(f, lam, adjoint=True)

    def face_fields(self, phi):
        """j = MfRhoI Grad phi and e = MfI Grad phi on the faces (``fields.py:130-156``)."""
        Gp = self.G @ phi
        mf_rho = self.F @ self.rho
        mf_one = self.F @ np.ones(self.ops.nC)
        j = Gp / (mf_rho[:, None] if Gp.ndim == 2 else mf_rho)
        e = Gp / (mf_one[:, None] if Gp.ndim == 2 else mf_one)
        return e, j
