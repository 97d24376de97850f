"""GPU ``Simulation3DNodal``: simpeg's nodal DC forward/sensitivity API on the CUDA engine.

Drop-in for ``simpeg.electromagnetics.static.resistivity.Simulation3DNodal``
(``simpeg/electromagnetics/static/resistivity/simulation.py:20-319,483-670``):
same constructor arguments, same ``fields / dpred / Jvec / Jtvec / getJ /
getJtJdiag`` signatures and data ordering.  The difference is underneath: A
is never assembled or factored; every solve is one multi-RHS call of the
matrix-free multigrid-PCG engine (``include/dcgpu.h``), sources and receivers
are GPU gathers/scatters of precomputed electrode tables, and ``getADeriv``
is a stencil (forward) or an edge-product reduction (adjoint) kernel.
"""

from __future__ import annotations

import warnings

import numpy as np
import scipy.sparse as sp
import torch

from ..engine import DCEngine, csr_spmv, fill_sparse
from ..maps import IdentityMap, ReciprocalMap, ComboMap
from .boundary import robin_face_weights
from .electrodes import SurveyTables
from .fields import Fields3DNodal
from .survey import Survey
from .utils import mini_pole_pole

__all__ = ["Simulation3DNodal"]


def _is_tensor_mesh(mesh):
    return hasattr(mesh, "h") and len(mesh.h) == 3 and hasattr(mesh, "origin")


class Simulation3DNodal:
    """3D nodal DC problem on a tensor mesh, solved on the GPU.

    Extra keyword arguments (not in the reference) select the arithmetic:
    ``precision`` ("mixed": fp32 multigrid-PCG inner solves wrapped in fp64
    iterative refinement; "fp64": plain fp64 multigrid-PCG), ``rtol`` (relative
    residual of every solve, default 1e-10) and ``device``.
    """

    _solutionType = "phiSolution"
    _formulation = "EB"
    fieldsPair = Fields3DNodal
    _grid = "N"  # where the unknowns live: nodes (electrodes interpolated trilinearly)
    _bc_types = ("Robin", "Neumann")

    def __init__(self, mesh, survey=None, bc_type="Robin", sigma=None, sigmaMap=None, rho=None, rhoMap=None,
                 solver=None, solver_opts=None, storeJ=False, miniaturize=False, surface_faces=None,
                 precision="mixed", rtol=1e-10, maxit=5000, device=None, engine_opts=None, verbose=False,
                 counter=None, **kwargs):
        if kwargs:
            raise TypeError(f"unexpected keyword arguments {sorted(kwargs)}")
        if not _is_tensor_mesh(mesh):
            raise NotImplementedError("the GPU nodal simulation supports 3D tensor meshes only")
        if getattr(mesh, "_meshType", "TENSOR").upper() != "TENSOR":
            raise NotImplementedError(f"mesh type {mesh._meshType} is not supported")
        self.mesh = mesh
        self.survey = survey
        self.storeJ = bool(storeJ)
        self.verbose = verbose
        self.counter = counter
        if solver is not None:
            warnings.warn(
                f"solver={getattr(solver, '__name__', solver)!r} is not used: Simulation3DNodal solves with its "
                "matrix-free multigrid-PCG engine on the GPU (precision, rtol and maxit select it); pass the "
                "solver class to a simulation that assembles A (e.g. GPUSolver for a CSR matrix)",
                UserWarning, stacklevel=2)
        self.solver = solver
        self.solver_opts = {} if solver_opts is None else dict(solver_opts)
        if bc_type == "Mixed":
            bc_type = "Robin"
        if bc_type == "Dirichlet" and "Dirichlet" not in self._bc_types:
            raise ValueError("Dirichlet conditions are not supported in the Nodal formulation")
        if bc_type not in self._bc_types:
            raise ValueError(f"bc_type must be one of {self._bc_types + ('Mixed',)}, not {bc_type!r}")
        self.bc_type = bc_type
        self.surface_faces = surface_faces
        if precision not in ("mixed", "fp64"):
            raise ValueError("precision must be 'mixed' or 'fp64'")
        self.precision = precision
        self.rtol = float(self.solver_opts.get("rtol", rtol))
        self.maxit = int(self.solver_opts.get("maxiter", maxit))
        self.device = torch.device(device if device is not None else "cuda")
        # physical property / map (props.Invertible + Reciprocal semantics)
        self._sigma = None if sigma is None else np.asarray(sigma, dtype=np.float64)
        self._rho = None if rho is None else np.asarray(rho, dtype=np.float64)
        self.sigmaMap = sigmaMap
        self.rhoMap = rhoMap
        self._model = None
        self._model_dev = None  # a model given as a device tensor (fields_dev); host copy made on request
        self._miniaturize = bool(miniaturize)
        self._mini_survey = None
        if self._miniaturize:
            self._dipoles, self._invs, self._mini_survey = mini_pole_pole(self.survey)
        self.engine = self._make_engine(dict(engine_opts or {}))
        self.nN = self.engine.nN
        self.nC = self.engine.nC
        self._tables = None
        self._clear()

    def _make_engine(self, eo):
        # Neumann: no Robin term; the engine reproduces the reference's row-0
        # pinned solve (simulation.py:535-540) on the symmetric operator.
        bface = robin_face_weights(self.mesh, self.surface_faces) if self.bc_type == "Robin" else None
        return DCEngine(self.mesh.h, bface, **eo)

    def _engine_set_property(self, sigma_dev):
        """Model update of the engine from the conductivity on the device."""
        self.engine.set_model(sigma_dev)

    # ------------------------------------------------------------ properties
    @property
    def survey(self):
        if self._survey is None:
            raise AttributeError("Simulation must have a survey")
        return self._survey

    @survey.setter
    def survey(self, value):
        self._survey = value
        self._tables = None

    @property
    def sigmaMap(self):
        if self._sigmaMap is not None:
            return self._sigmaMap
        if self._rhoMap is not None:
            return ComboMap([ReciprocalMap(), self._rhoMap])
        return None

    @sigmaMap.setter
    def sigmaMap(self, value):
        self._sigmaMap = value

    @property
    def rhoMap(self):
        return self._rhoMap

    @rhoMap.setter
    def rhoMap(self, value):
        self._rhoMap = value

    @property
    def model(self):
        if self._model is None and self._model_dev is not None:
            self._model = self._model_dev.detach().cpu().numpy().astype(np.float64).ravel()
        return self._model

    @model.setter
    def model(self, m):
        self._model_dev = None
        if m is None:
            self._model = None
            self._clear()
            return
        m = np.asarray(m, dtype=np.float64).ravel()
        nP = getattr(self.sigmaMap, "nP", "*") if self.sigmaMap is not None else "*"
        if isinstance(nP, (int, np.integer)) and m.size != nP:
            raise ValueError(f"model must have {nP} parameters, got {m.size}")
        if self._model is not None and self._model.shape == m.shape and np.array_equal(self._model, m):
            return
        self._model = m.copy()
        self._clear()

    def _clear(self):
        self._dsig_cache = None
        self._sigma_dev = None
        self._f_cache = None
        self._Jmatrix = None
        self._gtgdiag = None

    @property
    def sigma(self):
        if self._sigma is not None:
            return self._sigma
        if self._rho is not None:
            return 1.0 / self._rho
        if self.sigmaMap is None:
            raise AttributeError("Neither a value nor mapping for sigma/rho has been set")
        if self.model is None:
            raise AttributeError("A `model` is required for physical property sigma")
        return self.sigmaMap * self.model

    @property
    def rho(self):
        return 1.0 / self.sigma

    def _sigma_deriv(self):
        """Derivative of the property the operator is built from (here the conductivity) with
        respect to the model: its diagonal as an array, or a sparse matrix for general maps."""
        return self._conductivity_deriv()

    def _property_deriv_dev(self, d_sigma_dev):
        """:meth:`_sigma_deriv` on the device from the diagonal of d sigma / d m on the device."""
        return d_sigma_dev

    def _conductivity_deriv(self):
        """Diagonal of d sigma / d m as an array, or a sparse matrix for general maps."""
        mp = self.sigmaMap
        if mp is None:
            return None
        if hasattr(mp, "diag_deriv") and getattr(mp, "is_diagonal", True):
            return mp.diag_deriv(self.model)
        D = mp.deriv(self.model)
        if sp.issparse(D):
            D = D.tocsr()
            if D.shape[0] == D.shape[1] and D.nnz == np.count_nonzero(D.diagonal()):
                return np.asarray(D.diagonal(), dtype=np.float64)
        return D

    @property
    def sigmaDeriv(self):
        d = self._conductivity_deriv()
        if d is None:
            return None
        return sp.diags(d) if isinstance(d, np.ndarray) else d

    def _active_survey(self):
        return self._mini_survey if self._mini_survey is not None else self.survey

    def _get_tables(self):
        if self._tables is None:
            t = SurveyTables(self.mesh, self._active_survey().source_list, self.nN, grid=self._grid)
            dev = self.device
            self._tables = t
            self._tq = dict(
                q_idx=torch.from_numpy(t.q_idx).to(dev), q_val=torch.from_numpy(t.q_val).to(dev),
                P_ptr=torch.from_numpy(t.P_ptr).to(dev), P_idx=torch.from_numpy(t.P_idx).to(dev),
                P_w=torch.from_numpy(t.P_w).to(dev), PT_ptr=torch.from_numpy(t.PT_ptr).to(dev),
                PT_idx=torch.from_numpy(t.PT_idx).to(dev), PT_w=torch.from_numpy(t.PT_w).to(dev),
                PT_out=torch.from_numpy(t.PT_out).to(dev),
            )
        return self._tables, self._tq

    # ------------------------------------------------------------ device state
    def _ensure_model(self):
        if self._sigma_dev is None:
            mp = self.sigmaMap
            if (self._sigma is None and self._rho is None and self.model is not None and mp is not None
                    and hasattr(mp, "transform_dev") and np.size(self._model) == self.nC):
                # the model goes to the device once and is mapped there (elementwise maps)
                m = torch.from_numpy(np.ascontiguousarray(self._model, dtype=np.float64).ravel()).to(self.device)
                s = mp.transform_dev(m)
                if not bool(((s > 0) & torch.isfinite(s)).all()):
                    raise ValueError("conductivity must be positive and finite")
                self._sigma_dev = s.contiguous()
            else:
                s = self.sigma
                if s.size != self.nC:
                    raise NotImplementedError(
                        "Anisotropic conductivity is not supported for Robin boundary conditions")
                if np.any(~np.isfinite(s)) or np.any(s <= 0):
                    raise ValueError("conductivity must be positive and finite")
                self._sigma_dev = torch.from_numpy(np.ascontiguousarray(s)).to(self.device)
            self._engine_set_property(self._sigma_dev)
        return self._sigma_dev

    # device bytes the solver workspace may take per call; larger RHS sets are solved in chunks
    workspace_budget = 48 << 30

    def _solve(self, B):
        k = B.shape[0]
        per = max(1, self.engine.workspace_bytes(min(k, 1024), self.precision) // min(k, 1024))
        chunk = int(max(32, min(k, self.workspace_budget // per)))
        if chunk >= k:
            X, info = self.engine.solve(B, mode=self.precision, rtol=self.rtol, maxit=self.maxit)
            self.last_solve_info = info
            return X
        X = torch.empty_like(B)
        for c0 in range(0, k, chunk):
            c1 = min(k, c0 + chunk)
            X[c0:c1], info = self.engine.solve(B[c0:c1].contiguous(), mode=self.precision, rtol=self.rtol,
                                               maxit=self.maxit)
        self.last_solve_info = info
        return X

    def getRHS(self):
        """Source term q as a device tensor (nSrc, nN) == column-major (nN, nSrc)."""
        t, tq = self._get_tables()
        Q = torch.zeros(t.nSrc, self.nN, dtype=torch.float64, device=self.device)
        fill_sparse(tq["q_idx"], tq["q_val"], Q.view(-1))
        return Q

    getSourceTerm = getRHS

    # ------------------------------------------------------------ operator access (host arrays)
    def _to_dev_cols(self, a):
        a = np.asarray(a, dtype=np.float64)
        one = a.ndim == 1
        t = torch.from_numpy(np.ascontiguousarray((a[:, None] if one else a).T)).to(self.device)
        return t, one

    def getA(self):
        """A(sigma) at the current model (``simulation.py:523-555``) as a scipy ``LinearOperator``
        (nN x nN): ``A @ x`` runs the matrix-free stencil on the GPU, A is never assembled.  With
        Neumann conditions row 0 is the identity row, as in the reference's pinned matrix."""
        from scipy.sparse.linalg import LinearOperator

        self._ensure_model()
        pinned = self.bc_type == "Neumann"

        def sym(X):  # the symmetric operator the stencil applies (no pinned row)
            T, one = self._to_dev_cols(X)
            Y = self.engine.apply(T).cpu().numpy().T
            return Y[:, 0] if one else Y

        def mat(X):
            Y = sym(X)
            if pinned:
                Y[0] = np.asarray(X)[0]
            return Y

        def rmat(X):
            X = np.asarray(X, dtype=np.float64)
            if not pinned:
                return sym(X)
            # rows i >= 1 of A are those of the symmetric S, row 0 is e0: A^T x = S x' + e0 x0, x' = x with x0 = 0
            Xs = X.copy()
            Xs[0] = 0.0
            Y = sym(Xs)
            Y[0] += X[0]
            return Y

        return LinearOperator((self.nN, self.nN), matvec=mat, matmat=mat, rmatvec=rmat, rmatmat=rmat,
                              dtype=np.float64)

    def getADeriv(self, u, v, adjoint=False):
        """dA/dm products (``simulation.py:557-571``) on host arrays.  Forward: u (nN,) or (nN, k),
        v (nP,) -> (nN,) or (nN, k).  Adjoint: u and v (nN,) or (nN, k) -> (nP,), summed over the k
        columns.  Stencil kernels on the GPU (``dc_dadm_fwd`` / ``dc_dadm_adj``)."""
        self._ensure_model()
        U, one = self._to_dev_cols(u)
        if not adjoint:
            R = self.engine.dadm_fwd(U, self._dsig_dev(v), scale=1.0).cpu().numpy().T
            return R[:, 0] if one else R
        L, _ = self._to_dev_cols(v)
        g = self.engine.dadm_adj(U, L, None, scale=1.0).cpu().numpy()
        return self._map_adjoint(g)

    # ------------------------------------------------------------ forward
    def _device_model_ok(self):
        """True when a device model can be mapped on the device (an elementwise map, no fixed sigma/rho)."""
        mp = self.sigmaMap
        return (self._sigma is None and self._rho is None and mp is not None and hasattr(mp, "transform_dev")
                and getattr(mp, "is_diagonal", True))

    def fields_dev(self, m_dev):
        """Fields at a model given as a device tensor (nP,): the map runs on the device and the model is
        not copied to the host (a host copy is made only if a host-side method asks for ``model``)."""
        if not self._device_model_ok():
            raise NotImplementedError("device models need an elementwise sigmaMap with a diagonal derivative")
        m_dev = m_dev.detach().to(self.device, torch.float64).reshape(-1)
        nP = getattr(self.sigmaMap, "nP", "*")
        if isinstance(nP, (int, np.integer)) and m_dev.numel() != nP:
            raise ValueError(f"model must have {nP} parameters, got {m_dev.numel()}")
        self._model = None
        self._clear()
        self._model_dev = m_dev
        s = self.sigmaMap.transform_dev(m_dev)
        if not bool(((s > 0) & torch.isfinite(s)).all()):
            raise ValueError("conductivity must be positive and finite")
        self._sigma_dev = s.contiguous()
        self._engine_set_property(self._sigma_dev)
        f = self.fieldsPair(self, self._solve(self.getRHS()))
        self._f_cache = f
        return f

    def fields(self, m=None, calcJ=True):
        if m is not None:
            self.model = m
        self._ensure_model()
        Q = self.getRHS()
        U = self._solve(Q)
        f = self.fieldsPair(self, U)
        self._f_cache = f
        return f

    def _gather(self, U):
        t, tq = self._get_tables()
        d = torch.empty(t.nD, dtype=torch.float64, device=self.device)
        csr_spmv(tq["P_ptr"], tq["P_idx"], tq["P_w"], U.reshape(-1), d)
        return d

    def dpred(self, m=None, f=None):
        if f is None:
            if m is None:
                m = self.model
            f = self.fields(m)
        d = self._gather(f.phi_dev).cpu().numpy()
        return self._mini_survey_data(d)

    def residual(self, m, dobs, f=None):
        return self.dpred(m, f=f) - np.asarray(dobs)

    def make_synthetic_data(self, m, relative_error=0.0, noise_floor=0.0, f=None, add_noise=False, random_seed=None):
        from ..data import SyntheticData

        dclean = self.dpred(m, f=f)
        dobs = dclean.copy()
        if add_noise:
            rng = np.random.default_rng(random_seed)
            std = np.sqrt((relative_error * np.abs(dclean)) ** 2 + noise_floor ** 2)
            dobs = dclean + rng.standard_normal(dclean.size) * std
        return SyntheticData(self.survey, dobs=dobs, dclean=dclean, relative_error=relative_error,
                             noise_floor=noise_floor)

    # ------------------------------------------------------------ sensitivities
    def _fields_for(self, m, f):
        if f is None:
            if self._f_cache is not None and (m is None or (self._model is not None and np.array_equal(
                    np.asarray(m, dtype=np.float64).ravel(), self._model))):
                return self._f_cache  # m None: the fields of the current model
            return self.fields(m)
        return f

    def _dsig_dev(self, v):
        d = self._sigma_deriv()
        v = np.asarray(v, dtype=np.float64).ravel()
        if d is None:
            raise AttributeError("a sigmaMap (or rhoMap) is needed for sensitivities")
        dv = d * v if isinstance(d, np.ndarray) else np.asarray(d @ v).ravel()
        return torch.from_numpy(np.ascontiguousarray(dv)).to(self.device)

    def Jvec(self, m, v, f=None):
        f = self._fields_for(m, f)
        self.model = m
        self._ensure_model()
        if self.storeJ:
            return self.getJ(m, f=f).dot(v)
        dsig = self._dsig_dev(v)
        R = self.engine.dadm_fwd(f.phi_dev, dsig, scale=-1.0)
        dU = self._solve(R)
        return self._mini_survey_data(self._gather(dU).cpu().numpy())

    def _scatterT(self, v):
        t, tq = self._get_tables()
        vd = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(self.device)
        PTv = torch.zeros(t.nSrc, self.nN, dtype=torch.float64, device=self.device)
        csr_spmv(tq["PT_ptr"], tq["PT_idx"], tq["PT_w"], vd, PTv.view(-1), out_idx=tq["PT_out"])
        return PTv

    def _n_params(self):
        """Number of model parameters: the map's nP, else the model's size."""
        nP = getattr(self.sigmaMap, "nP", None) if self.sigmaMap is not None else None
        if isinstance(nP, (int, np.integer)):
            return int(nP)
        return int(np.size(self._model)) if self._model is not None else self.nC

    def _map_adjoint(self, g_sigma):
        d = self._sigma_deriv()
        if isinstance(d, np.ndarray):
            return d * g_sigma
        return np.asarray(d.T @ g_sigma).ravel()

    def Jtvec(self, m, v, f=None):
        f = self._fields_for(m, f)
        self.model = m
        self._ensure_model()
        if hasattr(v, "dobs"):
            v = v.dobs
        if self.storeJ:
            return np.asarray(self.getJ(m, f=f).T.dot(v))
        v = self._mini_survey_dataT(np.asarray(v, dtype=np.float64))
        PTv = self._scatterT(v)
        Lam = self._solve(PTv)
        g = self.engine.dadm_adj(f.phi_dev, Lam, None, scale=-1.0).cpu().numpy()
        return self._map_adjoint(g)

    # ------------------------------------------------------------ device-resident products
    def jvec_dev(self, v_dev, f=None):
        """J v with v a device tensor (nP,) at the current model; returns a device tensor (nD,).

        Same operations as :meth:`Jvec` (``simulation.py:156-187``) without host round trips:
        ``-dA/dm v`` by the stencil kernel, one multi-RHS solve, receiver gather."""
        if self._mini_survey is not None:
            raise NotImplementedError("device products need miniaturize=False (use Jvec)")
        f = f if f is not None else self._fields_for(None, None)
        d = self._sigma_deriv()
        if isinstance(d, np.ndarray):
            dsig = self._dsig_diag_dev() * v_dev
        else:  # sparse d sigma / d m (e.g. through InjectActiveCells): applied on the host
            dsig = self._dsig_dev(v_dev.detach().cpu().numpy())
        R = self.engine.dadm_fwd(f.phi_dev, dsig.contiguous(), scale=-1.0)
        return self._gather(self._solve(R))

    def jtvec_dev(self, w_dev, f=None):
        """J^T w with w a device tensor (nD,) at the current model; returns a device tensor (nP,)."""
        if self._mini_survey is not None:
            raise NotImplementedError("device products need miniaturize=False (use Jtvec)")
        f = f if f is not None else self._fields_for(None, None)
        t, tq = self._get_tables()
        PTv = torch.zeros(t.nSrc, self.nN, dtype=torch.float64, device=self.device)
        csr_spmv(tq["PT_ptr"], tq["PT_idx"], tq["PT_w"], w_dev.contiguous(), PTv.view(-1), out_idx=tq["PT_out"])
        Lam = self._solve(PTv)
        d = self._sigma_deriv()
        if isinstance(d, np.ndarray):
            return self.engine.dadm_adj(f.phi_dev, Lam, self._dsig_diag_dev(), scale=-1.0)
        # sparse d sigma / d m: the cell gradient is mapped back on the host
        g = self.engine.dadm_adj(f.phi_dev, Lam, None, scale=-1.0).cpu().numpy()
        return torch.from_numpy(self._map_adjoint(g)).to(self.device)

    def _dsig_diag_dev(self):
        """Diagonal of d sigma / d m on the device (maps with a diagonal derivative only)."""
        key = self._model_dev if self._model_dev is not None else self._model
        if getattr(self, "_dsig_cache", None) is None or self._dsig_cache[0] is not key:
            mp = self.sigmaMap
            if self._model_dev is not None and hasattr(mp, "diag_deriv_dev") and getattr(mp, "is_diagonal", True):
                dd = self._property_deriv_dev(mp.diag_deriv_dev(self._model_dev)).contiguous()
            else:
                d = self._sigma_deriv()
                if not isinstance(d, np.ndarray):
                    raise NotImplementedError("the map's derivative is not diagonal: no device diagonal exists")
                dd = torch.from_numpy(np.ascontiguousarray(d)).to(self.device)
            self._dsig_cache = (key, dd)
        return self._dsig_cache[1]

    def getJ(self, m, f=None):
        """Full sensitivity (nD, nP): one adjoint solve per datum, batched."""
        self.model = m
        if self._Jmatrix is not None:
            return self._Jmatrix
        f = self._fields_for(m, f)
        self._ensure_model()
        t, tq = self._get_tables()
        nD = t.nD
        J = np.zeros((nD, self._n_params()))
        PT = t.P.T.tocsc()
        owner = t.owner
        chunk = max(1, min(nD, 256))
        for s0 in range(0, nD, chunk):
            s1 = min(nD, s0 + chunk)
            cols = PT[:, s0:s1].tocoo()
            # each datum's P row lives in one source's block: fold to (k, nN)
            B = np.zeros((s1 - s0, self.nN))
            np.add.at(B, (cols.col, cols.row % self.nN), cols.data)
            Lam = self._solve(torch.from_numpy(B).to(self.device))
            for i in range(s1 - s0):
                s = int(owner[s0 + i])
                g = self.engine.dadm_adj(f.phi_dev[s:s + 1], Lam[i:i + 1], None, scale=-1.0)
                J[s0 + i] = self._map_adjoint(g.cpu().numpy())
        J = self._mini_J(J)
        self._Jmatrix = J
        return J

    def getJtJdiag(self, m, W=None, f=None):
        """diag(J^T W^T W J) (``simulation.py:137-154``), exact and without forming J.

        Uses electrode reciprocity: one pole solve per unique electrode of the
        survey, then the ``dc_jtj_diag`` kernel evaluates every datum's cell
        sensitivities from the pole solutions of its (up to) four electrodes and
        accumulates ``W_d^2 J_dc^2``.  Falls back to the batched full-J path for
        multipole sources, non-diagonal model maps or more unique electrodes
        than the kernel's shared-memory tile holds.
        """
        if self._gtgdiag is None:
            self.model = m
            w = None if W is None else np.asarray(W.diagonal(), dtype=np.float64)
            out = self._jtj_diag_reciprocity(w)
            if out is None:
                J = self.getJ(m, f=f)
                w2 = np.ones(J.shape[0]) if w is None else w ** 2
                out = (w2[:, None] * J * J).sum(axis=0)
            self._gtgdiag = out
        return self._gtgdiag

    def _electrode_tables(self):
        """Unique electrodes and, per datum, its source/receiver electrodes and weights."""
        src_pts, src_cur, d_src, M_all, N_all, has_n, fac_all = [], [], [], [], [], [], []
        for s, src in enumerate(self.survey.source_list):
            L = np.atleast_2d(np.asarray(src.location, dtype=np.float64))
            if L.shape[0] > 2:
                return None
            cur = np.asarray(src.electrode_currents() if hasattr(src, "electrode_currents") else src.current,
                             dtype=np.float64).ravel()
            if cur.size == 1 and L.shape[0] > 1:
                cur = np.full(L.shape[0], cur[0])
            src_pts.append(L)
            src_cur.append(cur)
            for rx in src.receiver_list:
                n = rx.nD
                fac = np.ones(n)
                if rx.data_type == "apparent_resistivity":
                    fac = 1.0 / np.asarray(rx.geometric_factor[src], dtype=np.float64)
                if isinstance(rx.locations, (list, tuple)):
                    M_all.append(np.atleast_2d(np.asarray(rx.locations[0], dtype=np.float64)))
                    N_all.append(np.atleast_2d(np.asarray(rx.locations[1], dtype=np.float64)))
                    has_n.append(np.ones(n, dtype=bool))
                else:
                    M = np.atleast_2d(np.asarray(rx.locations, dtype=np.float64))
                    M_all.append(M)
                    N_all.append(M)  # placeholder rows, not used (has_n False)
                    has_n.append(np.zeros(n, dtype=bool))
                fac_all.append(np.broadcast_to(fac, (n,)))
                d_src.append(np.full(n, s, dtype=np.int64))
        if not d_src:
            return None
        d_src = np.concatenate(d_src)
        M_all, N_all = np.concatenate(M_all), np.concatenate(N_all)
        has_n = np.concatenate(has_n)
        fac = np.concatenate(fac_all)
        n_e = np.array([L.shape[0] for L in src_pts])
        first = np.r_[0, np.cumsum(n_e)[:-1]]
        # one table of all electrode positions: the sources', the M's and the used N's
        allp = np.concatenate(src_pts + [M_all, N_all[has_n]])
        uniq, inv = np.unique(allp, axis=0, return_inverse=True)
        inv = np.asarray(inv).ravel().astype(np.int32)
        n_src_pts, nD = int(n_e.sum()), d_src.size
        e_src = inv[:n_src_pts]
        e_m = inv[n_src_pts:n_src_pts + nD]
        e_n = inv[n_src_pts + nD:]
        cur_first = np.array([c[0] for c in src_cur])
        cur_second = np.array([c[1] if c.size > 1 else 0.0 for c in src_cur])
        two = n_e[d_src] == 2
        sa = e_src[first[d_src]].astype(np.int32)
        sb = np.where(two, e_src[np.minimum(first[d_src] + 1, n_src_pts - 1)], -1).astype(np.int32)
        ia = cur_first[d_src].astype(np.float64)
        ib = np.where(two, cur_second[d_src], 0.0)
        rm = e_m.astype(np.int32)
        rn = np.full(nD, -1, np.int32)
        rn[has_n] = e_n
        wm = fac.astype(np.float64).copy()
        wn = np.where(has_n, -fac, 0.0)
        # Electrodes numbered by first appearance in datum order (A, B, M, N of each datum): the electrodes
        # that consecutive data use then have consecutive numbers, so the dc_jtj_diag kernel's reads of their
        # staged pole values (one warp = 32 consecutive data) fall in distinct shared-memory banks.  np.unique
        # numbers them by coordinates, which on line surveys puts consecutive stations a line count apart.
        seq = np.stack([sa, sb, rm, rn], axis=1).ravel()
        seq = seq[seq >= 0]
        old_ids, first = np.unique(seq, return_index=True)
        old_of_new = old_ids[np.argsort(first, kind="stable")]
        unused = np.setdiff1d(np.arange(uniq.shape[0]), old_of_new)
        old_of_new = np.concatenate([old_of_new, unused]).astype(np.int64)
        new_of_old = np.empty(uniq.shape[0], np.int32)
        new_of_old[old_of_new] = np.arange(uniq.shape[0], dtype=np.int32)
        renum = lambda e: np.where(e >= 0, new_of_old[np.maximum(e, 0)], -1).astype(np.int32)
        uniq = uniq[old_of_new]
        sa, sb, rm, rn = renum(sa), renum(sb), renum(rm), renum(rn)
        return uniq, dict(sa=sa, sb=sb, rm=rm, rn=rn, ia=ia, ib=ib, wm=wm, wn=wn)

    def _jtj_diag_reciprocity(self, w):
        import ctypes as C

        from .._lib import check, lib
        from .electrodes import interpolation_matrix

        dsig_np = self._sigma_deriv()
        if not isinstance(dsig_np, np.ndarray):
            return None
        tab = self._electrode_tables()
        if tab is None:
            return None
        uniq, t = tab
        nE = uniq.shape[0]
        if nE * 120 > 220 * 1024:  # the kernel's shared-memory tile: 8 + 4 + 27 * 4 bytes per electrode
            return None
        self._ensure_model()
        dev = self.device
        P = interpolation_matrix(self.mesh, uniq).tocoo()
        P.sum_duplicates()
        Q = torch.zeros(nE, self.nN, dtype=torch.float64, device=dev)
        flat = torch.from_numpy((P.row.astype(np.int64) * self.nN + P.col).astype(np.int64)).to(dev)
        fill_sparse(flat, torch.from_numpy(P.data.astype(np.float64)).to(dev), Q.view(-1))
        Phi = self._solve(Q)
        nD = t["sa"].size
        w2 = np.ones(nD) if w is None else w ** 2
        dv = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in t.items()}
        w2d = torch.from_numpy(np.ascontiguousarray(w2, dtype=np.float64)).to(dev)
        dsig = torch.from_numpy(np.ascontiguousarray(dsig_np)).to(dev)
        diag = torch.empty(self.nC, dtype=torch.float64, device=dev)
        p = lambda x: C.c_void_p(x.data_ptr())
        check(lib().dc_jtj_diag(self.engine._h, p(Phi), nE, nD, p(dv["sa"]), p(dv["sb"]), p(dv["ia"]), p(dv["ib"]),
                                p(dv["rm"]), p(dv["rn"]), p(dv["wm"]), p(dv["wn"]), p(w2d), p(dsig), p(diag),
                                C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return diag.cpu().numpy()

    # ------------------------------------------------------------ miniaturize
    def _mini_survey_data(self, d_mini):
        if self._mini_survey is None:
            return d_mini
        out = d_mini[self._invs[0]]
        out[self._dipoles[0]] -= d_mini[self._invs[1]]
        out[self._dipoles[1]] -= d_mini[self._invs[2]]
        out[self._dipoles[0] & self._dipoles[1]] += d_mini[self._invs[3]]
        return out

    def _mini_survey_dataT(self, v):
        if self._mini_survey is None:
            return v
        out = np.zeros(self._mini_survey.nD)
        np.add.at(out, self._invs[0], v)
        np.subtract.at(out, self._invs[1], v[self._dipoles[0]])
        np.subtract.at(out, self._invs[2], v[self._dipoles[1]])
        np.add.at(out, self._invs[3], v[self._dipoles[0] & self._dipoles[1]])
        return out

    def _mini_survey_data_dev(self, d_mini):
        """:meth:`_mini_survey_data` on a device tensor (same integer maps, gathered on the device)."""
        if self._mini_survey is None:
            return d_mini
        dev = d_mini.device
        if getattr(self, "_mini_dev", None) is None or self._mini_dev[0] != dev:
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
            self._mini_dev = (dev, [t(x.astype(np.int64)) for x in self._invs],
                              [t(x) for x in (self._dipoles[0], self._dipoles[1],
                                              self._dipoles[0] & self._dipoles[1])])
        _, inv, dip = self._mini_dev
        out = d_mini[inv[0]].clone()
        out[dip[0]] -= d_mini[inv[1]]
        out[dip[1]] -= d_mini[inv[2]]
        out[dip[2]] += d_mini[inv[3]]
        return out

    def _mini_survey_dataT_dev(self, v):
        """:meth:`_mini_survey_dataT` on a device tensor (index_add in place of np.add.at)."""
        if self._mini_survey is None:
            return v
        self._mini_survey_data_dev(torch.zeros(self._mini_survey.nD, dtype=v.dtype, device=v.device))
        _, inv, dip = self._mini_dev
        out = torch.zeros(self._mini_survey.nD, dtype=v.dtype, device=v.device)
        out.index_add_(0, inv[0], v)
        out.index_add_(0, inv[1], -v[dip[0]])
        out.index_add_(0, inv[2], -v[dip[1]])
        out.index_add_(0, inv[3], v[dip[2]])
        return out

    def _mini_J(self, J):
        if self._mini_survey is None:
            return J
        return self._mini_survey_data(J)
