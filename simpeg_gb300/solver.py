"""GPU solver for simpeg's Solver plug-in slot.

``BasePDESimulation.solver`` (``simpeg/base/pde_simulation.py:493-511``) takes a
*class* that subclasses ``pymatsolver.solvers.Base``; the simulation builds it
with the assembled matrix (``Ainv = solver(A, **solver_opts)``,
``resistivity/simulation.py:108``), solves with ``Ainv * RHS`` (``:111,181,245``)
and releases it with ``Ainv.clean()`` (``:106``).  :class:`GPUSolver` is such a
class: the CSR matrix goes to the GPU once and every ``Ainv * RHS`` is one
multi-RHS fp64 CG solve there (``dc_csr_solve`` in ``include/dcgpu.h``).

When pymatsolver is importable the class derives from its ``solvers.Base`` so
simpeg's ``issubclass`` check passes; otherwise a minimal base with the same
constructor arguments and calls (``solve``, ``*``, ``@``, ``.T``, ``clean``) is
used.  Symmetric positive-definite matrices are accepted (simpeg's Robin
nodal and cell-centred DC matrices are), and so are matrices that are
symmetric apart from pinned rows -- rows whose only entry is the diagonal, as
the reference's Neumann ``getA`` pins row 0 (``resistivity/simulation.py:535-540``).
A pinned unknown is known from its row (``x_p = b_p / A_pp``); its column is
moved to the right-hand side, which leaves a symmetric system for CG.  Any
other non-symmetric matrix raises.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import check, lib

try:  # the reference's own base class when available
    from pymatsolver.solvers import Base as _PMBase  # type: ignore
except Exception:  # pragma: no cover - pymatsolver is not installed in the build image
    _PMBase = None


class _MinimalBase:
    """The subset of ``pymatsolver.solvers.Base`` that simpeg calls."""

    def __init__(self, A, is_symmetric=None, is_positive_definite=False, is_hermitian=None, check_accuracy=False,
                 check_rtol=1e-6, check_atol=0, accuracy_tol=None, **kwargs):
        if kwargs:
            raise TypeError(f"unexpected solver arguments {sorted(kwargs)}")
        self._A = A
        self.is_symmetric = is_symmetric
        self.is_positive_definite = is_positive_definite
        self.is_hermitian = is_hermitian
        self.check_accuracy = check_accuracy
        self.check_rtol = check_rtol if accuracy_tol is None else accuracy_tol
        self.check_atol = check_atol

    @property
    def A(self):
        return self._A

    @property
    def shape(self):
        return self._A.shape

    @property
    def dtype(self):
        return self._A.dtype

    def solve(self, rhs):
        rhs = np.asarray(rhs)
        n = self.shape[0]
        if rhs.shape[0] != n:
            raise ValueError(f"Expected a vector of length {n}, got {rhs.shape}")
        if rhs.ndim == 1 or (rhs.ndim == 2 and rhs.shape[1] == 1):
            x = self._solve_single(rhs.reshape(n))
            x = x.reshape(rhs.shape)
        elif rhs.ndim == 2:
            x = self._solve_multiple(rhs)
        else:
            raise ValueError("rhs must be 1D or 2D")
        if self.check_accuracy:
            res = np.linalg.norm(self._A @ x - rhs)
            if res > self.check_rtol * np.linalg.norm(rhs) + self.check_atol:
                raise RuntimeError(f"Accuracy check failed: residual {res:.3e}")
        return x

    def __mul__(self, val):
        return self.solve(val)

    def __matmul__(self, val):
        return self.solve(val)

    @property
    def T(self):
        if self.is_symmetric:
            return self
        return type(self)(self._A.T)

    def clean(self):
        pass


_Base = _PMBase if _PMBase is not None else _MinimalBase


class GPUSolver(_Base):
    """Multi-RHS fp64 conjugate gradients on the GPU for an SPD scipy sparse matrix.

    Extra keyword arguments: ``rtol`` (relative residual per column, default
    1e-12) and ``maxiter`` (default 20000).
    """

    def __init__(self, A, rtol=1e-12, maxiter=20000, **kwargs):
        kwargs.setdefault("is_symmetric", True)
        kwargs.setdefault("is_positive_definite", True)
        super().__init__(A, **kwargs)
        A = sp.csr_matrix(A, dtype=np.float64)
        A.sum_duplicates()
        A.sort_indices()
        if A.shape[0] != A.shape[1]:
            raise ValueError("matrix must be square")
        A, self._pin = self._unpin(A)
        diff = abs(A - A.T)
        if diff.nnz and diff.max() > 1e-12 * abs(A).max():
            raise NotImplementedError("GPUSolver needs a symmetric positive-definite matrix (CG), or one that is "
                                      "symmetric apart from rows holding only their diagonal")
        self._csr = A
        self.rtol = float(rtol)
        self.maxiter = int(maxiter)
        self._h = None
        self._upload()

    @staticmethod
    def _unpin(A):
        """Split off pinned rows (only a diagonal entry) whose columns break the symmetry.

        Returns the matrix with those columns' off-diagonal entries removed and, per pinned row p,
        what the solve needs: the rows p, their diagonals and the removed column entries (a sparse
        (n, n_pinned) matrix), or None when nothing is pinned."""
        nnz_row = np.diff(A.indptr)
        cand = np.flatnonzero(nnz_row == 1)
        if cand.size:
            cand = cand[A.indices[A.indptr[cand]] == cand]
        if cand.size == 0:
            return A, None
        colmask = np.zeros(A.shape[0], dtype=bool)
        colmask[cand] = True
        coo = A.tocoo()
        off = colmask[coo.col] & (coo.row != coo.col)
        if not off.any():
            return A, None
        C_ = sp.csr_matrix((coo.data[off], (coo.row[off], np.searchsorted(cand, coo.col[off]))),
                           shape=(A.shape[0], cand.size))
        keep = ~off
        A2 = sp.csr_matrix((coo.data[keep], (coo.row[keep], coo.col[keep])), shape=A.shape)
        A2.sort_indices()
        return A2, (cand, np.asarray(A.diagonal()[cand], dtype=np.float64), C_)

    def _upload(self):
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("GPUSolver needs a CUDA device")
        A = self._csr
        ptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
        idx = np.ascontiguousarray(A.indices, dtype=np.int32)
        val = np.ascontiguousarray(A.data, dtype=np.float64)
        h = C.c_void_p()
        check(lib().dc_csr_create(A.shape[0], int(A.nnz), ptr.ctypes.data_as(C.POINTER(C.c_longlong)),
                                  idx.ctypes.data_as(C.POINTER(C.c_int)), val.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.byref(h)))
        self._h = h

    def _solve_multiple(self, rhs):
        import torch

        if self._h is None:
            self._upload()
        rhs = np.asarray(rhs, dtype=np.float64)
        n, k = rhs.shape
        if self._pin is not None:  # pinned unknowns to the right-hand side: b - A[:, P] x_P
            rows, diag, C_ = self._pin
            xp = rhs[rows] / diag[:, None]
            rhs = rhs - C_ @ xp
        b = torch.from_numpy(np.ascontiguousarray(rhs.T)).cuda()
        x = torch.empty_like(b)
        st = _lib.dc_stats()
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        check(lib().dc_csr_solve(self._h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), k, self.rtol,
                                 self.maxiter, C.byref(st), stream))
        self.last_iterations = st.iterations
        return x.cpu().numpy().T.copy()

    def _solve_single(self, rhs):
        return self._solve_multiple(np.asarray(rhs).reshape(-1, 1))[:, 0]

    def clean(self):
        if self._h is not None and self._h.value:
            lib().dc_csr_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.clean()
        except Exception:
            pass


_DEFAULT = [GPUSolver]


def get_default_solver():
    """Mirror of ``simpeg.utils.get_default_solver`` (``simpeg/utils/solver_utils.py:47-71``)."""
    return _DEFAULT[0]


def set_default_solver(solver_class):
    """Mirror of ``simpeg.utils.set_default_solver`` (``solver_utils.py:74-88``): same type checks."""
    import inspect

    if not inspect.isclass(solver_class):
        raise TypeError("Default solver must be a class.")
    if not issubclass(solver_class, _Base):
        raise TypeError(f"{solver_class.__qualname__} is not a subclass of the solver base class")
    _DEFAULT[0] = solver_class
