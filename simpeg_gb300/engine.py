"""Python handle over the CUDA nodal-DC engine (``include/dcgpu.h``).

Device memory is torch-owned: every array passed in is a CUDA ``torch.Tensor``
(float64, contiguous).  Multi-RHS arrays have shape ``(k, nN)`` -- i.e. the
column-major ``(nN, k)`` layout of simpeg's ``Fields`` store.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, lib

MODES = {"fp64": _lib.DC_MODE_FP64, "mixed": _lib.DC_MODE_MIXED}
MG_STORAGE = {"fp32": _lib.DC_MG_FP32, "fp16": _lib.DC_MG_FP16, "bf16": _lib.DC_MG_BF16}


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _dev64(t, shape=None, name="array"):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch tensor")
    if not t.is_cuda or t.dtype != torch.float64:
        raise TypeError(f"{name} must be a CUDA float64 tensor")
    if not t.is_contiguous():
        t = t.contiguous()
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    return t


class SolveInfo:
    def __init__(self, st):
        self.iterations = st.iterations
        self.outer = st.outer
        self.status = st.status
        self.n_levels = st.n_levels
        self.max_rel_res = st.max_rel_res

    def __repr__(self):
        return (f"SolveInfo(iterations={self.iterations}, outer={self.outer}, status={self.status}, "
                f"levels={self.n_levels}, max_rel_res={self.max_rel_res:.3e})")


class DCEngine:
    """One mesh + boundary condition on the GPU; model-dependent state after :meth:`set_model`.

    Parameters
    ----------
    h : three arrays of cell widths (nx, ny, nz)
    bface : packed Robin face weights (``boundary.robin_face_weights``) or None (Neumann)
    coarsening : selective coarsening factor of the multigrid hierarchy (``dc_set_coarsening``;
        0 = halve every axis at every level)
    """

    def __init__(self, h, bface=None, nu_pre=3, nu_post=3, cheb_ratio=30.0, coarse_max=64, check_every=1,
                 mg_storage="fp16", smoother=1, coarsening=1.0):
        if not torch.cuda.is_available():
            raise RuntimeError("the DC engine needs a CUDA device")
        L = lib()
        hx, hy, hz = [np.ascontiguousarray(w, dtype=np.float64) for w in h]
        self.shape_cells = (hx.size, hy.size, hz.size)
        self.nN = (hx.size + 1) * (hy.size + 1) * (hz.size + 1)
        self.nC = hx.size * hy.size * hz.size
        dp = C.POINTER(C.c_double)
        bf = None
        if bface is not None:
            bf = np.ascontiguousarray(bface, dtype=np.float64)
            nx, ny, nz = self.shape_cells
            if bf.size != 2 * (ny * nz + nx * nz + nx * ny):
                raise ValueError("bface has the wrong length")
        self._h = C.c_void_p()
        check(L.dc_create(hx.size, hy.size, hz.size, hx.ctypes.data_as(dp), hy.ctypes.data_as(dp),
                          hz.ctypes.data_as(dp), bf.ctypes.data_as(dp) if bf is not None else None,
                          C.byref(self._h)))
        check(L.dc_set_params(self._h, nu_pre, nu_post, cheb_ratio, coarse_max, check_every))
        check(L.dc_set_mg_storage(self._h, MG_STORAGE[mg_storage]))
        check(L.dc_set_smoother(self._h, int(smoother)))
        check(L.dc_set_coarsening(self._h, float(coarsening)))
        self.robin = bface is not None
        self._ws = {}
        self._model_set = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().dc_destroy(h)
            except Exception:
                pass
            self._h = None

    def close(self):
        self.__del__()

    # ------------------------------------------------------------------
    def set_params(self, nu_pre=0, nu_post=0, cheb_ratio=0.0, coarse_max=0, check_every=0):
        check(lib().dc_set_params(self._h, nu_pre, nu_post, cheb_ratio, coarse_max, check_every))

    def set_rhs_block(self, kb):
        """Force the RHS-block width (1..32 lanes per node; 0 = automatic)."""
        check(lib().dc_set_rhs_block(self._h, int(kb)))
        self._ws.clear()

    def set_coarsening(self, merge):
        """Selective coarsening factor (0 = full coarsening); before the first set_model."""
        check(lib().dc_set_coarsening(self._h, float(merge)))

    def set_mg_storage(self, storage):
        """Multigrid vector storage of the mixed solve: "fp16" (default), "bf16" or "fp32"."""
        check(lib().dc_set_mg_storage(self._h, MG_STORAGE[storage]))
        self._ws.clear()

    def set_smoother(self, kind):
        """Chebyshev smoother of the first (1) or fourth (4) kind."""
        check(lib().dc_set_smoother(self._h, int(kind)))

    def set_staging(self, enable):
        """Finest-level smoothing staged through shared memory by bulk copies (True) or direct loads;
        an int 10 * rows + depth forces the slab layout."""
        check(lib().dc_set_staging(self._h, int(enable)))

    def set_coarse_operator(self, mode):
        """Coarse multigrid operators (``dc_set_coarse_operator``): "series" (default: formed from the finer
        level, its couplings in series along each coarse edge), "galerkin" (collapsed P^T A P of the finer
        level) or "rediscretised" (from the volume-averaged conductivity); applies at the next set_model."""
        modes = {"rediscretised": 0, "galerkin": 1, "series": 2}
        check(lib().dc_set_coarse_operator(self._h, modes[mode]))

    def set_model(self, sigma):
        sigma = _dev64(sigma, (self.nC,), "sigma")
        check(lib().dc_set_model(self._h, _ptr(sigma), _stream()))
        self._model_set = True

    def levels(self):
        n = C.c_int()
        out = []
        nodes = C.c_longlong()
        cells = (C.c_int * 3)()
        check(lib().dc_level_info(self._h, 0, C.byref(n), C.byref(nodes), cells))
        for l in range(n.value):
            check(lib().dc_level_info(self._h, l, None, C.byref(nodes), cells))
            out.append((tuple(cells), nodes.value))
        return out

    def apply(self, x):
        x = _dev64(x, None, "x")
        x2 = x.reshape(-1, self.nN)
        y = torch.empty_like(x2)
        check(lib().dc_apply(self._h, _ptr(x2), _ptr(y), x2.shape[0], _stream()))
        return y.reshape(x.shape)

    def workspace_bytes(self, k, mode="mixed"):
        b = C.c_size_t()
        check(lib().dc_solve_workspace_bytes(self._h, MODES[mode], int(k), C.byref(b)))
        return b.value

    def solve(self, b, mode="mixed", rtol=1e-9, maxit=2000, inner_rtol=3e-5, inner_maxit=200, ws=None,
              raise_on_fail=True):
        """x = A^-1 b for b of shape (k, nN) or (nN,). Returns (x, SolveInfo)."""
        b = _dev64(b, None, "b")
        b2 = b.reshape(-1, self.nN)
        k = b2.shape[0]
        x = torch.empty_like(b2)
        st = _lib.dc_stats()
        if ws is None:
            need = self.workspace_bytes(k, mode)
            key = (mode,)
            cur = self._ws.get(key)
            if cur is None or cur.numel() < need:
                self._ws[key] = cur = torch.empty(need, dtype=torch.uint8, device=b.device)
            ws = cur
        rc = lib().dc_solve(self._h, MODES[mode], _ptr(b2), _ptr(x), k, float(rtol), int(maxit), float(inner_rtol),
                            int(inner_maxit), _ptr(ws), ws.numel(), C.byref(st), _stream())
        info = SolveInfo(st)
        if rc != 0 and (raise_on_fail or rc != _lib.DC_ERR_NOT_CONVERGED):
            check(rc)
        return x.reshape(b.shape), info

    def solve_fixed(self, b, n_inner, n_outer, mode="mixed", rtol=1e-9, ws=None):
        """Fixed-iteration solve (n_outer refinement sweeps of n_inner PCG iterations) with no host
        synchronisation, so that it can be recorded into a CUDA graph; RHS that converge earlier are
        frozen.  Returns (x, ws); ``check_fixed(ws, k, mode)`` reads the convergence state."""
        b = _dev64(b, None, "b")
        b2 = b.reshape(-1, self.nN)
        k = b2.shape[0]
        x = torch.empty_like(b2)
        if ws is None:
            ws = torch.empty(self.workspace_bytes(k, mode), dtype=torch.uint8, device=b.device)
        check(lib().dc_solve_fixed(self._h, MODES[mode], _ptr(b2), _ptr(x), k, float(rtol), int(n_inner),
                                   int(n_outer), _ptr(ws), ws.numel(), _stream()))
        return x.reshape(b.shape), ws

    def check_fixed(self, ws, k, mode="mixed"):
        """(max relative residual, RHS above rtol) left in ws by solve_fixed."""
        mr, na = C.c_double(), C.c_int()
        check(lib().dc_solve_check(self._h, MODES[mode], int(k), _ptr(ws), C.byref(mr), C.byref(na), None, None))
        return mr.value, na.value

    def stencil_timing(self, enable):
        """Start (True) or stop (False) event timing of the fine-level fp32 stencil launches.

        Stopping returns (total_ms, launches, algorithmic_bytes)."""
        ms, n, b = C.c_double(), C.c_longlong(), C.c_double()
        check(lib().dc_stencil_timing(self._h, 1 if enable else 0, C.byref(ms), C.byref(n), C.byref(b)))
        return (ms.value, n.value, b.value) if not enable else None

    STENCIL_KINDS = ("plain", "momentum", "zero_start", "plain_rz", "momentum_rz", "zero_start_rz")

    def stencil_timing_kinds(self):
        """Per kind of fine-level Chebyshev step (no momentum, momentum, second step of a zero start;
        each with or without the r.z partials) of the last timing interval:
        {kind: (launches, total_ms, algorithmic_bytes)} for the kinds that ran."""
        n = (C.c_longlong * 6)()
        ms = (C.c_double * 6)()
        b = (C.c_double * 6)()
        check(lib().dc_stencil_timing_kinds(self._h, n, ms, b))
        return {k: (n[i], ms[i], b[i]) for i, k in enumerate(self.STENCIL_KINDS) if n[i]}

    def reserve(self, k, mode="mixed"):
        """Allocate the solve workspace for k right-hand sides now (bounded, reused by later solves)."""
        need = self.workspace_bytes(k, mode)
        cur = self._ws.get((mode,))
        if cur is None or cur.numel() < need:
            self._ws[(mode,)] = torch.empty(need, dtype=torch.uint8, device="cuda")
        return need

    @staticmethod
    def make_stream():
        return torch.cuda.Stream()

    def release_workspace(self):
        self._ws.clear()

    @property
    def n_edges(self):
        nx, ny, nz = self.shape_cells
        return nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz

    def edge_fields(self, phi, e=True, j=True):
        """(e, j) on the edges for potentials phi of shape (k, nN) or (nN,); either may be skipped."""
        phi = _dev64(phi, None, "phi")
        p2 = phi.reshape(-1, self.nN)
        k = p2.shape[0]
        eo = torch.empty(k, self.n_edges, dtype=torch.float64, device=phi.device) if e else None
        jo = torch.empty(k, self.n_edges, dtype=torch.float64, device=phi.device) if j else None
        check(lib().dc_edge_fields(self._h, _ptr(p2), k, _ptr(eo), _ptr(jo), _stream()))
        shape = (self.n_edges,) if phi.dim() == 1 else (k, self.n_edges)
        return (eo.reshape(shape) if e else None, jo.reshape(shape) if j else None)

    def node_charge(self, e, eps0, density=False):
        """Node charge (k, nN) (and cell charge density (k, nC)) from the edge field e (k, nE)."""
        e = _dev64(e, None, "e")
        e2 = e.reshape(-1, self.n_edges)
        k = e2.shape[0]
        q = torch.empty(k, self.nN, dtype=torch.float64, device=e.device)
        rho = torch.empty(k, self.nC, dtype=torch.float64, device=e.device) if density else None
        check(lib().dc_node_charge(self._h, _ptr(e2), k, float(eps0), _ptr(q), _ptr(rho), _stream()))
        if e.dim() == 1:
            return q.reshape(self.nN), (rho.reshape(self.nC) if density else None)
        return q, rho

    def dadm_fwd(self, u, dsig, scale=1.0):
        u = _dev64(u, None, "u")
        u2 = u.reshape(-1, self.nN)
        dsig = _dev64(dsig, (self.nC,), "dsig")
        out = torch.empty_like(u2)
        check(lib().dc_dadm_fwd(self._h, _ptr(u2), _ptr(dsig), _ptr(out), u2.shape[0], float(scale), _stream()))
        return out.reshape(u.shape)

    def dadm_adj(self, u, lam, dsig=None, scale=1.0):
        u = _dev64(u, None, "u").reshape(-1, self.nN)
        lam = _dev64(lam, None, "lam").reshape(-1, self.nN)
        if u.shape != lam.shape:
            raise ValueError("u and lam must have the same shape")
        if dsig is not None:
            dsig = _dev64(dsig, (self.nC,), "dsig")
        g = torch.empty(self.nC, dtype=torch.float64, device=u.device)
        check(lib().dc_dadm_adj(self._h, _ptr(u), _ptr(lam), u.shape[0], _ptr(dsig), float(scale), _ptr(g),
                                _stream()))
        return g


class LaneSession:
    """A continuous-batching session of the mixed-precision solver on one engine (``dc_lanes_*`` in
    ``include/dcgpu.h``): right-hand sides are loaded into free lanes while the other lanes keep
    iterating, one refinement sweep at a time, and each lane's solution is fetched when it has
    converged.  The workspace is laid out once (``capacity`` lanes) and reused."""

    def __init__(self, engine, lanes, rtol=1e-9, inner_maxit=200, ws=None):
        self.engine = engine
        self._s = C.c_void_p()
        cap = C.c_int()
        if ws is None:
            ws = torch.empty(engine.workspace_bytes(lanes, "mixed"), dtype=torch.uint8, device="cuda")
        self._ws = ws
        check(lib().dc_lanes_open(engine._h, int(lanes), float(rtol), int(inner_maxit), _ptr(ws), ws.numel(),
                                  C.byref(self._s), C.byref(cap)))
        self.capacity = cap.value
        self.nN = engine.nN

    def _idx(self, lanes):
        return torch.as_tensor(np.asarray(lanes, dtype=np.int32), device=self._ws.device)

    def load(self, lanes, B):
        """Right-hand sides B (len(lanes), nN) (device, float64) into the given lanes."""
        B = _dev64(B, (len(lanes), self.nN), "B")
        idx = self._idx(lanes)
        check(lib().dc_lanes_load(self._s, _ptr(idx), len(lanes), _ptr(B), _stream()))

    def set_extent(self, n_lanes):
        """Sweeps cover lanes [0, n_lanes) only (whole RHS blocks; 0: all); no lane beyond may be active."""
        check(lib().dc_lanes_set_extent(self._s, int(n_lanes)))

    def sweep(self):
        """One refinement sweep of the active lanes; returns (lanes still active, inner iterations)."""
        n, it = C.c_int(), C.c_int()
        check(lib().dc_lanes_sweep(self._s, C.byref(n), C.byref(it), _stream()))
        return n.value, it.value

    def state(self):
        """(active flags, relative residuals) of every lane (host arrays)."""
        act = (C.c_int * self.capacity)()
        rel = (C.c_double * self.capacity)()
        check(lib().dc_lanes_state(self._s, act, rel, _stream()))
        return np.frombuffer(act, dtype=np.int32).copy(), np.frombuffer(rel, dtype=np.float64).copy()

    def fetch(self, lanes, out=None):
        """Solutions of the given lanes as a (len(lanes), nN) device tensor (into ``out`` if given)."""
        if out is None:
            out = torch.empty(len(lanes), self.nN, dtype=torch.float64, device=self._ws.device)
        idx = self._idx(lanes)
        check(lib().dc_lanes_fetch(self._s, _ptr(idx), len(lanes), _ptr(out), _stream()))
        return out

    def close(self):
        if getattr(self, "_s", None) is not None and self._s.value:
            torch.cuda.synchronize()
            lib().dc_lanes_close(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CCEngine(DCEngine):
    """The cell-centred operator ``A = Div MfRhoI Grad`` (``Simulation3DCellCentered``) of a tensor
    mesh, solved on its cell-centre grid (``include/dcgpu.h``: ``dc_set_model_cc``): one unknown per
    cell (``nN`` = the mesh's cells), the finest operator exact, the coarse multigrid levels
    rediscretised on the grid of cell centres.  ``nC`` is the number of model cells (the mesh's)."""

    def __init__(self, mesh, bc_type="Robin", surface_faces=None, **kw):
        from .resistivity.boundary import cc_boundary_weights, cc_grid_face_weights, cell_centre_grid

        grid = cell_centre_grid(mesh)
        super().__init__(grid.h, cc_grid_face_weights(mesh, bc_type), **kw)
        nx, ny, nz = (len(w) for w in mesh.h)
        self._cells = (nx, ny, nz)
        self.nN = nx * ny * nz  # unknowns: the cells (the grid's nodes)
        self.nC = self.nN       # model cells
        self.bc_type = bc_type
        dev = torch.device("cuda")
        self.hp = torch.from_numpy(np.concatenate([np.asarray(w, dtype=np.float64) for w in mesh.h])).to(dev)
        bw = cc_boundary_weights(mesh, bc_type, surface_faces)
        self.bw = None if bw is None else torch.from_numpy(np.ascontiguousarray(bw)).to(dev)
        self.rho = None

    def set_model(self, rho):
        """Model update from the cell resistivity (device, (nC,))."""
        rho = _dev64(rho, (self.nC,), "rho")
        check(lib().dc_set_model_cc(self._h, _ptr(rho), _ptr(self.hp), _ptr(self.bw), _stream()))
        self.rho = rho
        self._model_set = True

    def dadm_fwd(self, u, drho, scale=1.0):
        """scale * dA[drho] u for u of shape (k, nN) or (nN,)."""
        u = _dev64(u, None, "u")
        u2 = u.reshape(-1, self.nN)
        drho = _dev64(drho, (self.nC,), "drho")
        out = torch.empty_like(u2)
        check(lib().dc_cc_dadm_fwd(self._h, _ptr(self.rho), _ptr(drho), _ptr(self.hp), _ptr(self.bw), _ptr(u2),
                                   _ptr(out), u2.shape[0], float(scale), _stream()))
        return out.reshape(u.shape)

    def dadm_adj(self, u, lam, drho_dm=None, scale=1.0):
        """scale * drho_dm (.) sum_r dA^T[u_r, lam_r] (nC,)."""
        u = _dev64(u, None, "u").reshape(-1, self.nN)
        lam = _dev64(lam, None, "lam").reshape(-1, self.nN)
        if u.shape != lam.shape:
            raise ValueError("u and lam must have the same shape")
        if drho_dm is not None:
            drho_dm = _dev64(drho_dm, (self.nC,), "drho_dm")
        g = torch.empty(self.nC, dtype=torch.float64, device=u.device)
        check(lib().dc_cc_dadm_adj(self._h, _ptr(self.rho), _ptr(self.hp), _ptr(self.bw), _ptr(u), _ptr(lam),
                                   u.shape[0], _ptr(drho_dm), float(scale), _ptr(g), _stream()))
        return g

    @property
    def n_faces(self):
        nx, ny, nz = (int(round(v)) for v in self._cells)
        return (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)

    def face_fields(self, phi, e=True, j=True):
        """(e, j) on the faces for cell potentials phi of shape (k, nN) or (nN,); either may be skipped."""
        phi = _dev64(phi, None, "phi")
        p2 = phi.reshape(-1, self.nN)
        k = p2.shape[0]
        eo = torch.empty(k, self.n_faces, dtype=torch.float64, device=phi.device) if e else None
        jo = torch.empty(k, self.n_faces, dtype=torch.float64, device=phi.device) if j else None
        check(lib().dc_cc_face_fields(self._h, _ptr(self.rho), _ptr(self.hp), _ptr(self.bw), _ptr(p2), k, _ptr(eo),
                                      _ptr(jo), _stream()))
        shp = (self.n_faces,) if phi.dim() == 1 else (k, self.n_faces)
        return (eo.reshape(shp) if e else None), (jo.reshape(shp) if j else None)

    def cell_charge(self, e, eps0, density=False):
        """(charge, charge_density) on the cells from the face field e (k, nF)."""
        e = _dev64(e, None, "e")
        e2 = e.reshape(-1, self.n_faces)
        k = e2.shape[0]
        q = torch.empty(k, self.nN, dtype=torch.float64, device=e.device)
        qd = torch.empty_like(q) if density else None
        check(lib().dc_cc_charge(self._h, _ptr(self.hp), _ptr(e2), k, float(eps0), _ptr(q), _ptr(qd), _stream()))
        return q, qd

    def edge_fields(self, *a, **k):
        raise NotImplementedError("the cell-centred fields live on the faces (face_fields)")

    node_charge = edge_fields


def padded_rhs(k):
    """RHS count the engine pads k to (blocks of KB lanes, at most 1/8 of them idle)."""
    for kb in (32, 16, 8, 4, 2, 1):
        nb = (k + kb - 1) // kb
        if (nb * kb - k) * 8 <= nb * kb:
            return nb * kb
    return k


def kernel_launches():
    """Kernels launched by libdcgpu.so so far (process-wide)."""
    return int(lib().dc_kernel_launches())


def csr_spmv(rowptr, idx, w, x, y, out_idx=None, scale=1.0, accumulate=False):
    nrows = rowptr.numel() - 1
    check(lib().dc_csr_spmv(nrows, _ptr(rowptr), _ptr(idx), _ptr(w), _ptr(x), _ptr(out_idx), _ptr(y), float(scale),
                            int(bool(accumulate)), _stream()))
    return y


def fill_sparse(idx, val, y):
    check(lib().dc_fill_sparse(idx.numel(), _ptr(idx), _ptr(val), _ptr(y), _stream()))
    return y
