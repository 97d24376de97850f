/*
 * dcgpu.h -- C ABI of the GB300 nodal DC-resistivity engine (libdcgpu.so).
 *
 * Replaces, for simpeg's 3D nodal DC path, the sparse assembly + direct
 * factorisation + per-source loops of
 *   simpeg/electromagnetics/static/resistivity/simulation.py (reference repo).
 * The system A(sigma) = G^T Me(sigma) G + diag(AvgBC sigma) is never
 * assembled: it is applied as a matrix-free 7-point nodal stencil and solved
 * by geometric-multigrid-preconditioned, multi-RHS CG (fp64, or fp32 inner
 * iterations wrapped in fp64 iterative refinement).
 *
 * Conventions
 *  - All device arrays are caller-owned (any allocator; the Python layer uses
 *    torch).  Multi-RHS arrays are column-major (N x k) fp64: RHS r occupies
 *    [r*N, (r+1)*N), the layout of simpeg's Fields "phiSolution" store.
 *  - Nodes and cells are in Fortran order (x fastest), as in discretize.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Every function returns 0 on success or a DC_ERR_* code; the message of
 *    the last failure on the calling thread is dc_last_error().
 *  - A handle may be used from one thread at a time.
 */
#ifndef DCGPU_H
#define DCGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DC_OK 0
#define DC_ERR_ARG 1           /* bad argument (Python: ValueError/TypeError) */
#define DC_ERR_CUDA 2          /* CUDA runtime error                          */
#define DC_ERR_NOT_CONVERGED 3 /* solver hit its iteration limit              */
#define DC_ERR_BREAKDOWN 4     /* non-positive or non-finite curvature        */
#define DC_ERR_NOMEM 5         /* workspace too small / allocation failed      */
#define DC_ERR_STATE 6         /* call out of order (e.g. solve before model)  */

#define DC_MODE_FP64 0   /* plain fp64 MG-PCG                                 */
#define DC_MODE_MIXED 1  /* fp32 MG-PCG inner solves + fp64 refinement        */

typedef struct dc_handle dc_handle;

typedef struct dc_stats {
  int iterations;      /* inner PCG iterations summed over refinement sweeps */
  int outer;           /* refinement sweeps (1 in fp64 mode)                  */
  int status;          /* DC_OK or DC_ERR_NOT_CONVERGED / DC_ERR_BREAKDOWN    */
  int n_levels;        /* multigrid levels                                    */
  double max_rel_res;  /* max over RHS of |b - A x|_2 / |b|_2, fp64          */
} dc_stats;

/* Mesh + boundary set-up.  Replaces Simulation3DNodal.__init__/setBC
 * (resistivity/simulation.py:492-501, :573-644).
 * hx, hy, hz: host cell widths (nx, ny, nz).  bface: host array of
 * 0.25*alpha_f*area_f for every boundary face, packed by side
 * [x-lo (ny*nz), x-hi (ny*nz), y-lo (nx*nz), y-hi (nx*nz), z-lo (nx*ny), z-hi (nx*ny)],
 * each side in Fortran order of its two in-plane cell indices; this is the
 * diagonal of AvgBC's face weights.  bface == NULL selects the Neumann operator
 * (no Robin term). */
int dc_create(int nx, int ny, int nz, const double *hx, const double *hy, const double *hz, const double *bface,
              dc_handle **out);
void dc_destroy(dc_handle *h);
const char *dc_last_error(void);

/* Smoother / hierarchy parameters (before dc_set_model).  Non-positive values keep defaults:
 * nu_pre = nu_post = 3, cheb_ratio = 30, coarse_max = 64 nodes (<= 4096), check_every = 1. */
int dc_set_params(dc_handle *h, int nu_pre, int nu_post, double cheb_ratio, int coarse_max, int check_every);

/* Multigrid coarsening (before the first dc_set_model).  merge = 0: full
 * coarsening, every axis halved at every level.  merge in [1, 16]: selective
 * coarsening -- per axis, adjacent cells are merged in pairs only while their
 * combined width is at most merge x twice the narrowest cell of the level,
 * narrowest pairs first, so stretched padding cells stay unmerged while the
 * finer cells are coarsened (bounded coarse-cell aspect ratios, fewer PCG
 * iterations on padded meshes).  A level that would lose under 10 % of its
 * nodes that way is coarsened fully (on a padded mesh: every level below the
 * first).  Default 1 (on a uniform mesh identical to full
 * coarsening).  Solver option of the reference's solver_opts
 * (simpeg/base/pde_simulation.py:493-511); no reference counterpart of its own. */
int dc_set_coarsening(dc_handle *h, double merge);

/* RHS-block width of the solver's interleaved layout: 1, 2, 4, 8, 16 or 32
 * lanes per node (0 = automatic: the widest that pads at most 1/8 of the
 * lanes).  Set by the autotuner. */
int dc_set_rhs_block(dc_handle *h, int kb);

/* Storage of the multigrid vectors inside the mixed-precision solve:
 * DC_MG_FP16 (default), DC_MG_BF16 or DC_MG_FP32.  With 16-bit storage the
 * V-cycle input is the PCG residual scaled to unit norm per RHS and every
 * operation is done in fp32.  The preconditioner only steers the fp32 PCG,
 * which the fp64 refinement corrects, so this changes iteration counts, not
 * the accuracy the solve reaches.  The fp64 solve keeps fp64.  fp16 can
 * overflow for extreme conductivity contrasts (e.g. 1e-8 S/m air cells); a
 * dc_solve that breaks down with 16-bit storage is solved once more with
 * fp32 storage (in the handle's own workspace when the caller's is too small). */
#define DC_MG_FP32 0
#define DC_MG_FP16 1
#define DC_MG_BF16 2
int dc_set_mg_storage(dc_handle *h, int storage);

/* Multigrid smoother: Chebyshev polynomial of D^-1 A of the first kind on
 * [lmax/cheb_ratio, lmax] (kind 1, default) or of the fourth kind on
 * [0, lmax] (kind 4, which needs no lower bound), lmax the Gershgorin bound of
 * D^-1 A; degrees nu_pre / nu_post (dc_set_params). */
int dc_set_smoother(dc_handle *h, int kind);

/* Finest-level smoothing of the mixed solve with 16-bit multigrid storage:
 * 1 stages the iterate, residual and coefficients in shared memory with bulk
 * asynchronous copies (slabs of node rows marched through the z planes),
 * 0 (default) uses the direct-load kernel; a value 10 * rows + depth
 * (12, 13, 22, 23) forces the slab height and copy depth.  Same arithmetic
 * either way.  Measured on the 1M-node, 256-RHS forward solve: 102 ms staged
 * (best layout: two-row slabs, copy depth 2; 114 ms automatic) vs 85 ms
 * direct, the per-plane CTA barrier of the slab march costing more than the
 * latency it hides. */
int dc_set_staging(dc_handle *h, int enable);

/* Coarse-level operators (takes effect at the next dc_set_model / dc_set_model_cc):
 * 0 rediscretises every coarse level from the volume-averaged conductivity;
 * 1 forms it from the next finer level's operator, the Galerkin product with
 * the linear prolongation collapsed onto seven points; 2 (default) the same
 * with the fine couplings along a coarse edge combined in series.  The
 * operator of the finest level, and so every result, does not change; the
 * iterations a solve needs do (1M-cell solves, 256 RHS: cell-centred 19 -> 12
 * PCG iterations, nodal with the log-conductivity contrast doubled 31 -> 20,
 * the nodal headline solve 12 either way). */
int dc_set_coarse_operator(dc_handle *h, int mode);

/* Number of multigrid levels and nodes of level `lvl`. */
int dc_level_info(dc_handle *h, int lvl, int *n_levels, long long *nodes, int *cells3);

/* Model update: sigma_dev (nC fp64, device).  Builds the per-level stencil
 * coefficients and the coarsest-level Cholesky.  Replaces getA's MeSigma and
 * Robin assembly and the solver factorisation (simulation.py:107-108, :523-555). */
int dc_set_model(dc_handle *h, const double *sigma_dev, void *stream);

/* Cell-centred formulation (Simulation3DCellCentered, simulation.py:321-480).
 * The handle is created (dc_create) on the cell-centre grid: the tensor mesh
 * whose nodes are the cell centres (widths = distances between neighbouring
 * centres, so nx-1 x ny-1 x nz-1 "cells"), with Robin face weights of that
 * grid for the coarse multigrid levels (NULL for Neumann).  Model update from
 * the cell resistivity rho_dev (nC, device): the finest operator is
 * A = Div MfRhoI Grad (getA, :355-378) with MfRhoI the inverse diagonal face
 * inner product and the boundary term bw_f / rho_c of cell c on boundary face
 * f; hp_dev holds the widths hx|hy|hz of the mesh, bw_dev the boundary
 * weights (1 - a_f) A_f^2 / (V_c / 2) packed per side like the Robin face
 * weights (a_f the ghost-point factor of cell_gradient_weak_form_robin;
 * NULL: no boundary term, i.e. Neumann).  The coarse levels are rediscretised
 * from the mean of 1/rho around each cell of the cell-centre grid.  dc_solve
 * then solves A x = b; with a NULL-face handle the row-0 pin of the Neumann
 * getA (:365-373) is reproduced as for the nodal operator. */
int dc_set_model_cc(dc_handle *h, const double *rho_dev, const double *hp_dev, const double *bw_dev, void *stream);

/* out = scale * dA[drho] u for k column-major u (nC rows): the forward
 * getADeriv of the cell-centred simulation (simulation.py:380-391,
 * Div MfRhoIDeriv(Grad u, v) with drho = rhoDeriv @ v), a stencil whose
 * couplings are -(A_f^2 / Mf_f^2) dMf_f and boundary terms -bw_f drho / rho^2. */
int dc_cc_dadm_fwd(dc_handle *h, const double *rho_dev, const double *drho_dev, const double *hp_dev,
                   const double *bw_dev, const double *u_dev, double *out_dev, int k, double scale, void *stream);

/* g = scale * drho_dm (.) sum_r dA^T[u_r, lam_r] (nC): the adjoint getADeriv of
 * the cell-centred simulation summed over the k pairs (simulation.py:380-391,
 * MfRhoIDeriv(Grad u, Div^T v, adjoint=True)); drho_dm_dev the diagonal of
 * d rho / d m (NULL: with respect to rho itself). */
int dc_cc_dadm_adj(dc_handle *h, const double *rho_dev, const double *hp_dev, const double *bw_dev,
                   const double *u_dev, const double *lam_dev, int k, const double *drho_dm_dev, double scale,
                   double *g_dev, void *stream);

/* y = A(sigma) x for k column-major RHS, fp64.  (getA() @ x) */
int dc_apply(dc_handle *h, const double *x_dev, double *y_dev, int k, void *stream);

/* Workspace needed by dc_solve for k RHS in `mode`. */
int dc_solve_workspace_bytes(dc_handle *h, int mode, int k, size_t *bytes);

/* x = A^-1 b for k column-major RHS.  Replaces `Ainv * RHS`
 * (simulation.py:111, :181, :245).  Converged when |b - A x| <= rtol |b| per RHS.
 * inner_rtol / inner_maxit apply to the fp32 inner solves of DC_MODE_MIXED:
 * an inner solve stops at the tolerance that closes the remaining outer gap
 * (x0.3) but never asks for less than inner_rtol (<= 0 selects 3e-5).
 * ws may be NULL (the handle then allocates and caches its own). */
int dc_solve(dc_handle *h, int mode, const double *b_dev, double *x_dev, int k, double rtol, int maxit,
             double inner_rtol, int inner_maxit, void *ws, size_t ws_bytes, dc_stats *stats, void *stream);

/* Fixed-iteration solve that never synchronises with the host, so that it can
 * be recorded into a CUDA graph: exactly n_outer refinement sweeps of n_inner
 * fp32 PCG iterations (DC_MODE_MIXED) or n_inner fp64 PCG iterations
 * (DC_MODE_FP64).  Right-hand sides that reach rtol are frozen on the device,
 * so extra iterations do not change them.  ws must be caller-provided (sized by
 * dc_solve_workspace_bytes); the convergence state stays in it and
 * dc_solve_check reads it afterwards.  Same arithmetic as dc_solve. */
int dc_solve_fixed(dc_handle *h, int mode, const double *b_dev, double *x_dev, int k, double rtol, int n_inner,
                   int n_outer, void *ws, size_t ws_bytes, void *stream);
/* Convergence state left in ws by the last dc_solve_fixed or graph-recorded
 * solve on it: max relative residual, RHS still above rtol, inner iterations
 * summed over sweeps and refinement sweeps (the last two are counted by the
 * graph-recorded solves only; 0 after dc_solve_fixed).  Outputs may be NULL. */
int dc_solve_check(dc_handle *h, int mode, int k, const void *ws, double *max_rel_res, int *n_unconverged,
                   int *iterations, int *sweeps);

/* Independent problems (each its own handle: mesh, model, sources) solved by
 * ONE CUDA-graph launch.  Every problem's adaptive solve is recorded on its own
 * stream (forked from and joined to one capture), and its iteration loops
 * become conditional WHILE nodes whose conditions are set on the device from
 * the per-RHS convergence counters: a launch runs each problem exactly as far
 * as dc_solve would with its default inner settings (same arithmetic, same
 * stopping rule; at most maxit inner iterations in total, 200 per sweep, and
 * 30 refinement sweeps), the problems' kernels run
 * concurrently, and the host is not involved until the launch ends.  This is
 * the batched form of running the reference's per-simulation `fields` over
 * many simulations (simpeg/meta/simulation.py:194-330).  Arrays are per
 * problem (b[i], x[i] column-major N_i x k[i], k[i] <= 1024; ws[i] sized by
 * dc_solve_workspace_bytes); a handle may appear once per batch; read the
 * result's convergence with dc_solve_check. */
typedef struct dc_graph dc_graph;
int dc_batch_graph_create(int n, dc_handle *const *hs, int mode, const double *const *b, double *const *x,
                          const int *k, double rtol, int maxit, void *const *ws, const size_t *ws_bytes,
                          dc_graph **out);
int dc_graph_launch(dc_graph *g, void *stream);
void dc_graph_destroy(dc_graph *g);

/* out = scale * (dA/dsigma . dsig) u  for k column-major u.  Equals
 * scale * getADeriv(u, v) with dsig = sigmaDeriv @ v (simulation.py:557-571,
 * forward): A is linear in sigma, so this is the stencil built from dsig. */
int dc_dadm_fwd(dc_handle *h, const double *u_dev, const double *dsig_dev, double *out_dev, int k, double scale,
                void *stream);

/* g = scale * dsig (.) sum_r [ E^T (G u_r (.) G lam_r) + AvgBC^T (u_r (.) lam_r) ]  (nC).
 * Equals scale * getADeriv(u, lam, adjoint=True) summed over the k pairs
 * (simulation.py:557-571 adjoint; pde_simulation.py:15-83, :296-321).
 * dsig_dev may be NULL (derivative with respect to sigma itself). */
int dc_dadm_adj(dc_handle *h, const double *u_dev, const double *lam_dev, int k, const double *dsig_dev,
                double scale, double *g_dev, void *stream);

/* Electrode tables (built on the host from trilinear interpolation weights):
 * y[out_idx[r]] = (accumulate ? y[.] : 0) + scale * sum_{e in row r} w[e] * x[in_idx[e]].
 * out_idx == NULL means out_idx[r] = r.  Used for receiver projection
 * (receivers.py:156-244: P u, P^T v) with indices into the column-major arrays. */
int dc_csr_spmv(int nrows, const long long *rowptr_dev, const long long *in_idx_dev, const double *w_dev,
                const double *x_dev, const long long *out_idx_dev, double *y_dev, double scale, int accumulate,
                void *stream);

/* y[idx[e]] = val[e] (indices unique); with y zeroed first this is the source
 * term q (sources.py:64-88, simulation.py:265-289). */
int dc_fill_sparse(long long nnz, const long long *idx_dev, const double *val_dev, double *y_dev, void *stream);

/* diag(J^T W^T W J) for the model map's diagonal derivative dsig (nC; NULL: w.r.t.
 * sigma), without forming J.  Replaces getJ + the row loop of getJtJdiag
 * (resistivity/simulation.py:115-154).  phi: column-major (N x nE) pole
 * solutions A^-1 q_k of the survey's nE unique electrodes (from dc_solve).
 * Datum d uses source electrodes sa[d], sb[d] (-1: none) with currents
 * ia[d], ib[d], receiver electrodes rm[d], rn[d] (-1: none) with weights
 * wm[d], wn[d] (interpolation/apparent-resistivity factors absorbed), and
 * w2[d] = W_dd^2.  All tables are device arrays.  Needs nE * 116 bytes of
 * shared memory per block (nE up to ~1950 on GB300); more returns DC_ERR_ARG. */
int dc_jtj_diag(dc_handle *h, const double *phi, int nE, int nD, const int *sa, const int *sb, const double *ia,
                const double *ib, const int *rm, const int *rn, const double *wm, const double *wn, const double *w2,
                const double *dsig, double *diag, void *stream);

/* Regulariser of the inversion step: out = scale * R v and/or diag = scale * diag(R), with
 *   (R v)_c = alpha_s V_c v_c + sum_dir alpha_dir sum_{interior faces f} w_f (v_c - v_nbr) / dx_f^2,
 *   w_f = (V_c + V_nbr)/2, dx_f = cell-centre distance: half the second derivative of
 * WeightedLeastSquares' Smallness + SmoothnessFirstOrder on an all-active tensor mesh
 * (regularization/base.py:13-466, :758-1207).  v, out, diag: device (nC). */
int dc_reg_apply(dc_handle *h, double alpha_s, double alpha_x, double alpha_y, double alpha_z, const double *v,
                 double *out, double *diag, double scale, void *stream);

/* ---- Generic SPD sparse solver (the simpeg Solver plug-in, simpeg_gb300.solver.GPUSolver) ----
 * Replaces `solver(A)` / `Ainv * RHS` / `Ainv.clean()` of the pymatsolver
 * plug-in slot (base/pde_simulation.py:493-511, resistivity/simulation.py:105-111)
 * for any symmetric positive-definite CSR matrix simpeg assembles.
 * dc_csr_create: host CSR (int64 indptr[n+1], int32 indices, fp64 data) is
 * validated and uploaded.  dc_csr_solve: x = A^-1 b for k column-major device
 * RHS by Jacobi-preconditioned fp64 CG to |b - A x| <= rtol |b| per column. */
typedef struct dc_csr dc_csr;
int dc_csr_create(int n, long long nnz, const long long *indptr, const int *indices, const double *data,
                  dc_csr **out);
int dc_csr_solve(dc_csr *h, const double *b_dev, double *x_dev, int k, double rtol, int maxit, dc_stats *stats,
                 void *stream);
void dc_csr_destroy(dc_csr *h);

/* Allocation-free variant of dc_dadm_adj.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory when they need the
 * adjoint model derivative -- a host framework that has reserved the GPU's
 * memory for its own pool, or a caller that must not take the implicit device
 * synchronisation of cudaMalloc/cudaFree -- while dc_dadm_adj allocates its
 * scratch through the handle on first use.  Needs no handle: h_dev holds the
 * cell widths hx|hy|hz (nx+ny+nz doubles) and bface_dev the packed Robin face
 * weights of dc_create (NULL: no Robin term), both on the device.  Computes
 * exactly what dc_dadm_adj computes.  Scratch: a file-scope device array of
 * 4*DC_NOALLOC_MAX_NODES doubles (36.6 MiB) held by every GPU that loads the
 * library until exit; meshes with more nodes are rejected with DC_ERR_ARG.
 * Every call looks up the array's device address on the current device
 * (cudaGetSymbolAddress; the first call on a device also loads the module,
 * so it should come before any stream capture).  All
 * calls share the array: calls that overlap on the GPU race.  Calls no
 * cudaMalloc, cudaFree or other allocating routine. */
#define DC_NOALLOC_MAX_NODES 1200000
int dc_dadm_adj_noalloc(int nx, int ny, int nz, const double *h_dev, const double *bface_dev, const double *u_dev,
                        const double *lam_dev, int k, const double *dsig_dev, double scale, double *g_dev,
                        void *stream);

/* Derived fields of Fields3DNodal (simpeg/electromagnetics/static/resistivity/
 * fields.py:186-257) for k nodal potentials phi (column-major (N, k)), on the
 * edges ordered as discretize orders them (all x-edges, then y-, then z-edges,
 * each Fortran-ordered; column-major (nE, k)):
 *   e = -G phi  (Fields3DNodal._e, fields.py:227-236)
 *   j = MeI MeSigma e  (fields.py:214-225; the edge inner products are diagonal
 *       on a tensor mesh: j = e * sum_c sigma_c V_c / sum_c V_c over the cells
 *       holding the edge; uses the conductivity of dc_set_model).
 * Either output may be NULL.  Needs dc_set_model. */
int dc_edge_fields(dc_handle *h, const double *phi, int k, double *e, double *j, void *stream);

/* charge = -eps0 G^T Me(1) e at the nodes ((N, k); fields.py:238-248) and
 * charge_density = average of the cell's 8 node charges / V ((nC, k) or NULL;
 * fields.py:250-253), from the edge field e ((nE, k)).  eps0 is the vacuum
 * permittivity in F/m (the reference uses scipy.constants.epsilon_0). */
int dc_node_charge(dc_handle *h, const double *e, int k, double eps0, double *charge, double *charge_density,
                   void *stream);

/* The launches of the last dc_stencil_timing interval split by kind: c =
 * PREV + 3 * DOT, with PREV 0 (no momentum term), 1 (momentum, x_{k-1}
 * read) or 2 (second step of a zero start) and DOT 1 for the step that also
 * emits the r.z partials.  Fills launches[6], total_ms[6] and alg_bytes[6].
 * Call after dc_stencil_timing(h, 0, ...).  Instrumentation; no reference
 * counterpart. */
int dc_stencil_timing_kinds(dc_handle *h, long long *launches, double *total_ms, double *alg_bytes);

/* Fields3DCellCentered derived fields (fields.py:130-185) for k cell-centred
 * potentials phi (column-major (nC, k)) of a dc_set_model_cc handle: on the
 * faces (x|y|z, each Fortran-ordered; column-major (nF, k)) e = MfI Grad phi
 * and j = MfRhoI Grad phi, Grad = Div^T - B; either output may be NULL. */
int dc_cc_face_fields(dc_handle *h, const double *rho_dev, const double *hp_dev, const double *bw_dev,
                      const double *phi_dev, int k, double *e_dev, double *j_dev, void *stream);

/* charge = eps0 Div e and charge_density = charge / V on the cells ((nC, k)) from the
 * face field e of dc_cc_face_fields (fields.py:166-185); either output may be NULL. */
int dc_cc_charge(dc_handle *h, const double *hp_dev, const double *e_dev, int k, double eps0, double *charge_dev,
                 double *charge_density_dev, void *stream);

/* Continuous-batching session of the mixed-precision solver: the serving form
 * of fields (resistivity/simulation.py:100-113), whose Ainv * RHS solves all
 * sources of one model together.  A session holds the refinement state of
 * `lanes` right-hand-side lanes of one handle (its current model, Robin
 * conditions) between calls, so that right-hand sides join and leave while
 * the others keep iterating:
 *   dc_lanes_open   lays out (or allocates, ws == NULL) the lanes' workspace
 *                   (dc_solve_workspace_bytes(h, DC_MODE_MIXED, lanes));
 *                   *capacity receives the usable lane count (lanes rounded up
 *                   to whole RHS blocks); every lane starts empty
 *   dc_lanes_load   writes n right-hand sides b (column-major (N, n), device)
 *                   into lanes lanes_dev[0..n) (int, device), x = 0 there
 *   dc_lanes_sweep  one refinement sweep over the active lanes: inner fp32
 *                   multigrid-PCG of each lane to its own tolerance, x += d,
 *                   double-float residual; *n_active receives the lanes still
 *                   above rtol (a lane's iterates never depend on the others')
 *   dc_lanes_state  per lane (capacity entries, host): active flag and the
 *                   relative residual |b - A x| / |b| of the last sweep
 *   dc_lanes_fetch  x of lanes lanes_dev[0..n) into x_dev (column-major (N, n))
 * A lane is free again once its solution is fetched (load overwrites it).
 * Calls on one session are ordered on the caller's stream; sessions of
 * different handles run concurrently on different streams. */
typedef struct dc_lanes dc_lanes;
int dc_lanes_open(dc_handle *h, int lanes, double rtol, int inner_maxit, void *ws, size_t ws_bytes, dc_lanes **out,
                  int *capacity);
int dc_lanes_load(dc_lanes *s, const int *lanes_dev, int n, const double *b_dev, void *stream);
int dc_lanes_sweep(dc_lanes *s, int *n_active, int *iterations, void *stream);
int dc_lanes_state(dc_lanes *s, int *active, double *rel_res, void *stream);
int dc_lanes_fetch(dc_lanes *s, const int *lanes_dev, int n, double *x_dev, void *stream);
void dc_lanes_close(dc_lanes *s);

/* Sweeps cover only the lanes [0, n_lanes) from now on, rounded up to whole
 * RHS blocks (0 or the capacity: all lanes).  The caller promises that no lane
 * beyond is active; their state is left untouched.  Lanes handed out lowest
 * first keep a lightly loaded session's sweeps to the blocks in use. */
int dc_lanes_set_extent(dc_lanes *s, int n_lanes);

/* Number of CUDA kernels this library has launched since it was loaded
 * (all handles, all threads).  Instrumentation; no reference counterpart. */
long long dc_kernel_launches(void);

/* Event timing of the fine-level fp32 Chebyshev/stencil launches of h.
 * enable = 1: start recording (up to 4096 launches); enable = 0: stop and
 * return the summed device time, the number of timed launches and their
 * algorithmic bytes (per node: 16*K for a step with the momentum term --
 * read x_k, r, x_{k-1}, write x_{k+1} in fp32 -- or 12*K without it, plus
 * 16-byte coefficients and the 4-byte inverse diagonal).
 * Instrumentation; no reference counterpart. */
int dc_stencil_timing(dc_handle *h, int enable, double *total_ms, long long *launches, double *alg_bytes);

#ifdef __cplusplus
}
#endif
#endif /* DCGPU_H */
