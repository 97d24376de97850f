// Internal declarations of the nodal DC engine (not part of the C ABI).
//
// Data layout in HBM
// ------------------
// * Node n = i + Nx*(j + Ny*k) (Fortran order, x fastest), as in discretize.
// * Inside the solver a block of K right-hand sides is stored RHS-interleaved
//   in blocks of KB: element (node n, rhs r) lives at ((r / KB) * N + n) * KB + r % KB.
//   With KB = 32 one warp covers one node and 32 RHS, so every stencil load is
//   one 128-byte (fp32) line and the per-node coefficients are warp-uniform.
//   For K < 32 a smaller KB (1..16) packs several nodes per warp.  KB = 1 with
//   K blocks is exactly the column-major (N x K) layout of the C ABI.
// * The stencil coefficients of a level are one 4-vector per node
//   {cx, cy, cz, diag}: c* is the coupling to the +x/+y/+z neighbour (zero on
//   the last node of that axis), diag = sum of the six couplings + Robin term.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace dc {

struct alignas(32) Coef64 { double cx, cy, cz, d; };
struct alignas(16) Coef32 { float cx, cy, cz, d; };
// Row n of A D^-1 in fp32: d_n / d_n and each coupling times the inverse
// diagonal of the node it reaches (0 for an off-mesh neighbour).
struct alignas(32) RowDinv32 { float d, xp, xm, yp, ym, zp, zm, pad; };

struct Dims {
  int Nx, Ny, Nz;    // nodes per axis
  long long N;       // nodes
  unsigned mx, mxy;  // division magic for Nx and Nx*Ny (see fast_div in dc_stencil.cu)
  unsigned mn;       // division magic for N
};

// floor(2^32 / d) + 1: with q = umulhi(n, m), floor(n / d) is q or q - 1 for 0 <= n < 2^31, d >= 2.
inline unsigned div_magic(unsigned d) { return d > 1 ? (unsigned)(0x100000000ull / d + 1ull) : 0u; }

// Largest number of RHS blocks one solve kernel handles (k <= 32 * KB).
constexpr int kMaxRhsBlocks = 32;

// 1D transfer tables between a fine axis (nf nodes) and its coarse axis (nc nodes).
struct Axis1D {
  int nf = 0, nc = 0;
  std::vector<int> pl_idx;      // fine node -> left coarse node
  std::vector<double> pl_w;     // weight on the left coarse node (1 - w on the right one)
  std::vector<int> r_fi;        // coarse node -> fine node (also the cell map: coarse cell I = fine cells [fi[I], fi[I+1]))
  std::vector<double> r_wl, r_wr;  // restriction weights of fine fi-1 and fi+1
};

struct Level {
  int nx = 0, ny = 0, nz = 0;  // cells
  Dims dims{};
  std::vector<double> hx, hy, hz;
  std::vector<double> bface;        // host: 0.25*alpha*area, 6 sides packed
  double *d_h = nullptr;            // device: hx | hy | hz
  double *d_bface = nullptr;        // device copy of bface
  long long bface_off[7] = {0};     // xlo, xhi, ylo, yhi, zlo, zhi, end
  double *d_sigma = nullptr;        // cell conductivity (nC)
  Coef64 *d_coef64 = nullptr;
  Coef32 *d_coef32 = nullptr;
  double *d_invd64 = nullptr;       // 1/diag
  float *d_invd32 = nullptr;
  RowDinv32 *d_rows32 = nullptr;    // rows of A D^-1 (coarse levels with a coarser one): folded first step
  double lmax = 2.0;                // Gershgorin bound of D^-1 A
  // transfer to the next coarser level (valid when has_coarse)
  bool has_coarse = false;
  Axis1D ax[3];
  int *d_pl_idx = nullptr;
  double *d_pl_w = nullptr;
  float *d_pl_w32 = nullptr;
  int *d_r_fi = nullptr;
  double *d_r_wl = nullptr, *d_r_wr = nullptr;
  float *d_r_wl32 = nullptr, *d_r_wr32 = nullptr;
  long long pl_off[4] = {0}, r_off[4] = {0};
};

// Every kernel launch of the engine passes its grid through count_launch(),
// which counts launches for dc_kernel_launches().
std::atomic<long long> &launch_counter();
inline dim3 count_launch(dim3 g) {
  launch_counter().fetch_add(1, std::memory_order_relaxed);
  return g;
}

// ---- dc_stencil.cu -----------------------------------------------------------
void set_sm_count(int n);
// grid of the reduction kernels: one block per (node group) up to per_sm resident blocks per SM
int node_grid(long long nodes, int KB, int nb, int per_sm);

// Right-hand side of a smoothing kernel: on the finest level the PCG residual
// (type T; multiplied per RHS lane by `scale` when that is set), on coarser
// levels the restricted residual (the multigrid storage type V).
template <typename T, typename V> struct Rhs {
  const T *full = nullptr;
  const V *part = nullptr;
  const float *scale = nullptr;
};

// Launchers of the node kernels (dc_kernels.cuh).  T: arithmetic and PCG
// vector type; V: storage type of the multigrid vectors (T, or __half inside
// the mixed-precision solve); KB: RHS lanes per block.
template <typename T, typename V, int KB> struct Ops {
  // resident blocks per SM of the highest-occupancy reduction kernel (sizes the partial arrays)
  static int red_blocks_per_sm();
  // y = A x ; if partial: per-block partial sums of x.y
  static void apply(const Level &L, const T *x, T *y, int nb, double *partial, int gx, cudaStream_t s);
  // q = A p with p stored as V (the PCG search direction), per-block partials of p.q
  static void apply_v(const Level &L, const V *x, T *y, int nb, double *partial, int gx, cudaStream_t s);
  // res = r - A z
  static void residual(const Level &L, Rhs<T, V> r, const V *z, V *res, int nb, cudaStream_t s);
  // z = c0 D^-1 r (first Chebyshev step from zero)
  static void cheb_first(const Level &L, Rhs<T, V> r, V *z, int nb, double c0, cudaStream_t s);
  // zout = zin + c1 (zin - prev) + c2 D^-1 (r - A zin); prev: 0 none, 1 = zout's old content, 2 = zero;
  // 3 = zero with zin = c0 D^-1 r formed from r and the rows of A D^-1 (zin not read); 4 = prev formed as
  // c0 D^-1 r (zout's old content not read).  3 and 4: fp32 arithmetic, no partials.
  // With partial (finest level only): also per-block partials of r . zout.
  static void cheb_step(const Level &L, Rhs<T, V> r, const V *zin, V *zout, int prev, int nb, double c1,
                        double c2, double *partial, int gx, cudaStream_t s, double c0 = 0.0);
  // The same step (no partials) with x_k staged in shared memory by bulk asynchronous copies, for r and
  // the iterates in V; false when it does not apply (then use cheb_step).  Copy timeouts set bit 8 of *status.
  // shape = 10 * slab rows + copy depth to force one layout (0: automatic).
  static bool cheb_bulk(const Level &L, const V *r, const V *zin, V *zout, int prev, int nb, double c1, double c2,
                        int *status, int shape, cudaStream_t s);
  static void restrict_(const Level &f, const Level &c, const V *res, V *rc, int nb, cudaStream_t s);
  static void prolong_add(const Level &f, const Level &c, const V *zc, V *z, int nb, cudaStream_t s);
  static void coarse_solve(const T *Ainv, const Level &c, Rhs<T, V> rc, V *zc, int nb, cudaStream_t s);
  // x += a p ; r -= a q ; partial |r|^2.  With smooth != nullptr also z = c0 D^-1 (scale r) on that level
  // and, when rv_out is set, rv_out = V(scale r).
  // alpha / beta per RHS in fp64 (used when T is double) and fp32 (used when T is float: no
  // per-element fp64 -> fp32 conversion, which runs at GB300's fp64 rate)
  // x_zero: x is 0 and is written, not read (the first update of a solve from zero)
  static void update_xr(long long N, int nb, T *x, T *r, const V *p, const T *q, const double *alpha,
                        const float *alpha32, double *partial, int gx, const Level *smooth, double c0, V *z,
                        const float *scale, V *rv_out, cudaStream_t s, bool x_zero = false);
  // rv_out = V(scale r)
  static void scale_to(long long N, int nb, const T *r, const float *scale, V *rv_out, cudaStream_t s);
  static void dot(long long N, int nb, const T *a, const T *b, double *partial, int gx, cudaStream_t s);
  static void dot_z(long long N, int nb, const T *a, const V *b, double *partial, int gx, cudaStream_t s);
  // p = z + beta p (p and z in V)
  static void p_update(long long N, int nb, V *p, const V *z, const double *beta, const float *beta32,
                       cudaStream_t s);
  static void copy_z(long long N, int nb, V *dst, const V *src, cudaStream_t s);
};

template <int KB>
void ir_residual(const Level &L, const double *b, const double *x, double *r64, float *r32, int nb,
                 const int *active, double *partial, int gx, cudaStream_t s);
template <int KB>
int ir_blocks_per_sm();
// Double-float (fp32 pair) refinement of the mixed solve: hi/lo splits of fp64
// vectors and coefficients, b - A x and x += d in double-float arithmetic.
void split_df(const double *a, long long n, float *hi, float *lo, float *r32, cudaStream_t s);
void coef_split_df(const Level &L, Coef32 *hi, Coef32 *lo, cudaStream_t s);
template <int KB>
void ir_residual_df(const Level &L, const Coef32 *ch, const Coef32 *cl, const float *bh, const float *bl,
                    const float *xh, const float *xl, float *r32, int nb, const int *active, double *partial, int gx,
                    cudaStream_t s);
void ir_accumulate_df(long long n, float *xh, float *xl, const float *d32, cudaStream_t s);
// (xh, xl) = d: the accumulation into a zero iterate, without reading it
void ir_set_df(long long n, float *xh, float *xl, const float *d32, cudaStream_t s);

void fill_int(int *a, int n, int v, cudaStream_t s);
// alpha = rz / (p.q) per active RHS; also zeroes *n_active for the pcg_beta of the same iteration
// (alpha32, if given, receives alpha in fp32)
void pcg_alpha(int K, int KB, int gx, const double *part_pq, const double *rz, const int *active, double *alpha,
               float *alpha32, int *status, int *n_active, cudaStream_t s);
// rz = r.z (divided per RHS by rz_div when set: z came from the scaled input) ;
// rr = |r|^2 ; active &= rr > tol2*bb ; beta ; counts active ; scale_out = 1/sqrt(rr) when set
void pcg_beta(int K, int KB, int gx, const double *part_rz, const double *part_rr, double *rz, double *rr,
              const double *bb, const double *tol2, int *active, double *beta, float *beta32, int *n_active, int first,
              cudaStream_t s, const float *rz_div = nullptr, float *scale_out = nullptr);
// per-RHS sums of block partials; with scale, also scale = 1/sqrt(sum) (the V-cycle input scale)
void sum_partials(int K, int KB, int gx, const double *part, double *out, cudaStream_t s, float *scale = nullptr);
void outer_check(int K, const double *rr, const double *bb, double rtol2, int *active, int *n_active,
                 double *maxrel, double *inner_tol2, double inner_floor2, double safety2, cudaStream_t s);
void fill_double(double *a, int n, double v, cudaStream_t s);
// Condition kernels of the device-side (CUDA-graph WHILE node) solve loops;
// ctr = {inner iterations of this sweep, inner iterations in total, sweeps}.
void inner_loop_cond(cudaGraphConditionalHandle hc, int init, const int *n_active, const int *status, int *ctr,
                     int maxit, int total_max, cudaStream_t s);
void outer_loop_cond(cudaGraphConditionalHandle hc, int init, const int *n_active_out, const int *status, int *ctr,
                     int max_outer, int total_max, cudaStream_t s);


void coef_build(const Level &L, int robin, unsigned long long *d_lmax_bits, cudaStream_t s);
// L.d_rows32 from L's fp32 coefficients and inverse diagonal
void rows_dinv(const Level &L, cudaStream_t s);
void coarsen_sigma(const Level &f, const Level &c, cudaStream_t s);
// Coarse level c's operator from the finer level f's coefficients (mode 1: collapsed Galerkin product with
// the linear prolongation; mode 2: fine couplings in series along each coarse edge).
void coef_galerkin(const Level &f, const Level &c, int mode, unsigned long long *d_lmax_bits, cudaStream_t s);
void dense_assemble(const Level &L, double *dense, cudaStream_t s);
void dense_cholesky_inverse(double *dense, double *work, int n, double *Ainv64, float *Ainv32, int *flag,
                            cudaStream_t s);

// Neumann (row-0 pinned) solves, see dc_solve
void dense_pin0(double *A, int n, cudaStream_t s);
void neumann_rhs(const double *b, long long N, int K, int KB, double *B, double *sums, cudaStream_t s);
void neumann_shift(const double *b, long long N, int K, double *x, cudaStream_t s);

template <typename T>
void pack_colmajor(const double *src, long long N, int K, int KB, int nb, T *dst, cudaStream_t s);
template <typename T>
void unpack_colmajor(const T *src, long long N, int K, int KB, double *dst, cudaStream_t s);
void unpack_colmajor_df(const float *hi, const float *lo, long long N, int K, int KB, double *dst, cudaStream_t s);
// pack_colmajor and split_df in one pass (column-major fp64 -> RHS-blocked (hi, lo) pairs and r32 = hi)
void pack_split_df(const double *src, long long N, int K, int KB, int nb, float *hi, float *lo, float *r32,
                   cudaStream_t s);

// ---- dc_sens.cu -------------------------------------------------------------
void csr_spmv(int nrows, const long long *rowptr, const long long *in_idx, const double *w, const double *x,
              const long long *out_idx, double *y, double scale, int accumulate, cudaStream_t s);
void fill_sparse(long long nnz, const long long *idx, const double *val, double *y, cudaStream_t s);
void scale_vec(long long n, double *y, double a, cudaStream_t s);
void edge_products(const double *u, const double *l, int K, const Dims &d, double *P, double *Q, cudaStream_t s);

// ---- dc_lanes.cu: lanes of a continuous-batching session ------------------------
void lanes_load(const double *b, int n, const int *lanes, long long N, int KB, float *bh, float *bl, float *r32,
                float *xh, float *xl, double *bb, double *rr, cudaStream_t s);
void lanes_fetch(const float *xh, const float *xl, int n, const int *lanes, long long N, int KB, double *x,
                 cudaStream_t s);

// ---- dc_cc.cu: cell-centred formulation on the cell-centre grid ------------------
// rho (nC), hp the primal widths hx|hy|hz, bw the packed boundary weights (6 sides; NULL: none)
void cc_dual_sigma(const double *rho, int nx, int ny, int nz, double *sd, cudaStream_t s);
void cc_coef_build(const Level &L, const double *rho, const double *hp, const double *bw,
                   unsigned long long *d_lmax_bits, cudaStream_t s);
void cc_dcoef_build(const Dims &d, const double *rho, const double *drho, const double *hp, const double *bw,
                    Coef64 *c64, cudaStream_t s);
void cc_gradient(const Dims &d, const double *P, const double *Q, const double *rho, const double *hp,
                 const double *bw, const double *drho_dm, double scale, double *g, cudaStream_t s);
void cc_face_fields(const Dims &d, const double *phi, int K, const double *rho, const double *hp, const double *bw,
                    double *e, double *j, cudaStream_t s);
void cc_charge(const Dims &d, const double *e, int K, const double *hp, double eps0, double *q, double *qd,
               cudaStream_t s);
// Fields3DNodal's derived fields for K potentials (column-major (N, K)): e, j on
// the edges ((nE, K); either may be null; j needs L.d_sigma), the node charge
// q ((N, K)) and, from it, the cell charge density ((nC, K); may be null).
void edge_fields(const Level &L, const double *phi, int K, double *e, double *j, cudaStream_t s);
void node_charge(const Level &L, const double *e, int K, double eps0, double *q, double *rho, cudaStream_t s);
void cell_gradient(const Level &L, int robin, const double *P, const double *Q, const double *dsig, double scale,
                   double *g, cudaStream_t s);

// ---- dc_jtj.cu -------------------------------------------------------------
int jtj_diag_launch(const Level &L, int robin, const double *phi, int nE, int nD, const int *sa, const int *sb,
                    const double *ia, const double *ib, const int *rm, const int *rn, const double *wm,
                    const double *wn, const double *w2, const double *dsig, double *diag, cudaStream_t stream);

// regulariser apply (dc_sens.cu): out = scale * R v, dg = scale * diag(R) (either may be null; v null -> only dg)
void reg_apply(const Level &L, double as, double ax, double ay, double az, const double *v, double *out, double *dg,
               double scale, cudaStream_t s);

std::string &last_error();

}  // namespace dc
