// Host orchestration of the nodal DC engine and its C ABI (include/dcgpu.h):
// multigrid hierarchy set-up, model update, V-cycle, multi-RHS PCG and the
// fp32/fp64 iterative-refinement driver.
#include "../../include/dcgpu.h"
#include "dc_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>

namespace dc {

std::string &last_error() {
  thread_local std::string msg;
  return msg;
}

namespace {

int fail(int code, const std::string &msg) {
  last_error() = msg;
  return code;
}

#define CK(expr)                                                                    \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess) return fail(DC_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

template <typename T>
int dalloc(T **p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) return fail(DC_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return 0;
}

template <typename T>
int upload(T **p, const std::vector<T> &v) {
  int rc = dalloc(p, v.size());
  if (rc) return rc;
  if (!v.empty()) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

// Coarse node set of one axis.  Every coarse cell covers one or two adjacent
// fine cells.  With wmax <= 0, every second fine node is kept, plus the last
// one (full coarsening; an odd cell count leaves one single-cell coarse cell at
// the end).  With wmax > 0, pairs of adjacent cells whose combined width is at
// most wmax are merged, narrowest pairs first (ties: lower index first), and
// every other cell stays a single-cell coarse cell: stretched padding cells
// are left alone until the rest of the mesh has grown to their width, which
// keeps the coarse cells' aspect ratios bounded (a geometric form of
// semi-coarsening for the point smoother).
Axis1D make_axis(const std::vector<double> &h, bool coarsen, double wmax) {
  Axis1D a;
  const int n = (int)h.size();
  a.nf = n + 1;
  std::vector<double> x(n + 1, 0.0);
  for (int i = 0; i < n; ++i) x[i + 1] = x[i] + h[i];
  if (coarsen && wmax <= 0.0) {
    for (int i = 0; i <= n; i += 2) a.r_fi.push_back(i);
    if (a.r_fi.back() != n) a.r_fi.push_back(n);
  } else if (coarsen) {
    std::vector<int> cand;
    for (int i = 0; i + 1 < n; ++i)
      if (h[i] + h[i + 1] <= wmax) cand.push_back(i);
    std::stable_sort(cand.begin(), cand.end(), [&](int p, int q) { return h[p] + h[p + 1] < h[q] + h[q + 1]; });
    std::vector<char> used(n, 0), starts(n, 0);
    for (int i : cand)
      if (!used[i] && !used[i + 1]) {
        used[i] = used[i + 1] = 1;
        starts[i] = 1;
      }
    for (int i = 0; i < n; i += starts[i] ? 2 : 1) a.r_fi.push_back(i);
    a.r_fi.push_back(n);
  } else {
    for (int i = 0; i <= n; ++i) a.r_fi.push_back(i);
  }
  a.nc = (int)a.r_fi.size();
  a.pl_idx.assign(a.nf, 0);
  a.pl_w.assign(a.nf, 1.0);
  for (int I = 0; I + 1 < a.nc; ++I) {
    const int f0 = a.r_fi[I], f1 = a.r_fi[I + 1];
    for (int f = f0; f < f1; ++f) {
      a.pl_idx[f] = I;
      a.pl_w[f] = (f == f0) ? 1.0 : (x[f1] - x[f]) / (x[f1] - x[f0]);
    }
  }
  a.pl_idx[n] = a.nc - 1;
  a.pl_w[n] = 1.0;
  a.r_wl.assign(a.nc, 0.0);
  a.r_wr.assign(a.nc, 0.0);
  for (int I = 0; I < a.nc; ++I) {
    const int f = a.r_fi[I];
    if (f - 1 >= 0 && a.pl_idx[f - 1] == I - 1 && a.pl_w[f - 1] < 1.0) a.r_wl[I] = 1.0 - a.pl_w[f - 1];
    if (f + 1 <= n && a.pl_idx[f + 1] == I && a.pl_w[f + 1] < 1.0) a.r_wr[I] = a.pl_w[f + 1];
  }
  return a;
}

std::vector<double> coarse_widths(const std::vector<double> &h, const Axis1D &a) {
  std::vector<double> out;
  for (int I = 0; I + 1 < a.nc; ++I) {
    double s = 0.0;
    for (int f = a.r_fi[I]; f < a.r_fi[I + 1]; ++f) s += h[f];
    out.push_back(s);
  }
  return out;
}

void set_bface_offsets(Level &L) {
  const long long nyz = (long long)L.ny * L.nz, nxz = (long long)L.nx * L.nz, nxy = (long long)L.nx * L.ny;
  L.bface_off[0] = 0;
  L.bface_off[1] = nyz;
  L.bface_off[2] = 2 * nyz;
  L.bface_off[3] = 2 * nyz + nxz;
  L.bface_off[4] = 2 * nyz + 2 * nxz;
  L.bface_off[5] = 2 * nyz + 2 * nxz + nxy;
  L.bface_off[6] = 2 * nyz + 2 * nxz + 2 * nxy;
}

// Aggregate the Robin face weights of a fine level onto the coarse faces they tile.
std::vector<double> coarse_bface(const Level &f, const Level &c, const Axis1D ax[3]) {
  std::vector<double> out(c.bface_off[6], 0.0);
  auto cell_of = [&](int axis, int fine_cell) {
    const auto &fi = ax[axis].r_fi;
    int I = (int)(std::upper_bound(fi.begin(), fi.end(), fine_cell) - fi.begin()) - 1;
    return I;
  };
  // x sides: (j, k) in (ny, nz)
  for (int side = 0; side < 2; ++side)
    for (int k = 0; k < f.nz; ++k)
      for (int j = 0; j < f.ny; ++j)
        out[c.bface_off[side] + cell_of(1, j) + (long long)c.ny * cell_of(2, k)] +=
            f.bface[f.bface_off[side] + j + (long long)f.ny * k];
  for (int side = 0; side < 2; ++side)
    for (int k = 0; k < f.nz; ++k)
      for (int i = 0; i < f.nx; ++i)
        out[c.bface_off[2 + side] + cell_of(0, i) + (long long)c.nx * cell_of(2, k)] +=
            f.bface[f.bface_off[2 + side] + i + (long long)f.nx * k];
  for (int side = 0; side < 2; ++side)
    for (int j = 0; j < f.ny; ++j)
      for (int i = 0; i < f.nx; ++i)
        out[c.bface_off[4 + side] + cell_of(0, i) + (long long)c.nx * cell_of(1, j)] +=
            f.bface[f.bface_off[4 + side] + i + (long long)f.nx * j];
  return out;
}

void set_dims(Level &L) {
  L.dims.Nx = L.nx + 1;
  L.dims.Ny = L.ny + 1;
  L.dims.Nz = L.nz + 1;
  L.dims.N = (long long)L.dims.Nx * L.dims.Ny * L.dims.Nz;
  L.dims.mx = div_magic((unsigned)L.dims.Nx);
  L.dims.mxy = div_magic((unsigned)(L.dims.Nx * L.dims.Ny));
  L.dims.mn = div_magic((unsigned)L.dims.N);
}

struct Cheb {
  double theta, delta, sigma1;
};
Cheb cheb_params(double lmax, double ratio) {
  const double hi = lmax, lo = lmax / ratio;
  Cheb c;
  c.theta = 0.5 * (hi + lo);
  c.delta = 0.5 * (hi - lo);
  c.sigma1 = c.theta / c.delta;
  return c;
}

// Coefficients of a polynomial smoother of D^-1 A in three-term form:
// step k computes x_{k+1} = x_k + c1 (x_k - x_{k-1}) + c2 D^-1 (r - A x_k).
// `first` is the step from x_0 = 0 (x_1 = first D^-1 r); pre[k] (k >= 1) the
// following steps of that zero-start sequence (pre[1] has x_0 = 0: PREV 2);
// post[k] the steps from a nonzero start (post[0] without momentum).
//   kind 1: Chebyshev polynomials of the first kind on [lmax/ratio, lmax]
//           (the classical Chebyshev smoother);
//   kind 4: Chebyshev polynomials of the fourth kind on [0, lmax] (Lottes,
//           "Optimal polynomial smoothers for multigrid V-cycles", 2023):
//           x_1 = 4/(3 lmax) D^-1 r, then c1 = (2k-1)/(2k+3),
//           c2 = (8k+4)/((2k+3) lmax); no lower bound to choose.
struct SmoothStep {
  int prev;
  double c1, c2;
};
struct Smoother {
  double first;
  std::vector<SmoothStep> pre, post;
};
Smoother smoother(int kind, double lmax, double ratio, int nu_pre, int nu_post) {
  Smoother sm;
  if (kind == 4) {
    sm.first = 4.0 / (3.0 * lmax);
    sm.pre.push_back({0, 0.0, 0.0});
    for (int k = 1; k < nu_pre; ++k)
      sm.pre.push_back({k == 1 ? 2 : 1, (2.0 * k - 1.0) / (2.0 * k + 3.0), (8.0 * k + 4.0) / ((2.0 * k + 3.0) * lmax)});
    sm.post.push_back({0, 0.0, sm.first});
    for (int k = 1; k < nu_post; ++k)
      sm.post.push_back({1, (2.0 * k - 1.0) / (2.0 * k + 3.0), (8.0 * k + 4.0) / ((2.0 * k + 3.0) * lmax)});
    return sm;
  }
  const Cheb cp = cheb_params(lmax, ratio);
  sm.first = 1.0 / cp.theta;
  sm.pre.push_back({0, 0.0, 0.0});
  double rho_old = 1.0 / cp.sigma1;
  for (int k = 1; k < nu_pre; ++k) {
    const double rho = 1.0 / (2.0 * cp.sigma1 - rho_old);
    sm.pre.push_back({k == 1 ? 2 : 1, rho * rho_old, 2.0 * rho / cp.delta});
    rho_old = rho;
  }
  sm.post.push_back({0, 0.0, 1.0 / cp.theta});
  rho_old = 1.0 / cp.sigma1;
  for (int k = 1; k < nu_post; ++k) {
    const double rho = 1.0 / (2.0 * cp.sigma1 - rho_old);
    sm.post.push_back({1, rho * rho_old, 2.0 * rho / cp.delta});
    rho_old = rho;
  }
  return sm;
}

}  // namespace
}  // namespace dc

using namespace dc;

struct dc_handle {
  int robin = 1;
  std::vector<Level> lv;
  int nc = 0;
  double *d_Ainv64 = nullptr, *d_dense = nullptr, *d_work = nullptr;
  float *d_Ainv32 = nullptr;
  Coef32 *d_cdf_hi = nullptr, *d_cdf_lo = nullptr;  // finest-level fp64 coefficients as double-float pairs
  int *d_flag = nullptr;
  unsigned long long *d_lmax = nullptr;
  bool model_set = false;
  int nu_pre = 3, nu_post = 3;
  double cheb_ratio = 30.0;
  int coarse_max = 64;  // nodes of the coarsest level (dense Cholesky); 64 halves dc_set_model vs 200 at equal iterations
  double coarsen_merge = 1.0;  // selective coarsening factor (dc_set_coarsening); 0 = full coarsening
  int check_every = 1;
  int mg_storage = DC_MG_FP16;  // mixed solve: storage of the multigrid vectors (dc_set_mg_storage)
  int smoother_kind = 1;  // Chebyshev polynomials of the first or fourth kind (dc_set_smoother)
  int coarse_op = 2;           // coarse operators: 0 rediscretised, 1 collapsed Galerkin, 2 series (dc_set_coarse_operator)
  bool bulk_staging = false;  // finest-level smoothing with bulk-copy staged shared-memory tiles (dc_set_staging)
  int bulk_shape = 0;        // forced slab layout of the staged kernel (10 * rows + copy depth; 0 = automatic)
  int kb_force = 0;  // RHS-block width override (0: pick_kb)
  bool built = false;
  // cached internal workspace
  void *ws = nullptr;
  size_t ws_bytes = 0;
  // derivative scratch (coefficients of dA/dsigma . dsig, edge products)
  Level dlev;
  double *d_P = nullptr, *d_Q = nullptr;
  // pinned host mailbox for convergence polling
  int *h_mail = nullptr;
  double *h_maild = nullptr;
  cudaEvent_t ev = nullptr;
  // streams that record the bodies of device-side solve loops (graph capture)
  cudaStream_t body_s[2] = {nullptr, nullptr};
  // optional timing of the fine-level fp32 Chebyshev stencil launches
  bool prof = false;
  std::vector<cudaEvent_t> prof_ev;  // start/stop pairs
  std::vector<int> prof_kind;        // per pair: PREV + 3 * (r.z partials)
  std::vector<double> prof_alg;      // per pair: algorithmic bytes
  int prof_used = 0;
  double prof_bytes = 0.0;
};

namespace {

void free_level(Level &L, bool own_geometry) {
  if (own_geometry) {
    cudaFree(L.d_h);
    cudaFree(L.d_bface);
    cudaFree(L.d_pl_idx);
    cudaFree(L.d_pl_w);
    cudaFree(L.d_pl_w32);
    cudaFree(L.d_r_fi);
    cudaFree(L.d_r_wl);
    cudaFree(L.d_r_wr);
    cudaFree(L.d_r_wl32);
    cudaFree(L.d_r_wr32);
    cudaFree(L.d_sigma);
  }
  cudaFree(L.d_coef64);
  cudaFree(L.d_coef32);
  cudaFree(L.d_invd64);
  cudaFree(L.d_invd32);
  cudaFree(L.d_rows32);
}

int build_hierarchy(dc_handle *h) {
  // geometry of every level on the host
  for (;;) {
    Level &L = h->lv.back();
    if (L.dims.N <= h->coarse_max) break;
    bool cz[3] = {L.nx >= 4, L.ny >= 4, L.nz >= 4};
    if (!cz[0] && !cz[1] && !cz[2]) break;
    Level C;
    const std::vector<double> *hs[3] = {&L.hx, &L.hy, &L.hz};
    // selective coarsening: merge pairs up to coarsen_merge x twice the narrowest cell of the level.
    // Once a narrow padding cell is left unmerged, the next levels lose under 10 % of their nodes
    // this way and are coarsened fully: the selection acts where the fine cells are most anisotropic.
    double wmax = 0.0;
    if (h->coarsen_merge > 0.0) {
      double hmin = INFINITY;
      for (int a = 0; a < 3; ++a)
        for (double w : *hs[a]) hmin = std::min(hmin, w);
      wmax = h->coarsen_merge * 2.0 * hmin * (1.0 + 1e-9);  // widths equal up to rounding still merge
      long long nc = 1;
      for (int a = 0; a < 3; ++a) nc *= (long long)make_axis(*hs[a], cz[a], wmax).nc;
      if (nc * 10 > L.dims.N * 9) wmax = 0.0;  // under 10 % fewer nodes: coarsen every axis fully instead
    }
    for (int a = 0; a < 3; ++a) L.ax[a] = make_axis(*hs[a], cz[a], wmax);
    C.hx = coarse_widths(L.hx, L.ax[0]);
    C.hy = coarse_widths(L.hy, L.ax[1]);
    C.hz = coarse_widths(L.hz, L.ax[2]);
    C.nx = (int)C.hx.size();
    C.ny = (int)C.hy.size();
    C.nz = (int)C.hz.size();
    set_dims(C);
    set_bface_offsets(C);
    C.bface = coarse_bface(L, C, L.ax);
    L.has_coarse = true;
    h->lv.push_back(C);
  }
  // upload
  for (auto &L : h->lv) {
    std::vector<double> hh(L.hx);
    hh.insert(hh.end(), L.hy.begin(), L.hy.end());
    hh.insert(hh.end(), L.hz.begin(), L.hz.end());
    int rc;
    if ((rc = upload(&L.d_h, hh))) return rc;
    if ((rc = upload(&L.d_bface, L.bface))) return rc;
    const long long nC = (long long)L.nx * L.ny * L.nz;
    if ((rc = dalloc(&L.d_sigma, nC))) return rc;
    if ((rc = dalloc(&L.d_coef64, L.dims.N))) return rc;
    if ((rc = dalloc(&L.d_coef32, L.dims.N))) return rc;
    if ((rc = dalloc(&L.d_invd64, L.dims.N))) return rc;
    if ((rc = dalloc(&L.d_invd32, L.dims.N))) return rc;
    if (&L != &h->lv[0] && L.has_coarse && (rc = dalloc(&L.d_rows32, L.dims.N))) return rc;
    if (L.has_coarse) {
      std::vector<int> pl, rfi;
      std::vector<double> pw, rwl, rwr;
      for (int a = 0; a < 3; ++a) {
        L.pl_off[a] = (long long)pl.size();
        L.r_off[a] = (long long)rfi.size();
        pl.insert(pl.end(), L.ax[a].pl_idx.begin(), L.ax[a].pl_idx.end());
        pw.insert(pw.end(), L.ax[a].pl_w.begin(), L.ax[a].pl_w.end());
        rfi.insert(rfi.end(), L.ax[a].r_fi.begin(), L.ax[a].r_fi.end());
        rwl.insert(rwl.end(), L.ax[a].r_wl.begin(), L.ax[a].r_wl.end());
        rwr.insert(rwr.end(), L.ax[a].r_wr.begin(), L.ax[a].r_wr.end());
      }
      L.pl_off[3] = (long long)pl.size();
      L.r_off[3] = (long long)rfi.size();
      std::vector<float> pw32(pw.begin(), pw.end()), rwl32(rwl.begin(), rwl.end()), rwr32(rwr.begin(), rwr.end());
      if ((rc = upload(&L.d_pl_idx, pl))) return rc;
      if ((rc = upload(&L.d_pl_w, pw))) return rc;
      if ((rc = upload(&L.d_pl_w32, pw32))) return rc;
      if ((rc = upload(&L.d_r_fi, rfi))) return rc;
      if ((rc = upload(&L.d_r_wl, rwl))) return rc;
      if ((rc = upload(&L.d_r_wr, rwr))) return rc;
      if ((rc = upload(&L.d_r_wl32, rwl32))) return rc;
      if ((rc = upload(&L.d_r_wr32, rwr32))) return rc;
    }
  }
  h->nc = (int)h->lv.back().dims.N;
  int rc;
  const size_t nc2 = (size_t)h->nc * h->nc;
  if ((rc = dalloc(&h->d_Ainv64, nc2))) return rc;
  if ((rc = dalloc(&h->d_Ainv32, nc2))) return rc;
  if ((rc = dalloc(&h->d_dense, nc2))) return rc;
  if ((rc = dalloc(&h->d_work, nc2))) return rc;
  if ((rc = dalloc(&h->d_flag, 1))) return rc;
  if ((rc = dalloc(&h->d_lmax, h->lv.size()))) return rc;  // one Gershgorin bound per level
  h->built = true;
  return 0;
}

// ------------------------------------------------------------------ workspace
struct Carve {
  char *p;
  size_t used = 0, cap;
  template <typename T>
  T *take(size_t n) {
    size_t off = (used + 255) & ~size_t(255);
    used = off + n * sizeof(T) + 0;
    if (p == nullptr) return nullptr;
    return reinterpret_cast<T *>(p + off);
  }
};

int pick_kb(int k) {
  // largest KB in {32,16,8,4,2,1} whose padding wastes at most 1/8 of the lanes,
  // among those that keep the RHS blocks within kMaxRhsBlocks
  for (int kb = 32; kb >= 1; kb >>= 1) {
    const int nb = (k + kb - 1) / kb;
    if (nb > kMaxRhsBlocks) return kb * 2 > 32 ? 32 : kb * 2;
    if ((long long)(nb * kb - k) * 8 <= (long long)nb * kb) return kb;
  }
  return 1;
}

template <typename T>
struct MGWork {
  std::vector<T *> r, z, z2, res;
  T *r0 = nullptr;  // finest-level V-cycle input in the storage type (scaled PCG residual), when T differs
  int *status = nullptr;  // PCG status word (copy timeouts of the staged kernels set bit 8)
};

struct Scal {
  double *part_a, *part_b, *part_c;  // partials (gx * Kp each)
  double *rz, *rr, *bb, *alpha, *beta, *rr64, *bb64, *maxrel, *tol2;
  float *alpha32, *beta32;  // alpha, beta in fp32 for the fp32-arithmetic vector kernels
  int *active, *active_out, *n_active, *n_active_out, *status;
  int *loop;  // device-loop counters: {iterations this sweep, iterations in total, sweeps, unused}
  float *scale;  // per-RHS scale of the V-cycle input (1/|r|_2 of the latest residual)
};

template <typename T>
void carve_mg(Carve &c, const dc_handle *h, int Kp, MGWork<T> &w, bool r0 = false) {
  const int L = (int)h->lv.size();
  w.r.assign(L, nullptr);
  w.z.assign(L, nullptr);
  w.z2.assign(L, nullptr);
  w.res.assign(L, nullptr);
  for (int l = 0; l < L; ++l) {
    const size_t n = (size_t)h->lv[l].dims.N * Kp;
    if (l > 0) {
      w.r[l] = c.take<T>(n);
      w.z[l] = c.take<T>(n);
    }
    if (l + 1 < L || L == 1) {
      w.z2[l] = c.take<T>(n);
      w.res[l] = c.take<T>(n);
    }
  }
  if (r0) w.r0 = c.take<T>((size_t)h->lv[0].dims.N * Kp);
}

void carve_scal(Carve &c, int Kp, int gx, Scal &s) {
  s.part_a = c.take<double>((size_t)gx * Kp);
  s.part_b = c.take<double>((size_t)gx * Kp);
  s.part_c = c.take<double>((size_t)gx * Kp);
  s.rz = c.take<double>(Kp);
  s.rr = c.take<double>(Kp);
  s.bb = c.take<double>(Kp);
  s.alpha = c.take<double>(Kp);
  s.beta = c.take<double>(Kp);
  s.rr64 = c.take<double>(Kp);
  s.bb64 = c.take<double>(Kp);
  s.maxrel = c.take<double>(1);
  s.tol2 = c.take<double>(Kp);
  s.active = c.take<int>(Kp);
  s.active_out = c.take<int>(Kp);
  s.n_active = c.take<int>(1);
  s.n_active_out = c.take<int>(1);
  s.status = c.take<int>(1);
  s.loop = c.take<int>(4);
  s.scale = c.take<float>(Kp);
  s.alpha32 = c.take<float>(Kp);
  s.beta32 = c.take<float>(Kp);
}

// Lays out (or, with base == nullptr, sizes) the whole solve workspace.
struct SolveWS {
  int KB, nb, Kp, gx;
  double *B64, *X64, *R64;
  float *d32, *r32, *q32;
  void *pv;  // PCG search direction, multigrid storage type (the direction only steers the inner solve)
  void *zv;  // preconditioned vector, multigrid storage type
  double *p64, *q64, *z64;
  MGWork<float> mg32;
  MGWork<__half> mg16;
  MGWork<__nv_bfloat16> mgb16;
  MGWork<double> mg64;
  int storage;  // mixed solve: DC_MG_FP32 / DC_MG_FP16 / DC_MG_BF16 multigrid vectors
  Scal sc;
  size_t bytes;
};

// Resident blocks per SM of the highest-occupancy reduction kernel a solve of
// this kind launches: gx, the stride of the partial arrays, covers every
// reduction kernel's own resident-capped grid.
template <int KB>
int red_per_sm_kb(int mode, int storage) {
  if (mode == DC_MODE_FP64) return Ops<double, double, KB>::red_blocks_per_sm();
  const int m = storage == DC_MG_FP16   ? Ops<float, __half, KB>::red_blocks_per_sm()
                : storage == DC_MG_BF16 ? Ops<float, __nv_bfloat16, KB>::red_blocks_per_sm()
                                        : Ops<float, float, KB>::red_blocks_per_sm();
  return std::max(m, ir_blocks_per_sm<KB>());
}

int red_per_sm(int KB, int mode, int half) {
  switch (KB) {
    case 32: return red_per_sm_kb<32>(mode, half);
    case 16: return red_per_sm_kb<16>(mode, half);
    case 8: return red_per_sm_kb<8>(mode, half);
    case 4: return red_per_sm_kb<4>(mode, half);
    case 2: return red_per_sm_kb<2>(mode, half);
    default: return red_per_sm_kb<1>(mode, half);
  }
}

void layout_ws(const dc_handle *h, int mode, int k, char *base, SolveWS &w) {
  w.KB = pick_kb(k);
  if (h->kb_force > 0) {
    int kb = h->kb_force;
    while ((k + kb - 1) / kb > kMaxRhsBlocks && kb < 32) kb *= 2;
    w.KB = kb;
  }
  w.nb = (k + w.KB - 1) / w.KB;
  w.Kp = w.nb * w.KB;
  const long long N = h->lv[0].dims.N;
  w.gx = node_grid(N, w.KB, w.nb, red_per_sm(w.KB, mode, h->mg_storage));
  Carve c{base};
  const size_t n = (size_t)N * w.Kp;
  w.B64 = c.take<double>(n);
  w.X64 = c.take<double>(n);
  // fp64 mode: the PCG residual; mixed mode: b as a double-float pair (x64 is one too)
  w.R64 = c.take<double>(n);
  if (mode == DC_MODE_MIXED) {
    w.d32 = c.take<float>(n);
    w.r32 = c.take<float>(n);
    w.q32 = c.take<float>(n);
    w.storage = h->mg_storage;
    if (w.storage == DC_MG_FP16) {
      w.pv = c.take<__half>(n);
      w.zv = c.take<__half>(n);
      carve_mg(c, h, w.Kp, w.mg16, true);
    } else if (w.storage == DC_MG_BF16) {
      w.pv = c.take<__nv_bfloat16>(n);
      w.zv = c.take<__nv_bfloat16>(n);
      carve_mg(c, h, w.Kp, w.mgb16, true);
    } else {
      w.pv = c.take<float>(n);
      w.zv = c.take<float>(n);
      carve_mg(c, h, w.Kp, w.mg32);
    }
  } else {
    w.p64 = c.take<double>(n);
    w.q64 = c.take<double>(n);
    w.z64 = c.take<double>(n);
    carve_mg(c, h, w.Kp, w.mg64);
  }
  carve_scal(c, w.Kp, w.gx, w.sc);
  w.mg32.status = w.mg16.status = w.mgb16.status = w.mg64.status = w.sc.status;
  w.bytes = c.used + 256;
}

// ------------------------------------------------------------------ V-cycle
template <typename T>
const T *ainv(const dc_handle *h);
template <>
const float *ainv<float>(const dc_handle *h) { return h->d_Ainv32; }
template <>
const double *ainv<double>(const dc_handle *h) { return h->d_Ainv64; }

// Chebyshev step; the fine-level fp32 launches are bracketed by events when
// stencil timing is on (dc_stencil_timing).
template <typename T, typename V, int KB>
void timed_cheb(const dc_handle *hc, int l, const Level &F, Rhs<T, V> r, const V *zin, V *zout, int prev, int nb,
                double c1, double c2, double *partial, int gx, int *status, cudaStream_t s, double c0 = 0.0) {
  dc_handle *h = const_cast<dc_handle *>(hc);
  const bool rec = h->prof && l == 0 && sizeof(T) == 4 && h->prof_used + 2 <= (int)h->prof_ev.size();
  if (rec) cudaEventRecord(h->prof_ev[h->prof_used], s);
  // finest level, 16-bit storage, no partials: x_k staged in shared memory by bulk copies
  const bool staged = h->bulk_staging && l == 0 && !partial && r.part && sizeof(V) == 2 &&
                      Ops<T, V, KB>::cheb_bulk(F, r.part, zin, zout, prev, nb, c1, c2, status, h->bulk_shape, s);
  if (!staged) Ops<T, V, KB>::cheb_step(F, r, zin, zout, prev, nb, c1, c2, partial, gx, s, c0);
  if (rec) {
    cudaEventRecord(h->prof_ev[h->prof_used + 1], s);
    // algorithmic bytes: r (T, or V when stored narrow) and x_k (+ x_{k-1}) (V) read, x_{k+1} (V) written;
    // 16-byte coefficients and the 4-byte 1/diag per node
    const double per_lane = (r.full ? sizeof(T) : sizeof(V)) + (prev == 1 ? 3.0 : 2.0) * sizeof(V);
    const double bytes = (double)F.dims.N * (per_lane * KB * nb + 20.0);
    h->prof_kind[h->prof_used / 2] = prev + (partial ? 3 : 0);
    h->prof_alg[h->prof_used / 2] = bytes;
    h->prof_bytes += bytes;
    h->prof_used += 2;
  }
}

// Buffer that receives the first pre-smoothing step of level l, chosen so that
// after (nu_pre - 1) + nu_post ping-pong steps the result lands in z.
template <typename V>
V *first_buffer(const dc_handle *h, int l, V *z, const MGWork<V> &w) {
  const int steps = (h->nu_pre - 1) + h->nu_post;
  return (steps % 2) ? w.z2[l] : z;
}

// Whether level l's first pre-smoothing step x_1 = c0 D^-1 r is folded into
// the next two (never stored): the second forms A x_1 from r and the rows of
// A D^-1 (prev 3), the third forms its x_{k-1} = x_1 from r at the node
// (prev 4).  This saves a pass (k_cheb_first) on the coarse levels.  On the
// finest level the fused x, r update (k_update_xr) already writes x_1, and
// the folded step, with one vector stream in flight instead of two, measured
// slower than the plain zero-start step (440 vs 368 us at 1M nodes x 256 RHS,
// long-scoreboard stalls 7.5 vs 5.3 per issue), so it is not folded there.
// fp32 arithmetic only (the rows are fp32); not with a single pre-smoothing
// step (x_1 is then the residual's operand).
bool folds_first(const dc_handle *h, int l, bool fp32) {
  return fp32 && l > 0 && h->nu_pre >= 2 && h->lv[l].d_rows32;
}

// One V-cycle z = M r from level l.  r is the PCG residual (type T, scaled per
// RHS) on the finest level and the restricted residual below.  If
// `pre_done`, the first Chebyshev step (z1 = D^-1 r / theta into
// first_buffer) was already applied by the caller.  If `dot_partial`, the last
// smoothing step also emits per-block partials of r.z.  Two buffers per level
// (z and z2) alternate: every step writes the one that does not hold the
// current iterate, which also holds the previous iterate the three-term
// recurrence needs.
template <typename T, typename V, int KB>
void vcycle(const dc_handle *h, int l, Rhs<T, V> r, V *z, const MGWork<V> &w, int nb, cudaStream_t s,
            bool pre_done = false, double *dot_partial = nullptr, int gx = 0) {
  using O = Ops<T, V, KB>;
  const int L = (int)h->lv.size();
  if (l == L - 1) {
    O::coarse_solve(ainv<T>(h), h->lv.back(), r, z, nb, s);
    return;
  }
  const Level &F = h->lv[l];
  const Level &C = h->lv[l + 1];
  const Smoother sm = smoother(h->smoother_kind, F.lmax, h->cheb_ratio, h->nu_pre, h->nu_post);
  V *cur = first_buffer(h, l, z, w);
  auto other = [&](V *c) { return c == z ? w.z2[l] : z; };
  // pre-smoothing from zero
  const bool fold = folds_first(h, l, sizeof(T) == 4);
  if (!pre_done && !fold) O::cheb_first(F, r, cur, nb, sm.first, s);
  for (int it = 1; it < h->nu_pre; ++it) {
    V *out = other(cur);
    const SmoothStep &st = sm.pre[it];
    // folded: x_1 is formed from r by the second step (prev 3) and by the third (prev 4, its x_{k-1})
    const int prev = fold && it <= 2 ? it + 2 : st.prev;
    timed_cheb<T, V, KB>(h, l, F, r, cur, out, prev, nb, st.c1, st.c2, nullptr, 0, w.status, s, sm.first);
    cur = out;
  }
  // coarse-grid correction
  O::residual(F, r, cur, w.res[l], nb, s);
  O::restrict_(F, C, w.res[l], w.r[l + 1], nb, s);
  Rhs<T, V> rc;
  rc.part = w.r[l + 1];
  vcycle<T, V, KB>(h, l + 1, rc, w.z[l + 1], w, nb, s);
  O::prolong_add(F, C, w.z[l + 1], cur, nb, s);
  // post-smoothing (same polynomial, nonzero start)
  for (int it = 0; it < h->nu_post; ++it) {
    const bool last = it + 1 == h->nu_post;
    V *out = other(cur);
    const SmoothStep &st = sm.post[it];
    timed_cheb<T, V, KB>(h, l, F, r, cur, out, st.prev, nb, st.c1, st.c2, last ? dot_partial : nullptr, gx, w.status,
                         s);
    cur = out;
  }
  if (cur != z) cudaMemcpyAsync(z, cur, sizeof(V) * F.dims.N * KB * nb, cudaMemcpyDeviceToDevice, s);
}

// ------------------------------------------------------------------ loops
// How the iteration loops of a solve are driven:
//  LOOP_HOST   -- the host polls the device's convergence counter (one pinned
//                 read per check_every iterations) and stops issuing work;
//  LOOP_FIXED  -- a fixed iteration count, no host synchronisation;
//  LOOP_DEVICE -- the stream is being captured into a CUDA graph and every
//                 loop becomes a conditional WHILE node whose condition a
//                 one-thread kernel sets from the device-side counters, so a
//                 graph launch runs the adaptive solve with no host involvement.
enum { LOOP_HOST = 0, LOOP_FIXED = 1, LOOP_DEVICE = 2 };

// Creates the condition handle of a WHILE node in the graph being captured on s.
int while_handle(cudaStream_t s, cudaGraphConditionalHandle *hc) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr));
  if (st != cudaStreamCaptureStatusActive || !g) return fail(DC_ERR_STATE, "device-side loop outside stream capture");
  CK(cudaGraphConditionalHandleCreate(hc, g, 0, 0));
  return 0;
}

// Appends the WHILE node after the work captured so far on s and starts
// recording its body on `body`.
int open_while(cudaStream_t s, cudaGraphConditionalHandle hc, cudaStream_t body) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *edges = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, &edges, &nd));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = hc;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, edges, nd, &p));
  CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  CK(cudaStreamBeginCaptureToGraph(body, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                   cudaStreamCaptureModeThreadLocal));
  return 0;
}

int close_while(cudaStream_t body) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamEndCapture(body, &g));
  return 0;
}

int body_stream(dc_handle *h, int depth, cudaStream_t *out) {
  if (!h->body_s[depth]) CK(cudaStreamCreateWithFlags(&h->body_s[depth], cudaStreamNonBlocking));
  *out = h->body_s[depth];
  return 0;
}

// ------------------------------------------------------------------ PCG
// Solves A x = r0 (x = 0 on entry, r holds r0 and is overwritten by the residual).
// init_active (nullable): RHS with init_active[r] == 0 are left untouched.
// `depth` selects the body stream of a LOOP_DEVICE loop (0 unless nested in a
// refinement loop); total_max caps the iterations summed over sweeps.
// rr_part (nullable): per-block partials of |r|^2 (stride gx) left by the
// kernel that wrote r; without them they are computed here.
template <typename T, typename V, int KB>
int pcg(dc_handle *h, T *x, T *r, V *p, T *q, V *z, const MGWork<V> &w, const Scal &sc, int nb, int gx,
        const int *init_active, const double *tol2, int maxit, int total_max, int *iters, cudaStream_t s,
        int loop = LOOP_HOST, int depth = 0, bool x_unset = false, const double *rr_part = nullptr) {
  using O = Ops<T, V, KB>;
  const Level &F = h->lv[0];
  const long long N = F.dims.N;
  const int Kp = nb * KB;
  const bool fused = h->lv.size() > 1;
  // Multigrid vectors narrower than T (fp16): the V-cycle input is the
  // residual scaled to unit norm per RHS (scale from the latest |r|^2) and
  // stored in V (w.r0), so its vectors stay in range and the finest level
  // streams 2-byte residuals.  PCG is invariant under the per-iteration
  // scaling of z; the fused r.z partials (from w.r0) are divided by the scale.
  const bool split = !std::is_same<T, V>::value;
  float *scale = split ? sc.scale : nullptr;
  const float *rz_div = split && fused ? sc.scale : nullptr;
  Rhs<T, V> rin;
  if (split)
    rin.part = w.r0;
  else
    rin.full = r;
  if (init_active)
    CK(cudaMemcpyAsync(sc.active, init_active, sizeof(int) * Kp, cudaMemcpyDeviceToDevice, s));
  else
    fill_int(sc.active, Kp, 1, s);
  CK(cudaMemsetAsync(sc.status, 0, sizeof(int), s));
  const double *rrp = rr_part;
  if (!rrp) {
    O::dot(N, nb, r, r, sc.part_b, gx, s);
    rrp = sc.part_b;
  }
  sum_partials(Kp, KB, gx, rrp, sc.bb, s, scale);
  if (split) O::scale_to(N, nb, r, scale, w.r0, s);
  vcycle<T, V, KB>(h, 0, rin, z, w, nb, s, false, sc.part_c, gx);
  if (!fused) O::dot_z(N, nb, r, z, sc.part_c, gx, s);
  CK(cudaMemsetAsync(sc.n_active, 0, sizeof(int), s));
  pcg_beta(Kp, KB, gx, sc.part_c, rrp, sc.rz, sc.rr, sc.bb, tol2, sc.active, sc.beta, sc.beta32, sc.n_active, 1, s,
           rz_div, scale);
  O::copy_z(N, nb, p, z, s);
  const double c0 = smoother(h->smoother_kind, F.lmax, h->cheb_ratio, h->nu_pre, h->nu_post).first;
  V *z1 = fused ? first_buffer(h, 0, z, w) : nullptr;
  // one PCG iteration on stream st.  With x_unset (host-driven loops only) x holds no value yet and the
  // first iteration writes it (x = alpha p) instead of adding to zeros.
  bool x_zero = x_unset && loop != LOOP_DEVICE;
  auto iteration = [&](cudaStream_t st) {
    O::apply_v(F, p, q, nb, sc.part_a, gx, st);
    pcg_alpha(Kp, KB, gx, sc.part_a, sc.rz, sc.active, sc.alpha, sc.alpha32, sc.status, sc.n_active, st);
    if (fused) {
      O::update_xr(N, nb, x, r, p, q, sc.alpha, sc.alpha32, sc.part_b, gx, &F, c0, z1, scale, w.r0, st, x_zero);
      vcycle<T, V, KB>(h, 0, rin, z, w, nb, st, true, sc.part_c, gx);
    } else {
      O::update_xr(N, nb, x, r, p, q, sc.alpha, sc.alpha32, sc.part_b, gx, nullptr, 0.0, nullptr, nullptr, nullptr, st,
                   x_zero);
      if (split) O::scale_to(N, nb, r, scale, w.r0, st);
      vcycle<T, V, KB>(h, 0, rin, z, w, nb, st);
      O::dot_z(N, nb, r, z, sc.part_c, gx, st);
    }
    pcg_beta(Kp, KB, gx, sc.part_c, sc.part_b, sc.rz, sc.rr, sc.bb, tol2, sc.active, sc.beta, sc.beta32, sc.n_active, 0, st,
             rz_div, scale);
    O::p_update(N, nb, p, z, sc.beta, sc.beta32, st);
    x_zero = false;
  };
  if (loop == LOOP_DEVICE) {
    int rc;
    cudaGraphConditionalHandle hc;
    cudaStream_t sb;
    if ((rc = body_stream(h, depth, &sb))) return rc;
    if ((rc = while_handle(s, &hc))) return rc;
    inner_loop_cond(hc, 1, sc.n_active, sc.status, sc.loop, maxit, total_max, s);
    if ((rc = open_while(s, hc, sb))) return rc;
    iteration(sb);
    inner_loop_cond(hc, 0, sc.n_active, sc.status, sc.loop, maxit, total_max, sb);
    *iters = 0;
    return close_while(sb);
  }
  int it = 0;
  int since = 0;
  for (it = 0; it < maxit; ++it) {
    iteration(s);
    if (loop == LOOP_FIXED) continue;  // fixed iteration count: no host synchronisation
    if (++since >= h->check_every || it + 1 == maxit) {
      since = 0;
      CK(cudaMemcpyAsync(h->h_mail, sc.n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(h->h_mail + 1, sc.status, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaEventRecord(h->ev, s));
      CK(cudaEventSynchronize(h->ev));
      if (h->h_mail[1] != 0) {
        *iters = it + 1;
        return fail(DC_ERR_BREAKDOWN, (h->h_mail[1] & 8) ? "multigrid smoothing: a shared-memory copy did not complete"
                                                           : "PCG breakdown: non-positive or non-finite p.Ap");
      }
      if (h->h_mail[0] == 0) {
        ++it;
        break;
      }
    }
  }
  *iters = it;
  if (loop == LOOP_FIXED) return 0;
  CK(cudaMemcpyAsync(h->h_mail, sc.n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->ev, s));
  CK(cudaEventSynchronize(h->ev));
  return h->h_mail[0] == 0 ? 0 : DC_ERR_NOT_CONVERGED;
}

// Inner solves aim at 0.3x the remaining outer gap (squared: 0.09), down to a
// floor that fp32 iterations reach reliably; 3e-5 makes two refinement sweeps
// the usual count at rtol 1e-9 (measured: 196 ms vs 226 ms with a 1e-4 floor
// on the 1M-node, 256-RHS forward).
constexpr double kSafety2 = 0.09;
constexpr double kInnerRtol = 3e-5;

template <int KB>
int solve_kb(dc_handle *h, int mode, const double *b, double *x, int k, double rtol, int maxit, double inner_rtol,
             int inner_maxit, SolveWS &w, dc_stats *st, cudaStream_t s, int loop = LOOP_HOST, int max_outer = 30) {
  const bool fixed = loop == LOOP_FIXED;
  const bool device = loop == LOOP_DEVICE;
  const Level &F = h->lv[0];
  const long long N = F.dims.N;
  const int nb = w.nb, Kp = w.Kp, gx = w.gx;
  // the mixed Robin solve splits b straight from the column-major input (below); the others pack it
  const bool fused_split = mode != DC_MODE_FP64 && h->robin;
  if (!fused_split) pack_colmajor<double>(b, N, k, KB, nb, w.B64, s);
  if (!h->robin) {
    // Neumann: the reference pins row 0 of A to the identity
    // (resistivity/simulation.py:535-540).  Its solution solves the symmetric
    // singular system with row 0 of the RHS replaced by -(sum of the other
    // rows) (the compatible RHS), shifted so that u_0 = b_0.
    neumann_rhs(b, N, k, KB, w.B64, w.sc.rr64, s);
  }
  // the host-driven mixed solve writes its first correction into x instead of adding it to zeros
  bool first_sweep = mode != DC_MODE_FP64 && !device;
  if (!first_sweep) CK(cudaMemsetAsync(w.X64, 0, sizeof(double) * N * Kp, s));
  CK(cudaMemsetAsync(w.sc.loop, 0, 4 * sizeof(int), s));
  CK(cudaMemsetAsync(w.sc.status, 0, sizeof(int), s));  // read by the device-loop conditions before the first PCG
  int total_it = 0, outer = 0, status = 0;
  if (mode == DC_MODE_FP64) {
    CK(cudaMemcpyAsync(w.R64, w.B64, sizeof(double) * N * Kp, cudaMemcpyDeviceToDevice, s));
    int it = 0;
    fill_double(w.sc.tol2, Kp, rtol * rtol, s);
    status = pcg<double, double, KB>(h, w.X64, w.R64, w.p64, w.q64, w.z64, w.mg64, w.sc, nb, gx, nullptr,
                                     w.sc.tol2, maxit,
                             maxit, &it, s, loop, 0);
    if (status == DC_ERR_BREAKDOWN || (device && status)) return status;
    total_it = it;
    outer = 1;
    // true residual
    ir_residual<KB>(F, w.B64, w.X64, nullptr, nullptr, nb, w.sc.active, w.sc.part_a, gx, s);
    sum_partials(Kp, KB, gx, w.sc.part_a, w.sc.rr64, s);
    Ops<double, double, KB>::dot(N, nb, w.B64, w.B64, w.sc.part_b, gx, s);
    sum_partials(Kp, KB, gx, w.sc.part_b, w.sc.bb64, s);
    outer_check(Kp, w.sc.rr64, w.sc.bb64, rtol * rtol, w.sc.active_out, w.sc.n_active_out, w.sc.maxrel, nullptr,
                0.0, 0.0, s);
  } else {
    // Refinement in double-float: b and x as (hi, lo) fp32 pairs in the B64-sized regions R64 and X64.
    float *bh = reinterpret_cast<float *>(w.R64), *bl = bh + (size_t)N * Kp;
    float *xh = reinterpret_cast<float *>(w.X64), *xl = xh + (size_t)N * Kp;
    // also r32 = fp32(b), the first residual
    if (fused_split)
      pack_split_df(b, N, k, KB, nb, bh, bl, w.r32, s);
    else
      split_df(w.B64, (long long)N * Kp, bh, bl, w.r32, s);
    // |b|^2 from the fp32 copy of b (the stopping test needs it to ~1e-6 relatively; an fp64 dot runs at
    // the fp64 rate), initial outer flags.  part_a holds the |r32|^2 partials at the start of every sweep
    // (from here, then from the residual kernel), and the inner PCG starts from them.
    Ops<float, float, KB>::dot(N, nb, w.r32, w.r32, w.sc.part_a, gx, s);
    sum_partials(Kp, KB, gx, w.sc.part_a, w.sc.bb64, s);
    sum_partials(Kp, KB, gx, w.sc.part_a, w.sc.rr64, s);
    outer_check(Kp, w.sc.rr64, w.sc.bb64, rtol * rtol, w.sc.active_out, w.sc.n_active_out, w.sc.maxrel, w.sc.tol2,
                inner_rtol * inner_rtol, kSafety2, s);
    // one refinement sweep on stream so: inner fp32 PCG, accumulate, fp64 residual, new flags
    auto sweep = [&](cudaStream_t so, int inner_cap, int *it) -> int {
      // the inner correction starts at zero: a host-driven PCG that runs at least one iteration writes it
      // in its first update, otherwise it is zeroed here
      const bool unset = !device && inner_cap >= 1;
      if (!unset) CK(cudaMemsetAsync(w.d32, 0, sizeof(float) * N * Kp, so));
      int rc;
      if (w.storage == DC_MG_FP16)
        rc = pcg<float, __half, KB>(h, w.d32, w.r32, (__half *)w.pv, w.q32, (__half *)w.zv, w.mg16, w.sc, nb, gx,
                                    w.sc.active_out, w.sc.tol2, inner_cap, maxit, it, so, loop, device ? 1 : 0, unset,
                                    w.sc.part_a);
      else if (w.storage == DC_MG_BF16)
        rc = pcg<float, __nv_bfloat16, KB>(h, w.d32, w.r32, (__nv_bfloat16 *)w.pv, w.q32, (__nv_bfloat16 *)w.zv, w.mgb16, w.sc, nb,
                                           gx, w.sc.active_out, w.sc.tol2, inner_cap, maxit, it, so, loop,
                                           device ? 1 : 0, unset, w.sc.part_a);
      else
        rc = pcg<float, float, KB>(h, w.d32, w.r32, (float *)w.pv, w.q32, (float *)w.zv, w.mg32, w.sc, nb, gx,
                                   w.sc.active_out, w.sc.tol2, inner_cap, maxit, it, so, loop, device ? 1 : 0, unset,
                                   w.sc.part_a);
      if (rc == DC_ERR_BREAKDOWN || (device && rc)) return rc;
      if (first_sweep) {
        ir_set_df((long long)N * Kp, xh, xl, w.d32, so);
        first_sweep = false;
      } else {
        ir_accumulate_df((long long)N * Kp, xh, xl, w.d32, so);
      }
      ir_residual_df<KB>(F, h->d_cdf_hi, h->d_cdf_lo, bh, bl, xh, xl, w.r32, nb, w.sc.active_out, w.sc.part_a, gx,
                         so);
      sum_partials(Kp, KB, gx, w.sc.part_a, w.sc.rr64, so);
      outer_check(Kp, w.sc.rr64, w.sc.bb64, rtol * rtol, w.sc.active_out, w.sc.n_active_out, w.sc.maxrel,
                  w.sc.tol2, inner_rtol * inner_rtol, kSafety2, so);
      return 0;
    };
    if (device) {
      int rc, it = 0;
      cudaGraphConditionalHandle ho;
      cudaStream_t so;
      if ((rc = body_stream(h, 0, &so))) return rc;
      if ((rc = while_handle(s, &ho))) return rc;
      outer_loop_cond(ho, 1, w.sc.n_active_out, w.sc.status, w.sc.loop, max_outer, maxit, s);
      if ((rc = open_while(s, ho, so))) return rc;
      if ((rc = sweep(so, inner_maxit, &it))) return rc;
      outer_loop_cond(ho, 0, w.sc.n_active_out, w.sc.status, w.sc.loop, max_outer, maxit, so);
      if ((rc = close_while(so))) return rc;
    } else {
      for (outer = 0; outer < max_outer;) {
        if (!fixed) {
          CK(cudaMemcpyAsync(h->h_mail, w.sc.n_active_out, sizeof(int), cudaMemcpyDeviceToHost, s));
          CK(cudaEventRecord(h->ev, s));
          CK(cudaEventSynchronize(h->ev));
          if (h->h_mail[0] == 0) break;
          if (total_it >= maxit) {
            status = DC_ERR_NOT_CONVERGED;
            break;
          }
        }
        int it = 0;
        int rc = sweep(s, fixed ? inner_maxit : std::min(inner_maxit, maxit - total_it), &it);
        total_it += it;
        if (rc == DC_ERR_BREAKDOWN) return rc;
        ++outer;
      }
      if (outer >= max_outer && !fixed) status = DC_ERR_NOT_CONVERGED;
    }
    if (first_sweep) CK(cudaMemsetAsync(w.X64, 0, sizeof(double) * N * Kp, s));  // no sweep ran: x = 0
  }
  if (mode == DC_MODE_MIXED)
    unpack_colmajor_df(reinterpret_cast<const float *>(w.X64), reinterpret_cast<const float *>(w.X64) + (size_t)N * Kp,
                       N, k, KB, x, s);
  else
    unpack_colmajor<double>(w.X64, N, k, KB, x, s);
  if (!h->robin) neumann_shift(b, N, k, x, s);
  if (fixed || device) {  // the convergence state stays on the device (dc_solve_check)
    if (st) {
      st->iterations = total_it;
      st->outer = outer;
      st->status = 0;
      st->n_levels = (int)h->lv.size();
      st->max_rel_res = -1.0;
    }
    return 0;
  }
  CK(cudaMemcpyAsync(h->h_maild, w.sc.maxrel, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h->h_mail, w.sc.n_active_out, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->ev, s));
  CK(cudaEventSynchronize(h->ev));
  if (h->h_mail[0] != 0) status = DC_ERR_NOT_CONVERGED;
  if (st) {
    st->iterations = total_it;
    st->outer = outer;
    st->status = status;
    st->n_levels = (int)h->lv.size();
    st->max_rel_res = h->h_maild[0];
  }
  if (status) return fail(status, "solver did not reach the requested tolerance");
  return 0;
}

int solve_dispatch(dc_handle *h, int mode, const double *b, double *x, int k, double rtol, int maxit,
                   double inner_rtol, int inner_maxit, SolveWS &w, dc_stats *st, cudaStream_t s, int loop,
                   int max_outer) {
  switch (w.KB) {
    case 32: return solve_kb<32>(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, w, st, s, loop, max_outer);
    case 16: return solve_kb<16>(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, w, st, s, loop, max_outer);
    case 8: return solve_kb<8>(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, w, st, s, loop, max_outer);
    case 4: return solve_kb<4>(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, w, st, s, loop, max_outer);
    case 2: return solve_kb<2>(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, w, st, s, loop, max_outer);
    default: return solve_kb<1>(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, w, st, s, loop, max_outer);
  }
}

// One refinement sweep of a lane session (the sweep of solve_kb's mixed
// branch): inner fp32 PCG on the active lanes to their own tolerances,
// x += d, double-float residual, new per-lane flags and tolerances.
template <int KB>
int lanes_sweep_kb(dc_handle *h, SolveWS &w, double rtol, double inner_rtol, int inner_cap, int nb_use, int *it,
                   cudaStream_t s) {
  const Level &F = h->lv[0];
  const long long N = F.dims.N;
  // only the leading nb_use RHS blocks hold active lanes (the caller's promise): the sweep's kernels,
  // partial sums and flags cover those; the other lanes' state is left as it is
  const int nb = nb_use > 0 && nb_use < w.nb ? nb_use : w.nb, Kp = nb * KB, gx = w.gx;
  float *bh = reinterpret_cast<float *>(w.R64), *bl = bh + (size_t)N * w.Kp;
  float *xh = reinterpret_cast<float *>(w.X64), *xl = xh + (size_t)N * w.Kp;
  CK(cudaMemsetAsync(w.sc.status, 0, sizeof(int), s));
  // the inner correction starts at zero; with at least one iteration its first update writes it
  const bool unset = inner_cap >= 1;
  if (!unset) CK(cudaMemsetAsync(w.d32, 0, sizeof(float) * N * Kp, s));
  int rc;
  if (w.storage == DC_MG_FP16)
    rc = pcg<float, __half, KB>(h, w.d32, w.r32, (__half *)w.pv, w.q32, (__half *)w.zv, w.mg16, w.sc, nb, gx,
                                w.sc.active_out, w.sc.tol2, inner_cap, inner_cap, it, s, LOOP_HOST, 0, unset);
  else if (w.storage == DC_MG_BF16)
    rc = pcg<float, __nv_bfloat16, KB>(h, w.d32, w.r32, (__nv_bfloat16 *)w.pv, w.q32, (__nv_bfloat16 *)w.zv, w.mgb16,
                                       w.sc, nb, gx, w.sc.active_out, w.sc.tol2, inner_cap, inner_cap, it, s, LOOP_HOST, 0,
                                       unset);
  else
    rc = pcg<float, float, KB>(h, w.d32, w.r32, (float *)w.pv, w.q32, (float *)w.zv, w.mg32, w.sc, nb, gx,
                               w.sc.active_out, w.sc.tol2, inner_cap, inner_cap, it, s, LOOP_HOST, 0, unset);
  if (rc == DC_ERR_BREAKDOWN) return rc;
  ir_accumulate_df((long long)N * Kp, xh, xl, w.d32, s);
  ir_residual_df<KB>(F, h->d_cdf_hi, h->d_cdf_lo, bh, bl, xh, xl, w.r32, nb, w.sc.active_out, w.sc.part_a, gx, s);
  sum_partials(Kp, KB, gx, w.sc.part_a, w.sc.rr64, s);
  outer_check(Kp, w.sc.rr64, w.sc.bb64, rtol * rtol, w.sc.active_out, w.sc.n_active_out, w.sc.maxrel, w.sc.tol2,
              inner_rtol * inner_rtol, kSafety2, s);
  return 0;
}

int lanes_sweep(dc_handle *h, SolveWS &w, double rtol, double inner_rtol, int inner_cap, int nb_use, int *it,
                cudaStream_t s) {
  switch (w.KB) {
    case 32: return lanes_sweep_kb<32>(h, w, rtol, inner_rtol, inner_cap, nb_use, it, s);
    case 16: return lanes_sweep_kb<16>(h, w, rtol, inner_rtol, inner_cap, nb_use, it, s);
    case 8: return lanes_sweep_kb<8>(h, w, rtol, inner_rtol, inner_cap, nb_use, it, s);
    case 4: return lanes_sweep_kb<4>(h, w, rtol, inner_rtol, inner_cap, nb_use, it, s);
    case 2: return lanes_sweep_kb<2>(h, w, rtol, inner_rtol, inner_cap, nb_use, it, s);
    default: return lanes_sweep_kb<1>(h, w, rtol, inner_rtol, inner_cap, nb_use, it, s);
  }
}

}  // namespace

// A continuous-batching session: the mixed solve's state for a fixed set of
// lanes, kept between calls.
struct dc_lanes {
  dc_handle *h = nullptr;
  SolveWS w{};
  void *own = nullptr;
  double rtol = 1e-9, inner_rtol = 3e-5;
  int inner_maxit = 200;
  int nb_use = 0;  // RHS blocks the sweeps cover (0: all; dc_lanes_set_extent)
};

// ====================================================================== C ABI
extern "C" {

const char *dc_last_error(void) { return dc::last_error().c_str(); }

int dc_create(int nx, int ny, int nz, const double *hx, const double *hy, const double *hz, const double *bface,
              dc_handle **out) {
  if (!out) return fail(DC_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (nx < 1 || ny < 1 || nz < 1) return fail(DC_ERR_ARG, "cell counts must be positive");
  if (!hx || !hy || !hz) return fail(DC_ERR_ARG, "cell widths are NULL");
  const long long N = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  if (N >= (1LL << 31)) return fail(DC_ERR_ARG, "mesh too large (nodes must fit in int32)");
  for (int i = 0; i < nx; ++i) if (!(hx[i] > 0) || !std::isfinite(hx[i])) return fail(DC_ERR_ARG, "bad hx");
  for (int i = 0; i < ny; ++i) if (!(hy[i] > 0) || !std::isfinite(hy[i])) return fail(DC_ERR_ARG, "bad hy");
  for (int i = 0; i < nz; ++i) if (!(hz[i] > 0) || !std::isfinite(hz[i])) return fail(DC_ERR_ARG, "bad hz");
  int dev = 0, nsm = 152;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  set_sm_count(nsm);
  std::unique_ptr<dc_handle> h(new (std::nothrow) dc_handle());
  if (!h) return fail(DC_ERR_NOMEM, "host allocation failed");
  h->robin = bface != nullptr;
  Level L0;
  L0.nx = nx;
  L0.ny = ny;
  L0.nz = nz;
  L0.hx.assign(hx, hx + nx);
  L0.hy.assign(hy, hy + ny);
  L0.hz.assign(hz, hz + nz);
  set_dims(L0);
  set_bface_offsets(L0);
  L0.bface.assign(L0.bface_off[6], 0.0);
  if (bface) {
    for (long long i = 0; i < L0.bface_off[6]; ++i) {
      if (!std::isfinite(bface[i])) return fail(DC_ERR_ARG, "bad Robin face weight");
      L0.bface[i] = bface[i];
    }
  }
  h->lv.push_back(L0);
  CK(cudaMallocHost((void **)&h->h_mail, 4 * sizeof(int)));
  CK(cudaMallocHost((void **)&h->h_maild, 2 * sizeof(double)));
  CK(cudaEventCreateWithFlags(&h->ev, cudaEventDisableTiming));
  *out = h.release();
  return 0;
}

void dc_destroy(dc_handle *h) {
  if (!h) return;
  cudaDeviceSynchronize();
  for (auto &L : h->lv) free_level(L, true);
  cudaFree(h->dlev.d_coef64);
  cudaFree(h->dlev.d_coef32);
  cudaFree(h->dlev.d_invd64);
  cudaFree(h->dlev.d_invd32);
  cudaFree(h->d_P);
  cudaFree(h->d_Q);
  cudaFree(h->d_Ainv64);
  cudaFree(h->d_Ainv32);
  cudaFree(h->d_cdf_hi);
  cudaFree(h->d_cdf_lo);
  cudaFree(h->d_dense);
  cudaFree(h->d_work);
  cudaFree(h->d_flag);
  cudaFree(h->d_lmax);
  cudaFree(h->ws);
  if (h->h_mail) cudaFreeHost(h->h_mail);
  if (h->h_maild) cudaFreeHost(h->h_maild);
  if (h->ev) cudaEventDestroy(h->ev);
  for (auto st : h->body_s)
    if (st) cudaStreamDestroy(st);
  for (auto &e : h->prof_ev) cudaEventDestroy(e);
  delete h;
}

int dc_set_params(dc_handle *h, int nu_pre, int nu_post, double cheb_ratio, int coarse_max, int check_every) {
  if (!h) return fail(DC_ERR_ARG, "handle is NULL");
  if (coarse_max > 0 && h->built && coarse_max != h->coarse_max)
    return fail(DC_ERR_STATE, "coarse_max must be set before the first dc_set_model");
  if (nu_pre > 0) h->nu_pre = nu_pre;
  if (nu_post > 0) h->nu_post = nu_post;
  if (cheb_ratio > 1.0) h->cheb_ratio = cheb_ratio;
  if (coarse_max > 0) {
    if (coarse_max > 4096) return fail(DC_ERR_ARG, "coarse_max must be <= 4096");
    h->coarse_max = coarse_max;
  }
  if (check_every > 0) h->check_every = check_every;
  return 0;
}

int dc_set_coarsening(dc_handle *h, double merge) {
  if (!h) return fail(DC_ERR_ARG, "handle is NULL");
  if (!(merge == 0.0 || (merge >= 1.0 && merge <= 16.0)))
    return fail(DC_ERR_ARG, "coarsening factor must be 0 (full coarsening) or in [1, 16]");
  if (h->built && merge != h->coarsen_merge)
    return fail(DC_ERR_STATE, "the coarsening must be set before the first dc_set_model");
  h->coarsen_merge = merge;
  return 0;
}

int dc_set_rhs_block(dc_handle *h, int kb) {
  if (!h) return fail(DC_ERR_ARG, "handle is NULL");
  if (kb != 0 && kb != 1 && kb != 2 && kb != 4 && kb != 8 && kb != 16 && kb != 32)
    return fail(DC_ERR_ARG, "RHS block width must be 0 (automatic) or a power of two <= 32");
  h->kb_force = kb;
  return 0;
}

int dc_set_mg_storage(dc_handle *h, int storage) {
  if (!h) return fail(DC_ERR_ARG, "null handle");
  if (storage != DC_MG_FP32 && storage != DC_MG_FP16 && storage != DC_MG_BF16)
    return fail(DC_ERR_ARG, "multigrid storage must be DC_MG_FP32, DC_MG_FP16 or DC_MG_BF16");
  h->mg_storage = storage;
  return 0;
}

int dc_set_smoother(dc_handle *h, int kind) {
  if (!h) return fail(DC_ERR_ARG, "null handle");
  if (kind != 1 && kind != 4) return fail(DC_ERR_ARG, "smoother kind must be 1 or 4");
  h->smoother_kind = kind;
  return 0;
}

int dc_set_coarse_operator(dc_handle *h, int mode) {
  if (!h) return fail(DC_ERR_ARG, "null handle");
  if (mode < 0 || mode > 2) return fail(DC_ERR_ARG, "coarse operator mode must be 0, 1 or 2");
  h->coarse_op = mode;
  return 0;
}

int dc_set_staging(dc_handle *h, int enable) {
  if (!h) return fail(DC_ERR_ARG, "null handle");
  h->bulk_staging = enable != 0;
  h->bulk_shape = enable > 1 ? enable : 0;
  return 0;
}

int dc_level_info(dc_handle *h, int lvl, int *n_levels, long long *nodes, int *cells3) {
  if (!h) return fail(DC_ERR_ARG, "handle is NULL");
  if (!h->built) return fail(DC_ERR_STATE, "hierarchy is built by dc_set_model");
  if (n_levels) *n_levels = (int)h->lv.size();
  if (lvl < 0 || lvl >= (int)h->lv.size()) return fail(DC_ERR_ARG, "level out of range");
  if (nodes) *nodes = h->lv[lvl].dims.N;
  if (cells3) {
    cells3[0] = h->lv[lvl].nx;
    cells3[1] = h->lv[lvl].ny;
    cells3[2] = h->lv[lvl].nz;
  }
  return 0;
}

// The finest level of a cell-centred problem: its operator comes from the cell resistivity
// (dc_cc.cu), the coarse levels from the dual conductivity in L0.d_sigma.
struct CCFine {
  const double *rho, *hp, *bw;
};

static int set_model_impl(dc_handle *h, const double *sigma_dev, const CCFine *cc, cudaStream_t s) {
  if (!h->built) {
    int rc = build_hierarchy(h);
    if (rc) return rc;
  }
  Level &L0 = h->lv[0];
  const long long nC = (long long)L0.nx * L0.ny * L0.nz;
  if (cc)
    cc_dual_sigma(cc->rho, L0.dims.Nx, L0.dims.Ny, L0.dims.Nz, L0.d_sigma, s);
  else
    CK(cudaMemcpyAsync(L0.d_sigma, sigma_dev, sizeof(double) * nC, cudaMemcpyDeviceToDevice, s));
  for (size_t l = 0; l + 1 < h->lv.size(); ++l) coarsen_sigma(h->lv[l], h->lv[l + 1], s);
  // coefficients of every level, then one read-back of the levels' Gershgorin bounds
  const size_t nl = h->lv.size();
  CK(cudaMemsetAsync(h->d_lmax, 0, sizeof(unsigned long long) * nl, s));
  for (size_t l = 0; l < nl; ++l) {
    if (l == 0 && cc)
      cc_coef_build(L0, cc->rho, cc->hp, cc->bw, h->d_lmax, s);
    else if (l > 0 && h->coarse_op)
      coef_galerkin(h->lv[l - 1], h->lv[l], h->coarse_op, h->d_lmax + l, s);
    else
      coef_build(h->lv[l], h->robin, h->d_lmax + l, s);
  }
  std::vector<unsigned long long> bits(nl, 0);
  CK(cudaMemcpyAsync(bits.data(), h->d_lmax, sizeof(unsigned long long) * nl, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (size_t l = 0; l < nl; ++l) {
    double lm;
    std::memcpy(&lm, &bits[l], sizeof(lm));
    if (!(lm > 0.0) || !std::isfinite(lm)) return fail(DC_ERR_ARG, "conductivity must be positive and finite");
    h->lv[l].lmax = lm;
  }
  for (size_t l = 1; l + 1 < nl; ++l) rows_dinv(h->lv[l], s);
  if (!h->d_cdf_hi) {
    int rc;
    if ((rc = dalloc(&h->d_cdf_hi, L0.dims.N))) return rc;
    if ((rc = dalloc(&h->d_cdf_lo, L0.dims.N))) return rc;
  }
  coef_split_df(L0, h->d_cdf_hi, h->d_cdf_lo, s);
  CK(cudaMemsetAsync(h->d_flag, 0, sizeof(int), s));
  dense_assemble(h->lv.back(), h->d_dense, s);
  // The Neumann operator is singular (constants); its coarsest matrix is
  // pinned at node 0 so that the V-cycle stays an SPD preconditioner.
  if (!h->robin) dense_pin0(h->d_dense, h->nc, s);
  dense_cholesky_inverse(h->d_dense, h->d_work, h->nc, h->d_Ainv64, h->d_Ainv32, h->d_flag, s);
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, h->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  if (flag) return fail(DC_ERR_ARG, "coarsest operator is not positive definite (bad sigma)");
  h->model_set = true;
  return 0;
}

int dc_set_model(dc_handle *h, const double *sigma_dev, void *stream) {
  if (!h || !sigma_dev) return fail(DC_ERR_ARG, "NULL argument");
  return set_model_impl(h, sigma_dev, nullptr, (cudaStream_t)stream);
}

int dc_set_model_cc(dc_handle *h, const double *rho_dev, const double *hp_dev, const double *bw_dev, void *stream) {
  if (!h || !rho_dev || !hp_dev) return fail(DC_ERR_ARG, "NULL argument");
  if (h->lv[0].nx < 1 || h->lv[0].ny < 1 || h->lv[0].nz < 1)
    return fail(DC_ERR_ARG, "the cell-centre grid needs at least 2 cells per axis");
  CCFine cc{rho_dev, hp_dev, bw_dev};
  return set_model_impl(h, nullptr, &cc, (cudaStream_t)stream);
}

int dc_apply(dc_handle *h, const double *x, double *y, int k, void *stream) {
  if (!h || !x || !y || k < 1) return fail(DC_ERR_ARG, "bad argument");
  if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
  Ops<double, double, 1>::apply(h->lv[0], x, y, k, nullptr, 0, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

int dc_solve_workspace_bytes(dc_handle *h, int mode, int k, size_t *bytes) {
  if (!h || !bytes || k < 1) return fail(DC_ERR_ARG, "bad argument");
  if (k > 32 * kMaxRhsBlocks) k = 32 * kMaxRhsBlocks;
  if (mode != DC_MODE_FP64 && mode != DC_MODE_MIXED) return fail(DC_ERR_ARG, "bad mode");
  if (!h->built) {
    int rc = build_hierarchy(h);
    if (rc) return rc;
  }
  SolveWS w;
  layout_ws(h, mode, k, nullptr, w);
  *bytes = w.bytes;
  return 0;
}

static int solve_once(dc_handle *h, int mode, const double *b, double *x, int k, double rtol, int maxit,
                      double inner_rtol, int inner_maxit, void *ws, size_t ws_bytes, dc_stats *stats, void *stream);

int dc_solve(dc_handle *h, int mode, const double *b, double *x, int k, double rtol, int maxit, double inner_rtol,
             int inner_maxit, void *ws, size_t ws_bytes, dc_stats *stats, void *stream) {
  if (!h || !b || !x || k < 1) return fail(DC_ERR_ARG, "bad argument");
  const int kmax = 32 * kMaxRhsBlocks;
  if (k > kmax) {
    // solve in chunks of kmax right-hand sides (one RHS-block sweep each)
    if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
    const long long N = h->lv[0].dims.N;
    dc_stats agg{0, 0, 0, (int)h->lv.size(), 0.0};
    int rc_all = 0;
    for (int c0 = 0; c0 < k; c0 += kmax) {
      const int kc = std::min(kmax, k - c0);
      dc_stats st{};
      int rc = dc_solve(h, mode, b + (size_t)c0 * N, x + (size_t)c0 * N, kc, rtol, maxit, inner_rtol, inner_maxit,
                        ws, ws_bytes, &st, stream);
      agg.iterations = std::max(agg.iterations, st.iterations);
      agg.outer = std::max(agg.outer, st.outer);
      agg.max_rel_res = std::max(agg.max_rel_res, st.max_rel_res);
      if (rc && rc != DC_ERR_NOT_CONVERGED) return rc;
      if (rc) rc_all = rc;
    }
    agg.status = rc_all;
    if (stats) *stats = agg;
    return rc_all ? fail(rc_all, "solver did not reach the requested tolerance") : 0;
  }
  if (mode != DC_MODE_FP64 && mode != DC_MODE_MIXED) return fail(DC_ERR_ARG, "bad mode");
  if (!(rtol > 0.0) || maxit < 1) return fail(DC_ERR_ARG, "rtol must be > 0 and maxit >= 1");
  if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
  if (!(inner_rtol > 0.0)) inner_rtol = kInnerRtol;
  if (inner_maxit < 1) inner_maxit = 200;
  int rc = solve_once(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, ws, ws_bytes, stats, stream);
  if (rc == DC_ERR_BREAKDOWN && mode == DC_MODE_MIXED && h->mg_storage != DC_MG_FP32) {
    // 16-bit multigrid vectors can overflow for extreme conductivity contrasts
    // (e.g. 1e-8 S/m air cells): solve once more with fp32 multigrid storage,
    // in the handle's own workspace when the caller's is too small for it.
    const int keep = h->mg_storage;
    h->mg_storage = DC_MG_FP32;
    SolveWS w;
    layout_ws(h, mode, k, nullptr, w);
    const bool fits = ws && ws_bytes >= w.bytes;
    rc = solve_once(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, fits ? ws : nullptr, fits ? ws_bytes : 0,
                    stats, stream);
    h->mg_storage = keep;
  }
  return rc;
}

// One solve of k <= 1024 RHS (dc_solve without the chunking and the fp32 retry).
static int solve_once(dc_handle *h, int mode, const double *b, double *x, int k, double rtol, int maxit,
                      double inner_rtol, int inner_maxit, void *ws, size_t ws_bytes, dc_stats *stats, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  SolveWS w;
  layout_ws(h, mode, k, nullptr, w);
  char *base = (char *)ws;
  if (base) {
    if (ws_bytes < w.bytes) return fail(DC_ERR_NOMEM, "workspace too small");
  } else {
    if (h->ws_bytes < w.bytes) {
      CK(cudaStreamSynchronize(s));
      cudaFree(h->ws);
      h->ws = nullptr;
      h->ws_bytes = 0;
      if (cudaMalloc(&h->ws, w.bytes) != cudaSuccess) return fail(DC_ERR_NOMEM, "cannot allocate solve workspace");
      h->ws_bytes = w.bytes;
    }
    base = (char *)h->ws;
  }
  base = (char *)(((uintptr_t)base + 255) & ~(uintptr_t)255);
  layout_ws(h, mode, k, base, w);
  int rc = solve_dispatch(h, mode, b, x, k, rtol, maxit, inner_rtol, inner_maxit, w, stats, s, LOOP_HOST, 30);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(DC_ERR_CUDA, std::string("dc_solve: ") + cudaGetErrorString(e));
  return rc;
}

int dc_solve_fixed(dc_handle *h, int mode, const double *b, double *x, int k, double rtol, int n_inner, int n_outer,
                   void *ws, size_t ws_bytes, void *stream) {
  if (!h || !b || !x || k < 1 || !ws) return fail(DC_ERR_ARG, "bad argument (the workspace must be caller-provided)");
  if (mode != DC_MODE_FP64 && mode != DC_MODE_MIXED) return fail(DC_ERR_ARG, "bad mode");
  if (!(rtol > 0.0) || n_inner < 1 || n_outer < 1) return fail(DC_ERR_ARG, "rtol, n_inner, n_outer must be positive");
  if (k > 32 * kMaxRhsBlocks) return fail(DC_ERR_ARG, "k too large for one fixed solve");
  if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
  SolveWS w;
  layout_ws(h, mode, k, nullptr, w);
  if (ws_bytes < w.bytes) return fail(DC_ERR_NOMEM, "workspace too small");
  char *base = (char *)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
  layout_ws(h, mode, k, base, w);
  cudaStream_t s = (cudaStream_t)stream;
  const double inner_rtol = kInnerRtol;
  return solve_dispatch(h, mode, b, x, k, rtol, n_inner, inner_rtol, n_inner, w, nullptr, s, LOOP_FIXED, n_outer);
}

int dc_solve_check(dc_handle *h, int mode, int k, const void *ws, double *max_rel_res, int *n_unconverged,
                   int *iterations, int *sweeps) {
  if (!h || !ws || k < 1) return fail(DC_ERR_ARG, "bad argument");
  SolveWS w;
  char *base = (char *)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
  layout_ws(h, mode, k, base, w);
  double mr = 0.0;
  int na = 0, ctr[4] = {0, 0, 0, 0};
  CK(cudaMemcpy(&mr, w.sc.maxrel, sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&na, w.sc.n_active_out, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(ctr, w.sc.loop, sizeof(ctr), cudaMemcpyDeviceToHost));
  if (max_rel_res) *max_rel_res = mr;
  if (n_unconverged) *n_unconverged = na;
  if (iterations) *iterations = ctr[1];
  if (sweeps) *sweeps = mode == DC_MODE_FP64 ? 1 : ctr[2];
  return 0;
}

struct dc_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
};

void dc_graph_destroy(dc_graph *g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (auto e : g->events) cudaEventDestroy(e);
  for (auto st : g->streams) cudaStreamDestroy(st);
  delete g;
}

// Ends every capture still open on the given streams (error path).
static void abort_captures(const std::vector<cudaStream_t> &streams) {
  for (auto st : streams) {
    if (!st) continue;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t tmp = nullptr;
      cudaStreamEndCapture(st, &tmp);
      if (tmp) cudaGraphDestroy(tmp);
    }
  }
  cudaGetLastError();
}

int dc_batch_graph_create(int n, dc_handle *const *hs, int mode, const double *const *b, double *const *x,
                          const int *k, double rtol, int maxit, void *const *ws, const size_t *ws_bytes,
                          dc_graph **out) {
  if (n < 1 || !hs || !b || !x || !k || !ws || !ws_bytes || !out) return fail(DC_ERR_ARG, "bad argument");
  if (mode != DC_MODE_FP64 && mode != DC_MODE_MIXED) return fail(DC_ERR_ARG, "bad mode");
  if (!(rtol > 0.0) || maxit < 1) return fail(DC_ERR_ARG, "rtol and maxit must be positive");
  *out = nullptr;
  std::vector<SolveWS> wsl(n);
  for (int i = 0; i < n; ++i) {
    dc_handle *h = hs[i];
    if (!h || !b[i] || !x[i] || k[i] < 1 || !ws[i]) return fail(DC_ERR_ARG, "bad problem entry");
    if (k[i] > 32 * kMaxRhsBlocks) return fail(DC_ERR_ARG, "k too large for one graph-recorded solve");
    if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
    for (int j = 0; j < i; ++j)
      if (hs[j] == h) return fail(DC_ERR_ARG, "a handle appears twice in one batch");
    layout_ws(h, mode, k[i], nullptr, wsl[i]);
    if (ws_bytes[i] < wsl[i].bytes) return fail(DC_ERR_NOMEM, "workspace too small");
    layout_ws(h, mode, k[i], (char *)(((uintptr_t)ws[i] + 255) & ~(uintptr_t)255), wsl[i]);
  }
  std::unique_ptr<dc_graph, void (*)(dc_graph *)> g(new (std::nothrow) dc_graph(), dc_graph_destroy);
  if (!g) return fail(DC_ERR_NOMEM, "host allocation failed");
  for (int i = 0; i <= n; ++i) {
    cudaStream_t st;
    cudaEvent_t ev;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    g->streams.push_back(st);
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    g->events.push_back(ev);
  }
  // One capture: stream 0 forks every problem onto its own stream and joins them.
  std::vector<cudaStream_t> all(g->streams);
  for (int i = 0; i < n; ++i)
    for (auto bs : hs[i]->body_s) all.push_back(bs);
  cudaStream_t s0 = g->streams[0];
  CK(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  int rc = 0;
  if (cudaEventRecord(g->events[0], s0) != cudaSuccess) rc = fail(DC_ERR_CUDA, "event record in capture");
  const double inner_rtol = kInnerRtol;
  for (int i = 0; i < n && !rc; ++i) {
    dc_handle *h = hs[i];
    cudaStream_t st = g->streams[i + 1];
    if (cudaStreamWaitEvent(st, g->events[0], 0) != cudaSuccess) {
      rc = fail(DC_ERR_CUDA, "stream wait in capture");
      break;
    }
    const bool prof = h->prof;
    h->prof = false;  // no event records inside conditional bodies
    rc = solve_dispatch(h, mode, b[i], x[i], k[i], rtol, maxit, inner_rtol, std::min(maxit, 200), wsl[i], nullptr,
                        st, LOOP_DEVICE, 30);
    h->prof = prof;
    for (auto bs : h->body_s) all.push_back(bs);
    if (rc) break;
    if (cudaEventRecord(g->events[i + 1], st) != cudaSuccess || cudaStreamWaitEvent(s0, g->events[i + 1], 0) != cudaSuccess)
      rc = fail(DC_ERR_CUDA, "join in capture");
  }
  if (rc) {
    abort_captures(all);
    return rc;
  }
  cudaError_t e = cudaStreamEndCapture(s0, &g->graph);
  if (e != cudaSuccess) {
    abort_captures(all);
    return fail(DC_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
  }
  CK(cudaGraphInstantiate(&g->exec, g->graph, 0));
  *out = g.release();
  return 0;
}

int dc_graph_launch(dc_graph *g, void *stream) {
  if (!g || !g->exec) return fail(DC_ERR_ARG, "bad graph");
  CK(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return 0;
}

static int ensure_dlev(dc_handle *h) {
  if (h->dlev.d_coef64) return 0;
  const Level &L0 = h->lv[0];
  int rc;
  if ((rc = dalloc(&h->dlev.d_coef64, L0.dims.N))) return rc;
  if ((rc = dalloc(&h->dlev.d_coef32, L0.dims.N))) return rc;
  if ((rc = dalloc(&h->dlev.d_invd64, L0.dims.N))) return rc;
  if ((rc = dalloc(&h->dlev.d_invd32, L0.dims.N))) return rc;
  if ((rc = dalloc(&h->d_P, 3 * L0.dims.N))) return rc;
  if ((rc = dalloc(&h->d_Q, L0.dims.N))) return rc;
  return 0;
}

int dc_dadm_fwd(dc_handle *h, const double *u, const double *dsig, double *out, int k, double scale, void *stream) {
  if (!h || !u || !dsig || !out || k < 1) return fail(DC_ERR_ARG, "bad argument");
  if (!h->built) return fail(DC_ERR_STATE, "dc_set_model first");
  int rc = ensure_dlev(h);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Level D = h->lv[0];  // geometry of level 0, coefficients of dsig
  D.d_sigma = const_cast<double *>(dsig);
  D.d_coef64 = h->dlev.d_coef64;
  D.d_coef32 = h->dlev.d_coef32;
  D.d_invd64 = h->dlev.d_invd64;
  D.d_invd32 = h->dlev.d_invd32;
  coef_build(D, h->robin, h->d_lmax, s);
  Ops<double, double, 1>::apply(D, u, out, k, nullptr, 0, s);
  if (scale != 1.0) scale_vec(D.dims.N * (long long)k, out, scale, s);
  CK(cudaGetLastError());
  return 0;
}

int dc_cc_dadm_fwd(dc_handle *h, const double *rho, const double *drho, const double *hp, const double *bw,
                   const double *u, double *out, int k, double scale, void *stream) {
  if (!h || !rho || !drho || !hp || !u || !out || k < 1) return fail(DC_ERR_ARG, "bad argument");
  if (!h->built) return fail(DC_ERR_STATE, "dc_set_model_cc first");
  int rc = ensure_dlev(h);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Level D = h->lv[0];  // the cell-centre grid, coefficients of dA[drho]
  D.d_coef64 = h->dlev.d_coef64;
  D.d_coef32 = h->dlev.d_coef32;
  D.d_invd64 = h->dlev.d_invd64;
  D.d_invd32 = h->dlev.d_invd32;
  cc_dcoef_build(D.dims, rho, drho, hp, bw, D.d_coef64, s);
  Ops<double, double, 1>::apply(D, u, out, k, nullptr, 0, s);
  if (scale != 1.0) scale_vec(D.dims.N * (long long)k, out, scale, s);
  CK(cudaGetLastError());
  return 0;
}

int dc_cc_dadm_adj(dc_handle *h, const double *rho, const double *hp, const double *bw, const double *u,
                   const double *lam, int k, const double *drho_dm, double scale, double *g, void *stream) {
  if (!h || !rho || !hp || !u || !lam || !g || k < 1) return fail(DC_ERR_ARG, "bad argument");
  if (!h->built) return fail(DC_ERR_STATE, "dc_set_model_cc first");
  int rc = ensure_dlev(h);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const Level &L0 = h->lv[0];
  edge_products(u, lam, k, L0.dims, h->d_P, h->d_Q, s);
  cc_gradient(L0.dims, h->d_P, h->d_Q, rho, hp, bw, drho_dm, scale, g, s);
  CK(cudaGetLastError());
  return 0;
}

int dc_cc_face_fields(dc_handle *h, const double *rho, const double *hp, const double *bw, const double *phi, int k,
                      double *e, double *j, void *stream) {
  if (!h || !rho || !hp || !phi || k < 1 || (!e && !j)) return fail(DC_ERR_ARG, "bad argument");
  cc_face_fields(h->lv[0].dims, phi, k, rho, hp, bw, e, j, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

int dc_cc_charge(dc_handle *h, const double *hp, const double *e, int k, double eps0, double *charge,
                 double *charge_density, void *stream) {
  if (!h || !hp || !e || k < 1 || (!charge && !charge_density)) return fail(DC_ERR_ARG, "bad argument");
  cc_charge(h->lv[0].dims, e, k, hp, eps0, charge, charge_density, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

int dc_dadm_adj(dc_handle *h, const double *u, const double *lam, int k, const double *dsig, double scale, double *g,
                void *stream) {
  if (!h || !u || !lam || !g || k < 1) return fail(DC_ERR_ARG, "bad argument");
  if (!h->built) return fail(DC_ERR_STATE, "dc_set_model first");
  int rc = ensure_dlev(h);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const Level &L0 = h->lv[0];
  edge_products(u, lam, k, L0.dims, h->d_P, h->d_Q, s);
  cell_gradient(L0, h->robin, h->d_P, h->d_Q, dsig, scale, g, s);
  CK(cudaGetLastError());
  return 0;
}

int dc_edge_fields(dc_handle *h, const double *phi, int k, double *e, double *j, void *stream) {
  if (!h || !phi || k < 1 || (!e && !j)) return fail(DC_ERR_ARG, "bad argument");
  if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
  edge_fields(h->lv[0], phi, k, e, j, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

int dc_node_charge(dc_handle *h, const double *e, int k, double eps0, double *charge, double *charge_density,
                   void *stream) {
  if (!h || !e || k < 1 || !charge)
    return fail(DC_ERR_ARG, "bad argument (charge is required: the density is computed from it)");
  if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
  node_charge(h->lv[0], e, k, eps0, charge, charge_density, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

long long dc_kernel_launches(void) { return dc::launch_counter().load(); }

int dc_reg_apply(dc_handle *h, double alpha_s, double alpha_x, double alpha_y, double alpha_z, const double *v,
                 double *out, double *diag, double scale, void *stream) {
  if (!h || (!out && !diag) || (out && !v)) return fail(DC_ERR_ARG, "bad argument");
  if (!h->built) {
    int rc = build_hierarchy(h);
    if (rc) return rc;
  }
  reg_apply(h->lv[0], alpha_s, alpha_x, alpha_y, alpha_z, v, out, diag, scale, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

int dc_jtj_diag(dc_handle *h, const double *phi, int nE, int nD, const int *sa, const int *sb, const double *ia,
                const double *ib, const int *rm, const int *rn, const double *wm, const double *wn, const double *w2,
                const double *dsig, double *diag, void *stream) {
  if (!h || !phi || nE < 1 || nD < 0 || !diag) return fail(DC_ERR_ARG, "bad argument");
  if (nD > 0 && (!sa || !sb || !ia || !ib || !rm || !rn || !wm || !wn || !w2))
    return fail(DC_ERR_ARG, "NULL datum table");
  if (!h->built) {
    int rc = build_hierarchy(h);
    if (rc) return rc;
  }
  return jtj_diag_launch(h->lv[0], h->robin, phi, nE, nD, sa, sb, ia, ib, rm, rn, wm, wn, w2, dsig, diag,
                         (cudaStream_t)stream);
}

int dc_stencil_timing(dc_handle *h, int enable, double *total_ms, long long *launches, double *alg_bytes) {
  if (!h) return fail(DC_ERR_ARG, "handle is NULL");
  if (enable) {
    if (h->prof_ev.empty()) {
      h->prof_ev.resize(8192);
      for (auto &e : h->prof_ev) CK(cudaEventCreate(&e));
      h->prof_kind.assign(h->prof_ev.size() / 2, 0);
      h->prof_alg.assign(h->prof_ev.size() / 2, 0.0);
    }
    h->prof_used = 0;
    h->prof_bytes = 0.0;
    h->prof = true;
    return 0;
  }
  h->prof = false;
  double tot = 0.0;
  for (int i = 0; i + 1 < h->prof_used; i += 2) {
    CK(cudaEventSynchronize(h->prof_ev[i + 1]));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, h->prof_ev[i], h->prof_ev[i + 1]));
    tot += ms;
  }
  if (total_ms) *total_ms = tot;
  if (launches) *launches = h->prof_used / 2;
  if (alg_bytes) *alg_bytes = h->prof_bytes;
  return 0;
}

int dc_lanes_open(dc_handle *h, int lanes, double rtol, int inner_maxit, void *ws, size_t ws_bytes, dc_lanes **out,
                  int *capacity) {
  if (!h || !out || lanes < 1 || lanes > 32 * kMaxRhsBlocks || !(rtol > 0.0)) return fail(DC_ERR_ARG, "bad argument");
  if (!h->model_set) return fail(DC_ERR_STATE, "dc_set_model first");
  if (!h->robin) return fail(DC_ERR_ARG, "lane sessions need Robin boundary conditions (no row-0 pin)");
  dc_lanes *L = new dc_lanes();
  L->h = h;
  L->rtol = rtol;
  L->inner_rtol = kInnerRtol;
  L->inner_maxit = inner_maxit > 0 ? inner_maxit : 200;
  layout_ws(h, DC_MODE_MIXED, lanes, nullptr, L->w);
  char *base = (char *)ws;
  if (base) {
    if (ws_bytes < L->w.bytes) {
      delete L;
      return fail(DC_ERR_NOMEM, "workspace too small");
    }
  } else {
    if (cudaMalloc(&L->own, L->w.bytes) != cudaSuccess) {
      delete L;
      return fail(DC_ERR_NOMEM, "cannot allocate the lane workspace");
    }
    base = (char *)L->own;
  }
  base = (char *)(((uintptr_t)base + 255) & ~(uintptr_t)255);
  layout_ws(h, DC_MODE_MIXED, lanes, base, L->w);
  const size_t n = (size_t)h->lv[0].dims.N * L->w.Kp;
  SolveWS &w = L->w;
  // every lane empty: b = x = r = 0, |b|^2 = 0 (inactive)
  CK(cudaMemset(w.R64, 0, sizeof(double) * n));
  CK(cudaMemset(w.X64, 0, sizeof(double) * n));
  CK(cudaMemset(w.r32, 0, sizeof(float) * n));
  CK(cudaMemset(w.sc.bb64, 0, sizeof(double) * w.Kp));
  CK(cudaMemset(w.sc.rr64, 0, sizeof(double) * w.Kp));
  CK(cudaMemset(w.sc.active_out, 0, sizeof(int) * w.Kp));
  CK(cudaMemset(w.sc.n_active_out, 0, sizeof(int)));
  CK(cudaMemset(w.sc.tol2, 0, sizeof(double) * w.Kp));
  CK(cudaMemset(w.sc.loop, 0, 4 * sizeof(int)));
  CK(cudaDeviceSynchronize());
  *out = L;
  if (capacity) *capacity = w.Kp;
  return 0;
}

int dc_lanes_load(dc_lanes *L, const int *lanes_dev, int n, const double *b_dev, void *stream) {
  if (!L || !lanes_dev || !b_dev || n < 1 || n > L->w.Kp) return fail(DC_ERR_ARG, "bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  SolveWS &w = L->w;
  const long long N = L->h->lv[0].dims.N;
  float *bh = reinterpret_cast<float *>(w.R64), *bl = bh + (size_t)N * w.Kp;
  float *xh = reinterpret_cast<float *>(w.X64), *xl = xh + (size_t)N * w.Kp;
  lanes_load(b_dev, n, lanes_dev, N, w.KB, bh, bl, w.r32, xh, xl, w.sc.bb64, w.sc.rr64, s);
  outer_check(w.Kp, w.sc.rr64, w.sc.bb64, L->rtol * L->rtol, w.sc.active_out, w.sc.n_active_out, w.sc.maxrel,
              w.sc.tol2, L->inner_rtol * L->inner_rtol, kSafety2, s);
  CK(cudaGetLastError());
  return 0;
}

int dc_lanes_set_extent(dc_lanes *L, int n_lanes) {
  if (!L) return fail(DC_ERR_ARG, "NULL session");
  if (n_lanes < 0) return fail(DC_ERR_ARG, "negative lane extent");
  const int KB = L->w.KB;
  L->nb_use = (n_lanes <= 0 || n_lanes >= L->w.Kp) ? 0 : (n_lanes + KB - 1) / KB;
  return 0;
}

int dc_lanes_sweep(dc_lanes *L, int *n_active, int *iterations, void *stream) {
  if (!L) return fail(DC_ERR_ARG, "NULL session");
  cudaStream_t s = (cudaStream_t)stream;
  dc_handle *h = L->h;
  int it = 0;
  int rc = lanes_sweep(h, L->w, L->rtol, L->inner_rtol, L->inner_maxit, L->nb_use, &it, s);
  if (rc) return rc == DC_ERR_BREAKDOWN ? fail(rc, "PCG breakdown in a lane session") : rc;
  CK(cudaMemcpyAsync(h->h_mail, L->w.sc.n_active_out, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->ev, s));
  CK(cudaEventSynchronize(h->ev));
  if (n_active) *n_active = h->h_mail[0];
  if (iterations) *iterations = it;
  CK(cudaGetLastError());
  return 0;
}

int dc_lanes_state(dc_lanes *L, int *active, double *rel_res, void *stream) {
  if (!L || (!active && !rel_res)) return fail(DC_ERR_ARG, "bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int K = L->w.Kp;
  std::vector<double> rr(K), bb(K);
  if (active) CK(cudaMemcpyAsync(active, L->w.sc.active_out, sizeof(int) * K, cudaMemcpyDeviceToHost, s));
  if (rel_res) {
    CK(cudaMemcpyAsync(rr.data(), L->w.sc.rr64, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(bb.data(), L->w.sc.bb64, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (rel_res)
    for (int j = 0; j < K; ++j) rel_res[j] = bb[j] > 0.0 ? std::sqrt(rr[j] / bb[j]) : 0.0;
  return 0;
}

int dc_lanes_fetch(dc_lanes *L, const int *lanes_dev, int n, double *x_dev, void *stream) {
  if (!L || !lanes_dev || !x_dev || n < 1 || n > L->w.Kp) return fail(DC_ERR_ARG, "bad argument");
  SolveWS &w = L->w;
  const long long N = L->h->lv[0].dims.N;
  const float *xh = reinterpret_cast<const float *>(w.X64), *xl = xh + (size_t)N * w.Kp;
  lanes_fetch(xh, xl, n, lanes_dev, N, w.KB, x_dev, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

void dc_lanes_close(dc_lanes *L) {
  if (!L) return;
  if (L->own) {
    cudaDeviceSynchronize();
    cudaFree(L->own);
  }
  delete L;
}

int dc_stencil_timing_kinds(dc_handle *h, long long *launches, double *total_ms, double *alg_bytes) {
  if (!h || !launches || !total_ms || !alg_bytes) return fail(DC_ERR_ARG, "NULL argument");
  if (h->prof) return fail(DC_ERR_ARG, "stencil timing is still on: stop it with dc_stencil_timing first");
  for (int c = 0; c < 6; ++c) {
    launches[c] = 0;
    total_ms[c] = 0.0;
    alg_bytes[c] = 0.0;
  }
  for (int i = 0; i + 1 < h->prof_used; i += 2) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, h->prof_ev[i], h->prof_ev[i + 1]));
    const int c = h->prof_kind[i / 2];
    launches[c] += 1;
    total_ms[c] += ms;
    alg_bytes[c] += h->prof_alg[i / 2];
  }
  return 0;
}

int dc_csr_spmv(int nrows, const long long *rowptr, const long long *in_idx, const double *w, const double *x,
                const long long *out_idx, double *y, double scale, int accumulate, void *stream) {
  if (nrows < 0) return fail(DC_ERR_ARG, "nrows < 0");
  if (nrows == 0) return 0;
  if (!rowptr || !in_idx || !w || !x || !y) return fail(DC_ERR_ARG, "NULL argument");
  csr_spmv(nrows, rowptr, in_idx, w, x, out_idx, y, scale, accumulate, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

int dc_fill_sparse(long long nnz, const long long *idx, const double *val, double *y, void *stream) {
  if (nnz < 0) return fail(DC_ERR_ARG, "nnz < 0");
  if (nnz == 0) return 0;
  if (!idx || !val || !y) return fail(DC_ERR_ARG, "NULL argument");
  fill_sparse(nnz, idx, val, y, (cudaStream_t)stream);
  CK(cudaGetLastError());
  return 0;
}

}  // extern "C"
