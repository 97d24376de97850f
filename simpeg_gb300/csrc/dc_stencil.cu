// Scalar, coefficient, coarsest-level, Neumann and layout kernels of the
// nodal DC engine (the node kernels and their launchers are in
// dc_kernels.cuh, instantiated by dc_ops_*.cu), plus the launch bookkeeping.
#include "dc_dfbits.h"
#include "dc_kernels.cuh"

#include <cstdio>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <unordered_map>

namespace dc {

namespace {

__global__ void k_fill_int(int *__restrict__ a, int n, int v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

// ---------------------------------------------------------------- PCG scalars
// Partials layout: [nb][gx][KB]; RHS r = b*KB + l.  One block of SCAL_T
// threads reduces one RHS (threads stride over the gx block partials, fixed
// order, so the sums are deterministic); thread 0 then applies the CG scalar
// logic.  Cost: a few microseconds regardless of K and gx.
constexpr int SCAL_T = 128;

__device__ __forceinline__ double block_sum_partial(const double *p, int gx, int KB, int r) {
  __shared__ double red[SCAL_T / 32];
  const int b = r / KB, l = r % KB;
  const double *q = p + (long long)b * gx * KB + l;
  double s = 0.0;
  for (int i = threadIdx.x; i < gx; i += SCAL_T) s += q[(long long)i * KB];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < SCAL_T / 32; ++w) t += red[w];
  __syncthreads();
  return t;  // valid in thread 0
}

// Per-RHS scale of the multigrid input: 1/|r|_2 (1 for a zero or non-finite
// norm), so that the V-cycle's vectors stay O(1) whatever the residual's size.
// PCG is invariant under a per-iteration positive scaling of the
// preconditioner (alpha and beta absorb it), so this only affects rounding.
__device__ __forceinline__ float rss(double rr) {
  return (rr > 0.0 && isfinite(rr)) ? (float)(1.0 / sqrt(rr)) : 1.0f;
}

__global__ void __launch_bounds__(SCAL_T) k_pcg_alpha(int K, int KB, int gx, const double *__restrict__ part_pq,
                                                      const double *__restrict__ rz, const int *__restrict__ active,
                                                      double *__restrict__ alpha, float *__restrict__ alpha32,
                                                      int *__restrict__ status, int *__restrict__ n_active) {
  const int r = blockIdx.x;
  const double pq = block_sum_partial(part_pq, gx, KB, r);
  if (threadIdx.x == 0) {
    if (r == 0) *n_active = 0;  // recounted by k_pcg_beta later in the iteration
    double a = 0.0;
    if (active[r]) {
      if (!(pq > 0.0) || !isfinite(pq))
        atomicOr(status, 4);  // breakdown / non-finite
      else
        a = rz[r] / pq;
    }
    alpha[r] = a;
    if (alpha32) alpha32[r] = (float)a;
  }
}

// rz_new = r.z ; rr = |r|^2 ; active &= rr > tol2[r]*bb ; beta = rz_new/rz_old ; counts active
// (n_active must be zero on entry).
__global__ void __launch_bounds__(SCAL_T) k_pcg_beta(int K, int KB, int gx, const double *__restrict__ part_rz,
                                                     const double *__restrict__ part_rr, double *__restrict__ rz,
                                                     double *__restrict__ rr_out, const double *__restrict__ bb,
                                                     const double *__restrict__ tol2, int *__restrict__ active,
                                                     double *__restrict__ beta, float *__restrict__ beta32,
                                                     int *__restrict__ n_active, int first, const float *rz_div,
                                                     float *scale) {
  const int r = blockIdx.x;
  double rzn = block_sum_partial(part_rz, gx, KB, r);
  const double rr = block_sum_partial(part_rr, gx, KB, r);
  if (threadIdx.x == 0) {
    if (rz_div) rzn /= (double)rz_div[r];  // read before scale (possibly the same array) is renewed
    rr_out[r] = rr;
    if (scale) scale[r] = rss(rr);
    int act = active[r];
    if (act && !(rr > tol2[r] * bb[r])) act = 0;
    if (act && !isfinite(rr)) act = 0;
    double bt = 0.0;
    if (act && !first) bt = rz[r] != 0.0 ? rzn / rz[r] : 0.0;
    if (act) rz[r] = rzn;
    beta[r] = first ? 0.0 : bt;
    if (beta32) beta32[r] = first ? 0.0f : (float)bt;
    active[r] = act;
    if (act) atomicAdd(n_active, 1);
  }
}

// per-RHS sums of partials into out (used for |b|^2 and the outer residual norms)
__global__ void __launch_bounds__(SCAL_T) k_sum_partials(int K, int KB, int gx, const double *__restrict__ part,
                                                         double *__restrict__ out, float *__restrict__ scale) {
  const double v = block_sum_partial(part, gx, KB, blockIdx.x);
  if (threadIdx.x == 0) {
    out[blockIdx.x] = v;
    if (scale) scale[blockIdx.x] = rss(v);
  }
}

// Outer (refinement) convergence: active = rr > rtol2*bb ; counts ; max relative residual.
// Also the per-RHS tolerance of the next inner solve: the inner solve only has
// to close the remaining gap (with a factor `safety`), but never asks for less
// than a floor of inner_tol2 (what fp32 iterations can deliver).
__global__ void k_outer_check(int K, const double *__restrict__ rr, const double *__restrict__ bb, double rtol2,
                              int *__restrict__ active, int *__restrict__ n_active, double *__restrict__ maxrel,
                              double *__restrict__ inner_tol2, double inner_floor2, double safety2) {
  __shared__ int cnt;
  __shared__ double mx[1024];
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int mine = 0;
  double m = 0.0;
  for (int r = threadIdx.x; r < K; r += blockDim.x) {
    int act = (bb[r] > 0.0) && (rr[r] > rtol2 * bb[r]);
    if (!isfinite(rr[r])) act = 0;
    active[r] = act;
    mine += act;
    if (bb[r] > 0.0) m = fmax(m, sqrt(rr[r] / bb[r]));
    if (inner_tol2) {
      double t = (rr[r] > 0.0) ? safety2 * rtol2 * bb[r] / rr[r] : 1.0;
      inner_tol2[r] = fmin(fmax(t, inner_floor2), 0.25);
    }
  }
  atomicAdd(&cnt, mine);
  mx[threadIdx.x] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int i = 0; i < blockDim.x; ++i) v = fmax(v, mx[i]);
    *n_active = cnt;
    *maxrel = v;
  }
}

// Device-side loop control for solves recorded into a CUDA graph with
// conditional WHILE nodes.  ctr[0] = iterations of the current inner loop,
// ctr[1] = inner iterations summed over sweeps, ctr[2] = refinement sweeps.
// `init` kernels run before a WHILE node (reset the loop's counter, first
// test); `step` kernels end its body (count, test again).  Every loop is
// bounded by its iteration cap.
__global__ void k_inner_loop(cudaGraphConditionalHandle hc, int init, const int *__restrict__ n_active,
                             const int *__restrict__ status, int *__restrict__ ctr, int maxit, int total_max) {
  if (init) {
    ctr[0] = 0;
  } else {
    ctr[0] += 1;
    ctr[1] += 1;
  }
  const unsigned go = (*n_active > 0) && (*status == 0) && (ctr[0] < maxit) && (ctr[1] < total_max);
  cudaGraphSetConditional(hc, go);
}

__global__ void k_outer_loop(cudaGraphConditionalHandle hc, int init, const int *__restrict__ n_active_out,
                             const int *__restrict__ status, int *__restrict__ ctr, int max_outer, int total_max) {
  if (init) {
    ctr[1] = 0;
    ctr[2] = 0;
  } else {
    ctr[2] += 1;
  }
  const unsigned go = (*n_active_out > 0) && (*status == 0) && (ctr[2] < max_outer) && (ctr[1] < total_max);
  cudaGraphSetConditional(hc, go);
}

__global__ void k_fill_double(double *__restrict__ a, int n, double v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

// ---------------------------------------------------------------- coefficients
__device__ __forceinline__ double sig(const double *s, int nx, int ny, int i, int j, int k) {
  return s[i + (long long)nx * (j + (long long)ny * k)];
}

// Coupling of the x-edge (i -> i+1) at node row (j, k): sum over the <= 4 cells
// (i, j', k') of sigma * hy * hz / (4 hx_i).  Same pattern for y, z.
__device__ double cpl_x(const double *s, const double *hx, const double *hy, const double *hz, int nx, int ny,
                        int nz, int i, int j, int k) {
  double acc = 0.0;
  for (int b = k - 1; b <= k; ++b) {
    if (b < 0 || b >= nz) continue;
    for (int a = j - 1; a <= j; ++a) {
      if (a < 0 || a >= ny) continue;
      acc += sig(s, nx, ny, i, a, b) * hy[a] * hz[b];
    }
  }
  return acc / (4.0 * hx[i]);
}
__device__ double cpl_y(const double *s, const double *hx, const double *hy, const double *hz, int nx, int ny,
                        int nz, int i, int j, int k) {
  double acc = 0.0;
  for (int b = k - 1; b <= k; ++b) {
    if (b < 0 || b >= nz) continue;
    for (int a = i - 1; a <= i; ++a) {
      if (a < 0 || a >= nx) continue;
      acc += sig(s, nx, ny, a, j, b) * hx[a] * hz[b];
    }
  }
  return acc / (4.0 * hy[j]);
}
__device__ double cpl_z(const double *s, const double *hx, const double *hy, const double *hz, int nx, int ny,
                        int nz, int i, int j, int k) {
  double acc = 0.0;
  for (int b = j - 1; b <= j; ++b) {
    if (b < 0 || b >= ny) continue;
    for (int a = i - 1; a <= i; ++a) {
      if (a < 0 || a >= nx) continue;
      acc += sig(s, nx, ny, a, b, k) * hx[a] * hy[b];
    }
  }
  return acc / (4.0 * hz[k]);
}

struct BFace {
  const double *v;     // 0.25*alpha*area, sides packed
  long long off[6];    // xlo, xhi, ylo, yhi, zlo, zhi
};

// Robin diagonal of node (i,j,k): sum over boundary faces f touching the node of bface_f * sigma(cell(f)).
__device__ double robin_at(const double *s, BFace bf, int nx, int ny, int nz, int i, int j, int k) {
  double acc = 0.0;
  if (i == 0 || i == nx) {
    const double *v = bf.v + bf.off[i == 0 ? 0 : 1];
    const int ci = (i == 0) ? 0 : nx - 1;
    for (int b = k - 1; b <= k; ++b) {
      if (b < 0 || b >= nz) continue;
      for (int a = j - 1; a <= j; ++a) {
        if (a < 0 || a >= ny) continue;
        acc += v[a + (long long)ny * b] * sig(s, nx, ny, ci, a, b);
      }
    }
  }
  if (j == 0 || j == ny) {
    const double *v = bf.v + bf.off[j == 0 ? 2 : 3];
    const int cj = (j == 0) ? 0 : ny - 1;
    for (int b = k - 1; b <= k; ++b) {
      if (b < 0 || b >= nz) continue;
      for (int a = i - 1; a <= i; ++a) {
        if (a < 0 || a >= nx) continue;
        acc += v[a + (long long)nx * b] * sig(s, nx, ny, a, cj, b);
      }
    }
  }
  if (k == 0 || k == nz) {
    const double *v = bf.v + bf.off[k == 0 ? 4 : 5];
    const int ck = (k == 0) ? 0 : nz - 1;
    for (int b = j - 1; b <= j; ++b) {
      if (b < 0 || b >= ny) continue;
      for (int a = i - 1; a <= i; ++a) {
        if (a < 0 || a >= nx) continue;
        acc += v[a + (long long)nx * b] * sig(s, nx, ny, a, b, ck);
      }
    }
  }
  return acc;
}

__global__ void k_coef_build(const double *__restrict__ s, const double *__restrict__ h, int nx, int ny, int nz,
                             BFace bf, int robin, Coef64 *__restrict__ c64, Coef32 *__restrict__ c32,
                             double *__restrict__ invd64, float *__restrict__ invd32,
                             unsigned long long *__restrict__ lmax_bits) {
  const double *hx = h, *hy = h + nx, *hz = h + nx + ny;
  const int Nx = nx + 1, Ny = ny + 1, Nz = nz + 1;
  const long long N = (long long)Nx * Ny * Nz;
  double gmax = 0.0;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(n / ((long long)Nx * Ny));
    const int r = (int)(n - (long long)k * Nx * Ny);
    const int j = r / Nx, i = r - j * Nx;
    const double cxp = (i < nx) ? cpl_x(s, hx, hy, hz, nx, ny, nz, i, j, k) : 0.0;
    const double cxm = (i > 0) ? cpl_x(s, hx, hy, hz, nx, ny, nz, i - 1, j, k) : 0.0;
    const double cyp = (j < ny) ? cpl_y(s, hx, hy, hz, nx, ny, nz, i, j, k) : 0.0;
    const double cym = (j > 0) ? cpl_y(s, hx, hy, hz, nx, ny, nz, i, j - 1, k) : 0.0;
    const double czp = (k < nz) ? cpl_z(s, hx, hy, hz, nx, ny, nz, i, j, k) : 0.0;
    const double czm = (k > 0) ? cpl_z(s, hx, hy, hz, nx, ny, nz, i, j, k - 1) : 0.0;
    const double off = cxp + cxm + cyp + cym + czp + czm;
    const double rb = robin ? robin_at(s, bf, nx, ny, nz, i, j, k) : 0.0;
    const double dg = off + rb;
    Coef64 c;
    c.cx = cxp; c.cy = cyp; c.cz = czp; c.d = dg;
    c64[n] = c;
    Coef32 f;
    f.cx = (float)cxp; f.cy = (float)cyp; f.cz = (float)czp; f.d = (float)dg;
    c32[n] = f;
    const double id = dg > 0.0 ? 1.0 / dg : 0.0;
    invd64[n] = id;
    invd32[n] = (float)id;
    if (dg > 0.0) gmax = fmax(gmax, 1.0 + off / dg);
  }
  // positive doubles order like their bit patterns
  for (int o = 16; o > 0; o >>= 1) gmax = fmax(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(lmax_bits, (unsigned long long)__double_as_longlong(gmax));
}

// sigma_c = sum(sigma_f V_f) / sum(V_f) over the fine cells of each coarse cell.
__global__ void k_coarsen_sigma(const double *__restrict__ sf, const double *__restrict__ hf, int fnx, int fny, int fnz,
                                double *__restrict__ sc, int cnx, int cny, int cnz, const int *__restrict__ fi,
                                long long o0, long long o1, long long o2) {
  const double *hx = hf, *hy = hf + fnx, *hz = hf + fnx + fny;
  const long long nC = (long long)cnx * cny * cnz;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += (long long)gridDim.x * blockDim.x) {
    const int K = (int)(c / ((long long)cnx * cny));
    const int r = (int)(c - (long long)K * cnx * cny);
    const int J = r / cnx, I = r - J * cnx;
    double sv = 0.0, vv = 0.0;
    for (int k = fi[o2 + K]; k < fi[o2 + K + 1]; ++k)
      for (int j = fi[o1 + J]; j < fi[o1 + J + 1]; ++j)
        for (int i = fi[o0 + I]; i < fi[o0 + I + 1]; ++i) {
          const double v = hx[i] * hy[j] * hz[k];
          sv += sf[i + (long long)fnx * (j + (long long)fny * k)] * v;
          vv += v;
        }
    sc[c] = sv / vv;
  }
}

// ---------------------------------------------------------------- operator-based coarse levels
// A coarse level's seven-point operator formed from the finer level's
// couplings instead of rediscretised from an averaged conductivity (mode 1: the
// Galerkin product P^T A P with the engine's linear prolongation, collapsed
// onto the seven-point pattern; mode 2: the fine couplings along a coarse edge
// combined in series).  The energy of every fine edge goes to the coarse edge
// of its direction: along the edge with the squared prolongation weights of
// the fine nodes it joins (mode 1) or as resistors in series (mode 2), across
// it with the transverse nodes' linear prolongation weights (the cross terms
// P^T A P would put on diagonal neighbours are summed onto the axis ones).
// The diagonal excess of the fine rows (the Robin term) is lumped with the
// linear weights.  On a uniform mesh with a constant conductivity mode 1
// reproduces the rediscretised interior couplings.
struct AxisTab {
  const int *fi;      // coarse node -> fine node, per axis at fo[a]
  const int *pl;      // fine node -> left coarse node, per axis at po[a]
  const double *pw;   // weight of the left coarse node, per axis at po[a]
  long long fo[3], po[3];
};

__device__ __forceinline__ double pwgt(const AxisTab &t, int a, int f, int J) {
  const int L = t.pl[t.po[a] + f];
  const double w = t.pw[t.po[a] + f];
  return L == J ? w : (L + 1 == J ? 1.0 - w : 0.0);
}

// fine coupling along axis a at fine node (f0, f1, f2) (to its + neighbour)
__device__ __forceinline__ double fcpl(const Coef64 *c, const Dims &d, int a, int i, int j, int k) {
  const Coef64 v = c[i + (long long)d.Nx * (j + (long long)d.Ny * k)];
  return a == 0 ? v.cx : (a == 1 ? v.cy : v.cz);
}

// coarse coupling along axis a from coarse node (I0, I1, I2) to its + neighbour
__device__ double ccpl(const Coef64 *fc, const Dims &fd, const Dims &cd, const AxisTab &t, int mode, int a, int I0,
                       int I1, int I2) {
  const int I[3] = {I0, I1, I2};
  const int fN[3] = {fd.Nx, fd.Ny, fd.Nz};
  const int f[3] = {t.fi[t.fo[0] + I0], t.fi[t.fo[1] + I1], t.fi[t.fo[2] + I2]};
  const int fnext = t.fi[t.fo[a] + I[a] + 1];
  const int b = (a + 1) % 3, c = (a + 2) % 3;  // transverse axes
  double sum = 0.0;
  for (int db = -1; db <= 1; ++db) {
    const int fb = f[b] + db;
    if (fb < 0 || fb >= fN[b]) continue;
    const double wb = pwgt(t, b, fb, I[b]);
    if (wb == 0.0) continue;
    for (int dc = -1; dc <= 1; ++dc) {
      const int fc2 = f[c] + dc;
      if (fc2 < 0 || fc2 >= fN[c]) continue;
      const double wc = pwgt(t, c, fc2, I[c]);
      if (wc == 0.0) continue;
      int p[3];
      p[a] = f[a];
      p[b] = fb;
      p[c] = fc2;
      const double T1 = fcpl(fc, fd, a, p[0], p[1], p[2]);
      double tv = T1;
      if (fnext == f[a] + 2) {
        p[a] = f[a] + 1;
        const double T2 = fcpl(fc, fd, a, p[0], p[1], p[2]);
        if (mode == 1) {
          const double w = t.pw[t.po[a] + f[a] + 1];  // weight of the middle fine node on coarse node I[a]
          tv = T1 * (1.0 - w) * (1.0 - w) + T2 * w * w;
        } else {
          tv = (T1 > 0.0 && T2 > 0.0) ? T1 * T2 / (T1 + T2) : 0.0;
        }
      }
      sum += wb * wc * tv;
    }
  }
  (void)cd;
  return sum;
}

// The couplings along the + edges of every coarse node (the coupling of an
// edge is stored once, at its lower node).
__global__ void k_coef_galerkin_edges(const Coef64 *__restrict__ fc, Dims fd, Dims cd, AxisTab t, int mode,
                                      Coef64 *__restrict__ c64) {
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < cd.N; n += (long long)gridDim.x * blockDim.x) {
    const int K = (int)(n / ((long long)cd.Nx * cd.Ny));
    const int r = (int)(n - (long long)K * cd.Nx * cd.Ny);
    const int J = r / cd.Nx, I = r - J * cd.Nx;
    Coef64 c;
    c.cx = I + 1 < cd.Nx ? ccpl(fc, fd, cd, t, mode, 0, I, J, K) : 0.0;
    c.cy = J + 1 < cd.Ny ? ccpl(fc, fd, cd, t, mode, 1, I, J, K) : 0.0;
    c.cz = K + 1 < cd.Nz ? ccpl(fc, fd, cd, t, mode, 2, I, J, K) : 0.0;
    c.d = 0.0;
    c64[n] = c;
  }
}

// The diagonal of every coarse node from the couplings of k_coef_galerkin_edges
// (its - couplings read at the neighbours: each edge's series sum is formed
// once, where forming all six per node took 0.89 ms for the six coarse levels
// of the 1M-cell mesh) and the lumped diagonal excess of the fine rows around
// it; the fp32 copies, inverse diagonals and Gershgorin bound.
__global__ void k_coef_galerkin(const Coef64 *__restrict__ fc, Dims fd, Dims cd, AxisTab t,
                                Coef64 *__restrict__ c64, Coef32 *__restrict__ c32, double *__restrict__ invd64,
                                float *__restrict__ invd32, unsigned long long *__restrict__ lmax_bits) {
  double gmax = 0.0;
  const long long sy = cd.Nx, sz = (long long)cd.Nx * cd.Ny;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < cd.N; n += (long long)gridDim.x * blockDim.x) {
    const int K = (int)(n / ((long long)cd.Nx * cd.Ny));
    const int r = (int)(n - (long long)K * cd.Nx * cd.Ny);
    const int J = r / cd.Nx, I = r - J * cd.Nx;
    const Coef64 cn = c64[n];
    const double cxp = cn.cx, cyp = cn.cy, czp = cn.cz;
    const double cxm = I > 0 ? c64[n - 1].cx : 0.0;
    const double cym = J > 0 ? c64[n - sy].cy : 0.0;
    const double czm = K > 0 ? c64[n - sz].cz : 0.0;
    // lumped diagonal excess of the fine rows around the coarse node
    const int fx = t.fi[t.fo[0] + I], fy = t.fi[t.fo[1] + J], fz = t.fi[t.fo[2] + K];
    double ex = 0.0;
    for (int dk = -1; dk <= 1; ++dk) {
      const int k = fz + dk;
      if (k < 0 || k >= fd.Nz) continue;
      const double wz = pwgt(t, 2, k, K);
      if (wz == 0.0) continue;
      for (int dj = -1; dj <= 1; ++dj) {
        const int j = fy + dj;
        if (j < 0 || j >= fd.Ny) continue;
        const double wy = pwgt(t, 1, j, J);
        if (wy == 0.0) continue;
        for (int di = -1; di <= 1; ++di) {
          const int i = fx + di;
          if (i < 0 || i >= fd.Nx) continue;
          const double wx = pwgt(t, 0, i, I);
          if (wx == 0.0) continue;
          const long long m = i + (long long)fd.Nx * (j + (long long)fd.Ny * k);
          const Coef64 v = fc[m];
          double off = v.cx + v.cy + v.cz;
          if (i > 0) off += fc[m - 1].cx;
          if (j > 0) off += fc[m - fd.Nx].cy;
          if (k > 0) off += fc[m - (long long)fd.Nx * fd.Ny].cz;
          // the last node of an axis stores no + coupling of that axis
          if (i + 1 >= fd.Nx) off -= v.cx;
          if (j + 1 >= fd.Ny) off -= v.cy;
          if (k + 1 >= fd.Nz) off -= v.cz;
          ex += wx * wy * wz * fmax(v.d - off, 0.0);
        }
      }
    }
    const double off = cxp + cxm + cyp + cym + czp + czm;
    const double dg = off + ex;
    c64[n].d = dg;  // the couplings stay as the edge pass wrote them (neighbours read them)
    Coef32 f;
    f.cx = (float)cxp; f.cy = (float)cyp; f.cz = (float)czp; f.d = (float)dg;
    c32[n] = f;
    const double id = dg > 0.0 ? 1.0 / dg : 0.0;
    invd64[n] = id;
    invd32[n] = (float)id;
    if (dg > 0.0) gmax = fmax(gmax, 1.0 + off / dg);
  }
  for (int o = 16; o > 0; o >>= 1) gmax = fmax(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(lmax_bits, (unsigned long long)__double_as_longlong(gmax));
}

// ---------------------------------------------------------------- coarsest level
__global__ void k_dense_assemble(const Coef64 *__restrict__ coef, Dims d, double *__restrict__ A) {
  const int N = (int)d.N;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    double *row = A + (long long)n * N;
    const Coef64 c = coef[n];
    row[n] = c.d;
    if (i + 1 < d.Nx) row[n + 1] = -c.cx;
    if (i > 0) row[n - 1] = -coef[n - 1].cx;
    if (j + 1 < d.Ny) row[n + d.Nx] = -c.cy;
    if (j > 0) row[n - d.Nx] = -coef[n - d.Nx].cy;
    if (k + 1 < d.Nz) row[n + d.Nx * d.Ny] = -c.cz;
    if (k > 0) row[n - d.Nx * d.Ny] = -coef[n - d.Nx * d.Ny].cz;
  }
}

// In-place right-looking Cholesky (lower) of a dense SPD matrix, one CTA:
// warps own rows of the trailing update, lanes own columns.
__global__ void __launch_bounds__(1024) k_cholesky(double *__restrict__ A, int n, int *__restrict__ flag) {
  __shared__ double piv;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      double a = A[(long long)k * n + k];
      if (!(a > 0.0)) {
        atomicOr(flag, 1);
        a = 1.0;
      }
      piv = sqrt(a);
      A[(long long)k * n + k] = piv;
    }
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[(long long)i * n + k] /= piv;
    __syncthreads();
    for (int i = k + 1 + warp; i < n; i += nw) {
      const double lik = A[(long long)i * n + k];
      for (int j = k + 1 + lane; j <= i; j += 32) A[(long long)i * n + j] -= lik * A[(long long)j * n + k];
    }
    __syncthreads();
  }
}

// Column j of A^-1 = L^-T L^-1 e_j, one warp per column (lanes split the dot
// products); writes row-major (the inverse is symmetric).
__global__ void k_chol_inverse(const double *__restrict__ L, int n, double *__restrict__ work,
                               double *__restrict__ Ainv64, float *__restrict__ Ainv32) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  double *y = work + (long long)j * n;
  for (int i = lane; i < n; i += 32) y[i] = 0.0;
  __syncwarp();
  // forward: L y = e_j  (y_i = 0 for i < j)
  for (int i = j; i < n; ++i) {
    double s = 0.0;
    for (int m = j + lane; m < i; m += 32) s += L[(long long)i * n + m] * y[m];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[i] = ((i == j ? 1.0 : 0.0) - s) / L[(long long)i * n + i];
    __syncwarp();
  }
  // back: L^T x = y
  for (int i = n - 1; i >= 0; --i) {
    double s = 0.0;
    for (int m = i + 1 + lane; m < n; m += 32) s += L[(long long)m * n + i] * y[m];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[i] = (y[i] - s) / L[(long long)i * n + i];
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) {
    Ainv64[(long long)i * n + j] = y[i];
    Ainv32[(long long)i * n + j] = (float)y[i];
  }
}

// ---------------------------------------------------------------- Neumann pinning
__global__ void k_dense_pin0(double *__restrict__ A, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    A[i] = (i == 0) ? 1.0 : 0.0;             // row 0
    if (i) A[(long long)i * n] = 0.0;        // column 0
  }
}

// sums[r] = sum_n b[r*N + n] (column-major input), one block per column, fixed order.
__global__ void k_colsum(const double *__restrict__ b, long long N, double *__restrict__ sums) {
  __shared__ double red[TPB / 32];
  const double *c = b + (long long)blockIdx.x * N;
  double acc = 0.0;
  for (long long n = threadIdx.x; n < N; n += TPB) acc += c[n];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0;
    for (int w = 0; w < TPB / 32; ++w) sacc += red[w];
    sums[blockIdx.x] = sacc;
  }
}

// Row 0 of every packed RHS r: b_0 - sum(b) (= -sum of the other rows).
__global__ void k_neumann_row0(const double *__restrict__ b, long long N, int K, int KB, double *__restrict__ B,
                               const double *__restrict__ sums) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < K; r += gridDim.x * blockDim.x)
    B[(long long)(r / KB) * N * KB + (r % KB)] = b[(long long)r * N] - sums[r];
}

// x[:, r] += b[0, r] - x[0, r]  (column-major), one block per column.
__global__ void k_neumann_shift(const double *__restrict__ b, long long N, double *__restrict__ x) {
  __shared__ double delta;
  double *c = x + (long long)blockIdx.x * N;
  if (threadIdx.x == 0) delta = b[(long long)blockIdx.x * N] - c[0];
  __syncthreads();
  for (long long n = threadIdx.x; n < N; n += TPB) c[n] += delta;
}

// ---------------------------------------------------------------- layout conversion
// Column-major (K, N) <-> RHS-blocked [nb][N][KB] transposes through a
// 32 x 32 shared-memory tile (rows = RHS, columns = nodes), so that both the
// column-major side (contiguous in n) and the blocked side (contiguous in the
// RHS lane) are accessed in full lines.  Lanes r >= K of the blocked array are
// zero-filled by k_pack.
constexpr int TT = 32;  // tile edge
constexpr int TR = 8;   // tile rows per pass (blockDim = TT x TR)

template <typename T>
__global__ void __launch_bounds__(TT *TR) k_pack(const double *__restrict__ src, long long N, int K, int KB, int Kp,
                                                  T *__restrict__ dst) {
  __shared__ T tile[TT][TT + 1];
  const long long n0 = (long long)blockIdx.x * TT;
  const int r0 = blockIdx.y * TT;
  for (int i = threadIdx.y; i < TT; i += TR) {
    const int r = r0 + i;
    const long long n = n0 + threadIdx.x;
    tile[i][threadIdx.x] = (r < K && n < N) ? (T)src[(long long)r * N + n] : (T)0;
  }
  __syncthreads();
  const int r = r0 + threadIdx.x;
  if (r >= Kp) return;
  const int b = r / KB, l = r % KB;
  for (int j = threadIdx.y; j < TT; j += TR) {
    const long long n = n0 + j;
    if (n < N) dst[((long long)b * N + n) * KB + l] = tile[threadIdx.x][j];
  }
}

// (double)v split into fp32 (hi, lo) with the fp64 instructions, in a call of its
// own (kept out of the common path of k_pack_split_df).
__device__ __noinline__ void split_fp64_call(double v, float &h, float &l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

// k_pack and the double-float split in one pass: column-major fp64 (K, N) ->
// RHS-blocked fp32 (hi, lo) pairs (split_df_bits, the fp64 instructions only
// for values outside its range) and r32 = hi, lanes r >= K zero.
__global__ void __launch_bounds__(TT *TR) k_pack_split_df(const double *__restrict__ src, long long N, int K, int KB,
                                                         int Kp, float *__restrict__ hi, float *__restrict__ lo,
                                                         float *__restrict__ r32) {
  __shared__ double tile[TT][TT + 1];
  const long long n0 = (long long)blockIdx.x * TT;
  const int r0 = blockIdx.y * TT;
  for (int i = threadIdx.y; i < TT; i += TR) {
    const int r = r0 + i;
    const long long n = n0 + threadIdx.x;
    tile[i][threadIdx.x] = (r < K && n < N) ? src[(long long)r * N + n] : 0.0;
  }
  __syncthreads();
  const int r = r0 + threadIdx.x;
  if (r >= Kp) return;
  const int b = r / KB, l = r % KB;
  for (int j = threadIdx.y; j < TT; j += TR) {
    const long long n = n0 + j;
    if (n < N) {
      float h, w;
      if (__builtin_expect(!split_df_bits(tile[threadIdx.x][j], h, w), 0)) split_fp64_call(tile[threadIdx.x][j], h, w);
      const long long e = ((long long)b * N + n) * KB + l;
      hi[e] = h;
      lo[e] = w;
      if (r32) r32[e] = h;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(TT *TR) k_unpack(const T *__restrict__ src, long long N, int K, int KB,
                                                    double *__restrict__ dst) {
  __shared__ double tile[TT][TT + 1];
  const long long n0 = (long long)blockIdx.x * TT;
  const int r0 = blockIdx.y * TT;
  {
    const int r = r0 + threadIdx.x;
    const int b = r / KB, l = r % KB;
    for (int j = threadIdx.y; j < TT; j += TR) {
      const long long n = n0 + j;
      if (r < K && n < N) tile[threadIdx.x][j] = (double)src[((long long)b * N + n) * KB + l];
    }
  }
  __syncthreads();
  for (int i = threadIdx.y; i < TT; i += TR) {
    const int r = r0 + i;
    const long long n = n0 + threadIdx.x;
    if (r < K && n < N) dst[(long long)r * N + n] = tile[i][threadIdx.x];
  }
}

// (double)h + (double)l with the fp64 instructions, in a call of its own (kept
// out of the common path of k_unpack_df).
__device__ __noinline__ double df_sum_fp64(float h, float l) { return (double)h + (double)l; }

// The same transpose for a double-float (hi, lo) blocked array: dst = hi + lo in
// fp64, rounded as the fp64 addition rounds it, by integer operations for
// normalised pairs (df_sum_bits) and the fp64 instructions otherwise.  With one
// fp64 add per element the transpose ran at GB300's fp64 rate (1.34 ms at 1M
// nodes x 256 RHS; 1.21 ms by bits.  Tiles of 32 x 128 instead of 32 x 32
// measured slower, 1.45 ms).
__global__ void __launch_bounds__(TT *TR) k_unpack_df(const float *__restrict__ hi, const float *__restrict__ lo,
                                                     long long N, int K, int KB, double *__restrict__ dst) {
  __shared__ double tile[TT][TT + 1];
  const long long n0 = (long long)blockIdx.x * TT;
  const int r0 = blockIdx.y * TT;
  {
    const int r = r0 + threadIdx.x;
    const int b = r / KB, l = r % KB;
    for (int j = threadIdx.y; j < TT; j += TR) {
      const long long n = n0 + j;
      if (r < K && n < N) {
        const long long e = ((long long)b * N + n) * KB + l;
        const float fh = hi[e], fl = lo[e];
        double v;
        if (__builtin_expect(!df_sum_bits(fh, fl, v), 0)) v = df_sum_fp64(fh, fl);
        tile[threadIdx.x][j] = v;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.y; i < TT; i += TR) {
    const int r = r0 + i;
    const long long n = n0 + threadIdx.x;
    if (r < K && n < N) dst[(long long)r * N + n] = tile[i][threadIdx.x];
  }
}

}  // namespace

// Resident blocks per SM of a kernel (cached).  Grids are capped at what the
// GPU holds at once: a grid-stride sweep whose blocks do not all fit would be
// run as two sweeps, and the second re-reads from DRAM what the first one had
// in L2 (the stencil's neighbour planes).
int resident_blocks(const void *func) {
  static std::mutex mu;
  static std::unordered_map<const void *, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(func);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, func, TPB, 0) != cudaSuccess || n < 1) n = 1;
  cache[func] = n;
  return n;
}


int g_n_sm = 152;
std::atomic<long long> &launch_counter() {
  static std::atomic<long long> c{0};
  return c;
}
void set_sm_count(int n) { g_n_sm = n > 0 ? n : 152; }

int node_grid(long long nodes, int KB, int nb, int per_sm) {
  const int W = KB >= 4 ? 4 : KB;
  return grid_nodes(nodes, KB / W, nb, g_n_sm, per_sm);
}

void fill_int(int *a, int n, int v, cudaStream_t s) {
  if (n > 0) k_fill_int<<<count_launch((n + TPB - 1) / TPB), TPB, 0, s>>>(a, n, v);
}

void pcg_alpha(int K, int KB, int gx, const double *part_pq, const double *rz, const int *active, double *alpha,
               float *alpha32, int *status, int *n_active, cudaStream_t s) {
  k_pcg_alpha<<<count_launch(dim3(K)), SCAL_T, 0, s>>>(K, KB, gx, part_pq, rz, active, alpha, alpha32, status,
                                                       n_active);
}

void pcg_beta(int K, int KB, int gx, const double *part_rz, const double *part_rr, double *rz, double *rr,
              const double *bb, const double *tol2, int *active, double *beta, float *beta32, int *n_active,
              int first, cudaStream_t s, const float *rz_div, float *scale_out) {
  k_pcg_beta<<<count_launch(dim3(K)), SCAL_T, 0, s>>>(K, KB, gx, part_rz, part_rr, rz, rr, bb, tol2, active, beta,
                                                      beta32, n_active, first, rz_div, scale_out);
}

void sum_partials(int K, int KB, int gx, const double *part, double *out, cudaStream_t s, float *scale) {
  k_sum_partials<<<count_launch(dim3(K)), SCAL_T, 0, s>>>(K, KB, gx, part, out, scale);
}

void outer_check(int K, const double *rr, const double *bb, double rtol2, int *active, int *n_active,
                 double *maxrel, double *inner_tol2, double inner_floor2, double safety2, cudaStream_t s) {
  k_outer_check<<<count_launch(1), 1024, 0, s>>>(K, rr, bb, rtol2, active, n_active, maxrel, inner_tol2, inner_floor2, safety2);
}

void inner_loop_cond(cudaGraphConditionalHandle hc, int init, const int *n_active, const int *status, int *ctr,
                     int maxit, int total_max, cudaStream_t s) {
  k_inner_loop<<<count_launch(1), 1, 0, s>>>(hc, init, n_active, status, ctr, maxit, total_max);
}

void outer_loop_cond(cudaGraphConditionalHandle hc, int init, const int *n_active_out, const int *status, int *ctr,
                     int max_outer, int total_max, cudaStream_t s) {
  k_outer_loop<<<count_launch(1), 1, 0, s>>>(hc, init, n_active_out, status, ctr, max_outer, total_max);
}

void fill_double(double *a, int n, double v, cudaStream_t s) {
  if (n > 0) k_fill_double<<<count_launch((n + TPB - 1) / TPB), TPB, 0, s>>>(a, n, v);
}

void coef_build(const Level &L, int robin, unsigned long long *d_lmax_bits, cudaStream_t s) {
  BFace bf;
  bf.v = L.d_bface;
  for (int a = 0; a < 6; ++a) bf.off[a] = L.bface_off[a];
  k_coef_build<<<count_launch(grid_flat(L.dims.N, g_n_sm)), TPB, 0, s>>>(L.d_sigma, L.d_h, L.nx, L.ny, L.nz, bf, robin,
                                                            L.d_coef64, L.d_coef32, L.d_invd64, L.d_invd32,
                                                            d_lmax_bits);
}

// Rows of A D^-1: the couplings of row n scaled by the inverse diagonal of
// the neighbour they multiply, so that A (c0 D^-1 r) needs r and one 32-byte
// row per node (the folded first Chebyshev step).
__global__ void k_rows_dinv(const Coef32 *__restrict__ c, const float *__restrict__ invd, Dims d,
                            RowDinv32 *__restrict__ rows) {
  const long long sy = d.Nx, sz = (long long)d.Nx * d.Ny;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < d.N; n += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    node_ijk((int)n, d, i, j, k);
    const Coef32 cn = c[n];
    RowDinv32 w;
    w.d = cn.d * invd[n];
    w.xp = i + 1 < d.Nx ? cn.cx * invd[n + 1] : 0.f;
    w.xm = i > 0 ? c[n - 1].cx * invd[n - 1] : 0.f;
    w.yp = j + 1 < d.Ny ? cn.cy * invd[n + sy] : 0.f;
    w.ym = j > 0 ? c[n - sy].cy * invd[n - sy] : 0.f;
    w.zp = k + 1 < d.Nz ? cn.cz * invd[n + sz] : 0.f;
    w.zm = k > 0 ? c[n - sz].cz * invd[n - sz] : 0.f;
    w.pad = 0.f;
    rows[n] = w;
  }
}

void rows_dinv(const Level &L, cudaStream_t s) {
  k_rows_dinv<<<count_launch(grid_flat(L.dims.N, g_n_sm)), TPB, 0, s>>>(L.d_coef32, L.d_invd32, L.dims, L.d_rows32);
}

void coef_galerkin(const Level &f, const Level &c, int mode, unsigned long long *d_lmax_bits, cudaStream_t s) {
  AxisTab t;
  t.fi = f.d_r_fi;
  t.pl = f.d_pl_idx;
  t.pw = f.d_pl_w;
  for (int a = 0; a < 3; ++a) {
    t.fo[a] = f.r_off[a];
    t.po[a] = f.pl_off[a];
  }
  const unsigned g = count_launch(grid_flat(c.dims.N, g_n_sm)).x;
  k_coef_galerkin_edges<<<g, TPB, 0, s>>>(f.d_coef64, f.dims, c.dims, t, mode, c.d_coef64);
  k_coef_galerkin<<<count_launch(dim3(g)), TPB, 0, s>>>(f.d_coef64, f.dims, c.dims, t, c.d_coef64, c.d_coef32,
                                                        c.d_invd64, c.d_invd32, d_lmax_bits);
}

void coarsen_sigma(const Level &f, const Level &c, cudaStream_t s) {
  const long long nC = (long long)c.nx * c.ny * c.nz;
  k_coarsen_sigma<<<count_launch(grid_flat(nC, g_n_sm)), TPB, 0, s>>>(f.d_sigma, f.d_h, f.nx, f.ny, f.nz, c.d_sigma, c.nx, c.ny,
                                                         c.nz, f.d_r_fi, f.r_off[0], f.r_off[1], f.r_off[2]);
}

void dense_assemble(const Level &L, double *dense, cudaStream_t s) {
  cudaMemsetAsync(dense, 0, sizeof(double) * L.dims.N * L.dims.N, s);
  k_dense_assemble<<<count_launch(grid_flat(L.dims.N, g_n_sm)), TPB, 0, s>>>(L.d_coef64, L.dims, dense);
}

void dense_cholesky_inverse(double *dense, double *work, int n, double *Ainv64, float *Ainv32, int *flag,
                            cudaStream_t s) {
  k_cholesky<<<count_launch(1), 1024, 0, s>>>(dense, n, flag);
  k_chol_inverse<<<count_launch((n * 32 + 255) / 256), 256, 0, s>>>(dense, n, work, Ainv64, Ainv32);
}

void dense_pin0(double *A, int n, cudaStream_t s) {
  k_dense_pin0<<<count_launch(dim3((n + TPB - 1) / TPB)), TPB, 0, s>>>(A, n);
}

void neumann_rhs(const double *b, long long N, int K, int KB, double *B, double *sums, cudaStream_t s) {
  k_colsum<<<count_launch(dim3(K)), TPB, 0, s>>>(b, N, sums);
  k_neumann_row0<<<count_launch(dim3((K + TPB - 1) / TPB)), TPB, 0, s>>>(b, N, K, KB, B, sums);
}

void neumann_shift(const double *b, long long N, int K, double *x, cudaStream_t s) {
  k_neumann_shift<<<count_launch(dim3(K)), TPB, 0, s>>>(b, N, x);
}


template <typename T>
void pack_colmajor(const double *src, long long N, int K, int KB, int nb, T *dst, cudaStream_t s) {
  const int Kp = KB * nb;
  const dim3 grid((unsigned)((N + TT - 1) / TT), (unsigned)((Kp + TT - 1) / TT));
  k_pack<T><<<count_launch(grid), dim3(TT, TR), 0, s>>>(src, N, K, KB, Kp, dst);
}

void pack_split_df(const double *src, long long N, int K, int KB, int nb, float *hi, float *lo, float *r32,
                   cudaStream_t s) {
  const int Kp = KB * nb;
  const dim3 grid((unsigned)((N + TT - 1) / TT), (unsigned)((Kp + TT - 1) / TT));
  k_pack_split_df<<<count_launch(grid), dim3(TT, TR), 0, s>>>(src, N, K, KB, Kp, hi, lo, r32);
}

void unpack_colmajor_df(const float *hi, const float *lo, long long N, int K, int KB, double *dst, cudaStream_t s) {
  const dim3 grid((unsigned)((N + TT - 1) / TT), (unsigned)((K + TT - 1) / TT));
  k_unpack_df<<<count_launch(grid), dim3(TT, TR), 0, s>>>(hi, lo, N, K, KB, dst);
}

template <typename T>
void unpack_colmajor(const T *src, long long N, int K, int KB, double *dst, cudaStream_t s) {
  const dim3 grid((unsigned)((N + TT - 1) / TT), (unsigned)((K + TT - 1) / TT));
  k_unpack<T><<<count_launch(grid), dim3(TT, TR), 0, s>>>(src, N, K, KB, dst);
}

template void pack_colmajor<float>(const double *, long long, int, int, int, float *, cudaStream_t);
template void pack_colmajor<double>(const double *, long long, int, int, int, double *, cudaStream_t);
template void unpack_colmajor<float>(const float *, long long, int, int, double *, cudaStream_t);
template void unpack_colmajor<double>(const double *, long long, int, int, double *, cudaStream_t);

}  // namespace dc
