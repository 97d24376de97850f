// Electrode scatter/gather and model-derivative kernels of the nodal DC engine.
//
// All arrays here are column-major (N x K) fp64, i.e. RHS r occupies
// [r*N, (r+1)*N): the layout of simpeg's Fields "phiSolution" store.
#include "dc_internal.h"

namespace dc {

namespace {
constexpr int TPB = 256;

inline int grid_flat(long long total, int n_sm) {
  long long g = (total + TPB - 1) / TPB;
  long long cap = (long long)n_sm * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// y[out_idx[row]] (=|+=) scale * sum_e w[e] * x[in_idx[e]], e in [rowptr[row], rowptr[row+1])
__global__ void k_csr_spmv(int nrows, const long long *__restrict__ rowptr, const long long *__restrict__ in_idx,
                           const double *__restrict__ w, const double *__restrict__ x,
                           const long long *__restrict__ out_idx, double *__restrict__ y, double scale, int accumulate) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (long long e = rowptr[r]; e < rowptr[r + 1]; ++e) acc += w[e] * x[in_idx[e]];
    const long long o = out_idx ? out_idx[r] : (long long)r;
    if (accumulate)
      y[o] += scale * acc;
    else
      y[o] = scale * acc;
  }
}

__global__ void k_fill_sparse(long long nnz, const long long *__restrict__ idx, const double *__restrict__ val,
                              double *__restrict__ y) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (long long)gridDim.x * blockDim.x)
    y[idx[e]] = val[e];
}

__global__ void k_scale(long long n, double *__restrict__ y, double a) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    y[e] *= a;
}

// Edge products for the adjoint model derivative, summed over RHS:
//   P[a][n] = sum_s (u_s[n+da] - u_s[n]) * (l_s[n+da] - l_s[n])   (a = x, y, z edge leaving node n)
//   Q[n]    = sum_s u_s[n] * l_s[n]                               (boundary nodes only)
__global__ void k_edge_products(const double *__restrict__ u, const double *__restrict__ l, int K, Dims d,
                                double *__restrict__ P, double *__restrict__ Q) {
  const long long N = d.N;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(n / ((long long)d.Nx * d.Ny));
    const int rr = (int)(n - (long long)k * d.Nx * d.Ny);
    const int j = rr / d.Nx, i = rr - j * d.Nx;
    const bool ex = i + 1 < d.Nx, ey = j + 1 < d.Ny, ez = k + 1 < d.Nz;
    const bool bnd = (i == 0) || (j == 0) || (k == 0) || !ex || !ey || !ez;
    const long long sy = d.Nx, sz = (long long)d.Nx * d.Ny;
    double px = 0.0, py = 0.0, pz = 0.0, q = 0.0;
    for (int s = 0; s < K; ++s) {
      const double *us = u + (long long)s * N, *ls = l + (long long)s * N;
      const double u0 = us[n], l0 = ls[n];
      if (ex) px += (us[n + 1] - u0) * (ls[n + 1] - l0);
      if (ey) py += (us[n + sy] - u0) * (ls[n + sy] - l0);
      if (ez) pz += (us[n + sz] - u0) * (ls[n + sz] - l0);
      if (bnd) q += u0 * l0;
    }
    P[n] = px;
    P[N + n] = py;
    P[2 * N + n] = pz;
    Q[n] = q;
  }
}

// g_c = dsig_c * [ (V_c/4) sum_{12 edges e of c} P_e / h_e^2 + sum_{boundary faces f of c} bface_f sum_{4 nodes} Q_n ]
__global__ void k_cell_gradient(const double *__restrict__ P, const double *__restrict__ Q, const double *__restrict__ h,
                                int nx, int ny, int nz, const double *__restrict__ bface, long long o0, long long o1,
                                long long o2, long long o3, long long o4, long long o5,
                                const double *__restrict__ dsig, double scale, double *__restrict__ g) {
  const double *hx = h, *hy = h + nx, *hz = h + nx + ny;
  const int Nx = nx + 1, Ny = ny + 1, Nz = nz + 1;
  const long long N = (long long)Nx * Ny * Nz;
  const long long nC = (long long)nx * ny * nz;
  (void)Nz;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(c / ((long long)nx * ny));
    const int rr = (int)(c - (long long)k * nx * ny);
    const int j = rr / nx, i = rr - j * nx;
    auto node = [&](int a, int b, int e) { return a + (long long)Nx * (b + (long long)Ny * e); };
    const double *Px = P, *Py = P + N, *Pz = P + 2 * N;
    double sx = Px[node(i, j, k)] + Px[node(i, j + 1, k)] + Px[node(i, j, k + 1)] + Px[node(i, j + 1, k + 1)];
    double sy = Py[node(i, j, k)] + Py[node(i + 1, j, k)] + Py[node(i, j, k + 1)] + Py[node(i + 1, j, k + 1)];
    double sz = Pz[node(i, j, k)] + Pz[node(i + 1, j, k)] + Pz[node(i, j + 1, k)] + Pz[node(i + 1, j + 1, k)];
    const double V = hx[i] * hy[j] * hz[k];
    double acc = 0.25 * V * (sx / (hx[i] * hx[i]) + sy / (hy[j] * hy[j]) + sz / (hz[k] * hz[k]));
    if (bface) {
      if (i == 0)
        acc += bface[o0 + j + (long long)ny * k] *
               (Q[node(0, j, k)] + Q[node(0, j + 1, k)] + Q[node(0, j, k + 1)] + Q[node(0, j + 1, k + 1)]);
      if (i == nx - 1)
        acc += bface[o1 + j + (long long)ny * k] *
               (Q[node(nx, j, k)] + Q[node(nx, j + 1, k)] + Q[node(nx, j, k + 1)] + Q[node(nx, j + 1, k + 1)]);
      if (j == 0)
        acc += bface[o2 + i + (long long)nx * k] *
               (Q[node(i, 0, k)] + Q[node(i + 1, 0, k)] + Q[node(i, 0, k + 1)] + Q[node(i + 1, 0, k + 1)]);
      if (j == ny - 1)
        acc += bface[o3 + i + (long long)nx * k] *
               (Q[node(i, ny, k)] + Q[node(i + 1, ny, k)] + Q[node(i, ny, k + 1)] + Q[node(i + 1, ny, k + 1)]);
      if (k == 0)
        acc += bface[o4 + i + (long long)nx * j] *
               (Q[node(i, j, 0)] + Q[node(i + 1, j, 0)] + Q[node(i, j + 1, 0)] + Q[node(i + 1, j + 1, 0)]);
      if (k == nz - 1)
        acc += bface[o5 + i + (long long)nx * j] *
               (Q[node(i, j, nz)] + Q[node(i + 1, j, nz)] + Q[node(i, j + 1, nz)] + Q[node(i + 1, j + 1, nz)]);
    }
    g[c] = scale * (dsig ? dsig[c] : 1.0) * acc;
  }
}

}  // namespace

extern int g_n_sm;

void csr_spmv(int nrows, const long long *rowptr, const long long *in_idx, const double *w, const double *x,
              const long long *out_idx, double *y, double scale, int accumulate, cudaStream_t s) {
  if (nrows <= 0) return;
  k_csr_spmv<<<count_launch(grid_flat(nrows, g_n_sm)), TPB, 0, s>>>(nrows, rowptr, in_idx, w, x, out_idx, y, scale, accumulate);
}

void fill_sparse(long long nnz, const long long *idx, const double *val, double *y, cudaStream_t s) {
  if (nnz <= 0) return;
  k_fill_sparse<<<count_launch(grid_flat(nnz, g_n_sm)), TPB, 0, s>>>(nnz, idx, val, y);
}

void scale_vec(long long n, double *y, double a, cudaStream_t s) {
  if (n <= 0) return;
  k_scale<<<count_launch(grid_flat(n, g_n_sm)), TPB, 0, s>>>(n, y, a);
}

void edge_products(const double *u, const double *l, int K, const Dims &d, double *P, double *Q, cudaStream_t s) {
  k_edge_products<<<count_launch(grid_flat(d.N, g_n_sm)), TPB, 0, s>>>(u, l, K, d, P, Q);
}

void cell_gradient(const Level &L, int robin, const double *P, const double *Q, const double *dsig, double scale,
                   double *g, cudaStream_t s) {
  const long long nC = (long long)L.nx * L.ny * L.nz;
  k_cell_gradient<<<count_launch(grid_flat(nC, g_n_sm)), TPB, 0, s>>>(
      P, Q, L.d_h, L.nx, L.ny, L.nz, robin ? L.d_bface : nullptr, L.bface_off[0], L.bface_off[1], L.bface_off[2],
      L.bface_off[3], L.bface_off[4], L.bface_off[5], dsig, scale, g);
}

}  // namespace dc

// ---------------------------------------------------------------------------
// Model regularisation of the inversion that consumes this path
// (regularization/base.py WeightedLeastSquares: Smallness + SmoothnessFirstOrder
// on a tensor mesh with every cell active):
//   (R v)_c = a_s V_c v_c + sum_dir a_dir sum_{interior faces f of c} w_f (v_c - v_n) / dx_f^2
// with w_f = (V_c + V_n) / 2 and dx_f the distance between the two cell centres
// (zero gradient on boundary faces).  R = deriv2 / 2 of the regulariser.
namespace dc {
namespace {
__global__ void k_reg_apply(const double *__restrict__ h, int nx, int ny, int nz, double as, double ax, double ay,
                            double az, const double *__restrict__ v, double *__restrict__ out, double *__restrict__ dg,
                            double scale) {
  const double *hx = h, *hy = h + nx, *hz = h + nx + ny;
  const long long nC = (long long)nx * ny * nz;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(c / ((long long)nx * ny));
    const int r = (int)(c - (long long)k * nx * ny);
    const int j = r / nx, i = r - j * nx;
    const double V = hx[i] * hy[j] * hz[k];
    const double vc = v ? v[c] : 0.0;
    double acc = as * V * vc, d = as * V;
    auto face = [&](long long nb, double Vn, double dx, double a) {
      const double w = a * 0.5 * (V + Vn) / (dx * dx);
      d += w;
      if (v) acc += w * (vc - v[nb]);
    };
    if (i > 0) face(c - 1, hx[i - 1] * hy[j] * hz[k], 0.5 * (hx[i - 1] + hx[i]), ax);
    if (i + 1 < nx) face(c + 1, hx[i + 1] * hy[j] * hz[k], 0.5 * (hx[i] + hx[i + 1]), ax);
    if (j > 0) face(c - nx, hx[i] * hy[j - 1] * hz[k], 0.5 * (hy[j - 1] + hy[j]), ay);
    if (j + 1 < ny) face(c + nx, hx[i] * hy[j + 1] * hz[k], 0.5 * (hy[j] + hy[j + 1]), ay);
    if (k > 0) face(c - (long long)nx * ny, hx[i] * hy[j] * hz[k - 1], 0.5 * (hz[k - 1] + hz[k]), az);
    if (k + 1 < nz) face(c + (long long)nx * ny, hx[i] * hy[j] * hz[k + 1], 0.5 * (hz[k] + hz[k + 1]), az);
    if (out) out[c] = scale * acc;
    if (dg) dg[c] = scale * d;
  }
}
}  // namespace

void reg_apply(const Level &L, double as, double ax, double ay, double az, const double *v, double *out, double *dg,
               double scale, cudaStream_t s) {
  const long long nC = (long long)L.nx * L.ny * L.nz;
  k_reg_apply<<<count_launch(dim3(grid_flat(nC, g_n_sm))), TPB, 0, s>>>(L.d_h, L.nx, L.ny, L.nz, as, ax, ay, az, v,
                                                                        out, dg, scale);
}
}  // namespace dc

// ---------------------------------------------------------------- derived fields
// Fields3DNodal's e, j, charge and charge_density
// (simpeg/electromagnetics/static/resistivity/fields.py:186-257) from the nodal
// potentials.  Edges are ordered as discretize orders them: all x-edges
// (nx, ny+1, nz+1), then y-edges (nx+1, ny, nz+1), then z-edges
// (nx+1, ny+1, nz), each Fortran-ordered.  The edge inner products are
// diagonal on a tensor mesh: V_c / 4 from every cell c that holds the edge.
namespace dc {
namespace {
struct EdgeGeo {
  int nx, ny, nz;
  long long nEx, nEy, nEz;
};

__host__ __device__ inline EdgeGeo edge_geo(int nx, int ny, int nz) {
  EdgeGeo g{nx, ny, nz, (long long)nx * (ny + 1) * (nz + 1), (long long)(nx + 1) * ny * (nz + 1),
            (long long)(nx + 1) * (ny + 1) * nz};
  return g;
}

// Axis a (0..2) and cell-grid coordinates (i, j, k) of edge e; the edge runs from
// node (i, j, k) one cell along a.
__device__ inline void edge_ijk(const EdgeGeo &g, long long e, int &a, int &i, int &j, int &k) {
  int ex = g.nx, ey = g.ny + 1;
  if (e < g.nEx) {
    a = 0;
  } else if (e < g.nEx + g.nEy) {
    a = 1;
    e -= g.nEx;
    ex = g.nx + 1;
    ey = g.ny;
  } else {
    a = 2;
    e -= g.nEx + g.nEy;
    ex = g.nx + 1;
    ey = g.ny + 1;
  }
  k = (int)(e / ((long long)ex * ey));
  const long long r = e - (long long)k * ex * ey;
  j = (int)(r / ex);
  i = (int)(r - (long long)j * ex);
}

// Sum over the (up to 4) cells holding the edge of V_c (and of sigma_c V_c).
__device__ inline void edge_cells(const double *hx, const double *hy, const double *hz, const double *sigma,
                                  const EdgeGeo &g, int a, int i, int j, int k, double &vsum, double &svsum) {
  vsum = 0.0;
  svsum = 0.0;
  // the edge lies along a; the cells are offset by 0 / -1 in the two other axes
  for (int d1 = -1; d1 <= 0; ++d1)
    for (int d2 = -1; d2 <= 0; ++d2) {
      int ci = i, cj = j, ck = k;
      if (a == 0) {
        cj += d1;
        ck += d2;
      } else if (a == 1) {
        ci += d1;
        ck += d2;
      } else {
        ci += d1;
        cj += d2;
      }
      if (ci < 0 || cj < 0 || ck < 0 || ci >= g.nx || cj >= g.ny || ck >= g.nz) continue;
      const double V = hx[ci] * hy[cj] * hz[ck];
      vsum += V;
      if (sigma) svsum += sigma[ci + (long long)g.nx * (cj + (long long)g.ny * ck)] * V;
    }
}

// e = -G phi; j = e * (sum sigma_c V_c) / (sum V_c)  (MeI MeSigma e)
__global__ void k_edge_fields(const double *__restrict__ phi, int K, EdgeGeo g, const double *__restrict__ h,
                              const double *__restrict__ sigma, double *__restrict__ e, double *__restrict__ jf) {
  const double *hx = h, *hy = h + g.nx, *hz = h + g.nx + g.ny;
  const long long nE = g.nEx + g.nEy + g.nEz;
  const long long N = (long long)(g.nx + 1) * (g.ny + 1) * (g.nz + 1);
  const long long sy = g.nx + 1, sz = (long long)(g.nx + 1) * (g.ny + 1);
  for (long long ed = (long long)blockIdx.x * blockDim.x + threadIdx.x; ed < nE; ed += (long long)gridDim.x * blockDim.x) {
    int a, i, j, k;
    edge_ijk(g, ed, a, i, j, k);
    const long long n0 = i + sy * j + sz * k;
    const long long n1 = n0 + (a == 0 ? 1 : (a == 1 ? sy : sz));
    const double hinv = 1.0 / (a == 0 ? hx[i] : (a == 1 ? hy[j] : hz[k]));
    double ratio = 0.0;
    if (jf) {
      double vs, svs;
      edge_cells(hx, hy, hz, sigma, g, a, i, j, k, vs, svs);
      ratio = svs / vs;
    }
    for (int r = 0; r < K; ++r) {
      const double ev = -(phi[r * N + n1] - phi[r * N + n0]) * hinv;
      if (e) e[r * nE + ed] = ev;
      if (jf) jf[r * nE + ed] = ev * ratio;
    }
  }
}

// charge = -eps0 G^T diag(Me(1)) e at the nodes
__global__ void k_node_charge(const double *__restrict__ e, int K, EdgeGeo g, const double *__restrict__ h,
                              double eps0, double *__restrict__ q) {
  const double *hx = h, *hy = h + g.nx, *hz = h + g.nx + g.ny;
  const long long nE = g.nEx + g.nEy + g.nEz;
  const int Nx = g.nx + 1, Ny = g.ny + 1, Nz = g.nz + 1;
  const long long N = (long long)Nx * Ny * Nz;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(n / ((long long)Nx * Ny));
    const long long rr = n - (long long)k * Nx * Ny;
    const int j = (int)(rr / Nx), i = (int)(rr - (long long)j * Nx);
    // incident edges: (edge index, coefficient of e in (G^T Me1 e)_n)
    long long idx[6];
    double w[6];
    int m = 0;
    auto add = [&](int a, int ei, int ej, int ek, double sign, double hlen) {
      long long ed;
      if (a == 0)
        ed = ei + (long long)g.nx * (ej + (long long)Ny * ek);
      else if (a == 1)
        ed = g.nEx + ei + (long long)Nx * (ej + (long long)g.ny * ek);
      else
        ed = g.nEx + g.nEy + ei + (long long)Nx * (ej + (long long)Ny * ek);
      double vs, svs;
      edge_cells(hx, hy, hz, nullptr, g, a, ei, ej, ek, vs, svs);
      idx[m] = ed;
      w[m] = sign * 0.25 * vs / hlen;
      ++m;
    };
    if (i < g.nx) add(0, i, j, k, -1.0, hx[i]);
    if (i > 0) add(0, i - 1, j, k, 1.0, hx[i - 1]);
    if (j < g.ny) add(1, i, j, k, -1.0, hy[j]);
    if (j > 0) add(1, i, j - 1, k, 1.0, hy[j - 1]);
    if (k < g.nz) add(2, i, j, k, -1.0, hz[k]);
    if (k > 0) add(2, i, j, k - 1, 1.0, hz[k - 1]);
    for (int r = 0; r < K; ++r) {
      double acc = 0.0;
      for (int t = 0; t < m; ++t) acc += w[t] * e[r * nE + idx[t]];
      q[r * N + n] = -eps0 * acc;
    }
  }
}

// charge_density = (average of the cell's 8 node charges) / V_c
__global__ void k_cell_charge_density(const double *__restrict__ q, int K, EdgeGeo g, const double *__restrict__ h,
                                      double *__restrict__ rho) {
  const double *hx = h, *hy = h + g.nx, *hz = h + g.nx + g.ny;
  const long long nC = (long long)g.nx * g.ny * g.nz;
  const long long N = (long long)(g.nx + 1) * (g.ny + 1) * (g.nz + 1);
  const long long sy = g.nx + 1, sz = (long long)(g.nx + 1) * (g.ny + 1);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(c / ((long long)g.nx * g.ny));
    const long long rr = c - (long long)k * g.nx * g.ny;
    const int j = (int)(rr / g.nx), i = (int)(rr - (long long)j * g.nx);
    const long long n0 = i + sy * j + sz * k;
    const double inv = 0.125 / (hx[i] * hy[j] * hz[k]);
    for (int r = 0; r < K; ++r) {
      const double *qr = q + r * N + n0;
      const double s = qr[0] + qr[1] + qr[sy] + qr[sy + 1] + qr[sz] + qr[sz + 1] + qr[sz + sy] + qr[sz + sy + 1];
      rho[r * nC + c] = s * inv;
    }
  }
}
}  // namespace

void edge_fields(const Level &L, const double *phi, int K, double *e, double *j, cudaStream_t s) {
  const EdgeGeo g = edge_geo(L.nx, L.ny, L.nz);
  k_edge_fields<<<count_launch(dim3(grid_flat(g.nEx + g.nEy + g.nEz, g_n_sm))), TPB, 0, s>>>(phi, K, g, L.d_h,
                                                                                          L.d_sigma, e, j);
}

void node_charge(const Level &L, const double *e, int K, double eps0, double *q, double *rho, cudaStream_t s) {
  const EdgeGeo g = edge_geo(L.nx, L.ny, L.nz);
  k_node_charge<<<count_launch(dim3(grid_flat(L.dims.N, g_n_sm))), TPB, 0, s>>>(e, K, g, L.d_h, eps0, q);
  if (rho)
    k_cell_charge_density<<<count_launch(dim3(grid_flat((long long)L.nx * L.ny * L.nz, g_n_sm))), TPB, 0, s>>>(
        q, K, g, L.d_h, rho);
}
}  // namespace dc
