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
