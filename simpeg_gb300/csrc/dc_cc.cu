// Cell-centred formulation (simpeg Simulation3DCellCentered,
// resistivity/simulation.py:321-480): A = Div MfRhoI Grad with Div = V
// face_divergence and Grad = Div^T - B (B: the weak-form Robin term of
// cell_gradient_weak_form_robin).  On a tensor mesh with isotropic rho the
// face inner product is diagonal, Mf_f = sum over the cells c holding face f
// of V_c rho_c / 2, so A is a seven-point stencil on the cell centres:
//   coupling across interior face f:  T_f = A_f^2 / Mf_f
//   boundary face f of cell c:        bw_f / rho_c,  bw_f = (1 - a_f) A_f^2 / (V_c / 2)
// with a_f the ghost-point factor of the Robin condition (1 for Neumann, 0 for
// Dirichlet); bw is geometry only and packed per side like the nodal Robin
// face weights.  The engine solves it on the "dual" tensor mesh whose nodes
// are the cell centres (the same node kernels, multigrid and refinement): the
// finest level's coefficients come from here, the coarse levels are
// rediscretised from a dual conductivity (the mean of the 8 cells' 1/rho
// around each dual cell) with dual Robin weights, which only has to make the
// V-cycle a good preconditioner of the exact fine operator.
#include "../../include/dcgpu.h"
#include "dc_internal.h"

namespace dc {

extern int g_n_sm;

namespace {

constexpr int TPB = 256;

inline int grid_flat(long long total, int n_sm) {
  long long g = (total + TPB - 1) / TPB;
  const long long cap = (long long)n_sm * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

struct Geo {
  const double *hx, *hy, *hz;
  int nx, ny, nz;
  __device__ __forceinline__ double vol(int i, int j, int k) const { return hx[i] * hy[j] * hz[k]; }
  __device__ __forceinline__ long long cell(int i, int j, int k) const {
    return i + (long long)nx * (j + (long long)ny * k);
  }
};

__device__ __forceinline__ Geo geo(const double *h, int nx, int ny, int nz) {
  return Geo{h, h + nx, h + nx + ny, nx, ny, nz};
}

// face inner product of face f between cells (V0, r0) and (V1, r1)
__device__ __forceinline__ double mf2(double V0, double r0, double V1, double r1) { return 0.5 * (V0 * r0 + V1 * r1); }

// Boundary weight of cell (i, j, k) summed over its boundary faces (packed bw; NULL = none).
__device__ __forceinline__ double bnd_weight(const double *bw, const long long *off, int i, int j, int k, int nx,
                                             int ny, int nz) {
  if (!bw) return 0.0;
  double w = 0.0;
  if (i == 0) w += bw[off[0] + j + (long long)ny * k];
  if (i == nx - 1) w += bw[off[1] + j + (long long)ny * k];
  if (j == 0) w += bw[off[2] + i + (long long)nx * k];
  if (j == ny - 1) w += bw[off[3] + i + (long long)nx * k];
  if (k == 0) w += bw[off[4] + i + (long long)nx * j];
  if (k == nz - 1) w += bw[off[5] + i + (long long)nx * j];
  return w;
}

struct Off6 {
  long long o[6];
};

// Exact fine-level operator: per cell {c+x, c+y, c+z, diag} (couplings to the + neighbours), fp32
// copies, 1/diag and the Gershgorin bound of D^-1 A.
__global__ void k_cc_coef(const double *__restrict__ rho, const double *__restrict__ h, int nx, int ny, int nz,
                          const double *__restrict__ bw, Off6 off, Coef64 *__restrict__ c64, Coef32 *__restrict__ c32,
                          double *__restrict__ invd64, float *__restrict__ invd32,
                          unsigned long long *__restrict__ lmax_bits) {
  const Geo g = geo(h, nx, ny, nz);
  const long long nC = (long long)nx * ny * nz;
  double gmax = 0.0;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(c / ((long long)nx * ny));
    const int r = (int)(c - (long long)k * nx * ny);
    const int j = r / nx, i = r - j * nx;
    const double V = g.vol(i, j, k), rc = rho[c];
    const double Ax = g.hy[j] * g.hz[k], Ay = g.hx[i] * g.hz[k], Az = g.hx[i] * g.hy[j];
    auto T = [&](double A, long long nb, int ii, int jj, int kk) {
      return A * A / mf2(V, rc, g.vol(ii, jj, kk), rho[nb]);
    };
    const double txp = i + 1 < nx ? T(Ax, c + 1, i + 1, j, k) : 0.0;
    const double txm = i > 0 ? T(Ax, c - 1, i - 1, j, k) : 0.0;
    const double typ = j + 1 < ny ? T(Ay, c + nx, i, j + 1, k) : 0.0;
    const double tym = j > 0 ? T(Ay, c - nx, i, j - 1, k) : 0.0;
    const double tzp = k + 1 < nz ? T(Az, c + (long long)nx * ny, i, j, k + 1) : 0.0;
    const double tzm = k > 0 ? T(Az, c - (long long)nx * ny, i, j, k - 1) : 0.0;
    const double offd = txp + txm + typ + tym + tzp + tzm;
    const double dg = offd + bnd_weight(bw, off.o, i, j, k, nx, ny, nz) / rc;
    Coef64 cc;
    cc.cx = txp; cc.cy = typ; cc.cz = tzp; cc.d = dg;
    c64[c] = cc;
    Coef32 f;
    f.cx = (float)txp; f.cy = (float)typ; f.cz = (float)tzp; f.d = (float)dg;
    c32[c] = f;
    const double id = dg > 0.0 ? 1.0 / dg : 0.0;
    invd64[c] = id;
    invd32[c] = (float)id;
    if (dg > 0.0) gmax = fmax(gmax, 1.0 + offd / dg);
  }
  for (int o = 16; o > 0; o >>= 1) gmax = fmax(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(lmax_bits, (unsigned long long)__double_as_longlong(gmax));
}

// dA[drho] as a stencil: dT_f = -(A_f^2 / Mf_f^2) dMf_f, dMf_f = sum V_c drho_c / 2; boundary
// -bw_f drho_c / rho_c^2.
__global__ void k_cc_dcoef(const double *__restrict__ rho, const double *__restrict__ drho,
                           const double *__restrict__ h, int nx, int ny, int nz, const double *__restrict__ bw, Off6 off,
                           Coef64 *__restrict__ c64) {
  const Geo g = geo(h, nx, ny, nz);
  const long long nC = (long long)nx * ny * nz;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(c / ((long long)nx * ny));
    const int r = (int)(c - (long long)k * nx * ny);
    const int j = r / nx, i = r - j * nx;
    const double V = g.vol(i, j, k), rc = rho[c], dc_ = drho[c];
    const double Ax = g.hy[j] * g.hz[k], Ay = g.hx[i] * g.hz[k], Az = g.hx[i] * g.hy[j];
    auto dT = [&](double A, long long nb, int ii, int jj, int kk) {
      const double Vn = g.vol(ii, jj, kk);
      const double m = mf2(V, rc, Vn, rho[nb]);
      return -(A * A / (m * m)) * mf2(V, dc_, Vn, drho[nb]);
    };
    const double txp = i + 1 < nx ? dT(Ax, c + 1, i + 1, j, k) : 0.0;
    const double txm = i > 0 ? dT(Ax, c - 1, i - 1, j, k) : 0.0;
    const double typ = j + 1 < ny ? dT(Ay, c + nx, i, j + 1, k) : 0.0;
    const double tym = j > 0 ? dT(Ay, c - nx, i, j - 1, k) : 0.0;
    const double tzp = k + 1 < nz ? dT(Az, c + (long long)nx * ny, i, j, k + 1) : 0.0;
    const double tzm = k > 0 ? dT(Az, c - (long long)nx * ny, i, j, k - 1) : 0.0;
    Coef64 cc;
    cc.cx = txp; cc.cy = typ; cc.cz = tzp;
    cc.d = txp + txm + typ + tym + tzp + tzm - bnd_weight(bw, off.o, i, j, k, nx, ny, nz) * dc_ / (rc * rc);
    c64[c] = cc;
  }
}

// Adjoint: g_c = scale * drho_dm_c * [ sum over the faces f of c of -(A_f^2 / Mf_f^2)(V_c / 2) P_f
//                                      - (bw_c / rho_c^2) Q_c ]
// with P_f = sum_s (u_c - u_n)(l_c - l_n) across f and Q_c = sum_s u_c l_c (k_edge_products on the
// cell-centre grid: P[0..2] the +x, +y, +z face of each cell).
__global__ void k_cc_gradient(const double *__restrict__ P, const double *__restrict__ Q,
                              const double *__restrict__ rho, const double *__restrict__ h, int nx, int ny, int nz,
                              const double *__restrict__ bw, Off6 off, const double *__restrict__ drho_dm, double scale,
                              double *__restrict__ gout) {
  const Geo g = geo(h, nx, ny, nz);
  const long long nC = (long long)nx * ny * nz;
  const double *Px = P, *Py = P + nC, *Pz = P + 2 * nC;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(c / ((long long)nx * ny));
    const int r = (int)(c - (long long)k * nx * ny);
    const int j = r / nx, i = r - j * nx;
    const double V = g.vol(i, j, k), rc = rho[c];
    const double Ax = g.hy[j] * g.hz[k], Ay = g.hx[i] * g.hz[k], Az = g.hx[i] * g.hy[j];
    auto w = [&](double A, long long nb, int ii, int jj, int kk) {
      const double m = mf2(V, rc, g.vol(ii, jj, kk), rho[nb]);
      return -(A * A / (m * m)) * 0.5 * V;
    };
    double acc = 0.0;
    if (i + 1 < nx) acc += w(Ax, c + 1, i + 1, j, k) * Px[c];
    if (i > 0) acc += w(Ax, c - 1, i - 1, j, k) * Px[c - 1];
    if (j + 1 < ny) acc += w(Ay, c + nx, i, j + 1, k) * Py[c];
    if (j > 0) acc += w(Ay, c - nx, i, j - 1, k) * Py[c - nx];
    if (k + 1 < nz) acc += w(Az, c + (long long)nx * ny, i, j, k + 1) * Pz[c];
    if (k > 0) acc += w(Az, c - (long long)nx * ny, i, j, k - 1) * Pz[c - (long long)nx * ny];
    const double bwc = bnd_weight(bw, off.o, i, j, k, nx, ny, nz);
    if (bwc != 0.0) acc -= bwc / (rc * rc) * Q[c];
    gout[c] = scale * (drho_dm ? drho_dm[c] : 1.0) * acc;
  }
}

// Dual conductivity: the mean of 1/rho over the 8 cells around each cell of the cell-centre grid.
__global__ void k_cc_dual_sigma(const double *__restrict__ rho, int nx, int ny, int nz, double *__restrict__ sd) {
  const int mx = nx - 1, my = ny - 1, mz = nz - 1;
  const long long nD = (long long)mx * my * mz;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nD; e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e / ((long long)mx * my));
    const int r = (int)(e - (long long)k * mx * my);
    const int j = r / mx, i = r - j * mx;
    double s = 0.0;
    for (int c = 0; c < 8; ++c)
      s += 1.0 / rho[(i + (c & 1)) + (long long)nx * ((j + ((c >> 1) & 1)) + (long long)ny * (k + (c >> 2)))];
    sd[e] = 0.125 * s;
  }
}

// Fields3DCellCentered (fields.py:130-156): per face f and source s, (Grad phi)_f with
// Grad = Div^T - B: A_f (phi_L - phi_R) across an interior face (L on the face's - side),
// -/+ A_f (1 - a_f) phi_c on a boundary face of the mesh's -/+ side (A_f (1 - a_f) = bw_f h_n / 2);
// e = Grad phi / Mf(1) and j = Grad phi / Mf(rho).  Faces x|y|z, each Fortran-ordered;
// outputs column-major (nF, K).
__global__ void k_cc_face_fields(const double *__restrict__ phi, int K, const double *__restrict__ rho,
                                 const double *__restrict__ h, int nx, int ny, int nz, const double *__restrict__ bw,
                                 Off6 off, double *__restrict__ eo, double *__restrict__ jo) {
  const Geo g = geo(h, nx, ny, nz);
  const long long nC = (long long)nx * ny * nz;
  const long long nfx = (long long)(nx + 1) * ny * nz, nfy = (long long)nx * (ny + 1) * nz;
  const long long nF = nfx + nfy + (long long)nx * ny * (nz + 1);
  const long long total = nF * K;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(t / nF);
    const long long f = t - (long long)s * nF;
    const double *ph = phi + (long long)s * nC;
    int ax, i, j, k;
    long long r;
    if (f < nfx) {
      ax = 0; r = f;
      i = (int)(r % (nx + 1)); r /= (nx + 1); j = (int)(r % ny); k = (int)(r / ny);
    } else if (f < nfx + nfy) {
      ax = 1; r = f - nfx;
      i = (int)(r % nx); r /= nx; j = (int)(r % (ny + 1)); k = (int)(r / (ny + 1));
    } else {
      ax = 2; r = f - nfx - nfy;
      i = (int)(r % nx); r /= nx; j = (int)(r % ny); k = (int)(r / ny);
    }
    const int pos = ax == 0 ? i : (ax == 1 ? j : k);  // face index along the axis
    const int n_ax = ax == 0 ? nx : (ax == 1 ? ny : nz);
    const double A = ax == 0 ? g.hy[j] * g.hz[k] : (ax == 1 ? g.hx[i] * g.hz[k] : g.hx[i] * g.hy[j]);
    // the cells on the face's - side (L) and + side (R)
    int li = i, lj = j, lk = k;
    if (ax == 0) li = i - 1; else if (ax == 1) lj = j - 1; else lk = k - 1;
    double G, mrho, mone;
    if (pos > 0 && pos < n_ax) {
      const long long L = g.cell(li, lj, lk), R = g.cell(i, j, k);
      const double VL = g.vol(li, lj, lk), VR = g.vol(i, j, k);
      G = A * (ph[L] - ph[R]);
      mrho = 0.5 * (VL * rho[L] + VR * rho[R]);
      mone = 0.5 * (VL + VR);
    } else {
      const bool lo = pos == 0;  // the mesh's - side: the cell is on the face's + side
      const int ci = lo ? i : li, cj = lo ? j : lj, ck = lo ? k : lk;
      const long long c = g.cell(ci, cj, ck);
      const double V = g.vol(ci, cj, ck);
      double one_minus_a_A = 0.0;
      if (bw) {
        const int side = 2 * ax + (lo ? 0 : 1);
        const long long in = ax == 0 ? cj + (long long)ny * ck : (ax == 1 ? ci + (long long)nx * ck : ci + (long long)nx * cj);
        const double hn = ax == 0 ? g.hx[ci] : (ax == 1 ? g.hy[cj] : g.hz[ck]);
        one_minus_a_A = bw[off.o[side] + in] * 0.5 * hn;
      }
      G = (lo ? -1.0 : 1.0) * one_minus_a_A * ph[c];
      mrho = 0.5 * V * rho[c];
      mone = 0.5 * V;
    }
    if (eo) eo[t] = G / mone;
    if (jo) jo[t] = G / mrho;
  }
}

// charge = eps0 Div e (cells; fields.py:166-185) and charge_density = charge / V, per source.
__global__ void k_cc_charge(const double *__restrict__ e, int K, const double *__restrict__ h, int nx, int ny, int nz,
                            double eps0, double *__restrict__ q, double *__restrict__ qd) {
  const Geo g = geo(h, nx, ny, nz);
  const long long nC = (long long)nx * ny * nz;
  const long long nfx = (long long)(nx + 1) * ny * nz, nfy = (long long)nx * (ny + 1) * nz;
  const long long nF = nfx + nfy + (long long)nx * ny * (nz + 1);
  const long long total = nC * K;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(t / nC);
    const long long c = t - (long long)s * nC;
    const int k = (int)(c / ((long long)nx * ny));
    const int r = (int)(c - (long long)k * nx * ny);
    const int j = r / nx, i = r - j * nx;
    const double *es = e + (long long)s * nF;
    const long long fx = i + (long long)(nx + 1) * (j + (long long)ny * k);
    const long long fy = nfx + i + (long long)nx * (j + (long long)(ny + 1) * k);
    const long long fz = nfx + nfy + c;
    const double div = g.hy[j] * g.hz[k] * (es[fx + 1] - es[fx]) + g.hx[i] * g.hz[k] * (es[fy + nx] - es[fy]) +
                       g.hx[i] * g.hy[j] * (es[fz + (long long)nx * ny] - es[fz]);
    const double qv = eps0 * div;
    if (q) q[t] = qv;
    if (qd) qd[t] = qv / g.vol(i, j, k);
  }
}

Off6 offsets6(int nx, int ny, int nz) {
  const long long nyz = (long long)ny * nz, nxz = (long long)nx * nz, nxy = (long long)nx * ny;
  return Off6{{0, nyz, 2 * nyz, 2 * nyz + nxz, 2 * nyz + 2 * nxz, 2 * nyz + 2 * nxz + nxy}};
}

}  // namespace

void cc_dual_sigma(const double *rho, int nx, int ny, int nz, double *sd, cudaStream_t s) {
  const long long nD = (long long)(nx - 1) * (ny - 1) * (nz - 1);
  k_cc_dual_sigma<<<count_launch(grid_flat(nD, g_n_sm)), TPB, 0, s>>>(rho, nx, ny, nz, sd);
}

void cc_coef_build(const Level &L, const double *rho, const double *hp, const double *bw,
                   unsigned long long *d_lmax_bits, cudaStream_t s) {
  const int nx = L.dims.Nx, ny = L.dims.Ny, nz = L.dims.Nz;  // the cells are the level's nodes
  k_cc_coef<<<count_launch(grid_flat(L.dims.N, g_n_sm)), TPB, 0, s>>>(rho, hp, nx, ny, nz, bw, offsets6(nx, ny, nz),
                                                                     L.d_coef64, L.d_coef32, L.d_invd64, L.d_invd32,
                                                                     d_lmax_bits);
}

void cc_dcoef_build(const Dims &d, const double *rho, const double *drho, const double *hp, const double *bw,
                    Coef64 *c64, cudaStream_t s) {
  k_cc_dcoef<<<count_launch(grid_flat(d.N, g_n_sm)), TPB, 0, s>>>(rho, drho, hp, d.Nx, d.Ny, d.Nz, bw,
                                                                  offsets6(d.Nx, d.Ny, d.Nz), c64);
}

void cc_face_fields(const Dims &d, const double *phi, int K, const double *rho, const double *hp, const double *bw,
                    double *e, double *j, cudaStream_t s) {
  const long long nF = (long long)(d.Nx + 1) * d.Ny * d.Nz + (long long)d.Nx * (d.Ny + 1) * d.Nz +
                       (long long)d.Nx * d.Ny * (d.Nz + 1);
  k_cc_face_fields<<<count_launch(grid_flat(nF * K, g_n_sm)), TPB, 0, s>>>(phi, K, rho, hp, d.Nx, d.Ny, d.Nz, bw,
                                                                          offsets6(d.Nx, d.Ny, d.Nz), e, j);
}

void cc_charge(const Dims &d, const double *e, int K, const double *hp, double eps0, double *q, double *qd,
               cudaStream_t s) {
  k_cc_charge<<<count_launch(grid_flat(d.N * K, g_n_sm)), TPB, 0, s>>>(e, K, hp, d.Nx, d.Ny, d.Nz, eps0, q, qd);
}

void cc_gradient(const Dims &d, const double *P, const double *Q, const double *rho, const double *hp,
                 const double *bw, const double *drho_dm, double scale, double *g, cudaStream_t s) {
  k_cc_gradient<<<count_launch(grid_flat(d.N, g_n_sm)), TPB, 0, s>>>(P, Q, rho, hp, d.Nx, d.Ny, d.Nz, bw,
                                                                    offsets6(d.Nx, d.Ny, d.Nz), drho_dm, scale, g);
}

}  // namespace dc
