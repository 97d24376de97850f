// Exact diag(J^T W^T W J) without forming J, by electrode reciprocity.
//
// The reference forms the full sensitivity (one adjoint solve per datum, a
// dense (nD, nC) matrix) and sums W_d^2 J_d^2 row by row
// (resistivity/simulation.py:115-154).  Here, with Phi_k = A^-1 q_k the pole
// solution of unique electrode k (q_k its interpolation row), every datum d of
// source s is
//     J_dc = -sigma'_c * B_c(u_s, lambda_d),
//     u_s = sum_{k in src(s)} I_k Phi_k,   lambda_d = sum_{k in rx(d)} c_dk Phi_k,
// with B_c the cell-local bilinear form of dA/dsigma_c:
//     B_c(a, b) = (V_c/4) sum_{12 edges e of c} (G a)_e (G b)_e
//               + sum_{boundary faces f of c} bface_f sum_{4 nodes n of f} a_n b_n.
// One CTA owns a 2x2x2 tile of cells (27 nodes): it stages every electrode's
// pole solution on those nodes in shared memory (relative to the tile centre,
// in fp32, so gradients keep fp32 relative accuracy), then streams the data,
// accumulating W_d^2 J_dc^2 per cell in fp32 per thread (sums of positive
// terms; the per-thread sums are combined in fp64).  The per-datum arithmetic
// is fp32, the Robin term of boundary cells included (the tile-centre values
// and the cells' boundary weights are staged in fp32 once per tile), and the per-datum currents
// and weights are converted to fp32 once per call, not once per tile: on this
// part fp64 arithmetic and the fp64 <-> fp32 conversions issue at 1/64 of the
// fp32 rate.  Cost: nE pole solves plus O(nD * nC) fp32 arithmetic with no J
// in memory.
#include "../../include/dcgpu.h"
#include "dc_internal.h"

#include <mutex>
#include <string>

namespace dc {
namespace {

constexpr int JTPB = 384;

struct JtjData {
  const int *sa, *sb, *rm, *rn;  // electrode indices (-1 = none)
  const float *w;                // fp32 [ia | ib | wm | wn | w2], nD each: currents, receiver weights,
                                 // squared data weights
  int nD;
};

// The per-datum currents and weights in fp32, [ia | ib | wm | wn | w2]
__global__ void k_jtj_weights(int nD, const double *__restrict__ ia, const double *__restrict__ ib,
                              const double *__restrict__ wm, const double *__restrict__ wn,
                              const double *__restrict__ w2, float *__restrict__ w) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nD; d += gridDim.x * blockDim.x) {
    w[d] = (float)ia[d];
    w[nD + d] = (float)ib[d];
    w[2 * nD + d] = (float)wm[d];
    w[3 * nD + d] = (float)wn[d];
    w[4 * nD + d] = (float)w2[d];
  }
}

__global__ void __launch_bounds__(JTPB) k_jtj_diag(const double *__restrict__ phi, int nE, long long N,
                                                    int nx, int ny, int nz, const double *__restrict__ h,
                                                    const double *__restrict__ bface, long long bo0, long long bo1,
                                                    long long bo2, long long bo3, long long bo4, long long bo5,
                                                    const double *__restrict__ dsig, JtjData D,
                                                    double *__restrict__ diag) {
  extern __shared__ unsigned char smem_raw[];
  double *ref = reinterpret_cast<double *>(smem_raw);        // nE
  float *reff = reinterpret_cast<float *>(ref + nE);         // nE: ref in fp32
  float *dphi = reff + nE;                                   // nE * 27
  __shared__ double red[JTPB / 32][8];
  __shared__ float bwf[8][6];  // Robin face weights of the tile's cells (0 off the boundary)
  const double *hx = h, *hy = h + nx, *hz = h + nx + ny;
  const int Nx = nx + 1, Ny = ny + 1;
  const int tx = (nx + 1) / 2, ty = (ny + 1) / 2;
  const int tile = blockIdx.x;
  const int TI = tile % tx, TJ = (tile / tx) % ty, TK = tile / (tx * ty);
  const int i0 = 2 * TI, j0 = 2 * TJ, k0 = 2 * TK;
  // tile node (a, b, c) in {0,1,2}^3 clamped to the mesh
  auto node = [&](int a, int b, int c) {
    const int i = min(i0 + a, nx), j = min(j0 + b, ny), k = min(k0 + c, nz);
    return (long long)i + (long long)Nx * (j + (long long)Ny * k);
  };
  const long long centre = node(1, 1, 1);
  for (int k = threadIdx.x; k < nE; k += JTPB) {
    ref[k] = phi[(long long)k * N + centre];
    reff[k] = (float)ref[k];
  }
  if (threadIdx.x < 48) {
    // face f of tile cell c: x-lo, x-hi, y-lo, y-hi, z-lo, z-hi
    const int c = threadIdx.x / 6, f = threadIdx.x % 6;
    const int ci = i0 + (c & 1), cj = j0 + ((c >> 1) & 1), ck = k0 + (c >> 2);
    float w = 0.f;
    if (bface && ci < nx && cj < ny && ck < nz) {
      if (f == 0 && ci == 0) w = (float)bface[bo0 + cj + (long long)ny * ck];
      if (f == 1 && ci == nx - 1) w = (float)bface[bo1 + cj + (long long)ny * ck];
      if (f == 2 && cj == 0) w = (float)bface[bo2 + ci + (long long)nx * ck];
      if (f == 3 && cj == ny - 1) w = (float)bface[bo3 + ci + (long long)nx * ck];
      if (f == 4 && ck == 0) w = (float)bface[bo4 + ci + (long long)nx * cj];
      if (f == 5 && ck == nz - 1) w = (float)bface[bo5 + ci + (long long)nx * cj];
    }
    bwf[c][f] = w;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nE * 27; e += JTPB) {
    const int k = e / 27, j = e % 27;
    const long long n = node(j % 3, (j / 3) % 3, j / 9);
    dphi[e] = (float)(phi[(long long)k * N + n] - ref[k]);
  }
  __syncthreads();
  // cell geometry of the 8 tile cells
  bool have[8];
  float wx[8], wy[8], wz[8];
  float sg[8];
  int bnd[8];
  for (int c = 0; c < 8; ++c) {
    const int ci = i0 + (c & 1), cj = j0 + ((c >> 1) & 1), ck = k0 + (c >> 2);
    have[c] = ci < nx && cj < ny && ck < nz;
    wx[c] = wy[c] = wz[c] = 0.f;
    sg[c] = 0.f;
    bnd[c] = 0;
    if (have[c]) {
      const double V = hx[ci] * hy[cj] * hz[ck];
      wx[c] = (float)(0.25 * V / (hx[ci] * hx[ci]));
      wy[c] = (float)(0.25 * V / (hy[cj] * hy[cj]));
      wz[c] = (float)(0.25 * V / (hz[ck] * hz[ck]));
      sg[c] = dsig ? (float)dsig[ci + (long long)nx * (cj + (long long)ny * ck)] : 1.f;
      if (bface) bnd[c] = (ci == 0) | ((ci == nx - 1) << 1) | ((cj == 0) << 2) | ((cj == ny - 1) << 3) |
                          ((ck == 0) << 4) | ((ck == nz - 1) << 5);
    }
  }
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int d = threadIdx.x; d < D.nD; d += JTPB) {
    const int sa = D.sa[d], sb = D.sb[d], rm = D.rm[d], rn = D.rn[d];
    const int nD = D.nD;
    const float ia = D.w[d], ib = sb >= 0 ? D.w[nD + d] : 0.f;
    const float wm = D.w[2 * nD + d], wn = rn >= 0 ? D.w[3 * nD + d] : 0.f;
    const float *pa = dphi + sa * 27, *pb = dphi + (sb >= 0 ? sb : sa) * 27;
    const float *pm = dphi + rm * 27, *pn = dphi + (rn >= 0 ? rn : rm) * 27;
    float u[27], l[27];
#pragma unroll
    for (int j = 0; j < 27; ++j) {
      u[j] = ia * pa[j] + ib * pb[j];
      l[j] = wm * pm[j] + wn * pn[j];
    }
    const float w2 = D.w[4 * nD + d];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (!have[c]) continue;
      const int a0 = c & 1, b0 = (c >> 1) & 1, c0 = c >> 2;
      auto id = [&](int a, int b, int e) { return (a0 + a) + 3 * ((b0 + b) + 3 * (c0 + e)); };
      float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          sx += (u[id(1, p, q)] - u[id(0, p, q)]) * (l[id(1, p, q)] - l[id(0, p, q)]);
          sy += (u[id(p, 1, q)] - u[id(p, 0, q)]) * (l[id(p, 1, q)] - l[id(p, 0, q)]);
          sz += (u[id(p, q, 1)] - u[id(p, q, 0)]) * (l[id(p, q, 1)] - l[id(p, q, 0)]);
        }
      float a = wx[c] * sx + wy[c] * sy + wz[c] * sz;
      if (bnd[c]) {
        // Robin part: absolute potentials (tile-centre value + relative one) on the boundary faces of
        // the cell, in fp32 like the rest of the per-datum arithmetic (weights and centre values staged
        // in fp32 once per tile)
        const float ur = ia * reff[sa] + (sb >= 0 ? ib * reff[sb] : 0.f);
        const float lr = wm * reff[rm] + (rn >= 0 ? wn * reff[rn] : 0.f);
        auto ul = [&](int a2, int b2, int e2) {
          const int j = id(a2, b2, e2);
          return (u[j] + ur) * (l[j] + lr);
        };
        float ab = 0.f;
        if (bnd[c] & 1) ab += bwf[c][0] * (ul(0, 0, 0) + ul(0, 1, 0) + ul(0, 0, 1) + ul(0, 1, 1));
        if (bnd[c] & 2) ab += bwf[c][1] * (ul(1, 0, 0) + ul(1, 1, 0) + ul(1, 0, 1) + ul(1, 1, 1));
        if (bnd[c] & 4) ab += bwf[c][2] * (ul(0, 0, 0) + ul(1, 0, 0) + ul(0, 0, 1) + ul(1, 0, 1));
        if (bnd[c] & 8) ab += bwf[c][3] * (ul(0, 1, 0) + ul(1, 1, 0) + ul(0, 1, 1) + ul(1, 1, 1));
        if (bnd[c] & 16) ab += bwf[c][4] * (ul(0, 0, 0) + ul(1, 0, 0) + ul(0, 1, 0) + ul(1, 1, 0));
        if (bnd[c] & 32) ab += bwf[c][5] * (ul(0, 0, 1) + ul(1, 0, 1) + ul(0, 1, 1) + ul(1, 1, 1));
        a += ab;
      }
      const float jv = sg[c] * a;
      acc[c] += w2 * jv * jv;
    }
  }
  // block reduction of the 8 per-cell sums
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    double v = (double)acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8 && have[threadIdx.x]) {
    const int c = threadIdx.x;
    double s = 0.0;
    for (int w = 0; w < JTPB / 32; ++w) s += red[w][c];
    const int ci = i0 + (c & 1), cj = j0 + ((c >> 1) & 1), ck = k0 + (c >> 2);
    diag[ci + (long long)nx * (cj + (long long)ny * ck)] = s;
  }
}

}  // namespace
}  // namespace dc

namespace dc {

int jtj_diag_launch(const Level &L, int robin, const double *phi, int nE, int nD, const int *sa, const int *sb,
                    const double *ia, const double *ib, const int *rm, const int *rn, const double *wm,
                    const double *wn, const double *w2, const double *dsig, double *diag, cudaStream_t stream) {
  const size_t smem = (size_t)nE * (sizeof(double) + 28 * sizeof(float));
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t static_smem = 8 * 8 * (JTPB / 32) + 8 * 6 * sizeof(float);
  if (smem + static_smem > (size_t)maxsm) {
    last_error() = "dc_jtj_diag: " + std::to_string(nE) + " unique electrodes exceed the shared-memory tile (max " +
                   std::to_string((maxsm - static_smem) / (sizeof(double) + 28 * sizeof(float))) + ")";
    return DC_ERR_ARG;
  }
  // The dynamic shared-memory limit is raised once per device, to the largest tile the check above admits:
  // set per call, a concurrent call with a smaller tile could lower it between another's set and launch.
  {
    static std::mutex mu;
    static unsigned long long raised = 0;  // bit per device
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 64) {
      last_error() = "dc_jtj_diag: device ordinal above 63";
      return DC_ERR_ARG;
    }
    if (!(raised >> dev & 1ull)) {
      const cudaError_t e = cudaFuncSetAttribute(k_jtj_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)((size_t)maxsm - static_smem));
      if (e != cudaSuccess) {
        last_error() = std::string("dc_jtj_diag: ") + cudaGetErrorString(e);
        return DC_ERR_CUDA;
      }
      raised |= 1ull << dev;
    }
  }
  float *w32 = nullptr;
  if (cudaMallocAsync((void **)&w32, sizeof(float) * 5 * (size_t)(nD > 0 ? nD : 1), stream) != cudaSuccess) {
    last_error() = "dc_jtj_diag: cannot allocate the fp32 weights";
    return DC_ERR_NOMEM;
  }
  if (nD > 0) k_jtj_weights<<<count_launch(dim3((nD + 255) / 256)), 256, 0, stream>>>(nD, ia, ib, wm, wn, w2, w32);
  JtjData D{sa, sb, rm, rn, w32, nD};
  const int tiles = ((L.nx + 1) / 2) * ((L.ny + 1) / 2) * ((L.nz + 1) / 2);
  k_jtj_diag<<<count_launch(dim3(tiles)), JTPB, smem, stream>>>(
      phi, nE, L.dims.N, L.nx, L.ny, L.nz, L.d_h, robin ? L.d_bface : nullptr, L.bface_off[0], L.bface_off[1],
      L.bface_off[2], L.bface_off[3], L.bface_off[4], L.bface_off[5], dsig, D, diag);
  cudaFreeAsync(w32, stream);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    last_error() = std::string("dc_jtj_diag: ") + cudaGetErrorString(e);
    return DC_ERR_CUDA;
  }
  return DC_OK;
}

}  // namespace dc
