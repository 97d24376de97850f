// Generic sparse SPD solver behind the simpeg Solver plug-in slot.
//
// simpeg's BasePDESimulation accepts any pymatsolver-compatible solver class
// (base/pde_simulation.py:493-511) and calls `solver(A)` with the assembled
// CSR matrix, then `Ainv * RHS` (resistivity/simulation.py:108-111).  This
// file is the device side of that plug-in: the CSR matrix is uploaded once,
// and every solve is a multi-RHS Jacobi-preconditioned CG in fp64 on
// column-major (n x k) right-hand sides.  It serves any SPD matrix simpeg
// hands over; the matrix-free multigrid path (dc_engine.cu) is the fast path
// for Simulation3DNodal itself.
#include "../../include/dcgpu.h"
#include "dc_internal.h"

#include <cmath>
#include <memory>
#include <new>

using namespace dc;

namespace {

constexpr int TPB = 256;

int fail(int code, const std::string &msg) {
  last_error() = msg;
  return code;
}

#define CK(expr)                                                                                          \
  do {                                                                                                    \
    cudaError_t _e = (expr);                                                                              \
    if (_e != cudaSuccess) return fail(DC_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// q(:, c) = A p(:, c) for column c = blockIdx.y ; per-block partials of p.q, laid out
// [c][gridDim.x] like the engine's reductions with one lane per RHS block.
__global__ void __launch_bounds__(TPB) k_csr_apply_dot(int n, const long long *__restrict__ ptr,
                                                       const int *__restrict__ idx, const double *__restrict__ val,
                                                       const double *__restrict__ p, double *__restrict__ q,
                                                       double *__restrict__ partial) {
  __shared__ double red[TPB / 32];
  const long long base = (long long)blockIdx.y * n;
  double acc = 0.0;
  for (int r = blockIdx.x * TPB + threadIdx.x; r < n; r += gridDim.x * TPB) {
    double s = 0.0;
    for (long long e = ptr[r]; e < ptr[r + 1]; ++e) s += val[e] * p[base + idx[e]];
    q[base + r] = s;
    acc += s * p[base + r];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < TPB / 32; ++w) s += red[w];
    partial[(long long)blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}

// z = D^-1 r ; partial r.z  (column c = blockIdx.y)
__global__ void __launch_bounds__(TPB) k_jacobi_dot(int n, const double *__restrict__ dinv,
                                                    const double *__restrict__ r, double *__restrict__ z,
                                                    double *__restrict__ partial) {
  __shared__ double red[TPB / 32];
  const long long base = (long long)blockIdx.y * n;
  double acc = 0.0;
  for (int i = blockIdx.x * TPB + threadIdx.x; i < n; i += gridDim.x * TPB) {
    const double v = dinv[i] * r[base + i];
    z[base + i] = v;
    acc += v * r[base + i];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < TPB / 32; ++w) s += red[w];
    partial[(long long)blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void k_csr_diag_inv(int n, const long long *__restrict__ ptr, const int *__restrict__ idx,
                               const double *__restrict__ val, double *__restrict__ dinv, int *__restrict__ bad) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double d = 0.0;
    for (long long e = ptr[r]; e < ptr[r + 1]; ++e)
      if (idx[e] == r) d += val[e];
    if (!(d > 0.0)) atomicOr(bad, 1);
    dinv[r] = d > 0.0 ? 1.0 / d : 0.0;
  }
}

}  // namespace

struct dc_csr {
  int n = 0;
  long long nnz = 0;
  long long *ptr = nullptr;
  int *idx = nullptr;
  double *val = nullptr, *dinv = nullptr;
  int *bad = nullptr;
  void *ws = nullptr;
  size_t ws_bytes = 0;
  int *h_mail = nullptr;
  cudaEvent_t ev = nullptr;
};

extern "C" {

int dc_csr_create(int n, long long nnz, const long long *indptr, const int *indices, const double *data,
                  dc_csr **out) {
  if (!out || n < 1 || nnz < 1 || !indptr || !indices || !data) return fail(DC_ERR_ARG, "bad argument");
  *out = nullptr;
  if (indptr[0] != 0 || indptr[n] != nnz) return fail(DC_ERR_ARG, "indptr is inconsistent with nnz");
  for (int r = 0; r < n; ++r)
    if (indptr[r + 1] < indptr[r]) return fail(DC_ERR_ARG, "indptr must be non-decreasing");
  for (long long e = 0; e < nnz; ++e)
    if (indices[e] < 0 || indices[e] >= n) return fail(DC_ERR_ARG, "column index out of range");
  std::unique_ptr<dc_csr> h(new (std::nothrow) dc_csr());
  if (!h) return fail(DC_ERR_NOMEM, "host allocation failed");
  h->n = n;
  h->nnz = nnz;
  CK(cudaMalloc(&h->ptr, sizeof(long long) * (n + 1)));
  CK(cudaMalloc(&h->idx, sizeof(int) * nnz));
  CK(cudaMalloc(&h->val, sizeof(double) * nnz));
  CK(cudaMalloc(&h->dinv, sizeof(double) * n));
  CK(cudaMalloc(&h->bad, sizeof(int)));
  CK(cudaMemcpy(h->ptr, indptr, sizeof(long long) * (n + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->idx, indices, sizeof(int) * nnz, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->val, data, sizeof(double) * nnz, cudaMemcpyHostToDevice));
  CK(cudaMemset(h->bad, 0, sizeof(int)));
  k_csr_diag_inv<<<count_launch(dim3((n + TPB - 1) / TPB)), TPB>>>(n, h->ptr, h->idx, h->val, h->dinv, h->bad);
  int bad = 0;
  CK(cudaMemcpy(&bad, h->bad, sizeof(int), cudaMemcpyDeviceToHost));
  if (bad) {
    cudaFree(h->ptr); cudaFree(h->idx); cudaFree(h->val); cudaFree(h->dinv); cudaFree(h->bad);
    return fail(DC_ERR_ARG, "matrix has a non-positive diagonal entry (not SPD)");
  }
  CK(cudaMallocHost((void **)&h->h_mail, 4 * sizeof(int)));
  CK(cudaEventCreateWithFlags(&h->ev, cudaEventDisableTiming));
  *out = h.release();
  return 0;
}

void dc_csr_destroy(dc_csr *h) {
  if (!h) return;
  cudaDeviceSynchronize();
  cudaFree(h->ptr);
  cudaFree(h->idx);
  cudaFree(h->val);
  cudaFree(h->dinv);
  cudaFree(h->bad);
  cudaFree(h->ws);
  if (h->h_mail) cudaFreeHost(h->h_mail);
  if (h->ev) cudaEventDestroy(h->ev);
  delete h;
}

int dc_csr_solve(dc_csr *h, const double *b, double *x, int k, double rtol, int maxit, dc_stats *stats,
                 void *stream) {
  if (!h || !b || !x || k < 1 || !(rtol > 0.0) || maxit < 1) return fail(DC_ERR_ARG, "bad argument");
  if (k > kMaxRhsBlocks) {
    // columns in chunks of kMaxRhsBlocks (one column per RHS block here)
    dc_stats agg{0, 1, 0, 0, 0.0};
    for (int c0 = 0; c0 < k; c0 += kMaxRhsBlocks) {
      const int kc = k - c0 < kMaxRhsBlocks ? k - c0 : kMaxRhsBlocks;
      dc_stats st{};
      int rc = dc_csr_solve(h, b + (size_t)c0 * h->n, x + (size_t)c0 * h->n, kc, rtol, maxit, &st, stream);
      if (rc) return rc;
      if (st.iterations > agg.iterations) agg.iterations = st.iterations;
    }
    if (stats) *stats = agg;
    return 0;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int n = h->n;
  int gx = (n + TPB - 1) / TPB;
  if (gx > 1024) gx = 1024;
  const size_t nk = (size_t)n * k;
  // r, p, q, z + partials (3 x gx*k) + scalars (rz, rr, bb, alpha, beta, tol2) + flags
  const size_t need = sizeof(double) * (4 * nk + 3 * (size_t)gx * k + 6 * (size_t)k) + sizeof(int) * (k + 4) + 1024;
  if (h->ws_bytes < need) {
    CK(cudaStreamSynchronize(s));
    cudaFree(h->ws);
    h->ws = nullptr;
    h->ws_bytes = 0;
    if (cudaMalloc(&h->ws, need) != cudaSuccess) return fail(DC_ERR_NOMEM, "cannot allocate CSR solve workspace");
    h->ws_bytes = need;
  }
  double *r = (double *)h->ws, *p = r + nk, *q = p + nk, *z = q + nk;
  double *pa = z + nk, *pb = pa + (size_t)gx * k, *pc = pb + (size_t)gx * k;
  double *rz = pc + (size_t)gx * k, *rr = rz + k, *bb = rr + k, *al = bb + k, *be = al + k, *tol2 = be + k;
  int *active = (int *)(tol2 + k), *n_active = active + k, *status = n_active + 1;
  using O = Ops<double, double, 1>;
  CK(cudaMemsetAsync(x, 0, sizeof(double) * nk, s));
  CK(cudaMemcpyAsync(r, b, sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
  fill_int(active, k, 1, s);
  fill_double(tol2, k, rtol * rtol, s);
  CK(cudaMemsetAsync(status, 0, sizeof(int), s));
  const dim3 grid(gx, k);
  O::dot(n, k, r, r, pb, gx, s);
  sum_partials(k, 1, gx, pb, bb, s);
  k_jacobi_dot<<<count_launch(grid), TPB, 0, s>>>(n, h->dinv, r, z, pc);
  CK(cudaMemsetAsync(n_active, 0, sizeof(int), s));
  pcg_beta(k, 1, gx, pc, pb, rz, rr, bb, tol2, active, be, nullptr, n_active, 1, s);
  O::copy_z(n, k, p, z, s);
  int it = 0;
  for (; it < maxit; ++it) {
    k_csr_apply_dot<<<count_launch(grid), TPB, 0, s>>>(n, h->ptr, h->idx, h->val, p, q, pa);
    pcg_alpha(k, 1, gx, pa, rz, active, al, nullptr, status, n_active, s);
    O::update_xr(n, k, x, r, p, q, al, nullptr, pb, gx, nullptr, 0.0, nullptr, nullptr, nullptr, s);
    k_jacobi_dot<<<count_launch(grid), TPB, 0, s>>>(n, h->dinv, r, z, pc);
    pcg_beta(k, 1, gx, pc, pb, rz, rr, bb, tol2, active, be, nullptr, n_active, 0, s);
    O::p_update(n, k, p, z, be, nullptr, s);
    if ((it & 7) == 7 || it + 1 == maxit) {
      CK(cudaMemcpyAsync(h->h_mail, n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(h->h_mail + 1, status, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaEventRecord(h->ev, s));
      CK(cudaEventSynchronize(h->ev));
      if (h->h_mail[1]) return fail(DC_ERR_BREAKDOWN, "CG breakdown: matrix not SPD or non-finite data");
      if (h->h_mail[0] == 0) {
        ++it;
        break;
      }
    }
  }
  CK(cudaMemcpyAsync(h->h_mail, n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->ev, s));
  CK(cudaEventSynchronize(h->ev));
  CK(cudaGetLastError());
  const int status_out = h->h_mail[0] == 0 ? 0 : DC_ERR_NOT_CONVERGED;
  if (stats) {
    stats->iterations = it;
    stats->outer = 1;
    stats->status = status_out;
    stats->n_levels = 0;
    stats->max_rel_res = 0.0;
  }
  if (status_out) return fail(status_out, "CSR CG did not reach the requested tolerance");
  return 0;
}

}  // extern "C"
