// Instantiation of the node kernels for the fp64 solve (T = V = double) and
// the fp64 refinement kernels of the mixed-precision solve: the residual
// b - A x of the fp64 operator with its per-RHS norms, and the solution
// accumulation x64 += d32.
#include "dc_kernels.cuh"

namespace dc {

namespace {

// ---------------------------------------------------------------- refinement
template <int KB>
__global__ void __launch_bounds__(TPB) k_ir_residual(const Coef64 *__restrict__ coef, const double *__restrict__ bvec,
                                                     const double *__restrict__ x, double *__restrict__ r64,
                                                     float *__restrict__ r32, Dims d, int nb,
                                                     const int *__restrict__ active, double *__restrict__ partial,
                                                     int gs) {
  using T = double;
  constexpr int W = Lanes<T, KB>::W;
  sweep_reduce<T, KB, W>(d.N, nb, partial, gs, [&](int b, int n, int q, long long t, T(&acc)[W]) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    const Vec<T, W> ax = stencil_vec<T, KB, W>(coef, x, t, n, i, j, k, d);
    Vec<T, W> rv = ld<T, W>(bvec + t);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      rv.a[e] -= ax.a[e];
      acc[e] += rv.a[e] * rv.a[e];
      if (r32) r32[t + e] = active[b * KB + q * W + e] ? (float)rv.a[e] : 0.0f;
    }
    if (r64) st<T, W>(r64 + t, rv);
  });
}

__global__ void __launch_bounds__(TPB) k_ir_accumulate(long long total4, double *__restrict__ x64,
                                                       const float *__restrict__ d32) {
  // total4 = number of 4-element groups (the blocked arrays are padded to KB >= 1 lanes; tail handled by caller)
  for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < total4; t += (long long)gridDim.x * TPB) {
    const float4 dv = reinterpret_cast<const float4 *>(d32)[t];
    double2 a = reinterpret_cast<double2 *>(x64)[2 * t], b = reinterpret_cast<double2 *>(x64)[2 * t + 1];
    a.x += dv.x;
    a.y += dv.y;
    b.x += dv.z;
    b.y += dv.w;
    reinterpret_cast<double2 *>(x64)[2 * t] = a;
    reinterpret_cast<double2 *>(x64)[2 * t + 1] = b;
  }
}

__global__ void k_ir_accumulate_tail(long long start, long long total, double *__restrict__ x64,
                                     const float *__restrict__ d32) {
  for (long long t = start + (long long)blockIdx.x * TPB + threadIdx.x; t < total; t += (long long)gridDim.x * TPB)
    x64[t] += (double)d32[t];
}

}  // namespace

DC_OPS_INSTANTIATE(double, double)

template <int KB>
void ir_residual(const Level &L, const double *b, const double *x, double *r64, float *r32, int nb,
                 const int *active, double *partial, int gx, cudaStream_t s) {
  k_ir_residual<KB><<<RED_GRID(L.dims.N, k_ir_residual<KB>, (Lanes<double, KB>::LPN)), TPB, 0, s>>>(
      L.d_coef64, b, x, r64, r32, L.dims, nb, active, partial, gx);
}

template <int KB>
void ir_accumulate(long long N, int nb, double *x64, const float *d32, cudaStream_t s) {
  const long long total = N * KB * nb;
  const long long t4 = total / 4;
  if (t4 > 0) k_ir_accumulate<<<count_launch(grid_flat(t4, g_n_sm)), TPB, 0, s>>>(t4, x64, d32);
  if (t4 * 4 < total) k_ir_accumulate_tail<<<count_launch(1), TPB, 0, s>>>(t4 * 4, total, x64, d32);
}

// resident blocks per SM of the fp64 reduction kernels the mixed solve also runs
template <int KB>
int ir_blocks_per_sm() {
  return std::max(resident_blocks((const void *)k_ir_residual<KB>), resident_blocks((const void *)k_dot<double, double, KB>));
}

#define DC_INST_IR(KB)                                                                                       \
  template void ir_residual<KB>(const Level &, const double *, const double *, double *, float *, int,      \
                                const int *, double *, int, cudaStream_t);                                  \
  template void ir_accumulate<KB>(long long, int, double *, const float *, cudaStream_t);                  \
  template int ir_blocks_per_sm<KB>();
DC_INST_IR(1) DC_INST_IR(2) DC_INST_IR(4) DC_INST_IR(8) DC_INST_IR(16) DC_INST_IR(32)
#undef DC_INST_IR

}  // namespace dc
