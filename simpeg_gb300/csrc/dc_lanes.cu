// Lane kernels of the continuous-batching sessions (dc_lanes_* in
// include/dcgpu.h): right-hand sides loaded into, and solutions fetched from,
// chosen lanes of a running mixed-precision solve's RHS-blocked double-float
// state, while the other lanes keep iterating.  Element (node n, lane j) of
// the blocked layout is ((j / KB) * N + n) * KB + j % KB.
#include "dc_dfbits.h"
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

__device__ __forceinline__ long long lane_elem(int lane, long long node, long long N, int KB) {
  return ((long long)(lane / KB) * N + node) * KB + lane % KB;
}

// fp64 instructions only where the bit routines do not cover the value, in calls of their own
__device__ __noinline__ double sum_slow(float h, float l) { return (double)h + (double)l; }
__device__ __noinline__ void split_slow(double v, float &h, float &l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

// b (column-major (N, n)) -> lanes[i]: double-float pair of b, the fp32 first residual r = b, x = 0.
__global__ void k_lanes_load(const double *__restrict__ b, int n, const int *__restrict__ lanes, long long N, int KB,
                             float *__restrict__ bh, float *__restrict__ bl, float *__restrict__ r32,
                             float *__restrict__ xh, float *__restrict__ xl) {
  const long long total = (long long)n * N;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / N);
    const long long node = t - (long long)i * N;
    const long long e = lane_elem(lanes[i], node, N, KB);
    float h, l;
    if (__builtin_expect(!split_df_bits(b[t], h, l), 0)) split_slow(b[t], h, l);
    bh[e] = h;
    bl[e] = l;
    r32[e] = h;
    xh[e] = 0.f;
    xl[e] = 0.f;
  }
}

// |b_i|^2 of every loaded column (one block per column, fixed-order reduction) into bb and rr of its lane.
__global__ void k_lanes_norm2(const double *__restrict__ b, long long N, const int *__restrict__ lanes,
                              double *__restrict__ bb, double *__restrict__ rr) {
  __shared__ double red[TPB / 32];
  const int i = blockIdx.x;
  const double *bi = b + (long long)i * N;
  double s = 0.0;
  for (long long n = threadIdx.x; n < N; n += blockDim.x) s += bi[n] * bi[n];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < TPB / 32; ++w) v += red[w];
    bb[lanes[i]] = v;
    rr[lanes[i]] = v;
  }
}

// x (column-major (N, n)) <- hi + lo of lanes[i].
__global__ void k_lanes_fetch(const float *__restrict__ xh, const float *__restrict__ xl, int n,
                              const int *__restrict__ lanes, long long N, int KB, double *__restrict__ x) {
  const long long total = (long long)n * N;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / N);
    const long long node = t - (long long)i * N;
    const long long e = lane_elem(lanes[i], node, N, KB);
    const float fh = xh[e], fl = xl[e];
    double v;
    if (__builtin_expect(!df_sum_bits(fh, fl, v), 0)) v = sum_slow(fh, fl);
    x[t] = v;
  }
}

}  // namespace

void lanes_load(const double *b, int n, const int *lanes, long long N, int KB, float *bh, float *bl, float *r32,
                float *xh, float *xl, double *bb, double *rr, cudaStream_t s) {
  k_lanes_load<<<count_launch(grid_flat((long long)n * N, g_n_sm)), TPB, 0, s>>>(b, n, lanes, N, KB, bh, bl, r32,
                                                                                 xh, xl);
  k_lanes_norm2<<<count_launch(dim3(n)), TPB, 0, s>>>(b, N, lanes, bb, rr);
}

void lanes_fetch(const float *xh, const float *xl, int n, const int *lanes, long long N, int KB, double *x,
                 cudaStream_t s) {
  k_lanes_fetch<<<count_launch(grid_flat((long long)n * N, g_n_sm)), TPB, 0, s>>>(xh, xl, n, lanes, N, KB, x);
}

}  // namespace dc
