// Stencil, multigrid-transfer, PCG-vector and reduction kernels of the nodal
// DC engine.  Every kernel here is bandwidth-bound except the fp64 stencil,
// which on this part is bounded by fp64 issue rate (see the design notes).
//
// Thread mapping of every "node" kernel: a thread owns W consecutive RHS lanes
// (16 bytes) of one node, KB/W threads share a node, and a 1D grid sweeps the
// flat (RHS block, node) index with the RHS block slowest.  Lane l of node n
// in RHS block b is element (b*N + n)*KB + l, so a warp's loads are contiguous.
#include "dc_internal.h"

#include <cstdio>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <unordered_map>

namespace dc {

namespace {

constexpr int TPB = 256;

// floor(n / d) for 0 <= n < 2^31 with m = div_magic(d).
__device__ __forceinline__ int fast_div(int n, int d, unsigned m) {
  if (d == 1) return n;
  unsigned q = __umulhi((unsigned)n, m);
  q -= (q * (unsigned)d > (unsigned)n) ? 1u : 0u;
  return (int)q;
}

__device__ __forceinline__ void node_ijk(int n, const Dims &d, int &i, int &j, int &k) {
  const int nxy = d.Nx * d.Ny;
  k = fast_div(n, nxy, d.mxy);
  const int r = n - k * nxy;
  j = fast_div(r, d.Nx, d.mx);
  i = r - j * d.Nx;
}

template <typename C> struct CoefT;
template <> struct CoefT<double> { using type = Coef64; };
template <> struct CoefT<float> { using type = Coef32; };

// Vector width per thread: 16-byte accesses (4 fp32 / 2 fp64 RHS lanes of one node).
template <typename T, int KB> struct VWidth {
  static constexpr int v = (sizeof(T) == 4) ? (KB >= 4 ? 4 : KB) : (KB >= 2 ? 2 : 1);
};

template <typename T, int W> struct alignas(sizeof(T) * W) Vec {
  T a[W];
};

template <typename T, int W>
__device__ __forceinline__ Vec<T, W> ldv(const T *p) {
  return *reinterpret_cast<const Vec<T, W> *>(p);
}
template <typename T, int W>
__device__ __forceinline__ void stv(T *p, const Vec<T, W> &v) {
  *reinterpret_cast<Vec<T, W> *>(p) = v;
}

// Per-thread geometry of the "node x lane-group" mapping.  LPN threads share
// one node (each owning W consecutive RHS lanes of one RHS block).  Kernels
// sweep the RHS blocks one after the other (RHS block = slowest index of the
// flat work index), so the L2 working set of the stencil's z-neighbour planes
// is that of one RHS block at a time.
template <typename T, int KB> struct Map {
  static constexpr int W = VWidth<T, KB>::v;
  static constexpr int LPN = KB / W;  // threads per node
};


template <typename T, int KB>
__device__ __forceinline__ const typename CoefT<T>::type *coef_of(const void *c) {
  return reinterpret_cast<const typename CoefT<T>::type *>(c);
}

// (A x) for the W lanes at element t of node n = (i, j, k).
template <typename T, int KB, int W>
__device__ __forceinline__ Vec<T, W> stencil_vec(const typename CoefT<T>::type *__restrict__ coef,
                                                  const T *__restrict__ x, long long t, int n, int i, int j, int k,
                                                  const Dims &d) {
  const auto c = coef[n];
  Vec<T, W> acc = ldv<T, W>(x + t);
#pragma unroll
  for (int e = 0; e < W; ++e) acc.a[e] *= c.d;
  const long long sx = KB, sy = (long long)d.Nx * KB, sz = (long long)d.Nx * d.Ny * KB;
  auto sub = [&](T w, long long off) {
    const Vec<T, W> v = ldv<T, W>(x + t + off);
#pragma unroll
    for (int e = 0; e < W; ++e) acc.a[e] -= w * v.a[e];
  };
  if (i + 1 < d.Nx) sub(c.cx, sx);
  if (i > 0) sub(coef[n - 1].cx, -sx);
  if (j + 1 < d.Ny) sub(c.cy, sy);
  if (j > 0) sub(coef[n - d.Nx].cy, -sy);
  if (k + 1 < d.Nz) sub(c.cz, sz);
  if (k > 0) sub(coef[n - d.Nx * d.Ny].cz, -sz);
  return acc;
}

// Sweep over (RHS block b, node n, lane group q) with b slowest.  Defines W,
// LPN, q and, per iteration, ng (flat node index over all RHS blocks), b, n and
// t (offset of the thread's W lanes).
#define SWEEP(NN, MAGIC, NB)                                                                   \
  constexpr int W = Map<T, KB>::W, LPN = Map<T, KB>::LPN;                                      \
  const int q = threadIdx.x % LPN;                                                             \
  const long long total_ = (long long)(NN) * (NB) * LPN;                                       \
  for (long long g = (long long)blockIdx.x * TPB + threadIdx.x; g < total_; g += (long long)gridDim.x * TPB)

#define SWEEP_INDEX(NN, MAGIC)                        \
  const int ng = (int)(g / LPN);                      \
  const int b = fast_div(ng, (int)(NN), (MAGIC));     \
  const int n = ng - b * (int)(NN);                   \
  const long long t = (long long)ng * KB + q * W;     \
  (void)b;                                            \
  (void)n;

// Reductions (per-RHS dot products) are bitwise reproducible: every thread
// sums its own elements in sweep order, threads of one lane group are
// combined by warp shuffles, and the warps' sums in warp order -- no
// floating-point atomics, so a solve repeated on the same data (or recorded in
// a CUDA graph) takes the same iterations and returns the same bits.
// Block partials land in partial[(b * gridDim.x + blockIdx.x) * KB + lane].
template <typename T, int KB>
__device__ __forceinline__ void block_reduce(T (&acc)[Map<T, KB>::W], T *red, int b, double *partial) {
  constexpr int W = Map<T, KB>::W, LPN = Map<T, KB>::LPN;
#pragma unroll
  for (int o = 16; o >= LPN; o >>= 1)
#pragma unroll
    for (int e = 0; e < W; ++e) acc[e] += __shfl_xor_sync(0xffffffffu, acc[e], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane < LPN)
#pragma unroll
    for (int e = 0; e < W; ++e) red[warp * KB + lane * W + e] = acc[e];
  __syncthreads();
  if (threadIdx.x < KB) {
    T v = (T)0;
#pragma unroll
    for (int w = 0; w < TPB / 32; ++w) v += red[w * KB + threadIdx.x];
    partial[((long long)b * gridDim.x + blockIdx.x) * KB + threadIdx.x] = (double)v;
  }
  __syncthreads();
}

// Sweep of a reducing kernel: the RHS blocks one after the other (the whole
// grid on one RHS block at a time, as in the flat sweep), each closed by the
// block reduction of that RHS block's per-thread sums.
// body(b, n, q, t, acc): RHS block, node, lane group, element offset, sums.
template <typename T, int KB, typename Body>
__device__ __forceinline__ void sweep_reduce(int N, int nb, double *partial, Body body) {
  constexpr int W = Map<T, KB>::W, LPN = Map<T, KB>::LPN;
  __shared__ T red[(TPB / 32) * KB];
  const int q = threadIdx.x % LPN;
  const long long per = (long long)N * LPN;
  for (int b = 0; b < nb; ++b) {
    T acc[W];
#pragma unroll
    for (int e = 0; e < W; ++e) acc[e] = (T)0;
    const long long base = (long long)b * N;
    for (long long g = (long long)blockIdx.x * TPB + threadIdx.x; g < per; g += (long long)gridDim.x * TPB) {
      const int n = (int)(g / LPN);
      body(b, n, q, (base + n) * KB + q * W, acc);
    }
    block_reduce<T, KB>(acc, red, b, partial);
  }
}

// The same body over the flat (RHS block, node, lane group) sweep, no reduction.
template <typename T, int KB, typename Body>
__device__ __forceinline__ void sweep_flat(int N, unsigned mn, int nb, Body body) {
  constexpr int W = Map<T, KB>::W, LPN = Map<T, KB>::LPN;
  const int q = threadIdx.x % LPN;
  const long long total = (long long)N * nb * LPN;
  T acc[W];
  for (long long g = (long long)blockIdx.x * TPB + threadIdx.x; g < total; g += (long long)gridDim.x * TPB) {
    const int ng = (int)(g / LPN);
    const int b = fast_div(ng, N, mn);
    body(b, ng - b * N, q, (long long)ng * KB + q * W, acc);
  }
}

// ---------------------------------------------------------------- stencil ops
template <typename T, int KB, bool DOT>
__global__ void __launch_bounds__(TPB) k_apply(const void *__restrict__ cf, const T *__restrict__ x,
                                               T *__restrict__ y, Dims d, int nb, double *__restrict__ partial) {
  constexpr int W = Map<T, KB>::W;
  const auto *coef = coef_of<T, KB>(cf);
  auto body = [&](int b, int n, int q, long long t, T(&acc)[W]) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    const Vec<T, W> v = stencil_vec<T, KB, W>(coef, x, t, n, i, j, k, d);
    stv<T, W>(y + t, v);
    if (DOT) {
      const Vec<T, W> xv = ldv<T, W>(x + t);
#pragma unroll
      for (int e = 0; e < W; ++e) acc[e] += v.a[e] * xv.a[e];
    }
  };
  if (DOT)
    sweep_reduce<T, KB>(d.N, nb, partial, body);
  else
    sweep_flat<T, KB>(d.N, d.mn, nb, body);
}

template <typename T, int KB>
__global__ void __launch_bounds__(TPB) k_residual(const void *__restrict__ cf, const T *__restrict__ r,
                                                  const T *__restrict__ z, T *__restrict__ res, Dims d, int nb) {
  const auto *coef = coef_of<T, KB>(cf);
  SWEEP(d.N, d.mn, nb) {
    SWEEP_INDEX(d.N, d.mn)
    int i, j, k;
    node_ijk(n, d, i, j, k);
    const Vec<T, W> az = stencil_vec<T, KB, W>(coef, z, t, n, i, j, k, d);
    Vec<T, W> rv = ldv<T, W>(r + t);
#pragma unroll
    for (int e = 0; e < W; ++e) rv.a[e] -= az.a[e];
    stv<T, W>(res + t, rv);
  }
}

// First Chebyshev step from z = 0: z = c0 * D^-1 r.
template <typename T, int KB>
__global__ void __launch_bounds__(TPB) k_cheb_first(const T *__restrict__ invd, const T *__restrict__ r,
                                                    T *__restrict__ z, Dims d, int nb, T c0) {
  SWEEP(d.N, d.mn, nb) {
    SWEEP_INDEX(d.N, d.mn)
    const T s = c0 * invd[n];
    Vec<T, W> v = ldv<T, W>(r + t);
#pragma unroll
    for (int e = 0; e < W; ++e) v.a[e] *= s;
    stv<T, W>(z + t, v);
  }
}

// Chebyshev step in three-term form (x_{k+1} = x_k + c1 (x_k - x_{k-1}) + c2 D^-1 (r - A x_k)):
//   PREV = 0: no momentum term (first step from a nonzero start, c1 = 0)
//   PREV = 1: x_{k-1} read from zout (overwritten in place with x_{k+1})
//   PREV = 2: x_{k-1} = 0 (second step of a zero-start sequence)
// Four streams per RHS lane (x_k, r, x_{k-1} read; x_{k+1} write) instead of the
// five of the d-vector form.  With DOT, also per-block partials of r . x_{k+1}.
template <typename T, int KB, bool DOT, int PREV>
__global__ void __launch_bounds__(TPB) k_cheb_step(const void *__restrict__ cf, const T *__restrict__ invd,
                                                   const T *__restrict__ r, const T *__restrict__ zin,
                                                   T *zout, Dims d, int nb, T c1, T c2,
                                                   double *__restrict__ partial) {
  constexpr int W = Map<T, KB>::W;
  const auto *coef = coef_of<T, KB>(cf);
  auto body = [&](int b, int n, int q, long long t, T(&acc)[W]) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    const Vec<T, W> az = stencil_vec<T, KB, W>(coef, zin, t, n, i, j, k, d);
    const Vec<T, W> rv = ldv<T, W>(r + t);
    const Vec<T, W> zc = ldv<T, W>(zin + t);
    Vec<T, W> zo;
    if (PREV == 1) zo = ldv<T, W>(zout + t);
    const T s = c2 * invd[n];
#pragma unroll
    for (int e = 0; e < W; ++e) {
      T mom = (T)0;
      if (PREV == 1) mom = c1 * (zc.a[e] - zo.a[e]);
      if (PREV == 2) mom = c1 * zc.a[e];
      zo.a[e] = zc.a[e] + mom + s * (rv.a[e] - az.a[e]);
      if (DOT) acc[e] += rv.a[e] * zo.a[e];
    }
    stv<T, W>(zout + t, zo);
  };
  if (DOT)
    sweep_reduce<T, KB>(d.N, nb, partial, body);
  else
    sweep_flat<T, KB>(d.N, d.mn, nb, body);
}

// ---------------------------------------------------------------- transfers
struct XferTab {
  const int *fi;        // coarse node -> fine node, per axis at roff[a]
  const void *wl, *wr;  // T weights of fine fi-1 / fi+1
  const int *pl;        // fine node -> left coarse node, per axis at poff[a]
  const void *pw;       // T weight on pl
  long long roff[3], poff[3];
};

template <typename T, int KB>
__global__ void __launch_bounds__(TPB) k_restrict(const T *__restrict__ res, T *__restrict__ rc, Dims f, Dims c,
                                                  int nb, XferTab tb) {
  const T *wl = (const T *)tb.wl, *wr = (const T *)tb.wr;
  SWEEP(c.N, c.mn, nb) {
    SWEEP_INDEX(c.N, c.mn)
    int I, J, K;
    node_ijk(n, c, I, J, K);
    const int fx = tb.fi[tb.roff[0] + I], fy = tb.fi[tb.roff[1] + J], fz = tb.fi[tb.roff[2] + K];
    const T wx[3] = {wl[tb.roff[0] + I], (T)1, wr[tb.roff[0] + I]};
    const T wy[3] = {wl[tb.roff[1] + J], (T)1, wr[tb.roff[1] + J]};
    const T wz[3] = {wl[tb.roff[2] + K], (T)1, wr[tb.roff[2] + K]};
    const long long fb = (long long)b * f.N * KB + q * W;
    Vec<T, W> acc;
#pragma unroll
    for (int e = 0; e < W; ++e) acc.a[e] = 0;
#pragma unroll
    for (int cz = 0; cz < 3; ++cz) {
      if (wz[cz] == (T)0) continue;
#pragma unroll
      for (int cy = 0; cy < 3; ++cy) {
        if (wy[cy] == (T)0) continue;
        const T wyz = wy[cy] * wz[cz];
        const long long row = ((long long)(fz + cz - 1) * f.Ny + (fy + cy - 1)) * f.Nx;
#pragma unroll
        for (int cx = 0; cx < 3; ++cx) {
          if (wx[cx] == (T)0) continue;
          const T w = wx[cx] * wyz;
          const Vec<T, W> v = ldv<T, W>(res + fb + (row + fx + cx - 1) * KB);
#pragma unroll
          for (int e = 0; e < W; ++e) acc.a[e] += w * v.a[e];
        }
      }
    }
    stv<T, W>(rc + t, acc);
  }
}

template <typename T, int KB>
__global__ void __launch_bounds__(TPB) k_prolong_add(const T *__restrict__ zc, T *__restrict__ z, Dims f, Dims c,
                                                     int nb, XferTab tb) {
  const T *pw = (const T *)tb.pw;
  SWEEP(f.N, f.mn, nb) {
    SWEEP_INDEX(f.N, f.mn)
    int i, j, k;
    node_ijk(n, f, i, j, k);
    const int I = tb.pl[tb.poff[0] + i], J = tb.pl[tb.poff[1] + j], K = tb.pl[tb.poff[2] + k];
    const T ax = pw[tb.poff[0] + i], ay = pw[tb.poff[1] + j], az = pw[tb.poff[2] + k];
    const T wx[2] = {ax, (T)1 - ax}, wy[2] = {ay, (T)1 - ay}, wz[2] = {az, (T)1 - az};
    const long long cb = (long long)b * c.N * KB + q * W;
    Vec<T, W> acc = ldv<T, W>(z + t);
#pragma unroll
    for (int bz = 0; bz < 2; ++bz) {
      if (wz[bz] == (T)0) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        if (wy[a] == (T)0) continue;
        const T wyz = wy[a] * wz[bz];
        const long long row = ((long long)(K + bz) * c.Ny + (J + a)) * c.Nx;
#pragma unroll
        for (int e2 = 0; e2 < 2; ++e2) {
          if (wx[e2] == (T)0) continue;
          const T w = wx[e2] * wyz;
          const Vec<T, W> v = ldv<T, W>(zc + cb + (row + I + e2) * KB);
#pragma unroll
          for (int e = 0; e < W; ++e) acc.a[e] += w * v.a[e];
        }
      }
    }
    stv<T, W>(z + t, acc);
  }
}

// z_c = Ainv r_c on the coarsest level (dense, row-major Ainv[nc][nc]).
template <typename T, int KB>
__global__ void __launch_bounds__(TPB) k_coarse_solve(const T *__restrict__ Ainv, Dims c, int nb,
                                                      const T *__restrict__ rc, T *__restrict__ zc) {
  const int nc = (int)c.N;
  SWEEP(c.N, c.mn, nb) {
    SWEEP_INDEX(c.N, c.mn)
    const T *row = Ainv + (long long)n * nc;
    const long long base = (long long)b * nc * KB + q * W;
    Vec<T, W> acc;
#pragma unroll
    for (int e = 0; e < W; ++e) acc.a[e] = 0;
    for (int m = 0; m < nc; ++m) {
      const T w = row[m];
      const Vec<T, W> v = ldv<T, W>(rc + base + (long long)m * KB);
#pragma unroll
      for (int e = 0; e < W; ++e) acc.a[e] += w * v.a[e];
    }
    stv<T, W>(zc + t, acc);
  }
}

// ---------------------------------------------------------------- PCG vectors
// x += a p ; r -= a q ; partial |r|^2 (a per RHS).  With SMOOTH, also the first
// Chebyshev step of the fine level on the new residual: z = d = c0 D^-1 r.
template <typename T, int KB, bool SMOOTH>
__global__ void __launch_bounds__(TPB) k_update_xr(Dims d, int nb, T *__restrict__ x, T *__restrict__ r,
                                                   const T *__restrict__ p, const T *__restrict__ qv,
                                                   const double *__restrict__ alpha, double *__restrict__ partial,
                                                   const T *__restrict__ invd, T *__restrict__ z, T c0) {
  constexpr int W = Map<T, KB>::W;
  sweep_reduce<T, KB>(d.N, nb, partial, [&](int b, int n, int q, long long t, T(&acc)[W]) {
    Vec<T, W> xv = ldv<T, W>(x + t), rv = ldv<T, W>(r + t);
    const Vec<T, W> pv = ldv<T, W>(p + t), qq = ldv<T, W>(qv + t);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const T a = (T)alpha[b * KB + q * W + e];
      xv.a[e] += a * pv.a[e];
      rv.a[e] -= a * qq.a[e];
      acc[e] += rv.a[e] * rv.a[e];
    }
    stv<T, W>(x + t, xv);
    stv<T, W>(r + t, rv);
    if (SMOOTH) {
      const T s = c0 * invd[n];
#pragma unroll
      for (int e = 0; e < W; ++e) rv.a[e] *= s;
      stv<T, W>(z + t, rv);
    }
  });
}

template <typename T, int KB>
__global__ void __launch_bounds__(TPB) k_dot(Dims d, int nb, const T *__restrict__ a, const T *__restrict__ bb,
                                             double *__restrict__ partial) {
  constexpr int W = Map<T, KB>::W;
  sweep_reduce<T, KB>(d.N, nb, partial, [&](int, int, int, long long t, T(&acc)[W]) {
    const Vec<T, W> av = ldv<T, W>(a + t), bv = ldv<T, W>(bb + t);
#pragma unroll
    for (int e = 0; e < W; ++e) acc[e] += av.a[e] * bv.a[e];
  });
}

// p = z + beta p
template <typename T, int KB>
__global__ void __launch_bounds__(TPB) k_p_update(Dims d, int nb, T *__restrict__ p, const T *__restrict__ z,
                                                  const double *__restrict__ beta) {
  SWEEP(d.N, d.mn, nb) {
    SWEEP_INDEX(d.N, d.mn)
    Vec<T, W> pv = ldv<T, W>(p + t);
    const Vec<T, W> zv = ldv<T, W>(z + t);
#pragma unroll
    for (int e = 0; e < W; ++e) pv.a[e] = zv.a[e] + (T)beta[b * KB + q * W + e] * pv.a[e];
    stv<T, W>(p + t, pv);
  }
}

// ---------------------------------------------------------------- refinement
template <int KB>
__global__ void __launch_bounds__(TPB) k_ir_residual(const Coef64 *__restrict__ coef, const double *__restrict__ bvec,
                                                     const double *__restrict__ x, double *__restrict__ r64,
                                                     float *__restrict__ r32, Dims d, int nb,
                                                     const int *__restrict__ active, double *__restrict__ partial) {
  using T = double;
  constexpr int W = Map<T, KB>::W;
  sweep_reduce<T, KB>(d.N, nb, partial, [&](int b, int n, int q, long long t, T(&acc)[W]) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    const Vec<T, W> ax = stencil_vec<T, KB, W>(coef, x, t, n, i, j, k, d);
    Vec<T, W> rv = ldv<T, W>(bvec + t);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      rv.a[e] -= ax.a[e];
      acc[e] += rv.a[e] * rv.a[e];
      r32[t + e] = active[b * KB + q * W + e] ? (float)rv.a[e] : 0.0f;
    }
    stv<T, W>(r64 + t, rv);
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

__global__ void k_fill_int(int *__restrict__ a, int n, int v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

__global__ void k_ir_accumulate_tail(long long start, long long total, double *__restrict__ x64,
                                     const float *__restrict__ d32) {
  for (long long t = start + (long long)blockIdx.x * TPB + threadIdx.x; t < total; t += (long long)gridDim.x * TPB)
    x64[t] += (double)d32[t];
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

__global__ void __launch_bounds__(SCAL_T) k_pcg_alpha(int K, int KB, int gx, const double *__restrict__ part_pq,
                                                      const double *__restrict__ rz, const int *__restrict__ active,
                                                      double *__restrict__ alpha, int *__restrict__ status,
                                                      int *__restrict__ n_active) {
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
  }
}

// rz_new = r.z ; rr = |r|^2 ; active &= rr > tol2[r]*bb ; beta = rz_new/rz_old ; counts active
// (n_active must be zero on entry).
__global__ void __launch_bounds__(SCAL_T) k_pcg_beta(int K, int KB, int gx, const double *__restrict__ part_rz,
                                                     const double *__restrict__ part_rr, double *__restrict__ rz,
                                                     double *__restrict__ rr_out, const double *__restrict__ bb,
                                                     const double *__restrict__ tol2, int *__restrict__ active,
                                                     double *__restrict__ beta, int *__restrict__ n_active,
                                                     int first) {
  const int r = blockIdx.x;
  const double rzn = block_sum_partial(part_rz, gx, KB, r);
  const double rr = block_sum_partial(part_rr, gx, KB, r);
  if (threadIdx.x == 0) {
    rr_out[r] = rr;
    int act = active[r];
    if (act && !(rr > tol2[r] * bb[r])) act = 0;
    if (act && !isfinite(rr)) act = 0;
    double bt = 0.0;
    if (act && !first) bt = rz[r] != 0.0 ? rzn / rz[r] : 0.0;
    if (act) rz[r] = rzn;
    beta[r] = first ? 0.0 : bt;
    active[r] = act;
    if (act) atomicAdd(n_active, 1);
  }
}

// per-RHS sums of partials into out (used for |b|^2 and the outer residual norms)
__global__ void __launch_bounds__(SCAL_T) k_sum_partials(int K, int KB, int gx, const double *__restrict__ part,
                                                         double *__restrict__ out) {
  const double v = block_sum_partial(part, gx, KB, blockIdx.x);
  if (threadIdx.x == 0) out[blockIdx.x] = v;
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

__global__ void k_convert_d2f(const double *__restrict__ a, long long n, float *__restrict__ o) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    o[i] = (float)a[i];
}

// ---------------------------------------------------------------- layout conversion
template <typename T>
__global__ void k_pack(const double *__restrict__ src, long long N, int K, int KB, T *__restrict__ dst,
                       long long total) {
  // dst element t -> (b, n, l); rhs r = b*KB + l; src[r*N + n]
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(t % KB);
    const long long bn = t / KB;
    const long long n = bn % N;
    const int r = (int)(bn / N) * KB + l;
    dst[t] = (r < K) ? (T)src[(long long)r * N + n] : (T)0;
  }
}

template <typename T>
__global__ void k_unpack(const T *__restrict__ src, long long N, int K, int KB, double *__restrict__ dst) {
  const long long total = N * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / N);
    const long long n = e - (long long)r * N;
    dst[e] = (double)src[((long long)(r / KB) * N + n) * KB + (r % KB)];
  }
}

inline int grid_nodes(long long nodes, int LPN, int nb, int n_sm, int per_sm = 8) {
  long long g = (nodes * (nb > 0 ? nb : 1) * LPN + TPB - 1) / TPB;
  const long long cap = (long long)n_sm * per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

inline int grid_flat(long long total, int n_sm) {
  long long g = (total + TPB - 1) / TPB;
  long long cap = (long long)n_sm * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

inline Dims flat_dims(long long N) {
  Dims d{};
  d.Nx = 1;
  d.Ny = 1;
  d.Nz = (int)N;
  d.N = N;
  d.mn = div_magic((unsigned)N);
  return d;
}

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

}  // namespace

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

// ------------------------------------------------------------------ launchers
template <typename T>
static const void *coef_ptr(const Level &L) {
  return std::is_same<T, double>::value ? (const void *)L.d_coef64 : (const void *)L.d_coef32;
}
template <typename T>
static const T *invd_ptr(const Level &L) {
  return reinterpret_cast<const T *>(std::is_same<T, double>::value ? (const void *)L.d_invd64
                                                                    : (const void *)L.d_invd32);
}

#define GRID_K(NODES, KERNEL) \
  count_launch(dim3(grid_nodes((NODES), Map<T, KB>::LPN, nb, g_n_sm, resident_blocks((const void *)(KERNEL)))))

template <typename T, int KB>
void Ops<T, KB>::apply(const Level &L, const T *x, T *y, int nb, double *partial, int gx, cudaStream_t s) {
  if (partial)
    k_apply<T, KB, true><<<count_launch(dim3(gx)), TPB, 0, s>>>(coef_ptr<T>(L), x, y, L.dims, nb, partial);
  else
    k_apply<T, KB, false><<<GRID_K(L.dims.N, (k_apply<T, KB, false>)), TPB, 0, s>>>(coef_ptr<T>(L), x, y, L.dims, nb, nullptr);
}

template <typename T, int KB>
int Ops<T, KB>::red_blocks_per_sm() {
  int m = resident_blocks((const void *)k_apply<T, KB, true>);
  m = std::min(m, resident_blocks((const void *)k_cheb_step<T, KB, true, 0>));
  m = std::min(m, resident_blocks((const void *)k_cheb_step<T, KB, true, 1>));
  m = std::min(m, resident_blocks((const void *)k_cheb_step<T, KB, true, 2>));
  m = std::min(m, resident_blocks((const void *)k_update_xr<T, KB, true>));
  m = std::min(m, resident_blocks((const void *)k_update_xr<T, KB, false>));
  m = std::min(m, resident_blocks((const void *)k_dot<T, KB>));
  if (std::is_same<T, double>::value) m = std::min(m, resident_blocks((const void *)k_ir_residual<KB>));
  return m;
}

template <typename T, int KB>
void Ops<T, KB>::residual(const Level &L, const T *r, const T *z, T *res, int nb, cudaStream_t s) {
  k_residual<T, KB><<<GRID_K(L.dims.N, (k_residual<T, KB>)), TPB, 0, s>>>(coef_ptr<T>(L), r, z, res, L.dims, nb);
}

template <typename T, int KB>
void Ops<T, KB>::cheb_first(const Level &L, const T *r, T *z, int nb, double c0, cudaStream_t s) {
  k_cheb_first<T, KB><<<GRID_K(L.dims.N, (k_cheb_first<T, KB>)), TPB, 0, s>>>(invd_ptr<T>(L), r, z, L.dims, nb, (T)c0);
}

template <typename T, int KB>
template <bool DOT, int PREV>
void Ops<T, KB>::cheb_launch(const Level &L, const T *r, const T *zin, T *zout, int nb, double c1, double c2,
                             double *partial, int gx, cudaStream_t s) {
  const dim3 g = DOT ? count_launch(dim3(gx)) : GRID_K(L.dims.N, (k_cheb_step<T, KB, DOT, PREV>));
  k_cheb_step<T, KB, DOT, PREV><<<g, TPB, 0, s>>>(coef_ptr<T>(L), invd_ptr<T>(L), r, zin, zout, L.dims, nb, (T)c1,
                                                  (T)c2, partial);
}

template <typename T, int KB>
void Ops<T, KB>::cheb_step(const Level &L, const T *r, const T *zin, T *zout, int prev, int nb, double c1, double c2,
                           double *partial, int gx, cudaStream_t s) {
  if (partial) {
    if (prev == 1) cheb_launch<true, 1>(L, r, zin, zout, nb, c1, c2, partial, gx, s);
    else if (prev == 2) cheb_launch<true, 2>(L, r, zin, zout, nb, c1, c2, partial, gx, s);
    else cheb_launch<true, 0>(L, r, zin, zout, nb, c1, c2, partial, gx, s);
  } else {
    if (prev == 1) cheb_launch<false, 1>(L, r, zin, zout, nb, c1, c2, nullptr, gx, s);
    else if (prev == 2) cheb_launch<false, 2>(L, r, zin, zout, nb, c1, c2, nullptr, gx, s);
    else cheb_launch<false, 0>(L, r, zin, zout, nb, c1, c2, nullptr, gx, s);
  }
}

template <typename T>
static XferTab make_tab(const Level &f) {
  XferTab tb;
  const bool dbl = std::is_same<T, double>::value;
  tb.fi = f.d_r_fi;
  tb.wl = dbl ? (const void *)f.d_r_wl : (const void *)f.d_r_wl32;
  tb.wr = dbl ? (const void *)f.d_r_wr : (const void *)f.d_r_wr32;
  tb.pl = f.d_pl_idx;
  tb.pw = dbl ? (const void *)f.d_pl_w : (const void *)f.d_pl_w32;
  for (int a = 0; a < 3; ++a) {
    tb.roff[a] = f.r_off[a];
    tb.poff[a] = f.pl_off[a];
  }
  return tb;
}

template <typename T, int KB>
void Ops<T, KB>::restrict_(const Level &f, const Level &c, const T *res, T *rc, int nb, cudaStream_t s) {
  k_restrict<T, KB><<<GRID_K(c.dims.N, (k_restrict<T, KB>)), TPB, 0, s>>>(res, rc, f.dims, c.dims, nb, make_tab<T>(f));
}

template <typename T, int KB>
void Ops<T, KB>::prolong_add(const Level &f, const Level &c, const T *zc, T *z, int nb, cudaStream_t s) {
  k_prolong_add<T, KB><<<GRID_K(f.dims.N, (k_prolong_add<T, KB>)), TPB, 0, s>>>(zc, z, f.dims, c.dims, nb, make_tab<T>(f));
}

template <typename T, int KB>
void Ops<T, KB>::coarse_solve(const T *Ainv, const Level &c, const T *rc, T *zc, int nb, cudaStream_t s) {
  k_coarse_solve<T, KB><<<GRID_K(c.dims.N, (k_coarse_solve<T, KB>)), TPB, 0, s>>>(Ainv, c.dims, nb, rc, zc);
}

template <typename T, int KB>
void Ops<T, KB>::update_xr(long long N, int nb, T *x, T *r, const T *p, const T *q, const double *alpha,
                           double *partial, int gx, const Level *smooth, double c0, T *z, cudaStream_t s) {
  const Dims dd = flat_dims(N);
  if (smooth)
    k_update_xr<T, KB, true><<<count_launch(dim3(gx)), TPB, 0, s>>>(dd, nb, x, r, p, q, alpha, partial,
                                                                     invd_ptr<T>(*smooth), z, (T)c0);
  else
    k_update_xr<T, KB, false><<<count_launch(dim3(gx)), TPB, 0, s>>>(dd, nb, x, r, p, q, alpha, partial, nullptr,
                                                                      nullptr, (T)0);
}

template <typename T, int KB>
void Ops<T, KB>::dot(long long N, int nb, const T *a, const T *b, double *partial, int gx, cudaStream_t s) {
  k_dot<T, KB><<<count_launch(dim3(gx)), TPB, 0, s>>>(flat_dims(N), nb, a, b, partial);
}

template <typename T, int KB>
void Ops<T, KB>::p_update(long long N, int nb, T *p, const T *z, const double *beta, cudaStream_t s) {
  k_p_update<T, KB><<<GRID_K(N, (k_p_update<T, KB>)), TPB, 0, s>>>(flat_dims(N), nb, p, z, beta);
}

template <typename T, int KB>
void Ops<T, KB>::copy(long long N, int nb, T *dst, const T *src, cudaStream_t s) {
  cudaMemcpyAsync(dst, src, sizeof(T) * N * KB * nb, cudaMemcpyDeviceToDevice, s);
}

template <int KB>
void ir_residual(const Level &L, const double *b, const double *x, double *r64, float *r32, int nb,
                 const int *active, double *partial, int gx, cudaStream_t s) {
  k_ir_residual<KB><<<count_launch(dim3(gx)), TPB, 0, s>>>(L.d_coef64, b, x, r64, r32, L.dims, nb, active, partial);
}

template <int KB>
void ir_accumulate(long long N, int nb, double *x64, const float *d32, cudaStream_t s) {
  const long long total = N * KB * nb;
  const long long t4 = total / 4;
  if (t4 > 0) k_ir_accumulate<<<count_launch(grid_flat(t4, g_n_sm)), TPB, 0, s>>>(t4, x64, d32);
  if (t4 * 4 < total) k_ir_accumulate_tail<<<count_launch(1), TPB, 0, s>>>(t4 * 4, total, x64, d32);
}

void fill_int(int *a, int n, int v, cudaStream_t s) {
  if (n > 0) k_fill_int<<<count_launch((n + TPB - 1) / TPB), TPB, 0, s>>>(a, n, v);
}

void pcg_alpha(int K, int KB, int gx, const double *part_pq, const double *rz, const int *active, double *alpha,
               int *status, int *n_active, cudaStream_t s) {
  k_pcg_alpha<<<count_launch(dim3(K)), SCAL_T, 0, s>>>(K, KB, gx, part_pq, rz, active, alpha, status, n_active);
}

void pcg_beta(int K, int KB, int gx, const double *part_rz, const double *part_rr, double *rz, double *rr,
              const double *bb, const double *tol2, int *active, double *beta, int *n_active, int first,
              cudaStream_t s) {
  k_pcg_beta<<<count_launch(dim3(K)), SCAL_T, 0, s>>>(K, KB, gx, part_rz, part_rr, rz, rr, bb, tol2, active, beta,
                                                      n_active, first);
}

void sum_partials(int K, int KB, int gx, const double *part, double *out, cudaStream_t s) {
  k_sum_partials<<<count_launch(dim3(K)), SCAL_T, 0, s>>>(K, KB, gx, part, out);
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

void convert_d2f(const double *a, long long n, float *o, cudaStream_t s) {
  k_convert_d2f<<<count_launch(dim3(grid_flat(n, g_n_sm))), TPB, 0, s>>>(a, n, o);
}

template <typename T>
void pack_colmajor(const double *src, long long N, int K, int KB, int nb, T *dst, cudaStream_t s) {
  const long long total = N * (long long)KB * nb;
  k_pack<T><<<count_launch(grid_flat(total, g_n_sm)), TPB, 0, s>>>(src, N, K, KB, dst, total);
}

template <typename T>
void unpack_colmajor(const T *src, long long N, int K, int KB, double *dst, cudaStream_t s) {
  k_unpack<T><<<count_launch(grid_flat(N * K, g_n_sm)), TPB, 0, s>>>(src, N, K, KB, dst);
}

#define DC_INST(T, KB) template struct Ops<T, KB>;
DC_INST(float, 1) DC_INST(float, 2) DC_INST(float, 4) DC_INST(float, 8) DC_INST(float, 16) DC_INST(float, 32)
DC_INST(double, 1) DC_INST(double, 2) DC_INST(double, 4) DC_INST(double, 8) DC_INST(double, 16) DC_INST(double, 32)
#undef DC_INST
#define DC_INST_IR(KB)                                                                                       \
  template void ir_residual<KB>(const Level &, const double *, const double *, double *, float *, int,      \
                                const int *, double *, int, cudaStream_t);                                  \
  template void ir_accumulate<KB>(long long, int, double *, const float *, cudaStream_t);
DC_INST_IR(1) DC_INST_IR(2) DC_INST_IR(4) DC_INST_IR(8) DC_INST_IR(16) DC_INST_IR(32)
#undef DC_INST_IR
template void pack_colmajor<float>(const double *, long long, int, int, int, float *, cudaStream_t);
template void pack_colmajor<double>(const double *, long long, int, int, int, double *, cudaStream_t);
template void unpack_colmajor<float>(const float *, long long, int, int, double *, cudaStream_t);
template void unpack_colmajor<double>(const double *, long long, int, int, double *, cudaStream_t);

}  // namespace dc
