// Node kernels of the nodal DC engine: stencil, Chebyshev smoothing,
// multigrid transfers, PCG vector updates and fixed-order reductions, with the
// host-side launchers of Ops<T, V, KB>.  Included by the translation units
// that instantiate Ops for one (compute, storage) pair each, so the template
// instantiations compile in parallel.
//
// Thread mapping of every node kernel: a thread owns W consecutive RHS lanes
// of one node (16 bytes of the compute type T: 4 fp32 / 2 fp64 lanes),
// KB/W threads share a node, and a 1D grid sweeps the flat (RHS block, node)
// index with the RHS block slowest.  Lane l of node n in RHS block b is
// element (b*N + n)*KB + l, so a warp's accesses are contiguous.
//
// Types: T is the arithmetic type (float inside the mixed-precision inner
// solve, double in the fp64 solve).  V is the storage type of the multigrid
// vectors (smoother iterates, residuals and corrections on every level, and
// the preconditioned vector z): T itself, or __half for the mixed solve,
// which halves the bytes the V-cycle moves.  Arithmetic is always in T.
// R is the type of a smoother's right-hand side: the PCG residual (T) on the
// finest level, the restricted residual (V) below it.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <type_traits>

#include "dc_internal.h"

namespace dc {

extern int g_n_sm;
int resident_blocks(const void *func);

namespace {

constexpr int TPB = 256;

// Per-thread dot-product sums of the fp32 stencil kernels with partials
// (k_apply, k_cheb_step) kept in shared memory, which frees the registers the
// two-lane stencil needs.
constexpr bool DOT_SMEM = true;

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

template <typename T, int W> struct alignas(sizeof(T) * W) Vec {
  T a[W];
};

// W lanes of storage type S at p, converted to T (and back).  For S == T a
// plain vector access; for __half an 8-byte (W = 4) access and conversions.
template <typename T, int W, typename S>
__device__ __forceinline__ Vec<T, W> ld(const S *p) {
  if constexpr (std::is_same<S, T>::value) {
    return *reinterpret_cast<const Vec<T, W> *>(p);
  } else {
    const Vec<S, W> raw = *reinterpret_cast<const Vec<S, W> *>(p);
    Vec<T, W> v;
#pragma unroll
    for (int e = 0; e < W; ++e) v.a[e] = (T)(float)raw.a[e];
    return v;
  }
}

template <typename T, int W, typename S>
__device__ __forceinline__ void st(S *p, const Vec<T, W> &v) {
  if constexpr (std::is_same<S, T>::value) {
    *reinterpret_cast<Vec<T, W> *>(p) = v;
  } else {
    Vec<S, W> raw;
#pragma unroll
    for (int e = 0; e < W; ++e) raw.a[e] = S((float)v.a[e]);
    *reinterpret_cast<Vec<S, W> *>(p) = raw;
  }
}

// Per-thread geometry of the "node x lane-group" mapping: a thread owns W
// consecutive RHS lanes of one RHS block, 16 bytes of the storage type S the
// kernel streams (4 fp32, 2 fp64 or 8 fp16 lanes), and LPN threads share one
// node.  Kernels sweep the RHS blocks one after the other (RHS block =
// slowest index of the flat work index), so the L2 working set of the
// stencil's z-neighbour planes is that of one RHS block at a time.
template <typename S, int KB> struct Lanes {
  static constexpr int W = (int)(16 / sizeof(S)) < KB ? (int)(16 / sizeof(S)) : KB;
  static constexpr int LPN = KB / W;  // threads per node
};

template <typename T, int KB>
__device__ __forceinline__ const typename CoefT<T>::type *coef_of(const void *c) {
  return reinterpret_cast<const typename CoefT<T>::type *>(c);
}

// v rounded to the storage type S and back (what a store and a load of v give).
template <typename S, typename T, int W>
__device__ __forceinline__ Vec<T, W> rounded(const Vec<T, W> &v) {
  Vec<T, W> o;
#pragma unroll
  for (int e = 0; e < W; ++e) o.a[e] = std::is_same<S, T>::value ? v.a[e] : (T)(float)S((float)v.a[e]);
  return o;
}

// Packed fp32 arithmetic on lane pairs (Blackwell's two-lane FMA, add and
// multiply: one instruction for lanes 2p and 2p+1), each lane rounded as the
// scalar instruction rounds it.
template <int W>
__device__ __forceinline__ float2 pair(const Vec<float, W> &v, int p) {
  return make_float2(v.a[2 * p], v.a[2 * p + 1]);
}
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }

// Seven-point stencil arithmetic for W lanes: d v0 - sum of c* times the six
// neighbours, in this fixed order.  With PACK (fp32) lane pairs go through
// Blackwell's two-lane FMA: one instruction per pair and coupling, each lane
// rounded as the scalar FMA rounds it.
template <typename T, int W, bool PACK>
__device__ __forceinline__ Vec<T, W> stencil_terms(T cd, T cxp, T cxm, T cyp, T cym, T czp, T czm,
                                                    const Vec<T, W> &v0, const Vec<T, W> &vxp, const Vec<T, W> &vxm,
                                                    const Vec<T, W> &vyp, const Vec<T, W> &vym, const Vec<T, W> &vzp,
                                                    const Vec<T, W> &vzm) {
  Vec<T, W> acc;
  if constexpr (PACK && std::is_same<T, float>::value && W % 2 == 0) {
    // couplings enter negated so that every term is one FMA
    const float2 kd = dup2(cd), kxp = dup2(-cxp), kxm = dup2(-cxm), kyp = dup2(-cyp), kym = dup2(-cym),
                 kzp = dup2(-czp), kzm = dup2(-czm);
#pragma unroll
    for (int p = 0; p < W / 2; ++p) {
      float2 a = __fmul2_rn(kd, pair(v0, p));
      a = __ffma2_rn(kxp, pair(vxp, p), a);
      a = __ffma2_rn(kxm, pair(vxm, p), a);
      a = __ffma2_rn(kyp, pair(vyp, p), a);
      a = __ffma2_rn(kym, pair(vym, p), a);
      a = __ffma2_rn(kzp, pair(vzp, p), a);
      a = __ffma2_rn(kzm, pair(vzm, p), a);
      acc.a[2 * p] = a.x;
      acc.a[2 * p + 1] = a.y;
    }
  } else {
#pragma unroll
    for (int e = 0; e < W; ++e)
      acc.a[e] = cd * v0.a[e] - cxp * vxp.a[e] - cxm * vxm.a[e] - cyp * vyp.a[e] - cym * vym.a[e] -
                 czp * vzp.a[e] - czm * vzm.a[e];
  }
  return acc;
}

// The seven-point stencil (A x) at element t of node n = (i, j, k) for the W
// lanes, x stored as S.  Branch-free: all seven loads are issued
// unconditionally (off-mesh neighbours are redirected to the node itself and
// get weight 0; c* is zero on the last node of its axis), so they are all in
// flight at once.
template <typename T, int KB, int W, typename S, bool PACK = true>
__device__ __forceinline__ Vec<T, W> stencil_vec(const typename CoefT<T>::type *__restrict__ coef,
                                                  const S *__restrict__ x, long long t, int n, int i, int j, int k,
                                                  const Dims &d) {
  const int sxn = 1, syn = d.Nx, szn = d.Nx * d.Ny;
  const bool hx = i > 0, hy = j > 0, hz = k > 0;
  const bool px = i + 1 < d.Nx, py = j + 1 < d.Ny, pz = k + 1 < d.Nz;
  const auto c = coef[n];
  const T wxm = coef[hx ? n - sxn : n].cx, wym = coef[hy ? n - syn : n].cy, wzm = coef[hz ? n - szn : n].cz;
  const Vec<T, W> v0 = ld<T, W>(x + t);
  const Vec<T, W> vxp = ld<T, W>(x + t + (px ? (long long)sxn * KB : 0));
  const Vec<T, W> vxm = ld<T, W>(x + t - (hx ? (long long)sxn * KB : 0));
  const Vec<T, W> vyp = ld<T, W>(x + t + (py ? (long long)syn * KB : 0));
  const Vec<T, W> vym = ld<T, W>(x + t - (hy ? (long long)syn * KB : 0));
  const Vec<T, W> vzp = ld<T, W>(x + t + (pz ? (long long)szn * KB : 0));
  const Vec<T, W> vzm = ld<T, W>(x + t - (hz ? (long long)szn * KB : 0));
  return stencil_terms<T, W, PACK>(c.d, px ? c.cx : (T)0, hx ? wxm : (T)0, py ? c.cy : (T)0, hy ? wym : (T)0,
                                   pz ? c.cz : (T)0, hz ? wzm : (T)0, v0, vxp, vxm, vyp, vym, vzp, vzm);
}

// A (c0 D^-1 v) at element t of node n for the W lanes (v stored as S), from
// the rows of A D^-1: two 16-byte loads per node instead of the coefficient
// and seven inverse-diagonal loads, the seven neighbour loads as above.
template <typename T, int KB, int W, typename S>
__device__ __forceinline__ Vec<T, W> stencil_rows(const RowDinv32 *__restrict__ rows, const S *__restrict__ x,
                                                   long long t, int n, int i, int j, int k, const Dims &d, T c0) {
  static_assert(sizeof(T) == 4, "the rows of A D^-1 are fp32");
  const int sxn = 1, syn = d.Nx, szn = d.Nx * d.Ny;
  const bool hx = i > 0, hy = j > 0, hz = k > 0;
  const bool px = i + 1 < d.Nx, py = j + 1 < d.Ny, pz = k + 1 < d.Nz;
  const float4 *rp = reinterpret_cast<const float4 *>(rows + n);
  const float4 ra = __ldg(rp), rb = __ldg(rp + 1);  // (d, xp, xm, yp), (ym, zp, zm, 0)
  const Vec<T, W> v0 = ld<T, W>(x + t);
  const Vec<T, W> vxp = ld<T, W>(x + t + (px ? (long long)sxn * KB : 0));
  const Vec<T, W> vxm = ld<T, W>(x + t - (hx ? (long long)sxn * KB : 0));
  const Vec<T, W> vyp = ld<T, W>(x + t + (py ? (long long)syn * KB : 0));
  const Vec<T, W> vym = ld<T, W>(x + t - (hy ? (long long)syn * KB : 0));
  const Vec<T, W> vzp = ld<T, W>(x + t + (pz ? (long long)szn * KB : 0));
  const Vec<T, W> vzm = ld<T, W>(x + t - (hz ? (long long)szn * KB : 0));
  return stencil_terms<T, W, true>(c0 * ra.x, c0 * ra.y, c0 * ra.z, c0 * ra.w, c0 * rb.x, c0 * rb.y, c0 * rb.z, v0,
                                   vxp, vxm, vyp, vym, vzp, vzm);
}

// Right-hand side r (type R) of a smoothing kernel at element t, times the
// per-lane scale when given (the finest level's PCG residual, see Rhs).
// The W per-RHS parameters (alpha, beta, scale) of one thread's lanes, p
// pointing at entry b * KB + q * W.  When W of them fill whole 16-byte words
// they are read by 16-byte loads: the parameter arrays start 256-byte aligned
// in the workspace and KB is a multiple of W, so p is 16-byte aligned then.
template <typename T, int W, typename P>
__device__ __forceinline__ Vec<T, W> lane_par(const P *__restrict__ p) {
  Vec<T, W> v;
  constexpr int PER = 16 / (int)sizeof(P);
  if constexpr (W % PER == 0 && sizeof(P) == 8) {
    const double2 *pu = reinterpret_cast<const double2 *>(p);
#pragma unroll
    for (int i = 0; i < W / 2; ++i) {
      const double2 u = __ldg(pu + i);
      v.a[2 * i] = (T)u.x;
      v.a[2 * i + 1] = (T)u.y;
    }
  } else if constexpr (W % PER == 0 && sizeof(P) == 4) {
    const float4 *pu = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int i = 0; i < W / 4; ++i) {
      const float4 u = __ldg(pu + i);
      v.a[4 * i] = (T)u.x;
      v.a[4 * i + 1] = (T)u.y;
      v.a[4 * i + 2] = (T)u.z;
      v.a[4 * i + 3] = (T)u.w;
    }
  } else {
#pragma unroll
    for (int e = 0; e < W; ++e) v.a[e] = (T)p[e];
  }
  return v;
}

template <typename T, int KB, int W, typename R>
__device__ __forceinline__ Vec<T, W> rhs_at(const R *__restrict__ r, const float *__restrict__ scale, long long t,
                                             int b, int q) {
  Vec<T, W> v = ld<T, W>(r + t);
  if (scale) {
    const Vec<T, W> sv = lane_par<T, W>(scale + b * KB + q * W);
#pragma unroll
    for (int e = 0; e < W; ++e) v.a[e] *= sv.a[e];
  }
  return v;
}

// Sweep over (RHS block b, node n, lane group q) with b slowest, W lanes per
// thread.  Defines W,
// LPN, q and, per iteration, ng (flat node index over all RHS blocks), b, n and
// t (offset of the thread's W lanes).
#define SWEEP(NN, MAGIC, NB, WIDTH)                                                            \
  constexpr int W = (WIDTH), LPN = KB / W;                                                     \
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
// Block partials land in partial[(b * gs + blockIdx.x) * KB + lane]; gs >=
// gridDim.x is the stride the consumer sums over (block 0 zeroes the unused
// tail), so every reduction kernel can run its own resident-capped grid.
template <typename T, int KB, int W>
__device__ __forceinline__ void block_reduce(T (&acc)[W], T *red, int b, double *partial, int gs) {
  constexpr int LPN = KB / W;
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
    partial[((long long)b * gs + blockIdx.x) * KB + threadIdx.x] = (double)v;
  }
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < (gs - (int)gridDim.x) * KB; i += TPB)
      partial[((long long)b * gs + gridDim.x) * KB + i] = 0.0;
  __syncthreads();
}

// Software prefetch into L2 of the element offset a thread will touch in its
// next grid-stride iteration (one thread per 128-byte line), so the DRAM
// requests of two iterations are in flight at once without extra registers.
__device__ __forceinline__ void pf_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
template <typename S>
__device__ __forceinline__ void pf_line(const S *base, long long t) {
  if ((threadIdx.x & 7) == 0) pf_l2(base + t);
}
struct NoPf {
  __device__ __forceinline__ void operator()(long long) const {}
};

// Sweep of a reducing kernel: the RHS blocks one after the other (the whole
// grid on one RHS block at a time, as in the flat sweep), each closed by the
// block reduction of that RHS block's per-thread sums.
// body(b, n, q, t, acc): RHS block, node, lane group, element offset, sums.
// With SM the per-thread sums live in shared memory (the thread's own W
// entries, same operations in the same order: identical sums) instead of W
// registers across the sweep, which leaves those registers to the body.
template <typename T, int KB, int W, bool SM = false, typename Body, typename Pf = NoPf>
__device__ __forceinline__ void sweep_reduce(int N, int nb, double *partial, int gs, Body body, Pf pf = Pf()) {
  constexpr int LPN = KB / W;
  __shared__ T red[(TPB / 32) * KB];
  __shared__ Vec<T, W> sacc[SM ? TPB : 1];
  const int q = threadIdx.x % LPN;
  const long long per = (long long)N * LPN;
  const long long stride = (long long)gridDim.x * TPB;
  for (int b = 0; b < nb; ++b) {
    T racc[W];
    T(&acc)[W] = SM ? sacc[SM ? threadIdx.x : 0].a : racc;
#pragma unroll
    for (int e = 0; e < W; ++e) acc[e] = (T)0;
    const long long base = (long long)b * N;
    for (long long g = (long long)blockIdx.x * TPB + threadIdx.x; g < per; g += stride) {
      const int n = (int)(g / LPN);
      if (g + stride < per) pf((base + (g + stride) / LPN) * KB + q * W);
      body(b, n, q, (base + n) * KB + q * W, acc);
    }
    if constexpr (SM) {
#pragma unroll
      for (int e = 0; e < W; ++e) racc[e] = acc[e];
    }
    block_reduce<T, KB, W>(racc, red, b, partial, gs);
  }
}

// The same body over the flat (RHS block, node, lane group) sweep, no reduction.
template <typename T, int KB, int W, typename Body, typename Pf = NoPf>
__device__ __forceinline__ void sweep_flat(int N, unsigned mn, int nb, Body body, Pf pf = Pf()) {
  constexpr int LPN = KB / W;
  const int q = threadIdx.x % LPN;
  const long long total = (long long)N * nb * LPN;
  const long long stride = (long long)gridDim.x * TPB;
  T acc[W];
  for (long long g = (long long)blockIdx.x * TPB + threadIdx.x; g < total; g += stride) {
    const int ng = (int)(g / LPN);
    const int b = fast_div(ng, N, mn);
    if (g + stride < total) pf(((g + stride) / LPN) * KB + q * W);
    body(b, ng - b * N, q, (long long)ng * KB + q * W, acc);
  }
}

// ---------------------------------------------------------------- stencil ops
// y = A x (y in T, x stored as S); with DOT also per-block partials of x.y.
template <typename T, typename S, int KB, bool DOT>
__global__ void __launch_bounds__(TPB, (DOT && sizeof(T) == 4 && sizeof(S) == 2) ? 4 : 0) k_apply(const void *__restrict__ cf, const S *__restrict__ x,
                                               T *__restrict__ y, Dims d, int nb, double *__restrict__ partial,
                                               int gs) {
  constexpr int W = Lanes<S, KB>::W;
  const auto *coef = coef_of<T, KB>(cf);
  auto body = [&](int b, int n, int q, long long t, T(&acc)[W]) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    const Vec<T, W> v = stencil_vec<T, KB, W, S, !DOT || DOT_SMEM>(coef, x, t, n, i, j, k, d);
    st<T, W>(y + t, v);
    if (DOT) {
      const Vec<T, W> xv = ld<T, W>(x + t);
#pragma unroll
      for (int e = 0; e < W; ++e) acc[e] += v.a[e] * xv.a[e];
    }
  };
  // prefetch pays where load latency bounds the kernel (fp32 stencils), not in the fp64-issue-bound ones
  auto pf = [&](long long tn) {
    if constexpr (sizeof(T) == 4) pf_line(x, tn);
  };
  if (DOT)
    sweep_reduce<T, KB, W, DOT_SMEM && sizeof(T) == 4>(d.N, nb, partial, gs, body, pf);
  else
    sweep_flat<T, KB, W>(d.N, d.mn, nb, body, pf);
}

// res = r - A z (two-lane stencil and next-iteration L2 prefetch like the
// Chebyshev steps: 367 -> 355 us per fine-level launch at 1M nodes x 256 RHS;
// the same prefetch in k_prolong_add made it slower, 299 -> 315 us)
template <typename T, typename V, typename R, int KB>
__global__ void __launch_bounds__(TPB) k_residual(const void *__restrict__ cf, const R *__restrict__ r,
                                                  const float *__restrict__ scale, const V *__restrict__ z,
                                                  V *__restrict__ res, Dims d, int nb) {
  constexpr int W = Lanes<V, KB>::W;
  const auto *coef = coef_of<T, KB>(cf);
  auto pf = [&](long long tn) {
    if constexpr (sizeof(T) == 4) {
      pf_line(z, tn);
      pf_line(r, tn);
    }
  };
  sweep_flat<T, KB, W>(
      d.N, d.mn, nb,
      [&](int b, int n, int q, long long t, T(&)[W]) {
        int i, j, k;
        node_ijk(n, d, i, j, k);
        const Vec<T, W> az = stencil_vec<T, KB, W, V>(coef, z, t, n, i, j, k, d);
        Vec<T, W> rv = rhs_at<T, KB, W>(r, scale, t, b, q);
#pragma unroll
        for (int e = 0; e < W; ++e) rv.a[e] -= az.a[e];
        st<T, W>(res + t, rv);
      },
      pf);
}

// First Chebyshev step from z = 0: z = c0 * D^-1 r.
template <typename T, typename V, typename R, int KB>
__global__ void __launch_bounds__(TPB) k_cheb_first(const T *__restrict__ invd, const R *__restrict__ r,
                                                    const float *__restrict__ scale, V *__restrict__ z, Dims d,
                                                    int nb, T c0) {
  constexpr int W = Lanes<V, KB>::W;
  sweep_flat<T, KB, W>(d.N, d.mn, nb, [&](int b, int n, int q, long long t, T(&)[W]) {
    const T s = c0 * invd[n];
    Vec<T, W> v = rhs_at<T, KB, W>(r, scale, t, b, q);
#pragma unroll
    for (int e = 0; e < W; ++e) v.a[e] *= s;
    st<T, W>(z + t, v);
  });
}

// Chebyshev step in three-term form (x_{k+1} = x_k + c1 (x_k - x_{k-1}) + c2 D^-1 (r - A x_k)):
//   PREV = 0: no momentum term (first step from a nonzero start, c1 = 0)
//   PREV = 1: x_{k-1} read from zout (overwritten in place with x_{k+1})
//   PREV = 2: x_{k-1} = 0 (second step of a zero-start sequence)
//   PREV = 3: the second step of a zero start with x_1 = c0 D^-1 r formed from r
//             on the fly (zin unused): the first step is never stored, and
//             the step streams r and x_2 only
//   PREV = 4: the third step of that sequence: momentum with x_{k-1} = x_1 =
//             c0 D^-1 r formed pointwise from r (zout's old content not read)
// Four streams per RHS lane (x_k, r, x_{k-1} read; x_{k+1} write) instead of the
// five of the d-vector form.  With DOT (finest level), also per-block partials
// of r . x_{k+1} with the unscaled PCG residual r.
template <typename T, typename V, typename R, int KB, bool DOT, int PREV>
__global__ void __launch_bounds__(TPB) k_cheb_step(const void *__restrict__ cf, const T *__restrict__ invd,
                                                   const R *__restrict__ r, const float *__restrict__ scale,
                                                   const V *__restrict__ zin, V *zout, Dims d, int nb, T c1, T c2,
                                                   double *__restrict__ partial, int gs, T c0) {
  constexpr int W = Lanes<V, KB>::W;
  static_assert(!(DOT && PREV >= 3), "the r.z partials belong to the last post-smoothing step");
  // PREV 3: cf holds the rows of A D^-1 (RowDinv32), not the coefficients
  const auto *coef = coef_of<T, KB>(cf);
  auto body = [&](int b, int n, int q, long long t, T(&acc)[W]) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    // A x_k (two lanes per instruction), r loaded after the stencil's seven
    // loads, then the scalar update.  Registers are left to
    // the compiler (64, 4 blocks of TPB per SM): at 1M nodes x 256 RHS this
    // measured faster than 48 registers at 5 blocks, and than the zero-start
    // step as one r - A x chain of two-lane FMAs (405 -> 384 us per launch).
    Vec<T, W> az, zc, zo;
    if constexpr (PREV == 3)
      az = stencil_rows<T, KB, W, R>(static_cast<const RowDinv32 *>(cf), r, t, n, i, j, k, d, c0);
    else
      az = stencil_vec<T, KB, W, V, !DOT || DOT_SMEM>(coef, zin, t, n, i, j, k, d);
    const Vec<T, W> rv = ld<T, W>(r + t);
    if constexpr (PREV != 3) zc = ld<T, W>(zin + t);
    if (PREV == 1) zo = ld<T, W>(zout + t);
    const T dn = invd[n];
    const T s = c2 * dn;
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const T re = scale ? rv.a[e] * (T)scale[b * KB + q * W + e] : rv.a[e];
      T ae = az.a[e];
      if constexpr (PREV == 3) {
        // x_1 = c0 D^-1 (scale r); the per-lane scale factors out of A x_1
        zc.a[e] = (c0 * dn) * re;
        if (scale) ae *= (T)scale[b * KB + q * W + e];
      }
      if constexpr (PREV == 4) zo.a[e] = (c0 * dn) * re;  // x_{k-1} = x_1
      const T mom = (PREV == 1 || PREV == 4) ? c1 * (zc.a[e] - zo.a[e])
                                             : ((PREV == 2 || PREV == 3) ? c1 * zc.a[e] : (T)0);
      zo.a[e] = zc.a[e] + mom + s * (re - ae);
    }
    st<T, W>(zout + t, zo);
    if constexpr (DOT) {
      // r . z with z as stored (rounded to V): the preconditioned vector PCG uses
      const Vec<T, W> zs = rounded<V>(zo);
#pragma unroll
      for (int e = 0; e < W; ++e) acc[e] += rv.a[e] * zs.a[e];
    }
  };
  auto pf = [&](long long tn) {
    if constexpr (sizeof(T) == 4) {
      if (PREV != 3) pf_line(zin, tn);
      pf_line(r, tn);
      if (PREV == 1) pf_line(zout, tn);
    }
  };
  if (DOT)
    sweep_reduce<T, KB, W, DOT_SMEM && sizeof(T) == 4>(d.N, nb, partial, gs, body, pf);
  else
    sweep_flat<T, KB, W>(d.N, d.mn, nb, body, pf);
}

// ---------------------------------------------------------------- staged stencil
// Bulk asynchronous copies (cp.async.bulk, the Blackwell TMA engine) into
// shared memory, completed on mbarriers.  Every wait is bounded: a wait that
// gives up records bit 8 in the status word and the kernel drains its copies
// (again with a bound) before returning.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this thread's earlier generic-proxy shared accesses before later async-proxy (bulk copy) ones
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// global -> shared bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of `bar` (each try_wait itself suspends for a
// hardware-defined interval, so the bound is a time bound of seconds).
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it)
    if (mbar_test(bar, parity)) return true;
  return false;
}

constexpr int BULK_T = 512;  // threads of the staged kernel

// Bytes of shared memory k_cheb_bulk needs: x_k rows (4 plane slots of TY+2
// rows), r and x_{k-1} rows (NA slots of TY rows) and coefficient rows (NA+1
// slots of TY+1 rows) for Nx nodes, KB lanes of V, plus 4+NA mbarriers.
inline size_t cheb_bulk_smem(int Nx, int KB, size_t vbytes, int TY, int NA, bool prev) {
  const size_t row = (size_t)Nx * KB * vbytes;
  return (4 * (size_t)(TY + 2) + (size_t)NA * TY * (prev ? 2 : 1)) * row +
         (size_t)(NA + 1) * (TY + 1) * Nx * sizeof(Coef32) + (4 + (size_t)NA) * 8;
}

// Chebyshev step (PREV as in k_cheb_step, no dot partials) on the finest
// level with every stream staged in shared memory.  One CTA owns RHS block b
// and a slab of TY node rows (all x, all KB lanes) and marches through the z
// planes: while it updates plane k, the bulk-copy engine brings in x_k of
// plane k+2 (rows j0-1 .. j0+TY, four plane slots) and r, x_{k-1} and the
// coefficients of planes up to k+NA-1 (NA slots), so the DRAM streams stay in flight
// independently of the threads' registers; all stencil, coefficient and
// vector reads then come from shared memory and x_{k+1} is written straight
// from registers (1/diag is recomputed from the staged diagonal: a 1/diag row
// is not a multiple of 16 bytes).  Rows and planes beyond the mesh are redirected to the node
// itself with weight 0 (c+* is zero on the last node of an axis).  The node
// rows of one plane (and RHS block) are contiguous, so every copy is one
// contiguous range.
template <typename T, typename V, int KB, int PREV>
__global__ void __launch_bounds__(BULK_T) k_cheb_bulk(const Coef32 *__restrict__ coef,
                                                      const V *__restrict__ r, const V *__restrict__ zin, V *zout,
                                                      Dims d, int TY, int NA, T c1, T c2,
                                                      int *__restrict__ status) {
  static_assert(sizeof(T) == 4, "staged smoothing is for the fp32 inner solve");
  constexpr int W = Lanes<V, KB>::W, LPN = KB / W;
  extern __shared__ __align__(128) unsigned char smem[];
  const int Nx = d.Nx, Ny = d.Ny, Nz = d.Nz;
  const long long N = d.N, NxNy = (long long)Nx * Ny;
  const int nslab = (Ny + TY - 1) / TY;
  const int b = blockIdx.x / nslab, slab = blockIdx.x % nslab;
  const int j0 = slab * TY, j1 = min(j0 + TY, Ny);
  const int jlo = max(j0 - 1, 0), jhi = min(j1, Ny - 1);
  const int zrows = TY + 2, crows = TY + 1;
  const size_t row = (size_t)Nx * KB;  // elements per node row
  V *zb = reinterpret_cast<V *>(smem);
  V *rb = zb + 4 * (size_t)zrows * row;
  V *pb = rb + (size_t)NA * TY * row;
  Coef32 *cb = reinterpret_cast<Coef32 *>(pb + (PREV == 1 ? (size_t)NA * TY * row : 0));
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(cb + (size_t)(NA + 1) * crows * Nx);
  const long long base = (long long)b * N * KB;
  const unsigned zbytes = (unsigned)((size_t)(jhi - jlo + 1) * row * sizeof(V));
  const unsigned rbytes = (unsigned)((size_t)(j1 - j0) * row * sizeof(V));
  const unsigned cbytes = (unsigned)((size_t)(j1 - jlo) * Nx * sizeof(Coef32));
  auto issue_z = [&](int k) {
    unsigned long long *bb = bar + (k & 3);
    mbar_expect_tx(bb, zbytes);
    bulk_g2s(zb + (size_t)(k & 3) * zrows * row + (size_t)(jlo - (j0 - 1)) * row,
             zin + base + ((long long)k * NxNy + (long long)jlo * Nx) * KB, zbytes, bb);
  };
  // r, x_{k-1} and coefficients (rows jlo .. j1-1) of plane k
  auto issue_aux = [&](int k) {
    const int sa = k % NA;
    unsigned long long *bb = bar + 4 + sa;
    const long long node0 = (long long)k * NxNy + (long long)j0 * Nx;
    mbar_expect_tx(bb, (PREV == 1 ? 2 * rbytes : rbytes) + cbytes);
    bulk_g2s(rb + (size_t)sa * TY * row, r + base + node0 * KB, rbytes, bb);
    if (PREV == 1) bulk_g2s(pb + (size_t)sa * TY * row, zout + base + node0 * KB, rbytes, bb);
    bulk_g2s(cb + (size_t)(k % (NA + 1)) * crows * Nx + (size_t)(jlo - (j0 - 1)) * Nx,
             coef + (long long)k * NxNy + (long long)jlo * Nx, cbytes, bb);
  };
  if (threadIdx.x == 0) {
    for (int i = 0; i < 4 + NA; ++i) mbar_init(bar + i, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    issue_z(0);
    if (Nz > 1) issue_z(1);
    for (int k = 0; k < NA - 1 && k < Nz; ++k) issue_aux(k);
  }
  int issued_z = Nz > 1 ? 2 : 1, issued_aux = min(NA - 1, Nz);
  bool failed = false;
  for (int k = 0; k < Nz; ++k) {
    // slots refilled here were last read in iteration k-1 (closed by its __syncthreads)
    if (threadIdx.x == 0) {
      fence_proxy_async();
      if (k + 2 < Nz) issue_z(k + 2);
      if (k + NA - 1 < Nz) issue_aux(k + NA - 1);
    }
    if (k + 2 < Nz) issued_z = k + 3;
    if (k + NA - 1 < Nz) issued_aux = k + NA;
    bool ok = mbar_wait(bar + (k & 3), (k >> 2) & 1);
    if (k + 1 < Nz) ok = ok && mbar_wait(bar + ((k + 1) & 3), ((k + 1) >> 2) & 1);
    ok = ok && mbar_wait(bar + 4 + k % NA, (k / NA) & 1);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const V *z0 = zb + (size_t)(k & 3) * zrows * row;
    const V *zm = k > 0 ? zb + (size_t)((k + 3) & 3) * zrows * row : z0;
    const V *zp = k + 1 < Nz ? zb + (size_t)((k + 1) & 3) * zrows * row : z0;
    const V *rs = rb + (size_t)(k % NA) * TY * row;
    const V *ps = pb + (size_t)(k % NA) * TY * row;
    const Coef32 *c0 = cb + (size_t)(k % (NA + 1)) * crows * Nx;                      // row 0 = j0 - 1
    const Coef32 *cm = k > 0 ? cb + (size_t)((k + NA) % (NA + 1)) * crows * Nx : c0;  // plane k - 1
    const int items = (j1 - j0) * Nx * LPN;
    for (int it = threadIdx.x; it < items; it += BULK_T) {
      const int q = it % LPN, rem = it / LPN;
      const int jj = fast_div(rem, Nx, d.mx), i = rem - jj * Nx, j = j0 + jj;
      const bool hx = i > 0, px = i + 1 < Nx, hy = j > 0, py = j + 1 < Ny, hz = k > 0, pz = k + 1 < Nz;
      const int co = (jj + 1) * Nx + i;  // own node in the coefficient slots
      const Coef32 c = c0[co];
      const T cxp = px ? c.cx : (T)0, cyp = py ? c.cy : (T)0, czp = pz ? c.cz : (T)0;
      const T cxm = hx ? c0[co - 1].cx : (T)0, cym = hy ? c0[co - Nx].cy : (T)0, czm = hz ? cm[co].cz : (T)0;
      const size_t so = ((size_t)(jj + 1) * Nx + i) * KB + q * W;
      const Vec<T, W> v0 = ld<T, W>(z0 + so);
      const Vec<T, W> vxp = ld<T, W>(z0 + so + (px ? KB : 0));
      const Vec<T, W> vxm = ld<T, W>(z0 + so - (hx ? KB : 0));
      const Vec<T, W> vyp = ld<T, W>(z0 + so + (py ? row : 0));
      const Vec<T, W> vym = ld<T, W>(z0 + so - (hy ? row : 0));
      const Vec<T, W> vzp = ld<T, W>(zp + so);
      const Vec<T, W> vzm = ld<T, W>(zm + so);
      const size_t ro = ((size_t)jj * Nx + i) * KB + q * W;
      const Vec<T, W> rv = ld<T, W>(rs + ro);
      Vec<T, W> zo;
      if (PREV == 1) zo = ld<T, W>(ps + ro);
      const T sd = c2 / c.d;
#pragma unroll
      for (int e = 0; e < W; ++e) {
        const T az = c.d * v0.a[e] - cxp * vxp.a[e] - cxm * vxm.a[e] - cyp * vyp.a[e] - cym * vym.a[e] -
                     czp * vzp.a[e] - czm * vzm.a[e];
        T mom = (T)0;
        if (PREV == 1) mom = c1 * (v0.a[e] - zo.a[e]);
        if (PREV == 2) mom = c1 * v0.a[e];
        zo.a[e] = v0.a[e] + mom + sd * (rv.a[e] - az);
      }
      st<T, W>(zout + base + ((long long)k * NxNy + (long long)j * Nx + i) * KB + q * W, zo);
    }
    __syncthreads();
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicOr(status, 8);
      // drain: the copies issued into this CTA's shared memory must land before it exits;
      // wait for the latest issued phase of every slot
      for (int k = max(issued_z - 4, 0); k < issued_z; ++k) mbar_wait(bar + (k & 3), (k >> 2) & 1);
      for (int k = max(issued_aux - NA, 0); k < issued_aux; ++k) mbar_wait(bar + 4 + k % NA, (k / NA) & 1);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- transfers
struct XferTab {
  const int *fi;        // coarse node -> fine node, per axis at roff[a]
  const void *wl, *wr;  // T weights of fine fi-1 / fi+1
  const int *pl;        // fine node -> left coarse node, per axis at poff[a]
  const void *pw;       // T weight on pl
  long long roff[3], poff[3];
};

template <typename T, typename V, int KB>
__global__ void __launch_bounds__(TPB) k_restrict(const V *__restrict__ res, V *__restrict__ rc, Dims f, Dims c,
                                                  int nb, XferTab tb) {
  const T *wl = (const T *)tb.wl, *wr = (const T *)tb.wr;
  SWEEP(c.N, c.mn, nb, (Lanes<V, KB>::W)) {
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
          const Vec<T, W> v = ld<T, W>(res + fb + (row + fx + cx - 1) * KB);
#pragma unroll
          for (int e = 0; e < W; ++e) acc.a[e] += w * v.a[e];
        }
      }
    }
    st<T, W>(rc + t, acc);
  }
}

template <typename T, typename V, int KB>
__global__ void __launch_bounds__(TPB) k_prolong_add(const V *__restrict__ zc, V *__restrict__ z, Dims f, Dims c,
                                                     int nb, XferTab tb) {
  const T *pw = (const T *)tb.pw;
  SWEEP(f.N, f.mn, nb, (Lanes<V, KB>::W)) {
    SWEEP_INDEX(f.N, f.mn)
    int i, j, k;
    node_ijk(n, f, i, j, k);
    const int I = tb.pl[tb.poff[0] + i], J = tb.pl[tb.poff[1] + j], K = tb.pl[tb.poff[2] + k];
    const T ax = pw[tb.poff[0] + i], ay = pw[tb.poff[1] + j], az = pw[tb.poff[2] + k];
    const T wx[2] = {ax, (T)1 - ax}, wy[2] = {ay, (T)1 - ay}, wz[2] = {az, (T)1 - az};
    const long long cb = (long long)b * c.N * KB + q * W;
    Vec<T, W> acc = ld<T, W>(z + t);
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
          const Vec<T, W> v = ld<T, W>(zc + cb + (row + I + e2) * KB);
#pragma unroll
          for (int e = 0; e < W; ++e) acc.a[e] += w * v.a[e];
        }
      }
    }
    st<T, W>(z + t, acc);
  }
}

// z_c = Ainv r_c on the coarsest level (dense, row-major Ainv[nc][nc]).
template <typename T, typename V, typename R, int KB>
__global__ void __launch_bounds__(TPB) k_coarse_solve(const T *__restrict__ Ainv, Dims c, int nb,
                                                      const R *__restrict__ rc, const float *__restrict__ scale,
                                                      V *__restrict__ zc) {
  const int nc = (int)c.N;
  SWEEP(c.N, c.mn, nb, (Lanes<V, KB>::W)) {
    SWEEP_INDEX(c.N, c.mn)
    const T *row = Ainv + (long long)n * nc;
    const long long base = (long long)b * nc * KB + q * W;
    Vec<T, W> acc;
#pragma unroll
    for (int e = 0; e < W; ++e) acc.a[e] = 0;
    for (int m = 0; m < nc; ++m) {
      const T w = row[m];
      const Vec<T, W> v = rhs_at<T, KB, W>(rc, scale, base + (long long)m * KB, b, q);
#pragma unroll
      for (int e = 0; e < W; ++e) acc.a[e] += w * v.a[e];
    }
    st<T, W>(zc + t, acc);
  }
}

// ---------------------------------------------------------------- PCG vectors
// x += a p ; r -= a q ; partial |r|^2 (a per RHS).  With SMOOTH, also the first
// Chebyshev step of the fine level on the new residual: z = c0 D^-1 (scale r).
template <typename T, typename V, int KB, bool SMOOTH>
__global__ void __launch_bounds__(TPB) k_update_xr(Dims d, int nb, T *__restrict__ x, T *__restrict__ r,
                                                   const V *__restrict__ p, const T *__restrict__ qv,
                                                   const T *__restrict__ alpha, double *__restrict__ partial,
                                                   const T *__restrict__ invd, V *__restrict__ z, T c0,
                                                   const float *__restrict__ scale, V *__restrict__ rv_out, int gs,
                                                   int x_zero) {
  constexpr int W = Lanes<T, KB>::W;
  sweep_reduce<T, KB, W>(d.N, nb, partial, gs, [&](int b, int n, int q, long long t, T(&acc)[W]) {
    // x_zero: the first update of a solve from x = 0, whose x is not read (nor zeroed beforehand)
    Vec<T, W> xv, rv = ld<T, W>(r + t);
    if (x_zero) {
#pragma unroll
      for (int e = 0; e < W; ++e) xv.a[e] = (T)0;
    } else {
      xv = ld<T, W>(x + t);
    }
    const Vec<T, W> pv = ld<T, W>(p + t), qq = ld<T, W>(qv + t);
    const Vec<T, W> av = lane_par<T, W>(alpha + b * KB + q * W);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      xv.a[e] += av.a[e] * pv.a[e];
      rv.a[e] -= av.a[e] * qq.a[e];
      acc[e] += rv.a[e] * rv.a[e];
    }
    st<T, W>(x + t, xv);
    st<T, W>(r + t, rv);
    if (SMOOTH) {
      if (scale) {
        const Vec<T, W> sv = lane_par<T, W>(scale + b * KB + q * W);
#pragma unroll
        for (int e = 0; e < W; ++e) rv.a[e] *= sv.a[e];
      }
      if (rv_out) st<T, W>(rv_out + t, rv);
      const T s = c0 * invd[n];
#pragma unroll
      for (int e = 0; e < W; ++e) rv.a[e] *= s;
      st<T, W>(z + t, rv);
    }
  });
}

// rv_out = V(scale r): the finest level's V-cycle input in the storage type.
template <typename T, typename V, int KB>
__global__ void __launch_bounds__(TPB) k_scale_to(Dims d, int nb, const T *__restrict__ r,
                                                  const float *__restrict__ scale, V *__restrict__ rv_out) {
  SWEEP(d.N, d.mn, nb, (Lanes<V, KB>::W)) {
    SWEEP_INDEX(d.N, d.mn)
    st<T, W>(rv_out + t, rhs_at<T, KB, W>(r, scale, t, b, q));
  }
}

template <typename T, typename S, int KB>
__global__ void __launch_bounds__(TPB) k_dot(Dims d, int nb, const T *__restrict__ a, const S *__restrict__ bb,
                                             double *__restrict__ partial, int gs) {
  constexpr int W = Lanes<S, KB>::W;
  sweep_reduce<T, KB, W>(d.N, nb, partial, gs, [&](int, int, int, long long t, T(&acc)[W]) {
    const Vec<T, W> av = ld<T, W>(a + t), bv = ld<T, W>(bb + t);
#pragma unroll
    for (int e = 0; e < W; ++e) acc[e] += av.a[e] * bv.a[e];
  });
}

// p = z + beta p (p stored as V, like z)
template <typename T, typename V, int KB>
__global__ void __launch_bounds__(TPB) k_p_update(Dims d, int nb, V *__restrict__ p, const V *__restrict__ z,
                                                  const T *__restrict__ beta) {
  SWEEP(d.N, d.mn, nb, (Lanes<V, KB>::W)) {
    SWEEP_INDEX(d.N, d.mn)
    Vec<T, W> pv = ld<T, W>(p + t);
    const Vec<T, W> zv = ld<T, W>(z + t);
    const Vec<T, W> bv = lane_par<T, W>(beta + b * KB + q * W);
#pragma unroll
    for (int e = 0; e < W; ++e) pv.a[e] = zv.a[e] + bv.a[e] * pv.a[e];
    st<T, W>(p + t, pv);
  }
}

// ---------------------------------------------------------------- grids
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

template <typename T>
const void *coef_ptr(const Level &L) {
  return std::is_same<T, double>::value ? (const void *)L.d_coef64 : (const void *)L.d_coef32;
}
template <typename T>
const T *invd_ptr(const Level &L) {
  return reinterpret_cast<const T *>(std::is_same<T, double>::value ? (const void *)L.d_invd64
                                                                    : (const void *)L.d_invd32);
}

template <typename T>
XferTab make_tab(const Level &f) {
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

}  // namespace

// ------------------------------------------------------------------ launchers
// Grids of the non-reducing sweeps are capped at the blocks the GPU holds at
// once (resident_blocks), so every sweep is one wave and the stencil's
// neighbour planes are reused from L2.
#define GRID_KL(NODES, KERNEL, LPN) \
  count_launch(dim3(grid_nodes((NODES), (LPN), nb, g_n_sm, resident_blocks((const void *)(KERNEL)))))
#define GRID_K(NODES, KERNEL) GRID_KL(NODES, KERNEL, (Lanes<V, KB>::LPN))

// Grid of a reducing kernel: its own resident-capped grid, at most gx (the
// stride of the partial arrays).
#define RED_GRID(NODES, KERNEL, LPN) \
  count_launch(dim3(std::min(gx, grid_nodes((NODES), (LPN), nb, g_n_sm, resident_blocks((const void *)(KERNEL))))))

template <typename T, typename V, int KB>
void Ops<T, V, KB>::apply(const Level &L, const T *x, T *y, int nb, double *partial, int gx, cudaStream_t s) {
  if (partial)
    k_apply<T, T, KB, true><<<RED_GRID(L.dims.N, (k_apply<T, T, KB, true>), (Lanes<T, KB>::LPN)), TPB, 0, s>>>(
        coef_ptr<T>(L), x, y, L.dims, nb, partial, gx);
  else
    k_apply<T, T, KB, false><<<GRID_KL(L.dims.N, (k_apply<T, T, KB, false>), (Lanes<T, KB>::LPN)), TPB, 0, s>>>(
        coef_ptr<T>(L), x, y, L.dims, nb, nullptr, 0);
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::apply_v(const Level &L, const V *x, T *y, int nb, double *partial, int gx, cudaStream_t s) {
  k_apply<T, V, KB, true><<<RED_GRID(L.dims.N, (k_apply<T, V, KB, true>), (Lanes<V, KB>::LPN)), TPB, 0, s>>>(
      coef_ptr<T>(L), x, y, L.dims, nb, partial, gx);
}

template <typename T, typename V, int KB>
int Ops<T, V, KB>::red_blocks_per_sm() {
  int m = resident_blocks((const void *)k_apply<T, T, KB, true>);
  m = std::max(m, resident_blocks((const void *)k_apply<T, V, KB, true>));
  m = std::max(m, resident_blocks((const void *)k_cheb_step<T, V, T, KB, true, 1>));
  m = std::max(m, resident_blocks((const void *)k_cheb_step<T, V, V, KB, true, 1>));
  m = std::max(m, resident_blocks((const void *)k_update_xr<T, V, KB, true>));
  m = std::max(m, resident_blocks((const void *)k_update_xr<T, V, KB, false>));
  m = std::max(m, resident_blocks((const void *)k_dot<T, T, KB>));
  m = std::max(m, resident_blocks((const void *)k_dot<T, V, KB>));
  return m;
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::residual(const Level &L, Rhs<T, V> r, const V *z, V *res, int nb, cudaStream_t s) {
  if (r.full)
    k_residual<T, V, T, KB><<<GRID_K(L.dims.N, (k_residual<T, V, T, KB>)), TPB, 0, s>>>(
        coef_ptr<T>(L), r.full, r.scale, z, res, L.dims, nb);
  else
    k_residual<T, V, V, KB><<<GRID_K(L.dims.N, (k_residual<T, V, V, KB>)), TPB, 0, s>>>(
        coef_ptr<T>(L), r.part, nullptr, z, res, L.dims, nb);
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::cheb_first(const Level &L, Rhs<T, V> r, V *z, int nb, double c0, cudaStream_t s) {
  if (r.full)
    k_cheb_first<T, V, T, KB><<<GRID_K(L.dims.N, (k_cheb_first<T, V, T, KB>)), TPB, 0, s>>>(
        invd_ptr<T>(L), r.full, r.scale, z, L.dims, nb, (T)c0);
  else
    k_cheb_first<T, V, V, KB><<<GRID_K(L.dims.N, (k_cheb_first<T, V, V, KB>)), TPB, 0, s>>>(
        invd_ptr<T>(L), r.part, nullptr, z, L.dims, nb, (T)c0);
}

template <typename T, typename V, int KB, typename R, bool DOT, int PREV>
static void cheb_launch(const Level &L, const R *r, const float *scale, const V *zin, V *zout, int nb, double c1,
                        double c2, double *partial, int gx, cudaStream_t s, double c0 = 0.0) {
  const dim3 g = DOT ? RED_GRID(L.dims.N, (k_cheb_step<T, V, R, KB, DOT, PREV>), (Lanes<V, KB>::LPN))
                     : GRID_K(L.dims.N, (k_cheb_step<T, V, R, KB, DOT, PREV>));
  const void *cf = PREV == 3 ? (const void *)L.d_rows32 : (const void *)coef_ptr<T>(L);
  k_cheb_step<T, V, R, KB, DOT, PREV><<<g, TPB, 0, s>>>(cf, invd_ptr<T>(L), r, scale, zin, zout, L.dims, nb, (T)c1,
                                                        (T)c2, partial, gx, (T)c0);
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::cheb_step(const Level &L, Rhs<T, V> r, const V *zin, V *zout, int prev, int nb, double c1,
                              double c2, double *partial, int gx, cudaStream_t s, double c0) {
  if constexpr (sizeof(T) == 4) {
    if (prev == 3 && !partial) {
      if (r.full) cheb_launch<T, V, KB, T, false, 3>(L, r.full, r.scale, nullptr, zout, nb, c1, c2, nullptr, gx, s, c0);
      else cheb_launch<T, V, KB, V, false, 3>(L, r.part, nullptr, nullptr, zout, nb, c1, c2, nullptr, gx, s, c0);
      return;
    }
    if (prev == 4 && !partial) {
      if (r.full) cheb_launch<T, V, KB, T, false, 4>(L, r.full, r.scale, zin, zout, nb, c1, c2, nullptr, gx, s, c0);
      else cheb_launch<T, V, KB, V, false, 4>(L, r.part, nullptr, zin, zout, nb, c1, c2, nullptr, gx, s, c0);
      return;
    }
  }
  if (r.full) {
    const T *rp = r.full;
    const float *sc = r.scale;
    if (partial) {
      if (prev == 1) cheb_launch<T, V, KB, T, true, 1>(L, rp, sc, zin, zout, nb, c1, c2, partial, gx, s);
      else if (prev == 2) cheb_launch<T, V, KB, T, true, 2>(L, rp, sc, zin, zout, nb, c1, c2, partial, gx, s);
      else cheb_launch<T, V, KB, T, true, 0>(L, rp, sc, zin, zout, nb, c1, c2, partial, gx, s);
    } else {
      if (prev == 1) cheb_launch<T, V, KB, T, false, 1>(L, rp, sc, zin, zout, nb, c1, c2, nullptr, gx, s);
      else if (prev == 2) cheb_launch<T, V, KB, T, false, 2>(L, rp, sc, zin, zout, nb, c1, c2, nullptr, gx, s);
      else cheb_launch<T, V, KB, T, false, 0>(L, rp, sc, zin, zout, nb, c1, c2, nullptr, gx, s);
    }
  } else {
    const V *rp = r.part;
    if (partial) {
      if (prev == 1) cheb_launch<T, V, KB, V, true, 1>(L, rp, nullptr, zin, zout, nb, c1, c2, partial, gx, s);
      else if (prev == 2) cheb_launch<T, V, KB, V, true, 2>(L, rp, nullptr, zin, zout, nb, c1, c2, partial, gx, s);
      else cheb_launch<T, V, KB, V, true, 0>(L, rp, nullptr, zin, zout, nb, c1, c2, partial, gx, s);
    } else {
      if (prev == 1) cheb_launch<T, V, KB, V, false, 1>(L, rp, nullptr, zin, zout, nb, c1, c2, nullptr, gx, s);
      else if (prev == 2) cheb_launch<T, V, KB, V, false, 2>(L, rp, nullptr, zin, zout, nb, c1, c2, nullptr, gx, s);
      else cheb_launch<T, V, KB, V, false, 0>(L, rp, nullptr, zin, zout, nb, c1, c2, nullptr, gx, s);
    }
  }
}

// Staged Chebyshev step (k_cheb_bulk) when it applies: RHS and iterates in
// the multigrid storage type, node rows a multiple of 16 bytes and a slab of
// at least one row fitting in shared memory.  Returns false otherwise (the
// caller then uses cheb_step).
template <typename T, typename V, int KB>
bool Ops<T, V, KB>::cheb_bulk(const Level &L, const V *r, const V *zin, V *zout, int prev, int nb, double c1,
                              double c2, int *status, int shape, cudaStream_t s) {
  if constexpr (sizeof(T) != 4 || sizeof(V) != 2 || (KB * sizeof(V)) % 16 != 0) {
    return false;
  } else {
    if (!status) return false;
    // function-local statics: initialised once, thread-safe (server worker threads solve concurrently)
    static const int max_smem = [] {
      int dev = 0, v = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      return v;
    }();
    const size_t budget = (size_t)max_smem;
    // slab height and copy depth: the forced pair if given, else the first that fits
    int TY = 0, NA = 0;
    const int cand[4][2] = {{2, 3}, {1, 3}, {2, 2}, {1, 2}};
    for (auto &cnd : cand) {
      if (shape > 0 && cnd[0] * 10 + cnd[1] != shape) continue;
      if (cheb_bulk_smem(L.dims.Nx, KB, sizeof(V), cnd[0], cnd[1], true) <= budget) {
        TY = cnd[0];
        NA = cnd[1];
        break;
      }
    }
    if (TY == 0) return false;
    const size_t smem = cheb_bulk_smem(L.dims.Nx, KB, sizeof(V), TY, NA, prev == 1);
    // the shared-memory limit is raised once per kernel
    static const bool usable = [budget] {
      bool ok = true;
      for (const void *kern : {(const void *)k_cheb_bulk<T, V, KB, 0>, (const void *)k_cheb_bulk<T, V, KB, 1>,
                               (const void *)k_cheb_bulk<T, V, KB, 2>})
        ok = ok && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget) == cudaSuccess;
      if (!ok) cudaGetLastError();
      return ok;
    }();
    if (!usable) return false;
    const dim3 grid(count_launch(dim3((unsigned)(nb * ((L.dims.Ny + TY - 1) / TY)))));
    if (prev == 1)
      k_cheb_bulk<T, V, KB, 1><<<grid, BULK_T, smem, s>>>(L.d_coef32, r, zin, zout, L.dims, TY, NA, (T)c1,
                                                          (T)c2, status);
    else if (prev == 2)
      k_cheb_bulk<T, V, KB, 2><<<grid, BULK_T, smem, s>>>(L.d_coef32, r, zin, zout, L.dims, TY, NA, (T)c1,
                                                          (T)c2, status);
    else
      k_cheb_bulk<T, V, KB, 0><<<grid, BULK_T, smem, s>>>(L.d_coef32, r, zin, zout, L.dims, TY, NA, (T)c1,
                                                          (T)c2, status);
    return true;
  }
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::restrict_(const Level &f, const Level &c, const V *res, V *rc, int nb, cudaStream_t s) {
  k_restrict<T, V, KB><<<GRID_K(c.dims.N, (k_restrict<T, V, KB>)), TPB, 0, s>>>(res, rc, f.dims, c.dims, nb,
                                                                               make_tab<T>(f));
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::prolong_add(const Level &f, const Level &c, const V *zc, V *z, int nb, cudaStream_t s) {
  k_prolong_add<T, V, KB><<<GRID_K(f.dims.N, (k_prolong_add<T, V, KB>)), TPB, 0, s>>>(zc, z, f.dims, c.dims, nb,
                                                                                     make_tab<T>(f));
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::coarse_solve(const T *Ainv, const Level &c, Rhs<T, V> rc, V *zc, int nb, cudaStream_t s) {
  if (rc.full)
    k_coarse_solve<T, V, T, KB><<<GRID_K(c.dims.N, (k_coarse_solve<T, V, T, KB>)), TPB, 0, s>>>(
        Ainv, c.dims, nb, rc.full, rc.scale, zc);
  else
    k_coarse_solve<T, V, V, KB><<<GRID_K(c.dims.N, (k_coarse_solve<T, V, V, KB>)), TPB, 0, s>>>(
        Ainv, c.dims, nb, rc.part, nullptr, zc);
}

// The per-RHS parameter array in the arithmetic type T.
template <typename T>
const T *param_of(const double *d, const float *f);
template <>
inline const double *param_of<double>(const double *d, const float *) {
  return d;
}
template <>
inline const float *param_of<float>(const double *, const float *f) {
  return f;
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::update_xr(long long N, int nb, T *x, T *r, const V *p, const T *q, const double *alpha,
                              const float *alpha32, double *partial, int gx, const Level *smooth, double c0, V *z,
                              const float *scale, V *rv_out, cudaStream_t s, bool x_zero) {
  const Dims dd = flat_dims(N);
  const T *a = param_of<T>(alpha, alpha32);
  if (smooth)
    k_update_xr<T, V, KB, true><<<RED_GRID(N, (k_update_xr<T, V, KB, true>), (Lanes<T, KB>::LPN)), TPB, 0, s>>>(
        dd, nb, x, r, p, q, a, partial, invd_ptr<T>(*smooth), z, (T)c0, scale, rv_out, gx, x_zero ? 1 : 0);
  else
    k_update_xr<T, V, KB, false><<<RED_GRID(N, (k_update_xr<T, V, KB, false>), (Lanes<T, KB>::LPN)), TPB, 0, s>>>(
        dd, nb, x, r, p, q, a, partial, nullptr, nullptr, (T)0, nullptr, nullptr, gx, x_zero ? 1 : 0);
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::scale_to(long long N, int nb, const T *r, const float *scale, V *rv_out, cudaStream_t s) {
  k_scale_to<T, V, KB><<<GRID_K(N, (k_scale_to<T, V, KB>)), TPB, 0, s>>>(flat_dims(N), nb, r, scale, rv_out);
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::dot(long long N, int nb, const T *a, const T *b, double *partial, int gx, cudaStream_t s) {
  k_dot<T, T, KB><<<RED_GRID(N, (k_dot<T, T, KB>), (Lanes<T, KB>::LPN)), TPB, 0, s>>>(flat_dims(N), nb, a, b,
                                                                                     partial, gx);
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::dot_z(long long N, int nb, const T *a, const V *b, double *partial, int gx, cudaStream_t s) {
  k_dot<T, V, KB><<<RED_GRID(N, (k_dot<T, V, KB>), (Lanes<V, KB>::LPN)), TPB, 0, s>>>(flat_dims(N), nb, a, b,
                                                                                     partial, gx);
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::p_update(long long N, int nb, V *p, const V *z, const double *beta, const float *beta32,
                             cudaStream_t s) {
  k_p_update<T, V, KB><<<GRID_K(N, (k_p_update<T, V, KB>)), TPB, 0, s>>>(flat_dims(N), nb, p, z,
                                                                       param_of<T>(beta, beta32));
}

template <typename T, typename V, int KB>
void Ops<T, V, KB>::copy_z(long long N, int nb, V *dst, const V *src, cudaStream_t s) {
  cudaMemcpyAsync(dst, src, sizeof(V) * N * KB * nb, cudaMemcpyDeviceToDevice, s);
}

#define DC_OPS_INSTANTIATE(T, V)                                                                            \
  template struct Ops<T, V, 1>;                                                                             \
  template struct Ops<T, V, 2>;                                                                             \
  template struct Ops<T, V, 4>;                                                                             \
  template struct Ops<T, V, 8>;                                                                             \
  template struct Ops<T, V, 16>;                                                                            \
  template struct Ops<T, V, 32>;

}  // namespace dc
