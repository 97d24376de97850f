// Instantiation of the node kernels for the fp64 solve (T = V = double), the
// fp64 true-residual kernel, and the double-float refinement kernels of the
// mixed-precision solve (b - A x and x += d with fp32 pairs).
#include "dc_dfbits.h"
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


// ---------------------------------------------------------------- double-float refinement
// The refinement residual of the mixed solve in double-float arithmetic: every
// fp64 quantity is an unevaluated sum hi + lo of two fp32 numbers (about 48
// significant bits), so b - A x runs on the fp32 pipes instead of the fp64
// ones, which on this part issue 1/64 as fast.  Error-free transformations:
// Knuth's two-sum and the fused-multiply-add product error (Dekker, "A
// floating-point technique for extending the available precision", 1971).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (sh, sl) += (ph, pl), renormalised
__device__ __forceinline__ void df_acc(float &sh, float &sl, float ph, float pl) {
  float s, e;
  two_sum(sh, ph, s, e);
  e += sl + pl;
  sh = s + e;
  sl = e - (sh - s);
}

// Accurate dot product in the manner of Ogita, Rump and Oishi ("Accurate sum
// and dot product", SIAM J. Sci. Comput. 26, 2005; Dot2): the high parts of
// the products are summed with Knuth's error-free two-sum into s, and every
// low-order quantity (the products' exact rounding errors from an FMA, the
// cross terms w_hi v_lo and w_lo v_hi, the two-sum errors) into one plain
// fp32 sum c; s + c is the result.  Each term is w * v with w = wh + wl one
// coefficient of the node and v = vh + vl per lane.  Lane pairs go through the
// two-lane fp32 instructions; a - b is written fma(b, -1, a) (one instruction,
// the same rounding as the subtraction).
__device__ __forceinline__ void dot2_pair(float wh, float wl, float2 vh, float2 vl, float2 &s, float2 &c) {
  const float2 m1 = make_float2(-1.f, -1.f), kw = make_float2(wh, wh), kwl = make_float2(wl, wl),
               knw = make_float2(-wh, -wh);
  const float2 ph = __fmul2_rn(kw, vh);
  const float2 npe = __ffma2_rn(knw, vh, ph);  // -(wh vh - ph), exactly
  c = __ffma2_rn(kw, vl, c);
  c = __ffma2_rn(kwl, vh, c);
  c = __ffma2_rn(npe, m1, c);
  const float2 s1 = __fadd2_rn(s, ph);          // two-sum of s and ph
  const float2 bb = __ffma2_rn(s, m1, s1);      // s1 - s
  const float2 ea = __ffma2_rn(__ffma2_rn(bb, m1, s1), m1, s);  // s - (s1 - bb)
  const float2 eb = __ffma2_rn(bb, m1, ph);     // ph - bb
  c = __fadd2_rn(c, __fadd2_rn(ea, eb));
  s = s1;
}

__device__ __forceinline__ void dot2_one(float wh, float wl, float vh, float vl, float &s, float &c) {
  const float ph = wh * vh;
  const float npe = fmaf(-wh, vh, ph);
  c = fmaf(wh, vl, c);
  c = fmaf(wl, vh, c);
  c -= npe;
  float s1, e;
  two_sum(s, ph, s1, e);
  c += e;
  s = s1;
}

template <int W>
__device__ __forceinline__ void dot2_terms(float wh, float wl, const Vec<float, W> &vh, const Vec<float, W> &vl,
                                           Vec<float, W> &s, Vec<float, W> &c) {
  if constexpr (W % 2 == 0) {
#pragma unroll
    for (int p = 0; p < W / 2; ++p) {
      float2 sp = pair(s, p), cp = pair(c, p);
      dot2_pair(wh, wl, pair(vh, p), pair(vl, p), sp, cp);
      s.a[2 * p] = sp.x;
      s.a[2 * p + 1] = sp.y;
      c.a[2 * p] = cp.x;
      c.a[2 * p + 1] = cp.y;
    }
  } else {
#pragma unroll
    for (int e = 0; e < W; ++e) dot2_one(wh, wl, vh.a[e], vl.a[e], s.a[e], c.a[e]);
  }
}

// hi = fp32(v), lo = fp32(v - hi) with fp64 instructions: a call of its own, so
// that the compiler does not predicate these slow instructions into the common
// path of split_one.
__device__ __noinline__ void split_fp64(double v, float &h, float &l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

// Double-float split of one value: by bits (split_df_bits) where that covers it.
__device__ __forceinline__ void split_one(double v, float &h, float &l) {
  if (__builtin_expect(split_df_bits(v, h, l), 1)) return;
  split_fp64(v, h, l);
}

// (hi, lo) = double-float split of a; r32, if given, also receives hi (the fp32
// copy of a).  VEC: two elements per thread by 16-byte loads and 8-byte stores
// (every pointer aligned for that).
template <bool VEC>
__global__ void k_split_df(const double *__restrict__ a, long long n, float *__restrict__ hi, float *__restrict__ lo,
                           float *__restrict__ r32) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (VEC) {
    const double2 *a2 = reinterpret_cast<const double2 *>(a);
    float2 *h2 = reinterpret_cast<float2 *>(hi), *l2 = reinterpret_cast<float2 *>(lo);
    float2 *r2 = reinterpret_cast<float2 *>(r32);
    for (long long i = i0; i < n / 2; i += stride) {
      const double2 v = a2[i];
      float2 h, l;
      split_one(v.x, h.x, l.x);
      split_one(v.y, h.y, l.y);
      h2[i] = h;
      l2[i] = l;
      if (r32) r2[i] = h;
    }
    if ((n & 1) && i0 == 0) {
      float h, l;
      split_one(a[n - 1], h, l);
      hi[n - 1] = h;
      lo[n - 1] = l;
      if (r32) r32[n - 1] = h;
    }
  } else {
    for (long long i = i0; i < n; i += stride) {
      float h, l;
      split_one(a[i], h, l);
      hi[i] = h;
      lo[i] = l;
      if (r32) r32[i] = h;
    }
  }
}

__global__ void k_coef_split_df(const Coef64 *__restrict__ c, long long n, Coef32 *__restrict__ hi,
                                Coef32 *__restrict__ lo) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const Coef64 v = c[i];
    Coef32 h{(float)v.cx, (float)v.cy, (float)v.cz, (float)v.d};
    Coef32 l{(float)(v.cx - (double)h.cx), (float)(v.cy - (double)h.cy), (float)(v.cz - (double)h.cz),
             (float)(v.d - (double)h.d)};
    hi[i] = h;
    lo[i] = l;
  }
}

// r32 = (float)(b - A x) for active RHS (0 otherwise), per-block partials of |r|^2
template <int KB>
__global__ void __launch_bounds__(TPB) k_ir_residual_df(const Coef32 *__restrict__ ch, const Coef32 *__restrict__ cl,
                                                        const float *__restrict__ bh, const float *__restrict__ bl,
                                                        const float *__restrict__ xh, const float *__restrict__ xl,
                                                        float *__restrict__ r32, Dims d, int nb,
                                                        const int *__restrict__ active, double *__restrict__ partial,
                                                        int gs) {
  using T = float;
  constexpr int W = Lanes<T, KB>::W;
  sweep_reduce<T, KB, W, true>(d.N, nb, partial, gs, [&](int b, int n, int q, long long t, T(&acc)[W]) {
    int i, j, k;
    node_ijk(n, d, i, j, k);
    const bool hx = i > 0, px = i + 1 < d.Nx, hy = j > 0, py = j + 1 < d.Ny, hz = k > 0, pz = k + 1 < d.Nz;
    const int sy = d.Nx, sz = d.Nx * d.Ny;
    const Coef32 c0h = ch[n], c0l = cl[n];
    // couplings (hi, lo), zero off the mesh; neighbour element offsets (0 off the mesh)
    const float wh[6] = {px ? c0h.cx : 0.f, hx ? ch[n - 1].cx : 0.f, py ? c0h.cy : 0.f,
                         hy ? ch[hy ? n - sy : n].cy : 0.f, pz ? c0h.cz : 0.f, hz ? ch[hz ? n - sz : n].cz : 0.f};
    const float wl[6] = {px ? c0l.cx : 0.f, hx ? cl[n - 1].cx : 0.f, py ? c0l.cy : 0.f,
                         hy ? cl[hy ? n - sy : n].cy : 0.f, pz ? c0l.cz : 0.f, hz ? cl[hz ? n - sz : n].cz : 0.f};
    const long long off[6] = {px ? (long long)KB : 0,       hx ? -(long long)KB : 0,
                              py ? (long long)sy * KB : 0,  hy ? -(long long)sy * KB : 0,
                              pz ? (long long)sz * KB : 0,  hz ? -(long long)sz * KB : 0};
    const Vec<T, W> b0h = ld<T, W>(bh + t), b0l = ld<T, W>(bl + t);
    const Vec<T, W> x0h = ld<T, W>(xh + t), x0l = ld<T, W>(xl + t);
    // sum (s, c): s = b_hi, c = b_lo; the centre term enters with negated coefficients
    Vec<T, W> sv = b0h, cv = b0l;
    dot2_terms<W>(-c0h.d, -c0l.d, x0h, x0l, sv, cv);
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const Vec<T, W> vh = ld<T, W>(xh + t + off[m]), vl = ld<T, W>(xl + t + off[m]);
      dot2_terms<W>(wh[m], wl[m], vh, vl, sv, cv);
    }
    Vec<T, W> out;
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const float rv = sv.a[e] + cv.a[e];
      acc[e] += rv * rv;
      out.a[e] = active[b * KB + q * W + e] ? rv : 0.0f;
    }
    st<T, W>(r32 + t, out);
  });
}

// (xh, xl) += d, exactly rounded to double-float
__global__ void __launch_bounds__(TPB) k_ir_accumulate_df(long long n, float *__restrict__ xh, float *__restrict__ xl,
                                                          const float *__restrict__ d32) {
  for (long long i = (long long)blockIdx.x * TPB + threadIdx.x; i < n; i += (long long)gridDim.x * TPB) {
    float h = xh[i], l = xl[i];
    df_acc(h, l, d32[i], 0.0f);
    xh[i] = h;
    xl[i] = l;
  }
}

// (xh, xl) = 0 + d: what k_ir_accumulate_df gives from a zero iterate (hi = 0 + d, lo = +0), without
// reading the zeros
__global__ void __launch_bounds__(TPB) k_ir_set_df(long long n, float *__restrict__ xh, float *__restrict__ xl,
                                                   const float *__restrict__ d32) {
  for (long long i = (long long)blockIdx.x * TPB + threadIdx.x; i < n; i += (long long)gridDim.x * TPB) {
    xh[i] = __fadd_rn(0.0f, d32[i]);
    xl[i] = 0.0f;
  }
}

}  // namespace

DC_OPS_INSTANTIATE(double, double)

template <int KB>
void ir_residual(const Level &L, const double *b, const double *x, double *r64, float *r32, int nb,
                 const int *active, double *partial, int gx, cudaStream_t s) {
  k_ir_residual<KB><<<RED_GRID(L.dims.N, k_ir_residual<KB>, (Lanes<double, KB>::LPN)), TPB, 0, s>>>(
      L.d_coef64, b, x, r64, r32, L.dims, nb, active, partial, gx);
}


void split_df(const double *a, long long n, float *hi, float *lo, float *r32, cudaStream_t s) {
  const bool vec = ((uintptr_t)a % 16 == 0) && ((uintptr_t)hi % 8 == 0) && ((uintptr_t)lo % 8 == 0) &&
                   ((uintptr_t)r32 % 8 == 0);
  if (vec)
    k_split_df<true><<<count_launch(grid_flat(n / 2 + 1, g_n_sm)), TPB, 0, s>>>(a, n, hi, lo, r32);
  else
    k_split_df<false><<<count_launch(grid_flat(n, g_n_sm)), TPB, 0, s>>>(a, n, hi, lo, r32);
}

void coef_split_df(const Level &L, Coef32 *hi, Coef32 *lo, cudaStream_t s) {
  k_coef_split_df<<<count_launch(grid_flat(L.dims.N, g_n_sm)), TPB, 0, s>>>(L.d_coef64, L.dims.N, hi, lo);
}

template <int KB>
void ir_residual_df(const Level &L, const Coef32 *ch, const Coef32 *cl, const float *bh, const float *bl,
                    const float *xh, const float *xl, float *r32, int nb, const int *active, double *partial, int gx,
                    cudaStream_t s) {
  k_ir_residual_df<KB><<<RED_GRID(L.dims.N, k_ir_residual_df<KB>, (Lanes<float, KB>::LPN)), TPB, 0, s>>>(
      ch, cl, bh, bl, xh, xl, r32, L.dims, nb, active, partial, gx);
}

void ir_accumulate_df(long long n, float *xh, float *xl, const float *d32, cudaStream_t s) {
  k_ir_accumulate_df<<<count_launch(grid_flat(n, g_n_sm)), TPB, 0, s>>>(n, xh, xl, d32);
}

void ir_set_df(long long n, float *xh, float *xl, const float *d32, cudaStream_t s) {
  k_ir_set_df<<<count_launch(grid_flat(n, g_n_sm)), TPB, 0, s>>>(n, xh, xl, d32);
}

// resident blocks per SM of the fp64 reduction kernels the mixed solve also runs
template <int KB>
int ir_blocks_per_sm() {
  return std::max({resident_blocks((const void *)k_ir_residual<KB>), resident_blocks((const void *)k_ir_residual_df<KB>),
                   resident_blocks((const void *)k_dot<double, double, KB>)});
}

#define DC_INST_IR(KB)                                                                                       \
  template void ir_residual<KB>(const Level &, const double *, const double *, double *, float *, int,      \
                                const int *, double *, int, cudaStream_t);                                  \
  template int ir_blocks_per_sm<KB>();                                                                       \
  template void ir_residual_df<KB>(const Level &, const Coef32 *, const Coef32 *, const float *, const float *,    \
                                   const float *, const float *, float *, int, const int *, double *, int,         \
                                   cudaStream_t);
DC_INST_IR(1) DC_INST_IR(2) DC_INST_IR(4) DC_INST_IR(8) DC_INST_IR(16) DC_INST_IR(32)
#undef DC_INST_IR

}  // namespace dc
