// krylov.cu -- level-1 kernels, thick-restart Lanczos, plain Lanczos, the
// dynamical-structure-factor recursion and the continued fraction.
//
// Replaces my_l1_blas.f90:5-25 (my_zaxpy, my_zdscal), the BLAS calls zdotc /
// dznrm2 / zcopy / zscal / zgemm of eigen_solver.f90:69-261 and
// lanczos.f90:50-152, calcu_Sq_a + calcu_DSF_wavevector
// (get_expectation_values.f90:281-605) and DSFLan (source_DSFLan/main.f90).
//
// Reductions are deterministic: a fixed grid of kRedBlocks blocks each reduce
// a fixed grid-stride slice in a fixed tree order into a partial, and one
// block reduces the partials in a fixed order.  All Lanczos scalars (alpha,
// beta, overlaps) stay in device memory, so a Lanczos cycle is a chain of
// kernel launches with no host round trip; the host reads the scalars once
// per restart to solve the NOM x NOM Ritz problem.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <string>

#include "hosteig.h"
#include "qs3g_device.cuh"
#include "qs3g_internal.cuh"
#include "eft.cuh"
#include <chrono>

#include "krylov.h"

namespace qs3g {

// ================================================================ reductions
namespace {
constexpr int kRedThreads = 256;

template <class T>
struct Ld;
template <>
struct Ld<double2> {
  static __device__ __forceinline__ double re(const double2& v) { return v.x; }
  static __device__ __forceinline__ double im(const double2& v) { return v.y; }
};
template <>
struct Ld<float2> {
  static __device__ __forceinline__ double re(const float2& v) { return (double)v.x; }
  static __device__ __forceinline__ double im(const float2& v) { return (double)v.y; }
};

// part[b] = sum over the block's slice of conj(x_i) y_i
template <class T>
__global__ void __launch_bounds__(kRedThreads) k_dot_part(const T* __restrict__ x, const T* __restrict__ y,
                                                          int64_t n, double2* part) {
  __shared__ double2 sh[kRedThreads];
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T a = x[i], b = y[i];
    const double ar = Ld<T>::re(a), ai = Ld<T>::im(a), br = Ld<T>::re(b), bi = Ld<T>::im(b);
    acc.x = fma(ar, br, fma(ai, bi, acc.x));
    acc.y = fma(ar, bi, fma(-ai, br, acc.y));
  }
  const double2 s = block_sum2(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// part[b] = sum |x_i|^2
template <class T>
__global__ void __launch_bounds__(kRedThreads) k_nrm_part(const T* __restrict__ x, int64_t n, double2* part) {
  __shared__ double2 sh[kRedThreads];
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T a = x[i];
    const double ar = Ld<T>::re(a), ai = Ld<T>::im(a);
    acc.x = fma(ar, ar, fma(ai, ai, acc.x));
  }
  const double2 s = block_sum2(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// out = sum of np partials (mode 0: complex; 1: (sqrt(real), real); 2: real)
__global__ void __launch_bounds__(kRedThreads) k_red_final(const double2* part, int np, double2* out, int mode) {
  __shared__ double2 sh[kRedThreads];
  double2 acc = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    acc.x += part[i].x;
    acc.y += part[i].y;
  }
  const double2 s = block_sum2(acc, sh);
  if (threadIdx.x == 0) {
    if (mode == 1) *out = make_double2(sqrt(s.x), s.x);
    else if (mode == 2) *out = make_double2(s.x, 0.0);
    else *out = s;
  }
}

// ---------------------------------------------------------------- level-1 updates
// x *= 1/s.x  (my_zdscal with a = 1/beta, eigen_solver.f90:101)
template <class T>
__global__ void k_scale_inv(T* x, int64_t n, const double2* s) {
  const double inv = 1.0 / s->x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T v = x[i];
    v.x = (decltype(v.x))((double)v.x * inv);
    v.y = (decltype(v.y))((double)v.y * inv);
    x[i] = v;
  }
}

// w = q - a*v - b*u   (a complex or its real part, b real; u may be null)
template <class T>
__global__ void k_lanczos_w(T* w, const T* q, const T* __restrict__ v, const T* __restrict__ u, int64_t n, const double2* a, const double2* b,
                            int real_alpha) {
  const double ar = a->x, ai = real_alpha ? 0.0 : a->y;
  const double br = u ? b->x : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T qv = q[i], vv = v[i];
    double re = (double)qv.x - (ar * (double)vv.x - ai * (double)vv.y);
    double im = (double)qv.y - (ar * (double)vv.y + ai * (double)vv.x);
    if (u) {
      const T uv = u[i];
      re -= br * (double)uv.x;
      im -= br * (double)uv.y;
    }
    T o;
    o.x = (decltype(o.x))re;
    o.y = (decltype(o.y))im;
    w[i] = o;
  }
}

// y += a*x  (my_zaxpy, my_l1_blas.f90:5-14) with a from device memory, a_sign applied
template <class T>
__global__ void k_axpy(T* __restrict__ y, const T* __restrict__ x, int64_t n, const double2* a, double sgn) {
  const double ar = sgn * a->x, ai = sgn * a->y;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T xv = x[i];
    T yv = y[i];
    yv.x = (decltype(yv.x))((double)yv.x + (ar * (double)xv.x - ai * (double)xv.y));
    yv.y = (decltype(yv.y))((double)yv.y + (ar * (double)xv.y + ai * (double)xv.x));
    y[i] = yv;
  }
}

// ---------------------------------------------------------------- block GEMV for reorthogonalisation
// part[c*nb + b] = sum over slice of conj(V[:,c]) w   for c < ncols (chunks of 8 columns)
// RE: real vectors two rows per slot -- only the real part is accumulated
template <class T, bool RE>
__global__ void __launch_bounds__(kRedThreads) k_gemv_h_part(const T* __restrict__ V, int64_t ldv, int ncols,
                                                             const T* __restrict__ w, int64_t n, double2* part) {
  __shared__ double2 sh[kRedThreads];
  for (int c0 = 0; c0 < ncols; c0 += 8) {
    double2 acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = make_double2(0.0, 0.0);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const T b = w[i];
      const double br = Ld<T>::re(b), bi = Ld<T>::im(b);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (c0 + k < ncols) {
          const T a = V[(int64_t)(c0 + k) * ldv + i];
          const double ar = Ld<T>::re(a), ai = Ld<T>::im(a);
          acc[k].x = fma(ar, br, fma(ai, bi, acc[k].x));
          if constexpr (!RE) acc[k].y = fma(ar, bi, fma(-ai, br, acc[k].y));
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (c0 + k < ncols) {
        const double2 s = block_sum2(acc[k], sh);
        if (threadIdx.x == 0) part[(size_t)(c0 + k) * gridDim.x + blockIdx.x] = s;
        __syncthreads();
      }
    }
  }
}

// out[c] = sum_b part[c*nb + b]: one block per column, fixed-order tree
// (real != 0: the imaginary part is dropped)
__global__ void __launch_bounds__(kRedThreads) k_gemv_final(const double2* part, int nb, int ncols, double2* out,
                                                            int real) {
  __shared__ double2 sh[kRedThreads];
  const int c = blockIdx.x;
  double2 acc = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    acc.x += part[(size_t)c * nb + i].x;
    acc.y += part[(size_t)c * nb + i].y;
  }
  const double2 s = block_sum2(acc, sh);
  if (threadIdx.x == 0) out[c] = real ? make_double2(s.x, 0.0) : s;
}

// w -= V[:, :ncols] * coef   (coef from device memory; RE: coef real)
template <class T, bool RE>
__global__ void k_gemv_sub(const T* __restrict__ V, int64_t ldv, int ncols, const double2* __restrict__ coef,
                           T* __restrict__ w, int64_t n) {
  __shared__ double2 c[128];
  for (int k = threadIdx.x; k < ncols; k += blockDim.x) c[k] = coef[k];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T wv = w[i];
    double re = (double)wv.x, im = (double)wv.y;
    for (int k = 0; k < ncols; ++k) {
      const T a = V[(int64_t)k * ldv + i];
      if constexpr (RE) {
        re -= c[k].x * (double)a.x;
        im -= c[k].x * (double)a.y;
      } else {
        re -= c[k].x * (double)a.x - c[k].y * (double)a.y;
        im -= c[k].x * (double)a.y + c[k].y * (double)a.x;
      }
    }
    T o;
    o.x = (decltype(o.x))re;
    o.y = (decltype(o.y))im;
    w[i] = o;
  }
}

// In-place restart V[:, :nok] = V[:, :nom] * C (zgemm + zcopy, eigen_solver.f90:147-149).
// 32 rows per block; the rows' nom inputs are staged in shared memory first.
// RE: C real.
template <class T, bool RE>
__global__ void __launch_bounds__(256) k_restart(T* V, int64_t ldv, int nom, int nok, const double2* __restrict__ C,
                                                 int64_t n) {
  extern __shared__ double2 sm[];
  double2* tile = sm;                 // [nom][32]
  double2* cs = sm + (size_t)nom * 32;  // [nok][nom] column-major C(nom x nok)
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  for (int k = threadIdx.x; k < nom * nok; k += blockDim.x) cs[k] = C[k];
  for (int k = threadIdx.x; k < nom * 32; k += blockDim.x) {
    const int col = k / 32, r = k % 32;
    const int64_t i = r0 + r;
    double2 v = make_double2(0.0, 0.0);
    if (i < n) {
      const T a = V[(int64_t)col * ldv + i];
      v = make_double2((double)a.x, (double)a.y);
    }
    tile[k] = v;
  }
  __syncthreads();
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;  // 8 column groups
  const int64_t i = r0 + r;
  if (i < n) {
    for (int oc = g; oc < nok; oc += 8) {
      double re = 0.0, im = 0.0;
      for (int j = 0; j < nom; ++j) {
        const double2 a = tile[j * 32 + r], c = cs[(size_t)oc * nom + j];
        if constexpr (RE) {
          re = fma(a.x, c.x, re);
          im = fma(a.y, c.x, im);
        } else {
          re = fma(a.x, c.x, fma(-a.y, c.y, re));
          im = fma(a.x, c.y, fma(a.y, c.x, im));
        }
      }
      T o;
      o.x = (decltype(o.x))re;
      o.y = (decltype(o.y))im;
      V[(int64_t)oc * ldv + i] = o;
    }
  }
}

template <class T>
__global__ void k_copy_conv(T* __restrict__ y, const double2* __restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T o;
    o.x = (decltype(o.x))x[i].x;
    o.y = (decltype(o.y))x[i].y;
    y[i] = o;
  }
}

__global__ void k_f32_to_f64(double2* __restrict__ y, const float2* __restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = make_double2((double)x[i].x, (double)x[i].y);
}

// Seeded start vector: psi(l) = (u_{2l} - 0.5, u_{2l+1} - 0.5), u_k = mix64(seed + (k+1)*golden)
// >> 11 * 2^-53 (SplitMix64 finaliser), replacing random_number at eigen_solver.f90:92-96.
__device__ __forceinline__ double su(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * 0x1.0p-53;
}
template <class T>
__global__ void k_random_start(T* x, int64_t n, uint64_t seed) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T o;
    o.x = (decltype(o.x))(su(seed, 2 * (uint64_t)i) - 0.5);
    o.y = (decltype(o.y))(su(seed, 2 * (uint64_t)i + 1) - 0.5);
    x[i] = o;
  }
}

// w = q - e * v  (residual), FP64
// w = q - e v (w may be q)
__global__ void k_residual(double2* w, const double2* q, const double2* __restrict__ v, int64_t n, double e) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = make_double2(q[i].x - e * v[i].x, q[i].y - e * v[i].y);
}

// ---------------------------------------------------------------- complex(4) vectors on the FP32 pipe
// GB300 issues FP64 at 1/64 of the FP32 rate, and float <-> double conversions
// go through the FP64 pipe too, so complex(4) Krylov vectors are processed
// with FP32 instructions only while keeping FP64-class reductions:
//  * a product of two floats is split exactly into p + e (p = a*b rounded,
//    e = fma(a, b, -p)), and sums are carried as unevaluated float pairs
//    (hi, lo) with the TwoSum error-free transformation, so a thread's partial
//    dot product is accurate to about 2^-44 relative before it is widened to
//    FP64 for the fixed-order block reduction;
//  * FP64 scalars (alpha, beta, overlaps, Ritz coefficients) are split into
//    hi + lo floats, so updates round only once, to the FP32 result.
__global__ void __launch_bounds__(kRedThreads) k_dot_part32(const float2* __restrict__ x, const float2* __restrict__ y,
                                                            int64_t n, double2* part) {
  __shared__ double2 sh[kRedThreads];
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = x[i], b = y[i];
    df_add_prod(rh, rl, a.x, b.x);
    df_add_prod(rh, rl, a.y, b.y);
    df_add_prod(ih, il, a.x, b.y);
    df_add_prod(ih, il, -a.y, b.x);
  }
  const double2 s = block_sum2(make_double2((double)rh + (double)rl, (double)ih + (double)il), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedThreads) k_nrm_part32(const float2* __restrict__ x, int64_t n, double2* part) {
  __shared__ double2 sh[kRedThreads];
  float rh = 0.f, rl = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = x[i];
    df_add_prod(rh, rl, a.x, a.x);
    df_add_prod(rh, rl, a.y, a.y);
  }
  const double2 s = block_sum2(make_double2((double)rh + (double)rl, 0.0), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}


// w = q - a v - b u with a, b split into float pairs (one rounding to FP32)
__global__ void k_lanczos_w32(float2* w, const float2* q, const float2* __restrict__ v, const float2* __restrict__ u,
                              int64_t n, const double2* a, const double2* b, int real_alpha) {
  const float2 ar = split(a->x), ai = split(real_alpha ? 0.0 : a->y), br = split(u ? b->x : 0.0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 qv = q[i], vv = v[i];
    float re = qv.x, im = qv.y;
    // lo parts first, then hi parts
    re = fmaf(-ar.y, vv.x, re); re = fmaf(ai.y, vv.y, re);
    im = fmaf(-ar.y, vv.y, im); im = fmaf(-ai.y, vv.x, im);
    if (u) {
      const float2 uv = u[i];
      re = fmaf(-br.y, uv.x, re); im = fmaf(-br.y, uv.y, im);
      re = fmaf(-br.x, uv.x, re); im = fmaf(-br.x, uv.y, im);
    }
    re = fmaf(-ar.x, vv.x, re); re = fmaf(ai.x, vv.y, re);
    im = fmaf(-ar.x, vv.y, im); im = fmaf(-ai.x, vv.x, im);
    w[i] = make_float2(re, im);
  }
}

__global__ void k_scale_inv32(float2* x, int64_t n, const double2* s) {
  const float2 inv = split(1.0 / s->x);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = x[i];
    x[i] = make_float2(fmaf(v.x, inv.x, v.x * inv.y), fmaf(v.y, inv.x, v.y * inv.y));
  }
}

// y += sgn * a * x
__global__ void k_axpy32(float2* __restrict__ y, const float2* __restrict__ x, int64_t n, const double2* a, double sgn) {
  const float2 ar = split(sgn * a->x), ai = split(sgn * a->y);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 xv = x[i];
    float2 yv = y[i];
    float re = yv.x, im = yv.y;
    re = fmaf(ar.y, xv.x, re); re = fmaf(-ai.y, xv.y, re);
    im = fmaf(ar.y, xv.y, im); im = fmaf(ai.y, xv.x, im);
    re = fmaf(ar.x, xv.x, re); re = fmaf(-ai.x, xv.y, re);
    im = fmaf(ar.x, xv.y, im); im = fmaf(ai.x, xv.x, im);
    y[i] = make_float2(re, im);
  }
}

// w -= V[:, :ncols] * coef, coef split into float pairs in shared memory (RE: coef real)
template <bool RE>
__global__ void k_gemv_sub32(const float2* __restrict__ V, int64_t ldv, int ncols, const double2* __restrict__ coef,
                             float2* __restrict__ w, int64_t n) {
  __shared__ float4 c[128];  // (re hi, re lo, im hi, im lo)
  for (int k = threadIdx.x; k < ncols; k += blockDim.x) {
    const float2 r = split(coef[k].x), m = split(coef[k].y);
    c[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 wv = w[i];
    float re = wv.x, im = wv.y, rlo = 0.f, ilo = 0.f;
    for (int k = 0; k < ncols; ++k) {
      const float2 a = V[(int64_t)k * ldv + i];
      const float4 ck = c[k];
      rlo = fmaf(-ck.y, a.x, rlo);
      ilo = fmaf(-ck.y, a.y, ilo);
      re = fmaf(-ck.x, a.x, re);
      im = fmaf(-ck.x, a.y, im);
      if constexpr (!RE) {
        rlo = fmaf(ck.w, a.y, rlo);
        ilo = fmaf(-ck.w, a.x, ilo);
        re = fmaf(ck.z, a.y, re);
        im = fmaf(-ck.z, a.x, im);
      }
    }
    w[i] = make_float2(re + rlo, im + ilo);
  }
}

// In-place restart for complex(4): double-float accumulation, split C (RE: C real).
template <bool RE>
__global__ void __launch_bounds__(256) k_restart32(float2* V, int64_t ldv, int nom, int nok,
                                                   const double2* __restrict__ C, int64_t n) {
  extern __shared__ float4 sm4[];
  float4* cs = sm4;                                       // [nok][nom] split C
  float2* tile = reinterpret_cast<float2*>(sm4 + (size_t)nom * nok);  // [nom][32]
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  for (int k = threadIdx.x; k < nom * nok; k += blockDim.x) {
    const float2 r = split(C[k].x), m = split(C[k].y);
    cs[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  for (int k = threadIdx.x; k < nom * 32; k += blockDim.x) {
    const int col = k / 32, r = k % 32;
    const int64_t i = r0 + r;
    tile[k] = (i < n) ? V[(int64_t)col * ldv + i] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int64_t i = r0 + r;
  if (i < n) {
    for (int oc = g; oc < nok; oc += 8) {
      float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
      for (int j = 0; j < nom; ++j) {
        const float2 a = tile[j * 32 + r];
        const float4 c = cs[(size_t)oc * nom + j];
        if constexpr (RE) {
          df_add_prod(rh, rl, a.x, c.x);
          df_add_prod(ih, il, a.y, c.x);
          rl = fmaf(a.x, c.y, rl);
          il = fmaf(a.y, c.y, il);
        } else {
          df_add_prod(rh, rl, a.x, c.x);
          df_add_prod(rh, rl, -a.y, c.z);
          df_add_prod(ih, il, a.x, c.z);
          df_add_prod(ih, il, a.y, c.x);
          rl = fmaf(a.x, c.y, fmaf(-a.y, c.w, rl));
          il = fmaf(a.x, c.w, fmaf(a.y, c.y, il));
        }
      }
      V[(int64_t)oc * ldv + i] = make_float2(rh + rl, ih + il);
    }
  }
}

// ---------------------------------------------------------------- complex(8) vectors on the FP32 pipe
// The same double-float arithmetic for vectors STORED in FP64 (the fast FP64
// mode and the refinement phase of the complex(4) mode).  A double is split
// into hi + lo floats with integer instructions only (the FP64 pipe, which
// also carries double <-> float conversions, would be the bottleneck again):
// hi keeps the leading 24 significant bits (truncated), lo the remaining 29
// rounded to 23, so hi + lo equals the double to 2^-47 relative, unbiased.  Magnitudes below 2^-80 lose
// lo, below 2^-126 become 0; such entries are far below the rounding level of
// a normalised Krylov vector.  Results are widened back to FP64 once per
// element.
__global__ void __launch_bounds__(kRedThreads) k_dot_part64e(const double2* __restrict__ x,
                                                             const double2* __restrict__ y, int64_t n,
                                                             double2* part) {
  __shared__ double2 sh[kRedThreads];
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = x[i], b = y[i];
    const float2 ar = dsplit(a.x), ai = dsplit(a.y), br = dsplit(b.x), bi = dsplit(b.y);
    df_fma(rh, rl, ar, br);
    df_fma(rh, rl, ai, bi);
    df_fma(ih, il, ar, bi);
    df_fma(ih, il, fneg2(ai), br);
  }
  const double2 s = block_sum2(make_double2(djoin(rh, rl), djoin(ih, il)), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedThreads) k_nrm_part64e(const double2* __restrict__ x, int64_t n,
                                                             double2* part) {
  __shared__ double2 sh[kRedThreads];
  float rh = 0.f, rl = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = x[i];
    const float2 ar = dsplit(a.x), ai = dsplit(a.y);
    df_fma(rh, rl, ar, ar);
    df_fma(rh, rl, ai, ai);
  }
  const double2 s = block_sum2(make_double2(djoin(rh, rl), 0.0), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}


// Overlaps conj(V[:, c]) . w for c < ncols.  Grid (column groups of 4,
// row chunks): block (g, r) accumulates columns 4g..4g+3 over the rows of
// chunk r (threads stride the chunk), four independent double-float chains
// per thread at about 40 registers, so many warps hide the load latency.
// The column groups of one chunk are adjacent in launch order and read the
// same slice of w, which L2 serves after the first.  Each (column, chunk)
// partial is a fixed-order block reduction: part[c * nchunk + r].
constexpr int kGemvChunks = 304;

template <class T, bool RE>
__global__ void __launch_bounds__(256) k_gemv_h3(const T* __restrict__ V, int64_t ldv, int ncols,
                                                 const T* __restrict__ w, int64_t n, int64_t rows, double2* part) {
  __shared__ double2 sh[256];
  const int c0 = 4 * blockIdx.x;
  const int nc = min(4, ncols - c0);
  const int64_t r0 = (int64_t)blockIdx.y * rows;
  const int64_t r1 = min(n, r0 + rows);
  float acc[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k) acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.f;
  for (int64_t i = r0 + threadIdx.x; i < r1; i += 256) {
    const float4 b = SplitLd<T>::ld(w[i]);
    const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
    T a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < nc) a[k] = V[(int64_t)(c0 + k) * ldv + i];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k < nc) {
        const float4 av = SplitLd<T>::ld(a[k]);
        const float2 ar = make_float2(av.x, av.y), ai = make_float2(av.z, av.w);
        df_fma(acc[k][0], acc[k][1], ar, br);
        df_fma(acc[k][0], acc[k][1], ai, bi);
        if constexpr (!RE) {  // real vectors: the imaginary part is not needed
          df_fma(acc[k][2], acc[k][3], ar, bi);
          df_fma(acc[k][2], acc[k][3], fneg2(ai), br);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (k < nc) {
      const double2 s = block_sum2(make_double2(djoin(acc[k][0], acc[k][1]), djoin(acc[k][2], acc[k][3])), sh);
      if (threadIdx.x == 0) part[(size_t)(c0 + k) * gridDim.y + blockIdx.y] = s;
      __syncthreads();
    }
  }
}

// w -= V[:, :ncols] * coef: the sum over columns in double-float, one FP64
// subtraction per component at the end (RE: coef real)
template <bool RE>
__global__ void k_gemv_sub64e(const double2* __restrict__ V, int64_t ldv, int ncols, const double2* __restrict__ coef,
                              double2* __restrict__ w, int64_t n) {
  __shared__ float4 c[128];  // (re hi, re lo, im hi, im lo)
  for (int k = threadIdx.x; k < ncols; k += blockDim.x) {
    const float2 r = dsplit(coef[k].x), m = dsplit(coef[k].y);
    c[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int k = 0; k < ncols; ++k) {
      const double2 a = V[(int64_t)k * ldv + i];
      const float2 ar = dsplit(a.x), ai = dsplit(a.y);
      const float4 ck = c[k];
      const float2 cr = make_float2(ck.x, ck.y), ci = make_float2(ck.z, ck.w);
      df_fma(rh, rl, cr, ar);
      df_fma(ih, il, cr, ai);
      if constexpr (!RE) {
        df_fma(rh, rl, fneg2(ci), ai);
        df_fma(ih, il, ci, ar);
      }
    }
    double2 wv = w[i];
    wv.x -= djoin(rh, rl);
    wv.y -= djoin(ih, il);
    w[i] = wv;
  }
}

// In-place restart V[:, :nok] = V[:, :nom] * C with split inputs in shared memory (RE: C real).
template <bool RE>
__global__ void __launch_bounds__(256) k_restart64e(double2* V, int64_t ldv, int nom, int nok,
                                                    const double2* __restrict__ C, int64_t n) {
  extern __shared__ float4 smx[];
  float4* cs = smx;                          // [nok][nom] split C
  float4* tile = smx + (size_t)nom * nok;    // [nom][32] split V rows
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  for (int k = threadIdx.x; k < nom * nok; k += blockDim.x) {
    const float2 r = dsplit(C[k].x), m = dsplit(C[k].y);
    cs[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  for (int k = threadIdx.x; k < nom * 32; k += blockDim.x) {
    const int col = k / 32, r = k % 32;
    const int64_t i = r0 + r;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < n) {
      const double2 a = V[(int64_t)col * ldv + i];
      const float2 ar = dsplit(a.x), ai = dsplit(a.y);
      v = make_float4(ar.x, ar.y, ai.x, ai.y);
    }
    tile[k] = v;
  }
  __syncthreads();
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int64_t i = r0 + r;
  if (i < n) {
    for (int oc = g; oc < nok; oc += 8) {
      float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
      for (int j = 0; j < nom; ++j) {
        const float4 a = tile[j * 32 + r];
        const float4 c = cs[(size_t)oc * nom + j];
        const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
        const float2 cr = make_float2(c.x, c.y), ci = make_float2(c.z, c.w);
        df_fma(rh, rl, ar, cr);
        df_fma(ih, il, ai, cr);
        if constexpr (!RE) {
          df_fma(rh, rl, fneg2(ai), ci);
          df_fma(ih, il, ar, ci);
        }
      }
      V[(int64_t)oc * ldv + i] = make_double2(djoin(rh, rl), djoin(ih, il));
    }
  }
}

// Real vectors two rows per complex slot: out[r] = Re in[r] for r < D, and a
// zero pad when D is odd; unpack writes (x[r], 0).
__global__ void k_pack_real(double* __restrict__ out, const double2* __restrict__ in, int64_t D) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D + (D & 1);
       r += (int64_t)gridDim.x * blockDim.x)
    out[r] = r < D ? in[r].x : 0.0;
}
__global__ void k_unpack_real(double2* __restrict__ out, const double* __restrict__ in, int64_t D) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (int64_t)gridDim.x * blockDim.x)
    out[r] = make_double2(in[r], 0.0);
}

unsigned stream_grid(int64_t n) {
  const int64_t g = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}

}  // namespace

// ================================================================ Vec ops
// complex(8) vectors use FP64 arithmetic; complex(4) vectors use the FP32-pipe
// kernels above (error-free products, double-float sums, split scalars).
template <class T>
constexpr bool kF32 = std::is_same<T, float2>::value;

template <class T>
void Ops<T>::dot(const T* x, const T* y, int64_t n, double2* out) {
  if constexpr (kF32<T>) k_dot_part32<<<kRedBlocks, kRedThreads, 0, st>>>(x, y, n, part);
  else if (eft) k_dot_part64e<<<kRedBlocks, kRedThreads, 0, st>>>(x, y, n, part);
  else k_dot_part<T><<<kRedBlocks, kRedThreads, 0, st>>>(x, y, n, part);
  check_launch("k_dot_part");
  k_red_final<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, out, real ? 2 : 0);
  check_launch("k_red_final");
}
template <class T>
void Ops<T>::nrm(const T* x, int64_t n, double2* out) {
  if constexpr (kF32<T>) k_nrm_part32<<<kRedBlocks, kRedThreads, 0, st>>>(x, n, part);
  else if (eft) k_nrm_part64e<<<kRedBlocks, kRedThreads, 0, st>>>(x, n, part);
  else k_nrm_part<T><<<kRedBlocks, kRedThreads, 0, st>>>(x, n, part);
  check_launch("k_nrm_part");
  k_red_final<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, out, 1);
  check_launch("k_red_final");
}
template <class T>
void Ops<T>::scale_inv(T* x, int64_t n, const double2* s) {
  if constexpr (kF32<T>) k_scale_inv32<<<stream_grid(n), 256, 0, st>>>(x, n, s);
  else k_scale_inv<T><<<stream_grid(n), 256, 0, st>>>(x, n, s);
  check_launch("k_scale_inv");
}
template <class T>
void Ops<T>::lanczos_w(T* w, const T* q, const T* v, const T* u, int64_t n, const double2* a, const double2* b,
                       bool real_alpha) {
  const int ra = (real_alpha || real) ? 1 : 0;
  if constexpr (kF32<T>) k_lanczos_w32<<<stream_grid(n), 256, 0, st>>>(w, q, v, u, n, a, b, ra);
  else k_lanczos_w<T><<<stream_grid(n), 256, 0, st>>>(w, q, v, u, n, a, b, ra);
  check_launch("k_lanczos_w");
}
template <class T>
void Ops<T>::axpy(T* y, const T* x, int64_t n, const double2* a, double sgn) {
  if constexpr (kF32<T>) k_axpy32<<<stream_grid(n), 256, 0, st>>>(y, x, n, a, sgn);
  else k_axpy<T><<<stream_grid(n), 256, 0, st>>>(y, x, n, a, sgn);
  check_launch("k_axpy");
}
template <class T>
void Ops<T>::reorth(const T* V, int64_t ldv, int ncols, T* w, int64_t n, double2* ov) {
  if (ncols <= 0) return;
  overlaps(V, ldv, ncols, w, n, ov);
  gemv_sub(V, ldv, ncols, ov, w, n);
}
template <class T>
void Ops<T>::overlaps(const T* V, int64_t ldv, int ncols, const T* w, int64_t n, double2* ov) {
  if (ncols <= 0) return;
  int nb = kRedBlocks;
  if (kF32<T> || eft) {
    const int64_t tiles = (n + 255) / 256;
    nb = (int)std::min<int64_t>(kGemvChunks, tiles);
    const int64_t rows = (tiles + nb - 1) / nb * 256;
    const dim3 grid((unsigned)((ncols + 3) / 4), (unsigned)nb);
    if (real) k_gemv_h3<T, true><<<grid, 256, 0, st>>>(V, ldv, ncols, w, n, rows, part);
    else k_gemv_h3<T, false><<<grid, 256, 0, st>>>(V, ldv, ncols, w, n, rows, part);
  } else {
    if (real) k_gemv_h_part<T, true><<<kRedBlocks, kRedThreads, 0, st>>>(V, ldv, ncols, w, n, part);
    else k_gemv_h_part<T, false><<<kRedBlocks, kRedThreads, 0, st>>>(V, ldv, ncols, w, n, part);
  }
  check_launch("k_gemv_h_part");
  k_gemv_final<<<ncols, kRedThreads, 0, st>>>(part, nb, ncols, ov, real ? 1 : 0);
  check_launch("k_gemv_final");
}
template <class T>
void Ops<T>::gemv_sub(const T* V, int64_t ldv, int ncols, const double2* coef, T* w, int64_t n) {
  if (ncols <= 0) return;
  const unsigned g = stream_grid(n);
  if constexpr (kF32<T>) {
    if (real) k_gemv_sub32<true><<<g, 256, 0, st>>>(V, ldv, ncols, coef, w, n);
    else k_gemv_sub32<false><<<g, 256, 0, st>>>(V, ldv, ncols, coef, w, n);
  } else if (eft) {
    if (real) k_gemv_sub64e<true><<<g, 256, 0, st>>>(V, ldv, ncols, coef, w, n);
    else k_gemv_sub64e<false><<<g, 256, 0, st>>>(V, ldv, ncols, coef, w, n);
  } else {
    if (real) k_gemv_sub<T, true><<<g, 256, 0, st>>>(V, ldv, ncols, coef, w, n);
    else k_gemv_sub<T, false><<<g, 256, 0, st>>>(V, ldv, ncols, coef, w, n);
  }
  check_launch("k_gemv_sub");
}
// launch an in-place restart kernel with sm bytes of dynamic shared memory
template <class K, class... A>
static void launch_restart(K kernel, size_t sm, int64_t n, cudaStream_t st, A... args) {
  if (sm > 48 * 1024)
    QS3G_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  kernel<<<(unsigned)((n + 31) / 32), 256, sm, st>>>(args...);
}

template <class T>
void Ops<T>::restart(T* V, int64_t ldv, int nom, int nok, const double2* C, int64_t n) {
  if constexpr (kF32<T>) {
    const size_t sm = (size_t)nom * nok * sizeof(float4) + (size_t)nom * 32 * sizeof(float2);
    launch_restart(real ? k_restart32<true> : k_restart32<false>, sm, n, st, V, ldv, nom, nok, C, n);
  } else if (eft) {
    const size_t sm = ((size_t)nom * nok + (size_t)nom * 32) * sizeof(float4);
    launch_restart(real ? k_restart64e<true> : k_restart64e<false>, sm, n, st, V, ldv, nom, nok, C, n);
  } else {
    const size_t sm = ((size_t)nom * 32 + (size_t)nom * nok) * sizeof(double2);
    launch_restart(real ? k_restart<T, true> : k_restart<T, false>, sm, n, st, V, ldv, nom, nok, C, n);
  }
  check_launch("k_restart");
}
template <class T>
void Ops<T>::random_start(T* x, int64_t n, uint64_t seed) {
  k_random_start<T><<<stream_grid(n), 256, 0, st>>>(x, n, seed);
  check_launch("k_random_start");
}
template <class T>
void Ops<T>::from64(T* y, const double2* x, int64_t n) {
  k_copy_conv<T><<<stream_grid(n), 256, 0, st>>>(y, x, n);
  check_launch("k_copy_conv");
}
template struct Ops<double2>;
template struct Ops<float2>;

void f32_to_f64(double2* y, const float2* x, int64_t n, cudaStream_t st) {
  k_f32_to_f64<<<stream_grid(n), 256, 0, st>>>(y, x, n);
  check_launch("k_f32_to_f64");
}
void residual64(double2* w, const double2* q, const double2* v, int64_t n, double e, cudaStream_t st) {
  k_residual<<<stream_grid(n), 256, 0, st>>>(w, q, v, n, e);
  check_launch("k_residual");
}

// ================================================================ continued fraction
namespace {
// DSFLan (source_DSFLan/main.f90:52-84) for every (omega, q) pair.
__global__ void k_cfrac(int nq, int ldab, const int* __restrict__ nlev, const double* __restrict__ alpha,
                        const double* __restrict__ beta, const double* __restrict__ norm1,
                        const double* __restrict__ E0, double eta, int nomega, const double* __restrict__ omega,
                        int compat, double* __restrict__ S) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nq * nomega) return;
  const int q = (int)(t / nomega), o = (int)(t % nomega);
  const double* al = alpha + (size_t)q * ldab;
  const double* be = beta + (size_t)q * ldab;
  const int N = nlev[q];
  const double w = omega[o], e0 = E0[q];
  int n = N;
  double kr = w + e0 - al[n - 1] - 0.0;
  double bunbo = kr * kr + eta * eta;
  double tr = be[n - 1] * kr / bunbo;
  double ti = compat ? -be[n - 1] * eta : -be[n - 1] * eta / bunbo;
  for (n = N - 1; n >= 2; --n) {
    kr = w + e0 - al[n - 1] - tr;
    const double ki = eta - ti;
    bunbo = kr * kr + ki * ki;
    tr = be[n - 1] * kr / bunbo;
    ti = -be[n - 1] * ki / bunbo;
  }
  kr = w + e0 - al[0] - tr;
  const double ki = eta - ti;
  bunbo = kr * kr + ki * ki;
  ti = -norm1[q] * ki / bunbo;
  S[(size_t)q * nomega + o] = -ti / 3.14159265358979323846;
}
}  // namespace

void cfrac(int nq, int ldab, const int* nlev, const double* alpha, const double* beta2, const double* norm1,
           const double* E0, double eta, int nomega, const double* omega, int compat, double* S, cudaStream_t st) {
  for (int q = 0; q < nq; ++q) QS3G_REQUIRE(nlev[q] >= 1 && nlev[q] <= ldab, QS3G_EINVAL, "nlev out of range");
  DevBuf<int> d_nlev(nq);
  DevBuf<double> d_a((size_t)ldab * nq), d_b((size_t)ldab * nq), d_n(nq), d_e(nq), d_w(nomega),
      d_S((size_t)nomega * nq);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_nlev.get(), nlev, nq * 4, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_a.get(), alpha, (size_t)ldab * nq * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_b.get(), beta2, (size_t)ldab * nq * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_n.get(), norm1, nq * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_e.get(), E0, nq * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_w.get(), omega, (size_t)nomega * 8, cudaMemcpyHostToDevice, st));
  const int64_t tot = (int64_t)nq * nomega;
  k_cfrac<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nq, ldab, d_nlev.get(), d_a.get(), d_b.get(), d_n.get(),
                                                        d_e.get(), eta, nomega, d_w.get(), compat, d_S.get());
  check_launch("k_cfrac");
  QS3G_CHECK_CUDA(cudaMemcpyAsync(S, d_S.get(), (size_t)nomega * nq * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------- continued fraction without allocation
// For callers that cannot call cudaMalloc: the device copies of the inputs and
// of S live in one file-scope static device array of kCfracStaticDoubles
// doubles (4 MiB), which every GPU that loads the library holds until the
// process exits.  The host name g_cfrac_static is only a host-side stand-in
// for the array; its device address comes from cudaGetSymbolAddress, taken
// once per device (with that device current) on the first call on it, so that
// first call should come before any stream capture.  Every call reuses the
// same array and leaves the last call's data in it; the kernel writes every
// element of S it returns, so nothing has to start at zero.  Calls that
// overlap on the GPU (two host threads, or two processes sharing the array
// through MPS) race on the array.
constexpr size_t kCfracStaticDoubles = size_t(1) << 19;
static __device__ __align__(256) double g_cfrac_static[kCfracStaticDoubles];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_cfrac_static_mu;
double* g_cfrac_static_ptr[kMaxDevices] = {};

double* cfrac_static_area() {
  int dev = 0;
  QS3G_CHECK_CUDA(cudaGetDevice(&dev));
  QS3G_REQUIRE(dev >= 0 && dev < kMaxDevices, QS3G_ERANGE, "device ordinal beyond 64");
  std::lock_guard<std::mutex> lk(g_cfrac_static_mu);
  if (!g_cfrac_static_ptr[dev]) {
    void* p = nullptr;
    QS3G_CHECK_CUDA(cudaGetSymbolAddress(&p, g_cfrac_static));
    g_cfrac_static_ptr[dev] = static_cast<double*>(p);
  }
  return g_cfrac_static_ptr[dev];
}

size_t up32(size_t n) { return (n + 31) & ~size_t(31); }  // keep every region 256-byte aligned
}  // namespace

void cfrac_noalloc(int nq, int ldab, const int* nlev, const double* alpha, const double* beta2, const double* norm1,
                   const double* E0, double eta, int nomega, const double* omega, int compat, double* S) {
  for (int q = 0; q < nq; ++q) QS3G_REQUIRE(nlev[q] >= 1 && nlev[q] <= ldab, QS3G_EINVAL, "nlev out of range");
  const size_t nab = (size_t)ldab * nq, nS = (size_t)nomega * nq;
  const size_t o_a = 0, o_b = o_a + up32(nab), o_n = o_b + up32(nab), o_e = o_n + up32(nq), o_w = o_e + up32(nq),
               o_S = o_w + up32(nomega), o_l = o_S + up32(nS), total = o_l + up32(((size_t)nq + 1) / 2);
  if (total > kCfracStaticDoubles)
    throw Error(QS3G_ERANGE, "qs3g_cfrac_noalloc: these sizes need " + std::to_string(total * 8) +
                                 " bytes of device scratch; the static area holds " +
                                 std::to_string(kCfracStaticDoubles * 8) + " bytes (use qs3g_cfrac)");
  double* base = cfrac_static_area();
  int* d_nlev = reinterpret_cast<int*>(base + o_l);
  const cudaStream_t st = 0;  // the legacy default stream: no stream is created
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_nlev, nlev, (size_t)nq * 4, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(base + o_a, alpha, nab * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(base + o_b, beta2, nab * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(base + o_n, norm1, (size_t)nq * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(base + o_e, E0, (size_t)nq * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(base + o_w, omega, (size_t)nomega * 8, cudaMemcpyHostToDevice, st));
  const int64_t tot = (int64_t)nq * nomega;
  k_cfrac<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nq, ldab, d_nlev, base + o_a, base + o_b, base + o_n,
                                                        base + o_e, eta, nomega, base + o_w, compat, base + o_S);
  check_launch("k_cfrac(static scratch)");
  QS3G_CHECK_CUDA(cudaMemcpyAsync(S, base + o_S, nS * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

// ================================================================ thick-restart Lanczos
// Relative residual at which the complex(4) phase of precision 1 hands over
// to the complex(8) phase: TrlanParams::tol32 when set, else QS3G_TOL32 from
// the environment, else 1e-6.  The phase also stops when its residual
// estimate stagnates (the FP32 floor).
double phase1_tol(double tol32) {
  if (tol32 > 0) return tol32;
  static const double v = [] {
    const char* e = std::getenv("QS3G_TOL32");
    const double x = e ? std::atof(e) : 0.0;
    return x > 0 ? x : 1e-6;
  }();
  return v;
}

// With a residual target, the first attempt stops when the Ritz estimate
// |beta_NOM C(NOM, j)| reaches est_factor * tol; the FP64 residual is then
// recomputed (it can sit above the estimate).  QS3G_EST_FACTOR overrides the
// default 0.5.
double est_factor() {
  static const double v = [] {
    const char* e = std::getenv("QS3G_EST_FACTOR");
    const double x = e ? std::atof(e) : 0.0;
    return (x > 0 && x <= 1) ? x : 0.5;
  }();
  return v;
}

// Precision 1 with NOE = 1 runs the anchored solver (trlan_anchor.cu) unless
// QS3G_ANCHOR=0.
bool anchored_enabled() {
  static const bool v = [] {
    const char* e = std::getenv("QS3G_ANCHOR");
    return !(e && e[0] == '0');
  }();
  return v;
}

// QS3G_VERBOSE=1 prints one progress line per restart, as QS3 does.
bool verbose() {
  static const bool v = [] {
    const char* e = std::getenv("QS3G_VERBOSE");
    return e && e[0] && e[0] != '0';
  }();
  return v;
}

namespace {

template <class T>
struct HvOp;
template <>
struct HvOp<double2> {
  // eft: the double-float modes, which read a cached connection table in
  // double-float arithmetic too (FP64 arithmetic otherwise)
  static void apply(const Model& m, const Sector& s, const double2* x, double2* y, cudaStream_t st, double,
                    bool real, bool eft = false) {
    if (real) {
      auto* xr = reinterpret_cast<const double*>(x);
      auto* yr = reinterpret_cast<double*>(y);
      if (!(eft && hv64r_df(m, s, xr, yr, st, true))) hv64r(m, s, xr, yr, st, true);
    } else if (!(eft && hv64_df(m, s, x, y, st))) {
      hv64(m, s, x, y, st);
    }
  }
};
template <>
struct HvOp<float2> {
  static void apply(const Model& m, const Sector& s, const float2* x, float2* y, cudaStream_t st, double shift,
                    bool real, bool = false) {
    if (real) hv32r(m, s, reinterpret_cast<const float*>(x), reinterpret_cast<float*>(y), st, (float)shift, true);
    else hv32(m, s, x, y, st, (float)shift);
  }
};

struct TrlanOut {
  std::vector<double> ene;
  int hv_count = 0;
  bool converged = false;
  int restarts = 0;
  bool timed_out = false;
};

double wall_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// FP64 residual of the Ritz pairs in V[:, :NOE] with Ritz values ene[0..NOE):
// the largest, in the units of conv_mode.
using RitzCheck = std::function<double(const std::vector<double>& ene)>;

// lancz_eigen_val_complex (eigen_solver.f90:69-261) on device vectors of type T.
// V must hold NOM+1 columns of length ldv; V[:,0] holds the start vector.
// real: the vectors are real, two rows per T slot (real_sector(s)); every
// scalar of the recurrence (alpha, overlaps, Ritz coefficients) is then real.
// check (conv_mode 1, 2): once the Ritz estimate is within 4x of target, each
// restart also recomputes the true residual and stops as soon as it meets
// target -- an early exit only; the iteration itself is unchanged.
template <class T>
TrlanOut trlan_core(const Model& m, const Sector& s, T* V, int64_t ldv, T* Q, int NOE, int NOK, int NOM, int maxitr,
                    double tol, int conv_mode, cudaStream_t st, Scratch& sc, int reorth_passes,
                    double shift = 0.0, bool eft = false, bool real = false, const RitzCheck& check = RitzCheck(),
                    double target = 0.0, double deadline = 0.0) {
  const int64_t D = real ? (s.D + 1) / 2 : s.D;  // T slots per vector
  Ops<T> ops{st, sc.part.get(), eft, real};
  double2* alpha = sc.scal;              // [NOM+2]
  double2* beta = sc.scal + (NOM + 2);   // [NOM+2]
  double2* ov = sc.scal + 2 * (NOM + 2); // [NOM+2]
  double2* cb = sc.scal + 3 * (NOM + 2); // arrow couplings [NOM+2]
  TrlanOut out;
  auto col = [&](int j) { return V + (int64_t)j * ldv; };
  auto reorth = [&](int i) {  // against Fortran columns 1..i-1 = V[:, 0..i-2]
    for (int p = 0; p < reorth_passes; ++p) ops.reorth(V, ldv, i - 1, col(i), D, ov);
  };

  // ---- initial Lanczos pass (eigen_solver.f90:98-124)
  ops.nrm(col(0), D, beta + 0);
  for (int i = 1; i <= NOM; ++i) {
    ops.scale_inv(col(i - 1), D, beta + (i - 1));
    HvOp<T>::apply(m, s, col(i - 1), Q, st, shift, real, eft);
    ++out.hv_count;
    ops.dot(col(i - 1), Q, D, alpha + i);
    if (i > 1) {
      ops.lanczos_w(col(i), Q, col(i - 1), col(i - 2), D, alpha + i, beta + (i - 1), true);
      reorth(i);
    } else {
      ops.lanczos_w(col(i), Q, col(i - 1), nullptr, D, alpha + i, beta, true);
    }
    ops.nrm(col(i), D, beta + i);
  }
  ops.scale_inv(col(NOM), D, beta + NOM);
  std::vector<double2> ha(NOM + 2), hb(NOM + 2);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(ha.data(), alpha, (NOM + 2) * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(hb.data(), beta, (NOM + 2) * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  for (int i = 0; i <= NOM; ++i)
    QS3G_REQUIRE(std::isfinite(hb[i].x) && hb[i].x > 0.0 && std::isfinite(ha[i < 1 ? 1 : i].x),
                 QS3G_EBREAKDOWN, "Lanczos breakdown in the initial pass");
  // dstevx('V','A') on the NOM x NOM tridiagonal
  std::vector<zd> Tm((size_t)NOM * NOM, zd(0.0, 0.0));
  for (int j = 0; j < NOM; ++j) Tm[j + (size_t)j * NOM] = ha[j + 1].x;
  for (int j = 0; j < NOM - 1; ++j) Tm[j + (size_t)(j + 1) * NOM] = hb[j + 1].x;
  std::vector<double> ene;
  std::vector<zd> Cc;
  herm_jacobi(NOM, Tm, ene, Cc);
  std::vector<zd> calpha(NOM + 1), cbeta(NOM + 1);
  for (int j = 1; j <= NOM; ++j) calpha[j] = ha[j].x;
  for (int j = 0; j <= NOM; ++j) cbeta[j] = hb[j].x;
  int flag = 0, stall = 0;
  double best_conv = 1e300;
  std::vector<double2> hC((size_t)NOM * NOK);
  for (int tritr = 1; tritr <= maxitr; ++tritr) {
    out.restarts = tritr;
    for (int j = 0; j < NOK; ++j)
      for (int i = 0; i < NOM; ++i)
        hC[(size_t)j * NOM + i] = make_double2(Cc[i + (size_t)j * NOM].real(), real ? 0.0 : Cc[i + (size_t)j * NOM].imag());
    QS3G_CHECK_CUDA(cudaMemcpyAsync(sc.C, hC.data(), hC.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    ops.restart(V, ldv, NOM, NOK, sc.C, D);
    // convergence (eigen_solver.f90:150-159) or the Ritz residual bound
    double max_conv = 0.0;
    if (conv_mode == 0) {
      for (int j = 0; j < NOK; ++j) max_conv = std::max(max_conv, std::abs(calpha[j + 1] / ene[j] - 1.0));
    } else {
      for (int j = 0; j < NOE; ++j) {
        double rj = std::abs(cbeta[NOM] * Cc[(NOM - 1) + (size_t)j * NOM]);
        if (conv_mode == 2) rj /= std::max(1.0, std::fabs(ene[j]));
        max_conv = std::max(max_conv, rj);
      }
    }
    flag = (max_conv < tol) ? flag + 1 : 0;
    if (verbose())  // the progress line of eigen_solver.f90:157-158
      std::printf("tritr, ene(NOK), max_conv, flag: %5d %25.15e %11.1e %5d  (%s, hv=%d)\n", tritr, ene[NOK - 1],
                  max_conv, flag, sizeof(T) == 8 ? "complex(4)" : (ops.eft ? "complex(8) df" : "complex(8) fp64"),
                  out.hv_count);
    bool done = (conv_mode == 0 && flag == 2) || (conv_mode != 0 && flag >= 1);
    if (!done && check && max_conv < 4.0 * target) {
      const double worst = check(ene);
      out.hv_count += NOE;
      if (verbose()) std::printf("trlan: residual check at estimate %.2e: %.3e\n", max_conv, worst);
      done = worst <= target;
    }
    if (done) {
      out.converged = true;
      break;
    }
    if (conv_mode == 2) {  // complex(4) phase: stop once the residual estimate stagnates at the FP32 floor
      if (max_conv < 0.95 * best_conv) { best_conv = max_conv; stall = 0; }
      else if (++stall >= 20) break;
    }
    if (tritr == maxitr) break;
    if (deadline > 0.0 && wall_seconds() > deadline) {
      out.timed_out = true;
      break;
    }
    QS3G_CHECK_CUDA(cudaMemcpyAsync(col(NOK), col(NOM), D * sizeof(T), cudaMemcpyDeviceToDevice, st));
    for (int j = 0; j < NOK; ++j) calpha[j + 1] = ene[j];
    for (int j = 1; j <= NOK; ++j) cbeta[j] = cbeta[NOM] * Cc[(NOM - 1) + (size_t)(j - 1) * NOM];
    std::vector<double2> hcb(NOK);
    for (int j = 0; j < NOK; ++j) hcb[j] = make_double2(cbeta[j + 1].real(), real ? 0.0 : cbeta[j + 1].imag());
    QS3G_CHECK_CUDA(cudaMemcpyAsync(cb, hcb.data(), NOK * sizeof(double2), cudaMemcpyHostToDevice, st));
    int i = NOK + 1;
    HvOp<T>::apply(m, s, col(i - 1), Q, st, shift, real, eft);
    ++out.hv_count;
    ops.dot(col(i - 1), Q, D, alpha + i);
    ops.gemv_sub(V, ldv, NOK, cb, Q, D);
    ops.lanczos_w(col(i), Q, col(i - 1), nullptr, D, alpha + i, beta, false);
    reorth(i);
    ops.nrm(col(i), D, beta + i);
    for (i = NOK + 2; i <= NOM; ++i) {
      ops.scale_inv(col(i - 1), D, beta + (i - 1));
      HvOp<T>::apply(m, s, col(i - 1), Q, st, shift, real, eft);
      ++out.hv_count;
      ops.dot(col(i - 1), Q, D, alpha + i);
      ops.lanczos_w(col(i), Q, col(i - 1), col(i - 2), D, alpha + i, beta + (i - 1), false);
      reorth(i);
      ops.nrm(col(i), D, beta + i);
    }
    ops.scale_inv(col(NOM), D, beta + NOM);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(ha.data(), alpha, (NOM + 2) * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(hb.data(), beta, (NOM + 2) * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    for (int j = NOK + 1; j <= NOM; ++j) {
      calpha[j] = zd(ha[j].x, real ? 0.0 : ha[j].y);
      cbeta[j] = hb[j].x;
      QS3G_REQUIRE(std::isfinite(hb[j].x) && hb[j].x > 0.0 && std::isfinite(ha[j].x), QS3G_EBREAKDOWN,
                   "Lanczos breakdown after a restart");
    }
    std::fill(Tm.begin(), Tm.end(), zd(0.0, 0.0));
    for (int j = 0; j < NOM; ++j) Tm[j + (size_t)j * NOM] = calpha[j + 1];
    for (int j = 0; j < NOK; ++j) Tm[j + (size_t)NOK * NOM] = cbeta[j + 1];
    for (int j = NOK + 1; j <= NOM - 1; ++j) Tm[(j - 1) + (size_t)j * NOM] = cbeta[j];
    herm_jacobi(NOM, Tm, ene, Cc);
  }
  out.ene = ene;
  for (double& e : out.ene) e += shift;  // the Lanczos ran on H - shift
  return out;
}

}  // namespace

void Scratch::ensure(int nom) {
  if (part.n == 0) part.alloc((size_t)kRedBlocks * 128);
  if ((int)scal.n < 4 * (nom + 2)) scal.alloc(4 * (size_t)(nom + 2));
  if ((int)C.n < nom * nom) C.alloc((size_t)nom * nom);
}

int trlan(const Model& m, const Sector& s, const TrlanParams& p, const double2* h_start, double* ene_out,
          double2* h_psi, int* iters, double* resid, cudaStream_t st, TrlanStats* stats) {
  const double t_start = wall_seconds();
  const double deadline = p.time_limit > 0.0 ? t_start + p.time_limit : 0.0;
  int NOM = p.NOM;
  const int NOE = p.NOE, NOK = p.NOK;
  QS3G_REQUIRE(NOE >= 1 && NOK >= 1 && NOE <= NOK, QS3G_EINVAL, "need 1 <= NOE <= NOK");
  if (NOM < 2 * NOK) NOM = 2 * NOK;  // eigen_solver.f90:20
  const int64_t D = s.D;
  QS3G_REQUIRE(D >= NOE && D >= NOK && D >= NOM, QS3G_EINVAL, "sector dimension smaller than NOM (stop 999)");
  QS3G_REQUIRE(NOM <= 120, QS3G_EINVAL, "NOM must be <= 120");
  const bool real = p.real;
  QS3G_REQUIRE(!real || real_sector(s), QS3G_ENOTSUP, "real arithmetic needs a k = 0 chain sector or a U(1) sector");
  // complex slots per Krylov vector: D, or ceil(D/2) for real vectors (two
  // rows per slot, a zero pad row when D is odd)
  const int64_t n = real ? (D + 1) / 2 : D;
  const int64_t ldv = (n + 31) / 32 * 32;
  auto hv_fp64 = [&](const double2* x, double2* y) {
    if (real) hv64r(m, s, reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y), st, true);
    else hv64(m, s, x, y, st);
  };
  Scratch sc;
  sc.ensure(NOM);
  int hv_total = 0, restarts_total = 0;
  bool timed_out = false;
  std::vector<double> ene, ene_phase1;
  DevBuf<double2> d_start, d_pack;
  const double2* start64 = nullptr;
  if (h_start) {
    d_start.alloc(D);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(d_start.get(), h_start, D * sizeof(double2), cudaMemcpyHostToDevice, st));
    start64 = d_start.get();
    if (real) {  // the real part of the given start vector
      d_pack.alloc(n);
      k_pack_real<<<stream_grid(n), 256, 0, st>>>(reinterpret_cast<double*>(d_pack.get()), start64, D);
      check_launch("k_pack_real");
      start64 = d_pack.get();
    }
  }
  bool converged = false;
  DevBuf<double2> V64((size_t)ldv * (NOM + 1)), Q64(D);
  // Precision 1 for the lowest eigenpair: the anchored solver keeps the
  // approximation in FP64 and every Krylov vector in FP32 to the end; if its
  // residual stalls (an FP32 floor), the double-float attempts below continue
  // from its vector.  QS3G_ANCHOR=0 selects the two-phase form instead.
  bool anchored = false, anchored_done = false, anchored_conv = false;
  int hv_fp32 = 0;
  if (p.precision == 1 && NOE == 1 && anchored_enabled()) {
    anchored = true;
    Ops<double2> o64{st, sc.part.get()};
    if (start64) QS3G_CHECK_CUDA(cudaMemcpyAsync(V64.get(), start64, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    else o64.random_start(V64.get(), n, p.seed);
    if (real && (D & 1)) QS3G_CHECK_CUDA(cudaMemsetAsync(reinterpret_cast<double*>(V64.get()) + D, 0, sizeof(double), st));
    AnchorParams ap;
    ap.NOK = NOK; ap.NOM = NOM; ap.maxitr = p.maxitr; ap.conv_mode = p.conv_mode; ap.tol = p.tol;
    ap.real = real; ap.n = n; ap.ldv = ldv; ap.deadline = deadline;
    const AnchorOut a = trlan_anchored(m, s, ap, V64.get(), st);
    hv_fp32 = a.hv32;
    hv_total += a.hv32 + a.hv64;
    restarts_total += a.restarts;
    timed_out = a.timed_out;
    ene_phase1.assign(1, a.ene);
    anchored_done = !a.stalled;
    anchored_conv = a.converged;
    if (verbose())
      std::printf("trlan: anchored solve %s after %d cycles, ||r|| = %.3e\n",
                  a.converged ? "converged" : (a.stalled ? "stalled" : "stopped"), a.restarts, a.resid);
  } else if (p.precision == 1) {
    // phase 1: complex(4) Krylov storage, FP64 reductions and Ritz solve
    DevBuf<float2> V32((size_t)ldv * (NOM + 1)), Q32(n);
    Ops<float2> o32{st, sc.part.get()};
    if (start64) o32.from64(V32.get(), start64, n);
    else o32.random_start(V32.get(), n, p.seed);
    if (real && (D & 1)) QS3G_CHECK_CUDA(cudaMemsetAsync(reinterpret_cast<float*>(V32.get()) + D, 0, sizeof(float), st));
    const double tol1 = phase1_tol(p.tol32);
    // the complex(4) phase runs on H - sigma, sigma = sum_b Jz_b/4 (the fully polarised energy): the
    // large common diagonal then does not enter the FP32 rounding of H*v
    TrlanOut r1 = trlan_core<float2>(m, s, V32.get(), ldv, Q32.get(), NOE, NOK, NOM, p.maxitr, tol1, 2, st, sc,
                                     p.reorth_passes, m.Sz_all, false, real, RitzCheck(), 0.0, deadline);
    hv_total += r1.hv_count;
    restarts_total += r1.restarts;
    timed_out = r1.timed_out;
    ene_phase1 = r1.ene;
    hv_fp32 = r1.hv_count;
    // phase 2: FP64 thick-restart Lanczos from the sum of the NOE Ritz vectors
    Ops<double2> o64{st, sc.part.get()};
    f32_to_f64(V64.get(), V32.get(), n, st);
    for (int j = 1; j < NOE; ++j) {
      f32_to_f64(Q64.get(), V32.get() + (int64_t)j * ldv, n, st);
      std::vector<double2> one(1, make_double2(1.0, 0.0));
      QS3G_CHECK_CUDA(cudaMemcpyAsync(sc.C, one.data(), sizeof(double2), cudaMemcpyHostToDevice, st));
      o64.axpy(V64.get(), Q64.get(), n, sc.C, 1.0);
    }
  } else {
    Ops<double2> o64{st, sc.part.get()};
    if (start64) QS3G_CHECK_CUDA(cudaMemcpyAsync(V64.get(), start64, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    else o64.random_start(V64.get(), n, p.seed);
    if (real && (D & 1)) QS3G_CHECK_CUDA(cudaMemsetAsync(reinterpret_cast<double*>(V64.get()) + D, 0, sizeof(double), st));
  }
  const int hv_phase1 = hv_fp32;
  // With a residual target (conv_mode 1, 2) the Ritz estimate |beta C| can sit
  // below the true residual; the run is accepted only when the FP64 residual
  // ||H psi - E psi|| recomputed from the Ritz vectors meets the target, else it
  // continues from the Ritz vectors (a fresh Lanczos start: continuing the
  // same thick restart would keep the orthogonality its basis has lost against
  // the converged vector, which at L = 400 held the residual at 1.2e-10) with
  // a tighter estimate target.
  double tol_est = p.conv_mode == 0 ? p.tol : est_factor() * p.tol;
  // Precision 1 and 2 refine with double-float arithmetic on the FP32 pipe
  // and precision 0 in FP64.  The first continuation stays in double-float;
  // from the second on (at the double-float floor, about 1e-12 relative to
  // |E|) they run in FP64 arithmetic.  Every attempt stops early when the
  // recomputed residual meets the target (trlan_core's check).  A breakdown
  // in a continuation, which starts from a nearly exact eigenvector, keeps
  // the previous attempt's result (NOE = 1).
  RitzCheck check;
  if (p.conv_mode != 0) {
    check = [&](const std::vector<double>& e) {
      Ops<double2> o64{st, sc.part.get()};
      double worst = 0.0;
      for (int j = 0; j < NOE; ++j) {
        double2* pj = V64.get() + (int64_t)j * ldv;
        hv_fp64(pj, Q64.get());
        residual64(Q64.get(), Q64.get(), pj, n, e[j], st);
        o64.nrm(Q64.get(), n, sc.scal);  // sc.scal[0] = alpha[0], never used
        double2 rr;
        QS3G_CHECK_CUDA(cudaMemcpyAsync(&rr, sc.scal, sizeof(double2), cudaMemcpyDeviceToHost, st));
        QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
        const double scale = p.conv_mode == 2 ? std::max(1.0, std::fabs(e[j])) : 1.0;
        worst = std::max(worst, rr.x / scale);
      }
      return worst;
    };
  }
  TrlanOut r2;
  if (anchored_done) {
    r2.ene = ene_phase1;
    r2.converged = anchored_conv;
  }
  for (int attempt = 0; attempt < 4 && !timed_out && !anchored_done; ++attempt) {
    const bool eft = p.precision != 0 && attempt < 2;
    if (attempt == 0) {
      r2 = trlan_core<double2>(m, s, V64.get(), ldv, Q64.get(), NOE, NOK, NOM, p.maxitr, tol_est, p.conv_mode, st,
                               sc, p.reorth_passes, 0.0, eft, real, check, p.tol, deadline);
    } else {
      try {
        r2 = trlan_core<double2>(m, s, V64.get(), ldv, Q64.get(), NOE, NOK, NOM, p.maxitr, tol_est, p.conv_mode,
                                 st, sc, p.reorth_passes, 0.0, eft, real, check, p.tol, deadline);
      } catch (const Error& e) {
        // with NOE = 1 column 0 still holds the (normalised) previous Ritz
        // vector; with more, the other Ritz vectors were overwritten
        if (e.code != QS3G_EBREAKDOWN || NOE > 1) throw;
        if (verbose()) std::printf("trlan: continuation stopped (%s); keeping the previous Ritz pairs\n", e.what());
        break;
      }
    }
    hv_total += r2.hv_count;
    restarts_total += r2.restarts;
    timed_out = timed_out || r2.timed_out;
    if (p.conv_mode == 0 || !r2.converged) break;
    Ops<double2> o64{st, sc.part.get()};
    double worst = 0.0;
    for (int j = 0; j < NOE; ++j) {
      double2* pj = V64.get() + (int64_t)j * ldv;
      hv_fp64(pj, Q64.get());
      residual64(Q64.get(), Q64.get(), pj, n, r2.ene[j], st);
      o64.nrm(Q64.get(), n, sc.scal);
      double2 rr;
      QS3G_CHECK_CUDA(cudaMemcpyAsync(&rr, sc.scal, sizeof(double2), cudaMemcpyDeviceToHost, st));
      QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
      const double scale = p.conv_mode == 2 ? std::max(1.0, std::fabs(r2.ene[j])) : 1.0;
      worst = std::max(worst, rr.x / scale);
    }
    hv_total += NOE;
    if (verbose()) std::printf("trlan: Ritz estimate met %.2e, recomputed residual %.3e\n", tol_est, worst);
    if (worst <= p.tol) break;
    r2.converged = false;
    tol_est *= std::max(0.01, 0.5 * p.tol / worst);
    // continue from the Ritz vectors: sum of the NOE lowest as the new start
    for (int j = 1; j < NOE; ++j) {
      std::vector<double2> one(1, make_double2(1.0, 0.0));
      QS3G_CHECK_CUDA(cudaMemcpyAsync(sc.C, one.data(), sizeof(double2), cudaMemcpyHostToDevice, st));
      o64.axpy(V64.get(), V64.get() + (int64_t)j * ldv, n, sc.C, 1.0);
    }
  }
  if (verbose()) std::printf("trlan: %d H*v in the complex(4) phase, %d in the complex(8) phase\n", hv_phase1,
                             hv_total - hv_phase1);
  converged = r2.converged;
  ene = r2.ene;
  // a time limit reached in the complex(4) phase leaves that phase's Ritz values
  if ((int)ene.size() < NOE) ene = ene_phase1;
  if ((int)ene.size() < NOE) ene.assign(NOE, std::numeric_limits<double>::quiet_NaN());
  for (int j = 0; j < NOE; ++j) ene_out[j] = ene[j];
  if (iters) *iters = hv_total;
  // FP64 residuals ||H psi_j - E_j psi_j|| of the Ritz vectors in V[:, :NOE]
  if (resid || h_psi) {
    Ops<double2> o64{st, sc.part.get()};
    DevBuf<double2> W(D);
    for (int j = 0; j < NOE; ++j) {
      double2* pj = V64.get() + (int64_t)j * ldv;
      if (resid) {
        hv_fp64(pj, Q64.get());
        residual64(W.get(), Q64.get(), pj, n, ene[j], st);
        o64.nrm(W.get(), n, sc.scal);
        double2 r;
        QS3G_CHECK_CUDA(cudaMemcpyAsync(&r, sc.scal, sizeof(double2), cudaMemcpyDeviceToHost, st));
        QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
        resid[j] = r.x;
      }
      if (h_psi) {
        const double2* src = pj;
        if (real) {  // (psi_r, 0)
          k_unpack_real<<<stream_grid(D), 256, 0, st>>>(W.get(), reinterpret_cast<const double*>(pj), D);
          check_launch("k_unpack_real");
          src = W.get();
        }
        QS3G_CHECK_CUDA(cudaMemcpyAsync(h_psi + (int64_t)j * D, src, D * sizeof(double2), cudaMemcpyDeviceToHost, st));
      }
    }
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  if (stats) {
    stats->hv32 = hv_phase1;
    stats->hv64 = hv_total - hv_phase1;
    stats->restarts = restarts_total;
    stats->timed_out = timed_out;
    stats->seconds = wall_seconds() - t_start;
  }
  return converged ? QS3G_OK : QS3G_ENOTCONV;
}

// ================================================================ plain Lanczos (ALG=1)
int lanczos(const Model& m, const Sector& s, int maxitr, int minitr, int itrint, double tol, const double2* h_start,
            uint64_t seed, double* ene_out, double2* h_psi, int* iters, cudaStream_t st) {
  const int64_t D = s.D;
  QS3G_REQUIRE(D >= 1, QS3G_ESTATE, "empty sector");
  QS3G_REQUIRE(maxitr >= 1 && itrint >= 1, QS3G_EINVAL, "maxitr, itrint must be >= 1");
  Scratch sc;
  sc.ensure(8);
  Ops<double2> ops{st, sc.part.get()};
  DevBuf<double2> v1(D), v2(D), v3(D), io(D);
  DevBuf<double2> d_ab((size_t)2 * (maxitr + 2));  // alpha[i], beta[i] as double2
  double2* alpha = d_ab.get();
  double2* beta = d_ab.get() + (maxitr + 2);
  if (h_start) QS3G_CHECK_CUDA(cudaMemcpyAsync(v1.get(), h_start, D * sizeof(double2), cudaMemcpyHostToDevice, st));
  else ops.random_start(v1.get(), D, seed);
  ops.nrm(v1.get(), D, beta + 0);
  ops.scale_inv(v1.get(), D, beta + 0);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(io.get(), v1.get(), D * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  const int mitr = (int)std::min<int64_t>(maxitr, D);
  double tmp = 0.0, ene = 0.0;
  std::vector<double> z;
  int ite = -1;
  std::vector<double2> ha, hb;
  for (int i = 1; i <= mitr; ++i) {
    hv64(m, s, v1.get(), v2.get(), st);
    ops.dot(v1.get(), v2.get(), D, alpha + i);
    if (i > 1) ops.lanczos_w(v2.get(), v2.get(), v1.get(), v3.get(), D, alpha + i, beta + (i - 1), true);
    else ops.lanczos_w(v2.get(), v2.get(), v1.get(), nullptr, D, alpha + i, beta, true);
    ops.nrm(v2.get(), D, beta + i);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v3.get(), v1.get(), D * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v1.get(), v2.get(), D * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    ops.scale_inv(v1.get(), D, beta + i);
    if (i == mitr || (i >= minitr && i % itrint == 0)) {
      ha.resize(i + 1);
      hb.resize(i + 1);
      QS3G_CHECK_CUDA(cudaMemcpyAsync(ha.data(), alpha, (i + 1) * sizeof(double2), cudaMemcpyDeviceToHost, st));
      QS3G_CHECK_CUDA(cudaMemcpyAsync(hb.data(), beta, (i + 1) * sizeof(double2), cudaMemcpyDeviceToHost, st));
      QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
      if (i == 1) {  // lanczos.f90:99-106
        ene_out[0] = ha[1].x;
        if (h_psi) {
          std::vector<double2> e(D, make_double2(0.0, 0.0));
          e[0] = make_double2(1.0, 0.0);
          std::memcpy(h_psi, e.data(), D * sizeof(double2));
        }
        if (iters) *iters = 1;
        return QS3G_OK;
      }
      std::vector<double> d(i), e(i - 1);
      for (int k = 0; k < i; ++k) d[k] = ha[k + 1].x;
      for (int k = 0; k < i - 1; ++k) e[k] = hb[k + 1].x;
      tridiag_lowest(d, e, ene, z);
      const double conv = std::fabs(tmp / ene - 1.0);
      if (i == maxitr || conv < tol) { ite = i; break; }
      tmp = ene;
    }
  }
  QS3G_REQUIRE(ite > 0, QS3G_ENOTCONV, "Lanczos reached min(maxitr, dim) without converging");
  ene_out[0] = ene;
  if (iters) *iters = 2 * ite - 1;
  if (!h_psi) return QS3G_OK;
  // eigenvector replay (lanczos.f90:123-150)
  std::vector<double2> hz(ite);
  for (int k = 0; k < ite; ++k) hz[k] = make_double2(z[k], 0.0);
  DevBuf<double2> dz(ite);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(dz.get(), hz.data(), ite * sizeof(double2), cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(v1.get(), io.get(), D * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  // psi_io = z(1) * psi_io  (my_zdscal)
  QS3G_CHECK_CUDA(cudaMemsetAsync(io.get(), 0, D * sizeof(double2), st));
  ops.axpy(io.get(), v1.get(), D, dz.get(), 1.0);
  for (int i = 1; i <= ite - 1; ++i) {
    hv64(m, s, v1.get(), v2.get(), st);
    if (i > 1) ops.lanczos_w(v2.get(), v2.get(), v1.get(), v3.get(), D, alpha + i, beta + (i - 1), true);
    else ops.lanczos_w(v2.get(), v2.get(), v1.get(), nullptr, D, alpha + i, beta, true);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v3.get(), v1.get(), D * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v1.get(), v2.get(), D * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    ops.scale_inv(v1.get(), D, beta + i);
    ops.axpy(io.get(), v1.get(), D, dz.get() + i, 1.0);
  }
  ops.nrm(io.get(), D, beta + 0);
  ops.scale_inv(io.get(), D, beta + 0);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(h_psi, io.get(), D * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  return QS3G_OK;
}

}  // namespace qs3g
