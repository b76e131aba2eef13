// eft.cuh -- double-float (error-free transformation) arithmetic on the FP32
// pipe, shared by the level-1 kernels (krylov.cu) and their batched forms
// (batch_trlan.cu).  GB300 issues FP64 at 1/64 of the FP32 rate, and float <->
// double conversions use the FP64 pipe too, so FP64-accurate reductions and
// updates are carried out as unevaluated float pairs (hi, lo):
//  * a product of two floats is split exactly into p + e (p = a*b rounded,
//    e = fma(a, b, -p)); sums use the TwoSum transformation;
//  * FP64 operands are split into hi + lo floats with integer instructions
//    only (dsplit); FP64 scalars on the host side with a double subtraction
//    (split), which runs once per kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace qs3g {

__device__ __forceinline__ double2 block_sum2(double2 v, double2* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sh[threadIdx.x].x += sh[threadIdx.x + s].x;
      sh[threadIdx.x].y += sh[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  return sh[0];
}

__device__ __forceinline__ void df_add(float& hi, float& lo, float p) {
  const float t = __fadd_rn(hi, p);
  const float z = __fsub_rn(t, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(p, z));
  hi = t;
  lo = __fadd_rn(lo, err);
}
__device__ __forceinline__ void df_add_prod(float& hi, float& lo, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  df_add(hi, lo, p);
  lo = __fadd_rn(lo, e);
}
__device__ __forceinline__ float2 split(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

__device__ __forceinline__ float2 dsplit(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const unsigned h32 = (unsigned)(u >> 32), l32 = (unsigned)u;
  const int e = (int)((h32 >> 20) & 0x7ffu);
  const unsigned sgn = h32 & 0x80000000u;
  if (e < 897) return make_float2(0.f, 0.f);
  if (e > 1150) return make_float2(__uint_as_float(sgn | 0x7f800000u), 0.f);
  const float hi = __uint_as_float(sgn | ((unsigned)(e - 896) << 23) | ((h32 & 0xfffffu) << 3) | (l32 >> 29));
  float lo = 0.f;
  if (e >= 943) {
    // the 29 remaining bits rounded to 23 (half up; 2^23 when they carry), so
    // the split error is unbiased instead of always toward zero
    const unsigned t = ((l32 & 0x1fffffffu) + 32u) >> 6;
    const float f = __fsub_rn(__uint_as_float(0x4b000000u | t), 8388608.0f);  // = t exactly (t <= 2^23)
    lo = __fmul_rn(f, __uint_as_float(sgn | ((unsigned)(e - 942) << 23)));     // t * 2^(e-1069)
  }
  return make_float2(hi, lo);
}
__device__ __forceinline__ double djoin(float hi, float lo) { return (double)hi + (double)lo; }

// (hi, lo) += (ah + al) * (bh + bl): exact hi*hi product, cross terms into lo
__device__ __forceinline__ void df_fma(float& hi, float& lo, float2 a, float2 b) {
  df_add_prod(hi, lo, a.x, b.x);
  lo = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, lo));
}
__device__ __forceinline__ float2 fneg2(float2 a) { return make_float2(-a.x, -a.y); }

template <class T>
struct SplitLd;
template <>
struct SplitLd<double2> {
  static __device__ __forceinline__ float4 ld(const double2 a) {
    const float2 r = dsplit(a.x), i = dsplit(a.y);
    return make_float4(r.x, r.y, i.x, i.y);
  }
};
template <>
struct SplitLd<float2> {
  static __device__ __forceinline__ float4 ld(const float2 a) { return make_float4(a.x, 0.f, a.y, 0.f); }
};

}  // namespace qs3g
