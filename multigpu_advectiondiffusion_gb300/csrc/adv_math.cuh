// adv_math.cuh -- correctly rounded scalar ops that the compiler may not contract into FMAs.
// The heat stage and the FP64 WENO path evaluate their expressions in the reference's operand
// order with these, so results match the CPU oracle (built with -ffp-contract=off) bit for bit.
#pragma once
#include <cuda_runtime.h>

namespace adv {

__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

// Two FP32 lanes at once with Blackwell's paired instructions (FADD2 / FMUL2 / FFMA2): each lane
// is rounded exactly as the scalar operation, so packed code gives the scalar results bit for
// bit. a - b is issued as fma(b, -1, a) (one rounding of the exact difference).
__device__ __forceinline__ float2 add_rn(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub_rn(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul_rn(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 div_rn(float2 a, float2 b) {
  return make_float2(__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y));
}
__device__ __forceinline__ float2 operator-(float2 a) { return make_float2(-a.x, -a.y); }

// A constant of type T (both lanes for float2).
template <class T> __device__ __forceinline__ T bc(double v) { return T(v); }
template <> __device__ __forceinline__ float2 bc<float2>(double v) { return make_float2((float)v, (float)v); }

// SSP-RK3 stage combination (stage 1 is forward Euler), operand order of
// SingleGPU/Diffusion3d_baselineCode/kernels.cu:130-138:
//   1: un + dt*L;  2: 0.75*un + 0.25*(uin + dt*L);  3: (un + 2*(uin + dt*L)) / 3
template <class T>
__device__ __forceinline__ T stage_combine(int stage, T un, T uin, T dt, T L) {
  if (stage == 2) return add_rn(mul_rn(T(0.75), un), mul_rn(T(0.25), add_rn(uin, mul_rn(dt, L))));
  if (stage == 3) return div_rn(add_rn(un, mul_rn(T(2), add_rn(uin, mul_rn(dt, L)))), T(3));
  return add_rn(un, mul_rn(dt, L));
}

}  // namespace adv
