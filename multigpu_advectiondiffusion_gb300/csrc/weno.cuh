// weno.cuh -- WENO5-JS / WENO5-Z face reconstruction for the Lax-Friedrichs split Burgers flux.
//
// Face flux at i+1/2:  F = R(f+_{i-2..i+2}) + R(f-_{i+3..i-1} reversed), where R is the
// left-biased 5-point reconstruction of SingleGPU/Burgers3d_WENO5/kernels.cu:142-192 (WENO5-Z)
// and :92-140 (WENO5-JS); the right-biased half of those functions is R applied to the
// mirrored stencil (same smoothness indicators, linear weights 0.1/0.6/0.3 reversed).
//
// Two forms:
//  * weno_face_ref<double>: the reference's own expression, operand for operand, with
//    correctly rounded intrinsics -> equal to the FP64 oracle bit for bit.
//  * weno_side_fast<D>: the same weights with the common denominator b0*b1*b2 (WENO5-Z) or
//    (b0*b1*b2)^2 (WENO5-JS) multiplied through, leaving ONE division per side instead of four;
//    D selects that division: float (IEEE), double (FP64) or FastDiv (reciprocal based,
//    at most 2 ulp). Used for the FP32 state.
#pragma once
#include "adv_math.cuh"

namespace adv {

// Lax-Friedrichs split of f(u) = u^2/2 (kernels.cu:224-238): f+- = (f +- a u)/2.
// lf_split: the reference's operand order, correctly rounded (FP64 path, reference operators).
// lf_split_fast: u * (u/4 +- a/2), the FP32 path.
__device__ __forceinline__ void lf_split_fast(float u, float a, float& fp, float& fm) {
  const float hu = 0.25f * u, ha = 0.5f * a;
  fp = u * (hu + ha);
  fm = u * (hu - ha);
}
template <class T>
__device__ __forceinline__ void lf_split(T u, T a, T& fp, T& fm) {
  const T f = mul_rn(mul_rn(T(0.5), u), u);
  const T au = mul_rn(a, u);
  fp = mul_rn(T(0.5), add_rn(f, au));
  fm = mul_rn(T(0.5), sub_rn(f, au));
}

// ---------------------------------------------------------------- fast FP32 form
struct FastDiv {};  // division tag: __fdividef (reciprocal approximation, <= 2 ulp)
template <class D>
__device__ __forceinline__ float side_div(float num, float den) { return (float)((D)num / (D)den); }
template <>
__device__ __forceinline__ float side_div<FastDiv>(float num, float den) { return __fdividef(num, den); }

// Left-biased side of one face from a..e = f at i-2..i+2. With the second differences
// t0 = a-2b+c, t1 = b-2c+d, t2 = c-2d+e and first differences s0 = a-4b+3c, s1 = b-d,
// s2 = 3c-4d+e, the reference's quantities are
//   beta_k = 13/12 t_k^2 + 1/4 s_k^2,   q_k/6 = c + t_k/12 + s0/4 | - s1/4 | - s2/4
// (q_0 = 2a-7b+11c, q_1 = -b+5c+2d, q_2 = 2c+5d-e). The kernel uses 4 beta_k and 4 eps (the
// factor cancels in the normalised weights), linear weights times 10 (1, 6, 3), and the
// weighted mean of q_k/6, so each side costs one division and no separate scaling.
template <bool Z, class D>
__device__ __forceinline__ float weno_side_fast(float a, float b, float c, float d, float e) {
  const float t0 = fmaf(-2.f, b, a) + c, t1 = fmaf(-2.f, c, b) + d, t2 = fmaf(-2.f, d, c) + e;
  const float s0 = fmaf(3.f, c, fmaf(-4.f, b, a)), s1 = b - d, s2 = fmaf(3.f, c, fmaf(-4.f, d, e));
  const float k = 13.f / 3.f;
  const float b0 = fmaf(k * t0, t0, fmaf(s0, s0, 4e-6f));  // 4 (beta_k + eps)
  const float b1 = fmaf(k * t1, t1, fmaf(s1, s1, 4e-6f));
  const float b2 = fmaf(k * t2, t2, fmaf(s2, s2, 4e-6f));
  const float r12 = 1.f / 12.f;
  const float q0 = fmaf(0.25f, s0, fmaf(r12, t0, c));
  const float q1 = fmaf(-0.25f, s1, fmaf(r12, t1, c));
  const float q2 = fmaf(-0.25f, s2, fmaf(r12, t2, c));
  float w0, w1, w2;
  if (Z) {  // alpha_k = d_k (1 + tau/b_k), times 10 b0 b1 b2: d_k (P + tau P/b_k), P = b0 b1 b2
    const float tau = fabsf(b0 - b2);
    const float p12 = b1 * b2, P = b0 * p12;
    w0 = fmaf(tau, p12, P);
    w1 = 6.f * fmaf(tau, b0 * b2, P);
    w2 = 3.f * fmaf(tau, b0 * b1, P);
  } else {  // alpha_k = d_k / b_k^2, times 10 (b0 b1 b2)^2
    const float p12 = b1 * b2, p02 = b0 * b2, p01 = b0 * b1;
    w0 = p12 * p12;
    w1 = (6.f * p02) * p02;
    w2 = (3.f * p01) * p01;
  }
  const float num = fmaf(w2, q2, fmaf(w1, q1, w0 * q0));
  const float den = w0 + w1 + w2;
  return side_div<D>(num, den);
}

// f+ at i-2..i+2 (p0..p4) and f- at i-1..i+3 (m0..m4).
template <bool Z, class D>
__device__ __forceinline__ float weno_face_fast(float p0, float p1, float p2, float p3, float p4, float m0, float m1,
                                                float m2, float m3, float m4) {
  return weno_side_fast<Z, D>(p0, p1, p2, p3, p4) + weno_side_fast<Z, D>(m4, m3, m2, m1, m0);
}

// ------------------------------------------------------- packed FP32 (two faces at once)
// The same operations as weno_side_fast / weno_face_fast / lf_split_fast on two independent
// inputs, issued as Blackwell's paired FP32 instructions (FFMA2 / FADD2 / FMUL2, one
// instruction for both lanes, each lane rounded exactly as the scalar form): the results are the
// scalar results bit for bit at half the FP32 instruction count. a - b is issued as
// fma(b, -1, a), which rounds the exact difference once, like a subtraction.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ void lf_split_fast2(float2 u, float2 a, float2& fp, float2& fm) {
  const float2 hu = mul2(f2(0.25f), u), ha = mul2(f2(0.5f), a);
  fp = mul2(u, add2(hu, ha));
  fm = mul2(u, sub2(hu, ha));
}

template <bool Z, class D>
__device__ __forceinline__ float2 weno_side_fast2(float2 a, float2 b, float2 c, float2 d, float2 e) {
  const float2 t0 = add2(fma2(f2(-2.f), b, a), c), t1 = add2(fma2(f2(-2.f), c, b), d),
               t2 = add2(fma2(f2(-2.f), d, c), e);
  const float2 s0 = fma2(f2(3.f), c, fma2(f2(-4.f), b, a)), s1 = sub2(b, d),
               s2 = fma2(f2(3.f), c, fma2(f2(-4.f), d, e));
  const float2 k = f2(13.f / 3.f);
  const float2 b0 = fma2(mul2(k, t0), t0, fma2(s0, s0, f2(4e-6f)));
  const float2 b1 = fma2(mul2(k, t1), t1, fma2(s1, s1, f2(4e-6f)));
  const float2 b2 = fma2(mul2(k, t2), t2, fma2(s2, s2, f2(4e-6f)));
  const float2 r12 = f2(1.f / 12.f);
  const float2 q0 = fma2(f2(0.25f), s0, fma2(r12, t0, c));
  const float2 q1 = fma2(f2(-0.25f), s1, fma2(r12, t1, c));
  const float2 q2 = fma2(f2(-0.25f), s2, fma2(r12, t2, c));
  float2 w0, w1, w2;
  if (Z) {
    const float2 dd = sub2(b0, b2);
    const float2 tau = make_float2(fabsf(dd.x), fabsf(dd.y));
    const float2 p12 = mul2(b1, b2), P = mul2(b0, p12);
    w0 = fma2(tau, p12, P);
    w1 = mul2(f2(6.f), fma2(tau, mul2(b0, b2), P));
    w2 = mul2(f2(3.f), fma2(tau, mul2(b0, b1), P));
  } else {
    const float2 p12 = mul2(b1, b2), p02 = mul2(b0, b2), p01 = mul2(b0, b1);
    w0 = mul2(p12, p12);
    w1 = mul2(mul2(f2(6.f), p02), p02);
    w2 = mul2(mul2(f2(3.f), p01), p01);
  }
  const float2 num = fma2(w2, q2, fma2(w1, q1, mul2(w0, q0)));
  const float2 den = add2(add2(w0, w1), w2);
  return make_float2(side_div<D>(num.x, den.x), side_div<D>(num.y, den.y));
}

template <bool Z, class D>
__device__ __forceinline__ float2 weno_face_fast2(float2 p0, float2 p1, float2 p2, float2 p3, float2 p4, float2 m0,
                                                  float2 m1, float2 m2, float2 m3, float2 m4) {
  return add2(weno_side_fast2<Z, D>(p0, p1, p2, p3, p4), weno_side_fast2<Z, D>(m4, m3, m2, m1, m0));
}

// ------------------------------------------------------------------- fast FP64 form
// weno_side_fast's common-denominator weights and contracted products for an FP64 state: one
// IEEE division per side instead of the reference form's four, and fused multiply-adds. The
// same function of the inputs as the reference form, rounded differently (a few ulps of the
// face value); selected for FP64 states with ADV_DIV_FAST.
template <bool Z>
__device__ __forceinline__ double weno_side_fast64(double a, double b, double c, double d, double e) {
  const double t0 = fma(-2.0, b, a) + c, t1 = fma(-2.0, c, b) + d, t2 = fma(-2.0, d, c) + e;
  const double s0 = fma(3.0, c, fma(-4.0, b, a)), s1 = b - d, s2 = fma(3.0, c, fma(-4.0, d, e));
  const double k = 13.0 / 3.0;
  const double b0 = fma(k * t0, t0, fma(s0, s0, 4e-6));  // 4 (beta_k + eps)
  const double b1 = fma(k * t1, t1, fma(s1, s1, 4e-6));
  const double b2 = fma(k * t2, t2, fma(s2, s2, 4e-6));
  const double r12 = 1.0 / 12.0;
  const double q0 = fma(0.25, s0, fma(r12, t0, c));
  const double q1 = fma(-0.25, s1, fma(r12, t1, c));
  const double q2 = fma(-0.25, s2, fma(r12, t2, c));
  double w0, w1, w2;
  if (Z) {
    const double tau = fabs(b0 - b2);
    w0 = (b0 + tau) * (b1 * b2);
    w1 = (6.0 * (b1 + tau)) * (b0 * b2);
    w2 = (3.0 * (b2 + tau)) * (b0 * b1);
  } else {
    const double p12 = b1 * b2, p02 = b0 * b2, p01 = b0 * b1;
    w0 = p12 * p12;
    w1 = (6.0 * p02) * p02;
    w2 = (3.0 * p01) * p01;
  }
  const double num = fma(w2, q2, fma(w1, q1, w0 * q0));
  const double den = w0 + w1 + w2;
  return num / den;
}

template <bool Z>
__device__ __forceinline__ double weno_face_fast64(double p0, double p1, double p2, double p3, double p4, double m0,
                                                   double m1, double m2, double m3, double m4) {
  return weno_side_fast64<Z>(p0, p1, p2, p3, p4) + weno_side_fast64<Z>(m4, m3, m2, m1, m0);
}

__device__ __forceinline__ void lf_split_fast64(double u, double a, double& fp, double& fm) {
  const double hu = 0.25 * u, ha = 0.5 * a;
  fp = u * (hu + ha);
  fm = u * (hu - ha);
}

// ---------------------------------------------------------- reference literal form
// Operand order of kernels.cu:142-192 / :92-140 (and of the CPU oracle), correctly rounded.
// RECIP: the normalisation of SingleGPU/Burgers3d_WENO5_SharedMem/kernels.cu:51-198, which takes
// alphasum = 1/(a0 + a1 + a2) and multiplies by (1/6)*alphasum instead of dividing by 6*alphasum.
template <bool Z, class T, bool RECIP = false>
__device__ __forceinline__ T weno_face_ref(T vmm, T vm, T v, T vp, T vpp, T umm, T um, T u, T up, T upp) {
  const T c1312 = T(13. / 12.), c14 = T(1. / 4.), eps = T(1e-6);
  auto beta = [&](T a, T b, T c, T d, T e, T& B0, T& B1, T& B2) {
    const T A0 = add_rn(sub_rn(a, mul_rn(T(2), b)), c);
    const T C0 = add_rn(sub_rn(a, mul_rn(T(4), b)), mul_rn(T(3), c));
    B0 = add_rn(mul_rn(mul_rn(c1312, A0), A0), mul_rn(mul_rn(c14, C0), C0));
    const T A1 = add_rn(sub_rn(b, mul_rn(T(2), c)), d);
    const T C1 = sub_rn(b, d);
    B1 = add_rn(mul_rn(mul_rn(c1312, A1), A1), mul_rn(mul_rn(c14, C1), C1));
    const T A2 = add_rn(sub_rn(c, mul_rn(T(2), d)), e);
    const T C2 = add_rn(sub_rn(mul_rn(T(3), c), mul_rn(T(4), d)), e);
    B2 = add_rn(mul_rn(mul_rn(c1312, A2), A2), mul_rn(mul_rn(c14, C2), C2));
  };
  auto weights = [&](T B0, T B1, T B2, T d0, T d1, T d2, T& a0, T& a1, T& a2) {
    if (Z) {
      const T tau5 = fabs(sub_rn(B0, B2));
      a0 = mul_rn(d0, add_rn(T(1), div_rn(tau5, add_rn(B0, eps))));
      a1 = mul_rn(d1, add_rn(T(1), div_rn(tau5, add_rn(B1, eps))));
      a2 = mul_rn(d2, add_rn(T(1), div_rn(tau5, add_rn(B2, eps))));
    } else {
      a0 = div_rn(d0, mul_rn(add_rn(eps, B0), add_rn(eps, B0)));
      a1 = div_rn(d1, mul_rn(add_rn(eps, B1), add_rn(eps, B1)));
      a2 = div_rn(d2, mul_rn(add_rn(eps, B2), add_rn(eps, B2)));
    }
  };
  T B0, B1, B2, a0, a1, a2;
  beta(vmm, vm, v, vp, vpp, B0, B1, B2);
  weights(B0, B1, B2, T(1. / 10.), T(6. / 10.), T(3. / 10.), a0, a1, a2);
  T asum = add_rn(add_rn(a0, a1), a2);
  const T q0m = add_rn(sub_rn(mul_rn(T(2), vmm), mul_rn(T(7), vm)), mul_rn(T(11), v));
  const T q1m = add_rn(add_rn(-vm, mul_rn(T(5), v)), mul_rn(T(2), vp));
  const T q2m = sub_rn(add_rn(mul_rn(T(2), v), mul_rn(T(5), vp)), vpp);
  auto normalise = [&](T num, T sum) {
    return RECIP ? mul_rn(num, mul_rn(T(1. / 6.), div_rn(T(1), sum))) : div_rn(num, mul_rn(T(6), sum));
  };
  const T fm = normalise(add_rn(add_rn(mul_rn(a0, q0m), mul_rn(a1, q1m)), mul_rn(a2, q2m)), asum);

  beta(umm, um, u, up, upp, B0, B1, B2);
  weights(B0, B1, B2, T(3. / 10.), T(6. / 10.), T(1. / 10.), a0, a1, a2);
  asum = add_rn(add_rn(a0, a1), a2);
  const T q0p = add_rn(add_rn(-umm, mul_rn(T(5), um)), mul_rn(T(2), u));
  const T q1p = sub_rn(add_rn(mul_rn(T(2), um), mul_rn(T(5), u)), up);
  const T q2p = add_rn(sub_rn(mul_rn(T(11), u), mul_rn(T(7), up)), mul_rn(T(2), upp));
  const T fp = normalise(add_rn(add_rn(mul_rn(a0, q0p), mul_rn(a1, q1p)), mul_rn(a2, q2p)), asum);
  return add_rn(fm, fp);
}

}  // namespace adv
