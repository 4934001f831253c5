// vpm_device.cuh — device-side kernel functions of the rVPM pair sums.
//
// The regularised Biot–Savart law (FLOWUnsteady docs/src/theory/rvpm.md:88-99)
//   U(x) = -1/(4π) Σ_j q_j(r) (Δx × Γ_j),  q(r) = g(r/σ_j)/r³,  Δx = x - x_j
// and its gradient
//   J_ab = dU_a/dx_b = -1/(4π) Σ_j [ (q'(r)/r) (Δx×Γ_j)_a Δx_b + q(r) ε_abc Γ_jc ].
// A pair contributes (q, p) with p = KP·(q'/r): the accumulators hold
//   Uacc = Σ q c,  Aacc = Σ p c⊗Δx,  Wacc = Σ q Γ      (c = Δx × Γ)
// and the epilogue forms U = -Uacc/(4π), J = -(Aacc/KP + ε·Wacc)/(4π).
//
// Kernels (Winckelmans & Leonard 1993; Gaussian-erf), with ρ = r/σ:
//   Winckelmans: q = (r²+5/2σ²)/(r²+σ²)^{5/2},  q'/r = -3 (r²+7/2σ²)/(r²+σ²)^{7/2},
//                ζ(ρ) = 15/(8π) (ρ²+1)^{-7/2}.   Accumulated p = (r²+7/2σ²)/(r²+σ²)^{7/2}, KP = -1/3.
//   Gaussian-erf: g = erf(ρ/√2) - √(2/π) ρ e^{-ρ²/2},  g' = √(2/π) ρ² e^{-ρ²/2},
//                q'/r = (ρ g' - 3 g)/r⁵,  ζ(ρ) = (2π)^{-3/2} e^{-ρ²/2}.  Accumulated p = q'/r, KP = 1.
//   For small ρ the Gaussian-erf forms cancel; they are replaced by the series
//   (derived from g(ρ) = √(2/π) ∫_0^ρ t² e^{-t²/2} dt), in x = ρ²:
//     g/ρ³        =  √(2/π) Σ_n (-1/2)^n xⁿ / (n! (2n+3))
//     (ρg'-3g)/ρ⁵ = -√(2/π) Σ_n (-1/2)^n xⁿ / (n! (2n+5))
//   so q = (g/ρ³)/σ³ and q'/r = ((ρg'-3g)/ρ⁵)/σ⁵.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vpm_gpu.h"

namespace vpm {

constexpr double kPi = 3.14159265358979323846;
constexpr double kInv4Pi = 1.0 / (4.0 * kPi);
constexpr double kSqrt2overPi = 0.79788456080286535588;
constexpr double kInvSqrt2 = 0.70710678118654752440;
constexpr double kLog2e = 1.44269504088896340736;
constexpr double kZeta0Winck = 15.0 / (8.0 * kPi);
constexpr double kZeta0Gauss = 0.06349363593424096978;  // (2π)^{-3/2}

// ρ² below which the Gaussian-erf series replaces the direct forms.
constexpr float kSeriesRho2F = 0.5f;
constexpr double kSeriesRho2D = 0.25;

__host__ __device__ inline double zeta0_of(int kernel) {
  return kernel == VPM_KERNEL_WINCKELMANS ? kZeta0Winck : kZeta0Gauss;
}

// Series coefficients c_n = (-1/2)^n/(n!(2n+3)) and d_n = (-1/2)^n/(n!(2n+5)),
// n = 0..13 (evaluated exactly in double precision from the definition).
// The switch folds to immediates once the Horner loop below is unrolled.
__host__ __device__ constexpr double ser_c(int n) {
  switch (n) {
    case 0: return 0.3333333333333333;       case 1: return -0.1;
    case 2: return 0.017857142857142856;     case 3: return -0.0023148148148148147;
    case 4: return 0.00023674242424242425;   case 5: return -2.0032051282051282e-05;
    case 6: return 1.4467592592592592e-06;   case 7: return -9.118230625583566e-08;
    case 8: return 5.099010547201337e-09;    case 9: return -2.5629947194927355e-10;
    case 10: return 1.1700628067249444e-11;  case 11: return -4.892989919031586e-13;
    case 12: return 1.887727592218976e-14;   default: return -6.759767240041426e-16;
  }
}
__host__ __device__ constexpr double ser_d(int n) {
  switch (n) {
    case 0: return 0.2;                      case 1: return -0.07142857142857142;
    case 2: return 0.013888888888888888;     case 3: return -0.001893939393939394;
    case 4: return 0.00020032051282051281;   case 5: return -1.736111111111111e-05;
    case 6: return 1.2765522875816993e-06;   case 7: return -8.158416875522139e-08;
    case 8: return 4.613390495086924e-09;    case 9: return -2.340125613449889e-10;
    case 10: return 1.0764577821869489e-11;  case 11: return -4.5305462213255424e-13;
    case 12: return 1.7575394824107708e-14;  default: return -6.323653224554882e-16;
  }
}

// h1 = g/ρ³ and h2 = (ρg'-3g)/ρ⁵ by Horner's rule over the first N terms.
template <typename R, int N>
struct GaussSeries {
  __device__ static inline void eval(R x, R& h1, R& h2) {
    R s1 = R(0), s2 = R(0);
#pragma unroll
    for (int n = N - 1; n >= 0; --n) {
      s1 = s1 * x + R(ser_c(n));
      s2 = s2 * x + R(ser_d(n));
    }
    h1 = R(kSqrt2overPi) * s1;
    h2 = -R(kSqrt2overPi) * s2;
  }
};

// Per-source constants of the pair functions (computed once per source while
// the tile is staged).
//   Winckelmans:  a = σ²,   b = 5/2 σ² (so r²+σ²+b·... forms below)
//   Gaussian-erf: a = 1/σ², b = 1/σ
template <int KERNEL, typename R>
__device__ inline void source_consts(double sig, R& a, R& b) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    a = R(sig * sig);
    b = R(1.5 * sig * sig);
  } else {
    a = R(1.0 / (sig * sig));
    b = R(1.0 / sig);
  }
}

// (q, p) of one pair from r² and the source constants; the pair is dropped
// (q = p = 0) when r² == 0.
__device__ inline void pair_qp_f32_winck(float r2, float s2, float k15, float& q, float& p) {
  const float s = r2 + s2;
  const float rs = rsqrtf(s);
  const float rs2 = rs * rs;
  const float rs3 = rs2 * rs;
  const float rs5 = rs3 * rs2;
  const float rs7 = rs5 * rs2;
  q = fmaf(k15, rs5, rs3);             // (s + 3/2σ²)/s^{5/2} = (r²+5/2σ²)/s^{5/2}
  p = fmaf(k15 + s2, rs7, rs5);        // (s + 5/2σ²)/s^{7/2} = (r²+7/2σ²)/s^{7/2}
  q = r2 > 0.f ? q : 0.f;
}

__device__ inline void pair_qp_f32_gauss(float r2, float is2, float is1, float& q, float& p) {
  const float rho2 = r2 * is2;
  if (rho2 < kSeriesRho2F) {
    float h1, h2;
    GaussSeries<float, 8>::eval(rho2, h1, h2);
    const float is3 = is2 * is1;
    q = h1 * is3;
    p = h2 * is3 * is2;
    q = r2 > 0.f ? q : 0.f;
    p = r2 > 0.f ? p : 0.f;
  } else {
    const float ri = rsqrtf(r2);
    const float rho = r2 * ri * is1;
    const float e = exp2f(rho2 * float(-0.5 * kLog2e));
    const float g = erff(rho * float(kInvSqrt2)) - float(kSqrt2overPi) * rho * e;
    const float ri2 = ri * ri;
    const float ri3 = ri2 * ri;
    q = g * ri3;
    p = fmaf(float(kSqrt2overPi) * rho * rho2, e, -3.f * g) * ri3 * ri2;
  }
}

__device__ inline void pair_qp_f64_winck(double r2, double s2, double k15, double& q, double& p) {
  const double s = r2 + s2;
  const double rs = rsqrt(s);
  const double rs2 = rs * rs;
  const double rs5 = rs2 * rs2 * rs;
  const double rs7 = rs5 * rs2;
  q = (r2 + (s2 + k15)) * rs5;
  p = (r2 + (s2 + k15 + s2)) * rs7;
  q = r2 > 0.0 ? q : 0.0;
}

__device__ inline void pair_qp_f64_gauss(double r2, double is2, double is1, double& q, double& p) {
  const double rho2 = r2 * is2;
  if (rho2 < kSeriesRho2D) {
    double h1, h2;
    GaussSeries<double, 14>::eval(rho2, h1, h2);
    const double is3 = is2 * is1;
    q = h1 * is3;
    p = h2 * is3 * is2;
    q = r2 > 0.0 ? q : 0.0;
    p = r2 > 0.0 ? p : 0.0;
  } else {
    const double r = sqrt(r2);
    const double rho = r * is1;
    const double e = exp(-0.5 * rho2);
    const double g = erf(rho * kInvSqrt2) - kSqrt2overPi * rho * e;
    const double ir2 = 1.0 / r2;
    const double ir3 = ir2 / r;
    q = g * ir3;
    p = (kSqrt2overPi * rho2 * rho * e - 3.0 * g) * ir3 * ir2;
  }
}

template <int KERNEL>
__device__ inline void pair_qp(float r2, float a, float b, float& q, float& p) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) pair_qp_f32_winck(r2, a, b, q, p);
  else pair_qp_f32_gauss(r2, a, b, q, p);
}
template <int KERNEL>
__device__ inline void pair_qp(double r2, double a, double b, double& q, double& p) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) pair_qp_f64_winck(r2, a, b, q, p);
  else pair_qp_f64_gauss(r2, a, b, q, p);
}

// Factor that turns the accumulated p into q'/r.
template <int KERNEL>
__host__ __device__ constexpr double kp_to_qr() {
  return KERNEL == VPM_KERNEL_WINCKELMANS ? -3.0 : 1.0;
}

// ζ_σ(r) = ζ(r/σ)/σ³ per pair from r² and source constants
//   Winckelmans:  a = 1/σ², b = 15/(8π)/σ³   -> b (r²a + 1)^{-7/2}
//   Gaussian-erf: a = -log2(e)/(2σ²), b = (2π)^{-3/2}/σ³ -> b 2^{r² a}
template <int KERNEL, typename R>
__device__ inline void zeta_consts(double sig, R& a, R& b) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    a = R(1.0 / (sig * sig));
    b = R(kZeta0Winck / (sig * sig * sig));
  } else {
    a = R(-0.5 * kLog2e / (sig * sig));
    b = R(kZeta0Gauss / (sig * sig * sig));
  }
}

template <int KERNEL>
__device__ inline float pair_zeta(float r2, float a, float b) {
  float z;
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    const float rs = rsqrtf(fmaf(r2, a, 1.f));
    const float rs2 = rs * rs;
    const float rs4 = rs2 * rs2;
    z = b * rs4 * rs2 * rs;
  } else {
    z = b * exp2f(r2 * a);
  }
  return r2 > 0.f ? z : 0.f;
}
template <int KERNEL>
__device__ inline double pair_zeta(double r2, double a, double b) {
  double z;
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    const double s = fma(r2, a, 1.0);
    const double rs = rsqrt(s);
    const double rs2 = rs * rs;
    z = b * rs2 * rs2 * rs2 * rs;
  } else {
    z = b * exp2(r2 * a);
  }
  return r2 > 0.0 ? z : 0.0;
}

// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest, no reassociation).
__device__ inline void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fadd_rn(s, -a);
  const float ap = __fadd_rn(s, -bp);
  e = __fadd_rn(__fadd_rn(a, -ap), __fadd_rn(b, -bp));
}

}  // namespace vpm
