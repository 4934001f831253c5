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

// ρ² below which the FP64 Gaussian-erf series replaces the direct forms.
constexpr double kSeriesRho2D = 0.25;
// FP64 Gaussian-erf far form: for ρ² >= 90, e^{-ρ²/2}(erfcx(ρ/√2) + √(2/π)ρ) <
// 3e-19 and √(2/π)ρ³e^{-ρ²/2}/3 < 7e-18, both below half an FP64 ulp of 1,
// so g = 1 and q'/r = -3/r⁵ to FP64 rounding.
constexpr double kFarRho2D = 90.0;

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
//   (FP32 Gaussian-erf: a = -log2(e)/(2σ²), the exponent scale of e^{-ρ²/2})
template <int KERNEL, typename R>
__device__ inline void source_consts(double sig, R& a, R& b) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    a = R(sig * sig);
    b = R(1.5 * sig * sig);
  } else if (sizeof(R) == sizeof(float)) {
    a = R(-0.5 * kLog2e / (sig * sig));
    b = R(1.0 / sig);
  } else {
    a = R(1.0 / (sig * sig));
    b = R(1.0 / sig);
  }
}

// (q, p) of one FP64 pair from r² and the source constants; the pair is
// dropped (q = p = 0) when r² == 0.
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
  if (rho2 >= kFarRho2D) {   // no erf or exp (see kFarRho2D)
    const double ri = rsqrt(r2);
    const double ri2 = ri * ri;
    q = ri2 * ri;
    p = -3.0 * q * ri2;
    return;
  }
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

__device__ __forceinline__ float rsqrt_ftz(float x);
__device__ __forceinline__ float ex2_ftz(float x);

template <int KERNEL>
__device__ inline float pair_zeta(float r2, float a, float b) {
  float z;
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    const float rs = rsqrt_ftz(fmaf(r2, a, 1.f));
    const float rs2 = rs * rs;
    const float rs4 = rs2 * rs2;
    z = b * rs4 * rs2 * rs;
  } else {
    z = b * ex2_ftz(r2 * a);
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

// x ≈ h + l with h the float nearest x and l the float nearest x - h.
__host__ __device__ inline void split_f32(double x, float& h, float& l) {
  h = float(x);
  l = float(x - double(h));
}

// Position relative to a reference point, both in (h, l) form.  h - ch is
// taken exactly as s + e (Knuth's TwoSum), then s + (e + (l - cl)) is rounded
// once more: the result is the float nearest (h + l) - (ch + cl) except in
// rare double-rounding ties, as if the FP64 difference were rounded to FP32.
__device__ __forceinline__ float rel_f32(float h, float l, float ch, float cl) {
  const float s = __fadd_rn(h, -ch);
  const float bp = __fadd_rn(s, -h);
  const float ap = __fadd_rn(s, -bp);
  const float e = __fadd_rn(__fadd_rn(h, -ap), __fadd_rn(-ch, -bp));
  return __fadd_rn(s, __fadd_rn(e, __fadd_rn(l, -cl)));
}

// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest, no reassociation).
__device__ inline void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fadd_rn(s, -a);
  const float ap = __fadd_rn(s, -bp);
  e = __fadd_rn(__fadd_rn(a, -ap), __fadd_rn(b, -bp));
}

}  // namespace vpm

// ------------------------------------------------------------------------------
// FP32 pair routines of the U/∇U pass: one staged source against the T targets
// a thread holds.  They use the hardware approximations of the PTX ISA
// (rsqrt/ex2/rcp .approx.ftz) directly, one SFU instruction each.
namespace vpm {

__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float ex2_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Gaussian-erf for ρ² >= 3/2, without erf:
//   g(ρ) = erf(x) - √(2/π) ρ e^{-x²} = 1 - e^{-x²} (erfcx(x) + √(2/π) ρ),  x = ρ/√2,
// with erfcx(x) = e^{x²} erfc(x) ≈ t (a1 + t (a2 + t (a3 + t a4))), t = 1/(1 + P x).
// This is the structure of Hastings' approximation (Abramowitz & Stegun 7.1.26);
// P and a1..a4 were fitted for this code by Lawson-reweighted least squares to
// minimise the relative error of g over ρ in [1, 9] (max 7.5e-8; beyond ρ = 9
// the e^{-x²} factor is below 2e-18).  For ρ² < 3/2 the power series is used
// (10 terms); in FP32 the worst pair errors are then 4.4e-7 in q and 1.8e-6 in
// q'/r, both at the switch point where ρg' - 3g cancels.
constexpr float kErfcxP = 0.47729708f;  // P/√2: t = 1/(1 + kErfcxP ρ)
constexpr float kErfcxA1 = 0.39182437f;
constexpr float kErfcxA2 = 0.28743228f;
constexpr float kErfcxA3 = 0.59069124f;
constexpr float kErfcxA4 = -0.27144525f;
// ρ² = 3/2 expressed in the exponent argument r²·(-log2(e)/(2σ²)).
constexpr float kArgSeries = float(-0.5 * kLog2e * 1.5);
constexpr float kArgToRho2 = float(-2.0 / kLog2e);

// Accumulate one pair into the 14 FP32 sums of a target (A22 is not kept:
// J is trace-free pair by pair, c·Δx = 0, and the epilogue sets
// A22 = -(A00 + A11)).  acc: U 0..2, A 3..11 (11 unused), W 12..14.
__device__ __forceinline__ void accum_pair(float dx, float dy, float dz, float q, float p,
                                           float gx, float gy, float gz, float* acc) {
  const float c0 = dy * gz - dz * gy;
  const float c1 = dz * gx - dx * gz;
  const float c2 = dx * gy - dy * gx;
  acc[0] = fmaf(q, c0, acc[0]);
  acc[1] = fmaf(q, c1, acc[1]);
  acc[2] = fmaf(q, c2, acc[2]);
  const float p0 = p * c0, p1 = p * c1, p2 = p * c2;
  acc[3] = fmaf(p0, dx, acc[3]);
  acc[4] = fmaf(p0, dy, acc[4]);
  acc[5] = fmaf(p0, dz, acc[5]);
  acc[6] = fmaf(p1, dx, acc[6]);
  acc[7] = fmaf(p1, dy, acc[7]);
  acc[8] = fmaf(p1, dz, acc[8]);
  acc[9] = fmaf(p2, dx, acc[9]);
  acc[10] = fmaf(p2, dy, acc[10]);
  acc[12] = fmaf(q, gx, acc[12]);
  acc[13] = fmaf(q, gy, acc[13]);
  acc[14] = fmaf(q, gz, acc[14]);
}

// ---- packed FP32 -------------------------------------------------------------
// For an even number of targets per thread the routines below work on target
// pairs (k, k+1) with the packed FP32 instructions of sm_100+ (add/mul/fma
// .rn.f32x2): each lane rounds exactly as the scalar instruction does, and one
// issue slot carries two pair updates.  The SFU approximations stay scalar.
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// One staged source as broadcast pairs: -x (for the differences), Γ and -Γ.
struct Src2 {
  float2 nx, ny, nz, gx, gy, gz, ngx, ngy, ngz;
  __device__ __forceinline__ Src2(const float4 sa, const float4 sb)
      : nx(bc2(-sa.x)), ny(bc2(-sa.y)), nz(bc2(-sa.z)), gx(bc2(sb.x)), gy(bc2(sb.y)),
        gz(bc2(sb.z)), ngx(bc2(-sb.x)), ngy(bc2(-sb.y)), ngz(bc2(-sb.z)) {}
};

// acc[k][v] += a.x·b.x, acc[k+1][v] += a.y·b.y.
template <int T, int NV>
__device__ __forceinline__ void fma_acc2(float (&acc)[T][NV], int k, int v, float2 a, float2 b) {
  const float2 r = fma2(a, b, make_float2(acc[k][v], acc[k + 1][v]));
  acc[k][v] = r.x;
  acc[k + 1][v] = r.y;
}

// Differences and r² of targets (k, k+1) to the source.
template <int T>
__device__ __forceinline__ void diff2(const float (&tx)[T], const float (&ty)[T],
                                      const float (&tz)[T], int k, const Src2& s, float2& dx,
                                      float2& dy, float2& dz, float2& r2) {
  dx = add2(make_float2(tx[k], tx[k + 1]), s.nx);
  dy = add2(make_float2(ty[k], ty[k + 1]), s.ny);
  dz = add2(make_float2(tz[k], tz[k + 1]), s.nz);
  r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
}

// accum_pair for targets (k, k+1).
template <int T, int NV>
__device__ __forceinline__ void accum_pair2(float2 dx, float2 dy, float2 dz, float2 q, float2 p,
                                            const Src2& s, float (&acc)[T][NV], int k) {
  const float2 c0 = fma2(dz, s.ngy, mul2(dy, s.gz));
  const float2 c1 = fma2(dx, s.ngz, mul2(dz, s.gx));
  const float2 c2 = fma2(dy, s.ngx, mul2(dx, s.gy));
  fma_acc2(acc, k, 0, q, c0);
  fma_acc2(acc, k, 1, q, c1);
  fma_acc2(acc, k, 2, q, c2);
  const float2 p0 = mul2(p, c0), p1 = mul2(p, c1), p2 = mul2(p, c2);
  fma_acc2(acc, k, 3, p0, dx);
  fma_acc2(acc, k, 4, p0, dy);
  fma_acc2(acc, k, 5, p0, dz);
  fma_acc2(acc, k, 6, p1, dx);
  fma_acc2(acc, k, 7, p1, dy);
  fma_acc2(acc, k, 8, p1, dz);
  fma_acc2(acc, k, 9, p2, dx);
  fma_acc2(acc, k, 10, p2, dy);
  fma_acc2(acc, k, 12, q, s.gx);
  fma_acc2(acc, k, 13, q, s.gy);
  fma_acc2(acc, k, 14, q, s.gz);
}

// Winckelmans: source quads (x, y, z, σ²) and (Γx, Γy, Γz, 3/2 σ²).  MASK drops
// coincident pairs; the kernel sets it only for source tiles that can hold a
// target's own particle (the kernel is finite at r = 0, so an unmasked
// coincident pair adds the core term q(0) ε·Γ to J and nothing to U).
template <int T, bool MASK>
__device__ __forceinline__ void uj_source_winck(const float4 sa, const float4 sb,
                                                const float (&tx)[T], const float (&ty)[T],
                                                const float (&tz)[T], float (&acc)[T][15]) {
  const float s2 = sa.w, k15 = sb.w, k25 = sa.w + sb.w;
  if constexpr (T % 2 == 0) {
    const Src2 s(sa, sb);
    const float2 s2p = bc2(s2), k15p = bc2(k15), k25p = bc2(k25);
#pragma unroll
    for (int k = 0; k < T; k += 2) {
      float2 dx, dy, dz, r2, h;
      if (MASK) {
        diff2(tx, ty, tz, k, s, dx, dy, dz, r2);
        h = add2(r2, s2p);
      } else {   // r² + σ² in the same chain: r² itself is not needed
        dx = add2(make_float2(tx[k], tx[k + 1]), s.nx);
        dy = add2(make_float2(ty[k], ty[k + 1]), s.ny);
        dz = add2(make_float2(tz[k], tz[k + 1]), s.nz);
        h = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, s2p)));
      }
      const float2 rs = make_float2(rsqrt_ftz(h.x), rsqrt_ftz(h.y));
      const float2 rs2 = mul2(rs, rs);
      const float2 rs3 = mul2(rs2, rs);
      const float2 rs5 = mul2(rs3, rs2);
      const float2 rs7 = mul2(rs5, rs2);
      float2 q = fma2(k15p, rs5, rs3);
      if (MASK) {
        q.x = r2.x > 0.f ? q.x : 0.f;
        q.y = r2.y > 0.f ? q.y : 0.f;
      }
      const float2 p = fma2(k25p, rs7, rs5);
      accum_pair2(dx, dy, dz, q, p, s, acc, k);
    }
  } else {
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const float dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float rs = rsqrt_ftz(r2 + s2);
      const float rs2 = rs * rs;
      const float rs3 = rs2 * rs;
      const float rs5 = rs3 * rs2;
      const float rs7 = rs5 * rs2;
      float q = fmaf(k15, rs5, rs3);
      if (MASK) q = r2 > 0.f ? q : 0.f;
      const float p = fmaf(k25, rs7, rs5);
      accum_pair(dx, dy, dz, q, p, sb.x, sb.y, sb.z, acc[k]);
    }
  }
}

constexpr float kArgFar = float(-0.5 * kLog2e * 50.0);
constexpr float kArgZero = -128.f;

// uj_source_gauss on target pairs (T even; see "packed FP32").  g = 1 - e·h
// with h = kc·r + f is formed as fma(e, -h, 1), and -h from the negated
// coefficients, which rounds exactly as the scalar form.
template <int T, bool VOTE>
__device__ __forceinline__ void uj_source_gauss_x2(const float4 sa, const float4 sb,
                                                   const float (&tx)[T], const float (&ty)[T],
                                                   const float (&tz)[T], float (&acc)[T][15],
                                                   float kt, float kc, float k3) {
  constexpr int H = T / 2;
  const Src2 s(sa, sb);
  const float2 ea = bc2(sa.w), one = bc2(1.f);
  float2 dx[H], dy[H], dz[H], arg[H], ri[H], q[H], p[H];
  float amax = -INFINITY;
#pragma unroll
  for (int m = 0; m < H; ++m) {
    float2 r2;
    diff2(tx, ty, tz, 2 * m, s, dx[m], dy[m], dz[m], r2);
    arg[m] = mul2(r2, ea);
    amax = fmaxf(amax, fmaxf(arg[m].x, arg[m].y));
    ri[m] = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
    q[m] = r2;   // r², until the general form below replaces it by q
  }
  if (VOTE && __all_sync(0xffffffffu, amax <= kArgFar)) {
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const float2 ri2 = mul2(ri[m], ri[m]);
      const float2 qq = mul2(ri2, ri[m]);
      accum_pair2(dx[m], dy[m], dz[m], qq, mul2(qq, ri2), s, acc, 2 * m);
    }
    return;
  }
  const float2 ktp = bc2(kt), nkc = bc2(-kc), k3np = bc2(k3 * (-1.f / 3.f));
  const float2 nA4 = bc2(-kErfcxA4), nA3 = bc2(-kErfcxA3), nA2 = bc2(-kErfcxA2),
               nA1 = bc2(-kErfcxA1);
#pragma unroll
  for (int m = 0; m < H; ++m) {
    const float2 r = mul2(q[m], ri[m]);   // q holds r² here
    const float2 e = make_float2(ex2_ftz(arg[m].x), ex2_ftz(arg[m].y));
    const float2 u = fma2(ktp, r, one);
    const float2 t = make_float2(rcp_ftz(u.x), rcp_ftz(u.y));
    const float2 nf = mul2(t, fma2(t, fma2(t, fma2(t, nA4, nA3), nA2), nA1));
    const float2 g = fma2(e, fma2(nkc, r, nf), one);
    const float2 ri2 = mul2(ri[m], ri[m]);
    q[m] = mul2(g, mul2(ri2, ri[m]));
    p[m] = mul2(fma2(k3np, e, q[m]), ri2);
  }
  if (__any_sync(0xffffffffu, amax > kArgSeries)) {
    const float is1 = sb.w, is2 = is1 * is1, is3 = is2 * is1, is5n = is3 * is2 * (-1.f / 3.f);
#pragma unroll
    for (int m = 0; m < H; ++m) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float a = h ? arg[m].y : arg[m].x;
        if (a > kArgSeries) {
          float h1, h2;
          GaussSeries<float, 10>::eval(a * kArgToRho2, h1, h2);
          const bool self = a == 0.f;
          const float qs = self ? 0.f : h1 * is3, ps = self ? 0.f : h2 * is5n;
          if (h) { q[m].y = qs; p[m].y = ps; } else { q[m].x = qs; p[m].x = ps; }
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < H; ++m) accum_pair2(dx[m], dy[m], dz[m], q[m], p[m], s, acc, 2 * m);
}

// Gaussian-erf FP32 routines (U/J and α-derivative passes) accumulate
// p/(-3) instead of p = q'/r in the A sums, so that the far form's p is the one
// product q/r²; the kernels' epilogues multiply A by -3 (kGaussAScale).
constexpr double kGaussAScale = -3.0;

// Gaussian-erf: source quads (x, y, z, -log2(e)/(2σ²)) and (Γx, Γy, Γz, 1/σ).
// All T targets take the erf-free form, and a warp vote sends the rare warps
// holding a pair with ρ² < 3/2 (or the self pair) through the series.  With
// VOTE, a first warp vote takes the far form (q = 1/r³, p = -3/r⁵; see the
// far-field notes below) when every pair of the warp has ρ² >= 50; the caller
// uses it only for warps whose targets are compact enough for the vote to pay
// (it splits the straight-line code that overlaps the exp/rcp latencies).
template <int T, bool VOTE>
__device__ __forceinline__ void uj_source_gauss(const float4 sa, const float4 sb,
                                                const float (&tx)[T], const float (&ty)[T],
                                                const float (&tz)[T], float (&acc)[T][15]) {
  const float ea = sa.w, is1 = sb.w;
  const float kt = kErfcxP * is1;                      // t = 1/(1 + kt r)
  const float kc = float(kSqrt2overPi) * is1;          // √(2/π) ρ = kc r
  const float k3 = float(kSqrt2overPi) * is1 * is1 * is1;
  if constexpr (T % 2 == 0) {
    uj_source_gauss_x2<T, VOTE>(sa, sb, tx, ty, tz, acc, kt, kc, k3);
    return;
  }
  const float k3n = k3 * (-1.f / 3.f);
  float dx[T], dy[T], dz[T], arg[T], q[T], p[T];
  float amax = -INFINITY;
  if constexpr (VOTE) {
    float r2[T], ri[T];
#pragma unroll
    for (int k = 0; k < T; ++k) {
      dx[k] = tx[k] - sa.x;
      dy[k] = ty[k] - sa.y;
      dz[k] = tz[k] - sa.z;
      r2[k] = fmaf(dx[k], dx[k], fmaf(dy[k], dy[k], dz[k] * dz[k]));
      arg[k] = r2[k] * ea;
      amax = fmaxf(amax, arg[k]);
      ri[k] = rsqrt_ftz(r2[k]);
    }
    if (__all_sync(0xffffffffu, amax <= kArgFar)) {
#pragma unroll
      for (int k = 0; k < T; ++k) {
        const float ri2 = ri[k] * ri[k];
        const float qq = ri2 * ri[k];
        accum_pair(dx[k], dy[k], dz[k], qq, qq * ri2, sb.x, sb.y, sb.z, acc[k]);
      }
      return;
    }
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const float r = r2[k] * ri[k];
      const float e = ex2_ftz(arg[k]);
      const float t = rcp_ftz(fmaf(kt, r, 1.f));
      const float f = t * fmaf(t, fmaf(t, fmaf(t, kErfcxA4, kErfcxA3), kErfcxA2), kErfcxA1);
      const float g = fmaf(-e, fmaf(kc, r, f), 1.f);
      const float ri2 = ri[k] * ri[k];
      q[k] = g * (ri2 * ri[k]);
      p[k] = fmaf(k3n, e, q[k]) * ri2;
    }
  } else {
#pragma unroll
    for (int k = 0; k < T; ++k) {
      dx[k] = tx[k] - sa.x;
      dy[k] = ty[k] - sa.y;
      dz[k] = tz[k] - sa.z;
      const float r2 = fmaf(dx[k], dx[k], fmaf(dy[k], dy[k], dz[k] * dz[k]));
      arg[k] = r2 * ea;
      amax = fmaxf(amax, arg[k]);
      const float ri = rsqrt_ftz(r2);
      const float r = r2 * ri;
      const float e = ex2_ftz(arg[k]);
      const float t = rcp_ftz(fmaf(kt, r, 1.f));
      const float f = t * fmaf(t, fmaf(t, fmaf(t, kErfcxA4, kErfcxA3), kErfcxA2), kErfcxA1);
      const float g = fmaf(-e, fmaf(kc, r, f), 1.f);
      const float ri2 = ri * ri;
      q[k] = g * (ri2 * ri);
      p[k] = fmaf(k3n, e, q[k]) * ri2;
    }
  }
  if (__any_sync(0xffffffffu, amax > kArgSeries)) {
    const float is2 = is1 * is1, is3 = is2 * is1, is5n = is3 * is2 * (-1.f / 3.f);
#pragma unroll
    for (int k = 0; k < T; ++k) {
      if (arg[k] > kArgSeries) {
        float h1, h2;
        GaussSeries<float, 10>::eval(arg[k] * kArgToRho2, h1, h2);
        const bool self = arg[k] == 0.f;   // r² == 0 (the exponent argument is r²·(<0))
        q[k] = self ? 0.f : h1 * is3;
        p[k] = self ? 0.f : h2 * is5n;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < T; ++k) accum_pair(dx[k], dy[k], dz[k], q[k], p[k], sb.x, sb.y, sb.z, acc[k]);
}

// ---- Gaussian-erf far field ---------------------------------------------------
// With the exponent argument arg = r²·(-log2(e)/(2σ²)) = -log2(e)·ρ²/2:
//  - arg <= kArgFar (ρ² >= 50): e^{-ρ²/2}(erfcx(ρ/√2) + √(2/π)ρ) < 1e-10, far
//    below half an FP32 ulp of 1, so g rounds to 1; the √(2/π)ρ³e term of
//    q'/r is below 2e-9 of 3g.  The general path then yields q = 1/r³ and
//    p = -3/r⁵ (up to a tie-break in the last bit of p), which is what the
//    far routines compute, without erfcx, exp or the series test.
//  - arg <= kArgZero: 2^arg is subnormal and ex2.approx.ftz returns +0, so
//    ζ_σ, Dζ, Dq and Dp are exactly zero in FP32.
// The classification is made per warp and per 32 staged sources from bounding
// boxes (warp_target_box, warp_source_box): the box gap g² satisfies
// g² <= r² for every pair of the two boxes in the same FP32 arithmetic
// (rounding is monotone), so g²·max(a) >= arg for every pair.  Blocks that do
// not pass as a whole are classified again per source by warp votes
// (uj_source_gauss, ujd_source_gauss, zeta_source).  kArgFar and kArgZero are
// defined above uj_source_gauss.
// q = 1/r³, p = -3/r⁵ for one source against T targets; acc holds the plain
// sums first (U 0..2, A 3..10, W 12..14), so the α-derivative layout works too.
template <int T, int NV>
__device__ __forceinline__ void uj_source_gauss_far(const float4 sa, const float4 sb,
                                                    const float (&tx)[T], const float (&ty)[T],
                                                    const float (&tz)[T], float (&acc)[T][NV]) {
  if constexpr (T % 2 == 0) {
    const Src2 s(sa, sb);
#pragma unroll
    for (int k = 0; k < T; k += 2) {
      float2 dx, dy, dz, r2;
      diff2(tx, ty, tz, k, s, dx, dy, dz, r2);
      const float2 ri = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
      const float2 ri2 = mul2(ri, ri);
      const float2 q = mul2(ri2, ri);
      accum_pair2(dx, dy, dz, q, mul2(q, ri2), s, acc, k);
    }
  } else {
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const float dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float ri = rsqrt_ftz(r2);
      const float ri2 = ri * ri;
      const float q = ri2 * ri;
      const float p = q * ri2;
      accum_pair(dx, dy, dz, q, p, sb.x, sb.y, sb.z, acc[k]);
    }
  }
}

// 6 xor-shuffle reductions: every lane ends with the warp's box.
__device__ __forceinline__ void warp_box_reduce(float& lx, float& ly, float& lz, float& hx,
                                                float& hy, float& hz) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
    ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
    lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
    hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
    hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
    hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
  }
}

// Box of the T·32 targets of a warp, stored as (lo, extent²), (hi, 0) at box[0..1].
template <int T>
__device__ __forceinline__ void warp_target_box(const float (&tx)[T], const float (&ty)[T],
                                                const float (&tz)[T], float4* box) {
  float lx = tx[0], ly = ty[0], lz = tz[0], hx = tx[0], hy = ty[0], hz = tz[0];
#pragma unroll
  for (int k = 1; k < T; ++k) {
    lx = fminf(lx, tx[k]); ly = fminf(ly, ty[k]); lz = fminf(lz, tz[k]);
    hx = fmaxf(hx, tx[k]); hy = fmaxf(hy, ty[k]); hz = fmaxf(hz, tz[k]);
  }
  warp_box_reduce(lx, ly, lz, hx, hy, hz);
  if ((threadIdx.x & 31) == 0) {
    const float ex = hx - lx, ey = hy - ly, ez = hz - lz;
    box[0] = make_float4(lx, ly, lz, fmaf(ex, ex, fmaf(ey, ey, ez * ez)));
    box[1] = make_float4(hx, hy, hz, 0.f);
  }
}

// Box of the 32 sources a warp staged, with the largest exponent constant a
// (the widest core) in lo.w; padding sources are left out.
__device__ __forceinline__ void warp_source_box(float x, float y, float z, float a, bool valid,
                                                float4* box) {
  float lx = valid ? x : INFINITY, ly = valid ? y : INFINITY, lz = valid ? z : INFINITY;
  float hx = valid ? x : -INFINITY, hy = valid ? y : -INFINITY, hz = valid ? z : -INFINITY;
  float w = valid ? a : -INFINITY;
  warp_box_reduce(lx, ly, lz, hx, hy, hz);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
  if ((threadIdx.x & 31) == 0) {
    box[0] = make_float4(lx, ly, lz, w);
    box[1] = make_float4(hx, hy, hz, 0.f);
  }
}

// Upper bound of the exponent argument over all pairs of a target box and a
// source box (both read from shared memory; the result is warp-uniform), and
// the exponent argument of the target box's own extent (its diagonal at the
// block's widest core): per-source votes pay only when this is a few times
// the vote's threshold at most.
__device__ __forceinline__ float box_arg_bound(const float4* tbox, const float4* sbox,
                                               float& span) {
  const float4 tl = tbox[0], th = tbox[1], sl = sbox[0], sh = sbox[1];
  const float gx = fmaxf(0.f, fmaxf(sl.x - th.x, tl.x - sh.x));
  const float gy = fmaxf(0.f, fmaxf(sl.y - th.y, tl.y - sh.y));
  const float gz = fmaxf(0.f, fmaxf(sl.z - th.z, tl.z - sh.z));
  span = tl.w * sl.w;
  return fmaf(gx, gx, fmaf(gy, gy, gz * gz)) * sl.w;
}

// Per-source votes are used where the target box's extent argument is above
// kVoteSpan times the vote's threshold (both negative).
constexpr float kVoteSpan = 4.f;

// Classes of the 32-source blocks of a staged tile for one warp, 2 bits per
// block (NB <= 16 blocks): 3 where every pair has arg <= kArgZero, 2 where
// every pair has arg <= kArgFar, 1 where per-source votes pay (the target
// box's extent argument is >= vote_span), 0 otherwise.  0 for every block
// when the far field is off.
template <int NB>
__device__ __forceinline__ uint32_t classify_blocks(const float4* tbox, const float4* sbox,
                                                    int cnt, float vote_span, bool on) {
  uint32_t cls = 0;
  if (!on) return cls;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    if (b * 32 < cnt) {
      float span;
      const float bound = box_arg_bound(tbox, sbox + 2 * b, span);
      const uint32_t c = bound <= kArgZero ? 3u : bound <= kArgFar ? 2u : (span >= vote_span ? 1u : 0u);
      cls |= c << (2 * b);
    }
  }
  return cls;
}

// Bit b set where the warp's target box (tbox[0..1]) and staged block b's
// source box (sbox[2b..2b+1]) intersect.  Only there can a target and a source
// coincide (r² = 0 needs equal coordinates, which lie in both boxes); the
// test uses comparisons only, so it is exact.  Padding sources are outside
// every box (their block box is empty when all are padding).
template <int NB>
__device__ __forceinline__ uint32_t overlap_blocks(const float4* tbox, const float4* sbox,
                                                   int cnt) {
  const float4 tl = tbox[0], th = tbox[1];
  uint32_t m = 0;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    if (b * 32 < cnt) {
      const float4 sl = sbox[2 * b], sh = sbox[2 * b + 1];
      const bool o = sl.x <= th.x && tl.x <= sh.x && sl.y <= th.y && tl.y <= sh.y &&
                     sl.z <= th.z && tl.z <= sh.z;
      m |= uint32_t(o) << b;
    }
  }
  return m;
}

// 2-bit block codes: `code` at every block whose overlap bit is set, 0 elsewhere.
template <int NB>
__device__ __forceinline__ uint32_t overlap_codes(uint32_t ovl, uint32_t code) {
  uint32_t c = 0;
#pragma unroll
  for (int b = 0; b < NB; ++b)
    if ((ovl >> b) & 1u) c |= code << (2 * b);
  return c;
}

// End (exclusive, in sources) of the run of blocks that starts at source js and
// shares the class `key(block class)` of its first block.
template <typename Key>
__device__ __forceinline__ int block_run_end(uint32_t cls, int js, int cnt, Key key) {
  const int b0 = js >> 5;
  const uint32_t k0 = key((cls >> (2 * b0)) & 3u);
  int b = b0 + 1;
  while (b * 32 < cnt && key((cls >> (2 * b)) & 3u) == k0) ++b;
  return min(b * 32, cnt);
}

}  // namespace vpm

// ------------------------------------------------------------------------------
// α-derivative forms (d/dα at α = 1 of the sums with every σ scaled by α):
//   D q = -ρ g'(ρ)/r³,  D(q'/r) = (2ρg' - ρ²g'')/r⁵, which reduce to
//   Winckelmans:  D q = -15/2 σ⁴ s^{-7/2},  D p = D(q'/r)/KP = -35/2 σ⁴ s^{-9/2}
//   Gaussian-erf: D q = -√(2/π) e/σ³,      D p = D(q'/r)     = √(2/π) e/σ⁵
// (no cancellation in either), and D ζ_σ = ζ_σ (4 - 7/(ρ²+1)) or ζ_σ (ρ² - 3).
namespace vpm {

// 27 sums: U 0..2, A 3..11 (11 unused), W 12..14, DA 15..23 (23 unused), DW 24..26.
__device__ __forceinline__ void accum_pair_d(float dx, float dy, float dz, float q, float p,
                                             float dq, float dp, float gx, float gy, float gz,
                                             float* acc) {
  const float c0 = dy * gz - dz * gy;
  const float c1 = dz * gx - dx * gz;
  const float c2 = dx * gy - dy * gx;
  acc[0] = fmaf(q, c0, acc[0]);
  acc[1] = fmaf(q, c1, acc[1]);
  acc[2] = fmaf(q, c2, acc[2]);
  float a0 = p * c0, a1 = p * c1, a2 = p * c2;
  acc[3] = fmaf(a0, dx, acc[3]);
  acc[4] = fmaf(a0, dy, acc[4]);
  acc[5] = fmaf(a0, dz, acc[5]);
  acc[6] = fmaf(a1, dx, acc[6]);
  acc[7] = fmaf(a1, dy, acc[7]);
  acc[8] = fmaf(a1, dz, acc[8]);
  acc[9] = fmaf(a2, dx, acc[9]);
  acc[10] = fmaf(a2, dy, acc[10]);
  acc[12] = fmaf(q, gx, acc[12]);
  acc[13] = fmaf(q, gy, acc[13]);
  acc[14] = fmaf(q, gz, acc[14]);
  a0 = dp * c0; a1 = dp * c1; a2 = dp * c2;
  acc[15] = fmaf(a0, dx, acc[15]);
  acc[16] = fmaf(a0, dy, acc[16]);
  acc[17] = fmaf(a0, dz, acc[17]);
  acc[18] = fmaf(a1, dx, acc[18]);
  acc[19] = fmaf(a1, dy, acc[19]);
  acc[20] = fmaf(a1, dz, acc[20]);
  acc[21] = fmaf(a2, dx, acc[21]);
  acc[22] = fmaf(a2, dy, acc[22]);
  acc[24] = fmaf(dq, gx, acc[24]);
  acc[25] = fmaf(dq, gy, acc[25]);
  acc[26] = fmaf(dq, gz, acc[26]);
}

// accum_pair_d for targets (k, k+1) (see "packed FP32").
template <int T>
__device__ __forceinline__ void accum_pair_d2(float2 dx, float2 dy, float2 dz, float2 q, float2 p,
                                              float2 dq, float2 dp, const Src2& s,
                                              float (&acc)[T][27], int k) {
  const float2 c0 = fma2(dz, s.ngy, mul2(dy, s.gz));
  const float2 c1 = fma2(dx, s.ngz, mul2(dz, s.gx));
  const float2 c2 = fma2(dy, s.ngx, mul2(dx, s.gy));
  fma_acc2(acc, k, 0, q, c0);
  fma_acc2(acc, k, 1, q, c1);
  fma_acc2(acc, k, 2, q, c2);
  float2 a0 = mul2(p, c0), a1 = mul2(p, c1), a2 = mul2(p, c2);
  fma_acc2(acc, k, 3, a0, dx);
  fma_acc2(acc, k, 4, a0, dy);
  fma_acc2(acc, k, 5, a0, dz);
  fma_acc2(acc, k, 6, a1, dx);
  fma_acc2(acc, k, 7, a1, dy);
  fma_acc2(acc, k, 8, a1, dz);
  fma_acc2(acc, k, 9, a2, dx);
  fma_acc2(acc, k, 10, a2, dy);
  fma_acc2(acc, k, 12, q, s.gx);
  fma_acc2(acc, k, 13, q, s.gy);
  fma_acc2(acc, k, 14, q, s.gz);
  a0 = mul2(dp, c0); a1 = mul2(dp, c1); a2 = mul2(dp, c2);
  fma_acc2(acc, k, 15, a0, dx);
  fma_acc2(acc, k, 16, a0, dy);
  fma_acc2(acc, k, 17, a0, dz);
  fma_acc2(acc, k, 18, a1, dx);
  fma_acc2(acc, k, 19, a1, dy);
  fma_acc2(acc, k, 20, a1, dz);
  fma_acc2(acc, k, 21, a2, dx);
  fma_acc2(acc, k, 22, a2, dy);
  fma_acc2(acc, k, 24, dq, s.gx);
  fma_acc2(acc, k, 25, dq, s.gy);
  fma_acc2(acc, k, 26, dq, s.gz);
}

template <int T, bool MASK>
__device__ __forceinline__ void ujd_source_winck_x2(const float4 sa, const float4 sb,
                                                    const float (&tx)[T], const float (&ty)[T],
                                                    const float (&tz)[T], float (&acc)[T][27]) {
  const float s2 = sa.w;
  const Src2 s(sa, sb);
  const float2 s2p = bc2(s2), k15 = bc2(sb.w), k25 = bc2(sa.w + sb.w);
  const float2 c75 = bc2(-7.5f * s2 * s2), c175 = bc2(-17.5f * s2 * s2);
#pragma unroll
  for (int k = 0; k < T; k += 2) {
    float2 dx, dy, dz, r2, h;
    if (MASK) {
      diff2(tx, ty, tz, k, s, dx, dy, dz, r2);
      h = add2(r2, s2p);
    } else {
      dx = add2(make_float2(tx[k], tx[k + 1]), s.nx);
      dy = add2(make_float2(ty[k], ty[k + 1]), s.ny);
      dz = add2(make_float2(tz[k], tz[k + 1]), s.nz);
      h = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, s2p)));
    }
    const float2 rs = make_float2(rsqrt_ftz(h.x), rsqrt_ftz(h.y));
    const float2 rs2 = mul2(rs, rs);
    const float2 rs3 = mul2(rs2, rs);
    const float2 rs5 = mul2(rs3, rs2);
    const float2 rs7 = mul2(rs5, rs2);
    float2 q = fma2(k15, rs5, rs3);
    float2 dq = mul2(c75, rs7);
    if (MASK) {
      q.x = r2.x > 0.f ? q.x : 0.f;
      q.y = r2.y > 0.f ? q.y : 0.f;
      dq.x = r2.x > 0.f ? dq.x : 0.f;
      dq.y = r2.y > 0.f ? dq.y : 0.f;
    }
    const float2 p = fma2(k25, rs7, rs5);
    const float2 dp = mul2(c175, mul2(rs7, rs2));
    accum_pair_d2(dx, dy, dz, q, p, dq, dp, s, acc, k);
  }
}

template <int T, bool VOTE>
__device__ __forceinline__ void ujd_source_gauss_x2(const float4 sa, const float4 sb,
                                                    const float (&tx)[T], const float (&ty)[T],
                                                    const float (&tz)[T], float (&acc)[T][27]) {
  constexpr int H = T / 2;
  const float is1 = sb.w, is2 = is1 * is1;
  const float k3 = float(kSqrt2overPi) * is2 * is1;
  const Src2 s(sa, sb);
  const float2 ea = bc2(sa.w), one = bc2(1.f), k3p = bc2(k3), is2p = bc2(is2);
  float2 dx[H], dy[H], dz[H], r2[H], ri[H], arg[H], q[H], p[H], dq[H], dp[H];
  float amax = -INFINITY;
#pragma unroll
  for (int m = 0; m < H; ++m) {
    diff2(tx, ty, tz, 2 * m, s, dx[m], dy[m], dz[m], r2[m]);
    arg[m] = mul2(r2[m], ea);
    amax = fmaxf(amax, fmaxf(arg[m].x, arg[m].y));
    ri[m] = make_float2(rsqrt_ftz(r2[m].x), rsqrt_ftz(r2[m].y));
  }
  if (VOTE && __all_sync(0xffffffffu, amax <= kArgFar)) {
    const bool zero = __all_sync(0xffffffffu, amax <= kArgZero);
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const float2 ri2 = mul2(ri[m], ri[m]);
      const float2 qq = mul2(ri2, ri[m]);
      const float2 pp = mul2(qq, ri2);
      if (zero) {
        accum_pair2(dx[m], dy[m], dz[m], qq, pp, s, acc, 2 * m);
      } else {
        const float2 k3e = mul2(k3p, make_float2(ex2_ftz(arg[m].x), ex2_ftz(arg[m].y)));
        accum_pair_d2(dx[m], dy[m], dz[m], qq, pp, make_float2(-k3e.x, -k3e.y), mul2(k3e, is2p),
                      s, acc, 2 * m);
      }
    }
    return;
  }
  const float2 ktp = bc2(kErfcxP * is1), nkc = bc2(-float(kSqrt2overPi) * is1);
  const float2 nA4 = bc2(-kErfcxA4), nA3 = bc2(-kErfcxA3), nA2 = bc2(-kErfcxA2),
               nA1 = bc2(-kErfcxA1);
#pragma unroll
  for (int m = 0; m < H; ++m) {
    const float2 r = mul2(r2[m], ri[m]);
    const float2 e = make_float2(ex2_ftz(arg[m].x), ex2_ftz(arg[m].y));
    const float2 u = fma2(ktp, r, one);
    const float2 t = make_float2(rcp_ftz(u.x), rcp_ftz(u.y));
    const float2 nf = mul2(t, fma2(t, fma2(t, fma2(t, nA4, nA3), nA2), nA1));
    const float2 g = fma2(e, fma2(nkc, r, nf), one);
    const float2 ri2 = mul2(ri[m], ri[m]);
    const float2 k3e = mul2(k3p, e);
    q[m] = mul2(g, mul2(ri2, ri[m]));
    p[m] = mul2(fma2(k3e, bc2(-1.f / 3.f), q[m]), ri2);
    dq[m] = make_float2(-k3e.x, -k3e.y);
    dp[m] = mul2(k3e, is2p);
  }
  if (__any_sync(0xffffffffu, amax > kArgSeries)) {
    const float is3 = is2 * is1, is5n = is3 * is2 * (-1.f / 3.f);
#pragma unroll
    for (int m = 0; m < H; ++m) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float a = h ? arg[m].y : arg[m].x;
        if (a > kArgSeries) {
          float h1, h2;
          GaussSeries<float, 10>::eval(a * kArgToRho2, h1, h2);
          const bool self = a == 0.f;
          const float qs = self ? 0.f : h1 * is3, ps = self ? 0.f : h2 * is5n;
          if (h) {
            q[m].y = qs; p[m].y = ps;
            if (self) { dq[m].y = 0.f; dp[m].y = 0.f; }
          } else {
            q[m].x = qs; p[m].x = ps;
            if (self) { dq[m].x = 0.f; dp[m].x = 0.f; }
          }
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < H; ++m)
    accum_pair_d2(dx[m], dy[m], dz[m], q[m], p[m], dq[m], dp[m], s, acc, 2 * m);
}

template <int T, bool MASK>
__device__ __forceinline__ void ujd_source_winck(const float4 sa, const float4 sb,
                                                 const float (&tx)[T], const float (&ty)[T],
                                                 const float (&tz)[T], float (&acc)[T][27]) {
  if constexpr (T % 2 == 0) {
    ujd_source_winck_x2<T, MASK>(sa, sb, tx, ty, tz, acc);
    return;
  }
  const float s2 = sa.w, k15 = sb.w, k25 = sa.w + sb.w;
  const float c75 = -7.5f * s2 * s2, c175 = -17.5f * s2 * s2;
#pragma unroll
  for (int k = 0; k < T; ++k) {
    const float dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float rs = rsqrt_ftz(r2 + s2);
    const float rs2 = rs * rs;
    const float rs3 = rs2 * rs;
    const float rs5 = rs3 * rs2;
    const float rs7 = rs5 * rs2;
    float q = fmaf(k15, rs5, rs3);
    float dq = c75 * rs7;
    if (MASK) {
      q = r2 > 0.f ? q : 0.f;
      dq = r2 > 0.f ? dq : 0.f;
    }
    const float p = fmaf(k25, rs7, rs5);
    const float dp = c175 * (rs7 * rs2);
    accum_pair_d(dx, dy, dz, q, p, dq, dp, sb.x, sb.y, sb.z, acc[k]);
  }
}

// ujd_source_gauss: uj_source_gauss plus Dq, Dp.  With VOTE, per-source far
// forms as in uj_source_gauss (and only the plain sums where Dq = Dp = 0).
template <int T, bool VOTE>
__device__ __forceinline__ void ujd_source_gauss(const float4 sa, const float4 sb,
                                                 const float (&tx)[T], const float (&ty)[T],
                                                 const float (&tz)[T], float (&acc)[T][27]) {
  if constexpr (T % 2 == 0) {
    ujd_source_gauss_x2<T, VOTE>(sa, sb, tx, ty, tz, acc);
    return;
  }
  const float ea = sa.w, is1 = sb.w;
  const float is2 = is1 * is1;
  const float k3 = float(kSqrt2overPi) * is2 * is1;
  const float kt = kErfcxP * is1;
  const float kc = float(kSqrt2overPi) * is1;
  float dx[T], dy[T], dz[T], r2[T], ri[T], arg[T], q[T], p[T], dq[T], dp[T];
  float amax = -INFINITY;
#pragma unroll
  for (int k = 0; k < T; ++k) {
    dx[k] = tx[k] - sa.x;
    dy[k] = ty[k] - sa.y;
    dz[k] = tz[k] - sa.z;
    r2[k] = fmaf(dx[k], dx[k], fmaf(dy[k], dy[k], dz[k] * dz[k]));
    arg[k] = r2[k] * ea;
    amax = fmaxf(amax, arg[k]);
    ri[k] = rsqrt_ftz(r2[k]);
  }
  if (VOTE && __all_sync(0xffffffffu, amax <= kArgFar)) {
    const bool zero = __all_sync(0xffffffffu, amax <= kArgZero);
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const float ri2 = ri[k] * ri[k];
      const float qq = ri2 * ri[k];
      const float pp = qq * ri2;
      if (zero) {
        accum_pair(dx[k], dy[k], dz[k], qq, pp, sb.x, sb.y, sb.z, acc[k]);
      } else {
        const float k3e = k3 * ex2_ftz(arg[k]);
        accum_pair_d(dx[k], dy[k], dz[k], qq, pp, -k3e, k3e * is2, sb.x, sb.y, sb.z, acc[k]);
      }
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < T; ++k) {
    const float r = r2[k] * ri[k];
    const float e = ex2_ftz(arg[k]);
    const float t = rcp_ftz(fmaf(kt, r, 1.f));
    const float f = t * fmaf(t, fmaf(t, fmaf(t, kErfcxA4, kErfcxA3), kErfcxA2), kErfcxA1);
    const float g = fmaf(-e, fmaf(kc, r, f), 1.f);
    const float ri2 = ri[k] * ri[k];
    const float k3e = k3 * e;
    q[k] = g * (ri2 * ri[k]);
    p[k] = fmaf(k3e, -1.f / 3.f, q[k]) * ri2;
    dq[k] = -k3e;
    dp[k] = k3e * is2;
  }
  if (__any_sync(0xffffffffu, amax > kArgSeries)) {
    const float is3 = is2 * is1, is5n = is3 * is2 * (-1.f / 3.f);
#pragma unroll
    for (int k = 0; k < T; ++k) {
      if (arg[k] > kArgSeries) {
        float h1, h2;
        GaussSeries<float, 10>::eval(arg[k] * kArgToRho2, h1, h2);
        const bool self = arg[k] == 0.f;
        q[k] = self ? 0.f : h1 * is3;
        p[k] = self ? 0.f : h2 * is5n;
        dq[k] = self ? 0.f : dq[k];
        dp[k] = self ? 0.f : dp[k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < T; ++k)
    accum_pair_d(dx[k], dy[k], dz[k], q[k], p[k], dq[k], dp[k], sb.x, sb.y, sb.z, acc[k]);
}

// ujd_source_gauss for a source with arg <= kArgFar at every target: q and p
// as in uj_source_gauss_far, Dq = -√(2/π)e/σ³ and Dp = √(2/π)e/σ⁵ as in the
// general path.
template <int T>
__device__ __forceinline__ void ujd_source_gauss_far(const float4 sa, const float4 sb,
                                                     const float (&tx)[T], const float (&ty)[T],
                                                     const float (&tz)[T], float (&acc)[T][27]) {
  const float ea = sa.w, is1 = sb.w;
  const float is2 = is1 * is1;
  const float k3 = float(kSqrt2overPi) * is2 * is1;
  if constexpr (T % 2 == 0) {
    const Src2 s(sa, sb);
    const float2 eap = bc2(ea), k3p = bc2(k3), is2p = bc2(is2);
#pragma unroll
    for (int k = 0; k < T; k += 2) {
      float2 dx, dy, dz, r2;
      diff2(tx, ty, tz, k, s, dx, dy, dz, r2);
      const float2 ri = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
      const float2 ri2 = mul2(ri, ri);
      const float2 q = mul2(ri2, ri);
      const float2 p = mul2(q, ri2);
      const float2 a = mul2(r2, eap);
      const float2 k3e = mul2(k3p, make_float2(ex2_ftz(a.x), ex2_ftz(a.y)));
      accum_pair_d2(dx, dy, dz, q, p, make_float2(-k3e.x, -k3e.y), mul2(k3e, is2p), s, acc, k);
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < T; ++k) {
    const float dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float ri = rsqrt_ftz(r2);
    const float ri2 = ri * ri;
    const float q = ri2 * ri;
    const float p = q * ri2;
    const float k3e = k3 * ex2_ftz(r2 * ea);
    accum_pair_d(dx, dy, dz, q, p, -k3e, k3e * is2, sb.x, sb.y, sb.z, acc[k]);
  }
}

// FP64 α-derivatives of one pair (zero when r² == 0).
//   Winckelmans: a = σ², b = 3/2 σ²;  Gaussian-erf: a = 1/σ², b = 1/σ.
template <int KERNEL>
__device__ inline void pair_dqp_f64(double r2, double a, double b, double& dq, double& dp) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    const double s = r2 + a;
    const double rs = rsqrt(s);
    const double rs2 = rs * rs;
    const double rs7 = rs2 * rs2 * rs2 * rs;
    dq = -7.5 * a * a * rs7;
    dp = -17.5 * a * a * rs7 * rs2;
  } else {
    const double e = exp(-0.5 * r2 * a);
    const double k3 = kSqrt2overPi * b * b * b;
    dq = -k3 * e;
    dp = k3 * e * a;
  }
  if (!(r2 > 0.0)) {
    dq = 0.0;
    dp = 0.0;
  }
}

// ζ_σ and D ζ_σ of one pair from the ζ source constants (zero when r² == 0):
//   Winckelmans a = 1/σ², b = 15/(8π)/σ³;  Gaussian-erf a = -log2(e)/(2σ²), b = (2π)^{-3/2}/σ³.
template <int KERNEL>
__device__ inline void pair_zeta_d(float r2, float a, float b, float& z, float& dz) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    const float rs = rsqrt_ftz(fmaf(r2, a, 1.f));
    const float rs2 = rs * rs;
    z = b * (rs2 * rs2) * (rs2 * rs);
    dz = z * fmaf(-7.f, rs2, 4.f);
  } else {
    const float x = r2 * a;
    z = b * ex2_ftz(x);
    dz = z * fmaf(x, kArgToRho2, -3.f);
  }
  if (!(r2 > 0.f)) {
    z = 0.f;
    dz = 0.f;
  }
}
template <int KERNEL>
__device__ inline void pair_zeta_d(double r2, double a, double b, double& z, double& dz) {
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    const double s = fma(r2, a, 1.0);
    const double rs = rsqrt(s);
    const double rs2 = rs * rs;
    z = b * rs2 * rs2 * rs2 * rs;
    dz = z * (4.0 - 7.0 * rs2);
  } else {
    const double x = r2 * a;
    z = b * exp2(x);
    dz = z * (x * (-2.0 / kLog2e) - 3.0);
  }
  if (!(r2 > 0.0)) {
    z = 0.0;
    dz = 0.0;
  }
}

}  // namespace vpm

// ------------------------------------------------------------------------------
// Bulk asynchronous copies (TMA, 1-D form) into shared memory with mbarrier
// completion.  Source and destination must be 16-byte aligned and the size a
// multiple of 16 bytes; callers guarantee both.
namespace vpm {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also announces `bytes` of transactions for this phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Order this thread's earlier generic accesses to shared memory before later
// asynchronous-proxy (TMA) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- thread-block clusters ----------------------------------------------------
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Every thread of every CTA of the cluster arrives; shared-memory writes before
// the barrier are visible to reads of any CTA of the cluster after it.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Load a float from the same shared-memory offset in cluster CTA `rank`.
__device__ __forceinline__ float ld_cluster_f32(const float* local, uint32_t rank) {
  uint32_t remote;
  float v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(smem_u32(local)), "r"(rank));
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(remote) : "memory");
  return v;
}

// Wait for the phase of the given parity to complete, giving up after a bounded
// number of polls (returns false then).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int polls = 1 << 22) {
  const uint32_t addr = smem_u32(bar);
  for (int it = 0; it < polls; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// An L2 cache policy for every access it covers: evict_last (the lines are
// kept over normal ones) when last is true, else evict_normal.
__device__ __forceinline__ uint64_t l2_policy(bool last) {
  uint64_t keep, normal;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(normal));
  return last ? keep : normal;
}

// Store v at p with the L2 cache policy pol.
__device__ __forceinline__ void st_global_hint(double* p, double v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(__cvta_generic_to_global(p)),
               "d"(v), "l"(pol)
               : "memory");
}

// Store the float pair (h, l) in the 8 bytes at p with the L2 cache policy pol.
__device__ __forceinline__ void st_global_hint_f2(double* p, float h, float l, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(
                   __cvta_generic_to_global(p)),
               "f"(h), "f"(l), "l"(pol)
               : "memory");
}

// Drop the 128-byte L2 line at p (128-byte aligned, device memory) without a
// write-back: its contents become undefined, so only data that no one reads
// again may be discarded.
__device__ __forceinline__ void discard_l2_line(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(__cvta_generic_to_global(p)) : "memory");
}

}  // namespace vpm

// ------------------------------------------------------------------------------
// FP32 ζ pass: one staged source against the T targets of a thread.
//   Source quads: (x, y, z, a), (Γ, b), (v, c) [and (w, -) for the D form], with
//   Gaussian-erf: a = -log2(e)/(2σ²), b = (2π)^{-3/2}/σ³                 → ζ_σ = b·2^{r² a}
//   Winckelmans:  c' = (15/(8π)/σ³)^{-2/7}, a = c'/σ², b = c', c = -7c'  → with
//                 s' = r² a + b = c'(ρ²+1),  ζ_σ = s'^{-7/2}  (the prefactor is in c'),
//                 and 1/(ρ²+1) = c'/s' for the D form.
//   Dζ_σ = ζ_σ (ρ² - 3) (Gaussian) or ζ_σ (4 - 7/(ρ²+1)) (Winckelmans).
// Accumulators: Ω 0..2, V 3..5 (and DΩ 6..8, DV 9..11).  MASK drops coincident
// pairs (only tiles that can hold a target's own particle need it).
namespace vpm {

template <int KERNEL>
__device__ inline void zeta_consts_f32(double sig, float& a, float& b, float& c) {
  const double s3 = sig * sig * sig;
  if (KERNEL == VPM_KERNEL_WINCKELMANS) {
    const double cp = pow(kZeta0Winck / s3, -2.0 / 7.0);
    a = float(cp / (sig * sig));
    b = float(cp);
    c = float(-7.0 * cp);
  } else {
    a = float(-0.5 * kLog2e / (sig * sig));
    b = float(kZeta0Gauss / s3);
    c = 0.f;
  }
}

// ζ sums of one source against T targets.  With VOTE (Gaussian-erf only), a
// warp vote skips a source whose ζ underflows to +0 at every target.
template <int KERNEL, int T, bool MASK, bool D, bool VOTE>
__device__ __forceinline__ void zeta_source(const float4 sa, const float4 sb, const float4 sc,
                                            const float4 sd, const float (&tx)[T],
                                            const float (&ty)[T], const float (&tz)[T],
                                            float (&acc)[T][D ? 12 : 6]) {
  if constexpr (T % 2 == 0) {
    // Target pairs (see "packed FP32").
    constexpr int H = T / 2;
    const float2 nx = bc2(-sa.x), ny = bc2(-sa.y), nz = bc2(-sa.z), aw = bc2(sa.w);
    float2 r2[H];
    float amax = -INFINITY;
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const float2 dx = add2(make_float2(tx[2 * m], tx[2 * m + 1]), nx);
      const float2 dy = add2(make_float2(ty[2 * m], ty[2 * m + 1]), ny);
      const float2 dz = add2(make_float2(tz[2 * m], tz[2 * m + 1]), nz);
      r2[m] = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
      if (VOTE) amax = fmaxf(amax, fmaxf(r2[m].x * sa.w, r2[m].y * sa.w));
    }
    if (VOTE && KERNEL != VPM_KERNEL_WINCKELMANS && __all_sync(0xffffffffu, amax <= kArgZero))
      return;
    const float2 gx = bc2(sb.x), gy = bc2(sb.y), gz = bc2(sb.z);
    const float2 vx = bc2(sc.x), vy = bc2(sc.y), vz = bc2(sc.z);
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const int k = 2 * m;
      float2 z, dzz = bc2(0.f);
      if (KERNEL == VPM_KERNEL_WINCKELMANS) {
        const float2 h = fma2(r2[m], aw, bc2(sb.w));
        const float2 rs = make_float2(rsqrt_ftz(h.x), rsqrt_ftz(h.y));
        const float2 rs2 = mul2(rs, rs);
        z = mul2(mul2(rs2, rs2), mul2(rs2, rs));
        if (D) dzz = mul2(z, fma2(bc2(sc.w), rs2, bc2(4.f)));
      } else {
        const float2 x = mul2(r2[m], aw);
        z = mul2(bc2(sb.w), make_float2(ex2_ftz(x.x), ex2_ftz(x.y)));
        if (D) dzz = mul2(z, fma2(x, bc2(kArgToRho2), bc2(-3.f)));
      }
      if (MASK) {
        z.x = r2[m].x > 0.f ? z.x : 0.f;
        z.y = r2[m].y > 0.f ? z.y : 0.f;
        if (D) {
          dzz.x = r2[m].x > 0.f ? dzz.x : 0.f;
          dzz.y = r2[m].y > 0.f ? dzz.y : 0.f;
        }
      }
      fma_acc2(acc, k, 0, z, gx);
      fma_acc2(acc, k, 1, z, gy);
      fma_acc2(acc, k, 2, z, gz);
      fma_acc2(acc, k, 3, z, vx);
      fma_acc2(acc, k, 4, z, vy);
      fma_acc2(acc, k, 5, z, vz);
      if (D) {
        fma_acc2(acc, k, 6, dzz, gx);
        fma_acc2(acc, k, 7, dzz, gy);
        fma_acc2(acc, k, 8, dzz, gz);
        fma_acc2(acc, k, 9, z, bc2(sd.x));
        fma_acc2(acc, k, 10, z, bc2(sd.y));
        fma_acc2(acc, k, 11, z, bc2(sd.z));
        fma_acc2(acc, k, 9, dzz, vx);
        fma_acc2(acc, k, 10, dzz, vy);
        fma_acc2(acc, k, 11, dzz, vz);
      }
    }
    return;
  }
  float r2[T];
  float amax = -INFINITY;
#pragma unroll
  for (int k = 0; k < T; ++k) {
    const float dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
    r2[k] = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (VOTE) amax = fmaxf(amax, r2[k] * sa.w);
  }
  // Gaussian-erf: a source whose ζ underflows to +0 at every target of the
  // warp (exponent argument <= kArgZero) adds nothing.
  if (VOTE && KERNEL != VPM_KERNEL_WINCKELMANS && __all_sync(0xffffffffu, amax <= kArgZero)) return;
#pragma unroll
  for (int k = 0; k < T; ++k) {
    float z, dzz = 0.f;
    if (KERNEL == VPM_KERNEL_WINCKELMANS) {
      const float rs = rsqrt_ftz(fmaf(r2[k], sa.w, sb.w));
      const float rs2 = rs * rs;
      z = (rs2 * rs2) * (rs2 * rs);
      if (D) dzz = z * fmaf(sc.w, rs2, 4.f);
    } else {
      const float x = r2[k] * sa.w;
      z = sb.w * ex2_ftz(x);
      if (D) dzz = z * fmaf(x, kArgToRho2, -3.f);
    }
    if (MASK) {
      z = r2[k] > 0.f ? z : 0.f;
      if (D) dzz = r2[k] > 0.f ? dzz : 0.f;
    }
    acc[k][0] = fmaf(z, sb.x, acc[k][0]);
    acc[k][1] = fmaf(z, sb.y, acc[k][1]);
    acc[k][2] = fmaf(z, sb.z, acc[k][2]);
    acc[k][3] = fmaf(z, sc.x, acc[k][3]);
    acc[k][4] = fmaf(z, sc.y, acc[k][4]);
    acc[k][5] = fmaf(z, sc.z, acc[k][5]);
    if (D) {
      acc[k][6] = fmaf(dzz, sb.x, acc[k][6]);
      acc[k][7] = fmaf(dzz, sb.y, acc[k][7]);
      acc[k][8] = fmaf(dzz, sb.z, acc[k][8]);
      acc[k][9] = fmaf(dzz, sc.x, fmaf(z, sd.x, acc[k][9]));
      acc[k][10] = fmaf(dzz, sc.y, fmaf(z, sd.y, acc[k][10]));
      acc[k][11] = fmaf(dzz, sc.z, fmaf(z, sd.z, acc[k][11]));
    }
  }
}

}  // namespace vpm
