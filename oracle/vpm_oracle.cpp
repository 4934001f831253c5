// vpm_oracle.cpp — CPU FP64 restatement of the rVPM particle-field evaluation.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for libvpmgpu.so: only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
// may load it.  Nothing in the product links or calls it.
//
// PARITY UNPINNED.  The hot path's arithmetic lives in FLOWVPM (an external
// Julia package pinned by `[compat] FLOWVPM = "4.0"`, Project.toml:15,25 of
// FLOWUnsteady) and is not vendored with FLOWUnsteady; Julia is not available
// either.  This restatement follows the published mathematics cited below and
// the in-tree pair loop of FLOWUnsteady (_Ffv_direct,
// src/FLOWUnsteady_processing_force.jl:879-929); it is pinned against analytic
// known answers and an independent NumPy restatement (oracle/np_oracle.py),
// not against FLOWVPM's own outputs.
//
// Sources restated (paths inside byuflowlab/FLOWUnsteady):
//   U(x) = -1/(4π) Σ_p g_σp(x-x_p) (x-x_p)/|x-x_p|³ × Γ_p      docs/src/theory/rvpm.md:88-99
//   rVPM ODEs for x, Γ, σ (f, g constants; rVPM f=0, g=1/5)   docs/src/theory/rvpm.md:105-236
//   E_str, dynamic C_d = <Γ·L>/<Γ·m>, backscatter clipping     docs/src/theory/rvpm.md:249-297
//   transposed scheme, low-storage RK3, core spreading         docs/src/theory/rvpm.md:361-370
//   pair loop: source σ, r != 0 skip, 1/(4π)                   src/FLOWUnsteady_processing_force.jl:879-929
//   enstrophy ≈ ½ Σ Γ_p·ω(x_p)                                  src/FLOWUnsteady_monitors.jl:573-574
//   Winckelmans & Leonard (1993) algebraic kernel               docs/src/theory/rvpm.md:380
//   Williamson (1980) 2N-storage RK3: a=(0,-5/9,-153/128), b=(1/3,15/16,8/15)
//
// Conventions chosen here (FLOWVPM's own choices cannot be read in this tree):
//   - coincident pairs (r == 0) are skipped in U, J and E_str;
//   - E_str uses the source core size σ_q in ζ_σ;
//   - the dynamic procedure runs once per step on the first RK stage, with a
//     test filter ασ (α < 1) standing in for the unfiltered field
//     ("pseudo-three-level"): u - ū ≈ ū(ασ) - ū(σ) and ∂/∂σ ≈ [·(ασ) - ·(σ)]/((α-1)σ);
//     the common factor 1/((α-1)σ) cancels in C_d = <Γ·L>/<Γ·m>, leaving
//     numerator (3α-2) Γ·ΔS and denominator σ³/ζ(0) Γ·ΔE;
//   - clipping sets the stored C_d to 0 where C_d Γ·E_str < 0 (every stage);
//   - core spreading integrates d(σ²)/dt = 2ν with its own RK register after the
//     stretching update of σ;
//   - Z = 0 where |Γ| = 0 (instead of a 0/0).
//
// Layouts: row-major (n,3) for X, Γ, U, E, C; (n,9) for J with J[3a+b] = dU_a/dx_b.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/vpm_gpu.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kInv4Pi = 1.0 / (4.0 * kPi);
constexpr double kSqrt2overPi = 0.79788456080286535588;  // √(2/π)
constexpr double kInvSqrt2 = 0.70710678118654752440;

void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

// ζ(ρ): radial basis of the filter; ζ_σ(x) = ζ(|x|/σ)/σ³.
inline double zeta_of(int kernel, double rho2) {
  if (kernel == VPM_KERNEL_WINCKELMANS) {
    // 15/(8π) (ρ²+1)^(-7/2)
    double s = rho2 + 1.0;
    return 15.0 / (8.0 * kPi) / (s * s * s * std::sqrt(s));
  }
  // (2π)^(-3/2) exp(-ρ²/2)
  return std::exp(-0.5 * rho2) / std::pow(2.0 * kPi, 1.5);
}

// Gaussian-erf series in x = ρ² (derived from g(ρ) = √(2/π) ∫_0^ρ t² e^{-t²/2} dt):
//   g/ρ³          = √(2/π) Σ_n (-1/2)^n x^n / (n! (2n+3))
//   (ρg'-3g)/ρ⁵   = -√(2/π) Σ_m (-1/2)^m x^m / (m! (2m+5))
inline void gauss_series(double x, double* h1, double* h2) {
  double term = 1.0;  // (-1/2)^n x^n / n!
  double s1 = 0.0, s2 = 0.0;
  for (int n = 0; n < 24; ++n) {
    s1 += term / (2 * n + 3);
    s2 += term / (2 * n + 5);
    term *= -0.5 * x / (n + 1);
  }
  *h1 = kSqrt2overPi * s1;
  *h2 = -kSqrt2overPi * s2;
}

// q(r) = g(r/σ)/r³ and qr(r) = (dq/dr)/r for one pair.
inline void kernel_q(int kernel, double r2, double sig, double* q, double* qr) {
  if (kernel == VPM_KERNEL_WINCKELMANS) {
    // q = (r²+5/2σ²)/(r²+σ²)^{5/2};  (dq/dr)/r = -3(r²+7/2σ²)/(r²+σ²)^{7/2}
    double s2 = sig * sig;
    double s = r2 + s2;
    double rs = 1.0 / std::sqrt(s);
    double rs2 = rs * rs;
    double rs5 = rs2 * rs2 * rs;
    double rs7 = rs5 * rs2;
    *q = (r2 + 2.5 * s2) * rs5;
    *qr = -3.0 * (r2 + 3.5 * s2) * rs7;
    return;
  }
  double rho2 = r2 / (sig * sig);
  if (rho2 < 0.25) {
    double h1, h2;
    gauss_series(rho2, &h1, &h2);
    double is3 = 1.0 / (sig * sig * sig);
    *q = h1 * is3;
    *qr = h2 * is3 / (sig * sig);
    return;
  }
  double r = std::sqrt(r2);
  double rho = r / sig;
  double e = std::exp(-0.5 * rho2);
  double g = std::erf(rho * kInvSqrt2) - kSqrt2overPi * rho * e;
  double rhodg = kSqrt2overPi * rho2 * rho * e;  // ρ g'(ρ)
  double ir2 = 1.0 / r2;
  double ir3 = ir2 / r;
  *q = g * ir3;
  *qr = (rhodg - 3.0 * g) * ir3 * ir2;
}

// Analytic derivatives with respect to a common scale α of all core sizes,
// D = d/dα at α = 1 = Σ σ ∂/∂σ (used by the analytic dynamic procedure):
//   D q      = -ρ g'(ρ)/r³,  D (q'/r) = (2ρ g' - ρ² g'')/r⁵,
//   Winckelmans: D q = -15/2 σ⁴/s^{7/2},  D(q'/r) = 105/2 σ⁴/s^{9/2}  (s = r²+σ²)
//   Gaussian-erf: D q = -√(2/π) e/σ³,   D(q'/r) = √(2/π) e/σ⁵        (e = e^{-ρ²/2})
//   D ζ_σ = -3ζ_σ - ρ ζ'(ρ)/σ³:  Winckelmans ζ_σ (4 - 7/(ρ²+1)),  Gaussian ζ_σ (ρ² - 3).
inline void kernel_dq(int kernel, double r2, double sig, double* dq, double* dqr) {
  if (kernel == VPM_KERNEL_WINCKELMANS) {
    double s2 = sig * sig, s = r2 + s2;
    double rs = 1.0 / std::sqrt(s), rs2 = rs * rs;
    double rs7 = rs2 * rs2 * rs2 * rs;
    *dq = -7.5 * s2 * s2 * rs7;
    *dqr = 52.5 * s2 * s2 * rs7 * rs2;
    return;
  }
  double e = std::exp(-0.5 * r2 / (sig * sig));
  double k3 = kSqrt2overPi / (sig * sig * sig);
  *dq = -k3 * e;
  *dqr = k3 * e / (sig * sig);
}

inline double dzeta_factor(int kernel, double rho2) {
  return kernel == VPM_KERNEL_WINCKELMANS ? 4.0 - 7.0 / (rho2 + 1.0) : rho2 - 3.0;
}

// S(J, v): classic (J v) or transposed (Jᵀ v).
inline void stretch(const double* J, const double* v, int transposed, double* S) {
  if (transposed) {
    for (int a = 0; a < 3; ++a) S[a] = J[0 * 3 + a] * v[0] + J[1 * 3 + a] * v[1] + J[2 * 3 + a] * v[2];
  } else {
    for (int a = 0; a < 3; ++a) S[a] = J[a * 3 + 0] * v[0] + J[a * 3 + 1] * v[1] + J[a * 3 + 2] * v[2];
  }
}

}  // namespace

extern "C" {

// g(ρ), dg/dρ and ζ(ρ) of a kernel (known-answer tests).
int orc_kernel_eval(int kernel, int64_t n, const double* rho, double* g, double* dg, double* zeta) {
  for (int64_t i = 0; i < n; ++i) {
    double p = rho[i], p2 = p * p;
    if (kernel == VPM_KERNEL_WINCKELMANS) {
      double s = p2 + 1.0;
      g[i] = p2 * p * (p2 + 2.5) / (s * s * std::sqrt(s));
      dg[i] = 7.5 * p2 / (s * s * s * std::sqrt(s));
    } else {
      double e = std::exp(-0.5 * p2);
      if (p2 < 0.25) {
        double h1, h2;
        gauss_series(p2, &h1, &h2);
        g[i] = h1 * p2 * p;
      } else {
        g[i] = std::erf(p * kInvSqrt2) - kSqrt2overPi * p * e;
      }
      dg[i] = kSqrt2overPi * p2 * e;
    }
    zeta[i] = zeta_of(kernel, p2);
  }
  return 0;
}

// U, J at nt targets from ns sources; core sizes multiplied by sigma_scale.
// Direct restatement of UJ_direct (U from rvpm.md:88-99, J its analytic gradient).
int orc_uj_direct(int kernel, double sigma_scale, int64_t nt, const double* Xt, int64_t ns,
                  const double* Xs, const double* Gs, const double* Ss, double* U, double* J,
                  int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < nt; ++i) {
    const double xi = Xt[3 * i], yi = Xt[3 * i + 1], zi = Xt[3 * i + 2];
    double u[3] = {0, 0, 0}, jac[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t j = 0; j < ns; ++j) {
      const double dx = xi - Xs[3 * j], dy = yi - Xs[3 * j + 1], dz = zi - Xs[3 * j + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 == 0.0) continue;
      double q, qr;
      kernel_q(kernel, r2, Ss[j] * sigma_scale, &q, &qr);
      const double g0 = Gs[3 * j], g1 = Gs[3 * j + 1], g2 = Gs[3 * j + 2];
      const double c0 = dy * g2 - dz * g1, c1 = dz * g0 - dx * g2, c2 = dx * g1 - dy * g0;
      u[0] += q * c0; u[1] += q * c1; u[2] += q * c2;
      const double d[3] = {dx, dy, dz}, c[3] = {c0, c1, c2};
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) jac[3 * a + b] += qr * c[a] * d[b];
      // q ε_abc Γ_c
      jac[1] += q * g2; jac[2] -= q * g1;
      jac[3] -= q * g2; jac[5] += q * g0;
      jac[6] += q * g1; jac[7] -= q * g0;
    }
    for (int a = 0; a < 3; ++a) U[3 * i + a] = -kInv4Pi * u[a];
    for (int k = 0; k < 9; ++k) J[9 * i + k] = -kInv4Pi * jac[k];
  }
  return 0;
}

// E_str and the filtered vorticity ω at nt targets (rvpm.md:251-262, :76-84):
//   E_p = Σ_q ζ_σq(x_p-x_q) S(J_p - J_q, Γ_q) = S(J_p, Ω_p) - Σ_q ζ S(J_q, Γ_q)
//   ω_p = Σ_q ζ_σq(x_p-x_q) Γ_q   (self term included in ω, coincident pairs skipped in E)
// Jt: J at the targets, Js: J at the sources.  E or omega may be NULL.
int orc_estr_direct(int kernel, double sigma_scale, int transposed, int64_t nt, const double* Xt,
                    const double* Jt, const double* St, int64_t ns, const double* Xs,
                    const double* Gs, const double* Ss, const double* Js, double* E,
                    double* omega, int nthreads) {
  set_threads(nthreads);
  std::vector<double> v(3 * (size_t)ns, 0.0);
  if (Js) {
    for (int64_t q = 0; q < ns; ++q) stretch(Js + 9 * q, Gs + 3 * q, transposed, &v[3 * q]);
  }
  const double z0 = zeta_of(kernel, 0.0);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t p = 0; p < nt; ++p) {
    double om[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
    for (int64_t q = 0; q < ns; ++q) {
      const double dx = Xt[3 * p] - Xs[3 * q], dy = Xt[3 * p + 1] - Xs[3 * q + 1],
                   dz = Xt[3 * p + 2] - Xs[3 * q + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 == 0.0) continue;
      const double sg = Ss[q] * sigma_scale;
      const double z = zeta_of(kernel, r2 / (sg * sg)) / (sg * sg * sg);
      for (int a = 0; a < 3; ++a) {
        om[a] += z * Gs[3 * q + a];
        vv[a] += z * v[3 * q + a];
      }
    }
    if (E && Jt) {
      double s[3];
      stretch(Jt + 9 * p, om, transposed, s);
      for (int a = 0; a < 3; ++a) E[3 * p + a] = s[a] - vv[a];
    }
    if (omega) {
      // Self contribution ζ(0)/σ_p³ Γ_p (targets are sources here when St != NULL).
      double self = 0.0;
      if (St) {
        const double sp = St[p] * sigma_scale;
        self = z0 / (sp * sp * sp);
      }
      for (int a = 0; a < 3; ++a) omega[3 * p + a] = om[a];
      if (St && p < ns) {
        for (int a = 0; a < 3; ++a) omega[3 * p + a] += self * Gs[3 * p + a];
      }
    }
  }
  return 0;
}

// D J (the α-derivative of J) at nt targets, same conventions as orc_uj_direct.
int orc_uj_direct_dsigma(int kernel, int64_t nt, const double* Xt, int64_t ns, const double* Xs,
                         const double* Gs, const double* Ss, double* DJ, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < nt; ++i) {
    double jac[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t j = 0; j < ns; ++j) {
      const double dx = Xt[3 * i] - Xs[3 * j], dy = Xt[3 * i + 1] - Xs[3 * j + 1],
                   dz = Xt[3 * i + 2] - Xs[3 * j + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 == 0.0) continue;
      double dq, dqr;
      kernel_dq(kernel, r2, Ss[j], &dq, &dqr);
      const double g0 = Gs[3 * j], g1 = Gs[3 * j + 1], g2 = Gs[3 * j + 2];
      const double c[3] = {dy * g2 - dz * g1, dz * g0 - dx * g2, dx * g1 - dy * g0};
      const double d[3] = {dx, dy, dz};
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) jac[3 * a + b] += dqr * c[a] * d[b];
      jac[1] += dq * g2; jac[2] -= dq * g1;
      jac[3] -= dq * g2; jac[5] += dq * g0;
      jac[6] += dq * g1; jac[7] -= dq * g0;
    }
    for (int k = 0; k < 9; ++k) DJ[9 * i + k] = -kInv4Pi * jac[k];
  }
  return 0;
}

// D E_str with targets = sources: D E_p = S(DJ_p, Ω_p) + S(J_p, DΩ_p) - DV_p,
// DΩ_p = Σ Dζ Γ_q, DV_p = Σ [Dζ S(J_q,Γ_q) + ζ S(DJ_q,Γ_q)] (coincident pairs skipped).
int orc_estr_direct_dsigma(int kernel, int transposed, int64_t n, const double* X, const double* G,
                           const double* S, const double* J, const double* DJ, double* DE,
                           int nthreads) {
  set_threads(nthreads);
  std::vector<double> v(3 * (size_t)n), w(3 * (size_t)n);
  for (int64_t q = 0; q < n; ++q) {
    stretch(J + 9 * q, G + 3 * q, transposed, &v[3 * q]);
    stretch(DJ + 9 * q, G + 3 * q, transposed, &w[3 * q]);
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t p = 0; p < n; ++p) {
    double om[3] = {0, 0, 0}, dom[3] = {0, 0, 0}, dv[3] = {0, 0, 0};
    for (int64_t q = 0; q < n; ++q) {
      const double dx = X[3 * p] - X[3 * q], dy = X[3 * p + 1] - X[3 * q + 1],
                   dz = X[3 * p + 2] - X[3 * q + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 == 0.0) continue;
      const double sg = S[q], rho2 = r2 / (sg * sg);
      const double z = zeta_of(kernel, rho2) / (sg * sg * sg);
      const double dz_ = z * dzeta_factor(kernel, rho2);
      for (int a = 0; a < 3; ++a) {
        om[a] += z * G[3 * q + a];
        dom[a] += dz_ * G[3 * q + a];
        dv[a] += dz_ * v[3 * q + a] + z * w[3 * q + a];
      }
    }
    double s1[3], s2[3];
    stretch(DJ + 9 * p, om, transposed, s1);
    stretch(J + 9 * p, dom, transposed, s2);
    for (int a = 0; a < 3; ++a) DE[3 * p + a] = s1[a] + s2[a] - dv[a];
  }
  return 0;
}

// Free-vortex force, restated from _Ffv_direct
// (src/FLOWUnsteady_processing_force.jl:879-929): for every bound particle b,
// over every free particle f with r = |x_f - x_b| != 0 and the bound core σ_b,
//   U_b(x_f) = -g_σb(r)/(4π r³) (Δx × Γ_b),           Δx = x_f - x_b
//   M[0:3]  += U_b(x_f) × Γ_f
//   M[3:6]  += g_σb(r)/(4π r³) Δx × (Γ_b × Γ_f)
// (the reference writes 1/(4π) as 0.07957747154594767).  M is (nb, 6).
int orc_ffv_direct(int kernel, int64_t nb, const double* Xb, const double* Gb, const double* Sb,
                   int64_t nf, const double* Xf, const double* Gf, double* M, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t b = 0; b < nb; ++b) {
    double m[6] = {0, 0, 0, 0, 0, 0};
    const double* xb = Xb + 3 * b;
    const double* gb = Gb + 3 * b;
    for (int64_t f = 0; f < nf; ++f) {
      const double dX1 = Xf[3 * f] - xb[0], dX2 = Xf[3 * f + 1] - xb[1], dX3 = Xf[3 * f + 2] - xb[2];
      const double r = std::sqrt(dX1 * dX1 + dX2 * dX2 + dX3 * dX3);
      if (r == 0.0) continue;
      double g, dg, z;
      const double rho = r / Sb[b];
      orc_kernel_eval(kernel, 1, &rho, &g, &dg, &z);
      const double k = g * kInv4Pi / (r * r * r);
      const double U1 = -k * (dX2 * gb[2] - dX3 * gb[1]);
      const double U2 = -k * (dX3 * gb[0] - dX1 * gb[2]);
      const double U3 = -k * (dX1 * gb[1] - dX2 * gb[0]);
      const double* gf = Gf + 3 * f;
      m[0] += U2 * gf[2] - U3 * gf[1];
      m[1] += U3 * gf[0] - U1 * gf[2];
      m[2] += U1 * gf[1] - U2 * gf[0];
      const double c1 = gb[1] * gf[2] - gb[2] * gf[1];
      const double c2 = gb[2] * gf[0] - gb[0] * gf[2];
      const double c3 = gb[0] * gf[1] - gb[1] * gf[0];
      m[3] += k * (dX2 * c3 - dX3 * c2);
      m[4] += k * (dX3 * c1 - dX1 * c3);
      m[5] += k * (dX1 * c2 - dX2 * c1);
    }
    for (int c = 0; c < 6; ++c) M[6 * b + c] = m[c];
  }
  return 0;
}

// One time step of the full method on n particles, the last n_static of which
// act as sources only.  X, G, S are advanced in place; C (n,3) holds the SFS
// memory (C_d, <Γ·L>, <Γ·m>) across steps.  E_out (n,3) receives the last
// stage's E_str when non-NULL.
int orc_step(const vpm_scheme* sc, int64_t n, int64_t n_static, double dt, double* X, double* G,
             double* S, double* C, double* E_out, int nthreads) {
  if (!sc || n < 0 || n_static < 0 || n_static > n) return VPM_ERR_INVALID;
  const int64_t nf = n - n_static;
  const int kernel = sc->kernel;
  const bool rk3 = sc->integration == VPM_INTEGRATION_RK3;
  const int nstages = rk3 ? 3 : 1;
  const double A[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
  const double B[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
  const double f = sc->f, g = sc->g;
  const double zeta0 = zeta_of(kernel, 0.0);
  const bool sfs = sc->sfs != VPM_SFS_NONE;

  std::vector<double> U(3 * n), J(9 * n), E(3 * n, 0.0);
  std::vector<double> Jt(9 * n), Ut(3 * n), Et(3 * n);
  std::vector<double> Qx(3 * n, 0.0), QG(3 * n, 0.0), Qs(n, 0.0), Qs2(n, 0.0);

  for (int st = 0; st < nstages; ++st) {
    const double a = rk3 ? A[st] : 0.0, b = rk3 ? B[st] : 1.0;
    orc_uj_direct(kernel, 1.0, n, X, n, X, G, S, U.data(), J.data(), nthreads);
    if (sfs) {
      orc_estr_direct(kernel, 1.0, sc->transposed, n, X, J.data(), S, n, X, G, S, J.data(),
                      E.data(), nullptr, nthreads);
      if (sc->sfs == VPM_SFS_CONSTANT) {
        for (int64_t p = 0; p < nf; ++p) C[3 * p] = sc->sfs_Cd;
      } else if (st == 0) {
        const double al = sc->sfs_alpha;
        if (sc->sfs_flags & VPM_SFS_ANALYTIC_DSIGMA) {
          // Jt, Et := first-order test-filter values J + (α-1) DJ, E + (α-1) DE,
          // so the differences below are (α-1) DJ and (α-1) DE.
          std::vector<double> DJ(9 * n), DE(3 * n);
          orc_uj_direct_dsigma(kernel, n, X, n, X, G, S, DJ.data(), nthreads);
          orc_estr_direct_dsigma(kernel, sc->transposed, n, X, G, S, J.data(), DJ.data(),
                                 DE.data(), nthreads);
          for (int64_t k = 0; k < 9 * n; ++k) Jt[k] = J[k] + (al - 1.0) * DJ[k];
          for (int64_t k = 0; k < 3 * n; ++k) Et[k] = E[k] + (al - 1.0) * DE[k];
        } else {
        // Dynamic procedure with the test filter ασ.
        orc_uj_direct(kernel, al, n, X, n, X, G, S, Ut.data(), Jt.data(), nthreads);
        orc_estr_direct(kernel, al, sc->transposed, n, X, Jt.data(), S, n, X, G, S, Jt.data(),
                        Et.data(), nullptr, nthreads);
        }
        for (int64_t p = 0; p < nf; ++p) {
          double s1[3], s0[3];
          stretch(&Jt[9 * p], G + 3 * p, sc->transposed, s1);
          stretch(&J[9 * p], G + 3 * p, sc->transposed, s0);
          double nume = 0.0, deno = 0.0;
          for (int k = 0; k < 3; ++k) {
            nume += G[3 * p + k] * (s1[k] - s0[k]);
            deno += G[3 * p + k] * (Et[3 * p + k] - E[3 * p + k]);
          }
          nume *= 3.0 * al - 2.0;
          deno *= S[p] * S[p] * S[p] / zeta0;
          nume = sc->sfs_rlxf * nume + (1.0 - sc->sfs_rlxf) * C[3 * p + 1];
          deno = sc->sfs_rlxf * deno + (1.0 - sc->sfs_rlxf) * C[3 * p + 2];
          double cd = deno != 0.0 ? nume / deno : 0.0;
          if (sc->sfs_flags & VPM_SFS_FORCE_POSITIVE) cd = std::fabs(cd);
          if (sc->sfs_minC > 0 && std::fabs(cd) < sc->sfs_minC) cd = std::copysign(sc->sfs_minC, cd);
          if (sc->sfs_maxC > 0 && std::fabs(cd) > sc->sfs_maxC) cd = std::copysign(sc->sfs_maxC, cd);
          C[3 * p] = cd;
          C[3 * p + 1] = nume;
          C[3 * p + 2] = deno;
        }
      }
      if (sc->sfs_flags & VPM_SFS_CLIP_BACKSCATTER) {
        for (int64_t p = 0; p < nf; ++p) {
          double ge = G[3 * p] * E[3 * p] + G[3 * p + 1] * E[3 * p + 1] + G[3 * p + 2] * E[3 * p + 2];
          if (C[3 * p] * ge < 0.0) C[3 * p] = 0.0;
        }
      }
    }
    // rVPM update of the free particles (rvpm.md:196-236).
    for (int64_t p = 0; p < nf; ++p) {
      const double* gp = G + 3 * p;
      double s[3];
      stretch(&J[9 * p], gp, sc->transposed, s);
      const double gg = gp[0] * gp[0] + gp[1] * gp[1] + gp[2] * gp[2];
      const double sig = S[p];
      const double cz = sfs ? C[3 * p] * sig * sig * sig / zeta0 : 0.0;  // C_d/ζ_σ(0)
      const double* e = &E[3 * p];
      double Z = (f + g) / (1.0 + 3.0 * f) * (s[0] * gp[0] + s[1] * gp[1] + s[2] * gp[2]);
      if (sfs) Z -= f / (1.0 + 3.0 * f) * cz * (e[0] * gp[0] + e[1] * gp[1] + e[2] * gp[2]);
      Z = gg > 0.0 ? Z / gg : 0.0;
      for (int k = 0; k < 3; ++k) {
        Qx[3 * p + k] = a * Qx[3 * p + k] + dt * (U[3 * p + k] + sc->uinf[k]);
        QG[3 * p + k] = a * QG[3 * p + k] + dt * (s[k] - 3.0 * Z * gp[k] - (sfs ? cz * e[k] : 0.0));
      }
      Qs[p] = a * Qs[p] - dt * sig * Z;
    }
    for (int64_t p = 0; p < nf; ++p) {
      for (int k = 0; k < 3; ++k) {
        X[3 * p + k] += b * Qx[3 * p + k];
        G[3 * p + k] += b * QG[3 * p + k];
      }
      S[p] += b * Qs[p];
      if (sc->nu > 0.0) {
        Qs2[p] = a * Qs2[p] + dt * 2.0 * sc->nu;
        S[p] = std::sqrt(S[p] * S[p] + b * Qs2[p]);
      }
    }
  }
  if (E_out) std::memcpy(E_out, E.data(), sizeof(double) * 3 * n);
  return 0;
}

// Pedrizzetti relaxation of the free particles (vpm.pedrizzetti,
// src/FLOWUnsteady_simulation.jl:44,135; docs/src/theory/rvpm.md:363,388):
// Γ ← (1-r)Γ + r |Γ| ω̂ with ω = ∇×u from J at the particle.
int orc_relax_pedrizzetti(int64_t nf, double rlx, const double* J, double* G) {
  for (int64_t p = 0; p < nf; ++p) {
    const double* j = J + 9 * p;
    double w[3] = {j[7] - j[5], j[2] - j[6], j[3] - j[1]};
    double nw = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    double* gp = G + 3 * p;
    double ng = std::sqrt(gp[0] * gp[0] + gp[1] * gp[1] + gp[2] * gp[2]);
    if (nw == 0.0) continue;
    for (int k = 0; k < 3; ++k) gp[k] = (1.0 - rlx) * gp[k] + rlx * ng * w[k] / nw;
  }
  return 0;
}

// Diagnostics (layout VPM_DIAG_*): enstrophy from an ω pair pass, impulse, ΣΓ,
// C_d statistics over the free particles with C_d != 0, mean σ, non-finite count.
int orc_diagnostics(int kernel, int64_t n, int64_t n_static, const double* X, const double* G,
                    const double* S, const double* C, double* out, int nthreads) {
  std::vector<double> om(3 * n);
  orc_estr_direct(kernel, 1.0, 1, n, X, nullptr, S, n, X, G, S, nullptr, nullptr, om.data(),
                  nthreads);
  for (int k = 0; k < VPM_DIAG_COUNT; ++k) out[k] = 0.0;
  double ens = 0.0;
  for (int64_t p = 0; p < n; ++p) {
    ens += G[3 * p] * om[3 * p] + G[3 * p + 1] * om[3 * p + 1] + G[3 * p + 2] * om[3 * p + 2];
    const double* x = X + 3 * p;
    const double* gp = G + 3 * p;
    out[VPM_DIAG_IMPULSE_X] += 0.5 * (x[1] * gp[2] - x[2] * gp[1]);
    out[VPM_DIAG_IMPULSE_Y] += 0.5 * (x[2] * gp[0] - x[0] * gp[2]);
    out[VPM_DIAG_IMPULSE_Z] += 0.5 * (x[0] * gp[1] - x[1] * gp[0]);
    for (int k = 0; k < 3; ++k) out[VPM_DIAG_GAMMA_X + k] += gp[k];
    out[VPM_DIAG_SIGMA_MEAN] += S[p];
    bool fin = std::isfinite(x[0]) && std::isfinite(x[1]) && std::isfinite(x[2]) &&
               std::isfinite(gp[0]) && std::isfinite(gp[1]) && std::isfinite(gp[2]) &&
               std::isfinite(S[p]);
    if (!fin) out[VPM_DIAG_NONFINITE] += 1.0;
  }
  out[VPM_DIAG_ENSTROPHY] = 0.5 * ens;
  out[VPM_DIAG_SIGMA_MEAN] = n > 0 ? out[VPM_DIAG_SIGMA_MEAN] / n : 0.0;
  // C_d statistics over the free particles with C_d != 0 (vpm.monitor_Cd's
  // record, src/FLOWUnsteady_monitors.jl:697-703): mean, standard deviation,
  // skewness and excess kurtosis as population moments about the mean (two
  // passes), minimum and maximum; the zero ratio over all free particles.
  const int64_t nf = n - n_static;
  double s1 = 0, mn = 0, mx = 0;
  int64_t nz = 0, cnt = 0;
  for (int64_t p = 0; p < nf && C; ++p) {
    double c = C[3 * p];
    if (c == 0.0) { ++nz; continue; }
    if (cnt == 0) { mn = mx = c; }
    mn = std::min(mn, c); mx = std::max(mx, c);
    s1 += c; ++cnt;
  }
  if (cnt > 0) {
    const double mean = s1 / cnt;
    double m2 = 0, m3 = 0, m4 = 0;
    for (int64_t p = 0; p < nf; ++p) {
      const double c = C[3 * p];
      if (c == 0.0) continue;
      const double d = c - mean, d2 = d * d;
      m2 += d2; m3 += d2 * d; m4 += d2 * d2;
    }
    m2 /= cnt; m3 /= cnt; m4 /= cnt;
    out[VPM_DIAG_CD_MEAN] = mean;
    out[VPM_DIAG_CD_STD] = std::sqrt(m2);
    out[VPM_DIAG_CD_MIN] = mn;
    out[VPM_DIAG_CD_MAX] = mx;
    if (m2 > 0.0) {
      out[VPM_DIAG_CD_SKEW] = m3 / (m2 * std::sqrt(m2));
      out[VPM_DIAG_CD_KURT] = m4 / (m2 * m2) - 3.0;
    }
  }
  out[VPM_DIAG_CD_ZERO_RATIO] = nf > 0 && C ? double(nz) / double(nf) : 0.0;
  return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
