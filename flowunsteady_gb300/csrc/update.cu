// update.cu — the O(N), HBM-bound FP64 kernels of a time step.
//
// State layout (FP64 SoA, leading dimension ld = capacity): X[k*ld+i], Γ[k*ld+i],
// σ[i]; U[k*ld+i]; J[(3a+b)*ld+i] = dU_a/dx_b; E_str[k*ld+i]; C[k*ld+i] with
// k = 0: C_d, 1: <Γ·L>, 2: <Γ·m>; RK registers Q[r*ld+i], r = 0..2 x, 3..5 Γ,
// 6 σ, 7 σ² (core spreading).
//
// Restated from FLOWUnsteady docs/src/theory/rvpm.md:
//   stretching S = (Γ·∇)u (classic) or its transpose (:363, default transposed);
//   dΓ/dt = S - 3Z Γ - C_d/ζ_σ(0) E_str,  dσ/dt = -σ Z,
//   Z = [(f+g)/(1+3f) S·Γ - f/(1+3f) C_d/ζ_σ(0) E_str·Γ]/|Γ|²          (:196-236)
//   (equivalent to Eqs. 7-8: (g+f)/(1/3+f) = 3(g+f)/(1+3f));
//   dynamic C_d = <Γ·L>/<Γ·m> with backscatter clipping                  (:264-297);
//   low-storage RK3 (Williamson 1980) and core spreading d(σ²)/dt = 2ν   (:364-367).
#include "internal.h"
#include "update.h"
#include "vpm_device.cuh"

namespace vpm {

__device__ inline void stretch_dev(const double* J, int64_t ld, int64_t i, double v0, double v1,
                                   double v2, int transposed, double& s0, double& s1,
                                   double& s2) {
  const double j00 = J[0 * ld + i], j01 = J[1 * ld + i], j02 = J[2 * ld + i];
  const double j10 = J[3 * ld + i], j11 = J[4 * ld + i], j12 = J[5 * ld + i];
  const double j20 = J[6 * ld + i], j21 = J[7 * ld + i], j22 = J[8 * ld + i];
  if (transposed) {
    s0 = j00 * v0 + j10 * v1 + j20 * v2;
    s1 = j01 * v0 + j11 * v1 + j21 * v2;
    s2 = j02 * v0 + j12 * v1 + j22 * v2;
  } else {
    s0 = j00 * v0 + j01 * v1 + j02 * v2;
    s1 = j10 * v0 + j11 * v1 + j12 * v2;
    s2 = j20 * v0 + j21 * v1 + j22 * v2;
  }
}

// v = S(J, Γ) at every particle (the per-source term of the E_str pass).
__global__ void stretch_v_kernel(int64_t n, int64_t ld, const double* __restrict__ J,
                                 const double* __restrict__ G, int transposed, double* V) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s0, s1, s2;
  stretch_dev(J, ld, i, G[i], G[ld + i], G[2 * ld + i], transposed, s0, s1, s2);
  V[i] = s0; V[ld + i] = s1; V[2 * ld + i] = s2;
}

// E_str = S(J_p, Ω_p) - V_p from the raw ζ sums (rows 0..2 Ω, 3..5 V).
__global__ void estr_finish_kernel(int64_t n, int64_t ld, const double* __restrict__ raw,
                                   const double* __restrict__ J, int transposed, double* E) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s0, s1, s2;
  stretch_dev(J, ld, i, raw[i], raw[ld + i], raw[2 * ld + i], transposed, s0, s1, s2);
  E[i] = s0 - raw[3 * ld + i];
  E[ld + i] = s1 - raw[4 * ld + i];
  E[2 * ld + i] = s2 - raw[5 * ld + i];
}

// v = S(J, Γ) and w = S(DJ, Γ) (per-source terms of the α-derivative ζ pass).
__global__ void stretch_vw_kernel(int64_t n, int64_t ld, const double* __restrict__ J,
                                  const double* __restrict__ DJ, const double* __restrict__ G,
                                  int transposed, double* V, double* W) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double g0 = G[i], g1 = G[ld + i], g2 = G[2 * ld + i];
  double s0, s1, s2;
  stretch_dev(J, ld, i, g0, g1, g2, transposed, s0, s1, s2);
  V[i] = s0; V[ld + i] = s1; V[2 * ld + i] = s2;
  stretch_dev(DJ, ld, i, g0, g1, g2, transposed, s0, s1, s2);
  W[i] = s0; W[ld + i] = s1; W[2 * ld + i] = s2;
}

// E = S(J, Ω) - V and DE = S(DJ, Ω) + S(J, DΩ) - DV from the raw sums of the
// α-derivative ζ pass (rows 0..2 Ω, 3..5 V, 6..8 DΩ, 9..11 DV).
__global__ void estr_finish_d_kernel(int64_t n, int64_t ld, const double* __restrict__ raw,
                                     const double* __restrict__ J, const double* __restrict__ DJ,
                                     int transposed, double* E, double* DE) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double o0 = raw[i], o1 = raw[ld + i], o2 = raw[2 * ld + i];
  double s0, s1, s2, t0, t1, t2;
  stretch_dev(J, ld, i, o0, o1, o2, transposed, s0, s1, s2);
  E[i] = s0 - raw[3 * ld + i];
  E[ld + i] = s1 - raw[4 * ld + i];
  E[2 * ld + i] = s2 - raw[5 * ld + i];
  stretch_dev(DJ, ld, i, o0, o1, o2, transposed, s0, s1, s2);
  stretch_dev(J, ld, i, raw[6 * ld + i], raw[7 * ld + i], raw[8 * ld + i], transposed, t0, t1, t2);
  DE[i] = s0 + t0 - raw[9 * ld + i];
  DE[ld + i] = s1 + t1 - raw[10 * ld + i];
  DE[2 * ld + i] = s2 + t2 - raw[11 * ld + i];
}

// Non-finite test on the exponent bits (integer pipe; FP64 compares issue on
// the FP64 pipe, 1/64 of the FP32 rate on GB300).
__device__ inline bool finite_bits(double x) {
  return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000;
}

// Pseudo-three-level dynamic coefficient (once per step, first RK stage):
//   nume = (3α-2) Γ·[S(J(ασ)) - S(J(σ))],  deno = σ³/ζ(0) Γ·[E(ασ) - E(σ)],
//   Lagrangian average with rlxf, C_d = nume/deno, |C_d| forced/limited.
// Particles [0, nv); those with a nonzero static flag (stat may be null) are skipped.
__global__ void __launch_bounds__(256) sfs_dynamic_kernel(
    int64_t nv, const uint8_t* __restrict__ stat, int64_t ld, const double* __restrict__ G,
    const double* __restrict__ S, const double* __restrict__ J, const double* __restrict__ Jt,
    const double* __restrict__ E, const double* __restrict__ Et, double* __restrict__ C,
    SfsParams p) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv || (stat && stat[i])) return;
  const double g0 = G[i], g1 = G[ld + i], g2 = G[2 * ld + i];
  double a0, a1, a2, b0, b1, b2;
  double nume, deno;
  if (p.analytic) {
    // Jt = DJ, Et = DE: the test-filter differences are (α-1)·D to first order.
    const double h = p.alpha - 1.0;
    stretch_dev(Jt, ld, i, g0, g1, g2, p.transposed, a0, a1, a2);
    nume = h * (g0 * a0 + g1 * a1 + g2 * a2);
    deno = h * (g0 * Et[i] + g1 * Et[ld + i] + g2 * Et[2 * ld + i]);
  } else {
    stretch_dev(Jt, ld, i, g0, g1, g2, p.transposed, a0, a1, a2);
    stretch_dev(J, ld, i, g0, g1, g2, p.transposed, b0, b1, b2);
    nume = g0 * (a0 - b0) + g1 * (a1 - b1) + g2 * (a2 - b2);
    deno = g0 * (Et[i] - E[i]) + g1 * (Et[ld + i] - E[ld + i]) +
           g2 * (Et[2 * ld + i] - E[2 * ld + i]);
  }
  const double sg = S[i];
  nume *= 3.0 * p.alpha - 2.0;
  deno *= sg * sg * sg * p.inv_zeta0;
  nume = p.rlxf * nume + (1.0 - p.rlxf) * C[ld + i];
  deno = p.rlxf * deno + (1.0 - p.rlxf) * C[2 * ld + i];
  double cd = deno != 0.0 ? nume / deno : 0.0;
  if (p.force_positive) cd = fabs(cd);
  if (p.minC > 0.0 && fabs(cd) < p.minC) cd = copysign(p.minC, cd);
  if (p.maxC > 0.0 && fabs(cd) > p.maxC) cd = copysign(p.maxC, cd);
  C[i] = cd;
  C[ld + i] = nume;
  C[2 * ld + i] = deno;
}

// Backscatter clipping on its own (vpm.clipping_backscatter): C_d = 0 where
// C_d Γ·E_str < 0.
__global__ void sfs_clip_kernel(int64_t nv, const uint8_t* __restrict__ stat, int64_t ld,
                                const double* __restrict__ G, const double* __restrict__ E,
                                double* __restrict__ C) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv || (stat && stat[i])) return;
  const double ge = G[i] * E[i] + G[ld + i] * E[ld + i] + G[2 * ld + i] * E[2 * ld + i];
  if (C[i] * ge < 0.0) C[i] = 0.0;
}

__global__ void sfs_constant_kernel(int64_t nv, const uint8_t* __restrict__ stat, double cd,
                                    double* C) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < nv && !(stat && stat[i])) C[i] = cd;
}

// One RK stage (or an Euler step: a = 0, b = 1) of the free particles, fused:
// backscatter clipping, rVPM right-hand side, low-storage register update,
// state update, core spreading, non-finite detection.  FP64 throughout; the
// FP64 pipe (not HBM) bounds it, so each particle forms the right-hand side
// once, one reciprocal of |Γ|² and (with core spreading) one square root.
// Particles [0, nv); those with a nonzero static flag (stat may be null) are skipped.
__global__ void __launch_bounds__(256) rk_update_kernel(
    int64_t nv, const uint8_t* __restrict__ stat, int64_t ld, double* __restrict__ X,
    double* __restrict__ G, double* __restrict__ S, const double* __restrict__ U,
    const double* __restrict__ J, const double* __restrict__ E, double* __restrict__ C,
    double* __restrict__ Q, UpdateParams p, int* status) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv || (stat && stat[i])) return;
  const double g0 = G[i], g1 = G[ld + i], g2 = G[2 * ld + i];
  const double sg = S[i];
  double s0, s1, s2;
  stretch_dev(J, ld, i, g0, g1, g2, p.transposed, s0, s1, s2);
  const double gg = g0 * g0 + g1 * g1 + g2 * g2;
  double Z = p.zs * (s0 * g0 + s1 * g1 + s2 * g2);
  double cz = 0.0, e0 = 0.0, e1 = 0.0, e2 = 0.0;
  if (p.sfs) {
    e0 = E[i]; e1 = E[ld + i]; e2 = E[2 * ld + i];
    double cd = C[i];
    const double ge = g0 * e0 + g1 * e1 + g2 * e2;
    if (p.clip_backscatter && cd * ge < 0.0) {
      cd = 0.0;
      C[i] = 0.0;
    }
    cz = cd * (sg * sg) * (sg * p.inv_zeta0);   // C_d/ζ_σ(0)
    Z -= p.ze * cz * ge;
  }
  Z = gg > 0.0 ? Z * (1.0 / gg) : 0.0;
  const double a = p.a, b = p.b, dt = p.dt;
  // position
  const double q0 = a * Q[0 * ld + i] + dt * (U[i] + p.uinf0);
  const double q1 = a * Q[1 * ld + i] + dt * (U[ld + i] + p.uinf1);
  const double q2 = a * Q[2 * ld + i] + dt * (U[2 * ld + i] + p.uinf2);
  Q[0 * ld + i] = q0; Q[1 * ld + i] = q1; Q[2 * ld + i] = q2;
  const double x0 = X[i] + b * q0, x1 = X[ld + i] + b * q1, x2 = X[2 * ld + i] + b * q2;
  X[i] = x0; X[ld + i] = x1; X[2 * ld + i] = x2;
  // strength
  const double z3 = 3.0 * Z;
  const double r0 = a * Q[3 * ld + i] + dt * (s0 - z3 * g0 - cz * e0);
  const double r1 = a * Q[4 * ld + i] + dt * (s1 - z3 * g1 - cz * e1);
  const double r2 = a * Q[5 * ld + i] + dt * (s2 - z3 * g2 - cz * e2);
  Q[3 * ld + i] = r0; Q[4 * ld + i] = r1; Q[5 * ld + i] = r2;
  const double n0 = g0 + b * r0, n1 = g1 + b * r1, n2 = g2 + b * r2;
  G[i] = n0; G[ld + i] = n1; G[2 * ld + i] = n2;
  // core size: stretching, then core spreading
  const double qs = a * Q[6 * ld + i] - dt * sg * Z;
  Q[6 * ld + i] = qs;
  double ns = sg + b * qs;
  if (p.nu > 0.0) {
    const double qn = a * Q[7 * ld + i] + dt * 2.0 * p.nu;
    Q[7 * ld + i] = qn;
    ns = sqrt(ns * ns + b * qn);
  }
  S[i] = ns;
  if (!(finite_bits(n0) && finite_bits(n1) && finite_bits(n2) && finite_bits(ns) &&
        finite_bits(x0) && finite_bits(x1) && finite_bits(x2)))
    atomicOr(status, STATUS_NONFINITE);
}

// Pedrizzetti relaxation: Γ <- (1-r)Γ + r|Γ| ω/|ω|, ω = ∇×u from J.
__global__ void relax_kernel(int64_t nv, const uint8_t* __restrict__ stat, int64_t ld,
                             const double* __restrict__ J, double* G, double r) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv || (stat && stat[i])) return;
  const double w0 = J[7 * ld + i] - J[5 * ld + i];
  const double w1 = J[2 * ld + i] - J[6 * ld + i];
  const double w2 = J[3 * ld + i] - J[1 * ld + i];
  const double nw = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
  if (nw == 0.0) return;
  const double g0 = G[i], g1 = G[ld + i], g2 = G[2 * ld + i];
  const double ng = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
  G[i] = (1.0 - r) * g0 + r * ng * w0 / nw;
  G[ld + i] = (1.0 - r) * g1 + r * ng * w1 / nw;
  G[2 * ld + i] = (1.0 - r) * g2 + r * ng * w2 / nw;
}

__global__ void zero_kernel(double* p, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

// ------------------------------------------------------------ reductions --
// Deterministic two-level FP64 reductions: kRedBlocks blocks each reduce a
// fixed, strided share of the particles in a fixed tree order into a partial
// row; one block then reduces the rows in order.
constexpr int kRedThreads = 256;

struct DiagAcc {
  double v[kDiagSlots];
};

__device__ inline void diag_combine(DiagAcc& a, const DiagAcc& b) {
#pragma unroll
  for (int k = 0; k < kDiagSlots; ++k) {
    if (k == DS_CMIN) a.v[k] = fmin(a.v[k], b.v[k]);
    else if (k == DS_CMAX) a.v[k] = fmax(a.v[k], b.v[k]);
    else a.v[k] += b.v[k];
  }
}

__device__ inline void diag_identity(DiagAcc& a) {
#pragma unroll
  for (int k = 0; k < kDiagSlots; ++k) a.v[k] = 0.0;
  a.v[DS_CMIN] = INFINITY;
  a.v[DS_CMAX] = -INFINITY;
}

__device__ inline void block_reduce(DiagAcc& acc, DiagAcc* sh) {
  const int t = threadIdx.x;
  sh[t] = acc;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (t < s) {
      DiagAcc o = sh[t + s];
      diag_combine(sh[t], o);
    }
    __syncthreads();
  }
  acc = sh[0];
}

// raw: ζ sums (rows 0..2 Ω without self) or null (no enstrophy).
// C_d statistics cover the free particles: [0, nf) without flags, or every
// particle whose static flag is zero (stat non-null).
__global__ void __launch_bounds__(kRedThreads) diag_partial_kernel(
    int64_t n, int64_t nf, const uint8_t* __restrict__ stat, int64_t ld,
    const double* __restrict__ X, const double* __restrict__ G, const double* __restrict__ S,
    const double* __restrict__ C, const double* __restrict__ raw, double zeta0,
    double* partial) {
  __shared__ DiagAcc sh[kRedThreads];
  DiagAcc acc;
  diag_identity(acc);
  for (int64_t i = int64_t(blockIdx.x) * kRedThreads + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kRedThreads) {
    const double x0 = X[i], x1 = X[ld + i], x2 = X[2 * ld + i];
    const double g0 = G[i], g1 = G[ld + i], g2 = G[2 * ld + i];
    const double sg = S[i];
    if (raw) {
      const double self = zeta0 / (sg * sg * sg);
      acc.v[DS_ENS] += 0.5 * (g0 * (raw[i] + self * g0) + g1 * (raw[ld + i] + self * g1) +
                              g2 * (raw[2 * ld + i] + self * g2));
    }
    acc.v[DS_IX] += 0.5 * (x1 * g2 - x2 * g1);
    acc.v[DS_IY] += 0.5 * (x2 * g0 - x0 * g2);
    acc.v[DS_IZ] += 0.5 * (x0 * g1 - x1 * g0);
    acc.v[DS_GX] += g0;
    acc.v[DS_GY] += g1;
    acc.v[DS_GZ] += g2;
    acc.v[DS_SIG] += sg;
    const bool fin = isfinite(x0) && isfinite(x1) && isfinite(x2) && isfinite(g0) &&
                     isfinite(g1) && isfinite(g2) && isfinite(sg);
    acc.v[DS_NONFIN] += fin ? 0.0 : 1.0;
    if (C && (stat ? !stat[i] : i < nf)) {
      const double c = C[i];
      if (c == 0.0) {
        acc.v[DS_CZERO] += 1.0;
      } else {
        const double c2 = c * c;
        acc.v[DS_CCNT] += 1.0;
        acc.v[DS_CSUM] += c;
        acc.v[DS_CSUM2] += c2;
        acc.v[DS_CSUM3] += c2 * c;
        acc.v[DS_CSUM4] += c2 * c2;
        acc.v[DS_CMIN] = fmin(acc.v[DS_CMIN], c);
        acc.v[DS_CMAX] = fmax(acc.v[DS_CMAX], c);
      }
    }
  }
  block_reduce(acc, sh);
  if (threadIdx.x == 0)
    for (int k = 0; k < kDiagSlots; ++k) partial[int64_t(blockIdx.x) * kDiagSlots + k] = acc.v[k];
}

__global__ void __launch_bounds__(kRedThreads) diag_final_kernel(int nblocks,
                                                                 const double* __restrict__ partial,
                                                                 double* out) {
  __shared__ DiagAcc sh[kRedThreads];
  DiagAcc acc;
  diag_identity(acc);
  for (int b = threadIdx.x; b < nblocks; b += kRedThreads) {
    DiagAcc o;
    for (int k = 0; k < kDiagSlots; ++k) o.v[k] = partial[int64_t(b) * kDiagSlots + k];
    diag_combine(acc, o);
  }
  block_reduce(acc, sh);
  if (threadIdx.x == 0)
    for (int k = 0; k < kDiagSlots; ++k) out[k] = acc.v[k];
}

// Σ|Γ| x and Σ|Γ| over [i0, i1) -> out[4] (same two-level structure).
__global__ void __launch_bounds__(kRedThreads) centroid_partial_kernel(
    int64_t i0, int64_t i1, int64_t ld, const double* __restrict__ X,
    const double* __restrict__ G, double* partial) {
  __shared__ DiagAcc sh[kRedThreads];
  DiagAcc acc;
  diag_identity(acc);
  acc.v[DS_CMIN] = 0.0;
  acc.v[DS_CMAX] = 0.0;
  for (int64_t i = i0 + int64_t(blockIdx.x) * kRedThreads + threadIdx.x; i < i1;
       i += int64_t(gridDim.x) * kRedThreads) {
    const double g0 = G[i], g1 = G[ld + i], g2 = G[2 * ld + i];
    const double w = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
    acc.v[0] += w * X[i];
    acc.v[1] += w * X[ld + i];
    acc.v[2] += w * X[2 * ld + i];
    acc.v[3] += w;
  }
  block_reduce(acc, sh);
  if (threadIdx.x == 0)
    for (int k = 0; k < kDiagSlots; ++k) partial[int64_t(blockIdx.x) * kDiagSlots + k] = acc.v[k];
}

// ---------------------------------------------------------------- launchers --
static inline int grid_for(int64_t n, int bs) { return int((n + bs - 1) / bs); }

cudaError_t launch_stretch_v(int64_t n, int64_t ld, const double* J, const double* G,
                             int transposed, double* V, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  stretch_v_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, ld, J, G, transposed, V);
  return cudaGetLastError();
}

cudaError_t launch_estr_finish(int64_t n, int64_t ld, const double* raw, const double* J,
                               int transposed, double* E, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  estr_finish_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, ld, raw, J, transposed, E);
  return cudaGetLastError();
}

cudaError_t launch_stretch_vw(int64_t n, int64_t ld, const double* J, const double* DJ,
                              const double* G, int transposed, double* V, double* W,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  stretch_vw_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, ld, J, DJ, G, transposed, V, W);
  return cudaGetLastError();
}

cudaError_t launch_estr_finish_d(int64_t n, int64_t ld, const double* raw, const double* J,
                                 const double* DJ, int transposed, double* E, double* DE,
                                 cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  estr_finish_d_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, ld, raw, J, DJ, transposed, E, DE);
  return cudaGetLastError();
}

cudaError_t launch_sfs_dynamic(int64_t nv, const uint8_t* stat, int64_t ld, const double* G,
                               const double* S, const double* J, const double* Jt,
                               const double* E, const double* Et, double* C, const SfsParams& p,
                               cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  sfs_dynamic_kernel<<<grid_for(nv, 256), 256, 0, st>>>(nv, stat, ld, G, S, J, Jt, E, Et, C, p);
  return cudaGetLastError();
}

cudaError_t launch_sfs_clip(int64_t nv, const uint8_t* stat, int64_t ld, const double* G,
                            const double* E, double* C, cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  sfs_clip_kernel<<<grid_for(nv, 256), 256, 0, st>>>(nv, stat, ld, G, E, C);
  return cudaGetLastError();
}

cudaError_t launch_sfs_constant(int64_t nv, const uint8_t* stat, double cd, double* C,
                                cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  sfs_constant_kernel<<<grid_for(nv, 256), 256, 0, st>>>(nv, stat, cd, C);
  return cudaGetLastError();
}

cudaError_t launch_rk_update(int64_t nv, const uint8_t* stat, int64_t ld, double* X, double* G,
                             double* S, const double* U, const double* J, const double* E,
                             double* C, double* Q, const UpdateParams& p, int* status,
                             cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  rk_update_kernel<<<grid_for(nv, 256), 256, 0, st>>>(nv, stat, ld, X, G, S, U, J, E, C, Q, p,
                                                      status);
  return cudaGetLastError();
}

cudaError_t launch_relax(int64_t nv, const uint8_t* stat, int64_t ld, const double* J, double* G,
                         double r, cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  relax_kernel<<<grid_for(nv, 256), 256, 0, st>>>(nv, stat, ld, J, G, r);
  return cudaGetLastError();
}

cudaError_t launch_zero(double* p, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  zero_kernel<<<grid_for(n, 256), 256, 0, st>>>(p, n);
  return cudaGetLastError();
}

cudaError_t launch_diagnostics(int64_t n, int64_t nf, const uint8_t* stat, int64_t ld,
                               const double* X, const double* G, const double* S, const double* C,
                               const double* raw, double zeta0, double* partial, double* out,
                               cudaStream_t st) {
  diag_partial_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(n, nf, stat, ld, X, G, S, C, raw, zeta0,
                                                          partial);
  diag_final_kernel<<<1, kRedThreads, 0, st>>>(kRedBlocks, partial, out);
  return cudaGetLastError();
}

cudaError_t launch_centroid(int64_t i0, int64_t i1, int64_t ld, const double* X, const double* G,
                            double* partial, double* out, cudaStream_t st) {
  centroid_partial_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(i0, i1, ld, X, G, partial);
  diag_final_kernel<<<1, kRedThreads, 0, st>>>(kRedBlocks, partial, out);
  return cudaGetLastError();
}

}  // namespace vpm
