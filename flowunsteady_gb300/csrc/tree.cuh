// tree.cuh — Cartesian multipole arithmetic of the GPU treecode (tree.cu).
//
// The far field of the particles in a cell is taken from the vector potential
// of the singular kernel,
//   ψ(x) = 1/(4π) Σ_j Γ_j / |x - y_j|,   U = ∇ × ψ,   J = ∇U,
// expanded about the cell centre c.  With R = x - c and the Taylor
// coefficients of 1/|x - y| in the source displacement,
//   b_k(R) = (1/k!) ∂_y^k (1/|x - y|) at y = c,      1/|x - y| = Σ_k b_k(R) (y - c)^k,
// and the cell moments M_k^m = Σ_j Γ_j^m (y_j - c)^k (|k| <= P), the potential
// is ψ_m(x) = 1/(4π) Σ_k M_k^m b_k(R), and since ∂_{x_i} b_k = -(k_i + 1) b_{k+e_i},
//   ∂_i ψ_m     = -1/(4π) Σ_k (k_i + 1) M_k^m b_{k+e_i},
//   ∂_i ∂_j ψ_m =  1/(4π) Σ_k (k_i + 1)(k_j + δ_ij + 1) M_k^m b_{k+e_i+e_j}.
// The b_k follow from the recurrence for 1/|R| (Lindsay & Krasny, J. Comput.
// Phys. 172 (2001), written here for the coefficients in y):
//   b_0 = 1/|R|,
//   |k| |R|² b_k = (2|k| - 1) Σ_i R_i b_{k-e_i} - (|k| - 1) Σ_i b_{k-2e_i}.
// Multi-indices are stored in graded order (midx): all |k| = n after all
// |k| < n; within an order by decreasing k1, then decreasing k2.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace vpm {

// Number of multi-indices with |k| <= q.
__host__ __device__ constexpr int ncoef(int q) { return (q + 1) * (q + 2) * (q + 3) / 6; }

// Position of k = (a, b, c) in graded order.
__host__ __device__ constexpr int midx(int a, int b, int c) {
  return (a + b + c) * (a + b + c + 1) * (a + b + c + 2) / 6 + (b + c) * (b + c + 1) / 2 + c;
}

// Monomials d^k for |k| <= Q in graded order: p[midx(k)] = dx^a dy^b dz^c.
template <int Q, typename R>
__device__ __forceinline__ void monomials(R dx, R dy, R dz, R (&p)[ncoef(Q)]) {
  p[0] = R(1);
#pragma unroll
  for (int n = 1; n <= Q; ++n)
#pragma unroll
    for (int a = n; a >= 0; --a)
#pragma unroll
      for (int b = n - a; b >= 0; --b) {
        const int c = n - a - b;
        if (a > 0) p[midx(a, b, c)] = p[midx(a - 1, b, c)] * dx;
        else if (b > 0) p[midx(a, b, c)] = p[midx(a, b - 1, c)] * dy;
        else p[midx(a, b, c)] = p[midx(a, b, c - 1)] * dz;
      }
}

// Taylor coefficients b_k(R) of 1/|x - y| for |k| <= Q (see the header).
template <int Q, typename R>
__device__ __forceinline__ void taylor_coefficients(R rx, R ry, R rz, R (&bk)[ncoef(Q)]) {
  const R r2 = rx * rx + ry * ry + rz * rz;
  const R ir2 = R(1) / r2;
  bk[0] = sqrt(ir2);
#pragma unroll
  for (int n = 1; n <= Q; ++n) {
    const R f1 = R(2 * n - 1) * ir2 / R(n);
    const R f2 = R(n - 1) * ir2 / R(n);
#pragma unroll
    for (int a = n; a >= 0; --a)
#pragma unroll
      for (int b = n - a; b >= 0; --b) {
        const int c = n - a - b;
        R s1 = R(0), s2 = R(0);
        if (a > 0) s1 += rx * bk[midx(a - 1, b, c)];
        if (b > 0) s1 += ry * bk[midx(a, b - 1, c)];
        if (c > 0) s1 += rz * bk[midx(a, b, c - 1)];
        if (a > 1) s2 += bk[midx(a - 2, b, c)];
        if (b > 1) s2 += bk[midx(a, b - 2, c)];
        if (c > 1) s2 += bk[midx(a, b, c - 2)];
        bk[midx(a, b, c)] = f1 * s1 - f2 * s2;
      }
  }
}

// Contract the moments of one cell (mom[m·NC + k], NC = ncoef(P)) with the
// coefficients at R = x - c: dpsi[3i + m] += Σ_k -(k_i+1) M_k^m b_{k+e_i} and
// ddpsi[3·s + m] += Σ_k (k_i+1)(k_j+δ_ij+1) M_k^m b_{k+e_i+e_j} for the six
// pairs s = (00, 01, 02, 11, 12, 22), both without the 1/(4π).
template <int P, typename R, typename M>
__device__ __forceinline__ void m2p_accumulate(const R (&bk)[ncoef(P + 2)], const M* mom,
                                               R (&dpsi)[9], R (&ddpsi)[18]) {
  constexpr int NC = ncoef(P);
#pragma unroll
  for (int n = 0; n <= P; ++n)
#pragma unroll
    for (int a = n; a >= 0; --a)
#pragma unroll
      for (int b = n - a; b >= 0; --b) {
        const int c = n - a - b;
        const int k = midx(a, b, c);
        const R m0 = R(mom[k]), m1 = R(mom[NC + k]), m2 = R(mom[2 * NC + k]);
        const R g0 = R(-(a + 1)) * bk[midx(a + 1, b, c)];
        const R g1 = R(-(b + 1)) * bk[midx(a, b + 1, c)];
        const R g2 = R(-(c + 1)) * bk[midx(a, b, c + 1)];
        dpsi[0] += g0 * m0; dpsi[1] += g0 * m1; dpsi[2] += g0 * m2;
        dpsi[3] += g1 * m0; dpsi[4] += g1 * m1; dpsi[5] += g1 * m2;
        dpsi[6] += g2 * m0; dpsi[7] += g2 * m1; dpsi[8] += g2 * m2;
        const R h00 = R((a + 1) * (a + 2)) * bk[midx(a + 2, b, c)];
        const R h01 = R((a + 1) * (b + 1)) * bk[midx(a + 1, b + 1, c)];
        const R h02 = R((a + 1) * (c + 1)) * bk[midx(a + 1, b, c + 1)];
        const R h11 = R((b + 1) * (b + 2)) * bk[midx(a, b + 2, c)];
        const R h12 = R((b + 1) * (c + 1)) * bk[midx(a, b + 1, c + 1)];
        const R h22 = R((c + 1) * (c + 2)) * bk[midx(a, b, c + 2)];
        ddpsi[0] += h00 * m0;  ddpsi[1] += h00 * m1;  ddpsi[2] += h00 * m2;
        ddpsi[3] += h01 * m0;  ddpsi[4] += h01 * m1;  ddpsi[5] += h01 * m2;
        ddpsi[6] += h02 * m0;  ddpsi[7] += h02 * m1;  ddpsi[8] += h02 * m2;
        ddpsi[9] += h11 * m0;  ddpsi[10] += h11 * m1; ddpsi[11] += h11 * m2;
        ddpsi[12] += h12 * m0; ddpsi[13] += h12 * m1; ddpsi[14] += h12 * m2;
        ddpsi[15] += h22 * m0; ddpsi[16] += h22 * m1; ddpsi[17] += h22 * m2;
      }
}

// U = ∇ × ψ and J_ab = ∂_b U_a from ∂ψ and ∂∂ψ (already scaled by 1/(4π)).
template <typename R>
__device__ __forceinline__ void curl_from_potential(const R (&dp)[9], const R (&dd)[18], R (&u)[3],
                                                    R (&j)[9]) {
  // dp[3i + m] = ∂_i ψ_m;  dd[3s + m] with s(i,j) = 00 0, 01 1, 02 2, 11 3, 12 4, 22 5.
  auto D = [&](int i, int jj, int m) {
    const int lo = i < jj ? i : jj, hi = i < jj ? jj : i;
    const int s = lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
    return dd[3 * s + m];
  };
  u[0] = dp[3 * 1 + 2] - dp[3 * 2 + 1];
  u[1] = dp[3 * 2 + 0] - dp[3 * 0 + 2];
  u[2] = dp[3 * 0 + 1] - dp[3 * 1 + 0];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    j[0 * 3 + b] = D(b, 1, 2) - D(b, 2, 1);
    j[1 * 3 + b] = D(b, 2, 0) - D(b, 0, 2);
    j[2 * 3 + b] = D(b, 0, 1) - D(b, 1, 0);
  }
}


// ---------------------------------------------------------- local expansions --
// A far cell of centre c whose box is at least as large as the target group's
// (radius h, centre z) is taken once per group as a local expansion of ψ about
// z instead of once per target (M2P).  With R0 = z - c = |R0| R̂, ρ = 1/|R0|,
// s = hρ and the homogeneity b_j(R0) = ρ^{|j|+1} b_j(R̂), the expansion
//   ψ_m(z + y) = Σ_{|n|<=Q} L_n^m (y/h)^n,
//   L_n^m = ρ (-s)^{|n|} / n! · Σ_{|k|<=P} [M_k^m ρ^{|k|} / k!] [(k+n)! b_{k+n}(R̂)]
// follows from L_n^m h^{-|n|} = Σ_k M_k^m (-1)^{|n|} C(k+n, n) b_{k+n}(R0)
// (∂_{R_i} b_k = -(k_i + 1) b_{k+e_i}), with C(k+n, n) = (k+n)!/(k! n!).  Every
// factor is O(1) in these scaled variables (|R̂| = 1, s < θ), so FP32 holds
// them for any length unit.  B̃_j = j! b_j(R̂) follows from the recurrence of
// the header multiplied by j!:
//   B̃_0 = 1,  |j| B̃_j = (2|j| - 1) Σ_i j_i R̂_i B̃_{j-e_i} - (|j| - 1) Σ_i j_i (j_i - 1) B̃_{j-2e_i}.
// At a target x = z + h u (L2P), with the 1/(4π) left out as in m2p_accumulate,
//   ∂_i ψ_m     = (1/h)  Σ_n n_i L_n^m u^{n-e_i},
//   ∂_i ∂_j ψ_m = (1/h²) Σ_n n_i (n_j - δ_ij) L_n^m u^{n-e_i-e_j}.

// B̃_j (j! b_j at a unit vector) for |j| <= O into out[j] (shared memory), by
// the recurrence above (unrolled); each order reads the two before it back
// from out, which holds O(O³) values, more than the registers of a thread.
template <int O>
__device__ __forceinline__ void scaled_taylor_unit(float rx, float ry, float rz, float* out) {
  out[0] = 1.f;
#pragma unroll
  for (int n = 1; n <= O; ++n) {
    const float f1 = float(2 * n - 1) / float(n);
    const float f2 = float(n - 1) / float(n);
#pragma unroll
    for (int a = n; a >= 0; --a)
#pragma unroll
      for (int b = n - a; b >= 0; --b) {
        const int c = n - a - b;
        float s1 = 0.f, s2 = 0.f;
        if (a > 0) s1 += float(a) * rx * out[midx(a - 1, b, c)];
        if (b > 0) s1 += float(b) * ry * out[midx(a, b - 1, c)];
        if (c > 0) s1 += float(c) * rz * out[midx(a, b, c - 1)];
        if (a > 1) s2 += float(a * (a - 1)) * out[midx(a - 2, b, c)];
        if (b > 1) s2 += float(b * (b - 1)) * out[midx(a, b - 2, c)];
        if (c > 1) s2 += float(c * (c - 1)) * out[midx(a, b, c - 2)];
        out[midx(a, b, c)] = f1 * s1 - f2 * s2;
      }
  }
}

// L2P: add the derivatives of the local expansion L (L[m·NQ + n], scaled as
// above) at u = (x - z)/h to dpsi and ddpsi (layouts of m2p_accumulate).  One
// vorticity component at a time (not unrolled), so that only a third of the
// coefficients and sums is live at once.
template <int Q, typename R>
__device__ __forceinline__ void l2p_accumulate(const float* __restrict__ L, R ux, R uy, R uz,
                                               R ih, R (&dpsi)[9], R (&ddpsi)[18]) {
  constexpr int NQ = ncoef(Q);
  R pw[ncoef(Q - 1)];
  monomials<Q - 1, R>(ux, uy, uz, pw);
  const R ih2 = ih * ih;
#pragma unroll 1
  for (int m = 0; m < 3; ++m) {
    const float* Lm = L + m * NQ;
    R p0 = R(0), p1 = R(0), p2 = R(0);
    R q00 = R(0), q01 = R(0), q02 = R(0), q11 = R(0), q12 = R(0), q22 = R(0);
#pragma unroll
    for (int n = 1; n <= Q; ++n)
#pragma unroll
      for (int a = n; a >= 0; --a)
#pragma unroll
        for (int b = n - a; b >= 0; --b) {
          const int c = n - a - b;
          const R l = R(Lm[midx(a, b, c)]);
          if (a > 0) p0 += R(a) * pw[midx(a - 1, b, c)] * l;
          if (b > 0) p1 += R(b) * pw[midx(a, b - 1, c)] * l;
          if (c > 0) p2 += R(c) * pw[midx(a, b, c - 1)] * l;
          if (a > 1) q00 += R(a * (a - 1)) * pw[midx(a - 2, b, c)] * l;
          if (a > 0 && b > 0) q01 += R(a * b) * pw[midx(a - 1, b - 1, c)] * l;
          if (a > 0 && c > 0) q02 += R(a * c) * pw[midx(a - 1, b, c - 1)] * l;
          if (b > 1) q11 += R(b * (b - 1)) * pw[midx(a, b - 2, c)] * l;
          if (b > 0 && c > 0) q12 += R(b * c) * pw[midx(a, b - 1, c - 1)] * l;
          if (c > 1) q22 += R(c * (c - 1)) * pw[midx(a, b, c - 2)] * l;
        }
    // dpsi[3i + m], ddpsi[3s + m] with constant indices in each branch.
    auto put = [&](auto mm) {
      constexpr int M = decltype(mm)::value;
      dpsi[M] += ih * p0; dpsi[3 + M] += ih * p1; dpsi[6 + M] += ih * p2;
      ddpsi[M] += ih2 * q00; ddpsi[3 + M] += ih2 * q01; ddpsi[6 + M] += ih2 * q02;
      ddpsi[9 + M] += ih2 * q11; ddpsi[12 + M] += ih2 * q12; ddpsi[15 + M] += ih2 * q22;
    };
    if (m == 0) put(std::integral_constant<int, 0>());
    else if (m == 1) put(std::integral_constant<int, 1>());
    else put(std::integral_constant<int, 2>());
  }
}

}  // namespace vpm
