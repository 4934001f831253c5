// ffv.cu — free-vortex force terms of bound particles (FLOWUnsteady's
// _Ffv_direct, src/FLOWUnsteady_processing_force.jl:879-929) on the GPU.
//
// For every bound particle b and every free particle f with r = |x_f - x_b| > 0
// (kernel evaluated with the bound core σ_b, q = g(r/σ_b)/r³, Δx = x_f - x_b):
//   M[0:3] = Σ_f U_b(x_f) × Γ_f,  U_b(x_f) = -q/(4π) (Δx × Γ_b)
//   M[3:6] = Σ_f q/(4π) Δx × (Γ_b × Γ_f)
// With (Δx × Γ_b) × Γ_f = Γ_b (Δx·Γ_f) - Δx (Γ_b·Γ_f) and
// Δx × (Γ_b × Γ_f) = Γ_b (Δx·Γ_f) - Γ_f (Δx·Γ_b), seven sums per bound particle
// suffice: s = Σ q Δx·Γ_f, v1 = Σ q (Γ_b·Γ_f) Δx, v2 = Σ q (Δx·Γ_b) Γ_f, and
//   M[0:3] = -(Γ_b s - v1)/(4π),   M[3:6] = (Γ_b s - v2)/(4π).
// FP64 throughout (a force evaluation over bound particles).  One thread per
// bound particle; free particles are staged in shared-memory tiles; the free
// range is split into chunks summed afterwards in fixed order.
#include <cuda_runtime.h>

#include "capi_internal.h"

namespace vpm {

constexpr int kFfvBlock = 128;
constexpr int kFfvNval = 7;

template <int KERNEL>
__global__ void __launch_bounds__(kFfvBlock) ffv_kernel(int64_t nb, const double* __restrict__ xb,
                                                        const double* __restrict__ gb,
                                                        const double* __restrict__ sb, int64_t ldb,
                                                        int64_t nf, const double* __restrict__ xf,
                                                        const double* __restrict__ gf, int64_t ldf,
                                                        int64_t chunk, int n_tb, double* part,
                                                        double* M, int64_t ldm, int n_chunk) {
  __shared__ double sx[kFfvBlock], sy[kFfvBlock], sz[kFfvBlock];
  __shared__ double sgx[kFfvBlock], sgy[kFfvBlock], sgz[kFfvBlock];
  const int tid = threadIdx.x;
  const int tb = blockIdx.x % n_tb, c = blockIdx.x / n_tb;
  const int64_t b = int64_t(tb) * kFfvBlock + tid;
  const bool valid = b < nb;
  double bx = 0, by = 0, bz = 0, g0 = 0, g1 = 0, g2 = 0, sig = 1.0;
  if (valid) {
    bx = xb[b]; by = xb[ldb + b]; bz = xb[2 * ldb + b];
    g0 = gb[b]; g1 = gb[ldb + b]; g2 = gb[2 * ldb + b];
    sig = sb[b];
  }
  double ka, kb;
  source_consts<KERNEL, double>(sig, ka, kb);  // constants of the bound core σ_b
  double s = 0, v10 = 0, v11 = 0, v12 = 0, v20 = 0, v21 = 0, v22 = 0;
  const int64_t f0 = int64_t(c) * chunk, f1 = min(f0 + chunk, nf);
  for (int64_t tile0 = f0; tile0 < f1; tile0 += kFfvBlock) {
    __syncthreads();
    const int64_t j = tile0 + tid;
    if (j < f1) {
      sx[tid] = xf[j]; sy[tid] = xf[ldf + j]; sz[tid] = xf[2 * ldf + j];
      sgx[tid] = gf[j]; sgy[tid] = gf[ldf + j]; sgz[tid] = gf[2 * ldf + j];
    } else {
      sx[tid] = bx; sy[tid] = by; sz[tid] = bz;   // r = 0: skipped
      sgx[tid] = sgy[tid] = sgz[tid] = 0.0;
    }
    __syncthreads();
    const int cnt = int(min(int64_t(kFfvBlock), f1 - tile0));
    for (int js = 0; js < cnt; ++js) {
      const double dx = sx[js] - bx, dy = sy[js] - by, dz = sz[js] - bz;
      const double r2 = dx * dx + dy * dy + dz * dz;
      double q, p;
      pair_qp<KERNEL>(r2, ka, kb, q, p);   // q = 0 at r = 0
      const double fx = sgx[js], fy = sgy[js], fz = sgz[js];
      const double dgf = dx * fx + dy * fy + dz * fz;
      const double ggf = g0 * fx + g1 * fy + g2 * fz;
      const double dgb = dx * g0 + dy * g1 + dz * g2;
      s += q * dgf;
      const double qa = q * ggf, qb = q * dgb;
      v10 += qa * dx; v11 += qa * dy; v12 += qa * dz;
      v20 += qb * fx; v21 += qb * fy; v22 += qb * fz;
    }
  }
  if (!valid) return;
  if (n_chunk > 1) {
    const double v[kFfvNval] = {s, v10, v11, v12, v20, v21, v22};
    for (int k = 0; k < kFfvNval; ++k) part[(int64_t(c) * kFfvNval + k) * nb + b] = v[k];
    return;
  }
  const double w = kInv4Pi;
  M[b] = -w * (g0 * s - v10);
  M[ldm + b] = -w * (g1 * s - v11);
  M[2 * ldm + b] = -w * (g2 * s - v12);
  M[3 * ldm + b] = w * (g0 * s - v20);
  M[4 * ldm + b] = w * (g1 * s - v21);
  M[5 * ldm + b] = w * (g2 * s - v22);
}

__global__ void ffv_reduce_kernel(int64_t nb, const double* __restrict__ gb, int64_t ldb,
                                  const double* __restrict__ part, int n_chunk, double* M,
                                  int64_t ldm) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  double v[kFfvNval] = {0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < n_chunk; ++c)
    for (int k = 0; k < kFfvNval; ++k) v[k] += part[(int64_t(c) * kFfvNval + k) * nb + b];
  const double g0 = gb[b], g1 = gb[ldb + b], g2 = gb[2 * ldb + b], w = kInv4Pi;
  M[b] = -w * (g0 * v[0] - v[1]);
  M[ldm + b] = -w * (g1 * v[0] - v[2]);
  M[2 * ldm + b] = -w * (g2 * v[0] - v[3]);
  M[3 * ldm + b] = w * (g0 * v[0] - v[4]);
  M[4 * ldm + b] = w * (g1 * v[0] - v[5]);
  M[5 * ldm + b] = w * (g2 * v[0] - v[6]);
}

// Scratch (elements) an FFV launch of nb bound and nf free particles needs.
size_t ffv_plan(int64_t nb, int64_t nf, int num_sms, int64_t* chunk, int* n_chunk) {
  const int64_t n_tb = ceil_div(std::max<int64_t>(nb, 1), kFfvBlock);
  *n_chunk = plan_chunks(n_tb, nf, kFfvBlock, 8 * num_sms, chunk);
  return *n_chunk > 1 ? size_t(*n_chunk) * kFfvNval * size_t(nb) : 0;
}

cudaError_t launch_ffv(int kernel, int64_t nb, const double* xb, const double* gb,
                       const double* sb, int64_t ldb, int64_t nf, const double* xf,
                       const double* gf, int64_t ldf, double* part, double* M, int64_t ldm,
                       int num_sms, cudaStream_t st) {
  if (nb <= 0) return cudaSuccess;
  int64_t chunk = 0;
  int n_chunk = 1;
  ffv_plan(nb, nf, num_sms, &chunk, &n_chunk);
  const int n_tb = int(ceil_div(nb, kFfvBlock));
  const int grid = n_tb * n_chunk;
  if (kernel == VPM_KERNEL_WINCKELMANS)
    ffv_kernel<VPM_KERNEL_WINCKELMANS><<<grid, kFfvBlock, 0, st>>>(
        nb, xb, gb, sb, ldb, nf, xf, gf, ldf, chunk, n_tb, part, M, ldm, n_chunk);
  else
    ffv_kernel<VPM_KERNEL_GAUSSIANERF><<<grid, kFfvBlock, 0, st>>>(
        nb, xb, gb, sb, ldb, nf, xf, gf, ldf, chunk, n_tb, part, M, ldm, n_chunk);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || n_chunk <= 1) return e;
  ffv_reduce_kernel<<<int(ceil_div(nb, 256)), 256, 0, st>>>(nb, gb, ldb, part, n_chunk, M, ldm);
  return cudaGetLastError();
}

}  // namespace vpm
