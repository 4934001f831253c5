// pair.cu — instantiates the U/∇U and ζ pair passes (the kernel template is in
// pair_kernel.cuh) and dispatches every pass; the α-derivative passes are
// compiled in pair_d.cu.
#include "pair_kernel.cuh"

namespace vpm {

bool pair_shape_supported(int precision, Shape s) {
  if (precision == VPM_PREC_FP64) return s.block == 128 && s.tpt == 1;
  return (s.block == 128 && (s.tpt == 2 || s.tpt == 4)) || (s.block == 256 && s.tpt == 2);
}

size_t pair_smem_bytes(int pass, int precision, Shape s) {
  if (pass == PASS_UJ) return smem_of<PASS_UJ>(precision, s);
  if (pass == PASS_ZETA) return smem_of<PASS_ZETA>(precision, s);
  return pair_smem_bytes_d(pass, precision, s);
}

int pair_ctas_per_sm(int pass, int kernel, int precision, Shape s) {
  if (pass == PASS_UJ) return ctas_per_sm<PASS_UJ>(kernel, precision, s);
  if (pass == PASS_ZETA) return ctas_per_sm<PASS_ZETA>(kernel, precision, s);
  return pair_ctas_per_sm_d(pass, kernel, precision, s);
}

int pair_max_active_clusters(int pass, int kernel, int precision, Shape s, int cluster) {
  if (pass == PASS_UJ) return max_active_clusters<PASS_UJ>(kernel, precision, s, cluster);
  if (pass == PASS_ZETA) return max_active_clusters<PASS_ZETA>(kernel, precision, s, cluster);
  return pair_max_active_clusters_d(pass, kernel, precision, s, cluster);
}

cudaError_t launch_pair(int pass, int kernel, int precision, Shape s, const PairArgs& a, int grid,
                        cudaStream_t st) {
  if (pass == PASS_UJ) return launch<PASS_UJ>(kernel, precision, s, a, grid, st);
  if (pass == PASS_ZETA) return launch<PASS_ZETA>(kernel, precision, s, a, grid, st);
  return launch_pair_d(pass, kernel, precision, s, a, grid, st);
}

// Packed source records of the FP32 U/J passes, per source
//   (xh, yh, zh, a), (xl, yl, zl, b), (Γx, Γy, Γz, 0)
// with x ≈ xh + xl (split_f32) and (a, b) the kernel constants of σ·scale.
// Gaussian-erf: each warp (32 consecutive particles) also adds one to
// *compact when its bounding box is compact against the far radius (diagonal
// exponent argument >= kVoteSpan·kArgFar), the measure by which the pair
// kernels decide whether the far-field classification can pay.
template <int KERNEL>
__global__ void __launch_bounds__(256) pack_sources_kernel(int64_t n, const double* __restrict__ X,
                                                           const double* __restrict__ G,
                                                           const double* __restrict__ S, int64_t ld,
                                                           double scale, float4* __restrict__ rec,
                                                           unsigned int* compact) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  float xh = 0.f, xl, yh = 0.f, yl, zh = 0.f, zl, ka = -INFINITY, kb;
  if (valid) {
    split_f32(X[i], xh, xl);
    split_f32(X[ld + i], yh, yl);
    split_f32(X[2 * ld + i], zh, zl);
    source_consts<KERNEL, float>(S[i] * scale, ka, kb);
    rec[3 * i] = make_float4(xh, yh, zh, ka);
    rec[3 * i + 1] = make_float4(xl, yl, zl, kb);
    rec[3 * i + 2] = make_float4(float(G[i]), float(G[ld + i]), float(G[2 * ld + i]), 0.f);
  }
  if (KERNEL == VPM_KERNEL_GAUSSIANERF && compact) {
    if (__all_sync(0xffffffffu, !valid)) return;
    float4 box[2];
    warp_source_box(xh, yh, zh, ka, valid, box);
    if ((threadIdx.x & 31) == 0) {
      const float ex = box[1].x - box[0].x, ey = box[1].y - box[0].y, ez = box[1].z - box[0].z;
      const float span = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) * box[0].w;
      if (span >= kVoteSpan * kArgFar) atomicAdd(compact, 1u);
    }
  }
}

// Packed source records of the FP32 ζ passes, per source
//   (xh, yh, zh, a), (xl, yl, zl, b), (Γx, Γy, Γz, c), (v_q, 0) [, (w_q, 0)]
// with (a, b, c) the ζ constants of σ·scale (zeta_consts_f32) and v_q, w_q
// from the rows V, W (zero when V is null).  Staging these instead of the FP64
// rows keeps FP64 arithmetic (differences, the constants' divisions, and for
// Winckelmans a pow) out of the pair kernels, where every CTA would repeat it
// for every source it stages.
template <int KERNEL, bool D>
__global__ void __launch_bounds__(256) pack_zeta_sources_kernel(
    int64_t n, const double* __restrict__ X, const double* __restrict__ G,
    const double* __restrict__ S, const double* __restrict__ V, const double* __restrict__ W,
    int64_t ld, double scale, float4* __restrict__ rec) {
  constexpr int Q = D ? 5 : 4;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float xh, xl, yh, yl, zh, zl, ka, kb, kc;
  split_f32(X[i], xh, xl);
  split_f32(X[ld + i], yh, yl);
  split_f32(X[2 * ld + i], zh, zl);
  zeta_consts_f32<KERNEL>(S[i] * scale, ka, kb, kc);
  float4* r = rec + Q * i;
  r[0] = make_float4(xh, yh, zh, ka);
  r[1] = make_float4(xl, yl, zl, kb);
  r[2] = make_float4(float(G[i]), float(G[ld + i]), float(G[2 * ld + i]), kc);
  r[3] = V ? make_float4(float(V[i]), float(V[ld + i]), float(V[2 * ld + i]), 0.f)
           : make_float4(0.f, 0.f, 0.f, 0.f);
  if (D)
    r[Q - 1] = W ? make_float4(float(W[i]), float(W[ld + i]), float(W[2 * ld + i]), 0.f)
                 : make_float4(0.f, 0.f, 0.f, 0.f);
}

cudaError_t launch_pack_zeta_sources(int kernel, bool d, int64_t n, const double* X,
                                     const double* G, const double* S, const double* V,
                                     const double* W, int64_t ld, double scale, float4* rec,
                                     cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int grid = int((n + 255) / 256);
  auto go = [&](auto kern) { kern<<<grid, 256, 0, st>>>(n, X, G, S, V, W, ld, scale, rec); };
  if (kernel == VPM_KERNEL_WINCKELMANS) {
    if (d) go(pack_zeta_sources_kernel<VPM_KERNEL_WINCKELMANS, true>);
    else go(pack_zeta_sources_kernel<VPM_KERNEL_WINCKELMANS, false>);
  } else {
    if (d) go(pack_zeta_sources_kernel<VPM_KERNEL_GAUSSIANERF, true>);
    else go(pack_zeta_sources_kernel<VPM_KERNEL_GAUSSIANERF, false>);
  }
  return cudaGetLastError();
}

cudaError_t launch_pack_sources(int kernel, int64_t n, const double* X, const double* G,
                                const double* S, int64_t ld, double scale, float4* rec,
                                unsigned int* compact, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int grid = int((n + 255) / 256);
  if (compact) {
    cudaError_t e = cudaMemsetAsync(compact, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
  }
  if (kernel == VPM_KERNEL_WINCKELMANS)
    pack_sources_kernel<VPM_KERNEL_WINCKELMANS><<<grid, 256, 0, st>>>(n, X, G, S, ld, scale, rec,
                                                                      compact);
  else
    pack_sources_kernel<VPM_KERNEL_GAUSSIANERF><<<grid, 256, 0, st>>>(n, X, G, S, ld, scale, rec,
                                                                      compact);
  return cudaGetLastError();
}

cudaError_t launch_reduce(int pass, int kernel, int precision, const double* part, int64_t ldp,
                          const int64_t* foff, const int32_t* fchunks, int nfields,
                          int scalar_chunks, int64_t t_begin, int64_t t_end, double* u,
                          double* j, double* dj, int64_t ldo, cudaStream_t st) {
  if (pass == PASS_UJ)
    return reduce<PASS_UJ>(kernel, precision, part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin,
                           t_end, u, j, dj, ldo, st);
  if (pass == PASS_ZETA)
    return reduce<PASS_ZETA>(kernel, precision, part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin,
                             t_end, u, j, dj, ldo, st);
  return launch_reduce_d(pass, kernel, precision, part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin,
                         t_end, u, j, dj, ldo, st);
}

}  // namespace vpm
