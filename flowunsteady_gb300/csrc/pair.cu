// pair.cu — the O(N²) pair passes of the rVPM evaluation on sm_103a.
//
//  PASS_UJ   : U and J = ∇U at every target (FLOWVPM's UJ_direct; formulas in
//              vpm_device.cuh, from FLOWUnsteady docs/src/theory/rvpm.md:88-99).
//  PASS_ZETA : Ω_p = Σ_q ζ_σq(x_p-x_q) Γ_q and V_p = Σ_q ζ_σq(x_p-x_q) S(J_q,Γ_q),
//              from which E_str (rvpm.md:251-262) and the filtered vorticity of
//              the enstrophy monitor (src/FLOWUnsteady_monitors.jl:573-574) follow.
//
// Structure of a CTA (BLOCK threads, T targets per thread, TB = BLOCK·T targets):
//   - each thread holds T targets in registers (register blocking);
//   - the CTA walks its source range in tiles of BLOCK sources: every thread
//     stages one source (FP64 state -> kernel constants, positions relative to
//     the CTA's reference point for FP32C) into shared memory, then every
//     thread runs all BLOCK sources against its T targets, reading each source
//     with broadcast 16-byte shared loads;
//   - FP32C: the FP32 sums of one tile are folded into per-target (hi, lo) FP32
//     pairs with Knuth's TwoSum (kept in shared memory, thread-private slots),
//     so the long sum keeps ~48 bits while the pair arithmetic stays FP32;
//   - the epilogue converts to FP64 and writes final U/J (single source chunk)
//     or raw sums into a partial slot reduced later in fixed order.
// Work items are (target tile, source chunk); grids are sized by the host to
// a whole number of waves, or a persistent grid pulls items from a queue.
#include <type_traits>

#include "internal.h"
#include "vpm_device.cuh"

namespace vpm {

template <typename R>
struct alignas(4 * sizeof(R)) Quad {
  R x, y, z, w;
};

template <int PASS, int PREC>
struct PairTraits {
  using R = typename std::conditional<PREC == VPM_PREC_FP64, double, float>::type;
  static constexpr bool kComp = PREC == VPM_PREC_FP32C;
  static constexpr int kNval = PASS == PASS_UJ ? kNvalUJ : kNvalZeta;
  static constexpr int kQuads = PASS == PASS_UJ ? 2 : 3;   // shared quads per source
};

template <int PASS, int PREC>
__host__ __device__ constexpr size_t smem_bytes(int block, int tpt) {
  using Tr = PairTraits<PASS, PREC>;
  size_t src = size_t(block) * Tr::kQuads * sizeof(Quad<typename Tr::R>);
  size_t fold = Tr::kComp ? size_t(block) * tpt * Tr::kNval * 2 * sizeof(float) : 0;
  return src + fold;
}

// Minimum resident CTAs requested from the compiler: caps the FP32 U/J kernels
// at 128 (T=4) or 96 (T=2) registers per thread.
template <int PASS, int PREC, int BLOCK, int T>
constexpr int min_blocks() {
  return (PASS == PASS_UJ && PREC != VPM_PREC_FP64)
             ? (65536 / (BLOCK * (T >= 4 ? 128 : 96)) > 0 ? 65536 / (BLOCK * (T >= 4 ? 128 : 96)) : 1)
             : 1;
}

// Sources summed in FP32 between two folds into the compensated (hi, lo) pairs.
constexpr int kFoldSources = 256;

template <int PASS, int KERNEL, int PREC, int BLOCK, int T>
__global__ void __launch_bounds__(BLOCK, (min_blocks<PASS, PREC, BLOCK, T>()))
    pair_kernel(const PairArgs a) {
  using Tr = PairTraits<PASS, PREC>;
  using R = typename Tr::R;
  constexpr bool COMP = Tr::kComp;
  constexpr int NV = Tr::kNval;
  constexpr int TB = BLOCK * T;
  constexpr int FOLD_TILES = kFoldSources / BLOCK > 0 ? kFoldSources / BLOCK : 1;
  constexpr bool F32 = sizeof(R) == sizeof(float);

  extern __shared__ __align__(16) unsigned char smem_raw[];
  Quad<R>* tileA = reinterpret_cast<Quad<R>*>(smem_raw);
  Quad<R>* tileB = tileA + BLOCK;
  Quad<R>* tileC = tileB + BLOCK;  // PASS_ZETA only
  float* fold_hi = reinterpret_cast<float*>(smem_raw + size_t(BLOCK) * Tr::kQuads * sizeof(Quad<R>));
  float* fold_lo = fold_hi + size_t(BLOCK) * T * NV;
  __shared__ int s_item;

  const int tid = threadIdx.x;
  const int n_items = a.items ? a.n_items : a.n_tb * a.n_chunk;
  const bool same_arrays = a.xt == a.xs && a.ldt == a.lds;

  int item;
  if (a.counter) {
    if (tid == 0) s_item = int(atomicAdd(a.counter, 1u));
    __syncthreads();
    item = s_item;
  } else {
    item = blockIdx.x;
  }

  while (item < n_items) {
    int64_t t0, t1, s0, s1;
    int slot;
    if (a.items) {
      const PairItem it = a.items[item];
      t0 = it.t0; t1 = it.t1; s0 = it.s0; s1 = it.s1; slot = it.slot;
    } else {
      const int tb = item % a.n_tb, c = item / a.n_tb;
      t0 = a.t_off + int64_t(tb) * TB;
      t1 = min(t0 + TB, a.t_off + a.nt);
      s0 = int64_t(c) * a.chunk;
      s1 = min(s0 + a.chunk, a.ns);
      slot = a.n_chunk > 1 ? c : -1;
    }

    // Reference point of the CTA: its first target (FP32C only).
    double cx = 0.0, cy = 0.0, cz = 0.0;
    if (COMP) {
      cx = a.xt[t0];
      cy = a.xt[a.ldt + t0];
      cz = a.xt[2 * a.ldt + t0];
    }

    R tx[T], ty[T], tz[T];
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const int64_t i = t0 + k * BLOCK + tid;
      if (i < t1) {
        const double px = a.xt[i], py = a.xt[a.ldt + i], pz = a.xt[2 * a.ldt + i];
        tx[k] = R(px - cx); ty[k] = R(py - cy); tz[k] = R(pz - cz);
      } else {
        tx[k] = R(0); ty[k] = R(0); tz[k] = R(0);
      }
    }

    R acc[T][NV];
#pragma unroll
    for (int k = 0; k < T; ++k)
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[k][v] = R(0);
    if (COMP) {
#pragma unroll
      for (int k = 0; k < T; ++k)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          fold_hi[(v * T + k) * BLOCK + tid] = 0.f;
          fold_lo[(v * T + k) * BLOCK + tid] = 0.f;
        }
    }

    int tiles = 0;
    for (int64_t tile0 = s0; tile0 < s1; tile0 += BLOCK) {
      // ---- stage one tile of sources -------------------------------------
      __syncthreads();  // previous tile fully consumed
      {
        const int64_t jj = tile0 + tid;
        Quad<R> qa, qb, qc;
        if (jj < s1) {
          const double px = a.xs[jj], py = a.xs[a.lds + jj], pz = a.xs[2 * a.lds + jj];
          const double sig = a.ss[jj] * a.sigma_scale;
          qa.x = R(px - cx); qa.y = R(py - cy); qa.z = R(pz - cz);
          qb.x = R(a.gs[jj]); qb.y = R(a.gs[a.lds + jj]); qb.z = R(a.gs[2 * a.lds + jj]);
          if (PASS == PASS_UJ) {
            source_consts<KERNEL, R>(sig, qa.w, qb.w);
          } else {
            zeta_consts<KERNEL, R>(sig, qa.w, qb.w);
            if (a.vs) {
              qc.x = R(a.vs[jj]); qc.y = R(a.vs[a.lds + jj]); qc.z = R(a.vs[2 * a.lds + jj]);
            } else {
              qc.x = qc.y = qc.z = R(0);
            }
            qc.w = R(0);
          }
        } else {
          // Padding source: zero strength, unit core, far from everything relevant.
          qa.x = qa.y = qa.z = R(0);
          qb.x = qb.y = qb.z = R(0);
          if (PASS == PASS_UJ) source_consts<KERNEL, R>(1.0, qa.w, qb.w);
          else zeta_consts<KERNEL, R>(1.0, qa.w, qb.w);
          qc.x = qc.y = qc.z = qc.w = R(0);
        }
        tileA[tid] = qa;
        tileB[tid] = qb;
        if (PASS == PASS_ZETA) tileC[tid] = qc;
      }
      __syncthreads();

      // ---- all pairs of the tile ------------------------------------------
      const int cnt = int(min(int64_t(BLOCK), s1 - tile0));
      if constexpr (PASS == PASS_UJ && F32) {
        const float4* ta = reinterpret_cast<const float4*>(tileA);
        const float4* tb = reinterpret_cast<const float4*>(tileB);
        // Coincident pairs can only occur in tiles that overlap the CTA's own
        // targets (or anywhere when the targets are a separate array).
        const bool own = !same_arrays || (tile0 < t1 && tile0 + BLOCK > t0);
        if (KERNEL == VPM_KERNEL_WINCKELMANS && !own) {
#pragma unroll 2
          for (int js = 0; js < cnt; ++js)
            uj_source_winck<T, false>(ta[js], tb[js], tx, ty, tz, acc);
        } else if (KERNEL == VPM_KERNEL_WINCKELMANS) {
#pragma unroll 2
          for (int js = 0; js < cnt; ++js)
            uj_source_winck<T, true>(ta[js], tb[js], tx, ty, tz, acc);
        } else {
#pragma unroll 2
          for (int js = 0; js < cnt; ++js) uj_source_gauss<T>(ta[js], tb[js], tx, ty, tz, acc);
        }
      } else {
#pragma unroll 2
      for (int js = 0; js < cnt; ++js) {
        const Quad<R> sa = tileA[js];
        const Quad<R> sb = tileB[js];
        if constexpr (PASS == PASS_UJ && !F32) {
#pragma unroll
          for (int k = 0; k < T; ++k) {
            const R dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
            const R r2 = dx * dx + dy * dy + dz * dz;
            R q, p;
            pair_qp<KERNEL>(r2, sa.w, sb.w, q, p);
            const R c0 = dy * sb.z - dz * sb.y;
            const R c1 = dz * sb.x - dx * sb.z;
            const R c2 = dx * sb.y - dy * sb.x;
            acc[k][0] += q * c0; acc[k][1] += q * c1; acc[k][2] += q * c2;
            const R p0 = p * c0, p1 = p * c1, p2 = p * c2;
            acc[k][3] += p0 * dx; acc[k][4] += p0 * dy; acc[k][5] += p0 * dz;
            acc[k][6] += p1 * dx; acc[k][7] += p1 * dy; acc[k][8] += p1 * dz;
            acc[k][9] += p2 * dx; acc[k][10] += p2 * dy; acc[k][11] += p2 * dz;
            acc[k][12] += q * sb.x; acc[k][13] += q * sb.y; acc[k][14] += q * sb.z;
          }
        } else {
          const Quad<R> sc = tileC[js];
#pragma unroll
          for (int k = 0; k < T; ++k) {
            const R dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
            const R r2 = dx * dx + dy * dy + dz * dz;
            const R z = pair_zeta<KERNEL>(r2, sa.w, sb.w);
            acc[k][0] += z * sb.x; acc[k][1] += z * sb.y; acc[k][2] += z * sb.z;
            acc[k][3] += z * sc.x; acc[k][4] += z * sc.y; acc[k][5] += z * sc.z;
          }
        }
      }
      }

      if (COMP && (++tiles % FOLD_TILES == 0 || tile0 + BLOCK >= s1)) {
        // Fold the FP32 sums of the last kFoldSources sources into the (hi, lo) pairs.
#pragma unroll
        for (int k = 0; k < T; ++k)
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const int o = (v * T + k) * BLOCK + tid;
            float s, e;
            two_sum(fold_hi[o], float(acc[k][v]), s, e);
            fold_hi[o] = s;
            fold_lo[o] += e;
            acc[k][v] = R(0);
          }
      }
    }

    // ---- epilogue ------------------------------------------------------------
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const int64_t i = t0 + k * BLOCK + tid;
      if (i >= t1) continue;
      double v[NV];
#pragma unroll
      for (int w = 0; w < NV; ++w) {
        if (COMP) {
          const int o = (w * T + k) * BLOCK + tid;
          v[w] = double(fold_hi[o]) + double(fold_lo[o]);
        } else {
          v[w] = double(acc[k][w]);
        }
      }
      // FP32 U/J passes do not accumulate A22 (trace-free pairs): rebuild it.
      if (PASS == PASS_UJ && F32) v[11] = -(v[3] + v[7]);
      if (slot >= 0) {
#pragma unroll
        for (int w = 0; w < NV; ++w) a.part[(int64_t(slot) * NV + w) * a.ldp + i] = v[w];
      } else if (PASS == PASS_UJ) {
        const double s = -kInv4Pi, kp = kp_to_qr<KERNEL>();
        a.u[i] = s * v[0];
        a.u[a.ldo + i] = s * v[1];
        a.u[2 * a.ldo + i] = s * v[2];
        const double w0 = v[12], w1 = v[13], w2 = v[14];
        // J_ab = -(KP·A_ab + ε_abc W_c)/(4π)
        a.j[0 * a.ldo + i] = s * (kp * v[3]);
        a.j[1 * a.ldo + i] = s * (kp * v[4] + w2);
        a.j[2 * a.ldo + i] = s * (kp * v[5] - w1);
        a.j[3 * a.ldo + i] = s * (kp * v[6] - w2);
        a.j[4 * a.ldo + i] = s * (kp * v[7]);
        a.j[5 * a.ldo + i] = s * (kp * v[8] + w0);
        a.j[6 * a.ldo + i] = s * (kp * v[9] + w1);
        a.j[7 * a.ldo + i] = s * (kp * v[10] - w0);
        a.j[8 * a.ldo + i] = s * (kp * v[11]);
      } else {
#pragma unroll
        for (int w = 0; w < NV; ++w) a.u[w * a.ldo + i] = v[w];
      }
    }

    // ---- next item -------------------------------------------------------------
    if (a.counter) {
      __syncthreads();
      if (tid == 0) s_item = int(atomicAdd(a.counter, 1u));
      __syncthreads();
      item = s_item;
    } else {
      item += gridDim.x;
    }
  }
}

template <int PASS, int KERNEL>
__global__ void reduce_kernel(const double* __restrict__ part, int64_t ldp,
                              const int64_t* __restrict__ foff, const int32_t* __restrict__ fchunks,
                              int nfields, int scalar_chunks, int64_t t_begin, int64_t t_end,
                              double* u, double* j, int64_t ldo) {
  constexpr int NV = PASS == PASS_UJ ? kNvalUJ : kNvalZeta;
  const int64_t i = t_begin + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= t_end) return;
  int nc = scalar_chunks;
  if (foff) {
    int lo = 0, hi = nfields - 1;
    while (lo < hi) {  // last field with foff[f] <= i
      const int mid = (lo + hi + 1) >> 1;
      if (foff[mid] <= i) lo = mid; else hi = mid - 1;
    }
    nc = fchunks[lo];
  }
  if (nc <= 1) return;
  double v[NV];
#pragma unroll
  for (int w = 0; w < NV; ++w) v[w] = 0.0;
  for (int c = 0; c < nc; ++c)
#pragma unroll
    for (int w = 0; w < NV; ++w) v[w] += part[(int64_t(c) * NV + w) * ldp + i];
  if (PASS == PASS_UJ) {
    const double s = -kInv4Pi, kp = kp_to_qr<KERNEL>();
    u[i] = s * v[0];
    u[ldo + i] = s * v[1];
    u[2 * ldo + i] = s * v[2];
    j[0 * ldo + i] = s * (kp * v[3]);
    j[1 * ldo + i] = s * (kp * v[4] + v[14]);
    j[2 * ldo + i] = s * (kp * v[5] - v[13]);
    j[3 * ldo + i] = s * (kp * v[6] - v[14]);
    j[4 * ldo + i] = s * (kp * v[7]);
    j[5 * ldo + i] = s * (kp * v[8] + v[12]);
    j[6 * ldo + i] = s * (kp * v[9] + v[13]);
    j[7 * ldo + i] = s * (kp * v[10] - v[12]);
    j[8 * ldo + i] = s * (kp * v[11]);
  } else {
#pragma unroll
    for (int w = 0; w < NV; ++w) u[w * ldo + i] = v[w];
  }
}

// ---------------------------------------------------------------- dispatch --
namespace {

typedef void (*PairFn)(const PairArgs);

template <int PASS, int KERNEL, int PREC, int BLOCK, int T>
PairFn fn_ready() {
  static bool once = [] {
    cudaFuncSetAttribute(pair_kernel<PASS, KERNEL, PREC, BLOCK, T>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(smem_bytes<PASS, PREC>(BLOCK, T)));
    return true;
  }();
  (void)once;
  return pair_kernel<PASS, KERNEL, PREC, BLOCK, T>;
}

// Compiled shapes: FP64 {128x1}; FP32 and FP32C {128x2, 128x4, 256x2}.
template <int PASS, int KERNEL, int PREC>
PairFn pick(Shape s) {
  if constexpr (PREC == VPM_PREC_FP64) {
    if (s.block == 128 && s.tpt == 1) return fn_ready<PASS, KERNEL, PREC, 128, 1>();
    return nullptr;
  } else {
    if (s.block == 128 && s.tpt == 2) return fn_ready<PASS, KERNEL, PREC, 128, 2>();
    if (s.block == 128 && s.tpt == 4) return fn_ready<PASS, KERNEL, PREC, 128, 4>();
    if (s.block == 256 && s.tpt == 2) return fn_ready<PASS, KERNEL, PREC, 256, 2>();
    return nullptr;
  }
}

template <int PASS, int KERNEL>
PairFn pick_prec(int prec, Shape s) {
  switch (prec) {
    case VPM_PREC_FP64: return pick<PASS, KERNEL, VPM_PREC_FP64>(s);
    case VPM_PREC_FP32: return pick<PASS, KERNEL, VPM_PREC_FP32>(s);
    case VPM_PREC_FP32C: return pick<PASS, KERNEL, VPM_PREC_FP32C>(s);
  }
  return nullptr;
}

PairFn pick_all(int pass, int kernel, int prec, Shape s) {
  if (pass == PASS_UJ) {
    return kernel == VPM_KERNEL_WINCKELMANS ? pick_prec<PASS_UJ, VPM_KERNEL_WINCKELMANS>(prec, s)
                                            : pick_prec<PASS_UJ, VPM_KERNEL_GAUSSIANERF>(prec, s);
  }
  return kernel == VPM_KERNEL_WINCKELMANS ? pick_prec<PASS_ZETA, VPM_KERNEL_WINCKELMANS>(prec, s)
                                          : pick_prec<PASS_ZETA, VPM_KERNEL_GAUSSIANERF>(prec, s);
}

}  // namespace

bool pair_shape_supported(int precision, Shape s) {
  if (precision == VPM_PREC_FP64) return s.block == 128 && s.tpt == 1;
  return (s.block == 128 && (s.tpt == 2 || s.tpt == 4)) || (s.block == 256 && s.tpt == 2);
}

size_t pair_smem_bytes(int pass, int precision, Shape s) {
  if (pass == PASS_UJ) {
    switch (precision) {
      case VPM_PREC_FP64: return smem_bytes<PASS_UJ, VPM_PREC_FP64>(s.block, s.tpt);
      case VPM_PREC_FP32: return smem_bytes<PASS_UJ, VPM_PREC_FP32>(s.block, s.tpt);
      default: return smem_bytes<PASS_UJ, VPM_PREC_FP32C>(s.block, s.tpt);
    }
  }
  switch (precision) {
    case VPM_PREC_FP64: return smem_bytes<PASS_ZETA, VPM_PREC_FP64>(s.block, s.tpt);
    case VPM_PREC_FP32: return smem_bytes<PASS_ZETA, VPM_PREC_FP32>(s.block, s.tpt);
    default: return smem_bytes<PASS_ZETA, VPM_PREC_FP32C>(s.block, s.tpt);
  }
}

int pair_ctas_per_sm(int pass, int kernel, int precision, Shape s) {
  PairFn f = pick_all(pass, kernel, precision, s);
  if (!f) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, s.block,
                                                    pair_smem_bytes(pass, precision, s)) !=
      cudaSuccess)
    return 0;
  return n;
}

cudaError_t launch_pair(int pass, int kernel, int precision, Shape s, const PairArgs& a, int grid,
                        cudaStream_t st) {
  PairFn f = pick_all(pass, kernel, precision, s);
  if (!f) return cudaErrorInvalidConfiguration;
  if (grid <= 0) return cudaSuccess;
  f<<<grid, s.block, pair_smem_bytes(pass, precision, s), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_reduce(int pass, int kernel, const double* part, int64_t ldp,
                          const int64_t* foff, const int32_t* fchunks, int nfields,
                          int scalar_chunks, int64_t t_begin, int64_t t_end, double* u,
                          double* j, int64_t ldo, cudaStream_t st) {
  const int64_t n = t_end - t_begin;
  if (n <= 0) return cudaSuccess;
  const int bs = 256;
  const int grid = int((n + bs - 1) / bs);
  if (pass == PASS_UJ) {
    if (kernel == VPM_KERNEL_WINCKELMANS)
      reduce_kernel<PASS_UJ, VPM_KERNEL_WINCKELMANS><<<grid, bs, 0, st>>>(
          part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin, t_end, u, j, ldo);
    else
      reduce_kernel<PASS_UJ, VPM_KERNEL_GAUSSIANERF><<<grid, bs, 0, st>>>(
          part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin, t_end, u, j, ldo);
  } else {
    reduce_kernel<PASS_ZETA, VPM_KERNEL_WINCKELMANS><<<grid, bs, 0, st>>>(
        part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin, t_end, u, j, ldo);
  }
  return cudaGetLastError();
}

}  // namespace vpm
