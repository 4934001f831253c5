// pair_kernel.cuh — the O(N²) pair-pass kernel template of the rVPM evaluation
// on sm_103a, instantiated by pair.cu (PASS_UJ, PASS_ZETA) and pair_d.cu
// (PASS_UJD, PASS_ZETAD).
//
//  PASS_UJ    : U and J = ∇U at every target (FLOWVPM's UJ_direct; formulas in
//               vpm_device.cuh, from FLOWUnsteady docs/src/theory/rvpm.md:88-99).
//  PASS_ZETA  : Ω_p = Σ_q ζ_σq(x_p-x_q) Γ_q and V_p = Σ_q ζ_σq(x_p-x_q) S(J_q,Γ_q),
//               from which E_str (rvpm.md:251-262) and the filtered vorticity of
//               the enstrophy monitor (src/FLOWUnsteady_monitors.jl:573-574) follow.
//  PASS_UJD   : PASS_UJ plus DJ = dJ/dα (every core size scaled by α, at α = 1).
//  PASS_ZETAD : PASS_ZETA plus DΩ = Σ Dζ Γ_q and DV = Σ (Dζ v_q + ζ w_q), w_q = S(DJ_q,Γ_q).
//  The D passes serve the analytic form of the dynamic SFS procedure
//  (rvpm.md:264-294), which needs ∂/∂σ of the stretching and of E_str.
//
// Structure of a CTA (BLOCK threads, T targets per thread, TB = BLOCK·T targets):
//   - each thread holds T targets in registers (register blocking);
//   - the CTA walks its source range in tiles of BLOCK sources: every thread
//     stages one source (FP64 state -> kernel constants, positions relative to
//     the CTA's reference point for FP32C) into shared memory, then every
//     thread runs all BLOCK sources against its T targets, reading each source
//     with broadcast 16-byte shared loads;
//   - FP32C: the FP32 sums of kFoldSources sources are folded into per-target
//     (hi, lo) FP32 pairs with Knuth's TwoSum (kept in shared memory,
//     thread-private slots), so the long sum keeps ~48 bits while the pair
//     arithmetic stays FP32;
//   - the epilogue converts to FP64 and writes final values (single source
//     chunk) or raw sums into a partial slot, which a reduction launch sums in
//     fixed chunk order, or (the fused form) the last CTA of the target tile
//     does, in the same order.
// Work items are (target tile, source chunk); grids are sized by the host to
// a whole number of waves, or a persistent grid pulls items from a queue.
#pragma once

#include <cstring>
#include <type_traits>

#include "internal.h"
#include "update.h"
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
  static constexpr int kNval = nval_of(PASS);
  static constexpr bool kUJ = PASS == PASS_UJ || PASS == PASS_UJD;
  static constexpr bool kD = PASS == PASS_UJD || PASS == PASS_ZETAD;
  // shared quads per source: (x, a), (Γ, b), and for ζ passes v_q (and w_q)
  static constexpr int kQuads = kUJ ? 2 : (PASS == PASS_ZETA ? 3 : 4);
  // The FP32 passes read packed source records (pack_sources_kernel for U/J,
  // pack_zeta_sources_kernel for ζ); the plain U/J pass stages them with bulk
  // copies.
  static constexpr bool kRec = PREC != VPM_PREC_FP64;
  static constexpr bool kTma = PASS == PASS_UJ && PREC != VPM_PREC_FP64;
  // float4 per source record: U/J 3, ζ 4 (+ v_q), ζ + α-derivative 5 (+ w_q).
  static constexpr int kRecQuads = kUJ ? 3 : (PASS == PASS_ZETA ? 4 : 5);
  static constexpr int kRecBytes = 16 * kRecQuads;
};

// Shared memory: source quads, then (FP32) the far-field boxes (per warp two
// float4 for its staged sources and two for its targets), then (FP32C) the
// fold pairs, then (bulk copies) the staging records and the mbarrier.
template <int PASS, int PREC>
__host__ __device__ constexpr size_t box_bytes(int block) {
  return PREC == VPM_PREC_FP64 ? 0 : size_t(block / 32) * 4 * 16;
}

template <int PASS, int PREC>
__host__ __device__ constexpr size_t smem_bytes(int block, int tpt) {
  using Tr = PairTraits<PASS, PREC>;
  size_t src = size_t(block) * Tr::kQuads * sizeof(Quad<typename Tr::R>);
  size_t fold = Tr::kComp ? size_t(block) * tpt * Tr::kNval * 2 * sizeof(float) : 0;
  size_t stage = Tr::kTma ? size_t(block) * Tr::kRecBytes + 16 : 0;
  return src + box_bytes<PASS, PREC>(block) + fold + stage;
}

// Minimum resident CTAs requested from the compiler: caps the FP32 U/J kernels
// at 168 (T=4) or 96 (T=2) registers per thread (the D form: 255 and 168).
// With T=4 the fold pairs in shared memory (61 KB per 128-thread CTA) allow
// no more than 3 CTAs per SM either.
template <int PASS, int PREC, int BLOCK, int T>
constexpr int min_blocks() {
  constexpr int regs = PASS == PASS_UJD ? (T >= 4 ? 255 : 168) : (T >= 4 ? 168 : 96);
  return (PairTraits<PASS, PREC>::kUJ && PREC != VPM_PREC_FP64)
             ? (65536 / (BLOCK * regs) > 0 ? 65536 / (BLOCK * regs) : 1)
             : 1;
}

// Sources summed in FP32 between two folds into the compensated (hi, lo) pairs.
constexpr int kFoldSources = 256;

// J_ab = -(KP·A_ab + ε_abc W_c)/(4π) from 12 raw sums (A 9 then W 3) at v.
// The products and sums are fused explicitly, so that every kernel that forms
// final values (pass epilogue, reduction launch, fused reduction) rounds them
// the same way, whatever the compiler would contract in each.
template <int KERNEL>
__device__ inline void write_jacobian(const double* v, double* out, int64_t ld, int64_t i) {
  const double s = -kInv4Pi, kp = kp_to_qr<KERNEL>();
  const double w0 = v[9], w1 = v[10], w2 = v[11];
  out[0 * ld + i] = s * (kp * v[0]);
  out[1 * ld + i] = s * __fma_rn(kp, v[1], w2);
  out[2 * ld + i] = s * __fma_rn(kp, v[2], -w1);
  out[3 * ld + i] = s * __fma_rn(kp, v[3], -w2);
  out[4 * ld + i] = s * (kp * v[4]);
  out[5 * ld + i] = s * __fma_rn(kp, v[5], w0);
  out[6 * ld + i] = s * __fma_rn(kp, v[6], w1);
  out[7 * ld + i] = s * __fma_rn(kp, v[7], -w0);
  out[8 * ld + i] = s * (kp * v[8]);
}

// Final values of one target from its NV raw sums.
template <int PASS, int KERNEL>
__device__ inline void write_final(const double* v, const PairArgs& a, int64_t i) {
  if constexpr (PASS == PASS_UJ || PASS == PASS_UJD) {
    const double s = -kInv4Pi;
    a.u[i] = s * v[0];
    a.u[a.ldo + i] = s * v[1];
    a.u[2 * a.ldo + i] = s * v[2];
    write_jacobian<KERNEL>(v + 3, a.j, a.ldo, i);
    if constexpr (PASS == PASS_UJD) write_jacobian<KERNEL>(v + 15, a.dj, a.ldo, i);
  } else {
    constexpr int NV = nval_of(PASS);
#pragma unroll
    for (int w = 0; w < NV; ++w) a.u[w * a.ldo + i] = v[w];
  }
}

// Partial slots of the FP32 passes hold a chunk's raw FP32 sums as a float
// pair (hi, lo) in the 8 bytes of a slot element: the fold pair (FP32C) or
// (sum, 0) (FP32).  The chunks are summed in chunk order as a double-float
// (s, c): s + hi by Knuth's TwoSum, its error and lo into c, all FP32
// additions on the FMA pipe; the value is s + c in FP64.  (GB300 retires about
// two FP64 additions per SM and cycle, which bounded the FP64 form of this sum
// at small N: 21 µs for the 60 chunks of a U/J pass at N = 7,600.)  One chunk
// gives hi + lo exactly, as the pass epilogue does without slots.
struct PairSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float2 x) {
    const float t = __fadd_rn(s, x.x);
    const float bp = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x.x, bp));
    c = __fadd_rn(c, __fadd_rn(e, x.y));
    s = t;
  }
  __device__ __forceinline__ double value() const { return double(s) + double(c); }
};

// FP32 U/J passes: the Gaussian-erf A sums carry a scale, and A22 (DA22) is not
// accumulated (the pairs are trace-free); both are applied to the FP64 sums.
template <int PASS, int KERNEL>
__device__ __forceinline__ void finish_f32_sums(double* v) {
  if constexpr (PASS == PASS_UJ || PASS == PASS_UJD) {
    if constexpr (KERNEL == VPM_KERNEL_GAUSSIANERF) {
#pragma unroll
      for (int w = 3; w < 11; ++w) v[w] *= kGaussAScale;
    }
    v[11] = -(v[3] + v[7]);
    if constexpr (PASS == PASS_UJD) v[23] = -(v[15] + v[19]);
  }
}

// Cluster form of the epilogue (FP32C): after every rank's (hi, lo) pairs are
// final, rank r forms the values of the targets [r·per, (r+1)·per) of the
// tile from every rank's pairs, in rank order, as FP64 sums of each rank's
// hi + lo (the partial-slot form sums the same pairs as a double-float).
template <int PASS, int KERNEL, int PREC, int BLOCK, int T>
__device__ __forceinline__ void cluster_epilogue(const PairArgs& a, const float* fold_hi,
                                              const float* fold_lo, int64_t t0, int64_t t1) {
  using Tr = PairTraits<PASS, PREC>;
  constexpr int NV = Tr::kNval;
  constexpr int TB = BLOCK * T;
  const int tid = threadIdx.x;
  const uint32_t nc = uint32_t(a.cluster), rank = cluster_ctarank();
  const int per = (TB + int(nc) - 1) / int(nc);
  const int tend = min(TB, int(rank + 1) * per);
  for (int t = int(rank) * per + tid; t < tend; t += BLOCK) {
    const int64_t i = t0 + t;
    if (i >= t1) break;
    const int k = t / BLOCK, j = t % BLOCK;
    // Rank q's value w, as the partial-slot epilogue forms it.
    auto rank_value = [&](int w, uint32_t q) {
      const int o = (w * T + k) * BLOCK + j;
      double u = double(ld_cluster_f32(fold_hi + o, q)) + double(ld_cluster_f32(fold_lo + o, q));
      if (Tr::kUJ && KERNEL == VPM_KERNEL_GAUSSIANERF && w >= 3 && w < 11) u *= kGaussAScale;
      return u;
    };
    double v[NV];
#pragma unroll
    for (int w = 0; w < NV; ++w) {
      double sum = 0.0;
      for (uint32_t q = 0; q < nc; ++q) {
        // U/J: the trace-free A22 (and DA22) rebuilt per rank.
        if (Tr::kUJ && w == 11) sum += -(rank_value(3, q) + rank_value(7, q));
        else if (PASS == PASS_UJD && w == 23) sum += -(rank_value(15, q) + rank_value(19, q));
        else sum += rank_value(w, q);
      }
      v[w] = sum;
    }
    write_final<PASS, KERNEL>(v, a, i);
  }
}

// Chunk of the j-th item of a tile in the fused form: the chunk cs that holds
// the tile's own particles (targets and sources share an order) first, then
// outwards, alternating sides: cs, cs-1, cs+1, cs-2, ... (a permutation of
// [0, n)).  The near chunks are the costly ones (close pairs take the general
// form), so each tile's items end close together and its partial sums wait in
// L2 for a shorter time.
__device__ __forceinline__ int near_first_chunk(int j, int cs, int n) {
  const int m = min(cs, n - 1 - cs);
  if (j <= 2 * m) {
    const int d = (j + 1) >> 1;
    return (j & 1) ? cs - d : cs + d;
  }
  const int k = j - 2 * m;
  return cs > m ? cs - m - k : cs + m + k;
}

// Fused form of the reduction, run by the last CTA of target tile [t0, t1) to
// finish: the tile's partial slots summed in chunk order from L2 (the same FP64
// additions in the same order as reduce_kernel), the final values written, and
// the summed lines that hold only this tile's targets dropped from L2 without
// a write-back.
template <int PASS, int KERNEL, int BLOCK, int T, bool F2>
__device__ __noinline__ void tile_reduce(const PairArgs& a, int64_t t0, int64_t t1) {
  constexpr int NV = nval_of(PASS);
  // Values summed side by side: 2G loads in flight per thread, in few enough
  // registers that the summation adds little to the kernel's count.
  constexpr int G = 4;
  const int tid = threadIdx.x;
  const int64_t step = int64_t(NV) * a.ldp;
#pragma unroll 1
  for (int k = 0; k < T; ++k) {
    const int64_t i = t0 + k * BLOCK + tid;
    if (i >= t1) break;
    double v[NV];
#pragma unroll
    for (int w0 = 0; w0 < NV; w0 += G) {
      if constexpr (F2) {
        PairSum s[G];
        const float2* p = reinterpret_cast<const float2*>(a.part) + int64_t(w0) * a.ldp + i;
#pragma unroll 2
        for (int c = 0; c < a.n_chunk; ++c, p += step) {
#pragma unroll
          for (int g = 0; g < G; ++g)
            if (w0 + g < NV) s[g].add(__ldcg(p + int64_t(g) * a.ldp));
        }
#pragma unroll
        for (int g = 0; g < G; ++g)
          if (w0 + g < NV) v[w0 + g] = s[g].value();
      } else {
        double s[G];
#pragma unroll
        for (int g = 0; g < G; ++g) s[g] = 0.0;
        const double* p = a.part + int64_t(w0) * a.ldp + i;
#pragma unroll 2
        for (int c = 0; c < a.n_chunk; ++c, p += step) {
#pragma unroll
          for (int g = 0; g < G; ++g)
            if (w0 + g < NV) s[g] += __ldcg(p + int64_t(g) * a.ldp);
        }
#pragma unroll
        for (int g = 0; g < G; ++g)
          if (w0 + g < NV) v[w0 + g] = s[g];
      }
    }
    if constexpr (F2) finish_f32_sums<PASS, KERNEL>(v);
    write_final<PASS, KERNEL>(v, a, i);
  }
  __syncthreads();   // every read of the tile's slots is done
  // Row r = slot * NV + w holds the tile's targets at bytes [s, e); only the
  // 128-byte lines inside that range are dropped.
  constexpr int kLines = (BLOCK * T * 8) / 128 + 1;
  const int rows = a.n_chunk * NV;
  for (int idx = tid; idx < rows * kLines; idx += BLOCK) {
    const int r = idx / kLines, l = idx - r * kLines;
    const uintptr_t s = reinterpret_cast<uintptr_t>(a.part + int64_t(r) * a.ldp + t0);
    const uintptr_t e = s + uintptr_t(t1 - t0) * sizeof(double);
    const uintptr_t line = ((s + 127) & ~uintptr_t(127)) + uintptr_t(l) * 128;
    if (line + 128 <= e) discard_l2_line(reinterpret_cast<const void*>(line));
  }
}

// CLU: the split-source cluster form (FP32C only; launched with a cluster
// dimension of a.cluster CTAs, one item per CTA).
template <int PASS, int KERNEL, int PREC, int BLOCK, int T, bool CLU = false>
__global__ void __launch_bounds__(BLOCK, (min_blocks<PASS, PREC, BLOCK, T>()))
    pair_kernel(const PairArgs a) {
  static_assert(!CLU || PREC == VPM_PREC_FP32C, "the cluster form sums compensated pairs");
  using Tr = PairTraits<PASS, PREC>;
  using R = typename Tr::R;
  constexpr bool COMP = Tr::kComp;
  constexpr int NV = Tr::kNval;
  constexpr int TB = BLOCK * T;
  constexpr int FOLD_TILES = kFoldSources / BLOCK > 0 ? kFoldSources / BLOCK : 1;
  constexpr bool F32 = sizeof(R) == sizeof(float);

  extern __shared__ __align__(16) unsigned char smem_raw[];
  // Source quads: A (x, a) and B (Γ, b) for BLOCK sources, then for ζ passes
  // C (v_q) and for PASS_ZETAD D (w_q).
  Quad<R>* tileA = reinterpret_cast<Quad<R>*>(smem_raw);
  Quad<R>* tileB = tileA + BLOCK;
  Quad<R>* tileC = tileB + BLOCK;
  Quad<R>* tileD = tileC + BLOCK;
  constexpr size_t kQuadBytes = size_t(BLOCK) * Tr::kQuads * sizeof(Quad<R>);
  constexpr size_t kBoxBytes = box_bytes<PASS, PREC>(BLOCK);
  // Far-field boxes of warp w: its staged sources at sbox[2w + 0..1], its
  // targets at tbox[2w + 0..1].
  float4* sbox = reinterpret_cast<float4*>(smem_raw + kQuadBytes);
  float4* tbox = sbox + 2 * (BLOCK / 32);
  float* fold_hi = reinterpret_cast<float*>(smem_raw + kQuadBytes + kBoxBytes);
  float* fold_lo = fold_hi + size_t(BLOCK) * T * NV;
  // Bulk-copy staging: the records of BLOCK sources, then the mbarrier.
  float4* stage = reinterpret_cast<float4*>(smem_raw + kQuadBytes + kBoxBytes +
                                            (COMP ? size_t(BLOCK) * T * NV * 2 * sizeof(float) : 0));
  uint64_t* bar = reinterpret_cast<uint64_t*>(stage + size_t(BLOCK) * 3);
  __shared__ int s_item;
  __shared__ int s_last;

  const int tid = threadIdx.x;
  const int n_items = a.items ? a.n_items : a.n_tb * a.n_chunk;
  // Packed records replace the FP64 source reads (and their conversion) when
  // the host provides them; bulk copies need them.
  const bool use_rec = Tr::kRec && a.rec != nullptr;
  const bool use_tma = Tr::kTma && use_rec && a.tma != 0;
  // The targets are the sources (same rows): their records hold their split.
  const bool tgt_rec = use_rec && a.xt == a.xs && a.ldt == a.lds;
  // Gaussian-erf FP32 passes classify (warp, 32 sources) blocks by distance.
  constexpr bool kFarKernel = F32 && KERNEL == VPM_KERNEL_GAUSSIANERF;
  const bool use_far =
      kFarKernel && a.far != 0 && (!a.coh || 4 * uint64_t(*a.coh) >= uint64_t(a.coh_blocks));
  const int warp = tid >> 5;
  uint32_t phase = 0;
  if (use_tma) {
    if (tid == 0) mbar_init(bar, 1);
    __syncthreads();
  }
  // One bulk copy of the records of the source tile [tile, tile + cnt): 48·cnt
  // bytes from a 16-byte aligned address (48-byte records, aligned base).
  auto issue = [&](int64_t tile, int64_t send) {
    const int cnt = int(min(int64_t(BLOCK), send - tile));
    const uint32_t bytes = uint32_t(cnt) * uint32_t(Tr::kRecBytes);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, bytes);
    bulk_g2s(stage, a.rec + 3 * tile, bytes, bar);
  };

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
      // Clusters: consecutive CTAs share a target tile, cluster rank = chunk.
      // The fused reduction runs the chunks of a tile as consecutive items,
      // so that their partial sums are still in L2 when the last one sums
      // them; otherwise the items are chunk-major.
      const bool tile_major = CLU || a.tile_done;
      const int per = CLU ? a.cluster : a.n_chunk;
      const int tb = tile_major ? item / per : item % a.n_tb;
      int c = tile_major ? item % per : item / a.n_tb;
      t0 = a.t_off + int64_t(tb) * TB;
      // Split sources: the j-th item of a tile takes its j-th chunk counted from
      // the tile's own, outwards (near_first_chunk).  Gaussian-erf chunk-major
      // items so go in rounds from every tile's costly near chunks (general
      // form) to the cheap far ones, the order in which the block scheduler
      // balances them best: at N = 7,600 the U/J pass 0.136 -> 0.124 ms, at
      // 65,536 5.10 -> 4.94 ms.  Winckelmans pairs cost the same near and far
      // (65,536: 5.18 -> 5.25 ms), so its chunk-major items keep their order.
      // The slots keep their chunk index, so the sums are unchanged.
      if (!CLU && a.n_chunk > 1 && (a.tile_done || KERNEL == VPM_KERNEL_GAUSSIANERF))
        c = near_first_chunk(c, min(int(t0 / a.chunk), a.n_chunk - 1), a.n_chunk);
      t1 = min(t0 + TB, a.t_off + a.nt);
      s0 = int64_t(c) * a.chunk;
      s1 = min(s0 + a.chunk, a.ns);
      slot = (a.n_chunk > 1 && !CLU) ? c : -1;
    }

    // Reference point of the CTA: its first target (FP32C only).
    double cx = 0.0, cy = 0.0, cz = 0.0;
    // With records, relative positions come from the (hi, lo) float split of
    // both ends, (h - ch) + (l - cl), for targets and sources alike, so that
    // coincident particles stay exactly coincident.  Targets that are the
    // sources themselves take their split from the records, which hold the
    // same split_f32 pairs: no FP64 work per target (GB300's FP64 pipe
    // retires about two operations per SM and cycle, and every work item
    // loads its targets anew).
    float chx = 0.f, chy = 0.f, chz = 0.f, clx = 0.f, cly = 0.f, clz = 0.f;
    if (COMP) {
      if (tgt_rec) {
        const float4 r0 = a.rec[Tr::kRecQuads * t0], r1 = a.rec[Tr::kRecQuads * t0 + 1];
        chx = r0.x; chy = r0.y; chz = r0.z;
        clx = r1.x; cly = r1.y; clz = r1.z;
      } else {
        cx = a.xt[t0];
        cy = a.xt[a.ldt + t0];
        cz = a.xt[2 * a.ldt + t0];
        if (use_rec) {
          split_f32(cx, chx, clx);
          split_f32(cy, chy, cly);
          split_f32(cz, chz, clz);
        }
      }
    }

    R tx[T], ty[T], tz[T];
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const int64_t i = t0 + k * BLOCK + tid;
      if (i < t1 && tgt_rec) {
        const float4 r0 = a.rec[Tr::kRecQuads * i], r1 = a.rec[Tr::kRecQuads * i + 1];
        tx[k] = R(rel_f32(r0.x, r1.x, chx, clx));
        ty[k] = R(rel_f32(r0.y, r1.y, chy, cly));
        tz[k] = R(rel_f32(r0.z, r1.z, chz, clz));
      } else if (i < t1) {
        const double px = a.xt[i], py = a.xt[a.ldt + i], pz = a.xt[2 * a.ldt + i];
        if (use_rec) {
          float h, l;
          split_f32(px, h, l);
          tx[k] = R(rel_f32(h, l, chx, clx));
          split_f32(py, h, l);
          ty[k] = R(rel_f32(h, l, chy, cly));
          split_f32(pz, h, l);
          tz[k] = R(rel_f32(h, l, chz, clz));
        } else {
          tx[k] = R(px - cx); ty[k] = R(py - cy); tz[k] = R(pz - cz);
        }
      } else {
        tx[k] = R(0); ty[k] = R(0); tz[k] = R(0);
      }
    }

    // FP32: the warp's target box, against which every staged 32-source block
    // is tested for overlap (coincident pairs) and, for Gaussian-erf, distance.
    if constexpr (F32) warp_target_box<T>(tx, ty, tz, tbox + 2 * warp);

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
    bool aborted = false;
    if (use_tma && tid == 0 && s0 < s1) issue(s0, s1);
    for (int64_t tile0 = s0; tile0 < s1; tile0 += BLOCK) {
      // ---- stage one tile of sources -------------------------------------
      __syncthreads();  // previous tile fully consumed
      if constexpr (Tr::kTma) {
        if (use_tma) {
          const bool ok = mbar_wait(bar, phase);
          phase ^= 1u;
          if (__syncthreads_or(!ok)) {
            // A copy did not complete in time: record it, drain it with a
            // second, longer bounded wait, and leave together.  At most one
            // copy is ever in flight (the next tile's copy is issued only
            // after this wait succeeded and the records were consumed), so the
            // copy just waited on is the only one that could land late.
            if (tid == 0 && a.status) atomicOr(a.status, STATUS_TIMEOUT);
            mbar_wait(bar, phase ^ 1u, 1 << 26);
            if constexpr (!CLU) return;
            aborted = true;
            break;
          }
          const int64_t jj = tile0 + tid;
          Quad<R> qa, qb;
          if (jj < s1) {
            const float4 r0 = stage[3 * tid], r1 = stage[3 * tid + 1], r2 = stage[3 * tid + 2];
            qa.x = R(rel_f32(r0.x, r1.x, chx, clx));
            qa.y = R(rel_f32(r0.y, r1.y, chy, cly));
            qa.z = R(rel_f32(r0.z, r1.z, chz, clz));
            qa.w = R(r0.w);
            qb.x = R(r2.x); qb.y = R(r2.y); qb.z = R(r2.z);
            qb.w = R(r1.w);
          } else {
            qa.x = qa.y = qa.z = R(0);
            qb.x = qb.y = qb.z = R(0);
            source_consts<KERNEL, R>(1.0, qa.w, qb.w);
          }
          tileA[tid] = qa;
          tileB[tid] = qb;
          warp_source_box(qa.x, qa.y, qa.z, qa.w, jj < s1, sbox + 2 * warp);
          __syncthreads();  // quads ready, staging records consumed
          if (tid == 0 && tile0 + BLOCK < s1) issue(tile0 + BLOCK, s1);
        }
      }
      if (!use_tma) {
        const int64_t jj = tile0 + tid;
        Quad<R> qa, qb, qc, qd;
        qc.x = qc.y = qc.z = qc.w = R(0);
        qd.x = qd.y = qd.z = qd.w = R(0);
        if (use_rec && jj < s1) {
          const float4* r = a.rec + Tr::kRecQuads * jj;
          const float4 r0 = r[0], r1 = r[1], r2 = r[2];
          qa.x = R(rel_f32(r0.x, r1.x, chx, clx));
          qa.y = R(rel_f32(r0.y, r1.y, chy, cly));
          qa.z = R(rel_f32(r0.z, r1.z, chz, clz));
          qa.w = R(r0.w);
          qb.x = R(r2.x); qb.y = R(r2.y); qb.z = R(r2.z);
          qb.w = R(r1.w);
          if constexpr (!Tr::kUJ) {   // ζ: (v_q, c) and (w_q, 0)
            const float4 r3 = r[3];
            qc.x = R(r3.x); qc.y = R(r3.y); qc.z = R(r3.z);
            qc.w = R(r2.w);
            if constexpr (PASS == PASS_ZETAD) {
              const float4 r4 = r[4];
              qd.x = R(r4.x); qd.y = R(r4.y); qd.z = R(r4.z);
            }
          }
        } else if (jj < s1) {
          const double px = a.xs[jj], py = a.xs[a.lds + jj], pz = a.xs[2 * a.lds + jj];
          const double sig = a.ss[jj] * a.sigma_scale;
          qa.x = R(px - cx); qa.y = R(py - cy); qa.z = R(pz - cz);
          qb.x = R(a.gs[jj]); qb.y = R(a.gs[a.lds + jj]); qb.z = R(a.gs[2 * a.lds + jj]);
          if (Tr::kUJ) {
            source_consts<KERNEL, R>(sig, qa.w, qb.w);
          } else {
            if constexpr (F32) zeta_consts_f32<KERNEL>(sig, qa.w, qb.w, qc.w);
            else zeta_consts<KERNEL, R>(sig, qa.w, qb.w);
            if (a.vs) {
              qc.x = R(a.vs[jj]); qc.y = R(a.vs[a.lds + jj]); qc.z = R(a.vs[2 * a.lds + jj]);
            }
            if (PASS == PASS_ZETAD && a.ws) {
              qd.x = R(a.ws[jj]); qd.y = R(a.ws[a.lds + jj]); qd.z = R(a.ws[2 * a.lds + jj]);
            }
          }
        } else {
          // Padding source: zero strength, unit core.
          qa.x = qa.y = qa.z = R(0);
          qb.x = qb.y = qb.z = R(0);
          if (Tr::kUJ) source_consts<KERNEL, R>(1.0, qa.w, qb.w);
          else if constexpr (F32) zeta_consts_f32<KERNEL>(1.0, qa.w, qb.w, qc.w);
          else zeta_consts<KERNEL, R>(1.0, qa.w, qb.w);
        }
        tileA[tid] = qa;
        tileB[tid] = qb;
        if (!Tr::kUJ) tileC[tid] = qc;
        if (PASS == PASS_ZETAD) tileD[tid] = qd;
        if constexpr (F32) warp_source_box(qa.x, qa.y, qa.z, qa.w, jj < s1, sbox + 2 * warp);
        __syncthreads();
      }

      // ---- all pairs of the tile ------------------------------------------
      const int cnt = int(min(int64_t(BLOCK), s1 - tile0));
      // FP32: coincident pairs (r² = 0, skipped as the reference's direct sums
      // skip them) can only occur in 32-source blocks whose box intersects the
      // warp's target box; only those blocks run the masked pair forms.  The
      // test is exact in the kernel's own coordinates (comparisons only), so
      // a target's own particle and any other particle at the same position
      // are masked wherever they sit.  (FP64 masks every pair.)
      uint32_t ovl = 0;
      if constexpr (F32) ovl = overlap_blocks<BLOCK / 32>(tbox + 2 * warp, sbox, cnt);
      if constexpr (Tr::kUJ && F32) {
        const float4* ta = reinterpret_cast<const float4*>(tileA);
        const float4* tb = reinterpret_cast<const float4*>(tileB);
        if constexpr (PASS == PASS_UJ) {
          if (KERNEL == VPM_KERNEL_WINCKELMANS) {
            // Runs of blocks: masked where the boxes intersect.
            const uint32_t cls = overlap_codes<BLOCK / 32>(ovl, 1u);
            for (int js = 0; js < cnt;) {
              const int je = block_run_end(cls, js, cnt, [](uint32_t c) { return c; });
              if ((ovl >> (js >> 5)) & 1u) {
#pragma unroll 2
                for (; js < je; ++js) uj_source_winck<T, true>(ta[js], tb[js], tx, ty, tz, acc);
              } else {
#pragma unroll 2
                for (; js < je; ++js) uj_source_winck<T, false>(ta[js], tb[js], tx, ty, tz, acc);
              }
            }
          } else {
            // Gaussian-erf masks coincident pairs in its series branch, which
            // every warp holding a pair with ρ² < 3/2 takes.
            // Gaussian-erf by runs of 32-source blocks of one class: far blocks
            // skip erfcx/exp, vote blocks decide per source.
            const uint32_t cls = classify_blocks<BLOCK / 32>(tbox + 2 * warp, sbox, cnt,
                                                             kVoteSpan * kArgFar, use_far);
            auto key = [](uint32_t c) { return c >= 2u ? 2u : c; };
            for (int js = 0; js < cnt;) {
              const int je = block_run_end(cls, js, cnt, key);
              const uint32_t c = key((cls >> (2 * (js >> 5))) & 3u);
              if (c == 2u) {
#pragma unroll 2
                for (; js < je; ++js) uj_source_gauss_far<T>(ta[js], tb[js], tx, ty, tz, acc);
              } else if (c == 1u) {
#pragma unroll 2
                for (; js < je; ++js) uj_source_gauss<T, true>(ta[js], tb[js], tx, ty, tz, acc);
              } else {
#pragma unroll 2
                for (; js < je; ++js) uj_source_gauss<T, false>(ta[js], tb[js], tx, ty, tz, acc);
              }
            }
          }
        } else {
          if (KERNEL == VPM_KERNEL_WINCKELMANS) {
            const uint32_t cls = overlap_codes<BLOCK / 32>(ovl, 1u);
            for (int js = 0; js < cnt;) {
              const int je = block_run_end(cls, js, cnt, [](uint32_t c) { return c; });
              if ((ovl >> (js >> 5)) & 1u) {
                for (; js < je; ++js) ujd_source_winck<T, true>(ta[js], tb[js], tx, ty, tz, acc);
              } else {
                for (; js < je; ++js) ujd_source_winck<T, false>(ta[js], tb[js], tx, ty, tz, acc);
              }
            }
          } else {
            // Gaussian-erf: where Dq and Dp vanish only the plain sums take the
            // pair; far blocks skip erfcx.
            const uint32_t cls = classify_blocks<BLOCK / 32>(tbox + 2 * warp, sbox, cnt,
                                                             kVoteSpan * kArgFar, use_far);
            auto key = [](uint32_t c) { return c; };
            for (int js = 0; js < cnt;) {
              const int je = block_run_end(cls, js, cnt, key);
              const uint32_t c = (cls >> (2 * (js >> 5))) & 3u;
              if (c == 3u) {
                for (; js < je; ++js) uj_source_gauss_far<T>(ta[js], tb[js], tx, ty, tz, acc);
              } else if (c == 2u) {
                for (; js < je; ++js) ujd_source_gauss_far<T>(ta[js], tb[js], tx, ty, tz, acc);
              } else if (c == 1u) {
                for (; js < je; ++js) ujd_source_gauss<T, true>(ta[js], tb[js], tx, ty, tz, acc);
              } else {
                for (; js < je; ++js) ujd_source_gauss<T, false>(ta[js], tb[js], tx, ty, tz, acc);
              }
            }
          }
        }
      } else if constexpr (Tr::kUJ) {
        // FP64 U/J (and DJ).
#pragma unroll 2
        for (int js = 0; js < cnt; ++js) {
          const Quad<R> sa = tileA[js];
          const Quad<R> sb = tileB[js];
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
            if constexpr (PASS == PASS_UJD) {
              R dq, dp;
              pair_dqp_f64<KERNEL>(r2, sa.w, sb.w, dq, dp);
              const R e0 = dp * c0, e1 = dp * c1, e2 = dp * c2;
              acc[k][15] += e0 * dx; acc[k][16] += e0 * dy; acc[k][17] += e0 * dz;
              acc[k][18] += e1 * dx; acc[k][19] += e1 * dy; acc[k][20] += e1 * dz;
              acc[k][21] += e2 * dx; acc[k][22] += e2 * dy; acc[k][23] += e2 * dz;
              acc[k][24] += dq * sb.x; acc[k][25] += dq * sb.y; acc[k][26] += dq * sb.z;
            }
          }
        }
      } else if constexpr (F32) {
        // ζ passes, FP32.
        const float4* ta = reinterpret_cast<const float4*>(tileA);
        const float4* tb = reinterpret_cast<const float4*>(tileB);
        const float4* tc = reinterpret_cast<const float4*>(tileC);
        const float4* td = reinterpret_cast<const float4*>(PASS == PASS_ZETAD ? tileD : tileC);
        constexpr bool DD = PASS == PASS_ZETAD;
        // Block codes: 3 skip (Gaussian-erf ζ is exactly zero at every target
        // of the warp), 2 masked (boxes intersect), 1 per-source votes, 0 the
        // general form.
        uint32_t cls = overlap_codes<BLOCK / 32>(ovl, 2u);
        if (kFarKernel && use_far) {
          const uint32_t far = classify_blocks<BLOCK / 32>(tbox + 2 * warp, sbox, cnt,
                                                           kVoteSpan * kArgZero, true);
#pragma unroll
          for (int b = 0; b < BLOCK / 32; ++b) {
            const uint32_t f = (far >> (2 * b)) & 3u;
            if (f == 3u) cls |= 3u << (2 * b);            // zero blocks cannot coincide
            else if (f >= 1u && !((ovl >> b) & 1u)) cls |= 1u << (2 * b);
          }
        }
        for (int js = 0; js < cnt;) {
          const int je = block_run_end(cls, js, cnt, [](uint32_t c) { return c; });
          const uint32_t c = (cls >> (2 * (js >> 5))) & 3u;
          if (c == 3u) {
            js = je;
          } else if (c == 2u) {
#pragma unroll 2
            for (; js < je; ++js)
              zeta_source<KERNEL, T, true, DD, false>(ta[js], tb[js], tc[js], td[js], tx, ty, tz, acc);
          } else if (c == 1u) {
#pragma unroll 2
            for (; js < je; ++js)
              zeta_source<KERNEL, T, false, DD, true>(ta[js], tb[js], tc[js], td[js], tx, ty, tz, acc);
          } else {
#pragma unroll 2
            for (; js < je; ++js)
              zeta_source<KERNEL, T, false, DD, false>(ta[js], tb[js], tc[js], td[js], tx, ty, tz, acc);
          }
        }
      } else {
        // ζ passes, FP64.
#pragma unroll 2
        for (int js = 0; js < cnt; ++js) {
          const Quad<R> sa = tileA[js];
          const Quad<R> sb = tileB[js];
          const Quad<R> sc = tileC[js];
#pragma unroll
          for (int k = 0; k < T; ++k) {
            const R dx = tx[k] - sa.x, dy = ty[k] - sa.y, dz = tz[k] - sa.z;
            const R r2 = dx * dx + dy * dy + dz * dz;
            if constexpr (PASS == PASS_ZETA) {
              const R z = pair_zeta<KERNEL>(r2, sa.w, sb.w);
              acc[k][0] += z * sb.x; acc[k][1] += z * sb.y; acc[k][2] += z * sb.z;
              acc[k][3] += z * sc.x; acc[k][4] += z * sc.y; acc[k][5] += z * sc.z;
            } else {
              const Quad<R> sd = tileD[js];
              R z, dzz;
              pair_zeta_d<KERNEL>(r2, sa.w, sb.w, z, dzz);
              acc[k][0] += z * sb.x; acc[k][1] += z * sb.y; acc[k][2] += z * sb.z;
              acc[k][3] += z * sc.x; acc[k][4] += z * sc.y; acc[k][5] += z * sc.z;
              acc[k][6] += dzz * sb.x; acc[k][7] += dzz * sb.y; acc[k][8] += dzz * sb.z;
              acc[k][9] += dzz * sc.x + z * sd.x;
              acc[k][10] += dzz * sc.y + z * sd.y;
              acc[k][11] += dzz * sc.z + z * sd.z;
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

    // A CTA whose copy timed out leaves without results (the status word
    // reports it); in a cluster it still takes part in both cluster barriers
    // below, so that no CTA leaves while another may read its shared memory.

    // ---- epilogue: cluster form ----------------------------------------------
    if constexpr (CLU) {
      // Every rank's (hi, lo) pairs are final after the first barrier.
      cluster_sync_all();
      if (!aborted) cluster_epilogue<PASS, KERNEL, PREC, BLOCK, T>(a, fold_hi, fold_lo, t0, t1);
      cluster_sync_all();   // remote reads done before any CTA leaves
      return;
    }

    // ---- epilogue ------------------------------------------------------------
    // A slot is kept in L2 (evict_last) in the fused form until its tile is summed.
#pragma unroll
    for (int k = 0; k < T; ++k) {
      const int64_t i = t0 + k * BLOCK + tid;
      if (i >= t1) continue;
      if constexpr (F32) {
        if (slot >= 0) {   // the raw float pairs (PairSum)
          const uint64_t pol = l2_policy(a.tile_done != nullptr);
#pragma unroll
          for (int w = 0; w < NV; ++w) {
            const int o = (w * T + k) * BLOCK + tid;
            st_global_hint_f2(a.part + (int64_t(slot) * NV + w) * a.ldp + i,
                              COMP ? fold_hi[o] : acc[k][w], COMP ? fold_lo[o] : 0.f, pol);
          }
          continue;
        }
      }
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
      if constexpr (F32) finish_f32_sums<PASS, KERNEL>(v);
      if (slot >= 0) {
        const uint64_t pol = l2_policy(a.tile_done != nullptr);
#pragma unroll
        for (int w = 0; w < NV; ++w)
          st_global_hint(a.part + (int64_t(slot) * NV + w) * a.ldp + i, v[w], pol);
      } else {
        write_final<PASS, KERNEL>(v, a, i);
      }
    }
    if (!a.items && a.tile_done && slot >= 0) {
      // The slot reaches L2 before the tile's count; the CTA that counts the
      // tile's last chunk sums the slots (the counter pattern of a fenced
      // last-block reduction).
      __threadfence();
      __syncthreads();
      if (tid == 0) s_last = atomicAdd(a.tile_done + item / a.n_chunk, 1u) == unsigned(a.n_chunk - 1);
      __syncthreads();
      if (s_last) {
        __threadfence();
        tile_reduce<PASS, KERNEL, BLOCK, T, F32>(a, t0, t1);
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

// Fixed-order sum of the partial slots.  A block holds 32 targets (x) and
// reduce_rows(NV) value rows (y): thread (x, y) sums rows y, y + rows, ... of
// its target over the chunks in chunk order, loading kReduceLoads chunks ahead
// (the same additions in the same order as one thread per target walking every
// row, so the result is bitwise that one), and one warp then forms the final
// values from shared memory.  F2: the FP32 passes' float-pair slots, summed
// with PairSum; otherwise FP64 slots and FP64 additions.
__host__ __device__ constexpr int reduce_rows(int nv) { return nv <= 32 ? nv : (nv + 1) / 2; }
constexpr int kReduceLoads = 8;

template <int PASS, int KERNEL, bool F2>
__global__ void __launch_bounds__(32 * reduce_rows(nval_of(PASS))) reduce_kernel(
    const double* __restrict__ part, int64_t ldp, const int64_t* __restrict__ foff,
    const int32_t* __restrict__ fchunks, int nfields, int scalar_chunks, int64_t t_begin,
    int64_t t_end, PairArgs out) {
  constexpr int NV = nval_of(PASS);
  constexpr int kRows = reduce_rows(NV);
  __shared__ double sv[NV][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t i = t_begin + int64_t(blockIdx.x) * 32 + tx;
  int nc = 0;
  if (i < t_end) {
    nc = scalar_chunks;
    if (foff) {
      int lo = 0, hi = nfields - 1;
      while (lo < hi) {  // last field with foff[f] <= i
        const int mid = (lo + hi + 1) >> 1;
        if (foff[mid] <= i) lo = mid; else hi = mid - 1;
      }
      nc = fchunks[lo];
    }
  }
  const bool live = nc > 1;
  if (live) {
    const int64_t step = int64_t(NV) * ldp;
    for (int w = ty; w < NV; w += kRows) {
      int c = 0;
      if constexpr (F2) {
        const float2* p = reinterpret_cast<const float2*>(part) + int64_t(w) * ldp + i;
        PairSum sum;
        for (; c + kReduceLoads <= nc; c += kReduceLoads) {
          float2 a[kReduceLoads];
#pragma unroll
          for (int l = 0; l < kReduceLoads; ++l) a[l] = p[int64_t(c + l) * step];
#pragma unroll
          for (int l = 0; l < kReduceLoads; ++l) sum.add(a[l]);
        }
        for (; c < nc; ++c) sum.add(p[int64_t(c) * step]);
        sv[w][tx] = sum.value();
      } else {
        const double* p = part + int64_t(w) * ldp + i;
        double v = 0.0;
        for (; c + kReduceLoads <= nc; c += kReduceLoads) {
          double a[kReduceLoads];
#pragma unroll
          for (int l = 0; l < kReduceLoads; ++l) a[l] = p[int64_t(c + l) * step];
#pragma unroll
          for (int l = 0; l < kReduceLoads; ++l) v += a[l];
        }
        for (; c < nc; ++c) v += p[int64_t(c) * step];
        sv[w][tx] = v;
      }
    }
  }
  __syncthreads();
  if (ty == 0 && live) {
    double v[NV];
#pragma unroll
    for (int w = 0; w < NV; ++w) v[w] = sv[w][tx];
    if constexpr (F2) finish_f32_sums<PASS, KERNEL>(v);
    write_final<PASS, KERNEL>(v, out, i);
  }
}

// ---------------------------------------------------------------- dispatch --
typedef void (*PairFn)(const PairArgs);

template <int PASS, int KERNEL, int PREC, int BLOCK, int T, bool CLU = false>
PairFn fn_ready() {
  static bool once = [] {
    cudaFuncSetAttribute(pair_kernel<PASS, KERNEL, PREC, BLOCK, T, CLU>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(smem_bytes<PASS, PREC>(BLOCK, T)));
    // Clusters of up to 16 CTAs (beyond the portable 8) for the split-source form.
    if (CLU)
      cudaFuncSetAttribute(pair_kernel<PASS, KERNEL, PREC, BLOCK, T, CLU>,
                           cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return true;
  }();
  (void)once;
  return pair_kernel<PASS, KERNEL, PREC, BLOCK, T, CLU>;
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

template <int PASS>
PairFn pick_kernel(int kernel, int prec, Shape s) {
  return kernel == VPM_KERNEL_WINCKELMANS ? pick_prec<PASS, VPM_KERNEL_WINCKELMANS>(prec, s)
                                          : pick_prec<PASS, VPM_KERNEL_GAUSSIANERF>(prec, s);
}

// The cluster form of an FP32C shape (null for other precisions and shapes).
template <int PASS, int KERNEL>
PairFn pick_cluster_k(Shape s) {
  constexpr int P = VPM_PREC_FP32C;
  if (s.block == 128 && s.tpt == 2) return fn_ready<PASS, KERNEL, P, 128, 2, true>();
  if (s.block == 128 && s.tpt == 4) return fn_ready<PASS, KERNEL, P, 128, 4, true>();
  if (s.block == 256 && s.tpt == 2) return fn_ready<PASS, KERNEL, P, 256, 2, true>();
  return nullptr;
}

template <int PASS>
PairFn pick_cluster(int kernel, int prec, Shape s) {
  if (prec != VPM_PREC_FP32C) return nullptr;
  return kernel == VPM_KERNEL_WINCKELMANS ? pick_cluster_k<PASS, VPM_KERNEL_WINCKELMANS>(s)
                                          : pick_cluster_k<PASS, VPM_KERNEL_GAUSSIANERF>(s);
}

template <int PASS>
size_t smem_of(int precision, Shape s) {
  switch (precision) {
    case VPM_PREC_FP64: return smem_bytes<PASS, VPM_PREC_FP64>(s.block, s.tpt);
    case VPM_PREC_FP32: return smem_bytes<PASS, VPM_PREC_FP32>(s.block, s.tpt);
    default: return smem_bytes<PASS, VPM_PREC_FP32C>(s.block, s.tpt);
  }
}

template <int PASS>
int ctas_per_sm(int kernel, int precision, Shape s) {
  PairFn f = pick_kernel<PASS>(kernel, precision, s);
  if (!f) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, s.block, smem_of<PASS>(precision, s)) !=
      cudaSuccess)
    return 0;
  return n;
}

// Launch configuration of a cluster launch (`attr` receives the attribute).
inline cudaLaunchConfig_t cluster_config(int grid, int block, size_t smem, cudaStream_t st,
                                         int cluster, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(unsigned(grid), 1, 1);
  cfg.blockDim = dim3(unsigned(block), 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr->id = cudaLaunchAttributeClusterDimension;
  attr->val.clusterDim.x = unsigned(cluster);
  attr->val.clusterDim.y = 1;
  attr->val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <int PASS>
cudaError_t launch(int kernel, int precision, Shape s, const PairArgs& a, int grid,
                   cudaStream_t st) {
  PairFn f = pick_kernel<PASS>(kernel, precision, s);
  if (!f) return cudaErrorInvalidConfiguration;
  if (grid <= 0) return cudaSuccess;
  if (a.cluster > 1) {
    // One item per CTA, every CTA of a cluster on the same target tile.
    f = pick_cluster<PASS>(kernel, precision, s);
    if (!f || a.items || a.counter || grid % a.cluster != 0 ||
        int64_t(grid) != int64_t(a.n_tb) * a.n_chunk || a.n_chunk != a.cluster)
      return cudaErrorInvalidConfiguration;
    cudaLaunchAttribute attr;
    cudaLaunchConfig_t cfg = cluster_config(grid, s.block, smem_of<PASS>(precision, s), st,
                                            a.cluster, &attr);
    return cudaLaunchKernelEx(&cfg, f, a);
  }
  f<<<grid, s.block, smem_of<PASS>(precision, s), st>>>(a);
  return cudaGetLastError();
}

// Clusters of `cluster` CTAs of a shape that can be resident at once (0: none
// can be scheduled, or the query failed).
template <int PASS>
int max_active_clusters(int kernel, int precision, Shape s, int cluster) {
  PairFn f = pick_cluster<PASS>(kernel, precision, s);
  if (!f) return 0;
  cudaLaunchAttribute attr;
  cudaLaunchConfig_t cfg = cluster_config(cluster, s.block, smem_of<PASS>(precision, s), nullptr,
                                          cluster, &attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, f, &cfg) != cudaSuccess) {
    cudaGetLastError();   // clear the sticky-free error of a refused query
    return 0;
  }
  return n;
}

template <int PASS>
cudaError_t reduce(int kernel, int precision, const double* part, int64_t ldp,
                   const int64_t* foff, const int32_t* fchunks, int nfields, int scalar_chunks,
                   int64_t t_begin, int64_t t_end, double* u, double* j, double* dj,
                   int64_t ldo, cudaStream_t st) {
  const int64_t n = t_end - t_begin;
  if (n <= 0) return cudaSuccess;
  PairArgs out;
  memset(&out, 0, sizeof(out));
  out.u = u; out.j = j; out.dj = dj; out.ldo = ldo;
  const dim3 bs(32, reduce_rows(nval_of(PASS)));
  const int grid = int((n + 31) / 32);
  const bool f2 = precision != VPM_PREC_FP64;   // float-pair slots (PairSum)
  auto go = [&](auto kern) {
    kern<<<grid, bs, 0, st>>>(part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin, t_end,
                              out);
  };
  if (kernel == VPM_KERNEL_WINCKELMANS) {
    if (f2) go(reduce_kernel<PASS, VPM_KERNEL_WINCKELMANS, true>);
    else go(reduce_kernel<PASS, VPM_KERNEL_WINCKELMANS, false>);
  } else {
    if (f2) go(reduce_kernel<PASS, VPM_KERNEL_GAUSSIANERF, true>);
    else go(reduce_kernel<PASS, VPM_KERNEL_GAUSSIANERF, false>);
  }
  return cudaGetLastError();
}

}  // namespace vpm
