// internal.h — declarations shared by the translation units of libvpmgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vpm_gpu.h"

namespace vpm {

// Pair passes.  The D forms also accumulate the derivative with respect to a
// common scale α of every core size (d/dα at α = 1), for the analytic dynamic
// SFS procedure.
enum PairPass { PASS_UJ = 0, PASS_ZETA = 1, PASS_UJD = 2, PASS_ZETAD = 3 };
constexpr int kNvalUJ = 15;     // Uacc(3), Aacc(9), Wacc(3)
constexpr int kNvalZeta = 6;    // Ω(3) = Σ ζ Γ_q, V(3) = Σ ζ v_q
constexpr int kNvalUJD = 27;    // UJ values, then DAacc(9), DWacc(3)
constexpr int kNvalZetaD = 12;  // Ω, V, DΩ = Σ Dζ Γ_q, DV = Σ (Dζ v_q + ζ w_q)

__host__ __device__ constexpr int nval_of(int pass) {
  return pass == PASS_UJ ? kNvalUJ
         : pass == PASS_ZETA ? kNvalZeta
         : pass == PASS_UJD ? kNvalUJD
                            : kNvalZetaD;
}

// One work item: targets [t0, t1) against sources [s0, s1).  slot < 0 means the
// item covers all sources of its targets and writes final values; otherwise it
// writes raw sums into partial slot `slot`.
struct PairItem {
  int64_t t0, t1, s0, s1;
  int32_t slot;
  int32_t field;
};

struct PairArgs {
  // Sources: FP64 SoA rows of leading dimension lds.
  const double* xs;
  const double* gs;
  const double* ss;
  const double* vs;   // PASS_ZETA(D): per-source v_q = S(J_q, Γ_q), 3 rows (may be null)
  const double* ws;   // PASS_ZETAD: per-source w_q = S(DJ_q, Γ_q), 3 rows
  int64_t lds;
  // Target positions: FP64 SoA of leading dimension ldt.
  const double* xt;
  int64_t ldt;
  double sigma_scale;
  // Decomposition without a table: targets [t_off, t_off+nt) x sources [0, ns).
  int64_t t_off, nt, ns, chunk;
  int32_t n_tb, n_chunk;
  // Decomposition from a table (batches): n_items entries, dynamic queue when
  // counter != null.
  const PairItem* items;
  int32_t n_items;
  unsigned int* counter;
  // Outputs.  Final: UJ -> U rows 0..2 of `u` (ld ldo), J rows 0..8 of `j`
  // (UJD also DJ rows 0..8 of `dj`); ZETA(D) -> raw rows 0..5 (0..11) of `u`.
  // Partials: part[(slot*nval + k)*ldp + i].
  double* u;
  double* j;
  double* dj;
  int64_t ldo;
  double* part;
  int64_t ldp;
  // FP32 passes: packed source records, 3 float4 per source for U/J, 4 for ζ,
  // 5 for ζ + α-derivative (null: read and convert the FP64 rows in the
  // kernel).  Records are 16-byte aligned.
  const float4* rec;
  // Stage the records with bulk asynchronous copies (PASS_UJ; needs rec).
  int32_t tma;
  // Gaussian-erf FP32 passes: classify (warp, 32-source) blocks by their
  // bounding boxes and take the far-field forms (0 = always the general form).
  int32_t far;
  // When non-null: the number of compact 32-particle source blocks (counted
  // by the pack kernel); the classification runs only when at least a quarter
  // of the coh_blocks blocks are compact (coherent particle order).
  const unsigned int* coh;
  int64_t coh_blocks;
  int* status;   // STATUS_TIMEOUT is OR-ed here if a copy wait gives up (may be null)
  // FP32C single-field form only: > 1 when the n_chunk source chunks of a
  // target tile run as one thread-block cluster of `cluster` CTAs (grid =
  // n_tb x cluster, cluster rank = chunk) that sum their compensated partial
  // sums through distributed shared memory in rank order; no partial slots.
  int32_t cluster;
  // Single-field form with split sources, when non-null: the items run
  // tile-major (item = tile * n_chunk + chunk), and the last CTA of a target
  // tile to finish (n_tb counters, zero at launch) sums the tile's partial
  // slots in chunk order, writes the final values and discards the summed
  // lines from L2, so that they are not written back to DRAM.
  unsigned int* tile_done;
};

// Tile shape of a launch.
// Far-field classification of the Gaussian-erf FP32 passes is on unless the
// environment sets VPM_NO_FARFIELD (to non-zero).
bool farfield_enabled();
// Bulk-copy staging of the packed records is on unless VPM_NO_TMA is set (to
// non-zero); the kernels then read the records with plain loads.
bool tma_disabled();
// Whether the pack kernel counts compact source blocks for a field of n particles.
bool coherence_counted(int64_t n);

struct Shape {
  int block;   // threads per CTA
  int tpt;     // targets per thread
};

// Launch one pair pass (grid chosen by the caller through args/n_items).
cudaError_t launch_pair(int pass, int kernel, int precision, Shape shape, const PairArgs& a,
                        int grid, cudaStream_t st);
// Dynamic shared memory of a shape (bytes).
size_t pair_smem_bytes(int pass, int precision, Shape shape);
// Clusters of `cluster` CTAs of a shape that fit on the device at once (0: the
// shape cannot run as such clusters; only FP32C shapes do).
int pair_max_active_clusters(int pass, int kernel, int precision, Shape shape, int cluster);
int pair_max_active_clusters_d(int pass, int kernel, int precision, Shape shape, int cluster);
// Max resident CTAs per SM of a shape.
int pair_ctas_per_sm(int pass, int kernel, int precision, Shape shape);
// Whether a shape is compiled.
bool pair_shape_supported(int precision, Shape shape);

// Sum partial slots in fixed order and write the final values.  FP64 passes
// hold FP64 slots, summed in FP64; the FP32 passes hold float pairs (hi, lo),
// summed as a double-float (PairSum in pair_kernel.cuh).
//   UJ: U = -Uacc/(4π), J = -(Aacc·KP + ε·Wacc)/(4π); ZETA: raw sums.
// Targets are [t_begin, t_end); the slot count of target i is scalar_chunks
// when foff is null, else found from the device field table (foff[f] <= i,
// fchunks[f]); targets whose count is 1 are skipped (already final).
// Packed source records (3 float4 per source) of n particles for the FP32
// U/J passes with kernel constants of σ·scale.  Gaussian-erf: *compact (may
// be null) is reset and then counts the compact 32-particle blocks.
cudaError_t launch_pack_sources(int kernel, int64_t n, const double* X, const double* G,
                                const double* S, int64_t ld, double scale, float4* rec,
                                unsigned int* compact, cudaStream_t st);
// Packed source records of the FP32 ζ passes (4 float4 per source, 5 with d
// for PASS_ZETAD): split positions and ζ constants of σ·scale, Γ, v_q (V rows,
// zero when null) and w_q (W rows).
cudaError_t launch_pack_zeta_sources(int kernel, bool d, int64_t n, const double* X,
                                     const double* G, const double* S, const double* V,
                                     const double* W, int64_t ld, double scale, float4* rec,
                                     cudaStream_t st);
cudaError_t launch_reduce(int pass, int kernel, int precision, const double* part, int64_t ldp,
                          const int64_t* foff, const int32_t* fchunks, int nfields,
                          int scalar_chunks, int64_t t_begin, int64_t t_end, double* u,
                          double* j, double* dj, int64_t ldo, cudaStream_t st);

// The D passes live in pair_d.cu; launch_pair/launch_reduce/pair_ctas_per_sm/
// pair_smem_bytes forward to these for PASS_UJD and PASS_ZETAD.
cudaError_t launch_pair_d(int pass, int kernel, int precision, Shape shape, const PairArgs& a,
                          int grid, cudaStream_t st);
cudaError_t launch_reduce_d(int pass, int kernel, int precision, const double* part, int64_t ldp,
                            const int64_t* foff, const int32_t* fchunks, int nfields,
                            int scalar_chunks, int64_t t_begin, int64_t t_end, double* u,
                            double* j, double* dj, int64_t ldo, cudaStream_t st);
size_t pair_smem_bytes_d(int pass, int precision, Shape shape);
int pair_ctas_per_sm_d(int pass, int kernel, int precision, Shape shape);

}  // namespace vpm
