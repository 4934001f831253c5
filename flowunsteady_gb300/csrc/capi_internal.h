// capi_internal.h — host-side structures shared by capi.cu, batch.cu and device_api.cu.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "internal.h"
#include "update.h"
#include "vpm_device.cuh"

namespace vpm {

extern thread_local std::string g_last_error;
int set_error(std::string* slot, int code, const std::string& msg);
int64_t ceil_div(int64_t a, int64_t b);
int64_t round_up(int64_t a, int64_t b);

// One pair pass over targets [t0, t1) of xt against sources [0, ns).
struct PairCall {
  int pass, kernel, prec;
  int64_t t0, t1, ns;
  const double *xs, *gs, *ss, *vs;
  const double* ws = nullptr;   // PASS_ZETAD: w_q rows
  int64_t lds;
  const double* xt;
  int64_t ldt;
  double sigma_scale;
  double *u, *j;
  double* dj = nullptr;         // PASS_UJD: DJ rows
  int64_t ldo;
  int max_chunks = 0;   // upper bound on source chunks (0 = planner's choice)
  int64_t chunk = 0;    // pinned source chunk length (0 = planner's choice)
  // FP32 passes: packed records of the ns sources (launch_pack_sources for
  // U/J, launch_pack_zeta_sources for ζ), or null to read the FP64 rows in the
  // kernel.  Bulk copies stage the U/J records.
  const float4* rec = nullptr;
  const unsigned int* coh = nullptr;   // compact-block count (see PairArgs::coh)
  int* status = nullptr;
};

struct PairPlan {
  Shape shape = Shape{0, 0};
  int64_t n_tb = 0;
  int n_chunk = 1;      // source chunks per target tile
  int64_t chunk = 0;    // sources per chunk
  int cluster = 1;      // > 1: the chunks of a tile are one cluster, summed on chip
  // The last CTA of each target tile sums its partial slots (no reduction
  // launch); the tiles' counters follow the slots in the scratch.
  bool fused = false;
  // Partial slots the plan writes (and a reduction launch, or the fused form, sums).
  int slots() const { return (n_chunk > 1 && cluster <= 1) ? n_chunk : 1; }
  // Kernel launches of the pass: the pair kernel, and the reduction unless fused.
  int launches() const { return (slots() > 1 && !fused) ? 2 : 1; }
};

// Fused reduction of split source ranges: -1 (default) the planner's rule,
// 0 (VPM_FUSED_REDUCE=0) always a reduction launch, 1 (=1) always fused.
int fused_reduce_mode();

// Plan of the last stateless U/J call (vpm_uj_device_async/_noalloc) on this
// host thread, for vpm_debug_last_plan.
extern thread_local PairPlan g_last_stateless_plan;
// Split-source clusters: 0 (default) sums split source ranges through partial
// slots; 1 (VPM_CLUSTER=1) takes clusters whenever a cluster size fits.
int cluster_mode();

Shape default_shape(int pass, int precision, int64_t n);
Shape lookup_shape(int device, int pass, int kernel, int precision, int64_t n, const Shape* pinned);
void store_shape(int device, int pass, int kernel, int precision, int64_t n, Shape s);
// Size bucket (floor log2 n) under which tuned shapes are stored.
int shape_bucket(int64_t n);
int resident_ctas(int device, int pass, int kernel, int precision, Shape s, int num_sms);
int plan_chunks(int64_t n_tb, int64_t ns, int block, int resident, int64_t* chunk_out,
                int max_chunks = 0);
cudaError_t run_pair(const PairCall& pc, int device, int num_sms, const Shape* pinned,
                     double* part, int64_t ldp, size_t part_elems, size_t* need_part, bool dry,
                     cudaStream_t st, PairPlan* plan_out);

// Free-vortex force of bound particles (ffv.cu).
size_t ffv_plan(int64_t nb, int64_t nf, int num_sms, int64_t* chunk, int* n_chunk);
cudaError_t launch_ffv(int kernel, int64_t nb, const double* xb, const double* gb,
                       const double* sb, int64_t ldb, int64_t nf, const double* xf,
                       const double* gf, int64_t ldf, double* part, double* M, int64_t ldm,
                       int num_sms, cudaStream_t st);

struct GraphKey {
  int64_t n, n_static;
  double dt;
  int64_t relax;
  int64_t mixed;   // static particles not (only) at the tail: flag-tested updates
  vpm_scheme scheme;
};

struct GraphEntry {
  GraphKey key;
  cudaGraphExec_t exec;
  int64_t kernels;   // kernel nodes of one replay
};

// Flattened work queue of a batch of independent fields (see batch.cu): one
// group of items per tile shape, each group one persistent launch.
constexpr int kMaxBatchGroups = 4;
struct BatchGroup {
  Shape shape;
  int first = 0;        // items [first, first + n_items) of d_items
  int n_items = 0;
  int resident = 1;     // persistent grid of the group's launch
};
struct BatchPlan {
  std::vector<BatchGroup> groups;
  PairItem* d_items = nullptr;
  int n_items = 0;
  int64_t* d_foff = nullptr;
  int32_t* d_fchunks = nullptr;
  int nfields = 0;
  int max_chunks = 1;
  unsigned int* d_counter = nullptr;   // one queue counter per group
  int kernel = -1, precision = -1;   // plan built for this pair
  std::vector<int64_t> h_off, h_n;   // field offsets and sizes
  std::vector<Shape> h_shape;        // tile shape of each field in the current plan
  std::vector<Shape> h_tuned;        // per-field shapes chosen by vpm_batch_autotune (empty: table)
  int tuned_kernel = -1, tuned_precision = -1;   // the pass h_tuned was timed for
};

}  // namespace vpm

namespace vpm {
// Morton order of the direct pair passes of large fields (csrc/tree.cu).
struct SortWork;
void sort_free(SortWork* s);
cudaError_t sort_reserve(SortWork*& s, int64_t n, int nfields = 1);
cudaError_t sort_order(SortWork* s, int64_t n, const double* X, int64_t ld, cudaStream_t st,
                       const int** perm);
// Batches: each field (offsets foff) along the Morton curve of its own cube.
cudaError_t sort_order_fields(SortWork* s, int64_t n, const double* X, int64_t ld,
                              const int64_t* foff, int nfields, cudaStream_t st, const int** perm);
cudaError_t launch_gather_rows(int64_t n, int rows, const int* perm, const double* src,
                               int64_t lds, double* dst, int64_t ldd, cudaStream_t st);
cudaError_t launch_scatter_rows(int64_t n, int rows, const int* perm, const double* src,
                                int64_t lds, double* dst, int64_t ldd, cudaStream_t st);
struct FmmWork;
void fmm_free(FmmWork* w);
bool fmm_order_supported(int p);
// U and J (and, when dj is given, the near-field α-derivative DJ: FP32
// Gaussian-erf only) of every particle by the treecode.
// With local_order > 0 (7; p = 4, FP32/FP32C) far cells at least as large as
// the target group are taken by a local expansion per group.
cudaError_t fmm_eval(vpm_ctx* c, int kernel, int prec, int p, int ncrit, double theta,
                     double sfac, int local_order, double* dj, const char** why);
bool fmm_local_order_supported(int q);
// ζ sums over the near lists of the last fmm_eval of the same field.
cudaError_t fmm_zeta(vpm_ctx* c, bool d, const double* vs, const double* ws, double* out,
                     const char** why);
void fmm_stats(const FmmWork* w, int64_t* out);
}  // namespace vpm

struct vpm_ctx {
  int device = 0;
  int num_sms = 0;
  int64_t cap = 0, ld = 0;
  int64_t n = 0, n_static = 0;
  double t = 0.0;
  int64_t nt = 0;
  cudaStream_t own = nullptr, st = nullptr;
  double* base = nullptr;
  double *X = nullptr, *G = nullptr, *S = nullptr, *C = nullptr, *Q = nullptr;
  double *U = nullptr, *J = nullptr, *E = nullptr, *V = nullptr, *raw = nullptr;
  double *Ut = nullptr, *Jt = nullptr, *Et = nullptr;
  double* part = nullptr;
  size_t part_elems = 0;
  size_t part_need = 0;
  bool dry = false;
  double* red = nullptr;
  int* status = nullptr;
  int64_t uj_lo = 0, uj_hi = 0;
  double* h_stage = nullptr;
  size_t h_stage_elems = 0;
  vpm::Shape pinned[2][2][3];
  int64_t pinned_chunk[2][2][3];   // source chunk length pinned by vpm_set_tile (0: planner)
  std::vector<vpm::GraphEntry> graphs;
  int64_t fail_after = 0;
  std::string err;
  vpm::BatchPlan* bp = nullptr;   // set when the context backs a vpm_batch
  int order = VPM_ORDER_AUTO;     // vpm_set_particle_order
  vpm::FmmWork* fmm = nullptr;    // treecode workspace (allocated on first use)
  vpm::SortWork* sortw = nullptr; // Morton order of the direct pair passes (large fields)
  double* srt = nullptr;          // Morton-ordered inputs: X3 Γ3 σ1 v3 w3 (13 rows of ld)
  double* sout = nullptr;         // Morton-ordered outputs: U3 J9 DJ9 or ζ sums (21 rows of ld)
  float4* rec = nullptr;          // packed source records, 3 per particle (FP32 U/J passes)
  unsigned int* coh = nullptr;    // compact 32-particle blocks at the last packing
  double* ffv = nullptr;          // bound particles (X3 Γ3 σ1) and M (6) rows, ffv_cap apart
  int64_t ffv_cap = 0;
  int64_t launches = 0;           // kernels enqueued (graph replays add their kernel count)
  int64_t step_launches = 0;      // kernels of one captured step (counted while enqueuing)
  // Per-particle values the method carries but does not use: volume and
  // circulation rows (FLOWVPM's get_vol / get_circulation).
  double *vol = nullptr, *circ = nullptr;
  // Static (source-only) particles: a device flag per particle, its host copy
  // for particles [0, n), and one past the last free particle.  When the
  // static particles are exactly the tail [n - n_static, n) the update
  // kernels run over [0, n - n_static) without reading the flags.
  uint8_t* stat = nullptr;
  std::vector<uint8_t> hstat;
  int64_t last_free = 0;
};

// True when the static particles are exactly the tail of the field.
inline bool static_tail(const vpm_ctx* c) { return c->last_free == c->n - c->n_static; }

// Pair pass of a context over targets [t0, t1) of its own particles (queue form
// when the context backs a batch).
cudaError_t ctx_pair(vpm_ctx* c, int pass, int kernel, int prec, int64_t t0, int64_t t1,
                     double scale, const double* vs, double* u, double* j,
                     const double* ws = nullptr, double* dj = nullptr);
// Build (or rebuild for another kernel/precision) the batch queue.
int batch_plan(vpm_ctx* c, int kernel, int precision);
// Host transfer helpers of capi.cu, reused by batches.
int ctx_validate_host(vpm_ctx* c, int64_t n, const double* X, int64_t sx, const double* G,
                      int64_t sg, const double* S, int64_t ss);
int ctx_upload(vpm_ctx* c, int64_t i0, int64_t n, const double* X, int64_t sx, const double* G,
               int64_t sg, const double* S, int64_t ss);
// Static flags of particles [0, n) from a host array (nonzero = static); the
// particles must already be on the device.
int ctx_set_static_flags(vpm_ctx* c, const uint8_t* flags, int64_t n);
int ctx_download_rows(vpm_ctx* c, const double* dev, int rows, int64_t i0, int64_t n, double* out,
                      int64_t stride);
int ctx_prepare_scratch(vpm_ctx* c, int kernel, int precision);
