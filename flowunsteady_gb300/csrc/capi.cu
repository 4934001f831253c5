// capi.cu — host side of libvpmgpu.so: contexts, transfers, work planning,
// time stepping with CUDA graphs, diagnostics, autotuning.  The C ABI is
// declared in include/vpm_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "capi_internal.h"

using namespace vpm;

namespace vpm {

thread_local std::string g_last_error;

int set_error(std::string* slot, int code, const std::string& msg) {
  if (slot) *slot = msg;
  g_last_error = msg;
  return code;
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// --------------------------------------------------------- shape choices --
namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, int>, Shape> g_tune;  // (device, pass, kernel, prec, bucket)

int size_bucket(int64_t n) {
  int b = 0;
  while ((int64_t(1) << (b + 1)) <= n && b < 40) ++b;
  return b;
}
}  // namespace

// Untuned shapes.  The ζ passes do ~15 instructions of pair work per source
// against a fixed per-source cost, so on large fields they take more targets
// per thread; on small ones the smaller tiles give more target tiles to spread.
Shape default_shape(int pass, int precision, int64_t n) {
  if (precision == VPM_PREC_FP64) return Shape{128, 1};
  if (pass & 1) return n >= 32768 ? Shape{128, 4} : Shape{128, 2};
  // U/J and U/J + DJ, compensated: 4 targets per thread once the grid fills
  // the GPU evenly (N = 262,144: 74.8 -> 73.9 ms for U/J, 110 -> 104 ms for a
  // dynamic-SFS evaluation).
  return (precision == VPM_PREC_FP32C && n >= 196608) ? Shape{128, 4} : Shape{128, 2};
}

Shape lookup_shape(int device, int pass, int kernel, int precision, int64_t n,
                   const Shape* pinned) {
  if (pinned && pinned->block > 0) return *pinned;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  // Only the plain passes are tuned: the α-derivative passes carry about twice
  // the registers and keep their default shapes.
  auto it = g_tune.find(std::make_tuple(device, pass, kernel, precision, size_bucket(n)));
  if (it != g_tune.end()) return it->second;
  return default_shape(pass, precision, n);
}

int shape_bucket(int64_t n) { return size_bucket(n); }

void store_shape(int device, int pass, int kernel, int precision, int64_t n, Shape s) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[std::make_tuple(device, pass, kernel, precision, size_bucket(n))] = s;
}

int resident_ctas(int device, int pass, int kernel, int precision, Shape s, int num_sms) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int, int>, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_tuple(device, pass, kernel, precision, s.block, s.tpt);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int per = pair_ctas_per_sm(pass, kernel, precision, s);
  // A failed occupancy query or SM count leaves at least one resident CTA;
  // only a successful answer is cached.
  int r = std::max(1, per) * std::max(1, num_sms);
  if (per > 0 && num_sms > 0) cache[key] = r;
  return r;
}

// Source split: choose the number of source chunks so that the grid of
// n_tb x n_chunk items fills whole waves of resident CTAs, keeping chunks at
// least two tiles long and preferring fewer chunks at equal efficiency.
int plan_chunks(int64_t n_tb, int64_t ns, int block, int resident, int64_t* chunk_out,
                int max_chunks) {
  int best_c = 1;
  int64_t best_chunk = std::max<int64_t>(ns, 1);
  double best = -1.0;
  resident = std::max(resident, 1);
  const int cmax = max_chunks > 0 ? std::min(max_chunks, 128) : 128;
  for (int c = 1; c <= cmax; ++c) {
    int64_t chunk = round_up(std::max<int64_t>(ceil_div(ns, c), 1), block);
    if (c > 1 && chunk < 2 * block) break;
    const int cc = int(std::max<int64_t>(ceil_div(ns, chunk), 1));
    const int64_t items = n_tb * cc;
    const int64_t waves = ceil_div(items, resident);
    const double eff = double(items) / double(waves * resident);
    const double score = eff - 0.003 * cc;
    if (score > best + 1e-12) {
      best = score;
      best_c = cc;
      best_chunk = chunk;
    }
  }
  *chunk_out = best_chunk;
  return best_c;
}

// Clusters of `cluster` CTAs of a shape resident at once (cached per device).
int active_clusters(int device, int pass, int kernel, int precision, Shape s, int cluster) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int, int, int>, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_tuple(device, pass, kernel, precision, s.block, s.tpt, cluster);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  const int n = pair_max_active_clusters(pass, kernel, precision, s, cluster);
  cache[key] = n;
  return n;
}

int fused_reduce_mode() {
  static const int mode = [] {
    const char* v = std::getenv("VPM_FUSED_REDUCE");
    if (!v || !v[0]) return -1;
    return v[0] == '0' ? 0 : 1;
  }();
  return mode;
}

int cluster_mode() {
  static const int mode = [] {
    const char* v = std::getenv("VPM_CLUSTER");
    return (v && v[0] && v[0] != '0') ? 1 : 0;
  }();
  return mode;
}

// Largest cluster of the split-source form (16 needs the non-portable size).
constexpr int kMaxCluster = 16;

// Split-source clusters for an FP32C pass of n_tb target tiles over ns
// sources: the cluster size (1 = none fits) whose clusters fill whole waves
// best, with its chunk length and wave efficiency score (as plan_chunks').
// Measured on GB300 against partial slots (helical wake, Gaussian-erf, CUDA
// events): 7,600 particles 0.206 against 0.177 ms, 65,536 5.64 against 5.17 ms,
// 262,144 76.8 against 73.5 ms, although the clusters write no partial sums
// (DRAM writes of the pass: 0 against 50 MB at 131,072).  So partial slots are
// the default and clusters are taken only with VPM_CLUSTER=1.
static int plan_cluster(int device, const PairCall& pc, Shape sh, int64_t n_tb,
                        int64_t* chunk_out, double* score_out) {
  int best_nc = 1;
  double best = -1.0;
  for (int nc = 2; nc <= kMaxCluster; ++nc) {
    const int64_t chunk = round_up(std::max<int64_t>(ceil_div(pc.ns, nc), 1), sh.block);
    if (chunk < 2 * sh.block) break;
    if (ceil_div(pc.ns, chunk) != nc) continue;   // exactly nc non-empty chunks
    const int slots = active_clusters(device, pc.pass, pc.kernel, pc.prec, sh, nc);
    if (slots <= 0) continue;
    const int64_t waves = ceil_div(n_tb, slots);
    const double score = double(n_tb) / double(waves * slots) - 0.003 * nc;
    if (score > best + 1e-12) {
      best = score;
      best_nc = nc;
      *chunk_out = chunk;
    }
  }
  *score_out = best;
  return best_nc;
}

// Waves of work items a pass is split into: with fewer target tiles than
// resident CTAs, and with more.
constexpr int kSmallWaves = 8;
constexpr int kLargeWaves = 64;
constexpr int64_t kLargeField = 131072;

// Plan and enqueue one pair pass.  `need_part` (elements) is raised to what
// the launch needs; when dry, nothing is launched.  A split source range goes
// through partial slots summed by a reduction launch, or by the last CTA of
// each target tile (the fused form: plain U/J passes of large fields, or any
// split pass with VPM_FUSED_REDUCE=1), or (FP32C, single field, VPM_CLUSTER=1)
// through thread-block clusters that sum on chip.
// Measured on GB300 with FP32C (fused against a reduction launch):
// - U/J at N = 7,600: 0.324 against 0.150 ms; one CTA summing a tile's ~120
//   chunks is a serial tail;
// - U/J at 65,536: 5.15-5.25 against 5.12-5.13 ms;
// - U/J at 262,144: 70.46 against 70.63 ms (Gaussian-erf), with DRAM traffic
//   of 203 MB instead of 1.8 GB + 1.8 GB;
// - SFS evaluations at 262,144, fusing every pass: 0.2-0.6 % slower.
cudaError_t run_pair(const PairCall& pc, int device, int num_sms, const Shape* pinned,
                     double* part, int64_t ldp, size_t part_elems, size_t* need_part, bool dry,
                     cudaStream_t st, PairPlan* plan_out) {
  const int64_t nt = pc.t1 - pc.t0;
  if (nt <= 0) return cudaSuccess;
  const Shape sh = lookup_shape(device, pc.pass, pc.kernel, pc.prec, pc.ns, pinned);
  const int64_t TB = int64_t(sh.block) * sh.tpt;
  const int64_t n_tb = ceil_div(nt, TB);
  const int resident = resident_ctas(device, pc.pass, pc.kernel, pc.prec, sh, num_sms);
  int64_t chunk = 0;
  int n_chunk = plan_chunks(n_tb, pc.ns, sh.block, resident, &chunk, 0);
  int cluster = 1;
  if (pc.prec == VPM_PREC_FP32C && n_chunk > 1 && cluster_mode() == 1) {
    int64_t cchunk = 0;
    double cscore = -1.0;
    const int nc = plan_cluster(device, pc, sh, n_tb, &cchunk, &cscore);
    if (nc > 1) {
      cluster = nc;
      n_chunk = nc;
      chunk = cchunk;
    }
  }
  // Fewer target tiles than one wave: split the sources into about eight
  // waves of work items.  The items' costs differ (close pairs take the
  // general form), and more, shorter CTAs let the block scheduler balance
  // them; one wave of equal-length items waits for its slowest.  Measured
  // (helical wake and the two rings, FP32C U/J, 128x2, pass and reduction):
  // N = 7,600 170.9 -> 152.5 µs, 20,000 729.6 -> 620.2 µs, 40,000 2,100 ->
  // 2,010 µs, 65,536 5,182 -> 5,136 µs, 131,072 unchanged.  The ζ and
  // α-derivative passes took it too once their reductions summed float pairs
  // and the items ran near chunks first (they had kept one wave of items
  // before): a ring step 0.567 -> 0.541 ms (analytic ∂/∂σ), an analytic SFS
  // evaluation at 20,000 / 40,000 / 65,536 particles 1.09 / 3.51 / 7.74 ->
  // 1.02 / 3.27 / 7.06 ms; four waves for them measured in between, two
  // slower.
  // With a wave of tiles or more, every pass is split still finer, about
  // kLargeWaves waves of items: measured at N = 262,144 (128x4) the plain U/J
  // pass took 74.4 ms with whole waves of whole tiles (only the last wave
  // split), 71.8 / 71.0 / 70.6 ms with 16,384 / 8,192 / 4,096-source chunks,
  // and at N = 1,048,576 1,125 ms against 1,084-1,088 ms with 131,072 to
  // 16,384; an SFS evaluation at 262,144 84.3 -> 82.4 ms (prescribed C_d) and
  // 103.4 -> 99.2 ms (dynamic, analytic ∂/∂σ).  The partial sums this writes
  // (15 values per target and chunk for U/J) and the reduction reads back
  // cost about 0.7 ms of DRAM time per U/J pass at 262,144.
  // Every pass of a field of kLargeField sources or more takes the finer split
  // too: the ζ pass at 262,144 (128x4, fewer tiles than its resident CTAs)
  // measured 1.7 ms faster with 4,608-source chunks.
  const bool large = n_tb >= resident || pc.ns >= kLargeField;
  if (cluster <= 1 && pc.chunk <= 0) {
    const int waves = large ? kLargeWaves : kSmallWaves;
    const int64_t cc = ceil_div(int64_t(waves) * resident, n_tb);
    chunk = round_up(std::max<int64_t>(ceil_div(pc.ns, cc), 1), sh.block);
    n_chunk = int(std::max<int64_t>(ceil_div(pc.ns, chunk), 1));
  }
  if (cluster <= 1 && pc.chunk > 0) {   // pinned by vpm_set_tile: whole source tiles
    chunk = round_up(std::max<int64_t>(pc.chunk, sh.block), sh.block);
    n_chunk = int(std::max<int64_t>(ceil_div(pc.ns, chunk), 1));
  }
  if (cluster <= 1 && pc.max_chunks > 0 && n_chunk > pc.max_chunks)
    n_chunk = plan_chunks(n_tb, pc.ns, sh.block, resident, &chunk, pc.max_chunks);
  PairPlan plan;
  plan.shape = sh;
  plan.n_tb = n_tb;
  plan.n_chunk = n_chunk;
  plan.chunk = chunk;
  plan.cluster = cluster;
  const int fmode = fused_reduce_mode();
  plan.fused = plan.slots() > 1 && (fmode == 1 || (fmode < 0 && large && pc.pass == PASS_UJ));
  const int nv = nval_of(pc.pass);
  const size_t slot_elems = plan.slots() > 1 ? size_t(plan.slots()) * nv * size_t(ldp) : 0;
  // One 32-bit counter per target tile after the slots (two per double).
  const size_t need = slot_elems + (plan.fused ? size_t((n_tb + 1) / 2) : 0);
  if (need_part) *need_part = std::max(*need_part, need);
  if (plan_out) *plan_out = plan;
  if (dry) return cudaSuccess;
  if (need > part_elems) return cudaErrorMemoryAllocation;
  PairArgs a;
  std::memset(&a, 0, sizeof(a));
  a.xs = pc.xs; a.gs = pc.gs; a.ss = pc.ss; a.vs = pc.vs; a.ws = pc.ws; a.lds = pc.lds;
  a.xt = pc.xt; a.ldt = pc.ldt;
  a.sigma_scale = pc.sigma_scale;
  a.dj = pc.dj;
  a.t_off = pc.t0; a.nt = nt; a.ns = pc.ns; a.chunk = chunk;
  a.n_tb = int(n_tb); a.n_chunk = n_chunk;
  a.items = nullptr; a.n_items = 0; a.counter = nullptr;
  a.u = pc.u; a.j = pc.j; a.ldo = pc.ldo;
  a.part = part; a.ldp = ldp;
  a.status = pc.status;
  a.rec = pc.rec;
  a.tma = (pc.rec && !tma_disabled()) ? 1 : 0;
  a.far = farfield_enabled() ? 1 : 0;
  a.coh = pc.coh;
  a.coh_blocks = ceil_div(pc.ns, 32);
  a.cluster = cluster;
  a.tile_done = nullptr;
  cudaError_t e = cudaSuccess;
  if (plan.fused) {
    a.tile_done = reinterpret_cast<unsigned int*>(part + slot_elems);
    e = cudaMemsetAsync(a.tile_done, 0, size_t(n_tb) * sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
  }
  e = launch_pair(pc.pass, pc.kernel, pc.prec, sh, a, int(n_tb * n_chunk), st);
  if (e != cudaSuccess) return e;
  if (plan.slots() > 1 && !plan.fused) {
    e = launch_reduce(pc.pass, pc.kernel, pc.prec, part, ldp, nullptr, nullptr, 0, n_chunk, pc.t0, pc.t1,
                      pc.u, pc.j, pc.dj, pc.ldo, st);
  }
  return e;
}

// Below this size the far-field classification neither pays nor costs
// measurably, and the coherence count (a memset and atomics per pass) is
// left out: the classification then stays on.
bool coherence_counted(int64_t n) { return n >= 65536; }

bool tma_disabled() {
  static const bool off = [] {
    const char* v = std::getenv("VPM_NO_TMA");
    return v && v[0] && v[0] != '0';
  }();
  return off;
}

bool farfield_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("VPM_NO_FARFIELD");
    return !(v && v[0] && v[0] != '0');
  }();
  return on;
}

}  // namespace vpm

// ====================================================================== ctx ==

namespace {

int ctx_fail(vpm_ctx* c, int code, const std::string& msg) {
  return set_error(c ? &c->err : nullptr, code, msg);
}

int cuda_fail(vpm_ctx* c, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return ctx_fail(c, VPM_ERR_CUDA, buf);
}

#define CTX_CK(c, call)                                        \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return cuda_fail((c), e_, #call);  \
  } while (0)

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

int check_inject(vpm_ctx* c) {
  if (c->fail_after > 0 && --c->fail_after == 0)
    return ctx_fail(c, VPM_ERR_INJECTED, "fault injection: launch refused by the debug hook");
  return VPM_OK;
}

int ensure_stage(vpm_ctx* c, size_t elems) {
  if (elems <= c->h_stage_elems) return VPM_OK;
  if (c->h_stage) cudaFreeHost(c->h_stage);
  c->h_stage = nullptr;
  c->h_stage_elems = 0;
  CTX_CK(c, cudaMallocHost(&c->h_stage, elems * sizeof(double)));
  c->h_stage_elems = elems;
  return VPM_OK;
}

int ensure_part(vpm_ctx* c, size_t elems) {
  if (elems <= c->part_elems) return VPM_OK;
  if (c->part) cudaFree(c->part);
  c->part = nullptr;
  c->part_elems = 0;
  cudaError_t e = cudaMalloc(&c->part, elems * sizeof(double));
  if (e != cudaSuccess) return ctx_fail(c, VPM_ERR_NOMEM, "cannot allocate pair-pass scratch");
  c->part_elems = elems;
  return VPM_OK;
}

int ensure_test_filter(vpm_ctx* c) {
  if (c->Ut) return VPM_OK;
  const size_t ld = size_t(c->ld);
  if (cudaMalloc(&c->Ut, 15 * ld * sizeof(double)) != cudaSuccess)
    return ctx_fail(c, VPM_ERR_NOMEM, "cannot allocate test-filter buffers");
  c->Jt = c->Ut + 3 * ld;
  c->Et = c->Jt + 9 * ld;
  return VPM_OK;
}

// The host-side loops over particles (validation, AoS <-> SoA staging) run on
// all host threads from this many particles on.
constexpr int64_t kHostParallelMin = 16384;

// Host strided AoS -> pinned SoA staging -> device rows [i0, i0+n).  New
// particles get volume 0, circulation 1, empty SFS memory and the static flag
// is_static.
int upload(vpm_ctx* c, int64_t i0, int64_t n, const double* X, int64_t sx, const double* G,
           int64_t sg, const double* S, int64_t ss, int is_static) {
  if (n == 0) return VPM_OK;
  int rc = ensure_stage(c, size_t(9) * n);
  if (rc) return rc;
  double* h = c->h_stage;
#pragma omp parallel for schedule(static) if (n >= kHostParallelMin)
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      h[k * n + i] = X[i * sx + k];
      h[(3 + k) * n + i] = G[i * sg + k];
    }
    h[6 * n + i] = S[i * ss];
    h[7 * n + i] = 0.0;
    h[8 * n + i] = 1.0;
  }
  const size_t w = size_t(n) * sizeof(double), dp = size_t(c->ld) * sizeof(double);
  CTX_CK(c, cudaMemcpy2DAsync(c->X + i0, dp, h, w, w, 3, cudaMemcpyHostToDevice, c->st));
  CTX_CK(c, cudaMemcpy2DAsync(c->G + i0, dp, h + 3 * n, w, w, 3, cudaMemcpyHostToDevice, c->st));
  CTX_CK(c, cudaMemcpyAsync(c->S + i0, h + 6 * n, w, cudaMemcpyHostToDevice, c->st));
  CTX_CK(c, cudaMemcpyAsync(c->vol + i0, h + 7 * n, w, cudaMemcpyHostToDevice, c->st));
  CTX_CK(c, cudaMemcpyAsync(c->circ + i0, h + 8 * n, w, cudaMemcpyHostToDevice, c->st));
  CTX_CK(c, cudaMemsetAsync(c->stat + i0, is_static ? 1 : 0, size_t(n), c->st));
  // Fresh particles start with empty SFS memory.
  CTX_CK(c, cudaMemset2DAsync(c->C + i0, dp, 0, w, 3, c->st));
  CTX_CK(c, cudaStreamSynchronize(c->st));
  return VPM_OK;
}

// The particles the O(N) update kernels visit, and the flags they test: the
// free prefix [0, n - n_static) without flags when the static particles form
// the tail, else every particle with its flag.
void update_range(const vpm_ctx* c, int64_t* nv, const uint8_t** stat) {
  if (static_tail(c)) {
    *nv = c->n - c->n_static;
    *stat = nullptr;
  } else {
    *nv = c->n;
    *stat = c->stat;
  }
}

// Host bookkeeping of the static flags after particles [n0, n1) were added.
void note_added(vpm_ctx* c, int64_t n0, int64_t n1, bool is_static) {
  c->hstat.resize(size_t(n1), 0);
  for (int64_t i = n0; i < n1; ++i) c->hstat[size_t(i)] = is_static ? 1 : 0;
  if (is_static) c->n_static += n1 - n0;
  else if (n1 > n0) c->last_free = n1;
}

int validate_host(vpm_ctx* c, int64_t n, const double* X, int64_t sx, const double* G, int64_t sg,
                  const double* S, int64_t ss) {
  if (n < 0) return ctx_fail(c, VPM_ERR_INVALID, "negative particle count");
  if (n == 0) return VPM_OK;
  if (!X || !G || !S) return ctx_fail(c, VPM_ERR_INVALID, "null particle array");
  if (sx < 3 || sg < 3 || ss < 1) return ctx_fail(c, VPM_ERR_INVALID, "stride too small");
  // A parallel scan for any bad value; only then the ordered scan below names
  // the first one.
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad) if (n >= kHostParallelMin)
  for (int64_t i = 0; i < n; ++i) {
    const double s = S[i * ss];
    bool ok = std::isfinite(s) && s > 0.0;
    for (int k = 0; k < 3; ++k) ok = ok && std::isfinite(X[i * sx + k]) && std::isfinite(G[i * sg + k]);
    bad |= ok ? 0 : 1;
  }
  if (!bad) return VPM_OK;
  for (int64_t i = 0; i < n; ++i) {
    const double s = S[i * ss];
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(X[i * sx + k]) || !std::isfinite(G[i * sg + k]))
        return ctx_fail(c, VPM_ERR_NONFINITE, "non-finite position or strength in input");
    if (!std::isfinite(s)) return ctx_fail(c, VPM_ERR_NONFINITE, "non-finite core size in input");
    if (!(s > 0.0)) return ctx_fail(c, VPM_ERR_INVALID, "core size must be positive");
  }
  return VPM_OK;
}

// Download rows [i0, i0+n) of `rows` consecutive device rows (ld apart) into
// the host array out[i*stride + k].
int download_rows(vpm_ctx* c, const double* dev, int rows, int64_t i0, int64_t n, double* out,
                  int64_t stride) {
  if (!out || n == 0) return VPM_OK;
  if (stride < rows) return ctx_fail(c, VPM_ERR_INVALID, "stride too small");
  int rc = ensure_stage(c, size_t(rows) * n);
  if (rc) return rc;
  const size_t w = size_t(n) * sizeof(double), sp = size_t(c->ld) * sizeof(double);
  CTX_CK(c, cudaMemcpy2DAsync(c->h_stage, w, dev + i0, sp, w, rows, cudaMemcpyDeviceToHost, c->st));
  CTX_CK(c, cudaStreamSynchronize(c->st));
  const double* h = c->h_stage;
#pragma omp parallel for schedule(static) if (n >= kHostParallelMin)
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < rows; ++k) out[i * stride + k] = h[k * n + i];
  return VPM_OK;
}

bool valid_kernel(int k) { return k == VPM_KERNEL_WINCKELMANS || k == VPM_KERNEL_GAUSSIANERF; }
bool valid_prec(int p) { return p == VPM_PREC_FP64 || p == VPM_PREC_FP32 || p == VPM_PREC_FP32C; }

int validate_scheme(vpm_ctx* c, const vpm_scheme* s) {
  if (!s) return ctx_fail(c, VPM_ERR_INVALID, "null scheme");
  if (!valid_kernel(s->kernel)) return ctx_fail(c, VPM_ERR_INVALID, "unknown kernel");
  if (!valid_prec(s->precision)) return ctx_fail(c, VPM_ERR_INVALID, "unknown precision");
  if (s->integration != VPM_INTEGRATION_EULER && s->integration != VPM_INTEGRATION_RK3)
    return ctx_fail(c, VPM_ERR_INVALID, "unknown integration scheme");
  if (s->sfs != VPM_SFS_NONE && s->sfs != VPM_SFS_DYNAMIC && s->sfs != VPM_SFS_CONSTANT)
    return ctx_fail(c, VPM_ERR_INVALID, "unknown SFS model");
  if (s->relaxation != VPM_RELAX_NONE && s->relaxation != VPM_RELAX_PEDRIZZETTI)
    return ctx_fail(c, VPM_ERR_INVALID, "unknown relaxation scheme");
  if (!(s->nu >= 0.0) || !std::isfinite(s->nu)) return ctx_fail(c, VPM_ERR_INVALID, "bad viscosity");
  // Core spreading is only compatible with the Gaussian basis
  // (FLOWUnsteady checks kernel/viscous compatibility, src/FLOWUnsteady_simulation.jl:308-314).
  if (s->nu > 0.0 && s->kernel != VPM_KERNEL_GAUSSIANERF)
    return ctx_fail(c, VPM_ERR_UNSUPPORTED,
                    "core spreading requires the Gaussian-erf kernel");
  if (s->sfs == VPM_SFS_DYNAMIC && !(s->sfs_alpha > 0.0 && s->sfs_alpha != 1.0))
    return ctx_fail(c, VPM_ERR_INVALID, "dynamic SFS needs 0 < alpha != 1");
  if (!(1.0 + 3.0 * s->f != 0.0)) return ctx_fail(c, VPM_ERR_INVALID, "bad formulation f");
  if (s->uj_method != VPM_UJ_DIRECT && s->uj_method != VPM_UJ_TREE)
    return ctx_fail(c, VPM_ERR_INVALID, "unknown U/J method");
  if (s->uj_method == VPM_UJ_TREE) {
    if (!fmm_order_supported(s->fmm.p))
      return ctx_fail(c, VPM_ERR_UNSUPPORTED, "expansion order not compiled (2, 4, 6)");
    if (s->fmm.ncrit < 1 || !(s->fmm.theta > 0.0 && s->fmm.theta < 1.0) ||
        !(s->fmm.sigma_factor >= 0.0))
      return ctx_fail(c, VPM_ERR_INVALID, "treecode settings out of range");
    if (!fmm_local_order_supported(s->fmm.local_order))
      return ctx_fail(c, VPM_ERR_UNSUPPORTED, "local expansion order not compiled (0, 7)");
  }
  return VPM_OK;
}

}  // namespace

// Enqueue the pair pass of one context (targets [t0,t1) of its own particles).
// Large fields and batches are evaluated along a Morton curve: a full-range
// pair pass sorts the particles by the Morton code of their position
// (each field of a batch in its own cube and its own index range), gathers the
// state (and the ζ passes' v, w) into that order, runs the same pair pass there
// and scatters its outputs back.  Warps' targets and staged source blocks are
// then compact whatever the caller's particle order, so that the far-field
// forms of the Gaussian-erf kernel apply (uniform 262,144-particle box with the
// scalar FP32 routines: 114 → 88 ms).  Only the summation order changes;
// vpm_set_particle_order(VPM_ORDER_CALLER) keeps the caller's order for one
// context, VPM_NO_SORT=1 everywhere.
static bool sort_disabled() {
  static const bool off = [] {
    const char* v = std::getenv("VPM_NO_SORT");
    return v && v[0] && v[0] != '0';
  }();
  return off;
}

static bool sorted_pass(const vpm_ctx* c, int64_t t0, int64_t t1) {
  return !sort_disabled() && c->order == VPM_ORDER_AUTO && !c->bp && t0 == 0 && t1 == c->n &&
         c->n >= 65536;
}

static bool sorted_batch(const vpm_ctx* c) {
  return !sort_disabled() && c->order == VPM_ORDER_AUTO;
}

// Scratch of the sorted passes (allocated while planning, before any capture):
// c->srt rows 0-2 X, 3-5 Γ, 6 σ, 7-9 v, 10-12 w; c->sout rows 0-2 U (or the ζ
// sums), 3-11 J, 12-20 DJ.
static cudaError_t sort_scratch(vpm_ctx* c, int nfields) {
  cudaError_t e = sort_reserve(c->sortw, c->cap, nfields);
  if (e == cudaSuccess && !c->srt) e = cudaMalloc(&c->srt, 13 * size_t(c->ld) * sizeof(double));
  if (e == cudaSuccess && !c->sout) e = cudaMalloc(&c->sout, 21 * size_t(c->ld) * sizeof(double));
  return e;
}

static cudaError_t gather_inputs(vpm_ctx* c, const int* perm, const double* vs, const double* ws) {
  const int64_t n = c->n, ld = c->ld;
  cudaError_t e = launch_gather_rows(n, 3, perm, c->X, ld, c->srt, ld, c->st);
  if (e == cudaSuccess) e = launch_gather_rows(n, 3, perm, c->G, ld, c->srt + 3 * ld, ld, c->st);
  if (e == cudaSuccess) e = launch_gather_rows(n, 1, perm, c->S, ld, c->srt + 6 * ld, ld, c->st);
  if (e == cudaSuccess && vs) e = launch_gather_rows(n, 3, perm, vs, ld, c->srt + 7 * ld, ld, c->st);
  if (e == cudaSuccess && ws) e = launch_gather_rows(n, 3, perm, ws, ld, c->srt + 10 * ld, ld, c->st);
  c->launches += 3 + (vs ? 1 : 0) + (ws ? 1 : 0);
  return e;
}

static cudaError_t scatter_outputs(vpm_ctx* c, int pass, const int* perm, double* u, double* j,
                                   double* dj) {
  const int64_t n = c->n, ld = c->ld;
  if (pass == PASS_UJ || pass == PASS_UJD) {
    cudaError_t e = launch_scatter_rows(n, 3, perm, c->sout, ld, u, ld, c->st);
    if (e == cudaSuccess) e = launch_scatter_rows(n, 9, perm, c->sout + 3 * ld, ld, j, ld, c->st);
    if (e == cudaSuccess && dj)
      e = launch_scatter_rows(n, 9, perm, c->sout + 12 * ld, ld, dj, ld, c->st);
    c->launches += dj ? 3 : 2;
    return e;
  }
  c->launches += 1;
  return launch_scatter_rows(n, nval_of(pass), perm, c->sout, ld, u, ld, c->st);
}

static cudaError_t ctx_pair_sorted(vpm_ctx* c, int pass, int kernel, int prec, double scale,
                                   const double* vs, double* u, double* j, const double* ws,
                                   double* dj) {
  const int64_t n = c->n, ld = c->ld;
  const bool uj = pass == PASS_UJ || pass == PASS_UJD;
  const bool recs = prec != VPM_PREC_FP64;   // FP32 passes read packed records
  cudaError_t e = cudaSuccess;
  const int* perm = nullptr;
  if (c->dry) {
    e = sort_scratch(c, 1);
    if (e != cudaSuccess) return e;
  } else {
    if (!c->sortw || !c->srt || !c->sout) return cudaErrorInvalidValue;
    e = sort_order(c->sortw, n, c->X, ld, c->st, &perm);
    if (e == cudaSuccess) e = gather_inputs(c, perm, vs, ws);
    if (e == cudaSuccess && recs && uj)
      e = launch_pack_sources(kernel, n, c->srt, c->srt + 3 * ld, c->srt + 6 * ld, ld, scale,
                              c->rec, nullptr, c->st);
    else if (e == cudaSuccess && recs)
      e = launch_pack_zeta_sources(kernel, pass == PASS_ZETAD, n, c->srt, c->srt + 3 * ld,
                                   c->srt + 6 * ld, vs ? c->srt + 7 * ld : nullptr,
                                   ws ? c->srt + 10 * ld : nullptr, ld, scale, c->rec, c->st);
    if (e != cudaSuccess) return e;
    c->launches += 3 + (recs ? 1 : 0);
  }
  PairCall pc;
  pc.pass = pass; pc.kernel = kernel; pc.prec = prec;
  pc.t0 = 0; pc.t1 = n; pc.ns = n;
  pc.xs = c->srt; pc.gs = c->srt + 3 * ld; pc.ss = c->srt + 6 * ld; pc.lds = ld;
  pc.vs = vs ? c->srt + 7 * ld : nullptr;
  pc.ws = ws ? c->srt + 10 * ld : nullptr;
  pc.xt = c->srt; pc.ldt = ld;
  pc.sigma_scale = scale;
  pc.u = c->sout; pc.j = uj ? c->sout + 3 * ld : nullptr; pc.dj = dj ? c->sout + 12 * ld : nullptr;
  pc.ldo = ld;
  pc.status = c->status;
  pc.coh = nullptr;
  if (recs) pc.rec = c->rec;
  const Shape* pinned = &c->pinned[pass & 1][kernel][prec];
  pc.chunk = c->pinned_chunk[pass & 1][kernel][prec];
  PairPlan plan;
  e = run_pair(pc, c->device, c->num_sms, pinned, c->part, ld, c->part_elems, &c->part_need,
               c->dry, c->st, &plan);
  if (c->dry || e != cudaSuccess) return e;
  c->launches += plan.launches();
  return scatter_outputs(c, pass, perm, u, j, dj);
}

cudaError_t ctx_pair(vpm_ctx* c, int pass, int kernel, int prec, int64_t t0, int64_t t1,
                     double scale, const double* vs, double* u, double* j, const double* ws,
                     double* dj) {
  if (c->bp) {
    // Batch: one persistent launch over the flattened (field, target tile,
    // source chunk) queue, then the fixed-order reduction of split fields.
    BatchPlan* bp = c->bp;
    if (bp->kernel != kernel || bp->precision != prec) {
      if (c->dry) {
        if (batch_plan(c, kernel, prec) != VPM_OK) return cudaErrorInvalidValue;
      } else {
        return cudaErrorInvalidValue;  // plans are built outside capture (dry pass)
      }
    }
    const int nv = nval_of(pass);
    const size_t need = bp->max_chunks > 1 ? size_t(bp->max_chunks) * nv * size_t(c->ld) : 0;
    c->part_need = std::max(c->part_need, need);
    const bool srt = sorted_batch(c);
    if (c->dry) return srt ? sort_scratch(c, bp->nfields) : cudaSuccess;
    if (need > c->part_elems) return cudaErrorMemoryAllocation;
    const int64_t ld = c->ld;
    const double *xs = c->X, *gs = c->G, *ss = c->S, *vq = vs, *wq = ws;
    double *uo = u, *jo = j, *djo = dj;
    const int* perm = nullptr;
    cudaError_t e = cudaSuccess;
    if (srt) {
      if (!c->sortw || !c->srt || !c->sout) return cudaErrorInvalidValue;
      e = sort_order_fields(c->sortw, c->n, c->X, ld, bp->d_foff, bp->nfields, c->st, &perm);
      if (e == cudaSuccess) e = gather_inputs(c, perm, vs, ws);
      if (e != cudaSuccess) return e;
      c->launches += 2;
      xs = c->srt; gs = c->srt + 3 * ld; ss = c->srt + 6 * ld;
      vq = vs ? c->srt + 7 * ld : nullptr;
      wq = ws ? c->srt + 10 * ld : nullptr;
      uo = c->sout; jo = j ? c->sout + 3 * ld : nullptr; djo = dj ? c->sout + 12 * ld : nullptr;
    }
    unsigned int* coh = !srt && coherence_counted(c->n) ? c->coh : nullptr;
    e = cudaMemsetAsync(bp->d_counter, 0, kMaxBatchGroups * sizeof(unsigned int), c->st);
    if (e != cudaSuccess) return e;
    PairArgs a;
    std::memset(&a, 0, sizeof(a));
    a.xs = xs; a.gs = gs; a.ss = ss; a.vs = vq; a.ws = wq; a.lds = ld;
    a.xt = xs; a.ldt = ld;
    a.sigma_scale = scale;
    a.dj = djo;
    a.items = bp->d_items; a.n_items = bp->n_items;
    a.u = uo; a.j = jo; a.ldo = ld;
    a.part = c->part; a.ldp = ld;
    a.far = farfield_enabled() ? 1 : 0;
    a.coh = coh;
    a.coh_blocks = ceil_div(c->n, 32);
    if (prec != VPM_PREC_FP64 && (pass == PASS_UJ || pass == PASS_UJD)) {
      e = launch_pack_sources(kernel, c->n, xs, gs, ss, ld, scale, c->rec, coh, c->st);
      if (e != cudaSuccess) return e;
      c->launches += 1;
      a.rec = c->rec;
      a.tma = tma_disabled() ? 0 : 1;
    } else if (prec != VPM_PREC_FP64) {
      e = launch_pack_zeta_sources(kernel, pass == PASS_ZETAD, c->n, xs, gs, ss, vq, wq, ld, scale,
                                   c->rec, c->st);
      if (e != cudaSuccess) return e;
      c->launches += 1;
      a.rec = c->rec;
    }
    // One persistent launch per tile-shape group, each over its own queue.
    for (size_t g = 0; g < bp->groups.size(); ++g) {
      const BatchGroup& grp = bp->groups[g];
      PairArgs ag = a;
      ag.items = bp->d_items + grp.first;
      ag.n_items = grp.n_items;
      ag.counter = bp->d_counter + g;
      e = launch_pair(pass, kernel, prec, grp.shape, ag, std::min(grp.resident, grp.n_items),
                      c->st);
      if (e != cudaSuccess) return e;
      c->launches += 1;
    }
    if (bp->max_chunks > 1) {
      e = launch_reduce(pass, kernel, prec, c->part, ld, bp->d_foff, bp->d_fchunks, bp->nfields, 0,
                        0, c->n, uo, jo, djo, ld, c->st);
      c->launches += 1;
      if (e != cudaSuccess) return e;
    }
    return srt ? scatter_outputs(c, pass, perm, u, j, dj) : cudaSuccess;
  }
  if (sorted_pass(c, t0, t1))
    return ctx_pair_sorted(c, pass, kernel, prec, scale, vs, u, j, ws, dj);
  PairCall pc;
  pc.pass = pass; pc.kernel = kernel; pc.prec = prec;
  pc.t0 = t0; pc.t1 = t1; pc.ns = c->n;
  pc.xs = c->X; pc.gs = c->G; pc.ss = c->S; pc.vs = vs; pc.lds = c->ld;
  pc.xt = c->X; pc.ldt = c->ld;
  pc.sigma_scale = scale;
  pc.u = u; pc.j = j; pc.ldo = c->ld;
  pc.ws = ws; pc.dj = dj;
  pc.status = c->status;
  pc.coh = coherence_counted(c->n) ? c->coh : nullptr;
  if (prec != VPM_PREC_FP64 && (pass == PASS_UJ || pass == PASS_UJD)) {
    if (!c->dry) {
      cudaError_t e = launch_pack_sources(kernel, c->n, c->X, c->G, c->S, c->ld, scale, c->rec,
                                          pc.coh ? c->coh : nullptr, c->st);
      if (e != cudaSuccess) return e;
      c->launches += 1;
    }
    pc.rec = c->rec;
  } else if (prec != VPM_PREC_FP64) {
    if (!c->dry) {
      cudaError_t e = launch_pack_zeta_sources(kernel, pass == PASS_ZETAD, c->n, c->X, c->G, c->S,
                                               vs, ws, c->ld, scale, c->rec, c->st);
      if (e != cudaSuccess) return e;
      c->launches += 1;
    }
    pc.rec = c->rec;
  }
  const Shape* pinned = &c->pinned[pass & 1][kernel][prec];  // D passes share their plain pass's pin
  pc.chunk = c->pinned_chunk[pass & 1][kernel][prec];
  PairPlan plan;
  cudaError_t e = run_pair(pc, c->device, c->num_sms, pinned, c->part, c->ld, c->part_elems,
                           &c->part_need, c->dry, c->st, &plan);
  if (!c->dry && e == cudaSuccess && t1 > t0) c->launches += plan.launches();
  return e;
}

#define ENQ(c, call)                                        \
  do {                                                      \
    if (!(c)->dry) {                                        \
      cudaError_t e_ = (call);                              \
      if (e_ != cudaSuccess) return e_;                     \
      (c)->launches += 1;                                   \
    }                                                       \
  } while (0)
#define ENQP(c, call)                                       \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return e_;                       \
  } while (0)

// The plain U/J pass of a step at σ (U, J of every particle): the direct pair
// pass, or the treecode when the scheme asks for it (synchronous; nothing to
// plan in the dry pass).
static cudaError_t uj_pass(vpm_ctx* c, const vpm_scheme* s, bool direct = false) {
  if (s->uj_method == VPM_UJ_TREE && !direct) {
    if (c->dry) return cudaSuccess;
    const char* why = nullptr;
    cudaError_t e = fmm_eval(c, s->kernel, s->precision, s->fmm.p, s->fmm.ncrit, s->fmm.theta,
                             s->fmm.sigma_factor, s->fmm.local_order, nullptr, &why);
    if (e != cudaSuccess && why) c->err = why;
    return e;
  }
  return ctx_pair(c, PASS_UJ, s->kernel, s->precision, 0, c->n, 1.0, nullptr, c->U, c->J);
}

// The SFS passes can follow the treecode for Gaussian-erf cores in FP32: DJ,
// ζ and Dζ vanish beyond the near field (7.1σ) to FP32 significance.
static bool tree_sfs(const vpm_scheme* s) {
  return s->uj_method == VPM_UJ_TREE && s->kernel == VPM_KERNEL_GAUSSIANERF &&
         s->precision != VPM_PREC_FP64 && s->fmm.sigma_factor >= 7.1;
}

// U/J + DJ of the analytic dynamic SFS (stage 1).
static cudaError_t ujd_pass(vpm_ctx* c, const vpm_scheme* s) {
  if (tree_sfs(s)) {
    if (c->dry) return cudaSuccess;
    const char* why = nullptr;
    cudaError_t e = fmm_eval(c, s->kernel, s->precision, s->fmm.p, s->fmm.ncrit, s->fmm.theta,
                             s->fmm.sigma_factor, s->fmm.local_order, c->Jt, &why);
    if (e != cudaSuccess && why) c->err = why;
    return e;
  }
  return ctx_pair(c, PASS_UJD, s->kernel, s->precision, 0, c->n, 1.0, nullptr, c->U, c->J,
                  nullptr, c->Jt);
}

// ζ sums at σ (PASS_ZETA, or PASS_ZETAD with w rows) into c->raw.
static cudaError_t zeta_pass(vpm_ctx* c, const vpm_scheme* s, bool d, const double* W,
                             bool direct = false) {
  if (tree_sfs(s) && !direct) {
    if (c->dry) return cudaSuccess;
    const char* why = nullptr;
    cudaError_t e = fmm_zeta(c, d, c->V, W, c->raw, &why);
    if (e != cudaSuccess && why) c->err = why;
    return e;
  }
  if (d) return ctx_pair(c, PASS_ZETAD, s->kernel, s->precision, 0, c->n, 1.0, c->V, c->raw,
                         nullptr, W, nullptr);
  return ctx_pair(c, PASS_ZETA, s->kernel, s->precision, 0, c->n, 1.0, c->V, c->raw, nullptr);
}

// U/J and the SFS pass of a stage (the first stage of a dynamic step also
// computes C_d).  In the analytic form the first stage runs the α-derivative
// passes (U/J + DJ, then ζ + Dζ) instead of separate passes at σ and ασ.
static cudaError_t enqueue_uj_sfs(vpm_ctx* c, const vpm_scheme* s, int stage) {
  const int64_t n = c->n, ld = c->ld;
  int64_t nf = 0;
  const uint8_t* stat = nullptr;
  update_range(c, &nf, &stat);
  const int K = s->kernel, P = s->precision;
  const bool sfs = s->sfs != VPM_SFS_NONE;
  const bool dyn0 = s->sfs == VPM_SFS_DYNAMIC && stage == 0;
  const bool analytic = dyn0 && (s->sfs_flags & VPM_SFS_ANALYTIC_DSIGMA);
  double* W = c->V + 3 * ld;
  if (analytic) {
    // Jt := DJ, Et := DE.
    ENQP(c, ujd_pass(c, s));
    ENQ(c, launch_stretch_vw(n, ld, c->J, c->Jt, c->G, s->transposed, c->V, W, c->st));
    ENQP(c, zeta_pass(c, s, true, W));
    ENQ(c, launch_estr_finish_d(n, ld, c->raw, c->J, c->Jt, s->transposed, c->E, c->Et, c->st));
  } else {
    // The finite-difference C_d takes the difference of the passes at σ and at
    // ασ (amplifying errors by 1/(1-α)): both come from the direct sum.
    const bool fd = dyn0 && !analytic;
    ENQP(c, uj_pass(c, s, fd));
    if (sfs) {
      ENQ(c, launch_stretch_v(n, ld, c->J, c->G, s->transposed, c->V, c->st));
      ENQP(c, zeta_pass(c, s, false, nullptr, fd));
      ENQ(c, launch_estr_finish(n, ld, c->raw, c->J, s->transposed, c->E, c->st));
    }
  }
  if (s->sfs == VPM_SFS_CONSTANT) {
    ENQ(c, launch_sfs_constant(nf, stat, s->sfs_Cd, c->C, c->st));
  } else if (dyn0) {
    const double al = s->sfs_alpha;
    if (!analytic) {
      ENQP(c, ctx_pair(c, PASS_UJ, K, P, 0, n, al, nullptr, c->Ut, c->Jt));
      ENQ(c, launch_stretch_v(n, ld, c->Jt, c->G, s->transposed, c->V, c->st));
      ENQP(c, ctx_pair(c, PASS_ZETA, K, P, 0, n, al, c->V, c->raw, nullptr));
      ENQ(c, launch_estr_finish(n, ld, c->raw, c->Jt, s->transposed, c->Et, c->st));
    }
    SfsParams sp;
    sp.alpha = al; sp.rlxf = s->sfs_rlxf; sp.minC = s->sfs_minC; sp.maxC = s->sfs_maxC;
    sp.zeta0 = zeta0_of(K); sp.inv_zeta0 = 1.0 / sp.zeta0; sp.transposed = s->transposed;
    sp.force_positive = (s->sfs_flags & VPM_SFS_FORCE_POSITIVE) ? 1 : 0;
    sp.analytic = analytic ? 1 : 0;
    ENQ(c, launch_sfs_dynamic(nf, stat, ld, c->G, c->S, c->J, c->Jt, c->E, c->Et, c->C, sp,
                              c->st));
  }
  return cudaSuccess;
}

// One stage of a step: U/J, SFS, fused update.
static cudaError_t enqueue_stage(vpm_ctx* c, const vpm_scheme* s, double dt, double a, double b,
                                 int stage) {
  const int64_t ld = c->ld;
  int64_t nf = 0;
  const uint8_t* stat = nullptr;
  update_range(c, &nf, &stat);
  const int K = s->kernel;
  const bool sfs = s->sfs != VPM_SFS_NONE;
  ENQP(c, enqueue_uj_sfs(c, s, stage));
  UpdateParams up;
  up.a = a; up.b = b; up.dt = dt;
  up.uinf0 = s->uinf[0]; up.uinf1 = s->uinf[1]; up.uinf2 = s->uinf[2];
  up.zs = (s->f + s->g) / (1.0 + 3.0 * s->f);
  up.ze = s->f / (1.0 + 3.0 * s->f);
  up.zeta0 = zeta0_of(K);
  up.inv_zeta0 = 1.0 / up.zeta0;
  up.nu = s->nu;
  up.transposed = s->transposed;
  up.sfs = sfs ? 1 : 0;
  up.clip_backscatter = (sfs && (s->sfs_flags & VPM_SFS_CLIP_BACKSCATTER)) ? 1 : 0;
  ENQ(c, launch_rk_update(nf, stat, ld, c->X, c->G, c->S, c->U, c->J, c->E, c->C, c->Q, up,
                          c->status, c->st));
  return cudaSuccess;
}

static cudaError_t enqueue_step(vpm_ctx* c, const vpm_scheme* s, double dt, bool relax) {
  static const double A[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
  static const double B[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
  if (s->integration == VPM_INTEGRATION_RK3) {
    for (int st = 0; st < 3; ++st) ENQP(c, enqueue_stage(c, s, dt, A[st], B[st], st));
  } else {
    ENQP(c, enqueue_stage(c, s, dt, 0.0, 1.0, 0));
  }
  if (relax) {
    // Relaxation after the step on a fresh U/J (vpm.pedrizzetti).
    ENQP(c, uj_pass(c, s));
    int64_t nf = 0;
    const uint8_t* stat = nullptr;
    update_range(c, &nf, &stat);
    ENQ(c, launch_relax(nf, stat, c->ld, c->J, c->G, s->relax_factor, c->st));
  }
  return cudaSuccess;
}

static int check_status(vpm_ctx* c) {
  int st = 0;
  CTX_CK(c, cudaMemcpyAsync(&st, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CTX_CK(c, cudaStreamSynchronize(c->st));
  if (st) {
    CTX_CK(c, cudaMemsetAsync(c->status, 0, sizeof(int), c->st));
    CTX_CK(c, cudaStreamSynchronize(c->st));
    if (st & STATUS_NONFINITE)
      return ctx_fail(c, VPM_ERR_NONFINITE, "non-finite particle state after the update");
    if (st & STATUS_TIMEOUT)
      return ctx_fail(c, VPM_ERR_CUDA, "a source-tile copy did not complete in time");
    return ctx_fail(c, VPM_ERR_CUDA, "device status word set");
  }
  return VPM_OK;
}

int ctx_validate_host(vpm_ctx* c, int64_t n, const double* X, int64_t sx, const double* G,
                      int64_t sg, const double* S, int64_t ss) {
  return validate_host(c, n, X, sx, G, sg, S, ss);
}
int ctx_upload(vpm_ctx* c, int64_t i0, int64_t n, const double* X, int64_t sx, const double* G,
               int64_t sg, const double* S, int64_t ss) {
  DeviceGuard dg(c->device);
  return upload(c, i0, n, X, sx, G, sg, S, ss, 0);
}
int ctx_set_static_flags(vpm_ctx* c, const uint8_t* flags, int64_t n) {
  if (n != c->n) return ctx_fail(c, VPM_ERR_INVALID, "static flags must cover every particle");
  DeviceGuard dg(c->device);
  c->hstat.assign(flags, flags + n);
  c->n_static = 0;
  c->last_free = 0;
  for (int64_t i = 0; i < n; ++i) {
    c->hstat[size_t(i)] = c->hstat[size_t(i)] ? 1 : 0;
    if (c->hstat[size_t(i)]) ++c->n_static;
    else c->last_free = i + 1;
  }
  if (n > 0) {
    CTX_CK(c, cudaMemcpyAsync(c->stat, c->hstat.data(), size_t(n), cudaMemcpyHostToDevice, c->st));
    CTX_CK(c, cudaStreamSynchronize(c->st));
  }
  return VPM_OK;
}
int ctx_download_rows(vpm_ctx* c, const double* dev, int rows, int64_t i0, int64_t n, double* out,
                      int64_t stride) {
  DeviceGuard dg(c->device);
  return download_rows(c, dev, rows, i0, n, out, stride);
}
// Size the pair-pass scratch for a UJ pass over all particles.
int ctx_prepare_scratch(vpm_ctx* c, int kernel, int precision) {
  DeviceGuard dg(c->device);
  c->dry = true;
  c->part_need = 0;
  cudaError_t e = ctx_pair(c, PASS_UJ, kernel, precision, 0, c->n, 1.0, nullptr, c->U, c->J);
  c->dry = false;
  if (e != cudaSuccess) return cuda_fail(c, e, "planning a pair pass");
  return ensure_part(c, c->part_need);
}

// ===================================================================== C ABI ==
extern "C" {

void vpm_scheme_default(vpm_scheme* s) {
  if (!s) return;
  std::memset(s, 0, sizeof(*s));
  s->kernel = VPM_KERNEL_GAUSSIANERF;
  s->precision = VPM_PREC_FP32C;
  s->integration = VPM_INTEGRATION_RK3;
  s->uj_method = VPM_UJ_DIRECT;
  vpm_fmm_default(&s->fmm);
  s->transposed = 1;
  s->f = 0.0;
  s->g = 0.2;
  s->nu = 0.0;
  s->sfs = VPM_SFS_NONE;
  s->sfs_flags = VPM_SFS_CLIP_BACKSCATTER;
  s->sfs_alpha = 0.999;
  s->sfs_rlxf = 1.0;
  s->sfs_minC = 0.0;
  s->sfs_maxC = 1.0;
  s->sfs_Cd = 0.0;
  s->relaxation = VPM_RELAX_NONE;
  s->relax_nsteps = 1;
  s->relax_factor = 0.3;
}

int vpm_ctx_create(int device, int64_t capacity, vpm_ctx** out) {
  if (!out) return set_error(nullptr, VPM_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (capacity < 1) return set_error(nullptr, VPM_ERR_INVALID, "capacity must be >= 1");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return set_error(nullptr, VPM_ERR_CUDA, "no such CUDA device");
  DeviceGuard dg(device);
  vpm_ctx* c = new vpm_ctx();
  c->device = device;
  c->cap = capacity;
  c->ld = round_up(capacity, 32);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  std::memset(c->pinned, 0, sizeof(c->pinned));
  std::memset(c->pinned_chunk, 0, sizeof(c->pinned_chunk));
  const size_t ld = size_t(c->ld);
  // State + evaluation rows: X3 G3 S1 C3 Q8 U3 J9 E3 V6 raw12 vol1 circ1 = 53 rows.
  const size_t rows = 53;
  if (cudaMalloc(&c->base, rows * ld * sizeof(double)) != cudaSuccess) {
    delete c;
    return set_error(nullptr, VPM_ERR_NOMEM, "cannot allocate the particle field");
  }
  double* p = c->base;
  c->X = p; p += 3 * ld;
  c->G = p; p += 3 * ld;
  c->S = p; p += ld;
  c->C = p; p += 3 * ld;
  c->Q = p; p += 8 * ld;
  c->U = p; p += 3 * ld;
  c->J = p; p += 9 * ld;
  c->E = p; p += 3 * ld;
  c->V = p; p += 6 * ld;      // v rows 0..2, w rows 3..5
  c->raw = p; p += 12 * ld;   // raw ζ sums (12 rows for the α-derivative pass)
  c->vol = p; p += ld;
  c->circ = p; p += ld;
  cudaError_t e = cudaMemset(c->base, 0, rows * ld * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&c->stat, size_t(c->ld));
  if (e == cudaSuccess) e = cudaMemset(c->stat, 0, size_t(c->ld));
  // Packed source records: 3 float4 per particle for the U/J passes, up to 5 for ζ.
  if (e == cudaSuccess) e = cudaMalloc(&c->rec, 5 * ld * sizeof(float4));
  // Until the first packing the particle order counts as coherent.
  if (e == cudaSuccess) e = cudaMalloc(&c->coh, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(c->coh, 0xff, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&c->status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->status, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&c->red, (size_t(kRedBlocks) + 1) * kDiagSlots * sizeof(double));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    vpm_ctx_destroy(c);
    return set_error(nullptr, VPM_ERR_CUDA, std::string("context set-up: ") + cudaGetErrorString(e));
  }
  c->st = c->own;
  *out = c;
  return VPM_OK;
}

int vpm_ctx_destroy(vpm_ctx* c) {
  if (!c) return VPM_OK;
  DeviceGuard dg(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  if (c->own) cudaStreamDestroy(c->own);
  cudaFree(c->base);
  cudaFree(c->Ut);
  cudaFree(c->part);
  cudaFree(c->ffv);
  cudaFree(c->rec);
  cudaFree(c->coh);
  vpm::fmm_free(c->fmm);
  vpm::sort_free(c->sortw);
  cudaFree(c->srt);
  cudaFree(c->sout);
  cudaFree(c->status);
  cudaFree(c->red);
  cudaFree(c->stat);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  delete c;
  return VPM_OK;
}

int vpm_last_error(const vpm_ctx* c, char* buf, int64_t len) {
  if (!buf || len <= 0) return VPM_ERR_INVALID;
  const std::string& m = c ? c->err : g_last_error;
  std::snprintf(buf, size_t(len), "%s", m.c_str());
  return VPM_OK;
}

int vpm_ctx_set_stream(vpm_ctx* c, void* stream) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  DeviceGuard dg(c->device);
  cudaStreamSynchronize(c->st);
  c->st = stream ? static_cast<cudaStream_t>(stream) : c->own;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  return VPM_OK;
}

int vpm_get_time(const vpm_ctx* c, double* t, int64_t* nt) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (t) *t = c->t;
  if (nt) *nt = c->nt;
  return VPM_OK;
}

int vpm_set_time(vpm_ctx* c, double t, int64_t nt) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  c->t = t;
  c->nt = nt;
  return VPM_OK;
}

int vpm_set_particles(vpm_ctx* c, int64_t n, const double* X, int64_t sx, const double* G,
                      int64_t sg, const double* S, int64_t ss) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n > c->cap) return ctx_fail(c, VPM_ERR_CAPACITY, "particle count above capacity");
  int rc = validate_host(c, n, X, sx, G, sg, S, ss);
  if (rc) return rc;
  DeviceGuard dg(c->device);
  rc = upload(c, 0, n, X, sx, G, sg, S, ss, 0);
  if (rc) return rc;
  c->n = n;
  c->n_static = 0;
  c->last_free = 0;
  c->hstat.clear();
  note_added(c, 0, n, false);
  c->uj_lo = c->uj_hi = 0;
  return VPM_OK;
}

int vpm_append(vpm_ctx* c, int64_t n, const double* X, int64_t sx, const double* G, int64_t sg,
               const double* S, int64_t ss, int is_static) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n < 0) return ctx_fail(c, VPM_ERR_INVALID, "negative particle count");
  if (c->n + n > c->cap) return ctx_fail(c, VPM_ERR_CAPACITY, "particle count above capacity");
  int rc = validate_host(c, n, X, sx, G, sg, S, ss);
  if (rc) return rc;
  DeviceGuard dg(c->device);
  rc = upload(c, c->n, n, X, sx, G, sg, S, ss, is_static);
  if (rc) return rc;
  note_added(c, c->n, c->n + n, is_static != 0);
  c->n += n;
  return VPM_OK;
}

int vpm_truncate(vpm_ctx* c, int64_t n) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n < 0 || n > c->n) return ctx_fail(c, VPM_ERR_INVALID, "truncate beyond particle count");
  for (int64_t i = n; i < c->n; ++i) c->n_static -= c->hstat[size_t(i)];
  c->hstat.resize(size_t(n));
  if (c->last_free > n) {
    int64_t lf = n;
    while (lf > 0 && c->hstat[size_t(lf - 1)]) --lf;
    c->last_free = lf;
  }
  c->n = n;
  c->uj_hi = std::min(c->uj_hi, n);
  c->uj_lo = std::min(c->uj_lo, c->uj_hi);
  return VPM_OK;
}

int vpm_get_np(const vpm_ctx* c, int64_t* n, int64_t* n_static) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n) *n = c->n;
  if (n_static) *n_static = c->n_static;
  return VPM_OK;
}

int vpm_get_state(vpm_ctx* c, int64_t n, double* X, int64_t sx, double* G, int64_t sg, double* S,
                  int64_t ss) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n < 0 || n > c->n) return ctx_fail(c, VPM_ERR_INVALID, "range beyond particle count");
  DeviceGuard dg(c->device);
  int rc = download_rows(c, c->X, 3, 0, n, X, sx);
  if (!rc) rc = download_rows(c, c->G, 3, 0, n, G, sg);
  if (!rc) rc = download_rows(c, c->S, 1, 0, n, S, ss);
  return rc;
}

int vpm_get_sfs(vpm_ctx* c, int64_t n, double* C, int64_t sc, double* E, int64_t se) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n < 0 || n > c->n) return ctx_fail(c, VPM_ERR_INVALID, "range beyond particle count");
  DeviceGuard dg(c->device);
  int rc = download_rows(c, c->C, 3, 0, n, C, sc);
  if (!rc) rc = download_rows(c, c->E, 3, 0, n, E, se);
  return rc;
}

int vpm_set_attributes(vpm_ctx* c, int64_t i0, int64_t n, const double* vol, int64_t svol,
                       const double* circulation, int64_t scirc, const double* C, int64_t sc) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n < 0 || i0 < 0 || i0 + n > c->n) return ctx_fail(c, VPM_ERR_INVALID, "range beyond particle count");
  if ((vol && svol < 1) || (circulation && scirc < 1) || (C && sc < 3))
    return ctx_fail(c, VPM_ERR_INVALID, "stride too small");
  for (int64_t i = 0; i < n; ++i) {
    if ((vol && !std::isfinite(vol[i * svol])) ||
        (circulation && !std::isfinite(circulation[i * scirc])))
      return ctx_fail(c, VPM_ERR_NONFINITE, "non-finite particle attribute");
    for (int k = 0; C && k < 3; ++k)
      if (!std::isfinite(C[i * sc + k])) return ctx_fail(c, VPM_ERR_NONFINITE, "non-finite SFS memory");
  }
  if (n == 0) return VPM_OK;
  DeviceGuard dg(c->device);
  int rc = ensure_stage(c, size_t(5) * n);
  if (rc) return rc;
  double* h = c->h_stage;
  const size_t w = size_t(n) * sizeof(double), dp = size_t(c->ld) * sizeof(double);
  if (vol) {
    for (int64_t i = 0; i < n; ++i) h[i] = vol[i * svol];
    CTX_CK(c, cudaMemcpyAsync(c->vol + i0, h, w, cudaMemcpyHostToDevice, c->st));
  }
  if (circulation) {
    for (int64_t i = 0; i < n; ++i) h[n + i] = circulation[i * scirc];
    CTX_CK(c, cudaMemcpyAsync(c->circ + i0, h + n, w, cudaMemcpyHostToDevice, c->st));
  }
  if (C) {
    for (int64_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) h[(2 + k) * n + i] = C[i * sc + k];
    CTX_CK(c, cudaMemcpy2DAsync(c->C + i0, dp, h + 2 * n, w, w, 3, cudaMemcpyHostToDevice, c->st));
  }
  CTX_CK(c, cudaStreamSynchronize(c->st));
  return VPM_OK;
}

int vpm_get_attributes(vpm_ctx* c, int64_t i0, int64_t n, double* vol, int64_t svol,
                       double* circulation, int64_t scirc, int32_t* is_static) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n < 0 || i0 < 0 || i0 + n > c->n) return ctx_fail(c, VPM_ERR_INVALID, "range beyond particle count");
  DeviceGuard dg(c->device);
  int rc = download_rows(c, c->vol, 1, i0, n, vol, svol);
  if (!rc) rc = download_rows(c, c->circ, 1, i0, n, circulation, scirc);
  if (!rc && is_static)
    for (int64_t i = 0; i < n; ++i) is_static[i] = c->hstat[size_t(i0 + i)];
  return rc;
}

int vpm_eval_UJ_targets(vpm_ctx* c, int kernel, int precision, int64_t t0, int64_t t1) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!valid_kernel(kernel)) return ctx_fail(c, VPM_ERR_INVALID, "unknown kernel");
  if (!valid_prec(precision)) return ctx_fail(c, VPM_ERR_INVALID, "unknown precision");
  if (t0 < 0 || t1 < t0 || t1 > c->n) return ctx_fail(c, VPM_ERR_INVALID, "bad target range");
  int rc = check_inject(c);
  if (rc) return rc;
  DeviceGuard dg(c->device);
  c->dry = true;
  c->part_need = 0;
  ctx_pair(c, PASS_UJ, kernel, precision, t0, t1, 1.0, nullptr, c->U, c->J);
  c->dry = false;
  rc = ensure_part(c, c->part_need);
  if (rc) return rc;
  CTX_CK(c, ctx_pair(c, PASS_UJ, kernel, precision, t0, t1, 1.0, nullptr, c->U, c->J));
  c->uj_lo = t0;
  c->uj_hi = t1;
  return check_status(c);
}

int vpm_eval_UJ(vpm_ctx* c, int kernel, int precision) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  return vpm_eval_UJ_targets(c, kernel, precision, 0, c->n);
}

void vpm_fmm_default(vpm_fmm* f) {
  if (!f) return;
  f->p = 4;
  f->ncrit = 50;
  f->theta = 0.4;
  f->sigma_factor = 7.1;
  f->local_order = 7;
  f->reserved = 0;
}

int vpm_eval_UJ_fmm(vpm_ctx* c, int kernel, int precision, const vpm_fmm* f) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!f) return ctx_fail(c, VPM_ERR_INVALID, "null treecode settings");
  if (!valid_kernel(kernel) || !valid_prec(precision))
    return ctx_fail(c, VPM_ERR_INVALID, "unknown kernel or precision");
  if (!fmm_order_supported(f->p)) return ctx_fail(c, VPM_ERR_UNSUPPORTED, "expansion order not compiled (2, 4, 6)");
  if (f->ncrit < 1 || !(f->theta > 0.0 && f->theta < 1.0) || !(f->sigma_factor >= 0.0))
    return ctx_fail(c, VPM_ERR_INVALID, "treecode settings out of range");
  if (!fmm_local_order_supported(f->local_order))
    return ctx_fail(c, VPM_ERR_UNSUPPORTED, "local expansion order not compiled (0, 7)");
  int rc = check_inject(c);
  if (rc) return rc;
  DeviceGuard dg(c->device);
  const char* why = nullptr;
  cudaError_t e =
      fmm_eval(c, kernel, precision, f->p, f->ncrit, f->theta, f->sigma_factor, f->local_order,
               nullptr, &why);
  if (e == cudaErrorInvalidValue && why) return ctx_fail(c, VPM_ERR_CUDA, why);
  if (e != cudaSuccess)
    return cuda_fail(c, e, why ? (std::string("treecode evaluation, ") + why).c_str() : "treecode evaluation");
  c->uj_lo = 0;
  c->uj_hi = c->n;
  return VPM_OK;
}

int vpm_fmm_stats(const vpm_ctx* c, int64_t* out) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!out) return set_error(nullptr, VPM_ERR_INVALID, "null output");
  fmm_stats(c->fmm, out);
  return VPM_OK;
}

int vpm_get_UJ(vpm_ctx* c, int64_t i0, int64_t n, double* U, int64_t su, double* J, int64_t sj) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (n < 0 || i0 < 0) return ctx_fail(c, VPM_ERR_INVALID, "bad range");
  if (n > 0 && (i0 < c->uj_lo || i0 + n > c->uj_hi))
    return ctx_fail(c, VPM_ERR_STATE, "range not covered by the last U/J evaluation");
  DeviceGuard dg(c->device);
  int rc = download_rows(c, c->U, 3, i0, n, U, su);
  if (!rc) rc = download_rows(c, c->J, 9, i0, n, J, sj);
  return rc;
}

int vpm_eval_sfs(vpm_ctx* c, const vpm_scheme* s) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  int rc = validate_scheme(c, s);
  if (rc) return rc;
  if (s->sfs == VPM_SFS_NONE) return ctx_fail(c, VPM_ERR_INVALID, "scheme has no SFS model");
  rc = check_inject(c);
  if (rc) return rc;
  DeviceGuard dg(c->device);
  if (s->sfs == VPM_SFS_DYNAMIC && (rc = ensure_test_filter(c))) return rc;
  // The work of a step's first stage without the update: a dry pass sizes the
  // scratch, then the same sequence is enqueued for real.
  c->dry = true;
  c->part_need = 0;
  enqueue_uj_sfs(c, s, 0);
  c->dry = false;
  if ((rc = ensure_part(c, c->part_need))) return rc;
  CTX_CK(c, enqueue_uj_sfs(c, s, 0));
  if (s->sfs_flags & VPM_SFS_CLIP_BACKSCATTER) {
    // A step applies the backscatter clipping inside its update kernel; here
    // it is applied on its own, so C_d comes back as the SFS model leaves it.
    int64_t nf = 0;
    const uint8_t* stat = nullptr;
    update_range(c, &nf, &stat);
    CTX_CK(c, launch_sfs_clip(nf, stat, c->ld, c->G, c->E, c->C, c->st));
    c->launches += 1;
  }
  CTX_CK(c, cudaStreamSynchronize(c->st));
  c->uj_lo = 0;
  c->uj_hi = c->n;
  return VPM_OK;
}

int vpm_step(vpm_ctx* c, double dt, const vpm_scheme* s, int64_t nsteps, int use_graph) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  int rc = validate_scheme(c, s);
  if (rc) return rc;
  if (!std::isfinite(dt)) return ctx_fail(c, VPM_ERR_INVALID, "non-finite time step");
  if (nsteps < 0) return ctx_fail(c, VPM_ERR_INVALID, "negative step count");
  if (nsteps == 0 || c->n == 0) {
    c->t += dt * double(nsteps);
    c->nt += nsteps;
    return VPM_OK;
  }
  DeviceGuard dg(c->device);
  if (s->uj_method == VPM_UJ_TREE) use_graph = 0;   // the treecode reads sizes back on the host
  if (s->sfs == VPM_SFS_DYNAMIC && (rc = ensure_test_filter(c))) return rc;
  c->dry = true;
  c->part_need = 0;
  enqueue_step(c, s, dt, s->relaxation != VPM_RELAX_NONE);
  c->dry = false;
  if ((rc = ensure_part(c, c->part_need))) return rc;

  for (int64_t k = 0; k < nsteps; ++k) {
    if ((rc = check_inject(c))) return rc;
    const int64_t step_no = c->nt + 1;
    const bool relax = s->relaxation != VPM_RELAX_NONE && s->relax_nsteps >= 1 &&
                       step_no % s->relax_nsteps == 0;
    if (use_graph) {
      GraphKey key;
      key.n = c->n; key.n_static = c->n_static; key.dt = dt; key.relax = relax;
      key.mixed = static_tail(c) ? 0 : 1;
      key.scheme = *s;
      cudaGraphExec_t exec = nullptr;
      for (auto& g : c->graphs)
        if (std::memcmp(&g.key, &key, sizeof(key)) == 0) exec = g.exec;
      if (!exec) {
        cudaGraph_t graph = nullptr;
        CTX_CK(c, cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        const int64_t before = c->launches;
        cudaError_t e = enqueue_step(c, s, dt, relax);
        const int64_t per_step = c->launches - before;
        c->launches = before;
        cudaError_t e2 = cudaStreamEndCapture(c->st, &graph);
        if (e != cudaSuccess) {
          if (graph) cudaGraphDestroy(graph);
          return cuda_fail(c, e, "capturing a step");
        }
        CTX_CK(c, e2);
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CTX_CK(c, e);
        if (c->graphs.size() >= 8) {
          cudaGraphExecDestroy(c->graphs.front().exec);
          c->graphs.erase(c->graphs.begin());
        }
        GraphEntry ge;
        std::memset(&ge, 0, sizeof(ge));
        ge.key = key;
        ge.exec = exec;
        ge.kernels = per_step;
        c->graphs.push_back(ge);
      }
      int64_t nk = 0;
      for (auto& g : c->graphs)
        if (g.exec == exec) nk = g.kernels;
      CTX_CK(c, cudaGraphLaunch(exec, c->st));
      c->launches += nk;
    } else {
      CTX_CK(c, enqueue_step(c, s, dt, relax));
    }
    c->t += dt;
    c->nt += 1;
  }
  c->uj_lo = 0;
  c->uj_hi = c->n;
  return check_status(c);
}

int vpm_diagnostics(vpm_ctx* c, int kernel, int precision, double* out) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!out) return ctx_fail(c, VPM_ERR_INVALID, "null output");
  if (!valid_kernel(kernel) || !valid_prec(precision))
    return ctx_fail(c, VPM_ERR_INVALID, "unknown kernel or precision");
  int rc = check_inject(c);
  if (rc) return rc;
  DeviceGuard dg(c->device);
  const int64_t n = c->n, nfree = n - c->n_static;
  int64_t nf = 0;
  const uint8_t* stat = nullptr;
  update_range(c, &nf, &stat);
  for (int k = 0; k < VPM_DIAG_COUNT; ++k) out[k] = 0.0;
  if (n == 0) return VPM_OK;
  c->dry = true;
  c->part_need = 0;
  ctx_pair(c, PASS_ZETA, kernel, precision, 0, n, 1.0, nullptr, c->raw, nullptr);
  c->dry = false;
  if ((rc = ensure_part(c, c->part_need))) return rc;
  CTX_CK(c, ctx_pair(c, PASS_ZETA, kernel, precision, 0, n, 1.0, nullptr, c->raw, nullptr));
  double* partial = c->red;
  double* dout = c->red + size_t(kRedBlocks) * kDiagSlots;
  CTX_CK(c, launch_diagnostics(n, nf, stat, c->ld, c->X, c->G, c->S, c->C, c->raw, zeta0_of(kernel),
                               partial, dout, c->st));
  c->launches += 2;
  double v[kDiagSlots];
  CTX_CK(c, cudaMemcpyAsync(v, dout, sizeof v, cudaMemcpyDeviceToHost, c->st));
  CTX_CK(c, cudaStreamSynchronize(c->st));
  out[VPM_DIAG_ENSTROPHY] = v[DS_ENS];
  out[VPM_DIAG_IMPULSE_X] = v[DS_IX];
  out[VPM_DIAG_IMPULSE_Y] = v[DS_IY];
  out[VPM_DIAG_IMPULSE_Z] = v[DS_IZ];
  out[VPM_DIAG_GAMMA_X] = v[DS_GX];
  out[VPM_DIAG_GAMMA_Y] = v[DS_GY];
  out[VPM_DIAG_GAMMA_Z] = v[DS_GZ];
  if (v[DS_CCNT] > 0) {
    // Population moments of the nonzero C_d from the raw power sums.
    const double cnt = v[DS_CCNT];
    const double mean = v[DS_CSUM] / cnt;
    const double p2 = v[DS_CSUM2] / cnt, p3 = v[DS_CSUM3] / cnt, p4 = v[DS_CSUM4] / cnt;
    const double m2 = std::max(0.0, p2 - mean * mean);
    const double m3 = p3 - 3.0 * mean * p2 + 2.0 * mean * mean * mean;
    const double m4 = p4 - 4.0 * mean * p3 + 6.0 * mean * mean * p2 - 3.0 * mean * mean * mean * mean;
    out[VPM_DIAG_CD_MEAN] = mean;
    out[VPM_DIAG_CD_STD] = std::sqrt(m2);
    out[VPM_DIAG_CD_MIN] = v[DS_CMIN];
    out[VPM_DIAG_CD_MAX] = v[DS_CMAX];
    if (m2 > 0.0) {
      out[VPM_DIAG_CD_SKEW] = m3 / (m2 * std::sqrt(m2));
      out[VPM_DIAG_CD_KURT] = m4 / (m2 * m2) - 3.0;
    }
  }
  out[VPM_DIAG_CD_ZERO_RATIO] = nfree > 0 ? v[DS_CZERO] / double(nfree) : 0.0;
  out[VPM_DIAG_SIGMA_MEAN] = v[DS_SIG] / double(n);
  out[VPM_DIAG_NONFINITE] = v[DS_NONFIN];
  return VPM_OK;
}

int vpm_ffv_direct(vpm_ctx* c, int kernel, int64_t nb, const double* Xb, int64_t sxb,
                   const double* Gb, int64_t sgb, const double* Sb, int64_t ssb, double* M,
                   int64_t stride_m) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!valid_kernel(kernel)) return ctx_fail(c, VPM_ERR_INVALID, "unknown kernel");
  if (nb < 0) return ctx_fail(c, VPM_ERR_INVALID, "negative bound-particle count");
  if (nb == 0) return VPM_OK;
  if (!M || stride_m < 6) return ctx_fail(c, VPM_ERR_INVALID, "bad force output");
  int rc = validate_host(c, nb, Xb, sxb, Gb, sgb, Sb, ssb);
  if (rc) return rc;
  if ((rc = check_inject(c))) return rc;
  DeviceGuard dg(c->device);
  const int64_t ldb = round_up(nb, 32);
  if (ldb > c->ffv_cap) {
    cudaFree(c->ffv);
    c->ffv = nullptr;
    c->ffv_cap = 0;
    if (cudaMalloc(&c->ffv, 13 * size_t(ldb) * sizeof(double)) != cudaSuccess)
      return ctx_fail(c, VPM_ERR_NOMEM, "cannot allocate bound-particle buffers");
    c->ffv_cap = ldb;
  }
  const int64_t cap = c->ffv_cap;
  double* xb = c->ffv;
  double* gb = xb + 3 * cap;
  double* sb = gb + 3 * cap;
  double* md = sb + cap;
  int64_t chunk = 0;
  int n_chunk = 1;
  if ((rc = ensure_part(c, ffv_plan(nb, c->n, c->num_sms, &chunk, &n_chunk)))) return rc;
  if ((rc = ensure_stage(c, size_t(7) * nb))) return rc;
  double* h = c->h_stage;
  for (int64_t i = 0; i < nb; ++i) {
    for (int k = 0; k < 3; ++k) {
      h[k * nb + i] = Xb[i * sxb + k];
      h[(3 + k) * nb + i] = Gb[i * sgb + k];
    }
    h[6 * nb + i] = Sb[i * ssb];
  }
  const size_t w = size_t(nb) * sizeof(double), dp = size_t(cap) * sizeof(double);
  CTX_CK(c, cudaMemcpy2DAsync(xb, dp, h, w, w, 7, cudaMemcpyHostToDevice, c->st));
  CTX_CK(c, launch_ffv(kernel, nb, xb, gb, sb, cap, c->n, c->X, c->G, c->ld, c->part, md, cap,
                       c->num_sms, c->st));
  c->launches += n_chunk > 1 ? 2 : 1;
  CTX_CK(c, cudaStreamSynchronize(c->st));
  if ((rc = ensure_stage(c, size_t(6) * nb))) return rc;
  CTX_CK(c, cudaMemcpy2DAsync(c->h_stage, w, md, dp, w, 6, cudaMemcpyDeviceToHost, c->st));
  CTX_CK(c, cudaStreamSynchronize(c->st));
  for (int64_t i = 0; i < nb; ++i)
    for (int k = 0; k < 6; ++k) M[i * stride_m + k] = c->h_stage[k * nb + i];
  return VPM_OK;
}

int vpm_centroids(vpm_ctx* c, int nranges, const int64_t* starts, const int64_t* ends,
                  double* out) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (nranges < 0 || (nranges > 0 && (!starts || !ends || !out)))
    return ctx_fail(c, VPM_ERR_INVALID, "bad centroid ranges");
  DeviceGuard dg(c->device);
  double* partial = c->red;
  double* dout = c->red + size_t(kRedBlocks) * kDiagSlots;
  for (int r = 0; r < nranges; ++r) {
    if (starts[r] < 0 || ends[r] < starts[r] || ends[r] > c->n)
      return ctx_fail(c, VPM_ERR_INVALID, "centroid range beyond particle count");
    CTX_CK(c, launch_centroid(starts[r], ends[r], c->ld, c->X, c->G, partial, dout, c->st));
    double v[kDiagSlots];
    CTX_CK(c, cudaMemcpyAsync(v, dout, sizeof v, cudaMemcpyDeviceToHost, c->st));
    CTX_CK(c, cudaStreamSynchronize(c->st));
    for (int k = 0; k < 3; ++k) out[3 * r + k] = v[3] > 0 ? v[k] / v[3] : 0.0;
  }
  return VPM_OK;
}

int vpm_set_tile(vpm_ctx* c, int kernel, int precision, const vpm_tile* t) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!valid_kernel(kernel) || !valid_prec(precision))
    return ctx_fail(c, VPM_ERR_INVALID, "unknown kernel or precision");
  if (!t || t->block == 0) {  // unpin
    std::memset(&c->pinned[0][kernel][precision], 0, sizeof(Shape));
    std::memset(&c->pinned[1][kernel][precision], 0, sizeof(Shape));
    c->pinned_chunk[0][kernel][precision] = c->pinned_chunk[1][kernel][precision] = 0;
    return VPM_OK;
  }
  Shape s{t->block, t->tpt};
  if (!pair_shape_supported(precision, s))
    return ctx_fail(c, VPM_ERR_UNSUPPORTED, "tile shape not compiled for this precision");
  if (t->chunk < 0) return ctx_fail(c, VPM_ERR_INVALID, "negative source chunk length");
  c->pinned[0][kernel][precision] = s;
  c->pinned[1][kernel][precision] = s;
  c->pinned_chunk[0][kernel][precision] = c->pinned_chunk[1][kernel][precision] = t->chunk;
  return VPM_OK;
}

int vpm_set_particle_order(vpm_ctx* c, int mode) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (mode != VPM_ORDER_AUTO && mode != VPM_ORDER_CALLER)
    return ctx_fail(c, VPM_ERR_INVALID, "unknown particle order");
  if (mode != c->order) {
    DeviceGuard dg(c->device);
    cudaStreamSynchronize(c->st);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);   // captured for the old order
    c->graphs.clear();
    c->order = mode;
  }
  return VPM_OK;
}

// Time one pass of the context's particles with a given tile shape (best of 3).
static int time_pass(vpm_ctx* c, int pass, int kernel, int precision, Shape s, cudaEvent_t e0,
                     cudaEvent_t e1, float* out_ms) {
  const Shape saved = c->pinned[pass][kernel][precision];
  c->pinned[pass][kernel][precision] = s;
  auto enqueue = [&]() {
    return pass == PASS_UJ ? ctx_pair(c, PASS_UJ, kernel, precision, 0, c->n, 1.0, nullptr, c->U, c->J)
                           : ctx_pair(c, PASS_ZETA, kernel, precision, 0, c->n, 1.0, c->V, c->raw,
                                      nullptr);
  };
  c->dry = true;
  c->part_need = 0;
  enqueue();
  c->dry = false;
  int rc = ensure_part(c, c->part_need);
  if (rc) {
    c->pinned[pass][kernel][precision] = saved;
    return rc;
  }
  float best = 1e30f;
  cudaError_t e = enqueue();
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, c->st);
    e = enqueue();
    cudaEventRecord(e1, c->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    best = std::min(best, t);
  }
  c->pinned[pass][kernel][precision] = saved;
  if (e != cudaSuccess) return cuda_fail(c, e, "autotune launch");
  *out_ms = best;
  return VPM_OK;
}

// Pick the fastest compiled tile shape of the U/J pass and, separately, of the
// ζ pass for this size bucket; the choice is stored for every context on the
// device.
int vpm_autotune(vpm_ctx* c, int kernel, int precision, vpm_tile* chosen, double* ms) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!valid_kernel(kernel) || !valid_prec(precision))
    return ctx_fail(c, VPM_ERR_INVALID, "unknown kernel or precision");
  if (c->n == 0) return ctx_fail(c, VPM_ERR_STATE, "autotune needs particles");
  DeviceGuard dg(c->device);
  static const Shape cands[] = {{128, 2}, {128, 4}, {256, 2}, {128, 1}};
  cudaEvent_t e0, e1;
  CTX_CK(c, cudaEventCreate(&e0));
  CTX_CK(c, cudaEventCreate(&e1));
  Shape best[2] = {{0, 0}, {0, 0}};
  double best_ms[2] = {1e30, 1e30};
  int rc = VPM_OK;
  for (int pass = PASS_UJ; pass <= PASS_ZETA && rc == VPM_OK; ++pass) {
    for (const Shape& s : cands) {
      if (!pair_shape_supported(precision, s)) continue;
      float t = 0.f;
      rc = time_pass(c, pass, kernel, precision, s, e0, e1, &t);
      if (rc) break;
      if (t < best_ms[pass]) {
        best_ms[pass] = t;
        best[pass] = s;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (best[0].block == 0) return ctx_fail(c, VPM_ERR_UNSUPPORTED, "no tile shape compiled");
  store_shape(c->device, PASS_UJ, kernel, precision, c->n, best[0]);
  store_shape(c->device, PASS_ZETA, kernel, precision, c->n, best[1]);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  c->uj_lo = c->uj_hi = 0;   // U/J now hold timing runs of the last candidate
  if (chosen) {
    chosen->block = best[0].block;
    chosen->tpt = best[0].tpt;
    chosen->chunk = 0;
    chosen->reserved = best[1].block * 16 + best[1].tpt;   // ζ-pass shape, packed
  }
  if (ms) *ms = best_ms[0];
  return VPM_OK;
}

int vpm_debug_fail_after(vpm_ctx* c, int64_t k) {
  if (!c) return set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (k < 0) return ctx_fail(c, VPM_ERR_INVALID, "negative count");
  c->fail_after = k;
  return VPM_OK;
}

int vpm_get_launch_count(const vpm_ctx* c, int64_t* count) {
  if (!c || !count) return set_error(nullptr, VPM_ERR_INVALID, "null argument");
  *count = c->launches;
  return VPM_OK;
}

const char* vpm_build_info(void) {
  static char buf[160];
  std::snprintf(buf, sizeof buf, "libvpmgpu abi=%d arch=sm_103a nvcc=%d.%d", VPM_ABI_VERSION,
                __CUDACC_VER_MAJOR__, __CUDACC_VER_MINOR__);
  return buf;
}

}  // extern "C"
