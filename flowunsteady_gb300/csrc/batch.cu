// batch.cu — many independent particle fields of uneven size advanced together.
//
// The fields are concatenated in one context (field f owns particles
// [off_f, off_f + n_f)).  Every pair pass is one persistent launch over a
// flattened work queue of (field, target tile, source chunk) items, sorted by
// cost (largest first) and pulled from an atomic counter; fields split into
// several source chunks are summed afterwards in fixed order, so results do
// not depend on which CTA ran which item.  The O(N) update kernels run over
// all fields at once.  Each step of the batch is one CUDA graph replay.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace vpm;

struct vpm_batch {
  vpm_ctx* ctx = nullptr;
  BatchPlan plan;
  std::vector<char> set;   // field f uploaded
  std::string err;
};

namespace {

int bfail(vpm_batch* b, int code, const std::string& m) {
  return set_error(b ? &b->err : nullptr, code, m);
}

int from_ctx(vpm_batch* b, int rc) {
  if (rc != VPM_OK) b->err = b->ctx->err;
  return rc;
}

}  // namespace

// Items of the fields in `fields`, each field with its tile shape `shape[f]`,
// grouped by shape: within a group the source chunk length L is the smallest
// multiple of the block that keeps the group's queue near four items per
// resident CTA, and items are sorted by cost (largest first).  Writes the
// device queue, per-field chunk counts and groups into bp.
// Work items of a batch queue: the sources of a field are split into chunks of
// the shortest power-of-two length (in source tiles) for which the queue holds
// at most this many items per resident CTA.  Items of one field cost alike, but
// across fields and chunks they differ by orders of magnitude, and the
// persistent CTAs balance finer items better.  Measured on 48 fields of
// 2,302-120,610 particles (FP32C U/J pass): 4 items per CTA (whole source
// ranges) 93.7 ms, 16 90.0 ms, 32 89.4 ms, 64 89.1 ms; 32 bounds the partial
// sums at 8 chunks per field there.
constexpr int kBatchItemWaves = 32;

static int build_queue(vpm_ctx* c, int kernel, int precision, const std::vector<int>& fields,
                       const std::vector<Shape>& shape) {
  BatchPlan* bp = c->bp;
  const int nf = bp->nfields;
  std::vector<Shape> shapes;
  for (int f : fields) {
    bool seen = false;
    for (const Shape& s : shapes) seen = seen || (s.block == shape[f].block && s.tpt == shape[f].tpt);
    if (!seen) shapes.push_back(shape[f]);
  }
  if (int(shapes.size()) > kMaxBatchGroups)
    return set_error(&c->err, VPM_ERR_UNSUPPORTED, "too many tile shapes in one batch");
  std::vector<PairItem> items;
  std::vector<int32_t> fchunks(nf, 1);
  std::vector<BatchGroup> groups;
  int max_chunks = 1;
  for (const Shape& sh : shapes) {
    const int r_uj = resident_ctas(c->device, PASS_UJ, kernel, precision, sh, c->num_sms);
    const int r_z = resident_ctas(c->device, PASS_ZETA, kernel, precision, sh, c->num_sms);
    const int64_t TB = int64_t(sh.block) * sh.tpt;
    std::vector<int> mine;
    int64_t nmax = 1;
    for (int f : fields)
      if (shape[f].block == sh.block && shape[f].tpt == sh.tpt && bp->h_n[f] > 0) {
        mine.push_back(f);
        nmax = std::max(nmax, bp->h_n[f]);
      }
    auto count_items = [&](int64_t L) {
      int64_t cnt = 0;
      for (int f : mine) cnt += ceil_div(bp->h_n[f], TB) * ceil_div(bp->h_n[f], L);
      return cnt;
    };
    int64_t L = round_up(nmax, sh.block);
    for (int64_t cand = 2 * sh.block; cand < round_up(nmax, sh.block); cand *= 2) {
      if (count_items(cand) <= kBatchItemWaves * int64_t(r_uj)) {
        L = cand;
        break;
      }
    }
    BatchGroup g;
    g.shape = sh;
    g.first = int(items.size());
    g.resident = std::min(r_uj, r_z);
    for (int f : mine) {
      const int64_t n = bp->h_n[f], off = bp->h_off[f];
      const int64_t cf = ceil_div(n, L);
      fchunks[f] = int32_t(cf);
      max_chunks = std::max<int>(max_chunks, int(cf));
      for (int64_t t = 0; t < n; t += TB)
        for (int64_t ch = 0; ch < cf; ++ch) {
          PairItem it;
          it.t0 = off + t;
          it.t1 = off + std::min(n, t + TB);
          it.s0 = off + ch * L;
          it.s1 = off + std::min(n, (ch + 1) * L);
          it.slot = cf > 1 ? int32_t(ch) : -1;
          it.field = f;
          items.push_back(it);
        }
    }
    std::stable_sort(items.begin() + g.first, items.end(), [](const PairItem& a, const PairItem& b) {
      return (a.t1 - a.t0) * (a.s1 - a.s0) > (b.t1 - b.t0) * (b.s1 - b.s0);
    });
    g.n_items = int(items.size()) - g.first;
    if (g.n_items > 0) groups.push_back(g);
  }
  // The group with the most pair work launches first.
  auto work = [&](const BatchGroup& g) {
    double w = 0.0;
    for (int i = g.first; i < g.first + g.n_items; ++i)
      w += double(items[i].t1 - items[i].t0) * double(items[i].s1 - items[i].s0);
    return w;
  };
  std::stable_sort(groups.begin(), groups.end(),
                   [&](const BatchGroup& a, const BatchGroup& b) { return work(a) > work(b); });
  cudaFree(bp->d_items);
  bp->d_items = nullptr;
  if (!items.empty()) {
    if (cudaMalloc(&bp->d_items, items.size() * sizeof(PairItem)) != cudaSuccess)
      return set_error(&c->err, VPM_ERR_NOMEM, "cannot allocate the batch work queue");
    if (cudaMemcpy(bp->d_items, items.data(), items.size() * sizeof(PairItem),
                   cudaMemcpyHostToDevice) != cudaSuccess)
      return set_error(&c->err, VPM_ERR_CUDA, "cannot upload the batch work queue");
  }
  if (cudaMemcpy(bp->d_fchunks, fchunks.data(), nf * sizeof(int32_t), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return set_error(&c->err, VPM_ERR_CUDA, "cannot upload the batch chunk counts");
  bp->groups = groups;
  bp->n_items = int(items.size());
  bp->max_chunks = max_chunks;
  bp->h_shape = shape;
  return VPM_OK;
}

// Build the work queue for a kernel/precision: every field takes the tile
// shape of its size bucket (the autotuner's choice, or the default), so a
// batch makes one persistent launch per distinct shape.
int batch_plan(vpm_ctx* c, int kernel, int precision) {
  BatchPlan* bp = c->bp;
  const int nf = bp->nfields;
  std::vector<int> fields(nf);
  std::vector<Shape> shape(nf);
  const bool tuned = int(bp->h_tuned.size()) == nf && bp->tuned_kernel == kernel &&
                     bp->tuned_precision == precision;
  for (int f = 0; f < nf; ++f) {
    fields[f] = f;
    shape[f] = tuned ? bp->h_tuned[f]
                     : lookup_shape(c->device, PASS_UJ, kernel, precision,
                                    std::max<int64_t>(bp->h_n[f], 1),
                                    &c->pinned[PASS_UJ][kernel][precision]);
  }
  const int rc = build_queue(c, kernel, precision, fields, shape);
  if (rc != VPM_OK) return rc;
  bp->kernel = kernel;
  bp->precision = precision;
  return VPM_OK;
}

extern "C" {

int vpm_batch_create(int device, int nfields, const int64_t* n, vpm_batch** out) {
  if (!out) return set_error(nullptr, VPM_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (nfields < 1 || !n) return set_error(nullptr, VPM_ERR_INVALID, "need at least one field");
  int64_t total = 0;
  for (int f = 0; f < nfields; ++f) {
    if (n[f] < 0) return set_error(nullptr, VPM_ERR_INVALID, "negative field size");
    total += n[f];
  }
  vpm_batch* b = new vpm_batch();
  int rc = vpm_ctx_create(device, std::max<int64_t>(total, 1), &b->ctx);
  if (rc != VPM_OK) {
    delete b;
    return rc;
  }
  BatchPlan& bp = b->plan;
  bp.nfields = nfields;
  bp.h_n.assign(n, n + nfields);
  bp.h_off.resize(nfields);
  int64_t off = 0;
  for (int f = 0; f < nfields; ++f) {
    bp.h_off[f] = off;
    off += n[f];
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  cudaError_t e = cudaMalloc(&bp.d_foff, nfields * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&bp.d_fchunks, nfields * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&bp.d_counter, kMaxBatchGroups * sizeof(unsigned int));
  if (e == cudaSuccess)
    e = cudaMemcpy(bp.d_foff, bp.h_off.data(), nfields * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    vpm_batch_destroy(b);
    return set_error(nullptr, VPM_ERR_NOMEM, "cannot allocate the batch tables");
  }
  b->ctx->bp = &b->plan;
  b->ctx->n = total;
  b->set.assign(nfields, 0);
  *out = b;
  return VPM_OK;
}

int vpm_batch_destroy(vpm_batch* b) {
  if (!b) return VPM_OK;
  if (b->ctx) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->st);
    cudaFree(b->plan.d_items);
    cudaFree(b->plan.d_foff);
    cudaFree(b->plan.d_fchunks);
    cudaFree(b->plan.d_counter);
    cudaSetDevice(prev);
    b->ctx->bp = nullptr;
    vpm_ctx_destroy(b->ctx);
  }
  delete b;
  return VPM_OK;
}

int vpm_batch_last_error(const vpm_batch* b, char* buf, int64_t len) {
  if (!buf || len <= 0) return VPM_ERR_INVALID;
  std::snprintf(buf, size_t(len), "%s", b ? b->err.c_str() : g_last_error.c_str());
  return VPM_OK;
}

int vpm_batch_set_stream(vpm_batch* b, void* stream) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  return from_ctx(b, vpm_ctx_set_stream(b->ctx, stream));
}

int vpm_batch_set_field(vpm_batch* b, int f, const double* X, int64_t sx, const double* G,
                        int64_t sg, const double* S, int64_t ss) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  if (f < 0 || f >= b->plan.nfields) return bfail(b, VPM_ERR_INVALID, "no such field");
  const int64_t n = b->plan.h_n[f];
  int rc = ctx_validate_host(b->ctx, n, X, sx, G, sg, S, ss);
  if (rc == VPM_OK) rc = ctx_upload(b->ctx, b->plan.h_off[f], n, X, sx, G, sg, S, ss);
  if (rc == VPM_OK) b->set[f] = 1;
  return from_ctx(b, rc);
}

int vpm_batch_get_field(vpm_batch* b, int f, double* X, int64_t sx, double* G, int64_t sg,
                        double* S, int64_t ss) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  if (f < 0 || f >= b->plan.nfields) return bfail(b, VPM_ERR_INVALID, "no such field");
  const int64_t n = b->plan.h_n[f], o = b->plan.h_off[f];
  vpm_ctx* c = b->ctx;
  int rc = ctx_download_rows(c, c->X, 3, o, n, X, sx);
  if (!rc) rc = ctx_download_rows(c, c->G, 3, o, n, G, sg);
  if (!rc) rc = ctx_download_rows(c, c->S, 1, o, n, S, ss);
  return from_ctx(b, rc);
}

static int all_set(vpm_batch* b) {
  for (char s : b->set)
    if (!s) return bfail(b, VPM_ERR_STATE, "every field must be set before evaluating");
  return VPM_OK;
}

int vpm_batch_set_particle_order(vpm_batch* b, int mode) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  return from_ctx(b, vpm_set_particle_order(b->ctx, mode));
}

int vpm_batch_eval_UJ(vpm_batch* b, int kernel, int precision) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  int rc = all_set(b);
  if (rc) return rc;
  if (kernel != VPM_KERNEL_WINCKELMANS && kernel != VPM_KERNEL_GAUSSIANERF)
    return bfail(b, VPM_ERR_INVALID, "unknown kernel");
  if (precision != VPM_PREC_FP64 && precision != VPM_PREC_FP32 && precision != VPM_PREC_FP32C)
    return bfail(b, VPM_ERR_INVALID, "unknown precision");
  vpm_ctx* c = b->ctx;
  rc = ctx_prepare_scratch(c, kernel, precision);
  if (rc) return from_ctx(b, rc);
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  cudaError_t e = ctx_pair(c, PASS_UJ, kernel, precision, 0, c->n, 1.0, nullptr, c->U, c->J);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaSetDevice(prev);
  if (e != cudaSuccess) return bfail(b, VPM_ERR_CUDA, std::string("batch U/J: ") + cudaGetErrorString(e));
  c->uj_lo = 0;
  c->uj_hi = c->n;
  return VPM_OK;
}

int vpm_batch_get_UJ(vpm_batch* b, int f, double* U, int64_t su, double* J, int64_t sj) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  if (f < 0 || f >= b->plan.nfields) return bfail(b, VPM_ERR_INVALID, "no such field");
  return from_ctx(b, vpm_get_UJ(b->ctx, b->plan.h_off[f], b->plan.h_n[f], U, su, J, sj));
}

int vpm_batch_autotune(vpm_batch* b, int kernel, int precision, double* ms) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  int rc = all_set(b);
  if (rc) return rc;
  if (kernel != VPM_KERNEL_WINCKELMANS && kernel != VPM_KERNEL_GAUSSIANERF)
    return bfail(b, VPM_ERR_INVALID, "unknown kernel");
  if (precision != VPM_PREC_FP64 && precision != VPM_PREC_FP32 && precision != VPM_PREC_FP32C)
    return bfail(b, VPM_ERR_INVALID, "unknown precision");
  vpm_ctx* c = b->ctx;
  BatchPlan& bp = b->plan;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  // The U/J pass of the current queue, timed on the batch's stream (one
  // untimed pass first).
  auto time_queue = [&](float* t) -> int {
    bp.kernel = kernel;
    bp.precision = precision;
    int r = ctx_prepare_scratch(c, kernel, precision);
    if (r) return r;
    cudaError_t x = ctx_pair(c, PASS_UJ, kernel, precision, 0, c->n, 1.0, nullptr, c->U, c->J);
    if (x == cudaSuccess) x = cudaEventRecord(e0, c->st);
    if (x == cudaSuccess) x = ctx_pair(c, PASS_UJ, kernel, precision, 0, c->n, 1.0, nullptr, c->U, c->J);
    if (x == cudaSuccess) x = cudaEventRecord(e1, c->st);
    if (x == cudaSuccess) x = cudaEventSynchronize(e1);
    if (x == cudaSuccess) x = cudaEventElapsedTime(t, e0, e1);
    return x == cudaSuccess ? VPM_OK
                            : set_error(&c->err, VPM_ERR_CUDA,
                                        std::string("batch autotune: ") + cudaGetErrorString(x));
  };
  // Fields by size bucket; each bucket's fields alone are timed with every
  // compiled shape as one persistent queue, which gives the per-bucket
  // assignment.  Shapes of different buckets run as separate launches one after
  // another, each with its own tail, so the whole batch is then timed with that
  // assignment, with one shape for every field (each compiled shape), and with
  // the per-device table's shapes; the fastest whole-batch plan is kept for
  // this batch (the per-device table is left alone).
  std::vector<std::pair<int, std::vector<int>>> buckets;
  for (int f = 0; f < bp.nfields; ++f) {
    if (bp.h_n[f] == 0) continue;
    const int bk = shape_bucket(bp.h_n[f]);
    auto it = std::find_if(buckets.begin(), buckets.end(),
                           [&](const std::pair<int, std::vector<int>>& p) { return p.first == bk; });
    if (it == buckets.end()) buckets.push_back({bk, {f}});
    else it->second.push_back(f);
  }
  static const Shape cands[] = {{128, 2}, {128, 4}, {256, 2}, {128, 1}};
  std::vector<Shape> shape(bp.nfields, Shape{128, 2});
  bp.h_tuned.clear();
  for (size_t q = 0; q < buckets.size() && e == cudaSuccess && rc == VPM_OK; ++q) {
    const std::vector<int>& fs = buckets[q].second;
    Shape best{0, 0};
    float best_ms = 1e30f;
    for (const Shape& s : cands) {
      if (!pair_shape_supported(precision, s)) continue;
      for (int f : fs) shape[f] = s;
      rc = build_queue(c, kernel, precision, fs, shape);
      float t = 0.f;
      if (rc == VPM_OK) rc = time_queue(&t);
      if (rc != VPM_OK) break;
      if (t < best_ms) {
        best_ms = t;
        best = s;
      }
    }
    if (rc == VPM_OK && best.block > 0)
      for (int f : fs) shape[f] = best;
  }
  // Whole-batch candidates: the per-bucket assignment, one shape for all, the table.
  std::vector<std::vector<Shape>> plans;
  plans.push_back(shape);
  for (const Shape& s : cands)
    if (pair_shape_supported(precision, s)) plans.push_back(std::vector<Shape>(bp.nfields, s));
  {
    std::vector<Shape> table(bp.nfields);
    for (int f = 0; f < bp.nfields; ++f)
      table[f] = lookup_shape(c->device, PASS_UJ, kernel, precision,
                              std::max<int64_t>(bp.h_n[f], 1), &c->pinned[PASS_UJ][kernel][precision]);
    plans.push_back(table);
  }
  std::vector<int> all;
  for (int f = 0; f < bp.nfields; ++f)
    if (bp.h_n[f] > 0) all.push_back(f);
  float t = 1e30f;
  int best_plan = -1;
  for (size_t q = 0; q < plans.size() && e == cudaSuccess && rc == VPM_OK; ++q) {
    rc = build_queue(c, kernel, precision, all, plans[q]);
    float tq = 0.f;
    if (rc == VPM_OK) rc = time_queue(&tq);
    if (rc == VPM_OK && tq < t) {
      t = tq;
      best_plan = int(q);
    }
  }
  if (rc == VPM_OK && e == cudaSuccess && best_plan >= 0) {
    bp.h_tuned = plans[best_plan];
    bp.tuned_kernel = kernel;
    bp.tuned_precision = precision;
    rc = batch_plan(c, kernel, precision);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  c->uj_lo = c->uj_hi = 0;   // U/J hold timing runs
  cudaSetDevice(prev);
  if (e != cudaSuccess) return bfail(b, VPM_ERR_CUDA, std::string("batch autotune: ") + cudaGetErrorString(e));
  if (rc != VPM_OK) return from_ctx(b, rc);
  if (ms) *ms = t;
  return VPM_OK;
}

int vpm_batch_get_shapes(vpm_batch* b, int32_t* block, int32_t* tpt) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  if (b->plan.h_shape.size() != size_t(b->plan.nfields))
    return bfail(b, VPM_ERR_STATE, "no work plan yet (evaluate or step first)");
  for (int f = 0; f < b->plan.nfields; ++f) {
    if (block) block[f] = b->plan.h_shape[f].block;
    if (tpt) tpt[f] = b->plan.h_shape[f].tpt;
  }
  return VPM_OK;
}

int vpm_batch_step(vpm_batch* b, double dt, const vpm_scheme* s, int64_t nsteps, int use_graph) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  int rc = all_set(b);
  if (rc) return rc;
  return from_ctx(b, vpm_step(b->ctx, dt, s, nsteps, use_graph));
}

}  // extern "C"
