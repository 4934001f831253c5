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

// Build the work queue for a kernel/precision: the tile shape is the one the
// autotuner (or the default) gives the size bucket that carries most of the
// pair work; the source chunk length L is the smallest multiple of the block
// that keeps the queue near four items per resident CTA.
int batch_plan(vpm_ctx* c, int kernel, int precision) {
  BatchPlan* bp = c->bp;
  const int nf = bp->nfields;
  int64_t dom_n = 1;
  double dom_w = -1.0;
  for (int f = 0; f < nf; ++f) {
    const double w = double(bp->h_n[f]) * double(bp->h_n[f]);
    if (w > dom_w) {
      dom_w = w;
      dom_n = std::max<int64_t>(bp->h_n[f], 1);
    }
  }
  const Shape sh = lookup_shape(c->device, PASS_UJ, kernel, precision, dom_n,
                                &c->pinned[PASS_UJ][kernel][precision]);
  const int r_uj = resident_ctas(c->device, PASS_UJ, kernel, precision, sh, c->num_sms);
  const int r_z = resident_ctas(c->device, PASS_ZETA, kernel, precision, sh, c->num_sms);
  const int64_t TB = int64_t(sh.block) * sh.tpt;
  auto count_items = [&](int64_t L) {
    int64_t items = 0;
    for (int f = 0; f < nf; ++f) {
      const int64_t n = bp->h_n[f];
      if (n == 0) continue;
      items += ceil_div(n, TB) * ceil_div(n, L);
    }
    return items;
  };
  int64_t nmax = 1;
  for (int f = 0; f < nf; ++f) nmax = std::max(nmax, bp->h_n[f]);
  int64_t L = round_up(nmax, sh.block);
  for (int64_t cand = 2 * sh.block; cand < round_up(nmax, sh.block); cand *= 2) {
    if (count_items(cand) <= 4 * int64_t(r_uj)) {
      L = cand;
      break;
    }
  }
  std::vector<PairItem> items;
  std::vector<int32_t> fchunks(nf, 1);
  int max_chunks = 1;
  for (int f = 0; f < nf; ++f) {
    const int64_t n = bp->h_n[f], off = bp->h_off[f];
    if (n == 0) continue;
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
  std::stable_sort(items.begin(), items.end(), [](const PairItem& a, const PairItem& b) {
    return (a.t1 - a.t0) * (a.s1 - a.s0) > (b.t1 - b.t0) * (b.s1 - b.s0);
  });
  cudaFree(bp->d_items);
  bp->d_items = nullptr;
  if (!items.empty()) {
    if (cudaMalloc(&bp->d_items, items.size() * sizeof(PairItem)) != cudaSuccess)
      return set_error(&c->err, VPM_ERR_NOMEM, "cannot allocate the batch work queue");
    cudaMemcpy(bp->d_items, items.data(), items.size() * sizeof(PairItem), cudaMemcpyHostToDevice);
  }
  cudaMemcpy(bp->d_fchunks, fchunks.data(), nf * sizeof(int32_t), cudaMemcpyHostToDevice);
  bp->shape = sh;
  bp->n_items = int(items.size());
  bp->max_chunks = max_chunks;
  bp->resident = std::min(r_uj, r_z);
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
  if (e == cudaSuccess) e = cudaMalloc(&bp.d_counter, sizeof(unsigned int));
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

int vpm_batch_step(vpm_batch* b, double dt, const vpm_scheme* s, int64_t nsteps, int use_graph) {
  if (!b) return set_error(nullptr, VPM_ERR_INVALID, "null batch");
  int rc = all_set(b);
  if (rc) return rc;
  return from_ctx(b, vpm_step(b->ctx, dt, s, nsteps, use_graph));
}

}  // extern "C"
