// device_api.cu — stateless U/J on caller-owned device arrays
// (vpm_uj_device_async), for hosts that keep the particle field in their own
// CUDA memory (e.g. CUDA.jl arrays passed through ccall).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "capi_internal.h"

using namespace vpm;

namespace vpm {
thread_local PairPlan g_last_stateless_plan = PairPlan();
}  // namespace vpm

extern "C" int vpm_uj_device_async(int kernel, int precision, int64_t ns, const double* Xs,
                                   const double* Gs, const double* Ss, int64_t ld_s, int64_t nt,
                                   const double* Xt, int64_t ld_t, double* U, double* J,
                                   int64_t ld_o, void* cuda_stream) {
  if (kernel != VPM_KERNEL_WINCKELMANS && kernel != VPM_KERNEL_GAUSSIANERF)
    return set_error(nullptr, VPM_ERR_INVALID, "unknown kernel");
  if (precision != VPM_PREC_FP64 && precision != VPM_PREC_FP32 && precision != VPM_PREC_FP32C)
    return set_error(nullptr, VPM_ERR_INVALID, "unknown precision");
  if (ns < 0 || nt < 0) return set_error(nullptr, VPM_ERR_INVALID, "negative count");
  if (nt == 0) return VPM_OK;
  if ((ns > 0 && (!Xs || !Gs || !Ss)) || !U || !J)
    return set_error(nullptr, VPM_ERR_INVALID, "null device array");
  if (ld_s < ns || ld_o < nt) return set_error(nullptr, VPM_ERR_INVALID, "leading dimension too small");
  if (!Xt) {
    if (nt > ns) return set_error(nullptr, VPM_ERR_INVALID, "targets exceed sources");
    Xt = Xs;
    ld_t = ld_s;
  } else if (ld_t < nt) {
    return set_error(nullptr, VPM_ERR_INVALID, "leading dimension too small");
  }
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  int dev = 0, sms = 0;
  cudaError_t qe = cudaGetDevice(&dev);
  if (qe == cudaSuccess) qe = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (qe != cudaSuccess || sms <= 0)
    return set_error(nullptr, VPM_ERR_CUDA,
                     std::string("querying the current device: ") + cudaGetErrorString(qe));
  PairCall pc;
  pc.pass = PASS_UJ; pc.kernel = kernel; pc.prec = precision;
  pc.t0 = 0; pc.t1 = nt; pc.ns = ns;
  pc.xs = Xs; pc.gs = Gs; pc.ss = Ss; pc.vs = nullptr; pc.lds = ld_s;
  pc.xt = Xt; pc.ldt = ld_t;
  pc.sigma_scale = 1.0;
  pc.u = U; pc.j = J; pc.ldo = ld_o;
  size_t need = 0;
  PairPlan plan;
  run_pair(pc, dev, sms, nullptr, nullptr, nt, 0, &need, true, st, &plan);
  double* part = nullptr;
  if (need > 0) {
    cudaError_t e = cudaMallocAsync(&part, need * sizeof(double), st);
    if (e != cudaSuccess) return set_error(nullptr, VPM_ERR_NOMEM, "cannot allocate scratch");
  }
  // FP32 passes read packed source records, as the context path does.
  float4* rec = nullptr;
  cudaError_t e = cudaSuccess;
  if (precision != VPM_PREC_FP64 && ns > 0) {
    e = cudaMallocAsync(&rec, size_t(ns) * 3 * sizeof(float4), st);
    if (e != cudaSuccess) {
      if (part) cudaFreeAsync(part, st);
      return set_error(nullptr, VPM_ERR_NOMEM, "cannot allocate scratch");
    }
    e = launch_pack_sources(kernel, ns, Xs, Gs, Ss, ld_s, 1.0, rec, nullptr, st);
    pc.rec = rec;
  }
  if (e == cudaSuccess)
    e = run_pair(pc, dev, sms, nullptr, part, nt, need, nullptr, false, st, nullptr);
  if (rec) cudaFreeAsync(rec, st);
  if (part) cudaFreeAsync(part, st);
  if (e != cudaSuccess)
    return set_error(nullptr, VPM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  g_last_stateless_plan = plan;
  return VPM_OK;
}

extern "C" int vpm_debug_last_plan(int32_t* block, int32_t* tpt, int32_t* n_chunk,
                                   int32_t* cluster) {
  const PairPlan& p = g_last_stateless_plan;
  if (block) *block = p.shape.block;
  if (tpt) *tpt = p.shape.tpt;
  if (n_chunk) *n_chunk = p.n_tb > 0 ? p.n_chunk : 0;
  if (cluster) *cluster = p.n_tb > 0 ? p.cluster : 0;
  return VPM_OK;
}
