// noalloc.cu — U/∇U on caller-owned device arrays without any device
// allocation by the library (vpm_uj_device_noalloc).
//
// Why it exists: vpm_uj_device_async may need scratch for the partial sums of
// a split source range (and for packed FP32 source records), and allocates it
// with the stream-ordered allocator.  Some hosts of this code cannot let a
// library allocate: a simulation loop that must not allocate once it is
// running (fixed-memory or real-time co-simulation), or a host whose device
// memory is entirely pre-reserved by its own pool allocator (a Julia or Python
// caching allocator that owns nearly all of HBM).  This variant takes its
// scratch from the fixed array below instead.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds its 4 MiB until the process exits.  Its name is only a
// host-side stand-in in host code; the device address is looked up with
// cudaGetSymbolAddress once per device context, by the first call that runs
// on that device (so make that first call before any stream capture), and
// again after the context was replaced (cudaDeviceReset).
//
// The FP32/FP32C passes read the FP64 source rows directly and convert them
// in the kernel: no packed source records (they would need 48 bytes of
// scratch per source) and no bulk copies, so they run a few percent slower
// than the same pass through vpm_uj_device_async.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "capi_internal.h"

using namespace vpm;

namespace {

// Partial sums of a split source range: n_chunk x 15 FP64 values per target.
constexpr int64_t kScratchDoubles = int64_t(1) << 19;          // 4 MiB
// Largest target count accepted: two source chunks of 15 values per target fit.
constexpr int64_t kMaxTargets = 16384;
static_assert((2 * kNvalUJ + 1) * kMaxTargets <= kScratchDoubles, "scratch too small");

static __device__ __align__(256) double g_uj_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};   // context id the address belongs to

// Unique id of the current driver context (0 when none is current or the
// driver entry points are unavailable).  A context replaced by
// cudaDeviceReset gets a new id, so a cached symbol address is re-checked.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrent)(CUcontext*);
  typedef CUresult (*GetId)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_uj_scratch on the current device `dev`: looked up once
// per device context, with the device current.
int scratch_address(int dev, double** out) {
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(nullptr, VPM_ERR_UNSUPPORTED, "device index too large for the static scratch table");
  std::lock_guard<std::mutex> lk(g_mu);
  const unsigned long long id = current_context_id();
  if (!g_scratch_addr[dev] || id == 0 || id != g_scratch_ctx[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_uj_scratch);
    if (e != cudaSuccess || !p) {
      g_scratch_addr[dev] = nullptr;
      return set_error(nullptr, VPM_ERR_CUDA,
                       std::string("cudaGetSymbolAddress of the static scratch: ") +
                           cudaGetErrorString(e));
    }
    g_scratch_addr[dev] = static_cast<double*>(p);
    // The lookup made the device's context current if it was not yet.
    g_scratch_ctx[dev] = current_context_id();
  }
  *out = g_scratch_addr[dev];
  return VPM_OK;
}

}  // namespace

extern "C" int vpm_uj_device_noalloc(int kernel, int precision, int64_t ns, const double* Xs,
                                     const double* Gs, const double* Ss, int64_t ld_s, int64_t nt,
                                     const double* Xt, int64_t ld_t, double* U, double* J,
                                     int64_t ld_o, void* cuda_stream) {
  if (kernel != VPM_KERNEL_WINCKELMANS && kernel != VPM_KERNEL_GAUSSIANERF)
    return set_error(nullptr, VPM_ERR_INVALID, "unknown kernel");
  if (precision != VPM_PREC_FP64 && precision != VPM_PREC_FP32 && precision != VPM_PREC_FP32C)
    return set_error(nullptr, VPM_ERR_INVALID, "unknown precision");
  if (ns < 0 || nt < 0) return set_error(nullptr, VPM_ERR_INVALID, "negative count");
  if (nt > kMaxTargets)
    return set_error(nullptr, VPM_ERR_CAPACITY,
                     "vpm_uj_device_noalloc takes at most 16384 targets (its static scratch is "
                     "4 MiB); use vpm_uj_device_async for larger target sets");
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
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess || sms <= 0)
    return set_error(nullptr, VPM_ERR_CUDA,
                     std::string("querying the current device: ") + cudaGetErrorString(e));
  double* scratch = nullptr;
  int rc = scratch_address(dev, &scratch);
  if (rc != VPM_OK) return rc;

  PairCall pc;
  pc.pass = PASS_UJ; pc.kernel = kernel; pc.prec = precision;
  pc.t0 = 0; pc.t1 = nt; pc.ns = ns;
  pc.xs = Xs; pc.gs = Gs; pc.ss = Ss; pc.vs = nullptr; pc.lds = ld_s;
  pc.xt = Xt; pc.ldt = ld_t;
  pc.sigma_scale = 1.0;
  pc.u = U; pc.j = J; pc.ldo = ld_o;
  // Every partial slot a launch uses is written before it is read, so the
  // scratch needs no clearing between calls.
  // The room of nt doubles left over holds the fused form's tile counters.
  pc.max_chunks = int((kScratchDoubles - nt) / (int64_t(kNvalUJ) * nt));
  size_t need = 0;
  PairPlan plan;
  run_pair(pc, dev, sms, nullptr, nullptr, nt, 0, &need, true, nullptr, &plan);
  if (need > size_t(kScratchDoubles))
    return set_error(nullptr, VPM_ERR_CAPACITY, "work plan exceeds the static scratch");
  e = run_pair(pc, dev, sms, nullptr, scratch, nt, size_t(kScratchDoubles), nullptr, false,
               static_cast<cudaStream_t>(cuda_stream), nullptr);
  if (e != cudaSuccess)
    return set_error(nullptr, VPM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  g_last_stateless_plan = plan;
  return VPM_OK;
}
