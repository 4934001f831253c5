// peaks.cu — FP32 / FP64 FMA throughput of the device, the denominators of
// the pair kernels' roofline (the U+∇U sum is FMA-pipe bound, not tensor-core
// or HBM bound).  Every SM runs independent FMA chains (8 per thread, so the
// FMA latency is hidden); thread 0 of block 0 also records clock64() and the
// global nanosecond timer to report the SM clock seen during the run.
#include <cuda_runtime.h>

#include <cstring>

#include "capi_internal.h"

namespace {

template <typename R>
__global__ void fma_chains(R* out, int iters, R a, R b, long long* clk) {
  R x0 = R(threadIdx.x) * R(1e-7), x1 = x0 + R(1), x2 = x0 + R(2), x3 = x0 + R(3);
  R x4 = x0 + R(4), x5 = x0 + R(5), x6 = x0 + R(6), x7 = x0 + R(7);
  long long c0 = 0, t0 = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    c0 = clock64();
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    long long t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    clk[0] = clock64() - c0;
    clk[1] = t1 - t0;
  }
  const R s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == R(-12345)) out[threadIdx.x] = s;  // keeps the chains live
}

template <typename R>
int run(int dev, int iters, double* tflops, double* mhz) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  R* out = nullptr;
  long long* clk = nullptr;
  if (cudaMalloc(&out, threads * sizeof(R)) != cudaSuccess) return VPM_ERR_NOMEM;
  if (cudaMalloc(&clk, 2 * sizeof(long long)) != cudaSuccess) {
    cudaFree(out);
    return VPM_ERR_NOMEM;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<R><<<blocks, threads>>>(out, iters / 4, R(0.9999999), R(1e-7), clk);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    fma_chains<R><<<blocks, threads>>>(out, iters, R(0.9999999), R(1e-7), clk);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  long long hc[2] = {0, 0};
  cudaMemcpy(hc, clk, sizeof hc, cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaFree(clk);
  if (err != cudaSuccess) return VPM_ERR_CUDA;
  const double flops = 2.0 * 8.0 * 16.0 * double(iters) * double(threads) * double(blocks);
  *tflops = flops / (double(best) * 1e-3) / 1e12;
  if (mhz) *mhz = hc[1] > 0 ? double(hc[0]) / double(hc[1]) * 1e3 : 0.0;
  return VPM_OK;
}

}  // namespace

extern "C" int vpm_measure_fma_peaks(int device, double* fp32_tflops, double* fp64_tflops,
                                     double* sm_mhz) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return vpm::set_error(nullptr, VPM_ERR_CUDA, "no such CUDA device");
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  double f32 = 0, f64 = 0, mhz = 0, mhz64 = 0;
  int rc = run<float>(device, 4096, &f32, &mhz);
  if (rc == VPM_OK) rc = run<double>(device, 128, &f64, &mhz64);
  cudaSetDevice(prev);
  if (rc != VPM_OK) return vpm::set_error(nullptr, rc, "FMA microbenchmark failed");
  if (fp32_tflops) *fp32_tflops = f32;
  if (fp64_tflops) *fp64_tflops = f64;
  if (sm_mhz) *sm_mhz = mhz;
  return VPM_OK;
}
