// update.h — O(N) kernels of a time step (launchers in update.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vpm {

// Device status word bits (OR-ed by kernels, read by the host after a call).
enum : int { STATUS_NONFINITE = 1, STATUS_TIMEOUT = 2 };

struct SfsParams {
  double alpha, rlxf, minC, maxC, zeta0;
  double inv_zeta0;   // 1/ζ(0) (FP64 divides are scarce on the FP64 pipe)
  int transposed;
  int force_positive;
  int analytic;   // Jt, Et hold DJ, DE (analytic α-derivatives)
};

struct UpdateParams {
  double a, b, dt;          // low-storage RK coefficients of the stage, time step
  double uinf0, uinf1, uinf2;
  double zs;                // (f+g)/(1+3f)
  double ze;                // f/(1+3f)
  double zeta0;             // ζ(0) of the kernel
  double inv_zeta0;         // 1/ζ(0)
  double nu;                // core spreading viscosity (0 = off)
  int transposed;
  int sfs;                  // E_str / C_d terms on
  int clip_backscatter;
};

// Diagnostic reduction slots.
enum {
  DS_ENS = 0, DS_IX, DS_IY, DS_IZ, DS_GX, DS_GY, DS_GZ, DS_SIG, DS_NONFIN,
  DS_CCNT, DS_CSUM, DS_CSUM2, DS_CZERO, DS_CMIN, DS_CMAX, DS_CSUM3, DS_CSUM4, kDiagSlots
};
constexpr int kRedBlocks = 304;   // 2 x 152 SMs

cudaError_t launch_stretch_v(int64_t n, int64_t ld, const double* J, const double* G,
                             int transposed, double* V, cudaStream_t st);
cudaError_t launch_estr_finish(int64_t n, int64_t ld, const double* raw, const double* J,
                               int transposed, double* E, cudaStream_t st);
cudaError_t launch_stretch_vw(int64_t n, int64_t ld, const double* J, const double* DJ,
                              const double* G, int transposed, double* V, double* W,
                              cudaStream_t st);
cudaError_t launch_estr_finish_d(int64_t n, int64_t ld, const double* raw, const double* J,
                                 const double* DJ, int transposed, double* E, double* DE,
                                 cudaStream_t st);
// The per-particle kernels below visit particles [0, nv) and skip those whose
// static flag stat[i] is nonzero (stat may be null: no static particles in range).
cudaError_t launch_sfs_dynamic(int64_t nv, const uint8_t* stat, int64_t ld, const double* G,
                               const double* S, const double* J, const double* Jt,
                               const double* E, const double* Et, double* C, const SfsParams& p,
                               cudaStream_t st);
cudaError_t launch_sfs_constant(int64_t nv, const uint8_t* stat, double cd, double* C,
                                cudaStream_t st);
cudaError_t launch_sfs_clip(int64_t nv, const uint8_t* stat, int64_t ld, const double* G,
                            const double* E, double* C, cudaStream_t st);
cudaError_t launch_rk_update(int64_t nv, const uint8_t* stat, int64_t ld, double* X, double* G,
                             double* S, const double* U, const double* J, const double* E,
                             double* C, double* Q, const UpdateParams& p, int* status,
                             cudaStream_t st);
cudaError_t launch_relax(int64_t nv, const uint8_t* stat, int64_t ld, const double* J, double* G,
                         double r, cudaStream_t st);
cudaError_t launch_zero(double* p, int64_t n, cudaStream_t st);
// partial: kRedBlocks*kDiagSlots doubles; out: kDiagSlots doubles (device).
cudaError_t launch_diagnostics(int64_t n, int64_t nf, const uint8_t* stat, int64_t ld,
                               const double* X, const double* G, const double* S, const double* C,
                               const double* raw, double zeta0, double* partial, double* out,
                               cudaStream_t st);
cudaError_t launch_centroid(int64_t i0, int64_t i1, int64_t ld, const double* X, const double* G,
                            double* partial, double* out, cudaStream_t st);

}  // namespace vpm
