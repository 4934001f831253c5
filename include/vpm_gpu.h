/*
 * vpm_gpu.h — C ABI of libvpmgpu.so, a GB300 (sm_103a) implementation of the
 * reformulated vortex particle method (rVPM) particle-field evaluation that
 * FLOWUnsteady drives through FLOWVPM:
 *
 *   - all-pairs regularised Biot–Savart velocity U and gradient J = ∇U
 *     (FLOWVPM's UJ_direct, Winckelmans and Gaussian-erf kernels),
 *   - the stretching term and the dynamic subfilter-scale (SFS) pass,
 *   - the low-storage RK3 (or Euler) update of x, Γ and σ with viscous core
 *     spreading,
 *   - FP64 diagnostics (enstrophy, impulse, centroids, C_d statistics).
 *
 * Reference interface this replaces (paths inside byuflowlab/FLOWUnsteady):
 *   run_simulation(...; vpm_UJ=..., vpm_kernel=..., vpm_SFS=..., vpm_integration=...,
 *                  vpm_transposed=..., vpm_viscous=...)      src/FLOWUnsteady_simulation.jl:107-191
 *   vpm.ParticleField(max_particles; UJ=vpm_UJ, kernel=..., SFS=..., ...)
 *                                                              src/FLOWUnsteady_simulation.jl:239-244
 *   pfield.UJ(pfield)   (probe evaluation)                     src/FLOWUnsteady_simulation.jl:544
 *   pfield.UJ(pfield)   (vortex-sheet forces)                  src/FLOWUnsteady_processing_force.jl:238
 *   vpm.nextstep(pfield, dt; relax, custom_UJ)                 src/FLOWUnsteady_simulation.jl:358
 *   vpm.monitor_enstrophy / vpm.monitor_Cd                      src/FLOWUnsteady_monitors.jl:614,697
 *
 * Conventions
 *   - Every call returns an int status: VPM_OK (0) or a negative VPM_ERR_* code.
 *     vpm_last_error() gives the message of the last failing call on a context.
 *   - Host arrays are strided "array of structs": component k of particle i sits at
 *     ptr[i*stride + k], with a stride per array.  stride = 3 for an (n,3)
 *     row-major array and 1 for an (n,) array; Julia's FLOWVPM particle matrix
 *     (one column per particle) is passed with every stride = number of rows and
 *     each pointer offset to its row.
 *   - J is row-major per particle: J[i*stride + 3*a + b] = dU_a/dx_b.
 *   - The caller owns host memory; the library never retains a host pointer.
 *     The library owns device memory.  There are no callbacks.
 *   - A context is thread-compatible (one host thread at a time).  All work is
 *     issued on the context's stream; calls are synchronous at the ABI unless the
 *     name ends in _async.
 *   - Pair sums skip coincident pairs (r == 0), as FLOWVPM's direct sums do
 *     (src/FLOWUnsteady_processing_force.jl:895); pair counts in throughput
 *     figures still count N_targets x N_sources.
 */
#ifndef VPM_GPU_H
#define VPM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VPM_ABI_VERSION 3

/* ---------------------------------------------------------------- status -- */
enum {
  VPM_OK = 0,
  VPM_ERR_INVALID = -1,      /* bad argument (null pointer, bad enum, n < 0, ...) */
  VPM_ERR_CAPACITY = -2,     /* particle count above the context's capacity      */
  VPM_ERR_CUDA = -3,         /* CUDA runtime error                               */
  VPM_ERR_NONFINITE = -4,    /* NaN/Inf in an input or in the evolved state      */
  VPM_ERR_NOMEM = -5,        /* device allocation failed                         */
  VPM_ERR_UNSUPPORTED = -6,  /* e.g. core spreading with a non-Gaussian kernel   */
  VPM_ERR_STATE = -7,        /* call out of order (e.g. get_UJ before eval)      */
  VPM_ERR_INJECTED = -8      /* host-side fault-injection hook fired             */
};

/* --------------------------------------------------------------- choices -- */
/* Regularising kernels (FLOWVPM's vpm.winckelmans / vpm.gaussianerf,
 * src/FLOWUnsteady_simulation.jl:128). */
enum { VPM_KERNEL_WINCKELMANS = 0, VPM_KERNEL_GAUSSIANERF = 1 };

/* Arithmetic of the O(N^2) pair passes.  State, updates and reductions are
 * always FP64. */
enum {
  VPM_PREC_FP64 = 0,   /* plain FP64 pair sum (the parity form)                    */
  VPM_PREC_FP32 = 1,   /* naive FP32: absolute coordinates, one FP32 accumulator   */
  VPM_PREC_FP32C = 2   /* FP32 on tile-relative coordinates, per-tile FP32 partial  *
                        * sums folded into FP64 accumulators (compensated)          */
};

/* Time integration (FLOWVPM's vpm.euler / vpm.rungekutta3,
 * src/FLOWUnsteady_simulation.jl:131). */
enum { VPM_INTEGRATION_EULER = 0, VPM_INTEGRATION_RK3 = 1 };

/* Subfilter-scale model (FLOWVPM's vpm.SFS_none / vpm.DynamicSFS(vpm.Estr_direct, ...)). */
enum {
  VPM_SFS_NONE = 0,
  VPM_SFS_DYNAMIC = 1,   /* E_str pair pass + pseudo-three-level dynamic C_d          */
  VPM_SFS_CONSTANT = 2   /* E_str pair pass with a prescribed C_d (sfs_Cd)            */
};

/* sfs_flags bits */
#define VPM_SFS_CLIP_BACKSCATTER 1u   /* vpm.clipping_backscatter: C_d = 0 where C_d Γ·E_str < 0 */
#define VPM_SFS_FORCE_POSITIVE 2u     /* the "_positive" procedure: C_d = |C_d|                    */
/* Dynamic procedure with the σ-derivatives taken analytically (d/dα at α = 1,
 * computed inside the pair passes) instead of the finite difference between the
 * σ and ασ filter levels.  The two agree to O(1-α); the analytic form avoids the
 * 1/(1-α) amplification of rounding noise, which matters for FP32/FP32C passes. */
#define VPM_SFS_ANALYTIC_DSIGMA 4u

/* Relaxation of Γ towards the local vorticity (FLOWVPM's vpm.pedrizzetti). */
enum { VPM_RELAX_NONE = 0, VPM_RELAX_PEDRIZZETTI = 1 };

/* The scheme of one time step.  Fill with vpm_scheme_default() and edit. */
/* Settings of the treecode evaluation (the role of FLOWVPM's UJ_fmm with
 * vpm.FMM(p, ncrit, theta), src/FLOWUnsteady_simulation.jl:38,43). */
typedef struct vpm_fmm {
  int32_t p;             /* expansion order of the cell moments: 2, 4 or 6 (4)          */
  int32_t ncrit;         /* at most this many particles per leaf cell (50)               */
  double theta;          /* a cell is far for a target leaf when (R_t+R_s) < theta·d (0.4) */
  double sigma_factor;   /* ... and when d - R_t - R_s >= sigma_factor·(largest σ of the
                            cell): the far field uses the singular kernel, so this keeps
                            regularised pairs in the direct near field (7.1: Gaussian-erf
                            cores agree with the singular kernel to FP32 rounding there;
                            0 = as FLOWVPM's nonzero_sigma=false)                         */
  int32_t local_order;   /* far cells at least as large as the target group (64 consecutive
                            particles of the Morton order) are taken by one local expansion
                            of ψ of this order per group (M2L, then L2P at each target),
                            the others by their moments at every target (M2P); 0 = M2P
                            for every far cell.  Compiled: 0, 7.  Used with p = 4 and
                            FP32/FP32C; other settings take M2P throughout (7)          */
  int32_t reserved;      /* 0 */
} vpm_fmm;

/* U/J evaluation of the plain pair passes of vpm_step (FLOWUnsteady's vpm_UJ). */
enum { VPM_UJ_DIRECT = 0, VPM_UJ_TREE = 1 };

typedef struct vpm_scheme {
  int32_t kernel;        /* VPM_KERNEL_*                                            */
  int32_t precision;     /* VPM_PREC_* used by every pair pass of the step          */
  int32_t integration;   /* VPM_INTEGRATION_*                                       */
  int32_t transposed;    /* 1: S = (Γ·∇ᵀ)u = Jᵀ Γ (FLOWUnsteady default), 0: S = J Γ */
  double f;              /* rVPM formulation constants: rVPM f=0, g=1/5; cVPM f=g=0 */
  double g;
  double uinf[3];        /* freestream velocity added to dx/dt                      */
  double nu;             /* core-spreading viscosity, d(σ²)/dt = 2ν; 0 = inviscid   */
  int32_t sfs;           /* VPM_SFS_*                                               */
  uint32_t sfs_flags;    /* VPM_SFS_CLIP_BACKSCATTER | _FORCE_POSITIVE | _ANALYTIC_DSIGMA */
  double sfs_alpha;      /* test-filter ratio of the dynamic procedure (0.999)      */
  double sfs_rlxf;       /* Lagrangian-average relaxation factor (1 = no averaging) */
  double sfs_minC;       /* |C_d| floor (0 = none)                                  */
  double sfs_maxC;       /* |C_d| ceiling (0 = none)                                */
  double sfs_Cd;         /* prescribed coefficient for VPM_SFS_CONSTANT             */
  int32_t relaxation;    /* VPM_RELAX_*                                             */
  int32_t relax_nsteps;  /* relax every this many steps                             */
  double relax_factor;   /* Pedrizzetti relaxation factor                           */
  int32_t uj_method;     /* VPM_UJ_DIRECT, or VPM_UJ_TREE: the U/J passes (and the
                            relaxation's) by the treecode with `fmm`; the α-derivative
                            and ζ passes of SFS stay direct; no CUDA graphs        */
  int32_t reserved;
  vpm_fmm fmm;           /* treecode settings when uj_method == VPM_UJ_TREE          */
} vpm_scheme;

/* Defaults: Gaussian-erf, FP32C, RK3, transposed, rVPM (f=0, g=1/5), inviscid,
 * no SFS (alpha=0.999, rlxf=1, minC=0, maxC=1 preset for the dynamic model),
 * no relaxation, direct U/J (treecode settings preset to vpm_fmm_default). */
void vpm_scheme_default(vpm_scheme* s);

/* ----------------------------------------------------------- diagnostics -- */
/* vpm_diagnostics() output layout (all FP64). */
enum {
  VPM_DIAG_ENSTROPHY = 0,   /* ½ Σ_p Γ_p·ω(x_p), ω(x) = Σ_q Γ_q ζ_σq(x − x_q) (incl. self) */
  VPM_DIAG_IMPULSE_X = 1,   /* ½ Σ_p x_p × Γ_p                                               */
  VPM_DIAG_IMPULSE_Y = 2,
  VPM_DIAG_IMPULSE_Z = 3,
  VPM_DIAG_GAMMA_X = 4,     /* Σ_p Γ_p                                                       */
  VPM_DIAG_GAMMA_Y = 5,
  VPM_DIAG_GAMMA_Z = 6,
  VPM_DIAG_CD_MEAN = 7,     /* C_d statistics over the free particles with C_d != 0        */
  VPM_DIAG_CD_STD = 8,      /* (vpm.monitor_Cd's t, rationzero, mean, stddev, skew, kurt,   */
  VPM_DIAG_CD_ZERO_RATIO = 9, /* minC, maxC; src/FLOWUnsteady_monitors.jl:697-703):         */
  VPM_DIAG_CD_MIN = 10,     /* population moments; the zero ratio is over all free ones    */
  VPM_DIAG_CD_MAX = 11,
  VPM_DIAG_SIGMA_MEAN = 12,
  VPM_DIAG_NONFINITE = 13,  /* number of particles whose state holds a NaN/Inf            */
  VPM_DIAG_CD_SKEW = 14,    /* m3/m2^(3/2) of the nonzero C_d                              */
  VPM_DIAG_CD_KURT = 15,    /* excess kurtosis m4/m2² - 3 of the nonzero C_d               */
  VPM_DIAG_COUNT = 16
};

/* --------------------------------------------------------------- context -- */
typedef struct vpm_ctx vpm_ctx;

/* Create a context on CUDA device `device` holding up to `capacity` particles.
 * Replaces vpm.ParticleField(max_particles, Float64; ...)
 * (src/FLOWUnsteady_simulation.jl:239-244): the device SoA buffers, the stream,
 * the CUDA graphs and the tile-shape choices live here. */
int vpm_ctx_create(int device, int64_t capacity, vpm_ctx** out);
int vpm_ctx_destroy(vpm_ctx* ctx);

/* Copy the message of the last error on `ctx` (or the last global error when
 * ctx is NULL) into buf (NUL-terminated, at most len bytes). */
int vpm_last_error(const vpm_ctx* ctx, char* buf, int64_t len);

/* Issue the context's work on a caller-owned cudaStream_t (NULL restores the
 * context's own stream).  The stream must belong to the context's device. */
int vpm_ctx_set_stream(vpm_ctx* ctx, void* cuda_stream);

/* Simulation time and step counter (pfield.t, pfield.nt). */
int vpm_get_time(const vpm_ctx* ctx, double* t, int64_t* nt);
int vpm_set_time(vpm_ctx* ctx, double t, int64_t nt);

/* ------------------------------------------------------------ particles -- */
/* Replace the particle set with n particles from host arrays: component k of
 * particle i is X[i*stride_x + k], Gamma[i*stride_g + k], sigma[i*stride_s].
 * SFS memory (C_d and its Lagrangian averages) of every particle is reset to 0.
 * Rejects n > capacity (VPM_ERR_CAPACITY), σ <= 0 (VPM_ERR_INVALID) and
 * non-finite values (VPM_ERR_NONFINITE) without touching the state.
 * Replaces the vpm.add_particle loop that fills a ParticleField. */
int vpm_set_particles(vpm_ctx* ctx, int64_t n, const double* X, int64_t stride_x,
                      const double* Gamma, int64_t stride_g, const double* sigma,
                      int64_t stride_s);

/* Append n particles at the tail (vpm.add_particle, src/FLOWUnsteady_simulation.jl:455-489,
 * and add_probe, :572).  The appended particles are static (sources only, not
 * advanced by vpm_step) when is_static != 0.  Free and static particles may
 * be appended in any order, as FLOWUnsteady appends probes (plain particles,
 * Γ = 0) after the static ones (:516-541).  New particles start with vol 0,
 * circulation 1 and empty SFS memory (see vpm_set_attributes). */
int vpm_append(vpm_ctx* ctx, int64_t n, const double* X, int64_t stride_x, const double* Gamma,
               int64_t stride_g, const double* sigma, int64_t stride_s, int is_static);

/* Per-particle values FLOWVPM carries beside X, Γ, σ (vpm.add_particle's vol,
 * circulation and C keywords; get_vol, get_circulation, get_C), for particles
 * [i0, i0+n): the volume, the circulation magnitude, and the SFS memory C
 * (C_d, ⟨Γ·L⟩, ⟨Γ·m⟩) with stride sc >= 3.  A NULL pointer leaves that value.
 * vol and circulation are carried (saved, restored, read back) but do not
 * enter the method.  FLOWUnsteady's mirror images copy C this way (:527-532). */
int vpm_set_attributes(vpm_ctx* ctx, int64_t i0, int64_t n, const double* vol, int64_t stride_vol,
                       const double* circulation, int64_t stride_circ, const double* C,
                       int64_t stride_c);
/* Read them back, and the static flag (1 or 0) of each particle; any pointer may be NULL. */
int vpm_get_attributes(vpm_ctx* ctx, int64_t i0, int64_t n, double* vol, int64_t stride_vol,
                       double* circulation, int64_t stride_circ, int32_t* is_static);

/* Keep the first n particles (vpm.remove_particle from the tail,
 * src/FLOWUnsteady_simulation.jl:360-365, :550-552). */
int vpm_truncate(vpm_ctx* ctx, int64_t n);

/* Number of particles (vpm.get_np) and of static particles among them. */
int vpm_get_np(const vpm_ctx* ctx, int64_t* n, int64_t* n_static);

/* Download the state of the first n particles (any pointer may be NULL). */
int vpm_get_state(vpm_ctx* ctx, int64_t n, double* X, int64_t stride_x, double* Gamma,
                  int64_t stride_g, double* sigma, int64_t stride_s);

/* Download SFS memory: C (C_d, ⟨Γ·L⟩, ⟨Γ·m⟩) with stride_c, and E_str with stride_e
 * (either may be NULL). */
int vpm_get_sfs(vpm_ctx* ctx, int64_t n, double* C, int64_t stride_c, double* Estr,
                int64_t stride_e);

/* --------------------------------------------------------------- compute -- */
/* U and J at every particle from every particle (pfield.UJ(pfield) with
 * vpm.UJ_direct, src/FLOWUnsteady_simulation.jl:544).  Results stay on the
 * device until vpm_get_UJ. */
int vpm_eval_UJ(vpm_ctx* ctx, int kernel, int precision);

/* U and J at the targets [t0, t1) only, from all particles (the probe form of
 * Vvpm_on_Xs, src/FLOWUnsteady_simulation.jl:494-570). */
int vpm_eval_UJ_targets(vpm_ctx* ctx, int kernel, int precision, int64_t t0, int64_t t1);

/* Download U (stride_u) and J (stride_j) of particles [i0, i0+n) from the last
 * evaluation (either pointer may be NULL).  The range must lie inside the
 * targets of the last vpm_eval_UJ / vpm_eval_UJ_targets / vpm_step. */
int vpm_get_UJ(vpm_ctx* ctx, int64_t i0, int64_t n, double* U, int64_t stride_u, double* J,
               int64_t stride_j);

/* SFS pass on the current state: U/J, E_str and (for VPM_SFS_DYNAMIC) the
 * dynamic coefficient with its clippings, as the first stage of a step does. */
int vpm_eval_sfs(vpm_ctx* ctx, const vpm_scheme* s);

/* Advance the free particles by `nsteps` time steps of size dt
 * (vpm.nextstep, src/FLOWUnsteady_simulation.jl:358).  Static particles act as
 * sources but are not advanced.  When use_graph != 0 each step is a replay of
 * one CUDA graph captured on first use for this (n, scheme). */
int vpm_step(vpm_ctx* ctx, double dt, const vpm_scheme* s, int64_t nsteps, int use_graph);

/* FP64 diagnostics of the current state into out[VPM_DIAG_COUNT]
 * (vpm.monitor_enstrophy, vpm.monitor_Cd).  The enstrophy pair pass uses the
 * given kernel and precision. */
int vpm_diagnostics(vpm_ctx* ctx, int kernel, int precision, double* out);

/* Free-vortex force terms of nb bound particles (host arrays) from all particles
 * of the context (FLOWUnsteady's _Ffv_direct, src/FLOWUnsteady_processing_force.jl:879-929,
 * used by generate_calc_aerodynamicforce_freevortices, :746-857).  For each
 * bound particle b, over every particle f of the field with r = |x_f - x_b| > 0
 * and the bound core size σ_b:
 *   M[b*stride_m + 0..2] = Σ_f U_b(x_f) × Γ_f,  U_b(x) = -g_σb/(4π r³) (x - x_b) × Γ_b
 *   M[b*stride_m + 3..5] = Σ_f g_σb/(4π r³) (x_f - x_b) × (Γ_b × Γ_f)
 * (the reference's P.M[1:3] and P.M[4:6]).  FP64. */
int vpm_ffv_direct(vpm_ctx* ctx, int kernel, int64_t nb, const double* Xb, int64_t stride_x,
                   const double* Gb, int64_t stride_g, const double* Sb, int64_t stride_s,
                   double* M, int64_t stride_m);

/* ------------------------------------------------------------- treecode -- */
/* p 4, ncrit 50, theta 0.4 (FLOWUnsteady's defaults), sigma_factor 7.1,
 * local_order 7. */
void vpm_fmm_default(vpm_fmm* f);

/* U and J at every particle of the context by the treecode (replaces
 * pfield.UJ = vpm.UJ_fmm): particles sorted along a Morton curve, an octree
 * of leaves of at most ncrit particles, far cells from their order-p moments
 * of the singular kernel, near leaves by the direct regularised sum in the
 * given precision (FP32/FP32C: the FP32 pair routines with compensated sums;
 * FP64).  Results as from vpm_eval_UJ (read them with vpm_get_UJ). */
int vpm_eval_UJ_fmm(vpm_ctx* ctx, int kernel, int precision, const vpm_fmm* fmm);

/* Size of the last treecode evaluation into out[VPM_FMM_STATS]: cells, leaves,
 * target groups, far-cell list entries, near-range list entries, near
 * (target, source) pairs, far (target, cell) moment evaluations (M2P), far
 * (group, cell) local-expansion terms (M2L). */
enum { VPM_FMM_STATS = 8 };
int vpm_fmm_stats(const vpm_ctx* ctx, int64_t* out);

/* ------------------------------------------------------------ state files -- */
/* Write the particle field (the role of vpm.save, src/FLOWUnsteady_simulation.jl:436-440)
 * to <path>.pfield.<num>.bin and <path>.pfield.<num>.xmf (".<num>" left out
 * when num < 0).  The .bin file is a 64-byte header (magic "VPMFIELD", version
 * 2, n, n_static, t, nt) followed by X (n×3), Gamma (n×3), sigma (n), the SFS
 * memory C (n×3), a static flag (n), vol (n) and circulation (n), all
 * little-endian FP64, particle-major (version 1 files end after the static
 * flag); the .xmf file describes it for ParaView (XDMF 3, binary data items). */
int vpm_save(vpm_ctx* ctx, const char* path, int64_t num);

/* Restore a field written by vpm_save (the role of
 * vpm.read!(pfield, file; overwrite=true, load_time), :264): replaces the
 * particles with their static flags, SFS memory, vol and circulation (1 and 0
 * for version 1 files) and, when load_time != 0, the time and step counter.
 * A file whose static flags are not 0/1 or disagree with its static count is
 * VPM_ERR_INVALID. */
int vpm_load(vpm_ctx* ctx, const char* bin_file, int load_time);

/* Σ|Γ|-weighted centroids of index ranges: for r in [0, nranges) particles
 * [starts[r], ends[r]) -> centroid out[3r..3r+2]. */
int vpm_centroids(vpm_ctx* ctx, int nranges, const int64_t* starts, const int64_t* ends,
                  double* out);

/* ------------------------------------------------------- device pointers -- */
/* Stateless U/J on caller-owned device memory (for callers that hold the
 * particle field in their own CUDA arrays, e.g. CUDA.jl CuArrays).  Device
 * arrays are SoA: X[k*ld + i], k = 0..2; J[(3a+b)*ld + i].  Targets are the
 * sources [0, nt) when Xt == NULL.  Runs on `cuda_stream` (NULL = legacy
 * default stream) and returns after the work is enqueued. Scratch, if the
 * launch shape needs it, is allocated by the library. */
int vpm_uj_device_async(int kernel, int precision, int64_t ns, const double* Xs,
                        const double* Gs, const double* Ss, int64_t ld_s, int64_t nt,
                        const double* Xt, int64_t ld_t, double* U, double* J, int64_t ld_o,
                        void* cuda_stream);

/* The same evaluation as vpm_uj_device_async, for callers that cannot let the
 * library allocate device memory: a loop that must not allocate once it runs
 * (fixed-memory or real-time co-simulation), or a host whose device memory is
 * entirely held by its own pool allocator (a Julia or Python caching
 * allocator).  It has no counterpart in the reference.  It calls no
 * cudaMalloc, cudaFree or other allocating routine: the scratch for split
 * source ranges is a fixed 4 MiB array that every GPU loading the library
 * holds until the process exits.
 *   - nt may be at most 16384 targets; larger calls return VPM_ERR_CAPACITY
 *     without launching (use vpm_uj_device_async for them).
 *   - The first call on a device (and the first after the device's context
 *     was replaced, e.g. by cudaDeviceReset) looks up the array's device
 *     address (cudaGetSymbolAddress) with that device current; make that
 *     first call before any stream capture.
 *   - All calls share the one array and leave their partial sums in it; every
 *     slot a call uses is written before it is read.  Calls whose work
 *     overlaps on the GPU (different streams, or host threads) race on the
 *     array: serialise them.
 *   - The FP32/FP32C passes convert the FP64 sources in the kernel instead of
 *     reading packed source records (which would need scratch per source), so
 *     they run a few percent slower than through vpm_uj_device_async. */
int vpm_uj_device_noalloc(int kernel, int precision, int64_t ns, const double* Xs,
                          const double* Gs, const double* Ss, int64_t ld_s, int64_t nt,
                          const double* Xt, int64_t ld_t, double* U, double* J, int64_t ld_o,
                          void* cuda_stream);

/* --------------------------------------------------------------- batches -- */
typedef struct vpm_batch vpm_batch;

/* Many independent particle fields of uneven size advanced together: every
 * pair pass of a stage is one persistent launch over a flattened
 * (field, target tile, source chunk) work queue. */
int vpm_batch_create(int device, int nfields, const int64_t* n, vpm_batch** out);
int vpm_batch_destroy(vpm_batch* b);
int vpm_batch_last_error(const vpm_batch* b, char* buf, int64_t len);
int vpm_batch_set_stream(vpm_batch* b, void* cuda_stream);
int vpm_batch_set_field(vpm_batch* b, int field, const double* X, int64_t stride_x,
                        const double* Gamma, int64_t stride_g, const double* sigma,
                        int64_t stride_s);
int vpm_batch_get_field(vpm_batch* b, int field, double* X, int64_t stride_x, double* Gamma,
                        int64_t stride_g, double* sigma, int64_t stride_s);
int vpm_batch_eval_UJ(vpm_batch* b, int kernel, int precision);
int vpm_batch_get_UJ(vpm_batch* b, int field, double* U, int64_t stride_u, double* J,
                     int64_t stride_j);
int vpm_batch_step(vpm_batch* b, double dt, const vpm_scheme* s, int64_t nsteps, int use_graph);

/* Tile shapes of a batch by size bucket (log2 N): every field takes the shape
 * stored for its bucket in the per-device table (see vpm_autotune), and the
 * fields of one shape form one persistent launch per pair pass (the default,
 * before tuning: every bucket below 196,608 particles takes 128x2).
 * vpm_batch_autotune times, for each bucket present, that bucket's fields
 * alone as one persistent U/J launch with every compiled shape (the per-bucket
 * assignment); then one U/J pass of the whole batch with that assignment, with
 * each compiled shape for every field, and with the table's shapes.  Launches
 * of different shapes run one after another, so the per-bucket assignment can
 * lose to one shape for all.  The fastest whole-batch plan is kept for this
 * batch (the per-device table is not changed), the work queue is rebuilt, and
 * its time of one U/J pass is returned (ms).  vpm_batch_get_shapes reads the
 * shape of each field (arrays of nfields). */
int vpm_batch_autotune(vpm_batch* b, int kernel, int precision, double* ms);
int vpm_batch_get_shapes(vpm_batch* b, int32_t* block, int32_t* tpt);

/* ----------------------------------------------------------- utilities -- */
/* Tile shape of the pair kernels: block size, targets per thread and source
 * chunk length.  vpm_autotune times every compiled shape of the U/J pass and,
 * separately, of the ζ pass on the context's particles and stores the fastest
 * for that size bucket (log2 N) in a per-device table (mutex-guarded) that
 * every context then uses; vpm_set_tile pins a shape on one context. */
typedef struct vpm_tile {
  int32_t block;        /* threads per CTA                         */
  int32_t tpt;          /* targets per thread (register blocking)  */
  int32_t chunk;        /* sources per work item: 0 = the planner's choice; pinned by
                           vpm_set_tile, rounded up to whole tiles of `block` sources */
  int32_t reserved;     /* vpm_autotune: ζ-pass shape as block*16 + tpt */
} vpm_tile;
int vpm_autotune(vpm_ctx* ctx, int kernel, int precision, vpm_tile* chosen, double* ms);
int vpm_set_tile(vpm_ctx* ctx, int kernel, int precision, const vpm_tile* t);

/* Order in which the pair passes visit the particles (no counterpart in
 * FLOWVPM, whose sums run in the field's own order).
 *   VPM_ORDER_AUTO (default): pair passes over all particles of a field of
 *     65,536 or more, and every batch pass, sort the particles along a Morton
 *     curve of their positions (each batch field in its own cube), run there
 *     and scatter the results back to the caller's order.  Only the summation
 *     order changes; the Gaussian-erf far-field forms then apply whatever the
 *     caller's order.
 *   VPM_ORDER_CALLER: the caller's order.
 * The environment variable VPM_NO_SORT=1 forces VPM_ORDER_CALLER everywhere. */
enum { VPM_ORDER_AUTO = 0, VPM_ORDER_CALLER = 1 };
int vpm_set_particle_order(vpm_ctx* ctx, int mode);
int vpm_batch_set_particle_order(vpm_batch* b, int mode);

/* Measured FP32 and FP64 FMA throughput of the device (TFLOP/s, FMA = 2 flops),
 * from an all-SM independent-chain microbenchmark. */
int vpm_measure_fma_peaks(int device, double* fp32_tflops, double* fp64_tflops, double* sm_mhz);

/* Host fault-injection hook for tests: the next k-th launch-issuing call on the
 * context fails with VPM_ERR_INJECTED before it launches anything (0 disables). */
int vpm_debug_fail_after(vpm_ctx* ctx, int64_t k);

/* Work plan of the last successful vpm_uj_device_async / vpm_uj_device_noalloc
 * call on this host thread: tile shape (threads per CTA, targets per thread),
 * the number of source chunks each target tile is split into, and the cluster
 * size: 1 when the chunks' partial sums went through scratch (if n_chunk > 1),
 * n_chunk when the chunks ran as one thread-block cluster summing them in
 * shared memory.  Zeros before the first call.  Any pointer may be NULL. */
int vpm_debug_last_plan(int32_t* block, int32_t* tpt, int32_t* n_chunk, int32_t* cluster);

/* Number of kernels the context has enqueued since creation (pair passes,
 * reductions and updates; a graph replay counts its kernels). */
int vpm_get_launch_count(const vpm_ctx* ctx, int64_t* count);

/* Library build information ("sm_103a ..."). */
const char* vpm_build_info(void);

#ifdef __cplusplus
}
#endif

#endif /* VPM_GPU_H */
