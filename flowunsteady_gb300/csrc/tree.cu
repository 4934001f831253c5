// tree.cu — GPU treecode for U and ∇U (the role of FLOWVPM's UJ_fmm with
// vpm.FMM(p, ncrit, theta), src/FLOWUnsteady_simulation.jl:38,43).
//
// One evaluation runs entirely on the device, in this order:
//   1. bounding cube and 63-bit Morton codes of the particles; radix sort of
//      (code, index) pairs; gather of the state into Morton order and the
//      packed FP32 source records of that order;
//   2. octree built generation by generation: a cell with more than ncrit
//      particles whose codes differ is split at the first 3-bit Morton digit
//      where they differ (so no single-child chains), children are appended
//      with an atomic counter; cells are contiguous ranges of sorted particles;
//   3. upward pass, deepest generation first: leaves take their bounding box,
//      largest core and moments (order P) from their particles, parents from
//      their children (box union; moments shifted to the parent centre);
//   4. targets are taken in groups of 64 consecutive particles of the Morton
//      order (compact boxes, one full CTA each).  The walk for a group is
//      split over the subtrees of a frontier of at most 73 cells (the leaves
//      of generations 0-1 and generation 2), one thread per (group, subtree):
//      a cell s is far for group t when (R_t + R_s) < θ·d and
//      d - R_t - R_s >= sigma_factor·σmax_s (d = distance of the centres, FP32
//      boxes), then it is evaluated from its moments; otherwise its leaves are
//      summed directly, consecutive leaves merged into one range of particles
//      (two passes: count, fill); with local expansions, far cells at least
//      as large as the group are marked for them;
//   5. local expansions (FP32, P = 4): the marked cells' moments turned into
//      one local expansion of ψ per group (M2L, tree.cuh);
//   6. the direct near field: one CTA per group over its near ranges, with the
//      regularised kernels of the direct sum (FP32 pair routines on positions
//      relative to the group's first particle, or FP64);
//   7. the far field: one thread per target over the unmarked far cells of its
//      group (M2P, tree.cuh), added to the near field; results go to the
//      original order; then the local expansion at every target (L2P) is
//      added to them.
// The far field uses the singular kernel, as FLOWVPM's nonzero_sigma=false;
// sigma_factor keeps regularised pairs out of it (Gaussian-erf: beyond 7.1 σ
// the kernels agree to FP32 rounding).
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "capi_internal.h"
#include "tree.cuh"
#include "vpm_device.cuh"

namespace vpm {

constexpr int kMaxGen = 23;        // root + at most 21 Morton digits (+1 spare)
// Device counters: cells, leaves, error flags, target groups, then the first
// cell of every generation (generation g starts at counters[kGenBase + g]).
constexpr int kCntCells = 0, kCntLeaves = 1, kCntFlags = 2, kCntGroups = 3, kGenBase = 4;
constexpr int kNumCounters = kGenBase + kMaxGen + 2;
constexpr int kStack = 256;        // traversal stack (cells)
// Target group size (consecutive particles of the Morton order).  32-particle
// groups were measured at N = 1M too: at θ = 0.4 they take 0.131 s instead of
// 0.142 s but lose accuracy (rel-L2 U 5.3e-5, J 1.46e-5 against 4.4e-5, 1.15e-5),
// and at equal accuracy (θ ≈ 0.39) the two sizes take the same time.
constexpr int kTreeBlock = 64;     // threads of the far CTAs = group size
constexpr int kMaxFront = 1 + 8 + 64;   // walk roots: leaves of generations 0-1, generation 2

// ------------------------------------------------------------- workspace --
struct FmmWork {
  int64_t cap = 0;            // particles
  int64_t cell_cap = 0;       // cells (2·cap + 8 bounds any octree of cap points)
  int64_t mom_cells = 0;      // cells the moment buffers hold
  int mom_p = -1;
  int64_t list_cap = 0;       // interaction list entries
  // particles in Morton order
  uint64_t *codes = nullptr, *codes_alt = nullptr;
  int *idx = nullptr, *perm = nullptr;
  double* sorted = nullptr;   // X 3, Γ 3, σ 1 rows of length cap
  float4* rec = nullptr;      // packed FP32 source records of the sorted particles
  double* near_raw = nullptr; // up to 27 raw near-field sums per sorted particle
  float* vw = nullptr;        // v_q, w_q rows of the ζ passes in Morton order, FP32
  // cells
  int *lo = nullptr, *hi = nullptr, *child = nullptr, *nchild = nullptr;
  double* geom = nullptr;     // per cell: box min x y z, box max x y z, σmax, unused
  double* mom = nullptr;      // per cell: 3·ncoef(P) FP64 moments
  float* momf = nullptr;      // FP32 copy
  int* leaves = nullptr;      // leaf cell ids
  int* counters = nullptr;    // see kCntCells .. kGenBase
  int64_t meta_cap = 0;       // (group, frontier cell) walk slots
  float4* ggeom = nullptr;    // target-group boxes (centre, radius), FP32
  float4* cgeom = nullptr;    // walk records, two per cell (see cell_walk_kernel)
  int* front = nullptr;       // frontier cells (walk roots)
  unsigned long long* pairs = nullptr;   // [0] near source pairs, [1] far (target, cell) pairs
  double* box = nullptr;      // bounding cube: min x y z, size
  double* box_part = nullptr; // per-block min/max partials
  // interaction lists
  int *nfar = nullptr, *nnear = nullptr, *ofar = nullptr, *onear = nullptr;
  int* far_list = nullptr;    // far cell ids per target group (M2P at every target)
  int *nloc = nullptr, *oloc = nullptr;   // local-expansion list counts, offsets
  int* loc_list = nullptr;    // far cell ids per target group taken by its local expansion
  int64_t loc_list_cap = 0;
  int2* near_list = nullptr;  // near source ranges [x, y) per target group
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
  int h_counters[kNumCounters];
  // statistics of the last evaluation
  int64_t last_cells = 0, last_leaves = 0, last_groups = 0, last_far = 0, last_near = 0;
  int64_t last_nfront = 0, last_n = -1;
  unsigned long long h_pairs[3] = {0, 0, 0};
  float* loc = nullptr;       // per target group: 3·ncoef(Q) local coefficients
  int64_t loc_cap = 0;
};

void fmm_free(FmmWork* w) {
  if (!w) return;
  void* ptrs[] = {w->codes, w->codes_alt, w->idx, w->perm, w->sorted, w->rec, w->near_raw,
                  w->vw, w->lo, w->hi, w->child, w->nchild, w->geom, w->mom, w->momf, w->leaves,
                  w->ggeom, w->cgeom, w->front, w->pairs, w->counters, w->box, w->box_part,
                  w->nfar, w->nnear, w->ofar, w->onear, w->far_list, w->near_list, w->cub_tmp,
                  w->loc, w->nloc, w->oloc, w->loc_list};
  for (void* p : ptrs) cudaFree(p);
  delete w;
}

// ------------------------------------------------------ bounding cube, codes --
constexpr int kBoxBlocks = 256;

__global__ void box_partial_kernel(int64_t n, const double* __restrict__ X, int64_t ld,
                                   double* part) {
  __shared__ double s[6][256];
  double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double x = X[d * ld + i];
      v[d] = fmin(v[d], x);
      v[3 + d] = fmax(v[3 + d], x);
    }
  }
#pragma unroll
  for (int d = 0; d < 6; ++d) s[d][threadIdx.x] = v[d];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + o]);
        s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + o]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int d = 0; d < 6; ++d) part[blockIdx.x * 6 + d] = s[d][0];
}

// One block of kBoxBlocks threads, one per partial box.
__global__ void box_final_kernel(const double* part, int nblocks, double* box) {
  __shared__ double s[6][kBoxBlocks];
  const int t = threadIdx.x;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    s[d][t] = t < nblocks ? part[t * 6 + d] : INFINITY;
    s[3 + d][t] = t < nblocks ? part[t * 6 + 3 + d] : -INFINITY;
  }
  __syncthreads();
  for (int o = kBoxBlocks / 2; o > 0; o >>= 1) {
    if (t < o) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        s[d][t] = fmin(s[d][t], s[d][t + o]);
        s[3 + d][t] = fmax(s[3 + d][t], s[3 + d][t + o]);
      }
    }
    __syncthreads();
  }
  if (t == 0) {
    const double size = fmax(fmax(s[3][0] - s[0][0], s[4][0] - s[1][0]), s[5][0] - s[2][0]);
    box[0] = s[0][0];
    box[1] = s[1][0];
    box[2] = s[2][0];
    box[3] = size > 0 ? size * (1.0 + 1e-9) : 1.0;
  }
}

// Spread the low 21 bits of v to every third bit (Morton interleaving).
__device__ __forceinline__ uint64_t spread3(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

__global__ void morton_kernel(int64_t n, const double* __restrict__ X, int64_t ld,
                              const double* __restrict__ box, uint64_t* codes, int* idx) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double scale = double(1 << 21) / box[3];
  uint64_t q[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double t = floor((X[d * ld + i] - box[d]) * scale);
    q[d] = uint64_t(fmin(fmax(t, 0.0), double((1 << 21) - 1)));
  }
  codes[i] = spread3(q[0]) << 2 | spread3(q[1]) << 1 | spread3(q[2]);
  idx[i] = int(i);
}

// Sorted FP64 state (X 3, Γ 3, σ 1 rows of length ldw) in Morton order.
__global__ void gather_kernel(int64_t n, const int* __restrict__ perm, const double* __restrict__ X,
                              const double* __restrict__ G, const double* __restrict__ S,
                              int64_t ld, double* sorted, int64_t ldw) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t j = perm[i];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    sorted[d * ldw + i] = X[d * ld + j];
    sorted[(3 + d) * ldw + i] = G[d * ld + j];
  }
  sorted[6 * ldw + i] = S[j];
}

// ------------------------------------------------------------- tree build --
__global__ void tree_init_kernel(int64_t n, int* lo, int* hi, int* counters) {
  lo[0] = 0;
  hi[0] = int(n);
  counters[kCntCells] = 1;
  counters[kCntLeaves] = 0;
  counters[kCntFlags] = 0;
  counters[kCntGroups] = 0;
  counters[kGenBase + 0] = 0;   // generation 0 is the root
  counters[kGenBase + 1] = 1;
}

__device__ __forceinline__ int lower_bound_code(const uint64_t* codes, int lo, int hi,
                                                uint64_t key) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (codes[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Split or close the cells of generation g.
__global__ void tree_split_kernel(int g, int ncrit, int64_t cell_cap, const uint64_t* __restrict__ codes,
                                  int* lo, int* hi, int* child, int* nchild, int* leaves,
                                  int* counters) {
  const int begin = counters[kGenBase + g], end = counters[kGenBase + g + 1];
  for (int cell = begin + int(blockIdx.x * blockDim.x + threadIdx.x); cell < end;
       cell += int(gridDim.x * blockDim.x)) {
    const int a = lo[cell], b = hi[cell];
    const uint64_t first = codes[a], last = codes[b - 1];
    if (b - a <= ncrit || first == last) {
      child[cell] = -1;
      nchild[cell] = 0;
      leaves[atomicAdd(&counters[kCntLeaves], 1)] = cell;
      continue;
    }
    const int bit = 63 - __clzll((long long)(first ^ last));   // highest differing bit
    const int shift = (bit / 3) * 3;                            // its Morton digit
    const uint64_t prefix = first & ~((uint64_t(8) << shift) - 1);
    int bounds[9];
    bounds[0] = a;
    bounds[8] = b;
    for (int v = 1; v < 8; ++v) bounds[v] = lower_bound_code(codes, a, b, prefix | (uint64_t(v) << shift));
    int nc = 0;
    for (int v = 0; v < 8; ++v) nc += bounds[v + 1] > bounds[v];
    const int first_child = atomicAdd(&counters[kCntCells], nc);
    if (first_child + nc > cell_cap) {
      atomicOr(&counters[kCntFlags], 1);
      child[cell] = -1;
      nchild[cell] = 0;
      continue;
    }
    int k = first_child;
    for (int v = 0; v < 8; ++v) {
      if (bounds[v + 1] > bounds[v]) {
        lo[k] = bounds[v];
        hi[k] = bounds[v + 1];
        ++k;
      }
    }
    child[cell] = first_child;
    nchild[cell] = nc;
  }
}

// Generation g+1 ends where the cells appended while splitting generation g end.
__global__ void tree_advance_kernel(int g, int* counters) {
  counters[kGenBase + g + 2] = counters[kCntCells];
}

// ------------------------------------------------------------ upward pass --
// Cell geometry record (8 doubles): box min x y z, box max x y z, σmax, unused.
constexpr int kGeom = 8;

// Binomial coefficient, iteratively: a recursive form becomes a recursive
// device call wherever the loops around it are not fully unrolled, and
// recursion has no static stack bound.
__host__ __device__ constexpr int binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  int r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

__device__ __forceinline__ void cell_centre(const double* g, double& cx, double& cy, double& cz,
                                            double& r) {
  cx = 0.5 * (g[0] + g[3]);
  cy = 0.5 * (g[1] + g[4]);
  cz = 0.5 * (g[2] + g[5]);
  const double ex = 0.5 * (g[3] - g[0]), ey = 0.5 * (g[4] - g[1]), ez = 0.5 * (g[5] - g[2]);
  r = sqrt(ex * ex + ey * ey + ez * ez);
}

// Binomial coefficients C(n, k) for n, k <= 6 (the largest order is 6), as a
// table: the moment shift's loops are too large to unroll completely, and a
// binomial formed at run time costs integer divisions in its innermost loop.
__constant__ double c_binom[7][7] = {
    {1, 0, 0, 0, 0, 0, 0},   {1, 1, 0, 0, 0, 0, 0},    {1, 2, 1, 0, 0, 0, 0},
    {1, 3, 3, 1, 0, 0, 0},   {1, 4, 6, 4, 1, 0, 0},    {1, 5, 10, 10, 5, 1, 0},
    {1, 6, 15, 20, 15, 6, 1}};

// Cells of generation g: leaves from their particles, parents from their
// children (which belong to later generations, already done).  One thread per
// (cell, vorticity component m): the three threads of a cell form the same box;
// the one with m = 0 writes it.
template <int P>
__global__ void tree_upward_kernel(int g, const int* __restrict__ counters, const int* __restrict__ lo,
                                   const int* __restrict__ hi, const int* __restrict__ child,
                                   const int* __restrict__ nchild, const double* __restrict__ sorted,
                                   int64_t ldw, double* geom, double* mom) {
  constexpr int NC = ncoef(P);
  const int begin = counters[kGenBase + g], end = counters[kGenBase + g + 1];
  const int64_t nwork = int64_t(end - begin) * 3;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < nwork;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int cell = begin + int(t / 3), m = int(t % 3);
    double* gc = geom + int64_t(cell) * kGeom;
    const int nc = nchild[cell];
    double bx[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    double smax = 0.0;
    bool bad = false;
    if (nc == 0) {
      for (int i = lo[cell]; i < hi[cell]; ++i) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const double x = sorted[d * ldw + i];
          bx[d] = fmin(bx[d], x);
          bx[3 + d] = fmax(bx[3 + d], x);
        }
        smax = fmax(smax, sorted[6 * ldw + i]);
      }
    } else {
      for (int k = 0; k < nc; ++k) {
        if (child[cell] + k >= counters[kCntCells]) {
          atomicOr(const_cast<int*>(&counters[kCntFlags]), 32);
          bad = true;
          break;
        }
        const double* gk = geom + int64_t(child[cell] + k) * kGeom;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          bx[d] = fmin(bx[d], gk[d]);
          bx[3 + d] = fmax(bx[3 + d], gk[3 + d]);
        }
        smax = fmax(smax, gk[6]);
      }
    }
    if (m == 0) {
#pragma unroll
      for (int d = 0; d < 6; ++d) gc[d] = bx[d];
      gc[6] = smax;
      gc[7] = 0.0;
    }
    double cx, cy, cz, rad;
    {
      double b8[8] = {bx[0], bx[1], bx[2], bx[3], bx[4], bx[5], smax, 0.0};
      cell_centre(b8, cx, cy, cz, rad);
    }
    double* mc = mom + int64_t(cell) * 3 * NC;
    double acc[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) acc[k] = 0.0;
    if (nc == 0) {
      for (int i = lo[cell]; i < hi[cell]; ++i) {
        double pw[NC];
        monomials<P, double>(sorted[i] - cx, sorted[ldw + i] - cy, sorted[2 * ldw + i] - cz, pw);
        const double gm = sorted[(3 + m) * ldw + i];
#pragma unroll
        for (int k = 0; k < NC; ++k) acc[k] += gm * pw[k];
      }
    } else if (!bad) {
      for (int q = 0; q < nc; ++q) {
        const int ch = child[cell] + q;
        double qx, qy, qz, qr;
        cell_centre(geom + int64_t(ch) * kGeom, qx, qy, qz, qr);
        double tp[NC];
        monomials<P, double>(qx - cx, qy - cy, qz - cz, tp);
        const double* mq = mom + int64_t(ch) * 3 * NC + m * NC;
        // (y - c)^k = Σ_{j<=k} C(k, j) (y - c_q)^j (c_q - c)^{k-j}
#pragma unroll
        for (int n = 0; n <= P; ++n)
#pragma unroll
          for (int a = n; a >= 0; --a)
#pragma unroll
            for (int b = n - a; b >= 0; --b) {
              const int c = n - a - b;
              double s = 0.0;
#pragma unroll
              for (int ja = 0; ja <= a; ++ja)
#pragma unroll
                for (int jb = 0; jb <= b; ++jb)
#pragma unroll
                  for (int jc = 0; jc <= c; ++jc)
                    s += c_binom[a][ja] * c_binom[b][jb] * c_binom[c][jc] *
                         tp[midx(a - ja, b - jb, c - jc)] * mq[midx(ja, jb, jc)];
              acc[midx(a, b, c)] += s;
            }
      }
    }
#pragma unroll
    for (int k = 0; k < NC; ++k) mc[m * NC + k] = acc[k];
  }
}

__global__ void moments_to_f32_kernel(int64_t n, const double* __restrict__ a, float* b) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = float(a[i]);
}

// -------------------------------------------------------------- traversal --
// Targets are taken in groups of kTreeBlock consecutive particles of the Morton
// order (the last one shorter): compact boxes, full CTAs.  Each group's box
// (centre, radius) and each cell's (centre, radius) and largest core go to
// FP32 records for the walk; radii are inflated by 1e-6 of the coordinates'
// magnitude so that rounding cannot shrink them.
__global__ void group_geom_kernel(int64_t n, const double* __restrict__ sorted, int64_t ldw,
                                  float4* ggeom) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t a = g * kTreeBlock;
  if (a >= n) return;
  const int64_t b = a + kTreeBlock < n ? a + kTreeBlock : n;
  double bx[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = a; i < b; ++i)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double x = sorted[d * ldw + i];
      bx[d] = fmin(bx[d], x);
      bx[3 + d] = fmax(bx[3 + d], x);
    }
  double cx, cy, cz, r;
  cell_centre(bx, cx, cy, cz, r);
  const double pad = 1e-6 * (fabs(cx) + fabs(cy) + fabs(cz) + r);
  ggeom[g] = make_float4(float(cx), float(cy), float(cz), float(r + pad));
}

// Walk record of cell c, two float4 read together by the traversal:
//   rec[2c]     = centre x, y, z and radius (FP32, inflated as above);
//   rec[2c + 1] = largest core (FP32), then as integer bits: the first child
//                 (or the first particle of a leaf), the end of a leaf's
//                 particle range, the number of children (0 for a leaf).
__global__ void cell_walk_kernel(int ncells, const double* __restrict__ geom,
                                 const int* __restrict__ lo, const int* __restrict__ hi,
                                 const int* __restrict__ child, const int* __restrict__ nchild,
                                 float4* rec) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  double cx, cy, cz, r;
  cell_centre(geom + int64_t(c) * kGeom, cx, cy, cz, r);
  const double pad = 1e-6 * (fabs(cx) + fabs(cy) + fabs(cz) + r);
  rec[2 * c] = make_float4(float(cx), float(cy), float(cz), float(r + pad));
  const int nc = nchild[c];
  rec[2 * c + 1] = make_float4(float(geom[int64_t(c) * kGeom + 6]),
                               __int_as_float(nc == 0 ? lo[c] : child[c]), __int_as_float(hi[c]),
                               __int_as_float(nc));
}

// One thread per (target group g, frontier cell j), t = g·nfront + j: the
// walk of the subtree below frontier cell j for group g.  FILL = false counts
// the far cells and near source ranges, FILL = true writes them at the
// scanned offsets (same order); a group's lists are the concatenation over j.
// Near leaves that continue the previous near range in Morton order extend it.
template <bool FILL>
__global__ void traverse_kernel(int64_t nthreads, int nfront, const int* __restrict__ front,
                                const float4* __restrict__ ggeom, const float4* __restrict__ walk,
                                float theta, float sfac, int mark_local, int* nfar,
                                int* nnear, int* nloc, const int* __restrict__ ofar,
                                const int* __restrict__ onear, const int* __restrict__ oloc,
                                int* far_list, int2* near_list, int* loc_list, int* counters,
                                int ncells) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nthreads) return;
  const int64_t g = t / nfront;
  const float4 tg = ggeom[g];
  int stack[kStack];
  int sp = 0;
  stack[sp++] = front[t % nfront];
  int cf = 0, cn = 0, cl = 0, last_hi = -1;
  const int of = FILL ? ofar[t] : 0, on = FILL ? onear[t] : 0, ol = FILL && mark_local ? oloc[t] : 0;
  while (sp > 0) {
    const int s = stack[--sp];
    if (s < 0 || s >= ncells) {
      atomicOr(&counters[kCntFlags], 16);
      break;
    }
    const float4 cs = walk[2 * s], ck = walk[2 * s + 1];
    const int first = __float_as_int(ck.y), end = __float_as_int(ck.z), nc = __float_as_int(ck.w);
    const float dx = tg.x - cs.x, dy = tg.y - cs.y, dz = tg.z - cs.z;
    const float d = sqrtf(dx * dx + dy * dy + dz * dz);
    if (tg.w + cs.w < theta * d && d - tg.w - cs.w >= sfac * ck.x) {
      // Cells at least as large as the group go to its local expansion.
      if (mark_local && cs.w >= tg.w) {
        if (FILL) loc_list[ol + cl] = s;
        ++cl;
      } else {
        if (FILL) far_list[of + cf] = s;
        ++cf;
      }
    } else if (nc == 0) {
      if (cn > 0 && first == last_hi) {
        if (FILL) near_list[on + cn - 1].y = end;
      } else {
        if (FILL) near_list[on + cn] = make_int2(first, end);
        ++cn;
      }
      last_hi = end;
    } else {
      const int c0 = first;
      if (sp + nc > kStack) {   // cannot happen for 21 Morton levels (7·21 + 1 entries)
        atomicOr(&counters[kCntFlags], 2);
        break;
      }
      for (int k = nc - 1; k >= 0; --k) stack[sp++] = c0 + k;
    }
  }
  if (!FILL) {
    nfar[t] = cf;
    nnear[t] = cn;
    if (mark_local) nloc[t] = cl;
  }
}

// --------------------------------------------------------------- near field --
// One CTA of kNearThreads threads per target group against every particle of
// its near source ranges, with the pair routines of the direct sum
// (vpm_device.cuh) on T targets per thread:
//   - the group's kTreeBlock targets are held as TQ = kTreeBlock/T target sets of T targets
//     (target t = tq + TQ·k), each set by SL = kNearThreads/TQ threads, one per
//     source slice;
//   - the concatenated near ranges are staged kNearThreads sources at a time
//     (positions relative to the group's first particle, from the packed
//     records); slice s takes the staged sources s, s + SL, s + 2·SL, ..., so
//     every thread reads each of its sources with broadcast 16-byte loads and
//     applies it to T targets (packed FP32 pairs for T even);
//   - a tile is always full: slots past the sources hold a padding source at
//     1e18 with zero strength, which adds exactly 0 (its q and p underflow),
//     so the warp votes of the pair routines see the same trip count on every
//     lane;
//   - FP32 sums are folded into (hi, lo) pairs (Knuth's TwoSum) every
//     kNearFoldSources sources of a thread; the epilogue forms every target's raw
//     sums in FP64 as the slices' (hi + lo) in slice order.
// Raw sums go to raw[k·ldr + i] in Morton order:
//   PASS_UJ    U 3, A 9, W 3 (Gaussian-erf A sums hold p/(-3), as the direct
//              pass's do);
//   PASS_UJD   those plus DA 9, DW 3 (Gaussian-erf: Dq, Dp vanish beyond the
//              near field's 7.1σ to FP32 significance);
//   PASS_ZETA  Ω 3, V 3; PASS_ZETAD also DΩ 3, DV 3 (Gaussian-erf: ζ likewise),
//              with v_q (and w_q) taken from vw rows of the Morton order.
// Coincident pairs are dropped: the Winckelmans and ζ routines run masked,
// and the Gaussian-erf U/J routines drop them in their series branch.
constexpr int kNearThreads = 128;
constexpr float kNearPadX = 1e18f;
constexpr int kNearFoldSources = 256;   // sources a thread sums in FP32 between folds

template <int PASS>
struct NearShape {
  // Targets per thread.  U/J: four, at three CTAs per SM (168 registers, of
  // which the pass spills 192 bytes; measured at N = 1M it is still 4 % faster
  // than two targets at four CTAs).  U/J + DJ holds 27 sums per target: two.
  // The ζ passes (6 or 12 sums): four.
  static constexpr int T = PASS == PASS_UJD ? 2 : 4;
  static constexpr int TQ = kTreeBlock / T;
  static constexpr int SL = kNearThreads / TQ;
  static constexpr int NV = nval_of(PASS);
  static constexpr bool UJ = PASS == PASS_UJ || PASS == PASS_UJD;
  static constexpr int QUADS = UJ ? 2 : (PASS == PASS_ZETA ? 3 : 4);
  static constexpr size_t kQuadBytes = size_t(kNearThreads) * QUADS * sizeof(float4);
  static constexpr size_t kFoldBytes = size_t(kNearThreads) * T * NV * 2 * sizeof(float);
  static constexpr size_t kSmem = kQuadBytes + kFoldBytes;
  static constexpr int kMinBlocks = PASS == PASS_ZETA ? 4 : 3;
};

template <int KERNEL, int PASS>
__global__ void __launch_bounds__(kNearThreads, NearShape<PASS>::kMinBlocks) near_tile_kernel(
    int nfront, const int* __restrict__ onear, const int* __restrict__ nnear,
    const int2* __restrict__ near_list, const float4* __restrict__ rec,
    const float* __restrict__ vw, int64_t ldv, double* raw, int64_t ldr, int64_t n,
    int* counters, unsigned long long* pairs) {
  using Sh = NearShape<PASS>;
  constexpr int T = Sh::T, TQ = Sh::TQ, SL = Sh::SL, NV = Sh::NV;
  constexpr bool UJ = Sh::UJ;
  constexpr bool D = PASS == PASS_UJD || PASS == PASS_ZETAD;
  constexpr int PER = kNearThreads / SL;              // staged sources per thread and tile
  constexpr int FOLD_TILES = kNearFoldSources / PER;  // tiles between two folds
  static_assert(kNearThreads == 128 && kNearThreads % TQ == 0 && kTreeBlock <= kNearThreads,
                "four-warp scan below; whole target sets");
  extern __shared__ __align__(16) unsigned char near_smem[];
  float4* tA = reinterpret_cast<float4*>(near_smem);
  float4* tB = tA + kNearThreads;
  float4* tC = tB + kNearThreads;
  float4* tD = tC + kNearThreads;
  float* fold_hi = reinterpret_cast<float*>(near_smem + Sh::kQuadBytes);
  float* fold_lo = fold_hi + size_t(kNearThreads) * T * NV;
  __shared__ int s_start[kNearThreads], s_pref[kNearThreads + 1], s_wsum[4];

  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int tq = tid % TQ, sl = tid / TQ;
  const int a = int(blockIdx.x) * kTreeBlock, b = int(min(int64_t(a) + kTreeBlock, n));
  const float4 o0 = rec[3 * int64_t(a)], o1 = rec[3 * int64_t(a) + 1];
  const int64_t t0s = int64_t(blockIdx.x) * nfront, t1s = t0s + nfront - 1;
  const int l0 = onear[t0s], ln = onear[t1s] + nnear[t1s] - l0;

  float tx[T], ty[T], tz[T];
#pragma unroll
  for (int k = 0; k < T; ++k) {
    const int i = a + tq + TQ * k;
    tx[k] = ty[k] = tz[k] = 0.f;
    if (i < b) {
      const float4 r0 = rec[3 * int64_t(i)], r1 = rec[3 * int64_t(i) + 1];
      tx[k] = rel_f32(r0.x, r1.x, o0.x, o1.x);
      ty[k] = rel_f32(r0.y, r1.y, o0.y, o1.y);
      tz[k] = rel_f32(r0.z, r1.z, o0.z, o1.z);
    }
  }
  float acc[T][NV];
#pragma unroll
  for (int k = 0; k < T; ++k)
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      acc[k][v] = 0.f;
      fold_hi[(v * T + k) * kNearThreads + tid] = 0.f;
      fold_lo[(v * T + k) * kNearThreads + tid] = 0.f;
    }
  auto fold = [&]() {
#pragma unroll
    for (int k = 0; k < T; ++k)
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const int o = (v * T + k) * kNearThreads + tid;
        float s, e;
        two_sum(fold_hi[o], acc[k][v], s, e);
        fold_hi[o] = s;
        fold_lo[o] += e;
        acc[k][v] = 0.f;
      }
  };

  int tiles = 0;
  // The near ranges, kNearThreads at a time: their lengths' prefix sums in
  // shared memory; the concatenated sources are then staged in full tiles, each
  // slot finding its range by binary search.
  for (int rc0 = 0; rc0 < ln; rc0 += kNearThreads) {
    const int nr = min(kNearThreads, ln - rc0);
    int len = 0;
    __syncthreads();   // previous chunk's tiles consumed
    if (tid < nr) {
      const int2 rg = near_list[l0 + rc0 + tid];
      if (rg.x < 0 || rg.y > n || rg.x > rg.y) {
        atomicOr(&counters[kCntFlags], 8);
      } else {
        len = rg.y - rg.x;
      }
      s_start[tid] = rg.x;
    }
    int incl = len;   // inclusive scan over the 128 threads
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) s_wsum[wid] = incl;
    __syncthreads();
    for (int w = 0; w < wid; ++w) incl += s_wsum[w];
    s_pref[tid + 1] = incl;
    if (tid == 0) s_pref[0] = 0;
    __syncthreads();
    const int total = s_pref[nr];
    if (tid == 0 && pairs) atomicAdd(&pairs[0], (unsigned long long)total * (unsigned long long)(b - a));
    for (int q0 = 0; q0 < total; q0 += kNearThreads) {
      const int q = q0 + tid;
      float4 qa = make_float4(kNearPadX, kNearPadX, kNearPadX, 0.f);
      float4 qb = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 qc = make_float4(0.f, 0.f, 0.f, 0.f), qd = qc;
      // Padding constants: a unit core.
      if (UJ && KERNEL == VPM_KERNEL_WINCKELMANS) {
        qa.w = 1.f; qb.w = 1.5f;
      } else {
        qa.w = float(-0.5 * kLog2e);
        qb.w = UJ ? 1.f : float(kZeta0Gauss);
      }
      if (q < total) {
        int lo_r = 0, hi_r = nr - 1;   // last range r with s_pref[r] <= q
        while (lo_r < hi_r) {
          const int mid = (lo_r + hi_r + 1) >> 1;
          if (s_pref[mid] <= q) lo_r = mid;
          else hi_r = mid - 1;
        }
        const int64_t j = s_start[lo_r] + (q - s_pref[lo_r]);
        const float4 r0 = rec[3 * j], r1 = rec[3 * j + 1], r2 = rec[3 * j + 2];
        qa = make_float4(rel_f32(r0.x, r1.x, o0.x, o1.x), rel_f32(r0.y, r1.y, o0.y, o1.y),
                         rel_f32(r0.z, r1.z, o0.z, o1.z), r0.w);
        if (UJ) {
          qb = make_float4(r2.x, r2.y, r2.z, r1.w);
        } else {
          // Gaussian-erf ζ constants: a = -log2(e)/(2σ²) (as for U/J), b = ζ(0)/σ³.
          const float is1 = r1.w;
          qb = make_float4(r2.x, r2.y, r2.z, float(kZeta0Gauss) * is1 * is1 * is1);
          qc = make_float4(vw[j], vw[ldv + j], vw[2 * ldv + j], 0.f);
          if (D) qd = make_float4(vw[3 * ldv + j], vw[4 * ldv + j], vw[5 * ldv + j], 0.f);
        }
      }
      __syncthreads();   // previous tile consumed
      tA[tid] = qa;
      tB[tid] = qb;
      if (!UJ) {
        tC[tid] = qc;
        if (D) tD[tid] = qd;
      }
      __syncthreads();
#pragma unroll 1
      for (int m = 0; m < PER; ++m) {
        const int js = sl + SL * m;
        if constexpr (PASS == PASS_UJ) {
          if (KERNEL == VPM_KERNEL_WINCKELMANS) uj_source_winck<T, true>(tA[js], tB[js], tx, ty, tz, acc);
          else uj_source_gauss<T, true>(tA[js], tB[js], tx, ty, tz, acc);
        } else if constexpr (PASS == PASS_UJD) {
          if (KERNEL == VPM_KERNEL_WINCKELMANS) ujd_source_winck<T, true>(tA[js], tB[js], tx, ty, tz, acc);
          else ujd_source_gauss<T, true>(tA[js], tB[js], tx, ty, tz, acc);
        } else {
          zeta_source<KERNEL, T, true, D, true>(tA[js], tB[js], tC[js], D ? tD[js] : tC[js], tx,
                                                ty, tz, acc);
        }
      }
      if (++tiles % FOLD_TILES == 0) fold();
    }
  }
  fold();
  __syncthreads();
  if (tid < kTreeBlock) {
    const int i = a + tid;
    if (i < b) {
      const int k = tid / TQ, s0 = tid % TQ;
      // One value at a time (a fully unrolled epilogue would hold every slice's
      // pairs of every value in registers at once).
      double a00 = 0.0, a11 = 0.0, d00 = 0.0, d11 = 0.0;
#pragma unroll 1
      for (int w = 0; w < NV; ++w) {
        double v = 0.0;
#pragma unroll
        for (int l = 0; l < SL; ++l) {
          const int o = (w * T + k) * kNearThreads + l * TQ + s0;
          v += double(fold_hi[o]) + double(fold_lo[o]);
        }
        if (UJ && KERNEL == VPM_KERNEL_GAUSSIANERF && w >= 3 && w < 11)
          v *= kGaussAScale;   // A holds p/(-3) sums
        if (UJ) {   // A22: the FP32 forms keep J trace-free
          if (w == 3) a00 = v;
          if (w == 7) a11 = v;
          if (w == 11) v = -(a00 + a11);
        }
        if (PASS == PASS_UJD) {
          if (w == 15) d00 = v;
          if (w == 19) d11 = v;
          if (w == 23) v = -(d00 + d11);
        }
        raw[w * ldr + i] = v;
      }
    }
  }
}

template <int KERNEL, int PASS>
void launch_near(int ngroups, int nfront, const FmmWork* w, const float* vw, int64_t ldv,
                 int64_t ldr, int64_t n, unsigned long long* pairs, cudaStream_t st) {
  static const bool once = [] {
    cudaFuncSetAttribute(near_tile_kernel<KERNEL, PASS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(NearShape<PASS>::kSmem));
    return true;
  }();
  (void)once;
  near_tile_kernel<KERNEL, PASS><<<ngroups, kNearThreads, NearShape<PASS>::kSmem, st>>>(
      nfront, w->onear, w->nnear, w->near_list, w->rec, vw, ldv, w->near_raw, ldr, n, w->counters,
      pairs);
}

// Rows of a Morton-ordered array back to the original order.
__global__ void scatter_rows_kernel(int64_t n, int rows, const int* __restrict__ perm,
                                    const double* __restrict__ src, int64_t lds, double* dst,
                                    int64_t ldd) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = perm[i];
  for (int r = 0; r < rows; ++r) dst[r * ldd + o] = src[r * lds + i];
}

// Rows of an array in the original order into the Morton order.
__global__ void gather_rows_kernel(int64_t n, int rows, const int* __restrict__ perm,
                                   const double* __restrict__ src, int64_t lds, double* dst,
                                   int64_t ldd) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = perm[i];
  for (int r = 0; r < rows; ++r) dst[r * ldd + i] = src[r * lds + o];
}

// Rows of an FP64 array in the original order into FP32 rows of the Morton
// order: the ζ passes' v_q and w_q, converted once per pass rather than once
// per staged source in the near field (GB300 converts FP64 at its FP64 rate).
__global__ void gather_rows_f32_kernel(int64_t n, int rows, const int* __restrict__ perm,
                                       const double* __restrict__ src, int64_t lds, float* dst,
                                       int64_t ldd) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = perm[i];
  for (int r = 0; r < rows; ++r) dst[r * ldd + i] = float(src[r * lds + o]);
}

// FP64 near field on the sorted FP64 state (positions relative to the leaf's
// first particle; pairs with r = 0 skipped as in the direct FP64 sum).
template <int KERNEL>
__global__ void __launch_bounds__(kTreeBlock) near_f64_kernel(
    int nfront, const int* __restrict__ onear, const int* __restrict__ nnear,
    const int2* __restrict__ near_list, const double* __restrict__ sorted, int64_t ldw, double* raw,
    int64_t ldr, int64_t n, int* counters) {
  __shared__ double sx[kTreeBlock], sy[kTreeBlock], sz[kTreeBlock], sa_[kTreeBlock];
  __shared__ double sg0[kTreeBlock], sg1[kTreeBlock], sg2[kTreeBlock], sb_[kTreeBlock];
  const int tid = threadIdx.x;
  const int a = int(blockIdx.x) * kTreeBlock, b = int(min(int64_t(a) + kTreeBlock, n));
  const double cx = sorted[a], cy = sorted[ldw + a], cz = sorted[2 * ldw + a];
  const int64_t t0s = int64_t(blockIdx.x) * nfront, t1s = t0s + nfront - 1;
  const int l0 = onear[t0s], ln = onear[t1s] + nnear[t1s] - l0;
  for (int t0 = a; t0 < b; t0 += kTreeBlock) {
    const int i = t0 + tid;
    double tx = 0.0, ty = 0.0, tz = 0.0;
    if (i < b) {
      tx = sorted[i] - cx;
      ty = sorted[ldw + i] - cy;
      tz = sorted[2 * ldw + i] - cz;
    }
    double acc[15];
#pragma unroll
    for (int v = 0; v < 15; ++v) acc[v] = 0.0;
    for (int l = 0; l < ln; ++l) {
      const int2 rg = near_list[l0 + l];
      const int s_lo = rg.x, s_hi = rg.y;
      if (s_lo < 0 || s_hi > n || s_lo > s_hi) {
        if (tid == 0) atomicOr(&counters[kCntFlags], 8);
        continue;
      }
      for (int s0 = s_lo; s0 < s_hi; s0 += kTreeBlock) {
        __syncthreads();
        const int j = s0 + tid;
        if (j < s_hi) {
          sx[tid] = sorted[j] - cx;
          sy[tid] = sorted[ldw + j] - cy;
          sz[tid] = sorted[2 * ldw + j] - cz;
          sg0[tid] = sorted[3 * ldw + j];
          sg1[tid] = sorted[4 * ldw + j];
          sg2[tid] = sorted[5 * ldw + j];
          double ka, kb;
          source_consts<KERNEL, double>(sorted[6 * ldw + j], ka, kb);
          sa_[tid] = ka;
          sb_[tid] = kb;
        }
        __syncthreads();
        const int cnt = min(kTreeBlock, s_hi - s0);
        for (int js = 0; js < cnt; ++js) {
          const double dx = tx - sx[js], dy = ty - sy[js], dz = tz - sz[js];
          const double r2 = dx * dx + dy * dy + dz * dz;
          double q, p;
          pair_qp<KERNEL>(r2, sa_[js], sb_[js], q, p);
          if (r2 == 0.0) q = p = 0.0;
          const double gx = sg0[js], gy = sg1[js], gz = sg2[js];
          const double c0 = dy * gz - dz * gy, c1 = dz * gx - dx * gz, c2 = dx * gy - dy * gx;
          acc[0] += q * c0; acc[1] += q * c1; acc[2] += q * c2;
          const double p0 = p * c0, p1 = p * c1, p2 = p * c2;
          acc[3] += p0 * dx; acc[4] += p0 * dy; acc[5] += p0 * dz;
          acc[6] += p1 * dx; acc[7] += p1 * dy; acc[8] += p1 * dz;
          acc[9] += p2 * dx; acc[10] += p2 * dy; acc[11] += p2 * dz;
          acc[12] += q * gx; acc[13] += q * gy; acc[14] += q * gz;
        }
      }
    }
    if (i < b) {
#pragma unroll
      for (int k = 0; k < 15; ++k) raw[k * ldr + i] = acc[k];
    }
  }
}

// ------------------------------------------------------------ local expansions --
// Far cells at least as large as their target group are marked in the far
// list as ~s (negative) when local expansions are on: m2l_kernel turns them
// into the group's local expansion (tree.cuh), far_kernel evaluates it at each
// target (L2P) and skips them in its M2P loop.
constexpr int kLocalOrder = 7;   // Q for P = 4: L2P within a few per cent of M2P in J (tree.cuh)

// One warp per target group.  The group's local-expansion cells are taken
// kM2lChunk at a time; then
//   1. each of the first kM2lChunk lanes forms its cell's ρ, s and powers, and
//      B̃_j for |j| <= P + Q (one shared-memory row per cell);
//   2. the warp loads the chunk's moments coalesced and scales them by
//      ρ^{|k|}/k!;
//   3. lane l accumulates the local coefficients n = l + 32·q over the chunk's
//      cells, Σ_k M̃_k B̃_{k+n} times ρ(-s)^{|n|}/n!, two coefficients per
//      packed FP32 instruction.
// The group's coefficients go to loc[g·3·NQ + m·NQ + n].  Chunks of 16 cells
// keep the shared memory of a warp near 33 KB (six warps per SM).
constexpr int kM2lChunk = 16;

template <int P, int Q>
struct M2lShape {
  static constexpr int NC = ncoef(P), NQ = ncoef(Q), NB = ncoef(P + Q);
  static constexpr int ROW = NB % 2 ? NB : NB + 1;        // odd stride: lanes' rows hit distinct banks
  static constexpr int NPOW = (P + 1) + (Q + 1);          // ρ^0..ρ^P, then ρ(-s)^0..ρ(-s)^Q
  static constexpr int SLOTS = (NQ + 31) / 32;            // coefficients per lane
  static constexpr size_t kSmem = size_t(kM2lChunk) * ROW * sizeof(float) +
                                  size_t(kM2lChunk) * NC * sizeof(float4) +
                                  size_t(kM2lChunk) * NPOW * sizeof(float);
  static_assert(SLOTS % 2 == 0, "coefficient slots are packed in pairs");
};

__device__ __forceinline__ void decode_midx(int j, int& a, int& b, int& c) {
  int n = 0;
  while (ncoef(n) <= j) ++n;
  int r = j - (n > 0 ? ncoef(n - 1) : 0);
  a = n;
  while (r >= n - a + 1) {
    r -= n - a + 1;
    --a;
  }
  b = n - a - r;
  c = n - a - b;
}

__device__ __forceinline__ float inv_fact3(int a, int b, int c) {
  float f = 1.f;
  for (int i = 2; i <= a; ++i) f *= float(i);
  for (int i = 2; i <= b; ++i) f *= float(i);
  for (int i = 2; i <= c; ++i) f *= float(i);
  return 1.f / f;
}

template <int P, int Q>
__global__ void __launch_bounds__(32) m2l_kernel(int nfront, const int* __restrict__ oloc,
                                                 const int* __restrict__ nloc,
                                                 const int* __restrict__ loc_list,
                                                 const double* __restrict__ geom,
                                                 const float* __restrict__ momf,
                                                 const float4* __restrict__ ggeom, int ncells,
                                                 float* __restrict__ loc, int* counters) {
  using Sh = M2lShape<P, Q>;
  constexpr int NC = Sh::NC, NQ = Sh::NQ, ROW = Sh::ROW, NPOW = Sh::NPOW, SLOTS = Sh::SLOTS;
  constexpr int CH = kM2lChunk, H = SLOTS / 2;
  extern __shared__ __align__(16) unsigned char m2l_smem[];
  float4* sM = reinterpret_cast<float4*>(m2l_smem);                            // [cell][k]
  float* sB = reinterpret_cast<float*>(m2l_smem + size_t(CH) * NC * sizeof(float4));   // [cell][j]
  float* sP = sB + CH * ROW;                                                     // [cell][NPOW]
  __shared__ int ids[CH];
  const int lane = threadIdx.x;
  const int g = blockIdx.x;
  const float4 tg = ggeom[g];
  const double zx = tg.x, zy = tg.y, zz = tg.z;
  const double h = tg.w;

  // This lane's local coefficients n = lane + 32·q: index tables of k + n.
  int t3[SLOTS][P + 1], t2[SLOTS][P + 1], ncs[SLOTS], nord[SLOTS];
  float invf[SLOTS];
#pragma unroll
  for (int q = 0; q < SLOTS; ++q) {
    const int n = lane + 32 * q;
    int na = 0, nb = 0, nc = 0;
    if (n < NQ) decode_midx(n, na, nb, nc);
    const int nn = na + nb + nc;
    ncs[q] = nc;
    nord[q] = nn;
    invf[q] = n < NQ ? inv_fact3(na, nb, nc) : 0.f;
#pragma unroll
    for (int K = 0; K <= P; ++K) {
      const int N = K + nn;
      t3[q][K] = N * (N + 1) * (N + 2) / 6;
      const int M = K + nb + nc;
      t2[q][K] = M * (M + 1) / 2;
    }
  }
  // The moment elements e = lane + 32·i of a cell row this lane scales.
  constexpr int NE = (3 * NC + 31) / 32;
  int eord[NE];
  float efac[NE];
#pragma unroll
  for (int i = 0; i < NE; ++i) {
    const int e = lane + 32 * i;
    int a = 0, b = 0, c = 0;
    if (e < 3 * NC) decode_midx(e % NC, a, b, c);
    eord[i] = a + b + c;
    efac[i] = inv_fact3(a, b, c);
  }

  float Lacc[SLOTS][3];
#pragma unroll
  for (int q = 0; q < SLOTS; ++q) Lacc[q][0] = Lacc[q][1] = Lacc[q][2] = 0.f;

  const int64_t t0s = int64_t(g) * nfront, t1s = t0s + nfront - 1;
  const int f0 = oloc[t0s], fn = oloc[t1s] + nloc[t1s] - f0;
  for (int base = 0; base < fn; base += CH) {
    const int cnt = min(CH, fn - base);
    if (lane < cnt) {
      int cell = loc_list[f0 + base + lane];
      if (cell < 0 || cell >= ncells) {   // a list entry outside the tree: record, skip
        atomicOr(&counters[kCntFlags], 4);
        cell = -1;
      }
      ids[lane] = cell;
    }
    __syncwarp();
    // 1. this lane's cell: scale factors and B̃ row.
    if (lane < CH) {
      const int cell = lane < cnt ? ids[lane] : -1;
      double rho = 0.0;
      float rx = 1.f, ry = 0.f, rz = 0.f;
      if (cell >= 0) {
        double cx, cy, cz, cr;
        cell_centre(geom + int64_t(cell) * kGeom, cx, cy, cz, cr);
        const double dx = zx - cx, dy = zy - cy, dz = zz - cz;
        rho = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
        rx = float(dx * rho); ry = float(dy * rho); rz = float(dz * rho);
      }
      float* pw = sP + lane * NPOW;
      float v = 1.f;
#pragma unroll
      for (int j = 0; j <= P; ++j) {
        pw[j] = v;
        v *= float(rho);
      }
      const float ns = -float(h * rho);
      v = float(rho);
#pragma unroll
      for (int j = 0; j <= Q; ++j) {
        pw[P + 1 + j] = v;
        v *= ns;
      }
      scaled_taylor_unit<P + Q>(rx, ry, rz, sB + lane * ROW);
    }
    __syncwarp();
    // 2. moments of the chunk's cells, coalesced, scaled by ρ^{|k|}/k!.
    for (int c = 0; c < cnt; ++c) {
      const int cell = ids[c];
      const float* row = momf + int64_t(cell < 0 ? 0 : cell) * 3 * NC;
      const float* pw = sP + c * NPOW;
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        const int e = lane + 32 * i;
        if (e < 3 * NC) {
          const int m = e / NC, k = e % NC;
          reinterpret_cast<float*>(&sM[c * NC + k])[m] =
              cell < 0 ? 0.f : row[e] * pw[eord[i]] * efac[i];
        }
      }
    }
    __syncwarp();
    // 3. local coefficients, slots (2h, 2h + 1) packed.
    for (int c = 0; c < cnt; ++c) {
      const float* brow = sB + c * ROW;
      const float4* mrow = sM + c * NC;
      float2 acc[H][3];
#pragma unroll
      for (int q = 0; q < H; ++q) acc[q][0] = acc[q][1] = acc[q][2] = bc2(0.f);
#pragma unroll
      for (int n = 0; n <= P; ++n)
#pragma unroll
        for (int a = n; a >= 0; --a)
#pragma unroll
          for (int b = n - a; b >= 0; --b) {
            const int cc = n - a - b;
            const float4 mk = mrow[midx(a, b, cc)];
            const float2 m0 = bc2(mk.x), m1 = bc2(mk.y), m2 = bc2(mk.z);
#pragma unroll
            for (int q = 0; q < H; ++q) {
              const float2 bv =
                  make_float2(brow[t3[2 * q][n] + t2[2 * q][b + cc] + cc + ncs[2 * q]],
                              brow[t3[2 * q + 1][n] + t2[2 * q + 1][b + cc] + cc + ncs[2 * q + 1]]);
              acc[q][0] = fma2(m0, bv, acc[q][0]);
              acc[q][1] = fma2(m1, bv, acc[q][1]);
              acc[q][2] = fma2(m2, bv, acc[q][2]);
            }
          }
      const float* pw = sP + c * NPOW + P + 1;
#pragma unroll
      for (int q = 0; q < H; ++q) {
        const float fa = pw[nord[2 * q]] * invf[2 * q], fb2 = pw[nord[2 * q + 1]] * invf[2 * q + 1];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          Lacc[2 * q][m] = fmaf(fa, acc[q][m].x, Lacc[2 * q][m]);
          Lacc[2 * q + 1][m] = fmaf(fb2, acc[q][m].y, Lacc[2 * q + 1][m]);
        }
      }
    }
    __syncwarp();
  }
  float* out = loc + int64_t(g) * 3 * NQ;
#pragma unroll
  for (int q = 0; q < SLOTS; ++q) {
    const int n = lane + 32 * q;
    if (n < NQ) {
      out[n] = Lacc[q][0];
      out[NQ + n] = Lacc[q][1];
      out[2 * NQ + n] = Lacc[q][2];
    }
  }
}

// ---------------------------------------------------------------- far field --
// One thread per target (CTA per target group): the moments of the group's far
// cells at the target (M2P; the cells of the group's local expansion are on
// their own list, and l2p_kernel adds them afterwards), plus the near-field
// raw sums; U and J are written at the target's original index.
// The group's far cells are taken kFarChunk at a time: the CTA stages their
// moments and centres in shared memory with coalesced loads, then every thread
// reads them from there (broadcast) for its target.
template <int P, typename M>
__host__ __device__ constexpr int far_chunk() {
  return 12288 / int(3 * ncoef(P) * sizeof(M)) > 0 ? 12288 / int(3 * ncoef(P) * sizeof(M)) : 1;
}

template <int P, int KERNEL, typename R, typename M, bool D>
__global__ void __launch_bounds__(kTreeBlock) far_kernel(
    int64_t n, int nfront,
    const int* __restrict__ ofar, const int* __restrict__ nfar, const int* __restrict__ far_list,
    const double* __restrict__ geom, const M* __restrict__ mom, const double* __restrict__ sorted,
    int64_t ldw, const double* __restrict__ raw, int64_t ldr, const int* __restrict__ perm,
    double* U, double* J, double* DJ, int64_t ldo, int ncells, int* counters,
    unsigned long long* pairs) {
  constexpr int NC = ncoef(P), ROWM = 3 * NC, FCH = far_chunk<P, M>();
  __shared__ M smom[FCH * ROWM];
  __shared__ R sctr[FCH][3];
  const int a = int(blockIdx.x) * kTreeBlock, b = int(min(int64_t(a) + kTreeBlock, n));
  // Targets and cell centres relative to the group's first target, formed in
  // FP64 once per target and once per staged cell, so that the evaluations
  // subtract in R (GB300's FP64 pipe retires about two operations per SM and
  // cycle; three FP64 differences and conversions per evaluation cost more
  // than the FP32 work they feed).
  const double ox = sorted[a], oy = sorted[ldw + a], oz = sorted[2 * ldw + a];
  const int64_t t0s = int64_t(blockIdx.x) * nfront, t1s = t0s + nfront - 1;
  const int f0 = ofar[t0s], fn = ofar[t1s] + nfar[t1s] - f0;
  if (threadIdx.x == 0) atomicAdd(&pairs[1], (unsigned long long)fn * (unsigned long long)(b - a));
  const int i = a + int(threadIdx.x);
  const bool active = i < b;
  {
    const int ii = active ? i : a;
    const R x = R(sorted[ii] - ox), y = R(sorted[ldw + ii] - oy), z = R(sorted[2 * ldw + ii] - oz);
    R dp[9], dd[18];
#pragma unroll
    for (int k = 0; k < 9; ++k) dp[k] = R(0);
#pragma unroll
    for (int k = 0; k < 18; ++k) dd[k] = R(0);
    for (int c0 = 0; c0 < fn; c0 += FCH) {
      const int cnt = min(FCH, fn - c0);
      __syncthreads();   // previous chunk consumed
      for (int e = int(threadIdx.x); e < cnt * ROWM; e += kTreeBlock) {
        const int c = e / ROWM, k = e - c * ROWM;
        const int s = far_list[f0 + c0 + c];
        smom[e] = (s < 0 || s >= ncells) ? M(0) : mom[int64_t(s) * ROWM + k];
      }
      for (int c = int(threadIdx.x); c < cnt; c += kTreeBlock) {
        const int s = far_list[f0 + c0 + c];
        double sx = 1e18, sy = 0.0, sz = 0.0, sr;   // far away: finite, negligible terms
        if (s < 0 || s >= ncells) {   // a list entry outside the tree: record, skip (zero moments)
          atomicOr(&counters[kCntFlags], 4);
        } else {
          cell_centre(geom + int64_t(s) * kGeom, sx, sy, sz, sr);
        }
        sctr[c][0] = R(sx - ox); sctr[c][1] = R(sy - oy); sctr[c][2] = R(sz - oz);
      }
      __syncthreads();
      for (int c = 0; c < cnt; ++c) {
        R bk[ncoef(P + 2)];
        taylor_coefficients<P + 2, R>(x - sctr[c][0], y - sctr[c][1], z - sctr[c][2], bk);
        m2p_accumulate<P, R, M>(bk, smom + c * ROWM, dp, dd);
      }
    }
    if (!active) return;
    R uf[3], jf[9];
    curl_from_potential<R>(dp, dd, uf, jf);
    double v[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) v[k] = raw[k * ldr + i];
    const double w = kInv4Pi, kp = kp_to_qr<KERNEL>();
    const int64_t o = perm[i];
    U[o] = -w * v[0] + w * double(uf[0]);
    U[ldo + o] = -w * v[1] + w * double(uf[1]);
    U[2 * ldo + o] = -w * v[2] + w * double(uf[2]);
    const double w0 = v[12], w1 = v[13], w2 = v[14];
    const double jn[9] = {kp * v[3],      kp * v[4] + w2, kp * v[5] - w1,
                          kp * v[6] - w2, kp * v[7],      kp * v[8] + w0,
                          kp * v[9] + w1, kp * v[10] - w0, kp * v[11]};
#pragma unroll
    for (int k = 0; k < 9; ++k) J[k * ldo + o] = -w * jn[k] + w * double(jf[k]);
    if constexpr (D) {   // α-derivative: near field only (see near_tile_kernel)
      const double d0 = raw[24 * ldr + i], d1 = raw[25 * ldr + i], d2 = raw[26 * ldr + i];
      const double* a9 = raw + 15 * ldr + i;
      const double jd[9] = {kp * a9[0],          kp * a9[ldr] + d2,     kp * a9[2 * ldr] - d1,
                            kp * a9[3 * ldr] - d2, kp * a9[4 * ldr],    kp * a9[5 * ldr] + d0,
                            kp * a9[6 * ldr] + d1, kp * a9[7 * ldr] - d0, kp * a9[8 * ldr]};
#pragma unroll
      for (int k = 0; k < 9; ++k) DJ[k * ldo + o] = -w * jd[k];
    }
  }
}

// L2P: the group's local expansion at each of its targets, added to U and J
// (after far_kernel wrote them) at the target's original index.  A kernel of
// its own: inside far_kernel its registers would cut the M2P loop's occupancy.
template <int Q>
__global__ void __launch_bounds__(kTreeBlock) l2p_kernel(int64_t n, const float4* __restrict__ ggeom,
                                                        const float* __restrict__ loc,
                                                        const double* __restrict__ sorted,
                                                        int64_t ldw, const int* __restrict__ perm,
                                                        double* U, double* J, int64_t ldo) {
  const int64_t i = int64_t(blockIdx.x) * kTreeBlock + threadIdx.x;
  if (i >= n) return;
  const float4 tg = ggeom[blockIdx.x];
  const double ih = 1.0 / double(tg.w);
  float dp[9], dd[18];
#pragma unroll
  for (int k = 0; k < 9; ++k) dp[k] = 0.f;
#pragma unroll
  for (int k = 0; k < 18; ++k) dd[k] = 0.f;
  l2p_accumulate<Q, float>(loc + int64_t(blockIdx.x) * 3 * ncoef(Q),
                           float((sorted[i] - double(tg.x)) * ih),
                           float((sorted[ldw + i] - double(tg.y)) * ih),
                           float((sorted[2 * ldw + i] - double(tg.z)) * ih), float(ih), dp, dd);
  float uf[3], jf[9];
  curl_from_potential<float>(dp, dd, uf, jf);
  const int64_t o = perm[i];
#pragma unroll
  for (int k = 0; k < 3; ++k) U[k * ldo + o] += kInv4Pi * double(uf[k]);
#pragma unroll
  for (int k = 0; k < 9; ++k) J[k * ldo + o] += kInv4Pi * double(jf[k]);
}

// ------------------------------------------------------------------- host --
namespace {

template <typename T>
cudaError_t grow(T*& p, size_t& have, size_t need) {
  if (need <= have) return cudaSuccess;
  cudaFree(p);
  p = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc(&p, need * sizeof(T));
  if (e == cudaSuccess) have = need;
  return e;
}

cudaError_t reserve_particles(FmmWork* w, int64_t n) {
  if (n <= w->cap) return cudaSuccess;
  const int64_t cap = std::max<int64_t>(n, 1024);
  const int64_t cells = 2 * cap + 8;
  void* ptrs[] = {w->codes, w->codes_alt, w->idx, w->perm, w->sorted, w->rec, w->near_raw,
                  w->vw, w->lo, w->hi, w->child, w->nchild, w->geom, w->leaves, w->ggeom, w->cgeom,
                  w->front, w->pairs, w->counters, w->box, w->box_part, w->nfar, w->nnear,
                  w->ofar, w->onear, w->nloc, w->oloc, w->cub_tmp};
  for (void* p : ptrs) cudaFree(p);
  cudaError_t e = cudaSuccess;
  auto al = [&](auto*& p, size_t count) {
    if (e == cudaSuccess) e = cudaMalloc(&p, count * sizeof(*p));
  };
  al(w->codes, cap); al(w->codes_alt, cap); al(w->idx, cap); al(w->perm, cap);
  al(w->sorted, 7 * size_t(cap)); al(w->rec, 3 * size_t(cap)); al(w->near_raw, 27 * size_t(cap));
  al(w->vw, 6 * size_t(cap));
  al(w->lo, cells); al(w->hi, cells); al(w->child, cells); al(w->nchild, cells);
  const int64_t meta = (cap / kTreeBlock + 2) * kMaxFront;
  al(w->geom, size_t(cells) * kGeom); al(w->leaves, cells);
  al(w->ggeom, cap / kTreeBlock + 2); al(w->cgeom, 2 * size_t(cells));
  al(w->front, kMaxFront); al(w->pairs, 3);
  al(w->counters, kNumCounters); al(w->box, 4); al(w->box_part, kBoxBlocks * 6);
  al(w->nfar, meta); al(w->nnear, meta); al(w->ofar, meta); al(w->onear, meta);
  al(w->nloc, meta); al(w->oloc, meta);
  if (e != cudaSuccess) {
    w->cap = 0;
    return e;
  }
  size_t sort_bytes = 0, scan_bytes = 0;
  e = cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, w->codes, w->codes_alt, w->idx, w->perm,
                                      int(cap), 0, 63);
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, w->nfar, w->ofar, int(meta));
  if (e == cudaSuccess) {
    w->cub_bytes = std::max(sort_bytes, scan_bytes);
    e = cudaMalloc(&w->cub_tmp, w->cub_bytes);
  }
  if (e != cudaSuccess) {
    w->cap = 0;
    return e;
  }
  w->cap = cap;
  w->cell_cap = cells;
  w->meta_cap = meta;
  return cudaSuccess;
}

template <int P>
void launch_upward(FmmWork* w, int g, int ncells_in_gen, int64_t ldw, cudaStream_t st) {
  const int grid = std::max(1, std::min((3 * ncells_in_gen + 63) / 64, 4096));
  tree_upward_kernel<P><<<grid, 64, 0, st>>>(g, w->counters, w->lo, w->hi, w->child, w->nchild,
                                             w->sorted, ldw, w->geom, w->mom);
}

template <int P, int Q>
void launch_m2l(FmmWork* w, int ngroups, int nfront, int ncells, cudaStream_t st) {
  static const bool once = [] {
    cudaFuncSetAttribute(m2l_kernel<P, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(M2lShape<P, Q>::kSmem));
    return true;
  }();
  (void)once;
  m2l_kernel<P, Q><<<ngroups, 32, M2lShape<P, Q>::kSmem, st>>>(
      nfront, w->oloc, w->nloc, w->loc_list, w->geom, w->momf, w->ggeom, ncells, w->loc,
      w->counters);
}

// The far field with local expansions where `local` (FP32, p = 4; see
// fmm_eval), else M2P at every target.
template <int P>
cudaError_t launch_far(FmmWork* w, int kernel, bool f64, bool local, int64_t n, int ngroups,
                       int nfront, int ncells, int64_t ldw, double* U, double* J, double* DJ,
                       int64_t ldo, cudaStream_t st) {
  const dim3 grid(ngroups), block(kTreeBlock);
#define VPM_FAR(K, R, M, DD, mp)                                                                   \
  far_kernel<P, K, R, M, DD><<<grid, block, 0, st>>>(n, nfront, w->ofar, w->nfar, w->far_list,    \
                                                     w->geom, mp, w->sorted, ldw, w->near_raw, ldw, \
                                                     w->perm, U, J, DJ, ldo, ncells, w->counters,   \
                                                     w->pairs)
  if (DJ) {   // FP32 Gaussian-erf only (checked by the caller)
    VPM_FAR(VPM_KERNEL_GAUSSIANERF, float, float, true, w->momf);
  } else if (kernel == VPM_KERNEL_WINCKELMANS) {
    if (f64) VPM_FAR(VPM_KERNEL_WINCKELMANS, double, double, false, w->mom);
    else VPM_FAR(VPM_KERNEL_WINCKELMANS, float, float, false, w->momf);
  } else {
    if (f64) VPM_FAR(VPM_KERNEL_GAUSSIANERF, double, double, false, w->mom);
    else VPM_FAR(VPM_KERNEL_GAUSSIANERF, float, float, false, w->momf);
  }
#undef VPM_FAR
  if constexpr (P == 4) {
    if (local)
      l2p_kernel<kLocalOrder><<<grid, block, 0, st>>>(n, w->ggeom, w->loc, w->sorted, ldw, w->perm,
                                                      U, J, ldo);
  }
  return cudaGetLastError();
}

}  // namespace

bool fmm_order_supported(int p) { return p == 2 || p == 4 || p == 6; }
bool fmm_local_order_supported(int q) { return q == 0 || q == kLocalOrder; }

void fmm_stats(const FmmWork* w, int64_t* out) {
  out[0] = w ? w->last_cells : 0;
  out[1] = w ? w->last_leaves : 0;
  out[2] = w ? w->last_groups : 0;
  out[3] = w ? w->last_far : 0;
  out[4] = w ? w->last_near : 0;
  out[5] = w ? int64_t(w->h_pairs[0]) : 0;
  out[6] = w ? int64_t(w->h_pairs[1]) : 0;
  out[7] = w ? int64_t(w->h_pairs[2]) : 0;
}

// U and J of every particle of the context by the treecode (see the header).
// Returns a CUDA error, or cudaErrorInvalidValue with *why set for a tree that
// outgrew its bounds (cannot happen for the 2n + 8 cells reserved).
cudaError_t fmm_eval(vpm_ctx* c, int kernel, int prec, int p, int ncrit, double theta,
                     double sfac, int local_order, double* dj, const char** why) {
  *why = nullptr;
  const int64_t n = c->n;
  if (n == 0) return cudaSuccess;
  if (!c->fmm) c->fmm = new FmmWork();
  FmmWork* w = c->fmm;
  cudaError_t e = reserve_particles(w, n);
  if (e != cudaSuccess) return e;
  cudaStream_t st = c->st;
  const int64_t ldw = w->cap;
  const bool f64 = prec == VPM_PREC_FP64;
  // Local expansions: FP32 far fields of order-4 moments.
  const int local = local_order > 0 && p == 4 && !f64;
  // VPM_FMM_SYNC=1: synchronise after every stage so that an error names it.
  static const bool stage_sync = [] {
    const char* v = std::getenv("VPM_FMM_SYNC");
    return v && v[0] && v[0] != '0';
  }();
  const char* stage = "codes";
  auto launched = [&](int k) {
    c->launches += k;
    cudaError_t le = cudaGetLastError();
    if (le == cudaSuccess && stage_sync) le = cudaStreamSynchronize(st);
    if (le != cudaSuccess) *why = stage;
    return le;
  };

  // 1. codes, sort, gather
  box_partial_kernel<<<kBoxBlocks, 256, 0, st>>>(n, c->X, c->ld, w->box_part);
  box_final_kernel<<<1, kBoxBlocks, 0, st>>>(w->box_part, kBoxBlocks, w->box);
  morton_kernel<<<int((n + 255) / 256), 256, 0, st>>>(n, c->X, c->ld, w->box, w->codes, w->idx);
  if ((e = launched(3)) != cudaSuccess) return e;
  size_t bytes = w->cub_bytes;
  e = cub::DeviceRadixSort::SortPairs(w->cub_tmp, bytes, w->codes, w->codes_alt, w->idx, w->perm,
                                      int(n), 0, 63, st);
  if (e != cudaSuccess) return e;
  c->launches += 4;   // the radix sort's passes (counted approximately)
  const uint64_t* codes = w->codes_alt;
  gather_kernel<<<int((n + 255) / 256), 256, 0, st>>>(n, w->perm, c->X, c->G, c->S, c->ld,
                                                     w->sorted, ldw);
  if ((e = launched(1)) != cudaSuccess) return e;
  if (!f64) {
    e = launch_pack_sources(kernel, n, w->sorted, w->sorted + 3 * ldw, w->sorted + 6 * ldw, ldw,
                            1.0, w->rec, nullptr, st);
    if ((e = e == cudaSuccess ? launched(1) : e) != cudaSuccess) return e;
  }

  // 2. tree, generation by generation
  stage = "tree build";
  tree_init_kernel<<<1, 1, 0, st>>>(n, w->lo, w->hi, w->counters);
  const int split_grid = int(std::min<int64_t>((w->cell_cap + 255) / 256, 4 * 152));
  for (int g = 0; g < kMaxGen - 1; ++g) {
    tree_split_kernel<<<split_grid, 256, 0, st>>>(g, ncrit, w->cell_cap, codes, w->lo, w->hi,
                                                  w->child, w->nchild, w->leaves, w->counters);
    tree_advance_kernel<<<1, 1, 0, st>>>(g, w->counters);
  }
  if ((e = launched(1 + 2 * (kMaxGen - 1))) != cudaSuccess) return e;
  int* hc = w->h_counters;
  e = cudaMemcpyAsync(hc, w->counters, sizeof(int) * kNumCounters, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (hc[kCntFlags] != 0) {
    *why = "tree outgrew its cell bounds";
    return cudaErrorInvalidValue;
  }
  const int ncells = hc[kCntCells], nleaves = hc[kCntLeaves];
  const int ngroups = int((n + kTreeBlock - 1) / kTreeBlock);
  // Walk roots: the leaves among generations 0 and 1, and generation 2.
  int nfront = 0;
  {
    const int g2 = hc[kGenBase + 2], g3 = hc[kGenBase + 3];
    std::vector<int> nch(g2);
    e = cudaMemcpy(nch.data(), w->nchild, sizeof(int) * g2, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    int hf[kMaxFront];
    for (int cidx = 0; cidx < g2 && nfront < kMaxFront; ++cidx)
      if (nch[cidx] == 0) hf[nfront++] = cidx;
    const int leaves01 = nfront;
    for (int cidx = g2; cidx < g3 && nfront < kMaxFront; ++cidx) hf[nfront++] = cidx;
    if (nfront == 0 || nfront != leaves01 + (g3 - g2)) {   // at most 9 + 64 by construction
      *why = "tree frontier larger than expected";
      return cudaErrorInvalidValue;
    }
    e = cudaMemcpyAsync(w->front, hf, sizeof(int) * nfront, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
  }
  const int64_t nwalk = int64_t(ngroups) * nfront;
  if (nwalk > w->meta_cap) {
    *why = "treecode walk table too small";
    return cudaErrorInvalidValue;
  }

  // 3. upward pass (deepest generation first)
  const int NC = p == 2 ? ncoef(2) : p == 4 ? ncoef(4) : ncoef(6);
  if (w->mom_cells < ncells || w->mom_p != p) {
    cudaFree(w->mom);
    cudaFree(w->momf);
    w->mom = nullptr;
    w->momf = nullptr;
    w->mom_cells = 0;
    e = cudaMalloc(&w->mom, size_t(ncells) * 3 * NC * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&w->momf, size_t(ncells) * 3 * NC * sizeof(float));
    if (e != cudaSuccess) return e;
    w->mom_cells = ncells;
    w->mom_p = p;
  }
  stage = "upward pass";
  int last_gen = 0;
  for (int g = 0; g < kMaxGen; ++g)
    if (hc[kGenBase + g + 1] > hc[kGenBase + g]) last_gen = g;
  for (int g = last_gen; g >= 0; --g) {
    const int cnt = hc[kGenBase + g + 1] - hc[kGenBase + g];
    if (cnt <= 0) continue;
    if (p == 2) launch_upward<2>(w, g, cnt, ldw, st);
    else if (p == 4) launch_upward<4>(w, g, cnt, ldw, st);
    else launch_upward<6>(w, g, cnt, ldw, st);
    if ((e = launched(1)) != cudaSuccess) return e;
  }
  if (!f64) {
    const int64_t nm = int64_t(ncells) * 3 * NC;
    moments_to_f32_kernel<<<int((nm + 255) / 256), 256, 0, st>>>(nm, w->mom, w->momf);
    if ((e = launched(1)) != cudaSuccess) return e;
  }

  cell_walk_kernel<<<(ncells + 255) / 256, 256, 0, st>>>(ncells, w->geom, w->lo, w->hi, w->child,
                                                         w->nchild, w->cgeom);
  group_geom_kernel<<<(ngroups + 127) / 128, 128, 0, st>>>(n, w->sorted, ldw, w->ggeom);
  if ((e = launched(2)) != cudaSuccess) return e;

  // 4. interaction lists: count, scan, fill
  stage = "traversal";
  const int tgrid = int((nwalk + 127) / 128);
  traverse_kernel<false><<<tgrid, 128, 0, st>>>(nwalk, nfront, w->front, w->ggeom, w->cgeom,
                                                float(theta), float(sfac), local, w->nfar,
                                                w->nnear, w->nloc, nullptr, nullptr, nullptr,
                                                nullptr, nullptr, nullptr, w->counters, ncells);
  if ((e = launched(1)) != cudaSuccess) return e;
  bytes = w->cub_bytes;
  e = cub::DeviceScan::ExclusiveSum(w->cub_tmp, bytes, w->nfar, w->ofar, int(nwalk), st);
  if (e == cudaSuccess) {
    bytes = w->cub_bytes;
    e = cub::DeviceScan::ExclusiveSum(w->cub_tmp, bytes, w->nnear, w->onear, int(nwalk), st);
  }
  if (e == cudaSuccess && local) {
    bytes = w->cub_bytes;
    e = cub::DeviceScan::ExclusiveSum(w->cub_tmp, bytes, w->nloc, w->oloc, int(nwalk), st);
  }
  if (e != cudaSuccess) return e;
  c->launches += local ? 3 : 2;
  int tail[6] = {0, 0, 0, 0, 0, 0};
  e = cudaMemcpyAsync(&tail[0], w->ofar + nwalk - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&tail[1], w->nfar + nwalk - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&tail[2], w->onear + nwalk - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&tail[3], w->nnear + nwalk - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && local)
    e = cudaMemcpyAsync(&tail[4], w->oloc + nwalk - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && local)
    e = cudaMemcpyAsync(&tail[5], w->nloc + nwalk - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  const int64_t nf = int64_t(tail[0]) + tail[1], nn = int64_t(tail[2]) + tail[3];
  const int64_t nl = int64_t(tail[4]) + tail[5];
  if (nf > INT32_MAX || nn > INT32_MAX || nl > INT32_MAX) {
    *why = "treecode interaction lists exceed 2^31 entries";
    return cudaErrorInvalidValue;
  }
  const int64_t need = std::max<int64_t>(std::max(nf, nn), 1);
  if (need > w->list_cap) {
    cudaFree(w->far_list);
    cudaFree(w->near_list);
    w->far_list = nullptr;
    w->near_list = nullptr;
    w->list_cap = 0;
    e = cudaMalloc(&w->far_list, need * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&w->near_list, need * sizeof(int2));
    if (e != cudaSuccess) return e;
    w->list_cap = need;
  }
  if (local && std::max<int64_t>(nl, 1) > w->loc_list_cap) {
    cudaFree(w->loc_list);
    w->loc_list = nullptr;
    w->loc_list_cap = 0;
    e = cudaMalloc(&w->loc_list, std::max<int64_t>(nl, 1) * sizeof(int));
    if (e != cudaSuccess) return e;
    w->loc_list_cap = std::max<int64_t>(nl, 1);
  }
  e = cudaMemsetAsync(w->pairs, 0, 2 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  traverse_kernel<true><<<tgrid, 128, 0, st>>>(nwalk, nfront, w->front, w->ggeom, w->cgeom,
                                               float(theta), float(sfac), local, w->nfar,
                                               w->nnear, w->nloc, w->ofar, w->onear, w->oloc,
                                               w->far_list, w->near_list, w->loc_list,
                                               w->counters, ncells);
  if ((e = launched(1)) != cudaSuccess) return e;

  // 5. local expansions of the groups (M2L)
  if (local) {
    stage = "local expansions";
    constexpr int NQ = ncoef(kLocalOrder);
    if (int64_t(ngroups) * 3 * NQ > w->loc_cap) {
      cudaFree(w->loc);
      w->loc = nullptr;
      w->loc_cap = 0;
      e = cudaMalloc(&w->loc, size_t(ngroups) * 3 * NQ * sizeof(float));
      if (e != cudaSuccess) return e;
      w->loc_cap = int64_t(ngroups) * 3 * NQ;
    }
    launch_m2l<4, kLocalOrder>(w, ngroups, nfront, ncells, st);
    if ((e = launched(1)) != cudaSuccess) return e;
  }

  // 6. near field, 7. far field + output
  stage = "near field";
  if (f64) {
    if (kernel == VPM_KERNEL_WINCKELMANS)
      near_f64_kernel<VPM_KERNEL_WINCKELMANS><<<ngroups, kTreeBlock, 0, st>>>(
          nfront, w->onear, w->nnear, w->near_list, w->sorted, ldw, w->near_raw, ldw, n,
          w->counters);
    else
      near_f64_kernel<VPM_KERNEL_GAUSSIANERF><<<ngroups, kTreeBlock, 0, st>>>(
          nfront, w->onear, w->nnear, w->near_list, w->sorted, ldw, w->near_raw, ldw, n,
          w->counters);
  } else {
    if (dj)
      launch_near<VPM_KERNEL_GAUSSIANERF, PASS_UJD>(ngroups, nfront, w, nullptr, 0, ldw, n,
                                                    w->pairs, st);
    else if (kernel == VPM_KERNEL_WINCKELMANS)
      launch_near<VPM_KERNEL_WINCKELMANS, PASS_UJ>(ngroups, nfront, w, nullptr, 0, ldw, n,
                                                   w->pairs, st);
    else
      launch_near<VPM_KERNEL_GAUSSIANERF, PASS_UJ>(ngroups, nfront, w, nullptr, 0, ldw, n,
                                                   w->pairs, st);
  }
  if ((e = launched(1)) != cudaSuccess) return e;
  if (p == 2)
    e = launch_far<2>(w, kernel, f64, local, n, ngroups, nfront, ncells, ldw, c->U, c->J, dj,
                      c->ld, st);
  else if (p == 4)
    e = launch_far<4>(w, kernel, f64, local, n, ngroups, nfront, ncells, ldw, c->U, c->J, dj,
                      c->ld, st);
  else
    e = launch_far<6>(w, kernel, f64, local, n, ngroups, nfront, ncells, ldw, c->U, c->J, dj,
                      c->ld, st);
  stage = "far field";
  if ((e = e == cudaSuccess ? launched(local ? 2 : 1) : e) != cudaSuccess) return e;
  e = cudaMemcpyAsync(hc, w->counters, sizeof(int) * kGenBase, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(w->h_pairs, w->pairs, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (hc[kCntFlags] != 0) {
    *why = (hc[2] & 2) ? "tree traversal stack overflow" : "treecode index out of range (checked, skipped)";
    return cudaErrorInvalidValue;
  }
  w->last_cells = ncells;
  w->last_leaves = nleaves;
  w->last_groups = ngroups;
  w->last_nfront = nfront;
  w->last_far = nf + nl;
  w->h_pairs[2] = (unsigned long long)nl;
  w->last_near = nn;
  w->last_n = n;
  return cudaSuccess;
}

// The ζ sums of a pair pass (PASS_ZETA: Ω, V; PASS_ZETAD: also DΩ, DV; raw
// rows as the direct pass writes them) over the near lists of the last
// treecode evaluation, which must be of the same particle positions and cores
// (Gaussian-erf: ζ beyond the near field's 7.1σ is below FP32 significance).
cudaError_t fmm_zeta(vpm_ctx* c, bool d, const double* vs, const double* ws, double* out,
                     const char** why) {
  *why = nullptr;
  FmmWork* w = c->fmm;
  const int64_t n = c->n;
  if (!w || w->last_n != n || n == 0) {
    *why = "the treecode ζ pass needs a treecode U/J evaluation of the same field";
    return cudaErrorInvalidValue;
  }
  cudaStream_t st = c->st;
  const int64_t ldw = w->cap;
  const int ngroups = int(w->last_groups), nfront = int(w->last_nfront);
  const int grid = int((n + 255) / 256);
  gather_rows_f32_kernel<<<grid, 256, 0, st>>>(n, 3, w->perm, vs, c->ld, w->vw, ldw);
  if (d)
    gather_rows_f32_kernel<<<grid, 256, 0, st>>>(n, 3, w->perm, ws, c->ld, w->vw + 3 * ldw, ldw);
  if (d)
    launch_near<VPM_KERNEL_GAUSSIANERF, PASS_ZETAD>(ngroups, nfront, w, w->vw, ldw, ldw, n,
                                                    nullptr, st);
  else
    launch_near<VPM_KERNEL_GAUSSIANERF, PASS_ZETA>(ngroups, nfront, w, w->vw, ldw, ldw, n,
                                                   nullptr, st);
  scatter_rows_kernel<<<grid, 256, 0, st>>>(n, d ? 12 : 6, w->perm, w->near_raw, ldw, out, c->ld);
  c->launches += d ? 4 : 3;
  return cudaGetLastError();
}

}  // namespace vpm

// ------------------------------------------------------ Morton order of a pass --
namespace vpm {

// Buffers of the Morton order used by the direct pair passes (csrc/capi.cu):
// codes, the permutation and CUB scratch, apart from the treecode's own.
struct SortWork {
  int64_t cap = 0;
  int fcap = 0;                          // fields the per-field boxes hold
  uint64_t *codes = nullptr, *codes_alt = nullptr;
  int *idx = nullptr, *perm = nullptr;
  double *box = nullptr, *box_part = nullptr;
  double* fbox = nullptr;                // 4 per field: corner, cube edge
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
};

void sort_free(SortWork* s) {
  if (!s) return;
  void* ptrs[] = {s->codes, s->codes_alt, s->idx, s->perm, s->box, s->box_part, s->fbox, s->cub_tmp};
  for (void* p : ptrs) cudaFree(p);
  delete s;
}

cudaError_t sort_reserve(SortWork*& s, int64_t n, int nfields) {
  if (!s) s = new SortWork();
  if (n <= s->cap && nfields <= s->fcap) return cudaSuccess;
  n = std::max(n, s->cap);
  nfields = std::max(nfields, std::max(s->fcap, 1));
  void* ptrs[] = {s->codes, s->codes_alt, s->idx, s->perm, s->box, s->box_part, s->fbox, s->cub_tmp};
  for (void* p : ptrs) cudaFree(p);
  *s = SortWork();
  cudaError_t e = cudaSuccess;
  auto al = [&](auto*& p, size_t count) {
    if (e == cudaSuccess) e = cudaMalloc(&p, count * sizeof(*p));
  };
  al(s->codes, n); al(s->codes_alt, n); al(s->idx, n); al(s->perm, n);
  al(s->box, 4); al(s->box_part, kBoxBlocks * 6); al(s->fbox, 4 * size_t(nfields));
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(nullptr, s->cub_bytes, s->codes, s->codes_alt, s->idx,
                                        s->perm, int(n), 0, 64);
  if (e == cudaSuccess) e = cudaMalloc(&s->cub_tmp, s->cub_bytes);
  if (e != cudaSuccess) return e;
  s->cap = n;
  s->fcap = nfields;
  return cudaSuccess;
}

// perm = the particles of X (rows of leading dimension ld) along a Morton curve
// of their bounding cube, to 2^10 cells per axis (the top 30 bits of the code;
// ties keep their index order); 3 launches plus the radix sort's, no host sync.
cudaError_t sort_order(SortWork* s, int64_t n, const double* X, int64_t ld, cudaStream_t st,
                       const int** perm) {
  box_partial_kernel<<<kBoxBlocks, 256, 0, st>>>(n, X, ld, s->box_part);
  box_final_kernel<<<1, kBoxBlocks, 0, st>>>(s->box_part, kBoxBlocks, s->box);
  morton_kernel<<<int((n + 255) / 256), 256, 0, st>>>(n, X, ld, s->box, s->codes, s->idx);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  size_t bytes = s->cub_bytes;
  e = cub::DeviceRadixSort::SortPairs(s->cub_tmp, bytes, s->codes, s->codes_alt, s->idx, s->perm,
                                      int(n), 33, 63, st);
  *perm = s->perm;
  return e;
}

// Bounding cube of field f (particles [foff[f], foff[f+1]) or [foff[f], n)),
// one block per field.
__global__ void field_box_kernel(int64_t n, const int64_t* __restrict__ foff, int nfields,
                                 const double* __restrict__ X, int64_t ld, double* fbox) {
  __shared__ double s[6][256];
  const int f = blockIdx.x, t = threadIdx.x;
  const int64_t i0 = foff[f], i1 = f + 1 < nfields ? foff[f + 1] : n;
  double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = i0 + t; i < i1; i += blockDim.x)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double x = X[d * ld + i];
      v[d] = fmin(v[d], x);
      v[3 + d] = fmax(v[3 + d], x);
    }
#pragma unroll
  for (int d = 0; d < 6; ++d) s[d][t] = v[d];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (t < o) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        s[d][t] = fmin(s[d][t], s[d][t + o]);
        s[3 + d][t] = fmax(s[3 + d][t], s[3 + d][t + o]);
      }
    }
    __syncthreads();
  }
  if (t == 0) {
    const double size = fmax(fmax(s[3][0] - s[0][0], s[4][0] - s[1][0]), s[5][0] - s[2][0]);
    const bool any = i1 > i0;
    fbox[4 * f + 0] = any ? s[0][0] : 0.0;
    fbox[4 * f + 1] = any ? s[1][0] : 0.0;
    fbox[4 * f + 2] = any ? s[2][0] : 0.0;
    fbox[4 * f + 3] = any && size > 0 ? size * (1.0 + 1e-9) : 1.0;
  }
}

// Key of particle i: its field in the high bits, then the top 30 bits of its
// Morton code in the field's own cube.
__global__ void morton_fields_kernel(int64_t n, const double* __restrict__ X, int64_t ld,
                                     const int64_t* __restrict__ foff, int nfields,
                                     const double* __restrict__ fbox, uint64_t* codes, int* idx) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = nfields - 1;   // the last field whose offset is <= i
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (foff[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  const double* b = fbox + 4 * lo;
  const double scale = double(1 << 10) / b[3];
  uint64_t q[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double t = floor((X[d * ld + i] - b[d]) * scale);
    q[d] = uint64_t(fmin(fmax(t, 0.0), double((1 << 10) - 1)));
  }
  codes[i] = uint64_t(lo) << 30 | spread3(q[0]) << 2 | spread3(q[1]) << 1 | spread3(q[2]);
  idx[i] = int(i);
}

// perm for a batch of fields laid out one after another: each field's
// particles along the Morton curve of its own cube, within its own range.
cudaError_t sort_order_fields(SortWork* s, int64_t n, const double* X, int64_t ld,
                              const int64_t* foff, int nfields, cudaStream_t st, const int** perm) {
  if (nfields > s->fcap || n > s->cap) return cudaErrorInvalidValue;
  field_box_kernel<<<nfields, 256, 0, st>>>(n, foff, nfields, X, ld, s->fbox);
  morton_fields_kernel<<<int((n + 255) / 256), 256, 0, st>>>(n, X, ld, foff, nfields, s->fbox,
                                                            s->codes, s->idx);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int bits = 30;
  while (bits < 64 && (uint64_t(nfields - 1) >> (bits - 30)) != 0) ++bits;
  size_t bytes = s->cub_bytes;
  e = cub::DeviceRadixSort::SortPairs(s->cub_tmp, bytes, s->codes, s->codes_alt, s->idx, s->perm,
                                      int(n), 0, bits, st);
  *perm = s->perm;
  return e;
}

cudaError_t launch_gather_rows(int64_t n, int rows, const int* perm, const double* src,
                               int64_t lds, double* dst, int64_t ldd, cudaStream_t st) {
  if (n <= 0 || rows <= 0) return cudaSuccess;
  gather_rows_kernel<<<int((n + 255) / 256), 256, 0, st>>>(n, rows, perm, src, lds, dst, ldd);
  return cudaGetLastError();
}

cudaError_t launch_scatter_rows(int64_t n, int rows, const int* perm, const double* src,
                                int64_t lds, double* dst, int64_t ldd, cudaStream_t st) {
  if (n <= 0 || rows <= 0) return cudaSuccess;
  scatter_rows_kernel<<<int((n + 255) / 256), 256, 0, st>>>(n, rows, perm, src, lds, dst, ldd);
  return cudaGetLastError();
}

}  // namespace vpm
