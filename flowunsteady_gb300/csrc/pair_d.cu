// pair_d.cu — instantiates the α-derivative pair passes (PASS_UJD, PASS_ZETAD)
// of the analytic dynamic SFS procedure; see pair_kernel.cuh.
#include "pair_kernel.cuh"

namespace vpm {

size_t pair_smem_bytes_d(int pass, int precision, Shape s) {
  return pass == PASS_UJD ? smem_of<PASS_UJD>(precision, s) : smem_of<PASS_ZETAD>(precision, s);
}

int pair_ctas_per_sm_d(int pass, int kernel, int precision, Shape s) {
  return pass == PASS_UJD ? ctas_per_sm<PASS_UJD>(kernel, precision, s)
                          : ctas_per_sm<PASS_ZETAD>(kernel, precision, s);
}

int pair_max_active_clusters_d(int pass, int kernel, int precision, Shape s, int cluster) {
  return pass == PASS_UJD ? max_active_clusters<PASS_UJD>(kernel, precision, s, cluster)
                          : max_active_clusters<PASS_ZETAD>(kernel, precision, s, cluster);
}

cudaError_t launch_pair_d(int pass, int kernel, int precision, Shape s, const PairArgs& a,
                          int grid, cudaStream_t st) {
  return pass == PASS_UJD ? launch<PASS_UJD>(kernel, precision, s, a, grid, st)
                          : launch<PASS_ZETAD>(kernel, precision, s, a, grid, st);
}

cudaError_t launch_reduce_d(int pass, int kernel, int precision, const double* part, int64_t ldp,
                            const int64_t* foff, const int32_t* fchunks, int nfields,
                            int scalar_chunks, int64_t t_begin, int64_t t_end, double* u,
                            double* j, double* dj, int64_t ldo, cudaStream_t st) {
  if (pass == PASS_UJD)
    return reduce<PASS_UJD>(kernel, precision, part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin,
                            t_end, u, j, dj, ldo, st);
  return reduce<PASS_ZETAD>(kernel, precision, part, ldp, foff, fchunks, nfields, scalar_chunks, t_begin,
                            t_end, u, j, dj, ldo, st);
}

}  // namespace vpm
