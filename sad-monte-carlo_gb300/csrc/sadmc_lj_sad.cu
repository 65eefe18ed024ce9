// The LJ move kernel specialised for SAD, the method of the LJ-cluster workloads: the
// other methods' bookkeeping is compiled out (fewer registers, a smaller kernel).
#include "sadmc_lj_kernel.cuh"

namespace sadmc {

cudaError_t launch_lj_move_sad(const MoveLaunch& m, const LjSys& s, int lpw, cudaStream_t st) {
  SADMC_LJ_ALL_SHAPES(M_SAD, false)
  return cudaErrorInvalidConfiguration;
}

}  // namespace sadmc
