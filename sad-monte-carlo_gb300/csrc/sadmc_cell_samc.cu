// The periodic-cell move kernel specialised for SAMC, the method of the uneven WCA batches: the other methods'
// bookkeeping is compiled out.
#include "sadmc_cell_kernel.cuh"

namespace sadmc {

cudaError_t launch_cell_move_samc(const MoveLaunch& m, const CellSys& s, int lpw, cudaStream_t st) {
  SADMC_CELL_ALL_SHAPES(M_SAMC)
  return cudaErrorInvalidConfiguration;
}

}  // namespace sadmc
