// The periodic-cell move kernel specialised for Wang-Landau, the method of the square-well contact-count workloads: the other methods'
// bookkeeping is compiled out.
#include "sadmc_cell_kernel.cuh"

namespace sadmc {

cudaError_t launch_cell_move_wl(const MoveLaunch& m, const CellSys& s, int lpw, cudaStream_t st) {
  SADMC_CELL_ALL_SHAPES(M_WL)
  return cudaErrorInvalidConfiguration;
}

}  // namespace sadmc
