// batch_tc32.cu -- the persistent batched-FFT kernels of the TC32 form (both
// directions); see batch_kernels.cuh.
#include "batch_kernels.cuh"

namespace gbfft {

cudaError_t launch_batch_tc32(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_t<TC32, 1, IO_F2>(P, grid, st)
                  : launch_batch_t<TC32, -1, IO_F2>(P, grid, st);
}

int batch_blocks_per_sm_tc32(int sign) {
  return sign > 0 ? occupancy_t<TC32, 1, IO_F2>() : occupancy_t<TC32, -1, IO_F2>();
}

cudaError_t launch_batch_pf_tc32(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_pf_t<TC32, 1, IO_F2>(P, grid, st)
                  : launch_batch_pf_t<TC32, -1, IO_F2>(P, grid, st);
}

int batch_pf_blocks_per_sm_tc32(int sign) {
  return sign > 0 ? occupancy_pf_t<TC32, 1, IO_F2>() : occupancy_pf_t<TC32, -1, IO_F2>();
}

}  // namespace gbfft
