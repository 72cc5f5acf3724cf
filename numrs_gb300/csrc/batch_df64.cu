// batch_df64.cu -- the persistent batched-FFT kernels of the DF64 form (both
// directions); see batch_kernels.cuh.
#include "batch_kernels.cuh"

namespace gbfft {

cudaError_t launch_batch_df64(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_t<DF64, 1, IO_F4>(P, grid, st)
                  : launch_batch_t<DF64, -1, IO_F4>(P, grid, st);
}

int batch_blocks_per_sm_df64(int sign) {
  return sign > 0 ? occupancy_t<DF64, 1, IO_F4>() : occupancy_t<DF64, -1, IO_F4>();
}

cudaError_t launch_batch_pf_df64(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_pf_t<DF64, 1, IO_F4>(P, grid, st)
                  : launch_batch_pf_t<DF64, -1, IO_F4>(P, grid, st);
}

int batch_pf_blocks_per_sm_df64(int sign) {
  return sign > 0 ? occupancy_pf_t<DF64, 1, IO_F4>() : occupancy_pf_t<DF64, -1, IO_F4>();
}

}  // namespace gbfft
