// batch_umma.cu -- the persistent batched-FFT kernels of the tensor-core form
// on tcgen05 (both directions); see k_batch_umma in batch_kernels.cuh.
#include "batch_kernels.cuh"

namespace gbfft {

cudaError_t launch_batch_umma(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_umma_t<1, IO_F2>(P, grid, st)
                  : launch_batch_umma_t<-1, IO_F2>(P, grid, st);
}

int batch_blocks_per_sm_umma(int sign) {
  return sign > 0 ? occupancy_umma_t<1, IO_F2>() : occupancy_umma_t<-1, IO_F2>();
}

}  // namespace gbfft
