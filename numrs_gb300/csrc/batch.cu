// batch.cu -- form dispatch of the persistent batched-FFT launchers.  The
// kernels of each form live in their own translation unit (batch_<form>.cu).
#include "batch.h"

namespace gbfft {

cudaError_t launch_batch(Form f, int sign, const BatchParams& P, int grid, cudaStream_t st) {
  switch (f) {
    case FORM_F64: return launch_batch_f64(sign, P, grid, st);
    case FORM_F32: return launch_batch_f32(sign, P, grid, st);
    case FORM_TC32: return launch_batch_tc32(sign, P, grid, st);
    default: return launch_batch_df64(sign, P, grid, st);
  }
}

int batch_blocks_per_sm(Form f, int sign) {
  switch (f) {
    case FORM_F64: return batch_blocks_per_sm_f64(sign);
    case FORM_F32: return batch_blocks_per_sm_f32(sign);
    case FORM_TC32: return batch_blocks_per_sm_tc32(sign);
    default: return batch_blocks_per_sm_df64(sign);
  }
}

cudaError_t launch_batch_pf(Form f, int sign, const BatchParams& P, int grid, cudaStream_t st) {
  switch (f) {
    case FORM_F32: return launch_batch_pf_f32(sign, P, grid, st);
    case FORM_TC32: return launch_batch_pf_tc32(sign, P, grid, st);
    case FORM_DF64: return launch_batch_pf_df64(sign, P, grid, st);
    default: return cudaErrorInvalidValue;
  }
}

int batch_pf_blocks_per_sm(Form f, int sign) {
  switch (f) {
    case FORM_F32: return batch_pf_blocks_per_sm_f32(sign);
    case FORM_TC32: return batch_pf_blocks_per_sm_tc32(sign);
    case FORM_DF64: return batch_pf_blocks_per_sm_df64(sign);
    default: return 0;
  }
}

}  // namespace gbfft
