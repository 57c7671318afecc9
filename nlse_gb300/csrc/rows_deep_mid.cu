// Deep-prefetch pair row-pass instantiations (16 positions per thread) for
// the steps inside the loop: inverse row FFT, nonlinear step, next forward
// row FFT.  complex64, one component.
#include "pair_dispatch.cuh"

namespace nlse {
cudaError_t launch_rows_deep_mid(int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                                 bool prepare_only, int cap_per_sm) {
  return rows_pair_mode<16, ROW_INV_NL_FWD, true>(log2n, a, vshared, s, prepare_only, cap_per_sm);
}
}  // namespace nlse
