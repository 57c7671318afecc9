// Deep-prefetch pair row-pass instantiations (16 positions per thread) for
// the last step: inverse row FFT and the nonlinear step into the
// natural-layout field.  complex64, one component.
#include "pair_dispatch.cuh"

namespace nlse {
cudaError_t launch_rows_deep_last(int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                                  bool prepare_only, int cap_per_sm) {
  return rows_pair_mode<16, ROW_INV_NL, true>(log2n, a, vshared, s, prepare_only, cap_per_sm);
}
}  // namespace nlse
