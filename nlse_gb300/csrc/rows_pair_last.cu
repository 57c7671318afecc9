// Pair row-pass instantiations for the last step (inverse row FFT and the
// nonlinear step into the natural-layout field); complex64, one component.
#include "pair_dispatch.cuh"

namespace nlse {
cudaError_t launch_rows_pair_last(int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                                  bool prepare_only, int cap_per_sm) {
  return rows_pair_mode<ROW_INV_NL>(log2n, a, vshared, s, prepare_only, cap_per_sm);
}

cudaError_t launch_rows_pair_mid(int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                                 bool prepare_only, int cap_per_sm);

cudaError_t launch_rows_pair(int mode, int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                             bool prepare_only, int cap_per_sm) {
  switch (mode) {
    case ROW_INV_NL: return launch_rows_pair_last(log2n, a, vshared, s, prepare_only, cap_per_sm);
    case ROW_INV_NL_FWD: return launch_rows_pair_mid(log2n, a, vshared, s, prepare_only, cap_per_sm);
    default: return cudaErrorNotSupported;
  }
}
}  // namespace nlse
