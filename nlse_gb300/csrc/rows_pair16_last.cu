// Pair row-pass instantiations (16 positions per thread) for the last step:
// inverse row FFT and the nonlinear step into the natural-layout field.
// complex64, one component.
#include "pair_dispatch.cuh"

namespace nlse {
cudaError_t launch_rows_pair16_last(int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                                      bool prepare_only, int cap_per_sm) {
  return rows_pair_mode<16, ROW_INV_NL>(log2n, a, vshared, s, prepare_only, cap_per_sm);
}
}  // namespace nlse

namespace nlse {
cudaError_t launch_rows_pair16_mid(int, const StepArgs&, bool, cudaStream_t, bool, int);
cudaError_t launch_rows_pair8_mid(int, const StepArgs&, bool, cudaStream_t, bool, int);
cudaError_t launch_rows_pair8_last(int, const StepArgs&, bool, cudaStream_t, bool, int);
cudaError_t launch_rows_deep_mid(int, const StepArgs&, bool, cudaStream_t, bool, int);
cudaError_t launch_rows_deep_last(int, const StepArgs&, bool, cudaStream_t, bool, int);

cudaError_t launch_rows_pair(int mode, int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                             bool prepare_only, int cap_per_sm, int ep, bool deep) {
  const bool e8 = ep == 8;
  if (deep) {
    if (e8) return cudaErrorNotSupported;
    switch (mode) {
      case ROW_INV_NL: return launch_rows_deep_last(log2n, a, vshared, s, prepare_only, cap_per_sm);
      case ROW_INV_NL_FWD: return launch_rows_deep_mid(log2n, a, vshared, s, prepare_only, cap_per_sm);
      default: return cudaErrorNotSupported;
    }
  }
  switch (mode) {
    case ROW_INV_NL:
      return e8 ? launch_rows_pair8_last(log2n, a, vshared, s, prepare_only, cap_per_sm)
                : launch_rows_pair16_last(log2n, a, vshared, s, prepare_only, cap_per_sm);
    case ROW_INV_NL_FWD:
      return e8 ? launch_rows_pair8_mid(log2n, a, vshared, s, prepare_only, cap_per_sm)
                : launch_rows_pair16_mid(log2n, a, vshared, s, prepare_only, cap_per_sm);
    default: return cudaErrorNotSupported;
  }
}
}  // namespace nlse
