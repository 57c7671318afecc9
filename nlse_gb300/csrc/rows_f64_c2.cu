// Row-pass kernel instantiations, double elements, 2-component fields.
#include "dispatch_impl.cuh"

namespace nlse {
cudaError_t launch_rows_f64_c2(int mode, int log2n, const StepArgs& a, cudaStream_t s, bool prepare_only) {
  return rows_dispatch<double, 2>(mode, log2n, a, s, prepare_only);
}
}  // namespace nlse
