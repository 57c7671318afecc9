// Row-pass kernel instantiations, float elements, 1-component fields.
#include "dispatch_impl.cuh"

namespace nlse {
cudaError_t launch_rows_f32_c1(int mode, int log2n, const StepArgs& a, cudaStream_t s, bool prepare_only) {
  return rows_dispatch<float, 1>(mode, log2n, a, s, prepare_only);
}
}  // namespace nlse
