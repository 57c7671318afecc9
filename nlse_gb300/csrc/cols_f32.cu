// Column-pass kernel instantiations, float elements.
#include "dispatch_impl.cuh"

namespace nlse {
cudaError_t launch_cols_f32(int mode, int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only) {
  return cols_dispatch<float>(mode, log2n, a, s, prepare_only);
}
cudaError_t launch_cols_blk_f32(int mode, int log2n, const ColArgs& a, cudaStream_t s,
                                bool prepare_only) {
  return cols_blk_dispatch<float>(mode, log2n, a, s, prepare_only);
}
}  // namespace nlse
