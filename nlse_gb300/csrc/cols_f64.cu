// Column-pass kernel instantiations, double elements.
#include "dispatch_impl.cuh"

namespace nlse {
cudaError_t launch_cols_f64(int mode, int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only) {
  return cols_dispatch<double>(mode, log2n, a, s, prepare_only);
}
cudaError_t launch_cols_blk_f64(int mode, int log2n, const ColArgs& a, cudaStream_t s,
                                bool prepare_only) {
  return cols_blk_dispatch<double>(mode, log2n, a, s, prepare_only);
}
}  // namespace nlse
