// Deep-prefetch pair column-pass instantiations (complex64 fields and
// propagator, 16 positions per thread): three staging tiles, no exchange tile.
#include "pair_dispatch.cuh"

namespace nlse {
cudaError_t launch_cols_deep(int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only,
                             int cap_per_sm) {
  return cols_pair_dispatch<16, true>(log2n, a, s, prepare_only, cap_per_sm);
}
}  // namespace nlse
