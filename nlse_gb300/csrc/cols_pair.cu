// Pair column-pass instantiations (complex64 fields and propagator), 16 and 8
// positions per thread.
#include "pair_dispatch.cuh"

namespace nlse {
cudaError_t launch_cols_deep(int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only,
                             int cap_per_sm);

cudaError_t launch_cols_pair(int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only,
                             int cap_per_sm, int ep, bool deep) {
  if (deep)
    return ep == 8 ? cudaErrorNotSupported
                   : launch_cols_deep(log2n, a, s, prepare_only, cap_per_sm);
  return ep == 8 ? cols_pair_dispatch<8>(log2n, a, s, prepare_only, cap_per_sm)
                 : cols_pair_dispatch<16>(log2n, a, s, prepare_only, cap_per_sm);
}
}  // namespace nlse
