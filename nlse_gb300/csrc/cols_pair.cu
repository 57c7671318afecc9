// Pair column-pass instantiations (complex64 fields and propagator).
#include "pair_dispatch.cuh"

namespace nlse {
cudaError_t launch_cols_pair(int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only,
                             int cap_per_sm) {
  switch (log2n) {
    case 6: return cols_pair_n<64>(a, s, prepare_only, cap_per_sm);
    case 7: return cols_pair_n<128>(a, s, prepare_only, cap_per_sm);
    case 8: return cols_pair_n<256>(a, s, prepare_only, cap_per_sm);
    case 9: return cols_pair_n<512>(a, s, prepare_only, cap_per_sm);
    case 10: return cols_pair_n<1024>(a, s, prepare_only, cap_per_sm);
    case 11: return cols_pair_n<2048>(a, s, prepare_only, cap_per_sm);
    case 12: return cols_pair_n<4096>(a, s, prepare_only, cap_per_sm);
    default: return cudaErrorNotSupported;
  }
}
}  // namespace nlse
