// The multi-plan pair row pass (ROW_INV_NL): one persistent launch over the lines of
// every plan of a batch (step_multi.cuh).
#include "launch.h"
#include "step_multi.cuh"

namespace nlse {
cudaError_t rows_multi_last(const RowMulti& m, int nsm, cudaStream_t s, bool prep) {
  constexpr size_t smem = rows_multi_smem();
  static_assert(smem <= 227 * 1024, "multi row pass shared memory");
  auto kern = k_rows_pair_multi<ROW_INV_NL>;
  if (prep) return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  unsigned grid = (unsigned)nsm * per_sm;
  if (grid > m.items) grid = m.items;
  kern<<<grid, 128, smem, s>>>(m);
  return cudaGetLastError();
}
}  // namespace nlse
