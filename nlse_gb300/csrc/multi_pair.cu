// Launchers of the one-launch-per-pass kernels over several plans
// (step_multi.cuh); the row kernels are instantiated in multi_rows_*.cu.
#include <cstring>

#include "launch.h"
#include "step_multi.cuh"

namespace nlse {

cudaError_t rows_multi_mid(const RowMulti& m, int nsm, cudaStream_t s, bool prep);
cudaError_t rows_multi_last(const RowMulti& m, int nsm, cudaStream_t s, bool prep);

int multi_max_plans() { return kMultiMax; }

cudaError_t launch_rows_multi(int mode, int n, const StepArgs* a, const CUtensorMap* const* tm,
                              const int* log2n, int nsm, cudaStream_t s, bool prep) {
  static RowMulti dummy;
  if (prep) {
    cudaError_t e = rows_multi_mid(dummy, 0, s, true);
    if (e != cudaSuccess) return e;
    return rows_multi_last(dummy, 0, s, true);
  }
  if (n < 1 || n > kMultiMax) return cudaErrorInvalidValue;
  RowMulti m;
  memset(&m, 0, sizeof(m));
  unsigned items = 0;
  for (int k = 0; k < n; ++k) {
    if (log2n[k] < kMultiLog2Min || log2n[k] > kMultiLog2Max) return cudaErrorNotSupported;
    const int N = 1 << log2n[k], TPL = N / 16, PPC = TPL >= 128 ? 1 : 128 / TPL, LPC = 2 * PPC;
    m.tm[k] = *tm[k];
    m.p[k].a = a[k];
    m.p[k].log2n = log2n[k];
    m.p[k].item0 = items;
    m.p[k].items = (unsigned)((a[k].nq + LPC - 1) / LPC);
    items += m.p[k].items;
  }
  m.nplans = n;
  m.items = items;
  if (!items) return cudaSuccess;
  return mode == ROW_INV_NL ? rows_multi_last(m, nsm, s, false) : rows_multi_mid(m, nsm, s, false);
}

cudaError_t launch_cols_tile_multi(int n, const ColArgs* c, const int* log2n, cudaStream_t s,
                                   bool prep) {
  constexpr size_t smem = kMultiTileSmem;
  if (prep)
    return cudaFuncSetAttribute(k_cols_tile_multi<>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
  if (n < 1 || n > kMultiMax) return cudaErrorInvalidValue;
  ColMulti m;
  memset(&m, 0, sizeof(m));
  unsigned items = 0;
  for (int k = 0; k < n; ++k) {
    if (log2n[k] < kMultiLog2Min || log2n[k] > kMultiLog2Max) return cudaErrorNotSupported;
    const int sub = 2048 >> log2n[k];
    m.p[k].c = c[k];
    m.p[k].log2n = log2n[k];
    m.p[k].item0 = items;
    m.p[k].items = (unsigned)((c[k].nblocks + sub - 1) / sub);
    items += m.p[k].items;
  }
  m.nplans = n;
  m.items = items;
  if (!items) return cudaSuccess;
  k_cols_tile_multi<><<<items, kMultiTileThreads, smem, s>>>(m);
  return cudaGetLastError();
}

}  // namespace nlse
