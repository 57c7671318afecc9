// Compile-time-size dispatch of the pair kernels (step_pair.cuh).  Included by
// the rows_pair*.cu, rows_deep*.cu and cols_*.cu translation units.
#pragma once
#include "launch.h"
#include "step_pair.cuh"

namespace nlse {

template <typename F>
static cudaError_t pair_set_smem(F* kern, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Persistent grid: SMs x the CTAs that fit on one (capped at cap_per_sm when
// that is positive), at most `units`.
template <typename F>
static cudaError_t persistent_grid(F* kern, int threads, size_t smem, int nsm, int cap_per_sm,
                                   int64_t units, unsigned* grid) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (cap_per_sm > 0 && cap_per_sm < per_sm) per_sm = cap_per_sm;
  int64_t g = (int64_t)nsm * per_sm;
  if (g > units) g = units;
  if (g < 1) g = 1;
  *grid = (unsigned)g;
  return cudaSuccess;
}

template <int N, int EP, int MODE, bool VS, bool DEEP>
static cudaError_t rows_pair_nv(const StepArgs& a, cudaStream_t s, bool prep, int cap) {
  using RP = RowPair<N, EP>;
  constexpr size_t smem = rows_pair_smem<N, EP>();
  static_assert(smem <= 227 * 1024, "pair row pass shared memory");
  auto kern = k_rows_pair_tma<N, EP, MODE, VS, DEEP>;
  if (prep) return pair_set_smem(kern, smem);
  if (a.nq <= 0) return cudaSuccess;
  unsigned grid = 0;
  const int64_t groups = (a.nq + RP::LPC - 1) / RP::LPC;
  cudaError_t e = persistent_grid(kern, RP::THREADS, smem, a.tma_grid, cap, groups, &grid);
  if (e != cudaSuccess) return e;
  kern<<<grid, RP::THREADS, smem, s>>>(a, *a.tmap);
  return cudaGetLastError();
}

template <int N, int EP, int MODE, bool DEEP>
static cudaError_t rows_pair_n(const StepArgs& a, bool vshared, cudaStream_t s, bool prep, int cap) {
  if (prep) {
    cudaError_t e = rows_pair_nv<N, EP, MODE, true, DEEP>(a, s, true, cap);
    if (e != cudaSuccess) return e;
    return rows_pair_nv<N, EP, MODE, false, DEEP>(a, s, true, cap);
  }
  return vshared ? rows_pair_nv<N, EP, MODE, true, DEEP>(a, s, false, cap)
                 : rows_pair_nv<N, EP, MODE, false, DEEP>(a, s, false, cap);
}

// DEEP: the deep-prefetch form (k_rows_pair_tma)
template <int EP, int MODE, bool DEEP = false>
static cudaError_t rows_pair_mode(int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                                  bool prep, int cap) {
  switch (log2n) {
    case 6: return rows_pair_n<64, EP, MODE, DEEP>(a, vshared, s, prep, cap);
    case 7: return rows_pair_n<128, EP, MODE, DEEP>(a, vshared, s, prep, cap);
    case 8: return rows_pair_n<256, EP, MODE, DEEP>(a, vshared, s, prep, cap);
    case 9: return rows_pair_n<512, EP, MODE, DEEP>(a, vshared, s, prep, cap);
    case 10: return rows_pair_n<1024, EP, MODE, DEEP>(a, vshared, s, prep, cap);
    case 11: return rows_pair_n<2048, EP, MODE, DEEP>(a, vshared, s, prep, cap);
    case 12: return rows_pair_n<4096, EP, MODE, DEEP>(a, vshared, s, prep, cap);
    default: return cudaErrorNotSupported;
  }
}

// Sizes whose staging tiles (and exchange tile) fit in shared memory.
template <int N, int EP, bool DEEP>
static cudaError_t cols_pair_n(const ColArgs& a, cudaStream_t s, bool prep, int cap) {
  if constexpr (cols_pair_smem<N, EP, DEEP>() > 227 * 1024 || 2 * (N / Shape<N, EP>::E) > 1024) {
    return cudaErrorNotSupported;
  } else {
    constexpr int THREADS = 2 * (N / Shape<N, EP>::E);
    constexpr size_t smem = cols_pair_smem<N, EP, DEEP>();
    auto kern = k_cols_pair_tma<N, EP, DEEP>;
    if (prep) return pair_set_smem(kern, smem);
    if (a.nblocks <= 0) return cudaSuccess;
    unsigned grid = 0;
    cudaError_t e = persistent_grid(kern, THREADS, smem, a.tma_grid, cap, a.nblocks, &grid);
    if (e != cudaSuccess) return e;
    kern<<<grid, THREADS, smem, s>>>(a);
    return cudaGetLastError();
  }
}

template <int EP, bool DEEP = false>
static cudaError_t cols_pair_dispatch(int log2n, const ColArgs& a, cudaStream_t s, bool prep,
                                      int cap) {
  switch (log2n) {
    case 6: return cols_pair_n<64, EP, DEEP>(a, s, prep, cap);
    case 7: return cols_pair_n<128, EP, DEEP>(a, s, prep, cap);
    case 8: return cols_pair_n<256, EP, DEEP>(a, s, prep, cap);
    case 9: return cols_pair_n<512, EP, DEEP>(a, s, prep, cap);
    case 10: return cols_pair_n<1024, EP, DEEP>(a, s, prep, cap);
    case 11: return cols_pair_n<2048, EP, DEEP>(a, s, prep, cap);
    case 12: return cols_pair_n<4096, EP, DEEP>(a, s, prep, cap);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace nlse
