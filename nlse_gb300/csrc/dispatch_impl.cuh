// Compile-time-size dispatch of the row and column kernels.  Included by one
// translation unit per element type (rows_f32.cu, rows_f64.cu, ...), so the
// template instantiations compile in parallel.
#pragma once
#include "launch.h"

namespace nlse {

constexpr size_t kMaxSmemPerCta = 227 * 1024;

template <typename F>
static cudaError_t set_smem(F* kern, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// TMA-fed persistent variant of the inverse row passes on the blocked buffer.
template <typename T, int N, int MODE, int NC>
static cudaError_t rows_tma_n(const StepArgs& a, cudaStream_t s, bool prep, bool* used) {
  *used = false;
  constexpr bool OK_MODE = MODE == ROW_INV_NL || MODE == ROW_INV_NL_FWD;
  constexpr int W = BlkW<T>::W;
  if constexpr (OK_MODE && N >= 64 && (N / W) % ((N / W) < 256 ? (N / W) : 256) == 0 &&
                rows_tma_smem<T, N, NC>() <= kMaxSmemPerCta) {
    constexpr int E = Shape<N>::E;
    constexpr int THREADS = RowTma<T, N, NC>::THREADS;
    constexpr int LPC = RowTma<T, N, NC>::LPC;
    constexpr size_t smem = rows_tma_smem<T, N, NC>();
    auto kern = k_rows_tma<T, N, E, MODE, NC>;
    if (prep) {
      *used = true;
      return set_smem(kern, smem);
    }
    // the kernel indexes lines with 32-bit integers
    if (!(a.flags & F_IN_BLK) || a.tma_grid <= 0 || !a.tmap || a.nq >= (int64_t(1) << 31))
      return cudaSuccess;
    *used = true;
    if (a.nq <= 0) return cudaSuccess;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    if (a.cap_per_sm > 0 && a.cap_per_sm < per_sm) per_sm = a.cap_per_sm;
    const int64_t groups = (a.nq + LPC - 1) / LPC;
    int64_t g = (int64_t)a.tma_grid * per_sm;
    if (g > groups) g = groups;
    kern<<<(unsigned)g, THREADS, smem, s>>>(a, *a.tmap);
    return cudaGetLastError();
  }
  return cudaSuccess;
}

template <typename T, int N, int MODE, int NC>
static cudaError_t rows_n(const StepArgs& a, cudaStream_t s, bool prep) {
  constexpr int E = Shape<N>::E;
  using Cfg = RowCfg<N, E>;
  const size_t smem = size_t(Cfg::LPB) * Cfg::SL * sizeof(cpx<T>);
  auto kern = k_rows<T, N, E, MODE, NC>;
  {
    bool used = false;
    cudaError_t e = rows_tma_n<T, N, MODE, NC>(a, s, prep, &used);
    if (e != cudaSuccess) return e;
    if (used && !prep) return cudaSuccess;
  }
  if (prep) return set_smem(kern, smem);
  const int64_t per_block = Cfg::LPB / NC;
  const int64_t nblocks = (a.nq + per_block - 1) / per_block;
  if (nblocks <= 0) return cudaSuccess;
  kern<<<(unsigned)nblocks, Cfg::THREADS, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int MODE, int NC>
static cudaError_t rows_mode(int log2n, const StepArgs& a, cudaStream_t s, bool prep) {
  switch (log2n) {
    case 1: return rows_n<T, 2, MODE, NC>(a, s, prep);
    case 2: return rows_n<T, 4, MODE, NC>(a, s, prep);
    case 3: return rows_n<T, 8, MODE, NC>(a, s, prep);
    case 4: return rows_n<T, 16, MODE, NC>(a, s, prep);
    case 5: return rows_n<T, 32, MODE, NC>(a, s, prep);
    case 6: return rows_n<T, 64, MODE, NC>(a, s, prep);
    case 7: return rows_n<T, 128, MODE, NC>(a, s, prep);
    case 8: return rows_n<T, 256, MODE, NC>(a, s, prep);
    case 9: return rows_n<T, 512, MODE, NC>(a, s, prep);
    case 10: return rows_n<T, 1024, MODE, NC>(a, s, prep);
    case 11: return rows_n<T, 2048, MODE, NC>(a, s, prep);
    case 12: return rows_n<T, 4096, MODE, NC>(a, s, prep);
    default: return cudaErrorInvalidValue;
  }
}

// NC = 1: all modes; NC = 2: the modes that apply the nonlinear operator.
template <typename T, int NC>
static cudaError_t rows_dispatch(int mode, int log2n, const StepArgs& a, cudaStream_t s, bool prep) {
  switch (mode) {
    case ROW_FWD: return rows_mode<T, ROW_FWD, NC>(log2n, a, s, prep);
    case ROW_INV_NL: return rows_mode<T, ROW_INV_NL, NC>(log2n, a, s, prep);
    case ROW_INV_NL_FWD: return rows_mode<T, ROW_INV_NL_FWD, NC>(log2n, a, s, prep);
    case ROW_FULL: return rows_mode<T, ROW_FULL, NC>(log2n, a, s, prep);
    case ROW_INV:
      if constexpr (NC == 1) return rows_mode<T, ROW_INV, 1>(log2n, a, s, prep);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

template <typename T, int N, int MODE>
static cudaError_t cols_n(const ColArgs& a, cudaStream_t s, bool prep) {
  constexpr int E = Shape<N>::E;
  constexpr int TPL = N / E;
  const int w = prep ? (kColMaxThreads / TPL > 0 ? kColMaxThreads / TPL : 1) : a.w;
  const size_t smem = size_t(padded_len(N)) * w * sizeof(cpx<T>);
  // only the propagator pass has a complex128-propagator variant
  constexpr bool HASP = MODE == COL_FWD_PROP_INV;
  auto kern = k_cols<T, N, E, MODE, false>;
  if constexpr (HASP) {
    if (a.flags & F_PROP_C128) kern = k_cols<T, N, E, MODE, true>;
  }
  if (prep) {
    if constexpr (HASP) {
      cudaError_t e = set_smem(k_cols<T, N, E, MODE, true>, smem);
      if (e != cudaSuccess) return e;
    }
    return set_smem(k_cols<T, N, E, MODE, false>, smem);
  }
  if (w * TPL > kColMaxThreads) return cudaErrorInvalidConfiguration;
  if (a.nblocks <= 0) return cudaSuccess;
  kern<<<(unsigned)a.nblocks, w * TPL, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int MODE>
static cudaError_t cols_mode(int log2n, const ColArgs& a, cudaStream_t s, bool prep) {
  switch (log2n) {
    case 1: return cols_n<T, 2, MODE>(a, s, prep);
    case 2: return cols_n<T, 4, MODE>(a, s, prep);
    case 3: return cols_n<T, 8, MODE>(a, s, prep);
    case 4: return cols_n<T, 16, MODE>(a, s, prep);
    case 5: return cols_n<T, 32, MODE>(a, s, prep);
    case 6: return cols_n<T, 64, MODE>(a, s, prep);
    case 7: return cols_n<T, 128, MODE>(a, s, prep);
    case 8: return cols_n<T, 256, MODE>(a, s, prep);
    case 9: return cols_n<T, 512, MODE>(a, s, prep);
    case 10: return cols_n<T, 1024, MODE>(a, s, prep);
    case 11: return cols_n<T, 2048, MODE>(a, s, prep);
    case 12: return cols_n<T, 4096, MODE>(a, s, prep);
    default: return cudaErrorInvalidValue;
  }
}

// Persistent TMA-ring variant when two tiles and the exchange buffer fit in
// shared memory (one CTA per SM, grid set by the plan).

template <typename T, int N, int MODE>
static cudaError_t cols_blk_tma_n(const ColArgs& a, cudaStream_t s, bool prep, int grid, bool* used) {
  *used = false;
  if constexpr (MODE == COL_FWD_PROP_INV && cols_tma_smem<T, N>() <= kMaxSmemPerCta && N >= 64) {
    constexpr int E = Shape<N>::E;
    constexpr int THREADS = BlkW<T>::W * (N / E);
    constexpr size_t smem = cols_tma_smem<T, N>();
    auto kern = (a.flags & F_PROP_C128) ? k_cols_blk_tma<T, N, E, true>
                                        : k_cols_blk_tma<T, N, E, false>;
    *used = true;
    if (prep) {
      cudaError_t e = set_smem(k_cols_blk_tma<T, N, E, true>, smem);
      if (e != cudaSuccess) return e;
      return set_smem(k_cols_blk_tma<T, N, E, false>, smem);
    }
    if (a.nblocks <= 0) return cudaSuccess;
    // persistent grid: every CTA that fits on the SMs (one per SM for long
    // columns, several for short ones)
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    if (a.cap_per_sm > 0 && a.cap_per_sm < per_sm) per_sm = a.cap_per_sm;
    int64_t g = (int64_t)grid * per_sm;
    if (g > a.nblocks) g = a.nblocks;
    kern<<<(unsigned)g, THREADS, smem, s>>>(a);
    return cudaGetLastError();
  }
  return cudaSuccess;
}

template <typename T, int N, int MODE>
static cudaError_t cols_blk_n(const ColArgs& a, cudaStream_t s, bool prep) {
  constexpr int E = Shape<N>::E;
  constexpr int THREADS = BlkW<T>::W * (N / E);
  const size_t smem = size_t(padded_len(N)) * BlkW<T>::W * sizeof(cpx<T>);
  if (a.tma_grid > 0 || prep) {
    bool used = false;
    cudaError_t e = cols_blk_tma_n<T, N, MODE>(a, s, prep, a.tma_grid, &used);
    if (e != cudaSuccess) return e;
    if (used && !prep) return cudaSuccess;
  }
  auto kern = (a.flags & F_PROP_C128) ? k_cols_blk<T, N, E, MODE, true>
                                      : k_cols_blk<T, N, E, MODE, false>;
  if (prep) {
    cudaError_t e = set_smem(k_cols_blk<T, N, E, MODE, true>, smem);
    if (e != cudaSuccess) return e;
    return set_smem(k_cols_blk<T, N, E, MODE, false>, smem);
  }
  if (a.nblocks <= 0) return cudaSuccess;
  kern<<<(unsigned)a.nblocks, THREADS, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int MODE>
static cudaError_t cols_blk_mode(int log2n, const ColArgs& a, cudaStream_t s, bool prep) {
  switch (log2n) {
    case 4: return cols_blk_n<T, 16, MODE>(a, s, prep);
    case 5: return cols_blk_n<T, 32, MODE>(a, s, prep);
    case 6: return cols_blk_n<T, 64, MODE>(a, s, prep);
    case 7: return cols_blk_n<T, 128, MODE>(a, s, prep);
    case 8: return cols_blk_n<T, 256, MODE>(a, s, prep);
    case 9: return cols_blk_n<T, 512, MODE>(a, s, prep);
    case 10: return cols_blk_n<T, 1024, MODE>(a, s, prep);
    case 11: return cols_blk_n<T, 2048, MODE>(a, s, prep);
    case 12: return cols_blk_n<T, 4096, MODE>(a, s, prep);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
static cudaError_t cols_blk_dispatch(int mode, int log2n, const ColArgs& a, cudaStream_t s,
                                     bool prep) {
  switch (mode) {
    case COL_FWD_PROP_INV: return cols_blk_mode<T, COL_FWD_PROP_INV>(log2n, a, s, prep);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
static cudaError_t cols_dispatch(int mode, int log2n, const ColArgs& a, cudaStream_t s, bool prep) {
  switch (mode) {
    case COL_FWD: return cols_mode<T, COL_FWD>(log2n, a, s, prep);
    case COL_INV: return cols_mode<T, COL_INV>(log2n, a, s, prep);
    case COL_FWD_PROP_INV: return cols_mode<T, COL_FWD_PROP_INV>(log2n, a, s, prep);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace nlse
