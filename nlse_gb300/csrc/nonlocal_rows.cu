// Row passes of the nonlocal convolution on the zero-padded grid, fused with
// their neighbours (the convolution itself: NLSE/nlse.py:406-408, 444-447,
// oaconvolve(|A|^2, nl_profile, "same")):
//   k_pack_rows_fwd   |A|^2 of the field's components packed as one complex
//                     line (component 0 real, component 1 imaginary), zero-
//                     padded to the padded width, forward row transform;
//                     rows of the padding stored as zeros (their transform);
//   k_rows_inv_nl_pad inverse row transform of the field's rows (the padding
//                     rows are not needed), the 2-D transform's 1/N, and the
//                     nonlinear step of the field's pixels with the convolved
//                     intensities (nl_pad.cuh).
// The arithmetic is that of the separate passes (k_pack_asq, the ROW_FWD and
// ROW_INV row passes, k_nl_point_pad); complex64 fields, padded widths 512 to
// 4096.
#include "launch.h"
#include "nl_pad.cuh"

namespace nlse {

template <int N, int NC>
__global__ void __launch_bounds__(RowCfg<N, Shape<N>::E>::THREADS)
    k_pack_rows_fwd(const float2* __restrict__ A, float2* __restrict__ X, int64_t nlines,
                    int64_t ny, int64_t nx, int64_t py, const float2* __restrict__ tw) {
  using C = float2;
  constexpr int E = Shape<N>::E, TPL = N / E;
  using Cfg = RowCfg<N, E>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int li = threadIdx.x / TPL, t = threadIdx.x % TPL;
  const int64_t line = (int64_t)blockIdx.x * Cfg::LPB + li;  // over fields x padded rows
  const int64_t f = line / py, y = line % py;
  C* dst = X + line * N + t;
  // LPB divides ny and py: a block's lines are all field rows or all padding
  const int64_t y0 = ((int64_t)blockIdx.x * Cfg::LPB) % py;
  if (y0 >= ny) {
    if (line < nlines) {
#pragma unroll
      for (int j = 0; j < E; ++j) dst[j * TPL] = make_float2(0.f, 0.f);
    }
    return;
  }
  const int64_t pix = ny * nx;
  const C* src = A + (f * NC) * pix + y * nx;
  C x[E];
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const int64_t xi = t + j * TPL;
    x[j] = make_float2(0.f, 0.f);
    if (xi < nx) {
      x[j].x = abs2<float>(src[xi]);
      if (NC == 2) x[j].y = abs2<float>(src[pix + xi]);
    }
  }
  fft_line<float, N, E, 1, false>(x, t, sm + li * Cfg::SL, 1, tw);
#pragma unroll
  for (int j = 0; j < E; ++j) dst[j * TPL] = x[j];
}

template <int N, int NC>
__global__ void __launch_bounds__(RowCfg<N, Shape<N>::E>::THREADS)
    k_rows_inv_nl_pad(const StepArgs a, const float2* __restrict__ X, int64_t nlines, int64_t ny,
                      int64_t nx, int64_t py, int set, float inv_n, const float2* __restrict__ tw) {
  using C = float2;
  constexpr int E = Shape<N>::E, TPL = N / E;
  using Cfg = RowCfg<N, E>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int li = threadIdx.x / TPL, t = threadIdx.x % TPL;
  const int64_t line = (int64_t)blockIdx.x * Cfg::LPB + li;  // over fields x field rows
  const bool act = line < nlines;
  const int64_t lc = act ? line : nlines - 1;
  const int64_t f = lc / ny, y = lc % ny;
  const C* src = X + (f * py + y) * N + t;
  C x[E];
#pragma unroll
  for (int j = 0; j < E; ++j) x[j] = src[j * TPL];
  fft_line<float, N, E, 1, true>(x, t, sm + li * Cfg::SL, 1, tw);
  if (!act) return;
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const int64_t xi = t + j * TPL;
    if (xi < nx) nl_pad_point<float, NC>(a, f, y * nx + xi, cscale<float>(x[j], inv_n), set);
  }
}

template <int N>
static cudaError_t pack_fwd_n(int nc, const void* A, void* X, int64_t nfields, int64_t ny,
                              int64_t nx, int64_t py, const void* tw, cudaStream_t s) {
  using Cfg = RowCfg<N, Shape<N>::E>;
  const size_t smem = (size_t)Cfg::LPB * Cfg::SL * sizeof(float2);
  const int64_t nlines = nfields * py;
  const unsigned grid = (unsigned)((nlines + Cfg::LPB - 1) / Cfg::LPB);
  auto k1 = k_pack_rows_fwd<N, 1>;
  auto k2 = k_pack_rows_fwd<N, 2>;
  auto k = nc == 1 ? k1 : k2;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k<<<grid, Cfg::THREADS, smem, s>>>(reinterpret_cast<const float2*>(A),
                                    reinterpret_cast<float2*>(X), nlines, ny, nx, py,
                                    reinterpret_cast<const float2*>(tw));
  return cudaGetLastError();
}

template <int N>
static cudaError_t inv_nl_n(const StepArgs& a, const void* X, int64_t ny, int64_t nx, int64_t py,
                            int set, float inv_n, cudaStream_t s) {
  using Cfg = RowCfg<N, Shape<N>::E>;
  const size_t smem = (size_t)Cfg::LPB * Cfg::SL * sizeof(float2);
  const int64_t nf = a.nq / a.lines_per_comp;
  const int64_t nlines = nf * ny;
  const unsigned grid = (unsigned)((nlines + Cfg::LPB - 1) / Cfg::LPB);
  auto k1 = k_rows_inv_nl_pad<N, 1>;
  auto k2 = k_rows_inv_nl_pad<N, 2>;
  auto k = a.comps == 1 ? k1 : k2;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k<<<grid, Cfg::THREADS, smem, s>>>(a, reinterpret_cast<const float2*>(X), nlines, ny, nx, py,
                                    set, inv_n, reinterpret_cast<const float2*>(a.tw));
  return cudaGetLastError();
}

bool nonlocal_rows_fused(int dtype, int log2px, int64_t ny, int64_t py) {
  // complex64, padded widths 512 .. 4096, the lines of a block (LPB) dividing
  // both the field's and the padded row counts: every block's lines are all
  // field rows or all padding rows, and the line counts are whole blocks
  if (dtype != 0 || log2px < 9 || log2px > 12) return false;
  const int tpl = (1 << log2px) / 16, lpb = 256 / tpl >= 2 ? 256 / tpl : 2;
  return ny % lpb == 0 && py % lpb == 0;
}

cudaError_t launch_pack_rows_fwd(int log2px, int nc, const void* A, void* X, int64_t nfields,
                                 int64_t ny, int64_t nx, int64_t py, const void* tw,
                                 cudaStream_t s) {
  switch (log2px) {
    case 9: return pack_fwd_n<512>(nc, A, X, nfields, ny, nx, py, tw, s);
    case 10: return pack_fwd_n<1024>(nc, A, X, nfields, ny, nx, py, tw, s);
    case 11: return pack_fwd_n<2048>(nc, A, X, nfields, ny, nx, py, tw, s);
    case 12: return pack_fwd_n<4096>(nc, A, X, nfields, ny, nx, py, tw, s);
    default: return cudaErrorNotSupported;
  }
}

cudaError_t launch_rows_inv_nl_pad(int log2px, const StepArgs& a, const void* X, int64_t ny,
                                   int64_t nx, int64_t py, int set, float inv_n, cudaStream_t s) {
  switch (log2px) {
    case 9: return inv_nl_n<512>(a, X, ny, nx, py, set, inv_n, s);
    case 10: return inv_nl_n<1024>(a, X, ny, nx, py, set, inv_n, s);
    case 11: return inv_nl_n<2048>(a, X, ny, nx, py, set, inv_n, s);
    case 12: return inv_nl_n<4096>(a, X, ny, nx, py, set, inv_n, s);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace nlse
