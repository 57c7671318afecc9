// One persistent launch per pass for a batch of plans with different grids.
//
// A mixed batch (e.g. 96 fields at 256^2, 48 at 512^2, 16 at 1024^2 and 4 at
// 2048^2) is several plans; these kernels advance all of them in one launch
// per pass.  The work of every plan is one list of items:
//   k_rows_pair_multi  item = the LPC pixel-lines of one pair row-pass group
//                      of one plan (128 threads and the same 2 x 34.8 KB of
//                      shared memory at every grid size from 256 to 2048);
//   k_cols_tile_multi  item = 2048/N blocked column tiles of one plan, side
//                      by side (512 threads: W * N/16 per tile; one CTA per
//                      item, no persistence, as k_cols_blk).
// The row pass's persistent CTAs take items blockIdx.x, blockIdx.x +
// gridDim.x, ...; the next item's copies (possibly another plan's) are issued
// at the start of the current item (the deep form of step_pair.cuh, whose
// pair_row_item this shares).  Every wait is bounded.
#pragma once
#include "step_pair.cuh"

namespace nlse {

constexpr int kMultiMax = 8;      // plans per launch
constexpr int kMultiLog2Min = 8;  // grids of 256 ...
constexpr int kMultiLog2Max = 11; // ... to 2048 points per axis

// Row-pass buffer of one stage: LPC lines of SLS elements, the same for
// every N in [256, 2048] with 16 positions per thread.
constexpr int kMultiRowHalf = 2 * RowPair<2048>::SLS;
static_assert(RowPair<256>::LPC * RowPair<256>::SLS == kMultiRowHalf &&
                  RowPair<512>::LPC * RowPair<512>::SLS == kMultiRowHalf &&
                  RowPair<1024>::LPC * RowPair<1024>::SLS == kMultiRowHalf,
              "row-pass stage buffers of every grid size have one length");

// Every tensor-map copy of the multi row pass lands on a 128-byte boundary
// inside its stage buffer: line l < LPC of grid N at stage b goes to
// b * kMultiRowHalf + l * SLS(N) (+ 256 runs of 32 bytes per box).
__host__ __device__ constexpr bool multi_row_copies_aligned() {
  for (int lg = kMultiLog2Min; lg <= kMultiLog2Max; ++lg) {
    const int N = 1 << lg, TPL = N / 16, PPC = TPL >= 128 ? 1 : 128 / TPL, LPC = 2 * PPC;
    const int SLS = stage_len<float>(padded_len(N));
    const int NB = N / 4, BOXB = NB < 256 ? NB : 256;
    for (int b = 0; b < 2; ++b)
      for (int l = 0; l < LPC; ++l)
        for (int bx = 0; bx * BOXB < NB; ++bx) {
          const long off = ((long)b * kMultiRowHalf + (long)l * SLS + (long)bx * BOXB * 4) * 8;
          if (off % 128 != 0) return false;
        }
    if (LPC * SLS > kMultiRowHalf) return false;
  }
  return true;
}
static_assert(multi_row_copies_aligned(), "multi row pass: copy destinations aligned and in bounds");

struct RowPlanArgs {
  StepArgs a;       // the plan's step arguments (F_IN_BLK, out flags, parameters)
  unsigned items;   // its line groups
  unsigned item0;   // index of its first item in the launch's list
  int log2n;        // row length
};

struct __align__(64) RowMulti {
  CUtensorMap tm[kMultiMax];  // each plan's tensor map of its blocked buffer
  RowPlanArgs p[kMultiMax];
  int nplans;
  unsigned items;
};

__host__ __device__ constexpr size_t rows_multi_smem() {
  return (size_t)2 * kMultiRowHalf * sizeof(float2) + kRowStages * sizeof(uint64_t);
}

// Plan of a work item (the plans' items follow each other in the list).
template <typename M>
__device__ __forceinline__ int multi_plan_of(unsigned item, const M& m) {
  int k = 0;
  while (k + 1 < m.nplans && item >= m.p[k + 1].item0) ++k;
  return k;
}

template <int MODE>
__global__ void __launch_bounds__(128, 3) k_rows_pair_multi(const __grid_constant__ RowMulti m) {
  using C = float2;
  constexpr int W = BlkW<float>::W;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* X = reinterpret_cast<C*>(smraw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(X + 2 * kMultiRowHalf);
  if (!smem_base_aligned(X)) {  // tensor-map copies need a 128-byte aligned destination
    if (threadIdx.x == 0 && m.nplans > 0) atomicExch(m.p[0].a.status, DEV_SMEM_MISALIGNED);
    return;
  }
  // copies of item `item` into stage b (thread 0)
  auto issue = [&](int b, unsigned item) {
    const int k = multi_plan_of(item, m);
    const RowPlanArgs& P = m.p[k];
    const int N = 1 << P.log2n;
    const int TPL = N / 16, PPC = TPL >= 128 ? 1 : 128 / TPL, LPC = 2 * PPC;
    // the line stride pair_row_item reads with: the padded line rounded up to
    // 128 bytes (every line's tensor-map copy needs a 128-byte aligned destination)
    const int SLS = stage_len<float>(padded_len(N));
    const int NB = N / W, BOXB = NB < 256 ? NB : 256, NBOX = NB / BOXB;
    const unsigned nq = (unsigned)P.a.nq, nf = nq / (unsigned)P.a.lines_per_comp;
    const unsigned q0 = (item - P.item0) * LPC;
    const unsigned nl = nq - q0 < (unsigned)LPC ? nq - q0 : (unsigned)LPC;
    mbar_arrive_expect_tx(&bar[b], nl * (unsigned)N * (unsigned)sizeof(C));
    for (unsigned l = 0; l < nl; ++l) {
      const unsigned q = q0 + l, f = q % nf, y = q / nf;
      for (int bx = 0; bx < NBOX; ++bx)
        tensor_load_4d(X + b * kMultiRowHalf + l * SLS + bx * BOXB * W, &m.tm[k], 0, (int)y,
                       bx * BOXB, (int)f, &bar[b]);
    }
    switch (P.log2n) {
      case 8: pair_prefetch_inputs<256, 16>(P.a, item - P.item0); break;
      case 9: pair_prefetch_inputs<512, 16>(P.a, item - P.item0); break;
      case 10: pair_prefetch_inputs<1024, 16>(P.a, item - P.item0); break;
      default: pair_prefetch_inputs<2048, 16>(P.a, item - P.item0); break;
    }
  };
  if (threadIdx.x == 0) {
    for (int st = 0; st < kRowStages; ++st) mbar_init(&bar[st], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0 && blockIdx.x < m.items) issue(0, blockIdx.x);
  // the deep item form (the next item's copies issued at the item's start) with
  // the mid-loop pass's rows stored by tensor map from shared memory
  constexpr bool TST = MODE == ROW_INV_NL_FWD;
  int it = 0;
  for (unsigned item = blockIdx.x; item < m.items; item += gridDim.x, ++it) {
    const int st = it & 1;
    const unsigned par = (it >> 1) & 1;
    const int k = multi_plan_of(item, m);
    const StepArgs& a = m.p[k].a;
    // the previous item's row stores have read the buffer the next copy fills
    if (TST && threadIdx.x == 0) bulk_wait_read_all();
    const bool ok = mbar_wait_bounded(&bar[st], par);
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) {
        atomicExch(a.status, DEV_WAIT_TIMEOUT);
        mbar_wait_bounded(&bar[st], par);
      }
      return;
    }
    const unsigned g = item - m.p[k].item0, next = item + gridDim.x;
    C* Xs = X + st * kMultiRowHalf;
    C* Xn = X + (st ^ 1) * kMultiRowHalf;
    auto prefetch = [&] {
      if (next < m.items) {
        fence_proxy_async_smem();
        issue(st ^ 1, next);
      }
    };
    const CUtensorMap* tms = TST ? &m.tm[k] : nullptr;
    switch (m.p[k].log2n) {
      case 8: pair_row_item<256, 16, MODE, false, true>(a, g, Xs, Xn, prefetch, tms); break;
      case 9: pair_row_item<512, 16, MODE, false, true>(a, g, Xs, Xn, prefetch, tms); break;
      case 10: pair_row_item<1024, 16, MODE, false, true>(a, g, Xs, Xn, prefetch, tms); break;
      default: pair_row_item<2048, 16, MODE, false, true>(a, g, Xs, Xn, prefetch, tms); break;
    }
  }
  if (TST && threadIdx.x == 0) bulk_wait_all();
}

// ---- column pass --------------------------------------------------------------
struct ColPlanArgs {
  ColArgs c;      // the plan's blocked column arguments (S, blocked propagator)
  unsigned items; // its items (2048/N tiles each)
  unsigned item0;
  int log2n;      // column length
};

struct ColMulti {
  ColPlanArgs p[kMultiMax];
  int nplans;
  unsigned items;
};

// ---- column pass, tile form ------------------------------------------------
// One CTA of 512 threads per work item, no persistence: an item is 2048/N
// blocked tiles of one plan (W columns x N rows each, W * N/16 threads per
// tile), loaded straight from global memory, transformed with the scalar FFT
// (packed complex sums), multiplied by the blocked propagator and transformed
// back -- k_cols_blk's arithmetic.  Many resident warps instead of a copy
// ring hide the latency.
constexpr int kMultiTileThreads = BlkW<float>::W * (2048 / 16);
constexpr int kMultiTileSmem = padded_len(2048) * BlkW<float>::W * (int)sizeof(float2);

template <int N>
__device__ __forceinline__ void tile_col_item(const ColArgs& c, unsigned g, float2* smem) {
  using C = float2;
  constexpr int E = 16, TPL = N / E, W = BlkW<float>::W, THR = W * TPL, SUB = 2048 / N;
  constexpr int SLT = padded_len(N) * W;  // one tile's exchange buffer
  static_assert(THR * SUB == kMultiTileThreads, "sub-tiles fill the CTA");
  static_assert(SLT * SUB * (int)sizeof(C) <= kMultiTileSmem, "sub-tile buffers fit");
  const int s = threadIdx.x / THR, lt = threadIdx.x % THR;
  const int cc = lt % W, t = lt / W;
  const int64_t ti = (int64_t)g * SUB + s;
  const bool act = ti < c.nblocks;
  const int64_t tc = act ? ti : c.nblocks - 1;
  // a CTA's sub-tiles are adjacent column blocks of one field (contiguous)
  const int64_t b = tc % c.ncb, o = tc / c.ncb;
  const int64_t toff = b * (int64_t)(N * W) + t * W + cc;
  C* base = reinterpret_cast<C*>(c.A) + o * c.outer_stride + toff;
  const C* tw = reinterpret_cast<const C*>(c.tw);
  C* sm = smem + s * SLT + cc;
  C x[E];
#pragma unroll
  for (int j = 0; j < E; ++j) x[j] = base[j * TPL * W];
  fft_line<float, N, E, 1, false>(x, t, sm, W, tw);
  const int64_t pb = (o % c.comps) * c.prop_cstride + toff;
#pragma unroll
  for (int j = 0; j < E; ++j) x[j] = mul_prop<float, false>(x[j], c.prop, pb + j * TPL * W);
  fft_line<float, N, E, 1, true>(x, t, sm, W, tw);
  if (act) {
#pragma unroll
    for (int j = 0; j < E; ++j) base[j * TPL * W] = x[j];
  }
}

// two CTAs per SM (64 registers, 2 x 69.6 KB), as k_cols_blk at 2048 points
template <int UNUSED = 0>
__global__ void __launch_bounds__(kMultiTileThreads, 2) k_cols_tile_multi(
    const __grid_constant__ ColMulti m) {
  extern __shared__ __align__(128) unsigned char smraw[];
  float2* sm = reinterpret_cast<float2*>(smraw);
  const unsigned item = blockIdx.x;
  const int k = multi_plan_of(item, m);
  const ColArgs& c = m.p[k].c;
  const unsigned g = item - m.p[k].item0;
  switch (m.p[k].log2n) {
    case 8: tile_col_item<256>(c, g, sm); break;
    case 9: tile_col_item<512>(c, g, sm); break;
    case 10: tile_col_item<1024>(c, g, sm); break;
    default: tile_col_item<2048>(c, g, sm); break;
  }
}

}  // namespace nlse
