// Split-step passes on pairs of complex64 lines (packed FP32, fft_pair.cuh).
//
// The same passes as step_kernels.cuh's persistent TMA kernels, with every
// thread carrying one position of TWO lines:
//   k_rows_pair_tma  two consecutive pixel-lines (two fields at the same row
//                    when the batch has an even number of fields): inverse
//                    row FFT, 1/N, nonlinear step, [next forward row FFT];
//   k_cols_pair_tma  two adjacent columns of a blocked tile: forward column
//                    FFT, propagator, inverse column FFT.
// One-component fields, real or complex single-precision potential, real or
// complex dz; the two-component, Rabi and pump terms stay on the scalar
// kernels.  The nonlinear operator is the one of step_kernels.cuh
// (kernels_gpu.py:4-65) evaluated on both lines at once; its reciprocal is
// the hardware approximation refined by one Newton step (within an ulp of
// the reference's division).
#pragma once
#include "fft_pair.cuh"
#include "step_kernels.cuh"

namespace nlse {

__device__ __forceinline__ NLP2 load_nlp2(const float* __restrict__ P, int64_t fa, int64_t fb,
                                          int set) {
  const float* pa = P + fa * kParamStride;
  const float* pb = P + fb * kParamStride;
  NLP2 r;
  r.dz = f2(__ldg(pa + set * 16 + 0), __ldg(pb + set * 16 + 0));
  r.nalpha = f2(-__ldg(pa + set * 16 + 1), -__ldg(pb + set * 16 + 1));
  r.gs = f2(__ldg(pa + set * 16 + 2), __ldg(pb + set * 16 + 2));
  r.ris = f2(1.0f / __ldg(pa + set * 16 + 4), 1.0f / __ldg(pb + set * 16 + 4));
  r.vs = f2(__ldg(pa + set * 16 + 6), __ldg(pb + set * 16 + 6));
  r.dzi = f2(__ldg(pa + 32 + set), __ldg(pb + 32 + set));
  r.real_dz = r.dzi.x == 0.0f && r.dzi.y == 0.0f;
  return r;
}

// Shape of the pair row pass: EP positions per thread and line (16, or 8 for
// twice the threads on the same shared memory), PPC line pairs per CTA (at
// least 128 threads).
template <int N, int EP = 16>
struct RowPair {
  static constexpr int E = Shape<N, EP>::E, TPL = N / E;
  static constexpr int PPC = TPL >= 128 ? 1 : 128 / TPL;
  static constexpr int LPC = 2 * PPC;
  static constexpr int THREADS = PPC * TPL;
  static constexpr int SLS = stage_len<float>(padded_len(N));
};

template <int N, int EP = 16>
__host__ __device__ constexpr size_t rows_pair_smem() {
  return (size_t)2 * RowPair<N, EP>::LPC * RowPair<N, EP>::SLS * sizeof(float2) +
         kRowStages * sizeof(uint64_t);
}

// One work item of the pair row pass: LPC consecutive pixel-lines (PPC pairs),
// already in shared memory buffer Xs (line l at Xs + l * SLS); Xn is the other
// buffer (the second exchange buffer).  prefetch() is run by thread 0 once
// every read of Xn is complete, to refill it.  g: the item's index.
// The per-line inputs the nonlinear step of work item g reads from global
// memory -- a potential that differs between fields (v_fstride > 0) and the
// coefficient planes -- prefetched into L2 when the item's lines are
// requested (thread 0), so that those loads, issued after the inverse
// transform, hit L2 instead of waiting on HBM.  A potential shared by the
// fields stays in L2 by itself.
template <int N, int EP>
__device__ __forceinline__ void pair_prefetch_inputs(const StepArgs& a, unsigned g) {
  constexpr int LPC = RowPair<N, EP>::LPC;
  // (bulk prefetches need 16-byte aligned rows: a potential or planes at an
  // odd offset are simply not prefetched)
  const bool pv = (a.flags & F_HAS_V) && a.v_fstride != 0 &&
                  (reinterpret_cast<uintptr_t>(a.V) & 15) == 0;
  const bool pm = (a.flags & F_MAPS) && a.maps_mask &&
                  (reinterpret_cast<uintptr_t>(a.maps) & 15) == 0;
  if (!pv && !pm) return;
  const unsigned nq = (unsigned)a.nq, nf = nq / (unsigned)a.lines_per_comp;
  const unsigned q0 = g * LPC;
  const unsigned nl = nq - q0 < (unsigned)LPC ? nq - q0 : (unsigned)LPC;
  const unsigned vb = (a.flags & F_V_COMPLEX) ? 8u : 4u;
  for (unsigned l = 0; l < nl; ++l) {
    const int64_t f = (q0 + l) % nf, y = (q0 + l) / nf;
    if (pv)
      bulk_prefetch_l2(reinterpret_cast<const unsigned char*>(a.V) +
                           (f * a.v_fstride + y * (int64_t)N) * vb, N * vb);
    if (pm) {
      const float* M = reinterpret_cast<const float*>(a.maps) + f * a.maps_fstride + y * (int64_t)N;
      for (int k = 0; k < 3; ++k)
        if (a.maps_mask >> k & 1) bulk_prefetch_l2(M + k * a.maps_plane, N * 4u);
    }
  }
}

// DEEP: every exchange of both transforms in Xs (two barriers each), so Xn
// is free from the start and the next item's copies are issued right after
// the lines are read: they are in flight for the whole item, not only for the
// forward transform (twice the bytes in flight per CTA over an item).
// tms (mid-loop pass): the item's lines leave through shared memory and
// tensor-map stores issued by thread 0 instead of 8-byte stores per thread
// (a quarter of the L1 store wavefronts; the caller waits for the stores'
// reads before the buffer is written again); nullptr: direct stores.
template <int N, int EP, int MODE, bool VSHARED, bool DEEP = false, typename Prefetch>
__device__ __forceinline__ void pair_row_item(const StepArgs& a, unsigned g, float2* Xs,
                                              float2* Xn, Prefetch&& prefetch,
                                              const CUtensorMap* tms = nullptr) {
  using RP = RowPair<N, EP>;
  using C = float2;
  constexpr int E = RP::E, TPL = RP::TPL, W = BlkW<float>::W, LPC = RP::LPC, SLS = RP::SLS;
  constexpr int NEX = fft_exchanges(N, E);
  static_assert(NEX >= 1 && NEX <= 3, "one to three exchanges per transform");
  static_assert(padded_len(N) * sizeof(float4) <= 2 * SLS * sizeof(C),
                "a pair's exchange fits in its two staging lines");
  const int pp = threadIdx.x / TPL, t = threadIdx.x % TPL;
  const unsigned nq = (unsigned)a.nq;
  const unsigned nf = nq / (unsigned)a.lines_per_comp;
  auto q_f = [&](unsigned q) { return q % nf; };
  auto q_y = [&](unsigned q) { return q / nf; };
  auto buf = [&](C* B, int l) { return B + l * SLS; };
  const float2* tw = reinterpret_cast<const float2*>(a.tw);
  const float* P = a.params_f32;
  const bool has_v = a.flags & F_HAS_V;
  const bool v_cplx = a.flags & F_V_COMPLEX;
  // pairs past the end (last group) compute on in-range lines and store nothing
  const unsigned qa = g * LPC + 2 * pp;
  const bool act = qa + 1 < nq;
  const unsigned qca = act ? qa : nq - 2, qcb = qca + 1;
  const int64_t fa = q_f(qca), ma = q_y(qca), fb = q_f(qcb), mb = q_y(qcb);
  cp2 x[E];
  {
    const C* la = buf(Xs, 2 * pp);
    const C* lb = buf(Xs, 2 * pp + 1);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const C u = la[t + j * TPL], v = lb[t + j * TPL];
      x[j] = {f2(u.x, v.x), f2(u.y, v.y)};
    }
  }
  // potential: VSHARED (both lines read the same row of one shared real
  // potential) prefetches one value per position before the transform;
  // otherwise each lane's value is read when the nonlinear step needs it
  const int64_t va = fa * a.v_fstride + ma * (int64_t)N + t;
  const int64_t vb = fb * a.v_fstride + mb * (int64_t)N + t;
  float vpre[VSHARED ? E : 1];
  if constexpr (VSHARED) {
    if (has_v) {
      const float* V1 = reinterpret_cast<const float*>(a.V);
#pragma unroll
      for (int j = 0; j < E; ++j) vpre[j] = __ldg(V1 + va + j * TPL);
    }
  }
  // the first set's per-field parameters, requested before the transform
  const NLP2 pset0 = load_nlp2(P, fa, fb, 0);
  __syncthreads();  // every thread has read its lines from buffer st
  float4* sA = reinterpret_cast<float4*>(buf(Xs, 2 * pp));
  float4* sB = reinterpret_cast<float4*>(buf(Xn, 2 * pp));
  if constexpr (DEEP) {
    if (threadIdx.x == 0) prefetch();
    pfft_rest<N, E, 1, true, true>(x, t, sA, 1, tw);
  } else {
    pfft_db<N, E, 1, true, 0, 3>(x, t, sA, sB, 1, tw);
  }
  // (1/N: applied by the column pass through the blocked propagator)
  // V' = vscale * V rounded in single precision, as the reference's k/2*V array
  auto nl_all = [&](int set) {
    const NLP2 p0 = set == 0 ? pset0 : load_nlp2(P, fa, fb, set);
    if (has_v && !VSHARED && !v_cplx && !(a.flags & F_MAPS)) {
      // a real potential per field: every value of both lines requested
      // before the first use (one L2 round trip per item, not one per position)
      const float* V1 = reinterpret_cast<const float*>(a.V);
      float2 vv[E];
#pragma unroll
      for (int j = 0; j < E; ++j) vv[j] = f2(__ldg(V1 + va + j * TPL), __ldg(V1 + vb + j * TPL));
#pragma unroll
      for (int j = 0; j < E; ++j) x[j] = nl_pair_point(x[j], p0, true, mul2(p0.vs, vv[j]), f2s(0.f));
      return;
    }
#pragma unroll
    for (int j = 0; j < E; ++j) {
      NLP2 p = p0;
      if (a.flags & F_MAPS) {
        // per-pixel g, alpha/2, 1/Isat' planes replace the per-field values
        const float* M = reinterpret_cast<const float*>(a.maps);
        const int64_t ia = fa * a.maps_fstride + ma * (int64_t)N + t + j * TPL;
        const int64_t ib = fb * a.maps_fstride + mb * (int64_t)N + t + j * TPL;
        if (a.maps_mask & 1) p.gs = f2(__ldg(M + ia), __ldg(M + ib));
        if (a.maps_mask & 2)
          p.nalpha = f2(-__ldg(M + a.maps_plane + ia), -__ldg(M + a.maps_plane + ib));
        if (a.maps_mask & 4)
          p.ris = f2(__ldg(M + 2 * a.maps_plane + ia), __ldg(M + 2 * a.maps_plane + ib));
      }
      if (!has_v) {
        x[j] = nl_pair_point(x[j], p, false, f2s(0.f), f2s(0.f));
      } else if constexpr (VSHARED) {
        x[j] = nl_pair_point(x[j], p, true, mul2(p.vs, f2s(vpre[j])), f2s(0.f));
      } else if (v_cplx) {
        const float2* V2 = reinterpret_cast<const float2*>(a.V);
        const float2 u = __ldg(V2 + va + j * TPL), w = __ldg(V2 + vb + j * TPL);
        x[j] = nl_pair_point(x[j], p, true, mul2(p.vs, f2(u.x, w.x)), mul2(p.vs, f2(u.y, w.y)));
      } else {
        const float* V1 = reinterpret_cast<const float*>(a.V);
        const float2 u = f2(__ldg(V1 + va + j * TPL), __ldg(V1 + vb + j * TPL));
        x[j] = nl_pair_point(x[j], p, true, mul2(p.vs, u), f2s(0.f));
      }
    }
  };
  if (!(a.flags & F_NO_POST)) nl_all(0);
  if constexpr (MODE == ROW_INV_NL_FWD) {
    if (a.flags & F_PRE_NL) nl_all(1);
    if constexpr (DEEP) {
      pfft_rest<N, E, 1, false, true>(x, t, sA, 1, tw);
    } else {
      pfft_hook<N, E, false, true, NEX % 2 == 1>(x, t, sA, 1, tw, [&] {
        if (threadIdx.x == 0) prefetch();
      });
    }
    if (tms) {
      // the rows in natural order in this item's buffer (a row of the blocked
      // layout is its runs of W elements back to back: one tensor-map box)
      constexpr int NB = N / W, BOXB = NB < 256 ? NB : 256, NBOX = NB / BOXB;
      __syncthreads();  // every exchange read of the buffer is complete
      C* la = buf(Xs, 2 * pp);
      C* lb = buf(Xs, 2 * pp + 1);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        la[t + j * TPL] = f2(x[j].re.x, x[j].im.x);
        lb[t + j * TPL] = f2(x[j].re.y, x[j].im.y);
      }
      fence_proxy_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) {
        const unsigned q0 = g * LPC;
        const unsigned nl = nq - q0 < (unsigned)LPC ? nq - q0 : (unsigned)LPC;
        for (unsigned l = 0; l < nl; ++l) {
          const unsigned q = q0 + l;
#pragma unroll
          for (int bx = 0; bx < NBOX; ++bx)
            tensor_store_4d(tms, 0, (int)q_y(q), bx * BOXB, (int)q_f(q), buf(Xs, (int)l) + bx * BOXB * W);
        }
        bulk_commit_group();
      }
    } else if (act) {
      const int64_t lpc = a.lines_per_comp, dstr = (int64_t)TPL * lpc;
      C* da = reinterpret_cast<C*>(a.S) + fa * a.pix + ((t / W) * lpc + ma) * W + (t % W);
      C* db = reinterpret_cast<C*>(a.S) + fb * a.pix + ((t / W) * lpc + mb) * W + (t % W);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        da[j * dstr] = f2(x[j].re.x, x[j].im.x);
        db[j * dstr] = f2(x[j].re.y, x[j].im.y);
      }
    }
  } else {
    if constexpr (!DEEP) {
      __syncthreads();  // B is no longer read
      if (threadIdx.x == 0) prefetch();
    }
    if (act) {
      C* da = reinterpret_cast<C*>(a.A) + fa * a.pix + ma * N + t;
      C* db = reinterpret_cast<C*>(a.A) + fb * a.pix + mb * N + t;
#pragma unroll
      for (int j = 0; j < E; ++j) {
        da[j * TPL] = f2(x[j].re.x, x[j].im.x);
        db[j * TPL] = f2(x[j].re.y, x[j].im.y);
      }
    }
  }
}

// Persistent inverse row pass on pairs of lines of the blocked spectral
// buffer (the k_rows_tma schedule: two line buffers alternate as TMA staging
// and exchange buffers; every wait bounded).
// VSHARED: the potential is real and both lines of every pair read the same
// row of it (one potential for the batch and an even number of fields).
// (three CTAs per SM fit in shared memory: registers are capped to match)
// three CTAs per SM below 256 threads; one at 256 (4096-point rows: their
// 139 KB of staging allows no second, and a 3-CTA register cap spills)
template <int N, int EP, int MODE, bool VSHARED, bool DEEP = false>
__global__ void __launch_bounds__(RowPair<N, EP>::THREADS, RowPair<N, EP>::THREADS >= 256 ? 1 : 3)
    k_rows_pair_tma(
    const StepArgs a, const __grid_constant__ CUtensorMap tmS) {
  using RP = RowPair<N, EP>;
  using C = float2;
  constexpr int W = BlkW<float>::W, NB = N / W, LPC = RP::LPC, SLS = RP::SLS;
  constexpr int BOXB = NB < 256 ? NB : 256, NBOX = NB / BOXB;
  constexpr unsigned ROW_BYTES = N * sizeof(C);
  static_assert((SLS * sizeof(C)) % 128 == 0 && (BOXB * W * sizeof(C)) % 128 == 0,
                "tensor-map copies need 128-byte aligned shared destinations");
  extern __shared__ __align__(128) unsigned char smraw[];
  C* X = reinterpret_cast<C*>(smraw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(X + 2 * LPC * SLS);
  if (!smem_base_aligned(X)) {  // tensor-map copies need a 128-byte aligned destination
    if (threadIdx.x == 0) atomicExch(a.status, DEV_SMEM_MISALIGNED);
    return;
  }
  auto buf = [&](int b, int l) { return X + (b * LPC + l) * SLS; };
  const unsigned nq = (unsigned)a.nq;
  const unsigned ngroups = (nq + LPC - 1) / LPC;
  const unsigned nf = nq / (unsigned)a.lines_per_comp;
  auto q_f = [&](unsigned q) { return q % nf; };
  auto q_y = [&](unsigned q) { return q / nf; };
  auto issue = [&](int b, unsigned g) {
    const unsigned q0 = g * LPC;
    const unsigned nl = nq - q0 < (unsigned)LPC ? nq - q0 : (unsigned)LPC;
    mbar_arrive_expect_tx(&bar[b], nl * ROW_BYTES);
    for (unsigned l = 0; l < nl; ++l) {
      const unsigned f = q_f(q0 + l), y = q_y(q0 + l);
#pragma unroll
      for (int bx = 0; bx < NBOX; ++bx)
        tensor_load_4d(buf(b, (int)l) + bx * BOXB * W, &tmS, 0, (int)y, bx * BOXB, (int)f, &bar[b]);
    }
    pair_prefetch_inputs<N, EP>(a, g);
  };
  auto prefetch = [&](int b, unsigned gn) {
    if (gn < ngroups) {
      fence_proxy_async_smem();
      issue(b, gn);
    }
  };
  if (threadIdx.x == 0) {
    for (int st = 0; st < kRowStages; ++st) mbar_init(&bar[st], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0 && blockIdx.x < ngroups) issue(0, blockIdx.x);
  // the deep form stores the mid-loop pass's rows by tensor map from shared memory
  constexpr bool TST = DEEP && MODE == ROW_INV_NL_FWD;
  int it = 0;
  for (unsigned g = blockIdx.x; g < ngroups; g += gridDim.x, ++it) {
    const int st = it & 1;
    const unsigned par = (it >> 1) & 1;
    // the previous item's row stores have read the buffer it leaves behind
    // (written again below: exchanges or the next copy)
    if (TST && threadIdx.x == 0) bulk_wait_read_all();
    const bool ok = mbar_wait_bounded(&bar[st], par);
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) {
        atomicExch(a.status, DEV_WAIT_TIMEOUT);
        mbar_wait_bounded(&bar[st], par);
      }
      return;
    }
    pair_row_item<N, EP, MODE, VSHARED, DEEP>(
        a, g, buf(st, 0), buf(st ^ 1, 0), [&] { prefetch(st ^ 1, g + gridDim.x); },
        TST ? &tmS : nullptr);
  }
  if (TST && threadIdx.x == 0) bulk_wait_all();
}

}  // namespace nlse

namespace nlse {

// Persistent column pass over the blocked spectral buffer on column pairs:
// one tile (W = 4 columns x N rows, one contiguous run) per iteration by
// bulk copy into a two-stage ring, as k_cols_blk_tma; thread (t, p) carries
// columns 2p, 2p+1 at rows t + j*TPL (p alternates fastest, so a quarter-warp
// reads 128 contiguous bytes of the tile).  The exchanges use the staging
// tile just read (A) and one exchange tile (B), the pairs interleaved
// (element i of pair p at padi(i) * 2 + p, float4).  Forward column FFT,
// propagator, inverse column FFT; the propagator (blocked, complex64) values
// of the tile are requested before the forward transform.
// the transform's twiddles in shared memory when they fit
// DEEP: three staging tiles and no exchange tile; both transforms exchange in
// the tile just read (two barriers per exchange), so two tiles are in flight
// while one is transformed.
template <bool DEEP>
__host__ __device__ constexpr int cols_pair_stages() { return DEEP ? 3 : kColStages; }
template <int N, bool DEEP>
__host__ __device__ constexpr size_t cols_pair_base_smem() {
  return (size_t)(cols_pair_stages<DEEP>() + (DEEP ? 0 : 1)) *
             stage_len<float>(padded_len(N) * BlkW<float>::W) * sizeof(float2) +
         cols_pair_stages<DEEP>() * sizeof(uint64_t);
}
// the transform's twiddles in shared memory when they fit
template <int N, int EP, bool DEEP = false>
__host__ __device__ constexpr bool cols_pair_tws() {
  return cols_pair_base_smem<N, DEEP>() +
             (size_t)tw_compact_len(N, Shape<N, EP>::E) * sizeof(float2) + 16 <= kMaxSmemBytes;
}
template <int N, int EP = 16, bool DEEP = false>
__host__ __device__ constexpr size_t cols_pair_smem() {
  return cols_pair_base_smem<N, DEEP>() +
         (cols_pair_tws<N, EP, DEEP>() ? (size_t)tw_compact_len(N, Shape<N, EP>::E) * sizeof(float2) + 16
                                       : 0);
}

template <int N, int EP, bool DEEP = false>
__global__ void __launch_bounds__(2 * (N / Shape<N, EP>::E), 1) k_cols_pair_tma(const ColArgs a) {
  using C = float2;
  constexpr int E = Shape<N, EP>::E, TPL = N / E, W = BlkW<float>::W, TILE = N * W;
  constexpr int NST = cols_pair_stages<DEEP>();
  constexpr int SLW = stage_len<float>(padded_len(N) * W);
  static_assert((SLW * sizeof(C)) % 128 == 0, "bulk copies need aligned shared destinations");
  static_assert(padded_len(N) * 2 * sizeof(float4) <= SLW * sizeof(C),
                "both pairs' exchanges fit in one staging tile");
  constexpr unsigned TILE_BYTES = TILE * sizeof(C);
  // Exchanges alternate between the staging tile just read (A) and the
  // exchange tile (B): the forward transform starts in A, the inverse one in
  // B when the count is odd, so the inverse transform always ends in B and
  // A can be refilled right after it.
  constexpr int NEX = fft_exchanges(N, E);
  constexpr bool DB = NEX > 0;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* stage = reinterpret_cast<C*>(smraw);
  C* xch = stage + NST * SLW;
  uint64_t* bar = reinterpret_cast<uint64_t*>(xch + (DEEP ? 0 : SLW));
  constexpr bool TWS = cols_pair_tws<N, EP, DEEP>();
  C* twc = reinterpret_cast<C*>(reinterpret_cast<unsigned char*>(bar) + (NST == 3 ? 24 : 16));
  if constexpr (TWS) load_tw_compact<float, N, E>(twc, reinterpret_cast<const C*>(a.tw));
  const C* tw = TWS ? twc : reinterpret_cast<const C*>(a.tw);
  C* S = reinterpret_cast<C*>(a.A);
  const int p = threadIdx.x & 1, t = threadIdx.x >> 1;
  const int64_t ntiles = a.nblocks;
  const int64_t nouter = ntiles / a.ncb;
  auto tile_o = [&](int64_t i) { return i % nouter; };
  auto tile_b = [&](int64_t i) { return i / nouter; };
  auto tile_ptr = [&](int64_t i) { return S + tile_o(i) * a.outer_stride + tile_b(i) * TILE; };

  if (threadIdx.x == 0) {
    for (int st = 0; st < NST; ++st) mbar_init(&bar[st], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int st = 0; st < NST; ++st) {
      const int64_t i = blockIdx.x + (int64_t)st * gridDim.x;
      if (i < ntiles) {
        mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
        bulk_load(stage + st * SLW, tile_ptr(i), TILE_BYTES, &bar[st]);
      }
    }
  }
  auto refill = [&](int st, int64_t i) {
    const int64_t inext = i + (int64_t)NST * gridDim.x;
    if (inext < ntiles) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
      bulk_load(stage + st * SLW, tile_ptr(inext), TILE_BYTES, &bar[st]);
    }
  };
  int it = 0;
  for (int64_t i = blockIdx.x; i < ntiles; i += gridDim.x, ++it) {
    const int st = it % NST;
    const unsigned par = (it / NST) & 1;
    const bool ok = mbar_wait_bounded(&bar[st], par);
    if (!__syncthreads_and(ok)) {
      // give up: record it, let this tile's and the later tiles' copies land (bounded)
      if (threadIdx.x == 0) {
        atomicExch(a.status, DEV_WAIT_TIMEOUT);
        for (int k = 0; k < NST; ++k)
          if (i + (int64_t)k * gridDim.x < ntiles)
            mbar_wait_bounded(&bar[(it + k) % NST], ((it + k) / NST) & 1);
      }
      return;
    }
    cp2 x[E];
    {
      const float4* sp = reinterpret_cast<const float4*>(stage + st * SLW) + t * 2 + p;
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const float4 v = sp[j * TPL * 2];
        x[j] = {f2(v.x, v.z), f2(v.y, v.w)};
      }
    }
    const int64_t o = tile_o(i);
    const int64_t toff = tile_b(i) * (int64_t)TILE + (int64_t)t * W + 2 * p;
    const int64_t pb = (o % a.comps) * a.prop_cstride + toff;
    // propagator values of both columns (L2-resident), used after the forward FFT
    float4 pre[E];
#pragma unroll
    for (int j = 0; j < E; ++j)
      pre[j] = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const C*>(a.prop) + pb +
                                                     (int64_t)j * TPL * W));
    __syncthreads();  // every thread has read stage st
    float4* sA = reinterpret_cast<float4*>(stage + st * SLW) + p;
    float4* sB = reinterpret_cast<float4*>(xch) + p;
    if constexpr (DEEP) {
      pfft_rest<N, E, 1, false, true, TWS>(x, t, sA, 2, tw);
    } else if constexpr (DB) {
      pfft_db<N, E, 1, false, 0, 1, TWS>(x, t, sA, sB, 2, tw);
    } else {
      if (threadIdx.x == 0) refill(st, i);
      pfft_rest<N, E, 1, false, false, TWS>(x, t, sB, 2, tw);
    }
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const float2 pr = f2(pre[j].x, pre[j].z), pi = f2(pre[j].y, pre[j].w);
      x[j] = {fnma2(x[j].im, pi, mul2(x[j].re, pr)), fma2(x[j].re, pi, mul2(x[j].im, pr))};
    }
    if constexpr (DEEP) {
      pfft_rest<N, E, 1, true, true, TWS>(x, t, sA, 2, tw);
      __syncthreads();  // every read of stage st is complete
      if (threadIdx.x == 0) refill(st, i);
    } else if constexpr (DB) {
      pfft_db<N, E, 1, true, NEX % 2, 1, TWS>(x, t, sA, sB, 2, tw);
      if (threadIdx.x == 0) refill(st, i);
    } else {
      pfft_rest<N, E, 1, true, false, TWS>(x, t, sB, 2, tw);
    }
    float4* g = reinterpret_cast<float4*>(S + o * a.outer_stride + toff);
#pragma unroll
    for (int j = 0; j < E; ++j)
      g[(int64_t)j * TPL * 2] = make_float4(x[j].re.x, x[j].im.x, x[j].re.y, x[j].im.y);
  }
}

}  // namespace nlse
