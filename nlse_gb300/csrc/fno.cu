// Fourier-neural-operator surrogate of the 256 x 256 split-step propagation:
// forward, backward and optimiser kernels for sm_103a.
//
// Model (grid N = 256, C = 32 channels, retained modes kx in [0, 32) and
// ky in [0, 32) u [N-32, N): 2048 modes; bf16() is round-to-nearest-even):
//   h0      = bf16(lift(x))                      x: Re E0, Im E0, V + 2 scalars
//   z_l     = h_l . bf16(Wc_l) + s_l + b_l       1 x 1 convolution on tensor cores
//   s_l     = (1/N^2) Re( sum_{k in R} S_l(k) exp(+2 pi i k.x / N) )
//             (its row stage as a BF16 contraction: bf16(cos), bf16(sin) and
//             the row spectra as bf16(U / N^2), FP32 sums)
//   S_l(k)  = bf16(H_l(k)) . bf16(W_l(k))        per-mode 32 x 32 complex mixing
//   H_l(k)  = sum_x h_l(x) exp(-2 pi i k.x / N)  truncated transform
//             (its row stage as a BF16 contraction over quarter rows:
//             bf16(cos), bf16(sin) of 2 pi kx x'/N, exact (-i)^(kx q), FP32 sums)
//   h_{l+1} = bf16(GELU(z_l)) (l < 3),  h_4 = bf16(z_3)   GELU in its tanh form
//   out     = h_4 . Wp + bp                      two channels: Re, Im of E(L)
// Forward: the row stages of both truncated transforms are tcgen05 BF16 x
// BF16 -> FP32 contractions (the synthesis accumulated onto the 1 x 1
// convolution), the column stages 256-point transforms of the kept kx on the
// project's Stockham FFT (fft_core.cuh), the mode mixing a tcgen05 product per
// mode.  Backward: the same mixing and convolution products; the row
// transforms of the gradients on the FFT (256-point lines of channel pairs
// packed as one complex line).  Accumulators live in tensor memory
// (umma.cuh); weight gradients are FP32 reductions on the CUDA cores.
// Rounding steps pass gradients through unchanged.  No reference
// counterpart: the surrogate is new to this project.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "fft_core.cuh"
#include "internal.h"
#include "nlse_fno.h"
#include "nlse_gb300.h"
#include "tma.cuh"
#include "umma.cuh"

namespace nlse {
namespace fno {

constexpr int N = NLSE_FNO_N, C = NLSE_FNO_C, KX = 32, KY = 64, NM = NLSE_FNO_MODES;
static_assert(NM == KX * KY, "mode count");
constexpr int E = 16, TPL = N / E;  // 16 threads per 256-point line
constexpr int SL = padded_len(N);   // padded line length in shared memory
constexpr int ROWC = KX * C;        // complex values of one row's half spectrum [kx][c]
constexpr int TILE_M = 128;         // batch rows per mixing tile
constexpr int XK = 2 * C;           // mixing K: [Re | Im] of the 32 channels
constexpr int XTILE = TILE_M * XK;  // BF16 elements per mixing A tile
constexpr int WBIG = XK * XK;       // real 64 x 64 form of one mode's complex weights
constexpr int WCONV = C * C;
constexpr int PS = 17;              // pair stride of the [pixel][channel pair] buffers
constexpr size_t kPairBuf =
    (16 * SL > N * PS ? 16 * SL : N * PS) * sizeof(float2);  // shared by xl and the pairs

// GELU in its tanh form, 0.5 z (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3),
// with the hardware tanh (relative error ~2^-11, below the BF16 rounding of
// the stored activations)
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kGeluA = 0.7978845608028654f, kGeluB = 0.044715f;
__device__ __forceinline__ float gelu(float z) {
  const float t = tanh_hw(kGeluA * fmaf(kGeluB * z, z * z, z));
  return 0.5f * z * (1.f + t);
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float t = tanh_hw(kGeluA * fmaf(kGeluB * z, z * z, z));
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * kGeluA * fmaf(3.f * kGeluB, z * z, 1.f);
}
// kept row iy (0..63) of ky
__device__ __forceinline__ int iy_of(int ky) { return ky < KY / 2 ? ky : ky - (N - KY); }


__device__ __forceinline__ void load_bf16x32(const __nv_bfloat16* src, float (&v)[32]) {
  __align__(16) __nv_bfloat16 b[32];
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(b);
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] = s[i];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __bfloat162float(b[i]);
}

// 32 floats as 16 packed BF16 pairs (round to nearest even), element 2i in the
// low half of word i: the memory order of 32 consecutive BF16 values
struct Bf16x32 {
  uint4 q[4];
};
__device__ __forceinline__ Bf16x32 pack_bf16x32(const float (&v)[32]) {
  Bf16x32 r;
  uint32_t* w = reinterpret_cast<uint32_t*>(r.q);
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const __nv_bfloat162 b = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    w[i] = *reinterpret_cast<const uint32_t*>(&b);
  }
  return r;
}
__device__ __forceinline__ void store_packed(__nv_bfloat16* dst, const Bf16x32& b) {
  uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] = b.q[i];
}
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// ---- row transforms (one CTA of 256 threads per image row) ----------------
// The exchange lines xl (16 x SL) and the pair buffer [pixel][channel pair]
// (N x PS) are never live at once, so the kernels give both the same
// storage (kPairBuf bytes): row_analysis reads its input before the first
// exchange (whose leading barrier orders the reuse) and row_synthesis writes
// its output after a barrier that follows the last exchange.
// Forward half spectrum of one row of 32 real channels.  hs holds the row as
// channel pairs, hs[x*PS + j] = (h_2j(x), h_2j+1(x)); line j is transformed as
// z = h_2j + i h_2j+1 and split with H_2j = (Z(k) + conj Z(-k))/2,
// H_2j+1 = (Z(k) - conj Z(-k))/(2i).  out: [kx][c], kx < KX.
__device__ void row_analysis(const float2* hs, float2* xl, const float2* tw, float2* out) {
  const int j = threadIdx.x >> 4, t = threadIdx.x & 15;
  float2 x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) x[e] = hs[(t + TPL * e) * PS + j];
  float2* sl = xl + j * SL;
  fft_line<float, N, E, 1, false>(x, t, sl, 1, tw);
  __syncthreads();
#pragma unroll
  for (int e = 0; e < E; ++e) sl[padi(t + TPL * e)] = x[e];
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ROWC / 256; ++r) {
    const int i = threadIdx.x + 256 * r;
    const int kx = i >> 5, c = i & 31;
    const float2* z = xl + (c >> 1) * SL;
    const float2 a = z[padi(kx)], b = z[padi((N - kx) & (N - 1))];
    out[i] = (c & 1) ? make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x))
                     : make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
  }
}

// s_c(x) = scale * Re( sum_{kx < KX} U_c(kx) exp(+2 pi i kx x / N) ) for the 32
// channels of one row, from its half spectrum U[kx][c]; channel pairs share one
// inverse transform of Z(k) = (U_2j(k) + i U_2j+1(k))/2 at k = kx and
// (conj U_2j(kx) + i conj U_2j+1(kx))/2 at k = N - kx (both halves at k = 0).
// Result in ss[x*PS + j].
__device__ void row_synthesis(const float2* __restrict__ U, float scale, float2* xl,
                              const float2* tw, float2* ss) {
  const int j = threadIdx.x >> 4, t = threadIdx.x & 15;
  float2 x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) x[e] = make_float2(0.f, 0.f);
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const int kx = t + TPL * e;
    const float4 u = *reinterpret_cast<const float4*>(U + kx * C + 2 * j);
    x[e] = kx == 0 ? make_float2(u.x, u.z) : make_float2(0.5f * (u.x - u.w), 0.5f * (u.y + u.z));
  }
#pragma unroll
  for (int e = E - 2; e < E; ++e) {
    const int kx = N - (t + TPL * e);
    if (kx < KX) {
      const float4 u = *reinterpret_cast<const float4*>(U + kx * C + 2 * j);
      x[e] = make_float2(0.5f * (u.x + u.w), 0.5f * (u.z - u.y));
    }
  }
  fft_line<float, N, E, 1, true>(x, t, xl + j * SL, 1, tw);
  __syncthreads();  // ss may share storage with the exchange lines
#pragma unroll
  for (int e = 0; e < E; ++e) ss[(t + TPL * e) * PS + j] = make_float2(scale * x[e].x, scale * x[e].y);
}

// ---- column transforms -----------------------------------------------------
// 256-point transforms along y of 16 adjacent (kx, c) columns of one field.
// Analysis keeps ky in [0, 32) u [N-32, N): X (BF16, mixing A operand in the
// tcgen05 layout, rows = fields) and optionally Hs [m][b][c] (FP32; the BF16
// values when round_saved, else the unrounded ones).
__global__ void __launch_bounds__(256) k_cols_analysis(const float2* __restrict__ T, int nb, int nmt,
                                                        float scale, int round_saved,
                                                        __nv_bfloat16* __restrict__ Xc,
                                                        float2* __restrict__ Hs, const float2* tw) {
  __shared__ __align__(16) float2 sm[SL * 16];
  const int l = threadIdx.x & 15, t = threadIdx.x >> 4;
  const int b = blockIdx.x / (ROWC / 16), q = (blockIdx.x % (ROWC / 16)) * 16 + l;
  const float2* src = T + (int64_t)b * N * ROWC + q;
  float2 x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) x[e] = src[(int64_t)(t + TPL * e) * ROWC];
  fft_line<float, N, E, 1, false>(x, t, sm + l, 16, tw);
  const int kx = q >> 5, c = q & 31, mt = b / TILE_M, r = b % TILE_M;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int e = i < 2 ? i : i + (E - 4);
    const int m = iy_of(t + TPL * e) * KX + kx;
    const float vr = scale * x[e].x, vi = scale * x[e].y;
    const __nv_bfloat16 br = __float2bfloat16_rn(vr), bi = __float2bfloat16_rn(vi);
    __nv_bfloat16* tile = Xc + ((int64_t)m * nmt + mt) * XTILE;
    tile[umma_off(r, c, XK)] = br;
    tile[umma_off(r, C + c, XK)] = bi;
    if (Hs)
      Hs[((int64_t)m * nb + b) * C + c] =
          round_saved ? make_float2(__bfloat162float(br), __bfloat162float(bi)) : make_float2(vr, vi);
  }
}

// Zero-filled inverse column transforms (unnormalised) from the kept ky of
// Y [m][b][c] to U [b][y][kx][c].
__global__ void __launch_bounds__(256) k_cols_synthesis(const float2* __restrict__ Y, int nb,
                                                         float2* __restrict__ U, const float2* tw) {
  __shared__ __align__(16) float2 sm[SL * 16];
  const int l = threadIdx.x & 15, t = threadIdx.x >> 4;
  const int b = blockIdx.x / (ROWC / 16), q = (blockIdx.x % (ROWC / 16)) * 16 + l;
  const int kx = q >> 5, c = q & 31;
  float2 x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) x[e] = make_float2(0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int e = i < 2 ? i : i + (E - 4);
    const int m = iy_of(t + TPL * e) * KX + kx;
    x[e] = Y[((int64_t)m * nb + b) * C + c];
  }
  fft_line<float, N, E, 1, true>(x, t, sm + l, 16, tw);
  float2* dst = U + (int64_t)b * N * ROWC + q;
#pragma unroll
  for (int e = 0; e < E; ++e) dst[(int64_t)(t + TPL * e) * ROWC] = x[e];
}

// ---- tensor-core helpers shared by the kernels below -----------------------
struct TcState {
  uint64_t bar;
  uint32_t taddr;
};

__device__ __forceinline__ void tc_begin(TcState* st, uint32_t ncols) {
  if ((threadIdx.x >> 5) == 0) tmem_alloc(&st->taddr, ncols);
  if (threadIdx.x == 0) {
    mbar_init(&st->bar, 1);
    mbar_init_fence();
  }
}

// Operands staged by every thread with generic stores: make them visible to
// the tensor core and the TMEM address to every thread.
__device__ __forceinline__ uint32_t tc_operands_ready(TcState* st) {
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  return st->taddr;
}

// Wait for the MMAs committed to st->bar (phase 0).  On a timeout the status
// word records it and the (bounded) wait is repeated so that no MMA is in
// flight when tensor memory is released.
__device__ __forceinline__ bool tc_wait(TcState* st, int* status) {
  const bool ok = __syncthreads_and(mbar_wait_bounded(&st->bar, 0));
  if (!ok && threadIdx.x == 0) {
    atomicExch(status, DEV_WAIT_TIMEOUT);
    mbar_wait_bounded(&st->bar, 0);
  }
  tc_fence_after_sync();
  return ok;
}

__device__ __forceinline__ void tc_end(TcState* st, uint32_t tbase, uint32_t ncols) {
  tc_fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tmem_dealloc(tbase, ncols);
}

// 16-byte chunk of an R x K canonical tile holding row r, K-chunk k8
__device__ __forceinline__ int chunk_of(int r, int k8, int K) {
  return (r >> 3) * K + k8 * 8 + (r & 7);
}

// ---- per-mode channel mixing on tensor cores ---------------------------------
// Y[m][b][:] = X[m][b][:] . Wbig[m] in the real 64 x 64 form (Re | Im) for
// every item (mode m, 128-row tile mt), item = m * nmt + mt.  Persistent: a
// CTA walks items blockIdx.x, + gridDim.x, ...; both operands are stored in
// the tensor-core layout, so each arrives by two bulk copies, two items ahead
// of its product (stages alternate).  Rows at or beyond nb are multiplied
// from whatever the tile holds there and not stored (a product row depends
// only on its own A row).
constexpr size_t kMixStage = (size_t)(XTILE + WBIG) * 2;  // bytes of one item's operands
constexpr size_t kMixSmem = 2 * kMixStage + 4 * sizeof(uint64_t) + sizeof(uint32_t);
static_assert(kMixStage % 128 == 0 && (XTILE * 2) % 128 == 0, "mixing operand alignment");

__global__ void __launch_bounds__(128) k_mix(const __nv_bfloat16* __restrict__ Xc,
                                              const __nv_bfloat16* __restrict__ Wbig, int nb, int nmt,
                                              float2* __restrict__ Y, int* status) {
  extern __shared__ __align__(128) unsigned char smraw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smraw + 2 * kMixStage);  // operands landed, per stage
  uint64_t* done = full + 2;                                             // product complete, per stage
  uint32_t* taddr = reinterpret_cast<uint32_t*>(done + 2);
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned items = (unsigned)NM * (unsigned)nmt;
  if (blockIdx.x >= items) return;
  if (warp == 0) tmem_alloc(taddr, 64);
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&done[i], 1);
    }
    mbar_init_fence();
  }
  auto issue = [&](int st, unsigned item) {
    const unsigned m = item / (unsigned)nmt, mt = item % (unsigned)nmt;
    unsigned char* dst = smraw + st * kMixStage;
    mbar_arrive_expect_tx(&full[st], (unsigned)kMixStage);
    bulk_load(dst, Xc + ((int64_t)m * nmt + mt) * XTILE, XTILE * 2, &full[st]);
    bulk_load(dst + XTILE * 2, Wbig + (int64_t)m * WBIG, WBIG * 2, &full[st]);
  };
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t tbase = *taddr;
  if (tid == 0) {
    issue(0, blockIdx.x);
    if (blockIdx.x + gridDim.x < items) issue(1, blockIdx.x + gridDim.x);
  }
  const uint32_t idesc = umma_idesc_bf16(TILE_M, XK);
  int it = 0;
  for (unsigned item = blockIdx.x; item < items; item += gridDim.x, ++it) {
    const int st = it & 1;
    const unsigned par = (unsigned)((it >> 1) & 1);
    const unsigned ahead = item + gridDim.x;  // in flight into the other stage
    // this item's operands have landed; every thread's read-out of the
    // previous product is complete (fenced before the barrier)
    if (!__syncthreads_and(mbar_wait_bounded(&full[st], par))) {
      if (tid == 0) {
        atomicExch(status, DEV_WAIT_TIMEOUT);
        mbar_wait_bounded(&full[st], par);
        if (ahead < items) mbar_wait_bounded(&full[st ^ 1], (unsigned)(((it + 1) >> 1) & 1));
      }
      break;
    }
    tc_fence_after_sync();
    if (tid == 0) {
      const uint32_t a0 = smem_addr(smraw + st * kMixStage);
      const uint32_t b0 = a0 + XTILE * 2;
#pragma unroll
      for (int kk = 0; kk < XK / 16; ++kk)
        umma_bf16(tbase, umma_desc(a0 + kk * 256, kUmmaLbo, umma_sbo(XK)),
                  umma_desc(b0 + kk * 256, kUmmaLbo, umma_sbo(XK)), idesc, kk);
      umma_commit(&done[st]);
    }
    if (!__syncthreads_and(mbar_wait_bounded(&done[st], par))) {
      if (tid == 0) {
        atomicExch(status, DEV_WAIT_TIMEOUT);
        mbar_wait_bounded(&done[st], par);
        if (ahead < items) mbar_wait_bounded(&full[st ^ 1], (unsigned)(((it + 1) >> 1) & 1));
      }
      break;
    }
    tc_fence_after_sync();
    // the product has read this stage: the item two ahead goes into it
    if (tid == 0 && ahead + gridDim.x < items) issue(st, ahead + gridDim.x);
    const unsigned m = item / (unsigned)nmt, mt = item % (unsigned)nmt;
    float re[32], im[32];
    tmem_ld32(tmem_lane_addr(tbase, warp, 0), re);
    tmem_ld32(tmem_lane_addr(tbase, warp, 32), im);
    const int b = (int)mt * TILE_M + warp * 32 + (tid & 31);
    if (b < nb) {
      float4* dst = reinterpret_cast<float4*>(Y + ((int64_t)m * nb + b) * C);
#pragma unroll
      for (int o = 0; o < C; o += 2) dst[o / 2] = make_float4(re[o], im[o], re[o + 1], im[o + 1]);
    }
    tc_fence_before_sync();  // the next product overwrites the accumulator
  }
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, 64);
}

// ---- row analysis and synthesis as tensor-core contractions -----------------
// Synthesis, accumulated onto the 1 x 1 convolution: s[x][c] = sum_K Bs[x][K]
// Us[c][K] with the BF16 basis Bs[x][kx] = cos(2 pi kx x / N), Bs[x][KX + kx] =
// -sin(2 pi kx x / N) (256 pixel rows, two 128-row canonical tiles) and
// Us[c][kx] = bf16(Re U(kx) / N^2), Us[c][KX + kx] = bf16(Im U(kx) / N^2)
// (1/N^2 is a power of two: the scaling is exact).
// Analysis over quarter rows x = 64 q + x': D[(q, c)][K] = sum_x' h[64 q + x'][c]
// Ba[K][x'] with Ba[kx][x'] = cos(2 pi kx x' / N), Ba[KX + kx][x'] =
// -sin(2 pi kx x' / N) (M = 4 quarters x 32 channels = 128, N = 64, K = 64; the
// activations staged MN-major), then H_c(kx) = sum_q (-i)^(kx q) D_q: exact
// quarter-turn rotations of the partial sums.  FP32 accumulation throughout.
constexpr int KS = 2 * KX;           // contraction width: [Re | Im] of the kept kx
constexpr int QW = N / 4;            // quarter-row width
constexpr int kBasisSyn = N * KS;    // elements of Bs
constexpr int kBasisAna = KS * QW;   // elements of Ba
constexpr float kUScale = 1.0f / (N * N);
constexpr size_t kStageBytes = (size_t)N * C * 2;            // one row of BF16 activations
constexpr size_t kQuartBytes = (size_t)4 * 2 * KX * C * 4;   // D_q read back from TMEM
constexpr uint32_t kStageKStride = 16 * 128;                 // 8 x' of all 16 (q, c/8) groups

struct TcState2 {
  uint64_t bar[2];  // [0]: convolution + synthesis, [1]: analysis
  uint32_t taddr;
};

__device__ __forceinline__ void tc2_begin(TcState2* st, uint32_t ncols) {
  if ((threadIdx.x >> 5) == 0) tmem_alloc(&st->taddr, ncols);
  if (threadIdx.x == 0) {
    mbar_init(&st->bar[0], 1);
    mbar_init(&st->bar[1], 1);
    mbar_init_fence();
  }
}

// Shared-memory operands written by generic stores -> tensor core; TMEM
// address to every thread.
__device__ __forceinline__ uint32_t tc2_ready(TcState2* st) {
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  return st->taddr;
}

__device__ __forceinline__ void tc2_end(TcState2* st, uint32_t ncols) {
  tc_fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tmem_dealloc(st->taddr, ncols);
}

// Bounded wait for phase `par` of st->bar[i] by every thread; on a timeout the
// status word records it and thread 0 waits (bounded) once more so that no MMA
// is in flight when tensor memory is released.
__device__ __forceinline__ bool tc2_wait(TcState2* st, int i, unsigned par, int* status) {
  const bool ok = __syncthreads_and(mbar_wait_bounded(&st->bar[i], par));
  if (!ok && threadIdx.x == 0) {
    atomicExch(status, DEV_WAIT_TIMEOUT);
    mbar_wait_bounded(&st->bar[i], par);
  }
  tc_fence_after_sync();
  return ok;
}

// Pixel p's 32 BF16 activations into the MN-major analysis operand: core
// matrix (x'/8, q*4 + c/8) of 8 x' rows x 8 channels at
// (x'/8) * kStageKStride + (q*4 + c/8) * 128 bytes.
__device__ __forceinline__ void stage_analysis(unsigned char* stage, int p, const Bf16x32& hb) {
  const int q = p / QW, xq = p % QW;
#pragma unroll
  for (int c8 = 0; c8 < 4; ++c8)
    *reinterpret_cast<uint4*>(stage + (xq >> 3) * kStageKStride + (q * 4 + c8) * 128 + (xq & 7) * 16) =
        hb.q[c8];
}

// One thread: the four K = 16 analysis MMAs into TMEM columns [col, col + 64)
// (completion through the caller's next commit).
__device__ __forceinline__ void issue_analysis_async(uint32_t dcol, const unsigned char* stage,
                                                     const __nv_bfloat16* sBa) {
  const uint32_t idesc = umma_idesc_bf16(TILE_M, KS) | (1u << 15);  // A MN-major
  const uint32_t s0 = smem_addr(stage), b0 = smem_addr(sBa);
#pragma unroll
  for (int kk = 0; kk < QW / 16; ++kk)
    umma_bf16(dcol, umma_desc(s0 + kk * 2 * kStageKStride, kStageKStride, 128),
              umma_desc(b0 + kk * 256, kUmmaLbo, umma_sbo(QW)), idesc, kk);
}

// D_q from TMEM (warp w: quarter w % 4, columns (w / 4) * 32: Re or Im part)
// into quart [q][part][c][kx] (rows of 32 floats, float4 j of row c at
// position j ^ (c % 8): conflict-free 16-byte accesses); after a barrier
// thread (c, j) combines H_c(kx) = sum_q (-i)^(kx q) D_q for kx = 4j .. 4j+3,
// whose rotations (-i)^((kx q) % 4) = (-i)^((m q) % 4), m = kx % 4, are fixed
// per unrolled (m, q); out[kx][c] stores coalesced over c.
__device__ __forceinline__ void analysis_out(uint32_t dcol, float* quart, float2* out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  {
    float v[32];
    tmem_ld32(tmem_lane_addr(dcol, warp, (warp >> 2) * 32), v);
    float4* row = reinterpret_cast<float4*>(quart + (((warp & 3) * 2 + (warp >> 2)) * C + lane) * KX);
#pragma unroll
    for (int j = 0; j < KX / 4; ++j)
      row[j ^ (lane & 7)] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
  }
  __syncthreads();
  const int c = lane, j = warp;  // kx = 4j .. 4j+3
  float hr[4] = {0.f, 0.f, 0.f, 0.f}, hi[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 ar = reinterpret_cast<const float4*>(quart + ((q * 2) * C + c) * KX)[j ^ (c & 7)];
    const float4 ai = reinterpret_cast<const float4*>(quart + ((q * 2 + 1) * C + c) * KX)[j ^ (c & 7)];
    const float re[4] = {ar.x, ar.y, ar.z, ar.w}, im[4] = {ai.x, ai.y, ai.z, ai.w};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      // (a + i b) (-i)^r: r odd swaps the parts; r = 2, 3 negate the real
      // part, r = 1, 2 the imaginary part
      const int r = (m * q) & 3;
      const float x = (r & 1) ? im[m] : re[m], y = (r & 1) ? re[m] : im[m];
      hr[m] += (r & 2) ? -x : x;
      hi[m] += ((r + 1) & 2) ? -y : y;
    }
  }
#pragma unroll
  for (int m = 0; m < 4; ++m) out[(4 * j + m) * C + c] = make_float2(hr[m], hi[m]);
}

// ---- layer epilogue rows: synthesis + 1x1 conv + bias + GELU [+ next analysis | projection]
struct LayerArgs {
  const float2* U;
  const __nv_bfloat16* h;
  const __nv_bfloat16* wpack;  // 32 x 32 canonical, B[o][c] = Wc[c][o]
  const __nv_bfloat16* basis;  // shared-memory image of Bs then Ba
  const float* bias;
  int act;
  __nv_bfloat16* z;  // pre-activation (optional)
  __nv_bfloat16* hn;
  float2* Tn;       // next layer's row analysis (optional)
  const float* wp;  // projection [C][2] and bias [2] (optional, with out)
  const float* bp;
  float2* out;
  int* status;
  int64_t nrows;  // fields x N
};

// Shared memory of k_layer_rows (byte offsets; every operand 128-byte aligned)
constexpr size_t kLrStage = 0;                                    // analysis operand
constexpr size_t kLrQuart = kLrStage + kStageBytes;              // D_q read-back
constexpr size_t kLrBasis = kLrQuart + kQuartBytes;              // Bs then Ba
constexpr size_t kLrW = kLrBasis + (size_t)(kBasisSyn + kBasisAna) * 2;
constexpr size_t kLrA = kLrW + (size_t)WCONV * 2;                // row tile [N][C] (two 128-row tiles)
constexpr size_t kLrU = kLrA + kStageBytes;                      // spectral operand [C][KS]
constexpr size_t kLrState = kLrU + (size_t)C * KS * 2;
constexpr size_t kLayerSmem = kLrState + sizeof(TcState2);
static_assert(kLrQuart % 128 == 0 && kLrBasis % 128 == 0 && kLrW % 128 == 0 && kLrA % 128 == 0 &&
                  kLrU % 128 == 0 && kLrState % 8 == 0,
              "layer row pass: shared-memory operand alignment");
static_assert(2 * (kLayerSmem + 1024) <= 228 * 1024, "layer row pass: two CTAs per SM");

__device__ __forceinline__ void issue_row_conv(uint32_t tbase, const __nv_bfloat16* sA,
                                               const __nv_bfloat16* sW, TcState* st) {
  const uint32_t idesc = umma_idesc_bf16(TILE_M, C);
  const uint32_t a0 = smem_addr(sA), w0 = smem_addr(sW);
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int kk = 0; kk < C / 16; ++kk)
      umma_bf16(tbase + mt * C, umma_desc(a0 + mt * TILE_M * C * 2 + kk * 256, kUmmaLbo, umma_sbo(C)),
                umma_desc(w0 + kk * 256, kUmmaLbo, umma_sbo(C)), idesc, kk);
  umma_commit(&st->bar);
}

// One thread's share of a row's operands, loaded a row ahead: h (4 x 16 B of
// the 16 KB row) and U (2 x 16 B of the 8 KB half spectrum).
struct RowRegs {
  uint4 h[4];
  float2 u[4];
};

// 16-byte piece of the row's h (16 KB, 1024 pieces) handled by this thread in
// round j: the warp's 32 pieces are its 512 contiguous bytes (8 pixels x 4
// channel octets), lane l taking pixel l % 8 and octet l / 8, so that each
// quarter-warp of a shared-memory store fills one 128-byte row of core matrices.
__device__ __forceinline__ int h_piece(int j) {
  const int l = threadIdx.x & 31;
  return ((threadIdx.x & ~31) + 256 * j) + (l & 7) * 4 + (l >> 3);
}

__device__ __forceinline__ void load_row_regs(RowRegs& r, const LayerArgs& a, int64_t row) {
  const uint4* g4 = reinterpret_cast<const uint4*>(a.h + row * N * C);
#pragma unroll
  for (int j = 0; j < 4; ++j) r.h[j] = g4[h_piece(j)];
  // U[kx][c] for c = tid % 32 and kx = 4 (tid / 32) .. + 3 (coalesced over c)
  const float2* u = a.U + row * ROWC;
  const int c = threadIdx.x & 31, kb = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < 4; ++m) r.u[m] = u[(4 * kb + m) * C + c];
}

// h into the two canonical 128 x 32 tiles; U as bf16(U / N^2) into the
// [C][KS] canonical operand (row c, K = kx for Re, KX + kx for Im), four
// consecutive K per 8-byte store.
__device__ __forceinline__ void store_row_regs(const RowRegs& r, __nv_bfloat16* sA,
                                               __nv_bfloat16* sU) {
  uint4* s4 = reinterpret_cast<uint4*>(sA);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = h_piece(j), px = i >> 2, k8 = i & 3;
    s4[(px >> 7) * (TILE_M * C / 8) + chunk_of(px & 127, k8, C)] = r.h[j];
  }
  const int c = threadIdx.x & 31, kb = threadIdx.x >> 5;
  const __nv_bfloat162 r01 = __floats2bfloat162_rn(r.u[0].x * kUScale, r.u[1].x * kUScale);
  const __nv_bfloat162 r23 = __floats2bfloat162_rn(r.u[2].x * kUScale, r.u[3].x * kUScale);
  const __nv_bfloat162 i01 = __floats2bfloat162_rn(r.u[0].y * kUScale, r.u[1].y * kUScale);
  const __nv_bfloat162 i23 = __floats2bfloat162_rn(r.u[2].y * kUScale, r.u[3].y * kUScale);
  *reinterpret_cast<uint2*>(sU + umma_off(c, 4 * kb, KS)) =
      make_uint2(*reinterpret_cast<const uint32_t*>(&r01), *reinterpret_cast<const uint32_t*>(&r23));
  *reinterpret_cast<uint2*>(sU + umma_off(c, KX + 4 * kb, KS)) =
      make_uint2(*reinterpret_cast<const uint32_t*>(&i01), *reinterpret_cast<const uint32_t*>(&i23));
}

// Persistent: each CTA walks rows blockIdx.x, +gridDim.x, ...  Per row one
// round trip to the tensor core: the row's convolution + synthesis MMAs go
// out together with the previous row's analysis MMAs, and while they run the
// next row's operands are loaded into registers (stored once the MMAs have
// completed).  TMEM: columns [0, 64) convolution + synthesis (two 128-pixel
// tiles), [64, 128) analysis of the previous row.
__global__ void __launch_bounds__(256, 2) k_layer_rows(const LayerArgs a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  unsigned char* stage = smraw + kLrStage;
  float* quart = reinterpret_cast<float*>(smraw + kLrQuart);
  __nv_bfloat16* sB = reinterpret_cast<__nv_bfloat16*>(smraw + kLrBasis);
  __nv_bfloat16* sBa = sB + kBasisSyn;
  __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smraw + kLrW);
  __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smraw + kLrA);
  __nv_bfloat16* sU = reinterpret_cast<__nv_bfloat16*>(smraw + kLrU);
  TcState2* st = reinterpret_cast<TcState2*>(smraw + kLrState);
  __shared__ __align__(16) float sPar[C + 2 * C + 2];  // bias, then the projection wp [C][2] and bp [2]
  const int tid = threadIdx.x, warp = tid >> 5;
  if ((int64_t)blockIdx.x >= a.nrows) return;
  if (tid < C) sPar[tid] = a.bias[tid];
  if (a.out && tid < 2 * C + 2) sPar[C + tid] = tid < 2 * C ? a.wp[tid] : a.bp[tid - 2 * C];
  tc2_begin(st, 128);
  {
    const uint4* g4 = reinterpret_cast<const uint4*>(a.basis);
    uint4* s4 = reinterpret_cast<uint4*>(sB);
    for (int i = tid; i < (kBasisSyn + kBasisAna) / 8; i += 256) s4[i] = g4[i];
    if (tid < WCONV / 8)
      reinterpret_cast<uint4*>(sW)[tid] = reinterpret_cast<const uint4*>(a.wpack)[tid];
    RowRegs r0;
    load_row_regs(r0, a, blockIdx.x);
    store_row_regs(r0, sA, sU);
  }
  const int p = (warp >> 2) * TILE_M + (warp & 3) * 32 + (tid & 31);
  const uint32_t idesc = umma_idesc_bf16(TILE_M, C);
  bool ok = true;
  int it = 0;
  int64_t prev = -1;  // row whose analysis operand is staged
  for (int64_t row = blockIdx.x; row < a.nrows; row += gridDim.x, ++it) {
    // this row's operands and the previous row's staged activations (generic
    // stores by every thread) to the tensor core
    const uint32_t tbase = tc2_ready(st);
    if (tid == 0) {
      if (prev >= 0) issue_analysis_async(tbase + 2 * C, stage, sBa);
      const uint32_t a0 = smem_addr(sA), w0 = smem_addr(sW), b0 = smem_addr(sB), u0 = smem_addr(sU);
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
        for (int kk = 0; kk < C / 16; ++kk)
          umma_bf16(tbase + mt * C,
                    umma_desc(a0 + mt * TILE_M * C * 2 + kk * 256, kUmmaLbo, umma_sbo(C)),
                    umma_desc(w0 + kk * 256, kUmmaLbo, umma_sbo(C)), idesc, kk);
#pragma unroll
        for (int kk = 0; kk < KS / 16; ++kk)
          umma_bf16(tbase + mt * C,
                    umma_desc(b0 + mt * TILE_M * KS * 2 + kk * 256, kUmmaLbo, umma_sbo(KS)),
                    umma_desc(u0 + kk * 256, kUmmaLbo, umma_sbo(KS)), idesc, 1);
      }
      umma_commit(&st->bar[0]);
    }
    const int64_t next = row + gridDim.x;
    RowRegs nr;
    if (next < a.nrows) load_row_regs(nr, a, next);
    if (!(ok = tc2_wait(st, 0, (unsigned)(it & 1), a.status))) break;
    if (prev >= 0) analysis_out(tbase + 2 * C, quart, a.Tn + prev * ROWC);
    float v[32];
    tmem_ld32(tmem_lane_addr(tbase, warp, (warp >> 2) * C), v);
#pragma unroll
    for (int o = 0; o < C; o += 4) {  // z
      const float4 bq = *reinterpret_cast<const float4*>(sPar + o);
      v[o] += bq.x;
      v[o + 1] += bq.y;
      v[o + 2] += bq.z;
      v[o + 3] += bq.w;
    }
    const int64_t pix = row * N + p;
    if (a.z) store_packed(a.z + pix * C, pack_bf16x32(v));
    if (a.act) {
#pragma unroll
      for (int o = 0; o < C; ++o) v[o] = gelu(v[o]);
    }
    const Bf16x32 hb = pack_bf16x32(v);  // h' = bf16(GELU(z)) or bf16(z)
    if (a.hn) store_packed(a.hn + pix * C, hb);
    if (a.out) {
      float o0 = sPar[C + 2 * C], o1 = sPar[C + 2 * C + 1];
      const uint32_t* w = reinterpret_cast<const uint32_t*>(hb.q);
#pragma unroll
      for (int i = 0; i < C / 2; ++i) {
        const float h0 = bf16_lo(w[i]), h1 = bf16_hi(w[i]);
        const float4 wq = *reinterpret_cast<const float4*>(sPar + C + 4 * i);
        o0 = fmaf(h0, wq.x, o0);
        o1 = fmaf(h0, wq.y, o1);
        o0 = fmaf(h1, wq.z, o0);
        o1 = fmaf(h1, wq.w, o1);
      }
      a.out[pix] = make_float2(o0, o1);
    }
    // the MMAs have completed: the operand buffers and the stage are free
    if (next < a.nrows) store_row_regs(nr, sA, sU);
    if (a.Tn) {
      stage_analysis(stage, p, hb);
      prev = row;
    }
  }
  if (ok && prev >= 0) {  // the last row's analysis
    const uint32_t tbase = tc2_ready(st);
    if (tid == 0) {
      issue_analysis_async(tbase + 2 * C, stage, sBa);
      umma_commit(&st->bar[1]);
    }
    if (tc2_wait(st, 1, 0, a.status)) analysis_out(tbase + 2 * C, quart, a.Tn + prev * ROWC);
  }
  tc2_end(st, 128);
}

// ---- lift + first row analysis ---------------------------------------------
// xin [b][y][x][3] (Re E0, Im E0, V), xs [b][2] scalars; wl [5][C], bl [C].
// Persistent over rows; the analysis as in k_layer_rows (TMEM columns [0, 64)).
struct LiftArgs {
  const float* xin;
  const float* xs;
  const float* wl;
  const float* bl;
  __nv_bfloat16* h0;
  float2* T;
  const __nv_bfloat16* basis;  // Bs then Ba (Ba used)
  int* status;
  int64_t nrows;
};
constexpr size_t kLfStage = 0;                               // two stages
constexpr size_t kLfQuart = kLfStage + 2 * kStageBytes;
constexpr size_t kLfBa = kLfQuart + kQuartBytes;
constexpr size_t kLfState = kLfBa + (size_t)kBasisAna * 2;
constexpr size_t kLiftSmem = kLfState + sizeof(TcState2);

__global__ void __launch_bounds__(256, 3) k_lift_rows(const LiftArgs a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  float* quart = reinterpret_cast<float*>(smraw + kLfQuart);
  __nv_bfloat16* sBa = reinterpret_cast<__nv_bfloat16*>(smraw + kLfBa);
  TcState2* st = reinterpret_cast<TcState2*>(smraw + kLfState);
  __shared__ __align__(16) float sWl[6 * C];  // wl [5][C], then bl [C]
  const int p = threadIdx.x;
  if ((int64_t)blockIdx.x >= a.nrows) return;
  if (p < 5 * C) sWl[p] = a.wl[p];
  if (p < C) sWl[5 * C + p] = a.bl[p];
  tc2_begin(st, 128);
  {
    const uint4* g4 = reinterpret_cast<const uint4*>(a.basis + kBasisSyn);
    for (int i = p; i < kBasisAna / 8; i += 256) reinterpret_cast<uint4*>(sBa)[i] = g4[i];
  }
  __syncthreads();  // sWl
  // thread: channel octet c8 of pixel x' of each quarter (x = 64 q + x'), the
  // lift weights of its 8 channels for the three pixel inputs in registers
  const int xq = p & (QW - 1), c8 = p / QW;
  float w0[8], w1[8], w2[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    w0[j] = sWl[8 * c8 + j];
    w1[j] = sWl[C + 8 * c8 + j];
    w2[j] = sWl[2 * C + 8 * c8 + j];
  }
  // row i: stage and TMEM columns (i & 1); its MMAs run while row i - 1 is read out
  float xr[4][3];
  auto load_x = [&](int64_t row) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float* xi = a.xin + (row * N + q * QW + xq) * 3;
      xr[q][0] = xi[0];
      xr[q][1] = xi[1];
      xr[q][2] = xi[2];
    }
  };
  load_x(blockIdx.x);
  bool ok = true;
  int it = 0;
  int64_t prev = -1;
  for (int64_t row = blockIdx.x; row < a.nrows; row += gridDim.x, ++it) {
    const int64_t b = row / N;
    const float s0 = a.xs[2 * b], s1 = a.xs[2 * b + 1];
    float cst[8];  // bl + s0 wl[3] + s1 wl[4]: the field's part
#pragma unroll
    for (int j = 0; j < 8; j += 4) {
      const float4 bq = *reinterpret_cast<const float4*>(sWl + 5 * C + 8 * c8 + j);
      const float4 w3 = *reinterpret_cast<const float4*>(sWl + 3 * C + 8 * c8 + j);
      const float4 w4 = *reinterpret_cast<const float4*>(sWl + 4 * C + 8 * c8 + j);
      cst[j] = fmaf(s1, w4.x, fmaf(s0, w3.x, bq.x));
      cst[j + 1] = fmaf(s1, w4.y, fmaf(s0, w3.y, bq.y));
      cst[j + 2] = fmaf(s1, w4.z, fmaf(s0, w3.z, bq.z));
      cst[j + 3] = fmaf(s1, w4.w, fmaf(s0, w3.w, bq.w));
    }
    unsigned char* stage = smraw + kLfStage + (it & 1) * kStageBytes;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t wd[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        const float v0 = fmaf(xr[q][2], w2[j], fmaf(xr[q][1], w1[j], fmaf(xr[q][0], w0[j], cst[j])));
        const float v1 = fmaf(xr[q][2], w2[j + 1],
                              fmaf(xr[q][1], w1[j + 1], fmaf(xr[q][0], w0[j + 1], cst[j + 1])));
        const __nv_bfloat162 hb2 = __floats2bfloat162_rn(v0, v1);  // h0 = bf16(lift)
        wd[j / 2] = *reinterpret_cast<const uint32_t*>(&hb2);
      }
      const uint4 hq = make_uint4(wd[0], wd[1], wd[2], wd[3]);
      *reinterpret_cast<uint4*>(a.h0 + (row * N + q * QW + xq) * C + 8 * c8) = hq;
      *reinterpret_cast<uint4*>(stage + (xq >> 3) * kStageKStride + (q * 4 + c8) * 128 +
                                (xq & 7) * 16) = hq;
    }
    const int64_t next = row + gridDim.x;
    if (next < a.nrows) load_x(next);
    const uint32_t tbase = tc2_ready(st);
    if (p == 0) {
      issue_analysis_async(tbase + (it & 1) * KS, stage, sBa);
      umma_commit(&st->bar[it & 1]);
    }
    if (prev >= 0) {
      const int pb = (it - 1) & 1;
      if (!(ok = tc2_wait(st, pb, (unsigned)(((it - 1) >> 1) & 1), a.status))) {
        if (p == 0) mbar_wait_bounded(&st->bar[it & 1], (unsigned)((it >> 1) & 1));  // row it's MMAs
        break;
      }
      analysis_out(tbase + pb * KS, quart, a.T + prev * ROWC);
    }
    prev = row;
  }
  if (ok && prev >= 0) {
    const int pb = (it - 1) & 1;
    if (tc2_wait(st, pb, (unsigned)(((it - 1) >> 1) & 1), a.status))
      analysis_out(st->taddr + pb * KS, quart, a.T + prev * ROWC);
  }
  tc2_end(st, 128);
}

// ---- backward ---------------------------------------------------------------
// Projection: dh4 = dout . Wp^T; partials per row: gWp [C][2] then gbp [2].
__global__ void __launch_bounds__(256) k_proj_bwd(const float2* __restrict__ dout,
                                                   const float* __restrict__ wp,
                                                   const __nv_bfloat16* __restrict__ h4,
                                                   float* __restrict__ dh4, float* __restrict__ part) {
  __shared__ float red[8][NLSE_FNO_PART_PROJ];
  const int64_t row = blockIdx.x;
  const int p = threadIdx.x, lane = p & 31, warp = p >> 5;
  const int64_t pix = row * N + p;
  const float2 d = dout[pix];
  float h[32], g[32];
  load_bf16x32(h4 + pix * C, h);
#pragma unroll
  for (int o = 0; o < C; ++o) g[o] = d.x * wp[2 * o] + d.y * wp[2 * o + 1];
  float4* dst = reinterpret_cast<float4*>(dh4 + pix * C);
#pragma unroll
  for (int o = 0; o < C; o += 4) dst[o / 4] = make_float4(g[o], g[o + 1], g[o + 2], g[o + 3]);
  for (int i = 0; i < NLSE_FNO_PART_PROJ; ++i) {
    float v = i < 2 * C ? h[i >> 1] * ((i & 1) ? d.y : d.x) : ((i & 1) ? d.y : d.x);
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (lane == 0) red[warp][i] = v;
  }
  __syncthreads();
  if (p < NLSE_FNO_PART_PROJ) {
    float v = 0.f;
#pragma unroll
    for (int w = 0; w < 8; ++w) v += red[w][p];
    part[row * NLSE_FNO_PART_PROJ + p] = v;
  }
}

struct BwdArgs {
  const float* dhc_in;  // gradient from above, convolution part (FP32 [b][y][x][c])
  const float2* Uin;    // its spectral part as column-synthesised half spectra (optional)
  const __nv_bfloat16* z;
  int act;
  const __nv_bfloat16* h;      // layer input
  const __nv_bfloat16* wpack;  // 32 x 32 canonical, B[c][o] = Wc[c][o]
  float* dhc_out;              // dz . Wc^T
  float2* Tg;                  // row analysis of dz
  float* part;                 // per row: gWc [C][C] then gb [C]
  const float2* tw;
  int* status;
};

constexpr size_t kBwdSmem = kPairBuf + (size_t)N * C * 2 + (size_t)WCONV * 2 + sizeof(TcState) +
                           (size_t)N * (C + 1) * sizeof(float);

// dh = dhc_in + synthesis(Uin); dz = dh * GELU'(z) (or dh); dhc_out = dz Wc^T
// on the tensor core; partial weight and bias gradients; Tg = analysis of dz.
__global__ void __launch_bounds__(256) k_layer_rows_bwd(const BwdArgs a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  float2* xl = reinterpret_cast<float2*>(smraw);
  float2* ss = xl;
  __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smraw + kPairBuf);
  __nv_bfloat16* sW = sA + N * C;
  TcState* st = reinterpret_cast<TcState*>(sW + WCONV);
  float* hsm = reinterpret_cast<float*>(st + 1);  // [N][C+1]
  const int64_t row = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, p = tid;
  const int64_t pix = row * N + p;
  tc_begin(st, 64);
  if (a.Uin) {
    row_synthesis(a.Uin + row * ROWC, 1.0f, xl, a.tw, ss);
    __syncthreads();
  }
  float dz[32], zb[32], hv[32];
  {
    const float4* src = reinterpret_cast<const float4*>(a.dhc_in + pix * C);
#pragma unroll
    for (int o = 0; o < C; o += 4) {
      const float4 u = src[o / 4];
      dz[o] = u.x;
      dz[o + 1] = u.y;
      dz[o + 2] = u.z;
      dz[o + 3] = u.w;
    }
  }
  if (a.Uin) {
#pragma unroll
    for (int o = 0; o < C; ++o) {
      const float2 s2 = ss[p * PS + (o >> 1)];
      dz[o] += (o & 1) ? s2.y : s2.x;
    }
  }
  if (a.act) {
    load_bf16x32(a.z + pix * C, zb);
#pragma unroll
    for (int o = 0; o < C; ++o) dz[o] *= gelu_grad(zb[o]);
  }
  load_bf16x32(a.h + pix * C, hv);
  __syncthreads();  // ss no longer read
  // dz as the A operand (pixel rows), as FP32 pairs, and h for the weight gradient
  {
    __align__(16) __nv_bfloat16 bz[32];
#pragma unroll
    for (int o = 0; o < C; ++o) bz[o] = __float2bfloat16_rn(dz[o]);
    uint4* s4 = reinterpret_cast<uint4*>(sA);
    const uint4* b4 = reinterpret_cast<const uint4*>(bz);
#pragma unroll
    for (int k8 = 0; k8 < 4; ++k8) s4[(p >> 7) * (TILE_M * C / 8) + chunk_of(p & 127, k8, C)] = b4[k8];
  }
#pragma unroll
  for (int jj = 0; jj < C / 2; ++jj) ss[p * PS + jj] = make_float2(dz[2 * jj], dz[2 * jj + 1]);
#pragma unroll
  for (int c = 0; c < C; ++c) hsm[p * (C + 1) + c] = hv[c];
  if (tid < WCONV / 8)
    reinterpret_cast<uint4*>(sW)[tid] = reinterpret_cast<const uint4*>(a.wpack)[tid];
  const uint32_t tbase = tc_operands_ready(st);
  if (tid == 0) issue_row_conv(tbase, sA, sW, st);
  // gWc[c][o] = sum_p h[p][c] dz[p][o]: thread -> c = tid % 32, o = 4 * (tid / 32) .. +3
  {
    const int c = tid & 31, o0 = (tid >> 5) * 4;
    float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;
    for (int q = 0; q < N; ++q) {
      const float hq = hsm[q * (C + 1) + c];
      const float2 d01 = ss[q * PS + (o0 >> 1)], d23 = ss[q * PS + (o0 >> 1) + 1];
      g0 = fmaf(hq, d01.x, g0);
      g1 = fmaf(hq, d01.y, g1);
      g2 = fmaf(hq, d23.x, g2);
      g3 = fmaf(hq, d23.y, g3);
    }
    float* pr = a.part + row * NLSE_FNO_PART_LAYER;
    pr[c * C + o0] = g0;
    pr[c * C + o0 + 1] = g1;
    pr[c * C + o0 + 2] = g2;
    pr[c * C + o0 + 3] = g3;
    if (tid < C) {
      float gb = 0.f;
      for (int q = 0; q < N; ++q) {
        const float2 d = ss[q * PS + (tid >> 1)];
        gb += (tid & 1) ? d.y : d.x;
      }
      pr[WCONV + tid] = gb;
    }
  }
  row_analysis(ss, xl, a.tw, a.Tg + row * ROWC);
  if (!tc_wait(st, a.status)) {
    tc_end(st, tbase, 64);
    return;
  }
  float v[32];
  tmem_ld32(tmem_lane_addr(tbase, warp, (warp >> 2) * C), v);
  const int pp = (warp >> 2) * TILE_M + (warp & 3) * 32 + (tid & 31);
  float4* dst = reinterpret_cast<float4*>(a.dhc_out + (row * N + pp) * C);
#pragma unroll
  for (int o = 0; o < C; o += 4) dst[o / 4] = make_float4(v[o], v[o + 1], v[o + 2], v[o + 3]);
  tc_end(st, tbase, 64);
}

// Lift: dh0 = dhc_in + synthesis(Uin); per-row partials
// [0, 96): sum_p xin[p][i] dh0[p][o] (i < 3), [96, 128): xs0 * sum dh0,
// [128, 160): xs1 * sum dh0, [160, 192): sum dh0.
__global__ void __launch_bounds__(256) k_lift_bwd(const float* __restrict__ dhc_in,
                                                   const float2* __restrict__ Uin,
                                                   const float* __restrict__ xin,
                                                   const float* __restrict__ xs,
                                                   float* __restrict__ part, const float2* tw) {
  extern __shared__ __align__(128) unsigned char smraw[];
  float2* xl = reinterpret_cast<float2*>(smraw);
  float2* ss = xl;
  float* xsm = reinterpret_cast<float*>(smraw + kPairBuf);  // [N][3]
  const int64_t row = blockIdx.x, b = row / N;
  const int p = threadIdx.x;
  const int64_t pix = row * N + p;
  if (Uin) row_synthesis(Uin + row * ROWC, 1.0f, xl, tw, ss);
  __syncthreads();
  float d[32];
  const float4* src = reinterpret_cast<const float4*>(dhc_in + pix * C);
#pragma unroll
  for (int o = 0; o < C; o += 4) {
    const float4 u = src[o / 4];
    d[o] = u.x;
    d[o + 1] = u.y;
    d[o + 2] = u.z;
    d[o + 3] = u.w;
  }
  if (Uin) {
#pragma unroll
    for (int o = 0; o < C; ++o) {
      const float2 s2 = ss[p * PS + (o >> 1)];
      d[o] += (o & 1) ? s2.y : s2.x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int jj = 0; jj < C / 2; ++jj) ss[p * PS + jj] = make_float2(d[2 * jj], d[2 * jj + 1]);
#pragma unroll
  for (int i = 0; i < 3; ++i) xsm[p * 3 + i] = xin[pix * 3 + i];
  __syncthreads();
  if (p < 4 * C) {
    const int i = p >> 5, o = p & 31;
    float g = 0.f;
    for (int q = 0; q < N; ++q) {
      const float2 d2 = ss[q * PS + (o >> 1)];
      const float dv = (o & 1) ? d2.y : d2.x;
      g = fmaf(i < 3 ? xsm[q * 3 + i] : 1.f, dv, g);
    }
    float* pr = part + row * NLSE_FNO_PART_LIFT;
    if (i < 3) {
      pr[i * C + o] = g;
    } else {
      pr[3 * C + o] = xs[2 * b] * g;
      pr[4 * C + o] = xs[2 * b + 1] * g;
      pr[5 * C + o] = g;
    }
  }
}

// gW[m][c][o] = sum_b conj(H[m][b][c]) G[m][b][o] (complex, FP32).
__global__ void __launch_bounds__(256) k_mix_wgrad(const float2* __restrict__ Hs,
                                                    const float2* __restrict__ Gs, int nb,
                                                    float2* __restrict__ gW) {
  constexpr int BB = 32;
  __shared__ float2 sh[BB][C + 1], sg[BB][C + 1];
  const int m = blockIdx.x, tid = threadIdx.x;
  const int c = tid >> 3, o0 = (tid & 7) * 4;
  float2 acc[4] = {};
  for (int b0 = 0; b0 < nb; b0 += BB) {
    __syncthreads();
    for (int i = tid; i < BB * C; i += 256) {
      const int bb = i >> 5, cc = i & 31;
      const bool in = b0 + bb < nb;
      const int64_t off = ((int64_t)m * nb + b0 + bb) * C + cc;
      sh[bb][cc] = in ? Hs[off] : make_float2(0.f, 0.f);
      sg[bb][cc] = in ? Gs[off] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int bb = 0; bb < BB; ++bb) {
      const float2 h = sh[bb][c];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float2 g = sg[bb][o0 + u];
        acc[u].x = fmaf(h.x, g.x, fmaf(h.y, g.y, acc[u].x));
        acc[u].y = fmaf(h.x, g.y, fmaf(-h.y, g.x, acc[u].y));
      }
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) gW[((int64_t)m * C + c) * C + o0 + u] = acc[u];
}

// out[w] = sum over rows of part[row][w]
__global__ void __launch_bounds__(256) k_reduce(const float* __restrict__ part, int64_t rows,
                                                 int width, float* __restrict__ out) {
  __shared__ float red[8][32];
  const int w = blockIdx.x * 32 + (threadIdx.x & 31), g = threadIdx.x >> 5;
  float v = 0.f;
  if (w < width)
    for (int64_t r = g; r < rows; r += 8) v += part[r * width + w];
  red[g][threadIdx.x & 31] = v;
  __syncthreads();
  if (g == 0 && w < width) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += red[i][threadIdx.x];
    out[w] = s;
  }
}

// ---- weights ------------------------------------------------------------------
// Real 64 x 64 forms of one mode's complex weights W[c][o], as canonical BF16
// B operands (rows n, K contiguous):
//   forward  (Y = X W):         n = o: [Re W[:,o] | -Im W[:,o]],  n = 32+o: [Im W[:,o] | Re W[:,o]]
//   backward (G = Y conj(W)^T): n = c: [Re W[c,:] |  Im W[c,:]],  n = 32+c: [-Im W[c,:] | Re W[c,:]]
__global__ void __launch_bounds__(256) k_pack_spectral(const float2* __restrict__ W,
                                                        __nv_bfloat16* __restrict__ wf,
                                                        __nv_bfloat16* __restrict__ wb) {
  const int m = blockIdx.x;
  const float2* Wm = W + (int64_t)m * WCONV;
  for (int i = threadIdx.x; i < WBIG; i += 256) {
    const int n = i >> 6, k = i & 63;
    const int no = n & 31, ki = k & 31;
    const bool nim = n >= C, kim = k >= C;
    const float2 f = Wm[ki * C + no];  // W[c = ki][o = no]
    const float vf = !nim ? (!kim ? f.x : -f.y) : (!kim ? f.y : f.x);
    const float2 g = Wm[no * C + ki];  // W[c = no][o = ki]
    const float vb = !nim ? (!kim ? g.x : g.y) : (!kim ? -g.y : g.x);
    wf[(int64_t)m * WBIG + umma_off(n, k, XK)] = __float2bfloat16_rn(vf);
    wb[(int64_t)m * WBIG + umma_off(n, k, XK)] = __float2bfloat16_rn(vb);
  }
}

// 1 x 1 convolution weights Wc[c][o]: forward B[o][c], backward B[c][o].
__global__ void k_pack_conv(const float* __restrict__ wc, __nv_bfloat16* __restrict__ wf,
                            __nv_bfloat16* __restrict__ wb) {
  for (int i = threadIdx.x; i < WCONV; i += blockDim.x) {
    const int n = i >> 5, k = i & 31;
    wf[umma_off(n, k, C)] = __float2bfloat16_rn(wc[k * C + n]);
    wb[umma_off(n, k, C)] = __float2bfloat16_rn(wc[n * C + k]);
  }
}

// ---- loss and optimiser ----------------------------------------------------------
// Per field b: stats[2b] = ||out - tgt||^2, stats[2b+1] = ||ref||^2 (FP32 sums).
__global__ void __launch_bounds__(256) k_loss_stats(const float2* __restrict__ out,
                                                     const float2* __restrict__ tgt,
                                                     const float2* __restrict__ ref,
                                                     float* __restrict__ stats) {
  __shared__ float red[2][8];
  const int64_t b = blockIdx.x;
  const float2* o = out + b * N * N;
  const float2* g = tgt + b * N * N;
  const float2* q = ref + b * N * N;
  float e = 0.f, n = 0.f;
  for (int i = threadIdx.x; i < N * N; i += 256) {
    const float2 u = o[i], v = g[i], w = q[i];
    const float dx = u.x - v.x, dy = u.y - v.y;
    e = fmaf(dx, dx, fmaf(dy, dy, e));
    n = fmaf(w.x, w.x, fmaf(w.y, w.y, n));
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, s);
    n += __shfl_xor_sync(0xffffffffu, n, s);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = e;
    red[1][threadIdx.x >> 5] = n;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    float s = 0.f;
    for (int w = 0; w < 8; ++w) s += red[threadIdx.x][w];
    stats[2 * b + threadIdx.x] = s;
  }
}

// Loss = (1/nb) sum_b ||out_b - tgt_b||^2 / ||ref_b||^2; dout = its gradient.
__global__ void k_loss_grad(const float2* __restrict__ out, const float2* __restrict__ tgt,
                            const float* __restrict__ stats, int64_t nb, float2* __restrict__ dout) {
  const int64_t total = nb * N * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / (N * N);
    const float s = 2.f / ((float)nb * fmaxf(stats[2 * b + 1], 1e-30f));
    const float2 u = out[i], v = tgt[i];
    dout[i] = make_float2(s * (u.x - v.x), s * (u.y - v.y));
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2, float wd) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * ((mi / bc1) / (sqrtf(vi / bc2) + eps) + wd * p[i]);
  }
}

// ---- self-test of the tensor-core path --------------------------------------
// C (128 x n, FP32) = A (128 x k, BF16 row-major) . B (n x k, BF16 row-major)^T
__global__ void __launch_bounds__(128) k_gemm_selftest(const __nv_bfloat16* __restrict__ A,
                                                        const __nv_bfloat16* __restrict__ B,
                                                        float* __restrict__ Cm, int n, int k,
                                                        int* status) {
  __shared__ __align__(128) __nv_bfloat16 sA[TILE_M * 64];
  __shared__ __align__(128) __nv_bfloat16 sB[64 * 64];
  __shared__ TcState st;
  const int tid = threadIdx.x, warp = tid >> 5;
  tc_begin(&st, 64);
  for (int i = tid; i < TILE_M * k; i += 128) sA[umma_off(i / k, i % k, k)] = A[i];
  for (int i = tid; i < n * k; i += 128) sB[umma_off(i / k, i % k, k)] = B[i];
  const uint32_t tbase = tc_operands_ready(&st);
  if (tid == 0) {
    const uint32_t idesc = umma_idesc_bf16(TILE_M, n);
    const uint32_t a0 = smem_addr(sA), b0 = smem_addr(sB);
    for (int kk = 0; kk < k / 16; ++kk)
      umma_bf16(tbase, umma_desc(a0 + kk * 256, kUmmaLbo, umma_sbo(k)),
                umma_desc(b0 + kk * 256, kUmmaLbo, umma_sbo(k)), idesc, kk);
    umma_commit(&st.bar);
  }
  if (tc_wait(&st, status)) {
    const int r = warp * 32 + (tid & 31);
    for (int c0 = 0; c0 < n; c0 += 32) {
      float v[32];
      tmem_ld32(tmem_lane_addr(tbase, warp, c0), v);
      for (int j = 0; j < 32 && c0 + j < n; ++j) Cm[r * n + c0 + j] = v[j];
    }
  }
  tc_end(&st, tbase, 64);
}

// ---- host side -------------------------------------------------------------------
constexpr size_t kLiftBwdSmem = kPairBuf + (size_t)N * 3 * sizeof(float);

std::mutex g_attr_mu;
bool g_attr_done[64] = {};
const __nv_bfloat16* g_basis[64] = {};
int g_layer_ctas[64] = {};  // resident k_layer_rows CTAs of the device
int g_lift_ctas[64] = {};   // resident k_lift_rows CTAs of the device
int g_mix_ctas[64] = {};    // resident k_mix CTAs of the device

uint16_t host_bf16_bits(double v) {
  // double -> float (nearest) -> bfloat16 (nearest, ties to even)
  const float f = (float)v;
  uint32_t u;
  memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

// The contraction bases Bs then Ba in the kernels' shared-memory image
// (caller holds g_attr_mu).
int make_basis(int dev) {
  const long double pi = 3.141592653589793238462643383279502884L;
  auto val = [&](int k, int x) {
    const int kx = k < KX ? k : k - KX;
    const long double ang = 2.0L * pi * (long double)((kx * x) & (N - 1)) / (long double)N;
    return k < KX ? (double)cosl(ang) : -(double)sinl(ang);
  };
  std::vector<uint16_t> hb((size_t)(kBasisSyn + kBasisAna));
  for (int px = 0; px < N; ++px)
    for (int k = 0; k < KS; ++k)
      hb[(size_t)(px >> 7) * TILE_M * KS + umma_off(px & 127, k, KS)] = host_bf16_bits(val(k, px));
  for (int k = 0; k < KS; ++k)
    for (int x = 0; x < QW; ++x) hb[(size_t)kBasisSyn + umma_off(k, x, QW)] = host_bf16_bits(val(k, x));
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, hb.size() * 2);
  if (e == cudaSuccess) e = cudaMemcpy(d, hb.data(), hb.size() * 2, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (d) cudaFree(d);
    return shared_cuda_fail(e, "contraction bases");
  }
  g_basis[dev] = reinterpret_cast<const __nv_bfloat16*>(d);
  return NLSE_OK;
}

int prepare(const float2** tw) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return shared_cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return shared_fail(NLSE_ERR_UNSUPPORTED, "device ordinal");
  const void* t = nullptr;
  const int rc = shared_twiddles(dev, NLSE_C64, &t);
  if (rc != NLSE_OK) return rc;
  *tw = reinterpret_cast<const float2*>(t);
  std::lock_guard<std::mutex> lk(g_attr_mu);
  if (!g_attr_done[dev]) {
    e = cudaFuncSetAttribute(k_lift_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLiftSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_layer_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kLayerSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_layer_rows_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kBwdSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_lift_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kLiftBwdSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMixSmem);
    if (e != cudaSuccess) return shared_cuda_fail(e, "cudaFuncSetAttribute (FNO kernels)");
    // persistent grids: every CTA the multiprocessors can hold (shared memory,
    // registers and threads counted here from the kernels' attributes)
    int nsm = 0, smem_sm = 0, smem_res = 0, regs_sm = 0, thr_sm = 0;
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e == cudaSuccess)
      e = cudaDeviceGetAttribute(&smem_res, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (e == cudaSuccess)
      e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    if (e == cudaSuccess)
      e = cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    if (e != cudaSuccess) return shared_cuda_fail(e, "device attributes");
    auto resident = [&](const void* fn, size_t smem, int threads, int* out) {
      cudaFuncAttributes fa;
      const cudaError_t fe = cudaFuncGetAttributes(&fa, fn);
      if (fe != cudaSuccess) return fe;
      // registers are granted per warp in units of 256
      const int regs_cta = ((fa.numRegs * 32 + 255) / 256) * 256 * (threads / 32);
      int n = (int)(smem_sm / (smem + fa.sharedSizeBytes + smem_res));
      if (regs_cta > 0 && regs_sm / regs_cta < n) n = regs_sm / regs_cta;
      if (thr_sm / threads < n) n = thr_sm / threads;
      *out = nsm * (n > 0 ? n : 1);
      return cudaSuccess;
    };
    e = resident(reinterpret_cast<const void*>(k_layer_rows), kLayerSmem, 256, &g_layer_ctas[dev]);
    if (e == cudaSuccess)
      e = resident(reinterpret_cast<const void*>(k_lift_rows), kLiftSmem, 256, &g_lift_ctas[dev]);
    if (e == cudaSuccess)
      e = resident(reinterpret_cast<const void*>(k_mix), kMixSmem, 128, &g_mix_ctas[dev]);
    if (e != cudaSuccess) return shared_cuda_fail(e, "persistent grid sizes");
    const int brc = make_basis(dev);
    if (brc != NLSE_OK) return brc;
    g_attr_done[dev] = true;
  }
  return NLSE_OK;
}

int launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NLSE_OK : shared_cuda_fail(e, what);
}

bool bad_batch(int64_t nb) { return nb <= 0 || nb > (int64_t(1) << 20); }

int nmt_of(int64_t nb) { return (int)((nb + TILE_M - 1) / TILE_M); }

}  // namespace fno
}  // namespace nlse

using namespace nlse::fno;

extern "C" {

int nlse_fno_lift_rows(int64_t nb, const float* xin, const float* xs, const float* wl,
                       const float* bl, void* h0, void* T, int32_t* status, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !xin || !xs || !wl || !bl || !h0 || !T || !status)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_lift_rows: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* tw;
  int rc = prepare(&tw);
  if (rc != NLSE_OK) return rc;
  int dev = 0;
  cudaGetDevice(&dev);
  LiftArgs a;
  a.xin = xin;
  a.xs = xs;
  a.wl = wl;
  a.bl = bl;
  a.h0 = reinterpret_cast<__nv_bfloat16*>(h0);
  a.T = reinterpret_cast<float2*>(T);
  a.basis = g_basis[dev];
  a.status = status;
  a.nrows = nb * N;
  const int64_t grid = a.nrows < g_lift_ctas[dev] ? a.nrows : g_lift_ctas[dev];
  k_lift_rows<<<(unsigned)grid, 256, kLiftSmem, s>>>(a);
  return launched("nlse_fno_lift_rows");
}

int nlse_fno_cols_analysis(int64_t nb, const void* T, float scale, int32_t round_saved, void* Xc,
                           void* Hs, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !T || !Xc)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_cols_analysis: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* tw;
  int rc = prepare(&tw);
  if (rc != NLSE_OK) return rc;
  k_cols_analysis<<<(unsigned)(nb * (ROWC / 16)), 256, 0, s>>>(
      reinterpret_cast<const float2*>(T), (int)nb, nmt_of(nb), scale, round_saved,
      reinterpret_cast<__nv_bfloat16*>(Xc), reinterpret_cast<float2*>(Hs), tw);
  return launched("nlse_fno_cols_analysis");
}

int nlse_fno_mix(int64_t nb, const void* Xc, const void* wbig, void* Y, int32_t* status,
                 void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !Xc || !wbig || !Y || !status)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_mix: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* tw;
  int rc = prepare(&tw);
  if (rc != NLSE_OK) return rc;
  const int nmt = nmt_of(nb);
  int dev = 0;
  cudaGetDevice(&dev);
  const int64_t items = (int64_t)NM * nmt;
  const int64_t grid = items < g_mix_ctas[dev] ? items : g_mix_ctas[dev];
  k_mix<<<(unsigned)grid, 128, kMixSmem, s>>>(reinterpret_cast<const __nv_bfloat16*>(Xc),
                                              reinterpret_cast<const __nv_bfloat16*>(wbig), (int)nb,
                                              nmt, reinterpret_cast<float2*>(Y), status);
  return launched("nlse_fno_mix");
}

int nlse_fno_cols_synthesis(int64_t nb, const void* Y, void* U, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !Y || !U)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_cols_synthesis: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* tw;
  int rc = prepare(&tw);
  if (rc != NLSE_OK) return rc;
  k_cols_synthesis<<<(unsigned)(nb * (ROWC / 16)), 256, 0, s>>>(
      reinterpret_cast<const float2*>(Y), (int)nb, reinterpret_cast<float2*>(U), tw);
  return launched("nlse_fno_cols_synthesis");
}

int nlse_fno_layer_rows(int64_t nb, const void* U, const void* h, const void* wconv,
                        const float* bias, int32_t act, void* z, void* hn, void* Tn,
                        const float* wp, const float* bp, void* out, int32_t* status,
                        void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !U || !h || !wconv || !bias || !status || (out && (!wp || !bp)) ||
      (!hn && !out))
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_layer_rows: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* tw;
  int rc = prepare(&tw);
  if (rc != NLSE_OK) return rc;
  LayerArgs a;
  a.U = reinterpret_cast<const float2*>(U);
  a.h = reinterpret_cast<const __nv_bfloat16*>(h);
  a.wpack = reinterpret_cast<const __nv_bfloat16*>(wconv);
  a.bias = bias;
  a.act = act;
  a.z = reinterpret_cast<__nv_bfloat16*>(z);
  a.hn = reinterpret_cast<__nv_bfloat16*>(hn);
  a.Tn = reinterpret_cast<float2*>(Tn);
  a.wp = wp;
  a.bp = bp;
  a.out = reinterpret_cast<float2*>(out);
  a.status = status;
  int dev = 0;
  cudaGetDevice(&dev);
  a.basis = g_basis[dev];
  a.nrows = nb * N;
  const int64_t grid = a.nrows < g_layer_ctas[dev] ? a.nrows : g_layer_ctas[dev];
  k_layer_rows<<<(unsigned)grid, 256, kLayerSmem, s>>>(a);
  return launched("nlse_fno_layer_rows");
}

int nlse_fno_proj_bwd(int64_t nb, const void* dout, const float* wp, const void* h4, float* dh4,
                      float* part, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !dout || !wp || !h4 || !dh4 || !part)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_proj_bwd: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_proj_bwd<<<(unsigned)(nb * N), 256, 0, s>>>(reinterpret_cast<const float2*>(dout), wp,
                                                 reinterpret_cast<const __nv_bfloat16*>(h4), dh4,
                                                 part);
  return launched("nlse_fno_proj_bwd");
}

int nlse_fno_layer_rows_bwd(int64_t nb, const float* dhc_in, const void* Uin, const void* z,
                            int32_t act, const void* h, const void* wconv_bwd, float* dhc_out,
                            void* Tg, float* part, int32_t* status, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !dhc_in || (act && !z) || !h || !wconv_bwd || !dhc_out || !Tg || !part ||
      !status)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_layer_rows_bwd: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* tw;
  int rc = prepare(&tw);
  if (rc != NLSE_OK) return rc;
  BwdArgs a;
  a.dhc_in = dhc_in;
  a.Uin = reinterpret_cast<const float2*>(Uin);
  a.z = reinterpret_cast<const __nv_bfloat16*>(z);
  a.act = act;
  a.h = reinterpret_cast<const __nv_bfloat16*>(h);
  a.wpack = reinterpret_cast<const __nv_bfloat16*>(wconv_bwd);
  a.dhc_out = dhc_out;
  a.Tg = reinterpret_cast<float2*>(Tg);
  a.part = part;
  a.tw = tw;
  a.status = status;
  k_layer_rows_bwd<<<(unsigned)(nb * N), 256, kBwdSmem, s>>>(a);
  return launched("nlse_fno_layer_rows_bwd");
}

int nlse_fno_lift_bwd(int64_t nb, const float* dhc_in, const void* Uin, const float* xin,
                      const float* xs, float* part, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !dhc_in || !xin || !xs || !part)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_lift_bwd: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* tw;
  int rc = prepare(&tw);
  if (rc != NLSE_OK) return rc;
  k_lift_bwd<<<(unsigned)(nb * N), 256, kLiftBwdSmem, s>>>(
      dhc_in, reinterpret_cast<const float2*>(Uin), xin, xs, part, tw);
  return launched("nlse_fno_lift_bwd");
}

int nlse_fno_mix_wgrad(int64_t nb, const void* Hs, const void* Gs, void* gW, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !Hs || !Gs || !gW)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_mix_wgrad: bad argument");
  k_mix_wgrad<<<NM, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(Hs), reinterpret_cast<const float2*>(Gs), (int)nb,
      reinterpret_cast<float2*>(gW));
  return launched("nlse_fno_mix_wgrad");
}

int nlse_fno_reduce(const float* part, int64_t rows, int64_t width, float* out, void* stream) {
  nlse::shared_clear_error();
  if (!part || !out || rows <= 0 || width <= 0 || width > (1 << 20))
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_reduce: bad argument");
  k_reduce<<<(unsigned)((width + 31) / 32), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      part, rows, (int)width, out);
  return launched("nlse_fno_reduce");
}

int nlse_fno_pack_spectral(const void* W, void* wf, void* wb, void* stream) {
  nlse::shared_clear_error();
  if (!W || !wf || !wb) return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_pack_spectral: null");
  k_pack_spectral<<<NM, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(W), reinterpret_cast<__nv_bfloat16*>(wf),
      reinterpret_cast<__nv_bfloat16*>(wb));
  return launched("nlse_fno_pack_spectral");
}

int nlse_fno_pack_conv(const float* wc, void* wf, void* wb, void* stream) {
  nlse::shared_clear_error();
  if (!wc || !wf || !wb) return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_pack_conv: null");
  k_pack_conv<<<1, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      wc, reinterpret_cast<__nv_bfloat16*>(wf), reinterpret_cast<__nv_bfloat16*>(wb));
  return launched("nlse_fno_pack_conv");
}

int nlse_fno_loss(int64_t nb, const void* out, const void* tgt, const void* ref, float* stats,
                  void* dout, void* stream) {
  nlse::shared_clear_error();
  if (bad_batch(nb) || !out || !tgt || !stats)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_loss: bad argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_loss_stats<<<(unsigned)nb, 256, 0, s>>>(reinterpret_cast<const float2*>(out),
                                             reinterpret_cast<const float2*>(tgt),
                                             reinterpret_cast<const float2*>(ref ? ref : tgt), stats);
  if (dout)
    k_loss_grad<<<1024, 256, 0, s>>>(reinterpret_cast<const float2*>(out),
                                      reinterpret_cast<const float2*>(tgt), stats, nb,
                                      reinterpret_cast<float2*>(dout));
  return launched("nlse_fno_loss");
}

int nlse_fno_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1,
                  float b2, float eps, int32_t step, float wd, void* stream) {
  nlse::shared_clear_error();
  if (!p || !g || !m || !v || n <= 0 || step <= 0)
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_adam: bad argument");
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  const int64_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_adam<<<(unsigned)blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      p, g, m, v, n, lr, b1, b2, eps, bc1, bc2, wd);
  return launched("nlse_fno_adam");
}

int nlse_fno_gemm_selftest(const void* A, const void* B, void* Cm, int32_t n, int32_t k,
                           int32_t* status, void* stream) {
  nlse::shared_clear_error();
  if (!A || !B || !Cm || !status || (n != 32 && n != 64) || (k != 32 && k != 64))
    return nlse::shared_fail(NLSE_ERR_ARG, "nlse_fno_gemm_selftest: n, k in {32, 64}");
  k_gemm_selftest<<<1, 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const __nv_bfloat16*>(A), reinterpret_cast<const __nv_bfloat16*>(B),
      reinterpret_cast<float*>(Cm), n, k, status);
  return launched("nlse_fno_gemm_selftest");
}

}  // extern "C"
