// Stockham FFT on pairs of complex64 lines with packed FP32 arithmetic.
//
// A "pair" is the same position of two independent lines (two rows of two
// fields, or two adjacent columns) held as
//   re = (a.re, b.re), im = (a.im, b.im)
// so every butterfly addition and every twiddle multiply is one f32x2
// instruction (add.f32x2 / sub.f32x2 / mul.f32x2 / fma.f32x2 of sm_100+) for
// both lines: half the instructions of the scalar transform, which issue
// limits.  Both lines always see the same twiddles.
//
// The transform follows fft_core.cuh exactly: radix-min(16, E) passes with
// the remaining radix last, thread t owning positions t + j*TPL before the
// first and after the last pass, padded shared-memory exchanges (padi).  One
// exchange element is a float4 {a.re, b.re, a.im, b.im}; STRIDE interleaves
// several pairs (column pairs of one tile).
//
// Twiddles: the float2 pass tables of fft_core.cuh ([r-1][k] per (R, NS)
// pass, entry exp(-2 pi i r k / (NS R))), global or the compact shared copy
// (TWS); a twiddle enters the packed instructions as a broadcast operand
// (wr, wr) / (wi, wi), which costs no instruction.
#pragma once
#include "fft_core.cuh"

namespace nlse {


__device__ __forceinline__ cp2 pcadd(cp2 a, cp2 b) { return {add2(a.re, b.re), add2(a.im, b.im)}; }
__device__ __forceinline__ cp2 pcsub(cp2 a, cp2 b) { return {sub2(a.re, b.re), sub2(a.im, b.im)}; }

// x * w for a twiddle w = (wr, wi) shared by both lines (forward), conj(w)
// (inverse).
template <bool INV>
__device__ __forceinline__ cp2 pmul_tw(cp2 x, float2 w) {
  const float2 wr = f2s(w.x), wi = f2s(w.y);
  if (INV) return {fma2(x.im, wi, mul2(x.re, wr)), fnma2(x.re, wi, mul2(x.im, wr))};
  return {fnma2(x.im, wi, mul2(x.re, wr)), fma2(x.re, wi, mul2(x.im, wr))};
}

// x * exp(-i theta) forward, x * exp(+i theta) inverse, (c, s) = (cos, sin)
// of theta known at compile time (the same as mul_w(x, c, s) of fft_core.cuh).
template <bool INV>
__device__ __forceinline__ cp2 pmul_c(cp2 x, float c, float s) {
  const float2 c2 = f2s(c), s2 = f2s(INV ? -s : s), ns2 = f2s(INV ? s : -s);
  // forward: (re c + im s, im c - re s); inverse: (re c - im s, im c + re s)
  return {fma2(x.im, s2, mul2(x.re, c2)), fma2(x.re, ns2, mul2(x.im, c2))};
}

// 4-point DFT in place; the -i (forward) / +i (inverse) rotation of the odd
// difference is folded into the output additions.
template <bool INV>
__device__ __forceinline__ void pdft4(cp2& a0, cp2& a1, cp2& a2, cp2& a3) {
  const cp2 t0 = pcadd(a0, a2), t1 = pcsub(a0, a2);
  const cp2 t2 = pcadd(a1, a3), d = pcsub(a1, a3);
  a0 = pcadd(t0, t2);
  a2 = pcsub(t0, t2);
  if (INV) {
    a1 = {sub2(t1.re, d.im), add2(t1.im, d.re)};
    a3 = {add2(t1.re, d.im), sub2(t1.im, d.re)};
  } else {
    a1 = {add2(t1.re, d.im), sub2(t1.im, d.re)};
    a3 = {sub2(t1.re, d.im), add2(t1.im, d.re)};
  }
}

template <int R, bool INV> struct PDFT;

template <bool INV> struct PDFT<1, INV> {
  __device__ __forceinline__ static void run(cp2*) {}
};

template <bool INV> struct PDFT<2, INV> {
  __device__ __forceinline__ static void run(cp2* x) {
    const cp2 a = x[0], b = x[1];
    x[0] = pcadd(a, b);
    x[1] = pcsub(a, b);
  }
};

template <bool INV> struct PDFT<4, INV> {
  __device__ __forceinline__ static void run(cp2* x) { pdft4<INV>(x[0], x[1], x[2], x[3]); }
};

template <bool INV> struct PDFT<8, INV> {
  __device__ __forceinline__ static void run(cp2* x) {
    cp2 e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
    cp2 o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
    pdft4<INV>(e0, e1, e2, e3);
    pdft4<INV>(o0, o1, o2, o3);
    const float2 r = f2s(float(NLSE_R2)), nr = f2s(-float(NLSE_R2));
    // o1 *= W8^1, o3 *= W8^3 (conjugated for the inverse)
    if (INV) {
      o1 = {mul2(r, sub2(o1.re, o1.im)), mul2(r, add2(o1.re, o1.im))};
      o3 = {mul2(nr, add2(o3.re, o3.im)), mul2(r, sub2(o3.re, o3.im))};
    } else {
      o1 = {mul2(r, add2(o1.re, o1.im)), mul2(r, sub2(o1.im, o1.re))};
      o3 = {mul2(r, sub2(o3.im, o3.re)), mul2(nr, add2(o3.re, o3.im))};
    }
    x[0] = pcadd(e0, o0);
    x[4] = pcsub(e0, o0);
    x[1] = pcadd(e1, o1);
    x[5] = pcsub(e1, o1);
    // o2 *= W8^2 = -i (forward) / +i (inverse), folded into the additions
    if (INV) {
      x[2] = {sub2(e2.re, o2.im), add2(e2.im, o2.re)};
      x[6] = {add2(e2.re, o2.im), sub2(e2.im, o2.re)};
    } else {
      x[2] = {add2(e2.re, o2.im), sub2(e2.im, o2.re)};
      x[6] = {sub2(e2.re, o2.im), add2(e2.im, o2.re)};
    }
    x[3] = pcadd(e3, o3);
    x[7] = pcsub(e3, o3);
  }
};

// 16-point DFT as 4 x 4 (the factorisation of DFT<T, 16> in fft_core.cuh).
template <bool INV> struct PDFT<16, INV> {
  __device__ __forceinline__ static void run(cp2* x) {
    const float c8 = float(NLSE_C8), s8 = float(NLSE_S8), r2 = float(NLSE_R2);
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) pdft4<INV>(x[n2], x[4 + n2], x[8 + n2], x[12 + n2]);
    x[1 + 4 * 1] = pmul_c<INV>(x[1 + 4 * 1], c8, s8);    // W^1
    x[1 + 4 * 2] = pmul_c<INV>(x[1 + 4 * 2], r2, r2);    // W^2
    x[1 + 4 * 3] = pmul_c<INV>(x[1 + 4 * 3], s8, c8);    // W^3
    x[2 + 4 * 1] = pmul_c<INV>(x[2 + 4 * 1], r2, r2);    // W^2
    {                                                    // W^4 = -i / +i
      const cp2 v = x[2 + 4 * 2];
      x[2 + 4 * 2] = INV ? cp2{make_float2(-v.im.x, -v.im.y), v.re}
                         : cp2{v.im, make_float2(-v.re.x, -v.re.y)};
    }
    x[2 + 4 * 3] = pmul_c<INV>(x[2 + 4 * 3], -r2, r2);   // W^6
    x[3 + 4 * 1] = pmul_c<INV>(x[3 + 4 * 1], s8, c8);    // W^3
    x[3 + 4 * 2] = pmul_c<INV>(x[3 + 4 * 2], -r2, r2);   // W^6
    x[3 + 4 * 3] = pmul_c<INV>(x[3 + 4 * 3], -c8, -s8);  // W^9
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) pdft4<INV>(x[4 * k1 + 0], x[4 * k1 + 1], x[4 * k1 + 2], x[4 * k1 + 3]);
    cp2 y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) y[k1 + 4 * k2] = x[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = y[i];
  }
};

// One radix-R pass over the thread's E pair elements (stockham_pass of
// fft_core.cuh); TWS: tw is the compact shared table of the transform.
template <int N, int E, int R, int NS, bool INV, bool TWS>
__device__ __forceinline__ void pstockham_pass(cp2 (&x)[E], int t, const float2* __restrict__ tw) {
  constexpr int TPL = N / E, BPT = E / R;
  static_assert(NS * R <= kTwMaxLen, "twiddle tables cover sub-transforms up to kTwMaxLen");
#pragma unroll
  for (int s = 0; s < BPT; ++s) {
    cp2 y[R];
#pragma unroll
    for (int r = 0; r < R; ++r) y[r] = x[s + r * BPT];
    if constexpr (NS > 1) {
      int k = (t + s * TPL) & (NS - 1);
      asm volatile("" : "+r"(k)::"memory");
      const float2* twp = tw + (TWS ? tw_compact_offset(N, E, NS) : tw_offset(R, NS)) + k;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        if (r > 1 && (r - 1) % TWG == 0) asm volatile("" ::: "memory");
        const float2 w = TWS ? twp[(r - 1) * NS] : __ldg(twp + (r - 1) * NS);
        y[r] = pmul_tw<INV>(y[r], w);
      }
    }
    PDFT<R, INV>::run(y);
#pragma unroll
    for (int r = 0; r < R; ++r) x[s + r * BPT] = y[r];
  }
}

__device__ __forceinline__ void st4(float4* p, cp2 v) { *p = make_float4(v.re.x, v.re.y, v.im.x, v.im.y); }
__device__ __forceinline__ cp2 ld4(const float4* p) {
  const float4 v = *p;
  return {make_float2(v.x, v.y), make_float2(v.z, v.w)};
}

// Exchange halves (exchange_store / exchange_load of fft_core.cuh) on float4
// elements; element i of this pair's line at sm[padi(i) * stride].
template <int N, int E, int NS>
__device__ __forceinline__ void pexchange_store(const cp2 (&x)[E], int t, float4* sm, int stride) {
  constexpr int TPL = N / E;
  constexpr int R = PassRadix<N, E, NS>::R;
  constexpr int BPT = E / R;
#pragma unroll
  for (int s = 0; s < BPT; ++s) {
    const int b = t + s * TPL;
    const int base = (b / NS) * NS * R + (b & (NS - 1));
    if constexpr (NS % 16 == 0) {
      const int pb = padi(base) * stride;
#pragma unroll
      for (int r = 0; r < R; ++r) st4(sm + pb + r * (NS + NS / 16) * stride, x[s + r * BPT]);
    } else if constexpr (NS == 1 && R == 16) {
      const int pb = (17 * b) * stride;
#pragma unroll
      for (int r = 0; r < R; ++r) st4(sm + pb + r * stride, x[s + r * BPT]);
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) st4(sm + padi(base + r * NS) * stride, x[s + r * BPT]);
    }
  }
}

template <int N, int E>
__device__ __forceinline__ void pexchange_load(cp2 (&x)[E], int t, const float4* sm, int stride) {
  constexpr int TPL = N / E;
  if constexpr (TPL % 16 == 0) {
    const int pb = padi(t) * stride;
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = ld4(sm + pb + j * (TPL + TPL / 16) * stride);
  } else {
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = ld4(sm + padi(t + j * TPL) * stride);
  }
}

// Full transform of one pair with two exchange buffers used alternately
// (fft_line_db of fft_core.cuh: same caller contract; FM bit 0 / bit 1 fence
// the stores into A / B against later bulk copies into them).
template <int N, int E, int NS, bool INV, int P, int FM, bool TWS = false>
__device__ __forceinline__ void pfft_db(cp2 (&x)[E], int t, float4* smA, float4* smB, int stride,
                                        const float2* __restrict__ tw) {
  constexpr int R = PassRadix<N, E, NS>::R;
  static_assert((E / R) * R == E, "radix must divide the elements per thread");
  if constexpr (NS == 1) asm volatile("" : "+r"(t)::"memory");
  pstockham_pass<N, E, R, NS, INV, TWS>(x, t, tw);
  if constexpr (NS * R < N) {
    float4* sm = P ? smB : smA;
    pexchange_store<N, E, NS>(x, t, sm, stride);
    if constexpr ((FM >> P) & 1) fence_async_after_stores();
    __syncthreads();
    pexchange_load<N, E>(x, t, sm, stride);
    pfft_db<N, E, NS * R, INV, P ^ 1, FM, TWS>(x, t, smA, smB, stride, tw);
  }
}

// Transform on one exchange buffer (fft_line_hook of fft_core.cuh): the first
// exchange needs no leading barrier unless LEAD; hook() runs right after that
// exchange's barrier, when every shared-memory read issued before the
// transform has completed.
template <int N, int E, int NS, bool INV, bool FENCE, bool TWS = false>
__device__ __forceinline__ void pfft_rest(cp2 (&x)[E], int t, float4* sm, int stride,
                                          const float2* __restrict__ tw) {
  constexpr int R = PassRadix<N, E, NS>::R;
  pstockham_pass<N, E, R, NS, INV, TWS>(x, t, tw);
  if constexpr (NS * R < N) {
    __syncthreads();
    pexchange_store<N, E, NS>(x, t, sm, stride);
    if constexpr (FENCE) fence_async_after_stores();
    __syncthreads();
    pexchange_load<N, E>(x, t, sm, stride);
    pfft_rest<N, E, NS * R, INV, FENCE, TWS>(x, t, sm, stride, tw);
  }
}

template <int N, int E, bool INV, bool FENCE, bool LEAD, typename Hook>
__device__ __forceinline__ void pfft_hook(cp2 (&x)[E], int t, float4* sm, int stride,
                                          const float2* __restrict__ tw, Hook&& hook) {
  constexpr int R = PassRadix<N, E, 1>::R;
  static_assert((E / R) * R == E, "radix must divide the elements per thread");
  asm volatile("" : "+r"(t)::"memory");
  pstockham_pass<N, E, R, 1, INV, false>(x, t, tw);
  if constexpr (R < N) {
    if constexpr (LEAD) __syncthreads();
    pexchange_store<N, E, 1>(x, t, sm, stride);
    if constexpr (FENCE) fence_async_after_stores();
    __syncthreads();
    hook();
    pexchange_load<N, E>(x, t, sm, stride);
    pfft_rest<N, E, R, INV, FENCE, false>(x, t, sm, stride, tw);
  } else {
    hook();
  }
}

}  // namespace nlse
