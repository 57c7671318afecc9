// In-CTA Stockham FFT building blocks for sm_103a.
//
// A "line" is one 1-D transform of power-of-two length N.  The line is held
// by TPL = N / E threads, each owning E elements in registers.  Thread t owns
// the elements at positions t + j*TPL (j = 0..E-1) both before the first pass
// and after the last pass, so global loads and stores of a line are coalesced
// across consecutive threads and no shared-memory exchange is needed at
// either end of the transform.  Between radix passes the elements are
// scattered to their Stockham positions in shared memory and gathered back
// in the t + j*TPL pattern (P passes need P-1 exchanges).
//
// Radix order: radix-min(16, E) passes first, the remaining radix last,
// so that the small-stride scatter happens when the span NS is large.
// Shared-memory index padding: one spare slot per 16 elements (padi), which
// makes both the strided scatter of the first pass and the gathers
// conflict-free for 8- and 16-byte elements.
//
// Twiddles: one table per (radix R, span NS) pass, laid out [r-1][k] with
// entry exp(-2*pi*i*r*k/(NS*R)), r = 1..R-1, k = 0..NS-1, so that the lanes
// of a warp (consecutive k) read consecutive entries.  All pass tables live
// in one array built on the host in long double and rounded once to the
// element type (tw_offset gives each pass's start).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nlse {

constexpr int kTwMaxLen = 4096;  // largest sub-transform NS*R covered by the tables

// Start of the (R, NS) pass table: per radix R the tables for NS = 1, 2, 4, ...
// follow each other ((R-1)*NS entries each), radices in the order 2, 4, 8, 16.
__host__ __device__ constexpr int tw_radix_base(int R) {
  return R == 2 ? 0
       : R == 4 ? (kTwMaxLen - 1)
       : R == 8 ? (kTwMaxLen - 1) + 3 * (kTwMaxLen / 2 - 1)
                : (kTwMaxLen - 1) + 3 * (kTwMaxLen / 2 - 1) + 7 * (kTwMaxLen / 4 - 1);
}
__host__ __device__ constexpr int tw_offset(int R, int NS) {
  return tw_radix_base(R) + (R - 1) * (NS - 1);
}
constexpr int kTwTableLen = tw_radix_base(16) + 15 * (kTwMaxLen / 8 - 1);

template <typename T> struct CT;
template <> struct CT<float> { using t = float2; };
template <> struct CT<double> { using t = double2; };
template <typename T> using cpx = typename CT<T>::t;

template <typename T>
__device__ __forceinline__ cpx<T> mk(T x, T y) {
  cpx<T> r;
  r.x = x;
  r.y = y;
  return r;
}
// Packed FP32 (f32x2, sm_100+): one instruction on both halves of a 64-bit
// register pair, each half rounded as the scalar instruction would round it.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// c - a * b
__device__ __forceinline__ float2 fnma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, make_float2(-b.x, -b.y), c);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(r)
      : "l"(*reinterpret_cast<const unsigned long long*>(&a)),
        "l"(*reinterpret_cast<const unsigned long long*>(&b)));
  return *reinterpret_cast<const float2*>(&r);
}

// Two complex64 values, lane-wise: re = (a.re, b.re), im = (a.im, b.im) (two
// lines at one position, or two positions of one line).
struct __align__(16) cp2 {
  float2 re, im;
};

// Complex sums and differences; a complex64 value {re, im} is one register
// pair, so these are single packed instructions (same results as two scalar
// ones).
template <typename T>
__device__ __forceinline__ cpx<T> cadd(cpx<T> a, cpx<T> b) {
  if constexpr (sizeof(T) == 4) return add2(a, b);
  else return mk<T>(a.x + b.x, a.y + b.y);
}
template <typename T>
__device__ __forceinline__ cpx<T> csub(cpx<T> a, cpx<T> b) {
  if constexpr (sizeof(T) == 4) return sub2(a, b);
  else return mk<T>(a.x - b.x, a.y - b.y);
}
// a + rot(b) and a - rot(b), rot = multiplication by -i (forward) or +i
// (inverse), the rotation folded into scalar additions (a packed form would
// first have to build the rotated pair).
template <typename T, bool INV>
__device__ __forceinline__ cpx<T> cadd_rot(cpx<T> a, cpx<T> b) {
  return INV ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x + b.y, a.y - b.x);
}
template <typename T, bool INV>
__device__ __forceinline__ cpx<T> csub_rot(cpx<T> a, cpx<T> b) {
  return INV ? mk<T>(a.x + b.y, a.y - b.x) : mk<T>(a.x - b.y, a.y + b.x);
}
template <typename T>
__device__ __forceinline__ cpx<T> cmul(cpx<T> a, cpx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T>
__device__ __forceinline__ cpx<T> cscale(cpx<T> a, T s) {
  return mk<T>(a.x * s, a.y * s);
}
// a * w where w = (wr, -wi) forward (exp(-i*theta)), (wr, +wi) inverse.
template <typename T, bool INV>
__device__ __forceinline__ cpx<T> mul_w(cpx<T> a, T wr, T wi) {
  const T s = INV ? wi : -wi;
  if constexpr (sizeof(T) == 4) {
    // (re, im) = a.x (wr, s) + a.y (-s, wr): two packed instructions
    return fma2(f2s(a.y), f2(-s, wr), mul2(f2s(a.x), f2(wr, s)));
  } else {
    return mk<T>(a.x * wr - a.y * s, a.x * s + a.y * wr);
  }
}

// cos(pi/8), sin(pi/8), sqrt(1/2)
#define NLSE_C8 0.92387953251128675613
#define NLSE_S8 0.38268343236508977173
#define NLSE_R2 0.70710678118654752440

template <typename T, int R, bool INV> struct DFT;

template <typename T, bool INV> struct DFT<T, 1, INV> {
  __device__ __forceinline__ static void run(cpx<T>*) {}
};

template <typename T, bool INV> struct DFT<T, 2, INV> {
  __device__ __forceinline__ static void run(cpx<T>* x) {
    const cpx<T> a = x[0], b = x[1];
    x[0] = cadd<T>(a, b);
    x[1] = csub<T>(a, b);
  }
};

template <typename T, bool INV>
__device__ __forceinline__ void dft4(cpx<T>& a0, cpx<T>& a1, cpx<T>& a2, cpx<T>& a3) {
  const cpx<T> t0 = cadd<T>(a0, a2), t1 = csub<T>(a0, a2);
  const cpx<T> t2 = cadd<T>(a1, a3), d = csub<T>(a1, a3);
  a0 = cadd<T>(t0, t2);
  a1 = cadd_rot<T, INV>(t1, d);
  a2 = csub<T>(t0, t2);
  a3 = csub_rot<T, INV>(t1, d);
}
// dft4 of (a0, a1, rot(a2), a3): the rotation of the third input folded in.
template <typename T, bool INV>
__device__ __forceinline__ void dft4_rot2(cpx<T>& a0, cpx<T>& a1, cpx<T>& a2, cpx<T>& a3) {
  const cpx<T> t0 = cadd_rot<T, INV>(a0, a2), t1 = csub_rot<T, INV>(a0, a2);
  const cpx<T> t2 = cadd<T>(a1, a3), d = csub<T>(a1, a3);
  a0 = cadd<T>(t0, t2);
  a1 = cadd_rot<T, INV>(t1, d);
  a2 = csub<T>(t0, t2);
  a3 = csub_rot<T, INV>(t1, d);
}

template <typename T, bool INV> struct DFT<T, 4, INV> {
  __device__ __forceinline__ static void run(cpx<T>* x) { dft4<T, INV>(x[0], x[1], x[2], x[3]); }
};

template <typename T, bool INV> struct DFT<T, 8, INV> {
  __device__ __forceinline__ static void run(cpx<T>* x) {
    cpx<T> e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
    cpx<T> o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
    dft4<T, INV>(e0, e1, e2, e3);
    dft4<T, INV>(o0, o1, o2, o3);
    const T r = T(NLSE_R2);
    o1 = mul_w<T, INV>(o1, r, r);
    o3 = mul_w<T, INV>(o3, -r, r);
    x[0] = cadd<T>(e0, o0);
    x[4] = csub<T>(e0, o0);
    x[1] = cadd<T>(e1, o1);
    x[5] = csub<T>(e1, o1);
    x[2] = cadd_rot<T, INV>(e2, o2);
    x[6] = csub_rot<T, INV>(e2, o2);
    x[3] = cadd<T>(e3, o3);
    x[7] = csub<T>(e3, o3);
  }
};

// 16-point DFT as 4 x 4: n = 4*n1 + n2, k = k1 + 4*k2.
template <typename T, bool INV> struct DFT<T, 16, INV> {
  __device__ __forceinline__ static void run(cpx<T>* x) {
    const T c8 = T(NLSE_C8), s8 = T(NLSE_S8), r2 = T(NLSE_R2);
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4<T, INV>(x[n2], x[4 + n2], x[8 + n2], x[12 + n2]);
    // x[n2 + 4*k1] now holds X[n2][k1]; apply W16^(n2*k1)
    x[1 + 4 * 1] = mul_w<T, INV>(x[1 + 4 * 1], c8, s8);    // W^1
    x[1 + 4 * 2] = mul_w<T, INV>(x[1 + 4 * 2], r2, r2);    // W^2
    x[1 + 4 * 3] = mul_w<T, INV>(x[1 + 4 * 3], s8, c8);    // W^3
    x[2 + 4 * 1] = mul_w<T, INV>(x[2 + 4 * 1], r2, r2);    // W^2
    // x[2 + 4 * 2] times W^4 (the rotation), folded into its dft4 below
    x[2 + 4 * 3] = mul_w<T, INV>(x[2 + 4 * 3], -r2, r2);   // W^6
    x[3 + 4 * 1] = mul_w<T, INV>(x[3 + 4 * 1], s8, c8);    // W^3
    x[3 + 4 * 2] = mul_w<T, INV>(x[3 + 4 * 2], -r2, r2);   // W^6
    x[3 + 4 * 3] = mul_w<T, INV>(x[3 + 4 * 3], -c8, -s8);  // W^9
    dft4<T, INV>(x[0], x[1], x[2], x[3]);
    dft4<T, INV>(x[4], x[5], x[6], x[7]);
    dft4_rot2<T, INV>(x[8], x[9], x[10], x[11]);
    dft4<T, INV>(x[12], x[13], x[14], x[15]);
    // x[4*k1 + k2] holds y[k1 + 4*k2]; transpose the 4x4 index in registers.
    cpx<T> y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) y[k1 + 4 * k2] = x[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = y[i];
  }
};

__host__ __device__ constexpr int padi(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int n) { return padi(n - 1) + 1; }

// Elements per thread and threads per line for an N-point line.
template <int N, int EREQ = 16> struct Shape {
  static constexpr int E = N >= EREQ ? EREQ : N;
  static constexpr int TPL = N / E;
};

// One radix-R Stockham pass over the thread's E elements.  On entry x[j]
// holds input position t + j*TPL; element j = s + r*BPT is input r of
// butterfly b = t + s*TPL.  On exit x[s + r*BPT] holds output position
// (b / NS) * NS * R + (b % NS) + r * NS.
constexpr int TWG = 4;  // twiddles loaded per group

// Compact twiddle table of one N-point transform (E points per thread): the
// tables of its twiddled passes (NS > 1) back to back, [r-1][k] each.
__host__ __device__ constexpr int tw_compact_offset(int n, int e, int upto_ns) {
  int off = 0;
  for (int ns = 1; ns < upto_ns && ns < n;) {
    const int rmax = e < 16 ? e : 16;
    const int r = (n / ns) >= rmax ? rmax : n / ns;
    if (r < 2) break;
    if (ns > 1) off += (r - 1) * ns;
    ns *= r;
  }
  return off;
}
__host__ __device__ constexpr int tw_compact_len(int n, int e) { return tw_compact_offset(n, e, n); }

// Copy the compact table of an N-point transform from the full table (all threads).
template <typename T, int N, int E>
__device__ __forceinline__ void load_tw_compact(cpx<T>* dst, const cpx<T>* __restrict__ tw) {
  int ns = 1;
#pragma unroll 1
  while (ns < N) {
    const int rmax = E < 16 ? E : 16;
    const int r = (N / ns) >= rmax ? rmax : N / ns;
    if (ns > 1) {
      const int off = tw_compact_offset(N, E, ns), len = (r - 1) * ns;
      for (int i = threadIdx.x; i < len; i += blockDim.x) dst[off + i] = tw[tw_offset(r, ns) + i];
    }
    ns *= r;
  }
}

// TWS: tw is a compact table in shared memory (load_tw_compact) instead of
// the full table in global memory.
template <typename T, int N, int E, int R, int NS, bool INV, bool TWS = false>
__device__ __forceinline__ void stockham_pass(cpx<T> (&x)[E], int t, const cpx<T>* __restrict__ tw) {
  constexpr int TPL = N / E, BPT = E / R;
  static_assert(NS * R <= kTwMaxLen, "twiddle tables cover sub-transforms up to kTwMaxLen");
#pragma unroll
  for (int s = 0; s < BPT; ++s) {
    cpx<T> y[R];
#pragma unroll
    for (int r = 0; r < R; ++r) y[r] = x[s + r * BPT];
    if constexpr (NS > 1) {
      int k = (t + s * TPL) & (NS - 1);
      // Opaque to the optimiser: without this the inverse transform's twiddle
      // loads are merged with the forward ones and ~30 values stay live in
      // registers across both transforms (register spills).
      asm volatile("" : "+r"(k)::"memory");
      const cpx<T>* twp = tw + (TWS ? tw_compact_offset(N, E, NS) : tw_offset(R, NS)) + k;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        // load and apply the twiddles in groups of TWG so that at most TWG
        // of them are live at once (bounds register pressure)
        if (r > 1 && (r - 1) % TWG == 0) asm volatile("" ::: "memory");
        cpx<T> w;
        if constexpr (TWS) w = twp[(r - 1) * NS];
        else w = __ldg(twp + (r - 1) * NS);
        if (INV) w.y = -w.y;
        y[r] = cmul<T>(y[r], w);
      }
    }
    DFT<T, R, INV>::run(y);
#pragma unroll
    for (int r = 0; r < R; ++r) x[s + r * BPT] = y[r];
  }
}

// Radix of the pass at stride NS in a transform of N points, E per thread
// (a butterfly never spans more than a thread's elements).
template <int N, int E, int NS>
struct PassRadix {
  static constexpr int RMAX = E < 16 ? E : 16;
  static constexpr int R = (N / NS) >= RMAX ? RMAX : (N / NS);
};

// Number of shared-memory exchanges in one N-point transform.
__host__ __device__ constexpr int fft_exchanges(int n, int e) {
  int k = 0;
  for (int ns = 1;;) {
    const int rmax = e < 16 ? e : 16;
    const int r = (n / ns) >= rmax ? rmax : n / ns;
    if (ns * r >= n) return k;
    ns *= r;
    ++k;
  }
}

// Exchange halves after the pass at stride NS: every thread stores its
// butterfly outputs at their Stockham positions, then (after a barrier) loads
// the elements t + j*TPL of the next pass.
template <typename T, int N, int E, int NS>
__device__ __forceinline__ void exchange_store(const cpx<T> (&x)[E], int t, cpx<T>* sm,
                                               int stride) {
  constexpr int TPL = N / E;
  constexpr int R = PassRadix<N, E, NS>::R;
  constexpr int BPT = E / R;
#pragma unroll
  for (int s = 0; s < BPT; ++s) {
    const int b = t + s * TPL;
    const int base = (b / NS) * NS * R + (b & (NS - 1));
    // padi(base + r*NS) as one computed base plus compile-time offsets
    // whenever the 16-element padding groups allow it
    if constexpr (NS % 16 == 0) {
      const int pb = padi(base) * stride;
#pragma unroll
      for (int r = 0; r < R; ++r) sm[pb + r * (NS + NS / 16) * stride] = x[s + r * BPT];
    } else if constexpr (NS == 1 && R == 16) {
      const int pb = (17 * b) * stride;  // padi(16 b + r) = 17 b + r
#pragma unroll
      for (int r = 0; r < R; ++r) sm[pb + r * stride] = x[s + r * BPT];
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) sm[padi(base + r * NS) * stride] = x[s + r * BPT];
    }
  }
}

template <typename T, int N, int E>
__device__ __forceinline__ void exchange_load(cpx<T> (&x)[E], int t, const cpx<T>* sm,
                                              int stride) {
  constexpr int TPL = N / E;
  if constexpr (TPL % 16 == 0) {
    const int pb = padi(t) * stride;  // padi(t + j TPL) = padi(t) + j (TPL + TPL/16)
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = sm[pb + j * (TPL + TPL / 16) * stride];
  } else {
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = sm[padi(t + j * TPL) * stride];
  }
}

// Full N-point transform of one line.  sm points at the line's padded shared
// buffer; element i lives at sm[padi(i) * STRIDE] (STRIDE > 1 interleaves W
// column lines, the caller offsets sm by the column).  All threads of the
// CTA must call this (it contains __syncthreads).
// Order this thread's generic-proxy shared-memory stores before later bulk
// copies (async proxy) into the same buffer.
__device__ __forceinline__ void fence_async_after_stores() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// FENCE: the exchange buffer is also a bulk-copy staging buffer that is
// refilled later, so the exchange stores are fenced against that copy.
template <typename T, int N, int E, int NS, bool INV, bool FENCE = false, bool TWS = false>
__device__ __forceinline__ void fft_line(cpx<T> (&x)[E], int t, cpx<T>* sm, int stride,
                                         const cpx<T>* __restrict__ tw) {
  constexpr int R = PassRadix<N, E, NS>::R;
  static_assert((E / R) * R == E, "radix must divide the elements per thread");
  if constexpr (NS == 1) {
    // Recompute the shared-memory addresses in every transform instead of
    // keeping those of an earlier transform in this kernel live in registers.
    asm volatile("" : "+r"(t)::"memory");
  }
  stockham_pass<T, N, E, R, NS, INV, TWS>(x, t, tw);
  if constexpr (NS * R < N) {
    __syncthreads();
    exchange_store<T, N, E, NS>(x, t, sm, stride);
    if constexpr (FENCE) fence_async_after_stores();
    __syncthreads();
    exchange_load<T, N, E>(x, t, sm, stride);
    fft_line<T, N, E, NS * R, INV, FENCE, TWS>(x, t, sm, stride, tw);
  }
}

// fft_line with two exchange buffers used alternately (A for the first
// exchange, then B, A, ...), one barrier per exchange instead of two.
// Caller contract: when the transform starts, no thread still reads A or B
// from an earlier use unless a barrier has passed since; with an even number
// of exchanges the last one uses B, so A is free once the transform returns.
// FM: bit 0 / bit 1 fence the stores into A / B (buffers that later receive
// bulk copies).
template <typename T, int N, int E, int NS, bool INV, int P, int FM, bool TWS = false>
__device__ __forceinline__ void fft_line_db(cpx<T> (&x)[E], int t, cpx<T>* smA, cpx<T>* smB,
                                            int stride, const cpx<T>* __restrict__ tw) {
  constexpr int R = PassRadix<N, E, NS>::R;
  static_assert((E / R) * R == E, "radix must divide the elements per thread");
  if constexpr (NS == 1) asm volatile("" : "+r"(t)::"memory");
  stockham_pass<T, N, E, R, NS, INV, TWS>(x, t, tw);
  if constexpr (NS * R < N) {
    cpx<T>* sm = P ? smB : smA;
    exchange_store<T, N, E, NS>(x, t, sm, stride);
    if constexpr ((FM >> P) & 1) fence_async_after_stores();
    __syncthreads();
    exchange_load<T, N, E>(x, t, sm, stride);
    fft_line_db<T, N, E, NS * R, INV, P ^ 1, FM, TWS>(x, t, smA, smB, stride, tw);
  }
}

// fft_line on one buffer whose first exchange needs no leading barrier (the
// caller guarantees that no thread still reads sm, or passes LEAD), with hook() run by every
// thread right after that exchange's barrier: at that point every read of
// shared memory the caller issued before the transform has completed.
// LEAD: start the first exchange with a barrier (when threads may still read sm).
template <typename T, int N, int E, bool INV, bool FENCE, bool LEAD = false, typename Hook>
__device__ __forceinline__ void fft_line_hook(cpx<T> (&x)[E], int t, cpx<T>* sm, int stride,
                                              const cpx<T>* __restrict__ tw, Hook&& hook) {
  constexpr int R = PassRadix<N, E, 1>::R;
  static_assert((E / R) * R == E, "radix must divide the elements per thread");
  asm volatile("" : "+r"(t)::"memory");
  stockham_pass<T, N, E, R, 1, INV>(x, t, tw);
  if constexpr (R < N) {
    if constexpr (LEAD) __syncthreads();
    exchange_store<T, N, E, 1>(x, t, sm, stride);
    if constexpr (FENCE) fence_async_after_stores();
    __syncthreads();
    hook();
    exchange_load<T, N, E>(x, t, sm, stride);
    fft_line<T, N, E, R, INV, FENCE>(x, t, sm, stride, tw);
  } else {
    hook();
  }
}

}  // namespace nlse
