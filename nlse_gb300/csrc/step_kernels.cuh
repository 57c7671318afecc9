// Split-step kernels: row passes (contiguous axis), column passes (strided
// axes) and the pointwise nonlinear operator fused into them.
//
// The arithmetic of the nonlinear operator follows the GPU kernels of the
// reference package (NLSE/kernels_gpu.py):
//   nl_prop            kernels_gpu.py:4-35
//   nl_prop_without_V  kernels_gpu.py:38-65
//   nl_prop_c          kernels_gpu.py:68-104
//   nl_prop_without_V_c kernels_gpu.py:107-139
//   rabi_coupling      kernels_gpu.py:142-156
// and the DDGPE pump callback (NLSE/ddgpe.py:127-156).  All of them are one
// formula here: a single-component field is the two-component formula with
// the cross terms set to g12 = 0, Isat2 = inf, |A2|^2 = 0, which adds exact
// zeros.
#pragma once
#include <type_traits>

#include "fft_core.cuh"
#include "tma.cuh"

namespace nlse {

// ---- parameters -----------------------------------------------------------
// Per-field parameter block, 32 doubles (filled by the host, see capi.cu):
//   [set*16 + comp*7 + k]   set 0 = after the linear step, set 1 = before it
//                            (Strang "double" scheme); k = dz, alpha, g_self,
//                            g_cross, isat_self, isat_cross, vscale
//   [14], [15]              Rabi cos(omega*dz), sin(omega*dz)
//   [30]                    dz used by the pump term
constexpr int kParamStride = 40;

enum : uint32_t {
  F_HAS_V = 1u << 0,      // potential present
  F_V_COMPLEX = 1u << 1,  // potential stored complex (else real)
  F_PROP_C128 = 1u << 2,  // propagator stored as complex128
  F_RABI = 1u << 3,       // Rabi rotation after the nonlinear step
  F_PUMP = 1u << 4,       // DDGPE pump term on component 1
  F_PROBE = 1u << 5,      // DDGPE probe term on component 1
  F_PRE_NL = 1u << 6,     // nonlinear half step before the linear step
  F_ASQ_EXT = 1u << 7,    // |A|^2 read from the external (convolved) buffer
  F_NO_POST = 1u << 8,    // skip the post-linear nonlinear step (plain FFT use)
  F_V_F32 = 1u << 9,      // potential stored in single precision: V' = vscale*V is
                          // formed in FP32 and then widened, as the reference does
                          // for a complex64 V with a complex128 field
  F_IN_BLK = 1u << 10,    // row pass reads the blocked spectral buffer S
  F_OUT_BLK = 1u << 11,   // row pass writes the blocked spectral buffer S
  F_MAPS = 1u << 12,      // per-pixel g / alpha / 1/Isat planes (one-component fields)
};

// Blocked spectral layout of a 2-D slab [NY][NX]: element (y, x) at
// ((x / W) * NY + y) * W + x % W, W = 32 bytes / element size.  A column
// tile (W columns x NY rows) is then one contiguous run, and a row is NX/W
// runs of 32 bytes.
template <typename T> struct BlkW {
  static constexpr int W = 32 / int(sizeof(cpx<T>));
};

struct StepArgs {
  void* A;                  // field, complex T, natural layout
  void* S;                  // spectral scratch, blocked layout (2-D fast path), or null
  const void* V;            // potential: T or cpx<T>, null if absent
  const void* prop;         // propagator: cpx<float> or cpx<double>
  const double* params;     // [nfields][32]
  const void* pump_r;       // cpx<T> [pixels]
  const void* pump_t;       // cpx<T> [steps]
  const void* probe_r;
  const void* probe_t;
  const void* asq;          // T [nfields][comps][pixels] (nonlocal |A|^2), or null
  const void* tw;           // per-pass twiddle tables cpx<T> [kTwTableLen]
  const float* params_f32;  // FP32 mirror of params (complex64 kernels)
  int64_t nq;               // pixel-lines (fields * lines_per_comp)
  int64_t lines_per_comp;   // lines of one component of one field
  int64_t pix;              // pixels of one component of one field
  int64_t v_fstride;        // field stride of V (0: shared)
  int64_t prop_cstride;     // component stride of the propagator
  double inv_n;             // 1 / (number of pixels), inverse-FFT normalisation
  float inv_nf;             // the same in FP32 (exact: a power of two)
  int comps;                // 1 or 2
  int step;                 // step index (pump time profile)
  int nsteps;               // steps fused inside one launch (1-D full mode)
  uint32_t flags;
  int* status;              // plan status word (bounded waits record timeouts here)
  int tma_grid;             // >0: TMA-fed persistent inverse row pass on this many SMs
  const CUtensorMap* tmap;  // host pointer to the plan's tensor map of S (passed by value)
  int cap_per_sm;           // >0: at most this many persistent CTAs per SM
  const void* maps;         // T planes [3][map fields][pix]: g, alpha/2, 1/Isat' (F_MAPS)
  int64_t maps_fstride;     // field stride of the planes (0: shared)
  int64_t maps_plane;       // elements between planes
  int maps_mask;            // planes present (bit 0 g, 1 alpha, 2 1/Isat')
};

// Per-pixel nonlinear coefficients: the planes present replace the line's
// per-field values (idx = pixel index within the field).
template <typename T, typename P>
__device__ __forceinline__ void apply_maps(P& p, const StepArgs& a, int64_t f, int64_t idx) {
  const T* M = reinterpret_cast<const T*>(a.maps) + f * a.maps_fstride + idx;
  if (a.maps_mask & 1) p.gs = __ldg(M);
  if (a.maps_mask & 2) p.alpha = __ldg(M + a.maps_plane);
  if (a.maps_mask & 4) p.ris = __ldg(M + 2 * a.maps_plane);
}

struct ColArgs {
  void* A;
  int* status;              // plan status word (bounded waits record timeouts here)
  const void* prop;
  const void* tw;
  int64_t nblocks;          // column blocks * outer
  int64_t ncb;              // column blocks per outer slab
  int64_t outer_stride;     // elements between outer slabs
  int64_t ld;               // elements between consecutive points of a column
  int64_t prop_cstride;
  int comps;                // outer index % comps selects the propagator component
  int w;                    // columns per block (power of two)
  uint32_t flags;
  int tma_grid;             // >0: persistent TMA-ring column pass on this many SMs
  int cap_per_sm;           // >0: at most this many persistent CTAs per SM
};

template <typename T> struct NLP {
  T dz, alpha, gs, gc, is, ic, vs;
  T ris, ric;  // 1/is, 1/ic (per-thread reciprocals of the per-field constants)
  T dzi;       // imaginary part of dz (imaginary-time evolution), else 0
};

// Parameters in the kernel's precision: complex64 kernels read the FP32
// mirror of the block (rounded once per call by k_params_f32), so no FP64
// instruction runs in their hot loops.
template <typename T>
__device__ __forceinline__ const T* param_block(const StepArgs& a);

template <typename T>
__device__ __forceinline__ NLP<T> load_nlp(const T* __restrict__ p) {
  NLP<T> r;
  r.dz = __ldg(p + 0);
  r.alpha = __ldg(p + 1);
  r.gs = __ldg(p + 2);
  r.gc = __ldg(p + 3);
  r.is = __ldg(p + 4);
  r.ic = __ldg(p + 5);
  r.vs = __ldg(p + 6);
  r.ris = T(1) / r.is;
  r.ric = T(1) / r.ic;
  r.dzi = T(0);
  return r;
}

__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// ---- exp(re) * (cos(im), sin(im)) ------------------------------------------
// The split step's per-step arguments are small (|re| = alpha*sat*dz,
// |im| = phase per step), so the common case evaluates truncated Maclaurin
// polynomials of exp, sin and cos in Horner form with the coefficients 1/k!
// (one FMA per term).  The degrees are chosen so that the first omitted term
// is far below one unit in the last place on the range:
//   float:  |re| <= 1/16: exp to x^5 (next term < 1e-10);
//           |im| <= 1/4:  sin to x^7 (< 1e-11), cos to x^8 (< 3e-13)
//   double: |re| <= 1/32: exp to x^8 (< 3e-17);
//           |im| <= 1/4:  sin to x^11 (< 3e-18), cos to x^12 (< 2e-19)
// sin is formed as im + (im*x^2)*p(x^2), so its leading term is exact.
// Outside the range the CUDA library functions are called from a non-inlined
// helper, which keeps the unrolled kernels small.
static __device__ __noinline__ void cis_exp_lib(float re, float im, float* cr, float* ci) {
  float sn, cs;
  sincosf(im, &sn, &cs);
  const float e = expf(re);
  *cr = e * cs;
  *ci = e * sn;
}
static __device__ __noinline__ void cis_exp_lib(double re, double im, double* cr, double* ci) {
  double sn, cs;
  sincos(im, &sn, &cs);
  const double e = exp(re);
  *cr = e * cs;
  *ci = e * sn;
}

// 1/k! and (-1)^k/(2k+1)!, (-1)^k/(2k)! evaluated in double at compile time
__host__ __device__ constexpr double inv_fact(int k) {
  double r = 1.0;
  for (int i = 2; i <= k; ++i) r /= i;
  return r;
}
__host__ __device__ constexpr double sin_coef(int k) {  // coefficient of x^(2k+1)
  return (k % 2 ? -1.0 : 1.0) * inv_fact(2 * k + 1);
}
__host__ __device__ constexpr double cos_coef(int k) {  // coefficient of x^(2k)
  return (k % 2 ? -1.0 : 1.0) * inv_fact(2 * k);
}

template <typename T> struct CisRange;
template <> struct CisRange<float> {
  static constexpr float RE = 0.0625f, IM = 0.25f;
  static constexpr int EXP_DEG = 5, SIN_K = 3, COS_K = 4;  // sin to x^(2*3+1), cos to x^(2*4)
};
template <> struct CisRange<double> {
  static constexpr double RE = 0.03125, IM = 0.25;
  static constexpr int EXP_DEG = 8, SIN_K = 5, COS_K = 6;
};

template <typename T>
__device__ __forceinline__ void cis_exp(T re, T im, T* cr, T* ci) {
  using R = CisRange<T>;
  if (fabs(re) <= R::RE && fabs(im) <= R::IM) {
    T e = T(inv_fact(R::EXP_DEG));
#pragma unroll
    for (int k = R::EXP_DEG - 1; k >= 0; --k) e = fma(e, re, T(inv_fact(k)));
    const T x2 = im * im;
    T s = T(sin_coef(R::SIN_K));
#pragma unroll
    for (int k = R::SIN_K - 1; k >= 1; --k) s = fma(s, x2, T(sin_coef(k)));
    const T sn = fma(im * x2, s, im);
    T c = T(cos_coef(R::COS_K));
#pragma unroll
    for (int k = R::COS_K - 1; k >= 0; --k) c = fma(c, x2, T(cos_coef(k)));
    *cr = e * c;
    *ci = e * sn;
  } else {
    cis_exp_lib(re, im, cr, ci);
  }
}

// One nonlinear sub-step on one point (kernels_gpu.py:68-104 form):
//   sat = 1 / (1 + a_s/Isat_s + a_c/Isat_c)
//   arg = i*(g_s*a_s*sat + g_c*a_c*sat) - alpha*sat + i*V',  V' = vscale*V
//   A  *= exp(dz*arg)
// TWO: the partner component's |A|^2 enters the saturation.  The divisions
// a/Isat of the reference are multiplications by the per-field reciprocal
// (within one rounding of the quotient); 1/(...) is the correctly rounded
// reciprocal, identical to the reference's division of 1.
template <typename T, bool TWO = true>
__device__ __forceinline__ cpx<T> nl_point(cpx<T> A, T a_s, T a_c, const NLP<T>& p, bool has_v,
                                           cpx<T> vp) {
  T den = T(1) + a_s * p.ris;
  if (TWO) den = den + a_c * p.ric;
  const T sat = rcp_rn(den);
  T im = p.gs * a_s * sat;
  if (TWO) im = im + p.gc * a_c * sat;
  T re = -p.alpha * sat;
  if (has_v) {
    // arg += 1j * V'  ->  (re - Im V', im + Re V')
    re = re - vp.y;
    im = im + vp.x;
  }
  // (re + i im) * (dz + i dzi); with dzi = 0 exactly the rounded real products
  const T re0 = re, im0 = im;
  re = fma(-im0, p.dzi, mul_rn(re0, p.dz));
  im = fma(re0, p.dzi, mul_rn(im0, p.dz));
  T cr, ci;
  cis_exp<T>(re, im, &cr, &ci);
  return cmul<T>(A, mk<T>(cr, ci));
}

// Parameters of one nonlinear sub-step on two lanes (two lines, or two
// positions of one line: then both lanes hold the same values).
struct NLP2 {
  float2 dz, nalpha, gs, ris, vs, dzi;
  bool real_dz;
};

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// exp(re) * (cos(im), sin(im)) for both lanes: the truncated series of
// cis_exp in packed form, the library functions for a
// lane outside the series' range.
__device__ __forceinline__ void pcis_exp(float2 re, float2 im, float2* cr, float2* ci) {
  using R = CisRange<float>;
  float2 e = f2s(float(inv_fact(R::EXP_DEG)));
#pragma unroll
  for (int k = R::EXP_DEG - 1; k >= 0; --k) e = fma2(e, re, f2s(float(inv_fact(k))));
  const float2 x2 = mul2(im, im);
  float2 s = f2s(float(sin_coef(R::SIN_K)));
#pragma unroll
  for (int k = R::SIN_K - 1; k >= 1; --k) s = fma2(s, x2, f2s(float(sin_coef(k))));
  const float2 sn = fma2(mul2(im, x2), s, im);
  float2 c = f2s(float(cos_coef(R::COS_K)));
#pragma unroll
  for (int k = R::COS_K - 1; k >= 0; --k) c = fma2(c, x2, f2s(float(cos_coef(k))));
  *cr = mul2(e, c);
  *ci = mul2(e, sn);
  const bool ina = fabsf(re.x) <= R::RE && fabsf(im.x) <= R::IM;
  const bool inb = fabsf(re.y) <= R::RE && fabsf(im.y) <= R::IM;
  if (!(ina && inb)) {
    if (!ina) cis_exp_lib(re.x, im.x, &cr->x, &ci->x);
    if (!inb) cis_exp_lib(re.y, im.y, &cr->y, &ci->y);
  }
}

// One nonlinear sub-step on one pair point; v = vscale * V of each lane
// (v.x/v.y = real parts, vi = imaginary parts or zero).
__device__ __forceinline__ cp2 nl_pair_point(cp2 x, const NLP2& p, bool has_v, float2 vre,
                                             float2 vim) {
  const float2 one = f2s(1.0f);
  const float2 as = fma2(x.re, x.re, mul2(x.im, x.im));
  const float2 den = fma2(as, p.ris, one);
  float2 sat = f2(rcp_approx(den.x), rcp_approx(den.y));
  sat = fma2(sat, fnma2(den, sat, one), sat);  // one Newton step
  float2 im = mul2(mul2(p.gs, as), sat);
  float2 re = mul2(p.nalpha, sat);
  if (has_v) {
    re = sub2(re, vim);
    im = add2(im, vre);
  }
  float2 ar, ai;
  if (p.real_dz) {
    ar = mul2(re, p.dz);
    ai = mul2(im, p.dz);
  } else {
    ar = fnma2(im, p.dzi, mul2(re, p.dz));
    ai = fma2(re, p.dzi, mul2(im, p.dz));
  }
  float2 cr, ci;
  pcis_exp(ar, ai, &cr, &ci);
  return {fnma2(x.im, ci, mul2(x.re, cr)), fma2(x.re, ci, mul2(x.im, cr))};
}

// Rabi rotation (kernels_gpu.py:142-156): y' = c y - i s yo with c, s the
// cosine and sine of (omega/2) dz -- complex for a complex dz (ci, si their
// imaginary parts), else the real form of the reference's real step.
template <typename T>
__device__ __forceinline__ cpx<T> rabi_rot(cpx<T> y, cpx<T> yo, T rc, T rs, T ci, T si) {
  if (ci == T(0) && si == T(0)) return mk<T>(rc * y.x + rs * yo.y, rc * y.y - rs * yo.x);
  return mk<T>(rc * y.x - ci * y.y + rs * yo.y + si * yo.x,
               rc * y.y + ci * y.x + si * yo.y - rs * yo.x);
}

// F * dz for the DDGPE source term A2 -= F dz i (ddgpe.py:155-156): the
// product with a real step, or the complex product with dz = dr + i di (a
// complex delta_z).
template <typename T>
__device__ __forceinline__ cpx<T> pump_dz(cpx<T> u, T dr, T di) {
  if (di == T(0)) return mk<T>(mul_rn(u.x, dr), mul_rn(u.y, dr));
  return cmul<T>(u, mk<T>(dr, di));
}

template <typename T>
__device__ __forceinline__ T inv_n_of(const StepArgs& a) {
  if constexpr (std::is_same<T, float>::value) return a.inv_nf;
  else return a.inv_n;
}

template <typename T>
__device__ __forceinline__ T abs2(cpx<T> a) {
  return a.x * a.x + a.y * a.y;
}

template <>
__device__ __forceinline__ const float* param_block<float>(const StepArgs& a) {
  return a.params_f32;
}
template <>
__device__ __forceinline__ const double* param_block<double>(const StepArgs& a) {
  return a.params;
}

// V' = vscale * V rounded the way the reference rounds its k/2*V array: in
// the storage precision of V, then widened to the field precision.
template <typename T>
__device__ __forceinline__ cpx<T> load_vp(const void* V, uint32_t flags, int64_t idx, T vs) {
  // complex64 fields always carry a single-precision potential (checked on
  // the host); the FP64 branch must not even be if-converted into them
  if (std::is_same<T, float>::value || (flags & F_V_F32)) {
    const float fs = float(vs);
    float2 v;
    if (flags & F_V_COMPLEX) v = __ldg(reinterpret_cast<const float2*>(V) + idx);
    else v = make_float2(__ldg(reinterpret_cast<const float*>(V) + idx), 0.f);
    return mk<T>(T(__fmul_rn(fs, v.x)), T(__fmul_rn(fs, v.y)));
  }
  double2 v;
  if (flags & F_V_COMPLEX) v = __ldg(reinterpret_cast<const double2*>(V) + idx);
  else v = make_double2(__ldg(reinterpret_cast<const double*>(V) + idx), 0.0);
  return mk<T>(T(__dmul_rn(double(vs), v.x)), T(__dmul_rn(double(vs), v.y)));
}

// Field times propagator; PC128: the propagator is stored complex128 (a
// compile-time choice: a runtime branch gets if-converted, putting FP64
// multiplies, 1/64 of the FP32 rate on this part, into every complex64 step).
template <typename T, bool PC128>
__device__ __forceinline__ cpx<T> mul_prop(cpx<T> x, const void* prop, int64_t idx) {
  if constexpr (PC128) {
    const double2 p = __ldg(reinterpret_cast<const double2*>(prop) + idx);
    if constexpr (std::is_same<T, float>::value) {
      // complex64 field times complex128 propagator: product in FP64, rounded
      const double xr = x.x, xi = x.y;
      return mk<T>(T(xr * p.x - xi * p.y), T(xr * p.y + xi * p.x));
    } else {
      return cmul<T>(x, mk<T>(T(p.x), T(p.y)));
    }
  } else {
    const float2 p = __ldg(reinterpret_cast<const float2*>(prop) + idx);
    return cmul<T>(x, mk<T>(T(p.x), T(p.y)));
  }
}

// Nonlinear step (set 0 or 1) for the E points a thread owns of one line.
// x: own component, xo: partner component (two-component models only, same
// positions).  pix0: pixel index of position t within the component, the
// thread's points are pix0 + j*TPL.
// Real single-precision potential values of the thread's points, loaded at
// kernel entry (before the FFT's barriers) so their latency is hidden.
template <int E> struct VPre {
  float v[E];
  bool on;
};

template <typename T, int E, int TPL, int NC>
__device__ __forceinline__ void nl_line(cpx<T> (&x)[E], const cpx<T> (&xo)[E], const StepArgs& a,
                                        int64_t f, int comp, int64_t pix0, int set, bool post,
                                        const VPre<E>* vpre = nullptr) {
  const T* P = param_block<T>(a) + f * kParamStride + set * 16;
  NLP<T> ps = load_nlp<T>(P + comp * 7);
  ps.dzi = __ldg(param_block<T>(a) + f * kParamStride + 32 + set);
  constexpr bool two = NC == 2;
  const bool rabi = two && post && (a.flags & F_RABI);
  NLP<T> po;
  if (rabi) {
    po = load_nlp<T>(P + (1 - comp) * 7);
    po.dzi = ps.dzi;
  }
  const bool has_v = a.flags & F_HAS_V;
  const int64_t vb = f * a.v_fstride + pix0;
  const T* asq = reinterpret_cast<const T*>(a.asq);
  const int64_t qb_s = (f * NC + comp) * a.pix + pix0;
  const int64_t qb_o = (f * NC + (1 - comp)) * a.pix + pix0;
  T rc = T(0), rs = T(0), ric = T(0), ris = T(0);
  if (rabi) {
    rc = __ldg(param_block<T>(a) + f * kParamStride + 14);
    rs = __ldg(param_block<T>(a) + f * kParamStride + 15);
    ric = __ldg(param_block<T>(a) + f * kParamStride + 34);
    ris = __ldg(param_block<T>(a) + f * kParamStride + 35);
  }
#pragma unroll
  for (int j = 0; j < E; ++j) {
    T as, ao = T(0);
    if (a.flags & F_ASQ_EXT) {
      as = asq[qb_s + j * TPL];
      if (two) ao = asq[qb_o + j * TPL];
    } else {
      as = abs2<T>(x[j]);
      if (two) ao = abs2<T>(xo[j]);
    }
    cpx<T> v = mk<T>(T(0), T(0));
    if (has_v) {
      if (vpre && vpre->on)
        v = mk<T>(T(__fmul_rn(float(ps.vs), vpre->v[j])), T(0));
      else
        v = load_vp<T>(a.V, a.flags, vb + j * TPL, ps.vs);
    }
    NLP<T> pm = ps;
    if constexpr (!two) {
      if (a.flags & F_MAPS) apply_maps<T>(pm, a, f, pix0 + j * TPL);
    }
    cpx<T> y = nl_point<T, two>(x[j], as, ao, pm, has_v, v);
    if (two && rabi) {
      // kernels_gpu.py:154-156: A1' = cos*A1 - i*sin*A2, A2' = cos*A2 - i*sin*A1
      const cpx<T> vo = has_v ? load_vp<T>(a.V, a.flags, vb + j * TPL, po.vs) : mk<T>(T(0), T(0));
      const cpx<T> yo = nl_point<T, two>(xo[j], ao, as, po, has_v, vo);
      y = rabi_rot<T>(y, yo, rc, rs, ric, ris);
    }
    x[j] = y;
  }
  if (two && post && comp == 1 && (a.flags & (F_PUMP | F_PROBE))) {
    // ddgpe.py:155-156: A2 -= F_r * F_t[i] * dz * 1j  (pump, then probe)
    const T dz = __ldg(param_block<T>(a) + f * kParamStride + 30);
    const T dzi = __ldg(param_block<T>(a) + f * kParamStride + 31);
    const cpx<T>* pr = reinterpret_cast<const cpx<T>*>(a.pump_r);
    const cpx<T>* qr = reinterpret_cast<const cpx<T>*>(a.probe_r);
    const cpx<T> ptv = (a.flags & F_PUMP) ? reinterpret_cast<const cpx<T>*>(a.pump_t)[a.step]
                                          : mk<T>(T(0), T(0));
    const cpx<T> qtv = (a.flags & F_PROBE) ? reinterpret_cast<const cpx<T>*>(a.probe_t)[a.step]
                                           : mk<T>(T(0), T(0));
#pragma unroll
    for (int j = 0; j < E; ++j) {
      if (a.flags & F_PUMP) {
        const cpx<T> u = pump_dz<T>(cmul<T>(pr[pix0 + j * TPL], ptv), dz, dzi);
        x[j] = mk<T>(x[j].x + u.y, x[j].y - u.x);
      }
      if (a.flags & F_PROBE) {
        const cpx<T> u = pump_dz<T>(cmul<T>(qr[pix0 + j * TPL], qtv), dz, dzi);
        x[j] = mk<T>(x[j].x + u.y, x[j].y - u.x);
      }
    }
  }
}

// ---- row kernels ----------------------------------------------------------
enum RowMode : int {
  ROW_FWD = 0,         // [pre-NL] forward FFT
  ROW_INV_NL = 1,      // inverse FFT, 1/N, post-NL [Rabi, pump]
  ROW_INV_NL_FWD = 2,  // ROW_INV_NL, then [pre-NL] and the next forward FFT
  ROW_FULL = 3,        // 1-D: [pre-NL] FFT, propagator, iFFT, 1/N, post-NL; nsteps times
  ROW_INV = 4,         // inverse FFT with 1/N only
};

template <int N, int E> struct RowCfg {
  static constexpr int TPL = N / E;
  static constexpr int LPB = (256 / TPL) >= 2 ? 256 / TPL : 2;  // lines per block, even
  static constexpr int THREADS = LPB * TPL;
  static constexpr int SL = padded_len(N);
};

template <typename T, int N, int E>
__device__ __forceinline__ void exchange_partner(const cpx<T> (&x)[E], cpx<T> (&xo)[E], cpx<T>* sm,
                                                 int lb, int t) {
  constexpr int TPL = N / E, SL = RowCfg<N, E>::SL;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < E; ++j) sm[lb * SL + padi(t + j * TPL)] = x[j];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < E; ++j) xo[j] = sm[(lb ^ 1) * SL + padi(t + j * TPL)];
}

template <typename T, int N, int E, int MODE, int NC>
__global__ void __launch_bounds__(RowCfg<N, E>::THREADS) k_rows(const StepArgs a) {
  using C = cpx<T>;
  constexpr int TPL = RowCfg<N, E>::TPL, LPB = RowCfg<N, E>::LPB, SL = RowCfg<N, E>::SL;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const int lb = threadIdx.x / TPL, t = threadIdx.x % TPL;
  constexpr int nc = NC;
  const int comp = lb % nc;
  const int64_t q = (int64_t)blockIdx.x * (LPB / nc) + lb / nc;
  const bool act = q < a.nq;
  const int64_t qq = act ? q : 0;
  const int64_t f = qq / a.lines_per_comp, m = qq % a.lines_per_comp;
  const int64_t pix0 = m * N + t;
  C* sml = sm + lb * SL;
  constexpr bool two = NC == 2;
  // source and destination: natural rows of A, or blocked rows of S
  constexpr int W = BlkW<T>::W;
  const int64_t slab = (f * nc + comp) * a.pix;
  C* nat = reinterpret_cast<C*>(a.A) + slab + m * N + t;
  C* blk = reinterpret_cast<C*>(a.S) + slab + ((t / W) * a.lines_per_comp + m) * W + (t % W);
  const int64_t bstr = (int64_t)TPL * a.lines_per_comp;
  const C* src = (a.flags & F_IN_BLK) ? blk : nat;
  const int64_t sstr = (a.flags & F_IN_BLK) ? bstr : TPL;

  C x[E], xo[E];
#pragma unroll
  for (int j = 0; j < E; ++j) x[j] = act ? src[j * sstr] : mk<T>(T(0), T(0));
  VPre<E> vpre;
  vpre.on = (MODE == ROW_INV_NL || MODE == ROW_INV_NL_FWD) && (a.flags & F_HAS_V) &&
            (a.flags & F_V_F32) && !(a.flags & F_V_COMPLEX);
  if (vpre.on) {
    const float* vp = reinterpret_cast<const float*>(a.V) + f * a.v_fstride + pix0;
#pragma unroll
    for (int j = 0; j < E; ++j) vpre.v[j] = __ldg(vp + j * TPL);
  }

  if constexpr (MODE == ROW_FWD || MODE == ROW_FULL) {
    if (a.flags & F_PRE_NL) {
      if (two) exchange_partner<T, N, E>(x, xo, sm, lb, t);
      nl_line<T, E, TPL, NC>(x, xo, a, f, comp, pix0, 1, false);
    }
  }
  const int nsteps = (MODE == ROW_FULL) ? a.nsteps : 1;
  for (int st = 0; st < nsteps; ++st) {
    if constexpr (MODE == ROW_FULL) {
      if (st > 0 && (a.flags & F_PRE_NL)) {
        if (two) exchange_partner<T, N, E>(x, xo, sm, lb, t);
        nl_line<T, E, TPL, NC>(x, xo, a, f, comp, pix0, 1, false);
      }
      fft_line<T, N, E, 1, false>(x, t, sml, 1, tw);
      const int64_t pb = comp * a.prop_cstride + t;
      if (a.flags & F_PROP_C128) {
#pragma unroll
        for (int j = 0; j < E; ++j) x[j] = mul_prop<T, true>(x[j], a.prop, pb + j * TPL);
      } else {
#pragma unroll
        for (int j = 0; j < E; ++j) x[j] = mul_prop<T, false>(x[j], a.prop, pb + j * TPL);
      }
    }
    if constexpr (MODE == ROW_FWD) {
      fft_line<T, N, E, 1, false>(x, t, sml, 1, tw);
    } else {
      fft_line<T, N, E, 1, true>(x, t, sml, 1, tw);
      // the blocked buffer's column pass applied 1/N already (k_prop_to_blk)
      if (!(a.flags & F_IN_BLK)) {
        const T s = inv_n_of<T>(a);
#pragma unroll
        for (int j = 0; j < E; ++j) x[j] = cscale<T>(x[j], s);
      }
      if constexpr (MODE != ROW_INV) {
        if (!(a.flags & F_NO_POST)) {
          if (two) exchange_partner<T, N, E>(x, xo, sm, lb, t);
          nl_line<T, E, TPL, NC>(x, xo, a, f, comp, pix0, 0, true, &vpre);
        }
      }
      if constexpr (MODE == ROW_INV_NL_FWD) {
        if (a.flags & F_PRE_NL) {
          if (two) exchange_partner<T, N, E>(x, xo, sm, lb, t);
          nl_line<T, E, TPL, NC>(x, xo, a, f, comp, pix0, 1, false);
        }
        fft_line<T, N, E, 1, false>(x, t, sml, 1, tw);
      }
    }
  }
  if (act) {
    C* dst = (a.flags & F_OUT_BLK) ? blk : nat;
    const int64_t dstr = (a.flags & F_OUT_BLK) ? bstr : TPL;
#pragma unroll
    for (int j = 0; j < E; ++j) dst[j * dstr] = x[j];
  }
}

// Persistent inverse row pass (ROW_INV_NL / ROW_INV_NL_FWD) on the blocked
// spectral buffer, fed by tensor-map bulk copies: a blocked row is N/W runs
// of W elements; the 4-D map {2W scalars, NY, N/W, slabs} with a box of one
// row and up to 256 runs lands the row in shared memory in natural order.
// Two stages: row q+grid is in flight while row q is transformed.
// Elements of one staging line or tile: the padded exchange length rounded up
// so that every staging buffer starts on a 128-byte boundary (the alignment a
// tensor-map copy needs for its shared-memory destination).
template <typename T>
__host__ __device__ constexpr int stage_len(int n) {
  constexpr int q = 128 / (int)sizeof(cpx<T>);
  return (n + q - 1) / q * q;
}

constexpr int kRowStages = 2;

// Shape of the TMA row pass: LPC lines (of NC components) per CTA, so that a
// CTA has at least 128 threads when a line needs fewer.
template <typename T, int N, int NC>
struct RowTma {
  static constexpr int E = Shape<N>::E, TPL = N / E;
  static constexpr int LPC = (NC * TPL) >= 128 ? 1 : 128 / (NC * TPL);
  static constexpr int THREADS = LPC * NC * TPL;
  static constexpr int SLS = stage_len<T>(padded_len(N));
};

template <typename T, int N, int NC>
__host__ __device__ constexpr size_t rows_tma_smem() {
  // two buffers of LPC x NC padded lines that alternate as staging and
  // exchange buffers, and one mbarrier per buffer
  return (size_t)2 * RowTma<T, N, NC>::LPC * NC * RowTma<T, N, NC>::SLS * sizeof(cpx<T>) +
         kRowStages * sizeof(uint64_t);
}

template <typename T, int N, int E, int MODE, int NC>
__global__ void __launch_bounds__(RowTma<T, N, NC>::THREADS) k_rows_tma(
    const StepArgs a, const __grid_constant__ CUtensorMap tmS) {
  using C = cpx<T>;
  using RT = RowTma<T, N, NC>;
  constexpr int TPL = N / E, W = BlkW<T>::W, NB = N / W, LPC = RT::LPC, SLS = RT::SLS;
  constexpr int BOXB = NB < 256 ? NB : 256, NBOX = NB / BOXB;
  constexpr unsigned ROW_BYTES = N * sizeof(C);
  constexpr bool two = NC == 2;
  static_assert(E == RT::E, "shared-memory size assumes Shape<N>::E");
  static_assert((SLS * sizeof(C)) % 128 == 0 && (BOXB * W * sizeof(C)) % 128 == 0,
                "tensor-map copies need 128-byte aligned shared destinations");
  // A CTA takes a group of LPC consecutive lines per iteration.  Two buffers
  // X0, X1 (LPC x NC padded lines each) alternate: group i arrives in X[i&1]
  // by tensor-map copies; its inverse transform uses X[i&1] (A) and, with two
  // exchanges, X[(i+1)&1] (B); the forward transform uses A alone, and B
  // receives group i+1 as soon as the forward transform's first barrier has
  // passed.  With a single exchange per transform the forward transform
  // starts with a barrier (A was just read by the inverse one).
  constexpr int NEX = fft_exchanges(N, E);
  static_assert(NEX == 1 || NEX == 2, "one or two exchanges per transform");
  extern __shared__ __align__(128) unsigned char smraw[];
  C* X = reinterpret_cast<C*>(smraw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(X + 2 * LPC * NC * SLS);
  if (!smem_base_aligned(X)) {  // tensor-map copies need a 128-byte aligned destination
    if (threadIdx.x == 0) atomicExch(a.status, DEV_SMEM_MISALIGNED);
    return;
  }
  auto buf = [&](int b, int li, int cc) { return X + ((b * LPC + li) * NC + cc) * SLS; };
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const int li = threadIdx.x / (NC * TPL);
  const int comp = (threadIdx.x / TPL) % NC, t = threadIdx.x % TPL;
  // line indices fit 32 bits (checked when the kernel is chosen), so the
  // per-line division below is a 32-bit one
  const unsigned nq = (unsigned)a.nq;
  const unsigned ngroups = (nq + LPC - 1) / LPC;

  // pixel-line q = (line y, field f) with the field fastest: the lines of a
  // group and the CTAs of a wave share potential lines in L2
  const unsigned nf = nq / (unsigned)a.lines_per_comp;
  auto q_f = [&](unsigned q) { return q % nf; };
  auto q_y = [&](unsigned q) { return q / nf; };
  auto issue = [&](int b, unsigned g) {
    const unsigned q0 = g * LPC;
    const unsigned nl = nq - q0 < (unsigned)LPC ? nq - q0 : (unsigned)LPC;
    mbar_arrive_expect_tx(&bar[b], nl * NC * ROW_BYTES);
    for (unsigned l = 0; l < nl; ++l) {
      const unsigned f = q_f(q0 + l), y = q_y(q0 + l);
#pragma unroll
      for (int cc = 0; cc < NC; ++cc)
#pragma unroll
        for (int bx = 0; bx < NBOX; ++bx)
          tensor_load_4d(buf(b, (int)l, cc) + bx * BOXB * W, &tmS, 0, (int)y, bx * BOXB,
                         (int)(f * NC + cc), &bar[b]);
    }
  };
  // load group gn into buffer b once every generic access to b is complete
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
  int it = 0;
  for (unsigned g = blockIdx.x; g < ngroups; g += gridDim.x, ++it) {
    const int st = it & 1;  // kRowStages == 2
    const unsigned par = (it >> 1) & 1;
    // the previous group's row stores have read the buffer this group writes
    // as its second exchange buffer and refills
    if (MODE == ROW_INV_NL_FWD && threadIdx.x == 0) bulk_wait_read_all();
    const bool ok = mbar_wait_bounded(&bar[st], par);
    if (!__syncthreads_and(ok)) {
      // give up: record it, let the copy in flight land (bounded), leave
      if (threadIdx.x == 0) {
        atomicExch(a.status, DEV_WAIT_TIMEOUT);
        mbar_wait_bounded(&bar[st], par);
      }
      return;
    }
    // lines past the end (last group) compute on an in-range line and store nothing
    const unsigned q = g * LPC + li;
    const bool act = q < nq;
    const unsigned qc = act ? q : nq - 1;
    const int64_t f = q_f(qc), m = q_y(qc);
    const int64_t pix0 = m * (int64_t)N + t;
    C x[E], xo[E];
    C* sA = buf(st, li, comp);
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = sA[t + j * TPL];
    VPre<E> vpre;
    vpre.on = (a.flags & F_HAS_V) && (a.flags & F_V_F32) && !(a.flags & F_V_COMPLEX);
    if (vpre.on) {
      const float* vp = reinterpret_cast<const float*>(a.V) + f * a.v_fstride + pix0;
#pragma unroll
      for (int j = 0; j < E; ++j) vpre.v[j] = __ldg(vp + j * TPL);
    }
    __syncthreads();  // every thread has read its line from buffer st
    C* sB = buf(st ^ 1, li, comp);  // second exchange buffer
    C* xpart = buf(st ^ 1, li, 0);  // partner exchange region (NC lines)
    fft_line_db<T, N, E, 1, true, 0, 3>(x, t, sA, sB, 1, tw);
    // (1/N: applied by the column pass through the blocked propagator)
    if (!(a.flags & F_NO_POST)) {
      if (two) {
        exchange_partner<T, N, E>(x, xo, xpart, comp, t);
        fence_proxy_async_smem();
      }
      nl_line<T, E, TPL, NC>(x, xo, a, f, comp, pix0, 0, true, &vpre);
    }
    const int64_t slab = (f * NC + comp) * a.pix;
    if constexpr (MODE == ROW_INV_NL_FWD) {
      if (a.flags & F_PRE_NL) {
        if (two) {
          exchange_partner<T, N, E>(x, xo, xpart, comp, t);
          fence_proxy_async_smem();
        }
        nl_line<T, E, TPL, NC>(x, xo, a, f, comp, pix0, 1, false);
      }
      // forward transform in A alone; after its first barrier B is no longer read
      fft_line_hook<T, N, E, false, true, NEX == 1>(x, t, sA, 1, tw, [&] {
        if (threadIdx.x == 0) prefetch(st ^ 1, g + gridDim.x);
      });
      // the group's rows leave through A in natural order (a row of the
      // blocked layout is its runs of W elements back to back: one
      // tensor-map box) and tensor-map stores issued by thread 0, instead of
      // 8/16-byte stores per thread; the loop's next turn waits for the
      // stores' reads before A is written again
      __syncthreads();  // every exchange read of A is complete
#pragma unroll
      for (int j = 0; j < E; ++j) sA[t + j * TPL] = x[j];
      fence_proxy_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) {
        const unsigned q0 = g * LPC;
        const unsigned nl = nq - q0 < (unsigned)LPC ? nq - q0 : (unsigned)LPC;
        for (unsigned l = 0; l < nl; ++l) {
          const unsigned fl = q_f(q0 + l), yl = q_y(q0 + l);
#pragma unroll
          for (int cc = 0; cc < NC; ++cc)
#pragma unroll
            for (int bx = 0; bx < NBOX; ++bx)
              tensor_store_4d(&tmS, 0, (int)yl, bx * BOXB, (int)(fl * NC + cc),
                              buf(st, (int)l, cc) + bx * BOXB * W);
        }
        bulk_commit_group();
      }
    } else {
      __syncthreads();  // B is no longer read
      if (threadIdx.x == 0) prefetch(st ^ 1, g + gridDim.x);
      if (act) {
        C* dst = reinterpret_cast<C*>(a.A) + slab + m * N + t;
#pragma unroll
        for (int j = 0; j < E; ++j) dst[j * TPL] = x[j];
      }
    }
  }
  if (MODE == ROW_INV_NL_FWD && threadIdx.x == 0) bulk_wait_all();
}

// ---- column kernels -------------------------------------------------------
enum ColMode : int {
  COL_FWD = 0,
  COL_INV = 1,           // no normalisation (applied by the last row pass)
  COL_FWD_PROP_INV = 2,  // forward, propagator multiply, inverse
};

constexpr int kColMaxThreads = 512;

template <typename T, int N, int E, int MODE, bool PC128>
__global__ void __launch_bounds__(kColMaxThreads) k_cols(const ColArgs a) {
  using C = cpx<T>;
  constexpr int TPL = N / E;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const int W = a.w;
  const int c = threadIdx.x & (W - 1), t = threadIdx.x / W;
  const int64_t blk = blockIdx.x;
  const int64_t b = blk % a.ncb, o = blk / a.ncb;
  C* base = reinterpret_cast<C*>(a.A) + o * a.outer_stride + b * W + c;
  C x[E];
#pragma unroll
  for (int j = 0; j < E; ++j) x[j] = base[(int64_t)(t + j * TPL) * a.ld];
  fft_line<T, N, E, 1, MODE == COL_INV>(x, t, sm + c, W, tw);
  if constexpr (MODE == COL_FWD_PROP_INV) {
    const int64_t pb = (o % a.comps) * a.prop_cstride + b * W + c;
#pragma unroll
    for (int j = 0; j < E; ++j)
      x[j] = mul_prop<T, PC128>(x[j], a.prop, pb + (int64_t)(t + j * TPL) * a.ld);
    fft_line<T, N, E, 1, true>(x, t, sm + c, W, tw);
  }
#pragma unroll
  for (int j = 0; j < E; ++j) base[(int64_t)(t + j * TPL) * a.ld] = x[j];
}

// Column pass over the blocked spectral buffer: CTA = one contiguous tile of
// W columns x N rows (N = NY); a.A is S, a.prop the blocked propagator,
// a.outer_stride the slab size NY*NX, a.ncb = NX / W.
template <typename T, int N, int E, int MODE, bool PC128>
__global__ void __launch_bounds__(BlkW<T>::W * (N / E)) k_cols_blk(const ColArgs a) {
  using C = cpx<T>;
  constexpr int TPL = N / E, W = BlkW<T>::W;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const int c = threadIdx.x % W, t = threadIdx.x / W;
  // tiles field-fastest: the fields of one column block run together, so its
  // propagator tile is read from HBM once and from L2 by the other fields
  const int64_t nouter = a.nblocks / a.ncb;
  const int64_t o = blockIdx.x % nouter, b = blockIdx.x / nouter;
  const int64_t toff = b * (int64_t)(N * W) + t * W + c;
  C* base = reinterpret_cast<C*>(a.A) + o * a.outer_stride + toff;
  C x[E];
#pragma unroll
  for (int j = 0; j < E; ++j) x[j] = base[j * TPL * W];
  fft_line<T, N, E, 1, MODE == COL_INV>(x, t, sm + c, W, tw);
  if constexpr (MODE == COL_FWD_PROP_INV) {
    const int64_t pb = (o % a.comps) * a.prop_cstride + toff;
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = mul_prop<T, PC128>(x[j], a.prop, pb + j * TPL * W);
    fft_line<T, N, E, 1, true>(x, t, sm + c, W, tw);
  }
#pragma unroll
  for (int j = 0; j < E; ++j) base[j * TPL * W] = x[j];
}

// Persistent column pass over the blocked spectral buffer with a two-stage
// bulk-copy ring: while a CTA transforms tile i from shared memory, the copy
// engine brings tile i + gridDim.x into the other stage.  Results go straight
// back to global memory (coalesced stores).  Same arithmetic as k_cols_blk.
constexpr int kColStages = 2;
constexpr size_t kMaxSmemBytes = 227 * 1024;  // dynamic shared memory a CTA may opt into

template <typename T, int N>
__host__ __device__ constexpr size_t cols_tma_base_smem() {
  // kColStages staging tiles and one exchange tile, each padded
  return (size_t)(kColStages + 1) * stage_len<T>(padded_len(N) * BlkW<T>::W) * sizeof(cpx<T>) +
         kColStages * sizeof(uint64_t);
}
// The column pass keeps its transform's twiddles in shared memory when they fit.
template <typename T, int N>
__host__ __device__ constexpr bool cols_tma_tws() {
  return cols_tma_base_smem<T, N>() + (size_t)tw_compact_len(N, Shape<N>::E) * sizeof(cpx<T>) + 16 <=
         kMaxSmemBytes;
}
template <typename T, int N>
__host__ __device__ constexpr size_t cols_tma_smem() {
  return cols_tma_base_smem<T, N>() +
         (cols_tma_tws<T, N>() ? (size_t)tw_compact_len(N, Shape<N>::E) * sizeof(cpx<T>) + 16 : 0);
}

template <typename T, int N, int E, bool PC128>
__global__ void __launch_bounds__(BlkW<T>::W * (N / E), 1) k_cols_blk_tma(const ColArgs a) {
  using C = cpx<T>;
  constexpr int TPL = N / E, W = BlkW<T>::W, TILE = N * W;
  constexpr int SLW = stage_len<T>(padded_len(N) * W);  // one padded tile, 128-byte multiple
  static_assert((SLW * sizeof(C)) % 128 == 0, "bulk copies need aligned shared destinations");
  constexpr unsigned TILE_BYTES = TILE * sizeof(C);
  // With an even number of exchanges per transform, the staging tile just
  // read into registers is the transforms' second exchange buffer and is
  // refilled after them; otherwise it is refilled at once.
  constexpr int NEX = fft_exchanges(N, E);
  constexpr bool DB = NEX > 0 && NEX % 2 == 0;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* stage = reinterpret_cast<C*>(smraw);
  C* xch = stage + kColStages * SLW;
  uint64_t* bar = reinterpret_cast<uint64_t*>(xch + SLW);
  // the transform's twiddles, copied once per CTA into shared memory when they fit
  constexpr bool TWS = cols_tma_tws<T, N>();
  C* twc = reinterpret_cast<C*>(reinterpret_cast<unsigned char*>(bar) + 16);
  if constexpr (TWS) load_tw_compact<T, N, E>(twc, reinterpret_cast<const C*>(a.tw));
  const C* tw = TWS ? twc : reinterpret_cast<const C*>(a.tw);
  C* S = reinterpret_cast<C*>(a.A);
  const int c = threadIdx.x % W, t = threadIdx.x / W;
  const int64_t ntiles = a.nblocks;
  // tile i = (column block b, slab o) with the slab fastest: the CTAs of one
  // wave transform the same column block of all fields, so each propagator
  // tile is fetched from HBM once and then served from L2
  const int64_t nouter = ntiles / a.ncb;
  auto tile_o = [&](int64_t i) { return i % nouter; };
  auto tile_b = [&](int64_t i) { return i / nouter; };
  auto tile_ptr = [&](int64_t i) { return S + tile_o(i) * a.outer_stride + tile_b(i) * TILE; };

  if (threadIdx.x == 0) {
    for (int st = 0; st < kColStages; ++st) mbar_init(&bar[st], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int st = 0; st < kColStages; ++st) {
      const int64_t i = blockIdx.x + (int64_t)st * gridDim.x;
      if (i < ntiles) {
        mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
        bulk_load(stage + st * SLW, tile_ptr(i), TILE_BYTES, &bar[st]);
      }
    }
  }
  auto refill = [&](int st, int64_t i) {
    const int64_t inext = i + (int64_t)kColStages * gridDim.x;
    if (inext < ntiles) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
      bulk_load(stage + st * SLW, tile_ptr(inext), TILE_BYTES, &bar[st]);
    }
  };
  int it = 0;
  for (int64_t i = blockIdx.x; i < ntiles; i += gridDim.x, ++it) {
    const int st = it % kColStages;
    const unsigned par = (it / kColStages) & 1;
    const bool ok = mbar_wait_bounded(&bar[st], par);
    if (!__syncthreads_and(ok)) {
      // give up: record it, let the copies in flight land (bounded), leave
      if (threadIdx.x == 0) {
        atomicExch(a.status, DEV_WAIT_TIMEOUT);
        mbar_wait_bounded(&bar[st], par);
        if (i + gridDim.x < ntiles)
          mbar_wait_bounded(&bar[st ^ 1], ((it + 1) / kColStages) & 1);
      }
      return;
    }
    C x[E];
    const C* sp = stage + st * SLW + t * W + c;
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = sp[j * TPL * W];
    const int64_t o = tile_o(i);
    const int64_t toff = tile_b(i) * (int64_t)TILE + t * W + c;
    const int64_t pb = (o % a.comps) * a.prop_cstride + toff;
    float2 pre[PC128 ? 1 : E];
    if constexpr (!PC128) {
      // propagator values (L2-resident) requested now, used after the forward FFT
#pragma unroll
      for (int j = 0; j < E; ++j) pre[j] = __ldg(reinterpret_cast<const float2*>(a.prop) + pb + j * TPL * W);
    }
    __syncthreads();  // every thread has read stage st
    C* sA = stage + st * SLW + c;
    if constexpr (DB) {
      fft_line_db<T, N, E, 1, false, 0, 1, TWS>(x, t, sA, xch + c, W, tw);
    } else {
      if (threadIdx.x == 0) refill(st, i);
      fft_line<T, N, E, 1, false, false, TWS>(x, t, xch + c, W, tw);
    }
    if constexpr (PC128) {
#pragma unroll
      for (int j = 0; j < E; ++j) x[j] = mul_prop<T, true>(x[j], a.prop, pb + j * TPL * W);
    } else {
#pragma unroll
      for (int j = 0; j < E; ++j) x[j] = cmul<T>(x[j], mk<T>(T(pre[j].x), T(pre[j].y)));
    }
    if constexpr (DB) {
      fft_line_db<T, N, E, 1, true, 0, 1, TWS>(x, t, sA, xch + c, W, tw);
      // the last exchange used xch, so every read of stage st is behind a barrier
      if (threadIdx.x == 0) refill(st, i);
    } else {
      fft_line<T, N, E, 1, true, false, TWS>(x, t, xch + c, W, tw);
    }
    C* g = S + o * a.outer_stride + toff;
#pragma unroll
    for (int j = 0; j < E; ++j) g[j * TPL * W] = x[j];
  }
}

// Natural [comps][NY][NX] propagator -> blocked layout with block width W.
// The copy carries the inverse 2-D transform's 1/(NY NX), a power of two:
// the scaling is exact, so the field after the inverse column and row
// transforms has the same bits as when the row pass scaled it, and the row
// passes that read the blocked buffer multiply by nothing.
template <typename TP>
__global__ void k_prop_to_blk(const cpx<TP>* __restrict__ nat, cpx<TP>* __restrict__ blk,
                              int64_t total, int64_t ny, int64_t nx, int w, TP scale) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pix = ny * nx;
    const int64_t comp = i / pix, r = i % pix;
    const int64_t bx = r / (ny * w), rem = r % (ny * w);
    const int64_t y = rem / w, c = rem % w;
    blk[i] = cscale<TP>(nat[comp * pix + y * nx + bx * w + c], scale);
  }
}

}  // namespace nlse
