// The nonlinear step of one pixel with the nonlocal intensities: |A|^2 of
// component 0 from the real part and of component 1 from the imaginary part of
// c, the convolved value of the padded scratch (NLSE/nlse.py:406-408, 444-447:
// nl_prop on the oaconvolve result), then Rabi coupling and the DDGPE source
// term as in the row passes.
#pragma once
#include "step_kernels.cuh"

namespace nlse {

template <typename T, int NC>
__device__ __forceinline__ void nl_pad_point(const StepArgs& a, int64_t f, int64_t pxl, cpx<T> c,
                                             int set) {
  cpx<T>* A = reinterpret_cast<cpx<T>*>(a.A);
  const bool has_v = a.flags & F_HAS_V;
  const T* P = param_block<T>(a) + f * kParamStride + set * 16;
  const int64_t i0 = (f * NC) * a.pix + pxl;
  NLP<T> p0 = load_nlp<T>(P);
  p0.dzi = param_block<T>(a)[f * kParamStride + 32 + set];
  const int64_t vi = f * a.v_fstride + pxl;
  const cpx<T> v0 = has_v ? load_vp<T>(a.V, a.flags, vi, p0.vs) : mk<T>(T(0), T(0));
  if constexpr (NC == 1) {
    if (a.flags & F_MAPS) apply_maps<T>(p0, a, f, pxl);
    A[i0] = nl_point<T, false>(A[i0], c.x, T(0), p0, has_v, v0);
  } else {
    const int64_t i1 = i0 + a.pix;
    NLP<T> p1 = load_nlp<T>(P + 7);
    p1.dzi = p0.dzi;
    const cpx<T> v1 = has_v ? load_vp<T>(a.V, a.flags, vi, p1.vs) : mk<T>(T(0), T(0));
    cpx<T> y0 = nl_point<T>(A[i0], c.x, c.y, p0, has_v, v0);
    cpx<T> y1 = nl_point<T>(A[i1], c.y, c.x, p1, has_v, v1);
    if (a.flags & F_RABI) {
      const T rc = P[14], rs = P[15], ric = P[34], ris = P[35];
      const cpx<T> z0 = rabi_rot<T>(y0, y1, rc, rs, ric, ris);
      const cpx<T> z1 = rabi_rot<T>(y1, y0, rc, rs, ric, ris);
      y0 = z0;
      y1 = z1;
    }
    if (a.flags & (F_PUMP | F_PROBE)) {
      const T* Pf = param_block<T>(a) + f * kParamStride;
      const T dz = Pf[30], dzi = Pf[31];
      if (a.flags & F_PUMP) {
        const cpx<T> u = pump_dz<T>(cmul<T>(reinterpret_cast<const cpx<T>*>(a.pump_r)[pxl],
                                            reinterpret_cast<const cpx<T>*>(a.pump_t)[a.step]),
                                    dz, dzi);
        y1 = mk<T>(y1.x + u.y, y1.y - u.x);
      }
      if (a.flags & F_PROBE) {
        const cpx<T> u = pump_dz<T>(cmul<T>(reinterpret_cast<const cpx<T>*>(a.probe_r)[pxl],
                                            reinterpret_cast<const cpx<T>*>(a.probe_t)[a.step]),
                                    dz, dzi);
        y1 = mk<T>(y1.x + u.y, y1.y - u.x);
      }
    }
    A[i0] = y0;
    A[i1] = y1;
  }
}

}  // namespace nlse
