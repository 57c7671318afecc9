// C ABI of libnlse_sm103: plans, the split-step sequence and CUDA-graph
// replay of the z-loop.  Declarations and contracts: include/nlse_gb300.h.
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "launch.h"
#include "nlse_gb300.h"

using namespace nlse;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(NLSE_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define NLSE_CUDA(call, what)                  \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// Per-pass twiddle tables (fft_core.cuh), one array per device and
// precision, computed in long double and rounded once.
constexpr int kMaxDevices = 64;
std::mutex g_tw_mu;
void* g_tw[kMaxDevices][2] = {};

int get_twiddles(int dev, int dtype, const void** out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(NLSE_ERR_UNSUPPORTED, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lk(g_tw_mu);
  if (!g_tw[dev][dtype]) {
    const long double pi = 3.141592653589793238462643383279502884L;
    std::vector<double> hd(2 * (size_t)kTwTableLen);
    for (int R = 2; R <= 16; R *= 2)
      for (int NS = 1; NS * R <= kTwMaxLen; NS *= 2)
        for (int r = 1; r < R; ++r)
          for (int k = 0; k < NS; ++k) {
            const size_t i = (size_t)tw_offset(R, NS) + (size_t)(r - 1) * NS + k;
            const long double ang = 2.0L * pi * (long double)(r * k) / (long double)(NS * R);
            hd[2 * i] = (double)cosl(ang);
            hd[2 * i + 1] = (double)(-sinl(ang));
          }
    void* d = nullptr;
    size_t bytes;
    if (dtype == NLSE_C64) {
      std::vector<float> hf(2 * (size_t)kTwTableLen);
      for (size_t i = 0; i < hf.size(); ++i) hf[i] = (float)hd[i];
      bytes = hf.size() * sizeof(float);
      NLSE_CUDA(cudaMalloc(&d, bytes), "cudaMalloc(twiddles)");
      NLSE_CUDA(cudaMemcpy(d, hf.data(), bytes, cudaMemcpyHostToDevice), "cudaMemcpy(twiddles)");
    } else {
      bytes = hd.size() * sizeof(double);
      NLSE_CUDA(cudaMalloc(&d, bytes), "cudaMalloc(twiddles)");
      NLSE_CUDA(cudaMemcpy(d, hd.data(), bytes, cudaMemcpyHostToDevice), "cudaMemcpy(twiddles)");
    }
    g_tw[dev][dtype] = d;
  }
  *out = g_tw[dev][dtype];
  return NLSE_OK;
}

// Tensor map of the blocked spectral buffer: dimensions (innermost first)
// {2W scalars, NY, NX/W, nfields*comps}, one-row boxes of up to 256 runs.
bool encode_tmap_S(CUtensorMap* tm, void* S, const nlse_desc& d, int64_t pix) {
  using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return false;
  const bool c64 = d.dtype == NLSE_C64;
  const int64_t w = c64 ? 4 : 2;
  const int64_t scalar = c64 ? 4 : 8;
  const int64_t nb = d.shape[1] / w;
  const cuuint64_t dims[4] = {(cuuint64_t)(2 * w), (cuuint64_t)d.shape[0], (cuuint64_t)nb,
                              (cuuint64_t)(d.nfields * d.comps)};
  const cuuint64_t strides[3] = {(cuuint64_t)(2 * w * scalar),
                                 (cuuint64_t)(2 * w * scalar * d.shape[0]),
                                 (cuuint64_t)(pix * 2 * scalar)};
  const cuuint32_t box[4] = {(cuuint32_t)(2 * w), 1, (cuuint32_t)(nb < 256 ? nb : 256), 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = reinterpret_cast<EncodeFn>(fn)(
      tm, c64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, S, dims,
      strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int ilog2_pow2(int64_t n) {
  if (n < 2 || (n & (n - 1))) return -1;
  int l = 0;
  while ((int64_t(1) << l) < n) ++l;
  return l;
}

struct GraphKey {
  void* A;
  nlse_operator op;
  int64_t nsteps, step0;
  uint64_t kgen;
  bool operator==(const GraphKey& o) const {
    return A == o.A && nsteps == o.nsteps && step0 == o.step0 && kgen == o.kgen &&
           std::memcmp(&op, &o.op, sizeof(op)) == 0;
  }
};

}  // namespace

// Entry points shared with the other translation units of the library.
namespace nlse {
int shared_twiddles(int dev, int dtype, const void** out) { return get_twiddles(dev, dtype, out); }
int shared_fail(int code, const char* msg) { return fail(code, "%s", msg); }
int shared_cuda_fail(cudaError_t e, const char* what) { return cuda_fail(e, what); }
void shared_clear_error() { g_err.clear(); }
}  // namespace nlse

struct nlse_plan_s {
  nlse_desc d;
  int dev = 0;
  const void* tw = nullptr;
  int lg[3] = {0, 0, 0};
  int64_t pix = 0;  // pixels of one component of one field
  cudaStream_t cap = nullptr;  // private stream used only for graph capture
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t glaunched = nullptr;  // recorded after each launch of gexec
  GraphKey gkey;
  bool gvalid = false;
  // 2-D fast path: spectral scratch in the blocked layout and the
  // propagator converted to that layout (cached by pointer and format)
  bool blk = false;
  void* S = nullptr;
  void* prop_blk = nullptr;
  const void* prop_src = nullptr;
  int prop_src_c128 = -1;
  int64_t prop_src_cstride = -1;
  int64_t prop_src_version = -1;
  float* params_f32 = nullptr;  // FP32 mirror of the caller's parameter block
  bool fft_ok = true;           // all axes are supported transform lengths
  int* status = nullptr;        // device status word: DEV_* codes from bounded waits
  int nsm = 0;                  // multiprocessors (persistent grids)
  bool cols_tma = true;         // use the TMA-ring column pass where it fits
  bool rows_tma = false;        // use the TMA-fed inverse row passes
  bool cols_tma_ok = true;      // the TMA column pass is available (not disabled)
  bool rows_tma_ok = false;     // tensor map of S encoded: the TMA row passes are available
  int rows_var = NLSE_ROWS_LINE;  // inverse row pass variant (NLSE_ROWS_*)
  int cols_var = NLSE_COLS_TILE;  // column pass variant (NLSE_COLS_*)
  int rows_cap = 0, cols_cap = 0; // CTAs per SM of the persistent passes (0: all that fit)
  uint32_t rows_avail = 1u << NLSE_ROWS_LINE, cols_avail = 1u << NLSE_COLS_TILE;
  uint64_t kgen = 0;            // kernel-variant generation (part of every graph key)
  CUtensorMap tmS;              // S as {2W scalars, NY, NX/W, slabs}, box = one row (<= 256 runs)
  // nonlocal response: zero-padded grid (py x px), its scratch and FFT plan
  int64_t nl_py = 0, nl_px = 0;
  void* X = nullptr;
  nlse_plan_s* nlsub = nullptr;
};

namespace {

// The pair row pass serves this launch: complex64 one-component field on
// the blocked buffer through the tensor map, no Rabi, pump or external |A|^2.
bool rows_pair_fits(const nlse_plan_s* p, int mode, const StepArgs& a) {
  return (p->rows_var == NLSE_ROWS_PAIR || p->rows_var == NLSE_ROWS_PAIR8 ||
          p->rows_var == NLSE_ROWS_DEEP) &&
         p->d.dtype == NLSE_C64 && a.comps == 1 &&
         (mode == ROW_INV_NL || mode == ROW_INV_NL_FWD) && (a.flags & F_IN_BLK) && a.tmap &&
         a.tma_grid > 0 && !(a.flags & (F_RABI | F_PUMP | F_PROBE | F_ASQ_EXT)) &&
         (!(a.flags & F_HAS_V) || (a.flags & F_V_F32)) && a.nq % 2 == 0 &&
         a.nq < (int64_t(1) << 31);
}

cudaError_t rows(const nlse_plan_s* p, int mode, int log2n, const StepArgs& a, cudaStream_t s,
                 bool prep = false) {
  if (prep && p->d.dtype == NLSE_C64 && a.comps == 1 &&
      (mode == ROW_INV_NL || mode == ROW_INV_NL_FWD) && (p->rows_avail >> NLSE_ROWS_PAIR & 1)) {
    for (int form : {16, 8, 0}) {
      const cudaError_t e = launch_rows_pair(mode, log2n, a, false, s, true, 0, form ? form : 16,
                                             form == 0);
      if (e != cudaSuccess && e != cudaErrorNotSupported) return e;
    }
  }
  if (!prep && rows_pair_fits(p, mode, a)) {
    // the potential row is shared by both lines of every pair when one real
    // potential serves an even number of fields (lines are field-fastest)
    const bool vshared = (a.flags & F_HAS_V) && !(a.flags & F_V_COMPLEX) && a.v_fstride == 0 &&
                         p->d.nfields % 2 == 0;
    const int ep = p->rows_var == NLSE_ROWS_PAIR8 ? 8 : 16;
    const cudaError_t e = launch_rows_pair(mode, log2n, a, vshared, s, false, p->rows_cap, ep,
                                           p->rows_var == NLSE_ROWS_DEEP);
    if (e != cudaErrorNotSupported) return e;
  }
  if (p->d.dtype == NLSE_C64)
    return a.comps == 1 ? launch_rows_f32_c1(mode, log2n, a, s, prep)
                        : launch_rows_f32_c2(mode, log2n, a, s, prep);
  return a.comps == 1 ? launch_rows_f64_c1(mode, log2n, a, s, prep)
                      : launch_rows_f64_c2(mode, log2n, a, s, prep);
}

cudaError_t cols(const nlse_plan_s* p, int mode, int log2n, const ColArgs& a, cudaStream_t s,
                 bool prep = false) {
  if (p->d.dtype == NLSE_C64) return launch_cols_f32(mode, log2n, a, s, prep);
  return launch_cols_f64(mode, log2n, a, s, prep);
}

cudaError_t cols_blk(const nlse_plan_s* p, int mode, int log2n, const ColArgs& a, cudaStream_t s,
                     bool prep = false) {
  if (p->d.dtype == NLSE_C64 && mode == COL_FWD_PROP_INV) {
    if (prep && (p->cols_avail >> NLSE_COLS_PAIR & 1)) {
      for (int form : {16, 8, 0}) {
        const cudaError_t e = launch_cols_pair(log2n, a, s, true, 0, form ? form : 16, form == 0);
        if (e != cudaSuccess && e != cudaErrorNotSupported) return e;
      }
    }
    if (!prep &&
        (p->cols_var == NLSE_COLS_PAIR || p->cols_var == NLSE_COLS_PAIR8 ||
         p->cols_var == NLSE_COLS_DEEP) &&
        a.tma_grid > 0 && !(a.flags & F_PROP_C128)) {
      const int ep = p->cols_var == NLSE_COLS_PAIR8 ? 8 : 16;
      const cudaError_t e = launch_cols_pair(log2n, a, s, false, p->cols_cap, ep,
                                             p->cols_var == NLSE_COLS_DEEP);
      if (e != cudaErrorNotSupported) return e;
    }
  }
  if (p->d.dtype == NLSE_C64) return launch_cols_blk_f32(mode, log2n, a, s, prep);
  return launch_cols_blk_f64(mode, log2n, a, s, prep);
}

int blk_width(const nlse_plan_s* p) { return p->d.dtype == NLSE_C64 ? 4 : 2; }

// Whether a 2-D plan can use the blocked spectral layout: the row pass needs
// its threads-per-line (NX/16) and NX to be multiples of the block width,
// the column pass at most 1024 threads (W * NY/16).
bool blocked_ok(const nlse_desc& d) {
  if (d.ndim != 2) return false;
  const int64_t w = d.dtype == NLSE_C64 ? 4 : 2;
  const int64_t nx = d.shape[1], ny = d.shape[0];
  if (nx < 16 || ny < 16) return false;
  if ((nx / 16) % w != 0) return false;
  return w * (ny / 16) <= 1024;
}

// Column-pass arguments over the blocked spectral buffer.
ColArgs col_blk_args(const nlse_plan_s* p, const nlse_operator* op) {
  const nlse_desc& d = p->d;
  ColArgs c{};
  c.A = p->S;
  c.tw = p->tw;
  c.prop = p->prop_blk;
  c.prop_cstride = op && op->prop_cstride ? p->pix : 0;
  c.flags = (op && op->prop_c128) ? F_PROP_C128 : 0u;
  c.comps = d.comps;
  c.w = blk_width(p);
  c.ld = c.w;
  c.outer_stride = p->pix;
  c.ncb = d.shape[1] / c.w;
  c.nblocks = c.ncb * d.nfields * d.comps;
  c.status = p->status;
  c.tma_grid = p->cols_tma ? p->nsm : 0;
  c.cap_per_sm = p->cols_cap;
  return c;
}

// Convert op->prop to the blocked layout unless the cached copy is current.
int refresh_prop(nlse_plan_s* p, const nlse_operator* op, bool force, cudaStream_t s) {
  if (!force && p->prop_src == op->prop && p->prop_src_c128 == op->prop_c128 &&
      p->prop_src_cstride == op->prop_cstride && p->prop_src_version == op->prop_version)
    return NLSE_OK;
  const int64_t comps = op->prop_cstride ? p->d.comps : 1;
  cudaError_t e = launch_prop_to_blk(op->prop_c128, op->prop, p->prop_blk, comps, p->d.shape[0],
                                     p->d.shape[1], blk_width(p), s);
  if (e != cudaSuccess) return cuda_fail(e, "propagator layout");
  p->prop_src = op->prop;
  p->prop_src_c128 = op->prop_c128;
  p->prop_src_cstride = op->prop_cstride;
  p->prop_src_version = op->prop_version;
  return NLSE_OK;
}

// Columns per column-pass CTA: 64-byte row segments, bounded by the thread
// budget of one CTA and by the contiguous extent available.
int pick_w(const nlse_plan_s* p, int log2n, int64_t inner) {
  const int tpl = (1 << log2n) >= 16 ? (1 << log2n) / 16 : 1;
  int w = p->d.dtype == NLSE_C64 ? 8 : 4;
  while (w > 1 && (w * tpl > kColMaxThreads || w > inner || inner % w)) w >>= 1;
  return w;
}

// Column-pass arguments for axis `axis` (0 = outermost transform axis) of an
// ndim-D field.
ColArgs col_args(const nlse_plan_s* p, void* A, const nlse_operator* op, int axis) {
  const nlse_desc& d = p->d;
  ColArgs c{};
  c.A = A;
  c.tw = p->tw;
  c.prop = op ? op->prop : nullptr;
  c.prop_cstride = op ? op->prop_cstride : 0;
  c.flags = (op && op->prop_c128) ? F_PROP_C128 : 0u;
  c.comps = d.comps;
  int64_t inner = 1;
  for (int k = axis + 1; k < d.ndim; ++k) inner *= d.shape[k];
  const int64_t n = d.shape[axis];
  int64_t outer = d.nfields * d.comps;
  for (int k = 0; k < axis; ++k) outer *= d.shape[k];
  c.w = pick_w(p, p->lg[axis], inner);
  c.ld = inner;
  c.outer_stride = n * inner;
  c.ncb = inner / c.w;
  c.nblocks = c.ncb * outer;
  return c;
}

StepArgs row_args(const nlse_plan_s* p, void* A, const nlse_operator* op) {
  const nlse_desc& d = p->d;
  StepArgs a{};
  a.A = A;
  a.S = p->S;
  a.tw = p->tw;
  a.params_f32 = p->params_f32;
  a.status = p->status;
  a.tma_grid = p->rows_tma ? p->nsm : 0;
  a.tmap = p->rows_tma ? &p->tmS : nullptr;
  a.cap_per_sm = p->rows_cap;
  const int64_t n = d.shape[d.ndim - 1];
  a.lines_per_comp = p->pix / n;
  a.nq = d.nfields * a.lines_per_comp;
  a.pix = p->pix;
  a.inv_n = 1.0 / (double)p->pix;
  a.inv_nf = (float)a.inv_n;
  a.comps = d.comps;
  a.nsteps = 1;
  if (op) {
    a.V = op->V;
    a.prop = op->prop;
    a.params = op->params;
    a.pump_r = op->pump_r;
    a.pump_t = op->pump_t;
    a.probe_r = op->probe_r;
    a.probe_t = op->probe_t;
    a.v_fstride = op->v_fstride;
    a.prop_cstride = op->prop_cstride;
    uint32_t f = 0;
    if (op->V) f |= F_HAS_V;
    if (op->v_complex) f |= F_V_COMPLEX;
    if (op->v_f32) f |= F_V_F32;
    if (op->prop_c128) f |= F_PROP_C128;
    if (op->rabi && d.comps == 2 && op->scheme == 0) f |= F_RABI;
    if (op->pump_r && d.comps == 2) f |= F_PUMP;
    if (op->probe_r && d.comps == 2) f |= F_PROBE;
    if (op->nl_maps && op->maps_mask) {
      f |= F_MAPS;
      a.maps = op->nl_maps;
      a.maps_fstride = op->maps_fstride;
      a.maps_plane = op->maps_plane;
      a.maps_mask = op->maps_mask;
    }
    a.flags = f;
  }
  return a;
}

int check_op(const nlse_plan_s* p, const nlse_operator* op) {
  if (!op) return fail(NLSE_ERR_ARG, "operator is NULL");
  if (!op->prop) return fail(NLSE_ERR_ARG, "propagator is NULL");
  if (!op->params) return fail(NLSE_ERR_ARG, "parameter block is NULL");
  if (op->scheme != 0 && op->scheme != 1) return fail(NLSE_ERR_ARG, "scheme must be 0 or 1");
  if (p->d.dtype == NLSE_C64 && op->V && !op->v_f32)
    return fail(NLSE_ERR_ARG, "a complex64 field needs a single-precision potential");
  if ((op->pump_r && !op->pump_t) || (op->probe_r && !op->probe_t))
    return fail(NLSE_ERR_ARG, "pump/probe spatial profile given without time profile");
  if ((op->pump_r || op->probe_r) && (p->d.comps != 2 || p->d.ndim != 2))
    return fail(NLSE_ERR_UNSUPPORTED, "pump/probe terms need a two-component 2-D field");
  if (op->nl_maps && op->maps_mask) {
    if (p->d.comps != 1)
      return fail(NLSE_ERR_UNSUPPORTED, "coefficient maps are for one-component fields");
    if ((op->maps_mask & ~7) || op->maps_fstride < 0 || op->maps_plane < p->pix ||
        (op->maps_fstride && op->maps_plane < op->maps_fstride * p->d.nfields))
      return fail(NLSE_ERR_ARG, "coefficient maps: mask bits 0..2, plane of at least the "
                  "maps' elements");
  }
  return NLSE_OK;
}

// One pass of the step sequence (see nlse_pass).
int mirror_params(nlse_plan_s* p, const nlse_operator* op, cudaStream_t s) {
  if (p->d.dtype != NLSE_C64) return NLSE_OK;
  cudaError_t e = launch_params_f32(op->params, p->params_f32, p->d.nfields * kParamStride, s);
  if (e != cudaSuccess) return cuda_fail(e, "parameter mirror");
  return NLSE_OK;
}

int enqueue_pass(nlse_plan_s* p, void* A, const nlse_operator* op, int pass, int64_t step,
                 cudaStream_t s) {
  const nlse_desc& d = p->d;
  if (d.ndim == 1) return fail(NLSE_ERR_UNSUPPORTED, "1-D plans have a single fused pass");
  if (pass != NLSE_PASS_LINEAR) {
    const int rc = mirror_params(p, op, s);
    if (rc != NLSE_OK) return rc;
  }
  StepArgs a = row_args(p, A, op);
  const uint32_t pre = op->scheme == 1 ? F_PRE_NL : 0u;
  const int rl = p->lg[d.ndim - 1];
  a.step = (int)step;
  cudaError_t e = cudaSuccess;
  if (p->blk) {
    switch (pass) {
      case NLSE_PASS_FORWARD:
        a.flags |= pre | F_OUT_BLK;
        e = rows(p, ROW_FWD, rl, a, s);
        break;
      case NLSE_PASS_LINEAR: {
        const int rc = refresh_prop(p, op, false, s);
        if (rc != NLSE_OK) return rc;
        e = cols_blk(p, COL_FWD_PROP_INV, p->lg[0], col_blk_args(p, op), s);
        break;
      }
      case NLSE_PASS_INV_NL_FWD:
        a.flags |= pre | F_IN_BLK | F_OUT_BLK;
        e = rows(p, ROW_INV_NL_FWD, rl, a, s);
        break;
      case NLSE_PASS_INV_NL:
        a.flags |= F_IN_BLK;
        e = rows(p, ROW_INV_NL, rl, a, s);
        break;
      default:
        return fail(NLSE_ERR_ARG, "unknown pass %d", pass);
    }
    if (e != cudaSuccess) return cuda_fail(e, "pass");
    return NLSE_OK;
  }
  switch (pass) {
    case NLSE_PASS_FORWARD:
      a.flags |= pre;
      e = rows(p, ROW_FWD, rl, a, s);
      break;
    case NLSE_PASS_LINEAR:
      if (d.ndim == 2) {
        e = cols(p, COL_FWD_PROP_INV, p->lg[0], col_args(p, A, op, 0), s);
      } else {
        const ColArgs cx = col_args(p, A, op, 1);
        e = cols(p, COL_FWD, p->lg[1], cx, s);
        if (e == cudaSuccess) e = cols(p, COL_FWD_PROP_INV, p->lg[0], col_args(p, A, op, 0), s);
        if (e == cudaSuccess) e = cols(p, COL_INV, p->lg[1], cx, s);
      }
      break;
    case NLSE_PASS_INV_NL_FWD:
      a.flags |= pre;
      e = rows(p, ROW_INV_NL_FWD, rl, a, s);
      break;
    case NLSE_PASS_INV_NL:
      e = rows(p, ROW_INV_NL, rl, a, s);
      break;
    default:
      return fail(NLSE_ERR_ARG, "unknown pass %d", pass);
  }
  if (e != cudaSuccess) return cuda_fail(e, "pass");
  return NLSE_OK;
}

int fft_sub(nlse_plan_s* q, void* X, int inverse, cudaStream_t s);

// Nonlocal nonlinear step (parameter set `set`): pack |A|^2 into the padded
// scratch, convolve by the kernel spectrum on the project FFT, apply the
// pointwise step with the convolved intensities.
int conv_nl(nlse_plan_s* p, void* A, const nlse_operator* op, int set, int64_t step,
            cudaStream_t s) {
  const nlse_desc& d = p->d;
  const int64_t ny = d.ndim == 2 ? d.shape[0] : 1, nx = d.shape[d.ndim - 1];
  const int64_t py = d.ndim == 2 ? p->nl_py : 1, px = p->nl_px;
  const nlse_plan_s* q = p->nlsub;
  if (d.ndim == 2 && nonlocal_rows_fused(d.dtype, q->lg[1], ny, py)) {
    // |A|^2 packed inside the forward row pass; the spectrum multiply inside
    // the column pass; the nonlinear step inside the inverse row pass of the
    // field's rows
    cudaError_t e = launch_pack_rows_fwd(q->lg[1], d.comps, A, p->X, d.nfields, ny, nx, py, q->tw, s);
    if (e == cudaSuccess) {
      ColArgs ca = col_args(q, p->X, nullptr, 0);
      ca.prop = op->nl_khat;
      ca.prop_cstride = 0;
      ca.flags = 0u;
      e = cols(q, COL_FWD_PROP_INV, q->lg[0], ca, s);
    }
    if (e == cudaSuccess) {
      StepArgs a = row_args(p, A, op);
      a.step = (int)step;
      if (set == 1) a.flags &= ~(F_RABI | F_PUMP | F_PROBE);
      e = launch_rows_inv_nl_pad(q->lg[1], a, p->X, ny, nx, py, set,
                                 (float)(1.0 / ((double)py * (double)px)), s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "nonlocal convolution and nonlinear step");
    return NLSE_OK;
  }
  cudaError_t e = launch_pack_asq(d.dtype, d.comps, A, p->X, d.nfields, ny, nx, py, px, s);
  if (e != cudaSuccess) return cuda_fail(e, "nonlocal pack");
  if (d.ndim == 2) {
    // forward rows; one column pass: forward transform, times the kernel
    // spectrum (as a propagator), inverse transform; inverse rows with the
    // 2-D transform's 1/N (the products and their rounding are those of the
    // separate passes and spectrum multiply)
    StepArgs ra = row_args(q, p->X, nullptr);
    ra.flags = F_NO_POST;
    const int rl = q->lg[1];
    e = rows(q, ROW_FWD, rl, ra, s);
    if (e == cudaSuccess) {
      ColArgs ca = col_args(q, p->X, nullptr, 0);
      ca.prop = op->nl_khat;
      ca.prop_cstride = 0;
      ca.flags = d.dtype == NLSE_C128 ? F_PROP_C128 : 0u;
      e = cols(q, COL_FWD_PROP_INV, q->lg[0], ca, s);
    }
    if (e == cudaSuccess) e = rows(q, ROW_INV, rl, ra, s);
    if (e != cudaSuccess) return cuda_fail(e, "nonlocal convolution");
  } else {
    int rc = fft_sub(p->nlsub, p->X, 0, s);
    if (rc != NLSE_OK) return rc;
    e = launch_mul_spectrum(d.dtype, p->X, op->nl_khat, py * px, d.nfields * py * px, s);
    if (e != cudaSuccess) return cuda_fail(e, "nonlocal spectrum");
    rc = fft_sub(p->nlsub, p->X, 1, s);
    if (rc != NLSE_OK) return rc;
  }
  StepArgs a = row_args(p, A, op);
  a.step = (int)step;
  if (set == 1) a.flags &= ~(F_RABI | F_PUMP | F_PROBE);
  e = launch_nl_pointwise_pad(d.dtype, a, p->X, ny, nx, py, px, set, s);
  if (e != cudaSuccess) return cuda_fail(e, "nonlocal nonlinear step");
  return NLSE_OK;
}

// Split steps with the nonlocal response (no cross-step fusion: each
// nonlinear step needs the convolution of the real-space intensity).
int enqueue_steps_nonlocal(nlse_plan_s* p, void* A, const nlse_operator* op, int64_t nsteps,
                           int64_t step0, cudaStream_t s) {
  const nlse_desc& d = p->d;
  if (!p->X) return fail(NLSE_ERR_STATE, "nonlocal kernel given but nlse_plan_set_nonlocal not called");
  if (d.ndim == 3) return fail(NLSE_ERR_UNSUPPORTED, "nonlocal response of 3-D fields");
  const int mrc = mirror_params(p, op, s);
  if (mrc != NLSE_OK) return mrc;
  const int rl = p->lg[d.ndim - 1];
  cudaError_t e;
  for (int64_t st = 0; st < nsteps; ++st) {
    if (op->scheme == 1) {
      const int rc = conv_nl(p, A, op, 1, step0 + st, s);
      if (rc != NLSE_OK) return rc;
    }
    StepArgs a = row_args(p, A, op);
    a.flags &= ~(F_PRE_NL);
    if (d.ndim == 1) {
      a.flags |= F_NO_POST;
      a.nsteps = 1;
      e = rows(p, ROW_FULL, rl, a, s);
      if (e != cudaSuccess) return cuda_fail(e, "row pass (1-D linear step)");
    } else if (p->blk) {
      const int rc = refresh_prop(p, op, false, s);
      if (rc != NLSE_OK) return rc;
      StepArgs a0 = a;
      a0.flags |= F_OUT_BLK;
      e = rows(p, ROW_FWD, rl, a0, s);
      if (e == cudaSuccess) e = cols_blk(p, COL_FWD_PROP_INV, p->lg[0], col_blk_args(p, op), s);
      StepArgs a1 = a;
      a1.flags |= F_IN_BLK | F_NO_POST;
      if (e == cudaSuccess) e = rows(p, ROW_INV_NL, rl, a1, s);
      if (e != cudaSuccess) return cuda_fail(e, "linear step");
    } else {
      e = rows(p, ROW_FWD, rl, a, s);
      if (e == cudaSuccess) e = cols(p, COL_FWD_PROP_INV, p->lg[0], col_args(p, A, op, 0), s);
      StepArgs a1 = a;
      a1.flags |= F_NO_POST;
      if (e == cudaSuccess) e = rows(p, ROW_INV_NL, rl, a1, s);
      if (e != cudaSuccess) return cuda_fail(e, "linear step");
    }
    const int rc = conv_nl(p, A, op, 0, step0 + st, s);
    if (rc != NLSE_OK) return rc;
  }
  return NLSE_OK;
}

// Enqueue nsteps split steps (no capture handling here).
int enqueue_steps(nlse_plan_s* p, void* A, const nlse_operator* op, int64_t nsteps, int64_t step0,
                  cudaStream_t s) {
  const nlse_desc& d = p->d;
  if (nsteps <= 0) return NLSE_OK;
  if (op->nl_khat) return enqueue_steps_nonlocal(p, A, op, nsteps, step0, s);
  const int mrc = mirror_params(p, op, s);
  if (mrc != NLSE_OK) return mrc;
  StepArgs a = row_args(p, A, op);
  const uint32_t pre = op->scheme == 1 ? F_PRE_NL : 0u;
  const int rl = p->lg[d.ndim - 1];
  cudaError_t e;
  if (d.ndim == 1) {
    a.flags |= pre;
    if (a.flags & (F_PUMP | F_PROBE)) return fail(NLSE_ERR_UNSUPPORTED, "pump in 1-D");
    a.nsteps = (int)nsteps;
    a.step = (int)step0;
    e = rows(p, ROW_FULL, rl, a, s);
    if (e != cudaSuccess) return cuda_fail(e, "row pass (1-D full step)");
    return NLSE_OK;
  }
  if (p->blk) {
    // A (natural) -> S (blocked): forward rows; S: columns; S -> S: inverse
    // rows + nonlinear + next forward rows; S -> A: last inverse rows.
    int rc = refresh_prop(p, op, false, s);
    if (rc != NLSE_OK) return rc;
    const ColArgs c = col_blk_args(p, op);
    StepArgs a0 = a;
    a0.flags |= pre | F_OUT_BLK;
    e = rows(p, ROW_FWD, rl, a0, s);
    if (e != cudaSuccess) return cuda_fail(e, "row pass (forward)");
    for (int64_t st = 0; st < nsteps; ++st) {
      e = cols_blk(p, COL_FWD_PROP_INV, p->lg[0], c, s);
      if (e != cudaSuccess) return cuda_fail(e, "column pass (linear step)");
      StepArgs ai = a;
      ai.step = (int)(step0 + st);
      if (st + 1 < nsteps) {
        ai.flags |= pre | F_IN_BLK | F_OUT_BLK;
        e = rows(p, ROW_INV_NL_FWD, rl, ai, s);
      } else {
        ai.flags |= F_IN_BLK;
        e = rows(p, ROW_INV_NL, rl, ai, s);
      }
      if (e != cudaSuccess) return cuda_fail(e, "row pass (inverse + nonlinear)");
    }
    return NLSE_OK;
  }
  // first forward row pass, with the step's leading half nonlinear step
  StepArgs a0 = a;
  a0.flags |= pre;
  e = rows(p, ROW_FWD, rl, a0, s);
  if (e != cudaSuccess) return cuda_fail(e, "row pass (forward)");
  for (int64_t st = 0; st < nsteps; ++st) {
    if (d.ndim == 2) {
      const ColArgs c = col_args(p, A, op, 0);
      e = cols(p, COL_FWD_PROP_INV, p->lg[0], c, s);
      if (e != cudaSuccess) return cuda_fail(e, "column pass (linear step)");
    } else {
      const ColArgs cx = col_args(p, A, op, 1);
      const ColArgs cy = col_args(p, A, op, 0);
      e = cols(p, COL_FWD, p->lg[1], cx, s);
      if (e == cudaSuccess) e = cols(p, COL_FWD_PROP_INV, p->lg[0], cy, s);
      if (e == cudaSuccess) e = cols(p, COL_INV, p->lg[1], cx, s);
      if (e != cudaSuccess) return cuda_fail(e, "column pass (3-D linear step)");
    }
    StepArgs ai = a;
    ai.step = (int)(step0 + st);
    if (st + 1 < nsteps) {
      ai.flags |= pre;
      e = rows(p, ROW_INV_NL_FWD, rl, ai, s);
    } else {
      e = rows(p, ROW_INV_NL, rl, ai, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "row pass (inverse + nonlinear)");
  }
  return NLSE_OK;
}

// Raise the dynamic shared-memory limit of every kernel the plan can launch
// (outside any stream capture).
int prepare_kernels(nlse_plan_s* p) {
  StepArgs a = row_args(p, nullptr, nullptr);
  for (int nc = 1; nc <= p->d.comps; ++nc) {
    a.comps = nc;
    for (int m : {ROW_FWD, ROW_INV_NL, ROW_INV_NL_FWD, ROW_FULL, ROW_INV}) {
      if (m == ROW_INV && nc == 2) continue;
      cudaError_t e = rows(p, m, p->lg[p->d.ndim - 1], a, nullptr, true);
      if (e != cudaSuccess) return cuda_fail(e, "kernel attributes (rows)");
    }
  }
  if (p->blk) {
    ColArgs c{};
    cudaError_t e = cols_blk(p, COL_FWD_PROP_INV, p->lg[0], c, nullptr, true);
    if (e != cudaSuccess) return cuda_fail(e, "kernel attributes (blocked columns)");
  }
  for (int ax = 0; ax + 1 < p->d.ndim; ++ax) {
    ColArgs c{};
    for (int m : {COL_FWD, COL_INV, COL_FWD_PROP_INV}) {
      cudaError_t e = cols(p, m, p->lg[ax], c, nullptr, true);
      if (e != cudaSuccess) return cuda_fail(e, "kernel attributes (columns)");
    }
  }
  return NLSE_OK;
}

}  // namespace

extern "C" {

int nlse_abi_version(void) { return NLSE_ABI_VERSION; }

const char* nlse_last_error(void) { return g_err.c_str(); }

int nlse_plan_create(nlse_plan* out, const nlse_desc* desc) {
  g_err.clear();
  if (!out || !desc) return fail(NLSE_ERR_ARG, "null argument");
  *out = nullptr;
  const nlse_desc& d = *desc;
  if (d.ndim < 1 || d.ndim > 3) return fail(NLSE_ERR_ARG, "ndim must be 1, 2 or 3 (got %d)", d.ndim);
  if (d.dtype != NLSE_C64 && d.dtype != NLSE_C128) return fail(NLSE_ERR_ARG, "dtype %d", d.dtype);
  if (d.comps != 1 && d.comps != 2) return fail(NLSE_ERR_ARG, "comps must be 1 or 2");
  if (d.ndim == 3 && d.comps != 1)
    return fail(NLSE_ERR_UNSUPPORTED, "3-D fields have one component");
  if (d.nfields < 1) return fail(NLSE_ERR_ARG, "nfields must be >= 1");
  auto* p = new nlse_plan_s();
  p->d = d;
  p->pix = 1;
  for (int k = 0; k < d.ndim; ++k) {
    if (d.shape[k] < 1) {
      delete p;
      return fail(NLSE_ERR_ARG, "axis %d has length %lld", k, (long long)d.shape[k]);
    }
    const int l = ilog2_pow2(d.shape[k]);
    if (l < kMinLog2 || l > kMaxLog2) p->fft_ok = false;  // pointwise entry points only
    p->lg[k] = l;
    p->pix *= d.shape[k];
  }
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "cudaGetDevice");
  }
  int rc = get_twiddles(p->dev, d.dtype, &p->tw);
  p->blk = p->fft_ok && blocked_ok(d);
  if (rc == NLSE_OK) {
    e = cudaMalloc(&p->params_f32, (size_t)d.nfields * kParamStride * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p->status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->status, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, p->dev);
    if (e != cudaSuccess) rc = cuda_fail(e, "plan buffers");
    const char* env = getenv("NLSE_COLS_TMA");
    if (env && env[0] == '0') p->cols_tma = p->cols_tma_ok = false;
  }
  if (rc == NLSE_OK && p->blk) {
    const size_t es = d.dtype == NLSE_C64 ? 8 : 16;
    e = cudaMalloc(&p->S, (size_t)d.nfields * d.comps * p->pix * es);
    if (e == cudaSuccess) e = cudaMalloc(&p->prop_blk, (size_t)d.comps * p->pix * 16);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(spectral scratch)");
    const char* env = getenv("NLSE_ROWS_TMA");
    const bool want = !(env && env[0] == '0');
    const int64_t nb = d.shape[1] / blk_width(p);
    if (rc == NLSE_OK && want && (nb <= 256 || nb % 256 == 0) && d.nfields * d.comps < (1ll << 31))
      p->rows_tma = p->rows_tma_ok = encode_tmap_S(&p->tmS, p->S, d, p->pix);
    // variants: TMA row passes with the tensor map; pair passes (packed FP32,
    // two lines per thread) for one-component complex64 fields of 64 to 4096
    // points per row and 64 to 2048 per column, unless NLSE_PAIR=0
    const char* penv = getenv("NLSE_PAIR");
    const bool pair = !(penv && penv[0] == '0') && d.dtype == NLSE_C64 && d.comps == 1;
    if (p->rows_tma_ok) p->rows_avail |= 1u << NLSE_ROWS_TMA;
    if (p->rows_tma_ok && pair && p->lg[1] >= 6 && p->lg[1] <= 12)
      p->rows_avail |= (1u << NLSE_ROWS_PAIR) | (1u << NLSE_ROWS_PAIR8) | (1u << NLSE_ROWS_DEEP);
    if (p->cols_tma_ok) p->cols_avail |= 1u << NLSE_COLS_TMA;
    if (p->cols_tma_ok && pair && p->lg[0] >= 6 && p->lg[0] <= 11)
      p->cols_avail |= (1u << NLSE_COLS_PAIR) | (1u << NLSE_COLS_PAIR8) | (1u << NLSE_COLS_DEEP);
    p->rows_var = p->rows_tma ? NLSE_ROWS_TMA : NLSE_ROWS_LINE;
    // complex64 one-component plans: the tile column pass (fastest measured on
    // the 2048^2 batch); others keep the TMA ring where it fits
    if (d.dtype == NLSE_C64 && d.comps == 1) p->cols_tma = false;
    p->cols_var = p->cols_tma ? NLSE_COLS_TMA : NLSE_COLS_TILE;
  }
  if (rc == NLSE_OK && p->fft_ok) rc = prepare_kernels(p);
  if (rc == NLSE_OK) {
    e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
  }
  if (rc != NLSE_OK) {
    nlse_plan_destroy(p);
    return rc;
  }
  *out = p;
  return NLSE_OK;
}

int nlse_plan_destroy(nlse_plan p) {
  if (!p) return NLSE_OK;
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  if (p->glaunched) cudaEventDestroy(p->glaunched);
  if (p->cap) cudaStreamDestroy(p->cap);
  if (p->S) cudaFree(p->S);
  if (p->prop_blk) cudaFree(p->prop_blk);
  if (p->params_f32) cudaFree(p->params_f32);
  if (p->status) cudaFree(p->status);
  if (p->X) cudaFree(p->X);
  if (p->nlsub) nlse_plan_destroy(p->nlsub);
  delete p;
  return NLSE_OK;
}

}  // extern "C"

namespace {

// Whether a group runs as one launch per pass per step (step_multi.cuh):
// complex64 one-component 2-D plans of 256..2048 points per axis with the TMA
// row pass, the same number of steps, no nonlocal response or pump terms, a
// complex64 propagator; NLSE_GROUP_FUSED=0 turns it off.
bool group_fused_ok(int n, const nlse_plan* plans, const nlse_operator* ops,
                    const int64_t* nsteps) {
  const char* env = getenv("NLSE_GROUP_FUSED");
  if (env && env[0] == '0') return false;
  if (n < 1 || n > multi_max_plans()) return false;
  for (int i = 0; i < n; ++i) {
    const nlse_plan_s* p = plans[i];
    const nlse_operator* op = &ops[i];
    const nlse_desc& d = p->d;
    if (nsteps[i] != nsteps[0] || nsteps[i] < 1) return false;
    if (d.dtype != NLSE_C64 || d.comps != 1 || d.ndim != 2 || !p->blk || !p->rows_tma_ok)
      return false;
    if (p->lg[0] < 8 || p->lg[0] > 11 || p->lg[1] < 8 || p->lg[1] > 11) return false;
    if (op->nl_khat || op->pump_r || op->probe_r || op->prop_c128) return false;
    if (d.nfields * d.shape[0] >= (int64_t(1) << 31)) return false;
  }
  return true;
}

// The whole batch's loop with two launches per step (columns of every plan,
// then rows of every plan), after each plan's parameter mirror, propagator
// layout and first forward row pass.
int enqueue_group_fused(int n, const nlse_plan* plans, void* const* fields,
                        const nlse_operator* ops, int64_t nsteps, cudaStream_t s) {
  std::vector<StepArgs> mid(n), last(n);
  std::vector<ColArgs> col(n);
  std::vector<const CUtensorMap*> tm(n);
  std::vector<int> lr(n), lc(n);
  for (int i = 0; i < n; ++i) {
    nlse_plan_s* p = plans[i];
    const nlse_operator* op = &ops[i];
    int rc = mirror_params(p, op, s);
    if (rc == NLSE_OK) rc = refresh_prop(p, op, false, s);
    if (rc != NLSE_OK) return rc;
    StepArgs a = row_args(p, fields[i], op);
    a.tma_grid = p->nsm;
    const uint32_t pre = op->scheme == 1 ? F_PRE_NL : 0u;
    StepArgs a0 = a;
    a0.flags |= pre | F_OUT_BLK;
    cudaError_t e = rows(p, ROW_FWD, p->lg[1], a0, s);
    if (e != cudaSuccess) return cuda_fail(e, "row pass (forward)");
    mid[i] = a;
    mid[i].flags |= pre | F_IN_BLK | F_OUT_BLK;
    last[i] = a;
    last[i].flags |= F_IN_BLK;
    col[i] = col_blk_args(p, op);
    tm[i] = &p->tmS;
    lr[i] = p->lg[1];
    lc[i] = p->lg[0];
  }
  const int nsm = plans[0]->nsm;
  for (int64_t st = 0; st < nsteps; ++st) {
    cudaError_t e = launch_cols_tile_multi(n, col.data(), lc.data(), s, false);
    if (e != cudaSuccess) return cuda_fail(e, "column pass (all plans)");
    if (st + 1 < nsteps)
      e = launch_rows_multi(ROW_INV_NL_FWD, n, mid.data(), tm.data(), lr.data(), nsm, s, false);
    else
      e = launch_rows_multi(ROW_INV_NL, n, last.data(), tm.data(), lr.data(), nsm, s, false);
    if (e != cudaSuccess) return cuda_fail(e, "row pass (all plans)");
  }
  return NLSE_OK;
}

}  // namespace

struct nlse_group_s {
  cudaStream_t cap = nullptr;
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> ev;
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t launched = nullptr;  // recorded after each launch of gexec
  std::vector<uint8_t> key;  // serialized arguments of the captured graph
  int fused = 0;             // the captured graph runs two launches per step for the batch
};

extern "C" {

int nlse_group_create(nlse_group* out) {
  g_err.clear();
  if (!out) return fail(NLSE_ERR_ARG, "null argument");
  auto* g = new nlse_group_s();
  cudaError_t e = cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->launched, cudaEventDisableTiming);
  // kernel attributes of the one-launch-per-pass kernels (outside any capture)
  if (e == cudaSuccess) e = launch_rows_multi(0, 0, nullptr, nullptr, nullptr, 0, nullptr, true);
  if (e == cudaSuccess) e = launch_cols_tile_multi(0, nullptr, nullptr, nullptr, true);
  if (e != cudaSuccess) {
    nlse_group_destroy(g);
    return cuda_fail(e, "group create");
  }
  *out = g;
  return NLSE_OK;
}

int nlse_group_destroy(nlse_group g) {
  if (!g) return NLSE_OK;
  if (g->gexec) cudaGraphExecDestroy(g->gexec);
  for (auto st : g->branch) cudaStreamDestroy(st);
  for (auto ev : g->ev) cudaEventDestroy(ev);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->launched) cudaEventDestroy(g->launched);
  if (g->cap) cudaStreamDestroy(g->cap);
  delete g;
  return NLSE_OK;
}

}  // extern "C"

namespace {
// Make g's executable graph run `graph` (consumed): update the existing one in
// place when the topology is the same (a new call with new buffers or
// parameters), else instantiate anew.
cudaError_t group_exec_refresh(nlse_group_s* g, cudaGraph_t graph) {
  if (g->gexec) {
    // the previous launch of the executable graph has finished before it changes
    cudaEventSynchronize(g->launched);
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(g->gexec, graph, &info) == cudaSuccess) {
      cudaGraphDestroy(graph);
      return cudaSuccess;
    }
    cudaGetLastError();
    cudaGraphExecDestroy(g->gexec);
    g->gexec = nullptr;
  }
  const cudaError_t e = cudaGraphInstantiate(&g->gexec, graph, 0);
  cudaGraphDestroy(graph);
  return e;
}
}  // namespace

extern "C" {

int nlse_group_propagate(nlse_group g, int32_t n, const nlse_plan* plans, void* const* fields,
                         const nlse_operator* ops, const int64_t* nsteps, void* stream) {
  g_err.clear();
  if (!g || n <= 0 || !plans || !fields || !ops || !nsteps) return fail(NLSE_ERR_ARG, "null argument");
  for (int i = 0; i < n; ++i) {
    if (!plans[i] || !fields[i] || nsteps[i] < 0) return fail(NLSE_ERR_ARG, "group %d: bad entry", i);
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i])
        return fail(NLSE_ERR_ARG, "groups %d and %d share a plan (its scratch would be raced)", j, i);
    if (!plans[i]->fft_ok) return fail(NLSE_ERR_UNSUPPORTED, "group %d: transform lengths", i);
    const int rc = check_op(plans[i], &ops[i]);
    if (rc != NLSE_OK) return rc;
  }
  std::vector<uint8_t> key;
  auto put = [&](const void* p, size_t b) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    key.insert(key.end(), c, c + b);
  };
  put(&n, sizeof(n));
  put(plans, sizeof(nlse_plan) * n);
  put(fields, sizeof(void*) * n);
  put(ops, sizeof(nlse_operator) * n);
  put(nsteps, sizeof(int64_t) * n);
  for (int i = 0; i < n; ++i) put(&plans[i]->kgen, sizeof(uint64_t));
  const uint8_t fused = group_fused_ok(n, plans, ops, nsteps) ? 1 : 0;
  put(&fused, 1);
  g->fused = fused;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (fused && !(g->gexec && key == g->key)) {
    cudaGraph_t graph = nullptr;
    NLSE_CUDA(cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    const int rc = enqueue_group_fused(n, plans, fields, ops, nsteps[0], g->cap);
    const cudaError_t e2 = cudaStreamEndCapture(g->cap, &graph);
    if (rc != NLSE_OK || e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      if (rc != NLSE_OK) return rc;
      return cuda_fail(e2, "group capture");
    }
    const cudaError_t e = group_exec_refresh(g, graph);
    if (e != cudaSuccess) return cuda_fail(e, "group graph instantiate");
    g->key = key;
  }
  if (!(g->gexec && key == g->key)) {
    while ((int)g->branch.size() < n) {
      cudaStream_t st;
      cudaEvent_t ev;
      NLSE_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "branch stream");
      NLSE_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "branch event");
      g->branch.push_back(st);
      g->ev.push_back(ev);
    }
    cudaGraph_t graph = nullptr;
    NLSE_CUDA(cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    int rc = NLSE_OK;
    cudaError_t e = cudaEventRecord(g->fork, g->cap);
    for (int i = 0; i < n && rc == NLSE_OK && e == cudaSuccess; ++i) {
      e = cudaStreamWaitEvent(g->branch[i], g->fork, 0);
      if (e != cudaSuccess) break;
      rc = enqueue_steps(plans[i], fields[i], &ops[i], nsteps[i], 0, g->branch[i]);
      if (rc != NLSE_OK) break;
      e = cudaEventRecord(g->ev[i], g->branch[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(g->cap, g->ev[i], 0);
    }
    const cudaError_t e2 = cudaStreamEndCapture(g->cap, &graph);
    if (rc != NLSE_OK || e != cudaSuccess || e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      if (rc != NLSE_OK) return rc;
      return cuda_fail(e != cudaSuccess ? e : e2, "group capture");
    }
    e = group_exec_refresh(g, graph);
    if (e != cudaSuccess) return cuda_fail(e, "group graph instantiate");
    g->key = key;
  }
  NLSE_CUDA(cudaGraphLaunch(g->gexec, s), "group graph launch");
  NLSE_CUDA(cudaEventRecord(g->launched, s), "group graph launch");
  return NLSE_OK;
}

int nlse_group_fused(nlse_group g) { return g ? g->fused : 0; }

int nlse_plan_status(nlse_plan p, void* stream) {
  g_err.clear();
  if (!p) return fail(NLSE_ERR_ARG, "null plan");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int h = 0;
  NLSE_CUDA(cudaMemcpyAsync(&h, p->status, sizeof(int), cudaMemcpyDeviceToHost, s), "status read");
  NLSE_CUDA(cudaStreamSynchronize(s), "status sync");
  if (h != DEV_OK) {
    NLSE_CUDA(cudaMemsetAsync(p->status, 0, sizeof(int), s), "status reset");
    NLSE_CUDA(cudaStreamSynchronize(s), "status sync");
    return fail(NLSE_ERR_TIMEOUT, "a kernel stopped early (device code %d: %s); the results of "
                "the calls since the last status check are not valid", h,
                h == DEV_WAIT_TIMEOUT ? "a bounded wait gave up"
                : h == DEV_SMEM_MISALIGNED ? "shared memory not 128-byte aligned for its copies"
                                           : "unknown");
  }
  return NLSE_OK;
}

int nlse_propagate(nlse_plan p, void* A, const nlse_operator* op, int64_t nsteps, int64_t step0,
                   int32_t flags, void* stream) {
  g_err.clear();
  if (!p || !A) return fail(NLSE_ERR_ARG, "null plan or field");
  if (nsteps < 0 || step0 < 0) return fail(NLSE_ERR_ARG, "negative step count or index");
  if (!p->fft_ok)
    return fail(NLSE_ERR_UNSUPPORTED,
                "transform lengths must be powers of two from 2 to %d", 1 << kMaxLog2);

  int rc = check_op(p, op);
  if (rc != NLSE_OK) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (!(flags & NLSE_RUN_GRAPH)) return enqueue_steps(p, A, op, nsteps, step0, s);

  GraphKey key{A, *op, nsteps, step0, p->kgen};
  if (!(p->gvalid && p->gkey == key)) {
    // Capture on the plan's private stream, ordered after the caller's work
    // only at launch time (the graph itself has no external dependencies).
    cudaGraph_t g = nullptr;
    NLSE_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    rc = enqueue_steps(p, A, op, nsteps, step0, p->cap);
    cudaError_t e = cudaStreamEndCapture(p->cap, &g);
    if (rc != NLSE_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "end capture");
    bool updated = false;
    if (p->gexec) {
      // the previous launch of the executable graph has finished before it changes
      if (p->glaunched) cudaEventSynchronize(p->glaunched);
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(p->gexec, g, &info) == cudaSuccess) updated = true;
      else {
        cudaGetLastError();
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
      }
    }
    if (!updated) {
      e = cudaGraphInstantiate(&p->gexec, g, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        p->gvalid = false;
        return cuda_fail(e, "graph instantiate");
      }
    }
    cudaGraphDestroy(g);
    p->gkey = key;
    p->gvalid = true;
  }
  NLSE_CUDA(cudaGraphLaunch(p->gexec, s), "graph launch");
  if (!p->glaunched)
    NLSE_CUDA(cudaEventCreateWithFlags(&p->glaunched, cudaEventDisableTiming), "graph launch");
  NLSE_CUDA(cudaEventRecord(p->glaunched, s), "graph launch");
  return NLSE_OK;
}

int nlse_pass(nlse_plan p, void* A, const nlse_operator* op, int32_t pass, int64_t step,
              void* stream) {
  g_err.clear();
  if (!p || !A) return fail(NLSE_ERR_ARG, "null plan or field");
  if (step < 0) return fail(NLSE_ERR_ARG, "negative step index");
  if (!p->fft_ok)
    return fail(NLSE_ERR_UNSUPPORTED,
                "transform lengths must be powers of two from 2 to %d", 1 << kMaxLog2);

  int rc = check_op(p, op);
  if (rc != NLSE_OK) return rc;
  return enqueue_pass(p, A, op, pass, step, reinterpret_cast<cudaStream_t>(stream));
}

int nlse_plan_set_variant(nlse_plan p, int32_t rows, int32_t cols, int32_t rows_ctas_per_sm,
                          int32_t cols_ctas_per_sm) {
  g_err.clear();
  if (!p) return fail(NLSE_ERR_ARG, "null plan");
  if (rows < 0 || rows > NLSE_ROWS_DEEP || cols < 0 || cols > NLSE_COLS_DEEP ||
      rows_ctas_per_sm < 0 || cols_ctas_per_sm < 0 || rows_ctas_per_sm > 32 ||
      cols_ctas_per_sm > 32)
    return fail(NLSE_ERR_ARG, "variant codes 0..4, CTAs per SM 0..32");
  if (!(p->rows_avail >> rows & 1))
    return fail(NLSE_ERR_UNSUPPORTED, "row pass variant %d is not available for this plan", rows);
  if (!(p->cols_avail >> cols & 1))
    return fail(NLSE_ERR_UNSUPPORTED, "column pass variant %d is not available for this plan", cols);
  if (p->rows_var != rows || p->cols_var != cols || p->rows_cap != rows_ctas_per_sm ||
      p->cols_cap != cols_ctas_per_sm) {
    p->rows_var = rows;
    p->cols_var = cols;
    p->rows_tma = rows != NLSE_ROWS_LINE;
    p->cols_tma = cols != NLSE_COLS_TILE;
    p->rows_cap = rows_ctas_per_sm;
    p->cols_cap = cols_ctas_per_sm;
    ++p->kgen;  // captured graphs hold the old kernels
  }
  return NLSE_OK;
}

int nlse_plan_get_variant(nlse_plan p, int32_t* rows, int32_t* cols, int32_t* rows_ctas_per_sm,
                          int32_t* cols_ctas_per_sm, uint32_t* rows_avail, uint32_t* cols_avail) {
  g_err.clear();
  if (!p || !rows || !cols || !rows_ctas_per_sm || !cols_ctas_per_sm || !rows_avail || !cols_avail)
    return fail(NLSE_ERR_ARG, "null argument");
  *rows = p->rows_var;
  *cols = p->cols_var;
  *rows_ctas_per_sm = p->rows_cap;
  *cols_ctas_per_sm = p->cols_cap;
  *rows_avail = p->rows_avail;
  *cols_avail = p->cols_avail;
  return NLSE_OK;
}

int nlse_plan_set_kernels(nlse_plan p, int32_t rows_tma, int32_t cols_tma) {
  g_err.clear();
  if (!p) return fail(NLSE_ERR_ARG, "null plan");
  if (rows_tma && !p->rows_tma_ok)
    return fail(NLSE_ERR_UNSUPPORTED, "this plan has no TMA row pass (geometry or disabled)");
  if (cols_tma && !p->cols_tma_ok)
    return fail(NLSE_ERR_UNSUPPORTED, "the TMA column pass is disabled for this plan");
  return nlse_plan_set_variant(p, rows_tma ? NLSE_ROWS_TMA : NLSE_ROWS_LINE,
                               cols_tma ? NLSE_COLS_TMA : NLSE_COLS_TILE, 0, 0);
}

int nlse_plan_get_kernels(nlse_plan p, int32_t* rows_tma, int32_t* cols_tma,
                          int32_t* rows_tma_ok, int32_t* cols_tma_ok) {
  g_err.clear();
  if (!p || !rows_tma || !cols_tma || !rows_tma_ok || !cols_tma_ok)
    return fail(NLSE_ERR_ARG, "null argument");
  *rows_tma = p->rows_tma;
  *cols_tma = p->cols_tma;
  *rows_tma_ok = p->rows_tma_ok;
  *cols_tma_ok = p->cols_tma_ok;
  return NLSE_OK;
}

int nlse_plan_set_nonlocal(nlse_plan p, int64_t pad_y, int64_t pad_x) {
  g_err.clear();
  if (!p) return fail(NLSE_ERR_ARG, "null plan");
  const nlse_desc& d = p->d;
  if (p->nlsub) {
    nlse_plan_destroy(p->nlsub);
    p->nlsub = nullptr;
  }
  if (p->X) {
    cudaFree(p->X);
    p->X = nullptr;
  }
  p->nl_py = p->nl_px = 0;
  if (pad_x == 0) return NLSE_OK;
  if (d.ndim == 3) return fail(NLSE_ERR_UNSUPPORTED, "nonlocal response of 3-D fields");
  const int64_t nx = d.shape[d.ndim - 1], ny = d.ndim == 2 ? d.shape[0] : 1;
  if (d.ndim == 1) pad_y = 1;
  const int lx = ilog2_pow2(pad_x), ly = d.ndim == 2 ? ilog2_pow2(pad_y) : 1;
  if (lx < kMinLog2 || lx > kMaxLog2 || ly < kMinLog2 || ly > kMaxLog2 || pad_x < nx ||
      pad_y < ny)
    return fail(NLSE_ERR_UNSUPPORTED,
                "padded nonlocal grid %lld x %lld: powers of two from the grid size to %d",
                (long long)pad_y, (long long)pad_x, 1 << kMaxLog2);
  nlse_desc sd{};
  sd.ndim = d.ndim;
  if (d.ndim == 2) {
    sd.shape[0] = pad_y;
    sd.shape[1] = pad_x;
  } else {
    sd.shape[0] = pad_x;
  }
  sd.nfields = d.nfields;
  sd.comps = 1;
  sd.dtype = d.dtype;
  nlse_plan q = nullptr;
  int rc = nlse_plan_create(&q, &sd);
  if (rc != NLSE_OK) return rc;
  const size_t es = d.dtype == NLSE_C64 ? 8 : 16;
  cudaError_t e = cudaMalloc(&p->X, (size_t)d.nfields * pad_y * pad_x * es);
  if (e != cudaSuccess) {
    nlse_plan_destroy(q);
    return cuda_fail(e, "cudaMalloc(nonlocal scratch)");
  }
  p->nlsub = q;
  p->nl_py = pad_y;
  p->nl_px = pad_x;
  return NLSE_OK;
}

int nlse_fft(nlse_plan p, void* A, int32_t inverse, void* stream) {
  g_err.clear();
  if (!p || !A) return fail(NLSE_ERR_ARG, "null plan or field");
  if (!p->fft_ok)
    return fail(NLSE_ERR_UNSUPPORTED,
                "transform lengths must be powers of two from 2 to %d", 1 << kMaxLog2);

  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const nlse_desc& d = p->d;
  // components are independent transforms here: view them as fields
  nlse_plan_s q = *p;
  q.d.nfields = d.nfields * d.comps;
  q.d.comps = 1;
  StepArgs a = row_args(&q, A, nullptr);
  a.flags = F_NO_POST;
  const int rl = p->lg[d.ndim - 1];
  cudaError_t e = cudaSuccess;
  if (!inverse) {
    e = rows(&q, ROW_FWD, rl, a, s);
    for (int ax = d.ndim - 2; ax >= 0 && e == cudaSuccess; --ax)
      e = cols(&q, COL_FWD, p->lg[ax], col_args(&q, A, nullptr, ax), s);
  } else {
    for (int ax = 0; ax + 1 < d.ndim && e == cudaSuccess; ++ax)
      e = cols(&q, COL_INV, p->lg[ax], col_args(&q, A, nullptr, ax), s);
    if (e == cudaSuccess) e = rows(&q, ROW_INV, rl, a, s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "fft");
  return NLSE_OK;
}

int nlse_nonlinear(nlse_plan p, void* A, const void* asq, const nlse_operator* op, int64_t step,
                   void* stream) {
  g_err.clear();
  if (!p || !A || !op || !op->params) return fail(NLSE_ERR_ARG, "null argument");
  if (p->d.dtype == NLSE_C64 && op->V && !op->v_f32)
    return fail(NLSE_ERR_ARG, "a complex64 field needs a single-precision potential");
  const int mrc = mirror_params(p, op, reinterpret_cast<cudaStream_t>(stream));
  if (mrc != NLSE_OK) return mrc;
  StepArgs a = row_args(p, A, op);
  a.asq = asq;
  if (asq) a.flags |= F_ASQ_EXT;
  a.step = (int)step;
  cudaError_t e = launch_nl_pointwise(p->d.dtype, a, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "nonlinear step");
  return NLSE_OK;
}

size_t nlse_power_workspace_size(int64_t nseg, int64_t seg_len) {
  if (nseg <= 0 || seg_len <= 0) return 0;
  return (size_t)nseg * (size_t)power_chunks(seg_len) * sizeof(double);
}

int nlse_power(const void* A, int32_t dtype, int64_t nseg, int64_t seg_len, double* out,
               void* workspace, size_t workspace_bytes, void* stream) {
  g_err.clear();
  if (!A || !out) return fail(NLSE_ERR_ARG, "null argument");
  if (dtype != NLSE_C64 && dtype != NLSE_C128) return fail(NLSE_ERR_ARG, "dtype %d", dtype);
  if (nseg < 0 || seg_len <= 0) return fail(NLSE_ERR_ARG, "bad segment geometry");
  if (nseg > 65535) return fail(NLSE_ERR_UNSUPPORTED, "at most 65535 segments per call");
  const size_t need = nlse_power_workspace_size(nseg, seg_len);
  if (!workspace || workspace_bytes < need)
    return fail(NLSE_ERR_ARG, "workspace too small: %zu bytes needed", need);
  cudaError_t e = launch_power(dtype, A, nseg, seg_len, static_cast<double*>(workspace),
                               power_chunks(seg_len), out,
                               reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "power");
  return NLSE_OK;
}

int nlse_power_noalloc(const void* A, int32_t dtype, int64_t nseg, int64_t seg_len, double* out,
                       void* stream) {
  g_err.clear();
  if (!A || !out) return fail(NLSE_ERR_ARG, "null argument");
  if (dtype != NLSE_C64 && dtype != NLSE_C128) return fail(NLSE_ERR_ARG, "dtype %d", dtype);
  if (nseg < 0 || seg_len <= 0) return fail(NLSE_ERR_ARG, "bad segment geometry");
  if (nseg > 65535) return fail(NLSE_ERR_UNSUPPORTED, "at most 65535 segments per call");
  const int64_t need = nseg * (int64_t)power_chunks(seg_len);
  if (need > noalloc_partials_max())
    return fail(NLSE_ERR_ARG,
                "nlse_power_noalloc: %lld segments of %lld elements need %lld partial sums, the "
                "static array holds %lld (nseg * min(1024, ceil(seg_len / 8192)) must not exceed "
                "it); use nlse_power with a workspace",
                (long long)nseg, (long long)seg_len, (long long)need,
                (long long)noalloc_partials_max());
  cudaError_t e = launch_power_noalloc(dtype, A, nseg, seg_len, out,
                                       reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "power (no allocation)");
  return NLSE_OK;
}

int nlse_normalize(const void* in, void* out, int32_t dtype, int64_t nseg, int64_t seg_len,
                   const double* sums, const double* target, double coef, void* stream) {
  g_err.clear();
  if (!in || !out || !sums || !target) return fail(NLSE_ERR_ARG, "null argument");
  if (dtype != NLSE_C64 && dtype != NLSE_C128) return fail(NLSE_ERR_ARG, "dtype %d", dtype);
  if (nseg > 65535) return fail(NLSE_ERR_UNSUPPORTED, "at most 65535 segments per call");
  cudaError_t e = launch_scale(dtype, in, out, nseg, seg_len, sums, target, coef,
                               reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "normalize");
  return NLSE_OK;
}

int nlse_square_mod(const void* A, void* out, int32_t dtype, int64_t n, void* stream) {
  g_err.clear();
  if (!A || !out) return fail(NLSE_ERR_ARG, "null argument");
  if (dtype != NLSE_C64 && dtype != NLSE_C128) return fail(NLSE_ERR_ARG, "dtype %d", dtype);
  cudaError_t e = launch_abs2(dtype, A, out, n, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "square_mod");
  return NLSE_OK;
}

int nlse_add_noise(void* A, int32_t dtype, int64_t nfields, int64_t pix, double sigma0,
                   double sigma1, uint64_t seed, int64_t step, void* stream) {
  g_err.clear();
  if (!A || nfields <= 0 || pix <= 0 || step < 0 || step > 0xFFFFFFFFll ||
      (dtype != NLSE_C64 && dtype != NLSE_C128))
    return fail(NLSE_ERR_ARG, "nlse_add_noise: bad argument");
  cudaError_t e = launch_add_noise(dtype, A, nfields, pix, sigma0, sigma1, seed, (uint32_t)step,
                                   reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "add_noise");
  return NLSE_OK;
}

int nlse_wait_selftest(int32_t* status, uint64_t* elapsed_ns, int64_t limit_ns, void* stream) {
  g_err.clear();
  if (!status || !elapsed_ns || limit_ns <= 0 || limit_ns > (int64_t)kWaitLimitNs)
    return fail(NLSE_ERR_ARG, "nlse_wait_selftest: limit must be in (0, 1 s]");
  cudaError_t e = launch_wait_selftest(reinterpret_cast<int*>(status),
                                       reinterpret_cast<unsigned long long*>(elapsed_ns),
                                       (unsigned long long)limit_ns,
                                       reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "wait_selftest");
  return NLSE_OK;
}

int nlse_delta_n(const void* A, int32_t dtype, int64_t nseg, int64_t pix, const double* coef,
                 const double* isat, int32_t flags, void* out, void* stream) {
  g_err.clear();
  if (!A || !coef || !isat || !out || nseg <= 0 || pix <= 0 || (flags & ~3) ||
      (dtype != NLSE_C64 && dtype != NLSE_C128))
    return fail(NLSE_ERR_ARG, "nlse_delta_n: bad argument");
  cudaError_t e = launch_delta_n(dtype, A, nseg, pix, coef, isat, flags, out,
                                 reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "delta_n");
  return NLSE_OK;
}

int nlse_delta_n_max(const void* A, int32_t dtype, int64_t nseg, int64_t pix, const double* n2abs,
                     const double* isat, double c, double eps0, int32_t flags, double* out,
                     void* stream) {
  g_err.clear();
  if (!A || !n2abs || !isat || !out || nseg <= 0 || pix <= 0 || (flags & ~3) ||
      (dtype != NLSE_C64 && dtype != NLSE_C128))
    return fail(NLSE_ERR_ARG, "nlse_delta_n_max: bad argument");
  cudaError_t e = launch_delta_n_max(dtype, A, nseg, pix, n2abs, isat, c, eps0, flags, out,
                                     reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "delta_n_max");
  return NLSE_OK;
}

}  // extern "C"

namespace {
// In-place transform of a plan's own geometry (used for the nonlocal scratch).
int fft_sub(nlse_plan_s* q, void* X, int inverse, cudaStream_t s) {
  return nlse_fft(q, X, inverse, s);
}
}  // namespace
