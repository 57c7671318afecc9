/*
 * libnlse_sm103 — C ABI of the GB300 (sm_103a) split-step Fourier engine.
 *
 * The library replaces the device work of the reference package's GPU
 * backend (Quantum-Optics-LKB/NLSE v2.3.0, backend="GPU"): VkFFT plans, the
 * CuPy fused elementwise kernels and the z-loop of out_field.  Every pointer
 * passed in is a device pointer owned by the caller (Python passes
 * torch.Tensor.data_ptr()); the plan owns only its own tables.  All calls are
 * asynchronous on the given stream (a cudaStream_t passed as void*; NULL is
 * the legacy default stream).  Kernel faults surface at the caller's next
 * synchronisation.
 *
 * Return value of every int function: NLSE_OK (0) or a negative nlse_status;
 * nlse_last_error() then describes the failure (thread-local string).
 *
 * Layout of a field A (C order, complex64 or complex128 interleaved):
 *   ndim = 1: [nfields][comps][NX]
 *   ndim = 2: [nfields][comps][NY][NX]
 *   ndim = 3: [nfields][NY][NX][NT]            (comps = 1)
 * The transform runs over the ndim trailing axes, batched over the rest, the
 * way the reference plans VkFFTApp(A.shape, ndim=len(_last_axes)) over the
 * trailing axes (NLSE/nlse.py:199-218).  Transform axis lengths are powers
 * of two from 2 to 4096.
 */
#ifndef NLSE_GB300_H
#define NLSE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NLSE_ABI_VERSION 2

typedef enum { NLSE_C64 = 0, NLSE_C128 = 1 } nlse_dtype;

typedef enum {
  NLSE_OK = 0,
  NLSE_ERR_ARG = -1,         /* bad argument (null pointer, bad size, bad flag) */
  NLSE_ERR_UNSUPPORTED = -2, /* shape or option this build does not implement */
  NLSE_ERR_CUDA = -3,        /* a CUDA runtime call failed */
  NLSE_ERR_STATE = -4,       /* call not valid in the current state */
  NLSE_ERR_TIMEOUT = -5      /* a bounded wait inside a kernel gave up (see nlse_plan_status) */
} nlse_status;

/* nlse_propagate flags */
#define NLSE_RUN_GRAPH 1 /* capture the whole step sequence in a CUDA graph, replay it when
                            called again with the same pointers and step range */

typedef struct nlse_plan_s* nlse_plan;

/* Geometry of the fields a plan transforms. */
typedef struct {
  int32_t ndim;     /* 1, 2 or 3 transform axes */
  int64_t shape[3]; /* transform lengths, outermost first: {NX}, {NY,NX}, {NY,NX,NT} */
  int64_t nfields;  /* independent fields (product of the leading dimensions) */
  int32_t comps;    /* components per field: 1, or 2 (CNLSE/DDGPE, stacked before the axes) */
  int32_t dtype;    /* nlse_dtype of the field */
} nlse_desc;

/*
 * Per-field parameter block: nfields x NLSE_PARAM_STRIDE doubles in device
 * memory.  Index [set*16 + comp*7 + k], set 0 = the nonlinear step after the
 * linear step, set 1 = the half step before it ("double" scheme), k:
 *   0 dz, 1 alpha (already halved as the reference passes alpha/2),
 *   2 g_self, 3 g_cross, 4 Isat_self, 5 Isat_cross (converted units, inf for
 *   none), 6 vscale (V' = vscale * V).
 * [14], [15]: cos and sin of (omega/2)*dz for the Rabi rotation (real parts
 * when dz is complex); [34], [35]: their imaginary parts (0 for a real dz).
 * [30], [31]: real and imaginary parts of dz of the DDGPE pump term.
 * [32], [33]: imaginary part of dz of set 0 and set 1 (imaginary-time
 * evolution with a complex delta_z, NLSE/nlse.py:505-508; else 0).
 */
#define NLSE_PARAM_STRIDE 40

/* The operator of one split step. */
typedef struct {
  const void* V;         /* potential, or NULL */
  int32_t v_complex;     /* V holds complex values (else real) */
  int32_t v_f32;         /* V stored in single precision (else double) */
  int64_t v_fstride;     /* elements between two fields' potentials; 0 = shared */
  const void* prop;      /* linear propagator, [comps][transform axes] */
  int32_t prop_c128;     /* propagator stored as complex128 (else complex64) */
  int64_t prop_cstride;  /* elements between the components' propagators; 0 = shared */
  const double* params;  /* per-field parameter block, see above */
  int32_t scheme;        /* 0 = "single" (Lie), 1 = "double" (Strang) */
  int32_t rabi;          /* apply the Rabi rotation after the nonlinear step */
  const void* pump_r;    /* DDGPE pump spatial profile [pixels] (field dtype) or NULL */
  const void* pump_t;    /* DDGPE pump time profile [steps] (field dtype) */
  const void* probe_r;   /* DDGPE probe spatial profile or NULL */
  const void* probe_t;
  int64_t prop_version;  /* caller's version tag of the propagator contents: the plan keeps a
                            re-laid-out copy of the propagator and refreshes it whenever the
                            pointer, format or this tag changes */
  const void* nl_khat;   /* nonlocal response: spectrum (field dtype) of the kernel placed on the
                            plan's padded grid with its centre at the origin, or NULL for a local
                            response; see nlse_plan_set_nonlocal */
  const void* nl_maps;   /* spatially varying nonlinear coefficients of a one-component field
                            (the reference's n2, alpha or Isat given as arrays over the grid,
                            NLSE/nlse.py:309-328 and kernels_gpu.py:4-65), or NULL: planes
                            [3][map fields][pixels] in the field's real type (float for
                            complex64, double for complex128) holding g = k/2 n2 c eps0,
                            alpha/2 and 1/Isat' (Isat' = 2 Isat/(eps0 c)); a plane whose bit is
                            set in maps_mask replaces the parameter block's per-field value */
  int64_t maps_fstride;  /* elements between two fields' maps in a plane; 0 = shared */
  int64_t maps_plane;    /* elements between two planes */
  int32_t maps_mask;     /* bit 0: g plane, bit 1: alpha/2 plane, bit 2: 1/Isat' plane */
} nlse_operator;

/* ABI version of the loaded library (NLSE_ABI_VERSION). */
int nlse_abi_version(void);

/* Description of the last error on this thread ("" if none). */
const char* nlse_last_error(void);

/*
 * Create a plan on the current CUDA device: validates the geometry, uploads
 * the twiddle tables, allocates the plan's scratch (the blocked spectral
 * buffer of 2-D plans, an FP32 copy of the parameter block) and sets the
 * kernel attributes.  Replaces NLSE._build_fft_plan (NLSE/nlse.py:199-218).
 * Axis lengths that are not powers of two from 2 to 4096 give a plan usable
 * only by nlse_nonlinear; the transform entry points then return
 * NLSE_ERR_UNSUPPORTED.
 */
int nlse_plan_create(nlse_plan* out, const nlse_desc* desc);
int nlse_plan_destroy(nlse_plan plan);

/*
 * Synchronise `stream` and report whether any kernel of this plan gave up a
 * bounded wait since the last check (NLSE_ERR_TIMEOUT; the flag is then
 * cleared).  Kernels that wait on asynchronous copies never spin without a
 * deadline: on expiry they record the failure here and return.
 */
int nlse_plan_status(nlse_plan plan, void* stream);

/*
 * Advance A in place by nsteps split steps of the reference's
 * NLSE.split_step (NLSE/nlse.py:372-487), CNLSE.split_step
 * (NLSE/cnlse.py:204-423) or DDGPE.split_step (NLSE/ddgpe.py:247-457), i.e.
 * the body of the out_field z-loop (NLSE/nlse.py:570-588) without callbacks.
 * step0 is the loop index of the first step (selects pump_t[step0 + s]).
 * A is in real space on entry and on return.
 */
int nlse_propagate(nlse_plan plan, void* A, const nlse_operator* op, int64_t nsteps,
                   int64_t step0, int32_t flags, void* stream);

/*
 * Groups of fields with different geometries advanced together, the whole
 * batched z-loop one CUDA graph launch (replayed when called again with the
 * same arguments; NLSE_RUN_GRAPH is implied).  A batch of mixed grids (e.g.
 * 96 fields at 256^2, 48 at 512^2, 16 at 1024^2, 4 at 2048^2) is four
 * groups, each with its own plan, field and operator.
 * When every group is a one-component complex64 2-D field of 256..2048
 * points per axis with the TMA row pass, the same step count, no nonlocal
 * response or pump terms and a complex64 propagator (and at most 8 groups),
 * each step is TWO launches for the whole batch: one persistent column pass
 * over every group's tiles and one persistent row pass over every group's
 * lines (after each group's first forward row pass); NLSE_GROUP_FUSED=0
 * turns this off.  Otherwise each group runs its own step sequence on a
 * concurrent branch of the graph.  No reference counterpart as one call: the
 * reference runs one out_field per NLSE instance.
 */
typedef struct nlse_group_s* nlse_group;
int nlse_group_create(nlse_group* out);
int nlse_group_destroy(nlse_group group);
int nlse_group_propagate(nlse_group group, int32_t ngroups, const nlse_plan* plans,
                         void* const* fields, const nlse_operator* ops, const int64_t* nsteps,
                         void* stream);
/* 1 if the group's last nlse_group_propagate ran two launches per step for the
 * whole batch, 0 if it ran one branch per group. */
int nlse_group_fused(nlse_group group);

/* Kernel variants of a plan's 2-D passes: TMA-fed persistent row passes
 * (rows_tma) or one CTA per line, TMA-fed persistent column passes (cols_tma)
 * or one CTA per tile.  The arithmetic is the same either way (results agree
 * to rounding: the kernels fuse multiply-adds differently); the choice is a
 * speed one (nlse_gb300.autotune times them).  No reference counterpart (the
 * reference's VkFFTApp(tune=True) tunes its FFT plan, NLSE/nlse.py:216).
 * Returns NLSE_ERR_UNSUPPORTED for a variant the plan does not have. */
int nlse_plan_set_kernels(nlse_plan plan, int32_t rows_tma, int32_t cols_tma);
int nlse_plan_get_kernels(nlse_plan plan, int32_t* rows_tma, int32_t* cols_tma,
                          int32_t* rows_tma_ok, int32_t* cols_tma_ok);

/* The same choice with every variant and launch shape, as codes:
 *   rows: NLSE_ROWS_LINE (one CTA per line), NLSE_ROWS_TMA (TMA-fed
 *         persistent), NLSE_ROWS_PAIR (TMA-fed persistent, two lines per
 *         thread in packed FP32: one-component complex64 fields, rows of
 *         64..4096 points);
 *   cols: NLSE_COLS_TILE (one CTA per tile), NLSE_COLS_TMA (persistent bulk-
 *         copy ring), NLSE_COLS_PAIR (the ring with two columns per thread in
 *         packed FP32: complex64, columns of 64..2048 points).
 *   NLSE_ROWS_DEEP / NLSE_COLS_DEEP: the pair passes with deeper prefetch
 *         (the next work item's copies in flight during the whole current
 *         item; rows: exchanges in the item's own buffer and the mid-loop
 *         pass's rows stored by tensor map from shared memory, columns: three
 *         staging tiles and no exchange tile), same sizes as the pair ones.
 * rows_ctas_per_sm / cols_ctas_per_sm cap the persistent passes' CTAs per SM
 * (0: as many as fit), which sets their grid (SMs x CTAs per SM).  A launch
 * the chosen variant cannot serve (two components, Rabi or pump terms, a
 * complex128 propagator, an external |A|^2) runs the TMA variant instead.
 * get returns the current choice and bit masks of the available variants
 * (bit v set: variant code v).  The plan's default is NLSE_ROWS_TMA (where
 * the tensor map is available, else NLSE_ROWS_LINE) and, for one-component
 * complex64 fields, NLSE_COLS_TILE (else NLSE_COLS_TMA where available).  No reference counterpart (the
 * reference's VkFFTApp(tune=True) tunes its FFT plan, NLSE/nlse.py:216);
 * nlse_gb300.autotune searches these. */
#define NLSE_ROWS_LINE 0
#define NLSE_ROWS_TMA 1
#define NLSE_ROWS_PAIR 2
#define NLSE_ROWS_PAIR8 3 /* NLSE_ROWS_PAIR with 8 positions per thread: twice the threads */
#define NLSE_ROWS_DEEP 4
#define NLSE_COLS_TILE 0
#define NLSE_COLS_TMA 1
#define NLSE_COLS_PAIR 2
#define NLSE_COLS_PAIR8 3 /* NLSE_COLS_PAIR with 8 positions per thread: twice the threads */
#define NLSE_COLS_DEEP 4
int nlse_plan_set_variant(nlse_plan plan, int32_t rows, int32_t cols, int32_t rows_ctas_per_sm,
                          int32_t cols_ctas_per_sm);
int nlse_plan_get_variant(nlse_plan plan, int32_t* rows, int32_t* cols, int32_t* rows_ctas_per_sm,
                          int32_t* cols_ctas_per_sm, uint32_t* rows_avail, uint32_t* cols_avail);

/*
 * Nonlocal response (the reference's oaconvolve(|A|^2, nl_profile, "same")
 * over the transform axes, NLSE/nlse.py:143-155, 406-408, 444-447 and the
 * CNLSE counterparts): give the plan a zero-padded grid pad_y x pad_x (1-D:
 * pad_x only), powers of two at least N + M - 1 - (M-1)/2 per axis for a
 * kernel of M points, so the cyclic convolution equals the linear "same" one.
 * The plan allocates its padded scratch (nfields x pad_y x pad_x) here.
 * pad_x = 0 removes it.  The operator then passes the kernel spectrum in
 * nl_khat; each nonlinear step convolves |A|^2 (both components at once,
 * as the real and imaginary parts) on the project FFT.
 */
int nlse_plan_set_nonlocal(nlse_plan plan, int64_t pad_y, int64_t pad_x);

/*
 * One pass of the split-step sequence that nlse_propagate enqueues, so that
 * a caller can time or compose the kernels one at a time:
 *   NLSE_PASS_FORWARD     forward row pass (after the leading half nonlinear
 *                         step of the "double" scheme)
 *   NLSE_PASS_LINEAR      the strided-axis passes: forward column FFT,
 *                         propagator multiply, inverse column FFT
 *   NLSE_PASS_INV_NL_FWD  inverse row pass, 1/N, nonlinear step (step index
 *                         `step` for the pump), next step's forward row pass
 *   NLSE_PASS_INV_NL      inverse row pass, 1/N, nonlinear step
 * A full step is FORWARD, LINEAR, INV_NL; n fused steps are FORWARD,
 * (LINEAR, INV_NL_FWD) x (n-1), LINEAR, INV_NL.  Split of the loop body of
 * NLSE.split_step (NLSE/nlse.py:372-487).  Not for 1-D plans (whose step is
 * one pass: use nlse_propagate).
 */
#define NLSE_PASS_FORWARD 0
#define NLSE_PASS_LINEAR 1
#define NLSE_PASS_INV_NL_FWD 2
#define NLSE_PASS_INV_NL 3
int nlse_pass(nlse_plan plan, void* A, const nlse_operator* op, int32_t pass, int64_t step,
              void* stream);

/*
 * In-place transform over the plan's axes: forward (inverse = 0) or
 * normalised inverse (inverse = 1), matching VkFFTApp.fft / .ifft with
 * norm=1 (NLSE/nlse.py:435,438).
 */
int nlse_fft(nlse_plan plan, void* A, int32_t inverse, void* stream);

/*
 * Only the nonlinear step (parameter set 0, optional Rabi and pump) applied
 * pointwise to A: kernels_gpu.nl_prop / nl_prop_without_V / nl_prop_c /
 * nl_prop_without_V_c / rabi_coupling (NLSE/kernels_gpu.py:4-156) and
 * DDGPE.laser_excitation (NLSE/ddgpe.py:127-156).  asq: optional
 * [nfields][comps][pixels] real array used as |A|^2 (the reference's A_sq
 * after its nonlocal convolution); NULL computes |A|^2 from A.
 */
int nlse_nonlinear(nlse_plan plan, void* A, const void* asq, const nlse_operator* op,
                   int64_t step, void* stream);

/*
 * Per-segment sum of |A|^2 accumulated in FP64 (the integral of
 * _prepare_output_array, NLSE/nlse.py:293-303, and the callbacks' norms,
 * NLSE/callbacks.py:32-54).  A has nseg segments of seg_len elements; out
 * receives nseg doubles.  workspace: device scratch of at least
 * nlse_power_workspace_size(nseg, seg_len) bytes.
 */
size_t nlse_power_workspace_size(int64_t nseg, int64_t seg_len);
int nlse_power(const void* A, int32_t dtype, int64_t nseg, int64_t seg_len, double* out,
               void* workspace, size_t workspace_bytes, void* stream);

/*
 * nlse_power without a workspace argument, for callers that cannot allocate
 * device memory themselves -- for instance a plugin host whose device memory
 * belongs to another framework's allocator, or code running between the
 * launches of a replayed z-loop that must not allocate.  No counterpart in
 * the reference.  The partial sums go to a static array inside the library
 * (65,536 doubles, 512 KiB, held on every GPU that loads the library until
 * the process exits), so:
 *   - nseg * min(1024, ceil(seg_len / 8192)) must not exceed 65,536; larger
 *     requests return NLSE_ERR_ARG with the numbers in nlse_last_error();
 *   - the first call on a device looks the array's device address up
 *     (cudaGetSymbolAddress), so make that first call before any stream
 *     capture on that device; the address is kept per device and context,
 *     so after a cudaDeviceReset the next call looks it up again (make
 *     that call outside a capture too);
 *   - all calls share the array: calls whose kernels overlap on the GPU
 *     (different streams without ordering between them) race and may
 *     return wrong sums; order them on one stream.
 * Nothing in the array needs clearing between calls: each call writes
 * every partial it reads.  No device memory is allocated or freed.
 */
int nlse_power_noalloc(const void* A, int32_t dtype, int64_t nseg, int64_t seg_len, double* out,
                       void* stream);

/*
 * Power normalisation of _prepare_output_array (NLSE/nlse.py:284-307):
 * out[s] = in[s] * sqrt(target[s] / (sums[s] * coef)), the factor rounded to
 * the field precision.  in may equal out.
 */
int nlse_normalize(const void* in, void* out, int32_t dtype, int64_t nseg, int64_t seg_len,
                   const double* sums, const double* target, double coef, void* stream);

/* Complex Gaussian noise for the two components of DDGPE fields
 * [nfields][2][pix] (replaces DDGPE.add_noise's random draws,
 * NLSE/ddgpe.py:96-125): A[f][k][p] += sigma_k * (x + i y), x, y standard
 * normals from a counter-based generator (Philox4x32-10 keyed by `seed`,
 * counter (p, step)), the same for every field of the batch as the
 * reference's (NY, NX) draw.  Reproducible for a given (seed, step). */
int nlse_add_noise(void* A, int32_t dtype, int64_t nfields, int64_t pix, double sigma0,
                   double sigma1, uint64_t seed, int64_t step, void* stream);

/* Self-test of the bounded waits (no reference counterpart): one CTA waits
 * on an mbarrier that nothing completes, with the loop every wait of the
 * passes uses, and gives up after limit_ns (at most 1 s, the passes' limit).
 * On giving up it stores the device timeout code (1) into *status, as the
 * passes store it into a plan's status word, and the wait's duration into
 * *elapsed_ns (both device pointers).  The context stays usable. */
int nlse_wait_selftest(int32_t* status, uint64_t* elapsed_ns, int64_t limit_ns, void* stream);

/* Nonlinear refractive-index change of the callbacks (NLSE/callbacks.py).
 * The field is nseg segments of pix points; coef, n2abs and isat are device
 * arrays of nseg doubles (one value per segment: per field and component).
 * Evaluated as NumPy evaluates the callbacks' expressions, operation by
 * operation without contraction:
 *   q  = re*re + im*im                          (nlse_delta_n)
 *   q  = re*re + ((im*im*c)*eps0)/2             (nlse_delta_n_max, the
 *        precedence of adapt_delta_z, callbacks.py:109)
 *   dn = (coef * q) / (1 + q / isat)
 * in the field precision, except that flag NLSE_DN_COEF_F64 evaluates
 * coef * q and NLSE_DN_ISAT_F64 evaluates 1 + q / isat in FP64 (parameters
 * NumPy treats as float64 rather than as weak scalars); the quotient is FP64
 * if either is.  c and eps0 are rounded to the field precision. */
#define NLSE_DN_COEF_F64 1
#define NLSE_DN_ISAT_F64 2

/* evaluate_delta_n (NLSE/callbacks.py:57-82): out[s][p] = dn with
 * coef_s = c*eps0/2*n2 (computed by the caller); out is float32 for a
 * complex64 field without flags, float64 otherwise. */
int nlse_delta_n(const void* A, int32_t dtype, int64_t nseg, int64_t pix, const double* coef,
                 const double* isat, int32_t flags, void* out, void* stream);

/* adapt_delta_z's peak (NLSE/callbacks.py:85-112): *out (device double) =
 * max over all points of dn with coef_s = |n2_s|; a NaN anywhere gives NaN,
 * as NumPy's max.  Stream-ordered; the caller reads *out when it needs it. */
int nlse_delta_n_max(const void* A, int32_t dtype, int64_t nseg, int64_t pix, const double* n2abs,
                     const double* isat, double c, double eps0, int32_t flags, double* out,
                     void* stream);

/* |A|^2 into a real array of the field precision (kernels_gpu.square_mod,
 * NLSE/kernels_gpu.py:179-190). */
int nlse_square_mod(const void* A, void* out, int32_t dtype, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NLSE_GB300_H */
