// Host-side launchers shared by the translation units of libnlse_sm103.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "step_kernels.cuh"

namespace nlse {

constexpr int kMinLog2 = 1;   // smallest line: 2 points
constexpr int kMaxLog2 = 12;  // largest line handled by one CTA: 4096 points

// Row passes (contiguous axis).  prepare_only: set kernel attributes, launch
// nothing (done once per device before any stream capture).
cudaError_t launch_rows_f32_c1(int mode, int log2n, const StepArgs& a, cudaStream_t s, bool prepare_only);
cudaError_t launch_rows_f32_c2(int mode, int log2n, const StepArgs& a, cudaStream_t s, bool prepare_only);
cudaError_t launch_rows_f64_c1(int mode, int log2n, const StepArgs& a, cudaStream_t s, bool prepare_only);
cudaError_t launch_rows_f64_c2(int mode, int log2n, const StepArgs& a, cudaStream_t s, bool prepare_only);
// Column passes (strided axis).
cudaError_t launch_cols_f32(int mode, int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only);
cudaError_t launch_cols_f64(int mode, int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only);
// Column passes over the blocked spectral buffer (2-D fast path).
cudaError_t launch_cols_blk_f32(int mode, int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only);
cudaError_t launch_cols_blk_f64(int mode, int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only);

// Pair passes (two complex64 lines per thread, packed FP32; step_pair.cuh):
// the persistent TMA inverse row passes (ROW_INV_NL, ROW_INV_NL_FWD) on the
// blocked buffer, and the blocked column pass.  a.tma_grid / c.tma_grid hold
// the SM count; cap_per_sm > 0 caps the CTAs per SM.  vshared: real
// potential shared by the batch with an even number of fields.
// cudaErrorNotSupported for a size without a pair kernel.
// ep: positions per thread and line, 16 or 8 (twice the threads per line).
// deep (ep 16 only): the deep-prefetch forms, which keep the next work item's
// copies in flight for the whole current item (rows: every exchange in the
// item's own buffer; columns: three staging tiles, no exchange tile).
cudaError_t launch_rows_pair(int mode, int log2n, const StepArgs& a, bool vshared, cudaStream_t s,
                             bool prepare_only, int cap_per_sm, int ep, bool deep = false);
cudaError_t launch_cols_pair(int log2n, const ColArgs& a, cudaStream_t s, bool prepare_only,
                             int cap_per_sm, int ep, bool deep = false);

// One launch per pass over several plans (step_multi.cuh): complex64
// one-component 2-D plans of 256..2048 points per axis with TMA row passes.
// Rows: mode ROW_INV_NL or ROW_INV_NL_FWD, each plan's step arguments (on the
// blocked buffer) and tensor map.  Columns: each plan's blocked column
// arguments.  nsm: SMs of the device.  prepare_only: set kernel attributes.
int multi_max_plans();
// Columns: the blocked column pass of every plan in tile form (one 512-thread
// CTA per 2048/N tiles of a plan, no persistence; k_cols_blk's arithmetic).
cudaError_t launch_cols_tile_multi(int n, const ColArgs* c, const int* log2n, cudaStream_t s,
                                   bool prepare_only);
cudaError_t launch_rows_multi(int mode, int n, const StepArgs* a, const CUtensorMap* const* tm,
                              const int* log2n, int nsm, cudaStream_t s, bool prepare_only);


// Pointwise kernels (pointwise.cu).
int power_chunks(int64_t seg_len);  // partial sums per segment of the power reduction
int64_t noalloc_partials_max();     // capacity of the static partial-sum array
cudaError_t launch_power_noalloc(int dtype, const void* A, int64_t nseg, int64_t seg_len,
                                 double* out, cudaStream_t s);
cudaError_t launch_power(int dtype, const void* A, int64_t nseg, int64_t seg_len, double* partial,
                         int nchunks, double* out, cudaStream_t s);
cudaError_t launch_scale(int dtype, const void* in, void* out, int64_t nseg, int64_t seg_len,
                         const double* sums, const double* target, double coef, cudaStream_t s);
cudaError_t launch_nl_pointwise(int dtype, const StepArgs& a, cudaStream_t s);
cudaError_t launch_abs2(int dtype, const void* A, void* out, int64_t n, cudaStream_t s);
cudaError_t launch_add_noise(int dtype, void* A, int64_t nfields, int64_t pix, double s0, double s1,
                             uint64_t seed, uint32_t step, cudaStream_t s);
cudaError_t launch_params_f32(const double* p, float* q, int64_t n, cudaStream_t s);
// Nonlinear index change of the callbacks (flags: 1 = coef * |A|^2 in FP64,
// 2 = 1 + |A|^2 / isat in FP64); out is float unless a flag is set or the
// field is complex128.  The max variant writes one double to out.
// One CTA waits on an mbarrier nothing completes, giving up after limit_ns.
cudaError_t launch_wait_selftest(int* status, unsigned long long* elapsed_ns,
                                 unsigned long long limit_ns, cudaStream_t s);
cudaError_t launch_delta_n(int dtype, const void* A, int64_t nseg, int64_t pix, const double* coef,
                           const double* isat, int flags, void* out, cudaStream_t s);
cudaError_t launch_delta_n_max(int dtype, const void* A, int64_t nseg, int64_t pix,
                               const double* n2abs, const double* isat, double c, double eps0,
                               int flags, double* out, cudaStream_t s);
// Nonlocal response: pack |A|^2 into the padded scratch, multiply by the
// kernel spectrum, nonlinear step reading the convolved intensities.
cudaError_t launch_pack_asq(int dtype, int nc, const void* A, void* X, int64_t nfields, int64_t ny,
                            int64_t nx, int64_t py, int64_t px, cudaStream_t s);
// Fused row passes of the nonlocal convolution (nonlocal_rows.cu): whether
// they apply, |A|^2 packing + forward rows, inverse rows + the nonlinear step.
bool nonlocal_rows_fused(int dtype, int log2px, int64_t ny, int64_t py);
cudaError_t launch_pack_rows_fwd(int log2px, int nc, const void* A, void* X, int64_t nfields,
                                 int64_t ny, int64_t nx, int64_t py, const void* tw,
                                 cudaStream_t s);
cudaError_t launch_rows_inv_nl_pad(int log2px, const StepArgs& a, const void* X, int64_t ny,
                                   int64_t nx, int64_t py, int set, float inv_n, cudaStream_t s);
cudaError_t launch_mul_spectrum(int dtype, void* X, const void* K, int64_t per, int64_t total,
                                cudaStream_t s);
cudaError_t launch_nl_pointwise_pad(int dtype, const StepArgs& a, const void* X, int64_t ny,
                                    int64_t nx, int64_t py, int64_t px, int set, cudaStream_t s);
// Blocked copy of the propagator, scaled by 1/(ny nx) (exact: a power of two).
cudaError_t launch_prop_to_blk(int prop_c128, const void* nat, void* blk, int64_t comps, int64_t ny,
                               int64_t nx, int w, cudaStream_t s);

}  // namespace nlse
