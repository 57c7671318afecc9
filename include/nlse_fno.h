/* nlse_fno.h - C ABI of the Fourier-neural-operator surrogate kernels of
 * libnlse_sm103.so (sm_103a).
 *
 * No reference counterpart: the surrogate is new to this project.  It predicts
 * the output field E(z = L) of the 2-D NLSE split-step solver on a 256 x 256
 * grid from the input field, the potential and two scalar parameters; the
 * solver (nlse_propagate, nlse_gb300.h) generates its training pairs and is
 * its fallback.
 *
 * Model: lift (5 -> 32 channels), four layers
 *   z = h . Wc + (1/N^2) Re(F_R^-1 [F_R h . W]) + b,  h' = GELU(z) (plain z in
 *   the last layer), then a projection 32 -> 2 (Re, Im of the output field).
 * F_R: the 2-D DFT restricted to kx in [0, 32), ky in [0, 32) u [224, 256)
 * (NLSE_FNO_MODES modes); W: per-mode 32 x 32 complex weights.
 * Storage: activations h, z are BF16 [field][y][x][channel]; spectral rows T/U
 * are complex64 [field][y][kx][channel] (32 x 32 per row); mode-major arrays
 * Y/Hs are complex64 [mode][field][channel]; X is the BF16 mixing operand,
 * (ceil(fields/128) tiles of 128 x 64 per mode) in the tensor-core layout.
 *
 * All pointers are device pointers; every call is asynchronous on `stream`
 * and returns 0 or a negative NLSE_ERR_* code (nlse_last_error() explains).
 * `status` is a device int that a kernel sets to 1 if a bounded wait for its
 * tensor-core work gave up.
 */
#ifndef NLSE_FNO_H
#define NLSE_FNO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NLSE_FNO_N 256            /* grid side */
#define NLSE_FNO_C 32             /* channels */
#define NLSE_FNO_MODES 2048       /* retained modes (64 ky x 32 kx), index iy*32 + kx */
#define NLSE_FNO_PART_LAYER 1056  /* per-row partials of a layer: dWc [32][32], db [32] */
#define NLSE_FNO_PART_PROJ 66     /* per-row partials of the projection: dWp [32][2], dbp [2] */
#define NLSE_FNO_PART_LIFT 192    /* per-row partials of the lift (see nlse_fno_lift_bwd) */

/* h0 = bf16(lift(xin, xs)) and the first row analysis T (on tensor cores:
 * BF16 cos/sin over quarter rows, exact quarter-turn rotations, FP32 sums).
 * xin [nb][256][256][3] float (Re E0, Im E0, V); xs [nb][2] float;
 * wl [5][32], bl [32] float. */
int nlse_fno_lift_rows(int64_t nb, const float* xin, const float* xs, const float* wl,
                       const float* bl, void* h0, void* T, int32_t* status, void* stream);

/* Column transforms of T keeping the retained ky, times `scale`: the BF16
 * mixing operand Xc and (optional) Hs [mode][field][32] complex64, holding the
 * BF16-rounded values when round_saved != 0. */
int nlse_fno_cols_analysis(int64_t nb, const void* T, float scale, int32_t round_saved, void* Xc,
                           void* Hs, void* stream);

/* Per-mode complex mixing on tensor cores: Y[m] = X[m] . Wbig[m] with Wbig a
 * packed weight set (nlse_fno_pack_spectral: forward, or conjugate-transposed
 * for the backward pass).  Y [mode][field][32] complex64. */
int nlse_fno_mix(int64_t nb, const void* Xc, const void* wbig, void* Y, int32_t* status,
                 void* stream);

/* Zero-filled inverse column transforms of Y to the row half spectra U. */
int nlse_fno_cols_synthesis(int64_t nb, const void* Y, void* U, void* stream);

/* One layer's row pass: s = row synthesis of U, z = h . Wc + s + bias (the
 * 1 x 1 convolution and the synthesis both on tensor cores, the synthesis with
 * BF16 cos/sin and bf16(U / 256^2), FP32 sums; Tn's analysis as in
 * nlse_fno_lift_rows), hn = bf16(GELU(z)) if act else bf16(z); stores
 * z (optional), hn (optional) and the next layer's row analysis Tn (optional);
 * with out != NULL also the projection out = hn . wp + bp ([nb][256][256]
 * complex64).  wconv: nlse_fno_pack_conv's forward operand. */
int nlse_fno_layer_rows(int64_t nb, const void* U, const void* h, const void* wconv,
                        const float* bias, int32_t act, void* z, void* hn, void* Tn,
                        const float* wp, const float* bp, void* out, int32_t* status,
                        void* stream);

/* Backward of the projection: dh4 = dout . wp^T (float [nb][256][256][32]);
 * part [nb*256][NLSE_FNO_PART_PROJ] per-row partial gradients. */
int nlse_fno_proj_bwd(int64_t nb, const void* dout, const float* wp, const void* h4, float* dh4,
                      float* part, void* stream);

/* Backward of one layer: dh = dhc_in + synthesis(Uin) (Uin optional),
 * dz = dh * GELU'(z) (act) or dh; dhc_out = dz . Wc^T (tensor cores, float);
 * Tg = row analysis of dz; part [nb*256][NLSE_FNO_PART_LAYER] per-row
 * partials of dWc and db.  wconv_bwd: nlse_fno_pack_conv's backward operand. */
int nlse_fno_layer_rows_bwd(int64_t nb, const float* dhc_in, const void* Uin, const void* z,
                            int32_t act, const void* h, const void* wconv_bwd, float* dhc_out,
                            void* Tg, float* part, int32_t* status, void* stream);

/* Backward of the lift: dh0 = dhc_in + synthesis(Uin); per-row partials
 * [0,96) dWl rows 0-2, [96,128) and [128,160) dWl rows 3-4, [160,192) dbl. */
int nlse_fno_lift_bwd(int64_t nb, const float* dhc_in, const void* Uin, const float* xin,
                      const float* xs, float* part, void* stream);

/* Spectral weight gradient gW[m][c][o] = sum_fields conj(Hs[m][f][c]) Gs[m][f][o]. */
int nlse_fno_mix_wgrad(int64_t nb, const void* Hs, const void* Gs, void* gW, void* stream);

/* out[w] = sum_r part[r][w] (w < width). */
int nlse_fno_reduce(const float* part, int64_t rows, int64_t width, float* out, void* stream);

/* BF16 tensor-core operands of the spectral weights W [mode][32][32]
 * complex64: wf (forward) and wb (backward), NLSE_FNO_MODES x 64 x 64 each. */
int nlse_fno_pack_spectral(const void* W, void* wf, void* wb, void* stream);

/* BF16 operands of a 1 x 1 convolution wc [32][32] float (in x out). */
int nlse_fno_pack_conv(const float* wc, void* wf, void* wb, void* stream);

/* stats [nb][2] = (||out-tgt||^2, ||ref||^2) per field (ref = NULL: tgt); with
 * dout != NULL the gradient of mean_f ||out-tgt||^2 / ||ref||^2 (complex64
 * [nb][256][256]). */
int nlse_fno_loss(int64_t nb, const void* out, const void* tgt, const void* ref, float* stats,
                  void* dout, void* stream);

/* Adam step (FP32) with decoupled weight decay wd. */
int nlse_fno_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1,
                  float b2, float eps, int32_t step, float wd, void* stream);

/* Self-test of the tensor-core path: C (128 x n, float) = A (128 x k, BF16
 * row-major) . B (n x k, BF16 row-major)^T, n, k in {32, 64}. */
int nlse_fno_gemm_selftest(const void* A, const void* B, void* C, int32_t n, int32_t k,
                           int32_t* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NLSE_FNO_H */
