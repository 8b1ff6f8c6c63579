/*
 * lh_srnet.h -- BF16 tensor-core kernels of the learned warm start.
 *
 * No counterpart in the reference: its initial conditions are a restart file
 * or a parabolic profile (start.f90:1488-1784, getini and
 * mblock_ini_parabolic_profile).  These entry points are the building blocks
 * of a 3D convolutional super-resolution network that lifts a coarse-grid
 * field onto the fine grid; the network itself (layers, training loop) is
 * composed by the caller.
 *
 * Conventions (all pointers are DEVICE pointers, `stream` a cudaStream_t or
 * NULL for the default stream; calls are asynchronous on that stream):
 *   - activations are channels-last volumes [Y][Z][X][C] of bf16, C = 16 or
 *     32, X and Z periodic (the Fourier directions), Y zero-padded; X must be
 *     a multiple of 32 and Z a multiple of 8, and every activation pointer
 *     16-byte aligned;
 *   - a 3x3x3 convolution's weights are bf16 [27][Cout][Cin], tap index
 *     (dy+1)*9 + (dz+1)*3 + (dx+1) for the neighbour offset (dy, dz, dx);
 *   - return 0 or a negative LH_E* code of littleharsh.h; the reason of a
 *     failure is in lh_last_error(NULL).
 */
#ifndef LH_SRNET_H
#define LH_SRNET_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Flags of lh_sr_conv_fwd's epilogue, applied in this order. */
#define LH_SR_BIAS 8 /* + bias[co] (fp32)                              */
#define LH_SR_RELU 1 /* max(., 0)                                      */
#define LH_SR_GATE 4 /* 0 where gate[v][co] <= 0 (the ReLU derivative) */
#define LH_SR_RES 2  /* + res[v][co] (bf16, Cout channels)             */

/* out[v][co] = epilogue(sum over taps and ci of w[tap][co][ci] * in[v + offset(tap)][ci]).
 * (cin, cout) in {(16,32), (32,32), (32,16)}; out is bf16, or fp32 when out_f32
 * is set (only for (32,16)). */
int lh_sr_conv_fwd(int32_t cin, int32_t cout, const void* in, const void* w, const float* bias, void* out,
                   int32_t out_f32, const void* res, const void* gate, int32_t flags, int32_t X, int32_t Y, int32_t Z,
                   void* stream);

/* The same convolution on the tcgen05 tensor cores (TMEM accumulators, one
 * elected thread issuing the MMAs, producer warps staging the halos of the
 * next y offsets into a ring of buffers while the MMAs read the current one,
 * ordered by mbarriers); Z must also be a multiple of 8.  If an mbarrier wait
 * runs out, the CTA stops and records it for lh_sr_tc_status. */
int lh_sr_conv_fwd_tc(int32_t cin, int32_t cout, const void* in, const void* w, const float* bias, void* out,
                      int32_t out_f32, const void* res, const void* gate, int32_t flags, int32_t X, int32_t Y,
                      int32_t Z, void* stream);

/* Synchronous: *timed_out = 1 if a tcgen05 convolution gave up waiting since
 * the last call (and clears the record). */
int lh_sr_tc_status(int32_t* timed_out);

/* dw[tap][co][ci] += sum_v dout[v][co] * in[v + offset(tap)][ci]; db[co] += sum_v dout[v][co].
 * dw, db fp32 (accumulated into: zero them first). */
int lh_sr_conv_wgrad(int32_t cin, int32_t cout, const void* in, const void* dout, float* dw, float* db, int32_t X,
                     int32_t Y, int32_t Z, void* stream);

/* The same weight and bias gradients on the tcgen05 tensor cores: MMAs whose
 * reduction runs over 16 z voxels, both operands read as they lie in memory
 * (MN-major shared-memory layouts), fp32 accumulators in TMEM for the whole
 * persistent CTA, added to dw once.  Z must also be a multiple of 16.  A wait
 * that runs out is recorded for lh_sr_tc_status. */
int lh_sr_conv_wgrad_tc(int32_t cin, int32_t cout, const void* in, const void* dout, float* dw, float* db,
                        int32_t X, int32_t Y, int32_t Z, void* stream);

/* wt[tap][ci][co] = w[26 - tap][co][ci]: with these weights lh_sr_conv_fwd(cout, cin, ...)
 * computes the data gradient of the convolution. */
int lh_sr_flip_weights(int32_t cin, int32_t cout, const void* w, void* wt, void* stream);

/* Loss of one sample.  corr: fp32 [nvox][16] (channels 0..2 used), base and
 * target fp32 [nvox][3].  loss += sum((base + corr - target)^2) / (3 nvox);
 * dcorr (bf16 [nvox][16]) = its gradient with respect to corr. */
int lh_sr_mse(const float* corr, const float* base, const float* target, void* dcorr, double* loss, int64_t nvox,
              void* stream);

/* One AdamW update of n fp32 parameters (step >= 1); p_bf16, if not NULL,
 * receives the updated parameters rounded to bf16. */
int lh_sr_adam(float* p, const float* g, float* m, float* v, void* p_bf16, int32_t n, float lr, float beta1,
               float beta2, float eps, float weight_decay, int32_t step, void* stream);

#ifdef __cplusplus
}
#endif
#endif
