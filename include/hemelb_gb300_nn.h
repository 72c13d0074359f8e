/*
 * hemelb_gb300_nn.h -- BF16 tensor-core kernels of the warm-start surrogate.
 *
 * No counterpart in the reference (HemeLB has no learned component); these are the
 * building blocks of a 3-D convolutional U-Net that predicts velocity and pressure
 * from geometry features, trained and run on the GPU.  All pointers are device
 * pointers owned by the caller; tensors are channels-last (N, D, H, W, C), BF16
 * activations, weights [taps][C_out][C_in] BF16 (C_in fastest) with FP32 master
 * copies and FP32 gradients.  Every call enqueues on `stream` and returns 0 on
 * success, 1 for bad arguments, 3 for a launch error.
 */
#ifndef HEMELB_GB300_NN_H
#define HEMELB_GB300_NN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out = act(conv(in, w) + bias); taps 27 (3x3x3, zero padding) or 1 (1x1x1);
 * cin a multiple of 16; relu 0/1; out_f32 optional FP32 copy of the output. */
int hlbg_nn_conv3d(const void *in, int32_t cin, const void *w, const float *bias, void *out,
                   float *out_f32, int32_t cout, int32_t n, int32_t d, int32_t h, int32_t wd,
                   int32_t taps, int32_t relu, void *stream);
/* The same convolution on the fifth-generation tensor cores (tcgen05.mma, FP32
 * accumulator in tensor memory, TMA-staged operands): cin a multiple of 16, cout
 * a multiple of 16 up to 256, taps 27 or 1; in, w, out, out_f32 16-byte aligned.
 * Returns 1 for shapes it does not take (hlbg_nn_conv3d takes every shape). */
int hlbg_nn_conv3d_tc(const void *in, int32_t cin, const void *w, const float *bias, void *out,
                      float *out_f32, int32_t cout, int32_t n, int32_t d, int32_t h, int32_t wd,
                      int32_t taps, int32_t relu, void *stream);
/* Nonzero when a bounded wait of a tcgen05 convolution gave up since the last
 * reset (reset != 0 clears it); synchronous. */
int hlbg_nn_tc_error(int32_t reset);
/* dw[tap][co][ci] += sum over voxels of dy[m, co] * x[m + off(tap), ci] (FP32) */
int hlbg_nn_conv3d_wgrad(const void *x, int32_t cin, const void *dy, int32_t cout, float *dw,
                         int32_t n, int32_t d, int32_t h, int32_t wd, int32_t taps, void *stream);
/* wt[taps-1-tap][ci][co] = w[tap][co][ci]: weights of the data-gradient convolution */
int hlbg_nn_flip_transpose(const void *w, void *wt, int32_t cout, int32_t cin, int32_t taps,
                           void *stream);
int hlbg_nn_relu_bwd(void *dy, const void *y, int64_t n, void *stream);
int hlbg_nn_bias_grad(const void *dy, float *db, int64_t m, int32_t c, void *stream);
/* 2x average pooling; backward: x = dy (coarse), y = dx (fine), sizes fine */
int hlbg_nn_pool2(const void *x, void *y, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c,
                  int32_t backward, void *stream);
/* nearest 2x upsampling; forward sizes fine, backward: x = dy (fine), y = dx, sizes coarse */
int hlbg_nn_up2(const void *x, void *y, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c,
                int32_t backward, void *stream);
int hlbg_nn_concat(const void *a, int32_t ca, const void *b, int32_t cb, void *y, int64_t m,
                   void *stream);
int hlbg_nn_split(const void *y, void *da, int32_t ca, void *db, int32_t cb, int64_t m,
                  int32_t accumulate_b, void *stream);
int hlbg_nn_add(void *a, const void *b, int64_t n, void *stream);
/* masked MSE: loss += sum (mask (pred - target))^2, dpred = 2 mask (pred - target) * inv_count */
int hlbg_nn_mse(const float *pred, const float *target, const float *mask, void *dpred, float *loss,
                int64_t m, int32_t c, float inv_count, void *stream);
/* Adam step `step` (1-based) on FP32 weights, refreshing the BF16 copy wb (may be NULL) */
int hlbg_nn_adam(float *w, void *wb, const float *g, float *m, float *v, int64_t n, float lr,
                 float b1, float b2, float eps, int32_t step, void *stream);
int hlbg_nn_to_bf16(const float *x, void *y, int64_t n, void *stream);

#ifdef __cplusplus
}
#endif
#endif
