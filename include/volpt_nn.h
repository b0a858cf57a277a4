/*
 * volpt_nn.h — operators of the learned denoiser (libvolpt.so).
 *
 * No counterpart in the reference, whose denoisers are the a-trous filter and
 * OIDN: a U-Net on colour, albedo and normal, trained by these operators on
 * pairs of low- and high-path-count renders of the path tracer itself
 * (volview_gb300/learned_denoiser.py composes them).
 *
 * Tensors are device pointers in NHWC order (pixel-major, channels innermost)
 * of FP16 values; weights are FP16 [cout][3][3][cin], biases and gradients
 * FP32. Convolutions are 3x3 with zero padding (same size) and need widths
 * that are multiples of 16 and input channel counts that are multiples of 16.
 * `stream` is a cudaStream_t (NULL: the legacy default stream). Every call is
 * asynchronous; VV_ERR_ARG reports a shape the operators do not take.
 */
#ifndef VOLPT_NN_H
#define VOLPT_NN_H

#include <stddef.h>

#include "volpt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* y = act(conv3x3(x, weights) + bias), act = ReLU if relu else identity; bias
 * may be NULL. cout is one of 8, 16, 32, 48, 64, 80, 96, 112, 144, 176.
 * Widths that are multiples of 128 with cout <= 96 and small enough weights
 * and inputs run on tcgen05 (vv_nn_conv3x3_tc), the rest on mma.sync. */
vv_status vv_nn_conv3x3(const void* x, int n, int h, int w, int cin, const void* weights, const float* bias,
                        int cout, int relu, void* y, void* stream);
/* wt[ci][8 - tap][co] = weights[co][tap][ci]: with them vv_nn_conv3x3 of dy
 * gives dx, the gradient of a convolution's input. */
vv_status vv_nn_flip_weights(const void* weights, int cout, int cin, void* wt, void* stream);
/* dw[co][tap][ci] += sum over pixels of dy[p][co] * x[p + tap][ci] (FP32). */
vv_status vv_nn_conv3x3_wgrad(const void* x, const void* dy, int n, int h, int w, int cin, int cout, float* dw,
                              void* stream);
/* db[c] += sum over pixels of dy[p][c]. */
vv_status vv_nn_bias_grad(const void* dy, long pixels, int c, float* db, void* stream);
/* dy = 0 where y <= 0 (the gradient through a ReLU whose output is y). */
vv_status vv_nn_relu_backward(void* dy, const void* y, long count, void* stream);
/* 2x2 average pooling of x (n, h, w, c) into y (n, h/2, w/2, c); with
 * backward, x is the gradient of the pooled (n, h/2, w/2, c) tensor and y
 * receives that of the (n, h, w, c) input. */
vv_status vv_nn_avgpool2(const void* x, int n, int h, int w, int c, void* y, int backward, void* stream);
/* Nearest 2x upsampling of x (n, h, w, c) into y (n, 2h, 2w, c); with
 * backward, x is the gradient of the upsampled tensor and y that of the
 * (n, h, w, c) input (sums of 2x2). */
vv_status vv_nn_upsample2(const void* x, int n, int h, int w, int c, void* y, int backward, void* stream);
/* y[p] = a[p] (ca channels) followed by b[p] (cb channels). */
vv_status vv_nn_concat(const void* a, int ca, const void* b, int cb, long pixels, void* y, void* stream);
/* y (n, 2h, 2w, ca + cb) = vv_nn_upsample2 of a (n, h, w, ca) followed by b
 * (n, 2h, 2w, cb), channel-wise, in one pass (the decoder's input): ca and cb
 * multiples of 8, a, b and y 16-byte aligned; VV_ERR_ARG otherwise (then
 * vv_nn_upsample2 and vv_nn_concat give the same tensor). */
vv_status vv_nn_upsample_concat(const void* a, int n, int h, int w, int ca, const void* b, int cb, void* y,
                                void* stream);
/* The gradient of vv_nn_concat: da, db (either may be NULL) from dy. */
vv_status vv_nn_split(const void* dy, int ca, int cb, long pixels, void* da, void* db, void* stream);
/* The network's 16-channel input from an accumulation of n paths per pixel
 * (RGBA32F sums as vv_read_accumulation gives them, device pointers):
 * log(1 + radiance), albedo, normal, then zeros. */
vv_status vv_nn_features(const float* accum, const float* albedo, const float* normal, float n, long pixels,
                         void* x, void* stream);
/* loss += mean |pred - target| over the first 3 of c channels (target: 3
 * floats per pixel, log(1 + radiance)); dpred = its gradient times
 * grad_scale (c channels), the scale keeping FP16 gradients normal. */
vv_status vv_nn_l1_loss(const void* pred, int c, const float* target, long pixels, float grad_scale,
                        float* loss, void* dpred, void* stream);
/* One Adam step (Kingma and Ba; step counts from 1) on FP32 weights w with
 * moments m, v, for the gradient grad / grad_scale; w16 (may be NULL)
 * receives the FP16 copy. */
vv_status vv_nn_adam(float* w, void* w16, const float* grad, float* m, float* v, long count, float lr,
                     float beta1, float beta2, float eps, float grad_scale, int step, void* stream);
/* y += x (FP16 tensors of count values). */
vv_status vv_nn_add(void* y, const void* x, long count, void* stream);
/* The same input over a padded wp x hp image (zeros outside w x h) from
 * pixel-linear w x h accumulation images. */
vv_status vv_nn_features_image(const float* accum, const float* albedo, const float* normal, float n, int w, int h,
                               int wp, int hp, void* x, void* stream);
/* The HDR store (RGBA16F, w x h) of a prediction over a padded width wp:
 * exp(max(pred, 0)) - 1 of its first 3 channels, coverage accum.w / n. */
vv_status vv_nn_prediction_to_hdr(const void* pred, int c, int wp, int w, int h, const float* accum, float n,
                                  void* hdr, void* stream);
/* rgb = exp(max(pred, 0)) - 1 of the first 3 of c channels (3 floats per pixel). */
vv_status vv_nn_radiance(const void* pred, int c, long pixels, float* rgb, void* stream);
/* vv_nn_conv3x3 on tcgen05.mma with TMEM accumulators and TMA-fed inputs:
 * widths that are multiples of 128, cout a multiple of 8 up to 96, all nine
 * taps' weights plus two 128-pixel segments' input rows within 220 KB of
 * shared memory, 16-byte aligned pointers; VV_ERR_ARG for other shapes. */
vv_status vv_nn_conv3x3_tc(const void* x, int n, int h, int w, int cin, const void* weights, const float* bias,
                           int cout, int relu, void* y, void* stream);
/* Whether a tensor-core convolution gave up a bounded wait (1) since the last
 * clear; clear resets the flag. */
vv_status vv_nn_tc_status(int* failed, int clear);

#ifdef __cplusplus
}
#endif

#endif /* VOLPT_NN_H */
