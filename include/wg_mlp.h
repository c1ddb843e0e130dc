/* wg_mlp.h -- C ABI of the calibration-step network (libwg_gpu.so).
 *
 * No counterpart in the reference: its calibration (calibGammaClass::findNewGamma,
 * source/calibration.cpp:266-636) only bisects.  This network proposes a step of
 * (gamma, correction factor) from basin summaries; the plain model checks every
 * proposal.  It is a 4-layer MLP of width 128 -- inputs zero-padded to 128
 * features, ReLU hidden layers, 16 outputs of which the caller uses the first
 * out_dim -- with BF16 weights and activations and FP32 accumulation; forward
 * and backward passes run on the tensor cores (tcgen05), training is Adam on
 * FP32 master weights.
 *
 * Parameter vector (FP32), in this order: W0 [128][128], b0 [128], W1 [128][128],
 * b1 [128], W2 [128][128], b2 [128], W3 [16][128], b3 [16]; W as [out][in].
 * Host arrays throughout: x [n][128], targets [n][out_dim], outputs [n][16]. */
#ifndef WG_MLP_H
#define WG_MLP_H

#include <stdint.h>

#include "wg_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wg_mlp wg_mlp;

#define WG_MLP_IN 128
#define WG_MLP_OUT 16

int32_t wg_mlp_num_params(void);
/* Parameters drawn with the given seed (He-uniform weights, zero biases). */
wg_status wg_mlp_create(int32_t device, uint64_t seed, wg_mlp **out);
wg_status wg_mlp_destroy(wg_mlp *m);
wg_status wg_mlp_set_params(wg_mlp *m, const float *theta);
wg_status wg_mlp_get_params(wg_mlp *m, float *theta);
/* y [n][16] = network(x [n][128]) */
wg_status wg_mlp_forward(wg_mlp *m, const float *x, int32_t n, float *y);
/* Gradient of loss = sum over samples and the first out_dim outputs of
 * (y - target)^2 / n, for the n samples in one pass (grad: num_params floats). */
wg_status wg_mlp_gradient(wg_mlp *m, const float *x, const float *target, int32_t out_dim, int32_t n, float *grad,
                          float *loss);
/* Adam training on the n samples: `epochs` passes in shuffled minibatches of
 * `batch` (a multiple of 128), learning rate lr; the mean loss of the last
 * epoch in *final_loss. */
wg_status wg_mlp_train(wg_mlp *m, const float *x, const float *target, int32_t out_dim, int32_t n, int32_t epochs,
                       int32_t batch, float lr, uint64_t seed, float *final_loss);

#ifdef __cplusplus
}
#endif

#endif
