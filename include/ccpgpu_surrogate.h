/* C ABI of the contact-map surrogate: a sequence-to-contact-map network
 * trained on maps that the batched engine (ccpgpu.h) simulates, with its
 * own BF16 tensor-core (tcgen05) training and inference kernels on sm_103a.
 *
 * The reference has no counterpart to any function here: ccp only simulates
 * (Program/src/chrsim.cu) and analyses (Program/src/chrana.cu) contact maps.
 * The map the network predicts is the probability counterpart of ccp's
 * binned contact map (calc_cm, Program/src/chrana.cu:48-84): for bins I, J of
 * `bead_count / bins` consecutive beads, the fraction of frames x bead pairs
 * (i in I, j in J, i != j) closer than the contact cutoff.
 *
 * Network (all sizes from the configuration text, defaults in brackets):
 *   input     per bead: A / B type and LAD flag, zero-padded to 64 channels
 *   encoder   enc_layers [8] 1-D convolutions, width 128, kernel enc_kernel [5];
 *             the first maps 64 -> 128 channels, the rest are residual
 *             (h += relu(conv(h) + b))
 *   pooling   mean over seq_len / bins consecutive beads
 *   pairs     u, v = 1x1 projection (128 -> 64 + 64); z0[i][j] = u_i v_j +
 *             u_j v_i + E[|i - j|] (E learned, bins x 64)
 *   head      head_layers [6] residual 3x3 convolutions, width 64, dilations
 *             [1,2,4,8,1,2]
 *   output    y = w . z + b; yhat = (y + y^T) / 2 predicts log p, the map is
 *             exp(min(yhat, 0)); the loss gradient passes the clamp unchanged
 * Loss: the Poisson deviance of the observed probability p against exp(yhat),
 * w[s] (exp(yhat) - p - p (yhat - log p)) averaged over all values, weighted
 * per separation s = |i - j| by w[s] = bins / (P(s) x pairs(s)), P(s) the
 * dataset's mean contact probability at s (floored at 1e-6) and pairs(s) the
 * bin pairs at s, so that every separation carries the same weight. Optimiser:
 * AdamW (lr [1e-3], beta1 [0.9], beta2 [0.999], adam_eps [1e-8],
 * weight_decay [0.01] on weight matrices) after the gradient is clipped to a
 * global L2 norm of clip_norm [1] (0: no clip); with lr_steps > 0 the
 * learning rate decays from lr to lr_min [0] along a half cosine over the
 * first lr_steps steps and stays at lr_min after. The output weights start at
 * zero and the output bias at the log of the dataset's mean contact
 * probability. Weights are FP32 masters with BF16
 * copies; activations BF16; every contraction accumulates in FP32.
 *
 * Status codes and ccpgpu_last_error() are those of ccpgpu.h. A handle owns
 * one CUDA stream and all its device memory; calls on one handle are not
 * thread-safe. */
#ifndef CCPGPU_SURROGATE_H
#define CCPGPU_SURROGATE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ccpsur_net ccpsur_net;

typedef struct ccpsur_info {
  int32_t seq_len, bins, batch;
  int32_t enc_layers, enc_width, enc_kernel;
  int32_t head_layers, head_width;
  int32_t dataset_size;
  int64_t n_params;
  int64_t step; /* optimiser steps taken */
} ccpsur_info;

/* Builds the network. config_text: whitespace-separated "key value" pairs
 * (keys above plus seq_len [1024], bins [256], batch [32]); seq_len and bins
 * are multiples of 128 and bins divides seq_len. Weights are initialised from
 * `seed`. */
int ccpsur_create(const char *config_text, uint64_t seed, ccpsur_net **out);
int ccpsur_destroy(ccpsur_net *h);
int ccpsur_info_get(const ccpsur_net *h, ccpsur_info *out);

/* FP32 master parameters and the gradients of the last ccpsur_loss_grad /
 * ccpsur_train_step, as one flat vector: per encoder layer W [taps][128][cin]
 * then b [128] (cin = 64 for the first layer, 128 after), the projection W
 * [1][128][128] and b [128], E [bins][64], per head layer W [9][64][64] and
 * b [64], then w_out [64] and b_out [1]. Setting the parameters keeps the
 * optimiser state. */
int ccpsur_get_params(ccpsur_net *h, float *out, int64_t n);
int ccpsur_set_params(ccpsur_net *h, const float *in, int64_t n);
int ccpsur_get_grads(ccpsur_net *h, float *out, int64_t n);

/* Training set, copied to the device: types [n][seq_len] (0 = A, 1 = B), lad
 * [n][seq_len] (nonzero = LAD bead, may be NULL), maps [n][bins][bins]
 * contact probabilities in [0, 1] (symmetric). Sets the separation weights of
 * the loss and, before the first optimiser step, starts the output bias at
 * the log of the mean contact probability. */
int ccpsur_set_dataset(ccpsur_net *h, const uint8_t *types, const uint8_t *lad, const float *maps,
                       int32_t n);

/* Forward + backward on dataset rows `rows[0..n)` (n <= batch): the loss and
 * the gradients, no update. */
int ccpsur_loss_grad(ccpsur_net *h, const int32_t *rows, int32_t n, double *loss);

/* Forward + backward + one AdamW update. loss may be NULL (no synchronisation). */
int ccpsur_train_step(ccpsur_net *h, const int32_t *rows, int32_t n, double *loss);

/* Predicted contact-probability maps [n][bins][bins] for n sequences given in
 * host memory (any n; processed in batches). */
int ccpsur_predict(ccpsur_net *h, const uint8_t *types, const uint8_t *lad, int32_t n, float *maps);

/* The contact probability by bin separation of the predicted maps,
 * ps[n][bins] (ps[k][s] = the mean of the map's diagonal s), reduced on the
 * device: what screening needs, without copying every map to the host. */
int ccpsur_predict_ps(ccpsur_net *h, const uint8_t *types, const uint8_t *lad, int32_t n, float *ps);

/* The same for dataset rows; maps may be NULL (the result stays on the
 * device, for timing). */
int ccpsur_predict_rows(ccpsur_net *h, const int32_t *rows, int32_t n, float *maps);

int ccpsur_synchronize(ccpsur_net *h);
/* The handle's cudaStream_t. */
int ccpsur_stream_handle(ccpsur_net *h, void **stream);
/* Bit 0: a convolution kernel gave up waiting; bit 1: a weight-gradient
 * kernel did. Reading clears them. */
int ccpsur_error_flags(ccpsur_net *h, int32_t *flags);
/* Kernels launched by this handle so far. */
int ccpsur_kernel_count(const ccpsur_net *h, int64_t *n);

/* Single layers on host buffers (BF16 passed as uint16 bit patterns),
 * allocating device memory per call; for tests and for callers that want the
 * tensor-core convolution alone. Images are channels-last [B][H][W][C] with
 * W a multiple of 128 and C in {64, 128}; taps: (dh[t], dw[t]) input offsets.
 * conv: out[p][co] = bf16(relu?(sum_t,ci x[p + off_t][ci] w[t][co][ci] +
 * bias[co]) + resid[p][co]); bias, resid and mask_out (bits of acc + bias >
 * 0, [P][cout / 32]) may be NULL. */
int ccpsur_conv_bf16(int32_t B, int32_t H, int32_t W, int32_t cin, int32_t cout, int32_t ntaps,
                     const int32_t *dh, const int32_t *dw, const uint16_t *x, const uint16_t *w,
                     const float *bias, int32_t relu, const uint16_t *resid, uint16_t *out,
                     uint32_t *mask_out);
/* dw_out[t][co][ci] = sum_p x[p + off_t][ci] dy[p][co]; db_out[co] = sum_p
 * dy[p][co] (may be NULL). FP32 results. */
int ccpsur_wgrad_bf16(int32_t B, int32_t H, int32_t W, int32_t cin, int32_t cout, int32_t ntaps,
                      const int32_t *dh, const int32_t *dw, const uint16_t *x, const uint16_t *dy,
                      float *dw_out, float *db_out);

#ifdef __cplusplus
}
#endif

#endif /* CCPGPU_SURROGATE_H */
