/* Learned detector importance on one GB300: a BF16 network trained and evaluated by
 * hand-written tcgen05 kernels (libmonki_cuda.so, csrc/mlp.cu).
 *
 * No reference counterpart: the reference's transport is analog only. The network maps a
 * cell's features (at most 64 per row, float32, row-major) to the log of its detector
 * importance; its prediction becomes the per-cell roulette scale of guided transport
 * (monki_cuda_set_roulette_scale in monki_cuda.h).
 *
 * Network: features (zero-padded to 64) -> 256 -> 256 -> 256 -> 1, GELU after each hidden
 * layer; BF16 weights and activations, FP32 accumulation; FP32 master parameters updated
 * by Adam (beta1 0.9, beta2 0.999, epsilon 1e-8). Parameter vector (FP32, count from
 * monki_mlp_param_count): W1[256 x 64], b1[256], W2[256 x 256], b2[256], W3[256 x 256],
 * b3[256], w4[256], b4[1], all row-major.
 *
 * Every call returns 0 on success, or nonzero with a message in err (NULL handle from
 * create). One caller per network; not thread-safe. */
#ifndef MONKI_MLP_H
#define MONKI_MLP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

size_t monki_mlp_param_count(void);

/* A network for rows-per-pass <= rows (training minibatch and inference pass), on an
 * sm_103 device; parameters start at zero. */
void *monki_mlp_create(uint32_t device, uint32_t features, uint32_t rows, uint32_t seed, char *err, size_t errlen);

int monki_mlp_set_params(void *net, const float *params, size_t count, char *err, size_t errlen);
int monki_mlp_get_params(void *net, float *params, size_t count, char *err, size_t errlen);

/* y[rows] for x[rows x features] (host buffers), in passes of the network's rows. */
int monki_mlp_forward(void *net, const float *x, uint32_t rows, float *y, char *err, size_t errlen);

/* Loss sum w (y - t)^2 / sum w of one batch (rows <= the network's rows) and its gradient
 * in the parameter layout. */
int monki_mlp_gradients(void *net, const float *x, const float *target, const float *weight, uint32_t rows,
                        float *grads, float *loss, char *err, size_t errlen);

/* Keep a training set on the device, then run Adam steps on minibatches of batch rows
 * drawn with replacement (Philox4x32-10); losses[steps] (or NULL) gets each step's loss
 * sum w (y - t)^2 / batch. */
int monki_mlp_set_data(void *net, const float *x, const float *target, const float *weight, uint32_t rows,
                       char *err, size_t errlen);
int monki_mlp_train(void *net, uint32_t steps, uint32_t batch, float lr, float *losses, char *err, size_t errlen);

void monki_mlp_close(void *net);

/* Test hook: C (M x N, FP32) = A (M x K) B^T (N x K) from BF16 bit patterns through the
 * tcgen05 GEMM; K a multiple of 64, N a multiple of 16 in [16, 256]; splits > 1 splits K
 * (K / 64 divisible by splits) and accumulates. */
int monki_mlp_gemm_probe(uint32_t device, const uint16_t *a, const uint16_t *b, int m, int n, int k, int splits,
                         float *c, char *err, size_t errlen);

#ifdef __cplusplus
}
#endif

#endif
