/*
 * lgd_surrogate.h - C ABI of the learned surrogate for variable-coefficient
 * diffusion (no counterpart in the reference library).
 *
 * Network: four 3x3x3 convolutions on a periodic grid, channels
 * 2 -> C -> C -> C -> 1 (C = 24 for the configured surrogate; 8 is built
 * for tests), GELU after the first three, residual u' = u + conv4(...).
 * Inputs per voxel: the field u and the coefficient kappa.  BF16 weights and
 * activations on the tensor cores with FP32 accumulation; FP32 master
 * parameters and Adam.
 *
 * Parameters (flat FP32): W1 b1 W2 b2 W3 b3 W4 b4, W_l[tap][cin][cout] with
 * tap = (dz+1)*9 + (dy+1)*3 + (dx+1).
 *
 * Field arguments are DEVICE pointers to FP32 arrays [batch][nz][ny][nx]
 * (dense, x fastest).  Work runs on the handle's stream.
 * Status codes and lgd_gpu_last_error() are shared with lgd_gpu.h.
 */
#ifndef LGD_SURROGATE_H
#define LGD_SURROGATE_H

#include <stddef.h>
#include <stdint.h>

#include "lgd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lgd_net lgd_net;

int lgd_net_param_count(int channels, int64_t *count);

/* nx a multiple of 32, ny of 4; training != 0 allocates the buffers for the
 * backward pass and Adam.  Parameters start at zero: set them. */
int lgd_net_create(int nx, int ny, int nz, int batch, int channels, int training, lgd_net **out);
int lgd_net_destroy(lgd_net *h);

int lgd_net_set_params(lgd_net *h, const float *host, size_t count);
int lgd_net_get_params(lgd_net *h, float *host, size_t count);
int lgd_net_get_grads(lgd_net *h, float *host, size_t count);

/* Replaces the gradient of the last backward pass (FP32, the parameter
 * layout).  Data-parallel training: every rank runs forward and backward
 * on its own batch, the ranks average their gradients (an all-reduce) and
 * set the average before lgd_net_adam, so every rank takes the same step
 * and the replicas stay identical. */
int lgd_net_set_grads(lgd_net *h, const float *host, size_t count);

/* d_du = net(u, kappa) (the increment; u' = u + d_du). */
int lgd_net_forward(lgd_net *h, const float *d_u, const float *d_kappa, float *d_du);

/* After lgd_net_forward on a training handle: MSE loss of the increment
 * against d_target_du (mean over all voxels) and its parameter gradient;
 * *loss (may be NULL) receives the loss (synchronises). */
int lgd_net_backward(lgd_net *h, const float *d_target_du, double *loss);

/* One Adam step with the gradient of the last backward pass. */
int lgd_net_adam(lgd_net *h, float lr, float beta1, float beta2, float eps);

/* calls surrogate calls in place: u <- u + net(u, kappa). */
int lgd_net_advance(lgd_net *h, float *d_u, const float *d_kappa, int calls);

int lgd_net_synchronize(lgd_net *h);
int lgd_net_stream(lgd_net *h, void **stream);
int lgd_net_launch_count(lgd_net *h, uint64_t *count);

/* Inference path: 0 (default) runs the two C -> C layers on the tcgen05
 * tensor cores (TMA-fed input planes, accumulators in tensor memory) when
 * the handle has no training buffers, C = 24, nx is a multiple of 128 and
 * ny even; 1 runs every layer on the mma.sync kernels (the training
 * path's).  Results agree to BF16 rounding of the activations. */
int lgd_net_set_variant(lgd_net *h, int variant);
/* *yes = 1 when forward / advance run the tcgen05 layers. */
int lgd_net_uses_tensor_core_path(lgd_net *h, int *yes);

#ifdef __cplusplus
}
#endif

#endif
