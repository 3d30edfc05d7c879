/*
 * imodel_mlp.h -- the per-edge network of the learned TRSK correction.
 *
 * No counterpart in the reference: iModel has no learned component.  The
 * network (24 -> 64 -> 64 -> 1, GELU, BF16 operands, FP32 accumulation)
 * predicts the error of TRSK's tangential-velocity reconstruction
 * (vecrecon_trsk_tg, src/interpack.f90:3852-3976) from local inputs; its
 * inputs are defined in imodel_gb300/learned.py.  Training and inference run
 * on the GPU's tensor cores (tcgen05) with the library's own kernels.
 *
 * Parameters: 5825 FP32 values,
 *   W1[64][24] (out-major), b1[64], W2[64][64] (out-major), b2[64], w3[64], b3.
 * Inputs x[n][24]: BF16 bit patterns (uint16).  Status codes: imodel_swm.h.
 */
#ifndef IMODEL_MLP_H
#define IMODEL_MLP_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define IMODEL_MLP_NPARAM 5825
#define IMODEL_MLP_NIN 24

int imodel_mlp_create(int32_t device, void **mlp);
int imodel_mlp_set_params(void *mlp, const float *params, int32_t n);
int imodel_mlp_get_params(void *mlp, float *params, int32_t n);
/* y[n] = network(x[n][24]); host arrays. */
int imodel_mlp_forward(void *mlp, const uint16_t *x, int64_t n, float *y);
/* Gradient of the weighted mean squared error sum_b w_b (y_b - t_b)^2 / batch
 * over one batch of `batch` rows of (x, t, w) (w NULL: all weights 1):
 * seed 0 takes rows 0..batch-1, any other seed draws rows with replacement.
 * grad[5825]; *loss = the weighted mean squared error. */
int imodel_mlp_grad(void *mlp, const uint16_t *x, const float *t, const float *w, int64_t n,
                    uint64_t seed, int64_t batch, float *grad, double *loss);
/* Copies a training set (x[n][24], t[n], optional weights w[n]) to the device. */
int imodel_mlp_load_dataset(void *mlp, const uint16_t *x, const float *t, const float *w,
                            int64_t n);
/* `steps` Adam steps (beta 0.9/0.999, eps 1e-8) on random batches of the
 * loaded set; losses[steps] receives each batch's mean squared error. */
int imodel_mlp_train(void *mlp, int64_t steps, int64_t batch, float lr, uint64_t seed,
                     float *losses);
int imodel_mlp_destroy(void *mlp);
const char *imodel_mlp_last_error(void *mlp);

#ifdef __cplusplus
}
#endif
#endif
