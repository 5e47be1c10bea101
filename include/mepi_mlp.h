/*
 * mepi_mlp.h -- C ABI of the proposal network of the adaptive k-mesh
 * refinement (no counterpart in the reference, whose k-mesh is uniform:
 * src/k_space.f90:252-256).
 *
 * A fully connected network n_in -> width -> ... -> width -> 1 with `depth`
 * GELU hidden layers of `width` = 128 units.  Weights and activations are
 * stored in BF16, every product accumulates in FP32 (tcgen05 tensor-core
 * GEMMs with the accumulator in tensor memory), the master weights and the
 * Adam moments are FP32.  Training (forward, backward, Adam) and inference
 * run on the GPU; one training step is captured into a CUDA graph and
 * replayed.
 *
 * Parameter vector (FP32, mepi_mlp_param_count entries), layer by layer:
 *   for l = 0 .. depth-1:  W_l (width x in_l, row-major; in_0 = n_in,
 *                          in_l = width), b_l (width)
 *   then the head:         w_o (width), b_o (1)
 * Inputs are row-major x[row][n_in] (n_in <= 64); targets y[row].
 * Loss: mean over rows of (f(x) - y)^2.
 *
 * Every function returns 0 or a MEPI_ERR_* code of mepi.h.
 */
#ifndef MEPI_MLP_H
#define MEPI_MLP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mepi_mlp mepi_mlp;

/* n_in in 1..64, width 128, depth in 1..8; weights drawn from N(0, 1/in_l)
 * (biases 0) by a generator seeded with `seed`. */
int mepi_mlp_create(mepi_mlp **out, int32_t n_in, int32_t width, int32_t depth, uint64_t seed);
int mepi_mlp_destroy(mepi_mlp *net);
int64_t mepi_mlp_param_count(const mepi_mlp *net);
int mepi_mlp_get_params(const mepi_mlp *net, float *params);
/* also resets the Adam moments and step */
int mepi_mlp_set_params(mepi_mlp *net, const float *params);

/* y[row] = f(x[row]) for n_rows rows (host buffers). */
int mepi_mlp_forward(mepi_mlp *net, int64_t n_rows, const float *x, float *y);

/* Loss and its gradient (parameter-vector layout) over all n_rows rows as
 * one batch (n_rows <= 32768). */
int mepi_mlp_loss_grad(mepi_mlp *net, int64_t n_rows, const float *x, const float *y, double *loss, float *grad);

/* Adam (beta 0.9, 0.999, eps 1e-8, learning rate lr) over `epochs` passes
 * of the rows in batches of `batch` rows (a multiple of 128), in an order
 * shuffled per epoch by a generator seeded with `seed`.  loss_hist
 * (optional, `epochs` entries) receives each epoch's mean batch loss. */
int mepi_mlp_train(mepi_mlp *net, int64_t n_rows, const float *x, const float *y, int32_t epochs, int32_t batch,
                   float lr, uint64_t seed, float *loss_hist);

#ifdef __cplusplus
}
#endif

#endif /* MEPI_MLP_H */
