/*
 * chinium_guess.h -- the learned starting density: a per-atom-pair MLP
 * trained and evaluated by this library's own CUDA kernels.  No counterpart
 * in the reference, whose SCF starts from the SAP guess
 * (src/HartreeFockKohnSham/GuessSCF.cpp:17-99); the learned guess replaces
 * that starting point and falls back to it.
 *
 * Network: x (nin) -> [Linear, SiLU] x nlayers (width nhidden) -> Linear
 * (nout).  Parameters are one flat FP32 vector, layer by layer: W (fan_in x
 * fan_out, row-major) then b.  Batches are row-major host arrays.  Training
 * runs in FP32 (forward, backward, Adam on the device); inference may use
 * BF16 weights with FP32 accumulation.  Status codes as in chinium_xc.h.
 */
#ifndef CHINIUM_GUESS_H
#define CHINIUM_GUESS_H

#include "chinium_xc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xc_mlp xc_mlp;

int xc_mlp_create(int nin, int nhidden, int nlayers, int nout, xc_mlp** out);
int xc_mlp_destroy(xc_mlp* m);
int xc_mlp_nparams(const xc_mlp* m, long* n);
/* Sets the parameters and resets the optimiser state. */
int xc_mlp_set_params(xc_mlp* m, const float* params);
int xc_mlp_get_params(const xc_mlp* m, float* params);
/* Y (batch x nout) = net(X (batch x nin)); bf16 != 0 uses BF16 weights. */
int xc_mlp_forward(xc_mlp* m, int batch, const float* X, float* Y, int bf16);
/* Gradient of sum(dY * net(X)) with respect to the parameters (FP32). */
int xc_mlp_backward(xc_mlp* m, int batch, const float* X, const float* dY, float* grad);
/* One Adam step on the masked mean-squared error sum(mask (net(X) - T)^2) /
 * sum(mask); *loss is that error before the step. */
int xc_mlp_train_step(xc_mlp* m, int batch, const float* X, const float* T, const float* mask,
                      float lr, float* loss);

#ifdef __cplusplus
}
#endif
#endif
