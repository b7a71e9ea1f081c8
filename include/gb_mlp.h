/* gb_mlp.h -- the small fully connected network of the learned near-singular
 * quadrature (training and inference on the GPU, own kernels: gb_mlp.cu).
 *
 * A network of nl layers maps widths[0] inputs to widths[nl] outputs: layer l
 * computes Z = A W_l + b_l with W_l [widths[l]][widths[l+1]] (row-major),
 * then GELU (erf form) on every layer but the last.  The products use the
 * weights rounded to bfloat16 (round to nearest even) with FP32 operands
 * otherwise and FP32 accumulation; FP32 master weights are kept for the
 * optimiser.  Parameters are packed layer after layer as W_l then b_l (FP32).
 * Batches are row-major FP32 device arrays; every call synchronises.
 * Every call returns 0 or -1 (gb_last_error() explains). */
#ifndef GB_MLP_H
#define GB_MLP_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_mlp gb_mlp;

int gb_mlp_create(int nl, const int *widths, gb_mlp **out);
void gb_mlp_destroy(gb_mlp *m);
size_t gb_mlp_param_count(const gb_mlp *m);
/* host arrays of gb_mlp_param_count floats; set also resets the optimiser */
int gb_mlp_set_params(gb_mlp *m, const float *params);
int gb_mlp_get_params(gb_mlp *m, float *params);
/* Y [B][widths[nl]] = network(X [B][widths[0]]) */
int gb_mlp_forward(gb_mlp *m, int B, const float *X, float *Y);
/* loss = (1/B) sum over the batch of the squared error |Y - T|^2, and its
 * gradient with respect to the parameters (through the bfloat16 weights as
 * if they were the master weights), packed like them into grad (device) */
int gb_mlp_loss_grad(gb_mlp *m, int B, const float *X, const float *T, double *loss, float *grad);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) with learning rate lr on
 * the batch; *loss: the batch loss before the step */
int gb_mlp_train_step(gb_mlp *m, int B, const float *X, const float *T, float lr, double *loss);

/* The same with host arrays (uploaded for the call).  gb_mlp_train_host:
 * `steps` Adam steps over n samples held on the device for the call, in
 * consecutive batches of B rows, wrapping round; losses[s] (may be NULL): the
 * loss of step s's batch before the step. */
int gb_mlp_forward_host(gb_mlp *m, int B, const float *X, float *Y);
int gb_mlp_loss_grad_host(gb_mlp *m, int B, const float *X, const float *T, double *loss, float *grad);
int gb_mlp_train_host(gb_mlp *m, int n, const float *X, const float *T, int B, int steps, float lr, double *losses);

#ifdef __cplusplus
}
#endif
#endif
