/* CPU FP64 restatement of the learned-guess MLP (test infrastructure only). */
#ifndef FE_MLP_ORACLE_H
#define FE_MLP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int64_t mo_param_count(int nin, int h1, int h2, int nout);
void mo_forward(const double *params, int nin, int h1, int h2, int nout, const double *x, int64_t n,
                double *y);
/* Returns the masked mean-squared loss; writes its gradient when grad != NULL. */
double mo_loss_grad(const double *params, int nin, int h1, int h2, int nout, const double *x, const double *t,
                    const double *mask, int64_t n, double *grad);
/* One Adam step (step counts from 1). */
void mo_adam(double *params, double *m, double *v, const double *grad, int64_t np, double lr, double beta1,
             double beta2, double eps, int step);

#ifdef __cplusplus
}
#endif

#endif
