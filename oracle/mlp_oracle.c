/* CPU FP64 restatement of the per-node MLP of the learned Newton initial
 * guess: forward pass, loss and gradient, and the Adam update.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the device MLP kernels).  The MLP
 * has no counterpart in the reference; the algorithms restated are the
 * textbook ones: a fully connected network with tanh hidden layers, the mean
 * squared error, back-propagation, and Adam (Kingma & Ba, "Adam: A Method for
 * Stochastic Optimization", ICLR 2015, Algorithm 1, with bias correction).
 *
 * Parameter packing (shared with the device code): W1 [h1 x nin] row-major,
 * b1 [h1], W2 [h2 x h1], b2 [h2], W3 [nout x h2], b3 [nout].
 * Loss over a batch of n samples with a 0/1 mask per output:
 *     L = sum_{i,o} mask_io (y_io - t_io)^2 / (n * nout).
 */
#include "mlp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

int64_t mo_param_count(int nin, int h1, int h2, int nout)
{
  return (int64_t)h1 * nin + h1 + (int64_t)h2 * h1 + h2 + (int64_t)nout * h2 + nout;
}

typedef struct {
  const double *W1, *b1, *W2, *b2, *W3, *b3;
} Views;

static Views views(const double *p, int nin, int h1, int h2, int nout)
{
  Views v;
  v.W1 = p;
  v.b1 = v.W1 + (int64_t)h1 * nin;
  v.W2 = v.b1 + h1;
  v.b2 = v.W2 + (int64_t)h2 * h1;
  v.W3 = v.b2 + h2;
  v.b3 = v.W3 + (int64_t)nout * h2;
  (void)nout;
  return v;
}

/* One sample: hidden activations a1 [h1], a2 [h2] and output y [nout]. */
static void forward1(const Views *v, int nin, int h1, int h2, int nout, const double *x, double *a1,
                     double *a2, double *y)
{
  for(int j = 0; j < h1; ++j) {
    double z = v->b1[j];
    for(int k = 0; k < nin; ++k) z += v->W1[(int64_t)j * nin + k] * x[k];
    a1[j] = tanh(z);
  }
  for(int j = 0; j < h2; ++j) {
    double z = v->b2[j];
    for(int k = 0; k < h1; ++k) z += v->W2[(int64_t)j * h1 + k] * a1[k];
    a2[j] = tanh(z);
  }
  for(int o = 0; o < nout; ++o) {
    double z = v->b3[o];
    for(int k = 0; k < h2; ++k) z += v->W3[(int64_t)o * h2 + k] * a2[k];
    y[o] = z;
  }
}

void mo_forward(const double *params, int nin, int h1, int h2, int nout, const double *x, int64_t n,
                double *y)
{
  Views v = views(params, nin, h1, h2, nout);
  double *a1 = malloc(sizeof(double) * h1), *a2 = malloc(sizeof(double) * h2);
  for(int64_t i = 0; i < n; ++i) forward1(&v, nin, h1, h2, nout, x + i * nin, a1, a2, y + i * nout);
  free(a1);
  free(a2);
}

double mo_loss_grad(const double *params, int nin, int h1, int h2, int nout, const double *x, const double *t,
                    const double *mask, int64_t n, double *grad)
{
  Views v = views(params, nin, h1, h2, nout);
  const int64_t np = mo_param_count(nin, h1, h2, nout);
  if(grad) memset(grad, 0, sizeof(double) * np);
  double *gW1 = grad, *gb1 = gW1 ? gW1 + (int64_t)h1 * nin : NULL;
  double *gW2 = gb1 ? gb1 + h1 : NULL, *gb2 = gW2 ? gW2 + (int64_t)h2 * h1 : NULL;
  double *gW3 = gb2 ? gb2 + h2 : NULL, *gb3 = gW3 ? gW3 + (int64_t)nout * h2 : NULL;
  double *a1 = malloc(sizeof(double) * h1), *a2 = malloc(sizeof(double) * h2);
  double *y = malloc(sizeof(double) * nout), *dy = malloc(sizeof(double) * nout);
  double *d2 = malloc(sizeof(double) * h2), *d1 = malloc(sizeof(double) * h1);
  const double scale = 1.0 / ((double)n * nout);
  double loss = 0.;
  for(int64_t i = 0; i < n; ++i) {
    const double *xi = x + i * nin;
    forward1(&v, nin, h1, h2, nout, xi, a1, a2, y);
    for(int o = 0; o < nout; ++o) {
      const double m = mask ? mask[i * nout + o] : 1.0;
      const double e = y[o] - t[i * nout + o];
      loss += m * e * e * scale;
      dy[o] = 2.0 * m * e * scale;
    }
    if(!grad) continue;
    /* output layer */
    for(int o = 0; o < nout; ++o) {
      gb3[o] += dy[o];
      for(int k = 0; k < h2; ++k) gW3[(int64_t)o * h2 + k] += dy[o] * a2[k];
    }
    /* second hidden layer: d2 = (W3^T dy) * (1 - a2^2) */
    for(int k = 0; k < h2; ++k) {
      double s = 0.;
      for(int o = 0; o < nout; ++o) s += v.W3[(int64_t)o * h2 + k] * dy[o];
      d2[k] = s * (1.0 - a2[k] * a2[k]);
    }
    for(int j = 0; j < h2; ++j) {
      gb2[j] += d2[j];
      for(int k = 0; k < h1; ++k) gW2[(int64_t)j * h1 + k] += d2[j] * a1[k];
    }
    /* first hidden layer: d1 = (W2^T d2) * (1 - a1^2) */
    for(int k = 0; k < h1; ++k) {
      double s = 0.;
      for(int j = 0; j < h2; ++j) s += v.W2[(int64_t)j * h1 + k] * d2[j];
      d1[k] = s * (1.0 - a1[k] * a1[k]);
    }
    for(int j = 0; j < h1; ++j) {
      gb1[j] += d1[j];
      for(int k = 0; k < nin; ++k) gW1[(int64_t)j * nin + k] += d1[j] * xi[k];
    }
  }
  free(a1);
  free(a2);
  free(y);
  free(dy);
  free(d2);
  free(d1);
  return loss;
}

void mo_adam(double *params, double *m, double *v, const double *grad, int64_t np, double lr, double beta1,
             double beta2, double eps, int step)
{
  const double c1 = 1.0 - pow(beta1, step), c2 = 1.0 - pow(beta2, step);
  for(int64_t i = 0; i < np; ++i) {
    m[i] = beta1 * m[i] + (1.0 - beta1) * grad[i];
    v[i] = beta2 * v[i] + (1.0 - beta2) * grad[i] * grad[i];
    const double mh = m[i] / c1, vh = v[i] / c2;
    params[i] -= lr * mh / (sqrt(vh) + eps);
  }
}
