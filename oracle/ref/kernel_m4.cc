// kernel_m4.cc -- cubic B-spline (Monaghan M4, radial support 2h) that the
// Sod oracle build links in place of the reference's Gaussian weight() and
// d_weight() (sph_lib.cc:210-253 are compiled under other names with
// -Dweight=weight_gauss -Dd_weight=d_weight_gauss).  Same signature and
// meaning: s = (x_i - x_j)/h, result = W or dW/dx_dir.  Arithmetic matches
// weight_m4 / d_weight_m4 of oracle/sph_oracle.c.
#include <cmath>
#include "constant.h"

static const double M4_SIGMA = (DIMENSION == 1) ? 0.66666666666666663 : 0.31830988618379069;

double weight(double *s, double h)
{
  double r2 = 0;
  for (int i = 0; i < DIMENSION; i++) r2 += s[i] * s[i];
  double q = std::sqrt(r2);
  if (q >= 2.0) return 0;
  double norm = M4_SIGMA;
  for (int i = 0; i < DIMENSION; i++) norm = norm / h;
  double w;
  if (q < 1.0) {
    w = 1.0 - 1.5 * q * q + 0.75 * q * q * q;
  } else {
    double t = 2.0 - q;
    w = 0.25 * t * t * t;
  }
  return norm * w;
}

double d_weight(double *s, double h, int dir)
{
  double r2 = 0;
  for (int i = 0; i < DIMENSION; i++) r2 += s[i] * s[i];
  double q = std::sqrt(r2);
  if (q >= 2.0 || q == 0.0) return 0;
  double norm = M4_SIGMA;
  for (int i = 0; i < DIMENSION; i++) norm = norm / h;
  double dw;
  if (q < 1.0) {
    dw = -3.0 * q + 2.25 * q * q;
  } else {
    double t = 2.0 - q;
    dw = -0.75 * t * t;
  }
  return norm * dw * s[dir] / (q * h);
}
