// mlp_oracle.cpp -- CPU oracle of the per-contact warm-start network (TEST INFRASTRUCTURE ONLY,
// see oracle.h).
//
// The network has no counterpart in the reference (SCISim warm-starts only from its impulse
// cache, GeometricImpactFrictionMap.cpp:174-220).  This is the plain FP64 statement of the
// GPU's network, used to check its forward pass, its gradients and its features:
//   12 -> 64 -> 64 -> 3, GELU (erf form) after the two hidden layers;
//   parameters packed as W1 (64 x 12, row-major), b1 (64), W2 (64 x 64), b2 (64), W3 (3 x 64), b3 (3);
//   loss per sample 0.5 (y0 - t0)^2 + 0.5 (y1 - t1)^2 + softplus(y2) - t2 y2, averaged over samples.
#include "oracle.h"

#include <cmath>
#include <vector>

namespace {

constexpr int kIn = 12, kH = 64, kOut = 3;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
              oB3 = oW3 + kOut * kH, kParams = oB3 + kOut;

inline double gelu(double z) { return 0.5 * z * (1.0 + std::erf(z / std::sqrt(2.0))); }
inline double gelu_d(double z) {
  return 0.5 * (1.0 + std::erf(z / std::sqrt(2.0))) + z * std::exp(-0.5 * z * z) / std::sqrt(2.0 * M_PI);
}

struct Act {
  double z1[kH], h1[kH], z2[kH], h2[kH], y[kOut];
};

void forward(const float* p, const float* x, Act& a) {
  for (int j = 0; j < kH; ++j) {
    double s = p[oB1 + j];
    for (int i = 0; i < kIn; ++i) s += (double)p[oW1 + j * kIn + i] * x[i];
    a.z1[j] = s;
    a.h1[j] = gelu(s);
  }
  for (int j = 0; j < kH; ++j) {
    double s = p[oB2 + j];
    for (int i = 0; i < kH; ++i) s += (double)p[oW2 + j * kH + i] * a.h1[i];
    a.z2[j] = s;
    a.h2[j] = gelu(s);
  }
  for (int j = 0; j < kOut; ++j) {
    double s = p[oB3 + j];
    for (int i = 0; i < kH; ++i) s += (double)p[oW3 + j * kH + i] * a.h2[i];
    a.y[j] = s;
  }
}

}  // namespace

extern "C" int or_mlp_param_count(void) { return kParams; }

extern "C" void or_mlp_forward(const float* params, int n, const float* x, double* y) {
  Act a;
  for (int s = 0; s < n; ++s) {
    forward(params, x + kIn * s, a);
    for (int j = 0; j < kOut; ++j) y[kOut * s + j] = a.y[j];
  }
}

extern "C" double or_mlp_loss_grad(const float* params, int n, const float* x, const float* t, double* grad) {
  for (int i = 0; i < kParams; ++i) grad[i] = 0.0;
  double loss = 0.0;
  Act a;
  const double inv_n = n > 0 ? 1.0 / n : 0.0;
  for (int s = 0; s < n; ++s) {
    const float* xs = x + kIn * s;
    const float* ts = t + kOut * s;
    forward(params, xs, a);
    const double e0 = a.y[0] - ts[0], e1 = a.y[1] - ts[1];
    const double y2 = a.y[2];
    const double sp = y2 > 0.0 ? y2 + std::log1p(std::exp(-y2)) : std::log1p(std::exp(y2));
    loss += 0.5 * e0 * e0 + 0.5 * e1 * e1 + sp - ts[2] * y2;
    const double dy[kOut] = {e0 * inv_n, e1 * inv_n, (1.0 / (1.0 + std::exp(-y2)) - ts[2]) * inv_n};
    double dh2[kH] = {0.0};
    for (int j = 0; j < kOut; ++j) {
      grad[oB3 + j] += dy[j];
      for (int i = 0; i < kH; ++i) {
        grad[oW3 + j * kH + i] += dy[j] * a.h2[i];
        dh2[i] += dy[j] * params[oW3 + j * kH + i];
      }
    }
    double dh1[kH] = {0.0};
    for (int j = 0; j < kH; ++j) {
      const double dz = dh2[j] * gelu_d(a.z2[j]);
      grad[oB2 + j] += dz;
      for (int i = 0; i < kH; ++i) {
        grad[oW2 + j * kH + i] += dz * a.h1[i];
        dh1[i] += dz * params[oW2 + j * kH + i];
      }
    }
    for (int j = 0; j < kH; ++j) {
      const double dz = dh1[j] * gelu_d(a.z1[j]);
      grad[oB1 + j] += dz;
      for (int i = 0; i < kIn; ++i) grad[oW1 + j * kIn + i] += dz * xs[i];
    }
  }
  return loss * inv_n;
}
