// mlp_oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// CPU restatement of the spectrum surrogate's forward and backward passes
// (the network has no reference counterpart; this is the checker of the
// GPU kernels' gradients).  FP64 arithmetic, with the values rounded to
// BF16 (round to nearest even, via FP32) at the points where the GPU kernels
// store BF16: the input features, the weights W1..W4, the pre-activations Z,
// the activations X and the back-propagated gradients dH.  Biases, the head
// weights w5, b5 and the loss stay FP32 values.
//
// Layout of the flat parameter vector: W1 [256][7], b1 [256], W2 [256][256],
// b2, W3, b3, W4, b4, w5 [256], b5.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int W = 256, F = 7;
constexpr int oW1 = 0, oB1 = oW1 + W * F, oW2 = oB1 + W, oB2 = oW2 + W * W, oW3 = oB2 + W, oB3 = oW3 + W * W,
              oW4 = oB3 + W, oB4 = oW4 + W * W, oW5 = oB4 + W, oB5 = oW5 + W, NP = oB5 + 1;

double bf16(double v) {
  float f = (float)v;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  std::memcpy(&f, &u, 4);
  return f;
}
double silu(double z) { return z / (1.0 + std::exp(-z)); }
double silu_grad(double z) {
  const double s = 1.0 / (1.0 + std::exp(-z));
  return s * (1.0 + z * (1.0 - s));
}

struct Net {
  int in[4] = {F, W, W, W};
  int offW[4] = {oW1, oW2, oW3, oW4}, offB[4] = {oB1, oB2, oB3, oB4};
  std::vector<double> w[4];   // BF16-rounded weights [256][in]
  const float *P;
  explicit Net(const float *p) : P(p) {
    for (int l = 0; l < 4; ++l) {
      w[l].resize((size_t)W * in[l]);
      for (size_t k = 0; k < w[l].size(); ++k) w[l][k] = bf16(p[offW[l] + k]);
    }
  }
};

// Forward of one row; keeps Z (BF16) and X (BF16) per layer.
double forward_row(const Net &n, const float *x, double Z[4][W], double X[5][W]) {
  for (int i = 0; i < F; ++i) X[0][i] = bf16(x[i]);
  for (int l = 0; l < 4; ++l) {
    for (int o = 0; o < W; ++o) {
      double acc = 0.0;
      const double *wr = &n.w[l][(size_t)o * n.in[l]];
      for (int i = 0; i < n.in[l]; ++i) acc += X[l][i] * wr[i];
      const double z = (double)(float)acc + (double)n.P[n.offB[l] + o];
      Z[l][o] = bf16(z);
      X[l + 1][o] = bf16(silu(z));
    }
  }
  double y = 0.0;
  for (int o = 0; o < W; ++o) y += X[4][o] * (double)n.P[oW5 + o];
  return y + (double)n.P[oB5];
}

}  // namespace

extern "C" {

int gor_mlp_params(void) { return NP; }

void gor_mlp_forward(const float *P, const float *x, int n, double *y) {
  Net net(P);
  std::vector<double> Z(4 * W), X(5 * W);
  for (int m = 0; m < n; ++m)
    y[m] = forward_row(net, x + (size_t)m * F, reinterpret_cast<double(*)[W]>(Z.data()),
                       reinterpret_cast<double(*)[W]>(X.data()));
}

// Mean squared error over n rows and its gradient w.r.t. every parameter.
void gor_mlp_grad(const float *P, const float *x, const float *t, int n, double *loss, double *grad) {
  Net net(P);
  std::memset(grad, 0, sizeof(double) * NP);
  double se = 0.0;
  std::vector<double> Zb(4 * W), Xb(5 * W);
  auto Z = reinterpret_cast<double(*)[W]>(Zb.data());
  auto X = reinterpret_cast<double(*)[W]>(Xb.data());
  double dH[W], dX[W];
  for (int m = 0; m < n; ++m) {
    const double yh = forward_row(net, x + (size_t)m * F, Z, X);
    const double e = yh - (double)t[m];
    se += e * e;
    const double dy = (double)(float)(2.0 * e / n);
    for (int o = 0; o < W; ++o) grad[oW5 + o] += dy * X[4][o];
    grad[oB5] += dy;
    for (int o = 0; o < W; ++o) dH[o] = bf16((double)(float)(dy * (double)P[oW5 + o]) * silu_grad(Z[3][o]));
    for (int l = 3; l >= 0; --l) {
      const int in = net.in[l];
      for (int o = 0; o < W; ++o) {
        grad[net.offB[l] + o] += dH[o];
        double *g = grad + net.offW[l] + (size_t)o * in;
        for (int i = 0; i < in; ++i) g[i] += dH[o] * X[l][i];
      }
      if (l == 0) break;
      for (int i = 0; i < in; ++i) {
        double acc = 0.0;
        for (int o = 0; o < W; ++o) acc += dH[o] * net.w[l][(size_t)o * in + i];
        dX[i] = acc;
      }
      for (int i = 0; i < in; ++i) dH[i] = bf16((double)(float)dX[i] * silu_grad(Z[l - 1][i]));
    }
  }
  *loss = se / n;
}

}  // extern "C"
