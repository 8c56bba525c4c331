// Learned task-cost model: a 6 -> 64 -> 64 -> 1 multilayer perceptron with
// SiLU activations in FP32, trained with Adam on the log of measured per-task
// kernel times, and evaluated for every task of a list to order the work
// queues of the persistent grid kernels.
//
// Parameter layout (one flat float array, kMlpParams words):
//   W1[64][6]  b1[64]  W2[64][64]  b2[64]  w3[64]  b3
// with z1 = W1 x + b1, h1 = silu(z1), z2 = W2 h1 + b2, h2 = silu(z2),
// y = w3 . h2 + b3 and the loss  L = (1/N) sum_s (y_s - t_s)^2.
//
// Training kernels are deterministic: every block reduces its tile of
// samples into its own slot of a partial-gradient buffer, and a second
// kernel sums the slots in a fixed order.
#include "gb300_internal.h"

namespace gb300 {

constexpr int kIn = 6, kH = 64;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH,
              oW3 = oB2 + kH, oB3 = oW3 + kH, kMlpParams = oB3 + 1;
static_assert(kMlpParams == 4673, "parameter layout");
constexpr int kTile = 32;   // samples per training block
constexpr int kW2Pad = kH + 1; // padded row stride of W2 in shared memory

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s * (1.f + z * (1.f - s));
}

struct TrainSmem {
  float w1[kH * kIn], b1[kH], w2[kH * kW2Pad], b2[kH], w3[kH], b3;
  float x[kTile][kIn];
  float z1[kTile][kH], h1[kTile][kH], z2[kTile][kH];
  float g[kTile];
};

// One block of 64 threads (thread j <-> hidden unit j) per tile of kTile
// samples: forward pass, loss, backward pass, and the tile's gradient sums.
__global__ void __launch_bounds__(kH) mlp_train_tile(const float *__restrict__ P,
                                                     const float *__restrict__ X,
                                                     const float *__restrict__ T, int n,
                                                     float *__restrict__ partial,
                                                     float *__restrict__ loss_partial) {
  __shared__ TrainSmem sm;
  const int j = threadIdx.x;
  const int s0 = blockIdx.x * kTile;
  for (int k = 0; k < kIn; k++)
    sm.w1[j * kIn + k] = P[oW1 + j * kIn + k];
  sm.b1[j] = P[oB1 + j];
  for (int i = 0; i < kH; i++)
    sm.w2[j * kW2Pad + i] = P[oW2 + j * kH + i];
  sm.b2[j] = P[oB2 + j];
  sm.w3[j] = P[oW3 + j];
  if (j == 0)
    sm.b3 = P[oB3];
  for (int e = j; e < kTile * kIn; e += kH) {
    const int s = e / kIn, k = e % kIn;
    sm.x[s][k] = (s0 + s < n) ? X[(size_t)(s0 + s) * kIn + k] : 0.f;
  }
  __syncthreads();
  // layer 1
  for (int s = 0; s < kTile; s++) {
    float z = sm.b1[j];
    for (int k = 0; k < kIn; k++)
      z = fmaf(sm.w1[j * kIn + k], sm.x[s][k], z);
    sm.z1[s][j] = z;
    sm.h1[s][j] = silu(z);
  }
  __syncthreads();
  // layer 2
  for (int s = 0; s < kTile; s++) {
    float z = sm.b2[j];
    for (int i = 0; i < kH; i++)
      z = fmaf(sm.w2[j * kW2Pad + i], sm.h1[s][i], z);
    sm.z2[s][j] = z;
  }
  __syncthreads();
  // output, residual and dL/dy
  if (j < kTile) {
    const int s = j;
    float y = sm.b3;
    for (int i = 0; i < kH; i++)
      y = fmaf(sm.w3[i], silu(sm.z2[s][i]), y);
    const bool live = s0 + s < n;
    const float r = live ? y - T[s0 + s] : 0.f;
    sm.g[s] = 2.f * r / (float)n;
    float l = r * r / (float)n;
    for (int o = 16; o > 0; o >>= 1)
      l += __shfl_xor_sync(0xffffffffu, l, o);
    if (s == 0)
      loss_partial[blockIdx.x] = l;
  }
  __syncthreads();
  float *G = partial + (size_t)blockIdx.x * kMlpParams;
  // output layer gradients; dz2 replaces z2 (column j is owned by thread j)
  float dw3 = 0.f, db2 = 0.f;
  for (int s = 0; s < kTile; s++) {
    const float z = sm.z2[s][j];
    dw3 = fmaf(sm.g[s], silu(z), dw3);
    const float dz = sm.g[s] * sm.w3[j] * dsilu(z);
    sm.z2[s][j] = dz;
    db2 += dz;
  }
  G[oW3 + j] = dw3;
  G[oB2 + j] = db2;
  if (j == 0) {
    float gb = 0.f;
    for (int s = 0; s < kTile; s++)
      gb += sm.g[s];
    G[oB3] = gb;
  }
  __syncthreads();
  // dW2[j][i] = sum_s dz2[s][j] h1[s][i]
  for (int i = 0; i < kH; i++) {
    float a = 0.f;
    for (int s = 0; s < kTile; s++)
      a = fmaf(sm.z2[s][j], sm.h1[s][i], a);
    G[oW2 + j * kH + i] = a;
  }
  // dz1[s][i=j] = silu'(z1) * sum_q W2[q][j] dz2[s][q]; replaces h1 after use
  __syncthreads();
  float db1 = 0.f;
  float dw1[kIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int s = 0; s < kTile; s++) {
    float a = 0.f;
    for (int q = 0; q < kH; q++)
      a = fmaf(sm.w2[q * kW2Pad + j], sm.z2[s][q], a);
    const float dz = a * dsilu(sm.z1[s][j]);
    db1 += dz;
    for (int k = 0; k < kIn; k++)
      dw1[k] = fmaf(dz, sm.x[s][k], dw1[k]);
  }
  G[oB1 + j] = db1;
  for (int k = 0; k < kIn; k++)
    G[oW1 + j * kIn + k] = dw1[k];
}

// grad[p] = sum over tiles (fixed order); loss = sum of the tile losses
__global__ void mlp_reduce(const float *__restrict__ partial, const float *__restrict__ loss_partial,
                           int ntiles, float *__restrict__ grad, float *__restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kMlpParams) {
    float a = 0.f;
    for (int b = 0; b < ntiles; b++)
      a += partial[(size_t)b * kMlpParams + p];
    grad[p] = a;
  }
  if (p == 0 && loss) {
    float l = 0.f;
    for (int b = 0; b < ntiles; b++)
      l += loss_partial[b];
    *loss = l;
  }
}

__global__ void mlp_adam(float *__restrict__ P, const float *__restrict__ grad,
                         float *__restrict__ m, float *__restrict__ v, float lr, float beta1,
                         float beta2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParams)
    return;
  const float g = grad[p];
  const float mm = beta1 * m[p] + (1.f - beta1) * g;
  const float vv = beta2 * v[p] + (1.f - beta2) * g * g;
  m[p] = mm;
  v[p] = vv;
  P[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// Inference: one thread per sample, parameters in shared memory (uniform
// reads broadcast), h1 in registers.  Optional standardisation of the raw
// features: x_k <- (x_k - mean_k) / scale_k.
__global__ void __launch_bounds__(128) mlp_predict(const float *__restrict__ P,
                                                   const float *__restrict__ X, int n,
                                                   const float *__restrict__ norm,
                                                   float *__restrict__ Y) {
  __shared__ float sp[kMlpParams];
  __shared__ float snorm[2 * kIn];
  for (int p = threadIdx.x; p < kMlpParams; p += blockDim.x)
    sp[p] = P[p];
  if (threadIdx.x < 2 * kIn)
    snorm[threadIdx.x] = norm ? norm[threadIdx.x] : (threadIdx.x < kIn ? 0.f : 1.f);
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n)
    return;
  float x[kIn];
  for (int k = 0; k < kIn; k++)
    x[k] = (X[(size_t)s * kIn + k] - snorm[k]) / snorm[kIn + k];
  float h1[kH];
#pragma unroll
  for (int j = 0; j < kH; j++) {
    float z = sp[oB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; k++)
      z = fmaf(sp[oW1 + j * kIn + k], x[k], z);
    h1[j] = silu(z);
  }
  float y = sp[oB3];
  for (int j = 0; j < kH; j++) {
    float z = sp[oB2 + j];
#pragma unroll
    for (int i = 0; i < kH; i++)
      z = fmaf(sp[oW2 + j * kH + i], h1[i], z);
    y = fmaf(sp[oW3 + j], silu(z), y);
  }
  Y[s] = y;
}

int mlp_nparams() { return kMlpParams; }
int mlp_tiles(int n) { return (n + kTile - 1) / kTile; }

void launch_mlp_loss_grad(const float *P, const float *X, const float *T, int n, float *loss,
                          float *grad, float *work, cudaStream_t s) {
  const int nt = mlp_tiles(n);
  float *partial = work, *lp = work + (size_t)nt * kMlpParams;
  mlp_train_tile<<<nt, kH, 0, s>>>(P, X, T, n, partial, lp);
  mlp_reduce<<<(kMlpParams + 255) / 256, 256, 0, s>>>(partial, lp, nt, grad, loss);
  count_launch(2);
}

void launch_mlp_adam(float *P, const float *grad, float *m, float *v, int step, float lr,
                     float beta1, float beta2, float eps, cudaStream_t s) {
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(P, grad, m, v, lr, beta1, beta2, eps, c1, c2);
  count_launch();
}

void launch_mlp_predict(const float *P, const float *X, int n, const float *norm, float *Y,
                        cudaStream_t s) {
  if (n <= 0)
    return;
  mlp_predict<<<(n + 127) / 128, 128, 0, s>>>(P, X, n, norm, Y);
  count_launch();
}

} // namespace gb300
