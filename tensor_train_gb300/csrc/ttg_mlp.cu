// Rank model of the learned-sketch rounding: a 3-layer MLP
//   y = W3^T relu(W2^T relu(W1^T x + b1) + b2) + b3,   x in R^F, hidden H,
// trained on the GPU with these kernels (forward, backward, Adam).  Rows
// are bonds, features per bond come from tensor_train_gb300/sketch.py, the
// target is log(exact rank) from the exact rounder.  FP32 parameters and
// activations; the GEMMs run on the tensor cores with split-BF16 operands.
//
// Parameter layout (one device array): W1 (F x H) | b1 (H) | W2 (H x H) |
// b2 (H) | W3 (H) | b3 (1), all row-major.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ttg.h"
#include "ttg_kernels.h"

namespace ttg
{
namespace
{

// C(M x N) = op(A) op(B) (+ bias[n]) (relu), FP32 in and out, on the tcgen05
// tensor cores with split-BF16 operands (ttg_tc_gemm.cu).  op via strides:
// A(i, p) = A[i*ars + p*acs], B(p, j) = B[p*brs + j*bcs].
void gemm_f32(cudaStream_t st, int M, int N, int K, const float* A, int64_t ars, int64_t acs,
              const float* B, int64_t brs, int64_t bcs, float* C, int64_t ldc, const float* bias,
              bool relu)
{
  tc_gemm_f32(st, M, N, K, A, ars, acs, B, brs, bcs, C, ldc, bias, relu, false, 3);
}

// dy = 2 (y - t) / N; loss partial sums.
__global__ void mse_grad_kernel(const float* y, const float* t, int N, float* dy, double* loss)
{
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
  {
    const float e = y[i] - t[i];
    dy[i] = 2.f * e / static_cast<float>(N);
    s += static_cast<double>(e) * e;
  }
  for (int o = 16; o > 0; o >>= 1)
    s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0)
    atomicAdd(loss, s / N);
}

// out = max(in, 0).
__global__ void relu_kernel(const float* in, float* out, int64_t n)
{
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    out[i] = fmaxf(in[i], 0.f);
}

// dZ = dH * (Z > 0), in place on dH.
__global__ void relu_back_kernel(float* dH, const float* Z, int64_t n)
{
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (Z[i] <= 0.f)
      dH[i] = 0.f;
}

// db[j] = sum_i dZ[i, j] (one thread per column; rows are strided).
__global__ void colsum_kernel(const float* dZ, int rows, int cols, float* db)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols)
    return;
  float s = 0.f;
  for (int i = 0; i < rows; ++i)
    s += dZ[static_cast<int64_t>(i) * cols + j];
  db[j] = s;
}

// Adam (Kingma & Ba 2015) with bias correction.
__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int n, float lr, float b1,
                            float b2, float eps, float c1, float c2)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const float gi = g[i];
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
  }
}

}  // namespace
}  // namespace ttg

using namespace ttg;

struct ttg_mlp
{
  int F = 0, H = 0, nparams = 0;
  float* params = nullptr;  // device
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  int step = 0;
  // activations for the largest batch seen
  int cap_rows = 0;
  float *Z1 = nullptr, *Z2 = nullptr, *y = nullptr, *dy = nullptr, *H1 = nullptr,
        *H2 = nullptr;
  double* loss = nullptr;
  int64_t launches = 0;
  ~ttg_mlp()
  {
    for (void* p : {static_cast<void*>(params), static_cast<void*>(grads), static_cast<void*>(m),
                    static_cast<void*>(v), static_cast<void*>(Z1), static_cast<void*>(Z2),
                    static_cast<void*>(y), static_cast<void*>(dy), static_cast<void*>(H1),
                    static_cast<void*>(H2), static_cast<void*>(loss)})
      if (p)
        cudaFree(p);
  }
  float* W1() { return params; }
  float* b1() { return params + F * H; }
  float* W2() { return b1() + H; }
  float* b2() { return W2() + H * H; }
  float* W3() { return b2() + H; }
  float* b3() { return W3() + H; }
  float* gW1() { return grads; }
  float* gb1() { return grads + F * H; }
  float* gW2() { return gb1() + H; }
  float* gb2() { return gW2() + H * H; }
  float* gW3() { return gb2() + H; }
  float* gb3() { return gW3() + H; }
};

namespace
{

int32_t mfail(int32_t st, const std::string& m)
{
  set_last_error(m);
  return st;
}

#define MLP_CUDA(call)                                                                 \
  do                                                                                   \
  {                                                                                    \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return mfail(e_ == cudaErrorMemoryAllocation ? TTG_ERR_OOM : TTG_ERR_CUDA,       \
                   std::string(#call) + ": " + cudaGetErrorString(e_));               \
  } while (0)

int32_t ensure_rows(ttg_mlp* m, int rows)
{
  if (rows <= m->cap_rows)
    return TTG_OK;
  for (float** p : {&m->Z1, &m->Z2, &m->y, &m->dy, &m->H1, &m->H2})
  {
    if (*p)
      cudaFree(*p);
    *p = nullptr;
  }
  const size_t h = sizeof(float) * static_cast<size_t>(rows) * m->H;
  MLP_CUDA(cudaMalloc(&m->Z1, h));
  MLP_CUDA(cudaMalloc(&m->Z2, h));
  MLP_CUDA(cudaMalloc(&m->H1, h));
  MLP_CUDA(cudaMalloc(&m->H2, h));
  MLP_CUDA(cudaMalloc(&m->y, sizeof(float) * rows));
  MLP_CUDA(cudaMalloc(&m->dy, sizeof(float) * rows));
  m->cap_rows = rows;
  return TTG_OK;
}

// Forward pass: Z1 = x W1 + b1, H1 = relu(Z1), Z2 = H1 W2 + b2,
// H2 = relu(Z2), y = H2 W3 + b3.  Pre-activations and activations are kept
// for the backward pass.
void forward(ttg_mlp* m, const float* x, int rows, float* y, cudaStream_t st)
{
  const int F = m->F, H = m->H;
  const int64_t n = static_cast<int64_t>(rows) * H;
  gemm_f32(st, rows, H, F, x, F, 1, m->W1(), H, 1, m->Z1, H, m->b1(), false);
  relu_kernel<<<256, 256, 0, st>>>(m->Z1, m->H1, n);
  gemm_f32(st, rows, H, H, m->H1, H, 1, m->W2(), H, 1, m->Z2, H, m->b2(), false);
  relu_kernel<<<256, 256, 0, st>>>(m->Z2, m->H2, n);
  gemm_f32(st, rows, 1, H, m->H2, H, 1, m->W3(), 1, 1, y, 1, m->b3(), false);
  m->launches += 5;
}

}  // namespace

extern "C" {

int32_t ttg_mlp_create(int32_t in_features, int32_t hidden, uint64_t seed, ttg_mlp** out)
{
  set_last_error(std::string());
  if (!out || in_features <= 0 || hidden <= 0 || hidden > 4096 || in_features > 4096)
    return mfail(TTG_ERR_ARG, "mlp_create: bad arguments");
  auto* m = new ttg_mlp;
  m->F = in_features;
  m->H = hidden;
  m->nparams = in_features * hidden + hidden + hidden * hidden + hidden + hidden + 1;
  const size_t b = sizeof(float) * m->nparams;
  for (float** p : {&m->params, &m->grads, &m->m, &m->v})
    if (cudaMalloc(p, b) != cudaSuccess)
    {
      delete m;
      return mfail(TTG_ERR_OOM, "mlp_create: device allocation failed");
    }
  cudaMemset(m->m, 0, b);
  cudaMemset(m->v, 0, b);
  cudaMalloc(&m->loss, sizeof(double));
  // He-uniform initialisation from a seeded splitmix64 stream (host side).
  std::vector<float> h(static_cast<size_t>(m->nparams), 0.f);
  uint64_t z = seed;
  auto uni = [&]() {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return static_cast<float>((x >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
  };
  const float a1 = std::sqrt(6.f / in_features), a2 = std::sqrt(6.f / hidden);
  size_t o = 0;
  for (int i = 0; i < in_features * hidden; ++i)
    h[o++] = a1 * uni();
  o += hidden;
  for (int i = 0; i < hidden * hidden; ++i)
    h[o++] = a2 * uni();
  o += hidden;
  for (int i = 0; i < hidden; ++i)
    h[o++] = a2 * uni();
  cudaMemcpy(m->params, h.data(), b, cudaMemcpyHostToDevice);
  *out = m;
  return TTG_OK;
}

void ttg_mlp_destroy(ttg_mlp* m) { delete m; }

int32_t ttg_mlp_num_params(const ttg_mlp* m) { return m ? m->nparams : 0; }

int32_t ttg_mlp_get_params(ttg_mlp* m, float* host)
{
  if (!m || !host)
    return mfail(TTG_ERR_ARG, "mlp_get_params: null argument");
  MLP_CUDA(cudaMemcpy(host, m->params, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost));
  return TTG_OK;
}

int32_t ttg_mlp_set_params(ttg_mlp* m, const float* host)
{
  if (!m || !host)
    return mfail(TTG_ERR_ARG, "mlp_set_params: null argument");
  MLP_CUDA(cudaMemcpy(m->params, host, sizeof(float) * m->nparams, cudaMemcpyHostToDevice));
  return TTG_OK;
}

int32_t ttg_mlp_forward(ttg_mlp* m, const float* x_dev, int32_t rows, float* y_dev, void* stream)
{
  if (!m || rows < 0 || (rows > 0 && (!x_dev || !y_dev)))
    return mfail(TTG_ERR_ARG, "mlp_forward: bad arguments");
  if (rows == 0)
    return TTG_OK;
  if (int32_t st = ensure_rows(m, rows))
    return st;
  forward(m, x_dev, rows, y_dev, static_cast<cudaStream_t>(stream));
  MLP_CUDA(cudaGetLastError());
  if (tc_gemm_timed_out(static_cast<cudaStream_t>(stream)))
    return mfail(TTG_ERR_TIMEOUT, "mlp: a tensor-core MMA wait timed out");
  return TTG_OK;
}

// Gradient of the mean squared error at the current parameters into
// m->grads; loss written to *loss_host.  Synchronises `stream`.
static int32_t mlp_backward(ttg_mlp* m, const float* x, const float* t, int rows, cudaStream_t st,
                            double* loss_host)
{
  const int F = m->F, H = m->H;
  if (int32_t s = ensure_rows(m, rows))
    return s;
  const int64_t n = static_cast<int64_t>(rows) * H;
  forward(m, x, rows, m->y, st);
  MLP_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(double), st));
  mse_grad_kernel<<<64, 256, 0, st>>>(m->y, t, rows, m->dy, m->loss);
  // dW3 = H2^T dy (H x 1), db3 = sum dy
  gemm_f32(st, H, 1, rows, m->H2, 1, H, m->dy, 1, 1, m->gW3(), 1, nullptr, false);
  colsum_kernel<<<1, 32, 0, st>>>(m->dy, rows, 1, m->gb3());
  // dZ2 = (dy W3^T) * (Z2 > 0), into H2's buffer (H2 is consumed)
  gemm_f32(st, rows, H, 1, m->dy, 1, 1, m->W3(), 1, 1, m->H2, H, nullptr, false);
  relu_back_kernel<<<256, 256, 0, st>>>(m->H2, m->Z2, n);
  colsum_kernel<<<(H + 127) / 128, 128, 0, st>>>(m->H2, rows, H, m->gb2());
  // dW2 = H1^T dZ2
  gemm_f32(st, H, H, rows, m->H1, 1, H, m->H2, H, 1, m->gW2(), H, nullptr, false);
  // dZ1 = (dZ2 W2^T) * (Z1 > 0), into Z2's buffer (Z2 is consumed)
  gemm_f32(st, rows, H, H, m->H2, H, 1, m->W2(), 1, H, m->Z2, H, nullptr, false);
  relu_back_kernel<<<256, 256, 0, st>>>(m->Z2, m->Z1, n);
  colsum_kernel<<<(H + 127) / 128, 128, 0, st>>>(m->Z2, rows, H, m->gb1());
  // dW1 = x^T dZ1 (F x H)
  gemm_f32(st, F, H, rows, x, 1, F, m->Z2, H, 1, m->gW1(), H, nullptr, false);
  m->launches += 11;
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpyAsync(loss_host, m->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
  MLP_CUDA(cudaStreamSynchronize(st));
  if (tc_gemm_timed_out(st))
    return mfail(TTG_ERR_TIMEOUT, "mlp: a tensor-core MMA wait timed out");
  return TTG_OK;
}

int32_t ttg_mlp_gradients(ttg_mlp* m, const float* x_dev, const float* t_dev, int32_t rows,
                          float* grads_host, double* loss_host, void* stream)
{
  if (!m || rows <= 0 || !x_dev || !t_dev || !grads_host || !loss_host)
    return mfail(TTG_ERR_ARG, "mlp_gradients: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (int32_t s = mlp_backward(m, x_dev, t_dev, rows, st, loss_host))
    return s;
  MLP_CUDA(cudaMemcpy(grads_host, m->grads, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost));
  return TTG_OK;
}

int32_t ttg_mlp_train_step(ttg_mlp* m, const float* x_dev, const float* t_dev, int32_t rows,
                           float lr, double* loss_host, void* stream)
{
  if (!m || rows <= 0 || !x_dev || !t_dev || !loss_host)
    return mfail(TTG_ERR_ARG, "mlp_train_step: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (int32_t s = mlp_backward(m, x_dev, t_dev, rows, st, loss_host))
    return s;
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, static_cast<float>(m->step));
  const float c2 = 1.f - std::pow(b2, static_cast<float>(m->step));
  adam_kernel<<<64, 256, 0, st>>>(m->params, m->grads, m->m, m->v, m->nparams, lr, b1, b2, 1e-8f,
                                  c1, c2);
  m->launches += 1;
  MLP_CUDA(cudaGetLastError());
  return TTG_OK;
}

int64_t ttg_mlp_kernel_launches(const ttg_mlp* m) { return m ? m->launches : 0; }

}  // extern "C"
