// Learned cost model: a small MLP (n_in -> H -> H -> H -> 1, ReLU) trained on
// the GPU with hand-written forward, backward and Adam kernels (FP32 weights),
// with a bf16 inference path.  It predicts log(kernel time) of one pairwise
// contraction from shape features; the planner sums predictions over a plan's
// steps to rank candidate plans.
//
// Layout: activations are row-major [batch x features]; layer l has weights
// W_l [in x out] (row-major) and bias b_l [out].  Parameters are stored in one
// flat FP32 buffer in the order W1 b1 W2 b2 ... so they can be read/written
// as a single array.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "pq_internal.h"

namespace pq {
int check_status(Ctx* ctx);
}
using namespace pq;

namespace {

constexpr int TB = 16;  // tile of the small SIMT GEMMs

// C[M x N] = op(A) @ op(B) (+ bias[N]) with optional ReLU, FP32.
//   op(A) = A [M x K] (ta = 0) or A^T with A [K x M] (ta = 1)
//   op(B) = B [K x N] (tb = 0) or B^T with B [N x K] (tb = 1)
// beta = 1 accumulates into C.
__global__ void k_sgemm(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ C,
                        const float* __restrict__ bias, int M, int N, int K, int ta, int tb, int relu, float beta) {
  __shared__ float As[TB][TB + 1];
  __shared__ float Bs[TB][TB + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * TB + ty, col = blockIdx.x * TB + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += TB) {
    int ka = k0 + tx, kb = k0 + ty;
    float a = 0.f, b = 0.f;
    if (row < M && ka < K) a = ta ? A[(size_t)ka * M + row] : A[(size_t)row * K + ka];
    if (col < N && kb < K) b = tb ? B[(size_t)col * K + kb] : B[(size_t)kb * N + col];
    As[ty][tx] = a;
    Bs[ty][tx] = b;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TB; ++k) acc = fmaf(As[ty][k], Bs[k][tx], acc);
    __syncthreads();
  }
  if (row < M && col < N) {
    size_t o = (size_t)row * N + col;
    if (bias) acc += bias[col];
    if (beta != 0.f) acc += beta * C[o];
    if (relu) acc = acc > 0.f ? acc : 0.f;
    C[o] = acc;
  }
}

// Inference layer in bf16: weights and inputs rounded to bf16, FP32 accumulate.
__global__ void k_bf16_layer(const __nv_bfloat16* __restrict__ X, const __nv_bfloat16* __restrict__ W,
                             const float* __restrict__ bias, __nv_bfloat16* __restrict__ Y, float* __restrict__ yf,
                             int M, int N, int K, int relu) {
  __shared__ float Xs[TB][TB + 1];
  __shared__ float Ws[TB][TB + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * TB + ty, col = blockIdx.x * TB + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += TB) {
    int ka = k0 + tx, kb = k0 + ty;
    Xs[ty][tx] = (row < M && ka < K) ? __bfloat162float(X[(size_t)row * K + ka]) : 0.f;
    Ws[ty][tx] = (col < N && kb < K) ? __bfloat162float(W[(size_t)kb * N + col]) : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TB; ++k) acc = fmaf(Xs[ty][k], Ws[k][tx], acc);
    __syncthreads();
  }
  if (row < M && col < N) {
    acc += bias[col];
    if (relu) acc = acc > 0.f ? acc : 0.f;
    if (Y) Y[(size_t)row * N + col] = __float2bfloat16(acc);
    if (yf) yf[(size_t)row * N + col] = acc;
  }
}

// Gather training rows by index into the batch buffers.
__global__ void k_gather_rows(const float* __restrict__ X, const float* __restrict__ Y,
                              const int64_t* __restrict__ idx, int b, int n_in, float* __restrict__ xb,
                              float* __restrict__ yb) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= b) return;
  int64_t src = idx[r];
  for (int j = 0; j < n_in; ++j) xb[(size_t)r * n_in + j] = X[(size_t)src * n_in + j];
  yb[r] = Y[src];
}

__global__ void k_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// dY = 2 (y - t) / n for the MSE loss; also accumulates the loss sum.
__global__ void k_mse_grad(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy, int n,
                           float* loss) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < n) {
    float d = y[i] - t[i];
    dy[i] = 2.f * d / (float)n;
    l = d * d;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / (float)n);
}

// dZ *= (H > 0) (ReLU backward, H is the post-activation)
__global__ void k_relu_back(float* __restrict__ dz, const float* __restrict__ h, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && h[i] <= 0.f) dz[i] = 0.f;
}

// db[j] = sum_b dZ[b, j]
__global__ void k_colsum(const float* __restrict__ dz, float* __restrict__ db, int M, int N) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0.f;
  for (int b = 0; b < M; ++b) s += dz[(size_t)b * N + j];
  db[j] = s;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.f - b1) * gi;
  float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

void sgemm(const float* A, const float* B, float* C, const float* bias, int M, int N, int K, int ta, int tb, int relu,
           float beta, cudaStream_t s) {
  dim3 blk(TB, TB), grd((N + TB - 1) / TB, (M + TB - 1) / TB);
  k_sgemm<<<grd, blk, 0, s>>>(A, B, C, bias, M, N, K, ta, tb, relu, beta);
}

}  // namespace

struct pq_mlp {
  Ctx* ctx = nullptr;
  int n_in = 0, hidden = 0, layers = 0;  // `layers` hidden layers + 1 output layer
  std::vector<int> din, dout;            // per linear layer
  std::vector<int64_t> woff, boff;       // offsets in the flat parameter buffer
  int64_t n_params = 0;
  float* d_p = nullptr;
  float* d_g = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  int64_t step = 0;
  // workspace for a batch
  int cap = 0;
  std::vector<float*> act;  // act[0] = input, act[l+1] = output of layer l
  std::vector<float*> dact;
  float* d_t = nullptr;
  float* d_loss = nullptr;
  __nv_bfloat16* d_wbf = nullptr;
  __nv_bfloat16* d_xb[2] = {nullptr, nullptr};
};

namespace {

void free_ws(pq_mlp* m) {
  for (auto p : m->act) cudaFree(p);
  for (auto p : m->dact) cudaFree(p);
  m->act.clear();
  m->dact.clear();
  cudaFree(m->d_t);
  cudaFree(m->d_xb[0]);
  cudaFree(m->d_xb[1]);
  m->d_t = nullptr;
  m->d_xb[0] = m->d_xb[1] = nullptr;
  m->cap = 0;
}

int ensure_ws(pq_mlp* m, int n) {
  if (n <= m->cap) return PQ_OK;
  free_ws(m);
  const int L = (int)m->din.size();
  m->act.assign(L + 1, nullptr);
  m->dact.assign(L + 1, nullptr);
  cudaError_t e = cudaSuccess;
  for (int l = 0; l <= L; ++l) {
    int w = l == 0 ? m->n_in : m->dout[l - 1];
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->act[l], sizeof(float) * (size_t)n * w);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->dact[l], sizeof(float) * (size_t)n * w);
  }
  int wmax = std::max(m->n_in, m->hidden);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_t, sizeof(float) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_xb[0], sizeof(__nv_bfloat16) * (size_t)n * wmax);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_xb[1], sizeof(__nv_bfloat16) * (size_t)n * wmax);
  if (e != cudaSuccess) {
    free_ws(m);
    return cuda_fail(m->ctx, e, "mlp workspace");
  }
  m->cap = n;
  return PQ_OK;
}

// Forward pass (FP32) over n rows already in act[0].
void forward(pq_mlp* m, int n) {
  const int L = (int)m->din.size();
  for (int l = 0; l < L; ++l)
    sgemm(m->act[l], m->d_p + m->woff[l], m->act[l + 1], m->d_p + m->boff[l], n, m->dout[l], m->din[l], 0, 0,
          l + 1 < L ? 1 : 0, 0.f, m->ctx->stream);
}

// Backward pass: gradients of the mean squared error into d_g; returns with
// the loss in d_loss (device).
void backward(pq_mlp* m, int n) {
  const int L = (int)m->din.size();
  cudaStream_t s = m->ctx->stream;
  cudaMemsetAsync(m->d_loss, 0, sizeof(float), s);
  k_mse_grad<<<(n + 255) / 256, 256, 0, s>>>(m->act[L], m->d_t, m->dact[L], n, m->d_loss);
  for (int l = L - 1; l >= 0; --l) {
    // dW_l = act[l]^T dact[l+1];  db_l = colsum(dact[l+1])
    sgemm(m->act[l], m->dact[l + 1], m->d_g + m->woff[l], nullptr, m->din[l], m->dout[l], n, 1, 0, 0, 0.f, s);
    k_colsum<<<(m->dout[l] + 127) / 128, 128, 0, s>>>(m->dact[l + 1], m->d_g + m->boff[l], n, m->dout[l]);
    if (l > 0) {
      // dact[l] = dact[l+1] W_l^T, masked by ReLU of act[l]
      sgemm(m->dact[l + 1], m->d_p + m->woff[l], m->dact[l], nullptr, n, m->din[l], m->dout[l], 0, 1, 0, 0.f, s);
      int64_t sz = (int64_t)n * m->din[l];
      k_relu_back<<<(unsigned)((sz + 255) / 256), 256, 0, s>>>(m->dact[l], m->act[l], sz);
    }
  }
}

}  // namespace

extern "C" {

int pq_mlp_create(pq_ctx* c, int n_in, int hidden, int hidden_layers, uint64_t seed, pq_mlp** out) {
  if (!c || !out || n_in < 1 || hidden < 1 || hidden_layers < 1) return PQ_ERR_INVALID;
  Ctx* ctx = &c->impl;
  pq_mlp* m = new pq_mlp();
  m->ctx = ctx;
  m->n_in = n_in;
  m->hidden = hidden;
  m->layers = hidden_layers;
  int w = n_in;
  for (int l = 0; l < hidden_layers; ++l) {
    m->din.push_back(w);
    m->dout.push_back(hidden);
    w = hidden;
  }
  m->din.push_back(w);
  m->dout.push_back(1);
  for (size_t l = 0; l < m->din.size(); ++l) {
    m->woff.push_back(m->n_params);
    m->n_params += (int64_t)m->din[l] * m->dout[l];
    m->boff.push_back(m->n_params);
    m->n_params += m->dout[l];
  }
  // He-uniform initialisation (host, seeded), zero biases
  std::vector<float> h((size_t)m->n_params, 0.f);
  std::mt19937_64 rng(seed);
  for (size_t l = 0; l < m->din.size(); ++l) {
    float a = std::sqrt(6.f / (float)m->din[l]);
    std::uniform_real_distribution<float> U(-a, a);
    for (int64_t i = 0; i < (int64_t)m->din[l] * m->dout[l]; ++i) h[m->woff[l] + i] = U(rng);
  }
  cudaError_t e = cudaMalloc((void**)&m->d_p, sizeof(float) * m->n_params);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_g, sizeof(float) * m->n_params);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_m, sizeof(float) * m->n_params);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_v, sizeof(float) * m->n_params);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_wbf, sizeof(__nv_bfloat16) * m->n_params);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_p, h.data(), sizeof(float) * m->n_params, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, sizeof(float) * m->n_params);
  if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, sizeof(float) * m->n_params);
  if (e != cudaSuccess) {
    cudaFree(m->d_p);
    cudaFree(m->d_g);
    cudaFree(m->d_m);
    cudaFree(m->d_v);
    cudaFree(m->d_loss);
    cudaFree(m->d_wbf);
    delete m;
    return cuda_fail(ctx, e, "mlp create");
  }
  *out = m;
  return PQ_OK;
}

int pq_mlp_destroy(pq_mlp* m) {
  if (!m) return PQ_ERR_INVALID;
  cudaStreamSynchronize(m->ctx->stream);
  free_ws(m);
  cudaFree(m->d_p);
  cudaFree(m->d_g);
  cudaFree(m->d_m);
  cudaFree(m->d_v);
  cudaFree(m->d_loss);
  cudaFree(m->d_wbf);
  delete m;
  return PQ_OK;
}

int pq_mlp_num_params(pq_mlp* m, int64_t* n) {
  if (!m || !n) return PQ_ERR_INVALID;
  *n = m->n_params;
  return PQ_OK;
}

int pq_mlp_get_params(pq_mlp* m, float* w, int64_t n) {
  if (!m || !w || n < m->n_params) return PQ_ERR_INVALID;
  cudaError_t e = cudaMemcpyAsync(w, m->d_p, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost, m->ctx->stream);
  if (e != cudaSuccess) return cuda_fail(m->ctx, e, "mlp get params");
  return check_status(m->ctx);
}

int pq_mlp_set_params(pq_mlp* m, const float* w, int64_t n) {
  if (!m || !w || n != m->n_params) return PQ_ERR_INVALID;
  cudaError_t e = cudaMemcpyAsync(m->d_p, w, sizeof(float) * m->n_params, cudaMemcpyHostToDevice, m->ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_m, 0, sizeof(float) * m->n_params, m->ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_v, 0, sizeof(float) * m->n_params, m->ctx->stream);
  if (e != cudaSuccess) return cuda_fail(m->ctx, e, "mlp set params");
  m->step = 0;
  return check_status(m->ctx);
}

int pq_mlp_gradients(pq_mlp* m, const float* X, const float* y, int64_t n, float* grad, float* loss) {
  if (!m || !X || !y || !grad || n < 1 || n > (1 << 24)) return PQ_ERR_INVALID;
  int st = ensure_ws(m, (int)n);
  if (st) return st;
  cudaStream_t s = m->ctx->stream;
  cudaMemcpyAsync(m->act[0], X, sizeof(float) * n * m->n_in, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(m->d_t, y, sizeof(float) * n, cudaMemcpyHostToDevice, s);
  forward(m, (int)n);
  backward(m, (int)n);
  cudaMemcpyAsync(grad, m->d_g, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost, s);
  float l = 0;
  cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(m->ctx, e, "mlp gradients");
  st = check_status(m->ctx);
  if (loss) *loss = l;
  return st;
}

int pq_mlp_train(pq_mlp* m, const float* X, const float* y, int64_t n, int epochs, int batch, float lr,
                 uint64_t seed, float* final_loss) {
  if (!m || !X || !y || n < 1 || epochs < 1 || batch < 1) return PQ_ERR_INVALID;
  Ctx* ctx = m->ctx;
  cudaStream_t s = ctx->stream;
  // the whole data set lives on the device; batches are gathered by index
  float *dX = nullptr, *dY = nullptr;
  int64_t* dperm = nullptr;
  cudaError_t e = cudaMalloc((void**)&dX, sizeof(float) * n * m->n_in);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dY, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dperm, sizeof(int64_t) * n);
  if (e != cudaSuccess) {
    cudaFree(dX);
    cudaFree(dY);
    return cuda_fail(ctx, e, "mlp train data");
  }
  cudaMemcpyAsync(dX, X, sizeof(float) * n * m->n_in, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dY, y, sizeof(float) * n, cudaMemcpyHostToDevice, s);
  const int b = (int)std::min<int64_t>(batch, n);
  int st = ensure_ws(m, b);
  if (st) {
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dperm);
    return st;
  }
  std::mt19937_64 rng(seed);
  std::vector<int64_t> perm(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = i;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float last = 0.f;
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    // contiguous shuffled chunks: copy rows with one memcpy per chunk of the
    // permutation (rows are small, so gather on the host-side index list)
    e = cudaMemcpyAsync(dperm, perm.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) break;
    for (int64_t i0 = 0; i0 + b <= n; i0 += b) {
      k_gather_rows<<<(b + 127) / 128, 128, 0, s>>>(dX, dY, dperm + i0, b, m->n_in, m->act[0], m->d_t);
      forward(m, b);
      backward(m, b);
      ++m->step;
      float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
      k_adam<<<(unsigned)((m->n_params + 255) / 256), 256, 0, s>>>(m->d_p, m->d_g, m->d_m, m->d_v, m->n_params, lr,
                                                                    b1, b2, eps, c1, c2);
    }
    e = cudaMemcpyAsync(&last, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) break;
  }
  cudaFree(dX);
  cudaFree(dY);
  cudaFree(dperm);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp train");
  if (final_loss) *final_loss = last;
  return check_status(ctx);
}

int pq_mlp_predict(pq_mlp* m, const float* X, int64_t n, float* out, int bf16) {
  if (!m || !X || !out || n < 1 || n > (1 << 24)) return PQ_ERR_INVALID;
  int st = ensure_ws(m, (int)n);
  if (st) return st;
  cudaStream_t s = m->ctx->stream;
  const int L = (int)m->din.size();
  cudaMemcpyAsync(m->act[0], X, sizeof(float) * n * m->n_in, cudaMemcpyHostToDevice, s);
  if (!bf16) {
    forward(m, (int)n);
  } else {
    k_to_bf16<<<(unsigned)((m->n_params + 255) / 256), 256, 0, s>>>(m->d_p, m->d_wbf, m->n_params);
    k_to_bf16<<<(unsigned)((n * m->n_in + 255) / 256), 256, 0, s>>>(m->act[0], m->d_xb[0], n * m->n_in);
    int cur = 0;
    for (int l = 0; l < L; ++l) {
      dim3 blk(TB, TB), grd((m->dout[l] + TB - 1) / TB, (unsigned)((n + TB - 1) / TB));
      const bool last = l + 1 == L;
      k_bf16_layer<<<grd, blk, 0, s>>>(m->d_xb[cur], m->d_wbf + m->woff[l], m->d_p + m->boff[l],
                                        last ? nullptr : m->d_xb[1 - cur], last ? m->act[L] : nullptr, (int)n,
                                        m->dout[l], m->din[l], last ? 0 : 1);
      cur = 1 - cur;
    }
  }
  cudaMemcpyAsync(out, m->act[L], sizeof(float) * n, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(m->ctx, e, "mlp predict");
  return check_status(m->ctx);
}

}  // extern "C"
