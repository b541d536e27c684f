// hbi_mlp.cu -- training and inference kernels of the learned step-size
// proposer (no counterpart in the reference).
//
// The network is nin -> hid -> hid -> 1 with tanh hidden layers and a linear
// output, parameters packed [W1(hid x nin) b1 W2(hid x hid) b2 W3(hid) b3]
// row-major (the same packing the time loop's proposer reads).  The loss is
// the mean over a minibatch of the squared error, or (hbi_mlp_set_loss) of
// the pinball loss of quantile tau: (1 - tau) r for r = out - t > 0, -tau r
// otherwise, whose minimiser is the tau-quantile of the target given the
// inputs.
//
//   mlp_forward_kernel   one thread per sample: activations A1, A2, output,
//                        and the backpropagated deltas D2, D1 (weights in
//                        shared memory)
//   mlp_grad_kernel      one thread per parameter: the sum over the batch of
//                        delta x activation, in sample order (deterministic)
//   mlp_adam_kernel      one thread per parameter: Adam update
//   mlp_loss_kernel      one block: the batch loss, in sample order
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/hbi_gpu.h"

namespace hbi {
int set_error(int code, const char* msg);
}

namespace {

constexpr int kMaxHid = 128;
constexpr int kMaxIn = 32;

__host__ __device__ inline int mlp_nparams(int nin, int hid) { return hid * nin + hid + hid * hid + hid + hid + 1; }

// per-sample forward and backward; `idx` selects the minibatch rows of X, T
__global__ void __launch_bounds__(128) mlp_forward_kernel(const float* __restrict__ P, int nin, int hid,
                                                          const float* __restrict__ X, const float* __restrict__ T,
                                                          const int* __restrict__ idx, int batch,
                                                          float* __restrict__ A1, float* __restrict__ A2,
                                                          float* __restrict__ D1, float* __restrict__ D2,
                                                          float* __restrict__ DY, float* __restrict__ R,
                                                          float* __restrict__ Y, float tau) {
  extern __shared__ float sp[];
  const int np = mlp_nparams(nin, hid);
  for (int i = threadIdx.x; i < np; i += blockDim.x) sp[i] = P[i];
  __syncthreads();
  const float* W1 = sp;
  const float* b1 = W1 + hid * nin;
  const float* W2 = b1 + hid;
  const float* b2 = W2 + hid * hid;
  const float* W3 = b2 + hid;
  const float b3 = W3[hid];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= batch) return;
  const int row = idx ? idx[s] : s;
  float x[kMaxIn], a1[kMaxHid], a2[kMaxHid];
  for (int i = 0; i < nin; i++) x[i] = X[(size_t)row * nin + i];
  for (int o = 0; o < hid; o++) {
    float z = b1[o];
    for (int i = 0; i < nin; i++) z += W1[o * nin + i] * x[i];
    a1[o] = tanhf(z);
    A1[(size_t)s * hid + o] = a1[o];
  }
  float y = b3;
  for (int o = 0; o < hid; o++) {
    float z = b2[o];
    for (int i = 0; i < hid; i++) z += W2[o * hid + i] * a1[i];
    a2[o] = tanhf(z);
    A2[(size_t)s * hid + o] = a2[o];
    y += W3[o] * a2[o];
  }
  if (Y) Y[s] = y;
  if (!T) return;
  const float r = y - T[row];
  // per-sample loss and its derivative in the output (a subgradient of 0 at
  // r = 0 for the pinball loss)
  float dy;
  if (tau > 0.0f) {
    R[s] = r > 0.0f ? (1.0f - tau) * r : -tau * r;
    dy = (r > 0.0f ? 1.0f - tau : (r < 0.0f ? -tau : 0.0f)) / (float)batch;
  } else {
    R[s] = r * r;
    dy = 2.0f * r / (float)batch;
  }
  DY[s] = dy;
  // D2 = dy W3 (1 - a2^2); D1 = (W2^T D2) (1 - a1^2)
  for (int o = 0; o < hid; o++) {
    const float d = dy * W3[o] * (1.0f - a2[o] * a2[o]);
    a2[o] = d;
    D2[(size_t)s * hid + o] = d;
  }
  for (int i = 0; i < hid; i++) {
    float acc = 0.0f;
    for (int o = 0; o < hid; o++) acc += a2[o] * W2[o * hid + i];
    D1[(size_t)s * hid + i] = acc * (1.0f - a1[i] * a1[i]);
  }
}

// gradient of parameter p: sum over the batch in sample order
__global__ void __launch_bounds__(256) mlp_grad_kernel(int nin, int hid, const float* __restrict__ X,
                                                       const int* __restrict__ idx, int batch,
                                                       const float* __restrict__ A1, const float* __restrict__ A2,
                                                       const float* __restrict__ D1, const float* __restrict__ D2,
                                                       const float* __restrict__ DY, float* __restrict__ G) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int nW1 = hid * nin, ob1 = nW1, oW2 = ob1 + hid, ob2 = oW2 + hid * hid, oW3 = ob2 + hid, ob3 = oW3 + hid;
  if (p > ob3) return;
  float g = 0.0f;
  if (p < ob1) {
    const int o = p / nin, i = p % nin;
    for (int s = 0; s < batch; s++) g += D1[(size_t)s * hid + o] * X[(size_t)(idx ? idx[s] : s) * nin + i];
  } else if (p < oW2) {
    const int o = p - ob1;
    for (int s = 0; s < batch; s++) g += D1[(size_t)s * hid + o];
  } else if (p < ob2) {
    const int o = (p - oW2) / hid, i = (p - oW2) % hid;
    for (int s = 0; s < batch; s++) g += D2[(size_t)s * hid + o] * A1[(size_t)s * hid + i];
  } else if (p < oW3) {
    const int o = p - ob2;
    for (int s = 0; s < batch; s++) g += D2[(size_t)s * hid + o];
  } else if (p < ob3) {
    const int i = p - oW3;
    for (int s = 0; s < batch; s++) g += DY[s] * A2[(size_t)s * hid + i];
  } else {
    for (int s = 0; s < batch; s++) g += DY[s];
  }
  G[p] = g;
}

__global__ void mlp_adam_kernel(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                                float* __restrict__ V, int np, float lr, float b1, float b2, float eps, float c1,
                                float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const float g = G[p];
  const float m = b1 * M[p] + (1.0f - b1) * g;
  const float v = b2 * V[p] + (1.0f - b2) * g * g;
  M[p] = m;
  V[p] = v;
  P[p] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// mean of r^2 over the batch, summed in sample order by one block
__global__ void mlp_loss_kernel(const float* __restrict__ R, int batch, float* __restrict__ loss) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < batch; i += blockDim.x) s += (double)R[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = (float)(sh[0] / batch);
}

int mfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return hbi::set_error(code, buf);
}

#define MCK(x)                                                                                        \
  do {                                                                                                \
    cudaError_t e_ = (x);                                                                             \
    if (e_ != cudaSuccess) return mfail(HBI_ERR_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

}  // namespace

struct hbi_mlp_s {
  int nin = 0, hid = 0, np = 0, bmax = 0;
  long long nmax = 0;
  float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;
  float *A1 = nullptr, *A2 = nullptr, *D1 = nullptr, *D2 = nullptr, *DY = nullptr, *R = nullptr, *Y = nullptr;
  float *X = nullptr, *T = nullptr, *loss = nullptr;
  int* idx = nullptr;
  long long step = 0;
  float tau = -1.0f;  // <= 0: squared error; in (0, 1): pinball loss of that quantile
  cudaStream_t st = nullptr;
};

namespace {

int ensure_data(hbi_mlp* m, long long n) {
  if (n <= m->nmax) return HBI_OK;
  cudaFree(m->X);
  cudaFree(m->T);
  cudaFree(m->idx);
  m->X = m->T = nullptr;
  m->idx = nullptr;
  m->nmax = 0;
  MCK(cudaMalloc(&m->X, sizeof(float) * n * m->nin));
  MCK(cudaMalloc(&m->T, sizeof(float) * n));
  MCK(cudaMalloc(&m->idx, sizeof(int) * n));
  m->nmax = n;
  return HBI_OK;
}

void launch_fwd(hbi_mlp* m, const int* idx, int b, bool with_target) {
  const size_t shm = sizeof(float) * m->np;
  mlp_forward_kernel<<<(b + 127) / 128, 128, shm, m->st>>>(m->P, m->nin, m->hid, m->X, with_target ? m->T : nullptr,
                                                          idx, b, m->A1, m->A2, m->D1, m->D2, m->DY, m->R, m->Y,
                                                          m->tau);
}

void launch_bwd(hbi_mlp* m, const int* idx, int b) {
  mlp_grad_kernel<<<(m->np + 255) / 256, 256, 0, m->st>>>(m->nin, m->hid, m->X, idx, b, m->A1, m->A2, m->D1, m->D2,
                                                          m->DY, m->G);
}

}  // namespace

extern "C" int hbi_mlp_free(hbi_mlp* m) {
  if (!m) return HBI_OK;
  if (m->st) cudaStreamSynchronize(m->st);
  for (float* p : {m->P, m->G, m->M, m->V, m->A1, m->A2, m->D1, m->D2, m->DY, m->R, m->Y, m->X, m->T, m->loss})
    cudaFree(p);
  cudaFree(m->idx);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  return HBI_OK;
}

extern "C" int hbi_mlp_create(hbi_mlp** out, int nin, int hid, int batch_max) {
  if (!out || nin < 1 || nin > kMaxIn || hid < 1 || hid > kMaxHid || batch_max < 1)
    return mfail(HBI_ERR_ARG, "hbi_mlp_create: nin in 1..%d, hid in 1..%d, batch_max >= 1", kMaxIn, kMaxHid);
  hbi_mlp* m = new hbi_mlp_s();
  m->nin = nin;
  m->hid = hid;
  m->np = mlp_nparams(nin, hid);
  m->bmax = batch_max;
  const size_t bh = (size_t)batch_max * hid;
  bool ok = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) == cudaSuccess;
  for (auto pr : {std::make_pair(&m->P, (size_t)m->np), std::make_pair(&m->G, (size_t)m->np),
                  std::make_pair(&m->M, (size_t)m->np), std::make_pair(&m->V, (size_t)m->np),
                  std::make_pair(&m->A1, bh), std::make_pair(&m->A2, bh), std::make_pair(&m->D1, bh),
                  std::make_pair(&m->D2, bh), std::make_pair(&m->DY, (size_t)batch_max),
                  std::make_pair(&m->R, (size_t)batch_max), std::make_pair(&m->Y, (size_t)batch_max),
                  std::make_pair(&m->loss, (size_t)1)})
    ok = ok && cudaMalloc(pr.first, sizeof(float) * pr.second) == cudaSuccess;
  if (!ok) {
    hbi_mlp_free(m);
    return mfail(HBI_ERR_NOMEM, "hbi_mlp_create: allocation");
  }
  const size_t shm = sizeof(float) * m->np;
  if (shm > 48 * 1024 &&
      cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) != cudaSuccess) {
    hbi_mlp_free(m);
    return mfail(HBI_ERR_ARG, "hbi_mlp_create: %d parameters do not fit in shared memory", m->np);
  }
  cudaMemsetAsync(m->P, 0, sizeof(float) * m->np, m->st);
  cudaMemsetAsync(m->M, 0, sizeof(float) * m->np, m->st);
  cudaMemsetAsync(m->V, 0, sizeof(float) * m->np, m->st);
  *out = m;
  return HBI_OK;
}

extern "C" int hbi_mlp_set_params(hbi_mlp* m, const float* p) {
  if (!m || !p) return mfail(HBI_ERR_ARG, "null");
  MCK(cudaMemcpyAsync(m->P, p, sizeof(float) * m->np, cudaMemcpyHostToDevice, m->st));
  MCK(cudaMemsetAsync(m->M, 0, sizeof(float) * m->np, m->st));
  MCK(cudaMemsetAsync(m->V, 0, sizeof(float) * m->np, m->st));
  MCK(cudaStreamSynchronize(m->st));
  m->step = 0;
  return HBI_OK;
}

extern "C" int hbi_mlp_get_params(hbi_mlp* m, float* p) {
  if (!m || !p) return mfail(HBI_ERR_ARG, "null");
  MCK(cudaMemcpyAsync(p, m->P, sizeof(float) * m->np, cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  return HBI_OK;
}

extern "C" int hbi_mlp_set_loss(hbi_mlp* m, float tau) {
  if (!m || !(tau < 1.0f)) return mfail(HBI_ERR_ARG, "hbi_mlp_set_loss: tau must be below 1");
  m->tau = tau > 0.0f ? tau : -1.0f;
  return HBI_OK;
}

extern "C" int hbi_mlp_loss_grad(hbi_mlp* m, const float* x, const float* t, int batch, float* grad, float* loss,
                                 float* out) {
  if (!m || !x || !t || batch < 1 || batch > m->bmax) return mfail(HBI_ERR_ARG, "hbi_mlp_loss_grad: arguments");
  int rc = ensure_data(m, batch);
  if (rc) return rc;
  MCK(cudaMemcpyAsync(m->X, x, sizeof(float) * batch * m->nin, cudaMemcpyHostToDevice, m->st));
  MCK(cudaMemcpyAsync(m->T, t, sizeof(float) * batch, cudaMemcpyHostToDevice, m->st));
  launch_fwd(m, nullptr, batch, true);
  launch_bwd(m, nullptr, batch);
  mlp_loss_kernel<<<1, 256, 0, m->st>>>(m->R, batch, m->loss);
  MCK(cudaGetLastError());
  if (grad) MCK(cudaMemcpyAsync(grad, m->G, sizeof(float) * m->np, cudaMemcpyDeviceToHost, m->st));
  if (loss) MCK(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
  if (out) MCK(cudaMemcpyAsync(out, m->Y, sizeof(float) * batch, cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  return HBI_OK;
}

extern "C" int hbi_mlp_train(hbi_mlp* m, const float* x, const float* t, long long n, int epochs, int batch,
                             float lr, unsigned long long seed, float* loss_per_epoch) {
  if (!m || !x || !t || n < 1 || epochs < 1 || batch < 1 || batch > m->bmax)
    return mfail(HBI_ERR_ARG, "hbi_mlp_train: arguments");
  int rc = ensure_data(m, n);
  if (rc) return rc;
  MCK(cudaMemcpyAsync(m->X, x, sizeof(float) * n * m->nin, cudaMemcpyHostToDevice, m->st));
  MCK(cudaMemcpyAsync(m->T, t, sizeof(float) * n, cudaMemcpyHostToDevice, m->st));
  std::vector<int> perm(n);
  for (long long i = 0; i < n; i++) perm[i] = (int)i;
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
  auto rnd = [&]() {  // xorshift64*
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return s * 0x2545F4914F6CDD1Dull;
  };
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  std::vector<float> lossv;
  for (int e = 0; e < epochs; e++) {
    for (long long i = n - 1; i > 0; i--) std::swap(perm[i], perm[rnd() % (uint64_t)(i + 1)]);
    MCK(cudaMemcpyAsync(m->idx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->st));
    double sum = 0.0;
    int nb = 0;
    for (long long b0 = 0; b0 + batch <= n; b0 += batch) {
      launch_fwd(m, m->idx + b0, batch, true);
      launch_bwd(m, m->idx + b0, batch);
      m->step++;
      const float c1 = 1.0f - powf(b1, (float)m->step), c2 = 1.0f - powf(b2, (float)m->step);
      mlp_adam_kernel<<<(m->np + 255) / 256, 256, 0, m->st>>>(m->P, m->G, m->M, m->V, m->np, lr, b1, b2, eps, c1, c2);
      if (loss_per_epoch) {
        mlp_loss_kernel<<<1, 256, 0, m->st>>>(m->R, batch, m->loss);
        float l;
        MCK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
        MCK(cudaStreamSynchronize(m->st));
        sum += l;
        nb++;
      }
    }
    MCK(cudaGetLastError());
    if (loss_per_epoch) loss_per_epoch[e] = nb ? (float)(sum / nb) : 0.0f;
  }
  MCK(cudaStreamSynchronize(m->st));
  return HBI_OK;
}

extern "C" int hbi_mlp_predict(hbi_mlp* m, const float* x, long long n, float* out) {
  if (!m || !x || !out || n < 1) return mfail(HBI_ERR_ARG, "hbi_mlp_predict: arguments");
  int rc = ensure_data(m, n);
  if (rc) return rc;
  MCK(cudaMemcpyAsync(m->X, x, sizeof(float) * n * m->nin, cudaMemcpyHostToDevice, m->st));
  for (long long b0 = 0; b0 < n; b0 += m->bmax) {
    const int b = (int)std::min<long long>(m->bmax, n - b0);
    std::vector<int> ids(b);
    for (int i = 0; i < b; i++) ids[i] = (int)(b0 + i);
    MCK(cudaMemcpyAsync(m->idx, ids.data(), sizeof(int) * b, cudaMemcpyHostToDevice, m->st));
    launch_fwd(m, m->idx, b, false);
    MCK(cudaMemcpyAsync(out + b0, m->Y, sizeof(float) * b, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
  }
  return HBI_OK;
}
