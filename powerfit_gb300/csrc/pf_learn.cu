// Learned rotation proposal: the scoring network's forward, gradient and
// Adam kernels (C ABI in include/powerfit_gb300.h).
//
// The network scores one rotation from F features of the coarse search:
//   h1 = relu(W1 x + b1)   (H x F)
//   h2 = relu(W2 h1 + b2)  (H x H)
//   y  = w3 . h2 + b3
// Weights are held in bfloat16 for the forward and gradient kernels, with
// float32 accumulation; the optimiser keeps a float32 master copy and writes
// the bfloat16 copy after every step.  Parameters are one flat vector:
// [W1 (H*F), b1 (H), W2 (H*H), b2 (H), w3 (H), b3 (1)].
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "../../include/powerfit_gb300.h"

namespace {

thread_local char g_learn_err[256] = "";

int learn_fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_learn_err, sizeof(g_learn_err), fmt, ap);
  va_end(ap);
  return code;
}

constexpr int kMaxIn = 64;        // features per sample
constexpr int kTile = 128;        // samples per block in the gradient kernel

__host__ __device__ inline long long param_count(int F, int H) { return (long long)H * F + H + (long long)H * H + H + H + 1; }

// bfloat16 parameters -> float32 in shared memory
__device__ inline void load_params(const __nv_bfloat16* __restrict__ pb, float* w, int P) {
  for (int i = threadIdx.x; i < P; i += blockDim.x) w[i] = __bfloat162float(pb[i]);
}

template <int H>
__global__ void k_mlp_forward(const float* __restrict__ x, long long n, int F, const __nv_bfloat16* __restrict__ pb,
                              float* __restrict__ y) {
  extern __shared__ float w[];
  const int P = (int)param_count(F, H);
  load_params(pb, w, P);
  __syncthreads();
  const float* W1 = w;
  const float* b1 = W1 + H * F;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* w3 = b2 + H;
  const float b3 = w3[H];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float* xi = x + i * F;
    float h1[H];
#pragma unroll
    for (int h = 0; h < H; ++h) h1[h] = b1[h];
    for (int f = 0; f < F; ++f) {
      const float xv = xi[f];
#pragma unroll
      for (int h = 0; h < H; ++h) h1[h] = fmaf(W1[h * F + f], xv, h1[h]);
    }
#pragma unroll
    for (int h = 0; h < H; ++h) h1[h] = fmaxf(h1[h], 0.f);
    float out = b3;
#pragma unroll 4
    for (int j = 0; j < H; ++j) {
      float a = b2[j];
#pragma unroll
      for (int k = 0; k < H; ++k) a = fmaf(W2[j * H + k], h1[k], a);
      out = fmaf(w3[j], fmaxf(a, 0.f), out);
    }
    y[i] = out;
  }
}

// Gradient of  L = sum_i c_i (y_i - t_i)^2,  c_i = scale * (w_i or 1),  added
// into `grad` (P floats) and L into `loss`.  Each block takes tiles of kTile
// samples: one thread per sample runs the forward and the backward pass and
// leaves its activations and deltas in shared memory; then every thread sums
// its share of the P parameter gradients over the tile's samples and adds
// them into `grad` with one atomic each.
template <int H>
__global__ void __launch_bounds__(kTile) k_mlp_grad(const float* __restrict__ x, const float* __restrict__ t,
                                                    const float* __restrict__ wt, long long n, int F,
                                                    const __nv_bfloat16* __restrict__ pb, float scale,
                                                    float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ float sm[];
  const int P = (int)param_count(F, H);
  float* w = sm;                          // parameters (float)
  float* sx = w + P;                      // [kTile][F]
  float* sh1 = sx + kTile * F;            // [kTile][H] relu(W1 x + b1)
  float* sh2 = sh1 + kTile * H;           // [kTile][H] relu(W2 h1 + b2)
  float* sd2 = sh2 + kTile * H;           // [kTile][H] dL/d(W2 h1 + b2)
  float* sd1 = sd2 + kTile * H;           // [kTile][H] dL/d(W1 x + b1)
  float* sdy = sd1 + kTile * H;           // [kTile]
  __shared__ float s_loss[kTile / 32];
  load_params(pb, w, P);
  __syncthreads();
  const float* W1 = w;
  const float* b1 = W1 + H * F;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* w3 = b2 + H;
  const float b3 = w3[H];
  const int s = threadIdx.x;
  float lsum = 0.f;
  for (long long base = (long long)blockIdx.x * kTile; base < n; base += (long long)gridDim.x * kTile) {
    const long long i = base + s;
    const bool live = i < n;
    // forward and backward of sample i (zeros for a sample past the end)
    float h1[H], a2[H];
#pragma unroll
    for (int h = 0; h < H; ++h) h1[h] = b1[h];
    for (int f = 0; f < F; ++f) {
      const float xv = live ? x[i * F + f] : 0.f;
      sx[s * F + f] = xv;
#pragma unroll
      for (int h = 0; h < H; ++h) h1[h] = fmaf(W1[h * F + f], xv, h1[h]);
    }
#pragma unroll
    for (int h = 0; h < H; ++h) h1[h] = fmaxf(h1[h], 0.f);
    float out = b3;
#pragma unroll 4
    for (int j = 0; j < H; ++j) {
      float a = b2[j];
#pragma unroll
      for (int k = 0; k < H; ++k) a = fmaf(W2[j * H + k], h1[k], a);
      a2[j] = a;
      out = fmaf(w3[j], fmaxf(a, 0.f), out);
    }
    float dy = 0.f;
    if (live) {
      const float c = scale * (wt ? wt[i] : 1.f);
      const float r = out - t[i];
      lsum += c * r * r;
      dy = 2.f * c * r;
    }
    sdy[s] = dy;
    float d1[H];
#pragma unroll
    for (int k = 0; k < H; ++k) d1[k] = 0.f;
#pragma unroll 4
    for (int j = 0; j < H; ++j) {
      const float d2 = a2[j] > 0.f ? dy * w3[j] : 0.f;
      sh2[s * H + j] = fmaxf(a2[j], 0.f);
      sd2[s * H + j] = d2;
#pragma unroll
      for (int k = 0; k < H; ++k) d1[k] = fmaf(d2, W2[j * H + k], d1[k]);
    }
#pragma unroll
    for (int k = 0; k < H; ++k) {
      sh1[s * H + k] = h1[k];
      sd1[s * H + k] = h1[k] > 0.f ? d1[k] : 0.f;
    }
    __syncthreads();
    // parameter gradients summed over the tile
    for (int e = threadIdx.x; e < P; e += kTile) {
      float g = 0.f;
      if (e < H * F) {                                   // W1[h][f] += d1[h] x[f]
        const int h = e / F, f = e - h * F;
        for (int q = 0; q < kTile; ++q) g = fmaf(sd1[q * H + h], sx[q * F + f], g);
      } else if (e < H * F + H) {                        // b1
        const int h = e - H * F;
        for (int q = 0; q < kTile; ++q) g += sd1[q * H + h];
      } else if (e < H * F + H + H * H) {                // W2[j][k] += d2[j] h1[k]
        const int r = e - (H * F + H), j = r / H, k = r - j * H;
        for (int q = 0; q < kTile; ++q) g = fmaf(sd2[q * H + j], sh1[q * H + k], g);
      } else if (e < H * F + 2 * H + H * H) {            // b2
        const int j = e - (H * F + H + H * H);
        for (int q = 0; q < kTile; ++q) g += sd2[q * H + j];
      } else if (e < H * F + 3 * H + H * H) {            // w3[j] += dy h2[j]
        const int j = e - (H * F + 2 * H + H * H);
        for (int q = 0; q < kTile; ++q) g = fmaf(sdy[q], sh2[q * H + j], g);
      } else {                                           // b3
        for (int q = 0; q < kTile; ++q) g += sdy[q];
      }
      atomicAdd(grad + e, g);
    }
    __syncthreads();
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
  if ((threadIdx.x & 31) == 0) s_loss[threadIdx.x >> 5] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f;
    for (int k = 0; k < kTile / 32; ++k) a += s_loss[k];
    atomicAdd(loss, a);
  }
}

// Adam (bias-corrected) on the float32 master parameters; the bfloat16 copy
// is rounded to nearest from the updated master
__global__ void k_adam(float* __restrict__ p, __nv_bfloat16* __restrict__ pb, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, long long count, float lr, float beta1,
                       float beta2, float eps, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
  }
}

bool hidden_ok(int H) { return H == 16 || H == 32 || H == 64; }

size_t grad_smem(int F, int H) {
  return ((size_t)param_count(F, H) + (size_t)kTile * F + 4 * (size_t)kTile * H + kTile) * sizeof(float);
}

template <int H>
cudaError_t launch_forward(const float* x, long long n, int F, const void* pb, float* y, cudaStream_t s) {
  const size_t smem = (size_t)param_count(F, H) * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_forward<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long blocks = (n + 255) / 256;
  k_mlp_forward<H><<<(unsigned)(blocks < 4096 ? (blocks > 0 ? blocks : 1) : 4096), 256, smem, s>>>(
      x, n, F, (const __nv_bfloat16*)pb, y);
  return cudaGetLastError();
}

template <int H>
cudaError_t launch_grad(const float* x, const float* t, const float* wt, long long n, int F, const void* pb,
                        float scale, float* grad, float* loss, cudaStream_t s) {
  const size_t smem = grad_smem(F, H);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_grad<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long tiles = (n + kTile - 1) / kTile;
  k_mlp_grad<H><<<(unsigned)(tiles < 1184 ? (tiles > 0 ? tiles : 1) : 1184), kTile, smem, s>>>(
      x, t, wt, n, F, (const __nv_bfloat16*)pb, scale, grad, loss);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int64_t pf_mlp_param_count(int nin, int nh) { return param_count(nin, nh); }

int pf_mlp_error(char* buf, size_t len) {
  if (buf && len) snprintf(buf, len, "%s", g_learn_err);
  return PF_OK;
}

int pf_mlp_forward(const float* x, int64_t n, int nin, int nh, const void* params_bf16, float* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y)) || !params_bf16 || nin < 1 || nin > kMaxIn || !hidden_ok(nh))
    return learn_fail(PF_E_ARG, "pf_mlp_forward: bad arguments (nin 1..%d, nh 16, 32 or 64)", kMaxIn);
  if (n == 0) return PF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = nh == 16 ? launch_forward<16>(x, n, nin, params_bf16, y, s)
                : nh == 32 ? launch_forward<32>(x, n, nin, params_bf16, y, s)
                           : launch_forward<64>(x, n, nin, params_bf16, y, s);
  if (e != cudaSuccess) return learn_fail(PF_E_CUDA, "pf_mlp_forward: %s", cudaGetErrorString(e));
  return PF_OK;
}

int pf_mlp_grad(const float* x, const float* t, const float* w, int64_t n, int nin, int nh, const void* params_bf16,
                float scale, float* grad, float* loss, void* stream) {
  if (n < 0 || (n > 0 && (!x || !t)) || !params_bf16 || !grad || !loss || nin < 1 || nin > kMaxIn || !hidden_ok(nh))
    return learn_fail(PF_E_ARG, "pf_mlp_grad: bad arguments (nin 1..%d, nh 16, 32 or 64)", kMaxIn);
  if (grad_smem(nin, nh) > 227 * 1024) return learn_fail(PF_E_ARG, "pf_mlp_grad: nin %d with nh %d needs too much shared memory", nin, nh);
  if (n == 0) return PF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = nh == 16 ? launch_grad<16>(x, t, w, n, nin, params_bf16, scale, grad, loss, s)
                : nh == 32 ? launch_grad<32>(x, t, w, n, nin, params_bf16, scale, grad, loss, s)
                           : launch_grad<64>(x, t, w, n, nin, params_bf16, scale, grad, loss, s);
  if (e != cudaSuccess) return learn_fail(PF_E_CUDA, "pf_mlp_grad: %s", cudaGetErrorString(e));
  return PF_OK;
}

int pf_mlp_adam(float* params, void* params_bf16, const float* grad, float* m, float* v, int64_t count, float lr,
                float beta1, float beta2, float eps, int step, void* stream) {
  if (!params || !params_bf16 || !grad || !m || !v || count < 1 || step < 1)
    return learn_fail(PF_E_ARG, "pf_mlp_adam: bad arguments");
  double c1 = 1.0, c2 = 1.0;
  for (int i = 0; i < step && i < 100000; ++i) {
    c1 *= beta1;
    c2 *= beta2;
  }
  const long long blocks = (count + 255) / 256;
  k_adam<<<(unsigned)(blocks < 1024 ? blocks : 1024), 256, 0, (cudaStream_t)stream>>>(
      params, (__nv_bfloat16*)params_bf16, grad, m, v, count, lr, beta1, beta2, eps, (float)(1.0 - c1),
      (float)(1.0 - c2));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return learn_fail(PF_E_CUDA, "pf_mlp_adam: %s", cudaGetErrorString(e));
  return PF_OK;
}

}  // extern "C"
