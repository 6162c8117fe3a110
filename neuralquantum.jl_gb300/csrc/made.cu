// Learned autoregressive proposal: a MADE masked MLP (N -> H -> H -> N, ReLU,
// Bernoulli outputs) with its own sampling, log-probability and training
// kernels.  The reference has no learned proposal; the tests check these
// kernels against an FP64 restatement of the same network.
//
// Parameters (FP32 master, flat): W1 [H][N], b1 [H], W2 [H][H], b2 [H],
// W3 [N][H], b3 [N]; masked entries are zero and stay zero (their gradient is
// masked).  Inference reads a BF16 copy laid out for coalesced warp access:
// W1T [N][H], W2T [H][H] (W2T[k'][k] = W2[k][k']), W3 [N][H].
#include <cuda_bf16.h>

#include "made_device.cuh"

namespace {

using made::bf;
using made::degree;

// master (flat, masked on the fly) -> BF16 inference copy
__global__ void made_pack_kernel(MadeDevW m, int N, int H, const float* __restrict__ master) {
  const float* W1 = master;
  const float* b1 = W1 + H * N;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  const float* b3 = W3 + N * H;
  const int tot = H * N + H * H + N * H + 2 * H + N;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < tot; idx += gridDim.x * blockDim.x) {
    int r = idx;
    if (r < H * N) {
      const int i = r / H, k = r % H;
      m.W1T[i * H + k] = __float2bfloat16(degree(k, N) >= i + 1 ? W1[k * N + i] : 0.f);
      continue;
    }
    r -= H * N;
    if (r < H * H) {
      const int kp = r / H, k = r % H;
      m.W2T[kp * H + k] = __float2bfloat16(degree(k, N) >= degree(kp, N) ? W2[k * H + kp] : 0.f);
      continue;
    }
    r -= H * H;
    if (r < N * H) {
      const int i = r / H, k = r % H;
      m.W3[r] = __float2bfloat16(i + 1 > degree(k, N) ? W3[r] : 0.f);
      continue;
    }
    r -= N * H;
    if (r < H) { m.b1[r] = b1[r]; continue; }
    r -= H;
    if (r < H) { m.b2[r] = b2[r]; continue; }
    r -= H;
    m.b3[r] = b3[r];
  }
}

// one warp per configuration: log q(x)
template <int UPL>
__global__ void __launch_bounds__(256) made_logq_kernel(MadeDev m, const uint64_t* __restrict__ x, int n,
                                                        float* __restrict__ out) {
  const int s = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (s >= n) return;                      // whole warps exit together
  uint64_t xs = x[s];
  const float lq = made::walk<UPL, false>(m, xs, 0, 0, 0, 0, 0);
  if ((threadIdx.x & 31) == 0) out[s] = lq;
}

// one warp per proposal (chain, slot), chain-major: index chain*slots + slot
template <int UPL>
__global__ void __launch_bounds__(256)
made_sample_kernel(MadeDev m, int n_chains, int slots, uint32_t call, const uint32_t* call_ptr, uint32_t k0,
                   uint32_t k1, uint64_t* __restrict__ xout, float* __restrict__ lqout) {
  const long gid = (long)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (gid >= (long)n_chains * slots) return;
  if (call_ptr) call = *call_ptr;
  const uint32_t chain = (uint32_t)(gid / slots), slot = (uint32_t)(gid % slots);
  uint64_t x = 0;
  const float lq = made::walk<UPL, true>(m, x, slot, chain, call, k0, k1);
  if ((threadIdx.x & 31) == 0) {
    xout[gid] = x;
    lqout[gid] = lq;
  }
}

// Per-block gradient of the mean NLL over a chunk of CH samples (block of 256
// threads): forward for all samples of the chunk into shared memory, then
// backward and the weight-gradient contractions over the chunk.
template <int CH>
__global__ void __launch_bounds__(256)
made_grad_kernel(MadeTrain t, const uint64_t* __restrict__ x, int n, float inv_n, float* __restrict__ partial) {
  extern __shared__ __align__(16) float sm[];
  const int N = t.N, H = t.H;
  float* A1 = sm;                   // [CH][H]  (relu'(h1) folded in via sign)
  float* A2 = A1 + CH * H;          // [CH][H]
  float* D3 = A2 + CH * H;          // [CH][N]
  float* D2 = D3 + CH * N;          // [CH][H]
  float* D1 = D2 + CH * H;          // [CH][H]
  __shared__ uint64_t X[CH];
  const float* W1 = t.master;
  const float* b1 = W1 + H * N;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  const float* b3 = W3 + N * H;
  const int s0 = blockIdx.x * CH;
  for (int q = threadIdx.x; q < CH; q += blockDim.x) X[q] = (s0 + q < n) ? x[s0 + q] : 0ull;
  __syncthreads();
  // layer 1
  for (int e = threadIdx.x; e < CH * H; e += blockDim.x) {
    const int q = e / H, k = e % H;
    float h = b1[k];
    for (int i = 0; i < N; ++i)
      if ((X[q] >> i) & 1ull) h += W1[k * N + i];
    A1[e] = h;              // pre-activation kept; relu applied on use
  }
  __syncthreads();
  // layer 2
  for (int e = threadIdx.x; e < CH * H; e += blockDim.x) {
    const int q = e / H, k = e % H;
    float h = b2[k];
    const float* w = W2 + (size_t)k * H;
    const float* a = A1 + q * H;
    for (int kp = 0; kp < H; ++kp) h += w[kp] * fmaxf(a[kp], 0.f);
    A2[e] = h;
  }
  __syncthreads();
  // output layer and d nll / d logit = (σ(l) - x) / n   (padding samples: 0)
  for (int e = threadIdx.x; e < CH * N; e += blockDim.x) {
    const int q = e / N, i = e % N;
    float l = b3[i];
    const float* w = W3 + (size_t)i * H;
    const float* a = A2 + q * H;
    for (int k = 0; k < H; ++k) l += w[k] * fmaxf(a[k], 0.f);
    const float xi = (float)((X[q] >> i) & 1ull);
    D3[e] = (s0 + q < n) ? (1.0f / (1.0f + __expf(-l)) - xi) * inv_n : 0.f;
  }
  __syncthreads();
  // δ2 = (W3ᵀ δ3) ⊙ relu'(h2)
  for (int e = threadIdx.x; e < CH * H; e += blockDim.x) {
    const int q = e / H, k = e % H;
    float d = 0.f;
    for (int i = 0; i < N; ++i) d += W3[(size_t)i * H + k] * D3[q * N + i];
    D2[e] = A2[e] > 0.f ? d : 0.f;
  }
  __syncthreads();
  // δ1 = (W2ᵀ δ2) ⊙ relu'(h1)
  for (int e = threadIdx.x; e < CH * H; e += blockDim.x) {
    const int q = e / H, kp = e % H;
    float d = 0.f;
    for (int k = 0; k < H; ++k) d += W2[(size_t)k * H + kp] * D2[q * H + k];
    D1[e] = A1[e] > 0.f ? d : 0.f;
  }
  __syncthreads();
  // weight gradients over the chunk (masked entries: mask applied by the caller's mask multiply)
  float* out = partial + (size_t)blockIdx.x * t.n_params;
  const int nW1 = H * N, nW2 = H * H, nW3 = N * H;
  for (int e = threadIdx.x; e < t.n_params; e += blockDim.x) {
    float g = 0.f;
    int r = e;
    if (r < nW1) {
      const int k = r / N, i = r % N;
      for (int q = 0; q < CH; ++q) if ((X[q] >> i) & 1ull) g += D1[q * H + k];
    } else if ((r -= nW1) < H) {
      for (int q = 0; q < CH; ++q) g += D1[q * H + r];
    } else if ((r -= H) < nW2) {
      const int k = r / H, kp = r % H;
      for (int q = 0; q < CH; ++q) g += D2[q * H + k] * fmaxf(A1[q * H + kp], 0.f);
    } else if ((r -= nW2) < H) {
      for (int q = 0; q < CH; ++q) g += D2[q * H + r];
    } else if ((r -= H) < nW3) {
      const int i = r / H, k = r % H;
      for (int q = 0; q < CH; ++q) g += D3[q * N + i] * fmaxf(A2[q * H + k], 0.f);
    } else {
      r -= nW3;
      for (int q = 0; q < CH; ++q) g += D3[q * N + r];
    }
    out[e] = g;
  }
}

// sum of the block partials in a fixed order, masked
__global__ void made_reduce_kernel(int n_params, const float* __restrict__ mask, const float* __restrict__ partial,
                                   int nblk, float* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_params) return;
  float g = 0.f;
  for (int b = 0; b < nblk; ++b) g += partial[(size_t)b * n_params + e];
  grad[e] = g * mask[e];
}

// Adam (Kingma & Ba 2015; beta1 0.9, beta2 0.999, eps 1e-8) on the master
__global__ void made_adam_kernel(MadeTrain t, const float* __restrict__ grad, float lr, float b1c, float b2c) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.n_params) return;
  const float g = grad[e];
  const float mm = 0.9f * t.m[e] + 0.1f * g;
  const float vv = 0.999f * t.v[e] + 0.001f * g * g;
  t.m[e] = mm;
  t.v[e] = vv;
  t.master[e] -= t.mask[e] * (lr * (mm / b1c) / (sqrtf(vv / b2c) + 1e-8f));
}

__global__ void made_mask_kernel(int N, int H, float* __restrict__ mask) {
  const int n_params = 2 * H * N + H * H + 2 * H + N;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_params) return;
  int r = e;
  float v = 1.f;
  if (r < H * N) { const int k = r / N, i = r % N; v = degree(k, N) >= i + 1 ? 1.f : 0.f; }
  else if ((r -= H * N) < H) v = 1.f;
  else if ((r -= H) < H * H) { const int k = r / H, kp = r % H; v = degree(k, N) >= degree(kp, N) ? 1.f : 0.f; }
  else if ((r -= H * H) < H) v = 1.f;
  else if ((r -= H) < N * H) { const int i = r / H, k = r % H; v = (i + 1) > degree(k, N) ? 1.f : 0.f; }
  mask[e] = v;
}

__global__ void made_apply_mask_kernel(int n, const float* __restrict__ mask, float* __restrict__ master) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) master[e] *= mask[e];
}

}  // namespace

// ------------------------------- launchers ---------------------------------
int made_n_params(int N, int H) { return 2 * H * N + H * H + 2 * H + N; }

cudaError_t launch_made_mask(int N, int H, float* mask, cudaStream_t st) {
  const int n = made_n_params(N, H);
  made_mask_kernel<<<(n + 255) / 256, 256, 0, st>>>(N, H, mask);
  return cudaGetLastError();
}

cudaError_t launch_made_apply_mask(int n_params, const float* mask, float* master, cudaStream_t st) {
  made_apply_mask_kernel<<<(n_params + 255) / 256, 256, 0, st>>>(n_params, mask, master);
  return cudaGetLastError();
}

cudaError_t launch_made_pack(const MadeDev& m, const float* master, cudaStream_t st) {
  const MadeDevW w{const_cast<__nv_bfloat16*>(m.W1T), const_cast<__nv_bfloat16*>(m.W2T),
                   const_cast<__nv_bfloat16*>(m.W3), const_cast<float*>(m.b1), const_cast<float*>(m.b2),
                   const_cast<float*>(m.b3)};
  made_pack_kernel<<<64, 256, 0, st>>>(w, m.N, m.H, master);
  return cudaGetLastError();
}

cudaError_t launch_made_logq(const MadeDev& m, const uint64_t* x, int n, float* out, cudaStream_t st) {
  if (m.H != 128 || m.N < 2 || m.N > 64) return cudaErrorInvalidValue;
  if (n <= 0) return cudaSuccess;
  made_logq_kernel<4><<<(n + 7) / 8, 256, 0, st>>>(m, x, n, out);
  return cudaGetLastError();
}

cudaError_t launch_made_sample(const MadeDev& m, int n_chains, int slots, uint32_t call, uint32_t k0, uint32_t k1,
                               uint64_t* xout, float* lqout, cudaStream_t st, const uint32_t* call_ptr) {
  if (m.H != 128 || m.N < 2 || m.N > 64) return cudaErrorInvalidValue;
  const long n = (long)n_chains * slots;
  if (n <= 0) return cudaSuccess;
  made_sample_kernel<4><<<(unsigned)((n + 7) / 8), 256, 0, st>>>(m, n_chains, slots, call, call_ptr, k0, k1, xout,
                                                                  lqout);
  return cudaGetLastError();
}

int made_grad_chunk() { return 16; }

cudaError_t launch_made_grad(const MadeTrain& t, const uint64_t* x, int n, float* partial, float* grad,
                             cudaStream_t st) {
  constexpr int CH = 16;
  if (n <= 0) return cudaErrorInvalidValue;
  const int nblk = (n + CH - 1) / CH;
  const size_t smem = ((size_t)CH * (4 * t.H + t.N)) * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(made_grad_kernel<CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  made_grad_kernel<CH><<<nblk, 256, smem, st>>>(t, x, n, 1.0f / n, partial);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  made_reduce_kernel<<<(t.n_params + 255) / 256, 256, 0, st>>>(t.n_params, t.mask, partial, nblk, grad);
  return cudaGetLastError();
}

cudaError_t launch_made_adam(const MadeTrain& t, const float* grad, float lr, int step, cudaStream_t st) {
  const float b1c = 1.f - powf(0.9f, (float)step), b2c = 1.f - powf(0.999f, (float)step);
  made_adam_kernel<<<(t.n_params + 255) / 256, 256, 0, st>>>(t, grad, lr, b1c, b2c);
  return cudaGetLastError();
}
