// θ = W σ + b for every sample on the tensor cores (NQ_EVAL_TC_BF16X2 / X3).
// The reference computes θ with one gemm per batch (RBMBatched.jl:37-56,
// `mul!(θ, W, σ)`).  Here spins are exact in BF16 and W is split into BF16
// terms W_1 = bf16(W), W_2 = bf16(W - W_1), W_3 = bf16(W - W_1 - W_2); θ =
// Σ_t σ·W_tᵀ is accumulated in FP32 by tcgen05.mma kind::f16 (relative weight
// error about 2^-16 with two terms, about 2^-24, FP32-like, with three).
// One persistent CTA of 128 threads per SM:
//   * the W image (one block per term, rows 2h = Re W_h, 2h+1 = Im W_h, K =
//     sites padded to 64, 128-byte swizzled K-major) goes to shared memory once;
//   * per tile of 128 samples every thread writes its σ row (BF16, same
//     swizzle), thread 0 issues the MMAs (M = 128 samples, N <= 256 columns per
//     instruction, K = 16 per instruction) and commits to an mbarrier;
//   * every warp reads its 32 TMEM lanes (its 32 samples), adds b and writes
//     θ as complex FP32 [h][Ns], coalesced over samples.
// Waits are bounded (1 s) and report NQ_DEVERR_TIMEOUT.
#include <cuda_bf16.h>

#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int KPAD = 64;           // sites per row (128 bytes of BF16)
constexpr int ROWB = KPAD * 2;     // bytes per row

NQ_D uint32_t sw128(uint32_t r, uint32_t byte) {   // byte offset of (row, byte-in-row) in the swizzled image
  return r * ROWB + ((((byte >> 4) ^ (r & 7u)) & 7u) << 4) + (byte & 15u);
}

// image of W in the swizzled smem layout: term t at bytes [t*NPr*128, (t+1)*NPr*128)
__global__ void theta_pack_kernel(const cpx<float>* __restrict__ W, int M, int N, int NPr, int nterms,
                                  __nv_bfloat16* __restrict__ img) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;     // over NPr * KPAD
  if (idx >= NPr * KPAD) return;
  const int r = idx / KPAD, k = idx % KPAD;
  float w = 0.f;
  if (r < 2 * M && k < N) {
    const cpx<float> v = W[(r >> 1) + (size_t)M * k];
    w = (r & 1) ? v.y : v.x;
  }
  unsigned char* base = reinterpret_cast<unsigned char*>(img);
  const uint32_t off = sw128((uint32_t)r, (uint32_t)k * 2u);
  float rest = w;
  for (int t = 0; t < nterms; ++t) {
    const __nv_bfloat16 v = __float2bfloat16_rn(rest);
    rest -= __bfloat162float(v);
    *reinterpret_cast<__nv_bfloat16*>(base + (size_t)t * NPr * ROWB + off) = v;
  }
}

__global__ void __launch_bounds__(128, 1)
theta_bf16x2_kernel(const uint4* __restrict__ img, int NPr, int nterms, int tmem_cols, const cpx<float>* __restrict__ bias,
                    const uint64_t* __restrict__ samples, int Ns, int N, int M, int hilb,
                    cpx<float>* __restrict__ theta, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;                                 // 128 rows x 128 B
  unsigned char* sB = sA + 128 * ROWB;                      // nterms blocks of NPr rows
  uint64_t* bar = reinterpret_cast<uint64_t*>(sB + (size_t)nterms * NPr * ROWB);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // W image -> smem (16-byte vectors)
  const int nvec = nterms * NPr * ROWB / 16;
  for (int i = tid; i < nvec; i += blockDim.x) reinterpret_cast<uint4*>(sB)[i] = img[i];
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, (uint32_t)tmem_cols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int ksteps = (N + 15) / 16;
  const int ntiles = (Ns + 127) / 128;
  const __nv_bfloat16 one = __float2bfloat16_rn(1.f), mone = __float2bfloat16_rn(-1.f),
                      zero = __float2bfloat16_rn(0.f);
  uint32_t phase = 0;
  bool ok = true;
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    // σ row of this thread's sample (rows past Ns are zero)
    const int s = t * 128 + tid;
    const uint64_t bits = s < Ns ? samples[s] : 0ull;
#pragma unroll 1
    for (int c = 0; c < KPAD / 8; ++c) {
      __align__(16) __nv_bfloat16 v[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int k = c * 8 + e;
        const bool b = (bits >> k) & 1ull;
        v[e] = (s >= Ns || k >= N) ? zero : (hilb == HILB_SPIN ? (b ? one : mone) : (b ? one : zero));
      }
      *reinterpret_cast<uint4*>(sA + sw128((uint32_t)tid, (uint32_t)c * 16u)) = *reinterpret_cast<uint4*>(v);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint32_t a0 = smem_u32(sA);
      for (int c0 = 0; c0 < NPr; c0 += 256) {
        const int nc = min(256, NPr - c0);
        const uint32_t idesc = idesc_f32acc(1u, 128u, (uint32_t)nc);
        for (int h = 0; h < nterms; ++h) {
          const uint32_t b0 = smem_u32(sB) + (uint32_t)h * NPr * ROWB + (uint32_t)c0 * ROWB;
          for (int ks = 0; ks < ksteps; ++ks)
            mma_f16(tmem + (uint32_t)c0, sdesc_k_sw128(a0 + ks * 32u), sdesc_k_sw128(b0 + ks * 32u), idesc,
                    (h > 0 || ks > 0) ? 1u : 0u);
        }
      }
      mma_commit(bar);
    }
    bool landed = mbar_wait_bounded(bar, phase, err);
    if (!landed && tid == 0) landed = mbar_wait_bounded(bar, phase, err);   // issued MMAs before TMEM is freed
    if (!landed) ok = false;
    phase ^= 1u;
    ok = __syncthreads_and(ok ? 1 : 0) != 0;      // uniform: the TMEM loads below are warp-collective
    tc_fence_after();
    // epilogue: warp w owns TMEM lanes 32w..32w+31 = samples t*128 + 32w + lane
    const int sr = t * 128 + warp * 32 + lane;
    for (int c0 = 0; c0 < 2 * M && ok; c0 += 32) {
      uint32_t r[32];
      tmem_ld_32x32b_x32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
      tmem_ld_wait();
      if (sr < Ns) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int h = (c0 >> 1) + q;
          if (h < M) {
            const cpx<float> bb = bias[h];
            theta[(size_t)h * Ns + sr] = mk(__uint_as_float(r[2 * q]) + bb.x, __uint_as_float(r[2 * q + 1]) + bb.y);
          }
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, (uint32_t)tmem_cols);
  }
}

int pow2_cols(int n) {
  int c = 32;
  while (c < n) c <<= 1;
  return c;
}

}  // namespace

int theta_tc_rows(int M) { return (2 * M + 15) / 16 * 16; }
size_t theta_tc_image_elems(int M, int nterms) { return (size_t)nterms * theta_tc_rows(M) * KPAD; }
bool theta_tc_supported(int N, int M) { return N <= KPAD && theta_tc_rows(M) <= 512; }

cudaError_t launch_theta_pack(const cpx<float>* W, int M, int N, int nterms, __nv_bfloat16* img, cudaStream_t st) {
  const int NPr = theta_tc_rows(M);
  const int n = NPr * KPAD;
  theta_pack_kernel<<<(n + 255) / 256, 256, 0, st>>>(W, M, N, NPr, nterms, img);
  return cudaGetLastError();
}

cudaError_t launch_theta_bf16x2(const __nv_bfloat16* img, int nterms, int M, int N, const cpx<float>* b,
                                const uint64_t* samples, int Ns, int hilb, cpx<float>* theta, int* err,
                                cudaStream_t st) {
  if (!theta_tc_supported(N, M) || nterms < 1 || nterms > 3) return cudaErrorInvalidValue;
  const int NPr = theta_tc_rows(M);
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  const size_t smem = 1024 + 128 * (size_t)ROWB + (size_t)nterms * NPr * ROWB + 16;
  cudaError_t e = cudaFuncSetAttribute(theta_bf16x2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int ntiles = (Ns + 127) / 128;
  const int grid = ntiles < sms ? ntiles : sms;
  theta_bf16x2_kernel<<<grid, 128, smem, st>>>(reinterpret_cast<const uint4*>(img), NPr, nterms, pow2_cols(NPr), b,
                                               samples, Ns, N, M, hilb, theta, err);
  return cudaGetLastError();
}
