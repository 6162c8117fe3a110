// Warp-level MADE evaluation shared by the proposal kernels and the mixture
// sampler.  One warp walks the sites in autoregressive order; lane l owns the
// hidden units k = l + 32 j (j < UPL) of both layers and keeps their
// pre-activations in registers.  Because masked weights are stored as zeros,
// every contribution can be added as soon as its input is known:
//   * x_i enters layer 1 once it is drawn (or read);
//   * the layer-1 units of degree i+1 (k ≡ i mod N-1) are then final and are
//     folded into every layer-2 accumulator (one shuffle per unit);
//   * the logit of site i is Σ_k W3[i,k] relu(acc2_k) + b3[i]; masked W3
//     entries hide the layer-2 units that are not final yet.
// Each weight is touched once per walk: N·H + H·H + N·H multiply-adds per
// configuration, spread evenly over the lanes, with no shared memory.
#pragma once
#include <cuda_bf16.h>

#include "made_kernels.cuh"

namespace made {

NQ_D int degree(int k, int N) { return 1 + k % (N > 1 ? N - 1 : 1); }
NQ_D float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }
NQ_D float log_sigmoid(float z) { return z >= 0.f ? -log1pf(__expf(-z)) : z - log1pf(__expf(z)); }
NQ_D float warp_sum(float s) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}

// Returns log q(x) in every lane.  SAMPLE: x is drawn (bit i = [u_i < σ(l_i)],
// u_i = word slot*N + i of the chain's TAG_AR Philox stream); otherwise x is
// read.  Requires H == 32 * UPL, 2 <= N <= 64, all 32 lanes active.
template <int UPL, bool SAMPLE>
NQ_D float walk(const MadeDev& m, uint64_t& x, uint32_t slot, uint32_t chain, uint32_t call, uint32_t k0,
                uint32_t k1) {
  const int lane = threadIdx.x & 31, N = m.N, H = 32 * UPL;
  float acc1[UPL], acc2[UPL];
#pragma unroll
  for (int j = 0; j < UPL; ++j) {
    acc1[j] = m.b1[lane + 32 * j];
    acc2[j] = m.b2[lane + 32 * j];
  }
  u32x4 r = {0u, 0u, 0u, 0u};
  uint32_t b0 = 0;
  const uint32_t q0 = slot * (uint32_t)N;
  if (SAMPLE) {
    // lane l holds Philox block b0 + l; the walk needs at most 17 blocks (N <= 64)
    b0 = q0 >> 2;
    const uint32_t nblk = ((q0 + (uint32_t)N - 1u) >> 2) - b0 + 1u;
    if ((uint32_t)lane < nblk) r = philox4x32_10(b0 + (uint32_t)lane, call, chain, TAG_AR, k0, k1);
  } else {
    x = __shfl_sync(0xffffffffu, x, 0);
  }
  const int nm1 = N - 1;
  float lq = 0.f;
  for (int i = 0; i < N; ++i) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < UPL; ++j) s += bf(m.W3[i * H + lane + 32 * j]) * fmaxf(acc2[j], 0.f);
    const float l = warp_sum(s) + m.b3[i];
    bool bit;
    if (SAMPLE) {
      const uint32_t q = q0 + (uint32_t)i;
      const uint32_t wsel = q & 3u;
      uint32_t w = wsel == 0u ? r.x : wsel == 1u ? r.y : wsel == 2u ? r.z : r.w;
      w = __shfl_sync(0xffffffffu, w, (int)((q >> 2) - b0));
      const float p1 = 1.0f / (1.0f + __expf(-l));
      bit = uniform24(w) < p1;
      if (bit) x |= 1ull << i;
    } else {
      bit = (x >> i) & 1ull;
    }
    lq += log_sigmoid(bit ? l : -l);
    if (i == N - 1) break;
    if (bit) {
#pragma unroll
      for (int j = 0; j < UPL; ++j) acc1[j] += bf(m.W1T[i * H + lane + 32 * j]);
    }
    for (int kp = i; kp < H; kp += nm1) {          // layer-1 units of degree i+1
      const int jj = kp >> 5;
      float v = acc1[0];
#pragma unroll
      for (int j = 1; j < UPL; ++j)
        if (jj == j) v = acc1[j];
      v = __shfl_sync(0xffffffffu, fmaxf(v, 0.f), kp & 31);
#pragma unroll
      for (int j = 0; j < UPL; ++j) acc2[j] += bf(m.W2T[kp * H + lane + 32 * j]) * v;
    }
  }
  return lq;
}

}  // namespace made
