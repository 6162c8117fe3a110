// Mixture Metropolis sampler: at every step a chain makes either a local flip
// (the move of the local sampler) or an independent proposal x' drawn from
// the learned autoregressive model q.  The move type is drawn per step with a
// fixed probability p_ar (Philox stream TAG_MIX, word 0 below p_ar·2^32), so
// each move type is its own valid Metropolis–Hastings kernel:
//   local: accept iff u < |ψ(x')/ψ(x)|²               (symmetric proposal)
//   AR   : accept iff u < |ψ(x')|² q(x) / (|ψ(x)|² q(x'))
// u is the TAG_MH uniform of the step in both cases.  The chain's k-th AR step
// uses proposal slot k (uniforms TAG_AR word k*N + i); the first pre_slots
// slots of every chain are drawn ahead by the proposal kernel (they do not
// depend on the chain), later ones inline.  log q(x) of the current
// state is cached and recomputed only after a local move was accepted; θ(x')
// is rebuilt from scratch for an AR proposal and replaces the θ-cache when it
// is accepted.  One warp per chain (lane l owns hidden units l + 32 k).
#include "made_device.cuh"
#include "sampler_impl.cuh"

namespace {

template <typename R> NQ_D R warp_sum_r(R s) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}

template <typename R, int HPL, int ACT>
__global__ void __launch_bounds__(256, 1)
rbm_mix_sampler_kernel(RbmDev<R> net, SamplerRun run, MadeDev made, unsigned long long thr,
                       unsigned long long* __restrict__ ar_stats, const uint64_t* __restrict__ pre_x,
                       const float* __restrict__ pre_lq, int pre_slots) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = net.N, M = net.M;
  cpx<R>* s_t0 = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* s_t1 = s_t0 + N * M;
  cpx<R>* s_t2 = s_t1 + N * M;
  cpx<R>* s_w = s_t2 + N * M;                          // W[h, i] at i*M + h
  R* s_are = reinterpret_cast<R*>(s_w + N * M);        // 2 Re a_i log2(e)
  for (int k = threadIdx.x; k < N * M; k += blockDim.x) {
    s_t0[k] = net.t0[k];
    s_t1[k] = net.t1[k];
    if (ACT == ACT_LOGCOSH) s_t2[k] = net.t2[k];
    const int i = k / M, h = k % M;
    s_w[k] = net.W[h + M * i];
  }
  for (int k = threadIdx.x; k < N; k += blockDim.x) s_are[k] = R(2.8853900817779268) * net.a[k].x;
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int chain_raw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const bool active = chain_raw < run.B;
  const int chain = active ? chain_raw : run.B - 1;
  const int hilb = net.hilb;
  if (run.call_ptr) run.call = *run.call_ptr;

  uint64_t bits = 0;
  for (int q = 0; q < N; q += 4) {
    const u32x4 w = philox4x32_10((uint32_t)(q >> 2), run.call, (uint32_t)chain, TAG_INIT, run.k0, run.k1);
    const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (q + k < N && (ws[k] >> 31)) bits |= 1ull << (q + k);
  }

  cpx<R> th[HPL], g[HPL];
#pragma unroll
  for (int k = 0; k < HPL; ++k) {
    const int h = lane + 32 * k;
    th[k] = mk(R(0), R(0));
    g[k] = mk(R(0), R(0));
    if (h < M) {
      cpx<R> t = net.b[h];
      for (int j = 0; j < N; ++j) {
        const R v = site_value<R>(bits, j, hilb);
        const cpx<R> w = s_w[j * M + h];
        t.x += w.x * v;
        t.y += w.y * v;
      }
      th[k] = t;
      g[k] = act_df<ACT>(t);
    }
  }

  unsigned long long naccept = 0, n_ar = 0, n_ar_acc = 0;
  const int nsweeps = run.burn + run.n_record;
  uint32_t t = 0, ar_slot = 0;
  int my_site = 0;
  R my_lu = 0;
  bool my_ar = false;
  float lq_x = 0.f;
  bool lq_ok = false;
  for (int sweep = 0; sweep < nsweeps; ++sweep) {
    for (int pass = 0; pass < run.passes; ++pass, ++t) {
      const int slot = (int)(t & 31u);
      if (slot == 0) {
        const u32x4 r = philox4x32_10(t + (uint32_t)lane, run.call, (uint32_t)chain, TAG_MH, run.k0, run.k1);
        my_site = (int)uniform_site(r.x, (uint32_t)N);
        my_lu = fast_log2((R)uniform24(r.y));
        const u32x4 rm = philox4x32_10(t + (uint32_t)lane, run.call, (uint32_t)chain, TAG_MIX, run.k0, run.k1);
        my_ar = (unsigned long long)rm.x < thr;
      }
      const int i = __shfl_sync(0xffffffffu, my_site, slot);
      const R lu = __shfl_sync(0xffffffffu, my_lu, slot);
      const bool is_ar = __shfl_sync(0xffffffffu, (int)my_ar, slot) != 0;
      bool acc;
      if (!is_ar) {
        const int bit = (int)((bits >> i) & 1ull);
        const R dv = hilb == HILB_SPIN ? (bit ? R(-2) : R(2)) : (bit ? R(-1) : R(1));
        const bool pos = dv > 0;
        R prod = R(1);
#pragma unroll
        for (int k = 0; k < HPL; ++k) {
          const int h = lane + 32 * k;
          if (h < M) {
            cpx<R> rr;
            if (ACT == ACT_LOGCOSH) {
              cpx<R> c1 = s_t1[i * M + h];
              if (!pos) c1 = mk(-c1.x, -c1.y);
              rr = cfma(g[k], c1, s_t0[i * M + h]);
            } else {
              const cpx<R> bb = pos ? s_t0[i * M + h] : s_t1[i * M + h];
              rr = cfma(g[k], bb, mk(R(1), R(0)));
            }
            prod *= abs2c(rr);
          }
        }
        const R logA = s_are[i] * dv + warp_sum_r(fast_log2(prod));
        acc = lu < logA;
        if (acc) {
#pragma unroll
          for (int k = 0; k < HPL; ++k) {
            const int h = lane + 32 * k;
            if (h < M) {
              const cpx<R> w = s_w[i * M + h];
              th[k].x += w.x * dv;
              th[k].y += w.y * dv;
              cpx<R> num, den;
              if (ACT == ACT_LOGCOSH) {
                cpx<R> tau = s_t2[i * M + h];
                if (!pos) tau = mk(-tau.x, -tau.y);
                num = g[k] + tau;
                den = cfma(g[k], tau, mk(R(1), R(0)));
              } else {
                const cpx<R> bb = pos ? s_t0[i * M + h] : s_t1[i * M + h];
                num = g[k] * mk(R(1) + bb.x, bb.y);
                den = cfma(g[k], bb, mk(R(1), R(0)));
              }
              const R inv = fast_rcp(abs2c(den));
              g[k] = inv * (num * conjc(den));
            }
          }
          bits ^= 1ull << i;
          lq_ok = false;
        }
      } else {
        uint64_t xp = 0;
        float lqp;
        if ((int)ar_slot < pre_slots) {          // drawn ahead by the proposal kernel
          const size_t q = (size_t)chain * pre_slots + ar_slot;
          xp = pre_x[q];
          lqp = pre_lq[q];
        } else {
          lqp = made::walk<4, true>(made, xp, ar_slot, (uint32_t)chain, run.call, run.k0, run.k1);
        }
        ++ar_slot;
        if (!lq_ok) {
          uint64_t xc = bits;
          lq_x = made::walk<4, false>(made, xc, 0, 0, 0, 0, 0);
          lq_ok = true;
        }
        cpx<R> thp[HPL];
        R dre = R(0);
#pragma unroll
        for (int k = 0; k < HPL; ++k) {
          const int h = lane + 32 * k;
          thp[k] = mk(R(0), R(0));
          if (h < M) {
            cpx<R> tt = net.b[h];
            for (int j = 0; j < N; ++j) {
              const R v = site_value<R>(xp, j, hilb);
              const cpx<R> w = s_w[j * M + h];
              tt.x += w.x * v;
              tt.y += w.y * v;
            }
            thp[k] = tt;
            dre += act_f<ACT>(tt).x - act_f<ACT>(th[k]).x;
          }
        }
        R dvis = R(0);
        for (int j = lane; j < N; j += 32)
          dvis += s_are[j] * (site_value<R>(xp, j, hilb) - site_value<R>(bits, j, hilb));
        const R logA = warp_sum_r(dvis) + R(2.8853900817779268) * warp_sum_r(dre) +
                       R(1.4426950408889634) * (R)(lq_x - lqp);
        acc = lu < logA;
        ++n_ar;
        if (acc) {
#pragma unroll
          for (int k = 0; k < HPL; ++k) {
            th[k] = thp[k];
            if (lane + 32 * k < M) g[k] = act_df<ACT>(thp[k]);
          }
          bits = xp;
          lq_x = lqp;
          ++n_ar_acc;
        }
      }
      naccept += acc ? 1 : 0;
      if (run.accept_bits && active && lane == 0) run.accept_bits[(size_t)t * run.B + chain] = acc ? 1 : 0;
    }
    const int rec = sweep - run.burn;
    if (rec >= 0 && active && lane == 0) run.samples[(size_t)rec * run.B + chain] = bits;
#pragma unroll
    for (int k = 0; k < HPL; ++k)
      if (lane + 32 * k < M) g[k] = act_df<ACT>(th[k]);
  }
  if (run.write_last_at_end && active && lane == 0) run.samples[chain] = bits;
  if (active && lane == 0) {
    atomicAdd(run.accepted, naccept);
    if (ar_stats) {
      atomicAdd(ar_stats, n_ar);
      atomicAdd(ar_stats + 1, n_ar_acc);
    }
  }
}

template <int HPL, int ACT>
cudaError_t mix_inst(const RbmDev<float>& net, const SamplerRun& run, const MixParams& mix, cudaStream_t st) {
  const int threads = 256;
  const int blocks = (run.B + 7) / 8;
  const size_t smem = (size_t)4 * net.N * net.M * sizeof(cpx<float>) + net.N * sizeof(float);
  auto kern = rbm_mix_sampler_kernel<float, HPL, ACT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<blocks, threads, smem, st>>>(net, run, mix.made, mix.thr, mix.ar_stats, mix.pre_x, mix.pre_lq,
                                      mix.pre_x ? mix.pre_slots : 0);
  return cudaGetLastError();
}

template <int ACT>
cudaError_t mix_hpl(const RbmDev<float>& net, const SamplerRun& run, const MixParams& mix, cudaStream_t st) {
  switch ((net.M + 31) / 32) {
    case 1: return mix_inst<1, ACT>(net, run, mix, st);
    case 2: return mix_inst<2, ACT>(net, run, mix, st);
    case 3: return mix_inst<3, ACT>(net, run, mix, st);
    case 4: return mix_inst<4, ACT>(net, run, mix, st);
    case 5: return mix_inst<5, ACT>(net, run, mix, st);
    case 6: return mix_inst<6, ACT>(net, run, mix, st);
    case 8: return mix_inst<8, ACT>(net, run, mix, st);
    case 10: return mix_inst<10, ACT>(net, run, mix, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

bool mix_sampler_supported(int N, int M, int n_half, int H) {
  const int hpl = (M + 31) / 32;
  const size_t smem = (size_t)4 * N * M * sizeof(cpx<float>) + N * sizeof(float);
  return N >= 2 && N <= 64 && H == 128 && n_half == 0 && (hpl <= 6 || hpl == 8 || hpl == 10) &&
         smem <= 227 * 1024;
}

cudaError_t launch_rbm_mix_sampler(const RbmDev<float>& net, const SamplerRun& run, const MixParams& mix,
                                   cudaStream_t st) {
  if (!mix_sampler_supported(net.N, net.M, net.n_half, mix.made.H) || mix.made.N != net.N)
    return cudaErrorInvalidValue;
  if (net.act == ACT_LOGCOSH) return mix_hpl<ACT_LOGCOSH>(net, run, mix, st);
  return mix_hpl<ACT_SOFTPLUS>(net, run, mix, st);
}
