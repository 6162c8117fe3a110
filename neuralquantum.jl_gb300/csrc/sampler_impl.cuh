// Persistent Metropolis sampler for the RBM (local-flip rule) with an
// incremental θ-cache.  Reference: src/Samplers/Metropolis.jl:101-167,
// src/Samplers/MCMCRules/LocalRule.jl:19-28, flipat! of
// src/Hilbert/HomogeneousSpin.jl:95-104 and HomogeneousFock.jl:72-81.
#pragma once
#include <type_traits>

#include "nq_kernels.cuh"

namespace {

// ---------------------------------------------------------------------------
// Persistent Metropolis sampler.  G lanes advance one chain; lane l owns the
// hidden units h = l + G*k (k < HPL) and keeps θ_h and g_h = f'(θ_h) in
// registers.  A proposal flipping site i costs HPL complex FMAs per lane
// (ratio t0 + g*t1 per unit, tables in shared memory) plus a log2(G)-step
// shuffle reduction of log2|ratio|^2; an accepted flip updates θ additively
// and g by the Möbius map of the single-flip tables.  g is recomputed from θ
// at the end of every sweep, so rounding drift is bounded by one sweep.
// Random draws are software-pipelined: every G steps each lane evaluates the
// Philox block of one upcoming step and the chain's lanes broadcast (site, u)
// by shuffle one step ahead, together with the table rows of that site, so
// the loads of step t+1 overlap the decision of step t.
// ---------------------------------------------------------------------------
template <typename R> NQ_D R fast_log2(R x) { return log2(x); }
template <> NQ_D float fast_log2<float>(float x) { return __log2f(x); }
template <typename R> NQ_D R fast_rcp(R x) { return R(1) / x; }
template <> NQ_D float fast_rcp<float>(float x) { return __fdividef(1.0f, x); }

// two complex table entries of one (site, hidden unit) loaded together:
// {t0, t1} for the ratio, {t2, W} for an accepted flip
template <typename R> struct alignas(4 * sizeof(R)) cpx_pair {
  cpx<R> a, b;
};

// One block of the sampler: chains (blk * blockDim + tid) / G of the problem
// described by (net, run).  Shared by the single-problem kernel and the
// many-problem kernel below.
// Hidden units are padded to MP = G*HPL with neutral table entries (ratio
// factor 1, no θ change), so the proposal and accept loops have no unit-range
// branches.
// HALF: the first net.n_half units enter log|ψ|^2 with weight 1/2 (the λ
// units of a density matrix); without it no unit does, and the proposal loop
// keeps a single product.
// EXCH: the exchange rule (ExchangeRule.jl:38-68): a move draws a coupling
// (i, j) and swaps the two values; equal values leave the state unchanged
// (ratio 1, accepted).  The move tables are then per coupling.
// PRE: read the table rows one step ahead (below); the many-problem kernel
// runs without it, since there the extra registers cost more resident warps
// than the hidden latency gains.
template <typename R, int G, int HPL, int ACT, bool EXCH = false, bool HALF = false, bool PRE = true>
NQ_D void sampler_block(const RbmDev<R>& net, SamplerRun run, int blk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int MP = G * HPL;
  const int N = net.N, M = net.M, n_half = net.n_half;
  const int NR = EXCH ? net.n_rows : N;                          // rows of the move tables
  cpx_pair<R>* s_t01 = reinterpret_cast<cpx_pair<R>*>(smem_raw);   // {t0, t1} at r*MP + h
  cpx_pair<R>* s_t2w = s_t01 + NR * MP;                           // {t2, W[h, i] or W_hi - W_hj} at r*MP + h
  int2* s_pairs = reinterpret_cast<int2*>(s_t2w + NR * MP);       // EXCH: sites of coupling r
  R* s_are = reinterpret_cast<R*>(s_pairs + (EXCH ? NR : 0));     // 2 Re a_i log2(e) (EXCH: of a_i - a_j)
  for (int k = threadIdx.x; k < NR * MP; k += blockDim.x) {
    const int i = k / MP, h = k % MP;
    cpx_pair<R> p01, p2w;
    if (h < M) {
      p01.a = net.t0[i * M + h];
      p01.b = net.t1[i * M + h];
      p2w.a = ACT == ACT_LOGCOSH ? net.t2[i * M + h] : mk(R(0), R(0));
      p2w.b = EXCH ? net.rW[h + M * i] : net.W[h + M * i];
    } else {
      // logcosh: t0 + g t1 = 1; softplus: 1 + g t0 = 1; accepted flip: θ, g unchanged
      p01.a = ACT == ACT_LOGCOSH ? mk(R(1), R(0)) : mk(R(0), R(0));
      p01.b = mk(R(0), R(0));
      p2w.a = mk(R(0), R(0));
      p2w.b = mk(R(0), R(0));
    }
    s_t01[k] = p01;
    s_t2w[k] = p2w;
  }
  for (int k = threadIdx.x; k < NR; k += blockDim.x) {
    if (EXCH) {
      s_pairs[k] = net.pairs[k];
      s_are[k] = net.rare[k];
    } else {
      s_are[k] = R(2.8853900817779268) * net.a[k].x;
    }
  }
  __syncthreads();

  const int lane = threadIdx.x % G;
  const int chain_raw = (blk * blockDim.x + threadIdx.x) / G;
  const bool active = chain_raw < run.B;
  const int chain = active ? chain_raw : run.B - 1;
  const int hilb = net.hilb;
  if (run.call_ptr) run.call = *run.call_ptr;

  // random initial configuration (rand!, HomogeneousSpin.jl:130-135)
  uint64_t bits = 0;
  for (int q = 0; q < N; q += 4) {
    u32x4 w = philox4x32_10((uint32_t)(q >> 2), run.call, (uint32_t)chain, TAG_INIT, run.k0, run.k1);
    uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (q + k < N && (ws[k] >> 31)) bits |= 1ull << (q + k);
  }

  cpx<R> th[HPL], g[HPL];
  bool half[HPL];
#pragma unroll
  for (int k = 0; k < HPL; ++k) {
    const int h = lane + G * k;
    half[k] = HALF && h < n_half;
    cpx<R> t = h < M ? net.b[h] : mk(R(0), R(0));
    if (h < M)
      for (int j = 0; j < N; ++j) {
        const R v = site_value<R>(bits, j, hilb);
        const cpx<R> w = EXCH ? net.W[h + M * j] : s_t2w[j * MP + h].b;
        t.x += w.x * v;
        t.y += w.y * v;
      }
    th[k] = t;
    g[k] = act_df<ACT>(t);
  }
  const R dmag = hilb == HILB_SPIN ? R(2) : R(1);

  uint32_t naccept = 0;
  const bool rec_bits = run.accept_bits && active && lane == 0;
  const uint32_t nsteps = (uint32_t)(run.burn + run.n_record) * (uint32_t)run.passes;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
  int my_site = 0;
  R my_lu = 0;
  int pass = 0, sweep = 0;

  // Operands of one step, read one step ahead: the site and the uniform of
  // step t depend only on the Philox counter, never on the chain's state, so
  // the table rows of step t+1 are loaded while step t decides.  Two buffers
  // alternate (the loop below is unrolled by two), so nothing is copied.
  // The rows stay in shared memory where the buffers would not fit the
  // register file.
  constexpr bool PRE_T = PRE && HPL * sizeof(R) <= 40;       // {t0, t1} rows
  constexpr bool PRE_W = PRE && HPL * sizeof(R) <= 20;       // {t2, W} rows (accepted flips)
  struct Pre {
    cpx_pair<R> t01[PRE_T ? HPL : 1];
    cpx_pair<R> t2w[PRE_W ? HPL : 1];
    R are, lu;
    int i;
    int2 pr;
  };
  auto fetch = [&](uint32_t tn, Pre& p) {
    const int slot = (int)(tn & (G - 1));
    if (slot == 0) {
      // lane l draws the (site, u) of step tn + l
      const u32x4 r = philox4x32_10(tn + (uint32_t)lane, run.call, (uint32_t)chain, TAG_MH, run.k0, run.k1);
      my_site = (int)uniform_site(r.x, (uint32_t)NR);
      my_lu = fast_log2((R)uniform24(r.y));       // log2 u; u = 0 -> -inf (always accept)
    }
    p.i = __shfl_sync(gmask, my_site, slot, G);
    p.lu = __shfl_sync(gmask, my_lu, slot, G);
    if constexpr (EXCH) p.pr = s_pairs[p.i];
    if constexpr (PRE_T) {
#pragma unroll
      for (int k = 0; k < HPL; ++k) p.t01[k] = s_t01[p.i * MP + lane + G * k];
    }
    if constexpr (PRE_W) {
#pragma unroll
      for (int k = 0; k < HPL; ++k) p.t2w[k] = s_t2w[p.i * MP + lane + G * k];
    }
    p.are = s_are[p.i];
  };

  auto step = [&](uint32_t t, const Pre& p, Pre& nxt) {
    fetch(t + 1, nxt);
    const int i = p.i;
    uint64_t fmask = 1ull << i;
    int site_i = i;
    bool flip = true;
    if constexpr (EXCH) {
      site_i = p.pr.x;
      fmask = (1ull << p.pr.x) | (1ull << p.pr.y);
      // a swap of equal values is the same state: ratio 1, accepted (u < 1)
      flip = ((bits >> p.pr.x) & 1ull) != ((bits >> p.pr.y) & 1ull);
    }
    bool acc = true;
    if (flip) {
      const bool pos = !((bits >> site_i) & 1ull);
      const R dv = pos ? dmag : -dmag;
      R prod = R(1), prod_half = R(1);
#pragma unroll
      for (int k = 0; k < HPL; ++k) {
        const cpx_pair<R> tt = PRE_T ? p.t01[k] : s_t01[i * MP + lane + G * k];
        cpx<R> rr;
        if (ACT == ACT_LOGCOSH) {
          cpx<R> c1 = tt.b;
          if (!pos) c1 = mk(-c1.x, -c1.y);
          rr = cfma(g[k], c1, tt.a);
        } else {
          const cpx<R> bb = pos ? tt.a : tt.b;
          rr = cfma(g[k], bb, mk(R(1), R(0)));
        }
        if (HALF && half[k]) prod_half *= abs2c(rr);
        else prod *= abs2c(rr);
      }
      R lsum = fast_log2(prod);
      if (HALF) lsum += R(0.5) * fast_log2(prod_half);
#pragma unroll
      for (int off = G / 2; off > 0; off >>= 1) lsum += __shfl_xor_sync(gmask, lsum, off, G);
      const R logA = p.are * dv + lsum;                    // log2 of the acceptance ratio
      acc = p.lu < logA;
      if (acc) {
#pragma unroll
        for (int k = 0; k < HPL; ++k) {
          const cpx_pair<R> tw = PRE_W ? p.t2w[k] : s_t2w[i * MP + lane + G * k];
          const cpx<R> w = tw.b;
          th[k].x += w.x * dv;
          th[k].y += w.y * dv;
          cpx<R> num, den;
          if (ACT == ACT_LOGCOSH) {
            cpx<R> tau = tw.a;
            if (!pos) tau = mk(-tau.x, -tau.y);
            num = g[k] + tau;
            den = cfma(g[k], tau, mk(R(1), R(0)));
          } else {
            const cpx_pair<R> tt = PRE_T ? p.t01[k] : s_t01[i * MP + lane + G * k];
            const cpx<R> bb = pos ? tt.a : tt.b;
            num = g[k] * mk(R(1) + bb.x, bb.y);
            den = cfma(g[k], bb, mk(R(1), R(0)));
          }
          const R inv = fast_rcp(abs2c(den));
          g[k] = inv * (num * conjc(den));
        }
        bits ^= fmask;
      }
    }
    naccept += acc ? 1u : 0u;
    if (rec_bits) run.accept_bits[(size_t)t * run.B + chain] = acc ? 1 : 0;
    if (++pass == run.passes) {
      // end of sweep: record and resynchronise g with θ
      pass = 0;
      const int slot = sweep - run.burn;
      if (slot >= 0 && active && lane == 0) run.samples[(size_t)slot * run.B + chain] = bits;
#pragma unroll
      for (int k = 0; k < HPL; ++k) g[k] = act_df<ACT>(th[k]);
      ++sweep;
    }
  };

  if (nsteps > 0) {
    Pre pa, pb;
    fetch(0, pa);
    uint32_t t = 0;
    for (; t + 1 < nsteps; t += 2) {
      step(t, pa, pb);
      step(t + 1, pb, pa);
    }
    if (t < nsteps) step(t, pa, pb);
  }
  if (run.write_last_at_end && active && lane == 0) run.samples[chain] = bits;
  if (active && lane == 0) atomicAdd(run.accepted, (unsigned long long)naccept);
}

template <typename R, int G, int HPL, int ACT, bool EXCH, bool HALF>
__global__ void __launch_bounds__(256) rbm_sampler_kernel(RbmDev<R> net, SamplerRun run) {
  sampler_block<R, G, HPL, ACT, EXCH, HALF>(net, run, blockIdx.x);
}

// Many independent problems in one launch: job p owns blocks
// [blk_start[p], blk_start[p+1]); every block loads its own problem's tables.
// A problem whose hidden units fit in half the units per lane of the largest
// one runs the narrower loop (its blocks lay out their tables for it).
template <typename R, int G, int HPL, int ACT>
__global__ void __launch_bounds__(256)
rbm_sampler_batch_kernel(const SamplerJob<R>* __restrict__ jobs, const int* __restrict__ blk_start, int np) {
  int lo = 0, hi = np - 1;
  const int b = blockIdx.x;
  while (lo < hi) {                       // last p with blk_start[p] <= b
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(blk_start + mid) <= b) lo = mid; else hi = mid - 1;
  }
  const SamplerJob<R> job = jobs[lo];
  const int blk = b - __ldg(blk_start + lo);
  constexpr int HLO = (HPL + 1) / 2;
  if (HLO < HPL && job.net.M <= G * HLO)
    sampler_block<R, G, HLO, ACT, false, false, false>(job.net, job.run, blk);
  else
    sampler_block<R, G, HPL, ACT, false, false, false>(job.net, job.run, blk);
}

}  // namespace

template <typename R, int G, int HPL, int ACT, bool EXCH, bool HALF>
static cudaError_t sampler_inst(const RbmDev<R>& net, const SamplerRun& run, cudaStream_t st) {
  const int threads = run.block;
  const int chains_per_block = threads / G;
  const int blocks = (run.B + chains_per_block - 1) / chains_per_block;
  const int NR = EXCH ? net.n_rows : net.N;
  size_t smem = (size_t)4 * NR * (G * HPL) * sizeof(cpx<R>) + (EXCH ? NR * sizeof(int2) : 0) + NR * sizeof(R);
  auto kern = rbm_sampler_kernel<R, G, HPL, ACT, EXCH, HALF>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<blocks, threads, smem, st>>>(net, run);
  return cudaGetLastError();
}

template <typename R, int G, int ACT, bool EXCH, bool HALF>
static cudaError_t sampler_hpl(const RbmDev<R>& net, const SamplerRun& run, cudaStream_t st) {
  const int hpl = (net.M + G - 1) / G;
  switch (hpl) {
    case 1: return sampler_inst<R, G, 1, ACT, EXCH, HALF>(net, run, st);
    case 2: return sampler_inst<R, G, 2, ACT, EXCH, HALF>(net, run, st);
    case 3: return sampler_inst<R, G, 3, ACT, EXCH, HALF>(net, run, st);
    case 4: return sampler_inst<R, G, 4, ACT, EXCH, HALF>(net, run, st);
    case 5: return sampler_inst<R, G, 5, ACT, EXCH, HALF>(net, run, st);
    case 6: return sampler_inst<R, G, 6, ACT, EXCH, HALF>(net, run, st);
    case 8: return sampler_inst<R, G, 8, ACT, EXCH, HALF>(net, run, st);
    case 10: return sampler_inst<R, G, 10, ACT, EXCH, HALF>(net, run, st);
    default: return cudaErrorInvalidValue;
  }
}

template <typename R, int ACT, bool EXCH, bool HALF = false>
static cudaError_t sampler_g(const RbmDev<R>& net, const SamplerRun& run, int G, cudaStream_t st) {
  switch (G) {
    case 4: return sampler_hpl<R, 4, ACT, EXCH, HALF>(net, run, st);
    case 8: return sampler_hpl<R, 8, ACT, EXCH, HALF>(net, run, st);
    case 16: return sampler_hpl<R, 16, ACT, EXCH, HALF>(net, run, st);
    case 32: return sampler_hpl<R, 32, ACT, EXCH, HALF>(net, run, st);
    default: return cudaErrorInvalidValue;
  }
}

// hidden units per lane supported by the instantiations above
static inline bool hpl_ok(int hpl) { return hpl <= 6 || hpl == 8 || hpl == 10; }

template <typename R>
cudaError_t launch_rbm_sampler(const RbmDev<R>& net, const SamplerRun& run, int G, cudaStream_t st) {
  if (net.N > 64 || net.M > 320) return cudaErrorInvalidValue;
  if (!hpl_ok((net.M + G - 1) / G)) return cudaErrorInvalidValue;
  if (net.pairs || net.opm) {
    // exchange rule and OperatorRule: FP32 ket (RBM) handles only, instantiated
    // in sampler_exch.cu and sampler_oprule.cu
    if constexpr (std::is_same<R, float>::value)
      return net.opm ? launch_rbm_sampler_oprule(net, run, G, st) : launch_rbm_sampler_exchange(net, run, G, st);
    else return cudaErrorInvalidValue;
  }
  // units at weight 1/2 (density matrices): instantiated in sampler_half32.cu / sampler_half64.cu
  if (net.n_half > 0) return launch_rbm_sampler_half<R>(net, run, G, st);
  if (net.act == ACT_LOGCOSH) return sampler_g<R, ACT_LOGCOSH, false>(net, run, G, st);
  return sampler_g<R, ACT_SOFTPLUS, false>(net, run, G, st);
}


template <typename R, int G, int HPL, int ACT>
static cudaError_t sampler_batch_inst(const SamplerJob<R>* jobs, const int* blk_start, int np, int total_blocks,
                                      int N_max, cudaStream_t st) {
  const size_t smem = (size_t)4 * N_max * (G * HPL) * sizeof(cpx<R>) + N_max * sizeof(R);
  auto kern = rbm_sampler_batch_kernel<R, G, HPL, ACT>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<total_blocks, 256, smem, st>>>(jobs, blk_start, np);
  return cudaGetLastError();
}

template <typename R, int G, int ACT>
static cudaError_t sampler_batch_hpl(const SamplerJob<R>* jobs, const int* blk_start, int np, int total_blocks,
                                     int M_max, int N_max, cudaStream_t st) {
  switch ((M_max + G - 1) / G) {
    case 1: return sampler_batch_inst<R, G, 1, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    case 2: return sampler_batch_inst<R, G, 2, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    case 3: return sampler_batch_inst<R, G, 3, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    case 4: return sampler_batch_inst<R, G, 4, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    case 5: return sampler_batch_inst<R, G, 5, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    case 6: return sampler_batch_inst<R, G, 6, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    case 8: return sampler_batch_inst<R, G, 8, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    case 10: return sampler_batch_inst<R, G, 10, ACT>(jobs, blk_start, np, total_blocks, N_max, st);
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
cudaError_t launch_rbm_sampler_batch(const SamplerJob<R>* jobs, const int* blk_start, int np, int total_blocks,
                                     int M_max, int N_max, int act, int G, cudaStream_t st) {
  if (N_max > 64 || !hpl_ok((M_max + G - 1) / G)) return cudaErrorInvalidValue;
  switch (G) {
    case 4: return act == ACT_LOGCOSH ? sampler_batch_hpl<R, 4, ACT_LOGCOSH>(jobs, blk_start, np, total_blocks, M_max, N_max, st)
                                      : sampler_batch_hpl<R, 4, ACT_SOFTPLUS>(jobs, blk_start, np, total_blocks, M_max, N_max, st);
    case 8: return act == ACT_LOGCOSH ? sampler_batch_hpl<R, 8, ACT_LOGCOSH>(jobs, blk_start, np, total_blocks, M_max, N_max, st)
                                      : sampler_batch_hpl<R, 8, ACT_SOFTPLUS>(jobs, blk_start, np, total_blocks, M_max, N_max, st);
    case 16: return act == ACT_LOGCOSH ? sampler_batch_hpl<R, 16, ACT_LOGCOSH>(jobs, blk_start, np, total_blocks, M_max, N_max, st)
                                       : sampler_batch_hpl<R, 16, ACT_SOFTPLUS>(jobs, blk_start, np, total_blocks, M_max, N_max, st);
    case 32: return act == ACT_LOGCOSH ? sampler_batch_hpl<R, 32, ACT_LOGCOSH>(jobs, blk_start, np, total_blocks, M_max, N_max, st)
                                       : sampler_batch_hpl<R, 32, ACT_SOFTPLUS>(jobs, blk_start, np, total_blocks, M_max, N_max, st);
    default: return cudaErrorInvalidValue;
  }
}
