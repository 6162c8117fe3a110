// Exact sampler (reference: src/Samplers/Exact.jl:52-82, batched variant
// :133-176): the distribution |ψ(σ)|² over all 2^N configurations, its
// cumulative sum, and draws by inverse CDF (searchsortedfirst of a uniform).
//
// Configuration i has bit j = local index of site j (first site least
// significant, spin -1 / Fock 0 <-> 0), the order of set!(σ, hilb, i) in the
// reference.  The target is the Metropolis sampler's: log|ψ|² = 2 Re aᵀv +
// Σ_h c_h 2 Re f(θ_h) with c_h = 1/2 for the units h < n_half of the doubled
// density-matrix state.  The CDF is built in FP64 from exp(log|ψ|² - max), in
// a fixed order (block-local inclusive scans, one scan of the block totals,
// then an add-back), so it is deterministic and monotone.
#include "nq_kernels.cuh"

namespace {

constexpr int EB = 256;          // threads per block
constexpr int EPT = 8;           // configurations per thread in the scan pass
constexpr int ECH = EB * EPT;    // configurations per scan block

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

template <typename R, int ACT>
__global__ void __launch_bounds__(EB) exact_logprob_kernel(RbmDev<R> net, long nconf, double* __restrict__ lp,
                                                           double* __restrict__ bmax) {
  const long i = blockIdx.x * (long)EB + threadIdx.x;
  double v = -INFINITY;
  if (i < nconf) {
    const uint64_t bits = (uint64_t)i;
    const int N = net.N, M = net.M, hilb = net.hilb;
    R sa = R(0);
    for (int j = 0; j < N; ++j) sa += net.a[j].x * site_value<R>(bits, j, hilb);
    double acc = 2.0 * (double)sa;
    for (int h0 = 0; h0 < M; h0 += 4) {
      cpx<R> th[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) th[u] = h0 + u < M ? net.b[h0 + u] : mk(R(0), R(0));
      for (int j = 0; j < N; ++j) {
        const R s = site_value<R>(bits, j, hilb);
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (h0 + u < M) {
            const cpx<R> w = net.W[h0 + u + M * j];
            th[u].x += w.x * s;
            th[u].y += w.y * s;
          }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (h0 + u < M) acc += (h0 + u < net.n_half ? 1.0 : 2.0) * (double)act_f<ACT>(th[u]).x;
    }
    v = acc;
    lp[i] = v;
  }
  __shared__ double sh[EB / 32];
  v = warp_max(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double m = threadIdx.x < EB / 32 ? sh[threadIdx.x] : -INFINITY;
    m = warp_max(m);
    if (threadIdx.x == 0) bmax[blockIdx.x] = m;
  }
}

// one block: out[0] = max over vals[0..n)
__global__ void __launch_bounds__(1024) exact_max_kernel(const double* __restrict__ vals, long n,
                                                         double* __restrict__ out) {
  double m = -INFINITY;
  for (long k = threadIdx.x; k < n; k += blockDim.x) m = fmax(m, vals[k]);
  __shared__ double sh[32];
  m = warp_max(m);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : -INFINITY;
    v = warp_max(v);
    if (threadIdx.x == 0) out[0] = v;
  }
}

// exclusive scan of one value per thread over the block (fixed order)
__device__ double block_exclusive_scan(double x, double* total) {
  __shared__ double wsum[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double inc = x;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc += y;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    double s = lane < nw ? wsum[lane] : 0.0;
    double si = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, si, off);
      if (lane >= off) si += y;
    }
    if (lane < nw) wsum[lane] = si - s;       // exclusive warp offsets
    if (lane == 31) *total = si;
  }
  __syncthreads();
  const double r = wsum[w] + (inc - x);
  __syncthreads();
  return r;
}

// cdf[i] (in place over lp) = block-local inclusive sum of exp(lp - max); bsum = block totals
__global__ void __launch_bounds__(EB) exact_scan_kernel(double* __restrict__ cdf, long nconf,
                                                        const double* __restrict__ gmax, double* __restrict__ bsum) {
  const long base = blockIdx.x * (long)ECH + (long)threadIdx.x * EPT;
  const double mx = gmax[0];
  double p[EPT];
  double run = 0.0;
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const long i = base + e;
    run += i < nconf ? exp(cdf[i] - mx) : 0.0;
    p[e] = run;
  }
  __shared__ double total;
  const double off = block_exclusive_scan(run, &total);
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const long i = base + e;
    if (i < nconf) cdf[i] = off + p[e];
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// one block: boff[b] = Σ_{b' < b} bsum[b'] (fixed order), boff[nb] = total
__global__ void __launch_bounds__(1024) exact_block_offsets_kernel(const double* __restrict__ bsum, int nb,
                                                                   double* __restrict__ boff) {
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  double s = 0.0;
  for (int b = b0; b < min(nb, b0 + per); ++b) s += bsum[b];
  __shared__ double total;
  double run = block_exclusive_scan(s, &total);
  for (int b = b0; b < min(nb, b0 + per); ++b) {
    boff[b] = run;
    run += bsum[b];
  }
  if (threadIdx.x == 0) boff[nb] = total;
}

__global__ void __launch_bounds__(EB) exact_addback_kernel(double* __restrict__ cdf, long nconf,
                                                           const double* __restrict__ boff) {
  const long i = blockIdx.x * (long)EB + threadIdx.x;
  if (i < nconf) cdf[i] += boff[i / ECH];
}

// draw t of chain c (t < n_record: slot t; the stale-last-slot quirk's single
// draw goes to slot 0): u = 53-bit uniform of Philox (t, call, chain, TAG_EXACT),
// configuration = first i with cdf[i] >= u * total
__global__ void __launch_bounds__(EB) exact_draw_kernel(const double* __restrict__ cdf, long nconf,
                                                        const double* __restrict__ total, SamplerRun run,
                                                        int ndraws) {
  const long idx = blockIdx.x * (long)EB + threadIdx.x;
  const int B = run.B;
  if (idx == 0) atomicAdd(run.accepted, (unsigned long long)B * (unsigned long long)ndraws);
  if (idx >= (long)B * ndraws) return;
  const int chain = (int)(idx % B), t = (int)(idx / B);
  const uint32_t call = run.call_ptr ? *run.call_ptr : run.call;
  const u32x4 w = philox4x32_10((uint32_t)t, call, (uint32_t)chain, TAG_EXACT, run.k0, run.k1);
  const double u = uniform53(w.x, w.y);
  const double target = u * total[0];
  long lo = 0, hi = nconf - 1;
  while (lo < hi) {
    const long mid = (lo + hi) >> 1;
    if (cdf[mid] >= target) hi = mid;
    else lo = mid + 1;
  }
  const int slot = t < run.n_record ? t : 0;
  run.samples[(size_t)slot * B + chain] = (uint64_t)lo;
}

}  // namespace

size_t exact_sampler_work_doubles(int nsites) {
  const long nconf = 1L << nsites;
  const long nb1 = (nconf + EB - 1) / EB, nb2 = (nconf + ECH - 1) / ECH;
  return (size_t)(nconf + nb1 + 1 + nb2 + nb2 + 1);
}

template <typename R>
cudaError_t launch_exact_sampler(const RbmDev<R>& net, const SamplerRun& run, double* work, cudaStream_t st) {
  if (net.N < 1 || net.N > 26) return cudaErrorInvalidValue;
  const long nconf = 1L << net.N;
  const long nb1 = (nconf + EB - 1) / EB, nb2 = (nconf + ECH - 1) / ECH;
  double* cdf = work;
  double* bmax = cdf + nconf;
  double* gmax = bmax + nb1;
  double* bsum = gmax + 1;
  double* boff = bsum + nb2;        // [nb2 + 1], boff[nb2] = total
  if (net.act == ACT_LOGCOSH)
    exact_logprob_kernel<R, ACT_LOGCOSH><<<(unsigned)nb1, EB, 0, st>>>(net, nconf, cdf, bmax);
  else
    exact_logprob_kernel<R, ACT_SOFTPLUS><<<(unsigned)nb1, EB, 0, st>>>(net, nconf, cdf, bmax);
  exact_max_kernel<<<1, 1024, 0, st>>>(bmax, nb1, gmax);
  exact_scan_kernel<<<(unsigned)nb2, EB, 0, st>>>(cdf, nconf, gmax, bsum);
  exact_block_offsets_kernel<<<1, 1024, 0, st>>>(bsum, (int)nb2, boff);
  exact_addback_kernel<<<(unsigned)nb1, EB, 0, st>>>(cdf, nconf, boff);
  const int ndraws = run.n_record + (run.write_last_at_end ? 1 : 0);
  const long nd = (long)run.B * ndraws;
  exact_draw_kernel<<<(unsigned)((nd + EB - 1) / EB > 0 ? (nd + EB - 1) / EB : 1), EB, 0, st>>>(
      cdf, nconf, boff + nb2, run, ndraws);
  return cudaGetLastError();
}

template cudaError_t launch_exact_sampler<float>(const RbmDev<float>&, const SamplerRun&, double*, cudaStream_t);
template cudaError_t launch_exact_sampler<double>(const RbmDev<double>&, const SamplerRun&, double*, cudaStream_t);
