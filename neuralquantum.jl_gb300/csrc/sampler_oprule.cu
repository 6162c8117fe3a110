// Metropolis sampler with the OperatorRule (reference:
// src/Samplers/MCMCRules/OperatorRule.jl:23-58 inside samplenext!,
// src/Samplers/Metropolis.jl:124-167), FP32 RBM.
//
// A step of chain σ: n_f = number of connections of σ's rows in the
// operator's tables (row_valdiff: every operator of the sum in order, the
// diagonal entry first, KLocalOperator.jl:151-158), one of them drawn
// uniformly (k = floor(r0 n_f / 2^32) of the step's Philox word), its changes
// applied, n_b counted at σ', and σ' accepted iff u < exp(log p(σ') - log p(σ)
// + log(n_f / n_b)).  A connection without changes proposes σ itself (always
// accepted, as u < 1).
//
// The θ-cache of the local sampler carries over: the changing connections are
// grouped into move classes (the changed sites and their new local indices,
// up to complement); Δθ of a class is ±d rW with rW = Σ_q W[h, s_q](2b_q - 1),
// so the cosh/sinh/tanh (softplus: e^{±Δ} - 1) tables of the class give the
// ratio and the accepted update exactly as the single-flip tables do.  Row
// lengths are counted by the chain's G lanes over contiguous blocks of
// operators; when every operator has rows of one length the counts are
// constants and the move is located by a binary search of the operators'
// first move indices.
#include "sampler_impl.cuh"

namespace {

// row of an operator at `bits`: site d of the operator (byte d of `sites`)
// gives bit d of the row index (first site least significant)
NQ_D int op_row(unsigned long long sites, int ns, uint64_t bits) {
  int r = 0;
  for (int d = 0; d < ns; ++d) r |= (int)((bits >> ((sites >> (8 * d)) & 0xffull)) & 1ull) << d;
  return r;
}

__global__ void rbm_class_tables_kernel(RbmDev<float> net, OpMovesDev m, cpx<float>* t0, cpx<float>* t1,
                                        cpx<float>* t2, cpx<float>* rW, float* rare) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;   // idx = k*M + h
  const int M = net.M;
  if (idx < m.n_classes) {
    double s = 0.0;
    const int cb = m.class_bits[idx];
    for (int q = 0; q < 8; ++q) {
      const int site = m.class_sites[8 * idx + q];
      if (site < 0) break;
      s += (((cb >> q) & 1) ? 1.0 : -1.0) * (double)net.a[site].x;
    }
    rare[idx] = (float)(2.8853900817779268 * s);
  }
  if (idx >= m.n_classes * M) return;
  const int k = idx / M, h = idx % M;
  const int cb = m.class_bits[k];
  double wx = 0.0, wy = 0.0;
  for (int q = 0; q < 8; ++q) {
    const int site = m.class_sites[8 * k + q];
    if (site < 0) break;
    const double sg = ((cb >> q) & 1) ? 1.0 : -1.0;
    const cpx<float> w = net.W[h + M * site];
    wx += sg * (double)w.x;
    wy += sg * (double)w.y;
  }
  rW[h + M * k] = mk((float)wx, (float)wy);
  const double d = net.hilb == HILB_SPIN ? 2.0 : 1.0;
  const cpx<double> z = mk(wx * d, wy * d);
  cpx<double> c0, c1, c2;
  if (net.act == ACT_LOGCOSH) {
    c0 = ccoshc(z);
    c1 = csinhc(z);
    c2 = act_df<ACT_LOGCOSH>(z);
  } else {
    const cpx<double> ep = cexpc(z), em = cexpc(mk(-z.x, -z.y));
    c0 = mk(ep.x - 1.0, ep.y);
    c1 = mk(em.x - 1.0, em.y);
    c2 = mk(0.0, 0.0);
  }
  t0[idx] = mk((float)c0.x, (float)c0.y);
  t1[idx] = mk((float)c1.x, (float)c1.y);
  t2[idx] = mk((float)c2.x, (float)c2.y);
}

template <int G, int HPL, int ACT>
__global__ void __launch_bounds__(256) oprule_sampler_kernel(RbmDev<float> net, OpMovesDev mv, SamplerRun run) {
  using R = float;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int MP = G * HPL;
  const int N = net.N, M = net.M, NC = mv.n_classes, NO = mv.n_ops;
  cpx_pair<R>* s_t01 = reinterpret_cast<cpx_pair<R>*>(smem_raw);            // {t0, t1} at k*MP + h
  cpx_pair<R>* s_t2w = s_t01 + NC * MP;                                      // {t2, rW} at k*MP + h
  unsigned long long* s_cmask = reinterpret_cast<unsigned long long*>(s_t2w + NC * MP);   // [NC]
  unsigned long long* s_osites = s_cmask + NC;                               // [NO]
  unsigned long long* s_omask = s_osites + NO;                               // [NO]
  R* s_are = reinterpret_cast<R*>(s_omask + NO);                             // [NC]
  int* s_on = reinterpret_cast<int*>(s_are + NC);                            // [NO]
  int* s_orow = s_on + NO;                                                   // [NO]
  int* s_opre = s_orow + NO;                                                 // [NO + 1]
  int* s_rco = s_opre + NO + 1;                                              // [n_rows + 1]
  int* s_code = s_rco + mv.n_rows + 1;                                       // [n_conns]
  for (int k = threadIdx.x; k < NC * MP; k += blockDim.x) {
    const int i = k / MP, h = k % MP;
    cpx_pair<R> p01, p2w;
    if (h < M) {
      p01.a = net.t0[i * M + h];
      p01.b = net.t1[i * M + h];
      p2w.a = ACT == ACT_LOGCOSH ? net.t2[i * M + h] : mk(R(0), R(0));
      p2w.b = net.rW[h + M * i];
    } else {
      p01.a = ACT == ACT_LOGCOSH ? mk(R(1), R(0)) : mk(R(0), R(0));
      p01.b = mk(R(0), R(0));
      p2w.a = mk(R(0), R(0));
      p2w.b = mk(R(0), R(0));
    }
    s_t01[k] = p01;
    s_t2w[k] = p2w;
  }
  for (int k = threadIdx.x; k < NC; k += blockDim.x) {
    s_cmask[k] = mv.class_mask[k];
    s_are[k] = net.rare[k];
  }
  for (int k = threadIdx.x; k < NO; k += blockDim.x) {
    s_osites[k] = mv.op_sites[k];
    s_omask[k] = mv.op_mask[k];
    s_on[k] = mv.op_n_sites[k];
    s_orow[k] = mv.op_row_offset[k];
  }
  for (int k = threadIdx.x; k <= NO; k += blockDim.x) s_opre[k] = mv.const_counts ? mv.op_prefix[k] : 0;
  for (int k = threadIdx.x; k <= mv.n_rows; k += blockDim.x) s_rco[k] = mv.row_conn_offset[k];
  for (int k = threadIdx.x; k < mv.n_conns; k += blockDim.x) s_code[k] = mv.conn_code[k];
  __syncthreads();

  const int lane = threadIdx.x % G;
  const int chain_raw = (blockIdx.x * blockDim.x + threadIdx.x) / G;
  const bool active = chain_raw < run.B;
  const int chain = active ? chain_raw : run.B - 1;
  const int hilb = net.hilb;
  if (run.call_ptr) run.call = *run.call_ptr;

  uint64_t bits = 0;
  for (int q = 0; q < N; q += 4) {
    u32x4 w = philox4x32_10((uint32_t)(q >> 2), run.call, (uint32_t)chain, TAG_INIT, run.k0, run.k1);
    uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (q + k < N && (ws[k] >> 31)) bits |= 1ull << (q + k);
  }

  cpx<R> th[HPL], g[HPL];
#pragma unroll
  for (int k = 0; k < HPL; ++k) {
    const int h = lane + G * k;
    cpx<R> t = h < M ? net.b[h] : mk(R(0), R(0));
    if (h < M)
      for (int j = 0; j < N; ++j) {
        const R v = site_value<R>(bits, j, hilb);
        const cpx<R> w = net.W[h + M * j];
        t.x += w.x * v;
        t.y += w.y * v;
      }
    th[k] = t;
    g[k] = act_df<ACT>(t);
  }
  const R dmag = hilb == HILB_SPIN ? R(2) : R(1);
  // this lane's contiguous block of operators for the row-length counts
  const int per = (NO + G - 1) / G;
  const int o0 = min(NO, lane * per), o1 = min(NO, o0 + per);

  unsigned long long naccept = 0;
  const int nsweeps = run.burn + run.n_record;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
  uint32_t t = 0;
  uint32_t my_r0 = 0;
  R my_lu = 0;
  for (int sweep = 0; sweep < nsweeps; ++sweep) {
    for (int pass = 0; pass < run.passes; ++pass, ++t) {
      const int slot = (int)(t & (G - 1));
      if (slot == 0) {
        const u32x4 r = philox4x32_10(t + (uint32_t)lane, run.call, (uint32_t)chain, TAG_MH, run.k0, run.k1);
        my_r0 = r.x;
        my_lu = fast_log2((R)uniform24(r.y));
      }
      const uint32_t r0 = __shfl_sync(gmask, my_r0, slot, G);
      const R lu = __shfl_sync(gmask, my_lu, slot, G);
      int nf, code;
      if (mv.const_counts) {
        nf = mv.n_total;
        const int kk = (int)uniform_site(r0, (uint32_t)nf);
        int lo = 0, hi = NO - 1;                 // last operator whose first move is <= kk
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_opre[mid] <= kk) lo = mid;
          else hi = mid - 1;
        }
        const int row = s_orow[lo] + op_row(s_osites[lo], s_on[lo], bits);
        code = s_code[s_rco[row] + kk - s_opre[lo]];
      } else {
        int mine = 0;
        for (int o = o0; o < o1; ++o) {
          const int row = s_orow[o] + op_row(s_osites[o], s_on[o], bits);
          mine += s_rco[row + 1] - s_rco[row];
        }
        int incl = mine;
#pragma unroll
        for (int off = 1; off < G; off <<= 1) {
          const int y = __shfl_up_sync(gmask, incl, off, G);
          if (lane >= off) incl += y;
        }
        nf = __shfl_sync(gmask, incl, G - 1, G);
        const int kk = (int)uniform_site(r0, (uint32_t)nf);
        const int excl = incl - mine;
        const bool owner = kk >= excl && kk < incl;
        int my_code = -1;
        if (owner) {
          int acc = excl;
          for (int o = o0; o < o1; ++o) {
            const int row = s_orow[o] + op_row(s_osites[o], s_on[o], bits);
            const int cnt = s_rco[row + 1] - s_rco[row];
            if (kk < acc + cnt) {
              my_code = s_code[s_rco[row] + kk - acc];
              break;
            }
            acc += cnt;
          }
        }
        const unsigned own = __ballot_sync(gmask, owner);
        code = __shfl_sync(gmask, my_code, __ffs(own) - 1);
      }
      if (code < 0) {
        // a connection without changes proposes σ itself: ratio 1, accepted
        ++naccept;
        if (run.accept_bits && active && lane == 0) run.accept_bits[(size_t)t * run.B + chain] = 1;
        continue;
      }
      const int cls = code >> 1;
      const bool pos = !(code & 1);
      const uint64_t fmask = s_cmask[cls];
      const R dv = pos ? dmag : -dmag;
      const cpx_pair<R>* trow = s_t01 + cls * MP + lane;
      R prod = R(1);
#pragma unroll
      for (int k = 0; k < HPL; ++k) {
        const cpx_pair<R> tt = trow[G * k];
        cpx<R> rr;
        if (ACT == ACT_LOGCOSH) {
          cpx<R> c1 = tt.b;
          if (!pos) c1 = mk(-c1.x, -c1.y);
          rr = cfma(g[k], c1, tt.a);
        } else {
          const cpx<R> bb = pos ? tt.a : tt.b;
          rr = cfma(g[k], bb, mk(R(1), R(0)));
        }
        prod *= abs2c(rr);
      }
      R lsum = fast_log2(prod);
#pragma unroll
      for (int off = G / 2; off > 0; off >>= 1) lsum += __shfl_xor_sync(gmask, lsum, off, G);
      R logA = s_are[cls] * dv + lsum;               // log2 p(σ')/p(σ)
      if (!mv.const_counts) {
        // n_b: only operators touching the changed sites change their row
        const uint64_t nbits = bits ^ fmask;
        int d = 0;
        for (int o = o0; o < o1; ++o)
          if (s_omask[o] & fmask) {
            const int ra = s_orow[o] + op_row(s_osites[o], s_on[o], bits);
            const int rb = s_orow[o] + op_row(s_osites[o], s_on[o], nbits);
            d += (s_rco[rb + 1] - s_rco[rb]) - (s_rco[ra + 1] - s_rco[ra]);
          }
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) d += __shfl_xor_sync(gmask, d, off, G);
        logA += fast_log2((R)nf) - fast_log2((R)(nf + d));      // log2(n_f / n_b)
      }
      const bool acc = lu < logA;
      if (acc) {
#pragma unroll
        for (int k = 0; k < HPL; ++k) {
          const cpx_pair<R> tw = s_t2w[cls * MP + lane + G * k];
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
            const cpx_pair<R> tt = trow[G * k];
            const cpx<R> bb = pos ? tt.a : tt.b;
            num = g[k] * mk(R(1) + bb.x, bb.y);
            den = cfma(g[k], bb, mk(R(1), R(0)));
          }
          const R inv = fast_rcp(abs2c(den));
          g[k] = inv * (num * conjc(den));
        }
        bits ^= fmask;
        ++naccept;
      }
      if (run.accept_bits && active && lane == 0) run.accept_bits[(size_t)t * run.B + chain] = acc ? 1 : 0;
    }
    const int slot = sweep - run.burn;
    if (slot >= 0 && active && lane == 0) run.samples[(size_t)slot * run.B + chain] = bits;
#pragma unroll
    for (int k = 0; k < HPL; ++k) g[k] = act_df<ACT>(th[k]);
  }
  if (run.write_last_at_end && active && lane == 0) run.samples[chain] = bits;
  if (active && lane == 0) atomicAdd(run.accepted, naccept);
}

template <int G, int HPL, int ACT>
cudaError_t oprule_inst(const RbmDev<float>& net, const SamplerRun& run, cudaStream_t st) {
  const OpMovesDev& mv = *net.opm;
  const size_t smem = oprule_sampler_smem(mv, net.M, G);
  if (smem == 0) return cudaErrorInvalidValue;
  const int threads = run.block;
  const int blocks = (run.B + threads / G - 1) / (threads / G);
  auto kern = oprule_sampler_kernel<G, HPL, ACT>;
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<blocks, threads, smem, st>>>(net, mv, run);
  return cudaGetLastError();
}

template <int G, int ACT>
cudaError_t oprule_hpl(const RbmDev<float>& net, const SamplerRun& run, cudaStream_t st) {
  switch ((net.M + G - 1) / G) {
    case 1: return oprule_inst<G, 1, ACT>(net, run, st);
    case 2: return oprule_inst<G, 2, ACT>(net, run, st);
    case 3: return oprule_inst<G, 3, ACT>(net, run, st);
    case 4: return oprule_inst<G, 4, ACT>(net, run, st);
    case 5: return oprule_inst<G, 5, ACT>(net, run, st);
    case 6: return oprule_inst<G, 6, ACT>(net, run, st);
    case 8: return oprule_inst<G, 8, ACT>(net, run, st);
    case 10: return oprule_inst<G, 10, ACT>(net, run, st);
    default: return cudaErrorInvalidValue;
  }
}

template <int ACT>
cudaError_t oprule_g(const RbmDev<float>& net, const SamplerRun& run, int G, cudaStream_t st) {
  switch (G) {
    case 4: return oprule_hpl<4, ACT>(net, run, st);
    case 8: return oprule_hpl<8, ACT>(net, run, st);
    case 16: return oprule_hpl<16, ACT>(net, run, st);
    case 32: return oprule_hpl<32, ACT>(net, run, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

size_t oprule_sampler_smem(const OpMovesDev& m, int M, int G) {
  if (G < 1 || M < 1) return 0;
  const size_t MP = (size_t)G * ((M + G - 1) / G);
  const size_t s = 2 * (size_t)m.n_classes * MP * sizeof(cpx_pair<float>) +
                   ((size_t)m.n_classes + 2 * (size_t)m.n_ops) * sizeof(unsigned long long) +
                   (size_t)m.n_classes * sizeof(float) +
                   (3 * (size_t)m.n_ops + 1 + (size_t)m.n_rows + 1 + (size_t)m.n_conns) * sizeof(int);
  return s <= 232448 ? s : 0;
}

cudaError_t launch_rbm_class_tables(const RbmDev<float>& net, const OpMovesDev& m, cpx<float>* t0, cpx<float>* t1,
                                    cpx<float>* t2, cpx<float>* rW, float* rare, cudaStream_t st) {
  const int n = m.n_classes * net.M > m.n_classes ? m.n_classes * net.M : m.n_classes;
  if (n < 1) return cudaSuccess;
  rbm_class_tables_kernel<<<(n + 255) / 256, 256, 0, st>>>(net, m, t0, t1, t2, rW, rare);
  return cudaGetLastError();
}

cudaError_t launch_rbm_sampler_oprule(const RbmDev<float>& net, const SamplerRun& run, int G, cudaStream_t st) {
  if (!net.opm || net.opm->n_classes < 1 || net.opm->n_ops < 1 || net.n_half != 0 || net.N > 64)
    return cudaErrorInvalidValue;
  if (!hpl_ok((net.M + G - 1) / G)) return cudaErrorInvalidValue;
  if (net.act == ACT_LOGCOSH) return oprule_g<ACT_LOGCOSH>(net, run, G, st);
  return oprule_g<ACT_SOFTPLUS>(net, run, G, st);
}
