// RBM hot path: per-flip tables, the persistent Metropolis sampler with an
// incremental θ-cache, batched logψ / f'(θ) / local-estimator evaluation and
// the force partial sums.
//
// Reference: src/Networks/ClosedSystems/RBM.jl:40-105, RBMBatched.jl:37-91
// (network), src/Samplers/Metropolis.jl:101-167 + MCMCRules/LocalRule.jl:19-28
// (sampler), src/IterativeInterface/Accumulators/AccumulatorObsScalar.jl:52-137
// (estimator), src/IterativeInterface/Samplers/CostFun/BatchedValSampler.jl:97-115
// and BaseIterativeSampler.jl:19-26 (centring and force).
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "nq_kernels.cuh"

namespace {

// ---------------------------------------------------------------------------
// parameters: FP64 master (interleaved complex, reference order a, b, W) ->
// FP32 working copy
// ---------------------------------------------------------------------------
__global__ void master_to_f32_kernel(const double* m, long n, float* out) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)m[i];
}

template <typename R>
NQ_D void rbm_tables_elem(const RbmDev<R>& net, cpx<R>* t0, cpx<R>* t1, cpx<R>* t2, int idx) {   // idx = i*M + h
  if (idx >= net.N * net.M) return;
  int i = idx / net.M, h = idx % net.M;
  // compute in double for accuracy, store as R
  cpx<R> w = net.W[h + net.M * i];
  double d = net.hilb == HILB_SPIN ? 2.0 : 1.0;
  cpx<double> z = mk((double)w.x * d, (double)w.y * d);
  cpx<double> c0, c1, c2;
  if (net.act == ACT_LOGCOSH) {
    c0 = ccoshc(z);
    c1 = csinhc(z);
    c2 = act_df<ACT_LOGCOSH>(z);  // tanh(z)
  } else {
    cpx<double> ep = cexpc(z), em = cexpc(mk(-z.x, -z.y));
    c0 = mk(ep.x - 1.0, ep.y);
    c1 = mk(em.x - 1.0, em.y);
    c2 = mk(0.0, 0.0);
  }
  t0[idx] = mk((R)c0.x, (R)c0.y);
  t1[idx] = mk((R)c1.x, (R)c1.y);
  t2[idx] = mk((R)c2.x, (R)c2.y);
}

template <typename R>
__global__ void rbm_tables_kernel(RbmDev<R> net, cpx<R>* t0, cpx<R>* t1, cpx<R>* t2) {
  rbm_tables_elem<R>(net, t0, t1, t2, blockIdx.x * blockDim.x + threadIdx.x);
}

// per-flip tables of every problem of a grouped step from its FP32 parameters
__global__ void tables_group_kernel(SrGroup g) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.tab_elems) return;
  const int p = group_of(e, g.tab_elem, g.np);
  const SrJob& j = g.jobs[p];
  RbmDev<float> net;
  net.N = j.N; net.M = j.M; net.act = j.act; net.hilb = j.hilb;
  const cpx<float>* base = reinterpret_cast<const cpx<float>*>(j.p32);
  net.a = base;
  net.b = base + j.N;
  net.W = base + j.N + j.M;
  rbm_tables_elem<float>(net, reinterpret_cast<cpx<float>*>(j.t0), reinterpret_cast<cpx<float>*>(j.t1),
                         reinterpret_cast<cpx<float>*>(j.t2), e - __ldg(g.tab_elem + p));
}

template <typename R>
__global__ void rbm_exchange_tables_kernel(RbmDev<R> net, int n_rows, const int2* __restrict__ pairs,
                                           cpx<R>* t0, cpx<R>* t1, cpx<R>* t2, cpx<R>* rW, R* rare) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;   // idx = r*M + h
  if (idx < n_rows) {
    const int2 pr = pairs[idx];
    rare[idx] = (R)(2.8853900817779268 * ((double)net.a[pr.x].x - (double)net.a[pr.y].x));
  }
  if (idx >= n_rows * net.M) return;
  const int r = idx / net.M, h = idx % net.M;
  const int2 pr = pairs[r];
  const cpx<R> wi = net.W[h + net.M * pr.x], wj = net.W[h + net.M * pr.y];
  const cpx<double> w = mk((double)wi.x - (double)wj.x, (double)wi.y - (double)wj.y);
  rW[h + net.M * r] = mk((R)w.x, (R)w.y);
  const double d = net.hilb == HILB_SPIN ? 2.0 : 1.0;
  const cpx<double> z = mk(w.x * d, w.y * d);
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
  t0[idx] = mk((R)c0.x, (R)c0.y);
  t1[idx] = mk((R)c1.x, (R)c1.y);
  t2[idx] = mk((R)c2.x, (R)c2.y);
}

// ---------------------------------------------------------------------------
// Batched evaluation, one thread per sample: θ = Wσ + b, logψ = aᵀσ + Σ f(θ),
// g = f'(θ) and, if an operator is given, the local estimator
//   E_loc(σ) = Σ_diag mel + Σ_{σ'≠σ} mel ψ(σ')/ψ(σ)
// with ψ(σ')/ψ(σ) = exp(aᵀΔσ) Π_h [t0 + g t1] for single flips (table path)
// and exp(aᵀΔσ) Π_h [cosh Δθ + g sinh Δθ] (softplus: 1 + g (e^Δθ - 1)) for
// multi-site changes.  Zero matrix elements are skipped
// (AccumulatorObsScalar.jl:92).
// ---------------------------------------------------------------------------
// theta_in_g: gout already holds θ = Wσ + b ([h][Ns], from the tensor-core
// contraction); it is read and overwritten with g = f'(θ) by the same thread.
// p /= |p| into logscale when |p| leaves [1e-10, 1e10]
template <typename R> NQ_D void rescale(cpx<R>& p, R& logscale) {
  const R m2 = abs2c(p);
  if (m2 > R(1e20) || m2 < R(1e-20)) {
    const R m = sqrt(m2);
    logscale += r_log(m);
    p = (R(1) / m) * p;
  }
}

// {t0, t1} of one (site, hidden unit), one 16-byte (FP32) shared-memory load
template <typename R> struct alignas(16) cpx_t01 {
  cpx<R> t0, t1;
};

template <typename R, int ACT>
NQ_D void eval_block(const RbmDev<R>& net, const uint64_t* __restrict__ samples, int Ns, const DevOp& op,
                     int has_op, cpx<R>* __restrict__ logpsi, cpx<R>* __restrict__ gout,
                     cpx<R>* __restrict__ eloc, int blk, int theta_in_g = 0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = net.N, M = net.M, T = blockDim.x;
  const int M8 = (M + 7) & ~7;                           // hidden units padded to a multiple of 8
  cpx_t01<R>* s_t01 = reinterpret_cast<cpx_t01<R>*>(smem_raw);  // [N*M8] (if has_op)
  cpx<R>* s_W = reinterpret_cast<cpx<R>*>(s_t01 + (has_op ? N * M8 : 0));  // [M8*N], zero padding
  cpx<R>* s_b = s_W + M8 * N;                             // [M8]
  cpx<R>* s_a = s_b + M8;                                 // [N]
  cpx<R>* s_g = s_a + N;                                  // [M8][T], g = 0 on the padding
  for (int k = threadIdx.x; k < M8 * N; k += T) {
    const int h = k % M8, j = k / M8;
    s_W[k] = h < M ? net.W[h + M * j] : mk(R(0), R(0));
  }
  for (int k = threadIdx.x; k < M8; k += T) s_b[k] = k < M ? net.b[k] : mk(R(0), R(0));
  for (int k = threadIdx.x; k < N; k += T) s_a[k] = net.a[k];
  for (int k = threadIdx.x; k < (M8 - M) * T; k += T) s_g[M * T + k] = mk(R(0), R(0));
  if (has_op)
    for (int k = threadIdx.x; k < N * M8; k += T) {
      const int i = k / M8, h = k % M8;
      cpx_t01<R> t;
      // padding: single-flip factor t0 + g t1 = 1 (logcosh) or 1 + g t0 = 1 (softplus)
      t.t0 = h < M ? net.t0[i * M + h] : (ACT == ACT_LOGCOSH ? mk(R(1), R(0)) : mk(R(0), R(0)));
      t.t1 = h < M ? net.t1[i * M + h] : mk(R(0), R(0));
      s_t01[k] = t;
    }
  __syncthreads();
  const int s = blk * T + threadIdx.x;
  if (s >= Ns) return;
  const int hilb = net.hilb;
  const uint64_t bits = samples[s];

  cpx<R> lp = mk(R(0), R(0));
  for (int j = 0; j < N; ++j) {
    R v = site_value<R>(bits, j, hilb);
    lp.x += s_a[j].x * v;
    lp.y += s_a[j].y * v;
  }
  // θ of four hidden units per pass over the sites (one site value per j;
  // the weights are zero-padded to M8 units)
  for (int h0 = 0; h0 < M; h0 += 4) {
    cpx<R> th[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int h = h0 + u;
      th[u] = theta_in_g ? (h < M ? gout[(size_t)h * Ns + s] : mk(R(0), R(0))) : s_b[h];
    }
    if (!theta_in_g) {
      for (int j = 0; j < N; ++j) {
        const R v = site_value<R>(bits, j, hilb);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const cpx<R> w = s_W[h0 + u + M8 * j];
          th[u].x += w.x * v;
          th[u].y += w.y * v;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int h = h0 + u;
      if (h < M) {
        cpx<R> f, gh;
        if (ACT == ACT_LOGCOSH) {
          logcosh_tanh(th[u], &f, &gh);
        } else {
          f = act_f<ACT>(th[u]);
          gh = act_df<ACT>(th[u]);
        }
        lp = lp + f;
        s_g[h * T + threadIdx.x] = gh;
        if (gout) gout[(size_t)h * Ns + s] = gh;
      }
    }
  }
  logpsi[s] = lp;
  if (!has_op) return;

  const R dmag = hilb == HILB_SPIN ? R(2) : R(1);
  cpx<R> E = mk(R(0), R(0));
  for (int o = 0; o < op.n_ops; ++o) {
    const int4 om = __ldg(op.op_meta + o);             // {n_sites, row_offset, sites 0-3, sites 4-7}
    int r = 0;
    for (int d = 0; d < om.x; ++d) {
      const int site = ((d < 4 ? om.z : om.w) >> (8 * (d & 3))) & 0xff;
      r |= (int)((bits >> site) & 1ull) << d;
    }
    const int row = om.y + r;
    const int c0 = __ldg(op.row_conn_offset + row), c1 = __ldg(op.row_conn_offset + row + 1);
    for (int c = c0; c < c1; ++c) {
      const int4 cp = __ldg(op.conn_pack + c);          // {mel re, mel im, n_changes, first change}
      cpx<R> mel;
      if constexpr (std::is_same<R, float>::value) {
        mel = mk(__int_as_float(cp.x), __int_as_float(cp.y));   // FP32 copy: no FP64 compare or conversion
      } else {
        mel = mk((R)__ldg(op.conn_mel + 2 * c), (R)__ldg(op.conn_mel + 2 * c + 1));
      }
      if (mel.x == R(0) && mel.y == R(0)) continue;
      const int nch = cp.z;
      if (nch == 0) { E = E + mel; continue; }
      // exp(aᵀΔσ)
      cpx<R> aexp = mk(R(0), R(0));
      int i1 = -1; R dv1 = 0;
      for (int q = 0; q < nch; ++q) {
        const int site = q == 0 ? (cp.w & 0xff) : __ldg(op.conn_change_site + 8 * c + q);
        const R nv = q == 0 ? (R)(signed char)((cp.w >> 8) & 0xff) : (R)__ldg(op.conn_change_value + 8 * c + q);
        R dv = nv - site_value<R>(bits, site, hilb);
        aexp.x += s_a[site].x * dv;
        aexp.y += s_a[site].y * dv;
        i1 = site; dv1 = dv;
      }
      cpx<R> prod = mk(R(1), R(0));
      R logscale = R(0);
      if (nch == 1) {
        // Π_h (t0 + g t1) over two independent chains (even / odd h),
        // rescaled every eight units
        const bool pos = dv1 > 0;
        const cpx_t01<R>* tt = s_t01 + i1 * M8;
        cpx<R> pa = mk(R(1), R(0)), pb = mk(R(1), R(0));
        for (int h0 = 0; h0 < M8; h0 += 8) {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int h = h0 + u;
            const cpx_t01<R> t = tt[h];
            const cpx<R> gh = s_g[h * T + threadIdx.x];
            cpx<R> rr;
            if (ACT == ACT_LOGCOSH) {
              cpx<R> c1 = t.t1;
              if (!pos) c1 = mk(-c1.x, -c1.y);
              rr = cfma(gh, c1, t.t0);
            } else {
              rr = cfma(gh, pos ? t.t0 : t.t1, mk(R(1), R(0)));
            }
            if (u & 1) pb = pb * rr;
            else pa = pa * rr;
          }
          rescale(pa, logscale);
          rescale(pb, logscale);
        }
        prod = pa * pb;
      } else {
        for (int h = 0; h < M; ++h) {
          cpx<R> dth = mk(R(0), R(0));
          for (int q = 0; q < nch; ++q) {
            int site = __ldg(op.conn_change_site + 8 * c + q);
            R nv = (R)__ldg(op.conn_change_value + 8 * c + q);
            R dv = nv - site_value<R>(bits, site, hilb);
            cpx<R> w = s_W[h + M8 * site];
            dth.x += w.x * dv;
            dth.y += w.y * dv;
          }
          cpx<R> gh = s_g[h * T + threadIdx.x];
          cpx<R> rr;
          if (ACT == ACT_LOGCOSH) rr = cfma(gh, csinhc(dth), ccoshc(dth));
          else {
            cpx<R> e = cexpc(dth);
            rr = cfma(gh, mk(e.x - R(1), e.y), mk(R(1), R(0)));
          }
          prod = prod * rr;
          R m2 = abs2c(prod);
          if (m2 > R(1e20) || m2 < R(1e-20)) {
            R m = sqrt(m2);
            logscale += r_log(m);
            prod = (R(1) / m) * prod;
          }
        }
      }
      (void)dmag;
      cpx<R> ea = cexpc(mk(aexp.x + logscale, aexp.y));
      E = E + mel * (ea * prod);
    }
  }
  eloc[s] = E;
}

// largest block of the single-problem estimator: 512 threads in FP32; FP64
// keeps 256 (its 78 registers per thread would spill under a 512 bound)
template <typename R> constexpr int kEvalMaxThreads = sizeof(R) == 4 ? 512 : 256;

template <typename R, int ACT>
__global__ void __launch_bounds__(kEvalMaxThreads<R>)
rbm_eval_kernel(RbmDev<R> net, const uint64_t* __restrict__ samples, int Ns, DevOp op,
                int has_op, cpx<R>* __restrict__ logpsi, cpx<R>* __restrict__ gout,
                cpx<R>* __restrict__ eloc, int theta_in_g) {
  eval_block<R, ACT>(net, samples, Ns, op, has_op, logpsi, gout, eloc, blockIdx.x, theta_in_g);
}

// Many independent problems in one launch: problem p owns blocks
// [blk_start[p], blk_start[p+1]) of blockDim samples each.
template <typename R, int ACT>
__global__ void __launch_bounds__(128)
rbm_eval_batch_kernel(const EvalJob<R>* __restrict__ jobs, const int* __restrict__ blk_start, int np) {
  int lo = 0, hi = np - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(blk_start + mid) <= b) lo = mid; else hi = mid - 1;
  }
  const EvalJob<R>& job = jobs[lo];
  eval_block<R, ACT>(job.net, job.samples, job.Ns, job.op, job.has_op, job.logpsi, job.g, job.eloc,
                     b - __ldg(blk_start + lo));
}

// ---------------------------------------------------------------------------
// Force partial sums over chunks of CH samples (one block per chunk):
//   O_s  = [v(s), g(s), g(s) v(s)ᵀ]          (P = N + M + M N entries)
//   ΣO, Σ E conj(O), Σ E
// emitted in FP64 per chunk.  The W entries are register tiles of one hidden
// unit h and four sites: per sample, E conj(g_h) and g_h are formed once and
// multiplied by the four site values.  ΣO adds groups of 8 samples in FP32 and
// the group sums with Kahan compensation; the visible-bias sums Σ v are exact
// (integers).
// ---------------------------------------------------------------------------
template <typename R>
NQ_D void kahan_add(cpx<R>& s, cpx<R>& c, cpx<R> x) {
  const cpx<R> y = x - c;
  const cpx<R> t = s + y;
  c = (t - s) - y;
  s = t;
}

template <typename R>
NQ_D void force_partial_block(int N, int M, int hilb, const uint64_t* __restrict__ samples, int Ns,
                              const cpx<R>* __restrict__ g, const cpx<R>* __restrict__ eloc, int CH,
                              double* __restrict__ partial, double* __restrict__ partialE, int blk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int P = N + M + M * N;
  const int NJ = (N + 3) & ~3;                         // sites padded to groups of 4
  const int s0 = blk * CH;
  const int n = min(CH, Ns - s0);
  cpx<R>* s_g = reinterpret_cast<cpx<R>*>(smem_raw);   // [CH][M]: consecutive h conflict-free
  cpx<R>* s_e = s_g + (size_t)M * CH;                  // [CH]
  R* s_v = reinterpret_cast<R*>(s_e + CH);             // [CH][NJ]
  for (int k = threadIdx.x; k < M * CH; k += blockDim.x) {
    const int h = k / CH, t = k % CH;
    s_g[t * M + h] = t < n ? g[(size_t)h * Ns + s0 + t] : mk(R(0), R(0));
  }
  for (int t = threadIdx.x; t < CH; t += blockDim.x) {
    const uint64_t bits = t < n ? samples[s0 + t] : 0;
    s_e[t] = t < n ? eloc[s0 + t] : mk(R(0), R(0));
    for (int j = 0; j < NJ; ++j) s_v[t * NJ + j] = (t < n && j < N) ? site_value<R>(bits, j, hilb) : R(0);
  }
  __syncthreads();
  double* dst = partial + (size_t)blk * 4 * P;
  const int nW = M * (NJ / 4);
  for (int item = threadIdx.x; item < nW + M + N; item += blockDim.x) {
    if (item < nW) {
      const int h = item % M, jq = item / M;
      cpx<R> so[4], co[4], se[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) { so[q] = mk(R(0), R(0)); co[q] = so[q]; se[q] = so[q]; }
      for (int t0 = 0; t0 < n; t0 += 8) {
        cpx<R> po[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) po[q] = mk(R(0), R(0));
        const int t1 = min(n, t0 + 8);
        for (int t = t0; t < t1; ++t) {
          const cpx<R> gv = s_g[t * M + h];
          const cpx<R> a = s_e[t] * conjc(gv);
          const R* v = s_v + t * NJ + 4 * jq;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            po[q].x += gv.x * v[q];
            po[q].y += gv.y * v[q];
            se[q].x += a.x * v[q];
            se[q].y += a.y * v[q];
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) kahan_add(so[q], co[q], po[q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = 4 * jq + q;
        if (j >= N) break;
        const int p = N + M + h + M * j;
        dst[2 * p] = (double)so[q].x;
        dst[2 * p + 1] = (double)so[q].y;
        dst[2 * P + 2 * p] = (double)se[q].x;
        dst[2 * P + 2 * p + 1] = (double)se[q].y;
      }
    } else if (item < nW + M) {
      const int h = item - nW;
      cpx<R> so = mk(R(0), R(0)), co = so, se = so;
      for (int t0 = 0; t0 < n; t0 += 8) {
        cpx<R> po = mk(R(0), R(0));
        for (int t = t0; t < min(n, t0 + 8); ++t) {
          const cpx<R> gv = s_g[t * M + h];
          po = po + gv;
          se = se + s_e[t] * conjc(gv);
        }
        kahan_add(so, co, po);
      }
      const int p = N + h;
      dst[2 * p] = (double)so.x;
      dst[2 * p + 1] = (double)so.y;
      dst[2 * P + 2 * p] = (double)se.x;
      dst[2 * P + 2 * p + 1] = (double)se.y;
    } else {
      const int j = item - nW - M;
      R so = R(0);                                      // a sum of integers: exact
      cpx<R> se = mk(R(0), R(0));
      for (int t = 0; t < n; ++t) {
        const R v = s_v[t * NJ + j];
        so += v;
        se.x += s_e[t].x * v;
        se.y += s_e[t].y * v;
      }
      dst[2 * j] = (double)so;
      dst[2 * j + 1] = 0.0;
      dst[2 * P + 2 * j] = (double)se.x;
      dst[2 * P + 2 * j + 1] = (double)se.y;
    }
  }
  if (threadIdx.x == 0) {
    double ex = 0, ey = 0;
    for (int t = 0; t < n; ++t) { ex += (double)s_e[t].x; ey += (double)s_e[t].y; }
    partialE[2 * blk] = ex;
    partialE[2 * blk + 1] = ey;
  }
}

template <typename R>
__global__ void __launch_bounds__(512)
rbm_force_partial_kernel(int N, int M, int hilb, const uint64_t* __restrict__ samples, int Ns,
                         const cpx<R>* __restrict__ g, const cpx<R>* __restrict__ eloc, int CH,
                         double* __restrict__ partial, double* __restrict__ partialE) {
  force_partial_block<R>(N, M, hilb, samples, Ns, g, eloc, CH, partial, partialE, blockIdx.x);
}

// Deterministic FP64 reduction of the per-chunk partials: one warp per
// parameter (index P carries ΣE), lanes stride over chunks, fixed-order
// shuffle tree.  sums[0..2P) = ΣO, [2P..4P) = ΣE conj(O), [4P..4P+2) = ΣE.
NQ_D void force_sums_warp(int P, int nblk, const double* __restrict__ partial, const double* __restrict__ partialE,
                          double* __restrict__ sums, int w, int lane) {
  double a = 0, b = 0, c = 0, d = 0;
  if (w < P) {
    for (int k = lane; k < nblk; k += 32) {
      const double* src = partial + (size_t)k * 4 * P;
      a += src[2 * w]; b += src[2 * w + 1];
      c += src[2 * P + 2 * w]; d += src[2 * P + 2 * w + 1];
    }
  } else {
    for (int k = lane; k < nblk; k += 32) { a += partialE[2 * k]; b += partialE[2 * k + 1]; }
  }
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, off);
    b += __shfl_xor_sync(0xffffffffu, b, off);
    c += __shfl_xor_sync(0xffffffffu, c, off);
    d += __shfl_xor_sync(0xffffffffu, d, off);
  }
  if (lane == 0) {
    if (w < P) {
      sums[2 * w] = a; sums[2 * w + 1] = b;
      sums[2 * P + 2 * w] = c; sums[2 * P + 2 * w + 1] = d;
    } else {
      sums[4 * P] = a; sums[4 * P + 1] = b;
    }
  }
}

__global__ void force_sums_kernel(int P, int nblk, const double* __restrict__ partial,
                                  const double* __restrict__ partialE, double* __restrict__ sums) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w > P) return;
  force_sums_warp(P, nblk, partial, partialE, sums, w, lane);
}

// <O> = ΣO/Ns, <E> = ΣE/Ns, F = ΣE conj(O)/Ns - <E> conj(<O>)
NQ_D void force_finalize_elem(int P, int Ns, const double* __restrict__ sums, double* meanO, double* force,
                              double* meanE, int p) {
  const double ex = sums[4 * P] / Ns, ey = sums[4 * P + 1] / Ns;
  if (p == 0) { meanE[0] = ex; meanE[1] = ey; }
  if (p >= P) return;
  const double ox = sums[2 * p] / Ns, oy = sums[2 * p + 1] / Ns;
  double fx = sums[2 * P + 2 * p] / Ns, fy = sums[2 * P + 2 * p + 1] / Ns;
  meanO[2 * p] = ox; meanO[2 * p + 1] = oy;
  fx -= ex * ox + ey * oy;
  fy -= ey * ox - ex * oy;
  force[2 * p] = fx; force[2 * p + 1] = fy;
}

__global__ void force_finalize_kernel(int P, int Ns, const double* __restrict__ sums, double* meanO,
                                      double* force, double* meanE) {
  force_finalize_elem(P, Ns, sums, meanO, force, meanE, blockIdx.x * blockDim.x + threadIdx.x);
}

// ---- grouped forms (many-problem step, FP32): the problem of a unit from the prefix arrays
__global__ void __launch_bounds__(256) force_partial_group_kernel(SrGroup g) {
  const int p = group_of(blockIdx.x, g.force_blk, g.np);
  const SrJob& j = g.jobs[p];
  force_partial_block<float>(j.N, j.M, j.hilb, j.samples, j.Ns, reinterpret_cast<const cpx<float>*>(j.g),
                             reinterpret_cast<const cpx<float>*>(j.eloc), j.force_CH, j.fb.partial,
                             j.fb.partialE, blockIdx.x - __ldg(g.force_blk + p));
}

__global__ void force_sums_group_kernel(SrGroup g) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= g.force_warps) return;
  const int p = group_of(w, g.force_warp, g.np);
  const SrJob& j = g.jobs[p];
  force_sums_warp(j.P, j.force_nblk, j.fb.partial, j.fb.partialE, j.fb.sums, w - __ldg(g.force_warp + p), lane);
}

__global__ void force_finalize_group_kernel(SrGroup g) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.pelems) return;
  const int p = group_of(e, g.pelem, g.np);
  const SrJob& j = g.jobs[p];
  force_finalize_elem(j.P, j.Ns, j.fb.sums, j.fb.meanO, j.fb.force, j.fb.meanE, e - __ldg(g.pelem + p));
}

// w -= lr Δw on the FP64 master (complex parameters, 2P doubles) and its FP32 copy
__global__ void update_group_kernel(SrGroup g, double lr) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.master_elems) return;
  const int p = group_of(e, g.master_elem, g.np);
  const SrJob& j = g.jobs[p];
  const int i = e - __ldg(g.master_elem + p);
  const double w = j.master[i] - lr * j.x[i];
  j.master[i] = w;
  j.p32[i] = (float)w;
}

template <typename R>
__global__ void rbm_grad_matrix_kernel(const uint64_t* samples, int n, int N, int M, int hilb,
                                       const cpx<R>* g, double* out) {
  const int P = N + M + M * N;
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)P * n) return;
  int s = (int)(idx / P), p = (int)(idx % P);
  uint64_t bits = samples[s];
  cpx<R> o;
  if (p < N) o = mk(site_value<R>(bits, p, hilb), R(0));
  else if (p < N + M) o = g[(size_t)(p - N) * n + s];
  else {
    int q = p - N - M, h = q % M, j = q / M;
    o = site_value<R>(bits, j, hilb) * g[(size_t)h * n + s];
  }
  out[2 * idx] = (double)o.x;
  out[2 * idx + 1] = (double)o.y;
}

__global__ void pack_kernel(const signed char* v, int nsites, long n, int hilb, uint64_t* bits) {
  long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  uint64_t b = 0;
  for (int j = 0; j < nsites; ++j) {
    int x = v[s * nsites + j];
    int bit = hilb == HILB_SPIN ? (x > 0) : (x != 0);
    b |= (uint64_t)bit << j;
  }
  bits[s] = b;
}

__global__ void unpack_kernel(const uint64_t* bits, int nsites, long n, int hilb, signed char* v) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= n * nsites) return;
  long s = idx / nsites;
  int j = (int)(idx % nsites);
  int bit = (int)((bits[s] >> j) & 1ull);
  v[idx] = (signed char)(hilb == HILB_SPIN ? 2 * bit - 1 : bit);
}

}  // namespace

// ------------------------------- launchers ---------------------------------

cudaError_t launch_rbm_params_from_master(const double* master, int N, int M, float* f32_out,
                                          cudaStream_t st) {
  long n = 2L * (N + M + (long)M * N);
  master_to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(master, n, f32_out);
  return cudaGetLastError();
}

cudaError_t launch_master_to_f32(const double* master, long n, float* f32_out, cudaStream_t st) {
  master_to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(master, n, f32_out);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_rbm_exchange_tables(const RbmDev<R>& net, int n_rows, const int2* pairs, cpx<R>* t0,
                                       cpx<R>* t1, cpx<R>* t2, cpx<R>* rW, R* rare, cudaStream_t st) {
  const int n = n_rows * net.M > n_rows ? n_rows * net.M : n_rows;
  rbm_exchange_tables_kernel<R><<<(n + 255) / 256, 256, 0, st>>>(net, n_rows, pairs, t0, t1, t2, rW, rare);
  return cudaGetLastError();
}
template cudaError_t launch_rbm_exchange_tables<float>(const RbmDev<float>&, int, const int2*, cpx<float>*,
                                                       cpx<float>*, cpx<float>*, cpx<float>*, float*, cudaStream_t);

template <typename R>
cudaError_t launch_rbm_tables(const RbmDev<R>& net, cpx<R>* t0, cpx<R>* t1, cpx<R>* t2,
                              cudaStream_t st) {
  int n = net.N * net.M;
  rbm_tables_kernel<R><<<(n + 127) / 128, 128, 0, st>>>(net, t0, t1, t2);
  return cudaGetLastError();
}

static int eval_threads(int M, size_t csize, int Tmax = 128) {
  const size_t M8 = (size_t)(M + 7) & ~(size_t)7;
  int T = Tmax;
  while (T > 32 && M8 * T * csize > 96 * 1024) T /= 2;
  return T;
}

static size_t eval_smem(int N, int M, int T, bool has_op, size_t csize) {
  const size_t M8 = (size_t)(M + 7) & ~(size_t)7;
  return (M8 * N + M8 + N + M8 * T + (has_op ? 2 * (size_t)N * M8 : 0)) * csize;
}

// Threads per block of the single-problem estimator: one thread per sample,
// and the per-thread slices of g in shared memory bound the blocks per SM, so
// a fixed block size can leave a short second wave (81920 samples at 256
// threads: 320 blocks for 304 slots).  The block size (a multiple of 32 up to
// kEvalMaxThreads) with the fewest waves wins, then the one with the most
// resident threads per SM.  Cached per (N, M, Ns, operator, activation, precision).
template <typename R, typename K>
static int eval_block_threads(K kern, int N, int M, int Ns, bool has_op, int act) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int, int>, int> cache;
  const auto key = std::make_tuple(N, M, Ns, has_op ? 1 : 0, act, (int)sizeof(R));
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 0;
  int best = eval_threads(M, sizeof(cpx<R>), 256);
  long best_waves = -1;
  int best_res = 0;
  for (int T = 64; sms > 0 && T <= kEvalMaxThreads<R>; T += 32) {
    const size_t smem = eval_smem(N, M, T, has_op, sizeof(cpx<R>));
    if (smem > 227 * 1024) break;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      break;
    }
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, T, smem) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (bps < 1) continue;
    const long blocks = (Ns + T - 1) / T, slots = (long)sms * bps;
    const long waves = (blocks + slots - 1) / slots;
    const int res = bps * T;
    if (best_waves < 0 || waves < best_waves || (waves == best_waves && res > best_res)) {
      best_waves = waves;
      best_res = res;
      best = T;
    }
  }
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = best;
  return best;
}

template <typename R>
cudaError_t launch_rbm_eval(const RbmDev<R>& net, const uint64_t* samples, int Ns, const DevOp* op,
                            cpx<R>* logpsi, cpx<R>* g, cpx<R>* eloc, cudaStream_t st, int theta_in_g) {
  const int has_op = op != nullptr && eloc != nullptr;
  const int T = net.act == ACT_LOGCOSH
                    ? eval_block_threads<R>(rbm_eval_kernel<R, ACT_LOGCOSH>, net.N, net.M, Ns, has_op, net.act)
                    : eval_block_threads<R>(rbm_eval_kernel<R, ACT_SOFTPLUS>, net.N, net.M, Ns, has_op, net.act);
  const size_t smem = eval_smem(net.N, net.M, T, has_op, sizeof(cpx<R>));
  DevOp dop;
  if (has_op) dop = *op;
  const int blocks = (Ns + T - 1) / T;
  if (net.act == ACT_LOGCOSH) {
    auto kern = rbm_eval_kernel<R, ACT_LOGCOSH>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    kern<<<blocks, T, smem, st>>>(net, samples, Ns, dop, has_op, logpsi, g, eloc, theta_in_g);
  } else {
    auto kern = rbm_eval_kernel<R, ACT_SOFTPLUS>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    kern<<<blocks, T, smem, st>>>(net, samples, Ns, dop, has_op, logpsi, g, eloc, theta_in_g);
  }
  return cudaGetLastError();
}

int rbm_eval_threads(int M_max) { return eval_threads(M_max, sizeof(cpx<float>)); }

template <typename R>
cudaError_t launch_rbm_eval_batch(const EvalJob<R>* jobs, const int* blk_start, int np, int total_blocks,
                                  int M_max, int N_max, int act, int T, cudaStream_t st) {
  const size_t M8 = (size_t)(M_max + 7) & ~(size_t)7;
  const size_t smem = (M8 * N_max + M8 + N_max + M8 * T + 2 * (size_t)N_max * M8) * sizeof(cpx<R>);
  if (act == ACT_LOGCOSH) {
    auto kern = rbm_eval_batch_kernel<R, ACT_LOGCOSH>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    kern<<<total_blocks, T, smem, st>>>(jobs, blk_start, np);
  } else {
    auto kern = rbm_eval_batch_kernel<R, ACT_SOFTPLUS>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    kern<<<total_blocks, T, smem, st>>>(jobs, blk_start, np);
  }
  return cudaGetLastError();
}
template cudaError_t launch_rbm_eval_batch<float>(const EvalJob<float>*, const int*, int, int, int, int, int, int,
                                                  cudaStream_t);

static size_t force_smem(int N, int M, int CH, int csize) {
  const int NJ = (N + 3) & ~3;
  return (size_t)(M + 1) * CH * csize + (size_t)NJ * CH * (csize / 2);
}

static int force_chunk(int N, int M, int csize) {
  int CH = 256;
  while (CH > 32 && force_smem(N, M, CH, csize) > 64 * 1024) CH /= 2;
  return CH;
}

// Geometry of the force partial sums: one thread per work item (M ceil(N/4)
// blocks of W, M of b, N of a) in one round, and the samples per block (CH, a
// multiple of 8) that put every block in one wave with the most resident
// threads per SM, counted up to 1024 (32 warps hide the latency), then the
// largest CH (fewer partials to write and reduce).  The grouped many-problem
// force uses the same CH per problem.  Cached per (N, M, Ns, precision).
struct ForceGeom { int CH, T; };
template <typename R>
static ForceGeom force_geom(int N, int M, int Ns) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, ForceGeom> cache;
  const auto key = std::make_tuple(N, M, Ns, (int)sizeof(R));
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const int csize = (int)sizeof(cpx<R>);
  const int items = M * (((N + 3) & ~3) / 4) + M + N;
  ForceGeom best{force_chunk(N, M, csize), 256};
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 0;
  const int T = std::min(512, std::max(64, (items + 31) & ~31));
  long best_waves = -1;
  int best_res = 0;
  auto kern = rbm_force_partial_kernel<R>;
  for (int CH = 32; sms > 0 && CH <= 256; CH += 8) {
    const size_t smem = force_smem(N, M, CH, csize);
    if (smem > 227 * 1024) break;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      break;
    }
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, T, smem) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (bps < 1) continue;
    const long blocks = (Ns + CH - 1) / CH, slots = (long)sms * bps;
    const long waves = (blocks + slots - 1) / slots;
    const int res = std::min(bps * T, 1024);
    if (best_waves < 0 || waves < best_waves || (waves == best_waves && res >= best_res)) {
      best_waves = waves;
      best_res = res;
      best = ForceGeom{CH, T};
    }
  }
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = best;
  return best;
}

int rbm_force_nblocks(int Ns, int N, int M, int csize) {
  const int CH = csize == (int)sizeof(cpx<float>) ? force_geom<float>(N, M, Ns).CH : force_geom<double>(N, M, Ns).CH;
  return (Ns + CH - 1) / CH;
}

template <typename R>
cudaError_t launch_rbm_force(const RbmDev<R>& net, const uint64_t* samples, int Ns, const cpx<R>* g,
                             const cpx<R>* eloc, const ForceBufs& fb, cudaStream_t st) {
  const ForceGeom fg = force_geom<R>(net.N, net.M, Ns);
  const int CH = fg.CH;
  const int nblk = (Ns + CH - 1) / CH;
  const size_t smem = force_smem(net.N, net.M, CH, (int)sizeof(cpx<R>));
  auto kern = rbm_force_partial_kernel<R>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<nblk, fg.T, smem, st>>>(net.N, net.M, net.hilb, samples, Ns, g, eloc, CH, fb.partial,
                                 fb.partialE);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int P = net.N + net.M + net.M * net.N;
  force_sums_kernel<<<(32 * (P + 1) + 255) / 256, 256, 0, st>>>(P, nblk, fb.partial, fb.partialE, fb.sums);
  force_finalize_kernel<<<(P + 255) / 256, 256, 0, st>>>(P, Ns, fb.sums, fb.meanO, fb.force, fb.meanE);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_rbm_grad_matrix(const uint64_t* samples, int n, int N, int M, int hilb,
                                   const cpx<R>* g, double* out, cudaStream_t st) {
  long tot = (long)(N + M + M * N) * n;
  rbm_grad_matrix_kernel<R><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(samples, n, N, M, hilb, g, out);
  return cudaGetLastError();
}

cudaError_t launch_pack_int8(const signed char* v, int nsites, long n, int hilb, uint64_t* bits,
                             cudaStream_t st) {
  pack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(v, nsites, n, hilb, bits);
  return cudaGetLastError();
}

cudaError_t launch_unpack_int8(const uint64_t* bits, int nsites, long n, int hilb, signed char* v,
                               cudaStream_t st) {
  long tot = n * nsites;
  unpack_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(bits, nsites, n, hilb, v);
  return cudaGetLastError();
}

// explicit instantiations
template cudaError_t launch_rbm_tables<float>(const RbmDev<float>&, cpx<float>*, cpx<float>*, cpx<float>*, cudaStream_t);
template cudaError_t launch_rbm_tables<double>(const RbmDev<double>&, cpx<double>*, cpx<double>*, cpx<double>*, cudaStream_t);
template cudaError_t launch_rbm_eval<float>(const RbmDev<float>&, const uint64_t*, int, const DevOp*, cpx<float>*, cpx<float>*, cpx<float>*, cudaStream_t, int);
template cudaError_t launch_rbm_eval<double>(const RbmDev<double>&, const uint64_t*, int, const DevOp*, cpx<double>*, cpx<double>*, cpx<double>*, cudaStream_t, int);
template cudaError_t launch_rbm_force<float>(const RbmDev<float>&, const uint64_t*, int, const cpx<float>*, const cpx<float>*, const ForceBufs&, cudaStream_t);
template cudaError_t launch_rbm_force<double>(const RbmDev<double>&, const uint64_t*, int, const cpx<double>*, const cpx<double>*, const ForceBufs&, cudaStream_t);
template cudaError_t launch_rbm_grad_matrix<float>(const uint64_t*, int, int, int, int, const cpx<float>*, double*, cudaStream_t);
template cudaError_t launch_rbm_grad_matrix<double>(const uint64_t*, int, int, int, int, const cpx<double>*, double*, cudaStream_t);

cudaError_t launch_force_group(const SrGroup& g, cudaStream_t st) {
  if (g.force_smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(force_partial_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)g.force_smem);
    if (e != cudaSuccess) return e;
  }
  force_partial_group_kernel<<<g.force_blocks, 256, g.force_smem, st>>>(g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  force_sums_group_kernel<<<(g.force_warps + 7) / 8, 256, 0, st>>>(g);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  force_finalize_group_kernel<<<(g.pelems + 255) / 256, 256, 0, st>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_update_group(const SrGroup& g, double lr, cudaStream_t st) {
  update_group_kernel<<<(g.master_elems + 255) / 256, 256, 0, st>>>(g, lr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  tables_group_kernel<<<(g.tab_elems + 127) / 128, 128, 0, st>>>(g);
  return cudaGetLastError();
}

// the grouped force uses the single-problem chunking, so a handle's partial
// buffers (sized by rbm_force_nblocks) fit it and both give the same F
int rbm_force_chunk(int N, int M, int Ns) { return force_geom<float>(N, M, Ns).CH; }
size_t rbm_force_smem(int N, int M, int Ns) {
  return force_smem(N, M, rbm_force_chunk(N, M, Ns), (int)sizeof(cpx<float>));
}
