// Feed-forward ket networks: PureStateAnsatz(Chain(Dense..., sum_autobatch |
// WSum)) (reference: src/Networks/Chains/Chain.jl:24-90,
// Layers/Dense.jl:24-104, Layers/WeightedSum.jl, Layers/sum.jl,
// ClosedSystems/PureChainWrapper.jl).
//
// A chain is a list of Dense layers θ_l = W_l x_l + b_l, x_{l+1} = f_l(θ_l)
// (x_1 = σ) closed by sum_autobatch (logψ = Σ_i x_i) or WSum (logψ = Σ_i c_i x_i).
// Parameters follow the functor order: per Dense layer W (out x in,
// column-major) then b, then the WSum weights.  ∇logψ is the holomorphic
// derivative of Dense.jl:90-104 (∇W = δθ xᵀ, ∇b = δθ, δ_in = Wᵀ δθ with
// δθ = δ f'(θ), no conjugation) and WeightedSum.jl (∇c = x, δ = c).
//
// Work layout: one thread per sample (estimator, gradients) or per chain
// (sampler).  Per-thread slices of shared memory hold the pre-activations of
// every Dense layer (Σ out) and three vectors of the widest layer; a
// proposal or a connection changes only θ_1 (θ_1' = θ_1 + Σ_q W_1[:, s_q] dv_q),
// so the forward pass restarts from θ_1'.
//
// Density-matrix chains run the same kernels on the 2N doubled sites (σ, η):
// DenseSplit (Layers/DenseSplit.jl) is the Dense layer W = [Wr Wc], and
// PositiveDefR (Layers/PositiveDefR.jl) the Dense layer W = [Wr + i Wi,
// Wr − i Wi] written by chain_pdr_params_kernel, whose gradient entries
// chain_backprop takes with respect to (Wr, Wi).
#include "nq_kernels.cuh"

namespace {

template <typename R>
NQ_D cpx<R> chain_act(int act, cpx<R> x) {
  if (act == ACT_IDENTITY) return x;
  return act == ACT_LOGCOSH ? act_f<ACT_LOGCOSH>(x) : act_f<ACT_SOFTPLUS>(x);
}
template <typename R>
NQ_D cpx<R> chain_dact(int act, cpx<R> x) {
  if (act == ACT_IDENTITY) return mk(R(1), R(0));
  return act == ACT_LOGCOSH ? act_df<ACT_LOGCOSH>(x) : act_df<ACT_SOFTPLUS>(x);
}

// forward from the first layer's pre-activations t0 (stride T); the later
// Dense layers' pre-activations are stored at th (if given), ping-pong in xa/xb
template <typename R>
NQ_D cpx<R> chain_forward_from0(const ChainDev<R>& c, const cpx<R>* t0, cpx<R>* th, cpx<R>* xa, cpx<R>* xb,
                                int T) {
  const ChainLayerDev& L0 = c.L[0];
  for (int o = 0; o < L0.out; ++o) xa[(size_t)o * T] = chain_act<R>(L0.act, t0[(size_t)o * T]);
  cpx<R>* x = xa;
  cpx<R>* y = xb;
  int thoff = L0.out;
  for (int l = 1; l < c.n_layers; ++l) {
    const ChainLayerDev& Ly = c.L[l];
    if (Ly.kind == LAYER_SUM) {
      cpx<R> s = mk(R(0), R(0));
      for (int i = 0; i < Ly.in; ++i) s = s + x[(size_t)i * T];
      return s;
    }
    if (Ly.kind == LAYER_WSUM) {
      cpx<R> s = mk(R(0), R(0));
      for (int i = 0; i < Ly.in; ++i) s = s + c.p[Ly.w_off + i] * x[(size_t)i * T];
      return s;
    }
    for (int o = 0; o < Ly.out; ++o) {
      cpx<R> t = c.p[Ly.b_off + o];
      for (int i = 0; i < Ly.in; ++i) t = t + c.p[Ly.w_off + o + Ly.out * i] * x[(size_t)i * T];
      if (th) th[(size_t)(thoff + o) * T] = t;
      y[(size_t)o * T] = chain_act<R>(Ly.act, t);
    }
    thoff += Ly.out;
    cpx<R>* z = x; x = y; y = z;
  }
  return mk(R(0), R(0));        // unreachable: the last layer is a sum
}

// θ_1 of configuration `bits` into t0 (stride T)
template <typename R>
NQ_D void chain_theta0(const ChainDev<R>& c, uint64_t bits, cpx<R>* t0, int T) {
  const ChainLayerDev& L0 = c.L[0];
  for (int o = 0; o < L0.out; ++o) {
    cpx<R> t = c.p[L0.b_off + o];
    for (int j = 0; j < c.N; ++j) {
      const R v = site_value<R>(bits, j, c.hilb);
      const cpx<R> w = c.p[L0.w_off + o + L0.out * j];
      t.x += w.x * v;
      t.y += w.y * v;
    }
    t0[(size_t)o * T] = t;
  }
}

// ∂logψ/∂p_k for all parameters at the configuration whose pre-activations
// are stored in th (Σ out, stride T); x/d/e are scratch vectors of the widest
// layer.  out(k, value) receives every entry once.
template <typename R, typename Out>
NQ_D void chain_backprop(const ChainDev<R>& c, uint64_t bits, const cpx<R>* th, cpx<R>* x, cpx<R>* d, cpx<R>* e,
                         int T, Out out) {
  // offsets of the stored pre-activations per Dense layer
  int thoff[8];
  int o = 0;
  for (int l = 0; l < c.n_layers; ++l) {
    thoff[l] = o;
    if (c.L[l].kind == LAYER_DENSE) o += c.L[l].out;
  }
  const int last = c.n_layers - 1;
  const ChainLayerDev& Ls = c.L[last];
  // input of the closing layer: f(θ) of the last Dense layer
  const ChainLayerDev& Lp = c.L[last - 1];
  for (int i = 0; i < Ls.in; ++i) x[(size_t)i * T] = chain_act<R>(Lp.act, th[(size_t)(thoff[last - 1] + i) * T]);
  if (Ls.kind == LAYER_WSUM) {
    for (int i = 0; i < Ls.in; ++i) {
      out(Ls.w_off + i, x[(size_t)i * T]);
      d[(size_t)i * T] = c.p[Ls.w_off + i];
    }
  } else {
    for (int i = 0; i < Ls.in; ++i) d[(size_t)i * T] = mk(R(1), R(0));
  }
  for (int l = last - 1; l >= 0; --l) {
    const ChainLayerDev& Ly = c.L[l];
    // δθ = δ f'(θ) in place
    for (int q = 0; q < Ly.out; ++q)
      d[(size_t)q * T] = d[(size_t)q * T] * chain_dact<R>(Ly.act, th[(size_t)(thoff[l] + q) * T]);
    for (int q = 0; q < Ly.out; ++q) out(Ly.b_off + q, d[(size_t)q * T]);
    // inputs of this layer
    if (l > 0)
      for (int i = 0; i < Ly.in; ++i)
        x[(size_t)i * T] = chain_act<R>(c.L[l - 1].act, th[(size_t)(thoff[l - 1] + i) * T]);
    if (l == 0 && c.pdr) {
      // PositiveDefRBatched.jl backprop: ∇Wr = δθ (σ + η)ᵀ, ∇Wi = i δθ (σ − η)ᵀ
      const int n = Ly.in / 2;
      for (int i = 0; i < n; ++i) {
        const R sr = site_value<R>(bits, i, c.hilb), sc = site_value<R>(bits, n + i, c.hilb);
        for (int q = 0; q < Ly.out; ++q) {
          const cpx<R> dq = d[(size_t)q * T];
          out(Ly.w_off + q + Ly.out * i, mk(dq.x * (sr + sc), dq.y * (sr + sc)));
          out(Ly.w_off + q + Ly.out * (n + i), mk(-dq.y * (sr - sc), dq.x * (sr - sc)));
        }
      }
      break;
    }
    for (int i = 0; i < Ly.in; ++i) {
      const cpx<R> xi = l > 0 ? x[(size_t)i * T] : mk(site_value<R>(bits, i, c.hilb), R(0));
      cpx<R> back = mk(R(0), R(0));
      for (int q = 0; q < Ly.out; ++q) {
        const cpx<R> dq = d[(size_t)q * T];
        out(Ly.w_off + q + Ly.out * i, dq * xi);
        if (l > 0) back = back + dq * c.p[Ly.w_off + q + Ly.out * i];
      }
      if (l > 0) e[(size_t)i * T] = back;
    }
    if (l > 0)
      for (int i = 0; i < Ly.in; ++i) d[(size_t)i * T] = e[(size_t)i * T];
  }
}

// ---------------------------------------------------------------------------
// Estimator and gradients: logψ, E_loc (with an operator) and O written to
// the interleaved rows of X (uncentred FP32) and/or Oout (P x n complex FP64).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128)
chain_eval_kernel(ChainDev<R> c, const uint64_t* __restrict__ samples, int n, DevOp op, int has_op,
                  cpx<R>* __restrict__ logpsi, cpx<R>* __restrict__ eloc, float* X, int ldx, double* Oout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = blockDim.x;
  cpx<R>* th = reinterpret_cast<cpx<R>*>(smem_raw) + threadIdx.x;        // [n_theta][T]
  cpx<R>* xa = reinterpret_cast<cpx<R>*>(smem_raw) + (size_t)c.n_theta * T + threadIdx.x;
  cpx<R>* xb = xa + (size_t)c.max_w * T;
  cpx<R>* xc = xb + (size_t)c.max_w * T;
  const int s = blockIdx.x * T + threadIdx.x;
  if (s >= n) return;
  const uint64_t bits = samples[s];
  chain_theta0<R>(c, bits, th, T);
  const cpx<R> lp = chain_forward_from0<R>(c, th, th, xa, xb, T);
  if (logpsi) logpsi[s] = lp;
  if (has_op) {
    const ChainLayerDev& L0 = c.L[0];
    cpx<R> acc = mk(R(0), R(0));
    for (int o = 0; o < op.n_ops; ++o) {
      const int ns_o = __ldg(op.op_n_sites + o);
      int r = 0;
      for (int dd = 0; dd < ns_o; ++dd) r |= (int)((bits >> __ldg(op.op_sites + 8 * o + dd)) & 1ull) << dd;
      const int row = __ldg(op.op_row_offset + o) + r;
      const int c0 = __ldg(op.row_conn_offset + row), c1 = __ldg(op.row_conn_offset + row + 1);
      for (int cc = c0; cc < c1; ++cc) {
        const double mre = __ldg(op.conn_mel + 2 * cc), mim = __ldg(op.conn_mel + 2 * cc + 1);
        if (mre == 0.0 && mim == 0.0) continue;
        const int nch = __ldg(op.conn_n_changes + cc);
        if (nch == 0) {
          acc.x += (R)mre;
          acc.y += (R)mim;
          continue;
        }
        for (int q = 0; q < L0.out; ++q) xc[(size_t)q * T] = th[(size_t)q * T];
        for (int k = 0; k < nch; ++k) {
          const int site = __ldg(op.conn_change_site + 8 * cc + k);
          const R dv = (R)__ldg(op.conn_change_value + 8 * cc + k) - site_value<R>(bits, site, c.hilb);
          for (int q = 0; q < L0.out; ++q) {
            const cpx<R> w = c.p[L0.w_off + q + L0.out * site];
            xc[(size_t)q * T].x += w.x * dv;
            xc[(size_t)q * T].y += w.y * dv;
          }
        }
        const cpx<R> lq = chain_forward_from0<R>(c, xc, nullptr, xa, xb, T);
        acc = acc + mk((R)mre, (R)mim) * cexpc(lq - lp);
      }
    }
    eloc[s] = acc;
  }
  if (X || Oout) {
    chain_backprop<R>(c, bits, th, xa, xb, xc, T, [&](int k, cpx<R> v) {
      if (X) {
        X[(size_t)(2 * k) * ldx + s] = (float)v.x;
        X[(size_t)(2 * k + 1) * ldx + s] = (float)v.y;
      }
      if (Oout) {
        Oout[2 * ((size_t)k + (size_t)c.P * s)] = (double)v.x;
        Oout[2 * ((size_t)k + (size_t)c.P * s) + 1] = (double)v.y;
      }
    });
  }
}

// F_k = (1/Ns) Σ_s E_s conj(O_ks) - Ē conj(<O_k>) (BatchedValSampler.jl:97-115
// with the centring of BaseIterativeSampler.jl:19-26), one warp per parameter,
// from the uncentred FP32 rows of X; Ē = stats[0] + i stats[1].
template <typename R>
__global__ void chain_force_kernel(const float* __restrict__ X, int ldx, int P, int ns, const cpx<R>* __restrict__ E,
                                   const double* __restrict__ stats, double* __restrict__ force) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= P) return;
  const float* xr = X + (size_t)(2 * k) * ldx;
  const float* xi = X + (size_t)(2 * k + 1) * ldx;
  double ar = 0, ai = 0, sr = 0, si = 0;
  for (int s = lane; s < ns; s += 32) {
    const double o_r = xr[s], o_i = xi[s];
    const double e_r = (double)E[s].x, e_i = (double)E[s].y;
    ar += e_r * o_r + e_i * o_i;          // E conj(O)
    ai += e_i * o_r - e_r * o_i;
    sr += o_r;
    si += o_i;
  }
  for (int off = 16; off > 0; off >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, off);
    ai += __shfl_xor_sync(0xffffffffu, ai, off);
    sr += __shfl_xor_sync(0xffffffffu, sr, off);
    si += __shfl_xor_sync(0xffffffffu, si, off);
  }
  if (lane == 0) {
    const double mr = sr / ns, mi = si / ns, er = stats[0], ei = stats[1];
    force[2 * k] = ar / ns - (er * mr + ei * mi);
    force[2 * k + 1] = ai / ns - (ei * mr - er * mi);
  }
}

// ---------------------------------------------------------------------------
// Density-matrix chains (MixedStateAnsatz on the doubled sites): the
// gradient of the local Liouvillian, AccumulatorObsGrad.jl:62-113 --
// ∇L_loc(σ) = Σ_c w_c O(σ'_c), w_c = mel_c ρ(σ'_c)/ρ(σ), over every non-zero
// connection including those without changes, with no -O(σ) term.  One
// thread per sample writes G[k n + s] = conj(∇L_loc,k(σ_s)) (FP32 complex,
// accumulated over the connections); the force is reduced from it below.
// Each connection restarts the forward pass from θ_1' = θ_1 + Σ_q W_1[:, s_q] dv_q
// with its pre-activations kept for the backward pass at σ'.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128)
chain_liouv_grad_kernel(ChainDev<R> c, const uint64_t* __restrict__ samples, int n, DevOp op,
                        float2* __restrict__ G) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = blockDim.x;
  cpx<R>* th = reinterpret_cast<cpx<R>*>(smem_raw) + threadIdx.x;          // [n_theta][T] at σ
  cpx<R>* th2 = th + (size_t)c.n_theta * T;                                 // [n_theta][T] at σ'
  cpx<R>* xa = th2 + (size_t)c.n_theta * T;
  cpx<R>* xb = xa + (size_t)c.max_w * T;
  cpx<R>* xc = xb + (size_t)c.max_w * T;
  const int s = blockIdx.x * T + threadIdx.x;
  if (s >= n) return;
  const uint64_t bits = samples[s];
  chain_theta0<R>(c, bits, th, T);
  const cpx<R> lp = chain_forward_from0<R>(c, th, th, xa, xb, T);
  for (int k = 0; k < c.P; ++k) G[(size_t)k * n + s] = make_float2(0.f, 0.f);
  const ChainLayerDev& L0 = c.L[0];
  for (int o = 0; o < op.n_ops; ++o) {
    const int ns_o = __ldg(op.op_n_sites + o);
    int r = 0;
    for (int dd = 0; dd < ns_o; ++dd) r |= (int)((bits >> __ldg(op.op_sites + 8 * o + dd)) & 1ull) << dd;
    const int row = __ldg(op.op_row_offset + o) + r;
    const int c0 = __ldg(op.row_conn_offset + row), c1 = __ldg(op.row_conn_offset + row + 1);
    for (int cc = c0; cc < c1; ++cc) {
      const double mre = __ldg(op.conn_mel + 2 * cc), mim = __ldg(op.conn_mel + 2 * cc + 1);
      if (mre == 0.0 && mim == 0.0) continue;
      const int nch = __ldg(op.conn_n_changes + cc);
      for (int q = 0; q < L0.out; ++q) th2[(size_t)q * T] = th[(size_t)q * T];
      uint64_t nb = bits;
      for (int k = 0; k < nch; ++k) {
        const int site = __ldg(op.conn_change_site + 8 * cc + k);
        const R nv = (R)__ldg(op.conn_change_value + 8 * cc + k);
        const R dv = nv - site_value<R>(bits, site, c.hilb);
        for (int q = 0; q < L0.out; ++q) {
          const cpx<R> w = c.p[L0.w_off + q + L0.out * site];
          th2[(size_t)q * T].x += w.x * dv;
          th2[(size_t)q * T].y += w.y * dv;
        }
        const uint64_t bit = (c.hilb == HILB_SPIN) ? (nv > 0 ? 1ull : 0ull) : (nv != R(0) ? 1ull : 0ull);
        nb = (nb & ~(1ull << site)) | (bit << site);
      }
      const cpx<R> lq = chain_forward_from0<R>(c, th2, th2, xa, xb, T);
      const cpx<R> w = mk((R)mre, (R)mim) * cexpc(lq - lp);
      const cpx<R> cw = conjc(w);
      chain_backprop<R>(c, nb, th2, xa, xb, xc, T, [&](int k, cpx<R> v) {
        const cpx<R> add = cw * conjc(v);
        float2* gk = G + (size_t)k * n + s;
        gk->x += (float)add.x;
        gk->y += (float)add.y;
      });
    }
  }
}

// F_k = conj(Σ_s L_s G_ks)/Ns - C <O_k> with C = mean |L_loc|² (stats[0])
// and <O> from the uncentred rows of X (BatchedGradSampler.jl:99-120); one
// warp per parameter, FP64 sums in a fixed order.
template <typename R>
__global__ void chain_liouv_force_kernel(const float* __restrict__ X, int ldx, int P, int ns,
                                         const cpx<R>* __restrict__ L, const float2* __restrict__ G,
                                         const double* __restrict__ stats, double* __restrict__ force) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= P) return;
  const float* xr = X + (size_t)(2 * k) * ldx;
  const float* xi = X + (size_t)(2 * k + 1) * ldx;
  const float2* gk = G + (size_t)k * ns;
  double ar = 0, ai = 0, sr = 0, si = 0;
  for (int s = lane; s < ns; s += 32) {
    const double lr = (double)L[s].x, li = (double)L[s].y, gr = gk[s].x, gi = gk[s].y;
    ar += lr * gr - li * gi;
    ai += lr * gi + li * gr;
    sr += xr[s];
    si += xi[s];
  }
  for (int off = 16; off > 0; off >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, off);
    ai += __shfl_xor_sync(0xffffffffu, ai, off);
    sr += __shfl_xor_sync(0xffffffffu, sr, off);
    si += __shfl_xor_sync(0xffffffffu, si, off);
  }
  if (lane == 0) {
    const double C = stats[0];
    force[2 * k] = ar / ns - C * sr / ns;
    force[2 * k + 1] = -ai / ns - C * si / ns;
  }
}

// ---------------------------------------------------------------------------
// Metropolis sampler (Metropolis.jl:101-167 with LocalRule, the Philox schema
// of the RBM sampler): one thread per chain keeps θ_1 and logψ; a proposal
// flipping site i evaluates the chain from θ_1 + W_1[:, i] dv.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128) chain_sampler_kernel(ChainDev<R> c, SamplerRun run) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = blockDim.x;
  cpx<R>* t0 = reinterpret_cast<cpx<R>*>(smem_raw) + threadIdx.x;        // [out_1][T]
  cpx<R>* tp = t0 + (size_t)c.L[0].out * T;                              // proposal θ_1
  cpx<R>* xa = tp + (size_t)c.L[0].out * T;
  cpx<R>* xb = xa + (size_t)c.max_w * T;
  const int chain_raw = blockIdx.x * T + threadIdx.x;
  const bool active = chain_raw < run.B;
  if (!active) return;
  const int chain = chain_raw;
  if (run.call_ptr) run.call = *run.call_ptr;
  const int N = c.N, out0 = c.L[0].out, w0 = c.L[0].w_off;
  uint64_t bits = 0;
  for (int q = 0; q < N; q += 4) {
    u32x4 w = philox4x32_10((uint32_t)(q >> 2), run.call, (uint32_t)chain, TAG_INIT, run.k0, run.k1);
    uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (q + k < N && (ws[k] >> 31)) bits |= 1ull << (q + k);
  }
  chain_theta0<R>(c, bits, t0, T);
  R lp = R(2) * chain_forward_from0<R>(c, t0, nullptr, xa, xb, T).x;   // log|ψ|^2
  const R dmag = c.hilb == HILB_SPIN ? R(2) : R(1);
  unsigned long long naccept = 0;
  uint32_t t = 0;
  const int nsweeps = run.burn + run.n_record;
  for (int sweep = 0; sweep < nsweeps; ++sweep) {
    for (int pass = 0; pass < run.passes; ++pass, ++t) {
      const u32x4 r = philox4x32_10(t, run.call, (uint32_t)chain, TAG_MH, run.k0, run.k1);
      const int i = (int)uniform_site(r.x, (uint32_t)N);
      const double u = (double)uniform24(r.y);
      const R dv = ((bits >> i) & 1ull) ? -dmag : dmag;
      for (int o = 0; o < out0; ++o) {
        const cpx<R> w = c.p[w0 + o + out0 * i];
        tp[(size_t)o * T] = mk(t0[(size_t)o * T].x + w.x * dv, t0[(size_t)o * T].y + w.y * dv);
      }
      const R lpn = R(2) * chain_forward_from0<R>(c, tp, nullptr, xa, xb, T).x;
      const bool acc = u < exp((double)(lpn - lp));
      if (acc) {
        for (int o = 0; o < out0; ++o) t0[(size_t)o * T] = tp[(size_t)o * T];
        lp = lpn;
        bits ^= 1ull << i;
        ++naccept;
      }
      if (run.accept_bits) run.accept_bits[(size_t)t * run.B + chain] = acc ? 1 : 0;
    }
    const int slot = sweep - run.burn;
    if (slot >= 0) run.samples[(size_t)slot * run.B + chain] = bits;
  }
  if (run.write_last_at_end) run.samples[chain] = bits;
  atomicAdd(run.accepted, naccept);
}

template <typename R>
int chain_threads(const ChainDev<R>& c, int extra_vecs) {
  int T = 128;
  while (T > 32 && (size_t)(c.n_theta + extra_vecs * c.max_w) * T * sizeof(cpx<R>) > 96 * 1024) T /= 2;
  return T;
}

template <typename K>
cudaError_t set_smem(K kern, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

// PositiveDefR's θ = Wr (σ + η) + i Wi (σ − η) + b (PositiveDefR.jl:11-12)
// is the Dense layer W_σ σ + W_η η + b with W_σ = Wr + i Wi, W_η = Wr − i Wi;
// the later layers are copied.  One thread per complex entry k < P.
template <typename T>
__global__ void chain_pdr_params_kernel(const double* __restrict__ master, int P, int nw, T* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P) return;
  double re = master[2 * k], im = master[2 * k + 1];
  if (k < 2 * nw) {
    const int j = k < nw ? k : k - nw;                     // the same (unit, site) of Wr and Wi
    const double ar = master[2 * j], ai = master[2 * j + 1];
    const double br = master[2 * (nw + j)], bi = master[2 * (nw + j) + 1];
    const double s = k < nw ? 1.0 : -1.0;                  // Wr ± i Wi
    re = ar - s * bi;
    im = ai + s * br;
  }
  out[2 * k] = (T)re;
  out[2 * k + 1] = (T)im;
}

}  // namespace

cudaError_t launch_chain_pdr_params(const double* master, int P, int n_out, int n_sites, float* p32, double* p64,
                                    cudaStream_t st) {
  const int nw = n_out * n_sites;
  if (P < 2 * nw + n_out || (p32 == nullptr) == (p64 == nullptr)) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)((P + 255) / 256);
  if (p32) chain_pdr_params_kernel<float><<<grid, 256, 0, st>>>(master, P, nw, p32);
  else chain_pdr_params_kernel<double><<<grid, 256, 0, st>>>(master, P, nw, p64);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_chain_eval(const ChainDev<R>& c, const uint64_t* samples, int n, const DevOp* op, cpx<R>* logpsi,
                              cpx<R>* eloc, float* X, int ldx, double* Oout, cudaStream_t st) {
  if (n < 1) return cudaSuccess;
  const int T = chain_threads(c, 3);
  const size_t smem = (size_t)(c.n_theta + 3 * c.max_w) * T * sizeof(cpx<R>);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = set_smem(chain_eval_kernel<R>, smem);
  if (e != cudaSuccess) return e;
  DevOp d = op ? *op : DevOp();
  chain_eval_kernel<R><<<(n + T - 1) / T, T, smem, st>>>(c, samples, n, d, op && eloc ? 1 : 0, logpsi, eloc, X,
                                                         ldx, Oout);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_chain_force(const float* X, int ldx, int P, int ns, const cpx<R>* E, const double* stats,
                               double* force, cudaStream_t st) {
  chain_force_kernel<R><<<(32 * P + 255) / 256, 256, 0, st>>>(X, ldx, P, ns, E, stats, force);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_chain_liouv_force(const ChainDev<R>& c, const uint64_t* samples, int n, const DevOp& op,
                                     const cpx<R>* L, const float* X, int ldx, const double* stats, float2* G,
                                     double* force, cudaStream_t st) {
  if (n < 1) return cudaSuccess;
  int T = 128;
  auto need = [&](int t) { return (size_t)(2 * c.n_theta + 3 * c.max_w) * t * sizeof(cpx<R>); };
  while (T > 32 && need(T) > 96 * 1024) T /= 2;
  const size_t smem = need(T);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = set_smem(chain_liouv_grad_kernel<R>, smem);
  if (e != cudaSuccess) return e;
  chain_liouv_grad_kernel<R><<<(n + T - 1) / T, T, smem, st>>>(c, samples, n, op, G);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  chain_liouv_force_kernel<R><<<(32 * c.P + 255) / 256, 256, 0, st>>>(X, ldx, c.P, n, L, G, stats, force);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_chain_sampler(const ChainDev<R>& c, const SamplerRun& run, cudaStream_t st) {
  if (c.N > 64 || c.n_layers < 2) return cudaErrorInvalidValue;
  const int T = chain_threads(c, 2) < 128 ? chain_threads(c, 2) : 128;
  const size_t smem = (size_t)(2 * c.L[0].out + 2 * c.max_w) * T * sizeof(cpx<R>);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = set_smem(chain_sampler_kernel<R>, smem);
  if (e != cudaSuccess) return e;
  chain_sampler_kernel<R><<<(run.B + T - 1) / T, T, smem, st>>>(c, run);
  return cudaGetLastError();
}

template cudaError_t launch_chain_eval<float>(const ChainDev<float>&, const uint64_t*, int, const DevOp*, cpx<float>*,
                                              cpx<float>*, float*, int, double*, cudaStream_t);
template cudaError_t launch_chain_eval<double>(const ChainDev<double>&, const uint64_t*, int, const DevOp*,
                                               cpx<double>*, cpx<double>*, float*, int, double*, cudaStream_t);
template cudaError_t launch_chain_force<float>(const float*, int, int, int, const cpx<float>*, const double*, double*,
                                               cudaStream_t);
template cudaError_t launch_chain_force<double>(const float*, int, int, int, const cpx<double>*, const double*,
                                                double*, cudaStream_t);
template cudaError_t launch_chain_sampler<float>(const ChainDev<float>&, const SamplerRun&, cudaStream_t);
template cudaError_t launch_chain_sampler<double>(const ChainDev<double>&, const SamplerRun&, cudaStream_t);
template cudaError_t launch_chain_liouv_force<float>(const ChainDev<float>&, const uint64_t*, int, const DevOp&,
                                                     const cpx<float>*, const float*, int, const double*, float2*,
                                                     double*, cudaStream_t);
template cudaError_t launch_chain_liouv_force<double>(const ChainDev<double>&, const uint64_t*, int, const DevOp&,
                                                      const cpx<double>*, const float*, int, const double*, float2*,
                                                      double*, cudaStream_t);
