// NDM (purified neural density matrix) path: effective-network construction,
// batched logρ / ∇logρ on doubled states (σ, η), the Liouvillian local
// estimator L_loc and the cost gradient accumulation.
//
// Reference: src/Networks/MixedDensityMatrix/NDM.jl:76-96 and 241-337,
// NDMBatched.jl:94-280 (network and gradient), AccumulatorObsGrad.jl:39-127
// and BatchedGradSampler.jl:77-123 (estimator and gradient).
//
// With σ the row and η the column configuration, the NDM is written as a
// generalised RBM over the 2N doubled sites v = (σ, η) with U = 4Mh + Ma
// hidden units u of weight ω_u:
//   logρ = Σ_i a_i v_i + Σ_u ω_u f(x_u),  x_u = b_u + Σ_i C[u, i] v_i
//   units [λσ (Mh), λη (Mh), π (Ma), μσ (Mh), μη (Mh)] with
//   ω = 1/2, 1/2, 1, i/2, -i/2;  a_i = b_la/2 ± i b_mu/2 (row/column).
// The first Ms = 2Mh + Ma units are the ones that enter |ρ|^2, so the
// Metropolis sampler of the RBM runs unchanged on them (λ units at weight
// 1/2 through RbmDev::n_half).
//
// RBMSplit (src/Networks/MixedDensityMatrix/RBMSplit.jl:36-50, 111-129),
// logρ = ar·σ + ac·η + Σ_h f(b_h + Wr_h·σ + Wc_h·η) with complex parameters,
// is the same form with Mh = 0, U = Ma = M units of weight 1, a = (ar, ac)
// and C = (Wr | Wc): its parameter vector (ar, ac, b, Wr, Wc) is exactly the
// RBM layout over the 2N doubled sites, so the effective network is a copy of
// it and O_k is the RBM's (v_i, f'(x_h), f'(x_h) v_i).
#include "ndm_kernels.cuh"

namespace {

template <typename R>
__global__ void ndm_effective_kernel(NdmDev<R> n, cpx<R>* C, cpx<R>* bu, cpx<R>* a, cpx<R>* Cs, cpx<R>* bs) {
  const int N = n.N, Mh = n.Mh, Ma = n.Ma, U = 4 * Mh + Ma, Ms = 2 * Mh + Ma, N2 = 2 * N;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < U * N2) {
    const int u = idx % U, i = idx / U;
    const bool row = i < N;
    const int j = row ? i : i - N;
    cpx<R> c = mk(R(0), R(0));
    if (u < Mh) { if (row) c.x = n.w_la[u + Mh * j]; }
    else if (u < 2 * Mh) { if (!row) c.x = n.w_la[(u - Mh) + Mh * j]; }
    else if (u < 2 * Mh + Ma) {
      const int q = u - 2 * Mh;
      c.x = R(0.5) * n.u_la[q + Ma * j];
      c.y = (row ? R(0.5) : R(-0.5)) * n.u_mu[q + Ma * j];
    } else if (u < 3 * Mh + Ma) { if (row) c.x = n.w_mu[(u - 2 * Mh - Ma) + Mh * j]; }
    else { if (!row) c.x = n.w_mu[(u - 3 * Mh - Ma) + Mh * j]; }
    C[u + (size_t)U * i] = c;
    if (u < Ms) Cs[u + (size_t)Ms * i] = c;
  }
  if (idx < U) {
    const int u = idx;
    cpx<R> b = mk(R(0), R(0));
    if (u < 2 * Mh) b.x = n.h_la[u % Mh];
    else if (u < 2 * Mh + Ma) b.x = n.d_la[u - 2 * Mh];
    else b.x = n.h_mu[(u - 2 * Mh - Ma) % Mh];
    bu[u] = b;
    if (u < Ms) bs[u] = b;
  }
  if (idx < N2) {
    const int j = idx < N ? idx : idx - N;
    a[idx] = mk(R(0.5) * n.b_la[j], (idx < N ? R(0.5) : R(-0.5)) * n.b_mu[j]);
  }
}

template <typename R> NQ_D cpx<R> unit_weight(int u, int Mh, int Ma) {
  if (u < 2 * Mh) return mk(R(0.5), R(0));
  if (u < 2 * Mh + Ma) return mk(R(1), R(0));
  if (u < 3 * Mh + Ma) return mk(R(0), R(0.5));
  return mk(R(0), R(-0.5));
}

// O_k at a doubled configuration with unit derivatives g (real parameter k of
// the reference order b_mu, h_mu, w_mu, u_mu, b_la, h_la, d_la, w_la, u_la).
template <typename R>
NQ_D cpx<R> ndm_O(int k, int N, int Mh, int Ma, const cpx<R>* g, int gstride, uint64_t bits, int hilb,
                  int split) {
  if (split) {
    // RBMSplit: parameters (a over the 2N doubled sites, b, W column-major M x 2N)
    const int N2 = 2 * N, M = Ma;
    if (k < N2) return mk(site_value<R>(bits, k, hilb), R(0));
    k -= N2;
    if (k < M) return g[(size_t)k * gstride];
    k -= M;
    return site_value<R>(bits, k / M, hilb) * g[(size_t)(k % M) * gstride];
  }
  const cpx<R> half_i = mk(R(0), R(0.5));
  // unit offsets: λσ 0, λη Mh, π 2Mh, μσ 2Mh+Ma, μη 3Mh+Ma
  const int oLs = 0, oLe = Mh, oPi = 2 * Mh, oMs = 2 * Mh + Ma, oMe = 3 * Mh + Ma;
#define G_(u) g[(size_t)(u) * gstride]
  int o = 0;
  if (k < o + N) { const int j = k - o; return half_i * mk(site_value<R>(bits, j, hilb) - site_value<R>(bits, N + j, hilb), R(0)); }
  o += N;
  if (k < o + Mh) { const int h = k - o; return half_i * (G_(oMs + h) - G_(oMe + h)); }
  o += Mh;
  if (k < o + Mh * N) {
    const int q = k - o, h = q % Mh, j = q / Mh;
    return half_i * (site_value<R>(bits, j, hilb) * G_(oMs + h) - site_value<R>(bits, N + j, hilb) * G_(oMe + h));
  }
  o += Mh * N;
  if (k < o + Ma * N) {
    const int q = k - o, a = q % Ma, j = q / Ma;
    return (site_value<R>(bits, j, hilb) - site_value<R>(bits, N + j, hilb)) * (half_i * G_(oPi + a));
  }
  o += Ma * N;
  if (k < o + N) { const int j = k - o; return mk(R(0.5) * (site_value<R>(bits, j, hilb) + site_value<R>(bits, N + j, hilb)), R(0)); }
  o += N;
  if (k < o + Mh) { const int h = k - o; return R(0.5) * (G_(oLs + h) + G_(oLe + h)); }
  o += Mh;
  if (k < o + Ma) { const int a = k - o; return G_(oPi + a); }
  o += Ma;
  if (k < o + Mh * N) {
    const int q = k - o, h = q % Mh, j = q / Mh;
    return R(0.5) * (site_value<R>(bits, j, hilb) * G_(oLs + h) + site_value<R>(bits, N + j, hilb) * G_(oLe + h));
  }
  o += Mh * N;
  {
    const int q = k - o, a = q % Ma, j = q / Ma;
    return (R(0.5) * (site_value<R>(bits, j, hilb) + site_value<R>(bits, N + j, hilb))) * G_(oPi + a);
  }
#undef G_
}

// O of trainable parameter k: the network's own, or for NDMSymm the sum of
// the bare parameters' O that the symmetric parameter k stands for
// (symmetrize_∇logψ_NDM!, NDMSymm.jl:76-87)
template <typename R>
NQ_D cpx<R> ndm_O_train(const NdmEff<R>& e, int k, const cpx<R>* g, int gstride, uint64_t bits, int hilb) {
  if (!e.sym_off) return ndm_O<R>(k, e.N, e.Mh, e.Ma, g, gstride, bits, hilb, e.split);
  cpx<R> o = mk(R(0), R(0));
  for (int q = e.sym_off[k]; q < e.sym_off[k + 1]; ++q)
    o = o + (R)e.sym_coef[q] * ndm_O<R>(e.sym_idx[q], e.N, e.Mh, e.Ma, g, gstride, bits, hilb, 0);
  return o;
}

// unit pre-activations x_u and derivatives g_u at configuration `bits`
// into per-thread slices of shared memory (stride T)
// (θ read from e.theta[u n + s] when the tensor-core θ of the n samples is given)
template <typename R, int ACT>
NQ_D cpx<R> ndm_units(const NdmEff<R>& e, uint64_t bits, int hilb, cpx<R>* x, cpx<R>* g, int T, int s = 0,
                      int n = 0) {
  const int U = e.U, N2 = e.N2;
  cpx<R> lp = mk(R(0), R(0));
  for (int i = 0; i < N2; ++i) lp = lp + site_value<R>(bits, i, hilb) * e.a[i];
  for (int u = 0; u < U; ++u) {
    cpx<R> t;
    if (e.theta) {
      t = e.theta[(size_t)u * n + s];
    } else {
      t = e.b[u];
      for (int i = 0; i < N2; ++i) {
        const R v = site_value<R>(bits, i, hilb);
        if (v != R(0)) { const cpx<R> c = e.C[u + (size_t)U * i]; t.x += c.x * v; t.y += c.y * v; }
      }
    }
    x[(size_t)u * T] = t;
    g[(size_t)u * T] = act_df<ACT>(t);
    lp = lp + unit_weight<R>(u, e.Mh, e.Ma) * act_f<ACT>(t);
  }
  return lp;
}

// ---------------------------------------------------------------------------
// Evaluation: logρ and O (P entries) per sample.  O is written either to the
// interleaved real rows of X (row 2k = Re O_k, 2k+1 = Im O_k, sample-major
// columns, uncentred) or to a P x n complex double matrix.
// ---------------------------------------------------------------------------
template <typename R, int ACT>
__global__ void __launch_bounds__(128)
ndm_eval_kernel(NdmEff<R> e, const uint64_t* __restrict__ samples, int n, int hilb, cpx<R>* logrho,
                float* X, int ldx, double* Oout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = blockDim.x, U = e.U;
  cpx<R>* sx = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* sg = sx + (size_t)U * T;
  const int s = blockIdx.x * T + threadIdx.x;
  if (s >= n) return;
  const uint64_t bits = samples[s];
  const cpx<R> lp = ndm_units<R, ACT>(e, bits, hilb, sx + threadIdx.x, sg + threadIdx.x, T, s, n);
  logrho[s] = lp;
  for (int k = 0; k < e.P; ++k) {
    const cpx<R> o = ndm_O_train<R>(e, k, sg + threadIdx.x, T, bits, hilb);
    if (X) {
      X[(size_t)(2 * k) * ldx + s] = (float)o.x;
      X[(size_t)(2 * k + 1) * ldx + s] = (float)o.y;
    }
    if (Oout) {
      Oout[2 * ((size_t)k + (size_t)e.P * s)] = (double)o.x;
      Oout[2 * ((size_t)k + (size_t)e.P * s) + 1] = (double)o.y;
    }
  }
}

// Δlogρ of a connection: Σ_i a_i Δv_i + Σ_u ω_u [f(x_u + Δx_u) - f(x_u)]
template <typename R, int ACT>
NQ_D cpx<R> ndm_delta(const NdmEff<R>& e, const DevOp& op, int c, uint64_t bits, int hilb, const cpx<R>* x,
                      int T, int nch) {
  const int U = e.U;
  cpx<R> d = mk(R(0), R(0));
  int site[8];
  R dv[8];
  for (int q = 0; q < nch; ++q) {
    site[q] = __ldg(op.conn_change_site + 8 * c + q);
    dv[q] = (R)__ldg(op.conn_change_value + 8 * c + q) - site_value<R>(bits, site[q], hilb);
    d = d + dv[q] * e.a[site[q]];
  }
  for (int u = 0; u < U; ++u) {
    cpx<R> dx = mk(R(0), R(0));
    for (int q = 0; q < nch; ++q) {
      const cpx<R> cc = e.C[u + (size_t)U * site[q]];
      dx.x += cc.x * dv[q];
      dx.y += cc.y * dv[q];
    }
    if (dx.x == R(0) && dx.y == R(0)) continue;
    const cpx<R> xu = x[(size_t)u * T];
    d = d + unit_weight<R>(u, e.Mh, e.Ma) * (act_f<ACT>(xu + dx) - act_f<ACT>(xu));
  }
  return d;
}

// ---------------------------------------------------------------------------
// Local Liouvillian L_loc(σ,η) = Σ_c mel_c ρ(σ'_c)/ρ(σ,η) over every
// non-zero connection, including those without changes
// (AccumulatorObsGrad.jl:62-75); the weights w_c are kept for the gradient.
// ---------------------------------------------------------------------------
template <typename R, int ACT>
__global__ void __launch_bounds__(128)
ndm_loc_kernel(NdmEff<R> e, DevOp op, const uint64_t* __restrict__ samples, int n, int hilb, int maxc,
               cpx<R>* __restrict__ L, cpx<R>* __restrict__ w, int* __restrict__ wconn,
               int* __restrict__ nconn) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = blockDim.x, U = e.U;
  cpx<R>* sx = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* sg = sx + (size_t)U * T;
  const int s = blockIdx.x * T + threadIdx.x;
  if (s >= n) return;
  const uint64_t bits = samples[s];
  ndm_units<R, ACT>(e, bits, hilb, sx + threadIdx.x, sg + threadIdx.x, T, s, n);
  cpx<R> acc = mk(R(0), R(0));
  int cnt = 0;
  for (int o = 0; o < op.n_ops; ++o) {
    const int ns_o = __ldg(op.op_n_sites + o);
    int r = 0;
    for (int d = 0; d < ns_o; ++d) r |= (int)((bits >> __ldg(op.op_sites + 8 * o + d)) & 1ull) << d;
    const int row = __ldg(op.op_row_offset + o) + r;
    const int c0 = __ldg(op.row_conn_offset + row), c1 = __ldg(op.row_conn_offset + row + 1);
    for (int c = c0; c < c1; ++c) {
      const double mre = __ldg(op.conn_mel + 2 * c), mim = __ldg(op.conn_mel + 2 * c + 1);
      if (mre == 0.0 && mim == 0.0) continue;
      const int nch = __ldg(op.conn_n_changes + c);
      const cpx<R> d = ndm_delta<R, ACT>(e, op, c, bits, hilb, sx + threadIdx.x, T, nch);
      const cpx<R> wc = mk((R)mre, (R)mim) * cexpc(d);
      acc = acc + wc;
      if (cnt < maxc) {
        w[(size_t)s * maxc + cnt] = wc;
        wconn[(size_t)s * maxc + cnt] = c;
      }
      ++cnt;
    }
  }
  L[s] = acc;
  nconn[s] = min(cnt, maxc);
}

// ---------------------------------------------------------------------------
// Diagonal observables (BatchedObsDMSampler.jl:90-105 with
// AccumulatorObsScalar.jl:52-137 over a doubled buffer): at the doubled
// configuration (σ, σ) of a physical sample, O_loc(σ) = Σ_c mel_c
// ρ(σ'_c, σ)/ρ(σ, σ), the connection's changes applied to the row sites
// (ApplyStateChanges.jl:18-21), which are the doubled sites 0..N-1.  Zero
// elements are skipped and elements without changes add mel (:90-107).
// ---------------------------------------------------------------------------
template <typename R, int ACT>
__global__ void __launch_bounds__(128)
ndm_diag_obs_kernel(NdmEff<R> e, DevOp op, const uint64_t* __restrict__ samples, int n, int hilb,
                    cpx<R>* __restrict__ logrho, cpx<R>* __restrict__ O) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = blockDim.x, U = e.U;
  cpx<R>* sx = reinterpret_cast<cpx<R>*>(smem_raw);
  cpx<R>* sg = sx + (size_t)U * T;
  const int s = blockIdx.x * T + threadIdx.x;
  if (s >= n) return;
  const uint64_t phys = samples[s];
  const uint64_t bits = phys | (phys << e.N);
  const cpx<R> lp = ndm_units<R, ACT>(e, bits, hilb, sx + threadIdx.x, sg + threadIdx.x, T);
  if (logrho) logrho[s] = lp;
  cpx<R> acc = mk(R(0), R(0));
  for (int o = 0; o < op.n_ops; ++o) {
    const int ns_o = __ldg(op.op_n_sites + o);
    int r = 0;
    for (int d = 0; d < ns_o; ++d) r |= (int)((phys >> __ldg(op.op_sites + 8 * o + d)) & 1ull) << d;
    const int row = __ldg(op.op_row_offset + o) + r;
    const int c0 = __ldg(op.row_conn_offset + row), c1 = __ldg(op.row_conn_offset + row + 1);
    for (int c = c0; c < c1; ++c) {
      const double mre = __ldg(op.conn_mel + 2 * c), mim = __ldg(op.conn_mel + 2 * c + 1);
      if (mre == 0.0 && mim == 0.0) continue;
      const int nch = __ldg(op.conn_n_changes + c);
      if (nch == 0) {
        acc.x += (R)mre;
        acc.y += (R)mim;
        continue;
      }
      const cpx<R> d = ndm_delta<R, ACT>(e, op, c, bits, hilb, sx + threadIdx.x, T, nch);
      acc = acc + mk((R)mre, (R)mim) * cexpc(d);
    }
  }
  O[s] = acc;
}

// N-site tables of the diagonal logρ(σ,σ) = b_la·σ + Σ_h f(h_la + w_la σ) +
// Σ_k f(d_la + u_la σ) (NDM.jl:76-96 at η = σ: the μ units cancel and the
// ancilla unit has no phase), in the sampler's convention log p =
// 2 Re aᵀσ + Σ_u c_u 2 Re f(θ_u) with every unit at c_u = 1/2:
// a = b_la / 2, units [λ (Mh), ancilla (Ma)].
template <typename R>
__global__ void ndm_diagonal_kernel(NdmDev<R> n, cpx<R>* __restrict__ a, cpx<R>* __restrict__ b,
                                    cpx<R>* __restrict__ W) {
  const int N = n.N, Mh = n.Mh, Ma = n.Ma, Md = Mh + Ma;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < Md * N) {
    const int u = idx % Md, j = idx / Md;
    W[idx] = mk(u < Mh ? n.w_la[u + Mh * j] : n.u_la[(u - Mh) + Ma * j], R(0));
  }
  if (idx < Md) b[idx] = mk(idx < Mh ? n.h_la[idx] : n.d_la[idx - Mh], R(0));
  if (idx < N) a[idx] = mk(R(0.5) * n.b_la[idx], R(0));
}

// RBMSplit effective network: C = Cs = (Wr | Wc), b = bs = b, a = (ar, ac),
// copied from the parameter vector p (complex, RBM layout over 2N sites)
template <typename R>
__global__ void split_effective_kernel(const cpx<R>* __restrict__ p, int N2, int M, cpx<R>* C, cpx<R>* bu,
                                       cpx<R>* a, cpx<R>* Cs, cpx<R>* bs) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < M * N2) {
    const cpx<R> w = p[N2 + M + idx];
    C[idx] = w;
    Cs[idx] = w;
  }
  if (idx < M) {
    bu[idx] = p[N2 + idx];
    bs[idx] = p[N2 + idx];
  }
  if (idx < N2) a[idx] = p[idx];
}

// RBMSplit diagonal: logρ(σ,σ) = (ar + ac)·σ + Σ_h f(b_h + (Wr + Wc)_h·σ), in
// the sampler's convention with every unit at weight 1/2 (log p = Re logρ):
// a = (ar + ac)/2, W = Wr + Wc
template <typename R>
__global__ void split_diagonal_kernel(const cpx<R>* __restrict__ p, int N, int M, cpx<R>* __restrict__ a,
                                      cpx<R>* __restrict__ b, cpx<R>* __restrict__ W) {
  const int N2 = 2 * N;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < M * N) {
    const int h = idx % M, j = idx / M;
    const cpx<R> wr = p[N2 + M + h + M * j], wc = p[N2 + M + h + M * (N + j)];
    W[idx] = mk(wr.x + wc.x, wr.y + wc.y);
  }
  if (idx < M) b[idx] = p[N2 + idx];
  if (idx < N) a[idx] = mk(R(0.5) * (p[idx].x + p[N + idx].x), R(0.5) * (p[idx].y + p[N + idx].y));
}

// NDMSymm bare parameters (set_bare_params!, NDMSymm.jl:89-133): b = the
// (already averaged) symmetric b; bare hidden unit j + f ns has bias h_f and
// weights w[j + f ns, perm_j[i]] = w_symm[f, i]; ancilla units alike.
template <typename R>
__global__ void ndm_symm_bare_kernel(const R* __restrict__ symm, int N, int ah, int aa, int ns,
                                     const int* __restrict__ perms, R* __restrict__ bare) {
  const NdmDev<R> sv = ndm_view<R>(symm, N, ah, aa);
  const int Mh = ah * ns, Ma = aa * ns;
  const NdmDev<R> bv = ndm_view<R>(bare, N, Mh, Ma);
  R* b_mu = const_cast<R*>(bv.b_mu); R* h_mu = const_cast<R*>(bv.h_mu); R* w_mu = const_cast<R*>(bv.w_mu);
  R* u_mu = const_cast<R*>(bv.u_mu); R* b_la = const_cast<R*>(bv.b_la); R* h_la = const_cast<R*>(bv.h_la);
  R* d_la = const_cast<R*>(bv.d_la); R* w_la = const_cast<R*>(bv.w_la); R* u_la = const_cast<R*>(bv.u_la);
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  for (int i = tid; i < N; i += nth) {
    b_mu[i] = sv.b_mu[i];
    b_la[i] = sv.b_la[i];
  }
  for (int q = tid; q < Mh; q += nth) {
    h_mu[q] = sv.h_mu[q / ns];
    h_la[q] = sv.h_la[q / ns];
  }
  for (int q = tid; q < Ma; q += nth) d_la[q] = sv.d_la[q / ns];
  for (int q = tid; q < ah * ns * N; q += nth) {     // (f, j, i): symm (f, i) -> bare (j + f ns, perm_j[i])
    const int i = q % N, j = (q / N) % ns, f = q / (N * ns);
    const int row = j + f * ns, col = perms[j * N + i];
    w_mu[row + Mh * col] = sv.w_mu[f + ah * i];
    w_la[row + Mh * col] = sv.w_la[f + ah * i];
  }
  for (int q = tid; q < aa * ns * N; q += nth) {
    const int i = q % N, j = (q / N) % ns, f = q / (N * ns);
    const int row = j + f * ns, col = perms[j * N + i];
    u_mu[row + Ma * col] = sv.u_mu[f + aa * i];
    u_la[row + Ma * col] = sv.u_la[f + aa * i];
  }
}

// the symmetric b_mu and b_la become their means (NDMSymm.jl:97-98), in the FP64 master
__global__ void ndm_symm_project_kernel(double* symm, int N, int ah, int aa) {
  const NdmDev<double> v = ndm_view<double>(symm, N, ah, aa);
  double* b[2] = {const_cast<double*>(v.b_mu), const_cast<double*>(v.b_la)};
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w > 1) return;
  double s = 0.0;
  for (int i = lane; i < N; i += 32) s += b[w][i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  const double m = s / N;
  for (int i = lane; i < N; i += 32) b[w][i] = m;
}

// doubled configuration (σ, σ) of each physical configuration σ
__global__ void ndm_diag_expand_kernel(const uint64_t* in, int n, int N, uint64_t* out) {   // in == out allowed
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[s] = in[s] | (in[s] << N);
}

// ---------------------------------------------------------------------------
// Gradient accumulation G_k = Σ_s conj(L_s) Σ_c w_c O_k(σ'_c) (the
// conj(Σ L conj(∇L)) of BatchedGradSampler.jl:108-111).  One block per chunk
// of samples; connections are expanded 32 at a time into shared memory (their
// unit derivatives and configurations), then each thread accumulates its own
// parameters over them.  Partial sums per block in FP64.
// ---------------------------------------------------------------------------
template <typename R, int ACT>
__global__ void __launch_bounds__(256)
ndm_grad_kernel(NdmEff<R> e, DevOp op, const uint64_t* __restrict__ samples, int n, int hilb, int maxc,
                const cpx<R>* __restrict__ L, const cpx<R>* __restrict__ w, const int* __restrict__ wconn,
                const int* __restrict__ nconn, int chunk, double* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int CB = 32;
  const int U = e.U, P = e.P;
  cpx<R>* sgp = reinterpret_cast<cpx<R>*>(smem_raw);                 // [U][CB] derivatives at σ'
  cpx<R>* sbeta = sgp + (size_t)U * CB;                               // [CB]
  uint64_t* sbits = reinterpret_cast<uint64_t*>(sbeta + CB);          // [CB]
  __shared__ int s_list_s[CB], s_list_c[CB];
  const int s0 = blockIdx.x * chunk, s1 = min(n, s0 + chunk);
  // own-parameter accumulators (P <= 256 * PPT)
  constexpr int PPT = 24;
  cpx<double> acc[PPT];
#pragma unroll
  for (int q = 0; q < PPT; ++q) acc[q] = mk(0.0, 0.0);
  // enumerate (sample, connection) pairs of the chunk in batches of CB
  int cur_s = s0, cur_c = 0;
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) {
      int m = 0;
      while (m < CB && cur_s < s1) {
        if (cur_c < nconn[cur_s]) { s_list_s[m] = cur_s; s_list_c[m] = cur_c; ++m; ++cur_c; }
        else { ++cur_s; cur_c = 0; }
      }
      for (int q = m; q < CB; ++q) s_list_s[q] = -1;
    }
    __syncthreads();
    if (s_list_s[0] < 0) break;
    // expand: one thread per (pair, unit)
    for (int t = threadIdx.x; t < CB * U; t += blockDim.x) {
      const int m = t % CB, u = t / CB;
      const int s = s_list_s[m];
      if (s < 0) { sgp[(size_t)u * CB + m] = mk(R(0), R(0)); continue; }
      const int cc = wconn[(size_t)s * maxc + s_list_c[m]];
      const uint64_t bits = samples[s];
      // x_u at σ, then add the connection's change
      cpx<R> xu;
      if (e.theta) {
        xu = e.theta[(size_t)u * n + s];
      } else {
        xu = e.b[u];
        for (int i = 0; i < e.N2; ++i) {
          const R v = site_value<R>(bits, i, hilb);
          if (v != R(0)) { const cpx<R> c = e.C[u + (size_t)U * i]; xu.x += c.x * v; xu.y += c.y * v; }
        }
      }
      uint64_t nb = bits;
      const int nch = __ldg(op.conn_n_changes + cc);
      for (int q = 0; q < nch; ++q) {
        const int site = __ldg(op.conn_change_site + 8 * cc + q);
        const R nv = (R)__ldg(op.conn_change_value + 8 * cc + q);
        const R dv = nv - site_value<R>(bits, site, hilb);
        const cpx<R> c = e.C[u + (size_t)U * site];
        xu.x += c.x * dv;
        xu.y += c.y * dv;
        const uint64_t bit = (hilb == HILB_SPIN) ? (nv > 0 ? 1ull : 0ull) : (nv != R(0) ? 1ull : 0ull);
        nb = (nb & ~(1ull << site)) | (bit << site);
      }
      sgp[(size_t)u * CB + m] = act_df<ACT>(xu);
      if (u == 0) {
        sbits[m] = nb;
        sbeta[m] = conjc(L[s]) * w[(size_t)s * maxc + s_list_c[m]];
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
      const int k = threadIdx.x + q * blockDim.x;
      if (k < P) {
        for (int m = 0; m < CB; ++m) {
          if (s_list_s[m] < 0) break;
          const cpx<R> o = ndm_O_train<R>(e, k, sgp + m, CB, sbits[m], hilb);
          const cpx<R> b = sbeta[m];
          acc[q].x += (double)(b.x * o.x - b.y * o.y);
          acc[q].y += (double)(b.x * o.y + b.y * o.x);
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < PPT; ++q) {
    const int k = threadIdx.x + q * blockDim.x;
    if (k < P) {
      partial[(size_t)blockIdx.x * 2 * P + 2 * k] = acc[q].x;
      partial[(size_t)blockIdx.x * 2 * P + 2 * k + 1] = acc[q].y;
    }
  }
}

// deterministic reduction of the gradient partials, then
// F = G/Ns - C <O>  with C = mean |L|^2 (stats[0]); real parameters keep Re.
__global__ void ndm_force_finalize_kernel(int P, int nblk, int Ns, const double* __restrict__ partial,
                                          const double* __restrict__ meanO, const double* __restrict__ stats,
                                          double* __restrict__ force) {
  const int wp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (wp >= P) return;
  double gx = 0, gy = 0;
  for (int b = lane; b < nblk; b += 32) {
    gx += partial[(size_t)b * 2 * P + 2 * wp];
    gy += partial[(size_t)b * 2 * P + 2 * wp + 1];
  }
  for (int off = 16; off > 0; off >>= 1) {
    gx += __shfl_xor_sync(0xffffffffu, gx, off);
    gy += __shfl_xor_sync(0xffffffffu, gy, off);
  }
  if (lane == 0) {
    const double C = stats[0];
    force[2 * wp] = gx / Ns - C * meanO[2 * wp];
    force[2 * wp + 1] = gy / Ns - C * meanO[2 * wp + 1];
  }
}

// row means of X (FP64, one warp per row) -> meanO (complex per parameter)
__global__ void x_row_mean_kernel(const float* __restrict__ X, int rows, int ld, int ns, double* __restrict__ meanO) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (r >= rows) return;
  double s = 0;
  const float* row = X + (size_t)r * ld;
  for (int i = lane; i < ns; i += 32) s += (double)row[i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) meanO[r] = s / ns;        // row 2k -> Re <O_k>, 2k+1 -> Im <O_k>
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// centre X in place (padding columns stay 0); optionally round to TF32 and
// emit the TF32 remainder
__global__ void x_center_kernel(float* __restrict__ X, float* __restrict__ Xlo, int rows, int ld, int ns,
                                const double* __restrict__ meanO, int tf32) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)rows * ld) return;
  const int r = (int)(idx / ld), s = (int)(idx % ld);
  float v = s < ns ? (float)((double)X[idx] - meanO[r]) : 0.f;
  if (tf32) {
    const float hi = tf32_round(v);
    X[idx] = hi;
    if (Xlo) Xlo[idx] = tf32_round(v - hi);
  } else {
    X[idx] = v;
  }
}

template <typename R>
__global__ void ndm_grad_to_host_layout(const double* Oout, int P, int n, double* out) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx < 2L * P * n) out[idx] = Oout[idx];
}

}  // namespace

// ------------------------------- launchers ---------------------------------

template <typename R>
cudaError_t launch_ndm_effective(const NdmDev<R>& n, const NdmEffBufs<R>& b, cudaStream_t st) {
  const int U = 4 * n.Mh + n.Ma, tot = U * 2 * n.N;
  ndm_effective_kernel<R><<<(tot + 127) / 128, 128, 0, st>>>(n, b.C, b.b, b.a, b.Cs, b.bs);
  return cudaGetLastError();
}

template <typename R>
static size_t unit_smem(int U, int T) { return (size_t)2 * U * T * sizeof(cpx<R>); }

template <typename R>
static int ndm_threads(int U) {
  int T = 128;
  while (T > 32 && unit_smem<R>(U, T) > 96 * 1024) T /= 2;
  return T;
}

template <typename R, typename K>
static cudaError_t set_smem(K kern, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

template <typename R>
cudaError_t launch_ndm_eval(const NdmEff<R>& e, int act, const uint64_t* samples, int n, int hilb,
                            cpx<R>* logrho, float* X, int ldx, double* Oout, cudaStream_t st) {
  const int T = ndm_threads<R>(e.U);
  const size_t smem = unit_smem<R>(e.U, T);
  cudaError_t err;
  if (act == ACT_LOGCOSH) {
    if ((err = set_smem<R>(ndm_eval_kernel<R, ACT_LOGCOSH>, smem)) != cudaSuccess) return err;
    ndm_eval_kernel<R, ACT_LOGCOSH><<<(n + T - 1) / T, T, smem, st>>>(e, samples, n, hilb, logrho, X, ldx, Oout);
  } else {
    if ((err = set_smem<R>(ndm_eval_kernel<R, ACT_SOFTPLUS>, smem)) != cudaSuccess) return err;
    ndm_eval_kernel<R, ACT_SOFTPLUS><<<(n + T - 1) / T, T, smem, st>>>(e, samples, n, hilb, logrho, X, ldx, Oout);
  }
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_ndm_loc(const NdmEff<R>& e, int act, const DevOp& op, const uint64_t* samples, int n,
                           int hilb, int maxc, cpx<R>* L, cpx<R>* w, int* wconn, int* nconn, cudaStream_t st) {
  const int T = ndm_threads<R>(e.U);
  const size_t smem = unit_smem<R>(e.U, T);
  cudaError_t err;
  if (act == ACT_LOGCOSH) {
    if ((err = set_smem<R>(ndm_loc_kernel<R, ACT_LOGCOSH>, smem)) != cudaSuccess) return err;
    ndm_loc_kernel<R, ACT_LOGCOSH><<<(n + T - 1) / T, T, smem, st>>>(e, op, samples, n, hilb, maxc, L, w, wconn, nconn);
  } else {
    if ((err = set_smem<R>(ndm_loc_kernel<R, ACT_SOFTPLUS>, smem)) != cudaSuccess) return err;
    ndm_loc_kernel<R, ACT_SOFTPLUS><<<(n + T - 1) / T, T, smem, st>>>(e, op, samples, n, hilb, maxc, L, w, wconn, nconn);
  }
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_ndm_diag_obs(const NdmEff<R>& e_in, int act, const DevOp& op, const uint64_t* samples, int n,
                                int hilb, cpx<R>* logrho, cpx<R>* O, cudaStream_t st) {
  if (n < 1) return cudaSuccess;
  NdmEff<R> e = e_in;
  e.theta = nullptr;              // the (σ, σ) configurations are formed in the kernel
  const int T = ndm_threads<R>(e.U);
  const size_t smem = unit_smem<R>(e.U, T);
  cudaError_t err;
  if (act == ACT_LOGCOSH) {
    if ((err = set_smem<R>(ndm_diag_obs_kernel<R, ACT_LOGCOSH>, smem)) != cudaSuccess) return err;
    ndm_diag_obs_kernel<R, ACT_LOGCOSH><<<(n + T - 1) / T, T, smem, st>>>(e, op, samples, n, hilb, logrho, O);
  } else {
    if ((err = set_smem<R>(ndm_diag_obs_kernel<R, ACT_SOFTPLUS>, smem)) != cudaSuccess) return err;
    ndm_diag_obs_kernel<R, ACT_SOFTPLUS><<<(n + T - 1) / T, T, smem, st>>>(e, op, samples, n, hilb, logrho, O);
  }
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_ndm_diagonal(const NdmDev<R>& n, cpx<R>* a, cpx<R>* b, cpx<R>* W, cudaStream_t st) {
  const int md = n.Mh + n.Ma;
  const int tot = md * n.N > n.N ? md * n.N : n.N;
  ndm_diagonal_kernel<R><<<(tot + 127) / 128, 128, 0, st>>>(n, a, b, W);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_split_effective(const cpx<R>* p, int N, int M, const NdmEffBufs<R>& b, cudaStream_t st) {
  const int N2 = 2 * N, tot = M * N2;
  split_effective_kernel<R><<<(tot + 127) / 128, 128, 0, st>>>(p, N2, M, b.C, b.b, b.a, b.Cs, b.bs);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_split_diagonal(const cpx<R>* p, int N, int M, cpx<R>* a, cpx<R>* b, cpx<R>* W, cudaStream_t st) {
  const int tot = M * N > N ? M * N : N;
  split_diagonal_kernel<R><<<(tot + 127) / 128, 128, 0, st>>>(p, N, M, a, b, W);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_ndm_symm_bare(const R* symm, int N, int ah, int aa, int ns, const int* perms, R* bare,
                                 cudaStream_t st) {
  const int work = (ah > aa ? ah : aa) * ns * N + N;
  ndm_symm_bare_kernel<R><<<(work + 255) / 256, 256, 0, st>>>(symm, N, ah, aa, ns, perms, bare);
  return cudaGetLastError();
}

cudaError_t launch_ndm_symm_project(double* symm, int N, int ah, int aa, cudaStream_t st) {
  ndm_symm_project_kernel<<<1, 64, 0, st>>>(symm, N, ah, aa);
  return cudaGetLastError();
}

cudaError_t launch_ndm_diag_expand(const uint64_t* in, int n, int N, uint64_t* out, cudaStream_t st) {
  if (n < 1) return cudaSuccess;
  ndm_diag_expand_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, n, N, out);
  return cudaGetLastError();
}

int ndm_grad_chunk() { return 16; }

template <typename R>
cudaError_t launch_ndm_grad(const NdmEff<R>& e, int act, const DevOp& op, const uint64_t* samples, int n,
                            int hilb, int maxc, const cpx<R>* L, const cpx<R>* w, const int* wconn,
                            const int* nconn, double* partial, const double* meanO, const double* stats,
                            double* force, cudaStream_t st) {
  if (e.P > 256 * 24) return cudaErrorInvalidValue;
  const int chunk = ndm_grad_chunk();
  const int nblk = (n + chunk - 1) / chunk;
  const size_t smem = (size_t)e.U * 32 * sizeof(cpx<R>) + 32 * sizeof(cpx<R>) + 32 * sizeof(uint64_t);
  cudaError_t err;
  if (act == ACT_LOGCOSH) {
    if ((err = set_smem<R>(ndm_grad_kernel<R, ACT_LOGCOSH>, smem)) != cudaSuccess) return err;
    ndm_grad_kernel<R, ACT_LOGCOSH><<<nblk, 256, smem, st>>>(e, op, samples, n, hilb, maxc, L, w, wconn, nconn,
                                                             chunk, partial);
  } else {
    if ((err = set_smem<R>(ndm_grad_kernel<R, ACT_SOFTPLUS>, smem)) != cudaSuccess) return err;
    ndm_grad_kernel<R, ACT_SOFTPLUS><<<nblk, 256, smem, st>>>(e, op, samples, n, hilb, maxc, L, w, wconn, nconn,
                                                              chunk, partial);
  }
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  ndm_force_finalize_kernel<<<(32 * e.P + 255) / 256, 256, 0, st>>>(e.P, nblk, n, partial, meanO, stats, force);
  return cudaGetLastError();
}

int ndm_grad_nblocks(int n) { return (n + ndm_grad_chunk() - 1) / ndm_grad_chunk(); }

cudaError_t launch_x_center(float* X, float* Xlo, int rows, int ld, int ns, double* meanO, int tf32,
                            cudaStream_t st) {
  x_row_mean_kernel<<<(rows * 32 + 255) / 256, 256, 0, st>>>(X, rows, ld, ns, meanO);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long tot = (long)rows * ld;
  x_center_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(X, Xlo, rows, ld, ns, meanO, tf32);
  return cudaGetLastError();
}

template cudaError_t launch_ndm_effective<float>(const NdmDev<float>&, const NdmEffBufs<float>&, cudaStream_t);
template cudaError_t launch_ndm_effective<double>(const NdmDev<double>&, const NdmEffBufs<double>&, cudaStream_t);
template cudaError_t launch_ndm_eval<float>(const NdmEff<float>&, int, const uint64_t*, int, int, cpx<float>*, float*, int, double*, cudaStream_t);
template cudaError_t launch_ndm_eval<double>(const NdmEff<double>&, int, const uint64_t*, int, int, cpx<double>*, float*, int, double*, cudaStream_t);
template cudaError_t launch_ndm_loc<float>(const NdmEff<float>&, int, const DevOp&, const uint64_t*, int, int, int, cpx<float>*, cpx<float>*, int*, int*, cudaStream_t);
template cudaError_t launch_ndm_loc<double>(const NdmEff<double>&, int, const DevOp&, const uint64_t*, int, int, int, cpx<double>*, cpx<double>*, int*, int*, cudaStream_t);
template cudaError_t launch_ndm_grad<float>(const NdmEff<float>&, int, const DevOp&, const uint64_t*, int, int, int, const cpx<float>*, const cpx<float>*, const int*, const int*, double*, const double*, const double*, double*, cudaStream_t);
template cudaError_t launch_ndm_grad<double>(const NdmEff<double>&, int, const DevOp&, const uint64_t*, int, int, int, const cpx<double>*, const cpx<double>*, const int*, const int*, double*, const double*, const double*, double*, cudaStream_t);
template cudaError_t launch_ndm_diag_obs<float>(const NdmEff<float>&, int, const DevOp&, const uint64_t*, int, int, cpx<float>*, cpx<float>*, cudaStream_t);
template cudaError_t launch_ndm_diag_obs<double>(const NdmEff<double>&, int, const DevOp&, const uint64_t*, int, int, cpx<double>*, cpx<double>*, cudaStream_t);
template cudaError_t launch_ndm_diagonal<float>(const NdmDev<float>&, cpx<float>*, cpx<float>*, cpx<float>*, cudaStream_t);
template cudaError_t launch_ndm_diagonal<double>(const NdmDev<double>&, cpx<double>*, cpx<double>*, cpx<double>*, cudaStream_t);
template cudaError_t launch_split_effective<float>(const cpx<float>*, int, int, const NdmEffBufs<float>&, cudaStream_t);
template cudaError_t launch_split_effective<double>(const cpx<double>*, int, int, const NdmEffBufs<double>&, cudaStream_t);
template cudaError_t launch_split_diagonal<float>(const cpx<float>*, int, int, cpx<float>*, cpx<float>*, cpx<float>*, cudaStream_t);
template cudaError_t launch_split_diagonal<double>(const cpx<double>*, int, int, cpx<double>*, cpx<double>*, cpx<double>*, cudaStream_t);
template cudaError_t launch_ndm_symm_bare<float>(const float*, int, int, int, int, const int*, float*, cudaStream_t);
template cudaError_t launch_ndm_symm_bare<double>(const double*, int, int, int, int, const int*, double*, cudaStream_t);
