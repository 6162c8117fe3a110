// Launch interfaces of the NDM (purified density matrix) path.
#pragma once
#include "nq_kernels.cuh"

// Real NDM parameters (reference flat order), pointers into one array.
template <typename R> struct NdmDev {
  int N = 0, Mh = 0, Ma = 0;
  const R *b_mu = nullptr, *h_mu = nullptr, *w_mu = nullptr, *u_mu = nullptr;
  const R *b_la = nullptr, *h_la = nullptr, *d_la = nullptr, *w_la = nullptr, *u_la = nullptr;
};

template <typename R> NQ_HD NdmDev<R> ndm_view(const R* p, int N, int Mh, int Ma) {
  NdmDev<R> d;
  d.N = N; d.Mh = Mh; d.Ma = Ma;
  const R* q = p;
  d.b_mu = q; q += N;
  d.h_mu = q; q += Mh;
  d.w_mu = q; q += (size_t)Mh * N;
  d.u_mu = q; q += (size_t)Ma * N;
  d.b_la = q; q += N;
  d.h_la = q; q += Mh;
  d.d_la = q; q += Ma;
  d.w_la = q; q += (size_t)Mh * N;
  d.u_la = q;
  return d;
}

NQ_HD int ndm_n_params(int N, int Mh, int Ma) { return 2 * N + 2 * Mh + Ma + 2 * Mh * N + 2 * Ma * N; }

// Effective generalised-RBM form over the 2N doubled sites (see ndm.cu).
template <typename R> struct NdmEff {
  int N = 0, N2 = 0, Mh = 0, Ma = 0, U = 0, P = 0;
  int split = 0;               // RBMSplit: Mh = 0, Ma = U = M units of weight 1, RBM parameter layout
  // NDMSymm: the network is the bare NDM (Mh, Ma, C, b, a) and the trainable
  // parameters are the symmetric NDM's; O of trainable k is
  // Σ_q sym_coef[q] O_bare(sym_idx[q]) over q in [sym_off[k], sym_off[k+1]).  P
  // counts the trainable parameters.
  const int* sym_off = nullptr;
  const int* sym_idx = nullptr;
  const double* sym_coef = nullptr;
  const cpx<R>* C = nullptr;   // [U x N2] column-major
  const cpx<R>* b = nullptr;   // [U]
  const cpx<R>* a = nullptr;   // [N2]
  // optional [U][n] unit pre-activations θ_u = b_u + Σ_i C[u][i] v_i of the
  // n samples being evaluated (the tensor-core θ of NQ_EVAL_TC_BF16X2/X3);
  // null: the kernels form θ on CUDA cores
  const cpx<R>* theta = nullptr;
};

template <typename R> struct NdmEffBufs {
  cpx<R>* C = nullptr;    // [U x N2]
  cpx<R>* b = nullptr;    // [U]
  cpx<R>* a = nullptr;    // [N2]
  cpx<R>* Cs = nullptr;   // [Ms x N2] units entering |ρ|^2 (sampler)
  cpx<R>* bs = nullptr;   // [Ms]
};

template <typename R>
cudaError_t launch_ndm_effective(const NdmDev<R>& n, const NdmEffBufs<R>& b, cudaStream_t st);
template <typename R>
cudaError_t launch_ndm_eval(const NdmEff<R>& e, int act, const uint64_t* samples, int n, int hilb,
                            cpx<R>* logrho, float* X, int ldx, double* Oout, cudaStream_t st);
template <typename R>
cudaError_t launch_ndm_loc(const NdmEff<R>& e, int act, const DevOp& op, const uint64_t* samples, int n,
                           int hilb, int maxc, cpx<R>* L, cpx<R>* w, int* wconn, int* nconn, cudaStream_t st);
template <typename R>
cudaError_t launch_ndm_grad(const NdmEff<R>& e, int act, const DevOp& op, const uint64_t* samples, int n,
                            int hilb, int maxc, const cpx<R>* L, const cpx<R>* w, const int* wconn,
                            const int* nconn, double* partial, const double* meanO, const double* stats,
                            double* force, cudaStream_t st);
int ndm_grad_nblocks(int n);
// BatchedObsDMSampler: O_loc(σ) = Σ_σ' O_σσ' ρ(σ',σ)/ρ(σ,σ) of physical samples
// (N-site bits) and logρ(σ,σ) (nullable)
template <typename R>
cudaError_t launch_ndm_diag_obs(const NdmEff<R>& e, int act, const DevOp& op, const uint64_t* samples, int n,
                                int hilb, cpx<R>* logrho, cpx<R>* O, cudaStream_t st);
// N-site sampler tables of p(σ) ∝ ρ(σ,σ): a [N], b [Mh+Ma], W [(Mh+Ma) x N]
template <typename R>
cudaError_t launch_ndm_diagonal(const NdmDev<R>& n, cpx<R>* a, cpx<R>* b, cpx<R>* W, cudaStream_t st);
// RBMSplit: effective network copied from the complex parameters p (RBM layout over 2N sites)
template <typename R>
cudaError_t launch_split_effective(const cpx<R>* p, int N, int M, const NdmEffBufs<R>& b, cudaStream_t st);
// RBMSplit diagonal sampler tables: a [N], b [M], W [M x N]
template <typename R>
cudaError_t launch_split_diagonal(const cpx<R>* p, int N, int M, cpx<R>* a, cpx<R>* b, cpx<R>* W, cudaStream_t st);
// NDMSymm (MixedDensityMatrix/NDMSymm.jl:89-133): bare NDM parameters
// (hidden Mh = ah ns, ancilla Ma = aa ns) from the symmetric ones; perms [ns x N]
template <typename R>
cudaError_t launch_ndm_symm_bare(const R* symm, int N, int ah, int aa, int ns, const int* perms, R* bare,
                                 cudaStream_t st);
// NDMSymm: the symmetric visible biases b_mu, b_la replaced by their means (FP64 master, in place)
cudaError_t launch_ndm_symm_project(double* symm, int N, int ah, int aa, cudaStream_t st);
// out[s] = (σ, σ) as 2N-site bits
cudaError_t launch_ndm_diag_expand(const uint64_t* in, int n, int N, uint64_t* out, cudaStream_t st);

// centre the rows of X (rows x ld, first ns columns valid), meanO[r] = row mean;
// tf32: round to TF32 and write the remainder to Xlo (if given)
cudaError_t launch_x_center(float* X, float* Xlo, int rows, int ld, int ns, double* meanO, int tf32,
                            cudaStream_t st);
