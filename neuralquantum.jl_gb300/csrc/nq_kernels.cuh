// Kernel launch interfaces shared between the translation units of
// libnqcuda.  Every launcher returns a cudaError_t and enqueues on `st`.
#pragma once
#include <cuda_bf16.h>

#include <vector>

#include "nq_common.cuh"

// Flattened operator on the device (see nq_op_table in include/nqcuda.h).
struct DevOp {
  int n_ops = 0, n_rows = 0, n_conns = 0;
  const int* op_n_sites = nullptr;      // [n_ops]
  const int* op_sites = nullptr;        // [8*n_ops]
  const int* op_row_offset = nullptr;   // [n_ops]
  const int* row_conn_offset = nullptr; // [n_rows+1]
  const double* conn_mel = nullptr;     // [2*n_conns]
  const float2* conn_mel_f = nullptr;   // [n_conns] the same elements in FP32 (FP32 estimators)
  // packed copies for the RBM estimator's walk (one load per operator / connection):
  // op_meta[o] = {n_sites, row_offset, sites 0-3, sites 4-7} (one byte per site);
  // conn_pack[c] = {FP32 mel re, FP32 mel im (bit patterns), n_changes,
  //                 first changed site | (its new value as a byte) << 8}
  const int4* op_meta = nullptr;        // [n_ops]
  const int4* conn_pack = nullptr;      // [n_conns]
  const int* conn_n_changes = nullptr;  // [n_conns]
  const int* conn_change_site = nullptr;// [8*n_conns]
  const signed char* conn_change_value = nullptr; // [8*n_conns]
};

// ------------------------------- RBM ------------------------------------
// Per-(site i, hidden h) tables, index i*M + h, |Δσ| = d (2 spin, 1 Fock):
//   logcosh:  t0 = cosh(W d), t1 = sinh(W d), t2 = tanh(W d)
//   softplus: t0 = exp(W d) - 1, t1 = exp(-W d) - 1, t2 = 0
// With g = f'(θ), the ratio cosh(θ+Δ)/cosh(θ) (resp. (1+e^{θ+Δ})/(1+e^θ))
// of a single flip with Δ = W dv is t0 + g*sign(dv)*t1 (resp. 1 + g*t0|t1).
struct OpMovesDev;

template <typename R> struct RbmDev {
  int N = 0, M = 0, act = 0, hilb = 0;
  int n_half = 0;              // hidden units h < n_half enter log|ψ|^2 with weight 1/2
                               // (the λ units of the purified density matrix)
  const cpx<R>* a = nullptr;   // [N]
  const cpx<R>* b = nullptr;   // [M]
  const cpx<R>* W = nullptr;   // [M*N] column-major
  const cpx<R>* t0 = nullptr;  // [N*M] (exchange rule: [n_rows*M], per coupling)
  const cpx<R>* t1 = nullptr;
  const cpx<R>* t2 = nullptr;
  // Exchange rule (ExchangeRule.jl): the move of row r swaps the values of
  // sites pairs[r] = (i, j); with σ_i != σ_j it changes θ by Δv_i (W_hi - W_hj),
  // so the single-flip tables are taken of rW = W_hi - W_hj.  n_rows = 0:
  // local flips, row = site.
  int n_rows = 0;
  const int2* pairs = nullptr;   // [n_rows]
  const cpx<R>* rW = nullptr;    // [M*n_rows] at h + M*r
  const R* rare = nullptr;       // [n_rows] 2 log2(e) Re(a_i - a_j)
  // OperatorRule: the rows are the move classes of the operator's
  // connections (host pointer, read by the launcher only)
  const OpMovesDev* opm = nullptr;
};

// OperatorRule (src/Samplers/MCMCRules/OperatorRule.jl:23-58): the moves of a
// configuration σ are the connections of its rows in the operator's tables
// (row_valdiff, KLocalOperator.jl:151-158, KLocalOperatorSum.jl:40-46),
// drawn uniformly, with the Hastings factor n(σ)/n(σ') of the row lengths.
// Connections that change sites are grouped into move classes (changed sites
// and their new local indices, up to complement); a class's θ-tables are
// those of Δθ = Σ_q W[h, s_q] dv_q, like the single-flip tables.
struct OpMovesDev {
  int n_ops = 0, n_rows = 0, n_conns = 0, n_classes = 0;
  int const_counts = 0;                           // every row of an operator has the same length
  int n_total = 0;                                // const_counts: connections of every configuration
  const unsigned long long* op_sites = nullptr;   // [n_ops] site d in byte d
  const unsigned long long* op_mask = nullptr;    // [n_ops] sites of the operator
  const int* op_n_sites = nullptr;                // [n_ops]
  const int* op_row_offset = nullptr;             // [n_ops]
  const int* op_prefix = nullptr;                 // [n_ops + 1] const_counts: first move of each operator
  const int* row_conn_offset = nullptr;           // [n_rows + 1]
  const int* conn_code = nullptr;                 // [n_conns] -1: no change; 2 class + (complement ? 1 : 0)
  const unsigned long long* class_mask = nullptr; // [n_classes] changed sites
  const int* class_sites = nullptr;               // [8 n_classes] sites of the class (-1: unused)
  const int* class_bits = nullptr;                // [n_classes] canonical new local index of site q in bit q
};

cudaError_t launch_rbm_params_from_master(const double* master, int N, int M, float* f32_out,
                                          cudaStream_t st);
cudaError_t launch_master_to_f32(const double* master, long n, float* f32_out, cudaStream_t st);
template <typename R>
cudaError_t launch_rbm_tables(const RbmDev<R>& net, cpx<R>* t0, cpx<R>* t1, cpx<R>* t2,
                              cudaStream_t st);
// exchange-rule tables of the couplings (i, j) = pairs[r]: t0..t2 of Δ = d (W_hi - W_hj)
// at r*M + h, rW = W_hi - W_hj at h + M*r, rare[r] = 2 log2(e) Re(a_i - a_j)
template <typename R>
cudaError_t launch_rbm_exchange_tables(const RbmDev<R>& net, int n_rows, const int2* pairs, cpx<R>* t0,
                                       cpx<R>* t1, cpx<R>* t2, cpx<R>* rW, R* rare, cudaStream_t st);

struct SamplerRun {
  int B = 0, L = 0, burn = 0, passes = 1, n_record = 0, write_last_at_end = 0;
  uint32_t k0 = 0, k1 = 0, call = 0;
  const uint32_t* call_ptr = nullptr;          // if set, the call index is read here
  uint64_t* samples = nullptr;                 // [L][B]
  unsigned long long* accepted = nullptr;      // scalar counter
  unsigned char* accept_bits = nullptr;        // nullable [steps][B]
  int block = 256;                             // threads per block (64, 128 or 256)
};
// G = lanes per chain (4, 8, 16 or 32); rbm_sampler_valid_lanes lists the
// values instantiated for M hidden units (used by the autotuner).
template <typename R>
cudaError_t launch_rbm_sampler(const RbmDev<R>& net, const SamplerRun& run, int G, cudaStream_t st);
int rbm_sampler_valid_lanes(int N, int M, int csize, int* out, int max_out);
// the instantiations with units at weight 1/2 (net.n_half > 0, density matrices)
template <typename R>
cudaError_t launch_rbm_sampler_half(const RbmDev<R>& net, const SamplerRun& run, int G, cudaStream_t st);
// the exchange-rule instantiations of the FP32 sampler (net.pairs set)
cudaError_t launch_rbm_sampler_exchange(const RbmDev<float>& net, const SamplerRun& run, int G, cudaStream_t st);
// OperatorRule sampler (FP32 ket), net.opm set
cudaError_t launch_rbm_sampler_oprule(const RbmDev<float>& net, const SamplerRun& run, int G, cudaStream_t st);
// move-class tables of the OperatorRule: rW[h + M k] = Σ_q W[h, s_q] (2 b_q - 1),
// rare[k] = 2 log2(e) Σ_q Re a_{s_q} (2 b_q - 1), t0..t2 of Δθ = d rW at k*M + h
cudaError_t launch_rbm_class_tables(const RbmDev<float>& net, const OpMovesDev& m, cpx<float>* t0, cpx<float>* t1,
                                    cpx<float>* t2, cpx<float>* rW, float* rare, cudaStream_t st);
// shared memory of the OperatorRule sampler with G lanes per chain (0 if it does not fit)
size_t oprule_sampler_smem(const OpMovesDev& m, int M, int G);

// Feed-forward ket chains (Chain.jl, Dense.jl, WeightedSum.jl, sum.jl): Dense
// layers then one closing sum_autobatch or WSum; offsets into the complex
// parameter vector p (functor order).
enum { LAYER_DENSE = 0, LAYER_WSUM = 1, LAYER_SUM = 2 };
struct ChainLayerDev {
  int kind = 0, in = 0, out = 0, act = 0, w_off = 0, b_off = 0;
};
template <typename R> struct ChainDev {
  int N = 0, hilb = 0, n_layers = 0, P = 0;
  int n_theta = 0;             // Σ out over the Dense layers (stored pre-activations)
  int max_w = 0;               // widest Dense output
  ChainLayerDev L[8];
  // first layer PositiveDefR: p holds it in the Dense form over the doubled
  // sites (W_σ = Wr + i Wi, W_η = Wr − i Wi, b) and the gradient entries of
  // that layer are taken with respect to (Wr, Wi, b)
  int pdr = 0;
  const cpx<R>* p = nullptr;
};
// logψ, E_loc (op nullable) and O into X (uncentred FP32 rows 2k, 2k+1) and/or
// Oout (P x n complex FP64)
template <typename R>
cudaError_t launch_chain_eval(const ChainDev<R>& c, const uint64_t* samples, int n, const DevOp* op, cpx<R>* logpsi,
                              cpx<R>* eloc, float* X, int ldx, double* Oout, cudaStream_t st);
// density-matrix chains: G = conj(∇L_loc) per sample ([P][n] FP32 complex),
// then F = conj(Σ_s L_s G_s)/Ns - C <O> with C = stats[0] and <O> from the
// uncentred rows of X
template <typename R>
cudaError_t launch_chain_liouv_force(const ChainDev<R>& c, const uint64_t* samples, int n, const DevOp& op,
                                     const cpx<R>* L, const float* X, int ldx, const double* stats, float2* G,
                                     double* force, cudaStream_t st);
// F = E O_c† / Ns from the uncentred rows of X and the mean of E in stats[0..1]
template <typename R>
cudaError_t launch_chain_force(const float* X, int ldx, int P, int ns, const cpx<R>* E, const double* stats,
                               double* force, cudaStream_t st);
template <typename R>
cudaError_t launch_chain_sampler(const ChainDev<R>& c, const SamplerRun& run, cudaStream_t st);
// the working parameters of a chain that opens with PositiveDefR (n_out x
// n_sites weights): master (Wr, Wi, b, later layers; complex interleaved, P
// entries) into the Dense form (W_σ, W_η, b, later layers) as FP32 (p32) or
// FP64 (p64), whichever is non-null
// out = i F (P complex): the right-hand side of SR with time evolution
cudaError_t launch_times_i(const double* F, int P, double* out, cudaStream_t st);
cudaError_t launch_chain_pdr_params(const double* master, int P, int n_out, int n_sites, float* p32, double* p64,
                                    cudaStream_t st);

// Exact sampler (Exact.jl): all 2^N configurations of the sampler's space
// (N <= 26), FP64 CDF, inverse-CDF draws into run.samples (n_record draws per
// chain, plus one into slot 0 with write_last_at_end).  work:
// exact_sampler_work_doubles(N) doubles.
size_t exact_sampler_work_doubles(int nsites);
template <typename R>
cudaError_t launch_exact_sampler(const RbmDev<R>& net, const SamplerRun& run, double* work, cudaStream_t st);

// Many independent problems in one sampler launch (FP32): problem p runs on
// blocks [blk_start[p], blk_start[p+1]) of 256 threads (256/G chains each);
// M_max / N_max size the shared tables, G is common to all problems.
template <typename R> struct SamplerJob {
  RbmDev<R> net;
  SamplerRun run;
};
template <typename R>
cudaError_t launch_rbm_sampler_batch(const SamplerJob<R>* jobs, const int* blk_start, int np, int total_blocks,
                                     int M_max, int N_max, int act, int G, cudaStream_t st);

// Many-problem evaluation: problem p on blocks [blk_start[p], blk_start[p+1])
// of T threads (T = rbm_eval_threads(M_max)); the shared tables are sized for
// M_max x N_max and every job has an operator (has_op = 1).
template <typename R> struct EvalJob {
  RbmDev<R> net;
  const uint64_t* samples;
  int Ns;
  DevOp op;
  int has_op;
  cpx<R>* logpsi;
  cpx<R>* g;
  cpx<R>* eloc;
};
int rbm_eval_threads(int M_max);
template <typename R>
cudaError_t launch_rbm_eval_batch(const EvalJob<R>* jobs, const int* blk_start, int np, int total_blocks,
                                  int M_max, int N_max, int act, int T, cudaStream_t st);

// logψ, g = f'(θ) (hidden-major [M][Ns]) and the local estimator on Ns samples.
// theta_in_g = 1: g holds θ = Wσ + b on entry (launch_theta_bf16x2).
template <typename R>
cudaError_t launch_rbm_eval(const RbmDev<R>& net, const uint64_t* samples, int Ns,
                            const DevOp* op, cpx<R>* logpsi, cpx<R>* g, cpx<R>* eloc,
                            cudaStream_t st, int theta_in_g = 0);

// θ = Wσ + b on tcgen05 with W split into nterms BF16 terms (2: hi + lo,
// 3: hi + mid + lo; FP32 accumulation): the packed W image
// (theta_tc_image_elems(M, nterms) BF16) is rebuilt whenever W changes; θ is
// written as complex FP32 [h][Ns].  N <= 64, 2M <= 512.
int theta_tc_rows(int M);
size_t theta_tc_image_elems(int M, int nterms);
bool theta_tc_supported(int N, int M);
cudaError_t launch_theta_pack(const cpx<float>* W, int M, int N, int nterms, __nv_bfloat16* img, cudaStream_t st);
cudaError_t launch_theta_bf16x2(const __nv_bfloat16* img, int nterms, int M, int N, const cpx<float>* b,
                                const uint64_t* samples, int Ns, int hilb, cpx<float>* theta, int* err,
                                cudaStream_t st);

// Per-block partial sums of O, E conj(O) and E over sample chunks, then a
// deterministic FP64 reduction into <O> (meanO) and F.
struct ForceBufs {
  double* partial = nullptr;   // [nblk][2*P] complex (O, EO)
  double* partialE = nullptr;  // [nblk] complex
  double* meanO = nullptr;     // [P] complex
  double* force = nullptr;     // [P] complex
  double* meanE = nullptr;     // complex scalar
  double* sums = nullptr;      // [4P+2] reduction scratch
};
int rbm_force_nblocks(int Ns, int N, int M, int csize);
template <typename R>
cudaError_t launch_rbm_force(const RbmDev<R>& net, const uint64_t* samples, int Ns, const cpx<R>* g,
                             const cpx<R>* eloc, const ForceBufs& fb, cudaStream_t st);

// ------------------------------- SR -------------------------------------
// Structured O rows for the S accumulation: parameter k of the RBM vector
// [a (N), b (M), W (M x N)] at sample s is v_j(s), g_h(s), g_h(s) v_j(s).
struct RbmOSource {
  int N = 0, M = 0, hilb = 0, Ns = 0;
  const uint64_t* samples = nullptr;
  const float2* g = nullptr;       // [M][Ns] (FP32 storage)
  const double* meanO = nullptr;   // [P] complex
};
// G = X X^T over the real rows X = [Re O_c; Im O_c] interleaved (2P x Ns),
// upper tiles only, FP32 CUDA cores.  G is 2P x 2P row-major.
cudaError_t launch_gram_simt(const RbmOSource& src, int P, float* G, float* partial, int ksplit,
                             cudaStream_t st);
// materialise X (2P x Ns_pad, row-major, zero padded) rounded to TF32 for
// tcgen05; if Xlo is given it receives the TF32 remainder x - tf32(x).
// bf16 = 1: X is written as BF16 (round to nearest) for the BF16 S mode; Xlo unused
cudaError_t launch_build_X(const RbmOSource& src, int P, int Ns_pad, float* X, float* Xlo, cudaStream_t st,
                           int bf16 = 0);
// tcgen05 SYRK: G = X X^T (upper 128x128 tiles of the rows x rows row-major G).
// Persistent CTAs over (k-split, tile) items; each item writes a column-major
// 128x128 partial tile into `partial` (gram_tc_partial_elems floats), and a
// second kernel sums the k-splits into G.  split3 adds the hi*lo + lo*hi
// products (3xTF32); bf16 = 1 reads X as BF16.  err receives timeout bits.
cudaError_t launch_gram_tc(const void* X, const float* Xlo, int rows, int Ns_pad, int split3, float* G,
                           float* partial, int* err, cudaStream_t st, int bf16 = 0);
int gram_tc_supported();
int gram_tc_ksplit(int rows, int Ns_pad, int bf16 = 0);
size_t gram_tc_partial_elems(int rows, int Ns_pad, int bf16 = 0);
cudaError_t launch_gram_reduce(const float* partial, int rows, int rp, int tile, int ksplit, float* G,
                               cudaStream_t st);
// S (P x P complex double, full Hermitian) = combine(G)/Ns
cudaError_t launch_assemble_S(const float* G, int P, double inv_ns, bool real_params, double* S,
                              cudaStream_t st);

// block Gauss–Jordan inverse of the Hermitian positive-definite W in place (lower
// triangle: W <- -W^-1), one cooperative launch; ctl: sweep_ctl_bytes().
// launch_herm_fill then mirrors the lower triangle into the upper one.
size_t sweep_ctl_bytes();
// diagonal shift of the SR matrix: kind 0 eps, kind 1 lam * S_ii (sr_multiplicative)
NQ_D double sr_diag_shift(const double* S, int P, int i, int kind, double eps, double lam) {
  if (kind == 0) return eps;
  if (kind == 1) return lam * S[2 * ((size_t)i + (size_t)P * i)];
  return 0.0;
}
// the FP64-residual refinement (x0 = A⁻¹F, then corrections until |Δx_k|,
// or the error |Δx_k|²/|Δx_{k-1}| it leaves while the iteration contracts,
// is <= tol |x|, or max_corr of them) as one cooperative launch of at most
// kRefineMaxCtas CTAs; ctl: sweep_ctl_bytes(); norms: refine_norm_doubles();
// info (nullable): [corrections, the smaller of the last |Δx|/|x| and the
// estimated relative error after it]
constexpr int kRefineMaxCtas = 256;
constexpr double kRefineTol = 1e-13;
// dynamic shared memory of a refinement CTA: the GEMV vector (P complex
// doubles) when it fits 40 KiB (under the 48 KiB default with the kernel's
// static shared memory), else none and the vector is read from L2; the kernel
// stages a problem's vector only when it fits the launch's allocation
constexpr size_t kRefineStageMax = 40 * 1024;
constexpr size_t refine_stage_bytes(int P) { return (size_t)16 * P <= kRefineStageMax ? (size_t)16 * P : 0; }
constexpr size_t refine_norm_doubles() { return 2 * (size_t)kRefineMaxCtas * 8; }
cudaError_t launch_refine_coop(const float2* W, const double* S, int P, const double* F, int kind, double eps,
                               double lam, bool real_params, int max_corr, double tol, double* x, double* r,
                               float2* rf, double* norms, double* info, void* ctl, int* status, cudaStream_t st,
                               uint64_t wait_ns);
size_t sweep_work_elems(int P);
cudaError_t launch_spd_inverse(float2* W, int P, void* ctl, int* status, float2* work, cudaStream_t st,
                               uint64_t wait_ns = kNqWaitNs);
// many matrices in one cooperative launch (one CTA group per matrix, groups
// of total_ctas <= SMs); every job's ctl lies in ctl_base (zeroed here).
// The Hermitian fill is left to launch_herm_fill per matrix.
struct SweepJob {
  float2* W;
  int P;
  void* ctl;
  int* status;
  float2* work;
};
cudaError_t launch_spd_inverse_batch(const SweepJob* jobs, const int* cta_start, int np, int total_ctas,
                                     void* ctl_base, size_t ctl_bytes, cudaStream_t st);
cudaError_t launch_herm_fill(float2* W, int P, cudaStream_t st);
// Matrix-free conjugate-gradient solve of (S + shift) x = F for the RBM,
// S = conj(O_c) O_cᵀ / Ns applied from (σ, g, ⟨O⟩) without forming S; one
// cooperative launch (sr_cg_grid() CTAs).  shift_p = eps (kind 0),
// lam * S_pp (kind 1) or 0 (kind 2).  info = [iterations, |r| / |F|].
struct SrCgArgs {
  int N = 0, M = 0, P = 0, Ns = 0, hilb = 0, real_params = 0;
  const uint64_t* samples = nullptr;
  const float2* g = nullptr;       // [M][Ns] f'(θ)
  const double* meanO = nullptr;   // [P] complex
  const double* F = nullptr;       // [P] complex right-hand side
  double eps = 0.0, tol = 1e-4;
  int maxiter = 1000;
  double* x = nullptr;             // [P] complex solution
  double* r = nullptr;             // [P] complex work vectors
  double* pv = nullptr;
  double* w = nullptr;
  double* part = nullptr;          // [grid][P] complex adjoint partials
  double* tsum = nullptr;          // [grid] complex
  double* dots = nullptr;          // [grid][4]
  float2* t = nullptr;             // [Ns]
  double* shift = nullptr;         // [P]
  void* ctl = nullptr;             // sr_cg_ctl_bytes()
  int* status = nullptr;
  double* info = nullptr;          // [2]
  uint64_t wait_ns = kNqWaitNs;    // limit of every grid-barrier wait
  // O of the other networks (NDM family, chains): the centred O_c rows of X
  // (Re O_p at row 2p, Im O_p at row 2p + 1, FP32, row stride ldx); null
  // for the RBM, whose O is formed from (σ, g, ⟨O⟩)
  const float* X = nullptr;
  int ldx = 0;
};
int sr_cg_grid();
size_t sr_cg_ctl_bytes();
bool sr_cg_supported(int N, int M);   // the CG kernel's shared memory fits (RBM)
bool sr_cg_x_supported(int P);        // the same with O read from X
cudaError_t launch_sr_cg(const SrCgArgs& args, int kind, double lam, cudaStream_t st);

// y = -W x for the full Hermitian W
cudaError_t launch_herm_gemv_neg(const float2* W, int P, const float2* x, float2* y, cudaStream_t st);

struct SolveBufs {
  double* S = nullptr;        // [P*P] complex (input, untouched)
  float2* W = nullptr;        // [P*P] complex float: shifted S, then -(S + shift)^-1 (full Hermitian)
  float2* work = nullptr;     // sweep workspace: sweep_work_elems(P) complex floats
  double* x = nullptr;        // [P] complex solution
  double* r = nullptr;        // [P] complex residual
  float2* rf = nullptr;       // [P] complex float right-hand side of the next correction
  float2* yf = nullptr;       // [P] complex float correction
  int* status = nullptr;      // device status word
  void* ctl = nullptr;        // grid-barrier control block of the cooperative sweep
  double* norms = nullptr;    // refinement: per-CTA |y|², |x|² (refine_norm_doubles())
  double* info = nullptr;     // refinement: [corrections, |y|/|x| of the last correction]
  uint64_t wait_ns = kNqWaitNs;   // limit of every grid-barrier wait of the solve
  cudaEvent_t* ev = nullptr;  // optional [6] events: copy, inversion, fill+rhs, first solve, refinement, end
};
// shifted solve (S + shift) x = F: FP32 explicit inverse, then x_0 = A^-1 F and
// corrections x += A^-1 (F - A x) with the residual in FP64 until the
// correction, or the error it leaves, is below kRefineTol |x| (at most
// refine_iters of them);
// a pivot <= 0 sets bit 0 of status
cudaError_t launch_sr_solve(const SolveBufs& sb, int P, const double* F, int kind, double eps,
                            double lam, bool real_params, int refine_iters, cudaStream_t st);
// the two halves around the inversion, for callers that invert several matrices in one launch:
// W = S + shift; then (after the inversion) fill, x_0 and refine_iters
// correction steps (a fixed count: these kernels run inside a graph)
cudaError_t launch_sr_shift(const SolveBufs& sb, int P, int kind, double eps, double lam, cudaStream_t st);
cudaError_t launch_sr_finish(const SolveBufs& sb, int P, const double* F, int kind, double eps, double lam,
                             bool real_params, int refine_iters, cudaStream_t st);

// w[i] -= lr * dw[i*stride] on the FP64 master vector (complex parameters:
// 2P doubles, stride 1; real parameters: P doubles, stride 2 over the complex
// solution)
cudaError_t launch_descent(double* master, const double* dw, long n_doubles, int stride, double lr,
                           cudaStream_t st);
// G = X X^T from a materialised X (rows x ldx, first ns columns), FP32 CUDA cores
cudaError_t launch_gram_simt_x(const float* X, int ldx, int ns, int rows, float* G, float* partial, int ksplit,
                               cudaStream_t st);

// Measurement statistics (stats.jl:26-50) of a chains x samples matrix stored
// sample-major (value index s = chain + B*slot); mode 0: complex values,
// mode 1: |value|^2 (the Liouvillian cost).  chain_scratch:
// stats_scratch_doubles(B) doubles (5 per block of 64 chains).
constexpr size_t stats_scratch_doubles(long B) { return 5 * (size_t)((B + 63) / 64); }
template <typename R>
cudaError_t launch_stats(const cpx<R>* vals, int B, int L, int mode, double* chain_scratch,
                         double* out6, cudaStream_t st);

// bit-packed configurations <-> int8 site values (N x n column-major)
cudaError_t launch_pack_int8(const signed char* v, int nsites, long n, int hilb, uint64_t* bits,
                             cudaStream_t st);
cudaError_t launch_unpack_int8(const uint64_t* bits, int nsites, long n, int hilb, signed char* v,
                               cudaStream_t st);
// O matrix (P x n complex double, column-major) for logψ_and_∇logψ!
template <typename R>
cudaError_t launch_rbm_grad_matrix(const uint64_t* samples, int n, int N, int M, int hilb,
                                   const cpx<R>* g, double* out, cudaStream_t st);

// ---------------------------------------------------------------------------
// Grouped SR stages of the many-problem step: every stage of all problems is
// one launch.  A grouped kernel's work units (blocks, warps or elements) are
// split over the problems by a prefix array start[0..np] in device memory:
// problem p owns units [start[p], start[p+1]).
// ---------------------------------------------------------------------------
NQ_D int group_of(int unit, const int* __restrict__ start, int np) {
  int lo = 0, hi = np - 1;
  while (lo < hi) {                       // last p with start[p] <= unit
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(start + mid) <= unit) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One problem of a grouped FP32 RBM SR step: its sizes and device buffers
// (the problem handle's own, except X, which is a row slice of the batch's
// stacked X).
struct SrJob {
  int N, M, P, hilb, act, Ns, B, L, Ns_pad;
  int force_CH, force_nblk;                 // force partial sums: samples per block, blocks
  const uint64_t* samples;
  const float2* g;                          // [M][Ns] f'(θ)
  const float2* eloc;                       // [Ns]
  ForceBufs fb;
  double* chainstats;                       // stats_scratch_doubles(B)
  double* stats;                            // [6]
  float* X;                                 // [2P][Ns_pad] row slice of the stacked X
  float* Xlo;                               // 3xTF32 low part (or null)
  float* G;                                 // [2P][2P]
  double* S;                                // [P][P] complex
  float2* W;                                // shifted S, then -(S + shift)^-1
  double* x;                                // [P] complex solution
  double* r;                                // [P] complex residual
  float2* rf;                               // [P] FP32 right-hand side
  double* norms;                            // refine_norm_doubles()
  int* status;
  double* master;                           // FP64 parameters (complex)
  float* p32;                               // FP32 parameters
  float2* t0;                               // per-flip tables [N*M]
  float2* t1;
  float2* t2;
};

// Prefix arrays (device, np + 1 entries) and totals of the grouped stages.
struct SrGroup {
  int np = 0;
  const SrJob* jobs = nullptr;
  const int* force_blk = nullptr; int force_blocks = 0; size_t force_smem = 0;
  const int* force_warp = nullptr; int force_warps = 0;       // P + 1 warps per problem
  const int* pelem = nullptr; int pelems = 0;                 // P elements per problem
  const int* stat_blk = nullptr; int stat_blocks = 0;         // ceil(B / 64) blocks
  const int* x_blk = nullptr; int x_blocks = 0;               // ceil(Ns_pad / 1024) * (M + 1) blocks
  const int* pp_elem = nullptr; int pp_elems = 0;             // P * P elements
  const int* fill_blk = nullptr; int fill_blocks = 0;         // ceil(P / 32)^2 tiles
  const int* master_elem = nullptr; int master_elems = 0;     // 2P doubles
  const int* tab_elem = nullptr; int tab_elems = 0;           // N * M table entries
  int P_max = 0;                                              // largest P of the group
};
// force partial sums, their reductions and F of every problem
cudaError_t launch_force_group(const SrGroup& g, cudaStream_t st);
// FP32 force-kernel geometry of one problem: samples per block, shared memory
int rbm_force_chunk(int N, int M, int Ns);
size_t rbm_force_smem(int N, int M, int Ns);
// Measurement statistics of every problem's E_loc
cudaError_t launch_stats_group(const SrGroup& g, cudaStream_t st);
// X of every problem (TF32-rounded; Xlo when split3)
cudaError_t launch_build_X_group(const SrGroup& g, int split3, cudaStream_t st);
// S = conj(G)/Ns per problem, then the shifted copy W = S + eps I
cudaError_t launch_assemble_shift_group(const SrGroup& g, double eps, cudaStream_t st);
// Hermitian fill of every inverted W
cudaError_t launch_fill_group(const SrGroup& g, cudaStream_t st);
// FP64-residual refinement of every problem in one cooperative launch: problem
// p runs on CTAs [cta_start[p], cta_start[p+1]) with barrier block p of
// ctl_base (64 bytes each, zeroed here); max_corr corrections at most, each
// problem stopping once its correction is below kRefineTol of its solution
cudaError_t launch_refine_group(const SrGroup& g, const int* cta_start, int total_ctas, void* ctl_base,
                                double eps, int max_corr, cudaStream_t st);
// CTAs per SM of the many-problem inversion and refinement (1 or 2)
int batch_solve_ctas_per_sm();
// w -= lr Δw on the FP64 master, its FP32 copy and the per-flip tables
cudaError_t launch_update_group(const SrGroup& g, double lr, cudaStream_t st);
// G = X Xᵀ of every problem on tcgen05 from one stacked X (rows_total x Ns_pad,
// problem p's 2P_p rows starting at row_off[p]; Ns_pad equal for all).
// split3: 3xTF32 from X and Xlo.  The host plan lives in `plan` (built by
// gram_group_plan); slots: gram_group_partial_elems floats; geom: device
// buffer of gram_group_geom_bytes.  G of problem p goes to jobs[p].G.
struct GramGroupPlan {
  int np = 0, ks = 1, per = 0, nch = 0, items = 0, ncta = 0, tiles = 0;
  std::vector<int> rows, row_off, nblocks, item0, tile0;
};
GramGroupPlan gram_group_plan(const std::vector<int>& rows, int Ns_pad);
size_t gram_group_partial_elems(const GramGroupPlan& p);
size_t gram_group_geom_bytes(int np);
cudaError_t gram_group_upload(const GramGroupPlan& p, void* geom_dev, cudaStream_t st);
cudaError_t launch_gram_group(const float* X, const float* Xlo, int rows_total, int Ns_pad, int split3,
                              const GramGroupPlan& p, const void* geom_dev, const SrGroup& g, float* slots,
                              int* err, cudaStream_t st);
