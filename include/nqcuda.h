/*
 * libnqcuda -- GB300 (sm_103a) engine for the variational Monte Carlo step of
 * NeuralQuantum.jl.  C ABI only: plain pointers, sizes and enums.
 *
 * The reference plugs GPU support in through Julia multiple dispatch on
 * GPUArray state types (src/GPU/Base/GPUstates.jl:1-7).  This library
 * replaces that layer with coarse-grained calls, one per stage of the
 * reference's iterative interface:
 *
 *   reference call                                        entry point here
 *   ---------------------------------------------------   --------------------
 *   BatchedSampler(net, sampler, prob, algo; batch_sz)     nq_create +
 *     (src/IterativeInterface/build_Batched.jl:1-14)         nq_set_params +
 *                                                            nq_set_operator
 *   _sample_state!(is)  (BaseIterativeSampler.jl:5-17)     nq_sample
 *     init_sampler!/samplenext! (Metropolis.jl:101-167)
 *     propose_step!(LocalRule) (LocalRuleGPU.jl:23-36)
 *   logψ!/logψ_and_∇logψ! (RBMBatched.jl:37-91,           nq_logpsi, nq_logpsi_grad
 *     NDMBatched.jl:94-280)
 *   sample!(is) minus sampling: estimator loop, stats,     nq_estimate
 *     centring, gradient, setup_algorithm!
 *     (BatchedValSampler.jl:117-139,
 *      BatchedGradSampler.jl:77-123, SRDirect.jl:26-48)
 *   precondition!(prec, SR, iter) (SRDirect.jl:51-90)      nq_precondition
 *   Optimisers.update!(Descent(η), net, Δw)                nq_update_descent
 *     (src/Optimisers/apply.jl:25-32)
 *   one full iteration of the examples' loop               nq_vmc_step
 *     (examples/ising1d.jl:32-42)
 *
 * Conventions (the reference's own, so the Julia side needs no reshaping):
 *   - parameters cross the ABI as one flat vector in the reference order
 *     (functor field order, each array column-major; src/tuple_logic.jl:31-72):
 *     RBM: a, b, W (M x N).  NDM: b_mu, h_mu, w_mu, u_mu, b_la, h_la, d_la,
 *     w_la, u_la.  RBM parameters are complex, NDM parameters real.
 *   - configurations cross the ABI as int8 site values (spin: -1/+1, Fock:
 *     0/1), N x B x L column-major (the reference's samples array); doubled
 *     (density-matrix) states are the row array followed by the column array.
 *   - complex numbers are interleaved (re, im) pairs.
 *
 * Errors: every call returns an nq_status; the message of the last failure on
 * a handle is available from nq_last_error.  No C++ exception crosses the ABI.
 * Threading: a handle is not thread-safe; distinct handles are independent
 * (each owns its CUDA stream and device buffers).
 */
#ifndef NQCUDA_H
#define NQCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NQCUDA_ABI_VERSION 1

typedef enum {
  NQ_OK = 0,
  NQ_ERR_ARG = 1,          /* invalid argument or size */
  NQ_ERR_CUDA = 2,         /* CUDA runtime error */
  NQ_ERR_NOT_PD = 3,       /* SR matrix not positive definite */
  NQ_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up */
  NQ_ERR_NAN = 5,          /* non-finite values detected */
  NQ_ERR_STATE = 6,        /* call order violated (e.g. no operator set) */
  NQ_ERR_UNSUPPORTED = 7   /* configuration outside the supported envelope */
} nq_status;

/* Networks.  NQ_NET_RBM: RBM ket (ClosedSystems/RBM.jl), complex parameters.
 * NQ_NET_NDM: purified density matrix (MixedDensityMatrix/NDM.jl), real
 * parameters, n_hidden = αN, n_ancilla = βN.  NQ_NET_RBM_SPLIT: RBMSplit
 * density matrix (MixedDensityMatrix/RBMSplit.jl), complex parameters
 * (ar, ac, b, Wr, Wc), n_hidden = αN.  NQ_NET_NDM_SYMM: NDMSymm
 * (MixedDensityMatrix/NDMSymm.jl), an NDM whose n_symm x n_hidden hidden and
 * n_symm x n_ancilla ancilla units are the permutations (nq_set_symmetry) of
 * n_hidden / n_ancilla symmetric features; the trainable parameters are the
 * symmetric NDM's (real, NDM order, sizes n_hidden and n_ancilla).  The
 * density matrices sample the doubled space (σ, η) and take the Liouvillian
 * cost function. */
typedef enum { NQ_NET_RBM = 0, NQ_NET_NDM = 1, NQ_NET_RBM_SPLIT = 2, NQ_NET_NDM_SYMM = 3, NQ_NET_CHAIN = 4,
               NQ_NET_MIXED_CHAIN = 5 } nq_network;

/* Layers of a feed-forward ket, PureStateAnsatz(Chain(layers...), N)
 * (src/Networks/Chains/Chain.jl, Layers/Dense.jl, Layers/WeightedSum.jl,
 * Layers/sum.jl).  NQ_LAYER_DENSE: y = f(W x + b), W n_out x n_in, f an
 * nq_activation; NQ_LAYER_WSUM: logψ = Σ_i c_i x_i (n_in weights);
 * NQ_LAYER_SUM: logψ = Σ_i x_i (sum_autobatch).  A chain is 1..7 Dense
 * layers (the first with n_in = n_sites, widths <= 256) closed by one WSUM or
 * SUM.  Complex parameters in the functor order: per Dense layer W
 * (column-major) then b, then c.
 * A density-matrix chain, MixedStateAnsatz(Chain(DenseSplit(N, out, f),
 * Dense..., WSum | sum_autobatch), N) (MixedDensityMatrix/MixedChainWrapper.jl,
 * Layers/DenseSplit.jl): network NQ_NET_MIXED_CHAIN, first layer
 * NQ_LAYER_DENSE_SPLIT (n_in = N, θ = Wr σ + Wc η + b on the row and column
 * configurations, parameters Wr, Wc (out x N, column-major), b), then as a
 * ket chain; it samples |ρ(σ,η)|² on the doubled space and takes the
 * Liouvillian cost function like the NDM.
 * NQ_LAYER_POSITIVE_DEF_R may open a density-matrix chain instead of
 * DenseSplit (Layers/PositiveDefR.jl, PositiveDefRBatched.jl):
 * θ = Wr (σ + η) + i Wi (σ − η) + b, parameters Wr, Wi (out x N,
 * column-major) and b, real in the reference and passed here as complex
 * values with zero imaginary part; ∇Wr = δθ (σ + η)ᵀ, ∇Wi = i δθ (σ − η)ᵀ,
 * ∇b = δθ.  With that first layer the chain's first trainable array is real,
 * so SR runs in the reference's real mode (Algorithms/SR/SRDirect.jl:11-38):
 * S = Re(O_c O_c†)/Ns, F = Re(F) (nq_estimate returns F with zero imaginary
 * parts), a real Δw, and the Descent update moves only the real parts of
 * every parameter, later complex Dense and WSum weights included. */
typedef enum { NQ_LAYER_DENSE = 0, NQ_LAYER_WSUM = 1, NQ_LAYER_SUM = 2, NQ_LAYER_DENSE_SPLIT = 3,
               NQ_LAYER_POSITIVE_DEF_R = 4 } nq_layer_kind;
typedef struct {
  int32_t kind;            /* nq_layer_kind */
  int32_t n_in;
  int32_t n_out;           /* Dense only */
  int32_t activation;      /* Dense only: nq_activation */
} nq_layer;
/* NQ_ACT_IDENTITY: Dense layers of a chain only (fwd_der(identity) = 1). */
typedef enum { NQ_ACT_LOGCOSH = 0, NQ_ACT_SOFTPLUS = 1, NQ_ACT_IDENTITY = 2 } nq_activation;
typedef enum { NQ_HILB_SPIN = 0, NQ_HILB_FOCK = 1 } nq_hilbert;
typedef enum { NQ_DTYPE_C64 = 0, NQ_DTYPE_C128 = 1, NQ_DTYPE_F32 = 2, NQ_DTYPE_F64 = 3 } nq_dtype;

/* Precision of the network evaluation (θ contraction + estimator). */
typedef enum {
  NQ_EVAL_F32 = 0,         /* FP32 CUDA cores */
  NQ_EVAL_TC_BF16X2 = 1,   /* θ = Wσ+b on tcgen05, W split in bf16 hi+lo, FP32 accumulate */
  NQ_EVAL_F64 = 2,         /* FP64 (small reference-precision runs) */
  NQ_EVAL_TC_BF16X3 = 3    /* θ on tcgen05, W split in bf16 hi+mid+lo (FP32-like θ) */
} nq_eval_precision;

/* Precision of the S = O_c O_c† accumulation. */
typedef enum {
  NQ_S_F32 = 0,            /* FP32 accuracy: 3xTF32 on tcgen05 when X and its low part fit 16 GB,
                              else FP32 CUDA cores (no X buffers) */
  NQ_S_TF32 = 1,           /* tcgen05 kind::tf32, FP32 accumulate */
  NQ_S_TF32X3 = 2,         /* tcgen05 kind::tf32 with hi/lo split (3 products) */
  NQ_S_F64 = 3,            /* FP64 CUDA cores (not provided) */
  NQ_S_BF16 = 4            /* tcgen05 kind::f16 on BF16 O (RBM): half the bytes of TF32 */
} nq_s_precision;

/* Reference quirks that can be reproduced exactly (off by default). */
#define NQ_QUIRK_STALE_LAST_SLOT 0x1u  /* BaseIterativeSampler.jl:11-16 never writes slot L */

typedef struct {
  int32_t network;         /* nq_network */
  int32_t activation;      /* nq_activation */
  int32_t hilbert;         /* nq_hilbert (local dimension 2) */
  int32_t n_sites;         /* N (physical sites) */
  int32_t n_hidden;        /* RBM: M = αN; NDM: hidden units αN */
  int32_t n_ancilla;       /* NDM: βN; ignored for the RBM */
  int32_t n_chains;        /* batch_sz: independent Metropolis chains */
  int32_t chain_length;    /* samples recorded per chain per nq_sample */
  int32_t burn;            /* burn-in sweeps */
  int32_t passes;          /* Metropolis steps per sweep (even -> +1, Metropolis.jl:30-38) */
  uint64_t seed;           /* Philox key */
  int32_t eval_precision;  /* nq_eval_precision */
  int32_t s_precision;     /* nq_s_precision */
  uint32_t quirks;         /* NQ_QUIRK_* bits */
  int32_t sampler_lanes;   /* lanes per Metropolis chain (4, 8, 16, 32); 0 = autotune */
  int32_t sr_algorithm;    /* nq_sr_algorithm */
  int32_t sampler_kind;    /* nq_sampler_kind */
  int32_t rule;            /* nq_mcmc_rule (Metropolis sampler) */
  int32_t sampler_space;   /* nq_sampler_space */
  int32_t n_symm;          /* NQ_NET_NDM_SYMM: number of permutations */
  int32_t reserved[1];
} nq_config;

/* Space the sampler draws from.  NQ_SPACE_NETWORK: the network's own space
 * (the ket's N sites; the NDM's doubled (σ, η) space, p ∝ |ρ(σ,η)|²).
 * NQ_SPACE_DIAGONAL (NDM, RBMSplit): the physical space with p(σ) ∝ ρ(σ,σ), the
 * chains of BatchedObsDMSampler(net, sampler, hilb_doubled)
 * (src/IterativeInterface/Samplers/Obs/BatchedObsDMSampler.jl:24-53, log
 * probability real(logρ(σ,σ)) of src/base_networks.jl:157).  Such a handle
 * samples N-site configurations and serves nq_sample, nq_set_samples,
 * nq_logpsi / nq_logpsi_grad (logρ(σ,σ) of N-site σ) and nq_observable;
 * the cost-function entry points (nq_set_operator, nq_estimate, SR,
 * updates, nq_vmc_step) return NQ_ERR_UNSUPPORTED. */
typedef enum { NQ_SPACE_NETWORK = 0, NQ_SPACE_DIAGONAL = 1 } nq_sampler_space;

/* Metropolis transition rule (src/Samplers/MCMCRules/).  NQ_RULE_LOCAL:
 * LocalRule, one uniformly drawn site flips (LocalRule.jl:19-28).
 * NQ_RULE_EXCHANGE: ExchangeRule(H), a uniformly drawn coupling (i, j) of the
 * couplings given by nq_set_exchange swaps its two values (ExchangeRule.jl:
 * 38-68); the total magnetisation of a chain is conserved.
 * NQ_RULE_OPERATOR: OperatorRule(Ô) (OperatorRule.jl:23-58), a uniformly drawn
 * connection of the configuration's rows in the tables of the operator given
 * by nq_set_rule_operator, accepted with the Hastings factor n(σ)/n(σ') of
 * the row lengths.  The exchange and operator rules: RBM (ket), FP32. */
typedef enum { NQ_RULE_LOCAL = 0, NQ_RULE_EXCHANGE = 1, NQ_RULE_OPERATOR = 2 } nq_mcmc_rule;

/* Sampler (src/Samplers/).  NQ_SAMPLER_METROPOLIS: the local-flip chains of
 * MetropolisSampler + LocalRule (Metropolis.jl:101-167).  NQ_SAMPLER_EXACT:
 * ExactSampler (Exact.jl:52-82, batched :133-176): the full distribution
 * over the 2^N configurations of the sampler's space (N <= 26; 2N for the
 * NDM's doubled space), its cumulative sum and inverse-CDF draws, recomputed
 * at every nq_sample; each of the n_chains x chain_length slots holds an
 * independent draw (burn and passes are not used). */
typedef enum { NQ_SAMPLER_METROPOLIS = 0, NQ_SAMPLER_EXACT = 1 } nq_sampler_kind;

/* SR solver (SR.jl:5-6 SRAlgorithm).  NQ_SR_DIRECT forms S and solves the
 * shifted system exactly (sr_cholesky); NQ_SR_CG never forms S: conjugate
 * gradients on the operator v -> conj(O_c) O_cᵀ v / Ns + shift v
 * (SRIterative.jl with SR_notfull.jl's SrMatrixC), for the reference's
 * iterative algorithms (sr_cg; sr_minres / sr_qlp / sr_lsq solve the same
 * system to the same tolerance); no P x P storage.  The RBM (FP32
 * evaluation) forms O from (σ, f'(θ)) each iteration; the other networks
 * (NDM family, feed-forward and density-matrix chains, FP32 or FP64
 * evaluation) read the centred O rows they materialise for the force, with
 * P up to 28,000. */
typedef enum { NQ_SR_DIRECT = 0, NQ_SR_CG = 1 } nq_sr_algorithm;

/* Statistics of the local estimator (src/utils/stats.jl:1-50). */
typedef struct {
  double mean_re, mean_im;
  double error;
  double variance;
  double tau;
  double R;
  double acceptance;       /* accepted / proposed Metropolis steps of the last nq_sample */
} nq_measurement;

/*
 * A flattened k-local operator (KLocalOperatorSum, or the three operator
 * lists of a KLocalLiouvillian) in the order accumulate_connections! visits
 * them (KLocalOperatorSum.jl:65-72, KLocalLiouvillian.jl:46-52).  Sites index
 * the full configuration: 0..N-1 for a ket or the row (σ) of a doubled state,
 * N..2N-1 for its column (η).  One entry per local operator o:
 *   op_n_sites[o]        number of digit sites (1..8)
 *   op_sites[8*o + i]    site of digit i (first digit least significant,
 *                        KLocalOperator.jl local_index)
 *   op_row_offset[o]     first global row of this operator
 * A left-right tensor KLocalOperatorTensor(L, conj L) is one operator whose
 * digits are its row sites followed by its column sites; its rows list the
 * products mel_l * mel_r of all pairs (KLocalOperatorTensor.jl:149-156).
 *   row_conn_offset[r]   first connection of global row r (length n_rows + 1)
 *   conn_mel[2*c]        complex matrix element (re, im)
 *   conn_n_changes[c]    number of changed sites (0..8)
 *   conn_change_site[8*c + i]   changed site (0..2N-1)
 *   conn_change_value[8*c + i]  new site value (-1/+1 or 0/1)
 */
typedef struct {
  int32_t n_ops;
  int32_t n_rows;
  int32_t n_conns;
  const int32_t* op_n_sites;
  const int32_t* op_sites;
  const int32_t* op_row_offset;
  const int32_t* row_conn_offset;
  const double* conn_mel;
  const int32_t* conn_n_changes;
  const int32_t* conn_change_site;
  const int8_t* conn_change_value;
} nq_op_table;

typedef struct nq_handle nq_handle;

/* ---- lifecycle ----------------------------------------------------------- */
const char* nq_version(void);
int32_t nq_abi_version(void);
nq_status nq_create(const nq_config* cfg, nq_handle** out);
/* A handle for PureStateAnsatz(Chain(layers...)) (cfg->network =
 * NQ_NET_CHAIN) or MixedStateAnsatz(Chain(DenseSplit, layers...))
 * (NQ_NET_MIXED_CHAIN); n_hidden, n_ancilla and activation are not used;
 * local-flip Metropolis sampler, direct SR with NQ_S_F32 / NQ_S_TF32 /
 * NQ_S_TF32X3. */
nq_status nq_create_chain(const nq_config* cfg, int32_t n_layers, const nq_layer* layers, nq_handle** out);
void nq_destroy(nq_handle* h);
nq_status nq_last_error(const nq_handle* h, char* buf, size_t len);
int64_t nq_n_params(const nq_handle* h);

/* ---- parameters: BatchedSampler(net, ...) / load_from_dict! ---------------- */
nq_status nq_set_params(nq_handle* h, const void* flat, int64_t n, int32_t dtype);
nq_status nq_get_params(nq_handle* h, void* flat, int64_t n, int32_t dtype);

/* ---- operator: the `prob` argument of BatchedSampler ----------------------- */
nq_status nq_set_operator(nq_handle* h, const nq_op_table* op);

/* ---- _sample_state!: Metropolis sampling of all chains --------------------
 * call_index selects the Philox stream of this call (the reference re-seeds
 * nothing; each call continues its MersenneTwister).  samples_out (nullable)
 * receives N x B x L (doubled: 2N x B x L) int8 values.  accept_bits (nullable,
 * testing aid) receives one byte per (step, chain), step-major. */
nq_status nq_sample(nq_handle* h, uint64_t call_index, int8_t* samples_out,
                    uint8_t* accept_bits);
/* Replace the sample buffer (N x B x L int8), e.g. to evaluate given states. */
nq_status nq_set_samples(nq_handle* h, const int8_t* samples);
/* Read the current sample buffer (N x B x L int8, doubled: 2N x B x L): the
 * samples of the last nq_sample / nq_vmc_step / batched step, or of
 * nq_set_samples.  The reference keeps them in the sampler's `samples` field
 * (BaseIterativeSampler.jl:5-17) for the user to read. */
nq_status nq_get_samples(nq_handle* h, int8_t* samples_out);
/* Read the results of the last estimate and solve on this handle without
 * recomputing anything (all outputs nullable): loc_out B x L complex128 local
 * values, force_out P values and dw_out P values (complex128, real
 * parameters float64) of the force F and the update Δw.  After a batched step
 * (nq_batch_vmc_step) they are that step's values for this problem.  The
 * reference holds the same quantities in its accumulator and SR cache
 * (BatchedValSampler.jl:117-139, SRDirect.jl:51-90). */
nq_status nq_get_estimates(nq_handle* h, double* loc_out, double* force_out, double* dw_out);

/* ---- logψ! / logψ_and_∇logψ! on arbitrary host batches --------------------
 * sigma: n configurations, int8, column-major (N x n; doubled: row block
 * 2N x n with rows 0..N-1 = σ, N..2N-1 = η).  out: n complex128.
 * grad (nullable): P x n complex128, column-major. */
nq_status nq_logpsi(nq_handle* h, const int8_t* sigma, int64_t n, double* out);
nq_status nq_logpsi_grad(nq_handle* h, const int8_t* sigma, int64_t n, double* out,
                         double* grad);

/* ---- sample!(is) after sampling -------------------------------------------
 * Evaluates logψ and ∇logψ on the sample buffer, the local estimator of the
 * operator (E_loc, or L_loc and ∇L_loc for a Liouvillian), its statistics,
 * the centred gradient, the force F and the SR matrix S.
 * loc_out (nullable): B x L complex128 local values.  force_out (nullable):
 * P complex128 (real parameters: P float64). */
nq_status nq_estimate(nq_handle* h, nq_measurement* stats, double* loc_out,
                      double* force_out);

/* ---- compute_observable(BatchedObsKetSampler, Ô)
 * (src/IterativeInterface/Samplers/Obs/BatchedObsKetSampler.jl:42-60):
 * O_loc(σ) = Σ_σ' O_σσ' ψ(σ')/ψ(σ) over the samples of the last nq_sample /
 * nq_vmc_step (same estimator kernel as E_loc, another operator table) and
 * their Measurement.  loc_out (nullable): Ns complex128, [L][B].  The
 * handle's own operator, S and F are left untouched.
 * ---- compute_observable(BatchedObsDMSampler, Ô) (BatchedObsDMSampler.jl:
 * 80-105) on an NQ_SPACE_DIAGONAL NDM handle: Ô acts on the N physical
 * sites, O_loc(σ) = Σ_σ' O_σσ' ρ(σ',σ)/ρ(σ,σ) (the connection changes the
 * row, ApplyStateChanges.jl:18-21), so that the mean is Tr(ρÔ)/Tr(ρ).  An NDM
 * handle sampling the doubled space returns NQ_ERR_UNSUPPORTED. */
nq_status nq_observable(nq_handle* h, const nq_op_table* obs, nq_measurement* stats, double* loc_out);
/* S (nullable out): P x P column-major complex128 (real parameters: float64). */
nq_status nq_get_sr_matrix(nq_handle* h, double* s_out);
/* Iterative SR settings (NQ_SR_CG): relative residual tolerance |r|/|F|
 * (SR(precision=...), default 1e-4) and the iteration cap (default 10 P as
 * SRIterative.jl:99).  nq_sr_info returns [iterations, |r|/|F|] of the last
 * iterative solve; for the direct solve (NQ_SR_DIRECT) it returns
 * [FP64-residual corrections, relative error bound] of the last
 * single-problem solve: the corrections stop once the last one, or the error
 * it leaves (|Δx_k|²/|Δx_{k-1}| while each correction shrinks the previous by
 * more than half), is below 1e-13 |x|, at most 12; the bound is the smaller of
 * the two. */
nq_status nq_set_sr_tolerance(nq_handle* h, double tol, int32_t maxiter);
nq_status nq_sr_info(nq_handle* h, double* out2);
/* SR(time_evo=true) (SR.jl:51-57; setup_algorithm! in SRDirect.jl:26-48 and
 * SRIterative.jl:32-65): the solves of this handle (nq_precondition,
 * nq_vmc_step) take α F with α = i instead of F, Re(i F) for real
 * parameters, so that Δw drives real-time evolution; on = 0 restores α = 1.
 * The force that nq_estimate and nq_get_estimates return stays ∇C. */
nq_status nq_set_time_evolution(nq_handle* h, int32_t on);
/* Limit, in nanoseconds, of every grid-barrier wait in this handle's SR solve
 * kernels (the cooperative inversion, the refinement and the conjugate
 * gradients; 0 restores the default of 1 s).  A wait that runs out ends its
 * kernel early and the call reports NQ_ERR_TIMEOUT; the handle stays usable.
 * No counterpart in the reference (its solve runs on the host). */
nq_status nq_set_wait_limit(nq_handle* h, uint64_t limit_ns);

/* ---- precondition!(prec, SR, iter) ----------------------------------------
 * kind: 0 = sr_shift (S_ii += eps), 1 = sr_multiplicative
 * (S + max(lam0*b^iter, lam_min) diag S), 2 = sr_none.  The reference's
 * Cholesky solve of S Δw = F becomes an FP32 inverse of the shifted S (block
 * Gauss–Jordan) with FP64-residual refinement iterated until the error left
 * is below 1e-13 of Δw: Δw solves the FP64 system.  dw_out (nullable)
 * receives Δw (complex128 or float64).  NQ_ERR_NOT_PD: a non-positive pivot
 * (the shifted S is not positive definite); NQ_ERR_NAN: non-finite Δw. */
nq_status nq_precondition(nq_handle* h, int32_t kind, double eps, double lam0,
                          double b, double lam_min, int32_t iter, double* dw_out);

/* ---- Optimisers.update!(Descent(lr), net, Δw): w .-= lr Δw on device ------- */
nq_status nq_update_descent(nq_handle* h, double lr);

/* ---- one full VMC iteration: sample + estimate + precondition(shift) + update.
 * Replays a captured CUDA graph after the first call. */
nq_status nq_vmc_step(nq_handle* h, uint64_t call_index, double eps, double lr,
                      nq_measurement* stats);

/* Couplings of the exchange rule: n pairs (i, j) of 0-based sites, i != j,
 * in the order ExchangeRule(H) collects them from the 2-site terms of H
 * (ExchangeRule.jl:16-35; a pair listed twice is drawn twice as often).
 * Required before sampling with rule = NQ_RULE_EXCHANGE; replaces earlier
 * couplings. */
nq_status nq_set_exchange(nq_handle* h, int32_t n, const int32_t* pairs);
/* OperatorRule(Ô): the move operator of an NQ_RULE_OPERATOR handle, flattened
 * like nq_set_operator's table (ket sites).  It needs at least one connection
 * that changes the configuration; its move classes and tables must fit the
 * sampler's shared memory (NQ_ERR_UNSUPPORTED otherwise). */
nq_status nq_set_rule_operator(nq_handle* h, const nq_op_table* op);
/* NDMSymm permutations: n_perm (= n_symm) rows of n_sites 0-based sites,
 * row j the image perm_j(i) of site i (NDMSymm.jl:114-120: bare unit
 * j + f n_symm carries the symmetric weight (f, i) on site perm_j(i)).  Required
 * before the parameters of an NQ_NET_NDM_SYMM handle take effect. */
nq_status nq_set_symmetry(nq_handle* h, int32_t n_perm, const int32_t* perms);

/* ---- timing/diagnostics ----------------------------------------------------
 * Device milliseconds of the last staged calls (CUDA events on the handle's
 * stream), 12 floats: [sample, eval+estimator, force+stats, S, solve, update,
 * sampler kernel alone, S-accumulation kernel alone, inversion of the shifted
 * S, right-hand side, first solve, FP64 refinement].  With the direct solve
 * the right-hand side, the first solve and the refinement run as one
 * cooperative launch, reported in the last entry (the two before are 0). */
nq_status nq_stage_times(nq_handle* h, float* ms12);
/* Benchmark helper: n_steps whole iterations (graph replays, call indices
 * call0, call0+1, ...); between steps, outside the timed events, a kernel
 * writes flush_bytes to evict L2.  ms_out[i] = device time of step i. */
nq_status nq_bench_steps(nq_handle* h, uint64_t call0, int32_t n_steps, double eps, double lr,
                         int64_t flush_bytes, float* ms_out);
/* Autotuned launch choices of this handle: [lanes per Metropolis chain,
 * split-K of the S accumulation, threads per sampler block].  Tunes on first
 * use. */
nq_status nq_tuning(nq_handle* h, int32_t* out, int32_t n);
/* Number of kernel launches issued by this handle since creation. */
int64_t nq_kernel_launches(const nq_handle* h);

/* ---- many independent problems per step (no counterpart in the reference) --
 * The reference runs one problem per BatchedSampler (build_Batched.jl:1-14);
 * parallel problems are separate processes or threads
 * (src/Parallel/Threads/threads_wrappers.jl:14-31).  A batch owns n problem
 * handles (RBM, FP32 evaluation, one activation and Hilbert kind; sizes may
 * differ) and runs one SR step of all of them as one CUDA graph: the
 * Metropolis sampler, the estimator and the inversion of the shifted S of
 * every problem are one launch each; the force, S, refinement and update of
 * each problem are parallel branches of the graph.  The lanes per chain of the
 * batched sampler are autotuned on the batch's own schedule.  Parameters and
 * operators are set on the problem handles (nq_batch_handle), which stay
 * usable with every single-problem call. */
typedef struct nq_batch nq_batch;
nq_status nq_batch_create(const nq_config* cfgs, int32_t n, nq_batch** out);
void nq_batch_destroy(nq_batch* b);
nq_status nq_batch_last_error(const nq_batch* b, char* buf, size_t len);
int32_t nq_batch_size(const nq_batch* b);
nq_handle* nq_batch_handle(nq_batch* b, int32_t i);
/* one SR step (sr_shift eps, Descent lr) of every problem; stats (nullable) [n] */
nq_status nq_batch_vmc_step(nq_batch* b, uint64_t call_index, double eps, double lr, nq_measurement* stats);
/* n_steps graph replays timed with CUDA events, call indices call0+1, ... */
nq_status nq_batch_bench_steps(nq_batch* b, uint64_t call0, int32_t n_steps, double eps, double lr,
                               float* ms_out);
/* [lanes per chain, estimator threads per block, inversion CTAs, kernels per step] */
nq_status nq_batch_tuning(nq_batch* b, int32_t* out, int32_t n);
int64_t nq_batch_kernel_launches(const nq_batch* b);

/* ---- learned autoregressive proposal (no counterpart in the reference) ------
 * The reference samples with local rules only (src/Samplers/MCMCRules/
 * LocalRule.jl:19-28 under Metropolis.jl:101-167).  These calls attach a MADE
 * network q(x) = Π_i p(x_i | x_<i) (N -> hidden -> hidden -> N, ReLU,
 * Bernoulli outputs; FP32 master, BF16 inference copy) to an RBM handle with
 * N <= 64.  With a mixing probability p_ar > 0, nq_sample / nq_vmc_step run
 * the mixture sampler: every step is an AR independence move with probability
 * p_ar (accepted with |ψ(x')|² q(x) / (|ψ(x)|² q(x'))), else a local flip.
 * Configurations are passed as uint64 bit strings: bit i = local index of site
 * i (spin up / occupied = 1).  Parameter order: W1 [H][N], b1 [H], W2 [H][H],
 * b2 [H], W3 [N][H], b3 [N]; autoregressive-masked entries are forced to 0. */
nq_status nq_proposal_init(nq_handle* h, int32_t hidden, double p_ar, uint64_t seed);
nq_status nq_proposal_set_mix(nq_handle* h, double p_ar);
int64_t nq_proposal_n_params(const nq_handle* h);
nq_status nq_proposal_set_params(nq_handle* h, const float* p, int64_t n);
nq_status nq_proposal_get_params(nq_handle* h, float* p, int64_t n);
/* out[k] = log q(x[k]) */
nq_status nq_proposal_logq(nq_handle* h, const uint64_t* x, int64_t n, float* out);
/* The proposals the mixture sampler would draw in sample call `call_index`:
 * for chain c and AR slot s, x_out[c*slots + s] and lq_out[c*slots + s]. */
nq_status nq_proposal_sample(nq_handle* h, uint64_t call_index, int32_t slots, uint64_t* x_out,
                             float* lq_out);
/* Masked gradient of the mean negative log-likelihood of x[0..n) (grad_out,
 * nq_proposal_n_params floats, nullable) and that mean (nll_out, nullable). */
nq_status nq_proposal_grad(nq_handle* h, const uint64_t* x, int64_t n, float* grad_out, double* nll_out);
/* `steps` Adam steps (lr) on minibatches of `batch` configurations taken in
 * order from the samples of the last sample call; nll_out (nullable) = mean
 * NLL over all those samples after training. */
nq_status nq_proposal_train(nq_handle* h, int32_t steps, int32_t batch, double lr, double* nll_out);
/* AR moves proposed and accepted during the last sample call (2 values). */
nq_status nq_proposal_stats(nq_handle* h, uint64_t* out2);

/* ---- allocation-free chain statistics (no counterpart in the reference) -----
 * The Measurement of nq_estimate (mean, error, variance, tau, R, following
 * src/utils/stats.jl:26-50) computed from local values that already sit in
 * the caller's device memory, without a handle and without allocating any
 * device memory: no cudaMalloc, cudaFree or allocating library call.  It is
 * meant for callers that cannot allocate at this point: a host program that
 * hands all device memory to its own pool allocator (CUDA.jl's pool, PyTorch's
 * caching allocator) and runs close to the memory limit, where an allocation
 * from inside the library could fail or make the pool release its cache, and
 * latency-critical loops where cudaMalloc / cudaFree would synchronise the
 * device.
 *   d_values : n_chains * chain_length complex values on the current device,
 *              value of chain c at sweep l at index l * n_chains + c
 *              (dtype NQ_DTYPE_C64 or NQ_DTYPE_C128).
 *   kind     : 0 = statistics of the values, 1 = of their squared modulus.
 *   d_out6   : 6 doubles on the current device, written with
 *              [mean_re, mean_im, error, variance, tau, R].
 *   stream   : cudaStream_t the two kernels are queued on (NULL = default);
 *              the call returns without waiting for them.
 *   err      : optional buffer for a message when the status is not NQ_OK.
 * Limit: n_chains <= NQ_NOALLOC_MAX_CHAINS.  The scratch (5 doubles per
 * block of 64 chains: 40 KiB at the limit) is one fixed device array, held
 * by every device that loads the library until the process exits, and shared
 * by every call on a device; nothing in it needs to start at zero.  Calls
 * whose kernels can overlap in time (different streams, or several host
 * threads) race on that array: order them on one stream or with events.  The
 * first call on each device (and again after the device's context was reset)
 * looks the array's address up (cudaGetSymbolAddress), which may load the
 * library's device code on that device; make that first call before any
 * stream capture begins. */
#define NQ_NOALLOC_MAX_CHAINS 65536
nq_status nq_measurement_noalloc(const void* d_values, int32_t dtype, int32_t n_chains,
                                 int32_t chain_length, int32_t kind, double* d_out6, void* stream,
                                 char* err, size_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* NQCUDA_H */
