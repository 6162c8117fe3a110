// Internal state of a libnqcuda handle and the helpers shared by the C-ABI
// translation units (api.cu, proposal.cu).
#pragma once
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/nqcuda.h"
#include "ndm_kernels.cuh"
#include "made_kernels.cuh"

struct MadeState;   // learned proposal (proposal.cu)

struct nq_handle {
  nq_config cfg{};
  int N = 0, M = 0, nst = 0, P = 0, B = 0, L = 0, Ns = 0, passes = 1;
  int n_record = 0, write_last = 0;
  bool doubled = false, complex_params = true, f64 = false, ndm = false;
  int Mh = 0, Ma = 0, U = 0, Ms = 0, N2 = 0;   // NDM sizes (effective units, doubled sites)
  bool chain = false;              // feed-forward chain (chain_dev)
  bool mixed = false;              // density-matrix chain over the doubled sites (Liouvillian cost)
  float2* d_cgrad = nullptr;       // density-matrix chain: conj ∇L_loc per sample, [P][Ns]
  ChainDev<float> chain_spec;      // its layers (the parameter pointer is set per precision)
  bool split = false;              // RBMSplit on the doubled-space path (complex parameters)
  bool symm = false;               // NDMSymm: trainable symmetric NDM, evaluated as its bare NDM
  bool sym_ready = false;          // NDMSymm permutations set (nq_set_symmetry)
  int n_symm = 0, sym_h = 0, sym_a = 0, P_bare = 0;   // permutations, symmetric features, bare parameters
  void* d_bare = nullptr;          // bare NDM parameters (R)
  int* d_perms = nullptr;          // [n_symm x N]
  std::vector<void*> sym_allocs;   // symmetrisation map (offsets, bare indices, coefficients)
  const int* d_sym_off = nullptr;
  const int* d_sym_idx = nullptr;
  const double* d_sym_coef = nullptr;
  bool diag = false;               // NQ_SPACE_DIAGONAL: NDM chains on the physical space, p ∝ ρ(σ,σ)
  int Md = 0;                      // diagonal sampler units (Mh + Ma)
  void* d_diag[3] = {};            // diagonal sampler network a [N], b [Md], W [Md x N] (cpx<R>)
  void* d_eff[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // C, b, a, Cs, bs (cpx<R>)
  void* d_w = nullptr;             // NDM connection weights [Ns][maxc] cpx<R>
  int* d_wconn = nullptr;          // connection ids [Ns][maxc]
  int* d_nconn = nullptr;          // connections per sample [Ns]
  int maxc = 0;
  double* d_ndm_partial = nullptr; // [nblk][2P]
  int hilb = 0, act = 0;
  cudaStream_t st = nullptr;
  // side branch of the captured step: the ket path's measurement statistics
  // run beside the force, S and solve stages (they are read only at the end)
  int* h_status = nullptr;           // pinned copy of the device status word (nq_vmc_step)
  double* h_params = nullptr;        // pinned staging of nq_set_params / nq_get_params (2P doubles)
  cudaEvent_t ev_params = nullptr;   // the last upload out of h_params
  cudaStream_t st_side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool side_ok = false, side_pending = false;     // side_ok: set by nq_vmc_step's capture only
  std::string err;
  int64_t launches = 0;

  double* d_master = nullptr;      // FP64 master parameters (complex interleaved or real)
  float* d_p32 = nullptr;          // FP32 working copy (RBM, complex)
  double* d_pexp = nullptr;        // FP64 working copy of a PositiveDefR chain (Dense form)
  bool real_sr = false;            // S, F and Δw real: real parameters, or a PositiveDefR chain
  bool time_evo = false;           // SR(time_evo=true): the solves take i F (d_frhs)
  double* d_frhs = nullptr;        // [P] complex right-hand side i F
  void* d_tab[3] = {nullptr, nullptr, nullptr};
  uint64_t* d_samples = nullptr;   // [L][B]
  unsigned long long* d_accepted = nullptr;
  uint32_t* d_call = nullptr;
  void* d_logpsi = nullptr;        // cpx<R>[Ns]
  void* d_g = nullptr;             // cpx<R>[M][Ns]
  void* d_eloc = nullptr;          // cpx<R>[Ns]
  float2* d_g32 = nullptr;         // FP32 view of g for the S stage
  ForceBufs fb;
  int force_nblk = 0;
  double* d_stats = nullptr;       // 6 doubles
  double* d_chainstats = nullptr;  // statistics block summaries, stats_scratch_doubles(B)
  float* d_G = nullptr;
  float* d_Gpart = nullptr;
  int gram_ksplit = 1;
  float* d_X = nullptr;
  float* d_Xlo = nullptr;
  int Ns_pad = 0;
  double* d_S = nullptr;
  SolveBufs sb;
  double* d_dw = nullptr;          // Δw as stored for the update (complex or real)
  DevOp op;
  bool has_op = false;
  std::vector<void*> op_allocs;

  cudaGraphExec_t graph = nullptr;
  int64_t graph_kernels = 0;
  double graph_eps = -1, graph_lr = -1;
  uint32_t* h_call = nullptr;      // pinned
  double* h_stats = nullptr;       // pinned [8]
  unsigned long long* h_acc = nullptr;
  cudaEvent_t ev[7] = {};
  cudaEvent_t kev[4] = {};
  cudaEvent_t sev[6] = {};
  float stage_ms[12] = {};
  bool capturing = false;
  int sampler_lanes = 0;           // lanes per chain chosen by the autotuner (0 = not tuned)
  int sampler_block = 0;           // threads per sampler block chosen by the autotuner
  void* d_flush = nullptr;
  size_t flush_bytes = 0;
  MadeState* made = nullptr;       // learned proposal, null until nq_proposal_init
  bool cg = false;                 // NQ_SR_CG: matrix-free iterative SR, no S
  bool exact = false;              // NQ_SAMPLER_EXACT
  int rule = 0;                    // nq_mcmc_rule
  int n_exch = 0;                  // exchange couplings / OperatorRule move classes
  int2* d_pairs = nullptr;         // [n_exch]
  void* d_xtab[3] = {};            // exchange move tables t0..t2 [n_exch*M]
  void* d_xW = nullptr;            // W_hi - W_hj [M*n_exch]
  float* d_xare = nullptr;         // [n_exch]
  OpMovesDev opm;                  // OperatorRule move set (device pointers in opm_allocs)
  std::vector<void*> opm_allocs;
  double* d_exact = nullptr;       // exact sampler: CDF and block sums
  SrCgArgs cga;                    // device work of the iterative solve
  double cg_tol = 1e-4;
  int cg_maxiter = 0;
  double* h_cginfo = nullptr;      // pinned [2]
  bool tc_theta = false;           // NQ_EVAL_TC_BF16X2 / X3: θ = Wσ + b on tcgen05
  int theta_terms = 2;             // BF16 terms of W (2 or 3)
  bool x_borrowed = false;         // d_X / d_Xlo are row slices of a batch's stacked X
  __nv_bfloat16* d_theta_img = nullptr;   // packed BF16 hi/lo image of W (density matrices: of C)
  cpx<float>* d_ndm_theta = nullptr;      // density matrices with θ on tcgen05: [U][Ns] θ of the samples
};

// Device time between two events; 0 when one of them was not recorded in the
// last call (a stage that did not run), without leaving the error behind for
// the next cudaGetLastError.
inline float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0.f;
  }
  return ms;
}

inline nq_status fail(nq_handle* h, nq_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  return code;
}

#define CK(expr)                                                                          \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess)                                                                \
      return fail(h, NQ_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                  __FILE__, __LINE__);                                                    \
  } while (0)

#define CKL(expr)       \
  do {                  \
    ++h->launches;      \
    CK(expr);           \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc((void**)p, count * sizeof(T) + 16);
}

// Sampler / table view of the network: the RBM itself, for the NDM the
// effective network of the units entering |ρ|^2 over the 2N doubled sites,
// or on the diagonal space the N-site network of ρ(σ,σ).
template <typename R>
RbmDev<R> rbm_dev(nq_handle* h) {
  RbmDev<R> d;
  d.act = h->act; d.hilb = h->hilb;
  if (h->diag) {
    d.N = h->N; d.M = h->Md; d.n_half = h->Md;
    d.a = reinterpret_cast<const cpx<R>*>(h->d_diag[0]);
    d.b = reinterpret_cast<const cpx<R>*>(h->d_diag[1]);
    d.W = reinterpret_cast<const cpx<R>*>(h->d_diag[2]);
  } else if (h->ndm) {
    d.N = h->N2; d.M = h->Ms; d.n_half = 2 * h->Mh;
    d.a = reinterpret_cast<const cpx<R>*>(h->d_eff[2]);
    d.b = reinterpret_cast<const cpx<R>*>(h->d_eff[4]);
    d.W = reinterpret_cast<const cpx<R>*>(h->d_eff[3]);
  } else {
    d.N = h->N; d.M = h->M;
    const cpx<R>* base;
    if (h->f64) base = reinterpret_cast<const cpx<R>*>(h->d_master);
    else base = reinterpret_cast<const cpx<R>*>(h->d_p32);
    d.a = base;
    d.b = base + h->N;
    d.W = base + h->N + h->M;
  }
  d.t0 = reinterpret_cast<const cpx<R>*>(h->d_tab[0]);
  d.t1 = reinterpret_cast<const cpx<R>*>(h->d_tab[1]);
  d.t2 = reinterpret_cast<const cpx<R>*>(h->d_tab[2]);
  return d;
}

// the network as the Metropolis sampler sees it: with the exchange rule the
// move tables are the couplings', with the OperatorRule the move classes'
// (the estimators keep rbm_dev's per-site tables)
template <typename R>
RbmDev<R> rbm_sampler_dev(nq_handle* h) {
  RbmDev<R> d = rbm_dev<R>(h);
  if (h->rule != NQ_RULE_LOCAL && h->n_exch > 0) {
    d.n_rows = h->n_exch;
    if (h->rule == NQ_RULE_EXCHANGE) d.pairs = h->d_pairs;
    else d.opm = &h->opm;
    d.t0 = reinterpret_cast<const cpx<R>*>(h->d_xtab[0]);
    d.t1 = reinterpret_cast<const cpx<R>*>(h->d_xtab[1]);
    d.t2 = reinterpret_cast<const cpx<R>*>(h->d_xtab[2]);
    d.rW = reinterpret_cast<const cpx<R>*>(h->d_xW);
    d.rare = reinterpret_cast<const R*>(h->d_xare);
  }
  return d;
}

// the chain's layers over the handle's current parameters (master or FP32 copy)
template <typename R>
ChainDev<R> chain_dev(nq_handle* h) {
  ChainDev<R> c;
  const ChainDev<float>& s = h->chain_spec;
  c.N = s.N; c.hilb = s.hilb; c.n_layers = s.n_layers; c.P = s.P; c.n_theta = s.n_theta; c.max_w = s.max_w;
  for (int l = 0; l < 8; ++l) c.L[l] = s.L[l];
  c.pdr = s.pdr;
  c.p = !h->f64     ? reinterpret_cast<const cpx<R>*>(h->d_p32)
        : s.pdr     ? reinterpret_cast<const cpx<R>*>(h->d_pexp)
                    : reinterpret_cast<const cpx<R>*>(h->d_master);
  return c;
}

// learned-proposal hooks used by the stage sequence (proposal.cu)
void proposal_destroy(nq_handle* h);
// launches the mixture sampler when a proposal with p_ar > 0 is attached; *used = false otherwise
nq_status proposal_sample_stage(nq_handle* h, const SamplerRun& run, bool* used);
