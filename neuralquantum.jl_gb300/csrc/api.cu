// C-ABI of libnqcuda: handle lifecycle, device buffers, the stage sequence of
// one VMC iteration and its CUDA-graph replay.  See include/nqcuda.h for the
// mapping of every entry point onto the reference interface it replaces.
#include <type_traits>

#include "handle.cuh"

namespace {

// FP64-residual corrections after the first solve with the FP32 inverse; each
// gains about -log10(cond(S + shift) * 6e-8) digits
// FP64-residual corrections of the shifted solve: at most kSolveRefine in the
// single-problem cooperative refinement and at most kSolveRefineBatch in the
// grouped many-problem refinement (both stop once a correction, or the error
// it leaves, is below kRefineTol of the solution)
constexpr int kSolveRefine = 12;
// largest X + Xlo (bytes) for which an NQ_S_F32 request runs as 3xTF32 on tcgen05
constexpr double kSf32TensorBytes = 16e9;
constexpr int kSolveRefineBatch = 5;


template <typename R>
NdmEff<R> ndm_eff(nq_handle* h) {
  NdmEff<R> e;
  e.N = h->N; e.N2 = h->N2; e.Mh = h->Mh; e.Ma = h->Ma; e.U = h->U; e.P = h->P;
  e.split = h->split ? 1 : 0;
  e.sym_off = h->d_sym_off; e.sym_idx = h->d_sym_idx; e.sym_coef = h->d_sym_coef;
  e.C = reinterpret_cast<const cpx<R>*>(h->d_eff[0]);
  e.b = reinterpret_cast<const cpx<R>*>(h->d_eff[1]);
  e.a = reinterpret_cast<const cpx<R>*>(h->d_eff[2]);
  return e;
}

template <typename R>
nq_status ndm_refresh(nq_handle* h) {
  const R* p = h->f64 ? reinterpret_cast<const R*>(h->d_master) : reinterpret_cast<const R*>(h->d_p32);
  if (h->symm) {
    // NDMSymm: evaluate the bare NDM built from the symmetric parameters
    if (!h->sym_ready) return NQ_OK;
    CKL(launch_ndm_symm_bare<R>(p, h->N, h->sym_h, h->sym_a, h->n_symm, h->d_perms, (R*)h->d_bare, h->st));
    p = reinterpret_cast<const R*>(h->d_bare);
  }
  NdmEffBufs<R> b;
  b.C = (cpx<R>*)h->d_eff[0]; b.b = (cpx<R>*)h->d_eff[1]; b.a = (cpx<R>*)h->d_eff[2];
  b.Cs = (cpx<R>*)h->d_eff[3]; b.bs = (cpx<R>*)h->d_eff[4];
  if (h->split) {
    const cpx<R>* pc = reinterpret_cast<const cpx<R>*>(p);
    CKL(launch_split_effective<R>(pc, h->N, h->Ma, b, h->st));
    if (h->diag)
      CKL(launch_split_diagonal<R>(pc, h->N, h->Ma, (cpx<R>*)h->d_diag[0], (cpx<R>*)h->d_diag[1],
                                   (cpx<R>*)h->d_diag[2], h->st));
  } else {
    CKL(launch_ndm_effective<R>(ndm_view<R>(p, h->N, h->Mh, h->Ma), b, h->st));
    if (h->diag)
      CKL(launch_ndm_diagonal<R>(ndm_view<R>(p, h->N, h->Mh, h->Ma), (cpx<R>*)h->d_diag[0],
                                 (cpx<R>*)h->d_diag[1], (cpx<R>*)h->d_diag[2], h->st));
  }
  RbmDev<R> d = rbm_dev<R>(h);
  CKL(launch_rbm_tables<R>(d, (cpx<R>*)h->d_tab[0], (cpx<R>*)h->d_tab[1], (cpx<R>*)h->d_tab[2], h->st));
  if constexpr (std::is_same<R, float>::value)
    if (h->tc_theta) CKL(launch_theta_pack(b.C, h->U, h->N2, h->theta_terms, h->d_theta_img, h->st));
  return NQ_OK;
}

// refresh FP32 copies and the per-flip tables after a parameter change
nq_status refresh_params(nq_handle* h) {
  if (h->chain) {
    if (h->chain_spec.pdr)
      CKL(launch_chain_pdr_params(h->d_master, h->P, h->chain_spec.L[0].out, h->N, h->f64 ? nullptr : h->d_p32,
                                  h->f64 ? h->d_pexp : nullptr, h->st));
    else if (!h->f64) CKL(launch_master_to_f32(h->d_master, 2L * h->P, h->d_p32, h->st));
    return NQ_OK;
  }
  if (h->ndm) {
    if (h->symm) CKL(launch_ndm_symm_project(h->d_master, h->N, h->sym_h, h->sym_a, h->st));
    if (!h->f64) CKL(launch_master_to_f32(h->d_master, (h->complex_params ? 2L : 1L) * h->P, h->d_p32, h->st));
    return h->f64 ? ndm_refresh<double>(h) : ndm_refresh<float>(h);
  }
  if (!h->f64) CKL(launch_rbm_params_from_master(h->d_master, h->N, h->M, h->d_p32, h->st));
  if (h->f64) {
    RbmDev<double> d = rbm_dev<double>(h);
    CKL(launch_rbm_tables<double>(d, (cpx<double>*)h->d_tab[0], (cpx<double>*)h->d_tab[1],
                                  (cpx<double>*)h->d_tab[2], h->st));
  } else {
    RbmDev<float> d = rbm_dev<float>(h);
    CKL(launch_rbm_tables<float>(d, (cpx<float>*)h->d_tab[0], (cpx<float>*)h->d_tab[1],
                                 (cpx<float>*)h->d_tab[2], h->st));
    if (h->rule == NQ_RULE_EXCHANGE && h->n_exch > 0)
      CKL(launch_rbm_exchange_tables<float>(d, h->n_exch, h->d_pairs, (cpx<float>*)h->d_xtab[0],
                                            (cpx<float>*)h->d_xtab[1], (cpx<float>*)h->d_xtab[2],
                                            (cpx<float>*)h->d_xW, h->d_xare, h->st));
    if (h->rule == NQ_RULE_OPERATOR && h->n_exch > 0)
      CKL(launch_rbm_class_tables(d, h->opm, (cpx<float>*)h->d_xtab[0], (cpx<float>*)h->d_xtab[1],
                                  (cpx<float>*)h->d_xtab[2], (cpx<float>*)h->d_xW, h->d_xare, h->st));
    if (h->tc_theta) CKL(launch_theta_pack(d.W, h->M, h->N, h->theta_terms, h->d_theta_img, h->st));
  }
  return NQ_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: picks the lanes-per-chain of the Metropolis kernel by timing
// every instantiated candidate on a shortened schedule (a few sweeps into a
// scratch buffer) with the handle's current parameters.  Results are cached
// per (N, M, B, activation, Hilbert space, precision) for the process.
// ---------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int, int, int>, std::pair<int, int>> g_tune_cache;

// Lanes per chain and threads per block of the Metropolis sampler: every
// candidate runs a shortened schedule (up to 24 sweeps, one record) four
// times and the fastest of the last three counts.  Smaller blocks spread the
// chains more evenly over the SMs when there are few of them.
nq_status ensure_tuned(nq_handle* h) {
  if (h->exact || h->chain || (h->sampler_lanes && h->sampler_block)) return NQ_OK;
  if (h->rule == NQ_RULE_EXCHANGE && h->n_exch == 0)
    return fail(h, NQ_ERR_STATE, "exchange rule: no couplings (nq_set_exchange)");
  if (h->rule == NQ_RULE_OPERATOR && h->n_exch == 0)
    return fail(h, NQ_ERR_STATE, "operator rule: no move operator (nq_set_rule_operator)");
  const int sN = h->nst, sM = h->diag ? h->Md : (h->ndm ? h->Ms : h->M);
  const auto key = std::make_tuple(sN, sM, h->B, h->act, h->hilb,
                                   (h->f64 ? 1 : 0) + (h->ndm ? 2 : 0) + (h->diag ? 8 : 0) +
                                       (h->rule ? 16 * (h->rule + 4 * (h->n_exch + 4 * h->opm.n_ops)) : 0));
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      if (!h->sampler_lanes) h->sampler_lanes = it->second.first;
      h->sampler_block = it->second.second;
      return NQ_OK;
    }
  }
  int cand[4];
  const int rows = h->rule != NQ_RULE_LOCAL ? h->n_exch : h->nst;
  int nc = rbm_sampler_valid_lanes(rows, sM, h->f64 ? 16 : 8, cand, 4);
  if (h->rule == NQ_RULE_OPERATOR) {      // the move set shares the shared memory with the tables
    int k = 0;
    for (int c = 0; c < nc; ++c)
      if (oprule_sampler_smem(h->opm, sM, cand[c]) > 0) cand[k++] = cand[c];
    nc = k;
  }
  if (nc == 0) return fail(h, NQ_ERR_UNSUPPORTED, "no sampler instantiation for %d hidden units", sM);
  if (h->sampler_lanes) { cand[0] = h->sampler_lanes; nc = 1; }     // fixed by the caller
  const int blocks[3] = {64, 128, 256};
  uint64_t* scratch = nullptr;
  CK(cudaMalloc(&scratch, sizeof(uint64_t) * (size_t)h->B * 2));
  SamplerRun run;
  run.B = h->B; run.L = 1; run.burn = std::min(24, h->cfg.burn + h->L); run.passes = h->passes;
  run.n_record = 1; run.k0 = 0x1234u; run.k1 = 0x5678u; run.call = 0xFFFFFFFFu;
  run.samples = scratch; run.accepted = h->d_accepted;
  int best = cand[0], best_block = 256;
  float best_ms = 1e30f;
  for (int c = 0; c < nc; ++c) {
    for (int bb = 0; bb < 3; ++bb) {
      if (blocks[bb] < cand[c]) continue;
      run.block = blocks[bb];
      float best_c = 1e30f;
      for (int rep = 0; rep < 4; ++rep) {
        float ms = 0.f;
        CK(cudaEventRecord(h->kev[0], h->st));
        cudaError_t e = h->f64 ? launch_rbm_sampler<double>(rbm_sampler_dev<double>(h), run, cand[c], h->st)
                               : launch_rbm_sampler<float>(rbm_sampler_dev<float>(h), run, cand[c], h->st);
        ++h->launches;
        if (e != cudaSuccess) { cudaFree(scratch); return fail(h, NQ_ERR_CUDA, "autotune: %s", cudaGetErrorString(e)); }
        CK(cudaEventRecord(h->kev[1], h->st));
        CK(cudaEventSynchronize(h->kev[1]));
        CK(cudaEventElapsedTime(&ms, h->kev[0], h->kev[1]));
        if (rep > 0) best_c = std::min(best_c, ms);
      }
      if (best_c < best_ms) { best_ms = best_c; best = cand[c]; best_block = blocks[bb]; }
    }
  }
  cudaFree(scratch);
  h->sampler_lanes = best;
  h->sampler_block = best_block;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = std::make_pair(best, best_block);
  return NQ_OK;
}

nq_status stage_sample(nq_handle* h, uint32_t call, unsigned char* accept_bits_dev,
                       const uint32_t* call_ptr = nullptr) {
  SamplerRun run;
  run.B = h->B; run.L = h->L; run.burn = h->cfg.burn; run.passes = h->passes;
  run.n_record = h->n_record; run.write_last_at_end = h->write_last;
  run.k0 = (uint32_t)(h->cfg.seed & 0xffffffffu);
  run.k1 = (uint32_t)(h->cfg.seed >> 32);
  run.call = call;
  run.call_ptr = call_ptr;
  run.samples = h->d_samples;
  run.accepted = h->d_accepted;
  run.accept_bits = accept_bits_dev;
  run.block = h->sampler_block ? h->sampler_block : 256;
  CK(cudaMemsetAsync(h->d_accepted, 0, sizeof(unsigned long long), h->st));
  if (!h->capturing) CK(cudaEventRecord(h->kev[0], h->st));
  bool mixed = false;
  if (h->made) {
    const nq_status ms = proposal_sample_stage(h, run, &mixed);
    if (ms != NQ_OK) return ms;
  }
  if (mixed) {
  } else if (h->chain) {
    if (h->f64) CKL(launch_chain_sampler<double>(chain_dev<double>(h), run, h->st));
    else CKL(launch_chain_sampler<float>(chain_dev<float>(h), run, h->st));
  } else if (h->exact) {
    if (h->f64) CKL(launch_exact_sampler<double>(rbm_dev<double>(h), run, h->d_exact, h->st));
    else CKL(launch_exact_sampler<float>(rbm_dev<float>(h), run, h->d_exact, h->st));
  } else if (h->f64) CKL(launch_rbm_sampler<double>(rbm_sampler_dev<double>(h), run, h->sampler_lanes, h->st));
  else {
    if (h->rule != NQ_RULE_LOCAL && h->n_exch == 0)
      return fail(h, NQ_ERR_STATE, "rule without moves (nq_set_exchange / nq_set_rule_operator)");
    CKL(launch_rbm_sampler<float>(rbm_sampler_dev<float>(h), run, h->sampler_lanes, h->st));
  }
  if (!h->capturing) CK(cudaEventRecord(h->kev[1], h->st));
  return NQ_OK;
}

// θ of the sample buffer's doubled configurations on tcgen05 (density
// matrices with NQ_EVAL_TC_BF16X2 / X3), read by the evaluation, estimator and
// gradient kernels instead of forming θ on CUDA cores
template <typename R>
nq_status ndm_tc_theta(nq_handle* h, NdmEff<R>* e) {
  if constexpr (std::is_same<R, float>::value) {
    if (!h->tc_theta) return NQ_OK;
    CKL(launch_theta_bf16x2(h->d_theta_img, h->theta_terms, h->U, h->N2, e->b, h->d_samples, h->Ns, h->hilb,
                            h->d_ndm_theta, h->sb.status, h->st));
    e->theta = h->d_ndm_theta;
  }
  return NQ_OK;
}

template <typename R>
nq_status ndm_stage_eval(nq_handle* h) {
  NdmEff<R> e = ndm_eff<R>(h);
  if (nq_status s = ndm_tc_theta<R>(h, &e)) return s;
  const int sp = h->cfg.s_precision;
  const bool tc = sp == NQ_S_TF32 || sp == NQ_S_TF32X3;
  CKL(launch_ndm_eval<R>(e, h->act, h->d_samples, h->Ns, h->hilb, (cpx<R>*)h->d_logpsi, h->d_X, h->Ns_pad,
                         nullptr, h->st));
  CKL(launch_x_center(h->d_X, sp == NQ_S_TF32X3 ? h->d_Xlo : nullptr, 2 * h->P, h->Ns_pad, h->Ns, h->fb.meanO,
                      tc ? 1 : 0, h->st));
  CKL(launch_ndm_loc<R>(e, h->act, h->op, h->d_samples, h->Ns, h->hilb, h->maxc, (cpx<R>*)h->d_eloc,
                        (cpx<R>*)h->d_w, h->d_wconn, h->d_nconn, h->st));
  return NQ_OK;
}

nq_status stage_eval(nq_handle* h) {
  if (h->ndm) return h->f64 ? ndm_stage_eval<double>(h) : ndm_stage_eval<float>(h);
  if (h->chain) {
    // logψ, E_loc and the uncentred O rows of X (centred after the force)
    if (h->f64)
      CKL(launch_chain_eval<double>(chain_dev<double>(h), h->d_samples, h->Ns, &h->op, (cpx<double>*)h->d_logpsi,
                                    (cpx<double>*)h->d_eloc, h->d_X, h->Ns_pad, nullptr, h->st));
    else
      CKL(launch_chain_eval<float>(chain_dev<float>(h), h->d_samples, h->Ns, &h->op, (cpx<float>*)h->d_logpsi,
                                   (cpx<float>*)h->d_eloc, h->d_X, h->Ns_pad, nullptr, h->st));
    return NQ_OK;
  }
  const DevOp* op = h->has_op ? &h->op : nullptr;
  if (h->f64) {
    CKL(launch_rbm_eval<double>(rbm_dev<double>(h), h->d_samples, h->Ns, op, (cpx<double>*)h->d_logpsi,
                                (cpx<double>*)h->d_g, (cpx<double>*)h->d_eloc, h->st));
  } else if (h->tc_theta) {
    const RbmDev<float> d = rbm_dev<float>(h);
    CKL(launch_theta_bf16x2(h->d_theta_img, h->theta_terms, h->M, h->N, d.b, h->d_samples, h->Ns, h->hilb, (cpx<float>*)h->d_g,
                            h->sb.status, h->st));
    CKL(launch_rbm_eval<float>(d, h->d_samples, h->Ns, op, (cpx<float>*)h->d_logpsi, (cpx<float>*)h->d_g,
                               (cpx<float>*)h->d_eloc, h->st, 1));
  } else {
    CKL(launch_rbm_eval<float>(rbm_dev<float>(h), h->d_samples, h->Ns, op, (cpx<float>*)h->d_logpsi,
                               (cpx<float>*)h->d_g, (cpx<float>*)h->d_eloc, h->st));
  }
  return NQ_OK;
}

__global__ void g64_to_32_kernel(const double* g, long n, float2* out) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float2((float)g[2 * i], (float)g[2 * i + 1]);
}

template <typename R>
nq_status ndm_stage_force(nq_handle* h) {
  // cost C = mean |L_loc|^2 with its statistics, then F (θ of the samples from
  // the evaluation stage when it ran on tcgen05)
  NdmEff<R> e = ndm_eff<R>(h);
  if constexpr (std::is_same<R, float>::value)
    if (h->tc_theta) e.theta = h->d_ndm_theta;
  CKL(launch_stats<R>((cpx<R>*)h->d_eloc, h->B, h->L, 1, h->d_chainstats, h->d_stats, h->st));
  CKL(launch_ndm_grad<R>(e, h->act, h->op, h->d_samples, h->Ns, h->hilb, h->maxc,
                         (const cpx<R>*)h->d_eloc, (const cpx<R>*)h->d_w, h->d_wconn, h->d_nconn,
                         h->d_ndm_partial, h->fb.meanO, h->d_stats, h->fb.force, h->st));
  return NQ_OK;
}

nq_status stage_force(nq_handle* h) {
  if (h->ndm) return h->f64 ? ndm_stage_force<double>(h) : ndm_stage_force<float>(h);
  if (h->chain) {
    const int sp = h->cfg.s_precision;
    const bool tc = sp == NQ_S_TF32 || sp == NQ_S_TF32X3;
    if (h->mixed) {
      // density matrix: the cost C = mean |L_loc|² with its statistics, then F
      if (h->f64) {
        CKL(launch_stats<double>((cpx<double>*)h->d_eloc, h->B, h->L, 1, h->d_chainstats, h->d_stats, h->st));
        CKL(launch_chain_liouv_force<double>(chain_dev<double>(h), h->d_samples, h->Ns, h->op,
                                             (const cpx<double>*)h->d_eloc, h->d_X, h->Ns_pad, h->d_stats,
                                             h->d_cgrad, h->fb.force, h->st));
      } else {
        CKL(launch_stats<float>((cpx<float>*)h->d_eloc, h->B, h->L, 1, h->d_chainstats, h->d_stats, h->st));
        CKL(launch_chain_liouv_force<float>(chain_dev<float>(h), h->d_samples, h->Ns, h->op,
                                            (const cpx<float>*)h->d_eloc, h->d_X, h->Ns_pad, h->d_stats,
                                            h->d_cgrad, h->fb.force, h->st));
      }
    } else if (h->f64) {
      CKL(launch_stats<double>((cpx<double>*)h->d_eloc, h->B, h->L, 0, h->d_chainstats, h->d_stats, h->st));
      CKL(launch_chain_force<double>(h->d_X, h->Ns_pad, h->P, h->Ns, (const cpx<double>*)h->d_eloc, h->d_stats,
                                     h->fb.force, h->st));
    } else {
      CKL(launch_stats<float>((cpx<float>*)h->d_eloc, h->B, h->L, 0, h->d_chainstats, h->d_stats, h->st));
      CKL(launch_chain_force<float>(h->d_X, h->Ns_pad, h->P, h->Ns, (const cpx<float>*)h->d_eloc, h->d_stats,
                                    h->fb.force, h->st));
    }
    CKL(launch_x_center(h->d_X, sp == NQ_S_TF32X3 ? h->d_Xlo : nullptr, 2 * h->P, h->Ns_pad, h->Ns, h->fb.meanO,
                        tc ? 1 : 0, h->st));
    return NQ_OK;
  }
  // the statistics of E_loc feed only the step's measurement: inside the
  // captured step they run on the side branch, joined at its end
  const bool side = h->capturing && h->side_ok && h->st_side;
  cudaStream_t sst = side ? h->st_side : h->st;
  if (side) {
    CK(cudaEventRecord(h->ev_fork, h->st));
    CK(cudaStreamWaitEvent(h->st_side, h->ev_fork, 0));
  }
  if (h->f64) {
    CKL(launch_stats<double>((cpx<double>*)h->d_eloc, h->B, h->L, 0, h->d_chainstats, h->d_stats, sst));
    CKL(launch_rbm_force<double>(rbm_dev<double>(h), h->d_samples, h->Ns, (cpx<double>*)h->d_g,
                                 (cpx<double>*)h->d_eloc, h->fb, h->st));
  } else {
    CKL(launch_stats<float>((cpx<float>*)h->d_eloc, h->B, h->L, 0, h->d_chainstats, h->d_stats, sst));
    CKL(launch_rbm_force<float>(rbm_dev<float>(h), h->d_samples, h->Ns, (cpx<float>*)h->d_g,
                                (cpx<float>*)h->d_eloc, h->fb, h->st));
  }
  if (side) {
    CK(cudaEventRecord(h->ev_join, h->st_side));
    h->side_pending = true;
  }
  return NQ_OK;
}

nq_status stage_S(nq_handle* h) {
  if (h->cg) return NQ_OK;          // matrix-free SR: S is never formed
  if (h->ndm || h->chain) {
    const int sp = h->cfg.s_precision;
    if (!h->capturing) CK(cudaEventRecord(h->kev[2], h->st));
    if (sp == NQ_S_TF32 || sp == NQ_S_TF32X3) {
      CKL(launch_gram_tc(h->d_X, h->d_Xlo, 2 * h->P, h->Ns_pad, sp == NQ_S_TF32X3 ? 1 : 0, h->d_G, h->d_Gpart,
                         h->sb.status, h->st));
    } else {
      CKL(launch_gram_simt_x(h->d_X, h->Ns_pad, h->Ns, 2 * h->P, h->d_G, h->d_Gpart, h->gram_ksplit, h->st));
    }
    if (!h->capturing) CK(cudaEventRecord(h->kev[3], h->st));
    CKL(launch_assemble_S(h->d_G, h->P, 1.0 / h->Ns, h->real_sr, h->d_S, h->st));
    return NQ_OK;
  }
  RbmOSource src;
  src.N = h->N; src.M = h->M; src.hilb = h->hilb; src.Ns = h->Ns;
  src.samples = h->d_samples;
  if (h->f64) {
    long n = (long)h->M * h->Ns;
    ++h->launches;
    g64_to_32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, h->st>>>((const double*)h->d_g, n, h->d_g32);
    CK(cudaGetLastError());
    src.g = h->d_g32;
  } else {
    src.g = reinterpret_cast<const float2*>(h->d_g);
  }
  src.meanO = h->fb.meanO;
  const int sp = h->cfg.s_precision;
  if (sp == NQ_S_TF32 || sp == NQ_S_TF32X3 || sp == NQ_S_BF16) {
    const int bf16 = sp == NQ_S_BF16 ? 1 : 0;
    CKL(launch_build_X(src, h->P, h->Ns_pad, h->d_X, sp == NQ_S_TF32X3 ? h->d_Xlo : nullptr, h->st, bf16));
    if (!h->capturing) CK(cudaEventRecord(h->kev[2], h->st));
    CKL(launch_gram_tc(h->d_X, h->d_Xlo, 2 * h->P, h->Ns_pad, sp == NQ_S_TF32X3 ? 1 : 0, h->d_G, h->d_Gpart,
                       h->sb.status, h->st, bf16));
    if (!h->capturing) CK(cudaEventRecord(h->kev[3], h->st));
  } else {
    if (!h->capturing) CK(cudaEventRecord(h->kev[2], h->st));
    CKL(launch_gram_simt(src, h->P, h->d_G, h->d_Gpart, h->gram_ksplit, h->st));
    if (!h->capturing) CK(cudaEventRecord(h->kev[3], h->st));
  }
  CKL(launch_assemble_S(h->d_G, h->P, 1.0 / h->Ns, h->real_sr, h->d_S, h->st));
  return NQ_OK;
}

nq_status stage_solve(nq_handle* h, int kind, double eps, double lam) {
  // SR(time_evo=true): α F with α = i (SRDirect.jl:27, SRIterative.jl:33)
  const double* F = h->fb.force;
  if (h->time_evo) {
    CKL(launch_times_i(h->fb.force, h->P, h->d_frhs, h->st));
    ++h->launches;
    F = h->d_frhs;
  }
  if (h->cg) {
    SrCgArgs a = h->cga;
    a.F = F;
    a.eps = eps;
    a.tol = h->cg_tol;
    a.maxiter = h->cg_maxiter;
    a.real_params = h->real_sr ? 1 : 0;
    if (!h->capturing) CK(cudaEventRecord(h->sev[0], h->st));
    CKL(launch_sr_cg(a, kind, lam, h->st));
    ++h->launches;
    if (!h->capturing) {
      for (int k = 1; k < 6; ++k) CK(cudaEventRecord(h->sev[k], h->st));
    }
    return NQ_OK;
  }
  SolveBufs sb = h->sb;
  sb.ev = h->capturing ? nullptr : h->sev;
  CKL(launch_sr_solve(sb, h->P, F, kind, eps, lam, h->real_sr, kSolveRefine, h->st));
  h->launches += 8;
  return NQ_OK;
}

nq_status stage_update(nq_handle* h, double lr) {
  const long nd = h->complex_params ? 2L * h->P : h->P;
  CKL(launch_descent(h->d_master, h->sb.x, nd, h->complex_params ? 1 : 2, lr, h->st));
  return refresh_params(h);
}

// st_read: the status word already copied to the host after the last
// synchronisation (nq_vmc_step reads it with the measurement), else null
nq_status check_status_word(nq_handle* h, const int* st_read = nullptr) {
  int st = 0;
  if (st_read) {
    st = *st_read;
  } else {
    CK(cudaMemcpyAsync(&st, h->sb.status, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  if (st != 0) {
    CK(cudaMemsetAsync(h->sb.status, 0, sizeof(int), h->st));
    CK(cudaStreamSynchronize(h->st));
    if (st & NQ_DEVERR_TIMEOUT) return fail(h, NQ_ERR_TIMEOUT, "a bounded device-side wait gave up (status 0x%x)", st);
    if (st & 1) return fail(h, NQ_ERR_NOT_PD, "SR matrix is not positive definite after the diagonal shift");
    if (st & NQ_DEVERR_NONFINITE) return fail(h, NQ_ERR_NAN, "the SR solve produced a non-finite update");
    return fail(h, NQ_ERR_CUDA, "device status word 0x%x", st);
  }
  return NQ_OK;
}

void fill_measurement(nq_handle* h, nq_measurement* m) {
  if (!m) return;
  m->mean_re = h->h_stats[0];
  m->mean_im = h->h_stats[1];
  m->error = h->h_stats[2];
  m->variance = h->h_stats[3];
  m->tau = h->h_stats[4];
  m->R = h->h_stats[5];
  double steps = (double)h->B * h->passes * (h->cfg.burn + h->n_record);
  m->acceptance = steps > 0 ? (double)(*h->h_acc) / steps : 0.0;
}

void free_rule_operator(nq_handle* h) {
  for (void* p : h->opm_allocs) cudaFree(p);
  h->opm_allocs.clear();
  h->opm = OpMovesDev();
}

void free_op(nq_handle* h) {
  for (void* p : h->op_allocs) cudaFree(p);
  h->op_allocs.clear();
  h->has_op = false;
  h->op = DevOp();
}

template <typename T>
nq_status upload(nq_handle* h, const T* src, size_t count, const T** dst, std::vector<void*>* allocs = nullptr) {
  if (count == 0) count = 1;
  T* d = nullptr;
  CK(cudaMalloc((void**)&d, count * sizeof(T)));
  (allocs ? allocs : &h->op_allocs)->push_back(d);
  if (src) CK(cudaMemcpy(d, src, count * sizeof(T), cudaMemcpyHostToDevice));
  *dst = d;
  return NQ_OK;
}

// host-side validation of a flattened operator against the handle's sites
nq_status validate_op(nq_handle* h, const nq_op_table* t) {
  if (t->n_ops < 1 || t->n_rows < 1 || t->n_conns < 0) return fail(h, NQ_ERR_ARG, "empty operator");
  for (int o = 0; o < t->n_ops; ++o) {
    int k = t->op_n_sites[o];
    if (k < 1 || k > 8) return fail(h, NQ_ERR_ARG, "operator %d: %d sites (1..8 supported)", o, k);
    for (int d = 0; d < k; ++d)
      if (t->op_sites[8 * o + d] < 0 || t->op_sites[8 * o + d] >= h->nst)
        return fail(h, NQ_ERR_ARG, "operator %d: site out of range", o);
    if (t->op_row_offset[o] < 0 || t->op_row_offset[o] + (1 << k) > t->n_rows)
      return fail(h, NQ_ERR_ARG, "operator %d: row offset out of range", o);
  }
  for (int r = 0; r < t->n_rows; ++r)
    if (t->row_conn_offset[r] > t->row_conn_offset[r + 1] || t->row_conn_offset[r] < 0)
      return fail(h, NQ_ERR_ARG, "row offsets not monotone");
  if (t->row_conn_offset[t->n_rows] != t->n_conns) return fail(h, NQ_ERR_ARG, "row offsets do not end at n_conns");
  for (int c = 0; c < t->n_conns; ++c) {
    int nc = t->conn_n_changes[c];
    if (nc < 0 || nc > 8) return fail(h, NQ_ERR_ARG, "connection %d: bad change count", c);
    for (int q = 0; q < nc; ++q) {
      int s = t->conn_change_site[8 * c + q];
      int v = t->conn_change_value[8 * c + q];
      if (s < 0 || s >= h->nst) return fail(h, NQ_ERR_ARG, "connection %d: site out of range", c);
      bool ok = h->hilb == NQ_HILB_SPIN ? (v == 1 || v == -1) : (v == 0 || v == 1);
      if (!ok) return fail(h, NQ_ERR_ARG, "connection %d: invalid site value %d", c, v);
    }
  }
  return NQ_OK;
}

nq_status upload_op(nq_handle* h, const nq_op_table* t, DevOp* out, std::vector<void*>* allocs) {
  DevOp d;
  d.n_ops = t->n_ops; d.n_rows = t->n_rows; d.n_conns = t->n_conns;
  nq_status s;
  if ((s = upload(h, t->op_n_sites, t->n_ops, &d.op_n_sites, allocs)) != NQ_OK) return s;
  if ((s = upload(h, t->op_sites, 8 * (size_t)t->n_ops, &d.op_sites, allocs)) != NQ_OK) return s;
  if ((s = upload(h, t->op_row_offset, t->n_ops, &d.op_row_offset, allocs)) != NQ_OK) return s;
  if ((s = upload(h, t->row_conn_offset, (size_t)t->n_rows + 1, &d.row_conn_offset, allocs)) != NQ_OK) return s;
  if ((s = upload(h, t->conn_mel, 2 * (size_t)t->n_conns, &d.conn_mel, allocs)) != NQ_OK) return s;
  {
    std::vector<float2> mf(std::max(1, t->n_conns));
    std::vector<int4> cp(std::max(1, t->n_conns));
    for (int c = 0; c < t->n_conns; ++c) {
      mf[c] = make_float2((float)t->conn_mel[2 * c], (float)t->conn_mel[2 * c + 1]);
      int4 q;
      memcpy(&q.x, &mf[c].x, 4);
      memcpy(&q.y, &mf[c].y, 4);
      q.z = t->conn_n_changes[c];
      q.w = q.z > 0 ? ((t->conn_change_site[8 * c] & 0xff) | ((int)(unsigned char)t->conn_change_value[8 * c] << 8))
                    : 0;
      cp[c] = q;
    }
    if ((s = upload(h, (const float2*)mf.data(), mf.size(), &d.conn_mel_f, allocs)) != NQ_OK) return s;
    if ((s = upload(h, (const int4*)cp.data(), cp.size(), &d.conn_pack, allocs)) != NQ_OK) return s;
    std::vector<int4> om(std::max(1, t->n_ops));
    for (int o = 0; o < t->n_ops; ++o) {
      int lo = 0, hi = 0;
      for (int k = 0; k < t->op_n_sites[o]; ++k) {
        const int site = t->op_sites[8 * o + k] & 0xff;
        if (k < 4) lo |= site << (8 * k);
        else hi |= site << (8 * (k - 4));
      }
      om[o] = make_int4(t->op_n_sites[o], t->op_row_offset[o], lo, hi);
    }
    if ((s = upload(h, (const int4*)om.data(), om.size(), &d.op_meta, allocs)) != NQ_OK) return s;
  }
  if ((s = upload(h, t->conn_n_changes, (size_t)t->n_conns, &d.conn_n_changes, allocs)) != NQ_OK) return s;
  if ((s = upload(h, t->conn_change_site, 8 * (size_t)t->n_conns, &d.conn_change_site, allocs)) != NQ_OK) return s;
  if ((s = upload(h, (const signed char*)t->conn_change_value, 8 * (size_t)t->n_conns, &d.conn_change_value,
                  allocs)) != NQ_OK)
    return s;
  *out = d;
  return NQ_OK;
}

}  // namespace

// entry points of the cost function and the optimiser are not defined on a
// handle that samples the diagonal of the density matrix
#define NQ_REJECT_DIAG(h, what)                                                                           \
  do {                                                                                                    \
    if ((h)->diag)                                                                                        \
      return fail((h), NQ_ERR_UNSUPPORTED, "%s: the handle samples the diagonal space (observables only)", \
                  what);                                                                                  \
  } while (0)

// =============================== C ABI ======================================
extern "C" {

const char* nq_version(void) { return "libnqcuda 0.1.0 (sm_103a)"; }
int32_t nq_abi_version(void) { return NQCUDA_ABI_VERSION; }

}  // extern "C"

namespace {

// validated layer list of a chain into spec; "" or the reason it is refused
// A density-matrix chain's DenseSplit layer (θ = Wr σ + Wc η + b) is stored
// as a Dense layer on the 2N doubled sites: W = [Wr Wc] column-major is Wr
// then Wc, so the parameter vector is unchanged.  A PositiveDefR first layer
// (Wr, Wi, b) has the same sizes and runs as that Dense layer with
// W = [Wr + i Wi, Wr − i Wi] (spec->pdr).
const char* chain_layers(const nq_config& c, int n_layers, const nq_layer* layers, ChainDev<float>* spec) {
  if (!layers || n_layers < 2 || n_layers > 8) return "a chain has 2..8 layers";
  const bool mixed = c.network == NQ_NET_MIXED_CHAIN;
  int off = 0, n_theta = 0, max_w = 0, prev = c.n_sites;
  for (int l = 0; l < n_layers; ++l) {
    const nq_layer& y = layers[l];
    ChainLayerDev d;
    d.kind = y.kind; d.in = y.n_in; d.out = y.n_out; d.act = y.activation;
    if (y.n_in != prev) return "layer input width differs from the previous output";
    const bool split = y.kind == NQ_LAYER_DENSE_SPLIT || y.kind == NQ_LAYER_POSITIVE_DEF_R;
    if (mixed != (l == 0 && split) && l == 0)
      return mixed ? "a density-matrix chain starts with DenseSplit or PositiveDefR"
                   : "DenseSplit and PositiveDefR start a density-matrix chain";
    if (l > 0 && split) return "DenseSplit and PositiveDefR are the first layer only";
    const bool dense = y.kind == NQ_LAYER_DENSE || split;
    if (split) {
      d.kind = NQ_LAYER_DENSE;
      d.in = 2 * y.n_in;
      spec->pdr = y.kind == NQ_LAYER_POSITIVE_DEF_R ? 1 : 0;
    }
    const bool closing = l == n_layers - 1;
    if (closing != !dense) return "Dense layers, then exactly one closing WSum or sum";
    if (dense) {
      if (y.n_out < 1 || y.n_out > 256) return "Dense widths must be in 1..256";
      if (y.activation != NQ_ACT_LOGCOSH && y.activation != NQ_ACT_SOFTPLUS && y.activation != NQ_ACT_IDENTITY)
        return "unknown Dense activation";
      d.w_off = off; off += y.n_out * d.in;
      d.b_off = off; off += y.n_out;
      n_theta += y.n_out;
      max_w = std::max(max_w, y.n_out);
      prev = y.n_out;
    } else if (y.kind == NQ_LAYER_WSUM) {
      d.w_off = off; off += y.n_in;
      d.out = 1;
    } else if (y.kind == NQ_LAYER_SUM) {
      d.out = 1;
    } else {
      return "unknown layer kind";
    }
    spec->L[l] = d;
  }
  spec->N = mixed ? 2 * c.n_sites : c.n_sites;
  spec->hilb = c.hilbert; spec->n_layers = n_layers; spec->P = off;
  spec->n_theta = n_theta; spec->max_w = max_w;
  if (off > 256 * 24) return "too many chain parameters (max 6144)";
  return "";
}

nq_status create_impl(const nq_config* cfg, int n_layers, const nq_layer* layers, nq_handle** out) {
  if (!cfg || !out) return NQ_ERR_ARG;
  *out = nullptr;
  nq_handle* h = new nq_handle();
  h->cfg = *cfg;
  const nq_config& c = *cfg;
  auto bad = [&](const char* msg) {
    fprintf(stderr, "nq_create: %s\n", msg);
    delete h;
    return NQ_ERR_ARG;
  };
  if (c.network == NQ_NET_CHAIN || c.network == NQ_NET_MIXED_CHAIN) {
    if (!layers) return bad("chains are created with nq_create_chain");
    if (c.n_sites < 1 || c.n_sites > (c.network == NQ_NET_MIXED_CHAIN ? 32 : 64))
      return bad("n_sites must be in 1..64 (1..32 for a density-matrix chain)");
    const char* why = chain_layers(c, n_layers, layers, &h->chain_spec);
    if (*why) return bad(why);
    if (c.sampler_kind != NQ_SAMPLER_METROPOLIS || c.rule != NQ_RULE_LOCAL || c.sampler_space != NQ_SPACE_NETWORK)
      return bad("chains sample with the local-flip Metropolis rule");
    h->chain = true;
    h->mixed = c.network == NQ_NET_MIXED_CHAIN;
  }
  if (c.network != NQ_NET_RBM && c.network != NQ_NET_NDM && c.network != NQ_NET_RBM_SPLIT &&
      c.network != NQ_NET_NDM_SYMM && c.network != NQ_NET_CHAIN && c.network != NQ_NET_MIXED_CHAIN)
    return bad("unknown network");
  const bool matrix_net = c.network == NQ_NET_NDM || c.network == NQ_NET_RBM_SPLIT || c.network == NQ_NET_NDM_SYMM;
  if (c.network == NQ_NET_NDM_SYMM && (c.n_symm < 1 || c.n_symm > 64)) return bad("NDMSymm: n_symm must be in 1..64");
  if (!h->chain && c.activation != NQ_ACT_LOGCOSH && c.activation != NQ_ACT_SOFTPLUS) return bad("unknown activation");
  if (c.hilbert != NQ_HILB_SPIN && c.hilbert != NQ_HILB_FOCK) return bad("unknown hilbert space");
  if (c.n_sites < 1 || c.n_sites > 64) return bad("n_sites must be in 1..64");
  if (!h->chain && (c.n_hidden < 1 || c.n_hidden > 256)) return bad("n_hidden must be in 1..256");
  if (c.n_chains < 2 || c.chain_length < 1 || c.burn < 0 || c.passes < 1) return bad("bad sampler sizes");
  if (c.eval_precision != NQ_EVAL_F32 && c.eval_precision != NQ_EVAL_F64) {
    // θ on tcgen05: the RBM ket (θ = Wσ + b), and the density matrices on the
    // doubled space (the units of their effective network, θ_u = b_u + C_u·(σ, η))
    const bool tc = c.eval_precision == NQ_EVAL_TC_BF16X2 || c.eval_precision == NQ_EVAL_TC_BF16X3;
    const int eff_units = c.network == NQ_NET_RBM_SPLIT ? c.n_hidden
                          : 4 * c.n_hidden * (c.network == NQ_NET_NDM_SYMM ? std::max(1, c.n_symm) : 1) +
                                c.n_ancilla * (c.network == NQ_NET_NDM_SYMM ? std::max(1, c.n_symm) : 1);
    const bool ok = tc && gram_tc_supported() &&
                    ((c.network == NQ_NET_RBM && theta_tc_supported(c.n_sites, c.n_hidden)) ||
                     (matrix_net && c.sampler_space == NQ_SPACE_NETWORK &&
                      theta_tc_supported(2 * c.n_sites, eff_units)));
    if (!ok) {
      delete h;
      return NQ_ERR_UNSUPPORTED;
    }
  }
  if (c.s_precision == NQ_S_F64) { delete h; return NQ_ERR_UNSUPPORTED; }
  if (c.sr_algorithm != NQ_SR_DIRECT && c.sr_algorithm != NQ_SR_CG) return bad("unknown sr_algorithm");
  if (c.sampler_kind != NQ_SAMPLER_METROPOLIS && c.sampler_kind != NQ_SAMPLER_EXACT) return bad("unknown sampler_kind");
  if (c.rule != NQ_RULE_LOCAL && c.rule != NQ_RULE_EXCHANGE && c.rule != NQ_RULE_OPERATOR) return bad("unknown rule");
  if (c.rule != NQ_RULE_LOCAL && (c.network != NQ_NET_RBM || c.eval_precision == NQ_EVAL_F64))
    return bad("the exchange and operator rules are available for FP32 RBM handles");
  if (c.sampler_space != NQ_SPACE_NETWORK && c.sampler_space != NQ_SPACE_DIAGONAL) return bad("unknown sampler_space");
  if (c.sampler_space == NQ_SPACE_DIAGONAL && !matrix_net)
    return bad("the diagonal sampler space is defined for density-matrix networks (NDM, RBMSplit)");
  if (c.sampler_kind == NQ_SAMPLER_EXACT &&
      (matrix_net && c.sampler_space == NQ_SPACE_NETWORK ? 2 * c.n_sites : c.n_sites) > 26)
    return bad("the exact sampler enumerates 2^N configurations: N (2N for the NDM's doubled space) <= 26");
  // matrix-free SR: the RBM forms O from (σ, g) in FP32 evaluation; the other
  // networks read the centred O rows of X (size checked once P is known)
  if (c.sr_algorithm == NQ_SR_CG && c.network == NQ_NET_RBM &&
      (c.eval_precision == NQ_EVAL_F64 || !sr_cg_supported(c.n_sites, c.n_hidden))) {
    delete h;
    return NQ_ERR_UNSUPPORTED;
  }
  if ((c.s_precision == NQ_S_TF32 || c.s_precision == NQ_S_TF32X3 || c.s_precision == NQ_S_BF16) &&
      !gram_tc_supported()) {
    delete h;
    return NQ_ERR_UNSUPPORTED;
  }
  if (c.s_precision == NQ_S_BF16 && c.network != NQ_NET_RBM) { delete h; return NQ_ERR_UNSUPPORTED; }
  if (c.s_precision < NQ_S_F32 || c.s_precision > NQ_S_BF16) return bad("unknown s_precision");
  h->N = c.n_sites;
  h->M = c.n_hidden;
  if (matrix_net) {
    // density-matrix networks share the doubled-space path; RBMSplit is its
    // effective form with M units of weight 1 (Mh = 0, Ma = M)
    h->ndm = true;
    h->split = c.network == NQ_NET_RBM_SPLIT;
    h->symm = c.network == NQ_NET_NDM_SYMM;
    h->n_symm = h->symm ? c.n_symm : 1;
    h->sym_h = c.n_hidden;
    h->sym_a = c.n_ancilla;
    h->Mh = h->split ? 0 : c.n_hidden * h->n_symm;
    h->Ma = h->split ? c.n_hidden : c.n_ancilla * h->n_symm;
    if (!h->split && h->Ma < 1) return bad("the NDM needs n_ancilla >= 1");
    h->N2 = 2 * h->N;
    h->U = 4 * h->Mh + h->Ma;
    h->Ms = 2 * h->Mh + h->Ma;
    h->diag = c.sampler_space == NQ_SPACE_DIAGONAL;
    h->Md = h->Mh + h->Ma;
    h->nst = h->diag ? h->N : h->N2;
    h->P = h->split ? 2 * h->N + h->Ma + 2 * h->N * h->Ma
                    : (h->symm ? ndm_n_params(h->N, h->sym_h, h->sym_a) : ndm_n_params(h->N, h->Mh, h->Ma));
    h->P_bare = h->symm ? ndm_n_params(h->N, h->Mh, h->Ma) : h->P;
    if (h->N2 > 64) return bad("the NDM supports n_sites <= 32 (2N doubled sites)");
    if (h->Ms > 320) return bad("2*n_hidden + n_ancilla must be <= 320");
    if (h->P > 256 * 24) return bad("too many density-matrix parameters (max 6144)");
  } else if (h->chain) {
    h->nst = h->mixed ? 2 * h->N : h->N;
    h->M = h->chain_spec.L[0].out;
    h->P = h->chain_spec.P;
  } else {
    h->nst = h->N;
    h->P = h->N + h->M + h->M * h->N;
  }
  h->B = c.n_chains;
  h->L = c.chain_length;
  h->Ns = h->B * h->L;
  h->passes = (c.passes % 2 == 0) ? c.passes + 1 : c.passes;
  const bool stale = (c.quirks & NQ_QUIRK_STALE_LAST_SLOT) != 0;
  h->n_record = stale ? (h->L > 1 ? h->L - 1 : 0) : h->L;
  h->write_last = (stale && h->L == 1) ? 1 : 0;
  h->hilb = c.hilbert;
  h->act = c.activation;
  h->f64 = c.eval_precision == NQ_EVAL_F64;
  h->tc_theta = c.eval_precision == NQ_EVAL_TC_BF16X2 || c.eval_precision == NQ_EVAL_TC_BF16X3;
  h->theta_terms = c.eval_precision == NQ_EVAL_TC_BF16X3 ? 3 : 2;
  h->complex_params = !h->ndm || h->split;      // RBM, RBMSplit and chains
  h->real_sr = !h->complex_params || (h->chain && h->chain_spec.pdr);
  if (c.sr_algorithm == NQ_SR_CG && c.network != NQ_NET_RBM && !sr_cg_x_supported(h->P)) {
    delete h;
    return NQ_ERR_UNSUPPORTED;
  }
  const int sampler_M = h->diag ? h->Md : (h->ndm ? h->Ms : h->M), sampler_N = h->nst;
  if (c.sampler_lanes != 0 && !h->chain) {
    int cand[4];
    const int nc = rbm_sampler_valid_lanes(sampler_N, sampler_M, h->f64 ? 16 : 8, cand, 4);
    bool ok = false;
    for (int i = 0; i < nc; ++i) ok = ok || cand[i] == c.sampler_lanes;
    if (!ok) return bad("sampler_lanes not available for this number of hidden units");
    h->sampler_lanes = c.sampler_lanes;
  }
  if ((long)h->Ns * h->M > (1L << 31)) return bad("B*L*M too large");

  nq_status s = NQ_OK;
  auto step = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && s == NQ_OK) {
      fprintf(stderr, "nq_create: %s: %s\n", what, cudaGetErrorString(e));
      s = NQ_ERR_CUDA;
    }
  };
  step(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking), "stream");
  step(cudaStreamCreateWithFlags(&h->st_side, cudaStreamNonBlocking), "side stream");
  step(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming), "fork event");
  step(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming), "join event");
  const size_t csz = h->f64 ? sizeof(cpx<double>) : sizeof(cpx<float>);
  const int P = h->P;
  step(dalloc(&h->d_master, 2 * (size_t)P), "params");
  step(dalloc(&h->d_p32, 2 * (size_t)P), "params32");
  if (h->chain && h->chain_spec.pdr && h->f64) step(dalloc(&h->d_pexp, 2 * (size_t)P), "PositiveDefR params");
  for (int k = 0; k < 3; ++k) step(cudaMalloc(&h->d_tab[k], (size_t)sampler_N * sampler_M * csz + 16), "tables");
  if (h->ndm) {
    const size_t ne[5] = {(size_t)h->U * h->N2, (size_t)h->U, (size_t)h->N2, (size_t)h->Ms * h->N2, (size_t)h->Ms};
    for (int k = 0; k < 5; ++k) step(cudaMalloc(&h->d_eff[k], ne[k] * csz + 16), "effective network");
    if (h->symm) step(cudaMalloc(&h->d_bare, (size_t)h->P_bare * (h->f64 ? sizeof(double) : sizeof(float)) + 16),
                      "bare parameters");
    if (h->diag) {
      const size_t nd[3] = {(size_t)h->N, (size_t)h->Md, (size_t)h->Md * h->N};
      for (int k = 0; k < 3; ++k) step(cudaMalloc(&h->d_diag[k], nd[k] * csz + 16), "diagonal network");
    } else {
      step(dalloc(&h->d_ndm_partial, (size_t)ndm_grad_nblocks(h->Ns) * 2 * h->P), "ndm partial");
    }
  }
  step(dalloc(&h->d_samples, (size_t)h->Ns), "samples");
  step(dalloc(&h->d_accepted, 1), "accepted");
  step(dalloc(&h->d_call, 1), "call");
  step(cudaMalloc(&h->d_logpsi, (size_t)h->Ns * csz), "logpsi");
  if (!h->ndm && !h->chain) step(cudaMalloc(&h->d_g, (size_t)h->Ns * h->M * csz), "g");
  step(cudaMalloc(&h->d_eloc, (size_t)h->Ns * csz), "eloc");
  if (h->f64 && !h->ndm && !h->chain) step(dalloc(&h->d_g32, (size_t)h->Ns * h->M), "g32");
  h->force_nblk = (h->ndm || h->chain) ? 1 : rbm_force_nblocks(h->Ns, h->N, h->M, (int)csz);
  step(dalloc(&h->fb.partial, (size_t)h->force_nblk * 4 * P), "force partial");
  step(dalloc(&h->fb.partialE, 2 * (size_t)h->force_nblk), "force partialE");
  step(dalloc(&h->fb.meanO, 2 * (size_t)P), "meanO");
  step(dalloc(&h->fb.force, 2 * (size_t)P), "force");
  step(dalloc(&h->fb.meanE, 2), "meanE");
  step(dalloc(&h->d_stats, 8), "stats");
  step(dalloc(&h->d_chainstats, stats_scratch_doubles(h->B)), "chain stats");
  if (h->mixed) step(dalloc(&h->d_cgrad, (size_t)h->P * h->Ns), "Liouvillian gradient");
  step(dalloc(&h->fb.sums, 4 * (size_t)P + 2), "force sums");
  h->cg = c.sr_algorithm == NQ_SR_CG;
  h->exact = c.sampler_kind == NQ_SAMPLER_EXACT;
  h->rule = c.rule;
  if (h->exact) step(dalloc(&h->d_exact, exact_sampler_work_doubles(h->nst)), "exact sampler");
  // the diagonal-space handle estimates observables only: no S, X or solve buffers
  const bool sr_bufs = !h->cg && !h->diag;
  const int rows = 2 * P;
  const int rp = ((rows + 127) / 128) * 128;
  // NQ_S_F32 asks for S with FP32 accuracy.  Where the tensor-core Gram is
  // available and X with its low part fits kSf32TensorBytes, S is accumulated
  // as 3xTF32 on tcgen05 (hi/lo split, FP32-level error); otherwise in FP32 on
  // CUDA cores, which needs no X buffers.
  if (sr_bufs && c.s_precision == NQ_S_F32 && gram_tc_supported() &&
      2.0 * rows * (double)(((h->Ns + 127) / 128) * 128) * sizeof(float) <= kSf32TensorBytes)
    h->cfg.s_precision = NQ_S_TF32X3;
  // matrix-free SR over X (NDM family, chains): S is never formed, so X stays
  // plain FP32 (no TF32 rounding, no low part)
  const bool cg_x = h->cg && (h->ndm || h->chain) && !h->diag;
  if (cg_x) h->cfg.s_precision = NQ_S_F32;
  const int s_prec = h->cfg.s_precision;
  if (h->cg) {
    // matrix-free SR: O(P) vectors and per-CTA partials only
    const int G = sr_cg_grid();
    SrCgArgs& a = h->cga;
    a.N = h->N; a.M = h->M; a.P = P; a.Ns = h->Ns; a.hilb = h->hilb;
    a.samples = h->d_samples; a.g = reinterpret_cast<const float2*>(h->d_g); a.meanO = h->fb.meanO;
    a.F = h->fb.force;
    step(dalloc(&h->sb.x, 2 * (size_t)P), "x");
    step(dalloc(&a.r, 2 * (size_t)P), "cg r");
    step(dalloc(&a.pv, 2 * (size_t)P), "cg p");
    step(dalloc(&a.w, 2 * (size_t)P), "cg w");
    step(dalloc(&a.part, 2 * (size_t)G * P), "cg partials");
    step(dalloc(&a.tsum, 2 * (size_t)G), "cg tsum");
    step(dalloc(&a.dots, 4 * (size_t)G), "cg dots");
    step(dalloc(&a.t, (size_t)h->Ns), "cg t");
    step(dalloc(&a.shift, (size_t)P), "cg shift");
    step(cudaMalloc(&a.ctl, sr_cg_ctl_bytes()), "cg ctl");
    step(dalloc(&a.info, 2), "cg info");
    step(dalloc(&h->sb.status, 1), "status");
    step(cudaMallocHost((void**)&h->h_cginfo, 2 * sizeof(double)), "pinned");
    a.x = h->sb.x;
    a.status = h->sb.status;
    h->cg_maxiter = 10 * P;
  }
  // split-K so that the S stage fills the GPU with ~2 waves of tiles
  {
    const int nt = (rows + 63) / 64;
    const int tiles = nt * (nt + 1) / 2;
    int ks = 1;
    while (tiles * ks < 2 * 152 && ks < 16 && h->Ns / (ks * 2) >= 256) ks *= 2;
    h->gram_ksplit = ks;
  }
  if (sr_bufs) step(dalloc(&h->d_G, (size_t)rows * rows), "G");
  if (sr_bufs) step(dalloc(&h->d_Gpart, (size_t)h->gram_ksplit * rp * rp), "G partial");
  if (!sr_bufs && !cg_x) {
  } else if (sr_bufs && (s_prec == NQ_S_TF32 || s_prec == NQ_S_TF32X3 || s_prec == NQ_S_BF16)) {
    const int bf16 = s_prec == NQ_S_BF16 ? 1 : 0;
    h->Ns_pad = ((h->Ns + 127) / 128) * 128;
    h->gram_ksplit = gram_tc_ksplit(rows, h->Ns_pad, bf16);
    cudaFree(h->d_Gpart);
    h->d_Gpart = nullptr;
    step(dalloc(&h->d_Gpart, gram_tc_partial_elems(rows, h->Ns_pad, bf16)), "G partial");
    step(dalloc(&h->d_X, (size_t)rows * h->Ns_pad / (bf16 ? 2 : 1)), "X");     // BF16 X: half the bytes
    if (s_prec == NQ_S_TF32X3) step(dalloc(&h->d_Xlo, (size_t)rows * h->Ns_pad), "Xlo");
  } else if (h->ndm || h->chain) {
    h->Ns_pad = ((h->Ns + 127) / 128) * 128;
    step(dalloc(&h->d_X, (size_t)rows * h->Ns_pad), "X");
  }
  if (cg_x) {
    h->cga.X = h->d_X;
    h->cga.ldx = h->Ns_pad;
  }
  if (sr_bufs) {
    step(dalloc(&h->d_S, 2 * (size_t)P * P), "S");
    step(dalloc(&h->sb.W, (size_t)P * P), "W");
    step(dalloc(&h->sb.x, 2 * (size_t)P), "x");
    step(dalloc(&h->sb.r, 2 * (size_t)P), "r");
    step(dalloc(&h->sb.rf, (size_t)P), "rf");
    step(dalloc(&h->sb.status, 1), "status");
    step(cudaMalloc(&h->sb.ctl, sweep_ctl_bytes()), "sweep ctl");
    step(dalloc(&h->sb.work, sweep_work_elems(P)), "sweep work");
    step(dalloc(&h->sb.yf, (size_t)P), "yf");
    step(dalloc(&h->sb.norms, refine_norm_doubles()), "refinement norms");
    step(dalloc(&h->sb.info, 2), "refinement info");
  }
  if (h->diag) step(dalloc(&h->sb.status, 1), "status");
  if (h->tc_theta) {
    step(dalloc(&h->d_theta_img, theta_tc_image_elems(h->ndm ? h->U : h->M, h->theta_terms)), "theta image");
    if (h->ndm) step(dalloc(&h->d_ndm_theta, (size_t)h->U * h->Ns), "unit pre-activations");
  }
  h->sb.S = h->d_S;
  step(cudaMallocHost((void**)&h->h_call, sizeof(uint32_t)), "pinned");
  step(cudaMallocHost((void**)&h->h_stats, 8 * sizeof(double)), "pinned");
  step(cudaMallocHost((void**)&h->h_acc, sizeof(unsigned long long)), "pinned");
  step(cudaMallocHost((void**)&h->h_status, sizeof(int)), "pinned");
  step(cudaMallocHost((void**)&h->h_params, 2 * (size_t)P * sizeof(double)), "pinned");
  step(cudaEventCreateWithFlags(&h->ev_params, cudaEventDisableTiming), "params event");
  for (int k = 0; k < 7; ++k) step(cudaEventCreate(&h->ev[k]), "event");
  for (int k = 0; k < 4; ++k) step(cudaEventCreate(&h->kev[k]), "event");
  for (int k = 0; k < 6; ++k) step(cudaEventCreate(&h->sev[k]), "event");
  if (s == NQ_OK) {
    step(cudaMemsetAsync(h->d_master, 0, 2 * sizeof(double) * P, h->st), "memset");
    step(cudaMemsetAsync(h->sb.status, 0, sizeof(int), h->st), "memset");
    // sample buffer starts as the state() fill: all sites at local index 0
    step(cudaMemsetAsync(h->d_samples, 0, sizeof(uint64_t) * h->Ns, h->st), "memset");
    if (sr_bufs) step(cudaMemsetAsync(h->d_S, 0, 2 * sizeof(double) * P * P, h->st), "memset");
    if (refresh_params(h) != NQ_OK) s = NQ_ERR_CUDA;
    step(cudaStreamSynchronize(h->st), "sync");
  }
  if (s != NQ_OK) {
    nq_destroy(h);
    return s;
  }
  *out = h;
  return NQ_OK;
}

}  // namespace

extern "C" {

nq_status nq_create(const nq_config* cfg, nq_handle** out) { return create_impl(cfg, 0, nullptr, out); }

nq_status nq_create_chain(const nq_config* cfg, int32_t n_layers, const nq_layer* layers, nq_handle** out) {
  if (!cfg || (cfg->network != NQ_NET_CHAIN && cfg->network != NQ_NET_MIXED_CHAIN)) return NQ_ERR_ARG;
  return create_impl(cfg, n_layers, layers, out);
}

void nq_destroy(nq_handle* h) {
  if (!h) return;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->x_borrowed) { h->d_X = nullptr; h->d_Xlo = nullptr; }   // owned by the batch
  if (h->graph) cudaGraphExecDestroy(h->graph);
  proposal_destroy(h);
  free_op(h);
  free_rule_operator(h);
  void* bufs[] = {h->d_master, h->d_p32, h->d_pexp, h->d_frhs, h->d_tab[0], h->d_tab[1], h->d_tab[2], h->d_samples,
                  h->d_accepted, h->d_call, h->d_logpsi, h->d_g, h->d_eloc, h->d_g32,
                  h->fb.partial, h->fb.partialE, h->fb.meanO, h->fb.force, h->fb.meanE, h->fb.sums,
                  h->d_chainstats,
                  h->d_stats, h->d_G, h->d_Gpart, h->d_X, h->d_Xlo, h->d_S, h->sb.W, h->sb.work, h->sb.x, h->sb.r,
                  h->sb.rf, h->sb.yf, h->sb.status, h->sb.ctl, h->sb.norms, h->sb.info, h->d_theta_img, h->d_ndm_theta, h->d_cgrad, h->d_exact, h->d_pairs, h->d_xtab[0],
                  h->d_xtab[1], h->d_xtab[2], h->d_xW, h->d_xare, h->d_dw, h->d_eff[0], h->d_eff[1],
                  h->d_eff[2], h->d_eff[3], h->d_eff[4], h->d_w, h->d_wconn, h->d_nconn, h->d_ndm_partial,
                  h->d_diag[0], h->d_diag[1], h->d_diag[2], h->d_bare, h->d_perms};
  for (void* p : h->sym_allocs) cudaFree(p);
  for (void* p : bufs)
    if (p) cudaFree(p);
  {
    void* cgb[] = {h->cga.r, h->cga.pv, h->cga.w, h->cga.part, h->cga.tsum, h->cga.dots, h->cga.t, h->cga.shift,
                   h->cga.ctl, h->cga.info};
    for (void* p : cgb)
      if (p) cudaFree(p);
    if (h->h_cginfo) cudaFreeHost(h->h_cginfo);
  }
  if (h->h_call) cudaFreeHost(h->h_call);
  if (h->h_stats) cudaFreeHost(h->h_stats);
  if (h->h_status) cudaFreeHost(h->h_status);
  if (h->h_params) cudaFreeHost(h->h_params);
  if (h->ev_params) cudaEventDestroy(h->ev_params);
  if (h->h_acc) cudaFreeHost(h->h_acc);
  for (int k = 0; k < 7; ++k)
    if (h->ev[k]) cudaEventDestroy(h->ev[k]);
  for (int k = 0; k < 4; ++k)
    if (h->kev[k]) cudaEventDestroy(h->kev[k]);
  for (int k = 0; k < 6; ++k)
    if (h->sev[k]) cudaEventDestroy(h->sev[k]);
  if (h->d_flush) cudaFree(h->d_flush);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->st_side) cudaStreamDestroy(h->st_side);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
}

nq_status nq_last_error(const nq_handle* h, char* buf, size_t len) {
  if (!h || !buf || len == 0) return NQ_ERR_ARG;
  snprintf(buf, len, "%s", h->err.c_str());
  return NQ_OK;
}

int64_t nq_n_params(const nq_handle* h) { return h ? h->P : -1; }
int64_t nq_kernel_launches(const nq_handle* h) { return h ? h->launches : -1; }

nq_status nq_set_params(nq_handle* h, const void* flat, int64_t n, int32_t dtype) {
  if (!h || !flat) return NQ_ERR_ARG;
  if (n != h->P) return fail(h, NQ_ERR_ARG, "expected %d parameters, got %lld", h->P, (long long)n);
  const size_t nd = (h->complex_params ? 2 : 1) * (size_t)h->P;
  if (h->complex_params ? (dtype != NQ_DTYPE_C128 && dtype != NQ_DTYPE_C64)
                        : (dtype != NQ_DTYPE_F64 && dtype != NQ_DTYPE_F32))
    return fail(h, NQ_ERR_ARG, h->complex_params ? "RBM / RBMSplit parameters are complex (dtype c64 or c128)"
                                                 : "NDM parameters are real (dtype f32 or f64)");
  // the pinned staging buffer is reused once the previous upload out of it is done
  CK(cudaEventSynchronize(h->ev_params));
  double* buf = h->h_params;
  if (dtype == NQ_DTYPE_C128 || dtype == NQ_DTYPE_F64) {
    memcpy(buf, flat, nd * sizeof(double));
  } else {
    const float* f = (const float*)flat;
    for (size_t i = 0; i < nd; ++i) buf[i] = f[i];
  }
  for (size_t i = 0; i < nd; ++i)
    if (!std::isfinite(buf[i])) return fail(h, NQ_ERR_NAN, "non-finite parameter");
  // asynchronous upload from the pinned buffer; it and the refresh kernels
  // stay queued on the handle's stream ahead of its next call
  CK(cudaMemcpyAsync(h->d_master, buf, nd * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CK(cudaEventRecord(h->ev_params, h->st));
  return refresh_params(h);
}

nq_status nq_get_params(nq_handle* h, void* flat, int64_t n, int32_t dtype) {
  if (!h || !flat) return NQ_ERR_ARG;
  if (n != h->P) return fail(h, NQ_ERR_ARG, "expected %d parameters, got %lld", h->P, (long long)n);
  const bool want_c = dtype == NQ_DTYPE_C128 || dtype == NQ_DTYPE_C64;
  if (want_c != h->complex_params)
    return fail(h, NQ_ERR_ARG, h->complex_params ? "RBM / RBMSplit parameters are complex (dtype c64 or c128)"
                                                 : "NDM parameters are real (dtype f32 or f64)");
  const size_t nd = (h->complex_params ? 2 : 1) * (size_t)h->P;
  // into the pinned staging buffer (after any upload out of it, stream order)
  CK(cudaMemcpyAsync(h->h_params, h->d_master, nd * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (dtype == NQ_DTYPE_C128 || dtype == NQ_DTYPE_F64) memcpy(flat, h->h_params, nd * sizeof(double));
  else {
    float* f = (float*)flat;
    for (size_t i = 0; i < nd; ++i) f[i] = (float)h->h_params[i];
  }
  return NQ_OK;
}

nq_status nq_set_exchange(nq_handle* h, int32_t n, const int32_t* pairs) {
  if (!h || n < 1 || !pairs) return NQ_ERR_ARG;
  if (h->rule != NQ_RULE_EXCHANGE) return fail(h, NQ_ERR_STATE, "the handle was created with another rule");
  for (int k = 0; k < n; ++k) {
    const int i = pairs[2 * k], j = pairs[2 * k + 1];
    if (i < 0 || j < 0 || i >= h->N || j >= h->N || i == j)
      return fail(h, NQ_ERR_ARG, "coupling %d: sites (%d, %d) out of range or equal", k, i, j);
  }
  CK(cudaStreamSynchronize(h->st));
  cudaFree(h->d_pairs); cudaFree(h->d_xW); cudaFree(h->d_xare);
  for (void*& p : h->d_xtab) { cudaFree(p); p = nullptr; }
  h->d_pairs = nullptr; h->d_xW = nullptr; h->d_xare = nullptr; h->n_exch = 0;
  const size_t tab = (size_t)n * h->M * sizeof(cpx<float>);
  CK(cudaMalloc((void**)&h->d_pairs, (size_t)n * sizeof(int2)));
  for (void*& p : h->d_xtab) CK(cudaMalloc(&p, tab));
  CK(cudaMalloc(&h->d_xW, tab));
  CK(cudaMalloc((void**)&h->d_xare, (size_t)n * sizeof(float)));
  CK(cudaMemcpy(h->d_pairs, pairs, (size_t)n * sizeof(int2), cudaMemcpyHostToDevice));
  h->n_exch = n;
  h->sampler_lanes = h->cfg.sampler_lanes;      // re-tune: the tables changed size
  h->sampler_block = 0;
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  if (nq_status s = refresh_params(h)) return s;
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

// NDMSymm: permutations, and the map from the symmetric parameters to the bare
// ones for the gradient (construct_∇matrices, NDMSymm.jl:135-180): b_mu / b_la
// of every site average all bare sites' (coefficient 1/N), a hidden or
// ancilla bias sums its n_symm copies, weight (f, i) sums the bare weights
// (j + f n_symm, perm_j(i)).
nq_status nq_set_symmetry(nq_handle* h, int32_t n_perm, const int32_t* perms) {
  if (!h || !perms) return NQ_ERR_ARG;
  if (!h->symm) return fail(h, NQ_ERR_STATE, "the handle is not an NDMSymm");
  const int N = h->N, ns = h->n_symm, ah = h->sym_h, aa = h->sym_a, Mh = h->Mh, Ma = h->Ma;
  if (n_perm != ns) return fail(h, NQ_ERR_ARG, "expected %d permutations, got %d", ns, n_perm);
  for (int j = 0; j < ns; ++j) {
    std::vector<int> seen(N, 0);
    for (int i = 0; i < N; ++i) {
      const int v = perms[j * N + i];
      if (v < 0 || v >= N || seen[v]++) return fail(h, NQ_ERR_ARG, "permutation %d is not a permutation of 0..%d", j, N - 1);
    }
  }
  // symmetric and bare field offsets (b_mu, h_mu, w_mu, u_mu, b_la, h_la, d_la, w_la, u_la)
  auto offsets = [N](int mh, int ma, int* o) {
    o[0] = 0; o[1] = o[0] + N; o[2] = o[1] + mh; o[3] = o[2] + mh * N; o[4] = o[3] + ma * N;
    o[5] = o[4] + N; o[6] = o[5] + mh; o[7] = o[6] + ma; o[8] = o[7] + mh * N;
  };
  int so[9], bo[9];
  offsets(ah, aa, so);
  offsets(Mh, Ma, bo);
  std::vector<int> off(1, 0), idx;
  std::vector<double> coef;
  auto put = [&](int bare, double c) { idx.push_back(bare); coef.push_back(c); };
  for (int f9 = 0; f9 < 9; ++f9) {
    const bool isb = f9 == 0 || f9 == 4, ish = f9 == 1 || f9 == 5, isd = f9 == 6;
    const bool isw = f9 == 2 || f9 == 7;            // otherwise (f9 = 3, 8): the ancilla weights
    const int n = isb ? N : (ish ? ah : (isd ? aa : (isw ? ah * N : aa * N)));
    for (int k = 0; k < n; ++k) {
      if (isb) {
        for (int i = 0; i < N; ++i) put(bo[f9] + i, 1.0 / N);
      } else if (ish || isd) {
        for (int j = 0; j < ns; ++j) put(bo[f9] + k * ns + j, 1.0);
      } else {
        const int rows = isw ? ah : aa, brows = isw ? Mh : Ma;
        const int f = k % rows, i = k / rows;
        for (int j = 0; j < ns; ++j) put(bo[f9] + (j + f * ns) + brows * perms[j * N + i], 1.0);
      }
      off.push_back((int)idx.size());
    }
  }
  if ((int)off.size() != h->P + 1) return fail(h, NQ_ERR_ARG, "internal: symmetric parameter count");
  CK(cudaStreamSynchronize(h->st));
  for (void* p : h->sym_allocs) cudaFree(p);
  h->sym_allocs.clear();
  cudaFree(h->d_perms);
  h->d_perms = nullptr;
  h->sym_ready = false;
  nq_status s;
  if ((s = upload(h, (const int*)off.data(), off.size(), &h->d_sym_off, &h->sym_allocs)) != NQ_OK ||
      (s = upload(h, (const int*)idx.data(), idx.size(), &h->d_sym_idx, &h->sym_allocs)) != NQ_OK ||
      (s = upload(h, (const double*)coef.data(), coef.size(), &h->d_sym_coef, &h->sym_allocs)) != NQ_OK)
    return s;
  CK(cudaMalloc((void**)&h->d_perms, (size_t)ns * N * sizeof(int)));
  CK(cudaMemcpy(h->d_perms, perms, (size_t)ns * N * sizeof(int), cudaMemcpyHostToDevice));
  h->sym_ready = true;
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  if (nq_status r = refresh_params(h)) return r;
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

// OperatorRule move set from the operator's row tables: the operators' sites
// and rows as in the estimator, one code per connection (-1 without changes,
// else its move class and orientation), and the classes' changed sites with
// their canonical new local indices (first site at index 1).
nq_status nq_set_rule_operator(nq_handle* h, const nq_op_table* t) {
  if (!h || !t) return NQ_ERR_ARG;
  if (h->rule != NQ_RULE_OPERATOR) return fail(h, NQ_ERR_STATE, "the handle was created with another rule");
  if (nq_status v = validate_op(h, t)) return v;
  const int no = t->n_ops, nr = t->n_rows, nconn = t->n_conns;
  std::vector<unsigned long long> osites(no), omask(no);
  std::vector<int> prefix(no + 1, 0);
  bool const_counts = true;
  for (int o = 0; o < no; ++o) {
    unsigned long long packed = 0, mask = 0;
    for (int d = 0; d < t->op_n_sites[o]; ++d) {
      const int site = t->op_sites[8 * o + d];
      packed |= (unsigned long long)site << (8 * d);
      mask |= 1ull << site;
    }
    osites[o] = packed;
    omask[o] = mask;
    const int r0 = t->op_row_offset[o];
    const int len0 = t->row_conn_offset[r0 + 1] - t->row_conn_offset[r0];
    for (int r = 1; r < (1 << t->op_n_sites[o]); ++r)
      if (t->row_conn_offset[r0 + r + 1] - t->row_conn_offset[r0 + r] != len0) const_counts = false;
    prefix[o + 1] = prefix[o] + len0;
  }
  // move classes: key = (sites in connection order, new local indices normalised so that the
  // first changed site goes to index 1)
  std::map<std::pair<std::vector<int>, int>, int> classes;
  std::vector<int> code(nconn, -1), csites, cbits;
  std::vector<unsigned long long> cmask;
  for (int c = 0; c < nconn; ++c) {
    const int nch = t->conn_n_changes[c];
    if (nch == 0) continue;
    std::vector<int> sites(nch);
    int bitsv = 0;
    unsigned long long m = 0;
    for (int q = 0; q < nch; ++q) {
      sites[q] = t->conn_change_site[8 * c + q];
      const int v = t->conn_change_value[8 * c + q];
      const int b = h->hilb == NQ_HILB_SPIN ? (v > 0 ? 1 : 0) : v;
      bitsv |= b << q;
      m |= 1ull << sites[q];
    }
    const bool comp = (bitsv & 1) == 0;
    if (comp) bitsv ^= (1 << nch) - 1;
    auto key = std::make_pair(sites, bitsv);
    auto it = classes.find(key);
    int k;
    if (it == classes.end()) {
      k = (int)classes.size();
      classes.emplace(key, k);
      for (int q = 0; q < 8; ++q) csites.push_back(q < nch ? sites[q] : -1);
      cbits.push_back(bitsv);
      cmask.push_back(m);
    } else {
      k = it->second;
    }
    code[c] = 2 * k + (comp ? 1 : 0);
  }
  const int nclass = (int)classes.size();
  if (nclass == 0) return fail(h, NQ_ERR_ARG, "the move operator has no connection that changes a configuration");
  CK(cudaStreamSynchronize(h->st));
  free_rule_operator(h);
  cudaFree(h->d_xW); cudaFree(h->d_xare);
  for (void*& p : h->d_xtab) { cudaFree(p); p = nullptr; }
  h->d_xW = nullptr; h->d_xare = nullptr; h->n_exch = 0;
  OpMovesDev m;
  m.n_ops = no; m.n_rows = nr; m.n_conns = nconn; m.n_classes = nclass;
  m.const_counts = const_counts ? 1 : 0;
  m.n_total = prefix[no];
  nq_status s;
  if ((s = upload(h, osites.data(), osites.size(), &m.op_sites, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, omask.data(), omask.size(), &m.op_mask, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, t->op_n_sites, (size_t)no, &m.op_n_sites, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, t->op_row_offset, (size_t)no, &m.op_row_offset, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, (const int*)prefix.data(), prefix.size(), &m.op_prefix, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, t->row_conn_offset, (size_t)nr + 1, &m.row_conn_offset, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, (const int*)code.data(), code.size(), &m.conn_code, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, cmask.data(), cmask.size(), &m.class_mask, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, (const int*)csites.data(), csites.size(), &m.class_sites, &h->opm_allocs)) != NQ_OK ||
      (s = upload(h, (const int*)cbits.data(), cbits.size(), &m.class_bits, &h->opm_allocs)) != NQ_OK) {
    free_rule_operator(h);
    return s;
  }
  h->opm = m;
  bool fits = false;
  for (int G : {4, 8, 16, 32}) fits = fits || oprule_sampler_smem(m, h->M, G) > 0;
  if (!fits) {
    free_rule_operator(h);
    return fail(h, NQ_ERR_UNSUPPORTED, "operator rule: %d move classes x %d hidden units exceed the shared memory",
                nclass, h->M);
  }
  const size_t tab = (size_t)nclass * h->M * sizeof(cpx<float>);
  for (void*& p : h->d_xtab) CK(cudaMalloc(&p, tab));
  CK(cudaMalloc(&h->d_xW, tab));
  CK(cudaMalloc((void**)&h->d_xare, (size_t)nclass * sizeof(float)));
  h->n_exch = nclass;
  h->sampler_lanes = h->cfg.sampler_lanes;      // re-tune: the move set changed
  h->sampler_block = 0;
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  if (nq_status r = refresh_params(h)) return r;
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

nq_status nq_set_operator(nq_handle* h, const nq_op_table* t) {
  if (!h || !t) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_set_operator");
  if (nq_status v = validate_op(h, t)) return v;
  CK(cudaStreamSynchronize(h->st));
  free_op(h);
  DevOp d;
  if (nq_status s = upload_op(h, t, &d, nullptr)) return s;
  h->op = d;
  h->has_op = true;
  if (h->ndm) {
    // the Liouvillian estimator keeps the weight of every connection: bound
    // the connections per configuration by the longest row of each operator
    int maxc = 0;
    for (int o = 0; o < t->n_ops; ++o) {
      int longest = 0;
      const int nrows = 1 << t->op_n_sites[o];
      for (int r = 0; r < nrows; ++r) {
        const int row = t->op_row_offset[o] + r;
        longest = std::max(longest, t->row_conn_offset[row + 1] - t->row_conn_offset[row]);
      }
      maxc += longest;
    }
    maxc = std::max(maxc, 1);
    if (h->d_w) cudaFree(h->d_w);
    if (h->d_wconn) cudaFree(h->d_wconn);
    if (h->d_nconn) cudaFree(h->d_nconn);
    h->d_w = nullptr; h->d_wconn = nullptr; h->d_nconn = nullptr;
    const size_t csz = h->f64 ? sizeof(cpx<double>) : sizeof(cpx<float>);
    CK(cudaMalloc(&h->d_w, (size_t)h->Ns * maxc * csz));
    CK(cudaMalloc((void**)&h->d_wconn, (size_t)h->Ns * maxc * sizeof(int)));
    CK(cudaMalloc((void**)&h->d_nconn, (size_t)h->Ns * sizeof(int)));
    h->maxc = maxc;
  }
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  return NQ_OK;
}

nq_status nq_observable(nq_handle* h, const nq_op_table* obs, nq_measurement* stats, double* loc_out) {
  if (!h || !obs || !stats) return NQ_ERR_ARG;
  if (h->symm && !h->sym_ready) return fail(h, NQ_ERR_STATE, "NDMSymm: no permutations (nq_set_symmetry)");
  if (h->ndm && !h->diag)
    return fail(h, NQ_ERR_UNSUPPORTED,
                "observables of a density matrix are estimated on its diagonal (NQ_SPACE_DIAGONAL handle)");
  if (nq_status v = validate_op(h, obs)) return v;
  std::vector<void*> allocs;
  DevOp d;
  void* d_lp = nullptr;
  void* d_loc = nullptr;
  double* d_cs = nullptr;
  double* d_st = nullptr;
  const size_t csz = h->f64 ? sizeof(cpx<double>) : sizeof(cpx<float>);
  auto cleanup = [&](nq_status s) {
    cudaStreamSynchronize(h->st);
    for (void* p : allocs) cudaFree(p);
    cudaFree(d_lp); cudaFree(d_loc); cudaFree(d_cs); cudaFree(d_st);
    return s;
  };
  nq_status s = upload_op(h, obs, &d, &allocs);
  if (s != NQ_OK) return cleanup(s);
  if (cudaMalloc(&d_lp, (size_t)h->Ns * csz) != cudaSuccess || cudaMalloc(&d_loc, (size_t)h->Ns * csz) != cudaSuccess ||
      cudaMalloc((void**)&d_cs, stats_scratch_doubles(h->B) * sizeof(double)) != cudaSuccess ||
      cudaMalloc((void**)&d_st, 8 * sizeof(double)) != cudaSuccess)
    return cleanup(fail(h, NQ_ERR_CUDA, "observable buffers"));
  cudaError_t e;
  ++h->launches;
  if (h->chain) {
    if (h->f64) {
      e = launch_chain_eval<double>(chain_dev<double>(h), h->d_samples, h->Ns, &d, (cpx<double>*)d_lp,
                                    (cpx<double>*)d_loc, nullptr, 0, nullptr, h->st);
      if (e == cudaSuccess) e = launch_stats<double>((cpx<double>*)d_loc, h->B, h->L, 0, d_cs, d_st, h->st);
    } else {
      e = launch_chain_eval<float>(chain_dev<float>(h), h->d_samples, h->Ns, &d, (cpx<float>*)d_lp,
                                   (cpx<float>*)d_loc, nullptr, 0, nullptr, h->st);
      if (e == cudaSuccess) e = launch_stats<float>((cpx<float>*)d_loc, h->B, h->L, 0, d_cs, d_st, h->st);
    }
  } else if (h->diag) {
    if (h->f64) {
      e = launch_ndm_diag_obs<double>(ndm_eff<double>(h), h->act, d, h->d_samples, h->Ns, h->hilb,
                                      (cpx<double>*)d_lp, (cpx<double>*)d_loc, h->st);
      if (e == cudaSuccess) e = launch_stats<double>((cpx<double>*)d_loc, h->B, h->L, 0, d_cs, d_st, h->st);
    } else {
      e = launch_ndm_diag_obs<float>(ndm_eff<float>(h), h->act, d, h->d_samples, h->Ns, h->hilb,
                                     (cpx<float>*)d_lp, (cpx<float>*)d_loc, h->st);
      if (e == cudaSuccess) e = launch_stats<float>((cpx<float>*)d_loc, h->B, h->L, 0, d_cs, d_st, h->st);
    }
  } else if (h->f64) {
    e = launch_rbm_eval<double>(rbm_dev<double>(h), h->d_samples, h->Ns, &d, (cpx<double>*)d_lp, nullptr,
                                (cpx<double>*)d_loc, h->st);
    if (e == cudaSuccess) e = launch_stats<double>((cpx<double>*)d_loc, h->B, h->L, 0, d_cs, d_st, h->st);
  } else {
    e = launch_rbm_eval<float>(rbm_dev<float>(h), h->d_samples, h->Ns, &d, (cpx<float>*)d_lp, nullptr,
                               (cpx<float>*)d_loc, h->st);
    if (e == cudaSuccess) e = launch_stats<float>((cpx<float>*)d_loc, h->B, h->L, 0, d_cs, d_st, h->st);
  }
  h->launches += 2;
  if (e != cudaSuccess) return cleanup(fail(h, NQ_ERR_CUDA, "observable: %s", cudaGetErrorString(e)));
  double v[6];
  if (cudaMemcpyAsync(v, d_st, 6 * sizeof(double), cudaMemcpyDeviceToHost, h->st) != cudaSuccess ||
      cudaStreamSynchronize(h->st) != cudaSuccess)
    return cleanup(fail(h, NQ_ERR_CUDA, "observable copy"));
  stats->mean_re = v[0]; stats->mean_im = v[1]; stats->error = v[2]; stats->variance = v[3];
  stats->tau = v[4]; stats->R = v[5]; stats->acceptance = 0.0;
  if (loc_out) {
    std::vector<char> buf((size_t)h->Ns * csz);
    if (cudaMemcpy(buf.data(), d_loc, buf.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
      return cleanup(fail(h, NQ_ERR_CUDA, "observable copy"));
    if (h->f64) memcpy(loc_out, buf.data(), buf.size());
    else {
      const float* f = (const float*)buf.data();
      for (size_t i = 0; i < 2 * (size_t)h->Ns; ++i) loc_out[i] = f[i];
    }
  }
  return cleanup(NQ_OK);
}

nq_status nq_sample(nq_handle* h, uint64_t call_index, int8_t* samples_out, uint8_t* accept_bits) {
  if (h && h->symm && !h->sym_ready) return fail(h, NQ_ERR_STATE, "NDMSymm: no permutations (nq_set_symmetry)");
  if (!h) return NQ_ERR_ARG;
  if (nq_status ts = ensure_tuned(h)) return ts;
  unsigned char* d_bits = nullptr;
  size_t nbits = (size_t)h->B * h->passes * (h->cfg.burn + h->n_record);
  if (accept_bits) CK(cudaMalloc(&d_bits, nbits));
  CK(cudaEventRecord(h->ev[0], h->st));
  nq_status s = stage_sample(h, (uint32_t)call_index, d_bits);
  if (s != NQ_OK) { if (d_bits) cudaFree(d_bits); return s; }
  CK(cudaEventRecord(h->ev[1], h->st));
  CK(cudaMemcpyAsync(h->h_acc, h->d_accepted, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->st));
  if (samples_out) {
    signed char* d_v = nullptr;
    CK(cudaMalloc(&d_v, (size_t)h->Ns * h->nst));
    ++h->launches;
    CK(launch_unpack_int8(h->d_samples, h->nst, h->Ns, h->hilb, d_v, h->st));
    CK(cudaMemcpyAsync(samples_out, d_v, (size_t)h->Ns * h->nst, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    cudaFree(d_v);
  }
  if (d_bits) {
    CK(cudaMemcpyAsync(accept_bits, d_bits, nbits, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    cudaFree(d_bits);
  }
  CK(cudaStreamSynchronize(h->st));
  h->stage_ms[0] = elapsed_ms(h->ev[0], h->ev[1]);
  h->stage_ms[6] = elapsed_ms(h->kev[0], h->kev[1]);
  return NQ_OK;
}

nq_status nq_set_samples(nq_handle* h, const int8_t* samples) {
  if (!h || !samples) return NQ_ERR_ARG;
  signed char* d_v = nullptr;
  CK(cudaMalloc(&d_v, (size_t)h->Ns * h->nst));
  CK(cudaMemcpyAsync(d_v, samples, (size_t)h->Ns * h->nst, cudaMemcpyHostToDevice, h->st));
  ++h->launches;
  CK(launch_pack_int8(d_v, h->nst, h->Ns, h->hilb, h->d_samples, h->st));
  CK(cudaStreamSynchronize(h->st));
  cudaFree(d_v);
  return NQ_OK;
}

nq_status nq_get_samples(nq_handle* h, int8_t* samples_out) {
  if (!h || !samples_out) return NQ_ERR_ARG;
  signed char* d_v = nullptr;
  CK(cudaMalloc(&d_v, (size_t)h->Ns * h->nst));
  ++h->launches;
  CK(launch_unpack_int8(h->d_samples, h->nst, h->Ns, h->hilb, d_v, h->st));
  CK(cudaMemcpyAsync(samples_out, d_v, (size_t)h->Ns * h->nst, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  cudaFree(d_v);
  return NQ_OK;
}

nq_status nq_get_estimates(nq_handle* h, double* loc_out, double* force_out, double* dw_out) {
  if (!h) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_get_estimates");
  CK(cudaStreamSynchronize(h->st));
  if (loc_out) {
    const size_t csz = h->f64 ? sizeof(cpx<double>) : sizeof(cpx<float>);
    std::vector<char> buf((size_t)h->Ns * csz);
    CK(cudaMemcpy(buf.data(), h->d_eloc, buf.size(), cudaMemcpyDeviceToHost));
    if (h->f64) memcpy(loc_out, buf.data(), buf.size());
    else {
      const float* f = (const float*)buf.data();
      for (size_t i = 0; i < 2 * (size_t)h->Ns; ++i) loc_out[i] = f[i];
    }
  }
  double* srcs[2] = {h->fb.force, h->cg ? h->cga.x : h->sb.x};
  double* outs[2] = {force_out, dw_out};
  for (int k = 0; k < 2; ++k) {
    if (!outs[k]) continue;
    if (!srcs[k]) return fail(h, NQ_ERR_STATE, "no %s buffer on this handle", k ? "update" : "force");
    std::vector<double> f(2 * (size_t)h->P);
    CK(cudaMemcpy(f.data(), srcs[k], f.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (h->complex_params && h->real_sr)         // PositiveDefR chain: F and Δw are real
      for (int i = 0; i < h->P; ++i) f[2 * i + 1] = 0.0;
    if (h->complex_params) memcpy(outs[k], f.data(), f.size() * sizeof(double));
    else
      for (int i = 0; i < h->P; ++i) outs[k][i] = f[2 * i];
  }
  return NQ_OK;
}

static nq_status eval_host_batch(nq_handle* h, const int8_t* sigma, int64_t n, double* out, double* grad) {
  if (!h || !sigma || !out || n < 1) return NQ_ERR_ARG;
  if (h->symm && !h->sym_ready) return fail(h, NQ_ERR_STATE, "NDMSymm: no permutations (nq_set_symmetry)");
  for (int64_t i = 0; i < n * h->nst; ++i) {
    int v = sigma[i];
    bool ok = h->hilb == NQ_HILB_SPIN ? (v == 1 || v == -1) : (v == 0 || v == 1);
    if (!ok) return fail(h, NQ_ERR_ARG, "invalid site value %d at %lld", v, (long long)i);
  }
  const size_t csz = h->f64 ? sizeof(cpx<double>) : sizeof(cpx<float>);
  signed char* d_v = nullptr;
  uint64_t* d_bits = nullptr;
  void *d_lp = nullptr, *d_g = nullptr;
  double* d_out = nullptr;
  CK(cudaMalloc(&d_v, (size_t)n * h->nst));
  CK(cudaMalloc(&d_bits, (size_t)n * sizeof(uint64_t)));
  CK(cudaMalloc(&d_lp, (size_t)n * csz));
  if (!h->ndm && !h->chain) CK(cudaMalloc(&d_g, (size_t)n * h->M * csz));
  CK(cudaMemcpyAsync(d_v, sigma, (size_t)n * h->nst, cudaMemcpyHostToDevice, h->st));
  ++h->launches;
  CK(launch_pack_int8(d_v, h->nst, n, h->hilb, d_bits, h->st));
  if (h->diag) CKL(launch_ndm_diag_expand(d_bits, (int)n, h->N, d_bits, h->st));   // logρ(σ,σ)
  if (h->chain) {
    if (grad) CK(cudaMalloc(&d_out, (size_t)2 * h->P * n * sizeof(double)));
    if (h->f64) CKL(launch_chain_eval<double>(chain_dev<double>(h), d_bits, (int)n, nullptr, (cpx<double>*)d_lp,
                                              nullptr, nullptr, 0, d_out, h->st));
    else CKL(launch_chain_eval<float>(chain_dev<float>(h), d_bits, (int)n, nullptr, (cpx<float>*)d_lp, nullptr,
                                      nullptr, 0, d_out, h->st));
  } else if (h->ndm) {
    if (grad) CK(cudaMalloc(&d_out, (size_t)2 * h->P * n * sizeof(double)));
    if (h->f64) CKL(launch_ndm_eval<double>(ndm_eff<double>(h), h->act, d_bits, (int)n, h->hilb, (cpx<double>*)d_lp, nullptr, 0, d_out, h->st));
    else {
      NdmEff<float> e = ndm_eff<float>(h);
      if (h->tc_theta) {        // θ of the given configurations on tcgen05, as in the estimator
        CK(cudaMalloc(&d_g, (size_t)n * h->U * sizeof(cpx<float>)));
        CKL(launch_theta_bf16x2(h->d_theta_img, h->theta_terms, h->U, h->N2, e.b, d_bits, (int)n, h->hilb,
                                (cpx<float>*)d_g, h->sb.status, h->st));
        e.theta = (const cpx<float>*)d_g;
      }
      CKL(launch_ndm_eval<float>(e, h->act, d_bits, (int)n, h->hilb, (cpx<float>*)d_lp, nullptr, 0, d_out, h->st));
    }
  } else if (h->f64) CKL(launch_rbm_eval<double>(rbm_dev<double>(h), d_bits, (int)n, nullptr, (cpx<double>*)d_lp, (cpx<double>*)d_g, nullptr, h->st));
  else if (h->tc_theta) {
    const RbmDev<float> d = rbm_dev<float>(h);
    CKL(launch_theta_bf16x2(h->d_theta_img, h->theta_terms, h->M, h->N, d.b, d_bits, (int)n, h->hilb, (cpx<float>*)d_g,
                            h->sb.status, h->st));
    CKL(launch_rbm_eval<float>(d, d_bits, (int)n, nullptr, (cpx<float>*)d_lp, (cpx<float>*)d_g, nullptr, h->st, 1));
  } else CKL(launch_rbm_eval<float>(rbm_dev<float>(h), d_bits, (int)n, nullptr, (cpx<float>*)d_lp, (cpx<float>*)d_g, nullptr, h->st));
  std::vector<double> lp(2 * n);
  if (h->f64) CK(cudaMemcpyAsync(lp.data(), d_lp, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  else {
    std::vector<float> f(2 * n);
    CK(cudaMemcpyAsync(f.data(), d_lp, 2 * n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (int64_t i = 0; i < 2 * n; ++i) lp[i] = f[i];
  }
  if (grad && !h->ndm && !h->chain) {
    CK(cudaMalloc(&d_out, (size_t)2 * h->P * n * sizeof(double)));
    if (h->f64) CKL(launch_rbm_grad_matrix<double>(d_bits, (int)n, h->N, h->M, h->hilb, (cpx<double>*)d_g, d_out, h->st));
    else CKL(launch_rbm_grad_matrix<float>(d_bits, (int)n, h->N, h->M, h->hilb, (cpx<float>*)d_g, d_out, h->st));
    CK(cudaMemcpyAsync(grad, d_out, (size_t)2 * h->P * n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  }
  if (grad && (h->ndm || h->chain)) CK(cudaMemcpyAsync(grad, d_out, (size_t)2 * h->P * n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  memcpy(out, lp.data(), 2 * n * sizeof(double));
  cudaFree(d_v); cudaFree(d_bits); cudaFree(d_lp); cudaFree(d_g);
  if (d_out) cudaFree(d_out);
  return NQ_OK;
}

nq_status nq_logpsi(nq_handle* h, const int8_t* sigma, int64_t n, double* out) {
  return eval_host_batch(h, sigma, n, out, nullptr);
}

nq_status nq_logpsi_grad(nq_handle* h, const int8_t* sigma, int64_t n, double* out, double* grad) {
  return eval_host_batch(h, sigma, n, out, grad);
}

nq_status nq_estimate(nq_handle* h, nq_measurement* stats, double* loc_out, double* force_out) {
  if (!h) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_estimate");
  if (h->symm && !h->sym_ready) return fail(h, NQ_ERR_STATE, "NDMSymm: no permutations (nq_set_symmetry)");
  if (!h->has_op) return fail(h, NQ_ERR_STATE, "no operator set (nq_set_operator)");
  nq_status s;
  CK(cudaEventRecord(h->ev[1], h->st));
  if ((s = stage_eval(h)) != NQ_OK) return s;
  CK(cudaEventRecord(h->ev[2], h->st));
  if ((s = stage_force(h)) != NQ_OK) return s;
  CK(cudaEventRecord(h->ev[3], h->st));
  if ((s = stage_S(h)) != NQ_OK) return s;
  CK(cudaEventRecord(h->ev[4], h->st));
  CK(cudaMemcpyAsync(h->h_stats, h->d_stats, 6 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->stage_ms[1] = elapsed_ms(h->ev[1], h->ev[2]);
  h->stage_ms[2] = elapsed_ms(h->ev[2], h->ev[3]);
  h->stage_ms[3] = elapsed_ms(h->ev[3], h->ev[4]);
  h->stage_ms[7] = elapsed_ms(h->kev[2], h->kev[3]);
  fill_measurement(h, stats);
  if (!std::isfinite(h->h_stats[0]) || !std::isfinite(h->h_stats[1]))
    return fail(h, NQ_ERR_NAN, "non-finite local estimator mean");
  const size_t csz = h->f64 ? sizeof(cpx<double>) : sizeof(cpx<float>);
  if (loc_out) {
    std::vector<char> buf((size_t)h->Ns * csz);
    CK(cudaMemcpy(buf.data(), h->d_eloc, buf.size(), cudaMemcpyDeviceToHost));
    if (h->f64) memcpy(loc_out, buf.data(), buf.size());
    else {
      const float* f = (const float*)buf.data();
      for (size_t i = 0; i < 2 * (size_t)h->Ns; ++i) loc_out[i] = f[i];
    }
  }
  if (force_out) {
    std::vector<double> f(2 * (size_t)h->P);
    CK(cudaMemcpy(f.data(), h->fb.force, f.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (h->complex_params && h->real_sr)         // PositiveDefR chain: F is real
      for (int i = 0; i < h->P; ++i) f[2 * i + 1] = 0.0;
    if (h->complex_params) memcpy(force_out, f.data(), f.size() * sizeof(double));
    else
      for (int i = 0; i < h->P; ++i) force_out[i] = f[2 * i];
  }
  return NQ_OK;
}

nq_status nq_set_wait_limit(nq_handle* h, uint64_t limit_ns) {
  if (!h) return NQ_ERR_ARG;
  const uint64_t v = limit_ns ? limit_ns : kNqWaitNs;
  h->sb.wait_ns = v;
  h->cga.wait_ns = v;
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  return NQ_OK;
}

nq_status nq_set_time_evolution(nq_handle* h, int32_t on) {
  if (!h) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_set_time_evolution");
  if (on && !h->d_frhs) CK(cudaMalloc(&h->d_frhs, 2 * sizeof(double) * (size_t)h->P));
  if ((on != 0) != h->time_evo && h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  h->time_evo = on != 0;
  return NQ_OK;
}

nq_status nq_set_sr_tolerance(nq_handle* h, double tol, int32_t maxiter) {
  if (!h || !(tol > 0.0) || maxiter < 1) return NQ_ERR_ARG;
  h->cg_tol = tol;
  h->cg_maxiter = maxiter;
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  return NQ_OK;
}

nq_status nq_sr_info(nq_handle* h, double* out2) {
  if (!h || !out2) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_sr_info");
  if (!h->h_cginfo) CK(cudaMallocHost((void**)&h->h_cginfo, 2 * sizeof(double)));
  const double* src = h->cg ? h->cga.info : h->sb.info;
  if (!src) return fail(h, NQ_ERR_STATE, "no SR solve on this handle");
  CK(cudaMemcpyAsync(h->h_cginfo, src, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  out2[0] = h->h_cginfo[0];
  out2[1] = h->h_cginfo[1];
  return NQ_OK;
}

nq_status nq_get_sr_matrix(nq_handle* h, double* s_out) {
  if (h && h->cg) return fail(h, NQ_ERR_STATE, "S is not formed by the matrix-free SR solve (NQ_SR_CG)");
  if (!h || !s_out) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_get_sr_matrix");
  std::vector<double> S(2 * (size_t)h->P * h->P);
  CK(cudaMemcpyAsync(S.data(), h->d_S, S.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (h->complex_params) memcpy(s_out, S.data(), S.size() * sizeof(double));
  else
    for (size_t i = 0; i < (size_t)h->P * h->P; ++i) s_out[i] = S[2 * i];
  return NQ_OK;
}

nq_status nq_precondition(nq_handle* h, int32_t kind, double eps, double lam0, double b,
                          double lam_min, int32_t iter, double* dw_out) {
  if (!h) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_precondition");
  if (kind < 0 || kind > 2) return fail(h, NQ_ERR_ARG, "unknown precondition kind %d", kind);
  double lam = 0.0;
  if (kind == 1) lam = std::max(lam0 * std::pow(b, (double)iter), lam_min);
  CK(cudaEventRecord(h->ev[4], h->st));
  nq_status s = stage_solve(h, kind, eps, lam);
  if (s != NQ_OK) return s;
  CK(cudaEventRecord(h->ev[5], h->st));
  if ((s = check_status_word(h)) != NQ_OK) return s;
  h->stage_ms[4] = elapsed_ms(h->ev[4], h->ev[5]);
  for (int k = 0; k < 4; ++k) h->stage_ms[8 + k] = elapsed_ms(h->sev[k + 1], h->sev[k + 2]);
  if (dw_out) {
    std::vector<double> x(2 * (size_t)h->P);
    CK(cudaMemcpy(x.data(), h->sb.x, x.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (h->complex_params) memcpy(dw_out, x.data(), x.size() * sizeof(double));
    else
      for (int i = 0; i < h->P; ++i) dw_out[i] = x[2 * i];
  }
  return NQ_OK;
}

nq_status nq_update_descent(nq_handle* h, double lr) {
  if (!h) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_update_descent");
  CK(cudaEventRecord(h->ev[5], h->st));
  nq_status s = stage_update(h, lr);
  if (s != NQ_OK) return s;
  CK(cudaEventRecord(h->ev[6], h->st));
  CK(cudaStreamSynchronize(h->st));
  h->stage_ms[5] = elapsed_ms(h->ev[5], h->ev[6]);
  if (h->graph) { /* parameters live on the device; the graph stays valid */ }
  return NQ_OK;
}

// Whole iteration; replays a captured graph once built.  The call index
// reaches the sampler through a pinned host word copied by the first graph
// node, so one graph serves every iteration.
nq_status nq_vmc_step(nq_handle* h, uint64_t call_index, double eps, double lr, nq_measurement* stats) {
  if (!h) return NQ_ERR_ARG;
  NQ_REJECT_DIAG(h, "nq_vmc_step");
  if (h->symm && !h->sym_ready) return fail(h, NQ_ERR_STATE, "NDMSymm: no permutations (nq_set_symmetry)");
  if (!h->has_op) return fail(h, NQ_ERR_STATE, "no operator set (nq_set_operator)");
  // every graph launch of this handle ends with a synchronisation, so no
  // graph is in flight here and the pinned call word is free; work queued by
  // asynchronous calls (nq_set_params) runs ahead of the graph on the stream
  if (h->graph && (h->graph_eps != eps || h->graph_lr != lr)) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  if (nq_status ts = ensure_tuned(h)) return ts;
  *h->h_call = (uint32_t)call_index;
  if (!h->graph) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    h->capturing = true;
    h->side_ok = true;
    const int64_t before = h->launches;
    nq_status s = NQ_OK;
    cudaError_t ce = cudaMemcpyAsync(h->d_call, h->h_call, sizeof(uint32_t), cudaMemcpyHostToDevice, h->st);
    if (ce != cudaSuccess) s = fail(h, NQ_ERR_CUDA, "capture memcpy: %s", cudaGetErrorString(ce));
    if (s == NQ_OK) s = stage_sample(h, 0, nullptr, h->d_call);
    if (s == NQ_OK) s = stage_eval(h);
    if (s == NQ_OK) s = stage_force(h);
    if (s == NQ_OK) s = stage_S(h);
    if (s == NQ_OK) s = stage_solve(h, 0, eps, 0.0);
    if (s == NQ_OK) s = stage_update(h, lr);
    if (h->side_pending) {           // join the side branch before the capture ends
      cudaError_t je = cudaStreamWaitEvent(h->st, h->ev_join, 0);
      if (je != cudaSuccess && s == NQ_OK) s = fail(h, NQ_ERR_CUDA, "capture join: %s", cudaGetErrorString(je));
      h->side_pending = false;
    }
    h->side_ok = false;
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    h->capturing = false;
    h->graph_kernels = h->launches - before;
    h->launches = before;
    if (s != NQ_OK) { if (g) cudaGraphDestroy(g); return s; }
    CK(e);
    CK(cudaGraphInstantiate(&h->graph, g, 0));
    cudaGraphDestroy(g);
    h->graph_eps = eps;
    h->graph_lr = lr;
  }
  CK(cudaGraphLaunch(h->graph, h->st));
  h->launches += h->graph_kernels;
  CK(cudaMemcpyAsync(h->h_stats, h->d_stats, 6 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->h_acc, h->d_accepted, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->h_status, h->sb.status, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  nq_status s = check_status_word(h, h->h_status);
  fill_measurement(h, stats);
  if (s != NQ_OK) return s;
  if (!std::isfinite(h->h_stats[0]) || !std::isfinite(h->h_stats[1]))
    return fail(h, NQ_ERR_NAN, "non-finite local estimator mean");
  return NQ_OK;
}

nq_status nq_tuning(nq_handle* h, int32_t* out, int32_t n) {
  if (!h || !out || n < 1) return NQ_ERR_ARG;
  if (nq_status ts = ensure_tuned(h)) return ts;
  const int32_t v[3] = {h->sampler_lanes, h->gram_ksplit, h->sampler_block};
  for (int i = 0; i < n && i < 3; ++i) out[i] = v[i];
  return NQ_OK;
}

nq_status nq_stage_times(nq_handle* h, float* ms12) {
  if (!h || !ms12) return NQ_ERR_ARG;
  memcpy(ms12, h->stage_ms, sizeof(h->stage_ms));
  return NQ_OK;
}

nq_status nq_bench_steps(nq_handle* h, uint64_t call0, int32_t n_steps, double eps, double lr,
                         int64_t flush_bytes, float* ms_out) {
  if (!h || !ms_out || n_steps < 1 || flush_bytes < 0) return NQ_ERR_ARG;
  // build (or rebuild) the graph with one ordinary step
  nq_measurement m;
  nq_status s = nq_vmc_step(h, call0, eps, lr, &m);
  if (s != NQ_OK) return s;
  if (flush_bytes > 0 && (size_t)flush_bytes > h->flush_bytes) {
    if (h->d_flush) cudaFree(h->d_flush);
    h->d_flush = nullptr;
    CK(cudaMalloc(&h->d_flush, (size_t)flush_bytes));
    h->flush_bytes = (size_t)flush_bytes;
  }
  cudaEvent_t* evs = new cudaEvent_t[2 * n_steps];
  for (int i = 0; i < 2 * n_steps; ++i) cudaEventCreate(&evs[i]);
  for (int i = 0; i < n_steps; ++i) {
    if (flush_bytes > 0) CK(cudaMemsetAsync(h->d_flush, i & 0xff, (size_t)flush_bytes, h->st));
    CK(cudaStreamSynchronize(h->st));
    *h->h_call = (uint32_t)(call0 + 1 + i);
    CK(cudaEventRecord(evs[2 * i], h->st));
    CK(cudaGraphLaunch(h->graph, h->st));
    h->launches += h->graph_kernels;
    CK(cudaEventRecord(evs[2 * i + 1], h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  for (int i = 0; i < n_steps; ++i) ms_out[i] = elapsed_ms(evs[2 * i], evs[2 * i + 1]);
  for (int i = 0; i < 2 * n_steps; ++i) cudaEventDestroy(evs[i]);
  delete[] evs;
  return check_status_word(h);
}

}  // extern "C"

// ===========================================================================
// Many independent problems per step (nq_batch_*): the sampler, the
// estimator and the SR inversion of all problems run as one launch each; the
// per-problem force/S/solve-refinement/update stages run as parallel branches
// of the same CUDA graph.
// ===========================================================================
struct nq_batch {
  std::vector<nq_handle*> hs;
  std::string err;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t graph = nullptr;
  double geps = -1, glr = -1;
  int64_t graph_kernels = 0;
  uint32_t* h_call = nullptr;           // pinned
  uint32_t* d_call = nullptr;
  SamplerJob<float>* d_sjobs = nullptr;
  EvalJob<float>* d_ejobs = nullptr;
  SweepJob* d_wjobs = nullptr;
  int* d_sblk = nullptr;                // [np+1] sampler block starts
  int* d_eblk = nullptr;                // [np+1] estimator block starts
  int* d_wcta = nullptr;                // [np+1] inversion CTA starts
  int* d_rcta = nullptr;                // [np+1] refinement CTA starts
  int s_blocks = 0, e_blocks = 0, w_ctas = 0, r_ctas = 0, M_max = 0, N_max = 0, act = 0;
  int lanes = 0, eval_T = 0;
  void* d_ctl = nullptr;                // per-problem barrier blocks, 64 B each
  unsigned long long* d_acc = nullptr;  // [np] accepted-move counters
  double** d_stat_src = nullptr;        // [np] -> each problem's d_stats
  int** d_status_src = nullptr;         // [np] -> each problem's status word
  double* d_gather = nullptr;           // [np][8]
  double* h_gather = nullptr;           // pinned [np][8]
  int64_t launches = 0;
  // grouped SR stages (every stage of all problems one launch): equal sample
  // counts and S on tcgen05 (TF32 or 3xTF32)
  bool grouped = false;
  int split3 = 0;
  float* d_Xall = nullptr;              // stacked X of all problems [Σ 2P][Ns_pad]
  float* d_Xlo_all = nullptr;           // its 3xTF32 low part
  int rows_total = 0, Ns_pad = 0;
  float* d_slots = nullptr;             // Gram partial blocks of all problems
  void* d_geom = nullptr;               // Gram geometry
  GramGroupPlan gplan;
  SrJob* d_jobs = nullptr;
  int* d_prefix = nullptr;              // the prefix arrays of SrGroup, 9 x (np + 1)
  SrGroup grp;
};

namespace {

nq_status bfail(nq_batch* b, nq_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCK(expr)                                                                          \
  do {                                                                                     \
    cudaError_t _e = (expr);                                                               \
    if (_e != cudaSuccess)                                                                 \
      return bfail(b, NQ_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                   __FILE__, __LINE__);                                                    \
  } while (0)

__global__ void batch_gather_kernel(int np, double* const* __restrict__ stats, int* const* __restrict__ status,
                                    const unsigned long long* __restrict__ acc, double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  for (int k = 0; k < 6; ++k) out[8 * p + k] = stats[p][k];
  out[8 * p + 6] = (double)acc[p];
  out[8 * p + 7] = (double)*status[p];
}

// problem p gets CTAs in proportion to its inversion work (nblk^3), at least
// one and at most its number of column blocks
void split_ctas(const std::vector<int>& P, int total, std::vector<int>& start) {
  const int np = (int)P.size();
  std::vector<double> w(np);
  double sum = 0;
  for (int p = 0; p < np; ++p) {
    const double nb = (P[p] + 31) / 32;
    w[p] = nb * nb * nb;
    sum += w[p];
  }
  const int spare = std::max(0, total - np);
  start.assign(np + 1, 0);
  for (int p = 0; p < np; ++p) {
    const int nb = (P[p] + 31) / 32;
    int extra = (int)std::floor(spare * w[p] / sum);
    extra = std::min(extra, std::max(0, nb - 1));
    start[p + 1] = start[p] + 1 + extra;
  }
}

// CTAs of the grouped refinement: its passes are GEMVs (the FP64 residual on
// GB300's few FP64 units dominates), so the split follows P², with at least
// 8 rows (one per warp) per CTA
void split_ctas_refine(const std::vector<int>& P, int total, std::vector<int>& start) {
  const int np = (int)P.size();
  std::vector<double> w(np);
  double sum = 0;
  for (int p = 0; p < np; ++p) {
    w[p] = (double)P[p] * P[p];
    sum += w[p];
  }
  const int spare = std::max(0, total - np);
  start.assign(np + 1, 0);
  for (int p = 0; p < np; ++p) {
    int extra = (int)std::floor(spare * w[p] / sum);
    extra = std::min(extra, std::max(0, P[p] / 8 - 1));
    start[p + 1] = start[p] + 1 + extra;
  }
}

// Grouped SR stages: one stacked X for all problems (each handle's X becomes
// a row slice of it), the problem table and the prefix arrays of every
// grouped kernel.  Needs equal sample counts and S on tcgen05 (TF32 or
// 3xTF32); otherwise the step keeps one graph branch per problem.
nq_status batch_setup_grouped(nq_batch* b) {
  const int np = (int)b->hs.size();
  const int sp = b->hs[0]->cfg.s_precision;
  if (sp != NQ_S_TF32 && sp != NQ_S_TF32X3) return NQ_OK;
  for (nq_handle* h : b->hs)
    if (h->Ns != b->hs[0]->Ns || h->cfg.s_precision != sp || h->Ns_pad != b->hs[0]->Ns_pad) return NQ_OK;
  b->split3 = sp == NQ_S_TF32X3 ? 1 : 0;
  b->Ns_pad = b->hs[0]->Ns_pad;
  std::vector<int> rows(np), off(np);
  int tot = 0;
  for (int p = 0; p < np; ++p) {
    rows[p] = 2 * b->hs[p]->P;
    off[p] = tot;
    tot += rows[p];
  }
  b->rows_total = tot;
  BCK(cudaMalloc(&b->d_Xall, (size_t)tot * b->Ns_pad * sizeof(float) + 16));
  if (b->split3) BCK(cudaMalloc(&b->d_Xlo_all, (size_t)tot * b->Ns_pad * sizeof(float) + 16));
  b->gplan = gram_group_plan(rows, b->Ns_pad);
  BCK(cudaMalloc(&b->d_slots, gram_group_partial_elems(b->gplan) * sizeof(float) + 16));
  BCK(cudaMalloc(&b->d_geom, gram_group_geom_bytes(np)));
  BCK(gram_group_upload(b->gplan, b->d_geom, b->st));
  std::vector<SrJob> jobs(np);
  std::vector<int> pre(9 * (size_t)(np + 1), 0);
  auto P_ = [&](int k, int p) -> int& { return pre[(size_t)k * (np + 1) + p]; };
  size_t fsmem = 0;
  for (int p = 0; p < np; ++p) {
    nq_handle* h = b->hs[p];
    // the handle's own X is replaced by its slice of the stacked X
    if (!h->x_borrowed) {
      cudaFree(h->d_X);
      if (h->d_Xlo) cudaFree(h->d_Xlo);
    }
    h->d_X = b->d_Xall + (size_t)off[p] * b->Ns_pad;
    h->d_Xlo = b->split3 ? b->d_Xlo_all + (size_t)off[p] * b->Ns_pad : nullptr;
    h->x_borrowed = true;
    SrJob& j = jobs[p];
    j.N = h->N; j.M = h->M; j.P = h->P; j.hilb = h->hilb; j.act = h->act; j.Ns = h->Ns; j.B = h->B; j.L = h->L;
    j.Ns_pad = h->Ns_pad;
    j.force_CH = rbm_force_chunk(h->N, h->M, h->Ns);
    j.force_nblk = (h->Ns + j.force_CH - 1) / j.force_CH;
    if (j.force_nblk > h->force_nblk)      // the handle's partial buffers hold force_nblk blocks
      return bfail(b, NQ_ERR_STATE, "problem %d: grouped force needs %d partial blocks, %d allocated", p,
                   j.force_nblk, h->force_nblk);
    fsmem = std::max(fsmem, rbm_force_smem(h->N, h->M, h->Ns));
    j.samples = h->d_samples;
    j.g = reinterpret_cast<const float2*>(h->d_g);
    j.eloc = reinterpret_cast<const float2*>(h->d_eloc);
    j.fb = h->fb;
    j.chainstats = h->d_chainstats;
    j.stats = h->d_stats;
    j.X = h->d_X;
    j.Xlo = h->d_Xlo;
    j.G = h->d_G;
    j.S = h->d_S;
    j.W = h->sb.W;
    j.x = h->sb.x;
    j.r = h->sb.r;
    j.rf = h->sb.rf;
    j.norms = h->sb.norms;
    j.status = h->sb.status;
    j.master = h->d_master;
    j.p32 = h->d_p32;
    j.t0 = reinterpret_cast<float2*>(h->d_tab[0]);
    j.t1 = reinterpret_cast<float2*>(h->d_tab[1]);
    j.t2 = reinterpret_cast<float2*>(h->d_tab[2]);
    const int units[9] = {j.force_nblk, h->P + 1, h->P, (h->B + 63) / 64, ((h->Ns_pad + 1023) / 1024) * (h->M + 1),
                          h->P * h->P, ((h->P + 31) / 32) * ((h->P + 31) / 32), 2 * h->P, h->N * h->M};
    for (int k = 0; k < 9; ++k) P_(k, p + 1) = P_(k, p) + units[k];
  }
  BCK(cudaMalloc((void**)&b->d_jobs, np * sizeof(SrJob)));
  BCK(cudaMalloc((void**)&b->d_prefix, pre.size() * sizeof(int)));
  BCK(cudaMemcpy(b->d_jobs, jobs.data(), np * sizeof(SrJob), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_prefix, pre.data(), pre.size() * sizeof(int), cudaMemcpyHostToDevice));
  SrGroup& g = b->grp;
  g.np = np;
  g.jobs = b->d_jobs;
  const int* d = b->d_prefix;
  auto dp = [&](int k) { return d + (size_t)k * (np + 1); };
  g.force_blk = dp(0); g.force_blocks = P_(0, np); g.force_smem = fsmem;
  g.force_warp = dp(1); g.force_warps = P_(1, np);
  g.pelem = dp(2); g.pelems = P_(2, np);
  g.stat_blk = dp(3); g.stat_blocks = P_(3, np);
  g.x_blk = dp(4); g.x_blocks = P_(4, np);
  g.pp_elem = dp(5); g.pp_elems = P_(5, np);
  g.fill_blk = dp(6); g.fill_blocks = P_(6, np);
  g.master_elem = dp(7); g.master_elems = P_(7, np);
  g.tab_elem = dp(8); g.tab_elems = P_(8, np);
  g.P_max = 0;
  for (nq_handle* h : b->hs) g.P_max = std::max(g.P_max, h->P);
  b->grouped = true;
  return NQ_OK;
}

nq_status batch_build_tables(nq_batch* b) {
  const int np = (int)b->hs.size();
  std::vector<SamplerJob<float>> sj(np);
  std::vector<EvalJob<float>> ej(np);
  std::vector<SweepJob> wj(np);
  std::vector<int> sblk(np + 1, 0), eblk(np + 1, 0), Ps(np);
  std::vector<double*> sp(np);
  std::vector<int*> stp(np);
  b->M_max = 0;
  b->N_max = 0;
  for (nq_handle* h : b->hs) {
    b->M_max = std::max(b->M_max, h->M);
    b->N_max = std::max(b->N_max, h->N);
  }
  b->eval_T = rbm_eval_threads(b->M_max);
  const int cpb = 256 / b->lanes;          // chains per sampler block
  // sampler jobs longest first (steps per chain x units per lane, the narrower
  // loop of the batch kernel included), so the last wave holds short blocks
  const int hpl_max = (b->M_max + b->lanes - 1) / b->lanes, hpl_lo = (hpl_max + 1) / 2;
  std::vector<int> order(np);
  std::vector<double> work(np);
  for (int p = 0; p < np; ++p) {
    nq_handle* h = b->hs[p];
    const int hpl = (hpl_lo < hpl_max && h->M <= b->lanes * hpl_lo) ? hpl_lo : hpl_max;
    work[p] = (double)h->passes * (h->cfg.burn + h->n_record) * (hpl + 2);
    order[p] = p;
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work[x] > work[y]; });
  for (int q = 0; q < np; ++q) {
    nq_handle* h = b->hs[order[q]];
    SamplerRun run;
    run.B = h->B; run.L = h->L; run.burn = h->cfg.burn; run.passes = h->passes;
    run.n_record = h->n_record; run.write_last_at_end = h->write_last;
    run.k0 = (uint32_t)(h->cfg.seed & 0xffffffffu);
    run.k1 = (uint32_t)(h->cfg.seed >> 32);
    run.call_ptr = b->d_call;
    run.samples = h->d_samples;
    run.accepted = b->d_acc + order[q];
    sj[q].net = rbm_dev<float>(h);
    sj[q].run = run;
    sblk[q + 1] = sblk[q] + (h->B + cpb - 1) / cpb;
  }
  for (int p = 0; p < np; ++p) {
    nq_handle* h = b->hs[p];
    ej[p].net = rbm_dev<float>(h);
    ej[p].samples = h->d_samples;
    ej[p].Ns = h->Ns;
    ej[p].op = h->op;
    ej[p].has_op = 1;
    ej[p].logpsi = (cpx<float>*)h->d_logpsi;
    ej[p].g = (cpx<float>*)h->d_g;
    ej[p].eloc = (cpx<float>*)h->d_eloc;
    eblk[p + 1] = eblk[p] + (h->Ns + b->eval_T - 1) / b->eval_T;
    wj[p].W = h->sb.W;
    wj[p].P = h->P;
    wj[p].ctl = (char*)b->d_ctl + (size_t)p * 64;
    wj[p].status = h->sb.status;
    wj[p].work = h->sb.work;
    Ps[p] = h->P;
    sp[p] = h->d_stats;
    stp[p] = h->sb.status;
  }
  int sms = 0, dev = 0;
  BCK(cudaGetDevice(&dev));
  BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // the grouped step's inversion and refinement are throughput-bound: up to
  // two co-resident CTAs per SM
  const int slots = sms * (b->grouped ? batch_solve_ctas_per_sm() : 1);
  std::vector<int> wcta;
  split_ctas(Ps, slots, wcta);
  if (wcta[np] > slots)
    return bfail(b, NQ_ERR_UNSUPPORTED, "%d problems exceed the %d CTAs of the inversion launch", np, slots);
  b->s_blocks = sblk[np];
  b->e_blocks = eblk[np];
  b->w_ctas = wcta[np];
  std::vector<int> rcta;
  split_ctas_refine(Ps, slots, rcta);
  b->r_ctas = rcta[np];
  BCK(cudaMemcpy(b->d_sjobs, sj.data(), np * sizeof(SamplerJob<float>), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_ejobs, ej.data(), np * sizeof(EvalJob<float>), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_wjobs, wj.data(), np * sizeof(SweepJob), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_sblk, sblk.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_eblk, eblk.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_wcta, wcta.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_rcta, rcta.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_stat_src, sp.data(), np * sizeof(double*), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_status_src, stp.data(), np * sizeof(int*), cudaMemcpyHostToDevice));
  return NQ_OK;
}

// lanes per chain of the many-problem sampler: every candidate runs the
// batch's real schedule twice (the first launch warms up) and the fastest wins
nq_status batch_tune(nq_batch* b) {
  if (b->lanes) return NQ_OK;
  int cand[4];
  int M_max = 0, N_max = 0;
  for (nq_handle* h : b->hs) {
    M_max = std::max(M_max, h->M);
    N_max = std::max(N_max, h->N);
  }
  const int nc = rbm_sampler_valid_lanes(N_max, M_max, 8, cand, 4);
  if (nc == 0) return bfail(b, NQ_ERR_UNSUPPORTED, "no sampler instantiation for %d hidden units", M_max);
  cudaEvent_t e0, e1;
  BCK(cudaEventCreate(&e0));
  BCK(cudaEventCreate(&e1));
  *b->h_call = 0xFFFFFFFFu;
  BCK(cudaMemcpy(b->d_call, b->h_call, sizeof(uint32_t), cudaMemcpyHostToDevice));
  int best = cand[0];
  float best_ms = 1e30f;
  for (int c = 0; c < nc; ++c) {
    b->lanes = cand[c];
    if (nq_status s = batch_build_tables(b)) return s;
    float best_c = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {      // first launch warms up; fastest of the other three
      float ms = 0.f;
      BCK(cudaEventRecord(e0, b->st));
      BCK(launch_rbm_sampler_batch<float>(b->d_sjobs, b->d_sblk, (int)b->hs.size(), b->s_blocks, b->M_max,
                                          b->N_max, b->act, b->lanes, b->st));
      ++b->launches;
      BCK(cudaEventRecord(e1, b->st));
      BCK(cudaEventSynchronize(e1));
      BCK(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0) best_c = std::min(best_c, ms);
    }
    if (best_c < best_ms) {
      best_ms = best_c;
      best = cand[c];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->lanes = best;
  return batch_build_tables(b);
}

nq_status batch_capture(nq_batch* b, double eps, double lr) {
  const int np = (int)b->hs.size();
  cudaGraph_t g = nullptr;
  BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  for (nq_handle* h : b->hs) h->capturing = true;
  const int64_t before = b->launches;
  int64_t hbefore = 0;
  for (nq_handle* h : b->hs) hbefore += h->launches;
  nq_status s = NQ_OK;
  auto ck = [&](cudaError_t e, const char* what) {
    if (s == NQ_OK && e != cudaSuccess) s = bfail(b, NQ_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  };
  ck(cudaMemcpyAsync(b->d_call, b->h_call, sizeof(uint32_t), cudaMemcpyHostToDevice, b->st), "call copy");
  ck(cudaMemsetAsync(b->d_acc, 0, np * sizeof(unsigned long long), b->st), "acc reset");
  ck(launch_rbm_sampler_batch<float>(b->d_sjobs, b->d_sblk, np, b->s_blocks, b->M_max, b->N_max, b->act, b->lanes,
                                     b->st), "batched sampler");
  ck(launch_rbm_eval_batch<float>(b->d_ejobs, b->d_eblk, np, b->e_blocks, b->M_max, b->N_max, b->act, b->eval_T,
                                  b->st), "batched estimator");
  b->launches += 2;
  if (b->grouped) {
    // every SR stage of all problems as one launch (one kernel per stage)
    const SrGroup& gp = b->grp;
    ck(launch_force_group(gp, b->st), "grouped force");
    ck(launch_stats_group(gp, b->st), "grouped statistics");
    ck(launch_build_X_group(gp, b->split3, b->st), "grouped X");
    ck(launch_gram_group(b->d_Xall, b->d_Xlo_all, b->rows_total, b->Ns_pad, b->split3, b->gplan, b->d_geom, gp,
                         b->d_slots, b->hs[0]->sb.status, b->st), "grouped S accumulation");
    ck(launch_assemble_shift_group(gp, eps, b->st), "grouped S and shift");
    ck(launch_spd_inverse_batch(b->d_wjobs, b->d_wcta, np, b->w_ctas, b->d_ctl, (size_t)np * 64, b->st),
       "batched inversion");
    ck(launch_fill_group(gp, b->st), "grouped fill");
    ck(launch_refine_group(gp, b->d_rcta, b->r_ctas, b->d_ctl, eps, kSolveRefine, b->st), "grouped refinement");
    ck(launch_update_group(gp, lr, b->st), "grouped update");
    b->launches += 14;
  } else {
    // branches: force + statistics, S, shifted copy
    ck(cudaEventRecord(b->fork, b->st), "fork");
    for (int p = 0; p < np && s == NQ_OK; ++p) {
      nq_handle* h = b->hs[p];
      ck(cudaStreamWaitEvent(h->st, b->fork, 0), "branch");
      if (s == NQ_OK) s = stage_force(h);
      if (s == NQ_OK) s = stage_S(h);
      if (s == NQ_OK) {
        ck(launch_sr_shift(h->sb, h->P, 0, eps, 0.0, h->st), "shift");
        ++h->launches;
      }
      ck(cudaEventRecord(b->join[p], h->st), "join");
      ck(cudaStreamWaitEvent(b->st, b->join[p], 0), "join wait");
    }
    // one cooperative launch inverts every problem's shifted S
    ck(launch_spd_inverse_batch(b->d_wjobs, b->d_wcta, np, b->w_ctas, b->d_ctl, (size_t)np * 64, b->st),
       "batched inversion");
    ++b->launches;
    ck(cudaEventRecord(b->fork, b->st), "fork 2");
    for (int p = 0; p < np && s == NQ_OK; ++p) {
      nq_handle* h = b->hs[p];
      ck(cudaStreamWaitEvent(h->st, b->fork, 0), "branch 2");
      if (s == NQ_OK) {
        ck(launch_sr_finish(h->sb, h->P, h->fb.force, 0, eps, 0.0, !h->complex_params, kSolveRefineBatch, h->st),
           "solve");
        h->launches += 2 + 3 * (kSolveRefineBatch + 1);
      }
      if (s == NQ_OK) s = stage_update(h, lr);
      ck(cudaEventRecord(b->join[p], h->st), "join 2");
      ck(cudaStreamWaitEvent(b->st, b->join[p], 0), "join wait 2");
    }
  }
  if (s == NQ_OK) {
    batch_gather_kernel<<<(np + 63) / 64, 64, 0, b->st>>>(np, b->d_stat_src, b->d_status_src, b->d_acc,
                                                         b->d_gather);
    ck(cudaGetLastError(), "gather");
    ++b->launches;
  }
  cudaError_t e = cudaStreamEndCapture(b->st, &g);
  int64_t hafter = 0;
  for (nq_handle* h : b->hs) {
    h->capturing = false;
    hafter += h->launches;
  }
  b->graph_kernels = (b->launches - before) + (hafter - hbefore);
  b->launches = before;
  if (s != NQ_OK) {
    if (g) cudaGraphDestroy(g);
    return s;
  }
  BCK(e);
  BCK(cudaGraphInstantiate(&b->graph, g, 0));
  cudaGraphDestroy(g);
  b->geps = eps;
  b->glr = lr;
  return NQ_OK;
}

}  // namespace

extern "C" {

nq_status nq_batch_create(const nq_config* cfgs, int32_t n, nq_batch** out) {
  if (!cfgs || !out || n < 1 || n > 1024) return NQ_ERR_ARG;
  *out = nullptr;
  for (int p = 0; p < n; ++p) {
    const nq_config& c = cfgs[p];
    if (c.network != NQ_NET_RBM || c.eval_precision != NQ_EVAL_F32 || c.sr_algorithm != NQ_SR_DIRECT ||
        c.sampler_kind != NQ_SAMPLER_METROPOLIS)
      return NQ_ERR_UNSUPPORTED;
    if (c.activation != cfgs[0].activation || c.hilbert != cfgs[0].hilbert) return NQ_ERR_UNSUPPORTED;
  }
  nq_batch* b = new nq_batch();
  auto cleanup = [&](nq_status s) {
    nq_batch_destroy(b);
    return s;
  };
  b->act = cfgs[0].activation;
  for (int p = 0; p < n; ++p) {
    nq_handle* h = nullptr;
    nq_status s = nq_create(&cfgs[p], &h);
    if (s != NQ_OK) return cleanup(s);
    b->hs.push_back(h);
  }
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) return cleanup(NQ_ERR_CUDA);
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) return cleanup(NQ_ERR_CUDA);
  b->join.assign(n, nullptr);
  for (int p = 0; p < n; ++p)
    if (cudaEventCreateWithFlags(&b->join[p], cudaEventDisableTiming) != cudaSuccess) return cleanup(NQ_ERR_CUDA);
  const bool ok = cudaMallocHost((void**)&b->h_call, sizeof(uint32_t)) == cudaSuccess &&
                  cudaMallocHost((void**)&b->h_gather, (size_t)n * 8 * sizeof(double)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_call, sizeof(uint32_t)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_sjobs, n * sizeof(SamplerJob<float>)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_ejobs, n * sizeof(EvalJob<float>)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_wjobs, n * sizeof(SweepJob)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_sblk, (n + 1) * sizeof(int)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_eblk, (n + 1) * sizeof(int)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_wcta, (n + 1) * sizeof(int)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_rcta, (n + 1) * sizeof(int)) == cudaSuccess &&
                  cudaMalloc(&b->d_ctl, (size_t)n * 64) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_acc, n * sizeof(unsigned long long)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_stat_src, n * sizeof(double*)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_status_src, n * sizeof(int*)) == cudaSuccess &&
                  cudaMalloc((void**)&b->d_gather, (size_t)n * 8 * sizeof(double)) == cudaSuccess;
  if (!ok) return cleanup(NQ_ERR_CUDA);
  if (nq_status s = batch_setup_grouped(b)) return cleanup(s);
  *out = b;
  return NQ_OK;
}

void nq_batch_destroy(nq_batch* b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (nq_handle* h : b->hs) nq_destroy(h);
  void* bufs[] = {b->d_call, b->d_sjobs, b->d_ejobs, b->d_wjobs, b->d_sblk, b->d_eblk, b->d_wcta, b->d_rcta, b->d_ctl,
                  b->d_acc, b->d_stat_src, b->d_status_src, b->d_gather, b->d_Xall, b->d_Xlo_all, b->d_slots,
                  b->d_geom, b->d_jobs, b->d_prefix};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (b->h_call) cudaFreeHost(b->h_call);
  if (b->h_gather) cudaFreeHost(b->h_gather);
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

nq_status nq_batch_last_error(const nq_batch* b, char* buf, size_t len) {
  if (!b || !buf || len == 0) return NQ_ERR_ARG;
  snprintf(buf, len, "%s", b->err.c_str());
  return NQ_OK;
}

int32_t nq_batch_size(const nq_batch* b) { return b ? (int32_t)b->hs.size() : -1; }

nq_handle* nq_batch_handle(nq_batch* b, int32_t i) {
  if (!b || i < 0 || i >= (int32_t)b->hs.size()) return nullptr;
  return b->hs[i];
}

nq_status nq_batch_vmc_step(nq_batch* b, uint64_t call_index, double eps, double lr, nq_measurement* stats) {
  if (!b) return NQ_ERR_ARG;
  const int np = (int)b->hs.size();
  for (int p = 0; p < np; ++p)
    if (!b->hs[p]->has_op) return bfail(b, NQ_ERR_STATE, "problem %d has no operator (nq_set_operator)", p);
  if (b->graph && (b->geps != eps || b->glr != lr)) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  for (nq_handle* h : b->hs) BCK(cudaStreamSynchronize(h->st));
  BCK(cudaStreamSynchronize(b->st));
  if (nq_status s = batch_tune(b)) return s;
  *b->h_call = (uint32_t)call_index;
  if (!b->graph)
    if (nq_status s = batch_capture(b, eps, lr)) return s;
  BCK(cudaGraphLaunch(b->graph, b->st));
  b->launches += b->graph_kernels;
  BCK(cudaMemcpyAsync(b->h_gather, b->d_gather, (size_t)np * 8 * sizeof(double), cudaMemcpyDeviceToHost, b->st));
  BCK(cudaStreamSynchronize(b->st));
  nq_status worst = NQ_OK;
  for (int p = 0; p < np; ++p) {
    nq_handle* h = b->hs[p];
    const double* v = b->h_gather + 8 * p;
    const int st = (int)v[7];
    if (st != 0) {
      BCK(cudaMemsetAsync(h->sb.status, 0, sizeof(int), b->st));
      worst = (st & 0x10) ? NQ_ERR_TIMEOUT : NQ_ERR_NOT_PD;
      bfail(b, worst, "problem %d: status 0x%x after the step", p, st);
    }
    if (stats) {
      nq_measurement& m = stats[p];
      m.mean_re = v[0];
      m.mean_im = v[1];
      m.error = v[2];
      m.variance = v[3];
      m.tau = v[4];
      m.R = v[5];
      const double steps = (double)h->B * h->passes * (h->cfg.burn + h->n_record);
      m.acceptance = steps > 0 ? v[6] / steps : 0.0;
    }
  }
  if (worst != NQ_OK) BCK(cudaStreamSynchronize(b->st));
  return worst;
}

nq_status nq_batch_bench_steps(nq_batch* b, uint64_t call0, int32_t n_steps, double eps, double lr,
                               float* ms_out) {
  if (!b || !ms_out || n_steps < 1) return NQ_ERR_ARG;
  if (nq_status s = nq_batch_vmc_step(b, call0, eps, lr, nullptr)) return s;
  std::vector<cudaEvent_t> ev(2 * n_steps);
  for (auto& e : ev) BCK(cudaEventCreate(&e));
  for (int i = 0; i < n_steps; ++i) {
    BCK(cudaStreamSynchronize(b->st));
    *b->h_call = (uint32_t)(call0 + 1 + i);
    BCK(cudaEventRecord(ev[2 * i], b->st));
    BCK(cudaGraphLaunch(b->graph, b->st));
    b->launches += b->graph_kernels;
    BCK(cudaEventRecord(ev[2 * i + 1], b->st));
  }
  BCK(cudaStreamSynchronize(b->st));
  for (int i = 0; i < n_steps; ++i) ms_out[i] = elapsed_ms(ev[2 * i], ev[2 * i + 1]);
  for (auto& e : ev) cudaEventDestroy(e);
  return NQ_OK;
}

nq_status nq_batch_tuning(nq_batch* b, int32_t* out, int32_t n) {
  if (!b || !out || n < 1) return NQ_ERR_ARG;
  if (nq_status s = batch_tune(b)) return s;
  const int32_t v[4] = {b->lanes, b->eval_T, b->w_ctas, (int32_t)b->graph_kernels};
  for (int i = 0; i < n && i < 4; ++i) out[i] = v[i];
  return NQ_OK;
}

int64_t nq_batch_kernel_launches(const nq_batch* b) { return b ? b->launches : -1; }

}  // extern "C"
