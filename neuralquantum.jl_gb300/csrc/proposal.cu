// C-ABI of the learned autoregressive proposal: parameter storage, the
// mixture-sampler stage hook and training on the samples of the last call.
#include <cmath>

#include <cuda_bf16.h>

#include "handle.cuh"

struct MadeState {
  int N = 0, H = 128, P = 0;
  double p_ar = 0.0;
  unsigned long long thr = 0;
  float* master = nullptr;        // [P]
  float* m = nullptr;             // Adam moments [P]
  float* v = nullptr;
  float* mask = nullptr;          // [P]
  float* grad = nullptr;          // [P]
  float* partial = nullptr;       // [nblk_cap][P]
  int partial_cap = 0;            // samples covered by `partial`
  __nv_bfloat16* wbf = nullptr;   // W1T | W2T | W3
  float* bias = nullptr;          // b1 | b2 | b3
  unsigned long long* stats = nullptr;   // [2]
  uint64_t* x = nullptr;          // staging for host configurations
  float* lq = nullptr;
  size_t x_cap = 0;
  uint64_t* pre_x = nullptr;      // proposals drawn ahead of the chain kernel [B][pre_slots]
  float* pre_lq = nullptr;
  int pre_slots = 0;
  int adam_step = 0;
};

namespace {

MadeDev made_dev(const MadeState* s) {
  MadeDev d;
  d.N = s->N; d.H = s->H;
  d.W1T = s->wbf;
  d.W2T = s->wbf + (size_t)s->N * s->H;
  d.W3 = s->wbf + (size_t)s->N * s->H + (size_t)s->H * s->H;
  d.b1 = s->bias;
  d.b2 = s->bias + s->H;
  d.b3 = s->bias + 2 * s->H;
  return d;
}

MadeTrain made_train(MadeState* s) {
  MadeTrain t;
  t.N = s->N; t.H = s->H; t.n_params = s->P;
  t.master = s->master; t.m = s->m; t.v = s->v; t.mask = s->mask;
  return t;
}

nq_status need_made(nq_handle* h) {
  if (!h) return NQ_ERR_ARG;
  if (!h->made) return fail(h, NQ_ERR_STATE, "no proposal attached (nq_proposal_init)");
  return NQ_OK;
}

nq_status stage_x(nq_handle* h, const uint64_t* x, int64_t n) {
  MadeState* s = h->made;
  if ((size_t)n > s->x_cap) {
    if (s->x) cudaFree(s->x);
    if (s->lq) cudaFree(s->lq);
    s->x = nullptr; s->lq = nullptr; s->x_cap = 0;
    CK(cudaMalloc((void**)&s->x, (size_t)n * sizeof(uint64_t)));
    CK(cudaMalloc((void**)&s->lq, (size_t)n * sizeof(float)));
    s->x_cap = (size_t)n;
  }
  if (x) CK(cudaMemcpyAsync(s->x, x, (size_t)n * sizeof(uint64_t), cudaMemcpyHostToDevice, h->st));
  return NQ_OK;
}

nq_status ensure_partial(nq_handle* h, int n) {
  MadeState* s = h->made;
  if (n <= s->partial_cap) return NQ_OK;
  if (s->partial) cudaFree(s->partial);
  s->partial = nullptr;
  s->partial_cap = 0;
  const int ch = made_grad_chunk();
  const size_t nblk = (size_t)(n + ch - 1) / ch;
  CK(cudaMalloc((void**)&s->partial, nblk * s->P * sizeof(float)));
  s->partial_cap = n;
  return NQ_OK;
}

nq_status repack(nq_handle* h) {
  MadeState* s = h->made;
  CKL(launch_made_pack(made_dev(s), s->master, h->st));
  return NQ_OK;
}

// mean NLL of n staged configurations (s->x) from the logq kernel
nq_status mean_nll(nq_handle* h, const uint64_t* dx, int64_t n, double* out) {
  MadeState* s = h->made;
  if (nq_status st = stage_x(h, nullptr, n)) return st;
  CKL(launch_made_logq(made_dev(s), dx, (int)n, s->lq, h->st));
  std::vector<float> lq((size_t)n);
  CK(cudaMemcpyAsync(lq.data(), s->lq, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double acc = 0;
  for (float v : lq) acc -= v;
  *out = acc / (double)n;
  return NQ_OK;
}

// splitmix64 -> uniform (0,1] -> Box–Muller normal
struct HostNormal {
  uint64_t st;
  double next_u() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((double)(z >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  }
  double next() {
    const double u1 = next_u(), u2 = next_u();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

}  // namespace

void proposal_destroy(nq_handle* h) {
  if (!h || !h->made) return;
  MadeState* s = h->made;
  void* bufs[] = {s->master, s->m, s->v, s->mask, s->grad, s->partial, s->wbf, s->bias, s->stats, s->x, s->lq,
                  s->pre_x, s->pre_lq};
  for (void* p : bufs)
    if (p) cudaFree(p);
  delete s;
  h->made = nullptr;
}

nq_status proposal_sample_stage(nq_handle* h, const SamplerRun& run, bool* used) {
  *used = false;
  MadeState* s = h->made;
  if (!s || s->p_ar <= 0.0) return NQ_OK;
  CK(cudaMemsetAsync(s->stats, 0, 2 * sizeof(unsigned long long), h->st));
  // AR moves of one chain in this call: Binomial(T, p_ar); draw the slots up to
  // its mean + 6 standard deviations ahead (the rare rest is drawn inline)
  const double T = (double)run.passes * (run.burn + run.n_record);
  const int slots = (int)std::min(T, std::ceil(T * s->p_ar + 6.0 * std::sqrt(T * s->p_ar * (1.0 - s->p_ar))) + 8.0);
  if (slots > s->pre_slots) {
    if (s->pre_x) cudaFree(s->pre_x);
    if (s->pre_lq) cudaFree(s->pre_lq);
    s->pre_x = nullptr; s->pre_lq = nullptr; s->pre_slots = 0;
    CK(cudaMalloc((void**)&s->pre_x, (size_t)h->B * slots * sizeof(uint64_t)));
    CK(cudaMalloc((void**)&s->pre_lq, (size_t)h->B * slots * sizeof(float)));
    s->pre_slots = slots;
  }
  CKL(launch_made_sample(made_dev(s), h->B, slots, run.call, run.k0, run.k1, s->pre_x, s->pre_lq, h->st,
                         run.call_ptr));
  MixParams mp;
  mp.made = made_dev(s);
  mp.thr = s->thr;
  mp.ar_stats = s->stats;
  mp.pre_x = s->pre_x;
  mp.pre_lq = s->pre_lq;
  mp.pre_slots = slots;
  CKL(launch_rbm_mix_sampler(rbm_dev<float>(h), run, mp, h->st));
  *used = true;
  return NQ_OK;
}

extern "C" {

nq_status nq_proposal_init(nq_handle* h, int32_t hidden, double p_ar, uint64_t seed) {
  if (!h) return NQ_ERR_ARG;
  if (h->ndm || h->f64 || h->chain) return fail(h, NQ_ERR_UNSUPPORTED, "learned proposal: FP32 RBM handles only");
  if (h->exact) return fail(h, NQ_ERR_UNSUPPORTED, "learned proposal: the handle samples exactly (no chains)");
  if (h->rule != NQ_RULE_LOCAL) return fail(h, NQ_ERR_UNSUPPORTED, "learned proposal: mixes with LocalRule moves only");
  if (hidden != 128) return fail(h, NQ_ERR_UNSUPPORTED, "learned proposal: hidden must be 128 (got %d)", hidden);
  if (!(p_ar >= 0.0 && p_ar <= 1.0)) return fail(h, NQ_ERR_ARG, "p_ar must lie in [0, 1]");
  if (!mix_sampler_supported(h->N, h->M, 0, hidden))
    return fail(h, NQ_ERR_UNSUPPORTED, "learned proposal: N=%d, M=%d outside the mixture sampler's range",
                h->N, h->M);
  proposal_destroy(h);
  MadeState* s = new MadeState;
  h->made = s;
  s->N = h->N;
  s->H = hidden;
  s->P = made_n_params(s->N, s->H);
  const size_t P = (size_t)s->P;
  CK(cudaMalloc((void**)&s->master, P * sizeof(float)));
  CK(cudaMalloc((void**)&s->m, P * sizeof(float)));
  CK(cudaMalloc((void**)&s->v, P * sizeof(float)));
  CK(cudaMalloc((void**)&s->mask, P * sizeof(float)));
  CK(cudaMalloc((void**)&s->grad, P * sizeof(float)));
  const size_t nw = (size_t)s->N * s->H * 2 + (size_t)s->H * s->H;
  CK(cudaMalloc((void**)&s->wbf, nw * sizeof(__nv_bfloat16)));
  CK(cudaMalloc((void**)&s->bias, (size_t)(2 * s->H + s->N) * sizeof(float)));
  CK(cudaMalloc((void**)&s->stats, 2 * sizeof(unsigned long long)));
  CK(cudaMemsetAsync(s->m, 0, P * sizeof(float), h->st));
  CK(cudaMemsetAsync(s->v, 0, P * sizeof(float), h->st));
  CK(cudaMemsetAsync(s->stats, 0, 2 * sizeof(unsigned long long), h->st));
  CKL(launch_made_mask(s->N, s->H, s->mask, h->st));
  // N(0, 1/fan_in) weights, zero biases
  std::vector<float> p0(P, 0.f);
  HostNormal rng{seed};
  const int N = s->N, H = s->H;
  size_t o = 0;
  for (size_t k = 0; k < (size_t)H * N; ++k) p0[o++] = (float)(rng.next() / std::sqrt((double)N));
  o += H;
  for (size_t k = 0; k < (size_t)H * H; ++k) p0[o++] = (float)(rng.next() / std::sqrt((double)H));
  o += H;
  for (size_t k = 0; k < (size_t)N * H; ++k) p0[o++] = (float)(rng.next() / std::sqrt((double)H));
  CK(cudaMemcpyAsync(s->master, p0.data(), P * sizeof(float), cudaMemcpyHostToDevice, h->st));
  CKL(launch_made_apply_mask(s->P, s->mask, s->master, h->st));
  if (nq_status st = repack(h)) return st;
  CK(cudaStreamSynchronize(h->st));
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  return nq_proposal_set_mix(h, p_ar);
}

nq_status nq_proposal_set_mix(nq_handle* h, double p_ar) {
  if (nq_status st = need_made(h)) return st;
  if (!(p_ar >= 0.0 && p_ar <= 1.0)) return fail(h, NQ_ERR_ARG, "p_ar must lie in [0, 1]");
  MadeState* s = h->made;
  s->p_ar = p_ar;
  // AR move iff word < p_ar 2^32  <=>  word < ceil(p_ar 2^32)
  s->thr = (unsigned long long)std::ceil(p_ar * 4294967296.0);
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  return NQ_OK;
}

int64_t nq_proposal_n_params(const nq_handle* h) { return (h && h->made) ? h->made->P : -1; }

nq_status nq_proposal_set_params(nq_handle* h, const float* p, int64_t n) {
  if (nq_status st = need_made(h)) return st;
  MadeState* s = h->made;
  if (!p || n != s->P) return fail(h, NQ_ERR_ARG, "expected %d proposal parameters, got %lld", s->P, (long long)n);
  CK(cudaMemcpyAsync(s->master, p, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, h->st));
  CKL(launch_made_apply_mask(s->P, s->mask, s->master, h->st));
  CK(cudaMemsetAsync(s->m, 0, (size_t)n * sizeof(float), h->st));
  CK(cudaMemsetAsync(s->v, 0, (size_t)n * sizeof(float), h->st));
  s->adam_step = 0;
  if (nq_status st = repack(h)) return st;
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

nq_status nq_proposal_get_params(nq_handle* h, float* p, int64_t n) {
  if (nq_status st = need_made(h)) return st;
  MadeState* s = h->made;
  if (!p || n != s->P) return fail(h, NQ_ERR_ARG, "expected %d proposal parameters, got %lld", s->P, (long long)n);
  CK(cudaMemcpyAsync(p, s->master, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

nq_status nq_proposal_logq(nq_handle* h, const uint64_t* x, int64_t n, float* out) {
  if (nq_status st = need_made(h)) return st;
  if (!x || !out || n <= 0 || n > (1 << 30)) return fail(h, NQ_ERR_ARG, "bad configuration batch");
  MadeState* s = h->made;
  if (nq_status st = stage_x(h, x, n)) return st;
  CKL(launch_made_logq(made_dev(s), s->x, (int)n, s->lq, h->st));
  CK(cudaMemcpyAsync(out, s->lq, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

nq_status nq_proposal_sample(nq_handle* h, uint64_t call_index, int32_t slots, uint64_t* x_out, float* lq_out) {
  if (nq_status st = need_made(h)) return st;
  if (!x_out || !lq_out || slots <= 0) return fail(h, NQ_ERR_ARG, "bad proposal request");
  MadeState* s = h->made;
  const int64_t n = (int64_t)h->B * slots;
  if (n > (1 << 30)) return fail(h, NQ_ERR_ARG, "too many proposals");
  if (nq_status st = stage_x(h, nullptr, n)) return st;
  CKL(launch_made_sample(made_dev(s), h->B, slots, (uint32_t)call_index, (uint32_t)(h->cfg.seed & 0xffffffffu),
                         (uint32_t)(h->cfg.seed >> 32), s->x, s->lq, h->st));
  CK(cudaMemcpyAsync(x_out, s->x, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(lq_out, s->lq, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

nq_status nq_proposal_grad(nq_handle* h, const uint64_t* x, int64_t n, float* grad_out, double* nll_out) {
  if (nq_status st = need_made(h)) return st;
  if (!x || n <= 0 || n > (1 << 24)) return fail(h, NQ_ERR_ARG, "bad configuration batch");
  MadeState* s = h->made;
  if (nq_status st = stage_x(h, x, n)) return st;
  if (nq_status st = ensure_partial(h, (int)n)) return st;
  CKL(launch_made_grad(made_train(s), s->x, (int)n, s->partial, s->grad, h->st));
  ++h->launches;
  if (grad_out) CK(cudaMemcpyAsync(grad_out, s->grad, (size_t)s->P * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (nll_out) {
    // the FP32 master defines the gradient; the NLL comes from the BF16 copy
    if (nq_status st = mean_nll(h, s->x, n, nll_out)) return st;
  }
  return NQ_OK;
}

nq_status nq_proposal_train(nq_handle* h, int32_t steps, int32_t batch, double lr, double* nll_out) {
  if (nq_status st = need_made(h)) return st;
  if (steps < 0 || batch <= 0 || !(lr >= 0.0)) return fail(h, NQ_ERR_ARG, "bad training request");
  MadeState* s = h->made;
  const int Ns = h->Ns;
  const int nb = std::min(batch, Ns);
  if (nq_status st = ensure_partial(h, nb)) return st;
  const MadeTrain t = made_train(s);
  int off = 0;
  for (int k = 0; k < steps; ++k) {
    if (off + nb > Ns) off = 0;
    CKL(launch_made_grad(t, h->d_samples + off, nb, s->partial, s->grad, h->st));
    ++h->launches;
    CKL(launch_made_adam(t, s->grad, (float)lr, ++s->adam_step, h->st));
    off += nb;
  }
  if (nq_status st = repack(h)) return st;
  if (nll_out) {
    if (nq_status st = mean_nll(h, h->d_samples, Ns, nll_out)) return st;
  }
  CK(cudaStreamSynchronize(h->st));
  return NQ_OK;
}

nq_status nq_proposal_stats(nq_handle* h, uint64_t* out2) {
  if (nq_status st = need_made(h)) return st;
  if (!out2) return NQ_ERR_ARG;
  unsigned long long v[2];
  CK(cudaMemcpyAsync(v, h->made->stats, sizeof(v), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  out2[0] = v[0];
  out2[1] = v[1];
  return NQ_OK;
}

}  // extern "C"
