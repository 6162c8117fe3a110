/*
 * CPU restatement of the reference VMC iteration for the RBM ket path
 * (test infrastructure and timed CPU baseline; never linked into libnqcuda).
 *
 * It keeps the reference's algorithmic structure so that its timing stands in
 * for the Julia CPU path (no Julia runtime is available to run the reference
 * itself):
 *   - Metropolis (src/Samplers/Metropolis.jl:124-167): every pass re-evaluates
 *     log|ψ|^2 of the proposed batch from scratch, θ = Wσ + b included
 *     (RBMBatched.jl:37-56) -- no θ-cache;
 *   - logψ_and_∇logψ! on all samples (RBMBatched.jl:58-91);
 *   - the accumulator loop (AccumulatorObsScalar.jl:52-137): every connected
 *     configuration σ' with a change is evaluated with the full network.
 * The random stream is the engine's Philox schema (see oracle/philox.py), so
 * at equal parameters both produce the same chains up to floating-point ties.
 * OpenMP across chains / samples.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <tgmath.h>

/* Compiled twice: as is (FP64 complex, entry points port_*) and with
 * -DPORT_F32 (FP32 complex like the reference's default STD_REAL_PREC =
 * Float32, src/NeuralQuantum.jl:57; entry points port_*_f32).  The interface
 * is FP64 in both: parameters complex128, samples float64, outputs
 * complex128. */
#ifdef PORT_F32
typedef float real_t;
typedef float complex cplx;
#define PORT(name) name##_f32
#else
typedef double real_t;
typedef double complex cplx;
#define PORT(name) name
#endif

static uint32_t mulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }

static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = mulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = mulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

/* logℒ2 (activation.jl:9-13) and logℒ (activation.jl:20); tgmath picks the
 * float or double form of every function from its argument */
static real_t logcosh_re(real_t x) {
  real_t ax = fabs(x);
  return ax <= (real_t)12 ? log(cosh(x)) : ax - log((real_t)2);
}
static cplx act(int a, cplx z) {
  if (a == 0) return logcosh_re(creal(z)) + log(cos(cimag(z)) + I * tanh(creal(z)) * sin(cimag(z)));
  return log((real_t)1 + exp(z));
}
static cplx dact(int a, cplx z) {
  if (a == 0) return tanh(z);
  return (real_t)1 / ((real_t)1 + exp(-z));
}

static real_t site_val(int hilb, int bit) { return hilb == 0 ? (bit ? (real_t)1 : (real_t)-1) : (real_t)bit; }

/* parameters in the working precision (a copy of the complex128 input) */
static cplx* load_params(const double* params, int P) {
  cplx* p = (cplx*)malloc(sizeof(cplx) * (size_t)P);
  for (int k = 0; k < P; ++k) p[k] = (real_t)params[2 * k] + I * (real_t)params[2 * k + 1];
  return p;
}

/* logψ of one configuration (values v[N]); theta scratch [M] */
static cplx rbm_logpsi(int N, int M, int a, const cplx* pa, const cplx* pb, const cplx* W,
                       const real_t* v, cplx* theta) {
  cplx out = 0;
  for (int j = 0; j < N; ++j) out += pa[j] * v[j];
  for (int h = 0; h < M; ++h) theta[h] = pb[h];
  for (int j = 0; j < N; ++j) {
    const cplx* w = W + (size_t)M * j;
    real_t vj = v[j];
    for (int h = 0; h < M; ++h) theta[h] += w[h] * vj;
  }
  for (int h = 0; h < M; ++h) out += act(a, theta[h]);
  return out;
}

/*
 * Metropolis sampling of B chains; samples_out[(l*B + c)*N + j] site values.
 * Returns accepted steps.
 */
long PORT(port_sample)(int N, int M, int a, int hilb, const double* params, int B, int L, int burn,
                       int passes, uint64_t seed, uint32_t call, int chain_offset, double* samples_out) {
  cplx* p = load_params(params, N + M + M * N);
  const cplx *pa = p, *pb = p + N, *W = p + N + M;
  const uint32_t k0 = (uint32_t)(seed & 0xffffffffu), k1 = (uint32_t)(seed >> 32);
  long accepted = 0;
#pragma omp parallel for schedule(static) reduction(+ : accepted)
  for (int c = 0; c < B; ++c) {
    real_t v[128], vn[128];
    cplx theta[1024];
    const uint32_t chain = (uint32_t)(c + chain_offset);
    for (int q = 0; q < N; q += 4) {
      uint32_t w[4] = {(uint32_t)(q >> 2), call, chain, 0};
      philox(w, k0, k1);
      for (int k = 0; k < 4 && q + k < N; ++k) v[q + k] = site_val(hilb, (int)(w[k] >> 31));
    }
    real_t lp = 2 * creal(rbm_logpsi(N, M, a, pa, pb, W, v, theta));
    uint32_t t = 0;
    for (int sweep = 0; sweep < burn + L; ++sweep) {
      /* samplenext! recomputes the current log-probability first */
      lp = 2 * creal(rbm_logpsi(N, M, a, pa, pb, W, v, theta));
      for (int pass = 0; pass < passes; ++pass, ++t) {
        uint32_t r[4] = {t, call, chain, 1};
        philox(r, k0, k1);
        int i = (int)(((uint64_t)r[0] * (uint32_t)N) >> 32);
        real_t u = (real_t)(r[1] >> 8) * ((real_t)1 / (real_t)16777216);
        memcpy(vn, v, sizeof(real_t) * N);
        vn[i] = hilb == 0 ? -v[i] : (real_t)1 - v[i];
        real_t lpn = 2 * creal(rbm_logpsi(N, M, a, pa, pb, W, vn, theta));
        if (u < exp(lpn - lp)) {
          memcpy(v, vn, sizeof(real_t) * N);
          lp = lpn;
          ++accepted;
        }
      }
      int slot = sweep - burn;
      if (slot >= 0)
        for (int j = 0; j < N; ++j) samples_out[((size_t)slot * B + c) * N + j] = (double)v[j];
    }
  }
  free(p);
  return accepted;
}

/* logψ and O = ∇logψ (ns x P, row-major per sample), complex128 outputs */
void PORT(port_eval)(int N, int M, int a, const double* params, int ns, const double* samples,
                     double* logpsi_out, double* O_out) {
  const int P = N + M + M * N;
  cplx* p = load_params(params, P);
  const cplx *pa = p, *pb = p + N, *W = p + N + M;
#pragma omp parallel for schedule(static)
  for (int s = 0; s < ns; ++s) {
    cplx theta[1024], O[N + M];
    real_t v[128];
    for (int j = 0; j < N; ++j) v[j] = (real_t)samples[(size_t)s * N + j];
    cplx lp = rbm_logpsi(N, M, a, pa, pb, W, v, theta);
    logpsi_out[2 * s] = (double)creal(lp);
    logpsi_out[2 * s + 1] = (double)cimag(lp);
    double* out = O_out + 2 * (size_t)s * P;
    for (int j = 0; j < N; ++j) O[j] = v[j];
    for (int h = 0; h < M; ++h) O[N + h] = dact(a, theta[h]);
    for (int k = 0; k < N + M; ++k) {
      out[2 * k] = (double)creal(O[k]);
      out[2 * k + 1] = (double)cimag(O[k]);
    }
    for (int j = 0; j < N; ++j)
      for (int h = 0; h < M; ++h) {
        const cplx o = O[N + h] * v[j];
        const size_t k = (size_t)N + M + h + (size_t)M * j;
        out[2 * k] = (double)creal(o);
        out[2 * k + 1] = (double)cimag(o);
      }
  }
  free(p);
}

/*
 * Local energy with the flattened operator table of include/nqcuda.h: every
 * connection with a change evaluates logψ(σ') with the full network.
 */
void PORT(port_eloc)(int N, int M, int a, int hilb, const double* params, int ns, const double* samples,
                     const double* logpsi, int n_ops, const int* op_n_sites, const int* op_sites,
                     const int* op_row_offset, const int* row_conn_offset, const double* conn_mel,
                     const int* conn_n_changes, const int* conn_change_site,
                     const signed char* conn_change_value, double* eloc_out) {
  cplx* p = load_params(params, N + M + M * N);
  const cplx *pa = p, *pb = p + N, *W = p + N + M;
#pragma omp parallel for schedule(static)
  for (int s = 0; s < ns; ++s) {
    cplx theta[1024];
    real_t v[128], vp[128];
    for (int j = 0; j < N; ++j) v[j] = (real_t)samples[(size_t)s * N + j];
    const cplx lps = (real_t)logpsi[2 * s] + I * (real_t)logpsi[2 * s + 1];
    cplx E = 0;
    for (int o = 0; o < n_ops; ++o) {
      int r = 0;
      for (int d = 0; d < op_n_sites[o]; ++d) {
        real_t x = v[op_sites[8 * o + d]];
        int bit = hilb == 0 ? (x > 0) : (x != 0);
        r |= bit << d;
      }
      int row = op_row_offset[o] + r;
      for (int c = row_conn_offset[row]; c < row_conn_offset[row + 1]; ++c) {
        cplx mel = (real_t)conn_mel[2 * c] + I * (real_t)conn_mel[2 * c + 1];
        if (mel == 0) continue;
        int nch = conn_n_changes[c];
        if (nch == 0) { E += mel; continue; }
        memcpy(vp, v, sizeof(real_t) * N);
        for (int q = 0; q < nch; ++q) vp[conn_change_site[8 * c + q]] = (real_t)conn_change_value[8 * c + q];
        cplx lpp = rbm_logpsi(N, M, a, pa, pb, W, vp, theta);
        E += mel * exp(lpp - lps);
      }
    }
    eloc_out[2 * s] = (double)creal(E);
    eloc_out[2 * s + 1] = (double)cimag(E);
  }
  free(p);
}
