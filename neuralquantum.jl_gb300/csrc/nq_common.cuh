// Common device utilities for libnqcuda: complex arithmetic, the Philox
// counter-based generator, site encodings and the two activations of the
// reference (src/Networks/activation.jl:5-45).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define NQ_HD __host__ __device__ __forceinline__
#define NQ_D __device__ __forceinline__

// Bits of a handle's device status word beyond the solve's non-positive pivot
// (bit 0): a bounded wait gave up (host: NQ_ERR_TIMEOUT); the solve produced
// a non-finite update (host: NQ_ERR_NAN).
#define NQ_DEVERR_TIMEOUT 0x10
#define NQ_DEVERR_NONFINITE 0x20
// Default limit of a bounded device-side wait.
constexpr uint64_t kNqWaitNs = 1000000000ull;

// ---------------------------------------------------------------------------
// complex numbers as (re, im) pairs, templated on the real type
// ---------------------------------------------------------------------------
template <typename R> struct cpx { R x, y; };

template <typename R> NQ_HD cpx<R> mk(R x, R y) { cpx<R> c; c.x = x; c.y = y; return c; }
template <typename R> NQ_HD cpx<R> operator+(cpx<R> a, cpx<R> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename R> NQ_HD cpx<R> operator-(cpx<R> a, cpx<R> b) { return mk(a.x - b.x, a.y - b.y); }
template <typename R> NQ_HD cpx<R> operator*(cpx<R> a, cpx<R> b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R> NQ_HD cpx<R> operator*(R s, cpx<R> a) { return mk(s * a.x, s * a.y); }
template <typename R> NQ_HD cpx<R> conjc(cpx<R> a) { return mk(a.x, -a.y); }
template <typename R> NQ_HD R abs2c(cpx<R> a) { return a.x * a.x + a.y * a.y; }
template <typename R> NQ_HD cpx<R> divc(cpx<R> a, cpx<R> b) {
  R d = R(1) / (b.x * b.x + b.y * b.y);
  return mk((a.x * b.x + a.y * b.y) * d, (a.y * b.x - a.x * b.y) * d);
}
// a + b*c
template <typename R> NQ_HD cpx<R> cfma(cpx<R> b, cpx<R> c, cpx<R> a) {
  return mk(a.x + b.x * c.x - b.y * c.y, a.y + b.x * c.y + b.y * c.x);
}

// real-type dispatched math
NQ_D float r_exp(float x) { return expf(x); }
NQ_D double r_exp(double x) { return exp(x); }
NQ_D float r_log(float x) { return logf(x); }
NQ_D double r_log(double x) { return log(x); }
NQ_D float r_log1p(float x) { return log1pf(x); }
NQ_D double r_log1p(double x) { return log1p(x); }
NQ_D float r_cosh(float x) { return coshf(x); }
NQ_D double r_cosh(double x) { return cosh(x); }
NQ_D float r_sinh(float x) { return sinhf(x); }
NQ_D double r_sinh(double x) { return sinh(x); }
NQ_D float r_tanh(float x) { return tanhf(x); }
NQ_D double r_tanh(double x) { return tanh(x); }
NQ_D float r_atan2(float y, float x) { return atan2f(y, x); }
NQ_D double r_atan2(double y, double x) { return atan2(y, x); }
NQ_D void r_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
NQ_D void r_sincos(double x, double* s, double* c) { sincos(x, s, c); }
NQ_D float r_abs(float x) { return fabsf(x); }
NQ_D double r_abs(double x) { return fabs(x); }

template <typename R> NQ_D cpx<R> cexpc(cpx<R> z) {
  R e = r_exp(z.x), s, c;
  r_sincos(z.y, &s, &c);
  return mk(e * c, e * s);
}
// principal complex logarithm
template <typename R> NQ_D cpx<R> clogc(cpx<R> z) {
  return mk(R(0.5) * r_log(z.x * z.x + z.y * z.y), r_atan2(z.y, z.x));
}
template <typename R> NQ_D cpx<R> ccoshc(cpx<R> z) {
  R s, c;
  r_sincos(z.y, &s, &c);
  return mk(r_cosh(z.x) * c, r_sinh(z.x) * s);
}
template <typename R> NQ_D cpx<R> csinhc(cpx<R> z) {
  R s, c;
  r_sincos(z.y, &s, &c);
  return mk(r_sinh(z.x) * c, r_cosh(z.x) * s);
}

// ---------------------------------------------------------------------------
// Activations.  logcosh = logℒ2 (activation.jl:9-13), derivative tanh;
// softplus = logℒ = log1p(exp(x)) (activation.jl:20), derivative sigmoid.
// ---------------------------------------------------------------------------
enum { ACT_LOGCOSH = 0, ACT_SOFTPLUS = 1, ACT_IDENTITY = 2 };   // identity: Dense layers of a chain only

template <typename R> NQ_D R logcosh_real(R x) {
  R ax = r_abs(x);
  return ax <= R(12) ? r_log(r_cosh(x)) : ax - R(0.6931471805599453);
}

// f(z) for complex z
template <int ACT, typename R> NQ_D cpx<R> act_f(cpx<R> z) {
  if (ACT == ACT_LOGCOSH) {
    // logℒ2(re) + log(cos(im) + i tanh(re) sin(im))
    R s, c;
    r_sincos(z.y, &s, &c);
    cpx<R> w = mk(c, r_tanh(z.x) * s);
    cpx<R> lw = clogc(w);
    return mk(logcosh_real(z.x) + lw.x, lw.y);
  } else {
    // log1p(exp(z)) = log(1 + exp(z)); for large Re z use z + log1p(exp(-z))
    if (z.x > R(15)) {
      cpx<R> e = cexpc(mk(-z.x, -z.y));
      cpx<R> l = clogc(mk(R(1) + e.x, e.y));
      return mk(z.x + l.x, z.y + l.y);
    }
    cpx<R> e = cexpc(z);
    return clogc(mk(R(1) + e.x, e.y));
  }
}

// logcosh(z) and tanh(z) together, from e = exp(-2|x|) and sincos(y), z = x + iy:
//   log cosh z = |x| - log 2 + log1p(e) + log(cos y + i tanh(x) sin y)
//   tanh x     = sgn(x) (1 - e) / (1 + e)
//   tanh z     = (sgn(x) (1 - e)(1 + e) + 4i e sin y cos y) / ((1 - e)^2 + 4 e cos^2 y)
// The last is (sinh 2x + i sin 2y) / (cosh 2x + cos 2y) multiplied by 2e; its
// denominator is a sum of non-negative terms.  The first is the logℒ2 form of
// activation.jl:9-13 with log cosh x written without overflow.
template <typename R> NQ_D void logcosh_tanh(cpx<R> z, cpx<R>* f, cpx<R>* df) {
  const R ax = r_abs(z.x);
  const R e = r_exp(R(-2) * ax);
  R s, c;
  r_sincos(z.y, &s, &c);
  const R sg = z.x < R(0) ? R(-1) : R(1);
  const R ope = R(1) + e, ome = R(1) - e;
  const R thx = sg * ome / ope;
  const cpx<R> lw = clogc(mk(c, thx * s));
  *f = mk(ax - R(0.6931471805599453) + r_log1p(e) + lw.x, lw.y);
  const R inv = R(1) / (ome * ome + R(4) * e * c * c);
  *df = mk(sg * ome * ope * inv, R(4) * e * s * c * inv);
}

// f'(z): tanh or sigmoid of complex z
template <int ACT, typename R> NQ_D cpx<R> act_df(cpx<R> z) {
  if (ACT == ACT_LOGCOSH) {
    // tanh z = (sgn(x) (1 - e)(1 + e) + 4i e sin y cos y) / ((1 - e)^2 + 4 e cos^2 y),
    // e = exp(-2|x|): (sinh 2x + i sin 2y) / (cosh 2x + cos 2y) multiplied by 2e
    const R e = r_exp(R(-2) * r_abs(z.x));
    R s, c;
    r_sincos(z.y, &s, &c);
    const R sg = z.x < R(0) ? R(-1) : R(1);
    const R ope = R(1) + e, ome = R(1) - e;
    const R inv = R(1) / (ome * ome + R(4) * e * c * c);
    return mk(sg * ome * ope * inv, R(4) * e * s * c * inv);
  } else {
    // 1 / (1 + exp(-z))
    if (z.x < R(-30)) return cexpc(z);
    if (z.x > R(30)) return mk(R(1), R(0));
    cpx<R> e = cexpc(mk(-z.x, -z.y));
    return divc(mk(R(1), R(0)), mk(R(1) + e.x, e.y));
  }
}

// real activations (NDM hidden units have real pre-activations)
template <int ACT, typename R> NQ_D R act_f_real(R x) {
  if (ACT == ACT_LOGCOSH) return logcosh_real(x);
  return x > R(15) ? x + r_log1p(r_exp(-x)) : r_log1p(r_exp(x));
}
template <int ACT, typename R> NQ_D R act_df_real(R x) {
  if (ACT == ACT_LOGCOSH) return r_tanh(x);
  return R(1) / (R(1) + r_exp(-x));
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11).  Counter schema shared with the
// oracle: key = (seed lo, seed hi); init words (q/4, call, chain, 0);
// Metropolis step t (t, call, chain, 1); exact-sampler draw t (t, call, chain, 4).
// ---------------------------------------------------------------------------
enum { TAG_INIT = 0, TAG_MH = 1, TAG_AR = 2, TAG_MIX = 3, TAG_EXACT = 4 };

struct u32x4 { uint32_t x, y, z, w; };

NQ_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

NQ_HD u32x4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                          uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  u32x4 r; r.x = c0; r.y = c1; r.z = c2; r.w = c3;
  return r;
}

NQ_HD uint32_t uniform_site(uint32_t w, uint32_t nsites) {
  return (uint32_t)(((uint64_t)w * nsites) >> 32);
}
// u in [0,1) with 24 random bits: exact in float
NQ_HD float uniform24(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }
// u in [0,1) with 53 random bits (27 from a, 26 from b): exact in double
NQ_HD double uniform53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------
// Site encodings.  A configuration of up to 64 two-level sites is a bit mask;
// bit j is the local index of site j (spin: 0 <-> -1, 1 <-> +1; Fock: value).
// ---------------------------------------------------------------------------
enum { HILB_SPIN = 0, HILB_FOCK = 1 };

template <typename R> NQ_HD R site_value(uint64_t bits, int j, int hilb) {
  int b = (int)((bits >> j) & 1ull);
  return hilb == HILB_SPIN ? R(2 * b - 1) : R(b);
}
NQ_HD float site_valuef(uint64_t bits, int j, int hilb) { return site_value<float>(bits, j, hilb); }

#define NQ_CUDA_OK(expr)                                                     \
  do {                                                                       \
    cudaError_t _e = (expr);                                                 \
    if (_e != cudaSuccess) return _e;                                        \
  } while (0)
