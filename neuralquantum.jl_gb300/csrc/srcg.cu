// Matrix-free iterative SR solve (sr_cg; the reference's sr_minres / sr_qlp /
// sr_lsq solve the same system), SRIterative.jl:66-140 with the lazy operator
// SrMatrixC of SR_notfull.jl:59-79:
//   (S + shift) v = conj(O_c) O_cᵀ v / Ns + shift v,   S never formed.
// With O_s = [σ(s), g(s), g(s) σ(s)ᵀ] of the RBM (P = N + M + MN):
//   forward  t_s = Σ_q O_q(s) v_q − ⟨O⟩·v
//                = σ·v_a + Σ_h g_h (v_b,h + Σ_j v_W,hj σ_j) − ⟨O⟩·v
//   adjoint  y_p = (Σ_s conj(O_p(s)) t_s − conj⟨O_p⟩ Σ_s t_s) / Ns
// Conjugate gradients in FP64 vectors in ONE persistent cooperative launch:
// per iteration a forward pass (thread per sample, v in shared memory), an
// adjoint pass (CTA b accumulates its chunk of samples for every parameter in
// registers, FP32 inside 32-sample tiles, FP64 across), a fixed-order
// reduction of the CTA partials and the CG recurrences, separated by bounded
// grid barriers.  Every dot product is reduced in a fixed order, so the result
// does not depend on timing.  Memory: O(P · CTAs + Ns), no P x P matrix.
#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int THREADS = 256;
constexpr int EMAX = 24;          // parameters per thread in the adjoint: P <= 6144
constexpr int TS = 32;            // samples per shared-memory tile of the adjoint

struct CgCtl {
  unsigned count, gen;
  int abort, pad;
};

__device__ bool cg_barrier(CgCtl* ctl, int* err, uint64_t limit_ns) {
  return ticket_grid_barrier(&ctl->count, &ctl->gen, &ctl->abort, gridDim.x, err, limit_ns);
}

// fixed-order block sum of two doubles; result valid in every thread
__device__ void block_sum2d(double& a, double& b) {
  __shared__ double sh[2][THREADS / 32];
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, off);
    b += __shfl_xor_sync(0xffffffffu, b, off);
  }
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { sh[0][w] = a; sh[1][w] = b; }
  __syncthreads();
  a = 0.0; b = 0.0;
  for (int k = 0; k < THREADS / 32; ++k) { a += sh[0][k]; b += sh[1][k]; }
}

NQ_D double2 ldcg2(const double* p) { return make_double2(__ldcg(p), __ldcg(p + 1)); }

__global__ void __launch_bounds__(THREADS, 1) sr_cg_kernel(SrCgArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CgCtl* ctl = reinterpret_cast<CgCtl*>(a.ctl);
  const int N = a.N, M = a.M, P = a.P, Ns = a.Ns, hilb = a.hilb;
  float2* s_v = reinterpret_cast<float2*>(smem_raw);                 // [P] direction, FP32
  float2* s_g = s_v + P;                                              // [M][TS] g tile
  float2* s_t = s_g + (size_t)M * TS;                                 // [TS]
  uint64_t* s_bits = reinterpret_cast<uint64_t*>(s_t + TS);          // [TS]
  __shared__ double s_c[2];
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  // parameter slice of this CTA for the vector updates
  const int per = (P + G - 1) / G, p0 = min(P, b * per), p1 = min(P, p0 + per);
  // sample chunk of this CTA for the adjoint
  const int chunk = (Ns + G - 1) / G, s0 = min(Ns, b * chunk), s1 = min(Ns, s0 + chunk);
  const double inv_ns = 1.0 / Ns;

  // shift_p (multiplicative: lam * S_pp, with S_pp from a pass over the samples)
  // x = 0, r = F, p = F
  for (int p = p0 + tid; p < p1; p += THREADS) {
    const double fx = a.F[2 * p], fy = a.real_params ? 0.0 : a.F[2 * p + 1];
    a.x[2 * p] = 0.0; a.x[2 * p + 1] = 0.0;
    a.r[2 * p] = fx; a.r[2 * p + 1] = fy;
    a.pv[2 * p] = fx; a.pv[2 * p + 1] = fy;
  }
  {
    double rr = 0.0, ff = 0.0;
    for (int p = p0 + tid; p < p1; p += THREADS) {
      const double fx = a.F[2 * p], fy = a.real_params ? 0.0 : a.F[2 * p + 1];
      rr += fx * fx + fy * fy;
    }
    block_sum2d(rr, ff);
    if (tid == 0) { a.dots[4 * b] = rr; a.dots[4 * b + 1] = 0.0; }
  }
  if (!cg_barrier(ctl, a.status, a.wait_ns)) return;
  double rr = 0.0;
  for (int k = 0; k < G; ++k) rr += __ldcg(a.dots + 4 * k);
  const double rr0 = rr;
  const double stop = a.tol * a.tol * rr0;
  int it = 0;
  bool done = !(rr0 > 0.0);
  while (!done && it < a.maxiter) {
    // ---- forward: t_s = O_c(s)·p ----
    for (int p = tid; p < P; p += THREADS) {
      const double2 v = ldcg2(a.pv + 2 * p);
      s_v[p] = make_float2((float)v.x, (float)v.y);
    }
    {
      double cx = 0.0, cy = 0.0;      // ⟨O⟩·p, same fixed order in every CTA
      for (int p = tid; p < P; p += THREADS) {
        const double ox = a.meanO[2 * p], oy = a.meanO[2 * p + 1];
        const double2 v = ldcg2(a.pv + 2 * p);
        cx += ox * v.x - oy * v.y;
        cy += ox * v.y + oy * v.x;
      }
      block_sum2d(cx, cy);
      if (tid == 0) { s_c[0] = cx; s_c[1] = cy; }
    }
    __syncthreads();
    const float cx = (float)s_c[0], cy = (float)s_c[1];
    for (int s = b * THREADS + tid; s < Ns; s += G * THREADS) {
      const uint64_t bits = a.samples[s];
      float tx = -cx, ty = -cy;
      for (int j = 0; j < N; ++j) {
        const float sv = site_valuef(bits, j, hilb);
        tx += s_v[j].x * sv;
        ty += s_v[j].y * sv;
      }
      for (int h = 0; h < M; ++h) {
        float zx = s_v[N + h].x, zy = s_v[N + h].y;
        const float2* vw = s_v + N + M + h;
        for (int j = 0; j < N; ++j) {
          const float sv = site_valuef(bits, j, hilb);
          zx += vw[(size_t)M * j].x * sv;
          zy += vw[(size_t)M * j].y * sv;
        }
        const float2 gh = a.g[(size_t)h * Ns + s];
        tx += gh.x * zx - gh.y * zy;
        ty += gh.x * zy + gh.y * zx;
      }
      a.t[s] = make_float2(tx, ty);
    }
    if (!cg_barrier(ctl, a.status, a.wait_ns)) return;
    // ---- adjoint partials over this CTA's sample chunk ----
    double2 acc[EMAX];
#pragma unroll
    for (int e = 0; e < EMAX; ++e) acc[e] = make_double2(0.0, 0.0);
    float tsx = 0.f, tsy = 0.f;
    for (int c0 = s0; c0 < s1; c0 += TS) {
      const int nt = min(TS, s1 - c0);
      __syncthreads();
      for (int e = tid; e < M * TS; e += THREADS) {
        const int h = e / TS, q = e % TS;
        s_g[e] = q < nt ? a.g[(size_t)h * Ns + c0 + q] : make_float2(0.f, 0.f);
      }
      for (int q = tid; q < TS; q += THREADS) {
        s_t[q] = q < nt ? __ldcg(reinterpret_cast<const float2*>(a.t) + c0 + q) : make_float2(0.f, 0.f);
        s_bits[q] = q < nt ? a.samples[c0 + q] : 0ull;
      }
      __syncthreads();
      if (tid == 0)
        for (int q = 0; q < nt; ++q) { tsx += s_t[q].x; tsy += s_t[q].y; }
#pragma unroll
      for (int e = 0; e < EMAX; ++e) {
        const int p = tid + e * THREADS;
        if (p < P) {
          float ax = 0.f, ay = 0.f;
          if (p < N) {
            for (int q = 0; q < nt; ++q) {
              const float sv = site_valuef(s_bits[q], p, hilb);
              ax += sv * s_t[q].x;
              ay += sv * s_t[q].y;
            }
          } else if (p < N + M) {
            const float2* gr = s_g + (size_t)(p - N) * TS;
            for (int q = 0; q < nt; ++q) {      // conj(g) t
              ax += gr[q].x * s_t[q].x + gr[q].y * s_t[q].y;
              ay += gr[q].x * s_t[q].y - gr[q].y * s_t[q].x;
            }
          } else {
            const int k = p - N - M, h = k % M, j = k / M;
            const float2* gr = s_g + (size_t)h * TS;
            for (int q = 0; q < nt; ++q) {
              const float sv = site_valuef(s_bits[q], j, hilb);
              ax += sv * (gr[q].x * s_t[q].x + gr[q].y * s_t[q].y);
              ay += sv * (gr[q].x * s_t[q].y - gr[q].y * s_t[q].x);
            }
          }
          acc[e].x += ax;
          acc[e].y += ay;
        }
      }
    }
#pragma unroll
    for (int e = 0; e < EMAX; ++e) {
      const int p = tid + e * THREADS;
      if (p < P) {
        a.part[((size_t)b * P + p) * 2] = acc[e].x;
        a.part[((size_t)b * P + p) * 2 + 1] = acc[e].y;
      }
    }
    if (tid == 0) { a.tsum[2 * b] = tsx; a.tsum[2 * b + 1] = tsy; }
    if (!cg_barrier(ctl, a.status, a.wait_ns)) return;
    // ---- w = S p + shift p on this CTA's slice; p·w partial ----
    double tx = 0.0, ty = 0.0;
    for (int k = 0; k < G; ++k) { tx += __ldcg(a.tsum + 2 * k); ty += __ldcg(a.tsum + 2 * k + 1); }
    double pw = 0.0, dummy = 0.0;
    for (int p = p0 + tid; p < p1; p += THREADS) {
      double yx = 0.0, yy = 0.0;
      for (int k = 0; k < G; ++k) {
        yx += __ldcg(a.part + ((size_t)k * P + p) * 2);
        yy += __ldcg(a.part + ((size_t)k * P + p) * 2 + 1);
      }
      const double ox = a.meanO[2 * p], oy = a.meanO[2 * p + 1];
      yx -= ox * tx + oy * ty;                  // conj(⟨O⟩) Σ t
      yy -= ox * ty - oy * tx;
      yx *= inv_ns;
      yy *= inv_ns;
      const double2 v = ldcg2(a.pv + 2 * p);
      const double sh = a.shift[p];
      yx += sh * v.x;
      yy += sh * v.y;
      if (a.real_params) yy = 0.0;
      a.w[2 * p] = yx;
      a.w[2 * p + 1] = yy;
      pw += v.x * yx + v.y * yy;                // Re(p† w); S + shift is Hermitian, so p†w is real
    }
    block_sum2d(pw, dummy);
    if (tid == 0) a.dots[4 * b + 1] = pw;
    if (!cg_barrier(ctl, a.status, a.wait_ns)) return;
    double pwt = 0.0;
    for (int k = 0; k < G; ++k) pwt += __ldcg(a.dots + 4 * k + 1);
    if (!(pwt > 0.0)) {
      if (b == 0 && tid == 0) atomicOr(a.status, 1);    // not positive definite
      break;
    }
    const double alpha = rr / pwt;
    double rr_new = 0.0;
    for (int p = p0 + tid; p < p1; p += THREADS) {
      const double2 v = ldcg2(a.pv + 2 * p);
      const double2 w = make_double2(__ldcg(a.w + 2 * p), __ldcg(a.w + 2 * p + 1));
      a.x[2 * p] += alpha * v.x;
      a.x[2 * p + 1] += alpha * v.y;
      const double rx = a.r[2 * p] - alpha * w.x, ry = a.r[2 * p + 1] - alpha * w.y;
      a.r[2 * p] = rx;
      a.r[2 * p + 1] = ry;
      rr_new += rx * rx + ry * ry;
    }
    block_sum2d(rr_new, dummy);
    if (tid == 0) a.dots[4 * b + 2] = rr_new;
    if (!cg_barrier(ctl, a.status, a.wait_ns)) return;
    double rrn = 0.0;
    for (int k = 0; k < G; ++k) rrn += __ldcg(a.dots + 4 * k + 2);
    const double beta = rrn / rr;
    rr = rrn;
    ++it;
    done = rr <= stop;
    for (int p = p0 + tid; p < p1; p += THREADS) {
      a.pv[2 * p] = a.r[2 * p] + beta * a.pv[2 * p];
      a.pv[2 * p + 1] = a.r[2 * p + 1] + beta * a.pv[2 * p + 1];
    }
    if (!cg_barrier(ctl, a.status, a.wait_ns)) return;
  }
  if (b == 0 && tid == 0) {
    a.info[0] = (double)it;
    a.info[1] = rr0 > 0.0 ? sqrt(rr / rr0) : 0.0;
  }
}

// diag(S) for the multiplicative shift: S_pp = mean |O_p|^2 - |<O_p>|^2
__global__ void sr_diag_kernel(SrCgArgs a, double lam, int kind) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.P) return;
  if (kind == 0) { a.shift[p] = a.eps; return; }
  if (kind == 2) { a.shift[p] = 0.0; return; }
  const int N = a.N, M = a.M, Ns = a.Ns;
  double acc = 0.0;
  if (p < N) {
    for (int s = 0; s < Ns; ++s) {
      const double v = site_valuef(a.samples[s], p, a.hilb);
      acc += v * v;
    }
  } else if (p < N + M) {
    const float2* gr = a.g + (size_t)(p - N) * Ns;
    for (int s = 0; s < Ns; ++s) acc += (double)gr[s].x * gr[s].x + (double)gr[s].y * gr[s].y;
  } else {
    const int k = p - N - M, h = k % M, j = k / M;
    const float2* gr = a.g + (size_t)h * Ns;
    for (int s = 0; s < Ns; ++s) {
      const double v = site_valuef(a.samples[s], j, a.hilb);
      acc += v * v * ((double)gr[s].x * gr[s].x + (double)gr[s].y * gr[s].y);
    }
  }
  const double ox = a.meanO[2 * p], oy = a.meanO[2 * p + 1];
  a.shift[p] = lam * (acc / Ns - (ox * ox + oy * oy));
}

}  // namespace

int sr_cg_grid() {
  static int grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    grid = sms;
  }
  return grid;
}

size_t sr_cg_ctl_bytes() { return sizeof(CgCtl); }
bool sr_cg_supported(int P) { return P <= EMAX * THREADS; }

cudaError_t launch_sr_cg(const SrCgArgs& args, int kind, double lam, cudaStream_t st) {
  if (!sr_cg_supported(args.P)) return cudaErrorInvalidValue;
  sr_diag_kernel<<<(args.P + 255) / 256, 256, 0, st>>>(args, lam, kind);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(args.ctl, 0, sizeof(CgCtl), st);
  if (e != cudaSuccess) return e;
  const size_t smem = (size_t)args.P * sizeof(float2) + (size_t)args.M * TS * sizeof(float2) + TS * sizeof(float2) +
                      TS * sizeof(uint64_t);
  e = cudaFuncSetAttribute(sr_cg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(sr_cg_grid());
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, sr_cg_kernel, args);
}
