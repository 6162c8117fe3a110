// Matrix-free iterative SR solve (sr_cg; the reference's sr_minres / sr_qlp /
// sr_lsq solve the same system), SRIterative.jl:66-140 with the lazy operator
// SrMatrixC of SR_notfull.jl:59-79:
//   (S + shift) v = conj(O_c) O_cᵀ v / Ns + shift v,   S never formed.
// With O_s = [σ(s), g(s), g(s) σ(s)ᵀ] of the RBM (P = N + M + MN):
//   forward  t_s = Σ_q O_q(s) v_q − ⟨O⟩·v
//                = σ·v_a + Σ_h g_h (v_b,h + Σ_j v_W,hj σ_j) − ⟨O⟩·v
//   adjoint  y_p = (Σ_s conj(O_p(s)) t_s − conj⟨O_p⟩ Σ_s t_s) / Ns
// Conjugate gradients in FP64 vectors in ONE persistent cooperative launch:
// per iteration a forward pass (thread per sample, v in shared memory, the
// hidden units in register chunks), an adjoint pass (CTA b works through its
// chunk of samples in tiles of 32: σ and z = conj(g) t staged in shared
// memory, the W block as a register-tiled contraction; FP32 sums per tile and
// per CTA, FP64 across CTAs), a fixed-order reduction of the CTA partials and
// the CG recurrences, separated by bounded grid barriers.  Every dot product is reduced in a fixed order, so the result
// does not depend on timing.  Memory: O(P · CTAs + Ns), no P x P matrix.
//
// The other networks (NDM family, feed-forward and density-matrix chains)
// have O materialised as the centred rows of X (FP32, the SrMatrix's Ô):
// the forward pass is a thread per sample over the P complex rows, the
// adjoint a warp per parameter row over the CTA's sample chunk (fixed-order
// shuffle sums), and everything after the partials is shared.
#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int THREADS = 256;
constexpr int TS = 32;            // samples per shared-memory tile of the adjoint
constexpr int TSP = TS + 1;       // row stride of the z tile (odd: fewer bank conflicts)
constexpr int FH = 8;             // forward: hidden units per register chunk
constexpr int AH = 4, AJ = 8;     // adjoint: register tile of hidden units x sites

NQ_D int pad8(int n) { return (n + 7) & ~7; }
// dynamic shared memory of the CG kernel (bytes)
NQ_HD size_t cg_smem_bytes(int N, int M) {
  const size_t P = (size_t)N + M + (size_t)N * M;
  return 2 * P * sizeof(float2) + (size_t)M * TSP * sizeof(float2) + (size_t)TS * (((N + 7) & ~7)) * sizeof(float) +
         TS * sizeof(float2) + TS * sizeof(uint64_t) + 16;
}

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

// dynamic shared memory of the CG kernel with O read from X (bytes)
NQ_HD size_t cg_x_smem_bytes(int P) { return (size_t)P * sizeof(float2) + 16; }

__global__ void __launch_bounds__(THREADS, 1) sr_cg_kernel(SrCgArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CgCtl* ctl = reinterpret_cast<CgCtl*>(a.ctl);
  const int N = a.N, M = a.M, P = a.P, Ns = a.Ns, hilb = a.hilb;
  const int NP8 = pad8(N);
  float2* s_v = reinterpret_cast<float2*>(smem_raw);                 // [P] direction, FP32
  float2* s_acc = s_v + P;                                            // [P] this CTA's adjoint sums
  float2* s_z = s_acc + P;                                            // [M][TSP] conj(g) t of a tile
  float* s_sig = reinterpret_cast<float*>(
      (reinterpret_cast<uintptr_t>(s_z + (size_t)M * TSP) + 15) & ~(uintptr_t)15);   // [TS][NP8] σ of a tile
  float2* s_t = reinterpret_cast<float2*>(s_sig + (size_t)TS * NP8); // [TS]
  uint64_t* s_bits = reinterpret_cast<uint64_t*>(s_t + TS);          // [TS]
  __shared__ double s_c[2];
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  // parameter slice of this CTA for the vector updates
  const int per = (P + G - 1) / G, p0 = min(P, b * per), p1 = min(P, p0 + per);
  // sample chunk of this CTA for the adjoint
  const int chunk = (Ns + G - 1) / G, s0 = min(Ns, b * chunk), s1 = min(Ns, s0 + chunk);
  const double inv_ns = 1.0 / Ns;
  const bool xs = a.X != nullptr;      // O from the centred rows of X
  const size_t ldx = (size_t)a.ldx;

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
      double cx = 0.0, cy = 0.0;      // ⟨O⟩·p, same fixed order in every CTA (X is centred: 0)
      for (int p = tid; p < (xs ? 0 : P); p += THREADS) {
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
    // X: one thread per sample, t_s = Σ_p O_c,p(s) v_p over the rows of X
    for (int s = b * THREADS + tid; xs && s < Ns; s += G * THREADS) {
      const float* xc = a.X + s;
      float tx = 0.f, ty = 0.f;
#pragma unroll 16          // 32 independent loads in flight per thread
      for (int p = 0; p < P; ++p) {
        const float ore = __ldg(xc + (size_t)(2 * p) * ldx), oim = __ldg(xc + (size_t)(2 * p + 1) * ldx);
        const float2 v = s_v[p];
        tx += ore * v.x - oim * v.y;
        ty += ore * v.y + oim * v.x;
      }
      a.t[s] = make_float2(tx, ty);
    }
    // RBM: one thread per sample; the hidden units in register chunks of FH, so a
    // site value serves FH units: u_h = v_b,h + Σ_j v_W,hj σ_j, t += g_h u_h
    for (int s = b * THREADS + tid; !xs && s < Ns; s += G * THREADS) {
      const uint64_t bits = a.samples[s];
      float tx = -cx, ty = -cy;
      for (int j = 0; j < N; ++j) {
        const float sv = site_valuef(bits, j, hilb);
        tx += s_v[j].x * sv;
        ty += s_v[j].y * sv;
      }
      for (int h0 = 0; h0 < M; h0 += FH) {
        float2 z[FH];
#pragma unroll
        for (int u = 0; u < FH; ++u) z[u] = h0 + u < M ? s_v[N + h0 + u] : make_float2(0.f, 0.f);
        for (int j = 0; j < N; ++j) {
          const float sv = site_valuef(bits, j, hilb);
          const float2* vw = s_v + N + M + (size_t)M * j + h0;
#pragma unroll
          for (int u = 0; u < FH; ++u)
            if (h0 + u < M) {
              z[u].x += vw[u].x * sv;
              z[u].y += vw[u].y * sv;
            }
        }
#pragma unroll
        for (int u = 0; u < FH; ++u)
          if (h0 + u < M) {
            const float2 gh = a.g[(size_t)(h0 + u) * Ns + s];
            tx += gh.x * z[u].x - gh.y * z[u].y;
            ty += gh.x * z[u].y + gh.y * z[u].x;
          }
      }
      a.t[s] = make_float2(tx, ty);
    }
    if (!cg_barrier(ctl, a.status, a.wait_ns)) return;
    // ---- adjoint partials over this CTA's sample chunk ----
    if (xs) {
      // y_p = Σ_s conj(O_c,p(s)) t_s: a warp per row of X, lanes over the chunk
      const int lane = tid & 31;
      for (int p = tid >> 5; p < P; p += THREADS / 32) {
        const float* xr = a.X + (size_t)(2 * p) * ldx;
        const float* xi = xr + ldx;
        float ax = 0.f, ay = 0.f;
#pragma unroll 4
        for (int s = s0 + lane; s < s1; s += 32) {
          const float ore = __ldg(xr + s), oim = __ldg(xi + s);
          const float2 t = __ldcg(reinterpret_cast<const float2*>(a.t) + s);
          ax += ore * t.x + oim * t.y;
          ay += ore * t.y - oim * t.x;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          ax += __shfl_xor_sync(0xffffffffu, ax, o);
          ay += __shfl_xor_sync(0xffffffffu, ay, o);
        }
        if (lane == 0) {
          a.part[((size_t)b * P + p) * 2] = (double)ax;
          a.part[((size_t)b * P + p) * 2 + 1] = (double)ay;
        }
      }
      if (tid == 0) { a.tsum[2 * b] = 0.0; a.tsum[2 * b + 1] = 0.0; }
    }
    // y_a,j = Σ_s σ_sj t_s, y_b,h = Σ_s z_sh, y_W,hj = Σ_s σ_sj z_sh with
    // z_sh = conj(g_sh) t_s: per tile of TS samples, z and σ are staged in
    // shared memory and the W block is a register-tiled (AH x AJ) contraction
    // over the tile; FP32 sums per tile, added into this CTA's FP32 totals.
    for (int p = tid; !xs && p < P; p += THREADS) s_acc[p] = make_float2(0.f, 0.f);
    const int HT = (M + AH - 1) / AH, JT = (N + AJ - 1) / AJ, ntile = HT * JT;
    float tsx = 0.f, tsy = 0.f;
    for (int c0 = s0; !xs && c0 < s1; c0 += TS) {
      const int nt = min(TS, s1 - c0);
      __syncthreads();
      for (int q = tid; q < TS; q += THREADS) {
        s_t[q] = q < nt ? __ldcg(reinterpret_cast<const float2*>(a.t) + c0 + q) : make_float2(0.f, 0.f);
        s_bits[q] = q < nt ? a.samples[c0 + q] : 0ull;
      }
      __syncthreads();
      for (int e = tid; e < TS * NP8; e += THREADS) {
        const int q = e / NP8, j = e % NP8;
        s_sig[e] = (q < nt && j < N) ? site_valuef(s_bits[q], j, hilb) : 0.f;
      }
      for (int e = tid; e < M * TS; e += THREADS) {
        const int h = e / TS, q = e % TS;
        const float2 gv = q < nt ? a.g[(size_t)h * Ns + c0 + q] : make_float2(0.f, 0.f);
        const float2 tv = s_t[q];
        s_z[h * TSP + q] = make_float2(gv.x * tv.x + gv.y * tv.y, gv.x * tv.y - gv.y * tv.x);
      }
      if (tid == 0)
        for (int q = 0; q < nt; ++q) { tsx += s_t[q].x; tsy += s_t[q].y; }
      __syncthreads();
      for (int p = tid; p < N + M; p += THREADS) {
        float ax = 0.f, ay = 0.f;
        if (p < N) {
          for (int q = 0; q < nt; ++q) {
            const float sv = s_sig[q * NP8 + p];
            ax += sv * s_t[q].x;
            ay += sv * s_t[q].y;
          }
        } else {
          const float2* zr = s_z + (size_t)(p - N) * TSP;
          for (int q = 0; q < nt; ++q) { ax += zr[q].x; ay += zr[q].y; }
        }
        s_acc[p].x += ax;
        s_acc[p].y += ay;
      }
      for (int T = tid; T < ntile; T += THREADS) {
        const int j0 = AJ * (T % JT), h0 = AH * (T / JT);
        float2 acc[AH][AJ];
#pragma unroll
        for (int u = 0; u < AH; ++u)
#pragma unroll
          for (int v = 0; v < AJ; ++v) acc[u][v] = make_float2(0.f, 0.f);
        for (int q = 0; q < nt; ++q) {
          float2 z[AH];
#pragma unroll
          for (int u = 0; u < AH; ++u) z[u] = h0 + u < M ? s_z[(h0 + u) * TSP + q] : make_float2(0.f, 0.f);
          const float4 sa = *reinterpret_cast<const float4*>(s_sig + q * NP8 + j0);
          const float4 sb = *reinterpret_cast<const float4*>(s_sig + q * NP8 + j0 + 4);
          const float sg[AJ] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y, sb.z, sb.w};
#pragma unroll
          for (int u = 0; u < AH; ++u)
#pragma unroll
            for (int v = 0; v < AJ; ++v) {
              acc[u][v].x += z[u].x * sg[v];
              acc[u][v].y += z[u].y * sg[v];
            }
        }
#pragma unroll
        for (int u = 0; u < AH; ++u)
#pragma unroll
          for (int v = 0; v < AJ; ++v)
            if (h0 + u < M && j0 + v < N) {
              float2& d = s_acc[N + M + (h0 + u) + (size_t)M * (j0 + v)];
              d.x += acc[u][v].x;
              d.y += acc[u][v].y;
            }
      }
    }
    __syncthreads();
    for (int p = tid; !xs && p < P; p += THREADS) {
      a.part[((size_t)b * P + p) * 2] = (double)s_acc[p].x;
      a.part[((size_t)b * P + p) * 2 + 1] = (double)s_acc[p].y;
    }
    if (tid == 0 && !xs) { a.tsum[2 * b] = tsx; a.tsum[2 * b + 1] = tsy; }
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

// the same from the centred rows of X: S_pp = mean |O_c,p|², a warp per row
__global__ void sr_diag_x_kernel(SrCgArgs a, double lam, int kind) {
  const int lane = threadIdx.x & 31;
  const int p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (p >= a.P) return;                 // p is uniform across the warp
  if (kind != 1) {
    if (lane == 0) a.shift[p] = kind == 0 ? a.eps : 0.0;
    return;
  }
  const float* xr = a.X + (size_t)(2 * p) * a.ldx;
  const float* xi = xr + a.ldx;
  double acc = 0.0;
  for (int s = lane; s < a.Ns; s += 32) {
    const double r = xr[s], i = xi[s];
    acc += r * r + i * i;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) a.shift[p] = lam * (acc / a.Ns);
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
bool sr_cg_supported(int N, int M) { return cg_smem_bytes(N, M) <= 220 * 1024; }
bool sr_cg_x_supported(int P) { return P >= 1 && cg_x_smem_bytes(P) <= 220 * 1024; }

cudaError_t launch_sr_cg(const SrCgArgs& args, int kind, double lam, cudaStream_t st) {
  const bool xs = args.X != nullptr;
  if (xs ? (!sr_cg_x_supported(args.P) || args.ldx < args.Ns) : !sr_cg_supported(args.N, args.M))
    return cudaErrorInvalidValue;
  if (xs) sr_diag_x_kernel<<<(args.P + 7) / 8, 256, 0, st>>>(args, lam, kind);
  else sr_diag_kernel<<<(args.P + 255) / 256, 256, 0, st>>>(args, lam, kind);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(args.ctl, 0, sizeof(CgCtl), st);
  if (e != cudaSuccess) return e;
  const size_t smem = xs ? cg_x_smem_bytes(args.P) : cg_smem_bytes(args.N, args.M);
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
