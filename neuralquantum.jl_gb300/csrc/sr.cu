// Stochastic reconfiguration: the S = O_c O_c† accumulation (FP32 CUDA-core
// variant and the X materialisation for the tcgen05 variant), assembly of the
// Hermitian S, the diagonally shifted solve (FP32 inverse of the shifted S
// with FP64 iterative refinement, so the returned Δw solves the FP64 system), the
// Descent update and the Measurement statistics.
//
// Reference: src/Algorithms/SR/SRDirect.jl:26-90 (S, F, shift, Cholesky),
// src/Optimisers/apply.jl:25-32 + rules.jl:15-17 (Descent),
// src/utils/stats.jl:26-50 (Measurement).
#include <algorithm>
#include "nq_kernels.cuh"

namespace {

// value of real row `row` of X = [Re O_c; Im O_c] (interleaved) at sample s
__device__ __forceinline__ float x_value(const RbmOSource& src, int row, int s, uint64_t bits) {
  const int N = src.N, M = src.M;
  const int k = row >> 1, part = row & 1;
  float ox, oy;
  if (k < N) { ox = site_valuef(bits, k, src.hilb); oy = 0.f; }
  else if (k < N + M) { float2 g = src.g[(size_t)(k - N) * src.Ns + s]; ox = g.x; oy = g.y; }
  else {
    int q = k - N - M, h = q % M, j = q / M;
    float2 g = src.g[(size_t)h * src.Ns + s];
    float v = site_valuef(bits, j, src.hilb);
    ox = g.x * v; oy = g.y * v;
  }
  ox -= (float)src.meanO[2 * k];
  oy -= (float)src.meanO[2 * k + 1];
  return part ? oy : ox;
}

__device__ __forceinline__ void tile_of(int t, int nt, int* ti, int* tj) {
  // enumerate upper tiles row by row: (0,0),(0,1),...,(0,nt-1),(1,1),...
  int i = 0, rem = t;
  while (rem >= nt - i) { rem -= nt - i; ++i; }
  *ti = i; *tj = i + rem;
}

// 64x64 output tile per block, 16x16 threads with 4x4 micro tiles, K chunks of
// 16 samples generated on the fly from (σ, g, <O>).
constexpr int GT = 64, GK = 16;
template <bool FROM_X>
__global__ void __launch_bounds__(256)
gram_simt_kernel(RbmOSource src, const float* __restrict__ X, int ldx, int rows, int nt, int ksplit,
                 float* __restrict__ partial) {
  __shared__ float As[GK][GT + 4];
  __shared__ float Bs[GK][GT + 4];
  int ti, tj;
  tile_of(blockIdx.x, nt, &ti, &tj);
  const int kz = blockIdx.y;
  const int per = (src.Ns + ksplit - 1) / ksplit;
  const int kb = kz * per, ke = min(src.Ns, kb + per);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  // two-level accumulation: acc over <= 512 samples, folded into tot, keeps
  // the FP32 rounding error independent of Ns
  float acc[4][4] = {}, tot[4][4] = {};
  int nk = 0;
  for (int k0 = kb; k0 < ke; k0 += GK) {
    // generate: thread -> (sample t = tid % 16, rows tid/16 + 16 q)
    {
      const int t = threadIdx.x % GK;
      const int s = k0 + t;
      const bool ok = s < ke;
      const uint64_t bits = (ok && !FROM_X) ? src.samples[s] : 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int r = threadIdx.x / GK + 16 * q;
        int ra = ti * GT + r, rb = tj * GT + r;
        if (FROM_X) {
          As[t][r] = (ok && ra < rows) ? X[(size_t)ra * ldx + s] : 0.f;
          Bs[t][r] = (ok && rb < rows) ? X[(size_t)rb * ldx + s] : 0.f;
        } else {
          As[t][r] = (ok && ra < rows) ? x_value(src, ra, s, bits) : 0.f;
          Bs[t][r] = (ok && rb < rows) ? x_value(src, rb, s, bits) : 0.f;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { a[i] = As[kk][ty * 4 + i]; b[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
    if (++nk == 32) {
      nk = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) { tot[i][j] += acc[i][j]; acc[i][j] = 0.f; }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) tot[i][j] += acc[i][j];
  // partial layout: [ksplit][rows_pad][rows_pad] with rows_pad = nt*64
  const int rp = nt * GT;
  float* dst = partial + (size_t)kz * rp * rp;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      dst[(size_t)(ti * GT + ty * 4 + i) * rp + tj * GT + tx * 4 + j] = tot[i][j];
}

// sum split-K partials of the upper tiles into G (rows x rows, row-major)
__global__ void gram_reduce_kernel(const float* __restrict__ partial, int rows, int rp, int tile,
                                   int ksplit, float* __restrict__ G) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)rows * rows) return;
  int a = (int)(idx / rows), b = (int)(idx % rows);
  if (a / tile > b / tile) return;   // lower tiles were not computed
  float s = 0.f;
  for (int z = 0; z < ksplit; ++z) s += partial[(size_t)z * rp * rp + (size_t)a * rp + b];
  G[idx] = s;
}

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

template <bool BF16>
__device__ __forceinline__ void put_x_row(float* X, float* Xlo, int row, int Ns_pad, int s0, const float (&v)[4]) {
  if (BF16) {
    __align__(8) __nv_bfloat16 b[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) b[e] = __float2bfloat16_rn(v[e]);
    *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(X) + (size_t)row * Ns_pad + s0) =
        *reinterpret_cast<const uint2*>(b);
  } else {
    const float4 hi = make_float4(to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
    *reinterpret_cast<float4*>(X + (size_t)row * Ns_pad + s0) = hi;
    if (Xlo)
      *reinterpret_cast<float4*>(Xlo + (size_t)row * Ns_pad + s0) =
          make_float4(to_tf32(v[0] - hi.x), to_tf32(v[1] - hi.y), to_tf32(v[2] - hi.z), to_tf32(v[3] - hi.w));
  }
}

// X row 2k + part holds Re (part 0) or Im (part 1) of O_k - <O_k> over the
// samples, zero in the padding.  One block per (sample range, source unit u):
// u < M is hidden unit h = u and writes the rows of b_h (k = N + h) and of
// every weight W_hj (k = N + M + j M + h); u = M writes the rows of the
// visible units a_j (k = j).  Each thread loads σ and g_h of four consecutive
// samples once and writes all 2(N + 1) rows that depend on them, 16-byte
// stores coalesced across the warp: the kernel is bound by the X writes
// (4 rows Ns_pad bytes, twice with Xlo, half with BF16), not by re-reads.
template <bool BF16>
NQ_D void build_X_block(const RbmOSource& src, int Ns_pad, float* __restrict__ X, float* __restrict__ Xlo, int bx,
                        int u) {
  const int N = src.N, M = src.M, Ns = src.Ns, hilb = src.hilb;
  const int s0 = (bx * blockDim.x + threadIdx.x) * 4;
  if (s0 >= Ns_pad) return;
  uint64_t bits[4];
  float2 g[4];
  bool valid[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int s = s0 + e;
    valid[e] = s < Ns;
    bits[e] = valid[e] ? src.samples[s] : 0ull;
    g[e] = (valid[e] && u < M) ? src.g[(size_t)u * Ns + s] : make_float2(0.f, 0.f);
  }
  float vr[4], vi[4];
  if (u == M) {
    for (int j = 0; j < N; ++j) {
      const float mr = (float)src.meanO[2 * j], mi = (float)src.meanO[2 * j + 1];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        vr[e] = valid[e] ? site_valuef(bits[e], j, hilb) - mr : 0.f;
        vi[e] = valid[e] ? 0.f - mi : 0.f;
      }
      put_x_row<BF16>(X, Xlo, 2 * j, Ns_pad, s0, vr);
      put_x_row<BF16>(X, Xlo, 2 * j + 1, Ns_pad, s0, vi);
    }
    return;
  }
  const int h = u;
  {
    const int k = N + h;
    const float mr = (float)src.meanO[2 * k], mi = (float)src.meanO[2 * k + 1];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      vr[e] = valid[e] ? g[e].x - mr : 0.f;
      vi[e] = valid[e] ? g[e].y - mi : 0.f;
    }
    put_x_row<BF16>(X, Xlo, 2 * k, Ns_pad, s0, vr);
    put_x_row<BF16>(X, Xlo, 2 * k + 1, Ns_pad, s0, vi);
  }
  for (int j = 0; j < N; ++j) {
    const int k = N + M + j * M + h;
    const float mr = (float)src.meanO[2 * k], mi = (float)src.meanO[2 * k + 1];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float w = site_valuef(bits[e], j, hilb);
      vr[e] = valid[e] ? g[e].x * w - mr : 0.f;
      vi[e] = valid[e] ? g[e].y * w - mi : 0.f;
    }
    put_x_row<BF16>(X, Xlo, 2 * k, Ns_pad, s0, vr);
    put_x_row<BF16>(X, Xlo, 2 * k + 1, Ns_pad, s0, vi);
  }
}

template <bool BF16>
__global__ void __launch_bounds__(256) build_X_kernel(RbmOSource src, int Ns_pad, float* __restrict__ X,
                                                      float* __restrict__ Xlo) {
  build_X_block<BF16>(src, Ns_pad, X, Xlo, blockIdx.x, blockIdx.y);
}

// grouped: problem p owns blocks [x_blk[p], x_blk[p+1]) = (M + 1) units x
// ceil(Ns_pad / 1024) sample ranges, unit-major
__global__ void __launch_bounds__(256) build_X_group_kernel(SrGroup g, int split3) {
  const int p = group_of(blockIdx.x, g.x_blk, g.np);
  const SrJob& j = g.jobs[p];
  const int local = blockIdx.x - __ldg(g.x_blk + p);
  const int nbx = (j.Ns_pad + 1023) / 1024;
  RbmOSource src;
  src.N = j.N; src.M = j.M; src.hilb = j.hilb; src.Ns = j.Ns;
  src.samples = j.samples; src.g = j.g; src.meanO = j.fb.meanO;
  build_X_block<false>(src, j.Ns_pad, j.X, split3 ? j.Xlo : nullptr, local % nbx, local / nbx);
}

__device__ __forceinline__ float gsym(const float* G, int rows, int a, int b) {
  return a <= b ? G[(size_t)a * rows + b] : G[(size_t)b * rows + a];
}

// S[k + P l] (column-major, complex double):
//   Re = (G[2k][2l] + G[2k+1][2l+1]) / Ns,  Im = (G[2k][2l+1] - G[2k+1][2l]) / Ns
// which is conj(O_c O_c†)/Ns (SRDirect.jl:41-43); real parameters keep Re only.
__global__ void assemble_S_kernel(const float* __restrict__ G, int P, double inv_ns, int real_params,
                                  double* __restrict__ S) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)P * P) return;
  int k = (int)(idx % P), l = (int)(idx / P);
  const int rows = 2 * P;
  double re = ((double)gsym(G, rows, 2 * k, 2 * l) + (double)gsym(G, rows, 2 * k + 1, 2 * l + 1)) * inv_ns;
  double im = real_params ? 0.0
                          : ((double)gsym(G, rows, 2 * k, 2 * l + 1) - (double)gsym(G, rows, 2 * k + 1, 2 * l)) * inv_ns;
  S[2 * idx] = re;
  S[2 * idx + 1] = im;
}

// ---------------------------------------------------------------------------
// Shifted copy into the FP32 factor workspace (lower triangle, column-major).
// kind 0: S_ii += eps;  kind 1: S_ii += lam * S_ii;  kind 2: none.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double diag_shift(const double* S, int P, int i, int kind, double eps,
                                             double lam) {
  return sr_diag_shift(S, P, i, kind, eps, lam);
}

__global__ void shift_copy_kernel(const double* __restrict__ S, int P, int kind, double eps,
                                  double lam, float2* __restrict__ W) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)P * P) return;
  int i = (int)(idx % P), j = (int)(idx / P);
  double re = S[2 * idx], im = S[2 * idx + 1];
  if (i == j) { re += diag_shift(S, P, i, kind, eps, lam); im = 0.0; }
  W[idx] = make_float2((float)re, (float)im);
}

// grouped: S = conj(G)/Ns (complex parameters) and W = S + eps I of every
// problem, one element (k, l) per thread
__global__ void assemble_shift_group_kernel(SrGroup g, double eps) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.pp_elems) return;
  const int p = group_of(e, g.pp_elem, g.np);
  const SrJob& j = g.jobs[p];
  const int idx = e - __ldg(g.pp_elem + p), P = j.P, rows = 2 * P;
  const int k = idx % P, l = idx / P;
  const double inv_ns = 1.0 / j.Ns;
  const double re = ((double)gsym(j.G, rows, 2 * k, 2 * l) + (double)gsym(j.G, rows, 2 * k + 1, 2 * l + 1)) * inv_ns;
  const double im = ((double)gsym(j.G, rows, 2 * k, 2 * l + 1) - (double)gsym(j.G, rows, 2 * k + 1, 2 * l)) * inv_ns;
  j.S[2 * (size_t)idx] = re;
  j.S[2 * (size_t)idx + 1] = im;
  j.W[idx] = k == l ? make_float2((float)(re + eps), 0.f) : make_float2((float)re, (float)im);
}



__global__ void refine_update_kernel(double* x, const float2* __restrict__ d, int P, int first) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  if (first) { x[2 * i] = 0.0; x[2 * i + 1] = 0.0; }
  x[2 * i] += (double)d[i].x;
  x[2 * i + 1] += (double)d[i].y;
}

__global__ void __launch_bounds__(128)
residual_kernel(const double* __restrict__ S, int P, const double* __restrict__ F,
                const double* __restrict__ x, int kind, double eps, double lam, int real_params,
                double* __restrict__ r, float2* __restrict__ rf) {
  const int k = blockIdx.x;
  // (S x)_k = Σ_l S[k][l] x_l = Σ_l conj(S[l][k]) x_l (Hermitian; column k contiguous)
  double sx = 0.0, sy = 0.0;
#pragma unroll 4
  for (int l = threadIdx.x; l < P; l += blockDim.x) {
    double ar = S[2 * ((size_t)l + (size_t)P * k)], ai = -S[2 * ((size_t)l + (size_t)P * k) + 1];
    if (l == k) ai = 0.0;
    double xr = x[2 * l], xi = x[2 * l + 1];
    sx += ar * xr - ai * xi;
    sy += ar * xi + ai * xr;
  }
  __shared__ double red[2][4];
  for (int off = 16; off > 0; off >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, off);
    sy += __shfl_xor_sync(0xffffffffu, sy, off);
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = sx; red[1][threadIdx.x >> 5] = sy; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tx = red[0][0] + red[0][1] + red[0][2] + red[0][3];
    double ty = red[1][0] + red[1][1] + red[1][2] + red[1][3];
    double dsh = diag_shift(S, P, k, kind, eps, lam);
    tx += dsh * x[2 * k];
    ty += dsh * x[2 * k + 1];
    double fx = F[2 * k], fy = real_params ? 0.0 : F[2 * k + 1];
    double rx = fx - tx, ry = fy - ty;
    r[2 * k] = rx;
    r[2 * k + 1] = ry;
    rf[k] = make_float2((float)rx, (float)ry);
  }
}

__global__ void rhs_init_kernel(const double* F, int P, int real_params, float2* rf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  rf[i] = make_float2((float)F[2 * i], real_params ? 0.f : (float)F[2 * i + 1]);
}

__global__ void descent_kernel(double* w, const double* dw, long n, int stride, double lr) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) w[i] -= lr * dw[i * stride];
}

// ---------------------------------------------------------------------------
// Measurement statistics, one block; FP64 with fixed reduction order.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ cpx<double> stat_val(const cpx<R>* v, long i, int mode) {
  cpx<R> a = v[i];
  if (mode == 1) return mk((double)a.x * a.x + (double)a.y * a.y, 0.0);
  return mk((double)a.x, (double)a.y);
}


// pass 1 (one thread per chain, 64 chains per block): chain mean μ_c and
// unbiased variance var_c from two passes over the chain's L values; per
// block, with n_b valid chains, the block mean m_b = Σ μ_c / n_b, the centred
// sum M2_b = Σ |μ_c - m_b|² and Σ var_c, written as
// part[5 b ..] = [n_b, Re m_b, Im m_b, M2_b, Σ var_c] (fixed shuffle order).
// Centring inside the block keeps the spread of the chain means exact when
// it is tiny next to the mean itself (a local energy of -40 with a spread of
// 1e-6), where Σ|μ_c|² - B|μ|² would cancel to rounding noise.
template <typename R>
NQ_D void chain_stats_block(const cpx<R>* __restrict__ v, int B, int L, int mode, double* __restrict__ part,
                            int blk) {
  const int c = blk * blockDim.x + threadIdx.x;
  const bool valid = c < B;
  double mx = 0, my = 0, var = 0;
  if (valid) {
    for (int l = 0; l < L; ++l) { cpx<double> x = stat_val(v, c + (long)B * l, mode); mx += x.x; my += x.y; }
    mx /= L; my /= L;
    double vv = 0;
    for (int l = 0; l < L; ++l) {
      cpx<double> x = stat_val(v, c + (long)B * l, mode);
      vv += (x.x - mx) * (x.x - mx) + (x.y - my) * (x.y - my);
    }
    var = L > 1 ? vv / (L - 1) : 0.0;
  }
  __shared__ double sh[2][3];
  double q[3] = {valid ? mx : 0.0, valid ? my : 0.0, var};
#pragma unroll
  for (int k = 0; k < 3; ++k)
    for (int off = 16; off > 0; off >>= 1) q[k] += __shfl_xor_sync(0xffffffffu, q[k], off);
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; ++k) sh[threadIdx.x >> 5][k] = q[k];
  __syncthreads();
  const int nb = min(64, B - blk * 64);
  const double bx = (sh[0][0] + sh[1][0]) / nb, by = (sh[0][1] + sh[1][1]) / nb;
  const double vsum = sh[0][2] + sh[1][2];
  double d2 = valid ? (mx - bx) * (mx - bx) + (my - by) * (my - by) : 0.0;
  for (int off = 16; off > 0; off >>= 1) d2 += __shfl_xor_sync(0xffffffffu, d2, off);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][0] = d2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double* o = part + 5 * (size_t)blk;
    o[0] = (double)nb;
    o[1] = bx;
    o[2] = by;
    o[3] = sh[0][0] + sh[1][0];
    o[4] = vsum;
  }
}

// merge two (n, mean, M2) summaries of chain means (Chan, Golub and LeVeque's
// pairwise update), plus the summed chain variances
struct ChainSummary {
  double n, mx, my, m2, vs;
};
__device__ __forceinline__ ChainSummary merge_summary(const ChainSummary& a, const ChainSummary& b) {
  if (a.n == 0.0) return b;
  if (b.n == 0.0) return a;
  ChainSummary r;
  r.n = a.n + b.n;
  const double dx = b.mx - a.mx, dy = b.my - a.my, f = b.n / r.n;
  r.mx = a.mx + dx * f;
  r.my = a.my + dy * f;
  r.m2 = a.m2 + b.m2 + (dx * dx + dy * dy) * a.n * f;
  r.vs = a.vs + b.vs;
  return r;
}

// pass 2 (one warp, fixed order): lane l merges blocks l, l + 32, ... in
// order, then the lanes merge pairwise down a fixed tree.  With μ the mean of
// the chain means and Σ|μ_c - μ|² = M2:
// var_μ_ch = M2/(B-1); var_μ = [(L-1) Σ var_c + L M2]/(BL-1) (= the variance
// of all values about μ); variance = mean var_c; t = var_μ_ch/var_μ
// (stats.jl:26-50)
template <typename R>
__global__ void __launch_bounds__(64) chain_stats_kernel(const cpx<R>* __restrict__ v, int B, int L, int mode,
                                                         double* __restrict__ part) {
  chain_stats_block<R>(v, B, L, mode, part, blockIdx.x);
}

NQ_D void stats_final_warp(const double* __restrict__ part, int nblk, int B, int L, double* __restrict__ out) {
  ChainSummary s = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblk; b += 32) {
    const double* p = part + 5 * (size_t)b;
    const ChainSummary t = {p[0], p[1], p[2], p[3], p[4]};
    s = merge_summary(s, t);
  }
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    ChainSummary o;
    o.n = __shfl_down_sync(0xffffffffu, s.n, off);
    o.mx = __shfl_down_sync(0xffffffffu, s.mx, off);
    o.my = __shfl_down_sync(0xffffffffu, s.my, off);
    o.m2 = __shfl_down_sync(0xffffffffu, s.m2, off);
    o.vs = __shfl_down_sync(0xffffffffu, s.vs, off);
    if ((threadIdx.x & (2 * off - 1)) == 0 && threadIdx.x + off < 32) s = merge_summary(s, o);
  }
  if (threadIdx.x == 0) {
    const double dev = s.m2;                       // Σ|μ_c - μ|²
    const double var_mu_ch = B > 1 ? dev / (B - 1) : 0.0;
    const double var_mu = ((L - 1) * s.vs + L * dev) / ((double)B * L - 1);
    const double t = var_mu > 0.0 ? var_mu_ch / var_mu : 0.0;
    out[0] = s.mx;
    out[1] = s.my;
    out[2] = sqrt(var_mu_ch / B);
    out[3] = s.vs / B;
    out[4] = fmax(0.0, 0.5 * (t * L - 1.0));
    out[5] = sqrt((double)(L - 1) / L + t);
  }
}

__global__ void __launch_bounds__(32) stats_final_kernel(const double* __restrict__ part, int nblk, int B, int L,
                                                         double* __restrict__ out) {
  stats_final_warp(part, nblk, B, L, out);
}

// ---- grouped forms (many-problem step, FP32)
__global__ void __launch_bounds__(64) chain_stats_group_kernel(SrGroup g) {
  const int p = group_of(blockIdx.x, g.stat_blk, g.np);
  const SrJob& j = g.jobs[p];
  chain_stats_block<float>(reinterpret_cast<const cpx<float>*>(j.eloc), j.B, j.L, 0, j.chainstats,
                           blockIdx.x - __ldg(g.stat_blk + p));
}

__global__ void __launch_bounds__(32) stats_final_group_kernel(SrGroup g) {
  const SrJob& j = g.jobs[blockIdx.x];
  stats_final_warp(j.chainstats, (j.B + 63) / 64, j.B, j.L, j.stats);
}

}  // namespace

// ------------------------------- launchers ---------------------------------

cudaError_t launch_gram_simt(const RbmOSource& src, int P, float* G, float* partial, int ksplit,
                             cudaStream_t st) {
  const int rows = 2 * P;
  const int nt = (rows + GT - 1) / GT;
  const int ntiles = nt * (nt + 1) / 2;
  dim3 grid(ntiles, ksplit);
  gram_simt_kernel<false><<<grid, 256, 0, st>>>(src, nullptr, 0, rows, nt, ksplit, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  long tot = (long)rows * rows;
  gram_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(partial, rows, nt * GT, GT, ksplit, G);
  return cudaGetLastError();
}

cudaError_t launch_gram_simt_x(const float* X, int ldx, int ns, int rows, float* G, float* partial, int ksplit,
                               cudaStream_t st) {
  const int nt = (rows + GT - 1) / GT;
  const int ntiles = nt * (nt + 1) / 2;
  dim3 grid(ntiles, ksplit);
  RbmOSource src;
  src.Ns = ns;
  gram_simt_kernel<true><<<grid, 256, 0, st>>>(src, X, ldx, rows, nt, ksplit, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  long tot = (long)rows * rows;
  gram_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(partial, rows, nt * GT, GT, ksplit, G);
  return cudaGetLastError();
}

cudaError_t launch_build_X(const RbmOSource& src, int P, int Ns_pad, float* X, float* Xlo,
                           cudaStream_t st, int bf16) {
  if (Ns_pad % 4 != 0 || src.M + 1 > 65535 || P != src.N + src.M + src.N * src.M) return cudaErrorInvalidValue;
  const int per_block = 256 * 4;
  const dim3 grid((unsigned)((Ns_pad + per_block - 1) / per_block), (unsigned)(src.M + 1));
  if (bf16) build_X_kernel<true><<<grid, 256, 0, st>>>(src, Ns_pad, X, nullptr);
  else build_X_kernel<false><<<grid, 256, 0, st>>>(src, Ns_pad, X, Xlo);
  return cudaGetLastError();
}

cudaError_t launch_gram_reduce(const float* partial, int rows, int rp, int tile, int ksplit, float* G,
                               cudaStream_t st) {
  long tot = (long)rows * rows;
  gram_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(partial, rows, rp, tile, ksplit, G);
  return cudaGetLastError();
}

cudaError_t launch_assemble_S(const float* G, int P, double inv_ns, bool real_params, double* S,
                              cudaStream_t st) {
  long tot = (long)P * P;
  assemble_S_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(G, P, inv_ns, real_params ? 1 : 0, S);
  return cudaGetLastError();
}

cudaError_t launch_sr_shift(const SolveBufs& sb, int P, int kind, double eps, double lam, cudaStream_t st) {
  const long tot = (long)P * P;
  shift_copy_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(sb.S, P, kind, eps, lam, sb.W);
  return cudaGetLastError();
}

cudaError_t launch_sr_finish(const SolveBufs& sb, int P, const double* F, int kind, double eps, double lam,
                             bool real_params, int refine_iters, cudaStream_t st) {
  auto mark = [&](int k) { if (sb.ev) cudaEventRecord(sb.ev[k], st); };
  cudaError_t e = launch_herm_fill(sb.W, P, st);
  if (e != cudaSuccess) return e;
  mark(2);
  rhs_init_kernel<<<(P + 255) / 256, 256, 0, st>>>(F, P, real_params ? 1 : 0, sb.rf);
  mark(3);
  for (int it = 0; it <= refine_iters; ++it) {
    e = launch_herm_gemv_neg(sb.W, P, sb.rf, sb.yf, st);
    if (e != cudaSuccess) return e;
    if (it == 0) mark(4);
    refine_update_kernel<<<(P + 255) / 256, 256, 0, st>>>(sb.x, sb.yf, P, it == 0);
    residual_kernel<<<P, 128, 0, st>>>(sb.S, P, F, sb.x, kind, eps, lam, real_params ? 1 : 0, sb.r, sb.rf);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  mark(5);
  return cudaSuccess;
}

cudaError_t launch_sr_solve(const SolveBufs& sb, int P, const double* F, int kind, double eps,
                            double lam, bool real_params, int refine_iters, cudaStream_t st) {
  auto mark = [&](int k) { if (sb.ev) cudaEventRecord(sb.ev[k], st); };
  mark(0);
  cudaError_t e = launch_sr_shift(sb, P, kind, eps, lam, st);
  if (e != cudaSuccess) return e;
  mark(1);
  e = launch_spd_inverse(sb.W, P, sb.ctl, sb.status, sb.work, st, sb.wait_ns);
  if (e != cudaSuccess) return e;
  // one problem on the GPU: the refinement as one cooperative launch (the
  // many-problem step keeps launch_sr_finish, whose small kernels run side by
  // side in the graph branches)
  e = launch_herm_fill(sb.W, P, st);
  if (e != cudaSuccess) return e;
  mark(2);
  mark(3);
  mark(4);
  e = launch_refine_coop(sb.W, sb.S, P, F, kind, eps, lam, real_params, refine_iters, kRefineTol, sb.x, sb.r,
                         sb.rf, sb.norms, sb.info, sb.ctl, sb.status, st, sb.wait_ns);
  if (e != cudaSuccess) return e;
  mark(5);
  return cudaSuccess;
}

__global__ void times_i_kernel(const double* __restrict__ F, int P, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P) return;
  const double x = F[2 * k], y = F[2 * k + 1];
  out[2 * k] = -y;          // i (x + i y) = -y + i x; its real part is what a real solve reads
  out[2 * k + 1] = x;
}

cudaError_t launch_times_i(const double* F, int P, double* out, cudaStream_t st) {
  times_i_kernel<<<(P + 255) / 256, 256, 0, st>>>(F, P, out);
  return cudaGetLastError();
}

cudaError_t launch_descent(double* master, const double* dw, long n_doubles, int stride, double lr,
                           cudaStream_t st) {
  descent_kernel<<<(unsigned)((n_doubles + 255) / 256), 256, 0, st>>>(master, dw, n_doubles, stride, lr);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_stats(const cpx<R>* vals, int B, int L, int mode, double* chain_scratch, double* out6,
                         cudaStream_t st) {
  const int nblk = (B + 63) / 64;
  chain_stats_kernel<R><<<nblk, 64, 0, st>>>(vals, B, L, mode, chain_scratch);   // 5 nblk doubles
  stats_final_kernel<<<1, 32, 0, st>>>(chain_scratch, nblk, B, L, out6);
  return cudaGetLastError();
}
template cudaError_t launch_stats<float>(const cpx<float>*, int, int, int, double*, double*, cudaStream_t);
template cudaError_t launch_stats<double>(const cpx<double>*, int, int, int, double*, double*, cudaStream_t);

cudaError_t launch_stats_group(const SrGroup& g, cudaStream_t st) {
  chain_stats_group_kernel<<<g.stat_blocks, 64, 0, st>>>(g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  stats_final_group_kernel<<<g.np, 32, 0, st>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_build_X_group(const SrGroup& g, int split3, cudaStream_t st) {
  build_X_group_kernel<<<g.x_blocks, 256, 0, st>>>(g, split3);
  return cudaGetLastError();
}

cudaError_t launch_assemble_shift_group(const SrGroup& g, double eps, cudaStream_t st) {
  assemble_shift_group_kernel<<<(g.pp_elems + 255) / 256, 256, 0, st>>>(g, eps);
  return cudaGetLastError();
}
