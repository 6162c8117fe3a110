// Shifted SR solve, inversion part.  The reference factors the shifted S
// with cholesky! and solves once (SRDirect.jl:79-81).  Here the Hermitian
// positive-definite A = S + shift is inverted explicitly, in FP32, by a block
// Gauss–Jordan sweep over 32-wide blocks in ONE cooperative launch; every
// solve after that (the first one and each FP64-residual refinement step) is
// a Hermitian matrix-vector product spread over all SMs, instead of a chain of
// dependent triangular-solve steps.
//
// Sweep of block k on the lower triangle of W (W = A at the start):
//   piv = W_kk^-1;  C_i = W_ik piv  (i != k, old column k)
//   W_ij -= C_i W_jkᴴ    for lower tiles i >= j, i, j != k
//   W_ik  = C_i (i > k);  W_ki = C_iᴴ (i < k);  W_kk = -piv
// (Goodnight's sweep operator; every pivot is a Schur complement of A, so it
// is positive definite and no pivoting is needed).  After all blocks
// W = -A^-1.  Each step has two phases separated by grid barriers:
//   A. the CTAs owning a block i != k invert W_kk (32x32 Gauss–Jordan held in
//      registers, one column group per warp) and store C_i and the old W_ik;
//   B. every lower tile is either updated or, on row/column k, overwritten.
// The grid barrier is a generation counter with a bounded spin (1 s, sticky
// abort flag): a stalled barrier ends the kernel with a status bit.
#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int CB = 32;

struct SweepCtl {
  unsigned count;      // arrivals at the current barrier
  unsigned gen;        // barrier generation
  int abort;           // sticky abort flag
  int pad;
};

// Barrier over the `n` CTAs that share ctl (the whole grid, or one group).
__device__ bool group_barrier(SweepCtl* ctl, unsigned n, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    volatile unsigned* vgen = &ctl->gen;
    const unsigned g = *vgen;
    __threadfence();
    if (atomicAdd(&ctl->count, 1u) == n - 1) {
      atomicExch(&ctl->count, 0u);
      __threadfence();
      atomicAdd(&ctl->gen, 1u);
    } else {
      const uint64_t t0 = globaltimer_ns();
      unsigned it = 0;
      while (*vgen == g) {
        if (*(volatile int*)&ctl->abort) { s_ok = 0; break; }
        if ((++it & 255u) == 0 && globaltimer_ns() - t0 > 1000000000ull) {
          atomicOr(err, NQ_DEVERR_TIMEOUT);
          atomicExch(&ctl->abort, 1);
          s_ok = 0;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0;
}

NQ_D float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// In-place inverse of the Hermitian positive-definite 32x32 block T (shared
// memory, all 32x32 entries) by Gauss–Jordan without pivoting, 256 threads:
// lane = row, warp w owns columns 4w..4w+3 in registers.  Per pivot p the
// owner warp publishes the old column p (double-buffered), row p is taken by
// shuffles from lane p.  Returns false if a pivot was not positive.
__device__ bool hpd_inverse_32(float2 (*T)[CB + 1], float2 (*colbuf)[CB]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float2 a[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) a[q] = T[lane][4 * w + q];
  bool ok = true;
#pragma unroll 1
  for (int p = 0; p < CB; ++p) {
    if (w == (p >> 2)) {
      const int oq = p & 3;
      float2 v = a[0];
#pragma unroll
      for (int q = 1; q < 4; ++q)
        if (q == oq) v = a[q];
      colbuf[p & 1][lane] = v;
    }
    __syncthreads();
    const float2 f = colbuf[p & 1][lane];
    float d = colbuf[p & 1][p].x;
    if (!(d > 0.f)) { ok = false; d = 1.f; }
    const float inv = 1.0f / d;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = 4 * w + q;
      float2 rp;
      rp.x = __shfl_sync(0xffffffffu, a[q].x, p);
      rp.y = __shfl_sync(0xffffffffu, a[q].y, p);
      if (j == p) {
        a[q] = lane == p ? make_float2(inv, 0.f) : make_float2(-f.x * inv, -f.y * inv);
      } else {
        const float2 np = make_float2(rp.x * inv, rp.y * inv);
        if (lane == p) {
          a[q] = np;
        } else {
          const float2 t = cmul(f, np);
          a[q].x -= t.x;
          a[q].y -= t.y;
        }
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; ++q) T[lane][4 * w + q] = a[q];
  __syncthreads();
  return ok;
}

// X[r][c] = Σ_p U[r][p] V[p][c] (mode 0)  or  Σ_p U[r][p] conj(V[c][p]) (mode 1),
// element (tid & 31, 4 (tid >> 5) + q) per thread
template <int MODE>
NQ_D void tile_mm(const float2 (*U)[CB + 1], const float2 (*V)[CB + 1], float2 out[4]) {
  const int r = threadIdx.x & 31, cg = (threadIdx.x >> 5) * 4;
#pragma unroll
  for (int q = 0; q < 4; ++q) out[q] = make_float2(0.f, 0.f);
#pragma unroll 8
  for (int p = 0; p < CB; ++p) {
    const float2 u = U[r][p];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float2 v = MODE == 0 ? V[p][cg + q] : V[cg + q][p];
      if (MODE == 0) {
        out[q].x += u.x * v.x - u.y * v.y;
        out[q].y += u.x * v.y + u.y * v.x;
      } else {
        out[q].x += u.x * v.x + u.y * v.y;
        out[q].y += u.y * v.x - u.x * v.y;
      }
    }
  }
}

// The sweep of one matrix by the CTAs rank = 0..nranks-1 of its group.
NQ_D void sweep_group(float2* __restrict__ W, int P, SweepCtl* ctl, int* status, float2* __restrict__ Cbuf,
                      float2* __restrict__ Gbuf, float2* __restrict__ pivbuf, int rank, int nranks) {
  __shared__ float2 Dt[CB][CB + 1];
  __shared__ float2 Ut[CB][CB + 1];
  __shared__ float2 Vt[CB][CB + 1];
  __shared__ float2 colbuf[2][CB];
  const int nblk = (P + CB - 1) / CB;
  const int tr = threadIdx.x & 31, cg = (threadIdx.x >> 5) * 4;
  for (int kb = 0; kb < nblk; ++kb) {
    const int k0 = kb * CB, nbk = min(CB, P - k0);
    // ---------------- phase A: pivot inverse, C_i and the old column ----------------
    const int ncol = nblk - 1;
    const bool has_col = rank < ncol;
    if (has_col || rank == 0) {
      for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
        const int r = e & 31, c = e >> 5;
        float2 v;
        if (r < nbk && c < nbk) {
          v = r >= c ? __ldcg(W + (size_t)(k0 + r) + (size_t)P * (k0 + c))
                     : __ldcg(W + (size_t)(k0 + c) + (size_t)P * (k0 + r));
          if (r < c) v.y = -v.y;
          if (r == c) v.y = 0.f;
        } else {
          v = make_float2(r == c ? 1.f : 0.f, 0.f);
        }
        Dt[r][c] = v;
      }
      __syncthreads();
      const bool ok = hpd_inverse_32(Dt, colbuf);
      if (!ok && rank == 0 && threadIdx.x == 0) atomicOr(status, 1);
      if (rank == 0)
        for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) pivbuf[e] = Dt[e & 31][e >> 5];
    }
    for (int b = rank; b < ncol; b += nranks) {
      const int ib = b < kb ? b : b + 1;
      const int i0 = ib * CB;
      __syncthreads();
      for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
        const int r = e & 31, c = e >> 5;
        float2 v = make_float2(0.f, 0.f);
        if (i0 + r < P && c < nbk) {
          if (ib > kb) {
            v = __ldcg(W + (size_t)(i0 + r) + (size_t)P * (k0 + c));
          } else {
            v = __ldcg(W + (size_t)(k0 + c) + (size_t)P * (i0 + r));
            v.y = -v.y;
          }
        }
        Ut[r][c] = v;
        Gbuf[(size_t)ib * CB * CB + e] = v;
      }
      __syncthreads();
      float2 o[4];
      tile_mm<0>(Ut, Dt, o);
#pragma unroll
      for (int q = 0; q < 4; ++q) Cbuf[(size_t)ib * CB * CB + (cg + q) * CB + tr] = o[q];
    }
    if (!group_barrier(ctl, (unsigned)nranks, status)) return;
    // ---------------- phase B: lower tiles ----------------
    const int ntiles = nblk * (nblk + 1) / 2;
    for (int t = rank; t < ntiles; t += nranks) {
      int ti, tj;
      {
        int c = 0, r = t;
        while (r >= nblk - c) { r -= nblk - c; ++c; }
        tj = c; ti = c + r;
      }
      const int r0 = ti * CB, c0 = tj * CB;
      __syncthreads();
      if (ti != kb && tj != kb) {
        // W_ij -= C_i G_jᴴ
        for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
          const int r = e & 31, c = e >> 5;
          Ut[r][c] = __ldcg(Cbuf + (size_t)ti * CB * CB + e);
          Vt[r][c] = __ldcg(Gbuf + (size_t)tj * CB * CB + e);
        }
        __syncthreads();
        float2 o[4];
        tile_mm<1>(Ut, Vt, o);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int gi = r0 + tr, gj = c0 + cg + q;
          if (gi < P && gj < P && gi >= gj) {
            float2* a = W + (size_t)gi + (size_t)P * gj;
            float2 cur = __ldcg(a);
            cur.x -= o[q].x;
            cur.y -= o[q].y;
            *a = cur;
          }
        }
      } else {
        // row/column k: W_ik = C_i (i > k), W_kj = C_jᴴ (j < k), W_kk = -piv
        for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
          const int r = e & 31, c = e >> 5;
          const int gi = r0 + r, gj = c0 + c;
          if (gi >= P || gj >= P || gi < gj) continue;
          float2 v;
          if (ti == kb && tj == kb) {
            v = __ldcg(pivbuf + e);
            v.x = -v.x;
            v.y = -v.y;
          } else if (tj == kb) {
            v = __ldcg(Cbuf + (size_t)ti * CB * CB + e);
          } else {
            v = __ldcg(Cbuf + (size_t)tj * CB * CB + r * CB + c);   // (C_j)ᴴ[r][c] = conj(C_j[c][r])
            v.y = -v.y;
          }
          W[(size_t)gi + (size_t)P * gj] = v;
        }
      }
    }
    if (!group_barrier(ctl, (unsigned)nranks, status)) return;
  }
}

__global__ void __launch_bounds__(256) sweep_coop_kernel(float2* __restrict__ W, int P, SweepCtl* ctl,
                                                         int* status, float2* __restrict__ Cbuf,
                                                         float2* __restrict__ Gbuf, float2* __restrict__ pivbuf) {
  sweep_group(W, P, ctl, status, Cbuf, Gbuf, pivbuf, blockIdx.x, gridDim.x);
}

// Many matrices in one cooperative launch: matrix p is swept by CTAs
// [cta_start[p], cta_start[p+1]) with its own barrier block.
__global__ void __launch_bounds__(256) sweep_batch_kernel(const SweepJob* __restrict__ jobs,
                                                          const int* __restrict__ cta_start, int np) {
  int lo = 0, hi = np - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(cta_start + mid) <= b) lo = mid; else hi = mid - 1;
  }
  const SweepJob& j = jobs[lo];
  const int r0 = __ldg(cta_start + lo), n = __ldg(cta_start + lo + 1) - r0;
  sweep_group(j.W, j.P, reinterpret_cast<SweepCtl*>(j.ctl), j.status, j.work,
              j.work + (size_t)((j.P + CB - 1) / CB) * CB * CB, j.work + (size_t)2 * ((j.P + CB - 1) / CB) * CB * CB,
              b - r0, n);
}

// W upper = conj(W lower) so that column i holds row i of the Hermitian matrix
__global__ void herm_fill_kernel(float2* __restrict__ W, int P) {
  __shared__ float2 t[32][33];
  const int bi = blockIdx.y, bj = blockIdx.x;       // source tile (bi, bj), bi > bj, lower
  if (bi < bj) return;
  const int r = threadIdx.x, c0 = threadIdx.y;
  for (int c = c0; c < 32; c += blockDim.y) {
    const int gi = bi * 32 + r, gj = bj * 32 + c;
    t[r][c] = (gi < P && gj < P) ? W[(size_t)gi + (size_t)P * gj] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int c = c0; c < 32; c += blockDim.y) {
    // destination (bj*32 + r, bi*32 + c) = conj(source (bi*32 + c, bj*32 + r))
    const int gi = bj * 32 + r, gj = bi * 32 + c;
    if (gi < P && gj < P && gi < gj) {
      const float2 v = t[c][r];
      W[(size_t)gi + (size_t)P * gj] = make_float2(v.x, -v.y);
    }
  }
}

// y = -W x for the full Hermitian W (= A^-1 after the sweep): one warp per
// output i reads column i contiguously, y_i = -Σ_j conj(W_ji) x_j
__global__ void __launch_bounds__(256) herm_gemv_neg_kernel(const float2* __restrict__ W, int P,
                                                            const float2* __restrict__ x, float2* __restrict__ y) {
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= P) return;
  const float2* col = W + (size_t)P * i;
  float sx = 0.f, sy = 0.f;
  for (int j = lane; j < P; j += 32) {
    const float2 w = col[j], v = x[j];
    sx += w.x * v.x + w.y * v.y;
    sy += w.x * v.y - w.y * v.x;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, off);
    sy += __shfl_xor_sync(0xffffffffu, sy, off);
  }
  if (lane == 0) y[i] = make_float2(-sx, -sy);
}

}  // namespace

size_t sweep_ctl_bytes() { return sizeof(SweepCtl); }
size_t sweep_work_elems(int P) { return (size_t)(2 * ((P + CB - 1) / CB) + 1) * CB * CB; }

cudaError_t launch_spd_inverse(float2* W, int P, void* ctl, int* status, float2* work, cudaStream_t st) {
  static int grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_coop_kernel, 256, 0);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorCooperativeLaunchTooLarge;
    // two CTAs per SM where they fit: phase B has ~nblk^2/2 tiles per step, and
    // a second resident CTA halves the tiles per CTA (co-residency of every
    // CTA is guaranteed by the cooperative launch)
    grid = sms * (per >= 2 ? 2 : 1);
  }
  cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(SweepCtl), st);
  if (e != cudaSuccess) return e;
  const size_t tile = (size_t)CB * CB, nblk = (size_t)(P + CB - 1) / CB;
  float2* Cbuf = work;
  float2* Gbuf = work + nblk * tile;
  float2* pivbuf = work + 2 * nblk * tile;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SweepCtl* c = reinterpret_cast<SweepCtl*>(ctl);
  return cudaLaunchKernelEx(&cfg, sweep_coop_kernel, W, P, c, status, Cbuf, Gbuf, pivbuf);
}

cudaError_t launch_herm_gemv_neg(const float2* W, int P, const float2* x, float2* y, cudaStream_t st) {
  herm_gemv_neg_kernel<<<(P + 7) / 8, 256, 0, st>>>(W, P, x, y);
  return cudaGetLastError();
}

cudaError_t launch_spd_inverse_batch(const SweepJob* jobs, const int* cta_start, int np, int total_ctas,
                                     void* ctl_base, size_t ctl_bytes, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(ctl_base, 0, ctl_bytes, st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(total_ctas);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, sweep_batch_kernel, jobs, cta_start, np);
}

cudaError_t launch_herm_fill(float2* W, int P, cudaStream_t st) {
  const int nblk = (P + CB - 1) / CB;
  const dim3 tb(32, 8), tg((unsigned)nblk, (unsigned)nblk);
  herm_fill_kernel<<<tg, tb, 0, st>>>(W, P);
  return cudaGetLastError();
}
