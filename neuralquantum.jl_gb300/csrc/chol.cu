// Shifted SR solve, factorisation part: right-looking blocked Cholesky
// (A = L Lᴴ, lower, column-major, FP32 complex) in ONE persistent
// cooperative launch.  Each 32-column step is two phases separated by grid
// barriers:
//   A. every CTA factors the 32x32 diagonal block in registers of its warp 0
//      (pivots and rank-1 updates broadcast by shuffles); its 8 warps then
//      solve 32-row blocks of the panel below, X L_kkᴴ = A_ik, one row per
//      lane; CTA 0 writes the diagonal block back;
//   B. the trailing lower 32x32 tiles are updated, A_ij -= L_ik L_jkᴴ.
// The grid barrier is a generation counter with a bounded spin (1 s, sticky
// abort flag), so a stalled barrier ends the kernel with a status bit rather
// than a hang.  Reference: SRDirect.jl:79-81 (cholesky!(Hermitian(S))).
#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int CB = 32;

struct CholCtl {
  unsigned count;      // arrivals at the current barrier
  unsigned gen;        // barrier generation
  int abort;           // sticky abort flag
  int pad;
};

__device__ bool grid_barrier(CholCtl* ctl, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    volatile unsigned* vgen = &ctl->gen;
    const unsigned g = *vgen;
    __threadfence();
    if (atomicAdd(&ctl->count, 1u) == gridDim.x - 1) {
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

// Factor the 32x32 diagonal block held in shared memory (identity-padded
// beyond nb) in place: lane i keeps row i in registers; pivots and the column
// entries are broadcast by shuffles.  All indices are compile-time constants
// so the row stays in registers.
__device__ __forceinline__ void warp_potrf(float2 (*D)[CB + 1], bool* bad) {
  const int lane = threadIdx.x & 31;
  float2 a[CB];
#pragma unroll
  for (int k = 0; k < CB; ++k) a[k] = D[lane][k];
  bool b = false;
#pragma unroll
  for (int j = 0; j < CB; ++j) {
    float djj = __shfl_sync(0xffffffffu, a[j].x, j);
    if (!(djj > 0.f)) { b = true; djj = 1.f; }
    const float inv = rsqrtf(djj);
    if (lane == j) a[j] = make_float2(djj * inv, 0.f);
    if (lane > j) { a[j].x *= inv; a[j].y *= inv; }
#pragma unroll
    for (int k = 0; k < CB; ++k) {
      if (k > j) {
        const float lx = __shfl_sync(0xffffffffu, a[j].x, k);
        const float ly = __shfl_sync(0xffffffffu, a[j].y, k);
        if (lane >= k) {
          a[k].x -= a[j].x * lx + a[j].y * ly;
          a[k].y -= a[j].y * lx - a[j].x * ly;
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < CB; ++k) D[lane][k] = a[k];
  *bad = b;
}

__global__ void __launch_bounds__(256) chol_coop_kernel(float2* A, int P, CholCtl* ctl, int* status,
                                                        float2* __restrict__ Dinv) {
  __shared__ float2 Lk[CB][CB + 1];
  __shared__ float2 Di[CB][CB + 1];
  __shared__ float2 Li[CB][CB + 1];
  __shared__ float2 Lj[CB][CB + 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int nblk = (P + CB - 1) / CB;
  for (int kb = 0; kb < nblk; ++kb) {
    const int k0 = kb * CB, nb = min(CB, P - k0), t0 = k0 + nb, rem = P - t0;
    // ---- phase A: diagonal factor, its inverse, panel X = A_ik (L_kk^-1)ᴴ ----
    // (all loads of A are L2-coherent: other CTAs modified it before the barrier)
    const int nrb = (rem + CB - 1) / CB;
    const bool has_panel = blockIdx.x * nwarps < nrb;
    if (has_panel || blockIdx.x == 0) {
      for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
        const int i = e % CB, j = e / CB;
        Lk[i][j] = (i < nb && j < nb && j <= i) ? __ldcg(A + (size_t)(k0 + i) + (size_t)P * (k0 + j))
                                                : make_float2((i == j && i >= nb) ? 1.f : 0.f, 0.f);
      }
      __syncthreads();
      if (warp == 0) {
        bool bad = false;
        warp_potrf(Lk, &bad);
        if (bad && lane == 0 && blockIdx.x == 0) atomicOr(status, 1);
        __syncwarp();
        // lane c: column c of L_kk^-1 by forward substitution (identity-padded)
        const int c = lane;
        float2 x[CB];
#pragma unroll
        for (int i = 0; i < CB; ++i) {
          float2 v = make_float2(i == c ? 1.f : 0.f, 0.f);
#pragma unroll
          for (int p = 0; p < i; ++p) {
            const float2 l = Lk[i][p];
            v.x -= l.x * x[p].x - l.y * x[p].y;
            v.y -= l.x * x[p].y + l.y * x[p].x;
          }
          const float inv = 1.0f / Lk[i][i].x;
          x[i] = make_float2(v.x * inv, v.y * inv);
        }
#pragma unroll
        for (int i = 0; i < CB; ++i) Di[i][c] = x[i];
      }
      __syncthreads();
      for (int rb = blockIdx.x * nwarps + warp; rb < nrb; rb += gridDim.x * nwarps) {
        const int i = t0 + rb * CB + lane;
        if (i < P) {
          float2 a[CB];
#pragma unroll
          for (int j = 0; j < CB; ++j)
            a[j] = j < nb ? __ldcg(A + (size_t)i + (size_t)P * (k0 + j)) : make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < CB; ++c) {
            if (c < nb) {
              // X[i][c] = Σ_j a_j conj(Dinv[c][j])
              float sx = 0.f, sy = 0.f;
#pragma unroll
              for (int j = 0; j <= c; ++j) {
                const float2 d = Di[c][j];
                sx += a[j].x * d.x + a[j].y * d.y;
                sy += a[j].y * d.x - a[j].x * d.y;
              }
              A[(size_t)i + (size_t)P * (k0 + c)] = make_float2(sx, sy);
            }
          }
        }
      }
    }
    if (!grid_barrier(ctl, status)) return;
    // ---- phase B: trailing update of the lower tiles ----
    // (the diagonal block is written back now: every CTA has finished reading
    // the unfactored block in phase A)
    if (blockIdx.x == 0 && warp == 0 && lane < nb) {
#pragma unroll
      for (int j = 0; j < CB; ++j)
        if (j <= lane) A[(size_t)(k0 + lane) + (size_t)P * (k0 + j)] = Lk[lane][j];
    }
    if (blockIdx.x == 0) {
      float2* dst = Dinv + (size_t)kb * CB * CB;
      for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) dst[e] = Di[e / CB][e % CB];
    }
    const int ntt = nrb;
    const int ntiles = ntt * (ntt + 1) / 2;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      int ti, tj;
      {
        int c = 0, r = t;
        while (r >= ntt - c) { r -= ntt - c; ++c; }
        tj = c; ti = c + r;
      }
      const int r0 = t0 + ti * CB, c0 = t0 + tj * CB;
      __syncthreads();
      for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
        const int r = e % CB, p = e / CB;
        const bool in = p < nb;
        const int gi = r0 + r, gj = c0 + r;
        Li[r][p] = (in && gi < P) ? __ldcg(A + (size_t)gi + (size_t)P * (k0 + p)) : make_float2(0.f, 0.f);
        Lj[r][p] = (in && gj < P) ? __ldcg(A + (size_t)gj + (size_t)P * (k0 + p)) : make_float2(0.f, 0.f);
      }
      __syncthreads();
      const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;   // 8 column groups of 4
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int c = tc * 4 + q;
        const int gi = r0 + tr, gj = c0 + c;
        if (gi < P && gj < P && gi >= gj) {
          float sx = 0.f, sy = 0.f;
#pragma unroll
          for (int p = 0; p < CB; ++p) {
            const float2 u = Li[tr][p], w = Lj[c][p];    // u conj(w)
            sx += u.x * w.x + u.y * w.y;
            sy += u.y * w.x - u.x * w.y;
          }
          float2* a = A + (size_t)gi + (size_t)P * gj;
          float2 cur = __ldcg(a);
          cur.x -= sx;
          cur.y -= sy;
          *a = cur;
        }
      }
    }
    if (!grid_barrier(ctl, status)) return;
  }
}

// Single-CTA triangular solves with the factor, in place on rhs (P complex):
// L y = b then Lᴴ x = y.  The right-hand side lives in shared memory; each
// 32-row block is one matvec with the precomputed inverse diagonal block
// (Dinv_k for L, Dinv_kᴴ for Lᴴ) followed by a block-parallel update of the
// remaining rows; the update loads are issued before the block matvec so
// their latency overlaps it.
__global__ void __launch_bounds__(512) chol_solve_kernel(const float2* __restrict__ L,
                                                          const float2* __restrict__ LT,
                                                          const float2* __restrict__ Dinv, int P,
                                                          float2* __restrict__ rhs) {
  extern __shared__ float2 sb[];     // [P]
  __shared__ float2 D[CB][CB + 1];
  __shared__ float2 ys[CB];
  const int lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < P; i += blockDim.x) sb[i] = rhs[i];
  const int nblk = (P + CB - 1) / CB;
  const int maxrows = (P + blockDim.x - 1) / blockDim.x;   // rows per thread in an update
  // ---- forward ----
  for (int kb = 0; kb < nblk; ++kb) {
    const int k0 = kb * CB, nb = min(CB, P - k0);
    const float2* Dk = Dinv + (size_t)kb * CB * CB;
    for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) D[e / CB][e % CB] = Dk[e];
    __syncthreads();
    if (threadIdx.x < 32) {
      float2 y = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const float2 d = D[lane][j];
        const float2 r = j < nb ? sb[k0 + j] : make_float2(0.f, 0.f);
        y.x += d.x * r.x - d.y * r.y;
        y.y += d.x * r.y + d.y * r.x;
      }
      ys[lane] = lane < nb ? y : make_float2(0.f, 0.f);
      __syncwarp();
      if (lane < nb) sb[k0 + lane] = y;
    }
    __syncthreads();
    for (int q = 0; q < maxrows; ++q) {
      const int i = k0 + nb + threadIdx.x + q * blockDim.x;
      if (i < P) {
        float2 acc = sb[i];
#pragma unroll
        for (int j = 0; j < CB; ++j) {
          if (j < nb) {
            const float2 l = L[(size_t)i + (size_t)P * (k0 + j)], y = ys[j];
            acc.x -= l.x * y.x - l.y * y.y;
            acc.y -= l.x * y.y + l.y * y.x;
          }
        }
        sb[i] = acc;
      }
    }
    __syncthreads();
  }
  // ---- backward: Lᴴ x = y; the inverse of the diagonal block of Lᴴ is Dinv_kᴴ ----
  for (int kb = nblk - 1; kb >= 0; --kb) {
    const int k0 = kb * CB, nb = min(CB, P - k0);
    const float2* Dk = Dinv + (size_t)kb * CB * CB;
    for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) D[e / CB][e % CB] = Dk[e];
    __syncthreads();
    if (threadIdx.x < 32) {
      float2 x = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const float2 d = D[j][lane];      // conj(Dinv[j][lane])
        const float2 r = j < nb ? sb[k0 + j] : make_float2(0.f, 0.f);
        x.x += d.x * r.x + d.y * r.y;
        x.y += d.x * r.y - d.y * r.x;
      }
      ys[lane] = lane < nb ? x : make_float2(0.f, 0.f);
      __syncwarp();
      if (lane < nb) sb[k0 + lane] = x;
    }
    __syncthreads();
    for (int q = 0; q < maxrows; ++q) {
      const int i = threadIdx.x + q * blockDim.x;
      if (i < k0) {
        float2 acc = sb[i];
#pragma unroll
        for (int j = 0; j < CB; ++j) {
          if (j < nb) {
            const float2 l = LT[(size_t)i + (size_t)P * (k0 + j)], x = ys[j];
            acc.x -= l.x * x.x - l.y * x.y;
            acc.y -= l.x * x.y + l.y * x.x;
          }
        }
        sb[i] = acc;
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < P; i += blockDim.x) rhs[i] = sb[i];
}

}  // namespace

cudaError_t launch_chol_solve(const float2* L, const float2* LT, const float2* Dinv, int P, float2* rhs,
                              cudaStream_t st) {
  const size_t smem = (size_t)P * sizeof(float2);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(chol_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  chol_solve_kernel<<<1, 512, smem, st>>>(L, LT, Dinv, P, rhs);
  return cudaGetLastError();
}

size_t chol_ctl_bytes() { return sizeof(CholCtl); }

cudaError_t launch_chol_coop(float2* A, int P, void* ctl, int* status, float2* Dinv, cudaStream_t st) {
  static int grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, chol_coop_kernel, 256, 0);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorCooperativeLaunchTooLarge;
    grid = sms;     // one CTA per SM (co-residency guaranteed by the cooperative launch)
  }
  cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(CholCtl), st);
  if (e != cudaSuccess) return e;
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
  CholCtl* c = reinterpret_cast<CholCtl*>(ctl);
  return cudaLaunchKernelEx(&cfg, chol_coop_kernel, A, P, c, status, Dinv);
}
