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
// W = -A^-1.  Each step is one phase between grid barriers: the rank-32
// update of step k runs beside the preparation of step k+1 (its pivot
// inverse, a 32x32 Gauss–Jordan held in registers, and its C and G), see
// sweep_group.  The grid barrier is a ticket counter (ticket_grid_barrier)
// with a bounded spin (1 s by default, sticky abort flag): a stalled barrier
// ends the kernel with a status bit.
#include <algorithm>

#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int CB = 32;

struct SweepCtl {
  unsigned count;      // arrivals since the launch (tickets)
  unsigned gen;        // barriers completed
  int abort;           // sticky abort flag
  int pad;
};

// Barrier over the `n` CTAs that share ctl (the whole grid, or one group).
__device__ bool group_barrier(SweepCtl* ctl, unsigned n, int* err, uint64_t limit_ns) {
  return ticket_grid_barrier(&ctl->count, &ctl->gen, &ctl->abort, n, err, limit_ns);
}

NQ_D float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

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

NQ_D void bar_sync_128(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

// In-place inverse of the Hermitian positive-definite 32x32 block T by
// Gauss–Jordan without pivoting, run by warps 0-3 only (128 threads, named
// barrier 1): lane = row, warp w holds columns 8w..8w+7 in registers.  Per
// pivot p the owner warp publishes the old column p (double-buffered), row p
// is taken by shuffles from lane p; the pivot loop is unrolled so every
// register index is static.  Same arithmetic per element as a plain
// Gauss–Jordan sweep; 1/d is the correctly rounded reciprocal.  Returns false
// if a pivot was not positive.
NQ_D bool hpd_inverse_32_w4(float2 (*T)[CB + 1], float2 (*colbuf)[CB]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float2 a[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) a[q] = T[lane][8 * w + q];
  bool ok = true;
#pragma unroll
  for (int p = 0; p < CB; ++p) {
    if (w == (p >> 3)) colbuf[p & 1][lane] = a[p & 7];
    bar_sync_128(1);
    const float2 f = colbuf[p & 1][lane];
    float d = colbuf[p & 1][p].x;
    if (!(d > 0.f)) { ok = false; d = 1.f; }
    const float inv = __frcp_rn(d);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int j = 8 * w + q;
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
  bar_sync_128(1);
#pragma unroll
  for (int q = 0; q < 8; ++q) T[lane][8 * w + q] = a[q];
  bar_sync_128(1);
  return ok;
}

// tile_mm<MODE> for 128 threads t = 0..127: element (t & 31, 8 (t >> 5) + q)
template <int MODE>
NQ_D void tile_mm128(const float2 (*U)[CB + 1], const float2 (*V)[CB + 1], int t, float2 out[8]) {
  const int r = t & 31, cg = (t >> 5) * 8;
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = make_float2(0.f, 0.f);
#pragma unroll 4
  for (int p = 0; p < CB; ++p) {
    const float2 u = U[r][p];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
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

// Element (r, c) of block (bi, bj) of the Hermitian matrix held as its stored
// lower triangle; diagonal entries of a diagonal block are made real, padding
// outside P is the identity on a diagonal block and zero elsewhere.
NQ_D float2 herm_block_elem(const float2* __restrict__ W, int P, int bi, int bj, int r, int c) {
  const int gi = bi * CB + r, gj = bj * CB + c;
  if (gi >= P || gj >= P) return make_float2(bi == bj && r == c ? 1.f : 0.f, 0.f);
  float2 v = gi >= gj ? __ldcg(W + (size_t)gi + (size_t)P * gj) : __ldcg(W + (size_t)gj + (size_t)P * gi);
  if (gi < gj) v.y = -v.y;
  if (gi == gj) v.y = 0.f;
  return v;
}

// The sweep of one matrix by the CTAs rank = 0..nranks-1 of its group.
//
// Each step k is one phase between grid barriers.  Besides the rank-32
// update of the tiles off rows/columns k and k+1 and the store of
// W_kk = -piv_k, the phase prepares step k+1 ("column units", one per block
// i != k+1): each of them forms the updated pivot tile
// W_{k+1,k+1} - C_{k+1} G_{k+1}ᴴ and inverts it (redundantly, identically),
// forms the updated stored tile of (i, k+1) the way the rank-32 update would,
// and from it G_i and C_i of step k+1, and writes the step-(k+1) value C_i
// (or C_iᴴ) into W.  C, G and the pivot are double-buffered by step parity.
// A bootstrap phase does the same for step 0 from the unmodified matrix.  The
// arithmetic of every stored value is that of the two-phase sweep; one grid
// barrier per step instead of two, and the serial 32-step pivot inverse runs
// beside the rank-32 update instead of before it.
NQ_D void sweep_group(float2* __restrict__ W, int P, SweepCtl* ctl, int* status, float2* __restrict__ work,
                      int rank, int nranks, uint64_t limit_ns) {
  __shared__ float2 Dt[CB][CB + 1];
  __shared__ float2 Ut[CB][CB + 1];
  __shared__ float2 Vt[CB][CB + 1];
  __shared__ float2 Xt[CB][CB + 1];
  __shared__ float2 Yt[CB][CB + 1];
  __shared__ float2 colbuf[2][CB];
  const int nblk = (P + CB - 1) / CB;
  const size_t tile = (size_t)CB * CB;
  // [C even | C odd | G even | G odd | piv even | piv odd]
  auto Cb = [&](int par) { return work + (size_t)par * nblk * tile; };
  auto Gb = [&](int par) { return work + (size_t)(2 + par) * nblk * tile; };
  auto Pb = [&](int par) { return work + (size_t)4 * nblk * tile + (size_t)par * tile; };
  const int tr = threadIdx.x & 31, cg = (threadIdx.x >> 5) * 4;

  for (int k = -1; k < nblk; ++k) {
    const int kn = k + 1;                               // pivot block prepared in this phase
    const bool prep = kn < nblk;
    const int ncol = prep ? max(nblk - 1, 1) : 0;       // column units (a bare pivot unit if nblk == 1)
    const int m = nblk - (prep ? 2 : 1);                // blocks left for the rank-32 update
    const int nreg = k >= 0 ? m * (m + 1) / 2 : 0;
    const int nlight = k >= 0 ? 1 + nreg : 0;           // pivot store of step k + rank-32 tiles
    const float2* Cc = k >= 0 ? Cb(k & 1) : nullptr;
    const float2* Gc = k >= 0 ? Gb(k & 1) : nullptr;
    const float2* pc = k >= 0 ? Pb(k & 1) : nullptr;
    float2* Cn = Cb(kn & 1);
    float2* Gn = Gb(kn & 1);
    float2* pn = Pb(kn & 1);
    // heavy units on ranks [0, ncol), light units on the other ranks; with too
    // few ranks everything is dealt round-robin
    const bool split = nranks > ncol;
    const int nunits = ncol + nlight;
    // a CTA with several column units in this phase forms and inverts the
    // pivot tile once: Dt keeps the inverse for its later units
    bool piv_ready = false;
    for (int u0 = split ? (rank < ncol ? rank : ncol + (rank - ncol)) : rank; u0 < nunits;
         u0 += split ? (rank < ncol ? nunits : nranks - ncol) : nranks) {
      const int u = u0;
      __syncthreads();
      if (u < ncol) {
        // ---------------- column unit: pivot of step kn, then block i ----------------
        // Warps 0-3 form and invert the pivot of step kn while warps 4-7 form
        // V = block (i, kn) after step k from the stored tile of (sa, sb).
        // The tile both need is loaded once: G_kn (Vt) when i > kn, C_kn (Ut)
        // when i < kn; the other operand of V's product goes to Yt.
        const int i = nblk == 1 ? 0 : (u < kn ? u : u + 1);
        const int sa = max(i, kn), sb = min(i, kn);
        const bool v_from_c = k >= 0 && i == k;          // stored (kn, k) after step k is C_kn
        const bool v_update = k >= 0 && nblk > 1 && !v_from_c;
        // every global load of the five tiles is issued before the first
        // shared-memory store, so the phase costs one L2 round trip
        float2 ld[5][CB * CB / 256];
        const float2 z2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < CB * CB / 256; ++q) {
          const int e = q * 256 + threadIdx.x, r = e & 31, c = e >> 5;
          ld[0][q] = piv_ready ? z2 : herm_block_elem(W, P, kn, kn, r, c);
          ld[1][q] = k >= 0 ? __ldcg(Cc + (size_t)kn * tile + e) : z2;
          ld[2][q] = k >= 0 ? __ldcg(Gc + (size_t)kn * tile + e) : z2;
          const int gi = sa * CB + r, gj = sb * CB + c;
          ld[3][q] = nblk <= 1 ? z2
                     : v_from_c ? __ldcg(Cc + (size_t)kn * tile + e)
                     : (gi < P && gj < P) ? __ldcg(W + (size_t)gi + (size_t)P * gj) : z2;
          ld[4][q] = (nblk > 1 && v_update) ? __ldcg(i > kn ? Cc + (size_t)sa * tile + e : Gc + (size_t)sb * tile + e)
                                             : z2;
        }
#pragma unroll
        for (int q = 0; q < CB * CB / 256; ++q) {
          const int e = q * 256 + threadIdx.x, r = e & 31, c = e >> 5;
          if (!piv_ready) Dt[r][c] = ld[0][q];
          if (k >= 0) {
            Ut[r][c] = ld[1][q];
            Vt[r][c] = ld[2][q];
          }
          if (nblk > 1) {
            Xt[r][c] = ld[3][q];
            if (v_update) Yt[r][c] = ld[4][q];
          }
        }
        __syncthreads();
        if (k >= 0 && !piv_ready) {
          // updated pivot tile W_kn,kn - C_kn G_knᴴ on the stored lower triangle
          // (the lower part of Dt holds the stored values; the diagonal is
          // real), then mirrored
          float2 o[4];
          tile_mm<1>(Ut, Vt, o);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int c = cg + q;
            if (kn * CB + tr < P && kn * CB + c < P && tr >= c)
              Dt[tr][c] = make_float2(Dt[tr][c].x - o[q].x, tr == c ? 0.f : Dt[tr][c].y - o[q].y);
          }
          __syncthreads();
          for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
            const int r = e & 31, c = e >> 5;
            if (r < c && kn * CB + c < P) Dt[r][c] = make_float2(Dt[c][r].x, -Dt[c][r].y);
          }
          __syncthreads();
        }
        bool ok = true;
        if (piv_ready) {
          if (v_update) {
            // the pivot is inverted already: V on all 8 warps
            float2 o[4];
            tile_mm<1>(i > kn ? Yt : Ut, i > kn ? Vt : Yt, o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int c = cg + q;
              if (sa * CB + tr < P && sb * CB + c < P) {
                Xt[tr][c].x -= o[q].x;
                Xt[tr][c].y -= o[q].y;
              }
            }
          }
        } else if (threadIdx.x < 128) {
          ok = hpd_inverse_32_w4(Dt, colbuf);
        } else if (v_update) {
          // V = stored (sa, sb) - C_sa G_sbᴴ (the rank-32 update of that tile)
          float2 o[8];
          tile_mm128<1>(i > kn ? Yt : Ut, i > kn ? Vt : Yt, threadIdx.x - 128, o);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int r = threadIdx.x & 31, c = ((threadIdx.x - 128) >> 5) * 8 + q;
            if (sa * CB + r < P && sb * CB + c < P) {
              Xt[r][c].x -= o[q].x;
              Xt[r][c].y -= o[q].y;
            }
          }
        }
        __syncthreads();
        piv_ready = true;
        if (u == 0) {
          if (!ok && threadIdx.x == 0) atomicOr(status, 1);
          for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) pn[e] = Dt[e & 31][e >> 5];
        }
        if (nblk == 1) continue;
        // G_i = V (column-major), V into Ut for the product
        for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
          const int r = e & 31, c = e >> 5;
          float2 v = make_float2(0.f, 0.f);
          if (i * CB + r < P && kn * CB + c < P) {
            if (i > kn) v = Xt[r][c];
            else v = make_float2(Xt[c][r].x, -Xt[c][r].y);
          }
          Ut[r][c] = v;
          Gn[(size_t)i * tile + e] = v;
        }
        __syncthreads();
        float2 o[4];
        tile_mm<0>(Ut, Dt, o);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int c = cg + q;
          Cn[(size_t)i * tile + c * CB + tr] = o[q];
          // step-kn value of W on row/column kn: W_{i,kn} = C_i (i > kn), W_{kn,i} = C_iᴴ (i < kn)
          if (i > kn) {
            const int gi = i * CB + tr, gj = kn * CB + c;
            if (gi < P && gj < P) W[(size_t)gi + (size_t)P * gj] = o[q];
          } else {
            const int gi = kn * CB + c, gj = i * CB + tr;
            if (gi < P && gj < P) W[(size_t)gi + (size_t)P * gj] = make_float2(o[q].x, -o[q].y);
          }
        }
      } else if (u == ncol) {
        // ---------------- W_kk = -piv_k ----------------
        for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
          const int r = e & 31, c = e >> 5, gi = k * CB + r, gj = k * CB + c;
          if (gi < P && gj < P && gi >= gj) {
            const float2 v = __ldcg(pc + e);
            W[(size_t)gi + (size_t)P * gj] = make_float2(-v.x, -v.y);
          }
        }
      } else {
        // ---------------- rank-32 update of a tile off rows/columns k, kn ----------------
        int c0 = 0, rr = u - ncol - 1;
        while (rr >= m - c0) { rr -= m - c0; ++c0; }
        int ti = c0 + rr, tj = c0;
        ti += ti >= k ? (prep ? 2 : 1) : 0;
        tj += tj >= k ? (prep ? 2 : 1) : 0;
        for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
          const int r = e & 31, c = e >> 5;
          Ut[r][c] = __ldcg(Cc + (size_t)ti * tile + e);
          Vt[r][c] = __ldcg(Gc + (size_t)tj * tile + e);
        }
        __syncthreads();
        float2 o[4];
        tile_mm<1>(Ut, Vt, o);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int gi = ti * CB + tr, gj = tj * CB + cg + q;
          if (gi < P && gj < P && gi >= gj) {
            float2* a = W + (size_t)gi + (size_t)P * gj;
            float2 cur = __ldcg(a);
            cur.x -= o[q].x;
            cur.y -= o[q].y;
            *a = cur;
          }
        }
      }
    }
    if (k + 1 < nblk && !group_barrier(ctl, (unsigned)nranks, status, limit_ns)) return;
  }
}

__global__ void __launch_bounds__(256, 2) sweep_coop_kernel(float2* __restrict__ W, int P, SweepCtl* ctl,
                                                         int* status, float2* __restrict__ work, uint64_t limit_ns) {
  sweep_group(W, P, ctl, status, work, blockIdx.x, gridDim.x, limit_ns);
}

// Many matrices in one cooperative launch: matrix p is swept by CTAs
// [cta_start[p], cta_start[p+1]) with its own barrier block.
__global__ void __launch_bounds__(256, 2) sweep_batch_kernel(const SweepJob* __restrict__ jobs,
                                                          const int* __restrict__ cta_start, int np) {
  int lo = 0, hi = np - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(cta_start + mid) <= b) lo = mid; else hi = mid - 1;
  }
  const SweepJob& j = jobs[lo];
  const int r0 = __ldg(cta_start + lo), n = __ldg(cta_start + lo + 1) - r0;
  sweep_group(j.W, j.P, reinterpret_cast<SweepCtl*>(j.ctl), j.status, j.work, b - r0, n, kNqWaitNs);
}

// W upper = conj(W lower) so that column i holds row i of the Hermitian matrix
NQ_D void herm_fill_tile(float2* __restrict__ W, int P, int bi, int bj) {
  __shared__ float2 t[32][33];                      // source tile (bi, bj), bi > bj, lower
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

__global__ void herm_fill_kernel(float2* __restrict__ W, int P) { herm_fill_tile(W, P, blockIdx.y, blockIdx.x); }

__global__ void herm_fill_group_kernel(SrGroup g) {
  const int p = group_of(blockIdx.x, g.fill_blk, g.np);
  const SrJob& j = g.jobs[p];
  const int nb = (j.P + 31) / 32, local = blockIdx.x - __ldg(g.fill_blk + p);
  herm_fill_tile(j.W, j.P, local / nb, local % nb);
}

// y = -W x for the full Hermitian W (= A^-1 after the sweep): one warp per
// output i reads column i contiguously, y_i = -Σ_j conj(W_ji) x_j
__global__ void __launch_bounds__(256) herm_gemv_neg_kernel(const float2* __restrict__ W, int P,
                                                            const float2* __restrict__ x, float2* __restrict__ y) {
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= P) return;
  const float2* col = W + (size_t)P * i;
  float sx = 0.f, sy = 0.f;
#pragma unroll 8
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

// FP64-residual refinement of the shifted solve in one cooperative launch
// (one CTA per SM).  rf = F, then pass it = 0, 1, ...:
//   y = A⁻¹ rf (Hermitian GEMV with W = -A⁻¹ in FP32, one warp per row),
//   x = y (it = 0) or x + y (the same warp adds its row into x, in FP64),
//   grid barrier,
//   r = F - A x in FP64 from the FP64 S and the shift (one warp per row;
//   rf = FP32 copy of r),
// until the correction, or the error it leaves, is below tol |x|, or after
// max_corr corrections; a grid barrier separates the passes.  Every CTA sums
// the per-CTA |y|² and |x|² partials of the pass in the same fixed order, so
// all CTAs take the same decision.  Each correction shrinks the error by the
// FP32 inverse's error ‖I - A⁻¹₃₂ A‖, so x converges to the FP64 solution of
// the shifted system (limited by the FP64 residual, about cond(A) 1e-16).
// info = [corrections, relative error bound of the last one].  Each CTA
// copies the vector of a GEMV (rf, then x) into shared memory once per pass
// when P fits (refine_stage_bytes), instead of every warp reading it from L2.
// A non-finite x sets NQ_DEVERR_NONFINITE in the status word.
// The refinement of one matrix on the CTAs rank = 0..nranks-1 that share ctl.
NQ_D void refine_group_body(const float2* __restrict__ W, const double* __restrict__ S, int P,
                            const double* __restrict__ F, int kind, double eps, double lam, int real_params,
                            int max_corr, double tol, double* x, double* r, float2* rf, double* norms, double* info,
                            SweepCtl* ctl, int* status, uint64_t limit_ns, int rank, int nranks) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  // warps numbered across CTAs first, so the rows of both GEMVs spread over
  // every CTA (and SM) when there are fewer rows than warps
  const int gw = wib * nranks + rank, nw = nranks * (blockDim.x >> 5);
  __shared__ double s_red[2][8];
  extern __shared__ __align__(16) unsigned char s_vec[];
  unsigned dyn_smem;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn_smem));
  const bool stage = (size_t)16 * P <= dyn_smem;
  float2* const s_rf = reinterpret_cast<float2*>(s_vec);
  double2* const s_x = reinterpret_cast<double2*>(s_vec);
  for (int i = rank * blockDim.x + threadIdx.x; i < P; i += nranks * blockDim.x)
    rf[i] = make_float2((float)F[2 * i], real_params ? 0.f : (float)F[2 * i + 1]);
  if (!group_barrier(ctl, (unsigned)nranks, status, limit_ns)) return;
  double ty_prev = 0.0;
  for (int it = 0;; ++it) {
    double yy = 0.0, xx = 0.0;
    bool finite = true;
    if (stage) {
      for (int j = threadIdx.x; j < P; j += blockDim.x) s_rf[j] = __ldcg(rf + j);
      __syncthreads();
    }
    for (int i = gw; i < P; i += nw) {
      const float2* col = W + (size_t)P * i;
      float sx = 0.f, sy = 0.f;
      if (stage && !(P & 1)) {
        // two elements per 16-byte load (the column starts 16-byte aligned
        // when P is even): all of a column's loads are in flight at once
        const float4* col4 = reinterpret_cast<const float4*>(col);
#pragma unroll 16
        for (int j2 = lane; 2 * j2 < P; j2 += 32) {
          const float4 w = __ldcg(col4 + j2);
          const float2 v0 = s_rf[2 * j2], v1 = s_rf[2 * j2 + 1];
          sx += w.x * v0.x + w.y * v0.y;
          sy += w.x * v0.y - w.y * v0.x;
          sx += w.z * v1.x + w.w * v1.y;
          sy += w.z * v1.y - w.w * v1.x;
        }
      } else {
#pragma unroll 8
        for (int j = lane; j < P; j += 32) {
          const float2 w = __ldcg(col + j), v = stage ? s_rf[j] : __ldcg(rf + j);
          sx += w.x * v.x + w.y * v.y;
          sy += w.x * v.y - w.y * v.x;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
      }
      if (lane == 0) {
        const double yx = -(double)sx, yyv = -(double)sy;
        double nx = yx, ny = yyv;
        if (it > 0) {
          nx += x[2 * i];
          ny += x[2 * i + 1];
        }
        x[2 * i] = nx;
        x[2 * i + 1] = ny;
        yy += yx * yx + yyv * yyv;
        xx += nx * nx + ny * ny;
        finite = finite && isfinite(nx) && isfinite(ny);
      }
    }
    // the CTA's |y|² and |x|² partials, its warps summed in a fixed order
    if (lane == 0) {
      s_red[0][wib] = yy;
      s_red[1][wib] = xx;
      if (!finite) atomicOr(status, NQ_DEVERR_NONFINITE);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double cy = 0.0, cx = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        cy += s_red[0][w];
        cx += s_red[1][w];
      }
      norms[2 * rank] = cy;
      norms[2 * rank + 1] = cx;
    }
    if (!group_barrier(ctl, (unsigned)nranks, status, limit_ns)) return;
    // |y|² and |x|² of this pass, summed by every CTA in the same order
    double ty = 0.0, tx = 0.0;
    for (int w = threadIdx.x; w < nranks; w += blockDim.x) {
      ty += __ldcg(norms + 2 * w);
      tx += __ldcg(norms + 2 * w + 1);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      ty += __shfl_xor_sync(0xffffffffu, ty, off);
      tx += __shfl_xor_sync(0xffffffffu, tx, off);
    }
    if (lane == 0) {
      s_red[0][wib] = ty;
      s_red[1][wib] = tx;
    }
    __syncthreads();
    ty = 0.0;
    tx = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      ty += s_red[0][w];
      tx += s_red[1][w];
    }
    // Stop when the correction just applied, or the error it leaves, is below
    // tol |x|.  The iteration contracts by ρ ≈ |Δx_k| / |Δx_{k-1}|, so the
    // error after Δx_k is about ρ |Δx_k| = |Δx_k|² / |Δx_{k-1}| (trusted
    // when ρ < 1/2).  The residual of the final x is not formed.
    const bool small = it > 0 && ty <= tol * tol * tx;
    const bool contracting = it > 1 && ty < 0.25 * ty_prev;
    const bool est = contracting && ty * ty <= tol * tol * tx * ty_prev;
    const bool last = small || est || it >= max_corr || !(tx == tx);
    if (last && rank == 0 && threadIdx.x == 0 && info) {
      info[0] = (double)it;
      // the smaller of |Δx_k| / |x| and the estimated error after it
      double rel = tx > 0.0 ? sqrt(ty / tx) : 0.0;
      if (contracting && tx > 0.0 && ty_prev > 0.0) rel = fmin(rel, ty / sqrt(tx * ty_prev));
      info[1] = rel;
    }
    ty_prev = ty;
    if (last) break;
    if (stage) {
      for (int l = threadIdx.x; l < P; l += blockDim.x) s_x[l] = make_double2(__ldcg(x + 2 * l), __ldcg(x + 2 * l + 1));
      __syncthreads();
    }
    for (int k = gw; k < P; k += nw) {
      // (S x)_k = Σ_l conj(S[l][k]) x_l (Hermitian; column k contiguous)
      const double2* col = reinterpret_cast<const double2*>(S + 2 * (size_t)P * k);
      // four independent FP64 accumulators per lane
      double sx0 = 0.0, sy0 = 0.0, sx1 = 0.0, sy1 = 0.0;
#pragma unroll 4
      for (int l = lane; l < P; l += 64) {
        const int l1 = l + 32;
        const double2 a = __ldg(col + l);
        const double2 b = l1 < P ? __ldg(col + l1) : make_double2(0.0, 0.0);
        const double ar = a.x, ai = l == k ? 0.0 : -a.y;
        const double br = b.x, bi = l1 == k ? 0.0 : -b.y;
        const double2 xa = stage ? s_x[l] : make_double2(__ldcg(x + 2 * l), __ldcg(x + 2 * l + 1));
        const double2 xb = l1 >= P ? make_double2(0.0, 0.0)
                           : stage ? s_x[l1] : make_double2(__ldcg(x + 2 * l1), __ldcg(x + 2 * l1 + 1));
        sx0 += ar * xa.x - ai * xa.y;
        sy0 += ar * xa.y + ai * xa.x;
        sx1 += br * xb.x - bi * xb.y;
        sy1 += br * xb.y + bi * xb.x;
      }
      double sx = sx0 + sx1, sy = sy0 + sy1;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
      }
      if (lane == 0) {
        const double dsh = sr_diag_shift(S, P, k, kind, eps, lam);
        sx += dsh * __ldcg(x + 2 * k);
        sy += dsh * __ldcg(x + 2 * k + 1);
        const double rx = F[2 * k] - sx, ry = (real_params ? 0.0 : F[2 * k + 1]) - sy;
        r[2 * k] = rx;
        r[2 * k + 1] = ry;
        rf[k] = make_float2((float)rx, (float)ry);
      }
    }
    if (!group_barrier(ctl, (unsigned)nranks, status, limit_ns)) return;
  }
}

__global__ void __launch_bounds__(256) refine_coop_kernel(const float2* __restrict__ W, const double* __restrict__ S,
                                                          int P, const double* __restrict__ F, int kind, double eps,
                                                          double lam, int real_params, int max_corr, double tol,
                                                          double* x, double* r, float2* rf, double* norms,
                                                          double* info, SweepCtl* ctl, int* status,
                                                          uint64_t limit_ns) {
  refine_group_body(W, S, P, F, kind, eps, lam, real_params, max_corr, tol, x, r, rf, norms, info, ctl, status,
                    limit_ns, blockIdx.x, gridDim.x);
}

// every problem of a grouped step: problem p on CTAs [cta_start[p], cta_start[p+1])
// with barrier block p (64 bytes) of ctl_base; sr_shift (eps), complex parameters
__global__ void __launch_bounds__(256) refine_group_kernel(SrGroup g, const int* __restrict__ cta_start,
                                                           char* ctl_base, double eps, int max_corr) {
  const int p = group_of(blockIdx.x, cta_start, g.np);
  const SrJob& j = g.jobs[p];
  const int r0 = __ldg(cta_start + p), n = __ldg(cta_start + p + 1) - r0;
  refine_group_body(j.W, j.S, j.P, j.fb.force, 0, eps, 0.0, 0, max_corr, kRefineTol, j.x, j.r, j.rf, j.norms,
                    nullptr, reinterpret_cast<SweepCtl*>(ctl_base + (size_t)p * 64), j.status, kNqWaitNs,
                    blockIdx.x - r0, n);
}

}  // namespace

size_t sweep_ctl_bytes() { return sizeof(SweepCtl); }
// C and G of every block and the pivot inverse, each twice (step parity)
size_t sweep_work_elems(int P) { return (size_t)(4 * ((P + CB - 1) / CB) + 2) * CB * CB; }

cudaError_t launch_spd_inverse(float2* W, int P, void* ctl, int* status, float2* work, cudaStream_t st,
                               uint64_t wait_ns) {
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
    // one CTA per SM: the step time is the column units' (pivot inverse and
    // tile products), which run 20-25% faster without a second CTA on the SM
    // than the rank-32 update gains from one (measured: 0.46 vs 0.57 ms for
    // P = 860)
    grid = sms;
  }
  cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(SweepCtl), st);
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
  SweepCtl* c = reinterpret_cast<SweepCtl*>(ctl);
  return cudaLaunchKernelEx(&cfg, sweep_coop_kernel, W, P, c, status, work, wait_ns);
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

cudaError_t launch_refine_coop(const float2* W, const double* S, int P, const double* F, int kind, double eps,
                               double lam, bool real_params, int max_corr, double tol, double* x, double* r,
                               float2* rf, double* norms, double* info, void* ctl, int* status, cudaStream_t st,
                               uint64_t wait_ns) {
  static int grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, refine_coop_kernel, 256, 0);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorCooperativeLaunchTooLarge;
    grid = std::min(sms, kRefineMaxCtas);
  }
  cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(SweepCtl), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = refine_stage_bytes(P);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, refine_coop_kernel, W, S, P, F, kind, eps, lam, real_params ? 1 : 0, max_corr, tol,
                            x, r, rf, norms, info, reinterpret_cast<SweepCtl*>(ctl), status, wait_ns);
}

cudaError_t launch_fill_group(const SrGroup& g, cudaStream_t st) {
  herm_fill_group_kernel<<<g.fill_blocks, dim3(32, 8), 0, st>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_refine_group(const SrGroup& g, const int* cta_start, int total_ctas, void* ctl_base, double eps,
                                int max_corr, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(ctl_base, 0, (size_t)g.np * 64, st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(total_ctas);
  cfg.blockDim = dim3(256);
  // up to 40 KiB: the problems whose vector fits stage it
  cfg.dynamicSmemBytes = std::min((size_t)16 * g.P_max, kRefineStageMax);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, refine_group_kernel, g, cta_start, reinterpret_cast<char*>(ctl_base), eps,
                            max_corr);
}

// CTAs per SM that the many-problem inversion and refinement can keep
// co-resident (both run as cooperative launches over the same CTA split);
// at most two: the grouped step is throughput-bound, unlike the single
// problem, whose sweep runs fastest at one CTA per SM
int batch_solve_ctas_per_sm() {
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, sweep_batch_kernel, 256, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, refine_group_kernel, 256, 0) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return std::max(1, std::min(2, std::min(a, b)));
}
