// tcgen05 (5th-generation tensor core) kernels for sm_103a.
//
// gram_tf32_kernel: the SR matrix accumulation G = X Xᵀ over the real rows
// (TF32 operands, optionally 3xTF32 hi/lo, or BF16 operands with
// tcgen05.mma.kind::f16 — the same 128-byte swizzled row layout holds 32 fp32
// or 64 bf16 samples per stage)
// X = [Re O_c; Im O_c] (2P x Ns, sample index contiguous), i.e. the
// O_c O_c† of SRDirect.jl:32 written as one real symmetric rank-Ns update.
//
// A work item is (k-split y, block (ti, J)): rows [128 ti, +128) x columns
// [256 J, +256) of G for every J whose block reaches the upper triangle.
// One tcgen05.mma of M = 128, N = 256 covers the whole block: the MMA issue
// rate, not the operand bytes, bounds this kernel, and an N = 256 instruction
// costs about as much as an N = 128 one.  Items are ordered y-major so that
// the CTAs running at the same time read the same sample range of X and share
// it through L2.  One persistent CTA per SM walks items q = blockIdx.x +
// j * gridDim.x; its TMA ring runs on across item boundaries.
// Warp 8 issues TMA into the ring (128-byte swizzle, 128 x 128-byte boxes:
// B = X rows [256 J, +256) as two boxes, then A = X rows [128 ti, +128); when
// the A rows lie inside B the A box is not loaded and the MMA reads them from
// B), warp 9 issues tcgen05.mma into one of two TMEM accumulators.  The tensor
// core accumulates in FP32 without round-to-nearest, so long K chains drift
// low: every SEG chunks the accumulator is handed to warps 0-7, which add it
// into round-to-nearest FP32 sums held in registers (warp w: TMEM lanes
// 32 (w mod 4).., columns 128 (w div 4)..) while the MMAs continue in the other
// accumulator.  At the end of an item the sums go to the item's partial block,
// column-major, one 128-byte store per warp and column.  Every mbarrier wait
// is bounded (1 s); a timeout sets a status bit, drains outstanding copies,
// frees TMEM and exits.
#include <cudaTypedefs.h>

#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int TM = 128;                      // block rows; TMA box rows
constexpr int NW = 256;                      // block columns (MMA N)
constexpr int KC = 32;                       // fp32 K elements per stage (128 B rows)
constexpr int TILE_BYTES = TM * KC * 4;      // 16 KiB per 128-row box
constexpr int SEG = 32;                      // chunks per TMEM accumulation segment
constexpr int BLOCK_ELEMS = TM * NW;
constexpr int NDRAIN = 8;                    // drain warps
constexpr int THREADS = (NDRAIN + 2) * 32;

__host__ __device__ __forceinline__ int first_block(int ti) { return (ti * TM) / NW; }

// number of (ti, J) blocks in rows < ti, with nj = ceil(rows / NW) column blocks
__host__ __device__ __forceinline__ int blocks_before(int ti, int nj) {
  int s = 0;
  for (int i = 0; i < ti; ++i) s += nj - first_block(i);
  return s;
}

__device__ __forceinline__ void block_coords(int p, int nj, int* ti, int* J) {
  int i = 0, rem = p;
  while (rem >= nj - first_block(i)) { rem -= nj - first_block(i); ++i; }
  *ti = i; *J = first_block(i) + rem;
}

// Geometry of the many-problem Gram: per problem 8 ints {row offset in the
// stacked X, rows, nt, nj, nblocks, first item, first reduction tile, 0},
// then the item starts [np + 1] and the tile starts [np + 1].
constexpr int GEOM_INTS = 8;

// Work item q -> k-split y, block (ti, J) and the first row of its problem in
// X.  Single problem: geom == nullptr.
__device__ __forceinline__ void resolve_item(int q, int nj, int nblocks, const int* __restrict__ geom, int np,
                                             int* y, int* ti, int* J, int* roff) {
  int local = q, nbl = nblocks, njj = nj;
  *roff = 0;
  if (geom) {
    const int* item_start = geom + GEOM_INTS * np;
    int lo = 0, hi = np - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(item_start + mid) <= q) lo = mid; else hi = mid - 1;
    }
    const int* gm = geom + GEOM_INTS * lo;
    *roff = __ldg(gm + 0);
    njj = __ldg(gm + 3);
    nbl = __ldg(gm + 4);
    local = q - __ldg(gm + 5);
  }
  *y = local / nbl;
  block_coords(local - *y * nbl, njj, ti, J);
}

// chunk range of k-split y: [y * per, min(nch, (y + 1) * per))
__device__ __forceinline__ int item_chunks(int y, int per, int nch) { return min(nch, (y + 1) * per) - y * per; }

// Operand kinds of the Gram kernel; everything that depends on the kind (ring
// depth, boxes per stage, MMA kind and count) is a compile-time constant, as
// are the stage indices: a runtime kind branch and a runtime modulo in the
// issuing thread's loop measurably slowed the MMA issue on GB300.
enum GramKind { GRAM_TF32 = 0, GRAM_TF32X3 = 1, GRAM_BF16 = 2 };

template <int KIND>
__global__ void __launch_bounds__(THREADS, 1)
gram_tf32_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap xlomap,
                 int nj, int nblocks, int nch, int per, int items, float* __restrict__ slots,
                 int* __restrict__ err, const int* __restrict__ geom, int np) {
  constexpr bool split3 = KIND == GRAM_TF32X3;
  constexpr bool bf16 = KIND == GRAM_BF16;
  constexpr int stages = split3 ? 2 : 4;
  extern __shared__ unsigned char smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr int nbox = split3 ? 6 : 3;      // [B0 B1 A] (+ [B0lo B1lo Alo])
  constexpr uint32_t stage_bytes = (uint32_t)nbox * TILE_BYTES;
  uint8_t* ring = base;
  uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)stages * stage_bytes);
  uint64_t* empty = full + stages;
  uint64_t* seg_full = empty + stages;     // [2]
  uint64_t* seg_empty = seg_full + 2;      // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(seg_empty + 2);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&seg_full[b], 1);
      mbar_init(&seg_empty[b], NDRAIN);
    }
    s_abort = 0;
    fence_mbar_init();
  }
  if (warp == NDRAIN + 1) tmem_alloc(tmem_slot, 2 * NW);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == NDRAIN) {
    if (lane == 0) {
      // ---- TMA producer ----
      int k = 0;                      // stage counter across items
      bool stop = false;
      for (int q = blockIdx.x; q < items && !stop; q += gridDim.x) {
        int y, ti, J, roff;
        resolve_item(q, nj, nblocks, geom, np, &y, &ti, &J, &roff);
        const bool a_in_b = first_block(ti) == J;
        const int n = item_chunks(y, per, nch);
        const uint32_t bytes = (uint32_t)TILE_BYTES * (a_in_b ? 2u : 3u) * (split3 ? 2u : 1u);
        for (int c = 0; c < n; ++c, ++k) {
          if (*(volatile int*)&s_abort) { stop = true; break; }
          const int s = k % stages;
          const uint32_t round = (uint32_t)(k / stages);
          if (k >= stages && !mbar_wait_bounded(&empty[s], (round - 1) & 1u, err)) {
            s_abort = 1;
            stop = true;
            break;
          }
          uint8_t* buf = ring + (size_t)s * stage_bytes;
          const int kx = (y * per + c) * (bf16 ? 2 * KC : KC);     // elements of 128-byte rows
          mbar_arrive_expect_tx(&full[s], bytes);
          tma_load_2d(buf, &xmap, kx, roff + J * NW, &full[s]);
          tma_load_2d(buf + TILE_BYTES, &xmap, kx, roff + J * NW + TM, &full[s]);
          if (!a_in_b) tma_load_2d(buf + 2 * TILE_BYTES, &xmap, kx, roff + ti * TM, &full[s]);
          if (split3) {
            uint8_t* lb = buf + 3 * TILE_BYTES;
            tma_load_2d(lb, &xlomap, kx, roff + J * NW, &full[s]);
            tma_load_2d(lb + TILE_BYTES, &xlomap, kx, roff + J * NW + TM, &full[s]);
            if (!a_in_b) tma_load_2d(lb + 2 * TILE_BYTES, &xlomap, kx, roff + ti * TM, &full[s]);
          }
        }
      }
      // drain: every issued copy has landed before the CTA may exit
      for (int c = max(0, k - stages); c < k; ++c)
        mbar_wait_bounded(&full[c % stages], (uint32_t)(c / stages) & 1u, err);
    }
    __syncwarp();
  } else if (warp == NDRAIN + 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      constexpr uint32_t idesc = idesc_f32acc(bf16 ? 1u : 2u, (uint32_t)TM, (uint32_t)NW);
      // descriptors of the stage buffers: the start-address field counts 16 bytes
      const uint64_t desc0 = sdesc_k_sw128(smem_u32(ring));
      constexpr uint64_t desc_stage = stage_bytes >> 4, desc_box = TILE_BYTES >> 4, desc_k = 32 >> 4;
      int k = 0, seg = 0;
      bool stop = false;
      for (int q = blockIdx.x; q < items && !stop; q += gridDim.x) {
        int y, ti, J, roff;
        resolve_item(q, nj, nblocks, geom, np, &y, &ti, &J, &roff);
        const bool a_in_b = first_block(ti) == J;
        const uint64_t a_off = a_in_b ? (uint64_t)((ti * TM - J * NW) / TM) * desc_box : 2u * desc_box;
        const int n = item_chunks(y, per, nch);
        for (int c = 0; c < n; ++c, ++k) {
          const int b = seg & 1;
          const bool first = (c % SEG) == 0;
          const bool last = (c % SEG) == SEG - 1 || c == n - 1;
          if (first && seg >= 2 && !mbar_wait_bounded(&seg_empty[b], (uint32_t)(seg / 2 - 1) & 1u, err)) {
            s_abort = 1;
            stop = true;
            break;
          }
          const int s = k % stages;
          if (!mbar_wait_bounded(&full[s], (uint32_t)(k / stages) & 1u, err)) {
            s_abort = 1;
            stop = true;
            break;
          }
          tc_fence_after();
          const uint64_t db = desc0 + (uint64_t)s * desc_stage;
          const uint64_t da = db + a_off;
          const uint32_t d = tmem + (uint32_t)(b * NW);
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {           // K = 32 bytes per instruction (16 bf16 / 8 tf32)
            const uint32_t acc = (first && kk == 0) ? 0u : 1u;
            if (bf16) {
              mma_f16(d, da + kk * desc_k, db + kk * desc_k, idesc, acc);
            } else {
              mma_tf32(d, da + kk * desc_k, db + kk * desc_k, idesc, acc);
              if (split3) {
                mma_tf32(d, da + kk * desc_k, db + 3 * desc_box + kk * desc_k, idesc, 1u);
                mma_tf32(d, da + 3 * desc_box + kk * desc_k, db + kk * desc_k, idesc, 1u);
              }
            }
          }
          mma_commit(&empty[s]);
          if (last) {
            mma_commit(&seg_full[b]);
            ++seg;
          }
        }
      }
      // on an abort the drain warps may stop before the last segment: wait
      // (bounded) for the MMAs already issued, tracked by the commit of the
      // last stage, so that no MMA still reads shared memory or writes TMEM
      // when the CTA frees them
      if (stop && k > 0) mbar_wait_bounded(&empty[(k - 1) % stages], (uint32_t)((k - 1) / stages) & 1u, err);
    }
    __syncwarp();
  } else {
    // ---- warps 0-7: drain TMEM segments into round-to-nearest sums in registers ----
    const int lq = warp & 3, hc = warp >> 2;
    const int row = lq * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(hc * TM);
    int seg = 0;
    bool stop = false;
    for (int q = blockIdx.x; q < items && !stop; q += gridDim.x) {
      int y, ti_, J_, roff_;
      resolve_item(q, nj, nblocks, geom, np, &y, &ti_, &J_, &roff_);
      const int nseg = (item_chunks(y, per, nch) + SEG - 1) / SEG;
      float acc[TM];
#pragma unroll
      for (int c = 0; c < TM; ++c) acc[c] = 0.f;
      for (int j = 0; j < nseg; ++j, ++seg) {
        const int b = seg & 1;
        if (!mbar_wait_bounded(&seg_full[b], (uint32_t)(seg / 2) & 1u, err)) {
          s_abort = 1;
          stop = true;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int cc = 0; cc < TM; cc += 16) {
          uint32_t r[16];
          tmem_ld_32x32b_x16(lane_base + (uint32_t)(b * NW + cc), r);
          tmem_ld_wait();
#pragma unroll
          for (int e = 0; e < 16; ++e) acc[cc + e] += __uint_as_float(r[e]);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&seg_empty[b]);
      }
      if (stop || *(volatile int*)&s_abort) break;
      // item's partial block, column-major: element (r, c) at c * TM + r
      float* dst = slots + (size_t)q * BLOCK_ELEMS + (size_t)(hc * TM) * TM + row;
#pragma unroll
      for (int c = 0; c < TM; ++c) dst[(size_t)c * TM] = acc[c];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == NDRAIN + 1) tmem_dealloc(tmem, 2 * NW);
}

// G (rows x rows, row-major, upper 128 x 128 tiles) = sum over k-splits of the
// column-major partial blocks; 32 x 32 sub-blocks transposed through shared
// memory so that both the partial reads and the G writes are coalesced.
// blockIdx.x: upper tile t = (ti, tj) in row-major order, blockIdx.y: sub-block.
NQ_D void slot_reduce_tile(const float* __restrict__ slots, int rows, int nt, int nj, int nblocks, int ks,
                           float* __restrict__ G, int tile) {
  __shared__ float buf[32][33];
  const int sr = (blockIdx.y >> 2) * 32, sc = (blockIdx.y & 3) * 32;
  int ti = 0, rem = tile;
  while (rem >= nt - ti) { rem -= nt - ti; ++ti; }
  const int tj = ti + rem;
  const int J = (tj * TM) / NW;
  const int p = blocks_before(ti, nj) + (J - first_block(ti));
  const size_t col0 = (size_t)(tj * TM - J * NW);
  for (int cl = threadIdx.y; cl < 32; cl += 8) {
    const size_t off = (col0 + sc + cl) * TM + sr + threadIdx.x;
    float s = 0.f;
    for (int z = 0; z < ks; ++z) s += slots[((size_t)z * nblocks + p) * BLOCK_ELEMS + off];
    buf[cl][threadIdx.x] = s;
  }
  __syncthreads();
  for (int rl = threadIdx.y; rl < 32; rl += 8) {
    const int gr = ti * TM + sr + rl, gc = tj * TM + sc + threadIdx.x;
    if (gr < rows && gc < rows) G[(size_t)gr * rows + gc] = buf[threadIdx.x][rl];
  }
}

__global__ void __launch_bounds__(256) gram_slot_reduce_kernel(const float* __restrict__ slots, int rows, int nt,
                                                               int nj, int nblocks, int ks, float* __restrict__ G) {
  slot_reduce_tile(slots, rows, nt, nj, nblocks, ks, G, blockIdx.x);
}

// many problems: problem p owns the reduction tiles [tile_start[p], tile_start[p+1])
// and the partial blocks from its first item on; its G goes to jobs[p].G
__global__ void __launch_bounds__(256) gram_slot_reduce_group_kernel(const float* __restrict__ slots,
                                                                     const int* __restrict__ geom, int np, int ks,
                                                                     const SrJob* __restrict__ jobs) {
  const int* tile_start = geom + GEOM_INTS * np + np + 1;
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(tile_start + mid) <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
  }
  const int* gm = geom + GEOM_INTS * lo;
  slot_reduce_tile(slots + (size_t)__ldg(gm + 5) * BLOCK_ELEMS, __ldg(gm + 1), __ldg(gm + 2), __ldg(gm + 3),
                   __ldg(gm + 4), ks, jobs[lo].G, blockIdx.x - __ldg(gm + 6));
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// row-major [rows][cols] matrix of fp32 (bf16 = 0) or bf16 elements, box = one
// 128-byte row segment (32 fp32 / 64 bf16) x 128 rows, SW128
bool encode_rowmajor(CUtensorMap* map, const void* ptr, int rows, int cols, int bf16) {
  auto fn = encode_fn();
  if (!fn) return false;
  const size_t esz = bf16 ? 2 : 4;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * esz};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esz), (cuuint32_t)TM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                  const_cast<void*>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

int gram_tc_supported() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  int major = 0, minor = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) return 0;
  return (major == 10 && minor == 3 && encode_fn() != nullptr) ? 1 : 0;
}

namespace {

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
  }
  return n;
}

// Split of the sample dimension and grid of the persistent Gram kernel.  Each
// CTA takes ceil(items / ncta) items in turn; the cost counts the stages of
// the busiest CTA plus, per k-split, the write and read of one more set of
// partial blocks (about nblocks / 6 stage times).
struct GramPlan {
  int nt, nj, nblocks, nch, ks, per, items, ncta;
};

GramPlan gram_plan(int rows, int Ns_pad, int bf16) {
  GramPlan p;
  p.nt = (rows + TM - 1) / TM;
  p.nj = (rows + NW - 1) / NW;
  p.nblocks = blocks_before(p.nt, p.nj);
  p.nch = Ns_pad / (bf16 ? 2 * KC : KC);
  const int nsm = sm_count();
  long best = -1;
  p.ks = 1;
  for (int ks = 1; ks <= 32 && ks <= p.nch; ++ks) {
    const int per = (p.nch + ks - 1) / ks;
    if ((p.nch + per - 1) / per != ks) continue;       // same split as a smaller ks
    if (ks > 1 && per < 16) break;
    const long items = (long)p.nblocks * ks;
    const long rounds = (items + nsm - 1) / nsm;
    const long cost = 6L * rounds * per + (long)ks * p.nblocks;
    if (best < 0 || cost < best) { best = cost; p.ks = ks; }
  }
  p.per = (p.nch + p.ks - 1) / p.ks;
  p.items = p.nblocks * p.ks;
  p.ncta = std::min(nsm, p.items);
  return p;
}

}  // namespace

size_t gram_tc_partial_elems(int rows, int Ns_pad, int bf16) {
  const GramPlan p = gram_plan(rows, Ns_pad, bf16);
  return (size_t)p.items * BLOCK_ELEMS;
}

int gram_tc_ksplit(int rows, int Ns_pad, int bf16) { return gram_plan(rows, Ns_pad, bf16).ks; }

cudaError_t launch_gram_tc(const void* X, const float* Xlo, int rows, int Ns_pad, int split3, float* G,
                           float* partial, int* err, cudaStream_t st, int bf16) {
  const int kc = bf16 ? 2 * KC : KC;
  if (Ns_pad % kc != 0 || ((uintptr_t)X & 15u) != 0) return cudaErrorInvalidValue;
  if (bf16 && split3) return cudaErrorInvalidValue;
  if (split3 && (!Xlo || ((uintptr_t)Xlo & 15u) != 0)) return cudaErrorInvalidValue;
  CUtensorMap xmap, xlomap;
  if (!encode_rowmajor(&xmap, X, rows, Ns_pad, bf16)) return cudaErrorInvalidValue;
  if (!encode_rowmajor(&xlomap, split3 ? (const void*)Xlo : X, rows, Ns_pad, bf16)) return cudaErrorInvalidValue;
  const GramPlan p = gram_plan(rows, Ns_pad, bf16);
  const int stages = split3 ? 2 : 4;
  const size_t smem = (size_t)stages * (split3 ? 6 : 3) * TILE_BYTES + 1024 + 256;
  auto kernel = split3 ? gram_tf32_kernel<GRAM_TF32X3> : bf16 ? gram_tf32_kernel<GRAM_BF16> : gram_tf32_kernel<GRAM_TF32>;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kernel<<<p.ncta, THREADS, smem, st>>>(xmap, xlomap, p.nj, p.nblocks, p.nch, p.per, p.items, partial, err,
                                         nullptr, 0);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int tiles = p.nt * (p.nt + 1) / 2;
  gram_slot_reduce_kernel<<<dim3((unsigned)tiles, 16), dim3(32, 8), 0, st>>>(partial, rows, p.nt, p.nj, p.nblocks,
                                                                              p.ks, G);
  return cudaGetLastError();
}

// ---- many problems: one launch over the upper blocks of every problem's Gram
GramGroupPlan gram_group_plan(const std::vector<int>& rows, int Ns_pad) {
  GramGroupPlan p;
  p.np = (int)rows.size();
  p.rows = rows;
  p.nch = Ns_pad / KC;
  int total_blocks = 0, off = 0;
  p.row_off.resize(p.np);
  p.nblocks.resize(p.np);
  for (int i = 0; i < p.np; ++i) {
    const int nt = (rows[i] + TM - 1) / TM, nj = (rows[i] + NW - 1) / NW;
    p.nblocks[i] = blocks_before(nt, nj);
    p.row_off[i] = off;
    off += rows[i];
    total_blocks += p.nblocks[i];
  }
  // k-split as for one problem: stages of the busiest CTA plus a charge per split
  const int nsm = sm_count();
  long best = -1;
  for (int ks = 1; ks <= 32 && ks <= p.nch; ++ks) {
    const int per = (p.nch + ks - 1) / ks;
    if ((p.nch + per - 1) / per != ks) continue;
    if (ks > 1 && per < 16) break;
    const long items = (long)total_blocks * ks;
    const long rounds = (items + nsm - 1) / nsm;
    const long cost = 6L * rounds * per + (long)ks * total_blocks;
    if (best < 0 || cost < best) { best = cost; p.ks = ks; }
  }
  p.per = (p.nch + p.ks - 1) / p.ks;
  p.item0.assign(p.np + 1, 0);
  p.tile0.assign(p.np + 1, 0);
  for (int i = 0; i < p.np; ++i) {
    const int nt = (rows[i] + TM - 1) / TM;
    p.item0[i + 1] = p.item0[i] + p.nblocks[i] * p.ks;
    p.tile0[i + 1] = p.tile0[i] + nt * (nt + 1) / 2;
  }
  p.items = p.item0[p.np];
  p.tiles = p.tile0[p.np];
  p.ncta = std::min(nsm, p.items);
  return p;
}

size_t gram_group_partial_elems(const GramGroupPlan& p) { return (size_t)p.items * BLOCK_ELEMS; }
size_t gram_group_geom_bytes(int np) { return sizeof(int) * ((size_t)GEOM_INTS * np + 2 * (np + 1)); }

cudaError_t gram_group_upload(const GramGroupPlan& p, void* geom_dev, cudaStream_t st) {
  std::vector<int> h((size_t)GEOM_INTS * p.np + 2 * (p.np + 1), 0);
  for (int i = 0; i < p.np; ++i) {
    int* g = h.data() + GEOM_INTS * i;
    g[0] = p.row_off[i];
    g[1] = p.rows[i];
    g[2] = (p.rows[i] + TM - 1) / TM;
    g[3] = (p.rows[i] + NW - 1) / NW;
    g[4] = p.nblocks[i];
    g[5] = p.item0[i];
    g[6] = p.tile0[i];
  }
  for (int i = 0; i <= p.np; ++i) {
    h[(size_t)GEOM_INTS * p.np + i] = p.item0[i];
    h[(size_t)GEOM_INTS * p.np + p.np + 1 + i] = p.tile0[i];
  }
  cudaError_t e = cudaMemcpyAsync(geom_dev, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

cudaError_t launch_gram_group(const float* X, const float* Xlo, int rows_total, int Ns_pad, int split3,
                              const GramGroupPlan& p, const void* geom_dev, const SrGroup& g, float* slots,
                              int* err, cudaStream_t st) {
  if (Ns_pad % KC != 0 || ((uintptr_t)X & 15u) != 0) return cudaErrorInvalidValue;
  if (split3 && (!Xlo || ((uintptr_t)Xlo & 15u) != 0)) return cudaErrorInvalidValue;
  CUtensorMap xmap, xlomap;
  if (!encode_rowmajor(&xmap, X, rows_total, Ns_pad, 0)) return cudaErrorInvalidValue;
  if (!encode_rowmajor(&xlomap, split3 ? (const void*)Xlo : (const void*)X, rows_total, Ns_pad, 0))
    return cudaErrorInvalidValue;
  const int stages = split3 ? 2 : 4;
  const size_t smem = (size_t)stages * (split3 ? 6 : 3) * TILE_BYTES + 1024 + 256;
  auto kernel = split3 ? gram_tf32_kernel<GRAM_TF32X3> : gram_tf32_kernel<GRAM_TF32>;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int* geom = static_cast<const int*>(geom_dev);
  kernel<<<p.ncta, THREADS, smem, st>>>(xmap, xlomap, 0, 1, p.nch, p.per, p.items, slots, err, geom, p.np);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  gram_slot_reduce_group_kernel<<<dim3((unsigned)p.tiles, 16), dim3(32, 8), 0, st>>>(slots, geom, p.np, p.ks, g.jobs);
  return cudaGetLastError();
}
