// tcgen05 (5th-generation tensor core) kernels for sm_103a.
//
// gram_tf32_kernel: the SR matrix accumulation G = X Xᵀ over the real rows
// (TF32 operands, optionally 3xTF32 hi/lo, or BF16 operands with
// tcgen05.mma.kind::f16 — the same 128-byte swizzled row layout holds 32 fp32
// or 64 bf16 samples per stage)
// X = [Re O_c; Im O_c] (2P x Ns, sample index contiguous), i.e. the
// O_c O_c† of SRDirect.jl:32 written as one real symmetric rank-Ns update.
// One CTA owns a 128 x 128 upper tile of G and a contiguous range of the
// sample (K) dimension.  Warp 4 issues TMA into a shared-memory ring
// (128-byte swizzle, one 128 x 32 fp32 box per operand), warp 5 issues
// tcgen05.mma.kind::tf32 into one of two TMEM accumulators.  The tensor core
// accumulates in FP32 without round-to-nearest, so long K chains drift low;
// every SEG chunks (1024 samples) the accumulator is handed to warps 0-3,
// which drain it into a round-to-nearest FP32 tile in shared memory while the
// MMAs continue in the other TMEM buffer.  Every mbarrier wait is bounded
// (1 s); a timeout sets a status bit, drains outstanding copies, frees TMEM
// and exits.
#include <cudaTypedefs.h>

#include "nq_kernels.cuh"
#include "tc_common.cuh"

namespace {

constexpr int TM = 128;                      // tile rows = tile cols
constexpr int KC = 32;                       // fp32 K elements per stage (128 B rows)
constexpr int TILE_BYTES = TM * KC * 4;      // 16 KiB per operand per stage
constexpr int SEG = 32;                      // chunks per TMEM accumulation segment
constexpr int ACC_LD = TM + 1;               // padded leading dimension of the smem tile
constexpr int ACC_BYTES = TM * ACC_LD * 4;

__device__ __forceinline__ void upper_tile(int t, int nt, int* ti, int* tj) {
  int i = 0, rem = t;
  while (rem >= nt - i) { rem -= nt - i; ++i; }
  *ti = i; *tj = i + rem;
}

__global__ void __launch_bounds__(192, 1)
gram_tf32_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap xlomap,
                 int split3, int bf16, int stages, int nt, int nchunks_total, int ksplit, int rp,
                 float* __restrict__ partial, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int nops = split3 ? 4 : 2;
  uint8_t* ring = base;
  float* acc = reinterpret_cast<float*>(base + (size_t)stages * nops * TILE_BYTES);   // [col][ACC_LD]
  uint64_t* full = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(acc) + ACC_BYTES);
  uint64_t* empty = full + stages;
  uint64_t* seg_full = empty + stages;     // [2]
  uint64_t* seg_empty = seg_full + 2;      // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(seg_empty + 2);
  __shared__ int s_abort;

  int ti, tj;
  upper_tile(blockIdx.x, nt, &ti, &tj);
  const bool diag = ti == tj;
  const int per = (nchunks_total + ksplit - 1) / ksplit;
  const int c_begin = blockIdx.y * per;
  const int nch = max(0, min(nchunks_total, c_begin + per) - c_begin);
  const int nseg = (nch + SEG - 1) / SEG;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&seg_full[b], 1);
      mbar_init(&seg_empty[b], 4);
    }
    s_abort = 0;
    fence_mbar_init();
  }
  for (int i = threadIdx.x; i < TM * ACC_LD; i += blockDim.x) acc[i] = 0.f;
  if (warp == 5) tmem_alloc(tmem_slot, 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 4) {
    if (lane == 0) {
      // ---- TMA producer ----
      int issued = 0;
      for (int c = 0; c < nch && !*(volatile int*)&s_abort; ++c) {
        const int s = c % stages;
        const uint32_t round = (uint32_t)(c / stages);
        if (c >= stages && !mbar_wait_bounded(&empty[s], (round - 1) & 1u, err)) { s_abort = 1; break; }
        uint8_t* buf = ring + (size_t)s * nops * TILE_BYTES;
        const int kx = (c_begin + c) * (bf16 ? 2 * KC : KC);     // elements of 128-byte rows
        const uint32_t per_op = (uint32_t)TILE_BYTES * (diag ? 1u : 2u);
        mbar_arrive_expect_tx(&full[s], per_op * (split3 ? 2u : 1u));
        tma_load_2d(buf, &xmap, kx, ti * TM, &full[s]);
        if (!diag) tma_load_2d(buf + TILE_BYTES, &xmap, kx, tj * TM, &full[s]);
        if (split3) {
          tma_load_2d(buf + 2 * TILE_BYTES, &xlomap, kx, ti * TM, &full[s]);
          if (!diag) tma_load_2d(buf + 3 * TILE_BYTES, &xlomap, kx, tj * TM, &full[s]);
        }
        issued = c + 1;
      }
      // drain: every issued copy has landed before the CTA may exit
      for (int c = max(0, issued - stages); c < issued; ++c)
        mbar_wait_bounded(&full[c % stages], (uint32_t)(c / stages) & 1u, err);
    }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {
      // ---- MMA issuer ----
      const uint32_t idesc = idesc_f32acc(bf16 ? 1u : 2u, 128u, 128u);
      for (int c = 0; c < nch; ++c) {
        const int seg = c / SEG, b = seg & 1;
        const bool first = (c % SEG) == 0;
        const bool last = (c % SEG) == SEG - 1 || c == nch - 1;
        if (first && seg >= 2 && !mbar_wait_bounded(&seg_empty[b], (uint32_t)(seg / 2 - 1) & 1u, err)) {
          s_abort = 1;
          break;
        }
        const int s = c % stages;
        if (!mbar_wait_bounded(&full[s], (uint32_t)(c / stages) & 1u, err)) { s_abort = 1; break; }
        tc_fence_after();
        uint8_t* buf = ring + (size_t)s * nops * TILE_BYTES;
        const uint32_t a_hi = smem_u32(buf);
        const uint32_t b_hi = smem_u32(buf + (diag ? 0 : TILE_BYTES));
        const uint32_t a_lo = smem_u32(buf + 2 * TILE_BYTES);
        const uint32_t b_lo = smem_u32(buf + (diag ? 2 : 3) * TILE_BYTES);
        const uint32_t d = tmem + (uint32_t)(b * TM);
        if (bf16) {
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {         // K = 16 bf16 (32 bytes) per instruction
            const uint32_t off = kk * 32;
            mma_f16(d, sdesc_k_sw128(a_hi + off), sdesc_k_sw128(b_hi + off), idesc, (first && kk == 0) ? 0u : 1u);
          }
        } else {
#pragma unroll
          for (int kk = 0; kk < KC / 8; ++kk) {    // K = 8 tf32 (32 bytes) per instruction
            const uint32_t off = kk * 32;
            mma_tf32(d, sdesc_k_sw128(a_hi + off), sdesc_k_sw128(b_hi + off), idesc, (first && kk == 0) ? 0u : 1u);
            if (split3) {
              mma_tf32(d, sdesc_k_sw128(a_hi + off), sdesc_k_sw128(b_lo + off), idesc, 1u);
              mma_tf32(d, sdesc_k_sw128(a_lo + off), sdesc_k_sw128(b_hi + off), idesc, 1u);
            }
          }
        }
        mma_commit(&empty[s]);
        if (last) mma_commit(&seg_full[b]);
      }
    }
    __syncwarp();
  } else {
    // ---- warps 0-3: drain TMEM segments into the round-to-nearest smem tile ----
    const int row = warp * 32 + lane;
    for (int seg = 0; seg < nseg; ++seg) {
      const int b = seg & 1;
      if (!mbar_wait_bounded(&seg_full[b], (uint32_t)(seg / 2) & 1u, err)) { s_abort = 1; break; }
      tc_fence_after();
#pragma unroll 1
      for (int cc = 0; cc < TM; cc += 32) {
        uint32_t r[32];
        tmem_ld_32x32b_x32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * TM + cc), r);
        tmem_ld_wait();
#pragma unroll
        for (int q = 0; q < 32; ++q) acc[(cc + q) * ACC_LD + row] += __uint_as_float(r[q]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&seg_empty[b]);
    }
  }
  __syncthreads();
  // ---- write the tile (zeros for an empty K range) ----
  if (!s_abort) {
    float* dst = partial + (size_t)blockIdx.y * rp * rp + (size_t)(ti * TM) * rp + tj * TM;
    for (int i = threadIdx.x; i < TM * TM; i += blockDim.x) {
      const int r = i / TM, c = i % TM;
      dst[(size_t)r * rp + c] = acc[c * ACC_LD + r];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 5) tmem_dealloc(tmem, 256);
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

int gram_tc_ksplit(int rows, int Ns_pad, int bf16) {
  const int nt = (rows + TM - 1) / TM;
  const int tiles = nt * (nt + 1) / 2;
  const int nchunks = Ns_pad / (bf16 ? 2 * KC : KC);
  // fill >= 2 waves of 152 SMs, keep >= 8 chunks per CTA
  int ks = 1;
  while (tiles * ks < 2 * 152 && nchunks / (ks * 2) >= 8) ks *= 2;
  return ks;
}

cudaError_t launch_gram_tc(const void* X, const float* Xlo, int rows, int Ns_pad, int split3, float* G,
                           float* partial, int ksplit, int* err, cudaStream_t st, int bf16) {
  const int kc = bf16 ? 2 * KC : KC;
  if (Ns_pad % kc != 0 || ((uintptr_t)X & 15u) != 0) return cudaErrorInvalidValue;
  if (bf16 && split3) return cudaErrorInvalidValue;
  if (split3 && (!Xlo || ((uintptr_t)Xlo & 15u) != 0)) return cudaErrorInvalidValue;
  CUtensorMap xmap, xlomap;
  if (!encode_rowmajor(&xmap, X, rows, Ns_pad, bf16)) return cudaErrorInvalidValue;
  if (!encode_rowmajor(&xlomap, split3 ? (const void*)Xlo : X, rows, Ns_pad, bf16)) return cudaErrorInvalidValue;
  const int nt = (rows + TM - 1) / TM;
  const int tiles = nt * (nt + 1) / 2;
  const int stages = split3 ? 2 : 4;
  const size_t smem = (size_t)stages * (split3 ? 4 : 2) * TILE_BYTES + ACC_BYTES + 1024 + 256;
  cudaError_t e = cudaFuncSetAttribute(gram_tf32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(tiles, ksplit);
  const int rp = nt * TM;
  gram_tf32_kernel<<<grid, 192, smem, st>>>(xmap, xlomap, split3, bf16, stages, nt, Ns_pad / kc, ksplit, rp,
                                            partial, err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_gram_reduce(partial, rows, rp, TM, ksplit, G, st);
}
