// Inline-PTX building blocks for sm_103a: mbarriers with bounded waits, TMA
// (cp.async.bulk.tensor) loads, and the tcgen05 tensor-core instructions
// (TMEM alloc/dealloc, mma, commit, ld).
#pragma once
#include <cuda.h>
#include <stdint.h>

#include "nq_common.cuh"


NQ_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

NQ_D uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Barrier over the n CTAs that share (count, gen, abort), by tickets.  The
// counter only grows within a launch (it is zeroed before the launch), so the
// arrival with ticket t belongs to barrier t / n and the last arrival of
// barrier e publishes gen = e + 1.  Thread 0 arrives with an acquire-release
// add and waits with acquire loads (no separate fences), so the CTA's writes
// before the barrier are visible to every CTA after it; data written by other
// CTAs is read with L2 (.cg) loads.  The wait is bounded by limit_ns
// (%globaltimer, read every 256 polls or every poll under 0.1 ms): on timeout
// it sets NQ_DEVERR_TIMEOUT in *err and the abort flag, which ends the other
// waiters.  Returns false on abort.
NQ_D bool ticket_grid_barrier(unsigned* count, unsigned* gen, int* abort, unsigned n, int* err,
                              uint64_t limit_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    unsigned t;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(t) : "l"(count) : "memory");
    const unsigned target = t / n + 1;
    if (t % n == n - 1) {
      asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(gen), "r"(target) : "memory");
    } else {
      const uint64_t t0 = globaltimer_ns();
      unsigned it = 0;
      for (;;) {
        unsigned g;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(gen) : "memory");
        if ((int)(g - target) >= 0) break;
        if (*(volatile int*)abort) { s_ok = 0; break; }
        if (((++it & 255u) == 0 || limit_ns < 100000u) && globaltimer_ns() - t0 > limit_ns) {
          atomicOr(err, NQ_DEVERR_TIMEOUT);
          atomicExch(abort, 1);
          s_ok = 0;
          break;
        }
      }
    }
  }
  __syncthreads();
  return s_ok != 0;
}

NQ_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
NQ_D void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
NQ_D void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

NQ_D void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
NQ_D void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
NQ_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit_ns` of wall time, records the failure in
// *err (global) and returns false.  The polling loop and its %globaltimer
// check sit in one asm block: written as a C++ loop, the divergent loop made
// every tcgen05.mma issued by the same thread about 2.5x slower (measured on
// GB300, one wait per four 128x256x16 MMAs: 66 -> 165 ns per MMA).
NQ_D bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err, uint64_t limit_ns = kNqWaitNs) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " .reg .u64 t0, t1;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " @p bra WAIT_DONE;\n"
      " mov.u64 t0, %%globaltimer;\n"
      "WAIT_LOOP:\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " @p bra WAIT_DONE;\n"
      " mov.u64 t1, %%globaltimer;\n"
      " sub.u64 t1, t1, t0;\n"
      " setp.lt.u64 p, t1, %3;\n"
      " @p bra WAIT_LOOP;\n"
      " mov.u32 %0, 0;\n"
      " bra WAIT_END;\n"
      "WAIT_DONE:\n"
      " mov.u32 %0, 1;\n"
      "WAIT_END:\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "l"(limit_ns)
      : "memory");
  if (!ok && err) atomicOr(err, NQ_DEVERR_TIMEOUT);
  return ok != 0;
}

// 2-D TMA tile load into shared memory, completion signalled on `bar`.
NQ_D void tma_load_2d(void* smem_dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(smem_dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

// ---- tcgen05 ----------------------------------------------------------------
NQ_D void tmem_alloc(uint32_t* smem_dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
NQ_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
NQ_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
NQ_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, kind::tf32, single CTA.
NQ_D void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// D[tmem] (+)= A * B^T, kind::f16 (bf16 or fp16 operands, FP32 accumulate).
NQ_D void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on `bar` once all previously issued tcgen05.mma of this thread complete.
NQ_D void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns per warp.
NQ_D void tmem_ld_32x32b_x32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
// 32 lanes x 16 consecutive 32-bit columns per warp.
NQ_D void tmem_ld_32x32b_x16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
NQ_D void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor, K-major operand in the 128-byte swizzle
// layout written by TMA with CU_TENSOR_MAP_SWIZZLE_128B: rows of 128 bytes,
// 8-row atoms of 1024 bytes (stride byte offset), base 1024-byte aligned.
NQ_D uint64_t sdesc_k_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);      // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                        // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                        // swizzle: 128 B
  return d;
}

// Instruction descriptor: dense, D = FP32, A/B K-major, given formats.
// a/b format: kind::f16 -> 0 F16, 1 BF16; kind::tf32 -> 2 TF32.
NQ_HD constexpr uint32_t idesc_f32acc(uint32_t fmt, uint32_t M, uint32_t N) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}
