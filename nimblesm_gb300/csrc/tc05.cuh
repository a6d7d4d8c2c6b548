// Blackwell 5th-generation tensor-core primitives (sm_100a / sm_103a) as
// inline PTX: tensor-memory allocation, single-thread MMA issue with
// shared-memory operand descriptors, completion through an mbarrier, and
// tensor-memory loads.  Used by the MLP closure's training and inference
// kernels.
//
// Operand layout used throughout: K-major, no swizzle.  A [rows x K] bf16
// operand is stored as 8x8 "core matrices" (8 rows, 8 K-elements = 16 bytes
// per row, 128 contiguous bytes each):
//   byte offset(r, k) = (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 (K-adjacent core matrices contiguous) and SBO = 16 * K
// bytes (one 8-row group holds all its K chunks).  One MMA consumes K = 16
// (two core matrices along K); the next K-step starts 2 * LBO bytes later.
//
// Every wait on an mbarrier is bounded: on timeout the caller gets `false`
// and must record an error and unwind (free its tensor memory) instead of
// waiting forever.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace nsm {
namespace tc {

constexpr uint32_t kLBO = 128;  // bytes between K-adjacent core matrices

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) in a K-major no-swizzle tile with K columns.
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K)
{
  return (uint32_t)((r >> 3) * (16 * K) + (k >> 3) * kLBO + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor (64 bits): start address >> 4 in bits
// 0-13, leading byte offset >> 4 in 16-29, stride byte offset >> 4 in 32-45,
// descriptor version 1 in 46-47, base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor for kind::f16 with BF16 A and B, FP32 accumulator,
// both operands K-major, shape M x N: D format (bits 4-5) = 1 (F32), A format
// (7-9) = 1 (BF16), B format (10-12) = 1 (BF16), N >> 3 in bits 17-22,
// M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- tensor memory ----
// Allocation by one full warp; the allocated base address is written to
// shared memory at `slot`.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Make this thread's generic-proxy shared-memory writes visible to the
// tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// Arrive on `mbar` when all MMAs issued so far by this thread complete.
__device__ __forceinline__ void mma_commit(uint64_t* mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
               : "memory");
}

// 16 consecutive 32-bit columns of this thread's lane (32x32b shape): warp w
// of the warpgroup reads lanes 32w..32w+31; `taddr` carries that lane base.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- mbarrier ----
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
// One test of the phase parity.  A thread whose phase is not complete is
// suspended in hardware until it completes or up to kSuspendNs (the
// instruction's time hint) have passed, instead of spinning through issue
// slots that the CTA's other warps need.
constexpr uint32_t kSuspendNs = 1000000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t phase)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_addr(mbar)), "r"(phase), "n"(kSuspendNs)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for the given phase parity: false once `limit_ns` of wall
// time (the GPU's global timer) have passed without the phase completing.
// The time is read only after a test failed, so a wait that completes at its
// first test costs one instruction.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t phase, uint64_t limit_ns = 1000000000ull)
{
  if (mbar_try_wait(mbar, phase)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(mbar, phase)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

}  // namespace tc
}  // namespace nsm
