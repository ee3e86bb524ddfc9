// tc_ptx.cuh -- inline-PTX building blocks of the tcgen05 kernels (logreg_tc.cu, horseshoe_tc.cu):
// mbarriers with bounded waits (single thread and whole warp), TMA 2-D tile loads and L2
// prefetches, shared-memory matrix descriptors, the kind::f16 instruction descriptor,
// warp-issued tcgen05.mma / commit (A from shared memory or from TMEM), TMEM loads and stores,
// and the approximate special functions of the logistic epilogue.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace gbn {
namespace tc {

constexpr uint32_t WAIT_LIMIT = 1u << 22;  // polls of an mbarrier before a wait gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void bar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint32_t a) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(a) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(a),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool bar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false on timeout or when another role already aborted
__device__ __forceinline__ bool bar_wait(uint32_t a, uint32_t parity, volatile int* abort_flag, int* err) {
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
    if (bar_try(a, parity)) return true;
    if (*abort_flag) return false;
  }
  *abort_flag = 1;
  atomicExch(err, 4);
  return false;
}
// non-blocking probe of a phase (mbarrier.test_wait never suspends the thread)
__device__ __forceinline__ bool bar_test(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait of a whole converged warp for up to three phases at once (each only when its
// use flag is set): the probes are issued back to back, so their latencies overlap
__device__ __forceinline__ bool bar_wait3_warp(uint32_t a, uint32_t pa, bool use_a, uint32_t b, uint32_t pb,
                                               bool use_b, uint32_t c, uint32_t pc, bool use_c,
                                               volatile int* abort_flag, int* err) {
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
    const bool da = !use_a || bar_test(a, pa);
    const bool db = !use_b || bar_test(b, pb);
    const bool dc = !use_c || bar_test(c, pc);
    if (__all_sync(0xffffffffu, da && db && dc)) return true;
    if (__any_sync(0xffffffffu, *abort_flag != 0)) return false;
    // not all complete: suspend on the first pending phase instead of spinning (a spinning
    // warp takes issue slots from the warps it shares a scheduler with)
    if (!da) bar_try(a, pa);
    else if (!db) bar_try(b, pb);
    else bar_try(c, pc);
  }
  if ((threadIdx.x & 31) == 0) {
    *abort_flag = 1;
    atomicExch(err, 4);
  }
  __syncwarp();
  return false;
}
// bounded wait by a whole converged warp: every lane leaves on the same poll
__device__ __forceinline__ bool bar_wait_warp(uint32_t a, uint32_t parity, volatile int* abort_flag, int* err) {
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
    if (__all_sync(0xffffffffu, bar_try(a, parity))) return true;
    if (__any_sync(0xffffffffu, *abort_flag != 0)) return false;
  }
  if ((threadIdx.x & 31) == 0) {
    *abort_flag = 1;
    atomicExch(err, 4);
  }
  __syncwarp();
  return false;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// prefetch of a 2-D tile into L2 (no shared memory, no barrier)
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap* map, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y)
               : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor (tcgen05): start>>4 [0,14), LBO>>4 [16,30), SBO>>4 [32,46),
// fixed 0b001 at [46,49), base offset 0, swizzle mode at [61,64) (2 = 128-byte swizzle)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (2ull << 61);
}
// The descriptor of a tile `bytes` (a multiple of 16) further on: the start-address field is
// the low 14 bits of the low word, and shared-memory addresses stay below 256 KB, so the add
// never carries out of the field.  One 32-bit add instead of rebuilding the descriptor.
__device__ __forceinline__ uint64_t sdesc_at(uint64_t d, uint32_t bytes) {
  const uint32_t lo = (uint32_t)d + (bytes >> 4), hi = (uint32_t)(d >> 32);
  return ((uint64_t)hi << 32) | lo;
}
// instruction descriptor, kind::f16: D=f32 (bit 4), A=B=bf16 (bits 7, 10), A/B major at 15/16,
// N>>3 at [17,23), M>>4 at [24,29)
__host__ __device__ constexpr uint32_t idesc(int M, int N, int a_mn_major, int b_mn_major) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn_major << 15) | ((uint32_t)b_mn_major << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// tcgen05.mma (kind::f16, one CTA, D in TMEM, A and B from shared-memory descriptors; acc = 0
// overwrites D), executed by a whole converged warp: one elected lane issues the MMA.  Issuing
// from a converged warp keeps the descriptor arithmetic warp-uniform; from inside
// `if (lane == 0)` every MMA cost ~70-90 cycles of issue latency.
__device__ __forceinline__ void mma_bf16_warp(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p, e;\n\telect.sync _|e, 0xffffffff;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
// As mma_bf16_warp with the A operand (M lanes x K, two bf16 per 32-bit column, the lower
// half holding the even k) read from tensor memory at a_tmem instead of shared memory.
__device__ __forceinline__ void mma_bf16_tmem_a_warp(uint32_t tmem_d, uint32_t a_tmem, uint64_t b, uint32_t id,
                                                     uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p, e;\n\telect.sync _|e, 0xffffffff;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "@e tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
      "r"(a_tmem), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit_warp(uint32_t bar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\telect.sync _|e, 0xffffffff;\n\t"
      "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}" ::"r"(bar)
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}
// TMEM store of 16 columns (one 32-bit value per lane and column); tmem_wait_st before the
// values may be consumed by another thread or the tensor pipe
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// asynchronous TMEM load of 16 columns; the registers are valid only after tmem_wait16
__device__ __forceinline__ void tmem_ld16u(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// wait::ld with the loaded registers as operands, so no use can be scheduled before it
__device__ __forceinline__ void tmem_wait16(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15])
               :
               : "memory");
}

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}


}  // namespace tc
}  // namespace gbn
