// Device helpers shared by the tensor-core operators (sg_tc.cu, sg_tcsym.cu): TF32 splitting, the
// canonical no-swizzle K-major shared-memory layout and its matrix descriptor, bounded mbarrier
// waits, tcgen05 commit and tensor-memory loads/stores.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

static constexpr long long kTcWaitCycles = 2000000000LL;  // ~1 s at 2 GHz per wait
static constexpr unsigned kTcFull = 0xffffffffu;
static constexpr int kTcSmemBudget = 227 * 1024;

__device__ __forceinline__ float tf32_hi(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// float offset of element (row, k) in a canonical no-swizzle K-major tile with KC core columns:
// core matrix (row / 8, k / 4) is 8 rows x 16 bytes stored contiguously (128 bytes); core matrices
// adjacent in K are 128 bytes apart (LBO), adjacent 8-row groups KC * 128 bytes (SBO).
template <int KC>
__device__ __forceinline__ int tc_off(int row, int k) {
  return (((row >> 3) * KC + (k >> 2)) << 5) + ((row & 7) << 2) + (k & 3);
}

// shared-memory matrix descriptor: start, LBO = 128 B, SBO = KC * 128 B, no swizzle, version 1
template <int KC>
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)(((KC * 128) >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// true when the phase of `parity` has completed. A thread whose phase is still open is suspended
// until the phase completes or about 0.1 ms have passed (the suspend-time hint), so waiting roles
// take no issue slots from the producers while they wait.
__device__ __forceinline__ bool tc_poll(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(100000u)
      : "memory");
  return ok != 0;
}

// one thread: true when the phase of `parity` has completed, false when the budget ran out
__device__ __forceinline__ bool tc_wait1(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!tc_poll(bar, parity))
    if (clock64() - t0 > kTcWaitCycles) return false;
  return true;
}

// whole warp: every lane polls (each gets the barrier's acquire); one decision for the warp
__device__ __forceinline__ bool tc_waitw(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    if (__all_sync(kTcFull, tc_poll(bar, parity))) return true;
    const int late = (clock64() - t0 > kTcWaitCycles) ? 1 : 0;
    if (__shfl_sync(kTcFull, late, 0)) return false;
  }
}

__device__ __forceinline__ void tc_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]),
        "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
      "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
      : "memory");
}

}  // namespace sg
