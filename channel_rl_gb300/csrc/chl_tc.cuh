// tcgen05 (5th-generation tensor core) building blocks for sm_103a:
// TMEM allocation, shared-memory matrix descriptors (K-major, no swizzle),
// BF16 x BF16 -> FP32 MMA issue/commit, bounded mbarrier waits and TMEM
// loads.  Inline PTX only.
//
// Operand layout in shared memory ("canonical K-major, no swizzle"): a tile
// of R rows x K columns (BF16) is made of 8x8 core matrices of 128
// contiguous bytes (8 rows of 16 B).  Element (r, k) sits at
//   (r/8)*SBO + (k/8)*LBO + (r%8)*16 + (k%8)*2  bytes,
// with LBO = 128 (core matrices adjacent along K are contiguous) and
// SBO = (K/8)*128 (the next 8-row group follows all K core matrices).  One
// MMA consumes K = 16, i.e. two core matrices: the descriptor for k-step s
// starts 256*s bytes further.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t canon_off(int r, int k, uint32_t lbo, uint32_t sbo) {
  return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 3) * lbo + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

// Shared-memory matrix descriptor (tcgen05): start >> 4 in [0,14), LBO >> 4
// in [16,30), SBO >> 4 in [32,46), version 1 in [46,48), no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 in [17,23), M >> 4 in [24,29).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      :: "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait: returns false if the phase did not complete in max_iter polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, long max_iter) {
  const uint32_t addr = smem_u32(mbar);
  for (long it = 0; it < max_iter; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done) : "r"(addr), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Whole warp: allocate ncols TMEM columns, address written to *dst (smem).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               :: "r"(smem_u32(dst)), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}

// Warp-collective: 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Store one row of 64 BF16 values (r fixed, k = 0..63) into a canonical tile.
__device__ __forceinline__ void store_row64(unsigned char* tile, int r, const float* v, uint32_t lbo, uint32_t sbo) {
#pragma unroll
  for (int kb = 0; kb < 8; ++kb) {
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[8 * kb + 0], v[8 * kb + 1]);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v[8 * kb + 2], v[8 * kb + 3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v[8 * kb + 4], v[8 * kb + 5]);
    __nv_bfloat162 p3 = __floats2bfloat162_rn(v[8 * kb + 6], v[8 * kb + 7]);
    uint4 u;
    u.x = *reinterpret_cast<uint32_t*>(&p0); u.y = *reinterpret_cast<uint32_t*>(&p1);
    u.z = *reinterpret_cast<uint32_t*>(&p2); u.w = *reinterpret_cast<uint32_t*>(&p3);
    *reinterpret_cast<uint4*>(tile + canon_off(r, 8 * kb, lbo, sbo)) = u;
  }
}

__device__ __forceinline__ void store_elem(unsigned char* tile, int r, int k, float v, uint32_t lbo, uint32_t sbo) {
  *reinterpret_cast<__nv_bfloat16*>(tile + canon_off(r, k, lbo, sbo)) = __float2bfloat16_rn(v);
}

}  // namespace tc
