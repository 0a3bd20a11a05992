// Fifth-generation tensor-core primitives (sm_103a) for the learned
// preconditioner's dense layers: tcgen05.mma with operands in shared memory
// and the FP32 accumulator in tensor memory (TMEM).
//
// Operand layout: K-major, no swizzle.  An R x K BF16 tile is stored as 8 x 8
// core matrices (8 rows of 16 bytes, 128 contiguous bytes each); core
// matrices adjacent along K are 128 bytes apart (the descriptor's leading
// byte offset), core matrices adjacent along R are K * 16 bytes apart (its
// stride byte offset).  One kind::f16 instruction consumes K = 16, i.e. two
// core matrices along K, so step s of a K loop starts 256 * s bytes in.
//
// FP32 inputs are carried as three BF16 terms x = hi + mid + lo (each the
// BF16 rounding of what the previous terms leave), so a product with a BF16
// weight is exact to 2^-26 of |x| and the tensor core accumulates in FP32:
// the layer keeps FP32 activations, with weights that are BF16 by design.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace eolc {
namespace tc {

constexpr int kSplit = 3;  // BF16 terms per FP32 activation

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) in an R x K canonical tile
__host__ __device__ constexpr int tile_off(int r, int k, int K) {
  return ((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// the three BF16 terms of x
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m,
                                       __nv_bfloat16 &l) {
  h = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(h);
  m = __float2bfloat16_rn(r1);
  l = __float2bfloat16_rn(r1 - __bfloat162float(m));
}

// x (row r, column k) into the three tiles part0 .. part2 (part_bytes apart)
__device__ __forceinline__ void put3(uint8_t *part0, int part_bytes, int r, int k, int K,
                                     float x) {
  __nv_bfloat16 h, m, l;
  split3(x, h, m, l);
  const int o = tile_off(r, k, K);
  *reinterpret_cast<__nv_bfloat16 *>(part0 + o) = h;
  *reinterpret_cast<__nv_bfloat16 *>(part0 + part_bytes + o) = m;
  *reinterpret_cast<__nv_bfloat16 *>(part0 + 2 * part_bytes + o) = l;
}

// four consecutive columns k .. k + 3 (k a multiple of 4) of row r, as
// 8-byte stores into each of the three tiles
__device__ __forceinline__ void put3x4(uint8_t *part0, int part_bytes, int r, int k, int K,
                                       float x0, float x1, float x2, float x3) {
  const float x[4] = {x0, x1, x2, x3};
  __nv_bfloat16 t[3][4];
#pragma unroll
  for (int c = 0; c < 4; ++c) split3(x[c], t[0][c], t[1][c], t[2][c]);
  const int o = tile_off(r, k, K);
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const __nv_bfloat162 lo2 = __halves2bfloat162(t[p][0], t[p][1]);
    const __nv_bfloat162 hi2 = __halves2bfloat162(t[p][2], t[p][3]);
    *reinterpret_cast<uint2 *>(part0 + p * part_bytes + o) =
        make_uint2(*reinterpret_cast<const uint32_t *>(&lo2),
                   *reinterpret_cast<const uint32_t *>(&hi2));
  }
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (row-group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor, kind::f16: BF16 A and B (both K-major), FP32 D,
// M x N tile.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) |
         (uint32_t(M >> 4) << 24);
}

// ---- TMEM allocation (one full warp) -------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// ---- ordering --------------------------------------------------------------------
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- mbarrier --------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for phase `parity` to complete; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit) {
  for (long long k = 0; k < limit; ++k)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// ---- MMA ---------------------------------------------------------------------------
// D[tmem] = A B^T (+ D when accumulate), issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive once on bar when every MMA this thread issued has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// ---- TMEM -> registers -------------------------------------------------------------
// 32 consecutive columns of this warp's 32 TMEM lanes (lane = accumulator row)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

}  // namespace tc
}  // namespace eolc
