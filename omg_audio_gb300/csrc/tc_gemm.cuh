// Tensor-core GEMM building blocks for sm_103a (tcgen05 + TMEM), written as
// inline PTX: shared-memory matrix descriptors, the kind::f16 instruction
// descriptor, TMEM allocation, MMA issue / commit, bounded mbarrier waits and
// TMEM loads. Used by the surrogate MLP (mlp.cu).
//
// Operand layout in shared memory: K-major, no swizzle. A tile of R rows x 64
// K elements (bf16) is stored as 8-row x 8-element core matrices (8 rows of
// 16 bytes, 128 B each); the 8 core matrices along K of one 8-row group are
// contiguous (leading-dimension byte offset 128 B) and 8-row groups are
// 1024 B apart (stride-dimension byte offset). One MMA consumes K = 16, i.e.
// two core matrices along K: the k-th MMA of a 64-wide chunk starts 256 k
// bytes into the tile.
#pragma once
#include <cstdint>

namespace omg {
namespace tc {

constexpr uint32_t kChunkK = 64;        // K elements staged per round
constexpr uint32_t kLbo = 128;          // bytes between core matrices along K
constexpr uint32_t kSbo = 1024;         // bytes between 8-row groups

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 64-bit shared-memory matrix descriptor: start address, leading and stride
// byte offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((kLbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((kSbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: f32 accumulator, bf16 A
// and B, both K-major, N = n (multiple of 16, <= 256), M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t n, uint32_t m) {
  return (1u << 4)                 // D format: f32
         | (1u << 7)               // A format: bf16
         | (1u << 10)              // B format: bf16
         | ((n >> 3) << 17)        // N >> 3
         | ((m >> 4) << 24);       // M >> 4
}

// Byte offset of element (r, k) of a staged tile (k < 64).
__device__ __forceinline__ uint32_t tile_offset(uint32_t r, uint32_t k) {
  return (r >> 3) * kSbo + (k >> 3) * kLbo + (r & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] . B[smem]^T, one MMA, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// The MMAs issued so far by this thread arrive on the mbarrier when done.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Bounded wait for the mbarrier phase `parity`; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_polls) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t i = 0; i < max_polls; i++) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Asynchronous 16-byte global -> shared copies (cp.async, L2 only): `bytes`
// (0 or 16) are read, the rest of the 16 bytes is filled with zeros.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc, uint32_t bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem_dst)), "l"(gsrc), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// 16 consecutive f32 columns of this thread's TMEM lane (warp w of the CTA
// reads lanes 32 w .. 32 w + 31).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace omg
