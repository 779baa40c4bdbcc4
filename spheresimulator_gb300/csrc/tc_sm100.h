// tc_sm100.h — inline-PTX helpers for the 5th-generation tensor cores (tcgen05) of sm_100-class GPUs
// (sm_103a here): tensor-memory allocation, shared-memory matrix descriptors, the TF32 MMA with an
// FP32 accumulator in tensor memory, completion through an mbarrier, and tensor-memory loads.
//
// Operand layout used by every caller: K-major, no swizzle. A matrix of R rows (M for A, N for B) and
// K 32-bit elements is stored as "core matrices" of 8 rows x 16 bytes (4 TF32 values along K), each
// 128 contiguous bytes (row i of the core matrix at byte 16 i). Within one K chunk of KC elements the
// core matrices are ordered K-group fastest:
//     byte offset of (row r, k) = ((r / 8) * (KC / 4) + k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4
// so the K-adjacent core-matrix stride (leading byte offset) is 128 and the row-group stride
// (stride byte offset) is KC / 4 * 128. One MMA consumes K = 8 TF32 values (two core-matrix columns);
// the k-th K step of a chunk starts 256 bytes after the (k-1)-th.
//
// Written from the PTX ISA description of tcgen05 (instruction and shared-memory descriptor formats).
#pragma once

#include <cstdint>

namespace smob {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Instruction descriptor of tcgen05.mma.kind::tf32: D FP32, A and B TF32, both K-major, M x N tile.
//   bits 4-5 D format (1 = F32), 7-9 A format (2 = TF32), 10-12 B format (2 = TF32),
//   15/16 A/B major (0 = K), 17-22 N >> 3, 24-28 M >> 4.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// Shared-memory matrix descriptor (no swizzle): start address, leading (K-direction) and stride
// (row-group direction) byte offsets, all in 16-byte units; bits 46-47 hold the descriptor version (1).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
    uint64_t d = 0;
    d |= uint64_t((saddr >> 4) & 0x3FFFu);
    d |= uint64_t((lbo_bytes >> 4) & 0x3FFFu) << 16;
    d |= uint64_t((sbo_bytes >> 4) & 0x3FFFu) << 32;
    d |= uint64_t(1) << 46;
    return d;  // base offset 0, LBO mode 0, layout type 0 (no swizzle)
}

// ---- tensor memory (one warp, all lanes) ----
// ncols: power of two >= 32. The allocated base address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- MMA: D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread ----
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(uint32_t(accumulate))
        : "memory");
}
// the mbarrier gets one arrive when every tcgen05 operation this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

// ---- ordering between thread barriers and tcgen05 operations ----
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores (async proxy)
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- mbarriers ----
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the completion of the phase with the given parity; gives up after max_polls polls
// (returns false) so that a lost completion can never hang the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity, long long max_polls) {
    for (long long i = 0; i < max_polls; ++i) {
        if (mbar_try_wait(mbar, parity)) return true;
        if (i > 64) __nanosleep(32);
    }
    return false;
}

// ---- tensor memory -> registers: 32 lanes (the warp's quarter) x 32 consecutive 32-bit columns ----
__device__ __forceinline__ void tmem_ld_32x32b_x32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- TF32 splitting (3xTF32 products: hi*hi + hi*lo + lo*hi keep ~FP32 accuracy) ----
// hi: x rounded to TF32 (10 explicit mantissa bits, exactly representable), lo: the remainder (exact in FP32)
__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
    hi = tf32_hi(x);
    lo = x - hi;
}

// byte offset of element (row r, k) in a K-major no-swizzle chunk of kc (multiple of 4) elements per row
__host__ __device__ constexpr uint32_t kmajor_offset(int r, int k, int kc) {
    return uint32_t(((r >> 3) * (kc >> 2) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

}  // namespace tc
}  // namespace smob
