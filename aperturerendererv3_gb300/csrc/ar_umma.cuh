// Blackwell (sm_103a) tensor-core building blocks in inline PTX: TMEM
// allocation, tcgen05.mma (kind::f16, BF16 operands, FP32 accumulate) from
// shared-memory descriptors, completion through an mbarrier, and tcgen05.ld
// of the accumulator into registers.
//
// Operand layout: no swizzle, "core matrices" of 8 rows x 16 bytes (8 bf16)
// stored contiguously (128 B).  A tile of R rows x C columns keeps core matrix
// (row group g, column chunk c) at byte ((g * C/8) + c) * 128, row r of it at
// +16 * (r % 8).  The same bytes serve as
//   * a K-major operand (rows = M or N, columns = K), and
//   * an MN-major operand (rows = K, columns = M or N),
// the two descriptors differing only in which stride is called leading and
// which stride (see make_desc).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ar
{
namespace umma
{
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, c) in a tile with C columns (bf16)
__host__ __device__ __forceinline__ uint32_t tile_offset(int r, int c, int C)
{
    return (uint32_t)((((r >> 3) * (C >> 3)) + (c >> 3)) * 128 + (r & 7) * 16 + (c & 7) * 2);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (16-byte units), the fixed 0b001 at bits 46-48,
// no swizzle.  Without swizzling the leading offset is the distance between
// core matrices adjacent along K and the stride offset the distance between
// core matrices adjacent along M (or N), for K-major and MN-major operands
// alike (checked against a host GEMM by ar_diag_umma_gemm).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor for kind::f16 with BF16 A/B and FP32 D.
// a_mn / b_mn: operand stored MN-major instead of K-major.
__host__ __device__ __forceinline__ uint32_t make_idesc(int M, int N, bool a_mn, bool b_mn)
{
    uint32_t d = 0;
    d |= 1u << 4;   // D: F32
    d |= 1u << 7;   // A: BF16
    d |= 1u << 10;  // B: BF16
    d |= (a_mn ? 1u : 0u) << 15;
    d |= (b_mn ? 1u : 0u) << 16;
    d |= (uint32_t)(N >> 3) << 17;
    d |= (uint32_t)(M >> 4) << 24;
    return d;
}

// D[tmem] (+)= A * B^T, one instruction (K = 16), issued by one thread
__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1 : 0));
}

// arrive on the mbarrier once every previously issued tcgen05.mma of this thread completes
__device__ __forceinline__ void commit(uint64_t* mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}

// bounded wait for the phase with the given parity; false when the bound ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_iters = 1u << 26)
{
    const uint32_t a = smem_addr(mbar);
    for (uint32_t it = 0; it < max_iters; ++it)
    {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor cores' async proxy
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// TMEM allocation by one full warp; the base address is written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols) : "memory");
}

// Descriptor of a tile in the core-matrix layout (R rows x C columns, bf16),
// starting at (row, column) = (r0, c0) (multiples of 8), read as a K-major
// operand (rows along M/N, columns along K) or an MN-major one (rows along K).
__device__ __forceinline__ uint64_t tile_desc(uint32_t base, int C, int r0, int c0, bool mn_major)
{
    const uint32_t row_group = (uint32_t)(C >> 3) * 128u;  // next 8 rows
    const uint32_t col_chunk = 128u;                         // next 8 columns
    const uint32_t addr = base + (uint32_t)(r0 >> 3) * row_group + (uint32_t)(c0 >> 3) * col_chunk;
    return mn_major ? make_desc(addr, row_group, col_chunk) : make_desc(addr, col_chunk, row_group);
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32(w%4)..+31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
} // namespace umma
} // namespace ar
