// Blackwell (sm_100 family, here sm_103a) tensor-core building blocks in
// inline PTX: tcgen05.mma with its accumulator in tensor memory (TMEM), TMA
// tile loads (cp.async.bulk.tensor) completing on mbarriers, and the host-side
// encoders of the descriptors these instructions take.
//
// The encoders are plain constexpr functions of the bit layouts published in
// the PTX ISA (tcgen05 "Matrix Descriptors" and "Instruction descriptor"), so
// that host code can compute and check them and the kernels only add a shared
// memory address.  The CPU tests compile this header with the host compiler
// and compare against hand-worked encodings.
#pragma once
#include <cstdint>

namespace mlf {
namespace tc {

// ---- shared-memory matrix descriptor (64 bits) ---------------------------
//   [0,14)  matrix start address >> 4 (shared-window offset)
//   [16,30) leading-dimension byte offset >> 4
//   [32,46) stride-dimension byte offset >> 4
//   [46,48) descriptor version: 1 for the sm_100 family
//   [49,52) matrix base offset (0 when the swizzle atoms start 1024-aligned)
//   [52]    leading-dimension stride mode (0: relative offsets)
//   [61,64) swizzling: 0 none, 1 128-byte with 32-byte atom, 2 128-byte,
//           4 64-byte, 6 32-byte
constexpr uint64_t SWIZZLE_NONE = 0, SWIZZLE_128B = 2, SWIZZLE_64B = 4, SWIZZLE_32B = 6;

#if defined(__CUDACC__)
#define MLF_HD __host__ __device__
#else
#define MLF_HD
#endif

MLF_HD constexpr uint64_t smem_desc(uint32_t addr, uint32_t lbo_bytes, uint32_t sbo_bytes, uint64_t swizzle) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (swizzle << 61);
}

// K-major operand tile staged by TMA with 128-byte swizzling: rows of 128
// bytes (32 TF32 values), 8-row swizzle atoms of 1024 bytes stacked along M
// (or N).  The leading offset is unused for swizzled K-major layouts (encoded
// as 16 bytes); the stride between 8-row groups is 1024 bytes.  A K step of
// 8 TF32 values inside the 128-byte row moves the start address by 32 bytes.
MLF_HD constexpr uint64_t kmajor_sw128_desc(uint32_t addr) { return smem_desc(addr, 16, 1024, SWIZZLE_128B); }

// Byte offset of 16-byte chunk c (0..7) of row r in such a tile, for operands
// written by threads rather than TMA: the 128-byte swizzle places the chunk at
// c XOR (r mod 8) within its row (the tile 1024-byte aligned).
MLF_HD constexpr uint32_t sw128_offset(uint32_t r, uint32_t c) { return r * 128u + ((c ^ (r & 7u)) << 4); }

// ---- instruction descriptor of tcgen05.mma .kind::tf32 / .kind::f16 (32 bits)
//   [0,2) sparsity selector, [2] sparse, [3] saturate   (all 0: dense)
//   [4,6)   D format: 0 F16, 1 F32
//   [7,10)  A format, [10,13) B format: 0 F16, 1 BF16, 2 TF32
//   [13] negate A, [14] negate B
//   [15] A major, [16] B major: 0 K-major, 1 MN-major
//   [17,23) N >> 3
//   [24,29) M >> 4
//   [30,32) maximum shift (weight-stationary only; 0)
constexpr uint32_t FMT_F16 = 0, FMT_BF16 = 1, FMT_TF32 = 2;

MLF_HD constexpr uint32_t instr_desc_f32acc(uint32_t ab_format, int M, int N) {
    return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// shapes tcgen05.mma accepts for cta_group::1, dense .kind::tf32/.kind::f16:
// M = 64 with N a multiple of 8, or M = 128 with N a multiple of 16, N in [8|16, 256]
MLF_HD constexpr bool valid_shape(int M, int N) {
    return (M == 64 && N >= 8 && N <= 256 && N % 8 == 0) || (M == 128 && N >= 16 && N <= 256 && N % 16 == 0);
}

#if defined(__CUDACC__)
// ---- device wrappers --------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// make barrier initialisation visible to the async proxy (TMA, tensor cores)
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// one arrival of this thread (release: its earlier shared-memory writes are
// visible to whoever observes the phase complete)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// barrier among nthreads threads (a multiple of 32: whole warps) of the CTA, id 1..15
__device__ __forceinline__ void named_bar_sync(uint32_t id, uint32_t nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
// Wait for the phase with the given parity to complete; gives up after
// max_iter polls (each poll may itself suspend for a bounded time) and
// returns false then.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_iter) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t it = 0; it < max_iter; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// 2-D tile load global -> shared through a tensor map; x is the innermost
// (element) coordinate, y the row.  Completion is signalled on bar as bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
// The same with an L2 cache policy (createpolicy below) for the loaded lines.
__device__ __forceinline__ void tma_load_2d_hint(void* dst, const void* tmap, int x, int y, uint64_t* bar,
                                                 uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, "
        "%3}], [%4], %5;" ::"r"(smem_u32(dst)),
        "l"((uint64_t)tmap), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}
// L2 policy for lines streamed once: evicted first
__device__ __forceinline__ uint64_t l2_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void tma_prefetch_desc(const void* tmap) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)tmap) : "memory");
}

// TMEM: whole-warp allocation of ncols columns (power of two >= 32); the base
// address is written to shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] = (accumulate ? D : 0) + A * B, A (M x K) and B (N x K) K-major in
// shared memory, FP32 accumulation; issued by a single thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The same with BF16 (or F16, per the instruction descriptor) operands, .kind::f16.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// make this thread's generic-proxy shared-memory writes visible to the async
// proxy (tcgen05.mma operands written with st.shared)
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// The mbarrier receives one arrival when every tcgen05.mma this thread issued
// before has completed (their shared-memory operands are then free).
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive accumulator columns of the warp's 32 TMEM lanes: lane
// (taddr lane + laneid), columns taddr col .. +31 into v[0..31].
__device__ __forceinline__ void tmem_ld_32x32b_x32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

// TF32 split of an FP32 value: hi = round-to-nearest TF32 of x, lo = the TF32
// of the remainder; hi*b_hi + hi*b_lo + lo*b_hi recovers FP32 accuracy.
__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
#endif

}  // namespace tc
}  // namespace mlf
