// Fifth-generation tensor cores (tcgen05) for the FP32 rank updates of the
// factorisation: a 128 x 128 FP32 tile C = A * B in tensor memory.  The
// FP32 form takes three TF32 products per K step,
//     A * B ~= Ahi * Bhi + Ahi * Blo + Alo * Bhi,
// Ahi = tf32(A) (round to nearest), Alo = tf32(A - Ahi), which carries the
// product to about FP32 accuracy (the dropped Alo * Blo term is ~2^-22
// relative).  Operands arrive pre-split in the canonical K-major layout
// without swizzle (8-row x 16-byte core matrices, K-adjacent core matrices
// 128 bytes apart, 8-row groups SBO = KCH * 32 bytes apart), written by the
// panel kernel; this header holds the descriptors, the MMA, TMEM and mbarrier
// primitives, and the shared-memory plan of the packed pipeline.
// The BF16 form (SPK_BF16S) takes one kind::f16 product with BF16 A and B
// and FP32 accumulation per K step; its operands are single BF16 copies of
// the panels (a quarter of the TF32 hi + lo bytes), each block's L panel
// scaled by 2^e and its U panel by 2^-e (e from the block's diagonal), so
// that every product L U^T is unchanged and the scaled panels stay near 1.
#pragma once
#include <cstdint>

namespace spk {
namespace umma {

constexpr int TM = 128, TN = 128, KCH = 16;           // tile rows, tile columns, K per stage
constexpr int OPB = TM * KCH * 4;                     // bytes of one operand part (8 KB)
constexpr int SBO = KCH * 32;                         // bytes between 8-row groups
constexpr int STAGE = 4 * OPB;                        // Ahi, Alo, Bhi, Blo
constexpr unsigned WAIT_LIMIT = 1u << 20;             // polls of an mbarrier before giving up

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N)
// byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t desc_kmajor(uint32_t start, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((start & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Warp-wide: allocate `ncols` TMEM columns, address written to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Warp-wide: 32 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// Packed operands.  The panel kernel writes the L and U panels of a block a
// second time as TF32 hi / lo parts already in the canonical layout: for a
// 128-line tile and a chunk of KCH block columns, 16 KB = [hi 8 KB][lo 8 KB]
// (byte offset of element (line i, column kk) in a part: packed_offset).  A
// tile product then streams whole chunks with bulk asynchronous copies
// (cp.async.bulk, completion counted in bytes on an mbarrier) through a ring
// of PST stages; one thread issues the copies, one thread the MMAs, and four
// warps drain a double-buffered accumulator (2 x 128 TMEM columns), so the
// epilogue of a tile overlaps the MMAs of the next.
// ---------------------------------------------------------------------------
constexpr int PCHUNK = 2 * OPB;                       // one packed operand chunk (hi + lo), 16 KB
constexpr int PST = 5;                                // stages of the packed pipeline
constexpr int PSMEM = PST * STAGE + 2048;             // + alignment slack, barriers, TMEM address

__host__ __device__ constexpr uint32_t packed_offset(int i, int kk) {
    return (uint32_t)((i >> 3) * SBO + (kk >> 2) * 128 + (i & 7) * 16 + (kk & 3) * 4);
}

// BF16 packed operands: the same tiles and 16-column chunks, one BF16 part
// per chunk (4 KB: 8-row x 16-byte core matrices, the two K-adjacent ones
// 128 bytes apart, 8-row groups SBO16 apart).  The byte offset of a block's
// BF16 pack is a quarter of its TF32 pack offset.  A pipeline stage carries
// up to BF_GROUP consecutive chunks of one tile and block (one bulk copy per
// operand), i.e. BF_GROUP MMAs of K = 16.
constexpr int PCHUNK16 = TM * KCH * 2;                // 4 KB
constexpr int SBO16 = KCH * 16;                       // 256 bytes between 8-row groups
constexpr int BF_GROUP = 4;                           // chunks per stage: 16 KB per operand

__host__ __device__ constexpr uint32_t packed_offset16(int i, int kk) {
    return (uint32_t)((i >> 3) * SBO16 + (kk >> 3) * 128 + (i & 7) * 16 + (kk & 7) * 2);
}

// Two floats as round-to-nearest BF16, low half first.
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// 2^e as a float (e in the normal range).
__device__ __forceinline__ float exp2i(int e) { return __int_as_float((127 + e) << 23); }

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}

// Wait with a poll budget that collapses after the first timeout in the CTA
// (*dead set), so that a broken pipeline still ends quickly; false on timeout.
__device__ __forceinline__ bool wait_bounded(uint64_t* bar, uint32_t parity, volatile int* dead, int* err) {
    const unsigned limit = *dead ? 1u : WAIT_LIMIT;
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    *dead = 1;
    if (err) atomicExch(err, 1);
    return false;
}

// Wide tiles: a CTA computes NH adjacent 128 x 128 tiles of one tile row
// (128 x 128 NH), so that each A chunk it stages serves NH products.  A
// stage holds A (hi, lo) and NH B chunks (hi, lo), B tile h at (2 + 2h) OPB;
// the accumulator takes NH x 128 TMEM columns, double-buffered.
template <int NH>
struct PGeo {
    static constexpr int STAGE = (2 + 2 * NH) * OPB;
    static constexpr int NST = NH == 1 ? PST : 4;           // stages that fit beside the rest
    static constexpr int SMEM = NST * STAGE + 2048;
    static constexpr uint32_t TMEM_COLS = 2 * NH * TN;
};

// Barriers and TMEM of a packed-pipeline CTA (carved from dynamic shared memory).
struct PCtx {
    unsigned char* stage;   // NST * STAGE bytes, 1024-aligned
    uint64_t *full, *empty, *tfull, *tempty;
    uint32_t* tmem_slot;
};

template <int NH = 1>
__device__ __forceinline__ PCtx pctx_of(unsigned char* smem_raw) {
    unsigned char* base =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    PCtx c;
    c.stage = base;
    c.full = reinterpret_cast<uint64_t*>(base + PGeo<NH>::NST * PGeo<NH>::STAGE);
    c.empty = c.full + PGeo<NH>::NST;
    c.tfull = c.empty + PGeo<NH>::NST;
    c.tempty = c.tfull + 2;
    c.tmem_slot = reinterpret_cast<uint32_t*>(c.tempty + 2);
    return c;
}

}  // namespace umma
}  // namespace spk
