// tcgen05 (5th-generation tensor core) helpers for sm_103a: TMEM allocation, shared-memory
// matrix descriptors, BF16 MMA with FP32 accumulation in TMEM, commit / mbarrier wait,
// TMEM -> register loads.  Inline PTX only.
//
// Operand layout used throughout: no-swizzle K-major tiles made of 8-row x 16-byte core
// matrices (8 rows x 8 bf16).  Element (r, k) of a tile with R rows and 32 K-columns lives at
//     (r % 8) * 16 + (k % 8) * 2 + (k / 8) * KS + (r / 8) * 128,   KS = R / 8 * 128
// The descriptor's leading-byte-offset is the K-direction core-matrix stride (KS) and the
// stride-byte-offset the row-direction one (128).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace matpl {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t desc_kmajor(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: BF16 A and B (K-major), FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// The same with MN-major ("transposed") A and / or B operands.  An MN-major no-swizzle operand
// is made of the same 128-byte core matrices, each now 8 K-rows of 16 bytes (8 consecutive
// M / N elements): element (mn, k) at (k % 8) * 16 + (mn % 8) * 2 + (k / 8) * LBO +
// (mn / 8) * SBO.  With LBO = 128 and SBO = (K / 8) * 128 that is exactly the K-major
// activation layout above read with rows and columns exchanged, so a tile written row by row
// (thread r owns row r) serves as an MN-major operand whose K index is r.
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N, bool a_mn, bool b_mn) {
    return idesc_bf16(M, N) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}

__device__ __forceinline__ uint32_t tile_off(int r, int k, int KS) {
    return (uint32_t)((r & 7) * 16 + (k & 7) * 2 + (k >> 3) * KS + (r >> 3) * 128);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(mbar)));
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// Bounded wait for the given phase parity; returns false after `limit` polls (caller records
// the timeout and carries on, so a lost arrival never hangs the GPU).
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit; ++it) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity));
        if (done) return true;
    }
    return false;
}

// Non-blocking form: `limit` single checks with mbarrier.test_wait (no hardware suspend), so a
// small limit gives up after a fixed, short time.
__device__ __forceinline__ bool mbar_poll(uint64_t *mbar, uint32_t parity, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit; ++it) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity));
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

// One warp allocates `ncols` TMEM columns (power of two >= 32); the base address is written
// to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(dst)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t base, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols));
}

// Warp w reads TMEM lanes [32w, 32w+32): thread l of the warp gets row 32w+l, 32 columns.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

// Warp w reads TMEM lanes [32w, 32w+32), 16 columns.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// Warp w writes TMEM lanes [32w, 32w+32): thread l stores 32 columns of row 32w+l.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float v[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(
            taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])),
        "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])), "r"(__float_as_uint(v[20])),
        "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
        "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])),
        "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])),
        "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Single-instruction hardware tanh (MUFU), used by the mixed-precision fast form.
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 8 floats -> 8 bf16 (hi) and, with `lo`, the 8 bf16 of the remainders (v - hi), each packed
// as 16 bytes (element 0 at the lowest address).
__device__ __forceinline__ void split8(const float *v, uint4 &hi, uint4 *lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __nv_bfloat162 p = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
        h[q] = *reinterpret_cast<const uint32_t *>(&p);
        if (lo) {
            const __nv_bfloat162 r = __floats2bfloat162_rn(v[2 * q] - __low2float(p),
                                                           v[2 * q + 1] - __high2float(p));
            l[q] = *reinterpret_cast<const uint32_t *>(&r);
        }
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    if (lo) *lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Store 8 consecutive K values (k = 8*c .. 8*c+7) of row r as bf16 into a K-major tile.
__device__ __forceinline__ void store_row8(unsigned char *tile, int r, int c, int KS,
                                           const float *v) {
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v[4], v[5]);
    __nv_bfloat162 p3 = __floats2bfloat162_rn(v[6], v[7]);
    uint4 u;
    u.x = *reinterpret_cast<uint32_t *>(&p0);
    u.y = *reinterpret_cast<uint32_t *>(&p1);
    u.z = *reinterpret_cast<uint32_t *>(&p2);
    u.w = *reinterpret_cast<uint32_t *>(&p3);
    *reinterpret_cast<uint4 *>(tile + tile_off(r, 8 * c, KS)) = u;
}

}  // namespace tc
}  // namespace matpl
