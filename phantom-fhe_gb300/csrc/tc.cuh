// tc.cuh — 5th-generation tensor-core (tcgen05) building blocks for exact integer contractions.
//
// An RNS base conversion out_j = sum_i y_i * M_ij mod p_j becomes an exact bf16 GEMM:
//   y_i = sum_a y_ia 2^(8a)                       (bytes of the input residue, a < 8)
//   M'_iaj = 2^(8a) * M_ij mod p_j = sum_b m_iajb 2^(8b)   (host-side, bytes b < 8)
//   C_jb = sum_(i,a) y_ia * m_iajb                 (the GEMM: K = 8 alpha, N = 8 outputs)
//   out_j = (sum_b C_jb 2^(8b)) mod p_j            (epilogue, CUDA cores)
// Bytes are exact in bf16 (8 significant bits), every product is below 2^16 and with K <= 48 every
// C_jb is an integer below 2^22, so the f32 accumulation in tensor memory is exact and the result
// equals the 64-bit CUDA-core conversion word for word.
//
// Operands are K-major, no swizzle: 8-row x 16-byte core matrices, the K-direction neighbour
// 128 bytes on (leading byte offset), the next 8-row block (K/8) x 128 bytes on (stride byte
// offset).  One elected thread issues tcgen05.mma (kind::f16, bf16 inputs, f32 accumulator,
// M = 128) and commits to an mbarrier; the epilogue reads the accumulator with tcgen05.ld.
// Every wait is bounded: on timeout the kernel records an error in the context's status word,
// skips its remaining work, frees its tensor memory and returns.
#pragma once
#include <cstdint>

#include "modarith.cuh"

namespace pfg {

// One output of a tensor-core base conversion: its limb index in the output buffer, the index of
// its modulus in the context's table, and 1/p as f32.
struct TcOutMeta {
    uint32_t jj, tbl;
    float invp;
};

namespace tc {

constexpr int kRows = 128;           // MMA M: coefficients per tile
constexpr int kThreads = 256;        // two warps per tensor-memory lane quarter
constexpr int kTmemCols = 256;       // f32 accumulator columns per CTA
constexpr int kMaxOut = kTmemCols / 8;
constexpr int kSmemBytes = 80 * 1024;  // also caps residency at two CTAs per SM (2 x 256 columns)
constexpr int kPipeThreads = 512;        // pipelined kernels: four warps per lane quarter
constexpr int kPipeSmemBytes = 120 * 1024;  // one CTA per SM: it owns all 512 tensor-memory columns
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t kMagic = 0x4B000000u;  // bit pattern of 2^23

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading (K) and stride (row-block) byte offsets
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: f32 accumulator, bf16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(cols));
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(a), "l"(b), "r"(idesc), "r"(acc)
            : "memory");
}
__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// true when the phase of the given parity completed within the limit
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < kWaitLimit && !done; it++)
        asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(saddr(bar)), "r"(parity)
                : "memory");
    return done != 0;
}
// 32 lanes x 8 consecutive f32 columns (one output's byte planes) per thread
__device__ __forceinline__ void ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// bf16 bit patterns of bytes 2w and 2w+1 of v, packed (lower K index in the low half)
__device__ __forceinline__ uint32_t byte_pair_bf16(uint64_t v, int w) {
    const uint32_t src = (uint32_t)(v >> (32 * (w >> 1)));
    const int k0 = (w & 1) * 2;
    // 0x4B0000bb = 2^23 + b as float bits; minus 2^23 gives b exactly
    const float f0 = __uint_as_float(__byte_perm(src, kMagic, k0 | 0x7540)) - 8388608.0f;
    const float f1 = __uint_as_float(__byte_perm(src, kMagic, (k0 + 1) | 0x7540)) - 8388608.0f;
    return __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
}

// 16 bytes = the 8 bf16 byte planes of one 64-bit residue (one core-matrix row)
__device__ __forceinline__ uint4 bytes_bf16(uint64_t v) {
    return make_uint4(byte_pair_bf16(v, 0), byte_pair_bf16(v, 1), byte_pair_bf16(v, 2), byte_pair_bf16(v, 3));
}

// x = V mod p up to one multiple of p (x in [0, 2p)), V = sum_b C_b 2^(8b), from the f32 bit
// patterns r[b] of the NPL plane sums.  Every constant M'_(i,a) is below p, so V < 255 K p and
// the quotient is below 255 K <= 2^16 (K <= 258 nonzero byte terms).  The f32 value of V times
// 1/p has relative error below 2^-20.5, so absolute error below 0.05; minus 0.625 it rounds to
// floor(V / p) or floor(V / p) - 1, clamped at 0.  V and q p are only needed modulo 2^64 because
// the remainder is small.  [0, 2p) is a valid input of the lazy forward NTT.
template <int NPL>
__device__ __forceinline__ uint64_t reduce_planes_lazy(const uint32_t *r, uint64_t p, float invp) {
    // f32 estimate of V as a tree of pairs (C_2k + 2^8 C_2k+1, then 2^16-weighted pairs of those,
    // ...): the same number of roundings per term as a running sum, half the dependent chain
    float t[NPL];
#pragma unroll
    for (int b = 0; b < NPL; b++) t[b] = __uint_as_float(r[b]);
#pragma unroll
    for (int w = 1; w < NPL; w *= 2)
#pragma unroll
        for (int b = 0; b + w < NPL; b += 2 * w)
            t[b] = fmaf(t[b + w], __uint_as_float((uint32_t)(127 + 8 * w) << 23), t[b]);
    const float vf = t[0];
    const float qf = fmaf(vf, invp, -0.625f);
    const int32_t qs = (int32_t)(__float_as_uint(qf + 12582912.0f) - 0x4B400000u);  // round to nearest
    const uint32_t q = (uint32_t)max(qs, 0);
    uint32_t u[NPL];
#pragma unroll
    for (int b = 0; b < NPL; b++) u[b] = __float_as_uint(__uint_as_float(r[b]) + 8388608.0f);  // kMagic + C_b
    uint64_t v = (uint64_t)u[0] + (uint64_t)u[1] * 256u + (uint64_t)u[2] * 65536u + (uint64_t)u[3] * 16777216u;
    uint32_t hi = 0;
#pragma unroll
    for (int b = 4; b < NPL; b++) hi += u[b] << (8 * (b - 4));
    v += (uint64_t)hi << 32;
    uint64_t k = 0;  // kMagic * sum_(b < NPL) 2^(8b) mod 2^64
#pragma unroll
    for (int b = 0; b < NPL; b++) k += (uint64_t)kMagic << (8 * b);
    return v - ((uint64_t)q * p + k);
}

}  // namespace tc
}  // namespace pfg
