// modarith.cuh — 64-bit modular arithmetic for sm_103a CUDA cores.
//
// Written from the published methods: Shoup's precomputed-quotient multiplication
// (w' = floor(w * 2^64 / q)), Barrett reduction of 128-bit values with
// mu = floor(2^128 / q) (Barrett 1986), and Harvey's lazy NTT butterflies (values kept in
// [0, 4q) / [0, 2q), q < 2^62).  These replace the reference's primitives in
// include/uintmodmath.cuh:18-243 and include/butterfly.cuh:10-37; every function returns
// the canonical residue unless its name says "lazy".
#pragma once
#include <cstdint>

namespace pfg {

struct Mod {
    uint64_t q;
    uint64_t mu_lo;  // floor(2^128 / q), low word
    uint64_t mu_hi;  // floor(2^128 / q), high word  (= floor(2^64 / q) for q > 1)
};

__device__ __forceinline__ uint64_t mulhi(uint64_t a, uint64_t b) { return __umul64hi(a, b); }

__device__ __forceinline__ uint64_t csub(uint64_t x, uint64_t q) { return x >= q ? x - q : x; }

__device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b, uint64_t q) { return csub(a + b, q); }

__device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b, uint64_t q) {
    return a >= b ? a - b : a + q - b;
}

// x * w mod q in [0, 2q), any x < 2^64, w < q, ws = floor(w * 2^64 / q)
__device__ __forceinline__ uint64_t mul_shoup_lazy(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
    return x * w - mulhi(x, ws) * q;
}

// floor(x * y / 2^64) - e with e in {0, 1, 2}: of the four 32 x 32-bit partial products the
// low one is dropped and the middle ones contribute their high words only.  The dropped terms
// are 2^32 (lo(xh yl) + lo(xl yh)) + xl yl < 3 * 2^64, so they carry at most 2 into the result.
__device__ __forceinline__ uint64_t mulhi_trunc(uint64_t x, uint64_t y) {
    const uint32_t xl = (uint32_t)x, xh = (uint32_t)(x >> 32), yl = (uint32_t)y, yh = (uint32_t)(y >> 32);
    return (uint64_t)xh * yh + __umulhi(xh, yl) + __umulhi(xl, yh);
}

// x * w mod q in [0, 4q), any x < 2^64, w < q < 2^62, ws = floor(w * 2^64 / q): Shoup's product
// with the truncated quotient (short by at most 2, so at most 2q above Shoup's [0, 2q)).  Two
// 32-bit multiplies cheaper than mul_shoup_lazy; the NTT butterflies use it with lazy ranges
// widened to match.
__device__ __forceinline__ uint64_t mul_shoup_lazy4(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
    return x * w - mulhi_trunc(x, ws) * q;
}

// The same with nq = 2^64 - q given: x w + Q nq = x w - Q q (mod 2^64), and as a sum of products
// the final 64-bit addition folds into the multiply-add chain instead of taking two integer adds.
__device__ __forceinline__ uint64_t mul_shoup_lazy4n(uint64_t x, uint64_t w, uint64_t ws, uint64_t nq) {
    return x * w + mulhi_trunc(x, ws) * nq;
}

__device__ __forceinline__ uint64_t mul_shoup(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
    return csub(mul_shoup_lazy(x, w, ws, q), q);
}

struct u128 {
    uint64_t lo, hi;
};

__device__ __forceinline__ u128 mul_wide(uint64_t a, uint64_t b) {
    u128 r;
    r.lo = a * b;
    r.hi = mulhi(a, b);
    return r;
}

// acc += a * b (128-bit)
__device__ __forceinline__ void mac(u128 &acc, uint64_t a, uint64_t b) {
    uint64_t lo = a * b, hi = mulhi(a, b);
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(acc.lo), "+l"(acc.hi) : "l"(lo), "l"(hi));
}

__device__ __forceinline__ void add128(u128 &acc, const u128 &b) {
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(acc.lo), "+l"(acc.hi) : "l"(b.lo), "l"(b.hi));
}

// x mod q for a 128-bit x with x < q * 2^64 (so the quotient fits one word), q < 2^62.
// The quotient estimate t = x.hi*mu_hi + hi(x.lo*mu_hi) + hi(x.hi*mu_lo) drops the low
// partial product and two carries, so with floor(x*mu/2^128) >= floor(x/q) - 1 it is short
// by at most 3: the remainder x - t*q lies in [0, 4q) and two conditional subtractions
// make it canonical.
__device__ __forceinline__ uint64_t reduce128(u128 x, const Mod &m) {
    uint64_t t = x.hi * m.mu_hi + mulhi(x.lo, m.mu_hi) + mulhi(x.hi, m.mu_lo);
    uint64_t r = x.lo - t * m.q;
    r = csub(r, 2 * m.q);
    return csub(r, m.q);
}

__device__ __forceinline__ uint64_t mul_mod(uint64_t a, uint64_t b, const Mod &m) { return reduce128(mul_wide(a, b), m); }

// x mod q for a 64-bit x (quotient estimate floor(x * floor(2^64/q) / 2^64), short by <= 1)
__device__ __forceinline__ uint64_t reduce64(uint64_t x, const Mod &m) {
    uint64_t t = mulhi(x, m.mu_hi);
    return csub(x - t * m.q, m.q);
}

}  // namespace pfg
