// prng.cu — the reference's device samplers, bit for bit (src/prng.cu:17-244), and key
// generation from seeds (PhantomSecretKey::gen_secretkey, generate_one_kswitch_key,
// src/secretkey.cu:297-390).
//
// Generator.  The Salsa20/20 core (D. J. Bernstein's published design: ten double rounds of
// column and row quarter-rounds with rotations 7, 9, 13, 18, then the input state added back)
// over a 16-word state laid out as the reference lays it out: words 0-7 and 10-15 are the
// first 56 bytes of the 64-byte seed (little-endian), words 8-9 the 64-bit nonce, and there are
// no constant words.  One invocation gives 64 bytes: the 16 output words, little-endian.
//
// Samplers (the reference's nonce scheme, so the same seed gives the same polynomial):
//   uniform  — per limb k and group g of 8 coefficients, nonce k * N/8 + g; the block's eight
//              64-bit words are taken in order, a word above 2^64 - 1 - ((2^64 - 1) mod q) - 1 is
//              rejected by drawing a whole new block with nonce (k * N/8 + g) + tries * N * limbs
//              and continuing at the same word position; accepted words are reduced mod q.
//   ternary  — per coefficient i, nonce i: (byte 0 mod 3) - 1, the same on every limb.
//   cbd      — per coefficient i, nonce i: hw(b0) + hw(b1) + hw(b2 & 31) - hw(b3) - hw(b4) -
//              hw(b5 & 31), the same on every limb (centred binomial, sigma about 3.2).
#include <cstring>
#include <vector>

#include "capi_internal.hpp"
#include "context.cuh"
#include "launch.cuh"
#include "ops.hpp"

namespace pfg {

struct PrngKey {
    uint32_t w[14];
};

__device__ __forceinline__ uint32_t rotl32(uint32_t v, int c) { return __funnelshift_l(v, v, c); }

__device__ __forceinline__ void quarter(uint32_t &a, uint32_t &b, uint32_t &c, uint32_t &d) {
    b ^= rotl32(a + d, 7);
    c ^= rotl32(b + a, 9);
    d ^= rotl32(c + b, 13);
    a ^= rotl32(d + c, 18);
}

__device__ void salsa_block(const PrngKey &key, uint64_t nonce, uint32_t (&out)[16]) {
    uint32_t s[16];
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = key.w[i];
    s[8] = (uint32_t)nonce;
    s[9] = (uint32_t)(nonce >> 32);
#pragma unroll
    for (int i = 0; i < 6; i++) s[10 + i] = key.w[8 + i];
    uint32_t x[16];
#pragma unroll
    for (int i = 0; i < 16; i++) x[i] = s[i];
#pragma unroll 1
    for (int r = 0; r < 10; r++) {
        quarter(x[0], x[4], x[8], x[12]);  // columns
        quarter(x[5], x[9], x[13], x[1]);
        quarter(x[10], x[14], x[2], x[6]);
        quarter(x[15], x[3], x[7], x[11]);
        quarter(x[0], x[1], x[2], x[3]);  // rows
        quarter(x[5], x[6], x[7], x[4]);
        quarter(x[10], x[11], x[8], x[9]);
        quarter(x[15], x[12], x[13], x[14]);
    }
#pragma unroll
    for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}

// Retry cap of the uniform sampler's rejection loop: a word is rejected with probability
// below q / 2^64 <= 1/8, so the cap is never reached by a real seed; reaching it sets bit 8 of
// the status word and writes 0 instead of looping on.
constexpr int kUniformMaxTries = 4096;

__global__ void sample_uniform_kernel(uint64_t *out, PrngKey key, const Mod *mods, int log_n, int limbs,
                                      unsigned *status) {
    const size_t per_limb = (size_t)1 << (log_n - 3), total = per_limb * limbs;
    const uint64_t retry = (uint64_t)limbs << log_n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const Mod m = mods[t / per_limb];
        const uint64_t limit = ~0ull - (~0ull % m.q) - 1;
        uint32_t w[16];
        salsa_block(key, t, w);
        int tries = 1;
        for (int i = 0; i < 8; i++) {
            uint64_t v = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
            while (v > limit) {
                if (tries >= kUniformMaxTries) {
                    atomicOr(status, 8u);
                    v = 0;
                    break;
                }
                salsa_block(key, t + (uint64_t)tries * retry, w);
                tries++;
                v = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
            }
            out[t * 8 + i] = reduce64(v, m);
        }
    }
}

// kind 0: ternary, 1: centred binomial; out[i] as a signed integer
__global__ void sample_small_kernel(int64_t *out, PrngKey key, int log_n, int kind) {
    const size_t n = (size_t)1 << log_n;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t w[16];
        salsa_block(key, i, w);
        const uint32_t b0 = w[0] & 0xFF, b1 = (w[0] >> 8) & 0xFF, b2 = (w[0] >> 16) & 0xFF, b3 = w[0] >> 24;
        const uint32_t b4 = w[1] & 0xFF, b5 = (w[1] >> 8) & 0xFF;
        if (kind == 0)
            out[i] = (int64_t)(b0 % 3) - 1;
        else
            out[i] = (int64_t)(__popc(b0) + __popc(b1) + __popc(b2 & 0x1F)) -
                     (int64_t)(__popc(b3) + __popc(b4) + __popc(b5 & 0x1F));
    }
}

static PrngKey key_of(const uint8_t *seed) {
    PrngKey k;
    for (int i = 0; i < 14; i++)
        k.w[i] = (uint32_t)seed[4 * i] | ((uint32_t)seed[4 * i + 1] << 8) | ((uint32_t)seed[4 * i + 2] << 16) |
                 ((uint32_t)seed[4 * i + 3] << 24);
    return k;
}

static int grid_for(size_t work) { return (int)std::min<size_t>((work + 255) / 256, kGridStrideBlocks); }

void sample_uniform(const Context &c, const uint8_t *seed, int limbs, uint64_t *out, cudaStream_t s) {
    count_launch();
    sample_uniform_kernel<<<grid_for((size_t)limbs << (c.log_n - 3)), 256, 0, s>>>(
            out, key_of(seed), c.d_mods.as<Mod>(), c.log_n, limbs, c.d_status.as<unsigned>());
}

void sample_small(const Context &c, const uint8_t *seed, int kind, int64_t *out, cudaStream_t s) {
    count_launch();
    sample_small_kernel<<<grid_for(c.n), 256, 0, s>>>(out, key_of(seed), c.log_n, kind);
}

// gen_secretkey (src/secretkey.cu:343-380): ternary from the seed over every QP limb, NTT form.
// `scratch` holds N int64.
void secret_key_from_seed(const Context &c, const uint8_t *seed, uint64_t *s_ntt, int64_t *scratch, cudaStream_t s) {
    const int qp = c.nQ + c.nP;
    sample_small(c, seed, 0, scratch, s);
    small_to_rns_launch(c, s_ntt, scratch, qp, s);
    ntt_forward(c, s_ntt, 1, qp, 0, s);
}

// generate_one_kswitch_key with the reference's samplers: digit d's a from seeds_a[d] (uniform
// over QP, taken as NTT form, written straight into the key's second half) and its error from
// seeds_e[d] (centred binomial, then NTT), combined as kswitch_keygen does.
void kswitch_keygen_seeded(Context &c, uint32_t elt, const uint64_t *s_ntt, const uint8_t *seeds_a,
                           const uint8_t *seeds_e, uint64_t *key, uint64_t *scratch, cudaStream_t s) {
    const int qp = c.nQ + c.nP, dnum = c.beta(c.nQ);
    const size_t qpn = (size_t)qp << c.log_n;
    int64_t *e = reinterpret_cast<int64_t *>(scratch + (size_t)(dnum + 1) * qpn + 64);
    for (int d = 0; d < dnum; d++) {
        sample_uniform(c, seeds_a + 64 * d, qp, key + (size_t)d * 2 * qpn + qpn, s);
        sample_small(c, seeds_e + 64 * d, 1, e + ((size_t)d << c.log_n), s);
    }
    kswitch_keygen(c, elt, s_ntt, key + qpn, 2 * qpn, e, key, scratch, s);
}

}  // namespace pfg
