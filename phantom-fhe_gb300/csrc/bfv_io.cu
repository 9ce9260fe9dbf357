// bfv_io.cu — BFV plaintext side: batch encoding, symmetric encryption and decryption.
//
//   encode   PhantomBatchEncoder::encode (src/batchencoder.cu:51-92): slot i goes to coefficient
//            index_map[i] (negative int64 values + t), then the inverse NTT modulo t.
//   decode   PhantomBatchEncoder::decode (:100-118): the forward NTT modulo t, then slot i reads
//            coefficient index_map[i].
//   encrypt  PhantomSecretKey::encrypt_symmetric for BFV (src/secretkey.cu:463-485 with
//            encrypt_zero_symmetric :232-295, coefficient form, and
//            multiply_add_plain_with_scaling_variant, src/scalingvariant.cu:10-31):
//            c1 = iNTT(a), c0 = -(iNTT(a * s) + e) + (Q m + r) / t with r = (-Q m) mod t, i.e.
//            r * t^-1 mod q_i.
//   decrypt  bfv_decrypt (src/secretkey.cu:571-635): x = [c0 + iNTT(NTT(c1) * s)]_Ql, then HPS
//            scale-and-round (src/rns.cu:1519-1665) per coefficient: floor(t x / Ql) rounded, in
//            the reference's FP64 order.  Four variants as the reference chooses them from the
//            bit sizes (qMSB of the largest data prime, the limb count, t): the fractional sums
//            of x_i * frac(t QHatInv_i / q_i) either whole ("small") or with x_i split at
//            2^(qMSB / 2) ("large"), the integer sums reduced per term (Shoup) or only once
//            ("lazy").  nvcc fuses `sum += x * frac` into fma; the code calls __fma_rn so the
//            order is explicit.
#include <vector>

#include "context.cuh"
#include "launch.cuh"
#include "modarith.cuh"
#include "ops.hpp"

namespace pfg {

static int grid_of(size_t work) { return (int)std::min<size_t>((work + 255) / 256, kGridStrideBlocks); }

__global__ void bfv_encode_scatter(uint64_t *out, const uint64_t *in, size_t count, const uint32_t *map, uint64_t t,
                                   size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint64_t v = 0;
        if (i < count) {
            v = in[i];
            if (v >> 63) v += t;  // a negative slot value (two's complement) plus t
        }
        out[map[i]] = v;
    }
}

__global__ void bfv_decode_gather(uint64_t *out, const uint64_t *in, const uint32_t *map, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = in[map[i]];
}

// out = a * b mod q (element-wise over `limbs` limbs, table k)
__global__ void bfv_mul_kernel(uint64_t *out, const uint64_t *a, const uint64_t *b, const Mod *mods, int log_n,
                               size_t total) {
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x)
        out[x] = mul_mod(a[x], b[x], mods[x >> log_n]);
}

// c0 = -(c0 + e) + (r * t^-1 mod q_k), r = (m * (-Q mod t)) mod t
__global__ void bfv_encrypt_combine(uint64_t *c0, const int64_t *e, const uint64_t *m, const Mod *mods,
                                    const uint64_t *t_inv, uint64_t neg_q_t, uint64_t neg_q_t_s, uint64_t t, int log_n,
                                    size_t total) {
    const uint32_t nmask = (1u << log_n) - 1;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(x >> log_n);
        const uint64_t q = mods[k].q;
        const int64_t ev = e[x & nmask];
        const uint64_t em = ev < 0 ? (q - ((uint64_t)(-ev) % q)) % q : (uint64_t)ev % q;
        uint64_t v = add_mod(c0[x], em, q);
        v = v ? q - v : 0;
        const uint64_t r = mul_shoup(m[x & nmask], neg_q_t, neg_q_t_s, t);
        c0[x] = add_mod(v, mul_shoup(r, t_inv[2 * k], t_inv[2 * k + 1], q), q);
    }
}

// x = c0 + y (canonical), y = iNTT(NTT(c1) * s) computed in place in `y`
__global__ void bfv_add_kernel(uint64_t *y, const uint64_t *c0, const Mod *mods, int log_n, size_t total) {
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x)
        y[x] = add_mod(y[x], c0[x], mods[x >> log_n].q);
}

template <bool SPLIT, bool LAZY>
__global__ void bfv_decrypt_round(uint64_t *out, const uint64_t *x, const uint64_t *mt, const double *fr,
                                  const uint64_t *mtb, const double *frb, uint64_t t, int log_n, int l, int hf) {
    const size_t n = (size_t)1 << log_n;
    const double tinv = 1.0 / (double)t;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        double fs = 0.0;
        uint64_t is = 0;
        for (int i = 0; i < l; i++) {
            const uint64_t v = x[((size_t)i << log_n) + c];
            if constexpr (!SPLIT) {
                fs = __fma_rn((double)v, fr[i], fs);
                is += LAZY ? v * mt[2 * i] : mul_shoup(v, mt[2 * i], mt[2 * i + 1], t);
            } else {
                const uint64_t hi = v >> hf, lo = v & ((1ull << hf) - 1);
                fs = __fma_rn((double)lo, fr[i], fs);
                fs = __fma_rn((double)hi, frb[i], fs);
                if constexpr (LAZY) {
                    is += lo * mt[2 * i];
                    is += hi * mtb[2 * i];
                } else {
                    is += mul_shoup(lo, mt[2 * i], mt[2 * i + 1], t);
                    is += mul_shoup(hi, mtb[2 * i], mtb[2 * i + 1], t);
                }
            }
        }
        fs += (double)is;
        const uint64_t quot = (uint64_t)(fs * tinv);
        fs -= (double)(t * quot);
        out[c] = (uint64_t)llround(fs);
    }
}

static void need_batching(const Context &c) {
    if (c.scheme != kSchemeBFV || c.plain_tbl < 0)
        throw std::invalid_argument("batch encoding needs a BFV context with t prime and t = 1 mod 2N");
}

void bfv_encode(const Context &c, const uint64_t *values, size_t count, uint64_t *pt, cudaStream_t s) {
    need_batching(c);
    count_launch();
    bfv_encode_scatter<<<grid_of(c.n), 256, 0, s>>>(pt, values, count, c.bfv_index_map.as<uint32_t>(), c.t, c.n);
    ntt_inverse(c, pt, 1, 1, c.plain_tbl, s);
}

void bfv_decode(const Context &c, const uint64_t *pt, uint64_t *values, uint64_t *scratch, cudaStream_t s) {
    need_batching(c);
    cudaMemcpyAsync(scratch, pt, c.n * 8, cudaMemcpyDeviceToDevice, s);
    ntt_forward(c, scratch, 1, 1, c.plain_tbl, s);
    count_launch();
    bfv_decode_gather<<<grid_of(c.n), 256, 0, s>>>(values, scratch, c.bfv_index_map.as<uint32_t>(), c.n);
}

void bfv_encrypt_sk(const Context &c, const uint64_t *m, const uint64_t *s_ntt, const uint64_t *a, const int64_t *e,
                    uint64_t *out, cudaStream_t s) {
    const int l = c.nQ;
    const size_t lps = (size_t)l << c.log_n;
    uint64_t *c0 = out, *c1 = out + lps;
    count_launch();
    bfv_mul_kernel<<<grid_of(lps), 256, 0, s>>>(c0, a, s_ntt, c.d_mods.as<Mod>(), c.log_n, lps);
    cudaMemcpyAsync(c1, a, lps * 8, cudaMemcpyDeviceToDevice, s);
    ntt_inverse(c, out, 2, l, 0, s);
    count_launch();
    bfv_encrypt_combine<<<grid_of(lps), 256, 0, s>>>(c0, e, m, c.d_mods.as<Mod>(), c.bfv_t_inv.as<uint64_t>(),
                                                      c.neg_q_mod_t, c.neg_q_mod_t_shoup, c.t, c.log_n, lps);
}

void bfv_decrypt(const Context &c, const uint64_t *ct, int l, const uint64_t *s_ntt, uint64_t *pt, uint64_t *scratch,
                 cudaStream_t s) {
    const size_t lps = (size_t)l << c.log_n;
    cudaMemcpyAsync(scratch, ct + lps, lps * 8, cudaMemcpyDeviceToDevice, s);
    ntt_forward(c, scratch, 1, l, 0, s);
    count_launch();
    bfv_mul_kernel<<<grid_of(lps), 256, 0, s>>>(scratch, scratch, s_ntt, c.d_mods.as<Mod>(), c.log_n, lps);
    ntt_inverse(c, scratch, 1, l, 0, s);
    count_launch();
    bfv_add_kernel<<<grid_of(lps), 256, 0, s>>>(scratch, ct, c.d_mods.as<Mod>(), c.log_n, lps);
    // variant choice of DRNSTool::hps_decrypt_scale_and_round (src/rns.cu:1634-1665)
    int size_bits = 0;
    for (int v = l; v; v >>= 1) size_bits++;
    const bool split = c.q_msb + size_bits >= 52;
    const int hf = c.q_msb >> 1;
    const bool lazy = split ? (hf + c.t_msb + size_bits < 52) : (c.q_msb + c.t_msb + size_bits < 52);
    const size_t row = (size_t)(l - 1) * c.nQ;
    const uint64_t *mt = c.dec_mod_t.as<uint64_t>() + 2 * row, *mtb = c.dec_mod_t_b.as<uint64_t>() + 2 * row;
    const double *fr = c.dec_frac.as<double>() + row, *frb = c.dec_frac_b.as<double>() + row;
    count_launch();
    const int g = grid_of(c.n);
    if (split && lazy)
        bfv_decrypt_round<true, true><<<g, 256, 0, s>>>(pt, scratch, mt, fr, mtb, frb, c.t, c.log_n, l, hf);
    else if (split)
        bfv_decrypt_round<true, false><<<g, 256, 0, s>>>(pt, scratch, mt, fr, mtb, frb, c.t, c.log_n, l, hf);
    else if (lazy)
        bfv_decrypt_round<false, true><<<g, 256, 0, s>>>(pt, scratch, mt, fr, mtb, frb, c.t, c.log_n, l, hf);
    else
        bfv_decrypt_round<false, false><<<g, 256, 0, s>>>(pt, scratch, mt, fr, mtb, frb, c.t, c.log_n, l, hf);
}

}  // namespace pfg
