// ops_linear.cu — plaintext-ciphertext products, additions, rotations with NAF fallback, the
// baby-step/giant-step matrix-vector driver, and secret-key encryption / decryption / key
// generation for CKKS (randomness supplied by the caller).
//
// Reference behaviour restated:
//   multiply_plain (CKKS, NTT form), add_inplace          src/evaluate.cu (ckks branches)
//   rotate_inplace with NAF decomposition                   src/evaluate.cu:1633-1668
//   bsgs_complete_from_cpu (baby rotations, inner sums of
//   multiply_plain, giant rotations by g*G, rescale)        python/src/binding.cu:507-595
//   encrypt_symmetric / decrypt / generate_one_kswitch_key  src/secretkey.cu:130-341
#include <algorithm>
#include <cstdlib>
#include <stdexcept>

#include "host_tables.hpp"
#include "launch.cuh"
#include "ops.hpp"

namespace pfg {

static int grid_lin(size_t work) { return (int)std::min<size_t>((work + 255) / 256, kGridStrideBlocks); }

// out[p][e] = ct[p][e] * pt[e]  (p = 0, 1; e over l limbs x N)
__global__ void mul_plain_kernel(uint64_t *out, const uint64_t *ct, const uint64_t *pt, const Mod *mods, int log_n,
                                 size_t lps) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < lps; e += (size_t)gridDim.x * blockDim.x) {
        const Mod m = mods[e >> log_n];
        const uint64_t p = pt[e];
        out[e] = mul_mod(ct[e], p, m);
        out[lps + e] = mul_mod(ct[lps + e], p, m);
    }
}

// out = a + b over `total` words of l-limb polynomials
__global__ void add_kernel(uint64_t *out, const uint64_t *a, const uint64_t *b, const Mod *mods, int log_n,
                           size_t lps, size_t total) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const uint64_t q = mods[(e % lps) >> log_n].q;
        out[e] = add_mod(a[e], b[e], q);
    }
}

constexpr int kMaxTerms = 32;
struct MulPlainTerms {
    const uint64_t *ct[kMaxTerms];
    const uint64_t *pt[kMaxTerms];
    int count;
};

// out[p][e] (+)= sum_t ct_t[p][e] * pt_t[e]: the same words as a chain of multiply_plain and
// add_inplace calls (exact modular arithmetic, 128-bit accumulation reduced every 7 terms).
__global__ void mul_plain_sum_kernel(uint64_t *out, MulPlainTerms terms, const Mod *mods, int log_n, size_t lps,
                                     bool accumulate) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < lps; e += (size_t)gridDim.x * blockDim.x) {
        const Mod m = mods[e >> log_n];
        u128 a0{0, 0}, a1{0, 0};
        int n = 0;
        for (int t = 0; t < terms.count; t++) {
            if (n == 7) {
                a0 = u128{reduce128(a0, m), 0};
                a1 = u128{reduce128(a1, m), 0};
                n = 1;
            }
            const uint64_t p = terms.pt[t][e];
            mac(a0, terms.ct[t][e], p);
            mac(a1, terms.ct[t][lps + e], p);
            n++;
        }
        uint64_t r0 = reduce128(a0, m), r1 = reduce128(a1, m);
        if (accumulate) {
            r0 = add_mod(r0, out[e], m.q);
            r1 = add_mod(r1, out[lps + e], m.q);
        }
        out[e] = r0;
        out[lps + e] = r1;
    }
}

void ckks_multiply_plain(const Context &c, const uint64_t *ct, const uint64_t *pt, uint64_t *out, int l,
                         cudaStream_t s) {
    const size_t lps = (size_t)l << c.log_n;
    count_launch();
    mul_plain_kernel<<<grid_lin(lps), 256, 0, s>>>(out, ct, pt, c.d_mods.as<Mod>(), c.log_n, lps);
}

void ckks_add(const Context &c, const uint64_t *a, const uint64_t *b, uint64_t *out, int l, int polys,
              cudaStream_t s) {
    const size_t lps = (size_t)l << c.log_n;
    count_launch();
    add_kernel<<<grid_lin(lps * polys), 256, 0, s>>>(out, a, b, c.d_mods.as<Mod>(), c.log_n, lps, lps * polys);
}

static void mul_plain_sum(const Context &c, uint64_t *out, const std::vector<const uint64_t *> &cts,
                          const std::vector<const uint64_t *> &pts, int l, bool accumulate, cudaStream_t s) {
    const size_t lps = (size_t)l << c.log_n;
    for (size_t t0 = 0; t0 < cts.size(); t0 += kMaxTerms) {
        MulPlainTerms terms{};
        terms.count = (int)std::min<size_t>(kMaxTerms, cts.size() - t0);
        for (int i = 0; i < terms.count; i++) {
            terms.ct[i] = cts[t0 + i];
            terms.pt[i] = pts[t0 + i];
        }
        count_launch();
        mul_plain_sum_kernel<<<grid_lin(lps), 256, 0, s>>>(out, terms, c.d_mods.as<Mod>(), c.log_n, lps,
                                                           accumulate || t0 > 0);
    }
}

// rotate_inplace with the reference's NAF fallback (src/evaluate.cu:1633-1663).
void ckks_rotate(Context &c, const Workspace &w, uint64_t *ct, int l, int step,
                 const uint64_t *const *const *galois_keys, cudaStream_t s) {
    const uint32_t elt = host::elt_from_step(step, c.n);
    for (size_t i = 0; i < c.galois_elts.size(); i++) {
        if (c.galois_elts[i] != elt) continue;
        if (!galois_keys[i]) throw std::invalid_argument("Galois key not present");
        ckks_apply_galois(c, w, ct, l, c.perm_table(elt), galois_keys[i], s);
        return;
    }
    const auto naf = host::naf(step);
    if (naf.size() == 1) throw std::invalid_argument("Galois key not present");
    for (int t : naf)
        if ((uint64_t)std::abs(t) != (c.n >> 1)) ckks_rotate(c, w, ct, l, t, galois_keys, s);
}

// Scratch of the matrix-vector driver: (G + 1) ciphertexts at the key level's data size.
size_t bsgs_scratch_words(const Context &c, int G) { return (size_t)(G + 1) * 2 * c.nQ * c.n; }

// Scratch per item of the batched form: the babies and one inner sum per giant step (and at least
// the single call's, which runs when the batch falls back to it).
size_t bsgs_batch_scratch_words(const Context &c, int G, int B) {
    return (size_t)std::max(G - 1 + B, G + 1) * 2 * c.nQ * c.n;
}

void ckks_bsgs_matvec(Context &c, const Workspace &w, uint64_t *scratch, const uint64_t *ct, int l,
                      const uint64_t *diags, int D, int G, int B, const uint64_t *const *const *galois_keys,
                      uint64_t *out, bool hoisted, cudaStream_t s, int diag_limbs) {
    const size_t lps = (size_t)l << c.log_n, cts = 2 * lps;
    // one diagonal every diag_limbs limbs (its first l are read); 0: the diagonals are [D][l][N]
    const size_t dstride = (size_t)(diag_limbs > 0 ? diag_limbs : l) << c.log_n;
    // babies[0] = ct; babies[b] (b >= 1) in scratch; then `inner` and `result`
    std::vector<const uint64_t *> babies(G);
    babies[0] = ct;
    uint64_t *area = scratch;
    std::vector<uint64_t *> outs;
    for (int b = 1; b < G; b++) {
        babies[b] = area;
        outs.push_back(area);
        area += cts;
    }
    uint64_t *inner = area, *result = area + cts;
    auto terms = [&](int g, std::vector<const uint64_t *> &cv, std::vector<const uint64_t *> &pv) {
        cv.clear();
        pv.clear();
        for (int b = 0; b < G; b++) {
            const int k = g * G + b;
            if (k >= D) break;
            cv.push_back(babies[b]);
            pv.push_back(diags + (size_t)k * dstride);
        }
    };
    std::vector<const uint64_t *> cv, pv;
    if (hoisted) {
        // baby rotations share one mod-up; giant steps by Horner's rule, all rotations by G:
        // sum_g rot_{gG}(inner_g) = inner_0 + rot_G(inner_1 + rot_G(inner_2 + ...)).
        if (G > 1) {
            std::vector<StepKey> steps;
            for (int b = 1; b < G; b++) {
                const uint32_t elt = host::elt_from_step(b, c.n);
                int idx = -1;
                for (size_t i = 0; i < c.galois_elts.size(); i++)
                    if (c.galois_elts[i] == elt) idx = (int)i;
                if (idx < 0 || !galois_keys[idx]) throw std::invalid_argument("Galois key not present for a baby step");
                steps.push_back(StepKey{c.perm_table(elt), galois_keys[idx]});
            }
            ckks_rotations_hoisted(c, w, ct, l, steps, outs, s);
        }
        bool first = true;
        for (int g = B - 1; g >= 0; g--) {
            terms(g, cv, pv);
            if (!first) ckks_rotate(c, w, result, l, G, galois_keys, s);
            if (!cv.empty()) {
                mul_plain_sum(c, result, cv, pv, l, !first, s);
                first = false;
            }
        }
    } else {
        // the reference's loop: separate rotations, giant rotations by g * G
        for (int b = 1; b < G; b++) {
            cudaMemcpyAsync(outs[b - 1], ct, cts * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
            ckks_rotate(c, w, outs[b - 1], l, b, galois_keys, s);
        }
        bool have = false;
        for (int g = 0; g < B; g++) {
            terms(g, cv, pv);
            if (cv.empty()) continue;
            mul_plain_sum(c, g == 0 ? result : inner, cv, pv, l, false, s);
            if (g > 0) {
                ckks_rotate(c, w, inner, l, g * G, galois_keys, s);
                ckks_add(c, result, inner, result, l, 2, s);
            }
            have = true;
        }
        if (!have) throw std::invalid_argument("no diagonals");
    }
    ckks_rescale(c, w, result, out, 2, l, s);
}

// ------------------------------------------------------------------ encryption and keys

// dst[k][i] = e[i] mod q_k (e signed) for `limbs` limbs with table index tbl(k)
__global__ void small_to_rns(uint64_t *dst, const int64_t *e, const Mod *mods, int log_n, int limbs, int split,
                             int shift) {
    const size_t total = (size_t)limbs << log_n;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(x >> log_n);
        const uint64_t q = mods[k + (k >= split ? shift : 0)].q;
        const int64_t v = e[x & (((size_t)1 << log_n) - 1)];
        const uint64_t mag = (uint64_t)(v < 0 ? -v : v) % q;
        dst[x] = (v < 0 && mag) ? q - mag : mag;
    }
}

// c0 = m - (a*s + e) (e already in NTT form in c0), c1 = a: encrypt_zero_symmetric's
// [-(as + e), a] (src/secretkey.cu:232-295) plus the plaintext, as encrypt_symmetric adds it.
__global__ void encrypt_combine(uint64_t *c0, uint64_t *c1, const uint64_t *m, const uint64_t *a, const uint64_t *s,
                                const Mod *mods, int log_n, size_t lps) {
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < lps; x += (size_t)gridDim.x * blockDim.x) {
        const Mod md = mods[x >> log_n];
        const uint64_t ase = add_mod(mul_mod(a[x], s[x], md), c0[x], md.q);
        c0[x] = sub_mod(m ? m[x] : 0, ase, md.q);
        c1[x] = a[x];
    }
}

__global__ void decrypt_kernel(uint64_t *m, const uint64_t *c0, const uint64_t *c1, const uint64_t *s, const Mod *mods,
                               int log_n, size_t lps) {
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < lps; x += (size_t)gridDim.x * blockDim.x) {
        const Mod md = mods[x >> log_n];
        m[x] = add_mod(c0[x], mul_mod(c1[x], s[x], md), md.q);
    }
}

void ckks_encrypt_sk(const Context &c, const uint64_t *m, const uint64_t *s_ntt, const uint64_t *a, const int64_t *e,
                     uint64_t *out, int l, cudaStream_t st) {
    const size_t lps = (size_t)l << c.log_n;
    count_launch();
    small_to_rns<<<grid_lin(lps), 256, 0, st>>>(out, e, c.d_mods.as<Mod>(), c.log_n, l, 1 << 30, 0);
    ntt_forward(c, out, 1, l, 0, st);
    count_launch();
    encrypt_combine<<<grid_lin(lps), 256, 0, st>>>(out, out + lps, m, a, s_ntt, c.d_mods.as<Mod>(), c.log_n, lps);
}

void ckks_decrypt(const Context &c, const uint64_t *ct, const uint64_t *s_ntt, uint64_t *m, int l, cudaStream_t st) {
    const size_t lps = (size_t)l << c.log_n;
    count_launch();
    decrypt_kernel<<<grid_lin(lps), 256, 0, st>>>(m, ct, ct + lps, s_ntt, c.d_mods.as<Mod>(), c.log_n, lps);
}

// key[d] = (-(a_d s + e_d) + (P mod q_j) s_from on digit d's Q limbs, a_d) over all QP limbs
__global__ void kswitch_key_combine(uint64_t *key, const uint64_t *a, size_t a_stride, const uint64_t *e_ntt,
                                    const uint64_t *s, const uint64_t *s_from, const uint64_t *p_mod_q,
                                    const Mod *mods, int log_n, int qp, int nQ, int alpha, int dnum) {
    const size_t qpn = (size_t)qp << log_n, total = (size_t)dnum * qpn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const int d = (int)(x / qpn);
        const size_t r = x - (size_t)d * qpn;
        const int j = (int)(r >> log_n);
        const Mod md = mods[j];
        const uint64_t av = a[(size_t)d * a_stride + r];  // may alias key's second half (same word)
        uint64_t b = sub_mod(0, add_mod(mul_mod(av, s[r], md), e_ntt[x], md.q), md.q);
        if (j < nQ && j >= d * alpha && j < d * alpha + alpha) b = add_mod(b, mul_mod(p_mod_q[j], s_from[r], md), md.q);
        key[(size_t)d * 2 * qpn + r] = b;
        key[(size_t)d * 2 * qpn + qpn + r] = av;
    }
}

__global__ void square_kernel(uint64_t *out, const uint64_t *x, const Mod *mods, int log_n, size_t total) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        out[i] = mul_mod(x[i], x[i], mods[i >> log_n]);
}

__global__ void permute_kernel(uint64_t *dst, const uint64_t *src, const uint32_t *perm, int log_n, size_t total) {
    const uint32_t nmask = (1u << log_n) - 1;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        dst[e] = src[(e & ~(size_t)nmask) + __ldg(perm + ((uint32_t)e & nmask))];
}

// s_from: 0 = relinearisation (s^2), else the Galois element (sigma(s)).  `scratch` holds
// (dnum + 1) x QP x N + 64 words.
void small_to_rns_launch(const Context &c, uint64_t *dst, const int64_t *e, int limbs, cudaStream_t st) {
    count_launch();
    small_to_rns<<<grid_lin((size_t)limbs << c.log_n), 256, 0, st>>>(dst, e, c.d_mods.as<Mod>(), c.log_n, limbs,
                                                                     1 << 30, 0);
}

void kswitch_keygen(Context &c, uint32_t elt, const uint64_t *s_ntt, const uint64_t *a, size_t a_stride,
                    const int64_t *e, uint64_t *key, uint64_t *scratch, cudaStream_t st) {
    const int qp = c.nQ + c.nP, dnum = c.beta(c.nQ);
    const size_t qpn = (size_t)qp << c.log_n;
    uint64_t *s_from = scratch, *e_ntt = scratch + qpn;
    count_launch();
    if (elt == 0)
        square_kernel<<<grid_lin(qpn), 256, 0, st>>>(s_from, s_ntt, c.d_mods.as<Mod>(), c.log_n, qpn);
    else
        permute_kernel<<<grid_lin(qpn), 256, 0, st>>>(s_from, s_ntt, c.perm_table(elt), c.log_n, qpn);
    for (int d = 0; d < dnum; d++) {
        count_launch();
        small_to_rns<<<grid_lin(qpn), 256, 0, st>>>(e_ntt + d * qpn, e + ((size_t)d << c.log_n), c.d_mods.as<Mod>(),
                                                    c.log_n, qp, 1 << 30, 0);
    }
    ntt_forward(c, e_ntt, dnum, qp, 0, st);
    std::vector<uint64_t> pq(c.nQ);
    for (int j = 0; j < c.nQ; j++) {
        std::vector<uint64_t> P(c.mods.begin() + c.nQ, c.mods.begin() + qp);
        pq[j] = host::prod_mod(P, -1, c.mods[j]);
    }
    // P mod q_j travels after the dnum + 1 polynomials of the scratch
    uint64_t *pq_d = scratch + (size_t)(dnum + 1) * qpn;
    cudaMemcpyAsync(pq_d, pq.data(), c.nQ * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
    count_launch();
    kswitch_key_combine<<<grid_lin((size_t)dnum * qpn), 256, 0, st>>>(key, a, a_stride, e_ntt, s_ntt, s_from, pq_d,
                                                                       c.d_mods.as<Mod>(), c.log_n, qp, c.nQ, c.nP,
                                                                       dnum);
    cudaStreamSynchronize(st);  // the host copy of P mod q_j must outlive the transfer
}

}  // namespace pfg
