// context.cu — builds and uploads the device tables (see context.cuh).
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "context.cuh"
#include "host_tables.hpp"

namespace pfg {

static void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

DevBuf::~DevBuf() {
    if (p) cudaFree(p);
}

void DevBuf::upload(const void *src, size_t n) {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = n;
    if (!n) return;
    check(cudaMalloc(&p, n), "cudaMalloc(context table)");
    check(cudaMemcpy(p, src, n, cudaMemcpyHostToDevice), "cudaMemcpy(context table)");
}

template <class T>
static void up(DevBuf &b, const std::vector<T> &v) {
    b.upload(v.data(), v.size() * sizeof(T));
}

// bf16 bit pattern of an integer below 256 (exact: at most 8 significant bits)
static uint16_t bf16_of_byte(unsigned v) {
    const float f = (float)v;
    uint32_t bits;
    std::memcpy(&bits, &f, 4);
    return (uint16_t)(bits >> 16);
}

// element (row, k) of a K-major, no-swizzle tensor-core operand with kpad columns:
// 8-row x 16-byte core matrices, K neighbours 128 B apart, 8-row blocks kpad / 8 x 128 B apart
static size_t canon_index(int row, int k, int kpad) {
    const size_t byte = (size_t)(row & 7) * 16 + (size_t)(row >> 3) * (kpad / 8) * 128 + (size_t)(k & 7) * 2 +
                        (size_t)(k >> 3) * 128;
    return byte / 2;
}

const uint32_t *Context::perm_table(uint32_t elt) {
    std::lock_guard<std::mutex> g(perm_mu);
    auto it = perms.find(elt);
    if (it != perms.end()) return it->second->as<uint32_t>();
    auto perm = host::galois_perm(log_n, elt);
    auto buf = std::make_unique<DevBuf>();
    up(*buf, perm);
    const uint32_t *p = buf->as<uint32_t>();
    perms.emplace(elt, std::move(buf));
    return p;
}

// PhantomBatchEncoder::populate_matrix_reps_index_map (src/batchencoder.cu:25-49), the BFV
// scaling-variant constants (src/rns.cu negQl_mod_t, tInv_mod_q) and the HPS decryption tables
// (src/rns.cu:583-668), per data level.
static uint64_t reverse_low_bits(uint64_t v, int bits) {
    uint64_t r = 0;
    for (int i = 0; i < bits; i++) r |= ((v >> i) & 1) << (bits - 1 - i);
    return r;
}

static int bit_count(uint64_t v) {
    int b = 0;
    while (v) {
        b++;
        v >>= 1;
    }
    return b;
}

static void bfv_plain_tables(Context &c, const std::vector<uint64_t> &Q) {
    using namespace host;
    using u128 = unsigned __int128;
    const uint64_t n = c.n, t = c.t;
    const int nQ = c.nQ;
    if (c.plain_tbl >= 0) {
        std::vector<uint32_t> map(n);
        const uint64_t m = 2 * n, half = n / 2;
        uint64_t pos = 1;
        for (uint64_t i = 0; i < half; i++) {
            map[i] = (uint32_t)reverse_low_bits((pos - 1) >> 1, c.log_n);
            map[half + i] = (uint32_t)reverse_low_bits((m - pos - 1) >> 1, c.log_n);
            pos = (pos * 5) & (m - 1);
        }
        up(c.bfv_index_map, map);
    }
    uint64_t qt = 1;
    for (uint64_t q : Q) qt = mulmod(qt, q % t, t);
    c.neg_q_mod_t = qt ? t - qt : 0;
    c.neg_q_mod_t_shoup = shoup(c.neg_q_mod_t, t);
    std::vector<uint64_t> tinv(2 * nQ);
    for (int i = 0; i < nQ; i++) {
        tinv[2 * i] = invmod(t % Q[i], Q[i]);
        tinv[2 * i + 1] = shoup(tinv[2 * i], Q[i]);
    }
    up(c.bfv_t_inv, tinv);
    uint64_t qmax = 0;
    for (uint64_t q : Q) qmax = std::max(qmax, q);
    c.q_msb = bit_count(qmax);
    c.t_msb = bit_count(t);
    const int hf = c.q_msb >> 1;
    std::vector<uint64_t> mt((size_t)nQ * nQ * 2, 0), mtb((size_t)nQ * nQ * 2, 0);
    std::vector<double> fr((size_t)nQ * nQ, 0.0), frb((size_t)nQ * nQ, 0.0);
    for (int l = 1; l <= nQ; l++) {
        const std::vector<uint64_t> Ql(Q.begin(), Q.begin() + l);
        for (int i = 0; i < l; i++) {
            const uint64_t q = Q[i], hat_inv = invmod(prod_mod(Ql, i, q), q);
            const size_t r = (size_t)(l - 1) * nQ + i;
            const u128 v = (u128)t * hat_inv;
            mt[2 * r] = (uint64_t)((v / q) % t);
            mt[2 * r + 1] = shoup(mt[2 * r], t);
            fr[r] = (double)(uint64_t)(v % q) / (double)q;
            const uint64_t hat_inv_b = (uint64_t)(((u128)hat_inv << hf) % q);
            const u128 vb = (u128)t * hat_inv_b;
            mtb[2 * r] = (uint64_t)((vb / q) % t);
            mtb[2 * r + 1] = shoup(mtb[2 * r], t);
            frb[r] = (double)(uint64_t)(vb % q) / (double)q;
        }
    }
    up(c.dec_mod_t, mt);
    up(c.dec_mod_t_b, mtb);
    up(c.dec_frac, fr);
    up(c.dec_frac_b, frb);
}

std::unique_ptr<Context> make_context(int scheme, int mul_tech, uint64_t n, const std::vector<uint64_t> &coeff_modulus,
                                      int special_size, uint64_t plain_modulus,
                                      const std::vector<uint32_t> &galois_elts) {
    using namespace host;
    auto c = std::make_unique<Context>();
    int log_n = 0;
    while ((uint64_t(1) << log_n) < n) log_n++;
    if ((uint64_t(1) << log_n) != n || log_n < 12 || log_n > 17)
        throw std::invalid_argument("poly_modulus_degree must be a power of two in [2^12, 2^17]");
    if (coeff_modulus.size() < 2 || (int)coeff_modulus.size() <= special_size || special_size < 0)
        throw std::invalid_argument("coefficient modulus needs at least one data prime and two primes in total");
    if (coeff_modulus.size() > 64) throw std::invalid_argument("at most 64 primes are supported");
    if (scheme != kSchemeCKKS && scheme != kSchemeBFV) throw std::invalid_argument("unsupported scheme");
    for (uint64_t q : coeff_modulus) {
        if (q >> 61 || !is_prime(q) || (q - 1) % (2 * n))
            throw std::invalid_argument("every modulus must be a prime below 2^61 with q = 1 mod 2N");
    }
    c->scheme = scheme;
    c->mul_tech = mul_tech;
    c->log_n = log_n;
    c->n = n;
    c->nP = special_size;
    c->nQ = (int)coeff_modulus.size() - special_size;
    c->t = plain_modulus;
    c->mods = coeff_modulus;
    const int nQ = c->nQ, nP = c->nP;
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    c->device = dev;
    c->noalloc_scratch = noalloc_scratch_address(&c->noalloc_words);
    check(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev), "multiprocessor count");
    check(cudaDeviceGetAttribute(&c->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "shared memory limit");
    {
        const unsigned zero = 0;
        c->d_status.upload(&zero, sizeof(zero));
    }
    // the byte-plane GEMM is exact for K = 8 alpha <= 48 (every plane sum stays below 2^22)
    c->tc_avail = nP >= 1 && nP <= 6;
    c->tc_on = c->tc_avail;
    c->tc_kpad = (8 * nP + 15) / 16 * 16;
    std::vector<uint64_t> Q(coeff_modulus.begin(), coeff_modulus.begin() + nQ);
    std::vector<uint64_t> P(coeff_modulus.begin() + nQ, coeff_modulus.end());

    std::vector<uint64_t> R;
    if (scheme == kSchemeBFV) {
        if (!plain_modulus) throw std::invalid_argument("BFV needs a plain modulus");
        if (mul_tech != kMulHPS) throw std::invalid_argument("only mul_tech hps is supported for BFV");
        uint64_t minq = Q[0];
        for (uint64_t q : Q) minq = std::min(minq, q);
        R = get_primes_below(n, minq, nQ + 1);
        c->nR = nQ + 1;
        c->mods.insert(c->mods.end(), R.begin(), R.end());
    }

    // moduli and NTT tables for QP and R
    const size_t np = c->mods.size();
    std::vector<uint64_t> modw(3 * np), tw, itw, all_tw, all_itw, ninv(2 * np);
    all_tw.reserve(np * 2 * n);
    all_itw.reserve(np * 2 * n);
    for (size_t i = 0; i < np; i++) {
        modw[3 * i] = c->mods[i];
        barrett(c->mods[i], modw[3 * i + 1], modw[3 * i + 2]);
        ntt_tables(log_n, c->mods[i], tw, itw, ninv[2 * i], ninv[2 * i + 1]);
        all_tw.insert(all_tw.end(), tw.begin(), tw.end());
        all_itw.insert(all_itw.end(), itw.begin(), itw.end());
    }
    // BFV batching: t prime and 1 mod 2N gives the plaintext NTT (gpu_plain_tables)
    if (scheme == kSchemeBFV && plain_modulus > 2 && plain_modulus % (2 * n) == 1 && host::is_prime(plain_modulus)) {
        c->plain_tbl = (int)np;
        modw.push_back(plain_modulus);
        modw.push_back(0);
        modw.push_back(0);
        barrett(plain_modulus, modw[3 * np + 1], modw[3 * np + 2]);
        ninv.resize(2 * np + 2);
        ntt_tables(log_n, plain_modulus, tw, itw, ninv[2 * np], ninv[2 * np + 1]);
        all_tw.insert(all_tw.end(), tw.begin(), tw.end());
        all_itw.insert(all_itw.end(), itw.begin(), itw.end());
    }
    up(c->d_mods, modw);
    up(c->d_tw, all_tw);
    up(c->d_itw, all_itw);
    up(c->d_ninv, ninv);
    if (scheme == kSchemeBFV) bfv_plain_tables(*c, Q);

    std::vector<uint64_t> pmat((size_t)nQ * nP), pinv(2 * nQ);
    if (nP > 0) {
        // mod-down constants (rns.cu:107-124, BaseConverter(P -> Ql), host/rns.cu:438-498)
        std::vector<uint64_t> phi(2 * nP);
        for (int k = 0; k < nP; k++) {
            phi[2 * k] = invmod(prod_mod(P, k, P[k]), P[k]);
            phi[2 * k + 1] = shoup(phi[2 * k], P[k]);
        }
        for (int j = 0; j < nQ; j++) {
            for (int k = 0; k < nP; k++) pmat[(size_t)j * nP + k] = prod_mod(P, k, Q[j]);
            pinv[2 * j] = invmod(prod_mod(P, -1, Q[j]), Q[j]);
            pinv[2 * j + 1] = shoup(pinv[2 * j], Q[j]);
        }
        up(c->p_hat_inv, phi);
        up(c->p_mat, pmat);
        up(c->p_inv, pinv);
    }

    // per data level (rns.cu:66-195)
    c->levels.resize(nQ + 1);
    for (int l = 1; l <= nQ; l++) {
        auto lt = std::make_unique<LevelTables>();
        lt->l = l;
        if (nP > 0) {
            const int alpha = nP, beta = c->beta(l);
            lt->beta = beta;
            std::vector<uint64_t> phi(2 * l), mat((size_t)beta * (l + alpha) * alpha, 0);
            for (int d = 0; d < beta; d++) {
                const int s = d * alpha, sz = std::min(alpha, l - s);
                std::vector<uint64_t> dig(Q.begin() + s, Q.begin() + s + sz);
                for (int i = 0; i < sz; i++) {
                    phi[2 * (s + i)] = invmod(prod_mod(dig, i, Q[s + i]), Q[s + i]);
                    phi[2 * (s + i) + 1] = shoup(phi[2 * (s + i)], Q[s + i]);
                }
                for (int jj = 0; jj < l + alpha; jj++) {
                    if (jj >= s && jj < s + sz) continue;
                    const uint64_t p = c->mods[c->qlp_table(l, jj)];
                    for (int i = 0; i < sz; i++)
                        mat[((size_t)d * (l + alpha) + jj) * alpha + i] = prod_mod(dig, i, p);
                }
            }
            up(lt->part_hat_inv, phi);
            up(lt->modup_mat, mat);
            if (c->tc_avail && l + alpha - (l - (beta - 1) * alpha) <= 32) {
                // byte planes of M'_(i,a) = 2^(8a) M_d[jj][i] mod p_jj, rows (output o, plane b)
                const int kp = c->tc_kpad;
                std::vector<uint16_t> bm((size_t)beta * 256 * kp, 0);
                std::vector<TcOutMeta> meta((size_t)beta * 32);
                std::vector<int> nn(beta, 0);
                for (int d = 0; d < beta; d++) {
                    const int s = d * alpha, sz = std::min(alpha, l - s);
                    // output positions: limbs below 2^40 first (5 byte planes), then the others (8)
                    std::vector<int> pos;
                    for (int pass = 0; pass < 2; pass++)
                        for (int jj = 0; jj < l + alpha; jj++) {
                            if (jj >= s && jj < s + sz) continue;
                            const bool narrow = c->mods[c->qlp_table(l, jj)] < (1ull << 40);
                            if (narrow == (pass == 0)) pos.push_back(jj);
                            if (narrow && pass == 0) nn[d]++;
                        }
                    for (int o = 0; o < (int)pos.size(); o++) {
                        const int jj = pos[o];
                        const uint64_t p = c->mods[c->qlp_table(l, jj)];
                        meta[(size_t)d * 32 + o] = TcOutMeta{(uint32_t)jj, (uint32_t)c->qlp_table(l, jj), (float)(1.0 / (double)p)};
                        for (int i = 0; i < sz; i++) {
                            uint64_t mp = mat[((size_t)d * (l + alpha) + jj) * alpha + i];
                            for (int a = 0; a < 8; a++) {
                                for (int b = 0; b < 8; b++)
                                    bm[(size_t)d * 256 * kp + canon_index(o * 8 + b, i * 8 + a, kp)] =
                                            bf16_of_byte((unsigned)(mp >> (8 * b)) & 0xFF);
                                mp = mulmod(mp, 256 % p, p);
                            }
                        }
                    }
                }
                up(lt->tc_modup, bm);
                up(lt->tc_modup_meta, meta);
                up(lt->tc_modup_nn, nn);
                lt->tc_ok = true;
            }
        }
        if (nP > 0 && c->tc_avail && l <= 32) {
            // tensor-core P -> Ql conversions: positions = j < l, limbs below 2^40 first; for the
            // fused rescale the constants carry P^-1 mod q_j and j = l - 1 takes the last position
            const int kp = c->tc_kpad;
            auto build = [&](bool rescale, DevBuf &bbuf, DevBuf &mbuf, int &nn) {
                std::vector<int> pos;
                const int nlim = rescale ? l - 1 : l;
                nn = 0;
                for (int pass = 0; pass < 2; pass++)
                    for (int j = 0; j < nlim; j++) {
                        const bool narrow = Q[j] < (1ull << 40);
                        if (narrow == (pass == 0)) pos.push_back(j);
                        if (narrow && pass == 0) nn++;
                    }
                if (rescale) pos.push_back(l - 1);
                std::vector<uint16_t> bm((size_t)256 * kp, 0);
                std::vector<TcOutMeta> meta(32);
                for (int o = 0; o < (int)pos.size(); o++) {
                    const int j = pos[o];
                    const uint64_t q = Q[j];
                    meta[o] = TcOutMeta{(uint32_t)j, (uint32_t)j, (float)(1.0 / (double)q)};
                    for (int k = 0; k < nP; k++) {
                        uint64_t mp = pmat[(size_t)j * nP + k];
                        if (rescale) mp = mulmod(mp, pinv[2 * j], q);
                        for (int a = 0; a < 8; a++) {
                            for (int b = 0; b < 8; b++)
                                bm[canon_index(o * 8 + b, k * 8 + a, kp)] = bf16_of_byte((unsigned)(mp >> (8 * b)) & 0xFF);
                            mp = mulmod(mp, 256 % q, q);
                        }
                    }
                }
                up(bbuf, bm);
                up(mbuf, meta);
            };
            build(false, lt->tc_moddown, lt->tc_moddown_meta, lt->tc_moddown_nn);
            lt->tc_moddown_ok = true;
            if (l > 1) {
                bool fits = true;  // z < q_(l-1) <= 2 q_j keeps delta_j P^-1 + z below 4 q_j
                for (int j = 0; j < l - 1; j++) fits = fits && Q[l - 1] <= 2 * Q[j];
                if (fits) {
                    build(true, lt->tc_rescale, lt->tc_rescale_meta, lt->tc_rescale_nn);
                    lt->tc_rescale_ok = true;
                }
            }
        }
        if (l > 1) {
            std::vector<uint64_t> iq(2 * (l - 1));
            for (int j = 0; j < l - 1; j++) {
                iq[2 * j] = invmod(Q[l - 1] % Q[j], Q[j]);
                iq[2 * j + 1] = shoup(iq[2 * j], Q[j]);
            }
            up(lt->inv_qlast, iq);
        }
        c->levels[l] = std::move(lt);
    }

    if (scheme == kSchemeBFV) {
        // HPS constants (rns.cu:687-777; BaseConverter host/rns.cu:438-498; RNSBase inv_)
        const int nR = c->nR;
        std::vector<uint64_t> qhi(2 * nQ), rhi(2 * nR), q2r((size_t)nR * nQ), r2q((size_t)nQ * nR);
        std::vector<uint64_t> q2ra((size_t)(nQ + 1) * nR), r2qa((size_t)(nR + 1) * nQ);
        std::vector<double> qinv(nQ), rinv(nR), frac(nQ);
        std::vector<uint64_t> modr((size_t)nR * (nQ + 1));
        for (int i = 0; i < nQ; i++) {
            qhi[2 * i] = invmod(prod_mod(Q, i, Q[i]), Q[i]);
            qhi[2 * i + 1] = shoup(qhi[2 * i], Q[i]);
            qinv[i] = 1.0 / static_cast<double>(Q[i]);
        }
        for (int j = 0; j < nR; j++) {
            rhi[2 * j] = invmod(prod_mod(R, j, R[j]), R[j]);
            rhi[2 * j + 1] = shoup(rhi[2 * j], R[j]);
            rinv[j] = 1.0 / static_cast<double>(R[j]);
        }
        for (int j = 0; j < nR; j++)
            for (int i = 0; i < nQ; i++) q2r[(size_t)j * nQ + i] = prod_mod(Q, i, R[j]);
        for (int j = 0; j < nQ; j++)
            for (int i = 0; i < nR; i++) r2q[(size_t)j * nR + i] = prod_mod(R, i, Q[j]);
        for (int a = 0; a <= nQ; a++)
            for (int j = 0; j < nR; j++) q2ra[(size_t)a * nR + j] = mulmod(a, prod_mod(Q, -1, R[j]), R[j]);
        for (int a = 0; a <= nR; a++)
            for (int j = 0; j < nQ; j++) r2qa[(size_t)a * nQ + j] = mulmod(a, prod_mod(R, -1, Q[j]), Q[j]);
        // S = QR.  For q_i: X = t*R*[(S/q_i)^-1]_{q_i}; rem = X mod q_i; frac = rem / q_i;
        // floor(X / q_i) mod r_j = -rem * q_i^-1 (R divides X).  For r_j:
        // floor(X / r_j) = t * (R / r_j) * [(S/r_j)^-1]_{r_j}.
        std::vector<uint64_t> S(Q);
        S.insert(S.end(), R.begin(), R.end());
        for (int i = 0; i < nQ; i++) {
            const uint64_t q = Q[i];
            const uint64_t shat_inv = invmod(prod_mod(S, i, q), q);
            const uint64_t rem = mulmod(mulmod(plain_modulus % q, prod_mod(R, -1, q), q), shat_inv, q);
            frac[i] = static_cast<double>(rem) / static_cast<double>(q);
            for (int j = 0; j < nR; j++) {
                const uint64_t v = mulmod(rem % R[j], invmod(q % R[j], R[j]), R[j]);
                modr[(size_t)j * (nQ + 1) + i] = v ? R[j] - v : 0;
            }
        }
        for (int j = 0; j < nR; j++) {
            const uint64_t shat_inv = invmod(prod_mod(S, nQ + j, R[j]), R[j]);
            modr[(size_t)j * (nQ + 1) + nQ] =
                    mulmod(mulmod(plain_modulus % R[j], prod_mod(R, j, R[j]), R[j]), shat_inv, R[j]);
        }
        up(c->hps_q_hat_inv, qhi);
        up(c->hps_r_hat_inv, rhi);
        up(c->hps_q_inv, qinv);
        up(c->hps_r_inv, rinv);
        up(c->hps_q2r_mat, q2r);
        up(c->hps_r2q_mat, r2q);
        up(c->hps_q2r_alpha, q2ra);
        up(c->hps_r2q_alpha, r2qa);
        up(c->hps_frac, frac);
        up(c->hps_modr, modr);

        // tensor-core forms of the three HPS contractions (byte-plane operands, see tc.cuh); the
        // extra slot of a conversion carries its FP64 correction v with constant -Q (or -R)
        auto bytes_below = [](uint64_t m) {
            int b = 0;
            for (uint64_t v = m - 1; v; v >>= 8) b++;
            return b;
        };
        int qbytes = 0, rbytes = 0;
        for (uint64_t q : Q) qbytes += bytes_below(q);
        for (uint64_t r : R) rbytes += bytes_below(r);
        // every plane sum below 2^24: at most 258 nonzero byte products of at most 255 * 255
        const bool exact = qbytes + 1 <= 258 && rbytes + 1 <= 258 && qbytes + rbytes <= 258;
        if (exact && nQ <= 32 && nR <= 32 && nQ + nR <= 34) {
            auto operand = [&](int npos, int nslots, int kp, auto p_of, auto const_of) {
                std::vector<uint16_t> bm((size_t)256 * kp, 0);
                for (int o = 0; o < npos; o++) {
                    const uint64_t p = p_of(o);
                    for (int sl = 0; sl < nslots; sl++) {
                        uint64_t mp = const_of(o, sl);
                        if (!mp) continue;
                        for (int a = 0; a < 8; a++) {
                            for (int b = 0; b < 8; b++)
                                bm[canon_index(o * 8 + b, sl * 8 + a, kp)] = bf16_of_byte((unsigned)(mp >> (8 * b)) & 0xFF);
                            mp = mulmod(mp, 256 % p, p);
                        }
                    }
                }
                return bm;
            };
            auto kpad = [](int slots) { return (slots * 8 + 15) / 16 * 16; };
            c->tc_hps_kp_q2r = kpad(nQ + 1);
            c->tc_hps_kp_r2q = kpad(nR + 1);
            c->tc_hps_kp_scale = kpad(nQ + nR);
            up(c->tc_hps_q2r, operand(nR, nQ + 1, c->tc_hps_kp_q2r, [&](int o) { return R[o]; }, [&](int o, int sl) {
                   if (sl < nQ) return q2r[(size_t)o * nQ + sl];
                   const uint64_t qm = prod_mod(Q, -1, R[o]);
                   return qm ? R[o] - qm : 0;
               }));
            up(c->tc_hps_r2q, operand(nQ, nR + 1, c->tc_hps_kp_r2q, [&](int o) { return Q[o]; }, [&](int o, int sl) {
                   if (sl < nR) return r2q[(size_t)o * nR + sl];
                   const uint64_t rm = prod_mod(R, -1, Q[o]);
                   return rm ? Q[o] - rm : 0;
               }));
            up(c->tc_hps_scale, operand(nR, nQ + nR, c->tc_hps_kp_scale, [&](int o) { return R[o]; },
                                        [&](int o, int sl) -> uint64_t {
                                            if (sl < nQ) return modr[(size_t)o * (nQ + 1) + sl];
                                            return sl - nQ == o ? modr[(size_t)o * (nQ + 1) + nQ] : 0;
                                        }));
            // the scale-and-round tile (A, B, staged inputs, carries) must fit one CTA
            const size_t ncols = (size_t)(nR * 8 + 15) / 16 * 16;
            const size_t scale_smem = (size_t)128 * c->tc_hps_kp_scale * 2 + ncols * c->tc_hps_kp_scale * 2 +
                                      (size_t)(nQ + nR) * 128 * 8 + (size_t)nR * 128 * 8;
            c->tc_hps_ok = scale_smem + 4096 <= (size_t)c->smem_optin;
        }
    }

    c->galois_elts = galois_elts;
    if (c->galois_elts.empty() && scheme == kSchemeCKKS) {
        // all power-of-two rotations plus conjugation (src/galois.cu:41-65)
        const uint32_t m = (uint32_t)(2 * n);
        c->galois_elts.push_back(m - 1);
        uint64_t pos = 5, neg = invmod(5, m);
        for (int i = 0; i < log_n - 1; i++) {
            c->galois_elts.push_back((uint32_t)pos);
            pos = (pos * pos) & (m - 1);
            c->galois_elts.push_back((uint32_t)neg);
            neg = (neg * neg) & (m - 1);
        }
    }
    // permutation tables for every Galois element, built up front so that no evaluator call
    // allocates or copies host data (include/galois.cuh:98-113)
    for (uint32_t elt : c->galois_elts) c->perm_table(elt);
    if (scheme == kSchemeCKKS) build_codec_tables(*c);
    return c;
}

}  // namespace pfg
