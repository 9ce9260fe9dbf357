/*
 * fhe_oracle.h — CPU restatement of PhantomFHE's RNS ciphertext-arithmetic hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests, the smoke
 * check and the CPU-baseline leg of bench.py call it to compute the expected answer.
 * The GPU product path never links, loads or calls it.
 *
 * Parity pin: table generation (primes, Barrett ratios, minimal 2N-th roots, NTT
 * twiddle tables, RNS/base-converter matrices, HPS scale-and-round constants) is checked
 * word-for-word against the reference's own host code, compiled from its sources by
 * oracle/Makefile.ref into oracle/_ref/ and dumped into tests/golden/.  The kernels
 * themselves have no CPU implementation in the reference (its src/host/ only builds
 * tables); every function below restates the reference kernel named beside it, and the
 * reference's only known-answer test (NTT round trip on constant inputs,
 * test/ntt_test.cu:46-121) is reproduced in tests/test_oracle.py.
 *
 * Layout conventions follow the reference: a polynomial is [limb][N] uint64, a
 * ciphertext is [poly][limb][N]; key-switching keys are [dnum][2][QP][N] (the
 * reference holds dnum device pointers, include/secretkey.h:124-127, each to [2][QP][N]).
 * All residues are canonical, in [0, q).
 */
#ifndef FHE_ORACLE_H
#define FHE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar number theory (src/host/numth.cu, src/host/modulus.cu) ---- */
uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t q);
uint64_t orc_powmod(uint64_t a, uint64_t e, uint64_t q);
uint64_t orc_invmod(uint64_t a, uint64_t q);
int orc_is_prime(uint64_t v);
/* Barrett ratio floor(2^128 / q) as two words plus the remainder (modulus.cu:15-42). */
void orc_barrett_ratio(uint64_t q, uint64_t out[3]);
uint64_t orc_shoup(uint64_t w, uint64_t q);
/* get_primes (numth.cu:207-232): `count` primes = 1 mod 2N below 2^bits, descending. */
int orc_get_primes(uint64_t n, int bits, int count, uint64_t *out);
/* get_primes_below (numth.cu:234-261). */
int orc_get_primes_below(uint64_t n, uint64_t upper, int count, uint64_t *out);
/* CoeffModulus::Create ordering (modulus.cu:80-111). */
int orc_create_coeff_modulus(uint64_t n, const int *bit_sizes, int count, uint64_t *out);
/* try_minimal_primitive_root (numth.cu:309-331). */
uint64_t orc_minimal_root(uint64_t degree, uint64_t q);
/* NTT::NTT tables (src/host/ntt.cu:11-56): bit-reversed powers, n^-1 folded into inv[1]. */
int orc_ntt_tables(int log_n, uint64_t q, uint64_t *root, uint64_t *root_shoup, uint64_t *inv_root,
                   uint64_t *inv_root_shoup, uint64_t *n_inv);

/* ---- context: moduli QP = Q (nQ primes) followed by P (nP special primes) ---- */
typedef struct orc_ctx orc_ctx;
orc_ctx *orc_ctx_create(int log_n, const uint64_t *moduli, int nQ, int nP, uint64_t plain_modulus);
void orc_ctx_destroy(orc_ctx *ctx);
int orc_ctx_n(const orc_ctx *ctx);
/* Number of BFV HPS R primes (0 when no plain modulus was given). */
int orc_ctx_hps_r(const orc_ctx *ctx, uint64_t *r_out);
/* Set worker threads for the parallel loops (0 = OpenMP default). */
void orc_set_threads(int threads);

/* NTT over `num_limbs` limbs; limb k uses the QP table index tbl[k] (tbl==NULL: k). */
void orc_ntt_fwd(const orc_ctx *ctx, uint64_t *data, int num_limbs, const int *tbl);
void orc_ntt_inv(const orc_ctx *ctx, uint64_t *data, int num_limbs, const int *tbl);
/* NTT/iNTT over the HPS QlRl base (Q primes then R primes). */
void orc_ntt_fwd_qr(const orc_ctx *ctx, uint64_t *data, int num_limbs);
void orc_ntt_inv_qr(const orc_ctx *ctx, uint64_t *data, int num_limbs);

/* tensor_prod_2x2_rns_poly (src/polymath.cu:463-497) at level l (l limbs, NTT form). */
void orc_tensor(const orc_ctx *ctx, int l, const uint64_t *a, const uint64_t *b, uint64_t *out3);
/* tensor_square_2x2_rns_poly (src/polymath.cu:500-535). */
void orc_tensor_square(const orc_ctx *ctx, int l, const uint64_t *a, uint64_t *out3);

/* DRNSTool::modup (src/rns_bconv.cu:530-628).  scheme: 0 = CKKS (c2 in NTT form),
 * 1 = BFV (c2 in coefficient form).  out: beta x (l+nP) x N. */
void orc_modup(const orc_ctx *ctx, int l, const uint64_t *c2, uint64_t *out, int scheme);
/* key_switch_inner_prod_c2_and_evk (src/eval_key_switch.cu:14-69).
 * evk: [dnum][2][QP][N]; out: 2 x (l+nP) x N. */
void orc_inner_product(const orc_ctx *ctx, int l, const uint64_t *tmodup, const uint64_t *evk,
                       uint64_t *out);
/* DRNSTool::moddown_from_NTT (src/rns_bconv.cu:776-828): cx (l+nP limbs, NTT form) ->
 * out (l limbs; NTT form for CKKS, coefficient form for BFV). cx is clobbered. */
void orc_moddown(const orc_ctx *ctx, int l, uint64_t *cx, uint64_t *out, int scheme);
/* keyswitch_inplace (src/eval_key_switch.cu:95-182): ct (2 x l x N) += KS(c2). */
void orc_keyswitch(const orc_ctx *ctx, int l, uint64_t *ct, const uint64_t *c2, const uint64_t *evk,
                   int scheme);
/* relinearize_inplace (src/evaluate.cu:1342-1374): ct3 (3 x l x N) -> first 2 polys. */
void orc_relinearize(const orc_ctx *ctx, int l, uint64_t *ct3, const uint64_t *rlk, int scheme);
/* CKKS multiply_and_relin_inplace (src/evaluate.cu:1061-1104): out (2 x l x N). */
void orc_ckks_mul_relin(const orc_ctx *ctx, int l, const uint64_t *a, const uint64_t *b,
                        const uint64_t *rlk, uint64_t *out);
/* divide_and_round_q_last_ntt (src/rns.cu:1160-1184): in (size x l x N) -> out (size x (l-1) x N). */
void orc_rescale(const orc_ctx *ctx, int l, int size, const uint64_t *in, uint64_t *out);
/* divide_and_round_q_last (src/rns.cu:1082-1126), BFV coefficient domain. */
void orc_divide_round_q_last(const orc_ctx *ctx, int l, int size, const uint64_t *in, uint64_t *out);
/* acc[p][k] = (acc[p][k] + a[p][k] * b[k]) mod q_k, p < polys, k < l (canonical inputs) */
void orc_mul_add(const orc_ctx *ctx, int l, int polys, const uint64_t *a, const uint64_t *b, uint64_t *acc);
/* Galois tables (include/galois.cuh:16-49, 98-113). */
uint32_t orc_elt_from_step(int step, uint64_t n);
void orc_galois_perm(int log_n, uint32_t elt, uint32_t *perm);
/* apply_galois_ntt_permutation (src/galois.cu:11-18) over num_limbs limbs. */
void orc_apply_galois_ntt(const orc_ctx *ctx, const uint64_t *src, uint64_t *dst, int num_limbs,
                          uint32_t elt);
/* apply_galois_permutation (src/galois.cu:20-39), BFV coefficient domain; tbl as orc_ntt_fwd. */
void orc_apply_galois_coeff(const orc_ctx *ctx, const uint64_t *src, uint64_t *dst, int num_limbs,
                            uint32_t elt);
/* apply_galois_inplace for CKKS (src/evaluate.cu:1567-1630): ct (2 x l x N). */
void orc_ckks_apply_galois(const orc_ctx *ctx, int l, uint64_t *ct, uint32_t elt, const uint64_t *gk);
/* hoisting_inplace for CKKS (src/evaluate.cu:1670-1865): ct <- sum_s rot_s(ct);
 * gks: one key per element, each [dnum][2][QP][N]. */
void orc_ckks_hoisting(const orc_ctx *ctx, int l, uint64_t *ct, const uint32_t *elts, int n_elts,
                       const uint64_t *const *gks);

/* ---- BFV HPS (mul_tech::hps) ---- */
/* DBaseConverter::bConv_HPS (src/rns_bconv.cu:277-372): Q (nQ limbs) -> R limbs, or R -> Q. */
void orc_hps_bconv_q_to_r(const orc_ctx *ctx, const uint64_t *in, uint64_t *out);
void orc_hps_bconv_r_to_q(const orc_ctx *ctx, const uint64_t *in, uint64_t *out);
/* scaleAndRound_HPS_QR_R (src/rns.cu:1700-1747): in QlRl limbs -> out R limbs. */
void orc_hps_scale_round_qr_r(const orc_ctx *ctx, const uint64_t *in, uint64_t *out);
/* bfv_mul_relin_hps (src/evaluate.cu:820-1026): a,b (2 x nQ x N, coefficient form) -> out. */
void orc_bfv_mul_relin_hps(const orc_ctx *ctx, const uint64_t *a, const uint64_t *b,
                           const uint64_t *rlk, uint64_t *out);

/* ---- the reference's samplers (src/prng.cu:17-244) and key combination ---- */
/* uniform [limbs][N] modulo QP primes 0..limbs-1 (sample_uniform_poly); 64-byte seed */
void orc_sample_uniform(const orc_ctx *ctx, const uint8_t *seed, int limbs, uint64_t *out);
/* kind 0: ternary (sample_ternary_poly), 1: centred binomial (sample_error_poly); out [N] */
void orc_sample_small(const orc_ctx *ctx, const uint8_t *seed, int kind, int64_t *out);
/* generate_one_kswitch_key's combination (src/secretkey.cu:297-341, polymath.cu:318-370) */
void orc_kswitch_key_combine(const orc_ctx *ctx, const uint64_t *s, const uint64_t *s_src, const uint64_t *a,
                             const uint64_t *e_ntt, uint64_t *key);

/* ---- table access for golden checks ---- */
/* modup constants for level l, digit d: partQlHatInv (size_d) and the size_d x (l+nP-size_d)
 * base-change matrix (row = output prime). */
int orc_modup_tables(const orc_ctx *ctx, int l, int d, uint64_t *part_hat_inv, uint64_t *matrix);
/* moddown constants: PHatInv (nP), P->Ql matrix (l x nP), PInv mod q (l). */
int orc_moddown_tables(const orc_ctx *ctx, int l, uint64_t *p_hat_inv, uint64_t *matrix,
                       uint64_t *p_inv);
/* HPS constants: tRSHatInvModsDivsFrac (nQ), tRSHatInvModsDivsModr (nR x (nQ+1)). */
int orc_hps_tables(const orc_ctx *ctx, double *frac, uint64_t *modr);

#ifdef __cplusplus
}
#endif
#endif
