/*
 * phantom_gb300.h — C ABI of the GB300-native RNS ciphertext-arithmetic library.
 *
 * This is the drop-in boundary for PhantomFHE's hot path.  The reference ships a C++
 * source API (include/phantom.h, include/evaluate.cuh) with no C ABI of its own; every
 * entry point below names the reference interface it replaces (file:line in the
 * PhantomFHE tree).  The C++ compatibility layer (phantom-fhe_gb300/cpp/phantom.h) and the
 * Python bindings sit on top of these calls.
 *
 * Conventions
 *  - All ciphertext / key pointers are DEVICE pointers; layout is the reference's:
 *    ciphertext = [size][coeff_modulus_size][N] uint64 limb-major (include/ciphertext.h:44-72),
 *    key-switching key = dnum device pointers (a device array, as returned by
 *    PhantomRelinKey::public_keys_ptr(), include/secretkey.h:124-127), each to [2][QP][N]
 *    in NTT form.  Device buffers of residues (ciphertexts, plaintexts, keys, diagonals,
 *    scratch) must start on a 16-byte boundary: the kernels move them in 16-byte vectors.
 *    Every cudaMalloc / caching-allocator block is 256-byte aligned, and limb offsets
 *    (multiples of N words) keep that alignment.
 *  - `chain_index` follows the reference: 0 is the key level (QP), 1 the full data level Q,
 *    each further index drops one prime (src/context.cu:141-158).
 *  - Calls enqueue work on `stream` (a cudaStream_t; NULL = the legacy default stream) and
 *    return without synchronising.  Calls never allocate device memory: scratch comes from an
 *    fhe_workspace, which must not be shared by two calls that can run concurrently.
 *  - A context is read-only for the evaluation calls, so any number of host threads may use
 *    one context at once (each with its own workspace).  The tuning setters below
 *    (fhe_context_set_* and fhe_context_autotune) change it: call them before the context is
 *    shared, or with no other call on it in flight.
 *  - Return value: FHE_OK or a negative status.  FHE_ERR_INVALID_ARGUMENT and FHE_ERR_LOGIC
 *    correspond to the std::invalid_argument / std::logic_error the reference throws;
 *    fhe_last_error() returns the message of the calling thread's last failure.
 */
#ifndef PHANTOM_GB300_H
#define PHANTOM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FHE_OK 0
#define FHE_ERR_INVALID_ARGUMENT (-1)
#define FHE_ERR_LOGIC (-2)
#define FHE_ERR_CUDA (-3)
#define FHE_ERR_OUT_OF_MEMORY (-4)
#define FHE_ERR_UNSUPPORTED (-5)

/* scheme_type and mul_tech_type values of include/host/encryptionparams.h */
#define FHE_SCHEME_BGV 1 /* not supported */
#define FHE_SCHEME_BFV 2
#define FHE_SCHEME_CKKS 3
#define FHE_MUL_TECH_HPS 2

typedef struct fhe_context fhe_context;
typedef struct fhe_workspace fhe_workspace;

/* Mirrors phantom::EncryptionParameters (include/host/encryptionparams.h:12-246). */
typedef struct fhe_params {
    int scheme;                     /* FHE_SCHEME_* */
    int mul_tech;                   /* FHE_MUL_TECH_HPS for BFV; ignored for CKKS */
    uint64_t poly_modulus_degree;   /* N, a power of two in [2^12, 2^17] */
    const uint64_t *coeff_modulus;  /* QP: data primes Q first, then special primes P */
    size_t coeff_modulus_size;
    size_t special_modulus_size;    /* |P| = alpha */
    uint64_t plain_modulus;         /* BFV t; 0 for CKKS */
    const uint32_t *galois_elts;    /* NULL/0: all power-of-two rotations (src/galois.cu:41-65) */
    size_t galois_elts_size;
} fhe_params;

const char *fhe_last_error(void);

/* Number of CUDA kernels this library has launched so far in the process (all threads).
 * No counterpart in the reference; used to report launches per operation. */
uint64_t fhe_kernel_launches(void);

/* CoeffModulus::Create (include/host/modulus.h:295, src/host/modulus.cu:80-111). */
int fhe_create_coeff_modulus(uint64_t poly_modulus_degree, const int *bit_sizes, size_t count, uint64_t *out);

/* phantom::util::get_elt_from_step (include/galois.cuh:16-49).  Returns 0 on error. */
uint32_t fhe_galois_elt_from_step(int step, uint64_t poly_modulus_degree);

/* PhantomContext::PhantomContext(const EncryptionParameters&) (include/context.cuh:161,
 * src/context.cu:121-232): builds and uploads every table. */
int fhe_context_create(const fhe_params *params, fhe_context **out);
void fhe_context_destroy(fhe_context *ctx);

/* Base conversions of the key switch on the tensor cores (exact bf16 byte-plane GEMMs,
 * tcgen05) or on the CUDA cores (64-bit multiply-accumulate).  Both give the same words; the
 * tensor-core form is the default wherever it applies (1 <= special_modulus_size <= 6 and at
 * most 32 output limbs per digit).  No counterpart in the reference, whose conversions are
 * CUDA-core kernels (src/rns_bconv.cu:455-485). */
int fhe_context_set_tensor_cores(fhe_context *ctx, int enable);
int fhe_context_tensor_cores(const fhe_context *ctx);

/* NTT stage split (autotuner).  The forward transform runs its first l1 stages as a column
 * pass and the remaining log2(N) - l1 as a row pass; every supported split gives the same
 * words.  fhe_context_autotune times each supported split on scratch limbs (forward + inverse,
 * CUDA events, one-time setup call that allocates and synchronises) and keeps the fastest;
 * fhe_context_set_ntt_split applies a stored choice.  No counterpart in the reference, whose
 * radix-8 two-phase split is fixed per degree (src/ntt/fntt_2d.cu:620-653). */
int fhe_context_ntt_split(const fhe_context *ctx);
int fhe_context_set_ntt_split(fhe_context *ctx, int l1);
int fhe_context_autotune(fhe_context *ctx, int *chosen_l1, float *best_us);

/* The context's kernel shapes; every setting gives the same words.  No counterpart in the
 * reference, whose shapes are fixed (include/common.h, include/ntt.cuh:131-153). */
typedef struct fhe_tuning {
    int ntt_split;        /* NTT stages of the column pass (l1) */
    int ntt_tile;         /* coefficients per CTA of the 16-per-thread NTT passes: 2048 or 4096 */
    int ntt_small_tile;   /* ... of the 8-per-thread passes: 1024 or 2048 */
    int ntt_small_launch; /* passes of at most this many 4096-coefficient tiles run 8 per thread */
    int fused_keyswitch;  /* mod-up row pass fused with the inner product (CKKS) */
    int tensor_cores;     /* base conversions on the tensor cores (where available) */
    float best_us;        /* time of one timed operation with these shapes (autotuner) */
    int evaluated;        /* configurations the autotuner timed (0: taken from the cache) */
} fhe_tuning;

/* Autotuner over the operation itself: times the context's benchmark workload at its top level,
 * batch 1 (CKKS multiply + relinearise + rescale; BFV HPS multiply + relinearise), on uniform
 * residues, over the NTT split, both NTT tiles, the small-launch bound, the fused key switch and
 * the tensor-core conversions (coordinate descent, two sweeps), and applies the fastest.  With a
 * cache_path, a JSON-lines file keyed by GPU name, scheme, N, |Q|, |P| and batch holds the choice:
 * a matching entry is applied without timing (out->evaluated = 0), a new one is appended.  A
 * one-time set-up call: it allocates its inputs and a key and synchronises. */
int fhe_context_autotune_op(fhe_context *ctx, fhe_workspace *ws, const char *cache_path, fhe_tuning *out);
int fhe_context_tuning(const fhe_context *ctx, fhe_tuning *out);
int fhe_context_set_tuning(fhe_context *ctx, const fhe_tuning *t);

/* NTT passes over at most `tiles` tiles of 4096 coefficients (limbs x N / 4096) run the
 * 8-coefficients-per-thread kernels, which finish a tile in about half the time of the
 * 16-per-thread kernels and so suit launches of a few waves; larger passes run 16 per thread.
 * -1 restores the default (measured on GB300: 512 tiles for N >= 2^16, 1024 below); 0 disables the small
 * kernels.  Every setting gives the same words.  No counterpart in the reference. */
/* Kernel chains of one call launched with programmatic dependent launch (on by default): a
 * kernel may be scheduled while its predecessor drains its last wave and starts once that
 * predecessor's writes are visible.  Every setting gives the same words.  No counterpart in the
 * reference. */
int fhe_context_launch_overlap(const fhe_context *ctx);
int fhe_context_set_launch_overlap(fhe_context *ctx, int enable);

/* The mod-up's forward NTT row pass fused with the key-switching inner product (on by default):
 * one kernel finishes each digit's transform tile by tile and accumulates it against the key, so
 * the mod-up output (src/rns_bconv.cu:530-628) is never written to or read back from device
 * memory.  Used by the key switch, relinearisation, HMult, Galois and batched calls (in a batch,
 * the blocks of every ciphertext that read one key tile run together); hoisted rotations keep
 * the materialised mod-up (they reuse it).  Every setting gives the same words.  No counterpart
 * in the reference. */
int fhe_context_fused_keyswitch(const fhe_context *ctx);
int fhe_context_set_fused_keyswitch(fhe_context *ctx, int enable);

int fhe_context_ntt_small_launch(const fhe_context *ctx);
int fhe_context_set_ntt_small_launch(fhe_context *ctx, int tiles);

/* Coefficients per CTA of those small-launch passes: 1024 (the default) or 2048.  Smaller CTAs
 * spread a launch of a few hundred tiles evenly over the SMs and wait less at their barriers.
 * Every setting gives the same words.  No counterpart in the reference. */
int fhe_context_ntt_small_tile(const fhe_context *ctx);
int fhe_context_set_ntt_small_tile(fhe_context *ctx, int coefficients);

/* Coefficients per CTA of the larger (16 coefficients per thread) NTT passes: 2048 (the default)
 * or 4096.  Every setting gives the same words.  No counterpart in the reference. */
int fhe_context_ntt_tile(const fhe_context *ctx);
int fhe_context_set_ntt_tile(fhe_context *ctx, int coefficients);

/* Reads and clears the context's device status word (synchronises the device).  Non-zero
 * means a bounded wait inside a tensor-core kernel gave up and that call's output is invalid.
 * No counterpart in the reference. */
int fhe_context_status(const fhe_context *ctx, unsigned *out);

/* Sizes of a context: N, |Q|, |P|, |R| (BFV HPS base, else 0), dnum = ceil(|Q|/|P|). */
int fhe_context_sizes(const fhe_context *ctx, uint64_t *n, size_t *size_q, size_t *size_p, size_t *size_r,
                      size_t *dnum);
/* The context's prime list (QP then R); `out` holds at least |Q|+|P|+|R| words. */
int fhe_context_moduli(const fhe_context *ctx, uint64_t *out);
/* The Galois elements the context was built with (PhantomGaloisTool::galois_elts_). */
int fhe_context_galois_elts(const fhe_context *ctx, uint32_t *out, size_t *count);

/* Scratch for the evaluator calls (replaces the reference's per-call cudaMallocAsync,
 * src/eval_key_switch.cu:143-181).  Sized for the key level. */
size_t fhe_workspace_bytes(const fhe_context *ctx);
int fhe_workspace_create(const fhe_context *ctx, fhe_workspace **out);
void fhe_workspace_destroy(fhe_workspace *ws);
/* Workspace for the batched calls: scratch for min(max_items, 64) ciphertexts at the key level
 * (the reference has no batched calls; it loops over single calls). */
int fhe_workspace_create_batch(const fhe_context *ctx, size_t max_items, fhe_workspace **out);

/* nwt_2d_radix8_forward_inplace / nwt_2d_radix8_backward_inplace (include/ntt.cuh:157-226):
 * in-place transform of `num_polys` polynomials of `coeff_modulus_size` limbs each
 * (contiguous), limb k using prime start_modulus_idx + k of the context's QP list.
 * For BFV contexts, indices >= |Q|+|P| address the HPS base R. */
int fhe_ntt_forward(const fhe_context *ctx, uint64_t *data, size_t num_polys, size_t coeff_modulus_size,
                    size_t start_modulus_idx, void *stream);
int fhe_ntt_inverse(const fhe_context *ctx, uint64_t *data, size_t num_polys, size_t coeff_modulus_size,
                    size_t start_modulus_idx, void *stream);

/* bgv_ckks_multiply (src/evaluate.cu:345-397): CKKS tensor product.  ct1 holds 3
 * polynomials of capacity (the first two are the input), ct2 two; ct1 == ct2 squares. */
int fhe_ckks_multiply(const fhe_context *ctx, uint64_t *ct1, const uint64_t *ct2, size_t chain_index,
                      void *stream);

/* keyswitch_inplace (include/evaluate.cuh:29, src/eval_key_switch.cu:95-182):
 * ct (2 polynomials at chain_index) += KeySwitch(c2) under evk. */
int fhe_keyswitch(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, const uint64_t *c2,
                  size_t chain_index, const uint64_t *const *evk, void *stream);

/* relinearize_inplace (include/evaluate.cuh:125, src/evaluate.cu:1342-1374): ct holds 3
 * polynomials; on return its first two are the relinearised ciphertext. */
int fhe_relinearize(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index,
                    const uint64_t *const *rlk, void *stream);

/* multiply_and_relin_inplace (include/evaluate.cuh:115, src/evaluate.cu:1061-1104).
 * CKKS: ct1 (2 polys, NTT form) *= ct2, relinearised, written to ct1.  The tensor product is
 * fused into the key switch and never materialised, so ct1 needs room for 2 polynomials only.
 * BFV (mul_tech hps, src/evaluate.cu:820-1026): ct1, ct2 in coefficient form at chain 1. */
int fhe_multiply_and_relin(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct1, const uint64_t *ct2,
                           size_t chain_index, const uint64_t *const *rlk, void *stream);

/* rescale_to_next (include/evaluate.cuh:137-140, src/evaluate.cu:1545-1565 via
 * DRNSTool::divide_and_round_q_last_ntt, src/rns.cu:1160-1184): in (size polys at
 * chain_index) -> out (size polys at chain_index + 1).  in and out may not overlap. */
int fhe_rescale_to_next(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *in, uint64_t *out, size_t size,
                        size_t chain_index, void *stream);

/* No counterpart in the reference: fhe_rescale_to_next for callers that may not allocate
 * device memory (for example a plugin whose host process owns all device memory and passes
 * in only the input and output buffers), so cannot hold an fhe_workspace.  Its scratch is a
 * fixed 2 MiB array inside the library, which limits size * N to 2^18 words; larger requests
 * fail with FHE_ERR_INVALID_ARGUMENT.  It calls no allocator.  The driver commits the 2 MiB
 * on a device when it loads the library's module there, which (with lazy module loading) is
 * the address lookup fhe_context_create makes, and the device keeps it until the process
 * exits.  The address is kept in the context, so call this on the context's device (another
 * device is rejected) and create the context before any stream capture.  All calls on a device
 * share the array: calls that overlap on the GPU race and must be serialised by the caller. */
int fhe_rescale_to_next_noalloc(const fhe_context *ctx, const uint64_t *in, uint64_t *out, size_t size,
                                size_t chain_index, void *stream);

/* mod_switch_to_next for BFV (src/rns.cu:1082-1126): coefficient-domain divide by q_last. */
int fhe_bfv_mod_switch_to_next(const fhe_context *ctx, const uint64_t *in, uint64_t *out, size_t size,
                               size_t chain_index, void *stream);

/* HMult + relinearise + rescale as one call (multiply_and_relin_inplace followed by
 * rescale_to_next_inplace, src/evaluate.cu:1061-1104 and 1545-1565): out (2 polys at
 * chain_index + 1) = Rescale(Relin(ct1 * ct2)).  Bit-identical to the two-call sequence.
 * ct1 and ct2 may be the same ciphertext (squaring); out must not overlap either input. */
int fhe_ckks_multiply_relin_rescale(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *ct1,
                                    const uint64_t *ct2, uint64_t *out, size_t chain_index,
                                    const uint64_t *const *rlk, void *stream);

/* A batch of independent HMult + relinearise + rescale operations at their own chain indices
 * (uneven levels allowed), sharing one relinearisation key.  The reference runs a batch as a host
 * loop of multiply_and_relin_inplace + rescale_to_next_inplace (src/evaluate.cu:1061-1104,
 * 1545-1565); here every pipeline step is one launch over up to 64 ciphertexts and the key is
 * read from HBM once per launch set.  Each output equals the single call's, word for word.
 * `items` is a host array; ws must come from fhe_workspace_create_batch. */
typedef struct fhe_ckks_mul_item {
    const uint64_t *ct1;  /* 2 polys at chain_index, NTT form */
    const uint64_t *ct2;  /* 2 polys at chain_index */
    uint64_t *out;        /* 2 polys at chain_index + 1 */
    size_t chain_index;
} fhe_ckks_mul_item;
int fhe_ckks_multiply_relin_rescale_batch(const fhe_context *ctx, fhe_workspace *ws, const fhe_ckks_mul_item *items,
                                          size_t count, const uint64_t *const *rlk, void *stream);

/* A batch of independent key switches (keyswitch_inplace, src/eval_key_switch.cu:95-182, CKKS,
 * NTT form) at their own chain indices, sharing one key: items[i].ct (2 polys) += KeySwitch of
 * items[i].c2 (1 poly).  Every pipeline step is one launch over up to 64 ciphertexts with the
 * base conversions on the tensor cores; each result equals the single call's word for word.
 * ws must come from fhe_workspace_create_batch. */
typedef struct fhe_ks_item {
    uint64_t *ct;
    const uint64_t *c2;
    size_t chain_index;
} fhe_ks_item;
int fhe_keyswitch_batch(const fhe_context *ctx, fhe_workspace *ws, const fhe_ks_item *items, size_t count,
                        const uint64_t *const *evk, void *stream);

/* apply_galois_inplace (include/evaluate.cuh:215, src/evaluate.cu:1567-1630), CKKS:
 * ct (2 polys) <- KeySwitch of the automorphism X -> X^galois_elt under gk. */
int fhe_apply_galois(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index,
                     uint32_t galois_elt, const uint64_t *const *gk, void *stream);

/* rotate_inplace (include/evaluate.cuh:225, src/evaluate.cu:1633-1668), CKKS: rotation by
 * `step` slots; when no key exists for the step's element, the NAF decomposition of the
 * step is applied key by key.  galois_keys[i] is the key of the context's i-th element. */
int fhe_rotate(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index, int step,
               const uint64_t *const *const *galois_keys, void *stream);

/* hoisting_inplace (include/evaluate.cuh:237, src/evaluate.cu:1670-1865), CKKS:
 * ct <- sum over steps of rotate(ct, step), sharing one mod-up of c1. */
int fhe_hoisting(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index, const int *steps,
                 size_t num_steps, const uint64_t *const *const *galois_keys, void *stream);

/* Rotations of one ciphertext by several steps that share one mod-up of c1, each result kept
 * (the baby steps of a matrix-vector product).  The reference computes them as separate
 * rotate calls (python/src/binding.cu:529-533 calling src/evaluate.cu:1665).  outs[i] equals
 * hoisting(ct, {steps[i]}) (src/evaluate.cu:1670-1865) word for word: the same plaintext as
 * rotate(ct, steps[i]), with the noise of a mod-up taken before the permutation.  Each step
 * needs its own Galois key. */
int fhe_ckks_rotations_hoisted(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *ct, size_t chain_index,
                               const int *steps, size_t num_steps, const uint64_t *const *const *galois_keys,
                               uint64_t *const *outs, void *stream);

/* multiply_plain (include/evaluate.cuh:94-100, src/evaluate.cu:1224-1250, CKKS NTT form):
 * out (2 polys) = ct * pt, pt one polynomial over the same chain_index.  out may alias ct. */
int fhe_ckks_multiply_plain(const fhe_context *ctx, const uint64_t *ct, const uint64_t *pt, uint64_t *out,
                            size_t chain_index, void *stream);

/* add_inplace (include/evaluate.cuh:46, src/evaluate.cu:116-198): out = a + b, `size` polys. */
int fhe_ckks_add(const fhe_context *ctx, const uint64_t *a, const uint64_t *b, uint64_t *out, size_t size,
                 size_t chain_index, void *stream);

/* Baby-step/giant-step plaintext-matrix x ciphertext-vector product, the
 * bsgs_complete_from_cpu binding (python/src/binding.cu:507-595): D diagonals (device array
 * [D][limbs][N], already encoded at chain_index), G baby steps, B giant steps (G * B >= D);
 * out (2 polys at chain_index + 1) = Rescale(sum_g rot_{gG}(sum_b ct_b * diag_{gG+b})).
 * hoisted = 0 runs the reference's loop (one rotation per baby step, giant rotations by g*G,
 * keys for 1..G-1 and every g*G or their NAF parts) and gives its words exactly; hoisted = 1
 * computes the baby steps with one shared mod-up and the giant steps by Horner's rule with
 * rotations by G only (keys for 1..G-1 and G): the same plaintext, different noise.
 * scratch: fhe_bsgs_scratch_bytes(ctx, G) bytes of device memory. */
size_t fhe_bsgs_scratch_bytes(const fhe_context *ctx, size_t G);
int fhe_ckks_bsgs_matvec(const fhe_context *ctx, fhe_workspace *ws, uint64_t *scratch, const uint64_t *ct,
                         size_t chain_index, const uint64_t *diags, size_t D, size_t G, size_t B,
                         const uint64_t *const *const *galois_keys, uint64_t *out, int hoisted, void *stream);

/* A batch of matrix-vector products of the hoisted form above (baby steps sharing one mod-up,
 * giant steps by Horner's rule with rotations by G), one per ciphertext, at their own chain
 * indices (uneven levels allowed), sharing the Galois keys.  The reference serves such a batch
 * as a host loop of bsgs_complete_from_cpu (python/src/binding.cu:507-595); here every pipeline
 * step is one launch over up to 64 products, so each key is read once per launch set.  Each
 * output equals fhe_ckks_bsgs_matvec(..., hoisted = 1) word for word.  ws must come from
 * fhe_workspace_create_batch with at least min(count, 64) slots; scratch holds min(count, 64) x
 * fhe_bsgs_batch_scratch_bytes(ctx, G, B) bytes (each product's babies and inner sums). */
size_t fhe_bsgs_batch_scratch_bytes(const fhe_context *ctx, size_t G, size_t B);
typedef struct fhe_matvec_item {
    const uint64_t *ct;     /* 2 polys at chain_index, NTT form */
    const uint64_t *diags;  /* D plaintexts [D][diag_limbs][N], NTT form; limbs [0, l) are read */
    uint64_t *out;          /* 2 polys at chain_index + 1 */
    size_t chain_index;
    size_t diag_limbs;      /* limbs per diagonal (its stride), from l (the limbs at chain_index) to
                             * the data primes; 0 means l.  Items of one matrix may share one array
                             * encoded at the top level: the batch then reads each diagonal tile once
                             * for all of them. */
} fhe_matvec_item;
int fhe_ckks_bsgs_matvec_batch(const fhe_context *ctx, fhe_workspace *ws, uint64_t *scratch,
                               const fhe_matvec_item *items, size_t count, size_t D, size_t G, size_t B,
                               const uint64_t *const *const *galois_keys, void *stream);

/* PhantomSecretKey::encrypt_symmetric, CKKS (src/secretkey.cu:463-500 with
 * encrypt_zero_symmetric, 232-295) with the randomness supplied by the caller instead of the
 * reference's device PRNG: out = (pt - (a*s + NTT(e)), a).  s and a in NTT form over the
 * ciphertext's limbs, e an int64 polynomial of N coefficients; pt may be NULL (zero). */
int fhe_ckks_encrypt_symmetric(const fhe_context *ctx, const uint64_t *pt, const uint64_t *s_ntt, const uint64_t *a,
                               const int64_t *e, uint64_t *out, size_t chain_index, void *stream);

/* PhantomCKKSEncoder::encode (include/ckks.h, src/ckks.cu:68-138): `count` (1 .. N/2) complex
 * slot values (device memory, interleaved re/im doubles) at `scale` -> plaintext pt [l][N]
 * (device, NTT form) at chain_index.  The reference's FP64 special FFT (src/fft.cu), rounding and
 * residues (src/rns_base.cu:49-163), so pt equals the reference's words.  Errors as the reference:
 * "Input vector is empty" / "exceeds max slots", "scale out of bounds", "encoded values are too
 * large" (FHE_ERR_INVALID_ARGUMENT).  Synchronises the stream once (the magnitude check). */
int fhe_ckks_encode(const fhe_context *ctx, fhe_workspace *ws, const double *values, size_t count, double scale,
                    size_t chain_index, uint64_t *pt, void *stream);

/* PhantomCKKSEncoder::decode (src/ckks.cu:340-400): pt [l][N] (device, NTT form) at chain_index
 * with its scale -> N/2 complex slots (device, interleaved re/im doubles): inverse NTT, CRT
 * compose over every limb (src/rns_base.cu:169-253), FP64 special FFT, bit for bit the
 * reference's. */
int fhe_ckks_decode(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *pt, size_t chain_index, double scale,
                    double *values, void *stream);

/* PhantomSecretKey::decrypt, CKKS (src/secretkey.cu:693-720): pt = c0 + c1 * s (NTT form). */
int fhe_ckks_decrypt(const fhe_context *ctx, const uint64_t *ct, const uint64_t *s_ntt, uint64_t *pt,
                     size_t chain_index, void *stream);

/* PhantomSecretKey::generate_one_kswitch_key (src/secretkey.cu:297-341) for create_relin_keys
 * (galois_elt = 0, source key s^2) and create_galois_keys (source key sigma_elt(s)), with the
 * randomness supplied by the caller: a = dnum uniform polynomials [dnum][QP][N] in NTT form,
 * e = dnum int64 error polynomials [dnum][N].  key receives [dnum][2][QP][N] with
 * key[d] = (-(a_d s + e_d) + (P mod q_j) s_src on digit d's limbs, a_d).  s_ntt covers QP. */
int fhe_kswitch_keygen(const fhe_context *ctx, fhe_workspace *ws, uint32_t galois_elt, const uint64_t *s_ntt,
                       const uint64_t *a, const int64_t *e, uint64_t *key, void *stream);

/* BFV plaintexts, word for word as the reference:
 *   fhe_bfv_encode   PhantomBatchEncoder::encode (src/batchencoder.cu:51-92): values (device,
 *                    count <= N slots; int64 values below zero are taken plus t) -> pt [N] mod t.
 *                    Needs t prime and t = 1 mod 2N.
 *   fhe_bfv_decode   PhantomBatchEncoder::decode (:100-118): pt [N] -> values [N].
 *   fhe_bfv_encrypt_symmetric  PhantomSecretKey::encrypt_symmetric for BFV (src/secretkey.cu:
 *                    463-485, scalingvariant.cu:10-31) at the first data level: a = uniform
 *                    [nQ][N] (as fhe_sample_uniform draws it), e = int64 [N]; out [2][nQ][N].
 *   fhe_bfv_decrypt  PhantomSecretKey::decrypt for BFV (src/secretkey.cu:571-635) with the HPS
 *                    scale-and-round (src/rns.cu:1519-1665): pt [N] mod t. */
int fhe_bfv_encode(const fhe_context *ctx, const uint64_t *values, size_t count, uint64_t *pt, void *stream);
int fhe_bfv_decode(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *pt, uint64_t *values, void *stream);
int fhe_bfv_encrypt_symmetric(const fhe_context *ctx, const uint64_t *pt, const uint64_t *s_ntt, const uint64_t *a,
                              const int64_t *e, uint64_t *out, void *stream);
int fhe_bfv_decrypt(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *ct, size_t chain_index,
                    const uint64_t *s_ntt, uint64_t *pt, void *stream);

/* The reference's device samplers, bit for bit (src/prng.cu:17-244): the same 64-byte seed gives
 * the same polynomial as the reference's sample_uniform_poly / sample_ternary_poly /
 * sample_error_poly.  seed is a host pointer to 64 bytes (global_variables::prng_seed_byte_count);
 * the generator reads the first 56.
 *   fhe_sample_uniform: out [limbs][N], limb k uniform modulo QP prime k (limbs <= |QP|).
 *   fhe_sample_ternary: out [N] int64 in {-1, 0, 1}; fhe_sample_cbd: out [N] int64 in [-21, 21]
 *   (the reference's per-limb residues of the same values). */
int fhe_sample_uniform(const fhe_context *ctx, const uint8_t *seed, size_t limbs, uint64_t *out, void *stream);
int fhe_sample_ternary(const fhe_context *ctx, const uint8_t *seed, int64_t *out, void *stream);
int fhe_sample_cbd(const fhe_context *ctx, const uint8_t *seed, int64_t *out, void *stream);

/* PhantomSecretKey::gen_secretkey (src/secretkey.cu:343-380) with the seed its random_bytes
 * would have drawn: s_ntt [QP][N] = NTT(ternary(seed)). */
int fhe_secret_key_from_seed(const fhe_context *ctx, fhe_workspace *ws, const uint8_t *seed, uint64_t *s_ntt,
                             void *stream);

/* generate_one_kswitch_key (src/secretkey.cu:297-341, encrypt_zero_symmetric :232-295) with the
 * reference's samplers: digit d's a = uniform(seeds_a + 64 d) over QP (NTT form as drawn) and
 * its error cbd(seeds_e + 64 d); otherwise as fhe_kswitch_keygen.  seeds_a and seeds_e are host
 * arrays of dnum 64-byte seeds. */
int fhe_kswitch_keygen_seeded(const fhe_context *ctx, fhe_workspace *ws, uint32_t galois_elt, const uint64_t *s_ntt,
                              const uint8_t *seeds_a, const uint8_t *seeds_e, uint64_t *key, void *stream);

#ifdef __cplusplus
}
#endif
#endif
