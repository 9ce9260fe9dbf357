// ops.hpp — internal orchestration entry points behind the C ABI (capi.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "context.cuh"
#include "phantom_gb300.h"

namespace pfg {

// Caller-provided scratch; carved into regions by each operation.
struct Workspace {
    uint64_t *base = nullptr;
    size_t words = 0;
};

size_t workspace_words(const Context &c);

struct StepKey {  // one hoisted rotation: permutation table + key digits (device array)
    const uint32_t *perm;
    const uint64_t *const *key;
};

struct BatchItem {  // one HMult+relin+rescale of a batch: inputs at level l, output at l - 1
    const uint64_t *ct1, *ct2;
    uint64_t *out;
    int l;
};
constexpr int kBatchLaunch = 64;  // ciphertexts per launch set (larger batches run in chunks)

struct KsItem {  // one key switch of a batch: ct (2 polys, in place) += KeySwitch(c2), level l
    uint64_t *ct;
    const uint64_t *c2;
    int l;
};

struct MatvecItem {  // one matrix-vector product of a batch: ct (2 polys) at level l, diags [D][dl][N]
    const uint64_t *ct;
    const uint64_t *diags;  // limbs [0, l) of each diagonal are read; dl >= l is the limb stride
    uint64_t *out;          // 2 polys at level l - 1
    int l, dl;
};

void ntt_forward(const Context &c, uint64_t *data, int polys, int limbs, int start, cudaStream_t s);
void ntt_inverse(const Context &c, uint64_t *data, int polys, int limbs, int start, cudaStream_t s);

// CKKS (NTT form).  l = number of Q limbs of the operands.
void ckks_tensor(const Context &c, uint64_t *ct1, const uint64_t *ct2, int l, cudaStream_t s);
void ckks_keyswitch(const Context &c, const Workspace &w, uint64_t *ct, const uint64_t *c2, int l,
                    const uint64_t *const *evk, cudaStream_t s);
void ckks_mul_relin(const Context &c, const Workspace &w, uint64_t *ct1, const uint64_t *ct2, int l,
                    const uint64_t *const *rlk, cudaStream_t s);
void ckks_mul_relin_rescale(const Context &c, const Workspace &w, const uint64_t *ct1, const uint64_t *ct2,
                            uint64_t *out, int l, const uint64_t *const *rlk, cudaStream_t s);
// Batched HMult + relin + rescale; item i uses scratch ws_base + (i % 64) * item_words.
void ckks_mul_relin_rescale_batch(const Context &c, uint64_t *ws_base, size_t item_words,
                                  const std::vector<BatchItem> &items, const uint64_t *const *rlk, cudaStream_t s);
void ckks_keyswitch_batch(const Context &c, uint64_t *ws_base, size_t item_words, const std::vector<KsItem> &items,
                          const uint64_t *const *evk, cudaStream_t s);
void ckks_bsgs_matvec_batch(Context &c, uint64_t *ws_base, size_t item_words, uint64_t *scratch_base,
                            size_t scratch_words, const std::vector<MatvecItem> &items, int D, int G, int B,
                            const uint64_t *const *const *galois_keys, cudaStream_t s);
void ckks_rescale(const Context &c, const Workspace &w, const uint64_t *in, uint64_t *out, int size, int l,
                  cudaStream_t s);
void ckks_apply_galois(const Context &c, const Workspace &w, uint64_t *ct, int l, const uint32_t *perm,
                       const uint64_t *const *gk, cudaStream_t s);
void ckks_hoisting(const Context &c, const Workspace &w, uint64_t *ct, int l, const std::vector<StepKey> &steps,
                   cudaStream_t s);

void ckks_rotations_hoisted(const Context &c, const Workspace &w, const uint64_t *ct, int l,
                            const std::vector<StepKey> &steps, const std::vector<uint64_t *> &outs, cudaStream_t s);
void ckks_multiply_plain(const Context &c, const uint64_t *ct, const uint64_t *pt, uint64_t *out, int l,
                         cudaStream_t s);
void ckks_add(const Context &c, const uint64_t *a, const uint64_t *b, uint64_t *out, int l, int polys,
              cudaStream_t s);
void ckks_rotate(Context &c, const Workspace &w, uint64_t *ct, int l, int step,
                 const uint64_t *const *const *galois_keys, cudaStream_t s);
size_t bsgs_scratch_words(const Context &c, int G);
size_t bsgs_batch_scratch_words(const Context &c, int G, int B);
void ckks_bsgs_matvec(Context &c, const Workspace &w, uint64_t *scratch, const uint64_t *ct, int l,
                      const uint64_t *diags, int D, int G, int B, const uint64_t *const *const *galois_keys,
                      uint64_t *out, bool hoisted, cudaStream_t s, int diag_limbs = 0);
void ckks_encrypt_sk(const Context &c, const uint64_t *m, const uint64_t *s_ntt, const uint64_t *a, const int64_t *e,
                     uint64_t *out, int l, cudaStream_t st);
void ckks_decrypt(const Context &c, const uint64_t *ct, const uint64_t *s_ntt, uint64_t *m, int l, cudaStream_t st);
// a: digit d's uniform polynomial at a + d * a_stride (words)
void kswitch_keygen(Context &c, uint32_t elt, const uint64_t *s_ntt, const uint64_t *a, size_t a_stride,
                    const int64_t *e, uint64_t *key, uint64_t *scratch, cudaStream_t st);
// dst[k][i] = e[i] mod q_k over the first `limbs` QP primes
void small_to_rns_launch(const Context &c, uint64_t *dst, const int64_t *e, int limbs, cudaStream_t st);

// The reference's device samplers (prng.cu) and key generation from seeds (64-byte seeds).
void sample_uniform(const Context &c, const uint8_t *seed, int limbs, uint64_t *out, cudaStream_t s);
void sample_small(const Context &c, const uint8_t *seed, int kind, int64_t *out, cudaStream_t s);
void secret_key_from_seed(const Context &c, const uint8_t *seed, uint64_t *s_ntt, int64_t *scratch, cudaStream_t s);
void kswitch_keygen_seeded(Context &c, uint32_t elt, const uint64_t *s_ntt, const uint8_t *seeds_a,
                           const uint8_t *seeds_e, uint64_t *key, uint64_t *scratch, cudaStream_t s);

// Autotuner (autotune.cu): times the context's benchmark operation over its kernel shapes.
using Tuning = fhe_tuning;
Tuning autotune_op(Context &c, const Workspace &w, const char *cache_path);
Tuning tuning_of(const Context &c);
void apply_tuning(Context &c, const Tuning &t);

// CKKS encoder (ckks_codec.cu): values are complex doubles (re, im) in device memory.
size_t codec_encode_words(const Context &c);
size_t codec_decode_words(const Context &c, int l);
void ckks_encode(const Context &c, const Workspace &w, const double *values, size_t count, double scale, int l,
                 uint64_t *pt, cudaStream_t s);
void ckks_decode(const Context &c, const Workspace &w, const uint64_t *pt, double scale, int l, double *values,
                 cudaStream_t s);

// BFV plaintexts (bfv_io.cu).
void bfv_encode(const Context &c, const uint64_t *values, size_t count, uint64_t *pt, cudaStream_t s);
void bfv_decode(const Context &c, const uint64_t *pt, uint64_t *values, uint64_t *scratch, cudaStream_t s);
void bfv_encrypt_sk(const Context &c, const uint64_t *m, const uint64_t *s_ntt, const uint64_t *a, const int64_t *e,
                    uint64_t *out, cudaStream_t s);
void bfv_decrypt(const Context &c, const uint64_t *ct, int l, const uint64_t *s_ntt, uint64_t *pt, uint64_t *scratch,
                 cudaStream_t s);

// BFV (coefficient form).
void bfv_keyswitch(const Context &c, const Workspace &w, uint64_t *ct, const uint64_t *c2, int l,
                   const uint64_t *const *evk, cudaStream_t s);
void bfv_mul_relin_hps(const Context &c, const Workspace &w, uint64_t *ct1, const uint64_t *ct2,
                       const uint64_t *const *rlk, cudaStream_t s);
void bfv_divide_round_q_last(const Context &c, const uint64_t *in, uint64_t *out, int size, int l, cudaStream_t s);

}  // namespace pfg
