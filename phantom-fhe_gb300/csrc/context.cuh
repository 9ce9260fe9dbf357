// context.cuh — device-resident parameter tables for one parameter set.
//
// Plays the role of the reference's PhantomContext + per-level DRNSTool
// (src/context.cu:121-232, src/rns.cu:11-195, 573-777): the modulus chain, the NTT tables
// of every prime (Q, P and the BFV HPS base R), the hybrid key-switching constants of every
// data level, the mod-down and rescale constants, the HPS scale-and-round constants and the
// Galois permutation tables.  Everything is built once on the host and uploaded; kernels
// read it through the small POD views below.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "ntt.cuh"
#include "tc.cuh"

namespace pfg {

// Default small-launch bounds for the 8-coefficients-per-thread NTT passes, in 4096-coefficient
// tiles, measured on GB300 with 1024-coefficient tiles for those passes and 2048 for the others.
// N >= 2^16 (30 + 5 primes): 512 — the 30-limb inverse transform and the 12-limb mod-down
// transform at 8 per thread, the 58-limb forward transform of the mod-down / rescale at 16 —
// gives HMult 0.4012 ms against 0.4028 at 1024 and 0.4169 at 4096.  N = 2^15 (BFV, 16 + 2
// primes): 1024 gives mult+relin 0.3677 ms against 0.3718 at 512.
constexpr int kNttSmallLaunchTiles = 512;
constexpr int kNttSmallLaunchTilesBelow2_16 = 1024;

// Block cap of the grid-stride element-wise kernels: 16 blocks of 256 threads per SM of GB300's
// 152 SMs (8 resident per SM, two waves); a larger grid only adds block scheduling.
constexpr int kGridStrideBlocks = 152 * 16;

// values of phantom::scheme_type (include/host/encryptionparams.h)
enum Scheme { kSchemeNone = 0, kSchemeBGV = 1, kSchemeBFV = 2, kSchemeCKKS = 3 };
enum MulTech { kMulNone = 0, kMulBEHZ = 1, kMulHPS = 2, kMulHPSOverQ = 3, kMulHPSOverQLeveled = 4 };

// Device memory owned by the context (plain cudaMalloc, freed in the destructor).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf();
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
    void upload(const void *src, size_t n);  // allocates n bytes and copies
};

// Per data level l (number of Q limbs): hybrid key-switching and rescale constants.
struct LevelTables {
    int l = 0, beta = 0;
    // partQlHatInv (value, Shoup) per Ql limb: inverse of (Q_digit / q_i) mod q_i
    DevBuf part_hat_inv;  // [l][2]
    // modup base-change rows M_d[jj][i] = (Q_digit / q_{s+i}) mod p_jj, zero rows for the
    // digit's own limbs: [beta][l + alpha][alpha]
    DevBuf modup_mat;
    // q_last^-1 mod q_j (value, Shoup), j < l - 1
    DevBuf inv_qlast;  // [l-1][2]
    // tensor-core mod-up: per digit, the byte planes of 2^(8a) M_d[jj][i] mod p_jj as a bf16
    // operand [256 rows = (output, plane)][kpad = (input limb, byte)] in the canonical K-major
    // layout (see tc.cuh); tc_ok when every digit has at most 32 outputs
    DevBuf tc_modup;
    DevBuf tc_modup_meta;  // [beta][32 positions]: output limb jj and 1/p_jj (f32), limbs below 2^40 first
    DevBuf tc_modup_nn;    // [beta]: number of positions below 2^40
    bool tc_ok = false;
    // tensor-core P -> Ql conversions (mod-down; mod-down fused with the rescale), one operand
    // [256][kpad] each, positions j < l (limbs below 2^40 first; rescale: j = l - 1 last)
    DevBuf tc_moddown, tc_moddown_meta, tc_rescale, tc_rescale_meta;
    int tc_moddown_nn = 0, tc_rescale_nn = 0;
    bool tc_moddown_ok = false, tc_rescale_ok = false;
};

// CKKS encoder: CRT-compose constants of base Q_l (one data level), little-endian words
struct ComposeTables {
    DevBuf q_prod;     // [l] Q_l
    DevBuf q_hat;      // [l][l] Q_l / q_i
    DevBuf q_hat_inv;  // [l][2] (Q_l / q_i)^-1 mod q_i (value, Shoup)
    DevBuf upper;      // [l] (Q_l + 1) / 2
    int bits = 0;      // significant bits of Q_l
};

struct Context {
    int scheme = kSchemeCKKS, mul_tech = kMulHPS;
    int log_n = 0;
    uint64_t n = 0;
    int nQ = 0, nP = 0, nR = 0;
    uint64_t t = 0;
    std::vector<uint64_t> mods;  // QP, then R (BFV HPS)
    DevBuf d_mods, d_tw, d_itw, d_ninv;
    // mod-down (level independent): PHatInv (value, Shoup) [nP][2]; (P/p_k) mod q_j [nQ][nP];
    // P^-1 mod q_j (value, Shoup) [nQ][2]
    DevBuf p_hat_inv, p_mat, p_inv;
    std::vector<std::unique_ptr<LevelTables>> levels;  // index l = 1..nQ
    // BFV HPS
    DevBuf hps_q_hat_inv, hps_r_hat_inv;   // [nQ][2], [nR][2]
    DevBuf hps_q_inv, hps_r_inv;           // 1/q_i, 1/r_j as doubles
    DevBuf hps_q2r_mat, hps_r2q_mat;       // [nR][nQ], [nQ][nR]
    DevBuf hps_q2r_alpha, hps_r2q_alpha;   // [nQ+1][nR], [nR+1][nQ]
    DevBuf hps_frac;                        // [nQ] doubles
    DevBuf hps_modr;                        // [nR][nQ+1]
    // tensor-core operands of the HPS contractions ([256][kp] bf16 byte planes): Q -> R and
    // R -> Q conversions (input limbs + the FP64 correction slot) and the scale-and-round QR -> R
    DevBuf tc_hps_q2r, tc_hps_r2q, tc_hps_scale;
    int tc_hps_kp_q2r = 0, tc_hps_kp_r2q = 0, tc_hps_kp_scale = 0;
    bool tc_hps_ok = false;
    // BFV plaintexts (PhantomBatchEncoder, src/batchencoder.cu; encrypt's scaling variant,
    // src/scalingvariant.cu; HPS decryption, src/rns.cu:1519-1665): the NTT table of t at index
    // plain_tbl (-1 when t is not 1 mod 2N: no batching), the slot -> coefficient map, -Q mod t and
    // t^-1 mod q_i, and per data level l (rows (l - 1) * nQ .. + l) the decryption constants
    // floor(t QHatInv_i / q_i) mod t (value, Shoup) and frac(t QHatInv_i / q_i), plus the same
    // with QHatInv_i * 2^(qMSB / 2) for the split variants.
    int plain_tbl = -1;
    DevBuf bfv_index_map;  // [N] u32
    uint64_t neg_q_mod_t = 0, neg_q_mod_t_shoup = 0;
    DevBuf bfv_t_inv;      // [nQ][2]
    DevBuf dec_mod_t, dec_mod_t_b;    // [nQ levels][nQ][2]
    DevBuf dec_frac, dec_frac_b;      // [nQ levels][nQ] doubles
    int q_msb = 0, t_msb = 0;
    // CKKS encoder (ckks_codec.cu): the 2N-th roots of unity as complex doubles [2N], the rotation
    // group 5^i mod 2N [N/4] (u32) and, per data level l (index l), the compose constants
    DevBuf codec_roots, codec_group;
    std::vector<std::unique_ptr<ComposeTables>> compose;
    // Galois
    std::vector<uint32_t> galois_elts;
    std::map<uint32_t, std::unique_ptr<DevBuf>> perms;
    std::mutex perm_mu;
    // tensor-core base conversions: available (alpha <= 6) and switched on
    bool tc_avail = false, tc_on = false;
    int tc_kpad = 0;  // K of the byte-plane GEMM: 8 alpha rounded up to 16
    int num_sms = 0;
    int smem_optin = 0;  // largest dynamic shared memory a block may opt in to (bytes)
    DevBuf d_status;  // device error word (bounded waits that gave up), read by fhe_context_status

    // NTT stage split: the column pass runs the first l1 stages, the row pass the other l2.  Any
    // supported split gives the same words; the autotuner (fhe_context_autotune) picks one.
    int l1_sel = 0;  // 0: log_n / 2
    // NTT passes over at most this many 4096-coefficient tiles run 8 coefficients per thread
    // (NttShape<8>); larger ones 16.  -1: the default for the degree (kNttSmallLaunchTiles*).
    int ntt_small_tiles = -1;
    // coefficients per CTA of those small passes (1024 or 2048) and of the larger, 16-per-thread
    // passes (2048 or 4096); smaller CTAs spread a launch more evenly over the SMs and wait less
    // at their barriers.  Any setting gives the same words.
    int ntt_small_tile = kTileElems / 4;
    int ntt_tile = kTileElems / 2;
    // kernel chains launched with programmatic dependent launch (pdl.cuh); any setting gives the
    // same words
    bool pdl = true;
    // mod-up row pass fused with the inner product (ks_fused.cuh) for single calls and for batches
    // (the autotuner sets only the first; fhe_context_set_fused_keyswitch sets both); any setting
    // gives the same words
    bool ks_fused = true, ks_fused_batch = true;
    // device the context's tables live on, and the device address of the fixed scratch array of
    // fhe_rescale_to_next_noalloc on it (looked up at creation, with that device current, so the
    // address belongs to the CUDA context the tables were made in)
    int device = 0;
    uint64_t *noalloc_scratch = nullptr;
    size_t noalloc_words = 0;
    long long ntt_small_limit() const {
        if (ntt_small_tiles >= 0) return ntt_small_tiles;
        return log_n >= 16 ? kNttSmallLaunchTiles : kNttSmallLaunchTilesBelow2_16;
    }
    int l1() const { return l1_sel ? l1_sel : log_n / 2; }
    int l2() const { return log_n - l1(); }
    bool split_ok(int l) const { return l >= 6 && l <= 8 && log_n - l >= 6 && log_n - l <= 9; }
    NttTables ntt() const {
        return NttTables{d_mods.as<Mod>(), d_tw.as<TwPair>(), d_itw.as<TwPair>(), d_ninv.as<uint64_t>(), log_n,
                         l1(), l2()};
    }
    int beta(int l) const { return (l + nP - 1) / nP; }
    // Table index of QlP limb jj at level l.
    int qlp_table(int l, int jj) const { return jj < l ? jj : nQ + (jj - l); }
    const uint32_t *perm_table(uint32_t elt);  // builds and caches on first use
};

// Builds the CKKS encoder's tables (ckks_codec.cu).
void build_codec_tables(Context &c);

// Device address and size (words) of the no-allocation scratch array on the current device
// (noalloc.cu); throws std::runtime_error when the lookup fails.
uint64_t *noalloc_scratch_address(size_t *words);

// Builds every table; throws std::invalid_argument / std::logic_error on bad parameters.
std::unique_ptr<Context> make_context(int scheme, int mul_tech, uint64_t n, const std::vector<uint64_t> &coeff_modulus,
                                      int special_size, uint64_t plain_modulus,
                                      const std::vector<uint32_t> &galois_elts);

}  // namespace pfg
