// ks_fused.cuh — the mod-up's forward NTT row pass fused with the key-switching inner product.
//
// The reference materialises the mod-up output t_mod_up[beta][l + alpha][N] (src/rns_bconv.cu:
// 530-628, forward NTT src/ntt/ntt_modup.cu:610-657) and then reads it back in the inner product
// (key_switch_inner_prod_c2_and_evk, src/eval_key_switch.cu:14-69):
//   cx_t[jj] = sum_{d < beta} T_d[jj] * evk_d[t][twr(jj)]  mod p_jj.
// Here one CTA owns one output limb jj and one tile of rows and walks every digit d: it finishes
// T_d[jj]'s transform over its tile (the row pass's stages, from the column pass's lazy output), or
// reads the digit's own limb (the input itself, already in NTT form), and multiplies the tile into
// 128-bit accumulators held in registers with the key words at the same positions.  T never goes
// back to HBM and is never re-read; cx is written once.  The words equal the two-kernel form's
// (exact modular arithmetic, the sum reduced every 7 terms as there).
//
// Layout per thread: the row pass's last register phase leaves each thread E = 8 coefficients in
// runs of 2^K consecutive positions (the phase's smallest stride is 1), so the key words and the
// cx stores are 16-byte accesses at those positions, and no shared-memory sweep follows the
// transform.
#pragma once
#include "keyswitch.cuh"
#include "ntt.cuh"

namespace pfg {

constexpr int kFusedE = 8;       // coefficients per thread
constexpr int kFusedTile = 1024; // coefficients per CTA (128 threads)

// Shared-memory words of one CTA: its tile as V = TILE / M padded vectors of M = 2^LM words.
template <int LM>
__host__ __device__ constexpr int fused_smem_words() {
    return (kFusedTile >> LM) * ((1 << LM) + (1 << LM) / 16 + 1);
}

// One CTA's work: output limb jj (prime table index tbl) of the rows in tile `tile`, over every
// digit d < beta.  tm and cx are the ciphertext's mod-up and accumulator buffers, sm the CTA's
// shared tile.
template <int LM, class Own>
__device__ __forceinline__ void modup_ip_tile(uint64_t *sm, const NttTables &T, const uint64_t *tm, const Own &own,
                                              const uint64_t *const *evk, uint64_t *cx, int l, int nQ, int alpha,
                                              int beta, int qp, int jj, uint32_t tile) {
    constexpr int E = kFusedE, TILE = kFusedTile;
    constexpr int M = 1 << LM, TPV = M / E, V = TILE / M, VP = M + M / 16 + 1;
    using F = PhaseAt<LM, true, 0, E>;
    using L = PhaseAt<LM, true, F::NPH - 1, E>;
    constexpr int LG = E >> L::K, LS = 1 << L::K;  // last phase: groups per thread, group size
    static_assert(LS % 2 == 0, "the last phase pairs consecutive positions");
    static_assert(V * VP == fused_smem_words<LM>(), "shared tile size");
    const int log_n = T.log_n;
    const int qlp = l + alpha;
    const int tbl = jj < l ? jj : nQ + (jj - l);
    const Mod md = T.mods[tbl];
    const int vv = threadIdx.x / TPV, u = threadIdx.x % TPV;
    const uint32_t row = tile * V + vv;
    const uint32_t vbase = tile * TILE + vv * M;  // this thread's row within the limb
    uint64_t *vec = sm + vv * VP;
    const int own_d = jj < l ? jj / alpha : -1;
    const TwPair *tw = T.tw + ((size_t)tbl << log_n);
    u128 a0[E], a1[E];
#pragma unroll
    for (int i = 0; i < E; i++) a0[i] = a1[i] = u128{0, 0};
    int terms = 0;
    for (int d = 0; d < beta; d++) {
        uint64_t x[E];
        if (d == own_d) {
#pragma unroll
            for (int gg = 0; gg < LG; gg++)
#pragma unroll
                for (int j = 0; j < LS; j += 2) {
                    const uint32_t idx = vbase + grp_elem<LM, L::K, L::SA, E>(u, gg, j);
                    x[gg * LS + j] = own(jj, md, idx);
                    x[gg * LS + j + 1] = own(jj, md, idx + 1);
                }
        } else {
            __syncthreads();  // the previous digit's shared-memory reads are done
            const uint64_t *src = tm + (((size_t)d * qlp + jj) << log_n) + vbase;
#pragma unroll
            for (int gg = 0; gg < (E >> F::K); gg++)
#pragma unroll
                for (int j = 0; j < (1 << F::K); j++)
                    x[gg * (1 << F::K) + j] = __ldcs(src + grp_elem<LM, F::K, F::SA, E>(u, gg, j));
            run_pass<LM, true, E>(x, vec, u, tw, T.l1, row, md.q, 0, 0, 0);
#pragma unroll
            for (int i = 0; i < E; i++) x[i] = fwd_canonical(x[i], md);
        }
        if (terms == 7) {  // keep every sum below q * 2^64 (reduce128's precondition)
#pragma unroll
            for (int i = 0; i < E; i++) {
                a0[i] = u128{reduce128(a0[i], md), 0};
                a1[i] = u128{reduce128(a1[i], md), 0};
            }
            terms = 1;
        }
        const uint64_t *k0 = evk[d] + ((size_t)tbl << log_n), *k1 = evk[d] + ((size_t)(qp + tbl) << log_n);
#pragma unroll
        for (int gg = 0; gg < LG; gg++)
#pragma unroll
            for (int j = 0; j < LS; j += 2) {
                const uint32_t idx = vbase + grp_elem<LM, L::K, L::SA, E>(u, gg, j);
                const int i = gg * LS + j;
                // the key is read once per call: streaming loads
                const ulonglong2 w0 = __ldcs(reinterpret_cast<const ulonglong2 *>(k0 + idx));
                const ulonglong2 w1 = __ldcs(reinterpret_cast<const ulonglong2 *>(k1 + idx));
                mac(a0[i], x[i], w0.x);
                mac(a0[i + 1], x[i + 1], w0.y);
                mac(a1[i], x[i], w1.x);
                mac(a1[i + 1], x[i + 1], w1.y);
            }
        terms++;
    }
    const size_t total = (size_t)qlp << log_n;
    uint64_t *c0 = cx + ((size_t)jj << log_n);
#pragma unroll
    for (int gg = 0; gg < LG; gg++)
#pragma unroll
        for (int j = 0; j < LS; j += 2) {
            const uint32_t idx = vbase + grp_elem<LM, L::K, L::SA, E>(u, gg, j);
            const int i = gg * LS + j;
            *reinterpret_cast<ulonglong2 *>(c0 + idx) =
                    make_ulonglong2(reduce128(a0[i], md), reduce128(a0[i + 1], md));
            *reinterpret_cast<ulonglong2 *>(c0 + total + idx) =
                    make_ulonglong2(reduce128(a1[i], md), reduce128(a1[i + 1], md));
        }
}

// One ciphertext: grid (N / TILE row tiles, l + alpha output limbs).
template <int LM, class Own>
__global__ void __launch_bounds__(kFusedTile / kFusedE, 4)
        ks_modup_ip(NttTables T, const uint64_t *tm, Own own, const uint64_t *const *evk, uint64_t *cx, int l,
                    int nQ, int alpha, int beta, int qp) {
    pdl_wait();
    pdl_release();
    __shared__ uint64_t sm[fused_smem_words<LM>()];
    modup_ip_tile<LM>(sm, T, tm, own, evk, cx, l, nQ, alpha, beta, qp, (int)blockIdx.y, blockIdx.x);
}

}  // namespace pfg
