// ks_fused.cuh — the mod-up's forward NTT row pass fused with the key-switching inner product.
//
// The reference materialises the mod-up output t_mod_up[beta][l + alpha][N] (src/rns_bconv.cu:
// 530-628, forward NTT src/ntt/ntt_modup.cu:610-657) and then reads it back in the inner product
// (key_switch_inner_prod_c2_and_evk, src/eval_key_switch.cu:14-69):
//   cx_t[jj] = sum_{d < beta} T_d[jj] * evk_d[t][twr(jj)]  mod p_jj.
// Here one CTA owns one output limb jj and one tile of rows and walks every digit d: it finishes
// T_d[jj]'s transform over its tile (the row pass's stages, from the column pass's lazy output), or
// reads the digit's own limb (the input itself, already in NTT form), and multiplies the tile into
// 128-bit accumulators with the key words at the same positions.  T never goes back to HBM and is
// never re-read; cx is written once.  The words equal the two-kernel form's (exact modular
// arithmetic, the sum reduced every 7 terms as there).
//
// Layout per thread: the row pass's last register phase leaves each thread E coefficients (4 or 8)
// in runs of 2^K consecutive positions (the phase's smallest stride is 1), so the key words and
// the cx stores are 16-byte accesses at those positions, and no shared-memory sweep follows the
// transform.
//
// The accumulators (E coefficients x 2 polynomials x 128 bits a thread) live in tensor memory,
// not in registers: thread t owns lane t of the CTA's 8 E columns, one 16-column chunk per pair of
// its coefficients.  Each digit loads a chunk (tcgen05.ld), adds the pair's four products and
// stores it back (tcgen05.st), so 16 accumulator words are live at a time instead of 8 E, and the
// transform runs at the occupancy of the plain row pass.
#pragma once
#include "keyswitch.cuh"
#include "ntt.cuh"
#include "tc.cuh"

namespace pfg {

// CTA shape for FE coefficients per thread (128 threads): 4 for single ciphertexts, 8 for batches
// (measured: 4 per thread at 10 CTAs per SM took 125 us against 128 us at 8 per thread for one
// ciphertext; the batch, whose grid runs every item's blocks of one key tile together, was 1-2 %
// faster at 8 per thread).
template <int FE>
struct FusedShape {
    static_assert(FE == 4 || FE == 8, "4 or 8 coefficients per thread");
    static constexpr int kThreads = 128;
    static constexpr int kTile = kThreads * FE;  // coefficients per CTA
    static constexpr int kCols = FE * 2 * 4;     // tensor-memory columns: FE x 2 polynomials x 4 words
    // CTAs per SM: 8 x 64 columns fill the SM's 512 at 8 per thread; at 4 per thread the register
    // file bounds it (10 CTAs at 48 registers, 320 columns)
    static constexpr int kCtas = FE == 8 ? 8 : 10;
};
constexpr int kFusedSingleE = 4, kFusedBatchE = 8;

namespace tacc {
// One warp's 32 lanes x 16 consecutive 32-bit columns, one lane per thread.
__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}
// Waits for this thread's tensor-memory loads; the registers pass through, so no use of them
// moves above the wait.  These statements carry no memory clobber: the volatile statements keep
// their order among themselves, and global loads (the key words) may still move across them.
__device__ __forceinline__ void wait_ld(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]));
}
__device__ __forceinline__ void st16(uint32_t taddr, const uint32_t (&r)[16]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
                 ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
                   "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]));
}
// Waits for this thread's tensor-memory stores (before it loads the same columns again).
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;"); }

__device__ __forceinline__ u128 get(const uint32_t (&r)[16], int k) {
    return u128{(uint64_t)r[4 * k] | ((uint64_t)r[4 * k + 1] << 32), (uint64_t)r[4 * k + 2] | ((uint64_t)r[4 * k + 3] << 32)};
}
__device__ __forceinline__ void put(uint32_t (&r)[16], int k, const u128 &a) {
    r[4 * k] = (uint32_t)a.lo;
    r[4 * k + 1] = (uint32_t)(a.lo >> 32);
    r[4 * k + 2] = (uint32_t)a.hi;
    r[4 * k + 3] = (uint32_t)(a.hi >> 32);
}
}  // namespace tacc

// Shared-memory words of one CTA: its tile as V = TILE / M padded vectors of M = 2^LM words.
template <int LM, int FE>
__host__ __device__ constexpr int fused_smem_words() {
    return (FusedShape<FE>::kTile >> LM) * ((1 << LM) + (1 << LM) / 16 + 1);
}

// One CTA's work: output limb jj (prime table index tbl) of the rows in tile `tile`, over every
// digit d < beta.  tm and cx are the ciphertext's mod-up and accumulator buffers, sm the CTA's
// shared tile, tacc the tensor-memory address of this thread's lane (column 0).
template <int LM, int FE, class Own>
__device__ __forceinline__ void modup_ip_tile(uint64_t *sm, uint32_t tacc, const NttTables &T, const uint64_t *tm,
                                              const Own &own, const uint64_t *const *evk, uint64_t *cx, int l, int nQ,
                                              int alpha, int beta, int qp, int jj, uint32_t tile) {
    constexpr int E = FE, TILE = FusedShape<FE>::kTile;
    constexpr int M = 1 << LM, TPV = M / E, V = TILE / M, VP = M + M / 16 + 1;
    using F = PhaseAt<LM, true, 0, E>;
    using L = PhaseAt<LM, true, F::NPH - 1, E>;
    constexpr int LG = E >> L::K, LS = 1 << L::K;  // last phase: groups per thread, group size
    static_assert(LS % 2 == 0, "the last phase pairs consecutive positions");
    static_assert(V * VP == fused_smem_words<LM, FE>(), "shared tile size");
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
        // keep every sum below q * 2^64 (reduce128's precondition)
        const bool fold = terms == 7;
        if (fold) terms = 1;
        if (d > 0) tacc::wait_st();  // the previous digit's sums are in tensor memory
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
                // chunk i / 2: a0[i], a0[i + 1], a1[i], a1[i + 1]
                uint32_t r[16];
                u128 acc[4] = {u128{0, 0}, u128{0, 0}, u128{0, 0}, u128{0, 0}};
                if (d > 0) {
                    tacc::ld16(tacc + 8 * i, r);
                    tacc::wait_ld(r);
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        acc[k] = tacc::get(r, k);
                        if (fold) acc[k] = u128{reduce128(acc[k], md), 0};
                    }
                }
                mac(acc[0], x[i], w0.x);
                mac(acc[1], x[i + 1], w0.y);
                mac(acc[2], x[i], w1.x);
                mac(acc[3], x[i + 1], w1.y);
#pragma unroll
                for (int k = 0; k < 4; k++) tacc::put(r, k, acc[k]);
                tacc::st16(tacc + 8 * i, r);
            }
        terms++;
    }
    tacc::wait_st();
    const size_t total = (size_t)qlp << log_n;
    uint64_t *c0 = cx + ((size_t)jj << log_n);
#pragma unroll
    for (int gg = 0; gg < LG; gg++)
#pragma unroll
        for (int j = 0; j < LS; j += 2) {
            const uint32_t idx = vbase + grp_elem<LM, L::K, L::SA, E>(u, gg, j);
            const int i = gg * LS + j;
            uint32_t r[16];
            tacc::ld16(tacc + 8 * i, r);
            tacc::wait_ld(r);
            *reinterpret_cast<ulonglong2 *>(c0 + idx) =
                    make_ulonglong2(reduce128(tacc::get(r, 0), md), reduce128(tacc::get(r, 1), md));
            *reinterpret_cast<ulonglong2 *>(c0 + total + idx) =
                    make_ulonglong2(reduce128(tacc::get(r, 2), md), reduce128(tacc::get(r, 3), md));
        }
}

// The CTA's COLS tensor-memory columns: allocated by warp 0 after the grid dependency wait (so no
// CTA holds columns while it waits on another grid), freed once every thread's accesses are done.
// Eight CTAs of 64 columns fill an SM; a ninth would wait in the allocation until one finishes.
template <int COLS>
struct FusedTmem {
    __device__ __forceinline__ static uint32_t alloc(uint32_t *slot) {
        if (threadIdx.x < 32) tc::tmem_alloc(slot, COLS);
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        return *slot;
    }
    __device__ __forceinline__ static void free(uint32_t base) {
        tc::fence_before();
        __syncthreads();
        if (threadIdx.x < 32) {
            tc::fence_after();
            tc::tmem_free(base, COLS);
        }
    }
    // this thread's lane: warp w reads and writes lanes 32 w .. 32 w + 31
    __device__ __forceinline__ static uint32_t lane(uint32_t base) {
        return base + ((uint32_t)(threadIdx.x & ~31u) << 16);
    }
};

// One ciphertext: grid (N / TILE row tiles, l + alpha output limbs), kFusedSingleE per thread.
template <int LM, class Own>
__global__ void __launch_bounds__(FusedShape<kFusedSingleE>::kThreads, FusedShape<kFusedSingleE>::kCtas)
        ks_modup_ip(NttTables T, const uint64_t *tm, Own own, const uint64_t *const *evk, uint64_t *cx, int l,
                    int nQ, int alpha, int beta, int qp) {
    using S = FusedShape<kFusedSingleE>;
    using TM = FusedTmem<S::kCols>;
    pdl_wait();
    pdl_release();
    __shared__ uint64_t sm[fused_smem_words<LM, kFusedSingleE>()];
    __shared__ uint32_t tslot;
    const uint32_t tbase = TM::alloc(&tslot);
    modup_ip_tile<LM, kFusedSingleE>(sm, TM::lane(tbase), T, tm, own, evk, cx, l, nQ, alpha, beta, qp,
                                     (int)blockIdx.y, blockIdx.x);
    TM::free(tbase);
}

}  // namespace pfg
