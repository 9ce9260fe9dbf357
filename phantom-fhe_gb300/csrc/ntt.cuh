// ntt.cuh — negacyclic NTT / inverse NTT over RNS limbs for sm_103a.
//
// Computes the same transform as the reference's nwt_2d_radix8_forward_inplace /
// nwt_2d_radix8_backward_inplace (src/ntt/fntt_2d.cu:620-653, src/ntt/intt_2d.cu:724-757):
// Cooley-Tukey forward with bit-reversed powers of the minimal primitive 2N-th root,
// Gentleman-Sande inverse with n^-1 folded into the last stage, canonical outputs.
//
// Design.  N = N1 * N2 (N1 = 2^L1 rows, N2 = 2^L2 columns of the row-major limb).  The first
// L1 stages only pair elements of the same column, the last L2 stages only pair elements of
// the same row, so a transform is two passes: a column pass and a row pass.  Each CTA
// stages a tile of V whole vectors (columns or rows, V*M = 1024, 2048 or 4096 coefficients,
// 9-34 KB) in shared memory with one coalesced sweep, runs all of that pass's stages as
// register phases of up to four radix-2 stages (16 coefficients per thread; 8 and radix-8
// phases for small launches, see NttShape; Harvey-style lazy butterflies, twiddle and Shoup
// quotient fetched as one 16-byte pair), and writes the tile back with one coalesced sweep.  Every launch covers all limbs (and polynomials) of an operation; the
// load and store sweeps take functors so neighbouring element-wise work (base-conversion
// input, scaling, mod-down combine, inner-product accumulation) fuses into the pass.
#pragma once
#include <cstdint>

#include "modarith.cuh"
#include "pdl.cuh"

namespace pfg {

// Twiddle pairs (w, floor(w * 2^64 / q)) for one prime: 2*N words.
struct TwPair {
    uint64_t w, ws;
};

__device__ __forceinline__ TwPair ld_tw(const TwPair *t, uint32_t idx) {
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(t) + idx);
    return TwPair{v.x, v.y};
}

constexpr int kTileElems = 4096;  // V * M coefficients per CTA

// E coefficients per thread: 16 (radix-16 register phases) for large launches, or 8 (radix-8
// phases: half the serial work per thread) for launches of a few waves, which are
// latency-bound.  A tile holds TILE = 4096, 2048 or 1024 coefficients, TILE / E threads: the
// smaller tiles give more, smaller CTAs, which spread a launch of a few hundred tiles evenly
// over the SMs and stall less at their barriers (the defaults are 2048 at E = 16, 128 threads,
// and 1024 at E = 8, 128 threads).
template <int E, int TILE = kTileElems>
struct NttShape {
    static_assert(E == 4 || E == 8 || E == 16, "4, 8 or 16 coefficients per thread");
    static_assert(TILE == kTileElems || TILE == kTileElems / 2 || TILE == kTileElems / 4,
                  "4096, 2048 or 1024 coefficients per tile");
    static constexpr int LGE = E == 16 ? 4 : E == 8 ? 3 : 2;
    static constexpr int kThreads = TILE / E;
    // 80 registers a thread at 16 per thread, 64 at 8
    static constexpr int kMinBlocks = (E == 16 ? 3 : 2) * (kTileElems / TILE);
};

__host__ __device__ constexpr int ntt_num_phases(int lm, int lge) { return (lm + lge - 1) / lge; }
__host__ __device__ constexpr int ntt_phase_len(int lm, int ph, int lge) {
    return lm / ntt_num_phases(lm, lge) + (ph < lm % ntt_num_phases(lm, lge) ? 1 : 0);
}
__host__ __device__ constexpr int ntt_phase_start(int lm, int ph, int lge) {
    return ph == 0 ? 0 : ntt_phase_start(lm, ph - 1, lge) + ntt_phase_len(lm, ph - 1, lge);
}
__host__ __device__ constexpr int pad_idx(int x) { return x + (x >> 4); }

// Position inside the vector of member j of thread u's gg-th butterfly group in the phase
// covering local stages [SA, SA + K): groups are {(hi * 2^K + j) * tmin + lo}, tmin = M >> (SA+K).
template <int LM, int K, int SA, int E>
__device__ __forceinline__ int grp_elem(int u, int gg, int j) {
    constexpr int M = 1 << LM, TPV = M / E, TMIN = M >> (SA + K);
    const int g = u + gg * TPV;
    return ((g / TMIN) * (1 << K) + j) * TMIN + (g % TMIN);
}

// Forward (Cooley-Tukey) stages [SA, SA+K) on the E registers of thread u, Harvey-style lazy
// with the truncated-quotient product: inputs and outputs in [0, 8q) (8q < 2^64: every prime is
// below 2^61).  Butterfly: a = csub(x, 4q) < 4q, b = y * w in [0, 4q) (mul_shoup_lazy4), outputs
// a + b and a - b + 4q.  Twiddle for local stage s of vector `row`:
// tw[(1 << (loff + s)) + (row << s) + (element >> (LM - s))].  All of a group's twiddle pairs
// are fetched before its butterflies so their latency overlaps.
//
// SMALLQ (q < kFwdSmallQ): the csub is dropped, so each stage widens the range by 4q; after all
// stages of a transform of up to 2^17 coefficients the values stay below (8 + 4 * 17) q < 2^64,
// and the last pass reduces them with one truncated Barrett quotient (fwd_canonical).
template <int LM, int K, int SA, int E, bool SMALLQ>
__device__ __forceinline__ void fwd_regs(uint64_t (&x)[E], int u, const TwPair *tw, int loff, uint32_t row,
                                         uint64_t q) {
    constexpr int M = 1 << LM, TPV = M / E, G = E >> K, GS = 1 << K, TMIN = M >> (SA + K);
    const uint64_t q4 = 4 * q, nq = 0 - q;
#pragma unroll
    for (int gg = 0; gg < G; gg++) {
        const uint32_t hi = (uint32_t)((u + gg * TPV) / TMIN);
        TwPair w[GS - 1];
#pragma unroll
        for (int k = 0; k < K; k++)
#pragma unroll
            for (int m = 0; m < (1 << k); m++)
                w[(1 << k) - 1 + m] = ld_tw(tw, (1u << (loff + SA + k)) + (row << (SA + k)) + (hi << k) + m);
        uint64_t *y = x + gg * GS;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int h = GS >> (k + 1);
#pragma unroll
            for (int j = 0; j < GS; j++) {
                if (j & h) continue;
                const TwPair t = w[(1 << k) - 1 + (j >> (K - k))];
                const uint64_t a = SMALLQ ? y[j] : csub(y[j], q4);
                const uint64_t b = mul_shoup_lazy4n(y[j + h], t.w, t.ws, nq);
                y[j] = a + b;
                y[j + h] = a - b + q4;
            }
        }
    }
}

// Inverse (Gentleman-Sande) stages SA+K-1 .. SA, inputs and outputs in [0, 4q): sum a + b < 8q
// reduced by csub(., 4q), difference (a - b + 4q) * w in [0, 4q) (mul_shoup_lazy4).  The global
// stage-0 butterfly (loff == 0, local stage 0) scales its sum by n^-1 instead; its difference
// twiddle already carries n^-1 (src/host/ntt.cu:53-55).
//
// SMALLQ (q < kInvSmallQ): the sum's csub is dropped.  After d inverse stages every value lies
// below B_d = 4q 2^d (a sum doubles the bound, a product resets it to 4q), so the difference
// is taken as a - b + B_d; dep0 is the number of stages the transform's earlier pass ran.  With
// at most 17 stages, 2 B_17 = q 2^20 < 2^64, and the last stage's outputs are products again.
template <int LM, int K, int SA, int E, bool SMALLQ>
__device__ __forceinline__ void inv_regs(uint64_t (&x)[E], int u, const TwPair *itw, int loff, uint32_t row,
                                         uint64_t q, uint64_t ninv, uint64_t ninv_s, int dep0) {
    constexpr int M = 1 << LM, TPV = M / E, G = E >> K, GS = 1 << K, TMIN = M >> (SA + K);
    const uint64_t q4 = 4 * q, nq = 0 - q;
#pragma unroll
    for (int gg = 0; gg < G; gg++) {
        const uint32_t hi = (uint32_t)((u + gg * TPV) / TMIN);
        TwPair w[GS - 1];
#pragma unroll
        for (int k = 0; k < K; k++)
#pragma unroll
            for (int m = 0; m < (1 << k); m++)
                w[(1 << k) - 1 + m] = ld_tw(itw, (1u << (loff + SA + k)) + (row << (SA + k)) + (hi << k) + m);
        uint64_t *y = x + gg * GS;
#pragma unroll
        for (int k = K - 1; k >= 0; k--) {
            const int h = GS >> (k + 1);
            const bool first_stage = (SA + k == 0) && (loff == 0);
            const uint64_t bnd = SMALLQ ? q4 << (dep0 + (LM - 1 - (SA + k))) : q4;
#pragma unroll
            for (int j = 0; j < GS; j++) {
                if (j & h) continue;
                const TwPair t = w[(1 << k) - 1 + (j >> (K - k))];
                const uint64_t a = y[j], b = y[j + h];
                const uint64_t s = a + b;
                y[j] = first_stage ? mul_shoup_lazy4n(s, ninv, ninv_s, nq) : (SMALLQ ? s : csub(s, q4));
                y[j + h] = mul_shoup_lazy4n(a - b + bnd, t.w, t.ws, nq);
            }
        }
    }
}

template <int LM, int K, int SA, int E>
__device__ __forceinline__ void grp_store(const uint64_t (&x)[E], uint64_t *vec, int u) {
    constexpr int G = E >> K, GS = 1 << K;
#pragma unroll
    for (int gg = 0; gg < G; gg++)
#pragma unroll
        for (int j = 0; j < GS; j++) vec[pad_idx(grp_elem<LM, K, SA, E>(u, gg, j))] = x[gg * GS + j];
}

template <int LM, int K, int SA, int E>
__device__ __forceinline__ void grp_load(uint64_t (&x)[E], const uint64_t *vec, int u) {
    constexpr int G = E >> K, GS = 1 << K;
#pragma unroll
    for (int gg = 0; gg < G; gg++)
#pragma unroll
        for (int j = 0; j < GS; j++) x[gg * GS + j] = vec[pad_idx(grp_elem<LM, K, SA, E>(u, gg, j))];
}

// Phase order: forward runs phases 0..NPH-1, inverse NPH-1..0.
template <int LM, bool FWD, int PI, int E>
struct PhaseAt {
    static constexpr int NPH = ntt_num_phases(LM, NttShape<E>::LGE);
    static constexpr int PH = FWD ? PI : NPH - 1 - PI;
    static constexpr int K = ntt_phase_len(LM, PH, NttShape<E>::LGE);
    static constexpr int SA = ntt_phase_start(LM, PH, NttShape<E>::LGE);
};

// Runs processing steps PI..NPH-1 on the registers; between steps the vector goes through
// shared memory (group_store, barrier, group_load of the next step's groups).
template <int LM, bool FWD, int PI, int E, bool SMALLQ>
__device__ __forceinline__ void run_phases(uint64_t (&x)[E], uint64_t *vec, int u, const TwPair *tw, int loff,
                                           uint32_t row, uint64_t q, uint64_t ninv, uint64_t ninv_s, int dep0) {
    using P = PhaseAt<LM, FWD, PI, E>;
    if constexpr (FWD)
        fwd_regs<LM, P::K, P::SA, E, SMALLQ>(x, u, tw, loff, row, q);
    else
        inv_regs<LM, P::K, P::SA, E, SMALLQ>(x, u, tw, loff, row, q, ninv, ninv_s, dep0);
    if constexpr (PI + 1 < P::NPH) {
        using Q = PhaseAt<LM, FWD, PI + 1, E>;
        grp_store<LM, P::K, P::SA, E>(x, vec, u);
        __syncthreads();
        grp_load<LM, Q::K, Q::SA, E>(x, vec, u);
        run_phases<LM, FWD, PI + 1, E, SMALLQ>(x, vec, u, tw, loff, row, q, ninv, ninv_s, dep0);
    }
}

// Prime classes of the lazy butterflies (uniform per CTA: one limb per block): below these
// bounds the forward / inverse butterflies skip their conditional subtractions (fwd_regs,
// inv_regs).  Forward: (8 + 4 * 17) q < 2^64; inverse: 2 * 4q * 2^17 < 2^64.
constexpr uint64_t kFwdSmallQ = uint64_t(1) << 57;
constexpr uint64_t kInvSmallQ = uint64_t(1) << 44;

template <int LM, bool FWD, int E>
__device__ __forceinline__ void run_pass(uint64_t (&x)[E], uint64_t *vec, int u, const TwPair *tw, int loff,
                                         uint32_t row, uint64_t q, uint64_t ninv, uint64_t ninv_s, int dep0) {
    if (q < (FWD ? kFwdSmallQ : kInvSmallQ))
        run_phases<LM, FWD, 0, E, true>(x, vec, u, tw, loff, row, q, ninv, ninv_s, dep0);
    else
        run_phases<LM, FWD, 0, E, false>(x, vec, u, tw, loff, row, q, ninv, ninv_s, dep0);
}

// Canonical residue of a forward transform's output: [0, 8q) for the large class, below
// (8 + 4 log N) q for the small one (any value below 2^64: the truncated Barrett quotient by
// floor(2^64 / q) is short by at most 3, so x - t q lies in [0, 4q)).
__device__ __forceinline__ uint64_t fwd_canonical(uint64_t y, const Mod &m) {
    if (m.q < kFwdSmallQ) {
        y -= mulhi_trunc(y, m.mu_hi) * m.q;
        return csub(csub(y, 2 * m.q), m.q);
    }
    return csub(csub(csub(y, 4 * m.q), 2 * m.q), m.q);
}

struct NttTables {
    const Mod *mods;     // [primes]
    const TwPair *tw;    // [primes][N] forward
    const TwPair *itw;   // [primes][N] inverse (n^-1 folded into entry 1)
    const uint64_t *ninv;  // [primes][2]: n^-1, Shoup quotient
    int log_n, l1, l2;
};

// ---------------------------------------------------------------- generic pass kernels
//
// Map: bool operator()(int block_y, int &poly, int &limb, int &tbl) const — false idles the block.
// Functor interfaces (all device, all per coefficient):
//   Load:  uint64_t operator()(int poly, int limb, int tbl, uint32_t idx) const
//   Store: void operator()(int poly, int limb, int tbl, uint32_t idx, uint64_t v) const
// `idx` is the coefficient index within the limb (row * N2 + column).  A pass that is not
// the last of its transform stores lazy values ([0, 8q) forward, [0, 4q) inverse); the last
// pass hands canonical values to its Store functor.

// Column pass: vectors are V consecutive columns, each of M = N1 elements (stride N2).  Thread
// t works on column t % V, so every global access of a warp covers whole row segments of V
// words (128 bytes for 4096-coefficient tiles up to N1 = 256); the first and last register
// phases load and store global memory directly.
template <int LM, bool FWD, bool LAST, class Map, class Load, class Store, int E = 16, int TILE = kTileElems>
__global__ void __launch_bounds__(NttShape<E, TILE>::kThreads, NttShape<E, TILE>::kMinBlocks)
        ntt_col_pass(NttTables T, Map map, Load ld, Store st) {
    pdl_wait();
    pdl_release();
    constexpr int M = 1 << LM;
    constexpr int V = TILE / M;
    constexpr int VP = M + M / 16 + 1;  // padded vector length (odd: column sweeps hit distinct banks)
    using F = PhaseAt<LM, FWD, 0, E>;
    using L = PhaseAt<LM, FWD, F::NPH - 1, E>;
    __shared__ uint64_t sm[V * VP];
    int poly, k, tbl;
    if (!map((int)blockIdx.y, poly, k, tbl)) return;  // uniform per block, before any barrier
    const uint64_t q = T.mods[tbl].q;
    const int n2 = 1 << T.l2;
    const int v = threadIdx.x % V, u = threadIdx.x / V;
    const uint32_t col = blockIdx.x * V + v;
    uint64_t x[E];
#pragma unroll
    for (int gg = 0; gg < (E >> F::K); gg++)
#pragma unroll
        for (int j = 0; j < (1 << F::K); j++)
            x[gg * (1 << F::K) + j] = ld(poly, k, tbl, (uint32_t)grp_elem<LM, F::K, F::SA, E>(u, gg, j) * n2 + col);
    uint64_t ni = 0, nis = 0;
    if constexpr (!FWD) {
        ni = T.ninv[2 * tbl];
        nis = T.ninv[2 * tbl + 1];
    }
    // the inverse column pass runs after the row pass's l2 stages
    run_pass<LM, FWD, E>(x, sm + v * VP, u, (FWD ? T.tw : T.itw) + ((size_t)tbl << T.log_n), 0, 0u, q, ni, nis,
                         FWD ? 0 : T.l2);
    Mod md{};
    if constexpr (FWD && LAST) md = T.mods[tbl];
#pragma unroll
    for (int gg = 0; gg < (E >> L::K); gg++)
#pragma unroll
        for (int j = 0; j < (1 << L::K); j++) {
            uint64_t y = x[gg * (1 << L::K) + j];
            if (LAST) {
                if (FWD)
                    y = fwd_canonical(y, md);
                else
                    y = csub(csub(y, 2 * q), q);
            }
            st(poly, k, tbl, (uint32_t)grp_elem<LM, L::K, L::SA, E>(u, gg, j) * n2 + col, y);
        }
}

// Row pass: vectors are V consecutive rows of M = N2 contiguous elements.  The forward pass
// loads its first phase directly (lane-contiguous) and stores through a coalesced sweep;
// the inverse pass loads through the sweep and stores its last phase directly.
template <int LM, bool FWD, bool LAST, class Map, class Load, class Store, int E = 16, int TILE = kTileElems>
__global__ void __launch_bounds__(NttShape<E, TILE>::kThreads, NttShape<E, TILE>::kMinBlocks)
        ntt_row_pass(NttTables T, Map map, Load ld, Store st) {
    pdl_wait();
    pdl_release();
    constexpr int M = 1 << LM;
    constexpr int TPV = M / E;
    constexpr int V = TILE / M;
    constexpr int VP = M + M / 16 + 1;
    constexpr int NT = NttShape<E, TILE>::kThreads;
    using F = PhaseAt<LM, FWD, 0, E>;
    using L = PhaseAt<LM, FWD, F::NPH - 1, E>;
    __shared__ uint64_t sm[V * VP];
    int poly, k, tbl;
    if (!map((int)blockIdx.y, poly, k, tbl)) return;  // uniform per block, before any barrier
    const uint64_t q = T.mods[tbl].q;
    const uint32_t base = blockIdx.x * TILE;
    const int vv = threadIdx.x / TPV, u = threadIdx.x % TPV;
    const uint32_t row = blockIdx.x * V + vv;
    uint64_t *vec = sm + vv * VP;
    uint64_t x[E];
    if constexpr (FWD) {
#pragma unroll
        for (int gg = 0; gg < (E >> F::K); gg++)
#pragma unroll
            for (int j = 0; j < (1 << F::K); j++)
                x[gg * (1 << F::K) + j] = ld(poly, k, tbl, base + vv * M + grp_elem<LM, F::K, F::SA, E>(u, gg, j));
    } else {
#pragma unroll 4
        for (int i = threadIdx.x; i < V * M; i += NT) sm[(i / M) * VP + pad_idx(i % M)] = ld(poly, k, tbl, base + i);
        __syncthreads();
        grp_load<LM, F::K, F::SA, E>(x, vec, u);
    }
    uint64_t ni = 0, nis = 0;
    if constexpr (!FWD) {
        ni = T.ninv[2 * tbl];
        nis = T.ninv[2 * tbl + 1];
    }
    run_pass<LM, FWD, E>(x, vec, u, (FWD ? T.tw : T.itw) + ((size_t)tbl << T.log_n), T.l1, row, q, ni, nis, 0);
    if constexpr (FWD) {
        grp_store<LM, L::K, L::SA, E>(x, vec, u);
        Mod md{};
        if constexpr (LAST) md = T.mods[tbl];
        __syncthreads();
#pragma unroll 4
        for (int i = threadIdx.x; i < V * M; i += NT) {
            uint64_t y = sm[(i / M) * VP + pad_idx(i % M)];
            if (LAST) y = fwd_canonical(y, md);
            st(poly, k, tbl, base + i, y);
        }
    } else {
#pragma unroll
        for (int gg = 0; gg < (E >> L::K); gg++)
#pragma unroll
            for (int j = 0; j < (1 << L::K); j++) {
                uint64_t y = x[gg * (1 << L::K) + j];
                if (LAST) y = csub(csub(y, 2 * q), q);
                st(poly, k, tbl, base + vv * M + grp_elem<LM, L::K, L::SA, E>(u, gg, j), y);
            }
    }
}

}  // namespace pfg
