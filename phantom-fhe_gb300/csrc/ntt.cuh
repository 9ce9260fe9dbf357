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
// stages a tile of V whole vectors (columns or rows, V*M = 4096 coefficients, 34 KB) in
// shared memory with one coalesced sweep, runs all of that pass's stages as register
// phases of up to four radix-2 stages (16 coefficients per thread, Harvey lazy butterflies,
// twiddle and Shoup quotient fetched as one 16-byte pair), and writes the tile back with one
// coalesced sweep.  Every launch covers all limbs (and polynomials) of an operation; the
// load and store sweeps take functors so neighbouring element-wise work (base-conversion
// input, scaling, mod-down combine, inner-product accumulation) fuses into the pass.
#pragma once
#include <cstdint>

#include "modarith.cuh"

namespace pfg {

// Twiddle pairs (w, floor(w * 2^64 / q)) for one prime: 2*N words.
struct TwPair {
    uint64_t w, ws;
};

__device__ __forceinline__ TwPair ld_tw(const TwPair *t, uint32_t idx) {
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(t) + idx);
    return TwPair{v.x, v.y};
}

constexpr int kNttThreads = 256;
constexpr int kTileElems = 4096;  // V * M coefficients per CTA

__host__ __device__ constexpr int ntt_num_phases(int lm) { return (lm + 3) / 4; }
__host__ __device__ constexpr int ntt_phase_len(int lm, int ph) {
    return lm / ntt_num_phases(lm) + (ph < lm % ntt_num_phases(lm) ? 1 : 0);
}
__host__ __device__ constexpr int ntt_phase_start(int lm, int ph) {
    return ph == 0 ? 0 : ntt_phase_start(lm, ph - 1) + ntt_phase_len(lm, ph - 1);
}
__host__ __device__ constexpr int pad_idx(int x) { return x + (x >> 4); }

// One register phase of the forward transform on vector `vec` (padded shared memory):
// local stages [sa, sa + K).  tb(s) = twiddle-table base for local stage s:
// (1 << (loff + s)) + (row << s).
template <int LM, int K, int SA>
__device__ __forceinline__ void fwd_phase(uint64_t *vec, int u, const TwPair *tw, int loff, uint32_t row,
                                          uint64_t q) {
    constexpr int sa = SA;
    constexpr int M = 1 << LM;
    constexpr int TPV = M / 16;  // threads per vector
    constexpr int G = 16 >> K;   // butterfly groups per thread
    constexpr int GS = 1 << K;   // group size
    const int tmin = M >> (sa + K);
    const uint64_t q2 = 2 * q;
#pragma unroll
    for (int gg = 0; gg < G; gg++) {
        const int g = u + gg * TPV;
        const int hi = g / tmin, lo = g % tmin;
        uint64_t x[GS];
#pragma unroll
        for (int j = 0; j < GS; j++) x[j] = vec[pad_idx((hi * GS + j) * tmin + lo)];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int h = GS >> (k + 1);
            const uint32_t tb = (1u << (loff + sa + k)) + (row << (sa + k)) + ((uint32_t)hi << k);
#pragma unroll
            for (int j = 0; j < GS; j++) {
                if (j & h) continue;
                const TwPair w = ld_tw(tw, tb + (j >> (K - k)));
                uint64_t a = csub(x[j], q2);
                uint64_t t = mul_shoup_lazy(x[j + h], w.w, w.ws, q);
                x[j] = a + t;
                x[j + h] = a - t + q2;
            }
        }
#pragma unroll
        for (int j = 0; j < GS; j++) vec[pad_idx((hi * GS + j) * tmin + lo)] = x[j];
    }
}

// One register phase of the inverse transform: local stages sa+K-1 down to sa.
// glob0 = global stage index of local stage 0; the global stage 0 butterfly applies n^-1
// to its sum output (its difference twiddle already carries n^-1).
template <int LM, int K, int SA>
__device__ __forceinline__ void inv_phase(uint64_t *vec, int u, const TwPair *itw, int loff, uint32_t row,
                                          uint64_t q, uint64_t ninv, uint64_t ninv_s) {
    constexpr int sa = SA;
    constexpr int M = 1 << LM;
    constexpr int TPV = M / 16;
    constexpr int G = 16 >> K;
    constexpr int GS = 1 << K;
    const int tmin = M >> (sa + K);
    const uint64_t q2 = 2 * q;
#pragma unroll
    for (int gg = 0; gg < G; gg++) {
        const int g = u + gg * TPV;
        const int hi = g / tmin, lo = g % tmin;
        uint64_t x[GS];
#pragma unroll
        for (int j = 0; j < GS; j++) x[j] = vec[pad_idx((hi * GS + j) * tmin + lo)];
#pragma unroll
        for (int k = K - 1; k >= 0; k--) {
            const int h = GS >> (k + 1);
            const uint32_t tb = (1u << (loff + sa + k)) + (row << (sa + k)) + ((uint32_t)hi << k);
            const bool first_stage = (sa + k == 0) && (loff == 0);
#pragma unroll
            for (int j = 0; j < GS; j++) {
                if (j & h) continue;
                const TwPair w = ld_tw(itw, tb + (j >> (K - k)));
                uint64_t a = x[j], b = x[j + h];
                uint64_t s = a + b;
                if (first_stage)
                    s = mul_shoup_lazy(s, ninv, ninv_s, q);
                else
                    s = csub(s, q2);
                x[j] = s;
                x[j + h] = mul_shoup_lazy(a - b + q2, w.w, w.ws, q);
            }
        }
#pragma unroll
        for (int j = 0; j < GS; j++) vec[pad_idx((hi * GS + j) * tmin + lo)] = x[j];
    }
}

template <int LM, int PH>
__device__ __forceinline__ void fwd_phases(uint64_t *vec, int u, const TwPair *tw, int loff, uint32_t row,
                                           uint64_t q) {
    if constexpr (PH < ntt_num_phases(LM)) {
        fwd_phase<LM, ntt_phase_len(LM, PH), ntt_phase_start(LM, PH)>(vec, u, tw, loff, row, q);
        __syncthreads();
        fwd_phases<LM, PH + 1>(vec, u, tw, loff, row, q);
    }
}

template <int LM, int PH>
__device__ __forceinline__ void inv_phases(uint64_t *vec, int u, const TwPair *itw, int loff, uint32_t row,
                                           uint64_t q, uint64_t ninv, uint64_t ninv_s) {
    if constexpr (PH >= 0) {
        inv_phase<LM, ntt_phase_len(LM, PH), ntt_phase_start(LM, PH)>(vec, u, itw, loff, row, q, ninv, ninv_s);
        __syncthreads();
        inv_phases<LM, PH - 1>(vec, u, itw, loff, row, q, ninv, ninv_s);
    }
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
// the last of its transform stores lazy values ([0, 4q) forward, [0, 2q) inverse); the last
// pass hands canonical values to its Store functor.

// Column pass: vectors are V consecutive columns, each of M = N1 elements (stride N2).
template <int LM, bool FWD, bool LAST, class Map, class Load, class Store>
__global__ void __launch_bounds__(kNttThreads) ntt_col_pass(NttTables T, Map map, Load ld, Store st) {
    constexpr int M = 1 << LM;
    constexpr int TPV = M / 16;
    constexpr int V = kTileElems / M;
    constexpr int VP = M + M / 16 + 1;  // padded vector length (odd: column sweeps hit distinct banks)
    __shared__ uint64_t sm[V * VP];
    int poly, k, tbl;
    if (!map((int)blockIdx.y, poly, k, tbl)) return;  // uniform per block, before any barrier
    const uint64_t q = T.mods[tbl].q;
    const int n2 = 1 << T.l2;
    const int c0 = blockIdx.x * V;
    // coalesced tile load: thread handles column c0 + (i % V), row i / V
    for (int i = threadIdx.x; i < V * M; i += kNttThreads) {
        const int v = i % V, r = i / V;
        sm[v * VP + pad_idx(r)] = ld(poly, k, tbl, (uint32_t)(r * n2 + c0 + v));
    }
    __syncthreads();
    const int vv = threadIdx.x / TPV, u = threadIdx.x % TPV;
    uint64_t *vec = sm + vv * VP;
    if constexpr (FWD) {
        fwd_phases<LM, 0>(vec, u, T.tw + (size_t)tbl * (1 << T.log_n), 0, 0u, q);
    } else {
        const uint64_t ni = T.ninv[2 * tbl], nis = T.ninv[2 * tbl + 1];
        inv_phases<LM, ntt_num_phases(LM) - 1>(vec, u, T.itw + (size_t)tbl * (1 << T.log_n), 0, 0u, q, ni, nis);
    }
    for (int i = threadIdx.x; i < V * M; i += kNttThreads) {
        const int v = i % V, r = i / V;
        uint64_t x = sm[v * VP + pad_idx(r)];
        if (LAST) {
            if (FWD) x = csub(x, 2 * q);
            x = csub(x, q);
        }
        st(poly, k, tbl, (uint32_t)(r * n2 + c0 + v), x);
    }
}

// Row pass: vectors are V consecutive rows of M = N2 contiguous elements.
template <int LM, bool FWD, bool LAST, class Map, class Load, class Store>
__global__ void __launch_bounds__(kNttThreads) ntt_row_pass(NttTables T, Map map, Load ld, Store st) {
    constexpr int M = 1 << LM;
    constexpr int TPV = M / 16;
    constexpr int V = kTileElems / M;
    constexpr int VP = M + M / 16 + 1;
    __shared__ uint64_t sm[V * VP];
    int poly, k, tbl;
    if (!map((int)blockIdx.y, poly, k, tbl)) return;  // uniform per block, before any barrier
    const uint64_t q = T.mods[tbl].q;
    const uint32_t base = blockIdx.x * kTileElems;
    for (int i = threadIdx.x; i < V * M; i += kNttThreads) {
        const int v = i / M, e = i % M;
        sm[v * VP + pad_idx(e)] = ld(poly, k, tbl, base + i);
    }
    __syncthreads();
    const int vv = threadIdx.x / TPV, u = threadIdx.x % TPV;
    const uint32_t row = blockIdx.x * V + vv;
    uint64_t *vec = sm + vv * VP;
    if constexpr (FWD) {
        fwd_phases<LM, 0>(vec, u, T.tw + (size_t)tbl * (1 << T.log_n), T.l1, row, q);
    } else {
        const uint64_t ni = T.ninv[2 * tbl], nis = T.ninv[2 * tbl + 1];
        inv_phases<LM, ntt_num_phases(LM) - 1>(vec, u, T.itw + (size_t)tbl * (1 << T.log_n), T.l1, row, q, ni,
                                               nis);
    }
    for (int i = threadIdx.x; i < V * M; i += kNttThreads) {
        const int v = i / M, e = i % M;
        uint64_t x = sm[v * VP + pad_idx(e)];
        if (LAST) {
            if (FWD) x = csub(x, 2 * q);
            x = csub(x, q);
        }
        st(poly, k, tbl, base + i, x);
    }
}

}  // namespace pfg
