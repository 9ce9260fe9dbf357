// launch.cuh — NTT pass dispatch, limb maps and the shared element-wise functors.
#pragma once
#include <cuda_runtime.h>

#include "context.cuh"
#include "ntt.cuh"

namespace pfg {

// Kernel launches issued by this library (all threads), for the benchmark's launch count.
void count_launch(unsigned n = 1);

// ---------------------------------------------------------------- limb maps
// A map turns blockIdx.y into (poly, limb k, prime table index) and may idle a block.

// Contiguous [poly][limbs][N] data, limb k uses prime table start + k.
struct SeqMap {
    int limbs, start;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &tbl) const {
        poly = b / limbs;
        k = b % limbs;
        tbl = start + k;
        return true;
    }
};

// The same data with the blocks ordered limb-major: consecutive blockIdx.y values take the
// same limb of successive polynomials, so the CTAs in flight share one limb's twiddle table
// (1 MB at N = 2^16) in L2 instead of cycling through every limb's.
struct LimbMajorMap {
    int polys, start;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &tbl) const {
        k = b / polys;
        poly = b % polys;
        tbl = start + k;
        return true;
    }
};

// QlP limbs [0, l + alpha) of `polys` polynomials at level l, starting at limb k0.
struct QlpMap {
    int limbs, k0, l, nQ;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &tbl) const {
        poly = b / limbs;
        k = k0 + b % limbs;
        tbl = k < l ? k : nQ + (k - l);
        return true;
    }
};

// Mod-up digits: block b -> digit d = b / qlp, QlP limb jj = b % qlp; the digit's own
// limbs idle when skip_own (they are already in NTT form, CKKS).
struct ModupMap {
    int qlp, l, nQ, alpha;
    bool skip_own;
    __device__ __forceinline__ bool operator()(int b, int &d, int &jj, int &tbl) const {
        d = b / qlp;
        jj = b % qlp;
        tbl = jj < l ? jj : nQ + (jj - l);
        if (skip_own && jj >= d * alpha && jj < d * alpha + alpha && jj < l) return false;
        return true;
    }
};

// ---------------------------------------------------------------- generic functors

// base[poly * ps + k * N + idx]; a streaming load: every NTT pass overwrites or abandons what it
// reads, so the line need not stay in L2
struct PtrLoad {
    const uint64_t *base;
    long long ps;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int poly, int k, int, uint32_t idx) const {
        return __ldcs(base + poly * ps + ((long long)k << log_n) + idx);
    }
};

struct PtrStore {
    uint64_t *base;
    long long ps;
    int log_n;
    __device__ __forceinline__ void operator()(int poly, int k, int, uint32_t idx, uint64_t v) const {
        base[poly * ps + ((long long)k << log_n) + idx] = v;
    }
};

// Stores v * s[k] mod q (s as (value, Shoup) pairs indexed by logical limb k - kofs).
struct ScaleStore {
    uint64_t *base;
    long long ps;
    int log_n, kofs;
    const uint64_t *s;
    const Mod *mods;
    __device__ __forceinline__ void operator()(int poly, int k, int tbl, uint32_t idx, uint64_t v) const {
        const int i = k - kofs;
        base[poly * ps + ((long long)k << log_n) + idx] = mul_shoup(v, s[2 * i], s[2 * i + 1], mods[tbl].q);
    }
};

// ---------------------------------------------------------------- pass launchers

template <bool FWD, bool LAST, int E, int TILE, class Map, class Load, class Store>
void col_pass_e(const Context &c, dim3 grid, Map m, Load ld, Store st, cudaStream_t s) {
    constexpr int NT = NttShape<E, TILE>::kThreads;
    const NttTables T = c.ntt();
    switch (c.l1()) {
        case 6: launch_pdl(c.pdl, ntt_col_pass<6, FWD, LAST, Map, Load, Store, E, TILE>, grid, dim3(NT), 0, s, T, m, ld, st); break;
        case 7: launch_pdl(c.pdl, ntt_col_pass<7, FWD, LAST, Map, Load, Store, E, TILE>, grid, dim3(NT), 0, s, T, m, ld, st); break;
        case 8: launch_pdl(c.pdl, ntt_col_pass<8, FWD, LAST, Map, Load, Store, E, TILE>, grid, dim3(NT), 0, s, T, m, ld, st); break;
        default: break;
    }
}

template <bool FWD, bool LAST, int E, int TILE, class Map, class Load, class Store>
void row_pass_e(const Context &c, dim3 grid, Map m, Load ld, Store st, cudaStream_t s) {
    constexpr int NT = NttShape<E, TILE>::kThreads;
    const NttTables T = c.ntt();
    switch (c.l2()) {
        case 6: launch_pdl(c.pdl, ntt_row_pass<6, FWD, LAST, Map, Load, Store, E, TILE>, grid, dim3(NT), 0, s, T, m, ld, st); break;
        case 7: launch_pdl(c.pdl, ntt_row_pass<7, FWD, LAST, Map, Load, Store, E, TILE>, grid, dim3(NT), 0, s, T, m, ld, st); break;
        case 8: launch_pdl(c.pdl, ntt_row_pass<8, FWD, LAST, Map, Load, Store, E, TILE>, grid, dim3(NT), 0, s, T, m, ld, st); break;
        case 9: launch_pdl(c.pdl, ntt_row_pass<9, FWD, LAST, Map, Load, Store, E, TILE>, grid, dim3(NT), 0, s, T, m, ld, st); break;
        default: break;
    }
}

// One pass over `blocks` limbs (blockIdx.y) of N / TILE tiles each (blockIdx.x).  Launches of
// at most c.ntt_small_limit() 4096-coefficient tiles take the 8-coefficients-per-thread kernels
// on tiles of c.ntt_small_tile coefficients; larger ones 16 per thread on c.ntt_tile.
template <bool COL, bool FWD, bool LAST, int E, class Map, class Load, class Store>
void pass_tiles(const Context &c, int tile, int blocks, Map m, Load ld, Store st, cudaStream_t s) {
    auto go = [&]<int TILE>() {
        const dim3 grid((unsigned)(c.n / TILE), (unsigned)blocks);
        if constexpr (COL)
            col_pass_e<FWD, LAST, E, TILE>(c, grid, m, ld, st, s);
        else
            row_pass_e<FWD, LAST, E, TILE>(c, grid, m, ld, st, s);
    };
    // built shapes: 16 per thread on 2048 or 4096 coefficients, 8 per thread on 1024 or 2048
    if constexpr (E == 16) {
        if (tile == kTileElems)
            go.template operator()<kTileElems>();
        else
            go.template operator()<kTileElems / 2>();
    } else {
        if (tile == kTileElems / 2)
            go.template operator()<kTileElems / 2>();
        else
            go.template operator()<kTileElems / 4>();
    }
}

template <bool FWD, bool LAST, class Map, class Load, class Store>
void col_pass(const Context &c, int blocks, Map m, Load ld, Store st, cudaStream_t s) {
    count_launch();
    if ((long long)(c.n / kTileElems) * blocks > c.ntt_small_limit())
        pass_tiles<true, FWD, LAST, 16>(c, c.ntt_tile, blocks, m, ld, st, s);
    else
        pass_tiles<true, FWD, LAST, 8>(c, c.ntt_small_tile, blocks, m, ld, st, s);
}

template <bool FWD, bool LAST, class Map, class Load, class Store>
void row_pass(const Context &c, int blocks, Map m, Load ld, Store st, cudaStream_t s) {
    count_launch();
    if ((long long)(c.n / kTileElems) * blocks > c.ntt_small_limit())
        pass_tiles<false, FWD, LAST, 16>(c, c.ntt_tile, blocks, m, ld, st, s);
    else
        pass_tiles<false, FWD, LAST, 8>(c, c.ntt_small_tile, blocks, m, ld, st, s);
}

// Forward transform: column pass (load functor) -> row pass (store functor); the
// intermediate lazy values go to `mid` (which may alias the final destination).
template <class Map, class Load, class Store>
void ntt_fwd(const Context &c, int blocks, Map m, Load ld, PtrStore mid, Store st, cudaStream_t s) {
    col_pass<true, false>(c, blocks, m, ld, mid, s);
    row_pass<true, true>(c, blocks, m, PtrLoad{mid.base, mid.ps, mid.log_n}, st, s);
}

// Inverse transform: row pass (load functor) -> column pass (store functor).
template <class Map, class Load, class Store>
void ntt_inv(const Context &c, int blocks, Map m, Load ld, PtrStore mid, Store st, cudaStream_t s) {
    row_pass<false, false>(c, blocks, m, ld, mid, s);
    col_pass<false, true>(c, blocks, m, PtrLoad{mid.base, mid.ps, mid.log_n}, st, s);
}

// Variants with separate intermediate store / load functors (batched, per-item buffers).
template <class Map, class Load, class MidStore, class MidLoad, class Store>
void ntt_fwd2(const Context &c, int blocks, Map m, Load ld, MidStore ms, MidLoad ml, Store st, cudaStream_t s) {
    col_pass<true, false>(c, blocks, m, ld, ms, s);
    row_pass<true, true>(c, blocks, m, ml, st, s);
}

template <class Map, class Load, class MidStore, class MidLoad, class Store>
void ntt_inv2(const Context &c, int blocks, Map m, Load ld, MidStore ms, MidLoad ml, Store st, cudaStream_t s) {
    row_pass<false, false>(c, blocks, m, ld, ms, s);
    col_pass<false, true>(c, blocks, m, ml, st, s);
}

}  // namespace pfg
