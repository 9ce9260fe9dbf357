// bconv_tc.cuh — RNS base conversions of the key switch on the tensor cores (tcgen05), word for
// word equal to the CUDA-core kernels of bconv.cuh and to the reference's
//   mod-up    bconv_matmul_padded_unroll2_kernel (src/rns_bconv.cu:455-485, DRNSTool::modup :530-628)
//   mod-down  bConv_BEHZ (:212-229) in DRNSTool::moddown_from_NTT (:776-828)
// through the byte-plane GEMM of tc.cuh.
//
// One kernel serves every form.  A "group" is one conversion with a fixed constant operand: a
// digit of a mod-up, a polynomial of a mod-down, or either of one ciphertext of a batch.  A group
// has sz input limbs (rows = coefficients) and npos output positions; the work is (group,
// 128-row tile) units and each persistent CTA (one per SM, 512 threads) takes a contiguous range
// of them, so it reloads a group's constant operand (double-buffered in shared memory) only at
// group boundaries.  Iteration i of the tile pipeline fills tile i's A (loaded into registers
// during the previous iteration), issues its MMAs into one of two 256-column accumulators, starts
// the loads of tile i + 1 and runs tile i - 1's epilogue while the MMAs execute: one barrier per
// tile.  Outputs are lazy residues in [0, 2p) ([0, 4p) with the rescale term), the input range
// of the forward NTT that consumes every one of them.
#pragma once
#include <algorithm>

#include "launch.cuh"
#include "pdl.cuh"
#include "tc.cuh"

namespace pfg {

// One conversion: inputs in + (i << log_n) (i < sz), outputs out + (jj << log_n) for the
// positions of meta, constant operand bmat ([256][kpad], canonical layout), positions [0, nn)
// with 5 byte planes and [nn, nlim) with 8.  Rescale groups (see pq forms below) carry zc, zd
// (this polynomial's rows) and the level l.
struct TcGroup {
    const uint64_t *in;
    uint64_t *out;
    const uint16_t *bmat;
    const TcOutMeta *meta;
    const uint64_t *zc, *zd;
    int sz, npos, nn, l;
    // BFV mod-up (coefficient form): inputs are c2 itself; they are copied to `own` (the digit's
    // own limbs of the mod-up buffer) and scaled by phi (partQlHatInv pairs, moduli from in_tbl0)
    const uint64_t *phi = nullptr;
    uint64_t *own = nullptr;
    int in_tbl0 = 0;
};

// The tile pipeline; only thread 0 waits on the MMA barrier (bounded), the others sleep in
// __syncthreads.  On a timeout every thread returns after the same barrier.
template <class Load, class Fill, class Issue, class Epi>
__device__ __forceinline__ void tc_pipeline(int cnt, uint64_t *bar, uint32_t *ok_flag, unsigned *status, Load &&load,
                                            Fill &&fill, Issue &&issue, Epi &&epilogue) {
    const int tid = threadIdx.x;
    if (cnt <= 0) return;
    load(0);
    fill(0);
    tc::fence_smem_async();
    __syncthreads();
    if (tid == 0) issue(0);
    if (cnt > 1) load(1);
    for (int i = 1; i <= cnt; i++) {
        if (tid == 0) *ok_flag = tc::mbar_wait(&bar[(i - 1) & 1], ((i - 1) >> 1) & 1) ? 1u : 0u;
        if (i < cnt) fill(i);
        tc::fence_smem_async();
        tc::fence_before();
        __syncthreads();
        if (!*ok_flag) {
            if (tid == 0) atomicOr(status, 1u);
            return;
        }
        if (tid == 0 && i < cnt) issue(i);
        if (i + 1 < cnt) load(i + 1);
        tc::fence_after();
        epilogue(i - 1);
        tc::fence_before();
    }
}

// Per-output record of a tile group: modulus, limb offset in the output (words), 1/p.  One
// 16-byte shared-memory load per output.
struct TcOut {
    uint64_t p;
    uint32_t off;  // jj << log_n (below 2^23)
    float inv;
};

// Output positions [o, o1) of one row: accumulator columns [8 pos, 8 pos + 8) -> dst[off],
// plus extra(pos) (the rescale's z).
template <int NPL, class Extra>
__device__ __forceinline__ void tc_emit(uint32_t trow, uint64_t *dst, int o, int o1, const TcOut *meta,
                                        Extra extra) {
    for (; o + 1 < o1; o += 2) {
        uint32_t x0[8], x1[8];
        tc::ld8(trow + o * 8, x0);
        tc::ld8(trow + o * 8 + 8, x1);
        const TcOut m0 = meta[o], m1 = meta[o + 1];
        tc::wait_ld();
        dst[m0.off] = tc::reduce_planes_lazy<NPL>(x0, m0.p, m0.inv) + extra(o);
        dst[m1.off] = tc::reduce_planes_lazy<NPL>(x1, m1.p, m1.inv) + extra(o + 1);
    }
    if (o < o1) {
        uint32_t x0[8];
        tc::ld8(trow + o * 8, x0);
        const TcOut m0 = meta[o];
        tc::wait_ld();
        dst[m0.off] = tc::reduce_planes_lazy<NPL>(x0, m0.p, m0.inv) + extra(o);
    }
}

struct NoExtra {
    __device__ __forceinline__ uint64_t operator()(int) const { return 0; }
};

// RESCALE (HMult + relinearise + rescale, P -> Ql form): the constants carry P^-1 mod q_j, the
// last position is j = l - 1 with e = delta_(l-1) P^-1, z = zd + zc P^-1 - e mod q_(l-1)
// (canonical; one warp group computes it per row and shares it through shared memory), and the
// other outputs are delta_j P^-1 + z (below 4 q_j because q_(l-1) <= 2 q_j, checked on the host).
template <int KSTEPS, bool RESCALE, class Src>
__global__ void __launch_bounds__(tc::kPipeThreads, 1)
        tc_bconv_kernel(Src src, int ngroups, const Mod *mods, const uint64_t *pinv, unsigned *status, int log_n) {
    pdl_wait();
    pdl_release();
    constexpr int KP = KSTEPS * 16, KC = KP / 8;
    constexpr uint32_t SBO = KC * 128;
    constexpr int ABYTES = tc::kRows * KP * 2, BBYTES = tc::kTmemCols * KP * 2;
    constexpr int NSLOT = 3;  // per-tile metadata: slot i % 3 was last read two barriers before fill(i)
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;               // 2 x 128 x KP bf16
    uint8_t *sB = smem + 2 * ABYTES;  // 2 x 256 x KP bf16
    __shared__ uint32_t tmem_slot, ok_flag;
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ __align__(16) TcOut s_out[NSLOT][tc::kMaxOut];
    // raw storage: TcGroup's default member initialisers would ask for a dynamic initialisation
    // that shared memory does not have; every slot is written (thread 0, in fill) before it is read
    __shared__ __align__(alignof(TcGroup)) unsigned char s_grp_raw[NSLOT * sizeof(TcGroup)];
    TcGroup *const s_grp = reinterpret_cast<TcGroup *>(s_grp_raw);
    __shared__ int s_bslot[NSLOT];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles = 1 << (log_n - 7);
    const long long units = (long long)ngroups * tiles;
    const long long u0 = units * blockIdx.x / gridDim.x, u1 = units * (blockIdx.x + 1) / gridDim.x;
    const int cnt = (int)(u1 - u0);

    if (warp == 0) tc::tmem_alloc(&tmem_slot, 2 * tc::kTmemCols);
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    const int r = tid & (tc::kRows - 1), lq = warp & 3, grp = warp >> 2, i0 = tid >> 7;

    // every thread tracks the same group sequence
    int cur_group = -1, bslot = 1, lg = -1;
    int sg0 = -1, sg1 = -1, sg2 = -1;  // group whose metadata each slot holds (registers)
    TcGroup g{}, lgrp{};
    uint64_t ya = 0, yb = 0;
    const int tshift = log_n - 7;  // tiles per group is a power of two
    auto group_of = [&](int i) { return (int)((u0 + i) >> tshift); };
    auto tile_of = [&](int i) { return (int)((u0 + i) & (tiles - 1)); };
    auto load = [&](int i) {
        const int gi = group_of(i);
        if (gi != lg) {
            lg = gi;
            lgrp = src(gi);
        }
        const size_t n = (size_t)tile_of(i) * tc::kRows + r;
        if (i0 < lgrp.sz) ya = lgrp.in[((size_t)i0 << log_n) + n];
        if (i0 + 4 < lgrp.sz) yb = lgrp.in[((size_t)(i0 + 4) << log_n) + n];
    };
    auto fill = [&](int i) {
        const int gi = group_of(i), sl = i % NSLOT;
        if (gi != cur_group) {  // the group's constant operand goes to the other B slot
            cur_group = gi;
            g = src(gi);
            bslot ^= 1;
            const int ncols = (g.npos * 8 + 15) & ~15;
            const uint4 *bs = reinterpret_cast<const uint4 *>(g.bmat);
            uint4 *bd = reinterpret_cast<uint4 *>(sB + bslot * BBYTES);
            for (int k = tid; k < ncols * KP * 2 / 16; k += tc::kPipeThreads) bd[k] = bs[k];
        }
        const int have = sl == 0 ? sg0 : (sl == 1 ? sg1 : sg2);
        if (have != gi) {  // a slot keeps its metadata while its group does not change
            if (sl == 0) sg0 = gi;
            else if (sl == 1) sg1 = gi;
            else sg2 = gi;
            if (tid < g.npos) {
                const TcOutMeta m = g.meta[tid];
                s_out[sl][tid] = TcOut{mods[m.tbl].q, m.jj << log_n, m.invp};
            }
            if (tid == 0) {
                s_grp[sl] = g;
                s_bslot[sl] = bslot;
            }
        }
        if (g.phi) {
            const size_t n = (size_t)tile_of(i) * tc::kRows + r;
            if (i0 < g.sz) {
                g.own[((size_t)i0 << log_n) + n] = ya;
                ya = mul_shoup(ya, g.phi[2 * i0], g.phi[2 * i0 + 1], mods[g.in_tbl0 + i0].q);
            }
            if (i0 + 4 < g.sz) {
                g.own[((size_t)(i0 + 4) << log_n) + n] = yb;
                yb = mul_shoup(yb, g.phi[2 * (i0 + 4)], g.phi[2 * (i0 + 4) + 1], mods[g.in_tbl0 + i0 + 4].q);
            }
        }
        uint8_t *a = sA + (i & 1) * ABYTES + (r & 7) * 16 + (r >> 3) * SBO;
        if (i0 < KC) *reinterpret_cast<uint4 *>(a + i0 * 128) = i0 < g.sz ? tc::bytes_bf16(ya) : make_uint4(0, 0, 0, 0);
        if (i0 + 4 < KC)
            *reinterpret_cast<uint4 *>(a + (i0 + 4) * 128) =
                    i0 + 4 < g.sz ? tc::bytes_bf16(yb) : make_uint4(0, 0, 0, 0);
    };
    auto issue = [&](int i) {
        const int sl = i % NSLOT;
        const uint32_t idesc = tc::idesc_bf16(tc::kRows, (s_grp[sl].npos * 8 + 15) & ~15);
        const uint32_t base = tc::saddr(sA + (i & 1) * ABYTES), bb = tc::saddr(sB + s_bslot[sl] * BBYTES);
        tc::fence_after();
#pragma unroll
        for (int k = 0; k < KSTEPS; k++)
            tc::mma_bf16(tmem + (i & 1) * tc::kTmemCols, tc::sdesc(base + k * 256, 128, SBO),
                         tc::sdesc(bb + k * 256, 128, SBO), idesc, k > 0);
        tc::commit(&bar[i & 1]);
    };
    auto epilogue = [&](int i) {
        const int sl = i % NSLOT;
        const TcGroup gg = s_grp[sl];
        const uint32_t trow = tmem + (i & 1) * tc::kTmemCols + ((uint32_t)(lq * 32) << 16);
        const int row = lq * 32 + lane;
        const size_t n = (size_t)tile_of(i) * tc::kRows + row;
        uint64_t *dst = gg.out + n;
        const int nlim = RESCALE ? gg.npos - 1 : gg.npos, nw = nlim - gg.nn;
        const int a0 = grp * gg.nn / 4, a1 = (grp + 1) * gg.nn / 4;
        const int b0 = gg.nn + grp * nw / 4, b1 = gg.nn + (grp + 1) * nw / 4;
        if constexpr (RESCALE) {
            // every warp group computes its rows' z itself (the same words four times over) rather
            // than waiting at a barrier for one group to share it
            const int pl = gg.npos - 1;
            const TcOut ml = s_out[sl][pl];
            const uint64_t ql = ml.p;
            const uint64_t zcp = mul_shoup(gg.zc[n], pinv[2 * (gg.l - 1)], pinv[2 * (gg.l - 1) + 1], ql);
            const uint64_t zd = gg.zd[n];
            uint32_t x[8];
            tc::ld8(trow + pl * 8, x);
            tc::wait_ld();
            uint64_t e = ql < (1ull << 40) ? tc::reduce_planes_lazy<5>(x, ql, ml.inv)
                                           : tc::reduce_planes_lazy<8>(x, ql, ml.inv);
            e = csub(e, ql);
            const uint64_t z = sub_mod(add_mod(zd, zcp, ql), e, ql);
            auto addz = [z](int) { return z; };
            tc_emit<5>(trow, dst, a0, a1, s_out[sl], addz);
            tc_emit<8>(trow, dst, b0, b1, s_out[sl], addz);
        } else {
            tc_emit<5>(trow, dst, a0, a1, s_out[sl], NoExtra{});
            tc_emit<8>(trow, dst, b0, b1, s_out[sl], NoExtra{});
        }
    };
    tc_pipeline(cnt, bar, &ok_flag, status, load, fill, issue, epilogue);
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_free(tmem, 2 * tc::kTmemCols);
    }
}

// Mod-up of one ciphertext: group = digit d.  y [l][N] -> tm [beta][l + alpha][N].
struct ModupSrc {
    const uint64_t *y;
    uint64_t *tm;
    const uint16_t *bmat;
    const TcOutMeta *meta;
    const int *nn;
    int l, alpha, log_n, kpad;
    __device__ __forceinline__ TcGroup operator()(int d) const {
        const int s0 = d * alpha, sz = min(alpha, l - s0), qlp = l + alpha;
        return TcGroup{y + ((size_t)s0 << log_n), tm + (((size_t)d * qlp) << log_n), bmat + (size_t)d * 256 * kpad,
                       meta + d * tc::kMaxOut, nullptr, nullptr, sz, qlp - sz, nn[d], l};
    }
};

// BFV mod-up of c2 (coefficient form): group = digit d; own limbs copied, inputs scaled in the fill.
struct BfvModupSrc {
    const uint64_t *c2;
    uint64_t *tm;
    const uint16_t *bmat;
    const TcOutMeta *meta;
    const int *nn;
    const uint64_t *phi;  // partQlHatInv pairs per limb
    int l, alpha, log_n, kpad;
    __device__ __forceinline__ TcGroup operator()(int d) const {
        const int s0 = d * alpha, sz = min(alpha, l - s0), qlp = l + alpha;
        TcGroup g{c2 + ((size_t)s0 << log_n), tm + (((size_t)d * qlp) << log_n), bmat + (size_t)d * 256 * kpad,
                  meta + d * tc::kMaxOut, nullptr, nullptr, sz, qlp - sz, nn[d], l};
        g.phi = phi + 2 * s0;
        g.own = tm + (((size_t)d * qlp + s0) << log_n);
        g.in_tbl0 = s0;
        return g;
    }
};

// P -> Ql of one ciphertext: group = polynomial t.  Inputs: the P limbs of cx[t]; outputs out[t].
struct PqSrc {
    const uint64_t *cx;
    long long cps;
    uint64_t *out;
    long long ops;
    const uint16_t *bmat;
    const TcOutMeta *meta;
    const uint64_t *zc, *zd;  // rescale: [2][N] each
    int nn, l, nP, log_n;
    __device__ __forceinline__ TcGroup operator()(int t) const {
        return TcGroup{cx + t * cps + ((size_t)l << log_n), out + t * ops, bmat, meta,
                       zc ? zc + ((size_t)t << log_n) : nullptr, zd ? zd + ((size_t)t << log_n) : nullptr, nP, l, nn,
                       l};
    }
};

// KSTEPS = kpad / 16 in {1, 2, 3}
template <class F>
void with_tc_ksteps(int kpad, F &&f) {
    switch (kpad / 16) {
        case 1: f.template operator()<1>(); break;
        case 2: f.template operator()<2>(); break;
        default: f.template operator()<3>(); break;
    }
}

// Launch over ngroups groups: one persistent CTA per SM (it owns all 512 tensor-memory columns).
template <bool RESCALE, class Src>
void tc_bconv_launch(int kpad, int num_sms, int log_n, const Src &src, int ngroups, const Mod *mods,
                     const uint64_t *pinv, unsigned *status, cudaStream_t s, bool pdl = false) {
    const long long units = (long long)ngroups << (log_n - 7);
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>(num_sms, units));
    with_tc_ksteps(kpad, [&]<int KS>() {
        static bool attr = [] {
            cudaFuncSetAttribute(tc_bconv_kernel<KS, RESCALE, Src>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc::kPipeSmemBytes);
            return true;
        }();
        (void)attr;
        count_launch();
        launch_pdl(pdl, tc_bconv_kernel<KS, RESCALE, Src>, dim3(grid), dim3(tc::kPipeThreads), tc::kPipeSmemBytes, s,
                   src, ngroups, mods, pinv, status, log_n);
    });
}

}  // namespace pfg
