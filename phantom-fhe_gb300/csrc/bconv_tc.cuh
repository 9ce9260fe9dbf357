// bconv_tc.cuh — mod-up base conversion on the tensor cores (tcgen05), word-for-word equal to
// modup_bconv (bconv.cuh) and to the reference's bconv_matmul_padded_unroll2_kernel
// (src/rns_bconv.cu:455-485) fed by DRNSTool::modup (:530-628).
//
// Per digit d (blockIdx.y) the conversion of its sz input limbs to the l + alpha - sz other QlP
// limbs is the byte-plane GEMM of tc.cuh: A = [128 coefficients][8 alpha bytes] (filled from y,
// one 16-byte core-matrix row per input residue), B = the digit's constant byte planes (built at
// context creation, copied to shared memory once per CTA), D = [128][8 x outputs] f32 in tensor
// memory.  CTAs are persistent over 128-coefficient tiles; 256 threads: all fill A, one issues
// the MMAs, and each of the 8 warps reads its lane quarter of D for half of the outputs and
// writes canonical residues to tm[d][jj][n] (coalesced 8-byte stores).
#pragma once
#include "tc.cuh"

namespace pfg {

// The pipeline shared by the tensor-core conversions: one CTA per SM, 512 threads, two
// accumulators (2 x 256 tensor-memory columns) and two A buffers.  Iteration i writes tile i's A
// (loaded into registers during the previous iteration), issues tile i's MMAs, starts the loads
// of tile i + 1 and runs tile i - 1's epilogue while the MMAs execute: one barrier per tile.
// Only thread 0 waits on the MMA barrier (bounded); the others sleep in __syncthreads.
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

// TMEM columns [col0, col0 + 8) of output positions [o, o1) -> dst[s_off[pos]] (lazy residues);
// extra(pos) is added (rescale: z).
template <int NPL, class Extra>
__device__ __forceinline__ void tc_emit(uint32_t trow, uint64_t *dst, int o, int o1, const uint64_t *s_p,
                                        const uint64_t *s_off, const float *s_inv, Extra extra) {
    for (; o + 1 < o1; o += 2) {
        uint32_t x0[8], x1[8];
        tc::ld8(trow + o * 8, x0);
        tc::ld8(trow + o * 8 + 8, x1);
        tc::wait_ld();
        dst[s_off[o]] = tc::reduce_planes_lazy<NPL>(x0, s_p[o], s_inv[o]) + extra(o);
        dst[s_off[o + 1]] = tc::reduce_planes_lazy<NPL>(x1, s_p[o + 1], s_inv[o + 1]) + extra(o + 1);
    }
    if (o < o1) {
        uint32_t x0[8];
        tc::ld8(trow + o * 8, x0);
        tc::wait_ld();
        dst[s_off[o]] = tc::reduce_planes_lazy<NPL>(x0, s_p[o], s_inv[o]) + extra(o);
    }
}

struct NoExtra {
    __device__ __forceinline__ uint64_t operator()(int) const { return 0; }
};

// Mod-up conversion of digit d = blockIdx.y (lazy outputs, consumed by the forward NTT).
template <int KSTEPS>
__global__ void __launch_bounds__(tc::kPipeThreads, 1)
        modup_bconv_tc(uint64_t *tm, const uint64_t *y, const uint16_t *bmat, const TcOutMeta *meta,
                       const int *nnarrow, const Mod *mods, unsigned *status, int log_n, int l, int nQ, int alpha) {
    constexpr int KP = KSTEPS * 16;
    constexpr uint32_t SBO = KP / 8 * 128;
    constexpr int ABYTES = tc::kRows * KP * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;                   // 2 x 128 x KP bf16
    uint8_t *sB = smem + 2 * ABYTES;      // 256 x KP bf16
    __shared__ uint32_t tmem_slot, ok_flag;
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint64_t s_p[tc::kMaxOut];       // output modulus, by output position
    __shared__ uint64_t s_off[tc::kMaxOut];     // output limb offset in tm
    __shared__ float s_inv[tc::kMaxOut];        // 1 / p as f32
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int d = blockIdx.y, qlp = l + alpha, s0 = d * alpha, sz = min(alpha, l - s0), nout = qlp - sz;
    const int ncols = (nout * 8 + 15) & ~15;

    const uint4 *src = reinterpret_cast<const uint4 *>(bmat + (size_t)d * tc::kTmemCols * KP);
    for (int i = tid; i < ncols * KP * 2 / 16; i += tc::kPipeThreads) reinterpret_cast<uint4 *>(sB)[i] = src[i];
    for (int i = tid; i < 2 * tc::kRows * (KP / 8); i += tc::kPipeThreads) {  // K columns past the digit stay zero
        const int buf = i / (tc::kRows * (KP / 8)), rem = i % (tc::kRows * (KP / 8));
        const int r = rem / (KP / 8), kc = rem % (KP / 8);
        if (kc >= sz)
            *reinterpret_cast<uint4 *>(sA + buf * ABYTES + (r & 7) * 16 + (r >> 3) * SBO + kc * 128) =
                    make_uint4(0, 0, 0, 0);
    }
    if (tid < nout) {
        const TcOutMeta m = meta[d * tc::kMaxOut + tid];
        const int jj = (int)m.jj;
        s_p[tid] = mods[jj < l ? jj : nQ + (jj - l)].q;
        s_off[tid] = ((size_t)d * qlp + jj) << log_n;
        s_inv[tid] = m.invp;
    }
    const int nn = nnarrow[d], nw = nout - nn;
    if (warp == 0) tc::tmem_alloc(&tmem_slot, 2 * tc::kTmemCols);
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(tc::kRows, ncols);
    const int ntiles = 1 << (log_n - 7);
    const int cnt = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int r = tid & (tc::kRows - 1), lq = warp & 3, grp = warp >> 2;
    // positions [0, nn) have 5 byte planes, [nn, nout) have 8; each warp group takes a quarter of each
    const int a0 = grp * nn / 4, a1 = (grp + 1) * nn / 4;
    const int b0 = nn + grp * nw / 4, b1 = nn + (grp + 1) * nw / 4;
    // fill: thread -> (row r, limbs i0 and i0 + 4)
    const int i0 = tid >> 7;
    uint64_t ya = 0, yb = 0;
    auto load = [&](int i) {
        const size_t n0 = (size_t)((int)blockIdx.x + i * (int)gridDim.x) * tc::kRows;
        if (i0 < sz) ya = y[((size_t)(s0 + i0) << log_n) + n0 + r];
        if (i0 + 4 < sz) yb = y[((size_t)(s0 + i0 + 4) << log_n) + n0 + r];
    };
    auto fill = [&](int i) {
        uint8_t *a = sA + (i & 1) * ABYTES + (r & 7) * 16 + (r >> 3) * SBO;
        if (i0 < sz) *reinterpret_cast<uint4 *>(a + i0 * 128) = tc::bytes_bf16(ya);
        if (i0 + 4 < sz) *reinterpret_cast<uint4 *>(a + (i0 + 4) * 128) = tc::bytes_bf16(yb);
    };
    auto issue = [&](int i) {
        const uint32_t base = tc::saddr(sA + (i & 1) * ABYTES), bb = tc::saddr(sB);
        tc::fence_after();
#pragma unroll
        for (int k = 0; k < KSTEPS; k++)
            tc::mma_bf16(tmem + (i & 1) * tc::kTmemCols, tc::sdesc(base + k * 256, 128, SBO),
                         tc::sdesc(bb + k * 256, 128, SBO), idesc, k > 0);
        tc::commit(&bar[i & 1]);
    };
    auto epilogue = [&](int i) {
        const uint32_t trow = tmem + (i & 1) * tc::kTmemCols + ((uint32_t)(lq * 32) << 16);
        uint64_t *dst = tm + (size_t)((int)blockIdx.x + i * (int)gridDim.x) * tc::kRows + lq * 32 + lane;
        tc_emit<5>(trow, dst, a0, a1, s_p, s_off, s_inv, NoExtra{});
        tc_emit<8>(trow, dst, b0, b1, s_p, s_off, s_inv, NoExtra{});
    };
    tc_pipeline(cnt, bar, &ok_flag, status, load, fill, issue, epilogue);
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_free(tmem, 2 * tc::kTmemCols);
    }
}

// P -> Ql conversion of polynomial t = blockIdx.y on the tensor cores.  Input: the nP P limbs
// of cx[t] ([x_k PHatInv_k]_{p_k}, coefficient form).  Output positions (meta) cover j < l.
//   !RESCALE (DRNSTool::moddown_from_NTT, src/rns_bconv.cu:776-828, bConv_BEHZ :212-229):
//     out[t][j] = sum_k y_k (P/p_k) mod q_j (lazy), for the forward NTT of the mod-down.
//   RESCALE (HMult + relinearise + rescale, see ckks_mul_relin_rescale): the constants carry
//     P^-1 mod q_j, position l - 1 holds e = delta_(l-1) P^-1 and
//     z = zd + zc P^-1 - e mod q_(l-1) (canonical; one warp group computes it per row and
//     shares it through shared memory), then out[t][j] = delta_j P^-1 + z (j < l - 1, lazy:
//     below 4 q_j because q_(l-1) <= 2 q_j, checked on the host).
template <int KSTEPS, bool RESCALE>
__global__ void __launch_bounds__(tc::kPipeThreads, 1)
        pq_bconv_tc(uint64_t *out, long long ops, const uint64_t *cx, long long cps, const uint16_t *bmat,
                    const TcOutMeta *meta, int nn, const Mod *mods, unsigned *status, int log_n, int l, int nP,
                    const uint64_t *zc, const uint64_t *zd, const uint64_t *pinv) {
    constexpr int KP = KSTEPS * 16;
    constexpr uint32_t SBO = KP / 8 * 128;
    constexpr int ABYTES = tc::kRows * KP * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;
    uint8_t *sB = smem + 2 * ABYTES;
    __shared__ uint32_t tmem_slot, ok_flag;
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint64_t s_p[tc::kMaxOut], s_off[tc::kMaxOut];
    __shared__ float s_inv[tc::kMaxOut];
    __shared__ uint64_t s_z[tc::kRows];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int t = blockIdx.y, sz = nP, npos = l;
    const int ncols = (npos * 8 + 15) & ~15;
    const uint64_t *in = cx + t * cps + ((size_t)l << log_n);
    uint64_t *dst_t = out + t * ops;

    const uint4 *src = reinterpret_cast<const uint4 *>(bmat);
    for (int i = tid; i < ncols * KP * 2 / 16; i += tc::kPipeThreads) reinterpret_cast<uint4 *>(sB)[i] = src[i];
    for (int i = tid; i < 2 * tc::kRows * (KP / 8); i += tc::kPipeThreads) {
        const int buf = i / (tc::kRows * (KP / 8)), rem = i % (tc::kRows * (KP / 8));
        const int r = rem / (KP / 8), kc = rem % (KP / 8);
        if (kc >= sz)
            *reinterpret_cast<uint4 *>(sA + buf * ABYTES + (r & 7) * 16 + (r >> 3) * SBO + kc * 128) =
                    make_uint4(0, 0, 0, 0);
    }
    if (tid < npos) {
        const TcOutMeta m = meta[tid];
        s_p[tid] = mods[m.jj].q;
        s_off[tid] = (size_t)m.jj << log_n;
        s_inv[tid] = m.invp;
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, 2 * tc::kTmemCols);
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(tc::kRows, ncols);
    const int ntiles = 1 << (log_n - 7);
    const int cnt = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int r = tid & (tc::kRows - 1), lq = warp & 3, grp = warp >> 2;
    const int nlim = RESCALE ? npos - 1 : npos, nw = nlim - nn;
    const int a0 = grp * nn / 4, a1 = (grp + 1) * nn / 4;
    const int b0 = nn + grp * nw / 4, b1 = nn + (grp + 1) * nw / 4;
    const int i0 = tid >> 7;
    uint64_t ya = 0, yb = 0;
    auto load = [&](int i) {
        const size_t n0 = (size_t)((int)blockIdx.x + i * (int)gridDim.x) * tc::kRows;
        if (i0 < sz) ya = in[((size_t)i0 << log_n) + n0 + r];
        if (i0 + 4 < sz) yb = in[((size_t)(i0 + 4) << log_n) + n0 + r];
    };
    auto fill = [&](int i) {
        uint8_t *a = sA + (i & 1) * ABYTES + (r & 7) * 16 + (r >> 3) * SBO;
        if (i0 < sz) *reinterpret_cast<uint4 *>(a + i0 * 128) = tc::bytes_bf16(ya);
        if (i0 + 4 < sz) *reinterpret_cast<uint4 *>(a + (i0 + 4) * 128) = tc::bytes_bf16(yb);
    };
    auto issue = [&](int i) {
        const uint32_t base = tc::saddr(sA + (i & 1) * ABYTES), bb = tc::saddr(sB);
        tc::fence_after();
#pragma unroll
        for (int k = 0; k < KSTEPS; k++)
            tc::mma_bf16(tmem + (i & 1) * tc::kTmemCols, tc::sdesc(base + k * 256, 128, SBO),
                         tc::sdesc(bb + k * 256, 128, SBO), idesc, k > 0);
        tc::commit(&bar[i & 1]);
    };
    auto epilogue = [&](int i) {
        const uint32_t trow = tmem + (i & 1) * tc::kTmemCols + ((uint32_t)(lq * 32) << 16);
        const size_t n = (size_t)((int)blockIdx.x + i * (int)gridDim.x) * tc::kRows + lq * 32 + lane;
        uint64_t *dst = dst_t + n;
        if constexpr (RESCALE) {
            const int row = lq * 32 + lane;
            if (grp == 0) {
                const int pl = npos - 1;
                const uint64_t ql = s_p[pl];
                uint32_t x[8];
                tc::ld8(trow + pl * 8, x);
                tc::wait_ld();
                uint64_t e = ql < (1ull << 40) ? tc::reduce_planes_lazy<5>(x, ql, s_inv[pl])
                                               : tc::reduce_planes_lazy<8>(x, ql, s_inv[pl]);
                e = csub(e, ql);
                const size_t o = ((size_t)t << log_n) + n;
                const uint64_t zcp = mul_shoup(zc[o], pinv[2 * (l - 1)], pinv[2 * (l - 1) + 1], ql);
                s_z[row] = sub_mod(add_mod(zd[o], zcp, ql), e, ql);
            }
            asm volatile("bar.sync %0, 128;" ::"r"(1 + lq) : "memory");  // the four warps of this lane quarter
            const uint64_t z = s_z[row];
            auto addz = [z](int) { return z; };
            tc_emit<5>(trow, dst, a0, a1, s_p, s_off, s_inv, addz);
            tc_emit<8>(trow, dst, b0, b1, s_p, s_off, s_inv, addz);
        } else {
            tc_emit<5>(trow, dst, a0, a1, s_p, s_off, s_inv, NoExtra{});
            tc_emit<8>(trow, dst, b0, b1, s_p, s_off, s_inv, NoExtra{});
        }
    };
    tc_pipeline(cnt, bar, &ok_flag, status, load, fill, issue, epilogue);
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_free(tmem, 2 * tc::kTmemCols);
    }
}

// KSTEPS = kpad / 16 in {1, 2, 3}
template <class F>
void with_tc_ksteps(int kpad, F &&f) {
    switch (kpad / 16) {
        case 1: f.template operator()<1>(); break;
        case 2: f.template operator()<2>(); break;
        default: f.template operator()<3>(); break;
    }
}

}  // namespace pfg
