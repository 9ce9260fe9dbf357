// ntt_small.cuh — latency kernel for the N = 2^12 transform: one thread-block cluster per limb.
//
// Same transform as ntt.cuh (the reference's nwt_2d_radix8_forward_inplace /
// nwt_2d_radix8_backward_inplace, src/ntt/fntt_2d.cu:620-653, src/ntt/intt_2d.cu:724-757): CT
// forward with the bit-reversed powers of the minimal root, GS inverse with n^-1 folded into the
// last stage, Harvey lazy butterflies, canonical outputs.
//
// At batch 1 a limb on one SM is issue-bound (about 27k warp instructions), so the limb is spread
// over a cluster of 8 CTAs on 8 SMs, CTA c holding coefficients [512 c, 512 c + 512) in shared
// memory.  Stages 0..2 pair coefficients 2048, 1024 and 512 apart — across CTAs — and run as one
// radix-8 step over distributed shared memory (CTA c computes the eight-point groups
// {j + 512 m : m < 8} for j in [64 c, 64 c + 64), reading and writing its peers' shared memory),
// between cluster barriers; stages 3..11 stay inside each CTA (radix-4 phases, then one radix-2
// stage).  Each CTA stages the 511 twiddle pairs its local stages use next to its data.
#pragma once
#include <cooperative_groups.h>

#include "ntt.cuh"

namespace pfg {

constexpr int kSmallLogN = 12, kSmallN = 1 << kSmallLogN;
constexpr int kSmallCluster = 8, kSmallChunk = kSmallN / kSmallCluster, kSmallThreads = 128;

// forward CT butterfly on (x, y), twiddle w (Harvey: inputs < 4q, outputs < 4q)
__device__ __forceinline__ void ct_bfly(uint64_t &x, uint64_t &y, const TwPair &w, uint64_t q) {
    const uint64_t a = csub(x, 2 * q), b = mul_shoup_lazy(y, w.w, w.ws, q);
    x = a + b;
    y = a - b + 2 * q;
}
// inverse GS butterfly (inputs < 2q, outputs < 2q); `scale` multiplies the sum by n^-1
__device__ __forceinline__ void gs_bfly(uint64_t &x, uint64_t &y, const TwPair &w, uint64_t q, bool scale,
                                        uint64_t ni, uint64_t nis) {
    const uint64_t a = x, b = y;
    x = scale ? mul_shoup_lazy(a + b, ni, nis, q) : csub(a + b, 2 * q);
    y = mul_shoup_lazy(a - b + 2 * q, w.w, w.ws, q);
}

// cluster rank c = blockIdx.x % 8; limb = blockIdx.x / 8 -> polynomial limb / limbs, limb % limbs
template <bool FWD>
__global__ void __cluster_dims__(kSmallCluster, 1, 1) __launch_bounds__(kSmallThreads)
        ntt_n12(uint64_t *data, long long ps, int limbs, int start, NttTables T) {
    namespace cg = cooperative_groups;
    __shared__ uint64_t sm[kSmallChunk + kSmallChunk / 16];
    __shared__ __align__(16) TwPair ltw[kSmallChunk];  // stages 3..11: [2^(s-3) - 1 + local group]
    cg::cluster_group cluster = cg::this_cluster();
    const int c = (int)cluster.block_rank(), tid = threadIdx.x;
    const int lb = blockIdx.x / kSmallCluster, poly = lb / limbs, k = lb % limbs, tbl = start + k;
    uint64_t *x = data + poly * ps + ((size_t)k << kSmallLogN) + (size_t)c * kSmallChunk;
    const uint64_t q = T.mods[tbl].q;
    const TwPair *gtw = (FWD ? T.tw : T.itw) + ((size_t)tbl << kSmallLogN);
    // the twiddles come from the context's read-only tables: staged before waiting for the
    // previous kernel (launch overlap), the data only after
    for (int i = tid; i < kSmallChunk - 1; i += kSmallThreads) {  // i = 2^(s-3) - 1 + g, s = 3..11
        const int s = 3 + (31 - __clz(i + 1)), g = i + 1 - (1 << (s - 3));
        ltw[i] = ld_tw(gtw, (1u << s) + (uint32_t)(c << (s - 3)) + g);
    }
    pdl_wait();
    pdl_release();
    for (int i = tid; i < kSmallChunk; i += kSmallThreads) sm[pad_idx(i)] = x[i];
    const TwPair t0 = ld_tw(gtw, 1);
    auto local_tw = [&](int s, int e) { return ltw[(1 << (s - 3)) - 1 + (e >> (12 - s))]; };
    // cross-CTA radix-8 over stages 0..2 (CT forward order or GS inverse order)
    auto cross = [&]() {
        if (tid < kSmallChunk / kSmallCluster) {
            const int j = c * (kSmallChunk / kSmallCluster) + tid;
            uint64_t *peer[kSmallCluster];
            uint64_t v[kSmallCluster];
#pragma unroll
            for (int m = 0; m < kSmallCluster; m++) {
                peer[m] = cluster.map_shared_rank(sm, m);
                v[m] = peer[m][pad_idx(j)];
            }
            const TwPair t1a = ld_tw(gtw, 2), t1b = ld_tw(gtw, 3);
            TwPair t2[4];
#pragma unroll
            for (int m = 0; m < 4; m++) t2[m] = ld_tw(gtw, 4 + m);
            if constexpr (FWD) {
#pragma unroll
                for (int m = 0; m < 4; m++) ct_bfly(v[m], v[m + 4], t0, q);  // stage 0: 2048 apart
#pragma unroll
                for (int m = 0; m < 2; m++) {                              // stage 1: 1024 apart
                    ct_bfly(v[m], v[m + 2], t1a, q);
                    ct_bfly(v[m + 4], v[m + 6], t1b, q);
                }
#pragma unroll
                for (int m = 0; m < 4; m++) ct_bfly(v[2 * m], v[2 * m + 1], t2[m], q);  // stage 2: 512 apart
            } else {
                const uint64_t ni = T.ninv[2 * tbl], nis = T.ninv[2 * tbl + 1];
#pragma unroll
                for (int m = 0; m < 4; m++) gs_bfly(v[2 * m], v[2 * m + 1], t2[m], q, false, 0, 0);
#pragma unroll
                for (int m = 0; m < 2; m++) {
                    gs_bfly(v[m], v[m + 2], t1a, q, false, 0, 0);
                    gs_bfly(v[m + 4], v[m + 6], t1b, q, false, 0, 0);
                }
#pragma unroll
                for (int m = 0; m < 4; m++) gs_bfly(v[m], v[m + 4], t0, q, true, ni, nis);  // global stage 0
            }
#pragma unroll
            for (int m = 0; m < kSmallCluster; m++) peer[m][pad_idx(j)] = v[m];
        }
    };
    // local stages s, s + 1 (radix 4) on the chunk: quadruple {e, e + t2, e + t1, e + t1 + t2}
    auto local4 = [&](int s) {
        const int t1 = kSmallN >> (s + 1), t2 = t1 >> 1;
        const int e0 = (tid / t2) * (4 * t2) + (tid % t2), e1 = e0 + t2, e2 = e0 + t1, e3 = e2 + t2;
        uint64_t y0 = sm[pad_idx(e0)], y1 = sm[pad_idx(e1)], y2 = sm[pad_idx(e2)], y3 = sm[pad_idx(e3)];
        const TwPair wA = local_tw(s, e0), wB = local_tw(s + 1, e0), wC = local_tw(s + 1, e2);
        if constexpr (FWD) {
            ct_bfly(y0, y2, wA, q);
            ct_bfly(y1, y3, wA, q);
            ct_bfly(y0, y1, wB, q);
            ct_bfly(y2, y3, wC, q);
        } else {
            gs_bfly(y0, y1, wB, q, false, 0, 0);
            gs_bfly(y2, y3, wC, q, false, 0, 0);
            gs_bfly(y0, y2, wA, q, false, 0, 0);
            gs_bfly(y1, y3, wA, q, false, 0, 0);
        }
        sm[pad_idx(e0)] = y0;
        sm[pad_idx(e1)] = y1;
        sm[pad_idx(e2)] = y2;
        sm[pad_idx(e3)] = y3;
    };
    auto local2 = [&]() {  // stage 11 (pairs 1 apart), two butterflies per thread
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int e = 2 * (tid + h * kSmallThreads);
            uint64_t y0 = sm[pad_idx(e)], y1 = sm[pad_idx(e + 1)];
            const TwPair w = local_tw(11, e);
            if constexpr (FWD)
                ct_bfly(y0, y1, w, q);
            else
                gs_bfly(y0, y1, w, q, false, 0, 0);
            sm[pad_idx(e)] = y0;
            sm[pad_idx(e + 1)] = y1;
        }
    };
    cluster.sync();  // every chunk and twiddle table is in place
    if constexpr (FWD) {
        cross();
        cluster.sync();
        for (int s = 3; s < 11; s += 2) {
            local4(s);
            __syncthreads();
        }
        local2();
        __syncthreads();
        for (int i = tid; i < kSmallChunk; i += kSmallThreads) x[i] = csub(csub(sm[pad_idx(i)], 2 * q), q);
    } else {
        local2();
        __syncthreads();
        for (int s = 9; s >= 3; s -= 2) {
            local4(s);
            __syncthreads();
        }
        cluster.sync();
        cross();
        cluster.sync();
        for (int i = tid; i < kSmallChunk; i += kSmallThreads) x[i] = csub(sm[pad_idx(i)], q);
    }
}

}  // namespace pfg
