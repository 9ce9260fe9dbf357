// keyswitch.cuh — the key-switching inner product (shared by the CKKS and BFV paths).
//
// key_switch_inner_prod_c2_and_evk (src/eval_key_switch.cu:14-69):
//   cx_t[jj] = sum_{d < beta} T_d[jj] * evk_d[t][twr(jj)]  mod p_jj,
//   twr(jj) = jj for jj < l, |Q| + (jj - l) for the special limbs.
// The sum is kept in 128 bits and reduced once (every 7 terms when beta > 7, which keeps it
// below q * 2^64 for q < 2^61).
#pragma once
#include "modarith.cuh"
#include "pdl.cuh"
#include "pdl.cuh"

namespace pfg {

// ------------------------------------------------------------------ inner product

struct PlainOwn {  // the digit's own limbs are c2 itself (NTT form)
    const uint64_t *c2;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int jj, const Mod &, uint32_t idx) const {
        return c2[((size_t)jj << log_n) + idx];
    }
};

struct TensorOwn {  // ... or the tensor product's d2 = a1 * b1, recomputed
    const uint64_t *a1, *b1;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int jj, const Mod &m, uint32_t idx) const {
        const size_t o = ((size_t)jj << log_n) + idx;
        return mul_mod(a1[o], b1[o], m);
    }
};

// cx_t[jj] = sum_d T_d[jj] * evk_d[t][twr(jj)] mod p_jj  (2 coefficients per thread)
template <class Own, bool OWN_IN_TM>
__global__ void __launch_bounds__(256) ks_inner_product(uint64_t *cx, const uint64_t *tm, Own own,
                                                        const uint64_t *const *evk, const Mod *mods, int log_n,
                                                        int l, int nQ, int alpha, int beta, int qp) {
    pdl_wait();
    pdl_release();
    const int qlp = l + alpha;
    const size_t total = (size_t)qlp << log_n;
    const uint32_t nmask = (1u << log_n) - 1;
    for (size_t e = 2 * ((size_t)blockIdx.x * blockDim.x + threadIdx.x); e < total;
         e += 2 * (size_t)gridDim.x * blockDim.x) {
        const int jj = (int)(e >> log_n);
        const uint32_t idx = (uint32_t)e & nmask;
        const int tbl = jj < l ? jj : nQ + (jj - l);
        const Mod m = mods[tbl];
        const int own_d = jj < l ? jj / alpha : -1;
        u128 a0{0, 0}, a1{0, 0}, b0{0, 0}, b1{0, 0};
        int terms = 0;
        for (int d = 0; d < beta; d++) {
            uint64_t x0, x1;
            if (!OWN_IN_TM && d == own_d) {
                x0 = own(jj, m, idx);
                x1 = own(jj, m, idx + 1);
            } else {
                const ulonglong2 v =  // the mod-up output is dead after this read
                        __ldcs(reinterpret_cast<const ulonglong2 *>(tm + (((size_t)d * qlp + jj) << log_n) + idx));
                x0 = v.x;
                x1 = v.y;
            }
            // the key is read once per call: streaming loads (evict first) keep the mod-up output,
            // written just before and read once here, in L2
            const uint64_t *key = evk[d];
            const ulonglong2 k0 = __ldcs(reinterpret_cast<const ulonglong2 *>(key + ((size_t)tbl << log_n) + idx));
            const ulonglong2 k1 =
                    __ldcs(reinterpret_cast<const ulonglong2 *>(key + ((size_t)(qp + tbl) << log_n) + idx));
            if (terms == 7) {  // keep the sum below q * 2^64 (reduce128's precondition)
                a0 = u128{reduce128(a0, m), 0};
                a1 = u128{reduce128(a1, m), 0};
                b0 = u128{reduce128(b0, m), 0};
                b1 = u128{reduce128(b1, m), 0};
                terms = 1;
            }
            mac(a0, x0, k0.x);
            mac(a1, x1, k0.y);
            mac(b0, x0, k1.x);
            mac(b1, x1, k1.y);
            terms++;
        }
        *reinterpret_cast<ulonglong2 *>(cx + e) = make_ulonglong2(reduce128(a0, m), reduce128(a1, m));
        *reinterpret_cast<ulonglong2 *>(cx + total + e) = make_ulonglong2(reduce128(b0, m), reduce128(b1, m));
    }
}

struct NoOwn {  // every digit limb, own ones included, is read from tm (BFV)
    __device__ __forceinline__ uint64_t operator()(int, const Mod &, uint32_t) const { return 0; }
};

}  // namespace pfg
