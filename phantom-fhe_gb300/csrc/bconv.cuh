// bconv.cuh — fast RNS base conversion kernels (one input load, many outputs).
//
// The conversions of the key switch are small dense contractions per coefficient:
//   mod-up:   digit d (alpha limbs) -> every other QlP limb    (bconv_matmul_padded_unroll2_kernel,
//             src/rns_bconv.cu:455-485, fed by DRNSTool::modup, :530-628)
//   mod-down: P (alpha limbs) -> every Ql limb                  (DBaseConverter::bConv_BEHZ,
//             src/rns_bconv.cu:212-229, fed by moddown_from_NTT, :776-828)
// Each thread owns two adjacent coefficients, loads the digit's residues once (16-byte loads)
// and produces all output limbs with 128-bit accumulation and one Barrett reduction per output;
// the conversion matrix rows are warp-uniform loads.  Outputs are in coefficient form.
#pragma once
#include "pdl.cuh"
#include "modarith.cuh"

namespace pfg {

// A = compile-time bound on the digit size (alpha); the arrays below then live in registers.
// The dispatcher instantiates A in {1, 2, 3, 4, 5, 6, 8, 16}.

__device__ __forceinline__ ulonglong2 ld2(const uint64_t *p) { return *reinterpret_cast<const ulonglong2 *>(p); }
__device__ __forceinline__ void st2(uint64_t *p, uint64_t a, uint64_t b) {
    *reinterpret_cast<ulonglong2 *>(p) = make_ulonglong2(a, b);
}

// Mod-up base conversion of digit d = blockIdx.y.  CKKS: y holds [c2_i * partQlHatInv_i]_{q_i}
// in coefficient form (made by the inverse NTT's store).  BFV (SCALE): y is c2 itself in
// coefficient form and the scaling happens here, and the digit's own limbs are copied too.
// out tm[d][jj][i] for jj in QlP minus the digit (plus the own limbs when SCALE).
template <int A, bool SCALE>
__global__ void __launch_bounds__(256) modup_bconv(uint64_t *tm, const uint64_t *y, const uint64_t *phi,
                                                   const uint64_t *mat, const Mod *mods, int log_n, int l,
                                                   int nQ, int alpha) {
    pdl_wait();
    pdl_release();
    const int d = blockIdx.y, qlp = l + alpha;
    const int s0 = d * alpha, sz = min(alpha, l - s0);
    const size_t half = (size_t)1 << (log_n - 1);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = 2 * e;
        uint64_t y0[A], y1[A];
        uint64_t *td = tm + (((size_t)d * qlp) << log_n) + idx;
#pragma unroll
        for (int i = 0; i < A; i++) {
            if (i >= sz) break;
            const ulonglong2 v = ld2(y + ((size_t)(s0 + i) << log_n) + idx);
            if (SCALE) {
                const uint64_t q = mods[s0 + i].q, w = phi[2 * (s0 + i)], ws = phi[2 * (s0 + i) + 1];
                st2(td + ((size_t)(s0 + i) << log_n), v.x, v.y);  // own limb: c2 itself
                y0[i] = mul_shoup(v.x, w, ws, q);
                y1[i] = mul_shoup(v.y, w, ws, q);
            } else {
                y0[i] = v.x;
                y1[i] = v.y;
            }
        }
        for (int jj = 0; jj < qlp; jj++) {
            if (jj >= s0 && jj < s0 + sz) continue;
            const Mod m = mods[jj < l ? jj : nQ + (jj - l)];
            const uint64_t *row = mat + ((size_t)d * qlp + jj) * alpha;
            u128 a0{0, 0}, a1{0, 0};
#pragma unroll
            for (int i = 0; i < A; i++) {
                if (i >= sz) break;
                if (i == 8) {
                    a0 = u128{reduce128(a0, m), 0};
                    a1 = u128{reduce128(a1, m), 0};
                }
                const uint64_t w = __ldg(row + i);
                mac(a0, y0[i], w);
                mac(a1, y1[i], w);
            }
            st2(td + ((size_t)jj << log_n), reduce128(a0, m), reduce128(a1, m));
        }
    }
}

// Mod-down base conversion P -> Ql for polynomial t = blockIdx.y: cx's P limbs hold
// [x_k * PHatInv_k]_{p_k} (coefficient form); delta[t][j] = sum_k yp_k * (P/p_k) mod q_j.
template <int A>
__global__ void __launch_bounds__(256) moddown_bconv(uint64_t *delta, long long dps, const uint64_t *cx,
                                                     long long cps, const uint64_t *pmat, const Mod *mods, int log_n,
                                                     int l, int nP) {
    pdl_wait();
    pdl_release();
    const int t = blockIdx.y;
    const size_t half = (size_t)1 << (log_n - 1);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = 2 * e;
        uint64_t y0[A], y1[A];
        const uint64_t *yp = cx + t * cps + ((size_t)l << log_n) + idx;
#pragma unroll
        for (int k = 0; k < A; k++) {
            if (k >= nP) break;
            const ulonglong2 v = ld2(yp + ((size_t)k << log_n));
            y0[k] = v.x;
            y1[k] = v.y;
        }
        uint64_t *dd = delta + t * dps + idx;
        for (int j = 0; j < l; j++) {
            const Mod m = mods[j];
            const uint64_t *row = pmat + (size_t)j * nP;
            u128 a0{0, 0}, a1{0, 0};
#pragma unroll
            for (int k = 0; k < A; k++) {
                if (k >= nP) break;
                if (k == 8) {
                    a0 = u128{reduce128(a0, m), 0};
                    a1 = u128{reduce128(a1, m), 0};
                }
                const uint64_t w = __ldg(row + k);
                mac(a0, y0[k], w);
                mac(a1, y1[k], w);
            }
            st2(dd + ((size_t)j << log_n), reduce128(a0, m), reduce128(a1, m));
        }
    }
}

// HMult + rescale: w[t][j] = delta_j * P^-1 + (z mod q_j) for j < l - 1, with
// z = zd + (zc - delta_{l-1}) * P^-1 mod q_{l-1} (the coefficient form of the relinearised
// product's last limb; see ckks_mul_relin_rescale).
template <int A>
__global__ void __launch_bounds__(256) rescale_fused_bconv(uint64_t *w, long long wps, const uint64_t *cx,
                                                           long long cps, const uint64_t *zc, const uint64_t *zd,
                                                           const uint64_t *pmat, const uint64_t *pinv,
                                                           const Mod *mods, int log_n, int l, int nP) {
    pdl_wait();
    pdl_release();
    const int t = blockIdx.y;
    const size_t half = (size_t)1 << (log_n - 1);
    const Mod ml = mods[l - 1];
    const uint64_t pli = pinv[2 * (l - 1)], plis = pinv[2 * (l - 1) + 1];
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = 2 * e;
        uint64_t y0[A], y1[A];
        const uint64_t *yp = cx + t * cps + ((size_t)l << log_n) + idx;
#pragma unroll
        for (int k = 0; k < A; k++) {
            if (k >= nP) break;
            const ulonglong2 v = ld2(yp + ((size_t)k << log_n));
            y0[k] = v.x;
            y1[k] = v.y;
        }
        const uint64_t *pl = pmat + (size_t)(l - 1) * nP;
        u128 a0{0, 0}, a1{0, 0};
#pragma unroll
        for (int k = 0; k < A; k++) {
            if (k >= nP) break;
            if (k == 8) {
                a0 = u128{reduce128(a0, ml), 0};
                a1 = u128{reduce128(a1, ml), 0};
            }
            const uint64_t c = __ldg(pl + k);
            mac(a0, y0[k], c);
            mac(a1, y1[k], c);
        }
        const size_t o = ((size_t)t << log_n) + idx;
        const ulonglong2 vc = ld2(zc + o), vd = ld2(zd + o);
        const uint64_t z0 = add_mod(vd.x, mul_shoup(sub_mod(vc.x, reduce128(a0, ml), ml.q), pli, plis, ml.q), ml.q);
        const uint64_t z1 = add_mod(vd.y, mul_shoup(sub_mod(vc.y, reduce128(a1, ml), ml.q), pli, plis, ml.q), ml.q);
        uint64_t *wd = w + t * wps + idx;
        for (int j = 0; j < l - 1; j++) {
            const Mod m = mods[j];
            const uint64_t *row = pmat + (size_t)j * nP;
            u128 b0{0, 0}, b1{0, 0};
#pragma unroll
            for (int k = 0; k < A; k++) {
                if (k >= nP) break;
                if (k == 8) {
                    b0 = u128{reduce128(b0, m), 0};
                    b1 = u128{reduce128(b1, m), 0};
                }
                const uint64_t c = __ldg(row + k);
                mac(b0, y0[k], c);
                mac(b1, y1[k], c);
            }
            const uint64_t pj = pinv[2 * j], pjs = pinv[2 * j + 1];
            const uint64_t r0 = add_mod(mul_shoup(reduce128(b0, m), pj, pjs, m.q), reduce64(z0, m), m.q);
            const uint64_t r1 = add_mod(mul_shoup(reduce128(b1, m), pj, pjs, m.q), reduce64(z1, m), m.q);
            st2(wd + ((size_t)j << log_n), r0, r1);
        }
    }
}

// Instantiates body.template operator()<A>() for the smallest supported A >= alpha.
template <class F>
void with_digit_bound(int alpha, F &&f) {
    if (alpha <= 1) f.template operator()<1>();
    else if (alpha <= 2) f.template operator()<2>();
    else if (alpha <= 3) f.template operator()<3>();
    else if (alpha <= 4) f.template operator()<4>();
    else if (alpha <= 5) f.template operator()<5>();
    else if (alpha <= 6) f.template operator()<6>();
    else if (alpha <= 8) f.template operator()<8>();
    else f.template operator()<16>();
}

}  // namespace pfg
