// ops_ckks.cu — NTT entry points and the CKKS hybrid key-switching pipeline.
//
// Restates, with fused kernels, the reference's
//   modup                 DRNSTool::modup                  src/rns_bconv.cu:530-628
//   inner product         key_switch_inner_prod_c2_and_evk src/eval_key_switch.cu:14-69
//   moddown               DRNSTool::moddown_from_NTT       src/rns_bconv.cu:776-828
//   keyswitch_inplace                                      src/eval_key_switch.cu:95-182
//   tensor product        tensor_prod_2x2_rns_poly         src/polymath.cu:463-497
//   rescale               divide_and_round_q_last_ntt      src/rns.cu:1160-1184
//   Galois                apply_galois_inplace / hoisting  src/evaluate.cu:1567-1865
//
// Pipeline of one key switch at level l (alpha = |P|, beta = ceil(l / alpha)):
//   1. iNTT(c2) with the partQlHatInv scaling fused into the store          -> y   [l][N]
//   2. forward NTT of every digit's complement limbs, the base conversion
//      y -> complement limb computed in the column pass's load              -> tm  [beta][l+alpha][N]
//      (the digit's own limbs are c2 itself and are never copied)
//   3. inner product over digits, 128-bit accumulation, one reduction       -> cx  [2][l+alpha][N]
//   4. iNTT of cx's P limbs with the PHatInv scaling fused into the store     (in place)
//   5. forward NTT of delta_j = sum_k y_k (P/p_k) mod q_j, computed in the column pass's load,
//      with (cx_j - NTT(delta_j)) * P^-1 + base fused into the row pass's store.
// For HMult the tensor product is never written: step 1 loads a1*b1, step 3 recomputes it for
// the own limbs, and step 5's "base" is a0*b0 / a0*b1 + a1*b0.  HMult + rescale additionally
// folds the rescale's NTT into step 5 by linearity (see ckks_mul_relin_rescale).
#include <stdexcept>

#include "bconv.cuh"
#include "bconv_tc.cuh"
#include "keyswitch.cuh"
#include "ks_fused.cuh"
#include "launch.cuh"
#include "ntt_small.cuh"
#include "ops.hpp"

namespace pfg {

size_t workspace_words(const Context &c) {
    const size_t n = c.n, nQ = c.nQ, a = c.nP;
    size_t w = 0;
    if (a) {
        const size_t beta = c.beta((int)nQ), qlp = nQ + a;
        // y | tm | cx | g0,g1 (or acc0) | z (4 limbs) | h [2][nQ] (hoisted rotations' mod-down)
        w = n * (nQ + beta * qlp + 2 * qlp + 2 * nQ + 4 + 2 * nQ);
    }
    if (c.scheme == kSchemeBFV) {
        const size_t qr = nQ + c.nR;
        // ext(a), ext(b) [2][QR], t3 [3][QR], o3 [3][Q], r tmp [R], plus key switch scratch
        const size_t bfv = n * (4 * qr + 3 * qr + 3 * nQ + c.nR) + w;
        w = std::max(w, bfv);
    }
    // rescale / generic temporaries
    w = std::max(w, n * (2 * nQ + 2));
    return w;
}

// ------------------------------------------------------------------ NTT entry points

// N = 2^12 (batch-1 latency): one cluster of 8 CTAs per limb (ntt_small.cuh).
template <bool FWD>
static void ntt_n12_launch(const Context &c, uint64_t *data, int polys, int limbs, int start, cudaStream_t s) {
    count_launch();
    launch_pdl(c.pdl, ntt_n12<FWD>, dim3((unsigned)(polys * limbs * kSmallCluster)), dim3(kSmallThreads), 0, s, data,
               (long long)limbs << c.log_n, limbs, start, c.ntt());
}

void ntt_forward(const Context &c, uint64_t *data, int polys, int limbs, int start, cudaStream_t s) {
    if (c.log_n == 12) return ntt_n12_launch<true>(c, data, polys, limbs, start, s);
    const long long ps = (long long)limbs << c.log_n;
    PtrStore st{data, ps, c.log_n};
    ntt_fwd(c, polys * limbs, LimbMajorMap{polys, start}, PtrLoad{data, ps, c.log_n}, st, st, s);
}

void ntt_inverse(const Context &c, uint64_t *data, int polys, int limbs, int start, cudaStream_t s) {
    if (c.log_n == 12) return ntt_n12_launch<false>(c, data, polys, limbs, start, s);
    const long long ps = (long long)limbs << c.log_n;
    PtrStore st{data, ps, c.log_n};
    ntt_inv(c, polys * limbs, LimbMajorMap{polys, start}, PtrLoad{data, ps, c.log_n}, st, st, s);
}

// ------------------------------------------------------------------ functors

// a1 * b1 mod q: the tensor product's d2 term (c2 of the relinearisation)
struct TensorD2Load {
    const uint64_t *a1, *b1;
    const Mod *mods;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int, int k, int tbl, uint32_t idx) const {
        const size_t o = ((size_t)k << log_n) + idx;
        return mul_mod(a1[o], b1[o], mods[tbl]);
    }
};

// Bases added to the mod-down result.
struct InplaceBase {  // the ciphertext itself (keyswitch_inplace's add_to_ct_kernel)
    const uint64_t *ct;
    long long ps;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int t, int j, const Mod &, uint32_t idx) const {
        return ct[t * ps + ((long long)j << log_n) + idx];
    }
};

struct TensorBase {  // t = 0: a0*b0, t = 1: a0*b1 + a1*b0
    const uint64_t *a, *b;
    long long ps;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int t, int j, const Mod &m, uint32_t idx) const {
        const size_t o = ((size_t)j << log_n) + idx;
        const uint64_t a0 = a[o], b0 = b[o];
        if (t == 0) return mul_mod(a0, b0, m);
        u128 acc = mul_wide(a0, b[ps + o]);
        mac(acc, a[ps + o], b0);
        return reduce128(acc, m);
    }
};

struct FirstPolyBase {  // t = 0: g0, t = 1: 0 (Galois: c1 is wiped before the key switch)
    const uint64_t *g0;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int t, int j, const Mod &, uint32_t idx) const {
        return t == 0 ? g0[((size_t)j << log_n) + idx] : 0;
    }
};

static int grid_for(size_t work, int per_block) {
    size_t b = (work + per_block - 1) / per_block;
    return (int)std::min<size_t>(b, kGridStrideBlocks);
}

// ------------------------------------------------------------------ pipeline pieces

struct KsBuffers {
    uint64_t *y, *tm, *cx, *g, *z, *h;
};

static KsBuffers ks_buffers(const Context &c, const Workspace &w) {
    const size_t n = c.n, nQ = c.nQ, qlp = nQ + c.nP, beta = c.beta(c.nQ);
    KsBuffers b;
    b.y = w.base;
    b.tm = b.y + nQ * n;
    b.cx = b.tm + beta * qlp * n;
    b.g = b.cx + 2 * qlp * n;
    b.z = b.g + 2 * nQ * n;
    b.h = b.z + 4 * n;
    return b;
}

// Steps 1-2: y = iNTT(c2) * partQlHatInv; tm = NTT(bconv(y)) for every digit.
static unsigned bconv_blocks(const Context &c) { return (unsigned)std::max<uint64_t>(1, c.n / 2 / 256); }

// tensor-core P -> Ql conversion of both polynomials (rescale: fused with the rescale's z)
template <bool RESCALE>
static void pq_bconv_tc_launch(const Context &c, const LevelTables &lt, uint64_t *out, long long ops,
                               const uint64_t *cx, long long cps, int l, const uint64_t *zc, const uint64_t *zd,
                               cudaStream_t s) {
    const PqSrc src{cx, cps, out, ops,
                    (RESCALE ? lt.tc_rescale : lt.tc_moddown).as<uint16_t>(),
                    (RESCALE ? lt.tc_rescale_meta : lt.tc_moddown_meta).as<TcOutMeta>(), zc, zd,
                    RESCALE ? lt.tc_rescale_nn : lt.tc_moddown_nn, l, c.nP, c.log_n};
    tc_bconv_launch<RESCALE>(c.tc_kpad, c.num_sms, c.log_n, src, 2, c.d_mods.as<Mod>(), c.p_inv.as<uint64_t>(),
                             c.d_status.as<unsigned>(), s, c.pdl);
}

// tensor-core mod-up conversion of every digit
void modup_bconv_tc_launch(const Context &c, const LevelTables &lt, uint64_t *tm, const uint64_t *y, int l,
                           cudaStream_t s) {
    const ModupSrc src{y, tm, lt.tc_modup.as<uint16_t>(), lt.tc_modup_meta.as<TcOutMeta>(), lt.tc_modup_nn.as<int>(),
                       l, c.nP, c.log_n, c.tc_kpad};
    tc_bconv_launch<false>(c.tc_kpad, c.num_sms, c.log_n, src, lt.beta, c.d_mods.as<Mod>(), c.p_inv.as<uint64_t>(),
                           c.d_status.as<unsigned>(), s, c.pdl);
}

// y = iNTT(c2) * partQlHatInv; tm = bconv(y) for every digit's complement limbs, then the
// forward NTT's column pass over them (lazy output in tm).
template <class C2Load>
static void modup_to_column_pass(const Context &c, const KsBuffers &b, C2Load c2ld, int l, cudaStream_t s) {
    const LevelTables &lt = *c.levels[l];
    const int alpha = c.nP, qlp = l + alpha, beta = lt.beta;
    const long long yps = (long long)l << c.log_n;
    PtrStore ys{b.y, yps, c.log_n};
    ntt_inv(c, l, SeqMap{l, 0}, c2ld, ys,
            ScaleStore{b.y, yps, c.log_n, 0, lt.part_hat_inv.as<uint64_t>(), c.d_mods.as<Mod>()}, s);
    const long long tps = (long long)qlp << c.log_n;
    if (c.tc_on && lt.tc_ok) {
        modup_bconv_tc_launch(c, lt, b.tm, b.y, l, s);
    } else {
        dim3 g(bconv_blocks(c), beta);
        with_digit_bound(alpha, [&]<int A>() {
            count_launch();
            launch_pdl(c.pdl, modup_bconv<A, false>, dim3(g), dim3(256), 0, s, b.tm, b.y, nullptr, lt.modup_mat.as<uint64_t>(), c.d_mods.as<Mod>(), c.log_n, l, c.nQ, alpha);
        });
    }
    PtrStore ts{b.tm, tps, c.log_n};
    col_pass<true, false>(c, beta * qlp, ModupMap{qlp, l, c.nQ, alpha, true}, PtrLoad{b.tm, tps, c.log_n}, ts, s);
}

// Steps 1-2: the whole mod-up, T_d in NTT form in tm (hoisted rotations reuse it).
template <class C2Load>
static void modup_ckks(const Context &c, const KsBuffers &b, C2Load c2ld, int l, cudaStream_t s) {
    const int alpha = c.nP, qlp = l + alpha, beta = c.levels[l]->beta;
    const long long tps = (long long)qlp << c.log_n;
    modup_to_column_pass(c, b, c2ld, l, s);
    PtrStore ts{b.tm, tps, c.log_n};
    row_pass<true, true>(c, beta * qlp, ModupMap{qlp, l, c.nQ, alpha, true}, PtrLoad{b.tm, tps, c.log_n}, ts, s);
}

// Steps 2 (row pass) and 3 fused: one kernel per (output limb, row tile) over every digit.
template <class Own>
static void modup_row_inner_product(const Context &c, const KsBuffers &b, Own own, int l, const uint64_t *const *evk,
                                    cudaStream_t s) {
    const int alpha = c.nP, qlp = l + alpha;
    using S = FusedShape<kFusedSingleE>;
    const dim3 grid((unsigned)(c.n / S::kTile), (unsigned)qlp), block(S::kThreads);
    const NttTables T = c.ntt();
    const uint64_t *tm = b.tm;
    count_launch();
    switch (c.l2()) {
        case 6: launch_pdl(c.pdl, ks_modup_ip<6, Own>, grid, block, 0, s, T, tm, own, evk, b.cx, l, c.nQ, alpha, c.beta(l), c.nQ + c.nP); break;
        case 7: launch_pdl(c.pdl, ks_modup_ip<7, Own>, grid, block, 0, s, T, tm, own, evk, b.cx, l, c.nQ, alpha, c.beta(l), c.nQ + c.nP); break;
        case 8: launch_pdl(c.pdl, ks_modup_ip<8, Own>, grid, block, 0, s, T, tm, own, evk, b.cx, l, c.nQ, alpha, c.beta(l), c.nQ + c.nP); break;
        case 9: launch_pdl(c.pdl, ks_modup_ip<9, Own>, grid, block, 0, s, T, tm, own, evk, b.cx, l, c.nQ, alpha, c.beta(l), c.nQ + c.nP); break;
        default: throw std::logic_error("unsupported NTT split");
    }
}

// Step 3
template <class Own>
static void inner_product(const Context &c, const KsBuffers &b, Own own, int l, const uint64_t *const *evk,
                          cudaStream_t s) {
    const int qlp = l + c.nP;
    const size_t work = ((size_t)qlp << c.log_n) / 2;
    count_launch();
    launch_pdl(c.pdl, ks_inner_product<Own, false>, dim3(grid_for(work, 256)), dim3(256), 0, s, b.cx,
               (const uint64_t *)b.tm, own, evk, c.d_mods.as<Mod>(), c.log_n, l, c.nQ, c.nP, c.beta(l), c.nQ + c.nP);
}

// Steps 1-3: cx = <ModUp(c2), evk> (fused or as separate kernels; the same words).
template <class C2Load, class Own>
static void modup_inner_product(const Context &c, const KsBuffers &b, C2Load c2ld, Own own, int l,
                                const uint64_t *const *evk, cudaStream_t s) {
    if (c.ks_fused) {
        modup_to_column_pass(c, b, c2ld, l, s);
        modup_row_inner_product(c, b, own, l, evk, s);
    } else {
        modup_ckks(c, b, c2ld, l, s);
        inner_product(c, b, own, l, evk, s);
    }
}

// Step 4: P limbs of both cx polynomials back to coefficients, times PHatInv.
static void moddown_intt_p(const Context &c, const KsBuffers &b, int l, cudaStream_t s) {
    const int qlp = l + c.nP;
    const long long cps = (long long)qlp << c.log_n;
    PtrStore cs{b.cx, cps, c.log_n};
    ntt_inv(c, 2 * c.nP, QlpMap{c.nP, l, l, c.nQ}, PtrLoad{b.cx, cps, c.log_n}, cs,
            ScaleStore{b.cx, cps, c.log_n, l, c.p_hat_inv.as<uint64_t>(), c.d_mods.as<Mod>()}, s);
}

// out_t[j] = base_t[j] + (cx_t[j] - v_t[j]) P^-1 for both polynomials and j < l, two coefficients
// per thread (coalesced).  Each element is read and written by one thread, so out may alias the
// base (in-place key switch; HMult's poly 1 output over a1, read only by the same element).
template <class Base>
__global__ void __launch_bounds__(256) moddown_combine(uint64_t *out0, uint64_t *out1, const uint64_t *v,
                                                       long long vps, const uint64_t *cx, long long cps,
                                                       const uint64_t *pinv, const Mod *mods, int log_n, int l,
                                                       Base base) {
    pdl_wait();
    pdl_release();
    const size_t half = (size_t)1 << (log_n - 1), per_poly = (size_t)l * half;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < 2 * per_poly;
         e += (size_t)gridDim.x * blockDim.x) {
        const int t = e >= per_poly;
        const size_t r = e - t * per_poly;
        const int j = (int)(r >> (log_n - 1));
        const uint32_t idx = (uint32_t)(2 * (r & (half - 1)));
        const size_t o = ((size_t)j << log_n) + idx;
        const Mod m = mods[j];
        const uint64_t pj = pinv[2 * j], pjs = pinv[2 * j + 1];
        const ulonglong2 vv = __ldcs(reinterpret_cast<const ulonglong2 *>(v + t * vps + o));  // read once
        const ulonglong2 cc = __ldcs(reinterpret_cast<const ulonglong2 *>(cx + t * cps + o));
        const uint64_t y0 = add_mod(base(t, j, m, idx), mul_shoup(sub_mod(cc.x, vv.x, m.q), pj, pjs, m.q), m.q);
        const uint64_t y1 = add_mod(base(t, j, m, idx + 1), mul_shoup(sub_mod(cc.y, vv.y, m.q), pj, pjs, m.q), m.q);
        *reinterpret_cast<ulonglong2 *>((t == 0 ? out0 : out1) + o) = make_ulonglong2(y0, y1);
    }
}

// Step 5 over all l limbs of both polynomials, intermediate in `mid` ([2][l][N]): the forward NTT
// of delta (stored plainly), then the combine as one element-wise pass.
template <class Base>
static void moddown_ntt(const Context &c, const KsBuffers &b, uint64_t *mid, int l, uint64_t *out0, uint64_t *out1,
                        Base base, cudaStream_t s) {
    const int qlp = l + c.nP;
    const long long cps = (long long)qlp << c.log_n;
    const long long mps = (long long)l << c.log_n;
    const LevelTables &lt = *c.levels[l];
    if (c.tc_on && lt.tc_moddown_ok) {
        pq_bconv_tc_launch<false>(c, lt, mid, mps, b.cx, cps, l, nullptr, nullptr, s);
    } else {
        with_digit_bound(c.nP, [&]<int A>() {
            count_launch();
            launch_pdl(c.pdl, moddown_bconv<A>, dim3(dim3(bconv_blocks(c), 2)), dim3(256), 0, s, mid, mps, b.cx, cps, c.p_mat.as<uint64_t>(), c.d_mods.as<Mod>(), c.log_n, l, c.nP);
        });
    }
    PtrStore ms{mid, mps, c.log_n};
    ntt_fwd(c, 2 * l, QlpMap{l, 0, l, c.nQ}, PtrLoad{mid, mps, c.log_n}, ms, ms, s);
    count_launch();
    launch_pdl(c.pdl, moddown_combine<Base>, dim3(grid_for((size_t)l << c.log_n, 256)), dim3(256), 0, s, out0, out1,
               (const uint64_t *)mid, mps, (const uint64_t *)b.cx, cps, c.p_inv.as<uint64_t>(), c.d_mods.as<Mod>(),
               c.log_n, l, base);
}

void ckks_keyswitch(const Context &c, const Workspace &w, uint64_t *ct, const uint64_t *c2, int l,
                    const uint64_t *const *evk, cudaStream_t s) {
    const KsBuffers b = ks_buffers(c, w);
    const long long lps = (long long)l << c.log_n;
    modup_inner_product(c, b, PtrLoad{c2, lps, c.log_n}, PlainOwn{c2, c.log_n}, l, evk, s);
    moddown_intt_p(c, b, l, s);
    moddown_ntt(c, b, b.tm, l, ct, ct + lps, InplaceBase{ct, lps, c.log_n}, s);
}

void ckks_mul_relin(const Context &c, const Workspace &w, uint64_t *ct1, const uint64_t *ct2, int l,
                    const uint64_t *const *rlk, cudaStream_t s) {
    const KsBuffers b = ks_buffers(c, w);
    const long long lps = (long long)l << c.log_n;
    const uint64_t *a1 = ct1 + lps, *b1 = ct2 + lps;
    modup_inner_product(c, b, TensorD2Load{a1, b1, c.d_mods.as<Mod>(), c.log_n}, TensorOwn{a1, b1, c.log_n}, l, rlk,
                        s);
    moddown_intt_p(c, b, l, s);
    // poly 0 goes to scratch first: poly 1's base still reads a0 at every position
    moddown_ntt(c, b, b.tm, l, b.g, ct1 + lps, TensorBase{ct1, ct2, lps, c.log_n}, s);
    cudaMemcpyAsync(ct1, b.g, lps * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
}

// ------------------------------------------------------------------ rescale

struct ConstTblMap {  // block b = polynomial b, one limb at table `tbl`
    int tbl;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &t) const {
        poly = b;
        k = 0;
        t = tbl;
        return true;
    }
};

// z (coefficient form, mod q_last) reduced into q_j
struct ZLoad {
    const uint64_t *z;
    int log_n;
    const Mod *mods;
    __device__ __forceinline__ uint64_t operator()(int p, int, int tbl, uint32_t idx) const {
        return reduce64(z[((size_t)p << log_n) + idx], mods[tbl]);
    }
};

struct RescaleStore {  // out = (in - v) * q_last^-1
    const uint64_t *in;
    uint64_t *out;
    long long ips, ops;
    const uint64_t *iq;
    const Mod *mods;
    int log_n;
    __device__ __forceinline__ void operator()(int p, int j, int tbl, uint32_t idx, uint64_t v) const {
        const uint64_t q = mods[tbl].q;
        const size_t o = ((size_t)j << log_n) + idx;
        out[p * ops + o] = mul_shoup(sub_mod(in[p * ips + o], v, q), iq[2 * j], iq[2 * j + 1], q);
    }
};

void ckks_rescale(const Context &c, const Workspace &w, const uint64_t *in, uint64_t *out, int size, int l,
                  cudaStream_t s) {
    const LevelTables &lt = *c.levels[l];
    uint64_t *z = w.base;  // [size][N]
    const long long ips = (long long)l << c.log_n, ops = (long long)(l - 1) << c.log_n;
    const long long zps = 1LL << c.log_n;
    PtrStore zs{z, zps, c.log_n};
    ntt_inv(c, size, ConstTblMap{l - 1}, PtrLoad{in + ((size_t)(l - 1) << c.log_n), ips, c.log_n}, zs, zs, s);
    PtrStore ms{out, ops, c.log_n};
    ntt_fwd(c, size * (l - 1), SeqMap{l - 1, 0}, ZLoad{z, c.log_n, c.d_mods.as<Mod>()}, ms,
            RescaleStore{in, out, ips, ops, lt.inv_qlast.as<uint64_t>(), c.d_mods.as<Mod>(), c.log_n}, s);
}

// HMult + relinearise + rescale.  With out_j = d_j + (cx_j - NTT(delta_j)) P^-1 the
// relinearised product, the rescale is (out_j - NTT(z mod q_j)) q_last^-1 with
// z = iNTT(out_{l-1}).  By linearity of the NTT:
//   z     = iNTT(d_{l-1}) + (iNTT(cx_{l-1}) - delta_{l-1}) P^-1        (mod q_{l-1})
//   res_j = (d_j + cx_j P^-1 - NTT(delta_j P^-1 + z mod q_j)) q_last^-1  (mod q_j).
// So the inverse NTT of the P limbs also transforms cx's limb l-1 and the tensor product's
// limb l-1 (2 more limbs per polynomial), and one forward NTT over 2(l-1) limbs — whose load
// computes delta_j, delta_{l-1}, z and the sum, and whose store adds d_j + cx_j P^-1 and
// scales — finishes the whole operation.  Every step is exact modular arithmetic, so the result
// equals the reference's multiply_and_relin_inplace + rescale_to_next_inplace word for word.
struct LastLimbMap {  // per polynomial: alpha P limbs of cx, cx limb l-1, tensor limb l-1
    int alpha, l, nQ;
    __device__ __forceinline__ bool operator()(int b, int &t, int &k, int &tbl) const {
        t = b / (alpha + 2);
        k = b % (alpha + 2);
        tbl = k < alpha ? nQ + k : l - 1;
        return true;
    }
};

struct LastLimbLoad {
    const uint64_t *cx;
    long long cps;
    TensorBase tb;
    const Mod *mods;
    int log_n, l, alpha;
    __device__ __forceinline__ uint64_t operator()(int t, int k, int tbl, uint32_t idx) const {
        if (k < alpha) return cx[t * cps + ((size_t)(l + k) << log_n) + idx];
        if (k == alpha) return cx[t * cps + ((size_t)(l - 1) << log_n) + idx];
        return tb(t, l - 1, mods[tbl], idx);
    }
};

struct LastLimbStore {
    uint64_t *cx;
    long long cps;
    uint64_t *zc, *zd;
    const uint64_t *phi;
    const Mod *mods;
    int log_n, l, alpha;
    __device__ __forceinline__ void operator()(int t, int k, int tbl, uint32_t idx, uint64_t v) const {
        if (k < alpha)
            cx[t * cps + ((size_t)(l + k) << log_n) + idx] = mul_shoup(v, phi[2 * k], phi[2 * k + 1], mods[tbl].q);
        else
            (k == alpha ? zc : zd)[((size_t)t << log_n) + idx] = v;
    }
};

// Final step of HMult + relin + rescale as one coalesced element-wise pass (two coefficients per
// thread, 16-byte loads): out_t[j] = (d_j + cx_t[j] P^-1 - v_t[j]) q_last^-1, v = the forward NTT
// of delta_j P^-1 + z, d_0 = a0 b0, d_1 = a0 b1 + a1 b0.  Kept out of the NTT's row pass, whose
// store sweep would issue these scattered loads only after its butterflies.
__global__ void __launch_bounds__(256) rescale_combine(uint64_t *out, const uint64_t *v, const uint64_t *cx,
                                                       long long cps, const uint64_t *a, const uint64_t *b,
                                                       long long lps, const uint64_t *pinv, const uint64_t *iq,
                                                       const Mod *mods, int log_n, int lm1) {
    pdl_wait();
    pdl_release();
    // one thread per coefficient pair of both output polynomials: every input word is read once
    // (streaming loads: nothing here is read again by this call), the outputs stored streaming
    const size_t half = (size_t)1 << (log_n - 1), per_poly = (size_t)lm1 * half;
    const size_t lm1n = (size_t)lm1 << log_n;
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < per_poly; r += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(r >> (log_n - 1));
        const size_t o = ((size_t)j << log_n) + 2 * (r & (half - 1));
        const Mod m = mods[j];
        const uint64_t pj = pinv[2 * j], pjs = pinv[2 * j + 1], qj = iq[2 * j], qjs = iq[2 * j + 1];
        const ulonglong2 a0 = __ldcs(reinterpret_cast<const ulonglong2 *>(a + o));
        const ulonglong2 b0 = __ldcs(reinterpret_cast<const ulonglong2 *>(b + o));
        const ulonglong2 a1 = __ldcs(reinterpret_cast<const ulonglong2 *>(a + lps + o));
        const ulonglong2 b1 = __ldcs(reinterpret_cast<const ulonglong2 *>(b + lps + o));
        uint64_t d[2][2];
        d[0][0] = mul_mod(a0.x, b0.x, m);
        d[0][1] = mul_mod(a0.y, b0.y, m);
        u128 s0 = mul_wide(a0.x, b1.x), s1 = mul_wide(a0.y, b1.y);
        mac(s0, a1.x, b0.x);
        mac(s1, a1.y, b0.y);
        d[1][0] = reduce128(s0, m);
        d[1][1] = reduce128(s1, m);
#pragma unroll
        for (int t = 0; t < 2; t++) {
            const ulonglong2 vv = __ldcs(reinterpret_cast<const ulonglong2 *>(v + (size_t)t * lm1n + o));
            const ulonglong2 cc = __ldcs(reinterpret_cast<const ulonglong2 *>(cx + t * cps + o));
            const uint64_t x0 = sub_mod(add_mod(d[t][0], mul_shoup(cc.x, pj, pjs, m.q), m.q), vv.x, m.q);
            const uint64_t x1 = sub_mod(add_mod(d[t][1], mul_shoup(cc.y, pj, pjs, m.q), m.q), vv.y, m.q);
            __stcs(reinterpret_cast<ulonglong2 *>(out + (size_t)t * lm1n + o),
                   make_ulonglong2(mul_shoup(x0, qj, qjs, m.q), mul_shoup(x1, qj, qjs, m.q)));
        }
    }
}

void ckks_mul_relin_rescale(const Context &c, const Workspace &w, const uint64_t *ct1, const uint64_t *ct2,
                            uint64_t *out, int l, const uint64_t *const *rlk, cudaStream_t s) {
    const KsBuffers b = ks_buffers(c, w);
    const LevelTables &lt = *c.levels[l];
    const Mod *mods = c.d_mods.as<Mod>();
    const long long lps = (long long)l << c.log_n;
    const uint64_t *a1 = ct1 + lps, *b1 = ct2 + lps;
    const TensorBase tb{ct1, ct2, lps, c.log_n};
    modup_inner_product(c, b, TensorD2Load{a1, b1, mods, c.log_n}, TensorOwn{a1, b1, c.log_n}, l, rlk, s);
    const int alpha = c.nP, qlp = l + alpha;
    const long long cps = (long long)qlp << c.log_n, ops = (long long)(l - 1) << c.log_n;
    uint64_t *zc = b.z, *zd = b.z + (2 << c.log_n);
    PtrStore mid{b.tm, (long long)(alpha + 2) << c.log_n, c.log_n};
    ntt_inv(c, 2 * (alpha + 2), LastLimbMap{alpha, l, c.nQ}, LastLimbLoad{b.cx, cps, tb, mods, c.log_n, l, alpha},
            mid, LastLimbStore{b.cx, cps, zc, zd, c.p_hat_inv.as<uint64_t>(), mods, c.log_n, l, alpha}, s);
    if (c.tc_on && lt.tc_rescale_ok) {
        pq_bconv_tc_launch<true>(c, lt, b.tm, ops, b.cx, cps, l, zc, zd, s);
    } else {
        with_digit_bound(alpha, [&]<int A>() {
            count_launch();
            launch_pdl(c.pdl, rescale_fused_bconv<A>, dim3(dim3(bconv_blocks(c), 2)), dim3(256), 0, s, b.tm, ops, b.cx, cps, zc, zd, c.p_mat.as<uint64_t>(), c.p_inv.as<uint64_t>(), mods, c.log_n, l, c.nP);
        });
    }
    PtrStore ms{b.tm, ops, c.log_n};
    PtrLoad ld{b.tm, ops, c.log_n};
    ntt_fwd(c, 2 * (l - 1), QlpMap{l - 1, 0, l, c.nQ}, ld, ms, ms, s);
    count_launch();
    launch_pdl(c.pdl, rescale_combine, dim3(grid_for((size_t)(l - 1) << (c.log_n - 1), 256)), dim3(256), 0, s, out,
               (const uint64_t *)b.tm, (const uint64_t *)b.cx, cps, ct1, ct2, lps, c.p_inv.as<uint64_t>(),
               lt.inv_qlast.as<uint64_t>(), mods, c.log_n, l - 1);
}

void ckks_tensor(const Context &c, uint64_t *ct1, const uint64_t *ct2, int l, cudaStream_t s);

// ------------------------------------------------------------------ Galois

// g[p][k][i] = src[p][k][perm[i]] for 2 polynomials of l limbs
__global__ void galois_permute(uint64_t *dst, const uint64_t *src, const uint32_t *perm, int log_n, size_t total) {
    pdl_wait();
    pdl_release();
    const uint32_t nmask = (1u << log_n) - 1;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const uint32_t idx = (uint32_t)e & nmask;
        dst[e] = src[(e & ~(size_t)nmask) + __ldg(perm + idx)];
    }
}

void ckks_apply_galois(const Context &c, const Workspace &w, uint64_t *ct, int l, const uint32_t *perm,
                       const uint64_t *const *gk, cudaStream_t s) {
    const KsBuffers b = ks_buffers(c, w);
    const long long lps = (long long)l << c.log_n;
    const size_t total = 2 * (size_t)lps;
    count_launch();
    launch_pdl(c.pdl, galois_permute, dim3(grid_for(total, 256)), dim3(256), 0, s, b.g, ct, perm, c.log_n, total);
    const uint64_t *g1 = b.g + lps;
    modup_inner_product(c, b, PtrLoad{g1, lps, c.log_n}, PlainOwn{g1, c.log_n}, l, gk, s);
    moddown_intt_p(c, b, l, s);
    moddown_ntt(c, b, b.tm, l, ct, ct + lps, FirstPolyBase{b.g, c.log_n}, s);
}

// ------------------------------------------------------------------ hoisting

constexpr int kMaxSteps = 32;
struct HoistSteps {
    const uint32_t *perm[kMaxSteps];
    const uint64_t *const *key[kMaxSteps];
    int count;
};

// acc_t[jj] (+)= sum_s sum_d T_d[jj][perm_s[i]] * key_s,d[t][twr(jj)][i]; own limbs read c1.
__global__ void __launch_bounds__(256) ks_inner_product_hoisted(uint64_t *cx, const uint64_t *tm,
                                                                const uint64_t *c1, HoistSteps steps,
                                                                const Mod *mods, int log_n, int l, int nQ,
                                                                int alpha, int beta, int qp, bool accumulate) {
    pdl_wait();
    pdl_release();
    const int qlp = l + alpha;
    const size_t total = (size_t)qlp << log_n;
    const uint32_t nmask = (1u << log_n) - 1;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int jj = (int)(e >> log_n);
        const uint32_t idx = (uint32_t)e & nmask;
        const int tbl = jj < l ? jj : nQ + (jj - l);
        const Mod m = mods[tbl];
        const int own_d = jj < l ? jj / alpha : -1;
        uint64_t r0 = accumulate ? cx[e] : 0, r1 = accumulate ? cx[total + e] : 0;
        for (int st = 0; st < steps.count; st++) {
            const uint32_t src = __ldg(steps.perm[st] + idx);
            u128 a{0, 0}, b{0, 0};
            int terms = 0;
            for (int d = 0; d < beta; d++) {
                const uint64_t x = d == own_d ? c1[((size_t)jj << log_n) + src]
                                              : tm[(((size_t)d * qlp + jj) << log_n) + src];
                const uint64_t *key = steps.key[st][d];
                if (terms == 7) {
                    a = u128{reduce128(a, m), 0};
                    b = u128{reduce128(b, m), 0};
                    terms = 1;
                }
                mac(a, x, __ldg(key + ((size_t)tbl << log_n) + idx));
                mac(b, x, __ldg(key + ((size_t)(qp + tbl) << log_n) + idx));
                terms++;
            }
            r0 = add_mod(r0, reduce128(a, m), m.q);
            r1 = add_mod(r1, reduce128(b, m), m.q);
        }
        cx[e] = r0;
        cx[total + e] = r1;
    }
}

// acc0[i] = sum_s c0[perm_s[i]]
__global__ void galois_sum(uint64_t *dst, const uint64_t *src, HoistSteps steps, const Mod *mods, int log_n,
                           size_t total, bool accumulate) {
    pdl_wait();
    pdl_release();
    const uint32_t nmask = (1u << log_n) - 1;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const uint32_t idx = (uint32_t)e & nmask;
        const uint64_t q = mods[e >> log_n].q;
        const size_t base = e & ~(size_t)nmask;
        uint64_t r = accumulate ? dst[e] : 0;
        for (int st = 0; st < steps.count; st++) r = add_mod(r, src[base + __ldg(steps.perm[st] + idx)], q);
        dst[e] = r;
    }
}

void ckks_hoisting(const Context &c, const Workspace &w, uint64_t *ct, int l, const std::vector<StepKey> &steps,
                   cudaStream_t s) {
    const KsBuffers b = ks_buffers(c, w);
    const long long lps = (long long)l << c.log_n;
    const uint64_t *c1 = ct + lps;
    uint64_t *acc0 = b.g;
    modup_ckks(c, b, PtrLoad{c1, lps, c.log_n}, l, s);
    const int qlp = l + c.nP;
    for (size_t s0 = 0; s0 < steps.size(); s0 += kMaxSteps) {
        HoistSteps hs{};
        hs.count = (int)std::min<size_t>(kMaxSteps, steps.size() - s0);
        for (int i = 0; i < hs.count; i++) {
            hs.perm[i] = steps[s0 + i].perm;
            hs.key[i] = steps[s0 + i].key;
        }
        const bool acc = s0 > 0;
        count_launch();
        launch_pdl(c.pdl, galois_sum, dim3(grid_for((size_t)lps, 256)), dim3(256), 0, s, acc0, ct, hs, c.d_mods.as<Mod>(), c.log_n, (size_t)lps, acc);
        count_launch();
        launch_pdl(c.pdl, ks_inner_product_hoisted, dim3(grid_for((size_t)qlp << c.log_n, 256)), dim3(256), 0, s, b.cx, b.tm, c1, hs, c.d_mods.as<Mod>(), c.log_n, l, c.nQ, c.nP, c.beta(l), c.nQ + c.nP, acc);
    }
    moddown_intt_p(c, b, l, s);
    moddown_ntt(c, b, b.tm, l, ct, ct + lps, FirstPolyBase{acc0, c.log_n}, s);
}

// Individual rotations sharing one mod-up of c1 (GB300 addition; the reference's
// hoisting_inplace returns only their sum).  outs[i] (2 polys at level l) = rotation by steps[i]:
// (sigma(c0) + ModDown(<sigma(ModUp(c1)), gk>)_0, ModDown(...)_1).  The automorphism is applied
// to the mod-up digits, exactly as hoisting_inplace does, so outs[i] decrypts like rotate() but
// is not word-identical to it.
void ckks_rotations_hoisted(const Context &c, const Workspace &w, const uint64_t *ct, int l,
                            const std::vector<StepKey> &steps, const std::vector<uint64_t *> &outs, cudaStream_t s) {
    const KsBuffers b = ks_buffers(c, w);
    const long long lps = (long long)l << c.log_n;
    const uint64_t *c1 = ct + lps;
    modup_ckks(c, b, PtrLoad{c1, lps, c.log_n}, l, s);
    const int qlp = l + c.nP;
    for (size_t i = 0; i < steps.size(); i++) {
        count_launch();
        launch_pdl(c.pdl, galois_permute, dim3(grid_for((size_t)lps, 256)), dim3(256), 0, s, b.g, ct, steps[i].perm, c.log_n, (size_t)lps);
        HoistSteps hs{};
        hs.count = 1;
        hs.perm[0] = steps[i].perm;
        hs.key[0] = steps[i].key;
        count_launch();
        launch_pdl(c.pdl, ks_inner_product_hoisted, dim3(grid_for((size_t)qlp << c.log_n, 256)), dim3(256), 0, s, b.cx, b.tm, c1, hs, c.d_mods.as<Mod>(), c.log_n, l, c.nQ, c.nP, c.beta(l), c.nQ + c.nP, false);
        moddown_intt_p(c, b, l, s);
        // the mod-down's scratch must not be tm (it still holds the shared mod-up)
        moddown_ntt(c, b, b.h, l, outs[i], outs[i] + lps, FirstPolyBase{b.g, c.log_n}, s);
    }
}

// ------------------------------------------------------------------ tensor (standalone)

__global__ void tensor_2x2(uint64_t *ct1, const uint64_t *ct2, const Mod *mods, int log_n, size_t lps, bool square) {
    pdl_wait();
    pdl_release();
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < lps; e += (size_t)gridDim.x * blockDim.x) {
        const Mod m = mods[e >> log_n];
        const uint64_t a0 = ct1[e], a1 = ct1[lps + e];
        const uint64_t b0 = square ? a0 : ct2[e], b1 = square ? a1 : ct2[lps + e];
        u128 acc = mul_wide(a0, b1);
        mac(acc, a1, b0);
        ct1[e] = mul_mod(a0, b0, m);
        ct1[lps + e] = reduce128(acc, m);
        ct1[2 * lps + e] = mul_mod(a1, b1, m);
    }
}

void ckks_tensor(const Context &c, uint64_t *ct1, const uint64_t *ct2, int l, cudaStream_t s) {
    const size_t lps = (size_t)l << c.log_n;
    count_launch();
    launch_pdl(c.pdl, tensor_2x2, dim3(grid_for(lps, 256)), dim3(256), 0, s, ct1, ct2, c.d_mods.as<Mod>(), c.log_n, lps, ct1 == ct2);
}

}  // namespace pfg
