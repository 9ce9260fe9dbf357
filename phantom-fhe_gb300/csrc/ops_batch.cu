// ops_batch.cu — batched CKKS HMult + relinearise + rescale over ciphertexts at uneven levels.
//
// The reference processes a batch as a host loop of single calls
// (multiply_and_relin_inplace + rescale_to_next_inplace, src/evaluate.cu:1061-1104, 1545-1565),
// re-reading the whole relinearisation key for every ciphertext.  Here one launch per pipeline
// step covers every ciphertext of the batch (up to kMaxBatch per launch set): each block looks up
// its ciphertext from a per-launch prefix table passed by value, so ciphertexts at different
// levels (different limb counts, digit counts and constant tables) share every launch, and the
// inner product walks all ciphertexts for one key limb inside a block, so each key word comes
// from HBM once per batch and from L1/L2 for the other ciphertexts.  The per-ciphertext
// arithmetic is exactly that of ckks_mul_relin_rescale (ops_ckks.cu), so every output equals the
// single call's word for word.
#include "bconv.cuh"
#include "bconv_tc.cuh"
#include "host_tables.hpp"
#include "ks_fused.cuh"
#include "launch.cuh"
#include "ops.hpp"

namespace pfg {

constexpr int kMaxBatch = 64;
constexpr int kSub = 64;  // "poly" argument of batched functors = item * kSub + sub-index

struct BatchItems {
    int count;
    int keyswitch;  // 0: HMult (c2 = a1 * b1, rescale at the end); 1: key switch of (a = ct, b = c2)
    // key switch combine: 0 out[c] += KeySwitch (in place); 1 out[c] = (g0, 0) + KeySwitch with g0
    // the item's permuted first polynomial in its scratch region g (a Galois automorphism)
    int galois;
    int l[kMaxBatch];
    // key switch combine: when add[c] is set, the item's two polynomials there are added too
    const uint64_t *add[kMaxBatch];
    const uint64_t *a[kMaxBatch], *b[kMaxBatch];
    uint64_t *out[kMaxBatch];
    uint64_t *ws[kMaxBatch];
    const uint64_t *phi[kMaxBatch], *mat[kMaxBatch], *iq[kMaxBatch];
};

struct Prefix {
    int count;
    int p[kMaxBatch + 1];
    __device__ __forceinline__ int find(int b) const {
        int c = 0;
        while (c + 1 < count && p[c + 1] <= b) c++;
        return c;
    }
};

// Offsets of the per-item scratch regions (same layout as the single-call workspace).
// `mid` is where a key switch's mod-down keeps its intermediate polynomials: the mod-up region
// tm, which is free by then, or h when tm must survive (hoisted rotations share one mod-up).
struct ScratchLayout {
    long long y, tm, cx, g, z, h, mid;
};

static ScratchLayout scratch_layout(const Context &c) {
    const long long n = (long long)c.n, nQ = c.nQ, qlp = nQ + c.nP, beta = c.beta(c.nQ);
    ScratchLayout s;
    s.y = 0;
    s.tm = s.y + nQ * n;
    s.cx = s.tm + beta * qlp * n;
    s.g = s.cx + 2 * qlp * n;
    s.z = s.g + 2 * nQ * n;
    s.h = s.z + 4 * n;  // [2][nQ][N]
    s.mid = s.tm;
    return s;
}

// ------------------------------------------------------------------ maps

struct BSeqMap {  // item c: limbs [0, l_c), table k  (mod-up inverse NTT)
    Prefix pre;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &tbl) const {
        const int c = pre.find(b);
        k = b - pre.p[c];
        poly = c * kSub;
        tbl = k;
        return true;
    }
};

struct BModupMap {  // item c: beta_c digits x (l_c + alpha) limbs, own limbs idle
    Prefix pre;
    int l[kMaxBatch];
    int nQ, alpha;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &jj, int &tbl) const {
        const int c = pre.find(b), r = b - pre.p[c], lc = l[c], qlp = lc + alpha;
        const int d = r / qlp;
        jj = r % qlp;
        poly = c * kSub + d;
        tbl = jj < lc ? jj : nQ + (jj - lc);
        return !(jj >= d * alpha && jj < d * alpha + alpha && jj < lc);
    }
};

struct BLastLimbMap {  // item c, poly t: alpha P limbs, cx limb l-1, tensor limb l-1
    Prefix pre;
    int l[kMaxBatch];
    int nQ, alpha;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &tbl) const {
        const int c = pre.find(b), r = b - pre.p[c];
        const int t = r / (alpha + 2);
        k = r % (alpha + 2);
        poly = c * kSub + t;
        tbl = k < alpha ? nQ + k : l[c] - 1;
        return true;
    }
};

struct BFinalMap {  // item c, poly t: limbs [0, l_c - drop)
    Prefix pre;
    int l[kMaxBatch];
    int drop;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &j, int &tbl) const {
        const int c = pre.find(b), r = b - pre.p[c], m = l[c] - drop;
        const int t = r / m;
        j = r % m;
        poly = c * kSub + t;
        tbl = j;
        return true;
    }
};

// ------------------------------------------------------------------ functors

struct BItemsRef {
    BatchItems it;
    ScratchLayout sl;
    int log_n, alpha;
    int drop;  // limbs the operation drops: 1 (HMult + rescale) or 0 (key switch)
    __device__ __forceinline__ long long qlp_n(int c) const { return (long long)(it.l[c] + alpha) << log_n; }
};

struct BPMap {  // item c, poly t: the alpha P limbs of cx (key switch: inverse NTT before the mod-down)
    Prefix pre;
    int alpha, nQ;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &tbl) const {
        const int c = pre.find(b), r = b - pre.p[c];
        poly = c * kSub + r / alpha;
        k = r % alpha;
        tbl = nQ + k;
        return true;
    }
};

// tensor-product term t of item c at limb j: t = 0: a0*b0, 1: a0*b1 + a1*b0, 2: a1*b1
__device__ __forceinline__ uint64_t tensor_term(const BatchItems &it, int c, int t, int j, uint32_t idx, int log_n,
                                                const Mod &m) {
    const long long lps = (long long)it.l[c] << log_n;
    const size_t o = ((size_t)j << log_n) + idx;
    const uint64_t *a = it.a[c], *b = it.b[c];
    if (t == 2) return mul_mod(a[lps + o], b[lps + o], m);
    const uint64_t a0 = a[o], b0 = b[o];
    if (t == 0) return mul_mod(a0, b0, m);
    u128 acc = mul_wide(a0, b[lps + o]);
    mac(acc, a[lps + o], b0);
    return reduce128(acc, m);
}

// the polynomial that is key-switched: HMult's d2 = a1 * b1, or the given c2
__device__ __forceinline__ uint64_t c2_term(const BatchItems &it, int c, int j, uint32_t idx, int log_n,
                                            const Mod &m) {
    if (it.keyswitch) return it.b[c][((size_t)j << log_n) + idx];
    return tensor_term(it, c, 2, j, idx, log_n, m);
}

struct BD2Load {  // mod-up inverse NTT input: c2
    BItemsRef r;
    const Mod *mods;
    __device__ __forceinline__ uint64_t operator()(int poly, int k, int tbl, uint32_t idx) const {
        return c2_term(r.it, poly / kSub, k, idx, r.log_n, mods[tbl]);
    }
};

// generic scratch access: ws[c] + region + sub * sub_stride(c) + k * N + idx
template <int REGION>
struct BScratch {
    BItemsRef r;
    __device__ __forceinline__ uint64_t *addr(int poly, int k, uint32_t idx) const {
        const int c = poly / kSub, sub = poly % kSub;
        long long off;
        long long ss;
        if (REGION == 0) {  // y [l][N]
            off = r.sl.y;
            ss = 0;
        } else if (REGION == 1) {  // tm [beta][qlp][N]
            off = r.sl.tm;
            ss = r.qlp_n(c);
        } else if (REGION == 2) {  // the mod-down's region (tm or h) as [2][alpha+2][N]
            off = r.sl.mid;
            ss = (long long)(r.alpha + 2) << r.log_n;
        } else {  // the mod-down's region (tm or h) as [2][l - drop][N]
            off = r.sl.mid;
            ss = (long long)(r.it.l[c] - r.drop) << r.log_n;
        }
        return r.it.ws[c] + off + sub * ss + ((long long)k << r.log_n) + idx;
    }
    __device__ __forceinline__ uint64_t operator()(int poly, int k, int, uint32_t idx) const { return *addr(poly, k, idx); }
    __device__ __forceinline__ void operator()(int poly, int k, int, uint32_t idx, uint64_t v) const {
        *addr(poly, k, idx) = v;
    }
};

struct BScaleYStore {  // y[k] = v * partQlHatInv_k
    BItemsRef r;
    const Mod *mods;
    __device__ __forceinline__ void operator()(int poly, int k, int tbl, uint32_t idx, uint64_t v) const {
        const int c = poly / kSub;
        const uint64_t *phi = r.it.phi[c];
        r.it.ws[c][r.sl.y + ((long long)k << r.log_n) + idx] = mul_shoup(v, phi[2 * k], phi[2 * k + 1], mods[tbl].q);
    }
};

struct BLastLoad {
    BItemsRef r;
    const Mod *mods;
    __device__ __forceinline__ uint64_t operator()(int poly, int k, int tbl, uint32_t idx) const {
        const int c = poly / kSub, t = poly % kSub, lc = r.it.l[c];
        const uint64_t *cx = r.it.ws[c] + r.sl.cx + t * r.qlp_n(c);
        if (k < r.alpha) return cx[((size_t)(lc + k) << r.log_n) + idx];
        if (k == r.alpha) return cx[((size_t)(lc - 1) << r.log_n) + idx];
        return tensor_term(r.it, c, t, lc - 1, idx, r.log_n, mods[tbl]);
    }
};

struct BLastStore {
    BItemsRef r;
    const uint64_t *phi;  // PHatInv pairs
    const Mod *mods;
    __device__ __forceinline__ void operator()(int poly, int k, int tbl, uint32_t idx, uint64_t v) const {
        const int c = poly / kSub, t = poly % kSub, lc = r.it.l[c];
        uint64_t *ws = r.it.ws[c];
        if (k < r.alpha) {
            ws[r.sl.cx + t * r.qlp_n(c) + ((long long)(lc + k) << r.log_n) + idx] =
                    mul_shoup(v, phi[2 * k], phi[2 * k + 1], mods[tbl].q);
        } else {
            const long long zoff = r.sl.z + ((long long)((k == r.alpha ? 0 : 2) + t) << r.log_n);
            ws[zoff + idx] = v;
        }
    }
};

// Key-switch combine of every item, (item, polynomial) = block row: ct_t[j] += (cx_t[j] - v) P^-1
// (keyswitch_inplace's add_to_ct_kernel, src/rns_bconv.cu:763-769), two coefficients per thread.
__global__ void __launch_bounds__(256) batch_keyswitch_combine(BItemsRef r, Prefix pre, const uint64_t *pinv,
                                                               const Mod *mods) {
    pdl_wait();
    pdl_release();
    const int c = pre.find(blockIdx.y), t = blockIdx.y - pre.p[c];
    const int lc = r.it.l[c], log_n = r.log_n;
    const size_t half = (size_t)1 << (log_n - 1), work = (size_t)lc * half;
    const uint64_t *ws = r.it.ws[c];
    const uint64_t *v = ws + r.sl.mid + t * ((long long)lc << log_n);
    const uint64_t *cx = ws + r.sl.cx + t * r.qlp_n(c);
    uint64_t *ct = r.it.out[c] + t * ((long long)lc << log_n);
    // the base: the output itself (in place), or (g0, 0) for an automorphism
    const uint64_t *base = r.it.galois ? (t == 0 ? ws + r.sl.g : nullptr) : ct;
    const uint64_t *addend = r.it.add[c] ? r.it.add[c] + t * ((long long)lc << log_n) : nullptr;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < work; e += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(e >> (log_n - 1));
        const size_t o = ((size_t)j << log_n) + 2 * (e & (half - 1));
        const Mod m = mods[j];
        const uint64_t pj = pinv[2 * j], pjs = pinv[2 * j + 1];
        const ulonglong2 vv = ld2(v + o), cc = ld2(cx + o), b = base ? ld2(base + o) : make_ulonglong2(0, 0);
        uint64_t r0 = add_mod(b.x, mul_shoup(sub_mod(cc.x, vv.x, m.q), pj, pjs, m.q), m.q);
        uint64_t r1 = add_mod(b.y, mul_shoup(sub_mod(cc.y, vv.y, m.q), pj, pjs, m.q), m.q);
        if (addend) {
            const ulonglong2 a = ld2(addend + o);
            r0 = add_mod(r0, a.x, m.q);
            r1 = add_mod(r1, a.y, m.q);
        }
        st2(ct + o, r0, r1);
    }
}

// Final combine of every item, (item, polynomial) = block row: out = (d_j + cx_j P^-1 - v) q_last^-1
// with v the forward NTT of w (stored plainly in the item's scratch), two coefficients per thread.
__global__ void __launch_bounds__(256) batch_rescale_combine(BItemsRef r, Prefix pre, const uint64_t *pinv,
                                                             const Mod *mods) {
    pdl_wait();
    pdl_release();
    const int c = pre.find(blockIdx.y), t = blockIdx.y - pre.p[c];
    const int lc = r.it.l[c], log_n = r.log_n;
    const size_t half = (size_t)1 << (log_n - 1), work = (size_t)(lc - 1) * half;
    const uint64_t *ws = r.it.ws[c];
    const uint64_t *v = ws + r.sl.tm + t * ((long long)(lc - 1) << log_n);
    const uint64_t *cx = ws + r.sl.cx + t * r.qlp_n(c);
    const uint64_t *iq = r.it.iq[c];
    uint64_t *out = r.it.out[c] + t * ((long long)(lc - 1) << log_n);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < work; e += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(e >> (log_n - 1));
        const uint32_t idx = (uint32_t)(2 * (e & (half - 1)));
        const size_t o = ((size_t)j << log_n) + idx;
        const Mod m = mods[j];
        const uint64_t pj = pinv[2 * j], pjs = pinv[2 * j + 1], qj = iq[2 * j], qjs = iq[2 * j + 1];
        const ulonglong2 vv = ld2(v + o), cc = ld2(cx + o);
        const uint64_t x0 = sub_mod(add_mod(tensor_term(r.it, c, t, j, idx, log_n, m), mul_shoup(cc.x, pj, pjs, m.q), m.q),
                                    vv.x, m.q);
        const uint64_t x1 = sub_mod(add_mod(tensor_term(r.it, c, t, j, idx + 1, log_n, m),
                                            mul_shoup(cc.y, pj, pjs, m.q), m.q),
                                    vv.y, m.q);
        st2(out + o, mul_shoup(x0, qj, qjs, m.q), mul_shoup(x1, qj, qjs, m.q));
    }
}

// ------------------------------------------------------------------ element-wise batch kernels

// Mod-up base conversion for (item, digit) = block row.
template <int A>
__global__ void __launch_bounds__(256) modup_bconv_batch(BItemsRef r, Prefix pre, const Mod *mods, int nQ) {
    pdl_wait();
    pdl_release();
    const int c = pre.find(blockIdx.y), d = blockIdx.y - pre.p[c];
    const int l = r.it.l[c], alpha = r.alpha, qlp = l + alpha, log_n = r.log_n;
    const int s0 = d * alpha, sz = min(alpha, l - s0);
    const uint64_t *y = r.it.ws[c] + r.sl.y;
    uint64_t *tm = r.it.ws[c] + r.sl.tm + (((size_t)d * qlp) << log_n);
    const uint64_t *mat = r.it.mat[c];
    const size_t half = (size_t)1 << (log_n - 1);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = 2 * e;
        uint64_t y0[A], y1[A];
#pragma unroll
        for (int i = 0; i < A; i++) {
            if (i >= sz) break;
            const ulonglong2 v = ld2(y + ((size_t)(s0 + i) << log_n) + idx);
            y0[i] = v.x;
            y1[i] = v.y;
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
            st2(tm + ((size_t)jj << log_n) + idx, reduce128(a0, m), reduce128(a1, m));
        }
    }
}

// Inner product for key limb blockIdx.y over every item that has it; the key tile is read from
// HBM for the first item and from cache for the others.
__global__ void __launch_bounds__(256) ks_inner_product_batch(BItemsRef r, const uint64_t *const *evk,
                                                              const Mod *mods, int nQ, int qp) {
    pdl_wait();
    pdl_release();
    const int tk = blockIdx.y, alpha = r.alpha, log_n = r.log_n;
    const Mod m = mods[tk];
    const size_t half = (size_t)1 << (log_n - 1);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = 2 * e;
        for (int c = 0; c < r.it.count; c++) {
            const int l = r.it.l[c];
            if (tk >= l && tk < nQ) continue;  // this level has dropped q_tk
            const int jj = tk < nQ ? tk : l + (tk - nQ), qlp = l + alpha, beta = (l + alpha - 1) / alpha;
            const int own_d = jj < l ? jj / alpha : -1;
            const uint64_t *tm = r.it.ws[c] + r.sl.tm;
            u128 a0{0, 0}, a1{0, 0}, b0{0, 0}, b1{0, 0};
            int terms = 0;
            for (int d = 0; d < beta; d++) {
                uint64_t x0, x1;
                if (d == own_d) {
                    x0 = c2_term(r.it, c, jj, (uint32_t)idx, log_n, m);
                    x1 = c2_term(r.it, c, jj, (uint32_t)idx + 1, log_n, m);
                } else {
                    const ulonglong2 v = ld2(tm + (((size_t)d * qlp + jj) << log_n) + idx);
                    x0 = v.x;
                    x1 = v.y;
                }
                const uint64_t *key = evk[d];
                const ulonglong2 k0 = ld2(key + ((size_t)tk << log_n) + idx);
                const ulonglong2 k1 = ld2(key + ((size_t)(qp + tk) << log_n) + idx);
                if (terms == 7) {
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
            uint64_t *cx = r.it.ws[c] + r.sl.cx + ((size_t)jj << log_n) + idx;
            st2(cx, reduce128(a0, m), reduce128(a1, m));
            st2(cx + ((size_t)qlp << log_n), reduce128(b0, m), reduce128(b1, m));
        }
    }
}

// The own-limb term of item c's mod-up: HMult's d2 = a1 * b1, or the key switch's c2.
struct BatchOwn {
    const uint64_t *a, *b;
    long long lps;  // offset of polynomial 1 (HMult)
    int keyswitch, log_n;
    __device__ __forceinline__ uint64_t operator()(int jj, const Mod &m, uint32_t idx) const {
        const size_t o = ((size_t)jj << log_n) + idx;
        if (keyswitch) return b[o];
        return mul_mod(a[lps + o], b[lps + o], m);
    }
};

// Mod-up row pass fused with the inner product for every item (ks_fused.cuh): block (c, tile,
// tk) is item c's output limb for key limb tk over one row tile, idle where item c's level has
// dropped q_tk.  The item index is the fastest grid dimension, so the blocks of all items that
// read the same key tile (tk, tile) run together and the key comes from HBM once per batch.
template <int LM>
__global__ void __launch_bounds__(FusedShape<kFusedBatchE>::kThreads, FusedShape<kFusedBatchE>::kCtas)
        ks_modup_ip_batch(BItemsRef r, NttTables T, const uint64_t *const *evk, int nQ, int qp) {
    using TM = FusedTmem<FusedShape<kFusedBatchE>::kCols>;
    pdl_wait();
    pdl_release();
    __shared__ uint64_t sm[fused_smem_words<LM, kFusedBatchE>()];
    __shared__ uint32_t tslot;
    const int c = (int)blockIdx.x, tk = (int)blockIdx.z, l = r.it.l[c], alpha = r.alpha, log_n = r.log_n;
    if (tk < nQ && tk >= l) return;  // uniform per block, before any barrier or allocation
    const int jj = tk < nQ ? tk : l + (tk - nQ);
    uint64_t *ws = r.it.ws[c];
    const BatchOwn own{r.it.a[c], r.it.b[c], (long long)l << log_n, r.it.keyswitch, log_n};
    const uint32_t tbase = TM::alloc(&tslot);
    modup_ip_tile<LM, kFusedBatchE>(sm, TM::lane(tbase), T, ws + r.sl.tm, own, evk, ws + r.sl.cx, l, nQ, alpha,
                                    (l + alpha - 1) / alpha, qp, jj, blockIdx.y);
    TM::free(tbase);
}

// Rescale-folded mod-down conversion for (item, poly) = block row (see rescale_fused_bconv).
template <int A>
__global__ void __launch_bounds__(256) rescale_bconv_batch(BItemsRef r, Prefix pre, const uint64_t *pmat,
                                                           const uint64_t *pinv, const Mod *mods) {
    pdl_wait();
    pdl_release();
    const int c = pre.find(blockIdx.y), t = blockIdx.y - pre.p[c];
    const int l = r.it.l[c], nP = r.alpha, log_n = r.log_n;
    uint64_t *ws = r.it.ws[c];
    const long long cps = r.qlp_n(c);
    const uint64_t *yp = ws + r.sl.cx + t * cps + ((size_t)l << log_n);
    const uint64_t *zc = ws + r.sl.z + ((size_t)t << log_n), *zd = ws + r.sl.z + ((size_t)(2 + t) << log_n);
    uint64_t *w = ws + r.sl.tm + t * ((long long)(l - 1) << log_n);
    const Mod ml = mods[l - 1];
    const uint64_t pli = pinv[2 * (l - 1)], plis = pinv[2 * (l - 1) + 1];
    const size_t half = (size_t)1 << (log_n - 1);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = 2 * e;
        uint64_t y0[A], y1[A];
#pragma unroll
        for (int k = 0; k < A; k++) {
            if (k >= nP) break;
            const ulonglong2 v = ld2(yp + ((size_t)k << log_n) + idx);
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
            const uint64_t cc = __ldg(pl + k);
            mac(a0, y0[k], cc);
            mac(a1, y1[k], cc);
        }
        const ulonglong2 vc = ld2(zc + idx), vd = ld2(zd + idx);
        const uint64_t z0 = add_mod(vd.x, mul_shoup(sub_mod(vc.x, reduce128(a0, ml), ml.q), pli, plis, ml.q), ml.q);
        const uint64_t z1 = add_mod(vd.y, mul_shoup(sub_mod(vc.y, reduce128(a1, ml), ml.q), pli, plis, ml.q), ml.q);
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
                const uint64_t cc = __ldg(row + k);
                mac(b0, y0[k], cc);
                mac(b1, y1[k], cc);
            }
            const uint64_t pj = pinv[2 * j], pjs = pinv[2 * j + 1];
            const uint64_t r0 = add_mod(mul_shoup(reduce128(b0, m), pj, pjs, m.q), reduce64(z0, m), m.q);
            const uint64_t r1 = add_mod(mul_shoup(reduce128(b1, m), pj, pjs, m.q), reduce64(z1, m), m.q);
            st2(w + ((size_t)j << log_n) + idx, r0, r1);
        }
    }
}

// ------------------------------------------------------------------ tensor-core group sources

// Mod-up of a batch: group = (item, digit) through a prefix over digit counts.
struct BatchModupSrc {
    Prefix pre;
    uint64_t *ws[kMaxBatch];
    const uint16_t *bmat[kMaxBatch];
    const TcOutMeta *meta[kMaxBatch];
    const int *nn[kMaxBatch];
    int l[kMaxBatch];
    long long y_off, tm_off;
    int alpha, log_n, kpad;
    __device__ __forceinline__ TcGroup operator()(int gidx) const {
        const int c = pre.find(gidx), d = gidx - pre.p[c], lc = l[c], qlp = lc + alpha;
        const int s0 = d * alpha, sz = min(alpha, lc - s0);
        return TcGroup{ws[c] + y_off + ((size_t)s0 << log_n), ws[c] + tm_off + (((size_t)d * qlp) << log_n),
                       bmat[c] + (size_t)d * 256 * kpad, meta[c] + d * tc::kMaxOut, nullptr, nullptr, sz, qlp - sz,
                       nn[c][d], lc};
    }
};

// Mod-down of a batched key switch (P -> Ql, no rescale): group = (item, polynomial).
struct BatchModdownSrc {
    uint64_t *ws[kMaxBatch];
    const uint16_t *bmat[kMaxBatch];
    const TcOutMeta *meta[kMaxBatch];
    int nn[kMaxBatch];
    int l[kMaxBatch];
    long long cx_off, tm_off;
    int alpha, log_n;
    __device__ __forceinline__ TcGroup operator()(int gidx) const {
        const int c = gidx >> 1, t = gidx & 1, lc = l[c];
        uint64_t *w = ws[c];
        const long long qlp_n = (long long)(lc + alpha) << log_n;
        return TcGroup{w + cx_off + t * qlp_n + ((size_t)lc << log_n), w + tm_off + t * ((long long)lc << log_n),
                       bmat[c], meta[c], nullptr, nullptr, alpha, lc, nn[c], lc};
    }
};

// Step 6 of a batch (P -> Ql fused with the rescale): group = (item, polynomial).
struct BatchRescaleSrc {
    uint64_t *ws[kMaxBatch];
    const uint16_t *bmat[kMaxBatch];
    const TcOutMeta *meta[kMaxBatch];
    int nn[kMaxBatch];
    int l[kMaxBatch];
    long long cx_off, tm_off, z_off;
    int alpha, log_n;
    __device__ __forceinline__ TcGroup operator()(int gidx) const {
        const int c = gidx >> 1, t = gidx & 1, lc = l[c];
        uint64_t *w = ws[c];
        const long long qlp_n = (long long)(lc + alpha) << log_n;
        return TcGroup{w + cx_off + t * qlp_n + ((size_t)lc << log_n), w + tm_off + t * ((long long)(lc - 1) << log_n),
                       bmat[c], meta[c], w + z_off + ((size_t)t << log_n), w + z_off + ((size_t)(2 + t) << log_n),
                       alpha, lc, nn[c], lc};
    }
};

// ------------------------------------------------------------------ driver

template <class F>
static Prefix make_prefix(int count, F per_item) {
    Prefix p{};
    p.count = count;
    p.p[0] = 0;
    for (int c = 0; c < count; c++) p.p[c + 1] = p.p[c] + per_item(c);
    return p;
}

// Steps 3 (mod-up forward NTT) and 4 (inner product) of every item: fused (column pass, then the
// fused row pass + inner product) or as separate kernels; the same words.
static void batch_modup_ntt_inner_product(const Context &c, const BItemsRef &r, const std::vector<int> &lv,
                                          const uint64_t *const *evk, cudaStream_t s) {
    const int count = r.it.count, alpha = c.nP, nQ = c.nQ;
    BModupMap mm{make_prefix(count, [&](int i) { return c.beta(lv[i]) * (lv[i] + alpha); }), {}, nQ, alpha};
    for (int i = 0; i < count; i++) mm.l[i] = lv[i];
    BScratch<1> tm{r};
    if (c.ks_fused_batch) {
        col_pass<true, false>(c, mm.pre.p[count], mm, tm, tm, s);
        using S = FusedShape<kFusedBatchE>;
        const dim3 grid((unsigned)count, (unsigned)(c.n / S::kTile), (unsigned)(nQ + alpha));
        const NttTables T = c.ntt();
        count_launch();
        switch (c.l2()) {
            case 6: launch_pdl(c.pdl, ks_modup_ip_batch<6>, grid, dim3(S::kThreads), 0, s, r, T, evk, nQ, nQ + alpha); break;
            case 7: launch_pdl(c.pdl, ks_modup_ip_batch<7>, grid, dim3(S::kThreads), 0, s, r, T, evk, nQ, nQ + alpha); break;
            case 8: launch_pdl(c.pdl, ks_modup_ip_batch<8>, grid, dim3(S::kThreads), 0, s, r, T, evk, nQ, nQ + alpha); break;
            case 9: launch_pdl(c.pdl, ks_modup_ip_batch<9>, grid, dim3(S::kThreads), 0, s, r, T, evk, nQ, nQ + alpha); break;
            default: throw std::logic_error("unsupported NTT split");
        }
        return;
    }
    ntt_fwd2(c, mm.pre.p[count], mm, tm, tm, tm, tm, s);
    const unsigned gx = (unsigned)std::max<uint64_t>(1, c.n / 512);
    count_launch();
    launch_pdl(c.pdl, ks_inner_product_batch, dim3(gx, (unsigned)(nQ + alpha)), dim3(256), 0, s, r, evk,
               c.d_mods.as<Mod>(), nQ, nQ + alpha);
}

void ckks_mul_relin_rescale_batch(const Context &c, uint64_t *ws_base, size_t item_words,
                                  const std::vector<BatchItem> &items, const uint64_t *const *rlk, cudaStream_t s) {
    const Mod *mods = c.d_mods.as<Mod>();
    const int alpha = c.nP, nQ = c.nQ;
    const unsigned gx = (unsigned)std::max<uint64_t>(1, c.n / 512);
    for (size_t base = 0; base < items.size(); base += kMaxBatch) {
        const int count = (int)std::min<size_t>(kMaxBatch, items.size() - base);
        BItemsRef r{};
        r.it.count = count;
        r.sl = scratch_layout(c);
        r.log_n = c.log_n;
        r.alpha = alpha;
        r.drop = 1;
        r.it.keyswitch = 0;
        for (int i = 0; i < count; i++) {
            const BatchItem &b = items[base + i];
            const LevelTables &lt = *c.levels[b.l];
            r.it.l[i] = b.l;
            r.it.a[i] = b.ct1;
            r.it.b[i] = b.ct2;
            r.it.out[i] = b.out;
            r.it.ws[i] = ws_base + (size_t)i * item_words;
            r.it.phi[i] = lt.part_hat_inv.as<uint64_t>();
            r.it.mat[i] = lt.modup_mat.as<uint64_t>();
            r.it.iq[i] = lt.inv_qlast.as<uint64_t>();
        }
        auto lvl = [&](int i) { return r.it.l[i]; };
        auto beta_of = [&](int i) { return c.beta(lvl(i)); };
        // 1. mod-up inverse NTT of d2 = a1 * b1, scaled by partQlHatInv
        {
            Prefix pre = make_prefix(count, lvl);
            BScratch<0> y{r};
            ntt_inv2(c, pre.p[count], BSeqMap{pre}, BD2Load{r, mods}, y, y, BScaleYStore{r, mods}, s);
        }
        bool tc_up = c.tc_on, tc_rs = c.tc_on;
        for (int i = 0; i < count; i++) {
            tc_up = tc_up && c.levels[lvl(i)]->tc_ok;
            tc_rs = tc_rs && c.levels[lvl(i)]->tc_rescale_ok;
        }
        // 2. mod-up base conversion, per (item, digit)
        {
            Prefix pre = make_prefix(count, beta_of);
            if (tc_up) {
                BatchModupSrc src{};
                src.pre = pre;
                for (int i = 0; i < count; i++) {
                    const LevelTables &lt = *c.levels[lvl(i)];
                    src.ws[i] = r.it.ws[i];
                    src.bmat[i] = lt.tc_modup.as<uint16_t>();
                    src.meta[i] = lt.tc_modup_meta.as<TcOutMeta>();
                    src.nn[i] = lt.tc_modup_nn.as<int>();
                    src.l[i] = lvl(i);
                }
                src.y_off = r.sl.y;
                src.tm_off = r.sl.tm;
                src.alpha = alpha;
                src.log_n = c.log_n;
                src.kpad = c.tc_kpad;
                tc_bconv_launch<false>(c.tc_kpad, c.num_sms, c.log_n, src, pre.p[count], mods,
                                       c.p_inv.as<uint64_t>(), c.d_status.as<unsigned>(), s, c.pdl);
            } else {
                with_digit_bound(alpha, [&]<int A>() {
                    count_launch();
                    launch_pdl(c.pdl, modup_bconv_batch<A>, dim3(dim3(gx, pre.p[count])), dim3(256), 0, s, r, pre, mods, nQ);
                });
            }
        }
        // 3-4. mod-up forward NTT of every digit's complement limbs and the inner product
        batch_modup_ntt_inner_product(c, r, std::vector<int>(r.it.l, r.it.l + count), rlk, s);
        // 5. inverse NTT of the P limbs (x PHatInv), cx limb l-1 and tensor limb l-1
        {
            BLastLimbMap lm{make_prefix(count, [&](int) { return 2 * (alpha + 2); }), {}, nQ, alpha};
            for (int i = 0; i < count; i++) lm.l[i] = lvl(i);
            BScratch<2> mid{r};
            ntt_inv2(c, lm.pre.p[count], lm, BLastLoad{r, mods}, mid, mid,
                     BLastStore{r, c.p_hat_inv.as<uint64_t>(), mods}, s);
        }
        // 6. w_j = delta_j P^-1 + z mod q_j
        if (tc_rs) {
            BatchRescaleSrc src{};
            for (int i = 0; i < count; i++) {
                const LevelTables &lt = *c.levels[lvl(i)];
                src.ws[i] = r.it.ws[i];
                src.bmat[i] = lt.tc_rescale.as<uint16_t>();
                src.meta[i] = lt.tc_rescale_meta.as<TcOutMeta>();
                src.nn[i] = lt.tc_rescale_nn;
                src.l[i] = lvl(i);
            }
            src.cx_off = r.sl.cx;
            src.tm_off = r.sl.tm;
            src.z_off = r.sl.z;
            src.alpha = alpha;
            src.log_n = c.log_n;
            tc_bconv_launch<true>(c.tc_kpad, c.num_sms, c.log_n, src, 2 * count, mods, c.p_inv.as<uint64_t>(),
                                  c.d_status.as<unsigned>(), s, c.pdl);
        } else {
            Prefix pre = make_prefix(count, [&](int) { return 2; });
            with_digit_bound(alpha, [&]<int A>() {
                count_launch();
                launch_pdl(c.pdl, rescale_bconv_batch<A>, dim3(dim3(gx, pre.p[count])), dim3(256), 0, s, r, pre, c.p_mat.as<uint64_t>(), c.p_inv.as<uint64_t>(), mods);
            });
        }
        // 7. forward NTT of w with the final combine
        {
            BFinalMap fm{make_prefix(count, [&](int i) { return 2 * (lvl(i) - 1); }), {}, 1};
            for (int i = 0; i < count; i++) fm.l[i] = lvl(i);
            BScratch<3> w{r};
            ntt_fwd2(c, fm.pre.p[count], fm, w, w, w, w, s);
            Prefix pre = make_prefix(count, [&](int) { return 2; });
            count_launch();
            launch_pdl(c.pdl, batch_rescale_combine, dim3(dim3(gx, pre.p[count])), dim3(256), 0, s, r, pre, c.p_inv.as<uint64_t>(), mods);
        }
    }
}

// ------------------------------------------------------------------ key-switch pipeline pieces

// Steps 1-2 of a key switch for every item: y = iNTT(c2) * partQlHatInv, then the tensor-core
// mod-up conversion into tm (the column pass and the rest follow separately).
static void batch_modup_convert(const Context &c, const BItemsRef &r, cudaStream_t s) {
    const Mod *mods = c.d_mods.as<Mod>();
    const int count = r.it.count;
    auto lvl = [&](int i) { return r.it.l[i]; };
    {
        Prefix pre = make_prefix(count, lvl);
        BScratch<0> y{r};
        ntt_inv2(c, pre.p[count], BSeqMap{pre}, BD2Load{r, mods}, y, y, BScaleYStore{r, mods}, s);
    }
    Prefix pre = make_prefix(count, [&](int i) { return c.beta(lvl(i)); });
    BatchModupSrc src{};
    src.pre = pre;
    for (int i = 0; i < count; i++) {
        const LevelTables &lt = *c.levels[lvl(i)];
        src.ws[i] = r.it.ws[i];
        src.bmat[i] = lt.tc_modup.as<uint16_t>();
        src.meta[i] = lt.tc_modup_meta.as<TcOutMeta>();
        src.nn[i] = lt.tc_modup_nn.as<int>();
        src.l[i] = lvl(i);
    }
    src.y_off = r.sl.y;
    src.tm_off = r.sl.tm;
    src.alpha = c.nP;
    src.log_n = c.log_n;
    src.kpad = c.tc_kpad;
    tc_bconv_launch<false>(c.tc_kpad, c.num_sms, c.log_n, src, pre.p[count], mods, c.p_inv.as<uint64_t>(),
                           c.d_status.as<unsigned>(), s, c.pdl);
}

// Steps 5-7 for every item: the P limbs of cx back to coefficients (x PHatInv), delta = P -> Ql on
// the tensor cores into the mod-down region, its forward NTT and the combine into out (in place,
// or from the automorphism's base (g0, 0)).
static void batch_moddown_combine(const Context &c, const BItemsRef &r, cudaStream_t s) {
    const Mod *mods = c.d_mods.as<Mod>();
    const int count = r.it.count, alpha = c.nP, nQ = c.nQ;
    auto lvl = [&](int i) { return r.it.l[i]; };
    {
        BPMap pm{make_prefix(count, [&](int) { return 2 * alpha; }), alpha, nQ};
        BScratch<2> mid{r};
        ntt_inv2(c, pm.pre.p[count], pm, BLastLoad{r, mods}, mid, mid, BLastStore{r, c.p_hat_inv.as<uint64_t>(), mods},
                 s);
    }
    {
        BatchModdownSrc src{};
        for (int i = 0; i < count; i++) {
            const LevelTables &lt = *c.levels[lvl(i)];
            src.ws[i] = r.it.ws[i];
            src.bmat[i] = lt.tc_moddown.as<uint16_t>();
            src.meta[i] = lt.tc_moddown_meta.as<TcOutMeta>();
            src.nn[i] = lt.tc_moddown_nn;
            src.l[i] = lvl(i);
        }
        src.cx_off = r.sl.cx;
        src.tm_off = r.sl.mid;
        src.alpha = alpha;
        src.log_n = c.log_n;
        tc_bconv_launch<false>(c.tc_kpad, c.num_sms, c.log_n, src, 2 * count, mods, c.p_inv.as<uint64_t>(),
                               c.d_status.as<unsigned>(), s, c.pdl);
    }
    BFinalMap fm{make_prefix(count, [&](int i) { return 2 * lvl(i); }), {}, 0};
    for (int i = 0; i < count; i++) fm.l[i] = lvl(i);
    BScratch<3> w{r};
    ntt_fwd2(c, fm.pre.p[count], fm, w, w, w, w, s);
    Prefix pre = make_prefix(count, [&](int) { return 2; });
    const unsigned gx = (unsigned)std::max<uint64_t>(1, c.n / 512);
    count_launch();
    launch_pdl(c.pdl, batch_keyswitch_combine, dim3(gx, pre.p[count]), dim3(256), 0, s, r, pre,
               c.p_inv.as<uint64_t>(), mods);
}

// Every level of the batch has the tensor-core mod-up and mod-down tables.
static bool batch_tc_ready(const Context &c, const std::vector<int> &levels) {
    bool tc = c.tc_on;
    for (int l : levels) tc = tc && c.levels[l]->tc_ok && c.levels[l]->tc_moddown_ok;
    return tc;
}

// Batched key switch (keyswitch_inplace, src/eval_key_switch.cu:95-182, over many ciphertexts at
// uneven levels with one key): the HMult pipeline with c2 given instead of a1 * b1, the P limbs'
// inverse NTT alone, the plain mod-down on the tensor cores and an in-place combine.  Without the
// tensor-core conversions for every level present it runs the single-call key switch per item.
void ckks_keyswitch_batch(const Context &c, uint64_t *ws_base, size_t item_words, const std::vector<KsItem> &items,
                          const uint64_t *const *evk, cudaStream_t s) {
    std::vector<int> levels;
    for (const KsItem &k : items) levels.push_back(k.l);
    if (!batch_tc_ready(c, levels)) {
        for (size_t i = 0; i < items.size(); i++)
            ckks_keyswitch(c, Workspace{ws_base + (i % kMaxBatch) * item_words, item_words}, items[i].ct, items[i].c2,
                           items[i].l, evk, s);
        return;
    }
    for (size_t base = 0; base < items.size(); base += kMaxBatch) {
        const int count = (int)std::min<size_t>(kMaxBatch, items.size() - base);
        BItemsRef r{};
        r.it.count = count;
        r.it.keyswitch = 1;
        r.sl = scratch_layout(c);
        r.log_n = c.log_n;
        r.alpha = c.nP;
        r.drop = 0;
        for (int i = 0; i < count; i++) {
            const KsItem &k = items[base + i];
            const LevelTables &lt = *c.levels[k.l];
            r.it.l[i] = k.l;
            r.it.a[i] = k.ct;
            r.it.b[i] = k.c2;
            r.it.out[i] = k.ct;
            r.it.ws[i] = ws_base + (size_t)i * item_words;
            r.it.phi[i] = lt.part_hat_inv.as<uint64_t>();
            r.it.mat[i] = lt.modup_mat.as<uint64_t>();
            r.it.iq[i] = nullptr;
        }
        batch_modup_convert(c, r, s);
        batch_modup_ntt_inner_product(c, r, std::vector<int>(r.it.l, r.it.l + count), evk, s);
        batch_moddown_combine(c, r, s);
    }
}

// ------------------------------------------------------------------ batched matrix-vector product

// g = the Galois automorphism of both polynomials of src_c (item c's ciphertext at its level):
// g[t][j][i] = src[t][j][perm[i]], into the item's scratch region g.  Block row = (item, limb).
struct PtrList {
    const uint64_t *p[kMaxBatch];
};

__global__ void __launch_bounds__(256) batch_galois_permute(BItemsRef r, Prefix pre, PtrList src,
                                                            const uint32_t *perm) {
    pdl_wait();
    pdl_release();
    const int c = pre.find(blockIdx.y), k = blockIdx.y - pre.p[c];  // k < 2 l_c: polynomial k / l_c
    const int log_n = r.log_n;
    const size_t n = (size_t)1 << log_n;
    const uint64_t *in = src.p[c] + ((size_t)k << log_n);
    uint64_t *out = r.it.ws[c] + r.sl.g + ((size_t)k << log_n);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = in[__ldg(perm + i)];
}

// Hoisted inner product, block (item c, row tile, key limb tk): cx_c = sum_d perm(T_d) * key_d
// over two coefficients per thread, with item c's shared mod-up T (region tm) read through the
// permutation and the own limbs from its permuted c1 (region g, polynomial 1).  The item index is
// the fastest grid dimension, so the blocks of all items that read one key tile run together and
// the tile comes from HBM once per launch; the parallelism is in the grid, each thread's digit
// chain is short.  The permutation keeps every warp's 32 words within 8 sectors (a Galois
// automorphism of the bit-reversed NTT order moves words only inside aligned 256-byte blocks).
// The single-call form is ks_inner_product_hoisted (one step).
__global__ void __launch_bounds__(256) ks_inner_product_hoisted_batch(BItemsRef r, const uint32_t *perm,
                                                                      const uint64_t *const *key, const Mod *mods,
                                                                      int nQ, int qp) {
    pdl_wait();
    pdl_release();
    const int c = (int)blockIdx.x, tk = (int)blockIdx.z, l = r.it.l[c], alpha = r.alpha, log_n = r.log_n;
    if (tk >= l && tk < nQ) return;  // this level has dropped q_tk
    const int jj = tk < nQ ? tk : l + (tk - nQ), qlp = l + alpha, beta = (l + alpha - 1) / alpha;
    const int own_d = jj < l ? jj / alpha : -1;
    const Mod m = mods[tk];
    const uint32_t idx = 2 * (blockIdx.y * blockDim.x + threadIdx.x);
    const uint64_t *ws = r.it.ws[c];
    const uint64_t *tm = ws + r.sl.tm, *g1 = ws + r.sl.g + ((size_t)l << log_n);
    const uint2 src = *reinterpret_cast<const uint2 *>(perm + idx);
    u128 a0{0, 0}, a1{0, 0}, b0{0, 0}, b1{0, 0};
    int terms = 0;
#pragma unroll 2
    for (int d = 0; d < beta; d++) {
        uint64_t x0, x1;
        if (d == own_d) {
            const ulonglong2 v = ld2(g1 + ((size_t)jj << log_n) + idx);
            x0 = v.x;
            x1 = v.y;
        } else {
            const uint64_t *t = tm + (((size_t)d * qlp + jj) << log_n);
            x0 = t[src.x];
            x1 = t[src.y];
        }
        // each key tile serves every item's block: cached loads
        const uint64_t *kd = key[d];
        const ulonglong2 k0 = __ldg(reinterpret_cast<const ulonglong2 *>(kd + ((size_t)tk << log_n) + idx));
        const ulonglong2 k1 = __ldg(reinterpret_cast<const ulonglong2 *>(kd + ((size_t)(qp + tk) << log_n) + idx));
        if (terms == 7) {
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
    uint64_t *cx = r.it.ws[c] + r.sl.cx + ((size_t)jj << log_n) + idx;
    st2(cx, reduce128(a0, m), reduce128(a1, m));
    st2(cx + ((size_t)qlp << log_n), reduce128(b0, m), reduce128(b1, m));
}

// Per-item pointers of a batched matrix-vector product.
struct MvItems {
    const uint64_t *ct[kMaxBatch];     // baby 0 (the input), 2 polys at level l
    uint64_t *slots[kMaxBatch];        // babies 1..G-1, then one inner sum per giant step: [G-1+B][2][l][N]
    const uint64_t *diags[kMaxBatch];  // [D][dl][N], limbs [0, l) read
    int l[kMaxBatch], dl[kMaxBatch];
};

// Every giant step's inner sum of every item in one launch: slot G - 1 + g of item c receives
// inner_g = sum_b baby_b * diag_(g G + b) (128-bit accumulation; the same words as the single
// call's mul_plain_sum: exact modular arithmetic).  Block (item c, tile of 512 coefficients, limb
// j), two coefficients per thread with 16-byte loads.  The item index is the fastest grid
// dimension: when items share one diagonal array (one matrix, dl its limb stride) the blocks that
// read a diagonal tile run together and the tile comes from HBM about once per launch, not once
// per item.  Each thread walks the giant steps and reads its words of every baby again for each
// one, from L1 or L2 after the first.
__global__ void __launch_bounds__(256) mul_plain_sums_batch(MvItems mv, int G, int steps, int D, const Mod *mods,
                                                            int log_n) {
    pdl_wait();
    pdl_release();
    const int c = (int)blockIdx.x, j = (int)blockIdx.z, l = mv.l[c];
    if (j >= l) return;  // uniform per block
    const size_t lps = (size_t)l << log_n, cts = 2 * lps, jo = (size_t)j << log_n;
    const size_t dstride = (size_t)mv.dl[c] << log_n;
    const uint32_t i = 2 * (blockIdx.y * blockDim.x + threadIdx.x);
    const Mod m = mods[j];
    const uint64_t *dg = mv.diags[c] + jo + i;
    for (int g = 0; g < steps; g++) {
        const int nt = min(G, D - g * G);
        u128 a0{0, 0}, a1{0, 0}, b0{0, 0}, b1{0, 0};  // polynomial 0, 1 at coefficients i, i + 1
        int terms = 0;
#pragma unroll 2
        for (int b = 0; b < nt; b++) {
            const uint64_t *ct = (b == 0 ? mv.ct[c] : mv.slots[c] + (size_t)(b - 1) * cts) + jo + i;
            const ulonglong2 p = __ldg(reinterpret_cast<const ulonglong2 *>(dg + (size_t)(g * G + b) * dstride));
            const ulonglong2 x = __ldg(reinterpret_cast<const ulonglong2 *>(ct));
            const ulonglong2 y = __ldg(reinterpret_cast<const ulonglong2 *>(ct + lps));
            if (terms == 7) {
                a0 = u128{reduce128(a0, m), 0};
                a1 = u128{reduce128(a1, m), 0};
                b0 = u128{reduce128(b0, m), 0};
                b1 = u128{reduce128(b1, m), 0};
                terms = 1;
            }
            mac(a0, x.x, p.x);
            mac(a1, x.y, p.y);
            mac(b0, y.x, p.x);
            mac(b1, y.y, p.y);
            terms++;
        }
        uint64_t *out = mv.slots[c] + (size_t)(G - 1 + g) * cts + jo + i;
        st2(out, reduce128(a0, m), reduce128(a1, m));
        st2(out + lps, reduce128(b0, m), reduce128(b1, m));
    }
}

// Baby-step/giant-step products of many ciphertexts at uneven levels in the hoisted form of
// ckks_bsgs_matvec (ops_linear.cu), one launch per pipeline step over up to 64 of them: the
// baby rotations share each item's mod-up of c1 and read every key once per launch; the giant
// steps rotate every item's running sum by G together (Horner's rule); each output equals the
// single call's word for word.  Scratch per item: bsgs_batch_scratch_words(c, G, B) at
// scratch_base + i * scratch_words (the babies, then every giant step's inner sum).  Without the
// tensor-core conversions for every level it runs the single call per item.
void ckks_bsgs_matvec_batch(Context &c, uint64_t *ws_base, size_t item_words, uint64_t *scratch_base,
                            size_t scratch_words, const std::vector<MatvecItem> &items, int D, int G, int B,
                            const uint64_t *const *const *galois_keys, cudaStream_t s) {
    std::vector<int> levels;
    for (const MatvecItem &it : items) levels.push_back(it.l);
    const int alpha = c.nP, nQ = c.nQ;
    if (!batch_tc_ready(c, levels) || alpha + 2 > nQ) {
        for (size_t i = 0; i < items.size(); i++)
            ckks_bsgs_matvec(c, Workspace{ws_base + (i % kMaxBatch) * item_words, item_words},
                             scratch_base + (i % kMaxBatch) * scratch_words, items[i].ct, items[i].l, items[i].diags,
                             D, G, B, galois_keys, items[i].out, true, s, items[i].dl);
        return;
    }
    auto step_key = [&](int step) {
        const uint32_t elt = host::elt_from_step(step, c.n);
        for (size_t i = 0; i < c.galois_elts.size(); i++)
            if (c.galois_elts[i] == elt && galois_keys[i]) return StepKey{c.perm_table(elt), galois_keys[i]};
        throw std::invalid_argument("Galois key not present for a baby or giant step");
    };
    std::vector<StepKey> baby;
    for (int b = 1; b < G; b++) baby.push_back(step_key(b));
    const StepKey giant = B > 1 ? step_key(G) : StepKey{nullptr, nullptr};
    const Mod *mods = c.d_mods.as<Mod>();
    const unsigned gx = (unsigned)std::max<uint64_t>(1, c.n / 512);
    for (size_t base = 0; base < items.size(); base += kMaxBatch) {
        const int count = (int)std::min<size_t>(kMaxBatch, items.size() - base);
        BItemsRef r{};
        r.it.count = count;
        r.it.keyswitch = 1;
        r.it.galois = 1;
        r.sl = scratch_layout(c);
        r.log_n = c.log_n;
        r.alpha = alpha;
        r.drop = 0;
        MvItems mv{};
        std::vector<const uint64_t *> cts(count), res_ptr(count);
        for (int i = 0; i < count; i++) {
            const MatvecItem &m = items[base + i];
            const LevelTables &lt = *c.levels[m.l];
            r.it.l[i] = m.l;
            r.it.ws[i] = ws_base + (size_t)i * item_words;
            r.it.phi[i] = lt.part_hat_inv.as<uint64_t>();
            r.it.mat[i] = lt.modup_mat.as<uint64_t>();
            mv.ct[i] = m.ct;
            mv.slots[i] = scratch_base + (size_t)i * scratch_words;
            mv.diags[i] = m.diags;
            mv.l[i] = m.l;
            mv.dl[i] = m.dl;
            cts[i] = m.ct;
        }
        auto ptr_list = [&](const std::vector<const uint64_t *> &v) {
            PtrList pl{};
            for (int i = 0; i < count; i++) pl.p[i] = v[i];
            return pl;
        };
        Prefix limbs2 = make_prefix(count, [&](int i) { return 2 * mv.l[i]; });
        // 1. baby steps: one mod-up of each item's c1, kept in tm; per step the permuted input in g,
        //    the hoisted inner product, the mod-down into the region h (tm survives) and the combine
        //    into baby b
        if (G > 1) {
            for (int i = 0; i < count; i++) {
                r.it.a[i] = mv.ct[i];
                r.it.b[i] = mv.ct[i] + ((size_t)mv.l[i] << c.log_n);
            }
            batch_modup_convert(c, r, s);
            BModupMap mm{make_prefix(count, [&](int i) { return c.beta(mv.l[i]) * (mv.l[i] + alpha); }), {}, nQ,
                         alpha};
            for (int i = 0; i < count; i++) mm.l[i] = mv.l[i];
            BScratch<1> tm{r};
            ntt_fwd2(c, mm.pre.p[count], mm, tm, tm, tm, tm, s);
            r.sl.mid = r.sl.h;
            for (int b = 1; b < G; b++) {
                for (int i = 0; i < count; i++) r.it.out[i] = mv.slots[i] + (size_t)(b - 1) * 2 * ((size_t)mv.l[i] << c.log_n);
                count_launch();
                launch_pdl(c.pdl, batch_galois_permute, dim3(gx, limbs2.p[count]), dim3(256), 0, s, r, limbs2,
                           ptr_list(cts), baby[b - 1].perm);
                count_launch();
                launch_pdl(c.pdl, ks_inner_product_hoisted_batch,
                           dim3((unsigned)count, (unsigned)(c.n / 512), (unsigned)(nQ + alpha)), dim3(256), 0, s, r,
                           baby[b - 1].perm, baby[b - 1].key, mods, nQ, nQ + alpha);
                batch_moddown_combine(c, r, s);
            }
            r.sl.mid = r.sl.tm;
        }
        // 2. every giant step's inner sum in one launch (slots G - 1 ..), then Horner's rule:
        //    result = inner_gl (gl the last giant step with diagonals), result = rot_G(result) +
        //    inner_g for g = gl - 1 .. 0, the addition folded into the rotation's combine
        const int gl = (D - 1) / G;
        {
            int lmax = 0;
            for (int i = 0; i < count; i++) lmax = std::max(lmax, mv.l[i]);
            count_launch();
            launch_pdl(c.pdl, mul_plain_sums_batch, dim3((unsigned)count, (unsigned)(c.n / 512), (unsigned)lmax),
                       dim3(256), 0, s, mv, G, gl + 1, D, mods, c.log_n);
        }
        auto slot = [&](int i, int k) { return mv.slots[i] + (size_t)k * 2 * ((size_t)mv.l[i] << c.log_n); };
        for (int i = 0; i < count; i++) res_ptr[i] = slot(i, G - 1 + gl);
        for (int g = gl - 1; g >= 0; g--) {
            // rotate every item's result by G (permute, then key switch g1 onto (g0, 0)) plus inner_g
            for (int i = 0; i < count; i++) {
                r.it.out[i] = const_cast<uint64_t *>(res_ptr[i]);
                r.it.b[i] = r.it.ws[i] + r.sl.g + ((size_t)mv.l[i] << c.log_n);
                r.it.add[i] = slot(i, G - 1 + g);
            }
            count_launch();
            launch_pdl(c.pdl, batch_galois_permute, dim3(gx, limbs2.p[count]), dim3(256), 0, s, r, limbs2,
                       ptr_list(res_ptr), giant.perm);
            batch_modup_convert(c, r, s);
            batch_modup_ntt_inner_product(c, r, std::vector<int>(mv.l, mv.l + count), giant.key, s);
            batch_moddown_combine(c, r, s);
        }
        for (int i = 0; i < count; i++) r.it.add[i] = nullptr;
        // 3. rescale every result
        for (int i = 0; i < count; i++)
            ckks_rescale(c, Workspace{r.it.ws[i], item_words}, res_ptr[i], items[base + i].out, 2, mv.l[i], s);
    }
}

}  // namespace pfg
