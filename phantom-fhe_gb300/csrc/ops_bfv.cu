// ops_bfv.cu — BFV multiply + relinearise with the HPS method (mul_tech::hps), BFV key
// switching and BFV modulus switching.
//
// Restates src/evaluate.cu:820-1026 (bfv_mul_relin_hps):
//   1. ct1, ct2: Q -> R by DBaseConverter::bConv_HPS (src/rns_bconv.cu:354-372, kernel
//      :277-310) — FP64 correction v = llround(sum_i y_i * (1/q_i)), accumulated with fused
//      multiply-adds in the reference's loop order (nvcc contracts `acc += a * b`);
//   2. forward NTT over QR, tensor product, inverse NTT (the tensor is computed inside the
//      inverse NTT's load, never written);
//   3. scaleAndRound_HPS_QR_R (src/rns.cu:1700-1747) fused with the R -> Q bConv_HPS — note the
//      reference reduces its FP64 carry `alpha` in place, so prime r_j sees
//      (...(alpha mod r_0)... ) mod r_j; this is reproduced;
//   4. relinearisation of c2 in the coefficient domain (DRNSTool::modup / moddown_from_NTT BFV
//      branches, src/rns_bconv.cu:530-628, 776-828).
#include <stdexcept>
#include <string>

#include "bconv.cuh"
#include "bconv_tc.cuh"
#include "hps_tc.cuh"
#include "keyswitch.cuh"
#include "launch.cuh"
#include "ops.hpp"

namespace pfg {

static int grid_for_bfv(size_t work, int per_block) {
    size_t b = (work + per_block - 1) / per_block;
    return (int)std::min<size_t>(b, 2 * kGridStrideBlocks);
}

// ------------------------------------------------------------------ HPS base conversion

// Both HPS kernels work on a tile of kHpsTile coefficients per block of 256 threads, with the
// tile's inputs in shared memory: the per-coefficient FP64 sums run in the reference's loop order
// (one thread per coefficient), and the integer sums are spread over (output limb, coefficient)
// pairs so every thread is busy.
constexpr int kHpsTile = 64;

// out[j] = (sum_i y_i * mat[j][i] mod p_j) - alpha_tab[v][j],  y_i = x_i * hat_inv_i mod q_i,
// v = llround(sum_i fma(y_i, inv_i)).
__global__ void __launch_bounds__(256) hps_bconv(uint64_t *out, long long ops, const uint64_t *in, long long ips,
                                                 const Mod *mods, int ib0, int ni, int ob0, int no,
                                                 const uint64_t *hat_inv, const double *inv, const uint64_t *mat,
                                                 const uint64_t *alpha_tab, int log_n) {
    pdl_wait();
    pdl_release();
    extern __shared__ uint64_t sh[];
    uint64_t *ys = sh;                                  // [ni][kHpsTile]
    long long *vs = reinterpret_cast<long long *>(sh + (size_t)ni * kHpsTile);  // [kHpsTile]
    const uint32_t n = 1u << log_n;
    const int poly = blockIdx.y;
    const uint32_t c0 = blockIdx.x * kHpsTile;
    const uint64_t *x = in + poly * ips + c0;
    for (int p = threadIdx.x; p < ni * kHpsTile; p += blockDim.x) {
        const int i = p / kHpsTile, c = p % kHpsTile;
        ys[p] = mul_shoup(x[(size_t)i * n + c], hat_inv[2 * i], hat_inv[2 * i + 1], mods[ib0 + i].q);
    }
    __syncthreads();
    if (threadIdx.x < kHpsTile) {
        double acc = 0.0;
        for (int i = 0; i < ni; i++) acc = __fma_rn(__ull2double_rn(ys[i * kHpsTile + threadIdx.x]), inv[i], acc);
        vs[threadIdx.x] = llround(acc);
    }
    __syncthreads();
    uint64_t *o = out + poly * ops + c0;
    for (int p = threadIdx.x; p < no * kHpsTile; p += blockDim.x) {
        const int j = p / kHpsTile, c = p % kHpsTile;
        const Mod m = mods[ob0 + j];
        const uint64_t *row = mat + (size_t)j * ni;
        u128 acc{0, 0};
        int terms = 0;
        for (int i = 0; i < ni; i++) {
            if (terms == 7) {
                acc = u128{reduce128(acc, m), 0};
                terms = 1;
            }
            mac(acc, ys[i * kHpsTile + c], __ldg(row + i));
            terms++;
        }
        o[(size_t)j * n + c] = sub_mod(reduce128(acc, m), __ldg(alpha_tab + (size_t)vs[c] * no + j), m.q);
    }
}

// scaleAndRound_HPS_QR_R followed by bConv_HPS R -> Q.
__global__ void __launch_bounds__(256) hps_scale_round_to_q(uint64_t *out, long long ops, const uint64_t *in,
                                                            long long ips, const Mod *mods, int nQ, int rbase,
                                                            int nR, const double *frac, const uint64_t *modr,
                                                            const uint64_t *r_hat_inv, const double *r_inv,
                                                            const uint64_t *r2q, const uint64_t *r2q_alpha,
                                                            int log_n) {
    pdl_wait();
    pdl_release();
    extern __shared__ uint64_t sh[];
    const int nqr = nQ + nR;
    uint64_t *xs = sh;                                   // [nQ + nR][kHpsTile]
    uint64_t *ys = xs + (size_t)nqr * kHpsTile;          // [nR][kHpsTile]
    uint64_t *as = ys + (size_t)nR * kHpsTile;           // [nR][kHpsTile] carry alpha, reduced in place
    long long *vs = reinterpret_cast<long long *>(as + (size_t)nR * kHpsTile);  // [kHpsTile]
    const uint32_t n = 1u << log_n;
    const int poly = blockIdx.y;
    const uint32_t c0 = blockIdx.x * kHpsTile;
    const uint64_t *x = in + poly * ips + c0;
    for (int p = threadIdx.x; p < nqr * kHpsTile; p += blockDim.x)
        xs[p] = x[(size_t)(p / kHpsTile) * n + (p % kHpsTile)];
    __syncthreads();
    if (threadIdx.x < kHpsTile) {
        double nu = 0.5;
        for (int i = 0; i < nQ; i++) nu = __fma_rn(__ull2double_rn(xs[i * kHpsTile + threadIdx.x]), frac[i], nu);
        // the reference reduces alpha in place across r_0 .. r_j; keep every step of that chain
        uint64_t alpha = __double2ull_rz(nu);
        for (int j = 0; j < nR; j++) {
            alpha = reduce64(alpha, mods[rbase + j]);
            as[j * kHpsTile + threadIdx.x] = alpha;
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < nR * kHpsTile; p += blockDim.x) {
        const int j = p / kHpsTile, c = p % kHpsTile;
        const Mod m = mods[rbase + j];
        const uint64_t *row = modr + (size_t)j * (nQ + 1);
        u128 cur{0, 0};
        int terms = 0;
        for (int i = 0; i < nQ; i++) {
            if (terms == 7) {
                cur = u128{reduce128(cur, m), 0};
                terms = 1;
            }
            mac(cur, xs[i * kHpsTile + c], __ldg(row + i));
            terms++;
        }
        if (terms == 7) cur = u128{reduce128(cur, m), 0};
        mac(cur, xs[(nQ + j) * kHpsTile + c], __ldg(row + nQ));
        const uint64_t rt = add_mod(reduce128(cur, m), as[p], m.q);
        ys[p] = mul_shoup(rt, r_hat_inv[2 * j], r_hat_inv[2 * j + 1], m.q);
    }
    __syncthreads();
    if (threadIdx.x < kHpsTile) {
        double acc = 0.0;
        for (int j = 0; j < nR; j++) acc = __fma_rn(__ull2double_rn(ys[j * kHpsTile + threadIdx.x]), r_inv[j], acc);
        vs[threadIdx.x] = llround(acc);
    }
    __syncthreads();
    uint64_t *o = out + poly * ops + c0;
    for (int p = threadIdx.x; p < nQ * kHpsTile; p += blockDim.x) {
        const int i = p / kHpsTile, c = p % kHpsTile;
        const Mod m = mods[i];
        u128 s{0, 0};
        int terms = 0;
        for (int j = 0; j < nR; j++) {
            if (terms == 7) {
                s = u128{reduce128(s, m), 0};
                terms = 1;
            }
            mac(s, ys[j * kHpsTile + c], __ldg(r2q + (size_t)i * nR + j));
            terms++;
        }
        o[(size_t)i * n + c] = sub_mod(reduce128(s, m), __ldg(r2q_alpha + (size_t)vs[c] * nQ + i), m.q);
    }
}

// ------------------------------------------------------------------ QR transforms

struct QrMap {  // [poly][nQ + nR][N]; R limbs use tables nQ + nP + j
    int qr, nQ, nP;
    __device__ __forceinline__ bool operator()(int b, int &poly, int &k, int &tbl) const {
        poly = b / qr;
        k = b % qr;
        tbl = k < nQ ? k : k + nP;
        return true;
    }
};

// tensor product component `poly` of (ea, eb) over QR, computed in the inverse NTT's load
struct TensorQrLoad {
    const uint64_t *ea, *eb;
    long long ps;
    const Mod *mods;
    int log_n;
    __device__ __forceinline__ uint64_t operator()(int poly, int k, int tbl, uint32_t idx) const {
        const size_t o = ((size_t)k << log_n) + idx;
        const Mod m = mods[tbl];
        const uint64_t a0 = ea[o], a1 = ea[ps + o], b0 = eb[o], b1 = eb[ps + o];
        if (poly == 0) return mul_mod(a0, b0, m);
        if (poly == 2) return mul_mod(a1, b1, m);
        u128 acc = mul_wide(a0, b1);
        mac(acc, a1, b0);
        return reduce128(acc, m);
    }
};

// ------------------------------------------------------------------ relinearisation (BFV)

// After the inverse NTT of cx: Q limbs unchanged, P limbs times PHatInv.
struct BfvCxStore {
    uint64_t *cx;
    long long cps;
    int log_n, l;
    const uint64_t *phi;
    const Mod *mods;
    __device__ __forceinline__ void operator()(int t, int k, int tbl, uint32_t idx, uint64_t v) const {
        if (k >= l) v = mul_shoup(v, phi[2 * (k - l)], phi[2 * (k - l) + 1], mods[tbl].q);
        cx[t * cps + ((long long)k << log_n) + idx] = v;
    }
};

// out_t[j] = base_t[j] + (cx_t[j] - delta_j) * P^-1, delta_j = sum_k yp_k * (P/p_k) mod q_j
__global__ void bfv_moddown_combine(uint64_t *out, long long ops, const uint64_t *base, long long bps,
                                    const uint64_t *cx, long long cps, const uint64_t *pmat, const uint64_t *pinv,
                                    const Mod *mods, int l, int nP, int log_n) {
    pdl_wait();
    pdl_release();
    const size_t total = (size_t)2 * l << log_n;
    const uint32_t nmask = (1u << log_n) - 1;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int t = (int)(e / ((size_t)l << log_n));
        const size_t r = e - (size_t)t * ((size_t)l << log_n);
        const int j = (int)(r >> log_n);
        const uint32_t idx = (uint32_t)r & nmask;
        const Mod m = mods[j];
        const uint64_t *yp = cx + t * cps + ((size_t)l << log_n) + idx;
        u128 acc{0, 0};
        for (int k = 0; k < nP; k++) mac(acc, yp[(size_t)k << log_n], __ldg(pmat + (size_t)j * nP + k));
        const uint64_t delta = reduce128(acc, m);
        const uint64_t d = mul_shoup(sub_mod(cx[t * cps + r], delta, m.q), pinv[2 * j], pinv[2 * j + 1], m.q);
        out[t * ops + r] = add_mod(base[t * bps + r], d, m.q);
    }
}

// Key switch of c2 (coefficient form) added to `base` (2 polys), written to out (2 polys).
static void bfv_keyswitch_to(const Context &c, uint64_t *scratch, uint64_t *out, const uint64_t *base,
                             const uint64_t *c2, int l, const uint64_t *const *evk, cudaStream_t s) {
    const LevelTables &lt = *c.levels[l];
    const int alpha = c.nP, qlp = l + alpha, beta = lt.beta;
    uint64_t *tm = scratch;
    uint64_t *cx = tm + ((size_t)beta * qlp << c.log_n);
    const long long tps = (long long)qlp << c.log_n;
    // with two or fewer limbs per digit the CUDA-core conversion is as fast (measured at alpha = 2)
    if (c.tc_on && lt.tc_ok && alpha >= 3) {
        const BfvModupSrc src{c2, tm, lt.tc_modup.as<uint16_t>(), lt.tc_modup_meta.as<TcOutMeta>(),
                              lt.tc_modup_nn.as<int>(), lt.part_hat_inv.as<uint64_t>(), l, alpha, c.log_n, c.tc_kpad};
        tc_bconv_launch<false>(c.tc_kpad, c.num_sms, c.log_n, src, beta, c.d_mods.as<Mod>(), c.p_inv.as<uint64_t>(),
                               c.d_status.as<unsigned>(), s, c.pdl);
    } else {
        with_digit_bound(alpha, [&]<int A>() {
            count_launch();
            launch_pdl(c.pdl, modup_bconv<A, true>, dim3(dim3((unsigned)std::max<uint64_t>(1, c.n / 512), beta)), dim3(256), 0, s, tm, c2, lt.part_hat_inv.as<uint64_t>(), lt.modup_mat.as<uint64_t>(), c.d_mods.as<Mod>(), c.log_n, l, c.nQ, alpha);
        });
    }
    PtrStore ts{tm, tps, c.log_n};
    ntt_fwd(c, beta * qlp, ModupMap{qlp, l, c.nQ, alpha, false}, PtrLoad{tm, tps, c.log_n}, ts, ts, s);
    const size_t work = ((size_t)qlp << c.log_n) / 2;
    count_launch();
    launch_pdl(c.pdl, ks_inner_product<NoOwn, true>, dim3(grid_for_bfv(work, 256)), dim3(256), 0, s, cx, tm, NoOwn{}, evk, c.d_mods.as<Mod>(), c.log_n, l, c.nQ, alpha, beta, c.nQ + c.nP);
    PtrStore cs{cx, tps, c.log_n};
    ntt_inv(c, 2 * qlp, QlpMap{qlp, 0, l, c.nQ}, PtrLoad{cx, tps, c.log_n}, cs,
            BfvCxStore{cx, tps, c.log_n, l, c.p_hat_inv.as<uint64_t>(), c.d_mods.as<Mod>()}, s);
    const long long lps = (long long)l << c.log_n;
    count_launch();
    launch_pdl(c.pdl, bfv_moddown_combine, dim3(grid_for_bfv((size_t)2 * lps, 256)), dim3(256), 0, s, out, lps, base, lps, cx, tps, c.p_mat.as<uint64_t>(), c.p_inv.as<uint64_t>(), c.d_mods.as<Mod>(), l, c.nP, c.log_n);
}

void bfv_keyswitch(const Context &c, const Workspace &w, uint64_t *ct, const uint64_t *c2, int l,
                   const uint64_t *const *evk, cudaStream_t s) {
    bfv_keyswitch_to(c, w.base, ct, ct, c2, l, evk, s);
}

template <int MODE>
static void hps_tc_launch(const Context &c, const HpsTcArgs &a, cudaStream_t s) {
    const size_t smem = hps_tc_smem(a, MODE);
    if (smem + 4096 > (size_t)c.smem_optin) throw std::logic_error("HPS tensor-core tile exceeds shared memory");
    static int attr_set = 0;  // raised once to the device's opt-in limit (less the static part)
    if (!attr_set) {
        const cudaError_t e = cudaFuncSetAttribute(hps_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   c.smem_optin - 4096);
        if (e != cudaSuccess) throw std::runtime_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
        attr_set = 1;
    }
    const int per_sm = smem <= 100 * 1024 ? 2 : 1;  // 2 x 256 tensor-memory columns at most
    const int units = a.polys << (a.log_n - 7);
    count_launch();
    launch_pdl(c.pdl, hps_tc_kernel<MODE>, dim3(std::min(units, per_sm * c.num_sms)), dim3(256), smem, s, a);
}

// Q -> R (or R -> Q) HPS conversion of `polys` polynomials on the tensor cores.
static void hps_conv_tc(const Context &c, bool q2r, uint64_t *out, long long ops, const uint64_t *in, long long ips,
                        int polys, cudaStream_t s) {
    const int nQ = c.nQ, nR = c.nR, rbase = c.nQ + c.nP;
    HpsTcArgs a{};
    a.out = out;
    a.ops = ops;
    a.in = in;
    a.ips = ips;
    a.mods = c.d_mods.as<Mod>();
    a.in_tbl0 = q2r ? 0 : rbase;
    a.ni = q2r ? nQ : nR;
    a.out_tbl0 = q2r ? rbase : 0;
    a.no = q2r ? nR : nQ;
    a.hat_inv = (q2r ? c.hps_q_hat_inv : c.hps_r_hat_inv).as<uint64_t>();
    a.dinv = (q2r ? c.hps_q_inv : c.hps_r_inv).as<double>();
    a.bmat = (q2r ? c.tc_hps_q2r : c.tc_hps_r2q).as<uint16_t>();
    a.kp = q2r ? c.tc_hps_kp_q2r : c.tc_hps_kp_r2q;
    a.polys = polys;
    a.log_n = c.log_n;
    a.status = c.d_status.as<unsigned>();
    hps_tc_launch<kHpsConv>(c, a, s);
}

void bfv_mul_relin_hps(const Context &c, const Workspace &w, uint64_t *ct1, const uint64_t *ct2,
                       const uint64_t *const *rlk, cudaStream_t s) {
    const int nQ = c.nQ, nR = c.nR, qr = nQ + nR, rbase = c.nQ + c.nP;
    const size_t n = c.n;
    const long long qps = (long long)nQ * n, qrps = (long long)qr * n;
    uint64_t *ea = w.base, *eb = ea + 2 * qrps, *t3 = eb + 2 * qrps, *o3 = t3 + 3 * qrps, *ks = o3 + 3 * qps;
    const Mod *mods = c.d_mods.as<Mod>();
    const bool square = ct1 == ct2;
    // 1. extend both operands to QR
    cudaMemcpy2DAsync(ea, qrps * 8, ct1, qps * 8, qps * 8, 2, cudaMemcpyDeviceToDevice, s);
    dim3 g((unsigned)(n / kHpsTile), 2);
    const size_t sm_q = ((size_t)nQ + 1) * kHpsTile * 8, sm_r = ((size_t)3 * nR + nQ + 1) * kHpsTile * 8;
    if (sm_q > 48 * 1024) cudaFuncSetAttribute(hps_bconv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_q);
    if (sm_r > 48 * 1024)
        cudaFuncSetAttribute(hps_scale_round_to_q, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_r);
    const bool tc = c.tc_on && c.tc_hps_ok;
    if (tc) {
        hps_conv_tc(c, true, ea + qps, qrps, ct1, qps, 2, s);
    } else {
        count_launch();
        launch_pdl(c.pdl, hps_bconv, dim3(g), dim3(256), sm_q, s, ea + qps, qrps, ct1, qps, mods, 0, nQ, rbase, nR, c.hps_q_hat_inv.as<uint64_t>(), c.hps_q_inv.as<double>(), c.hps_q2r_mat.as<uint64_t>(), c.hps_q2r_alpha.as<uint64_t>(), c.log_n);
    }
    const uint64_t *ebp = ea;
    if (!square) {
        cudaMemcpy2DAsync(eb, qrps * 8, ct2, qps * 8, qps * 8, 2, cudaMemcpyDeviceToDevice, s);
        if (tc) {
            hps_conv_tc(c, true, eb + qps, qrps, ct2, qps, 2, s);
        } else {
            count_launch();
            launch_pdl(c.pdl, hps_bconv, dim3(g), dim3(256), sm_q, s, eb + qps, qrps, ct2, qps, mods, 0, nQ, rbase, nR, c.hps_q_hat_inv.as<uint64_t>(), c.hps_q_inv.as<double>(), c.hps_q2r_mat.as<uint64_t>(), c.hps_q2r_alpha.as<uint64_t>(), c.log_n);
        }
        ebp = eb;
    }
    // 2. NTT over QR, tensor (inside the inverse NTT's load), inverse NTT
    QrMap qm{qr, nQ, c.nP};
    PtrStore es{ea, qrps, c.log_n};
    ntt_fwd(c, (square ? 2 : 4) * qr, qm, PtrLoad{ea, qrps, c.log_n}, es, es, s);
    PtrStore t3s{t3, qrps, c.log_n};
    ntt_inv(c, 3 * qr, qm, TensorQrLoad{ea, ebp, qrps, mods, c.log_n}, t3s, t3s, s);
    // 3. scale and round to R, then back to Q
    if (tc) {
        // rt [3][nR][N] goes to ea (free once the tensor has been transformed)
        const long long rps = (long long)nR * n;
        HpsTcArgs a{};
        a.out = ea;
        a.ops = rps;
        a.in = t3;
        a.ips = qrps;
        a.mods = mods;
        a.in_tbl0 = 0;
        a.in_tbl_r = rbase;
        a.ni = nQ;
        a.nr = nR;
        a.out_tbl0 = rbase;
        a.no = nR;
        a.dinv = c.hps_frac.as<double>();
        a.bmat = c.tc_hps_scale.as<uint16_t>();
        a.kp = c.tc_hps_kp_scale;
        a.polys = 3;
        a.log_n = c.log_n;
        a.status = c.d_status.as<unsigned>();
        hps_tc_launch<kHpsScale>(c, a, s);
        hps_conv_tc(c, false, o3, qps, ea, rps, 3, s);
    } else {
        dim3 g3((unsigned)(n / kHpsTile), 3);
        count_launch();
        launch_pdl(c.pdl, hps_scale_round_to_q, dim3(g3), dim3(256), sm_r, s, o3, qps, t3, qrps, mods, nQ, rbase, nR, c.hps_frac.as<double>(), c.hps_modr.as<uint64_t>(), c.hps_r_hat_inv.as<uint64_t>(), c.hps_r_inv.as<double>(), c.hps_r2q_mat.as<uint64_t>(), c.hps_r2q_alpha.as<uint64_t>(), c.log_n);
    }
    // 4. relinearise c2 into (c0, c1), written to ct1
    bfv_keyswitch_to(c, ks, ct1, o3, o3 + 2 * qps, nQ, rlk, s);
}

__global__ void divide_round_q_last(uint64_t *out, const uint64_t *in, const uint64_t *iq, const Mod *mods, int l,
                                    int log_n, size_t total) {
    pdl_wait();
    pdl_release();
    const uint32_t nmask = (1u << log_n) - 1;
    const size_t lo = (size_t)(l - 1) << log_n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t p = e / lo, r = e - p * lo;
        const int j = (int)(r >> log_n);
        const uint32_t idx = (uint32_t)r & nmask;
        const Mod m = mods[j];
        const uint64_t *ci = in + p * ((size_t)l << log_n);
        const uint64_t last = reduce64(ci[lo + idx], m);
        out[e] = mul_shoup(sub_mod(ci[r], last, m.q), iq[2 * j], iq[2 * j + 1], m.q);
    }
}

void bfv_divide_round_q_last(const Context &c, const uint64_t *in, uint64_t *out, int size, int l, cudaStream_t s) {
    const size_t total = (size_t)size * ((size_t)(l - 1) << c.log_n);
    count_launch();
    launch_pdl(c.pdl, divide_round_q_last, dim3(grid_for_bfv(total, 256)), dim3(256), 0, s, out, in, c.levels[l]->inv_qlast.as<uint64_t>(), c.d_mods.as<Mod>(), l, c.log_n, total);
}

}  // namespace pfg
