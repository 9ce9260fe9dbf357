// hps_tc.cuh — BFV HPS contractions on the tensor cores (tcgen05), word for word equal to the
// CUDA-core kernels of ops_bfv.cu and to the reference's
//   DBaseConverter::bConv_HPS      src/rns_bconv.cu:354-372 (kernel :277-310)
//   scaleAndRound_HPS_QR_R         src/rns.cu:1700-1747
// through the byte-plane GEMM of tc.cuh (exact: at most 258 nonzero byte products per plane
// sum, checked when the operands are built).
//
// kHpsConv:  out_j = sum_i y_i M_ji - v (Q mod p_j),  y_i = x_i hatinv_i mod q_i,
//            v = llround(sum_i fma(y_i, 1/q_i)) in the reference's loop order (FP64, one thread
//            per coefficient); v rides in the GEMM as one more input slot whose constant is
//            -Q mod p_j.  Outputs canonical.
// kHpsScale: rt_j = (sum_i x_i modr_ji + x_(R_j) modr_j,nQ) + alpha_j mod r_j for the R limbs,
//            alpha from nu = 0.5 + sum_i fma(x_i, frac_i) (FP64) reduced in place across
//            r_0 .. r_j as the reference does; the R -> Q conversion of rt * rhatinv then runs as
//            kHpsConv.
//
// Tiles of 128 coefficients of one polynomial; per tile the CTA stages the inputs in shared
// memory, computes the FP64 terms (thread per coefficient), writes the byte-plane rows of A,
// issues ceil(K / 16) MMAs from one thread into 256 tensor-memory columns and runs the epilogue
// with 8 warps (lane quarter x half of the outputs).  Bounded wait on the MMA barrier.
#pragma once
#include "pdl.cuh"
#include "tc.cuh"

namespace pfg {

enum { kHpsConv = 0, kHpsScale = 1 };

struct HpsTcArgs {
    uint64_t *out;
    long long ops;        // output polynomial stride (words)
    const uint64_t *in;
    long long ips;        // input polynomial stride
    const Mod *mods;
    int in_tbl0;          // modulus table index of input slot 0 (conv); scale: Q limbs at 0
    int in_tbl_r;         // scale: table index of R limb 0
    int ni, nr;           // conv: ni inputs; scale: ni = nQ, nr = nR
    int out_tbl0, no;     // outputs
    const uint64_t *hat_inv;  // conv: (value, Shoup) per input
    const double *dinv;       // conv: 1 / q_i; scale: frac_i
    const uint16_t *bmat;
    int kp;               // K of the GEMM (multiple of 16)
    int polys, log_n;
    unsigned *status;
};

template <int MODE>
__global__ void __launch_bounds__(256, 1) hps_tc_kernel(HpsTcArgs a) {
    pdl_wait();
    pdl_release();
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_slot, ok_flag;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint64_t s_p[tc::kMaxOut];
    __shared__ float s_inv[tc::kMaxOut];
    __shared__ uint64_t s_v[tc::kRows];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int kp = a.kp, kslots = kp / 8, ksteps = kp / 16;
    const uint32_t sbo = (uint32_t)kslots * 128;
    const int nin = MODE == kHpsConv ? a.ni : a.ni + a.nr;
    const int ncols = (a.no * 8 + 15) & ~15;
    uint8_t *sA = smem;                                     // 128 x kp bf16
    uint8_t *sB = sA + tc::kRows * kp * 2;                  // ncols x kp bf16
    uint64_t *xs = reinterpret_cast<uint64_t *>(sB + ncols * kp * 2);  // [nin][128]
    uint64_t *as = xs + (size_t)nin * tc::kRows;            // scale: [nr][128] carries

    const uint4 *bs = reinterpret_cast<const uint4 *>(a.bmat);
    for (int i = tid; i < ncols * kp * 2 / 16; i += 256) reinterpret_cast<uint4 *>(sB)[i] = bs[i];
    if (tid < a.no) {
        const uint64_t p = a.mods[a.out_tbl0 + tid].q;
        s_p[tid] = p;
        s_inv[tid] = (float)(1.0 / (double)p);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, tc::kTmemCols);
    if (tid == 0) tc::mbar_init(&bar, 1);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(tc::kRows, ncols);
    const int tshift = a.log_n - 7, tiles = 1 << tshift, units = a.polys << tshift;
    const int lq = warp & 3, half = warp >> 2, row = lq * 32 + lane;
    const int o0 = half ? a.no / 2 : 0, o1 = half ? a.no : a.no / 2;
    const uint32_t trow = tmem + ((uint32_t)(lq * 32) << 16);
    uint32_t phase = 0;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int poly = unit >> tshift;
        const size_t n0 = (size_t)(unit & (tiles - 1)) * tc::kRows;
        const uint64_t *in = a.in + poly * a.ips + n0;
        // 1. stage the inputs (conv: scaled by hatinv)
        for (int p = tid; p < nin * tc::kRows; p += 256) {
            const int i = p / tc::kRows, r = p % tc::kRows;
            uint64_t x = in[((size_t)i << a.log_n) + r];
            if constexpr (MODE == kHpsConv) {
                const uint64_t q = a.mods[a.in_tbl0 + i].q;
                x = mul_shoup(x, a.hat_inv[2 * i], a.hat_inv[2 * i + 1], q);
            }
            xs[p] = x;
        }
        __syncthreads();
        // 2. FP64 terms, one thread per coefficient, in the reference's order
        if (tid < tc::kRows) {
            if constexpr (MODE == kHpsConv) {
                double acc = 0.0;
                for (int i = 0; i < a.ni; i++) acc = __fma_rn(__ull2double_rn(xs[i * tc::kRows + tid]), a.dinv[i], acc);
                s_v[tid] = (uint64_t)llround(acc);
            } else {
                double nu = 0.5;
                for (int i = 0; i < a.ni; i++) nu = __fma_rn(__ull2double_rn(xs[i * tc::kRows + tid]), a.dinv[i], nu);
                uint64_t alpha = __double2ull_rz(nu);
                for (int j = 0; j < a.nr; j++) {
                    alpha = reduce64(alpha, a.mods[a.in_tbl_r + j]);
                    as[j * tc::kRows + tid] = alpha;
                }
            }
        }
        __syncthreads();
        // 3. byte-plane rows of A (slots past the inputs are zero)
        for (int p = tid; p < kslots * tc::kRows; p += 256) {
            const int sl = p / tc::kRows, r = p % tc::kRows;
            uint64_t v = 0;
            if (sl < nin) v = xs[sl * tc::kRows + r];
            else if (MODE == kHpsConv && sl == nin) v = s_v[r];
            *reinterpret_cast<uint4 *>(sA + (r & 7) * 16 + (r >> 3) * sbo + sl * 128) = tc::bytes_bf16(v);
        }
        tc::fence_smem_async();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            for (int k = 0; k < ksteps; k++)
                tc::mma_bf16(tmem, tc::sdesc(tc::saddr(sA) + k * 256, 128, sbo),
                             tc::sdesc(tc::saddr(sB) + k * 256, 128, sbo), idesc, k > 0);
            tc::commit(&bar);
            ok_flag = tc::mbar_wait(&bar, phase) ? 1u : 0u;
        }
        __syncthreads();
        if (!ok_flag) {
            if (tid == 0) atomicOr(a.status, 4u);
            break;
        }
        phase ^= 1;
        tc::fence_after();
        // 4. epilogue: canonical residues (scale: plus the carry)
        uint64_t *dst = a.out + poly * a.ops + n0 + row;
        for (int o = o0; o < o1; o++) {
            uint32_t x[8];
            tc::ld8(trow + o * 8, x);
            tc::wait_ld();
            const uint64_t p = s_p[o];
            uint64_t v = csub(tc::reduce_planes_lazy<8>(x, p, s_inv[o]), p);
            if constexpr (MODE == kHpsScale) v = add_mod(v, as[o * tc::kRows + row], p);
            dst[(size_t)o << a.log_n] = v;
        }
        tc::fence_before();
        __syncthreads();
    }
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_free(tmem, tc::kTmemCols);
    }
}

inline size_t hps_tc_smem(const HpsTcArgs &a, int mode) {
    const int nin = mode == kHpsConv ? a.ni : a.ni + a.nr;
    const int ncols = (a.no * 8 + 15) & ~15;
    return (size_t)tc::kRows * a.kp * 2 + (size_t)ncols * a.kp * 2 + (size_t)nin * tc::kRows * 8 +
           (mode == kHpsScale ? (size_t)a.nr * tc::kRows * 8 : 0);
}

}  // namespace pfg
