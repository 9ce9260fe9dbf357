// ckks_codec.cu — CKKS encoding and decoding on the GPU with the reference's FP64 arithmetic.
//
// Restates PhantomCKKSEncoder (src/ckks.cu:17-140 encode, :340-400 decode), its special FFT
// (src/fft.cu:43-459) and the RNS decompose / compose of the plaintext's coefficients
// (src/rns_base.cu:49-253):
//   encode: slots -> bit-reversed order -> inverse special FFT (Gentleman-Sande butterflies with
//           conjugate twiddles, the last stage scaled by scale / slots) -> coefficient c_k = round(
//           Re z_k) for k < N/2, round(Im z_{k - N/2}) above -> residues mod q_i -> forward NTT;
//   decode: inverse NTT -> CRT compose of every coefficient into a multi-word integer mod Q_l,
//           centred and scaled by 1 / scale in FP64 -> forward special FFT -> bit-reversed order.
// Every butterfly, scale and accumulation is the reference's own FP64 operation in its order and
// in the contraction its compiled kernels use (written out with explicit round-to-nearest
// intrinsics; the same twiddle table), so encoded words and decoded slots equal the reference's
// bit for bit.  The integer parts are exact: a coefficient's residue
// is its exact value mod q_i (any magnitude a double holds), and negative values map to
// q_i - (|c| mod q_i) as the reference does (which gives q_i, not 0, for a multiple of q_i; the
// forward NTT takes it as a lazy input and returns the canonical transform).
#include <cuComplex.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>

#include "capi_internal.hpp"
#include "host_tables.hpp"
#include "launch.cuh"
#include "ops.hpp"

namespace pfg {

namespace {

constexpr int kCodecBlock = 256;
constexpr int kMaxComposeLimbs = 64;

__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int bits) { return __brev(x) >> (32 - bits); }

// dst[bitrev(i)] = src[i] for i < count (src/ckks.cu:9-15)
__global__ void codec_bitrev(cuDoubleComplex *dst, const cuDoubleComplex *src, uint32_t count, int log_slots) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        dst[brev_bits(i, log_slots)] = src[i];
}

// Complex product a * b with every FP64 operation written out, so that no compiler contraction
// can change a rounding.  Real part: form 0 fma(a.x, b.x, -(a.y b.y)), form 1 fma(-a.y, b.y,
// a.x b.x), form 2 a.x b.x - a.y b.y; imaginary part: form 0 fma(a.x, b.y, a.y b.x), form 1
// fma(a.y, b.x, a.x b.y), form 2 a.x b.y + a.y b.x (each product rounded where it is not fused).
template <int RE, int IM>
__device__ __forceinline__ cuDoubleComplex cmul_form(cuDoubleComplex a, cuDoubleComplex b) {
    double re, im;
    if constexpr (RE == 0)
        re = __fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y));
    else if constexpr (RE == 1)
        re = __fma_rn(-a.y, b.y, __dmul_rn(a.x, b.x));
    else
        re = __dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y));
    if constexpr (IM == 0)
        im = __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x));
    else if constexpr (IM == 1)
        im = __fma_rn(a.y, b.x, __dmul_rn(a.x, b.y));
    else
        im = __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x));
    return make_cuDoubleComplex(re, im);
}

// The reference runs its special FFT as two kernels (src/fft.cu:90-340): stages of a block of up
// to 2048 slots in shared memory (`base`) and, above 2048 slots, single global stages (`iter`).
// Compiled separately, the two evaluate the complex product of a butterfly with different FMA
// contractions, and the decoded doubles carry that difference.  Each form below is the one
// measured on the reference's compiled kernels (the same butterfly on seeded inputs, compared
// with exact evaluations of every candidate), and each stage here uses the form of the kernel
// that runs that stage in the reference.
constexpr int kFftBaseRe = 0, kFftBaseIm = 1;
constexpr int kFftIterRe = 0, kFftIterIm = 0;
constexpr int kIfftBaseRe = 0, kIfftBaseIm = 1;
constexpr int kIfftIterRe = 0, kIfftIterIm = 0;
constexpr int kFftBlockLog = 11;  // slots handled by the reference's shared-memory kernel: 2^11

// One stage `iter` of the special FFT over `slots` values (slots / 2 butterflies).  Butterfly
// tid pairs g = 2 k 2^lp + j and g + 2^lp (lp = log_slots - iter - 1, k = tid >> lp, j = tid mod
// 2^lp); its twiddle index is 5^r 2^lp mod 2N with r the bit-reversed k << lp (src/fft.cu:106-126).
// Forward (decode): Cooley-Tukey, x0 + w x1, x0 - w x1 with w = roots[idx].  Inverse (encode):
// Gentleman-Sande, x0 + x1, (x0 - x1) w with w = roots[2N - idx]; the last stage (iter 0)
// multiplies both outputs by `scalar` when it is nonzero (src/fft.cu:209-277).
template <bool FWD, int RE, int IM>
__global__ void codec_fft_stage(cuDoubleComplex *x, const cuDoubleComplex *roots, const uint32_t *group,
                                uint32_t slots, int log_slots, int iter, uint32_t m, double scalar) {
    const int lp = log_slots - iter - 1;
    const uint32_t pairs = 1u << lp;
    for (uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x; tid < (slots >> 1); tid += gridDim.x * blockDim.x) {
        const uint32_t k = tid >> lp, j = tid & (pairs - 1);
        const uint32_t g = 2 * k * pairs + j;
        uint32_t psi = group[__brev(k << lp) >> (33 - log_slots)];
        psi = (psi << lp) & (m - 1);
        const cuDoubleComplex x0 = x[g], x1 = x[g + pairs];
        if constexpr (FWD) {
            const cuDoubleComplex s1 = cmul_form<RE, IM>(x1, roots[psi]);
            x[g] = make_cuDoubleComplex(__dadd_rn(x0.x, s1.x), __dadd_rn(x0.y, s1.y));
            x[g + pairs] = make_cuDoubleComplex(__dsub_rn(x0.x, s1.x), __dsub_rn(x0.y, s1.y));
        } else {
            cuDoubleComplex y0 = make_cuDoubleComplex(__dadd_rn(x0.x, x1.x), __dadd_rn(x0.y, x1.y));
            cuDoubleComplex y1 = cmul_form<RE, IM>(make_cuDoubleComplex(__dsub_rn(x0.x, x1.x), __dsub_rn(x0.y, x1.y)),
                                                   roots[m - psi]);
            if (iter == 0 && scalar != 0.0) {
                y0 = make_cuDoubleComplex(__dmul_rn(y0.x, scalar), __dmul_rn(y0.y, scalar));
                y1 = make_cuDoubleComplex(__dmul_rn(y1.x, scalar), __dmul_rn(y1.y, scalar));
            }
            x[g] = y0;
            x[g + pairs] = y1;
        }
    }
}

// *out = max over the slots of |re| and |im| (non-negative doubles order as their bit patterns)
__global__ void codec_max_abs(const cuDoubleComplex *x, uint32_t slots, unsigned long long *out) {
    double mx = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x)
        mx = fmax(mx, fmax(fabs(x[i].x), fabs(x[i].y)));
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

__device__ __forceinline__ uint64_t mulmod_dev(uint64_t a, uint64_t b, const Mod &m) { return mul_mod(a, b, m); }

// 2^e mod q by square-and-multiply
__device__ uint64_t pow2_mod(int e, const Mod &m) {
    uint64_t r = 1 % m.q, b = 2 % m.q;
    while (e) {
        if (e & 1) r = mulmod_dev(r, b, m);
        b = mulmod_dev(b, b, m);
        e >>= 1;
    }
    return r;
}

// pt[i][c] = round(coefficient c) mod q_i (src/rns_base.cu:49-163): the magnitude m 2^e (m the
// 53-bit significand) reduced exactly, negatives as q_i - r.
__global__ void codec_decompose(uint64_t *pt, const cuDoubleComplex *x, const Mod *mods, int l, int log_n) {
    const uint32_t n = 1u << log_n, slots = n >> 1;
    const size_t total = (size_t)l << log_n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t >> log_n);
        const uint32_t c = (uint32_t)t & (n - 1);
        const double cd = round(c < slots ? x[c].x : x[c - slots].y);
        const bool neg = signbit(cd);
        const double a = fabs(cd);
        const Mod md = mods[i];
        uint64_t r = 0;
        if (a < 18446744073709551616.0) {
            r = reduce64((uint64_t)a, md);
        } else {
            int e = 0;
            const double f = frexp(a, &e);             // a = f 2^e, f in [0.5, 1)
            const uint64_t sig = (uint64_t)ldexp(f, 53);  // exact: a has at most 53 significant bits
            r = mulmod_dev(reduce64(sig, md), pow2_mod(e - 53, md), md);
        }
        pt[t] = neg ? md.q - r : r;
    }
}

// Exact CRT compose of one coefficient into acc (l words, < Q_l), then the reference's FP64
// centring and scaling (src/rns_base.cu:169-253): upper half -> sum of +-|acc_i - Q_i| 2^(64 i),
// lower half -> sum of acc_i 2^(64 i), each term times inv_scale 2^(64 i), accumulated from word 0.
__global__ void codec_compose(cuDoubleComplex *x, const uint64_t *src, const Mod *mods, const uint64_t *q_prod,
                              const uint64_t *q_hat, const uint64_t *q_hat_inv, const uint64_t *upper, int l,
                              int log_n, double inv_scale) {
    const uint32_t n = 1u << log_n, slots = n >> 1;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        uint64_t acc[kMaxComposeLimbs];
        if (l > 1) {
            for (int w = 0; w < l; w++) acc[w] = 0;
            for (int i = 0; i < l; i++) {
                const uint64_t q = mods[i].q;
                const uint64_t p = mul_shoup(src[((size_t)i << log_n) + c], q_hat_inv[2 * i], q_hat_inv[2 * i + 1], q);
                // acc = (acc + (Q / q_i) p) mod Q; (Q / q_i) p < Q, so one subtraction suffices
                const uint64_t *h = q_hat + (size_t)i * l;
                uint64_t mc = 0, ac = 0;
                for (int w = 0; w < l; w++) {
                    const unsigned __int128 pr = (unsigned __int128)h[w] * p + mc;
                    mc = (uint64_t)(pr >> 64);
                    const unsigned __int128 s = (unsigned __int128)acc[w] + (uint64_t)pr + ac;
                    acc[w] = (uint64_t)s;
                    ac = (uint64_t)(s >> 64);
                }
                bool ge = ac != 0;
                if (!ge) {
                    ge = true;
                    for (int w = l - 1; w >= 0; w--)
                        if (acc[w] != q_prod[w]) {
                            ge = acc[w] > q_prod[w];
                            break;
                        }
                }
                if (ge) {
                    uint64_t br = 0;
                    for (int w = 0; w < l; w++) {
                        const uint64_t a = acc[w], b = q_prod[w];
                        acc[w] = a - b - br;
                        br = (a < b) || (a - b < br);
                    }
                }
            }
        } else {
            acc[0] = src[c];
        }
        bool upper_half = true;
        for (int w = l - 1; w >= 0; w--)
            if (acc[w] != upper[w]) {
                upper_half = acc[w] > upper[w];
                break;
            }
        // each term rounded on its own, then added (the reference's compiled form: no fused
        // multiply-add here, measured with a scale that is not a power of two)
        double res = 0.0, scaled = inv_scale;
        if (upper_half) {
            for (int w = 0; w < l; w++, scaled = __dmul_rn(scaled, 18446744073709551616.0)) {
                if (acc[w] > q_prod[w]) {
                    const uint64_t diff = acc[w] - q_prod[w];
                    res = __dadd_rn(res, diff ? __dmul_rn(static_cast<double>(diff), scaled) : 0.0);
                } else {
                    const uint64_t diff = q_prod[w] - acc[w];
                    res = __dsub_rn(res, diff ? __dmul_rn(static_cast<double>(diff), scaled) : 0.0);
                }
            }
        } else {
            for (int w = 0; w < l; w++, scaled = __dmul_rn(scaled, 18446744073709551616.0)) {
                const uint64_t diff = acc[w];
                res = __dadd_rn(res, diff ? __dmul_rn(static_cast<double>(diff), scaled) : 0.0);
            }
        }
        if (c < slots)
            x[c].x = res;
        else
            x[c - slots].y = res;
    }
}

int codec_grid(size_t work) {
    return (int)std::min<size_t>((work + kCodecBlock - 1) / kCodecBlock, (size_t)kGridStrideBlocks);
}

void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void fft_stages(const Context &c, cuDoubleComplex *x, bool fwd, double scalar, cudaStream_t s) {
    const int log_slots = c.log_n - 1;
    const uint32_t slots = 1u << log_slots, m = (uint32_t)(2 * c.n);
    const auto *roots = c.codec_roots.as<cuDoubleComplex>();
    const auto *group = c.codec_group.as<uint32_t>();
    const int g = codec_grid(slots / 2);
    // stages iter < log_slots - 11 run in the reference's global-stage kernels, the rest in its
    // shared-memory kernels (src/fft.cu:340-413)
    const int split = log_slots - kFftBlockLog;
    for (int k = 0; k < log_slots; k++) {
        count_launch();
        if (fwd) {
            if (k < split)
                codec_fft_stage<true, kFftIterRe, kFftIterIm><<<g, kCodecBlock, 0, s>>>(x, roots, group, slots,
                                                                                       log_slots, k, m, 0.0);
            else
                codec_fft_stage<true, kFftBaseRe, kFftBaseIm><<<g, kCodecBlock, 0, s>>>(x, roots, group, slots,
                                                                                       log_slots, k, m, 0.0);
        } else {
            const int it = log_slots - 1 - k;
            if (it < split)
                codec_fft_stage<false, kIfftIterRe, kIfftIterIm><<<g, kCodecBlock, 0, s>>>(x, roots, group, slots,
                                                                                          log_slots, it, m, scalar);
            else
                codec_fft_stage<false, kIfftBaseRe, kIfftBaseIm><<<g, kCodecBlock, 0, s>>>(x, roots, group, slots,
                                                                                          log_slots, it, m, scalar);
        }
    }
}

}  // namespace

// Host tables: the reference's ComplexRoots (src/fft.cu:12-41: polar(1, 2 pi i / m) for i <= m/8,
// the other roots by its 8-fold symmetry), its rotation group 5^i mod 2N (src/ckks.cu:36-46) and
// per data level the compose constants of base Q_l (src/rns_base.cu:11-47).
void build_codec_tables(Context &c) {
    const uint64_t n = c.n, m = 2 * n;
    const double pi = 3.1415926535897932384626433832795028842;
    std::vector<double> base(2 * (m / 8 + 1));
    for (uint64_t i = 0; i <= m / 8; i++) {
        const double th = 2 * pi * static_cast<double>(i) / static_cast<double>(m);
        base[2 * i] = std::cos(th);
        base[2 * i + 1] = std::sin(th);
    }
    // get_root(i), with the reference's operations: mirror swaps the parts, the negation is
    // 0 - z (cuCsub from zero) and the conjugate flips the sign of the imaginary part
    struct Cplx {
        double x, y;
    };
    std::function<Cplx(uint64_t)> get_root = [&](uint64_t i) -> Cplx {
        i &= m - 1;
        if (i <= m / 8) return {base[2 * i], base[2 * i + 1]};
        if (i <= m / 4) return {base[2 * (m / 4 - i) + 1], base[2 * (m / 4 - i)]};
        if (i <= m / 2) {
            const Cplx r = get_root(m / 2 - i);
            return {0.0 - r.x, 0.0 - (-r.y)};
        }
        if (i <= 3 * m / 4) {
            const Cplx r = get_root(i - m / 2);
            return {0.0 - r.x, 0.0 - r.y};
        }
        const Cplx r = get_root(m - i);
        return {r.x, -r.y};
    };
    std::vector<double> roots(2 * m);
    for (uint64_t i = 0; i < m; i++) {
        const Cplx r = get_root(i);
        roots[2 * i] = r.x;
        roots[2 * i + 1] = r.y;
    }
    c.codec_roots.upload(roots.data(), roots.size() * sizeof(double));
    std::vector<uint32_t> group(n / 4);
    uint64_t pos = 1;
    for (uint64_t i = 0; i < n / 4; i++) {
        group[i] = (uint32_t)pos;
        pos = (pos * 5) & (m - 1);
    }
    c.codec_group.upload(group.data(), group.size() * sizeof(uint32_t));

    c.compose.clear();
    c.compose.resize(c.nQ + 1);
    for (int l = 1; l <= c.nQ; l++) {
        auto t = std::make_unique<ComposeTables>();
        // Q_l and Q_l / q_i as little-endian words
        auto mul_word = [](std::vector<uint64_t> &a, uint64_t b) {
            unsigned __int128 carry = 0;
            for (auto &w : a) {
                const unsigned __int128 p = (unsigned __int128)w * b + carry;
                w = (uint64_t)p;
                carry = p >> 64;
            }
        };
        std::vector<uint64_t> prod(l, 0);
        prod[0] = 1;
        for (int i = 0; i < l; i++) mul_word(prod, c.mods[i]);
        std::vector<uint64_t> hat((size_t)l * l), hinv(2 * l);
        for (int i = 0; i < l; i++) {
            std::vector<uint64_t> h(l, 0);
            h[0] = 1;
            uint64_t hm = 1 % c.mods[i];
            for (int j = 0; j < l; j++)
                if (j != i) {
                    mul_word(h, c.mods[j]);
                    hm = host::mulmod(hm, c.mods[j] % c.mods[i], c.mods[i]);
                }
            std::copy(h.begin(), h.end(), hat.begin() + (size_t)i * l);
            hinv[2 * i] = host::invmod(hm, c.mods[i]);
            hinv[2 * i + 1] = host::shoup(hinv[2 * i], c.mods[i]);
        }
        // (Q + 1) / 2
        std::vector<uint64_t> up(prod);
        for (int w = 0; w < l; w++)
            if (++up[w]) break;
        for (int w = 0; w < l; w++) up[w] = (up[w] >> 1) | (w + 1 < l ? up[w + 1] << 63 : 0);
        int bits = 0;
        for (int w = l - 1; w >= 0; w--)
            if (prod[w]) {
                bits = 64 * w + 64 - __builtin_clzll(prod[w]);
                break;
            }
        t->bits = bits;
        t->q_prod.upload(prod.data(), prod.size() * 8);
        t->q_hat.upload(hat.data(), hat.size() * 8);
        t->q_hat_inv.upload(hinv.data(), hinv.size() * 8);
        t->upper.upload(up.data(), up.size() * 8);
        c.compose[l] = std::move(t);
    }
}

size_t codec_encode_words(const Context &c) { return c.n + 8; }
size_t codec_decode_words(const Context &c, int l) { return ((size_t)l + 1) * c.n; }

// values: `count` complex doubles (device); pt [l][N] in NTT form.
void ckks_encode(const Context &c, const Workspace &w, const double *values, size_t count, double scale, int l,
                 uint64_t *pt, cudaStream_t s) {
    const ComposeTables &ct = *c.compose[l];
    const uint32_t slots = (uint32_t)(c.n / 2);
    const int log_slots = c.log_n - 1;
    if (count == 0) throw std::invalid_argument("Input vector is empty");
    if (count > slots) throw std::invalid_argument("Input vector exceeds max slots");
    if (!(scale > 0) || (static_cast<int>(std::log2(scale)) + 1 >= ct.bits))
        throw std::invalid_argument("scale out of bounds");
    if (w.words < codec_encode_words(c)) throw std::logic_error("workspace too small for encoding");
    auto *x = reinterpret_cast<cuDoubleComplex *>(w.base);
    auto *mx = reinterpret_cast<unsigned long long *>(w.base + c.n);
    check_cuda(cudaMemsetAsync(x, 0, slots * sizeof(cuDoubleComplex), s), "cudaMemsetAsync");
    check_cuda(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), s), "cudaMemsetAsync");
    count_launch();
    codec_bitrev<<<codec_grid(count), kCodecBlock, 0, s>>>(x, reinterpret_cast<const cuDoubleComplex *>(values),
                                                           (uint32_t)count, log_slots);
    fft_stages(c, x, false, scale / static_cast<double>(slots), s);
    count_launch();
    codec_max_abs<<<codec_grid(slots), kCodecBlock, 0, s>>>(x, slots, mx);
    unsigned long long bits = 0;
    check_cuda(cudaMemcpyAsync(&bits, mx, sizeof(bits), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    double max_coeff;
    std::memcpy(&max_coeff, &bits, sizeof(max_coeff));
    // bit count of the largest coefficient plus a sign bit (src/ckks.cu:104-118)
    const int max_bits = static_cast<int>(std::ceil(std::log2(std::max(max_coeff, 1.0)))) + 1;
    if (!(max_bits < ct.bits)) throw std::invalid_argument("encoded values are too large");
    count_launch();
    codec_decompose<<<codec_grid((size_t)l << c.log_n), kCodecBlock, 0, s>>>(pt, x, c.d_mods.as<Mod>(), l, c.log_n);
    ntt_forward(c, pt, 1, l, 0, s);
}

// pt [l][N] (NTT form) -> values: N/2 complex doubles (device).
void ckks_decode(const Context &c, const Workspace &w, const uint64_t *pt, double scale, int l, double *values,
                 cudaStream_t s) {
    const ComposeTables &ct = *c.compose[l];
    const uint32_t slots = (uint32_t)(c.n / 2);
    if (!(scale > 0) || static_cast<int>(std::log2(scale)) >= ct.bits) throw std::invalid_argument("scale out of bounds");
    if (l > kMaxComposeLimbs) throw std::invalid_argument("too many limbs to compose");
    if (w.words < codec_decode_words(c, l)) throw std::logic_error("workspace too small for decoding");
    uint64_t *copy = w.base;
    auto *x = reinterpret_cast<cuDoubleComplex *>(w.base + ((size_t)l << c.log_n));
    check_cuda(cudaMemcpyAsync(copy, pt, ((size_t)l << c.log_n) * 8, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
    ntt_inverse(c, copy, 1, l, 0, s);
    count_launch();
    codec_compose<<<codec_grid(c.n), kCodecBlock, 0, s>>>(x, copy, c.d_mods.as<Mod>(), ct.q_prod.as<uint64_t>(),
                                                          ct.q_hat.as<uint64_t>(), ct.q_hat_inv.as<uint64_t>(),
                                                          ct.upper.as<uint64_t>(), l, c.log_n, 1.0 / scale);
    fft_stages(c, x, true, 0.0, s);
    count_launch();
    codec_bitrev<<<codec_grid(slots), kCodecBlock, 0, s>>>(reinterpret_cast<cuDoubleComplex *>(values), x, slots,
                                                           c.log_n - 1);
}

}  // namespace pfg
