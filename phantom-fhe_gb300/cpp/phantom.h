// phantom.h — C++ compatibility layer: PhantomFHE's hot-path API on top of the GB300 C ABI.
//
// Source-compatible subset of the reference's public surface (include/phantom.h):
//   phantom::scheme_type / mul_tech_type / EncryptionParameters   (include/host/encryptionparams.h:12-246)
//   phantom::arith::Modulus, phantom::arith::CoeffModulus::Create   (include/host/modulus.h:14-317)
//   PhantomContext                                                  (include/context.cuh:153-273)
//   PhantomCiphertext with the same save/load byte format           (include/ciphertext.h:7-308)
//   PhantomRelinKey / PhantomGaloisKey load/save, public_keys_ptr()  (include/secretkey.h:102-219)
//   phantom:: multiply_inplace, multiply_and_relin_inplace, relinearize_inplace, rescale_to_next(_inplace),
//   mod_switch_to_next_inplace, apply_galois_inplace, rotate_inplace, hoisting_inplace, keyswitch_inplace,
//   multiply_plain(_inplace), add(_inplace)                         (include/evaluate.cuh:12-246)
//   PhantomPlaintext (CKKS, NTT form)                               (include/plaintext.h)
//   PhantomCKKSEncoder encode / decode                              (include/ckks.h:88-150)
//   PhantomSecretKey: gen_relinkey, create_galois_keys, encrypt_symmetric, decrypt (CKKS)
//                                                                   (include/secretkey.h:276-330)
// Randomness for keys and encryption comes from a host std::mt19937_64 (seeded from
// std::random_device unless a seed is given) instead of the reference's device Salsa20; the
// arithmetic runs on the GPU through the C ABI.
// Device memory is owned as in the reference: cudaMallocAsync / cudaFreeAsync on
// cudaStreamPerThread, and every evaluator call enqueues on cudaStreamPerThread.  Errors are
// thrown as std::invalid_argument / std::logic_error with the library's message.
// Header only: link against libphantom_gb300.so and the CUDA runtime.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <random>
#include <istream>
#include <map>
#include <memory>
#include <mutex>
#include <ostream>
#include <stdexcept>
#include <thread>
#include <utility>
#include <vector>

#include "phantom_gb300.h"

namespace phantom {

enum class scheme_type : std::uint8_t { none = 0, bgv = 1, bfv = 2, ckks = 3 };
enum class mul_tech_type : std::uint8_t { none = 0, behz = 1, hps = 2, hps_overq = 3, hps_overq_leveled = 4 };

namespace detail {
inline void check(int rc) {
    if (rc == FHE_OK) return;
    if (rc == FHE_ERR_INVALID_ARGUMENT) throw std::invalid_argument(fhe_last_error());
    if (rc == FHE_ERR_LOGIC || rc == FHE_ERR_UNSUPPORTED) throw std::logic_error(fhe_last_error());
    throw std::runtime_error(fhe_last_error());
}
inline void cuda_check(cudaError_t e) {
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}
}  // namespace detail

namespace arith {
class Modulus {
public:
    Modulus(std::uint64_t value = 0) : value_(value) {}
    [[nodiscard]] std::uint64_t value() const noexcept { return value_; }
    [[nodiscard]] bool is_zero() const noexcept { return value_ == 0; }

private:
    std::uint64_t value_;
};

struct CoeffModulus {
    static std::vector<Modulus> Create(std::size_t poly_modulus_degree, const std::vector<int> &bit_sizes) {
        std::vector<std::uint64_t> out(bit_sizes.size());
        detail::check(fhe_create_coeff_modulus(poly_modulus_degree, bit_sizes.data(), bit_sizes.size(), out.data()));
        return {out.begin(), out.end()};
    }
};
}  // namespace arith

class EncryptionParameters {
public:
    explicit EncryptionParameters(scheme_type scheme = scheme_type::none)
        : scheme_(scheme), mul_tech_(scheme == scheme_type::bfv ? mul_tech_type::hps : mul_tech_type::none) {}
    void set_poly_modulus_degree(std::size_t n) { n_ = n; }
    void set_coeff_modulus(const std::vector<arith::Modulus> &m) { coeff_modulus_ = m; }
    void set_special_modulus_size(std::size_t s) { special_ = s; }
    void set_plain_modulus(const arith::Modulus &t) { plain_ = t; }
    void set_galois_elts(const std::vector<std::uint32_t> &e) { galois_elts_ = e; }
    void set_mul_tech(mul_tech_type m) { mul_tech_ = m; }
    [[nodiscard]] scheme_type scheme() const noexcept { return scheme_; }
    [[nodiscard]] mul_tech_type mul_tech() const noexcept { return mul_tech_; }
    [[nodiscard]] std::size_t poly_modulus_degree() const noexcept { return n_; }
    [[nodiscard]] const std::vector<arith::Modulus> &coeff_modulus() const noexcept { return coeff_modulus_; }
    [[nodiscard]] std::size_t special_modulus_size() const noexcept { return special_; }
    [[nodiscard]] const arith::Modulus &plain_modulus() const noexcept { return plain_; }
    [[nodiscard]] const std::vector<std::uint32_t> &galois_elts() const noexcept { return galois_elts_; }

private:
    scheme_type scheme_;
    mul_tech_type mul_tech_;
    std::size_t n_ = 0, special_ = 1;
    std::vector<arith::Modulus> coeff_modulus_;
    arith::Modulus plain_;
    std::vector<std::uint32_t> galois_elts_;
};

namespace util {
inline std::uint32_t get_elt_from_step(int step, std::size_t coeff_count) {
    const std::uint32_t e = fhe_galois_elt_from_step(step, coeff_count);
    if (!e) throw std::invalid_argument(fhe_last_error());
    return e;
}
}  // namespace util
}  // namespace phantom

// Owning device buffer: cudaMallocAsync / cudaFreeAsync on cudaStreamPerThread, like the
// reference's cuda_auto_ptr (include/cuda_wrapper.cuh:66-190).
class PhantomDeviceBuffer {
public:
    PhantomDeviceBuffer() = default;
    explicit PhantomDeviceBuffer(std::size_t words) { reset(words); }
    PhantomDeviceBuffer(const PhantomDeviceBuffer &o) { copy_from(o); }
    PhantomDeviceBuffer &operator=(const PhantomDeviceBuffer &o) {
        if (this != &o) copy_from(o);
        return *this;
    }
    PhantomDeviceBuffer(PhantomDeviceBuffer &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
    PhantomDeviceBuffer &operator=(PhantomDeviceBuffer &&o) noexcept {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
        return *this;
    }
    ~PhantomDeviceBuffer() { release(); }
    void reset(std::size_t words) {
        release();
        if (words) phantom::detail::cuda_check(cudaMallocAsync(&p_, words * 8, cudaStreamPerThread));
        n_ = words;
    }
    [[nodiscard]] std::uint64_t *get() const noexcept { return p_; }
    [[nodiscard]] std::size_t size() const noexcept { return n_; }

private:
    void release() {
        if (p_) cudaFreeAsync(p_, cudaStreamPerThread);
        p_ = nullptr;
        n_ = 0;
    }
    void copy_from(const PhantomDeviceBuffer &o) {
        reset(o.n_);
        if (n_)
            phantom::detail::cuda_check(
                    cudaMemcpyAsync(p_, o.p_, n_ * 8, cudaMemcpyDeviceToDevice, cudaStreamPerThread));
    }
    std::uint64_t *p_ = nullptr;
    std::size_t n_ = 0;
};

class PhantomContext {
public:
    explicit PhantomContext(const phantom::EncryptionParameters &params) : params_(params) {
        std::vector<std::uint64_t> q;
        for (auto &m : params.coeff_modulus()) q.push_back(m.value());
        fhe_params p{static_cast<int>(params.scheme()), static_cast<int>(params.mul_tech()),
                     params.poly_modulus_degree(), q.data(), q.size(), params.special_modulus_size(),
                     params.plain_modulus().value(), params.galois_elts().data(), params.galois_elts().size()};
        phantom::detail::check(fhe_context_create(&p, &ctx_));
        size_t nq, np, nr, dnum;
        std::uint64_t n;
        phantom::detail::check(fhe_context_sizes(ctx_, &n, &nq, &np, &nr, &dnum));
        size_q_ = nq;
        size_p_ = np;
        moduli_.resize(nq + np + nr);
        phantom::detail::check(fhe_context_moduli(ctx_, moduli_.data()));
        size_t cnt = 0;
        phantom::detail::check(fhe_context_galois_elts(ctx_, nullptr, &cnt));
        galois_elts_.resize(cnt);
        phantom::detail::check(fhe_context_galois_elts(ctx_, galois_elts_.data(), &cnt));
    }
    PhantomContext(const PhantomContext &) = delete;
    PhantomContext &operator=(const PhantomContext &) = delete;
    ~PhantomContext() {
        for (auto &kv : ws_) fhe_workspace_destroy(kv.second);
        fhe_context_destroy(ctx_);
    }
    [[nodiscard]] const phantom::EncryptionParameters &parms() const noexcept { return params_; }
    [[nodiscard]] std::size_t get_first_index() const noexcept { return 1; }
    [[nodiscard]] std::size_t poly_modulus_degree() const noexcept { return params_.poly_modulus_degree(); }
    [[nodiscard]] std::size_t size_q() const noexcept { return size_q_; }
    [[nodiscard]] std::size_t size_p() const noexcept { return size_p_; }
    // data limbs at a chain index (src/context.cu:141-158)
    [[nodiscard]] std::size_t coeff_modulus_size(std::size_t chain_index) const {
        if (chain_index == 0) return size_q_ + size_p_;
        if (chain_index > size_q_) throw std::invalid_argument("chain_index out of range");
        return size_q_ - (chain_index - 1);
    }
    [[nodiscard]] std::uint64_t modulus(std::size_t i) const { return moduli_.at(i); }
    [[nodiscard]] const std::vector<std::uint32_t> &galois_elts() const noexcept { return galois_elts_; }
    [[nodiscard]] fhe_context *handle() const noexcept { return ctx_; }
    // One workspace per host thread (every call runs on that thread's cudaStreamPerThread).
    [[nodiscard]] fhe_workspace *workspace() const {
        std::lock_guard<std::mutex> g(mu_);
        auto &w = ws_[std::this_thread::get_id()];
        if (!w) phantom::detail::check(fhe_workspace_create(ctx_, &w));
        return w;
    }

private:
    phantom::EncryptionParameters params_;
    fhe_context *ctx_ = nullptr;
    std::size_t size_q_ = 0, size_p_ = 0;
    std::vector<std::uint64_t> moduli_;
    std::vector<std::uint32_t> galois_elts_;
    mutable std::mutex mu_;
    mutable std::map<std::thread::id, fhe_workspace *> ws_;
};

class PhantomCiphertext {
public:
    PhantomCiphertext() = default;

    // Reset to `size` polynomials at `chain_index` (keeps the leading words when it grows,
    // include/ciphertext.h:44-72).
    void resize(const PhantomContext &context, std::size_t chain_index, std::size_t size, const cudaStream_t & = cudaStreamPerThread) {
        const std::size_t limbs = context.coeff_modulus_size(chain_index), n = context.poly_modulus_degree();
        reshape(size, limbs, n);
        chain_index_ = chain_index;
    }
    void resize(std::size_t size, std::size_t coeff_modulus_size, std::size_t poly_modulus_degree,
                const cudaStream_t & = cudaStreamPerThread) {
        reshape(size, coeff_modulus_size, poly_modulus_degree);
    }
    [[nodiscard]] std::uint64_t *data() const noexcept { return data_.get(); }
    [[nodiscard]] std::size_t size() const noexcept { return size_; }
    [[nodiscard]] std::size_t chain_index() const noexcept { return chain_index_; }
    [[nodiscard]] std::size_t coeff_modulus_size() const noexcept { return coeff_modulus_size_; }
    [[nodiscard]] std::size_t poly_modulus_degree() const noexcept { return poly_modulus_degree_; }
    [[nodiscard]] double scale() const noexcept { return scale_; }
    [[nodiscard]] bool is_ntt_form() const noexcept { return is_ntt_form_; }
    [[nodiscard]] std::uint64_t correction_factor() const noexcept { return correction_factor_; }
    void set_scale(double s) noexcept { scale_ = s; }
    void set_ntt_form(bool b) noexcept { is_ntt_form_ = b; }
    void set_chain_index(std::size_t c) noexcept { chain_index_ = c; }
    void set_coeff_modulus_size(std::size_t s) noexcept { coeff_modulus_size_ = s; }
    PhantomDeviceBuffer &data_ptr() noexcept { return data_; }

    // Byte format of PhantomCiphertext::save / load (include/ciphertext.h:173-211).
    void save(std::ostream &os) const {
        os.write(reinterpret_cast<const char *>(&chain_index_), sizeof(std::size_t));
        os.write(reinterpret_cast<const char *>(&size_), sizeof(std::size_t));
        os.write(reinterpret_cast<const char *>(&poly_modulus_degree_), sizeof(std::size_t));
        os.write(reinterpret_cast<const char *>(&coeff_modulus_size_), sizeof(std::size_t));
        os.write(reinterpret_cast<const char *>(&scale_), sizeof(double));
        os.write(reinterpret_cast<const char *>(&correction_factor_), sizeof(std::uint64_t));
        os.write(reinterpret_cast<const char *>(&noise_scale_deg_), sizeof(std::size_t));
        os.write(reinterpret_cast<const char *>(&is_ntt_form_), sizeof(bool));
        os.write(reinterpret_cast<const char *>(&is_asymmetric_), sizeof(bool));
        std::vector<std::uint64_t> h(words());
        if (!h.empty()) {
            phantom::detail::cuda_check(cudaMemcpyAsync(h.data(), data_.get(), h.size() * 8, cudaMemcpyDeviceToHost,
                                                        cudaStreamPerThread));
            phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
        }
        os.write(reinterpret_cast<const char *>(h.data()), h.size() * 8);
    }
    void load(std::istream &is) {
        is.read(reinterpret_cast<char *>(&chain_index_), sizeof(std::size_t));
        is.read(reinterpret_cast<char *>(&size_), sizeof(std::size_t));
        is.read(reinterpret_cast<char *>(&poly_modulus_degree_), sizeof(std::size_t));
        is.read(reinterpret_cast<char *>(&coeff_modulus_size_), sizeof(std::size_t));
        is.read(reinterpret_cast<char *>(&scale_), sizeof(double));
        is.read(reinterpret_cast<char *>(&correction_factor_), sizeof(std::uint64_t));
        is.read(reinterpret_cast<char *>(&noise_scale_deg_), sizeof(std::size_t));
        is.read(reinterpret_cast<char *>(&is_ntt_form_), sizeof(bool));
        is.read(reinterpret_cast<char *>(&is_asymmetric_), sizeof(bool));
        if (!is) throw std::invalid_argument("truncated ciphertext stream");
        std::vector<std::uint64_t> h(words());
        is.read(reinterpret_cast<char *>(h.data()), h.size() * 8);
        if (!is) throw std::invalid_argument("truncated ciphertext stream");
        data_.reset(h.size());
        if (!h.empty()) {
            phantom::detail::cuda_check(cudaMemcpyAsync(data_.get(), h.data(), h.size() * 8, cudaMemcpyHostToDevice,
                                                        cudaStreamPerThread));
            phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
        }
    }

private:
    std::size_t words() const { return size_ * coeff_modulus_size_ * poly_modulus_degree_; }
    void reshape(std::size_t size, std::size_t limbs, std::size_t n) {
        const std::size_t old_words = words(), new_words = size * limbs * n;
        if (new_words != old_words) {
            PhantomDeviceBuffer nb(new_words);
            const std::size_t keep = std::min(old_words, new_words);
            if (keep)
                phantom::detail::cuda_check(cudaMemcpyAsync(nb.get(), data_.get(), keep * 8, cudaMemcpyDeviceToDevice,
                                                            cudaStreamPerThread));
            data_ = std::move(nb);
        }
        size_ = size;
        coeff_modulus_size_ = limbs;
        poly_modulus_degree_ = n;
    }

    std::size_t chain_index_ = 0, size_ = 0, poly_modulus_degree_ = 0, coeff_modulus_size_ = 0;
    double scale_ = 1.0;
    std::uint64_t correction_factor_ = 1;
    std::size_t noise_scale_deg_ = 1;
    bool is_ntt_form_ = true, is_asymmetric_ = false;
    PhantomDeviceBuffer data_;
};

// Relinearisation / key-switching key: dnum digits, each a size-2 ciphertext over QP in NTT form,
// plus the device array of digit pointers (include/secretkey.h:102-166).
class PhantomRelinKey {
public:
    PhantomRelinKey() = default;
    PhantomRelinKey(const PhantomRelinKey &) = delete;
    PhantomRelinKey &operator=(const PhantomRelinKey &) = delete;
    PhantomRelinKey(PhantomRelinKey &&) = default;
    PhantomRelinKey &operator=(PhantomRelinKey &&) = default;

    [[nodiscard]] const std::uint64_t *const *public_keys_ptr() const noexcept {
        return reinterpret_cast<const std::uint64_t *const *>(ptrs_.get());
    }
    [[nodiscard]] std::size_t dnum() const noexcept { return keys_.size(); }

    // Takes a generated key [dnum][2][QP][N] (device) as dnum size-2 ciphertexts at chain index 0.
    void assign(const PhantomContext &context, const std::uint64_t *key, std::size_t dnum) {
        keys_.clear();
        keys_.resize(dnum);
        const std::size_t words = 2 * context.coeff_modulus_size(0) * context.poly_modulus_degree();
        std::vector<std::uint64_t> p(dnum);
        for (std::size_t d = 0; d < dnum; d++) {
            keys_[d].resize(context, 0, 2);
            phantom::detail::cuda_check(cudaMemcpyAsync(keys_[d].data(), key + d * words, words * 8,
                                                        cudaMemcpyDeviceToDevice, cudaStreamPerThread));
            p[d] = reinterpret_cast<std::uint64_t>(keys_[d].data());
        }
        ptrs_.reset(dnum);
        phantom::detail::cuda_check(
                cudaMemcpyAsync(ptrs_.get(), p.data(), dnum * 8, cudaMemcpyHostToDevice, cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
    }

    void save(std::ostream &os) const {
        const std::size_t dnum = keys_.size();
        os.write(reinterpret_cast<const char *>(&dnum), sizeof(std::size_t));
        for (auto &k : keys_) k.save(os);
    }
    void load(std::istream &is) {
        std::size_t dnum = 0;
        is.read(reinterpret_cast<char *>(&dnum), sizeof(std::size_t));
        if (!is || dnum == 0 || dnum > 4096) throw std::invalid_argument("bad key stream");
        keys_.resize(dnum);
        for (auto &k : keys_) k.load(is);
        std::vector<std::uint64_t> p(dnum);
        for (std::size_t i = 0; i < dnum; i++) p[i] = reinterpret_cast<std::uint64_t>(keys_[i].data());
        ptrs_.reset(dnum);
        phantom::detail::cuda_check(
                cudaMemcpyAsync(ptrs_.get(), p.data(), dnum * 8, cudaMemcpyHostToDevice, cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
    }

private:
    std::vector<PhantomCiphertext> keys_;
    PhantomDeviceBuffer ptrs_;
};

class PhantomGaloisKey {
public:
    PhantomGaloisKey() = default;
    PhantomGaloisKey(const PhantomGaloisKey &) = delete;
    PhantomGaloisKey &operator=(const PhantomGaloisKey &) = delete;
    PhantomGaloisKey(PhantomGaloisKey &&) = default;
    PhantomGaloisKey &operator=(PhantomGaloisKey &&) = default;

    [[nodiscard]] const PhantomRelinKey &get_relin_keys(std::size_t index) const { return relin_keys_.at(index); }
    [[nodiscard]] std::size_t size() const noexcept { return relin_keys_.size(); }
    void save(std::ostream &os) const {
        const std::size_t n = relin_keys_.size();
        os.write(reinterpret_cast<const char *>(&n), sizeof(std::size_t));
        for (auto &k : relin_keys_) k.save(os);
    }
    void load(std::istream &is) {
        std::size_t n = 0;
        is.read(reinterpret_cast<char *>(&n), sizeof(std::size_t));
        if (!is || n > 4096) throw std::invalid_argument("bad Galois key stream");
        relin_keys_.resize(n);
        for (auto &k : relin_keys_) k.load(is);
    }
    void push_back(PhantomRelinKey &&k) { relin_keys_.push_back(std::move(k)); }
    // host array of the per-element digit-pointer arrays, for fhe_rotate / fhe_hoisting
    [[nodiscard]] std::vector<const std::uint64_t *const *> key_table() const {
        std::vector<const std::uint64_t *const *> t;
        for (auto &k : relin_keys_) t.push_back(k.public_keys_ptr());
        return t;
    }

private:
    std::vector<PhantomRelinKey> relin_keys_;
};

// CKKS plaintext in NTT form: [limbs][N] at a chain index, with its scale (include/plaintext.h).
class PhantomPlaintext {
public:
    PhantomPlaintext() = default;
    void resize(const PhantomContext &context, std::size_t chain_index) {
        limbs_ = context.coeff_modulus_size(chain_index);
        n_ = context.poly_modulus_degree();
        chain_index_ = chain_index;
        if (data_.size() != limbs_ * n_) data_.reset(limbs_ * n_);
    }
    [[nodiscard]] std::uint64_t *data() const noexcept { return data_.get(); }
    [[nodiscard]] std::size_t chain_index() const noexcept { return chain_index_; }
    [[nodiscard]] std::size_t coeff_modulus_size() const noexcept { return limbs_; }
    [[nodiscard]] std::size_t poly_modulus_degree() const noexcept { return n_; }
    [[nodiscard]] double scale() const noexcept { return scale_; }
    void set_scale(double s) noexcept { scale_ = s; }
    void set_chain_index(std::size_t c) noexcept { chain_index_ = c; }
    // raw shape (BFV plaintexts: one limb of N coefficients modulo t, include/plaintext.h)
    void resize(std::size_t coeff_modulus_size, std::size_t poly_modulus_degree) {
        limbs_ = coeff_modulus_size;
        n_ = poly_modulus_degree;
        if (data_.size() != limbs_ * n_) data_.reset(limbs_ * n_);
    }

private:
    std::size_t chain_index_ = 0, limbs_ = 0, n_ = 0;
    double scale_ = 1.0;
    PhantomDeviceBuffer data_;
};

// CKKS canonical embedding (PhantomCKKSEncoder, include/ckks.h:88-150): slot i of a plaintext
// holds m(zeta^(5^i mod 2N)) / scale, zeta = exp(i pi / N), i < N / 2.  encode and decode run on the
// GPU (fhe_ckks_encode / fhe_ckks_decode): the reference's FP64 special FFT, rounding and residues,
// and a CRT compose over every limb on decode, so the words and slots equal the reference's.
class PhantomCKKSEncoder {
public:
    explicit PhantomCKKSEncoder(const PhantomContext &context) : n_(context.poly_modulus_degree()) {}
    [[nodiscard]] std::size_t slot_count() const noexcept { return n_ / 2; }

    void encode(const PhantomContext &context, const std::vector<std::complex<double>> &values, double scale,
                PhantomPlaintext &destination, std::size_t chain_index = 1) const {
        if (values.empty()) throw std::invalid_argument("Input vector is empty");
        if (values.size() > n_ / 2) throw std::invalid_argument("Input vector exceeds max slots");
        destination.resize(context, chain_index);
        PhantomDeviceBuffer dv(2 * values.size());  // interleaved re, im doubles (8-byte words)
        phantom::detail::cuda_check(cudaMemcpyAsync(dv.get(), values.data(), values.size() * 16,
                                                    cudaMemcpyHostToDevice, cudaStreamPerThread));
        phantom::detail::check(fhe_ckks_encode(context.handle(), context.workspace(),
                                               reinterpret_cast<const double *>(dv.get()), values.size(), scale,
                                               chain_index, destination.data(), cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
        destination.set_scale(scale);
    }
    void encode(const PhantomContext &context, const std::vector<double> &values, double scale,
                PhantomPlaintext &destination, std::size_t chain_index = 1) const {
        encode(context, std::vector<std::complex<double>>(values.begin(), values.end()), scale, destination,
               chain_index);
    }
    template <class T>
    [[nodiscard]] PhantomPlaintext encode(const PhantomContext &context, const std::vector<T> &values, double scale,
                                          std::size_t chain_index = 1) const {
        PhantomPlaintext p;
        encode(context, values, scale, p, chain_index);
        return p;
    }

    void decode(const PhantomContext &context, const PhantomPlaintext &plain,
                std::vector<std::complex<double>> &destination) const {
        PhantomDeviceBuffer out(n_);  // N/2 complex doubles
        phantom::detail::check(fhe_ckks_decode(context.handle(), context.workspace(), plain.data(),
                                               plain.chain_index(), plain.scale(),
                                               reinterpret_cast<double *>(out.get()), cudaStreamPerThread));
        destination.resize(n_ / 2);
        phantom::detail::cuda_check(cudaMemcpyAsync(destination.data(), out.get(), n_ * 8, cudaMemcpyDeviceToHost,
                                                    cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
    }
    void decode(const PhantomContext &context, const PhantomPlaintext &plain, std::vector<double> &destination) const {
        std::vector<std::complex<double>> z;
        decode(context, plain, z);
        destination.resize(z.size());
        for (std::size_t i = 0; i < z.size(); i++) destination[i] = z[i].real();
    }
    template <class T>
    [[nodiscard]] std::vector<T> decode(const PhantomContext &context, const PhantomPlaintext &plain) const {
        std::vector<T> d;
        decode(context, plain, d);
        return d;
    }

private:
    std::size_t n_;
};

// Secret key (PhantomSecretKey, include/secretkey.h:276-330) for CKKS: uniform ternary s, the
// reference's key and encryption formulas on the GPU, randomness from a host generator (uniform
// a, centred binomial e: popcount of 21 bits minus popcount of 21 bits, as src/prng.cu:222-244).
// PhantomBatchEncoder (include/batchencoder.h, src/batchencoder.cu): N slots modulo t <-> a BFV
// plaintext, on the GPU (fhe_bfv_encode / fhe_bfv_decode).
class PhantomBatchEncoder {
public:
    explicit PhantomBatchEncoder(const PhantomContext &context) : n_(context.poly_modulus_degree()) {
        if (context.parms().scheme() != phantom::scheme_type::bfv)
            throw std::invalid_argument("PhantomBatchEncoder only supports BFV/BGV scheme");
    }
    [[nodiscard]] std::size_t slot_count() const noexcept { return n_; }
    void encode(const PhantomContext &context, const std::vector<std::uint64_t> &values_matrix,
                PhantomPlaintext &destination) const {
        if (values_matrix.size() > n_) throw std::logic_error("values_matrix size is too large");
        destination.resize(1, n_);
        destination.set_chain_index(0);
        PhantomDeviceBuffer dv(values_matrix.empty() ? 1 : values_matrix.size());
        phantom::detail::cuda_check(cudaMemcpyAsync(dv.get(), values_matrix.data(), values_matrix.size() * 8,
                                                    cudaMemcpyHostToDevice, cudaStreamPerThread));
        phantom::detail::check(fhe_bfv_encode(context.handle(), dv.get(), values_matrix.size(), destination.data(),
                                              cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
    }
    [[nodiscard]] PhantomPlaintext encode(const PhantomContext &context,
                                          const std::vector<std::uint64_t> &values_matrix) const {
        PhantomPlaintext p;
        encode(context, values_matrix, p);
        return p;
    }
    void decode(const PhantomContext &context, const PhantomPlaintext &plain,
                std::vector<std::uint64_t> &destination) const {
        destination.resize(n_);
        PhantomDeviceBuffer out(n_);
        phantom::detail::check(fhe_bfv_decode(context.handle(), context.workspace(), plain.data(), out.get(),
                                              cudaStreamPerThread));
        phantom::detail::cuda_check(cudaMemcpyAsync(destination.data(), out.get(), n_ * 8, cudaMemcpyDeviceToHost,
                                                    cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
    }
    [[nodiscard]] std::vector<std::uint64_t> decode(const PhantomContext &context, const PhantomPlaintext &plain) const {
        std::vector<std::uint64_t> v;
        decode(context, plain, v);
        return v;
    }

private:
    std::size_t n_;
};

class PhantomSecretKey {
public:
    // The secret key and every later key or encryption draw their randomness through the
    // reference's own device samplers (fhe_sample_*), each call keyed by a fresh 64-byte seed as
    // the reference's random_bytes supplies one; here the seeds come from a 64-bit generator
    // seeded by std::random_device, or by `seed` for reproducible runs.
    explicit PhantomSecretKey(const PhantomContext &context, std::uint64_t seed = std::random_device{}())
        : rng_(seed) {
        const std::size_t n = context.poly_modulus_degree(), qp = context.coeff_modulus_size(0);
        s_ntt_.reset(qp * n);
        const auto sd = seed_bytes();
        phantom::detail::check(fhe_secret_key_from_seed(context.handle(), context.workspace(), sd.data(), s_ntt_.get(),
                                                        cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
    }
    // gen_secretkey with the seed its random_bytes would have returned: the reference's key.
    PhantomSecretKey(const PhantomContext &context, const std::array<std::uint8_t, 64> &seed) : rng_(0) {
        const std::size_t n = context.poly_modulus_degree(), qp = context.coeff_modulus_size(0);
        s_ntt_.reset(qp * n);
        phantom::detail::check(fhe_secret_key_from_seed(context.handle(), context.workspace(), seed.data(),
                                                        s_ntt_.get(), cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
    }
    PhantomSecretKey(const PhantomSecretKey &) = delete;
    PhantomSecretKey &operator=(const PhantomSecretKey &) = delete;

    [[nodiscard]] PhantomRelinKey gen_relinkey(const PhantomContext &context) { return kswitch_key(context, 0); }

    [[nodiscard]] PhantomGaloisKey create_galois_keys(const PhantomContext &context) {
        PhantomGaloisKey g;
        for (std::uint32_t elt : context.galois_elts()) g.push_back(kswitch_key(context, elt));
        return g;
    }

    void encrypt_symmetric(const PhantomContext &context, const PhantomPlaintext &plain,
                           PhantomCiphertext &cipher) const {
        if (context.parms().scheme() == phantom::scheme_type::bfv) return bfv_encrypt(context, plain, cipher);
        const std::size_t n = context.poly_modulus_degree(), l = plain.coeff_modulus_size();
        PhantomDeviceBuffer da(l * n), de(n);
        const auto sa = seed_bytes(), se = seed_bytes();
        phantom::detail::check(fhe_sample_uniform(context.handle(), sa.data(), l, da.get(), cudaStreamPerThread));
        phantom::detail::check(fhe_sample_cbd(context.handle(), se.data(), reinterpret_cast<std::int64_t *>(de.get()),
                                              cudaStreamPerThread));
        cipher.resize(context, plain.chain_index(), 2);
        phantom::detail::check(fhe_ckks_encrypt_symmetric(context.handle(), plain.data(), s_ntt_.get(), da.get(),
                                                          reinterpret_cast<const std::int64_t *>(de.get()),
                                                          cipher.data(), plain.chain_index(), cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
        cipher.set_scale(plain.scale());
        cipher.set_ntt_form(true);
    }
    [[nodiscard]] PhantomCiphertext encrypt_symmetric(const PhantomContext &context,
                                                      const PhantomPlaintext &plain) const {
        PhantomCiphertext c;
        encrypt_symmetric(context, plain, c);
        return c;
    }

    void decrypt(const PhantomContext &context, const PhantomCiphertext &cipher, PhantomPlaintext &plain) {
        if (cipher.size() != 2) throw std::invalid_argument("decrypt needs a size-2 ciphertext");
        if (context.parms().scheme() == phantom::scheme_type::bfv) {
            plain.resize(1, context.poly_modulus_degree());
            plain.set_chain_index(0);
            phantom::detail::check(fhe_bfv_decrypt(context.handle(), context.workspace(), cipher.data(),
                                                   cipher.chain_index(), s_ntt_.get(), plain.data(),
                                                   cudaStreamPerThread));
            phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
            return;
        }
        plain.resize(context, cipher.chain_index());
        phantom::detail::check(fhe_ckks_decrypt(context.handle(), cipher.data(), s_ntt_.get(), plain.data(),
                                                cipher.chain_index(), cudaStreamPerThread));
        plain.set_scale(cipher.scale());
    }
    [[nodiscard]] PhantomPlaintext decrypt(const PhantomContext &context, const PhantomCiphertext &cipher) {
        PhantomPlaintext p;
        decrypt(context, cipher, p);
        return p;
    }

private:
    // BFV at the first data level (src/secretkey.cu:463-485): a and e from fresh seeds.
    void bfv_encrypt(const PhantomContext &context, const PhantomPlaintext &plain, PhantomCiphertext &cipher) const {
        const std::size_t n = context.poly_modulus_degree(), l = context.coeff_modulus_size(1);
        PhantomDeviceBuffer da(l * n), de(n);
        const auto sa = seed_bytes(), se = seed_bytes();
        phantom::detail::check(fhe_sample_uniform(context.handle(), sa.data(), l, da.get(), cudaStreamPerThread));
        phantom::detail::check(fhe_sample_cbd(context.handle(), se.data(), reinterpret_cast<std::int64_t *>(de.get()),
                                              cudaStreamPerThread));
        cipher.resize(context, 1, 2);
        phantom::detail::check(fhe_bfv_encrypt_symmetric(context.handle(), plain.data(), s_ntt_.get(), da.get(),
                                                         reinterpret_cast<const std::int64_t *>(de.get()),
                                                         cipher.data(), cudaStreamPerThread));
        phantom::detail::cuda_check(cudaStreamSynchronize(cudaStreamPerThread));
        cipher.set_scale(1.0);
        cipher.set_ntt_form(false);
    }
    std::array<std::uint8_t, 64> seed_bytes() const {
        std::array<std::uint8_t, 64> b;
        for (std::size_t i = 0; i < 64; i += 8) {
            const std::uint64_t r = rng_();
            for (std::size_t k = 0; k < 8; k++) b[i + k] = (std::uint8_t)(r >> (8 * k));
        }
        return b;
    }
    PhantomRelinKey kswitch_key(const PhantomContext &context, std::uint32_t elt) {
        const std::size_t n = context.poly_modulus_degree(), qp = context.coeff_modulus_size(0);
        std::size_t nq, np, nr, dnum;
        std::uint64_t nn;
        phantom::detail::check(fhe_context_sizes(context.handle(), &nn, &nq, &np, &nr, &dnum));
        std::vector<std::uint8_t> sa(64 * dnum), se(64 * dnum);
        for (std::size_t d = 0; d < dnum; d++) {
            const auto a = seed_bytes(), e = seed_bytes();
            std::copy(a.begin(), a.end(), sa.begin() + 64 * d);
            std::copy(e.begin(), e.end(), se.begin() + 64 * d);
        }
        PhantomDeviceBuffer key(dnum * 2 * qp * n);
        phantom::detail::check(fhe_kswitch_keygen_seeded(context.handle(), context.workspace(), elt, s_ntt_.get(),
                                                         sa.data(), se.data(), key.get(), cudaStreamPerThread));
        PhantomRelinKey k;
        k.assign(context, key.get(), dnum);
        return k;
    }

    mutable std::mt19937_64 rng_;
    PhantomDeviceBuffer s_ntt_;  // [QP][N], NTT form
};

namespace phantom {

namespace detail {
inline void same_level(const PhantomCiphertext &a, const PhantomCiphertext &b) {
    if (a.chain_index() != b.chain_index()) throw std::invalid_argument("encrypted1 and encrypted2 parameter mismatch");
    if (a.is_ntt_form() != b.is_ntt_form()) throw std::invalid_argument("NTT form mismatch");
    if (a.size() != b.size()) throw std::invalid_argument("poly number mismatch");
}
inline bool same_scale(double a, double b) { return std::fabs(a - b) <= 1e-9 * std::max(std::fabs(a), std::fabs(b)); }
}  // namespace detail

// keyswitch_inplace (include/evaluate.cuh:29): ct += KeySwitch(c2)
inline void keyswitch_inplace(const PhantomContext &context, PhantomCiphertext &encrypted, std::uint64_t *c2,
                              const PhantomRelinKey &relin_keys, bool /*is_relin*/, const cudaStream_t &stream) {
    detail::check(fhe_keyswitch(context.handle(), context.workspace(), encrypted.data(), c2, encrypted.chain_index(),
                                relin_keys.public_keys_ptr(), stream));
}

// multiply_inplace for CKKS (bgv_ckks_multiply, src/evaluate.cu:345-397): ct1 becomes size 3
inline void multiply_inplace(const PhantomContext &context, PhantomCiphertext &encrypted1,
                             const PhantomCiphertext &encrypted2) {
    if (context.parms().scheme() != scheme_type::ckks) throw std::invalid_argument("multiply_inplace: CKKS only");
    detail::same_level(encrypted1, encrypted2);
    if (!encrypted1.is_ntt_form()) throw std::invalid_argument("encrypted1 and encrypted2 must be in NTT form");
    const bool square = &encrypted1 == &encrypted2;
    encrypted1.resize(context, encrypted1.chain_index(), 3);
    detail::check(fhe_ckks_multiply(context.handle(), encrypted1.data(), square ? encrypted1.data() : encrypted2.data(),
                                    encrypted1.chain_index(), cudaStreamPerThread));
    encrypted1.set_scale(encrypted1.scale() * encrypted2.scale());
}

// relinearize_inplace (include/evaluate.cuh:125)
inline void relinearize_inplace(const PhantomContext &context, PhantomCiphertext &encrypted,
                                const PhantomRelinKey &relin_keys) {
    if (encrypted.size() != 3) throw std::invalid_argument("destination_size must be 3");
    detail::check(fhe_relinearize(context.handle(), context.workspace(), encrypted.data(), encrypted.chain_index(),
                                  relin_keys.public_keys_ptr(), cudaStreamPerThread));
    encrypted.resize(2, encrypted.coeff_modulus_size(), encrypted.poly_modulus_degree());
}

// multiply_and_relin_inplace (include/evaluate.cuh:115)
inline void multiply_and_relin_inplace(const PhantomContext &context, PhantomCiphertext &encrypted1,
                                       const PhantomCiphertext &encrypted2, const PhantomRelinKey &relin_keys) {
    detail::same_level(encrypted1, encrypted2);
    if (!detail::same_scale(encrypted1.scale(), encrypted2.scale())) throw std::invalid_argument("scale mismatch");
    if (encrypted1.size() != 2) throw std::invalid_argument("ciphertext size must be 2");
    detail::check(fhe_multiply_and_relin(context.handle(), context.workspace(), encrypted1.data(), encrypted2.data(),
                                         encrypted1.chain_index(), relin_keys.public_keys_ptr(), cudaStreamPerThread));
    if (context.parms().scheme() == scheme_type::ckks) encrypted1.set_scale(encrypted1.scale() * encrypted2.scale());
}

inline PhantomCiphertext multiply_and_relin(const PhantomContext &context, const PhantomCiphertext &encrypted1,
                                            const PhantomCiphertext &encrypted2, const PhantomRelinKey &relin_keys) {
    PhantomCiphertext r = encrypted1;
    multiply_and_relin_inplace(context, r, encrypted2, relin_keys);
    return r;
}

// rescale_to_next (include/evaluate.cuh:137): CKKS, divides by q_last and drops it
inline PhantomCiphertext rescale_to_next(const PhantomContext &context, const PhantomCiphertext &encrypted) {
    if (context.parms().scheme() != scheme_type::ckks) throw std::invalid_argument("unsupported scheme");
    if (encrypted.chain_index() == context.size_q()) throw std::invalid_argument("end of modulus switching chain reached");
    PhantomCiphertext dst;
    dst.resize(context, encrypted.chain_index() + 1, encrypted.size());
    detail::check(fhe_rescale_to_next(context.handle(), context.workspace(), encrypted.data(), dst.data(),
                                      encrypted.size(), encrypted.chain_index(), cudaStreamPerThread));
    dst.set_ntt_form(encrypted.is_ntt_form());
    dst.set_scale(encrypted.scale() /
                  static_cast<double>(context.modulus(context.coeff_modulus_size(encrypted.chain_index()) - 1)));
    return dst;
}

inline void rescale_to_next_inplace(const PhantomContext &context, PhantomCiphertext &encrypted) {
    encrypted = rescale_to_next(context, encrypted);
}

// mod_switch_to_next_inplace (include/evaluate.cuh:149): CKKS drops q_last; BFV divides by it
inline void mod_switch_to_next_inplace(const PhantomContext &context, PhantomCiphertext &encrypted) {
    if (encrypted.chain_index() == context.size_q()) throw std::invalid_argument("end of modulus switching chain reached");
    const std::size_t n = context.poly_modulus_degree(), l = encrypted.coeff_modulus_size(), size = encrypted.size();
    PhantomCiphertext dst;
    dst.resize(context, encrypted.chain_index() + 1, size);
    if (context.parms().scheme() == scheme_type::ckks) {
        detail::cuda_check(cudaMemcpy2DAsync(dst.data(), (l - 1) * n * 8, encrypted.data(), l * n * 8, (l - 1) * n * 8,
                                             size, cudaMemcpyDeviceToDevice, cudaStreamPerThread));
    } else {
        detail::check(fhe_bfv_mod_switch_to_next(context.handle(), encrypted.data(), dst.data(), size,
                                                 encrypted.chain_index(), cudaStreamPerThread));
    }
    dst.set_scale(encrypted.scale());
    dst.set_ntt_form(encrypted.is_ntt_form());
    encrypted = std::move(dst);
}

inline std::size_t galois_index(const PhantomContext &context, std::uint32_t elt) {
    const auto &e = context.galois_elts();
    for (std::size_t i = 0; i < e.size(); i++)
        if (e[i] == elt) return i;
    throw std::invalid_argument("Galois elt not present");
}

// apply_galois_inplace (include/evaluate.cuh:215)
inline void apply_galois_inplace(const PhantomContext &context, PhantomCiphertext &encrypted, std::size_t galois_elt,
                                 const PhantomGaloisKey &galois_keys) {
    if (encrypted.size() > 2) throw std::invalid_argument("encrypted size must be 2");
    const std::size_t idx = galois_index(context, static_cast<std::uint32_t>(galois_elt));
    detail::check(fhe_apply_galois(context.handle(), context.workspace(), encrypted.data(), encrypted.chain_index(),
                                   static_cast<std::uint32_t>(galois_elt),
                                   galois_keys.get_relin_keys(idx).public_keys_ptr(), cudaStreamPerThread));
}

// rotate_inplace (include/evaluate.cuh:225), NAF fallback included
inline void rotate_inplace(const PhantomContext &context, PhantomCiphertext &encrypted, int step,
                           const PhantomGaloisKey &galois_key) {
    const auto table = galois_key.key_table();
    detail::check(fhe_rotate(context.handle(), context.workspace(), encrypted.data(), encrypted.chain_index(), step,
                             table.data(), cudaStreamPerThread));
}

inline PhantomCiphertext rotate(const PhantomContext &context, const PhantomCiphertext &encrypted, int step,
                                const PhantomGaloisKey &galois_key) {
    PhantomCiphertext r = encrypted;
    rotate_inplace(context, r, step, galois_key);
    return r;
}

// hoisting_inplace (include/evaluate.cuh:237): ct <- sum_s rotate(ct, s)
inline void hoisting_inplace(const PhantomContext &context, PhantomCiphertext &ct, const PhantomGaloisKey &glk,
                             const std::vector<int> &steps) {
    if (ct.size() > 2) throw std::invalid_argument("ciphertext size must be 2");
    const auto table = glk.key_table();
    detail::check(fhe_hoisting(context.handle(), context.workspace(), ct.data(), ct.chain_index(), steps.data(),
                               steps.size(), table.data(), cudaStreamPerThread));
}

// multiply_plain_inplace (include/evaluate.cuh:94, src/evaluate.cu:1224-1250, CKKS NTT form)
inline void multiply_plain_inplace(const PhantomContext &context, PhantomCiphertext &encrypted,
                                   const PhantomPlaintext &plain) {
    if (encrypted.chain_index() != plain.chain_index()) throw std::invalid_argument("encrypted and plain parameter mismatch");
    if (encrypted.size() != 2) throw std::invalid_argument("multiply_plain needs a size-2 ciphertext");
    detail::check(fhe_ckks_multiply_plain(context.handle(), encrypted.data(), plain.data(), encrypted.data(),
                                          encrypted.chain_index(), cudaStreamPerThread));
    encrypted.set_scale(encrypted.scale() * plain.scale());
}

inline PhantomCiphertext multiply_plain(const PhantomContext &context, const PhantomCiphertext &encrypted,
                                        const PhantomPlaintext &plain) {
    PhantomCiphertext d = encrypted;
    multiply_plain_inplace(context, d, plain);
    return d;
}

// add_inplace (include/evaluate.cuh:46, src/evaluate.cu:116-198)
inline void add_inplace(const PhantomContext &context, PhantomCiphertext &encrypted1,
                        const PhantomCiphertext &encrypted2) {
    detail::same_level(encrypted1, encrypted2);
    if (encrypted1.size() != encrypted2.size()) throw std::invalid_argument("ciphertext sizes mismatch");
    if (!detail::same_scale(encrypted1.scale(), encrypted2.scale())) throw std::invalid_argument("scale mismatch");
    detail::check(fhe_ckks_add(context.handle(), encrypted1.data(), encrypted2.data(), encrypted1.data(),
                               encrypted1.size(), encrypted1.chain_index(), cudaStreamPerThread));
}

inline PhantomCiphertext add(const PhantomContext &context, const PhantomCiphertext &encrypted1,
                             const PhantomCiphertext &encrypted2) {
    PhantomCiphertext d = encrypted1;
    add_inplace(context, d, encrypted2);
    return d;
}

}  // namespace phantom
