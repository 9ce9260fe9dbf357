// Drives the C++ compatibility layer (phantom-fhe_gb300/cpp/phantom.h) the way a PhantomFHE
// program does: parameters, context, ciphertexts and keys loaded from streams in the
// reference's byte format, evaluator calls, results saved in the same format.
// Usage: compat_main <dir>   (reads a.bin b.bin rlk.bin gk.bin, writes out_*.bin)
#include <complex>
#include <cstdlib>
#include <fstream>
#include <random>
#include <iostream>
#include <sstream>
#include <string>

#include "phantom.h"

using namespace phantom;

template <class T>
static void load(T &obj, const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    obj.load(f);
}

static void save(const PhantomCiphertext &ct, const std::string &path) {
    std::ofstream f(path, std::ios::binary);
    ct.save(f);
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    EncryptionParameters parms(scheme_type::ckks);
    parms.set_poly_modulus_degree(4096);
    parms.set_coeff_modulus(arith::CoeffModulus::Create(4096, {60, 40, 40, 40, 40, 40, 60, 60}));
    parms.set_special_modulus_size(2);
    PhantomContext context(parms);

    PhantomCiphertext a, b;
    PhantomRelinKey rlk;
    PhantomGaloisKey gk;
    load(a, dir + "/a.bin");
    load(b, dir + "/b.bin");
    load(rlk, dir + "/rlk.bin");
    load(gk, dir + "/gk.bin");

    // HMult + relinearise + rescale, as two reference calls
    PhantomCiphertext m = multiply_and_relin(context, a, b, rlk);
    rescale_to_next_inplace(context, m);
    save(m, dir + "/out_mul_rescale.bin");

    // relinearize_inplace after multiply_inplace must equal multiply_and_relin
    PhantomCiphertext t = a;
    multiply_inplace(context, t, b);
    relinearize_inplace(context, t, rlk);
    save(t, dir + "/out_mul_then_relin.bin");

    // rotation by 3 has no key: NAF 4 - 1
    PhantomCiphertext r = a;
    rotate_inplace(context, r, 3, gk);
    save(r, dir + "/out_rotate3.bin");

    PhantomCiphertext h = a;
    hoisting_inplace(context, h, gk, {1, 2});
    save(h, dir + "/out_hoist12.bin");

    PhantomCiphertext d = a;
    mod_switch_to_next_inplace(context, d);
    save(d, dir + "/out_drop.bin");

    // save/load round trip
    std::stringstream ss;
    a.save(ss);
    PhantomCiphertext a2;
    a2.load(ss);
    std::stringstream s1, s2;
    a.save(s1);
    a2.save(s2);
    if (s1.str() != s2.str()) {
        std::cerr << "save/load round trip differs\n";
        return 1;
    }

    // the reference's error classes
    bool threw = false;
    try {
        multiply_and_relin_inplace(context, d, b, rlk);  // chain index mismatch
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    if (!threw) {
        std::cerr << "expected std::invalid_argument for a chain-index mismatch\n";
        return 1;
    }
    // end to end as in the reference's CKKS examples: keys, encode, encrypt, evaluate, decrypt, decode
    {
        PhantomCKKSEncoder encoder(context);
        PhantomSecretKey sk(context, 42);
        PhantomRelinKey rk = sk.gen_relinkey(context);
        PhantomGaloisKey gks = sk.create_galois_keys(context);
        const double scale = std::pow(2.0, 40);
        const std::size_t slots = encoder.slot_count();
        std::mt19937_64 g(7);
        std::uniform_real_distribution<double> u(-0.7, 0.7);
        std::vector<std::complex<double>> x(slots), y(slots);
        for (std::size_t i = 0; i < slots; i++) {
            x[i] = {u(g), u(g)};
            y[i] = {u(g), u(g)};
        }
        PhantomPlaintext px = encoder.encode(context, x, scale), py = encoder.encode(context, y, scale);
        PhantomCiphertext cx = sk.encrypt_symmetric(context, px), cy = sk.encrypt_symmetric(context, py);
        double err = 0;
        auto check = [&](const PhantomCiphertext &c, auto want, const char *what) {
            PhantomPlaintext p = sk.decrypt(context, c);
            std::vector<std::complex<double>> z = encoder.decode<std::complex<double>>(context, p);
            double e = 0;
            for (std::size_t i = 0; i < slots; i++) e = std::max(e, std::abs(z[i] - want(i)));
            if (!(e < 1e-3)) {
                std::cerr << what << ": max slot error " << e << "\n";
                std::exit(1);
            }
            err = std::max(err, e);
        };
        check(cx, [&](std::size_t i) { return x[i]; }, "encrypt/decrypt");
        PhantomCiphertext prod = multiply_and_relin(context, cx, cy, rk);
        rescale_to_next_inplace(context, prod);
        check(prod, [&](std::size_t i) { return x[i] * y[i]; }, "multiply_and_relin + rescale");
        rotate_inplace(context, prod, 1, gks);
        check(prod, [&](std::size_t i) { return x[(i + 1) % slots] * y[(i + 1) % slots]; }, "rotate by 1");
        PhantomCiphertext mp = multiply_plain(context, cx, py);
        rescale_to_next_inplace(context, mp);
        check(mp, [&](std::size_t i) { return x[i] * y[i]; }, "multiply_plain + rescale");
        PhantomCiphertext sum = add(context, cx, cy);
        check(sum, [&](std::size_t i) { return x[i] + y[i]; }, "add");
        std::cout << "ckks end to end max slot error " << err << "\n";
    }

    {  // BFV end to end: batch encoding, encryption, HPS multiply + relinearise, decryption
        EncryptionParameters bp(scheme_type::bfv);
        bp.set_poly_modulus_degree(4096);
        bp.set_coeff_modulus(arith::CoeffModulus::Create(4096, {50, 50, 50, 50, 60, 60}));
        bp.set_special_modulus_size(2);
        bp.set_plain_modulus(arith::Modulus(65537));
        PhantomContext bctx(bp);
        PhantomBatchEncoder benc(bctx);
        PhantomSecretKey bsk(bctx);
        PhantomRelinKey brk = bsk.gen_relinkey(bctx);
        const std::size_t slots = benc.slot_count();
        std::mt19937_64 g(11);
        std::vector<std::uint64_t> x(slots), y(slots);
        for (std::size_t i = 0; i < slots; i++) {
            x[i] = g() % 65537;
            y[i] = g() % 65537;
        }
        PhantomCiphertext cx = bsk.encrypt_symmetric(bctx, benc.encode(bctx, x));
        PhantomCiphertext cy = bsk.encrypt_symmetric(bctx, benc.encode(bctx, y));
        if (benc.decode(bctx, bsk.decrypt(bctx, cx)) != x) {
            std::cerr << "BFV encrypt/decrypt: slots differ\n";
            return 1;
        }
        multiply_and_relin_inplace(bctx, cx, cy, brk);
        const std::vector<std::uint64_t> z = benc.decode(bctx, bsk.decrypt(bctx, cx));
        for (std::size_t i = 0; i < slots; i++)
            if (z[i] != x[i] * y[i] % 65537) {
                std::cerr << "BFV multiply_and_relin: slot " << i << " is " << z[i] << "\n";
                return 1;
            }
        std::cout << "bfv end to end: " << slots << " slots exact\n";
    }

    cudaDeviceSynchronize();
    std::cout << "compat ok\n";
    return 0;
}
