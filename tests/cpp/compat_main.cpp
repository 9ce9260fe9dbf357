// Drives the C++ compatibility layer (phantom-fhe_gb300/cpp/phantom.h) the way a PhantomFHE
// program does: parameters, context, ciphertexts and keys loaded from streams in the
// reference's byte format, evaluator calls, results saved in the same format.
// Usage: compat_main <dir>   (reads a.bin b.bin rlk.bin gk.bin, writes out_*.bin)
#include <fstream>
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
    cudaDeviceSynchronize();
    std::cout << "compat ok\n";
    return 0;
}
