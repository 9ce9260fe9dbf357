// host_tables.hpp — host-side number theory and constant tables for the GPU library.
//
// Value-identical restatement of the reference's SEAL-derived host code:
//   primes            get_primes / get_primes_below   (src/host/numth.cu:207-261)
//   coeff modulus     CoeffModulus::Create            (src/host/modulus.cu:80-111)
//   Barrett ratio     Modulus::set_value              (src/host/modulus.cu:15-42)
//   2N-th root        try_minimal_primitive_root      (src/host/numth.cu:309-331)
//   NTT tables        NTT::NTT                        (src/host/ntt.cu:11-56)
//   RNS constants     RNSBase / BaseConverter / DRNSTool ctor
//                     (src/host/rns.cu:282-498, src/rns.cu:66-195, 687-777)
// Products of moduli are never formed as big integers: (prod_{k != i} q_k) mod p is the
// product of the residues, which gives the same words as the reference's multi-precision
// route.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <vector>

namespace pfg::host {

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t q);
uint64_t powmod(uint64_t a, uint64_t e, uint64_t q);
uint64_t invmod(uint64_t a, uint64_t q);  // throws if not invertible
bool is_prime(uint64_t v);
uint64_t shoup(uint64_t w, uint64_t q);
void barrett(uint64_t q, uint64_t &mu_lo, uint64_t &mu_hi);
std::vector<uint64_t> get_primes(uint64_t n, int bits, size_t count);
std::vector<uint64_t> get_primes_below(uint64_t n, uint64_t upper, size_t count);
std::vector<uint64_t> create_coeff_modulus(uint64_t n, const std::vector<int> &bit_sizes);
uint64_t minimal_root(uint64_t degree, uint64_t q);
uint32_t bitrev(uint32_t x, int bits);
// Interleaved (w, w') pairs, 2*N words each, plus n^-1 and its Shoup quotient.
void ntt_tables(int log_n, uint64_t q, std::vector<uint64_t> &tw, std::vector<uint64_t> &itw, uint64_t &n_inv,
                uint64_t &n_inv_shoup);
// prod_{k in idx, k != skip} mods[k]  mod p   (skip < 0: full product)
uint64_t prod_mod(const std::vector<uint64_t> &mods, int skip, uint64_t p);
// Galois automorphism helpers (include/galois.cuh:16-49, 98-113).
uint32_t elt_from_step(int step, uint64_t n);
std::vector<uint32_t> galois_perm(int log_n, uint32_t elt);
std::vector<int> naf(int value);  // include/host/numth.h:17-33

}  // namespace pfg::host
