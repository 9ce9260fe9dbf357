// host_tables.cpp — see host_tables.hpp.
#include "host_tables.hpp"

#include <algorithm>
#include <cstdlib>
#include <map>

namespace pfg::host {

typedef unsigned __int128 u128;

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t q) { return (uint64_t)(((u128)a * b) % q); }

uint64_t powmod(uint64_t a, uint64_t e, uint64_t q) {
    uint64_t r = 1 % q;
    a %= q;
    for (; e; e >>= 1) {
        if (e & 1) r = mulmod(r, a, q);
        a = mulmod(a, a, q);
    }
    return r;
}

uint64_t invmod(uint64_t a, uint64_t q) {
    a %= q;
    __int128 r0 = q, r1 = a, t0 = 0, t1 = 1;
    while (r1) {
        __int128 k = r0 / r1, tmp = r0 - k * r1;
        r0 = r1;
        r1 = tmp;
        tmp = t0 - k * t1;
        t0 = t1;
        t1 = tmp;
    }
    if (r0 != 1) throw std::invalid_argument("value is not invertible modulo the prime");
    if (t0 < 0) t0 += q;
    return (uint64_t)t0;
}

// Miller-Rabin with the first twelve prime bases: exact for every 64-bit integer, so it
// accepts exactly the primes the reference's randomised test accepts.
bool is_prime(uint64_t v) {
    static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (v < 2) return false;
    for (uint64_t b : bases) {
        if (v == b) return true;
        if (v % b == 0) return false;
    }
    uint64_t d = v - 1;
    int r = 0;
    while (!(d & 1)) {
        d >>= 1;
        r++;
    }
    for (uint64_t b : bases) {
        uint64_t x = powmod(b, d, v);
        if (x == 1 || x == v - 1) continue;
        bool witness = true;
        for (int i = 1; i < r && witness; i++) {
            x = mulmod(x, x, v);
            if (x == v - 1) witness = false;
        }
        if (witness) return false;
    }
    return true;
}

uint64_t shoup(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }

void barrett(uint64_t q, uint64_t &mu_lo, uint64_t &mu_hi) {
    u128 all = ~(u128)0;
    u128 quo = all / q, rem = all % q + 1;
    if (rem == q) quo += 1;
    mu_lo = (uint64_t)quo;
    mu_hi = (uint64_t)(quo >> 64);
}

static int sig_bits(uint64_t v) {
    int b = 0;
    for (; v; v >>= 1) b++;
    return b;
}

std::vector<uint64_t> get_primes(uint64_t n, int bits, size_t count) {
    std::vector<uint64_t> out;
    uint64_t factor = 2 * n, value = (uint64_t(1) << bits) - factor + 1, lower = uint64_t(1) << (bits - 1);
    while (out.size() < count && value > lower) {
        if (is_prime(value)) out.push_back(value);
        value -= factor;
    }
    if (out.size() < count) throw std::logic_error("failed to find enough qualifying primes");
    return out;
}

std::vector<uint64_t> get_primes_below(uint64_t n, uint64_t upper, size_t count) {
    std::vector<uint64_t> out;
    uint64_t factor = 2 * n, value = upper - factor, lower = uint64_t(1) << (sig_bits(upper) - 1);
    while (out.size() < count && value > lower) {
        if (is_prime(value)) out.push_back(value);
        value -= factor;
    }
    if (out.size() < count) throw std::logic_error("failed to find enough qualifying primes");
    return out;
}

std::vector<uint64_t> create_coeff_modulus(uint64_t n, const std::vector<int> &bit_sizes) {
    std::map<int, size_t> count;
    for (int b : bit_sizes) {
        if (b < 2 || b > 60) throw std::invalid_argument("bit_sizes is invalid");
        count[b]++;
    }
    std::map<int, std::vector<uint64_t>> primes;
    for (auto &kv : count) primes[kv.first] = get_primes(n, kv.first, kv.second);
    std::vector<uint64_t> out;
    for (int b : bit_sizes) {
        out.push_back(primes[b].back());
        primes[b].pop_back();
    }
    return out;
}

uint64_t minimal_root(uint64_t degree, uint64_t q) {
    if ((q - 1) % degree) throw std::invalid_argument("modulus has no primitive root of this degree");
    uint64_t quot = (q - 1) / degree, g = 0;
    for (uint64_t x = 2;; x++) {
        g = powmod(x, quot, q);
        if (powmod(g, degree / 2, q) == q - 1) break;
    }
    uint64_t g2 = mulmod(g, g, q), cur = g, best = g;
    for (uint64_t i = 0; i < degree / 2; i++) {
        best = std::min(best, cur);
        cur = mulmod(cur, g2, q);
    }
    return best;
}

uint32_t bitrev(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; i++, x >>= 1) r = (r << 1) | (x & 1);
    return r;
}

void ntt_tables(int log_n, uint64_t q, std::vector<uint64_t> &tw, std::vector<uint64_t> &itw, uint64_t &n_inv,
                uint64_t &n_inv_shoup) {
    const uint64_t n = uint64_t(1) << log_n;
    const uint64_t psi = minimal_root(2 * n, q), ipsi = invmod(psi, q);
    std::vector<uint64_t> r(n), ir(n);
    r[0] = ir[0] = 1;
    uint64_t p = psi, ip = ipsi;
    for (uint64_t i = 1; i < n; i++) {
        r[bitrev((uint32_t)i, log_n)] = p;
        ir[bitrev((uint32_t)i, log_n)] = ip;
        p = mulmod(p, psi, q);
        ip = mulmod(ip, ipsi, q);
    }
    n_inv = invmod(n, q);
    n_inv_shoup = shoup(n_inv, q);
    ir[1] = mulmod(ir[1], n_inv, q);
    tw.resize(2 * n);
    itw.resize(2 * n);
    for (uint64_t i = 0; i < n; i++) {
        tw[2 * i] = r[i];
        tw[2 * i + 1] = shoup(r[i], q);
        itw[2 * i] = ir[i];
        itw[2 * i + 1] = shoup(ir[i], q);
    }
}

uint64_t prod_mod(const std::vector<uint64_t> &mods, int skip, uint64_t p) {
    uint64_t r = 1 % p;
    for (size_t k = 0; k < mods.size(); k++)
        if ((int)k != skip) r = mulmod(r, mods[k] % p, p);
    return r;
}

uint32_t elt_from_step(int step, uint64_t n) {
    const uint32_t m32 = (uint32_t)(2 * n);
    const uint64_t m = m32;
    if (step == 0) return m32 - 1;
    const bool neg = step < 0;
    uint32_t pos = (uint32_t)std::abs(step);
    if (pos >= (n >> 1)) throw std::invalid_argument("step count too large");
    pos &= m32 - 1;
    int s = neg ? (int)(n >> 1) - (int)pos : (int)pos;
    uint64_t elt = 1;
    while (s--) elt = (elt * 5) & (m - 1);
    return (uint32_t)elt;
}

std::vector<uint32_t> galois_perm(int log_n, uint32_t elt) {
    const uint32_t n = 1u << log_n;
    std::vector<uint32_t> perm(n);
    for (uint32_t i = n; i < 2 * n; i++) {
        uint64_t raw = ((uint64_t)elt * bitrev(i, log_n + 1)) >> 1;
        perm[i - n] = bitrev((uint32_t)(raw & (n - 1)), log_n);
    }
    return perm;
}

std::vector<int> naf(int value) {
    std::vector<int> res;
    bool neg = value < 0;
    value = std::abs(value);
    for (int i = 0; value; i++) {
        int zi = (value & 1) ? 2 - (value & 3) : 0;
        value = (value - zi) >> 1;
        if (zi) res.push_back((neg ? -zi : zi) * (1 << i));
    }
    return res;
}

}  // namespace pfg::host
