// ref_dump.cpp — prints the reference's own host-side tables as JSON.
//
// TEST INFRASTRUCTURE ONLY.  Linked against PhantomFHE's host sources (src/host/*.cu,
// compiled unmodified as C++ by oracle/Makefile.ref into oracle/_ref/), it calls the
// reference's own routines — CoeffModulus::Create, Modulus, NTT, RNSBase, BaseConverter,
// get_primes_below and the multi-precision helpers — in the same order that the
// reference's context and DRNSTool constructors call them (src/context.cu:121-183,
// src/rns.cu:100-195 and 687-777).  tests/golden/make_golden_tables.py turns the output
// into the committed fixtures that pin the oracle's and the GPU library's tables.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "host/modulus.h"
#include "host/ntt.h"
#include "host/numth.h"
#include "host/rns.h"
#include "host/uintarith.h"
#include "host/uintarithsmallmod.h"

using namespace phantom::arith;
using std::vector;

static void arr(const char *key, const uint64_t *v, size_t n, bool last = false) {
    std::printf("\"%s\":[", key);
    for (size_t i = 0; i < n; i++) std::printf("%s%llu", i ? "," : "", (unsigned long long)v[i]);
    std::printf("]%s", last ? "" : ",");
}

static void darr(const char *key, const double *v, size_t n, bool last = false) {
    // doubles as their IEEE-754 bit patterns
    std::printf("\"%s\":[", key);
    for (size_t i = 0; i < n; i++) {
        uint64_t b;
        std::memcpy(&b, &v[i], 8);
        std::printf("%s%llu", i ? "," : "", (unsigned long long)b);
    }
    std::printf("]%s", last ? "" : ",");
}

static vector<uint64_t> values(const vector<Modulus> &m) {
    vector<uint64_t> v;
    for (auto &x : m) v.push_back(x.value());
    return v;
}

struct Cfg {
    const char *name;
    size_t n;
    vector<int> bits;
    size_t special;
    uint64_t t;
    vector<size_t> ntt_primes;  // QP indices whose NTT tables are dumped
    vector<size_t> levels;      // data levels (Ql sizes) whose key-switch tables are dumped
};

static void dump_cfg(const Cfg &c) {
    auto mods = CoeffModulus::Create(c.n, c.bits);
    size_t nQP = mods.size(), nP = c.special, nQ = nQP - nP;
    int logn = get_power_of_two(c.n);
    std::printf("\"%s\":{", c.name);
    std::printf("\"n\":%zu,\"special\":%zu,", c.n, c.special);
    auto v = values(mods);
    arr("moduli", v.data(), v.size());
    vector<uint64_t> r0, r1, r2, roots;
    for (auto &m : mods) {
        r0.push_back(m.const_ratio()[0]);
        r1.push_back(m.const_ratio()[1]);
        r2.push_back(m.const_ratio()[2]);
    }
    arr("ratio0", r0.data(), r0.size());
    arr("ratio1", r1.data(), r1.size());
    arr("ratio2", r2.data(), r2.size());
    std::printf("\"ntt\":{");
    for (size_t k = 0; k < c.ntt_primes.size(); k++) {
        size_t i = c.ntt_primes[k];
        NTT t(logn, mods[i]);
        std::printf("\"%zu\":{\"root\":%llu,\"n_inv\":%llu,", i, (unsigned long long)t.get_root(),
                    (unsigned long long)t.inv_degree_modulo());
        arr("root_powers", t.get_from_root_powers().data(), c.n);
        arr("root_powers_shoup", t.get_from_root_powers_shoup().data(), c.n);
        arr("inv_root_powers", t.get_from_inv_root_powers().data(), c.n);
        arr("inv_root_powers_shoup", t.get_from_inv_root_powers_shoup().data(), c.n, true);
        std::printf("}%s", k + 1 < c.ntt_primes.size() ? "," : "");
    }
    std::printf("},");

    // hybrid key switching tables per data level (rns.cu:100-190)
    std::printf("\"ks\":{");
    vector<Modulus> modP(mods.begin() + nQ, mods.end());
    for (size_t li = 0; li < c.levels.size() && nP > 0; li++) {
        size_t l = c.levels[li];
        vector<Modulus> modQl(mods.begin(), mods.begin() + l);
        vector<Modulus> modQlP = modQl;
        modQlP.insert(modQlP.end(), modP.begin(), modP.end());
        size_t alpha = nP, beta = (l + alpha - 1) / alpha;
        std::printf("\"%zu\":{\"digits\":[", l);
        for (size_t d = 0; d < beta; d++) {
            size_t s = alpha * d, sz = d == beta - 1 ? l - alpha * (beta - 1) : alpha;
            vector<Modulus> part(modQlP.begin() + s, modQlP.begin() + s + sz);
            vector<Modulus> compl_ = modQlP;
            compl_.erase(compl_.begin() + s, compl_.begin() + s + sz);
            RNSBase bpart(part), bcompl(compl_);
            BaseConverter conv(bpart, bcompl);
            std::printf("{");
            arr("part_hat_inv", bpart.QHatInvModq(), sz);
            vector<uint64_t> mat;
            for (size_t j = 0; j < compl_.size(); j++)
                for (size_t i = 0; i < sz; i++) mat.push_back(conv.QHatModp(j)[i]);
            arr("matrix", mat.data(), mat.size(), true);
            std::printf("}%s", d + 1 < beta ? "," : "");
        }
        std::printf("],");
        RNSBase bP(modP), bQl(modQl);
        BaseConverter pconv(bP, bQl);
        arr("p_hat_inv", bP.QHatInvModq(), nP);
        vector<uint64_t> pmat, pinv;
        for (size_t j = 0; j < l; j++)
            for (size_t k = 0; k < nP; k++) pmat.push_back(pconv.QHatModp(j)[k]);
        vector<uint64_t> vP = values(modP);
        vector<uint64_t> bigP(nP, 0);
        multiply_many_uint64(vP.data(), nP, bigP.data());
        for (size_t j = 0; j < l; j++) {
            uint64_t tmp = modulo_uint(bigP.data(), nP, modQl[j]);
            uint64_t inv;
            try_invert_uint_mod(tmp, modQl[j], inv);
            pinv.push_back(inv);
        }
        arr("p_matrix", pmat.data(), pmat.size());
        arr("p_inv", pinv.data(), pinv.size(), true);
        std::printf("}%s", li + 1 < c.levels.size() ? "," : "");
    }
    std::printf("}");

    if (c.t) {
        // BFV HPS tables at the first data level (rns.cu:687-777)
        vector<Modulus> modQ(mods.begin(), mods.begin() + nQ);
        uint64_t minq = modQ[0].value();
        for (auto &m : modQ) minq = std::min(minq, m.value());
        size_t nR = nQ + 1, nQR = nQ + nR;
        auto modR = get_primes_below(c.n, minq, nR);
        RNSBase bQ(modQ), bR(modR);
        RNSBase bQR(bQ.extend(bR));
        Modulus t(c.t);
        auto bigR = bR.big_modulus();
        vector<double> frac(nQ);
        vector<uint64_t> modr(nR * (nQ + 1));
        vector<vector<uint64_t>> tRS(nQR);
        for (size_t i = 0; i < nQR; i++) {
            tRS[i].resize(nR + 2, 0);
            vector<uint64_t> tR(nR + 1, 0);
            multiply_uint(bigR, nR, t.value(), nR + 1, tR.data());
            multiply_uint(tR.data(), nR + 1, bQR.QHatInvModq()[i], nR + 2, tRS[i].data());
        }
        for (size_t i = 0; i < nQ; i++) {
            uint64_t m = modulo_uint(tRS[i].data(), nR + 2, modQ[i]);
            frac[i] = static_cast<double>(m) / static_cast<double>(modQ[i].value());
        }
        vector<vector<uint64_t>> tRSd(nQR);
        for (size_t i = 0; i < nQR; i++) {
            tRSd[i].resize(nR + 2, 0);
            vector<uint64_t> bs(nR + 2, 0), rem(nR + 2, 0);
            bs[0] = bQR.base()[i].value();
            divide_uint(tRS[i].data(), bs.data(), nR + 2, tRSd[i].data(), rem.data());
        }
        for (size_t j = 0; j < nR; j++) {
            for (size_t i = 0; i < nQ; i++) modr[j * (nQ + 1) + i] = modulo_uint(tRSd[i].data(), nR + 2, modR[j]);
            modr[j * (nQ + 1) + nQ] = modulo_uint(tRSd[nQ + j].data(), nR + 2, modR[j]);
        }
        std::printf(",\"hps\":{");
        auto vr = values(modR);
        arr("r_primes", vr.data(), vr.size());
        darr("frac", frac.data(), frac.size());
        arr("modr", modr.data(), modr.size());
        BaseConverter q2r(bQ, bR), r2q(bR, bQ);
        vector<uint64_t> m1, m2, a1, a2;
        for (size_t j = 0; j < nR; j++)
            for (size_t i = 0; i < nQ; i++) m1.push_back(q2r.QHatModp(j)[i]);
        for (size_t j = 0; j < nQ; j++)
            for (size_t i = 0; i < nR; i++) m2.push_back(r2q.QHatModp(j)[i]);
        for (size_t a = 0; a <= nQ; a++)
            for (size_t j = 0; j < nR; j++) a1.push_back(q2r.alphaQModp(a)[j]);
        for (size_t a = 0; a <= nR; a++)
            for (size_t j = 0; j < nQ; j++) a2.push_back(r2q.alphaQModp(a)[j]);
        arr("q_hat_inv", bQ.QHatInvModq(), nQ);
        arr("r_hat_inv", bR.QHatInvModq(), nR);
        darr("q_inv", bQ.inv(), nQ);
        darr("r_inv", bR.inv(), nR);
        arr("q2r_matrix", m1.data(), m1.size());
        arr("r2q_matrix", m2.data(), m2.size());
        arr("q2r_alpha", a1.data(), a1.size());
        arr("r2q_alpha", a2.data(), a2.size(), true);
        std::printf("}");
    }
    std::printf("}");
}

int main() {
    vector<int> c2bits{60};
    for (int i = 0; i < 29; i++) c2bits.push_back(40);
    for (int i = 0; i < 5; i++) c2bits.push_back(60);
    vector<int> c4bits;
    for (int i = 0; i < 16; i++) c4bits.push_back(50);
    c4bits.push_back(60);
    c4bits.push_back(60);
    vector<int> c5bits{60};
    for (int i = 0; i < 19; i++) c5bits.push_back(40);
    for (int i = 0; i < 4; i++) c5bits.push_back(60);
    vector<Cfg> cfgs = {
            {"ntt_4096_3x60", 4096, {60, 60, 60}, 0, 0, {0, 1, 2}, {}},
            {"ckks_small", 4096, {60, 40, 40, 40, 40, 40, 60, 60}, 2, 0, {0, 1, 5, 6, 7}, {6, 5, 3, 1}},
            {"bfv_small", 4096, {50, 50, 50, 50, 60, 60}, 2, 65537, {0, 4}, {4}},
            {"ckks_n16_l30_dnum6", 65536, c2bits, 5, 0, {0, 1, 29, 30, 34}, {30, 29, 17, 5}},
            {"bfv_n15_16x50", 32768, c4bits, 2, 65537, {0, 15, 16, 17}, {16}},
            {"ckks_n16_l20_dnum5", 65536, c5bits, 4, 0, {0, 23}, {20}},
    };
    std::printf("{");
    for (size_t i = 0; i < cfgs.size(); i++) {
        dump_cfg(cfgs[i]);
        if (i + 1 < cfgs.size()) std::printf(",");
    }
    std::printf("}\n");
    return 0;
}
