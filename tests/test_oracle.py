"""The CPU oracle pinned against the reference's own host tables and against exact
big-integer / algebraic identities.  CPU only."""
import hashlib

import numpy as np
import pytest

from oracle import oracle as O


def _sha(a):
    return hashlib.sha256(np.asarray(a, dtype=np.uint64).tobytes()).hexdigest()


def _check(golden, arr):
    if isinstance(golden, dict):
        assert golden["len"] == len(arr)
        assert _sha(arr) == golden["sha256"]
    else:
        assert [int(x) for x in arr] == golden


CFG_BITS = {
    "ntt_4096_3x60": (4096, [60, 60, 60]),
    "ckks_small": (4096, [60, 40, 40, 40, 40, 40, 60, 60]),
    "bfv_small": (4096, [50, 50, 50, 50, 60, 60]),
    "ckks_n16_l30_dnum6": (65536, [60] + [40] * 29 + [60] * 5),
    "bfv_n15_16x50": (32768, [50] * 16 + [60, 60]),
    "ckks_n16_l20_dnum5": (65536, [60] + [40] * 19 + [60] * 4),
}


@pytest.mark.parametrize("name", list(CFG_BITS))
def test_moduli_and_barrett_match_reference(golden_tables, name):
    n, bits = CFG_BITS[name]
    g = golden_tables[name]
    mods = O.create_coeff_modulus(n, bits)
    assert mods == g["moduli"]
    for i, q in enumerate(mods):
        r = O.barrett_ratio(q)
        assert r == [g["ratio0"][i], g["ratio1"][i], g["ratio2"][i]]


@pytest.mark.parametrize("name", list(CFG_BITS))
def test_ntt_tables_match_reference(golden_tables, name):
    n, bits = CFG_BITS[name]
    g = golden_tables[name]
    log_n = n.bit_length() - 1
    for idx, t in g["ntt"].items():
        q = g["moduli"][int(idx)]
        root, root_sh, iroot, iroot_sh, ninv = O.ntt_tables(log_n, q)
        assert O.minimal_root(2 * n, q) == t["root"]
        assert ninv == t["n_inv"]
        _check(t["root_powers"], root)
        _check(t["root_powers_shoup"], root_sh)
        _check(t["inv_root_powers"], iroot)
        _check(t["inv_root_powers_shoup"], iroot_sh)


@pytest.mark.parametrize("name", ["ckks_small", "bfv_small", "ckks_n16_l30_dnum6", "bfv_n15_16x50",
                                  "ckks_n16_l20_dnum5"])
def test_keyswitch_tables_match_reference(golden_tables, name):
    n, bits = CFG_BITS[name]
    g = golden_tables[name]
    n_p = g["special"]
    ctx = O.Context(4, g["moduli"], len(bits) - n_p, n_p)  # tables do not depend on N
    for l, kt in g["ks"].items():
        l = int(l)
        for d, dig in enumerate(kt["digits"]):
            phi, mat = ctx.modup_tables(l, d)
            _check(dig["part_hat_inv"], phi)
            _check(dig["matrix"], mat)
        phi, mat, pinv = ctx.moddown_tables(l)
        _check(kt["p_hat_inv"], phi)
        _check(kt["p_matrix"], mat)
        _check(kt["p_inv"], pinv)


@pytest.mark.parametrize("name", ["bfv_small", "bfv_n15_16x50"])
def test_hps_tables_match_reference(golden_tables, name):
    n, bits = CFG_BITS[name]
    g = golden_tables[name]
    n_p = g["special"]
    ctx = O.Context(n.bit_length() - 1, g["moduli"], len(bits) - n_p, n_p, 65537)
    h = g["hps"]
    assert ctx.r_moduli == h["r_primes"]
    frac, modr = ctx.hps_tables()
    assert [int(x) for x in frac.view(np.uint64)] == h["frac"]
    _check(h["modr"], modr)


def test_ntt_round_trip_constant_inputs():
    # The reference's own known-answer test: forward then inverse of a constant
    # polynomial returns it unchanged (test/ntt_test.cu:46-68, 102-121).
    n, bits = CFG_BITS["ntt_4096_3x60"]
    mods = O.create_coeff_modulus(n, bits)
    ctx = O.Context(12, mods, 3, 0)
    for const in (1, 2):
        a = np.full((3, n), const, dtype=np.uint64)
        b = ctx.ntt_inv(ctx.ntt_fwd(a))
        assert np.array_equal(a, b)


def _bitrev(x, bits):
    return int(format(x, f"0{bits}b")[::-1], 2)


def test_ntt_is_negacyclic_evaluation_in_bit_reversed_order():
    log_n, n = 6, 64
    q = O.create_coeff_modulus(4096, [60])[0]
    ctx = O.Context(log_n, [q], 1, 0)
    rng = np.random.default_rng(1)
    a = rng.integers(0, q, size=n, dtype=np.uint64)
    got = ctx.ntt_fwd(a)
    psi = O.minimal_root(2 * n, q)
    for k in range(n):
        e = 2 * _bitrev(k, log_n) + 1
        want = sum(int(a[j]) * pow(psi, e * j, q) for j in range(n)) % q
        assert int(got[k]) == want


def test_ntt_convolution_property():
    log_n, n = 8, 256
    q = O.create_coeff_modulus(4096, [60])[0]
    ctx = O.Context(log_n, [q], 1, 0)
    rng = np.random.default_rng(2)
    a = rng.integers(0, q, size=n, dtype=np.uint64)
    b = rng.integers(0, q, size=n, dtype=np.uint64)
    want = [0] * n
    for i in range(n):
        for j in range(n):
            k = i + j
            v = int(a[i]) * int(b[j])
            if k >= n:
                want[k - n] -= v
            else:
                want[k] += v
    want = np.array([w % q for w in want], dtype=np.uint64)
    fa, fb = ctx.ntt_fwd(a), ctx.ntt_fwd(b)
    prod = np.array([(int(x) * int(y)) % q for x, y in zip(fa, fb)], dtype=np.uint64)
    assert np.array_equal(ctx.ntt_inv(prod), want)


def _small_ckks():
    n, bits = CFG_BITS["ckks_small"]
    mods = O.create_coeff_modulus(n, bits)
    return O.Context(6, mods, 6, 2), mods  # N = 64 keeps the big-integer checks quick


def test_modup_base_conversion_is_exact_fast_bconv():
    ctx, mods = _small_ckks()
    n, l = ctx.n, 5
    rng = np.random.default_rng(3)
    c2 = O.random_residues(rng, mods[:l], n)[0]
    coeff = c2  # BFV flavour: c2 in coefficient form, then every digit is NTT'd
    tm = ctx.modup(l, coeff, scheme=1)
    qlp = ctx.qlp(l)
    tbl = [j if j < l else ctx.n_q + j - l for j in range(l + ctx.n_p)]
    for d in range(ctx.beta(l)):
        s, sz = 2 * d, min(2, l - 2 * d)
        digit = mods[s:s + sz]
        Qd = int(np.prod([int(x) for x in digit], dtype=object))
        back = ctx.ntt_inv(tm[d], tbl)
        for jj, p in enumerate(qlp):
            for k in range(0, n, 7):
                if s <= jj < s + sz:
                    assert int(back[jj, k]) == int(coeff[jj, k])
                    continue
                acc = 0
                for i, q in enumerate(digit):
                    qh = Qd // q
                    y = int(coeff[s + i, k]) * pow(qh % q, -1, q) % q
                    acc += y * qh
                assert int(back[jj, k]) == acc % p


def test_moddown_divides_multiples_of_p_exactly():
    ctx, mods = _small_ckks()
    n, l = ctx.n, 4
    P = int(mods[6]) * int(mods[7])
    rng = np.random.default_rng(4)
    x = O.random_residues(rng, mods[:l], n)[0]
    qlp = ctx.qlp(l)
    cx = np.zeros((l + 2, n), dtype=np.uint64)
    for j in range(l):
        cx[j] = np.array([int(v) * P % qlp[j] for v in x[j]], dtype=np.uint64)
    tbl = [j if j < l else ctx.n_q + j - l for j in range(l + 2)]
    out = ctx.moddown(l, ctx.ntt_fwd(cx, tbl), scheme=0)
    assert np.array_equal(ctx.ntt_inv(out, list(range(l))), x)


def test_rescale_divides_multiples_of_q_last_exactly():
    ctx, mods = _small_ckks()
    n, l = ctx.n, 5
    ql = int(mods[l - 1])
    rng = np.random.default_rng(5)
    small = rng.integers(-1000, 1000, size=n)
    x = np.array([[(int(v) * ql) % int(q) for v in small] for q in mods[:l]], dtype=np.uint64)
    out = ctx.rescale(l, ctx.ntt_fwd(x, list(range(l))))
    want = np.array([[int(v) % int(q) for v in small] for q in mods[: l - 1]], dtype=np.uint64)
    assert np.array_equal(ctx.ntt_inv(out[0], list(range(l - 1))), want)


def test_galois_ntt_permutation_matches_coefficient_automorphism():
    ctx, mods = _small_ckks()
    n = ctx.n
    rng = np.random.default_rng(6)
    a = O.random_residues(rng, mods[:3], n)[0]
    for step in (1, 2, -1, 5, 0):
        elt = O.elt_from_step(step, n)
        lhs = ctx.ntt_fwd(ctx.apply_galois_coeff(a, elt), [0, 1, 2])
        rhs = ctx.apply_galois_ntt(ctx.ntt_fwd(a, [0, 1, 2]), elt)
        assert np.array_equal(lhs, rhs)


def _keygen_evk(ctx, l_key, s_coeff, s_new_coeff, rng):
    """Hybrid key-switching key [dnum][2][QP][N] in NTT form: evk_d = (-(a_d s + e_d) +
    P*s_new on digit d's limbs, a_d), the layout of generate_one_kswitch_key
    (src/secretkey.cu:297-341)."""
    n, nq, n_p = ctx.n, ctx.n_q, ctx.n_p
    mods = ctx.moduli
    qp = len(mods)
    P = 1
    for p in mods[nq:]:
        P *= int(p)
    dnum = (nq + n_p - 1) // n_p
    s_ntt = ctx.ntt_fwd(np.array([[v % q for v in s_coeff] for q in mods], dtype=np.uint64))
    sn_ntt = ctx.ntt_fwd(np.array([[v % q for v in s_new_coeff] for q in mods], dtype=np.uint64))
    evk = np.zeros((dnum, 2, qp, n), dtype=np.uint64)
    for d in range(dnum):
        a = O.random_residues(rng, mods, n)[0]
        e = rng.integers(-3, 4, size=n)
        e_ntt = ctx.ntt_fwd(np.array([[int(v) % q for v in e] for q in mods], dtype=np.uint64))
        for j, q in enumerate(mods):
            q = int(q)
            b = (-(a[j].astype(object) * s_ntt[j].astype(object) + e_ntt[j].astype(object))) % q
            if d * n_p <= j < min((d + 1) * n_p, nq):
                b = (b + (P % q) * sn_ntt[j].astype(object)) % q
            evk[d, 0, j] = b.astype(np.uint64)
            evk[d, 1, j] = a[j]
    return evk


def _centered(v, q):
    v = int(v) % q
    return v - q if v > q // 2 else v


def test_keyswitch_decrypts_to_c2_times_new_secret():
    ctx, mods = _small_ckks()
    n, l = ctx.n, 5
    rng = np.random.default_rng(7)
    s = rng.integers(-1, 2, size=n)
    s2 = rng.integers(-1, 2, size=n)
    evk = _keygen_evk(ctx, l, s, s2, rng)
    c2 = O.random_residues(rng, mods[:l], n)[0]
    ks = ctx.keyswitch(l, np.zeros((2, l, n), dtype=np.uint64), c2, evk, scheme=0)
    tbl = list(range(l))
    s_ntt = ctx.ntt_fwd(np.array([[v % q for v in s] for q in mods[:l]], dtype=np.uint64), tbl)
    s2_ntt = ctx.ntt_fwd(np.array([[v % q for v in s2] for q in mods[:l]], dtype=np.uint64), tbl)
    diff = np.zeros((l, n), dtype=np.uint64)
    for j in range(l):
        q = int(mods[j])
        d = (ks[0, j].astype(object) + ks[1, j].astype(object) * s_ntt[j].astype(object)
             - c2[j].astype(object) * s2_ntt[j].astype(object)) % q
        diff[j] = d.astype(np.uint64)
    coeff = ctx.ntt_inv(diff, tbl)
    # The residual is the key-switching noise: small and the same integer in every limb.
    for k in range(n):
        vals = {_centered(coeff[j, k], int(mods[j])) for j in range(l)}
        assert len(vals) == 1
        assert abs(vals.pop()) < 2 ** 30


def test_hps_bconv_is_exact_centered_conversion():
    n, bits = CFG_BITS["bfv_small"]
    mods = O.create_coeff_modulus(n, bits)
    ctx = O.Context(6, mods, 4, 2, 65537)
    Q = 1
    for q in mods[:4]:
        Q *= int(q)
    rng = np.random.default_rng(8)
    xs = [int(rng.integers(0, 2 ** 62)) * int(rng.integers(0, 2 ** 62)) * int(rng.integers(0, 2 ** 62)) % Q
          for _ in range(ctx.n)]
    res = np.array([[x % int(q) for x in xs] for q in mods[:4]], dtype=np.uint64)
    out = ctx.hps_bconv_q_to_r(res)
    for k, x in enumerate(xs):
        c = x if x < Q // 2 else x - Q
        for j, r in enumerate(ctx.r_moduli):
            assert int(out[j, k]) == c % r
