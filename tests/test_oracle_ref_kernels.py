"""The oracle against PhantomFHE's own CUDA kernels.

tests/golden/ref_kernels.json holds SHA-256 digests of the reference kernels' outputs
(tests/golden/make_golden_kernels.py replays the reference's launch sequences on a GPU, from
seeded inputs).  Each test regenerates the same inputs and checks that the oracle produces the
same words: NTT/iNTT, the CKKS key switch step by step (mod-up, inner product, mod-down +
add), rescale, the tensor product, the Galois permutation, and the BFV HPS conversions with
their FP64 corrections.  CPU only."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.json")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def _cases(prefix):
    with open(GOLDEN) as f:
        return [k for k in json.load(f) if k.startswith(prefix)]


@pytest.mark.parametrize("name", _cases("ntt_"))
def test_ntt_matches_reference_kernels(golden, name):
    g = golden[name]
    n = 1 << g["log_n"]
    mods = O.create_coeff_modulus(n, g["bits"])
    oc = O.Context(g["log_n"], mods, len(mods) - 1, 1)
    x = O.random_residues(np.random.default_rng(g["seed"]), mods, n, 1)[0]
    y = oc.ntt_fwd(x)
    assert sha(y) == g["forward"], "forward NTT"
    z = oc.ntt_inv(y)
    assert sha(z) == g["inverse_of_forward"] and np.array_equal(x, z)


@pytest.mark.parametrize("name", _cases("ks_"))
def test_keyswitch_matches_reference_kernels(golden, name):
    g = golden[name]
    n = 1 << g["log_n"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    oc = O.Context(g["log_n"], mods, nq, g["special"])
    rng = np.random.default_rng(g["seed"])
    dnum = -(-nq // g["special"])
    evk = O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)
    for l in sorted((int(k) for k in g["levels"]), reverse=True):  # the generator's draw order
        want = g["levels"][str(l)]
        ct = O.random_residues(rng, mods[:l], n, 2)
        c2 = O.random_residues(rng, mods[:l], n, 1)[0]
        tm = oc.modup(l, c2)
        assert sha(tm) == want["modup"], f"level {l}: mod-up"
        assert sha(oc.inner_product(l, tm, evk)) == want["inner_product"], f"level {l}: inner product"
        assert sha(oc.keyswitch(l, ct, c2, evk)) == want["keyswitch"], f"level {l}: key switch"


def test_rescale_matches_reference_kernels(golden):
    g = golden["rescale_n12"]
    n = 1 << g["log_n"]
    mods = O.create_coeff_modulus(n, g["bits"])
    oc = O.Context(g["log_n"], mods, len(mods) - g["special"], g["special"])
    ct = O.random_residues(np.random.default_rng(g["seed"]), mods[:g["l"]], n, 2)
    assert sha(oc.rescale(g["l"], ct)) == g["rescale"]


def test_tensor_and_galois_match_reference_kernels(golden):
    g = golden["tensor_galois_n12"]
    n, l = 1 << g["log_n"], g["l"]
    mods = O.create_coeff_modulus(n, g["bits"])
    oc = O.Context(g["log_n"], mods, len(mods) - g["special"], g["special"])
    rng = np.random.default_rng(g["seed"])
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    assert sha(oc.tensor(l, a, b)) == g["tensor"]
    x = O.random_residues(rng, mods[:l], n, 1)[0]
    for step, want in g["galois"].items():
        elt = O.elt_from_step(int(step), n)
        assert elt == want["elt"]
        assert sha(oc.apply_galois_ntt(x, elt)) == want["sha"], f"step {step}"


@pytest.mark.parametrize("name", _cases("hps_"))
def test_hps_matches_reference_kernels(golden, name):
    """FP64 corrections included: llround(sum y_i / q_i) in the Q -> R conversion and
    0.5 + sum x_i frac_i in scale-and-round, against the reference's compiled kernels."""
    g = golden[name]
    n = 1 << g["log_n"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    oc = O.Context(g["log_n"], mods, nq, g["special"], g["t"])
    rng = np.random.default_rng(g["seed"])
    x = O.random_residues(rng, mods[:nq], n, 1)[0]
    assert sha(oc.hps_bconv_q_to_r(x)) == g["bconv_q_to_r"]
    xr = O.random_residues(rng, list(mods[:nq]) + list(oc.r_moduli), n, 1)[0]
    assert sha(oc.hps_scale_round_qr_r(xr)) == g["scale_round_qr_r"]


@pytest.mark.parametrize("name", _cases("hmult_"))
def test_hmult_matches_reference_kernels(golden, name):
    """multiply_and_relin_inplace + rescale_to_next as the reference runs them (tensor product,
    key switch of the third polynomial, rescale), including N=2^16 at l=30 with dnum=6."""
    g = golden[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    oc = O.Context(g["log_n"], mods, nq, g["special"])
    rng = np.random.default_rng(g["seed"])
    dnum = -(-nq // g["special"])
    evk = O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    relin = oc.ckks_mul_relin(l, a, b, evk)
    assert sha(relin) == g["multiply_and_relin"]
    assert sha(oc.rescale(l, relin)) == g["rescaled"]


@pytest.mark.parametrize("name", _cases("bfv_"))
def test_bfv_mul_relin_matches_reference_kernels(golden, name):
    """The whole bfv_mul_relin_hps sequence (HPS conversions with FP64 corrections, NTTs over
    QlRl, tensor, scale-and-round, key switch in coefficient form) as the reference runs it."""
    g = golden[name]
    n = 1 << g["log_n"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    oc = O.Context(g["log_n"], mods, nq, g["special"], g["t"])
    rng = np.random.default_rng(g["seed"])
    dnum = -(-nq // g["special"])
    evk = O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)
    a = O.random_residues(rng, mods[:nq], n, 2)
    b = O.random_residues(rng, mods[:nq], n, 2)
    assert sha(oc.bfv_mul_relin_hps(a, b, evk)) == g["mul_relin"]


def _residues(v, mods, n):
    """Signed small polynomial -> [len(mods)][N] residues (as the reference's samplers store it)."""
    return np.stack([np.where(v < 0, np.uint64(q) - (-v).astype(np.uint64), v.astype(np.uint64)) for q in mods])


@pytest.mark.parametrize("name", _cases("prng_"))
def test_samplers_and_seeded_keygen_match_reference_kernels(golden, name):
    """The reference's Salsa20-based samplers (uniform with its rejection rule, ternary, centred
    binomial) and its seeded secret/relinearisation key generation."""
    g = golden[name]
    n = 1 << g["log_n"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq, qp = len(g["bits"]) - g["special"], len(g["bits"])
    oc = O.Context(g["log_n"], mods, nq, g["special"])
    sd = {k: bytes.fromhex(v) for k, v in g["seeds"].items() if isinstance(v, str)}
    assert sha(oc.sample_uniform(sd["uniform"], qp)) == g["uniform"]
    assert sha(_residues(oc.sample_small(sd["ternary"], 0), mods, n)) == g["ternary"]
    assert sha(_residues(oc.sample_small(sd["error"], 1), mods, n)) == g["error"]
    s = oc.ntt_fwd(_residues(oc.sample_small(sd["secret"], 0), mods, n))
    assert sha(s) == g["secret_key"]
    s2 = np.array([[int(x) * int(x) % q for x in row] for row, q in zip(s, mods)], dtype=np.uint64)
    a = np.stack([oc.sample_uniform(bytes.fromhex(h), qp) for h in g["seeds"]["a"]])
    e = np.stack([oc.ntt_fwd(_residues(oc.sample_small(bytes.fromhex(h), 1), mods, n)) for h in g["seeds"]["e"]])
    assert sha(oc.kswitch_key_combine(s, s2, a, e)) == g["relin_key"]


@pytest.mark.parametrize("name", _cases("rotate_"))
def test_rotate_matches_reference_kernels(golden, name):
    g = golden[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    oc = O.Context(g["log_n"], mods, nq, g["special"])
    rng = np.random.default_rng(g["seed"])
    dnum = -(-nq // g["special"])
    gk = O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)
    ct = O.random_residues(rng, mods[:l], n, 2)
    assert O.elt_from_step(g["step"], n) == g["elt"]
    assert sha(oc.ckks_apply_galois(l, ct, g["elt"], gk)) == g["rotate"]


@pytest.mark.parametrize("name", _cases("hoist_"))
def test_hoisting_matches_reference_kernels(golden, name):
    g = golden[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    oc = O.Context(g["log_n"], mods, nq, g["special"])
    rng = np.random.default_rng(g["seed"])
    dnum = -(-nq // g["special"])
    keys = [O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n) for _ in g["steps"]]
    ct = O.random_residues(rng, mods[:l], n, 2)
    assert [O.elt_from_step(s, n) for s in g["steps"]] == g["elts"]
    assert sha(oc.ckks_hoisting(l, ct, g["elts"], keys)) == g["hoisting"]


@pytest.mark.parametrize("name", _cases("modswitch_bfv_"))
def test_bfv_mod_switch_matches_reference_kernels(golden, name):
    g = golden[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = O.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    oc = O.Context(g["log_n"], mods, nq, g["special"], g["t"])
    ct = O.random_residues(np.random.default_rng(g["seed"]), mods[:l], n, 2)
    assert sha(oc.divide_round_q_last(l, ct)) == g["mod_switch"]
