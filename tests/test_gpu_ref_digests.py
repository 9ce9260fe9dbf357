"""The GPU library against PhantomFHE's own compiled kernels, with no oracle in between.

tests/golden/ref_kernels.json holds SHA-256 digests of the reference kernels' outputs on seeded
inputs (tests/golden/make_golden_kernels.py).  These tests draw the same inputs, run them through
this library's C ABI on the GPU (tensor-core and CUDA-core base conversions both), and compare
digests: NTT/iNTT, the CKKS key switch, rescale and the tensor product."""
import hashlib
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.json")
with open(GOLDEN) as _f:
    G = json.load(_f)


def sha(t):
    a = t.cpu().numpy().view(np.uint64) if isinstance(t, torch.Tensor) else t
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def pg():
    import phantom_gb300
    return phantom_gb300


@pytest.mark.parametrize("name", [k for k in G if k.startswith("ntt_")])
def test_ntt_digests(pg, name):
    g = G[name]
    n = 1 << g["log_n"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    ctx = pg.Context(n, mods, 1)
    x = O.random_residues(np.random.default_rng(g["seed"]), mods, n, 1)
    t = pg.to_device(x)
    ctx.ntt_forward(t, 1, len(mods))
    assert sha(t) == g["forward"]
    ctx.ntt_inverse(t, 1, len(mods))
    assert sha(t) == g["inverse_of_forward"]


@pytest.mark.parametrize("name", [k for k in G if k.startswith("ks_")])
def test_keyswitch_digests(pg, name):
    g = G[name]
    n = 1 << g["log_n"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"])
    ws = ctx.workspace()
    rng = np.random.default_rng(g["seed"])
    evk = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    key = pg.KeySwitchKey(pg.to_device(evk))
    for l in sorted((int(k) for k in g["levels"]), reverse=True):  # the generator's draw order
        ct = O.random_residues(rng, mods[:l], n, 2)
        c2 = O.random_residues(rng, mods[:l], n, 1)[0]
        for tc, fused in ((True, True), (False, True), (True, False)):
            ctx.tensor_cores, ctx.fused_keyswitch = tc, fused
            t = pg.to_device(ct)
            ctx.keyswitch(ws, t, pg.to_device(c2), nq - l + 1, key)
            assert sha(t) == g["levels"][str(l)]["keyswitch"], f"level {l}, tensor_cores={tc}, fused={fused}"
        assert ctx.device_status() == 0


def test_rescale_and_tensor_digests(pg):
    g = G["rescale_n12"]
    n, l = 1 << g["log_n"], g["l"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"])
    ws = ctx.workspace()
    ct = O.random_residues(np.random.default_rng(g["seed"]), mods[:l], n, 2)
    out = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
    ctx.rescale_to_next(ws, pg.to_device(ct), out, 2, nq - l + 1)
    assert sha(out) == g["rescale"]

    g = G["tensor_galois_n12"]
    l = g["l"]
    rng = np.random.default_rng(g["seed"])
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    t = torch.zeros((3, l, n), dtype=torch.int64, device="cuda")
    t[:2] = pg.to_device(a)
    ctx.ckks_multiply(t, pg.to_device(b), nq - l + 1)
    assert sha(t) == g["tensor"]


@pytest.mark.parametrize("name", [k for k in G if k.startswith("hmult_")])
def test_hmult_digests(pg, name):
    """The fused HMult + relinearise + rescale kernel chain and the two-call form give the
    reference's words (N=2^16, l=30, dnum=6 is the benchmark configuration)."""
    g = G[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"])
    ws = ctx.workspace()
    rng = np.random.default_rng(g["seed"])
    evk = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    key = pg.KeySwitchKey(pg.to_device(evk))
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    chain = nq - l + 1
    for tc, fused in ((True, True), (False, True), (True, False)):
        ctx.tensor_cores, ctx.fused_keyswitch = tc, fused
        out = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
        ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, chain, key)
        assert sha(out) == g["rescaled"], f"one call, tensor_cores={tc}, fused key switch={fused}"
        ta = pg.to_device(a)
        ctx.multiply_and_relin(ws, ta, pg.to_device(b), chain, key)
        assert sha(ta) == g["multiply_and_relin"], f"multiply_and_relin, tensor_cores={tc}, fused={fused}"
        out2 = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
        ctx.rescale_to_next(ws, ta, out2, 2, chain)
        assert sha(out2) == g["rescaled"], f"two calls, tensor_cores={tc}"
    assert ctx.device_status() == 0


@pytest.mark.parametrize("name", [k for k in G if k.startswith("bfv_")])
def test_bfv_mul_relin_digests(pg, name):
    g = G[name]
    n = 1 << g["log_n"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"], scheme=pg.SCHEME_BFV, plain_modulus=g["t"])
    ws = ctx.workspace()
    rng = np.random.default_rng(g["seed"])
    evk = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    key = pg.KeySwitchKey(pg.to_device(evk))
    a = O.random_residues(rng, mods[:nq], n, 2)
    b = O.random_residues(rng, mods[:nq], n, 2)
    for tc in (True, False):
        ctx.tensor_cores = tc
        ta = pg.to_device(a)
        ctx.multiply_and_relin(ws, ta, pg.to_device(b), 1, key)
        assert sha(ta) == g["mul_relin"], f"tensor_cores={tc}"
    assert ctx.device_status() == 0


@pytest.mark.parametrize("name", [k for k in G if k.startswith("prng_")])
def test_samplers_and_seeded_keygen_digests(pg, name):
    """The same seeds give the reference's polynomials and keys word for word."""
    g = G[name]
    n = 1 << g["log_n"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    qp = len(g["bits"])
    ctx = pg.Context(n, mods, g["special"])
    ws = ctx.workspace()
    sd = {k: bytes.fromhex(v) for k, v in g["seeds"].items() if isinstance(v, str)}
    u = torch.empty((qp, n), dtype=torch.int64, device="cuda")
    ctx.sample_uniform(sd["uniform"], qp, u)
    assert sha(u) == g["uniform"]
    small = torch.empty(n, dtype=torch.int64, device="cuda")

    def residues(t):
        v = t.cpu().numpy()
        return np.stack([np.where(v < 0, np.uint64(q) - (-v).astype(np.uint64), v.astype(np.uint64)) for q in mods])

    ctx.sample_ternary(sd["ternary"], small)
    assert sha(residues(small)) == g["ternary"]
    ctx.sample_cbd(sd["error"], small)
    assert sha(residues(small)) == g["error"]
    s = torch.empty((qp, n), dtype=torch.int64, device="cuda")
    ctx.secret_key_from_seed(ws, sd["secret"], s)
    assert sha(s) == g["secret_key"]
    key = torch.empty((ctx.dnum, 2, qp, n), dtype=torch.int64, device="cuda")
    ctx.kswitch_keygen_seeded(ws, 0, s, b"".join(bytes.fromhex(h) for h in g["seeds"]["a"]),
                              b"".join(bytes.fromhex(h) for h in g["seeds"]["e"]), key)
    assert sha(key) == g["relin_key"]
    assert ctx.device_status() == 0


@pytest.mark.parametrize("name", [k for k in G if k.startswith("bfvio_")])
def test_bfv_encode_encrypt_decrypt_digests(pg, name):
    """Batch encoding, symmetric encryption (the reference's samplers) and HPS decryption give the
    reference's words; the parameter sets cover its four decryption variants."""
    g = G[name]
    n = 1 << g["log_n"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq, qp, t = len(g["bits"]) - g["special"], len(g["bits"]), g["t"]
    ctx = pg.Context(n, mods, g["special"], scheme=pg.SCHEME_BFV, plain_modulus=t)
    ws = ctx.workspace()
    rng = np.random.default_rng(g["seed"])
    values = rng.integers(0, t, size=n, dtype=np.uint64)
    sd = dict(zip(("secret", "a", "e"), (rng.bytes(64) for _ in range(3))))  # the generator's draw order
    assert all(sd[k] == bytes.fromhex(v) for k, v in g["seeds"].items())
    pt = torch.empty(n, dtype=torch.int64, device="cuda")
    ctx.bfv_encode(pg.to_device(values), pt)
    assert sha(pt) == g["encode"]
    back = torch.empty(n, dtype=torch.int64, device="cuda")
    ctx.bfv_decode(ws, pt, back)
    assert np.array_equal(back.cpu().numpy().view(np.uint64), values)
    s = torch.empty((qp, n), dtype=torch.int64, device="cuda")
    ctx.secret_key_from_seed(ws, sd["secret"], s)
    a = torch.empty((nq, n), dtype=torch.int64, device="cuda")
    ctx.sample_uniform(sd["a"], nq, a)
    e = torch.empty(n, dtype=torch.int64, device="cuda")
    ctx.sample_cbd(sd["e"], e)
    ct = torch.empty((2, nq, n), dtype=torch.int64, device="cuda")
    ctx.bfv_encrypt_symmetric(pt, s, a, e, ct)
    assert sha(ct) == g["encrypt"]
    m = torch.empty(n, dtype=torch.int64, device="cuda")
    ctx.bfv_decrypt(ws, ct, 1, s, m)
    assert torch.equal(m, pt), "decryption of the encryption"
    rnd = pg.to_device(O.random_residues(rng, mods[:nq], n, 2))
    ctx.bfv_decrypt(ws, rnd, 1, s, m)
    assert sha(m) == g["decrypt_random"], f"decryption of random words ({g['decrypt_variant']} variant)"


@pytest.mark.parametrize("name", [k for k in G if k.startswith("rotate_")])
def test_rotate_digests(pg, name):
    """HRotate (apply_galois_inplace with the step's Galois key) gives the reference's words."""
    g = G[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"], galois_elts=[g["elt"]])
    ws = ctx.workspace()
    rng = np.random.default_rng(g["seed"])
    gk = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    key = pg.KeySwitchKey(pg.to_device(gk))
    ct = O.random_residues(rng, mods[:l], n, 2)
    for tc, fused in ((True, True), (False, True), (True, False)):
        ctx.tensor_cores, ctx.fused_keyswitch = tc, fused
        t = pg.to_device(ct)
        ctx.apply_galois(ws, t, nq - l + 1, g["elt"], key)
        assert sha(t) == g["rotate"], f"tensor_cores={tc}, fused={fused}"
    assert ctx.device_status() == 0


@pytest.mark.parametrize("name", [k for k in G if k.startswith("hoist_")])
def test_hoisting_digests(pg, name):
    """hoisting_inplace (one mod-up of c1, per-step permuted inner products summed, one mod-down)
    gives the reference's words, with the tensor-core and the CUDA-core conversions."""
    g = G[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"], galois_elts=g["elts"])
    ws = ctx.workspace()
    rng = np.random.default_rng(g["seed"])
    keys = [O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n) for _ in g["steps"]]
    gks = [None] * len(ctx.galois_elts)
    for e, k in zip(g["elts"], keys):
        gks[ctx.galois_elts.index(e)] = pg.KeySwitchKey(pg.to_device(k))
    ct = O.random_residues(rng, mods[:l], n, 2)
    for tc in (True, False):
        ctx.tensor_cores = tc
        t = pg.to_device(ct)
        ctx.hoisting(ws, t, nq - l + 1, g["steps"], gks)
        assert sha(t) == g["hoisting"], f"tensor_cores={tc}"
    assert ctx.device_status() == 0


@pytest.mark.parametrize("name", [k for k in G if k.startswith("modswitch_bfv_")])
def test_bfv_mod_switch_digests(pg, name):
    """BFV mod_switch_to_next (divide_and_round_q_last in the coefficient domain)."""
    g = G[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"], scheme=pg.SCHEME_BFV, plain_modulus=g["t"])
    ct = O.random_residues(np.random.default_rng(g["seed"]), mods[:l], n, 2)
    out = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
    ctx.bfv_mod_switch_to_next(pg.to_device(ct), out, 2, nq - l + 1)
    assert sha(out) == g["mod_switch"]


def _unit_disk(rng, count):
    r, th = np.sqrt(rng.uniform(0, 1, count)), 2 * np.pi * rng.uniform(0, 1, count)
    return r * np.cos(th) + 1j * r * np.sin(th)


@pytest.mark.parametrize("name", [k for k in G if k.startswith("codec_")])
def test_ckks_encoder_digests(pg, name):
    """The CKKS encoder (FP64 special FFT, rounding, residues, NTT) and decoder (inverse NTT, CRT
    compose over every limb, FP64 special FFT) give the reference's plaintext words and the
    reference's decoded doubles, bit for bit; decoding uniform random residues exercises both
    halves of the compose's centring."""
    g = G[name]
    n, l = 1 << g["log_n"], g["l"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    nq = len(g["bits"]) - g["special"]
    ctx = pg.Context(n, mods, g["special"])
    ws = ctx.workspace()
    chain = nq - l + 1
    rng = np.random.default_rng(g["seed"])
    vals = _unit_disk(rng, g["count"])
    vt = torch.from_numpy(np.stack([vals.real, vals.imag], axis=1).copy()).cuda()
    pt = torch.empty((l, n), dtype=torch.int64, device="cuda")
    ctx.ckks_encode(ws, vt, g["scale"], chain, pt)
    assert sha(pt) == g["encode"], "encode"
    out = torch.empty((n // 2, 2), dtype=torch.float64, device="cuda")
    ctx.ckks_decode(ws, pt, g["scale"], chain, out)
    assert sha(out.cpu().numpy().view(np.uint64)) == g["decode"], "decode of the encoding"
    rnd = pg.to_device(O.random_residues(rng, mods[:l], n, 1))
    ctx.ckks_decode(ws, rnd, g["scale"], chain, out)
    assert sha(out.cpu().numpy().view(np.uint64)) == g["decode_random"], "decode of random residues"
