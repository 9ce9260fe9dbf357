"""GPU library vs the CPU oracle, word for word, through the C ABI (sm_103a).

Inputs are seeded uniform residues; keys are uniform residues of the key layout
[dnum][2][QP][N] (parity does not need well-formed keys — tests/test_oracle.py checks the
key-switch algebra with real keys)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def pg():
    import phantom_gb300
    return phantom_gb300


def _ckks(pg, n, bits, special, galois_elts=None):
    mods = pg.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    ctx = pg.Context(n, mods, special, galois_elts=galois_elts)
    oc = O.Context(n.bit_length() - 1, mods, nq, special)
    return ctx, oc, mods, nq


@pytest.fixture(scope="module")
def small(pg):
    ctx, oc, mods, nq = _ckks(pg, 4096, [60, 40, 40, 40, 40, 40, 60, 60], 2)
    return ctx, oc, mods, nq, ctx.workspace()


def _key(rng, mods, dnum, n):
    return O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)


def _eq(got_t, want, what):
    got = got_t if isinstance(got_t, np.ndarray) else got_t.cpu().numpy().view(np.uint64)
    want = np.asarray(want, dtype=np.uint64).reshape(got.shape)
    bad = int((got != want).sum())
    assert bad == 0, f"{what}: {bad} of {got.size} words differ"


@pytest.mark.parametrize("log_n", [12, 13, 14, 15, 16, 17])
def test_ntt_matches_oracle_all_degrees(pg, log_n):
    n = 1 << log_n
    mods = pg.create_coeff_modulus(n, [60, 50, 40])
    ctx = pg.Context(n, mods, 1)
    oc = O.Context(log_n, mods, 2, 1)
    rng = np.random.default_rng(log_n)
    a = O.random_residues(rng, mods, n, 2)
    t = pg.to_device(a)
    ctx.ntt_forward(t, 2, 3, 0)
    want = np.stack([oc.ntt_fwd(a[p]) for p in range(2)])
    _eq(t, want, "forward NTT")
    ctx.ntt_inverse(t, 2, 3, 0)
    _eq(t, a, "inverse NTT round trip")
    b = pg.to_device(want)
    ctx.ntt_inverse(b, 2, 3, 0)
    _eq(b, a, "inverse NTT")


def test_ntt_start_index_and_constant_inputs(small, pg):
    ctx, oc, mods, nq, ws = small
    n = ctx.n
    for const in (1, 2):  # the reference's own round-trip test (test/ntt_test.cu:102-121)
        a = np.full((1, 3, n), const, dtype=np.uint64)
        t = pg.to_device(a)
        ctx.ntt_forward(t, 1, 3, 4)
        _eq(t, oc.ntt_fwd(a[0], [4, 5, 6]), "forward NTT from start index 4")
        ctx.ntt_inverse(t, 1, 3, 4)
        _eq(t, a, "round trip")


def _primes_below_2_61(n, count, bits=61):
    """The largest primes q = 1 mod 2n below 2^bits (deterministic Miller-Rabin for 64 bits)."""
    def is_prime(q):
        d, s = q - 1, 0
        while d % 2 == 0:
            d, s = d // 2, s + 1
        for a in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
            x = pow(a, d, q)
            if x in (1, q - 1):
                continue
            for _ in range(s - 1):
                x = x * x % q
                if x == q - 1:
                    break
            else:
                return False
        return True
    out, q = [], ((1 << bits) - 1) // (2 * n) * (2 * n) + 1
    while len(out) < count:
        if q < (1 << bits) and is_prime(q):
            out.append(q)
        q -= 2 * n
    return out


@pytest.mark.parametrize("small_launch", [-1, 0])
@pytest.mark.parametrize("log_n,bits", [(14, 61), (14, 57), (17, 57), (14, 44), (17, 44)])
def test_ntt_lazy_inputs_at_range_limits(pg, small_launch, log_n, bits):
    """Inside a transform the butterflies keep values in [0, 8q) (forward) and [0, 4q) (inverse)
    with a truncated-quotient Shoup product; producers fused into the passes hand over values in
    those ranges.  Below 2^57 the forward butterflies drop their conditional subtraction (the
    range grows by 4q a stage), below 2^44 the inverse ones too (the sums double a stage).  The
    largest primes of each class (just below 2^61, 2^57 and 2^44), the deepest transforms
    (N = 2^17) and inputs up to 8q - 1 / 4q - 1 put every bound at its edge; the outputs must
    still be the canonical transform."""
    n = 1 << log_n
    mods = _primes_below_2_61(n, 3, bits)
    ctx = pg.Context(n, mods, 1)
    ctx.ntt_small_launch = small_launch  # both the 8- and the 16-coefficient-per-thread passes
    oc = O.Context(log_n, mods, 2, 1)
    rng = np.random.default_rng(61)
    a = O.random_residues(rng, mods, n, 2)
    q = np.array(mods, dtype=np.uint64).reshape(1, 3, 1)
    k = rng.integers(0, 8, size=a.shape, dtype=np.uint64)
    k[..., :64] = 7  # the top of the range
    lazy = a + k * q
    assert int(lazy.max()) < (1 << 64)
    t = pg.to_device(lazy)
    ctx.ntt_forward(t, 2, 3, 0)
    want = np.stack([oc.ntt_fwd(a[p]) for p in range(2)])
    _eq(t, want, "forward NTT of inputs in [0, 8q)")
    k4 = rng.integers(0, 4, size=a.shape, dtype=np.uint64)
    k4[..., :64] = 3
    b = pg.to_device(want + k4 * q)
    ctx.ntt_inverse(b, 2, 3, 0)
    _eq(b, a, "inverse NTT of inputs in [0, 4q)")


def test_tensor(small, pg):
    ctx, oc, mods, nq, ws = small
    rng = np.random.default_rng(1)
    for chain in (1, 3):
        l = ctx.level(chain)
        a = O.random_residues(rng, mods[:l], ctx.n, 2)
        b = O.random_residues(rng, mods[:l], ctx.n, 2)
        t1 = torch.zeros((3, l, ctx.n), dtype=torch.int64, device="cuda")
        t1[:2] = pg.to_device(a)
        ctx.ckks_multiply(t1, pg.to_device(b), chain)
        _eq(t1, oc.tensor(l, a, b), "tensor")
        t2 = torch.zeros((3, l, ctx.n), dtype=torch.int64, device="cuda")
        t2[:2] = pg.to_device(a)
        ctx.ckks_multiply(t2, t2, chain)
        _eq(t2, oc.tensor(l, a, a), "square")


@pytest.mark.parametrize("chain", [1, 2, 3, 4, 5, 6])
def test_keyswitch_every_level(small, pg, chain):
    ctx, oc, mods, nq, ws = small
    l = ctx.level(chain)
    rng = np.random.default_rng(10 + chain)
    ct = O.random_residues(rng, mods[:l], ctx.n, 2)
    c2 = O.random_residues(rng, mods[:l], ctx.n, 1)[0]
    key = _key(rng, mods, ctx.dnum, ctx.n)
    t = pg.to_device(ct)
    ctx.keyswitch(ws, t, pg.to_device(c2), chain, pg.KeySwitchKey(pg.to_device(key)))
    _eq(t, oc.keyswitch(l, ct, c2, key), f"keyswitch chain {chain}")


def test_relinearize_and_multiply_and_relin(small, pg):
    ctx, oc, mods, nq, ws = small
    rng = np.random.default_rng(20)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    k = pg.KeySwitchKey(pg.to_device(key))
    for chain in (1, 4):
        l = ctx.level(chain)
        ct3 = O.random_residues(rng, mods[:l], ctx.n, 3)
        t = pg.to_device(ct3)
        ctx.relinearize(ws, t, chain, k)
        _eq(t[:2], oc.relinearize(l, ct3, key), "relinearize")
        a = O.random_residues(rng, mods[:l], ctx.n, 2)
        b = O.random_residues(rng, mods[:l], ctx.n, 2)
        ta = pg.to_device(a)
        ctx.multiply_and_relin(ws, ta, pg.to_device(b), chain, k)
        _eq(ta, oc.ckks_mul_relin(l, a, b, key), "multiply_and_relin")
        ts = pg.to_device(a)
        ctx.multiply_and_relin(ws, ts, ts, chain, k)
        _eq(ts, oc.ckks_mul_relin(l, a, a, key), "square_and_relin")


def test_rescale(small, pg):
    ctx, oc, mods, nq, ws = small
    rng = np.random.default_rng(30)
    for chain, size in ((1, 2), (2, 3), (5, 2)):
        l = ctx.level(chain)
        ct = O.random_residues(rng, mods[:l], ctx.n, size)
        out = torch.empty((size, l - 1, ctx.n), dtype=torch.int64, device="cuda")
        ctx.rescale_to_next(ws, pg.to_device(ct), out, size, chain)
        _eq(out, oc.rescale(l, ct), f"rescale chain {chain}")


def test_multiply_relin_rescale_fused_equals_sequence(small, pg):
    ctx, oc, mods, nq, ws = small
    rng = np.random.default_rng(40)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    k = pg.KeySwitchKey(pg.to_device(key))
    for chain in (1, 3, 5):
        l = ctx.level(chain)
        a = O.random_residues(rng, mods[:l], ctx.n, 2)
        b = O.random_residues(rng, mods[:l], ctx.n, 2)
        out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
        ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, chain, k)
        want = oc.rescale(l, oc.ckks_mul_relin(l, a, b, key))
        _eq(out, want, "fused multiply+relin+rescale vs oracle")
        ta = pg.to_device(a)
        ctx.multiply_and_relin(ws, ta, pg.to_device(b), chain, k)
        out2 = torch.empty_like(out)
        ctx.rescale_to_next(ws, ta, out2, 2, chain)
        assert torch.equal(out, out2)


def test_multiply_relin_rescale_squaring(small, pg):
    """ct1 and ct2 the same buffer (the reference's multiply_and_relin_inplace(ct, ct)), down to
    the lowest level that can still rescale (l = 2 -> 1)."""
    ctx, oc, mods, nq, ws = small
    rng = np.random.default_rng(41)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    k = pg.KeySwitchKey(pg.to_device(key))
    for chain in (1, nq - 1):
        l = ctx.level(chain)
        a = O.random_residues(rng, mods[:l], ctx.n, 2)
        ta = pg.to_device(a)
        out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
        ctx.multiply_relin_rescale(ws, ta, ta, out, chain, k)
        _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, a, key)), f"fused square chain {chain}")
        _eq(ta, a, "inputs untouched")


def test_apply_galois_rotate_and_naf(small, pg):
    ctx, oc, mods, nq, ws = small
    rng = np.random.default_rng(50)
    keys = [_key(rng, mods, ctx.dnum, ctx.n) for _ in ctx.galois_elts]
    gks = [pg.KeySwitchKey(pg.to_device(k)) for k in keys]
    for chain in (1, 3):
        l = ctx.level(chain)
        ct = O.random_residues(rng, mods[:l], ctx.n, 2)
        for step in (1, -1, 2, 0):
            elt = pg.elt_from_step(step, ctx.n)
            idx = ctx.galois_elts.index(elt)
            t = pg.to_device(ct)
            ctx.rotate(ws, t, chain, step, gks)
            _eq(t, oc.ckks_apply_galois(l, ct, elt, keys[idx]), f"rotate {step}")
        # step 3 has no key: NAF 3 = 4 - 1 applies the -1 then the 4 rotation
        t = pg.to_device(ct)
        ctx.rotate(ws, t, chain, 3, gks)
        want = ct
        for s in (-1, 4):
            elt = pg.elt_from_step(s, ctx.n)
            want = oc.ckks_apply_galois(l, want, elt, keys[ctx.galois_elts.index(elt)])
        _eq(t, want, "rotate 3 through NAF")


def test_hoisting(small, pg):
    ctx, oc, mods, nq, ws = small
    rng = np.random.default_rng(60)
    keys = [_key(rng, mods, ctx.dnum, ctx.n) for _ in ctx.galois_elts]
    gks = [pg.KeySwitchKey(pg.to_device(k)) for k in keys]
    steps = [1, 2, 4, -1]
    for chain in (1, 2):
        l = ctx.level(chain)
        ct = O.random_residues(rng, mods[:l], ctx.n, 2)
        t = pg.to_device(ct)
        ctx.hoisting(ws, t, chain, steps, gks)
        elts = [pg.elt_from_step(s, ctx.n) for s in steps]
        want = oc.ckks_hoisting(l, ct, elts, [keys[ctx.galois_elts.index(e)] for e in elts])
        _eq(t, want, "hoisting")


def test_errors_are_reported_not_crashed(small, pg):
    ctx, oc, mods, nq, ws = small
    t = torch.zeros((2, nq, ctx.n), dtype=torch.int64, device="cuda")
    with pytest.raises(pg.InvalidArgument):
        ctx.rescale_to_next(ws, t, t, 2, nq)  # chain index nq has one limb: end of chain
    with pytest.raises(pg.InvalidArgument):
        ctx.ckks_multiply(t, t, 0)  # key level is not a data level
    with pytest.raises(pg.FheError):
        ctx.bfv_mod_switch_to_next(t, t, 2, 1)
    with pytest.raises(pg.InvalidArgument):
        pg.Context(4096, [97, 193], 1)  # not NTT-friendly for N = 4096


# ---------------------------------------------------------------- BFV (HPS)

@pytest.fixture(scope="module")
def bfv_small(pg):
    n, bits, special = 4096, [50, 50, 50, 50, 60, 60], 2
    mods = pg.create_coeff_modulus(n, bits)
    ctx = pg.Context(n, mods, special, scheme=pg.SCHEME_BFV, plain_modulus=65537)
    oc = O.Context(12, mods, 4, special, 65537)
    assert ctx.moduli[6:] == oc.r_moduli
    return ctx, oc, mods, 4, ctx.workspace()


def test_bfv_mul_relin_hps(bfv_small, pg):
    ctx, oc, mods, nq, ws = bfv_small
    rng = np.random.default_rng(70)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    k = pg.KeySwitchKey(pg.to_device(key))
    a = O.random_residues(rng, mods[:nq], ctx.n, 2)
    b = O.random_residues(rng, mods[:nq], ctx.n, 2)
    ta = pg.to_device(a)
    ctx.multiply_and_relin(ws, ta, pg.to_device(b), 1, k)
    _eq(ta, oc.bfv_mul_relin_hps(a, b, key), "BFV HPS multiply_and_relin")
    ts = pg.to_device(a)
    ctx.multiply_and_relin(ws, ts, ts, 1, k)
    _eq(ts, oc.bfv_mul_relin_hps(a, a, key), "BFV HPS square_and_relin")


def test_bfv_keyswitch_and_mod_switch(bfv_small, pg):
    ctx, oc, mods, nq, ws = bfv_small
    rng = np.random.default_rng(71)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    ct = O.random_residues(rng, mods[:nq], ctx.n, 2)
    c2 = O.random_residues(rng, mods[:nq], ctx.n, 1)[0]
    t = pg.to_device(ct)
    ctx.keyswitch(ws, t, pg.to_device(c2), 1, pg.KeySwitchKey(pg.to_device(key)))
    _eq(t, oc.keyswitch(nq, ct, c2, key, scheme=1), "BFV keyswitch")
    out = torch.empty((2, nq - 1, ctx.n), dtype=torch.int64, device="cuda")
    ctx.bfv_mod_switch_to_next(pg.to_device(ct), out, 2, 1)
    _eq(out, oc.divide_round_q_last(nq, ct), "BFV mod switch")


def test_ntt_over_hps_r_base(bfv_small, pg):
    ctx, oc, mods, nq, ws = bfv_small
    rng = np.random.default_rng(72)
    r = oc.r_moduli
    a = O.random_residues(rng, r, ctx.n, 1)
    t = pg.to_device(a)
    ctx.ntt_forward(t, 1, len(r), nq + 2)
    full = np.zeros((nq + len(r), ctx.n), dtype=np.uint64)
    full[nq:] = a[0]
    _eq(t, oc.ntt_fwd_qr(full)[nq:], "forward NTT over R")


# ---------------------------------------------------------------- full-size parameter sets

@pytest.fixture(scope="module")
def ckks16(pg):
    ctx, oc, mods, nq = _ckks(pg, 1 << 16, [60] + [40] * 29 + [60] * 5, 5)
    return ctx, oc, mods, nq, ctx.workspace()


def test_n16_l30_multiply_relin_rescale_matches_oracle(ckks16, pg):
    ctx, oc, mods, nq, ws = ckks16
    rng = np.random.default_rng(80)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    l = nq
    a = O.random_residues(rng, mods[:l], ctx.n, 2)
    b = O.random_residues(rng, mods[:l], ctx.n, 2)
    out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
    ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, 1, pg.KeySwitchKey(pg.to_device(key)))
    _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, b, key)), "N=2^16 l=30 multiply+relin+rescale")


def test_n16_rotate_matches_oracle(ckks16, pg):
    ctx, oc, mods, nq, ws = ckks16
    rng = np.random.default_rng(81)
    elt = pg.elt_from_step(1, ctx.n)
    idx = ctx.galois_elts.index(elt)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    gks = [None] * len(ctx.galois_elts)
    gks[idx] = pg.KeySwitchKey(pg.to_device(key))
    chain = 8
    l = ctx.level(chain)
    ct = O.random_residues(rng, mods[:l], ctx.n, 2)
    t = pg.to_device(ct)
    ctx.rotate(ws, t, chain, 1, gks)
    _eq(t, oc.ckks_apply_galois(l, ct, elt, key), "N=2^16 rotate(1)")


def test_n16_ntt_round_trip_all_35_limbs(ckks16, pg):
    ctx, oc, mods, nq, ws = ckks16
    rng = np.random.default_rng(82)
    a = O.random_residues(rng, mods, ctx.n, 2)
    t = pg.to_device(a)
    ctx.ntt_forward(t, 2, len(mods), 0)
    ctx.ntt_inverse(t, 2, len(mods), 0)
    _eq(t, a, "N=2^16 round trip")


def test_n15_bfv_hps_multiply_relin_matches_oracle(pg):
    n, bits, special = 1 << 15, [50] * 16 + [60, 60], 2
    mods = pg.create_coeff_modulus(n, bits)
    ctx = pg.Context(n, mods, special, scheme=pg.SCHEME_BFV, plain_modulus=65537)
    oc = O.Context(15, mods, 16, special, 65537)
    ws = ctx.workspace()
    rng = np.random.default_rng(83)
    key = _key(rng, mods, ctx.dnum, n)
    a = O.random_residues(rng, mods[:16], n, 2)
    b = O.random_residues(rng, mods[:16], n, 2)
    ta = pg.to_device(a)
    ctx.multiply_and_relin(ws, ta, pg.to_device(b), 1, pg.KeySwitchKey(pg.to_device(key)))
    _eq(ta, oc.bfv_mul_relin_hps(a, b, key), "N=2^15 BFV HPS multiply_and_relin")


# ---------------------------------------------------------------- batched HMult (uneven levels)

def _batch_case(pg, ctx, mods, chains, seed):
    rng = np.random.default_rng(seed)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    k = pg.KeySwitchKey(pg.to_device(key))
    items, host = [], []
    for ch in chains:
        l = ctx.level(ch)
        a = O.random_residues(rng, mods[:l], ctx.n, 2)
        b = O.random_residues(rng, mods[:l], ctx.n, 2)
        out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
        items.append((pg.to_device(a), pg.to_device(b), out, ch))
        host.append((a, b, l))
    return key, k, items, host


@pytest.mark.parametrize("fused", [True, False])
def test_batch_multiply_relin_rescale_uneven_levels_small(small, pg, fused):
    """Both forms of the batched mod-up + inner product: the row pass fused with the inner
    product (key tiles shared by the items through L2) and the two-kernel form."""
    ctx, oc, mods, nq, ws = small
    chains = [1, 5, 3, 2, 4, 1, 3]
    key, k, items, host = _batch_case(pg, ctx, mods, chains, 90)
    wsb = ctx.workspace(batch_items=len(chains))
    ctx.fused_keyswitch = fused
    try:
        ctx.multiply_relin_rescale_batch(wsb, items, k)
    finally:
        ctx.fused_keyswitch = True
    for (a, b, l), (_, _, out, ch) in zip(host, items):
        _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, b, key)), f"batch item at chain {ch}, fused={fused}")
    assert ctx.device_status() == 0


@pytest.mark.parametrize("fused", [True, False])
def test_many_digits_fold_the_digit_sums(pg, fused):
    """One special prime over ten data primes: beta = l digits (8 to 10), so the 128-bit digit
    sums of the inner product are reduced after every 7 terms (in the fused kernel a tensor-memory
    load, reduce and store of the running sums).  Single key switch, HMult + relin + rescale and
    the batched call, each word for word against the oracle."""
    ctx, oc, mods, nq = _ckks(pg, 4096, [60] + [40] * 9 + [60], 1)
    ws = ctx.workspace()
    rng = np.random.default_rng(1010)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    k = pg.KeySwitchKey(pg.to_device(key))
    ctx.fused_keyswitch = fused
    try:
        for chain in (1, 2, 3):  # l = 10, 9, 8
            l = ctx.level(chain)
            ct = O.random_residues(rng, mods[:l], ctx.n, 2)
            c2 = O.random_residues(rng, mods[:l], ctx.n, 1)[0]
            t = pg.to_device(ct)
            ctx.keyswitch(ws, t, pg.to_device(c2), chain, k)
            _eq(t, oc.keyswitch(l, ct, c2, key), f"key switch, {l} digits, fused={fused}")
            a = O.random_residues(rng, mods[:l], ctx.n, 2)
            b = O.random_residues(rng, mods[:l], ctx.n, 2)
            out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
            ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, chain, k)
            _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, b, key)), f"HMult+relin+rescale, {l} digits, fused={fused}")
        chains = [1, 3, 2, 1]
        key_b, kb, items, host = _batch_case(pg, ctx, mods, chains, 1011)
        wsb = ctx.workspace(batch_items=len(chains))
        ctx.multiply_relin_rescale_batch(wsb, items, kb)
        for (a, b, l), (_, _, out, ch) in zip(host, items):
            _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, b, key_b)), f"batch item, {l} digits, fused={fused}")
    finally:
        ctx.fused_keyswitch = True
    assert ctx.device_status() == 0


def test_batch_more_than_one_launch_set(small, pg):
    ctx, oc, mods, nq, ws = small
    chains = [1 + (i * 7) % 5 for i in range(70)]  # 70 > 64: two launch sets
    key, k, items, host = _batch_case(pg, ctx, mods, chains, 91)
    wsb = ctx.workspace(batch_items=64)
    ctx.multiply_relin_rescale_batch(wsb, items, k)
    for (a, b, l), (_, _, out, ch) in list(zip(host, items))[::9]:
        _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, b, key)), f"batch item at chain {ch}")


def test_n16_batch_equals_single_calls(ckks16, pg):
    ctx, oc, mods, nq, ws = ckks16
    rng_chains = np.random.default_rng(92)
    chains = [int(31 - x) for x in rng_chains.integers(5, 31, size=12)]  # levels 5..30
    key, k, items, host = _batch_case(pg, ctx, mods, chains, 93)
    wsb = ctx.workspace(batch_items=len(chains))
    ctx.multiply_relin_rescale_batch(wsb, items, k)
    for (a, b, l), (ta, tb, out, ch) in zip(host, items):
        single = torch.empty_like(out)
        ctx.multiply_relin_rescale(ws, ta, tb, single, ch, k)
        assert torch.equal(out, single), f"chain {ch}"
    a, b, l = host[0]
    _eq(items[0][2], oc.rescale(l, oc.ckks_mul_relin(l, a, b, key)), "batch item 0 vs oracle")


def _ks_batch_case(pg, ctx, mods, chains, seed):
    rng = np.random.default_rng(seed)
    key = _key(rng, mods, ctx.dnum, ctx.n)
    items, host = [], []
    for ch in chains:
        l = ctx.level(ch)
        ct = O.random_residues(rng, mods[:l], ctx.n, 2)
        c2 = O.random_residues(rng, mods[:l], ctx.n, 1)[0]
        items.append((pg.to_device(ct), pg.to_device(c2), ch))
        host.append((ct, c2, l))
    return key, pg.KeySwitchKey(pg.to_device(key)), items, host


@pytest.mark.parametrize("fused", [True, False])
def test_keyswitch_batch_uneven_levels(small, pg, fused):
    ctx, oc, mods, nq, ws = small
    chains = [1, 5, 3, 2, 4, 1, 6, 3]
    key, k, items, host = _ks_batch_case(pg, ctx, mods, chains, 95)
    wsb = ctx.workspace(batch_items=len(chains))
    ctx.fused_keyswitch = fused
    try:
        ctx.keyswitch_batch(wsb, items, k)
    finally:
        ctx.fused_keyswitch = True
    for (ct, c2, l), (t, _, ch) in zip(host, items):
        _eq(t, oc.keyswitch(l, ct, c2, key), f"batched key switch at chain {ch}, fused={fused}")
    assert ctx.device_status() == 0


def test_n16_keyswitch_batch_equals_single_calls(ckks16, pg):
    ctx, oc, mods, nq, ws = ckks16
    rng_chains = np.random.default_rng(96)
    chains = [int(31 - x) for x in rng_chains.integers(5, 31, size=10)]  # levels 5..30
    key, k, items, host = _ks_batch_case(pg, ctx, mods, chains, 97)
    singles = [t.clone() for t, _, _ in items]
    wsb = ctx.workspace(batch_items=len(chains))
    ctx.keyswitch_batch(wsb, items, k)
    for (t, c2, ch), single in zip(items, singles):
        ctx.keyswitch(ws, single, c2, ch, k)
        assert torch.equal(t, single), f"chain {ch}"
    ct, c2, l = host[0]
    _eq(items[0][0], oc.keyswitch(l, ct, c2, key), "batched key switch item 0 vs oracle")


def test_n17_max_degree_keyswitch_and_fused(pg):
    """The largest supported degree (2^17): key switch, HMult+relin+rescale and a rotation."""
    n = 1 << 17
    bits = [60, 50, 50, 50, 50, 50, 60, 60]
    mods = pg.create_coeff_modulus(n, bits)
    nq = 6
    ctx = pg.Context(n, mods, 2)
    oc = O.Context(17, mods, nq, 2)
    ws = ctx.workspace()
    rng = np.random.default_rng(170)
    key = _key(rng, mods, ctx.dnum, n)
    k = pg.KeySwitchKey(pg.to_device(key))
    for chain in (1, 4):
        l = ctx.level(chain)
        ct = O.random_residues(rng, mods[:l], n, 2)
        c2 = O.random_residues(rng, mods[:l], n, 1)[0]
        t = pg.to_device(ct)
        ctx.keyswitch(ws, t, pg.to_device(c2), chain, k)
        _eq(t, oc.keyswitch(l, ct, c2, key), f"N=2^17 keyswitch chain {chain}")
        a = O.random_residues(rng, mods[:l], n, 2)
        b = O.random_residues(rng, mods[:l], n, 2)
        out = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
        ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, chain, k)
        _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, b, key)), f"N=2^17 HMult+relin+rescale chain {chain}")
    elt = pg.elt_from_step(1, n)
    gks = [k if e == elt else None for e in ctx.galois_elts]
    ct = O.random_residues(rng, mods[:nq], n, 2)
    t = pg.to_device(ct)
    ctx.rotate(ws, t, 1, 1, gks)
    _eq(t, oc.ckks_apply_galois(nq, ct, elt, key), "N=2^17 rotate by 1")
    assert ctx.device_status() == 0
