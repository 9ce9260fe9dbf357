"""Plaintext products, hoisted rotations, the baby-step/giant-step matrix-vector product and
secret-key encryption / key generation on the GPU.

Word-for-word cases compare against the CPU oracle (rotations, rescale) composed with exact
modular products written here in Python integers.  The end-to-end cases use real keys made on
the GPU from seeded randomness and check decrypted, decoded slots against an FP64 matmul."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def pg():
    import phantom_gb300
    return phantom_gb300


def _u(t):
    return t.cpu().numpy().view(np.uint64)


def _eq(got_t, want, what):
    got = got_t if isinstance(got_t, np.ndarray) else _u(got_t)
    want = np.asarray(want, dtype=np.uint64).reshape(got.shape)
    bad = int((got != want).sum())
    assert bad == 0, f"{what}: {bad} of {got.size} words differ"


def _mulmod(a, b, mods):
    """a [..., limbs, N] * b [limbs, N] mod q_limb, exact."""
    q = np.array(mods, dtype=object).reshape(-1, 1)
    return ((a.astype(object) * b.astype(object)) % q).astype(np.uint64)


def _addmod(a, b, mods):
    q = np.array(mods, dtype=object).reshape(-1, 1)
    return ((a.astype(object) + b.astype(object)) % q).astype(np.uint64)


def _key(rng, mods, dnum, n):
    return O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)


G, B, D = 4, 3, 10  # ragged: the last giant step has two diagonals
STEPS = sorted({*range(1, G), G, *[g * G for g in range(1, B)]})


@pytest.fixture(scope="module")
def lin(pg):
    n = 4096
    bits = [60, 40, 40, 40, 40, 40, 60, 60]
    mods = pg.create_coeff_modulus(n, bits)
    nq = 6
    elts = [pg.elt_from_step(s, n) for s in STEPS]
    ctx = pg.Context(n, mods, 2, galois_elts=elts)
    oc = O.Context(12, mods, nq, 2)
    rng = np.random.default_rng(501)
    keys = [_key(rng, mods, ctx.dnum, n) for _ in ctx.galois_elts]
    gks = [pg.KeySwitchKey(pg.to_device(k)) for k in keys]
    return ctx, oc, mods, keys, gks, ctx.workspace()


def _key_of(ctx, keys, step):
    from phantom_gb300 import elt_from_step
    e = elt_from_step(step, ctx.n)
    return e, keys[ctx.galois_elts.index(e)]


def test_multiply_plain_and_add(lin):
    ctx, oc, mods, keys, gks, ws = lin
    rng = np.random.default_rng(1)
    for chain in (1, 3):
        l = ctx.level(chain)
        ct = O.random_residues(rng, mods[:l], ctx.n, 2)
        pt = O.random_residues(rng, mods[:l], ctx.n, 1)[0]
        other = O.random_residues(rng, mods[:l], ctx.n, 2)
        from phantom_gb300 import to_device
        t, p, o = to_device(ct), to_device(pt), to_device(other)
        out = torch.empty_like(t)
        ctx.multiply_plain(t, p, out, chain)
        want = _mulmod(ct, pt, mods[:l])
        _eq(out, want, "multiply_plain")
        ctx.multiply_plain(t, p, t, chain)  # in place
        _eq(t, want, "multiply_plain in place")
        ctx.add(t, o, out, 2, chain)
        _eq(out, _addmod(want, other, mods[:l]), "add")


def test_rotations_hoisted_match_single_step_hoisting(lin, pg):
    ctx, oc, mods, keys, gks, ws = lin
    rng = np.random.default_rng(2)
    for chain in (1, 2):
        l = ctx.level(chain)
        ct = O.random_residues(rng, mods[:l], ctx.n, 2)
        t = pg.to_device(ct)
        steps = [1, 2, 3, 4]
        outs = [torch.empty_like(t) for _ in steps]
        ctx.rotations_hoisted(ws, t, chain, steps, gks, outs)
        _eq(t, ct, "input untouched")
        for s, o in zip(steps, outs):
            e, k = _key_of(ctx, keys, s)
            _eq(o, oc.ckks_hoisting(l, ct, [e], [k]), f"hoisted rotation by {s}")


def _diags(rng, mods, l, n):
    return O.random_residues(rng, mods[:l], n, D)


def _plain_sum(babies, diags, g, mods, l, G=G):
    acc = None
    for b in range(G):
        k = g * G + b
        if k >= D:
            break
        term = _mulmod(babies[b], diags[k], mods[:l])
        acc = term if acc is None else _addmod(acc, term, mods[:l])
    return acc


@pytest.mark.parametrize("chain", [1, 2])
def test_bsgs_reference_loop_word_for_word(lin, pg, chain):
    ctx, oc, mods, keys, gks, ws = lin
    rng = np.random.default_rng(10 + chain)
    l = ctx.level(chain)
    ct = O.random_residues(rng, mods[:l], ctx.n, 2)
    diags = _diags(rng, mods, l, ctx.n)
    t, dg = pg.to_device(ct), pg.to_device(diags)
    scratch = torch.empty(ctx.bsgs_scratch_bytes(G) // 8, dtype=torch.int64, device="cuda")
    out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
    ctx.bsgs_matvec(ws, scratch, t, chain, dg, D, G, B, gks, out, hoisted=False)

    babies = [ct] + [oc.ckks_apply_galois(l, ct, *_key_of(ctx, keys, b)) for b in range(1, G)]
    result = None
    for g in range(B):
        inner = _plain_sum(babies, diags, g, mods, l)
        if g > 0:
            inner = oc.ckks_apply_galois(l, inner, *_key_of(ctx, keys, g * G))
        result = inner if result is None else _addmod(result, inner, mods[:l])
    _eq(out, oc.rescale(l, result), "BSGS (reference loop)")


# (G, B): a ragged last giant step (G = 4, B = 3, D = 10) and a deeper Horner chain (G = 2, B = 5)
@pytest.mark.parametrize("chain,G,B", [(1, G, B), (3, G, B), (1, 2, 5)])
def test_bsgs_hoisted_horner_word_for_word(lin, pg, chain, G, B):
    ctx, oc, mods, keys, gks, ws = lin
    rng = np.random.default_rng(20 + chain)
    l = ctx.level(chain)
    ct = O.random_residues(rng, mods[:l], ctx.n, 2)
    diags = _diags(rng, mods, l, ctx.n)
    t, dg = pg.to_device(ct), pg.to_device(diags)
    scratch = torch.empty(ctx.bsgs_scratch_bytes(G) // 8, dtype=torch.int64, device="cuda")
    out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
    ctx.bsgs_matvec(ws, scratch, t, chain, dg, D, G, B, gks, out, hoisted=True)

    babies = [ct]
    for b in range(1, G):
        e, k = _key_of(ctx, keys, b)
        babies.append(oc.ckks_hoisting(l, ct, [e], [k]))
    result = None
    for g in reversed(range(B)):
        if result is not None:
            result = oc.ckks_apply_galois(l, result, *_key_of(ctx, keys, G))
        inner = _plain_sum(babies, diags, g, mods, l, G)
        result = inner if result is None else _addmod(result, inner, mods[:l])
    _eq(out, oc.rescale(l, result), "BSGS (hoisted, Horner)")


@pytest.mark.parametrize("G,B,tc", [(G, B, True), (2, 5, True), (G, B, False)])
def test_bsgs_batch_equals_single_calls(lin, pg, G, B, tc):
    """The batched hoisted matrix-vector product over ciphertexts at uneven levels (one launch
    per pipeline step for all of them) gives every single call's words; without the tensor-core
    conversions the batch runs the single calls."""
    ctx, oc, mods, keys, gks, ws = lin
    rng = np.random.default_rng(40 + G)
    chains = [1, 3, 2, 5, 1, 4]
    items, singles = [], []
    one = torch.empty(ctx.bsgs_scratch_bytes(G) // 8, dtype=torch.int64, device="cuda")
    ctx.tensor_cores = tc
    try:
        for ch in chains:
            l = ctx.level(ch)
            t = pg.to_device(O.random_residues(rng, mods[:l], ctx.n, 2))
            dg = pg.to_device(_diags(rng, mods, l, ctx.n))
            out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
            single = torch.empty_like(out)
            ctx.bsgs_matvec(ws, one, t, ch, dg, D, G, B, gks, single, hoisted=True)
            items.append((t, ch, dg, out))
            singles.append(single)
        wsb = ctx.workspace(batch_items=len(items))
        scratch = torch.empty(len(items) * ctx.bsgs_batch_scratch_bytes(G, B) // 8, dtype=torch.int64, device="cuda")
        ctx.bsgs_matvec_batch(wsb, scratch, items, D, G, B, gks)
    finally:
        ctx.tensor_cores = True
    for (t, ch, dg, out), single in zip(items, singles):
        assert torch.equal(out, single), f"chain {ch}, tensor_cores={tc}"
    assert ctx.device_status() == 0


@pytest.mark.parametrize("tc", [True, False])
def test_bsgs_batch_shared_diagonals(lin, pg, tc):
    """Items at uneven levels all reading one diagonal array encoded at the top level (its limb
    count is the stride, the first l limbs are read) give the words of single calls on contiguous
    per-level copies; without the tensor-core conversions the batch's single calls take the same
    stride."""
    ctx, oc, mods, keys, gks, ws = lin
    rng = np.random.default_rng(48)
    top = ctx.level(1)
    shared = pg.to_device(_diags(rng, mods, top, ctx.n))
    chains = [2, 1, 4, 3, 2]
    items, singles = [], []
    one = torch.empty(ctx.bsgs_scratch_bytes(G) // 8, dtype=torch.int64, device="cuda")
    ctx.tensor_cores = tc
    try:
        for ch in chains:
            l = ctx.level(ch)
            t = pg.to_device(O.random_residues(rng, mods[:l], ctx.n, 2))
            out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
            single = torch.empty_like(out)
            ctx.bsgs_matvec(ws, one, t, ch, shared[:, :l].contiguous(), D, G, B, gks, single, hoisted=True)
            items.append((t, ch, shared, out))
            singles.append(single)
        wsb = ctx.workspace(batch_items=len(items))
        scratch = torch.empty(len(items) * ctx.bsgs_batch_scratch_bytes(G, B) // 8, dtype=torch.int64, device="cuda")
        ctx.bsgs_matvec_batch(wsb, scratch, items, D, G, B, gks)
    finally:
        ctx.tensor_cores = True
    for (t, ch, dg, out), single in zip(items, singles):
        assert torch.equal(out, single), f"chain {ch}, tensor_cores={tc}"
    # a diagonal array with fewer limbs than the item's level is refused
    l = ctx.level(1)
    short = shared[:, : l - 1].contiguous()
    with pytest.raises(RuntimeError):
        ctx.bsgs_matvec_batch(wsb, scratch, [(items[1][0], 1, short, items[1][3])], D, G, B, gks)
    assert ctx.device_status() == 0


def test_bsgs_batch_many_babies_ragged(pg):
    """G = 14 babies (13 hoisted baby rotations, every giant step's inner sum over 14 diagonals)
    and a ragged last giant step (D = 20): every output equals the single call's words."""
    n = 4096
    mods = pg.create_coeff_modulus(n, [60, 40, 40, 40, 40, 40, 60, 60])
    g_, b_, d_ = 14, 2, 20
    ctx = pg.Context(n, mods, 2, galois_elts=[pg.elt_from_step(s, n) for s in range(1, g_ + 1)])
    ws = ctx.workspace()
    rng = np.random.default_rng(49)
    gks = [pg.KeySwitchKey(pg.to_device(_key(rng, mods, ctx.dnum, n))) for _ in ctx.galois_elts]
    one = torch.empty(ctx.bsgs_scratch_bytes(g_) // 8, dtype=torch.int64, device="cuda")
    items, singles = [], []
    for ch in (1, 3, 2):
        l = ctx.level(ch)
        t = pg.to_device(O.random_residues(rng, mods[:l], n, 2))
        dg = pg.to_device(O.random_residues(rng, mods[:l], n, d_))
        out = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
        single = torch.empty_like(out)
        ctx.bsgs_matvec(ws, one, t, ch, dg, d_, g_, b_, gks, single, hoisted=True)
        items.append((t, ch, dg, out))
        singles.append(single)
    wsb = ctx.workspace(batch_items=len(items))
    scratch = torch.empty(len(items) * ctx.bsgs_batch_scratch_bytes(g_, b_) // 8, dtype=torch.int64, device="cuda")
    ctx.bsgs_matvec_batch(wsb, scratch, items, d_, g_, b_, gks)
    for (t, ch, dg, out), single in zip(items, singles):
        assert torch.equal(out, single), f"chain {ch}"
    assert ctx.device_status() == 0


def test_bsgs_batch_more_than_one_launch_set(lin, pg):
    """70 products (more than one launch set of 64, the second one reusing the first's scratch)
    give the single calls' words."""
    ctx, oc, mods, keys, gks, ws = lin
    rng = np.random.default_rng(47)
    one = torch.empty(ctx.bsgs_scratch_bytes(G) // 8, dtype=torch.int64, device="cuda")
    items, singles = [], []
    for i in range(70):
        ch = 1 + (i * 3) % 5
        l = ctx.level(ch)
        t = pg.to_device(O.random_residues(rng, mods[:l], ctx.n, 2))
        dg = pg.to_device(_diags(rng, mods, l, ctx.n))
        out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
        single = torch.empty_like(out)
        ctx.bsgs_matvec(ws, one, t, ch, dg, D, G, B, gks, single, hoisted=True)
        items.append((t, ch, dg, out))
        singles.append(single)
    wsb = ctx.workspace(batch_items=64)
    scratch = torch.empty(64 * ctx.bsgs_batch_scratch_bytes(G, B) // 8, dtype=torch.int64, device="cuda")
    ctx.bsgs_matvec_batch(wsb, scratch, items, D, G, B, gks)
    for i, ((t, ch, dg, out), single) in enumerate(zip(items, singles)):
        assert torch.equal(out, single), f"item {i}, chain {ch}"
    assert ctx.device_status() == 0


def test_bsgs_rejects_bad_shapes(lin, pg):
    ctx, oc, mods, keys, gks, ws = lin
    l = ctx.level(1)
    t = torch.zeros((2, l, ctx.n), dtype=torch.int64, device="cuda")
    dg = torch.zeros((D, l, ctx.n), dtype=torch.int64, device="cuda")
    scratch = torch.empty(ctx.bsgs_scratch_bytes(G) // 8, dtype=torch.int64, device="cuda")
    out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
    with pytest.raises(pg.InvalidArgument):
        ctx.bsgs_matvec(ws, scratch, t, 1, dg, D, 2, 2, gks, out)  # G * B < D
    with pytest.raises(pg.InvalidArgument):
        ctx.bsgs_matvec(ws, scratch, t, ctx.size_q, dg, D, G, B, gks, out)  # one limb: cannot rescale


# ---------------------------------------------------------------- keys and encryption

def test_keygen_encrypt_decrypt_word_for_word(pg):
    """GPU key generation / encryption / decryption against the formulas restated exactly."""
    from phantom_gb300.ckks import CkksEncoder, SecretKey
    n = 4096
    mods = pg.create_coeff_modulus(n, [60, 40, 40, 40, 60, 60])
    elt = pg.elt_from_step(1, n)
    ctx = pg.Context(n, mods, 2, galois_elts=[elt])
    oc = O.Context(12, mods, 4, 2)
    ws = ctx.workspace()
    rng = np.random.default_rng(7)
    sk = SecretKey(ctx, rng)
    s_rns = CkksEncoder.to_rns(sk.coeffs, mods)
    s_ntt = oc.ntt_fwd(s_rns)
    _eq(sk.s_ntt, s_ntt, "secret key NTT")

    qp = len(mods)
    P = 1
    for p in mods[4:]:
        P *= p
    for g in (0, elt):
        a = O.random_residues(rng, mods, n, ctx.dnum)
        e = rng.integers(-20, 21, size=(ctx.dnum, n), dtype=np.int64)
        key = torch.empty((ctx.dnum, 2, qp, n), dtype=torch.int64, device="cuda")
        ctx.kswitch_keygen(ws, g, sk.s_ntt, pg.to_device(a), torch.from_numpy(e).cuda(), key)
        if g == 0:
            src = _mulmod(s_ntt, s_ntt, mods)
        else:
            # sigma_g in NTT form is the oracle's NTT-domain Galois permutation
            src = oc.apply_galois_ntt(s_ntt, g)
        for d in range(ctx.dnum):
            e_ntt = oc.ntt_fwd(CkksEncoder.to_rns(e[d], mods))
            b = _addmod(_mulmod(a[d], s_ntt, mods), e_ntt, mods)
            b = ((-b.astype(object)) % np.array(mods, dtype=object).reshape(-1, 1)).astype(np.uint64)
            for j in range(2 * d, 2 * d + 2):
                b[j] = ((int(P % mods[j]) * src[j].astype(object) + b[j].astype(object)) % mods[j]).astype(np.uint64)
            _eq(key[d, 0], b, f"key {g} digit {d} poly 0")
            _eq(key[d, 1], a[d], f"key {g} digit {d} poly 1")

    for chain in (1, 2):
        l = ctx.level(chain)
        m = O.random_residues(rng, mods[:l], n, 1)[0]
        a = O.random_residues(rng, mods[:l], n, 1)[0]
        e = rng.integers(-20, 21, size=n, dtype=np.int64)
        ct = torch.empty((2, l, n), dtype=torch.int64, device="cuda")
        ctx.encrypt_symmetric(pg.to_device(m), sk.s_ntt, pg.to_device(a), torch.from_numpy(e).cuda(), ct, chain)
        ase = _addmod(_mulmod(a, s_ntt[:l], mods[:l]), oc.ntt_fwd(CkksEncoder.to_rns(e, mods[:l])), mods[:l])
        q = np.array(mods[:l], dtype=object).reshape(-1, 1)
        c0 = ((m.astype(object) - ase.astype(object)) % q).astype(np.uint64)
        _eq(ct[0], c0, "encrypt c0")
        _eq(ct[1], a, "encrypt c1")
        pt = torch.empty((l, n), dtype=torch.int64, device="cuda")
        ctx.decrypt(ct, sk.s_ntt, pt, chain)
        want = _addmod(c0, _mulmod(a, s_ntt[:l], mods[:l]), mods[:l])
        _eq(pt, want, "decrypt")


# ---------------------------------------------------------------- end to end (real keys)

def _matvec_setup(pg, n, d, G_, B_, hoisted):
    from phantom_gb300.ckks import CkksEncoder, SecretKey
    bits = [60] + [40] * 5 + [60, 60]
    mods = pg.create_coeff_modulus(n, bits)
    steps = list(range(1, G_)) + ([G_] if hoisted else [g * G_ for g in range(1, B_)])
    ctx = pg.Context(n, mods, 2, galois_elts=sorted({pg.elt_from_step(s, n) for s in steps}))
    ws = ctx.workspace()
    rng = np.random.default_rng(2024 + d)
    sk = SecretKey(ctx, rng)
    gks = sk.galois_keys(ws, steps)
    return ctx, ws, rng, sk, gks, CkksEncoder(n)


@pytest.mark.parametrize("hoisted", [True, False])
def test_matvec_decrypts_to_fp64_matmul(pg, hoisted):
    n, d = 8192, 64
    G_, B_ = 8, 8
    ctx, ws, rng, sk, gks, enc = _matvec_setup(pg, n, d, G_, B_, hoisted)
    S = n // 2
    scale = 2.0 ** 40
    M = rng.uniform(-1, 1, size=(d, d))
    x = rng.uniform(-1, 1, size=d) + 1j * rng.uniform(-1, 1, size=d)
    x *= 1 / np.maximum(1, np.abs(x))
    chain = 2
    l = ctx.level(chain)
    ct = sk.encrypt(enc.encode(ctx, np.tile(x, S // d), scale, chain), chain)

    idx = np.arange(S)
    diag_pts = []
    for k in range(d):
        g = k // G_
        diag = M[idx % d, (idx + k) % d]
        diag_pts.append(enc.encode(ctx, np.roll(diag, g * G_), scale, chain))  # rot_{-gG}(diag_k)
    diags = torch.stack(diag_pts)
    scratch = torch.empty(ctx.bsgs_scratch_bytes(G_) // 8, dtype=torch.int64, device="cuda")
    out = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
    ctx.bsgs_matvec(ws, scratch, ct, chain, diags, d, G_, B_, gks, out, hoisted=hoisted)
    q_last = ctx.moduli[l - 1]
    y = enc.decode(ctx, sk.decrypt(out, chain + 1), scale * scale / q_last, chain + 1)
    want = np.tile(M @ x, S // d)
    err = float(np.max(np.abs(y - want)))
    assert err < 1e-5, f"max slot error {err}"


def test_rotate_decrypts_to_rotated_slots(pg):
    """Slot i of rotate(ct, r) holds slot i + r of ct (the encoder's 5^i slot order)."""
    from phantom_gb300.ckks import CkksEncoder, SecretKey
    n = 4096
    mods = pg.create_coeff_modulus(n, [60, 40, 40, 60])
    ctx = pg.Context(n, mods, 1)
    ws = ctx.workspace()
    rng = np.random.default_rng(3)
    sk = SecretKey(ctx, rng)
    enc = CkksEncoder(n)
    gks = sk.galois_keys(ws, [1, 2, 4, 8, 16, -1])
    z = rng.uniform(-1, 1, n // 2) + 1j * rng.uniform(-1, 1, n // 2)
    ct = sk.encrypt(enc.encode(ctx, z, 2.0 ** 40, 1), 1)
    for r in (1, 5, -1):  # 5 = 4 + 1 through the NAF fallback
        t = ct.clone()
        ctx.rotate(ws, t, 1, r, gks)
        got = enc.decode(ctx, sk.decrypt(t, 1), 2.0 ** 40, 1)
        assert np.max(np.abs(got - np.roll(z, -r))) < 1e-6, f"rotation by {r}"
