"""Word-for-word checks at the benchmark workloads' own parameters.

* BFV multiply + relinearise (HPS) at N = 2^15, 16 x 50-bit + 2 x 60-bit primes, t = 65537: 128
  operations captured in one CUDA graph and replayed give the same words as the same 128 calls
  made one by one, and those equal the oracle.
* The 128 x 128 diagonal-method matrix-vector product at N = 2^16, Q = 1 x 60 + 19 x 40-bit,
  P = 4 x 60-bit (dnum = 5), 11 baby steps and 12 giant steps over 128 diagonals: both drivers
  (the reference's loop and the hoisted Horner form) against the oracle's composition of the
  same calls."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def pg():
    import phantom_gb300
    return phantom_gb300


def _eq(t, want, what):
    got = t.cpu().numpy().view(np.uint64) if isinstance(t, torch.Tensor) else t
    bad = np.flatnonzero(got.reshape(-1) != np.asarray(want, dtype=np.uint64).reshape(-1))
    assert bad.size == 0, f"{what}: {bad.size} words differ, first at {bad[0]}"


def test_bfv_mult_relin_graph_of_128_equals_the_loop(pg):
    n = 1 << 15
    bits = [50] * 16 + [60, 60]
    mods = pg.create_coeff_modulus(n, bits)
    ctx = pg.Context(n, mods, 2, scheme=pg.SCHEME_BFV, plain_modulus=65537)
    ws = ctx.workspace()
    rng = np.random.default_rng(4096)
    key_h = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    key = pg.KeySwitchKey(pg.to_device(key_h))
    ins = [(O.random_residues(rng, mods[:16], n, 2), O.random_residues(rng, mods[:16], n, 2)) for _ in range(8)]
    dev = [(pg.to_device(a), pg.to_device(b)) for a, b in ins]
    ops = 128
    looped = [dev[i % 8][0].clone() for i in range(ops)]
    for i in range(ops):
        ctx.multiply_and_relin(ws, looped[i], dev[i % 8][1], 1, key)
    graphed = [dev[i % 8][0].clone() for i in range(ops)]
    warm = dev[0][0].clone()
    ctx.multiply_and_relin(ws, warm, dev[0][1], 1, key)  # first call outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for i in range(ops):
            ctx.multiply_and_relin(ws, graphed[i], dev[i % 8][1], 1, key)
    g.replay()
    torch.cuda.synchronize()
    for i in range(ops):
        assert torch.equal(graphed[i], looped[i]), f"operation {i}: graph replay differs from the call"
    oc = O.Context(15, mods, 16, 2, 65537)
    for i in range(8):
        _eq(looped[i], oc.bfv_mul_relin_hps(ins[i][0], ins[i][1], key_h), f"operation {i} against the oracle")
    assert ctx.device_status() == 0


MV_BITS = [60] + [40] * 19 + [60] * 4
MV_G, MV_B, MV_D = 11, 12, 128


@pytest.fixture(scope="module")
def mv(pg):
    n = 1 << 16
    mods = pg.create_coeff_modulus(n, MV_BITS)
    hsteps = list(range(1, MV_G + 1))
    xsteps = list(range(1, MV_G)) + [g * MV_G for g in range(1, MV_B)]
    steps = sorted(set(hsteps + xsteps))
    ctx = pg.Context(n, mods, 4, galois_elts=sorted({pg.elt_from_step(s, n) for s in steps}))
    oc = O.Context(16, mods, 20, 4)
    rng = np.random.default_rng(5005)
    keys = {s: O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n) for s in steps}
    gks = [None] * len(ctx.galois_elts)
    for s, k in keys.items():
        gks[ctx.galois_elts.index(pg.elt_from_step(s, n))] = pg.KeySwitchKey(pg.to_device(k))
    diags = O.random_residues(rng, mods[:20], n, MV_D)
    return ctx, oc, mods, keys, gks, diags, ctx.workspace(), rng


def _oracle_matvec(oc, pg, mods, keys, diags, ct, l, hoisted):
    n = oc.n
    elt = lambda s: pg.elt_from_step(s, n)  # noqa: E731
    if hoisted:
        babies = [ct] + [oc.ckks_hoisting(l, ct, [elt(b)], [keys[b]]) for b in range(1, MV_G)]
    else:
        babies = [ct] + [oc.ckks_apply_galois(l, ct, elt(b), keys[b]) for b in range(1, MV_G)]

    def inner(g):
        acc = np.zeros((2, l, n), dtype=np.uint64)
        for b in range(MV_G):
            k = g * MV_G + b
            if k < MV_D:
                oc.mul_add(l, acc, babies[b], diags[k, :l])
        return acc

    def add(x, y):
        q = np.array(mods[:l], dtype=np.uint64).reshape(1, -1, 1)
        s = x + y  # canonical residues below 2^61: no wrap
        return np.where(s >= q, s - q, s)

    if hoisted:  # Horner: inner_0 + rot_G(inner_1 + rot_G(inner_2 + ...))
        result = None
        for g in reversed(range(MV_B)):
            if result is not None:
                result = oc.ckks_apply_galois(l, result, elt(MV_G), keys[MV_G])
            result = inner(g) if result is None else add(result, inner(g))
    else:  # the reference's loop: sum_g rot_{g G}(inner_g)
        result = None
        for g in range(MV_B):
            x = inner(g)
            if g > 0:
                x = oc.ckks_apply_galois(l, x, elt(g * MV_G), keys[g * MV_G])
            result = x if result is None else add(result, x)
    return oc.rescale(l, result)


@pytest.mark.parametrize("hoisted,l", [(True, 20), (False, 20), (True, 7)])
def test_matvec128_at_its_parameters_word_for_word(mv, pg, hoisted, l):
    ctx, oc, mods, keys, gks, diags, ws, rng = mv
    chain = 20 - l + 1
    ct = O.random_residues(rng, mods[:l], ctx.n, 2)
    dg = pg.to_device(np.ascontiguousarray(diags[:, :l]))
    scratch = torch.empty(ctx.bsgs_scratch_bytes(MV_G) // 8, dtype=torch.int64, device="cuda")
    out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
    ctx.bsgs_matvec(ws, scratch, pg.to_device(ct), chain, dg, MV_D, MV_G, MV_B, gks, out, hoisted=hoisted)
    _eq(out, _oracle_matvec(oc, pg, mods, keys, diags, ct, l, hoisted),
        f"matrix-vector product ({'hoisted' if hoisted else 'reference loop'}, l = {l})")
    assert ctx.device_status() == 0


def test_matvec128_batch_at_its_parameters_equals_single_calls(mv, pg):
    """The batched hoisted 128 x 128 product at its own parameters, three vectors at uneven
    levels: every output equals the single call's words (which the test above pins to the
    oracle)."""
    ctx, oc, mods, keys, gks, diags, ws, rng = mv
    items, singles = [], []
    one = torch.empty(ctx.bsgs_scratch_bytes(MV_G) // 8, dtype=torch.int64, device="cuda")
    for l in (20, 7, 12):
        chain = 20 - l + 1
        t = pg.to_device(O.random_residues(rng, mods[:l], ctx.n, 2))
        dg = pg.to_device(np.ascontiguousarray(diags[:, :l]))
        out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
        single = torch.empty_like(out)
        ctx.bsgs_matvec(ws, one, t, chain, dg, MV_D, MV_G, MV_B, gks, single, hoisted=True)
        items.append((t, chain, dg, out))
        singles.append(single)
    del one
    wsb = ctx.workspace(batch_items=len(items))
    scratch = torch.empty(len(items) * ctx.bsgs_batch_scratch_bytes(MV_G, MV_B) // 8, dtype=torch.int64, device="cuda")
    ctx.bsgs_matvec_batch(wsb, scratch, items, MV_D, MV_G, MV_B, gks)
    for (t, chain, dg, out), single in zip(items, singles):
        assert torch.equal(out, single), f"chain {chain}"
    assert ctx.device_status() == 0
