"""Tensor-core (tcgen05, exact bf16 byte-plane GEMM) base conversions against the oracle and
against the CUDA-core form, word for word, over digit sizes 1..6, 40- and 60-bit primes (both
epilogue paths), partial last digits and every level of a chain."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def pg():
    import phantom_gb300
    return phantom_gb300


def _eq(got_t, want, what):
    got = got_t.cpu().numpy().view(np.uint64)
    want = np.asarray(want, dtype=np.uint64).reshape(got.shape)
    bad = int((got != want).sum())
    assert bad == 0, f"{what}: {bad} of {got.size} words differ"


PARAMS = {
    # name: (N, bit sizes, special primes, chain indices to test)
    "a1": (4096, [60, 40, 40, 40, 60], 1, [1, 3]),
    "a2_partial": (4096, [60, 40, 40, 40, 40, 60, 60], 2, [1, 2, 4]),
    "a3_all60": (8192, [60] * 7 + [60] * 3, 3, [1, 2, 5]),
    "a5_n16_l30": (65536, [60] + [40] * 29 + [60] * 5, 5, [1, 2, 13]),
    "a4_n16_l20": (65536, [60] + [40] * 19 + [60] * 4, 4, [1, 6, 17]),
    "a6": (4096, [60] + [50] * 11 + [60] * 6, 6, [1, 4]),
}


@pytest.mark.parametrize("name", list(PARAMS))
def test_keyswitch_tensor_core_matches_oracle_and_cuda_core(pg, name):
    n, bits, special, chains = PARAMS[name]
    mods = pg.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    ctx = pg.Context(n, mods, special)
    assert ctx.tensor_cores, "tensor-core conversions are the default for special_modulus_size <= 6"
    oc = O.Context(n.bit_length() - 1, mods, nq, special)
    ws = ctx.workspace()
    rng = np.random.default_rng(len(bits) * 7 + special)
    key = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    k = pg.KeySwitchKey(pg.to_device(key))
    for chain in chains:
        l = ctx.level(chain)
        ct = O.random_residues(rng, mods[:l], n, 2)
        c2 = O.random_residues(rng, mods[:l], n, 1)[0]
        want = oc.keyswitch(l, ct, c2, key)
        for tc in (True, False):
            ctx.tensor_cores = tc
            t = pg.to_device(ct)
            ctx.keyswitch(ws, t, pg.to_device(c2), chain, k)
            _eq(t, want, f"{name} chain {chain} tensor_cores={tc}")
        assert ctx.device_status() == 0
        ctx.tensor_cores = True


def test_fused_hmult_rescale_tensor_core(pg):
    n = 65536
    bits = [60] + [40] * 29 + [60] * 5
    mods = pg.create_coeff_modulus(n, bits)
    ctx = pg.Context(n, mods, 5)
    oc = O.Context(16, mods, 30, 5)
    ws = ctx.workspace()
    rng = np.random.default_rng(99)
    key = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    k = pg.KeySwitchKey(pg.to_device(key))
    l = 30
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    out = torch.empty((2, l - 1, n), dtype=torch.int64, device="cuda")
    ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, 1, k)
    _eq(out, oc.rescale(l, oc.ckks_mul_relin(l, a, b, key)), "HMult+relin+rescale (tensor cores)")
    assert ctx.device_status() == 0


def test_tensor_cores_unavailable_for_wide_digits(pg):
    n = 4096
    mods = pg.create_coeff_modulus(n, [60, 40, 40, 40] + [60] * 7)
    ctx = pg.Context(n, mods, 7)
    assert not ctx.tensor_cores
    with pytest.raises(pg.InvalidArgument):
        ctx.tensor_cores = True


BFV_PARAMS = {
    "bfv_n12_4x50": (4096, [50, 50, 50, 50, 60, 60], 2, 65537),
    "bfv_n15_16x50": (32768, [50] * 16 + [60, 60], 2, 65537),
    "bfv_n13_6x40": (8192, [40] * 6 + [60], 1, 786433),
    "bfv_n13_a3": (8192, [50] * 6 + [60] * 3, 3, 65537),  # key switch mod-up on the tensor cores
}


@pytest.mark.parametrize("name", list(BFV_PARAMS))
def test_bfv_hps_tensor_core_matches_oracle_and_cuda_core(pg, name):
    """HPS conversions and scale-and-round on the tensor cores (with the FP64 corrections in the
    reference's order) give the oracle's words, as the CUDA-core kernels do."""
    n, bits, special, t = BFV_PARAMS[name]
    mods = pg.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    ctx = pg.Context(n, mods, special, scheme=pg.SCHEME_BFV, plain_modulus=t)
    oc = O.Context(n.bit_length() - 1, mods, nq, special, t)
    ws = ctx.workspace()
    rng = np.random.default_rng(nq * 31 + special)
    key = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    k = pg.KeySwitchKey(pg.to_device(key))
    a = O.random_residues(rng, mods[:nq], n, 2)
    b = O.random_residues(rng, mods[:nq], n, 2)
    want = oc.bfv_mul_relin_hps(a, b, key)
    for tc in (True, False):
        ctx.tensor_cores = tc
        ta = pg.to_device(a)
        ctx.multiply_and_relin(ws, ta, pg.to_device(b), 1, k)
        _eq(ta, want, f"{name} BFV multiply_and_relin tensor_cores={tc}")
    ctx.tensor_cores = True
    ts = pg.to_device(a)
    ctx.multiply_and_relin(ws, ts, ts, 1, k)
    _eq(ts, oc.bfv_mul_relin_hps(a, a, key), f"{name} BFV square_and_relin (tensor cores)")
    assert ctx.device_status() == 0


@pytest.mark.parametrize("log_n,splits", [(13, [6, 7]), (15, [6, 7, 8]), (16, [7, 8])])
def test_every_ntt_split_gives_the_same_words(pg, log_n, splits):
    """The autotuner's choice (column-pass stages l1) never changes a result."""
    n = 1 << log_n
    bits = [60] + [40] * 5 + [60, 60]
    mods = pg.create_coeff_modulus(n, bits)
    ctx = pg.Context(n, mods, 2)
    oc = O.Context(log_n, mods, 6, 2)
    ws = ctx.workspace()
    rng = np.random.default_rng(log_n)
    a = O.random_residues(rng, mods, n, 1)
    key = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    k = pg.KeySwitchKey(pg.to_device(key))
    ct = O.random_residues(rng, mods[:6], n, 2)
    c2 = O.random_residues(rng, mods[:6], n, 1)[0]
    want_ntt = oc.ntt_fwd(a[0])
    want_ks = oc.keyswitch(6, ct, c2, key)
    for l1 in splits:
        ctx.ntt_split = l1
        assert ctx.ntt_split == l1
        t = pg.to_device(a)
        ctx.ntt_forward(t, 1, len(mods))
        _eq(t, want_ntt, f"forward NTT, split {l1}/{log_n - l1}")
        ctx.ntt_inverse(t, 1, len(mods))
        _eq(t, a, f"round trip, split {l1}/{log_n - l1}")
        tk = pg.to_device(ct)
        ctx.keyswitch(ws, tk, pg.to_device(c2), 1, k)
        _eq(tk, want_ks, f"keyswitch, split {l1}/{log_n - l1}")
    with pytest.raises(pg.InvalidArgument):
        ctx.ntt_split = 5
    tuned = ctx.autotune_ntt_split()
    assert tuned["ntt_split"] in splits and ctx.ntt_split == tuned["ntt_split"]


@pytest.mark.parametrize("log_n", [12, 13, 16])
def test_small_launch_kernels_give_the_same_words(pg, log_n):
    """NTT passes with 8 coefficients per thread (small launches, on 1024- or 2048-coefficient
    tiles) and with 16 (on 2048- or 4096-coefficient tiles) give the same words: every pass
    forced to one shape, then the others, on the NTT, a key switch and HMult."""
    n = 1 << log_n
    bits = [60] + [40] * 5 + [60, 60]
    mods = pg.create_coeff_modulus(n, bits)
    ctx = pg.Context(n, mods, 2)
    oc = O.Context(log_n, mods, 6, 2)
    ws = ctx.workspace()
    rng = np.random.default_rng(100 + log_n)
    x = O.random_residues(rng, mods, n, 2)
    key = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    k = pg.KeySwitchKey(pg.to_device(key))
    ct = O.random_residues(rng, mods[:6], n, 2)
    c2 = O.random_residues(rng, mods[:6], n, 1)[0]
    a = O.random_residues(rng, mods[:6], n, 2)
    b = O.random_residues(rng, mods[:6], n, 2)
    want_ntt = oc.ntt_fwd(x.reshape(-1, n), tbl=list(range(len(mods))) * 2).reshape(x.shape)
    want_ks = oc.keyswitch(6, ct, c2, key)
    want_hm = oc.rescale(6, oc.ckks_mul_relin(6, a, b, key))
    # (small-launch bound, coefficients per CTA at 8 per thread, at 16 per thread)
    for tiles, small, large in ((0, 1024, 4096), (0, 1024, 2048), (1 << 30, 2048, 2048),
                                (1 << 30, 1024, 2048), (-1, 1024, 2048)):
        ctx.ntt_small_launch = tiles
        ctx.ntt_small_tile = small
        ctx.ntt_tile = large
        what = f"small-launch bound {tiles}, tiles {small} / {large}"
        t = pg.to_device(x)
        ctx.ntt_forward(t, 2, len(mods))
        _eq(t, want_ntt, f"forward NTT, {what}")
        ctx.ntt_inverse(t, 2, len(mods))
        _eq(t, x, f"round trip, {what}")
        tk = pg.to_device(ct)
        ctx.keyswitch(ws, tk, pg.to_device(c2), 1, k)
        _eq(tk, want_ks, f"keyswitch, {what}")
        out = torch.empty((2, 5, n), dtype=torch.int64, device="cuda")
        ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, 1, k)
        _eq(out, want_hm, f"HMult, {what}")
    assert (ctx.ntt_small_launch, ctx.ntt_small_tile, ctx.ntt_tile) == (512 if log_n >= 16 else 1024, 1024, 2048)
    with pytest.raises(pg.InvalidArgument):
        ctx.ntt_small_launch = -2
    with pytest.raises(pg.InvalidArgument):
        ctx.ntt_small_tile = 4096
    with pytest.raises(pg.InvalidArgument):
        ctx.ntt_tile = 1024


@pytest.mark.parametrize("log_n", [12, 14])
def test_launch_overlap_off_gives_the_same_words(pg, log_n):
    """Programmatic dependent launch changes only when a kernel may be scheduled: with it switched
    off (plain stream order) the NTT (the cluster kernel at 2^12), a key switch, a rotation and
    HMult + relin + rescale give the oracle's words, as they do with it on."""
    n = 1 << log_n
    bits = [60] + [40] * 5 + [60, 60]
    mods = pg.create_coeff_modulus(n, bits)
    elt = pg.elt_from_step(1, n)
    ctx = pg.Context(n, mods, 2, galois_elts=[elt])
    oc = O.Context(log_n, mods, 6, 2)
    ws = ctx.workspace()
    rng = np.random.default_rng(300 + log_n)
    x = O.random_residues(rng, mods[:3], n, 1)
    key = O.random_residues(rng, mods, n, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), n)
    k = pg.KeySwitchKey(pg.to_device(key))
    ct = O.random_residues(rng, mods[:6], n, 2)
    c2 = O.random_residues(rng, mods[:6], n, 1)[0]
    a = O.random_residues(rng, mods[:6], n, 2)
    b = O.random_residues(rng, mods[:6], n, 2)
    want_ntt = oc.ntt_fwd(x[0], [0, 1, 2])
    want_ks = oc.keyswitch(6, ct, c2, key)
    want_rot = oc.ckks_apply_galois(6, ct, elt, key)
    want_hm = oc.rescale(6, oc.ckks_mul_relin(6, a, b, key))
    for on in (False, True):
        ctx.launch_overlap = on
        assert ctx.launch_overlap == on
        t = pg.to_device(x)
        ctx.ntt_forward(t, 1, 3)
        _eq(t, want_ntt, f"forward NTT, overlap {on}")
        ctx.ntt_inverse(t, 1, 3)
        _eq(t, x, f"round trip, overlap {on}")
        tk = pg.to_device(ct)
        ctx.keyswitch(ws, tk, pg.to_device(c2), 1, k)
        _eq(tk, want_ks, f"keyswitch, overlap {on}")
        tr = pg.to_device(ct)
        ctx.rotate(ws, tr, 1, 1, [k])
        _eq(tr, want_rot, f"rotate, overlap {on}")
        out = torch.empty((2, 5, n), dtype=torch.int64, device="cuda")
        ctx.multiply_relin_rescale(ws, pg.to_device(a), pg.to_device(b), out, 1, k)
        _eq(out, want_hm, f"HMult, overlap {on}")
