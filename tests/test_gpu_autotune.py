"""The operation autotuner (fhe_context_autotune_op): every shape it searches gives the
reference's words, and its choice round-trips through the cache file."""
import hashlib
import itertools
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.json")


def sha(t):
    return hashlib.sha256(np.ascontiguousarray(t.cpu().numpy().view(np.uint64), dtype="<u8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def pg():
    import phantom_gb300
    return phantom_gb300


@pytest.fixture(scope="module")
def hmult_case(pg):
    """HMult + relinearise + rescale at N = 2^16, l = 30, dnum = 6 (the benchmark workload) on the
    inputs of the reference-kernel digest hmult_ckks_n16_l30."""
    with open(GOLDEN) as f:
        g = json.load(f)["hmult_ckks_n16_l30"]
    n, l = 1 << g["log_n"], g["l"]
    mods = pg.create_coeff_modulus(n, g["bits"])
    rng = np.random.default_rng(g["seed"])
    dnum = -(-(len(g["bits"]) - g["special"]) // g["special"])
    evk = O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    return g, mods, pg.to_device(evk), pg.to_device(a), pg.to_device(b)


def _context(pg, g, mods):
    ctx = pg.Context(1 << g["log_n"], mods, g["special"])
    return ctx, ctx.workspace()


def _hmult(pg, ctx, ws, g, key, a, b):
    l = g["l"]
    out = torch.empty((2, l - 1, ctx.n), dtype=torch.int64, device="cuda")
    ctx.multiply_relin_rescale(ws, a, b, out, len(g["bits"]) - g["special"] - l + 1, key)
    return out


def test_every_searched_shape_gives_the_reference_words(pg, hmult_case):
    g, mods, evk, a, b = hmult_case
    ctx, ws = _context(pg, g, mods)
    key = pg.KeySwitchKey(evk)
    base = ctx.tuning
    variants = [{"ntt_split": s} for s in (7, 8)]
    variants += [{"ntt_small_launch": v} for v in (0, 256, 512, 1024, 2048, 4096)]
    variants += [{"tensor_cores": v} for v in (0, 1)]
    variants += [{"ntt_tile": t, "ntt_small_tile": st, "fused_keyswitch": f}
                 for t, st, f in itertools.product((2048, 4096), (1024, 2048), (0, 1))]
    for v in variants:
        ctx.tuning = dict(base, **v)
        assert sha(_hmult(pg, ctx, ws, g, key, a, b)) == g["rescaled"], f"shape {v}"
    assert ctx.device_status() == 0


def test_autotuner_choice_and_cache(pg, hmult_case, tmp_path):
    g, mods, evk, a, b = hmult_case
    key = pg.KeySwitchKey(evk)
    cache = str(tmp_path / "tuning.jsonl")
    ctx, ws = _context(pg, g, mods)
    tuned = ctx.autotune(ws, cache_path=cache)
    assert tuned["evaluated"] > 10 and tuned["best_us"] > 0
    assert {k: tuned[k] for k in ctx.tuning if k not in ("best_us", "evaluated")} == \
           {k: v for k, v in ctx.tuning.items() if k not in ("best_us", "evaluated")}
    assert sha(_hmult(pg, ctx, ws, g, key, a, b)) == g["rescaled"]
    with open(cache) as f:
        lines = [json.loads(x) for x in f if x.strip()]
    assert len(lines) == 1 and "|ckks|N=65536|Q=30|P=5|batch=1" in lines[0]["key"]
    ctx2, ws2 = _context(pg, g, mods)
    again = ctx2.autotune(ws2, cache_path=cache)
    assert again["evaluated"] == 0
    for k in ("ntt_split", "ntt_tile", "ntt_small_tile", "ntt_small_launch", "fused_keyswitch", "tensor_cores"):
        assert again[k] == tuned[k]
    assert sha(_hmult(pg, ctx2, ws2, g, key, a, b)) == g["rescaled"]
