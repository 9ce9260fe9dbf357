"""fhe_rescale_to_next_noalloc — the rescale for callers that may not allocate device memory
(a plugin whose host process owns all device memory, or a path that must not risk an
allocation), checked word for word against the workspace-based fhe_rescale_to_next through
the C ABI, on consecutive calls.  Collected last so that a stop-at-first-failure run has
already run every other test."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def pg():
    import phantom_gb300
    return phantom_gb300


def _call_noalloc(pg, ctx, src, dst, size, chain):
    lib = pg.lib
    return lib.fhe_rescale_to_next_noalloc(ctx._h, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                                           size, chain, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("log_n,bits,special,calls", [
    (16, [60] + [40] * 29 + [60] * 5, 5, ((1, 2), (3, 3), (1, 2))),
    (12, [60, 40, 40, 40, 40, 40, 60, 60], 2, ((1, 2), (3, 3), (1, 2))),
    # size * N = 2^18 exactly: the largest request the scratch accepts, twice in a row
    (17, [60, 40, 40, 40, 40, 60, 60], 2, ((1, 2), (2, 2))),
])
def test_noalloc_rescale_matches_workspace_rescale(pg, log_n, bits, special, calls):
    n = 1 << log_n
    mods = pg.create_coeff_modulus(n, bits)
    ctx = pg.Context(n, mods, special)
    ws = ctx.workspace()
    rng = np.random.default_rng(99 + log_n)
    for chain, size in calls:  # consecutive calls share the scratch
        l = ctx.level(chain)
        ct = pg.to_device(O.random_residues(rng, mods[:l], n, size))
        want = torch.empty((size, l - 1, n), dtype=torch.int64, device="cuda")
        got = torch.full((size, l - 1, n), -1, dtype=torch.int64, device="cuda")
        ctx.rescale_to_next(ws, ct, want, size, chain)
        assert _call_noalloc(pg, ctx, ct, got, size, chain) == 0, pg.lib.fhe_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, want)


@pytest.mark.parametrize("log_n,size", [(16, 5), (17, 3)])  # 5 * 2^16 and 3 * 2^17 words > 2^18
def test_noalloc_rescale_rejects_sizes_beyond_its_scratch(pg, log_n, size):
    n = 1 << log_n
    mods = pg.create_coeff_modulus(n, [60] + [40] * 5 + [60])
    ctx = pg.Context(n, mods, 1)
    l = ctx.level(1)
    ct = torch.zeros((size, l, n), dtype=torch.int64, device="cuda")
    out = torch.zeros((size, l - 1, n), dtype=torch.int64, device="cuda")
    assert _call_noalloc(pg, ctx, ct, out, size, 1) == -1
    assert b"exceeds the no-allocation scratch" in pg.lib.fhe_last_error()
