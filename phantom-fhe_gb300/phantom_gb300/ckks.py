"""CKKS host side: the encoder front end (the FP64 canonical embedding runs on the GPU, bit for
bit the reference's) and secret-key material with seeded randomness.

Encoder (PhantomCKKSEncoder, src/ckks.cu:17-400): slot i of a plaintext holds
m(zeta^(5^i mod 2N)) / scale, zeta = exp(i*pi/N), for i < N/2.  encode / decode call
fhe_ckks_encode / fhe_ckks_decode: the reference's special FFT in FP64, its rounding and residues,
and on decode the CRT compose over every limb of the plaintext, so any message below Q_l / 2
round-trips and the words equal the reference encoder's.

Keys (PhantomSecretKey, src/secretkey.cu:232-460): a uniform ternary secret, uniform `a`
polynomials and errors from the reference's centred binomial distribution (difference of the
popcounts of two 21-bit words, standard deviation ~3.24, src/prng.cu:222-244) drawn from a
numpy Generator the caller seeds, so a run is reproducible; the arithmetic (NTT of s,
a*s + e, P*s_src) runs on the GPU through the C ABI.
"""
import numpy as np

from . import Context, KeySwitchKey, to_device

CBD_BITS = 21  # e = popcount(21 random bits) - popcount(21 random bits)


def rotation_group(n):
    """5^i mod 2N for i < N/2 (src/ckks.cu:36-46)."""
    m = 2 * n
    g = np.empty(n // 2, dtype=np.int64)
    pos = 1
    for i in range(n // 2):
        g[i] = pos
        pos = (pos * 5) % m
    return g


class CkksEncoder:
    """GPU encoder for one context degree; keeps one workspace per context it has served."""

    def __init__(self, n):
        self.n = n
        self.slots = n // 2
        self.group = rotation_group(n)
        self._ws = {}

    def _workspace(self, ctx, ws):
        if ws is not None:
            return ws
        w = self._ws.get(id(ctx))
        if w is None or w[0] is not ctx:
            w = self._ws[id(ctx)] = (ctx, ctx.workspace())
        return w[1]

    @staticmethod
    def to_rns(coeffs, moduli):
        """int64 coefficients -> uint64 residues [len(moduli)][N]."""
        c = np.asarray(coeffs, dtype=np.int64)
        return np.stack([np.mod(c, np.int64(q)).astype(np.uint64) for q in moduli])

    def encode(self, ctx, values, scale, chain_index, ws=None):
        """Complex slot values (1..N/2 of them) -> device plaintext [limbs][N] in NTT form."""
        import torch
        v = np.asarray(values, dtype=np.complex128).reshape(-1)
        vt = torch.from_numpy(np.stack([v.real, v.imag], axis=1).copy()).cuda()
        l = ctx.level(chain_index)
        pt = torch.empty((l, ctx.n), dtype=torch.int64, device="cuda")
        ctx.ckks_encode(self._workspace(ctx, ws), vt, scale, chain_index, pt)
        return pt

    def decode(self, ctx, pt, scale, chain_index, ws=None):
        """Device plaintext (NTT form) -> N/2 complex slots (numpy), composed over every limb."""
        import torch
        out = torch.empty((self.slots, 2), dtype=torch.float64, device="cuda")
        ctx.ckks_decode(self._workspace(ctx, ws), pt, scale, chain_index, out)
        o = out.cpu().numpy()
        return o[:, 0] + 1j * o[:, 1]


class SecretKey:
    """Ternary secret with its NTT form over every QP limb, plus seeded key generation and
    symmetric encryption."""

    def __init__(self, ctx: Context, rng: np.random.Generator):
        self.ctx = ctx
        self.rng = rng
        qp = ctx.size_q + ctx.size_p
        self.coeffs = rng.integers(-1, 2, size=ctx.n, dtype=np.int64)
        self.s_ntt = to_device(CkksEncoder.to_rns(self.coeffs, ctx.moduli[:qp]))
        ctx.ntt_forward(self.s_ntt, 1, qp)

    def _uniform(self, polys, limbs):
        n = self.ctx.n
        out = np.empty((polys, limbs, n), dtype=np.uint64)
        for j in range(limbs):
            out[:, j, :] = self.rng.integers(0, self.ctx.moduli[j], size=(polys, n), dtype=np.uint64)
        return out

    def _error(self, polys):
        shape = (polys, self.ctx.n)
        return (self.rng.binomial(CBD_BITS, 0.5, size=shape) - self.rng.binomial(CBD_BITS, 0.5, size=shape)).astype(
            np.int64)

    def kswitch_key(self, ws, galois_elt=0):
        """Relinearisation key (galois_elt 0) or the Galois key of galois_elt."""
        import torch
        ctx = self.ctx
        qp = ctx.size_q + ctx.size_p
        a = to_device(self._uniform(ctx.dnum, qp))
        e = torch.from_numpy(self._error(ctx.dnum)).cuda()
        key = torch.empty((ctx.dnum, 2, qp, ctx.n), dtype=torch.int64, device="cuda")
        ctx.kswitch_keygen(ws, galois_elt, self.s_ntt, a, e, key)
        torch.cuda.current_stream().synchronize()
        return KeySwitchKey(key)

    def galois_keys(self, ws, steps):
        """List aligned with ctx.galois_elts: a key for each rotation step given, None elsewhere."""
        from . import elt_from_step
        want = {elt_from_step(s, self.ctx.n) for s in steps}
        return [self.kswitch_key(ws, g) if g in want else None for g in self.ctx.galois_elts]

    def encrypt(self, pt, chain_index):
        """pt: device plaintext [limbs][N] (NTT form) or None for an encryption of zero."""
        import torch
        ctx = self.ctx
        l = ctx.level(chain_index)
        a = to_device(self._uniform(1, l)[0])
        e = torch.from_numpy(self._error(1)[0]).cuda()
        out = torch.empty((2, l, ctx.n), dtype=torch.int64, device="cuda")
        ctx.encrypt_symmetric(pt, self.s_ntt, a, e, out, chain_index)
        return out

    def decrypt(self, ct, chain_index):
        import torch
        l = self.ctx.level(chain_index)
        pt = torch.empty((l, self.ctx.n), dtype=torch.int64, device="cuda")
        self.ctx.decrypt(ct, self.s_ntt, pt, chain_index)
        return pt
