"""CKKS host side: canonical-embedding encoder/decoder (FP64) and secret-key material with
seeded randomness.

Encoder (restates PhantomCKKSEncoder, src/ckks.cu:17-140 and its decode path): slot i of a
plaintext holds m(zeta^(5^i mod 2N)) / scale, zeta = exp(i*pi/N), for i < N/2; the conjugate
slots hold the conjugates, so m has real coefficients.  The reference evaluates the embedding
with its own special FFT on the device; here it is one length-2N numpy FFT per direction in
FP64, which gives the same rounded integer coefficients except where a coefficient lies within
FP64 rounding of a half-integer, and the same decoded slots to FP64 accuracy.  Only the
embedding runs on the host; residues, NTT and every ciphertext operation run on the device.

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
    def __init__(self, n):
        self.n = n
        self.slots = n // 2
        self.group = rotation_group(n)

    def encode_coeffs(self, values, scale):
        """Complex slot values (<= N/2 of them, zero-padded) -> int64 coefficients of
        round(scale * m)."""
        n = self.n
        z = np.zeros(self.slots, dtype=np.complex128)
        v = np.asarray(values, dtype=np.complex128)
        if v.size == 0 or v.size > self.slots:
            raise ValueError("need 1..N/2 slot values")
        z[: v.size] = v
        # m_k = (1/N) sum_i (z_i zeta^(-g_i k) + conj(z_i) zeta^(g_i k)) = (2/N) Re(sum_i z_i zeta^(-g_i k))
        w = np.zeros(2 * n, dtype=np.complex128)
        w[self.group] = z
        coeffs = np.fft.fft(w)[:n].real * (2.0 * scale / n)
        if np.max(np.abs(coeffs)) >= 2.0 ** 62:
            raise ValueError("encoded values are too large")
        return np.rint(coeffs).astype(np.int64)

    def decode_coeffs(self, coeffs, scale):
        """Real coefficients (float or int) -> N/2 complex slots."""
        n = self.n
        c = np.zeros(2 * n, dtype=np.complex128)
        c[:n] = np.asarray(coeffs, dtype=np.float64)
        v = np.fft.ifft(c) * (2 * n)  # v_j = sum_k c_k zeta^(j k)
        return v[self.group] / scale

    @staticmethod
    def to_rns(coeffs, moduli):
        """int64 coefficients -> uint64 residues [len(moduli)][N]."""
        c = np.asarray(coeffs, dtype=np.int64)
        return np.stack([np.mod(c, np.int64(q)).astype(np.uint64) for q in moduli])

    @staticmethod
    def centered(residues, q):
        """Residues of one limb -> centred integers (float64), valid when |m| < q / 2."""
        r = np.asarray(residues, dtype=np.uint64)
        half = np.uint64(q // 2)
        return np.where(r > half, -(np.uint64(q) - r).astype(np.float64), r.astype(np.float64))

    def encode(self, ctx, values, scale, chain_index):
        """-> device plaintext [limbs][N] in NTT form at chain_index."""
        l = ctx.level(chain_index)
        pt = to_device(self.to_rns(self.encode_coeffs(values, scale), ctx.moduli[:l]))
        ctx.ntt_forward(pt, 1, l)
        return pt

    def decode(self, ctx, pt, scale, chain_index):
        """Device plaintext (NTT form) -> complex slots, reading limb 0 (q_0 is the largest
        prime of the chain; the message must stay below q_0 / 2)."""
        l = ctx.level(chain_index)
        t = pt.clone()
        ctx.ntt_inverse(t, 1, l)
        limb0 = t[0].cpu().numpy().view(np.uint64)
        return self.decode_coeffs(self.centered(limb0, ctx.moduli[0]), scale)


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
