"""ctypes front end of the CPU oracle (oracle/fhe_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by the
CPU-baseline leg of bench.py, always as the checker.  The GPU product path never
imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfhe_oracle.so")

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_intp = ctypes.POINTER(ctypes.c_int)
_dblp = ctypes.POINTER(ctypes.c_double)
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-f", os.path.join(HERE, "Makefile")])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_mulmod.restype = ctypes.c_uint64
        L.orc_mulmod.argtypes = [ctypes.c_uint64] * 3
        L.orc_invmod.restype = ctypes.c_uint64
        L.orc_invmod.argtypes = [ctypes.c_uint64] * 2
        L.orc_is_prime.argtypes = [ctypes.c_uint64]
        L.orc_shoup.restype = ctypes.c_uint64
        L.orc_shoup.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_barrett_ratio.argtypes = [ctypes.c_uint64, _u64p]
        L.orc_get_primes.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _u64p]
        L.orc_get_primes_below.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, _u64p]
        L.orc_create_coeff_modulus.argtypes = [ctypes.c_uint64, _intp, ctypes.c_int, _u64p]
        L.orc_minimal_root.restype = ctypes.c_uint64
        L.orc_minimal_root.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_ntt_tables.argtypes = [ctypes.c_int, ctypes.c_uint64, _u64p, _u64p, _u64p, _u64p, _u64p]
        L.orc_ctx_create.restype = ctypes.c_void_p
        L.orc_ctx_create.argtypes = [ctypes.c_int, _u64p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64]
        L.orc_ctx_destroy.argtypes = [ctypes.c_void_p]
        L.orc_ctx_hps_r.argtypes = [ctypes.c_void_p, _u64p]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        for f in ("orc_ntt_fwd", "orc_ntt_inv"):
            getattr(L, f).argtypes = [ctypes.c_void_p, _u64p, ctypes.c_int, _intp]
        for f in ("orc_ntt_fwd_qr", "orc_ntt_inv_qr"):
            getattr(L, f).argtypes = [ctypes.c_void_p, _u64p, ctypes.c_int]
        L.orc_tensor.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, _u64p]
        L.orc_tensor_square.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p]
        L.orc_modup.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, ctypes.c_int]
        L.orc_inner_product.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, _u64p]
        L.orc_moddown.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, ctypes.c_int]
        L.orc_keyswitch.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, _u64p, ctypes.c_int]
        L.orc_relinearize.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, ctypes.c_int]
        L.orc_ckks_mul_relin.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, _u64p, _u64p]
        L.orc_rescale.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _u64p, _u64p]
        L.orc_divide_round_q_last.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _u64p, _u64p]
        L.orc_mul_add.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _u64p, _u64p, _u64p]
        L.orc_elt_from_step.restype = ctypes.c_uint32
        L.orc_elt_from_step.argtypes = [ctypes.c_int, ctypes.c_uint64]
        L.orc_galois_perm.argtypes = [ctypes.c_int, ctypes.c_uint32, _u32p]
        L.orc_apply_galois_ntt.argtypes = [ctypes.c_void_p, _u64p, _u64p, ctypes.c_int, ctypes.c_uint32]
        L.orc_apply_galois_coeff.argtypes = [ctypes.c_void_p, _u64p, _u64p, ctypes.c_int, ctypes.c_uint32]
        L.orc_ckks_apply_galois.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, ctypes.c_uint32, _u64p]
        L.orc_ckks_hoisting.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u32p, ctypes.c_int,
                                        ctypes.POINTER(_u64p)]
        for f in ("orc_hps_bconv_q_to_r", "orc_hps_bconv_r_to_q", "orc_hps_scale_round_qr_r"):
            getattr(L, f).argtypes = [ctypes.c_void_p, _u64p, _u64p]
        L.orc_bfv_mul_relin_hps.argtypes = [ctypes.c_void_p, _u64p, _u64p, _u64p, _u64p]
        L.orc_modup_tables.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _u64p, _u64p]
        L.orc_moddown_tables.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, _u64p]
        L.orc_hps_tables.argtypes = [ctypes.c_void_p, _dblp, _u64p]
        L.orc_sample_uniform.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, _u64p]
        L.orc_sample_small.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
        L.orc_kswitch_key_combine.argtypes = [ctypes.c_void_p, _u64p, _u64p, _u64p, _u64p, _u64p]
        _lib = L
    return _lib


def p64(a):
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_u64p)


def set_threads(n):
    lib().orc_set_threads(int(n))


def create_coeff_modulus(n, bits):
    out = np.zeros(len(bits), dtype=np.uint64)
    b = (ctypes.c_int * len(bits))(*bits)
    if lib().orc_create_coeff_modulus(n, b, len(bits), p64(out)):
        raise ValueError("not enough primes")
    return [int(x) for x in out]


def get_primes_below(n, upper, count):
    out = np.zeros(count, dtype=np.uint64)
    if lib().orc_get_primes_below(n, upper, count, p64(out)):
        raise ValueError("not enough primes")
    return [int(x) for x in out]


def ntt_tables(log_n, q):
    n = 1 << log_n
    arrs = [np.zeros(n, dtype=np.uint64) for _ in range(4)]
    ninv = np.zeros(1, dtype=np.uint64)
    if lib().orc_ntt_tables(log_n, q, *[p64(a) for a in arrs], p64(ninv)):
        raise ValueError("no 2N-th root")
    return arrs + [int(ninv[0])]


def barrett_ratio(q):
    out = np.zeros(3, dtype=np.uint64)
    lib().orc_barrett_ratio(q, p64(out))
    return [int(x) for x in out]


def minimal_root(degree, q):
    return int(lib().orc_minimal_root(degree, q))


def elt_from_step(step, n):
    return int(lib().orc_elt_from_step(step, n))


def galois_perm(log_n, elt):
    out = np.zeros(1 << log_n, dtype=np.uint32)
    lib().orc_galois_perm(log_n, elt, out.ctypes.data_as(_u32p))
    return out


class Context:
    """Oracle context over QP = Q (n_q primes) followed by P (n_p special primes)."""

    def __init__(self, log_n, moduli, n_q, n_p, plain_modulus=0):
        self.log_n, self.n = log_n, 1 << log_n
        self.moduli = [int(m) for m in moduli]
        self.n_q, self.n_p = n_q, n_p
        arr = np.array(self.moduli, dtype=np.uint64)
        self._h = lib().orc_ctx_create(log_n, p64(arr), n_q, n_p, plain_modulus)
        if not self._h:
            raise ValueError("bad oracle parameters")
        self.r_moduli = []
        if plain_modulus:
            r = np.zeros(64, dtype=np.uint64)
            k = lib().orc_ctx_hps_r(self._h, p64(r))
            self.r_moduli = [int(x) for x in r[:k]]

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_ctx_destroy(self._h)
            self._h = None

    def qlp(self, l):
        return [self.moduli[j] if j < l else self.moduli[self.n_q + j - l] for j in range(l + self.n_p)]

    def beta(self, l):
        return (l + self.n_p - 1) // self.n_p

    def ntt_fwd(self, data, tbl=None):
        data = np.ascontiguousarray(data, dtype=np.uint64).copy()
        limbs = data.size // self.n
        t = None if tbl is None else (ctypes.c_int * limbs)(*tbl)
        lib().orc_ntt_fwd(self._h, p64(data), limbs, t)
        return data

    def ntt_inv(self, data, tbl=None):
        data = np.ascontiguousarray(data, dtype=np.uint64).copy()
        limbs = data.size // self.n
        t = None if tbl is None else (ctypes.c_int * limbs)(*tbl)
        lib().orc_ntt_inv(self._h, p64(data), limbs, t)
        return data

    def ntt_fwd_qr(self, data):
        data = np.ascontiguousarray(data, dtype=np.uint64).copy()
        lib().orc_ntt_fwd_qr(self._h, p64(data), data.size // self.n)
        return data

    def ntt_inv_qr(self, data):
        data = np.ascontiguousarray(data, dtype=np.uint64).copy()
        lib().orc_ntt_inv_qr(self._h, p64(data), data.size // self.n)
        return data

    def tensor(self, l, a, b):
        out = np.zeros((3, l, self.n), dtype=np.uint64)
        if a is b:
            lib().orc_tensor_square(self._h, l, p64(a), p64(out))
        else:
            lib().orc_tensor(self._h, l, p64(a), p64(b), p64(out))
        return out

    def modup(self, l, c2, scheme=0):
        out = np.zeros((self.beta(l), l + self.n_p, self.n), dtype=np.uint64)
        lib().orc_modup(self._h, l, p64(np.ascontiguousarray(c2)), p64(out), scheme)
        return out

    def inner_product(self, l, tm, evk):
        out = np.zeros((2, l + self.n_p, self.n), dtype=np.uint64)
        lib().orc_inner_product(self._h, l, p64(tm), p64(evk), p64(out))
        return out

    def moddown(self, l, cx, scheme=0):
        cx = np.ascontiguousarray(cx, dtype=np.uint64).copy()
        out = np.zeros((l, self.n), dtype=np.uint64)
        lib().orc_moddown(self._h, l, p64(cx), p64(out), scheme)
        return out

    def keyswitch(self, l, ct, c2, evk, scheme=0):
        ct = np.ascontiguousarray(ct, dtype=np.uint64).copy()
        lib().orc_keyswitch(self._h, l, p64(ct), p64(np.ascontiguousarray(c2)), p64(evk), scheme)
        return ct

    def relinearize(self, l, ct3, rlk, scheme=0):
        ct3 = np.ascontiguousarray(ct3, dtype=np.uint64).copy()
        lib().orc_relinearize(self._h, l, p64(ct3), p64(rlk), scheme)
        return ct3[:2].copy()

    def ckks_mul_relin(self, l, a, b, rlk):
        out = np.zeros((2, l, self.n), dtype=np.uint64)
        lib().orc_ckks_mul_relin(self._h, l, p64(a), p64(b), p64(rlk), p64(out))
        return out

    def rescale(self, l, ct):
        size = ct.size // (l * self.n)
        out = np.zeros((size, l - 1, self.n), dtype=np.uint64)
        lib().orc_rescale(self._h, l, size, p64(np.ascontiguousarray(ct)), p64(out))
        return out

    def divide_round_q_last(self, l, ct):
        size = ct.size // (l * self.n)
        out = np.zeros((size, l - 1, self.n), dtype=np.uint64)
        lib().orc_divide_round_q_last(self._h, l, size, p64(np.ascontiguousarray(ct)), p64(out))
        return out

    def mul_add(self, l, acc, a, b):
        """acc (polys x l x N) += a (polys x l x N) * b (l x N) mod q, in place."""
        assert acc.flags["C_CONTIGUOUS"] and acc.dtype == np.uint64
        polys = acc.size // (l * self.n)
        lib().orc_mul_add(self._h, l, polys, p64(np.ascontiguousarray(a, dtype=np.uint64)),
                          p64(np.ascontiguousarray(b, dtype=np.uint64)), p64(acc))
        return acc

    def apply_galois_ntt(self, src, elt):
        src = np.ascontiguousarray(src, dtype=np.uint64)
        out = np.zeros_like(src)
        lib().orc_apply_galois_ntt(self._h, p64(src), p64(out), src.size // self.n, elt)
        return out

    def apply_galois_coeff(self, src, elt):
        src = np.ascontiguousarray(src, dtype=np.uint64)
        out = np.zeros_like(src)
        lib().orc_apply_galois_coeff(self._h, p64(src), p64(out), src.size // self.n, elt)
        return out

    def ckks_apply_galois(self, l, ct, elt, gk):
        ct = np.ascontiguousarray(ct, dtype=np.uint64).copy()
        lib().orc_ckks_apply_galois(self._h, l, p64(ct), elt, p64(gk))
        return ct

    def ckks_hoisting(self, l, ct, elts, gks):
        ct = np.ascontiguousarray(ct, dtype=np.uint64).copy()
        e = (ctypes.c_uint32 * len(elts))(*elts)
        ptrs = (_u64p * len(gks))(*[p64(g) for g in gks])
        lib().orc_ckks_hoisting(self._h, l, p64(ct), e, len(elts), ptrs)
        return ct

    def hps_bconv_q_to_r(self, x):
        out = np.zeros((len(self.r_moduli), self.n), dtype=np.uint64)
        lib().orc_hps_bconv_q_to_r(self._h, p64(np.ascontiguousarray(x)), p64(out))
        return out

    def hps_bconv_r_to_q(self, x):
        out = np.zeros((self.n_q, self.n), dtype=np.uint64)
        lib().orc_hps_bconv_r_to_q(self._h, p64(np.ascontiguousarray(x)), p64(out))
        return out

    def hps_scale_round_qr_r(self, x):
        out = np.zeros((len(self.r_moduli), self.n), dtype=np.uint64)
        lib().orc_hps_scale_round_qr_r(self._h, p64(np.ascontiguousarray(x)), p64(out))
        return out

    def bfv_mul_relin_hps(self, a, b, rlk):
        out = np.zeros((2, self.n_q, self.n), dtype=np.uint64)
        lib().orc_bfv_mul_relin_hps(self._h, p64(a), p64(b), p64(rlk), p64(out))
        return out

    def modup_tables(self, l, d):
        phi = np.zeros(self.n_p, dtype=np.uint64)
        mat = np.zeros(self.n_p * (l + self.n_p), dtype=np.uint64)
        sz = lib().orc_modup_tables(self._h, l, d, p64(phi), p64(mat))
        return phi[:sz], mat[: sz * (l + self.n_p - sz)]

    def moddown_tables(self, l):
        phi = np.zeros(self.n_p, dtype=np.uint64)
        mat = np.zeros(l * self.n_p, dtype=np.uint64)
        pinv = np.zeros(l, dtype=np.uint64)
        lib().orc_moddown_tables(self._h, l, p64(phi), p64(mat), p64(pinv))
        return phi, mat, pinv

    def sample_uniform(self, seed, limbs):
        """The reference's sample_uniform_poly: [limbs][N] modulo QP primes 0..limbs-1."""
        out = np.zeros((limbs, self.n), dtype=np.uint64)
        lib().orc_sample_uniform(self._h, bytes(seed), limbs, p64(out))
        return out

    def sample_small(self, seed, kind):
        """kind 0: sample_ternary_poly, 1: sample_error_poly, as signed integers [N]."""
        out = np.zeros(self.n, dtype=np.int64)
        lib().orc_sample_small(self._h, bytes(seed), kind, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        return out

    def kswitch_key_combine(self, s, s_src, a, e_ntt):
        dnum = (self.n_q + self.n_p - 1) // self.n_p
        qp = self.n_q + self.n_p
        key = np.zeros((dnum, 2, qp, self.n), dtype=np.uint64)
        lib().orc_kswitch_key_combine(self._h, p64(np.ascontiguousarray(s)), p64(np.ascontiguousarray(s_src)),
                                      p64(np.ascontiguousarray(a)), p64(np.ascontiguousarray(e_ntt)), p64(key))
        return key

    def hps_tables(self):
        frac = np.zeros(self.n_q, dtype=np.float64)
        modr = np.zeros(len(self.r_moduli) * (self.n_q + 1), dtype=np.uint64)
        lib().orc_hps_tables(self._h, frac.ctypes.data_as(_dblp), p64(modr))
        return frac, modr


def random_residues(rng, moduli, n, polys=1):
    """Uniform residues [polys][len(moduli)][n], limb k in [0, moduli[k])."""
    out = np.empty((polys, len(moduli), n), dtype=np.uint64)
    for k, q in enumerate(moduli):
        out[:, k, :] = rng.integers(0, q, size=(polys, n), dtype=np.uint64)
    return out
