"""Python bindings of the GB300 RNS ciphertext-arithmetic library (C ABI in
include/phantom_gb300.h, shared library phantom-fhe_gb300/_build/libphantom_gb300.so).

Device buffers are torch CUDA tensors of dtype int64 holding the uint64 residues bit for
bit; layouts follow PhantomFHE (ciphertext [size][limbs][N], key [dnum][2][QP][N]).  The
library is the only compute path: importing this module fails loudly when the shared
library is missing, and every call raises on a non-zero status.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(HERE, "_build", "libphantom_gb300.so")

SCHEME_BFV, SCHEME_CKKS = 2, 3  # phantom::scheme_type values
MUL_TECH_HPS = 2

_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_u64 = ctypes.c_uint64


class FheError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"status {code}: {msg}")
        self.code = code


class InvalidArgument(FheError, ValueError):
    pass


class _Params(ctypes.Structure):
    _fields_ = [("scheme", ctypes.c_int), ("mul_tech", ctypes.c_int), ("poly_modulus_degree", _u64),
                ("coeff_modulus", ctypes.POINTER(_u64)), ("coeff_modulus_size", _sz),
                ("special_modulus_size", _sz), ("plain_modulus", _u64),
                ("galois_elts", ctypes.POINTER(ctypes.c_uint32)), ("galois_elts_size", _sz)]


class _MulItem(ctypes.Structure):
    _fields_ = [("ct1", _vp), ("ct2", _vp), ("out", _vp), ("chain_index", _sz)]


class _KsItem(ctypes.Structure):
    _fields_ = [("ct", _vp), ("c2", _vp), ("chain_index", _sz)]


class _MatvecItem(ctypes.Structure):
    _fields_ = [("ct", _vp), ("diags", _vp), ("out", _vp), ("chain_index", _sz), ("diag_limbs", _sz)]


class Tuning(ctypes.Structure):
    """fhe_tuning: the context's kernel shapes (every setting gives the same words)."""
    _fields_ = [("ntt_split", ctypes.c_int), ("ntt_tile", ctypes.c_int), ("ntt_small_tile", ctypes.c_int),
                ("ntt_small_launch", ctypes.c_int), ("fused_keyswitch", ctypes.c_int),
                ("tensor_cores", ctypes.c_int), ("best_us", ctypes.c_float), ("evaluated", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}

    @classmethod
    def from_dict(cls, d):
        t = cls()
        for f, _ in cls._fields_:
            setattr(t, f, type(getattr(t, f))(d[f]))
        return t


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build()")
    L = ctypes.CDLL(LIB_PATH)
    L.fhe_last_error.restype = ctypes.c_char_p
    L.fhe_galois_elt_from_step.restype = ctypes.c_uint32
    L.fhe_galois_elt_from_step.argtypes = [ctypes.c_int, _u64]
    L.fhe_create_coeff_modulus.argtypes = [_u64, ctypes.POINTER(ctypes.c_int), _sz, ctypes.POINTER(_u64)]
    L.fhe_context_create.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_vp)]
    L.fhe_context_destroy.argtypes = [_vp]
    L.fhe_context_set_tensor_cores.argtypes = [_vp, ctypes.c_int]
    L.fhe_context_tensor_cores.argtypes = [_vp]
    L.fhe_context_status.argtypes = [_vp, ctypes.POINTER(ctypes.c_uint)]
    L.fhe_context_ntt_split.argtypes = [_vp]
    L.fhe_context_set_ntt_split.argtypes = [_vp, ctypes.c_int]
    L.fhe_context_launch_overlap.argtypes = [_vp]
    L.fhe_context_set_launch_overlap.argtypes = [_vp, ctypes.c_int]
    L.fhe_context_fused_keyswitch.argtypes = [_vp]
    L.fhe_context_set_fused_keyswitch.argtypes = [_vp, ctypes.c_int]
    L.fhe_context_ntt_small_tile.argtypes = [_vp]
    L.fhe_context_set_ntt_small_tile.argtypes = [_vp, ctypes.c_int]
    L.fhe_context_ntt_tile.argtypes = [_vp]
    L.fhe_context_set_ntt_tile.argtypes = [_vp, ctypes.c_int]
    L.fhe_context_ntt_small_launch.argtypes = [_vp]
    L.fhe_context_set_ntt_small_launch.argtypes = [_vp, ctypes.c_int]
    L.fhe_context_autotune.argtypes = [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)]
    L.fhe_context_autotune_op.argtypes = [_vp, _vp, ctypes.c_char_p, _vp]
    L.fhe_context_tuning.argtypes = [_vp, _vp]
    L.fhe_context_set_tuning.argtypes = [_vp, _vp]
    L.fhe_context_sizes.argtypes = [_vp] + [ctypes.POINTER(_u64)] + [ctypes.POINTER(_sz)] * 4
    L.fhe_context_moduli.argtypes = [_vp, ctypes.POINTER(_u64)]
    L.fhe_context_galois_elts.argtypes = [_vp, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(_sz)]
    L.fhe_workspace_bytes.restype = _sz
    L.fhe_workspace_bytes.argtypes = [_vp]
    L.fhe_workspace_create.argtypes = [_vp, ctypes.POINTER(_vp)]
    L.fhe_workspace_destroy.argtypes = [_vp]
    L.fhe_workspace_create_batch.argtypes = [_vp, _sz, ctypes.POINTER(_vp)]
    L.fhe_ckks_multiply_relin_rescale_batch.argtypes = [_vp, _vp, ctypes.POINTER(_MulItem), _sz, _vp, _vp]
    L.fhe_keyswitch_batch.argtypes = [_vp, _vp, ctypes.POINTER(_KsItem), _sz, _vp, _vp]
    for f in ("fhe_ntt_forward", "fhe_ntt_inverse"):
        getattr(L, f).argtypes = [_vp, _vp, _sz, _sz, _sz, _vp]
    L.fhe_ckks_multiply.argtypes = [_vp, _vp, _vp, _sz, _vp]
    L.fhe_keyswitch.argtypes = [_vp, _vp, _vp, _vp, _sz, _vp, _vp]
    L.fhe_relinearize.argtypes = [_vp, _vp, _vp, _sz, _vp, _vp]
    L.fhe_multiply_and_relin.argtypes = [_vp, _vp, _vp, _vp, _sz, _vp, _vp]
    L.fhe_rescale_to_next.argtypes = [_vp, _vp, _vp, _vp, _sz, _sz, _vp]
    L.fhe_rescale_to_next_noalloc.argtypes = [_vp, _vp, _vp, _sz, _sz, _vp]
    L.fhe_bfv_mod_switch_to_next.argtypes = [_vp, _vp, _vp, _sz, _sz, _vp]
    L.fhe_ckks_multiply_relin_rescale.argtypes = [_vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]
    L.fhe_apply_galois.argtypes = [_vp, _vp, _vp, _sz, ctypes.c_uint32, _vp, _vp]
    L.fhe_rotate.argtypes = [_vp, _vp, _vp, _sz, ctypes.c_int, ctypes.POINTER(_vp), _vp]
    L.fhe_hoisting.argtypes = [_vp, _vp, _vp, _sz, ctypes.POINTER(ctypes.c_int), _sz, ctypes.POINTER(_vp), _vp]
    L.fhe_ckks_rotations_hoisted.argtypes = [_vp, _vp, _vp, _sz, ctypes.POINTER(ctypes.c_int), _sz,
                                             ctypes.POINTER(_vp), ctypes.POINTER(_vp), _vp]
    L.fhe_ckks_multiply_plain.argtypes = [_vp, _vp, _vp, _vp, _sz, _vp]
    L.fhe_ckks_add.argtypes = [_vp, _vp, _vp, _vp, _sz, _sz, _vp]
    L.fhe_bsgs_scratch_bytes.restype = _sz
    L.fhe_bsgs_scratch_bytes.argtypes = [_vp, _sz]
    L.fhe_bsgs_batch_scratch_bytes.restype = _sz
    L.fhe_bsgs_batch_scratch_bytes.argtypes = [_vp, _sz, _sz]
    L.fhe_ckks_bsgs_matvec.argtypes = [_vp, _vp, _vp, _vp, _sz, _vp, _sz, _sz, _sz, ctypes.POINTER(_vp), _vp,
                                       ctypes.c_int, _vp]
    L.fhe_ckks_bsgs_matvec_batch.argtypes = [_vp, _vp, _vp, ctypes.POINTER(_MatvecItem), _sz, _sz, _sz, _sz,
                                             ctypes.POINTER(_vp), _vp]
    L.fhe_ckks_encrypt_symmetric.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]
    L.fhe_ckks_decrypt.argtypes = [_vp, _vp, _vp, _vp, _sz, _vp]
    L.fhe_ckks_encode.argtypes = [_vp, _vp, _vp, _sz, ctypes.c_double, _sz, _vp, _vp]
    L.fhe_ckks_decode.argtypes = [_vp, _vp, _vp, _sz, ctypes.c_double, _vp, _vp]
    L.fhe_kswitch_keygen.argtypes = [_vp, _vp, ctypes.c_uint32, _vp, _vp, _vp, _vp, _vp]
    L.fhe_bfv_encode.argtypes = [_vp, _vp, _sz, _vp, _vp]
    L.fhe_bfv_decode.argtypes = [_vp, _vp, _vp, _vp, _vp]
    L.fhe_bfv_encrypt_symmetric.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.fhe_bfv_decrypt.argtypes = [_vp, _vp, _vp, _sz, _vp, _vp, _vp]
    L.fhe_sample_uniform.argtypes = [_vp, ctypes.c_char_p, _sz, _vp, _vp]
    L.fhe_sample_ternary.argtypes = [_vp, ctypes.c_char_p, _vp, _vp]
    L.fhe_sample_cbd.argtypes = [_vp, ctypes.c_char_p, _vp, _vp]
    L.fhe_secret_key_from_seed.argtypes = [_vp, _vp, ctypes.c_char_p, _vp, _vp]
    L.fhe_kswitch_keygen_seeded.argtypes = [_vp, _vp, ctypes.c_uint32, _vp, ctypes.c_char_p, ctypes.c_char_p, _vp,
                                            _vp]
    return L


lib = _load()


def _check(rc):
    if rc != 0:
        msg = lib.fhe_last_error().decode()
        raise (InvalidArgument if rc == -1 else FheError)(rc, msg)


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def create_coeff_modulus(n, bits):
    out = (_u64 * len(bits))()
    _check(lib.fhe_create_coeff_modulus(n, (ctypes.c_int * len(bits))(*bits), len(bits), out))
    return [int(x) for x in out]


def elt_from_step(step, n):
    return int(lib.fhe_galois_elt_from_step(step, n))


def to_device(a):
    """numpy uint64 array -> torch int64 CUDA tensor (same bits)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def to_host(t):
    return t.cpu().numpy().view(np.uint64)


class KeySwitchKey:
    """A key-switching key [dnum][2][QP][N] on the device plus the device array of its dnum
    digit pointers (the layout of PhantomRelinKey::public_keys_ptr())."""

    def __init__(self, data):
        import torch
        self.data = data
        ptrs = [data[d].data_ptr() for d in range(data.shape[0])]
        self.ptrs = torch.tensor(ptrs, dtype=torch.int64, device=data.device)

    @property
    def ptr(self):
        return ctypes.c_void_p(self.ptrs.data_ptr())


class Context:
    """PhantomContext equivalent: QP = Q (data primes) then P (special primes)."""

    def __init__(self, n, coeff_modulus, special_modulus_size, scheme=SCHEME_CKKS, plain_modulus=0,
                 galois_elts=None, mul_tech=MUL_TECH_HPS):
        mods = (_u64 * len(coeff_modulus))(*coeff_modulus)
        elts = list(galois_elts or [])
        p = _Params(scheme, mul_tech, n, mods, len(coeff_modulus), special_modulus_size, plain_modulus,
                    (ctypes.c_uint32 * max(1, len(elts)))(*elts), len(elts))
        h = _vp()
        _check(lib.fhe_context_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        self.n = n
        sizes = [_u64()] + [_sz() for _ in range(4)]
        _check(lib.fhe_context_sizes(h, *[ctypes.byref(x) for x in sizes]))
        self.size_q, self.size_p, self.size_r, self.dnum = (int(x.value) for x in sizes[1:])
        out = (_u64 * (self.size_q + self.size_p + self.size_r))()
        _check(lib.fhe_context_moduli(h, out))
        self.moduli = [int(x) for x in out]
        cnt = _sz()
        _check(lib.fhe_context_galois_elts(h, None, ctypes.byref(cnt)))
        e = (ctypes.c_uint32 * max(1, cnt.value))()
        _check(lib.fhe_context_galois_elts(h, e, ctypes.byref(cnt)))
        self.galois_elts = [int(x) for x in e[: cnt.value]]
        self.scheme = scheme

    def __del__(self):
        if getattr(self, "_h", None):
            lib.fhe_context_destroy(self._h)
            self._h = None

    @property
    def tensor_cores(self):
        """Whether the key switch's base conversions run on the tensor cores."""
        return bool(lib.fhe_context_tensor_cores(self._h))

    @tensor_cores.setter
    def tensor_cores(self, on):
        _check(lib.fhe_context_set_tensor_cores(self._h, int(bool(on))))

    @property
    def ntt_split(self):
        """Number of NTT stages in the column pass (the row pass runs the rest)."""
        return int(lib.fhe_context_ntt_split(self._h))

    @ntt_split.setter
    def ntt_split(self, l1):
        _check(lib.fhe_context_set_ntt_split(self._h, int(l1)))

    @property
    def launch_overlap(self):
        """Kernel chains launched with programmatic dependent launch (same words either way)."""
        return bool(lib.fhe_context_launch_overlap(self._h))

    @launch_overlap.setter
    def launch_overlap(self, on):
        _check(lib.fhe_context_set_launch_overlap(self._h, int(bool(on))))

    @property
    def fused_keyswitch(self):
        """Mod-up row pass fused with the key-switching inner product (same words either way)."""
        return bool(lib.fhe_context_fused_keyswitch(self._h))

    @fused_keyswitch.setter
    def fused_keyswitch(self, on):
        _check(lib.fhe_context_set_fused_keyswitch(self._h, int(bool(on))))

    @property
    def ntt_tile(self):
        """Coefficients per CTA (2048 or 4096) of the 16-per-thread NTT passes (same words)."""
        return int(lib.fhe_context_ntt_tile(self._h))

    @ntt_tile.setter
    def ntt_tile(self, coefficients):
        _check(lib.fhe_context_set_ntt_tile(self._h, int(coefficients)))

    @property
    def ntt_small_tile(self):
        """Coefficients per CTA (1024 or 2048) of the small-launch NTT passes (same words)."""
        return int(lib.fhe_context_ntt_small_tile(self._h))

    @ntt_small_tile.setter
    def ntt_small_tile(self, coefficients):
        _check(lib.fhe_context_set_ntt_small_tile(self._h, int(coefficients)))

    @property
    def ntt_small_launch(self):
        """NTT passes over at most this many 4096-coefficient tiles use 8 coefficients per thread."""
        return int(lib.fhe_context_ntt_small_launch(self._h))

    @ntt_small_launch.setter
    def ntt_small_launch(self, tiles):
        _check(lib.fhe_context_set_ntt_small_launch(self._h, int(tiles)))

    def autotune(self, ws=None, cache_path=None):
        """Chooses the kernel shapes (NTT split and tiles, small-launch bound, fused key switch,
        tensor-core conversions) by timing the context's benchmark operation at its top level
        (CKKS HMult + relinearise + rescale, BFV multiply + relinearise), and applies them.  With
        cache_path, a JSON-lines file keyed by GPU, scheme, N, |Q|, |P| and batch keeps the choice
        so later contexts skip the timing.  Returns the chosen shapes as a dict."""
        t = Tuning()
        w = ws if ws is not None else self.workspace()
        path = cache_path.encode() if cache_path else None
        _check(lib.fhe_context_autotune_op(self._h, w._h, path, ctypes.byref(t)))
        return t.as_dict()

    def autotune_ntt_split(self):
        """Times every supported NTT stage split on scratch limbs and keeps the fastest."""
        l1, us = ctypes.c_int(), ctypes.c_float()
        _check(lib.fhe_context_autotune(self._h, ctypes.byref(l1), ctypes.byref(us)))
        return {"ntt_split": int(l1.value), "roundtrip_us": float(us.value)}

    @property
    def tuning(self):
        t = Tuning()
        _check(lib.fhe_context_tuning(self._h, ctypes.byref(t)))
        return t.as_dict()

    @tuning.setter
    def tuning(self, d):
        t = Tuning.from_dict(dict(self.tuning, **d))
        _check(lib.fhe_context_set_tuning(self._h, ctypes.byref(t)))

    def device_status(self):
        """Reads and clears the device status word (0 = every bounded wait completed)."""
        v = ctypes.c_uint()
        _check(lib.fhe_context_status(self._h, ctypes.byref(v)))
        return int(v.value)

    def level(self, chain_index):
        return self.size_q - (chain_index - 1)

    def workspace_bytes(self):
        return int(lib.fhe_workspace_bytes(self._h))

    def workspace(self, batch_items=None):
        return Workspace(self, batch_items)

    # --- NTT
    def ntt_forward(self, data, num_polys, limbs, start=0, stream=None):
        _check(lib.fhe_ntt_forward(self._h, _ptr(data), num_polys, limbs, start, _stream(stream)))

    def ntt_inverse(self, data, num_polys, limbs, start=0, stream=None):
        _check(lib.fhe_ntt_inverse(self._h, _ptr(data), num_polys, limbs, start, _stream(stream)))

    # --- evaluator
    def ckks_multiply(self, ct1, ct2, chain_index, stream=None):
        _check(lib.fhe_ckks_multiply(self._h, _ptr(ct1), _ptr(ct2), chain_index, _stream(stream)))

    def keyswitch(self, ws, ct, c2, chain_index, key, stream=None):
        _check(lib.fhe_keyswitch(self._h, ws._h, _ptr(ct), _ptr(c2), chain_index, key.ptr, _stream(stream)))

    def relinearize(self, ws, ct, chain_index, key, stream=None):
        _check(lib.fhe_relinearize(self._h, ws._h, _ptr(ct), chain_index, key.ptr, _stream(stream)))

    def multiply_and_relin(self, ws, ct1, ct2, chain_index, key, stream=None):
        _check(lib.fhe_multiply_and_relin(self._h, ws._h, _ptr(ct1), _ptr(ct2), chain_index, key.ptr,
                                          _stream(stream)))

    def rescale_to_next(self, ws, src, dst, size, chain_index, stream=None):
        _check(lib.fhe_rescale_to_next(self._h, ws._h, _ptr(src), _ptr(dst), size, chain_index, _stream(stream)))

    def rescale_to_next_noalloc(self, src, dst, size, chain_index, stream=None):
        """Rescale without a workspace: for callers that may not allocate device memory."""
        _check(lib.fhe_rescale_to_next_noalloc(self._h, _ptr(src), _ptr(dst), size, chain_index, _stream(stream)))

    def bfv_mod_switch_to_next(self, src, dst, size, chain_index, stream=None):
        _check(lib.fhe_bfv_mod_switch_to_next(self._h, _ptr(src), _ptr(dst), size, chain_index, _stream(stream)))

    def multiply_relin_rescale(self, ws, ct1, ct2, out, chain_index, key, stream=None):
        _check(lib.fhe_ckks_multiply_relin_rescale(self._h, ws._h, _ptr(ct1), _ptr(ct2), _ptr(out), chain_index,
                                                   key.ptr, _stream(stream)))

    def multiply_relin_rescale_batch(self, ws, items, key, stream=None):
        """items: list of (ct1, ct2, out, chain_index), uneven chain indices allowed."""
        arr = (_MulItem * len(items))(*[_MulItem(t1.data_ptr(), t2.data_ptr(), o.data_ptr(), c)
                                        for t1, t2, o, c in items])
        _check(lib.fhe_ckks_multiply_relin_rescale_batch(self._h, ws._h, arr, len(items), key.ptr, _stream(stream)))

    def keyswitch_batch(self, ws, items, key, stream=None):
        """items: list of (ct, c2, chain_index); each ct += KeySwitch(c2) in place, uneven levels."""
        arr = (_KsItem * len(items))(*[_KsItem(ct.data_ptr(), c2.data_ptr(), ci) for ct, c2, ci in items])
        _check(lib.fhe_keyswitch_batch(self._h, ws._h, arr, len(items), key.ptr, _stream(stream)))

    def apply_galois(self, ws, ct, chain_index, elt, key, stream=None):
        _check(lib.fhe_apply_galois(self._h, ws._h, _ptr(ct), chain_index, elt, key.ptr, _stream(stream)))

    def _gk_array(self, galois_keys):
        arr = (_vp * len(self.galois_elts))()
        for i, k in enumerate(galois_keys):
            arr[i] = None if k is None else k.ptrs.data_ptr()
        return arr

    def rotate(self, ws, ct, chain_index, step, galois_keys, stream=None):
        _check(lib.fhe_rotate(self._h, ws._h, _ptr(ct), chain_index, step, self._gk_array(galois_keys),
                              _stream(stream)))

    def hoisting(self, ws, ct, chain_index, steps, galois_keys, stream=None):
        st = (ctypes.c_int * len(steps))(*steps)
        _check(lib.fhe_hoisting(self._h, ws._h, _ptr(ct), chain_index, st, len(steps), self._gk_array(galois_keys),
                                _stream(stream)))


    def rotations_hoisted(self, ws, ct, chain_index, steps, galois_keys, outs, stream=None):
        """outs[i] <- ct rotated by steps[i]; one mod-up of c1 shared by all steps."""
        st = (ctypes.c_int * len(steps))(*steps)
        o = (_vp * len(outs))(*[t.data_ptr() for t in outs])
        _check(lib.fhe_ckks_rotations_hoisted(self._h, ws._h, _ptr(ct), chain_index, st, len(steps),
                                              self._gk_array(galois_keys), o, _stream(stream)))

    def multiply_plain(self, ct, pt, out, chain_index, stream=None):
        _check(lib.fhe_ckks_multiply_plain(self._h, _ptr(ct), _ptr(pt), _ptr(out), chain_index, _stream(stream)))

    def add(self, a, b, out, size, chain_index, stream=None):
        _check(lib.fhe_ckks_add(self._h, _ptr(a), _ptr(b), _ptr(out), size, chain_index, _stream(stream)))

    def bsgs_scratch_bytes(self, G):
        return int(lib.fhe_bsgs_scratch_bytes(self._h, G))

    def bsgs_batch_scratch_bytes(self, G, B):
        """Scratch per product of bsgs_matvec_batch (babies and inner sums)."""
        return int(lib.fhe_bsgs_batch_scratch_bytes(self._h, G, B))

    def bsgs_matvec(self, ws, scratch, ct, chain_index, diags, D, G, B, galois_keys, out, hoisted=True,
                    stream=None):
        """out <- Rescale(sum_g rot_{gG}(sum_b rot_b(ct) * diags[gG + b]))."""
        _check(lib.fhe_ckks_bsgs_matvec(self._h, ws._h, _ptr(scratch), _ptr(ct), chain_index, _ptr(diags), D, G, B,
                                        self._gk_array(galois_keys), _ptr(out), int(bool(hoisted)),
                                        _stream(stream)))

    def bsgs_matvec_batch(self, ws, scratch, items, D, G, B, galois_keys, stream=None):
        """items: list of (ct, chain_index, diags, out): the hoisted bsgs_matvec of every item in
        one launch per pipeline step (uneven levels); ws from workspace(batch_items=...), scratch
        of min(len(items), 64) x bsgs_batch_scratch_bytes(G, B) bytes."""
        # diags [D][limbs][N]: the limb count is the array's stride (an array encoded at a higher
        # level than the item's serves it too)
        arr = (_MatvecItem * len(items))(*[_MatvecItem(ct.data_ptr(), dg.data_ptr(), out.data_ptr(), ci,
                                                       dg.shape[1] if dg.dim() == 3 else 0)
                                           for ct, ci, dg, out in items])
        _check(lib.fhe_ckks_bsgs_matvec_batch(self._h, ws._h, _ptr(scratch), arr, len(items), D, G, B,
                                              self._gk_array(galois_keys), _stream(stream)))

    def encrypt_symmetric(self, pt, s_ntt, a, e, out, chain_index, stream=None):
        _check(lib.fhe_ckks_encrypt_symmetric(self._h, _ptr(pt), _ptr(s_ntt), _ptr(a), _ptr(e), _ptr(out),
                                              chain_index, _stream(stream)))

    def decrypt(self, ct, s_ntt, pt, chain_index, stream=None):
        _check(lib.fhe_ckks_decrypt(self._h, _ptr(ct), _ptr(s_ntt), _ptr(pt), chain_index, _stream(stream)))

    def ckks_encode(self, ws, values, scale, chain_index, pt, count=None, stream=None):
        """values: device float64 tensor [count][2] (re, im) -> pt [l][N] (NTT form), the
        reference's encoder word for word."""
        n = values.numel() // 2 if count is None else count
        _check(lib.fhe_ckks_encode(self._h, ws._h, _ptr(values), n, float(scale), chain_index, _ptr(pt),
                                   _stream(stream)))

    def ckks_decode(self, ws, pt, scale, chain_index, values, stream=None):
        """pt [l][N] (NTT form) -> values: device float64 tensor [N/2][2] (re, im)."""
        _check(lib.fhe_ckks_decode(self._h, ws._h, _ptr(pt), chain_index, float(scale), _ptr(values),
                                   _stream(stream)))

    def kswitch_keygen(self, ws, galois_elt, s_ntt, a, e, key, stream=None):
        """galois_elt 0: relinearisation key (s^2); else the Galois key of that element."""
        _check(lib.fhe_kswitch_keygen(self._h, ws._h, galois_elt, _ptr(s_ntt), _ptr(a), _ptr(e), _ptr(key),
                                      _stream(stream)))

    # --- BFV plaintexts
    def bfv_encode(self, values, pt, count=None, stream=None):
        """values: device int64 [count] slot values (negative taken plus t); pt: [N]."""
        count = values.numel() if count is None else count
        _check(lib.fhe_bfv_encode(self._h, _ptr(values), count, _ptr(pt), _stream(stream)))

    def bfv_decode(self, ws, pt, values, stream=None):
        _check(lib.fhe_bfv_decode(self._h, ws._h, _ptr(pt), _ptr(values), _stream(stream)))

    def bfv_encrypt_symmetric(self, pt, s_ntt, a, e, out, stream=None):
        """out [2][nQ][N] = BFV encryption of pt [N] under s with uniform a [nQ][N] and error e [N]."""
        _check(lib.fhe_bfv_encrypt_symmetric(self._h, _ptr(pt), _ptr(s_ntt), _ptr(a), _ptr(e), _ptr(out),
                                             _stream(stream)))

    def bfv_decrypt(self, ws, ct, chain_index, s_ntt, pt, stream=None):
        _check(lib.fhe_bfv_decrypt(self._h, ws._h, _ptr(ct), chain_index, _ptr(s_ntt), _ptr(pt), _stream(stream)))

    # --- the reference's samplers (64-byte seeds, bytes)
    @staticmethod
    def _seed(seed, count=1):
        seed = bytes(seed)
        if len(seed) != 64 * count:
            raise InvalidArgument(-1, f"expected {count} seed(s) of 64 bytes")
        return seed

    def sample_uniform(self, seed, limbs, out, stream=None):
        """out [limbs][N] (int64 view of uint64): the reference's sample_uniform_poly."""
        _check(lib.fhe_sample_uniform(self._h, self._seed(seed), limbs, _ptr(out), _stream(stream)))

    def sample_ternary(self, seed, out, stream=None):
        """out [N] int64 in {-1, 0, 1}: the reference's sample_ternary_poly."""
        _check(lib.fhe_sample_ternary(self._h, self._seed(seed), _ptr(out), _stream(stream)))

    def sample_cbd(self, seed, out, stream=None):
        """out [N] int64: the reference's sample_error_poly (centred binomial)."""
        _check(lib.fhe_sample_cbd(self._h, self._seed(seed), _ptr(out), _stream(stream)))

    def secret_key_from_seed(self, ws, seed, s_ntt, stream=None):
        """s_ntt [QP][N]: the reference's gen_secretkey for this seed."""
        _check(lib.fhe_secret_key_from_seed(self._h, ws._h, self._seed(seed), _ptr(s_ntt), _stream(stream)))

    def kswitch_keygen_seeded(self, ws, galois_elt, s_ntt, seeds_a, seeds_e, key, stream=None):
        """The reference's generate_one_kswitch_key with dnum seeds for a and for the errors."""
        _check(lib.fhe_kswitch_keygen_seeded(self._h, ws._h, galois_elt, _ptr(s_ntt), self._seed(seeds_a, self.dnum),
                                             self._seed(seeds_e, self.dnum), _ptr(key), _stream(stream)))


class Workspace:
    def __init__(self, ctx, batch_items=None):
        h = _vp()
        if batch_items:
            _check(lib.fhe_workspace_create_batch(ctx._h, batch_items, ctypes.byref(h)))
        else:
            _check(lib.fhe_workspace_create(ctx._h, ctypes.byref(h)))
        self._h = h
        self.ctx = ctx

    def __del__(self):
        if getattr(self, "_h", None):
            lib.fhe_workspace_destroy(self._h)
            self._h = None
