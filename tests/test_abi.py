"""The C-ABI shared library loads and exports every function include/phantom_gb300.h
declares; host-side helpers work without a GPU.  CPU only (no kernel launches)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "phantom-fhe_gb300", "_build", "libphantom_gb300.so")


def _declared():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^[a-z_ 0-9*]+?\b(fhe_[a-z0-9_]+)\s*\(", src, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        subprocess.check_call(["make", "-s", "-j8", "-f", os.path.join(ROOT, "phantom-fhe_gb300", "Makefile")],
                              cwd=ROOT)
    L = ctypes.CDLL(LIB)
    L.fhe_create_coeff_modulus.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_int), ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_uint64)]
    L.fhe_galois_elt_from_step.argtypes = [ctypes.c_int, ctypes.c_uint64]
    L.fhe_galois_elt_from_step.restype = ctypes.c_uint32
    L.fhe_last_error.restype = ctypes.c_char_p
    return L


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_create_coeff_modulus_matches_oracle(lib):
    from oracle import oracle as O
    bits = [60] + [40] * 29 + [60] * 5
    out = (ctypes.c_uint64 * len(bits))()
    assert lib.fhe_create_coeff_modulus(65536, (ctypes.c_int * len(bits))(*bits), len(bits), out) == 0
    assert [int(x) for x in out] == O.create_coeff_modulus(65536, bits)


def test_galois_elt_from_step(lib):
    from oracle import oracle as O
    lib.fhe_galois_elt_from_step.restype = ctypes.c_uint32
    for n in (4096, 65536):
        for step in (1, -1, 2, 7, 0, -300):
            assert lib.fhe_galois_elt_from_step(step, n) == O.elt_from_step(step, n)


def test_bad_arguments_return_status(lib):
    lib.fhe_last_error.restype = ctypes.c_char_p
    out = (ctypes.c_uint64 * 1)()
    rc = lib.fhe_create_coeff_modulus(65536, (ctypes.c_int * 1)(70), 1, out)
    assert rc == -1 and b"invalid" in lib.fhe_last_error()
    assert lib.fhe_context_create(None, None) == -1


def test_matvec_item_layout_and_batch_scratch_query(lib):
    """The Python mirror of fhe_matvec_item has the C layout (three pointers, then chain_index and
    diag_limbs as size_t), and the batch scratch query returns 0 for what it cannot size."""
    import phantom_gb300 as pg
    assert ctypes.sizeof(pg._MatvecItem) == 3 * ctypes.sizeof(ctypes.c_void_p) + 2 * ctypes.sizeof(ctypes.c_size_t)
    assert [f for f, _ in pg._MatvecItem._fields_] == ["ct", "diags", "out", "chain_index", "diag_limbs"]
    lib.fhe_bsgs_batch_scratch_bytes.restype = ctypes.c_size_t
    lib.fhe_bsgs_batch_scratch_bytes.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]
    assert lib.fhe_bsgs_batch_scratch_bytes(None, 11, 12) == 0
