"""The C++ compatibility layer (phantom.h): a PhantomFHE-style program, compiled here with the
host compiler, loads ciphertexts and keys in the reference's byte format, runs the evaluator
calls and saves the results; they must equal the CPU oracle word for word."""
import os
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N, BITS, SPECIAL = 4096, [60, 40, 40, 40, 40, 40, 60, 60], 2
HDR = struct.Struct("<QQQQdQQ??")  # PhantomCiphertext::save header (include/ciphertext.h:173-184)


def write_ct(f, chain, data, scale=2.0 ** 40, ntt=True):
    size, limbs, n = data.shape
    f.write(HDR.pack(chain, size, n, limbs, scale, 1, 1, ntt, False))
    f.write(np.ascontiguousarray(data, dtype=np.uint64).tobytes())


def read_ct(path):
    with open(path, "rb") as f:
        chain, size, n, limbs, scale, _, _, ntt, _ = HDR.unpack(f.read(HDR.size))
        data = np.frombuffer(f.read(size * limbs * n * 8), dtype=np.uint64).reshape(size, limbs, n)
    return chain, scale, data


def write_key(f, key):  # PhantomRelinKey::save: dnum, then one size-2 ciphertext per digit at chain 0
    f.write(struct.pack("<Q", key.shape[0]))
    for d in range(key.shape[0]):
        write_ct(f, 0, key[d])


@pytest.fixture(scope="module")
def compat_bin(tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp") / "compat_main"
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-o", str(out), os.path.join(ROOT, "tests", "cpp", "compat_main.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "phantom-fhe_gb300", "cpp"),
           "-I", os.path.join(cuda, "include"), "-L", os.path.join(ROOT, "phantom-fhe_gb300", "_build"),
           "-lphantom_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(ROOT, "phantom-fhe_gb300", "_build")]
    subprocess.check_call(cmd)
    return out


def test_cpp_layer_matches_oracle(compat_bin, tmp_path):
    mods = O.create_coeff_modulus(N, BITS)
    nq = len(BITS) - SPECIAL
    oc = O.Context(12, mods, nq, SPECIAL)
    rng = np.random.default_rng(123)
    dnum = oc.beta(nq)
    l = nq
    a = O.random_residues(rng, mods[:l], N, 2)
    b = O.random_residues(rng, mods[:l], N, 2)
    rlk = O.random_residues(rng, mods, N, 2 * dnum).reshape(dnum, 2, len(mods), N)
    # default Galois elements of the context: conjugation, then 5^(2^i) and its inverse
    elts = [2 * N - 1]
    pos, neg = 5, pow(5, -1, 2 * N)
    for _ in range(11):
        elts += [pos, neg]
        pos, neg = pos * pos % (2 * N), neg * neg % (2 * N)
    gks = [O.random_residues(rng, mods, N, 2 * dnum).reshape(dnum, 2, len(mods), N) for _ in elts]
    with open(tmp_path / "a.bin", "wb") as f:
        write_ct(f, 1, a)
    with open(tmp_path / "b.bin", "wb") as f:
        write_ct(f, 1, b)
    with open(tmp_path / "rlk.bin", "wb") as f:
        write_key(f, rlk)
    with open(tmp_path / "gk.bin", "wb") as f:
        f.write(struct.pack("<Q", len(gks)))
        for k in gks:
            write_key(f, k)
    r = subprocess.run([str(compat_bin), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "compat ok" in r.stdout
    assert "ckks end to end max slot error" in r.stdout  # keys, encode, encrypt, evaluate, decrypt, decode

    chain, scale, got = read_ct(tmp_path / "out_mul_rescale.bin")
    assert chain == 2 and scale == 2.0 ** 80 / mods[l - 1]
    assert np.array_equal(got, oc.rescale(l, oc.ckks_mul_relin(l, a, b, rlk)))
    _, _, got = read_ct(tmp_path / "out_mul_then_relin.bin")
    assert np.array_equal(got, oc.ckks_mul_relin(l, a, b, rlk))
    want = a
    for s in (-1, 4):
        e = O.elt_from_step(s, N)
        want = oc.ckks_apply_galois(l, want, e, gks[elts.index(e)])
    _, _, got = read_ct(tmp_path / "out_rotate3.bin")
    assert np.array_equal(got, want)
    e12 = [O.elt_from_step(s, N) for s in (1, 2)]
    _, _, got = read_ct(tmp_path / "out_hoist12.bin")
    assert np.array_equal(got, oc.ckks_hoisting(l, a, e12, [gks[elts.index(e)] for e in e12]))
    chain, _, got = read_ct(tmp_path / "out_drop.bin")
    assert chain == 2 and np.array_equal(got, a[:, : l - 1, :])
