"""Golden vectors from PhantomFHE's own CUDA kernels, for pinning the oracle.

TEST INFRASTRUCTURE ONLY.  Needs a GPU, torch, the oracle (for its tables, which
tests/test_oracle.py pins to the reference's host code) and the reference kernels compiled
device-only by `make -f oracle/Makefile.refgpu` (run where the reference checkout is; the
cubins in oracle/_ref/ are then portable to any host with the driver).  Usage:

    python tests/golden/make_golden_kernels.py OUT.json          # golden digests
    python tests/golden/make_golden_kernels.py --time OUT.json   # GB300 timings of the same kernels
    python tests/golden/make_golden_kernels.py --time-batched OUT.json   # ... over the batched workloads
    python tests/golden/make_golden_kernels.py --extra OUT.json  # only the cases of extra_cases()

Every case replays the reference's host-side launch sequence (grid, block, dynamic shared
memory, argument order) for one operation, citing the host function it follows, on seeded
uniform residues (numpy default_rng, `oracle.random_residues`), and records the SHA-256 of the
output words (little-endian u64).  tests/test_oracle_ref_kernels.py recomputes each case with
the oracle (CPU) and tests/test_gpu_ref_digests.py with this library's CUDA path, and both
compare digests.
"""
import hashlib
import json
import math
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
import refkern as R  # noqa: E402

GRID_NTT, BLOCK_NTT, PAD = 4096, 128, 4   # include/common.h:23-30 (gridDimNTT, blockDimNTT, per_block_pad)
BLOCK_GLB = 128                           # include/common.h:20 (blockDimGlb)


def sample_size(n):
    """SAMPLE_SIZE(n), include/ntt.cuh:131-153."""
    return {2048: 64, 4096: 64, 8192: 128}.get(n, 256)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def shoup(w, q):
    return (int(w) << 64) // int(q)


def dmod(mods):
    """DModulus {value, const_ratio[0], const_ratio[1]} (include/ntt.cuh:6-32) per prime."""
    rows = [[q] + O.barrett_ratio(q)[:2] for q in mods]
    return np.array(rows, dtype=np.uint64)


def pair(vals, mods):
    v = np.array([int(x) for x in vals], dtype=np.uint64)
    s = np.array([shoup(x, q) for x, q in zip(vals, mods)], dtype=np.uint64)
    return R.dev(v, 8), R.dev(s, 8)


class Tables:
    """DNTTTable over a list of primes (include/ntt.cuh:34-124, src/context.cu:170-183)."""

    def __init__(self, log_n, mods):
        n = 1 << log_n
        self.n, self.mods = n, list(mods)
        tw, tws, itw, itws, ninv = [], [], [], [], []
        for q in mods:
            t = O.ntt_tables(log_n, q)
            tw.append(t[0]), tws.append(t[1]), itw.append(t[2]), itws.append(t[3]), ninv.append(t[4])
        self.tw, self.tws = R.dev(np.stack(tw), n), R.dev(np.stack(tws), n)
        self.itw, self.itws = R.dev(np.stack(itw), n), R.dev(np.stack(itws), n)
        self.ninv, self.ninvs = pair(ninv, mods)
        self.mod = R.dev(dmod(mods), 8)


class Kernels:
    def __init__(self):
        m = {s: R.Module(s) for s in ("fntt_2d", "intt_2d", "ntt_modup", "ntt_moddown", "rns_bconv",
                                       "eval_key_switch", "rns", "polymath", "galois", "prng", "batchencoder")}
        self.m = m
        k = lambda stem, name: m[stem].kernel(name)  # noqa: E731
        self.f1, self.f2 = k("fntt_2d", "inplace_fnwt_radix8_phase1"), k("fntt_2d", "inplace_fnwt_radix8_phase2")
        self.i1, self.i2 = k("intt_2d", "inplace_inwt_radix8_phase1"), k("intt_2d", "inplace_inwt_radix8_phase2")
        self.i1_sp = k("intt_2d", "inplace_inwt_radix8_phase1_include_special_mod")
        self.i2_sp = k("intt_2d", "inplace_inwt_radix8_phase2_include_special_mod")
        self.mu_i1 = k("ntt_modup", "inwt_radix8_phase1")
        self.mu_i2s = k("ntt_modup", "inplace_inwt_radix8_phase2_scale")
        self.mu_f1x = k("ntt_modup", "inplace_fnwt_radix8_phase1_include_special_mod_exclude_range")
        self.mu_f2x = k("ntt_modup", "inplace_fnwt_radix8_phase2_include_special_mod_exclude_range")
        self.md_f1 = k("ntt_moddown", "inplace_fnwt_radix8_phase1")
        self.md_f2 = k("ntt_moddown", "inplace_fnwt_radix8_phase2_fuse_moddown")
        self.copy_partql = k("rns_bconv", "modup_copy_partQl_kernel")
        self.bconv_padded = k("rns_bconv", "bconv_matmul_padded_unroll2_kernel")
        self.bconv_mult = k("rns_bconv", "bconv_mult_unroll2_kernel")
        self.bconv_matmul = k("rns_bconv", "bconv_matmul_unroll2_kernel")
        self.bconv_hps = k("rns_bconv", "base_convert_matmul_hps_unroll2_kernel")
        self.add_to_ct = k("rns_bconv", "add_to_ct_kernel")
        self.ip = k("eval_key_switch", "key_switch_inner_prod_c2_and_evk")
        self.dr_reduce = k("rns", "divide_and_round_reduce_q_last_kernel")
        self.dr_q_last = k("rns", "divide_and_round_q_last_kernel")
        self.dr_scalar = k("rns", "divide_and_round_ntt_inv_scalar_kernel")
        self.sr_qr_r = k("rns", "scaleAndRound_HPS_QR_R_kernel")
        self.tensor = k("polymath", "tensor_prod_2x2_rns_poly")
        self.f1_sp = k("fntt_2d", "inplace_fnwt_radix8_phase1_include_special_mod")
        self.f2_sp = k("fntt_2d", "inplace_fnwt_radix8_phase2_include_special_mod")
        self.bconv_mult1 = k("rns_bconv", "bconv_mult_kernel")
        self.moddown_k = k("rns_bconv", "moddown_kernel")
        self.s_uniform = k("prng", "sample_uniform_poly")
        self.s_ternary = k("prng", "sample_ternary_poly")
        self.s_error = k("prng", "sample_error_poly")
        self.mul_poly = k("polymath", "multiply_rns_poly")
        self.mul_add_neg = k("polymath", "multiply_and_add_negate_rns_poly")
        self.temp_mod_add = k("polymath", "multiply_temp_mod_and_add_rns_poly")
        self.encode_gpu = k("batchencoder", "encode_gpu")
        self.decode_gpu = k("batchencoder", "decode_gpu")
        self.add_neg = k("polymath", "add_and_negate_rns_poly")
        self.add_timesq = k("polymath", "bfv_add_timesQ_overt_kernel")
        self.mul_add = k("polymath", "multiply_and_add_rns_poly")
        self.add_poly = k("polymath", "add_rns_poly")
        self.dec = {v: k("rns", "hps_decrypt_scale_and_round_kernel_" + v)
                    for v in ("small", "small_lazy", "large", "large_lazy")}
        self.galois = k("galois", "apply_galois_ntt_permutation")
        for stem in ("ckks", "fft", "rns_base"):
            m[stem] = R.Module(stem)
        self.bitrev = k("ckks", "bit_reverse_kernel")
        self.fft_base = k("fft", "inplace_special_ffft_base_kernel")
        self.fft_iter = k("fft", "inplace_special_ffft_iter_kernel")
        self.ifft_base = k("fft", "inplace_special_ifft_base_kernel")
        self.ifft_iter = k("fft", "inplace_special_ifft_iter_kernel")
        self.dec64 = k("rns_base", "decompose_array_uint64_kernel")
        self.dec128 = k("rns_base", "decompose_array_uint128_kernel")
        self.dec_slow1 = k("rns_base", "decompose_array_uint_slow_first_part")
        self.dec_slow2 = k("rns_base", "decompose_array_uint_slow_second_part")
        self.compose = k("rns_base", "compose_array_kernel")

    # nwt_2d_radix8_forward_inplace, src/ntt/fntt_2d.cu:620-653
    def ntt_fwd(self, T, buf, size, start):
        n, s1 = T.n, sample_size(T.n)
        self.f1(GRID_NTT, s1 // 8 * PAD, (s1 + PAD + 1) * PAD * 8, buf, T.tw, T.tws, T.mod, size, start, n, s1, PAD)
        self.f2(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, buf, T.tw, T.tws, T.mod, size, start, n, s1, n // s1)

    # nwt_2d_radix8_backward_inplace, src/ntt/intt_2d.cu:724-757
    def ntt_inv(self, T, buf, size, start):
        n = T.n
        s2 = sample_size(n)
        s1 = n // s2
        self.i1(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, buf, T.itw, T.itws, T.mod, size, start, n, s1, s2)
        self.i2(GRID_NTT, s1 // 8 * PAD, (s1 + PAD + 1) * PAD * 8, buf, T.itw, T.itws, T.ninv, T.ninvs, T.mod,
                size, start, n, s1, PAD)


def case_ntt(K, log_n, bits, seed):
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    T = Tables(log_n, mods)
    x = O.random_residues(np.random.default_rng(seed), mods, n, 1)[0]
    buf = R.dev(x, n)
    K.ntt_fwd(T, buf, len(mods), 0)
    fwd = R.host(buf, x.size)
    K.ntt_inv(T, buf, len(mods), 0)
    inv = R.host(buf, x.size)
    assert np.array_equal(inv, x.reshape(-1)), "reference NTT round trip"
    return {"log_n": log_n, "bits": bits, "seed": seed, "forward": sha(fwd), "inverse_of_forward": sha(inv)}


class KsLevel:
    """DRNSTool tables of one data level for key switching (src/rns.cu:140-200)."""

    def __init__(self, oc, T, l):
        n, nq, a = oc.n, oc.n_q, oc.n_p
        self.l, self.qlp, self.beta = l, l + a, (l + a - 1) // a
        mods = T.mods
        qlp_mods = mods[:l] + mods[nq:]
        self.qlp_mods = qlp_mods
        concat, self.digits = [], []
        for d in range(self.beta):
            phi, mat = oc.modup_tables(l, d)
            sz = len(phi)
            start = a * d
            concat += [int(v) for v in phi]
            compl = qlp_mods[:start] + qlp_mods[start + sz:]
            self.digits.append(dict(start=start, sz=sz, ibase=R.dev(dmod(qlp_mods[start:start + sz]), 8),
                                    obase=R.dev(dmod(compl), 8), osz=len(compl), mat=R.dev(mat, 8)))
        self.part_inv, self.part_inv_s = pair(concat, mods[:l])
        phi, mat, pinv = oc.moddown_tables(l)
        self.p_hat_inv, self.p_hat_inv_s = pair(phi, mods[nq:])
        self.p_to_ql = R.dev(mat, 8)
        self.p_inv, self.p_inv_s = pair(pinv, mods[:l])
        self.base_p = R.dev(dmod(mods[nq:]), 8)


class Scratch:
    """Device scratch buffers by name, allocated on first use and reused afterwards (so a
    sequence can be captured into a CUDA graph after one warm-up run).  Every buffer the
    reference allocates per call is fully written before it is read, so reuse changes no word."""

    def __init__(self):
        self.bufs, self.frozen = {}, False

    def __call__(self, key, words):
        t = self.bufs.get(key)
        if t is None or t.numel() < words:
            assert not self.frozen, f"allocation of {key} inside a capture"
            t = self.bufs[key] = R.zeros(words)
        return t


def ref_modup(K, T, oc, L, c2_d, S):
    """DRNSTool::modup for CKKS (src/rns_bconv.cu:530-628): c2_d (l x N, NTT form, device) ->
    t_mod_up [beta][l + alpha][N] (a scratch buffer of S)."""
    n, a, qp = oc.n, oc.n_p, oc.n_q + oc.n_p
    l, qlp, beta = L.l, L.qlp, L.beta
    s_fwd = sample_size(n)
    s2_inv = sample_size(n)
    s1_inv = n // s2_inv
    t_mod_up = S("t_mod_up", beta * qlp * n + n)
    t_cks = S("t_cks", l * n + n)
    # modup: nwt_2d_radix8_backward_scale (src/ntt/ntt_modup.cu:356-393)
    K.mu_i1(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, t_cks, c2_d, T.itw, T.itws, T.mod, l, 0, n, s1_inv, s2_inv)
    K.mu_i2s(GRID_NTT, s1_inv // 8 * PAD, (s1_inv + PAD + 1) * PAD * 8, t_cks, T.itw, T.itws, T.ninv, T.ninvs,
             T.mod, l, 0, n, s1_inv, PAD, L.part_inv, L.part_inv_s)
    K.copy_partql(n * l // BLOCK_GLB, BLOCK_GLB, 0, t_mod_up, c2_d, l * n, qlp * n, a * n)
    for d, D in enumerate(L.digits):
        part = R.Ptr(t_mod_up, d * qlp * n)
        K.bconv_padded(n * D["osz"] // BLOCK_GLB // 2, BLOCK_GLB, 8 * D["osz"] * D["sz"], part,
                       R.Ptr(t_cks, D["start"] * n), D["mat"], D["ibase"], D["sz"], D["obase"], D["osz"], n,
                       D["start"], D["sz"])
        # nwt_2d_radix8_forward_inplace_include_special_mod_exclude_range (src/ntt/ntt_modup.cu:610-657)
        lo, hi = D["start"], D["start"] + D["sz"]
        K.mu_f1x(GRID_NTT, s_fwd // 8 * PAD, (s_fwd + PAD + 1) * PAD * 8, part, T.tw, T.tws, T.mod, qlp, 0, qp, a,
                 n, s_fwd, PAD, lo, hi)
        K.mu_f2x(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, part, T.tw, T.tws, T.mod, qlp, 0, qp, a, n, s_fwd,
                 n // s_fwd, lo, hi)
    return t_mod_up


def ref_inner_product(K, T, oc, L, cx, t_mod_up, evk_ptrs):
    """key_switch_inner_prod_c2_and_evk launched as src/eval_key_switch.cu:156-160 (the
    reduction_threshold of :156-157): cx [2][l + alpha][N]."""
    n, nq, qp = oc.n, oc.n_q, oc.n_q + oc.n_p
    thr = (1 << (64 - int(np.log2(float(T.mods[0]))) - 1)) - 1
    K.ip(L.qlp * n // BLOCK_GLB, BLOCK_GLB, 0, cx, t_mod_up, evk_ptrs, T.mod, n, qp, qp * n, L.qlp, L.qlp * n, nq,
         L.l, L.beta, thr)


def ref_moddown(K, T, oc, L, cx, S):
    """DRNSTool::moddown_from_NTT for CKKS (src/rns_bconv.cu:776-828) on both polynomials of
    cx [2][l + alpha][N], in place (the first l limbs of each hold the result)."""
    n, a, qp = oc.n, oc.n_p, oc.n_q + oc.n_p
    l, qlp = L.l, L.qlp
    s_fwd = sample_size(n)
    s2_inv = sample_size(n)
    s1_inv = n // s2_inv
    for i in range(2):
        cx_i = R.Ptr(cx, i * qlp * n)
        # nwt_2d_radix8_backward_inplace_include_special_mod (src/ntt/intt_2d.cu:796-834)
        K.i1_sp(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, cx_i, T.itw, T.itws, T.mod, a, l, qp, a, n, s1_inv, s2_inv)
        K.i2_sp(GRID_NTT, s1_inv // 8 * PAD, (s1_inv + PAD + 1) * PAD * 8, cx_i, T.itw, T.itws, T.ninv, T.ninvs,
                T.mod, a, l, qp, a, n, s1_inv, PAD)
        # DBaseConverter::bConv_BEHZ (src/rns_bconv.cu:212-229), P -> Ql
        temp = S("temp", a * n + n)
        delta = S("delta", l * n + n)
        K.bconv_mult(a * n // 2 // BLOCK_GLB, BLOCK_GLB, 0, temp, R.Ptr(cx, i * qlp * n + l * n), L.p_hat_inv,
                     L.p_hat_inv_s, L.base_p, a, n)
        K.bconv_matmul(l * n // 2 // BLOCK_GLB, BLOCK_GLB, 8 * l * a, delta, temp, L.p_to_ql, L.base_p, a, T.mod,
                       l, n)
        # nwt_2d_radix8_forward_inplace_fuse_moddown (src/ntt/ntt_moddown.cu:222-261)
        K.md_f1(GRID_NTT, s_fwd // 8 * PAD, (s_fwd + PAD + 1) * PAD * 8, delta, T.tw, T.tws, T.mod, l, 0, n,
                s_fwd, PAD)
        K.md_f2(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, cx_i, cx_i, L.p_inv, L.p_inv_s, delta, T.tw, T.tws, T.mod,
                l, 0, n, s_fwd, n // s_fwd)


def ref_keyswitch(K, T, oc, L, ct_d, c2_d, evk_ptrs, scratch=None, keep=False):
    """keyswitch_inplace for CKKS, src/eval_key_switch.cu:95-182, with DRNSTool::modup
    (src/rns_bconv.cu:530-628), key_switch_inner_prod (src/eval_key_switch.cu:71-92) and
    DRNSTool::moddown_from_NTT (src/rns_bconv.cu:776-828).  ct_d (2 x l x N, device) is updated
    in place; with keep=True returns the host copies of t_mod_up and cx."""
    S = scratch or Scratch()
    n = oc.n
    l, qlp, beta = L.l, L.qlp, L.beta
    t_mod_up = ref_modup(K, T, oc, L, c2_d, S)
    tm = R.host(t_mod_up, beta * qlp * n) if keep else None
    cx = S("cx", 2 * qlp * n + n)
    ref_inner_product(K, T, oc, L, cx, t_mod_up, evk_ptrs)
    cxh = R.host(cx, 2 * qlp * n) if keep else None
    ref_moddown(K, T, oc, L, cx, S)
    for i in range(2):
        K.add_to_ct(l * n // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(ct_d, i * l * n), R.Ptr(cx, i * qlp * n), T.mod, n, l)
    return tm, cxh


def ref_hoisting(K, T, oc, L, ct_d, perms, keys, S):
    """hoisting_inplace for CKKS, src/evaluate.cu:1670-1865: one mod-up of c1; per step the Galois
    permutation of c0 and of every digit of the mod-up (apply_galois_ntt over Ql / QlP limbs,
    src/galois.cu:86-102), the inner product with that step's key, and the sums (add_rns_poly,
    src/polymath.cu:41-55); one mod-down of the summed products; ct = (acc_c0 + cx_0, cx_1)."""
    n = oc.n
    l, qlp, beta = L.l, L.qlp, L.beta
    qlp_mod = R.dev(dmod(L.qlp_mods), 8)
    c0 = S("h_c0", l * n + n)
    c0[: l * n].copy_(ct_d[: l * n])
    acc_c0 = S("h_acc_c0", l * n + n)
    K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, acc_c0, c0, perms[0], n, l)
    c1 = S("h_c1", l * n + n)
    c1[: l * n].copy_(ct_d[l * n: 2 * l * n])
    modup_c1 = ref_modup(K, T, oc, L, c1, S)
    tmp_mu = S("h_tmp_modup", beta * qlp * n + n)
    for b in range(beta):
        K.galois(qlp * n // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(tmp_mu, b * qlp * n), R.Ptr(modup_c1, b * qlp * n),
                 perms[0], n, qlp)
    acc_cx = S("h_acc_cx", 2 * qlp * n + n)
    ref_inner_product(K, T, oc, L, acc_cx, tmp_mu, keys[0])
    temp_c0 = S("h_temp_c0", l * n + n)
    temp_cx = S("h_temp_cx", 2 * qlp * n + n)
    for i in range(1, len(perms)):
        K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, temp_c0, c0, perms[i], n, l)
        K.add_poly(l * n // BLOCK_GLB, BLOCK_GLB, 0, acc_c0, temp_c0, T.mod, acc_c0, n, l)
        for b in range(beta):
            K.galois(qlp * n // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(tmp_mu, b * qlp * n),
                     R.Ptr(modup_c1, b * qlp * n), perms[i], n, qlp)
        ref_inner_product(K, T, oc, L, temp_cx, tmp_mu, keys[i])
        K.add_poly(qlp * n // BLOCK_GLB, BLOCK_GLB, 0, acc_cx, temp_cx, qlp_mod, acc_cx, n, qlp)
        K.add_poly(qlp * n // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(acc_cx, qlp * n), R.Ptr(temp_cx, qlp * n), qlp_mod,
                   R.Ptr(acc_cx, qlp * n), n, qlp)
    ref_moddown(K, T, oc, L, acc_cx, S)
    K.add_poly(l * n // BLOCK_GLB, BLOCK_GLB, 0, acc_c0, acc_cx, T.mod, ct_d, n, l)
    ct_d[l * n: 2 * l * n].copy_(acc_cx[qlp * n: qlp * n + l * n])


def rescale_tables(T, l):
    """inv_q_last_mod_q and its Shoup companions for level l (src/rns.cu:1160-1184)."""
    return pair([pow(T.mods[l - 1], -1, q) for q in T.mods[:l - 1]], T.mods[:l - 1])


def ref_rescale(K, T, src, dst, l, size, inv_tables=None):
    """DRNSTool::divide_and_round_q_last_ntt, src/rns.cu:1160-1184: src (size x l x N, device;
    its last limbs are turned to coefficient form, as the reference does) -> dst (size x (l-1) x N)."""
    n = T.n
    inv, inv_s = inv_tables or rescale_tables(T, l)
    g = n * (l - 1) // BLOCK_GLB
    s2 = sample_size(n)
    s1 = n // s2
    s = sample_size(n)
    for i in range(size):
        ci_in, ci_out = R.Ptr(src, i * l * n), R.Ptr(dst, i * (l - 1) * n)
        # nwt_2d_radix8_backward_inplace(ci_in, tables, 1, l - 1): the last limb only
        K.i1(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, ci_in, T.itw, T.itws, T.mod, 1, l - 1, n, s1, s2)
        K.i2(GRID_NTT, s1 // 8 * PAD, (s1 + PAD + 1) * PAD * 8, ci_in, T.itw, T.itws, T.ninv, T.ninvs, T.mod, 1,
             l - 1, n, s1, PAD)
        K.dr_reduce(g, BLOCK_GLB, 0, ci_out, ci_in, T.mod, n, l - 1)
        K.f1(GRID_NTT, s // 8 * PAD, (s + PAD + 1) * PAD * 8, ci_out, T.tw, T.tws, T.mod, l - 1, 0, n, s, PAD)
        K.f2(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, ci_out, T.tw, T.tws, T.mod, l - 1, 0, n, s, n // s)
        K.dr_scalar(g, BLOCK_GLB, 0, ci_out, ci_in, T.mod, inv, inv_s, n, l - 1)


def key_setup(rng, mods, n, nq, special):
    dnum = -(-nq // special)
    evk = O.random_residues(rng, mods, n, 2 * dnum).reshape(dnum, 2, len(mods), n)
    evk_t = R.dev(evk, n)
    ptrs = np.array([evk_t.data_ptr() + 8 * d * 2 * len(mods) * n for d in range(dnum)], dtype=np.uint64)
    return evk_t, R.dev(ptrs, 8)


def case_keyswitch(K, log_n, bits, special, levels, seed):
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    oc = O.Context(log_n, mods, nq, special)
    T = Tables(log_n, mods)
    rng = np.random.default_rng(seed)
    evk_t, evk_ptrs = key_setup(rng, mods, n, nq, special)
    out = {"log_n": log_n, "bits": bits, "special": special, "seed": seed, "levels": {}}
    for l in sorted(levels, reverse=True):  # inputs are drawn level by level, highest first
        ct = O.random_residues(rng, mods[:l], n, 2)
        c2 = O.random_residues(rng, mods[:l], n, 1)[0]
        ct_d = R.dev(ct, n)
        tm, cx = ref_keyswitch(K, T, oc, KsLevel(oc, T, l), ct_d, R.dev(c2, n), evk_ptrs, keep=True)
        out["levels"][str(l)] = {"modup": sha(tm), "inner_product": sha(cx), "keyswitch": sha(R.host(ct_d, 2 * l * n))}
    return out


def case_hmult(K, log_n, bits, special, l, seed):
    """CKKS multiply_and_relin_inplace (src/evaluate.cu:1061-1104: bgv_ckks_multiply's
    tensor_prod_2x2_rns_poly, then relinearize_inplace :1342-1374, i.e. keyswitch_inplace with
    c2 = the third polynomial) followed by rescale_to_next (:1545-1565)."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    oc = O.Context(log_n, mods, nq, special)
    T = Tables(log_n, mods)
    rng = np.random.default_rng(seed)
    evk_t, evk_ptrs = key_setup(rng, mods, n, nq, special)
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    d = R.zeros(3 * l * n + n)
    K.tensor(l * n // BLOCK_GLB, BLOCK_GLB, 0, R.dev(a, n), R.dev(b, n), T.mod, d, n, l)
    ref_keyswitch(K, T, oc, KsLevel(oc, T, l), d, R.Ptr(d, 2 * l * n), evk_ptrs)
    relin = R.host(d, 2 * l * n)
    out = R.zeros(2 * (l - 1) * n + n)
    ref_rescale(K, T, d, out, l, 2)
    return {"log_n": log_n, "bits": bits, "special": special, "l": l, "seed": seed,
            "multiply_and_relin": sha(relin), "rescaled": sha(R.host(out, 2 * (l - 1) * n))}


def case_rotate(K, log_n, bits, special, l, step, seed):
    """apply_galois_inplace for CKKS (src/evaluate.cu:1567-1630), as rotate_inplace calls it for a
    step with a Galois key: permute c0 into temp and copy it back, permute c1 into temp, zero c1,
    key-switch temp into (c0, c1).  The permutation table is this oracle's (the reference builds it
    on the host, include/galois.cuh:98-113; it is fixed by the NTT order, which is pinned)."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    oc = O.Context(log_n, mods, nq, special)
    T = Tables(log_n, mods)
    rng = np.random.default_rng(seed)
    evk_t, evk_ptrs = key_setup(rng, mods, n, nq, special)
    ct = R.dev(O.random_residues(rng, mods[:l], n, 2), n)
    elt = O.elt_from_step(step, n)
    perm = torch.from_numpy(O.galois_perm(log_n, elt).view(np.int32).copy()).cuda()
    temp = R.zeros(l * n + n)
    K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, temp, ct, perm, n, l)
    ct[: l * n].copy_(temp[: l * n])
    K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, temp, R.Ptr(ct, l * n), perm, n, l)
    ct[l * n: 2 * l * n].zero_()
    ref_keyswitch(K, T, oc, KsLevel(oc, T, l), ct, temp, evk_ptrs)
    return {"log_n": log_n, "bits": bits, "special": special, "l": l, "step": step, "elt": elt, "seed": seed,
            "rotate": sha(R.host(ct, 2 * l * n))}


def case_hoisting(K, log_n, bits, special, l, steps, seed):
    """hoisting_inplace for CKKS (src/evaluate.cu:1670-1865) with one Galois key per step, drawn
    in step order before the ciphertext."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    oc = O.Context(log_n, mods, nq, special)
    T = Tables(log_n, mods)
    rng = np.random.default_rng(seed)
    keys, elts, perms = [], [], []
    for st in steps:
        keys.append(key_setup(rng, mods, n, nq, special))
        elt = O.elt_from_step(st, n)
        elts.append(elt)
        perms.append(torch.from_numpy(O.galois_perm(log_n, elt).view(np.int32).copy()).cuda())
    ct = R.dev(O.random_residues(rng, mods[:l], n, 2), n)
    ref_hoisting(K, T, oc, KsLevel(oc, T, l), ct, perms, [k[1] for k in keys], Scratch())
    return {"log_n": log_n, "bits": bits, "special": special, "l": l, "steps": steps, "elts": elts, "seed": seed,
            "hoisting": sha(R.host(ct, 2 * l * n))}


def case_bfv_modswitch(K, log_n, bits, special, t, l, seed):
    """BFV mod_switch_to_next (src/evaluate.cu:1376-1427 -> DRNSTool::divide_and_round_q_last,
    src/rns.cu:1082-1126) on a size-2 ciphertext in coefficient form with l data limbs."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    T = Tables(log_n, mods)
    ct = O.random_residues(np.random.default_rng(seed), mods[:l], n, 2)
    src = R.dev(ct, n)
    dst = R.zeros(2 * (l - 1) * n + n)
    inv, inv_s = rescale_tables(T, l)
    for i in range(2):
        K.dr_q_last(n * (l - 1) // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(dst, i * (l - 1) * n), R.Ptr(src, i * l * n),
                    T.mod, inv, inv_s, n, l - 1)
    return {"log_n": log_n, "bits": bits, "special": special, "t": t, "l": l, "seed": seed,
            "mod_switch": sha(R.host(dst, 2 * (l - 1) * n))}


SWITCH_POINT, FFT_THREADS = 2048, 1024  # include/common.h:13-15


def ckks_roots(log_n):
    """The encoder's twiddle table: ComplexRoots of degree m = 2N (src/fft.cu:12-41, polar(1, 2 pi i
    / m) for i <= m/8) read through get_root for every index < m, as [m][2] doubles."""
    m = 2 << log_n
    base = [(math.cos(2 * math.pi * i / m), math.sin(2 * math.pi * i / m)) for i in range(m // 8 + 1)]

    def get_root(i):
        i &= m - 1
        if i <= m // 8:
            return base[i]
        if i <= m // 4:
            r = base[m // 4 - i]
            return (r[1], r[0])
        if i <= m // 2:
            r = get_root(m // 2 - i)
            return (0.0 - r[0], 0.0 - (-r[1]))
        if i <= 3 * m // 4:
            r = get_root(i - m // 2)
            return (0.0 - r[0], 0.0 - r[1])
        r = get_root(m - i)
        return (r[0], -r[1])

    return np.array([get_root(i) for i in range(m)], dtype=np.float64)


def rotation_group(log_n):
    """5^i mod 2N for i < N/4 (src/ckks.cu:36-46)."""
    m, out, pos = 2 << log_n, [], 1
    for _ in range((1 << log_n) // 4):
        out.append(pos)
        pos = pos * 5 % m
    return np.array(out, dtype=np.uint32)


class Codec:
    """Device tables of PhantomCKKSEncoder (src/ckks.cu:17-66) for one degree."""

    def __init__(self, log_n):
        self.log_n, self.n = log_n, 1 << log_n
        self.slots, self.m = self.n // 2, 2 * self.n
        self.roots = R.dev(ckks_roots(log_n))
        self.group = torch.from_numpy(rotation_group(log_n).view(np.int32).copy()).cuda()


def ref_fft_backward(K, C, buf, scalar):
    """special_fft_backward (src/fft.cu:374-413)."""
    n, logn = C.slots, C.log_n - 1
    if n <= SWITCH_POINT:
        K.ifft_base(1, n // 2, n * 16, buf, C.roots, C.group, n, logn, 1, 0, C.m, scalar)
        return
    it, groups = logn - 11, n // SWITCH_POINT
    blocks = -(-n // FFT_THREADS // 2)
    K.ifft_base(blocks, FFT_THREADS, SWITCH_POINT * 16, buf, C.roots, C.group, n, logn, groups, it, C.m, scalar)
    groups >>= 1
    while groups >= 1:
        it -= 1
        K.ifft_iter(blocks, FFT_THREADS, 0, buf, C.roots, C.group, n, logn, groups, it, C.m, scalar)
        groups >>= 1


def ref_fft_forward(K, C, buf):
    """special_fft_forward (src/fft.cu:340-368)."""
    n, logn = C.slots, C.log_n - 1
    if n <= SWITCH_POINT:
        K.fft_base(1, n // 2, n * 16, buf, C.roots, C.group, n, logn, 1, 0, C.m)
        return
    it, groups = 0, 1
    blocks = -(-n // FFT_THREADS // 2)
    while groups < n // SWITCH_POINT:
        K.fft_iter(blocks, FFT_THREADS, 0, buf, C.roots, C.group, n, logn, groups, it, C.m)
        it += 1
        groups <<= 1
    K.fft_base(blocks, FFT_THREADS, SWITCH_POINT * 16, buf, C.roots, C.group, n, logn, groups, it, C.m)


def ref_encode(K, T, C, values, scale, l):
    """PhantomCKKSEncoder::encode_internal (src/ckks.cu:68-138) of complex `values` at `scale`
    into l limbs; returns the plaintext (device, NTT form)."""
    n, slots = C.n, C.slots
    count = len(values)
    temp = R.dev(np.stack([values.real, values.imag], axis=1).astype(np.float64))
    buf = torch.zeros(2 * slots, dtype=torch.float64, device="cuda")
    K.bitrev(-(-count // BLOCK_GLB), BLOCK_GLB, 0, buf, temp, count, C.log_n - 1)
    ref_fft_backward(K, C, buf, scale / float(slots))
    z = buf.cpu().numpy()
    max_coeff = float(np.max(np.abs(z))) if z.size else 0.0
    max_bits = int(math.ceil(math.log2(max(max_coeff, 1.0)))) + 1
    q_bits = math.prod(int(q) for q in T.mods[:l]).bit_length()
    assert max_bits < q_bits, "encoded values are too large"
    pt = R.zeros(l * n + n)
    grid = n * l // BLOCK_GLB
    if max_bits <= 64:
        K.dec64(grid, BLOCK_GLB, 0, pt, buf, T.mod, n)
    elif max_bits <= 128:
        K.dec128(grid, BLOCK_GLB, 0, pt, buf, T.mod, n)
    else:
        coeffu = R.zeros(n * (l + 1))
        K.dec_slow1(grid, BLOCK_GLB, 0, coeffu, buf, n, l)
        K.dec_slow2(grid, BLOCK_GLB, 0, pt, coeffu, T.mod, n, l)
    K.ntt_fwd(T, pt, l, 0)
    return pt, max_bits


def compose_tables(mods):
    """DRNSBase of Q_l (src/rns_base.cu:11-47): Q_l, Q_l / q_i, (Q_l / q_i)^-1 mod q_i (+ Shoup)
    and the context's upper_half_threshold (Q_l + 1) / 2 (src/context.cu:106-110), as words."""
    l = len(mods)
    Q = math.prod(int(q) for q in mods)

    def words(v):
        return [(v >> (64 * w)) & ((1 << 64) - 1) for w in range(l)]
    hats = [Q // int(q) for q in mods]
    inv = [pow(h % int(q), -1, int(q)) for h, q in zip(hats, mods)]
    return (R.dev(np.array(words(Q), dtype=np.uint64), 8),
            R.dev(np.array([w for h in hats for w in words(h)], dtype=np.uint64), 8),
            *pair(inv, mods),
            R.dev(np.array(words((Q + 1) >> 1), dtype=np.uint64), 8))


def ref_decode(K, T, C, pt, scale, l):
    """PhantomCKKSEncoder::decode_internal (src/ckks.cu:340-400): plaintext (l limbs, NTT form)
    -> N/2 complex slots as [N/2][2] doubles (host)."""
    n, slots = C.n, C.slots
    copy = R.zeros(l * n + n)
    copy[: l * n].copy_(pt[: l * n])
    K.ntt_inv(T, copy, l, 0)
    qprod, qhat, qinv, qinv_s, upper = compose_tables(T.mods[:l])
    buf = torch.zeros(2 * slots, dtype=torch.float64, device="cuda")
    temp_prod, acc = R.zeros(n * l), R.zeros(n * l)
    K.compose(n // BLOCK_GLB, BLOCK_GLB, 0, buf, temp_prod, acc, copy, l, T.mod, qprod, qhat, qinv, qinv_s, upper,
              1.0 / scale, n)
    ref_fft_forward(K, C, buf)
    out = torch.zeros(2 * slots, dtype=torch.float64, device="cuda")
    K.bitrev(-(-slots // BLOCK_GLB), BLOCK_GLB, 0, out, buf, slots, C.log_n - 1)
    return out.cpu().numpy()


def unit_disk(rng, count):
    r, th = np.sqrt(rng.uniform(0, 1, count)), 2 * np.pi * rng.uniform(0, 1, count)
    return r * np.cos(th) + 1j * r * np.sin(th)


def case_codec(K, log_n, bits, special, l, scale, count, seed):
    """The CKKS encoder: encode `count` slots uniform in the unit disk at `scale` into l limbs,
    decode that plaintext, and decode a plaintext of uniform random residues (both halves of the
    compose's centring)."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    T = Tables(log_n, mods)
    C = Codec(log_n)
    rng = np.random.default_rng(seed)
    vals = unit_disk(rng, count)
    pt, max_bits = ref_encode(K, T, C, vals, scale, l)
    dec = ref_decode(K, T, C, pt, scale, l)
    rnd = R.dev(O.random_residues(rng, mods[:l], n, 1), n)
    dec_rnd = ref_decode(K, T, C, rnd, scale, l)
    return {"log_n": log_n, "bits": bits, "special": special, "l": l, "scale": scale, "count": count, "seed": seed,
            "max_coeff_bits": max_bits, "encode": sha(R.host(pt, l * n)), "decode": sha(dec.view(np.uint64)),
            "decode_random": sha(dec_rnd.view(np.uint64))}


def case_rescale(K, log_n, bits, special, l, seed):
    """DRNSTool::divide_and_round_q_last_ntt, src/rns.cu:1160-1184, on a size-2 ciphertext."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    T = Tables(log_n, mods)
    ct = O.random_residues(np.random.default_rng(seed), mods[:l], n, 2)
    src = R.dev(ct, n)
    dst = R.zeros(2 * (l - 1) * n + n)
    ref_rescale(K, T, src, dst, l, 2)
    return {"log_n": log_n, "bits": bits, "special": special, "l": l, "seed": seed,
            "rescale": sha(R.host(dst, 2 * (l - 1) * n))}


def case_tensor_galois(K, log_n, bits, special, l, steps, seed):
    """tensor_prod_2x2_rns_poly (src/polymath.cu:463-497, launched as src/evaluate.cu:379) and
    apply_galois_ntt_permutation (src/galois.cu:11-18) with the oracle's permutation table."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    T = Tables(log_n, mods)
    rng = np.random.default_rng(seed)
    a = O.random_residues(rng, mods[:l], n, 2)
    b = O.random_residues(rng, mods[:l], n, 2)
    out = R.zeros(3 * l * n + n)
    K.tensor(l * n // BLOCK_GLB, BLOCK_GLB, 0, R.dev(a, n), R.dev(b, n), T.mod, out, n, l)
    res = {"log_n": log_n, "bits": bits, "special": special, "l": l, "seed": seed,
           "tensor": sha(R.host(out, 3 * l * n)), "galois": {}}
    x = O.random_residues(rng, mods[:l], n, 1)[0]
    xd = R.dev(x, n)
    for step in steps:
        elt = O.elt_from_step(step, n)
        perm = torch.from_numpy(O.galois_perm(log_n, elt).view(np.int32).copy()).cuda()
        dst = R.zeros(l * n + n)
        K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, dst, xd, perm, n, l)
        res["galois"][str(step)] = {"elt": elt, "sha": sha(R.host(dst, l * n))}
    return res


def case_hps(K, log_n, bits, special, t, seed):
    """DBaseConverter::bConv_HPS Q -> R (src/rns_bconv.cu:354-372) and
    DRNSTool::scaleAndRound_HPS_QR_R (src/rns.cu:1740-1747), BFV at the top level."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    oc = O.Context(log_n, mods, nq, special, t)
    q, r = mods[:nq], oc.r_moduli
    big_q = 1
    for v in q:
        big_q *= v
    hat = [big_q // v for v in q]
    hat_inv, hat_inv_s = pair([pow(h % v, -1, v) for h, v in zip(hat, q)], q)
    qhat_mod_r = R.dev(np.array([[h % rj for h in hat] for rj in r], dtype=np.uint64), 8)
    alpha_q = R.dev(np.array([[(v * big_q) % rj for rj in r] for v in range(nq + 1)], dtype=np.uint64), 8)
    qinv = R.dev(np.array([1.0 / float(v) for v in q], dtype=np.float64), 8)
    base_q, base_r = R.dev(dmod(q), 8), R.dev(dmod(r), 8)
    rng = np.random.default_rng(seed)
    x = O.random_residues(rng, q, n, 1)[0]
    temp = R.zeros(nq * n + n)
    dst = R.zeros(len(r) * n + n)
    K.bconv_mult(nq * n // 2 // BLOCK_GLB, BLOCK_GLB, 0, temp, R.dev(x, n), hat_inv, hat_inv_s, base_q, nq, n)
    K.bconv_hps(len(r) * n // 2 // BLOCK_GLB, BLOCK_GLB, 8 * len(r) * nq, dst, temp, qhat_mod_r, alpha_q, qinv,
                base_q, nq, base_r, len(r), n)
    out = {"log_n": log_n, "bits": bits, "special": special, "t": t, "seed": seed,
           "bconv_q_to_r": sha(R.host(dst, len(r) * n))}
    frac, modr = oc.hps_tables()
    xr = O.random_residues(rng, list(q) + list(r), n, 1)[0]
    dst2 = R.zeros(len(r) * n + n)
    K.sr_qr_r(n // BLOCK_GLB, BLOCK_GLB, 0, dst2, R.dev(xr, n), R.dev(modr, 8), R.dev(frac, 8), base_r, n, nq,
              len(r))
    out["scale_round_qr_r"] = sha(R.host(dst2, len(r) * n))
    return out


class HpsConv:
    """DBaseConverter of the HPS bases (include/rns_bconv.cuh:26-60, src/host/rns.cu:420-470):
    QHatInvModq of the input base, QHatModp [out][in], alphaQModp [(in + 1)][out], 1/q_i."""

    def __init__(self, ibase, obase):
        big = 1
        for v in ibase:
            big *= v
        hat = [big // v for v in ibase]
        self.ni, self.no = len(ibase), len(obase)
        self.hat_inv, self.hat_inv_s = pair([pow(h % v, -1, v) for h, v in zip(hat, ibase)], ibase)
        self.hat_mod = R.dev(np.array([[h % p for h in hat] for p in obase], dtype=np.uint64), 8)
        self.alpha = R.dev(np.array([[(a * big) % p for p in obase] for a in range(len(ibase) + 1)],
                                    dtype=np.uint64), 8)
        self.inv = R.dev(np.array([1.0 / float(v) for v in ibase], dtype=np.float64), 8)
        self.ib, self.ob = R.dev(dmod(ibase), 8), R.dev(dmod(obase), 8)

    def run(self, K, dst, src, n, S):
        """DBaseConverter::bConv_HPS, src/rns_bconv.cu:354-372."""
        temp = S("hps_temp", self.ni * n + n)
        K.bconv_mult(self.ni * n // 2 // BLOCK_GLB, BLOCK_GLB, 0, temp, src, self.hat_inv, self.hat_inv_s, self.ib,
                     self.ni, n)
        K.bconv_hps(self.no * n // 2 // BLOCK_GLB, BLOCK_GLB, 8 * self.no * self.ni, dst, temp, self.hat_mod,
                    self.alpha, self.inv, self.ib, self.ni, self.ob, self.no, n)


class BfvSetup:
    def __init__(self, log_n, bits, special, t, rng):
        n = 1 << log_n
        self.n = n
        self.mods = O.create_coeff_modulus(n, bits)
        self.nq = nq = len(bits) - special
        self.special = special
        self.oc = O.Context(log_n, self.mods, nq, special, t)
        q, r = self.mods[:nq], self.oc.r_moduli
        self.q, self.r = q, r
        self.T = Tables(log_n, self.mods)
        self.Tqr = Tables(log_n, list(q) + list(r))
        self.q_to_r, self.r_to_q = HpsConv(q, r), HpsConv(r, q)
        frac, modr = self.oc.hps_tables()
        self.frac, self.modr = R.dev(frac, 8), R.dev(modr, 8)
        self.L = KsLevel(self.oc, self.T, nq)
        self.evk_t, self.evk_ptrs = key_setup(rng, self.mods, n, nq, special)


def ref_bfv_mul_relin(K, B, a_d, b_d, S):
    """bfv_mul_relin_hps with mul_tech hps (src/evaluate.cu:820-1026): a_d (2 x Q x N, device) is
    replaced by the relinearised product of a_d and b_d (coefficient form)."""
    n, nq, nr = B.n, B.nq, len(B.r)
    qr = nq + nr
    a_ = B.special
    qp = nq + a_
    ct1 = S("bfv_ct1", 3 * qr * n + n)
    ct2 = S("bfv_ct2", 2 * qr * n + n)
    for src, dst in ((a_d, ct1), (b_d, ct2)):
        for i in range(2):
            dst[i * qr * n: i * qr * n + nq * n].copy_(src[i * nq * n: (i + 1) * nq * n])
            B.q_to_r.run(K, R.Ptr(dst, i * qr * n + nq * n), R.Ptr(dst, i * qr * n), n, S)
    for buf in (ct1, ct2):
        for i in range(2):
            K.ntt_fwd(B.Tqr, R.Ptr(buf, i * qr * n), qr, 0)
    K.tensor(n * qr // BLOCK_GLB, BLOCK_GLB, 0, ct1, ct2, B.Tqr.mod, ct1, n, qr)
    for i in range(3):
        K.ntt_inv(B.Tqr, R.Ptr(ct1, i * qr * n), qr, 0)
    out3 = S("bfv_out3", 3 * nq * n + n)
    temp = S("bfv_rl", nr * n + n)
    for i in range(3):
        # DRNSTool::scaleAndRound_HPS_QR_R (src/rns.cu:1740-1747), then R -> Q
        K.sr_qr_r(n // BLOCK_GLB, BLOCK_GLB, 0, temp, R.Ptr(ct1, i * qr * n), B.modr, B.frac, B.r_to_q.ib, n, nq, nr)
        B.r_to_q.run(K, R.Ptr(out3, i * nq * n), temp, n, S)
    # key switch of c2 in BFV mode: modup (src/rns_bconv.cu:530-628, scheme bfv)
    L, T = B.L, B.T
    l, qlp, beta = L.l, L.qlp, L.beta
    c2 = R.Ptr(out3, 2 * nq * n)
    t_mod_up = S("t_mod_up", beta * qlp * n + n)
    t_cks = S("t_cks", l * n + n)
    s = sample_size(n)
    s2 = sample_size(n)
    s1 = n // s2
    K.copy_partql(n * l // BLOCK_GLB, BLOCK_GLB, 0, t_mod_up, c2, l * n, qlp * n, a_ * n)
    for d, D in enumerate(L.digits):
        part = R.Ptr(t_mod_up, d * qlp * n)
        K.bconv_mult1(n * D["sz"] // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(t_cks, D["start"] * n),
                      R.Ptr(out3, 2 * nq * n + D["start"] * n), R.Ptr(L.part_inv, D["start"]),
                      R.Ptr(L.part_inv_s, D["start"]), D["ibase"], D["sz"], n)
        K.bconv_padded(n * D["osz"] // BLOCK_GLB // 2, BLOCK_GLB, 8 * D["osz"] * D["sz"], part,
                       R.Ptr(t_cks, D["start"] * n), D["mat"], D["ibase"], D["sz"], D["obase"], D["osz"], n,
                       D["start"], D["sz"])
        # nwt_2d_radix8_forward_inplace_include_special_mod (src/ntt/fntt_2d.cu:695-736)
        K.f1_sp(GRID_NTT, s // 8 * PAD, (s + PAD + 1) * PAD * 8, part, T.tw, T.tws, T.mod, qlp, 0, qp, a_, n, s,
                PAD)
        K.f2_sp(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, part, T.tw, T.tws, T.mod, qlp, 0, qp, a_, n, s, n // s)
    thr = (1 << (64 - max(v.bit_length() for v in B.q) - 1)) - 1
    cx = S("cx", 2 * qlp * n + n)
    K.ip(qlp * n // BLOCK_GLB, BLOCK_GLB, 0, cx, t_mod_up, B.evk_ptrs, T.mod, n, qp, qp * n, qlp, qlp * n, nq, l,
         beta, thr)
    for i in range(2):
        cx_i = R.Ptr(cx, i * qlp * n)
        # moddown_from_NTT, scheme bfv (src/rns_bconv.cu:776-828)
        K.i1_sp(GRID_NTT, BLOCK_NTT, BLOCK_NTT * 64, cx_i, T.itw, T.itws, T.mod, qlp, 0, qp, a_, n, s1, s2)
        K.i2_sp(GRID_NTT, s1 // 8 * PAD, (s1 + PAD + 1) * PAD * 8, cx_i, T.itw, T.itws, T.ninv, T.ninvs, T.mod,
                qlp, 0, qp, a_, n, s1, PAD)
        temp2 = S("temp", a_ * n + n)
        delta = S("delta", l * n + n)
        K.bconv_mult(a_ * n // 2 // BLOCK_GLB, BLOCK_GLB, 0, temp2, R.Ptr(cx, i * qlp * n + l * n), L.p_hat_inv,
                     L.p_hat_inv_s, L.base_p, a_, n)
        K.bconv_matmul(l * n // 2 // BLOCK_GLB, BLOCK_GLB, 8 * l * a_, delta, temp2, L.p_to_ql, L.base_p, a_, T.mod,
                       l, n)
        K.moddown_k(l * n // BLOCK_GLB, BLOCK_GLB, 0, cx_i, cx_i, delta, T.mod, L.p_inv, L.p_inv_s, n, l)
    for i in range(2):
        K.add_to_ct(l * n // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(out3, i * nq * n), R.Ptr(cx, i * qlp * n), T.mod, n, l)
    a_d[: 2 * nq * n].copy_(out3[: 2 * nq * n])


def case_bfv(K, log_n, bits, special, t, seed):
    rng = np.random.default_rng(seed)
    B = BfvSetup(log_n, bits, special, t, rng)
    a = O.random_residues(rng, B.q, B.n, 2)
    b = O.random_residues(rng, B.q, B.n, 2)
    a_d, b_d = R.dev(a, B.n), R.dev(b, B.n)
    ref_bfv_mul_relin(K, B, a_d, b_d, Scratch())
    return {"log_n": log_n, "bits": bits, "special": special, "t": t, "seed": seed,
            "mul_relin": sha(R.host(a_d, 2 * B.nq * B.n))}


def seed_dev(seed):
    """A 64-byte seed in device memory (the reference's prng_seed arrays)."""
    return R.dev(np.frombuffer(seed, dtype="<u8").astype(np.uint64), 8)


def case_prng_keygen(K, log_n, bits, special, seed):
    """The reference's samplers (src/prng.cu:135-244, launched as src/secretkey.cu does, grid
    N * limbs / 128) and key generation from seeds: gen_secretkey (src/secretkey.cu:343-380),
    compute_secret_key_array (:196-230) and generate_one_kswitch_key (:297-341) with
    encrypt_zero_symmetric (:232-295) for the relinearisation key."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    nq, qp = len(bits) - special, len(bits)
    assert nq % special == 0, "the reference's key generation takes dnum = nQ / alpha"
    dnum = nq // special
    T = Tables(log_n, mods)
    rng = np.random.default_rng(seed)
    seed_u, seed_t, seed_e, seed_s = (rng.bytes(64) for _ in range(4))
    seeds_a = [rng.bytes(64) for _ in range(dnum)]
    seeds_e = [rng.bytes(64) for _ in range(dnum)]
    g = n * qp // BLOCK_GLB
    out = {"log_n": log_n, "bits": bits, "special": special, "seed": seed}
    u = R.zeros(qp * n + n)
    K.s_uniform(g, BLOCK_GLB, 0, u, seed_dev(seed_u), T.mod, n, qp)
    out["uniform"] = sha(R.host(u, qp * n))
    K.s_ternary(g, BLOCK_GLB, 0, u, seed_dev(seed_t), T.mod, n, qp)
    out["ternary"] = sha(R.host(u, qp * n))
    K.s_error(g, BLOCK_GLB, 0, u, seed_dev(seed_e), T.mod, n, qp)
    out["error"] = sha(R.host(u, qp * n))
    # gen_secretkey, then s^2
    sk = R.zeros(qp * n + n)
    K.s_ternary(g, BLOCK_GLB, 0, sk, seed_dev(seed_s), T.mod, n, qp)
    K.ntt_fwd(T, sk, qp, 0)
    out["secret_key"] = sha(R.host(sk, qp * n))
    s2 = R.zeros(qp * n + n)
    K.mul_poly(g, BLOCK_GLB, 0, sk, sk, T.mod, s2, n, qp)
    # generate_one_kswitch_key(s^2)
    pk = [R.zeros(2 * qp * n + n) for _ in range(dnum)]
    for d in range(dnum):
        err = R.zeros(qp * n + n)
        K.s_error(g, BLOCK_GLB, 0, err, seed_dev(seeds_e[d]), T.mod, n, qp)
        K.s_uniform(g, BLOCK_GLB, 0, R.Ptr(pk[d], qp * n), seed_dev(seeds_a[d]), T.mod, n, qp)
        K.ntt_fwd(T, err, qp, 0)
        K.mul_add_neg(g, BLOCK_GLB, 0, R.Ptr(pk[d], qp * n), sk, err, T.mod, pk[d], n, qp)
    ptrs = R.dev(np.array([t.data_ptr() for t in pk], dtype=np.uint64), 8)
    pmod = [1] * nq
    for j in range(nq):
        for p in mods[nq:]:
            pmod[j] = pmod[j] * p % mods[j]
    pm, pms = pair(pmod, mods[:nq])
    K.temp_mod_add(n * dnum * special // BLOCK_GLB, BLOCK_GLB, 0, s2, ptrs, T.mod, ptrs, n, dnum, special, pm, pms)
    out["relin_key"] = sha(np.concatenate([R.host(t, 2 * qp * n) for t in pk]))
    out["seeds"] = {"uniform": seed_u.hex(), "ternary": seed_t.hex(), "error": seed_e.hex(), "secret": seed_s.hex(),
                    "a": [x.hex() for x in seeds_a], "e": [x.hex() for x in seeds_e]}
    return out


def ref_bfv_decrypt(K, T, ct_d, sk, nq, t, q, n):
    """PhantomSecretKey::bfv_decrypt (src/secretkey.cu:571-635) with
    DRNSTool::hps_decrypt_scale_and_round (src/rns.cu:583-668 tables, 1634-1665 variant choice)."""
    g = n * nq // BLOCK_GLB
    temp = R.zeros(nq * n + n)
    temp[: nq * n].copy_(ct_d[nq * n: 2 * nq * n])
    K.ntt_fwd(T, temp, nq, 0)
    inner = R.zeros(nq * n + n)
    K.mul_add(g, BLOCK_GLB, 0, temp, sk, inner, T.mod, inner, n, nq)
    K.ntt_inv(T, inner, nq, 0)
    K.add_poly(g, BLOCK_GLB, 0, ct_d, inner, T.mod, inner, n, nq)
    qmsb, tmsb, smsb = max(v.bit_length() for v in q), t.bit_length(), nq.bit_length()
    big = 1
    for v in q:
        big *= v
    mt, fr, mtb, frb = [], [], [], []
    hf = qmsb >> 1
    for v in q:
        hinv = pow((big // v) % v, -1, v)
        x = t * hinv
        mt.append((x // v) % t)
        fr.append(float(x % v) / float(v))
        xb = t * ((hinv << hf) % v)
        mtb.append((xb // v) % t)
        frb.append(float(xb % v) / float(v))
    mt_d, mts_d = pair(mt, [t] * nq)
    mtb_d, mtbs_d = pair(mtb, [t] * nq)
    fr_d, frb_d = R.dev(np.array(fr), 8), R.dev(np.array(frb), 8)
    out = R.zeros(n + 8)
    gd = n // BLOCK_GLB
    if qmsb + smsb < 52:
        if qmsb + tmsb + smsb < 52:
            variant = "small_lazy"
            K.dec[variant](gd, BLOCK_GLB, 0, out, inner, mt_d, fr_d, t, n, nq)
        else:
            variant = "small"
            K.dec[variant](gd, BLOCK_GLB, 0, out, inner, mt_d, mts_d, fr_d, t, n, nq)
    elif hf + tmsb + smsb < 52:
        variant = "large_lazy"
        K.dec[variant](gd, BLOCK_GLB, 0, out, inner, mt_d, fr_d, mtb_d, frb_d, t, n, nq, hf)
    else:
        variant = "large"
        K.dec[variant](gd, BLOCK_GLB, 0, out, inner, mt_d, mts_d, fr_d, mtb_d, mtbs_d, frb_d, t, n, nq, hf)
    return R.host(out, n), variant


def case_bfv_io(K, log_n, bits, special, t, seed):
    """PhantomBatchEncoder encode / decode (src/batchencoder.cu:51-118, index map :25-49),
    BFV encrypt_symmetric (src/secretkey.cu:463-485 with encrypt_zero_symmetric :232-295 in
    coefficient form and src/scalingvariant.cu:10-31) and bfv_decrypt, on seeded values."""
    n = 1 << log_n
    mods = O.create_coeff_modulus(n, bits)
    nq, qp = len(bits) - special, len(bits)
    q = mods[:nq]
    T = Tables(log_n, mods)
    Tt = Tables(log_n, [t])
    rng = np.random.default_rng(seed)
    values = rng.integers(0, t, size=n, dtype=np.uint64)
    seed_s, seed_a, seed_e = (rng.bytes(64) for _ in range(3))
    # index map (src/batchencoder.cu:25-49)
    imap = np.zeros(n, dtype=np.uint64)
    pos, m = 1, 2 * n
    for i in range(n // 2):
        imap[i] = int(format((pos - 1) >> 1, f"0{log_n}b")[::-1], 2)
        imap[n // 2 + i] = int(format((m - pos - 1) >> 1, f"0{log_n}b")[::-1], 2)
        pos = (pos * 5) & (m - 1)
    imap_d = R.dev(imap, 8)
    pt = R.zeros(n + 8)
    gs = -(-n // BLOCK_GLB)
    K.encode_gpu(gs, BLOCK_GLB, 0, pt, R.dev(values, 8), n, imap_d, t, n)
    K.ntt_inv(Tt, pt, 1, 0)
    out = {"log_n": log_n, "bits": bits, "special": special, "t": t, "seed": seed, "encode": sha(R.host(pt, n))}
    cp = R.zeros(n + 8)
    cp[:n].copy_(pt[:n])
    K.ntt_fwd(Tt, cp, 1, 0)
    dec = R.zeros(n + 8)
    K.decode_gpu(gs, BLOCK_GLB, 0, dec, cp, imap_d, n)
    assert np.array_equal(R.host(dec, n), values), "reference batch encoder round trip"
    # secret key over QP (gen_secretkey), then encrypt at the first data level
    g = n * qp // BLOCK_GLB
    sk = R.zeros(qp * n + n)
    K.s_ternary(g, BLOCK_GLB, 0, sk, seed_dev(seed_s), T.mod, n, qp)
    K.ntt_fwd(T, sk, qp, 0)
    gq = n * nq // BLOCK_GLB
    ct = R.zeros(2 * nq * n + n)
    u = R.zeros(nq * n + n)
    K.s_error(gq, BLOCK_GLB, 0, u, seed_dev(seed_e), T.mod, n, nq)
    K.s_uniform(gq, BLOCK_GLB, 0, R.Ptr(ct, nq * n), seed_dev(seed_a), T.mod, n, nq)
    K.mul_poly(gq, BLOCK_GLB, 0, R.Ptr(ct, nq * n), sk, T.mod, ct, n, nq)
    K.ntt_inv(T, ct, nq, 0)
    K.add_neg(gq, BLOCK_GLB, 0, ct, u, T.mod, ct, n, nq)
    K.ntt_inv(T, R.Ptr(ct, nq * n), nq, 0)
    big = 1
    for v in q:
        big *= v
    negq = (-big) % t
    tinv, tinvs = pair([pow(t, -1, v) for v in q], q)
    K.add_timesq(gq, BLOCK_GLB, 0, ct, pt, negq, (negq << 64) // t, tinv, tinvs, T.mod, t, n, nq)
    out["encrypt"] = sha(R.host(ct, 2 * nq * n))
    m_dec, variant = ref_bfv_decrypt(K, T, ct, sk, nq, t, q, n)
    assert np.array_equal(m_dec, R.host(pt, n)), "reference decryption of its own encryption"
    out["decrypt_variant"] = variant
    rnd = R.dev(O.random_residues(rng, q, n, 2), n)
    m_rnd, _ = ref_bfv_decrypt(K, T, rnd, sk, nq, t, q, n)
    out["decrypt_random"] = sha(m_rnd)
    out["seeds"] = {"secret": seed_s.hex(), "a": seed_a.hex(), "e": seed_e.hex()}
    return out


def graph_time(fn, inner, reps, scratch=()):
    """Device time (ms) per call of fn(i), a sequence of reference launches and device copies:
    one synchronous warm-up run (allocates scratch), then `inner` calls captured in one CUDA graph,
    replayed `reps` times between CUDA events.  Host launch overhead is excluded, which can only
    favour the reference."""
    for i in range(inner):
        fn(i)
    torch.cuda.synchronize()
    for S in scratch:
        S.frozen = True
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        R.set_launch_mode(torch.cuda.current_stream().cuda_stream, sync=False)
        try:
            for i in range(inner):
                fn(i)
        finally:
            R.set_launch_mode()
    g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / (reps * inner)


def time_reference(K, path):
    """Times the replayed reference sequences on the N=2^16, 1x60 + 29x40 + 5x60, dnum=6
    parameter set at l=30 (HMult + relinearise + rescale, key switch, HRotate(1)), the forward
    NTT over 64 x 35 limbs, and the N=2^12 3x60 NTT round trip.  Four ciphertexts are cycled
    (working set > L2), one key shared, as in bench.py."""
    res = {}
    log_n, l, special = 16, 30, 5
    n = 1 << log_n
    bits = [60] + [40] * 29 + [60] * 5
    mods = O.create_coeff_modulus(n, bits)
    nq = len(bits) - special
    oc = O.Context(log_n, mods, nq, special)
    T = Tables(log_n, mods)
    L = KsLevel(oc, T, l)
    rt = rescale_tables(T, l)
    rng = np.random.default_rng(7)
    evk_t, evk_ptrs = key_setup(rng, mods, n, nq, special)
    S = Scratch()
    pairs = [(R.dev(O.random_residues(rng, mods[:l], n, 2), n), R.dev(O.random_residues(rng, mods[:l], n, 2), n))
             for _ in range(4)]
    d = [R.zeros(3 * l * n + n) for _ in range(4)]
    cp = R.zeros(2 * l * n + n)
    out = [R.zeros(2 * (l - 1) * n + n) for _ in range(4)]

    def hmult(i):
        a, b = pairs[i % 4]
        K.tensor(l * n // BLOCK_GLB, BLOCK_GLB, 0, a, b, T.mod, d[i % 4], n, l)
        ref_keyswitch(K, T, oc, L, d[i % 4], R.Ptr(d[i % 4], 2 * l * n), evk_ptrs, scratch=S)
        cp[: 2 * l * n].copy_(d[i % 4][: 2 * l * n])  # mod_switch_scale_to_next's encrypted_copy
        ref_rescale(K, T, cp, out[i % 4], l, 2, rt)

    res["ckks_hmult_relin_rescale_n16_l30_ms"] = graph_time(hmult, 4, 10, (S,))

    def keyswitch(i):
        a, b = pairs[i % 4]
        ref_keyswitch(K, T, oc, L, a, R.Ptr(b, 0), evk_ptrs, scratch=S)

    res["ckks_keyswitch_n16_l30_ms"] = graph_time(keyswitch, 4, 10, (S,))

    elt = O.elt_from_step(1, n)
    perm = torch.from_numpy(O.galois_perm(log_n, elt).view(np.int32).copy()).cuda()
    temp = R.zeros(l * n + n)

    def rotate(i):
        """apply_galois_inplace for CKKS, src/evaluate.cu:1567-1630."""
        c = pairs[i % 4][0]
        K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, temp, c, perm, n, l)
        c[: l * n].copy_(temp[: l * n])
        K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, temp, R.Ptr(c, l * n), perm, n, l)
        c[l * n: 2 * l * n].zero_()
        ref_keyswitch(K, T, oc, L, c, temp, evk_ptrs, scratch=S)

    res["ckks_hrotate_step1_n16_l30_ms"] = graph_time(rotate, 4, 10, (S,))
    del pairs, d, out, cp, evk_t, S
    torch.cuda.empty_cache()

    polys = 64
    Tq = Tables(log_n, mods)
    big = R.zeros(polys * len(mods) * n)

    def ntt64(i):
        for p in range(polys):
            K.ntt_fwd(Tq, R.Ptr(big, p * len(mods) * n), len(mods), 0)

    ms = graph_time(ntt64, 1, 10)
    res["ntt_forward_n16_64x35_ms"] = ms
    res["ntt_forward_n16_64x35_gbs"] = 16 * n * len(mods) * polys / (ms * 1e-3) / 1e9
    del big
    torch.cuda.empty_cache()

    rngb = np.random.default_rng(8)
    B = BfvSetup(15, [50] * 16 + [60, 60], 2, 65537, rngb)
    SB = Scratch()
    bins = [(R.dev(O.random_residues(rngb, B.q, B.n, 2), B.n), R.dev(O.random_residues(rngb, B.q, B.n, 2), B.n))
            for _ in range(4)]

    def bfv(i):
        a_d, b_d = bins[i % 4]
        ref_bfv_mul_relin(K, B, a_d, b_d, SB)

    res["bfv_mul_relin_n15_16x50_ms"] = graph_time(bfv, 4, 10, (SB,))
    del B, SB, bins
    torch.cuda.empty_cache()

    n12 = 4096
    m12 = O.create_coeff_modulus(n12, [60, 60, 60])
    T12 = Tables(12, m12)
    b12 = R.dev(O.random_residues(rng, m12, n12, 1), n12)

    def rt12(i):
        K.ntt_fwd(T12, b12, 3, 0)
        K.ntt_inv(T12, b12, 3, 0)

    res["ntt_n12_3x60_roundtrip_graph_us"] = 1e3 * graph_time(rt12, 50, 20)
    res["note"] = ("reference kernels compiled from source for sm_103a, replayed in CUDA graphs on the "
                   "reference's own launch configuration; device time only (no host launch or allocation cost)")
    with open(path, "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res))


def ref_apply_galois(K, T, oc, L, ct, perm, key_ptrs, temp, S):
    """apply_galois_inplace for CKKS (src/evaluate.cu:1567-1630) on ct (2 x l x N, device)."""
    n, l = oc.n, L.l
    K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, temp, ct, perm, n, l)
    ct[: l * n].copy_(temp[: l * n])
    K.galois(l * n // BLOCK_GLB, BLOCK_GLB, 0, temp, R.Ptr(ct, l * n), perm, n, l)
    ct[l * n: 2 * l * n].zero_()
    ref_keyswitch(K, T, oc, L, ct, temp, key_ptrs, scratch=S)


def time_reference_batched(K, path):
    """Device time of the reference's own kernels over the two batched workloads, as the reference
    serves a batch: a host loop of single-ciphertext calls (captured in CUDA graphs here, so host
    launch and allocation costs are excluded, which can only favour the reference).
    * 64 HMult + relinearise + rescale at levels drawn as bench.py draws them
      (default_rng(2000).integers(5, 31, 64)), N = 2^16, 1x60 + 29x40 + 5x60, one relinearisation key.
    * 32 matrix-vector products 128 x 128 by the reference's loop (bsgs_complete_from_cpu,
      python/src/binding.cu:507-595: G - 1 baby rotations, per giant step G plaintext products
      (multiply_plain: copy + multiply_rns_poly, src/evaluate.cu:1224-1250) summed by add_inplace
      (:116-195), a giant rotation by g G, the sum, one rescale) at N = 2^16, 1x60 + 19x40 + 4x60,
      G = 11, B = 12, at the levels of bench.py's draw."""
    res = {}
    log_n, n = 16, 1 << 16
    # ---- 64 HMult + relin + rescale at uneven levels
    bits, special = [60] + [40] * 29 + [60] * 5, 5
    mods = O.create_coeff_modulus(n, bits)
    nq = 30
    oc = O.Context(log_n, mods, nq, special)
    T = Tables(log_n, mods)
    levels = [int(x) for x in np.random.default_rng(2000).integers(5, 31, size=64)]
    Ls = {lv: KsLevel(oc, T, lv) for lv in sorted(set(levels))}
    rts = {lv: rescale_tables(T, lv) for lv in Ls}
    rng = np.random.default_rng(7)
    evk_t, evk_ptrs = key_setup(rng, mods, n, nq, special)
    S = Scratch()
    ins = [(R.dev(O.random_residues(rng, mods[:lv], n, 2), n), R.dev(O.random_residues(rng, mods[:lv], n, 2), n))
           for lv in levels]
    d = R.zeros(3 * nq * n + n)
    cp = R.zeros(2 * nq * n + n)
    outs = [R.zeros(2 * (lv - 1) * n + n) for lv in levels]

    def hmult(i):
        lv = levels[i]
        a, b = ins[i]
        K.tensor(lv * n // BLOCK_GLB, BLOCK_GLB, 0, a, b, T.mod, d, n, lv)
        ref_keyswitch(K, T, oc, Ls[lv], d, R.Ptr(d, 2 * lv * n), evk_ptrs, scratch=S)
        cp[: 2 * lv * n].copy_(d[: 2 * lv * n])
        ref_rescale(K, T, cp, outs[i], lv, 2, rts[lv])

    ms = graph_time(hmult, 64, 3, (S,))
    res["ckks_hmult_relin_rescale_batch64_levels5_30_ms_per_op"] = ms
    res["ckks_hmult_relin_rescale_batch64_levels5_30_ops_per_s"] = 1e3 / ms
    res["batch64_levels"] = levels
    del ins, outs, d, cp, evk_t, S, Ls
    torch.cuda.empty_cache()

    # ---- 32 matrix-vector products by the reference's loop
    bits, special = [60] + [40] * 19 + [60] * 4, 4
    mods = O.create_coeff_modulus(n, bits)
    nq, G, B, D = 20, 11, 12, 128
    oc = O.Context(log_n, mods, nq, special)
    T = Tables(log_n, mods)
    # bench.py's draw: 32 levels in 3..20 (default_rng(5000) after the key and matrix draws)
    mv_levels = [17, 19, 11, 6, 9, 10, 16, 20, 5, 18, 10, 8, 8, 12, 15, 4, 16, 5, 5, 11, 15, 7, 5, 15, 14, 11, 4, 7,
                 19, 4, 8, 19]
    Ls = {lv: KsLevel(oc, T, lv) for lv in sorted(set(mv_levels))}
    rts = {lv: rescale_tables(T, lv) for lv in Ls}
    rng = np.random.default_rng(8)
    steps = list(range(1, G)) + [g * G for g in range(1, B)]
    keys = {st: key_setup(rng, mods, n, nq, special) for st in steps}
    perms = {st: torch.from_numpy(O.galois_perm(log_n, O.elt_from_step(st, n)).view(np.int32).copy()).cuda()
             for st in steps}
    diags = R.dev(O.random_residues(rng, mods[:nq], n, D), n)  # [D][20][N]; level l reads limbs < l
    cts = [R.dev(O.random_residues(rng, mods[:lv], n, 2), n) for lv in mv_levels]
    S = Scratch()
    babies = [R.zeros(2 * nq * n + n) for _ in range(G)]
    term, inner, result = R.zeros(2 * nq * n + n), R.zeros(2 * nq * n + n), R.zeros(2 * nq * n + n)
    temp, cpy = R.zeros(nq * n + n), R.zeros(2 * nq * n + n)
    outs = [R.zeros(2 * (lv - 1) * n + n) for lv in mv_levels]

    def add_inplace(dst, src, lv):
        for p in range(2):
            K.add_poly(lv * n // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(dst, p * lv * n), R.Ptr(src, p * lv * n), T.mod,
                       R.Ptr(dst, p * lv * n), n, lv)

    def matvec(i):
        lv, ct = mv_levels[i], cts[i]
        L = Ls[lv]
        w = 2 * lv * n
        babies[0][:w].copy_(ct[:w])
        for b in range(1, G):  # phantom::rotate: copy, then rotate_inplace
            babies[b][:w].copy_(ct[:w])
            ref_apply_galois(K, T, oc, L, babies[b], perms[b], keys[b][1], temp, S)
        for g in range(B):
            first = True
            for b in range(G):
                k = g * G + b
                if k >= D:
                    continue
                dst = inner if first else term
                dst[:w].copy_(babies[b][:w])  # multiply_plain: copy, then multiply_plain_inplace
                for p in range(2):
                    K.mul_poly(lv * n // BLOCK_GLB, BLOCK_GLB, 0, R.Ptr(dst, p * lv * n), R.Ptr(diags, k * nq * n),
                               T.mod, R.Ptr(dst, p * lv * n), n, lv)
                if not first:
                    add_inplace(inner, term, lv)
                first = False
            if g > 0:
                ref_apply_galois(K, T, oc, L, inner, perms[g * G], keys[g * G][1], temp, S)
            if g == 0:
                result[:w].copy_(inner[:w])
            else:
                add_inplace(result, inner, lv)
        cpy[:w].copy_(result[:w])
        ref_rescale(K, T, cpy, outs[i], lv, 2, rts[lv])

    ms = graph_time(matvec, len(mv_levels), 2, (S,))
    res["ckks_matvec128_batch32_reference_loop_ms_per_matvec"] = ms
    res["ckks_matvec128_batch32_reference_loop_per_s"] = 1e3 / ms
    res["matvec_levels"] = mv_levels
    res["note"] = ("reference kernels compiled from source for sm_103a, replayed in CUDA graphs on the reference's "
                   "own launch configuration as a host loop of single-ciphertext calls; device time only")
    with open(path, "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res))


def extra_cases(K):
    """Hoisted rotations (hoisting_inplace) and the BFV modulus switch."""
    return {
        "hoist_ckks_n12_a2": case_hoisting(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 5, [1, 2, 4, -1], 1213),
        "hoist_ckks_n12_a2_l4": case_hoisting(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 4, [3, -5], 1214),
        "hoist_ckks_n16_l30": case_hoisting(K, 16, [60] + [40] * 29 + [60] * 5, 5, 30, [1, 2, 4, -1], 1608),
        "hoist_ckks_n16_l20_a4": case_hoisting(K, 16, [60] + [40] * 19 + [60] * 4, 4, 20, [1, 2, 11], 1609),
        "modswitch_bfv_n12_4x50": case_bfv_modswitch(K, 12, [50, 50, 50, 50, 60, 60], 2, 65537, 4, 1215),
        "modswitch_bfv_n15_16x50": case_bfv_modswitch(K, 15, [50] * 16 + [60, 60], 2, 65537, 16, 1504),
        "modswitch_bfv_n15_16x50_l9": case_bfv_modswitch(K, 15, [50] * 16 + [60, 60], 2, 65537, 9, 1505),
        "codec_n12_l5": case_codec(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 5, 2.0 ** 40, 2048, 1216),
        "codec_n12_l3_partial": case_codec(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 3, 2.0 ** 30, 1027, 1217),
        "codec_n12_l1": case_codec(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 1, 2.0 ** 40, 2048, 1218),
        "codec_n16_l30": case_codec(K, 16, [60] + [40] * 29 + [60] * 5, 5, 30, 2.0 ** 40, 32768, 1610),
        "codec_n16_l30_w128": case_codec(K, 16, [60] + [40] * 29 + [60] * 5, 5, 30, 2.0 ** 80, 32768, 1611),
        "codec_n16_l30_wide": case_codec(K, 16, [60] + [40] * 29 + [60] * 5, 5, 30, 2.0 ** 150, 20000, 1612),
        "codec_n16_l20_a4": case_codec(K, 16, [60] + [40] * 19 + [60] * 4, 4, 20, 2.0 ** 40, 32768, 1613),
        # a scale that is not a power of two: every FP64 product of the compose and the FFT rounds
        "codec_n16_l20_oddscale": case_codec(K, 16, [60] + [40] * 19 + [60] * 4, 4, 20, 1.2345 * 2.0 ** 40, 32768,
                                             1614),
        "codec_n12_l5_oddscale": case_codec(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 5, 0.7071 * 2.0 ** 40, 2048, 1219),
    }


def main(path):
    torch.zeros(1, device="cuda")
    K = Kernels()
    res = {
        "ntt_n12_3x60": case_ntt(K, 12, [60, 60, 60], 1201),
        "ntt_n16_4": case_ntt(K, 16, [60, 40, 40, 60], 1601),
        "ntt_n13_5": case_ntt(K, 13, [50, 50, 50, 50, 60], 1301),
        "ks_ckks_n12_a2": case_keyswitch(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, [5, 4, 2], 1202),
        "ks_ckks_n13_a3": case_keyswitch(K, 13, [60] + [50] * 5 + [60] * 3, 3, [6, 4, 1], 1302),
        "ks_ckks_n16_a5_l7": case_keyswitch(K, 16, [60] + [40] * 9 + [60] * 5, 5, [7], 1602),
        "hmult_ckks_n12_a2": case_hmult(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 5, 1206),
        "hmult_ckks_n16_l30": case_hmult(K, 16, [60] + [40] * 29 + [60] * 5, 5, 30, 1606),
        "hmult_ckks_n17_l8": case_hmult(K, 17, [60] + [50] * 7 + [60] * 4, 4, 8, 1701),
        "ks_ckks_n17_a4": case_keyswitch(K, 17, [60] + [50] * 7 + [60] * 4, 4, [8, 3], 1702),
        "ntt_n17_3": case_ntt(K, 17, [60, 50, 60], 1703),
        "rotate_ckks_n16_l30": case_rotate(K, 16, [60] + [40] * 29 + [60] * 5, 5, 30, 1, 1607),
        "rotate_ckks_n12_a2": case_rotate(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 5, -3, 1212),
        "rescale_n12": case_rescale(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 5, 1203),
        "tensor_galois_n12": case_tensor_galois(K, 12, [60, 40, 40, 40, 40, 60, 60], 2, 5, [1, -3, 7], 1204),
        "hps_n12": case_hps(K, 12, [50, 50, 50, 50, 60, 60], 2, 65537, 1205),
        "hps_n15": case_hps(K, 15, [50] * 16 + [60, 60], 2, 65537, 1501),
        "prng_keygen_n12": case_prng_keygen(K, 12, [60, 40, 40, 40, 60, 60], 2, 1208),
        "prng_keygen_n13_a3": case_prng_keygen(K, 13, [60] + [50] * 5 + [60] * 3, 3, 1304),
        "bfvio_n12_4x50": case_bfv_io(K, 12, [50, 50, 50, 50, 60, 60], 2, 65537, 1209),
        "bfvio_n13_6x40": case_bfv_io(K, 13, [40] * 6 + [60], 1, 786433, 1305),
        "bfvio_n15_16x50": case_bfv_io(K, 15, [50] * 16 + [60, 60], 2, 65537, 1503),
        "bfvio_n12_3x30": case_bfv_io(K, 12, [30, 30, 30, 60], 1, 65537, 1210),
        "bfvio_n12_3x60": case_bfv_io(K, 12, [60, 60, 60, 60], 1, 786433, 1211),
        "bfv_n12_4x50": case_bfv(K, 12, [50, 50, 50, 50, 60, 60], 2, 65537, 1207),
        "bfv_n13_a3": case_bfv(K, 13, [50] * 6 + [60] * 3, 3, 65537, 1303),
        "bfv_n15_16x50": case_bfv(K, 15, [50] * 16 + [60, 60], 2, 65537, 1502),
    }
    res.update(extra_cases(K))
    with open(path, "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps({k: "ok" for k in res}))


if __name__ == "__main__":
    if len(sys.argv) == 3 and sys.argv[1] == "--time":
        torch.zeros(1, device="cuda")
        time_reference(Kernels(), sys.argv[2])
    elif len(sys.argv) == 3 and sys.argv[1] == "--time-batched":
        torch.zeros(1, device="cuda")
        time_reference_batched(Kernels(), sys.argv[2])
    elif len(sys.argv) == 3 and sys.argv[1] == "--extra":  # only the cases of extra_cases()
        torch.zeros(1, device="cuda")
        res = extra_cases(Kernels())
        with open(sys.argv[2], "w") as f:
            json.dump(res, f, indent=1, sort_keys=True)
        print(json.dumps({k: "ok" for k in res}))
    else:
        main(sys.argv[1])
