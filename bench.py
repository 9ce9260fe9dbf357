#!/usr/bin/env python3
"""Benchmark: CKKS HMult + relinearise + rescale at N = 2^16, 30 data primes (1x60 + 29x40),
5 special primes (dnum = 6), on one GB300 per rank.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one HMult+relin+rescale of one ciphertext pair at chain index 1 (l = 30), batch 1,
through the library's C ABI (fhe_ckks_multiply_relin_rescale).  The per-step working set is
283 MB (2 ciphertexts + the 220 MB relinearisation key) > the 129 MB L2, and 4 ciphertext
pairs are cycled.  Inputs are seeded synthetic residues (uniform in [0, q_i)); keys are
uniform residues of the key layout.  `--impl reference` times the CPU restatement of the
same operation (the reference has no CPU implementation of this path) on the host cores.
Multi-GPU runs are independent replicas (the path has no cross-GPU exchange).
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "phantom-fhe_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

N = 1 << 16
BITS = [60] + [40] * 29 + [60] * 5
SPECIAL = 5
CHAIN = 1
PAIRS = 4
METRIC = "CKKS HMult+relin+rescale ops/s (N=2^16, l=30, dnum=6, bit-exact)"
CONFIG = {"workload": "ckks_hmult_relin_rescale", "poly_degree": N, "data_primes": "1x60+29x40",
          "special_primes": "5x60", "dnum": 6, "level": 30, "batch": 1,
          "l2": "per-step working set 283 MB (> 129 MB L2); 4 ciphertext pairs cycled"}


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(t, world, device):
    """The slowest rank's time: replicas are timed independently and the job ends with the last."""
    if world <= 1:
        return t
    import torch
    tt = torch.tensor([t], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def replica_throughput(steps, world, t):
    """Whole-job throughput of `world` replicas that each ran `steps` operations in at most t s."""
    return steps * world / t


def random_residues(rng, moduli, n, polys):
    out = np.empty((polys, len(moduli), n), dtype=np.uint64)
    for k, q in enumerate(moduli):
        out[:, k, :] = rng.integers(0, q, size=(polys, n), dtype=np.uint64)
    return out


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return {}


class Clocks:
    """nvidia-smi sampler running while the timed regions run."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "100", "-i", str(gpu)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_baseline_sample(mods, nq, threads):
    """One full HMult+relin+rescale on the host cores with the CPU restatement."""
    from oracle import oracle as O
    O.set_threads(threads)
    oc = O.Context(16, mods, nq, SPECIAL)
    rng = np.random.default_rng(7)
    l = nq
    a = random_residues(rng, mods[:l], N, 2)
    b = random_residues(rng, mods[:l], N, 2)
    dnum = (nq + SPECIAL - 1) // SPECIAL
    key = random_residues(rng, mods, N, 2 * dnum).reshape(dnum, 2, len(mods), N)
    oc.rescale(l, oc.ckks_mul_relin(l, a, b, key))  # warm-up (page-in, thread pool)
    t0 = time.perf_counter()
    reps = 0
    while True:
        oc.rescale(l, oc.ckks_mul_relin(l, a, b, key))
        reps += 1
        if time.perf_counter() - t0 > 10.0 or reps >= 200:
            break
    dt = time.perf_counter() - t0
    return reps / dt, reps, dt


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as O
    mods = O.create_coeff_modulus(N, BITS)
    nq = len(BITS) - SPECIAL
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    oc = O.Context(16, mods, nq, SPECIAL)
    rng = np.random.default_rng(7)
    l = nq
    a = random_residues(rng, mods[:l], N, 2)
    b = random_residues(rng, mods[:l], N, 2)
    dnum = (nq + SPECIAL - 1) // SPECIAL
    key = random_residues(rng, mods, N, 2 * dnum).reshape(dnum, 2, len(mods), N)
    for _ in range(min(args.warmup, 1)):
        oc.rescale(l, oc.ckks_mul_relin(l, a, b, key))
    # each step is the full operation; the step count is capped so the run stays bounded
    t0 = time.perf_counter()
    steps = 0
    while steps < args.steps:
        oc.rescale(l, oc.ckks_mul_relin(l, a, b, key))
        steps += 1
        if time.perf_counter() - t0 > 60.0:
            break
    dt = time.perf_counter() - t0
    value = steps / dt
    sample = f"{steps} full HMult+relin+rescale ops at N=2^16, l=30 (of {args.steps} requested)"
    line = {"impl": "reference", "arm": "cpu_port",
            "arm_note": ("PhantomFHE has no CPU implementation of this path: this arm is the CPU restatement "
                         "(oracle/) on the host cores, not the reference's CUDA kernels"),
            "metric": METRIC, "value": value, "unit": "ops/s", "n_gpus": world,
            "steps": steps, "warmup": min(args.warmup, 1), "ms_per_step": 1000 * dt / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic", "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": "ops/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "ops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


MV_BITS = [60] + [40] * 19 + [60] * 4  # Q = 1x60 + 19x40, P = 4x60 (dnum = 5)
MV_DIM, MV_G, MV_B, MV_BATCH = 128, 11, 12, 32


def matvec_bench(pg, torch, timed, stream, rank, profile_only=False):
    """128x128 plaintext matrix times encrypted vector by the diagonal method with baby-step /
    giant-step rotations at N = 2^16 (Q = 1x60 + 19x40, P = 4x60, dnum = 5): 32 vectors at
    levels drawn uniformly from 3..20, real keys from seeded randomness, matrix entries uniform
    in [-1, 1].  Hoisted form: baby steps 1..10 share one mod-up, giant steps by Horner's rule
    with rotations by 11 only (11 Galois keys); the reference's loop (giant rotations by g*11,
    21 keys) runs beside it.  The per-vector calls read diagonals encoded at each vector's level;
    the batched call reads one array encoded at the top level (its first l limbs are the same
    words).  Slot error of the decrypted results against an FP64 matmul."""
    from phantom_gb300.ckks import CkksEncoder, SecretKey
    n, d, G, B = N, MV_DIM, MV_G, MV_B
    mods = pg.create_coeff_modulus(n, MV_BITS)
    nq = 20
    hsteps = list(range(1, G + 1))
    xsteps = list(range(1, G)) + [g * G for g in range(1, B)]
    ctx = pg.Context(n, mods, 4, galois_elts=sorted({pg.elt_from_step(s, n) for s in hsteps + xsteps}))
    ws = ctx.workspace()
    ctx.autotune(ws)
    rng = np.random.default_rng(5000 + rank)
    sk = SecretKey(ctx, rng)
    gks = sk.galois_keys(ws, sorted(set(hsteps + xsteps)))
    enc = CkksEncoder(n)
    S = n // 2
    scale = 2.0 ** 40
    M = rng.uniform(-1, 1, size=(d, d))
    idx = np.arange(S)
    diag_full = torch.stack([enc.encode(ctx, np.roll(M[idx % d, (idx + k) % d], (k // G) * G), scale, 1)
                             for k in range(d)])
    levels = [int(x) for x in rng.integers(3, 21, size=MV_BATCH)]
    diags_at = {}
    for lv in sorted(set(levels)):
        diags_at[lv] = diag_full[:, :lv].contiguous()
    xs, cts, outs = [], [], []
    for lv in levels:
        x = rng.uniform(-1, 1, size=d) + 1j * rng.uniform(-1, 1, size=d)
        x /= np.maximum(1, np.abs(x))
        chain = nq - lv + 1
        xs.append(x)
        cts.append((sk.encrypt(enc.encode(ctx, np.tile(x, S // d), scale, chain), chain), chain, lv))
        outs.append(torch.empty((2, lv - 1, n), dtype=torch.int64, device="cuda"))
    scratch = torch.empty(ctx.bsgs_scratch_bytes(G) // 8, dtype=torch.int64, device="cuda")

    def batch(hoisted):
        for (ct, chain, lv), o in zip(cts, outs):
            ctx.bsgs_matvec(ws, scratch, ct, chain, diags_at[lv], d, G, B, gks, o, hoisted=hoisted, stream=stream)

    # the same 32 products through the batched call: one launch per pipeline step for all of them,
    # every item reading the one matrix's diagonals encoded at the top level (the first l limbs)
    wsb = ctx.workspace(batch_items=MV_BATCH)
    bscratch = torch.empty(MV_BATCH * ctx.bsgs_batch_scratch_bytes(G, B) // 8, dtype=torch.int64, device="cuda")
    bouts = [torch.empty_like(o) for o in outs]
    bitems = [(ct, chain, diag_full, o) for (ct, chain, lv), o in zip(cts, bouts)]

    def batched():
        ctx.bsgs_matvec_batch(wsb, bscratch, bitems, d, G, B, gks, stream=stream)

    batch(True)
    if profile_only:
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("matvec_case")  # lets a profiler skip the setup's launches
        if os.environ.get("BENCH_MATVEC_BATCHED", "0") == "1":
            batched()
        else:
            batch(True)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        return {}
    torch.cuda.synchronize()
    l0 = pg.lib.fhe_kernel_launches()
    k = 3
    t_h = timed(lambda i: batch(True), k) / k
    launches = (pg.lib.fhe_kernel_launches() - l0) / k
    errs = []
    for (ct, chain, lv), o, x in zip(cts, outs, xs):
        y = enc.decode(ctx, sk.decrypt(o, chain + 1), scale * scale / mods[lv - 1], chain + 1)
        errs.append(float(np.max(np.abs(y - np.tile(M @ x, S // d)))))
    err_h = max(errs)
    batched()
    torch.cuda.synchronize()
    same = all(torch.equal(a, b) for a, b in zip(outs, bouts))
    l0 = pg.lib.fhe_kernel_launches()
    t_b = timed(lambda i: batched(), k) / k
    launches_b = (pg.lib.fhe_kernel_launches() - l0) / k
    del bscratch, wsb
    batch(False)
    t_x = timed(lambda i: batch(False), k) / k
    errs = []
    for (ct, chain, lv), o, x in zip(cts, outs, xs):
        y = enc.decode(ctx, sk.decrypt(o, chain + 1), scale * scale / mods[lv - 1], chain + 1)
        errs.append(float(np.max(np.abs(y - np.tile(M @ x, S // d)))))
    return {"matvec128_batch32_uneven_hoisted_per_s": MV_BATCH / t_h,
            "matvec128_batch32_uneven_batched_per_s": MV_BATCH / t_b,
            "matvec128_batched_launches_per_batch": launches_b,
            "matvec128_batched_equals_single_calls": same,
            "matvec128_batch32_uneven_reference_loop_per_s": MV_BATCH / t_x,
            "matvec128_hoisted_max_slot_error": err_h,
            "matvec128_reference_loop_max_slot_error": max(errs),
            "matvec128_hoisted_launches_per_batch": launches,
            "matvec128_levels": levels}


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import phantom_gb300 as pg
    lib = pg.lib
    lib.fhe_kernel_launches.restype = ctypes.c_uint64

    mods = pg.create_coeff_modulus(N, BITS)
    nq = len(BITS) - SPECIAL
    l = nq
    ctx = pg.Context(N, mods, SPECIAL)
    ws = ctx.workspace()
    tuning = ctx.autotune(ws)  # kernel shapes, chosen by timing this operation (setup, outside every timed region)
    if args.case != "full" and "BENCH_FUSED" in os.environ:  # profiling cases: pick the key-switch form
        ctx.fused_keyswitch = os.environ["BENCH_FUSED"] == "1"
    rng = np.random.default_rng(1000 + rank)
    key = pg.KeySwitchKey(pg.to_device(random_residues(rng, mods, N, 2 * ctx.dnum).reshape(ctx.dnum, 2, len(mods), N)))
    elt1 = pg.elt_from_step(1, N)
    gks = [None] * len(ctx.galois_elts)
    gks[ctx.galois_elts.index(elt1)] = key
    a = [pg.to_device(random_residues(rng, mods[:l], N, 2)) for _ in range(PAIRS)]
    b = [pg.to_device(random_residues(rng, mods[:l], N, 2)) for _ in range(PAIRS)]
    out = [torch.empty((2, l - 1, N), dtype=torch.int64, device="cuda") for _ in range(PAIRS)]
    stream = torch.cuda.current_stream()

    def step(i):
        ctx.multiply_relin_rescale(ws, a[i % PAIRS], b[i % PAIRS], out[i % PAIRS], CHAIN, key, stream)

    def timed(fn, k):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for i in range(k):
            fn(i)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    if args.case == "bfv":  # profiling case: BFV HPS multiply + relinearise at N = 2^15
        nb = 1 << 15
        bmods = pg.create_coeff_modulus(nb, [50] * 16 + [60, 60])
        bctx = pg.Context(nb, bmods, 2, scheme=pg.SCHEME_BFV, plain_modulus=65537)
        bws = bctx.workspace()
        bkey = pg.KeySwitchKey(pg.to_device(random_residues(rng, bmods, nb, 2 * bctx.dnum)
                                            .reshape(bctx.dnum, 2, len(bmods), nb)))
        x = pg.to_device(random_residues(rng, bmods[:16], nb, 2))
        y = pg.to_device(random_residues(rng, bmods[:16], nb, 2))
        for _ in range(args.warmup + args.steps):
            bctx.multiply_and_relin(bws, x, y, 1, bkey, stream)
        torch.cuda.synchronize()
        return
    if args.case == "ntt":  # profiling case: forward NTT of 8 polys x 35 limbs (147 MB)
        big = torch.randint(0, 1 << 40, (8, len(mods), N), dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("ntt_case")  # lets a profiler skip the autotuner's launches
        for _ in range(args.warmup + args.steps):
            ctx.ntt_forward(big, 8, len(mods), 0, stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        return
    if args.case == "batch":  # profiling case: batched HMult+relin+rescale, 64 at levels 5..30
        brng = np.random.default_rng(2000 + rank)
        levels = [int(x) for x in brng.integers(5, 31, size=64)]
        items = []
        for lv in levels:
            ta = torch.randint(0, 1 << 40, (2, lv, N), dtype=torch.int64, device="cuda")
            tb = torch.randint(0, 1 << 40, (2, lv, N), dtype=torch.int64, device="cuda")
            items.append((ta, tb, torch.empty((2, lv - 1, N), dtype=torch.int64, device="cuda"), nq - lv + 1))
        wsb = ctx.workspace(batch_items=64)
        ctx.fused_keyswitch = os.environ.get("BENCH_BATCH_FUSED", "1") == "1"
        for _ in range(args.warmup + args.steps):
            ctx.multiply_relin_rescale_batch(wsb, items, key, stream)
        torch.cuda.synchronize()
        return
    if args.case == "matvec":  # profiling case: one batch of 32 hoisted matrix-vector products
        matvec_bench(pg, torch, timed, stream, rank, profile_only=True)
        return
    for i in range(max(args.warmup, 3)):
        step(i)
    torch.cuda.synchronize()
    if args.case == "hmult":  # profiling case: HMult+relin+rescale steps only
        for i in range(args.steps):
            step(i)
        torch.cuda.synchronize()
        return

    clocks = Clocks(local)
    time.sleep(0.3)
    barrier()
    l0 = lib.fhe_kernel_launches()
    t = timed(step, args.steps)
    launches = lib.fhe_kernel_launches() - l0
    barrier()
    t = max_over_ranks(t, world, "cuda")
    value = replica_throughput(args.steps, world, t)

    # companion measurements on the same parameters (same timing rules)
    k2 = max(args.steps // 2, 10)
    ct = pg.to_device(random_residues(rng, mods[:l], N, 2))
    c2 = pg.to_device(random_residues(rng, mods[:l], N, 1)[0])
    t_rot = timed(lambda i: ctx.rotate(ws, ct, CHAIN, 1, gks, stream), k2)
    t_ks = timed(lambda i: ctx.keyswitch(ws, ct, c2, CHAIN, key, stream), k2)
    # the same operations with the base conversions on the CUDA cores instead of the tensor cores
    tc_default = ctx.tensor_cores
    ctx.tensor_cores = False
    t_hm_cc = timed(step, k2)
    t_ks_cc = timed(lambda i: ctx.keyswitch(ws, ct, c2, CHAIN, key, stream), k2)
    ctx.tensor_cores = tc_default
    # ... and with the mod-up's row pass and the inner product as two kernels (t_mod_up written)
    # and as the fused kernel, whichever the autotuner chose
    tuned_fused = ctx.fused_keyswitch
    ctx.fused_keyswitch = False
    t_hm_unfused = timed(step, k2)
    t_ks_unfused = timed(lambda i: ctx.keyswitch(ws, ct, c2, CHAIN, key, stream), k2)
    ctx.fused_keyswitch = True
    t_hm_fused = timed(step, k2)
    t_ks_fused = timed(lambda i: ctx.keyswitch(ws, ct, c2, CHAIN, key, stream), k2)
    ctx.fused_keyswitch = tuned_fused
    tc_status = ctx.device_status()
    # NTT throughput: 64 polynomials x 35 limbs (1.17 GB > 4x L2), forward transform
    polys, limbs = 64, len(mods)
    big = torch.randint(0, 1 << 40, (polys, limbs, N), dtype=torch.int64, device="cuda")
    kn = 10
    # the transform's own shapes: every NTT split and tile (same words), the fastest kept; the
    # operation's tuned shapes are restored afterwards
    saved = ctx.tuning
    ntt_times = {}
    for split in (7, 8):  # the splits supported at N = 2^16
        for tile in (2048, 4096):
            ctx.tuning = {"ntt_split": split, "ntt_tile": tile}
            ctx.ntt_forward(big, polys, limbs, 0, stream)
            ntt_times[(split, tile)] = timed(lambda i: ctx.ntt_forward(big, polys, limbs, 0, stream), kn) / kn
    ctx.tuning = {k: v for k, v in saved.items() if k not in ("best_us", "evaluated")}
    ntt_shape = min(ntt_times, key=ntt_times.get)
    t_ntt = ntt_times[ntt_shape]
    ntt_bytes = 16 * N * limbs * polys
    ntt_gbs = ntt_bytes / t_ntt / 1e9
    del big

    # NTT forward + inverse round trip at N = 2^12 over 3 x 60-bit primes, batch 1 (latency)
    n12 = 1 << 12
    c12 = pg.Context(n12, pg.create_coeff_modulus(n12, [60, 60, 60]), 1)
    d12 = torch.randint(0, 1 << 59, (1, 3, n12), dtype=torch.int64, device="cuda")
    for _ in range(5):
        c12.ntt_forward(d12, 1, 3, 0, stream)
        c12.ntt_inverse(d12, 1, 3, 0, stream)
    # a latency of a few microseconds: the median of five trials of each form
    k12 = 200
    t12 = statistics.median(
            timed(lambda i: (c12.ntt_forward(d12, 1, 3, 0, stream), c12.ntt_inverse(d12, 1, 3, 0, stream)), k12) / k12
            for _ in range(5))
    # device-side latency without the per-call host path: 50 round trips captured in one CUDA graph
    g12 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g12):
        for _ in range(50):
            c12.ntt_forward(d12, 1, 3, 0)
            c12.ntt_inverse(d12, 1, 3, 0)
    g12.replay()
    t12g = statistics.median(timed(lambda i: g12.replay(), 4) / (4 * 50) for _ in range(5))
    del g12, c12, d12

    # batch of 64 HMult+relin+rescale at levels drawn uniformly from 5..30 (one call), and the
    # same 64 operations as a loop of single calls
    brng = np.random.default_rng(2000 + rank)
    levels = [int(x) for x in brng.integers(5, 31, size=64)]
    items = []
    for lv in levels:
        ta = torch.randint(0, 1 << 40, (2, lv, N), dtype=torch.int64, device="cuda")
        tb = torch.randint(0, 1 << 40, (2, lv, N), dtype=torch.int64, device="cuda")
        items.append((ta, tb, torch.empty((2, lv - 1, N), dtype=torch.int64, device="cuda"), nq - lv + 1))
    wsb = ctx.workspace(batch_items=64)
    kb = 5
    ks_items = [(x[0], x[1][1], x[3]) for x in items]  # ct = the first operand, c2 = one poly of the second
    t_batch, t_ksb = {}, {}
    # both forms of the batched mod-up + inner product: the row pass fused with the inner product
    # (every item's blocks for one key tile run together) and the two-kernel form
    for fused in (True, False):
        ctx.fused_keyswitch = fused
        ctx.multiply_relin_rescale_batch(wsb, items, key, stream)
        t_batch[fused] = timed(lambda i: ctx.multiply_relin_rescale_batch(wsb, items, key, stream), kb) / kb
        # the same 64 levels as a batch of key switches (ct += KeySwitch(c2))
        ctx.keyswitch_batch(wsb, ks_items, key, stream)
        t_ksb[fused] = timed(lambda i: ctx.keyswitch_batch(wsb, ks_items, key, stream), kb) / kb
    # the single calls keep the autotuner's choice; batches run fused unless told otherwise
    ctx.fused_keyswitch = True
    ctx.tuning = {k: v for k, v in tuning.items() if k not in ("best_us", "evaluated")}
    # ... and as loops of single calls
    t_loop = timed(lambda i: [ctx.multiply_relin_rescale(ws, x[0], x[1], x[2], x[3], key, stream) for x in items],
                   kb) / kb
    t_ksl = timed(lambda i: [ctx.keyswitch(ws, x[0], x[1], x[2], key, stream) for x in ks_items], kb) / kb
    # algorithmic bytes of the batch: per ciphertext 8N (4l + 2(l - 1)) (both inputs read, the
    # output written), the key once over the largest level's digits and QlP limbs
    lmax = max(levels)
    batch_bytes = sum(8 * N * (4 * lv + 2 * (lv - 1)) for lv in levels) + \
        8 * N * 2 * ((lmax + SPECIAL - 1) // SPECIAL) * (lmax + SPECIAL)
    del items, ks_items, wsb

    # BFV multiply + relinearise (HPS) at N = 2^15, 16x50-bit + 2x60-bit, t = 65537:
    # 128 operations captured in one CUDA graph, replayed
    bfv_bits = [50] * 16 + [60, 60]
    nb = 1 << 15
    bmods = pg.create_coeff_modulus(nb, bfv_bits)
    bctx = pg.Context(nb, bmods, 2, scheme=pg.SCHEME_BFV, plain_modulus=65537)
    bws = bctx.workspace()
    btuning = bctx.autotune(bws)
    bkey = pg.KeySwitchKey(pg.to_device(random_residues(rng, bmods, nb, 2 * bctx.dnum)
                                        .reshape(bctx.dnum, 2, len(bmods), nb)))
    bct = [pg.to_device(random_residues(rng, bmods[:16], nb, 2)) for _ in range(2)]
    bpairs = [(bct[0].clone(), bct[1]) for _ in range(128)]
    for x, y in bpairs[:3]:
        bctx.multiply_and_relin(bws, x, y, 1, bkey, stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for x, y in bpairs:
            bctx.multiply_and_relin(bws, x, y, 1, bkey)
    g.replay()
    t_graph = timed(lambda i: g.replay(), 3) / 3
    t_bloop = timed(lambda i: [bctx.multiply_and_relin(bws, x, y, 1, bkey, stream) for x, y in bpairs], 3) / 3
    bctx.tensor_cores = False
    t_bloop_cc = timed(lambda i: [bctx.multiply_and_relin(bws, x, y, 1, bkey, stream) for x, y in bpairs], 3) / 3
    bctx.tensor_cores = True
    del g, bpairs, bct, bws, bctx

    mv = matvec_bench(pg, torch, timed, stream, rank)

    # end to end through the C ABI with host buffers: H2D of both inputs, D2H of the result
    pin_a = [torch.empty((2, l, N), dtype=torch.int64).pin_memory() for _ in range(PAIRS)]
    pin_b = [torch.empty((2, l, N), dtype=torch.int64).pin_memory() for _ in range(PAIRS)]
    pin_o = [torch.empty((2, l - 1, N), dtype=torch.int64).pin_memory() for _ in range(PAIRS)]
    for i in range(PAIRS):
        pin_a[i].copy_(a[i].cpu())
        pin_b[i].copy_(b[i].cpu())
    # two buffer sets; the step's H2D runs on its own stream while the previous operation
    # computes, its D2H on another while the next one computes (operations stay serial on
    # `stream`, so this overlaps transfers only)
    da = [torch.empty((2, l, N), dtype=torch.int64, device="cuda") for _ in range(2)]
    db = [torch.empty((2, l, N), dtype=torch.int64, device="cuda") for _ in range(2)]
    do = [torch.empty((2, l - 1, N), dtype=torch.int64, device="cuda") for _ in range(2)]
    # the two input ciphertexts travel on two streams, so two copy engines carry them at once
    h2d_s, h2d_s2, d2h_s = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ("h2d", "h2d2", "comp", "d2h")}
    started = [False, False]

    def e2e_step(i):
        b = i % 2
        for hs, dst, src, e in ((h2d_s, da, pin_a, "h2d"), (h2d_s2, db, pin_b, "h2d2")):
            with torch.cuda.stream(hs):
                if started[b]:
                    hs.wait_event(ev["comp"][b])  # inputs of the operation two steps back consumed
                dst[b].copy_(src[i % PAIRS], non_blocking=True)
                ev[e][b].record(hs)
        stream.wait_event(ev["h2d"][b])
        stream.wait_event(ev["h2d2"][b])
        if started[b]:
            stream.wait_event(ev["d2h"][b])  # its output buffer read back
        ctx.multiply_relin_rescale(ws, da[b], db[b], do[b], CHAIN, key, stream)
        ev["comp"][b].record(stream)
        with torch.cuda.stream(d2h_s):
            d2h_s.wait_event(ev["comp"][b])
            pin_o[i % PAIRS].copy_(do[b], non_blocking=True)
            ev["d2h"][b].record(d2h_s)
        started[b] = True

    def e2e_timed(k):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h2d_s.wait_event(e0)
        h2d_s2.wait_event(e0)
        for i in range(k):
            e2e_step(i)
        stream.wait_stream(d2h_s)  # every result back on the host
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0

    for i in range(3):
        e2e_step(i)
    barrier()
    t_e2e = e2e_timed(args.steps)
    barrier()
    t_e2e = max_over_ranks(t_e2e, world, "cuda")
    ck = clocks.stop()

    # the host link's own rates for these buffers (the ceiling of the end-to-end figure): both
    # input ciphertexts host -> device on their two streams, the result device -> host
    def link_rate(fn, nbytes, reps=10):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return nbytes * reps / (time.perf_counter() - t0) / 1e9

    def h2d_pair():
        with torch.cuda.stream(h2d_s):
            da[0].copy_(pin_a[0], non_blocking=True)
        with torch.cuda.stream(h2d_s2):
            db[0].copy_(pin_b[0], non_blocking=True)

    def d2h_one():
        with torch.cuda.stream(d2h_s):
            pin_o[0].copy_(do[0], non_blocking=True)

    h2d_gbs = link_rate(h2d_pair, 2 * 2 * l * N * 8)
    d2h_gbs = link_rate(d2h_one, 2 * (l - 1) * N * 8)

    peak, peak_kind = measured_peaks()
    prof = profile_traffic()
    traffic = prof.get("ntt_forward_64x35_n16")
    # the NTT's binding limit is instruction issue into the integer pipes: warp instructions per
    # butterfly (ncu, committed) x butterflies per second against SMs x 4 schedulers x SM clock
    wipb = prof.get("ntt_forward_warp_inst_per_butterfly")
    butterflies = polys * limbs * (N // 2) * int(math.log2(N))
    issue = None
    if wipb and ck.get("sm_mhz"):
        got = butterflies * wipb / t_ntt
        top = torch.cuda.get_device_properties(local).multi_processor_count * 4 * ck["sm_mhz"] * 1e6
        issue = {"warp_inst_per_butterfly": wipb, "achieved": got, "peak": top, "unit": "warp inst/s",
                 "frac": got / top, "source": "ncu smsp__inst_executed.sum per butterfly; peak at the median SM clock",
                 "busiest_pipe_ncu": {"pipe": "fmaheavy (IMAD)",
                                      **prof.get("ntt_forward_fmaheavy_pipe_frac", {})}}
    line = {"metric": METRIC, "value": value, "unit": "ops/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1000 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": dict(CONFIG, tuning=dict({k: v for k, v in tuning.items() if k not in ("best_us",)},
                                               source="autotuned on this operation")),
            "clocks": ck,
            "e2e": {"value": replica_throughput(args.steps, world, t_e2e), "unit": "ops/s",
                    "h2d_bytes_per_step": 2 * 2 * l * N * 8, "d2h_bytes_per_step": 2 * (l - 1) * N * 8,
                    "h2d_gbs": h2d_gbs, "d2h_gbs": d2h_gbs,
                    "copy_bound_ops_per_s": 1.0 / max(2 * 2 * l * N * 8 / (h2d_gbs * 1e9),
                                                       2 * (l - 1) * N * 8 / (d2h_gbs * 1e9))},
            "gpu_launches": int(launches),
            "roofline": {"kernel": f"ntt forward (column + row pass), 64 polys x 35 limbs, N=2^16, split "
                                   f"{ntt_shape[0]}+{16 - ntt_shape[0]}, {ntt_shape[1]}-coefficient tiles",
                         "bound": "hbm", "achieved": ntt_gbs, "peak": peak, "unit": "GB/s",
                         "frac": ntt_gbs / peak, "peak_source": peak_kind,
                         "algorithmic_bytes": ntt_bytes, "traffic": traffic, "issue": issue},
            "extra": {"ntt_n12_3x60_roundtrip_us": 1e6 * t12,
                      "ntt_n12_3x60_roundtrip_graph_us": 1e6 * t12g,
                      "bfv_n15_mult_relin_graph128_ops_per_s": 128 * world / t_graph,
                      "bfv_n15_mult_relin_loop128_ops_per_s": 128 * world / t_bloop,
                      "bfv_n15_mult_relin_loop128_cuda_core_ops_per_s": 128 * world / t_bloop_cc,
                      "bfv_n15_tuning": btuning,
                      "batch64_uneven_levels_ops_per_s": 64 * world / min(t_batch.values()),
                      "batch64_uneven_levels_fused_ops_per_s": 64 * world / t_batch[True],
                      "batch64_uneven_levels_unfused_ops_per_s": 64 * world / t_batch[False],
                      "batch64_as_single_calls_ops_per_s": 64 * world / t_loop,
                      "batch64_algorithmic_bytes": batch_bytes,
                      "batch64_hbm_frac": batch_bytes / min(t_batch.values()) / 1e9 / measured_peaks()[0],
                      "keyswitch_batch64_uneven_levels_per_s": 64 * world / min(t_ksb.values()),
                      "keyswitch_batch64_uneven_levels_fused_per_s": 64 * world / t_ksb[True],
                      "keyswitch_batch64_uneven_levels_unfused_per_s": 64 * world / t_ksb[False],
                      "keyswitch_batch64_as_single_calls_per_s": 64 * world / t_ksl,
                      "hrotate_step1_per_s": k2 * world / t_rot, "keyswitch_per_s": k2 * world / t_ks,
                      "tensor_core_bconv": tc_default, "tensor_core_status": tc_status,
                      "hmult_relin_rescale_cuda_core_bconv_ops_per_s": k2 * world / t_hm_cc,
                      "keyswitch_cuda_core_bconv_per_s": k2 * world / t_ks_cc,
                      "hmult_relin_rescale_unfused_modup_ops_per_s": k2 * world / t_hm_unfused,
                      "keyswitch_unfused_modup_per_s": k2 * world / t_ks_unfused,
                      "hmult_relin_rescale_fused_modup_ops_per_s": k2 * world / t_hm_fused,
                      "keyswitch_fused_modup_per_s": k2 * world / t_ks_fused,
                      "ntt_forward_ms_64x35": 1000 * t_ntt,
                      "ntt_forward_ms_64x35_by_split_and_tile": {f"{k[0]}+{16 - k[0]}/{k[1]}": 1000 * v
                                                                 for k, v in ntt_times.items()},
                      "hmult_relin_rescale_algorithmic_bytes": 313524224,
                      "hmult_hbm_frac": 313524224 * value / world / 1e9 / peak,
                      "launches_per_step": launches / args.steps, **mv}}
    if rank == 0 and world == 1:
        v, reps, dt = cpu_baseline_sample(mods, nq, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": "ops/s", "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"{reps} full HMult+relin+rescale ops at N=2^16, l=30 in {dt:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--case", choices=["full", "hmult", "ntt", "bfv", "matvec", "batch"], default="full",
                    help="hmult / ntt: run only that part (for profiler captures), print nothing")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
