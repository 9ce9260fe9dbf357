// autotune.cu — fhe_context_autotune_op: chooses the context's kernel shapes by timing its own
// workload, and keeps the choice in a cache file.
//
// The knobs (every setting gives the same words): the NTT stage split l1, the tile of the
// 16-per-thread NTT passes (2048 / 4096 coefficients), the tile of the 8-per-thread passes (1024 /
// 2048), the small-launch bound that picks between them, the fused mod-up row pass + inner
// product, and the tensor-core base conversions.  The workload timed is the operation the
// benchmarks run at the context's top level, batch 1: CKKS HMult + relinearise + rescale, BFV
// HPS multiply + relinearise.  Inputs and the key are uniform residues (the timing does not depend
// on the words).  Search: coordinate descent from the current settings, two sweeps over the knobs
// in order, each candidate timed as the best of five bursts of five operations after two warm-up
// operations, a candidate kept only when it is at least 0.5 % faster.
//
// Cache: one JSON object per line, {"key": "<GPU>|<scheme>|N=..|Q=..|P=..|batch=1", knobs...,
// "us": ...}; a line whose key matches is applied without timing.  No counterpart in the
// reference, whose shapes are fixed constants (include/common.h, include/ntt.cuh:131-153).
#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <functional>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "capi_internal.hpp"
#include "ops.hpp"

namespace {

void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("autotune: ") + what + ": " + cudaGetErrorString(e));
}

// Device allocations, stream and events released on every exit path.
struct Scratch {
    std::vector<void *> bufs;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Scratch() {
        if (s) cudaStreamSynchronize(s);
        for (void *p : bufs) cudaFree(p);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (s) cudaStreamDestroy(s);
    }
    uint64_t *alloc(size_t words) {
        void *p = nullptr;
        ck(cudaMalloc(&p, words * 8), "cudaMalloc");
        bufs.push_back(p);
        return static_cast<uint64_t *>(p);
    }
};

// Uniform residues of the layout [polys][limbs][N] (limb k mod mods[k]), from a fixed seed.
__global__ void fill_residues(uint64_t *p, const pfg::Mod *mods, int limbs, int log_n, size_t total) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        uint64_t x = (i + 1) * 0x9E3779B97F4A7C15ull;  // splitmix64
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        p[i] = x % mods[(i >> log_n) % limbs].q;
    }
}

pfg::Tuning current(const pfg::Context &c) {
    pfg::Tuning t{};
    t.ntt_split = c.l1();
    t.ntt_tile = c.ntt_tile;
    t.ntt_small_tile = c.ntt_small_tile;
    t.ntt_small_launch = (int)c.ntt_small_limit();
    t.fused_keyswitch = c.ks_fused ? 1 : 0;
    t.tensor_cores = c.tc_on ? 1 : 0;
    return t;
}

void apply(pfg::Context &c, const pfg::Tuning &t) {
    if (t.ntt_small_launch < -1) throw std::invalid_argument("autotune: small-launch bound must be >= -1");
    if (!c.split_ok(t.ntt_split)) throw std::invalid_argument("autotune: unsupported NTT split");
    if (t.ntt_tile != pfg::kTileElems && t.ntt_tile != pfg::kTileElems / 2)
        throw std::invalid_argument("autotune: NTT tile must be 2048 or 4096");
    if (t.ntt_small_tile != pfg::kTileElems / 2 && t.ntt_small_tile != pfg::kTileElems / 4)
        throw std::invalid_argument("autotune: small NTT tile must be 1024 or 2048");
    c.l1_sel = t.ntt_split;
    c.ntt_tile = t.ntt_tile;
    c.ntt_small_tile = t.ntt_small_tile;
    c.ntt_small_tiles = t.ntt_small_launch < 0 ? -1 : t.ntt_small_launch;
    c.ks_fused = t.fused_keyswitch != 0;
    c.tc_on = c.tc_avail && t.tensor_cores != 0;
}

std::string cache_key(const pfg::Context &c) {
    cudaDeviceProp p{};
    ck(cudaGetDeviceProperties(&p, c.device), "cudaGetDeviceProperties");
    std::ostringstream k;
    k << p.name << "|" << (c.scheme == pfg::kSchemeBFV ? "bfv" : "ckks") << "|N=" << c.n << "|Q=" << c.nQ
      << "|P=" << c.nP << "|batch=1";
    return k.str();
}

std::string to_line(const std::string &key, const pfg::Tuning &t) {
    char buf[512];
    std::snprintf(buf, sizeof buf,
                  "{\"key\": \"%s\", \"ntt_split\": %d, \"ntt_tile\": %d, \"ntt_small_tile\": %d, "
                  "\"ntt_small_launch\": %d, \"fused_keyswitch\": %d, \"tensor_cores\": %d, \"us\": %.3f}",
                  key.c_str(), t.ntt_split, t.ntt_tile, t.ntt_small_tile, t.ntt_small_launch, t.fused_keyswitch,
                  t.tensor_cores, (double)t.best_us);
    return buf;
}

bool field(const std::string &line, const char *name, double &v) {
    const std::string pat = std::string("\"") + name + "\": ";
    const size_t i = line.find(pat);
    if (i == std::string::npos) return false;
    return std::sscanf(line.c_str() + i + pat.size(), "%lf", &v) == 1;
}

bool from_line(const std::string &line, const std::string &key, pfg::Tuning &t) {
    if (line.find("\"key\": \"" + key + "\"") == std::string::npos) return false;
    double v[7];
    const char *names[7] = {"ntt_split", "ntt_tile", "ntt_small_tile", "ntt_small_launch", "fused_keyswitch",
                            "tensor_cores", "us"};
    for (int i = 0; i < 7; i++)
        if (!field(line, names[i], v[i])) return false;
    t.ntt_split = (int)v[0];
    t.ntt_tile = (int)v[1];
    t.ntt_small_tile = (int)v[2];
    t.ntt_small_launch = (int)v[3];
    t.fused_keyswitch = (int)v[4];
    t.tensor_cores = (int)v[5];
    t.best_us = (float)v[6];
    return true;
}

}  // namespace

namespace pfg {

Tuning autotune_op(Context &c, const Workspace &w, const char *cache_path) {
    const std::string key = cache_key(c);
    std::vector<std::string> lines;
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            if (line.empty()) continue;
            Tuning t{};
            if (from_line(line, key, t)) {
                apply(c, t);
                t.evaluated = 0;
                return t;
            }
            lines.push_back(line);
        }
    }
    if (c.nP == 0) throw std::logic_error("autotune: the timed operation needs special primes");
    if (c.scheme == kSchemeCKKS && c.nQ < 2) throw std::logic_error("autotune: HMult + rescale needs two data primes");
    const int l = c.nQ;
    const size_t n = c.n, qp = c.nQ + c.nP;
    const size_t ct_words = 2 * (size_t)l * n, key_words = (size_t)c.beta(l) * 2 * qp * n;
    Scratch sc;
    ck(cudaStreamCreateWithFlags(&sc.s, cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
    ck(cudaEventCreate(&sc.e0), "cudaEventCreate");
    ck(cudaEventCreate(&sc.e1), "cudaEventCreate");
    uint64_t *a = sc.alloc(ct_words), *b = sc.alloc(ct_words), *o = sc.alloc(ct_words), *k = sc.alloc(key_words);
    const int dnum = c.beta(l);
    std::vector<uint64_t *> kp(dnum);
    for (int d = 0; d < dnum; d++) kp[d] = k + (size_t)d * 2 * qp * n;
    uint64_t **dkp = reinterpret_cast<uint64_t **>(sc.alloc(dnum));
    ck(cudaMemcpyAsync(dkp, kp.data(), dnum * 8, cudaMemcpyHostToDevice, sc.s), "cudaMemcpyAsync");
    const Mod *mods = c.d_mods.as<Mod>();
    fill_residues<<<152 * 4, 256, 0, sc.s>>>(a, mods, l, c.log_n, ct_words);
    fill_residues<<<152 * 4, 256, 0, sc.s>>>(b, mods, l, c.log_n, ct_words);
    // key limbs follow the QP order of [dnum][2][QP][N]
    fill_residues<<<152 * 4, 256, 0, sc.s>>>(k, mods, (int)qp, c.log_n, key_words);
    ck(cudaGetLastError(), "fill launch");
    const uint64_t *const *rlk = dkp;
    std::function<void()> op;
    if (c.scheme == kSchemeBFV) {
        op = [&] {
            ck(cudaMemcpyAsync(o, a, ct_words * 8, cudaMemcpyDeviceToDevice, sc.s), "cudaMemcpyAsync");
            bfv_mul_relin_hps(c, w, o, b, rlk, sc.s);
        };
    } else {
        op = [&] { ckks_mul_relin_rescale(c, w, a, b, o, l, rlk, sc.s); };
    }
    auto time_us = [&]() {
        for (int i = 0; i < 2; i++) op();
        float best = 0.f;
        for (int trial = 0; trial < 5; trial++) {
            ck(cudaEventRecord(sc.e0, sc.s), "cudaEventRecord");
            for (int i = 0; i < 5; i++) op();
            ck(cudaEventRecord(sc.e1, sc.s), "cudaEventRecord");
            ck(cudaGetLastError(), "timed launches");
            ck(cudaEventSynchronize(sc.e1), "cudaEventSynchronize");
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, sc.e0, sc.e1), "cudaEventElapsedTime");
            const float us = 1000.f * ms / 5;
            if (trial == 0 || us < best) best = us;
        }
        return best;
    };
    const Tuning start = current(c);
    Tuning best = start;
    int evaluated = 0;
    try {
        apply(c, best);
        best.best_us = time_us();
        evaluated++;
        // candidate values per knob
        std::vector<std::function<std::vector<Tuning>(const Tuning &)>> knobs;
        knobs.push_back([&](const Tuning &t) {
            std::vector<Tuning> v;
            for (int l1 = 6; l1 <= 9; l1++)
                if (c.split_ok(l1) && l1 != t.ntt_split) v.push_back(t), v.back().ntt_split = l1;
            return v;
        });
        knobs.push_back([&](const Tuning &t) {
            Tuning u = t;
            u.ntt_tile = t.ntt_tile == kTileElems ? kTileElems / 2 : kTileElems;
            return std::vector<Tuning>{u};
        });
        knobs.push_back([&](const Tuning &t) {
            Tuning u = t;
            u.ntt_small_tile = t.ntt_small_tile == kTileElems / 2 ? kTileElems / 4 : kTileElems / 2;
            return std::vector<Tuning>{u};
        });
        knobs.push_back([&](const Tuning &t) {
            std::vector<Tuning> v;
            for (int b : {0, 256, 512, 1024, 2048, 4096})
                if (b != t.ntt_small_launch) v.push_back(t), v.back().ntt_small_launch = b;
            return v;
        });
        if (c.scheme == kSchemeCKKS)
            knobs.push_back([&](const Tuning &t) {
                Tuning u = t;
                u.fused_keyswitch = !t.fused_keyswitch;
                return std::vector<Tuning>{u};
            });
        if (c.tc_avail)
            knobs.push_back([&](const Tuning &t) {
                Tuning u = t;
                u.tensor_cores = !t.tensor_cores;
                return std::vector<Tuning>{u};
            });
        for (int sweep = 0; sweep < 2; sweep++)
            for (auto &kn : knobs)
                for (Tuning cand : kn(best)) {
                    apply(c, cand);
                    cand.best_us = time_us();
                    evaluated++;
                    if (cand.best_us < best.best_us * 0.995f) best = cand;
                }
    } catch (...) {
        apply(c, start);
        throw;
    }
    apply(c, best);
    best.evaluated = evaluated;
    if (cache_path) {
        lines.push_back(to_line(key, best));
        std::ofstream out(cache_path, std::ios::trunc);
        for (auto &ln : lines) out << ln << "\n";
        if (!out) throw std::runtime_error(std::string("autotune: cannot write the cache file ") + cache_path);
    }
    return best;
}

Tuning tuning_of(const Context &c) { return current(c); }

void apply_tuning(Context &c, const Tuning &t) { apply(c, t); }

}  // namespace pfg
