// capi.cu — the extern "C" boundary (include/phantom_gb300.h): argument checks with the
// reference's error classes, chain-index bookkeeping, and dispatch to the kernels.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>

#include "context.cuh"
#include "host_tables.hpp"
#include "capi_internal.hpp"
#include "ops.hpp"
#include "phantom_gb300.h"

namespace {

thread_local std::string g_last_error;

struct unsupported : std::runtime_error {
    using std::runtime_error::runtime_error;
};

pfg::Workspace ws_of(const fhe_context *ctx, fhe_workspace *ws) {
    if (!ws || !ws->base) throw std::invalid_argument("workspace is null");
    if (ws->ctx != ctx) throw std::invalid_argument("workspace belongs to another context");
    return pfg::Workspace{ws->base, ws->words};
}

void need_ptr(const void *p, const char *what) {
    if (!p) throw std::invalid_argument(std::string(what) + " is null");
}

void need_keyswitching(const pfg::Context &c) {
    if (c.nP == 0) throw std::logic_error("key switching needs special primes (special_modulus_size > 0)");
}

cudaStream_t st(void *s) { return static_cast<cudaStream_t>(s); }

}  // namespace

int pfg_fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

namespace pfg {
static std::atomic<unsigned long long> g_launches{0};
void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace pfg

extern "C" {

const char *fhe_last_error(void) { return g_last_error.c_str(); }

uint64_t fhe_kernel_launches(void) { return pfg::g_launches.load(std::memory_order_relaxed); }

int fhe_create_coeff_modulus(uint64_t poly_modulus_degree, const int *bit_sizes, size_t count, uint64_t *out) {
    return guarded([&] {
        need_ptr(bit_sizes, "bit_sizes");
        need_ptr(out, "out");
        if (poly_modulus_degree < 2 || (poly_modulus_degree & (poly_modulus_degree - 1)))
            throw std::invalid_argument("poly_modulus_degree is invalid");
        auto v = pfg::host::create_coeff_modulus(poly_modulus_degree, std::vector<int>(bit_sizes, bit_sizes + count));
        std::copy(v.begin(), v.end(), out);
    }, false);
}

uint32_t fhe_galois_elt_from_step(int step, uint64_t poly_modulus_degree) {
    try {
        return pfg::host::elt_from_step(step, poly_modulus_degree);
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return 0;
    }
}

int fhe_context_create(const fhe_params *p, fhe_context **out) {
    return guarded([&] {
        need_ptr(p, "params");
        need_ptr(out, "out");
        need_ptr(p->coeff_modulus, "coeff_modulus");
        std::vector<uint64_t> mods(p->coeff_modulus, p->coeff_modulus + p->coeff_modulus_size);
        std::vector<uint32_t> elts;
        if (p->galois_elts && p->galois_elts_size) elts.assign(p->galois_elts, p->galois_elts + p->galois_elts_size);
        auto c = pfg::make_context(p->scheme, p->mul_tech, p->poly_modulus_degree, mods,
                                   (int)p->special_modulus_size, p->plain_modulus, elts);
        *out = new fhe_context{std::move(c)};
    });
}

void fhe_context_destroy(fhe_context *ctx) { delete ctx; }

int fhe_context_sizes(const fhe_context *ctx, uint64_t *n, size_t *size_q, size_t *size_p, size_t *size_r,
                      size_t *dnum) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (n) *n = c.n;
        if (size_q) *size_q = c.nQ;
        if (size_p) *size_p = c.nP;
        if (size_r) *size_r = c.nR;
        if (dnum) *dnum = c.nP ? c.beta(c.nQ) : 0;
    }, false);
}

int fhe_context_set_tensor_cores(fhe_context *ctx, int enable) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        if (enable && !c.tc_avail)
            throw std::invalid_argument("tensor-core base conversion needs 1 <= special_modulus_size <= 6");
        c.tc_on = enable != 0;
    }, false);
}

int fhe_context_tensor_cores(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return ctx->c->tc_on ? 1 : 0;
}

int fhe_context_status(const fhe_context *ctx, unsigned *out) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(out, "out");
        unsigned v = 0;
        if (cudaMemcpy(&v, c.d_status.p, sizeof(v), cudaMemcpyDeviceToHost) != cudaSuccess)
            throw std::runtime_error("reading the device status word failed");
        const unsigned zero = 0;
        if (cudaMemcpy(c.d_status.p, &zero, sizeof(zero), cudaMemcpyHostToDevice) != cudaSuccess)
            throw std::runtime_error("clearing the device status word failed");
        *out = v;
    }, false);
}

int fhe_context_ntt_split(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return ctx->c->l1();
}

int fhe_context_set_ntt_split(fhe_context *ctx, int l1) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        if (!c.split_ok(l1)) throw std::invalid_argument("unsupported NTT stage split for this degree");
        c.l1_sel = l1;
    }, false);
}

int fhe_context_ntt_small_launch(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return (int)std::min<long long>(ctx->c->ntt_small_limit(), INT32_MAX);
}

int fhe_context_set_ntt_small_launch(fhe_context *ctx, int tiles) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        if (tiles < -1) throw std::invalid_argument("small-launch bound must be >= -1");
        c.ntt_small_tiles = tiles;
    }, false);
}

int fhe_context_ntt_small_tile(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return ctx->c->ntt_small_tile;
}

int fhe_context_set_ntt_small_tile(fhe_context *ctx, int coefficients) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        if (coefficients != pfg::kTileElems / 2 && coefficients != pfg::kTileElems / 4)
            throw std::invalid_argument("small-launch tile must be 1024 or 2048 coefficients");
        c.ntt_small_tile = coefficients;
    }, false);
}

int fhe_context_ntt_tile(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return ctx->c->ntt_tile;
}

int fhe_context_set_ntt_tile(fhe_context *ctx, int coefficients) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        if (coefficients != pfg::kTileElems && coefficients != pfg::kTileElems / 2)
            throw std::invalid_argument("NTT tile must be 2048 or 4096 coefficients");
        c.ntt_tile = coefficients;
    }, false);
}

int fhe_context_launch_overlap(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return ctx->c->pdl ? 1 : 0;
}

int fhe_context_set_launch_overlap(fhe_context *ctx, int enable) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        c.pdl = enable != 0;
    }, false);
}

int fhe_context_fused_keyswitch(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return ctx->c->ks_fused ? 1 : 0;
}

int fhe_context_set_fused_keyswitch(fhe_context *ctx, int enable) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        c.ks_fused = c.ks_fused_batch = enable != 0;
    }, false);
}

int fhe_context_autotune(fhe_context *ctx, int *chosen_l1, float *best_us) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        // the operations' regime: every QP limb, enough polynomials for >= 256 MB (beyond L2)
        const int limbs = c.nQ + c.nP;
        const size_t poly_bytes = (size_t)limbs * c.n * 8;
        const int polys = (int)std::min<size_t>(64, std::max<size_t>(1, ((size_t)256 << 20) / poly_bytes + 1));
        const size_t words = (size_t)polys * limbs * c.n;
        struct Guard {  // scratch, stream and events released on every exit path
            uint64_t *buf = nullptr;
            cudaStream_t s = nullptr;
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            ~Guard() {
                if (s) cudaStreamSynchronize(s);
                if (buf) cudaFree(buf);
                if (e0) cudaEventDestroy(e0);
                if (e1) cudaEventDestroy(e1);
                if (s) cudaStreamDestroy(s);
            }
        } g;
        auto ck = [](cudaError_t e, const char *what) {
            if (e != cudaSuccess) throw std::runtime_error(std::string("autotune: ") + what + ": " + cudaGetErrorString(e));
        };
        ck(cudaMalloc(&g.buf, words * 8), "cudaMalloc");
        ck(cudaStreamCreateWithFlags(&g.s, cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
        ck(cudaEventCreate(&g.e0), "cudaEventCreate");
        ck(cudaEventCreate(&g.e1), "cudaEventCreate");
        ck(cudaMemsetAsync(g.buf, 0, words * 8, g.s), "cudaMemsetAsync");
        const int keep = c.l1_sel;
        int best = 0;
        float best_t = 0.f;
        try {
            for (int l1 = 6; l1 <= 8; l1++) {
                if (!c.split_ok(l1)) continue;
                c.l1_sel = l1;
                for (int i = 0; i < 2; i++) {
                    pfg::ntt_forward(c, g.buf, polys, limbs, 0, g.s);
                    pfg::ntt_inverse(c, g.buf, polys, limbs, 0, g.s);
                }
                const int reps = 3;
                float us = 0.f;
                for (int trial = 0; trial < 3; trial++) {  // best of three
                    ck(cudaEventRecord(g.e0, g.s), "cudaEventRecord");
                    for (int i = 0; i < reps; i++) {
                        pfg::ntt_forward(c, g.buf, polys, limbs, 0, g.s);
                        pfg::ntt_inverse(c, g.buf, polys, limbs, 0, g.s);
                    }
                    ck(cudaEventRecord(g.e1, g.s), "cudaEventRecord");
                    ck(cudaGetLastError(), "timed launches");
                    ck(cudaEventSynchronize(g.e1), "cudaEventSynchronize");
                    float ms = 0.f;
                    ck(cudaEventElapsedTime(&ms, g.e0, g.e1), "cudaEventElapsedTime");
                    const float t = 1000.f * ms / reps;
                    if (trial == 0 || t < us) us = t;
                }
                if (!best || us < best_t) {
                    best = l1;
                    best_t = us;
                }
            }
        } catch (...) {
            c.l1_sel = keep;
            throw;
        }
        c.l1_sel = best ? best : keep;
        if (chosen_l1) *chosen_l1 = c.l1();
        if (best_us) *best_us = best_t;
    });
}

int fhe_context_autotune_op(fhe_context *ctx, fhe_workspace *ws, const char *cache_path, fhe_tuning *out) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        const fhe_tuning t = pfg::autotune_op(c, w, cache_path);
        if (out) *out = t;
    });
}

int fhe_context_tuning(const fhe_context *ctx, fhe_tuning *out) {
    return guarded([&] {
        need_ptr(out, "out");
        *out = pfg::tuning_of(ctx_of(ctx));
    }, false);
}

int fhe_context_set_tuning(fhe_context *ctx, const fhe_tuning *t) {
    return guarded([&] {
        need_ptr(t, "tuning");
        pfg::apply_tuning(*const_cast<pfg::Context *>(&ctx_of(ctx)), *t);
    }, false);
}

int fhe_context_moduli(const fhe_context *ctx, uint64_t *out) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(out, "out");
        std::copy(c.mods.begin(), c.mods.end(), out);
    }, false);
}

int fhe_context_galois_elts(const fhe_context *ctx, uint32_t *out, size_t *count) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(count, "count");
        if (out) std::copy(c.galois_elts.begin(), c.galois_elts.end(), out);
        *count = c.galois_elts.size();
    }, false);
}

size_t fhe_workspace_bytes(const fhe_context *ctx) {
    if (!ctx || !ctx->c) return 0;
    return pfg::workspace_words(*ctx->c) * sizeof(uint64_t);
}

int fhe_workspace_create(const fhe_context *ctx, fhe_workspace **out) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(out, "out");
        auto *w = new fhe_workspace;
        w->ctx = ctx;
        w->words = pfg::workspace_words(c);
        cudaError_t e = cudaMalloc(&w->base, w->words * sizeof(uint64_t));
        if (e != cudaSuccess) {
            delete w;
            cudaGetLastError();
            throw std::bad_alloc();
        }
        *out = w;
    });
}

int fhe_workspace_create_batch(const fhe_context *ctx, size_t max_items, fhe_workspace **out) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(out, "out");
        if (max_items == 0) throw std::invalid_argument("max_items must be positive");
        const size_t slots = std::min<size_t>(max_items, pfg::kBatchLaunch);
        auto *w = new fhe_workspace;
        w->ctx = ctx;
        w->items = slots;
        w->words = pfg::workspace_words(c) * slots;
        cudaError_t e = cudaMalloc(&w->base, w->words * sizeof(uint64_t));
        if (e != cudaSuccess) {
            delete w;
            cudaGetLastError();
            throw std::bad_alloc();
        }
        *out = w;
    });
}

void fhe_workspace_destroy(fhe_workspace *ws) {
    if (!ws) return;
    if (ws->base) cudaFree(ws->base);
    delete ws;
}

static int ntt_common(const fhe_context *ctx, uint64_t *data, size_t num_polys, size_t size, size_t start,
                      void *stream, bool fwd) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(data, "data");
        if (size == 0 || num_polys == 0) return;
        if (start + size > c.mods.size()) throw std::invalid_argument("modulus index out of range");
        if (num_polys * size > 65535) throw std::invalid_argument("too many limbs in one call");
        if (fwd)
            pfg::ntt_forward(c, data, (int)num_polys, (int)size, (int)start, st(stream));
        else
            pfg::ntt_inverse(c, data, (int)num_polys, (int)size, (int)start, st(stream));
    });
}

int fhe_ntt_forward(const fhe_context *ctx, uint64_t *data, size_t num_polys, size_t coeff_modulus_size,
                    size_t start_modulus_idx, void *stream) {
    return ntt_common(ctx, data, num_polys, coeff_modulus_size, start_modulus_idx, stream, true);
}

int fhe_ntt_inverse(const fhe_context *ctx, uint64_t *data, size_t num_polys, size_t coeff_modulus_size,
                    size_t start_modulus_idx, void *stream) {
    return ntt_common(ctx, data, num_polys, coeff_modulus_size, start_modulus_idx, stream, false);
}

int fhe_ckks_multiply(const fhe_context *ctx, uint64_t *ct1, const uint64_t *ct2, size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("fhe_ckks_multiply needs a CKKS context");
        need_ptr(ct1, "ct1");
        need_ptr(ct2, "ct2");
        pfg::ckks_tensor(c, ct1, ct2, level_of(c, chain_index), st(stream));
    });
}

int fhe_keyswitch(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, const uint64_t *c2, size_t chain_index,
                  const uint64_t *const *evk, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        need_keyswitching(c);
        need_ptr(ct, "ct");
        need_ptr(c2, "c2");
        need_ptr(evk, "evk");
        const int l = level_of(c, chain_index);
        if (c.scheme == pfg::kSchemeBFV) {
            if (chain_index != 1) throw std::invalid_argument("BFV key switching works at chain index 1");
            pfg::bfv_keyswitch(c, w, ct, c2, l, evk, st(stream));
        } else {
            pfg::ckks_keyswitch(c, w, ct, c2, l, evk, st(stream));
        }
    });
}

int fhe_relinearize(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index,
                    const uint64_t *const *rlk, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        const int l = level_of(c, chain_index);
        need_ptr(ct, "ct");
        const uint64_t *c2 = ct + ((size_t)2 * l << c.log_n);
        int rc = fhe_keyswitch(ctx, ws, ct, c2, chain_index, rlk, stream);
        if (rc != FHE_OK) throw std::invalid_argument(g_last_error);
    });
}

int fhe_multiply_and_relin(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct1, const uint64_t *ct2,
                           size_t chain_index, const uint64_t *const *rlk, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        need_keyswitching(c);
        need_ptr(ct1, "ct1");
        need_ptr(ct2, "ct2");
        need_ptr(rlk, "rlk");
        const int l = level_of(c, chain_index);
        if (c.scheme == pfg::kSchemeBFV) {
            if (chain_index != 1) throw std::invalid_argument("BFV HPS multiplication works at chain index 1");
            pfg::bfv_mul_relin_hps(c, w, ct1, ct2, rlk, st(stream));
        } else {
            pfg::ckks_mul_relin(c, w, ct1, ct2, l, rlk, st(stream));
        }
    });
}

int fhe_rescale_to_next(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *in, uint64_t *out, size_t size,
                        size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("unsupported scheme");
        need_ptr(in, "in");
        need_ptr(out, "out");
        const int l = level_of(c, chain_index);
        if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
        if (size == 0 || size > (size_t)c.nQ) throw std::invalid_argument("bad ciphertext size");
        pfg::ckks_rescale(c, w, in, out, (int)size, l, st(stream));
    });
}

int fhe_bfv_mod_switch_to_next(const fhe_context *ctx, const uint64_t *in, uint64_t *out, size_t size,
                               size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeBFV) throw std::invalid_argument("fhe_bfv_mod_switch_to_next needs BFV");
        need_ptr(in, "in");
        need_ptr(out, "out");
        const int l = level_of(c, chain_index);
        if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
        pfg::bfv_divide_round_q_last(c, in, out, (int)size, l, st(stream));
    });
}

int fhe_ckks_multiply_relin_rescale(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *ct1,
                                    const uint64_t *ct2, uint64_t *out, size_t chain_index,
                                    const uint64_t *const *rlk, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("fhe_ckks_multiply_relin_rescale needs CKKS");
        need_keyswitching(c);
        need_ptr(ct1, "ct1");
        need_ptr(ct2, "ct2");
        need_ptr(out, "out");
        need_ptr(rlk, "rlk");
        const int l = level_of(c, chain_index);
        if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
        pfg::ckks_mul_relin_rescale(c, w, ct1, ct2, out, l, rlk, st(stream));
    });
}

int fhe_ckks_multiply_relin_rescale_batch(const fhe_context *ctx, fhe_workspace *ws, const fhe_ckks_mul_item *items,
                                          size_t count, const uint64_t *const *rlk, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("batched HMult needs a CKKS context");
        need_keyswitching(c);
        need_ptr(items, "items");
        need_ptr(rlk, "rlk");
        if (count == 0) return;
        if (ws->items < std::min<size_t>(count, pfg::kBatchLaunch))
            throw std::invalid_argument("workspace has too few ciphertext slots for this batch");
        std::vector<pfg::BatchItem> v;
        for (size_t i = 0; i < count; i++) {
            need_ptr(items[i].ct1, "items[i].ct1");
            need_ptr(items[i].ct2, "items[i].ct2");
            need_ptr(items[i].out, "items[i].out");
            const int l = level_of(c, items[i].chain_index);
            if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
            v.push_back(pfg::BatchItem{items[i].ct1, items[i].ct2, items[i].out, l});
        }
        pfg::ckks_mul_relin_rescale_batch(c, w.base, ws->words / ws->items, v, rlk, st(stream));
    });
}

int fhe_keyswitch_batch(const fhe_context *ctx, fhe_workspace *ws, const fhe_ks_item *items, size_t count,
                        const uint64_t *const *evk, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("batched key switching needs a CKKS context");
        need_keyswitching(c);
        need_ptr(items, "items");
        need_ptr(evk, "evk");
        if (count == 0) return;
        if (ws->items < std::min<size_t>(count, pfg::kBatchLaunch))
            throw std::invalid_argument("workspace has too few ciphertext slots for this batch");
        std::vector<pfg::KsItem> v;
        for (size_t i = 0; i < count; i++) {
            need_ptr(items[i].ct, "items[i].ct");
            need_ptr(items[i].c2, "items[i].c2");
            v.push_back(pfg::KsItem{items[i].ct, items[i].c2, level_of(c, items[i].chain_index)});
        }
        pfg::ckks_keyswitch_batch(c, w.base, ws->words / ws->items, v, evk, st(stream));
    });
}

int galois_index(const pfg::Context &c, uint32_t elt) {
    auto it = std::find(c.galois_elts.begin(), c.galois_elts.end(), elt);
    return it == c.galois_elts.end() ? -1 : (int)(it - c.galois_elts.begin());
}

int fhe_apply_galois(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index, uint32_t galois_elt,
                     const uint64_t *const *gk, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("Galois automorphisms are implemented for CKKS");
        need_keyswitching(c);
        need_ptr(ct, "ct");
        need_ptr(gk, "gk");
        if (galois_index(c, galois_elt) < 0) throw std::invalid_argument("Galois elt not present");
        pfg::ckks_apply_galois(c, w, ct, level_of(c, chain_index), c.perm_table(galois_elt), gk, st(stream));
    });
}

int fhe_rotate(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index, int step,
               const uint64_t *const *const *galois_keys, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("Galois automorphisms are implemented for CKKS");
        need_keyswitching(c);
        need_ptr(ct, "ct");
        need_ptr(galois_keys, "galois_keys");
        pfg::ckks_rotate(c, w, ct, level_of(c, chain_index), step, galois_keys, st(stream));
    });
}

int fhe_ckks_rotations_hoisted(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *ct, size_t chain_index,
                               const int *steps, size_t num_steps, const uint64_t *const *const *galois_keys,
                               uint64_t *const *outs, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("rotations are implemented for CKKS");
        need_keyswitching(c);
        need_ptr(ct, "ct");
        need_ptr(steps, "steps");
        need_ptr(galois_keys, "galois_keys");
        need_ptr(outs, "outs");
        std::vector<pfg::StepKey> sk;
        std::vector<uint64_t *> o;
        for (size_t i = 0; i < num_steps; i++) {
            const uint32_t elt = pfg::host::elt_from_step(steps[i], c.n);
            const int idx = galois_index(c, elt);
            if (idx < 0 || !galois_keys[idx]) throw std::logic_error("Galois key not present in hoisting");
            need_ptr(outs[i], "outs[i]");
            sk.push_back(pfg::StepKey{c.perm_table(elt), galois_keys[idx]});
            o.push_back(outs[i]);
        }
        if (!sk.empty()) pfg::ckks_rotations_hoisted(c, w, ct, level_of(c, chain_index), sk, o, st(stream));
    });
}

int fhe_ckks_multiply_plain(const fhe_context *ctx, const uint64_t *ct, const uint64_t *pt, uint64_t *out,
                            size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("multiply_plain: CKKS only");
        need_ptr(ct, "ct");
        need_ptr(pt, "pt");
        need_ptr(out, "out");
        pfg::ckks_multiply_plain(c, ct, pt, out, level_of(c, chain_index), st(stream));
    });
}

int fhe_ckks_add(const fhe_context *ctx, const uint64_t *a, const uint64_t *b, uint64_t *out, size_t size,
                 size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(a, "a");
        need_ptr(b, "b");
        need_ptr(out, "out");
        if (size == 0 || size > 3) throw std::invalid_argument("bad ciphertext size");
        pfg::ckks_add(c, a, b, out, level_of(c, chain_index), (int)size, st(stream));
    });
}

size_t fhe_bsgs_scratch_bytes(const fhe_context *ctx, size_t G) {
    if (!ctx || !ctx->c || G == 0) return 0;
    return pfg::bsgs_scratch_words(*ctx->c, (int)G) * sizeof(uint64_t);
}

size_t fhe_bsgs_batch_scratch_bytes(const fhe_context *ctx, size_t G, size_t B) {
    if (!ctx || !ctx->c || G == 0 || B == 0 || G > 256) return 0;
    return pfg::bsgs_batch_scratch_words(*ctx->c, (int)G, (int)B) * sizeof(uint64_t);
}

int fhe_ckks_bsgs_matvec(const fhe_context *ctx, fhe_workspace *ws, uint64_t *scratch, const uint64_t *ct,
                         size_t chain_index, const uint64_t *diags, size_t D, size_t G, size_t B,
                         const uint64_t *const *const *galois_keys, uint64_t *out, int hoisted, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("matrix-vector product: CKKS only");
        need_keyswitching(c);
        need_ptr(scratch, "scratch");
        need_ptr(ct, "ct");
        need_ptr(diags, "diags");
        need_ptr(galois_keys, "galois_keys");
        need_ptr(out, "out");
        if (D == 0 || G == 0 || B == 0 || G * B < D) throw std::invalid_argument("need D > 0 and G * B >= D");
        if (G > 256) throw std::invalid_argument("too many baby steps");
        const int l = level_of(c, chain_index);
        if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
        pfg::ckks_bsgs_matvec(c, w, scratch, ct, l, diags, (int)D, (int)G, (int)B, galois_keys, out, hoisted != 0,
                              st(stream));
    });
}

int fhe_ckks_bsgs_matvec_batch(const fhe_context *ctx, fhe_workspace *ws, uint64_t *scratch,
                               const fhe_matvec_item *items, size_t count, size_t D, size_t G, size_t B,
                               const uint64_t *const *const *galois_keys, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("matrix-vector product: CKKS only");
        need_keyswitching(c);
        need_ptr(scratch, "scratch");
        need_ptr(items, "items");
        need_ptr(galois_keys, "galois_keys");
        if (D == 0 || G == 0 || B == 0 || G * B < D) throw std::invalid_argument("need D > 0 and G * B >= D");
        if (G > 256) throw std::invalid_argument("too many baby steps");
        if (count == 0) return;
        if (ws->items < std::min<size_t>(count, pfg::kBatchLaunch))
            throw std::invalid_argument("workspace has too few ciphertext slots for this batch");
        std::vector<pfg::MatvecItem> v;
        for (size_t i = 0; i < count; i++) {
            need_ptr(items[i].ct, "items[i].ct");
            need_ptr(items[i].diags, "items[i].diags");
            need_ptr(items[i].out, "items[i].out");
            const int l = level_of(c, items[i].chain_index);
            if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
            const size_t dl = items[i].diag_limbs ? items[i].diag_limbs : (size_t)l;
            if (dl < (size_t)l || dl > (size_t)c.nQ)
                throw std::invalid_argument("items[i].diag_limbs must lie between the item's limbs and the data primes");
            v.push_back(pfg::MatvecItem{items[i].ct, items[i].diags, items[i].out, l, (int)dl});
        }
        pfg::ckks_bsgs_matvec_batch(c, w.base, ws->words / ws->items, scratch,
                                    pfg::bsgs_batch_scratch_words(c, (int)G, (int)B), v,
                                    (int)D, (int)G, (int)B, galois_keys, st(stream));
    });
}

int fhe_ckks_encrypt_symmetric(const fhe_context *ctx, const uint64_t *pt, const uint64_t *s_ntt, const uint64_t *a,
                               const int64_t *e, uint64_t *out, size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(s_ntt, "s");
        need_ptr(a, "a");
        need_ptr(e, "e");
        need_ptr(out, "out");
        pfg::ckks_encrypt_sk(c, pt, s_ntt, a, e, out, level_of(c, chain_index), st(stream));
    });
}

int fhe_ckks_encode(const fhe_context *ctx, fhe_workspace *ws, const double *values, size_t count, double scale,
                    size_t chain_index, uint64_t *pt, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("unsupported scheme");
        pfg::Workspace w = ws_of(ctx, ws);
        need_ptr(values, "values");
        need_ptr(pt, "pt");
        pfg::ckks_encode(c, w, values, count, scale, level_of(c, chain_index), pt, st(stream));
    });
}

int fhe_ckks_decode(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *pt, size_t chain_index, double scale,
                    double *values, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("unsupported scheme");
        pfg::Workspace w = ws_of(ctx, ws);
        need_ptr(pt, "pt");
        need_ptr(values, "values");
        pfg::ckks_decode(c, w, pt, scale, level_of(c, chain_index), values, st(stream));
    });
}

int fhe_ckks_decrypt(const fhe_context *ctx, const uint64_t *ct, const uint64_t *s_ntt, uint64_t *pt,
                     size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(ct, "ct");
        need_ptr(s_ntt, "s");
        need_ptr(pt, "pt");
        pfg::ckks_decrypt(c, ct, s_ntt, pt, level_of(c, chain_index), st(stream));
    });
}

int fhe_kswitch_keygen(const fhe_context *ctx, fhe_workspace *ws, uint32_t galois_elt, const uint64_t *s_ntt,
                       const uint64_t *a, const int64_t *e, uint64_t *key, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        need_keyswitching(c);
        need_ptr(s_ntt, "s");
        need_ptr(a, "a");
        need_ptr(e, "e");
        need_ptr(key, "key");
        if (galois_elt && galois_index(c, galois_elt) < 0) throw std::invalid_argument("Galois elt not present");
        const size_t need = (size_t)(c.beta(c.nQ) + 1) * (c.nQ + c.nP) * c.n + 64;
        if (w.words < need) throw std::logic_error("workspace too small for key generation");
        pfg::kswitch_keygen(c, galois_elt, s_ntt, a, (size_t)(c.nQ + c.nP) * c.n, e, key, w.base, st(stream));
    });
}

int fhe_bfv_encode(const fhe_context *ctx, const uint64_t *values, size_t count, uint64_t *pt, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(pt, "pt");
        if (count && !values) throw std::invalid_argument("values is null");
        if (count > c.n) throw std::logic_error("values_matrix size is too large");
        pfg::bfv_encode(c, values, count, pt, st(stream));
    });
}

int fhe_bfv_decode(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *pt, uint64_t *values, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        need_ptr(pt, "pt");
        need_ptr(values, "values");
        if (w.words < c.n) throw std::logic_error("workspace too small");
        pfg::bfv_decode(c, pt, values, w.base, st(stream));
    });
}

int fhe_bfv_encrypt_symmetric(const fhe_context *ctx, const uint64_t *pt, const uint64_t *s_ntt, const uint64_t *a,
                              const int64_t *e, uint64_t *out, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeBFV) throw std::invalid_argument("BFV context required");
        need_ptr(pt, "pt");
        need_ptr(s_ntt, "s_ntt");
        need_ptr(a, "a");
        need_ptr(e, "e");
        need_ptr(out, "out");
        pfg::bfv_encrypt_sk(c, pt, s_ntt, a, e, out, st(stream));
    });
}

int fhe_bfv_decrypt(const fhe_context *ctx, fhe_workspace *ws, const uint64_t *ct, size_t chain_index,
                    const uint64_t *s_ntt, uint64_t *pt, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeBFV) throw std::invalid_argument("BFV context required");
        need_ptr(ct, "ct");
        need_ptr(s_ntt, "s_ntt");
        need_ptr(pt, "pt");
        const int l = level_of(c, chain_index);
        if (w.words < ((size_t)l << c.log_n)) throw std::logic_error("workspace too small");
        pfg::bfv_decrypt(c, ct, l, s_ntt, pt, w.base, st(stream));
    });
}

int fhe_sample_uniform(const fhe_context *ctx, const uint8_t *seed, size_t limbs, uint64_t *out, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        need_ptr(seed, "seed");
        need_ptr(out, "out");
        if (limbs < 1 || limbs > (size_t)(c.nQ + c.nP)) throw std::invalid_argument("limbs out of range");
        pfg::sample_uniform(c, seed, (int)limbs, out, st(stream));
    });
}

int fhe_sample_ternary(const fhe_context *ctx, const uint8_t *seed, int64_t *out, void *stream) {
    return guarded([&] {
        need_ptr(seed, "seed");
        need_ptr(out, "out");
        pfg::sample_small(ctx_of(ctx), seed, 0, out, st(stream));
    });
}

int fhe_sample_cbd(const fhe_context *ctx, const uint8_t *seed, int64_t *out, void *stream) {
    return guarded([&] {
        need_ptr(seed, "seed");
        need_ptr(out, "out");
        pfg::sample_small(ctx_of(ctx), seed, 1, out, st(stream));
    });
}

int fhe_secret_key_from_seed(const fhe_context *ctx, fhe_workspace *ws, const uint8_t *seed, uint64_t *s_ntt,
                             void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        pfg::Workspace w = ws_of(ctx, ws);
        need_ptr(seed, "seed");
        need_ptr(s_ntt, "s_ntt");
        if (w.words < (size_t)c.n) throw std::logic_error("workspace too small for key generation");
        pfg::secret_key_from_seed(c, seed, s_ntt, reinterpret_cast<int64_t *>(w.base), st(stream));
    });
}

int fhe_kswitch_keygen_seeded(const fhe_context *ctx, fhe_workspace *ws, uint32_t galois_elt, const uint64_t *s_ntt,
                              const uint8_t *seeds_a, const uint8_t *seeds_e, uint64_t *key, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        need_keyswitching(c);
        need_ptr(s_ntt, "s");
        need_ptr(seeds_a, "seeds_a");
        need_ptr(seeds_e, "seeds_e");
        need_ptr(key, "key");
        if (galois_elt && galois_index(c, galois_elt) < 0) throw std::invalid_argument("Galois elt not present");
        const int dnum = c.beta(c.nQ);
        const size_t need = (size_t)(dnum + 1) * (c.nQ + c.nP) * c.n + 64 + (size_t)dnum * c.n;
        if (w.words < need) throw std::logic_error("workspace too small for key generation");
        pfg::kswitch_keygen_seeded(c, galois_elt, s_ntt, seeds_a, seeds_e, key, w.base, st(stream));
    });
}

int fhe_hoisting(const fhe_context *ctx, fhe_workspace *ws, uint64_t *ct, size_t chain_index, const int *steps,
                 size_t num_steps, const uint64_t *const *const *galois_keys, void *stream) {
    return guarded([&] {
        pfg::Context &c = *const_cast<pfg::Context *>(&ctx_of(ctx));
        pfg::Workspace w = ws_of(ctx, ws);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("hoisting is implemented for CKKS");
        need_keyswitching(c);
        need_ptr(ct, "ct");
        need_ptr(steps, "steps");
        need_ptr(galois_keys, "galois_keys");
        if (num_steps == 0) throw std::invalid_argument("no rotation steps");
        std::vector<pfg::StepKey> sk;
        for (size_t i = 0; i < num_steps; i++) {
            const uint32_t elt = pfg::host::elt_from_step(steps[i], c.n);
            const int idx = galois_index(c, elt);
            if (idx < 0) throw std::logic_error("Galois key not present in hoisting");
            sk.push_back(pfg::StepKey{c.perm_table(elt), galois_keys[idx]});
        }
        pfg::ckks_hoisting(c, w, ct, level_of(c, chain_index), sk, st(stream));
    });
}

}  // extern "C"
