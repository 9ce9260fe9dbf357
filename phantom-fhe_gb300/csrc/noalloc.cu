// noalloc.cu — fhe_rescale_to_next_noalloc: the CKKS rescale with no device allocation at all.
//
// Who needs it: code that runs where the library may not call cudaMalloc — a serving process
// or database extension whose host owns every byte of device memory through its own
// allocator and hands the plugin only the input and output buffers, or a latency-critical
// path that must not risk an allocation failure or an implicit synchronisation.  Such a
// caller cannot create an fhe_workspace, so this entry point keeps its scratch in a
// file-scope __device__ array instead.
//
// The array (kScratchWords words = 2 MiB) is part of this file's module image.  The driver
// commits it on a device when it loads the module there; with lazy module loading that happens
// on the module's first use on the device, which is the address lookup that fhe_context_create
// makes (below).  Every device that has done so holds the 2 MiB until the process exits.  It
// bounds size * N <= 2^18 words (for example two polynomials at N = 2^17, or three at
// N = 2^16).  All calls on a device share it: two calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on it and must be ordered by the
// caller.  The rescale writes every scratch word before reading it, so nothing has to be
// cleared between calls.
#include <stdexcept>
#include <string>

#include "capi_internal.hpp"
#include "ops.hpp"

namespace {

constexpr size_t kScratchWords = size_t(1) << 18;
__device__ __align__(256) uint64_t g_rescale_scratch[kScratchWords];

}  // namespace

namespace pfg {

// In host code the array's name is only a host-side stand-in, so its device address is looked
// up with the device current.  The context creation calls this once, and the address is kept in
// the context: it belongs to the CUDA context that the tables were built in and lives as long
// as they do (a device reset followed by a new fhe_context gets a fresh lookup).
uint64_t *noalloc_scratch_address(size_t *words) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_rescale_scratch);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *words = kScratchWords;
    return static_cast<uint64_t *>(p);
}

}  // namespace pfg

extern "C" int fhe_rescale_to_next_noalloc(const fhe_context *ctx, const uint64_t *in, uint64_t *out, size_t size,
                                           size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("unsupported scheme");
        if (!in || !out) throw std::invalid_argument("in / out is null");
        const int l = level_of(c, chain_index);
        if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
        if (size == 0 || size > (size_t)c.nQ) throw std::invalid_argument("bad ciphertext size");
        if (size * c.n > c.noalloc_words)
            throw std::invalid_argument("size * poly_modulus_degree = " + std::to_string(size * c.n) +
                                        " words exceeds the no-allocation scratch of " +
                                        std::to_string(c.noalloc_words) + " words; use fhe_rescale_to_next");
        int dev = -1;
        if (cudaGetDevice(&dev) != cudaSuccess || dev != c.device)
            throw std::invalid_argument("the current device is not the context's device");
        const pfg::Workspace w{c.noalloc_scratch, c.noalloc_words};
        pfg::ckks_rescale(c, w, in, out, (int)size, l, static_cast<cudaStream_t>(stream));
    });
}
