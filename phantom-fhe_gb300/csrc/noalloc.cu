// noalloc.cu — fhe_rescale_to_next_noalloc: the CKKS rescale with no device allocation at all.
//
// Who needs it: code that runs where the library may not call cudaMalloc — a serving process
// or database extension whose host owns every byte of device memory through its own
// allocator and hands the plugin only the input and output buffers, or a latency-critical
// path that must not risk an allocation failure or an implicit synchronisation.  Such a
// caller cannot create an fhe_workspace, so this entry point keeps its scratch in a
// file-scope __device__ array instead.
//
// The array (kScratchWords words = 2 MiB) is part of the module image: every GPU that loads
// the library holds it until the process exits.  It bounds size * N <= 2^18 words (for
// example two polynomials at N = 2^17, or three at N = 2^16).  All calls on a device share
// it: two calls whose kernels overlap on the GPU (different streams, or different host
// threads) race on it and must be ordered by the caller.  The rescale writes every scratch
// word before reading it, so nothing has to be cleared between calls.
#include <mutex>
#include <stdexcept>
#include <string>

#include "capi_internal.hpp"
#include "ops.hpp"

namespace {

constexpr size_t kScratchWords = size_t(1) << 18;
__device__ __align__(256) uint64_t g_rescale_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
uint64_t *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code the array's name
// is only a host-side stand-in, so its address is looked up once per device (with that
// device current) and cached; the first call on a device therefore does this set-up and
// should come before any stream capture.
uint64_t *scratch_on_current_device() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("device index out of range");
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_rescale_scratch);
        if (e != cudaSuccess) throw std::runtime_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<uint64_t *>(p);
    }
    return g_scratch_addr[dev];
}

}  // namespace

extern "C" int fhe_rescale_to_next_noalloc(const fhe_context *ctx, const uint64_t *in, uint64_t *out, size_t size,
                                           size_t chain_index, void *stream) {
    return guarded([&] {
        const pfg::Context &c = ctx_of(ctx);
        if (c.scheme != pfg::kSchemeCKKS) throw std::invalid_argument("unsupported scheme");
        if (!in || !out) throw std::invalid_argument("in / out is null");
        const int l = level_of(c, chain_index);
        if (l < 2) throw std::invalid_argument("end of modulus switching chain reached");
        if (size == 0 || size > (size_t)c.nQ) throw std::invalid_argument("bad ciphertext size");
        if (size * c.n > kScratchWords)
            throw std::invalid_argument("size * poly_modulus_degree = " + std::to_string(size * c.n) +
                                        " words exceeds the no-allocation scratch of " +
                                        std::to_string(kScratchWords) + " words; use fhe_rescale_to_next");
        const pfg::Workspace w{scratch_on_current_device(), kScratchWords};
        pfg::ckks_rescale(c, w, in, out, (int)size, l, static_cast<cudaStream_t>(stream));
    });
}
