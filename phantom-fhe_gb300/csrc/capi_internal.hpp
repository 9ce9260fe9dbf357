// capi_internal.hpp — shared pieces of the C-ABI translation units: the opaque handle
// types, the status/exception translation and the chain-index helper.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <new>
#include <stdexcept>
#include <string>

#include "context.cuh"
#include "phantom_gb300.h"

struct fhe_context {
    std::unique_ptr<pfg::Context> c;
};

struct fhe_workspace {
    const fhe_context *ctx = nullptr;
    uint64_t *base = nullptr;
    size_t words = 0;      // total
    size_t items = 1;      // ciphertext slots for the batched calls (words / items each)
};

// Records `msg` as the calling thread's last error (fhe_last_error) and returns `code`.
int pfg_fail(int code, const std::string &msg);

// Runs `body`, translating the reference's exception classes into status codes; with
// `launches` it also checks that every kernel launch the body made was accepted.
template <class F>
int guarded(F &&body, bool launches = true) {
    try {
        body();
        if (launches) {
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return pfg_fail(FHE_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e));
        }
        return FHE_OK;
    } catch (const std::invalid_argument &e) {
        return pfg_fail(FHE_ERR_INVALID_ARGUMENT, e.what());
    } catch (const std::logic_error &e) {
        return pfg_fail(FHE_ERR_LOGIC, e.what());
    } catch (const std::bad_alloc &) {
        return pfg_fail(FHE_ERR_OUT_OF_MEMORY, "out of host memory");
    } catch (const std::runtime_error &e) {
        return pfg_fail(FHE_ERR_CUDA, e.what());
    } catch (...) {
        return pfg_fail(FHE_ERR_LOGIC, "unknown error");
    }
}

inline const pfg::Context &ctx_of(const fhe_context *ctx) {
    if (!ctx || !ctx->c) throw std::invalid_argument("context is null");
    return *ctx->c;
}

// chain index -> number of data limbs (src/context.cu:141-158)
inline int level_of(const pfg::Context &c, size_t chain_index) {
    if (chain_index < 1 || chain_index > (size_t)c.nQ) throw std::invalid_argument("chain_index out of range");
    return c.nQ - (int)(chain_index - 1);
}
