// Shared host-side infrastructure: error reporting, the device context and
// small bit utilities.  Errors are C++ exceptions inside the library and are
// turned into hq_status codes at the C-ABI boundary (capi.cpp); the reference
// instead exits the process (src/utils.h:106-144).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/hyquas_gb300.h"

namespace hq {

struct Failure : std::runtime_error {
    hq_status code;
    Failure(hq_status c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] void fail(hq_status code, const char* fmt, ...);
void set_last_error(const std::string& msg);
void clear_last_error();

#define HQ_CHECK_CUDA(call)                                                                  \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            ::hq::fail(HQ_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
                       __FILE__, __LINE__);                                                   \
    } while (0)

#define HQ_REQUIRE(cond, code, ...)                                                           \
    do {                                                                                      \
        if (!(cond)) ::hq::fail(code, __VA_ARGS__);                                           \
    } while (0)

// One process, one GPU: the device, its stream and the allocation ledger used
// for HBM-budget admission.  Replaces MyGlobalVars (src/utils.cpp:17-60).
struct Context {
    int device = -1;
    int sm_count = 0;
    int smem_optin = 0;
    uint64_t hbm_bytes = 0;
    uint64_t budget = 0;  // 0 = no budget
    uint64_t in_use = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // asynchronous readbacks (made on first use)
    int* d_error = nullptr;        // device error word (bounded waits, bad indices)
    int* h_error = nullptr;        // its page-locked, device-mapped host copy
    int* h_error_dev = nullptr;    // h_error's device address
    double* d_partials = nullptr;  // reduction partials (FP64), see k_plain.cu
    size_t partials_cap = 0;       // doubles
    double* h_pinned = nullptr;    // pinned readback of reductions
    size_t pinned_cap = 0;
    // SM-driven readbacks to pinned host memory run on a few SMs of their
    // own; while the latest is in flight, the persistent group kernels launch
    // on the others so that none of their blocks waits for an SM
    cudaEvent_t rb_done = nullptr;
    int rb_sms = 0;
};

Context& ctx();               // initialises on first use (device 0 unless hq_init chose)
void ensure_init();
void* dev_alloc(size_t bytes);  // budget-checked cudaMalloc
void dev_free(void* p, size_t bytes);
// stream-ordered on the library stream (cudaMallocAsync / cudaFreeAsync): for
// memory only the library stream uses, so that freeing it does not wait for
// other streams (an asynchronous readback, say) the way cudaFree does
void* dev_alloc_ordered(size_t bytes);
void dev_free_ordered(void* p, size_t bytes);
void check_device_error();      // reads and clears the device error word
int compute_sms();               // SMs a persistent kernel may fill now

inline int popcount64(uint64_t x) { return __builtin_popcountll(x); }
inline int ctz64(uint64_t x) { return __builtin_ctzll(x); }

// Scatter the low bits of v into the set bits of mask (bit deposit).
inline uint64_t deposit(uint64_t v, uint64_t mask) {
    uint64_t r = 0;
    for (uint64_t m = mask; m; m &= m - 1) {
        if (v & 1) r |= m & (~m + 1);
        v >>= 1;
    }
    return r;
}

}  // namespace hq
