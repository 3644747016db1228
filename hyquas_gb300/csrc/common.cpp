#include "common.h"
#include "device.h"

#include <cstdarg>
#include <cstdio>

namespace hq {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }
void clear_last_error() { g_last_error.clear(); }
const std::string& last_error() { return g_last_error; }

void fail(hq_status code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw Failure(code, buf);
}

static Context g_ctx;

static void init_device(int device) {
    Context& c = g_ctx;
    int count = 0;
    HQ_CHECK_CUDA(cudaGetDeviceCount(&count));
    HQ_REQUIRE(device >= 0 && device < count, HQ_ERR_INVALID, "device %d not present (%d devices)",
               device, count);
    HQ_CHECK_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    HQ_CHECK_CUDA(cudaGetDeviceProperties(&prop, device));
    c.device = device;
    c.sm_count = prop.multiProcessorCount;
    c.smem_optin = (int)prop.sharedMemPerBlockOptin;
    c.hbm_bytes = prop.totalGlobalMem;
    HQ_CHECK_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    HQ_CHECK_CUDA(cudaMalloc(&c.d_error, sizeof(int) * 4));
    HQ_CHECK_CUDA(cudaMemset(c.d_error, 0, sizeof(int) * 4));
    c.partials_cap = 1 << 16;
    HQ_CHECK_CUDA(cudaMalloc(&c.d_partials, sizeof(double) * c.partials_cap));
    c.pinned_cap = 1 << 16;
    HQ_CHECK_CUDA(cudaMallocHost(&c.h_pinned, sizeof(double) * c.pinned_cap));
    HQ_CHECK_CUDA(cudaHostAlloc(&c.h_error, sizeof(int) * 4, cudaHostAllocMapped));
    HQ_CHECK_CUDA(cudaHostGetDevicePointer((void**)&c.h_error_dev, c.h_error, 0));
}

Context& ctx() {
    if (g_ctx.device < 0) init_device(0);
    HQ_CHECK_CUDA(cudaSetDevice(g_ctx.device));
    return g_ctx;
}

void ensure_init() { (void)ctx(); }

void init_explicit(int device) {
    if (g_ctx.device == device) return;
    HQ_REQUIRE(g_ctx.device < 0, HQ_ERR_STATE, "already initialised on device %d", g_ctx.device);
    init_device(device);
}

void* dev_alloc(size_t bytes) {
    Context& c = ctx();
    if (c.budget && c.in_use + bytes > c.budget)
        fail(HQ_ERR_NOMEM, "allocation of %zu bytes exceeds the HBM budget (%llu of %llu in use)",
             bytes, (unsigned long long)c.in_use, (unsigned long long)c.budget);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        fail(HQ_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    c.in_use += bytes;
    return p;
}

void dev_free(void* p, size_t bytes) {
    if (!p) return;
    Context& c = ctx();
    cudaFree(p);
    c.in_use = c.in_use >= bytes ? c.in_use - bytes : 0;
}

void* dev_alloc_ordered(size_t bytes) {
    Context& c = ctx();
    if (c.budget && c.in_use + bytes > c.budget)
        fail(HQ_ERR_NOMEM, "allocation of %zu bytes exceeds the HBM budget (%llu of %llu in use)",
             bytes, (unsigned long long)c.in_use, (unsigned long long)c.budget);
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, bytes, c.stream);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        fail(HQ_ERR_NOMEM, "cudaMallocAsync(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    c.in_use += bytes;
    return p;
}

void dev_free_ordered(void* p, size_t bytes) {
    if (!p) return;
    Context& c = ctx();
    cudaFreeAsync(p, c.stream);
    c.in_use = c.in_use >= bytes ? c.in_use - bytes : 0;
}

int compute_sms() {
    Context& c = ctx();
    if (c.rb_sms > 0 && c.rb_done) {
        const cudaError_t q = cudaEventQuery(c.rb_done);
        if (q == cudaErrorNotReady) return c.sm_count - c.rb_sms;
        HQ_CHECK_CUDA(q);
        c.rb_sms = 0;
    }
    return c.sm_count;
}

void check_device_error() {
    Context& c = ctx();
    // a one-thread kernel writes the word into mapped page-locked memory: no
    // copy-engine transfer, which on GB300 can wait tens of milliseconds
    // behind a large readback in flight to the same host
    launch_error_readout(c.d_error, c.h_error_dev, c.stream);
    HQ_CHECK_CUDA(cudaStreamSynchronize(c.stream));
    int h[4];
    for (int i = 0; i < 4; i++) h[i] = reinterpret_cast<volatile int*>(c.h_error)[i];
    if (h[0] != 0) {
        HQ_CHECK_CUDA(cudaMemsetAsync(c.d_error, 0, sizeof(int) * 4, c.stream));
        HQ_CHECK_CUDA(cudaStreamSynchronize(c.stream));
        if (h[0] == 1)
            fail(HQ_ERR_TIMEOUT, "device-side bounded wait expired (site %d, detail %d)", h[1], h[2]);
        fail(HQ_ERR_INVALID, "device-side check failed (code %d, site %d, detail %d)", h[0], h[1],
             h[2]);
    }
}

}  // namespace hq
