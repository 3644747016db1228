// Recording stand-in for the CUDA runtime -- TEST INFRASTRUCTURE ONLY.
//
// The reference's host code (src/circuit.cpp, src/executor.cpp, the host side of
// src/kernelOpt.cu and src/kernelSimple.cu) is linked against this file instead
// of libcudart on a machine without a GPU.  Every runtime call it makes is
// answered here without a device and written to a trace: allocations (fake
// device addresses), memsets, host-to-device copies with their bytes, uploads
// to __constant__ symbols, kernel launches with their configuration and
// argument bytes, stream synchronisations, and the cudaProfilerStart/Stop pair
// that brackets the reference's "Time Cost" region (src/circuit.cpp:17-52).
// oracle/ref_replay.cu replays the trace on a GPU with the reference's kernels
// compiled from the same sources, so the reference's own schedule, lowering and
// kernels run on the GB300 although its host code cannot be built there.
//
// Trace format (little-endian, see ref_trace.h): "HQRT" + version, then
// records of (u32 kind, payload).  Argument sizes of a launch come from the
// demangled kernel signature recorded at registration.
#include <cublas_v2.h>
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>
#include <cxxabi.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ref_trace.h"

namespace {

FILE* g_trace = nullptr;
uint64_t g_next_addr = 0x100000000000ull;  // fake device addresses start here
std::map<uint64_t, uint64_t> g_allocs;        // fake base -> size
std::map<const void*, std::string> g_funcs;   // host stub -> mangled device name
std::map<const void*, std::string> g_vars;    // host shadow -> device symbol name
std::map<const void*, std::vector<int>> g_arg_sizes;  // host stub -> bytes per argument
std::map<const void*, std::vector<int>> g_arg_ptrs;   // host stub -> 1 when a pointer
uint64_t g_last_d2h_src = 0;
int g_next_stream = 1;

struct PendingLaunch {
    dim3 grid, block;
    size_t shmem;
    void* stream;
} g_pending;

void put(const void* p, size_t n) {
    if (g_trace && fwrite(p, 1, n, g_trace) != n) {
        fprintf(stderr, "fake_cuda: trace write failed\n");
        exit(3);
    }
}
void put_u32(uint32_t v) { put(&v, 4); }
void put_u64(uint64_t v) { put(&v, 8); }
void put_str(const std::string& s) {
    put_u32((uint32_t)s.size());
    put(s.data(), s.size());
}

bool is_device(const void* p) {
    const uint64_t a = (uint64_t)p;
    auto it = g_allocs.upper_bound(a);
    if (it == g_allocs.begin()) return false;
    --it;
    return a >= it->first && a < it->first + it->second;
}

// Parameter list of a demangled signature "void f<...>(float2*, int, ...)":
// bytes per parameter and whether it is a pointer.  Covers the scalar types
// the reference's kernels take.
void parse_params(const std::string& sig, std::vector<int>& sizes, std::vector<int>& ptrs) {
    // the parameter list is the last top-level parenthesised group
    int depth = 0;
    size_t open = std::string::npos, close = std::string::npos;
    for (size_t i = sig.size(); i-- > 0;) {
        if (sig[i] == ')') {
            if (depth++ == 0) close = i;
        } else if (sig[i] == '(') {
            if (--depth == 0) { open = i; break; }
        }
    }
    if (open == std::string::npos || close == std::string::npos) return;
    std::string list = sig.substr(open + 1, close - open - 1);
    if (list.empty() || list == "void") return;
    std::vector<std::string> parts;
    int d = 0;
    std::string cur;
    for (char c : list) {
        if (c == '<' || c == '(') d++;
        if (c == '>' || c == ')') d--;
        if (c == ',' && d == 0) {
            parts.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    parts.push_back(cur);
    for (std::string p : parts) {
        while (!p.empty() && p.front() == ' ') p.erase(p.begin());
        while (!p.empty() && p.back() == ' ') p.pop_back();
        if (!p.empty() && p.back() == '*') { sizes.push_back(8); ptrs.push_back(1); continue; }
        int sz = -1;
        if (p == "int" || p == "unsigned int" || p == "float") sz = 4;
        else if (p == "long long" || p == "unsigned long long" || p == "long" || p == "unsigned long" ||
                 p == "double" || p == "float2")
            sz = 8;
        else if (p == "double2") sz = 16;
        else if (p == "char" || p == "unsigned char" || p == "bool" || p == "signed char") sz = 1;
        else if (p == "short" || p == "unsigned short") sz = 2;
        if (sz < 0) {
            fprintf(stderr, "fake_cuda: unknown parameter type '%s' in %s\n", p.c_str(), sig.c_str());
            exit(3);
        }
        sizes.push_back(sz);
        ptrs.push_back(0);
    }
}

}  // namespace

// ---- trace control (called by trace_main.cpp) ------------------------------

extern "C" int fake_trace_open(const char* path) {
    g_trace = fopen(path, "wb");
    if (!g_trace) return -1;
    put("HQRT", 4);
    put_u32(kRefTraceVersion);
    return 0;
}

extern "C" void fake_trace_info(int32_t num_qubits) {
    put_u32(REC_INFO);
    put_u32((uint32_t)num_qubits);
}

extern "C" void fake_trace_layout(const int32_t* pos, int32_t n) {
    put_u32(REC_LAYOUT);
    put_u32((uint32_t)n);
    put(pos, sizeof(int32_t) * (size_t)n);
}

extern "C" uint64_t fake_last_d2h_src() { return g_last_d2h_src; }

extern "C" uint64_t fake_alloc_base_of(uint64_t addr) {
    auto it = g_allocs.upper_bound(addr);
    if (it == g_allocs.begin()) return 0;
    --it;
    return addr < it->first + it->second ? it->first : 0;
}

extern "C" void fake_trace_close() {
    if (!g_trace) return;
    put_u32(REC_END);
    fclose(g_trace);
    g_trace = nullptr;
}

// ---- registration hooks the compiler-generated host code calls -------------

extern "C" void** __cudaRegisterFatBinary(void* fatCubin) {
    static void* handle = nullptr;
    (void)fatCubin;
    return &handle;
}
extern "C" void __cudaRegisterFatBinaryEnd(void** h) { (void)h; }
extern "C" void __cudaUnregisterFatBinary(void** h) { (void)h; }

extern "C" void __cudaRegisterVar(void** h, char* hostVar, char* deviceAddress,
                                  const char* deviceName, int ext, size_t size, int constant,
                                  int global) {
    (void)h; (void)deviceAddress; (void)ext; (void)size; (void)constant; (void)global;
    g_vars[hostVar] = deviceName;
}

extern "C" void __cudaRegisterFunction(void** h, const char* hostFun, char* deviceFun,
                                       const char* deviceName, int thread_limit, uint3* tid,
                                       uint3* bid, dim3* bDim, dim3* gDim, int* wSize) {
    (void)h; (void)deviceFun; (void)thread_limit; (void)tid; (void)bid; (void)bDim; (void)gDim;
    (void)wSize;
    g_funcs[hostFun] = deviceName;
    int status = 0;
    char* dem = abi::__cxa_demangle(deviceName, nullptr, nullptr, &status);
    std::vector<int> sizes, ptrs;
    if (status == 0 && dem) {
        parse_params(dem, sizes, ptrs);
        free(dem);
    }
    g_arg_sizes[hostFun] = sizes;
    g_arg_ptrs[hostFun] = ptrs;
}

extern "C" unsigned __cudaPushCallConfiguration(dim3 gridDim, dim3 blockDim, size_t sharedMem,
                                                struct CUstream_st* stream) {
    g_pending.grid = gridDim;
    g_pending.block = blockDim;
    g_pending.shmem = sharedMem;
    g_pending.stream = stream;
    return 0;
}

extern "C" cudaError_t __cudaPopCallConfiguration(dim3* gridDim, dim3* blockDim, size_t* sharedMem,
                                                  void* stream) {
    *gridDim = g_pending.grid;
    *blockDim = g_pending.block;
    *sharedMem = g_pending.shmem;
    *(void**)stream = g_pending.stream;
    return cudaSuccess;
}

// The launch stubs nvcc writes look a kernel up once (__cudaGetKernel, with the
// host stub as key) and launch through __cudaLaunchKernel; the handle here is
// the host stub itself.
extern "C" cudaError_t __cudaGetKernel(cudaKernel_t* kernel, const void* fun) {
    *kernel = (cudaKernel_t)fun;
    return cudaSuccess;
}

extern "C" cudaError_t __cudaLaunchKernel(cudaKernel_t kernel, dim3 gridDim, dim3 blockDim,
                                          void** args, size_t sharedMem, cudaStream_t stream) {
    return cudaLaunchKernel((const void*)kernel, gridDim, blockDim, args, sharedMem, stream);
}

// ---- runtime API ------------------------------------------------------------

cudaError_t cudaLaunchKernel(const void* func, dim3 gridDim, dim3 blockDim, void** args,
                             size_t sharedMem, cudaStream_t stream) {
    auto it = g_funcs.find(func);
    if (it == g_funcs.end()) {
        fprintf(stderr, "fake_cuda: launch of an unregistered kernel\n");
        exit(3);
    }
    const std::vector<int>& sizes = g_arg_sizes[func];
    const std::vector<int>& ptrs = g_arg_ptrs[func];
    put_u32(REC_LAUNCH);
    put_str(it->second);
    put_u32(gridDim.x); put_u32(gridDim.y); put_u32(gridDim.z);
    put_u32(blockDim.x); put_u32(blockDim.y); put_u32(blockDim.z);
    put_u64(sharedMem);
    put_u64((uint64_t)stream);
    put_u32((uint32_t)sizes.size());
    for (size_t i = 0; i < sizes.size(); i++) {
        put_u32((uint32_t)sizes[i]);
        put_u32((uint32_t)ptrs[i]);
        put(args[i], (size_t)sizes[i]);
    }
    return cudaSuccess;
}

cudaError_t cudaMalloc(void** p, size_t size) {
    const uint64_t a = g_next_addr;
    g_next_addr += (size + 0xFFFFull) & ~0xFFFFull;  // 64 KiB apart, like a real allocator's alignment
    g_allocs[a] = size;
    *p = (void*)a;
    put_u32(REC_MALLOC);
    put_u64(a);
    put_u64(size);
    return cudaSuccess;
}

cudaError_t cudaFree(void* p) {
    if (!p) return cudaSuccess;
    g_allocs.erase((uint64_t)p);
    put_u32(REC_FREE);
    put_u64((uint64_t)p);
    return cudaSuccess;
}

cudaError_t cudaHostAlloc(void** p, size_t size, unsigned int flags) {
    (void)flags;
    *p = calloc(1, size ? size : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t cudaFreeHost(void* p) {
    free(p);
    return cudaSuccess;
}

static cudaError_t record_copy(void* dst, const void* src, size_t count, void* stream, int async) {
    const bool dd = is_device(dst), sd = is_device(src);
    if (dd && !sd) {
        put_u32(REC_H2D);
        put_u64((uint64_t)dst);
        put_u64((uint64_t)stream);
        put_u32((uint32_t)async);
        put_u64(count);
        put(src, count);
    } else if (!dd && sd) {
        // device-to-host reads return zeros; the source address is kept for
        // the driver, which reads the reference's logical-to-physical map
        // through Circuit::ampAtGPU (src/circuit.cpp:120-142)
        g_last_d2h_src = (uint64_t)src;
        memset(dst, 0, count);
        put_u32(REC_D2H);
        put_u64((uint64_t)src);
        put_u64(count);
    } else if (dd && sd) {
        put_u32(REC_D2D);
        put_u64((uint64_t)dst);
        put_u64((uint64_t)src);
        put_u64((uint64_t)stream);
        put_u64(count);
    } else {
        memcpy(dst, src, count);
    }
    return cudaSuccess;
}

cudaError_t cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind kind) {
    (void)kind;
    return record_copy(dst, src, count, nullptr, 0);
}

cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t count, enum cudaMemcpyKind kind,
                            cudaStream_t stream) {
    (void)kind;
    return record_copy(dst, src, count, stream, 1);
}

cudaError_t cudaMemcpyToSymbolAsync(const void* symbol, const void* src, size_t count,
                                    size_t offset, enum cudaMemcpyKind kind, cudaStream_t stream) {
    (void)kind;
    auto it = g_vars.find(symbol);
    if (it == g_vars.end()) {
        fprintf(stderr, "fake_cuda: copy to an unregistered symbol\n");
        exit(3);
    }
    put_u32(REC_SYMBOL_H2D);
    put_str(it->second);
    put_u64(offset);
    put_u64((uint64_t)stream);
    put_u64(count);
    put(src, count);
    return cudaSuccess;
}

cudaError_t cudaMemsetAsync(void* dst, int value, size_t count, cudaStream_t stream) {
    put_u32(REC_MEMSET);
    put_u64((uint64_t)dst);
    put_u32((uint32_t)value);
    put_u64(count);
    put_u64((uint64_t)stream);
    return cudaSuccess;
}

cudaError_t cudaStreamCreate(cudaStream_t* s) {
    *s = (cudaStream_t)(uintptr_t)(g_next_stream++);
    return cudaSuccess;
}

cudaError_t cudaStreamSynchronize(cudaStream_t s) {
    put_u32(REC_SYNC);
    put_u64((uint64_t)s);
    return cudaSuccess;
}

cudaError_t cudaDeviceSynchronize(void) {
    put_u32(REC_SYNC);
    put_u64(~0ull);
    return cudaSuccess;
}

cudaError_t cudaStreamWaitEvent(cudaStream_t stream, cudaEvent_t event, unsigned int flags) {
    (void)stream; (void)event; (void)flags;  // one stream in the single-GPU paths
    return cudaSuccess;
}

cudaError_t cudaEventCreate(cudaEvent_t* e) {
    *e = (cudaEvent_t)(uintptr_t)1;
    return cudaSuccess;
}

cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s) {
    (void)e; (void)s;
    return cudaSuccess;
}

cudaError_t cudaProfilerStart(void) {
    put_u32(REC_REGION_BEGIN);
    return cudaSuccess;
}

cudaError_t cudaProfilerStop(void) {
    put_u32(REC_REGION_END);
    return cudaSuccess;
}

cudaError_t cudaSetDevice(int device) {
    return device == 0 ? cudaSuccess : cudaErrorInvalidDevice;
}

cudaError_t cudaGetDeviceCount(int* count) {
    *count = 1;
    return cudaSuccess;
}

cudaError_t cudaGetDeviceProperties(struct cudaDeviceProp* prop, int device) {
    (void)device;
    memset(prop, 0, sizeof(*prop));
    strcpy(prop->name, "trace recorder");
    return cudaSuccess;
}

cudaError_t cudaDeviceEnablePeerAccess(int peer, unsigned int flags) {
    (void)peer; (void)flags;
    return cudaSuccess;
}

cudaError_t cudaDeviceSetSharedMemConfig(enum cudaSharedMemConfig config) {
    (void)config;
    return cudaSuccess;
}

const char* cudaGetErrorString(cudaError_t e) {
    return e == cudaSuccess ? "no error" : "fake_cuda error";
}

cublasStatus_t cublasCreate_v2(cublasHandle_t* handle) {
    *handle = nullptr;
    return CUBLAS_STATUS_SUCCESS;
}

cublasStatus_t cublasSetStream_v2(cublasHandle_t handle, cudaStream_t stream) {
    (void)handle; (void)stream;
    return CUBLAS_STATUS_SUCCESS;
}
