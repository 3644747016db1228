// Replayer of the reference's traced single-GPU runs -- TEST INFRASTRUCTURE ONLY.
//
// A trace (oracle/ref_gpu/fake_cuda.cpp, written by the reference's own host
// code on a machine without a GPU) lists the device work of one reference run:
// allocations, memsets, host-to-device copies, __constant__ uploads and kernel
// launches with their argument bytes.  This file issues the same work on a GPU,
// in the same order, on one stream, launching the reference's kernels from
// cubins compiled from its sources (src/kernelOpt.cu, src/kernelSimple.cu).  The
// region between cudaProfilerStart and cudaProfilerStop is the reference's
// "Time Cost" (src/circuit.cpp:17-52); it is timed with the host clock (the
// reference's own measure) and with CUDA events.
//
// Checks before any launch: every kernel exists in the cubins, its parameter
// count and sizes (cuFuncGetParamInfo) equal the recorded argument sizes, and
// every pointer argument falls inside a replayed allocation.  A failed check
// returns an error without launching.  Only bench.py's baseline legs and the
// tests call this library.
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ref_trace.h"

namespace {

struct Reader {
    const std::vector<uint8_t>& b;
    size_t p = 0;
    bool ok = true;
    explicit Reader(const std::vector<uint8_t>& buf) : b(buf) {}
    bool take(void* dst, size_t n) {
        if (!ok || p + n > b.size()) return ok = false;
        memcpy(dst, b.data() + p, n);
        p += n;
        return true;
    }
    uint32_t u32() { uint32_t v = 0; take(&v, 4); return v; }
    uint64_t u64() { uint64_t v = 0; take(&v, 8); return v; }
    std::string str() {
        uint32_t n = u32();
        if (!ok || p + n > b.size()) { ok = false; return {}; }
        std::string s((const char*)b.data() + p, n);
        p += n;
        return s;
    }
    const uint8_t* bytes(uint64_t n) {
        if (!ok || p + n > b.size()) { ok = false; return nullptr; }
        const uint8_t* r = b.data() + p;
        p += n;
        return r;
    }
};

struct Alloc {
    void* real;
    uint64_t size;
};

struct Replay {
    std::vector<CUmodule> modules;
    std::map<uint64_t, Alloc> allocs;  // fake base -> real allocation
    std::map<std::string, CUfunction> funcs;
    cudaStream_t stream = nullptr;
    char* err;
    int errlen;

    bool fail(const char* fmt, const char* a = "", const char* b = "") {
        snprintf(err, (size_t)errlen, fmt, a, b);
        return false;
    }
    bool cuda(cudaError_t e, const char* what) {
        return e == cudaSuccess ? true : fail("%s: %s", what, cudaGetErrorString(e));
    }
    bool drv(CUresult r, const char* what) {
        if (r == CUDA_SUCCESS) return true;
        const char* s = "unknown";
        cuGetErrorString(r, &s);
        return fail("%s: %s", what, s);
    }
    bool translate(uint64_t fake, void** real) {
        if (fake == 0) { *real = nullptr; return true; }
        auto it = allocs.upper_bound(fake);
        if (it == allocs.begin()) return false;
        --it;
        if (fake >= it->first + it->second.size) return false;
        *real = (char*)it->second.real + (fake - it->first);
        return true;
    }
    bool function(const std::string& name, CUfunction* f) {
        auto it = funcs.find(name);
        if (it != funcs.end()) { *f = it->second; return true; }
        for (CUmodule m : modules) {
            if (cuModuleGetFunction(f, m, name.c_str()) == CUDA_SUCCESS) {
                funcs[name] = *f;
                return true;
            }
        }
        return fail("kernel %s not found in the reference cubins", name.c_str());
    }
    bool symbol(const std::string& name, CUdeviceptr* p, size_t* size) {
        for (CUmodule m : modules)
            if (cuModuleGetGlobal(p, size, m, name.c_str()) == CUDA_SUCCESS) return true;
        return fail("symbol %s not found in the reference cubins", name.c_str());
    }
};

}  // namespace

// Replays `repeats` times the trace at `trace_path` (after one untimed pass).
//   cubins      paths of the reference's kernel cubins
//   state_out   host buffer receiving the final state allocation (2^n complex64),
//               or NULL; state_bytes its size
//   layout_out  n ints: physical position of each logical qubit, or NULL
//   out[0]      best host-clock time of the "Time Cost" region (ms)
//   out[1]      mean host-clock time of that region (ms)
//   out[2]      best CUDA-event time of the region on the replay stream (ms)
//   out[3]      kernel launches in the region
//   out[4]      number of qubits
// Returns 0, or -1 with a message in err.
extern "C" int ref_replay_run(const char* trace_path, const char* const* cubins, int ncubins,
                              int repeats, void* state_out, uint64_t state_bytes,
                              int32_t* layout_out, double* out, char* err, int errlen) {
    Replay R;
    R.err = err;
    R.errlen = errlen;
    err[0] = 0;
    std::vector<uint8_t> buf;
    {
        FILE* f = fopen(trace_path, "rb");
        if (!f) return R.fail("cannot open %s", trace_path), -1;
        fseek(f, 0, SEEK_END);
        long len = ftell(f);
        fseek(f, 0, SEEK_SET);
        buf.resize(len > 0 ? (size_t)len : 0);
        size_t got = fread(buf.data(), 1, buf.size(), f);
        fclose(f);
        if (got != buf.size() || buf.size() < 8 || memcmp(buf.data(), "HQRT", 4) != 0)
            return R.fail("%s is not a reference trace", trace_path), -1;
        uint32_t ver;
        memcpy(&ver, buf.data() + 4, 4);
        if (ver != kRefTraceVersion) return R.fail("trace version mismatch"), -1;
    }
    bool good = R.cuda(cudaFree(nullptr), "context") && R.drv(cuInit(0), "cuInit");
    for (int i = 0; good && i < ncubins; i++) {
        CUmodule m;
        good = R.drv(cuModuleLoad(&m, cubins[i]), cubins[i]);
        if (good) R.modules.push_back(m);
    }
    good = good && R.cuda(cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking), "stream");
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    good = good && R.cuda(cudaEventCreate(&ev0), "event") && R.cuda(cudaEventCreate(&ev1), "event");

    int n = 0;
    uint64_t state_fake = 0;
    double best_host = 1e30, sum_host = 0, best_dev = 1e30;
    int launches_in_region = 0, timed = 0;
    std::vector<int32_t> layout;
    std::vector<uint64_t> frees;

    for (int pass = 0; good && pass <= repeats; pass++) {
        Reader rd(buf);
        rd.p = 8;
        bool in_region = false;
        int launches = 0;
        auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const uint32_t kind = rd.u32();
            if (!rd.ok) { good = R.fail("truncated trace"); break; }
            if (kind == REC_END) break;
            switch (kind) {
                case REC_INFO:
                    n = (int)rd.u32();
                    break;
                case REC_MALLOC: {
                    const uint64_t fake = rd.u64(), size = rd.u64();
                    if (pass == 0) {
                        void* p = nullptr;
                        good = R.cuda(cudaMalloc(&p, size ? size : 1), "cudaMalloc");
                        if (good) R.allocs[fake] = Alloc{p, size};
                        if (good && n > 0 && state_fake == 0 && size == (uint64_t(8) << n))
                            state_fake = fake;  // the state vector (src/kernelSimple.cu:9-37)
                    }
                    break;
                }
                case REC_FREE: {
                    const uint64_t fake = rd.u64();
                    if (pass == 0) frees.push_back(fake);  // freed after the last pass
                    break;
                }
                case REC_MEMSET: {
                    const uint64_t dst = rd.u64();
                    const uint32_t value = rd.u32();
                    const uint64_t count = rd.u64();
                    rd.u64();
                    void* real;
                    if (!R.translate(dst, &real)) { good = R.fail("memset outside any allocation"); break; }
                    good = R.cuda(cudaMemsetAsync(real, (int)value, count, R.stream), "memset");
                    break;
                }
                case REC_H2D: {
                    const uint64_t dst = rd.u64();
                    rd.u64();
                    rd.u32();
                    const uint64_t count = rd.u64();
                    const uint8_t* src = rd.bytes(count);
                    void *real, *last;
                    if (!src || count == 0 || !R.translate(dst + count - 1, &last) ||
                        !R.translate(dst, &real) || (char*)last - (char*)real != (ptrdiff_t)(count - 1)) {
                        good = R.fail("host-to-device copy outside any allocation");
                        break;
                    }
                    good = R.cuda(cudaMemcpyAsync(real, src, count, cudaMemcpyHostToDevice, R.stream),
                                  "H2D");
                    break;
                }
                case REC_D2H:  // the layout probes made after the run: nothing to do
                    rd.u64();
                    rd.u64();
                    break;
                case REC_D2D: {
                    const uint64_t dst = rd.u64(), src = rd.u64();
                    rd.u64();
                    const uint64_t count = rd.u64();
                    void *rd_, *rs;
                    if (!R.translate(dst, &rd_) || !R.translate(src, &rs)) {
                        good = R.fail("device copy outside any allocation");
                        break;
                    }
                    good = R.cuda(cudaMemcpyAsync(rd_, rs, count, cudaMemcpyDeviceToDevice, R.stream),
                                  "D2D");
                    break;
                }
                case REC_SYMBOL_H2D: {
                    const std::string name = rd.str();
                    const uint64_t offset = rd.u64();
                    rd.u64();
                    const uint64_t count = rd.u64();
                    const uint8_t* src = rd.bytes(count);
                    CUdeviceptr p;
                    size_t size;
                    if (!src) { good = R.fail("truncated symbol copy"); break; }
                    good = R.symbol(name, &p, &size);
                    if (good && offset + count > size) good = R.fail("copy past symbol %s", name.c_str());
                    if (good) good = R.drv(cuMemcpyHtoDAsync(p + offset, src, count, (CUstream)R.stream),
                                           "symbol upload");
                    break;
                }
                case REC_LAUNCH: {
                    const std::string name = rd.str();
                    unsigned g[3], b[3];
                    for (auto& x : g) x = rd.u32();
                    for (auto& x : b) x = rd.u32();
                    const uint64_t shmem = rd.u64();
                    rd.u64();
                    const uint32_t nargs = rd.u32();
                    if (!rd.ok || nargs > 64) { good = R.fail("bad launch record"); break; }
                    std::vector<std::vector<uint8_t>> args(nargs);
                    std::vector<void*> params(nargs);
                    for (uint32_t i = 0; good && i < nargs; i++) {
                        const uint32_t sz = rd.u32(), isptr = rd.u32();
                        const uint8_t* v = rd.bytes(sz);
                        if (!v || sz > 64) { good = R.fail("bad launch argument"); break; }
                        args[i].assign(v, v + sz);
                        if (isptr) {
                            uint64_t fake;
                            memcpy(&fake, v, 8);
                            void* real;
                            if (sz != 8 || !R.translate(fake, &real)) {
                                good = R.fail("pointer argument of %s outside any allocation",
                                              name.c_str());
                                break;
                            }
                            memcpy(args[i].data(), &real, 8);
                        }
                        params[i] = args[i].data();
                    }
                    if (!good) break;
                    CUfunction f;
                    if (!R.function(name, &f)) { good = false; break; }
                    if (pass == 0) {  // parameter layout of the cubin == the recorded arguments
                        for (uint32_t i = 0; good && i <= nargs; i++) {
                            size_t off = 0, sz = 0;
                            const CUresult r = cuFuncGetParamInfo(f, i, &off, &sz);
                            if (i == nargs) {
                                if (r == CUDA_SUCCESS) good = R.fail("%s takes more parameters than recorded", name.c_str());
                            } else if (r != CUDA_SUCCESS || sz != args[i].size()) {
                                good = R.fail("%s: parameter size differs from the recording", name.c_str());
                            }
                        }
                        if (!good) break;
                    }
                    good = R.drv(cuLaunchKernel(f, g[0], g[1], g[2], b[0], b[1], b[2], (unsigned)shmem,
                                                (CUstream)R.stream, params.data(), nullptr),
                                 name.c_str());
                    if (in_region) launches++;
                    break;
                }
                case REC_SYNC:
                    rd.u64();
                    good = R.cuda(cudaStreamSynchronize(R.stream), "synchronize");
                    break;
                case REC_REGION_BEGIN:
                    good = R.cuda(cudaStreamSynchronize(R.stream), "synchronize") &&
                           R.cuda(cudaEventRecord(ev0, R.stream), "event");
                    t0 = std::chrono::steady_clock::now();
                    in_region = true;
                    break;
                case REC_REGION_END: {
                    // the reference's region ends after its own synchronisation
                    // (Executor::finalize / kernelExecSimple); sync again to be sure
                    good = R.cuda(cudaEventRecord(ev1, R.stream), "event") &&
                           R.cuda(cudaStreamSynchronize(R.stream), "synchronize");
                    const double host_ms =
                        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                            .count();
                    float dev_ms = 0;
                    if (good) good = R.cuda(cudaEventElapsedTime(&dev_ms, ev0, ev1), "elapsed");
                    in_region = false;
                    if (pass > 0) {
                        best_host = host_ms < best_host ? host_ms : best_host;
                        sum_host += host_ms;
                        best_dev = dev_ms < best_dev ? dev_ms : best_dev;
                        timed++;
                    }
                    launches_in_region = launches;
                    break;
                }
                case REC_LAYOUT: {
                    const uint32_t m = rd.u32();
                    layout.resize(m);
                    if (m) rd.take(layout.data(), sizeof(int32_t) * m);
                    break;
                }
                default:
                    good = R.fail("unknown trace record");
            }
            if (!good) break;
        }
        if (good) good = R.cuda(cudaStreamSynchronize(R.stream), "synchronize");
    }

    if (good && state_out) {
        void* real = nullptr;
        if (!state_fake || !R.translate(state_fake, &real))
            good = R.fail("no state allocation in the trace");
        else if (state_bytes != (uint64_t(8) << n))
            good = R.fail("state buffer size does not match the traced state");
        else
            good = R.cuda(cudaMemcpy(state_out, real, state_bytes, cudaMemcpyDeviceToHost), "D2H");
    }
    if (good && layout_out) {
        if ((int)layout.size() != n) good = R.fail("no layout record");
        else memcpy(layout_out, layout.data(), sizeof(int32_t) * (size_t)n);
    }
    for (auto& kv : R.allocs) cudaFree(kv.second.real);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (R.stream) cudaStreamDestroy(R.stream);
    for (CUmodule m : R.modules) cuModuleUnload(m);
    if (!good) return -1;
    out[0] = timed ? best_host : 0;
    out[1] = timed ? sum_host / timed : 0;
    out[2] = timed ? best_dev : 0;
    out[3] = launches_in_region;
    out[4] = n;
    return 0;
}
