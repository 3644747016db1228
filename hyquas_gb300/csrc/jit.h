// Straight-line (specialised) OShareMem kernels compiled per gate group with
// NVRTC; see jit.cpp.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "compiler.h"

namespace hq {

struct JitKernel {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kern = nullptr;
    int threads = 0;
    size_t smem = 0;
    int blocks_per_sm = 1;
    size_t local_bytes = 0;  // local memory per thread (register spills)
};

bool jit_available();
// Compile (or fetch from the process-wide cache) one kernel per program.
std::vector<JitKernel> jit_compile_groups(const std::vector<const OshmProgram*>& progs);
// The kernels of every program when all are compiled already; false otherwise
// (nothing is compiled).
bool jit_lookup_cached(const std::vector<const OshmProgram*>& progs, std::vector<JitKernel>& out);
// `err`: the device error word (a RING kernel records a timed-out wait there)
// `copy`, when not null, is a device-accessible host buffer that receives the
// group's output as well (the last group of a run that leaves the final state
// on the host)
void jit_launch(const JitKernel& k, void* state, uint64_t ntiles, int* err, cudaStream_t st,
                void* copy = nullptr);
std::string jit_source(const OshmProgram& prog);

}  // namespace hq
