/* Minimal declarations for the cuTT transpose library, which is an empty git
 * submodule in the reference checkout.  Only the CPU parts of the reference
 * (gate factories, compiler, fused-unitary builder) are built for the oracle,
 * so every call here reports failure; none is reached by oracle/ref_driver.cpp. */
#pragma once
#include <cstddef>
#include <cuda_runtime.h>
typedef unsigned int cuttHandle;
typedef enum {
    CUTT_SUCCESS, CUTT_INVALID_PLAN, CUTT_INVALID_PARAMETER,
    CUTT_INVALID_DEVICE, CUTT_INTERNAL_ERROR, CUTT_UNDEFINED_ERROR
} cuttResult;
static inline cuttResult cuttInit() { return CUTT_SUCCESS; }
static inline cuttResult cuttPlan(cuttHandle*, int, int*, int*, size_t, cudaStream_t, bool) { return CUTT_UNDEFINED_ERROR; }
static inline cuttResult cuttActivatePlan(cuttHandle*, cuttHandle, cudaStream_t, int) { return CUTT_UNDEFINED_ERROR; }
static inline cuttResult cuttExecute(cuttHandle, void*, void*) { return CUTT_UNDEFINED_ERROR; }
